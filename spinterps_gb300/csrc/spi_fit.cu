// Variogram fitting on the GPU: empirical variograms of a batch of steps and
// batched differential evolution of the nested model parameters.
//
// Replaces, for every step at once, what variograms/vgs.py does per step
// (driven by variograms/fitvgs.py:143-278):
//   - all pairs i > j with their distance, sorted by distance
//     (vgs.py:311-391), here with an exact bucket sort: a histogram of
//     distances into ~P/4 buckets, a scatter, then a sort of each bucket by
//     (distance, pair index);
//   - the mdr cut-off (vgs.py:597-659) and bins of nk consecutive pairs with
//     their mean distance and Cressie-Hawkins estimate (vgs.py:414-422,
//     495-520), summed in numpy's pairwise order so that the bins agree with
//     the reference to the last bits;
//   - the differential-evolution fits of every model permutation
//     (vgs.py:680-764): one CTA per (step, permutation), population
//     50 * D^2 in [0,1]^D as scipy scales it, best/1/bin with a dithered
//     F in [0.5, 1) and CR 0.7, out-of-range components redrawn, stopping
//     when the population energies' std <= tol * |mean| (scipy's rule).
#include <algorithm>

#include "spi_common.cuh"

namespace spi {

// x^4 rounded once, as the correctly rounded pow of the host libm that the
// reference's ``** 4`` calls: x^2 = p + e and p^2 = hi + lo are exact
// (Dekker's product by FMA), x^4 = hi + (lo + 2pe) with the e^2 term below
// 2^-104 relative, and the final add rounds the exact two-term sum.
__device__ __forceinline__ double pow4_rn(double x) {
  const double p = __dmul_rn(x, x);
  const double e = __fma_rn(x, x, -p);
  const double hi = __dmul_rn(p, p);
  double lo = __fma_rn(p, p, -hi);
  lo = __fma_rn(__dmul_rn(2.0, p), e, lo);
  return __dadd_rn(hi, lo);
}

// numpy's pairwise sum (the reduction numpy.sum / numpy.mean use) for
// n <= 128 contiguous values: plain loop below 8, else 8 strided partial
// sums combined ((r0+r1)+(r2+r3))+((r4+r5)+(r6+r7)), then the tail.
template <typename F>
__device__ double np_pairwise_sum(int n, F at) {
  if (n < 8) {
    double res = 0.0;
    for (int i = 0; i < n; ++i) res = __dadd_rn(res, at(i));
    return res;
  }
  double r[8];
  for (int k = 0; k < 8; ++k) r[k] = at(k);
  int i = 8;
  for (; i < n - (n % 8); i += 8)
    for (int k = 0; k < 8; ++k) r[k] = __dadd_rn(r[k], at(i + k));
  double res = __dadd_rn(__dadd_rn(__dadd_rn(r[0], r[1]), __dadd_rn(r[2], r[3])),
                         __dadd_rn(__dadd_rn(r[4], r[5]), __dadd_rn(r[6], r[7])));
  for (; i < n; ++i) res = __dadd_rn(res, at(i));
  return res;
}

// pair index p -> (i, j), i > j, row order of numpy.tril_indices(n, -1)
__device__ __forceinline__ void pair_ij(int64_t p, int* i, int* j) {
  int64_t ii = (int64_t)((1.0 + sqrt(1.0 + 8.0 * (double)p)) * 0.5);
  while (ii * (ii - 1) / 2 > p) --ii;
  while ((ii + 1) * ii / 2 <= p) ++ii;
  *i = (int)ii;
  *j = (int)(p - ii * (ii - 1) / 2);
}

struct VgEmpArgs {
  int32_t n_steps;
  const int64_t* pt_off;
  const double *x, *y, *z;
  const int64_t* pair_off;
  const int64_t* bkt_off;
  const double* dmax;
  int32_t nk;
  double mdr;
  spi_vg_emp_ws_t ws;
  const int64_t* bin_off;
  double *bin_h, *bin_g, *bin_n;
  int32_t* n_bins;
  double* max_dist;
};

__device__ __forceinline__ double pair_dist(const VgEmpArgs& A, int64_t po, int i, int j) {
  double dx = __dsub_rn(A.x[po + i], A.x[po + j]);
  double dy = __dsub_rn(A.y[po + i], A.y[po + j]);
  return __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
}

__device__ __forceinline__ int64_t bucket_of(double d, double dmax, int64_t nb) {
  int64_t b = (int64_t)(d / dmax * (double)nb);
  return b < 0 ? 0 : (b >= nb ? nb - 1 : b);
}

__global__ void k_pair_dist(VgEmpArgs A) {
  const int s = blockIdx.y;
  const int64_t P = A.pair_off[s + 1] - A.pair_off[s];
  const int64_t nb = A.bkt_off[s + 1] - A.bkt_off[s];
  const int64_t po = A.pt_off[s];
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P;
       p += (int64_t)gridDim.x * blockDim.x) {
    int i, j;
    pair_ij(p, &i, &j);
    double d = pair_dist(A, po, i, j);
    A.ws.pd[A.pair_off[s] + p] = d;
    atomicAdd(&A.ws.bcnt[A.bkt_off[s] + bucket_of(d, A.dmax[s], nb)], 1);
  }
}

__global__ void k_bucket_scan(VgEmpArgs A) {
  const int s = blockIdx.x;
  const int64_t b0 = A.bkt_off[s], nb = A.bkt_off[s + 1] - b0;
  __shared__ int warp_sum[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t base = 0; base < nb; base += blockDim.x) {
    const int64_t b = base + threadIdx.x;
    int v = b < nb ? A.ws.bcnt[b0 + b] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += t;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = lane < nw ? warp_sum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      if (lane < nw) warp_sum[lane] = w;
    }
    __syncthreads();
    const int excl = carry + (warp ? warp_sum[warp - 1] : 0) + x - v;
    if (b < nb) {
      A.ws.bstart[b0 + b] = excl;
      A.ws.bcur[b0 + b] = excl;
    }
    __syncthreads();
    if (threadIdx.x == 0) carry += warp_sum[nw - 1];
    __syncthreads();
  }
}

__global__ void k_pair_scatter(VgEmpArgs A) {
  const int s = blockIdx.y;
  const int64_t P = A.pair_off[s + 1] - A.pair_off[s];
  const int64_t nb = A.bkt_off[s + 1] - A.bkt_off[s];
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P;
       p += (int64_t)gridDim.x * blockDim.x) {
    double d = A.ws.pd[A.pair_off[s] + p];
    int pos = atomicAdd(&A.ws.bcur[A.bkt_off[s] + bucket_of(d, A.dmax[s], nb)], 1);
    A.ws.pp[A.pair_off[s] + pos] = (int32_t)p;
  }
}

// each bucket sorted by (distance, pair index): deterministic, exact order
__global__ void k_bucket_sort(VgEmpArgs A) {
  const int s = blockIdx.y;
  const int64_t nb = A.bkt_off[s + 1] - A.bkt_off[s];
  const int64_t poff = A.pair_off[s];
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nb;
       b += (int64_t)gridDim.x * blockDim.x) {
    const int64_t st = A.ws.bstart[A.bkt_off[s] + b];
    const int64_t cnt = A.ws.bcnt[A.bkt_off[s] + b];
    int32_t* seg = A.ws.pp + poff + st;
    const double* pd = A.ws.pd + poff;
    // key order: (distance, pair index)
    auto less = [&](int32_t a, int32_t b) {
      const double da = pd[a], db = pd[b];
      return da < db || (da == db && a < b);
    };
    if (cnt <= 32) {
      for (int64_t k = 1; k < cnt; ++k) {
        int32_t key = seg[k];
        int64_t m = k - 1;
        while (m >= 0 && less(key, seg[m])) {
          seg[m + 1] = seg[m];
          --m;
        }
        seg[m + 1] = key;
      }
    } else {
      // heap sort: O(cnt log cnt) even when degenerate geometry (equal
      // distances) puts many pairs into one bucket
      auto sift = [&](int64_t root, int64_t end) {
        while (2 * root + 1 < end) {
          int64_t c = 2 * root + 1;
          if (c + 1 < end && less(seg[c], seg[c + 1])) ++c;
          if (!less(seg[root], seg[c])) return;
          int32_t t = seg[root];
          seg[root] = seg[c];
          seg[c] = t;
          root = c;
        }
      };
      for (int64_t r = cnt / 2 - 1; r >= 0; --r) sift(r, cnt);
      for (int64_t e = cnt - 1; e > 0; --e) {
        int32_t t = seg[0];
        seg[0] = seg[e];
        seg[e] = t;
        sift(0, e);
      }
    }
    for (int64_t k = 0; k < cnt; ++k) A.ws.sd[poff + st + k] = A.ws.pd[poff + seg[k]];
  }
}

// mdr cut-off and equal-count bins, one CTA per step
__global__ void k_vg_bins(VgEmpArgs A) {
  const int s = blockIdx.x;
  const int64_t P = A.pair_off[s + 1] - A.pair_off[s];
  const double* sd = A.ws.sd + A.pair_off[s];
  const int32_t* pp = A.ws.pp + A.pair_off[s];
  const int64_t po = A.pt_off[s];
  __shared__ int64_t K;
  if (threadIdx.x == 0) {
    int64_t keep = P;
    double md = 0.0;
    if (P > 0) {
      const double act_max = sd[P - 1];
      md = act_max * A.mdr;
      // first index of the minimum |d - max_dist| (sorted: around the
      // lower bound of max_dist)
      int64_t lo = 0, hi = P;
      while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (sd[mid] < md) lo = mid + 1; else hi = mid;
      }
      int64_t idx = lo < P ? lo : P - 1;
      if (lo > 0 && !(fabs(sd[lo - 1] - md) > fabs(sd[idx] - md))) idx = lo - 1;
      // ties of equal distances: the first of them
      while (idx > 0 && sd[idx - 1] == sd[idx]) --idx;
      double clip_ul = sd[idx];
      if (!(clip_ul - md > 0)) clip_ul = md;
      if (idx != P - 1) {
        lo = 0;
        hi = P;
        while (lo < hi) {
          int64_t mid = (lo + hi) >> 1;
          if (sd[mid] < clip_ul) lo = mid + 1; else hi = mid;
        }
        keep = lo;
      }
    }
    K = keep;
    A.max_dist[s] = md;
    const int64_t nb = (keep + A.nk - 1) / A.nk;
    A.n_bins[s] = (int32_t)nb;
  }
  __syncthreads();
  const int64_t nbins = (K + A.nk - 1) / A.nk;
  const int64_t bo = A.bin_off[s];
  for (int64_t m = threadIdx.x; m < nbins; m += blockDim.x) {
    const int64_t a0 = m * A.nk;
    const int cnt = (int)min((int64_t)A.nk, K - a0);
    double h = np_pairwise_sum(cnt, [&](int k) { return sd[a0 + k]; });
    double sq = np_pairwise_sum(cnt, [&](int k) {
      int i, j;
      pair_ij(pp[a0 + k], &i, &j);
      return __dsqrt_rn(fabs(__dsub_rn(A.z[po + i], A.z[po + j])));
    });
    double e = pow4_rn(__ddiv_rn(sq, (double)cnt));
    e = __ddiv_rn(__ddiv_rn(e, __dadd_rn(0.457, __ddiv_rn(0.494, (double)cnt))), 2.0);
    A.bin_h[bo + m] = __ddiv_rn(h, (double)cnt);
    A.bin_g[bo + m] = e;
    A.bin_n[bo + m] = (double)cnt;
  }
}

// ---------------------------------------------------------------- DE
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double urand(uint64_t seed, uint64_t a, uint64_t b, uint64_t c) {
  uint64_t h = mix64(seed ^ mix64(a * 0x100000001b3ull ^ mix64(b * 0xcbf29ce484222325ull ^ c)));
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// fitting models of vgs.py:553-595, arg = (range r, sill s), FP32
__device__ __forceinline__ float fit_model(int code, float h, float r, float s) {
  switch (code) {
    case SPI_VG_NUG:
      return s;
    case SPI_VG_SPH: {
      if (h > r) return s;
      float t = h / r;
      return s * (1.5f * t - 0.5f * t * t * t);
    }
    case SPI_VG_EXP:
      return s * (1.0f - expf(-3.0f * (h / r)));
    case SPI_VG_LIN:
      return h > r ? s : s * (h / r);
    case SPI_VG_GAU: {
      float t = h / r;
      return s * (1.0f - expf(-3.0f * t * t));
    }
    case SPI_VG_POW:
      return s * powf(h, r);
    case SPI_VG_HOL: {
      if (!(h > 0.f)) return 0.f;
      float a = (float)SPI_PI * h / r;
      return s * (1.0f - sinf(a) / a);
    }
    default:
      return 0.f;
  }
}
__device__ double fit_model_f64(int code, double h, double r, double s) {
  switch (code) {
    case SPI_VG_NUG:
      return s;
    case SPI_VG_SPH: {
      if (h > r) return s;
      double a = (1.5 * h) / r, b = (h * h * h) / (2 * r * r * r);
      return s * (a - b);
    }
    case SPI_VG_EXP:
      return s * (1 - exp(-3 * (h / r)));
    case SPI_VG_LIN:
      return h > r ? s : s * (h / r);
    case SPI_VG_GAU:
      return s * (1 - exp(-3 * ((h * h) / (r * r))));
    case SPI_VG_POW:
      return s * pow(h, r);
    case SPI_VG_HOL: {
      if (!(h > 0)) return 0;
      double a = (SPI_PI * h) / r;
      return s * (1 - (sin(a) / a));
    }
    default:
      return 0;
  }
}

// ---- proposal refinement for the learned warm start (no counterpart in
// the reference) ----
// For a permutation with one free structure (X, or Nug fixed at (h_0,
// gamma_0) + X) the sill is a linear parameter: for a fixed range its
// least-squares value is sum(rho (g - base)) / sum(rho^2), clipped to the
// sill bounds. The range is searched on a log grid around the proposal,
// then refined by golden section on the best bracket.
constexpr int RF_T = 256;
constexpr int RF_GRID = 32;
constexpr int RF_GOLD = 40;

__device__ void block_sum3(double& a, double& b, double& c, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) {
    red[w * 3] = a;
    red[w * 3 + 1] = b;
    red[w * 3 + 2] = c;
  }
  __syncthreads();
  a = b = c = 0.0;
  for (int k = 0; k < RF_T / 32; ++k) {
    a += red[k * 3];
    b += red[k * 3 + 1];
    c += red[k * 3 + 2];
  }
}

__global__ __launch_bounds__(RF_T) void k_vg_refine(int n_prob, const spi_de_problem_t* prob,
                                                    const int64_t* bin_off, const int32_t* n_bins,
                                                    const double* bin_h, const double* bin_g,
                                                    const double* r0, double span, double* out_x,
                                                    double* out_f, double* noise) {
  const int p = blockIdx.x;
  const spi_de_problem_t P = prob[p];
  const int64_t off = bin_off[P.step];
  const int nb = n_bins[P.step];
  const double* h = bin_h + off;
  const double* g = bin_g + off;
  __shared__ double red[RF_T / 32 * 3];
  const int tid = threadIdx.x;
  const double nan = __longlong_as_double(0x7ff8000000000000LL);
  // bin noise: sum of squares of the scatter, from successive differences
  double dd = 0.0, u0 = 0.0, u1 = 0.0;
  for (int i = tid; i + 1 < nb; i += RF_T) {
    const double t = g[i + 1] - g[i];
    dd += t * t;
  }
  block_sum3(dd, u0, u1, red);
  const bool fixed = P.fixed_first && P.n_comp == 2;
  const bool ok = nb > 0 && (P.n_comp == 1 || fixed);
  if (!ok) {
    if (tid < 4) out_x[p * 4 + tid] = nan;
    if (tid == 0) {
      out_f[p] = nan;
      noise[p] = nb > 2 ? 0.5 * dd * nb / (nb - 1) : 0.0;
    }
    return;
  }
  const double h0 = h[0], g0 = g[0];
  const int code = fixed ? P.code[1] : P.code[0];
  const double base = fixed ? g0 : 0.0;
  const double slo = 1e-5, shi = P.var2;
  // profile objective at log-range u: (objective, sill)
  auto prof = [&](double u, double& sill) -> double {
    const double r = exp(u);
    double srr = 0.0, srg = 0.0, sgg = 0.0;
    for (int i = tid; i < nb; i += RF_T) {
      const double rho = code == SPI_VG_NUG ? 1.0 : fit_model_f64(code, h[i], r, 1.0);
      const double y = g[i] - base;
      srr += rho * rho;
      srg += rho * y;
      sgg += y * y;
    }
    block_sum3(srr, srg, sgg, red);
    double sl = srr > 0.0 ? srg / srr : slo;
    sl = fmin(fmax(sl, slo), shi);
    sill = sl;
    return sgg - 2.0 * sl * srg + sl * sl * srr;
  };
  double ulo = log(fmax(h0, 1e-300)), uhi = log(1e9);
  const double uc = log(fmax(r0[p], 1e-300));
  if (code != SPI_VG_NUG && isfinite(uc) && span > 1.0) {
    const double ls = log(span);
    const double a = fmax(ulo, uc - ls), b = fmin(uhi, uc + ls);
    if (a < b) {
      ulo = a;
      uhi = b;
    }
  }
  double best_u = ulo, best_f = 1e300, sill = slo;
  if (code == SPI_VG_NUG) {
    best_f = prof(ulo, sill);
  } else {
    int bk = 0;
    for (int k = 0; k < RF_GRID; ++k) {
      const double u = ulo + (uhi - ulo) * k / (RF_GRID - 1);
      double sl;
      const double f = prof(u, sl);
      if (f < best_f) {
        best_f = f;
        bk = k;
      }
    }
    // golden section on the bracket around the best grid point
    const double step = (uhi - ulo) / (RF_GRID - 1);
    double a = ulo + step * max(bk - 1, 0), b = ulo + step * min(bk + 1, RF_GRID - 1);
    const double gr = 0.6180339887498949;
    double c = b - gr * (b - a), d = a + gr * (b - a), sc, sd;
    double fc = prof(c, sc), fd = prof(d, sd);
    for (int it = 0; it < RF_GOLD; ++it) {
      if (fc < fd) {
        b = d;
        d = c;
        fd = fc;
        c = b - gr * (b - a);
        fc = prof(c, sc);
      } else {
        a = c;
        c = d;
        fc = fd;
        d = a + gr * (b - a);
        fd = prof(d, sd);
      }
    }
    best_u = 0.5 * (a + b);
  }
  const double r = code == SPI_VG_NUG ? h0 : exp(best_u);
  prof(code == SPI_VG_NUG ? ulo : best_u, sill);
  // the objective at the result, summed directly (no expansion)
  double f = 0.0, z0 = 0.0, z1 = 0.0;
  for (int i = tid; i < nb; i += RF_T) {
    const double m = base + fit_model_f64(code, h[i], r, sill);
    const double t = g[i] - m;
    f += t * t;
  }
  block_sum3(f, z0, z1, red);
  if (tid == 0) {
    double* x = out_x + p * 4;
    if (fixed) {
      x[0] = h0;
      x[1] = g0;
      x[2] = r;
      x[3] = sill;
    } else {
      x[0] = r;
      x[1] = sill;
      x[2] = 0.0;
      x[3] = 0.0;
    }
    out_f[p] = f;
    noise[p] = nb > 2 ? 0.5 * dd * nb / (nb - 1) : 0.0;
  }
}

constexpr int DE_T = 256;
constexpr int DE_MAXNP = 800;    // 50 * 4^2
constexpr int DE_MAXBINS = 16384;   // bins kept in shared memory (more: read from L2)

struct DeArgs {
  int32_t n_prob;
  const spi_de_problem_t* prob;
  const int64_t* bin_off;
  const int32_t* n_bins;
  const double *bin_h, *bin_g;
  int32_t maxiter;
  double tol;
  double* best_x;
  double* best_f;
  int32_t* n_gen;
};

__global__ __launch_bounds__(DE_T) void k_de(DeArgs A) {
  const int q = blockIdx.x;
  const spi_de_problem_t P = A.prob[q];
  if (P.n_comp < 1 || P.n_comp > 2 || A.n_bins[P.step] < 1) {
    // unsupported problem size or no bins: no fit
    if (threadIdx.x == 0) {
      for (int j = 0; j < 4; ++j) A.best_x[(int64_t)q * 4 + j] = __longlong_as_double(0x7ff8000000000000LL);
      A.best_f[q] = __longlong_as_double(0x7ff8000000000000LL);
      A.n_gen[q] = 0;
    }
    return;
  }
  const int D = 2 * P.n_comp;
  const int NP = 50 * D * D;
  const int tid = threadIdx.x;
  extern __shared__ __align__(16) unsigned char sm[];
  double* pop = reinterpret_cast<double*>(sm);           // [NP][4] unit cube
  double* tri = pop + DE_MAXNP * 4;                       // [NP][4]
  double* E = tri + DE_MAXNP * 4;                          // [NP]
  double* Et = E + DE_MAXNP;                               // [NP]
  float* hb = reinterpret_cast<float*>(Et + DE_MAXNP);     // [nb]
  float* gb = hb + DE_MAXBINS;                             // [nb]
  __shared__ double lo[4], sc[4];
  __shared__ double red[DE_T];
  __shared__ int redi[DE_T];
  __shared__ int best, stop;
  __shared__ double Fsh;
  const int64_t bo = A.bin_off[P.step];
  const int nb = A.n_bins[P.step];
  const bool bins_in_smem = nb <= DE_MAXBINS;
  if (bins_in_smem)
    for (int b = tid; b < nb; b += DE_T) {
      hb[b] = (float)A.bin_h[bo + b];
      gb[b] = (float)A.bin_g[bo + b];
    }
  if (tid == 0) {
    // bounds of vgs.py:731-753
    const double h0 = A.bin_h[bo], g0 = A.bin_g[bo];
    for (int k = 0; k < P.n_comp; ++k) {
      double rl, rh, sl, shh;
      if (P.code[k] == SPI_VG_POW) {
        rl = 1e-5; rh = 2; sl = 1e-5; shh = P.var2;
      } else if (P.fixed_first && k == 0) {
        rl = rh = h0; sl = shh = g0;
      } else {
        rl = h0; rh = 1e9; sl = 1e-5; shh = P.var2;
      }
      lo[2 * k] = rl; sc[2 * k] = rh - rl;
      lo[2 * k + 1] = sl; sc[2 * k + 1] = shh - sl;
    }
    stop = 0;
  }
  __syncthreads();
  auto energy = [&](const double* u) -> float {
    float r[2], s[2];
    for (int k = 0; k < P.n_comp; ++k) {
      r[k] = (float)(lo[2 * k] + u[2 * k] * sc[2 * k]);
      s[k] = (float)(lo[2 * k + 1] + u[2 * k + 1] * sc[2 * k + 1]);
    }
    float acc = 0.f, cmp = 0.f;
    for (int b = 0; b < nb; ++b) {
      const float hv = bins_in_smem ? hb[b] : (float)A.bin_h[bo + b];
      const float gv = bins_in_smem ? gb[b] : (float)A.bin_g[bo + b];
      float m = 0.f;
      for (int k = 0; k < P.n_comp; ++k) m += fit_model(P.code[k], hv, r[k], s[k]);
      float d = gv - m;
      // compensated sum
      float y = d * d - cmp;
      float t = acc + y;
      cmp = (t - acc) - y;
      acc = t;
    }
    return acc;
  };
  // initial population: Latin hypercube, or the warm-start box
  for (int i = tid; i < NP; i += DE_T)
    for (int j = 0; j < 4; ++j) pop[i * 4 + j] = 0.0;
  __syncthreads();
  if (tid < D) {
    const int j = tid;
    // stratum i of dimension j goes to member perm(i): Fisher-Yates
    int* perm = reinterpret_cast<int*>(tri) + j * DE_MAXNP;  // scratch
    for (int i = 0; i < NP; ++i) perm[i] = i;
    for (int i = NP - 1; i > 0; --i) {
      int k = (int)(urand(P.seed, 0, j, i) * (i + 1));
      int t = perm[i];
      perm[i] = perm[k];
      perm[k] = t;
    }
    double wl = 0.0, ww = 1.0;
    if (P.warm) {
      wl = P.warm_lo[j];
      ww = P.warm_hi[j] - P.warm_lo[j];
    }
    for (int i = 0; i < NP; ++i) {
      double u = (i + urand(P.seed, 1, j, i)) / NP;
      pop[perm[i] * 4 + j] = wl + u * ww;
    }
  }
  __syncthreads();
  for (int i = tid; i < NP; i += DE_T) E[i] = energy(pop + i * 4);
  __syncthreads();
  int gen = 0;
  for (gen = 1; gen <= A.maxiter; ++gen) {
    // best member (first of the minimum energy)
    double bv = __longlong_as_double(0x7ff0000000000000LL);
    int bi = 0x7fffffff;
    for (int i = tid; i < NP; i += DE_T)
      if (E[i] < bv || (E[i] == bv && i < bi)) { bv = E[i]; bi = i; }
    red[tid] = bv;
    redi[tid] = bi;
    __syncthreads();
    for (int o = DE_T / 2; o > 0; o >>= 1) {
      if (tid < o && (red[tid + o] < red[tid] ||
                      (red[tid + o] == red[tid] && redi[tid + o] < redi[tid]))) {
        red[tid] = red[tid + o];
        redi[tid] = redi[tid + o];
      }
      __syncthreads();
    }
    if (tid == 0) {
      best = redi[0];
      Fsh = 0.5 + 0.5 * urand(P.seed, 2, gen, 0);
    }
    __syncthreads();
    const double F = Fsh;
    const double* pb = pop + best * 4;
    for (int i = tid; i < NP; i += DE_T) {
      // two distinct members other than i (bounded redraws)
      int r1 = (int)(urand(P.seed, 3, gen, (uint64_t)i * 64) * NP);
      for (int c = 1; c < 32 && r1 == i; ++c) r1 = (int)(urand(P.seed, 3, gen, (uint64_t)i * 64 + c) * NP);
      if (r1 == i) r1 = (i + 1) % NP;
      int r2 = (int)(urand(P.seed, 7, gen, (uint64_t)i * 64) * NP);
      for (int c = 1; c < 32 && (r2 == i || r2 == r1); ++c)
        r2 = (int)(urand(P.seed, 7, gen, (uint64_t)i * 64 + c) * NP);
      if (r2 == i || r2 == r1) r2 = (max(i, r1) + 1) % NP == min(i, r1) ? (max(i, r1) + 2) % NP : (max(i, r1) + 1) % NP;
      const int jr = (int)(urand(P.seed, 4, gen, i) * D);
      for (int j = 0; j < 4; ++j) {
        double v = pop[i * 4 + j];
        if (j < D && (urand(P.seed, 5, gen, (uint64_t)i * 4 + j) < 0.7 || j == jr)) {
          v = pb[j] + F * (pop[r1 * 4 + j] - pop[r2 * 4 + j]);
          if (v < 0.0 || v > 1.0) v = urand(P.seed, 6, gen, (uint64_t)i * 4 + j);
        }
        tri[i * 4 + j] = v;
      }
      Et[i] = energy(tri + i * 4);
    }
    __syncthreads();
    for (int i = tid; i < NP; i += DE_T)
      if (Et[i] <= E[i]) {
        E[i] = Et[i];
        for (int j = 0; j < 4; ++j) pop[i * 4 + j] = tri[i * 4 + j];
      }
    __syncthreads();
    // convergence: std(E) <= tol * |mean(E)|
    double s1 = 0.0;
    for (int i = tid; i < NP; i += DE_T) s1 += E[i];
    red[tid] = s1;
    __syncthreads();
    for (int o = DE_T / 2; o > 0; o >>= 1) {
      if (tid < o) red[tid] += red[tid + o];
      __syncthreads();
    }
    const double mean = red[0] / NP;
    __syncthreads();
    double s2 = 0.0;
    for (int i = tid; i < NP; i += DE_T) s2 += (E[i] - mean) * (E[i] - mean);
    red[tid] = s2;
    __syncthreads();
    for (int o = DE_T / 2; o > 0; o >>= 1) {
      if (tid < o) red[tid] += red[tid + o];
      __syncthreads();
    }
    if (tid == 0) stop = sqrt(red[0] / NP) <= A.tol * fabs(mean);
    __syncthreads();
    if (stop) break;
  }
  // best member, its FP64 objective
  double bv = __longlong_as_double(0x7ff0000000000000LL);
  int bi = 0x7fffffff;
  for (int i = tid; i < NP; i += DE_T)
    if (E[i] < bv || (E[i] == bv && i < bi)) { bv = E[i]; bi = i; }
  red[tid] = bv;
  redi[tid] = bi;
  __syncthreads();
  for (int o = DE_T / 2; o > 0; o >>= 1) {
    if (tid < o && (red[tid + o] < red[tid] ||
                    (red[tid + o] == red[tid] && redi[tid + o] < redi[tid]))) {
      red[tid] = red[tid + o];
      redi[tid] = redi[tid + o];
    }
    __syncthreads();
  }
  const int b = redi[0];
  __syncthreads();
  double x[4];
  for (int j = 0; j < 4; ++j) x[j] = (j < D) ? lo[j] + pop[b * 4 + j] * sc[j] : 0.0;
  double part = 0.0;
  for (int k = tid; k < A.n_bins[P.step]; k += DE_T) {
    double h = A.bin_h[bo + k];
    double m = 0.0;
    for (int c = 0; c < P.n_comp; ++c) m += fit_model_f64(P.code[c], h, x[2 * c], x[2 * c + 1]);
    double d = A.bin_g[bo + k] - m;
    part += d * d;
  }
  red[tid] = part;
  __syncthreads();
  for (int o = DE_T / 2; o > 0; o >>= 1) {
    if (tid < o) red[tid] += red[tid + o];
    __syncthreads();
  }
  if (tid == 0) {
    for (int j = 0; j < 4; ++j) A.best_x[(int64_t)q * 4 + j] = x[j];
    A.best_f[q] = red[0];
    A.n_gen[q] = gen > A.maxiter ? A.maxiter : gen;
  }
}

}  // namespace spi

using namespace spi;

extern "C" int spi_vg_empirical(int32_t n_steps, const int64_t* pt_off, const double* x,
                                const double* y, const double* z, const int64_t* pair_off,
                                const int64_t* bkt_off, const double* dmax, int64_t max_pairs,
                                int64_t max_buckets, int32_t nk, double mdr,
                                const spi_vg_emp_ws_t* ws, const int64_t* bin_off,
                                double* bin_h, double* bin_g, double* bin_n, int32_t* n_bins,
                                double* max_dist, spi_stream_t stream) {
  if (n_steps < 0 || nk < 1 || !(mdr > 0) || max_pairs < 0 || max_buckets < 0) return SPI_ERR_ARG;
  if (n_steps == 0) return SPI_OK;
  if (n_steps > 65535) return SPI_ERR_TOO_LARGE;
  if (!pt_off || !x || !y || !z || !pair_off || !bkt_off || !dmax || !ws || !ws->pd || !ws->pp ||
      !ws->sd || !ws->bcnt || !ws->bstart || !ws->bcur || !bin_off || !bin_h || !bin_g ||
      !bin_n || !n_bins || !max_dist)
    return SPI_ERR_ARG;
  VgEmpArgs A{n_steps, pt_off, x, y, z, pair_off, bkt_off, dmax, nk, mdr, *ws, bin_off,
              bin_h, bin_g, bin_n, n_bins, max_dist};
  cudaStream_t st = (cudaStream_t)stream;
  unsigned gp = (unsigned)std::min<int64_t>((max_pairs + 255) / 256 + 1, 4096);
  unsigned gb = (unsigned)std::min<int64_t>((max_buckets + 255) / 256 + 1, 4096);
  k_pair_dist<<<dim3(gp, n_steps), 256, 0, st>>>(A);
  SPI_LAUNCH_CHECK();
  k_bucket_scan<<<n_steps, 1024, 0, st>>>(A);
  SPI_LAUNCH_CHECK();
  k_pair_scatter<<<dim3(gp, n_steps), 256, 0, st>>>(A);
  SPI_LAUNCH_CHECK();
  k_bucket_sort<<<dim3(gb, n_steps), 256, 0, st>>>(A);
  SPI_LAUNCH_CHECK();
  k_vg_bins<<<n_steps, 256, 0, st>>>(A);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

extern "C" int spi_vg_de(int32_t n_prob, const spi_de_problem_t* prob, const int64_t* bin_off,
                         const int32_t* n_bins, const double* bin_h, const double* bin_g,
                         int32_t maxiter, double tol, double* best_x, double* best_f,
                         int32_t* n_gen, spi_stream_t stream) {
  if (n_prob < 0 || maxiter < 1 || !(tol >= 0)) return SPI_ERR_ARG;
  if (n_prob == 0) return SPI_OK;
  if (!prob || !bin_off || !n_bins || !bin_h || !bin_g || !best_x || !best_f || !n_gen)
    return SPI_ERR_ARG;
  size_t smem = (size_t)DE_MAXNP * 4 * 8 * 2 + (size_t)DE_MAXNP * 8 * 2 + (size_t)DE_MAXBINS * 4 * 2;
  if (cudaFuncSetAttribute(k_de, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return SPI_ERR_CUDA;
  DeArgs A{n_prob, prob, bin_off, n_bins, bin_h, bin_g, maxiter, tol, best_x, best_f, n_gen};
  k_de<<<n_prob, DE_T, smem, (cudaStream_t)stream>>>(A);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

extern "C" int spi_vg_refine(int32_t n_prob, const spi_de_problem_t* prob, const int64_t* bin_off,
                             const int32_t* n_bins, const double* bin_h, const double* bin_g,
                             const double* r0, double span, double* x, double* f, double* noise,
                             spi_stream_t stream) {
  if (n_prob < 0 || !(span >= 1.0)) return SPI_ERR_ARG;
  if (n_prob == 0) return SPI_OK;
  if (!prob || !bin_off || !n_bins || !bin_h || !bin_g || !r0 || !x || !f || !noise)
    return SPI_ERR_ARG;
  k_vg_refine<<<n_prob, RF_T, 0, (cudaStream_t)stream>>>(n_prob, prob, bin_off, n_bins, bin_h,
                                                        bin_g, r0, span, x, f, noise);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
