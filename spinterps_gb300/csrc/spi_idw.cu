// Inverse distance weighting and nearest neighbour over all cells and steps.
//
// Replaces the IDW and NNB branches of SpInterpSteps._get_interp
// (interp/steps.py:285-313) and cyth fill_wts_and_sum / get_mults_sum
// (cyth/interpmthds.pyx:784-808). The reference normalises each cell's
// distances by their maximum over the step group's stations before
// w = 1/d^p; that scale cancels in sum(w z) / sum(w), so here each cell's
// weights W[i] = (d_i / d_ref)^-p are computed once against ALL stations
// (d_ref = the cell's nearest non-zero station distance, which keeps the
// weights <= 1 and free of overflow) and every step is a masked
// contraction pair over stations (the "masked GEMM pair"):
//   num_j = sum_i W[i] m_ji z_ji,  den_j = sum_i W[i] m_ji,  est = num/den,
// with m_ji = 1 where station i has a value at step j. Stations missing at
// a step contribute exactly nothing, as when the reference leaves them out
// of the group. A cell lying on a station present at the step gets NaN
// (the reference's 1/0 weight); steps below min_value_to_interp_thresh get
// the step mean.
#include "spi_common.cuh"
#include "spi_contract.cuh"

namespace spi {

struct IdwArgs {
  spi_domain_t dom;
  int32_t n_steps;
  const int32_t* steps;
  const int32_t* out_row;
  const double* data;    // [T, N], NaN = missing
  const float* data_hi;  // FP32 (hi, lo) pair of data (precision 1)
  const float* data_lo;
  const uint8_t* flag;   // [T]
  const double* means;   // [T]
  double p;
  spi_out_t out;
};

// B loaders: vector 2k = masked values of step k, 2k+1 = its mask.
struct MaskLoader64 {
  const double* data;
  const int32_t* steps;
  int64_t n_stns;
  int v0;
  __device__ __forceinline__ double operator()(int v, int j) const {
    const int k = (v0 + v) >> 1;
    double x = data[(int64_t)steps[k] * n_stns + j];
    bool have = !isnan(x);
    return (v & 1) ? (have ? 1.0 : 0.0) : (have ? x : 0.0);
  }
};
struct MaskLoader32 {
  const float* hi;
  const float* lo;
  const int32_t* steps;
  int64_t n_stns;
  int v0;
  __device__ __forceinline__ float2 operator()(int v, int j) const {
    const int k = (v0 + v) >> 1;
    const int64_t e = (int64_t)steps[k] * n_stns + j;
    float h = hi[e];
    bool have = !isnan(h);
    if (v & 1) return make_float2(have ? 1.f : 0.f, 0.f);
    return have ? make_float2(h, lo[e]) : make_float2(0.f, 0.f);
  }
};

template <typename T, int TC, typename OutT>
__global__ __launch_bounds__(CT) void k_idw(IdwArgs A, int npad) {
  constexpr int CPT = TC / 16;
  const int64_t C = A.dom.n_cells;
  const int64_t N = A.dom.n_stns;
  const int64_t c0 = (int64_t)blockIdx.x * TC;
  if (c0 >= C) return;
  const int tid = threadIdx.x;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* W = reinterpret_cast<T*>(smraw);                          // [npad][TC]
  T* Bs = W + (int64_t)npad * TC;                              // KC * BSTR doubles
  double* dref = reinterpret_cast<double*>(Bs) + KC * BSTR;    // [TC]
  double* red = dref + TC;                                     // [CT]
  int* onst = reinterpret_cast<int*>(red + CT);                // [TC]
  int* redi = onst + TC;                                       // [CT]

  const int cell = tid % TC, jg = tid / TC, njg = CT / TC;
  const int64_t gc = c0 + cell;
  const bool live = gc < C;
  // ---- 1. reference distance: nearest non-zero; first on-station index ----
  double dmin = __longlong_as_double(0x7ff0000000000000LL);
  int on = 0x7fffffff;
  float4 cp = make_float4(0.f, 0.f, 0.f, 0.f);
  double cx = 0.0, cy = 0.0;
  if (live) {
    if constexpr (sizeof(T) == 8) {
      cx = A.dom.cell_x[gc];
      cy = A.dom.cell_y[gc];
    } else {
      cp = reinterpret_cast<const float4*>(A.dom.cell_split)[gc];
    }
  }
  const float4* sp4 = reinterpret_cast<const float4*>(A.dom.stn_split);
  auto dist_to = [&](int j) -> double {
    if constexpr (sizeof(T) == 8) {
      return dist_f64(cx, cy, A.dom.stn_x[j], A.dom.stn_y[j]);
    } else {
      const float4 sp = sp4[j];
      float dx = (cp.x - sp.x) + (cp.y - sp.y);
      float dy = (cp.z - sp.z) + (cp.w - sp.w);
      return (double)sqrtf(dx * dx + dy * dy);
    }
  };
  if (live) {
    for (int j = jg; j < N; j += njg) {
      double d = dist_to(j);
      if (d == 0.0) {
        if (j < on) on = j;
      } else if (d < dmin) {
        dmin = d;
      }
    }
  }
  red[tid] = dmin;
  redi[tid] = on;
  __syncthreads();
  if (tid < TC) {
    double b = red[tid];
    int o = redi[tid];
    for (int g = 1; g < njg; ++g) {
      b = fmin(b, red[g * TC + tid]);
      o = min(o, redi[g * TC + tid]);
    }
    dref[tid] = b;
    onst[tid] = (o == 0x7fffffff) ? -1 : o;
  }
  __syncthreads();
  // ---- 2. weights W[j][cell] = (d / d_ref)^-p, 0 on a station ----
  {
    const double dr = dref[cell];
    for (int j = jg; j < npad; j += njg) {
      T w = T(0);
      if (live && j < N) {
        double d = dist_to(j);
        if (d != 0.0) {
          if constexpr (sizeof(T) == 8) {
            double r = d / dr;
            w = (A.p == 2.0) ? 1.0 / (r * r) : (A.p == 1.0 ? 1.0 / r : 1.0 / pow(r, A.p));
          } else {
            float r = (float)d / (float)dr;
            float pf = (float)A.p;
            w = (pf == 2.0f) ? 1.0f / (r * r) : (pf == 1.0f ? 1.0f / r : exp2f(-pf * log2f(r)));
          }
        }
      }
      W[(int64_t)j * TC + cell] = w;
    }
  }
  // ---- 3. masked contraction pair, 32 steps (64 vectors) per block ----
  OutT* est_out = reinterpret_cast<OutT*>(A.out.est);
  const int cg = tid % 16, rg = tid / 16;
  for (int k0 = 0; k0 < A.n_steps; k0 += VB / 2) {
    const int nk = min(VB / 2, A.n_steps - k0);
    double acc[CPT][4];
    if constexpr (sizeof(T) == 8)
      tile_contract<T, TC, true>(W, Bs, MaskLoader64{A.data, A.steps, N, 2 * k0}, 2 * nk,
                                 (int)N, (int)N, acc);
    else
      tile_contract<T, TC, true>(W, Bs, MaskLoader32{A.data_hi, A.data_lo, A.steps, N, 2 * k0},
                                 2 * nk, (int)N, (int)N, acc);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int k = rg * 2 + h;
      if (k >= nk) continue;
      const int j = A.steps[k0 + k];
      const int64_t row = A.out_row[k0 + k];
#pragma unroll
      for (int c = 0; c < CPT; ++c) {
        const int cl = cg * CPT + c;
        const int64_t g = c0 + cl;
        if (g >= C) continue;
        double e;
        if (!A.flag[j]) {
          e = A.means[j];
        } else {
          int o = onst[cl];
          if (o >= 0 && !isnan(A.data[(int64_t)j * N + o])) {
            e = __longlong_as_double(0x7ff8000000000000LL);
          } else {
            e = acc[c][2 * h] / acc[c][2 * h + 1];
          }
        }
        e = clip_est(e, A.out);
        est_out[row * C + g] = cast_out<OutT>(e);
      }
    }
  }
}

// NNB: per cell the FP64 distances to all stations are kept in shared
// memory; per step the first present station of minimum distance is
// taken (np.argmin over the step's stations in ascending station order).
// Distances are non-negative doubles, compared through their bit patterns.
template <int TC, typename OutT>
__global__ __launch_bounds__(CT) void k_nnb(IdwArgs A) {
  const int64_t C = A.dom.n_cells, N = A.dom.n_stns;
  const int64_t c0 = (int64_t)blockIdx.x * TC;
  if (c0 >= C) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  unsigned long long* D = reinterpret_cast<unsigned long long*>(smraw);  // [N][TC]
  const int tid = threadIdx.x;
  for (int64_t e = tid; e < N * TC; e += CT) {
    int j = (int)(e / TC), cl = (int)(e % TC);
    int64_t g = c0 + cl;
    double d = g < C ? dist_f64(A.dom.cell_x[g], A.dom.cell_y[g], A.dom.stn_x[j], A.dom.stn_y[j])
                     : 0.0;
    D[e] = (unsigned long long)__double_as_longlong(d);
  }
  __syncthreads();
  OutT* est_out = reinterpret_cast<OutT*>(A.out.est);
  const int cl = tid % TC;
  const int64_t g = c0 + cl;
  for (int k = tid / TC; k < A.n_steps; k += CT / TC) {
    if (g >= C) continue;
    const int j = A.steps[k];
    const double* z = A.data + (int64_t)j * N;
    unsigned long long best = ~0ull;
    int bi = -1;
    for (int i = 0; i < N; ++i) {
      unsigned long long d = D[(int64_t)i * TC + cl];
      if (d < best && !isnan(z[i])) {
        best = d;
        bi = i;
      }
    }
    double e = bi >= 0 ? z[bi] : __longlong_as_double(0x7ff8000000000000LL);
    e = clip_est(e, A.out);
    est_out[(int64_t)A.out_row[k] * C + g] = cast_out<OutT>(e);
  }
}

template <typename OutT>
__global__ void k_fill_rows(int32_t n_rows, const int32_t* __restrict__ row,
                            const double* __restrict__ v, const double* __restrict__ vv,
                            int64_t C, spi_out_t o) {
  OutT* est = reinterpret_cast<OutT*>(o.est);
  OutT* var = reinterpret_cast<OutT*>(o.var);
  for (int r = blockIdx.y; r < n_rows; r += gridDim.y) {
    const double e = clip_est(v[r], o);
    const int64_t base = (int64_t)row[r] * C;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C;
         c += (int64_t)gridDim.x * blockDim.x) {
      est[base + c] = cast_out<OutT>(e);
      if (var && vv) var[base + c] = cast_out<OutT>(vv[r]);
    }
  }
}

template <typename T, int TC>
static size_t idw_smem(int npad) {
  return (size_t)npad * TC * sizeof(T) + (size_t)KC * BSTR * 8 + (size_t)TC * 8 +
         (size_t)CT * 8 + (size_t)TC * 4 + (size_t)CT * 4 + 16;
}

template <typename T, int TC, typename OutT>
static int launch_idw(const IdwArgs& A, cudaStream_t st) {
  int npad = (int)((A.dom.n_stns + KC - 1) / KC * KC);
  size_t smem = idw_smem<T, TC>(npad);
  auto kern = k_idw<T, TC, OutT>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return SPI_ERR_CUDA;
  int64_t tiles = (A.dom.n_cells + TC - 1) / TC;
  kern<<<(unsigned)tiles, CT, smem, st>>>(A, npad);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

template <typename T, typename OutT>
static int dispatch_idw(const IdwArgs& A, cudaStream_t st) {
  int npad = (int)((A.dom.n_stns + KC - 1) / KC * KC);
  const size_t cap = 225 * 1024;
  if (sizeof(T) == 4 && idw_smem<T, 64>(npad) <= cap) return launch_idw<T, 64, OutT>(A, st);
  if (idw_smem<T, 32>(npad) <= cap) return launch_idw<T, 32, OutT>(A, st);
  if (idw_smem<T, 16>(npad) <= cap) return launch_idw<T, 16, OutT>(A, st);
  return SPI_ERR_TOO_LARGE;
}

}  // namespace spi

using namespace spi;

static int idw_args(IdwArgs& A, const spi_domain_t* dom, int32_t n_steps, const int32_t* steps,
                    const int32_t* out_row, const double* data, const spi_out_t* out) {
  if (!dom || !out || n_steps < 0) return SPI_ERR_ARG;
  if (n_steps == 0 || dom->n_cells == 0) return 1;
  if (!steps || !out_row || !data || !out->est || dom->n_stns <= 0) return SPI_ERR_ARG;
  if (dom->n_stns > 0x7fffffff) return SPI_ERR_TOO_LARGE;
  A.dom = *dom;
  A.n_steps = n_steps;
  A.steps = steps;
  A.out_row = out_row;
  A.data = data;
  A.out = *out;
  return 0;
}

extern "C" int spi_idw_cells(const spi_domain_t* dom, int32_t n_steps, const int32_t* steps,
                             const int32_t* out_row, const double* data, const float* data_hi,
                             const float* data_lo, const uint8_t* flag, const double* means,
                             double idw_exp, int32_t precision, const spi_out_t* out,
                             spi_stream_t stream) {
  IdwArgs A;
  int rc = idw_args(A, dom, n_steps, steps, out_row, data, out);
  if (rc == 1) return SPI_OK;
  if (rc) return rc;
  if (!flag || !means) return SPI_ERR_ARG;
  if (precision == 1 && (!dom->stn_split || !dom->cell_split || !data_hi || !data_lo))
    return SPI_ERR_ARG;
  if (precision != 0 && precision != 1) return SPI_ERR_ARG;
  A.flag = flag;
  A.means = means;
  A.p = idw_exp;
  A.data_hi = data_hi;
  A.data_lo = data_lo;
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == 0)
    return out->out_f64 ? dispatch_idw<double, double>(A, st) : dispatch_idw<double, float>(A, st);
  return out->out_f64 ? dispatch_idw<float, double>(A, st) : dispatch_idw<float, float>(A, st);
}

extern "C" int spi_nnb_cells(const spi_domain_t* dom, int32_t n_steps, const int32_t* steps,
                             const int32_t* out_row, const double* data, const spi_out_t* out,
                             spi_stream_t stream) {
  IdwArgs A;
  int rc = idw_args(A, dom, n_steps, steps, out_row, data, out);
  if (rc == 1) return SPI_OK;
  if (rc) return rc;
  A.flag = nullptr;
  A.means = nullptr;
  A.p = 0.0;
  constexpr int TC = 16;
  size_t smem = (size_t)dom->n_stns * TC * 8;
  if (smem > 225 * 1024) return SPI_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  int64_t tiles = (dom->n_cells + TC - 1) / TC;
  if (out->out_f64) {
    if (cudaFuncSetAttribute(k_nnb<TC, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return SPI_ERR_CUDA;
    k_nnb<TC, double><<<(unsigned)tiles, CT, smem, st>>>(A);
  } else {
    if (cudaFuncSetAttribute(k_nnb<TC, float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
      return SPI_ERR_CUDA;
    k_nnb<TC, float><<<(unsigned)tiles, CT, smem, st>>>(A);
  }
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

extern "C" int spi_fill_rows(int32_t n_rows, const int32_t* row, const double* v,
                             const double* vv, int64_t n_cells, const spi_out_t* out,
                             spi_stream_t stream) {
  if (!out || n_rows < 0 || n_cells < 0) return SPI_ERR_ARG;
  if (n_rows == 0 || n_cells == 0) return SPI_OK;
  if (!row || !v || !out->est) return SPI_ERR_ARG;
  dim3 grid((unsigned)((n_cells + 255) / 256 < 1024 ? (n_cells + 255) / 256 : 1024),
            (unsigned)(n_rows < 65535 ? n_rows : 65535));
  if (out->out_f64)
    k_fill_rows<double><<<grid, 256, 0, (cudaStream_t)stream>>>(n_rows, row, v, vv, n_cells, *out);
  else
    k_fill_rows<float><<<grid, 256, 0, (cudaStream_t)stream>>>(n_rows, row, v, vv, n_cells, *out);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
