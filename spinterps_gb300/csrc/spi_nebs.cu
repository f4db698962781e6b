// Neighbour selection of every destination cell among a set of reference
// stations: SpInterpNeighborGrouping's 'nrst' and 'pie' methods
// (interp/grps.py:147-247 with cyth/interpmthds.pyx:811-890), one thread per
// destination, results as each destination's sorted station indices.
//
// nrst: the n_nebs nearest (FP64 distances, the correctly rounded root as
// numpy's ** 0.5), kept in an insertion-sorted list by (distance, index);
// an FP32 bound skips the stations that cannot enter it (k_neb_nrst).
// pie: every station's angle from the destination by the reference's rules
// (atan(dy / dx), pushed into [0, 2 pi) for dx < 0 or dy < 0 -- dx == 0
// gives 0, and dx < 0 with dy == 0 stays 0), its pie
// int(angle * n_pies / 2 pi), its rank by distance within its pie; the
// stations ordered by (rank, distance) -- the nearest of every pie first --
// and the first n_nebs taken. Each pie keeps only its n_nebs nearest (rank
// n_nebs and beyond is never taken).
//
// Ties: the reference orders equal distances with numpy's (unstable)
// argsort; here they order by index. A pie index that rounds up to n_pies
// (an angle within an ulp of 2 pi, where the reference writes past its
// count array) is taken as the last pie.
#include "spi_common.cuh"

namespace spi {

constexpr int NEB_MAX = 64;
constexpr int NEB_PIE_SLOTS = 512;   // n_pies * n_nebs

__device__ __forceinline__ bool neb_less(double da, int ia, double db, int ib) {
  return da < db || (da == db && ia < ib);
}

// insert (d, i) into the ascending list (ld, li) of length *len (cap k)
__device__ __forceinline__ void neb_insert(double* ld, int* li, int* len, int k, double d, int i) {
  int n = *len;
  if (n == k && !neb_less(d, i, ld[n - 1], li[n - 1])) return;
  int p = (n == k) ? n - 1 : n;
  while (p > 0 && neb_less(d, i, ld[p - 1], li[p - 1])) {
    ld[p] = ld[p - 1];
    li[p] = li[p - 1];
    --p;
  }
  ld[p] = d;
  li[p] = i;
  if (n < k) *len = n + 1;
}

__device__ __forceinline__ void sort_ints(int* a, int n) {
  for (int i = 1; i < n; ++i) {
    int v = a[i], p = i;
    while (p > 0 && a[p - 1] > v) {
      a[p] = a[p - 1];
      --p;
    }
    a[p] = v;
  }
}

// nrst: every destination's k nearest by (FP64 distance, index). The
// stations pass through shared memory in tiles as FP32 coordinates relative
// to station 0, with |x| + |y| beside them. Once a destination holds k
// stations, a station whose FP32 squared distance exceeds lim^2,
//   lim = thr (1 + 1e-5) + 2^-20 (|x_s| + |y_s| + |x_c| + |y_c|),
// thr the current k-th FP64 distance, is skipped: the rounding of the FP32
// coordinates and arithmetic moves a distance by at most 2^-23 (|x_s| + |y_s|
// + |x_c| + |y_c|) plus a few 1e-7 of it, so such a station's FP64 distance
// is above thr and neb_insert would reject it whatever its index. thr only
// falls during the scan, so the skipped stations stay out and the selection
// equals the FP64 scan of every station. The others take dist_f64 and
// neb_insert as before.
constexpr int NRST_T = 128;      // threads per CTA
constexpr int NRST_TILE = 1024;  // stations per shared-memory tile
constexpr float kNrstRel = 1.00001f;
constexpr float kNrstAbs = 9.5367431640625e-07f;  // 2^-20

__global__ __launch_bounds__(NRST_T) void k_neb_nrst(const double* __restrict__ dx_,
                                                     const double* __restrict__ dy_,
                                                     int64_t n_dst,
                                                     const double* __restrict__ rx,
                                                     const double* __restrict__ ry, int n_ref,
                                                     int k, int32_t* __restrict__ out) {
  __shared__ float4 tile[NRST_TILE];
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const bool act = i < n_dst;
  double ld[NEB_MAX];
  int li[NEB_MAX];
  int len = 0;
  const double ox = rx[0], oy = ry[0];
  const double x = act ? dx_[i] : ox, y = act ? dy_[i] : oy;
  const float xc = (float)(x - ox), yc = (float)(y - oy);
  const float sc = fabsf(xc) + fabsf(yc);
  float lim0 = INFINITY;  // thr (1 + 1e-5) once k stations are held
  for (int t0 = 0; t0 < n_ref; t0 += NRST_TILE) {
    const int tn = min(NRST_TILE, n_ref - t0);
    __syncthreads();
    for (int j = threadIdx.x; j < tn; j += NRST_T) {
      const float xs = (float)(rx[t0 + j] - ox), ys = (float)(ry[t0 + j] - oy);
      tile[j] = make_float4(xs, ys, fabsf(xs) + fabsf(ys), 0.0f);
    }
    __syncthreads();
    if (!act) continue;
    for (int j = 0; j < tn; ++j) {
      const float4 s = tile[j];
      const float ex = s.x - xc, ey = s.y - yc;
      const float lim = fmaf(kNrstAbs, s.z + sc, lim0);
      if (ex * ex + ey * ey > lim * lim) continue;
      const int js = t0 + j;
      neb_insert(ld, li, &len, k, dist_f64(x, y, rx[js], ry[js]), js);
      if (len == k) lim0 = (float)ld[k - 1] * kNrstRel;
    }
  }
  if (!act) return;
  sort_ints(li, len);
  for (int q = 0; q < k; ++q) out[i * k + q] = li[q];
}

__global__ void k_neb_pie(const double* __restrict__ dx_, const double* __restrict__ dy_,
                          int64_t n_dst, const double* __restrict__ rx,
                          const double* __restrict__ ry, int n_ref, int k, int n_pies,
                          int32_t* __restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n_dst) return;
  double pd[NEB_PIE_SLOTS];
  int pi_[NEB_PIE_SLOTS];
  int plen[16];
  for (int p = 0; p < n_pies; ++p) plen[p] = 0;
  const double x = dx_[i], y = dy_[i];
  const double two_pi = 2.0 * SPI_PI;
  for (int j = 0; j < n_ref; ++j) {
    const double xd = rx[j] - x, yd = ry[j] - y;
    double ang;
    if (xd == 0.0) {
      ang = 0.0;
    } else {
      ang = atan(yd / xd);
      if (xd < 0.0 && yd > 0.0)
        ang = SPI_PI + ang;
      else if (xd < 0.0 && yd < 0.0)
        ang = SPI_PI + ang;
      else if (xd > 0.0 && yd < 0.0)
        ang = two_pi + ang;
    }
    int p = (int)(ang * (double)n_pies / two_pi);
    p = min(max(p, 0), n_pies - 1);
    neb_insert(pd + p * k, pi_ + p * k, &plen[p], k, dist_f64(x, y, rx[j], ry[j]), j);
  }
  // the first k by (rank within pie, distance, index)
  int sel[NEB_MAX];
  int ns = 0;
  for (int r = 0; r < k && ns < k; ++r) {
    // this rank's stations, ascending by (distance, index), appended
    double rd[16];
    int ri[16];
    int nr = 0;
    for (int p = 0; p < n_pies; ++p)
      if (plen[p] > r) {
        int q = nr++;
        while (q > 0 && neb_less(pd[p * k + r], pi_[p * k + r], rd[q - 1], ri[q - 1])) {
          rd[q] = rd[q - 1];
          ri[q] = ri[q - 1];
          --q;
        }
        rd[q] = pd[p * k + r];
        ri[q] = pi_[p * k + r];
      }
    for (int q = 0; q < nr && ns < k; ++q) sel[ns++] = ri[q];
  }
  sort_ints(sel, ns);
  for (int q = 0; q < k; ++q) out[i * k + q] = q < ns ? sel[q] : -1;
}

}  // namespace spi

extern "C" int spi_neb_select(int32_t method, const double* dst_x, const double* dst_y,
                              int64_t n_dst, const double* ref_x, const double* ref_y,
                              int32_t n_ref, int32_t n_nebs, int32_t n_pies, int32_t* idxs,
                              spi_stream_t stream) {
  if (n_dst < 0 || n_ref < 1 || n_nebs < 1) return SPI_ERR_ARG;
  if (n_dst == 0) return SPI_OK;
  if (!dst_x || !dst_y || !ref_x || !ref_y || !idxs) return SPI_ERR_ARG;
  const int64_t blocks = (n_dst + 127) / 128;
  if (blocks > 0x7fffffff) return SPI_ERR_TOO_LARGE;
  cudaStream_t st = (cudaStream_t)stream;
  if (method == 1) {
    const int k = n_nebs < n_ref ? n_nebs : n_ref;
    if (k > spi::NEB_MAX) return SPI_ERR_TOO_LARGE;
    spi::k_neb_nrst<<<(unsigned)blocks, spi::NRST_T, 0, st>>>(dst_x, dst_y, n_dst, ref_x,
                                                               ref_y, n_ref, k, idxs);
  } else if (method == 2) {
    if (n_pies < 1 || n_nebs < n_pies || n_ref < n_nebs) return SPI_ERR_ARG;
    if (n_nebs > spi::NEB_MAX || n_pies > 16 || n_pies * n_nebs > spi::NEB_PIE_SLOTS)
      return SPI_ERR_TOO_LARGE;
    spi::k_neb_pie<<<(unsigned)blocks, 128, 0, st>>>(dst_x, dst_y, n_dst, ref_x, ref_y, n_ref,
                                                     n_nebs, n_pies, idxs);
  } else {
    return SPI_ERR_ARG;
  }
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
