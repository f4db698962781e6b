// Kernels of the driver flow around the step engine (interp/main.py,
// interp/prepare.py): the polygon cell mask and the per-step statistics.
//
// k_pts_in_polys: the cells to interpolate, as _select_nearby_cells selects
// them (interp/prepare.py:250-288 over misc.py:407-500, 617-627): a cell is
// kept when it lies strictly inside one of the polygons (ogr's Contains:
// boundary points are outside), after its coordinates went through
// "POINT (%f %f)", i.e. were rounded to 1e-6. Each polygon is one ring (the
// reference asserts GetGeometryCount() == 1), closed implicitly from its
// last vertex to its first. Crossing number with the half-open rule; the
// orientation of a point against an edge is a*b - c*d with both products
// split exactly by FMA, and a zero orientation inside the edge's box means
// the point is on the boundary.
//
// k_stats_partial / k_stats_final: min, mean, max, std and count of every
// row of a [rows, n] field over its finite entries (interp/main.py:474-525:
// pandas' skip-NaN statistics of the station data, ddof 1, and numpy's
// nanmin / nanmean / nanmax / nanstd / isfinite().sum() of each
// interpolated field, ddof 0). FP64 accumulation of count, sum and sum of
// squares per thread, blocks of a row combined in a second launch.
#include "spi_common.cuh"

namespace spi {

constexpr int PT = 256;          // points per CTA
constexpr int PCH = 1024;        // polygon vertices staged per chunk
constexpr int ST = 256;          // threads of a statistics CTA

__device__ __forceinline__ double round_1e6(double v) {
  // the value "%f" prints, read back: nearest multiple of 1e-6
  return rint(v * 1e6) / 1e6;
}

// sign of a*b - c*d, with both products split exactly
__device__ __forceinline__ int orient_sign(double a, double b, double c, double d) {
  const double p = a * b, q = c * d;
  const double ep = fma(a, b, -p), eq = fma(c, d, -q);
  const double r = (p - q) + (ep - eq);
  return (r > 0.0) - (r < 0.0);
}

__global__ __launch_bounds__(PT) void k_pts_in_polys(const double* __restrict__ px,
                                                     const double* __restrict__ py, int64_t n_pts,
                                                     int32_t n_polys,
                                                     const int64_t* __restrict__ ring_off,
                                                     const double* __restrict__ vx,
                                                     const double* __restrict__ vy,
                                                     const double* __restrict__ bbox,
                                                     uint8_t* __restrict__ inside) {
  __shared__ double sx[PCH + 1], sy[PCH + 1];
  __shared__ double rb[4][PT / 32];
  __shared__ double cb[4];
  const int tid = threadIdx.x;
  const int64_t i = (int64_t)blockIdx.x * PT + tid;
  const bool valid = i < n_pts;
  double x = 0.0, y = 0.0;
  if (valid) {
    x = round_1e6(px[i]);
    y = round_1e6(py[i]);
  }
  // the CTA's bounding box, to skip polygons far from every point
  double b0 = valid ? x : INFINITY, b1 = valid ? x : -INFINITY;
  double b2 = valid ? y : INFINITY, b3 = valid ? y : -INFINITY;
  for (int o = 16; o > 0; o >>= 1) {
    b0 = fmin(b0, __shfl_xor_sync(0xffffffffu, b0, o));
    b1 = fmax(b1, __shfl_xor_sync(0xffffffffu, b1, o));
    b2 = fmin(b2, __shfl_xor_sync(0xffffffffu, b2, o));
    b3 = fmax(b3, __shfl_xor_sync(0xffffffffu, b3, o));
  }
  if ((tid & 31) == 0) {
    rb[0][tid >> 5] = b0;
    rb[1][tid >> 5] = b1;
    rb[2][tid >> 5] = b2;
    rb[3][tid >> 5] = b3;
  }
  __syncthreads();
  if (tid == 0) {
    for (int w = 1; w < PT / 32; ++w) {
      b0 = fmin(b0, rb[0][w]);
      b1 = fmax(b1, rb[1][w]);
      b2 = fmin(b2, rb[2][w]);
      b3 = fmax(b3, rb[3][w]);
    }
    cb[0] = b0;
    cb[1] = b1;
    cb[2] = b2;
    cb[3] = b3;
  }
  __syncthreads();
  bool hit = false;
  for (int p = 0; p < n_polys; ++p) {
    const double* bb = bbox + 4 * p;  // x_min, x_max, y_min, y_max
    if (bb[0] > cb[1] || bb[1] < cb[0] || bb[2] > cb[3] || bb[3] < cb[2]) continue;
    const bool mine = valid && !hit && x >= bb[0] && x <= bb[1] && y >= bb[2] && y <= bb[3];
    const int64_t v0 = ring_off[p], v1 = ring_off[p + 1];
    const int64_t nv = v1 - v0;
    bool odd = false, onb = false;
    for (int64_t c0 = 0; c0 < nv; c0 += PCH) {
      const int cn = (int)min((int64_t)PCH, nv - c0);
      __syncthreads();
      for (int q = tid; q <= cn; q += PT) {
        // vertex c0 + q, and the ring's first vertex after its last
        const int64_t g = (c0 + q < nv) ? v0 + c0 + q : v0;
        sx[q] = vx[g];
        sy[q] = vy[g];
      }
      __syncthreads();
      if (mine && !onb)
        for (int e = 0; e < cn; ++e) {
          const double x1 = sx[e], y1 = sy[e], x2 = sx[e + 1], y2 = sy[e + 1];
          const bool up1 = y1 > y, up2 = y2 > y;
          const bool inbox = x >= fmin(x1, x2) && x <= fmax(x1, x2) && y >= fmin(y1, y2) &&
                             y <= fmax(y1, y2);
          if (up1 == up2 && !inbox) continue;
          const int s = orient_sign(x2 - x1, y - y1, y2 - y1, x - x1);
          if (s == 0 && inbox) {
            onb = true;
            break;
          }
          if (up1 != up2 && ((y2 > y1) ? (s > 0) : (s < 0))) odd = !odd;
        }
    }
    if (mine && odd && !onb) hit = true;
  }
  if (valid) inside[i] = hit ? 1 : 0;
}

template <typename T>
__global__ __launch_bounds__(ST) void k_stats_partial(const T* __restrict__ fld, int64_t n,
                                                      int64_t ld, int nb,
                                                      double* __restrict__ part) {
  const int row = blockIdx.y, b = blockIdx.x;
  const T* r = fld + (int64_t)row * ld;
  double cnt = 0.0, s = 0.0, q = 0.0, mn = INFINITY, mx = -INFINITY;
  for (int64_t j = (int64_t)b * ST + threadIdx.x; j < n; j += (int64_t)nb * ST) {
    const double v = (double)r[j];
    if (isfinite(v)) {
      cnt += 1.0;
      s += v;
      q = fma(v, v, q);
      mn = fmin(mn, v);
      mx = fmax(mx, v);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    s += __shfl_xor_sync(0xffffffffu, s, o);
    q += __shfl_xor_sync(0xffffffffu, q, o);
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  __shared__ double red[5][ST / 32];
  if ((threadIdx.x & 31) == 0) {
    const int w = threadIdx.x >> 5;
    red[0][w] = cnt;
    red[1][w] = s;
    red[2][w] = q;
    red[3][w] = mn;
    red[4][w] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < ST / 32; ++w) {
      cnt += red[0][w];
      s += red[1][w];
      q += red[2][w];
      mn = fmin(mn, red[3][w]);
      mx = fmax(mx, red[4][w]);
    }
    double* o = part + ((int64_t)row * nb + b) * 5;
    o[0] = cnt;
    o[1] = s;
    o[2] = q;
    o[3] = mn;
    o[4] = mx;
  }
}

// out[row] = (min, mean, max, std, count); NaN statistics for an empty row,
// std NaN where count <= ddof
__global__ void k_stats_final(const double* __restrict__ part, int rows, int nb, int ddof,
                              double* __restrict__ out) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= rows) return;
  double cnt = 0.0, s = 0.0, q = 0.0, mn = INFINITY, mx = -INFINITY;
  for (int b = 0; b < nb; ++b) {
    const double* p = part + ((int64_t)row * nb + b) * 5;
    cnt += p[0];
    s += p[1];
    q += p[2];
    mn = fmin(mn, p[3]);
    mx = fmax(mx, p[4]);
  }
  const double nan = __longlong_as_double(0x7ff8000000000000LL);
  double* o = out + (int64_t)row * 5;
  if (cnt == 0.0) {
    o[0] = o[1] = o[2] = o[3] = nan;
    o[4] = 0.0;
    return;
  }
  const double mean = s / cnt;
  const double m2 = fmax(0.0, q - s * mean);
  o[0] = mn;
  o[1] = mean;
  o[2] = mx;
  o[3] = (cnt > ddof) ? sqrt(m2 / (cnt - ddof)) : nan;
  o[4] = cnt;
}

// numpy.round(a, decimals) in a's own precision (interp/steps.py:899-901,
// 920-922 before the fields are written): y = a * 10^d, rint (half to even),
// y / 10^d; for d < 0 the division and product swap.
template <typename T>
__global__ void k_round(T* __restrict__ a, int64_t n, T f, int neg) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T v = a[i];
    T y = neg ? v / f : v * f;
    y = rint(y);
    a[i] = neg ? y * f : y / f;
  }
}

}  // namespace spi

extern "C" int spi_round_fields(void* fld, int32_t is_f64, int64_t n, int32_t decimals,
                                spi_stream_t stream) {
  if (n < 0 || decimals < -300 || decimals > 300) return SPI_ERR_ARG;
  if (n == 0) return SPI_OK;
  if (!fld) return SPI_ERR_ARG;
  const int neg = decimals < 0;
  const int d = neg ? -decimals : decimals;
  double f = 1.0;
  for (int k = 0; k < d; ++k) f *= 10.0;  // exact up to 10^22
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t want = (n + 255) / 256;
  const unsigned blocks = (unsigned)(want < 152 * 32 ? want : 152 * 32);
  if (is_f64)
    spi::k_round<double><<<blocks, 256, 0, st>>>((double*)fld, n, f, neg);
  else
    spi::k_round<float><<<blocks, 256, 0, st>>>((float*)fld, n, (float)f, neg);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

extern "C" int spi_points_in_polygons(const double* px, const double* py, int64_t n_pts,
                                      int32_t n_polys, const int64_t* ring_off,
                                      const double* vx, const double* vy, const double* bbox,
                                      uint8_t* inside, spi_stream_t stream) {
  if (n_pts < 0 || n_polys < 0) return SPI_ERR_ARG;
  if (n_pts == 0) return SPI_OK;
  if (!px || !py || !inside || (n_polys > 0 && (!ring_off || !vx || !vy || !bbox)))
    return SPI_ERR_ARG;
  const int64_t blocks = (n_pts + spi::PT - 1) / spi::PT;
  if (blocks > 0x7fffffff) return SPI_ERR_TOO_LARGE;
  spi::k_pts_in_polys<<<(unsigned)blocks, spi::PT, 0, (cudaStream_t)stream>>>(
      px, py, n_pts, n_polys, ring_off, vx, vy, bbox, inside);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

extern "C" int spi_field_stats(const void* fld, int32_t is_f64, int32_t rows, int64_t n,
                               int64_t ld, int32_t ddof, double* scratch, int64_t scratch_len,
                               double* out, spi_stream_t stream) {
  if (rows < 0 || n < 0 || ld < n || ddof < 0) return SPI_ERR_ARG;
  if (rows == 0) return SPI_OK;
  if (!fld || !scratch || !out) return SPI_ERR_ARG;
  if (rows > 65535) return SPI_ERR_TOO_LARGE;
  // enough blocks per row to cover the GPU about four times
  int64_t nb = (4 * 152 + rows - 1) / rows;
  const int64_t need = (n + spi::ST - 1) / spi::ST;
  if (nb > need) nb = need;
  if (nb < 1) nb = 1;
  if (scratch_len < (int64_t)rows * nb * 5) return SPI_ERR_WORKSPACE;
  cudaStream_t st = (cudaStream_t)stream;
  dim3 grid((unsigned)nb, (unsigned)rows);
  if (is_f64)
    spi::k_stats_partial<double><<<grid, spi::ST, 0, st>>>((const double*)fld, n, ld, (int)nb,
                                                           scratch);
  else
    spi::k_stats_partial<float><<<grid, spi::ST, 0, st>>>((const float*)fld, n, ld, (int)nb,
                                                          scratch);
  SPI_LAUNCH_CHECK();
  spi::k_stats_final<<<(rows + 127) / 128, 128, 0, st>>>(scratch, rows, (int)nb, ddof, out);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
