// Shared by the cell kernels (spi_cells.cu, spi_cells_stream.cu).
#pragma once
#include "spi_common.cuh"

namespace spi {

constexpr int GA = SPI_MAX_DRIFT + 1;

struct CellsArgs {
  spi_domain_t dom;
  spi_systems_t sys;
  spi_krige_ws_t ws;
  const double* vals;
  int want_var;
  int route_filter;
  double cond_split;
  spi_out_t out;
};

// Exact (FP64, reference-ordered) nearest station of a cell among a
// system's stations: first index of the minimum distance, as np.argmin.
__device__ inline int nnb_f64_warp(const spi_domain_t& dom, const int32_t* idx, int n, double cx,
                            double cy) {
  const int lane = threadIdx.x & 31;
  double best = __longlong_as_double(0x7ff0000000000000LL);
  int bj = 0x7fffffff;
  for (int j = lane; j < n; j += 32) {
    int st = idx[j];
    double d = dist_f64(cx, cy, dom.stn_x[st], dom.stn_y[st]);
    if (d < best) {
      best = d;
      bj = j;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    double ob = __shfl_xor_sync(0xffffffffu, best, o);
    int oj = __shfl_xor_sync(0xffffffffu, bj, o);
    if (ob < best || (ob == best && oj < bj)) {
      best = ob;
      bj = oj;
    }
  }
  return bj == 0x7fffffff ? 0 : bj;
}

// Systems an FP32 tier can take: the Cholesky path, and SK on the
// exact-inverse path (its weights lambda = P c contract the same
// covariances against the dual vectors P 1 and P z; the min_vg_val cut
// makes SK matrices indefinite, so Cholesky fails on many well-conditioned
// ones). OK / EDK keep the exact-inverse path in FP64: there it holds the
// numerically singular systems, whose answers only the same FP64
// arithmetic reproduces.
__device__ __forceinline__ bool fp32_route(int route, int sk) {
  return route == 0 || (sk && route == 1);
}

// The FP32 tier of the precision-1 kernels: the probe's verdict when there
// is one (spi_krige_tier), else an FP32-capable route under cond_split.
__device__ __forceinline__ bool fp32_tier(const spi_krige_ws_t& ws, int s, double cond_split,
                                          int sk) {
  if (ws.tier) return ws.tier[s] != 0;
  return fp32_route(ws.route[s], sk) && ws.cond[s] <= cond_split;
}

// Host-side dispatch of the streamed kernel (spi_cells_stream.cu): systems
// too large for the shared-memory right-hand side of k_krige_cells.
int launch_cells_stream(const CellsArgs& A, int precision, cudaStream_t st);

}  // namespace spi
