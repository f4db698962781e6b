// The OK variance term |Linv c|^2 of every cell in double-float on the FP32
// pipe: the mixed path's second FP32 tier, for systems whose tensor-core
// variance (spi_var_tc.cu, FP32 accumulation in tensor memory, ~1e-6 of the
// sill) misses the probe's tolerance. Here every product of the double-float
// right-hand side (rhs_df, ~1e-9) and Linv's FP32 (hi, lo) pair is split
// exactly by FMA and accumulated by TwoSum, so the sum carries ~2^-45
// relative error and the result ~1e-9 of the sill: FP64-level for the
// estimate and the variance, at ~12 FP32 operations per term against one
// FMA on GB300's 1/64-rate FP64 pipe.
//
// One CTA = 32 cells x 256 threads; rows of Linv go in blocks of 64, the
// stations (K) in chunks of 32 staged in shared memory: the cells' double-
// float right-hand sides (c_h, c_l [k][cell]) and the block's rows of Linv
// (l_h, l_l [k][row], triangular). Thread t owns cells 2 (t % 16) + {0, 1}
// and rows 4 (t / 16) + {0..3} of the block: 8 double-float accumulators.
// After a block, each thread adds the squares of its 8 values to its two
// cells' double-float sums; the 16 row groups are summed at the end.
#include "spi_cells.cuh"
#include "spi_rhs.cuh"

namespace spi {

constexpr int VD_C = 32;    // cells per CTA
constexpr int VD_R = 64;    // Linv rows per block
constexpr int VD_K = 32;    // stations per chunk
constexpr int VD_T = 256;   // threads

struct VarDfArgs {
  spi_domain_t dom;
  spi_systems_t sys;
  spi_krige_ws_t ws;
  double cond_cap;
};

__device__ __forceinline__ bool var_df_system(const spi_krige_ws_t& ws, int s, double cap) {
  if (ws.tier) return ws.tier[s] == 2;
  return ws.route[s] == 0 && ws.cond[s] <= cap;
}

// acc += a * b for double-floats a and b (b given as its FP32 pair)
__device__ __forceinline__ void df_fma_acc(df& acc, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  const df s = two_sum(acc.h, p);
  acc.h = s.h;
  acc.l = __fadd_rn(acc.l, __fadd_rn(s.l, e));
}

__global__ __launch_bounds__(VD_T) void k_var_df(VarDfArgs A) {
  const int s = blockIdx.y;
  const int64_t C = A.dom.n_cells;
  const int64_t c0 = (int64_t)blockIdx.x * VD_C;
  if (c0 >= C) return;
  if (A.sys.kind == SPI_KIND_SK) return;
  if (!var_df_system(A.ws, s, A.cond_cap)) return;
  const int64_t soff = A.sys.stn_off[s];
  const int n = (int)(A.sys.stn_off[s + 1] - soff);
  const int32_t* idx = A.sys.stn_idx + soff;
  const int64_t moff = A.sys.mat_off[s];
  const double sh = A.ws.shift[s];
  const float* Lh = A.ws.linv_hi + moff;
  const float* Ll = A.ws.linv_lo + moff;

  // (row stride of l_*: VD_R + 4 floats, 16-byte rows with 4-way store conflicts)
  __shared__ __align__(16) float c_h[VD_K][VD_C];
  __shared__ __align__(16) float c_l[VD_K][VD_C];
  __shared__ __align__(16) float l_h[VD_K][VD_R + 4];
  __shared__ __align__(16) float l_l[VD_K][VD_R + 4];
  __shared__ double part[VD_T / (VD_C / 2)][VD_C];
  __shared__ RhsDf kd;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) kd.init(A.sys.vg[s], sh, A.dom.min_vg_val);
  // staging role: this lane's cell for the right-hand sides
  const int64_t gc = c0 + lane;
  const bool live = gc < C;
  const float4 cp = live ? reinterpret_cast<const float4*>(A.dom.cell_split)[gc]
                         : make_float4(0.f, 0.f, 0.f, 0.f);
  const spi_vg_t* vgp = A.sys.vg + s;
  const float4* sp4 = reinterpret_cast<const float4*>(A.dom.stn_split);
  // contraction role
  const int cg = tid & 15, rg = tid >> 4;
  df yy0 = {0.f, 0.f}, yy1 = {0.f, 0.f};
  __syncthreads();

  for (int rb = 0; rb < n; rb += VD_R) {
    const int kend = min(n, rb + VD_R);
    df u[2][4];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
      for (int r = 0; r < 4; ++r) u[c][r] = df{0.f, 0.f};
    for (int k0 = 0; k0 < kend; k0 += VD_K) {
      __syncthreads();
      // right-hand sides: warp w stages stations k0 + w, w + 8, ... for
      // the 32 cells (a lane per cell)
      for (int k = warp; k < VD_K; k += VD_T / 32) {
        const int j = k0 + k;
        df c = {0.f, 0.f};
        if (live && j < n) c = rhs_df(A.dom, vgp, kd, 0, sh, cp, sp4[idx[j]], gc, idx + j);
        c_h[k][lane] = c.h;
        c_l[k][lane] = c.l;
      }
      // the block's rows of Linv (lower triangular: zero above the diagonal)
      for (int e = tid; e < VD_R * VD_K; e += VD_T) {
        const int r = e / VD_K, k = e % VD_K;
        const int row = rb + r, col = k0 + k;
        float vh = 0.f, vl = 0.f;
        if (row < n && col <= row) {
          vh = Lh[(int64_t)row * n + col];
          vl = Ll[(int64_t)row * n + col];
        }
        l_h[k][r] = vh;
        l_l[k][r] = vl;
      }
      __syncthreads();
      const int kn = min(VD_K, kend - k0);
      for (int k = 0; k < kn; ++k) {
        const float2 ah = *reinterpret_cast<const float2*>(&c_h[k][2 * cg]);
        const float2 al = *reinterpret_cast<const float2*>(&c_l[k][2 * cg]);
        const float4 bh = *reinterpret_cast<const float4*>(&l_h[k][4 * rg]);
        const float4 bl = *reinterpret_cast<const float4*>(&l_l[k][4 * rg]);
        const float bhv[4] = {bh.x, bh.y, bh.z, bh.w};
        const float blv[4] = {bl.x, bl.y, bl.z, bl.w};
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          df_fma_acc(u[0][r], ah.x, al.x, bhv[r], blv[r]);
          df_fma_acc(u[1][r], ah.y, al.y, bhv[r], blv[r]);
        }
      }
    }
    // squares of this block's values into the cells' sums
#pragma unroll
    for (int r = 0; r < 4; ++r) {
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const df v = u[c][r];
        const float p = __fmul_rn(v.h, v.h);
        const float e = __fmaf_rn(v.h, v.h, -p) + 2.0f * v.h * v.l;
        df& y = c ? yy1 : yy0;
        const df t = two_sum(y.h, p);
        y.h = t.h;
        y.l = __fadd_rn(y.l, __fadd_rn(t.l, e));
      }
    }
  }
  part[rg][2 * cg] = (double)yy0.h + (double)yy0.l;
  part[rg][2 * cg + 1] = (double)yy1.h + (double)yy1.l;
  __syncthreads();
  if (tid < VD_C && c0 + tid < C) {
    double t = 0.0;
    for (int g = 0; g < VD_T / (VD_C / 2); ++g) t += part[g][tid];
    A.ws.cell_yy[(int64_t)s * C + c0 + tid] = t;
  }
}

}  // namespace spi

using namespace spi;

extern "C" int spi_krige_var_df(const spi_domain_t* dom, const spi_systems_t* sys,
                                const spi_krige_ws_t* ws, double cond_cap, spi_stream_t stream) {
  if (!dom || !sys || !ws) return SPI_ERR_ARG;
  if (sys->n_sys < 0 || sys->n_sys > 65535) return SPI_ERR_TOO_LARGE;
  if (sys->n_sys == 0 || dom->n_cells == 0) return SPI_OK;
  if (!ws->cell_yy || !ws->linv_hi || !ws->linv_lo || !ws->route || !ws->cond || !ws->shift ||
      !dom->cell_split || !dom->stn_split || !sys->vg || !sys->stn_off || !sys->stn_idx ||
      !sys->mat_off)
    return SPI_ERR_ARG;
  const int64_t tiles = (dom->n_cells + VD_C - 1) / VD_C;
  if (tiles > 0x7fffffff) return SPI_ERR_TOO_LARGE;
  VarDfArgs A{*dom, *sys, *ws, cond_cap};
  dim3 grid((unsigned)tiles, (unsigned)sys->n_sys);
  k_var_df<<<grid, VD_T, 0, (cudaStream_t)stream>>>(A);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
