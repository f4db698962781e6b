// The OK variance term |Linv c|^2 of every cell on the tensor cores
// (tcgen05, sm_103a), for the FP32-tier systems of the mixed path.
//
// Per system: Y = C Linv' with C the cells' right-hand sides (covariances
// to the system's stations, generated from coordinates) and Linv the
// inverse Cholesky factor; the variance needs yy[cell] = sum_r Y[cell][r]^2
// (n^2 flops per cell, shared by every step of the system; the rest of the
// variance formula is in the cell kernel's FP64 epilogue).
//
// One CTA = 128 cells x 256 threads, two CTAs per SM (each holds 256 of the
// SM's 512 tensor-memory columns). The accumulator D [128 cells x 256 rows
// of Linv] lives in TMEM (lane = cell, column = row), so each lane squares
// and sums its own row of D. Rows of Linv go in blocks of 256 (the MMA's
// N), the stations (K) in chunks of 8, through a three-stage shared-memory
// ring:
//   - B, Linv's rows (256 x 8, triangular) as three TF32 terms (b0 + b1 +
//     b2, ~33 bits: Linv's rounding, amplified by the cancellation in
//     Linv c, dominates the variance's error), and the chunk's 8 stations'
//     split coordinates, are packed once per system in the MMA's tile
//     order (spi_krige_var_tc_pack) and arrive by one bulk copy
//     (cp.async.bulk, 24 KB) per chunk, issued one chunk ahead by one
//     thread and counted on the stage's mbarrier;
//   - A, the cells' right-hand sides (128 x 8), is generated by all threads
//     in FP32 (vt_rhs_f32 for a one-structure variogram, else the head of
//     the double-float rhs_df) from the stations in shared memory and
//     stored as two TF32 terms (a0 + a1, ~22 bits), in the no-swizzle
//     K-major layout (8-row x 16-byte core matrices). A third term (a2 b0, a sixth MMA) leaves the
//     probe's variance discrepancies unchanged: the FP32 accumulation in
//     TMEM, not A's split, bounds this kernel's accuracy.
// One thread issues the chunk's 5 MMAs (a0 b0 + a0 b1 + a1 b0 + a0 b2 +
// a1 b1, K = 8, FP32 accumulation in TMEM) and commits them to the stage's
// mbarrier; the threads go on to the next chunk while they run, and a stage
// is refilled only after the MMAs that read it completed. Every wait is
// bounded: on expiry the kernel raises err_flag, drains the copies and MMAs
// in flight on a best-effort basis (one more bounded wait each), frees its
// TMEM and returns; the probe's tier choice (spi_krige_tier) then keeps
// every system in FP64 and the host raises. Squares are summed in
// double-float (FP32 pairs: the FP64 pipe is 1/64 of FP32 on GB300); the
// mixed path's probe checks every system's variance against the FP64
// kernel.
#include "spi_cells.cuh"
#include "spi_rhs.cuh"
#include "spi_tc.cuh"

namespace spi {

constexpr int VT_M = 128;   // cells per CTA (MMA M, TMEM lanes)
constexpr int VT_N = 256;   // Linv rows per block (MMA N, TMEM columns)
constexpr int VT_KC = SPI_VAR_TC_KC;  // stations per chunk (one MMA K-step)
constexpr int VT_T = 256;   // threads
constexpr int VT_NST = 3;   // ring stages

constexpr size_t VT_A_BYTES = (size_t)VT_M * VT_KC * 4;       // one TF32 term of A
constexpr size_t VT_B_BYTES = (size_t)VT_N * VT_KC * 4;       // one TF32 term of B
constexpr size_t VT_S_BYTES = (size_t)VT_KC * 16;             // the chunk's stations (float4)
constexpr size_t VT_CHUNK_BYTES = 3 * VT_B_BYTES + VT_S_BYTES;  // one packed chunk
constexpr size_t VT_STAGE = 2 * VT_A_BYTES + VT_CHUNK_BYTES;  // A (2 terms), the chunk
constexpr size_t VT_SMEM = VT_NST * VT_STAGE;
constexpr int VT_CHUNK_FLOATS = (int)(VT_CHUNK_BYTES / 4);
static_assert(VT_CHUNK_FLOATS == SPI_VAR_TC_CHUNK_FLOATS, "packed chunk size");
static_assert(VT_KC == 8, "one MMA K-step (TF32: K = 8) per chunk");
static_assert(VT_STAGE % 16 == 0 && VT_CHUNK_BYTES % 16 == 0, "bulk copies: 16-byte units");

struct VarTcArgs {
  spi_domain_t dom;
  spi_systems_t sys;
  spi_krige_ws_t ws;
  double cond_split;
  int32_t* err;
};

// Chunks of VT_KC columns of B in the 256-row block starting at row rb.
__device__ __forceinline__ int vt_chunks(int n, int rb) { return (min(n, rb + VT_N) + VT_KC - 1) / VT_KC; }

// One thread: packed chunk (B and its stations) by one bulk copy into the
// stage, counted on the stage's mbarrier.
__device__ __forceinline__ void vt_load(uint32_t dst, const float* src, uint32_t mbar) {
  tc_bulk_load(dst, src, (uint32_t)VT_CHUNK_BYTES, mbar);
}

// One FP32 right-hand side of a single-structure variogram (CODE: Exp, Gau
// or Sph; kd.single indexes it) for the tensor-core variance. A keeps 22
// bits (two TF32 terms), so an FP32 entry (the distance from the split
// coordinates, the model in FP32 with CUDA's expf: a few 1e-7 relative)
// costs the variance little beside the split and the FP32
// accumulation in TMEM, at under half the instructions of the double-float
// entry. The min_vg_val cut as rhs_df_cut, with a band wide enough for
// FP32 (1e-6 of the cut and of the total sill): entries within it take
// rhs_f64.
template <int CODE>
__device__ __forceinline__ float vt_rhs_f32(const spi_domain_t& dom, const spi_vg_t* vgp,
                                            const RhsDf& kd, double sh, float4 cp, float4 sp,
                                            int64_t gc, const int32_t* stp) {
  const float dx = (cp.x - sp.x) + (cp.y - sp.y);
  const float dy = (cp.z - sp.z) + (cp.w - sp.w);
  const float d2 = __fmaf_rn(dx, dx, dy * dy);
  const int q = kd.single;
  float rho;
  if constexpr (CODE == SPI_VG_GAU) {
    rho = expf(d2 * kd.k2[q].h);
  } else if constexpr (CODE == SPI_VG_EXP) {
    rho = expf(sqrtf(d2) * kd.k1[q].h);
  } else {
    const float t = sqrtf(d2) * kd.inv_r[q].h;  // h / r
    const float u = 1.0f - t;
    rho = t < 1.0f ? u * u * (1.0f + 0.5f * t) : 0.0f;
  }
  const float c = kd.sill[q].h * rho;
  if (kd.mvv > 0.f && !kd.nug_clear) {
    const float gap = (kd.shift.h - c) - kd.mvv;  // gamma against the cut
    if (fabsf(gap) <= 1e-6f * (kd.mvv + kd.shift.h))
      return (float)rhs_f64(dom, *vgp, 0, false, sh, dom.cell_x[gc], dom.cell_y[gc], *stp);
    if (gap <= 0.f) return kd.shift.h;
  }
  return c;
}

// The chunk's right-hand sides of one thread: cell a_cell, stations
// k0 + kb .. k0 + kb + 3 (coordinates from the stage), as two TF32 terms
// into the A tiles. CODE: the single structure's model (vt_rhs_f32), or -1
// (the general double-float rhs_df, its head).
template <int CODE>
__device__ __forceinline__ void vt_gen(const spi_domain_t& dom, const spi_vg_t* vgp,
                                       const RhsDf& kd, double sh, float4 cp, bool live,
                                       int64_t gc, const int32_t* idx, int n, int k0, int kb,
                                       int a_cell, const float4* ssp, unsigned char* sAh,
                                       unsigned char* sAl) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int kk = kb + q, j = k0 + kk;
    float c = 0.f;
    if (live && j < n) {
      if constexpr (CODE < 0)
        c = rhs_df(dom, vgp, kd, 0, sh, cp, ssp[kk], gc, idx + j).h;
      else
        c = vt_rhs_f32<CODE>(dom, vgp, kd, sh, cp, ssp[kk], gc, idx + j);
    }
    float h, l;
    tf32_split(c, h, l);
    const int o = tile_off(VT_M, a_cell, kk);
    *reinterpret_cast<float*>(sAh + o) = h;
    *reinterpret_cast<float*>(sAl + o) = l;
  }
}

__global__ __launch_bounds__(VT_T, 2) void k_var_tc(VarTcArgs A) {
  const int s = blockIdx.y;
  const int64_t C = A.dom.n_cells;
  const int64_t c0 = (int64_t)blockIdx.x * VT_M;
  if (c0 >= C) return;
  if (A.sys.kind == SPI_KIND_SK) return;
  // tier 1 only (tier 2 takes its variance from spi_var_df.cu)
  if (A.ws.tier ? A.ws.tier[s] != 1 : !fp32_tier(A.ws, s, A.cond_split, 0)) return;
  const int64_t soff = A.sys.stn_off[s];
  const int n = (int)(A.sys.stn_off[s + 1] - soff);
  const int32_t* idx = A.sys.stn_idx + soff;
  const spi_vg_t vg = A.sys.vg[s];
  const double sh = A.ws.shift[s];
  const float* pk = A.ws.linv_tc + (int64_t)A.ws.linv_tc_off[s] * VT_CHUNK_FLOATS;
  extern __shared__ __align__(1024) unsigned char smv[];
  __shared__ __align__(8) uint64_t bbar[VT_NST];   // the stage's chunk arrived
  __shared__ __align__(8) uint64_t mbar[VT_NST];   // the stage's MMAs completed
  __shared__ uint32_t tbase;
  __shared__ int fail;
  __shared__ double half_yy[VT_M];
  auto stage = [&](int st) { return smv + st * VT_STAGE; };

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tbase)),
                 "r"(VT_N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  __shared__ RhsDf kd;
  if (tid == 0) {
    fail = 0;
    for (int q = 0; q < VT_NST; ++q) {
      mbar_init(smem_u32(&bbar[q]), 1);
      mbar_init(smem_u32(&mbar[q]), 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;");
    kd.init(vg, sh, A.dom.min_vg_val);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tbase;
  // kind::tf32, D FP32, A/B TF32 K-major, N = 256, M = 128
  const uint32_t idesc = tf32_idesc(VT_M, VT_N);
  // the single structure's model, uniform over the CTA (-1: general form)
  const int scode = (kd.exact && kd.single >= 0) ? kd.code[kd.single] : -1;

  // staging roles: A = cell (tid % 128), stations [kb, kb + 4) of a chunk
  const int a_cell = tid & (VT_M - 1), kb = (tid >> 7) * 4;
  const int64_t gc = c0 + a_cell;
  const bool live = gc < C;
  const float4 cp = live ? reinterpret_cast<const float4*>(A.dom.cell_split)[gc]
                         : make_float4(0.f, 0.f, 0.f, 0.f);
  const spi_vg_t* vgp = A.sys.vg + s;
  // epilogue roles: TMEM lanes of warp % 4, column half warp / 4
  const int e_cell = (warp & 3) * 32 + lane, e_half = warp >> 2;
  df yy = {0.f, 0.f};  // sum of squares, double-float (no FP64 pipe per row)
  int total = 0;  // the system's chunks over all row blocks
  for (int rb = 0; rb < n; rb += VT_N) total += vt_chunks(n, rb);
  // chunk g sits in stage g % 3; each of a stage's mbarriers completes once
  // per use, so chunk g's phase parity is (g / 3) & 1. seen: chunks whose
  // MMAs this thread has seen complete; issued: chunks whose copy thread 0
  // has started (one ahead of the chunk being generated).
  int g = 0, seen = 0, issued = 0;
  auto wait_mma = [&](int upto) {  // MMAs of chunks < upto complete
    while (seen < upto && !fail) {
      if (!mbar_wait_bounded(smem_u32(&mbar[seen % VT_NST]), (uint32_t)((seen / VT_NST) & 1)))
        atomicExch(&fail, 1);
      ++seen;
    }
  };
  if (tid == 0 && total > 0) {
    vt_load(smem_u32(stage(0) + 2 * VT_A_BYTES), pk, smem_u32(&bbar[0]));
    issued = 1;
  }
  for (int rb = 0; rb < n && !fail; rb += VT_N) {
    const int nc = vt_chunks(n, rb);
    for (int kc = 0; kc < nc; ++kc, ++g) {
      const int st = g % VT_NST;
      // chunk g + 1 refills the stage of chunk g - 2: its MMAs must be done
      wait_mma(g - 1);
      __syncthreads();
      if (fail) break;
      if (tid == 0 && g + 1 < total) {
        vt_load(smem_u32(stage((g + 1) % VT_NST) + 2 * VT_A_BYTES),
                pk + (int64_t)(g + 1) * VT_CHUNK_FLOATS, smem_u32(&bbar[(g + 1) % VT_NST]));
        issued = g + 2;
      }
      unsigned char* sAh = stage(st);
      unsigned char* sAl = sAh + VT_A_BYTES;
      unsigned char* sB = sAh + 2 * VT_A_BYTES;
      const float4* ssp = reinterpret_cast<const float4*>(sB + 3 * VT_B_BYTES);
      // chunk g's B and stations (on expiry the stage holds garbage: the
      // right-hand sides below stay in shared memory and the MMAs are not
      // issued)
      if (!mbar_wait_bounded(smem_u32(&bbar[st]), (uint32_t)((g / VT_NST) & 1)))
        atomicExch(&fail, 1);
      const int k0 = kc * VT_KC;
      switch (scode) {
        case SPI_VG_EXP:
          vt_gen<SPI_VG_EXP>(A.dom, vgp, kd, sh, cp, live, gc, idx, n, k0, kb, a_cell, ssp, sAh,
                             sAl);
          break;
        case SPI_VG_GAU:
          vt_gen<SPI_VG_GAU>(A.dom, vgp, kd, sh, cp, live, gc, idx, n, k0, kb, a_cell, ssp, sAh,
                             sAl);
          break;
        case SPI_VG_SPH:
          vt_gen<SPI_VG_SPH>(A.dom, vgp, kd, sh, cp, live, gc, idx, n, k0, kb, a_cell, ssp, sAh,
                             sAl);
          break;
        default:
          vt_gen<-1>(A.dom, vgp, kd, sh, cp, live, gc, idx, n, k0, kb, a_cell, ssp, sAh, sAl);
      }
      asm volatile("fence.proxy.async.shared::cta;");
      __syncthreads();
      if (tid == 0) {
        if (!fail) {
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint64_t ah = umma_desc(smem_u32(sAh), VT_M * 16, 128);
          const uint64_t al = umma_desc(smem_u32(sAl), VT_M * 16, 128);
          const uint32_t b = smem_u32(sB);
          const uint64_t b0 = umma_desc(b, VT_N * 16, 128);
          const uint64_t b1 = umma_desc(b + (uint32_t)VT_B_BYTES, VT_N * 16, 128);
          const uint64_t b2 = umma_desc(b + 2 * (uint32_t)VT_B_BYTES, VT_N * 16, 128);
          mma_tf32(tmem, ah, b0, idesc, kc > 0 ? 1u : 0u);
          mma_tf32(tmem, ah, b1, idesc, 1u);
          mma_tf32(tmem, al, b0, idesc, 1u);
          mma_tf32(tmem, ah, b2, idesc, 1u);
          mma_tf32(tmem, al, b1, idesc, 1u);
        }
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&mbar[st])));
      }
    }
    // this block's MMAs complete, then its rows: each lane's 128 columns
    // of its half
    wait_mma(g);
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
    if (fail) break;
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
      uint32_t r[32];
      const uint32_t addr =
          tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(e_half * 128 + cc * 32);
      tmem_ld32(addr, r);
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const float y = __uint_as_float(r[i]);
        const float p = __fmul_rn(y, y);
        const df t = two_sum(yy.h, p);
        yy.h = t.h;
        yy.l += t.l + __fmaf_rn(y, y, -p);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
  }
  if (fail) {
    // best-effort drain: copies and MMAs in flight may still be writing;
    // wait once more, with the same limit, for every copy started and every
    // stage's last commit before the columns are freed
    if (tid == 0) {
      // the copies of chunks g - 1 (its wait may have expired) and later
      for (int q = g > 0 ? g - 1 : 0; q < issued; ++q)
        mbar_wait_bounded(smem_u32(&bbar[q % VT_NST]), (uint32_t)((q / VT_NST) & 1));
      for (int q = seen; q < g; ++q)
        mbar_wait_bounded(smem_u32(&mbar[q % VT_NST]), (uint32_t)((q / VT_NST) & 1));
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
  }
  const double yy64 = (double)yy.h + (double)yy.l;
  if (e_half == 1) half_yy[e_cell] = yy64;
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (fail) {
    if (tid == 0) atomicExch(A.err, 1);
  } else if (e_half == 0 && c0 + e_cell < C) {
    A.ws.cell_yy[(int64_t)s * C + c0 + e_cell] = yy64 + half_yy[e_cell];
  }
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(VT_N));
}

// Linv's TF32 terms of chunk (blockIdx.x) of system blockIdx.y, and its
// stations' split coordinates, in the order k_var_tc reads them (see
// spi_krige_var_tc_pack).
__global__ __launch_bounds__(VT_T) void k_var_tc_pack(spi_domain_t dom, spi_systems_t sys,
                                                      spi_krige_ws_t ws) {
  const int s = blockIdx.y;
  if (ws.route[s] != 0) return;
  const int64_t soff = sys.stn_off[s];
  const int n = (int)(sys.stn_off[s + 1] - soff);
  // the chunk's row block and column chunk
  int t = blockIdx.x, rb = 0;
  while (rb < n && t >= vt_chunks(n, rb)) {
    t -= vt_chunks(n, rb);
    rb += VT_N;
  }
  if (rb >= n) return;
  const int k0 = t * VT_KC;
  const int64_t moff = sys.mat_off[s];
  const float* Lh = ws.linv_hi + moff;
  const float* Ll = ws.linv_lo + moff;
  float* dst = ws.linv_tc + (ws.linv_tc_off[s] + blockIdx.x) * (int64_t)VT_CHUNK_FLOATS;
  unsigned char* d0 = reinterpret_cast<unsigned char*>(dst);
  for (int i = 0; i < VT_N * VT_KC / VT_T; ++i) {
    const int e = threadIdx.x + VT_T * i, r = e / VT_KC, k = e % VT_KC;
    const int row = rb + r, col = k0 + k;
    float vh = 0.f, vl = 0.f;
    if (row < n && col <= row) {
      vh = Lh[(int64_t)row * n + col];
      vl = Ll[(int64_t)row * n + col];
    }
    // Linv in three TF32 terms (~33 bits)
    const float b0 = tf32_rn(vh);
    const float r1 = (vh - b0) + vl;
    const float b1 = tf32_rn(r1);
    const int o = tile_off(VT_N, r, k);
    *reinterpret_cast<float*>(d0 + o) = b0;
    *reinterpret_cast<float*>(d0 + VT_B_BYTES + o) = b1;
    *reinterpret_cast<float*>(d0 + 2 * VT_B_BYTES + o) = r1 - b1;
  }
  if (threadIdx.x < VT_KC) {
    const int j = k0 + threadIdx.x;
    reinterpret_cast<float4*>(d0 + 3 * VT_B_BYTES)[threadIdx.x] =
        j < n ? reinterpret_cast<const float4*>(dom.stn_split)[sys.stn_idx[soff + j]]
              : make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

}  // namespace spi

using namespace spi;

extern "C" int spi_krige_var_tc(const spi_domain_t* dom, const spi_systems_t* sys,
                                const spi_krige_ws_t* ws, double cond_split, int32_t* err_flag,
                                spi_stream_t stream) {
  if (!dom || !sys || !ws || !err_flag) return SPI_ERR_ARG;
  if (sys->n_sys < 0 || sys->n_sys > 65535) return SPI_ERR_TOO_LARGE;
  if (sys->n_sys == 0 || dom->n_cells == 0) return SPI_OK;
  if (!ws->cell_yy || !ws->linv_tc || !ws->linv_tc_off || !ws->route || !ws->cond ||
      !ws->shift || !dom->cell_split || !dom->stn_split || !sys->vg || !sys->stn_off ||
      !sys->stn_idx || !sys->mat_off)
    return SPI_ERR_ARG;
  const int64_t tiles = (dom->n_cells + VT_M - 1) / VT_M;
  if (tiles > 0x7fffffff) return SPI_ERR_TOO_LARGE;
  if (reinterpret_cast<uintptr_t>(ws->linv_tc) & 15) return SPI_ERR_ARG;
  if (!smem_opt_in(k_var_tc, VT_SMEM)) return SPI_ERR_CUDA;
  // two CTAs per SM need most of its shared memory
  if (cudaFuncSetAttribute(k_var_tc, cudaFuncAttributePreferredSharedMemoryCarveout, 100) !=
      cudaSuccess)
    return SPI_ERR_CUDA;
  VarTcArgs A{*dom, *sys, *ws, cond_split, err_flag};
  dim3 grid((unsigned)tiles, (unsigned)sys->n_sys);
  k_var_tc<<<grid, VT_T, VT_SMEM, (cudaStream_t)stream>>>(A);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

extern "C" int spi_krige_var_tc_pack(const spi_domain_t* dom, const spi_systems_t* sys,
                                     const spi_krige_ws_t* ws, spi_stream_t stream) {
  if (!dom || !sys || !ws) return SPI_ERR_ARG;
  if (sys->n_sys < 0 || sys->n_sys > 65535) return SPI_ERR_TOO_LARGE;
  if (sys->n_sys == 0) return SPI_OK;
  if (!ws->linv_hi || !ws->linv_lo || !ws->linv_tc || !ws->linv_tc_off || !ws->route ||
      !sys->stn_off || !sys->stn_idx || !sys->mat_off || !dom->stn_split || sys->max_n < 1)
    return SPI_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(ws->linv_tc) & 15) ||
      (reinterpret_cast<uintptr_t>(dom->stn_split) & 15))
    return SPI_ERR_ARG;
  // chunks of the largest system
  int most = 0;
  for (int rb = 0; rb < sys->max_n; rb += VT_N) {
    const int e = sys->max_n < rb + VT_N ? sys->max_n : rb + VT_N;
    most += (e + VT_KC - 1) / VT_KC;
  }
  dim3 grid((unsigned)most, (unsigned)sys->n_sys);
  k_var_tc_pack<<<grid, VT_T, 0, (cudaStream_t)stream>>>(*dom, *sys, *ws);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
