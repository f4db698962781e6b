// IDW on the tensor cores (tcgen05, sm_103a): the masked GEMM pair of the
// IDW branch (interp/steps.py:293-313, cyth/interpmthds.pyx:784-808) for the
// mixed path.
//
// As in k_idw (spi_idw.cu), each cell's weights W[cell][i] = (d_i / d_ref)^-p
// (d_ref the cell's nearest non-zero station distance, FP32 distances from
// the split coordinates) are shared by every step, and every step is a
// masked contraction pair over all stations:
//   num_t = sum_i W[i] m_ti z_ti,  den_t = sum_i W[i] m_ti,  est = num/den,
// m_ti = 1 where station i has a value at step t. Here both are one GEMM
// per group of 32 steps: D [128 cells x 64 columns] = W [128 x N] B [N x 64]
// with B's columns (2t, 2t + 1) = (m_t z_t, m_t) for the group's steps t.
//
// One CTA = 128 cells x 256 threads, two CTAs per SM. Stations go in chunks
// of 8 (one MMA K-step) through a three-stage ring: B's three TF32 terms
// (values to ~33 bits; the masks are exact) and the chunk's stations'
// split coordinates, packed once per launch (k_idw_tc_pack), arrive by one
// 6 KB bulk copy per chunk issued one chunk ahead; all threads compute the
// chunk's weights in FP32 and store them as two TF32 terms (w = a0 + a1).
// One thread issues per chunk g the large products a0 b0 into one of three
// accumulators D0[g % 3] (TMEM columns 0..191) and the corrections a0 b1 +
// a1 b0 + a0 b2 + a1 b1 into D1 (columns 192..255): each large-product
// accumulator takes every third chunk, so the FP32 roundings of these
// positive sums are a third of one running sum's, the corrections
// accumulate at their own scale, and the four are added in FP64 at the
// end. Every wait is bounded: on expiry the
// kernel raises err_flag, writes NaN over its cells, drains on a
// best-effort basis, frees its TMEM and returns.
#include "spi_common.cuh"
#include "spi_tc.cuh"

namespace spi {

constexpr int IT_M = 128;   // cells per CTA (MMA M)
constexpr int IT_N = 64;    // B columns: 32 steps x (value, mask)
constexpr int IT_SEG = 3;   // large-product accumulators
constexpr int IT_G = IT_N / 2;   // steps per group
constexpr int IT_KC = 8;    // stations per chunk
constexpr int IT_T = 256;
constexpr int IT_NST = 3;

constexpr size_t IT_A_BYTES = (size_t)IT_M * IT_KC * 4;
constexpr size_t IT_B_BYTES = (size_t)IT_N * IT_KC * 4;
constexpr size_t IT_S_BYTES = (size_t)IT_KC * 16;
constexpr size_t IT_CHUNK_BYTES = 3 * IT_B_BYTES + IT_S_BYTES;
constexpr size_t IT_STAGE = 2 * IT_A_BYTES + IT_CHUNK_BYTES;
constexpr size_t IT_SMEM = IT_NST * IT_STAGE;
constexpr int IT_CHUNK_FLOATS = (int)(IT_CHUNK_BYTES / 4);
static_assert(IT_CHUNK_FLOATS == SPI_IDW_TC_CHUNK_FLOATS, "packed chunk size");
static_assert(IT_STAGE % 16 == 0 && IT_CHUNK_BYTES % 16 == 0, "bulk copies: 16-byte units");

struct IdwTcArgs {
  spi_domain_t dom;
  int32_t n_steps;
  const int32_t* steps;
  const int32_t* out_row;
  const double* data;  // [T, N], NaN = missing
  const uint8_t* flag;
  const double* means;
  double p;
  const float* pack;
  spi_out_t out;
  int32_t* err;
};

// FP32 distance of k_idw<float> (split coordinates).
__device__ __forceinline__ float it_dist(float4 cp, float4 sp) {
  const float dx = (cp.x - sp.x) + (cp.y - sp.y);
  const float dy = (cp.z - sp.z) + (cp.w - sp.w);
  return sqrtf(dx * dx + dy * dy);
}

// k_idw<float>'s weight of a non-zero distance d against d_ref.
__device__ __forceinline__ float it_weight(float d, float dr, float pf) {
  const float r = d / dr;
  return (pf == 2.0f) ? 1.0f / (r * r) : (pf == 1.0f ? 1.0f / r : exp2f(-pf * log2f(r)));
}

__global__ __launch_bounds__(IT_T, 2) void k_idw_tc(IdwTcArgs A) {
  const int64_t C = A.dom.n_cells;
  const int N = (int)A.dom.n_stns;
  const int64_t c0 = (int64_t)blockIdx.x * IT_M;
  const int grp = blockIdx.y;
  if (c0 >= C) return;
  const int total = (N + IT_KC - 1) / IT_KC;
  const float* pk = A.pack + (int64_t)grp * total * IT_CHUNK_FLOATS;
  extern __shared__ __align__(1024) unsigned char smi[];
  __shared__ __align__(8) uint64_t bbar[IT_NST];
  __shared__ __align__(8) uint64_t mbar[IT_NST];
  __shared__ uint32_t tbase;
  __shared__ int fail;
  __shared__ float s_dmin[2][IT_M];
  __shared__ int s_on[2][IT_M];
  auto stage = [&](int st) { return smi + st * IT_STAGE; };
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tbase)),
                 "r"((IT_SEG + 1) * IT_N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    fail = 0;
    for (int q = 0; q < IT_NST; ++q) {
      mbar_init(smem_u32(&bbar[q]), 1);
      mbar_init(smem_u32(&mbar[q]), 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tbase;
  const uint32_t idesc = tf32_idesc(IT_M, IT_N);

  // ---- 1. per cell: d_ref (nearest non-zero distance), first on-station ----
  const int a_cell = tid & (IT_M - 1), half = tid >> 7;
  const int64_t gc = c0 + a_cell;
  const bool live = gc < C;
  const float4 cp = live ? reinterpret_cast<const float4*>(A.dom.cell_split)[gc]
                         : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4* sp4 = reinterpret_cast<const float4*>(A.dom.stn_split);
  {
    float dmin = __int_as_float(0x7f800000);
    int on = 0x7fffffff;
    if (live)
      for (int j = half; j < N; j += 2) {
        const float d = it_dist(cp, sp4[j]);
        if (d == 0.0f) on = min(on, j);
        else dmin = fminf(dmin, d);
      }
    s_dmin[half][a_cell] = dmin;
    s_on[half][a_cell] = on;
  }
  // the first chunk's copy
  if (tid == 0 && total > 0)
    tc_bulk_load(smem_u32(stage(0) + 2 * IT_A_BYTES), pk, (uint32_t)IT_CHUNK_BYTES,
                 smem_u32(&bbar[0]));
  __syncthreads();
  const float dref = fminf(s_dmin[0][a_cell], s_dmin[1][a_cell]);
  const float pf = (float)A.p;

  // ---- 2. the stations in chunks: weights (A) against the packed B ----
  const int kb = half * 4;
  int seen = 0, issued = total > 0 ? 1 : 0, g = 0;
  auto wait_mma = [&](int upto) {
    while (seen < upto && !fail) {
      if (!mbar_wait_bounded(smem_u32(&mbar[seen % IT_NST]), (uint32_t)((seen / IT_NST) & 1)))
        atomicExch(&fail, 1);
      ++seen;
    }
  };
  for (; g < total; ++g) {
    const int st = g % IT_NST;
    // chunk g + 1 refills the stage of chunk g - 2: its MMAs must be done
    wait_mma(g - 1);
    __syncthreads();
    if (fail) break;
    if (tid == 0 && g + 1 < total) {
      tc_bulk_load(smem_u32(stage((g + 1) % IT_NST) + 2 * IT_A_BYTES),
                   pk + (int64_t)(g + 1) * IT_CHUNK_FLOATS, (uint32_t)IT_CHUNK_BYTES,
                   smem_u32(&bbar[(g + 1) % IT_NST]));
      issued = g + 2;
    }
    unsigned char* sAh = stage(st);
    unsigned char* sAl = sAh + IT_A_BYTES;
    unsigned char* sB = sAh + 2 * IT_A_BYTES;
    const float4* ssp = reinterpret_cast<const float4*>(sB + 3 * IT_B_BYTES);
    if (!mbar_wait_bounded(smem_u32(&bbar[st]), (uint32_t)((g / IT_NST) & 1)))
      atomicExch(&fail, 1);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int kk = kb + q, j = g * IT_KC + kk;
      float w = 0.0f;
      if (live && j < N) {
        const float d = it_dist(cp, ssp[kk]);
        if (d != 0.0f) w = it_weight(d, dref, pf);
      }
      float h, l;
      tf32_split(w, h, l);
      const int o = tile_off(IT_M, a_cell, kk);
      *reinterpret_cast<float*>(sAh + o) = h;
      *reinterpret_cast<float*>(sAl + o) = l;
    }
    asm volatile("fence.proxy.async.shared::cta;");
    __syncthreads();
    if (tid == 0) {
      if (!fail) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint64_t ah = umma_desc(smem_u32(sAh), IT_M * 16, 128);
        const uint64_t al = umma_desc(smem_u32(sAl), IT_M * 16, 128);
        const uint32_t b = smem_u32(sB);
        const uint64_t b0 = umma_desc(b, IT_N * 16, 128);
        const uint64_t b1 = umma_desc(b + (uint32_t)IT_B_BYTES, IT_N * 16, 128);
        const uint64_t b2 = umma_desc(b + 2 * (uint32_t)IT_B_BYTES, IT_N * 16, 128);
        const uint32_t d1 = tmem + IT_SEG * IT_N;
        mma_tf32(tmem + (uint32_t)((g % IT_SEG) * IT_N), ah, b0, idesc, g >= IT_SEG ? 1u : 0u);
        mma_tf32(d1, ah, b1, idesc, g > 0 ? 1u : 0u);
        mma_tf32(d1, al, b0, idesc, 1u);
        mma_tf32(d1, ah, b2, idesc, 1u);
        mma_tf32(d1, al, b1, idesc, 1u);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&mbar[st])));
    }
  }
  wait_mma(g);
  asm volatile("tcgen05.fence::after_thread_sync;");
  __syncthreads();
  if (fail) {
    // best-effort drain of the copies and MMAs in flight
    if (tid == 0) {
      for (int q = g > 0 ? g - 1 : 0; q < issued; ++q)
        mbar_wait_bounded(smem_u32(&bbar[q % IT_NST]), (uint32_t)((q / IT_NST) & 1));
      for (int q = seen; q < g; ++q)
        mbar_wait_bounded(smem_u32(&mbar[q % IT_NST]), (uint32_t)((q / IT_NST) & 1));
      atomicExch(A.err, 1);
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
  }

  // ---- 3. per cell and step: num / den (the four accumulators added in
  // FP64), the mean for unflagged steps, NaN on a present co-located
  // station; TMEM lanes of warp % 4, steps of the column half warp / 4 (16
  // steps, 32 columns of each accumulator) ----
  const int e_cell = (warp & 3) * 32 + lane, e_half = warp >> 2;
  const int64_t ge = c0 + e_cell;
  const int on = min(s_on[0][e_cell], s_on[1][e_cell]);
  float* est_f = reinterpret_cast<float*>(A.out.est);
  double* est_d = reinterpret_cast<double*>(A.out.est);
  const int64_t N64 = N;
  const uint32_t lanes = (uint32_t)((warp & 3) * 32) << 16;
  // accumulators a chunk never reached (fewer than IT_SEG chunks) hold
  // whatever TMEM held: only the ones written count
  const int used = total < IT_SEG ? total : IT_SEG;
#pragma unroll 1
  for (int cc = 0; cc < 2; ++cc) {
    const uint32_t col = (uint32_t)(e_half * 32 + cc * 16);
    double num[8], den[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) num[i] = den[i] = 0.0;
#pragma unroll 1
    for (int a = 0; a <= IT_SEG; ++a) {
      uint32_t r[16];
      tmem_ld16(tmem + lanes + (uint32_t)(a * IT_N) + col, r);
      if (a < IT_SEG && a >= used) continue;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        num[i] += (double)__uint_as_float(r[2 * i]);
        den[i] += (double)__uint_as_float(r[2 * i + 1]);
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int k = grp * IT_G + e_half * 16 + cc * 8 + i;
      if (k >= A.n_steps || ge >= C) continue;
      const int j = A.steps[k];
      double e;
      if (fail) {
        e = __longlong_as_double(0x7ff8000000000000LL);
      } else if (!A.flag[j]) {
        e = A.means[j];
      } else if (on != 0x7fffffff && !isnan(A.data[(int64_t)j * N64 + on])) {
        e = __longlong_as_double(0x7ff8000000000000LL);
      } else {
        e = num[i] / den[i];
      }
      e = clip_est(e, A.out);
      const int64_t o = (int64_t)A.out_row[k] * C + ge;
      if (A.out.out_f64) est_d[o] = e;
      else est_f[o] = (float)e;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((IT_SEG + 1) * IT_N));
}

// B of chunk blockIdx.x (stations 8 chunk .. + 7) of step group blockIdx.y:
// column 2t the value of the group's step t (0 where missing), 2t + 1 its
// mask, in three TF32 terms, then the chunk's stations' split coordinates.
__global__ __launch_bounds__(IT_T) void k_idw_tc_pack(IdwTcArgs A) {
  const int N = (int)A.dom.n_stns;
  const int total = (N + IT_KC - 1) / IT_KC;
  const int kc = blockIdx.x, grp = blockIdx.y;
  unsigned char* d0 = reinterpret_cast<unsigned char*>(
      const_cast<float*>(A.pack) + ((int64_t)grp * total + kc) * IT_CHUNK_FLOATS);
  for (int e = threadIdx.x; e < IT_N * IT_KC; e += IT_T) {
    const int q = e / IT_KC, k = e % IT_KC;
    const int step = grp * IT_G + (q >> 1), j = kc * IT_KC + k;
    double v = 0.0;
    if (step < A.n_steps && j < N) {
      const double x = A.data[(int64_t)A.steps[step] * N + j];
      const bool have = !isnan(x);
      v = (q & 1) ? (have ? 1.0 : 0.0) : (have ? x : 0.0);
    }
    const float hi = (float)v;
    const float lo = (float)(v - (double)hi);
    const float b0 = tf32_rn(hi);
    const float r1 = (hi - b0) + lo;
    const float b1 = tf32_rn(r1);
    const int o = tile_off(IT_N, q, k);
    *reinterpret_cast<float*>(d0 + o) = b0;
    *reinterpret_cast<float*>(d0 + IT_B_BYTES + o) = b1;
    *reinterpret_cast<float*>(d0 + 2 * IT_B_BYTES + o) = r1 - b1;
  }
  if (threadIdx.x < IT_KC) {
    const int j = kc * IT_KC + threadIdx.x;
    reinterpret_cast<float4*>(d0 + 3 * IT_B_BYTES)[threadIdx.x] =
        j < N ? reinterpret_cast<const float4*>(A.dom.stn_split)[j]
              : make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

}  // namespace spi

using namespace spi;

extern "C" int spi_idw_cells_tc(const spi_domain_t* dom, int32_t n_steps, const int32_t* steps,
                                const int32_t* out_row, const double* data, const uint8_t* flag,
                                const double* means, double idw_exp, float* pack,
                                int64_t pack_floats, const spi_out_t* out, int32_t* err_flag,
                                spi_stream_t stream) {
  if (!dom || !out || n_steps < 0) return SPI_ERR_ARG;
  if (n_steps == 0 || dom->n_cells == 0) return SPI_OK;
  if (!steps || !out_row || !data || !out->est || !flag || !means || !pack || !err_flag ||
      dom->n_stns <= 0 || !dom->stn_split || !dom->cell_split)
    return SPI_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(pack) & 15) || (reinterpret_cast<uintptr_t>(dom->stn_split) & 15) ||
      (reinterpret_cast<uintptr_t>(dom->cell_split) & 15))
    return SPI_ERR_ARG;
  if (dom->n_stns > 0x7fffffff) return SPI_ERR_TOO_LARGE;
  const int64_t groups = (n_steps + IT_G - 1) / IT_G;
  const int64_t chunks = (dom->n_stns + IT_KC - 1) / IT_KC;
  if (pack_floats < groups * chunks * IT_CHUNK_FLOATS) return SPI_ERR_ARG;
  if (groups > 65535 || chunks > 0x7fffffff) return SPI_ERR_TOO_LARGE;
  const int64_t tiles = (dom->n_cells + IT_M - 1) / IT_M;
  if (tiles > 0x7fffffff) return SPI_ERR_TOO_LARGE;
  IdwTcArgs A{*dom, n_steps, steps, out_row, data, flag, means, idw_exp, pack, *out, err_flag};
  cudaStream_t st = (cudaStream_t)stream;
  k_idw_tc_pack<<<dim3((unsigned)chunks, (unsigned)groups), IT_T, 0, st>>>(A);
  SPI_LAUNCH_CHECK();
  if (!smem_opt_in(k_idw_tc, IT_SMEM)) return SPI_ERR_CUDA;
  k_idw_tc<<<dim3((unsigned)tiles, (unsigned)groups), IT_T, IT_SMEM, st>>>(A);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
