// Kriging estimates over all cells for systems too large for the
// shared-memory right-hand side of k_krige_cells (n stations x a cell tile
// beyond 227 KB: n > ~1600 in FP64, ~3500 in FP32), e.g. thousands of
// stations with external drifts. Estimates only: the right-hand side of a
// cell is used once per pass, so it is generated on the fly, never stored.
//
// Layout: one CTA = 32 cells x 8 warps. A lane owns a cell; the 8 warps
// split the system's stations (warp w takes stations w, w + 8, ...). Each
// lane generates its cell's entry for the warp's station (coordinates and
// station data are warp-uniform broadcast loads) and accumulates it against
// up to 4 vectors: the system's dual columns (Lagrange / drift rows, for
// the sum check of interp/steps.py:419) and the steps' dual weights. The 8
// partial sums per cell are reduced in shared memory; more steps than fit
// in one pass regenerate the right-hand side. Precision as k_krige_cells:
// FP64 throughout, or (the mixed path's FP32 tier) double-float entries
// (rhs_df, ~1e-9) against FP32 hi/lo vector pairs, accumulated in
// double-float and flushed to FP64 every 256 terms: the estimate's error is
// sum_i dc_i w_i, which large dual weights amplify. With ws.cell_yy (the
// tensor-core |Linv c|^2) the FP32 tier also writes the OK variance.
#include <type_traits>

#include "spi_cells.cuh"
#include "spi_rhs.cuh"

namespace spi {

constexpr int STC = 32;  // cells per CTA (one per lane)
constexpr int SNW = 8;   // warps per CTA (station groups)
constexpr int SSV = 4;   // vectors per pass
constexpr int SCH = 256; // stations per shared-memory chunk (FP32 tier)

// One shared-memory chunk of stations against the pass's vectors (FP32
// tier): double-float entries (rhs_df, or rhs_df_single<CODE> for a
// single-structure variogram) times hi/lo vector pairs, the product's head
// by the FMA error, the cross terms, TwoSum into a double-float partial,
// flushed to FP64 every 256 terms. Dual columns that feed only the sum
// check (v0 + v < plain_duals) take a plain FP32 product.
template <int CODE, bool TRACK>
__device__ __forceinline__ void stream_chunk(const CellsArgs& A, const spi_vg_t* vgp,
                                             const RhsDf& kd, int sk, double sh, float4 cp,
                                             bool live, int64_t gc, const int32_t* idxc,
                                             const float4* s_sp, const float2 (*s_w)[SCH],
                                             int nj, int warp, int nv, int v0, int plain_duals,
                                             float (&ph)[SSV], float (&pl)[SSV],
                                             double (&acc)[SSV], int& cnt, NearDf& nf,
                                             int j0, float esp) {
  for (int jj = warp; jj < nj; jj += SNW) {
    df c = {0.f, 0.f};
    if (live) {
      const df d2 = df_dist2(cp, s_sp[jj]);
      if constexpr (TRACK) nf.add(d2, j0 + jj, esp);
      if constexpr (CODE < 0)
        c = rhs_df_d2(A.dom, vgp, kd, sk, sh, d2, gc, idxc + jj);
      else
        c = rhs_df_single_d2<CODE>(A.dom, vgp, kd, sk, sh, d2, gc, idxc + jj);
    }
#pragma unroll
    for (int v = 0; v < SSV; ++v)
      if (v < nv && v0 + v < plain_duals) {
        ph[v] = __fmaf_rn(c.h, s_w[v][jj].x, ph[v]);
      } else if (v < nv) {
        const float2 w = s_w[v][jj];
        const float p = __fmul_rn(c.h, w.x);
        float e = __fmaf_rn(c.h, w.x, -p);
        e = __fmaf_rn(c.h, w.y, e);
        e = __fmaf_rn(c.l, w.x, e);
        const df s2 = two_sum(ph[v], p);
        ph[v] = s2.h;
        pl[v] += s2.l + e;
      }
    if (++cnt == 256) {
      cnt = 0;
#pragma unroll
      for (int v = 0; v < SSV; ++v) {
        acc[v] += (double)ph[v] + (double)pl[v];
        ph[v] = pl[v] = 0.f;
      }
    }
  }
}

template <typename T, typename OutT>
__global__ __launch_bounds__(STC * SNW, 2) void k_krige_cells_stream(CellsArgs A) {
  const int s = blockIdx.y;
  const int64_t C = A.dom.n_cells;
  const int64_t c0 = (int64_t)blockIdx.x * STC;
  if (c0 >= C) return;
  const int route = A.ws.route[s];
  {
    const bool fast = fp32_tier(A.ws, s, A.cond_split, A.sys.kind == SPI_KIND_SK);
    if ((A.route_filter == 1 && !fast) || (A.route_filter == 2 && fast)) return;
  }
  const bool prim = route == 1;
  const bool failed = route == 2;
  const int64_t soff = A.sys.stn_off[s];
  const int n = (int)(A.sys.stn_off[s + 1] - soff);
  const int32_t* idx = A.sys.stn_idx + soff;
  const int sk = A.sys.kind == SPI_KIND_SK;
  const int a = sk ? 1 : extra_rows(A.sys.kind, A.dom.n_drift);
  // (SK in an FP32 tier adds |u|, the bound of its sum check's rounding,
  // on either route)
  const int ndual = (sk && sizeof(T) == 4) ? 2 : (prim ? 1 : a);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t st0 = A.sys.step_off[s];
  const int nsteps = (int)(A.sys.step_off[s + 1] - st0);
  const int nvec = ndual + nsteps;
  // OK / EDK without the variance: the dual columns feed only the sum
  // check, and sum(lambda) = q0 - sum_k S_0k nu_k is 1 identically whatever
  // q is (nu = S^-1 (q - f)); they need no more than FP32 (the estimates,
  // SK's u'c and the OK variance's q0 keep double-float)
  const bool var_needed = A.want_var && A.out.var != nullptr && !sk;
  const int plain_duals = (sizeof(T) == 4 && !sk && !prim && !var_needed) ? ndual : 0;
  const spi_vg_t vg = A.sys.vg[s];
  const double sh = A.ws.shift[s];

  __shared__ double red[SNW][SSV][STC];
  __shared__ double vres[SSV][STC];
  __shared__ int okf[STC], nnb[STC];
  __shared__ double cvar[STC];
  __shared__ const double* vp64[SSV];
  __shared__ const float* vph[SSV];
  __shared__ const float* vpl[SSV];
  __shared__ int any_bad;
  __shared__ int any_chk;
  __shared__ float4 s_sp[sizeof(T) == 4 ? SCH : 1];
  __shared__ float2 s_w[SSV][sizeof(T) == 4 ? SCH : 1];
  // the FP32 tier's nearest-station candidates per station group (warp)
  // and cell, from the first pass's right-hand sides (written over red once
  // the pass's sums are reduced), and the cells they leave ambiguous
  NearDf* s_nf = reinterpret_cast<NearDf*>(&red[0][0][0]);
  static_assert(sizeof(NearDf) * SNW * STC <= sizeof(red), "candidates fit in red");
  __shared__ int namb[STC];
  const bool fuse_nnb = sizeof(T) == 4 && A.dom.split_res > 0.0;
  const float esp = (float)(A.dom.split_res * 0x1p-24);
  bool nf_ready = false;

  const int64_t gc = c0 + lane;
  const bool live = gc < C;
  OutT* est_out = reinterpret_cast<OutT*>(A.out.est);
  // the OK variance needs |Linv c|^2 per cell from the tensor-core kernel
  const bool var_out = sizeof(T) == 4 && A.want_var && A.out.var != nullptr && !sk &&
                       A.ws.cell_yy != nullptr;
  OutT* var_outp = reinterpret_cast<OutT*>(A.out.var);
  auto emit = [&](int cell, int vstep, double accv) {
    const int64_t g = c0 + cell;
    if (g >= C) return;
    const int j = A.sys.steps[st0 + vstep];
    const int64_t row = A.sys.out_row[j];
    double e;
    if (okf[cell]) {
      e = accv;
      if (!sk) {
        const double* bt = A.ws.beta + (int64_t)j * GA;
        e += bt[0];
        for (int k = 1; k < a; ++k) e += bt[k] * A.dom.cell_drift[(int64_t)(k - 1) * C + g];
      }
    } else {
      e = A.vals[A.sys.val_off[j] + nnb[cell]];
    }
    est_out[row * C + g] = cast_out<OutT>(clip_est(e, A.out));
    if (var_out) var_outp[row * C + g] = cast_out<OutT>(okf[cell] ? cvar[cell] : 0.0);
  };
  // the nearest station of every cell that failed the sum check: from the
  // right-hand sides' squared distances where they decide it, else (and
  // without them) the exact FP64 search
  auto nearest = [&]() {
    __syncthreads();
    if (any_bad) {
      if (tid < STC) {
        int amb = 1;
        if constexpr (sizeof(T) == 4) {
          if (nf_ready) {
            NearDf m = s_nf[tid];
#pragma unroll
            for (int w = 1; w < SNW; ++w) m.merge(s_nf[w * STC + tid]);
            if (!m.amb && m.bj >= 0) {
              nnb[tid] = m.bj;
              amb = 0;
            }
          }
        }
        namb[tid] = amb;
      }
      __syncthreads();
      for (int cell = warp; cell < STC; cell += SNW) {
        const int64_t g = c0 + cell;
        if (g >= C || okf[cell] || !namb[cell]) continue;
        const int j = nnb_f64_warp(A.dom, idx, n, A.dom.cell_x[g], A.dom.cell_y[g]);
        if (lane == 0) nnb[cell] = j;
      }
    }
    __syncthreads();
  };

  if (failed) {
    if (tid < STC) {
      okf[tid] = 0;
      cvar[tid] = 0.0;
    }
    if (tid == 0) any_bad = 1;
    nearest();
    for (int e = tid; e < nsteps * STC; e += STC * SNW) emit(e % STC, e / STC, 0.0);
    return;
  }

  double cx = 0.0, cy = 0.0;
  float4 cp = make_float4(0.f, 0.f, 0.f, 0.f);
  __shared__ RhsDf kd;
  // the variogram with its reciprocal ranges (FP64 right-hand sides)
  __shared__ VgPre vgp64;
  if constexpr (sizeof(T) == 8) {
    if (live) {
      cx = A.dom.cell_x[gc];
      cy = A.dom.cell_y[gc];
    }
    if (tid == 0) vgp64.init(vg);
  } else {
    if (live) cp = reinterpret_cast<const float4*>(A.dom.cell_split)[gc];
    if (tid == 0) kd.init(vg, sh, A.dom.min_vg_val);
  }
  const spi_vg_t* vgp = A.sys.vg + s;
  const float4* sp4 = reinterpret_cast<const float4*>(A.dom.stn_split);

  for (int v0 = 0; v0 < nvec; v0 += SSV) {
    const int nv = min(SSV, nvec - v0);
    __syncthreads();
    if (tid < SSV) {
      const int v = v0 + tid;
      const double* p64 = nullptr;
      const float *ph = nullptr, *pl = nullptr;
      if (tid < nv) {
        int64_t off;
        if (v < ndual) {
          off = soff * GA + (int64_t)v * n;
          p64 = A.ws.g_cols + off;
          if (A.ws.g_hi) ph = A.ws.g_hi + off, pl = A.ws.g_lo + off;
        } else {
          off = A.sys.val_off[A.sys.steps[st0 + (v - ndual)]];
          p64 = A.ws.w_hat + off;
          if (A.ws.w_hi) ph = A.ws.w_hi + off, pl = A.ws.w_lo + off;
        }
      }
      vp64[tid] = p64;
      vph[tid] = ph;
      vpl[tid] = pl;
    }
    __syncthreads();
    double acc[SSV];
#pragma unroll
    for (int v = 0; v < SSV; ++v) acc[v] = 0.0;
    // (OK / EDK on the Cholesky path pass the sum check on every cell:
    // their sum(lambda) is 1 up to rounding whatever the right-hand side)
    const bool track = sizeof(T) == 4 && fuse_nnb && v0 == 0 && sk;
    NearDf nf;
    nf.init();
    if constexpr (sizeof(T) == 8) {
      for (int j = warp; j < n; j += SNW) {
        const int st = idx[j];
        double c = 0.0;
        if (live) {
          const double g = vgp64.fill_d2(
              dist2_f64(cx, cy, A.dom.stn_x[st], A.dom.stn_y[st]), sk, A.dom.min_vg_val);
          c = (sk || prim) ? g : __dsub_rn(sh, g);
        }
#pragma unroll
        for (int v = 0; v < SSV; ++v)
          if (v < nv) acc[v] = fma(c, vp64[v][j], acc[v]);
      }
    } else {
      // double-float entries against hi/lo vectors (stream_chunk)
      float ph[SSV], pl[SSV];
#pragma unroll
      for (int v = 0; v < SSV; ++v) ph[v] = pl[v] = 0.f;
      int cnt = 0;
      // stations in chunks staged in shared memory: split coordinates and
      // the vectors' hi/lo pairs, read by every warp at a shared index
      for (int j0 = 0; j0 < n; j0 += SCH) {
        const int nj = min(SCH, n - j0);
        __syncthreads();
        for (int e = tid; e < nj; e += STC * SNW) {
          s_sp[e] = sp4[idx[j0 + e]];
#pragma unroll
          for (int v = 0; v < SSV; ++v)
            if (v < nv) s_w[v][e] = make_float2(vph[v][j0 + e], vpl[v][j0 + e]);
        }
        __syncthreads();
        // the single structure's model, uniform over the CTA
        const int scode = (kd.exact && kd.single >= 0) ? kd.code[kd.single] : -1;
        const int32_t* idxc = idx + j0;
        // the nearest-station tracking as a compile-time choice: kernels
        // that never need it carry none of its state through the loop
        auto chunk = [&](auto trk) {
          constexpr bool TR = decltype(trk)::value;
          switch (scode) {
            case SPI_VG_EXP:
              stream_chunk<SPI_VG_EXP, TR>(A, vgp, kd, sk, sh, cp, live, gc, idxc, s_sp, s_w, nj,
                                           warp, nv, v0, plain_duals, ph, pl, acc, cnt, nf, j0,
                                           esp);
              break;
            case SPI_VG_GAU:
              stream_chunk<SPI_VG_GAU, TR>(A, vgp, kd, sk, sh, cp, live, gc, idxc, s_sp, s_w, nj,
                                           warp, nv, v0, plain_duals, ph, pl, acc, cnt, nf, j0,
                                           esp);
              break;
            case SPI_VG_SPH:
              stream_chunk<SPI_VG_SPH, TR>(A, vgp, kd, sk, sh, cp, live, gc, idxc, s_sp, s_w, nj,
                                           warp, nv, v0, plain_duals, ph, pl, acc, cnt, nf, j0,
                                           esp);
              break;
            case SPI_VG_LIN:
              stream_chunk<SPI_VG_LIN, TR>(A, vgp, kd, sk, sh, cp, live, gc, idxc, s_sp, s_w, nj,
                                           warp, nv, v0, plain_duals, ph, pl, acc, cnt, nf, j0,
                                           esp);
              break;
            default:
              stream_chunk<-1, TR>(A, vgp, kd, sk, sh, cp, live, gc, idxc, s_sp, s_w, nj, warp, nv,
                                   v0, plain_duals, ph, pl, acc, cnt, nf, j0, esp);
          }
        };
        if (track)
          chunk(std::true_type{});
        else
          chunk(std::false_type{});
      }
#pragma unroll
      for (int v = 0; v < SSV; ++v) acc[v] += (double)ph[v] + (double)pl[v];
    }
#pragma unroll
    for (int v = 0; v < SSV; ++v) red[warp][v][lane] = acc[v];
    __syncthreads();
    for (int e = tid; e < nv * STC; e += STC * SNW) {
      const int v = e / STC, cell = e % STC;
      double t = 0.0;
#pragma unroll
      for (int w = 0; w < SNW; ++w) t += red[w][v][cell];
      vres[v][cell] = t;
    }
    __syncthreads();
    if (track) {
      s_nf[warp * STC + lane] = nf;  // red is free again
      nf_ready = true;
    }
    if (v0 == 0) {
      // the sum check of every cell, from the dual columns (all in pass 0)
      if (tid == 0) any_bad = any_chk = 0;
      __syncthreads();
      if (tid < STC) {
        const int cell = tid;
        const int64_t g = c0 + cell;
        double q[GA], f[GA], nu[GA];
        for (int k = 0; k < GA; ++k) q[k] = k < ndual ? vres[k][cell] : 0.0;
        f[0] = 1.0;
        for (int k = 1; k < GA; ++k)
          f[k] = (k < a && g < C && !sk) ? A.dom.cell_drift[(int64_t)(k - 1) * C + g] : 0.0;
        double sl;
        if (prim) {
          sl = q[0];
          if (!sk)
            for (int k = 0; k < a; ++k) sl += f[k] * A.ws.g_colsum[(int64_t)s * GA + k];
        } else if (sk) {
          sl = q[0];
        } else {
          const double* Si = A.ws.s_inv + (int64_t)s * GA * GA;
          for (int k = 0; k < a; ++k) {
            double t = 0.0;
            for (int l = 0; l < a; ++l) t += Si[k * GA + l] * (q[l] - f[l]);
            nu[k] = t;
          }
          sl = q[0];
          for (int k = 0; k < a; ++k) sl -= A.ws.g_colsum[(int64_t)s * GA + k] * nu[k];
          if (var_out && g < C)
            cvar[cell] = sh * sl - A.ws.cell_yy[(int64_t)s * C + g] + nu[0] * q[0] - 2.0 * nu[0];
        }
        int ok = isclose_one(sl) ? 1 : 0;
        // SK's FP32 sum(lambda) within its rounding bound of the check's
        // boundary: decided in FP64 (as k_krige_cells)
        if (sizeof(T) == 4 && sk && g < C &&
            near_isclose_boundary(sl, kSumLambdaRelErrDf * q[1])) {
          ok = 2;
          atomicOr(&any_chk, 1);
        }
        okf[cell] = ok;
        if (!ok && g < C) atomicOr(&any_bad, 1);
      }
      __syncthreads();
      if (any_chk)
        for (int cell = warp; cell < STC; cell += SNW) {
          if (okf[cell] != 2) continue;
          const int64_t g = c0 + cell;
          const double sl = sk_sum_lambda_f64(A.dom, vg, idx, n, A.ws.g_cols + soff * GA,
                                              A.dom.cell_x[g], A.dom.cell_y[g]);
          if (lane == 0) {
            const int ok = isclose_one(sl) ? 1 : 0;
            okf[cell] = ok;
            if (!ok) atomicOr(&any_bad, 1);
          }
        }
      nearest();
    }
    for (int e = tid; e < nv * STC; e += STC * SNW) {
      const int v = v0 + e / STC, cell = e % STC;
      if (v >= ndual) emit(cell, v - ndual, vres[e / STC][cell]);
    }
  }
}

int launch_cells_stream(const CellsArgs& A, int precision, cudaStream_t st) {
  const int64_t tiles = (A.dom.n_cells + STC - 1) / STC;
  if (tiles > 0x7fffffff) return SPI_ERR_TOO_LARGE;
  dim3 grid((unsigned)tiles, (unsigned)A.sys.n_sys);
  const bool f64 = A.out.out_f64 != 0;
  if (precision == 0) {
    if (f64) k_krige_cells_stream<double, double><<<grid, STC * SNW, 0, st>>>(A);
    else k_krige_cells_stream<double, float><<<grid, STC * SNW, 0, st>>>(A);
  } else {
    if (f64) k_krige_cells_stream<float, double><<<grid, STC * SNW, 0, st>>>(A);
    else k_krige_cells_stream<float, float><<<grid, STC * SNW, 0, st>>>(A);
  }
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

}  // namespace spi
