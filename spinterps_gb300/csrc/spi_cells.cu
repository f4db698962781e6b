// Kriging over all cells of all steps of a system batch.
//
// Replaces interp/steps.py:403-435 (_fill_krig_idw_dst_data: a Python loop
// over cells doing lambda = pinv @ rhs per cell and step) together with the
// cell x station variogram matrix it reads (interp/steps.py:639-650,
// cyth/interpmthds.pyx:146-226): here the right-hand sides of a tile of
// cells are generated in shared memory from coordinates (fused distance +
// variogram) and contracted against
//   - the system's dual columns G (Lagrange / drift rows, sum check),
//   - Linv (OK variance |Linv c|^2, triangular),
//   - the per-step dual weights w_hat (estimates of every step at once),
// all through one shared-memory-tiled contraction routine. The estimate
// of step j is c'w_hat_j + f'beta_j (dual form: 2n FLOP per cell-step
// instead of the reference's 2m^2), the variance costs n^2 FLOP per
// cell and is shared by every step of the system.
//
// precision 0: everything in FP64 (the plain path).
// precision 1: right-hand sides generated in FP32 from double-float
// coordinates (differences accurate relative to the distance itself),
// contracted in split FP32 (each FP64 factor / dual value as an FP32 hi/lo
// pair, FP32 partial sums flushed to FP64 every 64 terms), FP64 epilogue.
#include "spi_common.cuh"
#include "spi_contract.cuh"
#include "spi_rhs.cuh"
#include "spi_cells.cuh"

namespace spi {

template <typename T, int TC, bool W>
__device__ __forceinline__ void contract(const T* cvT, T* Bs, const double* const* vp64,
                                         const float* const* vph, const float* const* vpl,
                                         int nv, int jmax, int nload,
                                         double (&out)[Layout<TC, W>::CPT][Layout<TC, W>::VPT],
                                         int jmin = 0) {
  if constexpr (sizeof(T) == 8)
    tile_contract<T, TC, W>(cvT, Bs, PtrLoader64{vp64}, nv, jmax, nload, out, jmin);
  else
    tile_contract<T, TC, W>(cvT, Bs, PtrLoader32{vph, vpl}, nv, jmax, nload, out, jmin);
}

template <typename T, int TC, typename OutT>
__global__ __launch_bounds__(CT) void k_krige_cells(CellsArgs A, int npad) {
  using WL = Layout<TC, true>;
  using NL = Layout<TC, false>;
  constexpr int CPT = WL::CPT;
  const int s = blockIdx.y;
  const int64_t C = A.dom.n_cells;
  const int64_t c0 = (int64_t)blockIdx.x * TC;
  if (c0 >= C) return;
  const int route = A.ws.route[s];
  {
    // filter 1: well-conditioned Cholesky systems; filter 2: all others
    const bool fast = fp32_tier(A.ws, s, A.cond_split, A.sys.kind == SPI_KIND_SK);
    if ((A.route_filter == 1 && !fast) || (A.route_filter == 2 && fast)) return;
  }
  const bool prim = route == 1;   // exact-inverse path: primal formulas
  const bool failed = route == 2;
  const int64_t soff = A.sys.stn_off[s];
  const int n = (int)(A.sys.stn_off[s + 1] - soff);
  const int32_t* idx = A.sys.stn_idx + soff;
  const int sk = A.sys.kind == SPI_KIND_SK;
  // Lagrange / drift rows; on the Cholesky path SK contracts one dual
  // column (u = A^-1 1) in the same slot
  const int a = sk ? 1 : extra_rows(A.sys.kind, A.dom.n_drift);
  // dual columns contracted per cell; the FP32 tier adds SK's |u| column
  // (a rounding bound for its sum check)
  const int ndual = prim ? 1 : ((sk && sizeof(T) == 4) ? 2 : a);
  const int tid = threadIdx.x;
  const int64_t st0 = A.sys.step_off[s], st1 = A.sys.step_off[s + 1];
  const int nsteps = (int)(st1 - st0);
  const int64_t moff = A.sys.mat_off[s];

  extern __shared__ __align__(16) unsigned char smraw[];
  T* cvT = reinterpret_cast<T*>(smraw);                                // [npad][TC]
  T* Bs = cvT + (int64_t)npad * TC;                                     // KC * BSTR doubles
  double* qc = reinterpret_cast<double*>(Bs) + KC * BSTR;               // [TC][GA]
  double* cvar = qc + TC * GA;                                          // [TC]
  // per-cell partial sums reuse the staging buffer (free between passes)
  double* red = reinterpret_cast<double*>(Bs);                          // [16][TC]
  int* nnb = reinterpret_cast<int*>(cvar + TC);                         // [TC]
  int* okf = nnb + TC;                                                  // [TC]
  const double** vp64 = reinterpret_cast<const double**>(okf + TC);    // [VB]
  const float** vph = reinterpret_cast<const float**>(vp64 + VB);      // [VB]
  const float** vpl = vph + VB;                                         // [VB]
  __shared__ int any_bad;
  __shared__ int any_ok;
  __shared__ int any_chk;
  __shared__ int n_ok;
  __shared__ double wred[CT / 32];

  // vector v of the next pass: FP64 base + off, or its FP32 hi / lo copies
  auto setv = [&](int v, const double* b64, const float* bh, const float* bl, int64_t off,
                  bool valid) {
    vp64[v] = valid ? b64 + off : nullptr;
    vph[v] = (valid && bh) ? bh + off : nullptr;
    vpl[v] = (valid && bl) ? bl + off : nullptr;
  };

  const spi_vg_t vg = A.sys.vg[s];
  // the variogram with its reciprocal ranges (FP64 right-hand sides)
  __shared__ VgPre vgp64;
  if (sizeof(T) == 8 && tid == 0) vgp64.init(vg);
  // right-hand side: covariance form s - gamma on the Cholesky path, the
  // reference's gamma itself on the exact-inverse path
  const double sh = A.ws.shift[s];
  if (tid == 0) {
    any_bad = failed ? 1 : 0;
    any_ok = 0;
    any_chk = 0;
    n_ok = 0;
  }
  for (int e = tid; e < TC * GA; e += CT) qc[e] = 0.0;
  __syncthreads();  // vgp64

  if (!failed) {
    // ---- 1. right-hand sides, cell-contiguous: cvT[j][cell] ----
    {
      const int cell = tid % TC, jg = tid / TC, njg = CT / TC;
      const int64_t gc = c0 + cell;
      const bool live = gc < C;
      if constexpr (sizeof(T) == 8) {
        const double cx = live ? A.dom.cell_x[gc] : 0.0, cy = live ? A.dom.cell_y[gc] : 0.0;
        // the nearest station of the cell comes with its squared distances:
        // the first index of the smallest dist_f64 (as nnb_f64_warp). The
        // root is monotone, so a smaller square never has a larger root,
        // and squares more than 2^-50 apart (relative) never share one;
        // closer pairs compare their roots (a later index wins only with a
        // strictly smaller root)
        double best = __longlong_as_double(0x7ff0000000000000LL);
        int bj = 0x7fffffff;
        for (int j = jg; j < npad; j += njg) {
          double v = 0.0;
          if (live && j < n) {
            const int st = idx[j];
            const double d2 = dist2_f64(cx, cy, A.dom.stn_x[st], A.dom.stn_y[st]);
            if (d2 < best &&
                (best - d2 > 0x1p-50 * best || __dsqrt_rn(d2) < __dsqrt_rn(best))) {
              best = d2;
              bj = j;
            }
            const double g = vgp64.fill_d2(d2, sk, A.dom.min_vg_val);
            v = (sk || prim) ? g : __dsub_rn(sh, g);
          }
          if (prim && live && j >= n && j < n + a) {
            const int k = j - n;  // r = [gamma, 1, drifts] rows of the saddle system
            v = (k == 0) ? 1.0 : A.dom.cell_drift[(int64_t)(k - 1) * C + gc];
          }
          cvT[(int64_t)j * TC + cell] = (T)v;
        }
        // per cell, the minimum over the thread groups (Bs is free until
        // the contractions below)
        double* bd = reinterpret_cast<double*>(Bs);
        bd[jg * TC + cell] = __dsqrt_rn(best);
        bd[CT + jg * TC + cell] = (double)bj;
        __syncthreads();
        if (tid < TC) {
          double b = bd[tid];
          int bi = (int)bd[CT + tid];
          for (int g = 1; g < njg; ++g) {
            const double ob = bd[g * TC + tid];
            const int oi = (int)bd[CT + g * TC + tid];
            if (ob < b || (ob == b && oi < bi)) {
              b = ob;
              bi = oi;
            }
          }
          nnb[tid] = bi == 0x7fffffff ? 0 : bi;
        }
        __syncthreads();
      } else {
        const float4 cp = live ? reinterpret_cast<const float4*>(A.dom.cell_split)[gc]
                               : make_float4(0.f, 0.f, 0.f, 0.f);
        RhsF32 kf;
        kf.init(vg, sk, sh, A.dom.min_vg_val);
        const float4* sp4 = reinterpret_cast<const float4*>(A.dom.stn_split);
        for (int j = jg; j < npad; j += njg) {
          float v = 0.f;
          if (live && j < n) {
            const int st = idx[j];
            v = rhs_f32(A.dom, vg, kf, sk, sh, cp, sp4[st], gc, st);
          }
          cvT[(int64_t)j * TC + cell] = (T)v;
        }
      }
    }
    // ---- 2. dual columns (narrow passes): qc[cell][k] = G_k' c ----
    for (int v0 = 0; v0 < ndual; v0 += NL::NV) {
      const int nv = min(NL::NV, ndual - v0);
      __syncthreads();
      for (int v = tid; v < NL::NV; v += CT) {
        const int64_t off = soff * GA + (int64_t)(v0 + v) * n;
        setv(v, A.ws.g_cols, A.ws.g_hi, A.ws.g_lo, off, v < nv);
      }
      double acc[NL::CPT][NL::VPT];
      contract<T, TC, false>(cvT, Bs, vp64, vph, vpl, nv, n, n, acc);
      const int cell = tid % TC, k = v0 + tid / TC;
      if (tid / TC < nv) qc[cell * GA + k] = acc[0][0];
    }
    // ---- 3. OK variance |Linv c|^2, wide passes over Linv's rows
    // (triangular: a pass of rows r0..r0+63 stops at column r0+63) ----
    // (the FP32 tier may take it from the tensor-core kernel instead:
    // spi_krige_var_tc, ws.cell_yy)
    const bool yy_tc = sizeof(T) == 4 && A.ws.cell_yy != nullptr;
    double yy_part[CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c) yy_part[c] = 0.0;
    if (A.want_var && !prim && !yy_tc) {
      for (int r0 = 0; r0 < n; r0 += VB) {
        __syncthreads();
        for (int v = tid; v < VB; v += CT)
          setv(v, A.ws.linv_arena, A.ws.linv_hi, A.ws.linv_lo, moff + (int64_t)(r0 + v) * n,
               r0 + v < n);
        double acc[CPT][4];
        contract<T, TC, true>(cvT, Bs, vp64, vph, vpl, min(VB, n - r0), min(n, r0 + VB), n, acc);
#pragma unroll
        for (int c = 0; c < CPT; ++c) {
          double q = 0.0;
#pragma unroll
          for (int r = 0; r < 4; ++r) q += acc[c][r] * acc[c][r];
          yy_part[c] += q;
        }
      }
    }
    __syncthreads();
    {
      const int cg = tid % 16, rg = tid / 16;
#pragma unroll
      for (int c = 0; c < CPT; ++c) red[rg * TC + cg * CPT + c] = yy_part[c];
    }
    __syncthreads();
    // ---- 4. per cell: nu, sum(lambda), variance ----
    for (int cell = tid; cell < TC; cell += CT) {
      const int64_t gc = c0 + cell;
      double yy = 0.0;
      if (yy_tc) {
        if (A.want_var && gc < C) yy = A.ws.cell_yy[(int64_t)s * C + gc];
      } else {
        for (int g = 0; g < 16; ++g) yy += red[g * TC + cell];
      }
      double q[GA], nu[GA], f[GA];
      for (int k = 0; k < GA; ++k) q[k] = qc[cell * GA + k];
      f[0] = 1.0;
      for (int k = 1; k < GA; ++k)
        f[k] = (k < a && gc < C && !sk) ? A.dom.cell_drift[(int64_t)(k - 1) * C + gc] : 0.0;
      double sl;
      double vv = 0.0;
      if (prim) {
        // r = [gamma, f]: sum(lambda) = r'u with u = P [1; 0]
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
        vv = sh * sl - yy + nu[0] * q[0] - 2.0 * nu[0];
      }
      int ok = isclose_one(sl) ? 1 : 0;
      // SK's sum(lambda) varies from cell to cell: where the FP32 value
      // is within its rounding bound of the check's boundary, the FP64
      // value decides (otherwise estimate and nearest station can swap)
      if (sizeof(T) == 4 && sk && gc < C &&
          near_isclose_boundary(sl, kSumLambdaRelErr * q[1])) {
        ok = 2;
        atomicOr(&any_chk, 1);
      }
      okf[cell] = ok;
      cvar[cell] = ok == 1 ? vv : 0.0;
      if (!ok && gc < C) atomicOr(&any_bad, 1);
      if (ok == 1 && gc < C) {
        atomicOr(&any_ok, 1);
        atomicAdd(&n_ok, 1);
      }
    }
    __syncthreads();
    if constexpr (sizeof(T) == 4) {
      if (any_chk) {
        const int warp = tid >> 5, lane = tid & 31;
        for (int cell = warp; cell < TC; cell += CT / 32) {
          if (okf[cell] != 2) continue;
          const int64_t gc = c0 + cell;
          const double sl = sk_sum_lambda_f64(A.dom, vg, idx, n, A.ws.g_cols + soff * GA,
                                              A.dom.cell_x[gc], A.dom.cell_y[gc]);
          if (lane == 0) {
            const int ok = isclose_one(sl) ? 1 : 0;
            okf[cell] = ok;
            atomicOr(ok ? &any_ok : &any_bad, 1);
          }
        }
      }
    }
    // ---- 4b. exact-inverse path, OK variance of the cells that pass the
    // check: lambda = P r, var = lambda'r + lambda_n. A few passing cells
    // (numerically singular systems: the sum check passes on ~1% of
    // cells) take lambda = P r one cell at a time, a warp per row of P
    // (latency-bound: P streams from L2 for each cell, about 3x the time
    // per FMA of a wide pass); tiles where more than a quarter pass take
    // wide passes over P's rows for the whole tile; skipped when no cell
    // of the tile passes ----
    __syncthreads();
    if constexpr (sizeof(T) == 8) {
      const int m_prim = n + a;
      if (prim && A.want_var && !sk && any_ok && n_ok <= TC / 4 && m_prim <= KC * BSTR) {
        const int m = m_prim;
        if (tid == 0 && A.ws.var_cells) atomicAdd(A.ws.var_cells + s, n_ok);
        double* rv = reinterpret_cast<double*>(Bs);  // [m] the cell's r
        const double* P = A.ws.l_arena + moff;
        const int warp = tid >> 5, lane = tid & 31;
        for (int cell = 0; cell < TC; ++cell) {
          if (okf[cell] != 1 || c0 + cell >= C) continue;
          __syncthreads();
          for (int j = tid; j < m; j += CT) rv[j] = (double)cvT[(int64_t)j * TC + cell];
          __syncthreads();
          double part = 0.0;
          for (int i = warp; i < m; i += CT / 32) {
            const double* row = P + (int64_t)i * m;
            double t = 0.0;
            for (int j = lane; j < m; j += 32) t = fma(row[j], rv[j], t);
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            part += t * rv[i] + (i == n ? t : 0.0);
          }
          if (lane == 0) wred[warp] = part;
          __syncthreads();
          if (tid == 0) {
            double vv = 0.0;
            for (int w = 0; w < CT / 32; ++w) vv += wred[w];
            cvar[cell] = vv;
          }
        }
      } else if (prim && A.want_var && !sk && any_ok) {
        // the whole tile, as the symmetric quadratic form over P's block
        // upper triangle: with r' = r + e_n / 2 (r_n = 1, the unbiasedness
        // row), var = r'P r' - P_nn / 4, and per block of VB rows i
        // r'P r' gathers r'_i (D_i + 2 U_i): D over the block's own
        // columns, U over the columns right of it (about m^2 / 2 FMAs per
        // cell instead of m^2)
        const int m = m_prim;
        // cells whose tile ran this pass (the FLOP count of the roofline)
        if (tid == 0 && A.ws.var_cells)
          atomicAdd(A.ws.var_cells + s, (int)min((int64_t)TC, C - c0));
        __syncthreads();
        for (int cell = tid; cell < TC; cell += CT) cvT[(int64_t)n * TC + cell] = 1.5;
        double vpart[CPT];
#pragma unroll
        for (int c = 0; c < CPT; ++c) vpart[c] = 0.0;
        const int cg = tid % 16, rg = tid / 16;
        for (int r0 = 0; r0 < m; r0 += VB) {
          const int r1 = min(m, r0 + VB);
          __syncthreads();
          for (int v = tid; v < VB; v += CT)
            setv(v, A.ws.l_arena, nullptr, nullptr, moff + (int64_t)(r0 + v) * m, r0 + v < m);
          double dg[CPT][4], up[CPT][4];
          contract<T, TC, true>(cvT, Bs, vp64, vph, vpl, r1 - r0, r1, m, dg, r0);
#pragma unroll
          for (int c = 0; c < CPT; ++c)
#pragma unroll
            for (int r = 0; r < 4; ++r) up[c][r] = 0.0;
          if (r1 < m) contract<T, TC, true>(cvT, Bs, vp64, vph, vpl, r1 - r0, m, m, up, r1);
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const int row = r0 + rg * 4 + r;
            if (row >= m) continue;
#pragma unroll
            for (int c = 0; c < CPT; ++c) {
              const int cell = cg * CPT + c;
              vpart[c] += (double)cvT[(int64_t)row * TC + cell] * (dg[c][r] + 2.0 * up[c][r]);
            }
          }
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < CPT; ++c) red[rg * TC + cg * CPT + c] = vpart[c];
        for (int cell = tid; cell < TC; cell += CT)
          cvT[(int64_t)n * TC + cell] = c0 + cell < C ? 1.0 : 0.0;
        __syncthreads();
        const double pnn = A.ws.l_arena[moff + (int64_t)n * m + n];
        for (int cell = tid; cell < TC; cell += CT) {
          double vv = 0.0;
          for (int g = 0; g < 16; ++g) vv += red[g * TC + cell];
          if (okf[cell]) cvar[cell] = vv - 0.25 * pnn;
        }
      }
    }
  } else {
    for (int cell = tid; cell < TC; cell += CT) {
      okf[cell] = 0;
      cvar[cell] = 0.0;
    }
  }
  __syncthreads();
  // ---- 5. nearest station, only for cells that fall back (the FP64 path
  // found it with the right-hand sides) ----
  if (any_bad && (sizeof(T) == 4 || failed)) {
    const int warp = tid >> 5, lane = tid & 31;
    for (int cell = warp; cell < TC; cell += CT / 32) {
      const int64_t gc = c0 + cell;
      if (gc >= C || okf[cell]) continue;
      int j = nnb_f64_warp(A.dom, idx, n, A.dom.cell_x[gc], A.dom.cell_y[gc]);
      if (lane == 0) nnb[cell] = j;
    }
  }
  __syncthreads();
  // ---- 6. estimates of every step: wide passes of 64 steps while many
  // remain, narrow passes for the rest ----
  const bool var_out = A.want_var && A.out.var != nullptr && !sk;
  OutT* est_out = reinterpret_cast<OutT*>(A.out.est);
  OutT* var_outp = reinterpret_cast<OutT*>(A.out.var);
  auto emit = [&](int cell, int vstep, double accv) {
    const int64_t gc = c0 + cell;
    if (gc >= C) return;
    const int j = A.sys.steps[st0 + vstep];
    const int64_t row = A.sys.out_row[j];
    double e;
    if (okf[cell]) {
      e = accv;
      if (!sk) {
        const double* bt = A.ws.beta + (int64_t)j * GA;
        e += bt[0];
        for (int k = 1; k < a; ++k) e += bt[k] * A.dom.cell_drift[(int64_t)(k - 1) * C + gc];
      }
    } else {
      e = A.vals[A.sys.val_off[j] + nnb[cell]];
    }
    e = clip_est(e, A.out);
    est_out[row * C + gc] = cast_out<OutT>(e);
    if (var_out) var_outp[row * C + gc] = cast_out<OutT>(cvar[cell]);
  };
  for (int v0 = 0; v0 < nsteps;) {
    const int rem = nsteps - v0;
    const bool wide = rem >= 32;
    const int nv = min(wide ? VB : NL::NV, rem);
    __syncthreads();
    for (int v = tid; v < VB; v += CT) {
      const bool valid = v < nv && !failed;
      const int64_t off = valid ? A.sys.val_off[A.sys.steps[st0 + v0 + v]] : 0;
      setv(v, A.ws.w_hat, A.ws.w_hi, A.ws.w_lo, off, valid);
    }
    if (wide) {
      double acc[CPT][4];
      if (!failed) {
        contract<T, TC, true>(cvT, Bs, vp64, vph, vpl, nv, n, n, acc);
      } else {
#pragma unroll
        for (int c = 0; c < CPT; ++c)
#pragma unroll
          for (int r = 0; r < 4; ++r) acc[c][r] = 0.0;
      }
      const int cg = tid % 16, rg = tid / 16;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int vl = rg * 4 + r;
        if (vl >= nv) continue;
#pragma unroll
        for (int c = 0; c < CPT; ++c) emit(cg * CPT + c, v0 + vl, acc[c][r]);
      }
    } else {
      double acc[NL::CPT][NL::VPT];
      if (!failed) {
        contract<T, TC, false>(cvT, Bs, vp64, vph, vpl, nv, n, n, acc);
      } else {
        acc[0][0] = 0.0;
      }
      const int vl = tid / TC;
      if (vl < nv) emit(tid % TC, v0 + vl, acc[0][0]);
    }
    v0 += nv;
  }
}

template <typename T, int TC>
static size_t cells_smem(int npad) {
  return (size_t)npad * TC * sizeof(T) + (size_t)KC * BSTR * 8 +
         (size_t)TC * GA * 8 + (size_t)TC * 8 + (size_t)TC * 4 * 2 +
         (size_t)3 * VB * sizeof(void*) + 16;
}

template <typename T, int TC, typename OutT>
static int launch_cells(const CellsArgs& A, cudaStream_t st) {
  int npad = (A.sys.max_n + GA + KC - 1) / KC * KC;
  size_t smem = cells_smem<T, TC>(npad);
  auto kern = k_krige_cells<T, TC, OutT>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return SPI_ERR_CUDA;
  int64_t tiles = (A.dom.n_cells + TC - 1) / TC;
  if (tiles > 0x7fffffff) return SPI_ERR_TOO_LARGE;
  dim3 grid((unsigned)tiles, (unsigned)A.sys.n_sys);
  kern<<<grid, CT, smem, st>>>(A, npad);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

// Largest cell tile whose shared memory fits.
template <typename T>
static int pick_tc(int max_n) {
  int npad = (max_n + GA + KC - 1) / KC * KC;
  const size_t cap = 227 * 1024;
  if (sizeof(T) == 4 && cells_smem<T, 64>(npad) <= cap) return 64;
  if (cells_smem<T, 32>(npad) <= cap) return 32;
  if (cells_smem<T, 16>(npad) <= cap) return 16;
  return 0;
}

// Systems whose right-hand-side tile does not fit in shared memory take the
// streamed kernel (estimates only; the OK variance needs the stored tile).
// tile: 0 = the largest cell tile that fits; 16, 32 or 64 = that tile
// (SPI_ERR_TOO_LARGE when it does not fit), the choice of the host's
// autotuner.
template <typename T, typename OutT>
static int dispatch_cells(const CellsArgs& A, int tile, cudaStream_t st) {
  // the mixed path's FP32 tier: double-float right-hand sides in the
  // streamed kernel whenever no CUDA-core variance pass is needed
  if (sizeof(T) == 4 &&
      (A.ws.cell_yy != nullptr || !A.want_var || A.sys.kind == SPI_KIND_SK))
    return launch_cells_stream(A, 1, st);
  if (tile) {
    const int npad = (A.sys.max_n + GA + KC - 1) / KC * KC;
    const size_t cap = 227 * 1024;
    if (tile == 64 && cells_smem<T, 64>(npad) <= cap) return launch_cells<T, 64, OutT>(A, st);
    if (tile == 32 && cells_smem<T, 32>(npad) <= cap) return launch_cells<T, 32, OutT>(A, st);
    if (tile == 16 && cells_smem<T, 16>(npad) <= cap) return launch_cells<T, 16, OutT>(A, st);
    return SPI_ERR_TOO_LARGE;
  }
  int tc = pick_tc<T>(A.sys.max_n);
  if (tc == 64) return launch_cells<T, 64, OutT>(A, st);
  if (tc == 32) return launch_cells<T, 32, OutT>(A, st);
  if (tc == 16) return launch_cells<T, 16, OutT>(A, st);
  if (A.want_var && A.sys.kind != SPI_KIND_SK) return SPI_ERR_TOO_LARGE;
  return launch_cells_stream(A, sizeof(T) == 8 ? 0 : 1, st);
}

__global__ void k_split_f64(const double* __restrict__ x, float* __restrict__ hi,
                            float* __restrict__ lo, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = x[i];
    float h = (float)v;
    hi[i] = h;
    lo[i] = (float)(v - (double)h);
  }
}

}  // namespace spi

using namespace spi;

extern "C" int spi_split_f64(const double* x, float* hi, float* lo, int64_t n,
                             spi_stream_t stream) {
  if (n < 0) return SPI_ERR_ARG;
  if (n == 0) return SPI_OK;
  if (!x || !hi || !lo) return SPI_ERR_ARG;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_split_f64<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(x, hi, lo, n);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

extern "C" int spi_krige_cells_tiled(const spi_domain_t* dom, const spi_systems_t* sys,
                                     const double* vals, const spi_krige_ws_t* ws,
                                     int32_t want_var, int32_t precision, int32_t route_filter,
                                     double cond_split, const spi_out_t* out, int32_t tile,
                                     spi_stream_t stream) {
  if (!dom || !sys || !out || !ws) return SPI_ERR_ARG;
  if (tile != 0 && tile != 16 && tile != 32 && tile != 64) return SPI_ERR_ARG;
  if (sys->n_sys < 0 || sys->n_sys > 65535) return SPI_ERR_TOO_LARGE;
  if (dom->n_drift < 0 || dom->n_drift > SPI_MAX_DRIFT) return SPI_ERR_TOO_LARGE;
  if (route_filter < 0 || route_filter > 2) return SPI_ERR_ARG;
  if (precision != 0 && precision != 1) return SPI_ERR_ARG;
  if (sys->n_sys == 0 || dom->n_cells == 0) return SPI_OK;
  if (!vals || !out->est || !ws->route || !ws->shift || !ws->beta || !ws->s_inv ||
      !ws->g_colsum || !ws->l_arena || !ws->cond)
    return SPI_ERR_ARG;
  if (!ws->w_hat || !ws->g_cols) return SPI_ERR_ARG;
  // Linv (and its FP32 pair) only for the OK variance
  if (want_var && !ws->linv_arena) return SPI_ERR_ARG;
  if (precision == 1 && (!dom->cell_split || !dom->stn_split || !ws->g_hi || !ws->g_lo ||
                         !ws->w_hi || !ws->w_lo))
    return SPI_ERR_ARG;
  if (precision == 1 && want_var && !ws->cell_yy && (!ws->linv_hi || !ws->linv_lo))
    return SPI_ERR_ARG;
  // routed systems are computed in FP64 only
  if (precision == 1 && route_filter != 1) return SPI_ERR_ARG;
  CellsArgs A;
  A.dom = *dom;
  A.sys = *sys;
  A.ws = *ws;
  A.vals = vals;
  A.want_var = want_var ? 1 : 0;
  A.route_filter = route_filter;
  A.cond_split = cond_split;
  A.out = *out;
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == 0)
    return out->out_f64 ? dispatch_cells<double, double>(A, tile, st)
                        : dispatch_cells<double, float>(A, tile, st);
  return out->out_f64 ? dispatch_cells<float, double>(A, tile, st)
                      : dispatch_cells<float, float>(A, tile, st);
}

extern "C" int spi_krige_cells(const spi_domain_t* dom, const spi_systems_t* sys,
                               const double* vals, const spi_krige_ws_t* ws, int32_t want_var,
                               int32_t precision, int32_t route_filter, double cond_split,
                               const spi_out_t* out, spi_stream_t stream) {
  return spi_krige_cells_tiled(dom, sys, vals, ws, want_var, precision, route_filter,
                               cond_split, out, 0, stream);
}

namespace spi {
__global__ void k_split_coords(const double* __restrict__ x, const double* __restrict__ y,
                               int64_t n, double ox, double oy, double res,
                               float4* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double dx = x[i] - ox, dy = y[i] - oy;
    float xh, yh;
    if (res > 0.0) {
      xh = (float)(rint(dx / res) * res);
      yh = (float)(rint(dy / res) * res);
    } else {
      xh = (float)dx;
      yh = (float)dy;
    }
    out[i] = make_float4(xh, (float)(dx - (double)xh), yh, (float)(dy - (double)yh));
  }
}
}  // namespace spi

extern "C" int spi_split_coords(const double* x, const double* y, int64_t n, double ox,
                                double oy, double res, float* out, spi_stream_t stream) {
  if (n < 0) return SPI_ERR_ARG;
  if (n == 0) return SPI_OK;
  if (!x || !y || !out || (reinterpret_cast<uintptr_t>(out) & 15) || !(res >= 0.0))
    return SPI_ERR_ARG;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  spi::k_split_coords<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
      x, y, n, ox, oy, res, reinterpret_cast<float4*>(out));
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}

namespace spi {
// One CTA per system: the largest probe discrepancy over its steps.
__global__ __launch_bounds__(256) void k_tier(spi_systems_t sys, spi_krige_ws_t ws, int64_t P,
                                              const double* __restrict__ e64,
                                              const double* __restrict__ e32,
                                              const double* __restrict__ v64,
                                              const double* __restrict__ v32,
                                              const double* __restrict__ v32d, double tol_e,
                                              double tol_v, double cap, double cap_d,
                                              const int32_t* __restrict__ tc_err,
                                              int32_t* tier, double* disc) {
  const int s = blockIdx.x;
  __shared__ double red[3][256];
  // a timed-out tensor-core wait (spi_krige_var_tc) leaves var32 partly
  // unwritten: every system then stays in FP64
  const bool fr = fp32_route(ws.route[s], sys.kind == SPI_KIND_SK) && !(tc_err && *tc_err);
  const bool cand = fr && ws.cond[s] <= cap;
  const bool cand_d = fr && v32d != nullptr && ws.cond[s] <= cap_d;
  const double inf = __longlong_as_double(0x7ff0000000000000LL);
  auto gap = [&](double a, double r) {
    return isnan(a) != isnan(r) ? inf : (isnan(a) ? 0.0 : fabs(a - r));
  };
  double de = 0.0, dv = 0.0, dd = 0.0;
  if (cand || cand_d) {
    for (int64_t si = sys.step_off[s]; si < sys.step_off[s + 1]; ++si) {
      const int64_t row = sys.out_row[sys.steps[si]];
      for (int64_t c = threadIdx.x; c < P; c += blockDim.x) {
        const int64_t o = row * P + c;
        de = fmax(de, gap(e32[o], e64[o]));
        if (v64 && v32 && cand) dv = fmax(dv, gap(v32[o], v64[o]));
        if (v64 && cand_d) dd = fmax(dd, gap(v32d[o], v64[o]));
      }
    }
  }
  red[0][threadIdx.x] = de;
  red[1][threadIdx.x] = dv;
  red[2][threadIdx.x] = dd;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int q = 0; q < 3; ++q) red[q][threadIdx.x] = fmax(red[q][threadIdx.x], red[q][threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    de = red[0][0];
    dv = red[1][0];
    dd = red[2][0];
    int t = 0;
    if (cand && de <= tol_e && dv <= tol_v)
      t = 1;
    else if (cand_d && v64 && de <= tol_e && dd <= tol_v)
      t = 2;
    tier[s] = t;
    if (disc) {
      const double nan = __longlong_as_double(0x7ff8000000000000LL);
      disc[3 * s] = (cand || cand_d) ? de : nan;
      disc[3 * s + 1] = cand ? dv : nan;
      disc[3 * s + 2] = cand_d ? dd : nan;
    }
  }
}
}  // namespace spi

extern "C" int spi_krige_tier(const spi_systems_t* sys, const spi_krige_ws_t* ws, int64_t n_probe,
                              const double* est64, const double* est32, const double* var64,
                              const double* var32, const double* var32_df, double tol_est,
                              double tol_var, double cond_cap, double cond_cap_df,
                              const int32_t* tc_err, int32_t* tier, double* disc,
                              spi_stream_t stream) {
  if (!sys || !ws || !tier || n_probe < 0) return SPI_ERR_ARG;
  if (sys->n_sys < 0 || sys->n_sys > 65535) return SPI_ERR_TOO_LARGE;
  if (sys->n_sys == 0) return SPI_OK;
  if (n_probe > 0 && (!est64 || !est32)) return SPI_ERR_ARG;
  if (!ws->route || !ws->cond || !sys->step_off || !sys->steps || !sys->out_row)
    return SPI_ERR_ARG;
  spi::k_tier<<<sys->n_sys, 256, 0, (cudaStream_t)stream>>>(
      *sys, *ws, n_probe, est64, est32, var64, var32, var32_df, tol_est, tol_var, cond_cap,
      cond_cap_df, tc_err, tier, disc);
  SPI_LAUNCH_CHECK();
  return SPI_OK;
}
