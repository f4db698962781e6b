/*
 * spinterps_gb300 -- C ABI of the GB300 (sm_103a) gridded-interpolation path.
 *
 * Every entry point takes plain pointers and sizes. Arrays marked "device"
 * are CUDA device pointers (for example torch tensors' data_ptr()); all
 * launches go onto the caller's stream and are stream-ordered (no entry
 * point synchronises unless stated). The caller owns every buffer,
 * including the workspace. Every function returns an spi_status; no C++
 * exception crosses this boundary. Not reentrant on one stream: calls that
 * share a workspace must be ordered on one stream.
 *
 * Matrices are row-major and C-contiguous, like the typed memoryviews
 * (double[:, ::1]) of the reference's Cython kernels.
 */
#ifndef SPINTERPS_GB300_H
#define SPINTERPS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *spi_stream_t; /* same object as cudaStream_t */

typedef enum {
    SPI_OK = 0,
    SPI_ERR_ARG = 1,        /* null pointer, negative size, bad flag */
    SPI_ERR_VG = 2,         /* variogram string does not parse / unknown model */
    SPI_ERR_CUDA = 3,       /* a CUDA launch or call failed */
    SPI_ERR_WORKSPACE = 4,  /* caller's workspace is too small */
    SPI_ERR_TOO_LARGE = 5   /* a size exceeds a documented maximum */
} spi_status;

/* Variogram model codes: the model names of cyth/interpmthds.pyx:86-95. */
enum {
    SPI_VG_RNG = 0, SPI_VG_NUG = 1, SPI_VG_SPH = 2, SPI_VG_EXP = 3,
    SPI_VG_LIN = 4, SPI_VG_GAU = 5, SPI_VG_POW = 6, SPI_VG_HOL = 7
};

#define SPI_MAX_VG_COMP 4

/* One parsed variogram string: up to SPI_MAX_VG_COMP nested components,
 * range already clamped to max(1e-5, range). */
typedef struct {
    int32_t n_comp;
    int32_t code[SPI_MAX_VG_COMP];
    double sill[SPI_MAX_VG_COMP];
    double range[SPI_MAX_VG_COMP];
} spi_vg_t;

/* Kriging system kinds. */
enum { SPI_KIND_OK = 0, SPI_KIND_SK = 1, SPI_KIND_EDK = 2 };

/* ---- host helpers ------------------------------------------------------ */

/* Parse 's1 M1(r1) + s2 M2(r2)' with the split rules of fill_vg_var_arr
 * (replaces the parse in cyth/interpmthds.pyx:174-184): Python bytes.split
 * semantics, numbers in Python float()'s grammar, at most SPI_MAX_VG_COMP
 * components (SPI_ERR_TOO_LARGE otherwise, before any other check). */
int spi_parse_vg(const char *vg_str, spi_vg_t *out);

/* misc.py:1074-1105 check_full_nuggetness: *out = 1 when the total sill or
 * the largest range is <= min_vg_val. */
int spi_check_full_nuggetness(const char *vg_str, double min_vg_val, int32_t *out);

/* Library version string. */
const char *spi_version(void);

/* The CUDA error behind the calling thread's last SPI_ERR_CUDA status, as
 * "name: description" (cudaGetErrorName / cudaGetErrorString), else the
 * runtime's pending error; "" when there is none. Reading it clears it. */
const char *spi_cuda_error(void);

/* ---- drop-ins for the reference's Cython kernels (all device arrays) ---- */

/* Replaces fill_dists_2d_mat (cyth/interpmthds.pyx:123-143):
 * dists[i, j] = ((x1s[i]-x2s[j])^2 + (y1s[i]-y2s[j])^2)^0.5, shape [n1, n2]. */
int spi_fill_dists_2d_mat(const double *x1s, const double *y1s, int64_t n1,
                          const double *x2s, const double *y2s, int64_t n2,
                          double *dists, spi_stream_t stream);

/* Replaces fill_vg_var_arr (cyth/interpmthds.pyx:146-226): out = sum over
 * components of covar*sill + (covar ? -1 : +1)*gamma(dists); entries
 * <= min_vg_val set to 0; with diag_mat_flag the upper triangle is
 * computed and mirrored. vg is a HOST pointer. */
int spi_fill_vg_var_arr(const double *dists, int64_t rows, int64_t cols,
                        double *out, int32_t covar_flag, int32_t diag_mat_flag,
                        const spi_vg_t *vg, double min_vg_val,
                        spi_stream_t stream);

/* Replaces copy_2d_arr_at_idxs (cyth/interpmthds.pyx:229-248):
 * subset[i, j] = arr[row_idxs[i], col_idxs[j]], subset row stride
 * subset_cols (the reference allocates add_rc extra columns). */
int spi_copy_2d_arr_at_idxs(const double *arr, int64_t arr_rows, int64_t arr_cols,
                            const int64_t *row_idxs, int64_t n_rows,
                            const int64_t *col_idxs, int64_t n_cols,
                            double *subset, int64_t subset_cols,
                            spi_stream_t stream);

/* ---- neighbour selection -------------------------------------------------
 *
 * Replaces SpInterpNeighborGrouping._get_nrst_neb_idxs / _get_pie_neb_idxs
 * (interp/grps.py:147-247, with sel_equidist_refs, cyth/interpmthds.pyx:
 * 811-890): idxs [n_dst, k] = each destination's neighbour station indices,
 * ascending. method 1 'nrst': the k = min(n_nebs, n_ref) nearest. method 2
 * 'pie': stations ranked by distance within n_pies angular sectors, taken
 * nearest-of-every-sector first, k = n_nebs (requires n_pies <= n_nebs <=
 * n_ref). Equal distances order by index (the reference: numpy's argsort).
 * Limits: k <= 64, n_pies <= 16, n_pies * n_nebs <= 512. */
int spi_neb_select(int32_t method, const double *dst_x, const double *dst_y, int64_t n_dst,
                   const double *ref_x, const double *ref_y, int32_t n_ref, int32_t n_nebs,
                   int32_t n_pies, int32_t *idxs, spi_stream_t stream);

/* ---- batched step engine ------------------------------------------------
 *
 * Replaces the per-group loop of SpInterpSteps._get_interp
 * (interp/steps.py:245-435) for all time steps at once. The host groups
 * steps into "systems": one kriging system per (station set, variogram,
 * kind). Station sets are lists of station indices (int32, ascending),
 * concatenated, with int64 offsets. */

/* Stations, cells and drifts shared by every system (device arrays). */
typedef struct {
    int64_t n_stns;
    const double *stn_x, *stn_y;   /* [n_stns] */
    int64_t n_cells;
    const double *cell_x, *cell_y; /* [n_cells] */
    int32_t n_drift;               /* k for EDK, else 0 */
    const double *stn_drift;       /* [n_stns, n_drift] or NULL */
    const double *cell_drift;      /* [n_drift, n_cells] or NULL */
    double min_vg_val;
    /* FP32 double-float copies of the coordinates minus a common origin,
     * [n][4] = (x_hi, x_lo, y_hi, y_lo), 16-byte aligned; made by
     * spi_split_coords and required only by the precision-1 kernels. */
    const float *stn_split, *cell_split;
    /* the res of spi_split_coords (the heads' grid), or 0 when unknown:
     * with it the precision-1 kernels take a failed cell's nearest station
     * from their own squared distances wherever those decide it */
    double split_res;
} spi_domain_t;

/* out[i] = (x_hi, x_lo, y_hi, y_lo) with x_hi = (x[i] - ox) rounded to a
 * multiple of res and x_lo = (float)((x[i] - ox) - x_hi), likewise for y
 * (device arrays). res = 0: x_hi = (float)(x[i] - ox). With res a power of
 * two and every |x - ox| <= 2^22 res, heads are exact floats and so are
 * their differences: the double-float distance needs no TwoSum there. */
int spi_split_coords(const double *x, const double *y, int64_t n, double ox,
                     double oy, double res, float *out, spi_stream_t stream);

/* hi[i] = (float)x[i], lo[i] = (float)(x[i] - hi[i]) (device arrays): the
 * FP32 pair of the split-precision contractions, made once per system. */
int spi_split_f64(const double *x, float *hi, float *lo, int64_t n, spi_stream_t stream);

/* A batch of kriging systems (device arrays unless noted). Every system
 * lists the time steps that use it; step j reads its n station values at
 * val_off[j] of the values array (gathered in the system's station order),
 * writes output row out_row[j], and owns dual weights at the same offset. */
typedef struct {
    int32_t n_sys;
    int32_t kind;                  /* SPI_KIND_* for the whole batch */
    const int64_t *stn_off;        /* [n_sys + 1] offsets into stn_idx */
    const int32_t *stn_idx;        /* station indices of every system */
    const spi_vg_t *vg;            /* [n_sys] */
    const int64_t *mat_off;        /* [n_sys] offset (doubles) of each
                                      system's matrix in the arenas, 32-aligned,
                                      sized (n + SPI_MAX_DRIFT + 1)^2 */
    const int64_t *step_off;       /* [n_sys + 1] offsets into steps */
    const int32_t *steps;          /* step indices, grouped by system */
    const int64_t *val_off;        /* [n_steps] offset of step j's values */
    const int32_t *out_row;        /* [n_steps] output row of step j */
    int32_t max_n;                 /* max stations in one system */
} spi_systems_t;

/* Maximum drifts of EDK (a = 1 + n_drift Lagrange/drift rows). */
#define SPI_MAX_DRIFT 7
/* Largest exact-inverse system (rows m = n + Lagrange / drift rows) that
 * spi_krige_factor checks against numpy.linalg.pinv's cut-off, and the
 * scratch (doubles) that check needs: SPI_PINV_SLOTS systems at once, each
 * two m x m matrices. */
/* Iteration limit of the FP64 iterative refinement of the duals over an
 * FP32 factor (spi_krige_factor / spi_krige_duals with ws->l32). */
#define SPI_IR_MAX_ITERS 12
#define SPI_PINV_MAX_M 256
/* spi_krige_var_tc's packed chunks: 8 columns of Linv (the tensor cores'
 * K-step) as 3 TF32 tiles of 256 x 8, then the 8 stations' split
 * coordinates (float4 each) */
#define SPI_VAR_TC_KC 8
#define SPI_VAR_TC_CHUNK_FLOATS (3 * 256 * SPI_VAR_TC_KC + 4 * SPI_VAR_TC_KC)
/* spi_idw_cells_tc's packed chunks: 8 stations of 64 columns (32 steps x
 * value, mask) as 3 TF32 tiles, then the stations' split coordinates; one
 * chunk per 8 stations and group of 32 steps */
#define SPI_IDW_TC_CHUNK_FLOATS (3 * 64 * 8 + 4 * 8)
#define SPI_IDW_TC_PACK_FLOATS(n_stns, n_steps) \
    ((((int64_t)(n_steps) + 31) / 32) * (((int64_t)(n_stns) + 7) / 8) * SPI_IDW_TC_CHUNK_FLOATS)
#define SPI_PINV_SLOTS 16
#define SPI_PINV_SCRATCH_DOUBLES (SPI_PINV_SLOTS * 2 * SPI_PINV_MAX_M * SPI_PINV_MAX_M)

/* Per-batch workspace of the kriging entry points (device arrays, caller
 * owned). Arenas hold one matrix per system at sys->mat_off[s], sized for
 * (n + SPI_MAX_DRIFT + 1)^2 doubles; per-system arrays have n_sys entries;
 * w_hat has the layout of the values array; beta is [n_steps_total, GA] and
 * g_cols [total stations * GA], GA = SPI_MAX_DRIFT + 1. The float arrays are
 * FP32 (hi, lo) pairs of linv_arena, g_cols and w_hat (spi_split_f64),
 * read by the precision-1 cell kernel only. */
typedef struct {
    double *l_arena;     /* Cholesky factor L; for routed systems the
                            inverse of the reference's saddle matrix */
    double *linv_arena;  /* Linv = L^-1; NULL when no OK variance is wanted:
                            spi_krige_factor then forms no inverse and
                            estimates cond from triangular solves, and
                            spi_krige_duals solves with L */
    int32_t *status;     /* Cholesky: 0, or the 1-based failing pivot */
    int32_t *route;      /* 0 Cholesky path, 1 exact-inverse path,
                            2 singular (nearest-station fallback) */
    double *cond;        /* n * A_00 * ||Linv||_F^2 (>= cond_2(A)) */
    double *shift;       /* s of A = s 11' - Gamma (0 for SK) */
    double *w_hat;       /* per-step dual weights */
    double *beta;        /* per-step Lagrange / drift coefficients */
    double *g_cols;      /* per-system dual columns */
    double *s_inv;       /* per-system S^-1 [n_sys, GA * GA] */
    double *g_colsum;    /* per-system [n_sys, GA] */
    float *linv_hi, *linv_lo, *g_hi, *g_lo, *w_hi, *w_lo;
    double *cell_yy;     /* optional [n_sys, n_cells]: |Linv c|^2 of every cell
                            of the FP32-tier systems, written by
                            spi_krige_var_tc and read by the precision-1 cell
                            kernel instead of its own variance pass (NULL:
                            the cell kernel computes it) */
    int32_t *tier;       /* optional [n_sys]: 1 = the FP32 tier of the
                            precision-1 kernels with the tensor-core
                            variance, 2 = the FP32 tier with the
                            double-float variance, 0 = FP64
                            (spi_krige_tier); NULL: route 0 and
                            cond <= cond_split */
    int32_t *var_cells;  /* optional [n_sys]: the FP64 cell kernel adds the
                            cells whose exact-inverse variance (lambda =
                            P r, 2 m^2 FLOP per cell) it computed: only the
                            cells that pass the sum check where few of a
                            tile do, every cell of the tile where more than
                            a quarter do (NULL: not counted) */
    double *pinv_scratch; /* optional, SPI_PINV_SCRATCH_DOUBLES doubles: lets
                            spi_krige_factor take numpy.linalg.pinv's answer
                            for exact-inverse systems of m <= SPI_PINV_MAX_M
                            rows that pinv treats as singular (see
                            spi_krige_factor); NULL: Gauss-Jordan only */
    int32_t *pinv_used;  /* optional [n_sys]: 1 where that pinv replaced the
                            Gauss-Jordan inverse, else 0 */
    float *l32;          /* optional arena of the same layout as l_arena
                            (floats): with it, and without linv_arena,
                            spi_krige_factor factors every system in FP32
                            first; systems whose FP32 factor succeeds with
                            cond <= cond_ir keep it, and spi_krige_duals
                            solves with it by FP64 iterative refinement
                            (residuals b - A x in FP64 with the full
                            matrix A kept in l_arena); the others are
                            factored in FP64 as without it */
    int32_t *ir;         /* [n_sys] with l32: 1 where the FP32 factor is
                            kept, 2 where its refinement did not converge
                            and the system was factored and solved again in
                            FP64, 0 where it was factored in FP64 from the
                            start */
    int32_t *ir_iters;   /* [n_sys] with l32: refinement corrections the
                            duals took (the largest over their right-hand
                            sides; bit 30 set where the componentwise
                            backward error did not reach sqrt(n) eps in
                            SPI_IR_MAX_ITERS, or stopped halving) */
    double cond_ir;      /* with l32: the largest condition estimate that
                            tries the FP32 factor (1e10 if 0; the estimate
                            overstates the condition, and systems whose
                            refinement fails fall back to FP64) */
    double *gj_scratch;  /* optional, 1 + 2 * (total stations) + (2 * GA +
                            1) * n_sys doubles: spi_krige_factor then runs the
                            exact-inverse path's Gauss-Jordan elimination
                            step by step over the whole GPU (two launches per
                            step, the same arithmetic); NULL: one CTA per
                            system */
    float *linv_tc;      /* Linv's three TF32 terms per system, packed by
                            spi_krige_var_tc_pack in the tensor cores'
                            shared-memory tile order: per block of 256 rows,
                            per chunk of SPI_VAR_TC_KC columns (up to the
                            block's last row), 3 tiles of 256 x 8 TF32
                            values and the chunk's stations
                            (SPI_VAR_TC_CHUNK_FLOATS floats, 16-byte
                            aligned); required by spi_krige_var_tc */
    const int64_t *linv_tc_off; /* [n_sys + 1]: first packed chunk of each
                            system in linv_tc (see spi_krige_var_tc_pack) */
} spi_krige_ws_t;

/* Build and factor every system of the batch in FP64.
 * Cholesky path: A = s*11' - Gamma for OK/EDK (s = total sill, Gamma
 * filled exactly as fill_vg_var_arr with covar 0, diagonal included), the
 * covariance fill for SK; A = L L', Linv = L^-1 (with ws->linv_arena; without
 * it, cond uses ||Linv||_F^2 = trace(A^-1) estimated as the mean of |L^-1 g|^2
 * over 8 fixed Rademacher vectors g). Under sum(lambda) = 1 the
 * weights of [[A, F], [F', 0]] equal those of the reference's
 * [[Gamma, F], [F', 0]] (Lagrange multipliers change sign).
 * Systems whose Cholesky fails, whose cond exceeds cond_max, or (EDK)
 * whose drift rows are linearly dependent with the unbiasedness row
 * (F'F singular to 1e-12: their Schur complement is singular; status is
 * then n + 1) take the exact-inverse path (route 1): the reference's own
 * saddle matrix
 * (interp/steps.py:170-243) is inverted in place by Gauss-Jordan with
 * partial pivoting, i.e. numpy.linalg.pinv (interp/steps.py:351) without
 * its singular-value cut-off (1e-15 * s_max, numpy's default rcond), which
 * is the same matrix whenever the cut-off removes nothing. On the
 * exact-inverse path ws->cond holds ||M||_F ||P||_F (M the saddle matrix,
 * P its computed inverse), an upper bound of M's condition number.
 * With ws->pinv_scratch, a system of m <= SPI_PINV_MAX_M rows whose
 * Gauss-Jordan inverse failed (a zero pivot) or whose ||M||_F ||P||_F
 * exceeds 1e15 -- those pinv may cut -- is also diagonalised by a
 * parallel cyclic Jacobi eigen-decomposition (M is symmetric, so its
 * singular values are the |eigenvalues|). When the spectrum has
 * eigenvalues under pinv's cut-off 1e-15 max|lambda| and none within a
 * factor 30 of it either side (a rank deficiency with a gap: duplicated
 * stations, drifts collinear with the constant, badly scaled unbounded
 * models), pinv's answer is stable and the truncated pseudo-inverse
 * V diag(1/lambda) V' replaces the Gauss-Jordan inverse (route 1,
 * ws->pinv_used = 1); without a gap the cut falls inside rounding noise, no
 * solver reproduces the reference's pinv there, and the Gauss-Jordan
 * inverse is kept. Without the scratch (or above SPI_PINV_MAX_M), an exactly
 * singular saddle matrix gives route 2. */
int spi_krige_factor(const spi_domain_t *dom, const spi_systems_t *sys,
                     const spi_krige_ws_t *ws, double cond_max,
                     spi_stream_t stream);

/* Per-system and per-step dual quantities (FP64).
 * Route 0, with F = [1 | drift] (n x a, a = 1 + n_drift; SK: a = 0):
 *   E = Linv F, G = Linv' E = A^-1 F, S = E'E; per step with values z:
 *   OK/EDK: w_hat = A^-1 z - G beta, beta = S^-1 G'z;  SK: w_hat = A^-1 z,
 *   G = A^-1 1. g_colsum = 1'G.
 * Route 1, with P the inverse saddle matrix: w = P [z; 0] split into
 * w_hat = w[:n], beta = w[n:]; u = P [1; 0] split into g_cols column 0 =
 * u[:n], g_colsum = u[n:]. */
int spi_krige_duals(const spi_domain_t *dom, const spi_systems_t *sys,
                    const double *vals, const spi_krige_ws_t *ws,
                    spi_stream_t stream);

/* Output description of the cell kernels. */
typedef struct {
    int32_t out_f64;               /* 1: est/var are double, 0: float */
    void *est;                     /* [n_out_rows, n_cells] */
    void *var;                     /* [n_out_rows, n_cells] or NULL (OK only) */
    int32_t clip_min_on, clip_max_on;
    double clip_min, clip_max;     /* _mod_min_max on the estimate */
} spi_out_t;

/* Kriging estimates (and OK variances when want_var) for every cell of
 * every step of a system batch. precision 0: FP64 throughout; 1: the FP32
 * tier, double-float right-hand sides against the FP32 (hi, lo) pairs of
 * the FP64 duals in ws, accumulated as double-floats (the streamed kernel;
 * the OK variance from ws->cell_yy, or, without it, a split-FP32 pass over
 * Linv's pair). ws->linv_arena (and its pair) is needed only with
 * want_var. route_filter: 0 all systems; 1 the FP32-tier systems
 * (ws->tier != 0, or without ws->tier route 0 with cond <= cond_split);
 * 2 every other system. A
 * mixed-precision job runs precision 1 with filter 1, then precision 0 with
 * filter 2: ill-conditioned and routed systems are always computed in FP64
 * (precision 1 accepts only filter 1).
 * Route 0, per cell with c the right-hand side in covariance form and
 * f = [1, cell drifts]: nu = S^-1 (G'c - f), sum(lambda) = (G'c)_0 -
 * (1'G) nu, est_j = c'w_hat_j + f'beta_j, OK variance = s sum(lambda) -
 * |Linv c|^2 + nu (G'c)_0 - 2 nu, i.e. the reference's lambda'gamma + 2 mu
 * (interp/steps.py:429-434). Route 1, with r = [gamma, f]: est_j = r'w_j,
 * sum(lambda) = r'u, variance lambda'r + lambda_n with lambda = P r (the
 * reference's primal formula). Cells failing numpy.isclose(sum(lambda), 1),
 * and every cell of a route-2 system, take the nearest station's value
 * with variance 0 (interp/steps.py:363-426). */
int spi_krige_cells(const spi_domain_t *dom, const spi_systems_t *sys,
                    const double *vals, const spi_krige_ws_t *ws,
                    int32_t want_var, int32_t precision, int32_t route_filter,
                    double cond_split, const spi_out_t *out, spi_stream_t stream);

/* spi_krige_cells with the cell tile of the shared-memory kernel chosen by
 * the caller: tile 0 = the largest of 64 / 32 / 16 cells whose right-hand
 * sides fit in shared memory (spi_krige_cells itself), 16 / 32 / 64 = that
 * tile, SPI_ERR_TOO_LARGE when it does not fit (nothing is launched). Used
 * by the host's autotuner, which times the tiles on a plan's first
 * execution per station-count bucket. No reference counterpart (the
 * reference has no tiles). */
int spi_krige_cells_tiled(const spi_domain_t *dom, const spi_systems_t *sys,
                          const double *vals, const spi_krige_ws_t *ws, int32_t want_var,
                          int32_t precision, int32_t route_filter, double cond_split,
                          const spi_out_t *out, int32_t tile, spi_stream_t stream);

/* Tier of every system of a factored batch from a probe: est/var fields
 * [rows, n_probe] (row = sys->out_row[step]) of the same probe cells
 * computed by the FP64 kernel (route_filter 0) and by the FP32 tier
 * (precision 1, route_filter 1): var32 with the tensor-core variance
 * (spi_krige_var_tc), var32_df (optional) with the double-float one
 * (spi_krige_var_df). tier[s] = 1 when the system is on the Cholesky path,
 * cond <= cond_cap, and over its steps and the probe cells |est32 - est64|
 * <= tol_est and |var32 - var64| <= tol_var; else 2 when cond <= cond_cap_df
 * and the estimates and |var32_df - var64| pass the same tolerances; else
 * 0 (var arrays may be NULL; a NaN in one field and not the other fails).
 * disc (optional, [n_sys, 3]): each system's largest estimate, tensor-core
 * variance and double-float variance discrepancy over the probe (NaN where
 * not a candidate, +inf for a NaN mismatch). tc_err (optional, device):
 * the err_flag given to spi_krige_var_tc for the probe; when it is set, a
 * tensor-core wait timed out and var32 is incomplete, so every system gets
 * tier 0. The
 * mixed path's a-posteriori error control: the FP32 rounding of the
 * right-hand sides enters the estimate as sum_i dc_i w_i, which the dual
 * weights can amplify far beyond what the condition number predicts. */
int spi_krige_tier(const spi_systems_t *sys, const spi_krige_ws_t *ws, int64_t n_probe,
                   const double *est64, const double *est32, const double *var64,
                   const double *var32, const double *var32_df, double tol_est,
                   double tol_var, double cond_cap, double cond_cap_df,
                   const int32_t *tc_err, int32_t *tier, double *disc, spi_stream_t stream);

/* The OK variance term |Linv c|^2 of every cell of the FP32-tier systems
 * (ws->tier, else route 0 and cond <= cond_split; kinds OK / EDK) on the tensor cores
 * (tcgen05 kind::tf32: Linv as three TF32 terms b0 + b1 + b2, the right-hand
 * sides as two a0 + a1, five MMAs per product a0b0 + a0b1 + a1b0 + a0b2 +
 * a1b1, FP32 accumulation in tensor memory), into ws->cell_yy [n_sys, n_cells].
 * Requires ws->linv_tc (spi_krige_var_tc_pack) and the domain's split
 * coordinates. Replaces the variance half of interp/steps.py:403-435
 * (var = lambda'r + mu per cell and step). */
int spi_krige_var_tc(const spi_domain_t *dom, const spi_systems_t *sys,
                     const spi_krige_ws_t *ws, double cond_split, int32_t *err_flag,
                     spi_stream_t stream);

/* Pack Linv (ws->linv_hi / linv_lo, spi_split_f64 of linv_arena) of every
 * route-0 system into ws->linv_tc for spi_krige_var_tc: Linv = b0 + b1 + b2
 * in TF32 terms (b0 the TF32 rounding of hi, b1 of the remainder plus lo,
 * b2 what is left), each 256-row block's rows 0..255 by chunks of
 * SPI_VAR_TC_KC columns up to the block's last row, each chunk 3 tiles of
 * 256 x 8 values in the no-swizzle K-major core-matrix order the MMA reads,
 * followed by the chunk's stations' split coordinates (dom->stn_split; one
 * bulk copy per chunk). System s's chunks start at chunk
 * ws->linv_tc_off[s]; a system of n stations has sum over blocks b of
 * ceil(min(n, 256 (b + 1)) / 8) chunks. */
int spi_krige_var_tc_pack(const spi_domain_t *dom, const spi_systems_t *sys,
                          const spi_krige_ws_t *ws, spi_stream_t stream);

/* The same term |Linv c|^2 in double-float on the FP32 pipe (every product
 * split by FMA, sums by TwoSum: ~1e-9 of the sill), into ws->cell_yy, for
 * the systems with ws->tier[s] == 2 (without ws->tier: route 0 and cond <=
 * cond_cap; kinds OK / EDK): the FP32 tier's variance where the tensor-core
 * one misses the probe's tolerance. Requires ws->linv_hi / linv_lo and the
 * domain's split coordinates. */
int spi_krige_var_df(const spi_domain_t *dom, const spi_systems_t *sys,
                     const spi_krige_ws_t *ws, double cond_cap, spi_stream_t stream);

/* IDW (interp/steps.py:293-313, cyth/interpmthds.pyx:784-808) for every
 * cell of the listed steps. data [n_steps_total, n_stns] holds every
 * station's value, NaN where missing (the reference's data_df row). For
 * list entry k: j = steps[k] is the data row, out_row[k] the output row;
 * flag[j] = any present value >= min_value_to_interp_thresh (else the step
 * mean means[j] is written). Weights (d / d_ref)^-idw_exp per cell and
 * station are shared by every step; each step is a masked contraction pair
 * over stations, so missing stations drop out exactly. A cell on a station
 * present at the step gets NaN, as the reference's 1/0 weight does. Steps
 * with fewer than two stations must not be listed (the reference copies
 * the single value; use spi_fill_rows). precision 0: FP64; 1: FP32 weights
 * contracted against the FP32 (hi, lo) pair of data (data_hi / data_lo,
 * from spi_split_f64; NaN stays NaN in hi) with FP64 accumulation; requires
 * dom->stn_split / cell_split. */
int spi_idw_cells(const spi_domain_t *dom, int32_t n_steps, const int32_t *steps,
                  const int32_t *out_row, const double *data, const float *data_hi,
                  const float *data_lo, const uint8_t *flag, const double *means,
                  double idw_exp, int32_t precision, const spi_out_t *out,
                  spi_stream_t stream);

/* The same IDW on the tensor cores (tcgen05), for the mixed path: per group
 * of 32 listed steps one GEMM D [cells x 64] = W [cells x n_stns] B
 * [n_stns x 64], B's columns (2t, 2t + 1) = (the step's values with 0
 * where missing, its mask), the weights as in precision 1 (FP32 distances
 * from dom->stn_split / cell_split) split into two TF32 terms, B into
 * three; FP32 accumulation in tensor memory (the large products in three
 * accumulators taking every third 8-station chunk, the corrections in a
 * fourth, added in FP64). pack: a 16-byte aligned device
 * buffer of at least SPI_IDW_TC_PACK_FLOATS(n_stns, n_steps) floats that the
 * call fills with B (two launches: the pack, the contraction). A timed-out
 * wait sets *err_flag (device) and leaves NaN in the CTA's fields. Other
 * arguments and semantics as spi_idw_cells. */
int spi_idw_cells_tc(const spi_domain_t *dom, int32_t n_steps, const int32_t *steps,
                     const int32_t *out_row, const double *data, const uint8_t *flag,
                     const double *means, double idw_exp, float *pack, int64_t pack_floats,
                     const spi_out_t *out, int32_t *err_flag, spi_stream_t stream);

/* NNB (interp/steps.py:285-291): value of the first present station of
 * minimum distance (np.argmin order), per cell and listed step. */
int spi_nnb_cells(const spi_domain_t *dom, int32_t n_steps, const int32_t *steps,
                  const int32_t *out_row, const double *data, const spi_out_t *out,
                  spi_stream_t stream);

/* Fill whole output rows with per-row constants: est[row[j], :] = v[j]
 * (clipped like the estimates), var[row[j], :] = vv[j] when var and vv are
 * non-NULL (NaN allowed). Used for steps the reference answers without
 * interpolating: one station (its value), no value above the threshold or a
 * nugget-only variogram (the step mean, variance 0). */
int spi_fill_rows(int32_t n_rows, const int32_t *row, const double *v,
                  const double *vv, int64_t n_cells, const spi_out_t *out,
                  spi_stream_t stream);

/* Leave-one-out cross-validation residuals of every station of every step
 * of a factored batch (after spi_krige_factor and spi_krige_duals):
 * resid (layout of the values array) = z_i minus the kriging estimate at
 * station i from the other stations, in closed form, w_hat_i / (P11)_ii.
 * Route-0 systems only (NaN elsewhere). Cross-validation itself has no
 * counterpart in the reference's step engine; it judges fitted variograms. */
int spi_krige_loo(const spi_domain_t *dom, const spi_systems_t *sys,
                  const spi_krige_ws_t *ws, double *resid, spi_stream_t stream);

/* ---- variogram fitting --------------------------------------------------
 *
 * Replaces variograms/vgs.py (Variogram, with the settings of
 * variograms/fitvgs.py:187-206) for a batch of steps. Points of step s are
 * at pt_off[s] .. pt_off[s+1] of x, y, z (the stations with a value). */

/* Workspace of spi_vg_empirical (device arrays): pd, pp, sd sized for all
 * pairs of the batch (sum of n_s (n_s - 1) / 2), bcnt, bstart, bcur for all
 * buckets (sum of bucket counts); bcnt must be zero on entry. */
typedef struct {
    double *pd;       /* pair distances, pair order */
    int32_t *pp;      /* pair indices sorted by distance */
    double *sd;       /* sorted distances */
    int32_t *bcnt, *bstart, *bcur;
} spi_vg_emp_ws_t;

/* Empirical variograms (vgs.py:311-391, 495-520, 597-659 with a numeric
 * mdr): all pairs i > j, sorted by distance, cut at mdr * max distance,
 * bins of nk consecutive pairs with their mean distance, the robust
 * (Cressie-Hawkins) estimate and the pair count. pair_off / bkt_off [n+1]
 * are the per-step offsets of pairs and distance buckets, dmax[s] an upper
 * bound of step s's pair distances, max_pairs / max_buckets the largest
 * per-step counts. Outputs at bin_off[s] (room for ceil(pairs / nk) bins):
 * bin_h, bin_g, bin_n; n_bins[s] bins used, max_dist[s] = mdr * max
 * distance. */
int spi_vg_empirical(int32_t n_steps, const int64_t *pt_off, const double *x, const double *y,
                     const double *z, const int64_t *pair_off, const int64_t *bkt_off,
                     const double *dmax, int64_t max_pairs, int64_t max_buckets, int32_t nk,
                     double mdr, const spi_vg_emp_ws_t *ws, const int64_t *bin_off,
                     double *bin_h, double *bin_g, double *bin_n, int32_t *n_bins,
                     double *max_dist, spi_stream_t stream);

/* One differential-evolution problem: fit n_comp nested models (codes) to
 * step `step`'s empirical variogram. Parameters per component are (range,
 * sill) with the bounds of vgs.py:731-753: Pow (1e-5, 2) x (1e-5, var2);
 * the nugget placed first in a multi-model permutation fixed at (h_0,
 * gamma_0) when fixed_first; otherwise (h_0, 1e9) x (1e-5, var2), var2 = 2 *
 * variance of the step's values. With warm != 0 the initial population is
 * drawn in [warm_lo, warm_hi] (unit-cube coordinates within the bounds)
 * instead of the whole box. */
typedef struct {
    int32_t step;
    int32_t n_comp;
    int32_t code[2];
    int32_t fixed_first;
    int32_t warm;
    double var2;
    uint64_t seed;
    double warm_lo[4], warm_hi[4];
} spi_de_problem_t;

/* Differential evolution (scipy's best1bin scheme, population 50 D^2 for D
 * parameters, F dithered in [0.5, 1), CR 0.7) for every problem at once,
 * minimising sum over bins (gamma - model)^2 (vgs.py:661-678, no weights);
 * stops when std(energies) <= tol |mean(energies)| or after maxiter
 * generations. best_x [n_prob, 4] (range, sill per component), best_f the
 * FP64 objective at best_x, n_gen the generations used. n_comp must be 1 or
 * 2 (NaN results otherwise, and for steps without bins). */
int spi_vg_de(int32_t n_prob, const spi_de_problem_t *prob, const int64_t *bin_off,
              const int32_t *n_bins, const double *bin_h, const double *bin_g,
              int32_t maxiter, double tol, double *best_x, double *best_f, int32_t *n_gen,
              spi_stream_t stream);

/* Refined proposal of each problem's permutation (one free structure: X,
 * or Nug fixed at (h_0, gamma_0) + X; NaN for others and for steps without
 * bins): the least-squares sill (closed form, clipped to (1e-5, var2)) at
 * each range of a log grid over [r0 / span, r0 * span] (within (h_0,
 * 1e9)), refined by golden section. x [n_prob, 4] in spi_vg_de's layout, f
 * the objective there, noise the bins' scatter sum of squares
 * nb/(nb-1) * sum((g[i+1] - g[i])^2) / 2. No counterpart in the reference:
 * part of the learned warm start. */
int spi_vg_refine(int32_t n_prob, const spi_de_problem_t *prob, const int64_t *bin_off,
                  const int32_t *n_bins, const double *bin_h, const double *bin_g,
                  const double *r0, double span, double *x, double *f, double *noise,
                  spi_stream_t stream);

/* ---- learned warm start of the fitter ----------------------------------
 *
 * No counterpart in the reference: an MLP proposes each step's model
 * permutation and parameters so that the fitter's differential evolution
 * starts from a narrow box instead of the whole one (see spi_de_problem_t).
 * Device arrays, FP32. Network in -> h1 -> h2 -> out, tanh hidden layers,
 * parameters packed W1[in][h1], b1, W2[h1][h2], b2, W3[h2][out], b3
 * (spi_mlp_n_params of them); the first n_class outputs are class logits.
 * ws: B * (h1 + h2 + 2 * out + h2 + h1) floats. */

/* Features of step s (points at pt_off[s]): semivariance in n_bins (<= 64)
 * equal-width lag bins up to half the bounding-box diagonal, divided by the
 * variance. feat [n_steps, n_bins]. */
int spi_vg_features(int32_t n_steps, const int64_t *pt_off, const double *x, const double *y,
                    const double *z, int32_t n_bins, float *feat, spi_stream_t stream);

int64_t spi_mlp_n_params(int32_t in, int32_t h1, int32_t h2, int32_t out);

/* O [B, out] = network(X [B, in]). */
int spi_mlp_forward(int32_t in, int32_t h1, int32_t h2, int32_t out, int32_t n_class,
                    const float *params, const float *X, int32_t B, float *ws, float *O,
                    spi_stream_t stream);

/* Batch loss and gradient: loss[b] (summing to the batch mean of softmax
 * cross-entropy on the class cls[b] plus wp/2 * sum_k mask (o_k - yp_k)^2
 * over the out - n_class regression outputs) and grad [n_params]. */
int spi_mlp_grad(int32_t in, int32_t h1, int32_t h2, int32_t out, int32_t n_class,
                 const float *params, const float *X, const int32_t *cls, const float *yp,
                 const float *mask, float wp, int32_t B, float *ws, float *grad, float *loss,
                 spi_stream_t stream);

/* One Adam step (bias-corrected, step number t >= 1) over n_par parameters. */
int spi_mlp_adam(float *params, const float *grad, float *m, float *v, int64_t n_par,
                 float lr, float beta1, float beta2, float eps, int32_t t,
                 spi_stream_t stream);

/* ---- allocation-free variant ------------------------------------------ */

/* Limits of spi_krige_ok_noalloc and the size of its static scratch. */
#define SPI_NOALLOC_MAX_STNS 512
#define SPI_NOALLOC_MAX_STEPS 64
#define SPI_NOALLOC_SCRATCH_BYTES 5678080  /* 5.4 MiB on every GPU that loads the library */

/* No counterpart in the reference. Ordinary kriging (estimate, and the OK
 * variance when want_var) of ONE station set, n <= SPI_NOALLOC_MAX_STNS
 * stations and n_steps <= SPI_NOALLOC_MAX_STEPS steps, in FP64 -- the same
 * computation as spi_krige_factor + spi_krige_duals + spi_krige_cells for a
 * one-system batch -- for callers that cannot allocate device memory (hosts
 * whose pool allocator owns the whole GPU and forbids cudaMalloc, services
 * that cannot afford an allocation per call). It allocates nothing: its
 * workspace is a static device array of SPI_NOALLOC_SCRATCH_BYTES, reserved
 * on every GPU that loads the library until the process exits.
 * stn_idx [n] (device): the stations' indices into dom; vals [n_steps, n]
 * (device): their values per step; vg (host): the variogram; est / var of
 * out: [n_steps, dom->n_cells], row j = step j. dom->n_drift is ignored.
 * It needs 2 <= n: a step with one present station is the reference's
 * copy of that station's value (interp/steps.py:282-283), which the caller
 * does itself (spi_fill_rows), and n < 2 returns SPI_ERR_ARG.
 * Sizes above the limits return SPI_ERR_TOO_LARGE. The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress, with
 * that device current); make that first call before any stream capture.
 * Every call shares the one array: calls that overlap on the GPU (other
 * streams or host threads) race and must be serialised by the caller.
 * route_out (optional, device, one int32): the system's route, written in
 * stream order -- 0 Cholesky, 1 exact inverse (numpy.linalg.pinv's
 * truncated inverse where spi_krige_factor's pinv check takes it: systems
 * of up to SPI_PINV_MAX_M rows), 2 singular without that check: every
 * cell then took its nearest station and the estimate variance is 0, and
 * the step is one the reference reports as a problem step
 * (interp/steps.py:363-384). Without route_out such steps are not
 * reported. */
int spi_krige_ok_noalloc(const spi_domain_t *dom, const int32_t *stn_idx, int32_t n,
                         const spi_vg_t *vg, const double *vals, int32_t n_steps,
                         int32_t want_var, const spi_out_t *out, spi_stream_t stream,
                         int32_t *route_out);

/* Interpolation from each cell's own neighbours (the neighbour methods of
 * interp/steps.py:584-606, 673-833): for every listed step q (data row
 * steps[q], output row out_row[q]) and cell c, the reference's _get_interp
 * (interp/steps.py:245-401) over the stations nebs[c * k .. c * k + k)
 * (indices into dom's stations, -1 = empty slot, the valid ones first and
 * all present at the step): the value of a single neighbour; NNB; IDW
 * (idw_exp) over the neighbours; OK / SK / EDK (kind SPI_KIND_*, IDW = 3,
 * NNB = 4) from the neighbours' saddle matrix solved by Gauss-Jordan, with
 * the mean where no value reaches min_var_thr or nug[q] (nugget-only
 * variogram vg[q]), the sum check's nearest-neighbour fallback, and
 * prblm[q] = 1 where a system is exactly singular (nearest neighbour). The
 * OK variance (want_var, out->var) is lambda'r + lambda_n. data [.., ld]:
 * station values by row. FP64. k <= 64. Device arrays. Kriging here solves
 * one system per (cell, step); spi_local_groups solves one per neighbour
 * group and step, as the reference does, and follows its pinv on singular
 * groups. */
int spi_local_cells(const spi_domain_t *dom, int32_t kind, int32_t k, const int32_t *nebs,
                    int32_t n_steps, const int32_t *steps, const int32_t *out_row,
                    const double *data, int64_t ld, const spi_vg_t *vg, const int32_t *nug,
                    double min_var_thr, double idw_exp, int32_t want_var,
                    const spi_out_t *out, int32_t *prblm, spi_stream_t stream);

/* Neighbour slots of spi_local_cells and spi_local_groups. */
#define SPI_LOCAL_MAX_NEBS 64
/* CTAs of spi_local_groups' pinv check, and its scratch for systems of up
 * to mm rows (bytes, a multiple of 16). */
#define SPI_LOCAL_GRP_PINV_SLOTS 152
#define SPI_LOCAL_GRP_PINV_BYTES(mm) \
  ((((int64_t)SPI_LOCAL_GRP_PINV_SLOTS * 2 * (mm) * (mm) * 8) + 15) / 16 * 16)
/* Scratch of spi_local_groups per (group, step): the inverse, its status. */
#define SPI_LOCAL_GRP_BYTES(mm) ((int64_t)(mm) * (mm) * 8 + 4)

/* Kriging from each cell's own neighbours with one system per neighbour
 * group, as the reference's neighbour methods solve it (interp/steps.py:
 * 673-833: _get_interp once per group of cells with identical neighbour
 * lists, its pinv once per step, interp/steps.py:351-352, and lambda =
 * inv @ rhs per cell, interp/steps.py:403-435). Group g's stations are
 * grp_nebs[g * k .. g * k + k) (indices into dom's stations, -1 = empty
 * slot, the valid ones first, all present at the steps); cell c belongs to
 * group cell_grp[c]. cell_order (optional): a permutation of the cells
 * listing each group's cells together, so that neighbouring threads read
 * the same inverse. For every listed step q (data row steps[q], output row
 * out_row[q]) and kind OK / SK / EDK: the group's saddle matrix is
 * inverted once (FP64 Gauss-Jordan with partial pivoting; where
 * ||M||_F ||inv||_F > 1e15 or a pivot is zero, numpy.linalg.pinv's
 * truncated inverse by the rule of spi_krige_factor's pinv check, and the
 * nearest neighbour with prblm[q] = 1 where that check finds no valid
 * inverse); then per cell the estimate, the sum check's nearest-neighbour
 * fallback and the OK variance sum(lambda * rhs) + lambda_n (want_var,
 * out->var); the mean (variance 0) where no value reaches min_var_thr or
 * nug[q]; a single neighbour's value (variance NaN). scratch: 16-byte
 * aligned, at least spi_local_groups_scratch_bytes(kind, k, dom->n_drift,
 * n_grps, 1) bytes; steps are processed in chunks that fit it (all at once
 * with spi_local_groups_scratch_bytes(..., n_steps)). k <=
 * SPI_LOCAL_MAX_NEBS. Device arrays. */
int spi_local_groups(const spi_domain_t *dom, int32_t kind, int32_t k,
                     const int32_t *grp_nebs, int32_t n_grps, const int32_t *cell_grp,
                     const int32_t *cell_order, int32_t n_steps, const int32_t *steps,
                     const int32_t *out_row, const double *data, int64_t ld,
                     const spi_vg_t *vg, const int32_t *nug, double min_var_thr,
                     int32_t want_var, const spi_out_t *out, void *scratch,
                     int64_t scratch_bytes, int32_t *prblm, spi_stream_t stream);

/* Scratch bytes of spi_local_groups for n_steps steps at once (-1 for
 * invalid arguments). Host only. */
int64_t spi_local_groups_scratch_bytes(int32_t kind, int32_t k, int32_t n_drift,
                                       int32_t n_grps, int32_t n_steps);

/* ---- the driver flow around the step engine ------------------------------ */

/* The polygon cell mask of SpInterpPrepare._select_nearby_cells
 * (interp/prepare.py:250-288, misc.py:407-500, 617-627): inside[i] = 1 when
 * point i, its coordinates rounded to 1e-6 as "POINT (%f %f)" prints them,
 * lies strictly inside one of the polygons (ogr Contains: the boundary is
 * outside). Polygon p is the single ring of vertices ring_off[p] ..
 * ring_off[p + 1] - 1 of vx, vy, closed from its last vertex to its first;
 * bbox [n_polys, 4] = (x_min, x_max, y_min, y_max) of each ring. Device
 * arrays. */
int spi_points_in_polygons(const double *px, const double *py, int64_t n_pts,
                           int32_t n_polys, const int64_t *ring_off, const double *vx,
                           const double *vy, const double *bbox, uint8_t *inside,
                           spi_stream_t stream);

/* Per-row statistics of fld [rows, n] (row stride ld, float or double by
 * is_f64) over its finite entries: out [rows, 5] = (min, mean, max, std with
 * ddof, count), as SpInterpMain._save_stats_sers computes them
 * (interp/main.py:474-525: pandas' skip-NaN min/mean/max/std/count of the
 * station data, ddof 1; numpy's nanmin/nanmean/nanmax/nanstd and
 * isfinite().sum() of every interpolated field, ddof 0). A row without a
 * finite entry gets NaN statistics and count 0; std is NaN where count <=
 * ddof. scratch: at least 5 * (608 + rows) doubles. rows <= 65535. */
int spi_field_stats(const void *fld, int32_t is_f64, int32_t rows, int64_t n, int64_t ld,
                    int32_t ddof, double *scratch, int64_t scratch_len, double *out,
                    spi_stream_t stream);

/* numpy.round(fld, decimals) in place, in the field's own precision
 * (float, or double when is_f64): the rounding to nc_nmrl_prcn decimals the
 * reference applies before writing the fields (interp/steps.py:899-901,
 * 920-922). |decimals| <= 22 is exact in the scale factor. */
int spi_round_fields(void *fld, int32_t is_f64, int64_t n, int32_t decimals,
                     spi_stream_t stream);

/* ---- the single-neighbourhood classes ----------------------------------
 *
 * Replace the arithmetic of OrdinaryKriging, SimpleKriging,
 * ExternalDriftKriging, ExternalDriftKriging_MD, OrdinaryIndicatorKriging
 * and SimpleIndicatorKriging (cyth/interpmthds.pyx:251-765): one station
 * set, one variogram (vg: HOST pointer), kind SPI_KIND_OK / SK / EDK
 * (EDK: n_drift >= 1; ExternalDriftKriging is n_drift = 1). Device arrays.
 * Their semantics, unlike the step engine's: the station semivariogram
 * matrix is 0 on its diagonal and a point's right-hand side is 0 at distance
 * 0 (a nugget is a discontinuity), no min_vg_val cut, no sum check; the SK
 * matrix is -gamma with a zero diagonal (SimpleKriging fills its covariance
 * matrix with the total sill before summing it, i.e. with 0.0). */

/* in_dists [n, n], lhs and lhs_inv [m, m] (m = n for SK, else n + 1 +
 * n_drift): cyth/interpmthds.pyx:293-335 (OK), 405-445 (SK), 516-559
 * (EDK), 644-689 (EDK_MD). lhs_inv is the Gauss-Jordan inverse standing in
 * for numpy.linalg.pinv; *status (device int) = 0, or k + 1 when the matrix
 * is singular at elimination step k; *cond (device double, optional) =
 * ||lhs||_F ||lhs_inv||_F (+inf when singular), an upper bound of cond_2:
 * while cond * m * DBL_EPSILON <= 1, pinv's cut-off drops no singular value
 * and pinv equals this inverse; above it the caller takes an SVD
 * pseudo-inverse. si [n_drift, n]. Limit: m <= 10240. */
int spi_legacy_system(int32_t kind, const double *xi, const double *yi, int32_t n,
                      const double *si, int32_t n_drift, const spi_vg_t *vg,
                      double *in_dists, double *lhs, double *lhs_inv, int32_t *status,
                      double *cond, spi_stream_t stream);

/* Every output point k of xk, yk [n_out] (sk_drift [n_drift, n_out]):
 * rhss [n_out, m], lambdas [n_out, n], mus [m - n, n_out] (NULL for SK),
 * zk [n_out] = lambda'zi; est [n_out] (NULL to skip) = the OK est_vars
 * max(0, lambda'gamma + mu) or the SK est_covars max(0, total sill -
 * lambda'c). With ixi (the indicator values of ikrige, else NULL):
 * ik [n_out] = max(0, lambda'ixi) and est = max(0, ik (1 - ik)).
 * cyth/interpmthds.pyx:337-362 (OK), 447-471 (SK), 561-585 (EDK), 691-719
 * (EDK_MD), 722-765 (indicator). */
int spi_legacy_points(int32_t kind, const double *xi, const double *yi, const double *zi,
                      const double *ixi, int32_t n, const double *xk, const double *yk,
                      const double *sk_drift, int64_t n_out, int32_t n_drift,
                      const spi_vg_t *vg, const double *lhs_inv, double *rhss,
                      double *lambdas, double *mus, double *zk, double *est, double *ik,
                      spi_stream_t stream);

/* The pseudo-inverse P of a symmetric m x m matrix M (device arrays,
 * row-major, m <= SPI_PINV_MAX_M), for the single-neighbourhood classes'
 * numpy.linalg.pinv (cyth/interpmthds.pyx:335, 445, 559) where their
 * Gauss-Jordan inverse may differ from it: a cyclic Jacobi
 * eigen-decomposition of (M + M') / 2 in FP64 on one CTA (the singular
 * values of a symmetric matrix are its |eigenvalues|), eigenvalues with
 * |lambda| <= rtol max |lambda| dropped. scratch: 2 m^2 doubles. *status
 * (device): the number of eigenvalues dropped, or -1 when the sweeps did
 * not converge (P is then not to be used). */
int spi_sym_pinv(const double *M, int32_t m, double rtol, double *P, double *scratch,
                 int32_t *status, spi_stream_t stream);

/* ---- measurement ------------------------------------------------------ */

/* No counterpart in the reference: a CUDA-core FMA throughput kernel (FP64
 * when f64, else FP32) for the roofline of the FP64 / FP32 kernels: *threads
 * threads each run 8 independent FMA chains for iters rounds (iters a
 * multiple of 8; 2 * 8 * iters
 * * threads FLOP); the caller times the launch. sink: [*threads] elements of
 * the type, device (152 * 16 * 256 of them). */
int spi_peak_fma(int32_t f64, int64_t iters, void *sink, int64_t *threads,
                 spi_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* SPINTERPS_GB300_H */
