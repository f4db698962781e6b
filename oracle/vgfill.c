/*
 * CPU restatement of the reference's native kernels (cyth/interpmthds.pyx).
 *
 * TEST INFRASTRUCTURE ONLY: the oracle that the CUDA path is checked
 * against, and the CPU baseline that bench.py times beside it. The product
 * (spinterps_gb300/) never links, loads or calls this file.
 *
 * Each function follows the loop order and the floating-point expression of
 * the Cython source so that the results are bit-identical to the reference's
 * compiled kernels on the same libm. Build with -ffp-contract=off so that
 * no multiply-add is fused (the reference's x86-64 build has no FMA).
 *
 * Variogram model codes (shared with include/spinterps_gb300.h):
 *   0 Rng, 1 Nug, 2 Sph, 3 Exp, 4 Lin, 5 Gau, 6 Pow, 7 Hol
 */
#include <math.h>
#include <stdint.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* cyth/interpmthds.pyx:38-84 */
static double vg_eval(int code, double h, double r, double s)
{
    double a, b;
    switch (code) {
    case 0: return h;                                   /* rng_vg 38-39 */
    case 1: return s;                                   /* nug_vg 42-43 */
    case 2:                                             /* sph_vg 46-55 */
        if (h >= r) return s;
        a = (1.5 * h) / r;
        b = (h * h * h) / (2 * (r * r * r));
        return s * (a - b);
    case 3: return s * (1 - exp(-3 * h / r));           /* exp_vg 58-59 */
    case 4:                                             /* lin_vg 62-66 */
        if (h > r) return s;
        return s * (h / r);
    case 5: return s * (1 - exp(-3 * ((h * h) / (r * r))));  /* gau_vg 69-70 */
    case 6: return s * pow(h, r);                       /* pow_vg 73-74 */
    case 7:                                             /* hol_vg 77-83 */
        if (h == 0) return 0;
        a = (M_PI * h) / r;
        return s * (1 - (sin(a) / a));
    default: return NAN;
    }
}

double orc_vg_eval(int code, double h, double r, double s)
{
    return vg_eval(code, h, r, s);
}

/* fill_dists_2d_mat, cyth/interpmthds.pyx:123-143 */
void orc_fill_dists_2d_mat(const double *x1s, const double *y1s, int64_t n1,
                           const double *x2s, const double *y2s, int64_t n2,
                           double *dists)
{
    for (int64_t i = 0; i < n1; ++i) {
        double x = x1s[i], y = y1s[i];
        for (int64_t j = 0; j < n2; ++j) {
            double dx = x - x2s[j], dy = y - y2s[j];
            dists[i * n2 + j] = pow(pow(dx, 2.0) + pow(dy, 2.0), 0.5);
        }
    }
}

/* fill_vg_var_arr, cyth/interpmthds.pyx:146-226.  The model string is
 * parsed by the caller (oracle/port.py follows the same split rules) into
 * n_comp (code, sill, range) triples with range already max(1e-5, r). */
void orc_fill_vg_var_arr(const double *dists, int64_t rows, int64_t cols,
                         double *out, int covar_flag, int diag_flag,
                         int n_comp, const int *codes, const double *sills,
                         const double *ranges, double min_vg_val)
{
    int cov_sign = covar_flag ? -1 : +1;
    int cov_mult = covar_flag ? +1 : 0;
    for (int64_t h = 0; h < rows; ++h)
        for (int64_t g = 0; g < cols; ++g) out[h * cols + g] = 0.0;
    for (int c = 0; c < n_comp; ++c) {
        double r = ranges[c], s = sills[c];
        for (int64_t h = 0; h < rows; ++h)
            for (int64_t g = 0; g < cols; ++g) {
                if (diag_flag && g < h) continue;
                out[h * cols + g] += (cov_mult * s) +
                    (cov_sign * vg_eval(codes[c], dists[h * cols + g], r, s));
            }
    }
    for (int64_t h = 0; h < rows; ++h)
        for (int64_t g = 0; g < cols; ++g) {
            if (diag_flag && g < h) continue;
            if (out[h * cols + g] <= min_vg_val) out[h * cols + g] = 0.0;
        }
    if (diag_flag)
        for (int64_t h = 0; h < rows; ++h)
            for (int64_t g = 0; g < cols; ++g)
                if (g < h) out[h * cols + g] = out[g * cols + h];
}

/* copy_2d_arr_at_idxs, cyth/interpmthds.pyx:229-248 (subset has its own
 * row stride because the reference allocates add_rc extra columns). */
void orc_copy_2d_arr_at_idxs(const double *arr, int64_t arr_cols,
                             const int64_t *row_idxs, int64_t n_rows,
                             const int64_t *col_idxs, int64_t n_cols,
                             double *subset, int64_t subset_cols)
{
    for (int64_t i = 0; i < n_rows; ++i)
        for (int64_t j = 0; j < n_cols; ++j)
            subset[i * subset_cols + j] = arr[row_idxs[i] * arr_cols + col_idxs[j]];
}

/* fill_wts_and_sum, cyth/interpmthds.pyx:784-795 */
double orc_fill_wts_and_sum(const double *dists, int64_t n, double *wts,
                            double idw_exp)
{
    double wts_sum = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        wts[i] = 1.0 / pow(dists[i], idw_exp);
        wts_sum += wts[i];
    }
    return wts_sum;
}

/* get_mults_sum, cyth/interpmthds.pyx:798-808 */
double orc_get_mults_sum(const double *wts, const double *data, int64_t n)
{
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += wts[i] * data[i];
    return s;
}

/* The IDW branch of SpInterpSteps._get_interp (interp/steps.py:293-313) for
 * all cells of one station group: dists [n_dsts, n_refs] is normalised IN
 * PLACE by its row maximum, exactly as the reference does. Returns the index
 * of the first cell whose weight sum fails the >= 1e-14 assertion, or -1. */
int64_t orc_idw_group(double *dists, int64_t n_dsts, int64_t n_refs,
                      const double *ref_data, int64_t n_time,
                      const uint8_t *interp_flags, const double *ref_means,
                      double idw_exp, double *wts, double *dst_data)
{
    for (int64_t i = 0; i < n_dsts; ++i) {
        double *d = dists + i * n_refs;
        double dmax = d[0];
        for (int64_t k = 1; k < n_refs; ++k)
            if (d[k] > dmax || isnan(d[k])) dmax = d[k];
        if (dmax > 0)
            for (int64_t k = 0; k < n_refs; ++k) d[k] /= dmax;
        double wsum = orc_fill_wts_and_sum(d, n_refs, wts, idw_exp);
        if (!(wsum >= 1e-14)) return i;
        for (int64_t j = 0; j < n_time; ++j) {
            if (interp_flags[j])
                dst_data[j * n_dsts + i] =
                    orc_get_mults_sum(wts, ref_data + j * n_refs, n_refs) / wsum;
            else
                dst_data[j * n_dsts + i] = ref_means[j];
        }
    }
    return -1;
}
