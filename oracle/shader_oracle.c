/* Restatement in C of the arithmetic of the reference's GPU (Vulkan) path --
 * TEST INFRASTRUCTURE ONLY (loaded by oracle/shader_oracle.py for tests/).
 *
 * The reference runs two compute shaders around VkFFT:
 *   radis/gpu/vulkan/shaders/cmdFillLDM.comp:75-145 -- per line: shifted
 *     position v0 + p da, fractional grid index, log Doppler and log Lorentz
 *     widths against the node axes, the equilibrium intensity from the
 *     Einstein-A based S0, and 2x2x2 linear weights added into the LDM;
 *   radis/gpu/vulkan/shaders/cmdApplyLineshapes.comp:51-90 -- per rfft bin,
 *     the sum over nodes of LDM_FT x exp(-(pi x wG)^2 / (4 ln 2) - pi x wL) / dv
 *     (no folding, no normalisation).
 * The shaders run in FP32; this file is compiled twice, with REAL = float
 * (names ending _f32) and REAL = double (_f64), so a test can separate the
 * FP32 rounding of that design from its conventions.  Sums are sequential
 * here where the shaders add with atomics (order only changes rounding).
 *
 * LDM layout: [m][l][k], rows of n_row reals; spectrum FT: n_bins complex
 * values as (re, im) pairs.
 */
#include <math.h>
#include <stdint.h>

#ifndef REAL
#define REAL float
#define SUFFIX _f32
#endif
#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define NAME(x) CAT(x, SUFFIX)

#if defined(REAL_IS_DOUBLE)
#define R_EXP exp
#define R_LOG log
#else
#define R_EXP expf
#define R_LOG logf
#endif

/* Scalars the host sets per spectrum (radis/gpu/params.py:123-155 set_pTQ,
 * set_G_params, set_L_params; init_G_params / init_L_params). */
typedef struct {
    double v_min, dv;
    int64_t n_v, n_row;          /* window points; LDM row length (FFT length) */
    double dxG, dxL, log_wG_min, log_wL_min;
    int32_t n_G, n_L;
    double p;                    /* pressure in the shift and width formulas */
    double log_2p, hlog_T, log_rT, c2T, N;
    double x_self, x_air;        /* collision-partner fractions */
    double log_c2Mm[16], Q[16];
} shader_params;

/* cmdFillLDM: every line adds its intensity into 8 LDM cells. */
void NAME(fill_ldm)(const shader_params* P, int64_t n_lines, const uint32_t* iso, const double* v0_in,
                    const double* da_in, const double* S0_in, const double* El_in, const double* na_in,
                    const double* g_self_in, const double* g_air_in, REAL* ldm) {
    const REAL v_min = (REAL)P->v_min, dv = (REAL)P->dv, p = (REAL)P->p;
    const REAL dxG = (REAL)P->dxG, dxL = (REAL)P->dxL;
    const REAL lGmin = (REAL)P->log_wG_min, lLmin = (REAL)P->log_wL_min;
    const REAL log_2p = (REAL)P->log_2p, hlog_T = (REAL)P->hlog_T, log_rT = (REAL)P->log_rT;
    const REAL c2T = (REAL)P->c2T, N = (REAL)P->N, xs = (REAL)P->x_self, xa = (REAL)P->x_air;
    const int64_t row = P->n_row, plane = row * P->n_G;
    for (int64_t i = 0; i < n_lines; ++i) {
        const uint32_t j = iso ? iso[i] : 0;
        const REAL v0 = (REAL)v0_in[i], da = (REAL)da_in[i], S0 = (REAL)S0_in[i];
        const REAL El = (REAL)El_in[i], na = (REAL)na_in[i];
        /* grid index of the shifted centre */
        const REAL kf = (v0 + p * da - v_min) / dv;
        const int64_t k0 = (int64_t)kf;   /* truncation, as int() in the shader */
        if (k0 < 0 || k0 + 1 >= P->n_v) continue;   /* as the shader: int() truncates toward 0 */
        const REAL tv = kf - (REAL)k0;
        /* Gaussian node coordinate */
        const REAL gf = (R_LOG(v0) + (REAL)P->log_c2Mm[j] + hlog_T - lGmin) / dxG;
        const int64_t l0 = (int64_t)gf;
        const REAL tG = gf - (REAL)l0;
        /* Lorentzian node coordinate: partner-weighted HWHM coefficient */
        const REAL gam = xs * (REAL)g_self_in[i] + xa * (REAL)g_air_in[i];
        const REAL lf = (R_LOG(gam) + log_2p + na * log_rT - lLmin) / dxL;
        const int64_t m0 = (int64_t)lf;
        const REAL tL = lf - (REAL)m0;
        /* off the node axes: the shader has no check (its host sizes the axes to hold
         * every line); skipped here instead of written out of bounds */
        if (l0 < 0 || l0 + 1 >= P->n_G || m0 < 0 || m0 + 1 >= P->n_L) continue;
        /* equilibrium intensity from the Einstein-A based S0 */
        const REAL I = N * xs * S0 * (R_EXP(-c2T * El) - R_EXP(-c2T * (El + v0))) / (REAL)P->Q[j];
        REAL* c = ldm + m0 * plane + l0 * row + k0;
        const REAL w[2] = {1 - tv, tv}, g[2] = {1 - tG, tG}, h[2] = {1 - tL, tL};
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int d = 0; d < 2; ++d) c[d * plane + b * row + a] += w[a] * g[b] * h[d] * I;
    }
}

/* cmdApplyLineshapes: spectrum FT bin k = sum over nodes of LDM_FT x the
 * unnormalised Voigt FT / dv, x = k / (n_fft dv). */
void NAME(apply_lineshapes)(const shader_params* P, int64_t n_fft, int64_t n_bins, const REAL* ldm_ft,
                            REAL* out) {
    const REAL pi = (REAL)3.14159265358979323846, r4ln2 = (REAL)(1.0 / (4.0 * 0.69314718055994530942));
    const REAL dv = (REAL)P->dv;
    for (int64_t k = 0; k < n_bins; ++k) {
        const REAL x = (REAL)k / ((REAL)n_fft * dv);
        REAL re = 0, im = 0;
        for (int l = 0; l < P->n_G; ++l) {
            const REAL wG = R_EXP((REAL)P->log_wG_min + (REAL)l * (REAL)P->dxG);
            for (int m = 0; m < P->n_L; ++m) {
                const REAL wL = R_EXP((REAL)P->log_wL_min + (REAL)m * (REAL)P->dxL);
                const REAL gx = pi * x * wG;
                const REAL mul = R_EXP(-r4ln2 * gx * gx - pi * x * wL) / dv;
                const REAL* z = ldm_ft + 2 * (((int64_t)m * P->n_G + l) * n_bins + k);
                re += z[0] * mul;
                im += z[1] * mul;
            }
        }
        out[2 * k] = re;
        out[2 * k + 1] = im;
    }
}
