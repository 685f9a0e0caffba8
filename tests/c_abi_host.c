/* A plain C caller of the library's host-only entry points: the header
 * compiles as strict C99 and the shared library links and answers without a
 * GPU (compiled and run by tests/test_c_abi.py).  Prints "ok" and exits 0, or
 * names the first failed check and exits 1. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "radis_gb300.h"

static int failed(const char* what) {
    printf("FAILED: %s (%s)\n", what, rg_last_error());
    return 1;
}

int main(void) {
    /* version */
    if (rg_abi_version() != RG_ABI_VERSION) return failed("rg_abi_version");

    /* tabulated partition function: linear (np.interp: Q(250) between (200, 10)
     * and (300, 20), clamped beyond the table) and cubic (refused beyond
     * [0.95 Tmin, 1.05 Tmax]) */
    {
        const double T[4] = {200.0, 300.0, 400.0, 500.0}, Q[4] = {10.0, 20.0, 40.0, 70.0};
        double q = 0.0, dq = 0.0;
        if (rg_partition_eval(4, T, Q, RG_Q_LINEAR, 250.0, &q, &dq) != RG_OK) return failed("rg_partition_eval");
        if (q != 15.0 || dq != 0.1) return failed("linear Q value");
        if (rg_partition_eval(4, T, Q, RG_Q_LINEAR, 900.0, &q, &dq) != RG_OK || q != 70.0) return failed("clamp");
        if (rg_partition_eval(4, T, Q, RG_Q_CUBIC, 350.0, &q, &dq) != RG_OK || !(q > 20.0 && q < 40.0))
            return failed("cubic Q value");
        if (rg_partition_eval(4, T, Q, RG_Q_CUBIC, 900.0, &q, &dq) == RG_OK) return failed("out-of-table T accepted");
        if (strlen(rg_last_error()) == 0) return failed("no error text");
    }

    /* HITRAN-160 records from memory: two records, CRLF then LF */
    {
        const char* rec1 =
            " 51 2000.123456 1.234E-20 1.000E+00.0600.0800  100.00000.70-.002000"
            "                                                                               "
            "   12.0   10.0\r\n";
        const char* rec2 =
            " 52 2100.500000 2.500E-21 3.000E+00.0550.0750  250.50000.68-.001000"
            "                                                                               "
            "   14.0   12.0\n";
        char text[400];
        int64_t n = -1;
        snprintf(text, sizeof text, "%s%s", rec1, rec2);
        if (rg_hitran_count(text, (int64_t)strlen(text), 1, &n) != RG_OK || n != 2) return failed("rg_hitran_count");
        {
            int32_t id[2], iso[2];
            double v0[2], s[2], el[2], na[2], delta[2];
            rg_hitran_columns c;
            memset(&c, 0, sizeof c);
            c.n = n;
            c.id = id;
            c.iso = iso;
            c.v0 = v0;
            c.s_ref = s;
            c.e_low = el;
            c.n_air = na;
            c.delta = delta;
            if (rg_hitran_parse(text, (int64_t)strlen(text), 0, &c) != RG_OK) return failed("rg_hitran_parse");
            if (id[0] != 5 || iso[0] != 1 || iso[1] != 2) return failed("id / iso");
            if (v0[0] != strtod("2000.123456", NULL) || v0[1] != 2100.5) return failed("v0");
            if (s[0] != strtod("1.234E-20", NULL) || el[1] != 250.5 || na[1] != 0.68 || delta[0] != -0.002)
                return failed("float columns");
            c.n = 3;
            if (rg_hitran_parse(text, (int64_t)strlen(text), 0, &c) != RG_ERR_ARG) return failed("count mismatch");
        }
        text[10] = 'x';   /* inside the wav field of record 1 */
        {
            double v0[2];
            rg_hitran_columns c;
            memset(&c, 0, sizeof c);
            c.n = 2;
            c.v0 = v0;
            if (rg_hitran_parse(text, (int64_t)strlen(text), 0, &c) != RG_ERR_ARG) return failed("bad field");
            if (!strstr(rg_last_error(), "line 1, field wav")) return failed("bad field message");
        }
    }

    /* node grid of three lines (host arrays, no device) */
    {
        const double v0[3] = {2000.0, 2000.5, 2001.0}, s[3] = {1e-20, 2e-20, 3e-20};
        const float el[3] = {100.f, 200.f, 300.f}, ga[3] = {0.06f, 0.07f, 0.05f}, gs[3] = {0.08f, 0.09f, 0.07f},
                    na[3] = {0.7f, 0.75f, 0.65f};
        rg_line_arrays L;
        rg_isotopes I;
        rg_plan_desc d;
        rg_conditions c;
        rg_grid g;
        memset(&L, 0, sizeof L);
        memset(&I, 0, sizeof I);
        memset(&d, 0, sizeof d);
        memset(&c, 0, sizeof c);
        L.n = 3;
        L.v0 = v0;
        L.s_ref = s;
        L.e_low = el;
        L.g_air = ga;
        L.g_self = gs;
        L.n_air = na;
        I.n_iso = 1;
        I.molar_mass[0] = 28.0;
        I.t_ref = 296.0;
        d.vmin = 1999.0;
        d.dv = 0.002;
        d.n_v = 1501;
        d.n_G = 4;
        d.n_L = 6;
        d.folding_thresh = 1e-6;
        c.T = 700.0;
        c.p_bar = 1.0;
        c.x = 0.1;
        if (rg_grid_estimate(&L, &I, &d, &c, &g) != RG_OK) return failed("rg_grid_estimate");
        if (g.n_G != 4 || g.n_L != 6 || g.n_ft < 2 * d.n_v || g.n1 * g.n2 != g.n_ft) return failed("grid shape");
        if (!(g.dxG > 0) || !(g.dxL > 0) || !isfinite(g.log_wG_min) || !isfinite(g.log_wL_min))
            return failed("grid axes");
        d.n_v = 1;
        if (rg_grid_estimate(&L, &I, &d, &c, &g) != RG_ERR_ARG) return failed("n_v = 1 accepted");
    }

    /* a context: RG_ERR_CUDA without a GPU (no abort), a handle with one */
    {
        rg_ctx* ctx = NULL;
        const int rc = rg_ctx_create(0, &ctx);
        if (rc == RG_OK) {
            if (rg_ctx_destroy(ctx) != RG_OK) return failed("rg_ctx_destroy");
        } else if (rc != RG_ERR_CUDA) {
            return failed("rg_ctx_create status");
        }
    }
    printf("ok\n");
    return 0;
}
