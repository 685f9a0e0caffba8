// Tabulated partition functions Q(T) of a line list's isotopologues, evaluated
// on the host once per spectrum (a handful of scalars: cheaper than a launch).
//
// Two interpolations, as the reference's tabulators (paths relative to the
// radis project root):
//   RG_Q_LINEAR  np.interp, clamped to the end values outside the table
//                (radis/levels/partfunc.py:1191-1192, PartFuncExoMol._at);
//   RG_Q_CUBIC   the interpolating cubic spline of scipy splrep(k=3, s=0) /
//                splev (radis/levels/partfunc_cdsd.py:89-92,105-117): with
//                s = 0 FITPACK places no knot at the second and the
//                second-to-last points, which is the not-a-knot cubic
//                interpolant; the end cubics extend outside the table, and
//                temperatures beyond [0.95 Tmin, 1.05 Tmax] are refused
//                (partfunc_cdsd.py:101-103).
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "rg_internal.h"

namespace rg {

static int err_out(std::string* err, int code, const std::string& msg) {
    if (err) *err = msg;
    return code;
}

// Second derivatives of the not-a-knot cubic spline through (x, y), n >= 4:
// the interior equations h[i-1] M[i-1] + 2 (h[i-1] + h[i]) M[i] + h[i] M[i+1]
// = 6 (d[i] - d[i-1]) (d = divided differences) with M[0] and M[n-1]
// eliminated through the not-a-knot conditions (third derivative continuous
// at x[1] and x[n-2]), solved by the Thomas algorithm for M[1..n-2].
static void not_a_knot(const std::vector<double>& x, const std::vector<double>& y, std::vector<double>& M) {
    const size_t n = x.size();
    std::vector<double> h(n - 1), d(n - 1);
    for (size_t i = 0; i + 1 < n; ++i) {
        h[i] = x[i + 1] - x[i];
        d[i] = (y[i + 1] - y[i]) / h[i];
    }
    const size_t m = n - 2;   // unknowns M[1..n-2]
    std::vector<double> lo(m, 0.0), di(m, 0.0), up(m, 0.0), r(m, 0.0);
    for (size_t k = 0; k < m; ++k) {
        const size_t i = k + 1;
        lo[k] = h[i - 1];
        di[k] = 2.0 * (h[i - 1] + h[i]);
        up[k] = h[i];
        r[k] = 6.0 * (d[i] - d[i - 1]);
    }
    // M[0] = ((h0 + h1) M[1] - h0 M[2]) / h1
    di[0] += h[0] * (h[0] + h[1]) / h[1];
    up[0] -= h[0] * h[0] / h[1];
    // M[n-1] = ((h[n-3] + h[n-2]) M[n-2] - h[n-2] M[n-3]) / h[n-3]
    const double ha = h[n - 3], hb = h[n - 2];
    di[m - 1] += hb * (ha + hb) / ha;
    lo[m - 1] -= hb * hb / ha;
    for (size_t k = 1; k < m; ++k) {
        const double w = lo[k] / di[k - 1];
        di[k] -= w * up[k - 1];
        r[k] -= w * r[k - 1];
    }
    M.assign(n, 0.0);
    M[m] = r[m - 1] / di[m - 1];
    for (size_t k = m - 1; k-- > 0;) M[k + 1] = (r[k] - up[k] * M[k + 2]) / di[k];
    M[0] = ((h[0] + h[1]) * M[1] - h[0] * M[2]) / h[1];
    M[n - 1] = ((ha + hb) * M[n - 2] - hb * M[n - 3]) / ha;
}

int qtable_build(int64_t n, const double* T, const double* Q, int interp, QTable* out, std::string* err) {
    if (n < 2 || !T || !Q) return err_out(err, RG_ERR_ARG, "partition table needs at least 2 points");
    if (interp != RG_Q_LINEAR && interp != RG_Q_CUBIC)
        return err_out(err, RG_ERR_ARG, "unknown interpolation " + std::to_string(interp));
    if (interp == RG_Q_CUBIC && n < 4)
        return err_out(err, RG_ERR_ARG, "a cubic partition table needs at least 4 points");
    for (int64_t i = 0; i < n; ++i) {
        if (!std::isfinite(T[i]) || !std::isfinite(Q[i]) || !(Q[i] > 0))
            return err_out(err, RG_ERR_ARG,
                           "partition table point " + std::to_string(i) + " is not finite and positive");
        if (i && !(T[i] > T[i - 1])) return err_out(err, RG_ERR_ARG, "partition table temperatures must increase");
    }
    QTable t;
    t.interp = interp;
    t.T.assign(T, T + n);
    t.Q.assign(Q, Q + n);
    if (interp == RG_Q_CUBIC) not_a_knot(t.T, t.Q, t.M);
    *out = std::move(t);
    return RG_OK;
}

int qtable_eval(const QTable& t, double T, double* q, double* dq_dT, std::string* err) {
    const size_t n = t.T.size();
    if (n < 2) return err_out(err, RG_ERR_STATE, "empty partition table");
    if (!std::isfinite(T)) return err_out(err, RG_ERR_ARG, "temperature is not finite");
    if (t.interp == RG_Q_LINEAR) {   // np.interp
        if (T <= t.T[0] || T >= t.T[n - 1]) {
            *q = T <= t.T[0] ? t.Q[0] : t.Q[n - 1];
            if (dq_dT) *dq_dT = 0.0;
            return RG_OK;
        }
        size_t i = 0;
        while (i + 2 < n && T >= t.T[i + 1]) ++i;
        const double s = (t.Q[i + 1] - t.Q[i]) / (t.T[i + 1] - t.T[i]);
        *q = t.Q[i] + s * (T - t.T[i]);
        if (dq_dT) *dq_dT = s;
        return RG_OK;
    }
    if (T < 0.95 * t.T[0] || T > 1.05 * t.T[n - 1]) {
        char buf[160];
        snprintf(buf, sizeof buf, "temperature %g K outside the partition table (%g-%g K, 5%% extrapolation)", T,
                 t.T[0], t.T[n - 1]);
        return err_out(err, RG_ERR_RANGE, buf);
    }
    size_t i = 0;   // interval [T[i], T[i+1]], end intervals extended outside
    while (i + 2 < n && T >= t.T[i + 1]) ++i;
    const double h = t.T[i + 1] - t.T[i], a = t.T[i + 1] - T, b = T - t.T[i];
    const double c0 = t.Q[i] / h - t.M[i] * h / 6.0, c1 = t.Q[i + 1] / h - t.M[i + 1] * h / 6.0;
    *q = t.M[i] * a * a * a / (6.0 * h) + t.M[i + 1] * b * b * b / (6.0 * h) + c0 * a + c1 * b;
    if (dq_dT) *dq_dT = -t.M[i] * a * a / (2.0 * h) + t.M[i + 1] * b * b / (2.0 * h) - c0 + c1;
    return RG_OK;
}

}  // namespace rg
