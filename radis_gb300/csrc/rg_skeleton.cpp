// Interpolative decomposition of the LDM nodes' lineshape transforms (host,
// FP64).
//
// The FFT stage of the LDM method (radis/lbl/broadening.py:2521-2530) forms
// sum_n FFT(row_n) V_n(f) over every node n of the (wG, wL) grid.  The V_n
// (folded, normalised Voigt transforms on f in [0, 1/(2 dv)]) are smooth
// members of a two-parameter family, and a few of them span all the others
// to FP64-level accuracy: V_n = sum_r C[r][n] V_{s_r} + e_n with |e_n| <= tol.
// Then sum_n FFT(row_n) V_n = sum_r FFT(sum_n C[r][n] row_n) V_{s_r} + error,
// so only R projected rows are transformed.  The skeleton s_r and the
// coefficients come from a column-pivoted modified Gram-Schmidt QR of the
// sampled transforms (Businger-Golub pivoting): the residual of every column
// after r steps is exactly the error of its least-squares fit by the r chosen
// columns, and the decomposition stops when the largest residual sample is
// within tol.  The coefficients of column j are R11^-1 R[:, j], which keeps
// them bounded (|C| <= ~2 on the grids the method meets).
#include <algorithm>
#include <cmath>
#include <vector>

#include "rg_internal.h"

namespace rg {

namespace {

// dot product in four partial sums (vectorisable without reassociation flags)
inline double dot(const double* __restrict a, const double* __restrict b, int S) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int i = 0;
    for (; i + 4 <= S; i += 4) {
        s0 += a[i] * b[i];
        s1 += a[i + 1] * b[i + 1];
        s2 += a[i + 2] * b[i + 2];
        s3 += a[i + 3] * b[i + 3];
    }
    for (; i < S; ++i) s0 += a[i] * b[i];
    return (s0 + s1) + (s2 + s3);
}

inline double max_abs(const double* a, int S) {
    double m = 0.0;
    for (int i = 0; i < S; ++i) m = std::fmax(m, std::fabs(a[i]));
    return m;
}

}  // namespace

int interp_decomp(const double* A, int S, int n, double tol, int r_max, int* sk, double* C, int* R_out,
                  double* err_out) {
    if (S <= 0 || n <= 0 || r_max <= 0) return RG_ERR_ARG;
    std::vector<double> W(A, A + (size_t)S * n);   // residual columns (column-major, S per column)
    std::vector<double> Q((size_t)S * r_max);      // orthonormal directions
    std::vector<double> Rm((size_t)r_max * n, 0.0);   // Rm[r * n + j]: coefficient of q_r in column j
    std::vector<double> nrm2(n), nrm2_ref(n);      // residual norms^2, downdated; their last exact value
    std::vector<int> perm(n);
    auto col = [&](int j) { return &W[(size_t)j * S]; };
    for (int j = 0; j < n; ++j) {
        perm[j] = j;
        nrm2[j] = nrm2_ref[j] = dot(col(j), col(j), S);
    }
    auto swap_cols = [&](int a, int b) {
        if (a == b) return;
        std::swap_ranges(col(a), col(a) + S, col(b));
        for (int r = 0; r < r_max; ++r) std::swap(Rm[(size_t)r * n + a], Rm[(size_t)r * n + b]);
        std::swap(perm[a], perm[b]);
        std::swap(nrm2[a], nrm2[b]);
        std::swap(nrm2_ref[a], nrm2_ref[b]);
    };
    const double sqS = std::sqrt((double)S);
    int R = 0;
    double err = 0.0;
    for (;; ++R) {
        // pivot: the column of largest residual norm.  Stop when the largest
        // residual sample is within tol: sup <= norm <= sqrt(S) sup, so the
        // samples are scanned only when the norms leave it undecided.
        int piv = R;
        double best = -1.0;
        for (int j = R; j < n; ++j)
            if (nrm2[j] > best) {
                best = nrm2[j];
                piv = j;
            }
        const double bn = std::sqrt(std::fmax(best, 0.0));
        if (R == n) {
            err = 0.0;
            break;
        }
        if (bn <= sqS * tol) {
            err = 0.0;
            for (int j = R; j < n; ++j) err = std::fmax(err, max_abs(col(j), S));
            if (err <= tol) break;
        } else {
            err = bn / sqS;   // a lower bound: some sample is at least this large
        }
        if (R == r_max) {   // not within tol at the largest rank allowed
            *R_out = R;
            *err_out = err;
            return RG_ERR_RANGE;
        }
        swap_cols(R, piv);
        double* q = &Q[(size_t)R * S];
        std::copy(col(R), col(R) + S, q);
        // one re-orthogonalisation pass against the earlier directions
        for (int r = 0; r < R; ++r) {
            const double* qr = &Q[(size_t)r * S];
            const double d = dot(qr, q, S);
            for (int i = 0; i < S; ++i) q[i] -= d * qr[i];
            Rm[(size_t)r * n + R] += d;
        }
        const double nq = std::sqrt(dot(q, q, S));
        if (!(nq > 0.0)) break;   // exactly dependent: the rest is within tol already
        for (int i = 0; i < S; ++i) q[i] /= nq;
        Rm[(size_t)R * n + R] = nq;
        // the remaining columns: all projections first (independent dot
        // products), then the updates
        double* rrow = &Rm[(size_t)R * n];
        for (int j = R + 1; j < n; ++j) rrow[j] = dot(q, col(j), S);
        for (int j = R + 1; j < n; ++j) {
            double* __restrict w = col(j);
            const double d = rrow[j];
            for (int i = 0; i < S; ++i) w[i] -= d * q[i];
            // downdated norm, recomputed once it has lost most of its digits
            nrm2[j] -= d * d;
            if (nrm2[j] < 1e-6 * nrm2_ref[j]) nrm2[j] = nrm2_ref[j] = dot(w, w, S);
        }
    }
    // coefficients: skeleton column r -> unit vector; the others solve
    // R11 T = R12, row by row from the last (each row a contiguous sweep over
    // the columns)
    std::fill(C, C + (size_t)R * n, 0.0);
    const int m = n - R;
    std::vector<double> T((size_t)R * m);
    for (int r = R - 1; r >= 0; --r) {
        double* __restrict tr = &T[(size_t)r * m];
        const double* rr = &Rm[(size_t)r * n];
        for (int j = 0; j < m; ++j) tr[j] = rr[R + j];
        for (int k = r + 1; k < R; ++k) {
            const double f = rr[k];
            const double* __restrict tk = &T[(size_t)k * m];
            for (int j = 0; j < m; ++j) tr[j] -= f * tk[j];
        }
        const double inv = 1.0 / rr[r];
        for (int j = 0; j < m; ++j) tr[j] *= inv;
    }
    for (int r = 0; r < R; ++r) {
        C[(size_t)r * n + perm[r]] = 1.0;
        for (int j = 0; j < m; ++j) C[(size_t)r * n + perm[R + j]] = T[(size_t)r * m + j];
    }
    for (int r = 0; r < R; ++r) sk[r] = perm[r];
    *R_out = R;
    *err_out = err;
    return RG_OK;
}

}  // namespace rg
