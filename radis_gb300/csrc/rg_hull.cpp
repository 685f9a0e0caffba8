// Exact convex envelopes of large point sets, O(n) passes (split over host
// threads) plus a sort of the few survivors.
//
// The reference bounds the Lorentzian node axis by the lower/upper envelope of
// the lines' (n_air, log gamma) pairs as a function of log(296/T)
// (radis/gpu/params.py:8-67, evaluated in set_L_params :89-104).  The envelope
// min_i(b_i + a_i t) over all t is carried by the vertices of the lower convex
// hull of the points (a_i, b_i).  The same structure bounds the largest line
// intensity over temperature (points (E_low, log S')), which sets the FP32
// scaling of a spectrum.
//
// Algorithm: bucket the points by a into K buckets, keep the lowest point of
// each bucket, take the lower hull of those (a chain of real data points).
// The true hull lies on or below that chain, so any point strictly above it
// cannot be a hull vertex; the survivors (points on or below the chain, plus
// everything outside the chain's a-range) are sorted and run through Andrew's
// monotone chain.
#include <algorithm>
#include <cmath>
#include <limits>

#include "rg_internal.h"

namespace rg {

namespace {

struct Pt {
    double a, b;
};

inline double cross(const Pt& o, const Pt& p, const Pt& q) {
    return (p.a - o.a) * (q.b - o.b) - (p.b - o.b) * (q.a - o.a);
}

// Andrew's monotone chain, lower hull of points sorted by (a, b).
std::vector<Pt> monotone_lower(std::vector<Pt>& pts) {
    std::sort(pts.begin(), pts.end(), [](const Pt& p, const Pt& q) {
        return p.a < q.a || (p.a == q.a && p.b < q.b);
    });
    std::vector<Pt> h;
    for (const Pt& p : pts) {
        if (!h.empty() && h.back().a == p.a) continue;   // same a: keep lowest b
        while (h.size() >= 2 && cross(h[h.size() - 2], h.back(), p) <= 0) h.pop_back();
        h.push_back(p);
    }
    return h;
}

struct ArraySource : PointSource {
    const double* a;
    const double* b;
    int64_t n;
    double sign;
    int64_t size() const override { return n; }
    void get(int64_t i, double* pa, double* pb) const override {
        *pa = a[i];
        *pb = sign * b[i];
    }
};

struct NegSource : PointSource {
    const PointSource& s;
    explicit NegSource(const PointSource& src) : s(src) {}
    int64_t size() const override { return s.size(); }
    void get(int64_t i, double* pa, double* pb) const override {
        s.get(i, pa, pb);
        *pb = -*pb;
    }
    bool valid_a(int64_t i, double* pa) const override { return s.valid_a(i, pa); }
};

Hull lower_impl(const PointSource& src) {
    const int64_t n = src.size();
    Hull out;
    constexpr double kInf = std::numeric_limits<double>::infinity();
    // Three passes over the points, each split over host threads; the merges
    // (min / max, the per-bucket minimum under the total order (b, a), the
    // survivors concatenated in chunk order) give the sequential result.
    const int T = host_chunk_count(n, kHostMinPerThread);
    std::vector<double> lo(T, kInf), hi(T, -kInf);
    run_host_chunks(T, n, [&](int t, int64_t i0, int64_t i1) {
        double amin = kInf, amax = -kInf;
        for (int64_t i = i0; i < i1; ++i) {
            double a;
            if (!src.valid_a(i, &a)) continue;
            amin = std::min(amin, a);
            amax = std::max(amax, a);
        }
        lo[t] = amin;
        hi[t] = amax;
    });
    const double amin = *std::min_element(lo.begin(), lo.end());
    const double amax = *std::max_element(hi.begin(), hi.end());
    if (!(amin <= amax)) return out;   // no finite point
    const int K = 4096;
    const double span = amax - amin;
    const double scale = span > 0 ? K / span : 0.0;
    auto bucket_of = [&](double a) {
        int k = (int)((a - amin) * scale);
        return k < 0 ? 0 : (k >= K ? K - 1 : k);
    };
    auto lower = [](const Pt& p, const Pt& q) { return p.b < q.b || (p.b == q.b && p.a < q.a); };
    std::vector<std::vector<Pt>> part(T, std::vector<Pt>(K, Pt{0, kInf}));
    run_host_chunks(T, n, [&](int t, int64_t i0, int64_t i1) {
        std::vector<Pt>& bk = part[t];
        for (int64_t i = i0; i < i1; ++i) {
            double a, b;
            src.get(i, &a, &b);
            if (!std::isfinite(a) || !std::isfinite(b)) continue;
            Pt& q = bk[bucket_of(a)];
            if (lower(Pt{a, b}, q)) q = Pt{a, b};
        }
    });
    std::vector<Pt> mins;
    for (int k = 0; k < K; ++k) {
        Pt q{0, kInf};
        for (int t = 0; t < T; ++t)
            if (lower(part[t][k], q)) q = part[t][k];
        if (std::isfinite(q.b)) mins.push_back(q);
    }
    std::vector<Pt> chain = monotone_lower(mins);
    // survivors: on/below the chain or outside its a-range
    const double a_lo = chain.front().a, a_hi = chain.back().a;
    std::vector<std::vector<Pt>> kept(T);
    run_host_chunks(T, n, [&](int t, int64_t i0, int64_t i1) {
        std::vector<Pt>& keep = kept[t];
        for (int64_t i = i0; i < i1; ++i) {
            double a, b;
            src.get(i, &a, &b);
            if (!std::isfinite(a) || !std::isfinite(b)) continue;
            if (a < a_lo || a > a_hi) {
                keep.push_back(Pt{a, b});
                continue;
            }
            // segment of the chain containing a
            size_t up = std::upper_bound(chain.begin(), chain.end(), a,
                                         [](double v, const Pt& p) { return v < p.a; }) -
                        chain.begin();
            double cb;
            if (up == 0) {
                cb = chain[0].b;
            } else if (up >= chain.size()) {
                cb = chain.back().b;
            } else {
                const Pt& p = chain[up - 1];
                const Pt& q = chain[up];
                cb = p.b + (q.b - p.b) * (a - p.a) / (q.a - p.a);
            }
            // keep with a relative margin so that rounding never drops a vertex
            if (b <= cb + 1e-12 * (1.0 + std::fabs(cb))) keep.push_back(Pt{a, b});
        }
    });
    std::vector<Pt> keep;
    for (const auto& v : kept) keep.insert(keep.end(), v.begin(), v.end());
    keep.insert(keep.end(), chain.begin(), chain.end());
    std::vector<Pt> h = monotone_lower(keep);
    for (const Pt& p : h) {
        out.a.push_back(p.a);
        out.b.push_back(p.b);
    }
    return out;
}

}  // namespace

double Hull::min_at(double t) const {
    double v = std::numeric_limits<double>::infinity();
    for (size_t i = 0; i < a.size(); ++i) v = std::min(v, b[i] + a[i] * t);
    return v;
}

double Hull::max_at(double t) const {
    double v = -std::numeric_limits<double>::infinity();
    for (size_t i = 0; i < a.size(); ++i) v = std::max(v, b[i] + a[i] * t);
    return v;
}

Hull lower_hull_src(const PointSource& s) { return lower_impl(s); }

Hull upper_hull_src(const PointSource& s) {
    NegSource neg(s);
    Hull h = lower_impl(neg);
    for (double& v : h.b) v = -v;
    return h;
}

Hull lower_hull(const double* a, const double* b, int64_t n) {
    ArraySource s;
    s.a = a;
    s.b = b;
    s.n = n;
    s.sign = 1.0;
    return lower_impl(s);
}

Hull upper_hull(const double* a, const double* b, int64_t n) {
    ArraySource s;
    s.a = a;
    s.b = b;
    s.n = n;
    s.sign = 1.0;
    return upper_hull_src(s);
}

}  // namespace rg
