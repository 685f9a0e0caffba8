// HITRAN-2004 160-character line records -> columns (host only, no device).
//
// Column widths follow radis/api/hitranapi.py:82-105 (id a2, iso a1, wav a12,
// int a10, A a10, airbrd a5, selbrd a5, El a10, Tdpair a4, Pshft a8, four
// 15-character quanta fields, ierr a6, iref a12, lmix a1, gp a7, gpp a7).
// The reference reads the file as fixed-size byte records with numpy.fromfile
// and casts each field (radis/api/tools.py:25-78, 111-151); here the text is
// split into records at line terminators and the numeric fields are converted
// in parallel, each with a correctly rounded decimal-to-double conversion
// (Clinger's exact fast path for short decimals, std::from_chars for the
// rest), so every value equals Python's float() of the field.
//
// Record rules: a record ends at "\n", "\r\n" or a lone "\r" (or the end of
// the text); records shorter than 67 characters (the end of the Pshft field)
// are skipped; fields beyond the end of a shorter record are empty.  A field
// is stripped of blanks; an empty numeric field reads as NaN; id must be an
// integer; iso is one character: '1'-'9', '0' = 10, 'A'/'a' = 11, 'B' = 12, ...
// (HITEMP's labels for isotopologues above 9, radis/api/tools.py:141-143).
// Text is taken as ASCII bytes.
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "rg_internal.h"

namespace rg {
namespace {

constexpr int kMinRecord = 67;   // end of the Pshft field

struct Fld {
    int off, width;
    const char* name;
};
constexpr Fld kId{0, 2, "id"}, kIso{2, 1, "iso"}, kV0{3, 12, "wav"}, kS{15, 10, "int"}, kA{25, 10, "A"},
    kGair{35, 5, "airbrd"}, kGself{40, 5, "selbrd"}, kEl{45, 10, "El"}, kNair{55, 4, "Tdpair"},
    kDelta{59, 8, "Pshft"}, kGp{146, 7, "gp"}, kGpp{153, 7, "gpp"};

inline bool blank(char c) { return c == ' ' || c == '\t' || c == '\v' || c == '\f'; }

// [b, e) of field f in a record of length len, stripped of blanks
inline void field(const char* rec, int64_t len, const Fld& f, const char** b, const char** e) {
    int64_t lo = std::min<int64_t>(f.off, len), hi = std::min<int64_t>(f.off + f.width, len);
    const char* p = rec + lo;
    const char* q = rec + hi;
    while (p < q && blank(*p)) ++p;
    while (q > p && blank(q[-1])) --q;
    *b = p;
    *e = q;
}

// Exact powers of ten (10^22 is the largest that a double holds exactly).
constexpr double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                               1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};

// Clinger's fast path (W. D. Clinger, "How to read floating point numbers
// accurately", PLDI 1990): a decimal m 10^q with at most 15 significant digits
// (m < 2^53) and |q| <= 22 is m * 10^q or m / 10^-q of two exact doubles, one
// correctly rounded operation.  Returns false (the caller converts with
// from_chars) for anything else: more digits, larger exponents, inf/nan,
// malformed text.
inline bool fast_decimal(const char* b, const char* e, double* out) {
    const char* p = b;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) {
        neg = *p == '-';
        ++p;
    }
    uint64_t m = 0;
    int digits = 0, frac = 0;
    bool any = false, dot = false;
    for (; p < e; ++p) {
        const char c = *p;
        if (c >= '0' && c <= '9') {
            any = true;
            if (dot) ++frac;
            if (m == 0 && c == '0') continue;   // leading zeros are not significant
            if (++digits > 15) return false;
            m = m * 10 + (uint64_t)(c - '0');
        } else if (c == '.' && !dot) {
            dot = true;
        } else {
            break;
        }
    }
    if (!any) return false;
    int x = 0;
    if (p < e) {
        if (*p != 'e' && *p != 'E') return false;
        ++p;
        bool xneg = false;
        if (p < e && (*p == '+' || *p == '-')) {
            xneg = *p == '-';
            ++p;
        }
        if (p == e) return false;
        for (; p < e; ++p) {
            if (*p < '0' || *p > '9' || x > 1000) return false;
            x = x * 10 + (*p - '0');
        }
        if (xneg) x = -x;
    }
    const int q = x - frac;
    double v;
    if (m == 0) v = 0.0;
    else if (q >= 0 && q <= 22) v = (double)m * kPow10[q];
    else if (q < 0 && q >= -22) v = (double)m / kPow10[-q];
    else return false;
    *out = neg ? -v : v;
    return true;
}

// float() of a stripped field: optional sign, decimal or exponent form,
// inf/nan; the whole field must convert (no digit-group underscores, as in
// numpy's cast of the byte fields).
inline bool to_double(const char* b, const char* e, double* out) {
    if (b == e) {
        *out = std::numeric_limits<double>::quiet_NaN();
        return true;
    }
    if (fast_decimal(b, e, out)) return true;
    bool neg = false;
    if (*b == '+' || *b == '-') {
        neg = *b == '-';
        ++b;
        if (b == e || *b == '+' || *b == '-') return false;
    }
    if (std::find(b, e, '(') != e) return false;   // from_chars takes nan(...); float() does not
    double v = 0.0;
    const auto r = std::from_chars(b, e, v, std::chars_format::general);
    if (r.ptr != e) return false;
    if (r.ec == std::errc::result_out_of_range) {
        // from_chars leaves v untouched when the value is beyond the double
        // range; Python's float() rounds it to inf (positive exponent) or to 0
        // (negative exponent).  Fields are at most 12 characters, so only an
        // exponent can take a value out of range.
        const char* x = std::find_if(b, e, [](char c) { return c == 'e' || c == 'E'; });
        if (x == e) return false;
        v = (x + 1 < e && x[1] == '-') ? 0.0 : std::numeric_limits<double>::infinity();
    } else if (r.ec != std::errc()) {
        return false;
    }
    *out = neg ? -v : v;
    return true;
}

inline bool to_int(const char* b, const char* e, int32_t* out) {
    if (b == e) return false;
    if (*b == '+') {
        ++b;
        if (b == e || *b == '-') return false;
    }
    int32_t v;
    const auto r = std::from_chars(b, e, v, 10);
    if (r.ec != std::errc() || r.ptr != e) return false;
    *out = v;
    return true;
}

inline bool to_iso(const char* b, const char* e, int32_t* out) {
    if (b == e) {   // blank: isotopologue 1
        *out = 1;
        return true;
    }
    if (e - b != 1) return false;
    const char c = *b;
    if (c >= '1' && c <= '9') *out = c - '0';
    else if (c == '0') *out = 10;
    else if (c >= 'A' && c <= 'Z') *out = 11 + (c - 'A');
    else if (c >= 'a' && c <= 'z') *out = 11 + (c - 'a');
    else return false;
    return true;
}

// End of the line starting at p (the first '\n' or '\r' in [p, e), or e).
inline int64_t line_end(const char* t, int64_t p, int64_t e) {
    const void* nl = std::memchr(t + p, '\n', (size_t)(e - p));
    const int64_t q = nl ? (const char*)nl - t : e;
    const void* cr = std::memchr(t + p, '\r', (size_t)(q - p));
    return cr ? (const char*)cr - t : q;
}

// Start of the first record at or after byte s (s = 0 or just past a terminator).
int64_t record_start(const char* t, int64_t n, int64_t s) {
    if (s <= 0) return 0;
    if (s >= n) return n;
    if (t[s - 1] == '\n') return s;
    if (t[s - 1] == '\r' && t[s] != '\n') return s;
    const int64_t p = line_end(t, s, n);
    if (p >= n) return n;
    if (t[p] == '\r' && p + 1 < n && t[p + 1] == '\n') return p + 2;
    return p + 1;
}

// Calls f(rec, len) for every line in [b, e) (terminators removed).
template <typename F>
void for_lines(const char* t, int64_t b, int64_t e, F&& f) {
    int64_t p = b;
    while (p < e) {
        int64_t q = line_end(t, p, e);
        if (!f(t + p, q - p)) return;
        if (q < e && t[q] == '\r' && q + 1 < e && t[q + 1] == '\n') q += 2;
        else q += 1;
        p = q;
    }
}

int pick_threads(int threads, int64_t nbytes) {
    int T = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
    T = std::min(T, 128);
    const int64_t per = 1 << 20;   // at least 1 MB of text per thread
    return (int)std::max<int64_t>(1, std::min<int64_t>(T, (nbytes + per - 1) / per));
}

struct Chunk {
    int64_t b = 0, e = 0;
    int64_t records = 0, lines = 0;   // records kept / all lines
    int64_t bad_line = 0;             // 1-based line within the chunk of the first bad field
    const char* bad_field = nullptr;
    std::string bad_text;
};

void split(const char* t, int64_t n, int T, std::vector<Chunk>* ch) {
    ch->assign(T, Chunk());
    for (int i = 0; i < T; ++i) (*ch)[i].b = record_start(t, n, n * i / T);
    for (int i = 0; i < T; ++i) (*ch)[i].e = i + 1 < T ? (*ch)[i + 1].b : n;
}

template <typename F>
void run_chunks(int T, F&& f) {
    if (T == 1) {
        f(0);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(T);
    for (int i = 0; i < T; ++i) th.emplace_back([&f, i] { f(i); });
    for (auto& x : th) x.join();
}

}  // namespace

int hitran_count(const char* text, int64_t nbytes, int threads, int64_t* n_records) {
    const int T = pick_threads(threads, nbytes);
    std::vector<Chunk> ch;
    split(text, nbytes, T, &ch);
    run_chunks(T, [&](int i) {
        Chunk& c = ch[i];
        for_lines(text, c.b, c.e, [&](const char*, int64_t len) {
            c.records += len >= kMinRecord;
            return true;
        });
    });
    int64_t n = 0;
    for (const Chunk& c : ch) n += c.records;
    *n_records = n;
    return RG_OK;
}

int hitran_parse(const char* text, int64_t nbytes, int threads, const rg_hitran_columns* out, std::string* err) {
    const int T = pick_threads(threads, nbytes);
    std::vector<Chunk> ch;
    split(text, nbytes, T, &ch);
    // pass 1: records and lines per chunk
    run_chunks(T, [&](int i) {
        Chunk& c = ch[i];
        for_lines(text, c.b, c.e, [&](const char*, int64_t len) {
            c.records += len >= kMinRecord;
            c.lines += 1;
            return true;
        });
    });
    int64_t total = 0;
    std::vector<int64_t> first(T), line0(T);
    int64_t lines = 0;
    for (int i = 0; i < T; ++i) {
        first[i] = total;
        line0[i] = lines;
        total += ch[i].records;
        lines += ch[i].lines;
    }
    if (total != out->n) {
        *err = "the text holds " + std::to_string(total) + " records, the columns " + std::to_string(out->n);
        return RG_ERR_ARG;
    }
    // pass 2: convert
    run_chunks(T, [&](int i) {
        Chunk& c = ch[i];
        int64_t r = first[i], ln = 0;
        for_lines(text, c.b, c.e, [&](const char* rec, int64_t len) {
            ++ln;
            if (len < kMinRecord) return true;
            const char *b, *e;
            auto bad = [&](const Fld& f) {
                c.bad_line = ln;
                c.bad_field = f.name;
                c.bad_text.assign(b, e);
                return false;
            };
            auto dbl = [&](const Fld& f, double* col) {
                if (!col) return true;
                field(rec, len, f, &b, &e);
                double v;
                if (!to_double(b, e, &v)) return bad(f);
                col[r] = v;
                return true;
            };
            if (out->id) {
                field(rec, len, kId, &b, &e);
                int32_t v;
                if (!to_int(b, e, &v)) return bad(kId);
                out->id[r] = v;
            }
            if (out->iso) {
                field(rec, len, kIso, &b, &e);
                int32_t v;
                if (!to_iso(b, e, &v)) return bad(kIso);
                out->iso[r] = v;
            }
            if (!dbl(kV0, out->v0) || !dbl(kS, out->s_ref) || !dbl(kA, out->a) || !dbl(kGair, out->g_air) ||
                !dbl(kGself, out->g_self) || !dbl(kEl, out->e_low) || !dbl(kNair, out->n_air) ||
                !dbl(kDelta, out->delta) || !dbl(kGp, out->gp) || !dbl(kGpp, out->gpp))
                return false;
            ++r;
            return true;
        });
    });
    for (int i = 0; i < T; ++i)
        if (ch[i].bad_line) {
            *err = "line " + std::to_string(line0[i] + ch[i].bad_line) + ", field " + ch[i].bad_field + ": '" +
                   ch[i].bad_text + "' does not convert";
            return RG_ERR_ARG;
        }
    return RG_OK;
}

}  // namespace rg
