// Device kernels of the LDM/DIT synthesis for sm_103a.
//
// Pipeline of one spectrum (radis/gpu/gpu.py:255-282 is the reference order):
//   k_scatter       fused per-line scaling + 2x2x2 scatter into a shared-memory
//                   LDM tile, flushed once to HBM with plain stores
//                   (replaces cmdFillLDM.comp:75-145 and the buffer clear)
//   k_col_fft_fwd   first half of a four-step FFT: length-n1 DFTs down the
//                   columns of two packed node rows + twiddle
//   k_row_fft_voigt second half: length-n2 DFT of each row, times the analytic
//                   Voigt FT of the node pair, summed over pairs
//                   (replaces the R2C FFT + cmdApplyLineshapes.comp:51-90)
//   k_row_ifft      inverse row DFTs + twiddle, in place
//   k_col_ifft      inverse column DFTs, real part, scaled, first n_v samples
//                   (replaces the C2R IFFT)
// Two real node rows a, b are transformed as one complex row z = a + i b.
// With W = V_a - i V_b, sum_j Z_j W_j = G and abscoeff = Re(IFFT(G)) / (N dv):
// the Hermitian pairing of bins k and N-k is absorbed by taking the real part.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <type_traits>

#include "rg_internal.h"

namespace rg {

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float lg2(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }
// multiply by -i (forward-direction quarter turn)
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }

// ---------------------------------------------------------------------------
// forward DFTs of radix 2, 3, 4, 5, 8 in registers (exp(-2 pi i n k / R))
// ---------------------------------------------------------------------------
__device__ __forceinline__ void dft2(float2* v) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}
__device__ __forceinline__ void dft4(float2* v) {
    float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    float2 s13 = cadd(v[1], v[3]), d13 = mul_mi(csub(v[1], v[3]));
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13);
    v[3] = csub(d02, d13);
}
__device__ __forceinline__ void dft3(float2* v) {
    const float c1 = -0.5f, s1 = 0.86602540378443864676f;   // cos/sin(2 pi / 3)
    float2 t = cadd(v[1], v[2]);
    float2 d = csub(v[1], v[2]);
    float2 a0 = v[0];
    v[0] = cadd(a0, t);
    float2 m = make_float2(a0.x + c1 * t.x, a0.y + c1 * t.y);
    // -i * s1 * d
    float2 r = make_float2(s1 * d.y, -s1 * d.x);
    v[1] = cadd(m, r);
    v[2] = csub(m, r);
}
__device__ __forceinline__ void dft5(float2* v) {
    const float c1 = 0.30901699437494742410f, s1 = 0.95105651629515357212f;  // 2 pi / 5
    const float c2 = -0.80901699437494742410f, s2 = 0.58778525229247312917f; // 4 pi / 5
    float2 a0 = v[0];
    float2 t1 = cadd(v[1], v[4]), d1 = csub(v[1], v[4]);
    float2 t2 = cadd(v[2], v[3]), d2 = csub(v[2], v[3]);
    v[0] = make_float2(a0.x + t1.x + t2.x, a0.y + t1.y + t2.y);
    float2 m1 = make_float2(a0.x + c1 * t1.x + c2 * t2.x, a0.y + c1 * t1.y + c2 * t2.y);
    float2 m2 = make_float2(a0.x + c2 * t1.x + c1 * t2.x, a0.y + c2 * t1.y + c1 * t2.y);
    // forward: X1 = m1 - i (s1 d1 + s2 d2), X4 = m1 + i (...)
    float2 q1 = make_float2(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y);
    float2 q2 = make_float2(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y);
    v[1] = cadd(m1, mul_mi(q1));
    v[4] = csub(m1, mul_mi(q1));
    v[2] = cadd(m2, mul_mi(q2));
    v[3] = csub(m2, mul_mi(q2));
}
__device__ __forceinline__ void dft8(float2* v) {
    const float r = 0.70710678118654752440f;
    // radix-2 split: even / odd halves
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    dft4(e);
    dft4(o);
    // twiddles w8^k = exp(-i pi k / 4), k = 0..3
    float2 o1 = make_float2(r * (o[1].x + o[1].y), r * (o[1].y - o[1].x));
    float2 o2 = mul_mi(o[2]);
    float2 o3 = make_float2(r * (o[3].y - o[3].x), -r * (o[3].x + o[3].y));
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);
    v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);
    v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);
    v[7] = csub(e[3], o3);
}

// exp(-2 pi i M / N) at compile time: octant-free quadrant reduction of the
// exact fraction M / N, then Taylor series on [0, pi/2) (double, ~1e-16)
constexpr double kPiC = 3.14159265358979323846;
__host__ __device__ constexpr double csin_q(double y) {
    double t = y, s = y;
    for (int k = 1; k < 14; ++k) {
        t *= -y * y / ((2.0 * k) * (2.0 * k + 1.0));
        s += t;
    }
    return s;
}
__host__ __device__ constexpr double ccos_q(double y) {
    double t = 1.0, s = 1.0;
    for (int k = 1; k < 14; ++k) {
        t *= -y * y / ((2.0 * k - 1.0) * (2.0 * k));
        s += t;
    }
    return s;
}
__host__ __device__ constexpr double ctw(int m, int n, bool sine) {
    const int mm = ((m % n) + n) % n;
    const int q = 4 * mm / n;                                  // quadrant
    const double y = 2.0 * kPiC * (double)(4 * mm - q * n) / (4.0 * n);   // in [0, pi/2)
    const double c = ccos_q(y), sn = csin_q(y);
    if (!sine) return q == 0 ? c : q == 1 ? -sn : q == 2 ? -c : sn;
    return q == 0 ? sn : q == 1 ? c : q == 2 ? -sn : -c;
}
template <int M, int N>
struct TwConst {   // exp(-2 pi i M / N)
    static constexpr float re = (float)ctw(M, N, false);
    static constexpr float im = (float)-ctw(M, N, true);
};
template <int R>
__device__ __forceinline__ void dftR(float2* v);

// Stage 1 of a length-A B DFT, in place: for column n2 (N2), the A-point DFT
// of v[B n1 + n2] over n1, each output k1 times exp(-2 pi i n2 k1 / (A B))
// (compile-time constants), written back to v[B k1 + n2].
template <int A, int B, int N2, int K1>
__device__ __forceinline__ void twiddle_col(float2* v, const float2* t) {
    if constexpr (K1 < A) {
        constexpr int e = N2 * K1 % (A * B);
        if constexpr (e == 0)
            v[B * K1 + N2] = t[K1];
        else
            v[B * K1 + N2] = cmul(t[K1], make_float2(TwConst<e, A * B>::re, TwConst<e, A * B>::im));
        twiddle_col<A, B, N2, K1 + 1>(v, t);
    }
}
template <int A, int B, int N2>
__device__ __forceinline__ void dft_stage1(float2* v) {
    if constexpr (N2 < B) {
        float2 t[A];
#pragma unroll
        for (int n1 = 0; n1 < A; ++n1) t[n1] = v[B * n1 + N2];
        dftR<A>(t);
        twiddle_col<A, B, N2, 0>(v, t);
        dft_stage1<A, B, N2 + 1>(v);
    }
}

// DFT of length A B in registers, natural order in and out (Cooley-Tukey,
// n = B n1 + n2, k = k1 + A k2), in place: stage 1 above, then the B-point
// DFTs of v[B k1 + n2] over n2 back into the same slots, which leaves
// X[k1 + A k2] in v[B k1 + k2]; a compile-time register permutation restores
// natural order.
template <int A, int B>
__device__ __forceinline__ void dftAB(float2* v) {
    constexpr int N = A * B;
    dft_stage1<A, B, 0>(v);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) dftR<B>(v + B * k1);
    float2 t[N];
#pragma unroll
    for (int r = 0; r < N; ++r) t[r] = v[B * (r % A) + r / A];
#pragma unroll
    for (int r = 0; r < N; ++r) v[r] = t[r];
}

// radices of the FFT plans: 2, 3, 4, 5, 8 and the composites 6, 9, 10, 12 of
// the small factors
template <int R>
__device__ __forceinline__ void dftR(float2* v) {
    if constexpr (R == 2) dft2(v);
    else if constexpr (R == 3) dft3(v);
    else if constexpr (R == 4) dft4(v);
    else if constexpr (R == 5) dft5(v);
    else if constexpr (R == 8) dft8(v);
    else if constexpr (R == 6) dftAB<2, 3>(v);
    else if constexpr (R == 9) dftAB<3, 3>(v);
    else if constexpr (R == 10) dftAB<2, 5>(v);
    else if constexpr (R == 12) dftAB<4, 3>(v);
}
// dispatch of a run-time radix to f(integral_constant<R>), instantiating only
// the radices up to MAXR (other radices never reach the call)
template <int MAXR = 12, class F>
__device__ __forceinline__ void with_radix(int R, F&& f) {
    switch (R) {
        case 2: f(std::integral_constant<int, 2>()); break;
        case 3: f(std::integral_constant<int, 3>()); break;
        case 4: f(std::integral_constant<int, 4>()); break;
        case 5: f(std::integral_constant<int, 5>()); break;
        case 6: f(std::integral_constant<int, 6>()); break;
        case 9: if constexpr (MAXR >= 9) f(std::integral_constant<int, 9>()); break;
        case 10: if constexpr (MAXR >= 10) f(std::integral_constant<int, 10>()); break;
        case 12: if constexpr (MAXR >= 12) f(std::integral_constant<int, 12>()); break;
        default: f(std::integral_constant<int, 8>()); break;
    }
}

// Multiply v[1..R-1] by w^r, w = tw[s] (tw[t] = exp(-2 pi i t / L)); three
// table reads at most, the other powers by complex products.
template <int R>
__device__ __forceinline__ void twiddle(float2* v, const float2* __restrict__ tw, int s) {
    const float2 w1 = __ldg(&tw[s]);
    if (R == 2) {
        v[1] = cmul(v[1], w1);
    } else if (R == 3) {
        v[1] = cmul(v[1], w1);
        v[2] = cmul(v[2], __ldg(&tw[2 * s]));
    } else if (R == 4) {
        const float2 w2 = __ldg(&tw[2 * s]);
        v[1] = cmul(v[1], w1);
        v[2] = cmul(v[2], w2);
        v[3] = cmul(v[3], cmul(w1, w2));
    } else if (R == 5) {
        const float2 w2 = __ldg(&tw[2 * s]);
        v[1] = cmul(v[1], w1);
        v[2] = cmul(v[2], w2);
        v[3] = cmul(v[3], cmul(w1, w2));
        v[4] = cmul(v[4], cmul(w2, w2));
    } else if (R == 8) {
        const float2 w2 = __ldg(&tw[2 * s]);
        const float2 w4 = __ldg(&tw[4 * s]);
        const float2 w3 = cmul(w1, w2);
        v[1] = cmul(v[1], w1);
        v[2] = cmul(v[2], w2);
        v[3] = cmul(v[3], w3);
        v[4] = cmul(v[4], w4);
        v[5] = cmul(v[5], cmul(w1, w4));
        v[6] = cmul(v[6], cmul(w2, w4));
        v[7] = cmul(v[7], cmul(w3, w4));
    } else {   // composite radix: w^r by products, from the table at every 4th power
        float2 w = w1;
#pragma unroll
        for (int r = 1; r < R; ++r) {
            if (r > 1) w = (r % 4 == 0) ? __ldg(&tw[r * s]) : cmul(w, w1);
            v[r] = cmul(v[r], w);
        }
    }
}

// One Stockham autosort pass over a single transform of length L held in
// shared memory (sub-transforms of length Ns before the pass): butterfly j
// reads in[j + r L/R], twiddles by w_{Ns R}^{r (j mod Ns)} and writes
// out[(j / Ns) Ns R + (j mod Ns) + r Ns].
// Row buffers are padded by one element every 16 (index i lives at
// rp(i) = i + i/16) so that the stride-R writes of the first pass spread over
// the banks.
__device__ __forceinline__ int rp(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int row_buf_len(int n) { return n + (n >> 4) + 1; }

template <int R, bool PIN, bool POUT>
__device__ __forceinline__ void row_pass(const float2* __restrict__ in, float2* __restrict__ out, int L,
                                         int Ns, unsigned mag, const float2* __restrict__ tw) {
    const int M = L / R;
    const int twstep = L / (Ns * R);
    for (int j = threadIdx.x; j < M; j += blockDim.x) {
        const int q = Ns == 1 ? j : (int)__umulhi((unsigned)j, mag);
        const int k = j - q * Ns;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = in[PIN ? rp(j + r * M) : j + r * M];
        if (Ns > 1) twiddle<R>(v, tw, k * twstep);
        dftR<R>(v);
        const int base = q * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) out[POUT ? rp(base + r * Ns) : base + r * Ns] = v[r];
    }
}

template <bool PIN, bool POUT>
__device__ __forceinline__ void row_pass_r(int R, const float2* in, float2* out, int L, int Ns, unsigned mag,
                                           const float2* tw) {
    with_radix(R, [&](auto rc) { row_pass<decltype(rc)::value, PIN, POUT>(in, out, L, Ns, mag, tw); });
}

// Forward DFT of one row in shared memory; buf0 holds the input (plain
// layout).  Only the first pass's strided writes (and the second pass's reads
// of them) use the padded layout rp(); later passes access in plain layout.
// Returns the buffer holding the result; *padded tells its layout.  Ends with
// __syncthreads().
__device__ float2* fft_row(float2* buf0, float2* buf1, const FftLen& P, bool* padded) {
    float2* in = buf0;
    float2* out = buf1;
    for (int p = 0; p < P.npass; ++p) {
        const int R = P.radix[p];
        const int Ns = P.ns[p];
        const unsigned mag = P.mag[p];
        if (p == 0)
            row_pass_r<false, true>(R, in, out, P.L, Ns, mag, P.tw);
        else if (p == 1)
            row_pass_r<true, false>(R, in, out, P.L, Ns, mag, P.tw);
        else
            row_pass_r<false, false>(R, in, out, P.L, Ns, mag, P.tw);
        __syncthreads();
        float2* t = in;
        in = out;
        out = t;
    }
    *padded = P.npass == 1;
    return in;
}

// Column FFT of length N1 in {8, 64, 512} = 8^d, B columns per CTA, N1/8
// threads per column, one radix-8 butterfly per thread and pass with the
// eight values in registers; passes exchange through one shared buffer
// [N1][B].  On entry v[q] = x[j + q N1/8] of column b; on return
// v[r] = X[j + r N1/8].
template <int N1>
struct ColShape {
    static constexpr int TPC = N1 / 8;
    static constexpr int B = N1 == 512 ? 8 : 32;
    static constexpr int THREADS = TPC * B;
};

template <int N1>
__device__ __forceinline__ void col_fft8(float2 (&v)[8], float2* sm, int j, int b,
                                         const float2* __restrict__ tw1) {
    constexpr int TPC = ColShape<N1>::TPC;
    constexpr int B = ColShape<N1>::B;
    dft8(v);
    if constexpr (N1 > 8) {
        // pass 1 (Ns = 1) writes out[8 j + r]
#pragma unroll
        for (int r = 0; r < 8; ++r) sm[(8 * j + r) * B + b] = v[r];
        __syncthreads();
#pragma unroll
        for (int r = 0; r < 8; ++r) v[r] = sm[(j + r * TPC) * B + b];
        const int k = j & 7;
        twiddle<8>(v, tw1, (N1 / 64) * k);      // w_64^{r k}
        dft8(v);
        if constexpr (N1 > 64) {
            __syncthreads();
            // pass 2 (Ns = 8) writes out[(j - k) 8 + k + 8 r]
#pragma unroll
            for (int r = 0; r < 8; ++r) sm[((j - k) * 8 + k + 8 * r) * B + b] = v[r];
            __syncthreads();
#pragma unroll
            for (int r = 0; r < 8; ++r) v[r] = sm[(j + r * TPC) * B + b];
            twiddle<8>(v, tw1, j);              // w_512^{r j}
            dft8(v);
        }
    }
}

// exp(-2 pi i t / N) from a two-level table (t = hi * 1024 + lo)
__device__ __forceinline__ float2 twiddle_n(const float2* __restrict__ hi, const float2* __restrict__ lo,
                                            int t) {
    return cmul(__ldg(&hi[t >> 10]), __ldg(&lo[t & 1023]));
}

// ---------------------------------------------------------------------------
// line preparation at upload: (hi, lo) split of v0 and log2 of the intensity
// ---------------------------------------------------------------------------
__global__ void k_prepare_lines(const double* __restrict__ v0, const double* __restrict__ s, int64_t n,
                                double c2_tref, float2* __restrict__ v0_out, float* __restrict__ ls2,
                                int* unsorted) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = v0[i];
    float hi = (float)v;
    float lo = (float)(v - (double)hi);
    v0_out[i] = make_float2(hi, lo);
    double si = s[i];
    // log2 S_ref - log2(1 - exp(-c2 v0 / Tref)) : the stimulated-emission
    // denominator of base.py:2676 is constant per line
    double l = si > 0.0 ? log2(si) - log2(-expm1(-c2_tref * v)) : -INFINITY;
    ls2[i] = (float)l;
    if (i + 1 < n && v0[i + 1] < v) atomicExch(unsorted, 1);
}

// first line index with v0 >= vmin + c dv, for c = c_min + idx
__global__ void k_col_index(const float2* __restrict__ v0, int64_t n, double vmin, double dv, int c_min,
                            int count, int64_t* __restrict__ col_start) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count) return;
    const double target = vmin + (double)(c_min + idx) * dv;
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = lo + ((hi - lo) >> 1);
        float2 w = v0[mid];
        double v = (double)w.x + (double)w.y;
        if (v < target)
            lo = mid + 1;
        else
            hi = mid;
    }
    col_start[idx] = lo;
}

// most lines with v0 in columns [c - 1 - E, c + 1 + E) over the grid columns
__global__ void k_col_cmax(const int64_t* __restrict__ col_start, int col_off, int col_count, int n_v, int E,
                           int* __restrict__ cmax) {
    int m = 0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_v; c += gridDim.x * blockDim.x) {
        const int lo = max(0, min(c - 1 - E + col_off, col_count - 1));
        const int hi = max(0, min(c + 1 + E + col_off, col_count - 1));
        m = max(m, (int)min(col_start[hi] - col_start[lo], (int64_t)0x3fffffff));
    }
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(cmax, m);
}

// ---------------------------------------------------------------------------
// K1: fused line scaling + LDM scatter into a shared-memory tile
// ---------------------------------------------------------------------------
// Tile layout [node][TK + 1]: the odd row pitch puts column c of node n on
// bank (n + c) mod 32.  The lanes of a warp hold neighbouring (sorted) lines,
// i.e. the same few columns at scattered nodes, so their atomics spread over
// the banks, and every address is a row base plus a column offset.

// --- TMA (cp.async.bulk) + mbarrier helpers ---------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// The thread may stay suspended inside try_wait until the phase completes or
// the hint (ns) runs out, so waiting warps do not spin on the issue slots.
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    constexpr uint32_t kSuspendHintNs = 1000000;
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "n"(kSuspendHintNs)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Bounded wait (`limit` SM clock cycles); false when it gives up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit = kScatWaitCycles) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > limit) return false;
    return true;
}

struct Stage {
    const float2* v0;
    const float* ls2;
    const float* el;
    const float* ga;
    const float* gs;
    const float* na;
    const float* dl;
    const uint8_t* iso;
};

__device__ __forceinline__ Stage stage_view(unsigned char* base, int chunk, bool has_dl, bool has_iso) {
    Stage s;
    s.v0 = reinterpret_cast<const float2*>(base);
    s.ls2 = reinterpret_cast<const float*>(base + 8 * chunk);
    s.el = reinterpret_cast<const float*>(base + 12 * chunk);
    s.ga = reinterpret_cast<const float*>(base + 16 * chunk);
    s.gs = reinterpret_cast<const float*>(base + 20 * chunk);
    s.na = reinterpret_cast<const float*>(base + 24 * chunk);
    s.dl = has_dl ? reinterpret_cast<const float*>(base + 28 * chunk) : nullptr;
    s.iso = has_iso ? reinterpret_cast<const uint8_t*>(base + 32 * chunk) : nullptr;
    return s;
}

// One thread: copy lines [start, start + count) of every column into a stage
// buffer (16-line granularity: the arrays are padded to a multiple of 16).
__device__ __forceinline__ void issue_chunk(const ScatterArgs& a, unsigned char* base, uint64_t* bar, int start,
                                            int count) {
    const uint32_t cp = (uint32_t)((count + kLinePad - 1) / kLinePad * kLinePad);
    const int ch = a.chunk;
    uint32_t bytes = cp * 8 + cp * 4 * 5;
    if (a.dl) bytes += cp * 4;
    if (a.iso) bytes += cp;
    // the buffer was last read through the generic proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, bytes);
    tma_load_1d(base, a.v0 + start, cp * 8, bar);
    tma_load_1d(base + 8 * ch, a.ls2 + start, cp * 4, bar);
    tma_load_1d(base + 12 * ch, a.el + start, cp * 4, bar);
    tma_load_1d(base + 16 * ch, a.ga + start, cp * 4, bar);
    tma_load_1d(base + 20 * ch, a.gs + start, cp * 4, bar);
    tma_load_1d(base + 24 * ch, a.na + start, cp * 4, bar);
    if (a.dl) tma_load_1d(base + 28 * ch, a.dl + start, cp * 4, bar);
    if (a.iso) tma_load_1d(base + 32 * ch, a.iso + start, cp, bar);
}

// TF32 operands (round to nearest, ties away) and mma.sync m16n8k8 with FP32
// accumulators: a[0..3] = A (row g, col t), (g + 8, t), (g, t + 4),
// (g + 8, t + 4); b0, b1 = B (row t, col g), (t + 4, g); d = (g, 2t), (g, 2t
// + 1), (g + 8, 2t), (g + 8, 2t + 1), with g = lane / 4, t = lane % 4.
// TF32 rounding to nearest, ties away from zero (the rna mode) on the bit
// pattern: half a TF32 unit (bit 12) added to the magnitude bits, the 13 low
// mantissa bits cleared; a carry out of the mantissa bumps the exponent, as
// rounding up must.  Two integer instructions; finite inputs only (the
// operands here are sums of finite line contributions).
__device__ __forceinline__ uint32_t tf32_rna(float x) { return (__float_as_uint(x) + 0x1000u) & 0xFFFFE000u; }
__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// --- per-line quantities at the conditions of a ScatterArgs -----------------
// (shared by the scatter, the tangent scatter and the adjoint gather)

// Fractional grid position of the (pressure-shifted) line centre, in
// double-float: ((hi - vmin_hi) + (lo - vmin_lo + shift)) / dv = fk + tv,
// fk integral, tv in [0, 1).
__device__ __forceinline__ void line_position(const ScatterArgs& a, float2 v, float dl, float& fk, float& tv) {
    float s, e1;
    two_sum(v.x, -a.vmin_hi, s, e1);
    e1 += (v.y - a.vmin_lo) + dl * a.p_atm;
    const float p = s * a.inv_dv_hi;
    const float pe = fmaf(s, a.inv_dv_hi, -p) + fmaf(s, a.inv_dv_lo, e1 * a.inv_dv_hi);
    fk = floorf(p);
    tv = (p - fk) + pe;
    const float fl = floorf(tv);
    fk += fl;
    tv -= fl;
}

// Gaussian / Lorentzian node cell and fractions (FWHM, log space); log v0 is
// taken relative to v_ref so the FP32 log and offset do not cancel.
__device__ __forceinline__ void line_nodes(const ScatterArgs& a, float v0, float ga, float gs, float na, int is,
                                           int& l0, int& m0, float& tG, float& tL) {
    const float pl = fmaf(lg2(v0 * a.inv_vref), a.lgG_scale, a.cG[is]);
    const float gam = fmaf(a.x_self, gs - ga, ga);
    const float pm = fmaf(lg2(gam), a.lgL_scale, fmaf(na, a.tL, a.cL));
    l0 = min(max((int)floorf(pl), 0), a.NG - 2);
    m0 = min(max((int)floorf(pm), 0), a.NL - 2);
    tG = pl - (float)l0;
    tL = pm - (float)m0;
}

// Scaled intensity S(T) N x Qr exp(-log_scale): exponent log2(S') + a_T El +
// b_iso in double-float, times the stimulated-emission factor.
__device__ __forceinline__ float line_intensity(const ScatterArgs& a, float v0, float el, float ls2, int is) {
    const float ph = el * a.aT_hi;
    const float pe2 = fmaf(el, a.aT_hi, -ph) + el * a.aT_lo;
    float s1, f1, s2, f2;
    two_sum(ph, a.bI_hi[is], s1, f1);
    two_sum(s1, ls2, s2, f2);
    const float arg = s2 + (f1 + f2 + pe2 + a.bI_lo[is]);
    return ex2(arg) * (1.f - ex2(-a.stim_c * v0));
}

// Fixed-point words of the tile accumulator: 32 bits (one native shared
// integer atomic per add) or 64 bits for dense columns (see fx_wide).
template <typename Acc> struct Fx;
template <> struct Fx<unsigned> {
    static constexpr int kWidth = 31;
    __device__ static unsigned to_fx(float v) { return __float2uint_rn(v); }
    __device__ static float to_float(unsigned w) { return __uint2float_rn(w); }
};
template <> struct Fx<unsigned long long> {
    static constexpr int kWidth = 63;
    __device__ static unsigned long long to_fx(float v) { return __float2ull_rn(v); }
    __device__ static float to_float(unsigned long long w) { return __ull2float_rn(w); }
};

// Scale + scatter of the lines of one staged chunk into the tile accumulator.
template <typename Acc>
__device__ __forceinline__ unsigned scatter_chunk(const ScatterArgs& a, const Stage& st, int count, int k_start,
                                                  int tk, Acc* tile, float fxs, int t0, int nt) {
    unsigned counted = 0;
    for (int j = t0; j < count; j += nt) {
        const float2 v = st.v0[j];
        const float dl = st.dl ? st.dl[j] : 0.f;
        float fk, tv;
        line_position(a, v, dl, fk, tv);
        if (!(fk >= 0.f) || fk + 1.f >= (float)a.n_v) continue;   // drop (cmdFillLDM.comp:102)
        const int k0 = (int)fk;
        const int c0 = k0 - k_start;
        const bool own0 = (unsigned)c0 < (unsigned)tk;
        const bool own1 = (unsigned)(c0 + 1) < (unsigned)tk;
        if (!(own0 || own1)) continue;
        if (own0) ++counted;
        const int is = st.iso ? (int)st.iso[j] : 0;
        int l0, m0;
        float tG, tL;
        line_nodes(a, v.x, st.ga[j], st.gs[j], st.na[j], is, l0, m0, tG, tL);
        const float I = line_intensity(a, v.x, st.el[j], st.ls2[j], is) * fxs;
        const float I1 = tv * I;
        const float I0 = I - I1;
        const float w11 = tG * tL;
        const float w10 = tG - w11;          // tG (1 - tL)
        const float w01 = tL - w11;          // (1 - tG) tL
        const float w00 = 1.f - tG - w01;    // (1 - tG)(1 - tL)
        const int pitch = a.TK + 1;
        const int dL = a.NL * pitch;                          // next wG node
        Acc* t = tile + (l0 * a.NL + m0) * pitch + c0;   // (l0, m0) at column c0
        if (own0) {
            atomicAdd(t, Fx<Acc>::to_fx(I0 * w00));
            atomicAdd(t + pitch, Fx<Acc>::to_fx(I0 * w01));
            atomicAdd(t + dL, Fx<Acc>::to_fx(I0 * w10));
            atomicAdd(t + dL + pitch, Fx<Acc>::to_fx(I0 * w11));
        }
        if (own1) {
            atomicAdd(t + 1, Fx<Acc>::to_fx(I1 * w00));
            atomicAdd(t + 1 + pitch, Fx<Acc>::to_fx(I1 * w01));
            atomicAdd(t + 1 + dL, Fx<Acc>::to_fx(I1 * w10));
            atomicAdd(t + 1 + dL + pitch, Fx<Acc>::to_fx(I1 * w11));
        }
    }
    return counted;
}

// Zero `words` accumulator words from thread `i0` in steps of `step` threads,
// 16 bytes per store (the tile starts on a 16-byte boundary).
template <typename Acc>
__device__ __forceinline__ void zero_tile(Acc* tile, int words, int i0, int step) {
    const int n16 = (int)(((size_t)words * sizeof(Acc)) >> 4);
    uint4* z = reinterpret_cast<uint4*>(tile);
    for (int i = i0; i < n16; i += step) z[i] = make_uint4(0u, 0u, 0u, 0u);
    for (int i = (int)(((size_t)n16 << 4) / sizeof(Acc)) + i0; i < words; i += step) tile[i] = 0;
}

// Skeleton rows of a finished 32-bit tile on the tensor cores: Y^T[columns x
// rows] = T^T[columns x nodes] C^T[nodes x rows] with mma.sync m16n8k8 TF32,
// each product split into three (hi hi + lo hi + hi lo; x = hi + lo, hi =
// tf32(x), lo = tf32(x - hi)).  Warp task: 16 columns (M) x the NR row blocks
// of 8 (N); nodes (K) eight per step in the order of the staged node table
// offs[s][t] = (node(s, t), node(s, t + 4)) x pitch.  Tile rows have a pitch
// of 1 (mod 32) words and the table puts the nodes of t = 0..3 in the bank
// classes v, v + 8, v + 16, v + 24, so the A loads (column g / g + 8, node t /
// t + 4) are conflict-free; frag[s][nr][lane] = the coefficients' B fragments
// (b0, b1 hi, then lo), zero where the table repeats a node.
template <int NR, int U>
__device__ __forceinline__ void flush_tc(const ScatterArgs& a, const unsigned* tile, const float4* frag,
                                         const int2* offs, int k_start, int tk, float inv_fx, int cw, int ncw,
                                         int lane) {
    const int g = lane >> 2, t = lane & 3;
    const int n_mt = (tk + 15) >> 4;
    for (int mt = cw; mt < n_mt; mt += ncw) {
        const unsigned* col = tile + (mt << 4) + g;
        float d[NR][4];
#pragma unroll
        for (int nr = 0; nr < NR; ++nr)
#pragma unroll
            for (int i = 0; i < 4; ++i) d[nr][i] = 0.f;
#pragma unroll U
        for (int s = 0; s < a.proj_ks; ++s) {
            const int2 o = offs[s * 4 + t];
            const float v[4] = {__uint2float_rn(col[o.x]), __uint2float_rn(col[o.x + 8]),
                                __uint2float_rn(col[o.y]), __uint2float_rn(col[o.y + 8])};
            uint32_t ah[4], al[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                ah[i] = tf32_rna(v[i]);
                al[i] = tf32_rna(v[i] - __uint_as_float(ah[i]));
            }
            float4 f[NR];
#pragma unroll
            for (int nr = 0; nr < NR; ++nr) f[nr] = frag[(s * NR + nr) * 32 + lane];
#pragma unroll
            for (int nr = 0; nr < NR; ++nr) mma_tf32(d[nr], ah, __float_as_uint(f[nr].x), __float_as_uint(f[nr].y));
#pragma unroll
            for (int nr = 0; nr < NR; ++nr) mma_tf32(d[nr], al, __float_as_uint(f[nr].x), __float_as_uint(f[nr].y));
#pragma unroll
            for (int nr = 0; nr < NR; ++nr) mma_tf32(d[nr], ah, __float_as_uint(f[nr].z), __float_as_uint(f[nr].w));
        }
        // d[nr][i]: column 16 mt + g + 8 (i / 2), row 8 nr + 2 t + i % 2
        const int c = (mt << 4) + g;
#pragma unroll
        for (int nr = 0; nr < NR; ++nr)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = 8 * nr + 2 * t + (i & 1);
                const int cc = c + 8 * (i >> 1);
                if (r < a.proj_rows && cc < tk) __stcs(a.ldm + (int64_t)r * a.row_stride + k_start + cc, d[nr][i] * inv_fx);
            }
    }
}

// Persistent, warp-specialised scatter: CTA b owns tiles b, b + G, b + 2G,
// ...  Warp 0 (one thread) is the producer: it streams the tiles' line
// records chunk by chunk into a ring of `stages` buffers with TMA bulk copies,
// each buffer guarded by a "full" mbarrier (TMA completion) and an "empty"
// one (one arrival per consumer warp).  Warps 1..31 consume: each waits for a
// chunk, scatters its share of the lines into the tile accumulator (32-bit
// fixed point, native integer shared atomics, deterministic) and releases the
// buffer; warps meet only at tile boundaries (a named barrier of the consumer
// warps) to flush the finished tile to HBM with plain stores.  Every wait is
// bounded; a wait that gives up sets the error flag and the CTA stops after
// the copies it issued have landed (bounded).  Acc: the 32- or 64-bit
// fixed-point word of the tile.  U: unrolling of the tensor-core flush's node
// steps (4 where registers allow, 1 in the kernel that holds both variants).
template <typename Acc, int U = 4>
__device__ __forceinline__ void scatter_body(const ScatterArgs& a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int ch = a.chunk;
    const int S = a.stages;
    const size_t sb = scatter_stage_bytes(ch);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + S * sb);
    uint64_t* empty = full + kScatMaxStages;
    int2* rng = reinterpret_cast<int2*>(smem + S * sb + 16 * kScatMaxStages);
    Acc* tile = reinterpret_cast<Acc*>(smem + scatter_fixed_smem(ch, S, a.rng_cap));
    const int pitch = a.TK + 1;
    const int G = gridDim.x;
    const int nq = (a.n_tiles - (int)blockIdx.x + G - 1) / G;   // tiles of this CTA (<= a.rng_cap)
    const int n_words = a.n_nodes * pitch;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_cons_warps = (blockDim.x >> 5) - 1;

    if (nq > a.rng_cap) {   // the host sizes the table for every CTA: never taken
        if (threadIdx.x == 0) atomicExch(a.err, 1u);
        return;
    }
    auto col_idx = [&](int c) { return max(0, min(c + a.col_off, a.col_count - 1)); };
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        const int k_start = ((int)blockIdx.x + q * G) * a.TK;
        const int tk = min(a.TK, a.n_v - k_start);
        const int lo = (int)a.col_start[col_idx(k_start - 1 - a.margin_cols)];
        const int hi = (int)a.col_start[col_idx(k_start + tk + a.margin_cols)];
        rng[q] = make_int2(lo / kLinePad * kLinePad, hi);   // 16-line aligned start
    }
    zero_tile(tile, n_words, (int)threadIdx.x, (int)blockDim.x);
    // skeleton layout: the projection coefficients after the tile, as FP32
    // [node][row] or (32-bit tiles) the tensor-core flush's B fragments and
    // node table
    float* coef = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(tile) +
                                           scatter_coef_offset(n_words, sizeof(Acc)));
    const bool proj = a.proj_coef != nullptr;
    const bool proj_tc = sizeof(Acc) == 4 && proj && a.proj_frag != nullptr;
    const int n_frag = proj_tc ? a.proj_ks * a.proj_nr * 32 : 0;
    const float4* frag_s = reinterpret_cast<const float4*>(coef);
    const int2* offs_s = reinterpret_cast<const int2*>(frag_s + n_frag);
    if (proj_tc) {
        const float4* src = reinterpret_cast<const float4*>(a.proj_frag);
        for (int i = threadIdx.x; i < n_frag; i += blockDim.x) reinterpret_cast<float4*>(coef)[i] = __ldg(&src[i]);
        const int* tbl = reinterpret_cast<const int*>(src + n_frag);
        int* offs = reinterpret_cast<int*>(reinterpret_cast<float4*>(coef) + n_frag);
        for (int i = threadIdx.x; i < a.proj_ks * 8; i += blockDim.x) offs[i] = __ldg(&tbl[i]) * pitch;
    } else if (proj) {
        for (int i = threadIdx.x; i < a.n_real * a.proj_rp; i += blockDim.x) coef[i] = __ldg(&a.proj_coef[i]);
    }
    if (threadIdx.x == 0) {
        for (int b = 0; b < S; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], n_cons_warps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == 0) {   // producer
        if (lane != 0) return;
        uint32_t c = 0;       // chunks issued
        int buf = 0;          // ring slot of chunk c (c mod S, kept incrementally)
        uint32_t round = 0;   // c / S: slot reuse number
        bool bad = false;
        for (int q = 0; q < nq && !bad && !a.withhold; ++q)
            for (int cs = rng[q].x; cs < rng[q].y; cs += ch) {
                if (round > 0 && !mbar_wait(&empty[buf], (round - 1) & 1, a.wait_limit)) {
                    bad = true;
                    break;
                }
                issue_chunk(a, smem + buf * sb, &full[buf], cs, min(ch, rng[q].y - cs));
                ++c;
                if (++buf == S) {
                    buf = 0;
                    ++round;
                }
            }
        if (bad) atomicExch(a.err, 1u);
        // the last copies must land before the CTA may end (normally already
        // consumed); this drain keeps the full bound whatever a.wait_limit is
        for (uint32_t k = c > (uint32_t)S ? c - S : 0; k < c; ++k)
            mbar_wait(&full[k % (uint32_t)S], (k / (uint32_t)S) & 1);
        return;
    }

    // consumers
    const float fxs = fx_scale_of(*a.cmax, Fx<Acc>::kWidth);
    const float inv_fx = 1.f / fxs;
    const bool has_dl = a.dl != nullptr, has_iso = a.iso != nullptr;
    const int ct = threadIdx.x - 32, nct = blockDim.x - 32;
    const int cw = warp - 1;
    int buf = 0;            // ring slot of the next chunk (chunks consumed mod S)
    uint32_t par = 0;       // phase parity of its "full" barrier
    unsigned counted = 0;
    bool bad = false;
    for (int q = 0; q < nq; ++q) {
        const int k_start = ((int)blockIdx.x + q * G) * a.TK;
        const int tk = min(a.TK, a.n_v - k_start);
        const int b = rng[q].y;
        for (int cs = rng[q].x; cs < b && !bad; cs += ch) {
            // every lane acquires the TMA data through the mbarrier itself
            const bool ok = mbar_wait(&full[buf], par, a.wait_limit);
            if (!__all_sync(0xffffffffu, ok)) {
                bad = true;
                break;
            }
            counted += scatter_chunk<Acc>(a, stage_view(smem + buf * sb, ch, has_dl, has_iso), min(ch, b - cs),
                                          k_start, tk, tile, fxs, ct, nct);
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[buf]);   // this warp is done with the buffer
            if (++buf == S) {
                buf = 0;
                par ^= 1u;
            }
        }
        // all consumer warps done with the tile (and agree on failures)
        int any_bad;
        asm volatile(
            "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n barrier.cta.red.or.pred q, 1, %2, p;\n"
            " selp.u32 %0, 1, 0, q;\n}\n"
            : "=r"(any_bad)
            : "r"((unsigned)bad), "r"(nct)
            : "memory");
        if (any_bad) {
            if (threadIdx.x == 32) atomicExch(a.err, 1u);
            return;
        }
        if (proj_tc) {
            if constexpr (sizeof(Acc) == 4) {
                if (a.proj_nr == 2)
                    flush_tc<2, U>(a, tile, frag_s, offs_s, k_start, tk, inv_fx, cw, n_cons_warps, lane);
                else
                    flush_tc<1, U>(a, tile, frag_s, offs_s, k_start, tk, inv_fx, cw, n_cons_warps, lane);
            }
            asm volatile("bar.sync 1, %0;" ::"r"(nct) : "memory");   // every read of the tile done
            zero_tile(tile, n_words, ct, nct);
        } else if (proj) {
            // skeleton rows of the finished tile: warp task (64-column group,
            // block of 4 rows); lane l sums columns l and l + 32 of its group
            // (each load conflict-free across the warp) over the node rows, one
            // 16-byte broadcast coefficient load per node for 8 FMAs
            const int ncg = (tk + 63) >> 6, nrb = a.proj_rp >> 2;
            for (int t = cw; t < ncg * nrb; t += n_cons_warps) {
                const int cg = t % ncg, rb = t / ncg;
                const int c = (cg << 6) + lane;
                if (c >= tk) continue;
                const Acc* col = tile + c;
                const float4* cf = reinterpret_cast<const float4*>(coef) + rb;
                const int cstep = a.proj_rp >> 2;
                const bool two = c + 32 < tk;
                float y0 = 0.f, y1 = 0.f, y2 = 0.f, y3 = 0.f, z0 = 0.f, z1 = 0.f, z2 = 0.f, z3 = 0.f;
#pragma unroll 4
                for (int nd = 0; nd < a.n_real; ++nd) {
                    const float v = Fx<Acc>::to_float(col[nd * pitch]);
                    const float u = two ? Fx<Acc>::to_float(col[nd * pitch + 32]) : 0.f;
                    const float4 w = cf[nd * cstep];
                    y0 = fmaf(w.x, v, y0);
                    y1 = fmaf(w.y, v, y1);
                    y2 = fmaf(w.z, v, y2);
                    y3 = fmaf(w.w, v, y3);
                    z0 = fmaf(w.x, u, z0);
                    z1 = fmaf(w.y, u, z1);
                    z2 = fmaf(w.z, u, z2);
                    z3 = fmaf(w.w, u, z3);
                }
                const int r = rb << 2;
                float* dst = a.ldm + (int64_t)r * a.row_stride + k_start + c;
                const float ys[4] = {y0, y1, y2, y3}, zs[4] = {z0, z1, z2, z3};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    if (r + i >= a.proj_rows) break;
                    __stcs(dst + i * a.row_stride, ys[i] * inv_fx);
                    if (two) __stcs(dst + i * a.row_stride + 32, zs[i] * inv_fx);
                }
            }
            asm volatile("bar.sync 1, %0;" ::"r"(nct) : "memory");   // every read of the tile done
            zero_tile(tile, n_words, ct, nct);
        } else {
            // flush the finished tile as floats, word / fx_scale (a power of
            // two: exact scaling of the rounded word), with plain stores (this
            // CTA owns its columns), and re-zero it
            for (int node = cw; node < a.n_nodes; node += n_cons_warps) {
                Acc* row = tile + node * pitch;
                float* dst = a.ldm + node * a.row_stride + k_start;
                for (int c = lane; c < tk; c += 32) {   // one 128-byte store per warp step
                    // streaming store: the LDM is read once by the next stage, long after
                    __stcs(&dst[c], Fx<Acc>::to_float(row[c]) * inv_fx);
                    row[c] = 0;
                }
            }
        }
        asm volatile("bar.sync 1, %0;" ::"r"(nct) : "memory");
    }
    if (a.in_window) {   // one atomic per warp: per-thread atomics on one word serialise in L2
        const unsigned tot = __reduce_add_sync(0xffffffffu, counted);
        if (lane == 0 && tot) atomicAdd(a.in_window, (unsigned long long)tot);
    }
}

template <typename Acc>
__global__ void __launch_bounds__(kScatThreads, 1) k_scatter(const ScatterArgs a) {
    scatter_body<Acc>(a);
}

// The accumulator chosen on the device from the column bound *cmax (served and
// allocation-free spectra, whose bound is never read back): a32 / a64 are the
// shapes of the two variants; the launch covers the larger grid and shared
// memory (tiles are dealt out by gridDim.x, so the extra CTAs of the smaller
// variant only take fewer tiles each).
__global__ void __launch_bounds__(kScatThreads, 1) k_scatter_auto(const ScatterArgs a32, const ScatterArgs a64) {
    if (fx_wide(*a32.cmax))
        scatter_body<unsigned long long, 1>(a64);
    else
        scatter_body<unsigned, 1>(a32);
}

// ---------------------------------------------------------------------------
// K2: forward column FFT (length n1) of packed node pairs
// ---------------------------------------------------------------------------
// Column-stage output X[k1] of column n2i into y[pair][k1][n2i], times the
// four-step twiddle w_N^{n2i k1} when the row stage does not apply it
// (a.twiddle): w for k1 = j + r N1/8 is w_N^{n2i j} (w_N^{n2i N1/8})^r, two
// table reads and a product recurrence (rounding grows to ~8 ulp at r = 7).
template <int N1>
__device__ __forceinline__ void store_twiddled(float2 (&v)[8], const ColFftArgs& a, int pair, int j, int n2i) {
    constexpr int TPC = ColShape<N1>::TPC;
    float2* y = a.y + (int64_t)(a.pair_base + pair) * N1 * a.n2;
    if (a.twiddle) {
        float2 w = twiddle_n(a.tw_hi, a.tw_lo, n2i * j);
        const float2 step = twiddle_n(a.tw_hi, a.tw_lo, n2i * TPC);
#pragma unroll
        for (int r = 0; r < 8; ++r) {
            v[r] = cmul(v[r], w);
            w = cmul(w, step);
        }
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) y[(int64_t)(j + r * TPC) * a.n2 + n2i] = v[r];
}

template <int N1>
__global__ void __launch_bounds__(ColShape<N1>::THREADS, 3) k_col_fft_fwd(const ColFftArgs a) {
    constexpr int TPC = ColShape<N1>::TPC;
    constexpr int B = ColShape<N1>::B;
    extern __shared__ float2 sm[];
    const int b = threadIdx.x % B;
    const int j = threadIdx.x / B;
    const int c0 = blockIdx.x * B;
    const int pair = blockIdx.y;
    auto node_of = [&](int v) {   // -1: zero row (padding of an odd n_L block)
        if (!a.map_n) return v;
        const int m = v % a.map_NLv;
        return m < a.map_NL ? a.map_l[v / a.map_NLv] * a.map_NL + m : -1;
    };
    const int na = node_of(2 * pair), nb = node_of(2 * pair + 1);
    const float* ra = na >= 0 ? a.ldm + (int64_t)na * a.row_stride : nullptr;
    const float* rb = nb >= 0 ? a.ldm + (int64_t)nb * a.row_stride : nullptr;
    const int n2i = c0 + b;
    float2 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int64_t nidx = (int64_t)(j + q * TPC) * a.n2 + n2i;
        v[q] = nidx < a.n_v ? make_float2(ra ? __ldg(&ra[nidx]) : 0.f, rb ? __ldg(&rb[nidx]) : 0.f)
                            : make_float2(0.f, 0.f);
    }
    col_fft8<N1>(v, sm, j, b, a.f1.tw);
    store_twiddled<N1>(v, a, pair, j, n2i);
}

// ---------------------------------------------------------------------------
// K3: row FFT (length n2) of each pair, Voigt-FT weights, sum over pairs
// ---------------------------------------------------------------------------
constexpr int kRowThreads = 256;      // inverse row kernel

struct NodeV {
    float al, bm, nrm;
    int nf;
};

__device__ __forceinline__ NodeV node_params(const VoigtArgs& a, int node) {
    const int l = a.rowwise ? node : node / a.NL;
    const int m = a.rowwise ? node : node - l * a.NL;
    NodeV n;
    n.al = a.alpha[l];
    n.bm = a.beta[m];
    n.nrm = a.norm[node];
    n.nf = a.any_fold ? (int)a.nfold[node] : 0;
    return n;
}

// folded copies of the Voigt FT (broadening.py:1914-1926): alias frequencies
// q/(2 dv) + (f or 1/(2 dv) - f); rare, kept out of line
__device__ __noinline__ float voigt_folds(float al, float bm, int nf, float f, float half_fs) {
    float v = 0.f;
    for (int q = 1; q <= nf; ++q) {
        const float fq = q * half_fs + ((q & 1) ? half_fs - f : f);
        v += ex2(-fmaf(al * fq, fq, bm * fq));
    }
    return v;
}

__device__ __forceinline__ float voigt_eval(const NodeV& n, float f, float half_fs) {
    float v = ex2(-fmaf(n.al * f, f, n.bm * f));
    if (n.nf) v += voigt_folds(n.al, n.bm, n.nf, f, half_fs);
    return v * n.nrm;
}

// Unfolded Voigt FT with the normalisation folded into the exponent:
// nrm 2^-(al f^2 + bm f) = 2^(lnrm - bm f - al f^2), two FMAs and one ex2.
struct NodeF {
    float nal, nbm, lnrm;
};
__device__ __forceinline__ NodeF node_fast(const VoigtArgs& a, int node) {
    const int l = a.rowwise ? node : node / a.NL;
    NodeF n;
    n.nal = -a.alpha[l];
    n.nbm = -a.beta[a.rowwise ? node : node - l * a.NL];
    n.lnrm = a.lnorm[node];
    return n;
}
__device__ __forceinline__ float voigt_fast(const NodeF& n, float f, float f2) {
    return ex2(fmaf(n.nal, f2, fmaf(n.nbm, f, n.lnrm)));
}

// PAIRS = 2: two pairs travel together through the row transform as float4
// elements (row A in .xy, row B in .zw), sharing index arithmetic, twiddle
// loads and shared-memory instructions; buffers use rp8(i) = i + i/8, which
// keeps every 16-byte access pattern of the passes conflict-free.
// PAIRS = 1 (long rows): float2 elements, rp16(i) = i + i/16.
__device__ __forceinline__ int rp8(int i) { return i + (i >> 3); }
__device__ __forceinline__ int rp16(int i) { return i + (i >> 4); }
template <int PAIRS> struct RowT;
template <> struct RowT<2> {
    using E = float4;
    __device__ static int pad(int i) { return rp8(i); }
    __host__ __device__ static constexpr int len(int n) { return n + (n >> 3) + 1; }
    __device__ static void split(E t, float2& a, float2& b) {
        a = make_float2(t.x, t.y);
        b = make_float2(t.z, t.w);
    }
    __device__ static E join(float2 a, float2 b) { return make_float4(a.x, a.y, b.x, b.y); }
};
template <> struct RowT<1> {
    using E = float2;
    __device__ static int pad(int i) { return rp16(i); }
    // even, so the second work buffer starts 16-byte aligned (cp.async staging)
    __host__ __device__ static constexpr int len(int n) { return n + (n >> 4) + 2; }
    __device__ static void split(E t, float2& a, float2& b) {
        a = t;
        b = make_float2(0.f, 0.f);
    }
    __device__ static E join(float2 a, float2) { return a; }
};

// Row-pass twiddle sources, tw(t) = exp(-2 pi i t / n2): the global table,
// or a two-level table in shared memory, hi[t / 32] lo[t % 32] (one more
// rounding; used by the long-row layouts, whose n2-point table would not stay
// in the L1 left beside their work buffers).
struct TwGlobal {
    const float2* __restrict__ tw;
    __device__ __forceinline__ float2 operator()(int t) const { return __ldg(&tw[t]); }
};
struct TwShared {
    const float2* hi;
    const float2* lo;
    __device__ __forceinline__ float2 operator()(int t) const { return cmul(hi[t >> 5], lo[t & 31]); }
};

template <int R, int PAIRS, class TW>
__device__ __forceinline__ void twiddleP(float2* A, float2* B, const TW& tw, int s) {
    if constexpr (R == 2 || R == 3 || R == 4 || R == 5 || R == 8) {
        float2 w[R];
        w[0] = make_float2(1.f, 0.f);
        w[1] = tw(s);
        if (R >= 3) w[2] = tw(2 * s);
        if (R >= 4) w[3] = cmul(w[1], w[2]);
        if (R == 5) w[4] = cmul(w[2], w[2]);
        if (R == 8) {
            w[4] = tw(4 * s);
            w[5] = cmul(w[1], w[4]);
            w[6] = cmul(w[2], w[4]);
            w[7] = cmul(w[3], w[4]);
        }
#pragma unroll
        for (int r = 1; r < R; ++r) {
            A[r] = cmul(A[r], w[r]);
            if (PAIRS == 2) B[r] = cmul(B[r], w[r]);
        }
    } else {   // composite radix: w^r by products, from the table at every 4th power
        const float2 w1 = tw(s);
        float2 w = w1;
#pragma unroll
        for (int r = 1; r < R; ++r) {
            if (r > 1) w = (r % 4 == 0) ? tw(r * s) : cmul(w, w1);
            A[r] = cmul(A[r], w);
            if (PAIRS == 2) B[r] = cmul(B[r], w);
        }
    }
}

template <int R, int PAIRS, class TW>
__device__ __forceinline__ void row_mid(const typename RowT<PAIRS>::E* __restrict__ in,
                                        typename RowT<PAIRS>::E* __restrict__ out, int L, int Ns, unsigned mag,
                                        const TW& tw) {
    const int M = L / R;
    const int twstep = L / (Ns * R);
    for (int j = threadIdx.x; j < M; j += blockDim.x) {
        const int q = Ns == 1 ? j : (int)__umulhi((unsigned)j, mag);
        const int k = j - q * Ns;
        float2 A[R], B[R];
#pragma unroll
        for (int r = 0; r < R; ++r) RowT<PAIRS>::split(in[RowT<PAIRS>::pad(j + r * M)], A[r], B[r]);
        if (Ns > 1) twiddleP<R, PAIRS, TW>(A, B, tw, k * twstep);
        dftR<R>(A);
        if (PAIRS == 2) dftR<R>(B);
        const int base = q * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) out[RowT<PAIRS>::pad(base + r * Ns)] = RowT<PAIRS>::join(A[r], B[r]);
    }
}

// two work buffers, the optional twiddle table, and the optional staging
// buffer of the next two rows
template <int PAIRS>
__host__ __device__ inline size_t row_voigt_smem(int n2, bool with_twr, bool with_stage, bool with_tws = false) {
    return 2 * (size_t)RowT<PAIRS>::len(n2) * sizeof(typename RowT<PAIRS>::E) +
           (with_twr ? (size_t)n2 * sizeof(float2) : 0) + (with_stage ? 2 * (size_t)n2 * sizeof(float2) : 0) +
           (with_tws ? (size_t)(n2 / 32 + 32) * sizeof(float2) : 0);
}

// Layouts of the forward row kernel: MAXT threads at most, and the block is
// at least the n2/8 butterflies of the last (radix-8) pass, so each thread
// owns one butterfly's 8 output bins and their accumulators.
constexpr int kRowMaxT2 = 384;    // PAIRS = 2, two CTAs per SM (n2 <= 3072)
constexpr int kRowMaxT2L = 768;   // PAIRS = 2, one CTA per SM (n2 <= 6144, work buffers only)
constexpr int kRowMaxT1 = 1024;   // PAIRS = 1, long rows (n2 <= 8192)

// cp.async staging of the next rows of a pair group (16-byte copies that
// bypass L1, completed with wait_group before the first pass reads them)
__device__ __forceinline__ void stage_rows(float2* dst, const float2* ya, const float2* yb, int n2) {
    const int chunks = n2 / 2;   // 16-byte chunks per row
    for (int c = threadIdx.x; c < 2 * chunks; c += blockDim.x) {
        const bool second = c >= chunks;
        const float2* src = (second ? yb : ya) + 2 * (c - (second ? chunks : 0));
        if (second && !yb) continue;
        const uint32_t d = smem_u32(dst + 2 * c);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void stage_wait() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// first pass from the staged rows (stage = [row a | row b], n2 each; row a
// only for PAIRS = 1)
// first pass (sub-transform length 1) from the staged rows: (x four-step
// twiddle from the per-row table twr, when TWR; otherwise the column stage
// applied it) -> registers -> smem
template <int R, int PAIRS, bool TWR>
__device__ __forceinline__ void row_first_staged(const float2* stage, bool two, const float2* twr,
                                                 typename RowT<PAIRS>::E* out, int L) {
    const int M = L / R;
    for (int j = threadIdx.x; j < M; j += blockDim.x) {
        float2 A[R], B[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            A[r] = stage[j + r * M];
            B[r] = PAIRS == 2 && two ? stage[L + j + r * M] : make_float2(0.f, 0.f);
            if (TWR) {
                const float2 w = twr[j + r * M];
                A[r] = cmul(A[r], w);
                B[r] = cmul(B[r], w);
            }
        }
        dftR<R>(A);
        if (PAIRS == 2) dftR<R>(B);
#pragma unroll
        for (int r = 0; r < R; ++r) out[RowT<PAIRS>::pad(j * R + r)] = RowT<PAIRS>::join(A[r], B[r]);
    }
}

// STAGE: the next two rows are staged in a buffer of their own.  SF: the next
// rows are staged in the work buffer that the last pass does not read, and
// the first pass reads them from there (the buffers swap roles).
template <int PAIRS, int MAXT, bool TWR, bool STAGE, bool TWS, bool SF>
__global__ void __launch_bounds__(MAXT, MAXT <= 384 ? 2 : 1) k_row_fft_voigt(const VoigtArgs a) {
    static_assert(STAGE || SF, "the forward row kernel stages its rows");
    using E = typename RowT<PAIRS>::E;
    extern __shared__ float4 sm4[];
    const int n2 = a.n2;
    const int len = RowT<PAIRS>::len(n2);
    E* buf0 = reinterpret_cast<E*>(sm4);
    E* buf1 = buf0 + len;
    float2* twr = TWR ? reinterpret_cast<float2*>(buf1 + len) : nullptr;
    // STAGE (two pairs): the next two rows are staged with cp.async during the passes
    float2* stage = STAGE ? reinterpret_cast<float2*>(buf1 + len) + (TWR ? n2 : 0) : nullptr;
    const int k1 = blockIdx.x;
    const FftLen& P = a.f2;
    // TWS: two-level pass twiddle table after the other buffers (made visible
    // by the barrier after the first pass)
    float2* tws = TWS ? reinterpret_cast<float2*>(buf1 + len) + (TWR ? n2 : 0) + (STAGE ? 2 * n2 : 0) : nullptr;
    if (TWS) {
        for (int t = threadIdx.x; t < n2 / 32; t += blockDim.x) tws[t] = __ldg(&P.tw[32 * t]);
        for (int t = threadIdx.x; t < 32; t += blockDim.x) tws[n2 / 32 + t] = __ldg(&P.tw[t]);
    }
    using TwT = typename std::conditional<TWS, TwShared, TwGlobal>::type;
    TwT twp;
    if constexpr (TWS) twp = TwShared{tws, tws + n2 / 32};
    else twp = TwGlobal{P.tw};
    if (TWR)
        for (int t = threadIdx.x; t < n2; t += blockDim.x) twr[t] = twiddle_n(a.tw_hi, a.tw_lo, k1 * t);
    const int n = (int)a.n;
    const int j0 = blockIdx.y * kPairGroup;
    const int j1 = min(j0 + kPairGroup, a.n_pairs);
    const int ML = n2 / 8;    // butterflies of the last pass (radix 8, sub-length ML)
    const int jl = threadIdx.x;
    float2 acc[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) acc[r] = make_float2(0.f, 0.f);

    auto row_ptr = [&](int jj) { return a.y + ((int64_t)jj * a.n1 + k1) * n2; };
    auto stage_group = [&](float2* dst, int jj) {   // rows of pair group jj (two for PAIRS = 2)
        stage_rows(dst, row_ptr(jj), PAIRS == 2 && jj + 1 < j1 ? row_ptr(jj + 1) : nullptr, n2);
    };
    E* wbuf = buf0;   // first-pass output
    E* fbuf = buf1;   // SF: the staged rows of the current pair group
    if (STAGE && j0 < j1) stage_group(stage, j0);
    if (SF && j0 < j1) stage_group(reinterpret_cast<float2*>(fbuf), j0);
    for (int j = j0; j < j1; j += PAIRS) {
        const bool two = PAIRS == 2 && j + 1 < j1;
        if (STAGE || SF) {
            const float2* src = STAGE ? stage : reinterpret_cast<const float2*>(fbuf);
            stage_wait();
            __syncthreads();   // staged rows (and the twiddle tables) visible to all threads
            with_radix(P.radix[0], [&](auto rc) {
                row_first_staged<decltype(rc)::value, PAIRS, TWR>(src, two, twr, wbuf, n2);
            });
            __syncthreads();   // stage consumed: prefetch the next two rows under the remaining passes
            if (STAGE && j + 2 < j1) stage_group(stage, j + 2);
        }
        E* in = wbuf;
        E* out = fbuf;
        for (int p = 1; p < P.npass - 1; ++p) {
            const int Ns = P.ns[p];
            const unsigned mag = P.mag[p];
            with_radix<kMidRadixMax>(P.radix[p], [&](auto rc) {
                row_mid<decltype(rc)::value, PAIRS, TwT>(in, out, n2, Ns, mag, twp);
            });
            __syncthreads();
            E* t = in;
            in = out;
            out = t;
        }
        // `out` is free until the next first pass: stage the next pair group there
        if (SF && j + PAIRS < j1) stage_group(reinterpret_cast<float2*>(out), j + PAIRS);
        // last pass (radix 8, sub-length ML, no shuffle: output t = jl + r ML),
        // Voigt weights and accumulation in registers
        if (jl < ML) {
            float2 A[8], B[8];
#pragma unroll
            for (int r = 0; r < 8; ++r) RowT<PAIRS>::split(in[RowT<PAIRS>::pad(jl + r * ML)], A[r], B[r]);
            twiddleP<8, PAIRS, TwT>(A, B, twp, jl);   // w_{n2}^{r jl}
            dft8(A);
            if (PAIRS == 2) dft8(B);
            if (!a.any_fold) {
                const NodeF A0 = node_fast(a, 2 * j), A1 = node_fast(a, 2 * j + 1);
                NodeF B0 = A0, B1 = A1;
                if (two) {
                    B0 = node_fast(a, 2 * j + 2);
                    B1 = node_fast(a, 2 * j + 3);
                }
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    const int kk = k1 + a.n1 * (jl + r * ML);
                    const float f = (float)min(kk, n - kk) * a.inv_ndv;
                    const float f2 = f * f;
                    const float va = voigt_fast(A0, f, f2), vb = voigt_fast(A1, f, f2);
                    float2 c = acc[r];
                    c.x += A[r].x * va + A[r].y * vb;
                    c.y += A[r].y * va - A[r].x * vb;
                    if (two) {
                        const float wa = voigt_fast(B0, f, f2), wb = voigt_fast(B1, f, f2);
                        c.x += B[r].x * wa + B[r].y * wb;
                        c.y += B[r].y * wa - B[r].x * wb;
                    }
                    acc[r] = c;
                }
            } else {
                const NodeV A0 = node_params(a, 2 * j), A1 = node_params(a, 2 * j + 1);
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    const int kk = k1 + a.n1 * (jl + r * ML);
                    const float f = (float)min(kk, n - kk) * a.inv_ndv;
                    const float va = voigt_eval(A0, f, a.half_fs);
                    const float vb = voigt_eval(A1, f, a.half_fs);
                    float2 c = acc[r];
                    c.x += A[r].x * va + A[r].y * vb;
                    c.y += A[r].y * va - A[r].x * vb;
                    acc[r] = c;
                }
                if (two) {
                    const NodeV B0 = node_params(a, 2 * j + 2), B1 = node_params(a, 2 * j + 3);
#pragma unroll
                    for (int r = 0; r < 8; ++r) {
                        const int kk = k1 + a.n1 * (jl + r * ML);
                        const float f = (float)min(kk, n - kk) * a.inv_ndv;
                        const float wa = voigt_eval(B0, f, a.half_fs);
                        const float wb = voigt_eval(B1, f, a.half_fs);
                        float2 c = acc[r];
                        c.x += B[r].x * wa + B[r].y * wb;
                        c.y += B[r].y * wa - B[r].x * wb;
                        acc[r] = c;
                    }
                }
            }
        }
        __syncthreads();
        if (SF) {   // the staged rows are in `out`; the next first pass writes `in`
            wbuf = in;
            fbuf = out;
        }
    }
    if (a.inv_fused) {
        // K3b on the CTA's own sums: inverse DFT = conj(forward DFT(conj(G))),
        // through the work buffers (free after the last pair group), then the
        // inverse four-step twiddle w_N^{-t k1}; the row is stored once
        float2* f0 = reinterpret_cast<float2*>(sm4);
        float2* f1 = f0 + row_buf_len(n2);
        if (jl < ML) {
#pragma unroll
            for (int r = 0; r < 8; ++r) f0[jl + r * ML] = conjf2(acc[r]);
        }
        __syncthreads();
        bool padded;
        const float2* res = fft_row(f0, f1, a.f2, &padded);
        float2* g = a.g + (int64_t)k1 * n2;
        for (int t = threadIdx.x; t < n2; t += blockDim.x) {
            float2 z = conjf2(res[padded ? rp(t) : t]);
            if (k1 && t) z = cmul(z, conjf2(twiddle_n(a.tw_hi, a.tw_lo, t * k1)));
            g[t] = z;
        }
        return;
    }
    if (jl < ML) {
        float2* g = a.g + (int64_t)k1 * n2;
        if (a.store_g && gridDim.y == 1) {   // the only pair group of this row: plain stores
#pragma unroll
            for (int r = 0; r < 8; ++r) g[jl + r * ML] = acc[r];
        } else {
#pragma unroll
            for (int r = 0; r < 8; ++r) atomicAdd(&g[jl + r * ML], acc[r]);
        }
    }
}

// ---------------------------------------------------------------------------
// K3b: inverse row FFT (length n2) and inverse twiddle w_N^{-n2 k1}, in place
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kRowThreads) k_row_ifft(const RowIfftArgs a) {
    extern __shared__ float2 sm[];
    const int n2 = a.n2;
    float2* buf0 = sm;
    float2* buf1 = sm + row_buf_len(n2);
    const int k1 = blockIdx.x;
    float2* g = a.g + (int64_t)k1 * n2;
    for (int t = threadIdx.x; t < n2; t += blockDim.x) buf0[t] = conjf2(g[t]);
    __syncthreads();
    // inverse DFT = conj(forward DFT(conj(x)))
    bool padded;
    const float2* res = fft_row(buf0, buf1, a.f2, &padded);
    for (int t = threadIdx.x; t < n2; t += blockDim.x) {
        float2 z = conjf2(res[padded ? rp(t) : t]);
        if (k1 && t) z = cmul(z, conjf2(twiddle_n(a.tw_hi, a.tw_lo, t * k1)));
        g[t] = z;
    }
}

// ---------------------------------------------------------------------------
// K4: inverse column FFT (length n1), real part, scaled, first n_v samples
// ---------------------------------------------------------------------------
// Post-processing epilogue (radis/lbl/factory.py:1284-1297 and
// radis/spectrum/equations.py:21-44): absorbance A L, emissivity
// -expm1(-A L), transmittance 1 - emissivity, radiance emissivity x Planck
// (radis/phys/blackbody.py:35-74, mW / cm2 / sr / nm at lambda = 1e7/nu nm).
__device__ __forceinline__ void quantities_at(const ColFftArgs& a, int64_t k, float A) {
    const float tau = A * a.q_scale * a.q_path;      // absorbance in physical units
    const float eps = -expm1f(-tau);
    const float nu = (float)(a.q_vmin + a.q_dv * (double)k);
    const float lam = 0.01f / nu;                    // m
    // 2 h c^2 / lambda^5 / expm1(h c / (lambda k T)) W m-3 sr-1 -> mW cm-2 sr-1 nm-1 (x 1e-10)
    const float l2 = lam * lam;
    const float planck = 1.19104297e-16f / (l2 * l2 * lam) / expm1f(a.q_c2_T * nu) * 1e-10f;
    const int64_t n = a.n_v;
    a.q_out[k] = A * a.q_path;
    a.q_out[n + k] = eps;
    a.q_out[2 * n + k] = 1.f - eps;
    a.q_out[3 * n + k] = eps * planck;
}

template <int N1>
__global__ void __launch_bounds__(ColShape<N1>::THREADS) k_col_ifft(const ColFftArgs a) {
    constexpr int TPC = ColShape<N1>::TPC;
    constexpr int B = ColShape<N1>::B;
    extern __shared__ float2 sm[];
    const int b = threadIdx.x % B;
    const int j = threadIdx.x / B;
    const int n2i = blockIdx.x * B + b;
    float2 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = conjf2(a.h[(int64_t)(j + q * TPC) * a.n2 + n2i]);
    col_fft8<N1>(v, sm, j, b, a.f1.tw);
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int64_t nidx = (int64_t)(j + r * TPC) * a.n2 + n2i;
        if (nidx < a.n_v) {
            const float A = v[r].x * a.out_scale;   // Re(conj(z)) = Re(z)
            a.out[nidx] = A;
            if (a.q_out) quantities_at(a, nidx, A);
        }
    }
    // last kernel of the spectrum: hand the error flag to the host (mapped
    // memory, read after the stream synchronises) and clear it
    if (a.err_pub && blockIdx.x == 0 && threadIdx.x == 0) {
        *a.err_pub = *a.err;
        *a.err = 0u;
    }
}

// ---------------------------------------------------------------------------
// Derivatives with respect to (T, p, x), node axes held fixed.
//
// With the axes fixed the Voigt weights of the nodes are constants, so the
// spectrum is a fixed linear map C of the LDM and only the LDM depends on
// (T, p, x): dA/dtheta = C dLDM/dtheta.  Per line, the LDM holds
// I w(tv, tG, tL) in 8 cells (trilinear weights of the three fractional
// coordinates), so dLDM/dtheta is a scatter of
//   I (dlnI/dtheta w + dw/dtv dtv/dtheta + dw/dtG dtG/dtheta + dw/dtL dtL/dtheta).
// Forward mode (tangent): scatter that into a float LDM and run it through C
// (the ordinary FFT / Voigt / inverse FFT kernels).
// Reverse mode (adjoint): C restricted to one node is a symmetric circular
// convolution (V is real and even), so C^T g for node n is the same
// convolution of the upstream gradient g: Re(IFFT(FFT(g) V_n)) / (N dv).  The
// adjoint LDM for all nodes comes from one forward FFT of g and one inverse
// FFT per node pair (k_row_ifft_adj, k_col_ifft_adj; V_a + i V_b puts node a
// in the real and node b in the imaginary part), and the per-line chain rule
// gathers it back at each line's 8 cells (k_gather_grad).
// ---------------------------------------------------------------------------

// K2 on float rows: rows 2 pair and 2 pair + 1 of a.src, or (a.single) the
// single row a.src with a zero partner.
template <int N1>
__global__ void __launch_bounds__(ColShape<N1>::THREADS) k_col_fft_fwd_f(const ColFftArgs a) {
    constexpr int TPC = ColShape<N1>::TPC;
    constexpr int B = ColShape<N1>::B;
    extern __shared__ float2 sm[];
    const int b = threadIdx.x % B;
    const int j = threadIdx.x / B;
    const int pair = blockIdx.y;
    const float* ra = a.src + (a.single ? 0 : (int64_t)(2 * pair) * a.row_stride);
    const float* rb = a.single ? nullptr : ra + a.row_stride;
    const int n2i = blockIdx.x * B + b;
    float2 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int64_t nidx = (int64_t)(j + q * TPC) * a.n2 + n2i;
        // buffer offset of FFT index nidx, or -1 where the row is zero
        int64_t off = -1;
        if (a.ext == 0) {
            if (nidx < a.n_v) off = nidx;
        } else if (nidx < a.n_v + a.ext) {
            off = nidx + a.ext;
        } else if (nidx >= a.n - a.ext) {
            off = nidx - (a.n - a.ext);
        }
        v[q] = off >= 0 ? make_float2(__ldg(&ra[off]), rb ? __ldg(&rb[off]) : 0.f) : make_float2(0.f, 0.f);
    }
    col_fft8<N1>(v, sm, j, b, a.f1.tw);
    store_twiddled<N1>(v, a, pair, j, n2i);
}

// Gaussian stage of the merged layout (see GaussArgs).  One CTA: one merged
// row (wL node), kGaussTile consecutive outputs, kGaussPer per thread.  A merged row is
// sum over wide nodes l of (d_l conv LDM_{l,m}) with the symmetric residual
// kernel d_l[j] = c_l 2^(-a2_l j^2), |j| <= K_l, i.e. out[p] = sum_jj d[jj]
// x[p - ext - K + jj]; each thread keeps its outputs' input window in registers
// and advances it 8 taps at a time (two half-windows used alternately, so the
// window never moves between registers).  The shared base Gaussian of the
// wide nodes is applied after the FFT, by the row kernel.
template <int P>
__device__ __forceinline__ void gauss_step(float (&acc)[P], const float (&lo)[P], const float (&hi)[8],
                                           const float (&g)[8]) {
    // window = lo[0..P) followed by hi[0..8): acc[i] += sum_u g[u] window[i + u]
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int i = 0; i < P; ++i) acc[i] = fmaf(g[u], i + u < P ? lo[i + u] : hi[i + u - P], acc[i]);
}

__device__ __forceinline__ void load8(float (&d)[8], const float* s) {
    const float4 a = *reinterpret_cast<const float4*>(s);
    const float4 b = *reinterpret_cast<const float4*>(s + 4);
    d[0] = a.x; d[1] = a.y; d[2] = a.z; d[3] = a.w;
    d[4] = b.x; d[5] = b.y; d[6] = b.z; d[7] = b.w;
}

// acc[i] += sum_jj taps[jj] xs[t0 + i + jj], jj < KP (a multiple of 4; xs
// readable up to t0 + KP + 7): three 8-value register blocks rotate through
// the window (no moves): taps jj..jj+7 use A ++ B, jj+8.. use B ++ C, jj+16..
// use C ++ A'; a tail of up to two 8-tap steps and one 4-tap step ends the
// row of taps.
// Four taps on the same window form (the tail of a row of taps whose count
// is 4 mod 8): acc[i] += sum_{u < 4} g[u] window[i + u], window = lo ++ hi.
__device__ __forceinline__ void gauss_step4(float (&acc)[8], const float (&lo)[8], const float4 hi, const float4 g4) {
    const float hv[3] = {hi.x, hi.y, hi.z};
    const float g[4] = {g4.x, g4.y, g4.z, g4.w};
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i] = fmaf(g[u], i + u < 8 ? lo[i + u] : hv[i + u - 8], acc[i]);
}

__device__ __forceinline__ void conv_window(float (&acc)[8], const float* xs, const float* taps, int t0, int KP) {
    float A[8], B[8], C[8], g[8];
    load8(A, &xs[t0]);
    int jj = 0;
    for (; jj + 24 <= KP; jj += 24) {
        load8(B, &xs[t0 + jj + 8]);
        load8(g, &taps[jj]);
        gauss_step<8>(acc, A, B, g);
        load8(C, &xs[t0 + jj + 16]);
        load8(g, &taps[jj + 8]);
        gauss_step<8>(acc, B, C, g);
        load8(A, &xs[t0 + jj + 24]);
        load8(g, &taps[jj + 16]);
        gauss_step<8>(acc, C, A, g);
    }
    // tail of 0-20 taps: up to two 8-tap steps, then one 4-tap step
    const int r = KP - jj;
    if (r >= 8) {
        load8(B, &xs[t0 + jj + 8]);
        load8(g, &taps[jj]);
        gauss_step<8>(acc, A, B, g);
        if (r >= 16) {
            load8(C, &xs[t0 + jj + 16]);
            load8(g, &taps[jj + 8]);
            gauss_step<8>(acc, B, C, g);
            if (r & 4)
                gauss_step4(acc, C, *reinterpret_cast<const float4*>(&xs[t0 + jj + 24]),
                            *reinterpret_cast<const float4*>(&taps[jj + 16]));
        } else if (r & 4) {
            gauss_step4(acc, B, *reinterpret_cast<const float4*>(&xs[t0 + jj + 16]),
                        *reinterpret_cast<const float4*>(&taps[jj + 8]));
        }
    } else if (r & 4) {
        gauss_step4(acc, A, *reinterpret_cast<const float4*>(&xs[t0 + jj + 8]),
                    *reinterpret_cast<const float4*>(&taps[jj]));
    }
}

// Nodes are streamed through a ring of kGaussStages shared-memory slots, each
// holding one node's taps and window, filled with cp.async (zero-filled
// outside the row) kGaussStages - 1 nodes ahead of the convolution: one
// barrier per node and no staging through registers.
constexpr int kGaussStages = 4;

__device__ __forceinline__ void cp_async16(float* dst, const float* src, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__global__ void __launch_bounds__(256) k_gauss_merge(const GaussArgs a) {
    extern __shared__ __align__(16) float gsm[];
    constexpr int TW = kGaussTile;
    constexpr int P = kGaussPer;                     // outputs per thread (8)
    constexpr int S = kGaussStages;
    const int r = blockIdx.y;
    const int p0 = blockIdx.x * TW;                  // first output (buffer position)
    const int Lr = a.n_v + 2 * a.ext;
    float* orow = a.out + (int64_t)r * a.out_stride;
    const int m = r;   // merged row of wL node m
    float acc[P];
#pragma unroll
    for (int i = 0; i < P; ++i) acc[i] = 0.f;
    const int t0 = threadIdx.x * P;
    // Node w's window starts at LDM index base = p0 - ext - K_w; it is staged
    // from the 16-byte aligned index base & ~3, and the offset s = base & 3 is
    // absorbed by s leading zero taps.
    auto shift_of = [&](int w) { return (p0 - a.ext - a.K[w]) & 3; };
    auto taps_of = [&](int w) { return (2 * a.K[w] + 1 + shift_of(w) + 3) & ~3; };   // multiple of 4
    auto slot_taps = [&](int w) { return gsm + (w % S) * a.slot_len; };
    auto issue = [&](int w) {   // taps (plain stores) and window (cp.async) of node w into its slot
        float* taps = slot_taps(w);
        float* xs = taps + a.slot_taps;
        const int K = a.K[w];
        const int sh = shift_of(w);
        const int KP = taps_of(w);
        for (int jj = threadIdx.x; jj < KP; jj += blockDim.x) {
            const float j = (float)(jj - sh - K);
            taps[jj] = jj >= sh && jj <= sh + 2 * K ? a.c[w] * ex2(-a.a2[w] * j * j) : 0.f;
        }
        const int k0 = (p0 - a.ext - K) & ~3;        // LDM index of xs[0]
        const int n4 = (TW + KP + 8 + 3) / 4;        // 4 n4 <= slot_len - slot_taps
        const float* src = a.ldm + (int64_t)(a.wide_l[w] * a.NL + m) * a.row_stride;
        for (int q = threadIdx.x; q < n4; q += blockDim.x) {
            const int k = k0 + 4 * q;                // rows start 128-byte aligned; k is a multiple of 4
            const int bytes = (k >= 0 && k < a.n_v) ? 4 * min(4, a.n_v - k) : 0;   // zeros outside [0, n_v)
            cp_async16(xs + 4 * q, bytes ? src + k : src, bytes);
        }
    };
#pragma unroll
    for (int w = 0; w < S - 1; ++w) {
        if (w < a.n_wide) issue(w);
        cp_async_commit();
    }
    for (int w = 0; w < a.n_wide; ++w) {
        cp_async_wait<S - 2>();   // this thread's copies of node w have landed
        __syncthreads();          // everyone's have, and everyone is done with node w - 1
        if (w + S - 1 < a.n_wide) issue(w + S - 1);   // into node w - 1's slot
        cp_async_commit();
        const float* taps = slot_taps(w);
        conv_window(acc, taps + a.slot_taps, taps, t0, taps_of(w));
    }
    const int p = p0 + t0;
#pragma unroll
    for (int i = 0; i < P; i += 4) {
        if (p + i + 4 <= Lr) {
            *reinterpret_cast<float4*>(&orow[p + i]) = make_float4(acc[i], acc[i + 1], acc[i + 2], acc[i + 3]);
        } else {
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (p + i + u < Lr) orow[p + i + u] = acc[i + u];
        }
    }
}

// Instrument slit (radis/tools/slit.py:737 and remove_boundary, :1063-1072):
// out[i] = scale sum_j slit[j] in[i + (m-1)/2 - j], the 'same' part of the
// full convolution, zero outside [0, n); written as a correlation with the
// reversed slit r[u] = slit[m-1-u]: out[i] = scale sum_u r[u] in[i - m/2 + u].
// One CTA: kGaussTile outputs (8 per thread); taps in passes of kSlitPass,
// each with its own staged input window, through the same register-window
// convolution as the Gaussian stage.  'valid' mode: the first (la-1)/2 and
// last la/2 outputs are NaN, la = min(n, m).
__global__ void __launch_bounds__(256) k_slit_conv(const SlitArgs a) {
    extern __shared__ __align__(16) float ssm[];
    constexpr int TW = kGaussTile;
    constexpr int P = kGaussPer;
    float* taps = ssm;                       // kSlitPass (padded to 4)
    float* xs = ssm + kSlitPass + 16;        // TW + KP + 8 <= TW + kSlitPass + 16
    const int64_t p0 = (int64_t)blockIdx.x * TW;
    const int t0 = threadIdx.x * P;
    const int64_t half = a.m / 2;
    float acc[P];
#pragma unroll
    for (int i = 0; i < P; ++i) acc[i] = 0.f;
    for (int u0 = 0; u0 < a.m; u0 += kSlitPass) {
        const int kb = min(kSlitPass, a.m - u0);
        const int KP = (kb + 3) & ~3;
        const int64_t base = p0 - half + u0;   // input index of xs[0]
        __syncthreads();   // previous pass consumed
        for (int jj = threadIdx.x; jj < KP; jj += blockDim.x) taps[jj] = jj < kb ? a.slit[a.m - 1 - (u0 + jj)] : 0.f;
        for (int t = threadIdx.x; t < TW + KP + 8; t += blockDim.x) {
            const int64_t k = base + t;
            xs[t] = k >= 0 && k < a.n ? __ldg(&a.in[k]) : 0.f;
        }
        __syncthreads();
        conv_window(acc, xs, taps, t0, KP);
    }
    const int64_t la = a.n < (int64_t)a.m ? a.n : (int64_t)a.m;
    const int64_t ea = a.valid ? (la - 1) / 2 : 0, eb = a.valid ? la / 2 : 0;
#pragma unroll
    for (int i = 0; i < P; ++i) {
        const int64_t idx = p0 + t0 + i;
        if (idx < a.n) a.out[idx] = idx < ea || idx >= a.n - eb ? __int_as_float(0x7fc00000) : acc[i] * a.scale;
    }
}

// Adjoint row stage, one CTA per (row k1, pair j): H = Ghat (V_2j + i V_2j+1)
// on the row's bins k = k1 + n1 t, inverse row DFT, inverse four-step twiddle
// w_N^{-t k1}; output y[j][k1][t].
__global__ void __launch_bounds__(kRowThreads) k_row_ifft_adj(const AdjRowArgs a) {
    extern __shared__ float2 sm[];
    const VoigtArgs& v = a.v;
    const int n2 = v.n2;
    float2* buf0 = sm;
    float2* buf1 = sm + row_buf_len(n2);
    const int k1 = blockIdx.x;
    const int j = blockIdx.y;
    const int n = (int)v.n;
    const NodeV A = node_params(v, 2 * j), B = node_params(v, 2 * j + 1);
    const float2* gh = v.g + (int64_t)k1 * n2;
    for (int t = threadIdx.x; t < n2; t += blockDim.x) {
        const int kk = k1 + v.n1 * t;
        const float f = (float)min(kk, n - kk) * v.inv_ndv;
        const float va = voigt_eval(A, f, v.half_fs);
        const float vb = voigt_eval(B, f, v.half_fs);
        const float2 z = gh[t];
        // inverse DFT = conj(forward DFT(conj(x)))
        buf0[t] = make_float2(z.x * va - z.y * vb, -(z.y * va + z.x * vb));
    }
    __syncthreads();
    bool padded;
    const float2* res = fft_row(buf0, buf1, v.f2, &padded);
    float2* y = a.y + ((int64_t)j * v.n1 + k1) * n2;
    for (int t = threadIdx.x; t < n2; t += blockDim.x) {
        float2 z = conjf2(res[padded ? rp(t) : t]);
        if (k1 && t) z = cmul(z, conjf2(twiddle_n(v.tw_hi, v.tw_lo, t * k1)));
        y[t] = z;
    }
}

// Adjoint column stage: inverse column DFT (length n1) of pair `blockIdx.y`;
// real part -> float row 2 pair, imaginary part -> row 2 pair + 1 of a.out
// (first n_v samples, x out_scale).
template <int N1>
__global__ void __launch_bounds__(ColShape<N1>::THREADS) k_col_ifft_adj(const ColFftArgs a) {
    constexpr int TPC = ColShape<N1>::TPC;
    constexpr int B = ColShape<N1>::B;
    extern __shared__ float2 sm[];
    const int b = threadIdx.x % B;
    const int j = threadIdx.x / B;
    const int pair = blockIdx.y;
    const int n2i = blockIdx.x * B + b;
    const float2* h = a.h + (int64_t)pair * N1 * a.n2;
    float2 v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = conjf2(h[(int64_t)(j + q * TPC) * a.n2 + n2i]);
    col_fft8<N1>(v, sm, j, b, a.f1.tw);
    float* oa = a.out + (int64_t)(2 * pair) * a.row_stride;
    float* ob = oa + a.row_stride;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        const int64_t nidx = (int64_t)(j + r * TPC) * a.n2 + n2i;
        if (nidx < a.n_v) {
            oa[nidx] = v[r].x * a.out_scale;     // Re(conj(z))
            ob[nidx] = -v[r].y * a.out_scale;    // Im(conj(z))
        }
    }
}

// Per-line derivative coefficients: dlnI/dtheta and the rates of the three
// fractional coordinates, for theta = T, p_bar, x (radis/lbl/base.py:2664-2677
// for I, broadening.py:170-172 and 368-381 for the widths, base.py:2351-2370
// for the shift; number density p x / (k T)).
struct LineRates {
    float lnI[3], tv[3], tG[3], tL[3];
};

__device__ __forceinline__ LineRates line_rates(const GradArgs& g, float v0, float el, float ga, float gs, float na,
                                                float dl, int is) {
    LineRates r;
    const float x = g.c2_T * v0;
    // d/dT of ln(exp(-c2 El/T) (1 - exp(-c2 v0/T))), partition ratio and density
    r.lnI[0] = g.c2_T2 * el - g.c2_T2 * v0 / expm1f(x) + g.cT0[is];
    r.lnI[1] = g.iP;
    r.lnI[2] = g.iX;
    r.tv[0] = 0.f;
    r.tv[1] = dl * g.kP;
    r.tv[2] = 0.f;
    r.tG[0] = g.gT;
    r.tG[1] = 0.f;
    r.tG[2] = 0.f;
    const float gam = fmaf(g.s.x_self, gs - ga, ga);
    r.tL[0] = -na * g.lT;
    r.tL[1] = g.lP;
    r.tL[2] = (gs - ga) / gam * g.lX;
    return r;
}

// Reverse mode: out[theta] += sum over lines of I (dlnI S0 + dtv Sk + dtG SG +
// dtL SL), with S0 the adjoint LDM interpolated at the line and Sk, SG, SL its
// differences along the three cell axes.  One FP64 atomic per block and theta.
__global__ void __launch_bounds__(256) k_gather_grad(const GradArgs g) {
    extern __shared__ float gcs[];   // skeleton layout: the coefficients [proj_n][proj_rp]
    const ScatterArgs& a = g.s;
    if (g.proj_coef) {
        for (int i = threadIdx.x; i < g.proj_n * g.proj_rp; i += blockDim.x) gcs[i] = __ldg(&g.proj_coef[i]);
        __syncthreads();
    }
    float acc[3] = {0.f, 0.f, 0.f};
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < g.n_lines; i += stride) {
        const float2 v = a.v0[i];
        const float dl = a.dl ? a.dl[i] : 0.f;
        float fk, tv;
        line_position(a, v, dl, fk, tv);
        if (!(fk >= 0.f) || fk + 1.f >= (float)a.n_v) continue;
        const int k0 = (int)fk;
        const int is = a.iso ? (int)a.iso[i] : 0;
        const float ga = a.ga[i], gs = a.gs[i], na = a.na[i], el = a.el[i];
        int l0, m0;
        float tG, tL;
        line_nodes(a, v.x, ga, gs, na, is, l0, m0, tG, tL);
        const float I = line_intensity(a, v.x, el, a.ls2[i], is);
        if (!(I > 0.f)) continue;
        // the adjoint at the line's 4 nodes, columns k0 and k0 + 1
        float u0[4], u1[4];   // node order (l0, m0), (l0, m0 + 1), (l0 + 1, m0), (l0 + 1, m0 + 1)
        const int n00 = l0 * a.NL + m0;
        if (g.proj_coef) {   // from the skeleton rows
            const int nd[4] = {n00, n00 + 1, n00 + a.NL, n00 + a.NL + 1};
#pragma unroll
            for (int j = 0; j < 4; ++j) u0[j] = u1[j] = 0.f;
            const float* z = g.adj + k0;
            for (int r = 0; r < g.proj_rows; ++r, z += g.row_stride) {
                const float z0 = z[0], z1 = z[1];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float c = gcs[nd[j] * g.proj_rp + r];
                    u0[j] = fmaf(c, z0, u0[j]);
                    u1[j] = fmaf(c, z1, u1[j]);
                }
            }
        } else {
            const float* r00 = g.adj + (int64_t)n00 * g.row_stride + k0;
            const float* rr[4] = {r00, r00 + g.row_stride, r00 + (int64_t)a.NL * g.row_stride,
                                  r00 + (int64_t)(a.NL + 1) * g.row_stride};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                u0[j] = rr[j][0];
                u1[j] = rr[j][1];
            }
        }
        const float d00 = u1[0] - u0[0], d01 = u1[1] - u0[1];
        const float d10 = u1[2] - u0[2], d11 = u1[3] - u0[3];
        const float e00 = fmaf(tv, d00, u0[0]), e01 = fmaf(tv, d01, u0[1]);
        const float e10 = fmaf(tv, d10, u0[2]), e11 = fmaf(tv, d11, u0[3]);
        const float uG = 1.f - tG, uL = 1.f - tL;
        const float S0 = uG * (uL * e00 + tL * e01) + tG * (uL * e10 + tL * e11);
        const float Sk = uG * (uL * d00 + tL * d01) + tG * (uL * d10 + tL * d11);
        const float SG = uL * (e10 - e00) + tL * (e11 - e01);
        const float SL = uG * (e01 - e00) + tG * (e11 - e10);
        const LineRates r = line_rates(g, v.x, el, ga, gs, na, dl, is);
#pragma unroll
        for (int q = 0; q < 3; ++q) acc[q] += I * (r.lnI[q] * S0 + r.tv[q] * Sk + r.tG[q] * SG + r.tL[q] * SL);
    }
    __shared__ double part[3][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        double s = acc[q];
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) part[q][warp] = s;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[threadIdx.x][w];
        atomicAdd(&g.out[threadIdx.x], s);
    }
}

// Forward mode: scatter the tangent of each line's 8 LDM values in direction
// g.theta into the float rows g.tan (FP32 global atomics).
__global__ void __launch_bounds__(256) k_scatter_tangent(const GradArgs g) {
    const ScatterArgs& a = g.s;
    const int th = g.theta;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < g.n_lines; i += stride) {
        const float2 v = a.v0[i];
        const float dl = a.dl ? a.dl[i] : 0.f;
        float fk, tv;
        line_position(a, v, dl, fk, tv);
        if (!(fk >= 0.f) || fk + 1.f >= (float)a.n_v) continue;
        const int k0 = (int)fk;
        const int is = a.iso ? (int)a.iso[i] : 0;
        const float ga = a.ga[i], gs = a.gs[i], na = a.na[i], el = a.el[i];
        int l0, m0;
        float tG, tL;
        line_nodes(a, v.x, ga, gs, na, is, l0, m0, tG, tL);
        const float I = line_intensity(a, v.x, el, a.ls2[i], is);
        if (!(I > 0.f)) continue;
        const LineRates r = line_rates(g, v.x, el, ga, gs, na, dl, is);
        const float K[2] = {1.f - tv, tv}, dK[2] = {-r.tv[th], r.tv[th]};
        const float Gw[2] = {1.f - tG, tG}, dG[2] = {-r.tG[th], r.tG[th]};
        const float Lw[2] = {1.f - tL, tL}, dL[2] = {-r.tL[th], r.tL[th]};
        const float ln = r.lnI[th];
#pragma unroll
        for (int cl = 0; cl < 2; ++cl)
#pragma unroll
            for (int cm = 0; cm < 2; ++cm) {
                float* row = g.tan + (int64_t)((l0 + cl) * a.NL + m0 + cm) * g.row_stride + k0;
                const float gl = Gw[cl] * Lw[cm];
                const float dgl = dG[cl] * Lw[cm] + Gw[cl] * dL[cm];
#pragma unroll
                for (int ck = 0; ck < 2; ++ck) {
                    const float w = K[ck] * gl;
                    const float dw = dK[ck] * gl + K[ck] * dgl;
                    atomicAdd(&row[ck], I * fmaf(ln, w, dw));
                }
            }
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static thread_local const char* g_launch_err = nullptr;
const char* last_launch_error() { return g_launch_err; }

static int check_launch() {
    cudaError_t e = cudaGetLastError();
    g_launch_err = e == cudaSuccess ? nullptr : cudaGetErrorString(e);
    return e == cudaSuccess ? RG_OK : RG_ERR_CUDA;
}

int col_block(int n1) {
    switch (n1) {
        case 8: return ColShape<8>::B;
        case 64: return ColShape<64>::B;
        default: return ColShape<512>::B;
    }
}


// Opt the kernel in to the largest dynamic shared memory the device allows
// next to the kernel's own static shared memory; checks that `need` fits.
// (first call per kernel: queries the attributes and sets the limit; later
// calls only compare `need` with the cached limit)
template <typename K>
static int allow_smem(K kernel, std::atomic<size_t>& avail_cache, size_t need) {
    size_t avail = avail_cache.load();
    if (!avail) {
        int dev = 0, optin = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return RG_ERR_CUDA;
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
            return RG_ERR_CUDA;
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, kernel) != cudaSuccess) return RG_ERR_CUDA;
        avail = (size_t)optin - fa.sharedSizeBytes;
        if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)avail) != cudaSuccess)
            return RG_ERR_CUDA;
        avail_cache.store(avail);
    }
    return need > avail ? RG_ERR_RANGE : RG_OK;
}

#define ALLOW_SMEM(kernel, need)                          \
    do {                                                   \
        static std::atomic<size_t> avail_{0};              \
        int r_ = allow_smem(kernel, avail_, (need));       \
        if (r_ != RG_OK) return r_;                        \
    } while (0)

int launch_prepare_lines(const double* v0_d, const double* s_d, int64_t n, double c2_tref, float2* v0_out,
                         float* ls2_out, int* unsorted_flag, cudaStream_t st) {
    if (n <= 0) return RG_OK;
    int64_t blocks = (n + 255) / 256;
    k_prepare_lines<<<(unsigned)blocks, 256, 0, st>>>(v0_d, s_d, n, c2_tref, v0_out, ls2_out, unsorted_flag);
    return check_launch();
}

int launch_col_index(const float2* v0, int64_t n, double vmin, double dv, int c_min, int count,
                     int64_t* col_start, cudaStream_t st) {
    k_col_index<<<(count + 255) / 256, 256, 0, st>>>(v0, n, vmin, dv, c_min, count, col_start);
    return check_launch();
}

int launch_col_cmax(const int64_t* col_start, int col_off, int col_count, int n_v, int E, int* cmax,
                    cudaStream_t st) {
    if (cudaMemsetAsync(cmax, 0, sizeof(int), st) != cudaSuccess) return RG_ERR_CUDA;
    const int blocks = std::min((n_v + 255) / 256, 1024);
    k_col_cmax<<<std::max(blocks, 1), 256, 0, st>>>(col_start, col_off, col_count, n_v, E, cmax);
    return check_launch();
}

int launch_scatter(const ScatterArgs& a, int grid, int threads, size_t smem, bool wide, cudaStream_t st) {
    if (wide) {
        ALLOW_SMEM(k_scatter<unsigned long long>, smem);
        k_scatter<unsigned long long><<<grid, threads, smem, st>>>(a);
    } else {
        ALLOW_SMEM(k_scatter<unsigned>, smem);
        k_scatter<unsigned><<<grid, threads, smem, st>>>(a);
    }
    return check_launch();
}

int launch_scatter_auto(const ScatterArgs& a32, const ScatterArgs& a64, int grid, int threads, size_t smem,
                        cudaStream_t st) {
    ALLOW_SMEM(k_scatter_auto, smem);
    k_scatter_auto<<<grid, threads, smem, st>>>(a32, a64);
    return check_launch();
}

// Dynamic shared memory a scatter variant may have (one CTA per SM).
template <typename Acc>
static int scatter_optin(size_t* avail) {
    static std::atomic<size_t> cached{0};   // one GPU model per process
    size_t a = cached.load();
    if (!a) {
        int dev = 0, optin = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return RG_ERR_CUDA;
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
            return RG_ERR_CUDA;
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, k_scatter<Acc>) != cudaSuccess) return RG_ERR_CUDA;
        a = (size_t)optin - fa.sharedSizeBytes;
        cached.store(a);
    }
    *avail = a;
    return RG_OK;
}
int scatter_smem_optin(size_t* avail, bool wide) {
    // every variant (and k_scatter_auto) has the same static shared memory
    // (none); the opt-in limit of one serves for all
    return wide ? scatter_optin<unsigned long long>(avail) : scatter_optin<unsigned>(avail);
}

template <int N1>
static int col_fwd(const ColFftArgs& a, cudaStream_t st) {
    ALLOW_SMEM(k_col_fft_fwd<N1>, N1 * ColShape<N1>::B * sizeof(float2));
    dim3 grid(a.n2 / ColShape<N1>::B, a.n_pairs);
    k_col_fft_fwd<N1><<<grid, ColShape<N1>::THREADS, N1 * ColShape<N1>::B * sizeof(float2), st>>>(a);
    return check_launch();
}

int launch_col_fft_fwd(const ColFftArgs& a, cudaStream_t st) {
    switch (a.n1) {
        case 8: return col_fwd<8>(a, st);
        case 64: return col_fwd<64>(a, st);
        case 512: return col_fwd<512>(a, st);
        default: return RG_ERR_RANGE;
    }
}

template <int PAIRS, int MAXT, bool TWR, bool STAGE, bool TWS, bool SF>
static int row_voigt(const VoigtArgs& a, cudaStream_t st) {
    const size_t smem = row_voigt_smem<PAIRS>(a.n2, TWR, STAGE, TWS);
    ALLOW_SMEM((k_row_fft_voigt<PAIRS, MAXT, TWR, STAGE, TWS, SF>), smem);
    dim3 grid(a.n1, (a.n_pairs + kPairGroup - 1) / kPairGroup);
    k_row_fft_voigt<PAIRS, MAXT, TWR, STAGE, TWS, SF><<<grid, a.threads, smem, st>>>(a);
    return check_launch();
}

// Layout of the forward row kernel for rows of n2 points:
//  * n2 <= 3072: two pairs per float4 element, <= 384 threads, the next two
//    rows staged under the passes, and the per-row four-step twiddle table
//    while two CTAs still fit an SM;
//  * n2 <= 6144 (and the two work buffers fit): two pairs, <= 768 threads,
//    one CTA per SM, nothing else in shared memory;
//  * else one pair per element, <= 1024 threads.
// Without the table the column stage applies the four-step twiddle.
RowLayout row_layout(int n2) {
    RowLayout L{};
    if (n2 / 8 <= kRowMaxT2) {
        L.pairs = 2;
        L.maxt = kRowMaxT2;
        L.stage = 1;
        L.twr = row_voigt_smem<2>(n2, true, true) <= 113 * 1024;
    } else if (n2 / 8 <= kRowMaxT2L && row_voigt_smem<2>(n2, false, false, true) <= 227 * 1024) {
        L.pairs = 2;
        L.maxt = kRowMaxT2L;
    } else {
        L.pairs = 1;
        L.maxt = kRowMaxT1;
    }
    return L;
}

int launch_row_fft_voigt(const VoigtArgs& a, cudaStream_t st) {
    if (a.f2.npass < 2 || a.f2.radix[a.f2.npass - 1] != 8) return RG_ERR_RANGE;
    const RowLayout L = row_layout(a.n2);
    if (a.threads < a.n2 / 8 || a.threads > L.maxt || a.threads % 32) return RG_ERR_RANGE;
    if (L.pairs != a.pairs_per_pass || L.twr != a.row_twiddle_table) return RG_ERR_RANGE;
    if (L.maxt == kRowMaxT2)
        return L.twr ? row_voigt<2, kRowMaxT2, true, true, false, false>(a, st)
                     : row_voigt<2, kRowMaxT2, false, true, false, false>(a, st);
    if (L.maxt == kRowMaxT2L) return row_voigt<2, kRowMaxT2L, false, false, true, true>(a, st);
    return row_voigt<1, kRowMaxT1, false, false, true, true>(a, st);
}

int launch_row_ifft(const RowIfftArgs& a, cudaStream_t st) {
    const size_t smem = 2 * (size_t)row_buf_len(a.n2) * sizeof(float2);
    ALLOW_SMEM(k_row_ifft, smem);
    k_row_ifft<<<a.n1, kRowThreads, smem, st>>>(a);
    return check_launch();
}

template <int N1>
static int col_inv(const ColFftArgs& a, cudaStream_t st) {
    ALLOW_SMEM(k_col_ifft<N1>, N1 * ColShape<N1>::B * sizeof(float2));
    k_col_ifft<N1><<<a.n2 / ColShape<N1>::B, ColShape<N1>::THREADS, N1 * ColShape<N1>::B * sizeof(float2), st>>>(a);
    return check_launch();
}

int launch_col_ifft(const ColFftArgs& a, cudaStream_t st) {
    switch (a.n1) {
        case 8: return col_inv<8>(a, st);
        case 64: return col_inv<64>(a, st);
        case 512: return col_inv<512>(a, st);
        default: return RG_ERR_RANGE;
    }
}

template <int N1>
static int col_fwd_f(const ColFftArgs& a, cudaStream_t st) {
    ALLOW_SMEM(k_col_fft_fwd_f<N1>, N1 * ColShape<N1>::B * sizeof(float2));
    dim3 grid(a.n2 / ColShape<N1>::B, a.single ? 1 : a.n_pairs);
    k_col_fft_fwd_f<N1><<<grid, ColShape<N1>::THREADS, N1 * ColShape<N1>::B * sizeof(float2), st>>>(a);
    return check_launch();
}

int launch_col_fft_fwd_f(const ColFftArgs& a, cudaStream_t st) {
    switch (a.n1) {
        case 8: return col_fwd_f<8>(a, st);
        case 64: return col_fwd_f<64>(a, st);
        case 512: return col_fwd_f<512>(a, st);
        default: return RG_ERR_RANGE;
    }
}

int launch_row_ifft_adj(const AdjRowArgs& a, cudaStream_t st) {
    const size_t smem = 2 * (size_t)row_buf_len(a.v.n2) * sizeof(float2);
    ALLOW_SMEM(k_row_ifft_adj, smem);
    dim3 grid(a.v.n1, a.v.n_pairs);
    k_row_ifft_adj<<<grid, kRowThreads, smem, st>>>(a);
    return check_launch();
}

template <int N1>
static int col_inv_adj(const ColFftArgs& a, cudaStream_t st) {
    ALLOW_SMEM(k_col_ifft_adj<N1>, N1 * ColShape<N1>::B * sizeof(float2));
    dim3 grid(a.n2 / ColShape<N1>::B, a.n_pairs);
    k_col_ifft_adj<N1><<<grid, ColShape<N1>::THREADS, N1 * ColShape<N1>::B * sizeof(float2), st>>>(a);
    return check_launch();
}

int launch_col_ifft_adj(const ColFftArgs& a, cudaStream_t st) {
    switch (a.n1) {
        case 8: return col_inv_adj<8>(a, st);
        case 64: return col_inv_adj<64>(a, st);
        case 512: return col_inv_adj<512>(a, st);
        default: return RG_ERR_RANGE;
    }
}

// Row pitch of the projection coefficients: the rows rounded up to a multiple of 4.
int proj_rows_pad(int rows) { return (rows + 3) & ~3; }

// Tensor-core form of the projection pass: Y^T[columns x rows] = X^T[columns
// x nodes] C^T[nodes x rows] with mma.sync m16n8k8 TF32 (columns as M, rows
// as N in steps of 8, nodes as K), each product split into three TF32
// products (hi hi + lo hi + hi lo; x = hi + lo with hi = tf32(x), lo =
// tf32(x - hi)): ~22 significant bits per operand, FP32-level sums.  CTA = 8
// warps over a 256-column tile; warp w owns columns 32 w .. 32 w + 31 as two
// 16-column m-tiles, for every 8-row n-tile (NR of them), accumulators in
// registers; the three products of a k-step are issued part by part over all
// 2 NR accumulators (independent MMAs between dependent ones).  Node rows
// stream through kTcStages shared-memory stages of 16 rows (cp.async,
// zero-filled past n_v and past the last node), row pitch 264 floats: the A
// fragment loads (node t / t + 4, column g / g + 8 of each m-tile) are
// conflict-free.  The B fragments (coefficients, hi and lo parts, prepared on
// the host in fragment order) sit in shared memory, 8 bytes per lane per part.
constexpr int kTcTC = 256;                // columns per CTA tile (8 warps x 32)
constexpr int kTcKC = 16;                 // node rows per stage (two k-steps)
constexpr int kTcPitch = kTcTC + 8;       // staged row pitch (floats)
constexpr int kTcStages = 3;

size_t proj_tc_smem(int row_blocks, int ksteps) {
    return sizeof(float) * ((size_t)row_blocks * ksteps * 128 + (size_t)kTcStages * kTcKC * kTcPitch);
}


template <int NR>
__global__ void __launch_bounds__(256, 2) k_node_project_tc(const ProjArgs a) {
    constexpr int S = kTcStages;
    extern __shared__ __align__(16) float tsm[];
    const int KSP = a.ksteps;                             // node steps of 8 (even, covers n_nodes)
    const int n_chunks = KSP / 2;                         // 16-node chunks per tile
    float* fr = tsm;                                      // fragments [NR][KSP][2][32][2]
    float* xs = tsm + NR * KSP * 128;                     // stages [S][kTcKC][kTcPitch]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int n_tiles = (int)((a.n_v + kTcTC - 1) / kTcTC);
    const int my_tiles = (n_tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    const int total = my_tiles * n_chunks;
    auto tile_k0 = [&](int tt) { return (int64_t)((int)blockIdx.x + tt * (int)gridDim.x) * kTcTC; };
    // this thread's 16-byte pieces of a stage: rows r_0 + 4 i, columns 4 c4_t
    const int r_0 = threadIdx.x / (kTcTC / 4), c4_t = threadIdx.x % (kTcTC / 4);
    auto issue = [&](int gq) {
        const int64_t k = tile_k0(gq / n_chunks) + 4 * c4_t;
        const int nd0 = (gq % n_chunks) * kTcKC + r_0;
        float* dst = xs + (gq % S) * kTcKC * kTcPitch + r_0 * kTcPitch + 4 * c4_t;
        const float* src = a.ldm + (int64_t)nd0 * a.row_stride + k;
        const bool col_ok = k < a.n_v;   // a piece past n_v stays in the row's padding
#pragma unroll
        for (int i = 0; i < kTcKC * kTcTC / 4 / 256; ++i) {
            const bool ok = col_ok && nd0 + 4 * i < a.n_nodes;
            cp_async16(dst + 4 * i * kTcPitch, ok ? src + (int64_t)4 * i * a.row_stride : a.ldm, ok ? 16 : 0);
        }
    };
#pragma unroll
    for (int q = 0; q < S - 1; ++q) {
        if (q < total) issue(q);
        cp_async_commit();
    }
    {
        const float4* src = reinterpret_cast<const float4*>(a.frag);
        float4* dst = reinterpret_cast<float4*>(fr);
        for (int i = threadIdx.x; i < NR * KSP * 32; i += blockDim.x) dst[i] = __ldg(&src[i]);
    }
    for (int tt = 0; tt < my_tiles; ++tt) {
        float d[2][NR][4];
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int nr = 0; nr < NR; ++nr)
#pragma unroll
                for (int i = 0; i < 4; ++i) d[m][nr][i] = 0.f;
        for (int ch = 0; ch < n_chunks; ++ch) {
            const int gq = tt * n_chunks + ch;
            cp_async_wait<S - 2>();
            __syncthreads();
            if (gq + S - 1 < total) issue(gq + S - 1);
            cp_async_commit();
            const float* xb = xs + (gq % S) * kTcKC * kTcPitch + warp * 32 + g;
#pragma unroll
            for (int s2 = 0; s2 < 2; ++s2) {
                const int ks = 2 * ch + s2;
                // A fragments (two m-tiles): (col g / g + 8, node t / t + 4), hi and lo
                uint32_t ah[2][4], al[2][4];
#pragma unroll
                for (int m = 0; m < 2; ++m) {
                    const float* xm = xb + (8 * s2 + t) * kTcPitch + 16 * m;
                    const float v[4] = {xm[0], xm[8], xm[4 * kTcPitch], xm[4 * kTcPitch + 8]};
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        ah[m][i] = tf32_rna(v[i]);
                        al[m][i] = tf32_rna(v[i] - __uint_as_float(ah[m][i]));
                    }
                }
                uint32_t bh[NR][2], bl[NR][2];
#pragma unroll
                for (int nr = 0; nr < NR; ++nr) {
                    const float* f = fr + ((nr * KSP + ks) * 2) * 64 + lane * 2;
                    const float2 h = *reinterpret_cast<const float2*>(f);
                    const float2 l = *reinterpret_cast<const float2*>(f + 64);
                    bh[nr][0] = __float_as_uint(h.x);
                    bh[nr][1] = __float_as_uint(h.y);
                    bl[nr][0] = __float_as_uint(l.x);
                    bl[nr][1] = __float_as_uint(l.y);
                }
#pragma unroll
                for (int m = 0; m < 2; ++m)
#pragma unroll
                    for (int nr = 0; nr < NR; ++nr) mma_tf32(d[m][nr], ah[m], bh[nr][0], bh[nr][1]);
#pragma unroll
                for (int m = 0; m < 2; ++m)
#pragma unroll
                    for (int nr = 0; nr < NR; ++nr) mma_tf32(d[m][nr], al[m], bh[nr][0], bh[nr][1]);
#pragma unroll
                for (int m = 0; m < 2; ++m)
#pragma unroll
                    for (int nr = 0; nr < NR; ++nr) mma_tf32(d[m][nr], ah[m], bl[nr][0], bl[nr][1]);
            }
        }
        // the tile is complete: d[m][nr] = (column g / g + 8 of m-tile m, row 8 nr + 2 t / + 1)
        const int64_t kc = tile_k0(tt) + warp * 32 + g;
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int nr = 0; nr < NR; ++nr)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int r = 8 * nr + 2 * t + (i & 1);
                    const int64_t k = kc + 16 * m + 8 * (i >> 1);
                    if (r < a.rows && k < a.n_v) a.ldm[(int64_t)r * a.row_stride + k] = d[m][nr][i];
                }
    }
}

template <int NR>
int launch_proj_tc(const ProjArgs& a, cudaStream_t st) {
    const size_t smem = proj_tc_smem(NR, a.ksteps);
    ALLOW_SMEM((k_node_project_tc<NR>), smem);
    const int64_t tiles = (a.n_v + kTcTC - 1) / kTcTC;
    // two CTAs per SM where their shared memory fits (fragments of up to ~4 row
    // blocks of a 288-node grid), else one
    const int per_sm = smem <= 110 * 1024 ? 2 : 1;
    const int grid = (int)std::min<int64_t>(tiles, (int64_t)per_sm * std::max(a.sms, 1));
    k_node_project_tc<NR><<<grid, 256, smem, st>>>(a);
    return check_launch();
}

int launch_node_project(const ProjArgs& a, cudaStream_t st) {
    if (a.rows <= 0 || a.rows > kProjMaxRows || a.rows_pad != proj_rows_pad(a.rows) || a.n_nodes <= 0 ||
        a.n_v <= 0 || a.row_stride % 4 != 0 || !a.frag)
        return RG_ERR_ARG;
    if (a.mtiles != (a.rows + 7) / 8 || a.ksteps < (a.n_nodes + 7) / 8 || a.ksteps % 2) return RG_ERR_ARG;
    if (proj_tc_smem(a.mtiles, a.ksteps) > kProjTcSmemMax) return RG_ERR_RANGE;
    switch (a.mtiles) {
    case 1: return launch_proj_tc<1>(a, st);
    case 2: return launch_proj_tc<2>(a, st);
    case 3: return launch_proj_tc<3>(a, st);
    case 4: return launch_proj_tc<4>(a, st);
    case 5: return launch_proj_tc<5>(a, st);
    case 6: return launch_proj_tc<6>(a, st);
    case 7: return launch_proj_tc<7>(a, st);
    case 8: return launch_proj_tc<8>(a, st);
    default: return RG_ERR_ARG;
    }
}

int launch_gauss_merge(const GaussArgs& a0, int out_rows, cudaStream_t st) {
    GaussArgs a = a0;
    const int Lr = a.n_v + 2 * a.ext;
    if (a.n_wide < 0 || a.n_wide > kMaxAxis || a.row_stride % 4) return RG_ERR_RANGE;
    int kp_max = 4;   // taps of the widest node: 2 K + 1 + shift (<= 3), rounded up to 4
    for (int w = 0; w < a.n_wide; ++w) {
        if (a.K[w] < 0 || a.K[w] > kGaussMaxK) return RG_ERR_RANGE;
        kp_max = std::max(kp_max, (2 * a.K[w] + 1 + 3 + 3) & ~3);
    }
    a.slot_taps = kp_max;
    a.slot_len = kp_max + ((kGaussTile + kp_max + 8 + 3) / 4) * 4;   // taps + staged window, 16-byte multiple
    const size_t smem = sizeof(float) * (size_t)kGaussStages * a.slot_len;
    ALLOW_SMEM(k_gauss_merge, smem);
    dim3 grid((Lr + kGaussTile - 1) / kGaussTile, out_rows);
    k_gauss_merge<<<grid, 256, smem, st>>>(a);
    return check_launch();
}

int launch_slit_conv(const SlitArgs& a, cudaStream_t st) {
    if (a.n <= 0) return RG_OK;
    if (a.m <= 0) return RG_ERR_RANGE;
    const size_t smem = sizeof(float) * ((kSlitPass + 16) + (kGaussTile + kSlitPass + 16));
    const int64_t blocks = (a.n + kGaussTile - 1) / kGaussTile;
    if (blocks > 0x7fffffff) return RG_ERR_RANGE;
    k_slit_conv<<<(unsigned)blocks, 256, smem, st>>>(a);
    return check_launch();
}

int launch_gather_grad(const GradArgs& a, int grid, cudaStream_t st) {
    if (a.n_lines <= 0) return RG_OK;
    const size_t smem = a.proj_coef ? sizeof(float) * (size_t)a.proj_n * a.proj_rp : 0;
    ALLOW_SMEM(k_gather_grad, smem);
    k_gather_grad<<<grid, 256, smem, st>>>(a);
    return check_launch();
}

int launch_scatter_tangent(const GradArgs& a, int grid, cudaStream_t st) {
    if (a.n_lines <= 0) return RG_OK;
    k_scatter_tangent<<<grid, 256, 0, st>>>(a);
    return check_launch();
}

}  // namespace rg

namespace rg {
// Thread count of the forward row kernel for a row plan: the multiple of 32
// in [max(128, n2/8), layout limit] that wastes the fewest butterfly slots
// over the passes (ties -> fewer threads).
int row_threads(const FftLen& f) {
    const int maxt = row_layout(f.L).maxt;
    const int t_min = std::max(128, (f.L / 8 + 31) / 32 * 32);
    int best = t_min;
    double best_eff = -1.0;
    for (int T = t_min; T <= maxt; T += 32) {
        long slots = 0, work = 0;
        for (int p = 0; p < f.npass; ++p) {
            const int M = f.L / f.radix[p];
            slots += (long)((M + T - 1) / T) * T;
            work += M;
        }
        const double eff = (double)work / (double)slots;
        if (eff > best_eff + 1e-9) {
            best_eff = eff;
            best = T;
        }
    }
    return best;
}
}  // namespace rg
