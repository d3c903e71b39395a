// Mixed-radix Stockham FFT on lines held in shared memory.
//
// A tile of `nlines` lines of length n sits in shared memory with element
// stride `es` and line stride `ls` (in complex elements).  Each stage of radix
// R reads R elements n/R apart, multiplies by twiddles, applies an R-point
// DFT and writes them Ns apart into the other buffer (self-sorting, so no bit
// reversal).  Twiddles come from a per-CTA table tw[m] = exp(sign*2*pi*i*m/n).
#pragma once
#include <type_traits>
#include <utility>
#include "common.cuh"

namespace pyspec {

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { C r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { C r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename C, typename T> __device__ __forceinline__ C cscale(C a, T s) { C r; r.x = a.x * s; r.y = a.y * s; return r; }
// complex64 add, subtract and scale as packed two-lane FP32 instructions
// (add/sub/mul.rn.f32x2, sm_100+): one instruction per complex operation,
// same rounding as the two scalar ones.  The templates above serve complex128.
__device__ __forceinline__ unsigned long long pk_u64(float2 a) { return *reinterpret_cast<unsigned long long*>(&a); }
__device__ __forceinline__ float2 pk_f2(unsigned long long u) { return *reinterpret_cast<float2*>(&u); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk_u64(a)), "l"(pk_u64(b)));
    return pk_f2(r);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk_u64(a)), "l"(pk_u64(b)));
    return pk_f2(r);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pk_u64(a)), "l"(pk_u64(make_float2(s, s))));
    return pk_f2(r);
}
// multiply by sign*i
template <typename C> __device__ __forceinline__ C cmul_si(C a, int sign) {
    C r;
    if (sign > 0) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; }
    return r;
}

template <typename T> struct FftConst;
template <> struct FftConst<float> {
    static constexpr float s3 = 0.866025403784438647f;   // sin(2pi/3)
    static constexpr float c51 = 0.309016994374947424f;  // cos(2pi/5)
    static constexpr float c52 = -0.809016994374947424f; // cos(4pi/5)
    static constexpr float s51 = 0.951056516295153572f;  // sin(2pi/5)
    static constexpr float s52 = 0.587785252292473129f;  // sin(4pi/5)
    static constexpr float r2 = 0.707106781186547524f;   // 1/sqrt(2)
};
template <> struct FftConst<double> {
    static constexpr double s3 = 0.866025403784438647;
    static constexpr double c51 = 0.309016994374947424;
    static constexpr double c52 = -0.809016994374947424;
    static constexpr double s51 = 0.951056516295153572;
    static constexpr double s52 = 0.587785252292473129;
    static constexpr double r2 = 0.707106781186547524;
};

template <typename T, typename C>
__device__ __forceinline__ void dft2(C* v) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b); v[1] = csub(a, b);
}

template <typename T, typename C>
__device__ __forceinline__ void dft3(C* v, int sign) {
    C a = v[0], b = v[1], c = v[2];
    C s = cadd(b, c);
    C d = csub(b, c);
    C t = csub(a, cscale(s, (T)0.5));
    C u = cmul_si(cscale(d, FftConst<T>::s3), sign);
    v[0] = cadd(a, s);
    v[1] = cadd(t, u);
    v[2] = csub(t, u);
}

template <typename T, typename C>
__device__ __forceinline__ void dft4(C* v, int sign) {
    C a = v[0], b = v[1], c = v[2], d = v[3];
    C ac = cadd(a, c), amc = csub(a, c), bd = cadd(b, d);
    C bmd = cmul_si(csub(b, d), sign);
    v[0] = cadd(ac, bd);
    v[2] = csub(ac, bd);
    v[1] = cadd(amc, bmd);
    v[3] = csub(amc, bmd);
}

template <typename T, typename C>
__device__ __forceinline__ void dft5(C* v, int sign) {
    C a = v[0];
    C t1 = cadd(v[1], v[4]), t2 = csub(v[1], v[4]);
    C t3 = cadd(v[2], v[3]), t4 = csub(v[2], v[3]);
    C r1 = cadd(a, cadd(cscale(t1, FftConst<T>::c51), cscale(t3, FftConst<T>::c52)));
    C r2 = cadd(a, cadd(cscale(t1, FftConst<T>::c52), cscale(t3, FftConst<T>::c51)));
    C i1 = cmul_si(cadd(cscale(t2, FftConst<T>::s51), cscale(t4, FftConst<T>::s52)), sign);
    C i2 = cmul_si(csub(cscale(t2, FftConst<T>::s52), cscale(t4, FftConst<T>::s51)), sign);
    v[0] = cadd(a, cadd(t1, t3));
    v[1] = cadd(r1, i1);
    v[4] = csub(r1, i1);
    v[2] = cadd(r2, i2);
    v[3] = csub(r2, i2);
}

template <typename T, typename C>
__device__ __forceinline__ void dft8(C* v, int sign) {
    C e[4] = {v[0], v[2], v[4], v[6]};
    C o[4] = {v[1], v[3], v[5], v[7]};
    dft4<T>(e, sign);
    dft4<T>(o, sign);
    const T r2 = FftConst<T>::r2;
    // o[k] *= exp(sign*2*pi*i*k/8)
    C w1 = mk<T>(r2, sign * r2), w3 = mk<T>(-r2, sign * r2);
    o[1] = cmul(o[1], w1);
    o[2] = cmul_si(o[2], sign);
    o[3] = cmul(o[3], w3);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        v[k] = cadd(e[k], o[k]);
        v[k + 4] = csub(e[k], o[k]);
    }
}

// ---------------------------------------------------------------------------
// Composite radices R = A*B evaluated in registers (one Cooley-Tukey step):
//   X[k1 + A k2] = DFT_B over n2 of ( W_R^(n2 k1) * DFT_A over n1 of x[B n1 + n2] )
// so a Stockham stage of radix 12, 15, 16, ... replaces two stages of the
// small radices (one pass over shared memory instead of two).  The inner
// twiddles W_R^m are compile-time constants from a constexpr Taylor series
// (double precision, rounded once to T).
// ---------------------------------------------------------------------------
namespace twc {
constexpr double kPi = 3.14159265358979323846;
// sin / cos of x in [-pi, pi] by their Taylor series (terms up to x^41)
constexpr double sin_(double x) {
    double term = x, sum = x;
    for (int k = 1; k <= 20; ++k) { term *= -x * x / ((2.0 * k) * (2.0 * k + 1.0)); sum += term; }
    return sum;
}
constexpr double cos_(double x) {
    double term = 1.0, sum = 1.0;
    for (int k = 1; k <= 20; ++k) { term *= -x * x / ((2.0 * k - 1.0) * (2.0 * k)); sum += term; }
    return sum;
}
// angle 2 pi m / R reduced to (-pi, pi]
constexpr double angle(int m, int R) {
    int mm = m % R;
    if (2 * mm > R) mm -= R;
    return 2.0 * kPi * (double)mm / (double)R;
}
}  // namespace twc

// W_R^M = exp(2 pi i M / R) as compile-time constants
template <typename T, int R, int M>
struct Tw {
    static constexpr T c = (T)twc::cos_(twc::angle(M, R));
    static constexpr T s = (T)twc::sin_(twc::angle(M, R));
};

// compile-time loop: f(std::integral_constant<int, I>) for I = 0..N-1
template <typename F, int... I>
__device__ __forceinline__ void static_for_(F&& f, std::integer_sequence<int, I...>) {
    (f(std::integral_constant<int, I>{}), ...);
}
template <int N, typename F>
__device__ __forceinline__ void static_for(F&& f) {
    static_for_(f, std::make_integer_sequence<int, N>{});
}

template <typename T, typename C, int R>
__device__ __forceinline__ void small_dft(C* v, int sign);

template <typename T, typename C, int A, int B>
__device__ __forceinline__ void dft_composite(C* v, int sign) {
    constexpr int R = A * B;
    C y[R];
    static_for<B>([&](auto n2c) {
        constexpr int n2 = decltype(n2c)::value;
        C t[A];
#pragma unroll
        for (int n1 = 0; n1 < A; ++n1) t[n1] = v[B * n1 + n2];
        small_dft<T, C, A>(t, sign);
        static_for<A>([&](auto k1c) {
            constexpr int k1 = decltype(k1c)::value;
            constexpr int m = (n2 * k1) % R;
            if constexpr (m == 0) {
                y[n2 * A + k1] = t[k1];
            } else {
                const C w = mk<T>(Tw<T, R, m>::c, sign > 0 ? Tw<T, R, m>::s : -Tw<T, R, m>::s);
                y[n2 * A + k1] = cmul(t[k1], w);
            }
        });
    });
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
        C u[B];
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) u[n2] = y[n2 * A + k1];
        small_dft<T, C, B>(u, sign);
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = u[k2];
    }
}

// Composite radices R = A*B with gcd(A, B) = 1 by the prime-factor
// (Good-Thomas) mapping, which needs no inner twiddles: with input index
// n = (B n1 + A n2) mod R and output index k the solution of k = k1 (mod A),
// k = k2 (mod B),
//   X[k] = DFT_B over n2 of ( DFT_A over n1 of x[(B n1 + A n2) mod R] )[k1]
// (W_R^(nk) = W_A^(n1 k1) W_B^(n2 k2) for these index maps, since the cross
// terms are multiples of R).  All index maps are compile-time constants.
constexpr int crt_index(int k1, int A, int k2, int B) {
    int k = 0;
    while (k % A != k1 || k % B != k2) ++k;
    return k;
}

template <typename T, typename C, int A, int B>
__device__ __forceinline__ void dft_pfa(C* v, int sign) {
    constexpr int R = A * B;
    C y[R];
    static_for<B>([&](auto n2c) {
        constexpr int n2 = decltype(n2c)::value;
        C t[A];
        static_for<A>([&](auto n1c) {
            constexpr int n1 = decltype(n1c)::value;
            t[n1] = v[(B * n1 + A * n2) % R];
        });
        small_dft<T, C, A>(t, sign);
#pragma unroll
        for (int k1 = 0; k1 < A; ++k1) y[n2 * A + k1] = t[k1];
    });
    static_for<A>([&](auto k1c) {
        constexpr int k1 = decltype(k1c)::value;
        C u[B];
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) u[n2] = y[n2 * A + k1];
        small_dft<T, C, B>(u, sign);
        static_for<B>([&](auto k2c) {
            constexpr int k2 = decltype(k2c)::value;
            v[crt_index(k1, A, k2, B)] = u[k2];
        });
    });
}

template <typename T, typename C, int R>
__device__ __forceinline__ void small_dft(C* v, int sign) {
    if constexpr (R == 2) dft2<T>(v);
    else if constexpr (R == 3) dft3<T>(v, sign);
    else if constexpr (R == 4) dft4<T>(v, sign);
    else if constexpr (R == 5) dft5<T>(v, sign);
    else if constexpr (R == 8) dft8<T>(v, sign);
    else if constexpr (R == 6) dft_pfa<T, C, 3, 2>(v, sign);
    else if constexpr (R == 9) dft_composite<T, C, 3, 3>(v, sign);
    else if constexpr (R == 10) dft_pfa<T, C, 5, 2>(v, sign);
    else if constexpr (R == 12) dft_pfa<T, C, 4, 3>(v, sign);
    else if constexpr (R == 15) dft_pfa<T, C, 5, 3>(v, sign);
    else if constexpr (R == 16) dft_composite<T, C, 4, 4>(v, sign);
    else if constexpr (R == 20) dft_pfa<T, C, 5, 4>(v, sign);
    else if constexpr (R == 18) dft_pfa<T, C, 9, 2>(v, sign);
    else if constexpr (R == 24) dft_pfa<T, C, 8, 3>(v, sign);
    else static_assert(R == 2, "unsupported radix");
}

// Twiddle table tw[m] = exp(sign * 2*pi*i * m / n), m in [0, n).
template <typename T>
__device__ __forceinline__ void fill_twiddles(typename cplx_t<T>::type* tw, int n, int sign, int tid, int nthr) {
    for (int m = tid; m < n; m += nthr) {
        // reduce the angle to |2m/n| <= 1 before calling sincospi
        int mm = (2 * m > n) ? m - n : m;
        T s, c;
        if constexpr (sizeof(T) == 4) sincospif((2.0f * (float)mm) / (float)n, &s, &c);
        else sincospi((2.0 * (double)mm) / (double)n, &s, &c);
        tw[m] = mk<T>(c, sign * s);
    }
}

// One Stockham stage over all lines of the tile.  Work items are (butterfly,
// line).  With LINES > 0 (compile time, a power of two) the line index varies
// fastest across threads -- the layout of the strided passes, whose lines have
// unit stride in shared memory; with LINES == 0 the butterfly index varies
// fastest (contiguous lines).  All index arithmetic is shifts or
// multiply-high divisions.
template <typename T, int R, int LINES>
__device__ __forceinline__ void stockham_stage(const typename cplx_t<T>::type* __restrict__ src,
                                               typename cplx_t<T>::type* __restrict__ dst,
                                               const typename cplx_t<T>::type* __restrict__ tw,
                                               int n, const FastDiv& nsd, const FastDiv& nbd, int nlines, int es,
                                               int ls, int sign, int tid, int nthr) {
    using C = typename cplx_t<T>::type;
    const int nb = (int)nbd.d;
    const int Ns = (int)nsd.d;
    const int twstep = nb / Ns;      // n / (Ns * R)
    const int items = nb * (LINES > 0 ? LINES : nlines);
    for (int it = tid; it < items; it += nthr) {
        int j, line;
        if constexpr (LINES > 0) { line = it & (LINES - 1); j = it / LINES; }
        else { line = (int)fdiv((uint32_t)it, nbd); j = it - line * nb; }
        const C* s = src + line * ls;
        C v[R];
        const int jb = (int)fdiv((uint32_t)j, nsd);
        const int k = j - jb * Ns;
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = s[(j + r * nb) * es];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw[r * k * twstep]);  // r*k < R*Ns, so the index is < n
        }
        if constexpr (R == 2) dft2<T>(v);
        else if constexpr (R == 3) dft3<T>(v, sign);
        else if constexpr (R == 4) dft4<T>(v, sign);
        else if constexpr (R == 5) dft5<T>(v, sign);
        else dft8<T>(v, sign);
        C* d = dst + line * ls;
        const int base = jb * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) d[(base + r * Ns) * es] = v[r];
    }
}

// Runs the whole plan.  Data starts in buf0; returns the buffer holding the
// result.  Contains __syncthreads(); all threads of the block must call it.
// LINES > 0: LINES lines with element stride LINES (line stride 1);
// LINES == 0: nlines contiguous lines of length plan.n.
template <typename T, int LINES>
__device__ typename cplx_t<T>::type* fft_tile(typename cplx_t<T>::type* buf0, typename cplx_t<T>::type* buf1,
                                             const typename cplx_t<T>::type* tw, const RadixPlan& plan,
                                             int nlines, int sign) {
    using C = typename cplx_t<T>::type;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int es = LINES > 0 ? LINES : 1;
    const int ls = LINES > 0 ? 1 : plan.n;
    C* src = buf0;
    C* dst = buf1;
    for (int s = 0; s < plan.nstages; ++s) {
        const int R = plan.radix[s];
        switch (R) {
            case 2: stockham_stage<T, 2, LINES>(src, dst, tw, plan.n, plan.ns[s], plan.nb[s], nlines, es, ls, sign, tid, nthr); break;
            case 3: stockham_stage<T, 3, LINES>(src, dst, tw, plan.n, plan.ns[s], plan.nb[s], nlines, es, ls, sign, tid, nthr); break;
            case 4: stockham_stage<T, 4, LINES>(src, dst, tw, plan.n, plan.ns[s], plan.nb[s], nlines, es, ls, sign, tid, nthr); break;
            case 5: stockham_stage<T, 5, LINES>(src, dst, tw, plan.n, plan.ns[s], plan.nb[s], nlines, es, ls, sign, tid, nthr); break;
            default: stockham_stage<T, 8, LINES>(src, dst, tw, plan.n, plan.ns[s], plan.nb[s], nlines, es, ls, sign, tid, nthr); break;
        }
        __syncthreads();
        C* t = src; src = dst; dst = t;
    }
    return src;
}

}  // namespace pyspec

// ---------------------------------------------------------------------------
// Compile-time plans.  For the line lengths the estimator uses most (the
// grid sizes 96..512 and their halves) the radices, strides and loop trip
// counts are template constants, so every index is a constant multiply/shift
// and each stage's loop is fully unrolled.
// ---------------------------------------------------------------------------
namespace pyspec {
namespace ct {

constexpr int kRadices[5] = {8, 4, 5, 3, 2};

// Stage radices for the common lengths (composite radices: fewer passes over
// shared memory); other lengths factor greedily into 8, 4, 5, 3, 2.
struct Plan { int n, len, r[4]; };
constexpr Plan kPlans[] = {
    {360, 3, {12, 5, 6, 0}}, {180, 2, {12, 15, 0, 0}},
    {192, 2, {16, 12, 0, 0}}, {96, 2, {8, 12, 0, 0}},
    {256, 2, {16, 16, 0, 0}}, {128, 2, {16, 8, 0, 0}},
};
constexpr int find_plan(int n) {
    for (int i = 0; i < (int)(sizeof(kPlans) / sizeof(kPlans[0])); ++i)
        if (kPlans[i].n == n) return i;
    return -1;
}

constexpr int nstages(int n) {
    if (find_plan(n) >= 0) return kPlans[find_plan(n)].len;
    int m = n, s = 0;
    for (int k = 0; k < 5; ++k)
        while (m % kRadices[k] == 0) { m /= kRadices[k]; ++s; }
    return m == 1 ? s : -1;
}
constexpr int radix_at(int n, int stage) {
    if (find_plan(n) >= 0) return kPlans[find_plan(n)].r[stage];
    int m = n, s = 0;
    for (int k = 0; k < 5; ++k)
        while (m % kRadices[k] == 0) {
            if (s == stage) return kRadices[k];
            m /= kRadices[k];
            ++s;
        }
    return 0;
}
constexpr int ns_at(int n, int stage) {
    int p = 1;
    for (int s = 0; s < stage; ++s) p *= radix_at(n, s);
    return p;
}

template <typename T, int N, int LINES, int NL, int S>
__device__ __forceinline__ typename cplx_t<T>::type* stages(typename cplx_t<T>::type* __restrict__ src,
                                                           typename cplx_t<T>::type* __restrict__ dst,
                                                           const typename cplx_t<T>::type* __restrict__ tw,
                                                           int sign) {
    using C = typename cplx_t<T>::type;
    if constexpr (S >= nstages(N)) {
        return src;
    } else {
        constexpr int R = radix_at(N, S);
        constexpr int Ns = ns_at(N, S);
        constexpr int nb = N / R;
        constexpr int twstep = nb / Ns;
        constexpr int nlines = LINES > 0 ? LINES : NL;
        constexpr int items = nb * nlines;
        constexpr int es = LINES > 0 ? LINES : 1;
        constexpr int ls = LINES > 0 ? 1 : N;
        for (int it = threadIdx.x; it < items; it += blockDim.x) {
            int j, line;
            if constexpr (LINES > 0) { line = it % LINES; j = it / LINES; }
            else { line = it / nb; j = it - line * nb; }
            const C* s = src + line * ls;
            C v[R];
            const int jb = j / Ns;
            const int k = j - jb * Ns;
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = s[(j + r * nb) * es];
            if constexpr (Ns > 1) {
#pragma unroll
                for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw[r * k * twstep]);
            }
            small_dft<T, C, R>(v, sign);
            C* d = dst + line * ls;
            const int base = jb * Ns * R + k;
#pragma unroll
            for (int r = 0; r < R; ++r) d[(base + r * Ns) * es] = v[r];
        }
        __syncthreads();
        return stages<T, N, LINES, NL, S + 1>(dst, src, tw, sign);
    }
}

// Same contract as fft_tile<T, LINES>, for a line length N and (when
// LINES == 0) a line count NL known at compile time.
template <typename T, int N, int LINES, int NL>
__device__ __forceinline__ typename cplx_t<T>::type* fft_tile_ct(typename cplx_t<T>::type* buf0,
                                                                typename cplx_t<T>::type* buf1,
                                                                const typename cplx_t<T>::type* tw, int sign) {
    static_assert(nstages(N) > 0, "line length must factor into 2, 3 and 5");
    return stages<T, N, LINES, NL, 0>(buf0, buf1, tw, sign);
}

}  // namespace ct
}  // namespace pyspec
