// Register + shared-memory Stockham FFT building blocks for pencil passes.
//
// A pencil of N points is held by T = N/E threads, E points per thread.
// Thread t always holds the points at positions t + T*q (q < E) between
// stages: a stage of radix R runs E/R butterflies j = t + m*T (m < E/R) whose
// inputs j + r*N/R live in registers q = m + r*E/R, so stage inputs never
// need a shuffle.  Stage outputs go to the Stockham (autosort) position
// (j - k)*R + k + r*Ns (k = j mod Ns, Ns = product of earlier radices) and come
// back through shared memory.  After the last stage every output position is
// again t + T*q, so a spectral multiply followed by the inverse transform needs
// no exchange between the two transforms, and a pencil is loaded from and
// stored to global memory in the same t + T*q pattern.
//
// This replaces the cuFFT Z2Z calls of the reference evolution
// (dev/gpe_engine.cu:1050-1053, 1084-1087); the kinetic operator is applied
// axis by axis because exp(c k^2) = exp(c kx^2) exp(c ky^2) exp(c kz^2)
// (the reference tables at dev/gpe_engine.cu:183-216 are already per axis).
#pragma once
#include <cuda_runtime.h>

namespace gpe {

template <typename R> struct cplx_t;
template <> struct cplx_t<double> { using type = double2; };
template <> struct cplx_t<float> { using type = float2; };
template <typename R> using C2 = typename cplx_t<R>::type;

template <typename R> __device__ __forceinline__ C2<R> mk(R x, R y) { C2<R> c; c.x = x; c.y = y; return c; }
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    C c; c.x = a.x * b.x - a.y * b.y; c.y = a.x * b.y + a.y * b.x; return c;
}
template <typename C, typename S> __device__ __forceinline__ C cscale(C a, S s) { a.x = s * a.x; a.y = s * a.y; return a; }
// a * conj(b)
template <typename C> __device__ __forceinline__ C cmulc(C a, C b) {
    C c; c.x = a.x * b.x + a.y * b.y; c.y = a.y * b.x - a.x * b.y; return c;
}

// cos and sin of 2 pi m / 16
__host__ __device__ __forceinline__ constexpr double cos16(int m) {
    constexpr double c1 = 0.92387953251128675613, h = 0.70710678118654752440, c3 = 0.38268343236508977173;
    switch (m & 15) {
        case 0: return 1.0;   case 1: return c1;   case 2: return h;    case 3: return c3;
        case 4: return 0.0;   case 5: return -c3;  case 6: return -h;   case 7: return -c1;
        case 8: return -1.0;  case 9: return -c1;  case 10: return -h;  case 11: return -c3;
        case 12: return 0.0;  case 13: return c3;  case 14: return h;   default: return c1;
    }
}
__host__ __device__ __forceinline__ constexpr double sin16(int m) { return cos16(m - 4); }

// cos and sin of 2 pi m / 32 (the odd multiples of 2 pi / 32 that radix-32 butterflies add)
__host__ __device__ __forceinline__ constexpr double cos32(int m) {
    constexpr double c[9] = {1.0, 0.98078528040323044913, 0.92387953251128675613, 0.83146961230254523708,
                             0.70710678118654752440, 0.55557023301960222474, 0.38268343236508977173,
                             0.19509032201612826785, 0.0};
    m &= 31;
    return m <= 8 ? c[m] : m <= 16 ? -c[16 - m] : m <= 24 ? -c[m - 16] : c[32 - m];
}
__host__ __device__ __forceinline__ constexpr double sin32(int m) { return cos32(m - 8); }

// x * exp(-+ 2 pi i k / M) with compile-time k, M (M | 32); '-' forward, '+' inverse.
// Multiplications by +-1 and +-i cost nothing; the four 45-degree angles cost
// two multiplies.  Angles that are multiples of 2 pi / 16 take exactly the
// same operations whatever M is.
template <typename R, bool INV>
__device__ __forceinline__ C2<R> rot(C2<R> x, int M, int k) {
    const int m32 = (k * (32 / M)) & 31;
    if (m32 & 1) {
        const R cr = (R)cos32(m32), sr = (R)(INV ? sin32(m32) : -sin32(m32));
        return mk<R>(x.x * cr - x.y * sr, x.x * sr + x.y * cr);
    }
    const int m = m32 >> 1;
    const double c = cos16(m);
    const double s = INV ? sin16(m) : -sin16(m);
    if (m == 0) return x;
    if (m == 8) return mk<R>(-x.x, -x.y);
    if (m == 4 || m == 12) return (s > 0) ? mk<R>(-x.y, x.x) : mk<R>(x.y, -x.x);
    if ((m & 3) == 2) {
        const R h = (R)0.70710678118654752440;
        const R a = (c > 0) ? x.x : -x.x, b = (s > 0) ? x.y : -x.y;   // c*x.x, s*x.y up to h
        const R a2 = (s > 0) ? x.x : -x.x, b2 = (c > 0) ? x.y : -x.y;  // s*x.x, c*x.y up to h
        return mk<R>(h * (a - b), h * (a2 + b2));
    }
    const R cr = (R)c, sr = (R)s;
    return mk<R>(x.x * cr - x.y * sr, x.x * sr + x.y * cr);
}

template <int BITS> __host__ __device__ __forceinline__ constexpr int bitrev(int x) {
    int r = 0;
    for (int i = 0; i < BITS; i++) { r = (r << 1) | (x & 1); x >>= 1; }
    return r;
}
__host__ __device__ __forceinline__ constexpr int ilog2c(int x) { return x <= 1 ? 0 : 1 + ilog2c(x / 2); }

// In-register DFT of RAD points (RAD in {2,4,8,16,32}), natural order in and
// out.  Radix-2 decimation in frequency with compile-time twiddles; the final
// bit reversal is a compile-time register renaming.
template <typename R, int RAD, bool INV>
__device__ __forceinline__ void dft(C2<R> (&u)[RAD]) {
#pragma unroll
    for (int span = RAD / 2; span >= 1; span /= 2) {
#pragma unroll
        for (int b = 0; b < RAD; b += 2 * span) {
#pragma unroll
            for (int k = 0; k < span; k++) {
                const C2<R> a = u[b + k], c = u[b + k + span];
                u[b + k] = cadd(a, c);
                u[b + k + span] = rot<R, INV>(csub(a, c), 2 * span, k);
            }
        }
    }
    C2<R> t[RAD];
#pragma unroll
    for (int i = 0; i < RAD; i++) t[i] = u[bitrev<ilog2c(RAD)>(i)];
#pragma unroll
    for (int i = 0; i < RAD; i++) u[i] = t[i];
}

// ---------------------------------------------------------------- plans
// Radix sequence per pencil length; E = points per thread, T = threads per pencil.
// Plan<N, 0> is the default; Plan<N, 1> runs the same pencil with the other
// point count per thread (8 <-> 16), an alternative the autotuner may pick
// for FP32 lattices (pencils of 32 to 512 points).
template <int N> struct Plan0;
template <> struct Plan0<8> { static constexpr int E = 8, L = 1, R0 = 8, R1 = 1, R2 = 1; };
template <> struct Plan0<16> { static constexpr int E = 16, L = 1, R0 = 16, R1 = 1, R2 = 1; };
template <> struct Plan0<32> { static constexpr int E = 8, L = 2, R0 = 8, R1 = 4, R2 = 1; };
template <> struct Plan0<64> { static constexpr int E = 8, L = 2, R0 = 8, R1 = 8, R2 = 1; };
template <> struct Plan0<128> { static constexpr int E = 16, L = 2, R0 = 16, R1 = 8, R2 = 1; };
template <> struct Plan0<256> { static constexpr int E = 16, L = 2, R0 = 16, R1 = 16, R2 = 1; };
template <> struct Plan0<512> { static constexpr int E = 8, L = 3, R0 = 8, R1 = 8, R2 = 8; };

template <int N, int P = 0> struct Plan : Plan0<N> {};
template <> struct Plan<32, 1> { static constexpr int E = 16, L = 2, R0 = 16, R1 = 2, R2 = 1; };
template <> struct Plan<64, 1> { static constexpr int E = 16, L = 2, R0 = 16, R1 = 4, R2 = 1; };
template <> struct Plan<128, 1> { static constexpr int E = 8, L = 3, R0 = 8, R1 = 8, R2 = 2; };
template <> struct Plan<256, 1> { static constexpr int E = 8, L = 3, R0 = 8, R1 = 8, R2 = 4; };
// 512 points at 32 per thread: radix 32 then 16, one exchange per transform instead of two
template <> struct Plan<512, 1> { static constexpr int E = 32, L = 2, R0 = 32, R1 = 16, R2 = 1; };
__host__ __device__ constexpr bool has_plan1(int n) { return n >= 32 && n <= 512; }

template <int N, int P, int S> __host__ __device__ constexpr int plan_rad() {
    return S == 0 ? Plan<N, P>::R0 : S == 1 ? Plan<N, P>::R1 : Plan<N, P>::R2;
}
template <int N, int P, int S> __host__ __device__ constexpr int plan_ns() {
    return S == 0 ? 1 : S == 1 ? Plan<N, P>::R0 : Plan<N, P>::R0 * Plan<N, P>::R1;
}

// Stage-major twiddle table: stage S (Ns > 1) owns RAD*Ns entries at
// tw_off<N, P, S>(), entry r*Ns + k = exp(-2 pi i r k / (Ns RAD)), so the lanes of
// a stage (consecutive k) read consecutive entries.
template <int N, int P, int S> __host__ __device__ constexpr int tw_off() {
    return (S <= 1) ? 0 : plan_rad<N, P, 1>() * plan_ns<N, P, 1>();
}
template <int N, int P> __host__ __device__ constexpr int tw_len() {
    return (Plan<N, P>::L == 1) ? 1
         : (Plan<N, P>::L == 2) ? plan_rad<N, P, 1>() * plan_ns<N, P, 1>()
         : plan_rad<N, P, 1>() * plan_ns<N, P, 1>() + plan_rad<N, P, 2>() * plan_ns<N, P, 2>();
}

// Exchange layout: point p of a pencil sits at padp(p) * SSTR, one padding
// slot per 16 points, so the power-of-two strides of the Stockham stores
// spread over the shared-memory banks.
__host__ __device__ __forceinline__ constexpr int padp(int p) { return p + (p >> 4); }
template <int N> __host__ __device__ constexpr int padded_len() { return N + N / 16 + (N < 16 ? 1 : 0); }

// Barrier over the G threads that exchange one group of pencils: a warp
// barrier when the group lies inside one warp, else the CTA barrier (every
// group of a CTA runs the same stage sequence, so they meet at the same
// barriers; a CTA barrier keeps the per-CTA barrier count at one).
template <int G> __device__ __forceinline__ void group_sync(int bar) {
    (void)bar;
    if constexpr (G <= 32) {
        __syncwarp();
    } else {
        __syncthreads();
    }
}

// One Stockham stage, computed in place in registers.  `sb` addresses this
// thread's pencil in shared memory (point p at sb[padp(p) * SSTR]); `tw` is
// the stage-major twiddle table (tw_off / tw_len).  The last stage keeps its
// result in registers; the others exchange through `sb`.
template <typename R, int N, int P, int S, bool INV, int SSTR, int G>
__device__ __forceinline__ void stage(C2<R> (&v)[Plan<N, P>::E], C2<R>* sb, int t, const C2<R>* tw, int bar) {
    constexpr int E = Plan<N, P>::E, T = N / E, L = Plan<N, P>::L;
    constexpr int RAD = plan_rad<N, P, S>();
    constexpr int NS = plan_ns<N, P, S>();
    constexpr int MB = E / RAD;
    constexpr bool LAST = (S == L - 1);
    if constexpr (!LAST) group_sync<G>(bar);  // earlier readers of sb are done
#pragma unroll
    for (int m = 0; m < MB; m++) {
        const int j = t + m * T;
        const int k = j & (NS - 1);
        C2<R> u[RAD];
#pragma unroll
        for (int r = 0; r < RAD; r++) u[r] = v[m + r * MB];
        if constexpr (NS > 1) {
#pragma unroll
            for (int r = 1; r < RAD; r++) {
                C2<R> w = tw[tw_off<N, P, S>() + r * NS + k];
                if constexpr (INV) w.y = -w.y;
                u[r] = cmul(u[r], w);
            }
        }
        dft<R, RAD, INV>(u);
        if constexpr (LAST) {
#pragma unroll
            for (int r = 0; r < RAD; r++) v[m + r * MB] = u[r];
        } else {
            const int base = (j - k) * RAD + k;
#pragma unroll
            for (int r = 0; r < RAD; r++) sb[padp(base + r * NS) * SSTR] = u[r];
        }
    }
    if constexpr (!LAST) {
        group_sync<G>(bar);
#pragma unroll
        for (int q = 0; q < E; q++) v[q] = sb[padp(t + T * q) * SSTR];
    }
}

// Unnormalised transform, forward (exp(-2 pi i jk/N)) or inverse (exp(+...)).
template <typename R, int N, int P, bool INV, int SSTR, int G>
__device__ __forceinline__ void fft(C2<R> (&v)[Plan<N, P>::E], C2<R>* sb, int t, const C2<R>* tw, int bar) {
    stage<R, N, P, 0, INV, SSTR, G>(v, sb, t, tw, bar);
    if constexpr (Plan<N, P>::L > 1) stage<R, N, P, 1, INV, SSTR, G>(v, sb, t, tw, bar);
    if constexpr (Plan<N, P>::L > 2) stage<R, N, P, 2, INV, SSTR, G>(v, sb, t, tw, bar);
}

}  // namespace gpe
