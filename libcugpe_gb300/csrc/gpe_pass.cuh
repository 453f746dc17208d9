// Fused pencil pass: the one kernel shape of the split-step evolution.
//
// A launch walks every pencil of one axis of the lattice.  For each point it
// runs, in order,
//   load -> PRE op -> [LAP pair: FFT, x k_a^2 table, inverse FFT -> MID op]
//        -> [KIN pair: FFT, x exp(c k_a^2)/N_a table, inverse FFT] -> POST op
//        -> store (+ partial sums, finalised by the last CTA).
// The PRE/MID/POST ops are the reference's pointwise kernels
// (dev/gpe_engine.cu:716-918), fused into the pass that already holds the
// point in registers; a host-side schedule (gpe_engine.cu) strings the passes
// into the reference's step sequence (dev/gpe_engine.cu:1030-1109).
//
// Thread mapping: pencil length N, E points per thread, T = N/E threads per
// pencil, W pencils per CTA.  z pencils (contiguous) put t fastest, so thread
// t reads point t + T*q of its pencil and a pencil is one coalesced run;
// y and x pencils put the pencil index fastest, so a warp reads W adjacent
// columns of the same row.  Shared memory holds the Stockham exchanges.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "gpe_fft.cuh"
#include "gpe_hooks.cuh"
#include "gpe_physics.cuh"

namespace gpe {

enum : int { AX_X = 0, AX_Y = 1, AX_Z = 2 };

enum : int {  // PRE ops
    PRE_NONE = 0,
    PRE_VSTEP1 = 1,   // V = Vext(it) + dEDF(rho); x = x exp(c3 V)        (:719-742)
    PRE_PART2 = 2,    // corrector start from stored psi2                (:813-864)
    PRE_ENERGY = 3,   // eext, eint partial sums                        (:1631-1643)
};
enum : int {  // MID ops (after the Laplacian pair)
    MID_NONE = 0,
    MID_LAP_STORE = 1,  // lap = D_a psi
    MID_LAP_ACC = 2,    // lap += D_a psi
    MID_QF_VSTEP1 = 3,  // V_qf from lap + D_a psi, then Vstep1_qf         (:744-768, 907-918)
    MID_CURRENT = 4,    // V = Re(conj(psi) D_a psi), D_a = k_a/(Gamma N_a)  (:1817-1904)
};
enum : int {  // POST ops
    POST_NONE = 0,
    POST_VSTEP2 = 1,   // RTE corrector, writes psi                     (:770-797)
    POST_PART1 = 2,    // psi2 *= exp(c3 V) (+ norm partials)           (:799-811)
    POST_PART12 = 3,   // part1 + part2(_qf) without normalisation      (:799-864)
    POST_VSTEP3 = 4,   // psi *= exp(c3 V') (+ norm partials)           (:866-874)
};
enum : uint32_t {  // flags
    F_LAP = 1u << 0,        // run the Laplacian pair
    F_KIN = 1u << 1,        // run the kinetic pair
    F_SCALE_IN = 1u << 2,   // multiply loaded psi by the pending norm factor
    F_REDUCE = 1u << 3,     // norm partials of the stored value
    F_STORE = 1u << 4,      // store the result to `out`
    F_QF = 1u << 5,         // V_qf enters the corrector average
    F_AUX_CPLX = 1u << 6,   // corrector factor stored as complex exp(c3 V'), else real V'
    F_SCALE_PSI2 = 1u << 7, // psi2 read by PRE_PART2 is scaled by s2 (ITE)
    F_FIN_S2 = 1u << 8,     // last CTA: s2 = sqrt(npart / sum)
    F_FIN_STEP = 1u << 9,   // last CTA: s_prev, norm, mu from the sum (ITE); it += 1
    F_EKIN = 1u << 10,      // forward transform only, accumulate sum w_k |X_k|^2
    F_FIN_RED = 1u << 11,   // last CTA: store the NRED sums in dyn->red[red_slot..]
    F_VEXTRA = 1u << 12,    // time-sliced additive potential table
    F_LAP_OUT = 1u << 13,   // after the store: lap = D_a(result) (Laplacian of the new psi)
    F_WZ = 1u << 14,        // Weizsaecker gradient sums of this axis (wg, ws) from D1_a psi
    F_DIP = 1u << 15,       // dipolar convolution pass (mid = DIP_* mode)
    F_SCALE_OPD = 1u << 16, // dipolar step: the staged psi is scaled by the pending norm factor
    F_DIRECT = 1u << 17,    // psi, V, V_qf, lap and the psi copy are read where used, not staged
    F_PH_STORE = 1u << 18,  // Vstep1 also stores its phase factor exp(c3 V) in the (complex) aux buffer
    F_PH_LOAD = 1u << 19,   // the corrector takes exp(c3 V) from aux instead of recomputing it
};
enum : int {  // dipolar pass modes (in `mid` with F_DIP)
    DIP_DENS_FWD = 1,  // x = (Gamma |psi|^2, 0), forward FFT_a -> out      (dev/gpe_engine.cu:618-626)
    DIP_FWD = 2,       // forward FFT_a -> out
    DIP_VDD = 3,       // forward FFT_a, x gpe_Vpp_k(k)/nxyz, inverse FFT_a (dev/gpe_engine.cu:958-974)
    DIP_INV = 4,       // inverse FFT_a -> out
    DIP_STEP = 5,      // inverse FFT_a -> vdip; psi exp(c3 (Vext + dEDF + vdip)) [+ K_a]  (:979-1006)
    DIP_EN = 6,        // inverse FFT_a -> vdip; partial sums of rho vdip / 2     (:1774-1809)
};

// Scalars that change while a step runs; they live in device memory so one
// captured step can be replayed.
struct DynState {
    double s_prev;     // pending normalisation factor of psi
    double s2;         // normalisation factor of psi2 inside an ITE step
    double norm;       // last sum of Gamma |psi|^2
    double mu;         // -0.5 log(norm / npart) / dt  (dev/gpe_engine.cu:1101)
    double dmu;        // change of mu over the last step
    double mu_sum;     // running sum of mu over ITE steps (interval means for convergence tests)
    double red[16];    // results of generic reductions
    // device-side convergence test of a batched imaginary-time solve (gpe_gb_batch_solve): every
    // conv_check steps the mean of mu over the interval is compared with the previous interval's
    double conv_tol;   // retire when the interval means differ by less than conv_tol per step
    double conv_start; // mu_sum at the start of the current interval
    double conv_prev;  // mean of mu over the previous interval
    double conv_mu;    // interval mean at retirement
    unsigned int it;   // step counter since set_psi / set_time
    unsigned int ticket;
    unsigned int err;
    unsigned int pad;
    unsigned int conv_check;  // steps per interval (0: no test)
    unsigned int conv_n;      // steps into the current interval
    unsigned int conv_have;   // a previous interval mean exists
    unsigned int retired;     // converged: every pass of a batch skips this condensate
    unsigned int conv_step;   // step counter `it` after the step that converged
    unsigned int pad2[3];
};

constexpr int NRED = 3;

template <typename R>
struct PassArgs {
    const C2<R>* in;
    C2<R>* out;
    C2<R>* psi;          // psi, read/written by corrector ops
    const C2<R>* psi2;   // psi2 read by PRE_PART2
    C2<R>* lap;          // Laplacian accumulator (QF)
    void* aux;           // corrector factor: C2<R> (F_AUX_CPLX) or R
    R* V;                // predictor potential
    R* Vqf;              // frozen gradient potential: quantum friction (+ Weizsaecker)
    R* wg;               // Weizsaecker: sum over axes done so far of (d_a rho)^2
    R* ws;               // Weizsaecker: sum over axes done so far of |D1_a psi|^2
    const R* ld1;        // k_a / N_a of this axis (first derivative)
    const R* kgx; const R* kgy; const R* kgz;  // k grids of the three axes (dipolar kernel)
    const R* vx; const R* vy; const R* vz;   // trap tables
    const R* vextra;     // [slices][n] additive potential (F_VEXTRA); [2][n] ring when vring
    int vsteps, vslices;
    int vring;           // vextra holds two slices: slice s in slot s & 1 (the control problem)
    const C2<R>* ktab;   // kinetic factors of this axis, incl. 1/N_a
    const R* ltab;       // Laplacian / kinetic-energy weights of this axis
    const C2<R>* tw;     // stage twiddles of this axis's radix plan
    int plan;            // radix plan of this axis (Plan<N, plan>), matching tw
    DynState* dyn;
    double* partials;    // [gridDim.x][NRED]
    int lx, ly, lz;      // log2 of the lattice sides
    double npart, dt;
    int red_slot;
    const double* uparam; // user parameters (device copy; read by user hooks)
    double t0;            // initial time (user hooks)
    uint32_t npencils;   // pencils along this pass's axis
    uint32_t flags;
    int pre, mid, post;
    Phys<R> ph;
};

// The time-sliced additive potential at point idx, step `it` (F_VEXTRA), else 0.
template <typename R> __device__ __forceinline__ R vextra_at(const PassArgs<R>& a, uint32_t idx, unsigned it) {
    int s = (int)(it / (unsigned)a.vsteps);
    if (s >= a.vslices) s = a.vslices - 1;
    if (a.vring) s &= 1;
    return a.vextra[((size_t)s << (a.lx + a.ly + a.lz)) | idx];
}

// External potential at step `it`: the built-in harmonic trap (per-axis tables), or the user hook
// gpe_external_potential in a hook build; plus the time-sliced additive table when set.
template <typename R> __device__ __forceinline__ R vext_at(const PassArgs<R>& a, uint32_t idx, int ix, int iy, int iz,
                                                          unsigned it) {
#ifdef GPE_USER_HOOKS
    R v = (R)gpe_external_potential((uint)ix, (uint)iy, (uint)iz, (uint)it);
#else
    R v = (__ldg(a.vx + ix) + __ldg(a.vy + iy)) + __ldg(a.vz + iz);
#endif
    if (a.flags & F_VEXTRA) v += vextra_at(a, idx, it);
    return v;
}

// The same potential along one pencil (AX_X, AX_Y, AX_Z) or one plane row (AX = 3: ix and iy fixed):
// the two trap terms that are constant there are read once per thread, so a point reads one table
// entry; the sum keeps the order (vx + vy) + vz, so the values are those of vext_at.  FP32 only
// (measured at 128^3: 93.1 -> 91.9 us per step; the FP64 corrector pass ran 4 % slower with it).
template <typename R, int AX> struct PencilTrap {
    static constexpr bool ROWS = (sizeof(R) == 4);
    R c0 = (R)0, c1 = (R)0;
    // (ix, iy, iz): a point of the pencil (any point: only its constant coordinates are used); called
    // only for pencils inside the lattice
    __device__ __forceinline__ void init(const PassArgs<R>& a, int ix, int iy, int iz) {
#ifndef GPE_USER_HOOKS
        if constexpr (!ROWS) { (void)a; (void)ix; (void)iy; (void)iz; }
        else if constexpr (AX == 0) { c0 = __ldg(a.vy + iy); c1 = __ldg(a.vz + iz); }
        else if constexpr (AX == 1) { c0 = __ldg(a.vx + ix); c1 = __ldg(a.vz + iz); }
        else { c0 = __ldg(a.vx + ix) + __ldg(a.vy + iy); }
#else
        (void)a; (void)ix; (void)iy; (void)iz;
#endif
    }
    __device__ __forceinline__ R at(const PassArgs<R>& a, uint32_t idx, int ix, int iy, int iz, unsigned it) const {
#ifdef GPE_USER_HOOKS
        return vext_at(a, idx, ix, iy, iz, it);
#else
        if constexpr (!ROWS) return vext_at(a, idx, ix, iy, iz, it);
        R v;
        if constexpr (AX == 0) v = (__ldg(a.vx + ix) + c0) + c1;
        else if constexpr (AX == 1) v = (c0 + __ldg(a.vy + iy)) + c1;
        else v = c0 + __ldg(a.vz + iz);
        if (a.flags & F_VEXTRA) v += vextra_at(a, idx, it);
        return v;
#endif
    }
};

// Mean field dE/drho at step `it`: built-in functional, or the user hook gpe_dEDFdn.
template <typename R> __device__ __forceinline__ R mean_field(const PassArgs<R>& a, R rho, unsigned it) {
#ifdef GPE_USER_HOOKS
    (void)a;
    return (R)gpe_dEDFdn((double)rho, (uint)it);
#else
    (void)it;
    return dEDFdn(a.ph, rho);
#endif
}

// psi_n as a step reads it: unchanged, or passed through the user hook gpe_modify_psi.
template <typename R> __device__ __forceinline__ C2<R> modify_at(int ix, int iy, int iz, unsigned it, C2<R> v) {
#ifdef GPE_USER_HOOKS
    const cuDoubleComplex p = gpe_modify_psi((uint)ix, (uint)iy, (uint)iz, (uint)it,
                                             make_cuDoubleComplex((double)v.x, (double)v.y));
    return mk<R>((R)cuCreal(p), (R)cuCimag(p));
#else
    (void)ix; (void)iy; (void)iz; (void)it;
    return v;
#endif
}

template <typename C> __device__ __forceinline__ C ldc(const C* p) { return *p; }

// gpe_Vpp_k / nxyz (dev/gpe_user_defined.h:422-438, dev/gpe_engine.cu:972): Fourier transform of the
// contact + dipole-dipole pseudopotential, dipoles along z, with the inverse FFT normalisation
template <typename R> __device__ __forceinline__ R vdd_k(const PassArgs<R>& a, int ix, int iy, int iz) {
    const R kx = __ldg(a.kgx + ix), ky = __ldg(a.kgy + iy), kz = __ldg(a.kgz + iz);
    const R k2 = kx * kx + ky * ky + kz * kz;
    const R fpi = (R)(4.0 * M_PI);
    R v;
    if (k2 < (R)2.220446049250313e-16) v = fpi * a.ph.a_scat * (R)1;  // DBL_EPSILON
    else v = fpi * (a.ph.a_scat * (R)1 + a.ph.a_dip * ((R)3 * kz * kz / k2 - (R)1));
    return v / a.ph.nxyz;
}

// Deterministic block sum of the first NR of NRED doubles; result valid in thread 0.
template <int NT, int NR>
__device__ __forceinline__ void block_sum(double (&v)[NRED], double (*sred)[NRED]) {
#pragma unroll
    for (int r = 0; r < NR; r++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[r] += __shfl_down_sync(0xffffffffu, v[r], o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int r = 0; r < NR; r++) sred[w][r] = v[r];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int r = 0; r < NR; r++) {
            double s = 0.0;
            for (int i = 0; i < (NT + 31) / 32; i++) s += sred[i][r];
            v[r] = s;
        }
    }
}

// Float-float (unevaluated hi + lo) sums for the FP32 form's norm partials.
// FP64 arithmetic runs at a small fraction of the FP32 rate on this part, so
// per-point FP64 accumulation would cost more than the transforms; a
// float-float sum (Knuth's two-sum, Dekker's renormalisation) keeps ~44 bits
// on the FP32 pipes.  Result as a double in thread 0.
struct FF { float h, l; };
__device__ __forceinline__ FF ff_add(FF a, float b) {
    const float s = a.h + b, bb = s - a.h;
    const float e = (a.h - (s - bb)) + (b - bb) + a.l;
    FF r; r.h = s + e; r.l = e - (r.h - s); return r;
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const float s = a.h + b.h, bb = s - a.h;
    const float e = (a.h - (s - bb)) + (b.h - bb) + (a.l + b.l);
    FF r; r.h = s + e; r.l = e - (r.h - s); return r;
}
template <int NT>
__device__ __forceinline__ double block_sum_ff(FF v, double (*sred)[NRED]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        FF u;
        u.h = __shfl_down_sync(0xffffffffu, v.h, o);
        u.l = __shfl_down_sync(0xffffffffu, v.l, o);
        v = ff_add(v, u);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sred[w][0] = (double)v.h + (double)v.l;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (NT + 31) / 32; i++) s += sred[i][0];
    return s;
}

// Last CTA of the grid: sums the first NR per-CTA partials (when `sums`) in a
// fixed order and publishes the results.
template <typename R, int NT, int NR>
__device__ void finalize(const PassArgs<R>& a, double (*sred)[NRED], uint32_t nblk, bool sums) {
    double s[NRED] = {0.0, 0.0, 0.0};
    if (sums) {
        // each thread sums its partials (a fixed stride) with Neumaier's compensation, then the
        // block adds the compensated per-thread sums in a fixed order
        double c[NRED] = {0.0, 0.0, 0.0};
        for (int b = threadIdx.x; b < (int)nblk; b += NT) {
#pragma unroll
            for (int r = 0; r < NR; r++) {
                const double x = __ldcg(a.partials + (size_t)b * NRED + r);
                const double t = s[r] + x;
                c[r] += (fabs(s[r]) >= fabs(x)) ? (s[r] - t) + x : (x - t) + s[r];
                s[r] = t;
            }
        }
#pragma unroll
        for (int r = 0; r < NR; r++) s[r] += c[r];
        block_sum<NT, NR>(s, sred);
    }
    if (threadIdx.x == 0) {
        DynState* d = a.dyn;
        if (a.flags & F_FIN_S2) d->s2 = sqrt(a.npart / s[0]);
        if (a.flags & F_FIN_STEP) {
            if (a.flags & F_REDUCE) {
                d->norm = s[0];
                d->s_prev = sqrt(a.npart / s[0]);
                const double mu = -.5 * log(s[0] / a.npart) / a.dt;
                d->dmu = mu - d->mu;
                d->mu = mu;
                d->mu_sum += mu;
                if (d->conv_check && ++d->conv_n == d->conv_check) {
                    const double mean = (d->mu_sum - d->conv_start) / (double)d->conv_check;
                    if (d->conv_have && fabs(mean - d->conv_prev) < d->conv_tol * (double)d->conv_check) {
                        d->retired = 1;
                        d->conv_step = d->it + 1;
                        d->conv_mu = mean;
                    }
                    d->conv_prev = mean;
                    d->conv_have = 1;
                    d->conv_start = d->mu_sum;
                    d->conv_n = 0;
                }
            }
            d->it = d->it + 1;
        }
        if (a.flags & F_FIN_RED)
#pragma unroll
            for (int r = 0; r < NRED; r++) d->red[a.red_slot + r] = s[r];
        d->ticket = 0;
        __threadfence();
    }
}

// Operands that the MID/POST ops read after the transforms.  They are
// prefetched into shared memory with cp.async when the CTA starts, so their
// latency overlaps the transforms instead of stalling the epilogue.
enum : uint32_t {
    OP_PSI = 1u << 0,   // C2 psi            (corrector)
    OP_LAP = 1u << 1,   // C2 lap            (Laplacian accumulate / V_qf)
    OP_AUXC = 1u << 2,  // C2 exp(c3 V')     (Vstep3, FP64)
    OP_COPY = 1u << 3,  // C2 loaded value   (kept for V_qf, from registers)
    OP_V = 1u << 4,     // R  V              (corrector)
    OP_AUXR = 1u << 5,  // R  V'             (Vstep3, FP32)
    OP_VQF = 1u << 6,   // R  V_qf           (corrector with friction)
    OP_WG = 1u << 7,    // R  wg             (Weizsaecker sums, slot C)
    OP_WS = 1u << 8,    // R  ws             (Weizsaecker sums, slot D)
};

__host__ __device__ inline uint32_t staged_ops(int mid, int post, uint32_t flags) {
    uint32_t m = 0;
    if (flags & F_DIP) return (mid == DIP_STEP || mid == DIP_EN) ? OP_PSI : 0u;
    if (mid == MID_LAP_ACC) m |= OP_LAP;
    if (mid == MID_QF_VSTEP1) m |= OP_LAP | OP_COPY;
    if (mid == MID_CURRENT) m |= OP_COPY;
    if (flags & F_WZ) {
        m |= OP_COPY;
        if (mid == MID_LAP_ACC || mid == MID_QF_VSTEP1) m |= OP_WG | OP_WS;
    }
    if (post == POST_VSTEP2 || post == POST_PART12) m |= OP_PSI | OP_V;
    if (post == POST_PART12 && (flags & F_QF)) m |= OP_VQF;
    if (post == POST_PART1) m |= OP_V;
    if (post == POST_VSTEP3) m |= (flags & F_AUX_CPLX) ? OP_AUXC : OP_AUXR;
    if (flags & F_DIRECT) m &= ~(OP_PSI | OP_V | OP_VQF | OP_LAP | OP_COPY | OP_AUXC);
    return m;
}

// Slots: A (C2) = psi | lap | aux-complex, B (C2) = copy, C (R) = V | aux-real,
// D (R) = V_qf; each E*NT elements, element (q, thread) at q*NT + thread.
template <typename R>
__host__ __device__ inline size_t slot_bytes(uint32_t m, int per_cta) {
    size_t b = 0;
    if (m & (OP_PSI | OP_LAP | OP_AUXC)) b += (size_t)per_cta * sizeof(C2<R>);
    if (m & OP_COPY) b += (size_t)per_cta * sizeof(C2<R>);
    if (m & (OP_V | OP_AUXR | OP_WG)) b += (size_t)per_cta * sizeof(R);
    if (m & (OP_VQF | OP_WS)) b += (size_t)per_cta * sizeof(R);
    return b;
}

__device__ __forceinline__ void cp_async(void* dst, const void* src, int bytes) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    if (bytes == 16) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(src) : "memory");
    else if (bytes == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Columns per group of y/x pencils.  The rows of one x pencil are a whole
// plane apart and the rows of a y pencil a whole line apart, so each row a
// group touches should be a long contiguous run: 128 bytes for x and 64 for y
// in the FP32 form (a copy with 32-byte rows reaches less than half the HBM
// bandwidth of one with 128-byte rows on x pencils at 256^3 and 512^3).  The
// FP64 form (FP64-ALU-bound) keeps 32-byte rows.  A group never exceeds the
// CTA, so a fixed 128-thread CTA (the batched pass) narrows it.
template <typename R, int N, int AX> __host__ __device__ constexpr int cw_target() {
    return (sizeof(C2<R>) == 16) ? 2 : (AX == AX_X) ? 16 : 8;
}
template <typename R, int N, int AX, int NT, int P = 0> __host__ __device__ constexpr int pass_cw() {
    constexpr int T = N / Plan<N, P>::E;
    constexpr int want = ((32 / T) > cw_target<R, N, AX>()) ? (32 / T) : cw_target<R, N, AX>();
    return (T * want <= NT) ? want : ((NT / T) > 0 ? NT / T : 1);
}

// Geometry of one pass kernel instantiation.
//  z pencils: t fastest (coalesced rows); a warp holds 32/T whole pencils, or
//  one pencil spans T/32 warps (T > 32, 512 points).
//  y/x pencils: a group of G = T*CW threads holds CW adjacent columns, column
//  fastest, so a warp-wide access covers 32/T rows of CW contiguous points.
template <typename R, int N, int AX, int NT, int P = 0>
struct PassGeom {
    static constexpr int E = Plan<N, P>::E;
    static constexpr int T = N / E;
    static constexpr int CW = (AX == AX_Z) ? ((32 / T) > 0 ? 32 / T : 1) : pass_cw<R, N, AX, NT, P>();
    static constexpr int G = (AX == AX_Z) ? (T > 32 ? T : 32) : T * CW;
    static constexpr int W = NT / T;  // pencils per CTA
    static constexpr int ROW = padded_len<N>();
    static constexpr int TW = tw_len<N, P>();
    static constexpr size_t TAB_BYTES = (((size_t)(TW + N) * sizeof(C2<R>) + N * sizeof(R)) + 15) & ~(size_t)15;
    static constexpr size_t EXCH_BYTES = (size_t)W * ROW * sizeof(C2<R>);
    static constexpr size_t SMEM_BASE = TAB_BYTES + EXCH_BYTES;
    // the largest staged-operand set: lap + copy + the two Weizsaecker sums (two complex and two
    // real values per point); a launch that would need more than a CTA can hold is refused
    static constexpr size_t SMEM_FULL = SMEM_BASE + 2 * (size_t)E * NT * (sizeof(C2<R>) + sizeof(R));
    // dynamic shared memory cap: the 227 KiB per-CTA opt-in limit less room for the static arrays
    static constexpr size_t SMEM_CAP = 225 * 1024;
    static constexpr size_t SMEM_MAX = SMEM_FULL < SMEM_CAP ? SMEM_FULL : SMEM_CAP;
    // resident threads per SM the register allocation aims for: FP32 pencils up to 128 points fit
    // 7 CTAs of 128 threads in 72 registers without spills, 256-point ones 6 in 80, which runs the
    // 128^3 and 256^3 passes (1-2 waves of CTAs) in fewer rounds (measured: +8% RTE, +20% ITE
    // steps/s at 128^3, +2% / +16% at 256^3); pencils of 128 to 512 points at 8 points per thread
    // fit 1024 threads in 64 registers without spills (512 points: +16% steps/s at 512^3 against 16
    // points per thread in 512 threads)
    static constexpr int THREADS_SM = (sizeof(R) == 4)
        ? (E == 8 ? (N <= 64 ? 896 : 1024) : (N <= 128 ? 896 : N <= 256 ? 768 : 512)) : 256;
    static constexpr int MINB = (THREADS_SM / NT) > 0 ? THREADS_SM / NT : 1;
    static_assert(NT % G == 0 && NT % 32 == 0, "threads per CTA must hold whole groups");
    static_assert(SMEM_BASE + 2 * (size_t)E * NT * sizeof(C2<R>) <= SMEM_CAP,
                  "shared memory of a pass without the Weizsaecker sums exceeds the per-CTA limit");
};

// Kernel classes: each instantiation compiles only the code its passes use,
// which keeps register use and instruction footprint down.
enum : int { C_KIN = 0, C_EPI = 1, C_LAP = 2, C_EN = 3, C_DIP = 4, C_EPI_D = 5, C_LAP_D = 6, C_KINP = 7 };
// C_KINP: persistent kinetic pass (kin_pipe_body) chosen by the launcher for long FP32 pencils.
// C_EPI_D / C_LAP_D: the epilogue and Laplacian classes reading their operands where used (F_DIRECT),
// compiled separately so the staged variants keep their register allocation.

__host__ __device__ inline int op_class(int pre, int mid, int post, uint32_t flags) {
    (void)mid;
    if (flags & F_DIP) return C_DIP;
    if (flags & F_EKIN) return C_EN;
    if (flags & F_LAP) return (flags & F_DIRECT) ? C_LAP_D : C_LAP;
    if (pre != PRE_NONE || post != POST_NONE ||
        (flags & (F_LAP_OUT | F_REDUCE | F_FIN_STEP | F_FIN_S2 | F_FIN_RED)))
        return (flags & F_DIRECT) ? C_EPI_D : C_EPI;
    return C_KIN;
}

// The pass over the pencils of one lattice, as CTA `blk` of `nblk` CTAs
// working on it (a standalone launch, or one condensate of a batch).
template <typename R, int N, int AX, int NT, int CLS, int P = 0>
__device__ __forceinline__ void pass_body(const PassArgs<R>& a, uint32_t blk, uint32_t nblk) {
    constexpr bool DIRECT = (CLS == C_EPI_D || CLS == C_LAP_D);
    constexpr int K = (CLS == C_EPI_D) ? C_EPI : (CLS == C_LAP_D) ? C_LAP : CLS;  // base class
    using Geo = PassGeom<R, N, AX, NT, P>;
    constexpr int E = Geo::E, T = Geo::T, CW = Geo::CW, G = Geo::G, W = Geo::W, ROW = Geo::ROW;
    constexpr int SSTR = (AX == AX_Z) ? 1 : CW;
    constexpr bool FIN = (K == C_EPI || K == C_EN || K == C_DIP);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* stw = reinterpret_cast<C2<R>*>(smem_raw);
    C2<R>* skt = stw + Geo::TW;
    R* slt = reinterpret_cast<R*>(skt + N);
    C2<R>* sx = reinterpret_cast<C2<R>*>(smem_raw + Geo::TAB_BYTES);
    __shared__ double sred[FIN ? NT / 32 : 1][NRED];
    __shared__ bool last_cta;

    // Programmatic dependent launch: the FP32 pass kernels are launched so that their CTAs may start
    // while the previous pass drains.  The constant tables (written before any pass of the stream
    // ran) are staged first, overlapping that drain; every read of what earlier passes wrote (psi,
    // operands, the device state) comes after the wait for the previous pass to complete (a no-op
    // for a launch without the attribute).  Dependents may be launched as soon as every CTA of this
    // pass is running.
    const int tid = threadIdx.x;
    for (int i = tid; i < Geo::TW; i += NT) stw[i] = a.tw[i];
    if constexpr (K != C_EN) {
        for (int i = tid; i < N; i += NT) skt[i] = a.ktab[i];
    }
    if constexpr (K != C_KIN) {
        for (int i = tid; i < N; i += NT) slt[i] = a.ltab[i];
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    // a condensate that a batched solve has retired (converged) is left as it is
    if (a.dyn->retired) return;

    int pl, t, bar;
    C2<R>* sb;
    if constexpr (AX == AX_Z) {
        t = tid % T;
        pl = tid / T;
        sb = sx + pl * ROW;
        bar = 0;
    } else {
        const int gi = tid / G, loc = tid % G;
        const int c = loc % CW;
        t = loc / CW;
        pl = gi * CW + c;
        sb = sx + gi * (ROW * CW) + c;
        bar = 1 + gi;
    }

    // 32-bit point indices: the largest lattice (512^3) has 2^27 points.
    // CTAs past the last pencil (small lattices) compute on zeros and store nothing.
    const uint32_t gp = blk * (uint32_t)W + pl;  // pencil id
    const bool valid = gp < a.npencils;
    const int ly = a.ly, lz = a.lz;
    uint32_t base, lstr;  // first point of the pencil, log2 of the point stride
    if constexpr (AX == AX_Z) { base = gp << lz; lstr = 0; }
    else if constexpr (AX == AX_Y) {
        const uint32_t ix = gp >> lz, iz = gp & ((1u << lz) - 1);
        base = ((ix << ly) << lz) + iz; lstr = lz;
    } else { base = gp; lstr = ly + lz; }
    const uint32_t tbase = base + ((uint32_t)t << lstr);
    auto at = [&](int q) -> uint32_t { return tbase + ((uint32_t)(T * q) << lstr); };
    auto decode = [&](uint32_t idx, int& ix, int& iy, int& iz) {
        ix = (int)(idx >> (ly + lz));
        iy = (int)((idx >> lz) & ((1u << ly) - 1));
        iz = (int)(idx & ((1u << lz) - 1));
    };

    const DynState* dyn = a.dyn;
    const unsigned it = dyn->it;
    const R s_prev = (R)dyn->s_prev;
    const bool scale_in = (a.flags & F_SCALE_IN) != 0;
    PencilTrap<R, AX> trap;  // the trap terms constant along this pencil
    if (valid) {
        int ix0, iy0, iz0;
        decode(at(0), ix0, iy0, iz0);
        trap.init(a, ix0, iy0, iz0);
    }

    C2<R> x[E];
#pragma unroll
    for (int q = 0; q < E; q++) x[q] = valid ? ldc(a.in + at(q)) : mk<R>((R)0, (R)0);

    // staged operand slots (see staged_ops)
    uint32_t ops = 0;
    C2<R>* slotA = nullptr;
    C2<R>* slotB = nullptr;
    R* slotC = nullptr;
    R* slotD = nullptr;
    if constexpr (K == C_EPI || K == C_LAP || K == C_DIP) {
        ops = staged_ops(a.mid, a.post, a.flags);
        unsigned char* sop = smem_raw + Geo::SMEM_BASE;
        slotA = reinterpret_cast<C2<R>*>(sop);
        if (ops & (OP_PSI | OP_LAP | OP_AUXC)) sop += (size_t)E * NT * sizeof(C2<R>);
        slotB = reinterpret_cast<C2<R>*>(sop);
        if (ops & OP_COPY) sop += (size_t)E * NT * sizeof(C2<R>);
        slotC = reinterpret_cast<R*>(sop);
        if (ops & (OP_V | OP_AUXR | OP_WG)) sop += (size_t)E * NT * sizeof(R);
        slotD = reinterpret_cast<R*>(sop);
        if (ops && valid) {
            const void* srcA = (ops & OP_PSI) ? (const void*)a.psi : (ops & OP_LAP) ? (const void*)a.lap : a.aux;
            const void* srcC = (ops & OP_V) ? (const void*)a.V : (ops & OP_WG) ? (const void*)a.wg : a.aux;
            const R* srcD = (ops & OP_VQF) ? a.Vqf : a.ws;
#pragma unroll
            for (int q = 0; q < E; q++) {
                const uint32_t idx = at(q);
                if (ops & (OP_PSI | OP_LAP | OP_AUXC))
                    cp_async(slotA + q * NT + tid, reinterpret_cast<const C2<R>*>(srcA) + idx, sizeof(C2<R>));
                if (ops & (OP_V | OP_AUXR | OP_WG))
                    cp_async(slotC + q * NT + tid, reinterpret_cast<const R*>(srcC) + idx, sizeof(R));
                if (ops & (OP_VQF | OP_WS)) cp_async(slotD + q * NT + tid, srcD + idx, sizeof(R));
            }
        }
        cp_async_commit();
    }
    if (scale_in) {
#pragma unroll
        for (int q = 0; q < E; q++) x[q] = cscale(x[q], s_prev);
    }
#ifdef GPE_USER_HOOKS
    // run-time values the user hooks read (see gpe_hooks.cuh)
    if (tid < 32) gpe_hook_ctx.up[tid] = a.uparam[tid];
    if (tid == 0) {
        gpe_hook_ctx.nx = 1u << a.lx;
        gpe_hook_ctx.ny = 1u << a.ly;
        gpe_hook_ctx.nz = 1u << a.lz;
        gpe_hook_ctx.dt = a.dt;
        gpe_hook_ctx.t0 = a.t0;
        gpe_hook_ctx.npart = a.npart;
    }
#endif
    __syncthreads();  // tables staged

    double acc[NRED] = {0.0, 0.0, 0.0};
    FF nff = {0.0f, 0.0f};  // FP32 form: norm partial
    (void)nff;

    // The heavy pointwise ops run in rolled loops over this thread's own
    // cells of the exchange buffer (positions t + T*q, which only this thread
    // reads between transforms; every exchange starts with a group barrier),
    // so their transcendental-heavy bodies appear once in the instruction
    // stream instead of E times.
    auto own = [&](int q) -> C2<R>& { return sb[padp(t + T * q) * SSTR]; };
    // operands of the MID/POST ops: staged in shared memory, or read where used (F_DIRECT: frees the
    // slots' shared memory for more resident CTAs where the transforms are short)
    constexpr bool direct = DIRECT;
    auto op_psi = [&](int q, uint32_t idx) -> C2<R> { return direct ? a.psi[idx] : slotA[q * NT + tid]; };
    auto op_lap = [&](int q, uint32_t idx) -> C2<R> { return direct ? a.lap[idx] : slotA[q * NT + tid]; };
    auto op_v = [&](int q, uint32_t idx) -> R { return direct ? a.V[idx] : slotC[q * NT + tid]; };
    auto op_vqf = [&](int q, uint32_t idx) -> R { return direct ? a.Vqf[idx] : slotD[q * NT + tid]; };
    auto op_copy = [&](int q, uint32_t idx) -> C2<R> {  // the loaded (and scaled) psi
        if (!direct) return slotB[q * NT + tid];
        const C2<R> p = a.in[idx];
        return scale_in ? cscale(p, s_prev) : p;
    };
    auto to_cells = [&]() {
#pragma unroll
        for (int q = 0; q < E; q++) own(q) = x[q];
    };
    auto from_cells = [&]() {
#pragma unroll
        for (int q = 0; q < E; q++) x[q] = own(q);
    };
    // Weizsaecker gradient sums along this axis, from x = psi (a copy in slot B):
    // D1 = IFFT(i k_a FFT psi)/N_a, d_a rho = 2 Gamma Re(conj(psi) D1), and |D1|^2.
    // mode 0 stores them, 1 adds them to the sums of the earlier axes (rescaled by
    // the pending norm factor, as they were taken from the unscaled psi), 2 adds
    // them into slots C/D for the MID op.  x is psi again afterwards.
    auto wz_grad = [&](int mode) {
        fft<R, N, P, false, SSTR, G>(x, sb, t, stw, bar);
#pragma unroll
        for (int q = 0; q < E; q++) {
            const R k = __ldg(a.ld1 + t + T * q);
            x[q] = mk<R>(-k * x[q].y, k * x[q].x);
        }
        fft<R, N, P, true, SSTR, G>(x, sb, t, stw, bar);
        cp_async_wait_all();
        if (valid) {
            const R f2 = scale_in ? s_prev * s_prev : (R)1;
#pragma unroll
            for (int q = 0; q < E; q++) {
                const C2<R> p = slotB[q * NT + tid];
                const R d = (R)2 * a.ph.gamma * (p.x * x[q].x + p.y * x[q].y);
                const R g = d * d, s = x[q].x * x[q].x + x[q].y * x[q].y;
                if (mode == 0) {
                    a.wg[at(q)] = g;
                    a.ws[at(q)] = s;
                } else if (mode == 1) {
                    a.wg[at(q)] = slotC[q * NT + tid] * (f2 * f2) + g;
                    a.ws[at(q)] = slotD[q * NT + tid] * f2 + s;
                } else {
                    slotC[q * NT + tid] += g;
                    slotD[q * NT + tid] += s;
                }
            }
        }
#pragma unroll
        for (int q = 0; q < E; q++) x[q] = slotB[q * NT + tid];
    };
    (void)wz_grad;

    // ---------------------------------------------------------------- PRE
    if constexpr (K == C_EPI || K == C_EN) {
        if (a.pre != PRE_NONE && valid) {
            const R s2 = (R)dyn->s2;
            to_cells();
#pragma unroll 1
            for (int q = 0; q < E; q++) {
                const uint32_t idx = at(q);
                int ix, iy, iz;
                decode(idx, ix, iy, iz);
                C2<R> v = own(q);
                if (K == C_EPI && a.pre == PRE_VSTEP1) {
                    v = modify_at<R>(ix, iy, iz, it, v);
                    const R rho = density(a.ph, v);
                    const R V = trap.at(a, idx, ix, iy, iz, it) + mean_field(a, rho, it);
                    a.V[idx] = V;
                    const C2<R> ph = phase(a.ph, V);
                    if (a.flags & F_PH_STORE) reinterpret_cast<C2<R>*>(a.aux)[idx] = ph;
                    v = cmul(v, ph);
                } else if (K == C_EPI && a.pre == PRE_PART2) {
                    C2<R> p2 = a.psi2[idx];
                    if (a.flags & F_SCALE_PSI2) p2 = cscale(p2, s2);
                    const R rho = density(a.ph, p2);
                    R lv = (a.V[idx] + trap.at(a, idx, ix, iy, iz, it + 1)) + mean_field(a, rho, it + 1);
                    if (a.flags & F_QF) lv += a.Vqf[idx];
                    lv = (R)0.5 * lv;
                    const C2<R> e = phase(a.ph, lv);
                    if (a.flags & F_AUX_CPLX) reinterpret_cast<C2<R>*>(a.aux)[idx] = e;
                    else reinterpret_cast<R*>(a.aux)[idx] = lv;
                    v = cmul(modify_at<R>(ix, iy, iz, it, v), e);
                } else if (K == C_EN && a.pre == PRE_ENERGY) {
                    const double px = (double)v.x, py = (double)v.y;
                    const double rho = (double)a.ph.gamma * (px * px + py * py);
                    Phys<double> phd;
                    phd.inter = a.ph.inter; phd.c_bec = (double)a.ph.c_bec; phd.a_scat = (double)a.ph.a_scat;
                    acc[0] += rho * (double)vext_at(a, idx, ix, iy, iz, it);
#ifdef GPE_USER_HOOKS
                    acc[1] += gpe_EDF(rho, (uint)it);
#else
                    acc[1] += EDF(phd, rho);
#endif
                }
                own(q) = v;
            }
            from_cells();
        }
    }

    // ------------------------------------------ dipolar convolution (C_DIP)
    if constexpr (K == C_DIP) {
        const int dm = a.mid;
        if (dm == DIP_DENS_FWD) {
#pragma unroll
            for (int q = 0; q < E; q++) x[q] = mk<R>(density(a.ph, x[q]), (R)0);
        }
        if (dm == DIP_DENS_FWD || dm == DIP_FWD || dm == DIP_VDD) fft<R, N, P, false, SSTR, G>(x, sb, t, stw, bar);
        if (dm == DIP_VDD) {
#pragma unroll
            for (int q = 0; q < E; q++) {
                int ix, iy, iz;
                decode(at(q), ix, iy, iz);
                x[q] = cscale(x[q], vdd_k(a, ix, iy, iz));
            }
        }
        if (dm != DIP_DENS_FWD && dm != DIP_FWD) fft<R, N, P, true, SSTR, G>(x, sb, t, stw, bar);
        if (dm == DIP_STEP || dm == DIP_EN) {
            cp_async_wait_all();
            if (valid) {
                const bool sc = (a.flags & F_SCALE_OPD) != 0;
                to_cells();
#pragma unroll 1
                for (int q = 0; q < E; q++) {
                    const uint32_t idx = at(q);
                    int ix, iy, iz;
                    decode(idx, ix, iy, iz);
                    const R vdip = own(q).x;  // real part of the convolution (dev/gpe_engine.cu:997-998)
                    C2<R> p = slotA[q * NT + tid];
                    if (sc) p = cscale(p, s_prev);
                    if (dm == DIP_STEP) p = modify_at<R>(ix, iy, iz, it, p);
                    const R rho = density(a.ph, p);
                    if (dm == DIP_EN) {
                        acc[0] += 0.5 * (double)rho * (double)vdip;
                        own(q) = p;
                    } else {
                        const R V = (vext_at(a, idx, ix, iy, iz, it) + mean_field(a, rho, it)) + vdip;
                        own(q) = cmul(p, phase(a.ph, V));
                    }
                }
                from_cells();
            }
            if (dm == DIP_STEP && (a.flags & F_KIN)) {
                fft<R, N, P, false, SSTR, G>(x, sb, t, stw, bar);
#pragma unroll
                for (int q = 0; q < E; q++) x[q] = cmul(x[q], skt[t + T * q]);
                fft<R, N, P, true, SSTR, G>(x, sb, t, stw, bar);
            }
            if (a.flags & F_REDUCE) {
                if constexpr (sizeof(R) == 4) {
#pragma unroll
                    for (int q = 0; q < E; q++) nff = ff_add(nff, a.ph.gamma * (x[q].x * x[q].x + x[q].y * x[q].y));
                } else {
#pragma unroll
                    for (int q = 0; q < E; q++)
                        acc[0] += (double)a.ph.gamma * ((double)x[q].x * (double)x[q].x + (double)x[q].y * (double)x[q].y);
                }
            }
        }
    }

    // ------------------------------------------------- energy: forward only
    if constexpr (K == C_EN) {
        fft<R, N, P, false, SSTR, G>(x, sb, t, stw, bar);
#pragma unroll
        for (int q = 0; q < E; q++) {
            const double w = (double)slt[t + T * q];
            acc[2] += w * ((double)x[q].x * (double)x[q].x + (double)x[q].y * (double)x[q].y);
        }
    }

    // -------------------------------------------------- Laplacian pair + MID
    if constexpr (K == C_LAP) {
        if (ops & OP_COPY) {
#pragma unroll
            for (int q = 0; q < E; q++) slotB[q * NT + tid] = x[q];
        }
        if (a.flags & F_WZ) wz_grad(a.mid == MID_LAP_STORE ? 0 : a.mid == MID_LAP_ACC ? 1 : 2);
        fft<R, N, P, false, SSTR, G>(x, sb, t, stw, bar);
#pragma unroll
        for (int q = 0; q < E; q++) x[q] = cscale(x[q], slt[t + T * q]);
        fft<R, N, P, true, SSTR, G>(x, sb, t, stw, bar);
        cp_async_wait_all();
        if (valid) {
            if (a.mid == MID_LAP_STORE) {
#pragma unroll
                for (int q = 0; q < E; q++) a.lap[at(q)] = x[q];
            } else if (a.mid == MID_LAP_ACC) {
#pragma unroll
                for (int q = 0; q < E; q++) {
                    C2<R> l = op_lap(q, at(q));
                    if (scale_in) l = cscale(l, s_prev);  // stored from the unscaled psi
                    a.lap[at(q)] = cadd(l, x[q]);
                }
            } else if (a.mid == MID_QF_VSTEP1) {
                to_cells();
                // the Laplacian and psi of point q + 1 are loaded while point q is computed
                C2<R> nl = op_lap(0, at(0)), np = op_copy(0, at(0));
#pragma unroll 1
                for (int q = 0; q < E; q++) {
                    const uint32_t idx = at(q);
                    const C2<R> L = cadd(nl, own(q));
                    const C2<R> p = np;
                    if (q + 1 < E) {
                        nl = op_lap(q + 1, at(q + 1));
                        np = op_copy(q + 1, at(q + 1));
                    }
                    int ix, iy, iz;
                    decode(idx, ix, iy, iz);
                    const R rho = density(a.ph, p);
                    // (qf/Gamma) Im(conj(psi) L) / (rho + eps), L = -lap psi   (dev/gpe_engine.cu:893-918)
                    R vqf = (a.ph.qf_g * (p.x * L.y + (-p.y) * L.x)) / (rho + a.ph.qf_eps);
                    if (a.flags & F_WZ) {
                        // (lambda/8) [ |grad rho|^2/rho^2 - 2 lap(rho)/rho ],
                        // lap rho = 2 Gamma (Re(conj(psi) lap psi) + sum_a |D1_a psi|^2)
                        const R inv = (R)1 / (rho + a.ph.wz_eps);
                        const R lrho = (R)2 * a.ph.gamma * (slotD[q * NT + tid] - (p.x * L.x + p.y * L.y));
                        vqf += a.ph.wz8 * (slotC[q * NT + tid] * inv * inv - (R)2 * lrho * inv);
                    }
                    a.Vqf[idx] = vqf;
                    // the gradient potential is taken from psi_n as stored; the step itself starts
                    // from the (user-)modified psi_n (dev/gpe_engine.cu:1040-1041, 758-760)
                    const C2<R> pm = modify_at<R>(ix, iy, iz, it, p);
#ifdef GPE_USER_HOOKS
                    // an unchanged psi keeps the density already taken (recomputing it could round
                    // differently where the compiler fuses the other product)
                    const R rho_m = (pm.x == p.x && pm.y == p.y) ? rho : density(a.ph, pm);
#else
                    const R rho_m = rho;
#endif
                    const R V = (trap.at(a, idx, ix, iy, iz, it) + mean_field(a, rho_m, it)) + vqf;
                    a.V[idx] = V;
                    const C2<R> ph = phase(a.ph, V);
                    if (a.flags & F_PH_STORE) reinterpret_cast<C2<R>*>(a.aux)[idx] = ph;
                    own(q) = cmul(pm, ph);
                }
                from_cells();
            } else if (a.mid == MID_CURRENT) {
                // probability current along the pass axis: Re(conj(psi) IFFT(k_a/(Gamma N_a) FFT psi))
                // (cplxMulR of dev/gpe_engine.cu:1660-1667 after the k_a multiply of :1817-1854)
#pragma unroll
                for (int q = 0; q < E; q++) {
                    const C2<R> p = slotB[q * NT + tid];
                    a.V[at(q)] = p.x * x[q].x + p.y * x[q].y;
                }
            }
        }
    }

    // ---------------------------------------------------------- kinetic pair
    if constexpr (K != C_EN && K != C_DIP) {  // the dipolar passes run their own transforms
        if (K != C_LAP || (a.flags & F_KIN)) {
            fft<R, N, P, false, SSTR, G>(x, sb, t, stw, bar);
#pragma unroll
            for (int q = 0; q < E; q++) x[q] = cmul(x[q], skt[t + T * q]);
            fft<R, N, P, true, SSTR, G>(x, sb, t, stw, bar);
        }
    }

    // ------------------------------------------- POST, partial sums, store
    if constexpr (K == C_EPI) {
        if (a.post != POST_NONE && valid) {
            cp_async_wait_all();
            to_cells();
            // The operands of point q + 1 are loaded while point q is computed, so that their latency
            // (an L2 round trip where they are read in place) overlaps the transcendental work.
            if (a.post == POST_VSTEP2 || a.post == POST_PART12) {
                const bool qfop = (a.post == POST_PART12) && (a.flags & F_QF);
                // the predictor's phase factor exp(c3 V), stored by Vstep1 (the same bits as recomputing it)
                const bool phl = (a.flags & F_PH_LOAD) != 0;
                const C2<R>* auxc = reinterpret_cast<const C2<R>*>(a.aux);
                R nv = op_v(0, at(0)), nq = qfop ? op_vqf(0, at(0)) : (R)0;
                C2<R> np = op_psi(0, at(0)), nph = phl ? auxc[at(0)] : mk<R>((R)0, (R)0);
#pragma unroll 1
                for (int q = 0; q < E; q++) {
                    const uint32_t idx = at(q);
                    R lv = nv;
                    C2<R> p = np;
                    const C2<R> ph = nph;
                    const R vq = nq;
                    if (q + 1 < E) {
                        const uint32_t nidx = at(q + 1);
                        nv = op_v(q + 1, nidx);
                        np = op_psi(q + 1, nidx);
                        if (qfop) nq = op_vqf(q + 1, nidx);
                        if (phl) nph = auxc[nidx];
                    }
                    int ix, iy, iz;
                    decode(idx, ix, iy, iz);
                    const C2<R> pp = cmul(own(q), phl ? ph : phase(a.ph, lv));
                    const R rho = density(a.ph, pp);
                    lv = (lv + trap.at(a, idx, ix, iy, iz, it + 1)) + mean_field(a, rho, it + 1);
                    if (qfop) lv += vq;
                    lv = (R)0.5 * lv;
                    const C2<R> e = phase(a.ph, lv);
                    if (a.flags & F_AUX_CPLX) reinterpret_cast<C2<R>*>(a.aux)[idx] = e;
                    else reinterpret_cast<R*>(a.aux)[idx] = lv;
                    if (scale_in) p = cscale(p, s_prev);
                    own(q) = cmul(modify_at<R>(ix, iy, iz, it, p), e);
                }
            } else if (a.post == POST_PART1) {
                if (a.flags & F_PH_LOAD) {  // exp(c3 V) as Vstep1 stored it
                    const C2<R>* auxc = reinterpret_cast<const C2<R>*>(a.aux);
#pragma unroll
                    for (int q = 0; q < E; q++) own(q) = cmul(own(q), auxc[at(q)]);
                } else {
                    R nv = op_v(0, at(0));
#pragma unroll 1
                    for (int q = 0; q < E; q++) {
                        const R lv = nv;
                        if (q + 1 < E) nv = op_v(q + 1, at(q + 1));
                        own(q) = cmul(own(q), phase(a.ph, lv));
                    }
                }
            } else if (a.post == POST_VSTEP3) {
                if (a.flags & F_AUX_CPLX) {
                    // the stored factor: one complex multiply per point (unrolled: all loads in flight)
#pragma unroll
                    for (int q = 0; q < E; q++)
                        own(q) = cmul(own(q), direct ? reinterpret_cast<const C2<R>*>(a.aux)[at(q)] : slotA[q * NT + tid]);
                } else {
#pragma unroll 1
                    for (int q = 0; q < E; q++) own(q) = cmul(own(q), phase(a.ph, slotC[q * NT + tid]));
                }
            }
            from_cells();
        }
        if (a.flags & F_REDUCE) {
            if constexpr (sizeof(R) == 4) {
#pragma unroll
                for (int q = 0; q < E; q++) nff = ff_add(nff, a.ph.gamma * (x[q].x * x[q].x + x[q].y * x[q].y));
            } else {
#pragma unroll
                for (int q = 0; q < E; q++)
                    acc[0] += (double)a.ph.gamma * ((double)x[q].x * (double)x[q].x + (double)x[q].y * (double)x[q].y);
            }
        }
    }
    if constexpr (K != C_EN) {
        if ((a.flags & F_STORE) && valid) {
#pragma unroll
            for (int q = 0; q < E; q++) a.out[at(q)] = x[q];
        }
    }
    if constexpr (K == C_EPI) {
        if (a.flags & F_LAP_OUT) {
            if (a.flags & F_WZ) {
#pragma unroll
                for (int q = 0; q < E; q++) slotB[q * NT + tid] = x[q];
                wz_grad(0);
            }
            fft<R, N, P, false, SSTR, G>(x, sb, t, stw, bar);
#pragma unroll
            for (int q = 0; q < E; q++) x[q] = cscale(x[q], slt[t + T * q]);
            fft<R, N, P, true, SSTR, G>(x, sb, t, stw, bar);
            if (valid) {
#pragma unroll
                for (int q = 0; q < E; q++) a.lap[at(q)] = x[q];
            }
        }
    }

    // ------------------------------------------------- cross-CTA finalise
    if constexpr (FIN) {
        if (a.flags & (F_FIN_S2 | F_FIN_STEP | F_FIN_RED)) {
            // energy: 3 sums; norm: 1; a real-time step only advances the step counter
            constexpr int NR = (K == C_EN) ? 3 : 1;
            const bool sums = (K == C_EN) || (a.flags & (F_REDUCE | F_FIN_RED));
            if (sums) {
                if constexpr ((K == C_EPI || K == C_DIP) && sizeof(R) == 4) {
                    if (a.flags & F_REDUCE) acc[0] = block_sum_ff<NT>(nff, sred);
                    else block_sum<NT, NR>(acc, sred);
                } else {
                    block_sum<NT, NR>(acc, sred);
                }
            }
            if (tid == 0) {
                if (sums)
#pragma unroll
                    for (int r = 0; r < NR; r++) a.partials[(size_t)blk * NRED + r] = acc[r];
                __threadfence();
                const unsigned prev = atomicAdd(&a.dyn->ticket, 1u);
                last_cta = (prev == nblk - 1);
            }
            __syncthreads();
            if (last_cta) {
                __threadfence();
                finalize<R, NT, NR>(a, sred, nblk, sums);
            }
        }
    }
}

// Persistent kinetic pass (FFT_a, x kinetic factor, inverse FFT_a) for HBM-resident lattices: each CTA
// walks tiles of W pencils grid-stride, and while it transforms one tile the next tile's points are
// already on their way into shared memory (cp.async into a staging buffer that only the copying
// thread reads back), so the loads of one tile overlap the arithmetic of the previous one.
template <typename R, int N, int AX, int NT, int P>
__device__ __forceinline__ void kin_pipe_body(const PassArgs<R>& a) {
    using Geo = PassGeom<R, N, AX, NT, P>;
    constexpr int E = Geo::E, T = Geo::T, CW = Geo::CW, G = Geo::G, W = Geo::W, ROW = Geo::ROW;
    constexpr int SSTR = (AX == AX_Z) ? 1 : CW;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* stw = reinterpret_cast<C2<R>*>(smem_raw);
    C2<R>* skt = stw + Geo::TW;
    C2<R>* sx = reinterpret_cast<C2<R>*>(smem_raw + Geo::TAB_BYTES);
    C2<R>* stg = reinterpret_cast<C2<R>*>(smem_raw + Geo::SMEM_BASE);
    const int tid = threadIdx.x;
    // constant tables first (they overlap the previous pass's drain), then wait for that pass
    for (int i = tid; i < Geo::TW; i += NT) stw[i] = a.tw[i];
    for (int i = tid; i < N; i += NT) skt[i] = a.ktab[i];
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    int pl, t, bar;
    C2<R>* sb;
    if constexpr (AX == AX_Z) {
        t = tid % T;
        pl = tid / T;
        sb = sx + pl * ROW;
        bar = 0;
    } else {
        const int gi = tid / G, loc = tid % G;
        const int c = loc % CW;
        t = loc / CW;
        pl = gi * CW + c;
        sb = sx + gi * (ROW * CW) + c;
        bar = 1 + gi;
    }
    const int ly = a.ly, lz = a.lz;
    const uint32_t lstr = (AX == AX_Z) ? 0u : (AX == AX_Y) ? (uint32_t)lz : (uint32_t)(ly + lz);
    auto tbase = [&](uint32_t tile, bool& valid) -> uint32_t {
        const uint32_t gp = tile * (uint32_t)W + pl;
        valid = gp < a.npencils;
        uint32_t base;
        if constexpr (AX == AX_Z) base = gp << lz;
        else if constexpr (AX == AX_Y) base = (((gp >> lz) << ly) << lz) + (gp & ((1u << lz) - 1));
        else base = gp;
        return base + ((uint32_t)t << lstr);
    };
    const uint32_t ntiles = (a.npencils + W - 1) / W;
    auto prefetch = [&](uint32_t tile) {
        bool v;
        const uint32_t tb = tbase(tile, v);
        if (v) {
#pragma unroll
            for (int q = 0; q < E; q++)
                cp_async(stg + q * NT + tid, a.in + tb + ((uint32_t)(T * q) << lstr), sizeof(C2<R>));
        }
        cp_async_commit();
    };
    uint32_t tile = blockIdx.x;
    if (tile < ntiles) prefetch(tile);
    __syncthreads();  // tables staged
    for (; tile < ntiles; tile += gridDim.x) {
        bool valid;
        const uint32_t tb = tbase(tile, valid);
        cp_async_wait_all();
        C2<R> x[E];
#pragma unroll
        for (int q = 0; q < E; q++) x[q] = valid ? stg[q * NT + tid] : mk<R>((R)0, (R)0);
        if (tile + gridDim.x < ntiles) prefetch(tile + gridDim.x);
        fft<R, N, P, false, SSTR, G>(x, sb, t, stw, bar);
#pragma unroll
        for (int q = 0; q < E; q++) x[q] = cmul(x[q], skt[t + T * q]);
        fft<R, N, P, true, SSTR, G>(x, sb, t, stw, bar);
        if (valid) {
#pragma unroll
            for (int q = 0; q < E; q++) a.out[tb + ((uint32_t)(T * q) << lstr)] = x[q];
        }
    }
    cp_async_wait_all();
}

template <typename R, int N, int AX, int NT, int CLS, int P>
__global__ void __launch_bounds__(NT, PassGeom<R, N, AX, NT, P>::MINB)
pass_kernel(const PassArgs<R> a) {
    if constexpr (CLS == C_KINP) kin_pipe_body<R, N, AX, NT, P>(a);
    else pass_body<R, N, AX, NT, CLS, P>(a, blockIdx.x, gridDim.x);
}

}  // namespace gpe
