// Fused pencil pass: the one kernel shape of the split-step evolution.
//
// A launch walks every pencil of one axis of the lattice.  For each point it
// runs, in order,
//   load -> PRE op -> [LAP pair: FFT, x k_a^2 table, inverse FFT -> MID op]
//        -> [KIN pair: FFT, x exp(c k_a^2)/N_a table, inverse FFT] -> POST op
//        -> store (+ FP64 partial sums, finalised by the last CTA).
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
};

// Scalars that change while a step runs; they live in device memory so one
// captured step can be replayed.
struct DynState {
    double s_prev;     // pending normalisation factor of psi
    double s2;         // normalisation factor of psi2 inside an ITE step
    double norm;       // last sum of Gamma |psi|^2
    double mu;         // -0.5 log(norm / npart) / dt  (dev/gpe_engine.cu:1101)
    double red[16];    // results of generic reductions
    unsigned int it;   // step counter since set_psi / set_time
    unsigned int ticket;
    unsigned int err;
    unsigned int pad;
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
    R* Vqf;              // quantum-friction potential
    const R* vx; const R* vy; const R* vz;   // trap tables
    const R* vextra;     // [slices][n] additive potential (F_VEXTRA)
    int vsteps, vslices;
    const C2<R>* ktab;   // kinetic factors of this axis, incl. 1/N_a
    const R* ltab;       // Laplacian / kinetic-energy weights of this axis
    const C2<R>* tw;     // exp(-2 pi i p / N_a)
    DynState* dyn;
    double* partials;    // [gridDim.x][NRED]
    int lx, ly, lz;      // log2 of the lattice sides
    double npart, dt;
    int red_slot;
    uint32_t flags;
    int pre, mid, post;
    Phys<R> ph;
};

template <typename R> __device__ __forceinline__ R vext_at(const PassArgs<R>& a, size_t idx, int ix, int iy, int iz,
                                                          unsigned it) {
    R v = (__ldg(a.vx + ix) + __ldg(a.vy + iy)) + __ldg(a.vz + iz);
    if (a.flags & F_VEXTRA) {
        int s = (int)(it / (unsigned)a.vsteps);
        if (s >= a.vslices) s = a.vslices - 1;
        v += a.vextra[(size_t)s << (a.lx + a.ly + a.lz) | idx];
    }
    return v;
}

template <typename C> __device__ __forceinline__ C ldc(const C* p) { return *p; }

// Deterministic block sum of NRED doubles; result valid in thread 0.
template <int NT>
__device__ __forceinline__ void block_sum(double (&v)[NRED], double (*sred)[NRED]) {
#pragma unroll
    for (int r = 0; r < NRED; r++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[r] += __shfl_down_sync(0xffffffffu, v[r], o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int r = 0; r < NRED; r++) sred[w][r] = v[r];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int r = 0; r < NRED; r++) {
            double s = 0.0;
            for (int i = 0; i < (NT + 31) / 32; i++) s += sred[i][r];
            v[r] = s;
        }
    }
}

// Last CTA of the grid: sums the per-CTA partials in index order with
// Neumaier compensation and publishes the results.
template <typename R, int NT>
__device__ void finalize(const PassArgs<R>& a, double (*sred)[NRED]) {
    double s[NRED], c[NRED];
#pragma unroll
    for (int r = 0; r < NRED; r++) { s[r] = 0.0; c[r] = 0.0; }
    for (int b = threadIdx.x; b < (int)gridDim.x; b += NT) {
#pragma unroll
        for (int r = 0; r < NRED; r++) {
            const double x = __ldcg(a.partials + (size_t)b * NRED + r);
            const double t = s[r] + x;
            c[r] += (fabs(s[r]) >= fabs(x)) ? (s[r] - t) + x : (x - t) + s[r];
            s[r] = t;
        }
    }
#pragma unroll
    for (int r = 0; r < NRED; r++) s[r] += c[r];
    block_sum<NT>(s, sred);
    if (threadIdx.x == 0) {
        DynState* d = a.dyn;
        if (a.flags & F_FIN_S2) d->s2 = sqrt(a.npart / s[0]);
        if (a.flags & F_FIN_STEP) {
            if (a.flags & F_REDUCE) {
                d->norm = s[0];
                d->s_prev = sqrt(a.npart / s[0]);
                d->mu = -.5 * log(s[0] / a.npart) / a.dt;
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

template <typename R, int N, int AX, int W>
__global__ void __launch_bounds__(W * (N / Plan<N>::E))
pass_kernel(const PassArgs<R> a) {
    constexpr int E = Plan<N>::E, T = N / E, NT = W * T;
    constexpr int SSTR = (AX == AX_Z) ? 1 : W;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* smem = reinterpret_cast<C2<R>*>(smem_raw);
    __shared__ double sred[(NT + 31) / 32][NRED];
    __shared__ bool last_cta;

    const int tid = threadIdx.x;
    int pl, t;
    if constexpr (AX == AX_Z) { t = tid % T; pl = tid / T; }
    else { pl = tid % W; t = tid / W; }
    C2<R>* sb = (AX == AX_Z) ? smem + pl * (N + 1) : smem + pl;

    const size_t gp = (size_t)blockIdx.x * W + pl;  // pencil id
    const int lx = a.lx, ly = a.ly, lz = a.lz;
    size_t base, estr;
    if constexpr (AX == AX_Z) { base = gp << lz; estr = 1; }
    else if constexpr (AX == AX_Y) {
        const size_t ix = gp >> lz, iz = gp & ((1u << lz) - 1);
        base = ((ix << ly) << lz) + iz; estr = (size_t)1 << lz;
    } else { base = gp; estr = (size_t)1 << (ly + lz); }
    (void)lx;

    const DynState* dyn = a.dyn;
    const unsigned it = dyn->it;
    const R s_prev = (R)dyn->s_prev;

    C2<R> x[E];
#pragma unroll
    for (int q = 0; q < E; q++) x[q] = ldc(a.in + base + (size_t)(t + T * q) * estr);

    double acc[NRED] = {0.0, 0.0, 0.0};

    // ---------------------------------------------------------------- PRE
    if (a.flags & F_SCALE_IN) {
#pragma unroll
        for (int q = 0; q < E; q++) x[q] = cscale(x[q], s_prev);
    }
    if (a.pre != PRE_NONE) {
        const R s2 = (R)dyn->s2;
#pragma unroll
        for (int q = 0; q < E; q++) {
            const size_t idx = base + (size_t)(t + T * q) * estr;
            const int ix = (int)(idx >> (ly + lz)), iy = (int)((idx >> lz) & ((1u << ly) - 1)),
                      iz = (int)(idx & ((1u << lz) - 1));
            if (a.pre == PRE_VSTEP1) {
                const R rho = density(a.ph, x[q]);
                const R V = vext_at(a, idx, ix, iy, iz, it) + dEDFdn(a.ph, rho);
                a.V[idx] = V;
                x[q] = cmul(x[q], phase(a.ph, V));
            } else if (a.pre == PRE_PART2) {
                C2<R> p2 = a.psi2[idx];
                if (a.flags & F_SCALE_PSI2) p2 = cscale(p2, s2);
                const R rho = density(a.ph, p2);
                R lv = (a.V[idx] + vext_at(a, idx, ix, iy, iz, it + 1)) + dEDFdn(a.ph, rho);
                if (a.flags & F_QF) lv += a.Vqf[idx];
                lv = (R)0.5 * lv;
                const C2<R> e = phase(a.ph, lv);
                if (a.flags & F_AUX_CPLX) reinterpret_cast<C2<R>*>(a.aux)[idx] = e;
                else reinterpret_cast<R*>(a.aux)[idx] = lv;
                x[q] = cmul(x[q], e);
            } else if (a.pre == PRE_ENERGY) {
                const C2<double> pd = make_double2((double)x[q].x, (double)x[q].y);
                const double rho = (double)a.ph.gamma * (pd.x * pd.x + pd.y * pd.y);
                Phys<double> phd;
                phd.inter = a.ph.inter; phd.c_bec = (double)a.ph.c_bec; phd.a_scat = (double)a.ph.a_scat;
                acc[0] += rho * (double)vext_at(a, idx, ix, iy, iz, it);
                acc[1] += EDF(phd, rho);
            }
        }
    }

    // -------------------------------------------------- Laplacian pair + MID
    if (a.flags & (F_LAP | F_EKIN)) {
        C2<R> c[E];
#pragma unroll
        for (int q = 0; q < E; q++) c[q] = x[q];
        fft<R, N, false, SSTR>(c, sb, t, a.tw);
        if (a.flags & F_EKIN) {
#pragma unroll
            for (int q = 0; q < E; q++) {
                const double w = (double)__ldg(a.ltab + t + T * q);
                acc[2] += w * ((double)c[q].x * (double)c[q].x + (double)c[q].y * (double)c[q].y);
            }
        } else {
#pragma unroll
            for (int q = 0; q < E; q++) c[q] = cscale(c[q], __ldg(a.ltab + t + T * q));
            fft<R, N, true, SSTR>(c, sb, t, a.tw);
#pragma unroll
            for (int q = 0; q < E; q++) {
                const size_t idx = base + (size_t)(t + T * q) * estr;
                if (a.mid == MID_LAP_STORE) {
                    a.lap[idx] = c[q];
                } else if (a.mid == MID_LAP_ACC) {
                    a.lap[idx] = cadd(a.lap[idx], c[q]);
                } else if (a.mid == MID_QF_VSTEP1) {
                    const int ix = (int)(idx >> (ly + lz)), iy = (int)((idx >> lz) & ((1u << ly) - 1)),
                              iz = (int)(idx & ((1u << lz) - 1));
                    const C2<R> L = cadd(a.lap[idx], c[q]);
                    const R rho = density(a.ph, x[q]);
                    // Im(conj(psi) L) / (rho + eps)   (dev/gpe_engine.cu:916)
                    const R vqf = (x[q].x * L.y + (-x[q].y) * L.x) / (rho + a.ph.qf_eps);
                    a.Vqf[idx] = vqf;
                    const R V = (vext_at(a, idx, ix, iy, iz, it) + dEDFdn(a.ph, rho)) + vqf;
                    a.V[idx] = V;
                    x[q] = cmul(x[q], phase(a.ph, V));
                }
            }
        }
    }

    // ---------------------------------------------------------- kinetic pair
    if (a.flags & F_KIN) {
        fft<R, N, false, SSTR>(x, sb, t, a.tw);
#pragma unroll
        for (int q = 0; q < E; q++) x[q] = cmul(x[q], a.ktab[t + T * q]);
        fft<R, N, true, SSTR>(x, sb, t, a.tw);
    }

    // ---------------------------------------------------------------- POST
    if (a.post != POST_NONE) {
#pragma unroll
        for (int q = 0; q < E; q++) {
            const size_t idx = base + (size_t)(t + T * q) * estr;
            const int ix = (int)(idx >> (ly + lz)), iy = (int)((idx >> lz) & ((1u << ly) - 1)),
                      iz = (int)(idx & ((1u << lz) - 1));
            if (a.post == POST_VSTEP2 || a.post == POST_PART12) {
                R lv = a.V[idx];
                const C2<R> pp = cmul(x[q], phase(a.ph, lv));
                const R rho = density(a.ph, pp);
                lv = (lv + vext_at(a, idx, ix, iy, iz, it + 1)) + dEDFdn(a.ph, rho);
                if (a.post == POST_PART12 && (a.flags & F_QF)) lv += a.Vqf[idx];
                lv = (R)0.5 * lv;
                const C2<R> e = phase(a.ph, lv);
                if (a.flags & F_AUX_CPLX) reinterpret_cast<C2<R>*>(a.aux)[idx] = e;
                else reinterpret_cast<R*>(a.aux)[idx] = lv;
                C2<R> p = a.psi[idx];
                if (a.flags & F_SCALE_IN) p = cscale(p, s_prev);
                x[q] = cmul(p, e);
            } else if (a.post == POST_PART1) {
                x[q] = cmul(x[q], phase(a.ph, a.V[idx]));
            } else if (a.post == POST_VSTEP3) {
                C2<R> e;
                if (a.flags & F_AUX_CPLX) e = reinterpret_cast<const C2<R>*>(a.aux)[idx];
                else e = phase(a.ph, reinterpret_cast<const R*>(a.aux)[idx]);
                x[q] = cmul(x[q], e);
            }
        }
    }
    if (a.flags & F_REDUCE) {
#pragma unroll
        for (int q = 0; q < E; q++)
            acc[0] += (double)a.ph.gamma * ((double)x[q].x * (double)x[q].x + (double)x[q].y * (double)x[q].y);
    }
    if (a.flags & F_STORE) {
#pragma unroll
        for (int q = 0; q < E; q++) a.out[base + (size_t)(t + T * q) * estr] = x[q];
    }

    // ------------------------------------------------- cross-CTA finalise
    if (a.flags & (F_FIN_S2 | F_FIN_STEP | F_FIN_RED)) {
        block_sum<NT>(acc, sred);
        if (tid == 0) {
#pragma unroll
            for (int r = 0; r < NRED; r++) a.partials[(size_t)blockIdx.x * NRED + r] = acc[r];
            __threadfence();
            const unsigned prev = atomicAdd(&a.dyn->ticket, 1u);
            last_cta = (prev == gridDim.x - 1);
        }
        __syncthreads();
        if (last_cta) {
            __threadfence();
            finalize<R, NT>(a, sred);
        }
    }
}

}  // namespace gpe
