// yz-plane pass (FP32-mixed form): the y and z transforms of one x-plane in
// one CTA.
//
// A lattice plane [iy][iz] of N x N points (N = 128: 128 KiB of FP32 complex)
// is contiguous in memory and fits one CTA's shared memory, so the kinetic
// factor of both axes, exp(c3 k_y^2) exp(c3 k_z^2), is applied by one 2D
// transform pair inside the CTA instead of two pencil passes, each of which
// reads and writes the whole field through L2.  With the pointwise ops of the
// step fused in (Vstep1 before, the corrector or Vstep3 after) and the y+z
// spectral Laplacian of the result (quantum friction), a real-time step takes
// four launches (two plane passes, two x-pencil passes) instead of seven.
//
// Layout in shared memory: point (iy, iz) at padp(iy) * RP + padp(iz), with
// one pad slot per 16 points along each row and a row pitch RP = 146 slots
// (RP = 2 mod 16).  1024 threads; every 128-point row and every 128-point
// column is transformed by 8 threads of one warp (16 points each), so all
// transform exchanges run under warp barriers and the CTA meets only where
// rows hand over to columns and back.  Row phase: a half-warp holds two rows
// four apart (their slots differ by 4 RP = 8 mod 16); column phase: a
// half-warp holds two adjacent columns, each thread of a column on its own row
// (rows differ by RP = 2 mod 16): both phases address 16 distinct 8-byte bank
// pairs per half-warp.  Rows are loaded from and stored to global memory in
// the z-pass pattern (8 threads x 8 B = 64 contiguous bytes per row segment).
#pragma once
#include "gpe_pass.cuh"

namespace gpe {

struct PlaneArgs {
    PassArgs<float> a;   // field, ops, device state; a.ktab / a.ltab: z tables; a.tw: twiddles (plan 0)
    const float2* kty;   // y kinetic factors exp(c3 k_y^2) / N_y
    const float* lqy;    // y Laplacian weights k_y^2 / N_y
};

template <int N>
struct PlaneGeom {
    static constexpr int E = Plan<N, 0>::E;
    static constexpr int T = N / E;  // threads per row / per column
    static constexpr int NT = N * T;
    static constexpr int ROWS = padded_len<N>();            // padded row index range
    static constexpr int RP = ((padded_len<N>() + 13) / 16) * 16 + 2;  // row pitch, = 2 mod 16
    static constexpr int TW = tw_len<N, 0>();
    static constexpr size_t TAB_BYTES = (((size_t)(TW + 2 * N) * sizeof(float2) + 2 * N * sizeof(float)) + 15) & ~(size_t)15;
    static constexpr size_t PLANE_BYTES = (size_t)ROWS * RP * sizeof(float2);
    static_assert(RP >= padded_len<N>() && RP % 16 == 2, "row pitch");
    static_assert(T == 8 && N % 128 == 0, "8 threads per row and column, rows in groups of 8");
    static constexpr size_t SMEM = TAB_BYTES + PLANE_BYTES;
    static_assert(NT == 1024, "one plane per 1024-thread CTA");
    static_assert(SMEM <= 225 * 1024, "plane does not fit shared memory");
};

// Ops a plane pass supports (real time only: no reductions, no pending norm factor).
__host__ __device__ inline bool plane_supports(int pre, int mid, int post, uint32_t flags) {
    const uint32_t allowed = F_KIN | F_STORE | F_QF | F_AUX_CPLX | F_LAP_OUT | F_FIN_STEP | F_VEXTRA | F_LAP |
                             F_PH_STORE | F_PH_LOAD;
    if (flags & ~allowed) return false;
    if (pre != PRE_NONE && pre != PRE_VSTEP1) return false;
    if (mid != MID_NONE && mid != MID_LAP_STORE) return false;
    if (post != POST_NONE && post != POST_PART12 && post != POST_VSTEP3) return false;
    return true;
}

template <int N>
__global__ void __launch_bounds__(PlaneGeom<N>::NT, 1) plane_kernel(const PlaneArgs pa) {
    using R = float;
    using Geo = PlaneGeom<N>;
    constexpr int E = Geo::E, T = Geo::T, NT = Geo::NT, RP = Geo::RP;
    const PassArgs<R>& a = pa.a;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C2<R>* stw = reinterpret_cast<C2<R>*>(smem_raw);
    C2<R>* sky = stw + Geo::TW;
    C2<R>* skz = sky + N;
    R* sly = reinterpret_cast<R*>(skz + N);
    R* slz = sly + N;
    C2<R>* plane = reinterpret_cast<C2<R>*>(smem_raw + Geo::TAB_BYTES);
    __shared__ double sred[NT / 32][NRED];
    __shared__ bool last_cta;

    // constant tables before the wait for the previous pass (programmatic dependent launch)
    const int tid = threadIdx.x;
    for (int i = tid; i < Geo::TW; i += NT) stw[i] = a.tw[i];
    for (int i = tid; i < N; i += NT) {
        sky[i] = pa.kty[i];
        skz[i] = a.ktab[i];
        sly[i] = pa.lqy[i];
        slz[i] = a.ltab[i];
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

    // row phase: 8 threads per row (points iz = tr + T q); warp w holds rows 8(w/2) + 2(w%2) + {0, 1, 4, 5}
    // (a half-warp: two rows four apart).  Column phase: 8 threads per column (points iy = tc + T q),
    // warp w holds columns 4w .. 4w + 3.
    const int warp = tid >> 5, lane = tid & 31;
    const int tr = lane & 7;
    const int row = 8 * (warp >> 1) + 2 * (warp & 1) + ((lane >> 4) & 1) + 4 * ((lane >> 3) & 1);
    const int tc = lane & 7;
    const int col = 4 * warp + (lane >> 3);
    C2<R>* sbr = plane + padp(row) * RP;
    C2<R>* sbc = plane + padp(col);
    const uint32_t ix = blockIdx.x;
    const int ly = a.ly, lz = a.lz;
    const uint32_t rowbase = ((ix << ly) + (uint32_t)row) << lz;
    auto at = [&](int q) -> uint32_t { return rowbase + (uint32_t)(tr + T * q); };
    auto rcell = [&](int q) -> C2<R>& { return sbr[padp(tr + T * q)]; };
    auto ccell = [&](int q) -> C2<R>& { return sbc[padp(tc + T * q) * RP]; };

    const DynState* dyn = a.dyn;
    const unsigned it = dyn->it;
    PencilTrap<R, 3> trap;  // vx[ix] + vy[row], constant along the thread's row
    trap.init(a, (int)ix, row, 0);
    C2<R> x[E];
#pragma unroll
    for (int q = 0; q < E; q++) x[q] = a.in[at(q)];
#ifdef GPE_USER_HOOKS
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
    __syncthreads();  // tables (and hook context) staged

    // ------------------------------------------------------------ PRE (row cells)
    if (a.pre == PRE_VSTEP1) {
#pragma unroll
        for (int q = 0; q < E; q++) rcell(q) = x[q];
#pragma unroll 1
        for (int q = 0; q < E; q++) {
            const uint32_t idx = at(q);
            const int iz = tr + T * q;
            C2<R> v = modify_at<R>((int)ix, row, iz, it, rcell(q));
            const R rho = density(a.ph, v);
            const R V = trap.at(a, idx, (int)ix, row, iz, it) + mean_field(a, rho, it);
            a.V[idx] = V;
            const C2<R> ph = phase(a.ph, V);
            if (a.flags & F_PH_STORE) reinterpret_cast<C2<R>*>(a.aux)[idx] = ph;
            rcell(q) = cmul(v, ph);
        }
#pragma unroll
        for (int q = 0; q < E; q++) x[q] = rcell(q);
        __syncwarp();
    }

    // 2D transform pair: rows forward, columns forward, x mult(k_y, k_z), columns inverse, rows inverse.
    // `mode` 0: kinetic factors; 1: Laplacian weights (k_y^2 + k_z^2) / (N_y N_z)
    auto pair2d = [&](int mode) {
        fft<R, N, 0, false, 1, 32>(x, sbr, tr, stw, 0);
        __syncwarp();  // the row's exchange reads are done before its cells are overwritten
#pragma unroll
        for (int q = 0; q < E; q++) rcell(q) = x[q];
        __syncthreads();  // every row is in its cells
#pragma unroll
        for (int q = 0; q < E; q++) x[q] = ccell(q);
        fft<R, N, 0, false, RP, 32>(x, sbc, tc, stw, 0);
        if (mode == 0) {
            const C2<R> kz = skz[col];
#pragma unroll
            for (int q = 0; q < E; q++) x[q] = cmul(cmul(x[q], sky[tc + T * q]), kz);
        } else {
            const R lz_ = slz[col];
            const R inv = (R)1 / (R)N;
#pragma unroll
            for (int q = 0; q < E; q++) x[q] = cscale(x[q], (sly[tc + T * q] + lz_) * inv);
        }
        fft<R, N, 0, true, RP, 32>(x, sbc, tc, stw, 0);
        __syncwarp();  // the column's exchange reads are done before its cells are overwritten
#pragma unroll
        for (int q = 0; q < E; q++) ccell(q) = x[q];
        __syncthreads();  // every column is in its cells
#pragma unroll
        for (int q = 0; q < E; q++) x[q] = rcell(q);
        fft<R, N, 0, true, 1, 32>(x, sbr, tr, stw, 0);
    };

    // The transform pairs of the pass run in one rolled loop, so the four transforms appear once in the
    // instruction stream: k = 0 is the step's pair (kinetic, then the POST op and the store) or, with
    // F_LAP, the Laplacian of the input alone; k = 1 the Laplacian of the result (F_LAP_OUT).
    const bool lap_only = (a.flags & F_LAP) != 0;
#pragma unroll 1
    for (int k = 0; k < 2; k++) {
        if (k == 1) {
            if (lap_only || !(a.flags & F_LAP_OUT)) break;
            __syncthreads();  // the plane's cells are free again
        }
        const int mode = (k == 1 || lap_only) ? 1 : 0;
        if (mode == 1 || (a.flags & F_KIN)) pair2d(mode);
        if (mode == 1) {
            // y + z Laplacian (of the input with F_LAP, of the result with F_LAP_OUT)
#pragma unroll
            for (int q = 0; q < E; q++) a.lap[at(q)] = x[q];
            continue;
        }

        // -------------------------------------------------------- POST (row cells)
        if (a.post == POST_PART12) {
            // the operands of point q + 1 are loaded while point q is computed (their L2 latency
            // overlaps the transcendental work)
            __syncwarp();
#pragma unroll
            for (int q = 0; q < E; q++) rcell(q) = x[q];
            const bool qfop = (a.flags & F_QF) != 0;
            const bool phl = (a.flags & F_PH_LOAD) != 0;  // exp(c3 V) as Vstep1 stored it
            const C2<R>* auxc = reinterpret_cast<const C2<R>*>(a.aux);
            R nv = a.V[at(0)], nq = qfop ? a.Vqf[at(0)] : (R)0;
            C2<R> np = a.psi[at(0)], nph = phl ? auxc[at(0)] : mk<R>((R)0, (R)0);
#pragma unroll 1
            for (int q = 0; q < E; q++) {
                const uint32_t idx = at(q);
                const int iz = tr + T * q;
                R lv = nv;
                const C2<R> p = np;
                const C2<R> ph = nph;
                const R vq = nq;
                if (q + 1 < E) {
                    nv = a.V[at(q + 1)];
                    np = a.psi[at(q + 1)];
                    if (qfop) nq = a.Vqf[at(q + 1)];
                    if (phl) nph = auxc[at(q + 1)];
                }
                const C2<R> pp = cmul(rcell(q), phl ? ph : phase(a.ph, lv));
                const R rho = density(a.ph, pp);
                lv = (lv + trap.at(a, idx, (int)ix, row, iz, it + 1)) + mean_field(a, rho, it + 1);
                if (qfop) lv += vq;
                lv = (R)0.5 * lv;
                const C2<R> e = phase(a.ph, lv);
                if (a.flags & F_AUX_CPLX) reinterpret_cast<C2<R>*>(a.aux)[idx] = e;
                else reinterpret_cast<R*>(a.aux)[idx] = lv;
                rcell(q) = cmul(modify_at<R>((int)ix, row, iz, it, p), e);
            }
#pragma unroll
            for (int q = 0; q < E; q++) x[q] = rcell(q);
            __syncwarp();
        } else if (a.post == POST_VSTEP3) {
            if (a.flags & F_AUX_CPLX) {
#pragma unroll
                for (int q = 0; q < E; q++) x[q] = cmul(x[q], reinterpret_cast<const C2<R>*>(a.aux)[at(q)]);
            } else {
                __syncwarp();
#pragma unroll
                for (int q = 0; q < E; q++) rcell(q) = x[q];
#pragma unroll 1
                for (int q = 0; q < E; q++) rcell(q) = cmul(rcell(q), phase(a.ph, reinterpret_cast<const R*>(a.aux)[at(q)]));
#pragma unroll
                for (int q = 0; q < E; q++) x[q] = rcell(q);
                __syncwarp();
            }
        }
        if (a.flags & F_STORE) {
#pragma unroll
            for (int q = 0; q < E; q++) a.out[at(q)] = x[q];
        }
    }

    // ---------------------------------------------------- step counter (last CTA)
    if (a.flags & F_FIN_STEP) {
        if (tid == 0) {
            __threadfence();
            const unsigned prev = atomicAdd(&a.dyn->ticket, 1u);
            last_cta = (prev == gridDim.x - 1);
        }
        __syncthreads();
        if (last_cta) {
            __threadfence();
            finalize<R, NT, 1>(a, sred, gridDim.x, false);
        }
    }
}

}  // namespace gpe
