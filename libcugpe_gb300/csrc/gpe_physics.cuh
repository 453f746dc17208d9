// Per-point physics of the split-step evolution: density, external
// potential, energy-density functionals and the exp(c3 V) phase factor.
//
// Restates the reference hooks, which are compile-time inline functions in
// the reference (dev/gpe_user_defined.h) and are selected here at run time:
//   gpe_density            dev/gpe_engine.cu:600-603        rho = Gamma |psi|^2
//   gpe_external_potential dev/gpe_user_defined.h:488-513   harmonic trap
//   gpe_dEDFdn / gpe_EDF   dev/gpe_user_defined.h:118-135   unitary Fermi gas (INTERACTIONS 0)
//                          dev/gpe_user_defined.h:196-243   BEC side of the crossover (1)
//                          dev/gpe_user_defined.h:305-322   contact BEC (-1)
//                          dev/gpe_user_defined.h:380-438   dipolar BEC (-2): local part 0, contact and
//                                                           dipolar parts in the k-space kernel
//   cplxExp(c3 * V)        dev/gpe_complex.cuh:167-175, dev/gpe_engine.cu:738
// The trap is tabulated per axis on the host, V(ix,iy,iz) = vx[ix] + vy[iy]
// + vz[iz], with the same evaluation order as the reference expression.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include "gpe_fft.cuh"

namespace gpe {

enum : int { INTER_DIP = -2, INTER_BEC = -1, INTER_UFG = 0, INTER_BECSIDE = 1 };
enum : int { PHASE_GENERAL = 0, PHASE_ROTATE = 1, PHASE_DECAY = 2 };

// 3 pi^2 as the reference's left-to-right constant fold (3.0*M_PI)*M_PI
#define GPE_3PI2 29.608813203268074

template <typename R>
struct Phys {
    int inter;        // functional
    int phase_mode;   // which parts of c3 are non-zero
    R gamma;          // 1 particles, 2 dimers
    R c3x, c3y;       // c3 = Gamma dt/2 / (-beta + i alpha)   (dev/gpe_engine.cu:177-181)
    R c3y_pi;         // c3y / pi (the rotation angle in units of pi)
    R c_bec;          // (4 pi) a, contact BEC mean field
    R a_scat;         // scattering length (user param A_SCAT)
    R qf_eps;         // 1e-12 (dev/gpe_engine.cuh:53)
    R qf_g;           // quantum friction coefficient / Gamma
    R wz8;            // Weizsaecker weight / 8
    R wz_eps;         // density regularisation of the Weizsaecker potential
    R a_dip;          // dipolar length (user param A_DIP, INTERACTIONS -2)
    R nxyz;           // lattice points (FFT normalisation of the dipolar kernel)
};

__device__ __forceinline__ double gexp(double x) { return exp(x); }
__device__ __forceinline__ float gexp(float x) { return expf(x); }
__device__ __forceinline__ void gsincos(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ void gsincos(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void gsincospi(double x, double* s, double* c) { sincospi(x, s, c); }
__device__ __forceinline__ void gsincospi(float x, float* s, float* c) { sincospif(x, s, c); }
__device__ __forceinline__ double gcbrt(double x) { return cbrt(x); }
__device__ __forceinline__ float gcbrt(float x) { return cbrtf(x); }
__device__ __forceinline__ double gpow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float gpow(float x, float y) { return powf(x, y); }

template <typename R> __device__ __forceinline__ R density(const Phys<R>& p, C2<R> v) {
    return p.gamma * (v.x * v.x + v.y * v.y);
}

// variational derivative of the energy density functional
template <typename R> __device__ __forceinline__ R dEDFdn(const Phys<R>& p, R rho) {
    if (p.inter == INTER_BEC) return p.c_bec * rho;
    if (p.inter == INTER_DIP) return (R)0;  // dev/gpe_user_defined.h:400-404
    if (p.inter == INTER_UFG) {
        // 0.37 (3 pi^2 rho)^{2/3} / 2 ; (x^{1/3})^2 replaces pow(x, 2/3)
        const R t = gcbrt((R)GPE_3PI2 * rho);
        return (R)0.185 * (t * t);
    }
    // BEC side of the crossover (dev/gpe_user_defined.h:214-243)
    const R XI = (R)0.37, CT = (R)0.901, a = p.a_scat;
    if (rho > (R)1e-15) {
        const R kF = gcbrt((R)GPE_3PI2 * rho);
        const R eF = (R)0.5 * kF * kF;
        const R x = (R)1.0 / (a * kF);
        const R D = (XI + x * ((R)1.0 + CT) + (R)(3.0 * M_PI) * XI * x * x);
        return XI * eF * (XI + (R)0.8 * x) / D
             + (R)0.2 * XI * eF * (XI + x) * x * (((R)1.0 + CT) + (R)(6.0 * M_PI) * XI * x) / (D * D)
             - (R)1.0 / ((R)2.0 * a * a);
    }
    return -(R)1.0 / ((R)2.0 * a * a);
}

// energy density functional (only used by the energy reduction, in FP64)
__device__ __forceinline__ double EDF(const Phys<double>& p, double rho) {
    if (p.inter == INTER_BEC || p.inter == INTER_DIP) return 0.5 * p.c_bec * rho * rho;  // 2 pi a rho^2
    if (p.inter == INTER_UFG) return 0.37 * 0.6 * rho * pow(GPE_3PI2 * rho, 2.0 / 3.0) / 2.;
    const double XI = 0.37, CT = 0.901, a = p.a_scat;
    const double kF = cbrt(GPE_3PI2 * rho);
    const double eF = 0.5 * kF * kF;
    const double x = (kF > 2.2250738585072014e-308) ? 1.0 / (a * kF) : 1.7976931348623157e308;
    return 0.6 * eF * rho * XI * (XI + x) / (XI + x * (1.0 + CT) + 3.0 * M_PI * XI * x * x) - rho / (2.0 * a * a);
}

// sin and cos of the rotation angle c3y V.  FP32: sincospif of the angle in units of pi (its argument
// reduction is exact and short, and the kernels keep no local-memory reduction table; measured 2% faster
// at 128^3, FP32 rounding of the angle as before); FP64: sincos (sincospi measured slower there).
template <typename R> __device__ __forceinline__ void rotation(const Phys<R>& p, R V, R* s, R* c) {
    if constexpr (sizeof(R) == 4) gsincospi(p.c3y_pi * V, s, c);
    else gsincos(p.c3y * V, s, c);
}

// exp(c3 * V)
template <typename R> __device__ __forceinline__ C2<R> phase(const Phys<R>& p, R V) {
    C2<R> e;
    if (p.phase_mode == PHASE_ROTATE) {
        rotation(p, V, &e.y, &e.x);
    } else if (p.phase_mode == PHASE_DECAY) {
        e.x = gexp(p.c3x * V);
        e.y = (R)0;
    } else {
        R s, c;
        const R t = gexp(p.c3x * V);
        rotation(p, V, &s, &c);
        e.x = t * c;
        e.y = t * s;
    }
    return e;
}

}  // namespace gpe
