/*
 * User hooks of the split-step engine: the physics a user replaces.
 *
 * The reference keeps its physics in compile-time __device__ functions of
 * dev/gpe_user_defined.h, selected by INTERACTIONS and VEXT and edited by the
 * user.  This header keeps those hooks under the same names and signatures:
 *
 *   gpe_modify_psi(ix, iy, iz, it, psi)        dev/gpe_user_defined.h:81-85
 *   gpe_external_potential(ix, iy, iz, it)     dev/gpe_user_defined.h:488-513 (VEXT 0), 520-558 (VEXT 1)
 *   gpe_dEDFdn(rho, it), gpe_EDF(rho, it)      dev/gpe_user_defined.h:118-135 (INTERACTIONS 0),
 *                                              305-322 (INTERACTIONS -1)
 *
 * and evaluates them where the reference does (dev/gpe_engine.cu:733-735,
 * 758-760, 789, 794, 829-834, 855-861, 999-1002, 1618-1641): the potential and
 * mean field of the predictor at step `it`, of the corrector at `it + 1`;
 * gpe_modify_psi on psi_n, at `it`, wherever a step reads psi_n (predictor and
 * corrector), after the pending imaginary-time normalisation.
 *
 * How to use it.  Copy this file, edit the hooks, and build a library whose
 * pass kernels call them:
 *
 *     python -m libcugpe_gb300.build --hooks my_hooks.h --name mine -DVEXT=1
 *
 * gives libcugpe_gb300/_lib/libgpe_gb300_mine.so with the same C ABI
 * (include/gpe_gb300.h) and drop-in API (include/gpe_engine.h); link a driver
 * against it, or open it from Python with Engine(..., library=path).  The
 * library built without --hooks does not use this file: it runs the built-in
 * physics selected at run time, which the default hooks below reproduce.
 *
 * Run-time values the hooks may read, under the reference's names (provided by
 * the engine for the engine that runs the kernel; do not declare them):
 *   d_user_param[i]         the values of gpe_set_user_params (zero beyond `size`)
 *   d_nx, d_ny, d_nz        lattice sides; NX, NY, NZ are the same unless given with -D
 *   d_dt, d_t0, d_npart     time step, initial time, particle number
 *   `it`                    step counter since gpe_set_psi / gpe_set_time: time = d_t0 + it * d_dt
 *
 * Precision: the hooks compute in FP64 in both precision forms; the FP32-mixed
 * form rounds their results to FP32.  The functional of the build (INTERACTIONS,
 * default 0) must match the `interactions` argument of gpe_gb_create, which
 * sets Gamma (1 for particles, 2 for dimers); gpe_gb_create refuses a mismatch.
 * Built-in extensions that bypass these hooks: the dipolar k-space kernel, the
 * time-sliced additive potential (added to gpe_external_potential) and the
 * optimal-control problem (refused in a hook build).
 */
#ifndef GPE_USER_DEFINED_H
#define GPE_USER_DEFINED_H

#include <cuComplex.h>
#include <math.h>
#include <sys/types.h>

#ifndef INTERACTIONS
#define INTERACTIONS 0
#endif
#ifndef VEXT
#define VEXT 0
#endif

/* ----------------------------------------------------------- wavefunction */

/* Changes psi_n before each step (phase imprinting, a moving absorber, ...).
 * Called wherever a step reads psi_n; it must not change the norm. */
inline __device__ cuDoubleComplex gpe_modify_psi(uint ix, uint iy, uint iz, uint it, cuDoubleComplex psi)
{
    return psi;
}

/* --------------------------------------------------------------- functional */

#if (INTERACTIONS == 0) /* unitary Fermi gas of dimers */

typedef enum { OMEGA_X, OMEGA_Y, OMEGA_Z, A_SCAT } user_params_t;

/* E = 0.37 (3/5) rho (3 pi^2 rho)^{2/3} / 2 */
inline __device__ double gpe_EDF(double rho, uint it)
{
    return 0.37 * 0.6 * rho * pow(29.608813203268074 * rho, 2.0 / 3.0) / 2.;
}

/* dE/drho = 0.37 (3 pi^2 rho)^{2/3} / 2, written as 0.185 (cbrt(3 pi^2 rho))^2 */
inline __device__ double gpe_dEDFdn(double rho, uint it)
{
    const double t = cbrt(29.608813203268074 * rho);
    return 0.185 * (t * t);
}

#elif (INTERACTIONS == -1) /* contact BEC */

typedef enum { OMEGA_X, OMEGA_Y, OMEGA_Z, A_SCAT } user_params_t;

/* E = 2 pi a rho^2 (= g rho^2 / 2) */
inline __device__ double gpe_EDF(double rho, uint it)
{
    const double a = d_user_param[A_SCAT];
    return 0.5 * ((4 * M_PI * a) * rho) * rho;
}

/* dE/drho = 4 pi a rho */
inline __device__ double gpe_dEDFdn(double rho, uint it)
{
    const double a = d_user_param[A_SCAT];
    return (4 * M_PI * a) * rho;
}

#else
#error "gpe_user_defined.h: write gpe_EDF / gpe_dEDFdn for this INTERACTIONS value"
#endif

/* -------------------------------------------------------- external potential */

#if (VEXT == 0) /* harmonic trap, frequencies in d_user_param[OMEGA_X..OMEGA_Z] */

inline __device__ double gpe_external_potential(uint ix, uint iy, uint iz, uint it)
{
    const double wx = d_user_param[OMEGA_X], wy = d_user_param[OMEGA_Y], wz = d_user_param[OMEGA_Z];
    const double x = (double)ix - 1.0 * (NX / 2);
    const double y = (double)iy - 1.0 * (NY / 2);
    const double z = (double)iz - 1.0 * (NZ / 2);
    /* per-axis terms summed with separate roundings (no fused multiply-add), as the built-in trap
     * table sums them */
    return __dadd_rn(__dadd_rn(0.5 * x * x * wx * wx, 0.5 * y * y * wy * wy), 0.5 * z * z * wz * wz);
}

#elif (VEXT == 1) /* Woods-Saxon tube along z: V0 (1 - 1/(1 + exp((r - R)/a))), r^2 = x^2 + y^2 */

typedef enum { V_0, A, R } potential_params_t;

inline __device__ double gpe_external_potential(uint ix, uint iy, uint iz, uint it)
{
    const double v0 = d_user_param[V_0];
    const double width = d_user_param[A];
    const double radius = d_user_param[R];
    const double x = (double)ix - 1.0 * (NX / 2);
    const double y = (double)iy - 1.0 * (NY / 2);
    const double r = sqrt(x * x + y * y);
    return v0 * (1. - 1. / (1 + exp((r - radius) / width)));
}

#else
#error "gpe_user_defined.h: write gpe_external_potential for this VEXT value"
#endif

#endif /* GPE_USER_DEFINED_H */
