/*
 * Test hook header: time-dependent user physics for a contact BEC (INTERACTIONS -1).
 *
 * Written like a user's copy of include/gpe_user_defined.h, with every hook
 * depending on the step `it`:
 *   gpe_external_potential  harmonic trap whose centre moves along x:
 *                           x0(t) = d_user_param[4] sin(d_user_param[5] t), t = d_t0 + it d_dt
 *   gpe_dEDFdn / gpe_EDF    contact interaction with a modulated scattering length
 *                           a(t) = d_user_param[A_SCAT] (1 + d_user_param[6] cos(d_user_param[5] t))
 *   gpe_modify_psi          a norm-preserving phase kick exp(i k(it) (ix - NX/2)),
 *                           k(it) = d_user_param[7] sin(2 pi it / 16)
 */
#ifndef GPE_TEST_MOVING_TRAP_KICK_H
#define GPE_TEST_MOVING_TRAP_KICK_H

#include <cuComplex.h>
#include <math.h>
#include <sys/types.h>

typedef enum { OMEGA_X, OMEGA_Y, OMEGA_Z, A_SCAT, SHIFT_AMP, DRIVE_FREQ, A_MOD, KICK } user_params_t;

inline __device__ double hook_time(uint it) { return d_t0 + it * d_dt; }

inline __device__ double hook_scattering_length(uint it)
{
    return d_user_param[A_SCAT] * (1.0 + d_user_param[A_MOD] * cos(d_user_param[DRIVE_FREQ] * hook_time(it)));
}

inline __device__ cuDoubleComplex gpe_modify_psi(uint ix, uint iy, uint iz, uint it, cuDoubleComplex psi)
{
    const double k = d_user_param[KICK] * sin(2.0 * M_PI * (double)it / 16.0);
    const double x = (double)ix - 1.0 * (NX / 2);
    double s, c;
    sincos(k * x, &s, &c);
    return make_cuDoubleComplex(cuCreal(psi) * c - cuCimag(psi) * s, cuCreal(psi) * s + cuCimag(psi) * c);
}

inline __device__ double gpe_EDF(double rho, uint it)
{
    return 2.0 * M_PI * hook_scattering_length(it) * rho * rho;
}

inline __device__ double gpe_dEDFdn(double rho, uint it)
{
    return 4.0 * M_PI * hook_scattering_length(it) * rho;
}

inline __device__ double gpe_external_potential(uint ix, uint iy, uint iz, uint it)
{
    const double x0 = d_user_param[SHIFT_AMP] * sin(d_user_param[DRIVE_FREQ] * hook_time(it));
    const double x = (double)ix - 1.0 * (NX / 2) - x0;
    const double y = (double)iy - 1.0 * (NY / 2);
    const double z = (double)iz - 1.0 * (NZ / 2);
    const double wx = d_user_param[OMEGA_X], wy = d_user_param[OMEGA_Y], wz = d_user_param[OMEGA_Z];
    return 0.5 * (wx * wx * x * x + wy * wy * y * y + wz * wz * z * z);
}

#endif
