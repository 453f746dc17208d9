/*
 * Drop-in declaration of the libcugpe engine API for the GB300 engine.
 *
 * Same names, argument lists, default arguments and C++ linkage as the
 * reference header (KKobuszewski/libcugpe dev/gpe_engine.h:299-558), so a
 * driver written for the reference (e.g. test_compare/gpe_imag.c) compiles
 * unchanged with g++ and links against libgpe_gb300.so instead of the
 * reference's static library.  The itanium-mangled symbols match the
 * reference's (_Z17gpe_create_engineddddi, _Z13gpe_evolve_qfiPd, ...).
 *
 * The reference fixes the lattice and the functional at compile time with
 * -DNX -DNY -DNZ -DINTERACTIONS (dev/Makefile:44-46).  Drivers built with
 * those macros keep working: this header then registers them with the
 * engine before main() through gpe_configure().  Without the macros the
 * lattice comes from gpe_configure() or the GPE_NX/GPE_NY/GPE_NZ/
 * GPE_INTERACTIONS/GPE_PRECISION environment variables.
 *
 * The reference's other evolution and observable entry points (vortex
 * imprinting, phase enforcing, currents, dipolar evolution and energy) are
 * implemented on the same engine.  gpe_timing.h (b_t/e_t) and gpe_io.h
 * (gpe_save_info/gpe_get_info, save_info/get_info) stand in for the
 * reference's driver-side headers of the same names.
 */
#ifndef GPE_ENGINE_GB300_DROPIN_H
#define GPE_ENGINE_GB300_DROPIN_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <cuComplex.h>
#include "gpe_gb300.h"
#include "gpe_timing.h" /* b_t() / e_t(), as the reference engine header includes its timers */

typedef int gpe_result_t;
typedef unsigned int uint;
typedef cuDoubleComplex cuCplx;

#define GPE_SUCCESS 0
#define CUDA_ERRORS_BASE 0
#define CUFFT_ERRORS_BASE 100

/* user parameter slots (dev/gpe_user_defined.h:101; dipolar BEC :366) */
#if defined(INTERACTIONS) && (INTERACTIONS == -2)
typedef enum { OMEGA_X, OMEGA_Y, OMEGA_Z, A_CON, A_DIP } user_params_t;
#else
typedef enum { OMEGA_X, OMEGA_Y, OMEGA_Z, A_SCAT } user_params_t;
#endif

static inline const char* gpe_get_error_string(gpe_result_t r) { return gpe_gb_error_string(r); }

/* dev/gpe_engine.h:263-273 */
#define gpe_exec(cmd, ierr)                                                                  \
    {                                                                                        \
        ierr = cmd;                                                                          \
        if (ierr) {                                                                          \
            fprintf(stderr, "error: cannot execute: %s\t", #cmd);                            \
            fprintf(stderr, "file=`%s`, line=%d\t", __FILE__, __LINE__);                     \
            fprintf(stderr, "Error=%d (%s)\nExiting!\n", ierr, gpe_get_error_string(ierr)); \
            exit(EXIT_FAILURE);                                                              \
        }                                                                                    \
    }

/* Run-time stand-in for the reference's compile-time NX/NY/NZ/INTERACTIONS
 * (precision: GPE_PRECISION_FP64 or GPE_PRECISION_FP32).  Returns 0. */
int gpe_configure(int nx, int ny, int nz, int interactions, int precision);

void gpe_get_lattice(int* _nx, int* _ny, int* _nz);
int gpe_create_engine(double alpha, double beta, double dt, double npart, int nthreads = 1024);
int gpe_change_alpha_beta(double alpha, double beta);
int gpe_set_rte_evolution();
int gpe_set_ite_evolution();
int gpe_set_time(double t0);
int gpe_set_user_params(int size, double* params);
int gpe_set_quantum_friction_coeff(double qfcoeff);
int gpe_set_vortex(const double vortex_x0, const double vortex_y0, const int8_t Q = 1);
int gpe_get_phase(double* h_phase = NULL);
int gpe_set_phase(double* h_phase);
int gpe_set_psi(double t, cuCplx* psi);
int gpe_get_psi(double* t, cuCplx* psi);
int gpe_get_density(double* t, double* density);
int gpe_get_currents(double* t, double* jx, double* jy, double* jz);
int gpe_normalize_psi();
int gpe_get_norm(double* norm);
int gpe_evolve(int nt);
int gpe_evolve_qf(int nt, double* chemical_potential = NULL);
int gpe_evolve_vortex(int nt, double* chemical_potential = NULL);
int gpe_evolve_vortex2(int nt, double* chemical_potential = NULL);
int gpe_evolve_vortex3(int nt, double* chemical_potential = NULL);
int gpe_evolve_enforced_phase(int nt, double* chemical_potential = NULL);
int gpe_evolve_dipolar(int nt);
int gpe_evolve_dipolar(int nt, double* chemical_potential);
int gpe_energy_dipolar(double* t, double* edip);
int gpe_energy_dipolar2(double* t, double* edip);
int gpe_energy(double* t, double* ekin, double* eint, double* eext);
int gpe_destroy_engine();
void gpe_print_potential_type();

#if defined(NX) && defined(NY) && defined(NZ)
#ifndef INTERACTIONS
#define INTERACTIONS 0
#endif
#ifndef GPE_PRECISION
#define GPE_PRECISION GPE_PRECISION_FP64
#endif
static const int gpe__lattice_registered = gpe_configure(NX, NY, NZ, INTERACTIONS, GPE_PRECISION);
#endif

#endif
