// The reference's single-global-engine API (KKobuszewski/libcugpe
// dev/gpe_engine.h:299-558) on top of the handle-based C ABI.
//
// Same C++ signatures, so the mangled symbols match the reference library
// and its drivers link unchanged.  The reference's compile-time lattice and
// functional (NX/NY/NZ/INTERACTIONS) become run-time settings: gpe_configure()
// (which gpe_engine.h calls automatically when the macros are defined), or
// the GPE_NX/GPE_NY/GPE_NZ/GPE_INTERACTIONS/GPE_PRECISION environment
// variables.  Like the reference (dev/gpe_engine.cu:43), there is one engine
// per process and no locking.
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>

#include "../../include/gpe_engine.h"

static gpe_gb_engine* g_engine = nullptr;
static int g_nx = 0, g_ny = 0, g_nz = 0, g_inter = INT_MIN, g_prec = -1;

static int env_int(const char* name, int dflt) {
    const char* v = getenv(name);
    return (v && *v) ? atoi(v) : dflt;
}

static void lattice(int* nx, int* ny, int* nz) {
    *nx = g_nx ? g_nx : env_int("GPE_NX", 64);
    *ny = g_ny ? g_ny : env_int("GPE_NY", *nx);
    *nz = g_nz ? g_nz : env_int("GPE_NZ", *ny);
}

int gpe_configure(int nx, int ny, int nz, int interactions, int precision) {
    g_nx = nx;
    g_ny = ny;
    g_nz = nz;
    g_inter = interactions;
    g_prec = precision;
    return 0;
}

void gpe_get_lattice(int* _nx, int* _ny, int* _nz) { lattice(_nx, _ny, _nz); }

// nthreads sets the reference's 1D launch shape (dev/gpe_engine.cu:308-309);
// this engine sizes its own launches and ignores it.
int gpe_create_engine(double alpha, double beta, double dt, double npart, int nthreads) {
    (void)nthreads;
    if (g_engine) {
        gpe_gb_destroy(g_engine);
        g_engine = nullptr;
    }
    int nx, ny, nz;
    lattice(&nx, &ny, &nz);
    const int inter = (g_inter != INT_MIN) ? g_inter : env_int("GPE_INTERACTIONS", 0);
    const int prec = (g_prec >= 0) ? g_prec : env_int("GPE_PRECISION", GPE_PRECISION_FP64);
    return gpe_gb_create(&g_engine, nx, ny, nz, inter, prec, alpha, beta, dt, npart);
}

int gpe_destroy_engine() {
    if (!g_engine) return GPE_ERR_NO_ENGINE;
    const int rc = gpe_gb_destroy(g_engine);
    g_engine = nullptr;
    return rc;
}

int gpe_change_alpha_beta(double alpha, double beta) { return gpe_gb_change_alpha_beta(g_engine, alpha, beta); }
int gpe_set_rte_evolution() { return gpe_gb_change_alpha_beta(g_engine, 1.0, 0.0); }
int gpe_set_ite_evolution() { return gpe_gb_change_alpha_beta(g_engine, 0.0, 1.0); }
int gpe_set_time(double t0) { return gpe_gb_set_time(g_engine, t0); }
int gpe_set_user_params(int size, double* params) { return gpe_gb_set_user_params(g_engine, size, params); }
int gpe_set_quantum_friction_coeff(double q) { return gpe_gb_set_quantum_friction_coeff(g_engine, q); }
int gpe_set_psi(double t, cuCplx* psi) { return gpe_gb_set_psi(g_engine, t, reinterpret_cast<const double*>(psi)); }
int gpe_get_psi(double* t, cuCplx* psi) { return gpe_gb_get_psi(g_engine, t, reinterpret_cast<double*>(psi)); }
int gpe_get_density(double* t, double* density) { return gpe_gb_get_density(g_engine, t, density); }
int gpe_normalize_psi() { return gpe_gb_normalize_psi(g_engine); }
int gpe_get_norm(double* norm) { return gpe_gb_get_norm(g_engine, norm); }
int gpe_evolve_qf(int nt, double* mu) { return gpe_gb_evolve_qf(g_engine, nt, mu); }
int gpe_energy(double* t, double* ekin, double* eint, double* eext) {
    return gpe_gb_energy(g_engine, t, ekin, eint, eext);
}

// dev/gpe_engine.cu:1021-1025: a stub in the reference too
int gpe_evolve(int nt) {
    (void)nt;
    printf("Function not implemented!\n");
    return GPE_SUCCESS;
}

void gpe_print_potential_type() { printf("%s\n", "HARMONIC POTENTIAL\n"); }

int gpe_set_vortex(const double x0, const double y0, const int8_t Q) { return gpe_gb_set_vortex(g_engine, x0, y0, Q); }
int gpe_get_phase(double* h_phase) { return gpe_gb_get_phase(g_engine, h_phase); }
int gpe_set_phase(double* h_phase) { return gpe_gb_set_phase(g_engine, h_phase); }
int gpe_evolve_vortex(int nt, double* mu) { return gpe_gb_evolve_vortex(g_engine, nt, mu, 1); }
int gpe_evolve_vortex2(int nt, double* mu) { return gpe_gb_evolve_vortex(g_engine, nt, mu, 2); }
int gpe_evolve_vortex3(int nt, double* mu) { return gpe_gb_evolve_vortex(g_engine, nt, mu, 3); }
int gpe_evolve_enforced_phase(int nt, double* mu) { return gpe_gb_evolve_enforced_phase(g_engine, nt, mu); }

// Reference entry points outside the split-step evolution of this engine.
int gpe_get_currents(double* t, double* jx, double* jy, double* jz) {
    if (!g_engine) return GPE_ERR_NO_ENGINE;
    return gpe_gb_get_currents(g_engine, t, jx, jy, jz);
}
int gpe_evolve_dipolar(int nt) { return gpe_gb_evolve_dipolar(g_engine, nt, nullptr); }
int gpe_evolve_dipolar(int nt, double* mu) { return gpe_gb_evolve_dipolar(g_engine, nt, mu); }
// The reference sums rho(k) Vpp(k) rho(-k) in k space, indexing -k as n - i, which for the
// i = 0 planes reads past the transform (dev/gpe_engine.cu:1725); the intended value equals the
// real-space sum of gpe_energy_dipolar2 (Parseval), which both entry points return.
int gpe_energy_dipolar(double* t, double* edip) { return gpe_gb_energy_dipolar(g_engine, t, edip); }
int gpe_energy_dipolar2(double* t, double* edip) { return gpe_gb_energy_dipolar(g_engine, t, edip); }
