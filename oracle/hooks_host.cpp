// Host build of a user hook header (include/gpe_user_defined.h or a user's
// copy), so that the CPU oracle evaluates the same user physics as a hook
// build of the engine.
//
// TEST INFRASTRUCTURE ONLY.  The header is compiled here exactly as written;
// the run-time names it reads (d_user_param, d_nx, ..., NX) become this
// file's host variables, and the device rounding intrinsic __dadd_rn becomes a
// plain addition (this file is compiled without floating-point contraction, so
// the sum is rounded the same way).  GPE_USER_HOOKS names the header.
#include <cuComplex.h>
#include <math.h>
#include <sys/types.h>

static double hk_up[32];
static unsigned int hk_nx, hk_ny, hk_nz;
static double hk_dt, hk_t0, hk_npart;

#define d_user_param hk_up
#define d_nx hk_nx
#define d_ny hk_ny
#define d_nz hk_nz
#define d_dt hk_dt
#define d_t0 hk_t0
#define d_npart hk_npart
#ifndef NX
#define NX hk_nx
#endif
#ifndef NY
#define NY hk_ny
#endif
#ifndef NZ
#define NZ hk_nz
#endif
#define __dadd_rn(a, b) ((a) + (b))

#include GPE_USER_HOOKS
#ifndef INTERACTIONS
#define INTERACTIONS 0  // a hook header that does not name its functional: unitary Fermi gas
#endif

extern "C" {

int hooks_interactions(void) { return INTERACTIONS; }

void hooks_set(const double* up, int n, unsigned nx, unsigned ny, unsigned nz, double dt, double t0,
               double npart) {
    for (int i = 0; i < 32; i++) hk_up[i] = (i < n) ? up[i] : 0.0;
    hk_nx = nx; hk_ny = ny; hk_nz = nz;
    hk_dt = dt; hk_t0 = t0; hk_npart = npart;
}

double hooks_vext(unsigned ix, unsigned iy, unsigned iz, unsigned it) {
    return gpe_external_potential(ix, iy, iz, it);
}

double hooks_dedf(double rho, unsigned it) { return gpe_dEDFdn(rho, it); }

double hooks_edf(double rho, unsigned it) { return gpe_EDF(rho, it); }

void hooks_modify(unsigned ix, unsigned iy, unsigned iz, unsigned it, double* re, double* im) {
    const cuDoubleComplex p = gpe_modify_psi(ix, iy, iz, it, make_cuDoubleComplex(*re, *im));
    *re = cuCreal(p);
    *im = cuCimag(p);
}

}  // extern "C"
