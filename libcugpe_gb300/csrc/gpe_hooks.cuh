// User hooks compiled into the pass kernels (a library built with a hook
// header, GPE_USER_HOOKS = "path/to/header.h").
//
// The hooks keep the reference's signatures (dev/gpe_user_defined.h), which
// take no engine argument: the run-time values they read (d_user_param,
// d_nx, d_dt, ...) are therefore names of a per-CTA shared-memory context that
// every pass kernel fills from its own arguments before any hook runs.  So
// engines with different parameters can run at the same time, and a kernel
// reads the values of the engine that launched it.
#pragma once

#ifdef GPE_USER_HOOKS
#include <cuComplex.h>
#include <sys/types.h>

namespace gpe {
struct HookCtx {
    double up[32];               // user parameters (gpe_set_user_params)
    unsigned int nx, ny, nz, pad;
    double dt, t0, npart;
};
}  // namespace gpe

static __shared__ gpe::HookCtx gpe_hook_ctx;

#define d_user_param (gpe_hook_ctx.up)
#define d_nx (gpe_hook_ctx.nx)
#define d_ny (gpe_hook_ctx.ny)
#define d_nz (gpe_hook_ctx.nz)
#define d_dt (gpe_hook_ctx.dt)
#define d_t0 (gpe_hook_ctx.t0)
#define d_npart (gpe_hook_ctx.npart)
#ifndef NX
#define NX d_nx
#endif
#ifndef NY
#define NY d_ny
#endif
#ifndef NZ
#define NZ d_nz
#endif

#include GPE_USER_HOOKS
#ifndef INTERACTIONS
#define INTERACTIONS 0  // a hook header that does not name its functional: unitary Fermi gas
#endif

#endif  // GPE_USER_HOOKS
