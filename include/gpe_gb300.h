/*
 * C ABI of the GB300 split-step GPE engine (libgpe_gb300.so).
 *
 * Plain pointers and sizes only.  Each entry point is a handle-based form of
 * one reference engine call (KKobuszewski/libcugpe, dev/gpe_engine.h); the
 * reference's own C++-linkage, single-global-engine signatures are declared
 * in gpe_engine.h and implemented on top of these.
 *
 * Wavefunctions cross the boundary as interleaved complex128 (the reference's
 * cuDoubleComplex), C order [nx][ny][nz] with z fastest, in host memory
 * (pinned or pageable), exactly as gpe_set_psi / gpe_get_psi take them.
 *
 * Return codes: 0 on success; a positive value is the cudaError_t of the
 * failing CUDA call (as the reference's cuErrCheck, dev/gpe_engine.h:201-209);
 * negative values are the GPE_ERR_* codes below (-9 is the reference's
 * "too many user parameters", dev/gpe_engine.cu:428).
 */
#ifndef GPE_GB300_H
#define GPE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPE_ERR_TOO_MANY_PARAMS (-9)   /* dev/gpe_engine.cu:428 */
#define GPE_ERR_LATTICE (-10)          /* side not a power of two in [8, 512] */
#define GPE_ERR_NO_ENGINE (-11)        /* null handle / engine not created */
#define GPE_ERR_ARGUMENT (-12)         /* null pointer or bad value */
#define GPE_ERR_FUNCTIONAL (-13)       /* unknown interactions code */
#define GPE_ERR_NOALLOC_SIZE (-14)     /* more points than gpe_gb_norm_noalloc's scratch serves */
#define GPE_ERR_IO (-15)               /* a .dftc / .dftc.info file could not be opened, read or written */
#define GPE_ERR_NOT_IMPLEMENTED (-98)  /* reference entry point outside this engine */

#define GPE_PRECISION_FP64 0 /* plain FP64 drop-in */
#define GPE_PRECISION_FP32 1 /* FP32 field/FFT/phases, FP64 tables and reductions */

typedef struct gpe_gb_engine gpe_gb_engine;

/* gpe_create_engine (dev/gpe_engine.cu:286), with the lattice and functional
 * that the reference fixes at compile time (NX/NY/NZ, INTERACTIONS) given at
 * run time.  interactions: -1 contact BEC, 0 unitary Fermi gas (dimers),
 * 1 BEC side of the crossover (dimers). */
int gpe_gb_create(gpe_gb_engine** out, int nx, int ny, int nz, int interactions, int precision,
                  double alpha, double beta, double dt, double npart);
/* gpe_destroy_engine (dev/gpe_engine.cu:370) */
int gpe_gb_destroy(gpe_gb_engine* e);
/* gpe_get_lattice (dev/gpe_engine.cu:116) */
int gpe_gb_get_lattice(const gpe_gb_engine* e, int* nx, int* ny, int* nz);
/* gpe_change_alpha_beta (dev/gpe_engine.cu:389) */
int gpe_gb_change_alpha_beta(gpe_gb_engine* e, double alpha, double beta);
/* gpe_set_time (dev/gpe_engine.cu:417) */
int gpe_gb_set_time(gpe_gb_engine* e, double t0);
/* gpe_set_user_params (dev/gpe_engine.cu:426): copies `size` values, zero-fills the rest */
int gpe_gb_set_user_params(gpe_gb_engine* e, int size, const double* params);
/* gpe_set_quantum_friction_coeff (dev/gpe_engine.cu:435) */
int gpe_gb_set_quantum_friction_coeff(gpe_gb_engine* e, double qfcoeff);
/* Weizsaecker gradient term of weight lambda (no reference counterpart: the
 * reference declares gpe_gradient_corrections, dev/gpe_user_defined.h:158,
 * but never calls it).  Adds E_W = (lambda/8) sum |grad rho|^2 / rho to the
 * functional, i.e. V_W = (lambda/8) (|grad rho|^2/rho^2 - 2 lap(rho)/rho)
 * (lattice units, hbar = m = 1, rho = Gamma |psi|^2), with spectral
 * derivatives of psi and rho replaced by rho + eps in both denominators, so
 * V_W fades out where rho << eps (the far tails, whose derivatives are
 * round-off); eps <= 0 selects 1e-2 npart / (nx ny nz).  Like the friction
 * potential, V_W is evaluated once per step at the step's initial psi and
 * enters both halves of the step.  That explicit treatment of a term that
 * stiffens like k^2 is stable for dt |lambda| 3 pi^2 <= 0.4, so while the
 * term is on a step of dt runs as m = ceil(dt |lambda| 3 pi^2 / 0.4) equal
 * sub-steps (evolve(nt) still advances nt dt; the time-sliced potential's
 * steps_per_slice still counts steps of dt).  lambda = 0 turns it off.
 * FP32 form: x side <= 256. */
int gpe_gb_set_weizsacker(gpe_gb_engine* e, double lambda, double eps);
/* gpe_set_psi (dev/gpe_engine.cu:694): psi = 2*nx*ny*nz doubles */
int gpe_gb_set_psi(gpe_gb_engine* e, double t, const double* psi);
/* gpe_get_psi (dev/gpe_engine.cu:705) */
int gpe_gb_get_psi(gpe_gb_engine* e, double* t, double* psi);
/* gpe_get_density (dev/gpe_engine.cu:669): density = nx*ny*nz doubles */
int gpe_gb_get_density(gpe_gb_engine* e, double* t, double* density);
/* gpe_get_currents (dev/gpe_engine.cu:1856-1904): probability currents
 * j_a = Re(conj(psi) IFFT(k_a/(Gamma n) FFT psi)) along x, y, z into three
 * host arrays of n doubles (C order). */
int gpe_gb_get_currents(gpe_gb_engine* e, double* t, double* jx, double* jy, double* jz);
/* gpe_get_norm (dev/gpe_engine.cu:679) */
int gpe_gb_get_norm(gpe_gb_engine* e, double* norm);
/* gpe_normalize_psi (dev/gpe_engine.cu:648) */
int gpe_gb_normalize_psi(gpe_gb_engine* e);
/* gpe_evolve_qf (dev/gpe_engine.cu:1030); chemical_potential may be NULL */
int gpe_gb_evolve_qf(gpe_gb_engine* e, int nt, double* chemical_potential);
/* gpe_energy (dev/gpe_engine.cu:1669) */
int gpe_gb_energy(gpe_gb_engine* e, double* t, double* ekin, double* eint, double* eext);

/* gpe_set_vortex (dev/gpe_engine.cu:465): vortex line along z through
 * (x0, y0) in lattice offsets from the box centre, charge q. */
int gpe_gb_set_vortex(gpe_gb_engine* e, double x0, double y0, int q);
/* gpe_get_phase (dev/gpe_engine.cu:572): phase = arg psi kept for
 * gpe_gb_evolve_enforced_phase; copied to `phase` (nx*ny*nz doubles) if not NULL. */
int gpe_gb_get_phase(gpe_gb_engine* e, double* phase);
/* gpe_set_phase (dev/gpe_engine.cu:561) */
int gpe_gb_set_phase(gpe_gb_engine* e, const double* phase);
/* gpe_evolve_vortex (method 1), gpe_evolve_vortex2 (2), gpe_evolve_vortex3 (3)
 * (dev/gpe_engine.cu:1115, 1207, 1299): the vortex phase is imposed at the
 * start of every step; method 2 leaves points with |psi| <= 1e-15 alone. */
int gpe_gb_evolve_vortex(gpe_gb_engine* e, int nt, double* chemical_potential, int method);
/* gpe_evolve_enforced_phase (dev/gpe_engine.cu:1390) */
int gpe_gb_evolve_enforced_phase(gpe_gb_engine* e, int nt, double* chemical_potential);

/* Device-resident I/O (no reference counterpart; used when the caller keeps
 * the wavefunction in GPU memory): psi is a device pointer to nx*ny*nz
 * complex128 values. */
int gpe_gb_set_psi_device(gpe_gb_engine* e, double t, const void* psi);
int gpe_gb_get_psi_device(gpe_gb_engine* e, double* t, void* psi);
/* The CUDA stream (cudaStream_t) this engine launches on, for callers that
 * order their own work or events against it. */
void* gpe_gb_get_stream(const gpe_gb_engine* e);
/* mu of the last ITE step and the running sum of mu over all ITE steps of
 * this engine (differences of the sum give interval means; the reference
 * returns mu through gpe_evolve_qf only). */
int gpe_gb_chemical_potential(gpe_gb_engine* e, double* mu, double* mu_sum);
/* Runs all queued work to completion. */
int gpe_gb_synchronize(gpe_gb_engine* e);
/* Number of kernels this engine has launched so far. */
long long gpe_gb_kernel_launches(const gpe_gb_engine* e);
/* Measurement aid (no reference counterpart): runs nsteps steps launching
 * each fused pass directly, with CUDA events around every pass.  For pass p
 * of the step (p < min(*npass, cap)): ms[p] mean duration, bytes[p] the
 * arrays it must read and write (algorithmic bytes per launch), axis[p]
 * (0 x, 1 y, 2 z) and kind[p] (kernel class: 0 kinetic, 1 epilogue,
 * 2 Laplacian, 3 energy).  Advances psi by nsteps steps like evolve_qf. */
int gpe_gb_profile_passes(gpe_gb_engine* e, int nsteps, float* ms, double* bytes, int* axis, int* kind, int cap,
                          int* npass);
/* 1 to replay each step from a captured CUDA graph (default), 0 to launch directly. */
int gpe_gb_use_graphs(gpe_gb_engine* e, int enable);
/* Adds a time-sliced potential: `fields` holds nslices real fields of
 * nx*ny*nz doubles; step `it` uses slice min(it / steps_per_slice, nslices-1)
 * on top of the harmonic trap.  NULL removes it. */
int gpe_gb_set_potential_slices(gpe_gb_engine* e, const double* fields, int nslices, int steps_per_slice);
/* Pass layout of the step (no reference counterpart): enable = 1 (default) runs
 * real-time FP32 steps on 128 x 128 yz-planes as four launches (two yz-plane
 * passes, two x-pencil passes), enable = 0 keeps the seven pencil passes.
 * Both compute the same step (FP32 rounding apart). */
int gpe_gb_set_plane_passes(gpe_gb_engine* e, int enable);
/* Whether this library was built with a user hook header (include/gpe_user_defined.h;
 * no reference counterpart: the reference recompiles instead): *enabled = 1 and
 * *interactions = the functional the hooks were compiled for (gpe_gb_create
 * refuses any other), else *enabled = 0. */
int gpe_gb_user_hooks(int* enabled, int* interactions);
/* Measured FP64 fused multiply-add rate of the current device in TFLOP/s
 * (no reference counterpart; a measurement aid for the FP64 form's ALU
 * roofline): independent FMA chains, CUDA events, best of five launches. */
int gpe_gb_fp64_fma_rate(double* tflops);
/* Allocation-free norm (no counterpart in the reference library).
 * For callers that cannot allocate device memory when they need the norm:
 * code running while its stream is captured into a CUDA graph, applications
 * whose own pool owns all device memory, plugins in hosts that forbid
 * allocations after start-up.  Writes sum gamma |psi|^2 over n points of the
 * device array `psi` (complex128 for GPE_PRECISION_FP64, complex64 for
 * GPE_PRECISION_FP32) into the device double `norm_out`, ordered on
 * `stream` (NULL = legacy default stream), and allocates nothing: its
 * scratch is a fixed 4.25 KiB device array inside the library, held by every
 * GPU that loads the library until the process exits.  At most 2^27 points
 * (512^3); more returns GPE_ERR_NOALLOC_SIZE.  The first call on a device
 * looks up the scratch address (cudaGetSymbolAddress) and must come before
 * any stream capture; the address is kept for the life of the device's
 * primary context, so do not call this entry point on a device again after
 * cudaDeviceReset of that device.  All calls share the scratch: calls whose kernels can
 * overlap on the GPU (different streams, or host threads) race and must be
 * serialised by the caller. */
int gpe_gb_norm_noalloc(const void* psi, int precision, long long n, double gamma, double* norm_out, void* stream);
/* Batched solver (no reference counterpart; the reference runs one
 * condensate per process).  `count` independent condensates, condensate i on
 * a sides[3i] x sides[3i+1] x sides[3i+2] lattice (each side 32, 64, 128 or
 * 256) with its own time step dt[i] and npart[i]; common functional, alpha,
 * beta; FP32-mixed only.  Every fused pass of a step is one launch over all active
 * condensates, whatever their sizes, and runs of steps replay from one
 * captured CUDA graph.  Per-condensate parameters, psi and observables go
 * through the condensate's engine handle (gpe_gb_batch_engine).  All active
 * condensates must run the same step (all imaginary or all real time, all with
 * or all without quantum friction); the Weizsaecker term is not supported. */
typedef struct gpe_gb_batch gpe_gb_batch;
int gpe_gb_batch_create(gpe_gb_batch** out, int count, const int* sides, int interactions, int precision,
                        double alpha, double beta, const double* dt, const double* npart);
int gpe_gb_batch_destroy(gpe_gb_batch* b);
gpe_gb_engine* gpe_gb_batch_engine(gpe_gb_batch* b, int i);
/* Inactive condensates are skipped (e.g. once converged). */
int gpe_gb_batch_set_active(gpe_gb_batch* b, int i, int active);
/* nt steps of every active condensate (gpe_evolve_qf semantics per condensate). */
int gpe_gb_batch_evolve(gpe_gb_batch* b, int nt);
/* Imaginary-time solve of every active condensate (no reference counterpart):
 * each condensate steps until the mean of mu over an interval of `check` steps
 * differs from the previous interval's mean by less than tol[i] per step
 * (lattice units), at most max_steps steps.  The test runs on the device at the
 * end of every step and retires a converged condensate at once (its passes are
 * skipped from the next step on); the host reads the retirement flags once per
 * replayed graph.  Out: steps[i] = steps to convergence (-1: not converged),
 * mu[i] = the converged interval mean (the last step's mu if not converged).
 * The pending normalisation is applied on return, as after gpe_gb_batch_evolve. */
int gpe_gb_batch_solve(gpe_gb_batch* b, int max_steps, int check, const double* tol, int* steps, double* mu);
/* Per condensate: mu of the last ITE step and the running sum of mu. */
int gpe_gb_batch_chemical_potentials(gpe_gb_batch* b, double* mu, double* mu_sum);
long long gpe_gb_batch_kernel_launches(const gpe_gb_batch* b);
/* Optimal control (no reference counterpart): gradients of
 *   L(c) = 1 - |<psi_target|psi(T)>|^2
 * with respect to the controls c[s][k] of the time-sliced potential
 *   Vext(x, step) = trap + sum_k c[s][k] basis_k(x),  s = min(step / steps_per_slice, nslices - 1),
 * through the discrete real-time step of `engine` (FP64, real time, contact
 * BEC, no friction), by a hand-written adjoint of the step with forward
 * checkpoints every `checkpoint_every` steps (nsteps must be a multiple).
 * basis: nbasis real fields (nbasis <= 32), lattice units; controls:
 * nslices*nbasis, lattice units, row s = slice.  While the problem exists it
 * owns the engine's time-sliced potential and uses the engine's psi as
 * scratch.  Device memory: about (5 checkpoint_every + nsteps/checkpoint_every
 * + nbasis/2 + 8) complex128 fields (a segment's states and per-step
 * intermediates, the checkpoints, the basis). */
typedef struct gpe_gb_control gpe_gb_control;
int gpe_gb_control_create(gpe_gb_control** out, gpe_gb_engine* engine, int nbasis, const double* basis, int nslices,
                          int steps_per_slice, int nsteps, int checkpoint_every, const double* psi_target);
/* L(c) from psi0 (complex128 host array). */
int gpe_gb_control_loss(gpe_gb_control* c, const double* controls, const double* psi0, double* loss);
/* L(c) and dL/dc (nslices*nbasis doubles). */
int gpe_gb_control_loss_grad(gpe_gb_control* c, const double* controls, const double* psi0, double* loss,
                             double* grad);
int gpe_gb_control_destroy(gpe_gb_control* c);
/* Snapshots in the .dftc format (dev/gpe_io.h:45-166; frames as in
 * test_vortex/rte_vortex.c:64-90 with the queue of dev/gpe_queue.h:67-137).
 * open: creates `dftc_path` and nbuf (1..64) device + pinned frame buffers
 * of nx*ny*nz complex128 each, and a writer thread.  push: copies psi on the
 * engine's stream into a free frame buffer (waits while all nbuf are in
 * flight), returns with the engine free to evolve while the frame goes to
 * the host on a side stream and is appended to the file; *t = its time.
 * close: waits for every pushed frame, closes the file, frees everything;
 * *frames = frames written.  One pipeline per engine at a time. */
typedef struct gpe_gb_snapshots gpe_gb_snapshots;
int gpe_gb_snapshots_open(gpe_gb_snapshots** out, gpe_gb_engine* e, const char* dftc_path, int nbuf);
int gpe_gb_snapshots_push(gpe_gb_snapshots* s, double* t);
int gpe_gb_snapshots_close(gpe_gb_snapshots* s, long long* frames);
/* gpe_save_info (dev/gpe_io.h:45-104): writes `<dftc_path>.info`; system is
 * "bosons" or "fermions", mode "contact", "dipolar", "unitary" or "bec". */
int gpe_gb_dftc_write_info(const char* dftc_path, const char* system, const char* mode, int nx, int ny, int nz,
                           double dt, int nom, double a_scat, double aspect_ratio, double omega_x, double r0,
                           double npart, double total_time);
/* gpe_get_info (dev/gpe_io.h:130-166): reads `<dftc_path>.info`; system and
 * mode (may be NULL) receive the first word of their lines, at most len-1
 * characters; total_time (may be NULL) is 0 when the file has no such line. */
int gpe_gb_dftc_read_info(const char* dftc_path, char* system, char* mode, int len, int* nx, int* ny, int* nz,
                          double* dt, int* nom, double* a_scat, double* aspect_ratio, double* omega_x, double* r0,
                          double* npart, double* total_time);
/* gpe_evolve_dipolar (dev/gpe_engine.cu:1550-1602): nt Strang steps of the
 * dipolar BEC (interactions -2; user params OMEGA_X..Z, A_CON, A_DIP), the
 * contact + dipole-dipole potential recomputed by convolution for each half
 * step, no friction; ITE normalises each step and returns mu (may be NULL). */
int gpe_gb_evolve_dipolar(gpe_gb_engine* e, int nt, double* chemical_potential);
/* gpe_energy_dipolar2 (dev/gpe_engine.cu:1789-1809): E_dip = 1/2 sum rho vdip.
 * Also serves gpe_energy_dipolar (:1740), the same sum taken in k space. */
int gpe_gb_energy_dipolar(gpe_gb_engine* e, double* t, double* edip);
/* Radix plan of the pencil FFTs (no reference counterpart; replaces the
 * choice cuFFT makes inside the reference's Z2Z plans, dev/gpe_engine.cu:343-350):
 * 0 the default, 1 the alternative with the other point count per thread
 * (8 <-> 16; more or fewer radix stages and threads per pencil), for FP32
 * pencils of 32 to 512 points; FP64 engines and 8/16-point axes run plan 0
 * (plan 1 on an FP64 engine: GPE_ERR_ARGUMENT).  Both plans compute the same
 * transform; results differ only by FP32 rounding. */
int gpe_gb_set_fft_plan(gpe_gb_engine* e, int plan);
/* *plan: 0, 1, or 2 when the autotuner chose a plan per fused pass
 * (gpe_gb_set_fft_plan clears that choice). */
int gpe_gb_get_fft_plan(const gpe_gb_engine* e, int* plan);
/* Plan of every condensate's passes in a batch (one plan per launch). */
int gpe_gb_batch_set_fft_plan(gpe_gb_batch* b, int plan);
/* Autotuner (no reference counterpart): times nsteps steps of the engine's
 * own state for each launch configuration it can run -- FFT radix plan
 * (FP32), pass operands staged in shared memory or read where used (FP32,
 * pencils <= 128 points), and 8, 16 or 32 steps per replayed CUDA graph --
 * keeps the fastest, and puts psi, time and step counter back as they were.
 * With both radix plans timed, each fused pass of the steady schedule then
 * gets the plan under which it ran faster (CUDA events around every pass),
 * kept if the whole step is faster.  Outputs (may be NULL): the chosen
 * operand mode (-1 when there is no choice), graph steps, radix plan (0, 1,
 * or 2 for a plan per fused pass), ms per step. */
int gpe_gb_autotune(gpe_gb_engine* e, int nsteps, int* direct, int* graph_steps, int* fft_plan,
                    double* ms_per_step);
/* The same for a batch: radix plan, item order within each launch (0 as
 * created, 1 the condensates with most CTAs first) and steps per replayed graph. */
int gpe_gb_batch_autotune(gpe_gb_batch* b, int nsteps, int* order, int* graph_steps, int* fft_plan,
                          double* ms_per_step);
/* Message for a return code. */
const char* gpe_gb_error_string(int code);

#ifdef __cplusplus
}
#endif
#endif
