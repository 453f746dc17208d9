/*
 * CPU FP64 restatement of libcugpe's split-step evolution (gpe_evolve_qf)
 * and the observables around it.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA engine is
 * checked against and the timed CPU baseline; the product never links it.
 *
 * Every routine follows one reference routine, cited as file:line of
 * KKobuszewski/libcugpe:
 *   tables            dev/gpe_engine.cu:126-220 (gpe_reciprocal_lattice_init)
 *   step coefficient  dev/gpe_engine.cu:177-181
 *   density           dev/gpe_engine.cu:600-603
 *   normalisation     dev/gpe_engine.cu:628-667
 *   Vstep1/2/3, expT  dev/gpe_engine.cu:716-891
 *   quantum friction  dev/gpe_engine.cu:893-933, 435-460
 *   evolve loop       dev/gpe_engine.cu:1030-1109
 *   energy            dev/gpe_engine.cu:1631-1705
 *   functionals       dev/gpe_user_defined.h:118-135 (UFG), 196-243 (BEC side
 *                     of the crossover), 305-322 (contact BEC)
 *   harmonic trap     dev/gpe_user_defined.h:488-513
 *   phase enforcing   dev/gpe_engine.cu:465-591, 1112-1477 (gpe_set_vortex, gpe_evolve_vortex*,
 *                     gpe_get/set_phase, gpe_evolve_enforced_phase)
 *   currents          dev/gpe_engine.cu:1817-1904
 *   dipolar BEC       dev/gpe_engine.cu:1481-1809, dev/gpe_user_defined.h:356-451
 * Pinned: the reference engine's own outputs on the same seeded inputs
 * (tests/golden, every functional, ITE and RTE, friction, currents, dipolar
 * evolution and energy) match this restatement to <= 1e-12 relative L2.
 * The 3D FFT is cuFFT Z2Z in the reference (a third-party library absent from
 * the reference tree): unnormalised, e^{-2 pi i jk/n} forward and e^{+...}
 * inverse on a C-order [nx][ny][nz] array.  It is restated here as an
 * iterative radix-2 transform per axis.  Sums use fixed-order pairwise
 * summation over a fixed number of chunks (the reference's tree sum,
 * dev/reductions.cu:64-130, differs only in order).
 *
 * Extensions beyond the reference (no reference output pins them; they are
 * checked against closed forms and numpy restatements in tests/test_oracle.py):
 * an optional additive potential table, one real field per time slice,
 * selected by it / steps_per_slice (the time-dependent control problem), and
 * the Weizsaecker gradient term frozen per step with its sub-steps.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_USER_PARAMS 32
#define ORC_QF_EPSILON 1.0e-12
#define ORC_CHUNKS 256

typedef struct { double x, y; } cd;

static inline cd cmul(cd a, cd b) { cd c; c.x = a.x * b.x - a.y * b.y; c.y = a.x * b.y + a.y * b.x; return c; }
static inline cd cscale(cd a, double s) { cd c; c.x = s * a.x; c.y = s * a.y; return c; }
static inline cd cexp_(cd z) { double t = exp(z.x); cd r; r.x = t * cos(z.y); r.y = t * sin(z.y); return r; }

/* user hooks (a hook header compiled for the host by oracle/hooks_host.cpp); NULL = built-in physics */
typedef double (*orc_vext_fn)(unsigned ix, unsigned iy, unsigned iz, unsigned it);
typedef double (*orc_rho_fn)(double rho, unsigned it);
typedef void (*orc_modify_fn)(unsigned ix, unsigned iy, unsigned iz, unsigned it, double *re, double *im);

typedef struct {
    int nx, ny, nz;
    size_t n;
    int inter;            /* -1 contact BEC, 0 unitary Fermi gas, 1 BEC side of crossover */
    double gamma;         /* 1 particles, 2 dimers */
    double alpha, beta, dt, npart, t0, qfcoeff;
    unsigned it;
    double up[ORC_MAX_USER_PARAMS];
    double *kx, *ky, *kz;
    cd *ex, *ey, *ez;     /* ez includes 1/n */
    cd c3;
    cd *psi, *psi2, *wrkC, *wrk3C;
    double *V, *Vqf, *rho;
    cd *tw[3];            /* per-axis twiddles e^{-2 pi i k / n_axis}, k < n/2 */
    int nthreads;
    /* optional additive potential: nslices fields of n doubles */
    const double *vextra;
    int nslices, steps_per_slice;
    /* phase enforcing (dev/gpe_engine.cu:465-591) */
    double vx0, vy0;
    int vq;
    double *phase;
    /* Weizsaecker term (not in the reference): weight and scratch */
    double wz, wz_eps;
    double dt_step;       /* the caller's time step; dt = dt_step / sub */
    int sub;              /* sub-steps per step while the Weizsaecker term is on */
    cd *wz1;
    double *wzG, *wzS;
    /* user hooks (dev/gpe_user_defined.h names: gpe_external_potential, gpe_dEDFdn, gpe_EDF,
     * gpe_modify_psi) */
    orc_vext_fn hk_vext;
    orc_rho_fn hk_dedf, hk_edf;
    orc_modify_fn hk_modify;
} gpe_oracle;

/* ---------------------------------------------------------------- helpers */

static double pairwise_sum(const double *a, size_t n) {
    if (n <= 64) {
        double s = 0.0;
        for (size_t i = 0; i < n; i++) s += a[i];
        return s;
    }
    size_t h = n / 2;
    return pairwise_sum(a, h) + pairwise_sum(a + h, n - h);
}

/* deterministic sum: fixed chunking independent of the thread count */
static double det_sum(const gpe_oracle *o, const double *a) {
    double part[ORC_CHUNKS];
    size_t n = o->n;
    size_t chunk = (n + ORC_CHUNKS - 1) / ORC_CHUNKS;
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (int c = 0; c < ORC_CHUNKS; c++) {
        size_t b = (size_t)c * chunk, e = b + chunk;
        if (b > n) b = n;
        if (e > n) e = n;
        part[c] = pairwise_sum(a + b, e - b);
    }
    return pairwise_sum(part, ORC_CHUNKS);
}

static void fill_k(double *k, int n) {
    /* dev/gpe_engine.cu:147-154 */
    int i, j;
    for (i = 0; i <= n / 2 - 1; i++) k[i] = 2. * M_PI / n * (double)i;
    j = -i;
    for (i = n / 2; i < n; i++) { k[i] = 2. * M_PI / n * (double)j; j++; }
}

static void fill_tw(cd *tw, int n) {
    for (int k = 0; k < n / 2; k++) {
        long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)k / (long double)n;
        tw[k].x = (double)cosl(a);
        tw[k].y = (double)sinl(a);
    }
}

/* in-place radix-2 FFT of a contiguous buffer; sign -1 forward, +1 inverse */
static void fft1d(cd *a, int n, const cd *tw, int sign) {
    for (int i = 1, j = 0; i < n; i++) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) { cd t = a[i]; a[i] = a[j]; a[j] = t; }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1, step = n / len;
        for (int i = 0; i < n; i += len) {
            for (int k = 0; k < half; k++) {
                cd w = tw[k * step];
                if (sign > 0) w.y = -w.y;
                cd u = a[i + k], v = cmul(a[i + k + half], w);
                a[i + k].x = u.x + v.x; a[i + k].y = u.y + v.y;
                a[i + k + half].x = u.x - v.x; a[i + k + half].y = u.y - v.y;
            }
        }
    }
}

/* unnormalised 3D transform of a C-order [nx][ny][nz] array */
static void fft3d(const gpe_oracle *o, cd *a, int sign) {
    const int nx = o->nx, ny = o->ny, nz = o->nz;
    /* z: contiguous pencils */
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long p = 0; p < (long)nx * ny; p++) fft1d(a + (size_t)p * nz, nz, o->tw[2], sign);
    /* y: stride nz */
#pragma omp parallel num_threads(o->nthreads)
    {
        cd *buf = (cd *)malloc(sizeof(cd) * (size_t)ny);
#pragma omp for schedule(static)
        for (long p = 0; p < (long)nx * nz; p++) {
            size_t ix = (size_t)p / nz, iz = (size_t)p % nz;
            cd *base = a + ix * ny * nz + iz;
            for (int j = 0; j < ny; j++) buf[j] = base[(size_t)j * nz];
            fft1d(buf, ny, o->tw[1], sign);
            for (int j = 0; j < ny; j++) base[(size_t)j * nz] = buf[j];
        }
        free(buf);
    }
    /* x: stride ny*nz */
#pragma omp parallel num_threads(o->nthreads)
    {
        cd *buf = (cd *)malloc(sizeof(cd) * (size_t)nx);
        const size_t s = (size_t)ny * nz;
#pragma omp for schedule(static)
        for (long p = 0; p < (long)s; p++) {
            cd *base = a + p;
            for (int j = 0; j < nx; j++) buf[j] = base[(size_t)j * s];
            fft1d(buf, nx, o->tw[0], sign);
            for (int j = 0; j < nx; j++) base[(size_t)j * s] = buf[j];
        }
        free(buf);
    }
}

/* ----------------------------------------------------------- physics hooks */

static inline double density(const gpe_oracle *o, cd p) { return o->gamma * (p.x * p.x + p.y * p.y); }

static inline double vext(const gpe_oracle *o, size_t idx, int ix, int iy, int iz, unsigned it) {
    /* dev/gpe_user_defined.h:488-513, or the user hook gpe_external_potential */
    double v;
    if (o->hk_vext) {
        v = o->hk_vext((unsigned)ix, (unsigned)iy, (unsigned)iz, it);
    } else {
        const double wx = o->up[0], wy = o->up[1], wz = o->up[2];
        const double _ix = (double)ix - 1.0 * (o->nx / 2);
        const double _iy = (double)iy - 1.0 * (o->ny / 2);
        const double _iz = (double)iz - 1.0 * (o->nz / 2);
        v = 0.5 * _ix * _ix * wx * wx + 0.5 * _iy * _iy * wy * wy + 0.5 * _iz * _iz * wz * wz;
    }
    if (o->vextra) {
        int s = (int)(it / ((unsigned)o->steps_per_slice * (unsigned)o->sub));
        if (s >= o->nslices) s = o->nslices - 1;
        v += o->vextra[(size_t)s * o->n + idx];
    }
    return v;
}

#define ORC_XI 0.37
#define ORC_CONTACT 0.901

/* psi as a step reads it: the user hook gpe_modify_psi (dev/gpe_user_defined.h:81-85), called at
 * dev/gpe_engine.cu:733, 758, 794, 834, 861, 999 */
static inline cd modify(const gpe_oracle *o, int ix, int iy, int iz, unsigned it, cd p) {
    if (o->hk_modify) o->hk_modify((unsigned)ix, (unsigned)iy, (unsigned)iz, it, &p.x, &p.y);
    return p;
}

static inline double dEDFdn_builtin(const gpe_oracle *o, double rho);
static inline double EDF_builtin(const gpe_oracle *o, double rho);

/* functional at step `it`: the user hooks gpe_dEDFdn / gpe_EDF, or the built-in ones */
static inline double dEDFdn(const gpe_oracle *o, double rho, unsigned it) {
    return o->hk_dedf ? o->hk_dedf(rho, it) : dEDFdn_builtin(o, rho);
}
static inline double EDF(const gpe_oracle *o, double rho, unsigned it) {
    return o->hk_edf ? o->hk_edf(rho, it) : EDF_builtin(o, rho);
}

static inline double dEDFdn_builtin(const gpe_oracle *o, double rho) {
    if (o->inter == 0) return 0.37 * pow(3.0 * M_PI * M_PI * rho, 2.0 / 3.0) / 2.0;
    if (o->inter == -1) { const double a = o->up[3]; return 4 * M_PI * a * rho; }
    if (o->inter == -2) return 0.0; /* dipolar BEC: dev/gpe_user_defined.h:400-404 */
    if (o->inter == 1) {
        const double a = o->up[3];
        if (rho > 1e-15) {
            const double kF = pow(3.0 * M_PI * M_PI * rho, 1.0 / 3.0);
            const double eF = 0.5 * kF * kF;
            const double x = (kF > 2.2250738585072014e-308) ? 1.0 / (a * kF) : 1.7976931348623157e308;
            const double D = (ORC_XI + x * (1.0 + ORC_CONTACT) + 3.0 * M_PI * ORC_XI * x * x);
            return ORC_XI * eF * (ORC_XI + 0.8 * x) / D
                 + 0.2 * ORC_XI * eF * (ORC_XI + x) * x * ((1.0 + ORC_CONTACT) + 6.0 * M_PI * ORC_XI * x) / (D * D)
                 - 1.0 / (2.0 * a * a);
        }
        return -1.0 / (2.0 * a * a);
    }
    return 0.0;
}

static inline double EDF_builtin(const gpe_oracle *o, double rho) {
    if (o->inter == 0) return 0.37 * 0.6 * rho * pow(3.0 * M_PI * M_PI * rho, 2.0 / 3.0) / 2.;
    if (o->inter == -1 || o->inter == -2) { const double a = o->up[3]; return 2 * M_PI * a * rho * rho; }
    if (o->inter == 1) {
        const double a = o->up[3];
        const double kF = pow(3.0 * M_PI * M_PI * rho, 1.0 / 3.0);
        const double eF = 0.5 * kF * kF;
        const double x = (kF > 2.2250738585072014e-308) ? 1.0 / (a * kF) : 1.7976931348623157e308;
        return 0.6 * eF * rho * ORC_XI * (ORC_XI + x) / (ORC_XI + x * (1.0 + ORC_CONTACT) + 3.0 * M_PI * ORC_XI * x * x)
             - rho / (2.0 * a * a);
    }
    return 0.0;
}

/* -------------------------------------------------------------- lifecycle */

static void tables(gpe_oracle *o) {
    /* dev/gpe_engine.cu:177-216: c3 = Gamma*0.5*dt / (-beta + i alpha) */
    const double a = o->gamma * 0.5 * o->dt;
    const double br = -1.0 * o->beta, bi = o->alpha;
    const double den = br * br + bi * bi;
    o->c3.x = a * br / den;
    o->c3.y = -a * bi / den;
    const double g2 = o->gamma * o->gamma;
    for (int i = 0; i < o->nx; i++) {
        cd z = o->c3; z = cscale(z, o->kx[i]); z = cscale(z, o->kx[i]); z.x /= g2; z.y /= g2;
        o->ex[i] = cexp_(z);
    }
    for (int i = 0; i < o->ny; i++) {
        cd z = o->c3; z = cscale(z, o->ky[i]); z = cscale(z, o->ky[i]); z.x /= g2; z.y /= g2;
        o->ey[i] = cexp_(z);
    }
    for (int i = 0; i < o->nz; i++) {
        cd z = o->c3; z = cscale(z, o->kz[i]); z = cscale(z, o->kz[i]); z.x /= g2; z.y /= g2;
        z = cexp_(z);
        z.x /= (double)o->n; z.y /= (double)o->n;
        o->ez[i] = z;
    }
}

void *oracle_create(int nx, int ny, int nz, int inter, double gamma,
                    double alpha, double beta, double dt, double npart) {
    if (nx < 2 || ny < 2 || nz < 2) return NULL;
    if ((nx & (nx - 1)) || (ny & (ny - 1)) || (nz & (nz - 1))) return NULL;
    gpe_oracle *o = (gpe_oracle *)calloc(1, sizeof(gpe_oracle));
    o->nx = nx; o->ny = ny; o->nz = nz;
    o->n = (size_t)nx * ny * nz;
    o->inter = inter; o->gamma = gamma;
    o->alpha = alpha; o->beta = beta; o->dt = dt; o->npart = npart;
    o->dt_step = dt; o->sub = 1;
    o->nthreads = 1;
    o->kx = malloc(sizeof(double) * nx); o->ky = malloc(sizeof(double) * ny); o->kz = malloc(sizeof(double) * nz);
    fill_k(o->kx, nx); fill_k(o->ky, ny); fill_k(o->kz, nz);
    o->ex = malloc(sizeof(cd) * nx); o->ey = malloc(sizeof(cd) * ny); o->ez = malloc(sizeof(cd) * nz);
    int ns[3] = {nx, ny, nz};
    for (int a = 0; a < 3; a++) { o->tw[a] = malloc(sizeof(cd) * (ns[a] / 2 + 1)); fill_tw(o->tw[a], ns[a]); }
    tables(o);
    o->psi = calloc(o->n, sizeof(cd)); o->psi2 = calloc(o->n, sizeof(cd));
    o->wrkC = calloc(o->n, sizeof(cd)); o->wrk3C = calloc(o->n, sizeof(cd));
    o->V = calloc(o->n, sizeof(double)); o->Vqf = calloc(o->n, sizeof(double)); o->rho = calloc(o->n, sizeof(double));
    return o;
}

void oracle_destroy(void *h) {
    gpe_oracle *o = (gpe_oracle *)h;
    if (!o) return;
    free(o->kx); free(o->ky); free(o->kz); free(o->ex); free(o->ey); free(o->ez);
    for (int a = 0; a < 3; a++) free(o->tw[a]);
    free(o->psi); free(o->psi2); free(o->wrkC); free(o->wrk3C); free(o->V); free(o->Vqf); free(o->rho);
    free(o->wz1); free(o->wzG); free(o->wzS);
    free(o->phase);
    free(o);
}

void oracle_set_threads(void *h, int t) { ((gpe_oracle *)h)->nthreads = t > 0 ? t : 1; }

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int oracle_set_user_params(void *h, int size, const double *p) {
    gpe_oracle *o = (gpe_oracle *)h;
    if (size > ORC_MAX_USER_PARAMS || size < 0) return -9;
    memset(o->up, 0, sizeof o->up);
    memcpy(o->up, p, sizeof(double) * (size_t)size);
    return 0;
}

void oracle_change_alpha_beta(void *h, double alpha, double beta) {
    gpe_oracle *o = (gpe_oracle *)h;
    o->alpha = alpha; o->beta = beta;
    tables(o);
}

void oracle_set_hooks(void *h, void *vext_fn, void *dedf_fn, void *edf_fn, void *modify_fn) {
    gpe_oracle *o = (gpe_oracle *)h;
    o->hk_vext = (orc_vext_fn)vext_fn;
    o->hk_dedf = (orc_rho_fn)dedf_fn;
    o->hk_edf = (orc_rho_fn)edf_fn;
    o->hk_modify = (orc_modify_fn)modify_fn;
}

void oracle_set_time(void *h, double t0) { gpe_oracle *o = (gpe_oracle *)h; o->t0 = t0; o->it = 0; }

void oracle_set_qf(void *h, double q) {
    /* dev/gpe_engine.cu:435-460 */
    gpe_oracle *o = (gpe_oracle *)h;
    o->qfcoeff = (q != 0.0) ? q / (o->gamma * (double)o->n) : 0.0;
}

void oracle_set_wz(void *h, double lambda, double eps) {
    gpe_oracle *o = (gpe_oracle *)h;
    o->wz = lambda;
    o->wz_eps = (eps > 0.0) ? eps : 1e-2 * o->npart / (double)o->n;
    /* the frozen V_W is stable for dt |lambda| 3 pi^2 <= 0.4: longer steps run as sub-steps */
    const double x = o->dt_step * fabs(lambda) * 3.0 * M_PI * M_PI;
    o->sub = (x > 0.4) ? (int)ceil(x / 0.4) : 1;
    o->dt = o->dt_step / o->sub;
    tables(o);
    if (lambda != 0.0 && !o->wz1) {
        o->wz1 = calloc(o->n, sizeof(cd));
        o->wzG = calloc(o->n, sizeof(double));
        o->wzS = calloc(o->n, sizeof(double));
    }
}

void oracle_set_vextra(void *h, const double *v, int nslices, int steps_per_slice) {
    gpe_oracle *o = (gpe_oracle *)h;
    o->vextra = v; o->nslices = nslices; o->steps_per_slice = steps_per_slice > 0 ? steps_per_slice : 1;
}

void oracle_set_psi(void *h, double t, const double *psi) {
    gpe_oracle *o = (gpe_oracle *)h;
    o->t0 = t; o->it = 0;
    memcpy(o->psi, psi, sizeof(cd) * o->n);
}

void oracle_get_psi(void *h, double *t, double *psi) {
    gpe_oracle *o = (gpe_oracle *)h;
    memcpy(psi, o->psi, sizeof(cd) * o->n);
    if (t) *t = o->t0 + o->dt * o->it;
}

/* ------------------------------------------------------------- operations */

static double norm_of(gpe_oracle *o, const cd *p) {
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < (long)o->n; i++) o->rho[i] = density(o, p[i]);
    return det_sum(o, o->rho);
}

static double normalize(gpe_oracle *o, cd *p) {
    /* dev/gpe_engine.cu:628-646 */
    const double sum = norm_of(o, p);
    const double s = sqrt(o->npart / sum);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < (long)o->n; i++) p[i] = cscale(p[i], s);
    return sum;
}

void oracle_get_density(void *h, double *t, double *out) {
    gpe_oracle *o = (gpe_oracle *)h;
    for (size_t i = 0; i < o->n; i++) out[i] = density(o, o->psi[i]);
    if (t) *t = o->t0 + o->dt * o->it;
}

double oracle_get_norm(void *h) { gpe_oracle *o = (gpe_oracle *)h; return norm_of(o, o->psi); }

void oracle_normalize(void *h) { gpe_oracle *o = (gpe_oracle *)h; normalize(o, o->psi); }

#define DECODE(i)                                   \
    const int ix = (int)((i) / ((size_t)ny * nz));  \
    const int iy = (int)(((i) / nz) % ny);          \
    const int iz = (int)((i) % nz);

static void mult_expT(gpe_oracle *o, cd *p) {
    /* dev/gpe_engine.cu:876-891 */
    const int ny = o->ny, nz = o->nz;
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < (long)o->n; i++) {
        DECODE((size_t)i);
        cd w = p[i];
        w = cmul(w, o->ex[ix]);
        w = cmul(w, o->ey[iy]);
        w = cmul(w, o->ez[iz]);
        p[i] = w;
    }
}

static void qf_potential(gpe_oracle *o, const cd *psi) {
    /* dev/gpe_engine.cu:893-933 */
    const int ny = o->ny, nz = o->nz;
    memcpy(o->wrk3C, psi, sizeof(cd) * o->n);
    fft3d(o, o->wrk3C, -1);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < (long)o->n; i++) {
        DECODE((size_t)i);
        o->wrk3C[i] = cscale(o->wrk3C[i], o->qfcoeff * (o->kx[ix] * o->kx[ix] + o->ky[iy] * o->ky[iy] + o->kz[iz] * o->kz[iz]));
    }
    fft3d(o, o->wrk3C, +1);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < (long)o->n; i++) {
        cd a = psi[i]; a.y = -a.y;
        const cd b = o->wrk3C[i];
        const double lrho = density(o, psi[i]);
        o->Vqf[i] = (a.x * b.y + a.y * b.x) / (lrho + ORC_QF_EPSILON);
    }
}

/* Weizsaecker gradient term, added to Vqf (not in the reference; the hook
 * gpe_gradient_corrections of dev/gpe_user_defined.h:158 is never called):
 * E_W = (lambda/8) sum |grad rho|^2 / rho, so
 * V_W = (lambda/8) (|grad rho|^2 / rho^2 - 2 lap(rho) / rho), rho = Gamma |psi|^2,
 * grad rho = 2 Gamma Re(conj(psi) grad psi),
 * lap rho = 2 Gamma (Re(conj(psi) lap psi) + |grad psi|^2),
 * derivatives of psi spectral on the reference k grid (dev/gpe_engine.cu:147-154),
 * rho replaced by rho + wz_eps in both denominators. */
static void wz_sums(gpe_oracle *o, const cd *psi);

static void wz_potential(gpe_oracle *o, const cd *psi) {
    const long n = (long)o->n;
    const double g2 = 2.0 * o->gamma;
    wz_sums(o, psi);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < n; i++) {
        const cd p = psi[i], l = o->wz1[i];
        const double inv = 1.0 / (density(o, p) + o->wz_eps);
        const double lrho = g2 * ((p.x * l.x + p.y * l.y) + o->wzS[i]);
        o->Vqf[i] += (o->wz / 8.0) * (o->wzG[i] * inv * inv - 2.0 * lrho * inv);
    }
}

/* E_W = (lambda/8) sum |grad rho|^2 / (rho + eps) */
static double wz_energy(gpe_oracle *o, const cd *psi) {
    const long n = (long)o->n;
    wz_sums(o, psi);
    double *w = (double *)malloc(sizeof(double) * n);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < n; i++) w[i] = o->wzG[i] / (density(o, psi[i]) + o->wz_eps);
    const double e = (o->wz / 8.0) * det_sum(o, w);
    free(w);
    return e;
}

/* wzG = sum_a (d_a rho)^2, wzS = sum_a |d_a psi|^2, wz1 = lap psi */
static void wz_sums(gpe_oracle *o, const cd *psi) {
    const int ny = o->ny, nz = o->nz;
    const long n = (long)o->n;
    const double inv_n = 1.0 / (double)o->n, g2 = 2.0 * o->gamma;
    memcpy(o->wrk3C, psi, sizeof(cd) * o->n);
    fft3d(o, o->wrk3C, -1);
    memset(o->wzG, 0, sizeof(double) * o->n);
    memset(o->wzS, 0, sizeof(double) * o->n);
    const double *ks[3] = {o->kx, o->ky, o->kz};
    for (int a = 0; a < 3; a++) {
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
        for (long i = 0; i < n; i++) {
            DECODE((size_t)i);
            const double k = ks[a][(a == 0) ? ix : (a == 1) ? iy : iz] * inv_n;
            cd z; z.x = -k * o->wrk3C[i].y; z.y = k * o->wrk3C[i].x;  /* i k psi_hat / n */
            o->wz1[i] = z;
        }
        fft3d(o, o->wz1, +1);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
        for (long i = 0; i < n; i++) {
            const cd p = psi[i], d1 = o->wz1[i];
            const double d = g2 * (p.x * d1.x + p.y * d1.y);
            o->wzG[i] += d * d;
            o->wzS[i] += d1.x * d1.x + d1.y * d1.y;
        }
    }
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < n; i++) {
        DECODE((size_t)i);
        const double k2 = o->kx[ix] * o->kx[ix] + o->ky[iy] * o->ky[iy] + o->kz[iz] * o->kz[iz];
        o->wz1[i] = cscale(o->wrk3C[i], -k2 * inv_n);
    }
    fft3d(o, o->wz1, +1);
}

/* potential frozen over a step: friction (dev/gpe_engine.cu:893-933) and the Weizsaecker term */
static void frozen_potential(gpe_oracle *o, const cd *psi) {
    if (o->qfcoeff != 0.0) qf_potential(o, psi);
    else memset(o->Vqf, 0, sizeof(double) * o->n);
    if (o->wz != 0.0) wz_potential(o, psi);
}

/* V_W alone for the current psi (tests) */
void oracle_wz_potential(void *h, double *out) {
    gpe_oracle *o = (gpe_oracle *)h;
    memset(o->Vqf, 0, sizeof(double) * o->n);
    if (o->wz != 0.0) wz_potential(o, o->psi);
    memcpy(out, o->Vqf, sizeof(double) * o->n);
}

/* enforcing ops: 1 vortex imprint (dev/gpe_engine.cu:485-511), 2 imprint
 * where |psi| > 1e-15 (:520-548), 3 psi = |psi| exp(i phase) (:584-591) */
static void enforce(gpe_oracle *o, int mode) {
    const int ny = o->ny, nz = o->nz;
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < (long)o->n; i++) {
        DECODE((size_t)i);
        (void)iz;
        cd p = o->psi[i];
        if (mode == 3) {
            const double a = sqrt(p.x * p.x + p.y * p.y);
            p.x = a * cos(o->phase[i]);
            p.y = a * sin(o->phase[i]);
        } else {
            const double xx = (double)ix - 1.0 * (o->nx / 2) - o->vx0;
            const double yy = (double)iy - 1.0 * (o->ny / 2) - o->vy0;
            const double a = hypot(p.x, p.y);
            if (mode == 1 || a > 1e-15) {
                const double ph = atan2(xx, yy) * (double)o->vq;
                p.x = a * cos(ph);
                p.y = a * sin(ph);
            }
        }
        o->psi[i] = p;
    }
}

void oracle_set_vortex(void *h, double x0, double y0, int q) {
    gpe_oracle *o = (gpe_oracle *)h;
    o->vx0 = x0; o->vy0 = y0; o->vq = q;
}

void oracle_get_phase(void *h, double *out) {
    gpe_oracle *o = (gpe_oracle *)h;
    if (!o->phase) o->phase = malloc(sizeof(double) * o->n);
    for (size_t i = 0; i < o->n; i++) o->phase[i] = atan2(o->psi[i].y, o->psi[i].x);
    if (out) memcpy(out, o->phase, sizeof(double) * o->n);
}

void oracle_set_phase(void *h, const double *ph) {
    gpe_oracle *o = (gpe_oracle *)h;
    if (!o->phase) o->phase = malloc(sizeof(double) * o->n);
    memcpy(o->phase, ph, sizeof(double) * o->n);
}

static int evolve_impl(gpe_oracle *o, int nt, double *mu, int mode, int mid_repeat);

int oracle_evolve_qf(void *h, int nt, double *mu) {
    gpe_oracle *o = (gpe_oracle *)h;
    return evolve_impl(o, nt * o->sub, mu, 0, 0);
}

/* gpe_evolve_vortex{,2,3} and gpe_evolve_enforced_phase (dev/gpe_engine.cu:1115-1477):
 * kind 1, 2, 3 vortex methods, 4 enforced phase */
int oracle_evolve_enforced(void *h, int nt, double *mu, int kind) {
    const int mode = (kind == 2) ? 2 : (kind == 4) ? 3 : 1;
    gpe_oracle *o = (gpe_oracle *)h;
    return evolve_impl(o, nt * o->sub, mu, mode, kind != 3);
}

static int evolve_impl(gpe_oracle *o, int nt, double *mu, int mode, int mid_repeat) {
    const int ny = o->ny, nz = o->nz;
    const long n = (long)o->n;
    const int qf = o->qfcoeff != 0.0 || o->wz != 0.0;
    for (int step = 0; step < nt; step++) {
        const unsigned it = o->it;
        if (mode) enforce(o, mode);
        /* Vstep1 / Vstep1_qf: dev/gpe_engine.cu:719-768, 1038-1047 */
        if (qf) frozen_potential(o, o->psi);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
        for (long i = 0; i < n; i++) {
            DECODE((size_t)i);
            const cd lpsi = modify(o, ix, iy, iz, it, o->psi[i]);
            const double lrho = density(o, lpsi);
            double lv = vext(o, (size_t)i, ix, iy, iz, it) + dEDFdn(o, lrho, it);
            if (qf) lv += o->Vqf[i];
            o->V[i] = lv;
            o->psi2[i] = cmul(lpsi, cexp_(cscale(o->c3, lv)));
        }
        /* kinetic: dev/gpe_engine.cu:1050-1054 */
        fft3d(o, o->psi2, -1);
        mult_expT(o, o->psi2);
        fft3d(o, o->psi2, +1);
        if (o->beta == 0.0 && !qf) {
            /* Vstep2: dev/gpe_engine.cu:770-797 */
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
            for (long i = 0; i < n; i++) {
                DECODE((size_t)i);
                double lv = o->V[i];
                cd lpsi = cmul(o->psi2[i], cexp_(cscale(o->c3, lv)));
                const double lrho = density(o, lpsi);
                lv = 0.5 * (lv + vext(o, (size_t)i, ix, iy, iz, it + 1) + dEDFdn(o, lrho, it + 1));
                const cd e = cexp_(cscale(o->c3, lv));
                o->wrkC[i] = e;
                o->psi[i] = cmul(modify(o, ix, iy, iz, it, o->psi[i]), e);
            }
        } else {
            /* part1: dev/gpe_engine.cu:799-811 */
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
            for (long i = 0; i < n; i++) o->psi2[i] = cmul(o->psi2[i], cexp_(cscale(o->c3, o->V[i])));
            if (o->beta != 0.0) {
                normalize(o, o->psi2);
                if (mode && mid_repeat) enforce(o, mode); /* :1161, :1253, :1436 */
            }
            if (qf) frozen_potential(o, o->psi);
            /* part2 / part2_qf: dev/gpe_engine.cu:813-864 */
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
            for (long i = 0; i < n; i++) {
                DECODE((size_t)i);
                const double lrho = density(o, o->psi2[i]);
                double lv = o->V[i] + vext(o, (size_t)i, ix, iy, iz, it + 1) + dEDFdn(o, lrho, it + 1);
                if (qf) lv += o->Vqf[i];
                lv = 0.5 * lv;
                const cd e = cexp_(cscale(o->c3, lv));
                o->wrkC[i] = e;
                o->psi[i] = cmul(modify(o, ix, iy, iz, it, o->psi[i]), e);
            }
        }
        fft3d(o, o->psi, -1);
        mult_expT(o, o->psi);
        fft3d(o, o->psi, +1);
        /* Vstep3: dev/gpe_engine.cu:866-874 */
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
        for (long i = 0; i < n; i++) o->psi[i] = cmul(o->psi[i], o->wrkC[i]);
        if (o->beta != 0.0) {
            const double norm = normalize(o, o->psi);
            if (mu) *mu = -.5 * log(norm / o->npart) / o->dt;
        }
        o->it = o->it + 1;
    }
    return 0;
}

int oracle_energy(void *h, double *t, double *ekin, double *eint, double *eext) {
    /* dev/gpe_engine.cu:1669-1705 */
    gpe_oracle *o = (gpe_oracle *)h;
    const int ny = o->ny, nz = o->nz;
    const long n = (long)o->n;
    *t = o->t0 + o->dt * o->it;
    if (o->beta == 0.0) normalize(o, o->psi);
    double *w1 = (double *)malloc(sizeof(double) * n), *w2 = (double *)malloc(sizeof(double) * n);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < n; i++) {
        DECODE((size_t)i);
        const double lrho = density(o, o->psi[i]);
        w1[i] = lrho * vext(o, (size_t)i, ix, iy, iz, o->it);
        w2[i] = EDF(o, lrho, o->it);
    }
    *eext = det_sum(o, w1);
    *eint = det_sum(o, w2);
    if (o->wz != 0.0) *eint += wz_energy(o, o->psi);  /* Weizsaecker term (not in the reference) */
    memcpy(o->psi2, o->psi, sizeof(cd) * o->n);
    fft3d(o, o->psi2, -1);
    const double den = 2.0 * o->gamma * (double)o->n;
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < n; i++) {
        DECODE((size_t)i);
        o->psi2[i] = cscale(o->psi2[i], (o->kx[ix] * o->kx[ix] + o->ky[iy] * o->ky[iy] + o->kz[iz] * o->kz[iz]) / den);
    }
    fft3d(o, o->psi2, +1);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < n; i++) w1[i] = o->psi[i].x * o->psi2[i].x + o->psi[i].y * o->psi2[i].y;
    *ekin = det_sum(o, w1);
    free(w1); free(w2);
    return 0;
}

int oracle_get_currents(void *h, double *t, double *jx, double *jy, double *jz) {
    /* dev/gpe_engine.cu:1856-1904: psi2 = FFT psi; per axis a: IFFT(k_a/(Gamma n) psi2),
     * j_a = Re(conj(psi) .) (cplxMulR, :1660-1667) */
    gpe_oracle *o = (gpe_oracle *)h;
    const int ny = o->ny, nz = o->nz;
    const long n = (long)o->n;
    *t = o->t0 + o->dt * o->it;
    memcpy(o->psi2, o->psi, sizeof(cd) * o->n);
    fft3d(o, o->psi2, -1);
    double *out[3] = {jx, jy, jz};
    const double *ks[3] = {o->kx, o->ky, o->kz};
    const double den = o->gamma * (double)o->n;
    for (int a = 0; a < 3; a++) {
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
        for (long i = 0; i < n; i++) {
            DECODE((size_t)i);
            const int ia = (a == 0) ? ix : (a == 1) ? iy : iz;
            o->wrk3C[i] = cscale(o->psi2[i], ks[a][ia] / den);
        }
        fft3d(o, o->wrk3C, +1);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
        for (long i = 0; i < n; i++) out[a][i] = o->psi[i].x * o->wrk3C[i].x + o->psi[i].y * o->wrk3C[i].y;
    }
    return 0;
}

/* dipolar potential of psi: FFT of (rho, 0) (dev/gpe_engine.cu:618-626), times
 * gpe_Vpp_k / nxyz (dev/gpe_user_defined.h:422-438, dev/gpe_engine.cu:958-974),
 * inverse FFT, real part (:997-998) */
static void vdip_field(gpe_oracle *o, const cd *psi, double *vdip) {
    const int ny = o->ny, nz = o->nz;
    const long n = (long)o->n;
    const double a_con = o->up[3], a_dip = o->up[4];
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < n; i++) { o->wrk3C[i].x = density(o, psi[i]); o->wrk3C[i].y = 0.0; }
    fft3d(o, o->wrk3C, -1);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < n; i++) {
        DECODE((size_t)i);
        const double kx = o->kx[ix], ky = o->ky[iy], kz = o->kz[iz];
        const double k_sq = kx * kx + ky * ky + kz * kz;
        const double v = (k_sq < DBL_EPSILON) ? 4. * M_PI * a_con * 1.0
                                              : 4. * M_PI * (a_con * 1.0 + a_dip * (3. * kz * kz / k_sq - 1.));
        o->wrk3C[i] = cscale(o->wrk3C[i], v / (double)o->n);
    }
    fft3d(o, o->wrk3C, +1);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < n; i++) vdip[i] = o->wrk3C[i].x;
}

/* exp(c3 (Vext(it) + dEDF + vdip)) psi (dev/gpe_engine.cu:979-1006) */
static void dipolar_vstep(gpe_oracle *o, unsigned it) {
    const int ny = o->ny, nz = o->nz;
    const long n = (long)o->n;
    vdip_field(o, o->psi, o->V);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < n; i++) {
        DECODE((size_t)i);
        const cd lpsi = modify(o, ix, iy, iz, it, o->psi[i]);
        const double lrho = density(o, lpsi);
        const double lv = vext(o, (size_t)i, ix, iy, iz, it) + dEDFdn(o, lrho, it) + o->V[i];
        o->psi[i] = cmul(lpsi, cexp_(cscale(o->c3, lv)));
    }
}

/* gpe_evolve_dipolar (dev/gpe_engine.cu:1550-1602) */
int oracle_evolve_dipolar(void *h, int nt, double *mu) {
    gpe_oracle *o = (gpe_oracle *)h;
    for (int step = 0; step < nt; step++) {
        const unsigned it = o->it;
        dipolar_vstep(o, it);
        fft3d(o, o->psi, -1);
        mult_expT(o, o->psi);
        fft3d(o, o->psi, +1);
        dipolar_vstep(o, it);
        if (o->beta != 0.0) {
            const double norm = normalize(o, o->psi);
            if (mu) *mu = -.5 * log(norm / o->npart) / o->dt;
        }
        o->it = o->it + 1;
    }
    return 0;
}

/* gpe_energy_dipolar2 (dev/gpe_engine.cu:1789-1809): 1/2 sum rho vdip */
double oracle_energy_dipolar(void *h) {
    gpe_oracle *o = (gpe_oracle *)h;
    const long n = (long)o->n;
    vdip_field(o, o->psi, o->V);
    double *w = (double *)malloc(sizeof(double) * n);
#pragma omp parallel for num_threads(o->nthreads) schedule(static)
    for (long i = 0; i < n; i++) w[i] = density(o, o->psi[i]) * o->V[i];
    const double e = 0.5 * det_sum(o, w);
    free(w);
    return e;
}

/* raw 3D transform, exposed so the tests can pin the restated FFT against numpy */
void oracle_fft3d(int nx, int ny, int nz, double *a, int sign, int nthreads) {
    gpe_oracle o;
    memset(&o, 0, sizeof o);
    o.nx = nx; o.ny = ny; o.nz = nz; o.n = (size_t)nx * ny * nz; o.nthreads = nthreads > 0 ? nthreads : 1;
    int ns[3] = {nx, ny, nz};
    for (int k = 0; k < 3; k++) { o.tw[k] = malloc(sizeof(cd) * (ns[k] / 2 + 1)); fill_tw(o.tw[k], ns[k]); }
    fft3d(&o, (cd *)a, sign);
    for (int k = 0; k < 3; k++) free(o.tw[k]);
}
