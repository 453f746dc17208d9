/*
 * .dftc.info headers as the libcugpe drivers write and read them
 * (KKobuszewski/libcugpe dev/gpe_io.h), for source compatibility:
 *
 *   gpe_save_info / gpe_get_info   the 13-line header (system type, mode,
 *                                  lattice, dt, nom, a, aspect ratio, omega_x,
 *                                  r0, npart, total time; dev/gpe_io.h:46-166),
 *                                  through gpe_gb_dftc_write_info / _read_info
 *   save_info / get_info           the older 10-line header without the system,
 *                                  mode and total-time lines (dev/gpe_io.h:16-129;
 *                                  get_info takes the .info file name itself)
 *
 * The system type and mode follow the functional: INTERACTIONS -2 "bosons
 * dipolar", -1 "bosons contact", 0 "fermions unitary", 1 "fermions bec" (the
 * macro when the driver defines it, else the GPE_INTERACTIONS environment
 * variable the drop-in engine also reads, else -1).  As in the reference, a
 * header that cannot be read ends the program with an error message; one
 * that cannot be written does too.
 */
#ifndef GPE_GB300_IO_H
#define GPE_GB300_IO_H

#include <stdio.h>
#include <stdlib.h>
#include "gpe_gb300.h"

#define MAX_REC_LEN 256

static inline int gpe_io_interactions_(void) {
#ifdef INTERACTIONS
    return INTERACTIONS;
#else
    const char* v = getenv("GPE_INTERACTIONS");
    return v ? atoi(v) : -1;
#endif
}

static inline void gpe_io_fail_(const char* what, const char* path, const char* suffix) {
    printf("Error: Cannot %s file %s%s!\n", what, path, suffix);
    exit(EXIT_FAILURE);
}

#ifdef __cplusplus
static inline void gpe_save_info(const char* dftc_filename, const int nx, const int ny, const int nz,
                                 const double dt, const int nom, const double scat_lenght,
                                 const double aspect_ratio, const double omega_x, const double r0,
                                 const double npart, const double total_time = 0)
#else
static inline void gpe_save_info(const char* dftc_filename, const int nx, const int ny, const int nz,
                                 const double dt, const int nom, const double scat_lenght,
                                 const double aspect_ratio, const double omega_x, const double r0,
                                 const double npart, const double total_time)
#endif
{
    const int inter = gpe_io_interactions_();
    const char* system = inter < 0 ? "bosons" : "fermions";
    const char* mode = inter == -2 ? "dipolar" : inter == -1 ? "contact" : inter == 0 ? "unitary" : "bec";
    if (gpe_gb_dftc_write_info(dftc_filename, system, mode, nx, ny, nz, dt, nom, scat_lenght, aspect_ratio,
                               omega_x, r0, npart, total_time))
        gpe_io_fail_("write", dftc_filename, ".info");
}

#ifdef __cplusplus
static inline void gpe_get_info(const char* dftc_filename, int* nx, int* ny, int* nz, double* dt, int* nom,
                                double* scat_lenght, double* aspect_ratio, double* omega_x, double* r0,
                                double* npart, double* total_time = NULL)
#else
static inline void gpe_get_info(const char* dftc_filename, int* nx, int* ny, int* nz, double* dt, int* nom,
                                double* scat_lenght, double* aspect_ratio, double* omega_x, double* r0,
                                double* npart, double* total_time)
#endif
{
    if (gpe_gb_dftc_read_info(dftc_filename, NULL, NULL, 0, nx, ny, nz, dt, nom, scat_lenght, aspect_ratio,
                              omega_x, r0, npart, total_time))
        gpe_io_fail_("open", dftc_filename, ".info");
}

/* The older header: the ten numeric lines only, values as %lf. */
static inline void save_info(const char* dftc_filename, const int nx, const int ny, const int nz, const double dt,
                             const int nom, const double scat_lenght, const double aspect_ratio,
                             const double omega_x, const double r0, const double npart) {
    char name[MAX_REC_LEN + 8];
    snprintf(name, sizeof name, "%s.info", dftc_filename);
    FILE* f = fopen(name, "w");
    if (!f) gpe_io_fail_("write", name, "");
    fprintf(f, "%d   # nx\n%d   # ny\n%d   # nz\n", nx, ny, nz);
    fprintf(f, "%lf   # dt\n%d   # nom\n", dt, nom);
    fprintf(f, "%lf   # a_scattering\n%lf   # aspect_ratio\n", scat_lenght, aspect_ratio);
    fprintf(f, "%lf   # omega_x\n%lf   # r0\n%lf   # npart\n", omega_x, r0, npart);
    fclose(f);
}

static inline void get_info(const char* info_filename, int* nx, int* ny, int* nz, double* dt, int* nom,
                            double* scat_lenght, double* aspect_ratio, double* omega_x, double* r0,
                            double* npart) {
    FILE* f = fopen(info_filename, "r");
    if (!f) gpe_io_fail_("open", info_filename, "");
    char line[MAX_REC_LEN];
    int* ints[3] = {nx, ny, nz};
    for (int i = 0; i < 3; i++)
        if (fgets(line, sizeof line, f)) sscanf(line, "%d", ints[i]);
    if (fgets(line, sizeof line, f)) sscanf(line, "%lf", dt);
    if (fgets(line, sizeof line, f)) sscanf(line, "%d", nom);
    double* reals[5] = {scat_lenght, aspect_ratio, omega_x, r0, npart};
    for (int i = 0; i < 5; i++)
        if (fgets(line, sizeof line, f)) sscanf(line, "%lf", reals[i]);
    fclose(f);
}

#endif
