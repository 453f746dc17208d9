// Driver for the reference libcugpe engine, used only as a parity oracle and
// as the reference GPU timing.  TEST INFRASTRUCTURE ONLY.
//
// It is compiled by oracle/build_ref.py against edited copies of the reference
// sources (dev/gpe_engine.cu, dev/reductions.cu) for one compile-time lattice
// and functional, and calls only the reference's public API
// (dev/gpe_engine.h:299-558), in the order the reference's own drivers use it
// (test_compare/gpe_imag.c:92-133, test_compare/gpe_real.c:107-145).
//
// usage: ref_runner IN_PSI OUTDIR ALPHA BETA DT NPART QF P0 P1 P2 P3 CMDS
//   IN_PSI  raw nx*ny*nz complex128, C order (z fastest)
//   CMDS    comma-separated commands:
//     N      gpe_normalize_psi()
//     E      gpe_energy()             -> "E t ekin eint eext"
//     S<k>   gpe_evolve_qf(k, &mu)    -> "MU mu" (mu only meaningful in ITE)
//     B<k>   as S<k>, timed with CUDA events -> "TIME ms"
//     D      gpe_get_psi() -> OUTDIR/psi_<i>.bin
//     R / I  gpe_set_rte_evolution() / gpe_set_ite_evolution()
//     Q<x>   gpe_set_quantum_friction_coeff(x)
//     X<x0>/<y0>/<q>  gpe_set_vortex(x0, y0, q)
//     V<m>_<k>  gpe_evolve_vortex (m=1), _vortex2 (2), _vortex3 (3), k steps -> "MU mu"
//     G      gpe_get_phase(NULL)
//     P<k>   gpe_evolve_enforced_phase(k, &mu) -> "MU mu"
//     J      gpe_get_currents() -> OUTDIR/cur_<i>.bin (jx, jy, jz), "J t"
//     A<x>   fifth user parameter (A_DIP of the dipolar functional) = x, gpe_set_user_params(5, .)
//     Y<k>   gpe_evolve_dipolar(k, &mu) -> "MU mu"
//     W      gpe_energy_dipolar2() -> "W t edip"  (gpe_energy_dipolar itself indexes -k past the
//            transform for the k = 0 planes, dev/gpe_engine.cu:1725, and is not called)
//     Z      gpe_get_psi() then gpe_set_psi(0, psi): restart the clock and step counter on the
//            current state (the RTE half of the compare harness starts a fresh engine at t = 0)
//     C<k>/<tol>  ITE loop of test_compare/gpe_imag.c:125-144: gpe_evolve_qf(k), gpe_energy -> "E ...",
//            until |E_prev - E|/npart < tol (E_prev: the energy printed before)
//     T<k>/<tmax>  RTE loop of test_compare/gpe_real.c:145-163: gpe_evolve_qf(k), gpe_energy -> "E ...",
//            until t > tmax
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "gpe_engine.h"

#define CHECK(cmd) do { int _e = (cmd); if (_e) { fprintf(stderr, "FAIL %s -> %d\n", #cmd, _e); return 2; } } while (0)

int main(int argc, char** argv) {
    if (argc < 13) { fprintf(stderr, "usage: see source\n"); return 1; }
    const char* in_path = argv[1];
    std::string outdir = argv[2];
    double alpha = atof(argv[3]), beta = atof(argv[4]), dt = atof(argv[5]);
    double npart = atof(argv[6]), qf = atof(argv[7]);
    double params[5] = {atof(argv[8]), atof(argv[9]), atof(argv[10]), atof(argv[11]), 0.0};
    std::string cmds = argv[12];

    int nx, ny, nz;
    gpe_get_lattice(&nx, &ny, &nz);
    size_t n = (size_t)nx * ny * nz;
    std::vector<cuCplx> psi(n);
    FILE* f = fopen(in_path, "rb");
    if (!f || fread(psi.data(), sizeof(cuCplx), n, f) != n) { fprintf(stderr, "cannot read %s\n", in_path); return 1; }
    fclose(f);

    CHECK(gpe_create_engine(alpha, beta, dt, npart));
    CHECK(gpe_set_user_params(4, params));
    if (qf != 0.0) CHECK(gpe_set_quantum_friction_coeff(qf));
    CHECK(gpe_set_psi(0.0, psi.data()));

    int dump = 0, currents = 0;
    double etot_last = 0.0;
    size_t pos = 0;
    while (pos < cmds.size()) {
        size_t end = cmds.find(',', pos);
        if (end == std::string::npos) end = cmds.size();
        std::string c = cmds.substr(pos, end - pos);
        pos = end + 1;
        if (c.empty()) continue;
        if (c == "N") {
            CHECK(gpe_normalize_psi());
        } else if (c == "E") {
            double t, ek, ei, ee;
            CHECK(gpe_energy(&t, &ek, &ei, &ee));
            printf("E %.17g %.17g %.17g %.17g\n", t, ek, ei, ee);
            etot_last = ek + ei + ee;
        } else if (c[0] == 'C' || c[0] == 'T') {
            int k = 100;
            double lim = 0.0;
            sscanf(c.c_str() + 1, "%d/%lf", &k, &lim);
            for (int iter = 0; iter < 100000; iter++) {
                double t, ek, ei, ee;
                CHECK(gpe_evolve_qf(k));
                CHECK(gpe_energy(&t, &ek, &ei, &ee));
                printf("E %.17g %.17g %.17g %.17g\n", t, ek, ei, ee);
                const double et = ek + ei + ee, diff = (etot_last - et) / npart;
                etot_last = et;
                if (c[0] == 'C' ? fabs(diff) < lim : t > lim) break;
            }
        } else if (c == "Z") {
            double t;
            CHECK(gpe_get_psi(&t, psi.data()));
            CHECK(gpe_set_psi(0.0, psi.data()));
        } else if (c[0] == 'S' || c[0] == 'B') {
            int k = atoi(c.c_str() + 1);
            double mu = 0.0;
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0); cudaEventCreate(&e1);
            cudaEventRecord(e0);
            CHECK(gpe_evolve_qf(k, &mu));
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (c[0] == 'B') printf("TIME %.6f\n", ms);
            printf("MU %.17g\n", mu);
            cudaEventDestroy(e0); cudaEventDestroy(e1);
        } else if (c == "D") {
            double t;
            CHECK(gpe_get_psi(&t, psi.data()));
            char name[64];
            snprintf(name, sizeof name, "/psi_%d.bin", dump++);
            FILE* g = fopen((outdir + name).c_str(), "wb");
            if (!g) { fprintf(stderr, "cannot write\n"); return 1; }
            fwrite(psi.data(), sizeof(cuCplx), n, g);
            fclose(g);
            printf("D %.17g\n", t);
        } else if (c == "R") {
            CHECK(gpe_set_rte_evolution());
        } else if (c == "I") {
            CHECK(gpe_set_ite_evolution());
        } else if (c[0] == 'Q') {
            CHECK(gpe_set_quantum_friction_coeff(atof(c.c_str() + 1)));
        } else if (c[0] == 'X') {
            double x0 = 0, y0 = 0;
            int q = 1;
            sscanf(c.c_str() + 1, "%lf/%lf/%d", &x0, &y0, &q);
            CHECK(gpe_set_vortex(x0, y0, (int8_t)q));
        } else if (c[0] == 'V') {
            int m = 1, k = 0;
            sscanf(c.c_str() + 1, "%d_%d", &m, &k);
            double mu = 0.0;
            if (m == 1) CHECK(gpe_evolve_vortex(k, &mu));
            else if (m == 2) CHECK(gpe_evolve_vortex2(k, &mu));
            else CHECK(gpe_evolve_vortex3(k, &mu));
            printf("MU %.17g\n", mu);
        } else if (c == "J") {
            double t;
            std::vector<double> j(3 * n);
            CHECK(gpe_get_currents(&t, j.data(), j.data() + n, j.data() + 2 * n));
            char name[64];
            snprintf(name, sizeof name, "/cur_%d.bin", currents++);
            FILE* g = fopen((outdir + name).c_str(), "wb");
            if (!g) { fprintf(stderr, "cannot write\n"); return 1; }
            fwrite(j.data(), sizeof(double), 3 * n, g);
            fclose(g);
            printf("J %.17g\n", t);
        } else if (c[0] == 'A') {
            params[4] = atof(c.c_str() + 1);
            CHECK(gpe_set_user_params(5, params));
        } else if (c[0] == 'Y') {
            double mu = 0.0;
            CHECK(gpe_evolve_dipolar(atoi(c.c_str() + 1), &mu));
            printf("MU %.17g\n", mu);
        } else if (c == "W") {
            double t = 0.0, ed = 0.0;
            CHECK(gpe_energy_dipolar2(&t, &ed));
            printf("W %.17g %.17g\n", t, ed);
        } else if (c == "G") {
            CHECK(gpe_get_phase(NULL));
        } else if (c[0] == 'P') {
            double mu = 0.0;
            CHECK(gpe_evolve_enforced_phase(atoi(c.c_str() + 1), &mu));
            printf("MU %.17g\n", mu);
        } else {
            fprintf(stderr, "unknown command %s\n", c.c_str());
            return 1;
        }
        fflush(stdout);
    }
    CHECK(gpe_destroy_engine());
    return 0;
}
