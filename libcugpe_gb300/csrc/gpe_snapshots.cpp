// Wavefunction snapshots in the reference's .dftc format, written while the
// engine keeps evolving.
//
// Format (dev/gpe_io.h:45-104, python/gpe_dftcutils.py:31-56): the .dftc file
// is nom frames of nx*ny*nz complex128 values in C order, appended one after
// the other; `<file>.dftc.info` is a text file of one value per line with a
// trailing comment (system type, mode, nx, ny, nz, dt, nom, a_scattering,
// aspect_ratio, omega_x, r0, npart, total time; reals as %.15e).
//
// Pipeline (replaces the reference's gpe_queue, dev/gpe_queue.h:67-137, whose
// drivers copy psi to a pinned buffer synchronously and let a second OpenMP
// thread fwrite it): a snapshot copies psi on the engine's stream into one of
// `nbuf` device frame buffers (converting the FP32 form to complex128), the
// engine goes on with the next steps, a side stream copies the frame to a
// pinned host buffer, and a writer thread appends it to the file once that
// copy has finished.  A push waits only when all `nbuf` frames are still in
// flight.
#include <cuda_runtime.h>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "gpe_gb300.h"

struct gpe_gb_snapshots {
    gpe_gb_engine* e = nullptr;
    FILE* f = nullptr;
    int device = 0;
    size_t bytes = 0;
    int nbuf = 0;
    cudaStream_t side = nullptr;
    std::vector<void*> dev, host;
    std::vector<cudaEvent_t> done;
    std::vector<bool> busy;
    std::deque<int> queue;  // frames whose host copy is issued, in push order
    std::mutex m;
    std::condition_variable cv;
    std::thread writer;
    bool stop = false;
    int err = 0;
    long long frames = 0;
};

static void release(gpe_gb_snapshots* s) {
    for (void* p : s->dev) if (p) cudaFree(p);
    for (void* p : s->host) if (p) cudaFreeHost(p);
    for (cudaEvent_t ev : s->done) if (ev) cudaEventDestroy(ev);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->f) fclose(s->f);
    delete s;
}

static void writer_loop(gpe_gb_snapshots* s) {
    cudaSetDevice(s->device);
    for (;;) {
        int k;
        {
            std::unique_lock<std::mutex> lk(s->m);
            s->cv.wait(lk, [s] { return s->stop || !s->queue.empty(); });
            if (s->queue.empty()) return;  // stop requested and nothing left
            k = s->queue.front();
            s->queue.pop_front();
        }
        int rc = (int)cudaEventSynchronize(s->done[k]);
        if (rc == 0 && fwrite(s->host[k], 1, s->bytes, s->f) != s->bytes) rc = GPE_ERR_IO;
        {
            std::lock_guard<std::mutex> lk(s->m);
            if (rc && !s->err) s->err = rc;
            if (!rc) s->frames++;
            s->busy[k] = false;
        }
        s->cv.notify_all();
    }
}

extern "C" {

int gpe_gb_snapshots_open(gpe_gb_snapshots** out, gpe_gb_engine* e, const char* dftc_path, int nbuf) {
    if (!out) return GPE_ERR_ARGUMENT;
    *out = nullptr;
    if (!e) return GPE_ERR_NO_ENGINE;
    if (!dftc_path || nbuf < 1 || nbuf > 64) return GPE_ERR_ARGUMENT;
    int nx, ny, nz;
    int rc = gpe_gb_get_lattice(e, &nx, &ny, &nz);
    if (rc) return rc;
    gpe_gb_snapshots* s = new gpe_gb_snapshots;
    s->e = e;
    s->bytes = (size_t)nx * ny * nz * 2 * sizeof(double);
    s->nbuf = nbuf;
    s->f = fopen(dftc_path, "wb");
    if (!s->f) { release(s); return GPE_ERR_IO; }
    cudaError_t ce = cudaGetDevice(&s->device);
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
    s->dev.assign(nbuf, nullptr);
    s->host.assign(nbuf, nullptr);
    s->done.assign(nbuf, nullptr);
    s->busy.assign(nbuf, false);
    for (int k = 0; k < nbuf && ce == cudaSuccess; k++) {
        ce = cudaMalloc(&s->dev[k], s->bytes);
        if (ce == cudaSuccess) ce = cudaHostAlloc(&s->host[k], s->bytes, cudaHostAllocDefault);
        if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&s->done[k], cudaEventDisableTiming);
    }
    if (ce != cudaSuccess) { release(s); return (int)ce; }
    s->writer = std::thread(writer_loop, s);
    *out = s;
    return 0;
}

int gpe_gb_snapshots_push(gpe_gb_snapshots* s, double* t) {
    if (!s) return GPE_ERR_ARGUMENT;
    int k = -1;
    {
        std::unique_lock<std::mutex> lk(s->m);
        if (s->err) return s->err;
        s->cv.wait(lk, [s, &k] {
            for (int i = 0; i < s->nbuf; i++)
                if (!s->busy[i]) { k = i; return true; }
            return s->err != 0;
        });
        if (s->err) return s->err;
        s->busy[k] = true;
    }
    // frame copy on the engine's stream (it synchronises that stream once the frame is in place)
    int rc = gpe_gb_get_psi_device(s->e, t, s->dev[k]);
    cudaError_t ce = cudaSuccess;
    if (!rc) ce = cudaMemcpyAsync(s->host[k], s->dev[k], s->bytes, cudaMemcpyDeviceToHost, s->side);
    if (!rc && ce == cudaSuccess) ce = cudaEventRecord(s->done[k], s->side);
    if (!rc && ce != cudaSuccess) rc = (int)ce;
    {
        std::lock_guard<std::mutex> lk(s->m);
        if (rc) {
            s->busy[k] = false;
            if (!s->err) s->err = rc;
        } else {
            s->queue.push_back(k);
        }
    }
    s->cv.notify_all();
    return rc;
}

int gpe_gb_snapshots_close(gpe_gb_snapshots* s, long long* frames) {
    if (!s) return GPE_ERR_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(s->m);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->writer.joinable()) s->writer.join();
    int rc = s->err;
    if (frames) *frames = s->frames;
    if (fflush(s->f) != 0 && !rc) rc = GPE_ERR_IO;
    release(s);
    return rc;
}

int gpe_gb_dftc_write_info(const char* dftc_path, const char* system, const char* mode, int nx, int ny, int nz,
                           double dt, int nom, double a_scat, double aspect_ratio, double omega_x, double r0,
                           double npart, double total_time) {
    if (!dftc_path || !system || !mode) return GPE_ERR_ARGUMENT;
    std::string name = std::string(dftc_path) + ".info";
    FILE* f = fopen(name.c_str(), "w");
    if (!f) return GPE_ERR_IO;
    // line layout of gpe_save_info (dev/gpe_io.h:45-104)
    int bad = 0;
    bad |= fprintf(f, "%s   # system type\n", system) < 0;
    bad |= fprintf(f, "%s   # mode\n", mode) < 0;
    bad |= fprintf(f, "%d   # nx\n", nx) < 0;
    bad |= fprintf(f, "%d   # ny\n", ny) < 0;
    bad |= fprintf(f, "%d   # nz\n", nz) < 0;
    bad |= fprintf(f, "%.15e   # dt\n", dt) < 0;
    bad |= fprintf(f, "%d   # nom\n", nom) < 0;
    bad |= fprintf(f, "%.15e   # a_scattering\n", a_scat) < 0;
    bad |= fprintf(f, "%.15e   # aspect_ratio\n", aspect_ratio) < 0;
    bad |= fprintf(f, "%.15e   # omega_x\n", omega_x) < 0;
    bad |= fprintf(f, "%.15e   # r0\n", r0) < 0;
    bad |= fprintf(f, "%.15e   # npart\n", npart) < 0;
    bad |= fprintf(f, "%.15e   # total time\n", total_time) < 0;
    bad |= fclose(f) != 0;
    return bad ? GPE_ERR_IO : 0;
}

int gpe_gb_dftc_read_info(const char* dftc_path, char* system, char* mode, int len, int* nx, int* ny, int* nz,
                          double* dt, int* nom, double* a_scat, double* aspect_ratio, double* omega_x, double* r0,
                          double* npart, double* total_time) {
    if (!dftc_path || !nx || !ny || !nz || !dt || !nom || !a_scat || !aspect_ratio || !omega_x || !r0 || !npart)
        return GPE_ERR_ARGUMENT;
    std::string name = std::string(dftc_path) + ".info";
    FILE* f = fopen(name.c_str(), "r");
    if (!f) return GPE_ERR_IO;
    char line[256];
    auto next = [&]() -> bool { return fgets(line, sizeof line, f) != nullptr; };
    auto word = [&](char* dst) {  // first token of the line
        if (!dst || len <= 0) return;
        char tok[256] = {0};
        if (sscanf(line, "%255s", tok) != 1) tok[0] = 0;
        snprintf(dst, (size_t)len, "%s", tok);
    };
    // field order of gpe_get_info (dev/gpe_io.h:130-166)
    int ok = 1;
    ok &= next(); word(system);
    ok &= next(); word(mode);
    ok &= next() && sscanf(line, "%d", nx) == 1;
    ok &= next() && sscanf(line, "%d", ny) == 1;
    ok &= next() && sscanf(line, "%d", nz) == 1;
    ok &= next() && sscanf(line, "%lf", dt) == 1;
    ok &= next() && sscanf(line, "%d", nom) == 1;
    ok &= next() && sscanf(line, "%lf", a_scat) == 1;
    ok &= next() && sscanf(line, "%lf", aspect_ratio) == 1;
    ok &= next() && sscanf(line, "%lf", omega_x) == 1;
    ok &= next() && sscanf(line, "%lf", r0) == 1;
    ok &= next() && sscanf(line, "%lf", npart) == 1;
    if (total_time) {
        *total_time = 0.0;
        if (next()) sscanf(line, "%lf", total_time);
    }
    fclose(f);
    return ok ? 0 : GPE_ERR_IO;
}

}  // extern "C"
