/*
 * Frame queue of the reference drivers: the evolving thread copies psi into
 * one of a few pinned host buffers and queues it, a writer thread takes frames
 * off the queue and writes them out (dev/gpe_queue.h:42-137, used by
 * test_vortex/rte_vortex.c:59-90, 312-370).
 *
 * Same names and call pattern as the reference header, so such a driver
 * compiles against this library unchanged: the global `wf_queue` (defined by
 * the driver), `flag_stop`, create_gpe_queue / get_gpe_queue_buffer /
 * add_to_gpe_queue / take_off_gpe_queue / destroy_gpe_queue, and
 * `wf_queue.q.empty()` / `.size()` for the writer's polling loop.  Differences:
 * the queue is guarded by a mutex and add_to_gpe_queue waits on a condition
 * variable instead of spinning, and `flag_stop` is atomic, so the two threads
 * never race on the queue (the reference's std::queue and flag are shared
 * without synchronisation).  `cplx` is std::complex<double>, which has the
 * layout of the reference's C99 `double complex` and of cuCplx.
 *
 * The library's own snapshot pipeline (gpe_gb_snapshots_*, include/gpe_gb300.h)
 * does the same job without a host copy on the evolving thread.
 */
#ifndef GPE_QUEUE_H
#define GPE_QUEUE_H

#include <atomic>
#include <complex>
#include <condition_variable>
#include <mutex>
#include <queue>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <cuda_runtime.h>

#include "gpe_engine.h"

typedef std::complex<double> cplx;

/* The writer thread polls this flag (with an empty queue) to know that no more frames will come. */
inline std::atomic<uint8_t> flag_stop{0};

/* The queue of frames: the std::queue operations the reference drivers use, each under a lock. */
class gpe_frame_queue {
  public:
    bool empty() const {
        std::lock_guard<std::mutex> g(m_);
        return q_.empty();
    }
    size_t size() const {
        std::lock_guard<std::mutex> g(m_);
        return q_.size();
    }
    cplx* front() const {
        std::lock_guard<std::mutex> g(m_);
        return q_.front();
    }
    void push(cplx* psi) {
        {
            std::lock_guard<std::mutex> g(m_);
            q_.push(psi);
        }
        cv_.notify_all();
    }
    void pop() {
        {
            std::lock_guard<std::mutex> g(m_);
            q_.pop();
        }
        cv_.notify_all();
    }
    /* Pushes once fewer than `limit - 1` frames are queued (the reference's admission rule; a
     * one-frame queue admits a frame when it is empty, where the reference would wait forever). */
    void push_when_below(cplx* psi, size_t limit) {
        const size_t lim = limit < 2 ? 2 : limit;
        std::unique_lock<std::mutex> g(m_);
        cv_.wait(g, [&] { return q_.size() + 1 < lim; });
        q_.push(psi);
        g.unlock();
        cv_.notify_all();
    }
    void clear() {
        std::lock_guard<std::mutex> g(m_);
        std::queue<cplx*>().swap(q_);
    }

  private:
    mutable std::mutex m_;
    std::condition_variable cv_;
    std::queue<cplx*> q_;
};

typedef struct {
    gpe_frame_queue q;
    uint16_t counter;
    uint16_t max_size;
    cplx** data;
} gpe_queue;

/* defined by the driver: `gpe_queue wf_queue;` */
extern gpe_queue wf_queue;

/* Allocates `queue_size` pinned frames of nxyz points (at most 5, as the reference).  Returns the
 * only frame when the queue holds one, else NULL; exits on an allocation failure, as the reference. */
static inline void* create_gpe_queue(const uint64_t nxyz, uint16_t queue_size = 5) {
    const uint16_t queue_max_size = 5;
    wf_queue.q.clear();
    wf_queue.counter = 0;
    if (queue_size > queue_max_size) {
        printf("Error: Queue buffer is too big! Truncating queue size to %d\n", queue_max_size);
        queue_size = queue_max_size;
    }
    if (queue_size == 0) queue_size = 1;
    printf("GPE Queue size (wavefunctions to be buffered at once): %u\n", queue_size);
    wf_queue.max_size = queue_size;
    wf_queue.data = (cplx**)malloc(queue_size * sizeof(cplx*));
    if (!wf_queue.data) {
        printf("Error: Cannot allocate memory for gpe_queue!\n");
        exit(EXIT_FAILURE);
    }
    for (uint16_t i = 0; i < queue_size; i++) {
        void* p = nullptr;
        if (cudaHostAlloc(&p, sizeof(cplx) * nxyz, cudaHostAllocDefault) != cudaSuccess) {
            printf("Error: Cannot allocate memory for gpe_queue!\n");
            exit(EXIT_FAILURE);
        }
        wf_queue.data[i] = static_cast<cplx*>(p);
    }
    flag_stop = 0;
    return queue_size == 1 ? (void*)wf_queue.data[0] : NULL;
}

/* The frame the next gpe_get_psi should fill (frames are used round robin). */
static inline cplx* get_gpe_queue_buffer() { return wf_queue.data[wf_queue.counter % wf_queue.max_size]; }

/* Queues a filled frame; waits while the queue is full. */
static inline void add_to_gpe_queue(cplx* psi) {
    wf_queue.q.push_when_below(psi, wf_queue.max_size);
    wf_queue.counter++;
}

/* Takes the oldest frame off the queue (the caller checked that it is not empty). */
static inline cplx* take_off_gpe_queue() {
    cplx* psi = wf_queue.q.front();
    wf_queue.q.pop();
    return psi;
}

/* Frees the frames and raises flag_stop; exits on a CUDA failure, as the reference. */
static inline void destroy_gpe_queue() {
    for (uint16_t i = 0; i < wf_queue.max_size; i++) {
        if (cudaFreeHost(wf_queue.data[i]) != cudaSuccess) {
            printf("Error: Cannot free the memory of gpe_queue!\n");
            exit(EXIT_FAILURE);
        }
    }
    flag_stop = 1;
    free(wf_queue.data);
    wf_queue.data = NULL;
}

#endif /* GPE_QUEUE_H */
