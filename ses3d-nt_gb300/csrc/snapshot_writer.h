// Background writer of volume snapshots. The stepping thread copies a field
// from the device into one of a few pinned host buffers (cudaMemcpyAsync on
// its own stream) and queues the buffer with an event recorded after the
// copy; this writer waits for the event, converts the element-local copy to
// the reference raw layout (float32, Fortran order) and writes the file, so
// that file output overlaps the following time steps. The reference does the
// same with non-blocking MPI-IO (src/output_raw.f90:129-168).
#pragma once

#include <cuda_runtime.h>

#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace sesnt {

class SnapshotWriter {
public:
    SnapshotWriter() = default;
    SnapshotWriter(const SnapshotWriter &) = delete;
    SnapshotWriter &operator=(const SnapshotWriter &) = delete;
    ~SnapshotWriter();

    // Sizes the pool (nbuf pinned buffers of `bytes`) and starts the thread on
    // `device`. Idempotent once started. Returns 0 or a SESNT_* error.
    int start(int device, size_t bytes, int nbuf, std::string &err);
    bool started() const { return started_; }
    // A free pinned buffer; blocks while every buffer is queued for writing.
    void *acquire();
    // Queues the write of `buf` (element-local [nel][NP] of `esize`-byte
    // reals) to `path` once `ev` (owned by the writer from here) completed.
    void submit(void *buf, cudaEvent_t ev, int nx, int ny, int nz, int lpd, int esize, const std::string &path,
                bool override);
    // Waits until the queue is empty; returns the first error since the last
    // call (0 if none) with its message.
    int wait(std::string &err);

private:
    struct Job {
        void *buf;
        cudaEvent_t ev;
        int nx, ny, nz, lpd, esize;
        std::string path;
        bool override;
    };
    void run();
    void release(void *buf);

    int device_ = 0;
    bool started_ = false, stop_ = false;
    std::vector<void *> all_, free_;
    std::deque<Job> queue_;
    int busy_ = 0;
    int err_code_ = 0;
    std::string err_msg_;
    std::vector<float> fortran_;  // writer-thread conversion buffer
    std::mutex mu_;
    std::condition_variable cv_work_, cv_free_, cv_idle_;
    std::thread thread_;
};

}  // namespace sesnt
