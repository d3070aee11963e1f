// Background writer of volume snapshots (see snapshot_writer.h).
#include "snapshot_writer.h"

#include <cstdio>

#include "sesnt.h"

namespace sesnt {

SnapshotWriter::~SnapshotWriter() {
    if (started_) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_work_.notify_all();
        thread_.join();
    }
    for (void *b : all_) cudaFreeHost(b);
}

int SnapshotWriter::start(int device, size_t bytes, int nbuf, std::string &err) {
    if (started_) return SESNT_OK;
    device_ = device;
    for (int q = 0; q < nbuf; ++q) {
        void *p = nullptr;
        cudaError_t e = cudaMallocHost(&p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            err = std::string("cudaMallocHost for snapshot buffers: ") + cudaGetErrorString(e);
            for (void *b : all_) cudaFreeHost(b);
            all_.clear();
            return SESNT_ENOMEM;
        }
        all_.push_back(p);
    }
    free_ = all_;
    thread_ = std::thread(&SnapshotWriter::run, this);
    started_ = true;
    return SESNT_OK;
}

void *SnapshotWriter::acquire() {
    std::unique_lock<std::mutex> lk(mu_);
    cv_free_.wait(lk, [&] { return !free_.empty(); });
    void *b = free_.back();
    free_.pop_back();
    return b;
}

void SnapshotWriter::release(void *buf) {
    {
        std::lock_guard<std::mutex> lk(mu_);
        free_.push_back(buf);
    }
    cv_free_.notify_one();
}

void SnapshotWriter::submit(void *buf, cudaEvent_t ev, int nx, int ny, int nz, int lpd, int esize,
                            const std::string &path, bool override) {
    {
        std::lock_guard<std::mutex> lk(mu_);
        queue_.push_back({buf, ev, nx, ny, nz, lpd, esize, path, override});
    }
    cv_work_.notify_one();
}

int SnapshotWriter::wait(std::string &err) {
    std::unique_lock<std::mutex> lk(mu_);
    cv_idle_.wait(lk, [&] { return queue_.empty() && busy_ == 0; });
    const int rc = err_code_;
    if (rc) err = err_msg_;
    err_code_ = 0;
    err_msg_.clear();
    return rc;
}

void SnapshotWriter::run() {
    cudaSetDevice(device_);
    for (;;) {
        Job job;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_work_.wait(lk, [&] { return stop_ || !queue_.empty(); });
            if (queue_.empty()) return;  // stop requested and nothing left
            job = queue_.front();
            queue_.pop_front();
            ++busy_;
        }
        int rc = SESNT_OK;
        std::string msg;
        cudaError_t e = cudaEventSynchronize(job.ev);
        cudaEventDestroy(job.ev);
        if (e != cudaSuccess) {
            rc = SESNT_ECUDA;
            msg = std::string("snapshot copy: ") + cudaGetErrorString(e);
        } else {
            const int P = job.lpd + 1, NP = P * P * P;
            const long long nel = (long long)job.nx * job.ny * job.nz;
            fortran_.resize((size_t)nel * NP);
            // element-local [e][p] -> raw layout [p][e] (element x fastest)
            for (long long el = 0; el < nel; ++el)
                for (int p = 0; p < NP; ++p) {
                    const size_t src = (size_t)el * NP + p;
                    fortran_[(size_t)p * nel + el] = job.esize == 8 ? (float)((const double *)job.buf)[src]
                                                                    : ((const float *)job.buf)[src];
                }
            rc = sesnt_write_raw_field(job.path.c_str(), job.nx, job.ny, job.nz, job.lpd, fortran_.data(),
                                       job.override ? 1 : 0);
            if (rc) msg = std::string("snapshot ") + job.path + ": " + sesnt_io_last_error();
        }
        release(job.buf);
        {
            std::lock_guard<std::mutex> lk(mu_);
            if (rc && !err_code_) {
                err_code_ = rc;
                err_msg_ = msg;
            }
            --busy_;
        }
        cv_idle_.notify_all();
    }
}

}  // namespace sesnt
