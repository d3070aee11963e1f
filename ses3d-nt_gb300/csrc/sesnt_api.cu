// C ABI of the GB300 time step (include/sesnt.h): handle management, model
// import and FP64 precompute, source/receiver bookkeeping, step launches
// (direct or replayed from a captured CUDA graph), and readback in the
// reference raw layout.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <limits>
#include <sstream>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/sesnt.h"
#include "sesnt_internal.h"
#include "snapshot_writer.h"

using namespace sesnt;


namespace sesnt {
template <>
const LpdOps<float> *lpd_ops<float>(int lpd) {
    switch (lpd) {
        case 2: return lpd_ops_n<2, float>();
        case 3: return lpd_ops_n<3, float>();
        case 4: return lpd_ops_n<4, float>();
        case 5: return lpd_ops_n<5, float>();
        case 6: return lpd_ops_n<6, float>();
        case 7: return lpd_ops_n<7, float>();
        default: return nullptr;
    }
}
template <>
const LpdOps<double> *lpd_ops<double>(int lpd) {
    switch (lpd) {
        case 2: return lpd_ops_n<2, double>();
        case 3: return lpd_ops_n<3, double>();
        case 4: return lpd_ops_n<4, double>();
        case 5: return lpd_ops_n<5, double>();
        case 6: return lpd_ops_n<6, double>();
        case 7: return lpd_ops_n<7, double>();
        default: return nullptr;
    }
}
}  // namespace sesnt

namespace {

thread_local std::string g_create_error;

// NVTX range over one API call (visible in Nsight timelines; a no-op
// without a profiler attached).
struct Range {
    explicit Range(const char *name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
};

__global__ void k_set_it(int *d_it, int v) { *d_it = v; }

// One component of the element-blocked stress / memory-variable state
// (StateLayout: `unit` values per (element, simulation), components `cs`
// apart from `src`) as an element-local field [e][NP] of simulation `sim`.
template <typename T>
__global__ void k_extract(const T *__restrict__ src, int S, long long unit, int cs, int sim, int c, int NP,
                          long long nel, T *__restrict__ out) {
    const size_t li = (size_t)blockIdx.x * 256 + threadIdx.x;
    if (li >= (size_t)nel * NP) return;
    const size_t e = li / NP, p = li % NP;
    out[li] = src[(e * S + sim) * (size_t)unit + (size_t)c * cs + p];
}
__global__ void k_advance_it(int *d_it, int by) { *d_it += by; }

// out[e*NP + p] = in[p*nel + e]: reference raw layout -> element-major, via
// 32x32 shared-memory tiles so both sides stay coalesced.
template <typename T>
__global__ void k_import(const float *__restrict__ in, T *__restrict__ out, int NP, long long nel) {
    __shared__ float tile[32][33];
    const long long e0 = (long long)blockIdx.x * 32, p0 = (long long)blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += 8) {
        long long p = p0 + r, e = e0 + threadIdx.x;
        if (p < NP && e < nel) tile[r][threadIdx.x] = in[p * nel + e];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) {
        long long e = e0 + r, p = p0 + threadIdx.x;
        if (p < NP && e < nel) out[e * NP + p] = (T)tile[threadIdx.x][r];
    }
}

// Model checks on a raw host array staged on the device, before anything of
// the handle changes. res[0]: smallest index that fails the check (mode 0:
// not positive or not finite, rhoinv; mode 1: not finite, lambda and mu), or
// ~0; res[1]: 1 if any value differs from `other` (mode 2: q differs from
// FLT_MAX, i.e. attenuation is on; mode 3: a nonzero anisotropy term).
constexpr int kCheckBlocks = 4 * 152;  // grid-stride blocks of k_check_model
__global__ void k_check_model(const float *__restrict__ x, long long n, int mode, float other,
                              unsigned long long *res) {
    bool any = false;
    unsigned long long first = ~0ull;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float v = x[i];
        if (mode <= 1) {
            const bool ok = isfinite(v) && (mode == 1 || v > 0.0f);
            if (!ok && (unsigned long long)i < first) first = (unsigned long long)i;
        } else if (v != other) {
            any = true;
        }
    }
    if (mode <= 1) {
        if (first != ~0ull) atomicMin(res, first);
    } else if (__any_sync(0xffffffffu, any) && (threadIdx.x & 31) == 0) {
        atomicOr(res + 1, 1ull);
    }
}

// tau = 6.0814 * q^-1.015 (src/model_paras.F90:407), evaluated in FP64, in
// place over the element-major q. One thread per element walks its NP
// points and evaluates the power only where q differs from the previous
// point's, so a per-element Q costs one FP64 pow per element; equal inputs
// reuse the identical result.
template <typename T>
__global__ void k_tau(const T *q, T *tau, long long nel, int NP) {
    const long long e = (long long)blockIdx.x * 256 + threadIdx.x;
    if (e >= nel) return;
    const T *qe = q + e * NP;
    T *te = tau + e * NP;
    T last_q = qe[0], last_t = (T)(6.0814 * pow((double)last_q, -1.015));
    for (int p = 0; p < NP; ++p) {
        const T x = qe[p];
        if (x != last_q) {
            last_q = x;
            last_t = (T)(6.0814 * pow((double)x, -1.015));
        }
        te[p] = last_t;
    }
}

// Min, max and a non-finite flag of v (float32 keys), reduced per block
// (shuffles, then shared memory) so that each block makes one atomic per
// word; four independent loads per iteration keep memory busy. The last
// block to finish (counted in mm[3] after a fence) copies the result to
// `out` (mapped host memory, or device memory where that is not had) and
// resets mm for the next call, so a call is one launch and one
// synchronisation. No block waits for another.
// mm: [0] ordered bits of the minimum, [1] of the maximum, [2] non-finite
// flag, [3] finished blocks; all four start at {~0, 0, 0, 0}. out: the
// three result words.
template <typename T>
__global__ void __launch_bounds__(256) k_minmax(const T *v, long long n, unsigned long long *mm,
                                                unsigned long long *out) {
    float lo = INFINITY, hi = -INFINITY;
    int nonfinite = 0;
    auto take = [&](float x) {
        if (!isfinite(x)) nonfinite = 1;
        lo = fminf(lo, x);
        hi = fmaxf(hi, x);
    };
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
        const float x0 = (float)v[i], x1 = (float)v[i + stride], x2 = (float)v[i + 2 * stride],
                    x3 = (float)v[i + 3 * stride];
        take(x0);
        take(x1);
        take(x2);
        take(x3);
    }
    for (; i < n; i += stride) take((float)v[i]);
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        nonfinite |= __shfl_xor_sync(0xffffffffu, nonfinite, o);
    }
    __shared__ float slo[8], shi[8];
    __shared__ int snf[8];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        slo[w] = lo;
        shi[w] = hi;
        snf[w] = nonfinite;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) {
            lo = fminf(lo, slo[q]);
            hi = fmaxf(hi, shi[q]);
            nonfinite |= snf[q];
        }
        auto key = [](float f) -> unsigned long long {
            unsigned b = __float_as_uint(f);
            return (unsigned long long)((b & 0x80000000u) ? ~b : (b | 0x80000000u));
        };
        atomicMin(&mm[0], key(lo));
        atomicMax(&mm[1], key(hi));
        if (nonfinite) atomicOr(&mm[2], 1ULL);
        __threadfence();
        if (atomicAdd(&mm[3], 1ULL) == (unsigned long long)gridDim.x - 1) {
            // every other block's atomics precede its count: the words are final
            __threadfence();
            out[0] = atomicAdd(&mm[0], 0ULL);
            out[1] = atomicAdd(&mm[1], 0ULL);
            out[2] = atomicAdd(&mm[2], 0ULL);
            mm[0] = ~0ULL;
            mm[1] = 0ULL;
            mm[2] = 0ULL;
            mm[3] = 0ULL;
        }
    }
}

// Kinetic energy of one simulation, 0.5*jac*sum over element-local points of
// |v|^2 * r^2 sin(theta) * rho * w_i w_j w_k (src/elastic_vars.F90:218-246).
// Every copy of a shared point carries the same v, and the assembled mass of
// a unique point is the sum of -jac*r^2 sin(theta)*rho*w_i w_j w_k over its
// copies (src/model_paras.F90:410-415), so the sum is -0.5 * sum over unique
// points of |v|^2 / invM: one pass over v and 1/M. Each block sums in FP64
// in a fixed order and writes its partial; the host adds the partials in
// block order, so the result is the same on every call.
template <typename T>
__global__ void __launch_bounds__(256) k_kinetic(const T *__restrict__ v, const T *__restrict__ invM, long long nuni,
                                                 double *__restrict__ partial) {
    double acc = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x; u < nuni; u += stride) {
        const double x = (double)v[u], y = (double)v[nuni + u], z = (double)v[2 * nuni + u];
        acc += (x * x + y * y + z * z) / (double)invM[u];
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double sw[8];
    if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) b += sw[q];
        partial[blockIdx.x] = -0.5 * b;
    }
}

float unkey(unsigned long long k) {
    unsigned b = (unsigned)k;
    b = (b & 0x80000000u) ? (b & 0x7fffffffu) : ~b;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
};

struct HostSource {
    int sim, elem;
    std::vector<float> vm;
    bool present[9];
    std::vector<float> data[9];
};

}  // namespace

// The library's device-memory pool of each device, made at the first
// sesnt_create on that device: it keeps up to kPoolKeep bytes of freed
// buffers mapped for the next handle (the release threshold), and returns the
// rest to the device at each synchronisation. nullptr where none could be
// made (the handles then use cudaMalloc).
constexpr unsigned long long kPoolKeep = 8ull << 30;
cudaMemPool_t library_pool(int device) {
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    static bool tried[64] = {};
    if (device < 0 || device >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!tried[device]) {
        tried[device] = true;
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t p = nullptr;
        unsigned long long keep = kPoolKeep;
        if (cudaMemPoolCreate(&p, &props) == cudaSuccess &&
            cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep) == cudaSuccess) {
            pools[device] = p;
        } else {
            if (p) cudaMemPoolDestroy(p);
            cudaGetLastError();
        }
    }
    return pools[device];
}

// Resident-block budgets of the column kernels (kColsMinb and kCols2Minb in
// element_cols.cuh), for the host's prefetch distances.
constexpr int kColsMinbHost[4] = {4, 5, 6, 8};
constexpr int kCols2MinbHost[4] = {4, 3, 2, 2};

struct sesnt_handle {
    sesnt_grid_t g{};
    int N = 0, P = 0, NP = 0, nel = 0, S = 1;
    long long nloc = 0, nuni = 0;
    int NXU = 0, NYU = 0, NZU = 0;
    bool dbl = false, sls = false, aniso = false, kahan = false, use_graph = true, model_set = false;
    int esize = 4;
    cudaStream_t stream = nullptr;
    // second stream for the small per-step kernels (sources, receivers),
    // forked from and joined back into `stream` within every enqueue
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_src = nullptr, ev_node = nullptr, ev_join = nullptr;
    // progress marks: an event recorded after the step mark_it[q] of the
    // current pass, so a read of step it waits for that step only; reads go
    // through their own stream while later steps keep running
    static constexpr int kMarks = 16;
    cudaEvent_t mark_ev[kMarks] = {};
    int mark_it[kMarks] = {};
    int mark_next = 0;
    cudaStream_t copy_stream = nullptr;
    std::string err;
    std::vector<DevBuf> bufs;
    size_t dev_bytes = 0;
    // device buffers (typed by precision)
    void *tabD = nullptr, *w = nullptr, *sin_t = nullptr, *cot_t = nullptr, *r = nullptr;
    double tabz[2][64] = {};  // host copy of Dz | Dt (rounded to the working precision)
    void *inv_r = nullptr, *inv_sin = nullptr;
    void *px = nullptr, *py = nullptr, *pz = nullptr;
    double *dsin = nullptr, *dr = nullptr, *dw = nullptr;
    void *lam = nullptr, *mu = nullptr, *A = nullptr, *B = nullptr, *C = nullptr, *tau = nullptr;
    void *sig = nullptr, *mem = nullptr, *v = nullptr, *vc = nullptr, *F = nullptr, *invM = nullptr;
    double *F64 = nullptr;  // SESNT_FLAG_FORCE64 on FP32 handles: the force accumulated in FP64
    void *sigc = nullptr;   // SESNT_FLAG_KAHAN_STRESS: stress compensation terms [units][6][CS]
    int *d_it = nullptr;
    int *d_err = nullptr;  // set by a kernel whose bounded wait ran out
    int wait_polls = 1 << 22, drop_completion = 0;
    double dt = 0, c1 = 0, c2 = 0, c3 = 0, jac = 0, alpha = 0, two_over_d[3] = {0, 0, 0};
    // sources and receivers
    std::vector<HostSource> sources;
    bool src_dirty = true;
    void *d_src = nullptr, *d_src_vm = nullptr, *d_src_data = nullptr;
    int nsrc_rec = 0, n_src_vm = 0, n_src_data = 0;
    std::vector<int> rec_elem;
    std::vector<float> rec_vm;
    std::vector<unsigned> rec_mask;
    bool rec_dirty = true;
    int *d_rec_elem = nullptr;
    void *d_rec_vm = nullptr, *d_seis = nullptr;
    int nrec_dev = 0;
    // float32 mirror of d_seis in mapped pinned host memory, written by the
    // receiver kernel: sesnt_get_samples reads a finished step from it with
    // no device copy. Made with the receiver upload when it takes at most
    // kEagerMirrorBytes, else by the first sesnt_get_samples call (null
    // until then, or if mapped memory could not be had: seis_mirror_failed).
    float *h_seis = nullptr, *h_seis_dev = nullptr;
    size_t h_seis_n = 0;
    bool seis_mirror_failed = false;
    // receiver channels beyond vx, vy, vz: per receiver the device-computed
    // channel bits, first trace slot and rotation-strain slot; per (sim,
    // receiver) the source record of its element
    std::vector<int> rec_xslot;
    std::vector<SrcRec> src_recs;
    unsigned *d_rec_xmask = nullptr;
    int *d_rec_xslot = nullptr, *d_rec_rot = nullptr, *d_rec_src = nullptr, *d_rot_elems = nullptr;
    void *d_xseis = nullptr, *d_rot_rec = nullptr;
    int nxtr = 0, nrot = 0;
    // optional state: displacement gradient [S][9][nloc] (SESNT_FLAG_STRAIN)
    // and the rotation strain of the whole volume [S][6][nloc]
    void *du = nullptr, *rot_full = nullptr;
    int rot_full_it = -1;  // step whose rotation strain rot_full holds
    int last_it = 0;       // last step enqueued
    // volume snapshots
    struct Snapshot {
        int sim, which, start, inc, end;
        std::string prefix, attribute;
        bool override;
    };
    std::vector<Snapshot> snaps;
    void *snap_stage = nullptr;
    int device = 0;
    std::unique_ptr<SnapshotWriter> writer;
    // graph
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    cudaGraphExec_t graph1 = nullptr;  // one step, for sesnt_step
    cudaGraphExec_t graph1a = nullptr; // one step that advances the step counter (first runs)
    // graphs of 16, 8, 4 and 2 steps that advance the step counter, for the
    // remainder of a run below kGraphSteps (index log2(steps) - 1), built
    // when a run first needs them
    static constexpr int kLadder = 4;
    cudaGraphExec_t ladder[kLadder] = {};
    // v_ptp: device reduction words and the mapped host words of the result
    unsigned long long *d_ptp = nullptr, *h_ptp = nullptr, *h_ptp_dev = nullptr;
    // element-kernel variant (ElementVariant), its argument and the bulk-copy
    // piece size: the launch rules by default, set by sesnt_tune (or the
    // tuning cache under SESNT_FLAG_AUTOTUNE) or sesnt_set_element_variant
    int variant = kVarAuto, variant_arg = 0, piece = 8192;
    std::string tune_report;
    // kinetic energy: per-block partial sums (kinetic_blocks doubles)
    double *d_kin = nullptr;
    int sms = 0;  // multiprocessors of the handle's device (grid sizes of the reductions)

    // events for timing
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int launches_per_step = 0;

    int fail(int code, const char *fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char *what) {
        return fail(SESNT_ECUDA, "%s: %s", what, cudaGetErrorString(e));
    }
    // After a synchronisation: the error word written by a kernel whose
    // bounded completion wait ran out (the tensor-core element kernel).
    // Whether an element kernel of this handle has bounded device-side waits
    // (tensor-core, persistent bulk-copy, or the staged SLS kernel of degrees
    // 4-7), i.e. whether the error word can be set without the bounds check.
    bool bounded_waits() const;
    int wait_status() {
#ifndef SESNT_BOUNDS_CHECK
        if (!bounded_waits()) return SESNT_OK;
#endif
        int word = 0;
        cudaError_t e = cudaMemcpy(&word, d_err, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "reading the error word");
        if (word & 2) return fail(SESNT_ERANGE, "bounds check: a kernel index was outside its buffer");
        if (word) return fail(SESNT_ETIMEOUT, "a bounded completion wait of the element kernel ran out; the results of this run are invalid");
        return SESNT_OK;
    }
    // Device buffers come from the library's memory pool on the handle's
    // device (stream-ordered allocation on the handle's stream, complete
    // before the call returns), or from cudaMalloc where no pool could be
    // made. The pool keeps up to kPoolKeep bytes of freed buffers mapped, so
    // the next handle's buffers need no new mapping: a model set-up right
    // after another handle was destroyed took 25-30 ms instead of 2.5 ms.
    cudaMemPool_t pool = nullptr;
    int alloc(void **out, size_t bytes, const char *what) {
        void *p = nullptr;
        if (bytes == 0) bytes = 16;
        cudaError_t e = pool ? cudaMallocFromPoolAsync(&p, bytes, pool, stream) : cudaMalloc(&p, bytes);
        if (e == cudaSuccess && pool) {
            e = cudaStreamSynchronize(stream);  // usable from every stream, also the legacy default one
            if (e != cudaSuccess) {
                cudaFreeAsync(p, stream);
                p = nullptr;
            }
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(SESNT_ENOMEM, "allocation of %zu bytes for %s failed: %s", bytes, what,
                        cudaGetErrorString(e));
        }
        bufs.push_back({p, bytes});
        dev_bytes += bytes;
        *out = p;
        return SESNT_OK;
    }
    void release(void *p) {
        if (!p) return;
        for (size_t i = 0; i < bufs.size(); ++i)
            if (bufs[i].p == p) {
                dev_bytes -= bufs[i].n;
                free_buffer(p);
                bufs.erase(bufs.begin() + i);
                return;
            }
    }
    // After the handle's work that uses p (all of it is ordered on or joined into `stream`).
    void free_buffer(void *p) {
        if (pool) cudaFreeAsync(p, stream);
        else cudaFree(p);
    }
    void clear_marks() {
        for (int &m : mark_it) m = -1;
    }
    void mark(int it) {
        if (!mark_ev[mark_next] || cudaEventRecord(mark_ev[mark_next], stream) != cudaSuccess) return;
        mark_it[mark_next] = it;
        mark_next = (mark_next + 1) % kMarks;
    }
    // layout of the stress and memory-variable units (StateLayout)
    size_t state_unit() const { return sesnt::state_unit(NP, sls ? kNsls : 0); }
    int state_cs() const { return sesnt::state_cs(NP, sls); }
    void drop_graph() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        graph_steps = 0;
        if (graph1) cudaGraphExecDestroy(graph1);
        graph1 = nullptr;
        if (graph1a) cudaGraphExecDestroy(graph1a);
        graph1a = nullptr;
        for (cudaGraphExec_t &l : ladder) {
            if (l) cudaGraphExecDestroy(l);
            l = nullptr;
        }
    }
    void free_seis_mirror() {
        if (h_seis) cudaFreeHost(h_seis);
        h_seis = h_seis_dev = nullptr;
        h_seis_n = 0;
    }
    ~sesnt_handle() {
        drop_graph();
        if (stream) cudaStreamSynchronize(stream);
        writer.reset();  // writes what is queued, then joins
        free_seis_mirror();
        if (h_ptp) cudaFreeHost(h_ptp);
        for (auto &b : bufs) free_buffer(b.p);
        if (pool && stream) cudaStreamSynchronize(stream);  // the buffers are back in the pool
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        for (cudaEvent_t ev : {ev_fork, ev_src, ev_node, ev_join})
            if (ev) cudaEventDestroy(ev);
        for (cudaEvent_t ev : mark_ev)
            if (ev) cudaEventDestroy(ev);
        if (side) cudaStreamDestroy(side);
        if (copy_stream) cudaStreamDestroy(copy_stream);
        if (stream) cudaStreamDestroy(stream);
    }

    template <typename T>
    StepArgs<T> args() const {
        StepArgs<T> a{};
        a.nx = g.nx; a.ny = g.ny; a.nz = g.nz; a.nel = nel; a.S = S;
        a.NXU = NXU; a.NYU = NYU; a.NZU = NZU; a.nuni = nuni; a.nloc = nloc;
        a.dt = (T)dt; a.c1 = (T)c1; a.c2 = (T)c2; a.c3 = (T)c3; a.jac = (T)jac; a.alpha = (T)alpha;
        a.inv_alpha = alpha > 0 ? (T)(1.0 / alpha) : T(0);
        for (int q = 0; q < kNsls; ++q) {
            a.tau_p[q] = (T)kTauP[q];
            a.mem_rate[q] = (T)(dt / kTauP[q]);
            a.mem_drive[q] = (T)(dt / (kNsls * kTauP[q]));
        }
        a.inv_r = (const T *)inv_r; a.inv_sin = (const T *)inv_sin;
        for (int q = 0; q < 64; ++q) {
            a.tabz[0][q] = (T)tabz[0][q];
            a.tabz[1][q] = (T)tabz[1][q];
        }
        a.tabD = (const T *)tabD; a.w = (const T *)w; a.sin_t = (const T *)sin_t; a.cot_t = (const T *)cot_t;
        a.r = (const T *)r; a.px = (const T *)px; a.py = (const T *)py; a.pz = (const T *)pz;
        a.lam = (const T *)lam; a.mu = (const T *)mu; a.A = (const T *)A; a.B = (const T *)B; a.C = (const T *)C;
        a.tau = (const T *)tau;
        a.sig = (T *)sig; a.mem = (T *)mem; a.v = (T *)v; a.vc = (T *)vc; a.F = (T *)F; a.invM = (const T *)invM;
        a.F64 = F64;
        a.sigc = (T *)sigc;
        a.st_cs = state_cs(); a.st_unit = (long long)state_unit();
        a.nsrc = nsrc_rec; a.nt = g.nt; a.n_src_vm = n_src_vm; a.n_src_data = n_src_data; a.src = (const SrcRec *)d_src; a.src_vm = (const T *)d_src_vm;
        a.src_data = (const T *)d_src_data;
        a.nrec = nrec_dev; a.rec_elem = d_rec_elem; a.rec_vm = (const T *)d_rec_vm; a.seis = (T *)d_seis;
        a.seis_host = h_seis_dev;
        a.d_it = d_it; a.step_off = 0;
        a.persistent = (g.flags & SESNT_FLAG_PERSISTENT_ELEMENT) ? 1 : 0;
        a.pair = (g.flags & SESNT_FLAG_NO_PAIR) ? 0 : 1;
        a.stage = (g.flags & SESNT_FLAG_NO_STAGE) ? 0 : 1;
        a.contraction = (g.flags & SESNT_FLAG_TC_TF32X3) ? 1 : ((g.flags & SESNT_FLAG_TC_BF16X3) ? 2 : 0);
        a.variant = variant;
        a.variant_arg = variant_arg;
        a.piece = piece;
        {
            // L2 prefetch distance: 0, 1/4, 1/2 or 1 wave of resident blocks, in
            // units of the kernel: the staged kernel has 8 blocks of one
            // (element, simulation) unit per SM; the column kernels the budget
            // of arg bits 0-1 with G units per block ((element, simulation
            // pair) units for k_element_cols2)
            static const int kQuarters[4] = {0, 1, 2, 4};
            if (variant == kVarColumns || variant == kVarColumnsStaged || variant == kVarColumnsPair) {
                const int pp = (N + 1) * (N + 1), gpb = pp <= 128 ? 128 / pp : 1;
                const int minb = dbl ? 1 : (variant == kVarColumnsPair ? kCols2MinbHost : kColsMinbHost)[variant_arg & 3];
                a.prefetch = kQuarters[(variant_arg >> 2) & 3] * minb * gpb * sms / 4;
            } else if (variant == kVarAuto) {
                // the launch rules' staged kernel prefetches half a wave ahead at degree 4 in
                // FP32 (config 2: 0.2552 -> 0.2422 ms per element launch); at degree 6 it is slower
                a.prefetch = (sls && N == 4 && !dbl) ? 2 * 8 * sms / 4 : 0;
            } else {
                a.prefetch = kQuarters[(variant_arg >> 1) & 3] * 8 * sms / 4;
            }
        }
        a.two_over_d[0] = (T)two_over_d[0];
        a.two_over_d[1] = (T)two_over_d[1];
        a.two_over_d[2] = (T)two_over_d[2];
        a.err = d_err;
        a.wait_polls = wait_polls;
        a.drop_completion = drop_completion;
        a.du = (T *)du;
        a.rec_xmask = nxtr > 0 ? d_rec_xmask : nullptr;
        a.rec_xslot = d_rec_xslot; a.rec_rot = d_rec_rot; a.rec_src = d_rec_src;
        a.xseis = (T *)d_xseis; a.rot_rec = (const T *)d_rot_rec; a.nxtr = nxtr; a.nrot = nrot;
        return a;
    }
};

namespace sesnt {
const sesnt_grid *handle_grid(const sesnt_handle *h) { return &h->g; }
int handle_device(const sesnt_handle *h) { return h->device; }
int handle_fail(sesnt_handle *h, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    h->err = buf;
    return code;
}
}  // namespace sesnt

namespace {

int check_grid(const sesnt_grid_t *g, std::string &why) {
    char b[256];
    auto bad = [&](const char *m) { why = m; return SESNT_EINVAL; };
    if (!g) return bad("grid is NULL");
    // src/config/config.F90:106-115, 168-179, 214-217
    if (g->nx < 4 || g->ny < 4 || g->nz < 4) return bad("nx, ny and nz must be at least 4");
    if (g->lpd < kMinLpd || g->lpd > kMaxLpd) {
        snprintf(b, sizeof b, "lpd=%d not supported (this library is built for lpd %d..%d)", g->lpd, kMinLpd,
                 kMaxLpd);
        why = b;
        return SESNT_EUNSUPPORTED;
    }
    if (g->taper_width < 0 || 2 * g->taper_width + 1 > std::min(g->nx, std::min(g->ny, g->nz)))
        return bad("taper_width too wide (2*taper_width+1 must not exceed nx, ny, nz)");
    if (!(g->lat_min <= g->lat_max) || !(g->lon_min <= g->lon_max) || !(g->rad_min <= g->rad_max))
        return bad("domain bounds out of order");
    if (!(std::fabs(g->lat_min) <= 90.f && std::fabs(g->lat_max) <= 90.f)) return bad("invalid latitude");
    if (!(std::fabs(g->lon_min) <= 180.f && std::fabs(g->lon_max) <= 180.f)) return bad("invalid longitude");
    if (!(g->rad_min >= 1.0f && g->rad_max >= 1.0f)) return bad("invalid radius");
    if (g->nt < 2 || g->nt > 50000) return bad("nt must be in [2, 50000]");
    if (!(g->dt > 0.0f)) return bad("dt must be positive");
    if (g->taper_width > 0 && !(g->taper_slope > 0.0f)) return bad("taper_slope must be positive");
    if (g->n_sls != 0 && g->n_sls != kNsls) return bad("n_sls must be 0 or 3");
    if (g->precision != 4 && g->precision != 8) return bad("precision must be 4 (FP32) or 8 (FP64)");
    if ((g->flags & (SESNT_FLAG_TC_TF32X3 | SESNT_FLAG_TC_BF16X3)) == (SESNT_FLAG_TC_TF32X3 | SESNT_FLAG_TC_BF16X3))
        return bad("choose one tensor-core contraction mode");
    if ((g->flags & (SESNT_FLAG_TC_TF32X3 | SESNT_FLAG_TC_BF16X3)) && g->precision != 4) {
        why = "tensor-core contractions are built for FP32 wavefields only";
        return SESNT_EUNSUPPORTED;
    }
    if ((g->flags & SESNT_FLAG_STRAIN) &&
        (g->flags & (SESNT_FLAG_TC_TF32X3 | SESNT_FLAG_TC_BF16X3 | SESNT_FLAG_PERSISTENT_ELEMENT))) {
        why = "the displacement gradient is built into the default element kernel only";
        return SESNT_EUNSUPPORTED;
    }
    if ((g->flags & SESNT_FLAG_KAHAN_STRESS) && (g->flags & (SESNT_FLAG_TC_TF32X3 | SESNT_FLAG_TC_BF16X3 |
                                                             SESNT_FLAG_PERSISTENT_ELEMENT | SESNT_FLAG_STRAIN))) {
        why = "compensated stress integration is built into the staged and one-point-per-thread kernels only";
        return SESNT_EUNSUPPORTED;
    }
    if (g->batch < 1) return bad("batch must be >= 1");
    const long long P = g->lpd + 1;
    const long long nuni = (g->nx * (long long)g->lpd + 1) * (g->ny * (long long)g->lpd + 1) *
                           (g->nz * (long long)g->lpd + 1);
    const long long nloc = (long long)g->nx * g->ny * g->nz * P * P * P;
    if (nuni >= (1LL << 31) || nloc >= (1LL << 40)) return bad("grid too large for 32-bit unique indices");
    return SESNT_OK;
}

template <typename T>
int upload(sesnt_t *h, void *dst, const std::vector<T> &src, const char *what) {
    cudaError_t e = cudaMemcpy(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? SESNT_OK : h->cuda_fail(e, what);
}

template <typename T>
int setup_tables(sesnt_t *h) {
    const sesnt_grid_t &g = h->g;
    const int N = g.lpd, P = N + 1;
    Domain<T> d = make_domain<T>(g.nx, g.ny, g.nz, g.lat_min, g.lat_max, g.lon_min, g.lon_max, g.rad_min, g.rad_max);
    // FP64 derived quantities from the working-precision domain
    const double dx = (double)d.dx_elm, dy = (double)d.dy_elm, dz = (double)d.dz_elm;
    h->jac = dx * dy * dz / 8.0;                // src/geometric_paras.f90:129
    h->c1 = (2.0 / dx) * h->jac;                // src/evolution.f90:337-339
    h->c2 = (2.0 / dy) * h->jac;
    h->c3 = -((2.0 / dz) * h->jac);
    h->two_over_d[0] = 2.0 / dx;
    h->two_over_d[1] = 2.0 / dy;
    h->two_over_d[2] = 2.0 / dz;
    h->dt = (double)(T)g.dt;
    h->alpha = (double)(T)g.taper_slope;
    std::vector<double> dl = lagrange_derivative_matrix<double>(N);
    std::vector<T> tab(4 * P * P);
    for (int q = 0; q < P; ++q)
        for (int i = 0; i < P; ++i) {
            tab[0 * P * P + q * P + i] = (T)(2.0 * dl[q * P + i] / dx);  // strain, :133-135
            tab[1 * P * P + q * P + i] = (T)(2.0 * dl[q * P + i] / dy);
            tab[2 * P * P + q * P + i] = (T)(2.0 * dl[q * P + i] / dz);
            tab[3 * P * P + i * P + q] = (T)dl[i * P + q];  // divergence, :344-346
        }
    std::vector<double> wd = gll_quadrature_weights<double>(N);
    std::vector<T> wt(P);
    for (int i = 0; i < P; ++i) wt[i] = (T)wd[i];
    std::vector<T> xc = element_coordinates<T>(g.nx, N, d.x_loc_min, d.x_loc_max);
    std::vector<T> zc = element_coordinates<T>(g.nz, N, d.z_loc_max, d.z_loc_min);  // radius decreases with k
    std::vector<T> st(xc.size()), ct(xc.size()), ist(xc.size()), rr(zc.size()), irr(zc.size());
    std::vector<double> dsin(xc.size()), drr(zc.size());
    for (size_t a = 0; a < xc.size(); ++a) {
        const double th = (double)xc[a];
        dsin[a] = std::sin(th);
        st[a] = (T)dsin[a];
        ct[a] = (T)(std::cos(th) / std::sin(th));
        ist[a] = (T)(1.0 / dsin[a]);
    }
    for (size_t a = 0; a < zc.size(); ++a) {
        drr[a] = (double)zc[a];
        rr[a] = zc[a];
        irr[a] = (T)(1.0 / drr[a]);
    }
    std::vector<T> pxv, pyv, pzv;
    taper_profiles<T>(g.nx, g.ny, g.nz, N, g.taper_width, (T)g.taper_slope, d, pxv, pyv, pzv);
    for (int x = 0; x < P * P; ++x) {
        h->tabz[0][x] = (double)tab[2 * P * P + x];
        h->tabz[1][x] = (double)tab[3 * P * P + x];
    }
    int rc;
    if ((rc = upload(h, h->tabD, tab, "tables"))) return rc;
    if ((rc = upload(h, h->w, wt, "weights"))) return rc;
    if ((rc = upload(h, h->sin_t, st, "sin"))) return rc;
    if ((rc = upload(h, h->cot_t, ct, "cot"))) return rc;
    if ((rc = upload(h, h->r, rr, "r"))) return rc;
    if ((rc = upload(h, h->inv_r, irr, "1/r"))) return rc;
    if ((rc = upload(h, h->inv_sin, ist, "1/sin"))) return rc;
    if ((rc = upload(h, h->px, pxv, "px"))) return rc;
    if ((rc = upload(h, h->py, pyv, "py"))) return rc;
    if ((rc = upload(h, h->pz, pzv, "pz"))) return rc;
    if ((rc = upload(h, h->dsin, dsin, "dsin"))) return rc;
    if ((rc = upload(h, h->dr, drr, "dr"))) return rc;
    if ((rc = upload(h, h->dw, wd, "dw"))) return rc;
    return SESNT_OK;
}

template <typename T>
const LpdOps<T> *ops(const sesnt_t *h) {
    return lpd_ops<T>(h->N);
}

}  // namespace

// Whether the element kernel a step launches has bounded device-side waits
// (the staged, persistent, tensor-core and staged-column kernels), i.e.
// whether the error word can be set without the bounds check.
bool sesnt_handle::bounded_waits() const {
    const char *n = dbl ? ops<double>(this)->element_name(args<double>(), sls, aniso)
                        : ops<float>(this)->element_name(args<float>(), sls, aniso);
    return std::strstr(n, "stage") || std::strstr(n, "_tma") || std::strstr(n, "_tc");
}

namespace {

int zero_state(sesnt_t *h) {
    const size_t E = h->esize;
    struct Z { void *p; size_t n; } zs[] = {
        {h->sig, E * h->state_unit() * (size_t)h->nel * h->S},  // with the memory variables (StateLayout)
        {h->v, E * 3 * (size_t)h->nuni * h->S},
        {h->vc, h->kahan ? E * 3 * (size_t)h->nuni * h->S : 0},
        {h->F, E * 3 * (size_t)h->nuni * h->S},
        {h->F64, h->F64 ? 8 * 3 * (size_t)h->nuni * h->S : 0},
        {h->sigc, h->sigc ? E * 6 * (size_t)h->state_cs() * h->nel * h->S : 0},
        {h->d_seis, E * (size_t)h->S * h->rec_elem.size() * 3 * h->g.nt},
        {h->d_xseis, E * (size_t)h->S * h->nxtr * h->g.nt},
        {h->du, E * 9 * (size_t)h->nloc * h->S},
        {h->h_seis_dev, h->h_seis_n * sizeof(float)}};
    for (auto &z : zs)
        if (z.p && z.n) {
            cudaError_t e = cudaMemsetAsync(z.p, 0, z.n, h->stream);
            if (e != cudaSuccess) return h->cuda_fail(e, "zeroing state");
        }
    h->rot_full_it = -1;
    h->last_it = 0;
    h->clear_marks();
    return SESNT_OK;
}

// Resolve sources per (simulation, element): for each component the last
// registered source defining it wins (the reference assigns element slabs,
// src/config/channel_mod.f90:866-867), then upload.
template <typename T>
int upload_sources(sesnt_t *h) {
    h->release(h->d_src); h->release(h->d_src_vm); h->release(h->d_src_data);
    h->d_src = h->d_src_vm = h->d_src_data = nullptr;
    h->nsrc_rec = 0;
    h->src_dirty = false;
    h->src_recs.clear();
    if (h->sources.empty()) return SESNT_OK;
    std::vector<SrcRec> recs;
    std::vector<T> vm, data;
    int nvm = 0, ndata = 0;
    std::vector<std::vector<int>> data_row(h->sources.size(), std::vector<int>(9, -1));
    for (size_t s = 0; s < h->sources.size(); ++s) {
        const HostSource &hs = h->sources[s];
        for (float x : hs.vm) vm.push_back((T)x);
        for (int c = 0; c < 9; ++c)
            if (hs.present[c]) {
                for (float x : hs.data[c]) data.push_back((T)x);
                data_row[s][c] = ndata++;
            }
        ++nvm;
    }
    for (size_t s = 0; s < h->sources.size(); ++s) {
        const HostSource &hs = h->sources[s];
        SrcRec *r = nullptr;
        for (auto &x : recs)
            if (x.sim == hs.sim && x.elem == hs.elem) r = &x;
        if (!r) {
            SrcRec nr{};
            nr.sim = hs.sim;
            nr.elem = hs.elem;
            for (int c = 0; c < 9; ++c) nr.vm[c] = nr.data[c] = -1;
            recs.push_back(nr);
            r = &recs.back();
        }
        for (int c = 0; c < 9; ++c)
            if (hs.present[c]) {
                r->vm[c] = (int)s;
                r->data[c] = data_row[s][c];
            }
    }
    int rc;
    if ((rc = h->alloc(&h->d_src, recs.size() * sizeof(SrcRec), "source records"))) return rc;
    if ((rc = h->alloc(&h->d_src_vm, vm.size() * sizeof(T), "source weights"))) return rc;
    if ((rc = h->alloc(&h->d_src_data, std::max<size_t>(1, data.size()) * sizeof(T), "source data"))) return rc;
    h->src_recs = recs;
    cudaError_t e = cudaMemcpy(h->d_src, recs.data(), recs.size() * sizeof(SrcRec), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_src_vm, vm.data(), vm.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !data.empty())
        e = cudaMemcpy(h->d_src_data, data.data(), data.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return h->cuda_fail(e, "uploading sources");
    h->nsrc_rec = (int)recs.size();
    h->n_src_vm = nvm;
    h->n_src_data = ndata;
    return SESNT_OK;
}

// Device tables of the receiver channels beyond vx, vy, vz (rotation rates,
// recorded source fields): trace slots in receiver order, so traces of
// receivers registered earlier keep their slots and samples.
constexpr unsigned kDeviceChannels = 0xFFF0u;

template <typename T>
int upload_receiver_channels(sesnt_t *h) {
    const size_t nrec = h->rec_elem.size();
    std::vector<unsigned> xm(nrec);
    std::vector<int> slot(nrec), rot(nrec, -1), rot_elems;
    int nx = 0;
    for (size_t r = 0; r < nrec; ++r) {
        xm[r] = h->rec_mask[r] & kDeviceChannels;
        slot[r] = nx;
        nx += __builtin_popcount(xm[r]);
        if (xm[r] & (SESNT_CH_ROT_VX | SESNT_CH_ROT_VY | SESNT_CH_ROT_VZ)) {
            rot[r] = (int)rot_elems.size();
            rot_elems.push_back(h->rec_elem[r]);
        }
    }
    const size_t nt = h->g.nt, S = h->S;
    std::vector<T> old;
    const int old_nx = h->nxtr;
    if (h->d_xseis && old_nx > 0) {
        old.resize(S * old_nx * nt);
        cudaError_t e = cudaMemcpy(old.data(), h->d_xseis, old.size() * sizeof(T), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return h->cuda_fail(e, "reading receiver traces");
    }
    for (void *p : {(void *)h->d_rec_xmask, (void *)h->d_rec_xslot, (void *)h->d_rec_rot, (void *)h->d_rot_elems,
                    h->d_xseis, h->d_rot_rec})
        h->release(p);
    h->d_rec_xmask = nullptr;
    h->d_rec_xslot = h->d_rec_rot = h->d_rot_elems = nullptr;
    h->d_xseis = h->d_rot_rec = nullptr;
    h->nxtr = h->nrot = 0;
    h->rec_xslot = slot;
    if (nx == 0) return SESNT_OK;
    int rc;
    if ((rc = h->alloc((void **)&h->d_rec_xmask, nrec * sizeof(unsigned), "receiver channels")) ||
        (rc = h->alloc((void **)&h->d_rec_xslot, nrec * sizeof(int), "receiver trace slots")) ||
        (rc = h->alloc((void **)&h->d_rec_rot, nrec * sizeof(int), "receiver rotation slots")) ||
        (rc = h->alloc((void **)&h->d_rot_elems, std::max<size_t>(1, rot_elems.size()) * sizeof(int),
                       "rotation elements")) ||
        (rc = h->alloc(&h->d_rot_rec, std::max<size_t>(1, S * 6 * rot_elems.size() * h->NP) * sizeof(T),
                       "rotation strain")) ||
        (rc = h->alloc(&h->d_xseis, S * nx * nt * sizeof(T), "receiver traces")))
        return rc;
    std::vector<T> xs(S * nx * nt, T(0));
    for (size_t s = 0; s < S && old_nx > 0; ++s)
        std::copy(old.begin() + s * old_nx * nt, old.begin() + (s + 1) * old_nx * nt, xs.begin() + s * nx * nt);
    cudaError_t e = cudaMemcpy(h->d_rec_xmask, xm.data(), nrec * sizeof(unsigned), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_rec_xslot, slot.data(), nrec * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_rec_rot, rot.data(), nrec * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !rot_elems.empty())
        e = cudaMemcpy(h->d_rot_elems, rot_elems.data(), rot_elems.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_xseis, xs.data(), xs.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return h->cuda_fail(e, "uploading receiver channels");
    h->nxtr = nx;
    h->nrot = (int)rot_elems.size();
    return SESNT_OK;
}

// Source record of each (simulation, receiver element), for the recorded
// source-field channels.
int upload_receiver_sources(sesnt_t *h) {
    h->release(h->d_rec_src);
    h->d_rec_src = nullptr;
    if (h->nxtr == 0) return SESNT_OK;
    const size_t nrec = h->rec_elem.size();
    std::vector<int> rs((size_t)h->S * nrec, -1);
    for (size_t q = 0; q < h->src_recs.size(); ++q)
        for (size_t r = 0; r < nrec; ++r)
            if (h->src_recs[q].elem == h->rec_elem[r]) rs[(size_t)h->src_recs[q].sim * nrec + r] = (int)q;
    int rc;
    if ((rc = h->alloc((void **)&h->d_rec_src, rs.size() * sizeof(int), "receiver sources"))) return rc;
    cudaError_t e = cudaMemcpy(h->d_rec_src, rs.data(), rs.size() * sizeof(int), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? SESNT_OK : h->cuda_fail(e, "uploading receiver sources");
}

// Host mirrors of the seismograms up to this size are made with the
// receiver upload; larger ones (batched runs with many receivers and steps)
// only when per-step samples are first read.
constexpr size_t kEagerMirrorBytes = 16u << 20;

template <typename T>
int upload_receivers(sesnt_t *h) {
    h->rec_dirty = false;
    const size_t nrec = h->rec_elem.size();
    if (nrec == (size_t)h->nrec_dev && h->d_seis) return SESNT_OK;
    // keep already recorded samples of existing receivers
    std::vector<T> old;
    const size_t per = (size_t)3 * h->g.nt;
    if (h->d_seis) {
        cudaError_t e = cudaStreamSynchronize(h->stream);  // no step still writes the old buffers
        if (e != cudaSuccess) return h->cuda_fail(e, "synchronize");
    }
    if (h->d_seis && h->nrec_dev > 0) {
        old.resize((size_t)h->S * h->nrec_dev * per);
        cudaError_t e = cudaMemcpy(old.data(), h->d_seis, old.size() * sizeof(T), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return h->cuda_fail(e, "reading seismograms");
    }
    h->release(h->d_rec_elem); h->release(h->d_rec_vm); h->release(h->d_seis);
    h->d_rec_elem = nullptr; h->d_rec_vm = h->d_seis = nullptr;
    h->free_seis_mirror();
    h->nrec_dev = 0;
    if (nrec == 0) return SESNT_OK;
    int rc;
    if ((rc = h->alloc((void **)&h->d_rec_elem, nrec * sizeof(int), "receiver elements"))) return rc;
    if ((rc = h->alloc(&h->d_rec_vm, nrec * h->NP * sizeof(T), "receiver weights"))) return rc;
    if ((rc = h->alloc(&h->d_seis, (size_t)h->S * nrec * per * sizeof(T), "seismograms"))) return rc;
    std::vector<T> vm(h->rec_vm.begin(), h->rec_vm.end());
    std::vector<T> seis((size_t)h->S * nrec * per, T(0));
    if (!old.empty()) {
        const size_t oldn = old.size() / ((size_t)h->S * per);
        for (int s = 0; s < h->S; ++s)
            std::copy(old.begin() + (size_t)s * oldn * per, old.begin() + (size_t)(s + 1) * oldn * per,
                      seis.begin() + (size_t)s * nrec * per);
    }
    cudaError_t e = cudaMemcpy(h->d_rec_elem, h->rec_elem.data(), nrec * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_rec_vm, vm.data(), vm.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_seis, seis.data(), seis.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return h->cuda_fail(e, "uploading receivers");
    h->seis_mirror_failed = false;
    if (seis.size() * sizeof(float) <= kEagerMirrorBytes) {
        void *hm = nullptr, *hd = nullptr;
        if (cudaHostAlloc(&hm, seis.size() * sizeof(float), cudaHostAllocMapped) == cudaSuccess &&
            cudaHostGetDevicePointer(&hd, hm, 0) == cudaSuccess) {
            h->h_seis = (float *)hm;
            h->h_seis_dev = (float *)hd;
            h->h_seis_n = seis.size();
            for (size_t x = 0; x < seis.size(); ++x) h->h_seis[x] = (float)seis[x];
        } else {
            if (hm) cudaFreeHost(hm);
            cudaGetLastError();  // made (or given up) at the first sesnt_get_samples
        }
    }
    h->nrec_dev = (int)nrec;
    int rc2 = upload_receiver_channels<T>(h);
    return rc2 ? rc2 : upload_receiver_sources(h);
}

template <typename T>
int prepare_run(sesnt_t *h) {
    if (!h->model_set) return h->fail(SESNT_ESTATE, "sesnt_set_model must be called before stepping");
    int rc;
    const bool changed = h->src_dirty || h->rec_dirty;
    if (h->src_dirty) {
        h->drop_graph();
        if ((rc = upload_sources<T>(h))) return rc;
    }
    if (h->rec_dirty) {
        h->drop_graph();
        if ((rc = upload_receivers<T>(h))) return rc;
    }
    if (changed && (rc = upload_receiver_sources(h))) return rc;
    return SESNT_OK;
}

// Enqueue steps [it, it+n) given that *d_it == it. Per step:
//   main:  [whole-volume rotation strain]  element ............ node
//   side:  [receiver rotation strain]  sources ........ ^        `-> receivers
// The source slab only adds into the force that the element kernel also adds
// into, so it runs beside it; the receivers of step it read the velocity the
// element kernel of step it+1 only reads, so they overlap that launch. The
// node kernel waits for the side stream's sources (and, through the side
// stream's order, the previous receivers). Side is joined back into main at
// the end, also inside a graph capture.
template <typename T>
int enqueue_steps(sesnt_t *h, int n, bool rot_full = false) {
    const LpdOps<T> *o = ops<T>(h);
    StepArgs<T> a = h->args<T>();
    rot_full = rot_full || (h->g.flags & SESNT_FLAG_ROTATION);
    auto launch_fail = [&](const char *what) {
        return h->fail(SESNT_ECUDA, "%s kernel launch failed: %s", what, cudaGetErrorString(cudaGetLastError()));
    };
    cudaError_t e = cudaSuccess;
    for (int q = 0; q < n; ++q) {
        a.step_off = q;
        if ((e = cudaEventRecord(h->ev_fork, h->stream)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(h->side, h->ev_fork, 0)) != cudaSuccess)
            return h->cuda_fail(e, "fork");
        // rotation strain of the receivers' elements from the velocity before this step's update
        if (h->nrot > 0 && o->rot_strain(a, h->d_rot_elems, h->nrot, (T *)h->d_rot_rec, h->side))
            return launch_fail("rotation-strain");
        if (o->sources(a, h->side)) return launch_fail("source");
        if (rot_full && o->rot_strain(a, nullptr, h->nel, (T *)h->rot_full, h->stream))
            return launch_fail("rotation-strain");
        if (o->element(a, h->sls, h->aniso, h->stream)) return launch_fail("element");
        if ((e = cudaEventRecord(h->ev_src, h->side)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(h->stream, h->ev_src, 0)) != cudaSuccess)
            return h->cuda_fail(e, "join before the node update");
        if (o->node(a, h->kahan, h->stream)) return launch_fail("node");
        if ((e = cudaEventRecord(h->ev_node, h->stream)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(h->side, h->ev_node, 0)) != cudaSuccess)
            return h->cuda_fail(e, "fork after the node update");
        if (o->receivers(a, h->side)) return launch_fail("receiver");
    }
    if ((e = cudaEventRecord(h->ev_join, h->side)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(h->stream, h->ev_join, 0)) != cudaSuccess)
        return h->cuda_fail(e, "join");
    return SESNT_OK;
}

constexpr int kGraphSteps = 32;

// Captures n steps starting at the step counter into *exec; with `advance`
// the graph ends by advancing the counter by n (graphs replayed back to back
// within one run), without it the counter is left as it was (the one-step
// graph of sesnt_step, whose run sets the counter first).
template <typename T>
int capture_steps(sesnt_t *h, int n, cudaGraphExec_t *exec, bool advance) {
    cudaGraph_t gr = nullptr;
    cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return h->cuda_fail(e, "cudaStreamBeginCapture");
    int rc = enqueue_steps<T>(h, n);
    if (!rc && advance) k_advance_it<<<1, 1, 0, h->stream>>>(h->d_it, n);
    e = cudaStreamEndCapture(h->stream, &gr);
    if (rc) {
        if (gr) cudaGraphDestroy(gr);
        return rc;
    }
    if (e != cudaSuccess) return h->cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(exec, gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) {
        *exec = nullptr;
        return h->cuda_fail(e, "cudaGraphInstantiate");
    }
    return SESNT_OK;
}

template <typename T>
int build_graph(sesnt_t *h) {
    int rc = capture_steps<T>(h, kGraphSteps, &h->graph, true);
    if (rc) return rc;
    h->graph_steps = kGraphSteps;
    return SESNT_OK;
}

// Every graph a run of this handle can replay (runs of kGraphSteps, the
// 16/8/4/2-step ladder and the single step), captured after a run's own
// launches, so that the host captures while the device executes them and
// later runs, of any length, replay without capturing.
template <typename T>
int prebuild_graphs(sesnt_t *h) {
    int rc;
    if (!h->graph && (rc = build_graph<T>(h))) return rc;
    for (int q = 0; q < sesnt_handle::kLadder; ++q)
        if (!h->ladder[q] && (rc = capture_steps<T>(h, 2 << q, &h->ladder[q], true))) return rc;
    if (!h->graph1 && (rc = capture_steps<T>(h, 1, &h->graph1, false))) return rc;
    if (!h->graph1a && (rc = capture_steps<T>(h, 1, &h->graph1a, true))) return rc;
    return SESNT_OK;
}

// Steps it0 .. it0+nsteps-1 (prepared): graph replays (runs of kGraphSteps,
// then the remainder as graphs of 16, 8, 4, 2 and 1 steps, so a short run
// costs at most five graph launches), or direct launches without graphs.
// A run of 2..31 steps launched directly measured about 15 us per step slower
// than replayed (config 2: 0.302 against 0.287 ms): the per-step stream
// fork and join cost more as launches than as graph edges.
// A chunk whose graph the handle has not captured yet (its first runs)
// replays a one-step graph instead, which costs a fraction of a 16- or
// 32-step capture, so the device starts at once; the 32-step graph is
// captured while the device runs that first chunk, and prebuild_graphs
// captures the rest after the run's launches.
template <typename T>
int run_steps(sesnt_t *h, int it0, int nsteps) {
    int rc;
    k_set_it<<<1, 1, 0, h->stream>>>(h->d_it, it0);
    int left = nsteps;
    auto replay1 = [&](int n) -> int {
        if (!h->graph1a && (rc = capture_steps<T>(h, 1, &h->graph1a, true))) return rc;
        for (int q = 0; q < n; ++q) {
            cudaError_t e = cudaGraphLaunch(h->graph1a, h->stream);
            if (e != cudaSuccess) return h->cuda_fail(e, "cudaGraphLaunch");
        }
        return SESNT_OK;
    };
    if (h->use_graph && nsteps >= kGraphSteps) {
        while (left >= kGraphSteps) {
            if (!h->graph) {
                if ((rc = replay1(kGraphSteps))) return rc;
                if ((rc = build_graph<T>(h))) return rc;
            } else {
                cudaError_t e = cudaGraphLaunch(h->graph, h->stream);
                if (e != cudaSuccess) return h->cuda_fail(e, "cudaGraphLaunch");
            }
            left -= kGraphSteps;
            h->mark(it0 + nsteps - left - 1);
        }
    }
    for (int q = sesnt_handle::kLadder - 1; h->use_graph && q >= 0; --q) {
        const int n = 2 << q;  // 16, 8, 4, 2
        if (left < n) continue;
        if (!h->ladder[q]) {
            if ((rc = replay1(n))) return rc;
        } else {
            cudaError_t e = cudaGraphLaunch(h->ladder[q], h->stream);
            if (e != cudaSuccess) return h->cuda_fail(e, "cudaGraphLaunch");
        }
        left -= n;
        h->mark(it0 + nsteps - left - 1);
    }
    if (left == 1 && h->use_graph) {
        // a single step (the last of a run, or the sesnt_step loop of a
        // driver): one graph launch
        if (!h->graph1 && (rc = capture_steps<T>(h, 1, &h->graph1, false))) return rc;
        cudaError_t e = cudaGraphLaunch(h->graph1, h->stream);
        if (e != cudaSuccess) return h->cuda_fail(e, "cudaGraphLaunch");
        h->mark(it0 + nsteps - 1);
        left = 0;
    }
    if (left > 0) {
        if ((rc = enqueue_steps<T>(h, left))) return rc;
        h->mark(it0 + nsteps - 1);
    }
    if (h->use_graph && (rc = prebuild_graphs<T>(h))) return rc;
    h->last_it = it0 + nsteps - 1;
    if (h->g.flags & SESNT_FLAG_ROTATION) h->rot_full_it = h->last_it;
    return SESNT_OK;
}

// volume_snapshot_cls%process (src/volume_snapshot.f90:123-135)
bool snapshot_due(const sesnt_handle::Snapshot &q, int it) {
    return it >= q.start && it <= q.end && (it - q.start) % q.inc == 0;
}

// First step in [it, last] at which a snapshot is due, or last + 1.
int next_snapshot_step(const sesnt_t *h, int it, int last) {
    int best = last + 1;
    for (const auto &q : h->snaps) {
        int c = it <= q.start ? q.start : q.start + ((it - q.start + q.inc - 1) / q.inc) * q.inc;
        if (c <= q.end && c < best) best = c;
    }
    return best;
}

bool is_rotation(int which) { return which >= SESNT_FIELD_ROT_VX && which <= SESNT_FIELD_ROT_VZ; }

// Enqueues field `which` of simulation `sim` as an element-local array on the
// handle's stream: either computed into `scratch` or a pointer into the state.
// Sets *inverse when the host must invert the values (the mass matrix).
template <typename T>
int field_source(sesnt_t *h, int sim, int which, T *scratch, const T **out, bool *inverse) {
    const LpdOps<T> *o = ops<T>(h);
    StepArgs<T> a = h->args<T>();
    const size_t nloc = (size_t)h->nloc, nuni = (size_t)h->nuni;
    *out = scratch;
    *inverse = false;
    int rc = 0;
    if (which >= 0 && which <= 2) {
        rc = o->gather_local(a, (const T *)h->v + ((size_t)sim * 3 + which) * nuni, scratch, h->stream);
    } else if (which >= 3 && which <= 8) {
        k_extract<T><<<(unsigned)((nloc + 255) / 256), 256, 0, h->stream>>>(
            (const T *)h->sig, h->S, (long long)h->state_unit(), h->state_cs(), sim, which - 3, h->NP, h->nel, scratch);
        rc = cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
    } else if (which == SESNT_FIELD_TAPER) {
        rc = o->taper_local(a, scratch, h->stream);
    } else if (which == SESNT_FIELD_MASS) {
        rc = o->gather_local(a, (const T *)h->invM, scratch, h->stream);
        *inverse = true;
    } else if (which >= SESNT_FIELD_MEMORY && which < SESNT_FIELD_MEMORY + 6 * kNsls && h->sls) {
        // memory variable (component c, mechanism q) at slot c*kNsls + q
        k_extract<T><<<(unsigned)((nloc + 255) / 256), 256, 0, h->stream>>>(
            (const T *)h->mem, h->S, (long long)h->state_unit(), h->state_cs(), sim, which - SESNT_FIELD_MEMORY, h->NP,
            h->nel, scratch);
        rc = cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
    } else if (which == SESNT_FIELD_PRESSURE) {
        rc = o->derived(a, which, sim, nullptr, scratch, h->stream);
    } else if (which >= SESNT_FIELD_EXX && which <= SESNT_FIELD_EZZ) {
        if (!h->du) return h->fail(SESNT_ESTATE, "strain fields need SESNT_FLAG_STRAIN at sesnt_create");
        rc = o->derived(a, which, sim, nullptr, scratch, h->stream);
    } else if (is_rotation(which)) {
        if (!h->rot_full || h->rot_full_it != h->last_it || h->last_it < 1)
            return h->fail(SESNT_ESTATE, "rotation fields need SESNT_FLAG_ROTATION, or a rotation snapshot due at "
                                         "the last step");
        rc = o->derived(a, which, sim, (const T *)h->rot_full, scratch, h->stream);
    } else if (which == SESNT_FIELD_LAMBDA) {
        *out = (const T *)h->lam;
    } else if (which == SESNT_FIELD_MU) {
        *out = (const T *)h->mu;
    } else if (which >= SESNT_FIELD_A && which <= SESNT_FIELD_C) {
        void *src = which == SESNT_FIELD_A ? h->A : (which == SESNT_FIELD_B ? h->B : h->C);
        if (src) {
            *out = (const T *)src;
        } else {
            cudaError_t e = cudaMemsetAsync(scratch, 0, nloc * sizeof(T), h->stream);
            if (e != cudaSuccess) return h->cuda_fail(e, "zeroing field");
        }
    } else {
        return h->fail(SESNT_EINVAL, "unknown or unavailable field %d", which);
    }
    if (rc) return h->fail(SESNT_ECUDA, "field kernel failed: %s", cudaGetErrorString(cudaGetLastError()));
    return SESNT_OK;
}

// After step `it`: copy every snapshot due at `it` into a pinned buffer
// behind the step's kernels and queue it for the writer thread.
template <typename T>
int capture_snapshots(sesnt_t *h, int it) {
    Range r("snapshot capture");
    for (const auto &q : h->snaps) {
        if (!snapshot_due(q, it)) continue;
        const T *src = nullptr;
        bool inverse = false;
        int rc = field_source<T>(h, q.sim, q.which, (T *)h->snap_stage, &src, &inverse);
        if (rc) return rc;
        void *buf = h->writer->acquire();
        cudaError_t e = cudaMemcpyAsync(buf, src, (size_t)h->nloc * sizeof(T), cudaMemcpyDeviceToHost, h->stream);
        cudaEvent_t ev = nullptr;
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(ev, h->stream);
        if (e != cudaSuccess) {
            if (ev) cudaEventDestroy(ev);
            return h->cuda_fail(e, "snapshot copy");
        }
        const std::string path = q.prefix + q.attribute + "_" + std::to_string(it) + ".vol";
        h->writer->submit(buf, ev, h->g.nx, h->g.ny, h->g.nz, h->g.lpd, (int)sizeof(T), path, q.override);
    }
    return SESNT_OK;
}

// The reference forward loop over steps it0 .. it0+nsteps-1: runs of steps
// without snapshots go through run_steps; a step with snapshots due runs on
// its own (with the whole-volume rotation strain when a rotation snapshot is
// due) and is followed by the snapshot copies.
template <typename T>
int run_impl(sesnt_t *h, int it0, int nsteps) {
    if (nsteps <= 0) return SESNT_OK;
    if (it0 < 1 || it0 + nsteps - 1 > h->g.nt)
        return h->fail(SESNT_ERANGE, "steps %d..%d outside 1..nt=%d", it0, it0 + nsteps - 1, h->g.nt);
    int rc;
    if ((rc = prepare_run<T>(h))) return rc;
    if (it0 <= h->last_it) h->clear_marks();  // a step again: earlier marks no longer say "done"
    if (h->snaps.empty()) return run_steps<T>(h, it0, nsteps);
    const int last = it0 + nsteps - 1;
    int it = it0;
    while (it <= last) {
        const int due = next_snapshot_step(h, it, last);
        if (due > it && (rc = run_steps<T>(h, it, due - it))) return rc;
        if (due > last) break;
        bool rot = false;
        for (const auto &q : h->snaps) rot = rot || (is_rotation(q.which) && snapshot_due(q, due));
        k_set_it<<<1, 1, 0, h->stream>>>(h->d_it, due);
        if ((rc = enqueue_steps<T>(h, 1, rot))) return rc;
        h->mark(due);
        h->last_it = due;
        if (rot || (h->g.flags & SESNT_FLAG_ROTATION)) h->rot_full_it = due;
        if ((rc = capture_snapshots<T>(h, due))) return rc;
        it = due + 1;
    }
    return SESNT_OK;
}

int run_any(sesnt_t *h, int it0, int nsteps) {
    return h->dbl ? run_impl<double>(h, it0, nsteps) : run_impl<float>(h, it0, nsteps);
}

// Element-major [e][p] -> reference raw layout [p][e], with conversion.
template <typename TI, typename TO>
void export_layout(const TI *in, TO *out, long long nel, int NP) {
    for (long long e = 0; e < nel; ++e)
        for (int p = 0; p < NP; ++p) out[(size_t)p * nel + e] = (TO)in[(size_t)e * NP + p];
}

template <typename T>
int get_field_impl(sesnt_t *h, int sim, int which, void *out, int out_prec) {
    const size_t nloc = (size_t)h->nloc;
    void *scratch = nullptr;
    int rc;
    if ((rc = h->alloc(&scratch, nloc * sizeof(T), "field scratch"))) return rc;
    const T *src = nullptr;
    bool inverse = false;
    if ((rc = field_source<T>(h, sim, which, (T *)scratch, &src, &inverse))) {
        h->release(scratch);
        return rc;
    }
    std::vector<T> host(nloc);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess) e = cudaMemcpy(host.data(), src, nloc * sizeof(T), cudaMemcpyDeviceToHost);
    h->release(scratch);
    if (e != cudaSuccess) return h->cuda_fail(e, "reading field");
    if (inverse)
        for (auto &x : host) x = T(1) / x;
    if (out_prec == 8) export_layout(host.data(), (double *)out, h->nel, h->NP);
    else export_layout(host.data(), (float *)out, h->nel, h->NP);
    return SESNT_OK;
}

int autotune(sesnt_t *h);

template <typename T>
int set_model_impl(sesnt_t *h, const float *rhoinv, const float *lambda, const float *mu, const float *a,
                   const float *b, const float *c, const float *q) {
    const size_t nloc = (size_t)h->nloc;
    int rc;
    void *stage = nullptr, *checks = nullptr;
    // [array][first bad index, any different]: rhoinv, lambda, mu, q, a, b, c
    const float *arrays[7] = {rhoinv, lambda, mu, q, a, b, c};
    // Every given host array is copied to the device once, into its own slot
    // of the staging buffer; the checks and then the import read it there.
    // One H2D pass instead of two: a check pass and an import pass through a
    // single slot copied the config-2 model (110 MB) twice, 1.2 ms.
    int slot[7], nslots = 0;
    for (int x = 0; x < 7; ++x) slot[x] = arrays[x] ? nslots++ : -1;
    if ((rc = h->alloc(&stage, (size_t)nslots * nloc * sizeof(float), "model staging"))) return rc;
    auto staged = [&](int x) { return (float *)stage + (size_t)slot[x] * nloc; };
    // Checks: the handle is left as it was if the model is rejected.
    const int modes[7] = {0, 1, 1, 2, 3, 3, 3};
    const float others[7] = {0.0f, 0.0f, 0.0f, std::numeric_limits<float>::max(), 0.0f, 0.0f, 0.0f};
    if ((rc = h->alloc(&checks, 7 * 2 * sizeof(unsigned long long), "model checks"))) {
        h->release(stage);
        return rc;
    }
    unsigned long long res[7][2];
    {
        cudaError_t e = cudaSuccess;
        for (int x = 0; x < 7; ++x) {
            res[x][0] = ~0ull;
            res[x][1] = 0;
        }
        e = cudaMemcpyAsync(checks, res, sizeof(res), cudaMemcpyHostToDevice, h->stream);
        for (int x = 0; x < 7 && e == cudaSuccess; ++x) {
            if (!arrays[x]) continue;
            e = cudaMemcpyAsync(staged(x), arrays[x], nloc * sizeof(float), cudaMemcpyHostToDevice, h->stream);
            if (e == cudaSuccess) {
                k_check_model<<<kCheckBlocks, 256, 0, h->stream>>>(staged(x), (long long)nloc, modes[x],
                                                                    others[x], (unsigned long long *)checks + 2 * x);
                e = cudaGetLastError();
            }
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(res, checks, sizeof(res), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        h->release(checks);
        if (e != cudaSuccess) {
            h->release(stage);
            return h->cuda_fail(e, "checking model");
        }
    }
    // attenuation and anisotropy switches (src/evolution.f90:64-74)
    const bool has_q = q && res[3][1] != 0;
    const bool aniso = res[4][1] || res[5][1] || res[6][1];
    const unsigned long long bad = std::min(res[0][0], std::min(res[1][0], res[2][0]));
    const char *why = nullptr;
    if (has_q && !h->sls) why = "model has attenuation (q) but the handle was created with n_sls=0";
    else if (h->sls && !has_q) why = "n_sls=3 needs a q model";
    if (why || bad != ~0ull) {
        h->release(stage);
        if (why) return h->fail(SESNT_EINVAL, "%s", why);
        return h->fail(SESNT_EINVAL, "rhoinv must be positive and lambda, mu finite (first bad point %llu)", bad);
    }
    h->drop_graph();
    // (re)allocate the optional model arrays
    if (aniso && !h->A) {
        if ((rc = h->alloc(&h->A, nloc * sizeof(T), "A"))) return rc;
        if ((rc = h->alloc(&h->B, nloc * sizeof(T), "B"))) return rc;
        if ((rc = h->alloc(&h->C, nloc * sizeof(T), "C"))) return rc;
    }
    h->aniso = aniso;
    void *rho_loc = nullptr;
    if ((rc = h->alloc(&rho_loc, nloc * sizeof(T), "rhoinv"))) { h->release(stage); return rc; }
    dim3 tb(32, 8), tg((unsigned)((h->nel + 31) / 32), (unsigned)((h->NP + 31) / 32));
    // array x (index into `arrays`) from its staging slot into the handle's layout
    auto import = [&](int x, void *dst) -> int {
        k_import<T><<<tg, tb, 0, h->stream>>>(staged(x), (T *)dst, h->NP, h->nel);
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? SESNT_OK : h->cuda_fail(e, "importing model");
    };
    rc = import(0, rho_loc);
    if (!rc) rc = import(1, h->lam);
    if (!rc) rc = import(2, h->mu);
    if (!rc && aniso) {
        auto imp_or_zero = [&](int x, void *dst) -> int {
            if (arrays[x]) return import(x, dst);
            cudaError_t e = cudaMemsetAsync(dst, 0, nloc * sizeof(T), h->stream);
            return e == cudaSuccess ? SESNT_OK : h->cuda_fail(e, "zeroing anisotropy");
        };
        rc = imp_or_zero(4, h->A);
        if (!rc) rc = imp_or_zero(5, h->B);
        if (!rc) rc = imp_or_zero(6, h->C);
    }
    if (!rc && h->sls) {
        rc = import(3, h->tau);  // q imported in place, then mapped to tau
        if (!rc) {
            k_tau<T><<<(unsigned)((h->nel + 255) / 256), 256, 0, h->stream>>>((const T *)h->tau, (T *)h->tau,
                                                                              (long long)h->nel, h->NP);
        }
    }
    if (!rc) {
        StepArgs<T> sa = h->args<T>();
        if (ops<T>(h)->inv_mass(sa, (const T *)rho_loc, h->dsin, h->dr, h->dw, h->jac, h->stream))
            rc = h->fail(SESNT_ECUDA, "inverse mass kernel failed");
    }
    cudaError_t e = cudaStreamSynchronize(h->stream);
    h->release(stage);
    h->release(rho_loc);
    if (rc) return rc;
    if (e != cudaSuccess) return h->cuda_fail(e, "model precompute");
    h->model_set = true;
    if ((rc = zero_state(h))) return rc;
    e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "zeroing state");
    return (h->g.flags & SESNT_FLAG_AUTOTUNE) ? autotune(h) : SESNT_OK;
}

template <typename T>
int get_seis_impl(sesnt_t *h, float *out) {
    const size_t nrec = h->rec_elem.size(), per = (size_t)3 * h->g.nt;
    if (nrec == 0) return SESNT_OK;
    int rc;
    if (h->rec_dirty && (rc = upload_receivers<T>(h))) return rc;
    std::vector<T> host((size_t)h->S * nrec * per);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpy(host.data(), h->d_seis, host.size() * sizeof(T), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return h->cuda_fail(e, "reading seismograms");
    if ((rc = h->wait_status())) return rc;
    for (int s = 0; s < h->S; ++s)
        for (size_t r = 0; r < nrec; ++r)
            for (int c = 0; c < 3; ++c) {
                const bool on = (h->rec_mask[r] >> c) & 1u;
                const size_t base = (((size_t)s * nrec + r) * 3 + c) * h->g.nt;
                for (int t = 0; t < h->g.nt; ++t) out[base + t] = on ? (float)host[base + t] : 0.0f;
            }
    return SESNT_OK;
}

template <typename T>
int v_ptp_impl(sesnt_t *h, int sim, float out[2]) {
    int rc;
    // per call: reduce and copy back on the handle's stream, one
    // synchronisation; the words live in the handle. d_ptp: [0..3] the
    // reduction words, [4..6] the result where mapped host memory is not had.
    if (!h->d_ptp) {
        if ((rc = h->alloc((void **)&h->d_ptp, 8 * sizeof(unsigned long long), "ptp"))) return rc;
        const unsigned long long init[4] = {~0ULL, 0ULL, 0ULL, 0ULL};
        cudaError_t e = cudaMemcpy(h->d_ptp, init, sizeof init, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return h->cuda_fail(e, "v_ptp");
        void *hm = nullptr, *hd = nullptr;
        if (h->h_ptp) {
            // kept from an earlier call
        } else if (cudaHostAlloc(&hm, 3 * sizeof(unsigned long long), cudaHostAllocMapped) == cudaSuccess &&
                   cudaHostGetDevicePointer(&hd, hm, 0) == cudaSuccess) {
            h->h_ptp = (unsigned long long *)hm;
            h->h_ptp_dev = (unsigned long long *)hd;
        } else {
            if (hm) cudaFreeHost(hm);
            cudaGetLastError();  // results come back by copy
        }
    }
    // 8 blocks of 256 threads per SM, each thread 4 loads in flight
    k_minmax<T><<<8 * h->sms, 256, 0, h->stream>>>((const T *)h->v + (size_t)sim * 3 * h->nuni, 3 * h->nuni, h->d_ptp,
                                                h->h_ptp ? h->h_ptp_dev : h->d_ptp + 4);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    unsigned long long res[3];
    if (e == cudaSuccess) {
        if (h->h_ptp) std::memcpy(res, h->h_ptp, sizeof res);
        else e = cudaMemcpy(res, h->d_ptp + 4, sizeof res, cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess) {
        // the words may be left mid-reduction: set them up again next call
        h->release(h->d_ptp);
        h->d_ptp = nullptr;
        return h->cuda_fail(e, "v_ptp");
    }
    out[0] = unkey(res[0]);
    out[1] = unkey(res[1]);
    if (res[2]) return h->fail(SESNT_ENONFINITE, "wavefield of simulation %d contains NaN or Inf", sim);
    return SESNT_OK;
}

template <typename T>
int kinetic_impl(sesnt_t *h, int sim, double *out) {
    const int blocks = 4 * h->sms;  // 4 blocks of 256 threads per SM
    int rc;
    if (!h->d_kin && (rc = h->alloc((void **)&h->d_kin, (size_t)blocks * sizeof(double), "kinetic energy")))
        return rc;
    k_kinetic<T><<<blocks, 256, 0, h->stream>>>((const T *)h->v + (size_t)sim * 3 * h->nuni, (const T *)h->invM,
                                                h->nuni, h->d_kin);
    cudaError_t e = cudaPeekAtLastError();
    std::vector<double> part(blocks);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(part.data(), h->d_kin, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "kinetic_energy");
    double sum = 0.0;
    for (double x : part) sum += x;
    *out = sum;
    if (!std::isfinite(sum)) return h->fail(SESNT_ENONFINITE, "wavefield of simulation %d contains NaN or Inf", sim);
    return SESNT_OK;
}

template <typename T>
int assemble_impl(sesnt_t *h, float *field) {
    const size_t nloc = (size_t)h->nloc, nuni = (size_t)h->nuni;
    void *loc = nullptr, *uni = nullptr, *stage = nullptr;
    int rc;
    if ((rc = h->alloc(&stage, nloc * sizeof(float), "assemble staging"))) return rc;
    if ((rc = h->alloc(&loc, nloc * sizeof(T), "assemble local"))) { h->release(stage); return rc; }
    if ((rc = h->alloc(&uni, nuni * sizeof(T), "assemble unique"))) { h->release(stage); h->release(loc); return rc; }
    dim3 tb(32, 8), tg((unsigned)((h->nel + 31) / 32), (unsigned)((h->NP + 31) / 32));
    cudaError_t e = cudaMemcpy(stage, field, nloc * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemsetAsync(uni, 0, nuni * sizeof(T), h->stream);
    StepArgs<T> a = h->args<T>();
    if (e == cudaSuccess) {
        k_import<T><<<tg, tb, 0, h->stream>>>((const float *)stage, (T *)loc, h->NP, h->nel);
        if (ops<T>(h)->scatter_unique(a, (const T *)loc, (T *)uni, h->stream) ||
            ops<T>(h)->gather_local(a, (const T *)uni, (T *)loc, h->stream))
            e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    }
    std::vector<T> host(nloc);
    if (e == cudaSuccess) e = cudaMemcpy(host.data(), loc, nloc * sizeof(T), cudaMemcpyDeviceToHost);
    h->release(stage); h->release(loc); h->release(uni);
    if (e != cudaSuccess) return h->cuda_fail(e, "assemble_field");
    export_layout(host.data(), field, h->nel, h->NP);
    return SESNT_OK;
}

// ---------------------------------------------------------------------------
// Tuner: element-kernel variant, tile shape and bulk-copy piece size per grid.
// ---------------------------------------------------------------------------
struct TuneChoice {
    int variant, arg, piece;
};

// Candidates for this handle: every element kernel that computes this step
// (tensor-core contractions change the arithmetic and are never chosen):
// one point per thread; paired simulations (even elastic batches); one
// thread per column at each instantiated resident-block count, with the
// stress loaded per point or staged per block, and with two simulations per
// column thread (elastic);
// the staged kernel with bulk or register stores, one copy per unit or 8 KB
// pieces, the stage's wait polled by every thread or by one lane per warp,
// and an L2 prefetch of the state a quarter, half or whole wave of resident
// blocks ahead (SLS);
// the persistent kernel.
std::vector<TuneChoice> tune_candidates(const sesnt_t *h) {
    std::vector<TuneChoice> c = {{kVarPoint, 0, 8192}};
    if (!h->sls) {
        if (h->S % 2 == 0) c.push_back({kVarPair, 0, 8192});
        for (int m = 0; m < 3; ++m)
            for (int q = 0; q < 4; ++q) c.push_back({kVarColumns, m | (q << 2), 8192});
        c.push_back({kVarColumns, 3, 8192});
        for (int m = 0; m < 2; ++m) c.push_back({kVarColumnsStaged, m, 0});
        if (h->S % 2 == 0)
            for (int m = 0; m < 3; ++m)
                for (int q : {0, 2}) c.push_back({kVarColumnsPair, m | (q << 2), 8192});
    } else {
        for (int v : {kVarStage, kVarStageReg}) {
            for (int arg : {0, 1, 2, 4, 6}) c.push_back({v, arg, 0});
            c.push_back({v, 0, 8192});
        }
    }
    for (int piece : {0, 8192}) c.push_back({kVarPersistent, 0, piece});
    return c;
}

std::string tune_key(const sesnt_t *h) {
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, h->device) != cudaSuccess) {
        cudaGetLastError();
        std::snprintf(prop.name, sizeof prop.name, "unknown");
    }
    std::string name = prop.name;
    for (char &ch : name)
        if (ch == ' ' || ch == '|') ch = '_';
    char buf[384];
    std::snprintf(buf, sizeof buf, "%s|sm=%d|lpd=%d|prec=%d|sls=%d|aniso=%d|batch=%d|grid=%dx%dx%d|strain=%d", name.c_str(),
                  h->sms, h->g.lpd, h->g.precision, h->sls ? kNsls : 0, h->aniso ? 1 : 0, h->S, h->g.nx, h->g.ny,
                  h->g.nz, (h->g.flags & SESNT_FLAG_STRAIN) ? 1 : 0);
    return buf;
}

std::string tune_cache_path() {
    const char *p = std::getenv("SESNT_TUNE_CACHE");
    if (p && *p) return p;
    const char *home = std::getenv("HOME");
    if (!home || !*home) return "";
    return std::string(home) + "/.cache/sesnt-tune.txt";
}

// The last entry for `key` in the cache file: "key variant arg piece ms".
bool tune_cache_lookup(const std::string &key, TuneChoice *out) {
    const std::string path = tune_cache_path();
    if (path.empty()) return false;
    std::ifstream f(path);
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        std::string k;
        TuneChoice c{};
        if (is >> k >> c.variant >> c.arg >> c.piece && k == key && c.variant > kVarAuto && c.variant < kVarCount) {
            *out = c;
            found = true;
        }
    }
    return found;
}

void tune_cache_store(const std::string &key, const TuneChoice &c, double ms) {
    const std::string path = tune_cache_path();
    if (path.empty()) return;
    std::error_code ec;  // the cache's directory (e.g. $HOME/.cache) may not exist yet
    const std::filesystem::path dir = std::filesystem::path(path).parent_path();
    if (!dir.empty()) std::filesystem::create_directories(dir, ec);
    std::ofstream f(path, std::ios::app);
    if (f) f << key << ' ' << c.variant << ' ' << c.arg << ' ' << c.piece << ' ' << ms << '\n';
}

// Times every candidate on the handle's own grid: the element kernel alone,
// launched on the zero wavefield (which it leaves exactly zero: zero
// velocity, stress and memory variables give zero rates and zero forces),
// with CUDA events on the handle's stream, a few launches warm and then
// enough launches for at least about 2 ms, best of 3 repeats. The fastest
// becomes the handle's choice; the wavefield is zeroed again afterwards.
template <typename T>
int tune_impl(sesnt_t *h, TuneChoice *best_out, double *best_ms) {
    const LpdOps<T> *o = ops<T>(h);
    // the handle's choice before tuning, restored if tuning fails
    struct Keep {
        sesnt_t *h;
        int variant, arg, piece;
        bool done = false;
        ~Keep() {
            if (!done) {
                h->variant = variant;
                h->variant_arg = arg;
                h->piece = piece;
            }
        }
    } keep{h, h->variant, h->variant_arg, h->piece};
    std::ostringstream rep;
    rep << "tuning " << tune_key(h) << "\n";
    TuneChoice best{kVarAuto, h->variant_arg, h->piece};
    double best_t = 1e30;
    std::vector<std::string> seen;
    for (const TuneChoice &c : tune_candidates(h)) {
        h->variant = c.variant;
        h->variant_arg = c.arg;
        h->piece = c.piece;
        StepArgs<T> a = h->args<T>();
        a.nsrc = 0;
        const std::string name = o->element_name(a, h->sls, h->aniso);
        // a variant the configuration does not have falls back to the rules: skip it
        const bool applicable = (c.variant == kVarPoint && name == "k_element") ||
                                (c.variant == kVarPair && name == "k_element_pair") ||
                                (c.variant == kVarStage && name == "k_element_stage") ||
                                (c.variant == kVarStageReg && name == "k_element_stage (register stores)") ||
                                (c.variant == kVarPersistent && name == "k_element_tma") ||
                                (c.variant == kVarColumns && name == "k_element_cols") ||
                                (c.variant == kVarColumnsStaged && name == "k_element_cols (staged stress)") ||
                                (c.variant == kVarColumnsPair && name == "k_element_cols2");
        if (!applicable) continue;
        // n launches between two events on the handle's stream; milliseconds, or < 0 on an error
        auto timed = [&](int n) -> float {
            float ms = -1.0f;
            if (cudaEventRecord(h->ev0, h->stream) != cudaSuccess) return -1.0f;
            for (int q = 0; q < n; ++q)
                if (o->element(a, h->sls, h->aniso, h->stream)) return -1.0f;
            if (cudaEventRecord(h->ev1, h->stream) != cudaSuccess || cudaEventSynchronize(h->ev1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, h->ev0, h->ev1) != cudaSuccess)
                return -1.0f;
            return ms;
        };
        const float ms1 = timed(2) >= 0.0f ? timed(1) : -1.0f;  // two warm launches, then one timed
        if (ms1 < 0.0f) return h->fail(SESNT_ECUDA, "tuning launch failed: %s", cudaGetErrorString(cudaGetLastError()));
        const int n = std::max(3, std::min(200, (int)(2.0 / std::max(ms1, 1e-3f))));
        double t = 1e30;
        for (int rep_i = 0; rep_i < 3; ++rep_i) {
            const float ms = timed(n);
            if (ms < 0.0f) return h->fail(SESNT_ECUDA, "tuning launch failed: %s", cudaGetErrorString(cudaGetLastError()));
            t = std::min(t, (double)ms / n);
        }
        char line[256];
        std::snprintf(line, sizeof line, "  %-34s variant %d arg %d piece %5d: %.4f ms\n", name.c_str(), c.variant,
                      c.arg, c.piece, t);
        rep << line;
        if (t < best_t) {
            best_t = t;
            best = c;
        }
    }
    int rc = h->wait_status();
    if (rc) return rc;
    h->variant = best.variant;
    h->variant_arg = best.arg;
    h->piece = best.piece;
    keep.done = true;
    char line[160];
    std::snprintf(line, sizeof line, "chosen: variant %d arg %d piece %d (%.4f ms per element launch)\n", best.variant,
                  best.arg, best.piece, best_t);
    rep << line;
    h->tune_report = rep.str();
    *best_out = best;
    *best_ms = best_t;
    if ((rc = zero_state(h))) return rc;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    return e == cudaSuccess ? SESNT_OK : h->cuda_fail(e, "tuning");
}

// Under SESNT_FLAG_AUTOTUNE, after the model is set: the cached choice for
// this GPU and grid, or a tuning run whose result is cached.
int autotune(sesnt_t *h) {
    if (h->g.flags & (SESNT_FLAG_TC_TF32X3 | SESNT_FLAG_TC_BF16X3)) return SESNT_OK;
    const std::string key = tune_key(h);
    TuneChoice c{};
    if (tune_cache_lookup(key, &c)) {
        h->variant = c.variant;
        h->variant_arg = c.arg;
        h->piece = c.piece;
        h->drop_graph();
        h->tune_report = "cached: " + key + "\n";
        return SESNT_OK;
    }
    double ms = 0;
    h->drop_graph();
    const int rc = h->dbl ? tune_impl<double>(h, &c, &ms) : tune_impl<float>(h, &c, &ms);
    if (rc == SESNT_OK) tune_cache_store(key, c, ms);
    return rc;
}

size_t footprint(const sesnt_grid_t *g, bool aniso) {
    const size_t P = g->lpd + 1, NP = P * P * P;
    const size_t nel = (size_t)g->nx * g->ny * g->nz, nloc = nel * NP;
    const size_t nuni = ((size_t)g->nx * g->lpd + 1) * ((size_t)g->ny * g->lpd + 1) * ((size_t)g->nz * g->lpd + 1);
    const size_t E = g->precision == 8 ? 8 : 4, S = g->batch;
    size_t b = 0;
    b += nloc * E * (2 + (aniso ? 3 : 0) + (g->n_sls ? 1 : 0));    // lambda, mu, A,B,C, tau
    b += nel * state_unit((int)NP, g->n_sls ? kNsls : 0) * E * S;  // sigma and memory variables (StateLayout)
    b += nuni * E * (1 + S * (6 + ((g->flags & SESNT_FLAG_KAHAN) ? 3 : 0)));  // invM, v, F, comp
    if ((g->flags & SESNT_FLAG_FORCE64) && E == 4) b += nuni * 8 * 3 * S;     // FP64 force
    if (g->flags & SESNT_FLAG_KAHAN_STRESS)                                     // stress compensation
        b += nel * 6 * (size_t)state_cs((int)NP, g->n_sls != 0) * E * S;
    b += nloc * E * S * (((g->flags & SESNT_FLAG_STRAIN) ? 9 : 0) + ((g->flags & SESNT_FLAG_ROTATION) ? 6 : 0));
    // set_model (transient): a float32 staging slot per model array, and rhoinv in the handle's layout
    b += nloc * (sizeof(float) * (3 + (g->n_sls ? 1 : 0) + (aniso ? 3 : 0)) + E);
    b += 1 << 20;                                                   // tables, counters
    return b;
}

}  // namespace

extern "C" {

int sesnt_create(const sesnt_grid_t *grid, sesnt_t **out) {
    Range r("sesnt_create");
    if (!out) {
        g_create_error = "out is NULL";
        return SESNT_EINVAL;
    }
    *out = nullptr;
    std::string why;
    int rc = check_grid(grid, why);
    if (rc) {
        g_create_error = why;
        return rc;
    }
    std::unique_ptr<sesnt_handle> h(new sesnt_handle());
    h->g = *grid;
    h->N = grid->lpd;
    h->P = h->N + 1;
    h->NP = h->P * h->P * h->P;
    h->nel = grid->nx * grid->ny * grid->nz;
    h->nloc = (long long)h->nel * h->NP;
    h->NXU = grid->nx * h->N + 1;
    h->NYU = grid->ny * h->N + 1;
    h->NZU = grid->nz * h->N + 1;
    h->nuni = (long long)h->NXU * h->NYU * h->NZU;
    h->S = grid->batch;
    h->dbl = grid->precision == 8;
    h->esize = h->dbl ? 8 : 4;
    h->sls = grid->n_sls > 0;
    h->kahan = (grid->flags & SESNT_FLAG_KAHAN) != 0;
    h->use_graph = (grid->flags & SESNT_FLAG_NO_GRAPH) == 0;
    h->launches_per_step = 4;
    cudaGetDevice(&h->device);
    if (cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess || h->sms <= 0) {
        cudaGetLastError();
        h->sms = 152;
    }
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaGetLastError();
        g_create_error = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
        return SESNT_ECUDA;
    }
    cudaEventCreate(&h->ev0);
    cudaEventCreate(&h->ev1);
    e = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking);
    for (cudaEvent_t &ev : h->mark_ev)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    h->clear_marks();
    for (cudaEvent_t *ev : {&h->ev_fork, &h->ev_src, &h->ev_node, &h->ev_join})
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaGetLastError();
        g_create_error = std::string("creating the side stream: ") + cudaGetErrorString(e);
        return SESNT_ECUDA;
    }
    h->pool = library_pool(h->device);
    const size_t E = h->esize, P = h->P, nloc = (size_t)h->nloc, nuni = (size_t)h->nuni, S = h->S;
    struct A { void **p; size_t n; const char *w; } allocs[] = {
        {&h->tabD, 4 * P * P * E, "tables"}, {&h->w, P * E, "weights"},
        {&h->sin_t, grid->nx * P * E, "sin"}, {&h->cot_t, grid->nx * P * E, "cot"},
        {&h->r, grid->nz * P * E, "r"}, {&h->px, grid->nx * P * E, "px"},
        {&h->inv_r, grid->nz * P * E, "1/r"}, {&h->inv_sin, grid->nx * P * E, "1/sin"},
        {&h->py, grid->ny * P * E, "py"}, {&h->pz, grid->nz * P * E, "pz"},
        {(void **)&h->dsin, grid->nx * P * 8, "dsin"}, {(void **)&h->dr, grid->nz * P * 8, "dr"},
        {(void **)&h->dw, P * 8, "dw"},
        {&h->lam, nloc * E, "lambda"}, {&h->mu, nloc * E, "mu"},
        {&h->sig, h->state_unit() * (size_t)h->nel * E * S, "stress and memory variables"},
        {&h->v, 3 * nuni * E * S, "velocity"}, {&h->F, 3 * nuni * E * S, "force"},
        {&h->invM, nuni * E, "inverse mass"}, {(void **)&h->d_it, sizeof(int), "step counter"},
        {(void **)&h->d_err, sizeof(int), "error word"}};
    for (auto &a : allocs)
        if ((rc = h->alloc(a.p, a.n, a.w))) {
            g_create_error = h->err;
            return rc;
        }
    if (h->sls) {
        // the memory variables follow the stress inside each unit (StateLayout)
        h->mem = (char *)h->sig + (size_t)6 * h->state_cs() * E;
        if ((rc = h->alloc(&h->tau, nloc * E, "tau"))) {
            g_create_error = h->err;
            return rc;
        }
    }
    if ((grid->flags & SESNT_FLAG_FORCE64) && !h->dbl &&
        (rc = h->alloc((void **)&h->F64, 3 * nuni * 8 * S, "FP64 force"))) {
        g_create_error = h->err;
        return rc;
    }
    if ((grid->flags & SESNT_FLAG_KAHAN_STRESS) &&
        (rc = h->alloc(&h->sigc, 6 * (size_t)h->state_cs() * h->nel * E * S, "stress compensation"))) {
        g_create_error = h->err;
        return rc;
    }
    if (h->kahan && (rc = h->alloc(&h->vc, 3 * nuni * E * S, "compensation"))) {
        g_create_error = h->err;
        return rc;
    }
    if ((grid->flags & SESNT_FLAG_STRAIN) && (rc = h->alloc(&h->du, 9 * nloc * E * S, "displacement gradient"))) {
        g_create_error = h->err;
        return rc;
    }
    if ((grid->flags & SESNT_FLAG_ROTATION) && (rc = h->alloc(&h->rot_full, 6 * nloc * E * S, "rotation strain"))) {
        g_create_error = h->err;
        return rc;
    }
    if ((h->dbl ? lpd_ops<double>(h->N)->prepare() : lpd_ops<float>(h->N)->prepare()) != 0) {
        g_create_error = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(cudaGetLastError());
        return SESNT_ECUDA;
    }
    rc = h->dbl ? setup_tables<double>(h.get()) : setup_tables<float>(h.get());
    if (rc) {
        g_create_error = h->err;
        return rc;
    }
    if ((rc = zero_state(h.get()))) {
        g_create_error = h->err;
        return rc;
    }
    if (cudaMemset(h->d_err, 0, sizeof(int)) != cudaSuccess) {
        g_create_error = "zeroing the error word failed";
        return SESNT_ECUDA;
    }
    *out = h.release();
    return SESNT_OK;
}

int sesnt_destroy(sesnt_t *h) {
    delete h;
    return SESNT_OK;
}

const char *sesnt_last_error(const sesnt_t *h) {
    if (!h) return g_create_error.c_str();
    return h->err.c_str();
}

int sesnt_set_model(sesnt_t *h, const float *rhoinv, const float *lambda, const float *mu, const float *a,
                    const float *b, const float *c, const float *q) {
    if (!h) return SESNT_EINVAL;
    Range r("sesnt_set_model");
    if (!rhoinv || !lambda || !mu) return h->fail(SESNT_EINVAL, "rhoinv, lambda and mu are required");
    return h->dbl ? set_model_impl<double>(h, rhoinv, lambda, mu, a, b, c, q)
                  : set_model_impl<float>(h, rhoinv, lambda, mu, a, b, c, q);
}

int sesnt_locate_point(const sesnt_grid_t *grid, float lat, float lon, float depth, int elem[3], float *vanderm) {
    if (!grid || !elem || !vanderm) {
        g_create_error = "grid, elem and vanderm are required";
        return SESNT_EINVAL;
    }
    std::string why;
    if (grid->lpd < kMinLpd || grid->lpd > kMaxLpd || grid->nx < 1 || grid->ny < 1 || grid->nz < 1) {
        g_create_error = "invalid grid";
        return SESNT_EINVAL;
    }
    int rc = locate_point(grid->nx, grid->ny, grid->nz, grid->lpd, grid->lat_min, grid->lat_max, grid->lon_min,
                          grid->lon_max, grid->rad_min, grid->rad_max, lat, lon, depth, elem, vanderm, why);
    if (rc) {
        char b[256];
        snprintf(b, sizeof b, "%s (lat=%g lon=%g depth=%g)", why.c_str(), (double)lat, (double)lon, (double)depth);
        g_create_error = b;
        return rc == -1 ? SESNT_EINVAL : SESNT_ENOTFOUND;
    }
    return SESNT_OK;
}

int sesnt_source_signature(int wavelet, float onset, float width, float dt, int nt, float *out) {
    if (!out || nt < 1) return SESNT_EINVAL;
    return source_signature(wavelet, onset, width, dt, nt, out) ? SESNT_EINVAL : SESNT_OK;
}

int sesnt_add_source(sesnt_t *h, int sim, int ex, int ey, int ez, const float *vanderm, int kind, const float *comp,
                     const float *stf, int nt) {
    if (!h) return SESNT_EINVAL;
    if (!vanderm || !comp || !stf) return h->fail(SESNT_EINVAL, "vanderm, comp and stf are required");
    if (sim < 0 || sim >= h->S) return h->fail(SESNT_ERANGE, "simulation %d outside 0..%d", sim, h->S - 1);
    if (ex < 0 || ex >= h->g.nx || ey < 0 || ey >= h->g.ny || ez < 0 || ez >= h->g.nz)
        return h->fail(SESNT_ERANGE, "element (%d,%d,%d) outside the grid", ex, ey, ez);
    if (nt != h->g.nt) return h->fail(SESNT_EINVAL, "stf has %d samples, nt=%d", nt, h->g.nt);
    if (kind != SESNT_SOURCE_MT && kind != SESNT_SOURCE_SF) return h->fail(SESNT_EINVAL, "unknown source kind %d", kind);
    HostSource s;
    s.sim = sim;
    s.elem = ex + h->g.nx * (ey + h->g.ny * ez);
    s.vm.assign(vanderm, vanderm + h->NP);
    const int nc = kind == SESNT_SOURCE_MT ? 6 : 3, off = kind == SESNT_SOURCE_MT ? 0 : 6;
    for (int c = 0; c < 9; ++c) s.present[c] = false;
    for (int c = 0; c < nc; ++c) {
        std::vector<float> d(nt);
        bool nonzero = false;
        for (int t = 0; t < nt; ++t) {
            d[t] = stf[t] * comp[c];  // channel data in REAL32, src/config/source.f90:307-312
            nonzero = nonzero || d[t] != 0.0f;
        }
        // moment-tensor channels that are zero throughout are dropped
        // (src/config/source.f90:318-321); force channels are all kept.
        if (kind == SESNT_SOURCE_MT && !nonzero) continue;
        s.present[off + c] = true;
        s.data[off + c] = std::move(d);
    }
    h->sources.push_back(std::move(s));
    h->src_dirty = true;
    return SESNT_OK;
}

int sesnt_add_receiver(sesnt_t *h, int ex, int ey, int ez, const float *vanderm, unsigned channel_mask) {
    if (!h) return SESNT_EINVAL;
    if (!vanderm) return h->fail(SESNT_EINVAL, "vanderm is required");
    if (channel_mask & ~0xFFFFu) return h->fail(SESNT_EINVAL, "unknown channel bits 0x%x", channel_mask & ~0xFFFFu);
    if (ex < 0 || ex >= h->g.nx || ey < 0 || ey >= h->g.ny || ez < 0 || ez >= h->g.nz)
        return h->fail(SESNT_ERANGE, "element (%d,%d,%d) outside the grid", ex, ey, ez);
    h->rec_elem.push_back(ex + h->g.nx * (ey + h->g.ny * ez));
    h->rec_vm.insert(h->rec_vm.end(), vanderm, vanderm + h->NP);
    h->rec_mask.push_back(channel_mask);
    h->rec_dirty = true;
    return (int)h->rec_elem.size() - 1;
}

int sesnt_step(sesnt_t *h, int it) {
    if (!h) return SESNT_EINVAL;
    Range r("sesnt_step");
    const bool g = h->use_graph;
    h->use_graph = false;
    int rc = run_any(h, it, 1);
    h->use_graph = g;
    return rc;
}

int sesnt_run(sesnt_t *h, int it0, int nsteps) {
    if (!h) return SESNT_EINVAL;
    Range r("sesnt_run");
    return run_any(h, it0, nsteps);
}

int sesnt_run_timed(sesnt_t *h, int it0, int nsteps, float *ms) {
    if (!h || !ms) return SESNT_EINVAL;
    Range r("sesnt_run_timed");
    // prepare (uploads, graphs) outside the timed region
    int rc = h->dbl ? prepare_run<double>(h) : prepare_run<float>(h);
    if (rc) return rc;
    if (h->use_graph) {
        rc = h->dbl ? prebuild_graphs<double>(h) : prebuild_graphs<float>(h);
        if (rc) return rc;
    }
    cudaEventRecord(h->ev0, h->stream);
    rc = run_any(h, it0, nsteps);
    cudaEventRecord(h->ev1, h->stream);
    cudaError_t e = cudaEventSynchronize(h->ev1);
    if (rc) return rc;
    if (e != cudaSuccess) return h->cuda_fail(e, "timed run");
    cudaEventElapsedTime(ms, h->ev0, h->ev1);
    return h->wait_status();
}

int sesnt_run_profiled(sesnt_t *h, int it0, int nsteps, float ms[4]) {
    if (!h || !ms) return SESNT_EINVAL;
    Range r("sesnt_run_profiled");
    for (int q = 0; q < 4; ++q) ms[q] = 0.0f;
    if (it0 < 1 || it0 + nsteps - 1 > h->g.nt)
        return h->fail(SESNT_ERANGE, "steps %d..%d outside 1..nt=%d", it0, it0 + nsteps - 1, h->g.nt);
    int rc = h->dbl ? prepare_run<double>(h) : prepare_run<float>(h);
    if (rc) return rc;
    cudaEvent_t ev[5];
    for (auto &e : ev) cudaEventCreate(&e);
    k_set_it<<<1, 1, 0, h->stream>>>(h->d_it, it0);
    cudaError_t err = cudaSuccess;
    for (int n = 0; n < nsteps && !rc; ++n) {
        auto launch = [&](auto tag) -> int {
            using T = decltype(tag);
            const LpdOps<T> *o = ops<T>(h);
            StepArgs<T> a = h->args<T>();
            a.step_off = n;
            cudaEventRecord(ev[0], h->stream);
            if (h->nrot > 0 && o->rot_strain(a, h->d_rot_elems, h->nrot, (T *)h->d_rot_rec, h->stream)) return -1;
            if ((h->g.flags & SESNT_FLAG_ROTATION) && o->rot_strain(a, nullptr, h->nel, (T *)h->rot_full, h->stream))
                return -1;
            if (o->element(a, h->sls, h->aniso, h->stream)) return -1;
            cudaEventRecord(ev[1], h->stream);
            if (o->sources(a, h->stream)) return -1;
            cudaEventRecord(ev[2], h->stream);
            if (o->node(a, h->kahan, h->stream)) return -1;
            cudaEventRecord(ev[3], h->stream);
            if (o->receivers(a, h->stream)) return -1;
            cudaEventRecord(ev[4], h->stream);
            return 0;
        };
        if (h->dbl ? launch(double(0)) : launch(float(0))) {
            rc = h->fail(SESNT_ECUDA, "kernel launch failed: %s", cudaGetErrorString(cudaGetLastError()));
            break;
        }
        err = cudaEventSynchronize(ev[4]);
        if (err != cudaSuccess) break;
        for (int q = 0; q < 4; ++q) {
            float t = 0.0f;
            cudaEventElapsedTime(&t, ev[q], ev[q + 1]);
            ms[q] += t;
        }
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if (rc) return rc;
    return err == cudaSuccess ? h->wait_status() : h->cuda_fail(err, "profiled run");
}

// The host mirror of the seismograms (see sesnt_handle::h_seis): made from
// the device array once all queued steps are done; the captured steps are
// dropped so that the next ones write to it too.
int make_seis_mirror(sesnt_t *h) {
    const size_t n = (size_t)h->S * h->rec_elem.size() * 3 * h->g.nt, E = h->esize;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "synchronize");
    void *hm = nullptr, *hd = nullptr;
    std::vector<char> dev(n * E);
    if (cudaHostAlloc(&hm, n * sizeof(float), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer(&hd, hm, 0) != cudaSuccess ||
        cudaMemcpy(dev.data(), h->d_seis, n * E, cudaMemcpyDeviceToHost) != cudaSuccess) {
        if (hm) cudaFreeHost(hm);
        cudaGetLastError();
        h->seis_mirror_failed = true;  // sesnt_get_samples copies from the device
        return SESNT_OK;
    }
    float *f = (float *)hm;
    for (size_t x = 0; x < n; ++x) {
        if (E == 8) {
            double v;
            std::memcpy(&v, dev.data() + x * 8, 8);
            f[x] = (float)v;
        } else {
            std::memcpy(&f[x], dev.data() + x * 4, 4);
        }
    }
    h->h_seis = f;
    h->h_seis_dev = (float *)hd;
    h->h_seis_n = n;
    h->drop_graph();
    return SESNT_OK;
}

int sesnt_get_samples(sesnt_t *h, int it, float *out) {
    if (!h || !out) return SESNT_EINVAL;
    Range r("sesnt_get_samples");
    if (it < 1 || it > h->g.nt) return h->fail(SESNT_ERANGE, "step %d outside 1..%d", it, h->g.nt);
    const size_t nrec = h->rec_elem.size();
    if (nrec == 0) return SESNT_OK;
    if (h->rec_dirty) return h->fail(SESNT_ESTATE, "receivers added after the last step");
    const size_t E = h->esize, nt = h->g.nt;
    int rc;
    if (!h->h_seis && !h->seis_mirror_failed && h->d_seis && (rc = make_seis_mirror(h))) return rc;
    // wait for step it only (the earliest progress mark at or after it), or
    // for everything queued when no mark covers it
    int best = -1;
    for (int q = 0; q < sesnt_handle::kMarks; ++q)
        if (h->mark_it[q] >= it && (best < 0 || h->mark_it[q] < h->mark_it[best])) best = q;
    if (best >= 0 && h->h_seis) {
        // the mark's event follows the receiver kernel of step it: its
        // mapped-memory writes are visible once the event has completed
        cudaError_t e = cudaEventSynchronize(h->mark_ev[best]);
        if (e != cudaSuccess) return h->cuda_fail(e, "reading samples");
        for (size_t x = 0; x < (size_t)h->S * nrec * 3; ++x) {
            const size_t r = (x / 3) % nrec;
            const bool on = (h->rec_mask[r] >> (x % 3)) & 1u;
            out[x] = on ? h->h_seis[x * nt + (it - 1)] : 0.0f;
        }
        return SESNT_OK;
    }
    std::vector<double> tmp(h->S * nrec * 3);
    cudaStream_t cs = best >= 0 ? h->copy_stream : h->stream;
    cudaError_t e = best >= 0 ? cudaEventSynchronize(h->mark_ev[best]) : cudaSuccess;
    // one strided 2-D copy: rows [s][r][c] of the seismogram array, column it-1
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(tmp.data(), E, (const char *)h->d_seis + (size_t)(it - 1) * E, nt * E, E,
                              (size_t)h->S * nrec * 3, cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess) return h->cuda_fail(e, "reading samples");
    for (size_t x = 0; x < tmp.size(); ++x) {
        const size_t r = (x / 3) % nrec;
        const bool on = (h->rec_mask[r] >> (x % 3)) & 1u;
        float v;
        if (E == 8) v = (float)tmp[x];
        else std::memcpy(&v, (const char *)tmp.data() + x * 4, 4);
        out[x] = on ? v : 0.0f;
    }
    return SESNT_OK;
}

int sesnt_synchronize(sesnt_t *h) {
    if (!h) return SESNT_EINVAL;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "synchronize");
    return h->wait_status();
}

int sesnt_reset(sesnt_t *h) {
    if (!h) return SESNT_EINVAL;
    int rc = zero_state(h);
    if (rc) return rc;
    cudaError_t e = cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "clearing the error word");
    return sesnt_synchronize(h);
}

int sesnt_set_wait_limit(sesnt_t *h, int polls, int drop_completion) {
    if (!h) return SESNT_EINVAL;
    if (polls < 1) return h->fail(SESNT_EINVAL, "polls must be >= 1");
    h->drop_graph();  // the limit is a launch argument captured in the graph
    h->wait_polls = polls;
    h->drop_completion = drop_completion ? 1 : 0;
    return SESNT_OK;
}

int sesnt_get_seismograms(sesnt_t *h, float *out) {
    if (!h || !out) return SESNT_EINVAL;
    Range r("sesnt_get_seismograms");
    return h->dbl ? get_seis_impl<double>(h, out) : get_seis_impl<float>(h, out);
}

int sesnt_get_field(sesnt_t *h, int sim, int which, void *out, int out_precision) {
    if (!h || !out) return SESNT_EINVAL;
    Range r("sesnt_get_field");
    if (sim < 0 || sim >= h->S) return h->fail(SESNT_ERANGE, "simulation %d outside 0..%d", sim, h->S - 1);
    if (out_precision != 4 && out_precision != 8) return h->fail(SESNT_EINVAL, "out_precision must be 4 or 8");
    if (!h->model_set && which != SESNT_FIELD_TAPER)
        return h->fail(SESNT_ESTATE, "sesnt_set_model must be called first");
    return h->dbl ? get_field_impl<double>(h, sim, which, out, out_precision)
                  : get_field_impl<float>(h, sim, which, out, out_precision);
}

int sesnt_v_ptp(sesnt_t *h, int sim, float out[2]) {
    if (!h || !out) return SESNT_EINVAL;
    if (sim < 0 || sim >= h->S) return h->fail(SESNT_ERANGE, "simulation %d outside 0..%d", sim, h->S - 1);
    return h->dbl ? v_ptp_impl<double>(h, sim, out) : v_ptp_impl<float>(h, sim, out);
}

int sesnt_kinetic_energy(sesnt_t *h, int sim, double *out) {
    Range r("sesnt_kinetic_energy");
    if (!h || !out) return SESNT_EINVAL;
    if (sim < 0 || sim >= h->S) return h->fail(SESNT_ERANGE, "simulation %d outside 0..%d", sim, h->S - 1);
    if (!h->model_set) return h->fail(SESNT_ESTATE, "sesnt_set_model must be called before sesnt_kinetic_energy");
    return h->dbl ? kinetic_impl<double>(h, sim, out) : kinetic_impl<float>(h, sim, out);
}

int sesnt_assemble_field(sesnt_t *h, float *field) {
    if (!h || !field) return SESNT_EINVAL;
    return h->dbl ? assemble_impl<double>(h, field) : assemble_impl<float>(h, field);
}

int sesnt_tune(sesnt_t *h, char *report, int report_len) {
    Range r("sesnt_tune");
    if (!h) return SESNT_EINVAL;
    if (!h->model_set) return h->fail(SESNT_ESTATE, "sesnt_set_model must be called before sesnt_tune");
    if (h->last_it != 0)
        return h->fail(SESNT_ESTATE, "sesnt_tune times the step on the zero wavefield: call it after sesnt_set_model "
                                     "or sesnt_reset, before stepping");
    if (h->g.flags & (SESNT_FLAG_TC_TF32X3 | SESNT_FLAG_TC_BF16X3))
        return h->fail(SESNT_EUNSUPPORTED, "the tensor-core contractions have no variants to tune");
    TuneChoice c{};
    double ms = 0;
    h->drop_graph();
    const int rc = h->dbl ? tune_impl<double>(h, &c, &ms) : tune_impl<float>(h, &c, &ms);
    if (rc) return rc;
    tune_cache_store(tune_key(h), c, ms);
    if (report && report_len > 0) std::snprintf(report, (size_t)report_len, "%s", h->tune_report.c_str());
    return SESNT_OK;
}

int sesnt_set_element_variant(sesnt_t *h, int variant, int arg, int piece) {
    if (!h) return SESNT_EINVAL;
    if (variant < kVarAuto || variant >= kVarCount) return h->fail(SESNT_EINVAL, "unknown element variant %d", variant);
    if (arg < 0 || arg > 15) return h->fail(SESNT_EINVAL, "variant argument %d outside 0..15", arg);
    if ((variant == kVarStage || variant == kVarStageReg) && arg > 7)
        return h->fail(SESNT_EINVAL, "staged-kernel argument %d outside 0..7", arg);
    if (piece < 0 || piece % 16 != 0) return h->fail(SESNT_EINVAL, "piece size %d is not a multiple of 16 bytes", piece);
    h->drop_graph();  // the graphs hold the launch arguments
    h->variant = variant;
    h->variant_arg = arg;
    h->piece = piece;
    return SESNT_OK;
}

int sesnt_element_kernel(const sesnt_t *h, char *name, int name_len, int choice[3]) {
    if (!h || !name || name_len <= 0) return SESNT_EINVAL;
    const char *n = h->dbl ? ops<double>(h)->element_name(h->args<double>(), h->sls, h->aniso)
                           : ops<float>(h)->element_name(h->args<float>(), h->sls, h->aniso);
    std::snprintf(name, (size_t)name_len, "%s", n);
    if (choice) {
        choice[0] = h->variant;
        choice[1] = h->variant_arg;
        choice[2] = h->piece;
    }
    return SESNT_OK;
}

int sesnt_info(const sesnt_t *h, long long out[6]) {
    if (!h || !out) return SESNT_EINVAL;
    out[0] = h->nel;
    out[1] = h->nloc;
    out[2] = h->nuni;
    out[3] = (long long)h->dev_bytes;
    out[4] = algorithmic_bytes(h->nloc, h->nuni, h->sls ? kNsls : 0, h->aniso, h->S, h->esize);
    bool rot_rec = false;
    for (unsigned m : h->rec_mask) rot_rec = rot_rec || (m & (SESNT_CH_ROT_VX | SESNT_CH_ROT_VY | SESNT_CH_ROT_VZ));
    out[5] = 2 + (h->nsrc_rec > 0 || !h->sources.empty() ? 1 : 0) + (h->rec_elem.empty() ? 0 : 1) + (rot_rec ? 1 : 0) +
             ((h->g.flags & SESNT_FLAG_ROTATION) ? 1 : 0);
    return SESNT_OK;
}

long long sesnt_footprint_bytes(const sesnt_grid_t *grid) {
    std::string why;
    if (check_grid(grid, why)) return -1;
    return (long long)footprint(grid, false);
}

void *sesnt_stream(const sesnt_t *h) { return h ? (void *)h->stream : nullptr; }

namespace {
// Checkpoint layout: a fixed header, then the state buffers in this order.
struct StateHeader {
    char magic[8];
    int nx, ny, nz, lpd, batch, precision, n_sls, nrec, nxtr, last_it;
    unsigned flags;
    int pad;
};

std::vector<std::pair<void *, size_t>> state_buffers(sesnt_t *h) {
    const size_t E = h->esize, S = h->S, nel = h->nel, nuni = h->nuni;
    // stress with the memory variables (StateLayout)
    std::vector<std::pair<void *, size_t>> b = {{h->v, 3 * nuni * E * S}, {h->sig, h->state_unit() * nel * E * S}};
    if (h->vc) b.push_back({h->vc, 3 * nuni * E * S});
    if (h->sigc) b.push_back({h->sigc, 6 * (size_t)h->state_cs() * nel * E * S});  // stress compensation
    if (h->du) b.push_back({h->du, 9 * (size_t)h->nloc * E * S});
    if (h->d_seis) b.push_back({h->d_seis, S * h->rec_elem.size() * 3 * (size_t)h->g.nt * E});
    if (h->d_xseis) b.push_back({h->d_xseis, S * (size_t)h->nxtr * h->g.nt * E});
    return b;
}

int prepare_receivers(sesnt_t *h) {
    if (!h->rec_dirty) return SESNT_OK;
    int rc = h->dbl ? upload_receivers<double>(h) : upload_receivers<float>(h);
    return rc ? rc : upload_receiver_sources(h);
}

StateHeader state_header(const sesnt_t *h) {
    StateHeader hd{};
    std::memcpy(hd.magic, "SESNTST1", 8);
    hd.nx = h->g.nx; hd.ny = h->g.ny; hd.nz = h->g.nz; hd.lpd = h->g.lpd; hd.batch = h->S;
    hd.precision = h->g.precision; hd.n_sls = h->g.n_sls; hd.nrec = (int)h->rec_elem.size(); hd.nxtr = h->nxtr;
    hd.flags = h->g.flags & (SESNT_FLAG_KAHAN | SESNT_FLAG_KAHAN_STRESS | SESNT_FLAG_STRAIN);
    hd.last_it = h->last_it;
    return hd;
}
}  // namespace

long long sesnt_state_bytes(sesnt_t *h) {
    if (!h) return SESNT_EINVAL;
    int rc = prepare_receivers(h);
    if (rc) return rc;
    long long n = sizeof(StateHeader);
    for (auto &b : state_buffers(h)) n += (long long)b.second;
    return n;
}

int sesnt_save_state(sesnt_t *h, void *buf) {
    if (!h || !buf) return SESNT_EINVAL;
    int rc = prepare_receivers(h);
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "synchronize");
    if ((rc = h->wait_status())) return rc;
    const StateHeader hd = state_header(h);
    char *o = (char *)buf;
    std::memcpy(o, &hd, sizeof hd);
    o += sizeof hd;
    for (auto &b : state_buffers(h)) {
        if ((e = cudaMemcpy(o, b.first, b.second, cudaMemcpyDeviceToHost)) != cudaSuccess)
            return h->cuda_fail(e, "saving state");
        o += b.second;
    }
    return SESNT_OK;
}

int sesnt_load_state(sesnt_t *h, const void *buf) {
    if (!h || !buf) return SESNT_EINVAL;
    int rc = prepare_receivers(h);
    if (rc) return rc;
    StateHeader hd, want = state_header(h);
    std::memcpy(&hd, buf, sizeof hd);
    want.last_it = hd.last_it;
    if (std::memcmp(&hd, &want, sizeof hd) != 0)
        return h->fail(SESNT_EINVAL, "state was saved from a handle with another grid, precision, flags or receivers");
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "synchronize");
    const char *in = (const char *)buf + sizeof hd;
    for (auto &b : state_buffers(h)) {
        if ((e = cudaMemcpy(b.first, in, b.second, cudaMemcpyHostToDevice)) != cudaSuccess)
            return h->cuda_fail(e, "loading state");
        if (b.first == h->d_seis && h->h_seis)  // the host mirror of the restored samples
            for (size_t x = 0; x < h->h_seis_n; ++x) {
                if (h->esize == 8) {
                    double v;
                    std::memcpy(&v, in + x * 8, 8);
                    h->h_seis[x] = (float)v;
                } else {
                    std::memcpy(&h->h_seis[x], in + x * 4, 4);
                }
            }
        in += b.second;
    }
    h->last_it = hd.last_it;
    h->rot_full_it = -1;
    h->clear_marks();
    return SESNT_OK;
}

int sesnt_get_trace(sesnt_t *h, int sim, int receiver, unsigned channel, float *out) {
    if (!h || !out) return SESNT_EINVAL;
    if (sim < 0 || sim >= h->S) return h->fail(SESNT_ERANGE, "simulation %d outside 0..%d", sim, h->S - 1);
    if (receiver < 0 || receiver >= (int)h->rec_elem.size())
        return h->fail(SESNT_ERANGE, "receiver %d outside 0..%d", receiver, (int)h->rec_elem.size() - 1);
    if (channel == 0 || (channel & (channel - 1)) || channel > SESNT_CH_FZ)
        return h->fail(SESNT_EINVAL, "channel must be one SESNT_CH_* bit");
    if (!(h->rec_mask[receiver] & channel))
        return h->fail(SESNT_EINVAL, "channel 0x%x was not requested for receiver %d", channel, receiver);
    int rc;
    if (h->rec_dirty) {
        if ((rc = h->dbl ? upload_receivers<double>(h) : upload_receivers<float>(h))) return rc;
        if ((rc = upload_receiver_sources(h))) return rc;
    }
    const size_t nt = h->g.nt, nrec = h->rec_elem.size(), E = h->esize;
    const void *src;
    double sign = 1.0;
    if (channel <= SESNT_CH_N) {
        const int c = channel == SESNT_CH_N ? 0 : __builtin_ctz(channel);
        if (channel == SESNT_CH_N) sign = -1.0;  // record_n: SUM(-1.0*vanderm*vx)
        src = (const char *)h->d_seis + (((size_t)sim * nrec + receiver) * 3 + c) * nt * E;
    } else {
        const unsigned xm = h->rec_mask[receiver] & kDeviceChannels;
        const int slot = h->rec_xslot[receiver] + __builtin_popcount(xm & (channel - 1));
        src = (const char *)h->d_xseis + ((size_t)sim * h->nxtr + slot) * nt * E;
    }
    std::vector<double> tmp(nt);
    std::vector<float> tf(nt);
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess) e = cudaMemcpy(h->dbl ? (void *)tmp.data() : (void *)tf.data(), src, nt * E, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return h->cuda_fail(e, "reading trace");
    if ((rc = h->wait_status())) return rc;
    for (size_t t = 0; t < nt; ++t) out[t] = h->dbl ? (float)(sign * tmp[t]) : (float)(sign * tf[t]);
    return SESNT_OK;
}

namespace {
struct FieldName { int id; const char *name; };
const FieldName kFieldNames[] = {
    {SESNT_FIELD_VX, "vx"}, {SESNT_FIELD_VY, "vy"}, {SESNT_FIELD_VZ, "vz"},
    {SESNT_FIELD_SXX, "sxx"}, {SESNT_FIELD_SXY, "sxy"}, {SESNT_FIELD_SXZ, "sxz"},
    {SESNT_FIELD_SYY, "syy"}, {SESNT_FIELD_SYZ, "syz"}, {SESNT_FIELD_SZZ, "szz"},
    {SESNT_FIELD_TAPER, "taper"}, {SESNT_FIELD_MASS, "mm"},
    {SESNT_FIELD_PRESSURE, "pressure"},
    {SESNT_FIELD_EXX, "exx"}, {SESNT_FIELD_EXY, "exy"}, {SESNT_FIELD_EXZ, "exz"},
    {SESNT_FIELD_EYY, "eyy"}, {SESNT_FIELD_EYZ, "eyz"}, {SESNT_FIELD_EZZ, "ezz"},
    {SESNT_FIELD_ROT_VX, "rot_vx"}, {SESNT_FIELD_ROT_VY, "rot_vy"}, {SESNT_FIELD_ROT_VZ, "rot_vz"},
    {SESNT_FIELD_LAMBDA, "lambda"}, {SESNT_FIELD_MU, "mu"},
    {SESNT_FIELD_A, "a"}, {SESNT_FIELD_B, "b"}, {SESNT_FIELD_C, "c"}};
}  // namespace

const char *sesnt_field_name(int which) {
    for (const auto &f : kFieldNames)
        if (f.id == which) return f.name;
    return nullptr;
}

int sesnt_field_id(const char *name) {
    if (!name) return -1;
    std::string n(name);
    while (!n.empty() && (n.back() == ' ' || n.back() == '\t')) n.pop_back();
    size_t b = 0;
    while (b < n.size() && (n[b] == ' ' || n[b] == '\t')) ++b;
    n = n.substr(b);
    for (auto &ch : n) ch = (char)std::tolower((unsigned char)ch);
    for (const auto &f : kFieldNames)
        if (n == f.name) return f.id;
    return -1;
}

int sesnt_add_snapshot(sesnt_t *h, int sim, int which, int ts_start, int ts_increment, int ts_end,
                       const char *prefix, const char *attribute, int override) {
    if (!h) return SESNT_EINVAL;
    if (sim < 0 || sim >= h->S) return h->fail(SESNT_ERANGE, "simulation %d outside 0..%d", sim, h->S - 1);
    const char *name = sesnt_field_name(which);
    if (!name || which == SESNT_FIELD_MASS) return h->fail(SESNT_EINVAL, "field %d cannot be snapshotted", which);
    if (which >= SESNT_FIELD_EXX && which <= SESNT_FIELD_EZZ && !h->du)
        return h->fail(SESNT_ESTATE, "strain snapshots need SESNT_FLAG_STRAIN at sesnt_create");
    if (ts_end <= 0) ts_end = h->g.nt;
    // range checks of volume_snapshot_cls' constructor (src/volume_snapshot.f90:71-113)
    if (ts_start < 1) return h->fail(SESNT_ERANGE, "timestep_start out of range");
    if (ts_increment < 1 || ts_increment > h->g.nt) return h->fail(SESNT_ERANGE, "timestep_increment out of range");
    if (ts_end < ts_start) return h->fail(SESNT_ERANGE, "timestep_end out of range");
    int rc;
    const size_t bytes = (size_t)h->nloc * h->esize;
    if (!h->writer) h->writer.reset(new SnapshotWriter());
    std::string err;
    if ((rc = h->writer->start(h->device, bytes, 3, err))) return h->fail(rc, "%s", err.c_str());
    if (!h->snap_stage && (rc = h->alloc(&h->snap_stage, bytes, "snapshot staging"))) return rc;
    if (is_rotation(which) && !h->rot_full &&
        (rc = h->alloc(&h->rot_full, 6 * bytes * h->S, "rotation strain")))
        return rc;
    sesnt_handle::Snapshot q;
    q.sim = sim;
    q.which = which;
    q.start = ts_start;
    q.inc = ts_increment;
    q.end = ts_end;
    q.prefix = (prefix && *prefix) ? prefix : "./";
    q.attribute = attribute ? attribute : name;
    q.override = override != 0;
    h->snaps.push_back(q);
    return (int)h->snaps.size() - 1;
}

int sesnt_snapshots_wait(sesnt_t *h) {
    if (!h) return SESNT_EINVAL;
    if (!h->writer) return SESNT_OK;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return h->cuda_fail(e, "synchronize");
    std::string err;
    const int rc = h->writer->wait(err);
    if (rc) return h->fail(rc, "%s", err.c_str());
    return SESNT_OK;
}

}  // extern "C"
