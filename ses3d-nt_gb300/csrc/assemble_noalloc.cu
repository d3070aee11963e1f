// sesnt_assemble_field_noalloc: assembly of shared GLL points without any
// device allocation, for callers that cannot call cudaMalloc at that point:
// a Fortran time loop that must not synchronise the whole device (as
// cudaMalloc/cudaFree may), or a host program that sized and reserved all
// device memory up front and has nothing left to allocate from.
//
// The unique-point accumulator lives in a file-scope device array of fixed
// size (kNoAllocMaxUnique floats, 16 MiB). Every GPU that loads this library
// holds that array until the process exits. All calls share it: the array
// keeps the previous call's sums, so each call clears the part it uses, and
// calls whose work overlaps on the GPU (different handles or streams at the
// same time) race on it. The sums are float32 for every handle precision.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/sesnt.h"
#include "sesnt_internal.h"

namespace {

constexpr long long kNoAllocMaxUnique = 4LL << 20;  // 4,194,304 unique points

static __device__ __align__(256) float g_noalloc_unique[kNoAllocMaxUnique];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
float *g_unique_ptr[kMaxDevices] = {};

// Device address of the accumulator on device `dev` (the current device),
// looked up once per device with that device current and cached.
int unique_scratch(int dev, float **out) {
    if (dev < 0 || dev >= kMaxDevices) return -1;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_unique_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_unique) != cudaSuccess || !p) return -1;
        g_unique_ptr[dev] = static_cast<float *>(p);
    }
    *out = g_unique_ptr[dev];
    return 0;
}

struct RawGrid {
    int nx, ny, nz, N, NP, NXU, NYU;
    long long nel, nloc, nuni;
};

__device__ __forceinline__ long long raw_to_unique(const RawGrid &g, long long a) {
    const long long e = a % g.nel;
    const int p = (int)(a / g.nel);
    const int P = g.N + 1;
    const int i = p % P, j = (p / P) % P, k = p / (P * P);
    const int ex = (int)(e % g.nx), ey = (int)((e / g.nx) % g.ny), ez = (int)(e / ((long long)g.nx * g.ny));
    return (long long)(ex * g.N + i) + (long long)g.NXU * ((long long)(ey * g.N + j) + (long long)g.NYU * (ez * g.N + k));
}

__global__ void k_zero(float *x, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = 0.0f;
}

// reference raw layout in -> unique sums
__global__ void k_scatter_raw(const RawGrid g, const float *__restrict__ in, float *uni) {
    const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (a < g.nloc) atomicAdd(uni + raw_to_unique(g, a), in[a]);
}

// unique sums -> every element-local copy, reference raw layout
__global__ void k_gather_raw(const RawGrid g, const float *__restrict__ uni, float *out) {
    const long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (a < g.nloc) out[a] = uni[raw_to_unique(g, a)];
}

}  // namespace

extern "C" int sesnt_assemble_field_noalloc(sesnt_t *h, const float *d_in, float *d_out) {
    if (!h || !d_in || !d_out) return SESNT_EINVAL;
    const sesnt_grid_t *gr = sesnt::handle_grid(h);
    RawGrid g;
    g.nx = gr->nx; g.ny = gr->ny; g.nz = gr->nz; g.N = gr->lpd;
    const int P = g.N + 1;
    g.NP = P * P * P;
    g.NXU = g.nx * g.N + 1;
    g.NYU = g.ny * g.N + 1;
    g.nel = (long long)g.nx * g.ny * g.nz;
    g.nloc = g.nel * g.NP;
    g.nuni = (long long)g.NXU * g.NYU * (long long)(g.nz * g.N + 1);
    if (g.nuni > kNoAllocMaxUnique)
        return sesnt::handle_fail(h, SESNT_ERANGE,
                                  "sesnt_assemble_field_noalloc: grid has %lld unique points, the fixed scratch "
                                  "holds at most %lld; use sesnt_assemble_field",
                                  g.nuni, kNoAllocMaxUnique);
    // the handle's stream and the array's address belong to the handle's device
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return sesnt::handle_fail(h, SESNT_ECUDA, "sesnt_assemble_field_noalloc: cudaGetDevice failed: %s",
                                  cudaGetErrorString(cudaGetLastError()));
    if (dev != sesnt::handle_device(h))
        return sesnt::handle_fail(h, SESNT_EINVAL,
                                  "sesnt_assemble_field_noalloc: the current device is %d but the handle was "
                                  "created on device %d; make the handle's device current first",
                                  dev, sesnt::handle_device(h));
    float *uni = nullptr;
    if (unique_scratch(dev, &uni))
        return sesnt::handle_fail(h, SESNT_ECUDA, "sesnt_assemble_field_noalloc: cudaGetSymbolAddress failed: %s",
                                  cudaGetErrorString(cudaGetLastError()));
    cudaStream_t st = (cudaStream_t)sesnt_stream(h);
    const unsigned bu = (unsigned)((g.nuni + 255) / 256), bl = (unsigned)((g.nloc + 255) / 256);
    k_zero<<<bu, 256, 0, st>>>(uni, g.nuni);  // the array keeps the previous call's sums
    k_scatter_raw<<<bl, 256, 0, st>>>(g, d_in, uni);
    k_gather_raw<<<bl, 256, 0, st>>>(g, uni, d_out);
    // launch errors of these three kernels, before the synchronisation can
    // report (and clear) an error left by unrelated earlier work
    cudaError_t e = cudaPeekAtLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return sesnt::handle_fail(h, SESNT_ECUDA, "sesnt_assemble_field_noalloc: %s", cudaGetErrorString(e));
    return SESNT_OK;
}
