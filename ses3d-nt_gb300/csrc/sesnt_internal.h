// Internal declarations shared by the host set-up code, the kernels and the
// C ABI implementation.
//
// Device data layout (one handle, `batch` = S simulations sharing a model):
//   element-local arrays  x[e*NP + p]      e = ex + nx*(ey + ny*ez),
//                                          p = i + P*(j + P*k), P = lpd+1,
//                                          NP = P^3 (an element's points are
//                                          contiguous, so a thread block that
//                                          owns a few elements streams one
//                                          contiguous range per component)
//   per-simulation blocks sigma[s][6][N_loc], memory[s][6*n_sls][N_loc]
//   unique-point arrays   v[s][3][N_uni], force[s][3][N_uni], inv_mass[N_uni]
//                         u = gx + NXU*(gy + NYU*gz), gx = ex*lpd + i, ...
// The unique numbering is arithmetic (structured grid), so assembly needs no
// connectivity array: every element computes the unique index of its points.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

struct sesnt_handle;
struct sesnt_grid;

namespace sesnt {

// Handle accessors for entry points defined outside sesnt_api.cu.
const sesnt_grid *handle_grid(const sesnt_handle *h);
int handle_device(const sesnt_handle *h);  // the device current at sesnt_create
int handle_fail(sesnt_handle *h, int code, const char *fmt, ...);

constexpr int kMaxLpd = 7;
constexpr int kMinLpd = 2;
constexpr int kNsls = 3;  // relaxation mechanisms, src/geometric_paras.f90:41

// Relaxation times tau_p [s], src/geometric_paras.f90:42.
constexpr double kTauP[kNsls] = {1000.00, 70.00, 5.25};

// One source channel set resolved for one (simulation, element): for each of
// the 9 components (mxx mxy mxz myy myz mzz fx fy fz) the index of the
// Vandermonde row and of the data row to use, or -1.
struct SrcRec {
    int sim;
    int elem;
    int vm[9];
    int data[9];
};

// Element-kernel variants (StepArgs::variant). kVarAuto applies the launch
// rules of launch_element; the others are chosen by the tuner
// (sesnt_tune) or set by the caller (sesnt_set_element_variant) and fall
// back to the rules where the handle's configuration has no such kernel.
enum ElementVariant : int {
    kVarAuto = 0,
    kVarPoint = 1,       // k_element: one thread per element-local point
    kVarPair = 2,        // k_element_pair: two simulations per thread (even-batch elastic)
    kVarStage = 3,       // k_element_stage, state out by bulk store (SLS, degrees 4-7)
    kVarStageReg = 4,    // k_element_stage, state out from registers
    kVarPersistent = 5,  // k_element_tma: persistent, state by bulk copies
    kVarColumns = 6,     // k_element_cols: one thread per column (elastic)
    kVarColumnsStaged = 7,  // k_element_cols with the block's stress staged by bulk copy
    kVarColumnsPair = 8,    // k_element_cols2: two simulations per column thread (even-batch elastic)
    kVarCount
};

template <typename T>
struct StepArgs {
    // grid
    int nx, ny, nz, nel, S;
    int NXU, NYU, NZU;
    long long nuni, nloc;
    T dt, c1, c2, c3, jac, alpha, inv_alpha;
    T tau_p[kNsls];
    T mem_rate[kNsls];   // dt/tau_p(k)
    T mem_drive[kNsls];  // dt/(n_sls*tau_p(k))
    // small tables (device): tabD = [Dx | Dy | Dz | Dt], each P*P
    const T *tabD, *w, *sin_t, *cot_t, *r, *px, *py, *pz;
    // Dz and Dt again in the launch parameters (constant bank), for kernels
    // that index them with compile-time indices only (the column kernels)
    T tabz[2][64];
    const T *inv_r, *inv_sin;  // 1/r [nz*P], 1/sin(theta) [nx*P]
    // model (element-local)
    const T *lam, *mu, *A, *B, *C, *tau;
    // state
    T *sig, *mem, *v, *vc, *F;
    double *F64;  // the force in FP64 (SESNT_FLAG_FORCE64 on FP32 handles), or null
    T *sigc;      // stress compensation terms [units][6][CS] (SESNT_FLAG_KAHAN_STRESS), or null
    const T *invM;
    // sources
    int nsrc, nt;
    int n_src_vm, n_src_data;  // rows of src_vm and src_data (bounds-check builds)
    const SrcRec *src;
    const T *src_vm;    // [n_vm][NP]
    const T *src_data;  // [n_data][nt]
    // receivers
    int nrec;
    const int *rec_elem;
    const T *rec_vm;    // [nrec][NP]
    T *seis;            // [S][nrec][3][nt]
    int st_cs;          // state layout (StateLayout): component stride
    long long st_unit;  // and values per (element, simulation) unit
    float *seis_host;   // the same samples in float32, mapped pinned host memory (or null)
    // step counter: it = *d_it + step_off
    const int *d_it;
    int step_off;
    int persistent;  // element kernel: persistent prefetching variant (1) or one block per group (0)
    int pair;        // batched elastic steps: two simulations per thread (k_element_pair)
    int stage;       // SLS steps: state staged in shared memory by bulk copy (k_element_stage)
    int contraction; // element kernel contractions: 0 CUDA cores, 1 tensor cores TF32x3, 2 tensor cores BF16x3
    int variant;     // ElementVariant
    int variant_arg; // k_element_cols: bits 0-1 index of the resident-block count (kColsMinb),
                     // bits 2-3 L2 prefetch distance (0: none, 1: 1/4, 2: 1/2, 3: 1 wave);
                     // k_element_stage: bit 0 = one lane per warp polls the stage's mbarrier,
                     // bits 1-2 = L2 prefetch distance in resident waves (0: none, 1: 1/4,
                     // 2: 1/2, 3: 1 wave of 8 blocks per SM)
    int piece;       // bulk copies of a state unit in pieces of this many bytes (multiple of 16; 0: whole)
    int prefetch;    // k_element_stage: L2 prefetch of the unit this many units ahead (0: none)
    T two_over_d[3]; // 2/dx_elm, 2/dy_elm, 2/dz_elm
    int *err;        // device error word (a bounded wait ran out)
    int wait_polls;  // bound of every device-side completion wait (mbarrier polls)
    int drop_completion;  // failure-detection test hook: the tensor-core and bulk-copy kernels signal no completion
    // displacement gradient [S][9][nloc] (order kDu*), or null when not kept
    T *du;
    // receiver channels beyond vx, vy, vz (SESNT_CH_ROT_* , _M**, _F*):
    // per receiver the device-computed channel bits and its first trace slot;
    // the rotation-strain slot of its element (or -1); per (sim, receiver)
    // the source record of the receiver's element (or -1)
    const unsigned *rec_xmask;
    const int *rec_xslot, *rec_rot, *rec_src;
    T *xseis;            // [S][nxtr][nt]
    const T *rot_rec;    // [S][6][nrot][NP] rotation strain of the receiver elements
    int nxtr, nrot;
};

// Points per element in the element-blocked stress of elastic handles
// [e][s][comp][NPS]: NP padded to a multiple of 4 so that every chunk starts
// on a 16-byte boundary (coalesced warps, bulk-copy alignment).
#ifdef __CUDACC__
#define SESNT_HD __host__ __device__
#else
#define SESNT_HD
#endif
SESNT_HD constexpr int state_stride(int np) { return (np + 3) & ~3; }

// The state of one (element, simulation) unit, element-blocked: the stress
// [6][CS], then for visco-elastic handles the memory variables [6*NSLS][CS]
// (the handle's mem pointer is sig + 6*CS), one contiguous unit that one
// bulk copy moves. CS is NP padded to a multiple of 4, so that every
// component chunk starts on a 16-byte boundary for per-thread access, except
// for visco-elastic degree 4 (NP = 125). There the default kernel moves the
// state only as whole units by bulk copy, 24*125*4 bytes is a multiple of 16,
// and padding would cost 2.4% of the state bytes (measured 1.1% of the step).
// Degree 6, whose kernel stores per thread, measured 4.7% slower unpadded.
SESNT_HD constexpr int state_cs(int np, bool sls) { return sls && np == 125 ? np : state_stride(np); }
SESNT_HD constexpr size_t state_unit(int np, int nsls) {
    return (size_t)(6 + 6 * nsls) * state_cs(np, nsls > 0);
}
template <int NP, int NSLS>
struct StateLayout {
    static constexpr int CS = state_cs(NP, NSLS > 0);  // component stride
    static constexpr size_t UNIT = state_unit(NP, NSLS);  // values per unit
};
// Every unit is a legal bulk copy (the bulk-copy kernels move whole units
// only): its size is a multiple of 16 bytes for degrees 2-7 in FP32 and FP64,
// so every unit of an allocation starts on a 16-byte boundary.
constexpr bool state_layout_aligned(int lpd) {
    const int np = (lpd + 1) * (lpd + 1) * (lpd + 1);
    for (int nsls : {0, 3})
        for (int e : {4, 8})
            if ((state_unit(np, nsls) * e) % 16 != 0) return false;
    return true;
}
static_assert(state_layout_aligned(2) && state_layout_aligned(3) && state_layout_aligned(4) &&
                  state_layout_aligned(5) && state_layout_aligned(6) && state_layout_aligned(7),
              "state units must be multiples of 16 bytes");

// Displacement-gradient components (src/evolution.f90:179-187).
enum { kDuXX = 0, kDuYY, kDuZZ, kDuXY, kDuYX, kDuXZ, kDuZX, kDuYZ, kDuZY };
// Rotation strain: the gradient components the reference's rot_v channels
// read after a step (src/config/channel_mod.f90:620-812), i.e. the completed
// gradient with exy, exz, eyz already symmetrised (src/evolution.f90:206-208).
enum { kRotEYZ = 0, kRotEZY, kRotEZX, kRotEXZ, kRotEXY, kRotEYX };

// Kernel launchers for one polynomial degree and one precision, filled in by
// the per-degree translation units.
template <typename T>
struct LpdOps {
    int (*element)(const StepArgs<T> &, bool sls, bool aniso, void *stream);
    int (*node)(const StepArgs<T> &, bool kahan, void *stream);
    int (*sources)(const StepArgs<T> &, void *stream);
    int (*receivers)(const StepArgs<T> &, void *stream);
    // FP64 inverse mass per unique point from element-local rhoinv and the
    // FP64 metric tables sin(theta)[nx*P], r[nz*P], GLL weights[P].
    int (*inv_mass)(const StepArgs<T> &, const T *rhoinv_loc, const double *dsin, const double *dr,
                    const double *dw, double jac, void *stream);
    // element-local copy of a unique-point field (for get_field), T -> T.
    int (*gather_local)(const StepArgs<T> &, const T *uni, T *loc, void *stream);
    // sum element-local copies into unique points, T (for assemble_field).
    int (*scatter_unique)(const StepArgs<T> &, const T *loc, T *uni, void *stream);
    // element-local taper (for get_field).
    int (*taper_local)(const StepArgs<T> &, T *loc, void *stream);
    // rotation strain of `count` elements (elems, or all elements when null)
    // from the current velocity: out[((s*6 + c)*count + idx)*NP + p].
    int (*rot_strain)(const StepArgs<T> &, const int *elems, int count, T *out, void *stream);
    // element-local derived field of simulation `sim`: SESNT_FIELD_PRESSURE,
    // _EXX.._EZZ (from du), _ROT_VX.._ROT_VZ (from the full-volume rotation
    // strain `rot` [S][6][nloc] and the current velocity).
    int (*derived)(const StepArgs<T> &, int which, int sim, const T *rot, T *loc, void *stream);
    // one-time kernel attributes (large dynamic shared memory)
    int (*prepare)();
    // name of the element kernel a step launches with these arguments
    const char *(*element_name)(const StepArgs<T> &, bool sls, bool aniso);
    int threads_element;
    size_t smem_element;
};

template <int N, typename T>
const LpdOps<T> *lpd_ops_n();  // defined in kern_lpd<N>.cu

template <typename T>
const LpdOps<T> *lpd_ops(int lpd);

// ---------------------------------------------------------------------------
// Host set-up (setup.cpp). Float32 routines reproduce the reference's FP32
// formula order; the templated ones are evaluated in the requested precision.
// ---------------------------------------------------------------------------
template <typename T>
std::vector<T> gll_points(int lpd);
template <typename T>
std::vector<T> gll_quadrature_weights(int lpd);
template <typename T>
std::vector<T> lagrange_derivative_matrix(int lpd);  // d[i*P+j] = l_i'(xi_j)

template <typename T>
struct Domain {
    T x_glb_min, x_glb_max, y_glb_min, y_glb_max, z_glb_min, z_glb_max;
    T dx_elm, dy_elm, dz_elm;
    T x_loc_min, x_loc_max, y_loc_min, y_loc_max, z_loc_min, z_loc_max;
};
template <typename T>
Domain<T> make_domain(int nx, int ny, int nz, float lat_min, float lat_max, float lon_min, float lon_max,
                      float rad_min, float rad_max);

template <typename T>
std::vector<T> element_coordinates(int elms, int lpd, T lo, T hi);  // [e*P+n]

// Damping profiles of the absorbing taper (before corner normalisation),
// one 1-D table per direction indexed [e*P+n].
template <typename T>
void taper_profiles(int nx, int ny, int nz, int lpd, int width, T alpha, const Domain<T> &d, std::vector<T> &px,
                    std::vector<T> &py, std::vector<T> &pz);

int locate_point(int nx, int ny, int nz, int lpd, float lat_min, float lat_max, float lon_min, float lon_max,
                 float rad_min, float rad_max, float lat, float lon, float depth, int elem[3], float *vanderm,
                 std::string &why);

int source_signature(int wavelet, float onset, float width, float dt, int nt, float *out);

// Algorithmic HBM bytes of one time step (the fixed formula of the roofline).
long long algorithmic_bytes(long long nloc, long long nuni, int n_sls, bool aniso, int S, int elem_bytes);

}  // namespace sesnt
