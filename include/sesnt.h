/*
 * sesnt.h - C ABI of the GB300 spectral-element time step for Ses3d-NT.
 *
 * The reference drives one time step through argument-less module
 * procedures and module globals:
 *   - init_temp / ses3d_evolution        src/evolution.f90:48-84, 87-444
 *   - model + auxiliary precompute      src/model_paras.F90:206-416
 *   - geometry + taper precompute       src/geometric_paras.f90:108-325
 *   - source_cls%add(it)                src/config/source.f90:359-370
 *   - receiver_cls%record(it)           src/config/receiver.f90:136-142
 *   - point location / Vandermonde      src/config/point.f90:150-254
 * called from the forward loop at src/ses3d-nt.F90:240-270.
 * This header replaces them with explicit, handle-based entry points that a
 * Fortran driver binds through ISO_C_BINDING.
 *
 * Conventions
 *   - Every function returns SESNT_OK (0) or a negative SESNT_E* code; the
 *     library never aborts. sesnt_last_error() gives the message.
 *   - Model and field arrays use the reference raw layout: Fortran order,
 *     shape (nx, ny, nz, lpd+1, lpd+1, lpd+1), element x index fastest
 *     (src/mpi_parallel_io.F90:61-110). The library copies inputs; callers
 *     keep ownership of their buffers.
 *   - A handle owns its device memory and one CUDA stream. Handles are not
 *     thread-safe: use one handle per host thread.
 *   - Time steps are numbered 1..nt as in the reference loop.
 */
#ifndef SESNT_H
#define SESNT_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SESNT_OK 0
#define SESNT_EINVAL (-1)       /* invalid argument */
#define SESNT_ECUDA (-2)        /* CUDA runtime error */
#define SESNT_ENOMEM (-3)       /* device or host allocation failed */
#define SESNT_ESTATE (-4)       /* call out of order (e.g. step before model) */
#define SESNT_ERANGE (-5)       /* index or size out of range */
#define SESNT_ETIMEOUT (-6)     /* a bounded device wait ran out */
#define SESNT_ENOTFOUND (-7)    /* point outside the computational domain */
#define SESNT_EUNSUPPORTED (-8) /* configuration not built into this library */
#define SESNT_ENONFINITE (-9)   /* the wavefield contains NaN or Inf */

/* flags (sesnt_grid_t.flags) */
#define SESNT_FLAG_KAHAN 1u      /* compensated velocity update */
#define SESNT_FLAG_NO_GRAPH 2u   /* sesnt_run launches kernels directly, no CUDA graph */
#define SESNT_FLAG_TC_TF32X3 8u   /* derivative and divergence contractions on the tensor cores
                                     (tcgen05) in split TF32 (3 products), FP32 accumulation */
#define SESNT_FLAG_TC_BF16X3 16u  /* the same in split BF16 (3 products); FP32 wavefields only */
#define SESNT_FLAG_PERSISTENT_ELEMENT 4u /* persistent element kernel fed by bulk copies (TMA):
                                            each element's stress and memory variables move as
                                            whole chunks, loaded a few elements ahead (same results) */
#define SESNT_FLAG_STRAIN 32u     /* keep the displacement gradient (src/evolution.f90:179-187):
                                     9 more element-local fields read and written each step;
                                     enables SESNT_FIELD_EXX .. _EZZ */
#define SESNT_FLAG_NO_PAIR 128u   /* batched elastic steps: one simulation per thread instead of two
                                     (same results up to the order of the atomic adds) */
#define SESNT_FLAG_NO_STAGE 256u  /* SLS steps: each thread loads its stress and memory variables
                                     (k_element) instead of one bulk copy per element staging
                                     them in shared memory (k_element_stage); same results */
#define SESNT_FLAG_ROTATION 64u   /* compute the rotation strain of the whole volume every step;
                                     enables SESNT_FIELD_ROT_* after any step (without it they
                                     are available after the steps of a rotation snapshot) */
#define SESNT_FLAG_AUTOTUNE 512u  /* sesnt_set_model applies the tuning cache's choice for this GPU
                                     and grid, or runs sesnt_tune and caches its choice */
#define SESNT_FLAG_KAHAN_STRESS 2048u /* compensated (Kahan) stress integration: six compensation
                                         terms per point carry what the stored stress loses to
                                         rounding at each step, the dominant FP32 error against FP64
                                         over long runs; +48 bytes per point and step. Runs the
                                         staged kernel (SLS, degrees 4-7) or one point per thread;
                                         not with the tensor-core, persistent or strain flags */
#define SESNT_FLAG_FORCE64 1024u  /* FP32 wavefields: assemble the force of shared points in FP64
                                     (FP64 atomic adds, 12 more bytes per unique point and step);
                                     FP64 handles already do */

/* element-kernel variants (sesnt_set_element_variant); every variant computes
 * the same step, up to the order of the atomic adds */
#define SESNT_ELEMENT_AUTO 0        /* the launch rules: staged for SLS degrees 4-7, paired for even
                                       elastic batches, else one point per thread */
#define SESNT_ELEMENT_POINT 1       /* one thread per element-local point */
#define SESNT_ELEMENT_PAIR 2        /* two simulations per thread (even elastic batches) */
#define SESNT_ELEMENT_STAGE 3       /* SLS state staged by bulk copy, stored by bulk copy (degrees 4-7);
                                       arg bit 0: one lane per warp waits for the copy; bits 1-2: L2
                                       prefetch of the state 1/4, 1/2 or 1 resident wave ahead (both
                                       also for _STAGE_REG) */
#define SESNT_ELEMENT_STAGE_REG 4   /* the same, stored from registers */
#define SESNT_ELEMENT_PERSISTENT 5  /* persistent blocks fed by bulk copies */
#define SESNT_ELEMENT_COLUMNS 6     /* one thread per (i, j) column of an element (elastic); arg
                                       bits 0-1 select the resident blocks per SM the kernel is sized
                                       for (0: 4, 1: 5, 2: 6, 3: 8), bits 2-3 an L2 prefetch of the
                                       stress 1/4, 1/2 or 1 resident wave ahead */
#define SESNT_ELEMENT_COLUMNS_STAGED 7 /* the same with each block's stress staged by bulk copy */
#define SESNT_ELEMENT_COLUMNS_PAIR 8 /* one thread per column and pair of simulations (even elastic
                                        batches); arg bits 0-1 select the resident blocks per SM
                                        (0: 4, 1: 3, 2 and 3: 2), bits 2-3 the L2 prefetch as for
                                        _COLUMNS */

/* source kinds (sesnt_add_source) */
#define SESNT_SOURCE_MT 0 /* moment tensor: comp = Mxx Mxy Mxz Myy Myz Mzz */
#define SESNT_SOURCE_SF 1 /* single force:  comp = fx fy fz (direction) */

/* wavelets (sesnt_source_signature), src/misc/source_signature_mod.f90 */
#define SESNT_WAVELET_DELTA 0
#define SESNT_WAVELET_RICKER 1
#define SESNT_WAVELET_GAUSS 2
#define SESNT_WAVELET_SIN3 3
#define SESNT_WAVELET_BRUNE 4

/* receiver channels (sesnt_add_receiver), the receiver channel classes of
 * src/config/channel_mod.f90 (construct_channel_container_receiver :270-342):
 * vx vy vz (:505-592; 'e' = vy, 'z' = vz), n = -vx (:532-540), rot_vx rot_vy
 * rot_vz (:620-812), the recorded source fields mxx .. mzz and fx fy fz
 * (:859-1095). */
#define SESNT_CH_VX 1u
#define SESNT_CH_VY 2u
#define SESNT_CH_VZ 4u
#define SESNT_CH_N 8u
#define SESNT_CH_ROT_VX 16u
#define SESNT_CH_ROT_VY 32u
#define SESNT_CH_ROT_VZ 64u
#define SESNT_CH_MXX 128u
#define SESNT_CH_MXY 256u
#define SESNT_CH_MXZ 512u
#define SESNT_CH_MYY 1024u
#define SESNT_CH_MYZ 2048u
#define SESNT_CH_MZZ 4096u
#define SESNT_CH_FX 8192u
#define SESNT_CH_FY 16384u
#define SESNT_CH_FZ 32768u

/* fields (sesnt_get_field) */
#define SESNT_FIELD_VX 0
#define SESNT_FIELD_VY 1
#define SESNT_FIELD_VZ 2
#define SESNT_FIELD_SXX 3 /* the reference's sxx_pml .. szz_pml */
#define SESNT_FIELD_SXY 4
#define SESNT_FIELD_SXZ 5
#define SESNT_FIELD_SYY 6
#define SESNT_FIELD_SYZ 7
#define SESNT_FIELD_SZZ 8
#define SESNT_FIELD_TAPER 9
#define SESNT_FIELD_MASS 10     /* assembled mass matrix MM */
#define SESNT_FIELD_MEMORY 13   /* + comp*3 + k: Mxx,Myy,Mzz,Mxy,Mxz,Myz x 3 mechanisms */
/* volume-snapshot fields (get_field, src/volume_snapshot.f90:192-298) */
#define SESNT_FIELD_PRESSURE 40 /* -(sxx + syy + szz)/3 */
#define SESNT_FIELD_EXX 41      /* strain from the displacement gradient (SESNT_FLAG_STRAIN) */
#define SESNT_FIELD_EXY 42
#define SESNT_FIELD_EXZ 43
#define SESNT_FIELD_EYY 44
#define SESNT_FIELD_EYZ 45
#define SESNT_FIELD_EZZ 46
#define SESNT_FIELD_ROT_VX 47   /* rotation rate as the reference evaluates it after a step */
#define SESNT_FIELD_ROT_VY 48
#define SESNT_FIELD_ROT_VZ 49
#define SESNT_FIELD_LAMBDA 50   /* model fields held on the device */
#define SESNT_FIELD_MU 51
#define SESNT_FIELD_A 52
#define SESNT_FIELD_B 53
#define SESNT_FIELD_C 54

typedef struct sesnt_handle sesnt_t;

/* Grid, domain and time configuration. Field names and meanings follow the
 * reference NAMELIST groups &grid, &model and &time
 * (src/parser/parser.f90:45-69); the last four fields select the GPU build. */
typedef struct sesnt_grid {
    int nx, ny, nz;    /* global element counts (one domain, no partitions) */
    int lpd;           /* Lagrange polynomial degree, 2..7 */
    int taper_width;   /* absorbing taper width in elements */
    float taper_slope; /* taper strength alpha */
    float lat_min, lat_max, lon_min, lon_max; /* degrees */
    float rad_min, rad_max;                   /* metres */
    float dt;          /* time increment in seconds */
    int nt;            /* number of time steps */
    int n_sls;         /* 0 = elastic; 3 = three standard linear solids (needs q) */
    int precision;     /* 4 = FP32 wavefields, 8 = FP64 wavefields */
    int batch;         /* simulations sharing one Earth model (one per source), >= 1 */
    unsigned flags;    /* SESNT_FLAG_* */
} sesnt_grid_t;

/* Replaces the set-up half of the reference driver (src/ses3d-nt.F90:84-160):
 * configuration checks (src/config/config.F90:97-233), geometry and taper
 * (src/geometric_paras.f90:108-325) and init_temp (src/evolution.f90:48-84).
 * Allocates every device buffer the run needs. */
int sesnt_create(const sesnt_grid_t *grid, sesnt_t **out);

/* Frees the handle and its device memory. NULL is accepted. */
int sesnt_destroy(sesnt_t *h);

/* Message of the last failed call on this handle (or, when h is NULL, of the
 * last failed handle-less call on this thread: sesnt_create,
 * sesnt_locate_point). Never NULL. */
const char *sesnt_last_error(const sesnt_t *h);

/* Replaces make_model_parameters / read_model_parameters and
 * init_auxiliary_model_parameters (src/model_paras.F90:97-137, 206-343,
 * 389-416): copies the model (reference raw layout, float32), derives
 * 2mu, kappa, tau, mu_tau and the assembled inverse mass matrix in FP64 on the
 * device. a, b, c may be NULL (isotropic); q may be NULL (elastic). n_sls > 0
 * requires q. Resets the wavefield. */
int sesnt_set_model(sesnt_t *h, const float *rhoinv, const float *lambda, const float *mu, const float *a,
                    const float *b, const float *c, const float *q);

/* Replaces construct_point_cls (src/config/point.f90:150-254): maps
 * (lat [deg], lon [deg], depth [m]) to element indices elem[3] (0-based ex,
 * ey, ez) and the (lpd+1)^3 Vandermonde weights (Fortran order), in float32
 * with the reference's formula order. Returns SESNT_EINVAL for invalid
 * coordinates and SESNT_ENOTFOUND outside the domain. Host-only: needs no
 * GPU and no handle. */
int sesnt_locate_point(const sesnt_grid_t *grid, float lat, float lon, float depth, int elem[3], float *vanderm);

/* Replaces make_source_signature_ for the built-in wavelets
 * (src/config/source.f90:564-652, src/misc/source_signature_mod.f90:50-147):
 * out[i] = wavelet(t = i*dt), i = 0..nt-1, float32. */
int sesnt_source_signature(int wavelet, float onset, float width, float dt, int nt, float *out);

/* Replaces create_from_source_mt / create_from_source_sf and source_cls%add
 * (src/config/source.f90:215-370; channel_mod.f90:859-1095). Registers a
 * source in simulation `sim` (0..batch-1) at element (ex,ey,ez) with
 * Vandermonde weights `vanderm`. kind SESNT_SOURCE_MT takes comp[6] =
 * Mxx Mxy Mxz Myy Myz Mzz; SESNT_SOURCE_SF takes comp[3] = fx fy fz.
 * stf[nt] is the source-time function; channel data are stf*comp in float32.
 * As in the reference, the value injected in step it+1 is the one set after
 * step it (step 1 sees no source), and two sources in one element overwrite
 * each other channel by channel (the later one wins). */
int sesnt_add_source(sesnt_t *h, int sim, int ex, int ey, int ez, const float *vanderm, int kind,
                     const float *comp, const float *stf, int nt);

/* Replaces receiver_cls%record (src/config/receiver.f90:136-142,
 * channel_mod.f90:505-592): registers a receiver at element (ex,ey,ez) with
 * Vandermonde weights; channel_mask is a set of SESNT_CH_*. Every receiver is
 * recorded in every simulation of the batch. Returns the receiver index
 * (>= 0) or an error. */
int sesnt_add_receiver(sesnt_t *h, int ex, int ey, int ez, const float *vanderm, unsigned channel_mask);

/* One pass of the reference forward loop body for step `it` (1..nt):
 * ses3d_evolution, then source add(it), then receiver record(it)
 * (src/ses3d-nt.F90:240-250). Asynchronous on the handle's stream; replayed
 * from a captured one-step CUDA graph unless SESNT_FLAG_NO_GRAPH is set. */
int sesnt_step(sesnt_t *h, int it);

/* Steps it0 .. it0+nsteps-1. Long runs are replayed from a captured CUDA
 * graph unless SESNT_FLAG_NO_GRAPH is set. Asynchronous. */
int sesnt_run(sesnt_t *h, int it0, int nsteps);

/* Same as sesnt_run, bracketed by CUDA events recorded on the handle's own
 * stream; waits for completion and stores the elapsed milliseconds. */
int sesnt_run_timed(sesnt_t *h, int it0, int nsteps, float *ms);

/* Runs steps it0 .. it0+nsteps-1 with direct launches and CUDA events
 * recorded on the handle's stream between the kernels of each step; stores
 * the summed device milliseconds of the element, source, node and receiver
 * kernels in ms[0..3]. Does the full work of sesnt_run. Synchronous. */
int sesnt_run_profiled(sesnt_t *h, int it0, int nsteps, float ms[4]);

/* Waits for all work queued on the handle. */
int sesnt_synchronize(sesnt_t *h);

/* No counterpart in the reference. Tunes the element kernel on this handle's
 * grid, precision and batch: times every variant that computes this step
 * (one point per thread, paired simulations, one thread per column at four
 * register budgets with the stress loaded per point or staged per block,
 * the staged kernel with bulk or register stores, 0/8 KB copy pieces, its
 * wait polled by every thread or by one lane per warp and an L2 prefetch of
 * the state 1/4, 1/2 or 1 wave of resident blocks ahead, the persistent
 * kernel) with CUDA events on the
 * handle's stream, keeps the fastest and appends it to the tuning cache
 * ($SESNT_TUNE_CACHE, else $HOME/.cache/sesnt-tune.txt), keyed by GPU name,
 * SM count, degree, precision, SLS, anisotropy, batch and grid. Runs the
 * kernel on the zero wavefield, which it leaves zero: call it after
 * sesnt_set_model or sesnt_reset and before stepping (SESNT_ESTATE
 * otherwise). report (may be NULL) receives the timings as text.
 * Synchronous. */
int sesnt_tune(sesnt_t *h, char *report, int report_len);

/* No counterpart in the reference. Sets the element-kernel variant
 * (SESNT_ELEMENT_*), its argument and the bulk-copy piece size in bytes
 * (a multiple of 16, 0 = one copy per state unit; default 8192). A variant
 * the handle's configuration does not have falls back to the launch rules. */
int sesnt_set_element_variant(sesnt_t *h, int variant, int arg, int piece);

/* The element kernel a step of this handle launches (its name) and the
 * current choice[3] = {variant, arg, piece} (choice may be NULL). */
int sesnt_element_kernel(const sesnt_t *h, char *name, int name_len, int choice[3]);

/* Zeroes the wavefield, memory variables and seismograms (model kept) and
 * clears the error word of an earlier SESNT_ETIMEOUT. */
int sesnt_reset(sesnt_t *h);

/* No counterpart in the reference. Failure-detection hook: every device-side
 * completion wait (the mbarrier waits of the tensor-core and of the
 * bulk-copy element kernels) gives up
 * after `polls` polls (default 4,194,304), sets the handle's error word and
 * leaves the state of its points unchanged; the next synchronising call then
 * returns SESNT_ETIMEOUT until sesnt_reset. drop_completion != 0 makes that
 * kernel signal no completion, so its waits run out: a test of the path
 * that faults nothing. */
int sesnt_set_wait_limit(sesnt_t *h, int polls, int drop_completion);

/* Seismograms, float32 [batch][nrec][3][nt] with components vx, vy, vz
 * (channels not requested at sesnt_add_receiver are zero). Synchronous. */
int sesnt_get_seismograms(sesnt_t *h, float *out);

/* The samples of step `it` (1..nt) of every receiver, float32
 * [batch][nrec][3] (vx, vy, vz): what receiver_cls%record(it) stores on the
 * host each step in the reference (src/config/receiver.f90:136-142).
 * Synchronous, but it waits only until step `it` is done: later steps
 * already queued keep running. The receiver kernel also writes every sample
 * into a float32 copy in mapped, pinned host memory, so once the step is done
 * the samples are read from host memory with no device copy. Where mapped
 * memory is unavailable, they are copied through the handle's own copy
 * stream. For a Fortran driver that keeps its own traces. */
int sesnt_get_samples(sesnt_t *h, int it, float *out);

/* Checkpoint and resume (no counterpart in the reference, which keeps no
 * restartable state). sesnt_state_bytes gives the size of the host buffer;
 * sesnt_save_state copies the time-stepping state into it: velocity,
 * stress, memory variables, the compensation terms of the velocity and of the
 * stress (SESNT_FLAG_KAHAN, SESNT_FLAG_KAHAN_STRESS), displacement gradient,
 * the recorded traces and the last step. sesnt_load_state restores it into a
 * handle with the same grid, precision, flags and receivers (model and
 * sources are not part of the state), after which stepping continues at
 * the saved step + 1. Synchronous. */
long long sesnt_state_bytes(sesnt_t *h);
int sesnt_save_state(sesnt_t *h, void *buf);
int sesnt_load_state(sesnt_t *h, const void *buf);

/* One receiver channel of simulation `sim` (SESNT_CH_*, a single bit that
 * was requested for that receiver), float32 [nt]. Synchronous. No single
 * counterpart in the reference: channel_cls%data of one receiver channel
 * (src/config/channel_mod.f90:44-50). */
int sesnt_get_trace(sesnt_t *h, int sim, int receiver, unsigned channel, float *out);

/* Replaces output_raw_cls%mpi_write (src/output_raw.f90:117-168) with the
 * step window of volume_snapshot_cls (src/volume_snapshot.f90:123-135): after every step it with ts_start <= it <= ts_end and
 * (it - ts_start) % ts_increment == 0, field `which` of simulation `sim` is
 * copied asynchronously to pinned host memory and written by a background
 * thread to "<prefix><attribute>_<it>.vol" in the reference raw layout
 * (float32, Fortran order). ts_end <= 0 means nt; prefix NULL or "" means
 * "./"; attribute NULL means the field's name (sesnt_field_name). Existing
 * files are replaced only with override != 0. Returns the snapshot index or
 * an error (range checks of the reference constructor, :71-113). */
int sesnt_add_snapshot(sesnt_t *h, int sim, int which, int ts_start, int ts_increment, int ts_end,
                       const char *prefix, const char *attribute, int override);

/* Waits until every snapshot file queued so far is written; returns the
 * first write error since the last call (message in sesnt_last_error). */
int sesnt_snapshots_wait(sesnt_t *h);

/* Name of a field (the attribute of get_field in
 * src/volume_snapshot.f90:192-298) or NULL, and the field of a name
 * (case-insensitive; "cs"/"vs", "cp"/"vp" aliases have no device field) or
 * -1. */
const char *sesnt_field_name(int which);
int sesnt_field_id(const char *name);

/* Copies field `which` (SESNT_FIELD_*) of simulation `sim` to `out` in the
 * reference raw layout (element-local copies of shared nodes included), as
 * float32 (out_precision 4) or float64 (8). Synchronous. */
int sesnt_get_field(sesnt_t *h, int sim, int which, void *out, int out_precision);

/* Global minimum and maximum of the velocity components of simulation `sim`,
 * the quantity the reference prints every step (v_ptp_glb,
 * src/elastic_vars.F90:179-213). Returns SESNT_ENONFINITE if any value is
 * NaN or Inf. Synchronous: one reduction launch on the handle's stream,
 * whose result arrives in mapped host memory. */
int sesnt_v_ptp(sesnt_t *h, int sim, float out[2]);

/* Kinetic energy of simulation `sim`, the reference's kinetic_energy
 * (src/elastic_vars.F90:218-246): 0.5 * jac * sum over element-local points
 * of (vx^2 + vy^2 + vz^2) * r^2 sin(theta) * rho * w_i w_j w_k, in joules.
 * Computed on the device in FP64 from the unique-point velocity and the
 * assembled mass (every copy of a shared point holds the same velocity), with
 * a fixed summation order, so repeated calls give identical results.
 * SESNT_ENONFINITE if the result is NaN or Inf. Synchronous. */
int sesnt_kinetic_energy(sesnt_t *h, int sim, double *out);

/* Sums an element-local field over every copy of each shared GLL point and
 * writes the sum back to every copy: the effect of
 * communicate_local_boundaries (src/communicate_fields.F90:48-79) on one
 * rank, done on the device through the library's unique-point numbering.
 * field is float32 in the reference raw layout; in place. Synchronous. */
int sesnt_assemble_field(sesnt_t *h, float *field);

/* No counterpart in the reference. The assembly of sesnt_assemble_field, for
 * callers that cannot allocate device memory at the time of the call (a time
 * loop that must not synchronise the whole device as cudaMalloc/cudaFree may,
 * a host that reserved all device memory up front). d_in and d_out are device
 * pointers to float32 fields in the reference raw layout and may be the same
 * buffer. Nothing is allocated: the unique-point sums use a fixed device
 * array of 4,194,304 floats (16 MiB) that every GPU loading this library
 * holds until exit; grids with more unique points get SESNT_ERANGE. The sums
 * are float32 whatever the handle's precision (sesnt_assemble_field sums an
 * FP64 handle's field in float64), so on FP64 handles the two can differ by
 * float32 rounding. The first call on a device looks up that array's address
 * (a set-up step): make that first call before any stream capture. All calls
 * share the array: calls that overlap on the GPU race. The calling thread's
 * current device must be the handle's (SESNT_EINVAL otherwise). Runs on the
 * handle's stream and synchronises that stream before it returns. */
int sesnt_assemble_field_noalloc(sesnt_t *h, const float *d_in, float *d_out);

/* Sizes: out[0] elements, out[1] element-local GLL points (N_loc), out[2]
 * unique GLL points (N_uni), out[3] device bytes held by the handle,
 * out[4] algorithmic HBM bytes of one time step (whole batch),
 * out[5] device kernel launches per time step. */
int sesnt_info(const sesnt_t *h, long long out[6]);

/* Device bytes sesnt_create + sesnt_set_model would allocate for `grid`
 * (used by a scheduler to admit work by HBM footprint). */
long long sesnt_footprint_bytes(const sesnt_grid_t *grid);

/* The stream the handle launches on (cudaStream_t), for callers that order
 * their own work after the library's. */
void *sesnt_stream(const sesnt_t *h);

/* ------------------------------------------------------------------------
 * Files and configuration (host only, no GPU needed)
 * ------------------------------------------------------------------------ */

/* Message of the last failed call of this section on this thread. */
const char *sesnt_io_last_error(void);
const char *sesnt_config_last_error(void);

/* Reads a raw model or field file: native float32 in the reference raw
 * layout, no header, with the file-size check of src/mpi_parallel_io.F90:
 * 300-309 (a size mismatch is SESNT_EINVAL, "wrong file size"). */
int sesnt_read_raw_field(const char *path, int nx, int ny, int nz, int lpd, float *out);

/* Writes a raw field (src/mpi_parallel_io.F90:121-190); an existing file is
 * only replaced when override is nonzero. */
int sesnt_write_raw_field(const char *path, int nx, int ny, int nz, int lpd, const float *data, int override);

/* Header values of one SAC trace (src/sac_io/sac_io_mod.f90:178-222). Text
 * fields need not be NUL-terminated; they are blank padded like Fortran
 * CHARACTER assignments. date_time = [year, month, day, GMT offset minutes,
 * hour, minute, second, millisecond] as in the &time group. */
typedef struct sesnt_sac_info {
    float lat, lon, depth, dt;
    char network[8], station[8], location[8], channel[8], event[16];
    int override;
    int date_time[8];
} sesnt_sac_info_t;

/* Writes a SAC trace as the reference's receiver_cls%write does
 * (src/config/receiver.f90:154-192, src/sac_io/sac_io_mod.f90:453-506). */
int sesnt_write_sac(const char *path, const sesnt_sac_info_t *info, const float *data, int npts);

/* "[network].[station].[location].[channel].sac" (auto_file_name,
 * src/sac_io/sac_io_mod.f90:407-427). */
int sesnt_sac_file_name(const sesnt_sac_info_t *info, char *out, int out_len);

/* Day of the year of a Gregorian date (iday in src/sac_io/sac_header_mod.f90). */
int sesnt_day_of_year(int year, int month, int day);

/* Courant number (out[0]) and maximum resolved frequency in Hz (out[1]) of a
 * model on a grid: cfl_loc and f_c_loc of src/model_paras.F90:464-561, in
 * float32. Model arrays in the reference raw layout. */
int sesnt_courant(const sesnt_grid_t *grid, const float *rhoinv, const float *lambda, const float *mu, float out[2]);

/* The reference configuration file (NAMELIST groups, src/parser/parser.f90),
 * parsed. */
typedef struct sesnt_config sesnt_config_t;
int sesnt_config_load(const char *path, sesnt_config_t **out);
int sesnt_config_free(sesnt_config_t *cfg);
/* Number of groups called `group` (e.g. "receiver"). */
int sesnt_config_count(const sesnt_config_t *cfg, const char *group);
/* &grid, &model and &time as a grid (precision 4, batch 1, n_sls 3 when a q
 * model file is named). */
int sesnt_config_grid(const sesnt_config_t *cfg, sesnt_grid_t *grid);
/* Value of `key` in the idx-th `group` as text (several values separated by
 * blanks; logicals as T/F). SESNT_ENOTFOUND when absent. */
int sesnt_config_get(const sesnt_config_t *cfg, const char *group, int idx, const char *key, char *out, int out_len);
/* JSON image of the whole file: {"group": [{key: value | [values]}...]}.
 * With out == NULL only *needed (bytes incl. NUL) is set. */
int sesnt_config_json(const sesnt_config_t *cfg, char *out, long long out_len, long long *needed);

/* The reference forward workflow (src/ses3d-nt.F90:77-275, workflow
 * 'forward') on the GPU: config, raw model files, sources (&source_mt,
 * &source_sf with built-in wavelets), receivers (vx, vy, vz channels), all nt
 * steps, one SAC file per receiver channel. precision 4 or 8. *n_traces gets
 * the number of SAC files written. */
int sesnt_forward(const char *config_path, int precision, int *n_traces);

/* ------------------------------------------------------------------------
 * Serving many simulations on one GPU. No counterpart in the reference
 * (which runs one event per MPI job); built on the entry points above.
 * ------------------------------------------------------------------------ */

typedef struct sesnt_server sesnt_server_t;

typedef struct sesnt_server_config {
    long long device_bytes; /* HBM budget for admitted work; <= 0: 85% of free memory */
    int max_active;         /* simultaneously running simulation batches (<= 0: 16) */
    int chunk_steps;        /* steps a batch advances per scheduling turn (<= 0: 64) */
    int max_batch;          /* simulations per batch (<= 0: all sources of a request) */
} sesnt_server_config_t;

/* One forward request: a model, its sources (one simulation each) and a
 * receiver set recorded in every simulation. Arrays are copied at submit. */
typedef struct sesnt_request {
    sesnt_grid_t grid;        /* grid.batch is ignored */
    const float *rhoinv, *lambda, *mu, *a, *b, *c, *q; /* reference raw layout; a..q may be NULL */
    int n_sources;
    const int *src_elem;      /* [n_sources][3] element indices (0-based) */
    const int *src_kind;      /* [n_sources] SESNT_SOURCE_* */
    const float *src_vanderm; /* [n_sources][(lpd+1)^3] */
    const float *src_comp;    /* [n_sources][6] (MT) or first 3 used (SF) */
    const float *src_stf;     /* [n_sources][nt] */
    int n_receivers;
    const int *rec_elem;      /* [n_receivers][3] */
    const float *rec_vanderm; /* [n_receivers][(lpd+1)^3] */
    const unsigned *rec_mask; /* [n_receivers] SESNT_CH_* sets, or NULL for vx|vy|vz */
} sesnt_request_t;

typedef struct sesnt_server_stats {
    long long completed, failed, queued, active;
    long long device_bytes_used, device_bytes_budget;
    long long total_updates;      /* GLL-point-updates of completed requests */
    double latency_p50, latency_p99, latency_max, queue_wait_p50; /* seconds, submit to done */
    double wall_seconds;          /* first submit to last completion (completed requests) */
    double updates_per_second;    /* total_updates / wall_seconds */
} sesnt_server_stats_t;

/* Starts the scheduler thread on the current device. */
int sesnt_server_create(const sesnt_server_config_t *cfg, sesnt_server_t **out);
/* Stops the scheduler after the work in flight, frees everything. */
int sesnt_server_destroy(sesnt_server_t *s);
/* Queues a request; returns at once with its id. SESNT_ENOMEM if even one
 * simulation of it can never fit the budget. */
int sesnt_server_submit(sesnt_server_t *s, const sesnt_request_t *req, long long *id);
/* Waits up to timeout_s seconds; SESNT_ETIMEOUT if not done by then. */
int sesnt_server_wait(sesnt_server_t *s, long long id, double timeout_s);
/* Seismograms [n_sources][n_receivers][3][nt] of a finished request and
 * times[0] = latency (submit to done), times[1] = queue wait. */
int sesnt_server_result(sesnt_server_t *s, long long id, float *seis, double times[2]);
/* Forgets a finished request (frees its host copies and results). */
int sesnt_server_release(sesnt_server_t *s, long long id);
/* Cancels a request that has not started; started work is not interrupted. */
int sesnt_server_cancel(sesnt_server_t *s, long long id);
int sesnt_server_stats(sesnt_server_t *s, sesnt_server_stats_t *out);
const char *sesnt_server_last_error(const sesnt_server_t *s);

#ifdef __cplusplus
}
#endif

#endif /* SESNT_H */
