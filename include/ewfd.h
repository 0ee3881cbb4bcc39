/*
 * ewfd.h -- C ABI of the GB300 staggered-grid elastic FDTD solver (libewfd.so).
 *
 * Drop-in boundary for the reference's time loop.  The reference is one executable per
 * scenario whose main() reads fixed-name float32 files from the current directory, runs the
 * loop and writes "0_0_<name>.res" files (src/FastWaveED_GPU3D_v1_DC_Earthquake_FULL_OK4_final/
 * FastWaveED_GPU3D_v1.cu:390-559, "OK4" below; src/FastWaveED_GPU3D_v1_9km_station_ANISO/
 * FastWaveED_GPU3D_v1_9kmst_ANISO.cu:391-608, "ANISO" below).  Everything that executable
 * fixes at compile time (-DNBX.. grid, nt, source cell, receiver cells, precision) is a
 * runtime value here.
 *
 * Conventions
 *   - Every function returns 0 (EWF_OK) or a negative ewf_status; none calls exit/abort.
 *   - Host arrays use the reference layout: x fastest, idx = i + j*Px + k*Px*Py with the
 *     array's own extents (Vx (nx+1,ny,nz), sxy (nx+1,ny+1,nz), ... OK4:431-439).
 *   - Buffers passed in are owned by the caller and copied; the handle owns device memory.
 *   - A handle is not thread-safe; it owns one CUDA stream on the device current at create.
 */
#ifndef EWFD_H
#define EWFD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EWF_ABI_VERSION 6

typedef enum ewf_status {
    EWF_OK = 0,
    EWF_ERR_ARG = -1,         /* invalid argument / size mismatch */
    EWF_ERR_CUDA = -2,        /* CUDA runtime error (message in ewf_last_error) */
    EWF_ERR_NOMEM = -3,       /* device or host allocation failed */
    EWF_ERR_IO = -4,          /* legacy file missing, unreadable or of the wrong size */
    EWF_ERR_STATE = -5,       /* call out of order (e.g. run before inputs are set) */
    EWF_ERR_CFL = -6,         /* time step above the stability limit */
    EWF_ERR_NONFINITE = -7,   /* NaN/Inf detected in the receiver traces */
    EWF_ERR_UNSUPPORTED = -8, /* combination the reference leaves undefined / not built */
    EWF_ERR_NODEVICE = -9     /* no CUDA device */
} ewf_status;

typedef enum ewf_model {
    EWF_MODEL_ISO = 0,    /* isotropic: c11/c12 fields, scalar shear modulus and 1/rho (OK4:285-388) */
    EWF_MODEL_ORTHO = 1,  /* orthorhombic: 9 C_ij fields + staggered buoyancy (ANISO:287-389) */
    EWF_MODEL_ISO_HET = 2 /* isotropic with heterogeneous staggered shear moduli and buoyancy, the
                           * 9 km station scheme (FastWaveED_GPU3D_v1_9kmst.cu:287-388): c11/c12
                           * cell fields (EWF_M_C11/C12), c44u_hetxy/xz/yz edge fields in the
                           * EWF_M_C66XY/C55XZ/C44YZ slots, 1/rho in EWF_M_BX/BY/BZ; 3-D or separable
                           * weights; the ANISO loop order (BC1, then the source) */
} ewf_model;

typedef enum ewf_precision {
    EWF_PREC_F32 = 0,       /* FP32, reference arithmetic (OK4:15-19) */
    EWF_PREC_F32_KAHAN = 1, /* FP32 fields, compensated velocity time accumulation */
    EWF_PREC_F64 = 2        /* FP64 (OK4:20-23 with USE_SINGLE_PRECISION off) */
} ewf_precision;

typedef enum ewf_damping {
    EWF_DAMP_PML1D = 0,    /* 1-D profiles weights_x/y/z (n+1 each), OK4 usage (OK4:307-329, 361-375) */
    EWF_DAMP_W3D = 1,      /* 3-D weights field (nx,ny,nz), ANISO usage (ANISO:312-386) */
    EWF_DAMP_SEPARABLE = 2, /* ANISO usage with W[i,j,k] = (px[i]*py[j])*pz[k] formed on the fly */
    EWF_DAMP_PERCOMP = 3    /* isotropic model only: one 3-D weight field per stress component, the
                             * normal-stress ones also weighting the velocities, w*(sigma + ...) and
                             * w*(V/dt + b*div)*dt, shear moduli c66 (xy), c55 (xz), c44 (yz): the
                             * DC_Earthquake solver (src/FastWaveED_GPU3D_v1_DC_Earthquake/
                             * FastWaveED_GPU3D_v1.cu:298-320, 344-360), ANISO's loop order */
} ewf_damping;

typedef enum ewf_step_form {
    EWF_STEP_SPLIT = 0, /* stress kernel, injection, velocity kernel (reference order OK4:485-498) */
    EWF_STEP_FUSED = 1, /* one-pass step kernel, double-buffered state (models 0 and 1): tiles
                         * that recompute their stress halo, bands of full-width rows (one
                         * thread-block cluster each) or TMA-staged tiles (ewf_set_onepass) */
    EWF_STEP_WAVE = 2   /* one persistent launch of the stress and velocity updates over tile x slab
                         * items in dependency order, in place: the velocity update reads the new
                         * stresses back from L2 (every model, damping and precision) */
} ewf_step_form;

typedef enum ewf_free_surface {
    EWF_FS_BC1 = 0,  /* BC1 after the stress update: szz = 0 on plane 0, sxz/syz on plane 1 = plane 2 / 3
                      * (OK4:271-283, ANISO:270-285; every shipped scheme but the two below) */
    EWF_FS_NONE = 1  /* no BC1: the stress planes are left as updated -- the "diff_BC" schemes, whose
                      * BC1 launch is commented out (src/FastWaveED_GPU3D_v1_DC_Earthquake_FULL_diff_BC_OK2/
                      * FastWaveED_GPU3D_v1.cu:453, ..._diff_BC2_OK3/FastWaveED_GPU3D_v1.cu:476) */
} ewf_free_surface;

typedef enum ewf_src_order {
    EWF_SRC_BEFORE_BC1 = 0, /* OK4: injection inside the stress kernel, BC1 after (OK4:336-342, 490) */
    EWF_SRC_AFTER_BC1 = 1   /* ANISO: BC1, then the source kernel (ANISO:533-535) */
} ewf_src_order;

/* Field ids for ewf_set_field / ewf_get_field.  Extents are the reference's. */
typedef enum ewf_field {
    EWF_F_VX = 0, EWF_F_VY = 1, EWF_F_VZ = 2,          /* (nx+1,ny,nz) (nx,ny+1,nz) (nx,ny,nz+1) */
    EWF_F_SXX = 3, EWF_F_SYY = 4, EWF_F_SZZ = 5,       /* (nx,ny,nz) */
    EWF_F_SXY = 6, EWF_F_SXZ = 7, EWF_F_SYZ = 8,       /* (nx+1,ny+1,nz) (nx+1,ny,nz+1) (nx,ny+1,nz+1) */
    /* materials, isotropic: c11u_het.dat, c12u_het.dat (OK4:415-418) */
    EWF_M_C11 = 16, EWF_M_C12 = 17,
    /* materials, orthorhombic (ANISO:411-447): C22m C33m C13m C23m, edge moduli, buoyancy */
    EWF_M_C22 = 18, EWF_M_C33 = 19, EWF_M_C13 = 20, EWF_M_C23 = 21,
    EWF_M_C66XY = 22, /* (nx+1,ny+1,nz) C66mxy.dat */
    EWF_M_C55XZ = 23, /* (nx+1,ny,nz+1) C55mxz.dat */
    EWF_M_C44YZ = 24, /* (nx,ny+1,nz+1) C44myz.dat */
    EWF_M_BX = 25,    /* (nx+1,ny,nz) vrho_x_11_hc.dat */
    EWF_M_BY = 26,    /* (nx,ny+1,nz) vrho_y_11_hc.dat */
    EWF_M_BZ = 27,    /* (nx,ny,nz+1) vrho_z_11_hc.dat */
    /* damping */
    EWF_D_WX = 32, EWF_D_WY = 33, EWF_D_WZ = 34, /* PML1D: n+1 each (weights_x/y/z.dat); SEPARABLE: n each */
    EWF_D_W3D = 35,                              /* (nx,ny,nz) weights.dat */
    /* PERCOMP weights in their component's layout: weights_x/y/z.dat (Vx, Vy, Vz extents),
     * weights_xy/xz/yz.dat (sxy, sxz, syz extents, as the DC_Earthquake driver writes them) */
    EWF_D_PX = 36, EWF_D_PY = 37, EWF_D_PZ = 38, EWF_D_PXY = 39, EWF_D_PXZ = 40, EWF_D_PYZ = 41
} ewf_field;

typedef struct ewf_params {
    int32_t nx, ny, nz;   /* grid; replaces nx = 64*NBX - OVERX etc. (OK4:39-41) */
    int32_t nt;           /* time steps of a full run; replaces const nt (OK4:43) */
    int32_t model;        /* ewf_model */
    int32_t precision;    /* ewf_precision */
    int32_t damping;      /* ewf_damping */
    int32_t src_order;    /* ewf_src_order */
    int32_t over_y;       /* legacy OVERY: BC1 rows are j < min(nx, ny + over_y) (OK4:279-281) */
    int32_t nout;         /* progress line every nout steps (OK4:502-504); 0 = quiet */
    int32_t kchunk;       /* planes per CTA of the z-marching kernels; 0 = autotuned/default */
    int32_t graph_steps;  /* steps captured per CUDA graph; 0 = default, <0 = no graph */
    int32_t check_finite; /* 1: ewf_run checks the receiver traces for NaN/Inf */
    int32_t fused;        /* ewf_step_form: 0 (default) two kernels; 1 one-pass kernel; 2 wavefront */
    double dx, dy, dz, dt; /* pa1[0..3] (OK4:404) */
    double c66;            /* isotropic shear modulus pa2[7] (OK4:405); PERCOMP: the xy one */
    double c44, c55;       /* PERCOMP shear moduli of yz and xz, pa2[5], pa2[6] */
    double bx, by, bz;     /* isotropic 1/rho pa3[0..2] (OK4:407) */
    double vdamp;          /* linear velocity damping: V_new = update - vdamp * V_old (16 km station
                            * scheme, FastWaveED_GPU3D_v1_16kmst.cu:337-349, vdamp = 2.2 * 4.6729e-04
                            * in float); 0 = off.  Models 1 and 2, FP32 / FP64, not the one-pass step. */
    const char *workdir;   /* legacy *.dat inputs and *.res outputs (NULL = ".") */
    int32_t free_surface;  /* ewf_free_surface: 0 (default) BC1, 1 none; not the one-pass step */
    int32_t reserved;      /* 0 */
    double surface_mu;     /* isotropic scheme with 1-D PML: > 0 replaces the shear modulus c66 on the plane
                            * k = 1 (the diff_BC2_OK3 scheme's c44u = 1e-5 there,
                            * ..._diff_BC2_OK3/FastWaveED_GPU3D_v1.cu:309-314); 0 = off; not the one-pass
                            * step.  The other schemes carry such a layer in their edge shear-modulus fields. */
} ewf_params;

typedef struct ewf_handle ewf_handle;

int ewf_abi_version(void);
const char *ewf_strerror(int status);
/* Text of the last error on this thread (CUDA message, file name, ...). */
const char *ewf_last_error(void);

/* Defaults: FP32, iso, PML1D, before-BC1 order, over_y 0, graph on, two-kernel step. */
void ewf_params_default(ewf_params *p);

/* Fills dx, dy, dz, dt, c66, bx, by, bz of p from p->workdir's pa1/pa2/pa3.dat (OK4:401-407)
 * and, when p->nt is 0, nt from the length of Src.dat (the reference's compile-time nt, OK4:43). */
int ewf_legacy_params(ewf_params *p);

/* Validates sizes and allocates device memory (replaces OK4:428-459 zeros/cudaMalloc). */
int ewf_create(const ewf_params *p, ewf_handle **out);
void ewf_destroy(ewf_handle *h);
int ewf_get_params(const ewf_handle *h, ewf_params *out);

/* Reads pa1/pa2/pa3/MTS/Src and the model files of p->model from p->workdir exactly as
 * OK4:401-454 (iso) / ANISO:402-487 (ortho), checks their sizes, sets the legacy source cell
 * (OK4:450-452 / ANISO:483-485, overridable with ewf_set_moment_tensor afterwards) and the 4
 * legacy receivers (OK4:383-386 / ANISO:263-266). */
int ewf_load_legacy_inputs(ewf_handle *h);

/* Copies a host array (dtype_bytes 4 = float32, 8 = float64) into a field (replaces
 * load3 + cudaMemcpy, OK4:195-198).  n must equal the field's element count. */
int ewf_set_field(ewf_handle *h, int32_t field, const void *host, size_t n, int32_t dtype_bytes);
/* Snapshot of a field back to the host in the reference layout (replaces gather, OK4:75). */
int ewf_get_field(ewf_handle *h, int32_t field, void *host, size_t n, int32_t dtype_bytes);
/* Element count of a field for this grid (0 for an unknown id). */
size_t ewf_field_size(const ewf_handle *h, int32_t field);

/* Source time function Src[it] (Src.dat, OK4:454); n >= steps that will be run. */
int ewf_set_stf(ewf_handle *h, const double *stf, size_t n);
/* Moment tensor (xx,yy,zz,xy,xz,yz) injected at the reference's stencil around cell
 * (xs,ys,zs): stencil 0 = OK4 offsets (OK4:336-342), 1 = ANISO offsets (ANISO:233-247). */
int ewf_set_moment_tensor(ewf_handle *h, const double mt[6], int32_t xs, int32_t ys, int32_t zs, int32_t stencil);
/* General point sources: n <= 64 entries of (field id 3..8, i, j, k) and coefficients. */
int ewf_set_sources(ewf_handle *h, int32_t n, const int32_t *comp_ijk, const double *coef);
/* Receivers: n entries of (i, j, k, field id 0..8), sampled after every velocity update. */
int ewf_set_receivers(ewf_handle *h, int32_t n, const int32_t *ijk_comp);

/* Number of receivers currently set. */
int ewf_receiver_count(const ewf_handle *h, int32_t *n);

/* Zeroes the 9 state fields, compensation, traces and the step counter. */
int ewf_reset(ewf_handle *h);
/* Advances nsteps time steps (OK4:485-505 / ANISO:519-555); resumable; synchronous. */
int ewf_run(ewf_handle *h, int32_t nsteps);
/* Steps completed so far. */
int ewf_get_step(const ewf_handle *h, int32_t *it);
/* Receiver traces, FP64, out[r*nt + it] for r < n_rec, it < nt. */
int ewf_get_seismograms(ewf_handle *h, double *out, size_t n);
/* Device time of the last ewf_run in milliseconds (CUDA events on the handle's stream). */
int ewf_last_run_ms(const ewf_handle *h, double *ms);

/* Diagnostics: advances nsteps time steps launching each kernel between CUDA events on the
 * handle's stream (no graph) and returns the average device time per launch in ms of
 * out_ms[0] stress (the whole step for the one-pass and wavefront forms), [1] injection, [2] velocity, [3] receiver
 * gather (0 for kernels the step does not launch). */
int ewf_time_kernels(ewf_handle *h, int32_t nsteps, double out_ms[4]);
/* Number of kernel launches one time step issues. */
int ewf_launches_per_step(const ewf_handle *h, int32_t *n);

/* Autotuner: times `nsteps` steps for each z-chunk candidate (planes per CTA) with CUDA events,
 * keeps the fastest (returned in *kchunk, may be NULL) and resets the state.  The two-kernel step
 * also tunes its tile height (4, 8, 16 rows; ewf_get_tile) and then its L2 prefetch distance
 * (0, 2, 3, 4 planes; ewf_get_l2_prefetch), the wavefront step its lag (all kept in the handle). */
int ewf_autotune(ewf_handle *h, int32_t nsteps, int32_t *kchunk);

/* Two-kernel step (fused = EWF_STEP_SPLIT): the height of a CTA's tile in rows of 32 columns
 * (a power of two, 1..16 in FP32, 1..8 in FP64; default 8), set by ewf_autotune together with the
 * z-chunk; results do not depend on it.  ewf_set_tile: EWF_ERR_STATE for the other step forms. */
int ewf_set_tile(ewf_handle *h, int32_t tile_y);
int ewf_get_tile(const ewf_handle *h, int32_t *tile_y);
/* One-pass step (fused = EWF_STEP_FUSED): the kernel that runs it.
 *   EWF_ONEPASS_TILE (default): tiles of 32 x 8 columns that recompute their stress halo (any grid,
 *     every precision);
 *   EWF_ONEPASS_BAND4 / _BAND8: bands of 4 / 8 full-width rows, each one thread-block cluster of
 *     CTAs of 64 columns that hand their stress edge columns to each other through distributed
 *     shared memory (nx <= 16 * 64; BAND8 in FP32 only);
 *   EWF_ONEPASS_STAGED: tiles of 64 x 8 columns whose planes (with their halo) are staged in
 *     shared memory by TMA copies two planes ahead; the stress ring the velocity update reads is
 *     recomputed from the staged plane (FP32 without compensation).
 * ewf_autotune picks the kernel with the z-chunk.  EWF_ERR_UNSUPPORTED where a kernel cannot run,
 * EWF_ERR_STATE for the other step forms.  Results do not depend on it.  (Replaces nothing in the
 * reference: its time loop is the two-launch step, OK4:485-505.) */
typedef enum ewf_onepass {
    EWF_ONEPASS_TILE = 0,
    EWF_ONEPASS_BAND4 = 1,
    EWF_ONEPASS_BAND8 = 2,
    EWF_ONEPASS_STAGED = 3
} ewf_onepass;
int ewf_set_onepass(ewf_handle *h, int32_t kernel);
int ewf_get_onepass(const ewf_handle *h, int32_t *kernel);
/* Test hook of the staged kernel's failure path: with plane >= 0, the first CTA of every later
 * staged launch never issues the copies of that plane (a stage fill nothing completes) and every
 * wait for a plane stage gives up after `polls` polls; the launch still ends and ewf_run returns
 * EWF_ERR_CUDA (the state of that run is invalid; the handle stays usable after ewf_reset).
 * plane < 0 restores normal operation (default limit 2^22 polls). */
int ewf_staged_test_hold(int32_t plane, int32_t polls);
/* Two-kernel step: launch each kernel as a programmatic dependent of the previous one (1, the
 * default), so its CTAs are scheduled while the previous kernel finishes instead of after a launch
 * gap; every kernel still waits for the previous grid before it touches the state.  0: plain
 * stream-ordered launches.  The handle turns it off by itself if graph capture refuses it.
 * Results do not depend on it. */
int ewf_set_dependent_launch(ewf_handle *h, int32_t on);
int ewf_get_dependent_launch(const ewf_handle *h, int32_t *on);
/* Two-kernel step: the velocity kernel asks L2 for the input lines of the plane `planes` ahead
 * (0..8; 0 = off, the default; ewf_autotune picks it).  A hint: results do not depend on it. */
int ewf_set_l2_prefetch(ewf_handle *h, int32_t planes);
int ewf_get_l2_prefetch(const ewf_handle *h, int32_t *planes);

/* Wavefront step (fused = EWF_STEP_WAVE): the lag of the velocity items behind the stress items
 * in percent of the resident CTAs, 1..100000 (set by ewf_autotune; results do not depend on it).
 * EWF_ERR_STATE for the other step forms. */
int ewf_set_wave(ewf_handle *h, int32_t lag_pct);
int ewf_get_wave(const ewf_handle *h, int32_t *lag_pct);
/* Diagnostic for tests of the failure path: stress item `item` of the wavefront step never
 * publishes its done flag, so the velocity items that depend on it give up after their bounded
 * wait and ewf_run returns EWF_ERR_CUDA (the state of that run is invalid; the handle stays
 * usable after ewf_reset).  -1 restores normal operation. */
int ewf_wave_hold(ewf_handle *h, int32_t item);

/* Writes 0_infos.inf and 0_0_{Src,Rec,Rec_x,Rec_y,Rec_y2,Vx,Vy,Vz}.res into workdir
 * (OK4:521-532).  Rec* are the first four receivers. */
int ewf_write_legacy_outputs(ewf_handle *h);
/* Writes "<isave>_0_<name>.res" snapshots of Vx, Vy, Vz (the nsave stub of the 16 km scenario). */
int ewf_write_snapshot(ewf_handle *h, int32_t isave);
/* The same snapshot without stalling the time loop (the reference's nsave stub, 16kmst.cu:
 * 478-484, made to work): Vx, Vy, Vz are copied on the device in the solver's stream order (later
 * steps cannot overwrite them), brought to pinned host memory on a second stream while the next
 * steps run, and written to <isave>_0_V?.res by a library thread.  Two snapshots may be in
 * flight; a third call waits for the oldest to be written.  ewf_snapshot_wait blocks until every
 * queued snapshot is on disk and returns the first write error (0 if none); ewf_destroy waits
 * too. */
int ewf_write_snapshot_async(ewf_handle *h, int32_t isave);
int ewf_snapshot_wait(ewf_handle *h);

/* Layout conversion that allocates nothing (no counterpart in the reference).
 *
 * Some callers cannot call cudaMalloc: a host application whose device memory is already
 * handed out by another framework's pool (a MATLAB gpuArray, a caching allocator that reserved
 * the GPU up front) or that runs under a fixed device-memory budget.  They own the device array
 * and want the solver's layout in it.  This copies a host array in the reference layout
 * (ex x ey x ez, x fastest, float32 or float64) into the caller's device array `dst` in the box
 * layout of the kernels -- element (i,j,k) at dst[i + j*sx + k*sy], converted to
 * dst_dtype_bytes -- the same conversion ewf_set_field does.  Its only scratch is a fixed
 * EWF_NOALLOC_SCRATCH_BYTES array compiled into the library (every GPU that loads the library
 * holds it until exit); arrays larger than that are rejected with EWF_ERR_ARG.  It calls no
 * cudaMalloc/cudaFree.  `stream` is a cudaStream_t (NULL = the default stream); the call
 * returns once the copy is complete.
 *   - dst must be device memory of the current device (or managed memory), aligned to
 *     dst_dtype_bytes, and the extent at the given pitches must end inside dst's allocation;
 *     anything else is rejected with EWF_ERR_ARG before any device work.
 *   - Each call looks up the scratch's device address on the current device (a host-side
 *     query; it stays valid after a device reset).  The first call on a device also loads the
 *     library's device code there: make that first call before any stream capture.
 *   - All calls share the one scratch array: calls that overlap on the GPU (from several host
 *     threads or streams) race.  Only dst's cells inside the extent are written.
 */
#define EWF_NOALLOC_SCRATCH_BYTES (16u << 20)
int ewf_pack_field_noalloc(void *dst, int32_t dst_dtype_bytes, int32_t sx, int64_t sy, const void *host,
                           int32_t host_dtype_bytes, int32_t ex, int32_t ey, int32_t ez, void *stream);

/* Seismogram post-processing: a cascade of second-order IIR sections applied in place to `ntr`
 * traces of `n` samples each (trace-major), FP64 -- the isotropic MATLAB driver's 4th-order
 * Butterworth band-pass, `sos = zp2sos(butter(4, [flo fhi], 'bandpass')); y = sosfilt(sos, x)`
 * (src/FastWaveED_GPU3D_v1_DC_Earthquake_FULL_OK4_final/vizme_FastBiotED_GPU3D_OK_2024_final.m
 * :551-558, 579-582, 604-607).  sos: nsec rows of (b0 b1 b2 a0 a1 a2) as MATLAB and scipy lay
 * them out; each section is the direct form II transposed recursion from zero state.
 * ewf_sosfilt works on host arrays; ewf_sosfilt_device on device arrays (one thread per trace,
 * on `stream`), with the same bits. */
#define EWF_SOS_MAX_SECTIONS 16
int ewf_sosfilt(const double *sos, int32_t nsec, double *x, int64_t ntr, int64_t n);
int ewf_sosfilt_device(const double *sos, int32_t nsec, double *x, int64_t ntr, int64_t n, void *stream);

/* Checkpoint / resume: state fields, compensation, traces and step counter. */
int ewf_checkpoint(ewf_handle *h, const char *path);
int ewf_restore(ewf_handle *h, const char *path);

/* ---------------------------------------------------------------------------------------------
 * Batched solver (no counterpart in the reference, which runs one model and one source per
 * process): n problems -- models of any size and family -- each with n_rhs[i] right-hand sides
 * (independent source sets sharing the problem's model, e.g. the 6 elementary moment tensors of
 * a moment-tensor inversion), advanced together.  Per time step one persistent launch per model
 * family for each of the stress and velocity phases (materials read once per cell for all the
 * problem's RHS), one injection and one receiver launch, replayed from a CUDA graph.  FP32;
 * every problem runs the same nt; state starts at zero.
 * ------------------------------------------------------------------------------------------- */
typedef struct ewf_batch ewf_batch;
int ewf_batch_create(int32_t n, const ewf_params *p, const int32_t *n_rhs, ewf_batch **out);
void ewf_batch_destroy(ewf_batch *b);
/* materials and damping of problem `prob` (shared by its RHS); reference layout as ewf_set_field */
int ewf_batch_set_field(ewf_batch *b, int32_t prob, int32_t field, const void *host, size_t n, int32_t dtype_bytes);
int ewf_batch_set_stf(ewf_batch *b, int32_t prob, const double *stf, size_t n);
int ewf_batch_set_sources(ewf_batch *b, int32_t prob, int32_t rhs, int32_t n, const int32_t *comp_ijk, const double *coef);
int ewf_batch_set_moment_tensor(ewf_batch *b, int32_t prob, int32_t rhs, const double mt[6], int32_t xs, int32_t ys,
                                int32_t zs, int32_t stencil);
/* receivers of problem `prob`, recorded for every RHS */
int ewf_batch_set_receivers(ewf_batch *b, int32_t prob, int32_t n, const int32_t *ijk_comp);
int ewf_batch_reset(ewf_batch *b);
int ewf_batch_run(ewf_batch *b, int32_t nsteps);
int ewf_batch_last_run_ms(const ewf_batch *b, double *ms);
/* traces of (prob, rhs): out[r*nt + it] for the problem's n_rec receivers */
int ewf_batch_get_seismograms(ewf_batch *b, int32_t prob, int32_t rhs, double *out, size_t n);
int ewf_batch_get_field(ewf_batch *b, int32_t prob, int32_t rhs, int32_t field, void *host, size_t n, int32_t dtype_bytes);
/* the autotuner over the whole batch: launch form, z-chunk and CTA tile height, then the
 * multi-RHS velocity kernel's L2 prefetch distance (leaves the batch reset) */
int ewf_batch_autotune(ewf_batch *b, int32_t nsteps, int32_t *kchunk);
/* CTA tile height of every launch of the batch, in rows of 32 columns: 4, 8 (default) or 16;
 * results do not depend on it */
int ewf_batch_set_tile(ewf_batch *b, int32_t tile_y);
int ewf_batch_get_tile(const ewf_batch *b, int32_t *tile_y);
/* Problems with several RHS: their velocity kernel asks L2 for the state lines `planes` planes
 * ahead (0..8; 0 = off, the default; ewf_batch_autotune picks it).  A hint: results do not
 * depend on it. */
int ewf_batch_set_l2_prefetch(ewf_batch *b, int32_t planes);
/* Launch form of the single-RHS problems: 0 (default) -- those of one model family share one
 * persistent launch per phase; 1 -- every problem gets launches of its own, spread over four
 * parallel branches (streams of the captured graph) balanced by cell-updates.  Problems with
 * several RHS always have their own launches.  Results do not depend on it. */
int ewf_batch_set_launch(ewf_batch *b, int32_t own);
int ewf_batch_get_launch(const ewf_batch *b, int32_t *own);
int ewf_batch_get_l2_prefetch(const ewf_batch *b, int32_t *planes);

/* ---------------------------------------------------------------------------------------------
 * Kernels of the learned Green's-function surrogate (no counterpart in the reference).  All
 * buffers are caller-owned device memory; bf16 = __nv_bfloat16 stored as 16-bit words; `stream`
 * is a cudaStream_t (NULL = default).  Calls are asynchronous on the stream.
 * ------------------------------------------------------------------------------------------- */
/* C[M,N] = A[M,K] . B[N,K]^T (+ bias[N]); A, B bf16 row-major, 16-byte aligned; tcgen05 tensor
 * cores fed by TMA, fp32 accumulation in tensor memory.  Optional outputs: Cf fp32, Cb bf16,
 * pre (fp32 value before the activation), 16 / 4 / 16-byte aligned; act 0 = none, 1 = GELU (erf
 * form).  M, N multiples of 128, K a multiple of 32. */
int ewf_mlp_gemm(const void *A, const void *B, const float *bias, float *Cf, void *Cb, float *pre, int32_t M, int32_t N,
                 int32_t K, int32_t act, void *stream);
/* Synchronises and reports (then clears) a failed bounded wait of ewf_mlp_gemm. */
int ewf_mlp_status(void);
/* Test hook of the failure path: with tile >= 0, the MMA issuer of the first CTA of every later
 * ewf_mlp_gemm launch withholds the accumulator-ready signal of its tile number `tile` (a signal
 * nothing else gives), and every mbarrier wait gives up after `polls` polls; the epilogue's wait
 * on that tile runs out, the launch still ends and ewf_mlp_status reports it.  tile < 0 restores
 * normal operation (default limit 2^22 polls). */
int ewf_mlp_test_hold(int32_t tile, int32_t polls);
/* bf16 [rows, cols] -> [cols, rows] */
int ewf_mlp_transpose(const void *in, void *out, int32_t rows, int32_t cols, void *stream);
/* dx = dy * GELU'(pre), bf16 out */
int ewf_mlp_gelu_grad(const void *dy, const float *pre, void *dx, size_t n, void *stream);
/* db[n] = sum over m of dy[m, n] */
int ewf_mlp_bias_grad(const void *dy, float *db, int32_t M, int32_t N, void *stream);
/* dy = 2 (y - t) * scale (bf16); part[b] = sum of (y - t)^2 over block b's elements, b < nblocks */
int ewf_mlp_mse_grad(const float *y, const float *t, void *dy, size_t n, float scale, float *part, int32_t nblocks,
                     void *stream);
/* one Adam step (bias-corrected, step >= 1, decoupled weight decay folded into the gradient) on
 * fp32 master weights w with moments m, v; refreshes the bf16 copy wb when not NULL */
int ewf_mlp_adam(float *w, float *m, float *v, const float *g, void *wb, size_t n, float lr, float b1, float b2, float eps,
                 int32_t step, float weight_decay, void *stream);
/* out[m, o, t] = sum_f R[m, o, f] * G[m, f, t] for M samples (fp32): mixes the predicted
 * fundamental traces of each sample into its moment-tensor x component traces with the sample's
 * azimuth-dependent matrix R.  M <= 65535, nout * nin <= 2048. */
int ewf_mlp_combine(const float *R, const float *G, float *out, int32_t M, int32_t nout, int32_t nin, int32_t T,
                    void *stream);

#ifdef __cplusplus
}
#endif

#endif /* EWFD_H */
