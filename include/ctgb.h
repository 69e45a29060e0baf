/*
 * ctgb.h -- C ABI of the GB300 (sm_103a) fan-beam / cone-beam CT operators.
 *
 * This is the drop-in boundary for the four TensorFlow-1 custom ops of
 * FanBeamCTRecon_TensorflowOp:
 *
 *   FPFanCurve      (FP/transform.cc:17-37, kernel FP/transform.cu:64-146)
 *   BPFanCurve      (BP/transform.cc:17-36, kernel BP/transform.cu:67-95)
 *   FBPFanCurve     (FBP/transform.cc:17-36, kernel FBP/transform.cu:61-89,
 *                    host ramp filter FBP/transform.cu:147-178)
 *   BackProjection  (FDK/FBP.cc:16-35, kernel FDK/GPURecon_GPU.cu:15-50,
 *                    host ramp filter FDK/GPURecon_GPU.cu:184-217)
 *
 * Conventions shared by every entry point:
 *   - All array pointers prefixed d_ are DEVICE pointers; the caller owns them.
 *   - Images are float32 [batch][ny][nx] (x fastest), as the reference's
 *     cudaArray copies read them (FP/transform.cu:222,231; BP/transform.cu:87).
 *   - Sinograms are float32 [batch][n_views][n_cols] (FP/transform.cu:250).
 *   - Every operator OVERWRITES its output (the reference FDK op accumulated
 *     into an unzeroed buffer, FDK/GPURecon_GPU.cu:237-238; this one does not).
 *   - Work is enqueued on `stream` (a cudaStream_t; NULL = legacy default
 *     stream).  Calls return after enqueueing; no device-wide synchronisation.
 *   - Plans are immutable after creation and may be used concurrently from
 *     several host threads and streams (the reference kept geometry in
 *     module-global __constant__ memory, FP/transform.cu:15-62, so two
 *     differently-configured instances clobbered each other).
 *   - Errors are returned as ct_status; the library never exits the process
 *     (the reference's checkCudaErrors called exit()).
 */
#ifndef CTGB_H_
#define CTGB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A cudaStream_t, declared without including the CUDA headers. */
typedef struct CUstream_st *ct_stream;

typedef enum ct_status {
    CT_OK = 0,
    CT_ERR_INVALID_ARGUMENT = 1, /* bad geometry, sizes or enum values */
    CT_ERR_NULL_POINTER = 2,     /* a required pointer was NULL */
    CT_ERR_WORKSPACE = 3,        /* workspace given but smaller than required */
    CT_ERR_CUDA = 4,             /* a CUDA runtime call or launch failed */
    CT_ERR_ALLOC = 5,            /* device or host allocation failed */
    CT_ERR_UNSUPPORTED = 6,      /* valid request this build cannot run */
    CT_ERR_TIMEOUT = 7,          /* a bounded device-side wait gave up */
    CT_ERR_DEVICE_CHECK = 8      /* debug builds: a kernel's index check failed */
} ct_status;

/* Fan-beam geometry decoded from the reference's 16-float `parameter`
 * attribute.  Field meanings and the float arithmetic of the derived fields
 * follow the op constructors exactly: FP/transform.cc:59-76,
 * BP/transform.cc:55-72, FBP/transform.cc:55-72, FDK/FBP.cc:61-84.
 * (PI there is the float literal 3.14159265359f, GPURecon_GPU.h:3.) */
typedef struct ct_fan_geom {
    /* raw attribute values */
    float sdd;           /* parameter[0]  source-detector distance D (mm)     */
    float sid;           /* parameter[1]  source-isocentre distance R (mm)    */
    int32_t n_views;     /* int(parameter[2])                                  */
    float full_angle;    /* parameter[3]  angular range (degrees)             */
    int32_t n_cols;      /* int(parameter[4]) detector channels                */
    int32_t nx;          /* int(parameter[5])                                  */
    int32_t ny;          /* int(parameter[6])                                  */
    float rfov;          /* parameter[7]  reconstruction FOV radius (mm)      */
    float shift;         /* parameter[9]  detector shift (channels; BP/FBP/FDK only) */
    int32_t n_slices;    /* int(parameter[11]) slices per call in the ref op   */
    float det_bottom;    /* parameter[13] FDK op only                          */
    float drow;          /* parameter[14] FDK op only                          */
    float dz;            /* parameter[15] FDK op only                          */
    /* derived, in float, exactly as the reference constructors compute them */
    float d_angle;       /* full_angle / n_views * PI / 180 (rad)              */
    float dx, dy;        /* 2 * rfov / nx, 2 * rfov / ny (mm)                  */
    float xmin, ymin;    /* -0.5 * nx * dx, -0.5 * ny * dy (mm)                */
    float dcol;          /* parameter[8]  * PI / 180 (rad per channel)         */
    float left;          /* parameter[10] * PI / 180 (rad, detector left edge) */
    float start_angle;   /* parameter[12] * PI / 180 (decoded, unused by all ops) */
} ct_fan_geom;

/* Ramp-filter window of the FBP / FDK filter. */
typedef enum ct_filter_window {
    /* The reference kernel: Hsieh's h'' equiangular Ram-Lak form, 0.5 factor
     * for 360-degree redundancy, scaled by R*d_angle*dcol
     * (FBP/transform.cu:149-162, FDK/GPURecon_GPU.cu:184-200). */
    CT_WINDOW_RAMLAK = 0,
    /* Shepp-Logan: the parallel-beam Shepp-Logan taps 2/(pi^2 tau^2 (1-4n^2))
     * with tau = dcol, mapped to the equiangular fan by (n dcol / sin(n dcol))^2,
     * same 0.5 factor and R*d_angle*dcol scale.  config.py:42 names it
     * (FilterType=1 "S-L") but no reference op reads it. */
    CT_WINDOW_SHEPP_LOGAN = 1
} ct_filter_window;

/* How the row filter executes on the device. */
typedef enum ct_filter_algo {
    CT_FILTER_AUTO = 0,      /* the library picks (measured fastest accurate path) */
    CT_FILTER_DIRECT = 1,    /* FP32 direct convolution (Ram-Lak: odd taps only) */
    /* Toeplitz GEMM on the tcgen05 tensor cores: TF32 three-term split
     * (x_hi*h_hi + x_hi*h_lo + x_lo*h_hi), FP32 accumulation in tensor
     * memory; needs n_cols % 4 == 0 and n_cols <= 4032. */
    CT_FILTER_TOEPLITZ_TC = 2
} ct_filter_algo;

typedef struct ct_plan_opts {
    int32_t filter_window;  /* ct_filter_window */
    int32_t filter_algo;    /* ct_filter_algo   */
    /* 1: short-scan data; FBP, FDK and their adjoints weight every ray with
     * Parker's weights (Parker 1982), doubled to undo the filter's 0.5
     * full-scan redundancy factor.  config.py:24 names ParkWeighting but no
     * reference op reads it.  0: full scan (the reference). */
    int32_t short_scan;
    /* 1: Feldkamp cosine pre-weighting (Feldkamp, Davis & Kress 1984): FBP,
     * FDK and their adjoints weight channel i, row r by cos(gamma_i) (fan
     * plans) or cos(gamma_i) * sdd / sqrt(sdd^2 + h_r^2) (cone plans), with
     * gamma_i = left + (i + 1/2 - shift) dcol and h_r the row height.  The
     * reference has none (FBP/transform.cu:61-89 weights by 1/L^2 only).
     * 0: no pre-weighting (the reference). */
    int32_t cosine_weight;
    /* 1: backprojectors interpolate with the GPU texture unit's weights, as
     * the reference's tex1D/tex2D did (BP/transform.cu:90,
     * FBP/transform.cu:85, FDK/GPURecon_GPU.cu:45): each fraction rounded to
     * 1/256, ties up, and in 2-D the far-corner weight rounded to 1/256 with
     * the other three completing exact row and column sums.  Applies to BP,
     * FBP, the FDK ops and their adjoints (which stay exact transposes).
     * The forward projectors keep exact weights: their cell sums have no
     * per-sample weight to round.  ct_batch_run and the ct_plain_* loop
     * reject such plans (CT_ERR_UNSUPPORTED).
     * 0: exact FP32 weights (default). */
    int32_t texture_weights;
    int32_t reserved[3];    /* must be zero      */
} ct_plan_opts;

/* Operators, for ct_workspace_size. */
typedef enum ct_op {
    CT_OP_FP = 0,
    CT_OP_FP_ADJOINT = 1,
    CT_OP_BP = 2,
    CT_OP_FBP = 3,
    CT_OP_FBP_ADJOINT = 4,
    CT_OP_FDK_BP = 5,
    CT_OP_BP_ADJOINT = 6,
    CT_OP_FP_CONE = 7,
    CT_OP_FDK_CONE = 8,
    CT_OP_FDK_CONE_ADJOINT = 9
} ct_op;

typedef struct ct_plan ct_plan;

/* ---- status / build info ------------------------------------------------ */

const char *ct_status_string(ct_status status);
const char *ct_version(void);
/* Last CUDA error text seen by this thread ("" if none). */
const char *ct_last_error(void);
/* Number of kernels this library has launched in this process. */
uint64_t ct_launch_count(void);

/* Build flags: CT_BUILD_INDEX_CHECKS is set in debug builds (compiled with
 * -DCT_DEBUG), whose kernels test every gather index against the array it
 * reads, skip an access outside it (reading zero) and record where; the next
 * ct_plan_check then returns CT_ERR_DEVICE_CHECK (ct_last_error names the
 * source line).  Release builds carry no checks and return 0.  No counterpart
 * in the reference (its kernels checked no index; checkCudaErrors exited the
 * process on any CUDA error, FP/transform.cu:4). */
#define CT_BUILD_INDEX_CHECKS 1u
uint32_t ct_build_flags(void);

/* ---- device memory ----------------------------------------------------------- */

/* A caller-supplied device allocator.  The library takes device memory in
 * exactly two places: the tables of a plan (ct_plan_create*, given back by
 * ct_plan_destroy) and the scratch of an operator called with d_work == NULL
 * (given back after the call's last kernel is enqueued).  The reference
 * instead malloc'ed and freed its buffers inside every call and exited the
 * process when one failed (FP/transform.cu:198-217, checkCudaErrors).
 *   alloc(ctx, bytes, stream): device memory for work that will be enqueued
 *     on `stream` (NULL for plan tables), 256-byte aligned as cudaMalloc's
 *     (kernels read plan tables with 32-byte loads); NULL on failure, which
 *     the call reports as CT_ERR_ALLOC after releasing what it already took.
 *     A block that is not 256-byte aligned is given back and reported the
 *     same way.
 *   free(ctx, ptr, stream): ptr is no longer needed once the work already
 *     enqueued on `stream` has run (stream-ordered, as cudaFreeAsync); for
 *     plan tables stream is NULL and the plan's work must have finished. */
typedef struct ct_allocator {
    void *ctx;
    void *(*alloc)(void *ctx, size_t bytes, ct_stream stream);
    void (*free)(void *ctx, void *ptr, ct_stream stream);
} ct_allocator;

/* Installs `allocator` for all later allocations of this process (a copy is
 * kept; plans remember the allocator they were created with and give their
 * tables back to it).  NULL restores the CUDA runtime (cudaMalloc for plan
 * tables, cudaMallocAsync / cudaFreeAsync for scratch).  alloc and free must
 * both be set.  Not synchronised with calls in flight on other threads: set
 * it at start-up.  No counterpart in the reference. */
ct_status ct_set_allocator(const ct_allocator *allocator);

/* Number of device allocations this library has made in this process, by
 * either route (ct_set_allocator's or the CUDA runtime's). */
uint64_t ct_device_alloc_count(void);

/* Whether host_ptr lies in page-locked host memory mapped into the current
 * device's address space; if so *device_ptr receives the address kernels use
 * for it (the same value under unified addressing).  An operator may then
 * write its output there directly: ct_fp_fan stores every output element
 * exactly once, so its sinogram crosses to the host while it runs and no
 * device-to-host copy follows.  CT_ERR_INVALID_ARGUMENT for pageable or
 * unmapped memory.  No counterpart in the reference (its ops returned TF
 * tensors). */
ct_status ct_host_mapped(const void *host_ptr, void **device_ptr);

/* ---- geometry ------------------------------------------------------------ */

/* Decodes the 16-float parameter vector.  Replaces the attr decoding of
 * FPFanCurveOp / BPFanCurveOp / FBPFanCurveOp / BackProjectionOp
 * (FP/transform.cc:59-76, BP/transform.cc:55-72, FBP/transform.cc:55-72,
 * FDK/FBP.cc:61-84).  Host-only; needs no GPU. */
ct_status ct_geom_from_param16(const float param[16], ct_fan_geom *out);

/* The forward projector's per-ray table, evaluated on the host in FP64 exactly
 * as plans build it: for ray (v, i), v-major, ray4[4r..4r+3] = start x, start y,
 * step x, step y in texture pixel coordinates and nsamp[r] = floor(chord/0.125)
 * (0 for rays missing the FOV).  Restates
 * GenerateRayTraceMap_FB_ReconImage_OneView_kernel (FP/transform.cu:64-101).
 * ray4 holds 4*n_views*n_cols floats, nsamp n_views*n_cols.  Needs no GPU. */
ct_status ct_fp_ray_table(const ct_fan_geom *geom, const float *angles, int n_angles,
                          float *ray4, int32_t *nsamp);

/* ---- plans ----------------------------------------------------------------- */

/* Builds the per-view (FP64-derived) geometry tables on the current device.
 * `angles` is the host float32 array of n_angles view angles in radians (the
 * `angle` attr, utils.py:49-54); n_angles must equal geom->n_views.
 * Replaces para_setup_fan_curve (FP/transform.cu:20-62, BP/transform.cu:20-64,
 * FBP/transform.cu:23-58) and the constructors' angle copy
 * (FP/transform.cc:81-90).  opts may be NULL. */
ct_status ct_plan_create(const ct_fan_geom *geom, const float *angles, int n_angles,
                         const ct_plan_opts *opts, ct_plan **out);
ct_status ct_plan_destroy(ct_plan *plan);
/* Waits for the device and reports CT_ERR_TIMEOUT (and clears the flag) if
 * a kernel of this plan hit the iteration limit of one of its bounded waits
 * since the last check (only the tensor-core filter waits on barriers).  In
 * debug builds (ct_build_flags) it then reports CT_ERR_DEVICE_CHECK (and
 * clears the flags) if any kernel of the library failed an index check since
 * the last call; those flags are per device, not per plan. */
ct_status ct_plan_check(const ct_plan *plan);
/* Failure-path self-test: enqueues one thread that waits, with the filter's
 * bounded-wait code, on a barrier nothing completes, gives up after budget_us
 * microseconds (1 .. 1,000,000) and raises the plan's error flag, so that the
 * next ct_plan_check returns CT_ERR_TIMEOUT.  The context stays usable. */
ct_status ct_plan_selftest_wait_timeout(const ct_plan *plan, int32_t budget_us,
                                        ct_stream stream);
/* The geometry a plan was built from. */
ct_status ct_plan_geom(const ct_plan *plan, ct_fan_geom *out);

/* Device scratch bytes an operator needs for `batch` slices.  Operators that
 * take d_work accept d_work == NULL, in which case they allocate the scratch
 * stream-ordered (cudaMallocAsync/cudaFreeAsync) on `stream`.  A given d_work
 * must be 16-byte aligned (CT_ERR_WORKSPACE otherwise). */
ct_status ct_workspace_size(const ct_plan *plan, ct_op op, int batch, size_t *bytes);

/* ---- fan-beam operators ---------------------------------------------------- */

/* Ray-driven forward projection, d_img [batch][ny][nx] -> d_sino
 * [batch][n_views][n_cols].  Per ray: the FOV-chord sample rule
 * floor(chord/0.125 px), a left Riemann sum of bilinear, clamp-to-edge image
 * samples, times 0.125*dx; rays missing the FOV give 0.  Bilinear weights are
 * full FP32 (the reference used 8-bit texture weights).
 * Replaces project_fan_curve (FP/transform.cu:173-269) with its kernels
 * GenerateRayTraceMap_FB_ReconImage_OneView_kernel (:64-101) and
 * RayTrace_ReconImage_OneView_kernel (:103-146). */
ct_status ct_fp_fan(const ct_plan *plan, const float *d_img, float *d_sino, int batch,
                    void *d_work, size_t work_bytes, ct_stream stream);

/* Exact adjoint (transpose) of ct_fp_fan: d_sino [batch][n_views][n_cols] ->
 * d_img [batch][ny][nx].  No counterpart in the reference (it registers no
 * gradient, utils.py:5). */
ct_status ct_fp_fan_adjoint(const ct_plan *plan, const float *d_sino, float *d_img, int batch,
                            void *d_work, size_t work_bytes, ct_stream stream);

/* Unweighted pixel-driven backprojection: for every pixel inside the FOV disc
 * and every view, adds the linearly interpolated (clamped) detector value at
 * col = (atan(t/U) - left)/dcol + shift when 0 < col < n_cols.
 * Replaces backproject_fan_curve (BP/transform.cu:123-176) and
 * BackProjOneView_fan_curve_kernel (BP/transform.cu:67-95). */
ct_status ct_bp_fan(const ct_plan *plan, const float *d_sino, float *d_img, int batch,
                    ct_stream stream);

/* Exact adjoint of ct_bp_fan: d_img [batch][ny][nx] -> d_sino
 * [batch][n_views][n_cols].  No counterpart in the reference. */
ct_status ct_bp_fan_adjoint(const ct_plan *plan, const float *d_img, float *d_sino, int batch,
                            ct_stream stream);

/* Row ramp filter only: each detector row of d_sino is convolved with the
 * plan's window (middle n_cols samples of the full linear convolution).
 * d_out may not alias d_sino.  Replaces the host ippsConv_32f loop
 * (FBP/transform.cu:147-174).  The filter is symmetric, so it is its own
 * adjoint. */
ct_status ct_ramp_filter(const ct_plan *plan, const float *d_sino, float *d_out, int rows,
                         ct_stream stream);

/* Filtered backprojection: ramp filter, then BP weighted by 1/(U^2+t^2).
 * Replaces backproject_fan_curve of FBP/transform.cu:117-201 (kernel :61-89). */
ct_status ct_fbp_fan(const ct_plan *plan, const float *d_sino, float *d_img, int batch,
                     void *d_work, size_t work_bytes, ct_stream stream);

/* Exact adjoint of ct_fbp_fan: d_img [batch][ny][nx] -> d_sino
 * [batch][n_views][n_cols] (weighted-BP transpose, then the filter).
 * No counterpart in the reference. */
ct_status ct_fbp_fan_adjoint(const ct_plan *plan, const float *d_img, float *d_sino, int batch,
                             void *d_work, size_t work_bytes, ct_stream stream);

/* The reference "BackProjection" op of FDK/FBP.cc (nZ = 1, nRows = 1,
 * FDK/FBP.cc:85,98): ramp filter, then the CB_EA backprojection kernel with
 * 1/L^2 weight and detector shift (FDK/GPURecon_GPU.cu:15-50,163-268).  With
 * one detector row its result equals ct_fbp_fan; unlike the reference, every
 * one of the `batch` slices is processed (the reference copied only the first,
 * FDK/GPURecon_GPU.cu:178-179) and the output is zeroed first. */
ct_status ct_fdk_bp(const ct_plan *plan, const float *d_sino, float *d_img, int batch,
                    void *d_work, size_t work_bytes, ct_stream stream);

/* ---- cone beam ------------------------------------------------------------- */
/* Volumes are float32 [batch][nz][ny][nx], voxel centres z = zmin + dz(k+1/2)
 * with zmin = -dz*nz/2 (FDK/FBP.cc:86); projections are float32
 * [batch][n_views][n_rows][n_cols] (the view layout of the reference's FDK
 * filter, FDK/GPURecon_GPU.cu:211).  Detector row r is at height
 * det_bottom + (r+1/2)*drow; the source orbits at z = 0.  geom->det_bottom,
 * drow and dz are parameter[13..15] of the FDK op (FDK/FBP.cc:82-84). */

/* A plan for nz slices and n_rows detector rows (the reference's FDK op fixes
 * both to 1, FDK/FBP.cc:85,98; ct_plan_create makes such a plan).  Requires
 * drow > 0, dz > 0 and sdd > sid. */
ct_status ct_plan_create_cone(const ct_fan_geom *geom, int n_rows, int nz, const float *angles,
                              int n_angles, const ct_plan_opts *opts, ct_plan **out);

/* ct_plan_create_cone with the source at height source_z[v] (mm) in view v:
 * a z-offset circular orbit (all equal) or a helix (source_z[v] = z0 +
 * pitch * (angle[v] - angle[0]) / (2 pi)).  The reference's view record has
 * these fields (ViewInfo.fSourceZ / fDeltaZ, FDK/GPURecon_GPU.h:27-33) but
 * always passes 0 (FDK/GPURecon_GPU.cu:226).  Every cone operator then uses
 * row = ((z - source_z[v]) * D / U - det_bottom) / drow and rays from the
 * source at that height.  source_z == NULL is ct_plan_create_cone. */
ct_status ct_plan_create_cone_ex(const ct_fan_geom *geom, int n_rows, int nz,
                                 const float *angles, const float *source_z, int n_angles,
                                 const ct_plan_opts *opts, ct_plan **out);

/* The reference's CB_EA backprojection (FDK/GPURecon_GPU.cu:15-50) over all
 * views, unfiltered: per voxel in the FOV disc and view, the bilinear
 * (col, row) sample of the view with col as in ct_bp_fan and
 * row = (z*D/U - det_bottom)/drow (clamped rows), times 1/(U^2+t^2).
 * Needs no scratch: it gathers the four taps of each sample from d_proj
 * (ct_fdk_cone reads them from per-view tap images in its workspace). */
ct_status ct_cone_bp(const ct_plan *plan, const float *d_proj, float *d_vol, int batch,
                     ct_stream stream);

/* FDK: ramp filter of every (view, row), then ct_cone_bp.  Replaces
 * BP_One_Rot_3D_GPU (FDK/GPURecon_GPU.cu:163-268) for nz, n_rows >= 1. */
ct_status ct_fdk_cone(const ct_plan *plan, const float *d_proj, float *d_vol, int batch,
                      void *d_work, size_t work_bytes, ct_stream stream);

/* Exact adjoint of ct_fdk_cone (CB_EA transpose, then the symmetric filter):
 * d_vol -> d_proj.  No counterpart in the reference. */
ct_status ct_fdk_cone_adjoint(const ct_plan *plan, const float *d_vol, float *d_proj, int batch,
                              void *d_work, size_t work_bytes, ct_stream stream);

/* Cone-beam forward projection, d_vol -> d_proj.  No counterpart in the
 * reference (only its unused 3-D textures, FDK/GPURecon_GPU.cu:10,12, remain).
 * The ray from the source to detector cell (view, row r, channel i) is
 * sampled at the fan-beam projector's in-plane positions; at in-plane
 * distance s from the source its height is h_r*s/D.  Samples are trilinear
 * and clamp-to-edge; the sum is weighted by 0.125*dx*sqrt(1 + (h_r/D)^2). */
ct_status ct_fp_cone(const ct_plan *plan, const float *d_vol, float *d_proj, int batch,
                     void *d_work, size_t work_bytes, ct_stream stream);

/* ---- uneven batches ---------------------------------------------------------- */

/* Element type of an operator's input and output storage; arithmetic is FP32. */
typedef enum ct_dtype {
    CT_DTYPE_F32 = 0,
    CT_DTYPE_BF16 = 1 /* bfloat16 storage, FP32 accumulation */
} ct_dtype;

#define CT_BATCH_MAX_ITEMS 64

/* One slice of an uneven batch: a fan-beam plan (any geometry; plans made by
 * ct_plan_create), one of CT_OP_FP, CT_OP_BP, CT_OP_FBP, CT_OP_FBP_ADJOINT,
 * the storage type of d_in and d_out, and device pointers to one input slice
 * (image [ny][nx] or sinogram [n_views][n_cols]) and one output slice. */
typedef struct ct_batch_item {
    const ct_plan *plan;
    int32_t op;
    int32_t dtype;
    const void *d_in;
    void *d_out;
} ct_batch_item;

/* Device scratch bytes ct_batch_run needs for these items. */
ct_status ct_batch_workspace_size(const ct_batch_item *items, int n, size_t *bytes);

/* Runs up to CT_BATCH_MAX_ITEMS slices of different geometries and
 * operators: one launch builds every FP item's quad images, one persistent
 * launch projects all FP items, the FBP / FBP-adjoint items are filtered with
 * their plans' filters, and one persistent launch backprojects all BP / FBP
 * items.  Two or more items with the same plan (the same ct_plan handle),
 * operator and dtype form a slice group: they are gathered into the
 * workspace and run through the plan's multi-slice kernels (as ct_fp_fan,
 * ct_bp_fan, ct_fbp_fan, ct_fbp_fan_adjoint on the group), so give slices of
 * one geometry one plan.  Item descriptors are passed as kernel parameters, so the call makes
 * no host-to-device copy and can be captured in a CUDA graph (pass d_work; the
 * first call of a process should come before capture).  All plans must be on
 * one device.  d_work == NULL allocates stream-ordered, as the operators do.
 * No counterpart in the reference (one op instance per geometry, one slice
 * loop per call). */
ct_status ct_batch_run(const ct_batch_item *items, int n, void *d_work, size_t work_bytes,
                       ct_stream stream);

/* Launch shapes of ct_batch_run's two persistent launches.  The library
 * keeps one configuration per batch shape (the ops, storage types and sizes
 * of the items, in order); ct_batch_run uses it, or the default below for a
 * shape that was never tuned or set. */
typedef struct ct_batch_config {
    int32_t fp_blocks_per_sm; /* FP launch: 256-thread blocks per SM, 1..16 (default 3)  */
    int32_t fp_dynamic;       /* 1: warps take (item, view, 32 channels) units from an
                                 atomic counter, largest item first; 0: fixed stride */
    int32_t bp_blocks_per_sm; /* BP launch: 256-thread blocks per SM, 1..16 (default 4)  */
    int32_t bp_dynamic;       /* as fp_dynamic, for BP tiles                               */
    int32_t bp_tile_rows;     /* BP tile height in pixels: 32 or 16 (tiles are 32 wide)  */
    int32_t reserved[3];      /* zero                                                     */
} ct_batch_config;

/* Project-written autotuner: runs the batch (its outputs are overwritten)
 * with every candidate launch shape, `reps` times each (reps <= 0: 3), timing
 * the FP and BP launches separately with CUDA events, and keeps the fastest
 * FP shape and the fastest BP shape for this batch shape.  Synchronises
 * `stream`; must not run during stream capture.  The chosen configuration is
 * written to *out when out != NULL. */
ct_status ct_batch_tune(const ct_batch_item *items, int n, void *d_work, size_t work_bytes,
                        int32_t reps, ct_stream stream, ct_batch_config *out);

/* The configuration ct_batch_run uses for this batch shape; *tuned = 1 if it
 * was tuned or set, 0 for the default. */
ct_status ct_batch_get_config(const ct_batch_item *items, int n, ct_batch_config *out,
                              int32_t *tuned);

/* Records a configuration for this batch shape (e.g. one saved from an
 * earlier ct_batch_tune); config == NULL forgets it. */
ct_status ct_batch_set_config(const ct_batch_item *items, int n, const ct_batch_config *config);

/* ---- filtered backprojection that allocates nothing ----------------------- */

/* Capacity, in floats, of the fixed device array ct_fbp_fan_static_scratch
 * uses: 8 Mi floats = 32 MiB, i.e. batch * n_views * n_cols <= 8,388,608
 * (nine 984 x 888 sinograms per call). */
#define CT_FBP_STATIC_SCRATCH_FLOATS (8u * 1024u * 1024u)

/* Same result as ct_fbp_fan, for callers that cannot allocate device memory:
 * plugins whose host framework owns all device memory and passes the plugin
 * only its input and output buffers, and real-time pipelines that allow no
 * device allocation after start-up (an allocation can synchronise the device
 * and has no latency bound).  It calls no cudaMalloc, cudaMallocAsync,
 * cudaFree or allocating library routine; the filtered sinogram lives in a
 * fixed array of CT_FBP_STATIC_SCRATCH_FLOATS floats inside this library's
 * device code, which every GPU it has been set up on (below) holds until the
 * process exits.  The caller still passes the input and output buffers.
 *   - batch * n_views * n_cols above the capacity returns CT_ERR_WORKSPACE
 *     (ct_last_error says by how much); split the batch.
 *   - The first call on each device is its set-up: it loads this part of
 *     the library's device code on that device, which reserves the array
 *     (the CUDA runtime loads device code lazily), and looks up and caches
 *     the array's device address with that device current.  That call can
 *     therefore fail with CT_ERR_ALLOC on a full device; make it once at
 *     start-up (a warm-up call, e.g. with a small batch), before any device
 *     memory is handed to the host framework and before capturing any
 *     stream into a CUDA graph.  Later calls reserve nothing.  A
 *     cudaDeviceReset invalidates the cached address: do not call this entry
 *     point after resetting a device.
 *   - All calls on a device share the one array, which keeps the last call's
 *     contents (each call overwrites all it reads, so nothing needs clearing).
 *     Calls whose work overlaps on the GPU -- on different streams, or from
 *     different host threads -- race on it; serialise them.
 * No counterpart in the reference (its FBP malloc'ed and freed host and
 * device buffers on every call). */
ct_status ct_fbp_fan_static_scratch(const ct_plan *plan, const float *d_sino, float *d_img,
                                    int batch, ct_stream stream);

/* ---- the plain per-view launch loop (comparison baseline) ----------------- */

/* The reference's execution structure on the same GPU: for each slice and
 * each view one kernel launch followed by a stream synchronisation
 * (FP/transform.cu:162-169, BP/transform.cu:110-119), with explicit FP32
 * lerp instead of texture references.  Same results as the fused operators;
 * kept only to measure against. */
ct_status ct_plain_fp_fan(const ct_plan *plan, const float *d_img, float *d_sino, int batch,
                          ct_stream stream);
ct_status ct_plain_fp_fan_adjoint(const ct_plan *plan, const float *d_sino, float *d_img,
                                  int batch, ct_stream stream);
ct_status ct_plain_bp_fan(const ct_plan *plan, const float *d_sino, float *d_img, int batch,
                          ct_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* CTGB_H_ */
