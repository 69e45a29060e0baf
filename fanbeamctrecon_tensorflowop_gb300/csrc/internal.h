// Internal declarations shared by the ctgb translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "../../include/ctgb.h"

// Float literal the reference uses for pi in every op (FP/transform.h:1,
// GPURecon_GPU.h:3).  Geometry decoding keeps it so decoded values match.
#define CT_REF_PI 3.14159265359f

// Sample step of the ray-driven projector, in pixels (FP/transform.cu:10).
#define CT_FP_STEP 0.125

// Host-side (FP64-derived) geometry tables; built without CUDA.
struct ct_host_tables {
    // Per view: rotation constants as the reference BP kernels take them,
    // c = -cos(beta), s = -sin(beta) (BP/transform.cu:116).
    std::vector<float> view_cs;      // [2*V]
    // the rounding left by view_cs: (-cos(beta) - c, -sin(beta) - s) (float-float pairs)
    std::vector<float> view_cs_lo;   // [2*V]
    // per column boundary y = b (b = 0..C): tan(left + (b - shift - 1/2) dcol) as hi, lo
    std::vector<float> col_tan;      // [2*(C+1)]
    // Per ray (view-major, [V][C]): start (x, y) and step (x, y) in texture
    // pixel coordinates, and the sample count floor(chord/0.125)
    // (FP/transform.cu:64-101).
    std::vector<float> ray;          // [4*V*C]
    std::vector<int32_t> nsamp;      // [V*C]
    std::vector<float> taps;         // [2C-1] ramp filter taps, index n + C - 1
    // Per channel: in-plane distance (mm) from the source to the ray's first
    // sample, and the FOV chord length (mm) (cone-beam projector heights).
    std::vector<float> chan_s;       // [2*C]
    std::vector<float> parker;       // [V*C] short-scan weights (x2), when requested
    std::vector<float> cosw;         // [n_rows*C] Feldkamp cosine weights, when requested
    std::vector<float> view_z;       // [V] source heights (mm), when given
    int32_t max_nsamp = 0;
    double total_samples = 0;        // sum of nsamp over all rays
};

// Gather-form BP transpose (bp_gather.cu): per view, channel groups of
// kBptOut output channels (32 strips per warp), boundary rays in 32.32 fixed
// point along the image lines the warp walks.
constexpr int kBptOut = 31;
struct ct_bpt_tables {
    int W = 0;                        // channel groups per view
    bool ok = false;                  // false: a ray of some group runs along its lines
    std::vector<int32_t> warp;        // [V][W][4]: layout | orient << 1, first line, last line, 0
    std::vector<int64_t> bnd;         // [V][W][33][2]: crossing of the first line, step per line
    std::vector<float> ray;           // [V][W][32][4]: L at the first line, dL per line, na, da
    std::vector<int32_t> fov_row;     // [ny][2]: pixels of row j inside the FOV (inclusive)
    std::vector<int32_t> fov_col;     // [nx][2]: pixels of column i inside the FOV
};

// geometry.cpp
void ct_build_bpt_tables(const ct_fan_geom *g, const float *angles, ct_bpt_tables *t);
ct_status ct_decode_param16(const float p[16], ct_fan_geom *g);
ct_status ct_validate_geom(const ct_fan_geom *g);
void ct_build_view_table(const ct_fan_geom *g, const float *angles, ct_host_tables *t);
void ct_build_ray_table(const ct_fan_geom *g, const float *angles, ct_host_tables *t);
void ct_build_filter_taps(const ct_fan_geom *g, int window, ct_host_tables *t);
void ct_build_channel_table(const ct_fan_geom *g, ct_host_tables *t);
void ct_build_parker(const ct_fan_geom *g, const float *angles, ct_host_tables *t);
void ct_build_cosine(const ct_fan_geom *g, int n_rows, bool cone, ct_host_tables *t);
// Largest |t/U| = tan(gamma) over the FOV disc: rfov / sqrt(R^2 - rfov^2).
double ct_max_tan_gamma(const ct_fan_geom *g);
// Fits atan(z) = z * sum_k coef[k] (z^2)^k on |z| <= zmax (interpolation at
// Chebyshev nodes in z^2); returns the degree used (4 or 8) or 0 when no
// degree <= 8 reaches 3e-8 absolute error (callers then use atanf).
int ct_fit_atan(double zmax, float coef[9]);

struct ct_plan {
    ct_fan_geom g;
    ct_plan_opts opts;
    ct_allocator alloc;              // allocator of the tables below (ct_set_allocator)
    int device;
    int filter_algo;                 // resolved ct_filter_algo (never AUTO)
    float fp_weight;                 // 0.125*dx (FP/transform.cu:144)
    float fov_r2;                    // rfov^2 (BP/transform.cu:116)
    int n_rows, nz;                  // cone plans; 1 and 1 for fan plans
    float view_z_min, view_z_max;    // range of the source heights (0, 0 without them)
    int atan_deg;                    // 4 or 8: polynomial atan on the FOV; 0: atanf
    float atan_coef[9];
    int gather_atan_deg;             // the same fit on the FOV widened by 1.5 pixels
    float gather_atan_coef[9];
    double total_samples;
    int32_t max_nsamp;
    std::vector<float> h_view_cs;    // host copy of the view table
    // device copies of ct_host_tables (owned)
    float *d_view_cs;                // [2V]
    float *d_view_cs_lo;             // [2V] float-float remainder of d_view_cs
    float *d_col_tan;                // [2(C+1)] tan of the column boundaries (hi, lo)
    float *d_ray;                    // [4VC]
    float *d_ray_rec;                // [8VC] per ray, for the adjoint gather: start (x, y),
                                     // step (x, y), 1/step (1e30 for a zero step), sample
                                     // count (int32 bits), 0 (one 32-byte record)
    int32_t *d_nsamp;                // [VC]
    int32_t *d_fp_order;             // launch order of the forward projector's blocks
                                     // (fp_block_order)
    float *d_taps;                   // [2C-1]
    float *d_chan_s;                 // [2C]
    float *d_tc_hi, *d_tc_lo;        // tensor-core filter: TF32 split of the Toeplitz taps
    int *d_err;                      // raised by kernels whose bounded waits gave up
    float *d_parker;                 // [V*C] short-scan weights, or NULL (full scan)
    float *d_cosw;                   // [n_rows*C] cosine pre-weights, or NULL
    float *d_view_z;                 // [V] source heights (mm), or NULL (orbit at z = 0)
    // gather-form BP transpose (fan plans whose ct_bpt_tables are ok), else NULL
    int bpt_W;
    int32_t *d_bpt_warp;             // [V][W] int4
    int64_t *d_bpt_bnd;              // [V][W][33] longlong2
    float *d_bpt_ray;                // [V][W][32] float4
    int32_t *d_fov_row, *d_fov_col;  // [ny] int2, [nx] int2
};

// Kernel launchers (defined in the .cu files).  Each returns the launch error.
namespace ctk {
// work: fp_fan_work_bytes(p, batch) bytes (quad images of up to 64 slices)
int fp_fan(const ct_plan *p, const float *img, float *sino, int batch, void *work,
           void *stream);
size_t fp_fan_work_bytes(const ct_plan *p, int batch);
// The forward projector's block order (host, at plan creation): its blocks
// (32 channels x 4 adjacent views) sorted by the quad layout most of their
// rays walk, channel-group-major within a layout.
std::vector<int32_t> fp_block_order(int V, int C, const std::vector<float> &ray,
                                    const std::vector<int32_t> &nsamp);
// work: fp_fan_adjoint_work_bytes(p, batch) bytes (corner sums of up to 64 slices)
size_t fp_fan_adjoint_work_bytes(const ct_plan *p, int batch);
int fp_fan_adjoint(const ct_plan *p, const float *sino, float *img, int batch, void *work,
                   void *stream);

// mode 0: unweighted BP, 1: 1/(U^2+t^2)-weighted (FBP / FDK 2-D)
// work: bp_fan_work_bytes(p, batch) bytes (tap images of up to 16 slice groups
// of four; 0 below four slices) or NULL (gathers)
size_t bp_fan_work_bytes(const ct_plan *p, int batch);
int bp_fan(const ct_plan *p, const float *sino, float *img, int batch, int weighted, void *work,
           void *stream);
// work: bp_fan_transpose_work_bytes(p, batch) bytes (slice-quad images of up
// to 64 slices in both layouts) for the gather form; NULL, or a plan without
// its tables or with texture weights, takes the atomic scatter form
size_t bp_fan_transpose_work_bytes(const ct_plan *p, int batch);
// bp_gather.cu: the gather form (plans with the tables, exact weights)
bool bp_gather_usable(const ct_plan *p);
size_t bp_gather_work_bytes(const ct_plan *p, int batch);
int bp_gather(const ct_plan *p, const float *img, float *sino, int batch, int weighted,
              void *work, void *stream);
int bp_fan_transpose(const ct_plan *p, const float *img, float *sino, int batch, int weighted,
                     void *work, void *stream);
int ramp_filter(const ct_plan *p, const float *in, float *out, int rows, void *stream);
size_t ramp_direct_smem(int C);
int tc_padded(int C);
bool ramp_tc_supported(int C);
void build_tc_taps(const float *taps, int C, std::vector<float> &hi, std::vector<float> &lo);
int ramp_filter_tc(const ct_plan *p, const float *in, float *out, int rows, void *stream);
// One bounded wait that nothing completes; raises the plan's error flag.
int wait_selftest(const ct_plan *p, unsigned long long budget_ns, void *stream);
// Whether FBP / FDK weight the projections before filtering (short scan or
// cosine pre-weighting).
inline bool has_preweight(const ct_plan *p) { return p->d_parker || p->d_cosw; }
// out = in * parker[v][c] * cosw[r][c] (each factor when present), over
// [batch][V][n_rows][C]
int apply_preweight(const ct_plan *p, const float *in, float *out, int batch, void *stream);
// work: cone_bp_work_bytes(p) bytes (one volume's quad images of the views;
// 0 where they would not fit in 4 GB) or NULL (four gathers per sample)
size_t cone_bp_work_bytes(const ct_plan *p);
int cone_bp(const ct_plan *p, const float *proj, float *vol, int batch, void *work,
            void *stream);
// work: cone_bp_transpose_work_bytes(p, batch) bytes (per-volume max |vol|;
// where every detector row of a view fits in shared memory, also pixel tables
// and a z-major copy of the volumes)
size_t cone_bp_transpose_work_bytes(const ct_plan *p, int batch);
bool cone_bp_transpose_supported(const ct_plan *p);  // its detector rows fit in shared memory
int cone_bp_transpose(const ct_plan *p, const float *vol, float *proj, int batch, void *work,
                      void *stream);
int cone_fp(const ct_plan *p, const float *vol, float *proj, int batch, void *work, void *stream);
size_t cone_fp_work_bytes(const ct_plan *p, int batch);
ct_status batch_workspace(const ct_batch_item *items, int n, size_t *bytes);
// Enqueues the batch with launch shape `cfg`; when `ev` (four cudaEvent_t)
// is not NULL, records ev[0], ev[1] around the persistent FP launch and
// ev[2], ev[3] around the persistent BP launch.
int batch_run(const ct_batch_item *items, int n, void *work, void *stream,
              const ct_batch_config &cfg, void **ev);
ct_batch_config batch_default_config();
ct_status batch_check_config(const ct_batch_config &c);
// The configuration kept for this batch shape (default when none); *tuned
// tells which.
ct_batch_config batch_lookup(const ct_batch_item *items, int n, bool *tuned);
void batch_store(const ct_batch_item *items, int n, const ct_batch_config *c);
// Times the candidate launch shapes (see ct_batch_tune); returns a CUDA error.
int batch_tune(const ct_batch_item *items, int n, void *work, void *stream, int reps,
               ct_batch_config *best);
int plain_fp_fan(const ct_plan *p, const float *img, float *sino, int batch, void *stream);
int plain_fp_fan_adjoint(const ct_plan *p, const float *sino, float *img, int batch, void *stream);
int plain_bp_fan(const ct_plan *p, const float *sino, float *img, int batch, void *stream);
}  // namespace ctk

// Launch accounting (api.cu).
void ct_count_launch(uint64_t n = 1);
// Sets the text ct_last_error() returns on this thread (api.cu).
void ct_set_last_error(const char *msg);
