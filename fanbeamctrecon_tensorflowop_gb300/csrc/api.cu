// The C ABI (include/ctgb.h): argument validation, plans, workspace, dispatch.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "common.cuh"

namespace {

thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};

// Device memory: the caller's allocator (ct_set_allocator) or, when none is
// set, the CUDA runtime.  Every allocation the library makes goes through
// dev_alloc, which counts the successful ones (ct_device_alloc_count).
std::mutex g_alloc_mu;
ct_allocator g_alloc{};  // alloc == NULL: cudaMalloc / cudaMallocAsync
std::atomic<uint64_t> g_alloc_count{0};

ct_allocator current_allocator() {
    std::lock_guard<std::mutex> lock(g_alloc_mu);
    return g_alloc;
}

// stream_ordered: scratch of one call (cudaMallocAsync on `s`); otherwise a
// plan table (cudaMalloc).
cudaError_t dev_alloc(const ct_allocator &a, void **p, size_t bytes, cudaStream_t s,
                      bool stream_ordered) {
    *p = nullptr;
    if (a.alloc) {
        *p = a.alloc(a.ctx, bytes, reinterpret_cast<ct_stream>(s));
        if (!*p) return cudaErrorMemoryAllocation;
        if (reinterpret_cast<uintptr_t>(*p) % 256) {  // the documented alignment
            a.free(a.ctx, *p, reinterpret_cast<ct_stream>(s));
            *p = nullptr;
            return cudaErrorMemoryAllocation;
        }
    } else {
        cudaError_t e = stream_ordered ? cudaMallocAsync(p, bytes, s) : cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            *p = nullptr;
            return e;
        }
    }
    g_alloc_count.fetch_add(1, std::memory_order_relaxed);
    return cudaSuccess;
}

void dev_free(const ct_allocator &a, void *p, cudaStream_t s, bool stream_ordered) {
    if (!p) return;
    if (a.alloc)
        a.free(a.ctx, p, reinterpret_cast<ct_stream>(s));
    else if (stream_ordered)
        cudaFreeAsync(p, s);
    else
        cudaFree(p);
}

ct_status cuda_status(cudaError_t e, const char *where) {
    if (e == cudaSuccess) return CT_OK;
    char buf[256];
    std::snprintf(buf, sizeof(buf), "%s: %s (%d)", where, cudaGetErrorString(e), (int)e);
    g_last_error = buf;
    return e == cudaErrorMemoryAllocation ? CT_ERR_ALLOC : CT_ERR_CUDA;
}

ct_status launch_status(int e, const char *where) { return cuda_status((cudaError_t)e, where); }

// Makes the plan's device current for the duration of a call and restores
// the caller's device afterwards.
struct DeviceScope {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceScope(int dev) {
        err = cudaGetDevice(&prev);
        if (err == cudaSuccess && prev != dev) err = cudaSetDevice(dev);
    }
    ~DeviceScope() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

// Caller-provided scratch, or a stream-ordered allocation released after the
// last kernel that uses it.
struct Workspace {
    void *ptr = nullptr;
    bool owned = false;
    cudaStream_t stream = nullptr;
    ct_allocator alloc{};
    ~Workspace() {
        if (owned && ptr) dev_free(alloc, ptr, stream, true);
    }
};

ct_status acquire(Workspace &w, void *given, size_t given_bytes, size_t need, cudaStream_t s) {
    w.stream = s;
    if (need == 0) return CT_OK;
    if (given) {
        if (given_bytes < need) {
            g_last_error = "workspace smaller than ct_workspace_size";
            return CT_ERR_WORKSPACE;
        }
        if (reinterpret_cast<uintptr_t>(given) % 16) {
            g_last_error = "workspace not 16-byte aligned";
            return CT_ERR_WORKSPACE;
        }
        w.ptr = given;
        return CT_OK;
    }
    w.alloc = current_allocator();
    cudaError_t e = dev_alloc(w.alloc, &w.ptr, need, s, true);
    if (e != cudaSuccess) return cuda_status(e, "device allocation (workspace)");
    w.owned = true;
    return CT_OK;
}

size_t sino_bytes(const ct_plan *p, int batch) {
    return sizeof(float) * (size_t)batch * p->g.n_views * p->g.n_cols;
}

ct_status check_call(const ct_plan *p, const void *in, const void *out, int batch) {
    if (!p) return CT_ERR_NULL_POINTER;
    if (batch < 0) return CT_ERR_INVALID_ARGUMENT;
    if (batch > 0 && (!in || !out)) return CT_ERR_NULL_POINTER;
    if (in && out && in == out) return CT_ERR_INVALID_ARGUMENT;
    return CT_OK;
}

size_t proj_bytes(const ct_plan *p, int batch) {
    return sizeof(float) * (size_t)batch * p->g.n_views * p->n_rows * p->g.n_cols;
}

// where FBP's backprojection work starts (after its sinogram copies,
// 256-byte aligned)
size_t fbp_work_offset(const ct_plan *p, int batch) {
    const size_t copies = ctk::has_preweight(p) ? 2 : 1;
    return (copies * sino_bytes(p, batch) + 255) & ~(size_t)255;
}

// where FDK's backprojection work starts (after its projection copies,
// 256-byte aligned)
size_t fdk_cone_work_offset(const ct_plan *p, int batch) {
    const size_t copies = ctk::has_preweight(p) ? 2 : 1;
    return (copies * proj_bytes(p, batch) + 255) & ~(size_t)255;
}

// where the FBP adjoint's transpose work starts (after its sinogram
// copies, 256-byte aligned)
size_t fbp_adjoint_work_offset(const ct_plan *p, int batch) {
    const size_t copies = ctk::has_preweight(p) ? 2 : 1;
    return (copies * sino_bytes(p, batch) + 255) & ~(size_t)255;
}

// where the FDK adjoint's transpose work starts (after its projection
// copies, 256-byte aligned)
size_t fdk_adjoint_work_offset(const ct_plan *p, int batch) {
    const size_t copies = ctk::has_preweight(p) ? 2 : 1;
    return (copies * proj_bytes(p, batch) + 255) & ~(size_t)255;
}

size_t op_workspace(const ct_plan *p, ct_op op, int batch) {
    const size_t parker = ctk::has_preweight(p) ? 2 : 1;  // weighted copy + filtered copy
    switch (op) {
        case CT_OP_FP_CONE:
            return ctk::cone_fp_work_bytes(p, batch);
        case CT_OP_FDK_CONE:  // + the backprojection's quad images
            return fdk_cone_work_offset(p, batch) + ctk::cone_bp_work_bytes(p);
        case CT_OP_FDK_CONE_ADJOINT:  // + the transpose's own work
            return fdk_adjoint_work_offset(p, batch) + ctk::cone_bp_transpose_work_bytes(p, batch);
        case CT_OP_FP:
            return ctk::fp_fan_work_bytes(p, batch);
        case CT_OP_FP_ADJOINT:
            return ctk::fp_fan_adjoint_work_bytes(p, batch);
        case CT_OP_FBP:  // + the backprojection's tap images
        case CT_OP_FDK_BP:
            return fbp_work_offset(p, batch) + ctk::bp_fan_work_bytes(p, batch);
        case CT_OP_FBP_ADJOINT:  // + the transpose's slice-quad images
            return fbp_adjoint_work_offset(p, batch) + ctk::bp_fan_transpose_work_bytes(p, batch);
        case CT_OP_BP_ADJOINT:
            return ctk::bp_fan_transpose_work_bytes(p, batch);
        default:
            return 0;
    }
}

void free_plan(ct_plan *p) {
    if (!p) return;
    for (void *t : {(void *)p->d_view_cs, (void *)p->d_view_cs_lo, (void *)p->d_col_tan,
                    (void *)p->d_ray, (void *)p->d_ray_rec,
                    (void *)p->d_nsamp, (void *)p->d_fp_order, (void *)p->d_taps,
                    (void *)p->d_chan_s,
                    (void *)p->d_tc_hi, (void *)p->d_tc_lo, (void *)p->d_err,
                    (void *)p->d_parker, (void *)p->d_cosw, (void *)p->d_view_z,
                    (void *)p->d_bpt_warp, (void *)p->d_bpt_bnd, (void *)p->d_bpt_ray,
                    (void *)p->d_fov_row, (void *)p->d_fov_col})
        dev_free(p->alloc, t, nullptr, false);
    delete p;
}

// Allocates a plan table with the plan's allocator and copies `src` into it.
template <typename T>
ct_status upload(const ct_plan *p, T **dst, const std::vector<T> &src) {
    *dst = nullptr;
    if (src.empty()) return CT_OK;
    void *d = nullptr;
    cudaError_t e = dev_alloc(p->alloc, &d, sizeof(T) * src.size(), nullptr, false);
    if (e != cudaSuccess) return cuda_status(e, "device allocation (plan table)");
    *dst = static_cast<T *>(d);
    e = cudaMemcpy(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice);
    return cuda_status(e, "cudaMemcpy(plan table)");
}

// Filtered backprojection shared by ct_fbp_fan and ct_fdk_bp.
ct_status filtered_bp(const ct_plan *p, const float *d_sino, float *d_img, int batch,
                      void *d_work, size_t work_bytes, cudaStream_t s, const char *name) {
    Workspace w;
    ct_status st = acquire(w, d_work, work_bytes, op_workspace(p, CT_OP_FBP, batch), s);
    if (st != CT_OK) return st;
    float *filt = static_cast<float *>(w.ptr);
    const float *src = d_sino;
    if (ctk::has_preweight(p)) {  // short scan / cosine: weight, then filter
        float *wtd = filt + (size_t)batch * p->g.n_views * p->g.n_cols;
        st = launch_status(ctk::apply_preweight(p, d_sino, wtd, batch, s), name);
        if (st != CT_OK) return st;
        src = wtd;
    }
    st = launch_status(ctk::ramp_filter(p, src, filt, batch * p->g.n_views, s), name);
    if (st != CT_OK) return st;
    void *bwork = ctk::bp_fan_work_bytes(p, batch)
                      ? static_cast<char *>(w.ptr) + fbp_work_offset(p, batch)
                      : nullptr;
    return launch_status(ctk::bp_fan(p, filt, d_img, batch, 1, bwork, s), name);
}

}  // namespace

void ct_count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

#ifdef CT_DEBUG
namespace ctk {
namespace dbg {
namespace {
struct FlagReader {
    TakeFn fn;
    const char *file;
};
std::vector<FlagReader> &registry() {
    static std::vector<FlagReader> r;
    return r;
}
}  // namespace
void add_flag(TakeFn fn, const char *file) { registry().push_back(FlagReader{fn, file}); }
}  // namespace dbg
}  // namespace ctk

// Reads and clears every file's index-check flag (debug builds); returns the
// first raised one as "file:line" in *where, or false.
static bool take_debug_flags(std::string *where) {
    bool any = false;
    for (const auto &r : ctk::dbg::registry()) {
        const unsigned line = r.fn();
        if (line && !any) {
            *where = std::string(r.file) + ":" + std::to_string(line);
            any = true;
        }
    }
    return any;
}
#endif

void ct_set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }

extern "C" {

const char *ct_status_string(ct_status s) {
    switch (s) {
        case CT_OK: return "CT_OK";
        case CT_ERR_INVALID_ARGUMENT: return "CT_ERR_INVALID_ARGUMENT: invalid geometry, size or option";
        case CT_ERR_NULL_POINTER: return "CT_ERR_NULL_POINTER: a required pointer is NULL";
        case CT_ERR_WORKSPACE: return "CT_ERR_WORKSPACE: workspace smaller than required";
        case CT_ERR_CUDA: return "CT_ERR_CUDA: a CUDA call failed";
        case CT_ERR_ALLOC: return "CT_ERR_ALLOC: allocation failed";
        case CT_ERR_UNSUPPORTED: return "CT_ERR_UNSUPPORTED: not supported by this build";
        case CT_ERR_TIMEOUT: return "CT_ERR_TIMEOUT: a bounded device wait gave up";
        case CT_ERR_DEVICE_CHECK: return "CT_ERR_DEVICE_CHECK: a debug build's index check failed";
    }
    return "unknown ct_status";
}

const char *ct_version(void) { return "ctgb 0.1.0 (sm_103a)"; }

const char *ct_last_error(void) { return g_last_error.c_str(); }

uint64_t ct_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

uint32_t ct_build_flags(void) { return CT_DEBUG_BUILD ? CT_BUILD_INDEX_CHECKS : 0u; }

ct_status ct_set_allocator(const ct_allocator *allocator) {
    ct_allocator a{};
    if (allocator) {
        if (!allocator->alloc || !allocator->free) return CT_ERR_NULL_POINTER;
        a = *allocator;
    }
    std::lock_guard<std::mutex> lock(g_alloc_mu);
    g_alloc = a;
    return CT_OK;
}

uint64_t ct_device_alloc_count(void) { return g_alloc_count.load(std::memory_order_relaxed); }

ct_status ct_host_mapped(const void *host_ptr, void **device_ptr) {
    if (!host_ptr || !device_ptr) return CT_ERR_NULL_POINTER;
    *device_ptr = nullptr;
    cudaPointerAttributes at;
    const cudaError_t e = cudaPointerGetAttributes(&at, host_ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();  // an unknown pointer leaves no error on the context
        g_last_error = "ct_host_mapped: not CUDA host memory";
        return CT_ERR_INVALID_ARGUMENT;
    }
    if (at.type != cudaMemoryTypeHost || at.devicePointer == nullptr) {
        g_last_error = "ct_host_mapped: not page-locked host memory mapped for the device";
        return CT_ERR_INVALID_ARGUMENT;
    }
    *device_ptr = at.devicePointer;
    return CT_OK;
}

ct_status ct_geom_from_param16(const float param[16], ct_fan_geom *out) {
    return ct_decode_param16(param, out);
}

ct_status ct_fp_ray_table(const ct_fan_geom *geom, const float *angles, int n_angles,
                          float *ray4, int32_t *nsamp) {
    if (!geom || !angles || !ray4 || !nsamp) return CT_ERR_NULL_POINTER;
    ct_status st = ct_validate_geom(geom);
    if (st != CT_OK) return st;
    if (n_angles != geom->n_views) return CT_ERR_INVALID_ARGUMENT;
    ct_host_tables t;
    ct_build_ray_table(geom, angles, &t);
    std::memcpy(ray4, t.ray.data(), sizeof(float) * t.ray.size());
    std::memcpy(nsamp, t.nsamp.data(), sizeof(int32_t) * t.nsamp.size());
    return CT_OK;
}

static ct_status plan_create(const ct_fan_geom *geom, int n_rows, int nz, bool cone,
                             const float *angles, const float *source_z, int n_angles,
                             const ct_plan_opts *opts, ct_plan **out) {
    if (!geom || !angles || !out) return CT_ERR_NULL_POINTER;
    *out = nullptr;
    ct_status st = ct_validate_geom(geom);
    if (st != CT_OK) return st;
    if (n_rows < 1 || nz < 1) return CT_ERR_INVALID_ARGUMENT;
    if ((int64_t)geom->n_views * n_rows * geom->n_cols >= (int64_t)1 << 31 ||
        (int64_t)nz * geom->nx * geom->ny >= (int64_t)1 << 31)
        return CT_ERR_INVALID_ARGUMENT;
    if (n_angles != geom->n_views) return CT_ERR_INVALID_ARGUMENT;
    for (int v = 0; v < n_angles; ++v)
        if (!std::isfinite(angles[v]) || (source_z && !std::isfinite(source_z[v])))
            return CT_ERR_INVALID_ARGUMENT;
    ct_plan_opts o;
    std::memset(&o, 0, sizeof(o));
    if (opts) {
        o = *opts;
        for (int r : o.reserved)
            if (r != 0) return CT_ERR_INVALID_ARGUMENT;
        if (o.short_scan != 0 && o.short_scan != 1) return CT_ERR_INVALID_ARGUMENT;
        if (o.cosine_weight != 0 && o.cosine_weight != 1) return CT_ERR_INVALID_ARGUMENT;
        if (o.texture_weights != 0 && o.texture_weights != 1) return CT_ERR_INVALID_ARGUMENT;
    }
    if (o.filter_window != CT_WINDOW_RAMLAK && o.filter_window != CT_WINDOW_SHEPP_LOGAN)
        return CT_ERR_INVALID_ARGUMENT;
    if (o.filter_algo < CT_FILTER_AUTO || o.filter_algo > CT_FILTER_TOEPLITZ_TC)
        return CT_ERR_INVALID_ARGUMENT;
    if (o.filter_algo == CT_FILTER_TOEPLITZ_TC && !ctk::ramp_tc_supported(geom->n_cols))
        return CT_ERR_UNSUPPORTED;

    ct_host_tables t;
    ct_build_view_table(geom, angles, &t);
    ct_build_ray_table(geom, angles, &t);
    ct_build_filter_taps(geom, o.filter_window, &t);
    ct_build_channel_table(geom, &t);
    if (o.short_scan) ct_build_parker(geom, angles, &t);
    if (o.cosine_weight) ct_build_cosine(geom, n_rows, cone, &t);
    if (source_z) t.view_z.assign(source_z, source_z + n_angles);
    ct_bpt_tables bt;
    if (!cone) ct_build_bpt_tables(geom, angles, &bt);

    ct_plan *p = new (std::nothrow) ct_plan();
    if (!p) return CT_ERR_ALLOC;
    p->g = *geom;
    p->opts = o;
    // AUTO: the tensor-core Toeplitz filter wherever it applies (measured
    // 4-6x faster than the direct FP32 filter at 984 x 888, same accuracy)
    p->filter_algo = (o.filter_algo == CT_FILTER_TOEPLITZ_TC ||
                      (o.filter_algo == CT_FILTER_AUTO && ctk::ramp_tc_supported(geom->n_cols)))
                         ? CT_FILTER_TOEPLITZ_TC
                         : CT_FILTER_DIRECT;
    p->fp_weight = (float)(CT_FP_STEP * (double)geom->dx);
    p->fov_r2 = geom->rfov * geom->rfov;
    p->atan_deg = ct_fit_atan(1.02 * ct_max_tan_gamma(geom), p->atan_coef);
    {
        // cells up to 1.5 pixels outside the FOV disc (the adjoint gather)
        const double r = (double)geom->rfov + 1.5 * (double)geom->dx, R = geom->sid;
        p->gather_atan_deg =
            r < R ? ct_fit_atan(1.02 * r / std::sqrt(R * R - r * r), p->gather_atan_coef) : 0;
        if (!(r < R))
            for (float &c : p->gather_atan_coef) c = 0.0f;
    }
    // the adjoint gather's 32-byte ray records (one load per candidate ray)
    std::vector<float> ray_rec(t.ray.size() * 2);
    for (size_t r = 0; r < t.ray.size() / 4; ++r) {
        for (int k = 0; k < 4; ++k) ray_rec[8 * r + k] = t.ray[4 * r + k];
        for (int k = 0; k < 2; ++k) {
            const float st = t.ray[4 * r + 2 + k];
            // a zero step gets 1e30: the adjoint's support bounds become +-inf-like
            ray_rec[8 * r + 4 + k] = st != 0.0f ? (float)(1.0 / (double)st) : 1e30f;
        }
        std::memcpy(&ray_rec[8 * r + 6], &t.nsamp[r], sizeof(float));
        ray_rec[8 * r + 7] = 0.0f;
    }
    p->n_rows = n_rows;
    p->nz = nz;
    p->view_z_min = p->view_z_max = 0.0f;
    for (size_t v = 0; v < t.view_z.size(); ++v) {
        p->view_z_min = v ? std::min(p->view_z_min, t.view_z[v]) : t.view_z[v];
        p->view_z_max = v ? std::max(p->view_z_max, t.view_z[v]) : t.view_z[v];
    }
    p->total_samples = t.total_samples;
    p->max_nsamp = t.max_nsamp;
    p->h_view_cs = t.view_cs;
    p->alloc = current_allocator();
    cudaError_t e = cudaGetDevice(&p->device);
    if (e != cudaSuccess) {
        delete p;
        return cuda_status(e, "cudaGetDevice");
    }
    if ((st = upload(p, &p->d_view_cs, t.view_cs)) != CT_OK ||
        (st = upload(p, &p->d_view_cs_lo, t.view_cs_lo)) != CT_OK ||
        (st = upload(p, &p->d_col_tan, t.col_tan)) != CT_OK ||
        (st = upload(p, &p->d_ray, t.ray)) != CT_OK ||
        (st = upload(p, &p->d_nsamp, t.nsamp)) != CT_OK ||
        (st = upload(p, &p->d_fp_order,
                     ctk::fp_block_order(geom->n_views, geom->n_cols, t.ray, t.nsamp))) !=
            CT_OK ||
        (st = upload(p, &p->d_ray_rec, ray_rec)) != CT_OK ||
        (st = upload(p, &p->d_taps, t.taps)) != CT_OK ||
        (st = upload(p, &p->d_chan_s, t.chan_s)) != CT_OK ||
        (st = upload(p, &p->d_parker, t.parker)) != CT_OK ||
        (st = upload(p, &p->d_cosw, t.cosw)) != CT_OK ||
        (st = upload(p, &p->d_view_z, t.view_z)) != CT_OK) {
        free_plan(p);
        return st;
    }
    if (p->filter_algo == CT_FILTER_TOEPLITZ_TC) {
        std::vector<float> hi, lo;
        ctk::build_tc_taps(t.taps.data(), geom->n_cols, hi, lo);
        if ((st = upload(p, &p->d_tc_hi, hi)) != CT_OK ||
            (st = upload(p, &p->d_tc_lo, lo)) != CT_OK) {
            free_plan(p);
            return st;
        }
    }
    if (bt.ok) {
        p->bpt_W = bt.W;
        if ((st = upload(p, &p->d_bpt_warp, bt.warp)) != CT_OK ||
            (st = upload(p, &p->d_bpt_bnd, bt.bnd)) != CT_OK ||
            (st = upload(p, &p->d_bpt_ray, bt.ray)) != CT_OK ||
            (st = upload(p, &p->d_fov_row, bt.fov_row)) != CT_OK ||
            (st = upload(p, &p->d_fov_col, bt.fov_col)) != CT_OK) {
            free_plan(p);
            return st;
        }
    }
    {
        const std::vector<int> zero(1, 0);
        if ((st = upload(p, &p->d_err, zero)) != CT_OK) {
            free_plan(p);
            return st;
        }
    }
    *out = p;
    return CT_OK;
}

ct_status ct_plan_create(const ct_fan_geom *geom, const float *angles, int n_angles,
                         const ct_plan_opts *opts, ct_plan **out) {
    return plan_create(geom, 1, 1, false, angles, nullptr, n_angles, opts, out);
}

ct_status ct_plan_create_cone_ex(const ct_fan_geom *geom, int n_rows, int nz,
                                 const float *angles, const float *source_z, int n_angles,
                                 const ct_plan_opts *opts, ct_plan **out) {
    if (!geom) return CT_ERR_NULL_POINTER;
    if (!(geom->drow > 0.0f) || !(geom->dz > 0.0f) || !(geom->sdd > geom->sid))
        return CT_ERR_INVALID_ARGUMENT;
    return plan_create(geom, n_rows, nz, true, angles, source_z, n_angles, opts, out);
}

ct_status ct_plan_create_cone(const ct_fan_geom *geom, int n_rows, int nz, const float *angles,
                              int n_angles, const ct_plan_opts *opts, ct_plan **out) {
    return ct_plan_create_cone_ex(geom, n_rows, nz, angles, nullptr, n_angles, opts, out);
}

ct_status ct_plan_destroy(ct_plan *plan) {
    if (!plan) return CT_OK;
    DeviceScope ds(plan->device);
    free_plan(plan);
    return CT_OK;
}

ct_status ct_plan_check(const ct_plan *plan) {
    if (!plan) return CT_ERR_NULL_POINTER;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    int flag = 0;
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda_status(e, "ct_plan_check");
    e = cudaMemcpy(&flag, plan->d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_status(e, "ct_plan_check");
    if (flag) {
        const int zero = 0;
        cudaMemcpy(plan->d_err, &zero, sizeof(int), cudaMemcpyHostToDevice);
        g_last_error = "a kernel's bounded wait gave up";
        return CT_ERR_TIMEOUT;
    }
#ifdef CT_DEBUG
    std::string where;
    if (take_debug_flags(&where)) {
        g_last_error = "index check failed at " + where;
        return CT_ERR_DEVICE_CHECK;
    }
#endif
    return CT_OK;
}

ct_status ct_plan_selftest_wait_timeout(const ct_plan *plan, int32_t budget_us,
                                        ct_stream stream) {
    if (!plan) return CT_ERR_NULL_POINTER;
    if (budget_us < 1 || budget_us > 1000000) return CT_ERR_INVALID_ARGUMENT;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    return launch_status(ctk::wait_selftest(plan, 1000ull * (unsigned long long)budget_us, stream),
                         "ct_plan_selftest_wait_timeout");
}

ct_status ct_plan_geom(const ct_plan *plan, ct_fan_geom *out) {
    if (!plan || !out) return CT_ERR_NULL_POINTER;
    *out = plan->g;
    return CT_OK;
}

ct_status ct_workspace_size(const ct_plan *plan, ct_op op, int batch, size_t *bytes) {
    if (!plan || !bytes) return CT_ERR_NULL_POINTER;
    if (batch < 0 || op < CT_OP_FP || op > CT_OP_FDK_CONE_ADJOINT) return CT_ERR_INVALID_ARGUMENT;
    *bytes = op_workspace(plan, op, batch);
    return CT_OK;
}

ct_status ct_fp_fan(const ct_plan *plan, const float *d_img, float *d_sino, int batch,
                    void *d_work, size_t work_bytes, ct_stream stream) {
    ct_status st = check_call(plan, d_img, d_sino, batch);
    if (st != CT_OK || batch == 0) return st;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    Workspace w;
    st = acquire(w, d_work, work_bytes, op_workspace(plan, CT_OP_FP, batch), stream);
    if (st != CT_OK) return st;
    return launch_status(
        ctk::fp_fan(plan, d_img, d_sino, batch, w.ptr, stream),
        "ct_fp_fan");
}

ct_status ct_fp_fan_adjoint(const ct_plan *plan, const float *d_sino, float *d_img, int batch,
                            void *d_work, size_t work_bytes, ct_stream stream) {
    ct_status st = check_call(plan, d_sino, d_img, batch);
    if (st != CT_OK || batch == 0) return st;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    Workspace w;
    st = acquire(w, d_work, work_bytes, op_workspace(plan, CT_OP_FP_ADJOINT, batch), stream);
    if (st != CT_OK) return st;
    return launch_status(ctk::fp_fan_adjoint(plan, d_sino, d_img, batch, w.ptr, stream),
                         "ct_fp_fan_adjoint");
}

ct_status ct_bp_fan(const ct_plan *plan, const float *d_sino, float *d_img, int batch,
                    ct_stream stream) {
    ct_status st = check_call(plan, d_sino, d_img, batch);
    if (st != CT_OK || batch == 0) return st;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    Workspace w;
    st = acquire(w, nullptr, 0, ctk::bp_fan_work_bytes(plan, batch), stream);
    if (st != CT_OK) return st;
    return launch_status(ctk::bp_fan(plan, d_sino, d_img, batch, 0, w.ptr, stream), "ct_bp_fan");
}

ct_status ct_bp_fan_adjoint(const ct_plan *plan, const float *d_img, float *d_sino, int batch,
                            ct_stream stream) {
    ct_status st = check_call(plan, d_img, d_sino, batch);
    if (st != CT_OK || batch == 0) return st;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    Workspace w;
    st = acquire(w, nullptr, 0, op_workspace(plan, CT_OP_BP_ADJOINT, batch), stream);
    if (st != CT_OK) return st;
    return launch_status(ctk::bp_fan_transpose(plan, d_img, d_sino, batch, 0, w.ptr, stream),
                         "ct_bp_fan_adjoint");
}

ct_status ct_ramp_filter(const ct_plan *plan, const float *d_sino, float *d_out, int rows,
                         ct_stream stream) {
    ct_status st = check_call(plan, d_sino, d_out, rows);
    if (st != CT_OK || rows == 0) return st;
    if (plan->filter_algo != CT_FILTER_TOEPLITZ_TC &&
        ctk::ramp_direct_smem(plan->g.n_cols) > 227 * 1024)
        return CT_ERR_UNSUPPORTED;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    return launch_status(ctk::ramp_filter(plan, d_sino, d_out, rows, stream), "ct_ramp_filter");
}

ct_status ct_fbp_fan(const ct_plan *plan, const float *d_sino, float *d_img, int batch,
                     void *d_work, size_t work_bytes, ct_stream stream) {
    ct_status st = check_call(plan, d_sino, d_img, batch);
    if (st != CT_OK || batch == 0) return st;
    if (plan->filter_algo != CT_FILTER_TOEPLITZ_TC &&
        ctk::ramp_direct_smem(plan->g.n_cols) > 227 * 1024)
        return CT_ERR_UNSUPPORTED;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    return filtered_bp(plan, d_sino, d_img, batch, d_work, work_bytes, stream, "ct_fbp_fan");
}

ct_status ct_fbp_fan_adjoint(const ct_plan *plan, const float *d_img, float *d_sino, int batch,
                             void *d_work, size_t work_bytes, ct_stream stream) {
    ct_status st = check_call(plan, d_img, d_sino, batch);
    if (st != CT_OK || batch == 0) return st;
    if (plan->filter_algo != CT_FILTER_TOEPLITZ_TC &&
        ctk::ramp_direct_smem(plan->g.n_cols) > 227 * 1024)
        return CT_ERR_UNSUPPORTED;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    Workspace w;
    st = acquire(w, d_work, work_bytes, op_workspace(plan, CT_OP_FBP_ADJOINT, batch), stream);
    if (st != CT_OK) return st;
    float *tmp = static_cast<float *>(w.ptr);
    void *twork = ctk::bp_fan_transpose_work_bytes(plan, batch)
                      ? static_cast<char *>(w.ptr) + fbp_adjoint_work_offset(plan, batch)
                      : nullptr;
    st = launch_status(ctk::bp_fan_transpose(plan, d_img, tmp, batch, 1, twork, stream),
                       "ct_fbp_fan_adjoint");
    if (st != CT_OK) return st;
    // The row filter is a symmetric Toeplitz matrix: its transpose is itself;
    // the short-scan weights are diagonal.
    if (!ctk::has_preweight(plan))
        return launch_status(ctk::ramp_filter(plan, tmp, d_sino, batch * plan->g.n_views, stream),
                             "ct_fbp_fan_adjoint");
    float *filt = tmp + (size_t)batch * plan->g.n_views * plan->g.n_cols;
    st = launch_status(ctk::ramp_filter(plan, tmp, filt, batch * plan->g.n_views, stream),
                       "ct_fbp_fan_adjoint");
    if (st != CT_OK) return st;
    return launch_status(ctk::apply_preweight(plan, filt, d_sino, batch, stream),
                         "ct_fbp_fan_adjoint");
}

ct_status ct_fdk_bp(const ct_plan *plan, const float *d_sino, float *d_img, int batch,
                    void *d_work, size_t work_bytes, ct_stream stream) {
    ct_status st = check_call(plan, d_sino, d_img, batch);
    if (st != CT_OK || batch == 0) return st;
    if (plan->filter_algo != CT_FILTER_TOEPLITZ_TC &&
        ctk::ramp_direct_smem(plan->g.n_cols) > 227 * 1024)
        return CT_ERR_UNSUPPORTED;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    // nZ = nRows = 1 (FDK/FBP.cc:85,98): the single-row view texture clamps
    // every row index to row 0, so CB_EA reduces to the weighted fan BP with
    // detector shift.
    return filtered_bp(plan, d_sino, d_img, batch, d_work, work_bytes, stream, "ct_fdk_bp");
}

ct_status ct_cone_bp(const ct_plan *plan, const float *d_proj, float *d_vol, int batch,
                     ct_stream stream) {
    ct_status st = check_call(plan, d_proj, d_vol, batch);
    if (st != CT_OK || batch == 0) return st;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    // no scratch: four gathers per sample (FDK's tap images need a workspace)
    return launch_status(ctk::cone_bp(plan, d_proj, d_vol, batch, nullptr, stream), "ct_cone_bp");
}

ct_status ct_fdk_cone(const ct_plan *plan, const float *d_proj, float *d_vol, int batch,
                      void *d_work, size_t work_bytes, ct_stream stream) {
    ct_status st = check_call(plan, d_proj, d_vol, batch);
    if (st != CT_OK || batch == 0) return st;
    if (plan->filter_algo != CT_FILTER_TOEPLITZ_TC &&
        ctk::ramp_direct_smem(plan->g.n_cols) > 227 * 1024)
        return CT_ERR_UNSUPPORTED;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    Workspace w;
    st = acquire(w, d_work, work_bytes, op_workspace(plan, CT_OP_FDK_CONE, batch), stream);
    if (st != CT_OK) return st;
    float *filt = static_cast<float *>(w.ptr);
    const float *src = d_proj;
    if (ctk::has_preweight(plan)) {
        float *wtd = filt + proj_bytes(plan, batch) / sizeof(float);
        st = launch_status(ctk::apply_preweight(plan, d_proj, wtd, batch, stream), "ct_fdk_cone");
        if (st != CT_OK) return st;
        src = wtd;
    }
    st = launch_status(
        ctk::ramp_filter(plan, src, filt, batch * plan->g.n_views * plan->n_rows, stream),
        "ct_fdk_cone");
    if (st != CT_OK) return st;
    void *bwork = ctk::cone_bp_work_bytes(plan)
                      ? static_cast<char *>(w.ptr) + fdk_cone_work_offset(plan, batch)
                      : nullptr;
    return launch_status(ctk::cone_bp(plan, filt, d_vol, batch, bwork, stream), "ct_fdk_cone");
}

ct_status ct_fdk_cone_adjoint(const ct_plan *plan, const float *d_vol, float *d_proj, int batch,
                              void *d_work, size_t work_bytes, ct_stream stream) {
    ct_status st = check_call(plan, d_vol, d_proj, batch);
    if (st != CT_OK || batch == 0) return st;
    if (plan->filter_algo != CT_FILTER_TOEPLITZ_TC &&
        ctk::ramp_direct_smem(plan->g.n_cols) > 227 * 1024)
        return CT_ERR_UNSUPPORTED;
    if (!ctk::cone_bp_transpose_supported(plan)) return CT_ERR_UNSUPPORTED;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    Workspace w;
    st = acquire(w, d_work, work_bytes, op_workspace(plan, CT_OP_FDK_CONE_ADJOINT, batch),
                 stream);
    if (st != CT_OK) return st;
    float *tmp = static_cast<float *>(w.ptr);
    void *twork = static_cast<char *>(w.ptr) + fdk_adjoint_work_offset(plan, batch);
    st = launch_status(ctk::cone_bp_transpose(plan, d_vol, tmp, batch, twork, stream),
                       "ct_fdk_cone_adjoint");
    if (st != CT_OK) return st;
    const int rows = batch * plan->g.n_views * plan->n_rows;
    if (!ctk::has_preweight(plan))
        return launch_status(ctk::ramp_filter(plan, tmp, d_proj, rows, stream),
                             "ct_fdk_cone_adjoint");
    float *filt = tmp + proj_bytes(plan, batch) / sizeof(float);
    st = launch_status(ctk::ramp_filter(plan, tmp, filt, rows, stream), "ct_fdk_cone_adjoint");
    if (st != CT_OK) return st;
    return launch_status(ctk::apply_preweight(plan, filt, d_proj, batch, stream),
                         "ct_fdk_cone_adjoint");
}

ct_status ct_fp_cone(const ct_plan *plan, const float *d_vol, float *d_proj, int batch,
                     void *d_work, size_t work_bytes, ct_stream stream) {
    ct_status st = check_call(plan, d_vol, d_proj, batch);
    if (st != CT_OK || batch == 0) return st;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    Workspace w;
    st = acquire(w, d_work, work_bytes, ctk::cone_fp_work_bytes(plan, batch), stream);
    if (st != CT_OK) return st;
    return launch_status(ctk::cone_fp(plan, d_vol, d_proj, batch, w.ptr, stream), "ct_fp_cone");
}

ct_status ct_batch_workspace_size(const ct_batch_item *items, int n, size_t *bytes) {
    if (!bytes) return CT_ERR_NULL_POINTER;
    return ctk::batch_workspace(items, n, bytes);
}

ct_status ct_batch_run(const ct_batch_item *items, int n, void *d_work, size_t work_bytes,
                       ct_stream stream) {
    size_t need = 0;
    ct_status st = ctk::batch_workspace(items, n, &need);
    if (st != CT_OK || n == 0) return st;
    DeviceScope ds(items[0].plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    Workspace w;
    st = acquire(w, d_work, work_bytes, need, stream);
    if (st != CT_OK) return st;
    const ct_batch_config cfg = ctk::batch_lookup(items, n, nullptr);
    return launch_status(ctk::batch_run(items, n, w.ptr, stream, cfg, nullptr), "ct_batch_run");
}

ct_status ct_batch_tune(const ct_batch_item *items, int n, void *d_work, size_t work_bytes,
                        int32_t reps, ct_stream stream, ct_batch_config *out) {
    size_t need = 0;
    ct_status st = ctk::batch_workspace(items, n, &need);
    if (st != CT_OK || n == 0) return st;
    DeviceScope ds(items[0].plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(stream, &cap);
    if (e != cudaSuccess) return cuda_status(e, "cudaStreamIsCapturing");
    if (cap != cudaStreamCaptureStatusNone) {
        ct_set_last_error("ct_batch_tune: the stream is being captured; tune before capture");
        return CT_ERR_INVALID_ARGUMENT;
    }
    Workspace w;
    st = acquire(w, d_work, work_bytes, need, stream);
    if (st != CT_OK) return st;
    ct_batch_config best{};
    st = launch_status(ctk::batch_tune(items, n, w.ptr, stream, reps > 0 ? reps : 3, &best),
                       "ct_batch_tune");
    if (st != CT_OK) return st;
    ctk::batch_store(items, n, &best);
    if (out) *out = best;
    return CT_OK;
}

ct_status ct_batch_get_config(const ct_batch_item *items, int n, ct_batch_config *out,
                              int32_t *tuned) {
    if (!out) return CT_ERR_NULL_POINTER;
    size_t need = 0;
    ct_status st = ctk::batch_workspace(items, n, &need);
    if (st != CT_OK) return st;
    bool t = false;
    *out = ctk::batch_lookup(items, n, &t);
    if (tuned) *tuned = t ? 1 : 0;
    return CT_OK;
}

ct_status ct_batch_set_config(const ct_batch_item *items, int n, const ct_batch_config *config) {
    size_t need = 0;
    ct_status st = ctk::batch_workspace(items, n, &need);
    if (st != CT_OK) return st;
    if (config && (st = ctk::batch_check_config(*config)) != CT_OK) return st;
    ctk::batch_store(items, n, config);
    return CT_OK;
}

ct_status ct_plain_fp_fan(const ct_plan *plan, const float *d_img, float *d_sino, int batch,
                          ct_stream stream) {
    ct_status st = check_call(plan, d_img, d_sino, batch);
    if (st != CT_OK || batch == 0) return st;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    return launch_status(ctk::plain_fp_fan(plan, d_img, d_sino, batch, stream), "ct_plain_fp_fan");
}

ct_status ct_plain_fp_fan_adjoint(const ct_plan *plan, const float *d_sino, float *d_img,
                                  int batch, ct_stream stream) {
    ct_status st = check_call(plan, d_sino, d_img, batch);
    if (st != CT_OK || batch == 0) return st;
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    return launch_status(ctk::plain_fp_fan_adjoint(plan, d_sino, d_img, batch, stream),
                         "ct_plain_fp_fan_adjoint");
}

ct_status ct_plain_bp_fan(const ct_plan *plan, const float *d_sino, float *d_img, int batch,
                          ct_stream stream) {
    ct_status st = check_call(plan, d_sino, d_img, batch);
    if (st != CT_OK || batch == 0) return st;
    if (plan->opts.texture_weights) return CT_ERR_UNSUPPORTED;  // the loop keeps exact weights
    DeviceScope ds(plan->device);
    if (ds.err != cudaSuccess) return cuda_status(ds.err, "cudaSetDevice");
    return launch_status(ctk::plain_bp_fan(plan, d_sino, d_img, batch, stream), "ct_plain_bp_fan");
}

}  // extern "C"
