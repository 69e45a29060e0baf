// Filtered backprojection without any device allocation.
//
// ct_fbp_fan needs a scratch buffer for the filtered sinogram and takes it
// from the caller or from cudaMallocAsync.  Some callers can do neither:
// plugins inside a host framework that owns all device memory and hands a
// plugin only its input and output buffers, and real-time pipelines that
// forbid device allocation after start-up because an allocation can
// synchronise the device and has no latency bound.  ct_fbp_fan_static_scratch
// serves them from a fixed array in this library's own device memory.
//
// The array is a file-scope __device__ variable: every GPU on which this
// file's device code is loaded holds its CT_FBP_STATIC_SCRATCH_FLOATS floats
// until the process exits.  The CUDA runtime loads a module lazily (by
// default since CUDA 12.2), so the array is reserved when the first call on a
// device looks up its address: that first call, the set-up, takes the 32 MiB
// and can fail with CT_ERR_ALLOC when the device is full.  Host code cannot
// use the symbol itself as a device address, so that set-up looks the
// address up once per device, with the device current, and caches it; a
// cudaDeviceReset in between invalidates the cached address (a process that
// resets a device must not call this entry point afterwards).
#include <mutex>
#include <string>

#include "common.cuh"

namespace {

static __device__ __align__(256) float g_fbp_scratch[CT_FBP_STATIC_SCRATCH_FLOATS];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
float *g_scratch_ptr[kMaxDevices] = {};

// Device address of g_fbp_scratch on `dev` (which must be current).
cudaError_t scratch_address(int dev, float **out) {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_fbp_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = static_cast<float *>(p);
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

struct CurrentDevice {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit CurrentDevice(int dev) {
        err = cudaGetDevice(&prev);
        if (err == cudaSuccess && prev != dev) err = cudaSetDevice(dev);
    }
    ~CurrentDevice() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

ct_status fail_cuda(cudaError_t e, const char *where) {
    ct_set_last_error((std::string(where) + ": " + cudaGetErrorString(e)).c_str());
    return e == cudaErrorMemoryAllocation ? CT_ERR_ALLOC : CT_ERR_CUDA;
}

}  // namespace

extern "C" ct_status ct_fbp_fan_static_scratch(const ct_plan *plan, const float *d_sino,
                                               float *d_img, int batch, ct_stream stream) {
    if (!plan) return CT_ERR_NULL_POINTER;
    if (batch < 0) return CT_ERR_INVALID_ARGUMENT;
    if (batch == 0) return CT_OK;
    if (!d_sino || !d_img) return CT_ERR_NULL_POINTER;
    if (static_cast<const void *>(d_sino) == static_cast<const void *>(d_img))
        return CT_ERR_INVALID_ARGUMENT;
    const size_t need = (size_t)batch * plan->g.n_views * plan->g.n_cols;
    if (need > (size_t)CT_FBP_STATIC_SCRATCH_FLOATS) {
        ct_set_last_error(("ct_fbp_fan_static_scratch: batch * n_views * n_cols = " +
                           std::to_string(need) + " floats exceeds the static scratch of " +
                           std::to_string((size_t)CT_FBP_STATIC_SCRATCH_FLOATS) +
                           " floats; split the batch")
                              .c_str());
        return CT_ERR_WORKSPACE;
    }
    // the same width limit as ct_fbp_fan: only the direct filter's shared
    // memory bounds the width; tensor-core plans take up to 4032 channels
    if (plan->filter_algo != CT_FILTER_TOEPLITZ_TC &&
        ctk::ramp_direct_smem(plan->g.n_cols) > 227 * 1024)
        return CT_ERR_UNSUPPORTED;
    if (ctk::has_preweight(plan)) {
        ct_set_last_error("ct_fbp_fan_static_scratch: short-scan and cosine-weighted plans "
                          "need a second scratch sinogram; use ct_fbp_fan");
        return CT_ERR_UNSUPPORTED;
    }
    if (plan->device < 0 || plan->device >= kMaxDevices) return CT_ERR_UNSUPPORTED;
    CurrentDevice cd(plan->device);
    if (cd.err != cudaSuccess) return fail_cuda(cd.err, "cudaSetDevice");
    float *scratch = nullptr;
    cudaError_t e = scratch_address(plan->device, &scratch);
    if (e != cudaSuccess) return fail_cuda(e, "cudaGetSymbolAddress(g_fbp_scratch)");
    // The filter writes every one of the `need` scratch floats before the
    // backprojection reads them, so nothing left by an earlier call is used.
    e = (cudaError_t)ctk::ramp_filter(plan, d_sino, scratch, batch * plan->g.n_views, stream);
    if (e != cudaSuccess) return fail_cuda(e, "ct_fbp_fan_static_scratch (filter)");
    e = (cudaError_t)ctk::bp_fan(plan, scratch, d_img, batch, 1, nullptr, stream);
    if (e != cudaSuccess) return fail_cuda(e, "ct_fbp_fan_static_scratch (backprojection)");
    return CT_OK;
}
