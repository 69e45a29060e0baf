// The plain per-slice, per-view launch loop: the reference's execution
// structure (FP/transform.cu:162-169, BP/transform.cu:110-119) rebuilt on the
// same GPU with explicit FP32 lerp, because CUDA 13 no longer compiles the
// reference's texture references.  For every slice and every view one kernel
// is launched and the stream is synchronised before the next view, exactly as
// the reference's cudaDeviceSynchronize after each launch.  It exists only as
// the measured comparison for the fused operators.
#include "common.cuh"

namespace ctk {
namespace {

constexpr int kPlainThreads = 256;  // threadsPerBlockRayTrace (FP/transform.cu:11)

// One block per ray, threads stride the samples, shared-memory tree reduction
// (the shape of RayTrace_ReconImage_OneView_kernel, FP/transform.cu:103-146).
__global__ void __launch_bounds__(kPlainThreads)
    plain_fp_view_kernel(const float *__restrict__ im, float *__restrict__ out,
                         const float4 *__restrict__ ray, const int *__restrict__ nsamp, int nx,
                         int ny, float w) {
    __shared__ float cache[kPlainThreads];
    const int c = blockIdx.x;
    const int n = nsamp[c];
    const float4 q = ray[c];
    float acc = 0.0f;
    for (int k = threadIdx.x; k < n; k += kPlainThreads) {
        const float fk = (float)k;
        acc += bilerp_clamp(im, nx, ny, fmaf(fk, q.z, q.x), fmaf(fk, q.w, q.y));
    }
    cache[threadIdx.x] = acc;
    __syncthreads();
    for (int h = kPlainThreads / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) cache[threadIdx.x] += cache[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[c] = cache[0] * w;
}

// Transpose of one view: each sample scatters its four weights with atomics.
__global__ void __launch_bounds__(kPlainThreads)
    plain_fp_adjoint_view_kernel(const float *__restrict__ sino_v, float *__restrict__ im,
                                 const float4 *__restrict__ ray, const int *__restrict__ nsamp,
                                 int nx, int ny, float w) {
    const int c = blockIdx.x;
    const int n = nsamp[c];
    const float val = sino_v[c] * w;
    if (val == 0.0f) return;
    const float4 q = ray[c];
    for (int k = threadIdx.x; k < n; k += kPlainThreads) {
        const float fk = (float)k;
        const float xb = fmaf(fk, q.z, q.x) - 0.5f, yb = fmaf(fk, q.w, q.y) - 0.5f;
        const float fx = floorf(xb), fy = floorf(yb);
        const float ax = xb - fx, ay = yb - fy;
        const int i = (int)fx, j = (int)fy;
        const int i0 = min(max(i, 0), nx - 1), i1 = min(max(i + 1, 0), nx - 1);
        const int j0 = min(max(j, 0), ny - 1), j1 = min(max(j + 1, 0), ny - 1);
        atomicAdd(im + j0 * nx + i0, val * (1.f - ax) * (1.f - ay));
        atomicAdd(im + j0 * nx + i1, val * ax * (1.f - ay));
        atomicAdd(im + j1 * nx + i0, val * (1.f - ax) * ay);
        atomicAdd(im + j1 * nx + i1, val * ax * ay);
    }
}

// One view of the unweighted BP, read-modify-writing the image
// (BackProjOneView_fan_curve_kernel, BP/transform.cu:67-95).
__global__ void plain_bp_view_kernel(const float *__restrict__ row, float *__restrict__ im, int C,
                                     int nx, int ny, float xmin, float ymin, float dx, float dy,
                                     float R, float left, float dcol, float shift, float sa,
                                     float ca, double fov_r2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= nx || j >= ny) return;
    const double xd = (double)xmin + (double)dx * (i + 0.5);
    const double yd = (double)ymin + (double)dy * (j + 0.5);
    if (!(xd * xd + yd * yd <= fov_r2)) return;
    const float x = (float)xd, y = (float)yd;
    const float U = R + x * ca + y * sa;
    const float t = -x * sa + y * ca;
    const float col = (atanf(t / U) - left) / dcol + shift;
    if (col > 0.0f && col < (float)C) {
        const float cb = col - 0.5f;
        const float fi = floorf(cb);
        const float f = cb - fi;
        const int k = (int)fi;
        const int k0 = max(k, 0), k1 = min(k + 1, C - 1);
        im[j * nx + i] += fmaf(f, row[k1] - row[k0], row[k0]);
    }
}

}  // namespace

int plain_fp_fan(const ct_plan *p, const float *img, float *sino, int batch, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    const int V = p->g.n_views, C = p->g.n_cols, nx = p->g.nx, ny = p->g.ny;
    const float4 *ray = reinterpret_cast<const float4 *>(p->d_ray);
    for (int b = 0; b < batch; ++b) {
        for (int v = 0; v < V; ++v) {
            plain_fp_view_kernel<<<C, kPlainThreads, 0, s>>>(
                img + (size_t)b * nx * ny, sino + ((size_t)b * V + v) * C, ray + (size_t)v * C,
                p->d_nsamp + (size_t)v * C, nx, ny, p->fp_weight);
            ct_count_launch();
            cudaError_t e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return (int)e;
        }
    }
    return (int)cudaGetLastError();
}

int plain_fp_fan_adjoint(const ct_plan *p, const float *sino, float *img, int batch,
                         void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    const int V = p->g.n_views, C = p->g.n_cols, nx = p->g.nx, ny = p->g.ny;
    const float4 *ray = reinterpret_cast<const float4 *>(p->d_ray);
    for (int b = 0; b < batch; ++b) {
        cudaError_t e = cudaMemsetAsync(img + (size_t)b * nx * ny, 0, sizeof(float) * nx * ny, s);
        if (e != cudaSuccess) return (int)e;
        for (int v = 0; v < V; ++v) {
            plain_fp_adjoint_view_kernel<<<C, kPlainThreads, 0, s>>>(
                sino + ((size_t)b * V + v) * C, img + (size_t)b * nx * ny, ray + (size_t)v * C,
                p->d_nsamp + (size_t)v * C, nx, ny, p->fp_weight);
            ct_count_launch();
            e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return (int)e;
        }
    }
    return (int)cudaGetLastError();
}

int plain_bp_fan(const ct_plan *p, const float *sino, float *img, int batch, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    const ct_fan_geom &g = p->g;
    const int V = g.n_views, C = g.n_cols, nx = g.nx, ny = g.ny;
    const double fov_r2 = (double)g.rfov * (double)g.rfov;
    // The per-view angle terms are kernel arguments, as in the reference
    // (BP/transform.cu:116), taken from the plan's FP64-derived host table.
    const std::vector<float> &cs = p->h_view_cs;
    cudaError_t e;
    dim3 block(32, 32, 1);
    dim3 grid((nx + 31) / 32, (ny + 31) / 32, 1);
    for (int b = 0; b < batch; ++b) {
        float *im = img + (size_t)b * nx * ny;
        e = cudaMemsetAsync(im, 0, sizeof(float) * nx * ny, s);
        if (e != cudaSuccess) return (int)e;
        for (int v = 0; v < V; ++v) {
            plain_bp_view_kernel<<<grid, block, 0, s>>>(
                sino + ((size_t)b * V + v) * C, im, C, nx, ny, g.xmin, g.ymin, g.dx, g.dy, g.sid,
                g.left, g.dcol, g.shift, cs[2 * v + 1], cs[2 * v + 0], fov_r2);
            ct_count_launch();
            e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return (int)e;
        }
    }
    return (int)cudaGetLastError();
}

}  // namespace ctk
