// Ray-driven fan-beam forward projector and its exact transpose.
//
// Forward (replaces FP/transform.cu:103-146 and the per-view launch loop
// :162-169): one warp per ray; lane l takes samples l, l+32, ... of the ray,
// p = 0.125*dx * sum_k bilinear_clamp(img, start + k*step), k < n.  All views
// and all slices of the batch run in one launch; the ray table (start, step, n)
// comes from the plan (FP64-derived on the host).
//
// Transpose: the same samples, each spreading w*y[ray] times its four bilinear
// weights onto the (clamped) taps.  Consecutive samples of a ray usually fall
// in the same bilinear cell, so each lane walks a contiguous run of samples,
// sums the weights per cell and issues four global atomic adds per cell visit.
#include "common.cuh"

namespace ctk {
namespace {

constexpr int kFpWarps = 8;  // rays per 256-thread block

__global__ void __launch_bounds__(kFpWarps * 32)
    fp_fan_kernel(const float *__restrict__ img, float *__restrict__ sino,
                  const float4 *__restrict__ ray, const int *__restrict__ nsamp, int n_rays,
                  int nx, int ny, float w, int batch) {
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * kFpWarps + (threadIdx.x >> 5);
    if (r >= n_rays) return;
    const int n = __ldg(nsamp + r);
    const float4 q = __ldg(ray + r);
    for (int b = blockIdx.y; b < batch; b += gridDim.y) {
        const float *im = img + (size_t)b * nx * ny;
        float acc = 0.0f;
        for (int k = lane; k < n; k += 32) {
            const float fk = static_cast<float>(k);
            acc += bilerp_clamp(im, nx, ny, fmaf(fk, q.z, q.x), fmaf(fk, q.w, q.y));
        }
        acc = warp_sum(acc);
        if (lane == 0) sino[(size_t)b * n_rays + r] = acc * w;
    }
}

__device__ __forceinline__ void flush_cell(float *__restrict__ im, int nx, int ny, int i, int j,
                                           float val, float w00, float w10, float w01,
                                           float w11) {
    const int i0 = min(max(i, 0), nx - 1), i1 = min(max(i + 1, 0), nx - 1);
    const int j0 = min(max(j, 0), ny - 1), j1 = min(max(j + 1, 0), ny - 1);
    if (w00 != 0.0f) atomicAdd(im + j0 * nx + i0, val * w00);
    if (w10 != 0.0f) atomicAdd(im + j0 * nx + i1, val * w10);
    if (w01 != 0.0f) atomicAdd(im + j1 * nx + i0, val * w01);
    if (w11 != 0.0f) atomicAdd(im + j1 * nx + i1, val * w11);
}

__global__ void __launch_bounds__(kFpWarps * 32)
    fp_fan_adjoint_kernel(const float *__restrict__ sino, float *__restrict__ img,
                          const float4 *__restrict__ ray, const int *__restrict__ nsamp,
                          int n_rays, int nx, int ny, float w, int batch) {
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * kFpWarps + (threadIdx.x >> 5);
    if (r >= n_rays) return;
    const int n = __ldg(nsamp + r);
    if (n == 0) return;
    const float4 q = __ldg(ray + r);
    const int chunk = (n + 31) >> 5;
    const int k0 = lane * chunk, k1 = min(n, k0 + chunk);
    for (int b = blockIdx.y; b < batch; b += gridDim.y) {
        const float val = __ldg(sino + (size_t)b * n_rays + r) * w;
        if (val == 0.0f) continue;  // contributes exactly nothing
        float *im = img + (size_t)b * nx * ny;
        int ci = 0, cj = 0;
        bool have = false;
        float w00 = 0.f, w10 = 0.f, w01 = 0.f, w11 = 0.f;
        for (int k = k0; k < k1; ++k) {
            const float fk = static_cast<float>(k);
            const float xb = fmaf(fk, q.z, q.x) - 0.5f, yb = fmaf(fk, q.w, q.y) - 0.5f;
            const float fx = floorf(xb), fy = floorf(yb);
            const float ax = xb - fx, ay = yb - fy;
            const int i = static_cast<int>(fx), j = static_cast<int>(fy);
            if (!have || i != ci || j != cj) {
                if (have) flush_cell(im, nx, ny, ci, cj, val, w00, w10, w01, w11);
                ci = i;
                cj = j;
                have = true;
                w00 = w10 = w01 = w11 = 0.f;
            }
            const float bx = 1.0f - ax, by = 1.0f - ay;
            w00 = fmaf(bx, by, w00);
            w10 = fmaf(ax, by, w10);
            w01 = fmaf(bx, ay, w01);
            w11 = fmaf(ax, ay, w11);
        }
        if (have) flush_cell(im, nx, ny, ci, cj, val, w00, w10, w01, w11);
    }
}

inline dim3 batch_grid(int blocks_x, int batch) {
    return dim3(blocks_x, batch < 65535 ? batch : 65535, 1);
}

}  // namespace

int fp_fan(const ct_plan *p, const float *img, float *sino, int batch, void *stream) {
    const int n_rays = p->g.n_views * p->g.n_cols;
    const int bx = (n_rays + kFpWarps - 1) / kFpWarps;
    fp_fan_kernel<<<batch_grid(bx, batch), kFpWarps * 32, 0, (cudaStream_t)stream>>>(
        img, sino, reinterpret_cast<const float4 *>(p->d_ray), p->d_nsamp, n_rays, p->g.nx,
        p->g.ny, p->fp_weight, batch);
    ct_count_launch();
    return (int)cudaGetLastError();
}

int fp_fan_adjoint(const ct_plan *p, const float *sino, float *img, int batch, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(img, 0, sizeof(float) * (size_t)batch * p->g.nx * p->g.ny, s);
    if (e != cudaSuccess) return (int)e;
    const int n_rays = p->g.n_views * p->g.n_cols;
    const int bx = (n_rays + kFpWarps - 1) / kFpWarps;
    fp_fan_adjoint_kernel<<<batch_grid(bx, batch), kFpWarps * 32, 0, s>>>(
        sino, img, reinterpret_cast<const float4 *>(p->d_ray), p->d_nsamp, n_rays, p->g.nx,
        p->g.ny, p->fp_weight, batch);
    ct_count_launch();
    return (int)cudaGetLastError();
}

}  // namespace ctk
