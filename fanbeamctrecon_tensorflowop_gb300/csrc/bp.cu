// Pixel-driven fan-beam backprojection (unweighted BP and 1/L^2-weighted FBP /
// FDK-2D) and its transpose.
//
// Per pixel centre (x, y) inside the FOV disc and view beta, with
// c = -cos(beta), s = -sin(beta):
//   U = R + x c + y s,  t = -x s + y c,  col = (atan(t/U) - left)/dcol + shift,
// and when 0 < col < n_cols the pixel gains the linearly interpolated,
// clamped detector value at col (texel centres at +1/2), times 1/(U^2+t^2) in
// the weighted form (BP/transform.cu:76-92, FBP/transform.cu:70-87,
// FDK/GPURecon_GPU.cu:25-49).  One launch covers all views and slices; each
// thread keeps four pixels of a 32x32 tile in registers across all views, so
// the image is written once instead of read-modified-written per view.
#include "common.cuh"

namespace ctk {
namespace {

constexpr int kTile = 32;      // tile edge (pixels)
constexpr int kRowsPerThr = 4;  // 32x8 threads cover 32x32 pixels

struct BpArgs {
    int V, C, nx, ny;
    float xmin, ymin, dx, dy;
    float R, left, dcol, shift;
    double fov_r2;
};

template <bool WEIGHTED>
__global__ void __launch_bounds__(256)
    bp_fan_kernel(const float *__restrict__ sino, float *__restrict__ img,
                  const float2 *__restrict__ view_cs, BpArgs a, int batch) {
    const int ix = blockIdx.x * kTile + threadIdx.x;
    const int iy0 = blockIdx.y * kTile + threadIdx.y;
    const int b = blockIdx.z;
    if (b >= batch) return;
    float px = 0.f, py[kRowsPerThr];
    bool in[kRowsPerThr];
    const double xd = (double)a.xmin + (double)a.dx * (ix + 0.5);
    px = (float)xd;
    bool any = false;
#pragma unroll
    for (int k = 0; k < kRowsPerThr; ++k) {
        const int iy = iy0 + 8 * k;
        const double yd = (double)a.ymin + (double)a.dy * (iy + 0.5);
        py[k] = (float)yd;
        in[k] = ix < a.nx && iy < a.ny && (xd * xd + yd * yd <= a.fov_r2);
        any |= in[k];
    }
    float acc[kRowsPerThr] = {0.f, 0.f, 0.f, 0.f};
    if (__syncthreads_or(any)) {
        const float *sb = sino + (size_t)b * a.V * a.C;
        const float fC = (float)a.C;
        for (int v = 0; v < a.V; ++v) {
            const float2 cs = __ldg(view_cs + v);
            const float *row = sb + (size_t)v * a.C;
#pragma unroll
            for (int k = 0; k < kRowsPerThr; ++k) {
                const float U = a.R + px * cs.x + py[k] * cs.y;
                const float t = -px * cs.y + py[k] * cs.x;
                const float col = (atanf(t / U) - a.left) / a.dcol + a.shift;
                if (in[k] && col > 0.0f && col < fC) {
                    const float cb = col - 0.5f;
                    const float fi = floorf(cb);
                    const float f = cb - fi;
                    const int i = (int)fi;
                    const int i0 = max(i, 0), i1 = min(i + 1, a.C - 1);
                    const float v0 = __ldg(row + i0), v1 = __ldg(row + i1);
                    const float val = fmaf(f, v1 - v0, v0);
                    if (WEIGHTED)
                        acc[k] = fmaf(val, 1.0f / (U * U + t * t), acc[k]);
                    else
                        acc[k] += val;
                }
            }
        }
    }
    float *ib = img + (size_t)b * a.nx * a.ny;
#pragma unroll
    for (int k = 0; k < kRowsPerThr; ++k) {
        const int iy = iy0 + 8 * k;
        if (ix < a.nx && iy < a.ny) ib[(size_t)iy * a.nx + ix] = acc[k];
    }
}

// Transpose of bp_fan_kernel: each pixel-view scatters x * weight * (1-f, f)
// onto the two clamped detector taps with global atomics.
template <bool WEIGHTED>
__global__ void __launch_bounds__(256)
    bp_fan_transpose_kernel(const float *__restrict__ img, float *__restrict__ sino,
                            const float2 *__restrict__ view_cs, BpArgs a, int batch) {
    const int ix = blockIdx.x * kTile + threadIdx.x;
    const int iy0 = blockIdx.y * kTile + threadIdx.y;
    const int b = blockIdx.z;
    if (b >= batch) return;
    const float *ib = img + (size_t)b * a.nx * a.ny;
    const double xd = (double)a.xmin + (double)a.dx * (ix + 0.5);
    const float px = (float)xd;
    float py[kRowsPerThr], xv[kRowsPerThr];
    bool any = false;
#pragma unroll
    for (int k = 0; k < kRowsPerThr; ++k) {
        const int iy = iy0 + 8 * k;
        const double yd = (double)a.ymin + (double)a.dy * (iy + 0.5);
        py[k] = (float)yd;
        const bool in = ix < a.nx && iy < a.ny && (xd * xd + yd * yd <= a.fov_r2);
        xv[k] = in ? ib[(size_t)iy * a.nx + ix] : 0.0f;
        any |= (xv[k] != 0.0f);
    }
    if (!__syncthreads_or(any)) return;
    float *sb = sino + (size_t)b * a.V * a.C;
    const float fC = (float)a.C;
    for (int v = 0; v < a.V; ++v) {
        const float2 cs = __ldg(view_cs + v);
        float *row = sb + (size_t)v * a.C;
#pragma unroll
        for (int k = 0; k < kRowsPerThr; ++k) {
            if (xv[k] == 0.0f) continue;
            const float U = a.R + px * cs.x + py[k] * cs.y;
            const float t = -px * cs.y + py[k] * cs.x;
            const float col = (atanf(t / U) - a.left) / a.dcol + a.shift;
            if (col > 0.0f && col < fC) {
                const float cb = col - 0.5f;
                const float fi = floorf(cb);
                const float f = cb - fi;
                const int i = (int)fi;
                const int i0 = max(i, 0), i1 = min(i + 1, a.C - 1);
                float val = xv[k];
                if (WEIGHTED) val *= 1.0f / (U * U + t * t);
                atomicAdd(row + i0, val * (1.0f - f));
                atomicAdd(row + i1, val * f);
            }
        }
    }
}

BpArgs make_args(const ct_plan *p) {
    BpArgs a;
    a.V = p->g.n_views;
    a.C = p->g.n_cols;
    a.nx = p->g.nx;
    a.ny = p->g.ny;
    a.xmin = p->g.xmin;
    a.ymin = p->g.ymin;
    a.dx = p->g.dx;
    a.dy = p->g.dy;
    a.R = p->g.sid;
    a.left = p->g.left;
    a.dcol = p->g.dcol;
    a.shift = p->g.shift;
    a.fov_r2 = (double)p->g.rfov * (double)p->g.rfov;
    return a;
}

}  // namespace

int bp_fan(const ct_plan *p, const float *sino, float *img, int batch, int weighted,
           void *stream) {
    const BpArgs a = make_args(p);
    const float2 *vcs = reinterpret_cast<const float2 *>(p->d_view_cs);
    cudaStream_t s = (cudaStream_t)stream;
    for (int b0 = 0; b0 < batch; b0 += 65535) {
        const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
        dim3 grid((a.nx + kTile - 1) / kTile, (a.ny + kTile - 1) / kTile, nb);
        dim3 block(kTile, 8, 1);
        const float *sp = sino + (size_t)b0 * a.V * a.C;
        float *ip = img + (size_t)b0 * a.nx * a.ny;
        if (weighted)
            bp_fan_kernel<true><<<grid, block, 0, s>>>(sp, ip, vcs, a, nb);
        else
            bp_fan_kernel<false><<<grid, block, 0, s>>>(sp, ip, vcs, a, nb);
        ct_count_launch();
    }
    return (int)cudaGetLastError();
}

int bp_fan_transpose(const ct_plan *p, const float *img, float *sino, int batch, int weighted,
                     void *stream) {
    const BpArgs a = make_args(p);
    const float2 *vcs = reinterpret_cast<const float2 *>(p->d_view_cs);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(sino, 0, sizeof(float) * (size_t)batch * a.V * a.C, s);
    if (e != cudaSuccess) return (int)e;
    for (int b0 = 0; b0 < batch; b0 += 65535) {
        const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
        dim3 grid((a.nx + kTile - 1) / kTile, (a.ny + kTile - 1) / kTile, nb);
        dim3 block(kTile, 8, 1);
        const float *ip = img + (size_t)b0 * a.nx * a.ny;
        float *sp = sino + (size_t)b0 * a.V * a.C;
        if (weighted)
            bp_fan_transpose_kernel<true><<<grid, block, 0, s>>>(ip, sp, vcs, a, nb);
        else
            bp_fan_transpose_kernel<false><<<grid, block, 0, s>>>(ip, sp, vcs, a, nb);
        ct_count_launch();
    }
    return (int)cudaGetLastError();
}

}  // namespace ctk
