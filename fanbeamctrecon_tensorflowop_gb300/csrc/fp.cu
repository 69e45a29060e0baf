// Ray-driven fan-beam forward projector (its transpose is in fp_adjoint.cu).
//
// Forward (replaces FP/transform.cu:103-146 and the per-view launch loop
// :162-169): all views and slices in one launch.  Each launch first builds
// "quad images" (per slice and layout, a float4 of the four clamped bilinear
// taps of every cell), then fp_warp (fp_body.cuh) walks 32 adjacent rays of a
// view per warp, row-synchronously, summing each cell's samples in closed
// form (cellwalk.cuh): one 16-byte gather per cell instead of four per
// sample.  Up to 16 slices share one walk.  Output:
// p = 0.125*dx * sum_k bilinear_clamp(img, start + k*step), k < n.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <vector>

#include "cellwalk.cuh"
#include "fp_body.cuh"

namespace ctk {
namespace {

// A block is one 32-channel group of kFpViews adjacent views (their rays
// cross nearly the same cells, so the block's warps share L1 lines), and
// blocks run channel-group-major: the warps resident at any time cover a few
// channel groups of every view.  Against 8 channel groups of one view per
// 256-thread block, in view order: 11.04 -> 8.72 ms per 32 clinical slices
// (2 views per block 8.74, 8 views 8.97, 16 views 9.27; 1 view, channel-major
// alone 8.87).  The plan's order table (fp_block_order) then runs the blocks
// whose rays walk the transposed layout after the others, so the resident
// warps read one layout's quad images at a time (8.73 -> 8.56 ms).
constexpr int kFpViews = 4;
constexpr int kFpThreads = 32 * kFpViews;
constexpr int kFpChunk = 64;  // slices per quad-workspace chunk
#ifndef CT_FP_MIN_BLOCKS
#define CT_FP_MIN_BLOCKS 4
#endif
#ifndef CT_FP_MAX_SB
#define CT_FP_MAX_SB 16
#endif

// Builds both quad layouts of nz slices (grid: 32 x 32-quad tiles x slices).
// A block stages the tile's 33 x 33 clamped texels in shared memory with
// coalesced reads, then writes the tile's quads of layout 0 (rows of quads
// along x) and of layout 1 (the transposed image, rows along y), both
// coalesced; the values are build_quad's (fp_body.cuh).  The former
// one-quad-per-thread form read the transposed layout's taps down image
// columns: 0.147 ms per 32 clinical slices.
__global__ void __launch_bounds__(256)
    build_quads_kernel(const float *__restrict__ img, float4 *__restrict__ quads, int nx, int ny) {
    __shared__ float t[33][33];
    const int Q = nx + 1;
    const int TX = blockIdx.x * 32, TY = blockIdx.y * 32, b = blockIdx.z;
    const float *im = img + (size_t)b * nx * ny;
    // texel (TX - 1 + xx, TY - 1 + yy), clamped to the image
    for (int k = threadIdx.y * 32 + threadIdx.x; k < 33 * 33; k += 256) {
        const int yy = k / 33, xx = k - yy * 33;
        const int x = min(max(TX - 1 + xx, 0), nx - 1), y = min(max(TY - 1 + yy, 0), ny - 1);
        t[yy][xx] = __ldg(im + (size_t)y * nx + x);
    }
    __syncthreads();
    const int i = threadIdx.x;
    float4 *q0 = quads + (size_t)b * 2 * Q * Q, *q1 = q0 + (size_t)Q * Q;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int j = threadIdx.y + 8 * r;
        // layout 0: quad (TX + i, TY + j) = cell (TX - 1 + i, TY - 1 + j)
        if (TX + i < Q && TY + j < Q)
            q0[(size_t)(TY + j) * Q + TX + i] =
                make_float4(t[j][i], t[j][i + 1], t[j + 1][i], t[j + 1][i + 1]);
        // layout 1: quad (TY + i, TX + j) = cell (u, v) = (TY - 1 + i, TX - 1 + j), u along y
        if (TY + i < Q && TX + j < Q)
            q1[(size_t)(TX + j) * Q + TY + i] =
                make_float4(t[i][j], t[i + 1][j], t[i][j + 1], t[i + 1][j + 1]);
    }
}

template <int SB>
__global__ void __launch_bounds__(kFpThreads, CT_FP_MIN_BLOCKS)
    fp_fan_kernel(const float4 *__restrict__ quads, float *__restrict__ sino,
                  const float4 *__restrict__ ray, const int *__restrict__ nsamp,
                  const int *__restrict__ order, int V, int C, int wpv, int nx, float w,
                  int batch, int max_iter) {
    const int nvg = (V + kFpViews - 1) / kFpViews;
    const int bid = __ldg(order + blockIdx.x);
    const int cgroup = bid / nvg, vgroup = bid - cgroup * nvg;
    const int v = vgroup * kFpViews + (threadIdx.x >> 5);
    if (v >= V) return;  // warp-uniform
    const int gw = v * wpv + cgroup;
    const int b0 = blockIdx.y * SB;
    const size_t lsz = (size_t)(nx + 1) * (nx + 1);
    // slices beyond the batch read slice b0's quads (results dropped)
    fp_warp<SB, float>(quads + (size_t)b0 * 2 * lsz, 2 * lsz, sino + (size_t)b0 * V * C,
                       (size_t)V * C, ray, nsamp, V, C, wpv, nx, w, min(SB, batch - b0),
                       max_iter, gw);
}

}  // namespace

std::vector<int32_t> fp_block_order(int V, int C, const std::vector<float> &ray,
                                    const std::vector<int32_t> &nsamp) {
    const int wpv = (C + 31) / 32, nvg = (V + kFpViews - 1) / kFpViews;
    const int blocks = nvg * wpv;
    std::vector<int32_t> order(blocks);
    std::vector<char> transposed(blocks);
    for (int b = 0; b < blocks; ++b) {
        const int cg = b / nvg, vg = b - cg * nvg;
        int along_x = 0, valid = 0;
        for (int v = vg * kFpViews; v < std::min(V, (vg + 1) * kFpViews); ++v)
            for (int c = cg * 32; c < std::min(C, (cg + 1) * 32); ++c) {
                const size_t r = (size_t)v * C + c;
                if (nsamp[r] <= 0) continue;
                ++valid;
                // the warps' vote (fp_body.cuh): |step x| > |step y| walks the transposed layout
                along_x += std::fabs(ray[4 * r + 2]) > std::fabs(ray[4 * r + 3]);
            }
        transposed[b] = 2 * along_x > valid;
        order[b] = b;
    }
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t x, int32_t y) { return transposed[x] < transposed[y]; });
    return order;
}

size_t fp_fan_work_bytes(const ct_plan *p, int batch) {
    const size_t q = (size_t)(p->g.nx + 1) * (p->g.nx + 1);
    const size_t chunk = batch < kFpChunk ? (size_t)batch : (size_t)kFpChunk;
    return chunk * 2 * q * sizeof(float4);
}

int fp_fan(const ct_plan *p, const float *img, float *sino, int batch, void *work,
           void *stream) {
    const int V = p->g.n_views, C = p->g.n_cols;
    const int nx = p->g.nx, ny = p->g.ny;
    const int max_iter = 2 * (nx > ny ? nx : ny) + 8;
    const size_t plane = (size_t)nx * ny;
    const size_t n_rays = (size_t)V * C;
    const float4 *ray = reinterpret_cast<const float4 *>(p->d_ray);
    float4 *quads = static_cast<float4 *>(work);
    cudaStream_t s = (cudaStream_t)stream;
    const int wpv = (C + 31) / 32;
    const int blocks = (V + kFpViews - 1) / kFpViews * wpv;
    const int Q = nx + 1;
    // chunks of at most kFpChunk slices share the quad workspace
    for (int c0 = 0; c0 < batch; c0 += kFpChunk) {
        const int nb = batch - c0 < kFpChunk ? batch - c0 : kFpChunk;
        build_quads_kernel<<<dim3((Q + 31) / 32, (Q + 31) / 32, nb), dim3(32, 8), 0, s>>>(
            img + (size_t)c0 * plane, quads, nx, ny);
        ct_count_launch();
        float *out = sino + (size_t)c0 * n_rays;
        int b = 0;
        if (CT_FP_MAX_SB >= 16 && nb >= 16) {
            const int n16 = nb / 16 * 16;
            fp_fan_kernel<16><<<dim3(blocks, n16 / 16), kFpThreads, 0, s>>>(
                quads, out, ray, p->d_nsamp, p->d_fp_order, V, C, wpv, nx, p->fp_weight, n16,
                max_iter);
            ct_count_launch();
            b = n16;
        }
        if (nb - b >= 8) {
            const int n8 = (nb - b) / 8 * 8;
            fp_fan_kernel<8><<<dim3(blocks, n8 / 8), kFpThreads, 0, s>>>(
                quads + (size_t)b * 2 * Q * Q, out + (size_t)b * n_rays, ray, p->d_nsamp,
                p->d_fp_order, V, C, wpv, nx, p->fp_weight, n8, max_iter);
            ct_count_launch();
            b += n8;
        }
        if (nb - b >= 4) {
            fp_fan_kernel<4><<<dim3(blocks, 1), kFpThreads, 0, s>>>(
                quads + (size_t)b * 2 * Q * Q, out + (size_t)b * n_rays, ray, p->d_nsamp,
                p->d_fp_order, V, C, wpv, nx, p->fp_weight, 4, max_iter);
            ct_count_launch();
            b += 4;
        }
        if (nb > b) {
            fp_fan_kernel<1><<<dim3(blocks, nb - b), kFpThreads, 0, s>>>(
                quads + (size_t)b * 2 * Q * Q, out + (size_t)b * n_rays, ray, p->d_nsamp,
                p->d_fp_order, V, C, wpv, nx, p->fp_weight, nb - b, max_iter);
            ct_count_launch();
        }
    }
    return (int)cudaGetLastError();
}

}  // namespace ctk
