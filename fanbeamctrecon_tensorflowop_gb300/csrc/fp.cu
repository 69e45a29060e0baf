// Ray-driven fan-beam forward projector and its exact transpose.
//
// Forward (replaces FP/transform.cu:103-146 and the per-view launch loop
// :162-169): one thread per ray, all views and slices in one launch.  The
// thread walks the bilinear cells its ray crosses and adds each cell's
// samples in closed form (cellwalk.cuh), so the image is read once per cell
// instead of four times per sample; SB slices share one walk.  Output:
// p = 0.125*dx * sum_k bilinear_clamp(img, start + k*step), k < n.
//
// Transpose: one block per 32x32 image tile and slice keeps the tile in
// shared memory.  For every view it takes the rays that can reach the tile,
// clips each ray's samples to the tile's cells (plus the one-cell halo whose
// taps touch the tile), walks those cells and adds val*W to the taps the
// tile owns.  Every pixel is written exactly once; there are no global
// atomics.
#include <cfloat>

#include "cellwalk.cuh"

namespace ctk {
namespace {

constexpr int kFpThreads = 256;

template <int SB>
__global__ void __launch_bounds__(kFpThreads)
    fp_fan_kernel(const float *__restrict__ img, float *__restrict__ sino,
                  const float4 *__restrict__ ray, const int *__restrict__ nsamp, int n_rays,
                  int nx, int ny, float w, int batch, int max_iter) {
    const int r = blockIdx.x * kFpThreads + threadIdx.x;
    if (r >= n_rays) return;
    const int b0 = blockIdx.y * SB;
    const int n = __ldg(nsamp + r);
    const size_t plane = (size_t)nx * ny;
    float acc[SB];
#pragma unroll
    for (int s = 0; s < SB; ++s) acc[s] = 0.0f;
    if (n > 0) {
        const float4 q = __ldg(ray + r);
        const RaySeg seg{q.x - 0.5f, q.y - 0.5f, q.z, q.w};
        const float *im[SB];
#pragma unroll
        for (int s = 0; s < SB; ++s) im[s] = img + (size_t)min(b0 + s, batch - 1) * plane;
        walk_cells(seg, 0.0f, (float)n, max_iter,
                   [&](int cu, int cv, float cnt, float a, float b) {
                       const CellWeights cw = cell_weights(cnt, a, b, seg.su, seg.sv);
                       // clamp-to-edge taps (for nx != ny the FOV circle, of
                       // radius nx/2 in both axes, can leave the image rows)
                       const int i0 = min(max(cu, 0), nx - 1), i1 = min(max(cu + 1, 0), nx - 1);
                       const int r0 = min(max(cv, 0), ny - 1) * nx;
                       const int r1 = min(max(cv + 1, 0), ny - 1) * nx;
#pragma unroll
                       for (int s = 0; s < SB; ++s) {
                           const float *p = im[s];
                           float v = cw.w00 * __ldg(p + r0 + i0);
                           v = fmaf(cw.w10, __ldg(p + r0 + i1), v);
                           v = fmaf(cw.w01, __ldg(p + r1 + i0), v);
                           v = fmaf(cw.w11, __ldg(p + r1 + i1), v);
                           acc[s] += v;
                       }
                   });
    }
#pragma unroll
    for (int s = 0; s < SB; ++s)
        if (b0 + s < batch) sino[(size_t)(b0 + s) * n_rays + r] = acc[s] * w;
}

// ---- transpose ----------------------------------------------------------------

constexpr int kTile = 32;
constexpr int kAdjThreads = 256;

struct AdjArgs {
    int V, C, nx, ny;
    float w;          // 0.125*dx
    float src;        // R (mm)
    float dx;         // pixel pitch used by the ray table (mm)
    float fov_px;     // rfov/dx: texture coordinate of the isocentre
    float left, dcol; // detector (rad)
    int max_iter;
};

// Channel coordinate (channel i centred at i) of world point (X, Y) in a view
// with c = -cos(beta), s = -sin(beta): gamma = atan2(t, U).
__device__ __forceinline__ float channel_of(const AdjArgs &a, float c, float s, float X,
                                            float Y) {
    const float U = a.src + X * c + Y * s;
    const float t = -X * s + Y * c;
    return (atan2f(t, U) - a.left) / a.dcol - 0.5f;
}

__global__ void __launch_bounds__(kAdjThreads)
    fp_fan_adjoint_tile_kernel(const float *__restrict__ sino, float *__restrict__ img,
                               const float4 *__restrict__ ray, const int *__restrict__ nsamp,
                               const float2 *__restrict__ view_cs, AdjArgs a, int batch) {
    __shared__ float acc[kTile][kTile + 1];
    const int X0 = blockIdx.x * kTile, Y0 = blockIdx.y * kTile;
    const int b = blockIdx.z;
    if (b >= batch) return;
    for (int k = threadIdx.x; k < kTile * (kTile + 1); k += kAdjThreads) (&acc[0][0])[k] = 0.0f;
    // Cells whose taps touch owned pixels: cu in [X0-1, X0+kTile-1]; in cell
    // coordinates the box is u in [X0-1, X0+kTile), v likewise.  Tiles on the
    // image border also own the clamped taps of cells beyond it, so their box
    // reaches the edge of the FOV disc (u, v in [-1/2, 2*fov_px - 1/2]).
    const float far = fmaxf((float)max(a.nx, a.ny), 2.0f * a.fov_px) + 2.0f;
    const float Ulo = X0 == 0 ? -2.0f : (float)(X0 - 1);
    const float Uhi = X0 + kTile >= a.nx ? far : (float)(X0 + kTile);
    const float Vlo = Y0 == 0 ? -2.0f : (float)(Y0 - 1);
    const float Vhi = Y0 + kTile >= a.ny ? far : (float)(Y0 + kTile);
    // Skip tiles whose box misses the FOV disc (centre fov_px - 1/2, radius fov_px).
    const float cx = a.fov_px - 0.5f;
    const float qx = fminf(fmaxf(cx, Ulo), Uhi) - cx, qy = fminf(fmaxf(cx, Vlo), Vhi) - cx;
    const bool live = qx * qx + qy * qy <= a.fov_px * a.fov_px * 1.0001f;
    __syncthreads();
    if (live) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const float *sb = sino + (size_t)b * a.V * a.C;
        for (int v = warp; v < a.V; v += kAdjThreads / 32) {
            // channel range of the rays that can reach the box, from its corners
            const float2 cs = __ldg(view_cs + v);
            float cmin = FLT_MAX, cmax = -FLT_MAX;
            if (lane < 4) {
                const float uc = (lane & 1) ? Uhi : Ulo, vc = (lane & 2) ? Vhi : Vlo;
                const float X = (uc + 0.5f - a.fov_px) * a.dx, Y = (vc + 0.5f - a.fov_px) * a.dx;
                cmin = cmax = channel_of(a, cs.x, cs.y, X, Y);
            }
#pragma unroll
            for (int o = 2; o > 0; o >>= 1) {
                cmin = fminf(cmin, __shfl_xor_sync(0xffffffffu, cmin, o));
                cmax = fmaxf(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
            }
            cmin = __shfl_sync(0xffffffffu, cmin, 0);
            cmax = __shfl_sync(0xffffffffu, cmax, 0);
            const int c_lo = max(0, (int)floorf(cmin) - 1);
            const int c_hi = min(a.C - 1, (int)ceilf(cmax) + 1);
            for (int c = c_lo + lane; c <= c_hi; c += 32) {
                const int r = v * a.C + c;
                const int n = __ldg(nsamp + r);
                if (n == 0) continue;
                const float val = __ldg(sb + r) * a.w;
                if (val == 0.0f) continue;
                const float4 q = __ldg(ray + r);
                const RaySeg seg{q.x - 0.5f, q.y - 0.5f, q.z, q.w};
                // samples with u in [Ulo, Uhi) and v in [Vlo, Vhi)
                float klo = 0.0f, khi = (float)n;
                if (seg.su != 0.0f) {
                    const float t0 = (Ulo - seg.u0) / seg.su, t1 = (Uhi - seg.u0) / seg.su;
                    klo = fmaxf(klo, ceilf(fminf(t0, t1)));
                    khi = fminf(khi, ceilf(fmaxf(t0, t1)));
                } else if (!(seg.u0 >= Ulo && seg.u0 < Uhi)) {
                    continue;
                }
                if (seg.sv != 0.0f) {
                    const float t0 = (Vlo - seg.v0) / seg.sv, t1 = (Vhi - seg.v0) / seg.sv;
                    klo = fmaxf(klo, ceilf(fminf(t0, t1)));
                    khi = fminf(khi, ceilf(fmaxf(t0, t1)));
                } else if (!(seg.v0 >= Vlo && seg.v0 < Vhi)) {
                    continue;
                }
                if (!(klo < khi)) continue;
                walk_cells(seg, klo, khi, a.max_iter,
                           [&](int cu, int cv, float cnt, float fa, float fb) {
                               const CellWeights cw = cell_weights(cnt, fa, fb, seg.su, seg.sv);
                               const int i0 = min(max(cu, 0), a.nx - 1) - X0;
                               const int i1 = min(max(cu + 1, 0), a.nx - 1) - X0;
                               const int j0 = min(max(cv, 0), a.ny - 1) - Y0;
                               const int j1 = min(max(cv + 1, 0), a.ny - 1) - Y0;
                               const bool oi0 = (unsigned)i0 < (unsigned)kTile;
                               const bool oi1 = (unsigned)i1 < (unsigned)kTile;
                               const bool oj0 = (unsigned)j0 < (unsigned)kTile;
                               const bool oj1 = (unsigned)j1 < (unsigned)kTile;
                               if (oj0 && oi0) atomicAdd(&acc[j0][i0], val * cw.w00);
                               if (oj0 && oi1) atomicAdd(&acc[j0][i1], val * cw.w10);
                               if (oj1 && oi0) atomicAdd(&acc[j1][i0], val * cw.w01);
                               if (oj1 && oi1) atomicAdd(&acc[j1][i1], val * cw.w11);
                           });
            }
        }
    }
    __syncthreads();
    float *ib = img + (size_t)b * a.nx * a.ny;
    for (int k = threadIdx.x; k < kTile * kTile; k += kAdjThreads) {
        const int jj = k / kTile, ii = k - jj * kTile;
        const int X = X0 + ii, Y = Y0 + jj;
        if (X < a.nx && Y < a.ny) ib[(size_t)Y * a.nx + X] = acc[jj][ii];
    }
}

}  // namespace

int fp_fan(const ct_plan *p, const float *img, float *sino, int batch, void *stream) {
    const int n_rays = p->g.n_views * p->g.n_cols;
    const int bx = (n_rays + kFpThreads - 1) / kFpThreads;
    const int max_iter = 2 * (p->g.nx > p->g.ny ? p->g.nx : p->g.ny) + 8;
    const float4 *ray = reinterpret_cast<const float4 *>(p->d_ray);
    cudaStream_t s = (cudaStream_t)stream;
    // four slices per walk while at least four remain, then one at a time
    const int b4 = batch / 4 * 4;
    for (int b0 = 0; b0 < b4; b0 += 4 * 65535) {
        const int nb = b4 - b0 < 4 * 65535 ? b4 - b0 : 4 * 65535;
        fp_fan_kernel<4><<<dim3(bx, nb / 4), kFpThreads, 0, s>>>(
            img + (size_t)b0 * p->g.nx * p->g.ny, sino + (size_t)b0 * n_rays, ray, p->d_nsamp,
            n_rays, p->g.nx, p->g.ny, p->fp_weight, nb, max_iter);
        ct_count_launch();
    }
    if (batch > b4) {
        fp_fan_kernel<1><<<dim3(bx, batch - b4), kFpThreads, 0, s>>>(
            img + (size_t)b4 * p->g.nx * p->g.ny, sino + (size_t)b4 * n_rays, ray, p->d_nsamp,
            n_rays, p->g.nx, p->g.ny, p->fp_weight, batch - b4, max_iter);
        ct_count_launch();
    }
    return (int)cudaGetLastError();
}

int fp_fan_adjoint(const ct_plan *p, const float *sino, float *img, int batch, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    AdjArgs a;
    a.V = p->g.n_views;
    a.C = p->g.n_cols;
    a.nx = p->g.nx;
    a.ny = p->g.ny;
    a.w = p->fp_weight;
    a.src = p->g.sid;
    a.dx = p->g.dx;
    a.fov_px = (float)((double)p->g.rfov / (double)p->g.dx);
    a.left = p->g.left;
    a.dcol = p->g.dcol;
    a.max_iter = 2 * ((p->g.nx > p->g.ny ? p->g.nx : p->g.ny) + kTile) + 8;
    const float2 *vcs = reinterpret_cast<const float2 *>(p->d_view_cs);
    const float4 *ray = reinterpret_cast<const float4 *>(p->d_ray);
    for (int b0 = 0; b0 < batch; b0 += 65535) {
        const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
        dim3 grid((a.nx + kTile - 1) / kTile, (a.ny + kTile - 1) / kTile, nb);
        fp_fan_adjoint_tile_kernel<<<grid, kAdjThreads, 0, s>>>(
            sino + (size_t)b0 * a.V * a.C, img + (size_t)b0 * a.nx * a.ny, ray, p->d_nsamp, vcs,
            a, nb);
        ct_count_launch();
    }
    return (int)cudaGetLastError();
}

}  // namespace ctk
