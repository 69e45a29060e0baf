// Ray-driven fan-beam forward projector and its exact transpose.
//
// Forward (replaces FP/transform.cu:103-146 and the per-view launch loop
// :162-169): one thread per ray, all views and slices in one launch.  The
// thread walks the bilinear cells its ray crosses and adds each cell's
// samples in closed form (cellwalk.cuh), so the image is read once per cell
// instead of four times per sample; SB slices share one walk.  Output:
// p = 0.125*dx * sum_k bilinear_clamp(img, start + k*step), k < n.
// The lanes of a warp are adjacent rays of one view.  A ray running mostly
// along x reads a transposed copy of the image (built per launch in the
// workspace), so that for every view the lanes' taps lie along memory rows
// and a warp's gather touches one or two cache lines per tap, not one line
// per lane.
//
// Transpose: one block per 32x32 image tile and slice keeps the tile in
// shared memory.  For every view it takes the rays that can reach the tile,
// clips each ray's samples to the tile's cells (plus the one-cell halo whose
// taps touch the tile), walks those cells and adds val*W to the taps the
// tile owns.  Every pixel is written exactly once; there are no global
// atomics.
#include <cfloat>
#include <climits>

#include "cellwalk.cuh"

namespace ctk {
namespace {

constexpr int kFpThreads = 256;
constexpr int kFpChunk = 64;  // slices per quad-workspace chunk

// Quad images: for every bilinear cell (cu, cv) of the walked layout, the
// four clamp-to-edge taps (cu,cv), (cu+1,cv), (cu,cv+1), (cu+1,cv+1) as one
// float4, so a cell's gather is a single 16-byte load.  Samples lie inside
// the FOV circle of radius nx/2 texels, so cells run over [-1, nx-1] in both
// axes of both layouts; quad (qi, qj) holds cell (qi-1, qj-1) and a layout
// is (nx+1)^2 quads.  Layout 0 walks (u, v) = (x, y); layout 1 walks the
// transposed image, (u, v) = (y, x).
__global__ void __launch_bounds__(256)
    build_quads_kernel(const float *__restrict__ img, float4 *__restrict__ quads, int nx, int ny) {
    const int Q = nx + 1;
    const int qi = blockIdx.x * 32 + threadIdx.x, qj = blockIdx.y * 8 + threadIdx.y;
    if (qi >= Q || qj >= Q) return;
    const int layout = blockIdx.z & 1, b = blockIdx.z >> 1;
    const float *im = img + (size_t)b * nx * ny;
    const int cu = qi - 1, cv = qj - 1;
    // tap (du, dv) of the cell is image pixel x = cu+du, y = cv+dv (layout 0)
    // or x = cv+dv, y = cu+du (layout 1), clamped to the image
    float4 t;
    float *tv = &t.x;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int du = k & 1, dv = k >> 1;
        int x = layout ? cv + dv : cu + du;
        int y = layout ? cu + du : cv + dv;
        x = min(max(x, 0), nx - 1);
        y = min(max(y, 0), ny - 1);
        tv[k] = __ldg(im + (size_t)y * nx + x);
    }
    quads[((size_t)b * 2 + layout) * Q * Q + (size_t)qj * Q + qi] = t;
}

template <int SB>
struct Taps {
    const float4 *q;  // this warp's layout of slice b0; slice s adds s * stride
    size_t stride;    // quads between consecutive slices
    int Q;            // quads per row (nx + 1)
    float acc[SB];
    __device__ __forceinline__ void add(const CellWeights &cw, int cu, int cv) {
        const int qi = min(max(cu + 1, 0), Q - 1), qj = min(max(cv + 1, 0), Q - 1);
        const float4 *p = q + (size_t)qj * Q + qi;
#pragma unroll
        for (int s = 0; s < SB; ++s) {
            const float4 t = __ldg(p + s * stride);
            float v = cw.w00 * t.x;
            v = fmaf(cw.w10, t.y, v);
            v = fmaf(cw.w01, t.z, v);
            v = fmaf(cw.w11, t.w, v);
            acc[s] += v;
        }
    }
};

// One warp = 32 consecutive channels of one view (warps never straddle views;
// wpv warps per view).  The warp votes its layout (transposed when most rays
// run along x) and its row direction, then steps through the rows of that
// layout in lockstep: in each row every lane sums the (one to three) cells its
// ray crosses there.  Lanes therefore gather from the same one or two rows at
// a time, whatever depth their rays entered the FOV at.  A lane whose ray
// runs against the warp's direction (possible only at a layout boundary)
// walks on its own afterwards.
template <int SB>
__global__ void __launch_bounds__(kFpThreads)
    fp_fan_kernel(const float4 *__restrict__ quads, float *__restrict__ sino,
                  const float4 *__restrict__ ray, const int *__restrict__ nsamp, int V, int C,
                  int wpv, int nx, float w, int batch, int max_iter) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (kFpThreads / 32) + (threadIdx.x >> 5);
    if (gw >= V * wpv) return;  // warp-uniform
    const int v = gw / wpv;
    const int c = (gw - v * wpv) * 32 + lane;
    const bool has_c = c < C;
    const int r = v * C + (has_c ? c : C - 1);
    const int b0 = blockIdx.y * SB;
    const int n = has_c ? __ldg(nsamp + r) : 0;
    const bool valid = n > 0;
    const float4 q = valid ? __ldg(ray + r) : make_float4(0.f, 0.f, 0.f, 0.f);

    const unsigned vm = __ballot_sync(FULL, valid);
    const unsigned xm = __ballot_sync(FULL, valid && fabsf(q.z) > fabsf(q.w));
    const bool along_x = 2 * __popc(xm) > __popc(vm);
    const RaySeg seg = along_x ? RaySeg{q.y - 0.5f, q.x - 0.5f, q.w, q.z}
                               : RaySeg{q.x - 0.5f, q.y - 0.5f, q.z, q.w};
    Taps<SB> tp;
    tp.Q = nx + 1;
    const size_t lsz = (size_t)tp.Q * tp.Q;
    tp.stride = 2 * lsz;
    // slices beyond the batch read the last slice's quads (results dropped)
    tp.q = quads + (size_t)b0 * tp.stride + (along_x ? lsz : 0);
#pragma unroll
    for (int s = 0; s < SB; ++s) tp.acc[s] = 0.0f;
    const unsigned pm = __ballot_sync(FULL, valid && seg.sv > 0.0f);
    const int dir = 2 * __popc(pm) >= __popc(vm) ? 1 : -1;
    const bool synced = valid && (dir > 0 ? seg.sv > 0.0f : seg.sv < 0.0f);
    const float nf = (float)n;
    // rows of the first and last sample, one row of slack on each side
    const int jf = (int)floorf(seg.v0);
    const int jl = (int)floorf(fmaf(seg.sv, nf - 1.0f, seg.v0));
    int J0, J1;
    if (dir > 0) {
        J0 = __reduce_min_sync(FULL, synced ? jf : INT_MAX) - 1;
        J1 = __reduce_max_sync(FULL, synced ? jl : INT_MIN) + 1;
    } else {
        J0 = __reduce_max_sync(FULL, synced ? jf : INT_MIN) + 1;
        J1 = __reduce_min_sync(FULL, synced ? jl : INT_MAX) - 1;
    }
    if (__any_sync(FULL, synced)) {
        const float INF = __int_as_float(0x7f800000);
        const float iu = seg.su != 0.0f ? 1.0f / seg.su : 0.0f;
        const float iv = synced ? 1.0f / seg.sv : 0.0f;
        const float du = seg.su >= 0.0f ? 1.0f : -1.0f;
        const int rows = (J1 - J0) * dir + 1;
        for (int it = 0; it < rows; ++it) {
            const int j = J0 + it * dir;
            if (!synced) continue;
            const float tA = ((float)j - seg.v0) * iv, tB = ((float)(j + 1) - seg.v0) * iv;
            const float ka = fmaxf(0.0f, ceilf(fminf(tA, tB)));
            const float kb = fminf(nf, ceilf(fmaxf(tA, tB)));
            if (!(ka < kb)) continue;
            float cu = floorf(fmaf(seg.su, ka, seg.u0));
            float bu = seg.su >= 0.0f ? cu + 1.0f : cu;
            float k = ka;
            for (int t = 0; t < 8 && k < kb; ++t) {
                const float tu = seg.su != 0.0f ? (bu - seg.u0) * iu : INF;
                const float ke = fminf(kb, ceilf(tu));
                const float cnt = ke - k;
                if (cnt > 0.0f) {
                    const float a = fmaf(seg.su, k, seg.u0) - cu;
                    const float b = fmaf(seg.sv, k, seg.v0) - (float)j;
                    tp.add(cell_weights(cnt, a, b, seg.su, seg.sv), (int)cu, j);
                    k = ke;
                }
                cu += du;
                bu += du;
            }
        }
    }
    if (valid && !synced) {
        walk_cells(seg, 0.0f, nf, max_iter, [&](int cu, int cv, float cnt, float a, float b) {
            tp.add(cell_weights(cnt, a, b, seg.su, seg.sv), cu, cv);
        });
    }
    if (has_c) {
#pragma unroll
        for (int s = 0; s < SB; ++s)
            if (b0 + s < batch) sino[((size_t)(b0 + s) * V + v) * C + c] = tp.acc[s] * w;
    }
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
    const int blocks = (V * wpv + kFpThreads / 32 - 1) / (kFpThreads / 32);
    const int Q = nx + 1;
    // chunks of at most kFpChunk slices share the quad workspace
    for (int c0 = 0; c0 < batch; c0 += kFpChunk) {
        const int nb = batch - c0 < kFpChunk ? batch - c0 : kFpChunk;
        build_quads_kernel<<<dim3((Q + 31) / 32, (Q + 7) / 8, 2 * nb), dim3(32, 8), 0, s>>>(
            img + (size_t)c0 * plane, quads, nx, ny);
        ct_count_launch();
        float *out = sino + (size_t)c0 * n_rays;
        int b = 0;
        if (nb >= 8) {
            const int n8 = nb / 8 * 8;
            fp_fan_kernel<8><<<dim3(blocks, n8 / 8), kFpThreads, 0, s>>>(
                quads, out, ray, p->d_nsamp, V, C, wpv, nx, p->fp_weight, n8, max_iter);
            ct_count_launch();
            b = n8;
        }
        if (nb - b >= 4) {
            fp_fan_kernel<4><<<dim3(blocks, 1), kFpThreads, 0, s>>>(
                quads + (size_t)b * 2 * Q * Q, out + (size_t)b * n_rays, ray, p->d_nsamp, V, C,
                wpv, nx, p->fp_weight, 4, max_iter);
            ct_count_launch();
            b += 4;
        }
        if (nb > b) {
            fp_fan_kernel<1><<<dim3(blocks, nb - b), kFpThreads, 0, s>>>(
                quads + (size_t)b * 2 * Q * Q, out + (size_t)b * n_rays, ray, p->d_nsamp, V, C,
                wpv, nx, p->fp_weight, nb - b, max_iter);
            ct_count_launch();
        }
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
