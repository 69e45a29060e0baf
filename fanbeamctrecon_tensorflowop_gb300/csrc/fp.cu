// Ray-driven fan-beam forward projector and its exact transpose.
//
// Forward (replaces FP/transform.cu:103-146 and the per-view launch loop
// :162-169): all views and slices in one launch.  Each launch first builds
// "quad images" (per slice and layout, a float4 of the four clamped bilinear
// taps of every cell), then fp_warp (fp_body.cuh) walks 32 adjacent rays of a
// view per warp, row-synchronously, summing each cell's samples in closed
// form (cellwalk.cuh): one 16-byte gather per cell instead of four per
// sample.  Eight slices share one walk.  Output:
// p = 0.125*dx * sum_k bilinear_clamp(img, start + k*step), k < n.
//
// Transpose: the image is cut into bands of 4 rows (for rays running mostly
// along y) or 4 columns (rays mostly along x), each held with 8 slices in
// shared memory by one block.  For every view the block's warps take the
// rays of its layout that reach the band, clip them to the band's cells (plus
// the one-cell halo whose taps touch it), walk those cells row-synchronously
// and add val*W to the taps the band owns.  Layout 0 writes the image,
// layout 1 adds to it; no global atomics.  (Measured on GB300: shared-memory
// FP32 atomicAdd executes as a load + compare-and-swap loop, which bounds this
// kernel; square tiles are kept for images too wide for a band.)
#include <cfloat>
#include <climits>

#include "cellwalk.cuh"
#include "fp_body.cuh"

namespace ctk {
namespace {

constexpr int kFpThreads = 256;
constexpr int kFpChunk = 64;  // slices per quad-workspace chunk
#ifndef CT_FP_MIN_BLOCKS
#define CT_FP_MIN_BLOCKS 1
#endif
#ifndef CT_ADJ_TILE
#define CT_ADJ_TILE 32
#endif
#ifndef CT_ADJ_SLICES
#define CT_ADJ_SLICES 8
#endif
constexpr int kAdjTile = CT_ADJ_TILE;      // adjoint tile edge (pixels)
constexpr int kAdjSlices = CT_ADJ_SLICES;  // slices per adjoint walk
#ifndef CT_ADJ_BAND
#define CT_ADJ_BAND 4
#endif
constexpr int kAdjBand = CT_ADJ_BAND;  // rows (columns) per adjoint band

// Builds both quad layouts of nz slices (grid.z = 2 * slices).
__global__ void __launch_bounds__(256)
    build_quads_kernel(const float *__restrict__ img, float4 *__restrict__ quads, int nx, int ny) {
    const int Q = nx + 1;
    const int qi = blockIdx.x * 32 + threadIdx.x, qj = blockIdx.y * 8 + threadIdx.y;
    if (qi >= Q || qj >= Q) return;
    const int layout = blockIdx.z & 1, b = blockIdx.z >> 1;
    build_quad(img + (size_t)b * nx * ny,
               quads + ((size_t)b * 2 + layout) * Q * Q + (size_t)qj * Q + qi, nx, ny, layout,
               qi, qj);
}

template <int SB>
__global__ void __launch_bounds__(kFpThreads, CT_FP_MIN_BLOCKS)
    fp_fan_kernel(const float4 *__restrict__ quads, float *__restrict__ sino,
                  const float4 *__restrict__ ray, const int *__restrict__ nsamp, int V, int C,
                  int wpv, int nx, float w, int batch, int max_iter) {
    const int gw = blockIdx.x * (kFpThreads / 32) + (threadIdx.x >> 5);
    if (gw >= V * wpv) return;  // warp-uniform
    const int b0 = blockIdx.y * SB;
    const size_t lsz = (size_t)(nx + 1) * (nx + 1);
    // slices beyond the batch read slice b0's quads (results dropped)
    fp_warp<SB, float>(quads + (size_t)b0 * 2 * lsz, 2 * lsz, sino + (size_t)b0 * V * C,
                       (size_t)V * C, ray, nsamp, V, C, wpv, nx, w, min(SB, batch - b0),
                       max_iter, gw);
}

// ---- transpose ----------------------------------------------------------------

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

// One block per T x T image tile and group of SB slices; the tile's SB
// accumulators live in shared memory.  Each warp takes views in turn; for a
// view it takes the channels whose rays can reach the tile's cell box, 32 at
// a time (lane = channel), clips each ray to the box and walks the box's rows
// in lockstep like the forward projector (transposed when most rays run
// along x), adding val_s * W to the taps the tile owns for all SB slices.
// Every pixel is written once; no global atomics.
template <int T, int SB>
__global__ void __launch_bounds__(kAdjThreads)
    fp_fan_adjoint_tile_kernel(const float *__restrict__ sino, float *__restrict__ img,
                               const float4 *__restrict__ ray, const int *__restrict__ nsamp,
                               const float2 *__restrict__ view_cs, AdjArgs a, int batch) {
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ float acc[SB][T][T + 1];
    const int X0 = blockIdx.x * T, Y0 = blockIdx.y * T;
    const int b0 = blockIdx.z * SB;
    for (int k = threadIdx.x; k < SB * T * (T + 1); k += kAdjThreads) (&acc[0][0][0])[k] = 0.0f;
    // Cells whose taps touch owned pixels: cu in [X0-1, X0+T-1]; in cell
    // coordinates the box is x in [X0-1, X0+T), y likewise.  Tiles on the
    // image border also own the clamped taps of cells beyond it, so their box
    // reaches the edge of the FOV disc (x, y in [-1/2, 2*fov_px - 1/2]).
    const float far = fmaxf((float)max(a.nx, a.ny), 2.0f * a.fov_px) + 2.0f;
    const float Xlo = X0 == 0 ? -2.0f : (float)(X0 - 1);
    const float Xhi = X0 + T >= a.nx ? far : (float)(X0 + T);
    const float Ylo = Y0 == 0 ? -2.0f : (float)(Y0 - 1);
    const float Yhi = Y0 + T >= a.ny ? far : (float)(Y0 + T);
    // skip tiles whose box misses the FOV disc (centre fov_px - 1/2, radius fov_px)
    const float cx = a.fov_px - 0.5f;
    const float qx = fminf(fmaxf(cx, Xlo), Xhi) - cx, qy = fminf(fmaxf(cx, Ylo), Yhi) - cx;
    const bool live = qx * qx + qy * qy <= a.fov_px * a.fov_px * 1.0001f;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t slice = (size_t)a.V * a.C;
    for (int v = warp; live && v < a.V; v += kAdjThreads / 32) {
        // channel range of the rays that can reach the box, from its corners
        const float2 cs = __ldg(view_cs + v);
        float cmin = FLT_MAX, cmax = -FLT_MAX;
        if (lane < 4) {
            const float uc = (lane & 1) ? Xhi : Xlo, vc = (lane & 2) ? Yhi : Ylo;
            const float X = (uc + 0.5f - a.fov_px) * a.dx, Y = (vc + 0.5f - a.fov_px) * a.dx;
            cmin = cmax = channel_of(a, cs.x, cs.y, X, Y);
        }
#pragma unroll
        for (int o = 2; o > 0; o >>= 1) {
            cmin = fminf(cmin, __shfl_xor_sync(FULL, cmin, o));
            cmax = fmaxf(cmax, __shfl_xor_sync(FULL, cmax, o));
        }
        cmin = __shfl_sync(FULL, cmin, 0);
        cmax = __shfl_sync(FULL, cmax, 0);
        const int c_lo = max(0, (int)floorf(cmin) - 1);
        const int c_hi = min(a.C - 1, (int)ceilf(cmax) + 1);
        for (int cbase = c_lo; cbase <= c_hi; cbase += 32) {
            const int c = cbase + lane;
            const int r = v * a.C + min(c, a.C - 1);
            int n = c <= c_hi ? __ldg(nsamp + r) : 0;
            float val[SB];
            bool nz = false;
#pragma unroll
            for (int s = 0; s < SB; ++s) {
                val[s] = (n > 0 && b0 + s < batch) ? __ldg(sino + (b0 + s) * slice + r) * a.w : 0.0f;
                nz |= val[s] != 0.0f;
            }
            if (!nz) n = 0;
            const float4 q = n > 0 ? __ldg(ray + r) : make_float4(0.f, 0.f, 0.f, 0.f);
            const unsigned vm = __ballot_sync(FULL, n > 0);
            if (vm == 0) continue;
            const unsigned xm = __ballot_sync(FULL, n > 0 && fabsf(q.z) > fabsf(q.w));
            const bool along_x = 2 * __popc(xm) > __popc(vm);
            // walked coordinates: (u, v) = (x, y), or (y, x) when along_x
            const RaySeg seg = along_x ? RaySeg{q.y - 0.5f, q.x - 0.5f, q.w, q.z}
                                       : RaySeg{q.x - 0.5f, q.y - 0.5f, q.z, q.w};
            const float Ulo = along_x ? Ylo : Xlo, Uhi = along_x ? Yhi : Xhi;
            const float Vlo = along_x ? Xlo : Ylo, Vhi = along_x ? Xhi : Yhi;
            // samples inside the box
            float klo = 0.0f, khi = (float)n;
            if (n > 0) {
                if (seg.su != 0.0f) {
                    const float t0 = (Ulo - seg.u0) / seg.su, t1 = (Uhi - seg.u0) / seg.su;
                    klo = fmaxf(klo, ceilf(fminf(t0, t1)));
                    khi = fminf(khi, ceilf(fmaxf(t0, t1)));
                } else if (!(seg.u0 >= Ulo && seg.u0 < Uhi)) {
                    khi = 0.0f;
                }
                if (seg.sv != 0.0f) {
                    const float t0 = (Vlo - seg.v0) / seg.sv, t1 = (Vhi - seg.v0) / seg.sv;
                    klo = fmaxf(klo, ceilf(fminf(t0, t1)));
                    khi = fminf(khi, ceilf(fmaxf(t0, t1)));
                } else if (!(seg.v0 >= Vlo && seg.v0 < Vhi)) {
                    khi = 0.0f;
                }
            }
            const bool act = n > 0 && klo < khi;
            const unsigned am = __ballot_sync(FULL, act);
            if (am == 0) continue;
            const unsigned pm = __ballot_sync(FULL, act && seg.sv > 0.0f);
            const int dir = 2 * __popc(pm) >= __popc(am) ? 1 : -1;
            const bool synced = act && (dir > 0 ? seg.sv > 0.0f : seg.sv < 0.0f);
            // adds val_s * W to the owned taps of walked cell (cu, cv)
            auto scatter = [&](int cu, int cv, float cnt, float fa, float fb) {
                const CellWeights cw = cell_weights(cnt, fa, fb, seg.su, seg.sv);
                const int xc = along_x ? cv : cu, yc = along_x ? cu : cv;
                // tap (du, dv) of the walked cell is pixel (xc + du, yc + dv), or
                // (xc + dv, yc + du) when along_x; weights follow (du, dv)
                const int x0 = min(max(xc, 0), a.nx - 1) - X0;
                const int x1 = min(max(xc + 1, 0), a.nx - 1) - X0;
                const int y0 = min(max(yc, 0), a.ny - 1) - Y0;
                const int y1 = min(max(yc + 1, 0), a.ny - 1) - Y0;
                const bool ox0 = (unsigned)x0 < (unsigned)T, ox1 = (unsigned)x1 < (unsigned)T;
                const bool oy0 = (unsigned)y0 < (unsigned)T, oy1 = (unsigned)y1 < (unsigned)T;
                // weight of pixel (x0,y0), (x1,y0), (x0,y1), (x1,y1)
                const float p00 = cw.w00;
                const float p10 = along_x ? cw.w01 : cw.w10;
                const float p01 = along_x ? cw.w10 : cw.w01;
                const float p11 = cw.w11;
#pragma unroll
                for (int s = 0; s < SB; ++s) {
                    if (oy0 && ox0) atomicAdd(&acc[s][y0][x0], val[s] * p00);
                    if (oy0 && ox1) atomicAdd(&acc[s][y0][x1], val[s] * p10);
                    if (oy1 && ox0) atomicAdd(&acc[s][y1][x0], val[s] * p01);
                    if (oy1 && ox1) atomicAdd(&acc[s][y1][x1], val[s] * p11);
                }
            };
            const int jf = (int)floorf(fmaf(seg.sv, klo, seg.v0));
            const int jl = (int)floorf(fmaf(seg.sv, khi - 1.0f, seg.v0));
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
                    const float ka = fmaxf(klo, ceilf(fminf(tA, tB)));
                    const float kb = fminf(khi, ceilf(fmaxf(tA, tB)));
                    if (!(ka < kb)) continue;
                    float cu = floorf(fmaf(seg.su, ka, seg.u0));
                    float bu = seg.su >= 0.0f ? cu + 1.0f : cu;
                    float k = ka;
                    for (int t = 0; t < 8 && k < kb; ++t) {
                        const float tu = seg.su != 0.0f ? (bu - seg.u0) * iu : INF;
                        const float ke = fminf(kb, ceilf(tu));
                        const float cnt = ke - k;
                        if (cnt > 0.0f) {
                            scatter((int)cu, j, cnt, fmaf(seg.su, k, seg.u0) - cu,
                                    fmaf(seg.sv, k, seg.v0) - (float)j);
                            k = ke;
                        }
                        cu += du;
                        bu += du;
                    }
                }
            }
            if (act && !synced) walk_cells(seg, klo, khi, a.max_iter, scatter);
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < T * T; k += kAdjThreads) {
        const int jj = k / T, ii = k - jj * T;
        const int X = X0 + ii, Y = Y0 + jj;
        if (X >= a.nx || Y >= a.ny) continue;
#pragma unroll
        for (int s = 0; s < SB; ++s)
            if (b0 + s < batch) img[((size_t)(b0 + s) * a.ny + Y) * a.nx + X] = acc[s][jj][ii];
    }
}

// Band form of the transpose.  The image is cut into bands of R rows (layout
// 0, for rays that run mostly along y) or R columns (layout 1, rays mostly
// along x); a block holds one band of SB slices in shared memory, walked
// coordinates (u along the band, v across it).  Every ray of the block's
// layout crosses the band from side to side, so for each view the warp's 32
// lanes take consecutive channels, clip their rays to the band's cell box and
// step the band's R+2 rows in lockstep, adding val_s * W to owned taps.
// Layout 0 writes the image, layout 1 adds to it (every pixel has one owner
// band per layout): deterministic, no global atomics.
template <int R, int SB, int LAYOUT>
__global__ void __launch_bounds__(kAdjThreads)
    fp_fan_adjoint_band_kernel(const float *__restrict__ sino, float *__restrict__ img,
                               const float4 *__restrict__ ray, const int *__restrict__ nsamp,
                               const float2 *__restrict__ view_cs, AdjArgs a, int batch) {
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ float band[];  // [SB][R][Wd]
    const int Wd = LAYOUT ? a.ny : a.nx;  // walked u extent (band length)
    const int Hd = LAYOUT ? a.nx : a.ny;  // walked v extent
    const int V0 = blockIdx.x * R;
    const int b0 = blockIdx.y * SB;
    for (int k = threadIdx.x; k < SB * R * Wd; k += kAdjThreads) band[k] = 0.0f;
    const float far = fmaxf((float)max(a.nx, a.ny), 2.0f * a.fov_px) + 2.0f;
    const float Ulo = -2.0f, Uhi = far;
    const float Vlo = V0 == 0 ? -2.0f : (float)(V0 - 1);
    const float Vhi = V0 + R >= Hd ? far : (float)(V0 + R);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t slice = (size_t)a.V * a.C;
    for (int v = warp; v < a.V; v += kAdjThreads / 32) {
        // channels whose rays can reach the band's box (world corners of the box)
        const float2 cs = __ldg(view_cs + v);
        float cmin = FLT_MAX, cmax = -FLT_MAX;
        if (lane < 4) {
            const float uc = (lane & 1) ? Uhi : Ulo, vc = (lane & 2) ? Vhi : Vlo;
            const float xt = LAYOUT ? vc : uc, yt = LAYOUT ? uc : vc;
            const float X = (xt + 0.5f - a.fov_px) * a.dx, Y = (yt + 0.5f - a.fov_px) * a.dx;
            cmin = cmax = channel_of(a, cs.x, cs.y, X, Y);
        }
#pragma unroll
        for (int o = 2; o > 0; o >>= 1) {
            cmin = fminf(cmin, __shfl_xor_sync(FULL, cmin, o));
            cmax = fmaxf(cmax, __shfl_xor_sync(FULL, cmax, o));
        }
        cmin = __shfl_sync(FULL, cmin, 0);
        cmax = __shfl_sync(FULL, cmax, 0);
        const int c_lo = max(0, (int)floorf(cmin) - 1);
        const int c_hi = min(a.C - 1, (int)ceilf(cmax) + 1);
        for (int cbase = c_lo; cbase <= c_hi; cbase += 32) {
            const int c = cbase + lane;
            const int r = v * a.C + min(c, a.C - 1);
            int n = c <= c_hi ? __ldg(nsamp + r) : 0;
            float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
            if (n > 0) {
                q = __ldg(ray + r);
                const bool along_x = fabsf(q.z) > fabsf(q.w);
                if (along_x != (LAYOUT == 1)) n = 0;  // the other layout's band owns it
            }
            float val[SB];
            bool nz = false;
#pragma unroll
            for (int s = 0; s < SB; ++s) {
                val[s] = (n > 0 && b0 + s < batch) ? __ldg(sino + (b0 + s) * slice + r) * a.w
                                                   : 0.0f;
                nz |= val[s] != 0.0f;
            }
            if (!nz) n = 0;
            if (__ballot_sync(FULL, n > 0) == 0) continue;
            const RaySeg seg = LAYOUT ? RaySeg{q.y - 0.5f, q.x - 0.5f, q.w, q.z}
                                      : RaySeg{q.x - 0.5f, q.y - 0.5f, q.z, q.w};
            float klo = 0.0f, khi = (float)n;
            if (n > 0) {
                // |sv| >= |su| > 0 is not guaranteed (su may be 0); sv != 0 here
                const float iv = 1.0f / seg.sv;
                const float t0 = (Vlo - seg.v0) * iv, t1 = (Vhi - seg.v0) * iv;
                klo = fmaxf(klo, ceilf(fminf(t0, t1)));
                khi = fminf(khi, ceilf(fmaxf(t0, t1)));
            }
            const bool act = n > 0 && klo < khi;
            const unsigned am = __ballot_sync(FULL, act);
            if (am == 0) continue;
            const unsigned pm = __ballot_sync(FULL, act && seg.sv > 0.0f);
            const int dir = 2 * __popc(pm) >= __popc(am) ? 1 : -1;
            const bool synced = act && (dir > 0 ? seg.sv > 0.0f : seg.sv < 0.0f);
            auto scatter = [&](int cu, int cv, float cnt, float fa, float fb) {
                const CellWeights cw = cell_weights(cnt, fa, fb, seg.su, seg.sv);
                const int u0 = min(max(cu, 0), Wd - 1), u1 = min(max(cu + 1, 0), Wd - 1);
                const int r0 = min(max(cv, 0), Hd - 1) - V0, r1 = min(max(cv + 1, 0), Hd - 1) - V0;
                const bool o0 = (unsigned)r0 < (unsigned)R, o1 = (unsigned)r1 < (unsigned)R;
#pragma unroll
                for (int s = 0; s < SB; ++s) {
                    float *bs = band + (size_t)s * R * Wd;
                    if (o0) {
                        atomicAdd(bs + r0 * Wd + u0, val[s] * cw.w00);
                        atomicAdd(bs + r0 * Wd + u1, val[s] * cw.w10);
                    }
                    if (o1) {
                        atomicAdd(bs + r1 * Wd + u0, val[s] * cw.w01);
                        atomicAdd(bs + r1 * Wd + u1, val[s] * cw.w11);
                    }
                }
            };
            const int jf = (int)floorf(fmaf(seg.sv, klo, seg.v0));
            const int jl = (int)floorf(fmaf(seg.sv, khi - 1.0f, seg.v0));
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
                    const float ka = fmaxf(klo, ceilf(fminf(tA, tB)));
                    const float kb = fminf(khi, ceilf(fmaxf(tA, tB)));
                    if (!(ka < kb)) continue;
                    float cu = floorf(fmaf(seg.su, ka, seg.u0));
                    float bu = seg.su >= 0.0f ? cu + 1.0f : cu;
                    float k = ka;
                    for (int t = 0; t < 8 && k < kb; ++t) {
                        const float tu = seg.su != 0.0f ? (bu - seg.u0) * iu : INF;
                        const float ke = fminf(kb, ceilf(tu));
                        const float cnt = ke - k;
                        if (cnt > 0.0f) {
                            scatter((int)cu, j, cnt, fmaf(seg.su, k, seg.u0) - cu,
                                    fmaf(seg.sv, k, seg.v0) - (float)j);
                            k = ke;
                        }
                        cu += du;
                        bu += du;
                    }
                }
            }
            if (act && !synced) walk_cells(seg, klo, khi, a.max_iter, scatter);
        }
    }
    __syncthreads();
    // write (layout 0) or add (layout 1) the owned pixels
    for (int k = threadIdx.x; k < R * Wd; k += kAdjThreads) {
        const int rr = k / Wd, uu = k - rr * Wd;
        const int vv = V0 + rr;
        if (vv >= Hd) continue;
        const int X = LAYOUT ? vv : uu, Y = LAYOUT ? uu : vv;
#pragma unroll
        for (int s = 0; s < SB; ++s) {
            if (b0 + s >= batch) break;
            float *dst = img + ((size_t)(b0 + s) * a.ny + Y) * a.nx + X;
            const float val = band[(size_t)s * R * Wd + k];
            if (LAYOUT)
                *dst += val;
            else
                *dst = val;
        }
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
    a.max_iter = 2 * ((p->g.nx > p->g.ny ? p->g.nx : p->g.ny) + 64) + 8;
    const float2 *vcs = reinterpret_cast<const float2 *>(p->d_view_cs);
    const float4 *ray = reinterpret_cast<const float4 *>(p->d_ray);
    constexpr int R = kAdjBand, SB = kAdjSlices;
    const size_t plane = (size_t)a.nx * a.ny, slice = (size_t)a.V * a.C;
    const int per_launch = 65535 * SB;
    const size_t smem0 = sizeof(float) * SB * R * a.nx, smem1 = sizeof(float) * SB * R * a.ny;
    if (smem0 <= 200 * 1024 && smem1 <= 200 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fp_fan_adjoint_band_kernel<R, SB, 0>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem0);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(fp_fan_adjoint_band_kernel<R, SB, 1>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
        if (e != cudaSuccess) return (int)e;
        for (int b0 = 0; b0 < batch; b0 += per_launch) {
            const int nb = batch - b0 < per_launch ? batch - b0 : per_launch;
            const int groups = (nb + SB - 1) / SB;
            fp_fan_adjoint_band_kernel<R, SB, 0><<<dim3((a.ny + R - 1) / R, groups),
                                                     kAdjThreads, smem0, s>>>(
                sino + b0 * slice, img + b0 * plane, ray, p->d_nsamp, vcs, a, nb);
            fp_fan_adjoint_band_kernel<R, SB, 1><<<dim3((a.nx + R - 1) / R, groups),
                                                     kAdjThreads, smem1, s>>>(
                sino + b0 * slice, img + b0 * plane, ray, p->d_nsamp, vcs, a, nb);
            ct_count_launch(2);
        }
        return (int)cudaGetLastError();
    }
    // very wide images: square tiles
    constexpr int T = kAdjTile;
    for (int b0 = 0; b0 < batch; b0 += per_launch) {
        const int nb = batch - b0 < per_launch ? batch - b0 : per_launch;
        dim3 grid((a.nx + T - 1) / T, (a.ny + T - 1) / T, (nb + SB - 1) / SB);
        fp_fan_adjoint_tile_kernel<T, SB><<<grid, kAdjThreads, 0, s>>>(
            sino + b0 * slice, img + b0 * plane, ray, p->d_nsamp, vcs, a, nb);
        ct_count_launch();
    }
    return (int)cudaGetLastError();
}

}  // namespace ctk
