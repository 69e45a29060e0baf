// Pixel-driven fan-beam backprojection (unweighted BP and 1/L^2-weighted FBP /
// FDK-2D) and its transpose.
//
// Per pixel centre (x, y) inside the FOV disc and view beta, with
// c = -cos(beta), s = -sin(beta):
//   U = R + x c + y s,  t = -x s + y c,  col = (atan(t/U) - left)/dcol + shift,
// and when 0 < col < n_cols the pixel gains the linearly interpolated,
// clamped detector value at col (texel centres at +1/2), times 1/(U^2+t^2) in
// the weighted form (BP/transform.cu:76-92, FBP/transform.cu:70-87,
// FDK/GPURecon_GPU.cu:25-49).
//
// One launch covers all views and slices.  Each thread keeps four pixels of a
// 32x32 tile in registers across all views (the image is written once, not
// read-modified-written per view), and evaluates the per-pixel geometry once
// for up to four slices.  t/U uses the SFU reciprocal; atan(z) is a
// polynomial in z^2 fitted per plan over the FOV's |z| range (to FP32 atanf
// accuracy, 3e-8 absolute), with atanf kept for fans wider than 90 degrees.
// Plans with texture_weights = 1 round the interpolation weight as the
// reference's texture unit does (tex_weight); the default keeps exact FP32.
#include <cstdint>

#include "bp_body.cuh"

namespace ctk {
namespace {

constexpr int kTile = kBpTile;
// slices per transpose thread for batches of 4 or more (32 clinical slices:
// 1 -> 16.2 ms, 4 -> 15.5, 8 -> 17.2); smaller batches take one per thread
constexpr int kBptSlices = 4;
constexpr int kRowsPerThr = kBpRowsPerThr;

// PAIRS: slice group z reads the SB/4 four-slice tap planes SB/4 z ..
// ([V][C+1] x 2 float4 each); ROWS pixels per thread (tiles of 32 x 8 ROWS).
// Resident blocks per SM of the tap-image forms, measured for 32 clinical
// slices (all forms give the same bits):
//   four slices per thread: BP (2 rows) 3.42 / 3.21 ms with 6 / 5 blocks,
//     the weighted form (1 row) 3.78 / 4.62 ms;
//   eight slices per thread: BP (2 rows) 2.89 / 2.99 ms with 4 / 3 blocks; BP
//     at 1 row 2.98 ms with 4; the weighted form at 2 rows 3.50 ms with 4
//     blocks, at 1 row 3.71 / 4.53 / 4.03 ms with 4 / 5 / 6 (5 and 6 spill).
#ifndef CT_BP4_MINB1
#define CT_BP4_MINB1 6
#endif
#ifndef CT_BP4_MINB2
#define CT_BP4_MINB2 5
#endif
#ifndef CT_BP8_MINB1
#define CT_BP8_MINB1 4
#endif
#ifndef CT_BP8_MINB2
#define CT_BP8_MINB2 4
#endif
constexpr int bp_min_blocks(bool pairs, int sb, int rows) {
    return !pairs || rows > 2 ? 1
           : sb == 8          ? (rows == 1 ? CT_BP8_MINB1 : CT_BP8_MINB2)
                              : (rows == 1 ? CT_BP4_MINB1 : CT_BP4_MINB2);
}
template <bool WEIGHTED, int SB, int DEG, bool TEX, bool PAIRS, int ROWS = kBpRowsPerThr>
__global__ void __launch_bounds__(256, bp_min_blocks(PAIRS, SB, ROWS))
    bp_fan_kernel(const float *__restrict__ sino, const float4 *__restrict__ pairs,
                  float *__restrict__ img, const float2 *__restrict__ view_cs, BpArgs a,
                  int batch) {
    const int b0 = blockIdx.z * SB;
    const size_t slice = (size_t)a.V * a.C, plane = (size_t)a.nx * a.ny;
    const float4 *pz =
        PAIRS ? pairs + (size_t)blockIdx.z * a.V * (a.C + 1) * (SB / 2) : pairs;
    bp_tile<WEIGHTED, SB, DEG, float, ROWS, TEX, PAIRS>(sino + b0 * slice, slice,
                                                        img + b0 * plane, plane, view_cs, a,
                                                        min(SB, batch - b0), blockIdx.x,
                                                        blockIdx.y, pz);
}

// Tap images of slice groups of SB: group z, view v, column position i in
// [0, C]: the taps (i0, i1) = (max(i-1, 0), min(i, C-1)) of slices
// SB z .. SB z + SB-1 (zero past `batch`), as SB/2 float4; float4 h holds
// slices (2h, 2h+1) as (i0 of both, i1 of both), the f32x2 operands of the
// backprojector's paired interpolation.
template <int SB>
__global__ void __launch_bounds__(256)
    bp_pairs_kernel(const float *__restrict__ sino, float4 *__restrict__ pairs, int V, int C,
                    int batch) {
    const int i = blockIdx.x * 256 + threadIdx.x, v = blockIdx.y, z = blockIdx.z;
    if (i > C) return;
    const int i0 = max(i - 1, 0), i1 = min(i, C - 1);
    float4 *q = pairs + (((size_t)z * V + v) * (C + 1) + i) * (SB / 2);
#pragma unroll
    for (int h = 0; h < SB / 2; ++h) {
        float t[4];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const int b = SB * z + 2 * h + s;
            const float *row = sino + ((size_t)b * V + v) * C;
            t[s] = b < batch ? __ldg(row + i0) : 0.0f;
            t[2 + s] = b < batch ? __ldg(row + i1) : 0.0f;
        }
        q[h] = make_float4(t[0], t[1], t[2], t[3]);
    }
}

// Transpose of bp_fan_kernel in scatter form (plans with texture weights, or
// without a workspace): each pixel-view scatters x * weight * (1-f, f)
// onto the two clamped detector taps with global atomics (L2 reductions).  A
// thread evaluates each pixel-view's geometry once for GSB slices.
// Atomics of one warp instruction that hit the same address serialise, so the
// 32 lanes of a warp always lie across the view's rays (where their columns
// differ): grid.z pairs a row pass (lanes along x, pixels of a thread 8 apart
// in y), which takes the views whose rays run along y, with a column pass
// (lanes along y) for the views whose rays run along x.  With one layout for
// all views, half of them put a warp's lanes along a ray onto a few columns
// (32 clinical slices: 15.6 -> 12.4 ms).  Adjacent lanes' columns are about
// one apart, so a lane adds its right neighbour's lower part into its own
// upper atomic when they share the address (12.4 -> 11.4 ms; 16-byte vector
// atomics covering both taps measured 24 ms).  (A shared-memory, fixed-point form
// with one block per view measured slower: every block then sweeps the
// whole image.)
template <bool WEIGHTED, int DEG, int GSB, bool TEX>
__global__ void __launch_bounds__(256)
    bp_fan_transpose_kernel(const float *__restrict__ img, float *__restrict__ sino,
                            const float2 *__restrict__ view_cs, BpArgs a, int batch) {
    // grid.z = 2 * slice groups: even z maps lanes along x and takes the views
    // whose rays run along y, odd z maps lanes along y and takes the others
    const bool colmode = blockIdx.z & 1;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int b0 = (blockIdx.z >> 1) * GSB;
    if (b0 >= batch) return;
    const int nsl = min(GSB, batch - b0);
    float px[kRowsPerThr], py[kRowsPerThr], xv[GSB][kRowsPerThr];
    bool nz[kRowsPerThr];
    bool any = false;
#pragma unroll
    for (int k = 0; k < kRowsPerThr; ++k) {
        // row mode: lane = x, the thread's pixels step 8 in y; column mode: swapped
        const int ix = colmode ? blockIdx.x * kTile + ty + 8 * k : blockIdx.x * kTile + tx;
        const int iy = colmode ? blockIdx.y * kTile + tx : blockIdx.y * kTile + ty + 8 * k;
        const double xd = (double)a.xmin + (double)a.dx * (ix + 0.5);
        const double yd = (double)a.ymin + (double)a.dy * (iy + 0.5);
        px[k] = (float)xd;
        py[k] = (float)yd;
        const bool in = ix < a.nx && iy < a.ny && (xd * xd + yd * yd <= a.fov_r2);
        nz[k] = false;
#pragma unroll
        for (int s = 0; s < GSB; ++s) {
            xv[s][k] = in && s < nsl
                           ? img[(size_t)(b0 + s) * a.nx * a.ny + (size_t)iy * a.nx + ix]
                           : 0.0f;
            nz[k] |= xv[s][k] != 0.0f;
        }
        any |= nz[k];
    }
    if (!__syncthreads_or(any)) return;
    for (int v = 0; v < a.V; ++v) {
        const float2 cs = __ldg(view_cs + v);
        // rays run along (c, s) = cs: row pass for |c| < |s|, column pass otherwise
        if ((fabsf(cs.x) >= fabsf(cs.y)) != colmode) continue;  // block-uniform
#pragma unroll
        for (int k = 0; k < kRowsPerThr; ++k) {
            if (!__any_sync(0xffffffffu, nz[k])) continue;  // warp-uniform
            const float U = fmaf(px[k], cs.x, fmaf(py[k], cs.y, a.R));
            const float t = fmaf(py[k], cs.x, -px[k] * cs.y);
            const float rU = __fdividef(1.0f, U);
            const float g = fov_atan<DEG>(t * rU, a.coef);
            const float y = fmaf(g, a.inv_dcol, a.pos_off);
            const bool ok = nz[k] && y > 0.5f && y < a.fC + 0.5f;
            int i;
            float f;
            split_pos(ok ? y : 1.0f, i, f);
            if constexpr (TEX) f = tex_weight(f);
            const int i0 = max(i - 1, 0), i1 = min(i, a.C - 1);
            const float w = WEIGHTED ? __fdividef(1.0f, fmaf(U, U, t * t)) : 1.0f;
            // the next lane's lower tap is usually this lane's upper one: this
            // lane adds the next lane's lower part there, and the next lane
            // skips that atomic
            const int lane = threadIdx.x;
            const int nb_i0 = __shfl_down_sync(0xffffffffu, ok ? i0 : -1, 1);
            const int pv_i1 = __shfl_up_sync(0xffffffffu, ok ? i1 : -2, 1);
            const bool take = ok && lane < 31 && nb_i0 == i1;
            const bool given = ok && lane > 0 && pv_i1 == i0;
#pragma unroll
            for (int s = 0; s < GSB; ++s) {
                const float val = ok ? xv[s][k] * w : 0.0f;
                const float lo = val * (1.0f - f), hi = val * f;
                const float nb_lo = __shfl_down_sync(0xffffffffu, lo, 1);
                const float up = take ? hi + nb_lo : hi;
                if (ok && s < nsl) {
                    float *row = sino + ((size_t)(b0 + s) * a.V + v) * a.C;
                    if (!given && lo != 0.0f) atomicAdd(row + i0, lo);
                    if (up != 0.0f) atomicAdd(row + i1, up);
                }
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
    const double inv = 1.0 / (double)p->g.dcol;
    a.inv_dcol = (float)inv;
    a.pos_off = (float)((double)p->g.shift - (double)p->g.left * inv + 0.5);
    a.fC = (float)a.C;
    a.fov_r2 = (double)p->g.rfov * (double)p->g.rfov;
    for (int k = 0; k < 9; ++k) a.coef[k] = p->atan_coef[k];
    return a;
}

template <bool W, int SB, bool TEX, bool PAIRS, int ROWS>
void launch_bp(int deg, dim3 grid, cudaStream_t s, const float *sp, const float4 *pairs,
               float *ip, const float2 *vcs, const BpArgs &a, int nb) {
    dim3 block(kTile, 8, 1);
    if (deg == 4)
        bp_fan_kernel<W, SB, 4, TEX, PAIRS, ROWS><<<grid, block, 0, s>>>(sp, pairs, ip, vcs, a,
                                                                         nb);
    else if (deg == 8)
        bp_fan_kernel<W, SB, 8, TEX, PAIRS, ROWS><<<grid, block, 0, s>>>(sp, pairs, ip, vcs, a,
                                                                         nb);
    else
        bp_fan_kernel<W, SB, 0, TEX, PAIRS, ROWS><<<grid, block, 0, s>>>(sp, pairs, ip, vcs, a,
                                                                         nb);
}

template <int SB, bool PAIRS, int ROWS = kRowsPerThr>
void launch_bp_any(bool w, bool tex, int deg, dim3 grid, cudaStream_t s, const float *sp,
                   const float4 *pairs, float *ip, const float2 *vcs, const BpArgs &a, int nb) {
    if (w)
        (tex ? launch_bp<true, SB, true, PAIRS, ROWS> : launch_bp<true, SB, false, PAIRS, ROWS>)(
            deg, grid, s, sp, pairs, ip, vcs, a, nb);
    else
        (tex ? launch_bp<false, SB, true, PAIRS, ROWS>
             : launch_bp<false, SB, false, PAIRS, ROWS>)(deg, grid, s, sp, pairs, ip, vcs, a, nb);
}

template <bool W, int G, bool TEX>
void launch_bpt(int deg, dim3 grid, cudaStream_t s, const float *ip, float *sp, const float2 *vcs,
                const BpArgs &a, int nb) {
    dim3 block(kTile, 8, 1);
    if (deg == 4)
        bp_fan_transpose_kernel<W, 4, G, TEX><<<grid, block, 0, s>>>(ip, sp, vcs, a, nb);
    else if (deg == 8)
        bp_fan_transpose_kernel<W, 8, G, TEX><<<grid, block, 0, s>>>(ip, sp, vcs, a, nb);
    else
        bp_fan_transpose_kernel<W, 0, G, TEX><<<grid, block, 0, s>>>(ip, sp, vcs, a, nb);
}

template <int G>
void launch_bpt_any(bool w, bool tex, int deg, dim3 grid, cudaStream_t s, const float *ip,
                    float *sp, const float2 *vcs, const BpArgs &a, int nb) {
    if (w)
        (tex ? launch_bpt<true, G, true> : launch_bpt<true, G, false>)(deg, grid, s, ip, sp, vcs,
                                                                      a, nb);
    else
        (tex ? launch_bpt<false, G, true> : launch_bpt<false, G, false>)(deg, grid, s, ip, sp,
                                                                        vcs, a, nb);
}

}  // namespace

// Tap images of slice groups of four, one pass per 64 slices.  (Groups of
// eight with 2 pixel rows per thread, the same accumulators per thread,
// measured 5.25 ms for 32 clinical slices against 4.08 ms.)
constexpr int kPairSlices = 64;
#ifndef CT_BP_SB8
#define CT_BP_SB8 1
#endif
#ifndef CT_BP8_ROWS
#define CT_BP8_ROWS 2
#endif
#ifndef CT_BP8_ROWS_W
#define CT_BP8_ROWS_W 2
#endif

int pair_group(int batch) { return batch >= 4 ? 4 : 0; }

size_t bp_fan_work_bytes(const ct_plan *p, int batch) {
    const int sb = pair_group(batch);
    if (!sb) return 0;
    const int per = batch < kPairSlices ? batch : kPairSlices;
    const int groups = (per + sb - 1) / sb;
    // + 16 bytes to start the 32-byte entries on a 32-byte boundary
    return sizeof(float4) * (sb / 2) * (size_t)groups * p->g.n_views * (p->g.n_cols + 1) + 16;
}

int bp_fan(const ct_plan *p, const float *sino, float *img, int batch, int weighted, void *work,
           void *stream) {
    const BpArgs a = make_args(p);
    const float2 *vcs = reinterpret_cast<const float2 *>(p->d_view_cs);
    cudaStream_t s = (cudaStream_t)stream;
    const bool tex = p->opts.texture_weights != 0;
    const size_t slice = (size_t)a.V * a.C, plane = (size_t)a.nx * a.ny;
    if (const int sb = work ? pair_group(batch) : 0) {
        // 32-byte entries read by 32-byte loads (the workspace is 16-byte aligned)
        float4 *pairs = reinterpret_cast<float4 *>((reinterpret_cast<uintptr_t>(work) + 31) &
                                                   ~(uintptr_t)31);
        for (int b0 = 0; b0 < batch; b0 += kPairSlices) {
            const int nb = batch - b0 < kPairSlices ? batch - b0 : kPairSlices;
            const int groups = (nb + sb - 1) / sb;
            const float *sp = sino + (size_t)b0 * slice;
            float *ip = img + (size_t)b0 * plane;
            bp_pairs_kernel<4><<<dim3((a.C + 1 + 255) / 256, a.V, groups), 256, 0, s>>>(
                sp, pairs, a.V, a.C, nb);
            ct_count_launch();
            // Groups of eight slices read two four-slice planes per pixel-view and
            // share its geometry over eight slices; the rest take groups of four
            // (32 clinical slices: BP 3.21 -> 2.89 ms, FBP 3.78 -> 3.50 ms).
            // Pixel rows per thread (tiles of 32 x 8 rows): fewer rows, fewer
            // registers, more blocks (four slices per thread, before the f32x2
            // pairs: BP 4.10 / 3.64 / 3.73 ms with 4 / 2 / 1 rows, FBP 4.94 / 4.29 /
            // 4.21 ms).
            const int n8 = CT_BP_SB8 ? nb / 8 * 8 : 0;
            const size_t plane4 = (size_t)a.V * (a.C + 1) * 2;  // float4 per tap plane
            if (n8) {
                if (weighted) {
                    dim3 grid((a.nx + kTile - 1) / kTile, (a.ny + 8 * CT_BP8_ROWS_W - 1) /
                                                              (8 * CT_BP8_ROWS_W), n8 / 8);
                    launch_bp_any<8, true, CT_BP8_ROWS_W>(true, tex, p->atan_deg, grid, s, sp,
                                                          pairs, ip, vcs, a, n8);
                } else {
                    dim3 grid((a.nx + kTile - 1) / kTile, (a.ny + 8 * CT_BP8_ROWS - 1) /
                                                              (8 * CT_BP8_ROWS), n8 / 8);
                    launch_bp_any<8, true, CT_BP8_ROWS>(false, tex, p->atan_deg, grid, s, sp,
                                                        pairs, ip, vcs, a, n8);
                }
                ct_count_launch();
            }
            if (nb > n8) {
                const int g4 = (nb - n8 + 3) / 4;
                const float *sp4 = sp + (size_t)n8 * slice;
                const float4 *pairs4 = pairs + (size_t)(n8 / 4) * plane4;
                float *ip4 = ip + (size_t)n8 * plane;
                if (weighted) {
                    dim3 grid((a.nx + kTile - 1) / kTile, (a.ny + 7) / 8, g4);
                    launch_bp_any<4, true, 1>(true, tex, p->atan_deg, grid, s, sp4, pairs4, ip4,
                                              vcs, a, nb - n8);
                } else {
                    dim3 grid((a.nx + kTile - 1) / kTile, (a.ny + 15) / 16, g4);
                    launch_bp_any<4, true, 2>(false, tex, p->atan_deg, grid, s, sp4, pairs4,
                                              ip4, vcs, a, nb - n8);
                }
                ct_count_launch();
            }
        }
        return (int)cudaGetLastError();
    }
    const int SB = batch >= 4 ? 4 : 1;
    const int per_launch = 65535 * SB;
    for (int b0 = 0; b0 < batch; b0 += per_launch) {
        const int nb = batch - b0 < per_launch ? batch - b0 : per_launch;
        dim3 grid((a.nx + kTile - 1) / kTile, (a.ny + kTile - 1) / kTile, (nb + SB - 1) / SB);
        const float *sp = sino + (size_t)b0 * slice;
        float *ip = img + (size_t)b0 * plane;
        if (SB == 4)
            launch_bp_any<4, false>(weighted != 0, tex, p->atan_deg, grid, s, sp, nullptr, ip,
                                    vcs, a, nb);
        else
            launch_bp_any<1, false>(weighted != 0, tex, p->atan_deg, grid, s, sp, nullptr, ip,
                                    vcs, a, nb);
        ct_count_launch();
    }
    return (int)cudaGetLastError();
}

size_t bp_fan_transpose_work_bytes(const ct_plan *p, int batch) {
    return bp_gather_work_bytes(p, batch);
}

// The gather form (bp_gather.cu) where the plan has its tables, the
// exact-weight interpolation and a workspace; otherwise the scatter below
// (texture-weight plans keep it: it repeats the forward's own column
// arithmetic, so the adjoint stays the exact transpose of those weights).
int bp_fan_transpose(const ct_plan *p, const float *img, float *sino, int batch, int weighted,
                     void *work, void *stream) {
    if (work && bp_gather_usable(p)) return bp_gather(p, img, sino, batch, weighted, work, stream);
    const BpArgs a = make_args(p);
    const float2 *vcs = reinterpret_cast<const float2 *>(p->d_view_cs);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(sino, 0, sizeof(float) * (size_t)batch * a.V * a.C, s);
    if (e != cudaSuccess) return (int)e;
    const int G = batch >= kBptSlices ? kBptSlices : 1;
    for (int b0 = 0; b0 < batch; b0 += 32767 * G) {
        const int nb = batch - b0 < 32767 * G ? batch - b0 : 32767 * G;
        dim3 grid((a.nx + kTile - 1) / kTile, (a.ny + kTile - 1) / kTile, 2 * ((nb + G - 1) / G));
        const float *ip = img + (size_t)b0 * a.nx * a.ny;
        float *sp = sino + (size_t)b0 * a.V * a.C;
        const bool tex = p->opts.texture_weights != 0;
        if (G == kBptSlices)
            launch_bpt_any<kBptSlices>(weighted != 0, tex, p->atan_deg, grid, s, ip, sp, vcs, a,
                                       nb);
        else
            launch_bpt_any<1>(weighted != 0, tex, p->atan_deg, grid, s, ip, sp, vcs, a, nb);
        ct_count_launch();
    }
    return (int)cudaGetLastError();
}

}  // namespace ctk
