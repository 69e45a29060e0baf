// Cone-beam operators: the reference's CB_EA backprojection for nz slices and
// n_rows detector rows (FDK), its transpose (the FDK adjoint), and a cone-beam
// forward projector.
//
// Volumes are [B][nz][ny][nx]; projections [B][V][n_rows][C], the view layout
// the reference's FDK filter walks (FDK/GPURecon_GPU.cu:211).  Voxel centres
// are x = xmin + dx(i+1/2), y likewise, z = zmin + dz(k+1/2) with
// zmin = -dz*nz/2 (FDK/FBP.cc:86); the source of view v is at height
// view_z[v] (0 when the plan has no per-view heights, the reference's
// FDK/GPURecon_GPU.cu:226).
#include <cfloat>
#include <climits>

#include "cellwalk.cuh"
#include "colprec.cuh"
#include "fp_body.cuh"

// Cone FP launch shape and per-row arithmetic (one clinical volume, CUDA
// events): 6 detector rows per lane, the per-row update in f32x2 pairs, 7
// resident blocks per SM: 80.7 ms, against 94.4 ms for 8 rows in scalar FP32
// at the compiler's 96 registers in the same run (8 rows + pairs + 6 blocks
// 82.4, 4 rows + pairs + 8 blocks 83.4, 12 / 16 rows 90.5 / 100.3)
#ifndef CT_CONE_FP_ROWS
#define CT_CONE_FP_ROWS 6
#endif
#ifndef CT_CONE_FP_PAIRS
#define CT_CONE_FP_PAIRS 1
#endif

namespace ctk {
namespace {

constexpr int kThreads = 256;

struct ConeArgs {
    int V, C, nx, ny, nz, n_rows;
    float xmin, ymin, dx, dy, zmin, dz;
    float R, D;
    float inv_dcol, pos_off, fC;  // column coordinate y = atan*inv_dcol + pos_off = col + 1/2
    float row_scale;              // D / drow
    float row_off;                // -det_bottom / drow + 1/2: row + 1/2 = z*row_scale/U + row_off
    double fov_r2;
    float coef[9];
    int atan_deg;
    // fixed-point bounds of the transposes (see cone_bp_transpose_kernel);
    // fix_edge: slices that can reach the first or last row (nz when samples
    // can clamp onto them, fix_slices otherwise)
    float fix_npix, fix_slices, fix_wmax, fix_edge;
};

template <int DEG>
__device__ __forceinline__ float cone_atan(float z, const ConeArgs &a) {
    if constexpr (DEG == 0) {
        return atanf(z);
    } else {
        const float s = z * z;
        float p = a.coef[DEG];
#pragma unroll
        for (int k = DEG - 1; k >= 0; --k) p = fmaf(p, s, a.coef[k]);
        return z * p;
    }
}

// y >= 0: i = trunc(y), f = frac(y) without conversion instructions.
__device__ __forceinline__ void split_pos(float y, int &i, float &f) {
    const float m = __fadd_rz(y, 12582912.0f);
    i = __float_as_int(m) - 0x4B400000;
    f = y - (m - 12582912.0f);
}

// The texture unit's 2-D weights (tex2D with linear filtering, the reference's
// FDK/GPURecon_GPU.cu:45): A, B = the column and row fractions in 1/256
// (tex_weight * 256); the far corner gets round(A B / 256) and the other
// three complete exact row and column sums (measured on GB300).  Returns
// w00 (r0, i0), w01 (r0, i1), w10 (r1, i0), w11 (r1, i1), in units of 1/256.
__device__ __forceinline__ float4 tex_weights2d(float A, float B) {
    const float w11 = floorf(fmaf(A, B, 128.0f) * (1.0f / 256.0f));
    return make_float4(256.0f - A - B + w11, A - w11, B - w11, w11);
}

// Slices per thread of cone_bp_kernel.  The row coordinate of slice k is
// formed from the height of its group's first slice, group_z(k & ~(kZC-1)),
// plus (k mod kZC) row steps; the transpose forms it the same way, so both
// sample each slice at the same fp32 row coordinate.  Measured per two
// clinical volumes (CUDA events): 16 slices, 6 blocks per SM: FDK 33.3 ms,
// FDK adjoint 58.9 ms; 8 slices, 7 blocks: 32.2 / 56.4 ms (6 blocks: 39.0 ms
// FDK).
#ifndef CT_CONE_ZC
#define CT_CONE_ZC 8
#endif
constexpr int kZC = CT_CONE_ZC;
__device__ __forceinline__ float group_z(const ConeArgs &a, int k0) {
    return fmaf(a.dz, (float)k0 + 0.5f, a.zmin);
}

// ---- CB_EA backprojection ----------------------------------------------------
// Thread = one (x, y) pixel and ZC consecutive z slices; block = 32 x 8 pixels.
// Per view the column, the 1/(U^2+t^2) weight and the row slope are computed
// once; each slice then needs one row coordinate and a bilinear (col, row)
// sample of the view (FDK/GPURecon_GPU.cu:33-47).
// QUAD: the samples come from the views' quad images (one volume), where cell
// (ir, ic) holds the four clamped taps (r0, i0), (r1, i0), (r0, i1), (r1, i1)
// of row and column positions ir, ic: one 16-byte load per sample instead of
// four 4-byte gathers, the same four values, and the two column lerps (rows
// r0 and r1) as one f32x2 pair: the same operations per lane as the scalar
// form, so the same bits.
// Resident blocks of 256 threads per SM.  With 16 slices per thread, 6 (40
// registers) gave 17.9 ms per clinical FDK volume, where the compiler's own
// choice (74-80 registers) took 32.4 ms and 5 blocks 21.0 ms; with 8 slices
// per thread, 7 blocks (32 registers).
#ifndef CT_CONE_BP_MINB
#define CT_CONE_BP_MINB 7
#endif
template <int ZC, int DEG, bool TEX, bool QUAD>
__global__ void __launch_bounds__(kThreads, CT_CONE_BP_MINB)
    cone_bp_kernel(const float *__restrict__ proj, const float4 *__restrict__ pq,
                   float *__restrict__ vol, const float2 *__restrict__ view_cs,
                   const float *__restrict__ view_z, ConeArgs a, int batch) {
    const int ix = blockIdx.x * 32 + threadIdx.x;
    const int iy = blockIdx.y * 8 + threadIdx.y;
    const int zgroups = (a.nz + ZC - 1) / ZC;
    const int b = blockIdx.z / zgroups;
    const int k0 = (blockIdx.z - b * zgroups) * ZC;
    const double xd = (double)a.xmin + (double)a.dx * (ix + 0.5);
    const double yd = (double)a.ymin + (double)a.dy * (iy + 0.5);
    const bool in = b < batch && ix < a.nx && iy < a.ny && (xd * xd + yd * yd <= a.fov_r2);
    const float px = (float)xd, py = (float)yd;
    float acc[ZC];
#pragma unroll
    for (int k = 0; k < ZC; ++k) acc[k] = 0.0f;
    const size_t pview = (size_t)a.n_rows * a.C;
    if (__syncthreads_or(in) && in) {
        const float *pb = proj + (size_t)b * a.V * pview;
        const float z0 = group_z(a, k0);
        const float rmax = (float)a.n_rows;
        for (int v = 0; v < a.V; ++v) {
            const float2 cs = __ldg(view_cs + v);
            const float U = fmaf(px, cs.x, fmaf(py, cs.y, a.R));
            const float t = fmaf(py, cs.x, -px * cs.y);
            const float rU = __fdividef(1.0f, U);
            const float y = fmaf(cone_atan<DEG>(t * rU, a), a.inv_dcol, a.pos_off);
            if (!(y > 0.5f && y < a.fC + 0.5f)) continue;
            int ic;
            float f;
            split_pos(y, ic, f);
            const unsigned long long ff = pack2(f, f);
            const float A = floorf(fmaf(f, 256.0f, 0.5f));  // used with TEX only
            const int i0 = max(ic - 1, 0), i1 = min(ic, a.C - 1);
            const float wgt = __fdividef(1.0f, fmaf(U, U, t * t));
            const float *pv = pb + (size_t)v * pview;
            const float4 *qv = QUAD ? pq + (size_t)v * (a.n_rows + 1) * (a.C + 1) + ic : pq;
            // row + 1/2 of slice k0 + kk: rr0 + kk * drr
            const float slope = a.row_scale * rU;
            const float zs = view_z ? __ldg(view_z + v) : 0.0f;
            const float rr0 = fmaf(z0 - zs, slope, a.row_off);
            const float drr = a.dz * slope;
#pragma unroll
            for (int kk = 0; kk < ZC; ++kk) {
                if (k0 + kk >= a.nz) break;
                // clamp rows (the reference's texture clamps; no row range test)
                const float rr = fminf(fmaxf(fmaf((float)kk, drr, rr0), 0.0f), rmax + 0.5f);
                int ir;
                float fr;
                split_pos(rr, ir, fr);
                float va0, va1, vc0, vc1;
                if constexpr (QUAD) {
                    const bool ok = (unsigned)ir <= (unsigned)a.n_rows &&
                                    (unsigned)ic <= (unsigned)a.C;
                    const float4 t = CT_DLOAD(ok, qv + (size_t)ir * (a.C + 1));
                    if constexpr (!TEX) {
                        // (lo, hi) = the column lerps of rows r0 and r1
                        const unsigned long long p0 = pack2(t.x, t.y), p1 = pack2(t.z, t.w);
                        const float2 lh = unpack2(fma2(ff, sub2(p1, p0), p0));
                        acc[kk] = fmaf(fmaf(fr, lh.y - lh.x, lh.x), wgt, acc[kk]);
                        continue;
                    }
                    va0 = t.x;
                    vc0 = t.y;
                    va1 = t.z;
                    vc1 = t.w;
                } else {
                    const int r0 = min(max(ir - 1, 0), a.n_rows - 1), r1 = min(ir, a.n_rows - 1);
                    const float *ra = pv + (size_t)r0 * a.C, *rc = pv + (size_t)r1 * a.C;
                    va0 = __ldg(ra + i0);
                    va1 = __ldg(ra + i1);
                    vc0 = __ldg(rc + i0);
                    vc1 = __ldg(rc + i1);
                }
                if constexpr (TEX) {
                    const float4 w = tex_weights2d(A, floorf(fmaf(fr, 256.0f, 0.5f)));
                    const float val = fmaf(w.x, va0, fmaf(w.y, va1, fmaf(w.z, vc0, w.w * vc1)));
                    acc[kk] = fmaf(val * (1.0f / 256.0f), wgt, acc[kk]);
                } else {
                    const float lo = fmaf(f, va1 - va0, va0), hi = fmaf(f, vc1 - vc0, vc0);
                    acc[kk] = fmaf(fmaf(fr, hi - lo, lo), wgt, acc[kk]);
                }
            }
        }
    }
    if (b < batch && ix < a.nx && iy < a.ny) {
        float *vb = vol + (size_t)b * a.nz * a.ny * a.nx;
#pragma unroll
        for (int kk = 0; kk < ZC; ++kk)
            if (k0 + kk < a.nz) vb[((size_t)(k0 + kk) * a.ny + iy) * a.nx + ix] = acc[kk];
    }
}

// Quad images of the views of one volume: [V][n_rows+1][C+1] float4, cell
// (ir, ic) = taps (r0, i0), (r1, i0), (r0, i1), (r1, i1) with
// r0 = min(max(ir-1, 0), n_rows-1), r1 = min(ir, n_rows-1), i0 = max(ic-1, 0),
// i1 = min(ic, C-1): cone_bp_kernel's clamped taps for row and column
// positions ir in [0, n_rows] and ic in [0, C].
__global__ void __launch_bounds__(256)
    cone_proj_quads_kernel(const float *__restrict__ proj, float4 *__restrict__ pq, int R,
                           int C) {
    const int ic = blockIdx.x * 256 + threadIdx.x, ir = blockIdx.y, v = blockIdx.z;
    if (ic > C) return;
    const int i0 = max(ic - 1, 0), i1 = min(ic, C - 1);
    const int r0 = min(max(ir - 1, 0), R - 1), r1 = min(ir, R - 1);
    const float *pv = proj + (size_t)v * R * C;
    const float *ra = pv + (size_t)r0 * C, *rc = pv + (size_t)r1 * C;
    pq[((size_t)v * (R + 1) + ir) * (C + 1) + ic] =
        make_float4(__ldg(ra + i0), __ldg(rc + i0), __ldg(ra + i1), __ldg(rc + i1));
}

// ---- CB_EA transpose ---------------------------------------------------------
// Block = one view and RB detector rows of one volume; the block's rows of
// the view accumulate in shared memory.  Threads sweep the FOV pixels; for
// each they compute column, weight and row slope once and visit only the z
// slices whose row coordinate reaches the block's rows.
// The accumulation is in 32-bit fixed point: FP32 shared-memory atomicAdd is
// a compare-and-swap loop on this GPU, int32 atomicAdd is native.  Every
// contribution is at most max|vol| * w_max (w = 1/L^2, L >= R - rFOV; the
// bilinear weights are <= 1), and a detector cell receives at most npix
// (pixels within two channels of it) x slices (within one row of it) of them,
// so with scale = 2^30 / (npix * slices * max|vol| * w_max) no sum can
// overflow; each contribution is rounded to 1/scale.  Samples whose row
// coordinate is clamped onto the first or last row (slices beyond the
// detector's reach, which can pile up there from every slice) add into two
// separate fixed-point rows whose bound counts all nz slices, so they do not
// coarsen the others.
constexpr int kRB = 16;
#ifndef CT_CONE_T_TILES
#define CT_CONE_T_TILES 1
#endif

template <int DEG, bool TEX>
__global__ void __launch_bounds__(kThreads)
    cone_bp_transpose_kernel(const float *__restrict__ vol, float *__restrict__ proj,
                             const float2 *__restrict__ view_cs,
                             const float2 *__restrict__ view_cs_lo,
                             const float2 *__restrict__ col_tan, const float *__restrict__ view_z,
                             const int *__restrict__ vmax_bits, ConeArgs a, int batch) {
    // [kRB][C] fixed point, then [2][C]: the first and the last detector row's
    // clamped samples, fixed point at their own scale
    extern __shared__ int rows_acc[];
    int *rows_clamped = rows_acc + kRB * a.C;
    const int rblocks = (a.n_rows + kRB - 1) / kRB;
    const int v = blockIdx.x;
    const int rb = blockIdx.y % rblocks, b = blockIdx.y / rblocks;
    const int R0 = rb * kRB;
    const int nr = min(kRB, a.n_rows - R0);
    for (int k = threadIdx.x; k < (kRB + 2) * a.C; k += kThreads) rows_acc[k] = 0;
    const float vmax = __int_as_float(__ldg(vmax_bits + b));
    const float bound = a.fix_npix * a.fix_slices * a.fix_wmax * vmax;
    const float scale = bound > 0.0f ? 1073741824.0f / bound : 0.0f;
    const float bound_c = a.fix_npix * (float)a.nz * a.fix_wmax * vmax;
    const float scale_c = bound_c > 0.0f ? 1073741824.0f / bound_c : 0.0f;
    __syncthreads();
    const float2 cs = __ldg(view_cs + v);
    const float2 csl = __ldg(view_cs_lo + v);
    const float zfirst = a.zmin + 0.5f * a.dz - (view_z ? __ldg(view_z + v) : 0.0f);
    const float *vb = vol + (size_t)b * a.nz * a.ny * a.nx;
    const float rmax = (float)a.n_rows;
    const size_t plane = (size_t)a.nx * a.ny;
    // a warp takes a 4 x 8 pixel tile whose short side runs along the view's
    // rays: pixels along a ray share detector columns, so the lanes of a warp
    // spread over 8 columns instead of competing for a few
    const bool along_x = fabsf(cs.x) > fabsf(cs.y);
    const int tw = CT_CONE_T_TILES ? (along_x ? 4 : 8) : 32, th = 32 / tw;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ntx = (a.nx + tw - 1) / tw, ntiles = ntx * ((a.ny + th - 1) / th);
    for (int tile = warp; tile < ntiles; tile += kThreads / 32) {
        const int ty = tile / ntx, tx = tile - ty * ntx;
        const int ix = tx * tw + lane % tw, iy = ty * th + lane / tw;
        if (ix >= a.nx || iy >= a.ny) continue;
        const int p = iy * a.nx + ix;
        const double xd = (double)a.xmin + (double)a.dx * (ix + 0.5);
        const double yd = (double)a.ymin + (double)a.dy * (iy + 0.5);
        if (!(xd * xd + yd * yd <= a.fov_r2)) continue;
        const float px = (float)xd, py = (float)yd;
        const float U = fmaf(px, cs.x, fmaf(py, cs.y, a.R));
        const float t = fmaf(py, cs.x, -px * cs.y);
        const float rU = __fdividef(1.0f, U);
        const float y = fmaf(cone_atan<DEG>(t * rU, a), a.inv_dcol, a.pos_off);
        if (!(y > 0.5f && y < a.fC + 0.5f)) continue;
        int ic;
        float f;
        split_pos(y, ic, f);
        const float A = floorf(fmaf(f, 256.0f, 0.5f));  // used with TEX only
        if constexpr (TEX) {
            f = A * (1.0f / 256.0f);
        } else {  // the column fraction from float-float geometry (colprec.cuh)
            FF Uf, tf;
            ff_ut(px, (float)(xd - (double)px), py, (float)(yd - (double)py), cs.x, csl.x, cs.y,
                  csl.y, a.R, Uf, tf);
            precise_strip(Uf, tf, col_tan, a.inv_dcol, a.C, ic, f);
        }
        const int i0 = max(ic - 1, 0), i1 = min(ic, a.C - 1);
        const float wgt = __fdividef(1.0f, fmaf(U, U, t * t));
        const float slope = a.row_scale * rU;
        const float rr_first = fmaf(zfirst, slope, a.row_off);  // slice 0
        const float drr = a.dz * slope;
        // slices whose row coordinate (clamped) touches rows [R0-1, R0+nr]:
        // rr in (R0 - 0.5, R0 + nr + 0.5], widened by one slice each way
        int klo = 0, khi = a.nz;
        if (drr > 0.0f) {
            const float lo = floorf((R0 - 1.0f - rr_first) / drr);
            const float hi = ceilf((R0 + nr + 1.0f - rr_first) / drr) + 1.0f;
            klo = (int)fminf(fmaxf(lo, 0.0f), (float)a.nz);
            khi = (int)fminf(fmaxf(hi, 0.0f), (float)a.nz);
            if (R0 == 0) klo = 0;
            if (R0 + nr >= a.n_rows) khi = a.nz;
        }
        for (int k = klo; k < khi; ++k) {
            const float val = __ldg(vb + (size_t)k * plane + p) * wgt;
            if (val == 0.0f) continue;
            const float rr = fminf(fmaxf(fmaf((float)k, drr, rr_first), 0.0f), rmax + 0.5f);
            int ir;
            float fr;
            split_pos(rr, ir, fr);
            const int r0 = min(max(ir - 1, 0), a.n_rows - 1) - R0;
            const int r1 = min(ir, a.n_rows - 1) - R0;
            if (ir < 1 || ir >= a.n_rows) {
                // clamped onto an edge row: both row taps are that row
                const int e = ir < 1 ? 0 : 1, re = e ? a.n_rows - 1 : 0;
                if ((unsigned)(re - R0) < (unsigned)nr) {
                    const float vc = val * scale_c;
                    atomicAdd(&rows_clamped[e * a.C + i0], __float2int_rn(vc * (1.0f - f)));
                    atomicAdd(&rows_clamped[e * a.C + i1], __float2int_rn(vc * f));
                }
                continue;
            }
            const float vs = val * scale;
            float w00, w01, w10, w11;  // (r0, i0), (r0, i1), (r1, i0), (r1, i1)
            if constexpr (TEX) {
                const float4 w = tex_weights2d(A, floorf(fmaf(fr, 256.0f, 0.5f)));
                w00 = w.x * (1.0f / 256.0f);
                w01 = w.y * (1.0f / 256.0f);
                w10 = w.z * (1.0f / 256.0f);
                w11 = w.w * (1.0f / 256.0f);
            } else {
                w00 = (1.0f - fr) * (1.0f - f);
                w01 = (1.0f - fr) * f;
                w10 = fr * (1.0f - f);
                w11 = fr * f;
            }
            if ((unsigned)r0 < (unsigned)nr) {
                atomicAdd(&rows_acc[r0 * a.C + i0], __float2int_rn(vs * w00));
                atomicAdd(&rows_acc[r0 * a.C + i1], __float2int_rn(vs * w01));
            }
            if ((unsigned)r1 < (unsigned)nr) {
                atomicAdd(&rows_acc[r1 * a.C + i0], __float2int_rn(vs * w10));
                atomicAdd(&rows_acc[r1 * a.C + i1], __float2int_rn(vs * w11));
            }
        }
    }
    __syncthreads();
    float *pv = proj + ((size_t)b * a.V + v) * a.n_rows * a.C;
    const float inv = scale > 0.0f ? bound * (1.0f / 1073741824.0f) : 0.0f;
    const float inv_c = scale_c > 0.0f ? bound_c * (1.0f / 1073741824.0f) : 0.0f;
    for (int k = threadIdx.x; k < nr * a.C; k += kThreads) {
        const int row = R0 + k / a.C, col = k - (k / a.C) * a.C;
        float c = 0.0f;
        if (row == 0) c += (float)rows_clamped[col] * inv_c;
        if (row == a.n_rows - 1) c += (float)rows_clamped[a.C + col] * inv_c;
        pv[(size_t)R0 * a.C + k] = fmaf((float)rows_acc[k], inv, c);
    }
}

// vmax_bits[b] = bits of max |vol[b]| (non-negative floats order as their bits);
// vmax_bits must start at zero.
__global__ void __launch_bounds__(256)
    volume_absmax_kernel(const float *__restrict__ vol, size_t per_volume, int *vmax_bits) {
    const float *vb = vol + (size_t)blockIdx.y * per_volume;
    float m = 0.0f;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < per_volume;
         e += (size_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(__ldg(vb + e)));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(vmax_bits + blockIdx.y, __float_as_int(m));
}

// ---- CB_EA transpose, lanes along z --------------------------------------------
// Used when all detector rows of a view fit in shared memory.  Block = one
// view of one volume, with its [C][n_rows] fixed-point accumulators
// (column-major with an odd column stride, so that neither the lanes' row
// updates nor the write-out across a row conflict in the banks).  A lane
// takes 8 consecutive slices of one pixel, read as two float4 from a z-major
// copy of the volume; a warp takes 32 / 2^lg pixels of an image row (2^lg
// lanes per pixel, 4 pixels for 64 slices).  Along its slices a lane's
// detector rows only move forward, so it keeps the last row it touched in
// registers and adds each row to shared memory once it is complete: for a
// row step of about one row per slice that is two atomics per slice instead
// of four.  Row indices and weights follow cone_bp_kernel exactly (rows
// clamped onto the first and last row included).  Rows 0 and n_rows-1 are
// kept at a fixed-point scale whose bound counts all nz slices where samples
// can clamp onto them, the other rows at the fine one.
#ifndef CT_CONE_ZT_THREADS
#define CT_CONE_ZT_THREADS 1024
#endif
constexpr int kZThreads = CT_CONE_ZT_THREADS;
#ifndef CT_CONE_ZS
#define CT_CONE_ZS 8
#endif
constexpr int kZS = CT_CONE_ZS;  // consecutive slices per lane (8 or 16)
constexpr int kZQ = kZS / 4;     // their float4 loads

// [B][nz][ny*nx] -> [B][ny*nx][nzp] (nzp = nz rounded up to kZS, zero-filled),
// and per volume max |vol| into vmax_bits (which must start at zero).
__global__ void __launch_bounds__(256)
    cone_zmajor_kernel(const float *__restrict__ vol, float *__restrict__ vol_t,
                       int *vmax_bits, int nz, int npix, int nzp) {
    __shared__ float tile[32][33];
    const int p0 = blockIdx.x * 32, kc = blockIdx.y * 32, b = blockIdx.z;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const float *vb = vol + (size_t)b * nz * npix;
    float m = 0.0f;
#pragma unroll
    for (int j = ty; j < 32; j += 8) {
        const int k = kc + j, p = p0 + tx;
        const float x = (k < nz && p < npix) ? __ldg(vb + (size_t)k * npix + p) : 0.0f;
        tile[j][tx] = x;
        m = fmaxf(m, fabsf(x));
    }
    __syncthreads();
    float *tb = vol_t + (size_t)b * npix * nzp;
#pragma unroll
    for (int j = ty; j < 32; j += 8) {
        const int p = p0 + j;
        if (p < npix && kc + tx < nzp) tb[(size_t)p * nzp + kc + tx] = tile[tx][j];
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (tx == 0 && m > 0.0f) atomicMax(vmax_bits + b, __float_as_int(m));
}

// Per image row iy: the fp32 pixel centre py[iy] (and its rounding, pyl[iy])
// and the span [lo, hi) of columns whose centres lie in the FOV disc (an
// interval: the test is monotone in |x|); px[ix], pxl[ix] likewise.  Same double expressions as
// cone_bp_kernel's FOV test, so both select the same pixels.
__global__ void __launch_bounds__(32)
    cone_fov_tables_kernel(ConeArgs a, float *__restrict__ px_tab, float *__restrict__ py_tab,
                           float *__restrict__ pxl_tab, float *__restrict__ pyl_tab,
                           int2 *__restrict__ span) {
    const int iy = blockIdx.x, lane = threadIdx.x;
    const double yd = (double)a.ymin + (double)a.dy * (iy + 0.5);
    int lo = INT_MAX, hi = -1;
    for (int x0 = 0; x0 < a.nx; x0 += 32) {
        const int ix = x0 + lane;
        const double xd = (double)a.xmin + (double)a.dx * (ix + 0.5);
        if (ix < a.nx && (xd * xd + yd * yd <= a.fov_r2)) {
            lo = min(lo, ix);
            hi = max(hi, ix);
        }
        if (iy == 0 && ix < a.nx) {
            px_tab[ix] = (float)xd;
            pxl_tab[ix] = (float)(xd - (double)(float)xd);
        }
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (lane == 0) {
        span[iy] = hi >= 0 ? make_int2(lo, hi + 1) : make_int2(0, 0);
        py_tab[iy] = (float)yd;
        pyl_tab[iy] = (float)(yd - (double)(float)yd);
    }
}

// Column pairs (i0, i1) in one 64-bit register for the f32x2 instructions
// (each lane rounds as the FP32 instruction does; 27.35 -> 26.80 ms per
// clinical FDK adjoint against the scalar form).
__device__ __forceinline__ unsigned long long zt_pack(float x, float y) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
    return r;
}
__device__ __forceinline__ float2 zt_unpack(unsigned long long r) {
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
    return v;
}
__device__ __forceinline__ unsigned long long zt_mul2(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long zt_add2(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long zt_sub2(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// A warp's pixels: image rows in order, in each the tiles of `per` pixels
// t = (warp + iy) mod NW + NW m of the row's FOV span [x0, end).
struct ZtCursor {
    int iy, t, ntile, x0, end;
    __device__ __forceinline__ bool next(const int2 *__restrict__ span, int ny, int warp, int nw,
                                         int per) {
        t += nw;
        while (t >= ntile) {
            if (++iy >= ny) return false;
            const int2 sp = __ldg(span + iy);
            x0 = sp.x;
            end = sp.y;
            ntile = (sp.y - sp.x + per - 1) / per;
            t = (warp + iy) % nw;
        }
        return true;
    }
};

template <int DEG, bool TEX>
__global__ void __launch_bounds__(kZThreads, 1)
    cone_bp_transpose_z_kernel(const float *__restrict__ vol_t, float *__restrict__ proj,
                               const float2 *__restrict__ view_cs,
                               const float2 *__restrict__ view_cs_lo,
                               const float2 *__restrict__ col_tan,
                               const float *__restrict__ view_z, const int *__restrict__ vmax_bits,
                               const float *__restrict__ px_tab, const float *__restrict__ py_tab,
                               const float *__restrict__ pxl_tab, const float *__restrict__ pyl_tab,
                               const int2 *__restrict__ span, ConeArgs a, int nzp, int lg) {
    extern __shared__ int4 acc4[];
    int *acc = reinterpret_cast<int *>(acc4);
    const int ld = a.n_rows | 1;
    const int nacc4 = (a.C * ld + 3) / 4;
    for (int k = threadIdx.x; k < nacc4; k += kZThreads) acc4[k] = make_int4(0, 0, 0, 0);
    const int v = blockIdx.x, b = blockIdx.y;
    const float vmax = __int_as_float(__ldg(vmax_bits + b));
    const float bound = a.fix_npix * a.fix_slices * a.fix_wmax * vmax;
    const float scale = bound > 0.0f ? 1073741824.0f / bound : 0.0f;
    const float bound_c = a.fix_npix * a.fix_edge * a.fix_wmax * vmax;
    const float scale_c = bound_c > 0.0f ? 1073741824.0f / bound_c : 0.0f;
    __syncthreads();
    const float2 cs = __ldg(view_cs + v);
    const float2 csl = __ldg(view_cs_lo + v);
    const float zs = view_z ? __ldg(view_z + v) : 0.0f;
    const float rmax = (float)a.n_rows;
    const int last = a.n_rows - 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int NW = kZThreads / 32;
    const int gp = 1 << lg, per = 32 >> lg;  // lanes per pixel, pixels per warp
    const int slot = lane >> lg, g = lane & (gp - 1);
    const int G = nzp / kZS;                 // slice groups per pixel
    const float *vb = vol_t + (size_t)b * a.nx * a.ny * nzp;
    const float4 zero4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    auto load = [&](const ZtCursor &c, float4 *x) {
        const int ix = c.x0 + c.t * per + slot;
#pragma unroll
        for (int q = 0; q < kZQ; ++q) x[q] = zero4;
        if (ix < c.end && g < G) {
            const float4 *q4 = reinterpret_cast<const float4 *>(
                vb + ((size_t)c.iy * a.nx + ix) * nzp + g * kZS);
#pragma unroll
            for (int q = 0; q < kZQ; ++q) x[q] = __ldg(q4 + q);
        }
    };
    ZtCursor cur{-1, 0, 0, 0, 0};
    bool have = cur.next(span, a.ny, warp, NW, per);
    float4 va[kZQ];  // this lane's kZS slices of the current pixel
    if (have) load(cur, va);
    // Per-pixel geometry, computed once per pixel instead of once per lane:
    // the warp's next gp tiles hold 32 pixels (per per tile), and lane
    // q*per + s computes tile q's pixel s -- its column strip ic (-1: none),
    // the column fraction f (float-float, colprec.cuh), the 1/(U^2+t^2)
    // weight and the row slope -- which the pixel's gp lanes then read by
    // shuffles (measured: the FDK adjoint's precise column fraction cost
    // 26.8 -> 33.2 ms per clinical volume while every lane computed it).
    int gq = gp;  // tiles of the current geometry batch already used
    int g_ic = -1;
    float g_f = 0.0f, g_w = 0.0f, g_sl = 0.0f;
    auto batch_geometry = [&]() {
        ZtCursor c = cur;
        const int q = lane >> (5 - lg), s_ = lane & (per - 1);
        bool ok = true;
        for (int k = 0; k < q && ok; ++k) ok = c.next(span, a.ny, warp, NW, per);
        g_ic = -1;
        const int ix = c.x0 + c.t * per + s_;
        if (!ok || ix >= c.end) return;
        const float px = __ldg(px_tab + ix), py = __ldg(py_tab + c.iy);
        const float U = fmaf(px, cs.x, fmaf(py, cs.y, a.R));
        const float t = fmaf(py, cs.x, -px * cs.y);
        const float rU = __fdividef(1.0f, U);
        const float y = fmaf(cone_atan<DEG>(t * rU, a), a.inv_dcol, a.pos_off);
        if (!(y > 0.5f && y < a.fC + 0.5f)) return;
        int ic;
        float f;
        split_pos(y, ic, f);
        if constexpr (!TEX) {
            FF trow, urow, Uf, tf;
            ff_row(py, __ldg(pyl_tab + c.iy), cs.x, csl.x, cs.y, csl.y, a.R, trow, urow);
            ff_pixel(px, __ldg(pxl_tab + ix), cs.x, csl.x, cs.y, csl.y, trow, urow, Uf, tf);
            precise_strip(Uf, tf, col_tan, a.inv_dcol, a.C, ic, f);
        }
        g_ic = ic;
        g_f = f;
        g_w = __fdividef(1.0f, fmaf(U, U, t * t));
        g_sl = a.row_scale * rU;
    };
    while (have) {
        // the next tile's loads go out before this tile's work
        ZtCursor nxt = cur;
        const bool more = nxt.next(span, a.ny, warp, NW, per);
        float4 na[kZQ];
        if (more) load(nxt, na);
        if (gq == gp) {  // warp-uniform
            batch_geometry();
            gq = 0;
        }
        const int src = gq * per + slot;
        const int ic = __shfl_sync(0xffffffffu, g_ic, src);
        const float f = __shfl_sync(0xffffffffu, g_f, src);
        const float wgt = __shfl_sync(0xffffffffu, g_w, src);
        const float slope = __shfl_sync(0xffffffffu, g_sl, src);
        ++gq;
        const int ix = cur.x0 + cur.t * per + slot;
        if (ic >= 0 && g < G) {
            {
                const float A = floorf(fmaf(f, 256.0f, 0.5f));  // used with TEX only
                int *c0 = acc + max(ic - 1, 0) * ld;
                int *c1 = acc + min(ic, a.C - 1) * ld;
                const float drr = a.dz * slope;
                const unsigned long long g01 = zt_pack(1.0f - f, f);  // column weights
                const bool cols_ok = (unsigned)ic <= (unsigned)a.C;
                auto emit = [&](int row, unsigned long long X) {
                    const float sc = (unsigned)(row - 1) < (unsigned)(last - 1) ? scale : scale_c;
                    const float2 v = zt_unpack(zt_mul2(X, zt_pack(sc, sc)));
                    if (!CT_DCHECK(cols_ok && (unsigned)row < (unsigned)a.n_rows)) return;
                    atomicAdd(c0 + row, __float2int_rn(v.x));
                    atomicAdd(c1 + row, __float2int_rn(v.y));
                };
                // passes of gp groups (one pass unless nz > 32 * kZS)
                for (int kb = g * kZS; kb < a.nz; kb += gp * kZS) {
                    float x[kZS];
                    if (kb == g * kZS) {
#pragma unroll
                        for (int q = 0; q < kZQ; ++q)
                            x[4 * q] = va[q].x, x[4 * q + 1] = va[q].y, x[4 * q + 2] = va[q].z,
                                   x[4 * q + 3] = va[q].w;
                    } else {
                        const float4 *q4 = reinterpret_cast<const float4 *>(
                            vb + ((size_t)cur.iy * a.nx + ix) * nzp + kb);
#pragma unroll
                        for (int q = 0; q < kZQ; ++q) {
                            const float4 u = __ldg(q4 + q);
                            x[4 * q] = u.x, x[4 * q + 1] = u.y, x[4 * q + 2] = u.z,
                                   x[4 * q + 3] = u.w;
                        }
                    }
                    // the lane's slices lie in one group of kZC (kZS divides kZC)
                    const int kg = kb & ~(kZC - 1);
                    const float rr0 = fmaf(group_z(a, kg) - zs, slope, a.row_off);
                    const float kk0 = (float)(kb - kg);
                    // the pending row and its column pair (i0, i1), packed for f32x2
                    int prow = -1;
                    unsigned long long P = 0ull;
#pragma unroll
                    for (int j = 0; j < kZS; ++j) {
                        // (slices beyond nz read zero and add nothing)
                        const float rr =
                            fminf(fmaxf(fmaf(kk0 + (float)j, drr, rr0), 0.0f), rmax + 0.5f);
                        int ir;
                        float fr;
                        split_pos(rr, ir, fr);
                        const int lo = min(max(ir - 1, 0), last), hi = min(ir, last);
                        const float vw = x[j] * wgt;
                        unsigned long long L, H;  // rows lo and hi, columns (i0, i1)
                        if constexpr (TEX) {
                            const float4 w = tex_weights2d(A, floorf(fmaf(fr, 256.0f, 0.5f)));
                            const float sw = vw * (1.0f / 256.0f);
                            const unsigned long long ss = zt_pack(sw, sw);
                            L = zt_mul2(ss, zt_pack(w.x, w.y));
                            H = zt_mul2(ss, zt_pack(w.z, w.w));
                        } else {
                            const float hb = vw * fr, lb = vw - hb;
                            L = zt_mul2(zt_pack(lb, lb), g01);
                            H = zt_mul2(zt_pack(hb, hb), g01);
                        }
                        const bool flush = prow != lo;
                        if (flush && prow >= 0) emit(prow, P);
                        const unsigned long long Q = flush ? L : zt_add2(P, L);
                        if (hi == lo) {  // both row taps on one row (clamped): keep it
                            P = zt_add2(Q, H);
                        } else {
                            emit(lo, Q);
                            P = H;
                        }
                        prow = hi;
                    }
                    emit(prow, P);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < kZQ; ++q) va[q] = na[q];
        cur = nxt;
        have = more;
    }
    __syncthreads();
    float *pv = proj + ((size_t)b * a.V + v) * a.n_rows * a.C;
    const float inv = scale > 0.0f ? bound * (1.0f / 1073741824.0f) : 0.0f;
    const float inv_c = scale_c > 0.0f ? bound_c * (1.0f / 1073741824.0f) : 0.0f;
    for (int e = threadIdx.x; e < a.n_rows * a.C; e += kZThreads) {
        const int r = e / a.C, c = e - r * a.C;
        pv[e] = (float)acc[c * ld + r] * ((unsigned)(r - 1) < (unsigned)(last - 1) ? inv : inv_c);
    }
}

// ---- cone-beam forward projection -----------------------------------------------
// Warp = 32 consecutive channels of one view, as in the fan-beam projector:
// the warp walks its rays' in-plane cells row-synchronously over quad images
// of every slice (layout 0, or the transposed layout 1 when most rays run
// along x) and, per lane, handles RB detector rows at once.  Detector row r
// sits at height h_r = det_bottom + (r+1/2) drow on the cylinder of radius D
// about the source; at in-plane distance s from the source the ray is at
// height z = z_s + h_r s / D, so its z cell coordinate is w0 + dw k in the
// sample index k.
// Inside an in-plane cell the four bilinear weights are quadratics q_c(j) in
// the sample offset j, and the z fraction is cz + dw j.  Per cell the walk
// forms W_c = sum q_c(j) and M_c = sum j q_c(j) once (from sum j^m, m <= 3);
// a detector row whose z cell does not change inside the cell (all but a few
// percent) then adds
//   sum_c [(W_c (1 - cz) - dw M_c) t0_c + (W_c cz + dw M_c) t1_c]
// with t0, t1 the cell's quads of slices kz and kz+1 (two 16-byte loads).
// No row may cross a z boundary inside the samples summed this way, so the
// walk also ends a segment where any of the lane's rows enters a new z cell
// (per row it keeps the sample index of its next crossing): segments are the
// in-plane cells cut at those indices, each summed from its first sample's
// fractions.  Handling the few crossing rows separately instead (a branch per
// row and cell) idled most lanes of a warp on almost every cell.
// Weight: 0.125*dx*sqrt(1 + (h_r/D)^2), the 3-D length of one in-plane step.
// Bound on the segments of one image row (x cells and z crossings); every
// step makes progress, so this only guards against a malformed geometry.
constexpr int kConeSteps = 64;

struct ConeFpArgs {
    int V, C, nx, ny, nz, n_rows, wpv;
    float w;        // 0.125*dx
    float D, det_bottom, drow, dz, zmin;
    int max_iter;
};

// sum over j in [js, je) of j^0..j^3
__device__ __forceinline__ void power_sums(float js, float je, float &S0, float &S1, float &S2,
                                           float &S3) {
    auto p1 = [](float n) { return 0.5f * n * (n + 1.0f); };  // sum_{0..n} j
    auto p2 = [](float n) { return n * (n + 1.0f) * (2.0f * n + 1.0f) * (1.0f / 6.0f); };
    S0 = je - js;
    S1 = p1(je - 1.0f) - p1(js - 1.0f);
    S2 = p2(je - 1.0f) - p2(js - 1.0f);
    const float a = p1(je - 1.0f), b = p1(js - 1.0f);
    S3 = a * a - b * b;
}

__device__ __forceinline__ float dot4(float4 a, float4 t) {
    return fmaf(a.x, t.x, fmaf(a.y, t.y, fmaf(a.z, t.z, a.w * t.w)));
}

// moments sum q_c(j) j^m over a piece, from its power sums: c0 S_m + c1 S_{m+1} + c2 S_{m+2}
__device__ __forceinline__ float4 moment(float4 c0, float4 c1, float4 c2, float Sa, float Sb,
                                         float Sc) {
    return make_float4(fmaf(c0.x, Sa, fmaf(c1.x, Sb, c2.x * Sc)),
                       fmaf(c0.y, Sa, fmaf(c1.y, Sb, c2.y * Sc)),
                       fmaf(c0.z, Sa, fmaf(c1.z, Sb, c2.z * Sc)),
                       fmaf(c0.w, Sa, fmaf(c1.w, Sb, c2.w * Sc)));
}

// 128-thread blocks: at ~96 registers they fill an SM with 20 warps where
// 256-thread blocks stop at 16 (measured 143 -> 108 ms per clinical volume).
constexpr int kConeFpThreads = 128;

#ifndef CT_CONE_FP_MINB
#define CT_CONE_FP_MINB 7
#endif
template <int RB>
__global__ void __launch_bounds__(kConeFpThreads, CT_CONE_FP_MINB)
    cone_fp_kernel(const float4 *__restrict__ quads, float *__restrict__ proj,
                   const float4 *__restrict__ ray, const int *__restrict__ nsamp,
                   const float2 *__restrict__ chan_s, const float *__restrict__ view_z,
                   ConeFpArgs a) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    // a block is one channel group of adjacent views, blocks channel-group-major
    // (as the fan-beam projector; 98.5 -> 87.3 ms per clinical volume)
    constexpr int NV = kConeFpThreads / 32;
    const int nvg = (a.V + NV - 1) / NV;
    const int cgroup = blockIdx.x / nvg, vgroup = blockIdx.x - cgroup * nvg;
    const int vv = vgroup * NV + (threadIdx.x >> 5);
    if (vv >= a.V) return;  // warp-uniform
    const int gw = vv * a.wpv + cgroup;
    const int r0 = blockIdx.y * RB;
    const int v = gw / a.wpv;
    const int c = (gw - v * a.wpv) * 32 + lane;
    const bool has_c = c < a.C;
    const int r = v * a.C + (has_c ? c : a.C - 1);
    const int n = has_c ? __ldg(nsamp + r) : 0;
    const bool valid = n > 0;
    const float4 q = valid ? __ldg(ray + r) : make_float4(0.f, 0.f, 0.f, 0.f);
    const unsigned vm = __ballot_sync(FULL, valid);
    const unsigned xm = __ballot_sync(FULL, valid && fabsf(q.z) > fabsf(q.w));
    const bool along_x = 2 * __popc(xm) > __popc(vm);
    const RaySeg seg = along_x ? RaySeg{q.y - 0.5f, q.x - 0.5f, q.w, q.z}
                               : RaySeg{q.x - 0.5f, q.y - 0.5f, q.z, q.w};
    const int Q = a.nx + 1;
    const size_t lsz = (size_t)Q * Q, sstride = 2 * lsz;
    // slice k's quads of this warp's layout: ql + k * 2 lsz
    const float4 *ql = quads + (along_x ? lsz : 0);
    // z cell coordinate of sample k for row rr: w0[rr] + dw[rr] * k; in-plane
    // distance from the source of sample k: s0 - k * chord / n (mm)
    const float2 sd = has_c ? __ldg(chan_s + c) : make_float2(0.f, 0.f);
    const float ds = valid ? -sd.y / (float)n : 0.0f;
    const float zs = view_z ? __ldg(view_z + v) : 0.0f;
    const float INF = __int_as_float(0x7f800000);
    float w0[RB], dw[RB], acc[RB];
#pragma unroll
    for (int rr = 0; rr < RB; ++rr) {
        const float h = a.det_bottom + a.drow * ((float)(r0 + rr) + 0.5f);
        w0[rr] = (h * sd.x / a.D + zs - a.zmin) / a.dz - 0.5f;
        dw[rr] = h * ds / (a.D * a.dz);
        acc[rr] = 0.0f;
    }
    // the first sample index after k whose z cell differs from sample k's, for
    // row rr (INF if the row's z never changes); at least k + 1
    auto next_z = [&](int rr, float k) {
        const float d = dw[rr];
        if (r0 + rr >= a.n_rows || d == 0.0f) return INF;
        // the split's exact position does not matter (the interpolant is
        // continuous), so the fast reciprocal divide serves
        const float kzc = floorf(fmaf(d, k, w0[rr]));
        const float ks = d > 0.0f ? ceilf(__fdividef(kzc + 1.0f - w0[rr], d))
                                  : floorf(__fdividef(kzc - w0[rr], d)) + 1.0f;
        return fmaxf(ks, k + 1.0f);
    };
    // adds the segment of cell (cu, cv) holding samples k .. k+cnt-1 (no row
    // changes z cell inside it) with entry fractions fa, fb
    auto cell = [&](int cu, int cv, float cnt, float fa, float fb, float k) {
        // bilinear weights as quadratics in j: (1-fu)(1-fv), fu(1-fv), (1-fu)fv, fu fv
        const float Au = 1.0f - fa, Av = 1.0f - fb, uv = seg.su * seg.sv;
        const float4 c0 = make_float4(Au * Av, fa * Av, Au * fb, fa * fb);
        const float4 c1 = make_float4(-(Au * seg.sv + Av * seg.su), seg.su * Av - fa * seg.sv,
                                      Au * seg.sv - seg.su * fb, fa * seg.sv + fb * seg.su);
        const float4 c2 = make_float4(uv, -uv, -uv, uv);
        const int qi = min(max(cu + 1, 0), Q - 1), qj = min(max(cv + 1, 0), Q - 1);
        const float4 *qc = ql + (size_t)qj * Q + qi;
        float S0, S1, S2, S3;
        power_sums(0.0f, cnt, S0, S1, S2, S3);
        const float4 W = moment(c0, c1, c2, S0, S1, S2), M = moment(c0, c1, c2, S1, S2, S3);
#if CT_CONE_FP_PAIRS
        const unsigned long long W01 = pack2(W.x, W.y), W23 = pack2(W.z, W.w);
        const unsigned long long M01 = pack2(M.x, M.y), M23 = pack2(M.z, M.w);
#endif
#pragma unroll
        for (int rr = 0; rr < RB; ++rr) {
            if (r0 + rr >= a.n_rows) break;
            const float wk = fmaf(dw[rr], k, w0[rr]);
            const float kz = floorf(wk);
            const float cz = wk - kz, d = dw[rr];
            const int z0 = min(max((int)kz, 0), a.nz - 1);
            const int z1 = min(max((int)kz + 1, 0), a.nz - 1);
            const bool ok = (unsigned)(cu + 1) < (unsigned)Q && (unsigned)(cv + 1) < (unsigned)Q;
            const float4 t0 = CT_DLOAD(ok, qc + (size_t)z0 * sstride);
            const float4 t1 = CT_DLOAD(ok, qc + (size_t)z1 * sstride);
#if CT_CONE_FP_PAIRS
            // W.t0 + (cz W + d M).(t1 - t0) in f32x2 pairs (x, y), (z, w)
            const unsigned long long d01 = zt_sub2(pack2(t1.x, t1.y), pack2(t0.x, t0.y));
            const unsigned long long d23 = zt_sub2(pack2(t1.z, t1.w), pack2(t0.z, t0.w));
            const unsigned long long czp = pack2(cz, cz), dp = pack2(d, d);
            const unsigned long long e01 = fma2(czp, W01, zt_mul2(dp, M01));
            const unsigned long long e23 = fma2(czp, W23, zt_mul2(dp, M23));
            unsigned long long s2 = zt_mul2(W01, pack2(t0.x, t0.y));
            s2 = fma2(W23, pack2(t0.z, t0.w), s2);
            s2 = fma2(e01, d01, s2);
            s2 = fma2(e23, d23, s2);
            const float2 sv = unpack2(s2);
            acc[rr] += sv.x + sv.y;
#else
            const float4 B = make_float4(fmaf(W.x, cz, d * M.x), fmaf(W.y, cz, d * M.y),
                                         fmaf(W.z, cz, d * M.z), fmaf(W.w, cz, d * M.w));
            const float4 A = make_float4(W.x - B.x, W.y - B.y, W.z - B.z, W.w - B.w);
            acc[rr] += dot4(A, t0) + dot4(B, t1);
#endif
        }
    };
    const unsigned pm = __ballot_sync(FULL, valid && seg.sv > 0.0f);
    const int dir = 2 * __popc(pm) >= __popc(vm) ? 1 : -1;
    const bool synced = valid && (dir > 0 ? seg.sv > 0.0f : seg.sv < 0.0f);
    const float nf = (float)n;
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
    float kzn[RB];  // next z crossing per row, from sample 0
#pragma unroll
    for (int rr = 0; rr < RB; ++rr) kzn[rr] = next_z(rr, 0.0f);
    auto next_crossing = [&]() {
        float m = kzn[0];
#pragma unroll
        for (int rr = 1; rr < RB; ++rr) m = fminf(m, kzn[rr]);
        return m;
    };
    auto advance_z = [&](float k) {
#pragma unroll
        for (int rr = 0; rr < RB; ++rr)
            if (kzn[rr] <= k) kzn[rr] = next_z(rr, k);
    };
    if (__any_sync(FULL, synced)) {
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
            // each step reaches the next x boundary, z crossing or the row's
            // end: k grows or the x cell advances
            for (int t = 0; t < kConeSteps && k < kb; ++t) {
                const float tu = seg.su != 0.0f ? (bu - seg.u0) * iu : INF;
                const float kx = ceilf(tu);
                const float kzm = next_crossing();
                const float ke = fminf(fminf(kb, kx), kzm);
                if (ke > k) {
                    cell((int)cu, j, ke - k, fmaf(seg.su, k, seg.u0) - cu,
                         fmaf(seg.sv, k, seg.v0) - (float)j, k);
                    k = ke;
                    if (ke >= kzm) advance_z(k);
                }
                if (ke >= kx) {
                    cu += du;
                    bu += du;
                }
            }
        }
    }
    if (valid && !synced) {
        walk_cells(seg, 0.0f, nf, a.max_iter, [&](int cu, int cv, float cnt, float fa, float fb) {
            // the walk gives the fractions at the cell's first sample; recover k
            // from the u (or v) position: k = (cu + fa - u0) / su
            const float kf = fabsf(seg.su) >= fabsf(seg.sv) ? rintf((cu + fa - seg.u0) / seg.su)
                                                             : rintf((cv + fb - seg.v0) / seg.sv);
            // the cell's samples, cut at z crossings (kzn starts at sample 0
            // and the walk visits samples in order)
            float k = kf;
            const float kend = kf + cnt;
            for (int t = 0; t < kConeSteps && k < kend; ++t) {
                const float ke = fminf(kend, next_crossing());
                cell(cu, cv, ke - k, fmaf(seg.su, k, seg.u0) - (float)cu,
                     fmaf(seg.sv, k, seg.v0) - (float)cv, k);
                k = ke;
                advance_z(k);
            }
        });
    }
    if (has_c) {
        float *pv = proj + (size_t)v * a.n_rows * a.C;
#pragma unroll
        for (int rr = 0; rr < RB; ++rr) {
            if (r0 + rr >= a.n_rows) break;
            const float h = a.det_bottom + a.drow * ((float)(r0 + rr) + 0.5f);
            pv[(size_t)(r0 + rr) * a.C + c] = acc[rr] * a.w * sqrtf(1.0f + (h / a.D) * (h / a.D));
        }
    }
}

// Quad images of every slice of one volume ([nz][2 layouts][(nx+1)^2]), as the
// fan-beam projector builds them per slice.
__global__ void __launch_bounds__(256)
    cone_quads_kernel(const float *__restrict__ vol, float4 *__restrict__ quads, int nx,
                      int ny) {
    const int Q = nx + 1;
    const int qi = blockIdx.x * 32 + threadIdx.x, qj = blockIdx.y * 8 + threadIdx.y;
    if (qi >= Q || qj >= Q) return;
    const int layout = blockIdx.z & 1, k = blockIdx.z >> 1;
    build_quad(vol + (size_t)k * nx * ny,
               quads + ((size_t)k * 2 + layout) * Q * Q + (size_t)qj * Q + qi, nx, ny, layout,
               qi, qj);
}

// ---- cone-beam forward projection, one in-plane walk per ray for all rows ---------
// The projector above walks a ray's in-plane cells once per group of RB
// detector rows, and its lanes idle where neighbouring rays cut segments at
// different z crossings.  This one gives a warp G adjacent channels of one
// view and walks each ray's in-plane cells once for every row:
//  - walk: lane L takes cell line m of ray L mod G along the ray's major axis
//    (32/G lines of each ray per chunk), splits the line's samples at its one
//    minor-axis boundary (a line holds at most two cells) and queues, per
//    cell segment, its cell, first sample k, count and entry fractions and
//    the moments W_c = sum_j q_c(j), M_c = sum_j j q_c(j) of the bilinear
//    weights, in shared memory;
//  - drain: for every queued segment all lanes take the detector rows (lane
//    l: rows l, l+32, ...) and add W.t0 + cz W.(t1 - t0) + dw M.(t1 - t0) with
//    t0, t1 the four bilinear taps of slices kz, kz+1, cz the row's z
//    fraction at sample k and dw its z step per sample.  The taps come from
//    z-major columns of x pairs (two 8-byte loads per slice, each landing as
//    an f32x2 operand); rows read consecutive slices, so one warp load covers
//    a few lines.  The dw M.(t1 - t0) term is summed per row and scaled by dw
//    at the end;
//  - crossings: that sum is the linear extension, from the segment's first
//    sample, of the clamped piecewise-linear z interpolant.  Past each slice
//    boundary b that a row crosses inside the segment the interpolant differs
//    from it by sign(dw) (w - b) D2_b, D2_b the second difference of the
//    quads about b.  The drain marks those (segment, row) pairs in per-lane
//    bit masks, and after the chunk the lanes add the corrections together
//    from the partial moments over the samples past b.
// Columns hold slices -1 .. nz (slices -1 and nz repeat 0 and nz-1, so the
// clamped interpolant needs no index clamp: z positions clamp to [-1, nz-1]),
// nzp = nz + 2 entries per column.
constexpr int kSegPerLane = 3;  // cell segments of one line (two, plus a rounding spare)
constexpr int kSegSlots = 32 * kSegPerLane;

struct SegQueue {
    float4 e[kSegSlots];   // (column offset bits, second column offset bits, first sample k,
                           //  count - 1)
    float4 W[kSegSlots];   // sum_j q_c(j)
    float4 M[kSegSlots];   // sum_j j q_c(j)
    float2 f[kSegSlots];   // entry fractions (u, v)
    float4 ray;            // the warp's ray: entry point and steps (read per chunk, which
                           // keeps the walk's state out of the drain's registers)
};

// Launch shape (one clinical volume, CUDA events): 4-warp blocks, 7 resident
// per SM (72 registers) 36.8 ms; 6 / 5 per SM 39.0 / 41.7 ms, 8 per SM (spills)
// 40.1 ms.  z-major float4 quad columns instead of x pairs: 36.6 ms at twice
// the workspace; view-major block order or tiles of 4 .. 64 views instead of
// channel-group-major: 41 .. 51 ms.
#ifndef CT_CONE_SEG_WARPS
#define CT_CONE_SEG_WARPS 4
#endif
#ifndef CT_CONE_SEG_MINB
#define CT_CONE_SEG_MINB 7
#endif

// x-pair columns: for image row y and xq in [0, nx] the pairs
// (v(xq-1, y, z), v(xq, y, z)) of slices z = -1 .. nz (x and z clamped), nzp
// float2 per column; a cell (cu, cv) reads the columns (cu+1, cv) and
// (cu+1, cv+1), y clamped.
__global__ void __launch_bounds__(256)
    cone_pairs_z_kernel(const float *__restrict__ vol, float2 *__restrict__ pz, int nx, int ny,
                        int nz, int nzp) {
    __shared__ float2 tile[32][33];
    const int X = nx + 1;
    const int xq0 = blockIdx.x * 32, y = blockIdx.y, z0 = blockIdx.z * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int zz = ty; zz < 32; zz += 8) {
        const int zp = z0 + zz, xq = xq0 + tx;
        if (xq < X && zp < nzp) {
            const float *sl = vol + (size_t)min(max(zp - 1, 0), nz - 1) * nx * ny + (size_t)y * nx;
            tile[tx][zz] = make_float2(__ldg(sl + max(xq - 1, 0)), __ldg(sl + min(xq, nx - 1)));
        }
    }
    __syncthreads();
    for (int ii = ty; ii < 32; ii += 8) {
        const int zp = z0 + tx;
        if (xq0 + ii < X && zp < nzp) pz[((size_t)y * X + xq0 + ii) * nzp + zp] = tile[ii][tx];
    }
}

// The correction of one (segment, row) pair for the slice boundaries the row
// crosses inside the segment (see above); col points at slice 0 of the cell's
// column.
template <class Taps>
__device__ __forceinline__ float cone_seg_crossings(Taps tap, float4 E, float2 f, float su,
                                                    float sv, float w0r, float dwr, float nzm1) {
    const float k = E.z, cm1 = E.w, fa = f.x, fb = f.y, cnt = cm1 + 1.0f;
    const float wk = fmaf(dwr, k, w0r), wl = fmaf(dwr, cm1, wk);
    const float kz = floorf(fminf(fmaxf(wk, -1.0f), nzm1));
    const float kl = floorf(fminf(fmaxf(wl, -1.0f), nzm1));
    const int nb = (int)fabsf(kl - kz);
    const float Au = 1.0f - fa, Av = 1.0f - fb, uv = su * sv;
    const float4 c0 = make_float4(Au * Av, fa * Av, Au * fb, fa * fb);
    const float4 c1 = make_float4(-(Au * sv + Av * su), su * Av - fa * sv, Au * sv - su * fb,
                                  fa * sv + fb * su);
    const float4 c2 = make_float4(uv, -uv, -uv, uv);
    const float sg = dwr > 0.0f ? 1.0f : -1.0f;
    float corr = 0.0f;
    for (int i = 0; i < nb; ++i) {
        // boundary b between slices b-1 and b, in [0, nz-1]
        const float b = dwr > 0.0f ? kz + 1.0f + (float)i : kz - (float)i;
        // first sample past it (its exact position does not matter: the
        // correction vanishes at the boundary)
        const float tb = __fdividef(b - wk, dwr);
        const float js = fminf(fmaxf(dwr > 0.0f ? ceilf(tb) : floorf(tb) + 1.0f, 0.0f), cnt);
        float S0, S1, S2, S3;
        power_sums(js, cnt, S0, S1, S2, S3);
        const float4 P0 = moment(c0, c1, c2, S0, S1, S2), P1 = moment(c0, c1, c2, S1, S2, S3);
        const int ibd = (int)b;
        const bool ok = ibd >= 0 && (float)ibd <= nzm1;
        const float4 tm = tap(ok, ibd - 1), t0 = tap(ok, ibd), tp = tap(ok, ibd + 1);
        // sum_j q(j) sg (w_j - b) = sg (wk - b) P0 + sg dw P1
        const float x = sg * (wk - b), y = sg * dwr;
        const float4 P = make_float4(fmaf(x, P0.x, y * P1.x), fmaf(x, P0.y, y * P1.y),
                                     fmaf(x, P0.z, y * P1.z), fmaf(x, P0.w, y * P1.w));
        const float4 d2 = make_float4(tp.x + tm.x - 2.0f * t0.x, tp.y + tm.y - 2.0f * t0.y,
                                      tp.z + tm.z - 2.0f * t0.z, tp.w + tm.w - 2.0f * t0.w);
        corr += dot4(P, d2);
    }
    return corr;
}

// A shared-memory load the compiler keeps where it is written (not hoisted
// out of a loop into a register held across it).
__device__ __forceinline__ float4 lds_fresh(const float4 *p) {
    float4 v;
    asm volatile("ld.volatile.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"((unsigned)__cvta_generic_to_shared(p)));
    return v;
}

// (more rows per lane hold more accumulators: fewer blocks per SM)
template <int RPL>
__global__ void __launch_bounds__(CT_CONE_SEG_WARPS * 32,
                                  RPL <= 2 ? CT_CONE_SEG_MINB : 12 - RPL * 2)
    cone_fp_seg_kernel(const unsigned long long *__restrict__ cols, float *__restrict__ proj,
                       const float4 *__restrict__ ray, const int *__restrict__ nsamp,
                       const float2 *__restrict__ chan_s, const float *__restrict__ view_z,
                       ConeFpArgs a, int nzp) {
    constexpr unsigned FULL = 0xffffffffu;
    constexpr int NW = CT_CONE_SEG_WARPS;
    __shared__ SegQueue sq[NW];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    SegQueue &q = sq[wid];
    // a block is NW adjacent channels of one view
    // blocks channel-group-major: the resident blocks hold most views of a
    // few channel groups
    const int cg = blockIdx.x / a.V, v = blockIdx.x - cg * a.V;
    const int c = cg * NW + wid;  // the warp's channel
    if (c >= a.C) return;         // warp-uniform
    const float zs = view_z ? __ldg(view_z + v) : 0.0f;
    const int Q = a.nx + 1;
    const float nzm1 = (float)(a.nz - 1);
    const unsigned long long *pz = cols + 1;  // slice 0 of column 0
    // the ray: steps, sample count, and per row the z cell coordinate
    // w0 + dw k of sample k
    const int n = __ldg(nsamp + (size_t)v * a.C + c);
    const float mn = (float)n;
    const float4 my = n > 0 ? __ldg(ray + (size_t)v * a.C + c) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 sd = n > 0 ? __ldg(chan_s + c) : make_float2(0.f, 0.f);
    const float ds = n > 0 ? -sd.y / mn : 0.0f;
    float w0[RPL], dw[RPL];
#pragma unroll
    for (int s = 0; s < RPL; ++s) {
        const int r = lane + 32 * s;
        const float h = a.det_bottom + a.drow * ((float)r + 0.5f);
        const bool live = n > 0 && r < a.n_rows;
        w0[s] = live ? (h * sd.x / a.D + zs - a.zmin) / a.dz - 0.5f : 0.0f;
        dw[s] = live ? h * ds / (a.D * a.dz) : 0.0f;
    }
    // lines floor(A0) - dir .. floor(A0 + SA (n-1)) + dir of the walk's major
    // axis hold every sample
    int nchunk = 0;
    if (n > 0) {
        const bool vmaj = fabsf(my.w) >= fabsf(my.z);
        const float A0 = (vmaj ? my.y : my.x) - 0.5f, SA = vmaj ? my.w : my.z;
        const int dir = SA >= 0.0f ? 1 : -1;
        const int ja = (int)floorf(A0), jb = (int)floorf(fmaf(SA, mn - 1.0f, A0));
        nchunk = ((jb - ja) * dir + 3 + 31) / 32;
    }
    if (lane == 0) q.ray = my;

    unsigned long long A2[RPL], M2[RPL];
    float Cx[RPL];
#pragma unroll
    for (int s = 0; s < RPL; ++s) {
        A2[s] = 0ull;
        M2[s] = 0ull;
        Cx[s] = 0.0f;
    }
    // one row's taps at a segment: slices kz and kz+1 as f32x2 pairs, its z
    // fraction and whether its z cell may change inside the segment
    struct RowTap {
        unsigned long long a01, a23, c01, c23;
        float cz;
        bool cross;
    };
    auto fetch = [&](const float4 &E, int s) {
        RowTap r;
        const float wk = fmaf(dw[s], E.z, w0[s]);
        const float wc = fminf(fmaxf(wk, -1.0f), nzm1);
        const float kz = floorf(wc);
        r.cz = wc - kz;
        // the clamped z cell of the segment's last sample differs
        r.cross = floorf(fminf(fmaxf(fmaf(dw[s], E.w, wk), -1.0f), nzm1)) != kz;
        const int iz = (int)kz;
        const unsigned long long *c0p = pz + __float_as_int(E.x);
        const unsigned long long *c1p = pz + __float_as_int(E.y);
        r.a01 = __ldg(c0p + iz);
        r.a23 = __ldg(c1p + iz);
        r.c01 = __ldg(c0p + iz + 1);
        r.c23 = __ldg(c1p + iz + 1);
        return r;
    };
    auto accumulate = [&](const RowTap &r, const float4 &W, const float4 &M, int s) {
        const unsigned long long d01 = zt_sub2(r.c01, r.a01), d23 = zt_sub2(r.c23, r.a23);
        const unsigned long long czp = pack2(r.cz, r.cz);
        A2[s] = fma2(pack2(W.x, W.y), fma2(czp, d01, r.a01), A2[s]);
        A2[s] = fma2(pack2(W.z, W.w), fma2(czp, d23, r.a23), A2[s]);
        M2[s] = fma2(pack2(M.x, M.y), d01, M2[s]);
        M2[s] = fma2(pack2(M.z, M.w), d23, M2[s]);
    };

    for (int ch = 0; ch < nchunk; ++ch) {
        __syncwarp();
        // walk: the segments of this lane's line, in (major, minor) axes
        const float4 ry = lds_fresh(&q.ray);
        const float u0 = ry.x - 0.5f, v0 = ry.y - 0.5f, su = ry.z, sv = ry.w;
        const bool vmaj = fabsf(sv) >= fabsf(su);
        const float A0 = vmaj ? v0 : u0, SA = vmaj ? sv : su;
        const float B0 = vmaj ? u0 : v0, SB = vmaj ? su : sv;
        const float ia = 1.0f / SA, ib = SB != 0.0f ? 1.0f / SB : 0.0f;
        const int dir = SA >= 0.0f ? 1 : -1;
        const float dB = SB >= 0.0f ? 1.0f : -1.0f;
        const int ja = (int)floorf(A0), jb = (int)floorf(fmaf(SA, mn - 1.0f, A0));
        const int J0 = ja - dir, lines = (jb - ja) * dir + 3;
        const int m = ch * 32 + lane;
        int ns = 0;
        if (m < lines) {
            const int jm = J0 + dir * m;
            const float tA = ((float)jm - A0) * ia, tB = ((float)(jm + 1) - A0) * ia;
            const float ka = fmaxf(0.0f, ceilf(fminf(tA, tB)));
            const float kb = fminf(mn, ceilf(fmaxf(tA, tB)));
            float k = ka;
            float cb = floorf(fmaf(SB, ka, B0));
            for (int it = 0; it <= kSegPerLane && k < kb && ns < kSegPerLane; ++it) {
                const float bb = SB >= 0.0f ? cb + 1.0f : cb;
                const float ke = SB != 0.0f ? fminf(kb, ceilf((bb - B0) * ib)) : kb;
                if (ke > k) {
                    const float cu = vmaj ? cb : (float)jm, cv = vmaj ? (float)jm : cb;
                    const float fa = fmaf(su, k, u0) - cu, fb = fmaf(sv, k, v0) - cv;
                    const float cnt = ke - k;
                    const float Au = 1.0f - fa, Av = 1.0f - fb, uv = su * sv;
                    const float4 c0 = make_float4(Au * Av, fa * Av, Au * fb, fa * fb);
                    const float4 c1 =
                        make_float4(-(Au * sv + Av * su), su * Av - fa * sv, Au * sv - su * fb,
                                    fa * sv + fb * su);
                    const float4 c2 = make_float4(uv, -uv, -uv, uv);
                    float S0, S1, S2, S3;
                    power_sums(0.0f, cnt, S0, S1, S2, S3);
                    const int qi = (int)cu + 1, qj = (int)cv + 1;
                    (void)CT_DCHECK((unsigned)qi < (unsigned)Q && (unsigned)qj < (unsigned)Q);
                    const int xq = min(max(qi, 0), a.nx);
                    const int off0 = (min(max(qj - 1, 0), a.ny - 1) * Q + xq) * nzp;
                    const int off1 = (min(max(qj, 0), a.ny - 1) * Q + xq) * nzp;
                    const int slot = lane * kSegPerLane + ns;
                    q.e[slot] = make_float4(__int_as_float(off0), __int_as_float(off1), k,
                                            cnt - 1.0f);
                    q.W[slot] = moment(c0, c1, c2, S0, S1, S2);
                    q.M[slot] = moment(c0, c1, c2, S1, S2, S3);
                    q.f[slot] = make_float2(fa, fb);
                    ++ns;
                    k = ke;
                }
                cb += dB;
            }
        }
        __syncwarp();
        // drain: every queued segment for every row
        unsigned xm[RPL][kSegPerLane];
#pragma unroll
        for (int t = 0; t < kSegPerLane; ++t) {
#pragma unroll
            for (int s = 0; s < RPL; ++s) xm[s][t] = 0u;
            unsigned mask = __ballot_sync(FULL, ns > t);
            while (mask) {
                const int L = __ffs(mask) - 1;
                mask &= mask - 1;
                const int e = L * kSegPerLane + t;
                const float4 E = q.e[e];
                RowTap r[RPL];
#pragma unroll
                for (int s = 0; s < RPL; ++s) r[s] = fetch(E, s);
                const float4 W = q.W[e], M = q.M[e];
#pragma unroll
                for (int s = 0; s < RPL; ++s) {
                    accumulate(r[s], W, M, s);
                    xm[s][t] |= r[s].cross ? 1u << L : 0u;
                }
            }
        }
        // crossings: each lane works through its marked (segment, row) pairs
        for (;;) {
            bool have = false;
            int ps = 0, pt = 0;
            unsigned bits = 0u;
#pragma unroll
            for (int s = 0; s < RPL; ++s)
#pragma unroll
                for (int t = 0; t < kSegPerLane; ++t)
                    if (!have && xm[s][t]) {
                        have = true;
                        ps = s;
                        pt = t;
                        bits = xm[s][t];
                    }
            if (!__any_sync(FULL, have)) break;
            if (have) {
                const int L = __ffs(bits) - 1;
                float w0r = 0.0f, dwr = 0.0f;
#pragma unroll
                for (int s = 0; s < RPL; ++s) {
#pragma unroll
                    for (int t = 0; t < kSegPerLane; ++t)
                        if (s == ps && t == pt) xm[s][t] &= xm[s][t] - 1u;
                    if (s == ps) {
                        w0r = w0[s];
                        dwr = dw[s];
                    }
                }
                const int e = L * kSegPerLane + pt;
                const float4 E = q.e[e];
                const unsigned long long *c0p = pz + __float_as_int(E.x);
                const unsigned long long *c1p = pz + __float_as_int(E.y);
                auto tap = [&](bool ok, int z) {
                    const float2 lo = zt_unpack(CT_DLOAD(ok, c0p + z));
                    const float2 hi = zt_unpack(CT_DLOAD(ok, c1p + z));
                    return make_float4(lo.x, lo.y, hi.x, hi.y);
                };
                const float4 ry = lds_fresh(&q.ray);
                const float corr = cone_seg_crossings(tap, E, q.f[e], ry.z, ry.w, w0r, dwr, nzm1);
#pragma unroll
                for (int s = 0; s < RPL; ++s)
                    if (s == ps) Cx[s] += corr;
            }
        }
        __syncwarp();  // the queue is rewritten by the next chunk
    }
#pragma unroll
    for (int s = 0; s < RPL; ++s) {
        const int r = lane + 32 * s;
        if (r >= a.n_rows) continue;
        const float h = a.det_bottom + a.drow * ((float)r + 0.5f);
        const float2 av = unpack2(A2[s]), mv = unpack2(M2[s]);
        const float val = (av.x + av.y) + Cx[s] + dw[s] * (mv.x + mv.y);
        proj[((size_t)v * a.n_rows + r) * a.C + c] = val * a.w * sqrtf(1.0f + (h / a.D) * (h / a.D));
    }
}

ConeArgs make_cone_args(const ct_plan *p) {
    ConeArgs a;
    a.V = p->g.n_views;
    a.C = p->g.n_cols;
    a.nx = p->g.nx;
    a.ny = p->g.ny;
    a.nz = p->nz;
    a.n_rows = p->n_rows;
    a.xmin = p->g.xmin;
    a.ymin = p->g.ymin;
    a.dx = p->g.dx;
    a.dy = p->g.dy;
    a.dz = p->g.dz;
    a.zmin = -0.5f * p->g.dz * (float)p->nz;
    a.R = p->g.sid;
    a.D = p->g.sdd;
    const double inv = 1.0 / (double)p->g.dcol;
    a.inv_dcol = (float)inv;
    a.pos_off = (float)((double)p->g.shift - (double)p->g.left * inv + 0.5);
    a.fC = (float)a.C;
    a.row_scale = (float)((double)p->g.sdd / (double)p->g.drow);
    a.row_off = (float)(-(double)p->g.det_bottom / (double)p->g.drow + 0.5);
    a.fov_r2 = (double)p->g.rfov * (double)p->g.rfov;
    for (int k = 0; k < 9; ++k) a.coef[k] = p->atan_coef[k];
    a.atan_deg = p->atan_deg;
    return a;
}

}  // namespace

size_t cone_bp_work_bytes(const ct_plan *p) {
    // one volume's quad images, where they stay within 4 GB
    const size_t q = sizeof(float4) * (size_t)p->g.n_views * (p->n_rows + 1) * (p->g.n_cols + 1);
    return q <= ((size_t)4 << 30) ? q : 0;
}

int cone_bp(const ct_plan *p, const float *proj, float *vol, int batch, void *work,
            void *stream) {
    const ConeArgs a = make_cone_args(p);
    constexpr int ZC = kZC;
    const int zgroups = (a.nz + ZC - 1) / ZC;
    const float2 *vcs = reinterpret_cast<const float2 *>(p->d_view_cs);
    cudaStream_t s = (cudaStream_t)stream;
    const bool tex = p->opts.texture_weights != 0;
    const size_t per_proj = (size_t)a.V * a.n_rows * a.C, per_vol = (size_t)a.nz * a.ny * a.nx;
    if (work && cone_bp_work_bytes(p)) {
        float4 *pq = static_cast<float4 *>(work);
        auto kern = a.atan_deg == 4
                        ? (tex ? cone_bp_kernel<ZC, 4, true, true> : cone_bp_kernel<ZC, 4, false, true>)
                    : a.atan_deg == 8
                        ? (tex ? cone_bp_kernel<ZC, 8, true, true> : cone_bp_kernel<ZC, 8, false, true>)
                        : (tex ? cone_bp_kernel<ZC, 0, true, true> : cone_bp_kernel<ZC, 0, false, true>);
        for (int b = 0; b < batch; ++b) {
            const float *pp = proj + (size_t)b * per_proj;
            for (int v0 = 0; v0 < a.V; v0 += 65535) {
                const int nv = a.V - v0 < 65535 ? a.V - v0 : 65535;
                cone_proj_quads_kernel<<<dim3((a.C + 1 + 255) / 256, a.n_rows + 1, nv), 256, 0,
                                         s>>>(pp + (size_t)v0 * a.n_rows * a.C,
                                              pq + (size_t)v0 * (a.n_rows + 1) * (a.C + 1),
                                              a.n_rows, a.C);
                ct_count_launch();
            }
            kern<<<dim3((a.nx + 31) / 32, (a.ny + 7) / 8, zgroups), dim3(32, 8), 0, s>>>(
                pp, pq, vol + (size_t)b * per_vol, vcs, p->d_view_z, a, 1);
            ct_count_launch();
        }
        return (int)cudaGetLastError();
    }
    auto kern = a.atan_deg == 4
                    ? (tex ? cone_bp_kernel<ZC, 4, true, false> : cone_bp_kernel<ZC, 4, false, false>)
                : a.atan_deg == 8
                    ? (tex ? cone_bp_kernel<ZC, 8, true, false> : cone_bp_kernel<ZC, 8, false, false>)
                    : (tex ? cone_bp_kernel<ZC, 0, true, false> : cone_bp_kernel<ZC, 0, false, false>);
    for (int b0 = 0; b0 < batch; b0 += 4096) {
        const int nb = batch - b0 < 4096 ? batch - b0 : 4096;
        dim3 grid((a.nx + 31) / 32, (a.ny + 7) / 8, zgroups * nb);
        kern<<<grid, dim3(32, 8), 0, s>>>(proj + (size_t)b0 * per_proj, nullptr,
                                          vol + (size_t)b0 * per_vol, vcs, p->d_view_z, a, nb);
        ct_count_launch();
    }
    return (int)cudaGetLastError();
}

namespace {

size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

// shared-memory accumulators of the lanes-along-z transpose (0: does not fit)
size_t zt_smem(const ct_plan *p) {
    const size_t ints = ((size_t)p->g.n_cols * (size_t)(p->n_rows | 1) + 3) & ~(size_t)3;
    return sizeof(int) * ints <= 227 * 1024 ? sizeof(int) * ints : 0;
}

int zt_nzp(const ct_plan *p) { return (p->nz + kZS - 1) / kZS * kZS; }

// log2 of the lanes per pixel: slice groups rounded up to a power of two, <= 32
int zt_lg(const ct_plan *p) {
    const int groups = zt_nzp(p) / kZS;
    int lg = 0;
    while ((1 << lg) < groups && lg < 5) ++lg;
    return lg;
}

// Work of the transpose: per-volume maxima, then (lanes-along-z path) the
// pixel tables and the z-major copy of the volumes.
struct ZtWork {
    size_t vmax, px, py, pxl, pyl, span, vol_t, total;
};

ZtWork zt_work(const ct_plan *p, int batch) {
    ZtWork w{};
    w.vmax = 0;
    size_t o = align256(sizeof(int) * (size_t)batch);
    if (!zt_smem(p)) {
        w.total = o;
        return w;
    }
    w.px = o;
    o += align256(sizeof(float) * (size_t)p->g.nx);
    w.py = o;
    o += align256(sizeof(float) * (size_t)p->g.ny);
    w.pxl = o;
    o += align256(sizeof(float) * (size_t)p->g.nx);
    w.pyl = o;
    o += align256(sizeof(float) * (size_t)p->g.ny);
    w.span = o;
    o += align256(sizeof(int2) * (size_t)p->g.ny);
    w.vol_t = o;
    o += sizeof(float) * (size_t)batch * p->g.nx * p->g.ny * zt_nzp(p);
    w.total = o;
    return w;
}

}  // namespace

size_t cone_bp_transpose_work_bytes(const ct_plan *p, int batch) {
    return zt_work(p, batch).total;
}

bool cone_bp_transpose_supported(const ct_plan *p) {
    return zt_smem(p) || sizeof(int) * (kRB + 2) * (size_t)p->g.n_cols <= 227 * 1024;
}

int cone_bp_transpose(const ct_plan *p, const float *vol, float *proj, int batch, void *work,
                      void *stream) {
    ConeArgs a = make_cone_args(p);
    {
        // Bounds of a detector cell's weighted sample counts (rigorous; the
        // fixed-point scale is 2^30 over their product with max|vol| and max w).
        // Columns: a cell's pixels carry the column hat weight (unit integral,
        // support two channels).  Layer by layer the hat's level sets are
        // wedges from the source cut by the FOV disc, convex, and a convex set
        // holds at most area/(dx dy) + perimeter/(2 min(dx, dy)) + 1 lattice
        // points (Nosarzewska); summed over the layers, the area term is
        // dcol (L2^2 - L1^2)/2 <= dcol 2 R rf and the perimeter term at most
        // (4 rf + 2 pi dcol (R + rf))/2.  The same holds for the clamped edge
        // channels, whose weight is a trapezoid of the same integral.  Rows:
        // a pixel's slices sample the row coordinate at a step of at least
        // dz D / ((R + rf) drow), so a row's hat weights sum to at most
        // 1/step + 1 (a unimodal function's Riemann sum exceeds its integral by
        // at most its maximum).  (2-channel and 2-row counts, 4.8x and 2x
        // looser at the clinical geometry, quantised the FDK adjoint into a
        // 1.5e-4 error after its ramp filter.)
        const double pix = p->g.dx < p->g.dy ? p->g.dx : p->g.dy;
        const double R = p->g.sid, rf = p->g.rfov, D = p->g.sdd;
        const double dcol = p->g.dcol;
        a.fix_npix = (float)(dcol * 2.0 * R * rf / ((double)p->g.dx * (double)p->g.dy) +
                             (2.0 * rf + 3.14159265358979 * dcol * (R + rf)) / pix + 1.0);
        const double rstep = (double)p->g.dz * D / ((R + rf) * (double)p->g.drow);
        a.fix_slices = (float)(1.0 / rstep + 1.0);
        a.fix_wmax = (float)(1.0 / ((R - rf) * (R - rf)));
        // row + 1/2 = z row_scale / U + row_off over the slice centres
        // relative to every source height and U in [R - rf, R + rf]; no
        // clamping when it stays inside [1, n_rows) with a margin
        const double z0 = (double)a.zmin + 0.5 * p->g.dz - p->view_z_max;
        const double z1 = -(double)a.zmin - 0.5 * p->g.dz - p->view_z_min;
        const double rs = (double)p->g.sdd / p->g.drow, ro = a.row_off;
        const double lo = ro + rs * (z0 < 0.0 ? z0 / (R - rf) : z0 / (R + rf));
        const double hi = ro + rs * (z1 > 0.0 ? z1 / (R - rf) : z1 / (R + rf));
        const bool clamps = !(lo >= 1.01 && hi <= p->n_rows - 0.01);
        a.fix_edge = clamps ? (float)a.nz : a.fix_slices;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const ZtWork zw = zt_work(p, batch);
    char *wb = static_cast<char *>(work);
    int *vmax_bits = reinterpret_cast<int *>(wb + zw.vmax);
    cudaError_t e0 = cudaMemsetAsync(vmax_bits, 0, sizeof(int) * (size_t)batch, s);
    if (e0 != cudaSuccess) return (int)e0;
    const float2 *vcs = reinterpret_cast<const float2 *>(p->d_view_cs);
    const float2 *vcs_lo = reinterpret_cast<const float2 *>(p->d_view_cs_lo);
    const float2 *col_tan = reinterpret_cast<const float2 *>(p->d_col_tan);
    const bool tex = p->opts.texture_weights != 0;
    const size_t per_volume = (size_t)a.nz * a.ny * a.nx;
    if (const size_t smem = zt_smem(p)) {
        const int npix = a.nx * a.ny, nzp = zt_nzp(p);
        float *px = reinterpret_cast<float *>(wb + zw.px);
        float *py = reinterpret_cast<float *>(wb + zw.py);
        float *pxl = reinterpret_cast<float *>(wb + zw.pxl);
        float *pyl = reinterpret_cast<float *>(wb + zw.pyl);
        int2 *span = reinterpret_cast<int2 *>(wb + zw.span);
        float *vol_t = reinterpret_cast<float *>(wb + zw.vol_t);
        cone_fov_tables_kernel<<<a.ny, 32, 0, s>>>(a, px, py, pxl, pyl, span);
        ct_count_launch();
        auto kern = a.atan_deg == 4   ? (tex ? cone_bp_transpose_z_kernel<4, true>
                                             : cone_bp_transpose_z_kernel<4, false>)
                    : a.atan_deg == 8 ? (tex ? cone_bp_transpose_z_kernel<8, true>
                                             : cone_bp_transpose_z_kernel<8, false>)
                                      : (tex ? cone_bp_transpose_z_kernel<0, true>
                                             : cone_bp_transpose_z_kernel<0, false>);
        cudaError_t e =
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return (int)e;
        for (int b0 = 0; b0 < batch; b0 += 65535) {
            const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
            cone_zmajor_kernel<<<dim3((npix + 31) / 32, (nzp + 31) / 32, nb), 256, 0, s>>>(
                vol + (size_t)b0 * per_volume, vol_t, vmax_bits + b0, a.nz, npix, nzp);
            kern<<<dim3(a.V, nb), kZThreads, smem, s>>>(
                vol_t, proj + (size_t)b0 * a.V * a.n_rows * a.C, vcs, vcs_lo, col_tan,
                p->d_view_z, vmax_bits + b0, px, py, pxl, pyl, span, a, nzp, zt_lg(p));
            ct_count_launch(2);
        }
        return (int)cudaGetLastError();
    }
    volume_absmax_kernel<<<dim3(152, batch), 256, 0, s>>>(vol, per_volume, vmax_bits);
    ct_count_launch();
    const size_t smem = sizeof(int) * (kRB + 2) * a.C;
    auto kern = a.atan_deg == 4
                    ? (tex ? cone_bp_transpose_kernel<4, true> : cone_bp_transpose_kernel<4, false>)
                : a.atan_deg == 8
                    ? (tex ? cone_bp_transpose_kernel<8, true> : cone_bp_transpose_kernel<8, false>)
                    : (tex ? cone_bp_transpose_kernel<0, true> : cone_bp_transpose_kernel<0, false>);
    cudaError_t e =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    const int rblocks = (a.n_rows + kRB - 1) / kRB;
    const int per = 65535 / rblocks;
    for (int b0 = 0; b0 < batch; b0 += per) {
        const int nb = batch - b0 < per ? batch - b0 : per;
        kern<<<dim3(a.V, rblocks * nb), kThreads, smem, (cudaStream_t)stream>>>(
            vol + (size_t)b0 * a.nz * a.ny * a.nx, proj + (size_t)b0 * a.V * a.n_rows * a.C, vcs,
            vcs_lo, col_tan, p->d_view_z, vmax_bits + b0, a, nb);
        ct_count_launch();
    }
    return (int)cudaGetLastError();
}

// Up to 128 detector rows the single-walk projector runs (its rows are lanes
// of one warp, four per lane at most); taller detectors use the row-group one.
#ifndef CT_CONE_FP_WALK_ROWS
#define CT_CONE_FP_WALK_ROWS 128
#endif
// (column offsets are int32)
static bool cone_fp_single_walk(const ct_plan *p) {
    const double cells = (double)(p->g.nx + 1) * (double)(p->g.nx + 1) * (double)(p->nz + 2);
    return p->n_rows <= (CT_CONE_FP_WALK_ROWS < 128 ? CT_CONE_FP_WALK_ROWS : 128) &&
           cells < 2147483647.0;
}

size_t cone_fp_work_bytes(const ct_plan *p, int batch) {
    // the quad images of one volume at a time: z-major columns of slices
    // -1 .. nz for the single-walk projector, two layouts per slice otherwise
    (void)batch;
    const size_t cells = (size_t)(p->g.nx + 1) * (p->g.nx + 1);
    if (!cone_fp_single_walk(p)) return sizeof(float4) * 2 * (size_t)p->nz * cells;
    return sizeof(float2) * (size_t)(p->nz + 2) * (p->g.nx + 1) * p->g.ny;
}

int cone_fp(const ct_plan *p, const float *vol, float *proj, int batch, void *work,
            void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    const int nx = p->g.nx, ny = p->g.ny, nz = p->nz;
    float4 *quads = static_cast<float4 *>(work);
    ConeFpArgs a;
    a.V = p->g.n_views;
    a.C = p->g.n_cols;
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.n_rows = p->n_rows;
    a.wpv = (a.C + 31) / 32;
    a.w = p->fp_weight;
    a.D = p->g.sdd;
    a.det_bottom = p->g.det_bottom;
    a.drow = p->g.drow;
    a.dz = p->g.dz;
    a.zmin = -0.5f * p->g.dz * (float)nz;
    a.max_iter = 2 * (nx > ny ? nx : ny) + 8;
    const int Q = nx + 1;
    if (cone_fp_single_walk(p)) {
        constexpr int CPB = CT_CONE_SEG_WARPS;
        const int nzp = nz + 2;
        const int rpl = (a.n_rows + 31) / 32;
        auto kern = rpl == 1   ? cone_fp_seg_kernel<1>
                    : rpl == 2 ? cone_fp_seg_kernel<2>
                    : rpl == 3 ? cone_fp_seg_kernel<3>
                               : cone_fp_seg_kernel<4>;
        const unsigned blocks = (unsigned)((a.C + CPB - 1) / CPB) * (unsigned)a.V;
        for (int b = 0; b < batch; ++b) {
            cone_pairs_z_kernel<<<dim3((Q + 31) / 32, ny, (nzp + 31) / 32), dim3(32, 8), 0, s>>>(
                vol + (size_t)b * nz * nx * ny, reinterpret_cast<float2 *>(work), nx, ny, nz,
                nzp);
            kern<<<blocks, CT_CONE_SEG_WARPS * 32, 0, s>>>(
                static_cast<const unsigned long long *>(work), proj + (size_t)b * a.V * a.n_rows * a.C,
                reinterpret_cast<const float4 *>(p->d_ray), p->d_nsamp,
                reinterpret_cast<const float2 *>(p->d_chan_s), p->d_view_z, a, nzp);
            ct_count_launch(2);
        }
        return (int)cudaGetLastError();
    }
    constexpr int RB = CT_CONE_FP_ROWS;
    const int rgroups = (a.n_rows + RB - 1) / RB;
    const int blocks = (a.V + kConeFpThreads / 32 - 1) / (kConeFpThreads / 32) * a.wpv;
    for (int b = 0; b < batch; ++b) {
        cone_quads_kernel<<<dim3((Q + 31) / 32, (Q + 7) / 8, 2 * nz), dim3(32, 8), 0, s>>>(
            vol + (size_t)b * nz * nx * ny, quads, nx, ny);
        cone_fp_kernel<RB><<<dim3(blocks, rgroups), kConeFpThreads, 0, s>>>(
            quads, proj + (size_t)b * a.V * a.n_rows * a.C,
            reinterpret_cast<const float4 *>(p->d_ray), p->d_nsamp,
            reinterpret_cast<const float2 *>(p->d_chan_s), p->d_view_z, a);
        ct_count_launch(2);
    }
    return (int)cudaGetLastError();
}

}  // namespace ctk
