// Gather-form transpose of the pixel-driven backprojector (BP and the
// 1/L^2-weighted FBP / FDK-2D form): deterministic, no atomics.
//
// The backprojector adds, per pixel p inside the FOV disc and view, the
// linearly interpolated detector value at column coordinate y = col + 1/2
// (texel centres at +1/2, clamped taps) when 1/2 < y < C + 1/2
// (BP/transform.cu:76-92, FBP/transform.cu:70-87).  Its transpose sends x_p w
// to the two taps: (1 - f) to max(i-1, 0) and f to min(i, C-1), i = trunc(y),
// f = y - i.  Gathered per detector column: strip b = the pixels with
// trunc(y) = b lies between the rays y = b and y = b + 1 from the source, so
// a lane owns strip b, walks the image lines (rows or columns) across it, and
// sums A_b = sum (1 - f) x w and B_b = sum f x w over its pixels; channel c
// is then B_c + A_{c+1} (channel 0 adds A_0, channel C-1 adds B_C: the
// clamped taps).  A warp holds strips 31k .. 31k+31 and writes channels
// 31k .. 31k+30, so every channel is written by one lane: no atomics, and
// each lane sums in a fixed order.
//
// Geometry per (view, strip group), from host FP64 tables (ct_build_bpt_tables):
// each boundary ray's crossing of the first line and its step per line, in
// 32.32 fixed point along the line, so that the crossings are exact integers
// plus fractions; two lanes sharing a boundary read the same table entry, so
// every pixel belongs to exactly one strip.  A pixel's offset from its
// strip's lower boundary along the line is then small and exact in FP32,
// and its angle from that boundary, atan(n / L) with n its normal distance
// and L its distance along the ray, needs no large coordinate: f is accurate
// to ~1e-7 of a channel, where the absolute column coordinate in FP32 (up to
// ~900 channels) carries ~6e-5 -- noise the ramp filter of the FBP adjoint
// amplifies about 80-fold (the scatter form reached 1.5e-4 relative L2 at
// 512^2 / 984 x 888; the contract is 1e-4).
//
// Slices: per launch 4, 8 or 16 slices share every lane's geometry; the
// images come as slice-quad planes (float4 = 4 slices) in both layouts
// (rows [quad][y][x] for row walks, columns [quad][x][y] for column walks) so
// that adjacent lanes -- adjacent strips -- read adjacent 16-byte pixels.
// Blocks are 4 warps = 4 adjacent views of one channel group (their strips
// cross nearly the same pixels), ordered channel-group-major as the forward
// projector's.
#include "bp_body.cuh"

namespace ctk {
namespace {

struct BptArgs {
    int V, C, W, nx, ny;
    int vq;           // view quads (blocks per channel group)
    float inv_dcol;   // 1 / dcol
};

__device__ __forceinline__ unsigned long long dup2(float x) { return pack2(x, x); }

// 5 resident blocks per SM (96 registers): 32 clinical slices, BP / FBP
// adjoint 2.70 / 3.34 ms, against 3.71 / 4.25 ms at the compiler's 102
// registers (4 blocks) and 3.42 / 3.99 ms at 6 blocks (80 registers)
#ifndef CT_BPG_MINB
#define CT_BPG_MINB 5
#endif
// at most NQ slice quads per lane (16 slices); 8 slices measured 5.18 ms
#ifndef CT_BPG_NQ
#define CT_BPG_NQ 4
#endif

// NQ quads = 4 NQ slices per launch slice group (blockIdx.y).
template <bool WEIGHTED, int NQ>
__global__ void __launch_bounds__(128, CT_BPG_MINB)
    bp_gather_kernel(const float4 *__restrict__ rows, const float4 *__restrict__ cols,
                     size_t qplane, float *__restrict__ sino, int nsl,
                     const int4 *__restrict__ wtab, const longlong2 *__restrict__ btab,
                     const float4 *__restrict__ rtab, const int2 *__restrict__ fov_row,
                     const int2 *__restrict__ fov_col, BptArgs a) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k = blockIdx.x / a.vq;
    const int v = (blockIdx.x - k * a.vq) * 4 + warp;
    if (v >= a.V) return;  // warp-uniform
    const size_t e = (size_t)v * a.W + k;
    const int4 wi = __ldg(wtab + e);
    const bool colwalk = wi.x & 1, pos = (wi.x >> 1) & 1;
    const int J0 = wi.y, J1 = wi.z;
    const int strip = k * kBptOut + lane;
    const bool active = strip <= a.C;
    const longlong2 bl = __ldg(btab + e * 33 + lane), bh = __ldg(btab + e * 33 + lane + 1);
    const float4 rr = __ldg(rtab + e * 32 + lane);
    const int npx = colwalk ? a.ny : a.nx;
    const float4 *img = (colwalk ? cols : rows) + (size_t)blockIdx.y * NQ * qplane;
    const int2 *fov = colwalk ? fov_col : fov_row;

    unsigned long long A[2 * NQ], B[2 * NQ];  // slice pairs (2h, 2h+1) of (1-f) and f sums
#pragma unroll
    for (int h = 0; h < 2 * NQ; ++h) A[h] = B[h] = 0ull;

    long long Xl = bl.x, Xh = bh.x;
    const int lines = active ? J1 - J0 + 1 : 0;
    for (int t = 0; t < lines; ++t) {
        const int j = J0 + t;
        const int hl = (int)(Xl >> 32), hh = (int)(Xh >> 32);
        const unsigned fl = (unsigned)Xl, fh = (unsigned)Xh;
        // the strip's pixels on this line: between the two crossings, the
        // lower boundary included (gamma_b <= gamma_p < gamma_{b+1})
        int i0, i1;
        if (pos) {
            i0 = hl + (fl != 0u);
            i1 = hh + (fh != 0u) - 1;
        } else {
            i0 = hh + 1;
            i1 = hl;
        }
        const int2 fr = __ldg(fov + j);
        i0 = max(i0, fr.x);
        i1 = min(i1, fr.y);
        if (i0 <= i1) {
            const float F = __uint2float_rn(fl) * 2.3283064365386963e-10f;  // 2^-32
            const float Lb = fmaf((float)t, rr.y, rr.x);
            const float4 *line = img + (size_t)j * npx;
            const int nlines = colwalk ? a.nx : a.ny;
            for (int i = i0; i <= i1; ++i) {
                const bool ok = (unsigned)i < (unsigned)npx && (unsigned)j < (unsigned)nlines;
                const float dp = (float)(i - hl) - F;  // offset from the lower boundary (pixels)
                const float n = dp * rr.z;              // normal distance (mm)
                const float L = fmaf(dp, rr.w, Lb);     // distance along the boundary ray (mm)
                const float q = __fdividef(n, L);
                const float q2 = q * q;
                // atan(q) for |q| <= dcol: q (1 - q^2/3 + q^4/5)
                const float f = q * fmaf(q2, fmaf(q2, 0.2f, -0.33333334f), 1.0f) * a.inv_dcol;
                float wa = 1.0f - f, wb = f;
                if (WEIGHTED) {
                    const float w = __fdividef(1.0f, fmaf(L, L, n * n));  // 1 / (U^2 + t^2)
                    wa *= w;
                    wb *= w;
                }
                const unsigned long long pa = dup2(wa), pb = dup2(wb);
#pragma unroll
                for (int h = 0; h < NQ; ++h) {
                    const float4 x = CT_DLOAD(ok, line + h * qplane + i);
                    const unsigned long long x01 = pack2(x.x, x.y), x23 = pack2(x.z, x.w);
                    A[2 * h] = fma2(pa, x01, A[2 * h]);
                    A[2 * h + 1] = fma2(pa, x23, A[2 * h + 1]);
                    B[2 * h] = fma2(pb, x01, B[2 * h]);
                    B[2 * h + 1] = fma2(pb, x23, B[2 * h + 1]);
                }
            }
        }
        Xl += bl.y;
        Xh += bh.y;
    }
    // channel c = strip c's f sum + strip c+1's (1-f) sum (+ the clamped taps)
    const int c = strip;
    const bool writes = lane < kBptOut && c < a.C;
    const size_t sstride = (size_t)a.V * a.C;
    float *out = sino + (size_t)blockIdx.y * 4 * NQ * sstride + (size_t)v * a.C + c;
    const int s0 = blockIdx.y * 4 * NQ;
#pragma unroll
    for (int h = 0; h < 2 * NQ; ++h) {
        const float2 av = unpack2(A[h]), bv = unpack2(B[h]);
        const float an0 = __shfl_down_sync(0xffffffffu, av.x, 1);
        const float an1 = __shfl_down_sync(0xffffffffu, av.y, 1);
        const float bn0 = __shfl_down_sync(0xffffffffu, bv.x, 1);
        const float bn1 = __shfl_down_sync(0xffffffffu, bv.y, 1);
        float r0 = bv.x + an0, r1 = bv.y + an1;
        if (c == 0) {
            r0 += av.x;
            r1 += av.y;
        }
        if (c == a.C - 1) {
            r0 += bn0;
            r1 += bn1;
        }
        if (writes) {
            if (s0 + 2 * h < nsl) out[(size_t)(2 * h) * sstride] = r0;
            if (s0 + 2 * h + 1 < nsl) out[(size_t)(2 * h + 1) * sstride] = r1;
        }
    }
}

// Slice-quad planes of `nq` quads (slices 4q .. 4q+3 of img, zero past
// `batch`): rows[q][y][x] and cols[q][x][y], through a shared-memory tile.
__global__ void __launch_bounds__(256)
    bpt_quads_kernel(const float *__restrict__ img, float4 *__restrict__ rows,
                     float4 *__restrict__ cols, int nx, int ny, int batch) {
    __shared__ float4 tile[32][33];
    const int q = blockIdx.z;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    const size_t plane = (size_t)nx * ny;
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int x = x0 + threadIdx.x, y = y0 + r;
        float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
        if (x < nx && y < ny) {
            float *tv = &t.x;
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                const int b = 4 * q + s;
                if (b < batch) tv[s] = __ldg(img + (size_t)b * plane + (size_t)y * nx + x);
            }
            rows[q * plane + (size_t)y * nx + x] = t;
        }
        tile[r][threadIdx.x] = t;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int x = x0 + r, y = y0 + threadIdx.x;
        if (x < nx && y < ny) cols[q * plane + (size_t)x * ny + y] = tile[threadIdx.x][r];
    }
}

constexpr int kChunk = 64;  // slices per pass (quad planes of 16 slice quads)

int quads_per_group(int nb) { return nb <= 4 ? 1 : (nb <= 8 || CT_BPG_NQ < 4 ? 2 : 4); }

int padded_quads(int nb) {
    const int nq = quads_per_group(nb);
    return ((nb + 3) / 4 + nq - 1) / nq * nq;
}

template <bool W, int NQ>
void launch_gather(const ct_plan *p, const BptArgs &a, dim3 grid, cudaStream_t s,
                   const float4 *rows, const float4 *cols, size_t qplane, float *sino, int nsl) {
    bp_gather_kernel<W, NQ><<<grid, 128, 0, s>>>(
        rows, cols, qplane, sino, nsl, reinterpret_cast<const int4 *>(p->d_bpt_warp),
        reinterpret_cast<const longlong2 *>(p->d_bpt_bnd),
        reinterpret_cast<const float4 *>(p->d_bpt_ray),
        reinterpret_cast<const int2 *>(p->d_fov_row),
        reinterpret_cast<const int2 *>(p->d_fov_col), a);
}

}  // namespace

bool bp_gather_usable(const ct_plan *p) {
    return p->d_bpt_warp != nullptr && p->opts.texture_weights == 0;
}

size_t bp_gather_work_bytes(const ct_plan *p, int batch) {
    if (!bp_gather_usable(p) || batch <= 0) return 0;
    const int nb = batch < kChunk ? batch : kChunk;
    return 2 * sizeof(float4) * (size_t)padded_quads(nb) * p->g.nx * p->g.ny;
}

int bp_gather(const ct_plan *p, const float *img, float *sino, int batch, int weighted,
              void *work, void *stream) {
    cudaStream_t s = (cudaStream_t)stream;
    BptArgs a;
    a.V = p->g.n_views;
    a.C = p->g.n_cols;
    a.W = p->bpt_W;
    a.nx = p->g.nx;
    a.ny = p->g.ny;
    a.vq = (a.V + 3) / 4;
    a.inv_dcol = (float)(1.0 / (double)p->g.dcol);
    const size_t plane = (size_t)a.nx * a.ny, sl = (size_t)a.V * a.C;
    for (int b0 = 0; b0 < batch; b0 += kChunk) {
        const int nb = batch - b0 < kChunk ? batch - b0 : kChunk;
        const int nq = quads_per_group(nb), pq = padded_quads(nb);
        float4 *rows = static_cast<float4 *>(work);
        float4 *cols = rows + (size_t)pq * plane;
        bpt_quads_kernel<<<dim3((a.nx + 31) / 32, (a.ny + 31) / 32, pq), dim3(32, 8), 0, s>>>(
            img + (size_t)b0 * plane, rows, cols, a.nx, a.ny, nb);
        dim3 grid((unsigned)(a.W * a.vq), (unsigned)(pq / nq));
        float *out = sino + (size_t)b0 * sl;
        if (weighted) {
            if (nq == 4)
                launch_gather<true, 4>(p, a, grid, s, rows, cols, plane, out, nb);
            else if (nq == 2)
                launch_gather<true, 2>(p, a, grid, s, rows, cols, plane, out, nb);
            else
                launch_gather<true, 1>(p, a, grid, s, rows, cols, plane, out, nb);
        } else {
            if (nq == 4)
                launch_gather<false, 4>(p, a, grid, s, rows, cols, plane, out, nb);
            else if (nq == 2)
                launch_gather<false, 2>(p, a, grid, s, rows, cols, plane, out, nb);
            else
                launch_gather<false, 1>(p, a, grid, s, rows, cols, plane, out, nb);
        }
        ct_count_launch(2);
    }
    return (int)cudaGetLastError();
}

}  // namespace ctk
