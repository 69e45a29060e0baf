// The backprojector's per-tile work, shared by the per-plan kernel and the
// uneven-batch kernel (geometry and arithmetic are described in bp.cu).
#pragma once

#include "fp_body.cuh"

namespace ctk {

constexpr int kBpTile = 32;       // tile edge (pixels)
constexpr int kBpRowsPerThr = 4;  // 32x8 threads cover 32x32 pixels

struct BpArgs {
    int V, C, nx, ny;
    float xmin, ymin, dx, dy;
    float R;
    float inv_dcol;   // 1/dcol
    float pos_off;    // shift - left/dcol + 1/2: y = atan*inv_dcol + pos_off = col + 1/2
    float fC;         // n_cols
    double fov_r2;
    float coef[9];    // atan(z) = z * sum coef[k] z^(2k) (zero-padded to degree 8)
};

template <int DEG>
__device__ __forceinline__ float fov_atan(float z, const float *c) {
    if constexpr (DEG == 0) {
        return atanf(z);
    } else {
        const float s = z * z;
        float p = c[DEG];
#pragma unroll
        for (int k = DEG - 1; k >= 0; --k) p = fmaf(p, s, c[k]);
        return z * p;
    }
}

// y = col + 1/2 >= 0: i = trunc(y) = floor(col - 1/2) + 1 and f = frac(y),
// without float-to-int conversion instructions (valid for 0 <= y < 2^22).
__device__ __forceinline__ void split_pos(float y, int &i, float &f) {
    const float m = __fadd_rz(y, 12582912.0f);
    i = __float_as_int(m) - 0x4B400000;
    f = y - (m - 12582912.0f);
}

// The GPU texture unit's linear-filter weight for a fraction f in [0, 1): f
// rounded to a multiple of 1/256, ties up (8 fractional bits; measured on
// GB300 against texture objects with the reference's sampler state).  The
// reference interpolates its sinogram rows through the texture unit
// (BP/transform.cu:90, FBP/transform.cu:85, FDK/GPURecon_GPU.cu:45); plans
// created with texture_weights = 1 reproduce it.  f * 256 + 1/2 is exact in
// FP32, so this is the rounding itself, not an approximation of it.
__device__ __forceinline__ float tex_weight(float f) {
    return floorf(fmaf(f, 256.0f, 0.5f)) * (1.0f / 256.0f);
}

// One 32 x (8 ROWS) tile (tx, ty) of nsl <= SB slices: sino slice s at
// sino + s * sstride ([V][C]), image slice s at img + s * istride ([ny][nx]).
// Block of 32 x 8 threads, ROWS pixels per thread (32 x 32 tiles by default);
// block-uniform call.  TEX: texture-unit weights (tex_weight) instead of
// exact FP32 ones.  PAIRS (SB = 4 or 8): the taps come from SB/4 consecutive
// four-slice tap planes at `pairs` ([V][C+1] x 2 float4 each, 32-byte
// aligned: for column position i, the clamped taps (i0, i1) of four slices,
// float4 h holding (i0, i1) of slices (2h, 2h+1) as (i0, i0, i1, i1)), SB/4
// 32-byte loads per pixel-view instead of 2 SB 4-byte gathers, and the
// interpolation and accumulation of two slices per f32x2 instruction; same
// values, same per-slice operations, so the same bits.
template <bool WEIGHTED, int SB, int DEG, typename OutT, int ROWS = kBpRowsPerThr,
          bool TEX = false, bool PAIRS = false>
__device__ __forceinline__ void bp_tile(const float *__restrict__ sino, size_t sstride,
                                        OutT *__restrict__ img, size_t istride,
                                        const float2 *__restrict__ view_cs, const BpArgs &a,
                                        int nsl, int tx, int ty,
                                        const float4 *__restrict__ pairs = nullptr) {
    static_assert(!PAIRS || SB == 4 || SB == 8, "tap images hold four or eight slices");
    const int ix = tx * kBpTile + threadIdx.x;
    const int iy0 = ty * (8 * ROWS) + threadIdx.y;
    float py[ROWS];
    bool in[ROWS];
    const double xd = (double)a.xmin + (double)a.dx * (ix + 0.5);
    const float px = (float)xd;
    bool any = false;
#pragma unroll
    for (int k = 0; k < ROWS; ++k) {
        const int iy = iy0 + 8 * k;
        const double yd = (double)a.ymin + (double)a.dy * (iy + 0.5);
        py[k] = (float)yd;
        in[k] = ix < a.nx && iy < a.ny && (xd * xd + yd * yd <= a.fov_r2);
        any |= in[k];
    }
    float acc[SB][ROWS];
    // PAIRS: slices (2j, 2j+1) as one f32x2 accumulator
    unsigned long long acc2[PAIRS ? SB / 2 : 1][ROWS];
#pragma unroll
    for (int s = 0; s < SB; ++s)
#pragma unroll
        for (int k = 0; k < ROWS; ++k) acc[s][k] = 0.0f;
#pragma unroll
    for (int j = 0; j < (PAIRS ? SB / 2 : 1); ++j)
#pragma unroll
        for (int k = 0; k < ROWS; ++k) acc2[j][k] = 0ull;
    if (__syncthreads_or(any)) {
        const float *sb[SB];
#pragma unroll
        for (int s = 0; s < SB; ++s) sb[s] = sino + (size_t)min(s, nsl - 1) * sstride;
        for (int v = 0; v < a.V; ++v) {
            const float2 cs = __ldg(view_cs + v);
            const size_t ro = (size_t)v * a.C;
#pragma unroll
            for (int k = 0; k < ROWS; ++k) {
                const float U = fmaf(px, cs.x, fmaf(py[k], cs.y, a.R));
                const float t = fmaf(py[k], cs.x, -px * cs.y);
                const float rU = __fdividef(1.0f, U);
                const float g = fov_atan<DEG>(t * rU, a.coef);
                const float y = fmaf(g, a.inv_dcol, a.pos_off);
                if (in[k] && y > 0.5f && y < a.fC + 0.5f) {
                    int i;
                    float f;
                    split_pos(y, i, f);
                    if constexpr (TEX) f = tex_weight(f);
                    const int i0 = max(i - 1, 0), i1 = min(i, a.C - 1);
                    float wgt = 1.0f;
                    if (WEIGHTED) wgt = __fdividef(1.0f, fmaf(U, U, t * t));
                    if constexpr (PAIRS) {
                        // one 32-byte load per four slices (the entries are 32-byte
                        // aligned); per slice pair the scalar path's operations as
                        // f32x2 instructions (each lane rounds as the FP32 one)
                        const float4 *q = pairs + ((size_t)v * (a.C + 1) + i) * 2;
                        const size_t plane4 = (size_t)a.V * (a.C + 1) * 2;
                        const bool ok = (unsigned)i <= (unsigned)a.C;
                        const unsigned long long ff = pack2(f, f), ww = pack2(wgt, wgt);
#pragma unroll
                        for (int h = 0; h < SB / 4; ++h) {
                            float4 t, u;
                            ldg_v8(ok, q + h * plane4, t, u);
                            const unsigned long long a0 = pack2(t.x, t.y), a1 = pack2(t.z, t.w);
                            const unsigned long long b0 = pack2(u.x, u.y), b1 = pack2(u.z, u.w);
                            const unsigned long long va = fma2(ff, sub2(a1, a0), a0);
                            const unsigned long long vb = fma2(ff, sub2(b1, b0), b0);
                            unsigned long long &ca = acc2[2 * h][k], &cb = acc2[2 * h + 1][k];
                            ca = WEIGHTED ? fma2(va, ww, ca) : add2(ca, va);
                            cb = WEIGHTED ? fma2(vb, ww, cb) : add2(cb, vb);
                        }
                    } else {
                        float v0[SB], v1[SB];
                        const bool ok = (unsigned)i0 < (unsigned)a.C && (unsigned)i1 < (unsigned)a.C;
#pragma unroll
                        for (int s = 0; s < SB; ++s) {
                            v0[s] = CT_DLOAD(ok, sb[s] + ro + i0);
                            v1[s] = CT_DLOAD(ok, sb[s] + ro + i1);
                        }
#pragma unroll
                        for (int s = 0; s < SB; ++s) {
                            const float val = fmaf(f, v1[s] - v0[s], v0[s]);
                            acc[s][k] = WEIGHTED ? fmaf(val, wgt, acc[s][k]) : acc[s][k] + val;
                        }
                    }
                }
            }
        }
    }
#pragma unroll
    for (int s = 0; s < SB; ++s) {
        if (s >= nsl) break;
        OutT *ib = img + (size_t)s * istride;
#pragma unroll
        for (int k = 0; k < ROWS; ++k) {
            const int iy = iy0 + 8 * k;
            float r = acc[s][k];
            if constexpr (PAIRS) {
                const float2 pr = unpack2(acc2[s / 2][k]);
                r = (s & 1) ? pr.y : pr.x;
            }
            if (ix < a.nx && iy < a.ny) store_val(ib + (size_t)iy * a.nx + ix, r);
        }
    }
}

}  // namespace ctk
