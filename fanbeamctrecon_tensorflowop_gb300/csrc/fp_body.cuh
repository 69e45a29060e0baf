// The forward projector's per-warp work, shared by the per-plan kernel and the
// uneven-batch kernel.  Quad images, the row-synchronous walk and the closed
// form per cell are described in fp.cu.
#pragma once

#include <climits>

#include <cuda_bf16.h>

#include "cellwalk.cuh"

namespace ctk {

__device__ __forceinline__ void store_val(float *p, float v) { *p = v; }
__device__ __forceinline__ void store_val(__nv_bfloat16 *p, float v) { *p = __float2bfloat16(v); }
__device__ __forceinline__ float load_val(const float *p) { return __ldg(p); }
__device__ __forceinline__ float load_val(const __nv_bfloat16 *p) {
    return __bfloat162float(__ldg(p));
}

// Two FP32 lanes in one 64-bit register for the f32x2 FMA (each lane rounds
// as fmaf does).
__device__ __forceinline__ unsigned long long pack2(float x, float y) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
    return r;
}
__device__ __forceinline__ float2 unpack2(unsigned long long r) {
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
    return v;
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b,
                                                   unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ unsigned long long add2(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long sub2(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// Per slice the cell's dot product w . taps runs as two f32x2 FMAs into a
// pair (w00 t.x + w01 t.z, w10 t.y + w11 t.w), summed at the end.
template <int SB>
struct Taps {
    const float4 *q;  // this warp's layout of the first slice; slice s adds s * stride
    size_t stride;    // quads between consecutive slices
    int Q;            // quads per row (nx + 1)
    unsigned long long acc[SB];
    __device__ __forceinline__ void add(const CellWeights &cw, int cu, int cv) {
        const int qi = min(max(cu + 1, 0), Q - 1), qj = min(max(cv + 1, 0), Q - 1);
        // the walk stays on cells -1 .. nx-1 (quads 0 .. nx): the clamp is a guard
        const bool ok = (unsigned)(cu + 1) < (unsigned)Q && (unsigned)(cv + 1) < (unsigned)Q;
        const float4 *p = q + (size_t)qj * Q + qi;
        const unsigned long long wa = pack2(cw.w00, cw.w10), wb = pack2(cw.w01, cw.w11);
#pragma unroll
        for (int s = 0; s < SB; ++s) {
            const float4 t = CT_DLOAD(ok, p + s * stride);
            acc[s] = fma2(wa, pack2(t.x, t.y), acc[s]);
            acc[s] = fma2(wb, pack2(t.z, t.w), acc[s]);
        }
    }
    __device__ __forceinline__ float sum(int s) const {
        const float2 v = unpack2(acc[s]);
        return v.x + v.y;
    }
};

// One warp = 32 consecutive channels of one view (unit gw: view gw / wpv,
// channels 32 * (gw % wpv) + lane); warps never straddle views.  The warp
// votes its layout (transposed when most rays run along x) and its row
// direction, then steps through the rows of that layout in lockstep: in each
// row every lane sums the (one to three) cells its ray crosses there, so the
// lanes gather from the same one or two rows at a time whatever depth their
// rays entered the FOV at.  A lane whose ray runs against the warp's
// direction (possible only at a layout boundary) walks on its own afterwards.
// quads: both layouts of slice 0, slices `qstride` quads apart; out: the
// [V][C] sinogram of slice 0, slices `ostride` apart; nsl valid slices.
template <int SB, typename OutT>
__device__ __forceinline__ void fp_warp(const float4 *__restrict__ quads, size_t qstride,
                                        OutT *__restrict__ out, size_t ostride,
                                        const float4 *__restrict__ ray,
                                        const int *__restrict__ nsamp, int V, int C, int wpv,
                                        int nx, float w, int nsl, int max_iter, int gw) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int v = gw / wpv;
    const int c = (gw - v * wpv) * 32 + lane;
    const bool has_c = c < C;
    const int r = v * C + (has_c ? c : C - 1);
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
    tp.stride = qstride;
    tp.q = quads + (along_x ? lsz : 0);
#pragma unroll
    for (int s = 0; s < SB; ++s) tp.acc[s] = 0ull;
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
            if (s < nsl) store_val(out + (size_t)s * ostride + (size_t)v * C + c, tp.sum(s) * w);
    }
}

// Quad images (layout 0 walks (u, v) = (x, y); layout 1 the transposed image,
// (u, v) = (y, x)): for every bilinear cell (cu, cv) of the walked layout the
// four clamp-to-edge taps (cu,cv), (cu+1,cv), (cu,cv+1), (cu+1,cv+1) as one
// float4.  Samples lie inside the FOV circle of radius nx/2 texels, so cells
// run over [-1, nx-1] in both axes of both layouts; quad (qi, qj) holds cell
// (qi-1, qj-1) and a layout is (nx+1)^2 quads.
template <typename T>
__device__ __forceinline__ void build_quad(const T *__restrict__ im, float4 *__restrict__ dst,
                                           int nx, int ny, int layout, int qi, int qj) {
    const int cu = qi - 1, cv = qj - 1;
    float4 t;
    float *tv = &t.x;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int du = k & 1, dv = k >> 1;
        int x = layout ? cv + dv : cu + du;
        int y = layout ? cu + du : cv + dv;
        x = min(max(x, 0), nx - 1);
        y = min(max(y, 0), ny - 1);
        tv[k] = load_val(im + (size_t)y * nx + x);
    }
    *dst = t;
}

}  // namespace ctk
