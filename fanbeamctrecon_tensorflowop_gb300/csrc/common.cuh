// Device helpers shared by the ctgb kernels.
#pragma once

#include <cuda_runtime.h>

#include "dbgcheck.cuh"
#include "internal.h"

namespace ctk {

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// 32 bytes at p (32-byte aligned) as two float4, one ld.global.nc.v8.f32
// (sm_100 and later).  When adjacent lanes read adjacent 32-byte entries the
// L1 load path completes it in about the time of one 16-byte load (measured:
// 148 against 78 TB/s of L1 hits), so such a gather costs half the load
// instructions of two 16-byte ones.  Gathers whose lanes scatter over many
// lines gain nothing (the forward projector's quads and its adjoint's
// sinogram measured slower with it).  `ok` is the debug build's index check
// (both halves read zero when it fails).
__device__ __forceinline__ void ldg_v8(bool ok, const float4 *p, float4 &a, float4 &b) {
    if (CT_DCHECK(ok)) {
        asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
            : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z),
              "=f"(b.w)
            : "l"(p));
    } else {
        a = b = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// Bilinear sample of a row-major [ny][nx] image at texture coordinates (x, y)
// -- texel (i, j) centred at (i + 1/2, j + 1/2) -- with clamp-to-edge
// addressing: the semantics of tex2D on a cudaFilterModeLinear,
// cudaAddressModeClamp texture (FP/transform.cu:224-227), with full FP32
// weights instead of the hardware's 8-bit fractions.
__device__ __forceinline__ float bilerp_clamp(const float *__restrict__ im, int nx, int ny,
                                              float x, float y) {
    const float xb = x - 0.5f, yb = y - 0.5f;
    const float fx = floorf(xb), fy = floorf(yb);
    const float ax = xb - fx, ay = yb - fy;
    const int i = static_cast<int>(fx), j = static_cast<int>(fy);
    const int i0 = min(max(i, 0), nx - 1), i1 = min(max(i + 1, 0), nx - 1);
    const int j0 = min(max(j, 0), ny - 1), j1 = min(max(j + 1, 0), ny - 1);
    const float *r0 = im + j0 * nx;
    const float *r1 = im + j1 * nx;
    const float v00 = __ldg(r0 + i0), v10 = __ldg(r0 + i1);
    const float v01 = __ldg(r1 + i0), v11 = __ldg(r1 + i1);
    const float a = fmaf(ax, v10 - v00, v00);
    const float b = fmaf(ax, v11 - v01, v01);
    return fmaf(ay, b - a, a);
}

}  // namespace ctk
