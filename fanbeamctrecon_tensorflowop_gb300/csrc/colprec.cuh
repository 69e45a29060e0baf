// Precise column fraction of a pixel-view, for the transposes of the
// pixel-driven backprojectors.
//
// The backprojectors place pixel p of view beta at column coordinate
// y = (atan(t/U) - left)/dcol + shift + 1/2 (BP/transform.cu:82-86), with
// U = R + x c + y s and t = -x s + y c.  In FP32, y (up to ~C) carries
// ~6e-5 of a channel of rounding from its own size, from U and t (sums of
// terms of hundreds of mm) and from atan: per-pixel noise that the ramp
// filter of the FBP / FDK adjoints amplifies about 80-fold (1.5e-4 relative
// L2 at the clinical geometry, against a 1e-4 contract).  Here U and t are
// formed in float-float (pixel centres, cos and sin of the view as hi + lo
// pairs, exact products by FMA), z = t/U likewise, and the angle is measured
// from the boundary ray y = b of the pixel's column strip,
//   tan(gamma - gamma_b) = (z - tan gamma_b) / (1 + z tan gamma_b),
// with tan gamma_b from a per-column FP64 table (hi + lo): a small argument,
// so its atan and the fraction f = (gamma - gamma_b)/dcol are accurate to
// ~1e-7 of a channel.  The FP32 y still picks the strip b = trunc(y) and the
// FOV/detector tests; where it lands one strip off (within its rounding of a
// boundary) f comes out just outside [0, 1) and the strip moves by one.
#pragma once

#include "common.cuh"

namespace ctk {

struct FF {
    float h, l;
};

__device__ __forceinline__ FF ff_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return FF{s, (a - (s - bb)) + (b - bb)};
}

// U and t of pixel (x, y) (hi + lo each) in view (c, s) (hi + lo each)
__device__ __forceinline__ void ff_ut(float xh, float xl, float yh, float yl, float ch, float cl,
                                      float sh, float sl, float R, FF &U, FF &t) {
    // t = y c - x s
    const float a1 = yh * ch, e1 = fmaf(yh, ch, -a1);
    const float a2 = -xh * sh, e2 = fmaf(-xh, sh, -a2);
    const FF ts = ff_two_sum(a1, a2);
    t.h = ts.h;
    t.l = ts.l + e1 + e2 + fmaf(yh, cl, fmaf(yl, ch, fmaf(-xh, sl, -xl * sh)));
    // U = R + x c + y s
    const float b1 = xh * ch, f1 = fmaf(xh, ch, -b1);
    const float b2 = yh * sh, f2 = fmaf(yh, sh, -b2);
    const FF s12 = ff_two_sum(b1, b2);
    const FF us = ff_two_sum(R, s12.h);
    U.h = us.h;
    U.l = us.l + s12.l + f1 + f2 + fmaf(xh, cl, fmaf(xl, ch, fmaf(yh, sl, yl * sh)));
}

// The row part of ff_ut for an image row at y: t_row = y c, U_row = R + y s.
__device__ __forceinline__ void ff_row(float yh, float yl, float ch, float cl, float sh,
                                       float sl, float R, FF &t_row, FF &U_row) {
    const float a = yh * ch;
    t_row.h = a;
    t_row.l = fmaf(yh, ch, -a) + fmaf(yh, cl, yl * ch);
    const float b = yh * sh;
    const FF us = ff_two_sum(R, b);
    U_row.h = us.h;
    U_row.l = us.l + fmaf(yh, sh, -b) + fmaf(yh, sl, yl * sh);
}

// Completes ff_row for the pixel at x: t = t_row - x s, U = U_row + x c.
__device__ __forceinline__ void ff_pixel(float xh, float xl, float ch, float cl, float sh,
                                         float sl, const FF &t_row, const FF &U_row, FF &U,
                                         FF &t) {
    const float p = -xh * sh;
    const FF ts = ff_two_sum(t_row.h, p);
    t.h = ts.h;
    t.l = ts.l + fmaf(-xh, sh, -p) + t_row.l + fmaf(-xh, sl, -xl * sh);
    const float q = xh * ch;
    const FF us = ff_two_sum(U_row.h, q);
    U.h = us.h;
    U.l = us.l + fmaf(xh, ch, -q) + U_row.l + fmaf(xh, cl, xl * ch);
}

// Strip ic (from the FP32 column coordinate) and the precise fraction f of
// the pixel's angle from the strip's lower boundary, in channels; ic and f
// are corrected when the FP32 strip was one off.  tan_b: [C+1] (hi, lo) of
// tan(gamma_b), gamma_b = left + (b - shift - 1/2) dcol.
__device__ __forceinline__ void precise_strip(const FF &U, const FF &t,
                                              const float2 *__restrict__ tan_b, float inv_dcol,
                                              int C, int &ic, float &f) {
    const float rU = __fdividef(1.0f, U.h);
    const float zh = t.h * rU;
    const float r = fmaf(-zh, U.h, t.h) + fmaf(-zh, U.l, t.l);
    const float zl = r * rU;
    const float2 tb = __ldg(tan_b + ic);
    const float u = __fdividef((zh - tb.x) + (zl - tb.y), fmaf(zh, tb.x, 1.0f));
    const float u2 = u * u;
    f = u * fmaf(u2, fmaf(u2, 0.2f, -0.33333334f), 1.0f) * inv_dcol;
    if (f < 0.0f && ic > 0) {
        ic -= 1;
        f += 1.0f;
    } else if (f >= 1.0f && ic < C) {
        ic += 1;
        f -= 1.0f;
    }
    f = fminf(fmaxf(f, 0.0f), 1.0f);
}

}  // namespace ctk
