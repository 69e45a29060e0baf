// Exact per-cell summation of the ray-driven projector's samples.
//
// The reference's forward projector sums a bilinear, clamp-to-edge image
// sample at every point start + k*step, k < n (FP/transform.cu:125-129).  In
// cell coordinates (u, v) = texture coordinates - 1/2, the bilinear
// interpolant inside one cell [cu, cu+1) x [cv, cv+1) is
//   (1-fu)(1-fv) T00 + fu (1-fv) T10 + (1-fu) fv T01 + fu fv T11,
// and along a ray the fractions are linear in k: fu = a + su*j, fv = b + sv*j
// for the j-th sample inside the cell.  The sum over the cnt samples of one
// cell therefore needs only sum 1, sum j and sum j^2:
//   S1 = cnt(cnt-1)/2, S2 = S1 (2cnt-1)/3,
//   Su = cnt a + su S1, Sv = cnt b + sv S1,
//   Suv = cnt a b + (a sv + b su) S1 + su sv S2,
//   W11 = Suv, W10 = Su - Suv, W01 = Sv - Suv, W00 = cnt - Su - Sv + Suv.
// walk_cells visits the cells a ray crosses in order (the next boundary in u
// or v, whichever comes first in k) and hands each non-empty cell's sample
// count and entry fractions to a callback.  A sample that lies within
// rounding of a cell boundary may be attributed to the neighbouring cell;
// because the clamped bilinear interpolant is continuous across cell
// boundaries this changes its value only by that rounding.
#pragma once

#include "common.cuh"

namespace ctk {

struct RaySeg {
    float u0, v0;  // cell coordinates of sample 0
    float su, sv;  // step per sample
};

struct CellWeights {
    float w00, w10, w01, w11;
};

__device__ __forceinline__ CellWeights cell_weights(float cnt, float a, float b, float su,
                                                    float sv) {
    const float s1 = 0.5f * cnt * (cnt - 1.0f);
    const float s2 = s1 * (2.0f * cnt - 1.0f) * (1.0f / 3.0f);
    const float su_sum = fmaf(cnt, a, su * s1);
    const float sv_sum = fmaf(cnt, b, sv * s1);
    const float suv = fmaf(cnt * a, b, fmaf(fmaf(a, sv, b * su), s1, su * sv * s2));
    CellWeights w;
    w.w11 = suv;
    w.w10 = su_sum - suv;
    w.w01 = sv_sum - suv;
    w.w00 = (cnt - su_sum) - (sv_sum - suv);
    return w;
}

// Visits the cells holding samples k in [k0, k1) (integer-valued floats,
// k1 <= 2^24).  f(cu, cv, cnt, a, b) receives the cell, its sample count and
// the fractions (a, b) of its first sample.  At most max_iter cells are
// visited (a segment inside an nx-by-ny image crosses fewer than nx+ny+2).
template <class F>
__device__ __forceinline__ void walk_cells(const RaySeg &s, float k0, float k1, int max_iter,
                                           F &&f) {
    const float INF = __int_as_float(0x7f800000);
    float cu = floorf(fmaf(s.su, k0, s.u0));
    float cv = floorf(fmaf(s.sv, k0, s.v0));
    const float du = s.su >= 0.0f ? 1.0f : -1.0f;
    const float dv = s.sv >= 0.0f ? 1.0f : -1.0f;
    const float iu = s.su != 0.0f ? 1.0f / s.su : 0.0f;
    const float iv = s.sv != 0.0f ? 1.0f / s.sv : 0.0f;
    // next boundary in u (v): cu + 1 when moving up, cu when moving down
    float bu = s.su >= 0.0f ? cu + 1.0f : cu;
    float bv = s.sv >= 0.0f ? cv + 1.0f : cv;
    float tu = s.su != 0.0f ? (bu - s.u0) * iu : INF;
    float tv = s.sv != 0.0f ? (bv - s.v0) * iv : INF;
    float k = k0;
    for (int it = 0; it < max_iter && k < k1; ++it) {
        const bool take_u = tu < tv;
        const float tn = take_u ? tu : tv;
        const float ke = fminf(k1, ceilf(tn));
        const float cnt = ke - k;
        if (cnt > 0.0f) {
            const float a = fmaf(s.su, k, s.u0) - cu;
            const float b = fmaf(s.sv, k, s.v0) - cv;
            f(static_cast<int>(cu), static_cast<int>(cv), cnt, a, b);
            k = ke;
        }
        if (take_u) {
            cu += du;
            bu += du;
            tu = (bu - s.u0) * iu;
        } else {
            cv += dv;
            bv += dv;
            tv = (bv - s.v0) * iv;
        }
    }
}

}  // namespace ctk
