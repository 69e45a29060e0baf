// Exact transpose of the ray-driven projector (fp.cu) as a gather: no
// atomics, deterministic, one write per output value.
//
// The projector computes p[v,c] = w * sum_{k<n} B(x0 + k sx, y0 + k sy) with
// B the clamp-to-edge bilinear interpolation in texture coordinates (texel
// (i,j) centred at (i+1/2, j+1/2)) and (x0, y0, sx, sy, n) the ray table
// (FP/transform.cu:64-101, 119-144).  A sample in the cell between texel
// centres (ci+1/2 .. ci+3/2, cj+1/2 .. cj+3/2) gives its four corner texels
// the bilinear weights (1-fu)(1-fv), fu(1-fv), (1-fu)fv, fu fv, which are
// products of linear functions of the sample index inside the cell.
//
// Thread = one cell.  Per view it finds the few rays that can cross it, and
// for each computes the range of samples inside the cell (both neighbours of
// a cell boundary use the same threshold, so every sample lands in exactly
// one cell) and the four corner sums in closed form from sum j and sum j^2,
// times p[v,c] for up to 8 slices.  A second pass adds, per texel, the
// matching corner of its four cells.
//
// Candidate rays of a view: the ray through the cell centre has fan angle
// gamma_p = atan(t/U) (the backprojector's geometry in texture units); a ray
// meets the cell only if its angle is within asin(h/L) of gamma_p, with
// h = (|cos th| + |sin th|)/2 the cell's half-width across the ray direction
// th (plus 1/L for the change of th across the range) and L the distance to
// the source.  Candidates are conservative: a ray that misses adds zero.
//
// The border cells ci = -1 and ci = nx-1 (likewise in v) extend to the FOV
// edge: the clamped taps put both of their corners on one texel, so all of
// the weight goes to that corner; they take their candidate rays from the
// angular range of their bounding box.
#include "common.cuh"

namespace ctk {
namespace {

constexpr int kGThreads = 256;  // 32 x 8 cells per block

struct CellArgs {
    int V, C, nx, ny;
    float coef[9];   // atan(z) = z * sum coef[k] z^(2k) on the FOV widened by 1.5 pixels
    float src;       // sid / dx (texture units)
    float fov;       // rfov / dx: the FOV disc is centred at (fov, fov)
    float left, inv_dcol;
    float skip_r2;   // (fov + 0.75)^2: cells whose centre is farther see no sample
};

// Channel coordinate c + 1/2 = (gamma - left)/dcol of a texture-space point;
// DEG > 0: the plan's atan polynomial (valid within the widened FOV).
template <int DEG>
__device__ __forceinline__ float chan_of(float u, float v, float2 cs, const CellArgs &a,
                                         float &U, float &T) {
    const float x = u - a.fov, y = v - a.fov;
    U = fmaf(x, cs.x, fmaf(y, cs.y, a.src));
    T = fmaf(y, cs.x, -x * cs.y);
    float g;
    if constexpr (DEG == 0) {
        g = atanf(T / U);
    } else {
        const float z = T * __fdividef(1.0f, U), s2 = z * z;
        float p = a.coef[DEG];
#pragma unroll
        for (int k = DEG - 1; k >= 0; --k) p = fmaf(p, s2, a.coef[k]);
        g = z * p;
    }
    return (g - a.left) * a.inv_dcol;
}

template <int SB, int DEG>
__global__ void __launch_bounds__(kGThreads)
    fp_adjoint_cells_kernel(const float *__restrict__ sino, float *__restrict__ corners,
                            const float4 *__restrict__ ray, const float2 *__restrict__ ray_inv,
                            const int *__restrict__ nsamp, const float2 *__restrict__ view_cs,
                            CellArgs a, int batch) {
    const int NXC = a.nx + 1, NYC = a.ny + 1;
    const int ic = blockIdx.x * 32 + threadIdx.x, jc = blockIdx.y * 8 + threadIdx.y;
    const int ci = ic - 1, cj = jc - 1;
    const int b0 = blockIdx.z * SB;
    const int nsl = min(SB, batch - b0);
    const bool xlo = ci == -1, xhi = ci == a.nx - 1, ylo = cj == -1, yhi = cj == a.ny - 1;
    const bool ext = xlo || xhi || ylo || yhi;
    const float INF = __int_as_float(0x7f800000);
    // cell span [lo, hi) in texture coordinates
    const float ulo = xlo ? -INF : (float)ci + 0.5f, uhi = xhi ? INF : (float)ci + 1.5f;
    const float vlo = ylo ? -INF : (float)cj + 0.5f, vhi = yhi ? INF : (float)cj + 1.5f;
    const float uc = (float)ci + 1.0f, vcn = (float)cj + 1.0f;  // centre of an interior cell
    const bool inside = ic < NXC && jc < NYC;
    const float dxc = uc - a.fov, dyc = vcn - a.fov;
    const bool act = inside && (ext || dxc * dxc + dyc * dyc <= a.skip_r2);
    float w00[SB], w10[SB], w01[SB], w11[SB];
#pragma unroll
    for (int s = 0; s < SB; ++s) w00[s] = w10[s] = w01[s] = w11[s] = 0.0f;
    const size_t slice = (size_t)a.V * a.C;
    const float *sb = sino + (size_t)b0 * slice;
    if (__syncthreads_or(act) && act) {
        for (int v = 0; v < a.V; ++v) {
            const float2 cs = __ldg(view_cs + v);
            const size_t row = (size_t)v * a.C;
            float clo, chi;
            if (!ext) {
                float U, T;
                const float cp = chan_of<DEG>(uc, vcn, cs, a, U, T) - 0.5f;
                const float rL = rsqrtf(fmaf(U, U, T * T));
                // half-width of the cell across the ray, plus the drift of th
                const float h = 0.5f * (fabsf(fmaf(cs.y, T, -cs.x * U)) +
                                        fabsf(fmaf(cs.y, U, cs.x * T))) * rL + rL;
                const float z = h * rL;
                const float hw = z * fmaf(z, z, 1.0f) * a.inv_dcol + 0.01f;
                clo = cp - hw;
                chi = cp + hw;
            } else {
                const float u0 = xlo ? -1.0f : ulo, u1 = xhi ? 2.0f * a.fov + 1.0f : uhi;
                const float v0 = ylo ? -1.0f : vlo, v1 = yhi ? 2.0f * a.fov + 1.0f : vhi;
                float U, T;
                const float q0 = chan_of<0>(u0, v0, cs, a, U, T);
                const float q1 = chan_of<0>(u1, v0, cs, a, U, T);
                const float q2 = chan_of<0>(u0, v1, cs, a, U, T);
                const float q3 = chan_of<0>(u1, v1, cs, a, U, T);
                clo = fminf(fminf(q0, q1), fminf(q2, q3)) - 0.5f - 0.01f;
                chi = fmaxf(fmaxf(q0, q1), fmaxf(q2, q3)) - 0.5f + 0.01f;
            }
            const int c0 = max(0, (int)ceilf(fmaxf(clo, -1.0f)));
            const int c1 = min(a.C - 1, (int)floorf(fminf(chi, (float)a.C)));
            for (int c = c0; c <= c1; ++c) {
                const int n = __ldg(nsamp + row + c);
                if (n <= 0) continue;
                const float4 q = __ldg(ray + row + c);
                const float2 iv = __ldg(ray_inv + row + c);
                // samples with lo <= x0 + k s < hi; both neighbours of a cell
                // boundary use the same threshold, so every sample lands in
                // exactly one cell (a zero step has iv = 1e30: all or none)
                float ka, kb, ta, tb;
                ta = (ulo - q.x) * iv.x;
                tb = (uhi - q.x) * iv.x;
                if (q.z >= 0.0f) {
                    ka = ceilf(ta);
                    kb = ceilf(tb) - 1.0f;
                } else {
                    ka = floorf(tb) + 1.0f;
                    kb = floorf(ta);
                }
                ta = (vlo - q.y) * iv.y;
                tb = (vhi - q.y) * iv.y;
                if (q.w >= 0.0f) {
                    ka = fmaxf(ka, ceilf(ta));
                    kb = fminf(kb, ceilf(tb) - 1.0f);
                } else {
                    ka = fmaxf(ka, floorf(tb) + 1.0f);
                    kb = fminf(kb, floorf(ta));
                }
                ka = fmaxf(ka, 0.0f);
                kb = fminf(kb, (float)(n - 1));
                if (!(ka <= kb)) continue;
                const float cnt = kb - ka + 1.0f;
                // fractions toward the upper corners, linear in j = k - ka; a
                // border cell puts all of its weight on its in-image corner
                const float fu = xlo ? 1.0f : (xhi ? 0.0f : fmaf(ka, q.z, q.x) - ulo);
                const float su = (xlo || xhi) ? 0.0f : q.z;
                const float fv = ylo ? 1.0f : (yhi ? 0.0f : fmaf(ka, q.w, q.y) - vlo);
                const float sv = (ylo || yhi) ? 0.0f : q.w;
                const float S1 = 0.5f * cnt * (cnt - 1.0f);
                const float S2 = S1 * (2.0f * cnt - 1.0f) * (1.0f / 3.0f);
                const float P = fu * fv * cnt + fmaf(fu, sv, fv * su) * S1 + su * sv * S2;
                const float F = fmaf(fu, cnt, su * S1), G = fmaf(fv, cnt, sv * S1);
                const float W11 = P, W10 = F - P, W01 = G - P, W00 = cnt - F - G + P;
#pragma unroll
                for (int s = 0; s < SB; ++s) {
                    if (s < nsl) {
                        const float val = __ldg(sb + s * slice + row + c);
                        w00[s] = fmaf(W00, val, w00[s]);
                        w10[s] = fmaf(W10, val, w10[s]);
                        w01[s] = fmaf(W01, val, w01[s]);
                        w11[s] = fmaf(W11, val, w11[s]);
                    }
                }
            }
        }
    }
    if (inside) {
        const size_t plane = (size_t)NXC * NYC, o = (size_t)jc * NXC + ic;
#pragma unroll
        for (int s = 0; s < SB; ++s) {
            if (s >= nsl) break;
            float *cb = corners + (size_t)(b0 + s) * 4 * plane;
            cb[o] = w00[s];
            cb[plane + o] = w10[s];
            cb[2 * plane + o] = w01[s];
            cb[3 * plane + o] = w11[s];
        }
    }
}

// texel (i, j) = corner 00 of cell (i, j) + 10 of (i-1, j) + 01 of (i, j-1)
// + 11 of (i-1, j-1), times the projector weight
__global__ void __launch_bounds__(256)
    fp_adjoint_combine_kernel(const float *__restrict__ corners, float *__restrict__ img, int nx,
                              int ny, float w, int batch) {
    const int NXC = nx + 1, NYC = ny + 1;
    const size_t plane = (size_t)NXC * NYC;
    const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
    if (i >= nx || j >= ny) return;
    for (int b = blockIdx.z; b < batch; b += gridDim.z) {
        const float *cb = corners + (size_t)b * 4 * plane;
        const size_t o00 = (size_t)(j + 1) * NXC + (i + 1);  // cell (i, j)
        const float t = cb[o00] + cb[plane + o00 - 1] + cb[2 * plane + o00 - NXC] +
                        cb[3 * plane + o00 - NXC - 1];
        img[(size_t)b * nx * ny + (size_t)j * nx + i] = t * w;
    }
}

}  // namespace

size_t fp_fan_adjoint_work_bytes(const ct_plan *p, int batch) {
    const int chunk = batch < 64 ? batch : 64;
    return sizeof(float) * 4 * (size_t)chunk * (p->g.nx + 1) * (p->g.ny + 1);
}

int fp_fan_adjoint(const ct_plan *p, const float *sino, float *img, int batch, void *work,
                   void *stream) {
    CellArgs a;
    a.V = p->g.n_views;
    a.C = p->g.n_cols;
    a.nx = p->g.nx;
    a.ny = p->g.ny;
    const double dx = p->g.dx;
    a.src = (float)((double)p->g.sid / dx);
    const double fov = (double)p->g.rfov / dx;
    a.fov = (float)fov;
    a.left = p->g.left;
    a.inv_dcol = (float)(1.0 / (double)p->g.dcol);
    a.skip_r2 = (float)((fov + 0.75) * (fov + 0.75));
    for (int k = 0; k < 9; ++k) a.coef[k] = p->gather_atan_coef[k];
    const int deg = p->gather_atan_deg;
    const float2 *vcs = reinterpret_cast<const float2 *>(p->d_view_cs);
    const float4 *ray = reinterpret_cast<const float4 *>(p->d_ray);
    const float2 *rinv = reinterpret_cast<const float2 *>(p->d_ray_inv);
    cudaStream_t s = (cudaStream_t)stream;
    float *corners = static_cast<float *>(work);
    const size_t plane = (size_t)a.nx * a.ny, slice = (size_t)a.V * a.C;
    for (int b0 = 0; b0 < batch; b0 += 64) {
        const int nb = batch - b0 < 64 ? batch - b0 : 64;
        const int SB = nb >= 8 ? 8 : (nb >= 4 ? 4 : 1);
        dim3 grid((a.nx + 1 + 31) / 32, (a.ny + 1 + 7) / 8, (nb + SB - 1) / SB);
        const float *sp = sino + b0 * slice;
        auto go = [&](auto kern) {
            kern<<<grid, dim3(32, 8), 0, s>>>(sp, corners, ray, rinv, p->d_nsamp, vcs, a, nb);
        };
        if (SB == 8)
            deg == 8 ? go(fp_adjoint_cells_kernel<8, 8>)
                     : deg == 4 ? go(fp_adjoint_cells_kernel<8, 4>) : go(fp_adjoint_cells_kernel<8, 0>);
        else if (SB == 4)
            deg == 8 ? go(fp_adjoint_cells_kernel<4, 8>)
                     : deg == 4 ? go(fp_adjoint_cells_kernel<4, 4>) : go(fp_adjoint_cells_kernel<4, 0>);
        else
            deg == 8 ? go(fp_adjoint_cells_kernel<1, 8>)
                     : deg == 4 ? go(fp_adjoint_cells_kernel<1, 4>) : go(fp_adjoint_cells_kernel<1, 0>);
        fp_adjoint_combine_kernel<<<dim3((a.nx + 31) / 32, (a.ny + 7) / 8, nb < 64 ? nb : 64),
                                    dim3(32, 8), 0, s>>>(corners, img + b0 * plane, a.nx, a.ny,
                                                         p->fp_weight, nb);
        ct_count_launch(2);
    }
    return (int)cudaGetLastError();
}

}  // namespace ctk
