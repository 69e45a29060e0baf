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
// times p[v,c] for up to 16 slices.  A second pass adds, per texel, the
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

constexpr int kGThreads = 256;  // 16 x 16 cells per block
// Views whose candidate rays share one loop (32 clinical slices, the same bits:
// 1 / 2 / 4 / 8 views 10.00 / 8.44 / 8.95 / 9.75 ms).
#ifndef CT_ADJ_VIEWS
#define CT_ADJ_VIEWS 2
#endif
constexpr int kAdjViews = CT_ADJ_VIEWS;
constexpr int kCellTile = 16;
#ifndef CT_ADJ_MAX_SB
#define CT_ADJ_MAX_SB 16
#endif
// Resident blocks per SM the register allocation must allow (measured best on
// GB300 for 32 clinical slices: 16 slices x 2 blocks 11.4 ms, 8 x 3 15.0 ms,
// 8 x 2 19.7 ms, 16 x 1 19.1 ms).
constexpr int adj_min_blocks(int sb) { return sb >= 16 ? 2 : (sb >= 8 ? 3 : 4); }

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

// Two FP32 lanes in one 64-bit register: the f32x2 FMA does both slices of a
// pair in one instruction (each lane rounds as fmaf does).
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

// [nb][V][C] -> [ceil(nb/SB)][V][C][SB] (missing slices of the last group are
// zero): one (view, channel) holds its SB slices in SB/4 aligned float4s.
template <int SB>
__global__ void __launch_bounds__(256)
    interleave_kernel(const float *__restrict__ sino, float *__restrict__ out, int nb,
                      size_t slice) {
    const size_t groups = (nb + SB - 1) / SB;
    const size_t total = groups * slice;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x) {
        const size_t g = e / slice, r = e - g * slice;
        float v[SB];
#pragma unroll
        for (int s = 0; s < SB; ++s) {
            const size_t b = g * SB + s;
            v[s] = b < (size_t)nb ? __ldg(sino + b * slice + r) : 0.0f;
        }
        float4 *o = reinterpret_cast<float4 *>(out + e * SB);
#pragma unroll
        for (int q = 0; q < SB / 4; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
}

// Thread = one cell; the SB slices of a group come interleaved
// ([V][C][SB], SB = 4, 8 or 16) and accumulate in f32x2 pairs.
template <int SB, int DEG>
__global__ void __launch_bounds__(kGThreads, adj_min_blocks(SB))
    fp_adjoint_cells_kernel(const float *__restrict__ sino, float *__restrict__ corners,
                            const float4 *__restrict__ ray_rec,
                            const float2 *__restrict__ view_cs,
                            CellArgs a, int batch) {
    const int NXC = a.nx + 1, NYC = a.ny + 1;
    // block = 16 x 16 cells; a warp takes a 4 x 8 patch, whose cells see more
    // similar candidate-ray counts than a 32-cell row (measured for 32
    // clinical slices: 32 x 1 rows 11.38 ms, 8 x 4 10.99, 4 x 8 10.31)
    const int tid = threadIdx.y * 32 + threadIdx.x, w = tid >> 5, ln = tid & 31;
    const int ic = blockIdx.x * kCellTile + (w & 3) * 4 + (ln & 3);
    const int jc = blockIdx.y * kCellTile + (w >> 2) * 8 + (ln >> 2);
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
    static_assert(SB == 4 || SB == 8 || SB == 16, "slices per group");
    constexpr int NP = SB / 2;  // f32x2 pairs
    unsigned long long w00[NP], w10[NP], w01[NP], w11[NP];
#pragma unroll
    for (int s = 0; s < NP; ++s) w00[s] = w10[s] = w01[s] = w11[s] = 0ull;
    const size_t slice = (size_t)a.V * a.C;
    const float4 *sb = reinterpret_cast<const float4 *>(sino + (size_t)blockIdx.z * slice * SB);
    if (__syncthreads_or(act) && act) {
        // the candidate channels [c0, c0 + n) of view v
        auto candidates = [&](int v, int &c0, int &n) {
            const float2 cs = __ldg(view_cs + v);
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
            c0 = max(0, (int)ceilf(fmaxf(clo, -1.0f)));
            n = max(0, min(a.C - 1, (int)floorf(fminf(chi, (float)a.C))) - c0 + 1);
        };
        // Views in groups of kAdjViews: one loop runs over the candidates of
        // all of them, so a warp iterates max over its lanes of the group's
        // total, not the sum of the per-view maxima; the candidates still come
        // in view order (the same sums).
        for (int v = 0; v < a.V; v += kAdjViews) {
            int c0g[kAdjViews], ng[kAdjViews], tot = 0;
#pragma unroll
            for (int h = 0; h < kAdjViews; ++h) {
                c0g[h] = 0;
                ng[h] = 0;
                if (v + h < a.V) candidates(v + h, c0g[h], ng[h]);
                tot += ng[h];
            }
            for (int t = 0; t < tot; ++t) {
                // candidate t: view v + h, channel c0g[h] + o
                int h = 0, o = t;
#pragma unroll
                for (int k = 0; k + 1 < kAdjViews; ++k)
                    if (h == k && o >= ng[k]) {
                        o -= ng[k];
                        h = k + 1;
                    }
                int cb = c0g[0];
#pragma unroll
                for (int k = 1; k < kAdjViews; ++k) cb = h == k ? c0g[k] : cb;
                const int c = cb + o;
                const size_t row = (size_t)(v + h) * a.C;
                // the ray's 32-byte record: start and step (q), 1/step, count
                float4 q, iv;
                ldg_v8((unsigned)c < (unsigned)a.C, ray_rec + 2 * (row + c), q, iv);
                const int n = __float_as_int(iv.z);
                if (n <= 0) continue;
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
                const unsigned long long p00 = pack2(W00, W00), p10 = pack2(W10, W10);
                const unsigned long long p01 = pack2(W01, W01), p11 = pack2(W11, W11);
                const bool ok = (unsigned)c < (unsigned)a.C;
#pragma unroll
                for (int q = 0; q < SB / 4; ++q) {
                    const float4 val = CT_DLOAD(ok, sb + (row + c) * (SB / 4) + q);
                    const unsigned long long lo = pack2(val.x, val.y), hi = pack2(val.z, val.w);
                    w00[2 * q] = fma2(p00, lo, w00[2 * q]);
                    w00[2 * q + 1] = fma2(p00, hi, w00[2 * q + 1]);
                    w10[2 * q] = fma2(p10, lo, w10[2 * q]);
                    w10[2 * q + 1] = fma2(p10, hi, w10[2 * q + 1]);
                    w01[2 * q] = fma2(p01, lo, w01[2 * q]);
                    w01[2 * q + 1] = fma2(p01, hi, w01[2 * q + 1]);
                    w11[2 * q] = fma2(p11, lo, w11[2 * q]);
                    w11[2 * q + 1] = fma2(p11, hi, w11[2 * q + 1]);
                }
            }
        }
    }
    if (inside) {
        const size_t plane = (size_t)NXC * NYC, o = (size_t)jc * NXC + ic;
#pragma unroll
        for (int q = 0; q < NP; ++q) {
            const float2 c00 = unpack2(w00[q]), c10 = unpack2(w10[q]);
            const float2 c01 = unpack2(w01[q]), c11 = unpack2(w11[q]);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int s = 2 * q + h;
                if (s >= nsl) break;
                float *cb = corners + (size_t)(b0 + s) * 4 * plane;
                cb[o] = h ? c00.y : c00.x;
                cb[plane + o] = h ? c10.y : c10.x;
                cb[2 * plane + o] = h ? c01.y : c01.x;
                cb[3 * plane + o] = h ? c11.y : c11.x;
            }
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
    const size_t chunk = batch < 64 ? batch : 64;
    // corner sums of a chunk, then the chunk's sinograms in groups of 8
    return sizeof(float) * chunk * (4 * (size_t)(p->g.nx + 1) * (p->g.ny + 1) +
                                    (size_t)p->g.n_views * p->g.n_cols) +
           sizeof(float) * 16 * (size_t)p->g.n_views * p->g.n_cols + 256;
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
    const float4 *rrec = reinterpret_cast<const float4 *>(p->d_ray_rec);
    cudaStream_t s = (cudaStream_t)stream;
    const size_t plane = (size_t)a.nx * a.ny, slice = (size_t)a.V * a.C;
    const int chunk = batch < 64 ? batch : 64;
    float *corners = static_cast<float *>(work);
    // interleaved sinograms after the corner sums, 16-byte aligned
    const size_t coff = ((4 * (size_t)chunk * (a.nx + 1) * (a.ny + 1) * sizeof(float) + 255) / 256) * 256;
    float *inter = reinterpret_cast<float *>(static_cast<char *>(work) + coff);
    for (int b0 = 0; b0 < batch; b0 += 64) {
        const int nb = batch - b0 < 64 ? batch - b0 : 64;
        const int SB = nb >= 16 && CT_ADJ_MAX_SB >= 16 ? 16 : (nb >= 8 ? 8 : 4);
        const int groups = (nb + SB - 1) / SB;
        const float *sp = sino + b0 * slice;
        const long long work_items = (long long)groups * slice;
        const int ib = (int)((work_items + 255) / 256 < 152 * 16 ? (work_items + 255) / 256 : 152 * 16);
        if (SB == 16)
            interleave_kernel<16><<<ib, 256, 0, s>>>(sp, inter, nb, slice);
        else if (SB == 8)
            interleave_kernel<8><<<ib, 256, 0, s>>>(sp, inter, nb, slice);
        else
            interleave_kernel<4><<<ib, 256, 0, s>>>(sp, inter, nb, slice);
        dim3 grid((a.nx + kCellTile) / kCellTile, (a.ny + kCellTile) / kCellTile, groups);
        auto go = [&](auto kern) {
            kern<<<grid, dim3(32, 8), 0, s>>>(inter, corners, rrec, vcs, a, nb);
        };
        if (CT_ADJ_MAX_SB >= 16 && SB == 16)
            deg == 8 ? go(fp_adjoint_cells_kernel<16, 8>)
                     : deg == 4 ? go(fp_adjoint_cells_kernel<16, 4>) : go(fp_adjoint_cells_kernel<16, 0>);
        else if (SB == 8)
            deg == 8 ? go(fp_adjoint_cells_kernel<8, 8>)
                     : deg == 4 ? go(fp_adjoint_cells_kernel<8, 4>) : go(fp_adjoint_cells_kernel<8, 0>);
        else
            deg == 8 ? go(fp_adjoint_cells_kernel<4, 8>)
                     : deg == 4 ? go(fp_adjoint_cells_kernel<4, 4>) : go(fp_adjoint_cells_kernel<4, 0>);
        fp_adjoint_combine_kernel<<<dim3((a.nx + 31) / 32, (a.ny + 7) / 8, nb),
                                    dim3(32, 8), 0, s>>>(corners, img + b0 * plane, a.nx, a.ny,
                                                         p->fp_weight, nb);
        ct_count_launch(3);
    }
    return (int)cudaGetLastError();
}

}  // namespace ctk
