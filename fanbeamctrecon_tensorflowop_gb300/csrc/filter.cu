// Ramp filter of every detector row: q[i] = sum_j h[i - j] p[j], i, j in
// [0, C) -- the middle C samples of ippsConv_32f's full linear convolution of
// the row with the 2C-1 taps (FBP/transform.cu:166-174,
// FDK/GPURecon_GPU.cu:207-215), which ran serially on the host CPU in the
// reference.  Direct FP32 form: a block stages kRows rows and the taps in
// shared memory; each thread produces outputs of all kRows rows so a tap read
// is reused kRows times.  For the Ram-Lak window the even taps (n != 0) are
// exactly zero and are skipped.
#include "common.cuh"

namespace ctk {
namespace {

constexpr int kRows = 8;
constexpr int kThreads = 256;

template <bool ODD_ONLY>
__global__ void __launch_bounds__(kThreads)
    ramp_direct_kernel(const float *__restrict__ in, float *__restrict__ out,
                       const float *__restrict__ taps, int C, int rows) {
    extern __shared__ float sm[];
    float *st = sm;                      // [2C-1] taps (index n + C - 1)
    float *sp = sm + (2 * C - 1 + 3) / 4 * 4;  // [kRows][C]
    const int r0 = blockIdx.x * kRows;
    const int nr = min(kRows, rows - r0);
    for (int k = threadIdx.x; k < 2 * C - 1; k += kThreads) st[k] = __ldg(taps + k);
    for (int k = threadIdx.x; k < kRows * C; k += kThreads) {
        const int rr = k / C;
        sp[k] = rr < nr ? __ldg(in + (size_t)(r0 + rr) * C + (k - rr * C)) : 0.0f;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < C; i += kThreads) {
        float acc[kRows];
        const float *ti = st + i + C - 1;  // ti[-j] = h[i - j]
        if (ODD_ONLY) {
            const float h0 = st[C - 1];  // h[0]
#pragma unroll
            for (int r = 0; r < kRows; ++r) acc[r] = h0 * sp[r * C + i];
            for (int j = (i & 1) ^ 1; j < C; j += 2) {
                const float h = ti[-j];
#pragma unroll
                for (int r = 0; r < kRows; ++r) acc[r] = fmaf(h, sp[r * C + j], acc[r]);
            }
        } else {
#pragma unroll
            for (int r = 0; r < kRows; ++r) acc[r] = 0.0f;
            for (int j = 0; j < C; ++j) {
                const float h = ti[-j];
#pragma unroll
                for (int r = 0; r < kRows; ++r) acc[r] = fmaf(h, sp[r * C + j], acc[r]);
            }
        }
#pragma unroll
        for (int r = 0; r < kRows; ++r)
            if (r < nr) out[(size_t)(r0 + r) * C + i] = acc[r];
    }
}

// Elementwise pre-weights over [batch][V][rows][C]: wv[v][c] (short scan)
// and wr[r][c] (cosine), either may be NULL.
__global__ void __launch_bounds__(256)
    preweight_kernel(const float *__restrict__ in, float *__restrict__ out,
                     const float *__restrict__ wv, const float *__restrict__ wr, long long total,
                     int C, int rows, int V) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
        const int i = (int)(e % C);
        const long long vr = e / C;
        const int r = (int)(vr % rows);
        const int v = (int)((vr / rows) % V);
        float w = 1.0f;
        if (wv) w = __ldg(wv + (size_t)v * C + i);
        if (wr) w *= __ldg(wr + (size_t)r * C + i);
        out[e] = in[e] * w;
    }
}

}  // namespace

int apply_preweight(const ct_plan *p, const float *in, float *out, int batch, void *stream) {
    const long long total = (long long)batch * p->g.n_views * p->n_rows * p->g.n_cols;
    const long long blocks = (total + 255) / 256;
    preweight_kernel<<<(int)(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0,
                       (cudaStream_t)stream>>>(in, out, p->d_parker, p->d_cosw, total,
                                               p->g.n_cols, p->n_rows, p->g.n_views);
    ct_count_launch();
    return (int)cudaGetLastError();
}

size_t ramp_direct_smem(int C) { return sizeof(float) * ((2 * C - 1 + 3) / 4 * 4 + kRows * C); }

int ramp_filter(const ct_plan *p, const float *in, float *out, int rows, void *stream) {
    if (p->filter_algo == CT_FILTER_TOEPLITZ_TC) return ramp_filter_tc(p, in, out, rows, stream);
    const int C = p->g.n_cols;
    const size_t smem = ramp_direct_smem(C);
    const bool odd_only = p->opts.filter_window == CT_WINDOW_RAMLAK;
    cudaError_t e;
    if (odd_only)
        e = cudaFuncSetAttribute(ramp_direct_kernel<true>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    else
        e = cudaFuncSetAttribute(ramp_direct_kernel<false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    const int blocks = (rows + kRows - 1) / kRows;
    if (blocks == 0) return 0;
    if (odd_only)
        ramp_direct_kernel<true><<<blocks, kThreads, smem, (cudaStream_t)stream>>>(
            in, out, p->d_taps, C, rows);
    else
        ramp_direct_kernel<false><<<blocks, kThreads, smem, (cudaStream_t)stream>>>(
            in, out, p->d_taps, C, rows);
    ct_count_launch();
    return (int)cudaGetLastError();
}

}  // namespace ctk
