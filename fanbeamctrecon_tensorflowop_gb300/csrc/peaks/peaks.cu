// Peak microbenchmarks for the benchmark's roofline denominators.
//
// The interpolation kernels of this library (the forward projector's quad
// gathers, the backprojectors' tap loads) are bound by the L1 data path, not
// by HBM or the tensor pipe, so their roofline needs a measured L1 load peak:
//   - ctpk_l1_load: every thread streams 16-byte read-only loads (the same
//     ld.global.nc.v4 the kernels issue) over a 32 KiB buffer that stays
//     resident in each SM's L1; adjacent lanes read adjacent 16 bytes, so a
//     warp's load is four full 128-byte lines, the best case of the L1 path.
//   - ctpk_l1_load_v8: the same with 32-byte loads (ld.global.nc.v8.f32,
//     sm_100 and later), a warp's load eight full lines.
//   - ctpk_fma: independent FP32 FMA chains, scalar (fma.rn.f32) or packed
//     (fma.rn.f32x2), the FP32 pipe's peak.
// Both time one launch with CUDA events on the legacy default stream after a
// warm-up launch, and return the rate and the launch's milliseconds.  This
// file is built into its own library (libctpeaks.so); the operators never
// call it.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

constexpr int kL1Bytes = 32 * 1024;  // per-SM working set: well inside L1
constexpr int kL1Vec = kL1Bytes / 16;

__device__ __forceinline__ float4 ld_nc(const float4 *p) {
    float4 v;
    asm volatile("ld.global.nc.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p));
    return v;
}

// 32 bytes at p (32-byte aligned): two float4 halves.
__device__ __forceinline__ void ld_nc8(const float4 *p, float4 &a, float4 &b) {
    asm volatile("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z),
                   "=f"(b.w)
                 : "l"(p));
}

// Each iteration a warp reads 8 x 512 contiguous bytes; the window moves by
// 32 float4 per iteration, so no load repeats an address of the previous
// iteration (the volatile loads are never merged or hoisted either).
__global__ void __launch_bounds__(512) l1_load_kernel(const float4 *__restrict__ buf, int iters,
                                                      float *__restrict__ sink) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    int idx = threadIdx.x;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float4 v = ld_nc(buf + ((idx + k * 512) & (kL1Vec - 1)));
            acc.x += v.x;
            acc.y += v.y;
            acc.z += v.z;
            acc.w += v.w;
        }
        idx = (idx + 32) & (kL1Vec - 1);
    }
    // the buffer holds zeros: this store never happens, but the compiler
    // cannot know it, so every load stays
    if (acc.x + acc.y + acc.z + acc.w != 0.0f) sink[blockIdx.x * blockDim.x + threadIdx.x] = acc.x;
}

// 32-byte loads: each iteration a warp reads 8 x 1024 contiguous bytes (pairs
// of float4), the window moving by 32 pairs per iteration.
__global__ void __launch_bounds__(512) l1_load8_kernel(const float4 *__restrict__ buf, int iters,
                                                       float *__restrict__ sink) {
    constexpr int kPairs = kL1Vec / 2;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    int idx = threadIdx.x;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            float4 a, b;
            ld_nc8(buf + 2 * ((idx + k * 512) & (kPairs - 1)), a, b);
            acc.x += a.x + b.x;
            acc.y += a.y + b.y;
            acc.z += a.z + b.z;
            acc.w += a.w + b.w;
        }
        idx = (idx + 32) & (kPairs - 1);
    }
    if (acc.x + acc.y + acc.z + acc.w != 0.0f) sink[blockIdx.x * blockDim.x + threadIdx.x] = acc.x;
}

template <bool PACKED>
__global__ void __launch_bounds__(256) fma_kernel(float seed, int iters, float *__restrict__ sink) {
    constexpr int kChains = 8;
    float a[kChains], b[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) {
        a[c] = seed + c + threadIdx.x;
        b[c] = seed - c;
    }
    const float m = 0.999999f, d = 1e-7f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
#pragma unroll
            for (int c = 0; c < kChains; ++c) {
                if constexpr (PACKED) {
                    unsigned long long x, mm, dd, r;
                    asm("mov.b64 %0, {%1, %2};" : "=l"(x) : "f"(a[c]), "f"(b[c]));
                    asm("mov.b64 %0, {%1, %1};" : "=l"(mm) : "f"(m));
                    asm("mov.b64 %0, {%1, %1};" : "=l"(dd) : "f"(d));
                    asm volatile("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(x), "l"(mm), "l"(dd));
                    asm("mov.b64 {%0, %1}, %2;" : "=f"(a[c]), "=f"(b[c]) : "l"(r));
                } else {
                    a[c] = fmaf(a[c], m, d);
                    b[c] = fmaf(b[c], m, d);
                }
            }
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += a[c] + b[c];
    if (s == 1.2345f) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int sm_count(int *out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaDeviceGetAttribute(out, cudaDevAttrMultiProcessorCount, dev);
}

template <class F>
int time_launch(F &&launch, float *ms) {
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (e != cudaSuccess) return (int)e;
    if ((e = cudaEventCreate(&e1)) != cudaSuccess) {
        cudaEventDestroy(e0);
        return (int)e;
    }
    launch();  // warm-up
    cudaEventRecord(e0, 0);
    launch();
    cudaEventRecord(e1, 0);
    e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return (int)e;
}

int l1_load(int bytes_per_load, int blocks_per_sm, int iters, double *gbs, double *ms_out) {
    int sms = 0;
    int rc = sm_count(&sms);
    if (rc) return rc;
    float4 *buf = nullptr;
    float *sink = nullptr;
    const int blocks = sms * blocks_per_sm;
    cudaError_t e = cudaMalloc(&buf, kL1Bytes);
    if (e != cudaSuccess) return (int)e;
    if ((e = cudaMalloc(&sink, sizeof(float) * (size_t)blocks * 512)) != cudaSuccess) {
        cudaFree(buf);
        return (int)e;
    }
    cudaMemset(buf, 0, kL1Bytes);
    float ms = 0.0f;
    rc = time_launch(
        [&] {
            if (bytes_per_load == 32)
                l1_load8_kernel<<<blocks, 512>>>(buf, iters, sink);
            else
                l1_load_kernel<<<blocks, 512>>>(buf, iters, sink);
        },
        &ms);
    cudaFree(buf);
    cudaFree(sink);
    if (rc) return rc;
    const double bytes = (double)bytes_per_load * 8.0 * (double)iters * 512.0 * (double)blocks;
    *gbs = bytes / ((double)ms * 1e-3) / 1e9;
    *ms_out = ms;
    return 0;
}

}  // namespace

extern "C" {

// Number of SMs of the current device.
int ctpk_sm_count(int *out) { return sm_count(out); }

// L1 load bandwidth of the current device: bytes loaded by all threads /
// launch time, in GB/s (1e9 B/s).  blocks_per_sm blocks of 512 threads per SM.
int ctpk_l1_load(int blocks_per_sm, int iters, double *gbs, double *ms_out) {
    return l1_load(16, blocks_per_sm, iters, gbs, ms_out);
}

// The same with 32-byte loads.
int ctpk_l1_load_v8(int blocks_per_sm, int iters, double *gbs, double *ms_out) {
    return l1_load(32, blocks_per_sm, iters, gbs, ms_out);
}

// FP32 FMA throughput of the current device in TFLOP/s (an FMA = 2 FLOP);
// packed != 0 issues fma.rn.f32x2 (two FMAs per instruction).
int ctpk_fma(int packed, int blocks_per_sm, int iters, double *tflops, double *ms_out) {
    int sms = 0;
    int rc = sm_count(&sms);
    if (rc) return rc;
    float *sink = nullptr;
    const int blocks = sms * blocks_per_sm;
    cudaError_t e = cudaMalloc(&sink, sizeof(float) * (size_t)blocks * 256);
    if (e != cudaSuccess) return (int)e;
    float ms = 0.0f;
    rc = time_launch(
        [&] {
            if (packed)
                fma_kernel<true><<<blocks, 256>>>(1.0f, iters, sink);
            else
                fma_kernel<false><<<blocks, 256>>>(1.0f, iters, sink);
        },
        &ms);
    cudaFree(sink);
    if (rc) return rc;
    // 16 unrolled x 8 chains x 2 FMAs (a and b) per iteration and thread
    const double fmas = 16.0 * 8.0 * 2.0 * (double)iters * 256.0 * (double)blocks;
    *tflops = 2.0 * fmas / ((double)ms * 1e-3) / 1e12;
    *ms_out = ms;
    return 0;
}

}  // extern "C"
