// Ramp filter as a Toeplitz GEMM on the 5th-generation tensor cores.
//
// out[m][i] = sum_j in[m][j] h[i - j] is OUT = IN * T with T[j][i] = h[i - j];
// T is symmetric, so the K-major B operand (B[n][k] = T[k][n] = h[n - k]) is
// T itself.  FP32 operands are split for the TF32 tensor path: x = x_hi +
// x_lo with x_hi rounded to TF32 and x_lo = x - x_hi (which the tensor core
// reads truncated to TF32), and D = A_hi B_hi + A_hi B_lo + A_lo B_hi is
// accumulated in FP32 in tensor memory (the dropped A_lo B_lo term and the
// truncation of the low parts are ~2^-21 relative per product).  The taps'
// split is built once per plan; the input's split is made in shared memory.
//
// One CTA computes a 128-row x 224-column tile: per K step of 32 it loads an
// input tile (128 x 32 FP32) and the two tap tiles (224 x 32 each) with TMA
// (128-byte swizzle), splits the input tile, and one thread issues 4 K-slices
// x 3 tcgen05.mma (M=128, N=224, K=8, kind::tf32) into a 128 x 256-column
// TMEM accumulator; four warps then read the accumulator with tcgen05.ld.
// All mbarrier waits are bounded: on a timeout the CTA raises the plan's
// error flag, releases its tensor memory and exits.
#include <cuda.h>

#include <cstring>

#include "common.cuh"
#include "tma.cuh"

namespace ctk {
namespace {

using tma::mbar_expect_tx;
using tma::mbar_init;
using tma::mbar_wait;
using tma::smem_u32;

constexpr int TC_BM = 128;
constexpr int TC_BN = 224;
constexpr int TC_BK = 32;           // FP32 elements per 128-byte swizzle row
constexpr int TC_TMEM_COLS = 256;   // power of two >= TC_BN
constexpr int TC_THREADS = 128;
constexpr unsigned TC_A_BYTES = TC_BM * TC_BK * 4;  // 16 KB
constexpr unsigned TC_B_BYTES = TC_BN * TC_BK * 4;  // 28 KB
constexpr unsigned TC_SMEM = 1024 /*align slack*/ + 3 * TC_A_BYTES + 2 * TC_B_BYTES + 64;

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// K-major operand with 128-byte swizzle: rows of 128 bytes, 8-row atoms
// 1024 bytes apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                   // leading byte offset (unused for SW128 K-major)
    d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset
    d |= (uint64_t)1 << 46;                   // descriptor version
    d |= (uint64_t)2 << 61;                   // layout: 128-byte swizzle
    return d;
}

// kind::tf32 instruction descriptor: D FP32, A/B TF32, both K-major, M, N.
__host__ __device__ constexpr uint32_t tf32_idesc(int M, int N) {
    return (1u << 4)                       // D format F32
           | (2u << 7) | (2u << 10)        // A, B format TF32
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ float tf32_hi(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

__global__ void __launch_bounds__(TC_THREADS)
    ramp_tc_kernel(const __grid_constant__ CUtensorMap map_in,
                   const __grid_constant__ CUtensorMap map_bhi,
                   const __grid_constant__ CUtensorMap map_blo, float *__restrict__ out, int rows,
                   int C, int k_tiles, int *__restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte aligned buffers (the 128-byte swizzle atom)
    uint8_t *base = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    float *sA = reinterpret_cast<float *>(base);
    float *sAhi = reinterpret_cast<float *>(base + TC_A_BYTES);
    float *sAlo = reinterpret_cast<float *>(base + 2 * TC_A_BYTES);
    float *sBhi = reinterpret_cast<float *>(base + 3 * TC_A_BYTES);
    float *sBlo = reinterpret_cast<float *>(base + 3 * TC_A_BYTES + TC_B_BYTES);
    uint64_t *bars = reinterpret_cast<uint64_t *>(base + 3 * TC_A_BYTES + 2 * TC_B_BYTES);
    uint64_t *full_bar = bars, *mma_bar = bars + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2);

    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.x * TC_BM;
    const int n0 = blockIdx.y * TC_BN;

    if (tid == 0) {
        mbar_init(full_bar, 1);
        mbar_init(mma_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = tf32_idesc(TC_BM, TC_BN);

    bool ok = true;
    for (int kt = 0; kt < k_tiles && ok; ++kt) {
        const uint32_t phase = kt & 1;
        if (tid == 0) {
            mbar_expect_tx(full_bar, TC_A_BYTES + 2 * TC_B_BYTES);
            tma_load_2d(sA, &map_in, kt * TC_BK, m0, full_bar);
            tma_load_2d(sBhi, &map_bhi, kt * TC_BK, n0, full_bar);
            tma_load_2d(sBlo, &map_blo, kt * TC_BK, n0, full_bar);
        }
        ok = mbar_wait(full_bar, phase);
        // split the input tile in place of layout (elementwise, swizzle kept)
        if (ok) {
            const float4 *src = reinterpret_cast<const float4 *>(sA);
            float4 *dhi = reinterpret_cast<float4 *>(sAhi);
            float4 *dlo = reinterpret_cast<float4 *>(sAlo);
            for (int q = tid; q < (int)(TC_A_BYTES / 16); q += TC_THREADS) {
                const float4 x = src[q];
                float4 h, l;
                h.x = tf32_hi(x.x); l.x = x.x - h.x;
                h.y = tf32_hi(x.y); l.y = x.y - h.y;
                h.z = tf32_hi(x.z); l.z = x.z - h.z;
                h.w = tf32_hi(x.w); l.w = x.w - h.w;
                dhi[q] = h;
                dlo[q] = l;
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        ok = __syncthreads_and(ok);
        if (!ok) break;
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t ahi = smem_u32(sAhi), alo = smem_u32(sAlo);
            const uint32_t bhi = smem_u32(sBhi), blo = smem_u32(sBlo);
#pragma unroll
            for (int s = 0; s < TC_BK / 8; ++s) {
                const uint32_t off = s * 32;  // 8 TF32 = 32 bytes along K
                const uint32_t acc0 = (kt > 0 || s > 0) ? 1u : 0u;
                mma_tf32(tmem, sw128_desc(ahi + off), sw128_desc(bhi + off), idesc, acc0);
                mma_tf32(tmem, sw128_desc(ahi + off), sw128_desc(blo + off), idesc, 1u);
                mma_tf32(tmem, sw128_desc(alo + off), sw128_desc(bhi + off), idesc, 1u);
            }
            mma_commit(mma_bar);
        }
        // the MMAs must finish reading shared memory before the next loads
        ok = mbar_wait(mma_bar, phase);
        ok = __syncthreads_and(ok);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        // epilogue: warp w reads accumulator lanes 32w..32w+31 (rows m0+32w+lane)
        const int row = m0 + 32 * warp + (tid & 31);
        for (int c0 = 0; c0 < TC_BN; c0 += 32) {
            uint32_t r[32];
            const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,"
                "%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31},"
                " [%32];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                  "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                  "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]),
                  "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                  "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
                  "=r"(r[30]), "=r"(r[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < rows) {
                float *o = out + (size_t)row * C + n0 + c0;
                const int lim = min(32, C - (n0 + c0));
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    if (j < lim) o[j] = __uint_as_float(r[j]);
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TC_TMEM_COLS)
                     : "memory");
    }
}

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// 2-D FP32 row-major [outer][inner] map with a (32 x box_rows) box, 128B swizzle.
bool make_map(CUtensorMap *m, const void *ptr, uint64_t inner, uint64_t outer,
              uint64_t row_bytes, uint32_t box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {inner, outer};
    const cuuint64_t strides[1] = {row_bytes};
    const cuuint32_t box[2] = {TC_BK, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(ptr), dims, strides, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Exercises the timeout path of mbar_wait: one thread waits on a barrier
// that nothing arrives at, gives up after budget_ns and raises `err`, as the
// filter kernel does.
__global__ void wait_selftest_kernel(int *err, unsigned long long budget_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait(&bar, 0, budget_ns)) atomicExch(err, 1);
}

}  // namespace

int wait_selftest(const ct_plan *p, unsigned long long budget_ns, void *stream) {
    wait_selftest_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(p->d_err, budget_ns);
    ct_count_launch();
    return (int)cudaGetLastError();
}

int tc_padded(int C) { return (C + TC_BN - 1) / TC_BN * TC_BN; }

bool ramp_tc_supported(int C) {
    // TMA rows must be 16-byte multiples; the padded tap matrix must stay modest
    return C % 4 == 0 && C >= 32 && tc_padded(C) <= 4096 && encode_fn() != nullptr;
}

// Host: the taps' TF32 split as [Np][Kp] K-major matrices B[n][k] = h[n - k]
// (zero outside the C x C block), Np = Kp = tc_padded(C).
void build_tc_taps(const float *taps, int C, std::vector<float> &hi, std::vector<float> &lo) {
    const int P = tc_padded(C);
    hi.assign((size_t)P * P, 0.0f);
    lo.assign((size_t)P * P, 0.0f);
    for (int n = 0; n < C; ++n)
        for (int k = 0; k < C; ++k) {
            const float h = taps[n - k + C - 1];
            uint32_t u;
            std::memcpy(&u, &h, 4);
            u = (u + 0x1000u) & 0xFFFFE000u;
            float hh;
            std::memcpy(&hh, &u, 4);
            hi[(size_t)n * P + k] = hh;
            lo[(size_t)n * P + k] = h - hh;
        }
}

int ramp_filter_tc(const ct_plan *p, const float *in, float *out, int rows, void *stream) {
    const int C = p->g.n_cols;
    const int P = tc_padded(C);
    CUtensorMap m_in, m_hi, m_lo;
    if (!make_map(&m_in, in, (uint64_t)C, (uint64_t)rows, (uint64_t)C * 4, TC_BM) ||
        !make_map(&m_hi, p->d_tc_hi, (uint64_t)P, (uint64_t)P, (uint64_t)P * 4, TC_BN) ||
        !make_map(&m_lo, p->d_tc_lo, (uint64_t)P, (uint64_t)P, (uint64_t)P * 4, TC_BN))
        return (int)cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(ramp_tc_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    if (e != cudaSuccess) return (int)e;
    const int k_tiles = (C + TC_BK - 1) / TC_BK;
    dim3 grid((rows + TC_BM - 1) / TC_BM, P / TC_BN, 1);
    ramp_tc_kernel<<<grid, TC_THREADS, TC_SMEM, (cudaStream_t)stream>>>(m_in, m_hi, m_lo, out,
                                                                         rows, C, k_tiles,
                                                                         p->d_err);
    ct_count_launch();
    return (int)cudaGetLastError();
}

}  // namespace ctk
