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
// Tiles of 128 rows x 224 columns, K steps of 16 FP32 (64-byte swizzled
// rows): per step TMA brings the input tile (8 KB) and the two tap tiles
// (14 KB each), three warps split the input tile, and one thread issues 2
// K-slices x 3 tcgen05.mma (M=128, N=224, K=8, kind::tf32).  A ring of four
// such stages (176 KB) lets the copies and the split of later steps run while
// the tensor core works.  Measured per 32 clinical slices (31,488 rows of 888
// channels, CUDA events): one single-stage step at a time 0.389 ms; two
// stages of K 32 0.282 ms; persistent with a double-buffered accumulator
// 0.275 ms; four stages of K 16 0.244 ms (three 0.287, five 0.251; tiles of
// 128 / 96 / 64 columns 0.33 .. 0.53 ms); three splitter warps instead of two
// 0.233 ms.  All forms give identical bits.
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
#ifndef CT_TC2_BN
#define CT_TC2_BN 224
#endif
#ifndef CT_TC2_STAGES
#define CT_TC2_STAGES 4
#endif
#ifndef CT_TC2_BK
#define CT_TC2_BK 16
#endif
constexpr int TC2_BN = CT_TC2_BN;
constexpr int TC2_STAGES = CT_TC2_STAGES;
constexpr int TC2_BK = CT_TC2_BK;  // 32: 128-byte swizzle rows; 16: 64-byte rows
static_assert(TC2_BK == 32 || TC2_BK == 16, "K step of 16 or 32 FP32");
constexpr int TC2_TMEM_COLS = TC2_BN <= 32 ? 32 : TC2_BN <= 64 ? 64 : TC2_BN <= 128 ? 128 : 256;
constexpr unsigned TC2_A_BYTES = TC_BM * TC2_BK * 4;
constexpr unsigned TC2_B_BYTES = TC2_BN * TC2_BK * 4;
constexpr unsigned TC2_STAGE_BYTES = 2 * TC2_A_BYTES + 2 * TC2_B_BYTES;
// past the stages: the barriers
constexpr unsigned TC2_SMEM = 1024 + TC2_STAGES * TC2_STAGE_BYTES + 128;
static_assert(TC2_SMEM <= 227 * 1024, "stages exceed shared memory");

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

// K-major operand with 64-byte swizzle: rows of 64 bytes, 8-row atoms 512
// bytes apart (stride byte offset), descriptor version 1, layout code 4.
__device__ __forceinline__ uint64_t sw64_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                   // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(512 >> 4) << 32;          // stride byte offset
    d |= (uint64_t)1 << 46;                   // descriptor version
    d |= (uint64_t)4 << 61;                   // layout: 64-byte swizzle
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

__device__ __forceinline__ uint64_t tc2_desc(uint32_t saddr) {
    return TC2_BK == 32 ? sw128_desc(saddr) : sw64_desc(saddr);
}

__device__ __forceinline__ float tf32_hi(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// Persistent kernel: one CTA per SM walks tiles blockIdx.x, + gridDim.x, ...
// (N tile fastest, so the CTAs of one row tile run together and read its
// input from DRAM once); the stage ring runs on across tile boundaries, and
// the accumulator is double-buffered in tensor memory (2 x 256 columns) so
// that four epilogue warps drain tile j while the tensor core works on tile
// j+1.  Warps:
//   0, one lane: TMA producer (a stage is refilled once the MMAs that read it
//     have completed, tracked by tcgen05.commit on empty[s]);
//   1, one lane: MMA issuer (waits for the stage's split, and for the
//     epilogue to have drained the accumulator it reuses);
//   2 .. 1+TC_SPLIT: split the input tile in place (A -> A_hi) and into A_lo;
//   the last four: epilogue (warp w reads accumulator lanes 32 (w mod 4) ..,
//     the lanes tcgen05.ld gives a warp).
// Every wait is bounded; on a timeout the roles stop issuing, the MMA lane
// still commits what it issued, the producer waits (bounded) for copies in
// flight, the plan's error flag is raised and the tensor memory is freed.
// Splitter warps (32 clinical slices: 2 / 3 / 4 warps 0.244 / 0.233 / 0.237 ms).
#ifndef CT_TC_SPLIT
#define CT_TC_SPLIT 3
#endif
constexpr int TC_SPLIT = CT_TC_SPLIT;
constexpr int TC3_THREADS = 32 * (2 + TC_SPLIT + 4);

__global__ void __launch_bounds__(TC3_THREADS)
    ramp_tc_kernel(const __grid_constant__ CUtensorMap map_in,
                    const __grid_constant__ CUtensorMap map_bhi,
                    const __grid_constant__ CUtensorMap map_blo, float *__restrict__ out,
                    int rows, int C, int k_tiles, int n_tiles_n, int n_tiles,
                    int *__restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *base = reinterpret_cast<uint8_t *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    auto sA = [&](int s) { return reinterpret_cast<float *>(base + s * TC2_STAGE_BYTES); };
    auto sAlo = [&](int s) { return sA(s) + TC2_A_BYTES / 4; };
    auto sBhi = [&](int s) { return sA(s) + 2 * TC2_A_BYTES / 4; };
    auto sBlo = [&](int s) { return sA(s) + (2 * TC2_A_BYTES + TC2_B_BYTES) / 4; };
    uint64_t *bars = reinterpret_cast<uint64_t *>(base + TC2_STAGES * TC2_STAGE_BYTES);
    uint64_t *full = bars, *split = bars + TC2_STAGES, *empty = bars + 2 * TC2_STAGES;
    uint64_t *acc_full = bars + 3 * TC2_STAGES, *acc_empty = acc_full + 2;
    uint64_t *done = acc_empty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    int *fail = reinterpret_cast<int *>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < TC2_STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&split[s], TC_SPLIT);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&acc_full[a], 1);
            mbar_init(&acc_empty[a], 4);
        }
        mbar_init(done, 1);
        *fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(2 * TC2_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    volatile int *vfail = fail;
    const int my_tiles = blockIdx.x < n_tiles ? (n_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

    if (warp == 0) {
        if (lane == 0) {
            int g = 0;  // K steps issued by this CTA
            for (int j = 0; j < my_tiles && !*vfail; ++j) {
                const int tile = blockIdx.x + j * gridDim.x;
                const int n0 = (tile % n_tiles_n) * TC2_BN, m0 = (tile / n_tiles_n) * TC_BM;
                for (int kt = 0; kt < k_tiles; ++kt, ++g) {
                    const int s = g % TC2_STAGES;
                    const uint32_t u = g / TC2_STAGES;
                    if (g >= TC2_STAGES && !mbar_wait(&empty[s], (u - 1) & 1)) *vfail = 1;
                    if (*vfail) break;
                    mbar_expect_tx(&full[s], TC2_A_BYTES + 2 * TC2_B_BYTES);
                    tma_load_2d(sA(s), &map_in, kt * TC2_BK, m0, &full[s]);
                    tma_load_2d(sBhi(s), &map_bhi, kt * TC2_BK, n0, &full[s]);
                    tma_load_2d(sBlo(s), &map_blo, kt * TC2_BK, n0, &full[s]);
                }
            }
            if (*vfail) {
                // copies still in flight land before the CTA gives up its memory
                for (int q = g > TC2_STAGES ? g - TC2_STAGES : 0; q < g; ++q)
                    mbar_wait(&full[q % TC2_STAGES], (q / TC2_STAGES) & 1);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = tf32_idesc(TC_BM, TC2_BN);
            int g = 0;
            for (int j = 0; j < my_tiles && !*vfail; ++j) {
                const int a = j & 1;
                if (j >= 2 && !mbar_wait(&acc_empty[a], ((j >> 1) - 1) & 1)) {
                    *vfail = 1;
                    break;
                }
                const uint32_t d = tmem + (uint32_t)(a * TC2_TMEM_COLS);
                for (int kt = 0; kt < k_tiles; ++kt, ++g) {
                    const int s = g % TC2_STAGES;
                    const uint32_t u = g / TC2_STAGES;
                    if (!mbar_wait(&split[s], u & 1)) *vfail = 1;
                    if (*vfail) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t ahi = smem_u32(sA(s)), alo = smem_u32(sAlo(s));
                    const uint32_t bhi = smem_u32(sBhi(s)), blo = smem_u32(sBlo(s));
#pragma unroll
                    for (int q = 0; q < TC2_BK / 8; ++q) {
                        const uint32_t off = q * 32;  // 8 TF32 = 32 bytes along K
                        const uint32_t acc0 = (kt > 0 || q > 0) ? 1u : 0u;
                        mma_tf32(d, tc2_desc(ahi + off), tc2_desc(bhi + off), idesc, acc0);
                        mma_tf32(d, tc2_desc(ahi + off), tc2_desc(blo + off), idesc, 1u);
                        mma_tf32(d, tc2_desc(alo + off), tc2_desc(bhi + off), idesc, 1u);
                    }
                    mma_commit(&empty[s]);
                }
                if (*vfail) break;
                mma_commit(&acc_full[a]);
            }
            // completes once every MMA issued above has
            mma_commit(done);
        }
    } else if (warp < 2 + TC_SPLIT) {
        // splitters: 32 TC_SPLIT threads, each stage's float4 in place
        const int t = tid - 64;
        int g = 0;
        for (int j = 0; j < my_tiles; ++j) {
            bool stop = false;
            for (int kt = 0; kt < k_tiles; ++kt, ++g) {
                const int s = g % TC2_STAGES;
                const uint32_t u = g / TC2_STAGES;
                const bool ok = mbar_wait(&full[s], u & 1);
                if (!ok) *vfail = 1;
                stop = __any_sync(0xffffffffu, !ok || *vfail);  // warp-uniform
                if (stop) break;
                float4 *a = reinterpret_cast<float4 *>(sA(s));
                float4 *lo = reinterpret_cast<float4 *>(sAlo(s));
#pragma unroll 4
                for (int q = t; q < (int)(TC2_A_BYTES / 16); q += 32 * TC_SPLIT) {
                    const float4 x = a[q];
                    float4 h, l;
                    h.x = tf32_hi(x.x); l.x = x.x - h.x;
                    h.y = tf32_hi(x.y); l.y = x.y - h.y;
                    h.z = tf32_hi(x.z); l.z = x.z - h.z;
                    h.w = tf32_hi(x.w); l.w = x.w - h.w;
                    a[q] = h;
                    lo[q] = l;
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0)
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                                     smem_u32(&split[s]))
                                 : "memory");
            }
            if (stop) break;
        }
    } else {
        // epilogue warps: accumulator lanes 32 (warp mod 4) ..
        const int q4 = warp & 3;
        for (int j = 0; j < my_tiles; ++j) {
            const int a = j & 1;
            const bool ok = mbar_wait(&acc_full[a], (j >> 1) & 1);
            if (!ok) *vfail = 1;
            if (__any_sync(0xffffffffu, !ok || *vfail)) break;  // warp-uniform
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int tile = blockIdx.x + j * gridDim.x;
            const int n0 = (tile % n_tiles_n) * TC2_BN, m0 = (tile / n_tiles_n) * TC_BM;
            const int row = m0 + 32 * q4 + lane;
            for (int c0 = 0; c0 < TC2_BN; c0 += 32) {
                uint32_t r[32];
                const uint32_t taddr =
                    tmem + ((uint32_t)(32 * q4) << 16) + (uint32_t)(a * TC2_TMEM_COLS + c0);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,"
                    "%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,"
                    "%30,%31}, [%32];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                      "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                      "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
                      "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                      "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]),
                      "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (row < rows) {
                    float *o = out + (size_t)row * C + n0 + c0;
                    const int lim = min(32, C - (n0 + c0));
                    if (lim == 32) {
                        float4 *o4 = reinterpret_cast<float4 *>(o);
#pragma unroll
                        for (int i = 0; i < 8; ++i)
                            o4[i] = make_float4(__uint_as_float(r[4 * i]),
                                                __uint_as_float(r[4 * i + 1]),
                                                __uint_as_float(r[4 * i + 2]),
                                                __uint_as_float(r[4 * i + 3]));
                    } else {
#pragma unroll
                        for (int i = 0; i < 32; ++i)
                            if (i < lim) o[i] = __uint_as_float(r[i]);
                    }
                }
            }
            // this warp is done reading accumulator a
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                                 smem_u32(&acc_empty[a]))
                             : "memory");
        }
    }
    __syncwarp();
    // every MMA has completed before the tensor memory is released
    const bool fin = mbar_wait(done, 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool good = __syncthreads_and(fin && !*vfail);
    if (!good && tid == 0) atomicExch(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(2 * TC2_TMEM_COLS)
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

// 2-D FP32 row-major [outer][inner] map with a (box_k x box_rows) box, swizzled
// by the box row (128 or 64 bytes).
bool make_map(CUtensorMap *m, const void *ptr, uint64_t inner, uint64_t outer,
              uint64_t row_bytes, uint32_t box_rows, uint32_t box_k) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {inner, outer};
    const cuuint64_t strides[1] = {row_bytes};
    const cuuint32_t box[2] = {box_k, box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void *>(ptr), dims, strides, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              box_k == 32 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
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

int tc_padded(int C) { return (C + TC2_BN - 1) / TC2_BN * TC2_BN; }

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
    constexpr int bk = TC2_BK;
    CUtensorMap m_in, m_hi, m_lo;
    if (!make_map(&m_in, in, (uint64_t)C, (uint64_t)rows, (uint64_t)C * 4, TC_BM, bk) ||
        !make_map(&m_hi, p->d_tc_hi, (uint64_t)P, (uint64_t)P, (uint64_t)P * 4, TC2_BN, bk) ||
        !make_map(&m_lo, p->d_tc_lo, (uint64_t)P, (uint64_t)P, (uint64_t)P * 4, TC2_BN, bk))
        return (int)cudaErrorInvalidValue;
    const int k_tiles = (C + bk - 1) / bk;
    cudaError_t e = cudaFuncSetAttribute(ramp_tc_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, TC2_SMEM);
    if (e != cudaSuccess) return (int)e;
    int dev = 0, sms = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return (int)e;
    const int nn = P / TC2_BN, nt = nn * ((rows + TC_BM - 1) / TC_BM);
    const int ctas = nt < sms ? nt : sms;
    ramp_tc_kernel<<<ctas, TC3_THREADS, TC2_SMEM, (cudaStream_t)stream>>>(
        m_in, m_hi, m_lo, out, rows, C, k_tiles, nn, nt, p->d_err);
    ct_count_launch();
    return (int)cudaGetLastError();
}

}  // namespace ctk
