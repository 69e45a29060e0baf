// Uneven batches: one call runs FP, BP, FBP and FBP-adjoint work on up to
// CT_BATCH_MAX_ITEMS slices whose geometries (image size, views, channels)
// differ, with FP32 or BF16 storage and FP32 arithmetic throughout.
//
//   1. one launch builds the quad images of every FP item;
//   2. one persistent FP launch: warps pull (item, view, 32-channel) units
//      until all items' rays are projected (fp_warp, fp_body.cuh);
//   3. per item: BF16 inputs are widened, FBP items are ramp-filtered with
//      their plan's filter (the tensor-core Toeplitz GEMM where it applies),
//      FBP-adjoint items run the weighted-BP transpose and the filter;
//   4. one persistent BP launch: blocks pull (item, 32x32 tile) units of every
//      BP / FBP item (bp_tile, bp_body.cuh);
//   5. one launch narrows the FBP-adjoint results that are stored as BF16.
// Slices that share a plan, an operator and a storage type (a "slice group"
// of two or more items) take the plan's own multi-slice kernels instead,
// which walk up to 16 slices at once: their inputs are gathered (and
// widened) into contiguous workspace, and their results scattered (and
// narrowed) to the items' buffers.  The persistent launches take the rest.
// Item descriptors travel as __grid_constant__ kernel parameters, so a call
// needs no host-to-device copy and can be captured in a CUDA graph.
//
// The two persistent launches take their shape from a ct_batch_config: grid
// size (blocks per SM), fixed-stride or dynamic (atomic counter, largest item
// first) distribution of units, and the BP tile height.  batch_tune times the
// candidates on the caller's batch and keeps the fastest per batch shape.
#include <cuda_bf16.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "bp_body.cuh"
#include "fp_body.cuh"

namespace ctk {
namespace {

constexpr int kMax = CT_BATCH_MAX_ITEMS;

struct QuadItem {
    const void *img;
    float4 *quads;
    int nx, ny, bf16;
    int blocks_x, blocks_y;  // of this item's 32 x 8 quad blocks
    int unit0;               // first block index of this item
};
struct QuadBatch {
    int n, total;
    QuadItem it[kMax];
};

struct FpItem {
    const float4 *quads;
    void *out;
    const float4 *ray;
    const int *nsamp;
    int V, C, wpv, nx, max_iter, out_bf16, unit0;
    float w;
};
struct FpBatch {
    int n, total;
    FpItem it[kMax];
};

struct BpItem {
    const float *sino;
    void *img;
    const float2 *view_cs;
    BpArgs a;
    int tiles_x, unit0, out_bf16, weighted, use_atanf;
};
struct BpBatch {
    int n, total;
    BpItem it[kMax];
};

enum ConvMode { kWiden = 0, kNarrow = 1, kCopy = 2 };  // BF16 -> F32, F32 -> BF16, F32
struct ConvItem {
    const void *src;
    void *dst;
    long long count;
    int mode;
};
struct ConvBatch {
    int n;
    ConvItem it[kMax];
};

template <typename Item>
__device__ __forceinline__ int find_item(const Item *it, int n, int unit) {
    int i = 0;
    while (i + 1 < n && it[i + 1].unit0 <= unit) ++i;
    return i;
}

__global__ void __launch_bounds__(256) quads_batch_kernel(const __grid_constant__ QuadBatch P) {
    for (int u = blockIdx.x; u < P.total; u += gridDim.x) {
        const QuadItem &it = P.it[find_item(P.it, P.n, u)];
        const int local = u - it.unit0;
        const int per_layout = it.blocks_x * it.blocks_y;
        const int layout = local / per_layout, rem = local - layout * per_layout;
        const int by = rem / it.blocks_x, bx = rem - by * it.blocks_x;
        const int Q = it.nx + 1;
        const int qi = bx * 32 + threadIdx.x, qj = by * 8 + threadIdx.y;
        if (qi >= Q || qj >= Q) continue;
        float4 *dst = it.quads + (size_t)layout * Q * Q + (size_t)qj * Q + qi;
        if (it.bf16)
            build_quad(static_cast<const __nv_bfloat16 *>(it.img), dst, it.nx, it.ny, layout, qi,
                       qj);
        else
            build_quad(static_cast<const float *>(it.img), dst, it.nx, it.ny, layout, qi, qj);
    }
}

// Next unit of a warp: fixed stride, or the next value of the launch's
// atomic counter (units are ordered largest item first in that mode).
template <bool DYN>
__device__ __forceinline__ int next_warp_unit(int *ctr, int prev, int first, int step) {
    if constexpr (DYN) {
        int u = 0;
        if ((threadIdx.x & 31) == 0) u = atomicAdd(ctr, 1);
        return __shfl_sync(0xffffffffu, u, 0);
    } else {
        return prev < 0 ? first : prev + step;
    }
}

template <bool DYN>
__global__ void __launch_bounds__(256)
    fp_batch_kernel(const __grid_constant__ FpBatch P, int *ctr) {
    const int step = gridDim.x * 8;
    const int first = blockIdx.x * 8 + (threadIdx.x >> 5);
    for (int gw = next_warp_unit<DYN>(ctr, -1, first, step); gw < P.total;
         gw = next_warp_unit<DYN>(ctr, gw, first, step)) {
        const FpItem &it = P.it[find_item(P.it, P.n, gw)];  // warp-uniform
        // channel-group-major within the item: consecutive units are adjacent
        // views of one channel group, whose rays cross the same cells
        const int u = gw - it.unit0, cg = u / it.V;
        const int unit = (u - cg * it.V) * it.wpv + cg;
        if (it.out_bf16)
            fp_warp<1, __nv_bfloat16>(it.quads, 0, static_cast<__nv_bfloat16 *>(it.out), 0,
                                      it.ray, it.nsamp, it.V, it.C, it.wpv, it.nx, it.w, 1,
                                      it.max_iter, unit);
        else
            fp_warp<1, float>(it.quads, 0, static_cast<float *>(it.out), 0, it.ray, it.nsamp,
                              it.V, it.C, it.wpv, it.nx, it.w, 1, it.max_iter, unit);
    }
}

template <bool W, int DEG, int ROWS>
__device__ __forceinline__ void bp_item_tile(const BpItem &it, int tx, int ty) {
    if (it.out_bf16)
        bp_tile<W, 1, DEG, __nv_bfloat16, ROWS>(it.sino, 0, static_cast<__nv_bfloat16 *>(it.img),
                                                0, it.view_cs, it.a, 1, tx, ty);
    else
        bp_tile<W, 1, DEG, float, ROWS>(it.sino, 0, static_cast<float *>(it.img), 0, it.view_cs,
                                        it.a, 1, tx, ty);
}

// Next tile of a block (block-uniform): fixed stride or the atomic counter.
template <bool DYN>
__device__ __forceinline__ int next_block_unit(int *ctr, int prev) {
    if constexpr (DYN) {
        __shared__ int s_unit;
        __syncthreads();  // every thread has read the previous value
        if (threadIdx.x == 0 && threadIdx.y == 0) s_unit = atomicAdd(ctr, 1);
        __syncthreads();
        return s_unit;
    } else {
        return prev < 0 ? (int)blockIdx.x : prev + (int)gridDim.x;
    }
}

template <bool DYN, int ROWS>
__global__ void __launch_bounds__(256)
    bp_batch_kernel(const __grid_constant__ BpBatch P, int *ctr) {
    for (int u = next_block_unit<DYN>(ctr, -1); u < P.total; u = next_block_unit<DYN>(ctr, u)) {
        const BpItem &it = P.it[find_item(P.it, P.n, u)];
        const int local = u - it.unit0;
        const int ty = local / it.tiles_x, tx = local - ty * it.tiles_x;
        if (it.use_atanf) {
            if (it.weighted)
                bp_item_tile<true, 0, ROWS>(it, tx, ty);
            else
                bp_item_tile<false, 0, ROWS>(it, tx, ty);
        } else {
            if (it.weighted)
                bp_item_tile<true, 8, ROWS>(it, tx, ty);
            else
                bp_item_tile<false, 8, ROWS>(it, tx, ty);
        }
    }
}

__global__ void __launch_bounds__(256) convert_batch_kernel(const __grid_constant__ ConvBatch P) {
    const ConvItem &it = P.it[blockIdx.y];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < it.count;
         k += stride) {
        if (it.mode == kNarrow)
            static_cast<__nv_bfloat16 *>(it.dst)[k] =
                __float2bfloat16(static_cast<const float *>(it.src)[k]);
        else if (it.mode == kWiden)
            static_cast<float *>(it.dst)[k] =
                __bfloat162float(static_cast<const __nv_bfloat16 *>(it.src)[k]);
        else
            static_cast<float *>(it.dst)[k] = static_cast<const float *>(it.src)[k];
    }
}

BpArgs bp_args(const ct_plan *p) {
    BpArgs a;
    a.V = p->g.n_views;
    a.C = p->g.n_cols;
    a.nx = p->g.nx;
    a.ny = p->g.ny;
    a.xmin = p->g.xmin;
    a.ymin = p->g.ymin;
    a.dx = p->g.dx;
    a.dy = p->g.dy;
    a.R = p->g.sid;
    const double inv = 1.0 / (double)p->g.dcol;
    a.inv_dcol = (float)inv;
    a.pos_off = (float)((double)p->g.shift - (double)p->g.left * inv + 0.5);
    a.fC = (float)a.C;
    a.fov_r2 = (double)p->g.rfov * (double)p->g.rfov;
    // degree-4 fits are the degree-8 polynomial with zero high coefficients
    for (int k = 0; k < 9; ++k) a.coef[k] = p->atan_coef[k];
    return a;
}

size_t align256(size_t n) { return (n + 255) / 256 * 256; }

// Slice groups: the items, in order, of every (plan, op, dtype) that two or
// more items share; group_of[i] is item i's group or -1.
constexpr int kGroupMin = 2;
struct Groups {
    std::vector<std::vector<int>> members;
    std::vector<int> group_of;
};
Groups slice_groups(const ct_batch_item *items, int n) {
    Groups G;
    G.group_of.assign(n, -1);
    std::vector<std::vector<int>> all;
    for (int i = 0; i < n; ++i) {
        int g = -1;
        for (size_t k = 0; k < all.size() && g < 0; ++k) {
            const ct_batch_item &f = items[all[k][0]];
            if (f.plan == items[i].plan && f.op == items[i].op && f.dtype == items[i].dtype)
                g = (int)k;
        }
        if (g < 0) {
            g = (int)all.size();
            all.emplace_back();
        }
        all[(size_t)g].push_back(i);
    }
    for (auto &m : all) {
        if ((int)m.size() < kGroupMin) continue;
        for (int i : m) G.group_of[(size_t)i] = (int)G.members.size();
        G.members.push_back(m);
    }
    return G;
}

// Per-slice element counts of an item's input and output.
long long in_count(const ct_batch_item &it) {
    const ct_plan *p = it.plan;
    return (it.op == CT_OP_FP || it.op == CT_OP_FBP_ADJOINT) ? (long long)p->g.nx * p->g.ny
                                                            : (long long)p->g.n_views * p->g.n_cols;
}
long long out_count(const ct_batch_item &it) {
    const ct_plan *p = it.plan;
    return (it.op == CT_OP_FP || it.op == CT_OP_FBP_ADJOINT) ? (long long)p->g.n_views * p->g.n_cols
                                                            : (long long)p->g.nx * p->g.ny;
}

struct Layout {
    // byte offsets into the workspace, per item (SIZE_MAX = unused); the
    // first 256 bytes hold the dynamic-schedule counters
    std::vector<size_t> quads, in32, filt, out32, wtd;
    // per slice group: gathered inputs, results before the scatter, and the
    // plan path's workspace (all FP32, slices contiguous)
    std::vector<size_t> g_in, g_out, g_work;
    // slice-quad images of the single FBP-adjoint items' transposes (they run
    // one after another on the stream, so they share one buffer); SIZE_MAX
    // when none uses the gather form
    size_t tquads = SIZE_MAX;
    size_t total = 0;
};
constexpr size_t kCounterBytes = 256;

// Where an FBP slice group's tap images (an FBP-adjoint group's slice-quad
// images) start in its workspace (after the filtered and pre-weighted
// sinograms, 256-byte aligned).
size_t group_pairs_offset(const ct_batch_item &it, int g) {
    const ct_plan *p = it.plan;
    const size_t sino = sizeof(float) * (size_t)g * p->g.n_views * p->g.n_cols;
    return ((has_preweight(p) ? 2 : 1) * sino + 255) & ~(size_t)255;
}

// Workspace of a slice group's plan path.
size_t group_work_bytes(const ct_batch_item &it, int g) {
    const ct_plan *p = it.plan;
    switch (it.op) {
        case CT_OP_FP:
            return fp_fan_work_bytes(p, g);
        case CT_OP_BP:  // tap images
            return bp_fan_work_bytes(p, g);
        case CT_OP_FBP:  // filtered (+ pre-weighted) sinograms, then tap images
            return group_pairs_offset(it, g) + bp_fan_work_bytes(p, g);
        case CT_OP_FBP_ADJOINT:  // transposed (+ filtered) sinograms, then slice quads
            return group_pairs_offset(it, g) + bp_fan_transpose_work_bytes(p, g);
        default:
            return 0;
    }
}

Layout plan_layout(const ct_batch_item *items, int n, const Groups &G) {
    Layout L;
    L.quads.assign(n, SIZE_MAX);
    L.in32.assign(n, SIZE_MAX);
    L.filt.assign(n, SIZE_MAX);
    L.out32.assign(n, SIZE_MAX);
    L.wtd.assign(n, SIZE_MAX);
    size_t off = kCounterBytes;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += align256(bytes);
        return o;
    };
    for (const auto &m : G.members) {
        const ct_batch_item &f = items[m[0]];
        const int g = (int)m.size();
        L.g_in.push_back(take(sizeof(float) * (size_t)g * in_count(f)));
        L.g_out.push_back(take(sizeof(float) * (size_t)g * out_count(f)));
        L.g_work.push_back(take(group_work_bytes(f, g)));
    }
    for (int i = 0; i < n; ++i) {
        if (G.group_of[(size_t)i] >= 0) continue;
        const ct_plan *p = items[i].plan;
        const size_t img = sizeof(float) * (size_t)p->g.nx * p->g.ny;
        const size_t sino = sizeof(float) * (size_t)p->g.n_views * p->g.n_cols;
        const bool bf = items[i].dtype == CT_DTYPE_BF16;
        switch (items[i].op) {
            case CT_OP_FP:
                L.quads[i] = take(sizeof(float4) * 2 * (size_t)(p->g.nx + 1) * (p->g.nx + 1));
                break;
            case CT_OP_BP:
                if (bf) L.in32[i] = take(sino);
                break;
            case CT_OP_FBP:
                if (bf) L.in32[i] = take(sino);
                L.filt[i] = take(sino);
                if (has_preweight(p)) L.wtd[i] = take(sino);
                break;
            case CT_OP_FBP_ADJOINT:
                if (bf) L.in32[i] = take(img);
                L.filt[i] = take(sino);
                if (bf) L.out32[i] = take(sino);
                if (has_preweight(p)) L.wtd[i] = take(sino);
                break;
            default:
                break;
        }
    }
    size_t tq = 0;
    for (int i = 0; i < n; ++i)
        if (G.group_of[(size_t)i] < 0 && items[i].op == CT_OP_FBP_ADJOINT) {
            const size_t b = bp_fan_transpose_work_bytes(items[i].plan, 1);
            tq = b > tq ? b : tq;
        }
    if (tq) L.tquads = take(tq);
    L.total = off;
    return L;
}

ct_status check_items(const ct_batch_item *items, int n) {
    if (n < 0 || n > kMax) return CT_ERR_INVALID_ARGUMENT;
    if (n > 0 && !items) return CT_ERR_NULL_POINTER;
    for (int i = 0; i < n; ++i) {
        const ct_batch_item &it = items[i];
        if (!it.plan || !it.d_in || !it.d_out) return CT_ERR_NULL_POINTER;
        if (it.plan->n_rows != 1 || it.plan->nz != 1) return CT_ERR_INVALID_ARGUMENT;
        if (it.dtype != CT_DTYPE_F32 && it.dtype != CT_DTYPE_BF16) return CT_ERR_INVALID_ARGUMENT;
        if (it.op != CT_OP_FP && it.op != CT_OP_BP && it.op != CT_OP_FBP &&
            it.op != CT_OP_FBP_ADJOINT)
            return CT_ERR_INVALID_ARGUMENT;
        if (it.d_in == it.d_out) return CT_ERR_INVALID_ARGUMENT;
        if (it.plan->device != items[0].plan->device) return CT_ERR_INVALID_ARGUMENT;
        // the persistent backprojection keeps exact weights only
        if (it.op != CT_OP_FP && it.plan->opts.texture_weights) return CT_ERR_UNSUPPORTED;
        if ((it.op == CT_OP_FBP || it.op == CT_OP_FBP_ADJOINT) &&
            it.plan->filter_algo != CT_FILTER_TOEPLITZ_TC &&
            ramp_direct_smem(it.plan->g.n_cols) > 227 * 1024)
            return CT_ERR_UNSUPPORTED;
    }
    return CT_OK;
}

int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace

ct_status batch_workspace(const ct_batch_item *items, int n, size_t *bytes) {
    ct_status st = check_items(items, n);
    if (st != CT_OK) return st;
    *bytes = plan_layout(items, n, slice_groups(items, n)).total;
    return CT_OK;
}

// Enqueues the whole batch on `stream`; returns a CUDA error code.
// Items in launch order: as given, or (dynamic schedule) by decreasing work
// so that the largest items are taken first.
std::vector<int> order_by_work(const ct_batch_item *items, int n, bool largest_first, bool fp) {
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    if (largest_first) {
        auto work = [&](int i) {
            const ct_plan *p = items[i].plan;
            // FP: rays x path length; BP: pixels x views
            return fp ? (double)p->g.n_views * p->g.n_cols * p->g.nx
                      : (double)p->g.nx * p->g.ny * p->g.n_views;
        };
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return work(a) > work(b); });
    }
    return idx;
}

int batch_run(const ct_batch_item *items, int n, void *work, void *stream,
              const ct_batch_config &cfg, void **ev) {
    cudaStream_t s = (cudaStream_t)stream;
    const Groups G = slice_groups(items, n);
    const Layout L = plan_layout(items, n, G);
    auto grouped = [&](int i) { return G.group_of[(size_t)i] >= 0; };
    uint8_t *ws = static_cast<uint8_t *>(work);
    auto at = [&](size_t off) { return static_cast<void *>(ws + off); };
    const int sms = sm_count();
    cudaError_t e = cudaSuccess;

    int *ctr = static_cast<int *>(work);  // [0]: FP units, [1]: BP tiles
    const bool dyn_any = cfg.fp_dynamic || cfg.bp_dynamic;
    if (dyn_any && (e = cudaMemsetAsync(ctr, 0, 2 * sizeof(int), s)) != cudaSuccess) return (int)e;
    cudaEvent_t *evs = reinterpret_cast<cudaEvent_t *>(ev);

    // 0: slice groups: gather (widen), the plan's multi-slice kernels, scatter
    // (narrow)
    if (!G.members.empty()) {
        auto convert = [&](const ConvBatch &CB, long long maxc) {
            const int bx = (int)((maxc + 255) / 256 < 1024 ? (maxc + 255) / 256 : 1024);
            convert_batch_kernel<<<dim3(bx, CB.n), 256, 0, s>>>(CB);
            ct_count_launch();
            return cudaGetLastError();
        };
        ConvBatch gather{}, scatter{};
        long long max_in = 0, max_out = 0;
        for (size_t gi = 0; gi < G.members.size(); ++gi) {
            const auto &m = G.members[gi];
            const long long ci = in_count(items[m[0]]), co = out_count(items[m[0]]);
            for (size_t k = 0; k < m.size(); ++k) {
                const ct_batch_item &it = items[m[k]];
                const bool bf = it.dtype == CT_DTYPE_BF16;
                gather.it[gather.n++] =
                    ConvItem{it.d_in, static_cast<float *>(at(L.g_in[gi])) + (size_t)k * ci, ci,
                             bf ? kWiden : kCopy};
                scatter.it[scatter.n++] =
                    ConvItem{static_cast<float *>(at(L.g_out[gi])) + (size_t)k * co, it.d_out, co,
                             bf ? kNarrow : kCopy};
            }
            max_in = std::max(max_in, ci);
            max_out = std::max(max_out, co);
        }
        if ((e = convert(gather, max_in)) != cudaSuccess) return (int)e;
        for (size_t gi = 0; gi < G.members.size(); ++gi) {
            const ct_batch_item &f = items[G.members[gi][0]];
            const ct_plan *p = f.plan;
            const int g = (int)G.members[gi].size();
            const float *in = static_cast<const float *>(at(L.g_in[gi]));
            float *out = static_cast<float *>(at(L.g_out[gi]));
            float *wk = static_cast<float *>(at(L.g_work[gi]));
            const size_t sino = (size_t)g * p->g.n_views * p->g.n_cols;
            const int rows = g * p->g.n_views;
            int r = 0;
            if (f.op == CT_OP_FP) {
                r = fp_fan(p, in, out, g, wk, s);
            } else if (f.op == CT_OP_BP) {
                r = bp_fan(p, in, out, g, 0, bp_fan_work_bytes(p, g) ? wk : nullptr, s);
            } else if (f.op == CT_OP_FBP) {  // as ct_fbp_fan
                const float *src = in;
                if (has_preweight(p)) {
                    if ((r = apply_preweight(p, in, wk + sino, g, s)) == 0) src = wk + sino;
                }
                if (r == 0) r = ramp_filter(p, src, wk, rows, s);
                void *pw = bp_fan_work_bytes(p, g)
                               ? static_cast<char *>(static_cast<void *>(wk)) +
                                     group_pairs_offset(f, g)
                               : nullptr;
                if (r == 0) r = bp_fan(p, wk, out, g, 1, pw, s);
            } else {  // CT_OP_FBP_ADJOINT, as ct_fbp_fan_adjoint
                void *tw = bp_fan_transpose_work_bytes(p, g)
                               ? static_cast<char *>(static_cast<void *>(wk)) +
                                     group_pairs_offset(f, g)
                               : nullptr;
                r = bp_fan_transpose(p, in, wk, g, 1, tw, s);
                if (r == 0 && !has_preweight(p)) {
                    r = ramp_filter(p, wk, out, rows, s);
                } else if (r == 0) {
                    r = ramp_filter(p, wk, wk + sino, rows, s);
                    if (r == 0) r = apply_preweight(p, wk + sino, out, g, s);
                }
            }
            if (r != 0) return r;
        }
        if ((e = convert(scatter, max_out)) != cudaSuccess) return (int)e;
    }

    // 1-2: forward projections
    {
        QuadBatch QB{};
        FpBatch FB{};
        for (int i : order_by_work(items, n, cfg.fp_dynamic != 0, true)) {
            if (items[i].op != CT_OP_FP || grouped(i)) continue;
            const ct_plan *p = items[i].plan;
            const int Q = p->g.nx + 1;
            QuadItem &q = QB.it[QB.n++];
            q.img = items[i].d_in;
            q.quads = static_cast<float4 *>(at(L.quads[i]));
            q.nx = p->g.nx;
            q.ny = p->g.ny;
            q.bf16 = items[i].dtype == CT_DTYPE_BF16;
            q.blocks_x = (Q + 31) / 32;
            q.blocks_y = (Q + 7) / 8;
            q.unit0 = QB.total;
            QB.total += 2 * q.blocks_x * q.blocks_y;
            FpItem &f = FB.it[FB.n++];
            f.quads = q.quads;
            f.out = items[i].d_out;
            f.ray = reinterpret_cast<const float4 *>(p->d_ray);
            f.nsamp = p->d_nsamp;
            f.V = p->g.n_views;
            f.C = p->g.n_cols;
            f.wpv = (f.C + 31) / 32;
            f.nx = p->g.nx;
            f.max_iter = 2 * (p->g.nx > p->g.ny ? p->g.nx : p->g.ny) + 8;
            f.out_bf16 = q.bf16;
            f.w = p->fp_weight;
            f.unit0 = FB.total;
            FB.total += f.V * f.wpv;
        }
        if (QB.n > 0) {
            quads_batch_kernel<<<QB.total < sms * 16 ? QB.total : sms * 16, dim3(32, 8), 0, s>>>(
                QB);
            const int cap = sms * cfg.fp_blocks_per_sm, want = (FB.total + 7) / 8;
            if (evs) cudaEventRecord(evs[0], s);
            if (cfg.fp_dynamic)
                fp_batch_kernel<true><<<want < cap ? want : cap, 256, 0, s>>>(FB, ctr);
            else
                fp_batch_kernel<false><<<want < cap ? want : cap, 256, 0, s>>>(FB, ctr);
            if (evs) cudaEventRecord(evs[1], s);
            ct_count_launch(2);
            if ((e = cudaGetLastError()) != cudaSuccess) return (int)e;
        }
    }
    // 3: widen BF16 inputs of the BP / FBP / FBP-adjoint items
    {
        ConvBatch CB{};
        int maxc = 0;
        for (int i = 0; i < n; ++i) {
            if (items[i].op == CT_OP_FP || items[i].dtype != CT_DTYPE_BF16 || grouped(i)) continue;
            const ct_plan *p = items[i].plan;
            const long long cnt = items[i].op == CT_OP_FBP_ADJOINT
                                      ? (long long)p->g.nx * p->g.ny
                                      : (long long)p->g.n_views * p->g.n_cols;
            CB.it[CB.n++] = ConvItem{items[i].d_in, at(L.in32[i]), cnt, kWiden};
            maxc = cnt > maxc ? (int)cnt : maxc;
        }
        if (CB.n > 0) {
            const int bx = (maxc + 255) / 256 < 1024 ? (maxc + 255) / 256 : 1024;
            convert_batch_kernel<<<dim3(bx, CB.n), 256, 0, s>>>(CB);
            ct_count_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) return (int)e;
        }
    }
    // filters (FBP) and transposes + filters (FBP adjoint), per item
    for (int i = 0; i < n; ++i) {
        if (grouped(i)) continue;
        const ct_plan *p = items[i].plan;
        const bool bf = items[i].dtype == CT_DTYPE_BF16;
        const float *in32 = bf ? static_cast<const float *>(at(L.in32[i]))
                               : static_cast<const float *>(items[i].d_in);
        if (items[i].op == CT_OP_FBP) {
            const float *src = in32;
            if (has_preweight(p)) {  // short scan / cosine: weight, then filter
                float *w = static_cast<float *>(at(L.wtd[i]));
                if ((e = (cudaError_t)apply_preweight(p, in32, w, 1, s)) != cudaSuccess) return (int)e;
                src = w;
            }
            if ((e = (cudaError_t)ramp_filter(p, src, static_cast<float *>(at(L.filt[i])),
                                              p->g.n_views, s)) != cudaSuccess)
                return (int)e;
        } else if (items[i].op == CT_OP_FBP_ADJOINT) {
            float *t = static_cast<float *>(at(L.filt[i]));
            void *tw = bp_fan_transpose_work_bytes(p, 1) && L.tquads != SIZE_MAX
                           ? at(L.tquads)
                           : nullptr;
            if ((e = (cudaError_t)bp_fan_transpose(p, in32, t, 1, 1, tw, s)) != cudaSuccess)
                return (int)e;
            float *dst = bf ? static_cast<float *>(at(L.out32[i]))
                            : static_cast<float *>(items[i].d_out);
            float *fdst = has_preweight(p) ? static_cast<float *>(at(L.wtd[i])) : dst;
            if ((e = (cudaError_t)ramp_filter(p, t, fdst, p->g.n_views, s)) != cudaSuccess)
                return (int)e;
            if (has_preweight(p) &&
                (e = (cudaError_t)apply_preweight(p, fdst, dst, 1, s)) != cudaSuccess)
                return (int)e;
        }
    }
    // 4: backprojections of BP and FBP items
    {
        BpBatch BB{};
        const int tile_h = cfg.bp_tile_rows;
        for (int i : order_by_work(items, n, cfg.bp_dynamic != 0, false)) {
            if ((items[i].op != CT_OP_BP && items[i].op != CT_OP_FBP) || grouped(i)) continue;
            const ct_plan *p = items[i].plan;
            const bool bf = items[i].dtype == CT_DTYPE_BF16;
            BpItem &b = BB.it[BB.n++];
            if (items[i].op == CT_OP_FBP)
                b.sino = static_cast<const float *>(at(L.filt[i]));
            else
                b.sino = bf ? static_cast<const float *>(at(L.in32[i]))
                            : static_cast<const float *>(items[i].d_in);
            b.img = items[i].d_out;
            b.view_cs = reinterpret_cast<const float2 *>(p->d_view_cs);
            b.a = bp_args(p);
            b.tiles_x = (p->g.nx + kBpTile - 1) / kBpTile;
            b.unit0 = BB.total;
            b.out_bf16 = bf;
            b.weighted = items[i].op == CT_OP_FBP;
            b.use_atanf = p->atan_deg == 0;
            BB.total += b.tiles_x * ((p->g.ny + tile_h - 1) / tile_h);
        }
        if (BB.n > 0) {
            const int cap = sms * cfg.bp_blocks_per_sm;
            const dim3 grid(BB.total < cap ? BB.total : cap), block(32, 8);
            if (evs) cudaEventRecord(evs[2], s);
            if (cfg.bp_dynamic) {
                if (tile_h == 16)
                    bp_batch_kernel<true, 2><<<grid, block, 0, s>>>(BB, ctr + 1);
                else
                    bp_batch_kernel<true, 4><<<grid, block, 0, s>>>(BB, ctr + 1);
            } else {
                if (tile_h == 16)
                    bp_batch_kernel<false, 2><<<grid, block, 0, s>>>(BB, ctr + 1);
                else
                    bp_batch_kernel<false, 4><<<grid, block, 0, s>>>(BB, ctr + 1);
            }
            if (evs) cudaEventRecord(evs[3], s);
            ct_count_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) return (int)e;
        }
    }
    // 5: narrow the BF16 FBP-adjoint results
    {
        ConvBatch CB{};
        int maxc = 0;
        for (int i = 0; i < n; ++i) {
            if (items[i].op != CT_OP_FBP_ADJOINT || items[i].dtype != CT_DTYPE_BF16 || grouped(i))
                continue;
            const ct_plan *p = items[i].plan;
            const long long cnt = (long long)p->g.n_views * p->g.n_cols;
            CB.it[CB.n++] = ConvItem{at(L.out32[i]), items[i].d_out, cnt, kNarrow};
            maxc = cnt > maxc ? (int)cnt : maxc;
        }
        if (CB.n > 0) {
            const int bx = (maxc + 255) / 256 < 1024 ? (maxc + 255) / 256 : 1024;
            convert_batch_kernel<<<dim3(bx, CB.n), 256, 0, s>>>(CB);
            ct_count_launch();
        }
    }
    return (int)cudaGetLastError();
}

ct_batch_config batch_default_config() {
    ct_batch_config c{};
    c.fp_blocks_per_sm = 3;
    c.fp_dynamic = 0;
    c.bp_blocks_per_sm = 4;
    c.bp_dynamic = 0;
    c.bp_tile_rows = 32;
    return c;
}

ct_status batch_check_config(const ct_batch_config &c) {
    if (c.fp_blocks_per_sm < 1 || c.fp_blocks_per_sm > 16 || c.bp_blocks_per_sm < 1 ||
        c.bp_blocks_per_sm > 16 || (c.fp_dynamic != 0 && c.fp_dynamic != 1) ||
        (c.bp_dynamic != 0 && c.bp_dynamic != 1) ||
        (c.bp_tile_rows != 16 && c.bp_tile_rows != 32))
        return CT_ERR_INVALID_ARGUMENT;
    for (int r : c.reserved)
        if (r != 0) return CT_ERR_INVALID_ARGUMENT;
    return CT_OK;
}

namespace {

std::mutex g_cfg_mu;
std::map<std::string, ct_batch_config> g_cfg;

// Batch shape: device and, per item, operator, storage type and sizes.
std::string batch_key(const ct_batch_item *items, int n) {
    std::string k = std::to_string(n > 0 ? items[0].plan->device : -1);
    for (int i = 0; i < n; ++i) {
        const ct_plan *p = items[i].plan;
        k += '|' + std::to_string(items[i].op) + ',' + std::to_string(items[i].dtype) + ',' +
             std::to_string(p->g.nx) + ',' + std::to_string(p->g.ny) + ',' +
             std::to_string(p->g.n_views) + ',' + std::to_string(p->g.n_cols);
    }
    return k;
}

}  // namespace

ct_batch_config batch_lookup(const ct_batch_item *items, int n, bool *tuned) {
    std::lock_guard<std::mutex> lock(g_cfg_mu);
    auto it = g_cfg.find(batch_key(items, n));
    if (tuned) *tuned = it != g_cfg.end();
    return it != g_cfg.end() ? it->second : batch_default_config();
}

void batch_store(const ct_batch_item *items, int n, const ct_batch_config *c) {
    std::lock_guard<std::mutex> lock(g_cfg_mu);
    if (c)
        g_cfg[batch_key(items, n)] = *c;
    else
        g_cfg.erase(batch_key(items, n));
}

// Candidates: FP {1,2,3,4,6,8} blocks/SM x {stride, dynamic}; BP {2,3,4,6,8,
// 12} blocks/SM x {stride, dynamic} x {32, 16}-row tiles.  Run k pairs FP
// candidate k mod 12 with BP candidate k mod 24, so 24 runs per repetition
// time every candidate of both launches; each candidate keeps its fastest
// repetition.
int batch_tune(const ct_batch_item *items, int n, void *work, void *stream, int reps,
               ct_batch_config *best) {
    static const int kFpBlocks[] = {1, 2, 3, 4, 6, 8};
    static const int kBpBlocks[] = {2, 3, 4, 6, 8, 12};
    std::vector<ct_batch_config> fpc, bpc;
    for (int dyn = 0; dyn < 2; ++dyn)
        for (int b : kFpBlocks) {
            ct_batch_config c = batch_default_config();
            c.fp_blocks_per_sm = b;
            c.fp_dynamic = dyn;
            fpc.push_back(c);
        }
    for (int rows : {32, 16})
        for (int dyn = 0; dyn < 2; ++dyn)
            for (int b : kBpBlocks) {
                ct_batch_config c = batch_default_config();
                c.bp_blocks_per_sm = b;
                c.bp_dynamic = dyn;
                c.bp_tile_rows = rows;
                bpc.push_back(c);
            }
    const int runs = (int)std::max(fpc.size(), bpc.size());
    std::vector<float> fpt(fpc.size(), 1e30f), bpt(bpc.size(), 1e30f);
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t ev[4] = {};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = cudaEventCreate(&ev[k]);
    // only the persistent launches (items outside slice groups) have shapes
    bool has_fp = false, has_bp = false;
    const Groups G = slice_groups(items, n);
    for (int i = 0; i < n; ++i) {
        if (G.group_of[(size_t)i] >= 0) continue;
        has_fp |= items[i].op == CT_OP_FP;
        has_bp |= items[i].op == CT_OP_BP || items[i].op == CT_OP_FBP;
    }
    // one untimed run first (module load, first-touch of the workspace)
    if (e == cudaSuccess)
        e = (cudaError_t)batch_run(items, n, work, stream, batch_default_config(), nullptr);
    for (int r = 0; r < reps && e == cudaSuccess; ++r) {
        for (int k = 0; k < runs && e == cudaSuccess; ++k) {
            ct_batch_config c = fpc[k % fpc.size()];
            const ct_batch_config &b = bpc[k % bpc.size()];
            c.bp_blocks_per_sm = b.bp_blocks_per_sm;
            c.bp_dynamic = b.bp_dynamic;
            c.bp_tile_rows = b.bp_tile_rows;
            e = (cudaError_t)batch_run(items, n, work, stream, c, reinterpret_cast<void **>(ev));
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            float ms = 0.0f;
            if (e == cudaSuccess && has_fp && cudaEventElapsedTime(&ms, ev[0], ev[1]) == cudaSuccess)
                fpt[k % fpc.size()] = std::min(fpt[k % fpc.size()], ms);
            if (e == cudaSuccess && has_bp && cudaEventElapsedTime(&ms, ev[2], ev[3]) == cudaSuccess)
                bpt[k % bpc.size()] = std::min(bpt[k % bpc.size()], ms);
        }
    }
    for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
    if (e != cudaSuccess) return (int)e;
    const size_t bf = std::min_element(fpt.begin(), fpt.end()) - fpt.begin();
    const size_t bb = std::min_element(bpt.begin(), bpt.end()) - bpt.begin();
    ct_batch_config c = batch_default_config();
    if (has_fp) {
        c.fp_blocks_per_sm = fpc[bf].fp_blocks_per_sm;
        c.fp_dynamic = fpc[bf].fp_dynamic;
    }
    if (has_bp) {
        c.bp_blocks_per_sm = bpc[bb].bp_blocks_per_sm;
        c.bp_dynamic = bpc[bb].bp_dynamic;
        c.bp_tile_rows = bpc[bb].bp_tile_rows;
    }
    *best = c;
    return (int)cudaSuccess;
}

}  // namespace ctk
