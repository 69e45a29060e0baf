// harness.cpp -- runs the reference's TensorFlow ops, compiled from their own
// sources against the host stand-ins in standin/, and exposes them through a
// small C ABI for the tests.  TEST INFRASTRUCTURE ONLY: it is the
// executed-reference checker that golden vectors are made with; no product
// code links it.
//
// Pieces:
//  - the block scheduler behind ::ctref::launch: blocks in parallel on
//    OpenMP threads, the threads of one block as ucontext fibers on one host
//    thread, switched at __syncthreads();
//  - the op and kernel registries the stand-in REGISTER_OP /
//    REGISTER_KERNEL_BUILDER macros fill;
//  - ctref_run (construct a registered kernel from attribute values, call
//    Compute on one input) and ctref_shape (call the op's shape function).
#include <ucontext.h>

#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "standin/ctref_cuda.h"
#include "standin/ctref_tf.h"

namespace ctref {
namespace {

constexpr size_t kFiberStack = 64 * 1024;

enum : unsigned char { kRunnable = 0, kWaiting = 1, kFinished = 2 };

struct BlockRunner {
    std::vector<ucontext_t> ctx;
    std::vector<char *> stacks;
    std::vector<unsigned char> state;
    ucontext_t main_ctx;
    int cur = -1;
    void (*body)(void *) = nullptr;
    void *arg = nullptr;

    ~BlockRunner() {
        for (char *s : stacks) std::free(s);
    }
    void reserve(int n) {
        while ((int)stacks.size() < n) {
            char *s = static_cast<char *>(std::malloc(kFiberStack));
            if (!s) fail("out of memory for fiber stacks");
            stacks.push_back(s);
        }
        ctx.resize((size_t)n);
        state.resize((size_t)n);
    }
};

thread_local BlockRunner *t_runner = nullptr;

void fiber_entry() {
    BlockRunner *r = t_runner;
    r->body(r->arg);
    r->state[(size_t)r->cur] = kFinished;
    // returning resumes uc_link (the scheduler)
}

void run_block(BlockRunner &r, const dim3 &b) {
    const int n = (int)(b.x * b.y * b.z);
    for (int t = 0; t < n; ++t) {
        ucontext_t &c = r.ctx[(size_t)t];
        if (getcontext(&c) != 0) fail("getcontext failed");
        c.uc_stack.ss_sp = r.stacks[(size_t)t];
        c.uc_stack.ss_size = kFiberStack;
        c.uc_link = &r.main_ctx;
        makecontext(&c, fiber_entry, 0);
        r.state[(size_t)t] = kRunnable;
    }
    for (;;) {
        for (int t = 0; t < n; ++t) {
            if (r.state[(size_t)t] != kRunnable) continue;
            threadIdx = uint3{(unsigned)t % b.x, ((unsigned)t / b.x) % b.y,
                              (unsigned)t / (b.x * b.y)};
            r.cur = t;
            __atomic_signal_fence(__ATOMIC_SEQ_CST);
            swapcontext(&r.main_ctx, &r.ctx[(size_t)t]);
            __atomic_signal_fence(__ATOMIC_SEQ_CST);
        }
        // every thread now waits at a barrier or has finished; a barrier
        // opens once all threads that have not exited reach it
        int waiting = 0;
        for (int t = 0; t < n; ++t) waiting += r.state[(size_t)t] == kWaiting;
        if (waiting == 0) break;
        for (int t = 0; t < n; ++t)
            if (r.state[(size_t)t] == kWaiting) r.state[(size_t)t] = kRunnable;
    }
    r.cur = -1;
}

}  // namespace

[[noreturn]] void fail(const std::string &what) {
    if (t_runner && t_runner->cur >= 0) {
        // no unwinding across fiber stacks: report and stop
        std::fprintf(stderr, "ctref: %s (inside a kernel)\n", what.c_str());
        std::abort();
    }
    throw std::runtime_error(what);
}

void barrier() {
    BlockRunner *r = t_runner;
    if (!r || r->cur < 0) fail("__syncthreads() outside a kernel");
    const int t = r->cur;
    r->state[(size_t)t] = kWaiting;
    __atomic_signal_fence(__ATOMIC_SEQ_CST);
    swapcontext(&r->ctx[(size_t)t], &r->main_ctx);
    __atomic_signal_fence(__ATOMIC_SEQ_CST);
}

void run_grid(const dim3 &g, const dim3 &b, void (*body)(void *), void *arg) {
    const long nb = (long)g.x * g.y * g.z;
    const int nt = (int)(b.x * b.y * b.z);
    if (nt <= 0 || nt > 1024 || nb <= 0) fail("launch configuration out of range");
#pragma omp parallel
    {
        thread_local BlockRunner runner;
        runner.reserve(nt);
        runner.body = body;
        runner.arg = arg;
        t_runner = &runner;
        blockDim = b;
        gridDim = g;
#pragma omp for schedule(dynamic, 4)
        for (long k = 0; k < nb; ++k) {
            blockIdx = uint3{(unsigned)(k % g.x), (unsigned)((k / g.x) % g.y),
                             (unsigned)(k / ((long)g.x * g.y))};
            run_block(runner, b);
        }
        t_runner = nullptr;
    }
}

}  // namespace ctref

namespace tensorflow {
std::map<std::string, OpDef> &op_registry() {
    static std::map<std::string, OpDef> m;
    return m;
}
std::map<std::string, std::pair<KernelDef, KernelFactory>> &kernel_registry() {
    static std::map<std::string, std::pair<KernelDef, KernelFactory>> m;
    return m;
}
[[noreturn]] void check_failed(const char *expr, const char *file, int line) {
    throw std::runtime_error(std::string("check failed: ") + expr + " at " + file + ":" +
                             std::to_string(line));
}
}  // namespace tensorflow

namespace {

std::mutex g_mu;  // the reference keeps its geometry in file-scope statics

int report(char *err, long long err_len, const std::string &msg) {
    if (err && err_len > 0) std::snprintf(err, (size_t)err_len, "%s", msg.c_str());
    return 1;
}

tensorflow::TensorShape shape_of(const long long *d, int rank) {
    std::vector<int64_t> v;
    for (int i = 0; i < rank; ++i) v.push_back(d[i]);
    return tensorflow::TensorShape(v);
}

bool input_is_volume(const tensorflow::OpDef &def) {
    return !def.inputs.empty() && def.inputs[0].rfind("volume", 0) == 0;
}

}  // namespace

extern "C" {

// Names of the registered ops, ';'-separated.
int ctref_ops(char *buf, long long len) {
    std::string s;
    for (auto &kv : tensorflow::kernel_registry()) s += kv.first + ";";
    std::snprintf(buf, (size_t)len, "%s", s.c_str());
    return 0;
}

// Runs op `name` with attributes parameter / angle / vol_shape / proj_shape on
// one input (shaped vol_shape for an op whose input is "volume", proj_shape
// otherwise) and copies its output, whose element count must be n_output.
int ctref_run(const char *name, const float *parameter, long long n_parameter,
              const float *angle, long long n_angle, const long long *vol_shape, int vol_rank,
              const long long *proj_shape, int proj_rank, const float *input, long long n_input,
              float *output, long long n_output, char *err, long long err_len) {
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        auto &kr = tensorflow::kernel_registry();
        auto &orr = tensorflow::op_registry();
        auto it = kr.find(name);
        auto od = orr.find(name);
        if (it == kr.end() || od == orr.end())
            return report(err, err_len, std::string("no op named ") + name);
        tensorflow::OpKernelConstruction c;
        c.tensor_attrs["parameter"] = tensorflow::Tensor(
            tensorflow::TensorShape({n_parameter}),
            std::vector<float>(parameter, parameter + n_parameter));
        c.tensor_attrs["angle"] = tensorflow::Tensor(
            tensorflow::TensorShape({n_angle}), std::vector<float>(angle, angle + n_angle));
        c.shape_attrs["vol_shape"] = shape_of(vol_shape, vol_rank);
        c.shape_attrs["proj_shape"] = shape_of(proj_shape, proj_rank);
        std::unique_ptr<tensorflow::OpKernel> op(it->second.second(&c));
        if (!c.status.ok()) return report(err, err_len, c.status.error_message());
        const tensorflow::TensorShape in_shape = input_is_volume(od->second)
                                                     ? shape_of(vol_shape, vol_rank)
                                                     : shape_of(proj_shape, proj_rank);
        if (in_shape.num_elements() != n_input)
            return report(err, err_len, "input size does not match its shape attribute");
        tensorflow::OpKernelContext ctx;
        ctx.inputs.emplace_back(in_shape, std::vector<float>(input, input + n_input));
        op->Compute(&ctx);
        if (!ctx.status.ok()) return report(err, err_len, ctx.status.error_message());
        if (ctx.outputs.empty()) return report(err, err_len, "the op allocated no output");
        const tensorflow::Tensor &out = ctx.outputs[0];
        if (out.shape().num_elements() != n_output)
            return report(err, err_len, "output size mismatch");
        std::memcpy(output, out.raw(), sizeof(float) * (size_t)n_output);
        return 0;
    } catch (const std::exception &e) {
        return report(err, err_len, e.what());
    }
}

// Calls op `name`'s shape function on an input of shape in_shape; writes the
// inferred output shape (rank into *out_rank, at most 8 dims).
int ctref_shape(const char *name, const long long *in_shape, int in_rank,
                const long long *vol_shape, int vol_rank, const long long *proj_shape,
                int proj_rank, long long *out_shape, int *out_rank, char *err,
                long long err_len) {
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        auto od = tensorflow::op_registry().find(name);
        if (od == tensorflow::op_registry().end() || !od->second.shape_fn)
            return report(err, err_len, std::string("no shape function for ") + name);
        tensorflow::shape_inference::ShapeHandle in;
        in.rank = in_rank;
        for (int i = 0; i < in_rank; ++i) in.dims.push_back(in_shape[i]);
        std::map<std::string, tensorflow::TensorShapeProto> attrs;
        for (int i = 0; i < vol_rank; ++i) attrs["vol_shape"].dims.push_back(vol_shape[i]);
        for (int i = 0; i < proj_rank; ++i) attrs["proj_shape"].dims.push_back(proj_shape[i]);
        tensorflow::shape_inference::InferenceContext ic({in}, attrs);
        tensorflow::Status s = od->second.shape_fn(&ic);
        if (!s.ok()) return report(err, err_len, s.error_message());
        if (ic.outputs().empty() || ic.outputs()[0].rank > 8)
            return report(err, err_len, "no output shape");
        *out_rank = ic.outputs()[0].rank;
        for (int i = 0; i < *out_rank; ++i) out_shape[i] = ic.outputs()[0].dims[(size_t)i];
        return 0;
    } catch (const std::exception &e) {
        return report(err, err_len, e.what());
    }
}

}  // extern "C"
