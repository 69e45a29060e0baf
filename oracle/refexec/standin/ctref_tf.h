// ctref_tf.h -- stand-in for the slice of TensorFlow's C++ op API that the
// reference's op wrappers use (FP/transform.cc, BP/transform.cc,
// FBP/transform.cc, FDK/FBP.cc): op and kernel registration, attributes,
// tensors of float, output allocation and the shape-function context.  The
// executed-reference harness constructs a registered kernel from attribute
// values and calls its Compute, as TensorFlow's executor would.
// TEST INFRASTRUCTURE ONLY.
//
// Deviations from TensorFlow, all on paths the reference does not rely on:
// tensors hold float only; allocate_output zero-fills (TensorFlow leaves the
// buffer uninitialised); DCHECK_EQ is always checked.
#pragma once

#include <cstdint>
#include <functional>
#include <initializer_list>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "third_party/eigen3/unsupported/Eigen/CXX11/Tensor"

namespace tensorflow {

class Status {
  public:
    Status() = default;
    explicit Status(std::string msg) : ok_(false), msg_(std::move(msg)) {}
    static Status OK() { return Status(); }
    bool ok() const { return ok_; }
    const std::string &error_message() const { return msg_; }
    void Update(const Status &s) {
        if (ok_ && !s.ok_) *this = s;
    }

  private:
    bool ok_ = true;
    std::string msg_;
};

class TensorShapeProto {
  public:
    std::vector<int64_t> dims;
};

class TensorShape {
  public:
    TensorShape() = default;
    TensorShape(std::initializer_list<int64_t> d) : d_(d) {}
    explicit TensorShape(std::vector<int64_t> d) : d_(std::move(d)) {}
    int dims() const { return (int)d_.size(); }
    int64_t dim_size(int i) const { return d_.at((size_t)i); }
    int64_t num_elements() const {
        int64_t n = 1;
        for (int64_t v : d_) n *= v;
        return n;
    }
    const std::vector<int64_t> &dim_sizes() const { return d_; }

  private:
    std::vector<int64_t> d_;
};

// The Eigen::TensorMap a Tensor hands out: element access and data().
template <class T, int N>
class TensorView {
  public:
    TensorView(T *p, std::vector<int64_t> d) : p_(p), d_(std::move(d)) {}
    T *data() const { return p_; }
    T &operator()(int64_t i) const {
        static_assert(N == 1, "indexing is used on rank-1 attributes only");
        if (i < 0 || i >= d_.at(0)) throw std::out_of_range("tensor index");
        return p_[i];
    }

  private:
    T *p_;
    std::vector<int64_t> d_;
};

class Tensor {
  public:
    Tensor() = default;
    Tensor(const TensorShape &s, std::vector<float> v)
        : shape_(s), buf_(std::make_shared<std::vector<float>>(std::move(v))) {
        if ((int64_t)buf_->size() != s.num_elements()) throw std::invalid_argument("tensor size");
    }
    const TensorShape &shape() const { return shape_; }
    template <class T, int N>
    TensorView<T, N> tensor() const {
        static_assert(std::is_same<T, float>::value, "the stand-in holds float tensors only");
        if (shape_.dims() != N) throw std::invalid_argument("tensor rank mismatch");
        return TensorView<T, N>(buf_ ? buf_->data() : nullptr, shape_.dim_sizes());
    }
    float *raw() const { return buf_ ? buf_->data() : nullptr; }

  private:
    TensorShape shape_;
    std::shared_ptr<std::vector<float>> buf_;
};

namespace shape_inference {
struct ShapeHandle {
    int rank = -1;
    std::vector<int64_t> dims;
};
class InferenceContext {
  public:
    InferenceContext(std::vector<ShapeHandle> inputs,
                     std::map<std::string, TensorShapeProto> shape_attrs)
        : inputs_(std::move(inputs)), attrs_(std::move(shape_attrs)) {}
    ShapeHandle input(int i) const { return inputs_.at((size_t)i); }
    Status WithRank(ShapeHandle s, int rank, ShapeHandle *out) {
        if (s.rank != rank)
            return Status("Shape must be rank " + std::to_string(rank) + " but is rank " +
                          std::to_string(s.rank));
        *out = s;
        return Status::OK();
    }
    Status GetAttr(const std::string &name, TensorShapeProto *out) const {
        auto it = attrs_.find(name);
        if (it == attrs_.end()) return Status("No attr named '" + name + "'");
        *out = it->second;
        return Status::OK();
    }
    Status MakeShapeFromShapeProto(const TensorShapeProto &p, ShapeHandle *out) const {
        out->rank = (int)p.dims.size();
        out->dims = p.dims;
        return Status::OK();
    }
    void set_output(int i, ShapeHandle s) {
        if ((int)outputs_.size() <= i) outputs_.resize((size_t)i + 1);
        outputs_[(size_t)i] = s;
    }
    const std::vector<ShapeHandle> &outputs() const { return outputs_; }

  private:
    std::vector<ShapeHandle> inputs_;
    std::map<std::string, TensorShapeProto> attrs_;
    std::vector<ShapeHandle> outputs_;
};
}  // namespace shape_inference

using ShapeFn = std::function<Status(shape_inference::InferenceContext *)>;

// ---- op registration --------------------------------------------------------
struct OpDef {
    std::string name;
    std::vector<std::string> inputs, outputs, attrs;
    ShapeFn shape_fn;
};
std::map<std::string, OpDef> &op_registry();

class OpDefBuilder {
  public:
    explicit OpDefBuilder(const char *name) { def_.name = name; }
    OpDefBuilder &Input(const char *s) {
        def_.inputs.push_back(s);
        return *this;
    }
    OpDefBuilder &Output(const char *s) {
        def_.outputs.push_back(s);
        return *this;
    }
    OpDefBuilder &Attr(const char *s) {
        def_.attrs.push_back(s);
        return *this;
    }
    template <class F>
    OpDefBuilder &SetShapeFn(F f) {
        def_.shape_fn = f;
        return *this;
    }
    const OpDef &def() const { return def_; }

  private:
    OpDef def_;
};
struct OpDefBuilderReceiver {
    OpDefBuilderReceiver(const OpDefBuilder &b) { op_registry()[b.def().name] = b.def(); }
};

// ---- kernels ----------------------------------------------------------------
class OpKernelConstruction {
  public:
    std::map<std::string, Tensor> tensor_attrs;
    std::map<std::string, TensorShape> shape_attrs;
    Status status;
    Status GetAttr(const std::string &name, TensorShape *out) const {
        auto it = shape_attrs.find(name);
        if (it == shape_attrs.end()) return Status("No attr named '" + name + "'");
        *out = it->second;
        return Status::OK();
    }
    Status GetAttr(const std::string &name, Tensor *out) const {
        auto it = tensor_attrs.find(name);
        if (it == tensor_attrs.end()) return Status("No attr named '" + name + "'");
        *out = it->second;
        return Status::OK();
    }
    void CtxFailure(const Status &s) { status.Update(s); }
};

class OpKernelContext {
  public:
    std::vector<Tensor> inputs, outputs;
    Status status;
    int num_inputs() const { return (int)inputs.size(); }
    const Tensor &input(int i) const { return inputs.at((size_t)i); }
    Status allocate_output(int i, const TensorShape &s, Tensor **out) {
        if (i < 0) return Status("bad output index");
        if ((int)outputs.size() <= i) outputs.resize((size_t)i + 1);
        outputs[(size_t)i] = Tensor(s, std::vector<float>((size_t)s.num_elements(), 0.0f));
        *out = &outputs[(size_t)i];
        return Status::OK();
    }
    void CtxFailure(const Status &s) { status.Update(s); }
};

class OpKernel {
  public:
    explicit OpKernel(OpKernelConstruction *) {}
    virtual ~OpKernel() = default;
    virtual void Compute(OpKernelContext *ctx) = 0;
};

using KernelFactory = std::function<OpKernel *(OpKernelConstruction *)>;
struct KernelDef {
    std::string op, device;
};
std::map<std::string, std::pair<KernelDef, KernelFactory>> &kernel_registry();

class KernelDefBuilder {
  public:
    explicit KernelDefBuilder(const char *op) { def_.op = op; }
    KernelDefBuilder &Device(const char *d) {
        def_.device = d;
        return *this;
    }
    const KernelDef &def() const { return def_; }

  private:
    KernelDef def_;
};
inline KernelDefBuilder Name(const char *op) { return KernelDefBuilder(op); }
constexpr const char *DEVICE_GPU = "GPU";
constexpr const char *DEVICE_CPU = "CPU";

struct KernelRegistrar {
    KernelRegistrar(const KernelDefBuilder &b, KernelFactory f) {
        kernel_registry()[b.def().op] = {b.def(), std::move(f)};
    }
};

[[noreturn]] void check_failed(const char *expr, const char *file, int line);

}  // namespace tensorflow

#define CTREF_CAT2(a, b) a##b
#define CTREF_CAT(a, b) CTREF_CAT2(a, b)
#define REGISTER_OP(name)                                                                  \
    static ::tensorflow::OpDefBuilderReceiver CTREF_CAT(ctref_op_, __COUNTER__) =          \
        ::tensorflow::OpDefBuilder(name)
#define REGISTER_KERNEL_BUILDER(builder, cls)                                              \
    static ::tensorflow::KernelRegistrar CTREF_CAT(ctref_kernel_, __COUNTER__)(            \
        ::tensorflow::builder,                                                             \
        [](::tensorflow::OpKernelConstruction *c) -> ::tensorflow::OpKernel * {            \
            return new cls(c);                                                             \
        })
#define OP_REQUIRES_OK(ctx, expr)                                                          \
    do {                                                                                   \
        ::tensorflow::Status ctref_s_ = (expr);                                            \
        if (!ctref_s_.ok()) {                                                              \
            (ctx)->CtxFailure(ctref_s_);                                                   \
            return;                                                                        \
        }                                                                                  \
    } while (0)
#define TF_RETURN_IF_ERROR(expr)                                                           \
    do {                                                                                   \
        ::tensorflow::Status ctref_s_ = (expr);                                            \
        if (!ctref_s_.ok()) return ctref_s_;                                               \
    } while (0)
#define DCHECK_EQ(a, b)                                                                    \
    do {                                                                                   \
        if (!((a) == (b))) ::tensorflow::check_failed(#a " == " #b, __FILE__, __LINE__);   \
    } while (0)
