// Device-side index checks of debug builds (compiled with -DCT_DEBUG; the
// release library has none: every macro below expands to the plain access).
//
// The reference stopped the process on any CUDA error (checkCudaErrors,
// FP/transform.cu:4) and checked no index.  In a debug build every gather
// of the interpolation kernels tests its index against the array it reads;
// an index outside makes the kernel skip that access (it reads zero
// instead) and record the source line in a per-file device flag, which
// ct_plan_check reports as CT_ERR_DEVICE_CHECK (and clears).  Nothing traps
// and nothing is read out of bounds, so the context stays usable.
#pragma once

#include <cuda_runtime.h>

#ifdef CT_DEBUG
namespace ctk {
namespace dbg {
// one flag per translation unit: 0, or the first failing check's line
static __device__ unsigned int g_flag;
__device__ __forceinline__ void raise_line(unsigned line) { atomicCAS(&g_flag, 0u, line); }
// Host: the registry of every file's flag reader (api.cu).
using TakeFn = unsigned (*)();
void add_flag(TakeFn fn, const char *file);
// Reads and clears this file's flag.
static unsigned take_flag() {
    unsigned v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_flag, sizeof(v)) != cudaSuccess) return 0;
    if (v) cudaMemcpyToSymbol(g_flag, &zero, sizeof(zero));
    return v;
}
struct Registrar {
    explicit Registrar(const char *file) { add_flag(&take_flag, file); }
};
static Registrar g_registrar(__FILE__);
}  // namespace dbg
}  // namespace ctk
// true when the check holds; otherwise records the line and gives false
#define CT_DCHECK(cond) ((cond) ? true : (::ctk::dbg::raise_line(__LINE__), false))
// *(ptr) when ok, else zero of its type (and the line recorded)
#define CT_DLOAD(ok, ptr) (CT_DCHECK(ok) ? __ldg(ptr) : decltype(__ldg(ptr)){})
#define CT_DEBUG_BUILD 1
#else
// release: no test is made (sizeof does not evaluate its operand)
#define CT_DCHECK(cond) (static_cast<void>(sizeof(cond)), true)
#define CT_DLOAD(ok, ptr) (static_cast<void>(sizeof(ok)), __ldg(ptr))
#define CT_DEBUG_BUILD 0
#endif
