// helper_cuda.h stand-in (the CUDA samples' error check), for the
// executed-reference checker.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include "ctref_cuda.h"

namespace ctref {
inline void check(cudaError_t e, const char *expr, const char *file, int line) {
    if (e != cudaSuccess)
        fail(std::string(file) + ":" + std::to_string(line) + ": " + expr + " -> " +
             cudaGetErrorString(e));
}
}  // namespace ctref
#define checkCudaErrors(val) ::ctref::check((val), #val, __FILE__, __LINE__)
