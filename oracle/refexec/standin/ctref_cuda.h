// ctref_cuda.h -- host stand-in for the CUDA runtime pieces that the
// reference's kernel sources use (FP/transform.cu, BP/transform.cu,
// FBP/transform.cu, FDK/GPURecon_GPU.cu), so that those sources compile with
// g++ and run unchanged on the CPU.  TEST INFRASTRUCTURE ONLY: it builds the
// executed-reference checker; no product code includes it.
//
// What it provides, and how each piece behaves:
//  - __global__/__device__/__host__/__constant__ expand to nothing; a
//    __shared__ variable becomes a static thread_local (one block runs at a
//    time on a host thread, so each block sees its own copy).
//  - A launch `k<<<g, b>>>(args)` is rewritten by the build recipe (text
//    only) into `::ctref::launch(&k, g, b)(args)`.  Blocks run in parallel on
//    OpenMP threads; the threads of a block run as cooperative fibers, in
//    index order, switching only at __syncthreads(): a valid CUDA schedule.
//  - Device memory is host memory.  cudaMalloc returns zero-filled memory
//    with 64 KiB of zeroed slack past the end (the reference's FP ray-table
//    kernel writes up to 63 floats past its arrays, FP/transform.cu:152,178).
//  - Texture references keep their bound array; tex1D/tex2D filter it with
//    the GPU texture unit's linear-filter rule (oracle/texture_rule.h).
//  - floor() in kernel sources returns a value whose conversion to int
//    follows the GPU's float-to-int conversion (NaN -> 0, saturating), since
//    FP/transform.cu:92 converts floor(NaN) for rays that miss the FOV.
#pragma once

#include <algorithm>
#include <assert.h>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <math.h>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>

extern "C" {
#include "../../texture_rule.h"
}

#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__ static thread_local
#define __forceinline__ inline

struct uint3 {
    unsigned x, y, z;
};
struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

inline thread_local uint3 threadIdx;
inline thread_local uint3 blockIdx;
inline thread_local dim3 blockDim;
inline thread_local dim3 gridDim;

// ---- runtime types --------------------------------------------------------
enum cudaError_t {
    cudaSuccess = 0,
    cudaErrorInvalidValue = 1,
    cudaErrorMemoryAllocation = 2,
    cudaErrorNotSupported = 801
};
typedef cudaError_t cudaError;
enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3,
    cudaMemcpyDefault = 4
};
enum cudaTextureAddressMode {
    cudaAddressModeWrap = 0,
    cudaAddressModeClamp = 1,
    cudaAddressModeMirror = 2,
    cudaAddressModeBorder = 3
};
enum cudaTextureFilterMode { cudaFilterModePoint = 0, cudaFilterModeLinear = 1 };
enum cudaTextureReadMode { cudaReadModeElementType = 0, cudaReadModeNormalizedFloat = 1 };
enum cudaChannelFormatKind {
    cudaChannelFormatKindSigned = 0,
    cudaChannelFormatKindUnsigned = 1,
    cudaChannelFormatKindFloat = 2
};
struct cudaChannelFormatDesc {
    int x, y, z, w;
    cudaChannelFormatKind f;
};
inline cudaChannelFormatDesc cudaCreateChannelDesc(int x, int y, int z, int w,
                                                   cudaChannelFormatKind f) {
    return cudaChannelFormatDesc{x, y, z, w, f};
}
struct cudaDeviceProp {
    char name[256];
    int major, minor, multiProcessorCount;
};

// A cudaArray of fp32 texels: width x height x depth, row-major.
struct cudaArray {
    float *data;
    size_t w, h, d;
};
typedef cudaArray *cudaArray_t;

struct cudaPitchedPtr {
    void *ptr;
    size_t pitch, xsize, ysize;
};
struct cudaExtent {
    size_t width, height, depth;
};
struct cudaPos {
    size_t x, y, z;
};
struct cudaMemcpy3DParms {
    cudaArray *srcArray;
    cudaPos srcPos;
    cudaPitchedPtr srcPtr;
    cudaArray *dstArray;
    cudaPos dstPos;
    cudaPitchedPtr dstPtr;
    cudaExtent extent;
    cudaMemcpyKind kind;
};
inline cudaPitchedPtr make_cudaPitchedPtr(void *p, size_t pitch, size_t xs, size_t ys) {
    return cudaPitchedPtr{p, pitch, xs, ys};
}
inline cudaExtent make_cudaExtent(size_t w, size_t h, size_t d) { return cudaExtent{w, h, d}; }
inline cudaPos make_cudaPos(size_t x, size_t y, size_t z) { return cudaPos{x, y, z}; }

namespace ctref {

constexpr size_t kSlack = 65536;

[[noreturn]] void fail(const std::string &what);
void barrier();
void run_grid(const dim3 &grid, const dim3 &block, void (*body)(void *), void *ctx);

// GPU float-to-int conversion (round toward zero, NaN -> 0, saturating).
inline int gpu_f2i(double v) {
    if (!(v == v)) return 0;
    if (v >= 2147483647.0) return 2147483647;
    if (v <= -2147483648.0) return (-2147483647 - 1);
    return (int)v;
}

struct DevFloor {
    float v;
    explicit operator int() const { return gpu_f2i(v); }
    explicit operator float() const { return v; }
    explicit operator double() const { return v; }
};
inline DevFloor dev_floor(float x) { return DevFloor{std::floor(x)}; }

template <class F>
struct Launch;

template <class... P>
struct Launch<void (*)(P...)> {
    void (*k)(P...);
    dim3 g, b;
    template <class... A>
    void operator()(A &&...a) const {
        std::tuple<P...> args(std::forward<A>(a)...);  // by-value kernel parameters
        struct Ctx {
            void (*k)(P...);
            std::tuple<P...> *args;
        } c{k, &args};
        run_grid(g, b, [](void *p) {
            Ctx *cx = static_cast<Ctx *>(p);
            std::apply(cx->k, *cx->args);
        }, &c);
    }
};

template <class... P>
Launch<void (*)(P...)> launch(void (*k)(P...), dim3 g, dim3 b, size_t shmem = 0,
                              void *stream = nullptr) {
    if (shmem != 0 || stream != nullptr) fail("launch with dynamic shared memory or a stream");
    return Launch<void (*)(P...)>{k, g, b};
}

}  // namespace ctref

inline void __syncthreads() { ctref::barrier(); }

// ---- memory ---------------------------------------------------------------
inline cudaError_t cudaMalloc(void **p, size_t n) {
    *p = std::calloc(1, n + ctref::kSlack);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
inline cudaError_t cudaFree(void *p) {
    std::free(p);
    return cudaSuccess;
}
inline cudaError_t cudaMemset(void *p, int v, size_t n) {
    std::memset(p, v, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemcpy(void *dst, const void *src, size_t n, cudaMemcpyKind) {
    std::memmove(dst, src, n);
    return cudaSuccess;
}
template <class T>
cudaError_t cudaMemcpyToSymbol(T &sym, const void *src, size_t n, size_t off = 0,
                               cudaMemcpyKind = cudaMemcpyHostToDevice) {
    if (off + n > sizeof(T)) return cudaErrorInvalidValue;
    std::memcpy(reinterpret_cast<char *>(&sym) + off, src, n);
    return cudaSuccess;
}
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
inline cudaError_t cudaGetDevice(int *d) {
    *d = 0;
    return cudaSuccess;
}
inline cudaError_t cudaGetDeviceProperties(cudaDeviceProp *p, int) {
    std::memset(p, 0, sizeof(*p));
    std::strcpy(p->name, "host stand-in");
    return cudaSuccess;
}
inline const char *cudaGetErrorString(cudaError_t e) {
    switch (e) {
        case cudaSuccess: return "no error";
        case cudaErrorInvalidValue: return "invalid argument";
        case cudaErrorMemoryAllocation: return "out of memory";
        case cudaErrorNotSupported: return "not supported by the host stand-in";
    }
    return "unknown error";
}

inline cudaError_t cudaMallocArray(cudaArray **a, const cudaChannelFormatDesc *d, size_t w,
                                   size_t h = 0, unsigned = 0) {
    if (d->x != 32 || d->y || d->z || d->w || d->f != cudaChannelFormatKindFloat)
        return cudaErrorNotSupported;
    cudaArray *r = new cudaArray{nullptr, w, h ? h : 1, 1};
    r->data = static_cast<float *>(std::calloc(r->w * r->h, sizeof(float)));
    *a = r;
    return cudaSuccess;
}
inline cudaError_t cudaFreeArray(cudaArray *a) {
    if (a) {
        std::free(a->data);
        delete a;
    }
    return cudaSuccess;
}
// wOffset in bytes, hOffset in rows, count in bytes (row-major fill).
inline cudaError_t cudaMemcpyToArray(cudaArray *a, size_t wOffset, size_t hOffset,
                                     const void *src, size_t count, cudaMemcpyKind) {
    const size_t off = hOffset * a->w * sizeof(float) + wOffset;
    if (off + count > a->w * a->h * a->d * sizeof(float)) return cudaErrorInvalidValue;
    std::memcpy(reinterpret_cast<char *>(a->data) + off, src, count);
    return cudaSuccess;
}
inline cudaError_t cudaMemcpy3D(const cudaMemcpy3DParms *) { return cudaErrorNotSupported; }

// ---- texture references ---------------------------------------------------
template <class T, int Dim = 1, cudaTextureReadMode Mode = cudaReadModeElementType>
struct texture {
    cudaTextureAddressMode addressMode[3] = {cudaAddressModeClamp, cudaAddressModeClamp,
                                             cudaAddressModeClamp};
    cudaTextureFilterMode filterMode = cudaFilterModePoint;
    int normalized = 0;
    const cudaArray *array = nullptr;
};

template <class T, int Dim, cudaTextureReadMode Mode>
cudaError_t cudaBindTextureToArray(texture<T, Dim, Mode> &t, const cudaArray *a,
                                   const cudaChannelFormatDesc &) {
    t.array = a;
    return cudaSuccess;
}
template <class T, int Dim, cudaTextureReadMode Mode>
cudaError_t cudaUnbindTexture(texture<T, Dim, Mode> &t) {
    t.array = nullptr;
    return cudaSuccess;
}

namespace ctref {
template <class T, int Dim, cudaTextureReadMode Mode>
const cudaArray *checked(const texture<T, Dim, Mode> &t, int axes) {
    if (!t.array) fail("fetch from an unbound texture");
    if (t.filterMode != cudaFilterModeLinear || t.normalized)
        fail("only linear filtering with unnormalised coordinates is emulated");
    for (int k = 0; k < axes; ++k)
        if (t.addressMode[k] != cudaAddressModeClamp) fail("only clamp addressing is emulated");
    return t.array;
}
}  // namespace ctref

template <cudaTextureReadMode Mode>
inline float tex1D(const texture<float, 1, Mode> &t, float x) {
    const cudaArray *a = ctref::checked(t, 1);
    return ctex_fetch1d(a->data, (int)a->w, x);
}
template <cudaTextureReadMode Mode>
inline float tex2D(const texture<float, 2, Mode> &t, float x, float y) {
    const cudaArray *a = ctref::checked(t, 2);
    return ctex_fetch2d(a->data, (int)a->w, (int)a->h, x, y);
}
template <cudaTextureReadMode Mode>
inline float tex3D(const texture<float, 3, Mode> &, float, float, float) {
    ctref::fail("3-D texture fetches are not on the operators' path");
}

// The reference's kernel sources are compiled with CTREF_KERNEL_SOURCE, so
// that only they see the GPU conversion semantics of floor().
#ifdef CTREF_KERNEL_SOURCE
#define floor(x) ::ctref::dev_floor(x)
#endif
