// texture_probe.cu -- fetches through a real GPU texture object with the
// reference's sampler state (cudaFilterModeLinear, cudaAddressModeClamp,
// unnormalised coordinates, fp32 texels), so that the texture-unit rule the
// oracle and the executed reference use (oracle/texture_rule.h) can be held
// against the hardware.  TEST INFRASTRUCTURE ONLY: make_golden_texture.py and
// the GPU texture test load it; no product code does.
//
// Every fetch is in bounds by construction: the texture unit clamps any
// coordinate to the array, and the kernel guards its index against n.
#include <cuda_runtime.h>

namespace {

__global__ void fetch_kernel(cudaTextureObject_t t, const float *x, const float *y, float *out,
                             int n, int two_d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = two_d ? tex2D<float>(t, x[i], y[i]) : tex1D<float>(t, x[i]);
}

}  // namespace

// table: h rows of w fp32 texels (h = 0 for a 1-D texture); x, y, out: n
// values in host memory (y unused in 1-D).  Returns a cudaError_t code.
extern "C" int texprobe_fetch(const float *table, int w, int h, const float *x, const float *y,
                              float *out, int n) {
    if (w <= 0 || h < 0 || n <= 0) return (int)cudaErrorInvalidValue;
    const int two_d = h > 0;
    const int rows = two_d ? h : 1;
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    float *dx = nullptr, *dy = nullptr, *dout = nullptr;
    cudaError_t e;
    cudaChannelFormatDesc d = cudaCreateChannelDesc(32, 0, 0, 0, cudaChannelFormatKindFloat);
    do {
        if ((e = cudaMallocArray(&arr, &d, w, two_d ? h : 0)) != cudaSuccess) break;
        if ((e = cudaMemcpy2DToArray(arr, 0, 0, table, w * sizeof(float), w * sizeof(float),
                                     rows, cudaMemcpyHostToDevice)) != cudaSuccess)
            break;
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr;
        cudaTextureDesc td = {};
        td.addressMode[0] = td.addressMode[1] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModeLinear;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        if ((e = cudaCreateTextureObject(&tex, &rd, &td, nullptr)) != cudaSuccess) break;
        const size_t bytes = (size_t)n * sizeof(float);
        if ((e = cudaMalloc(&dx, bytes)) != cudaSuccess) break;
        if ((e = cudaMalloc(&dy, bytes)) != cudaSuccess) break;
        if ((e = cudaMalloc(&dout, bytes)) != cudaSuccess) break;
        if ((e = cudaMemcpy(dx, x, bytes, cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((e = cudaMemcpy(dy, two_d ? y : x, bytes, cudaMemcpyHostToDevice)) != cudaSuccess)
            break;
        fetch_kernel<<<(n + 255) / 256, 256>>>(tex, dx, dy, dout, n, two_d);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        e = cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost);
    } while (0);
    if (tex) cudaDestroyTextureObject(tex);
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(dout);
    if (arr) cudaFreeArray(arr);
    return (int)e;
}
