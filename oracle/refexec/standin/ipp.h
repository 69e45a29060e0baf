// ipp.h stand-in for the executed-reference checker: the two Intel IPP
// signal functions the reference's filters call (FBP/transform.cu:162,171,
// FDK/GPURecon_GPU.cu:77,89,200,212), restated from their documented
// definitions.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstddef>

typedef float Ipp32f;
typedef int IppStatus;
enum { ippStsNoErr = 0, ippStsNullPtrErr = -8, ippStsSizeErr = -6 };

// In place: pSrcDst[i] = pSrcDst[i] * val, in fp32.
inline IppStatus ippsMulC_32f_I(Ipp32f val, Ipp32f *pSrcDst, int len) {
    if (!pSrcDst) return ippStsNullPtrErr;
    if (len <= 0) return ippStsSizeErr;
    for (int i = 0; i < len; ++i) pSrcDst[i] = pSrcDst[i] * val;
    return ippStsNoErr;
}

// Full linear convolution: pDst[n] = sum_k pSrc1[k] pSrc2[n - k] for
// n = 0 .. len1 + len2 - 2.  Summed in double and rounded once (IPP's own
// summation order is not documented).
inline IppStatus ippsConv_32f(const Ipp32f *pSrc1, int len1, const Ipp32f *pSrc2, int len2,
                              Ipp32f *pDst) {
    if (!pSrc1 || !pSrc2 || !pDst) return ippStsNullPtrErr;
    if (len1 <= 0 || len2 <= 0) return ippStsSizeErr;
    for (int n = 0; n < len1 + len2 - 1; ++n) {
        const int k0 = n - (len2 - 1) > 0 ? n - (len2 - 1) : 0;
        const int k1 = n < len1 - 1 ? n : len1 - 1;
        double acc = 0.0;
        for (int k = k0; k <= k1; ++k) acc += (double)pSrc1[k] * (double)pSrc2[n - k];
        pDst[n] = (Ipp32f)acc;
    }
    return ippStsNoErr;
}
