// store_acc.cuh -- FP64 values of the distributions in and out of a block's
// stored form (FP64 f, or the offsets g = f - w_i in FP32, FP16, BF16), for
// the kernels that touch a few face cells of any form (block refinement).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "fsi_common.cuh"
#include "../../include/fsi_gpu.h"

namespace fsi {

template <int P> struct FAcc;
template <> struct FAcc<FSI_PREC_F64> {
    static __device__ __forceinline__ double load(const void *f, long long i, int) { return ((const double *)f)[i]; }
    static __device__ __forceinline__ void store(void *f, long long i, int, double v) { ((double *)f)[i] = v; }
};
template <> struct FAcc<FSI_PREC_F64_FAST> : FAcc<FSI_PREC_F64> {};
template <> struct FAcc<FSI_PREC_F32> {
    static __device__ __forceinline__ double load(const void *f, long long i, int q) {
        return (double)((const float *)f)[i] + wt_(q);
    }
    static __device__ __forceinline__ void store(void *f, long long i, int q, double v) {
        ((float *)f)[i] = (float)(v - wt_(q));
    }
};
template <> struct FAcc<FSI_PREC_F16> {
    static __device__ __forceinline__ double load(const void *f, long long i, int q) {
        return (double)__half2float(((const __half *)f)[i]) + wt_(q);
    }
    static __device__ __forceinline__ void store(void *f, long long i, int q, double v) {
        ((__half *)f)[i] = __float2half_rn((float)(v - wt_(q)));
    }
};
template <> struct FAcc<FSI_PREC_BF16> {
    static __device__ __forceinline__ double load(const void *f, long long i, int q) {
        return (double)__bfloat162float(((const __nv_bfloat16 *)f)[i]) + wt_(q);
    }
    static __device__ __forceinline__ void store(void *f, long long i, int q, double v) {
        ((__nv_bfloat16 *)f)[i] = __float2bfloat16_rn((float)(v - wt_(q)));
    }
};

// tau_all of a cell: FP64 array, FP32 array (offset forms) or the uniform tau
struct TauSrc {
    double tau;
    const double *d;
    const float *f;
    __device__ __forceinline__ double at(long long c) const { return d ? d[c] : (f ? (double)f[c] : tau); }
};

}  // namespace fsi
