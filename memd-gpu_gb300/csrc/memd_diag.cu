// memd_diag.cu -- FMA pipe rate of the GPU in use (roofline denominators for
// the CUDA-core kernels; the HBM and tensor denominators come from the
// pool's measured copy and GEMM figures).
#include <cuda_runtime.h>

#include "memd_device.cuh"
#include "memd_internal.h"

namespace memd {

// 8 independent fma chains per thread; the result is stored so the compiler
// keeps every operation.  flops = 2 * 8 * iters per thread.
template <typename real>
__global__ void __launch_bounds__(256) k_fma_rate(real* out, int iters, real a, real b)
{
    real x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = real(threadIdx.x + j);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = fmad_(x[j], a, b);
    }
    real s = real(0);
#pragma unroll
    for (int j = 0; j < 8; ++j) s += x[j];
    if (s == real(-1.2345)) out[threadIdx.x] = s;
}

template <typename real>
static memd_status fma_rate(double* flops_per_s)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    real* out = nullptr;
    if (cudaMalloc((void**)&out, 256 * sizeof(real)) != cudaSuccess) return set_cuda_error("diag: alloc");
    const int blocks = sms * 8;
    const int iters = sizeof(real) == 8 ? 2048 : 65536;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma_rate<real><<<blocks, 256>>>(out, iters / 8, real(0.999), real(1e-3));
    cudaEventRecord(e0);
    k_fma_rate<real><<<blocks, 256>>>(out, iters, real(0.999), real(1e-3));
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return set_cuda_error("diag: run", e);
    *flops_per_s = 2.0 * 8.0 * (double)iters * (double)blocks * 256.0 / (ms * 1e-3);
    return MEMD_OK;
}

}  // namespace memd

extern "C" memd_status memd_diag_fma_rate(int32_t precision, double* flops_per_s)
{
    if (!flops_per_s) return memd::set_error(MEMD_ERR_INVALID, "diag: null output");
    return precision == MEMD_PREC_F64 ? memd::fma_rate<double>(flops_per_s) : memd::fma_rate<float>(flops_per_s);
}
