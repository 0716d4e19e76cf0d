// memd_diag.cu -- FMA pipe rate of the GPU in use (roofline denominators for
// the CUDA-core kernels; the HBM and tensor denominators come from the
// pool's measured copy and GEMM figures).
#include <cuda_runtime.h>

#include "memd_device.cuh"
#include "memd_internal.h"
#include "memd_ptx.cuh"

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

// A wait that can never complete: an mbarrier initialised for one arrival that
// no thread makes.  Every thread waits on it with the bounded wait of the
// tensor-core kernels; when the limit runs out the kernel records
// MEMD_FLAG_DEVICE_TIMEOUT and returns, and the context stays usable.
__global__ void k_wait_timeout(int* flags, long long max_clocks)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const bool got = mbar_wait_bounded(&bar, 0u, max_clocks);
    if (__syncthreads_or(!got) && threadIdx.x == 0) atomicOr(flags, MEMD_FLAG_DEVICE_TIMEOUT);
}

}  // namespace memd

extern "C" memd_status memd_diag_wait_timeout(int64_t max_clocks, int32_t* flags)
{
    if (!flags || max_clocks < 1 || max_clocks > (1ll << 32))
        return memd::set_error(MEMD_ERR_INVALID, "diag_wait_timeout: bad arguments");
    int* d = nullptr;
    if (cudaMalloc((void**)&d, sizeof(int)) != cudaSuccess) return memd::set_cuda_error("diag_wait_timeout: alloc");
    cudaMemset(d, 0, sizeof(int));
    memd::k_wait_timeout<<<1, 64>>>(d, (long long)max_clocks);
    int h = 0;
    cudaError_t e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return memd::set_cuda_error("diag_wait_timeout: run", e);
    *flags = h;
    return MEMD_OK;
}

extern "C" memd_status memd_diag_fma_rate(int32_t precision, double* flops_per_s)
{
    if (!flops_per_s) return memd::set_error(MEMD_ERR_INVALID, "diag: null output");
    return precision == MEMD_PREC_F64 ? memd::fma_rate<double>(flops_per_s) : memd::fma_rate<float>(flops_per_s);
}
