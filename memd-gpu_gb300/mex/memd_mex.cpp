// memd_mex.cpp -- MATLAB entry with the reference MEX's interface
// (memdMatlabCuda.cu:996-1347, usage assistMatlabCuda.m:1-17), running the
// decomposition through libmemd_gb300.so.
//
//   IMFs = memdMatlabCuda(signalDim, numDirVector, numIMFs, maxiter, data,
//                         samplesIndex, primesSet, outputData)
//
//   signalDim, numDirVector, numIMFs, maxiter   int32 scalars (prhs[0..3])
//   data          single gpuArray, L x signalDim (channel c is column c, so
//                 the memory is channel-major, MEX:1019-1039)        prhs[4]
//   samplesIndex  int32 gpuArray 0..L-1                              prhs[5]
//   primesSet     int32 gpuArray, the first signalDim primes (the
//                 direction set's bases, MEX:1131-1152)             prhs[6]
//   outputData    single gpuArray (L, signalDim, numIMFs): only its size
//                 and class are used (MEX:1031-1036)                 prhs[7]
//   IMFs          new single gpuArray of outputData's size; IMF i is
//                 IMFs(:, :, i), the residual is IMFs(:, :, numIMFs) plhs[0]
//
// Build (MATLAB):  mexcuda -output memdMatlabCuda memd_mex.cpp
//                  -I<repo>/include -L<repo>/memd-gpu_gb300/lib -lmemd_gb300
// The precision form is FP32 (the reference's) unless the environment
// variable MEMD_MEX_FORM=mixed selects the mixed-precision form.  Unlike the
// reference, the arguments are checked and errors are raised as MATLAB errors,
// and the workspace is kept between calls of the same size.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <vector>

#include "gpu/mxGPUArray.h"
#include "mex.h"
#include "memd_gb300.h"

namespace {

memd_plan* g_plan = nullptr;
memd_config g_cfg;

void release_plan()
{
    if (g_plan) memd_plan_destroy(g_plan);
    g_plan = nullptr;
}

int scalar_int32(mxArray const* a, const char* what)
{
    if (!a || mxGetClassID(a) != mxINT32_CLASS || mxGetNumberOfElements(a) != 1)
        mexErrMsgIdAndTxt("memd:args", "%s must be an int32 scalar", what);
    return *(int const*)mxGetData(a);
}

}  // namespace

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, mxArray const* prhs[])
{
    (void)nlhs;
    if (nrhs != 8) mexErrMsgIdAndTxt("memd:args", "expected 8 inputs, got %d", nrhs);
    mxInitGPU();
    const int C = scalar_int32(prhs[0], "signalDim");
    const int K = scalar_int32(prhs[1], "numDirVector");
    const int nimf = scalar_int32(prhs[2], "numIMFs");
    const int maxit = scalar_int32(prhs[3], "maxiter");
    if (C < 1 || K < 1 || nimf < 1 || maxit < 0) mexErrMsgIdAndTxt("memd:args", "sizes must be positive");

    mxGPUArray const* data = mxGPUCreateFromMxArray(prhs[4]);
    mxGPUArray const* index = mxGPUCreateFromMxArray(prhs[5]);
    mxGPUArray const* primes = mxGPUCreateFromMxArray(prhs[6]);
    mxGPUArray const* tmpl = mxGPUCreateFromMxArray(prhs[7]);
    if (mxGPUGetClassID(data) != mxSINGLE_CLASS || mxGPUGetClassID(tmpl) != mxSINGLE_CLASS)
        mexErrMsgIdAndTxt("memd:args", "data and outputData must be single gpuArrays");
    if (mxGPUGetClassID(index) != mxINT32_CLASS || mxGPUGetClassID(primes) != mxINT32_CLASS)
        mexErrMsgIdAndTxt("memd:args", "samplesIndex and primesSet must be int32 gpuArrays");
    const int64_t numel = (int64_t)mxGPUGetNumberOfElements(data);
    const int64_t L = numel / C;  // MEX:1038-1039
    if (L * C != numel) mexErrMsgIdAndTxt("memd:args", "numel(data) is not a multiple of signalDim");
    if ((int64_t)mxGPUGetNumberOfElements(index) != L) mexErrMsgIdAndTxt("memd:args", "samplesIndex must have L entries");
    if ((int64_t)mxGPUGetNumberOfElements(primes) < C) mexErrMsgIdAndTxt("memd:args", "primesSet needs signalDim entries");
    if ((int64_t)mxGPUGetNumberOfElements(tmpl) != (int64_t)nimf * C * L)
        mexErrMsgIdAndTxt("memd:args", "outputData must have L*signalDim*numIMFs elements");

    mwSize const* dims = mxGPUGetDimensions(tmpl);
    mxGPUArray* out = mxGPUCreateGPUArray(mxGPUGetNumberOfDimensions(tmpl), dims, mxGPUGetClassID(tmpl),
                                          mxGPUGetComplexity(tmpl), MX_GPU_DO_NOT_INITIALIZE);
    mxFree((void*)dims);
    const mwSize ddims[2] = {(mwSize)C, (mwSize)K};  // K x C row-major = C x K column-major
    mxGPUArray* dirs = mxGPUCreateGPUArray(2, ddims, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);

    // direction set from the caller's primes, as the reference MEX does
    std::vector<int32_t> hp((size_t)C);
    cudaMemcpy(hp.data(), mxGPUGetDataReadOnly(primes), sizeof(int32_t) * (size_t)C, cudaMemcpyDeviceToHost);
    if (memd_directions_f32(C, K, hp.data(), (float*)mxGPUGetData(dirs), nullptr) != MEMD_OK)
        mexErrMsgIdAndTxt("memd:cuda", "direction set: %s", memd_last_error());

    memd_config cfg;
    memd_default_config(&cfg);
    cfg.channels = C;
    cfg.length = L;
    cfg.directions = K;
    cfg.num_imfs = nimf;
    cfg.max_iter = maxit;
    const char* form = std::getenv("MEMD_MEX_FORM");
    cfg.precision = (form && std::strcmp(form, "mixed") == 0) ? MEMD_PREC_MIXED : MEMD_PREC_F32;
    if (!g_plan || g_cfg.channels != cfg.channels || g_cfg.length != cfg.length || g_cfg.directions != cfg.directions ||
        g_cfg.num_imfs != cfg.num_imfs || g_cfg.max_iter != cfg.max_iter || g_cfg.precision != cfg.precision) {
        release_plan();
        if (memd_plan_create(&cfg, &g_plan) != MEMD_OK)
            mexErrMsgIdAndTxt("memd:plan", "plan: %s", memd_last_error());
        g_cfg = cfg;
        mexAtExit(release_plan);
    }
    if (memd_run_f32(g_plan, (int32_t const*)mxGPUGetDataReadOnly(index), (float const*)mxGPUGetDataReadOnly(data),
                     (float const*)mxGPUGetDataReadOnly(dirs), (float*)mxGPUGetData(out), nullptr, nullptr) != MEMD_OK)
        mexErrMsgIdAndTxt("memd:run", "decomposition: %s", memd_last_error());
    cudaDeviceSynchronize();

    plhs[0] = mxGPUCreateMxArrayOnGPU(out);
    mxGPUDestroyGPUArray(data);
    mxGPUDestroyGPUArray(index);
    mxGPUDestroyGPUArray(primes);
    mxGPUDestroyGPUArray(tmpl);
    mxGPUDestroyGPUArray(dirs);
    mxGPUDestroyGPUArray(out);
}
