// mex_stub.cpp -- TEST STUB implementation of the mex/mxGPU calls used by the
// MEX entry, plus a harness that builds the reference MEX's eight inputs
// (assistMatlabCuda.m:1-17) around caller-owned device buffers, calls
// mexFunction and copies plhs[0] out.  Built into libmemd_mex_stub.so for the
// tests only.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpu/mxGPUArray.h"
#include "mex.h"

struct mxArray_tag {
    mxClassID cls = mxUNKNOWN_CLASS;
    std::vector<mwSize> dims;
    void* host = nullptr;   // scalars live on the host
    void* dev = nullptr;    // gpuArrays live on the device
    bool owns_dev = false;
};
struct mxGPUArray_tag {
    mxClassID cls = mxUNKNOWN_CLASS;
    mxComplexity cx = mxREAL;
    std::vector<mwSize> dims;
    void* dev = nullptr;
    bool owns = false;
};

static size_t elem_size(mxClassID c) { return c == mxDOUBLE_CLASS ? 8 : 4; }
static size_t numel(const std::vector<mwSize>& d)
{
    size_t n = 1;
    for (mwSize v : d) n *= v;
    return n;
}

static std::string g_last;
static std::vector<void (*)(void)> g_exit;

extern "C" {
void* mxGetData(const mxArray* a) { return a->host; }
mxClassID mxGetClassID(const mxArray* a) { return a->cls; }
size_t mxGetNumberOfElements(const mxArray* a) { return numel(a->dims); }
void mxFree(void* p) { std::free(p); }
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw std::runtime_error(std::string(id) + ": " + buf);
}
int mexAtExit(void (*fn)(void))
{
    g_exit.push_back(fn);
    return 0;
}
int mxInitGPU(void) { return 0; }
mxGPUArray const* mxGPUCreateFromMxArray(mxArray const* a)
{
    mxGPUArray* g = new mxGPUArray_tag();
    g->cls = a->cls;
    g->dims = a->dims;
    g->dev = a->dev;
    return g;
}
void const* mxGPUGetDataReadOnly(mxGPUArray const* g) { return g->dev; }
void* mxGPUGetData(mxGPUArray* g) { return g->dev; }
mxGPUArray* mxGPUCreateGPUArray(mwSize ndims, mwSize const* dims, mxClassID cid, mxComplexity ccx, mxGPUInitialize init)
{
    mxGPUArray* g = new mxGPUArray_tag();
    g->cls = cid;
    g->cx = ccx;
    g->dims.assign(dims, dims + ndims);
    const size_t bytes = numel(g->dims) * elem_size(cid);
    if (cudaMalloc(&g->dev, bytes ? bytes : 4) != cudaSuccess) throw std::runtime_error("stub: cudaMalloc");
    if (init == MX_GPU_INITIALIZE_VALUES) cudaMemset(g->dev, 0, bytes);
    g->owns = true;
    return g;
}
mwSize mxGPUGetNumberOfDimensions(mxGPUArray const* g) { return (mwSize)g->dims.size(); }
mwSize const* mxGPUGetDimensions(mxGPUArray const* g)
{
    mwSize* d = (mwSize*)std::malloc(sizeof(mwSize) * g->dims.size());
    std::memcpy(d, g->dims.data(), sizeof(mwSize) * g->dims.size());
    return d;
}
mxClassID mxGPUGetClassID(mxGPUArray const* g) { return g->cls; }
mxComplexity mxGPUGetComplexity(mxGPUArray const* g) { return g->cx; }
mwSize mxGPUGetNumberOfElements(mxGPUArray const* g) { return (mwSize)numel(g->dims); }
mxArray* mxGPUCreateMxArrayOnGPU(mxGPUArray const* g)
{
    mxArray* a = new mxArray_tag();
    a->cls = g->cls;
    a->dims = g->dims;
    a->dev = g->dev;
    a->owns_dev = g->owns;
    const_cast<mxGPUArray*>(g)->owns = false;  // the mxArray takes the buffer over
    return a;
}
void mxGPUDestroyGPUArray(mxGPUArray const* g)
{
    if (g->owns) cudaFree(g->dev);
    delete g;
}

// Harness: IMFs = memdMatlabCuda(C, K, nimf, maxit, data, index, primes, template)
// d_data: L*C floats, d_index: L ints, d_primes: C ints, d_out: nimf*C*L floats.
int mex_stub_call(int C, int K, int nimf, int maxit, const float* d_data, long L, const int* d_index,
                  const int* d_primes, float* d_out)
{
    mxArray s[4];
    int v[4] = {C, K, nimf, maxit};
    for (int i = 0; i < 4; ++i) {
        s[i].cls = mxINT32_CLASS;
        s[i].dims = {1, 1};
        s[i].host = &v[i];
    }
    mxArray data, index, primes, tmpl;
    data.cls = mxSINGLE_CLASS;
    data.dims = {(mwSize)L, (mwSize)C};
    data.dev = (void*)d_data;
    index.cls = mxINT32_CLASS;
    index.dims = {1, (mwSize)L};
    index.dev = (void*)d_index;
    primes.cls = mxINT32_CLASS;
    primes.dims = {1, (mwSize)C};
    primes.dev = (void*)d_primes;
    tmpl.cls = mxSINGLE_CLASS;
    tmpl.dims = {(mwSize)L, (mwSize)C, (mwSize)nimf};
    tmpl.dev = d_out;  // only its size and class matter
    mxArray const* prhs[8] = {&s[0], &s[1], &s[2], &s[3], &data, &index, &primes, &tmpl};
    mxArray* plhs[1] = {nullptr};
    try {
        mexFunction(1, plhs, 8, prhs);
    } catch (const std::exception& e) {
        g_last = e.what();
        return 1;
    }
    cudaMemcpy(d_out, plhs[0]->dev, sizeof(float) * (size_t)nimf * C * L, cudaMemcpyDeviceToDevice);
    if (plhs[0]->owns_dev) cudaFree(plhs[0]->dev);
    delete plhs[0];
    return 0;
}

const char* mex_stub_last_error(void) { return g_last.c_str(); }

void mex_stub_at_exit(void)
{
    for (auto fn : g_exit) fn();
    g_exit.clear();
}
}
