// memd_directions.cu -- Hammersley direction sets on the device.
//
// Restates the reference's direction generator (memReducedEpochs_dev.cu
// GenerateDirectionVector :1029-1072 with RadicalInverse :934-946,
// Sequence2Vector :948-990, GenerateHammSeq :992-1005, isPrimes :1014-1027;
// MEX variant memdMatlabCuda.cu:1131-1152 with the caller's prime table):
//   coordinate 0 of direction k:  (k + 1.5) / (-p[0])   (double, then real)
//   coordinate c >= 1:            radical inverse of k+1 in base p[c], in float
//   s = 2 h - 1;  theta_i = atan2(sqrt(sum_{j>i} s_j^2), s_i)
//   dir = (cos t0, sin t0 cos t1, ..., prod_{j<C-1} sin t_j)
// The standalone table is p = {-K, 2, 3, 5, 7, ...} (first C-1 primes).
#include <cuda_runtime.h>

#include <cstdlib>
#include <vector>

#include "memd_device.cuh"
#include "memd_internal.h"

namespace memd {

__device__ __forceinline__ float radical_inverse(int base, unsigned i)
{
    float digit, radical, inv;
    digit = radical = (float)(1.0 / (double)base);
    inv = 0.0f;
    while (i) {
        inv = __fmaf_rn(digit, (float)(i % (unsigned)base), inv);
        digit = __fmul_rn(digit, radical);
        i /= (unsigned)base;
    }
    return inv;
}

// One thread per direction; the output row doubles as scratch for the
// sequence and the angles (dir[k*C + c]).
template <typename real>
__global__ void k_directions(const int* __restrict__ primes, int C, int K, real* __restrict__ dir)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    real* v = dir + (size_t)k * C;
    v[0] = real(((double)(unsigned)k + 1.5) / (double)(-primes[0]));
    for (int c = 1; c < C; ++c) v[c] = real(radical_inverse(primes[c], (unsigned)(k + 1)));
    for (int c = 0; c < C; ++c) v[c] = fmad_(real(2), v[c], real(-1));
    if (C == 1) {
        // one coordinate: no angles, the vector is the constant 1 (REF:969-974)
        v[0] = real(1);
        return;
    }
    // angles, last to first: tem_i = sum_{j = C-1 .. i+1} s_j^2 accumulated
    // from the end, exactly the order the reference sums in.
    real carry = v[C - 1];
    real tem = real(0);
    for (int i = C - 2; i >= 0; --i) {
        tem = fmad_(carry, carry, tem);
        const real si = v[i];
        v[i] = atan2(sqrt(tem), si);
        carry = si;
    }
    real prod = real(1);
    for (int i = 0; i < C - 1; ++i) {
        const real th = v[i];
        v[i] = mul_(prod, cos(th));
        prod = mul_(prod, sin(th));
    }
    v[C - 1] = prod;
}

void prime_table(int C, int K, std::vector<int>& p)
{
    p.assign((size_t)C, 0);
    int cnt = 1, cand = 2;
    while (cnt < C) {
        bool composite = false;
        for (int d = 2; d <= cand / 2; ++d)
            if (cand % d == 0) { composite = true; break; }
        if (!composite) p[(size_t)cnt++] = cand;
        ++cand;
    }
    p[0] = -K;
}

template <typename real>
static memd_status directions_impl(int64_t C, int64_t K, const int32_t* primes, real* d_dir, void* stream)
{
    if (C < 1 || K < 1 || C > 4096 || K > (1 << 20) || !d_dir) return set_error(MEMD_ERR_INVALID, "directions: bad arguments");
    std::vector<int> p;
    if (primes) p.assign(primes, primes + C);
    else prime_table((int)C, (int)K, p);
    if (p[0] == 0) return set_error(MEMD_ERR_INVALID, "directions: primes[0] must be nonzero");
    for (int64_t c = 1; c < C; ++c)
        if (p[(size_t)c] < 2) return set_error(MEMD_ERR_INVALID, "directions: bases must be >= 2");
    cudaStream_t s = (cudaStream_t)stream;
    int* d_p = nullptr;
    // The prime table is tiny; stream-ordered allocation keeps the call free of
    // device-wide synchronisation.
    if (cudaMallocAsync((void**)&d_p, sizeof(int) * (size_t)C, s) != cudaSuccess)
        return set_cuda_error("directions: cudaMallocAsync");
    cudaMemcpyAsync(d_p, p.data(), sizeof(int) * (size_t)C, cudaMemcpyHostToDevice, s);
    k_directions<real><<<(unsigned)((K + 127) / 128), 128, 0, s>>>(d_p, (int)C, (int)K, d_dir);
    cudaError_t e = cudaGetLastError();
    cudaFreeAsync(d_p, s);
    // the host table must outlive the asynchronous copy
    cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_cuda_error("directions: launch", e);
    return MEMD_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant.  The prime table the kernel reads lives in this
// file-scope device array instead of a per-call allocation.  The array holds
// kNoAllocMaxChannels entries on every GPU that loads the library, until the
// process exits.  Host code may not hand the array's name to a kernel (on the
// host it is only a stand-in for the device symbol), so every call looks up
// its device address with cudaGetSymbolAddress, with the caller's device and
// context current.  The lookup allocates nothing and costs a few
// microseconds; an address kept from an earlier call could belong to a
// context that has since been destroyed (cudaDeviceReset, a MATLAB
// reset(gpuDevice) while the MEX file stays loaded) or to another context on
// the same device.
// ---------------------------------------------------------------------------
constexpr int kNoAllocMaxChannels = 4096;
static __device__ __align__(256) int g_noalloc_primes[kNoAllocMaxChannels];

// Device address of g_noalloc_primes in the current context.
static memd_status noalloc_table(int** out)
{
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_primes);
    if (e != cudaSuccess || !ptr) return set_cuda_error("directions_noalloc: cudaGetSymbolAddress", e);
    *out = static_cast<int*>(ptr);
    return MEMD_OK;
}

static memd_status directions_noalloc(int64_t C, int64_t K, const int32_t* primes, double* d_dir, void* stream)
{
    if (C < 1 || K < 1 || K > (1 << 20) || !d_dir) return set_error(MEMD_ERR_INVALID, "directions_noalloc: bad arguments");
    if (C > kNoAllocMaxChannels)
        return set_error(MEMD_ERR_INVALID,
                         "directions_noalloc: channels exceeds the 4096-entry static prime table; use memd_directions_f64");
    // the table is built on the stack: no heap or device allocation anywhere
    int table[kNoAllocMaxChannels];
    if (primes) {
        for (int64_t c = 0; c < C; ++c) table[c] = primes[c];
    } else {
        int cnt = 1, cand = 2;
        while (cnt < C) {
            bool composite = false;
            for (int d = 2; d <= cand / 2; ++d)
                if (cand % d == 0) { composite = true; break; }
            if (!composite) table[cnt++] = cand;
            ++cand;
        }
        table[0] = -(int)K;
    }
    if (table[0] == 0) return set_error(MEMD_ERR_INVALID, "directions_noalloc: primes[0] must be nonzero");
    for (int64_t c = 1; c < C; ++c)
        if (table[c] < 2) return set_error(MEMD_ERR_INVALID, "directions_noalloc: bases must be >= 2");
    int* d_table = nullptr;
    memd_status st = noalloc_table(&d_table);
    if (st != MEMD_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    // From pageable (stack) memory the copy has taken the data by the time it
    // returns, so the table may go out of scope afterwards.  Every entry the
    // kernel reads (0..C-1) is written here, so nothing needs clearing first.
    cudaError_t e = cudaMemcpyAsync(d_table, table, sizeof(int) * (size_t)C, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return set_cuda_error("directions_noalloc: copy of the prime table", e);
    k_directions<double><<<(unsigned)((K + 127) / 128), 128, 0, s>>>(d_table, (int)C, (int)K, d_dir);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error("directions_noalloc: launch", e);
    return MEMD_OK;
}

}  // namespace memd

extern "C" memd_status memd_directions_noalloc_f64(int64_t channels, int64_t directions, const int32_t* primes,
                                                   double* d_dir, void* stream)
{
    return memd::directions_noalloc(channels, directions, primes, d_dir, stream);
}

extern "C" memd_status memd_directions_f64(int64_t channels, int64_t directions, const int32_t* primes,
                                           double* d_dir, void* stream)
{
    return memd::directions_impl<double>(channels, directions, primes, d_dir, stream);
}

extern "C" memd_status memd_directions_f32(int64_t channels, int64_t directions, const int32_t* primes,
                                           float* d_dir, void* stream)
{
    return memd::directions_impl<float>(channels, directions, primes, d_dir, stream);
}
