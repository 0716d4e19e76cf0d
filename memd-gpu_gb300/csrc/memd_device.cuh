// memd_device.cuh -- device-side types and helpers shared by the MEMD kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "memd_gb300.h"

namespace memd {

// Spline solution and knot value of one (direction, envelope, knot, channel):
// written by the tridiagonal solve, read by the envelope evaluation.
template <typename real>
struct alignas(2 * sizeof(real)) SY {
    real s;   // half the second derivative at the knot (the solve's unknown)
    real y;   // knot value after the end-point clamp
};

// Channel-independent factorisation of the natural-spline system of one
// (direction, envelope), per knot row i (Thomas elimination without pivoting):
//   g_i = d_i - l_i * cp_{i-1};  m = 1/g_i;  lm = l_i/g_i;  cp = u_i/g_i;
//   ih = 1 / (x_{i+1} - x_i)  (0 for the last row).
template <typename real>
struct alignas(4 * sizeof(real)) Fac {
    real m, lm, cp, ih;
};

// Geometry of one record (or the widest epoch of a batch).
struct Geom {
    int C;      // channels
    int L;      // samples
    int K;      // directions (all chunks)
    int W;      // 32-bit words per direction bitmask = ceil(L / 32)
    int cap;    // knot capacity per (direction, envelope)
    int cov;    // last interior sample tested for extrema
};

// Per-run device state (counters and sticky flags).
struct RunState {
    int flags;                 // MEMD_FLAG_* bits
    int n_imfs;                // IMFs written so far
    int sifts[64];             // sifts per IMF
    int nbit;                  // stop mode: sifts applied to the current IMF
    int pass;                  // stop mode: envelope passes of the current IMF
    int imf_done;              // stop mode: the residual has too few extrema
    int apply;                 // stop mode: subtract the mean of the last pass
    unsigned long long over1;  // stop mode: samples with sigma > sd in the last pass
    unsigned long long over2;  // stop mode: samples with sigma > sd2 in the last pass
    int q;                     // qualified directions of the last pass
    int trace_row;             // stop mode: trace row of the current pass (-1: none)
    int pad[4];                // [0] passes over the run, [1] sift loop continues,
                               // [2] IMF loop continues (mirrors of the graph conditions)
};

__device__ __forceinline__ uint64_t splitmix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// fma with an explicit rounding mode so that the compiler's contraction
// choices never change results between builds.
__device__ __forceinline__ double fmad_(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fmad_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double mul_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double sub_(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float sub_(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double div_(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_(float a, float b) { return __fdiv_rn(a, b); }

}  // namespace memd
