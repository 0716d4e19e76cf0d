// memd_device.cuh -- device-side types and helpers shared by the MEMD kernels.
#pragma once

#include <climits>
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "memd_gb300.h"

namespace memd {

// Double-float arithmetic: a value hi + lo with |lo| <= ulp(hi)/2, ~48
// significant bits, computed on the FP32 pipe with error-free transformations
// (Knuth two-sum, fma two-product; Dekker 1971, Shewchuk 1997).  Every
// operation renormalises its result.
struct dd {
    float hi, lo;
    dd() = default;
    __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
    __device__ explicit dd(int v) : hi((float)v), lo((float)(v - (int)(float)v)) {}
    __device__ explicit dd(float v) : hi(v), lo(0.f) {}
    __device__ explicit dd(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
    __device__ explicit operator double() const { return (double)hi + (double)lo; }
    __device__ explicit operator float() const { return hi; }
};
__device__ __forceinline__ dd dd_renorm(float s, float e)
{
    const float h = __fadd_rn(s, e);
    return dd(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ dd operator+(dd a, dd b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    return dd_renorm(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dd operator-(dd a) { return dd(-a.hi, -a.lo); }
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }
__device__ __forceinline__ dd operator*(dd a, dd b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return dd_renorm(p, e);
}
// a * t for a plain float t (exact small integers in the evaluation)
__device__ __forceinline__ dd dd_mulf(dd a, float t)
{
    const float p = __fmul_rn(a.hi, t);
    const float e = __fmaf_rn(a.lo, t, __fmaf_rn(a.hi, t, -p));
    return dd_renorm(p, e);
}
__device__ __forceinline__ dd operator/(dd a, dd b)
{
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const dd r = a - b * dd(q1, 0.f);
    const float q2 = __fdiv_rn(r.hi, b.hi);
    return dd_renorm(q1, q2);
}
__device__ __forceinline__ bool operator>(dd a, dd b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__device__ __forceinline__ bool operator<(dd a, dd b) { return b > a; }
__device__ __forceinline__ dd dd_sqrt(dd a)
{
    if (!(a.hi > 0.f)) return dd(0.f, 0.f);
    const float r = sqrtf(a.hi);
    const dd e = a - dd(r, 0.f) * dd(r, 0.f);
    return dd_renorm(r, __fdiv_rn(e.hi, 2.f * r));
}

// Working-signal storage: double (FP64 path), float (FP32 path) or float2,
// a double-float (hi + lo, |lo| <= ulp(hi)/2) carrying ~48 significant bits
// for the mixed-precision path.  xval() is the value the spline arithmetic of
// type real sees.
template <typename real>
__device__ __forceinline__ real xval(double v) { return real(v); }
template <typename real>
__device__ __forceinline__ real xval(float v) { return real(v); }
template <typename real>
__device__ __forceinline__ real xval(float2 v) { return real(v.x); }
template <>
__device__ __forceinline__ dd xval<dd>(float2 v) { return dd(v.x, v.y); }
template <>
__device__ __forceinline__ dd xval<dd>(double v) { return dd(v); }
template <>
__device__ __forceinline__ dd xval<dd>(float v) { return dd(v); }

// x - m for the three storage types; the double-float version is an
// error-free two-sum followed by renormalisation.
__device__ __forceinline__ double xsub(double x, double m) { return __dsub_rn(x, m); }
__device__ __forceinline__ float xsub(float x, float m) { return __fsub_rn(x, m); }
__device__ __forceinline__ float2 xsub(float2 x, float m)
{
    const float nm = -m;
    const float s = __fadd_rn(x.x, nm);
    const float bb = __fsub_rn(s, x.x);
    const float e = __fadd_rn(__fsub_rn(x.x, __fsub_rn(s, bb)), __fsub_rn(nm, bb));
    const float lo = __fadd_rn(x.y, e);
    const float hi = __fadd_rn(s, lo);
    return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}
// x - y for double-float operands
__device__ __forceinline__ float2 xsub(float2 x, float2 y)
{
    const float s = __fsub_rn(x.x, y.x);
    const float bb = __fsub_rn(s, x.x);
    const float e = __fadd_rn(__fsub_rn(x.x, __fsub_rn(s, bb)), __fsub_rn(-y.x, bb));
    const float lo = __fadd_rn(__fsub_rn(x.y, y.y), e);
    const float hi = __fadd_rn(s, lo);
    return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}
__device__ __forceinline__ float2 xsub(float2 x, dd m)
{
    const dd r = dd(x.x, x.y) - m;
    return make_float2(r.hi, r.lo);
}
template <typename XT> __device__ __forceinline__ XT xzero();
template <> __device__ __forceinline__ double xzero<double>() { return 0.0; }
template <> __device__ __forceinline__ float xzero<float>() { return 0.0f; }
template <> __device__ __forceinline__ float2 xzero<float2>() { return make_float2(0.f, 0.f); }
// conversions between storage and plain types
template <typename T> __device__ __forceinline__ T xfrom(double v);
template <> __device__ __forceinline__ double xfrom<double>(double v) { return v; }
template <> __device__ __forceinline__ float xfrom<float>(double v) { return (float)v; }
template <> __device__ __forceinline__ float2 xfrom<float2>(double v)
{
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
}
template <typename T> __device__ __forceinline__ T xfrom(float v) { return xfrom<T>((double)v); }
template <typename T> __device__ __forceinline__ T xfrom(float2 v);
template <> __device__ __forceinline__ double xfrom<double>(float2 v) { return (double)v.x + (double)v.y; }
template <> __device__ __forceinline__ float xfrom<float>(float2 v) { return v.x; }
template <> __device__ __forceinline__ float2 xfrom<float2>(float2 v) { return v; }

// Channel-independent factorisation of the natural-spline system of one
// (direction, envelope), per knot row i (Thomas elimination without pivoting):
//   g_i = d_i - l_i * cp_{i-1};  m = 1/g_i;  lm = l_i/g_i;  cp = u_i/g_i;
//   ih = 1 / (x_{i+1} - x_i)  (0 for the last row); for the double-float
//   form 3 / (x_{i+1} - x_i), the factor 3 of the right-hand side
//   3 (slope_i - slope_{i-1}) folded in.
template <typename real>
struct alignas(4 * sizeof(real)) Fac {
    real m, lm, cp, ih;
};
template <typename real>
constexpr bool kFacIh3 = false;
template <>
constexpr bool kFacIh3<dd> = true;
__device__ __forceinline__ double fac_ih(double r) { return r; }
__device__ __forceinline__ float fac_ih(float r) { return r; }
__device__ __forceinline__ dd fac_ih(dd r) { return dd_mulf(r, 3.0f); }

// Geometry of one record (or the widest epoch of a batch).
struct Geom {
    int C;      // channels
    int L;      // samples
    int K;      // directions (all chunks)
    int W;      // 32-bit words per direction bitmask = ceil(L / 32)
    int cap;    // knot capacity per (direction, envelope)
    int cov;    // last interior sample tested for extrema
    int nak;    // not-a-knot end conditions (MEMD_SPLINE_NOT_A_KNOT)
    int mirror; // mirrored end knots (MEMD_BOUNDARY_MIRROR)
};

// Batched runs: the epochs are concatenated along the sample axis, each
// starting at a multiple of kEpochAlign samples (so that no 32-sample word,
// evaluation tile or anchor span holds samples of two epochs; the gap samples
// are zero and never tested, fitted or written).  n == 0: a single record
// described by Geom alone.
constexpr int kEpochAlign = 512;
struct Epochs {
    int n;
    const int* off;  // [n] first sample of epoch e in the concatenated record
    const int* len;  // [n] its length
    const int* cov;  // [n] last interior sample tested for extrema (epoch-local index)
    const int* w0;   // [n + 1] first word of epoch e; w0[n] = W
    const int* wep;  // [W] epoch of each word
    int* cnt;        // [2][K][n] knots per (envelope, direction, epoch)
};

// Extremum rule of sample n: inside the record, a forced end point (first or
// last sample of its record), or an interior sample that is tested.
__device__ __forceinline__ void sample_rule(const Geom& g, const Epochs& ep, int n, bool& inrange, bool& endpt,
                                            bool& interior)
{
    if (ep.n == 0) {
        inrange = n < g.L;
        endpt = !g.mirror && ((n == 0) || (n == g.L - 1));
        interior = (n >= 1) && (n <= min(g.cov, g.L - 2));
        return;
    }
    if (n >= g.L) {
        inrange = endpt = interior = false;
        return;
    }
    const int e = ep.wep[n >> 5];
    const int t = n - ep.off[e], Le = ep.len[e];
    inrange = t < Le;
    endpt = (t == 0) || (t == Le - 1);
    interior = (t >= 1) && (t <= min(ep.cov[e], Le - 2));
}

// Is knot i (at sample x, of E knots) the first or last knot of its record?
__device__ __forceinline__ bool record_end_knot(const Epochs& ep, int x, int i, int E)
{
    if (ep.n == 0) return i == 0 || i == E - 1;
    const int e = ep.wep[x >> 5];
    const int o = ep.off[e];
    return x == o || x == o + ep.len[e] - 1;
}
// First and last sample of the record (epoch) holding sample x of a batch.
__device__ __forceinline__ void record_bounds(const Epochs& ep, int x, int& first, int& last)
{
    const int e = ep.wep[x >> 5];
    first = ep.off[e];
    last = first + ep.len[e] - 1;
}

// Do both envelopes of direction k have more than 3 knots in epoch e?
__device__ __forceinline__ bool dir_qualifies(const Geom& g, const Epochs& ep, const int* cnt, int k, int e)
{
    if (ep.n == 0) return cnt[k] > 3 && cnt[g.K + k] > 3;
    return ep.cnt[(size_t)k * ep.n + e] > 3 && ep.cnt[((size_t)g.K + k) * ep.n + e] > 3;
}

// Mirrored end knots of one direction (boundary mode MEMD_BOUNDARY_MIRROR),
// written by k_mirror, [K][kMirWords] ints: the symmetry samples, the counts
// of left / right mirrored knots per envelope (0 = maxima) and their source
// samples in ascending order of mirrored position 2 sym - src.
constexpr int kMirWords = 16;
enum { kMirLsym = 0, kMirRsym = 1, kMirNl = 2, kMirNr = 4, kMirLsrc = 6, kMirRsrc = 10 };

// Bounds-checked build (-DMEMD_CHECKED): MEMD_CHECK(cond) is false when an
// index check fails, which also records the failure in g_memd_check (read and
// cleared by the host after each run, reported as MEMD_FLAG_CHECK_FAILED); the
// guarded access is then skipped instead of touching memory out of bounds.
// In the normal build the checks compile away.
#ifdef MEMD_CHECKED
__device__ int g_memd_check;
__device__ __forceinline__ bool memd_check(bool ok)
{
    if (!ok) atomicOr(&g_memd_check, 1);
    return ok;
}
#define MEMD_CHECK(cond) memd::memd_check((cond))
#else
#define MEMD_CHECK(cond) true
#endif

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
                               // [2] IMF loop continues (mirrors of the graph conditions),
                               // [3] extremum tests re-decided in double-float
};

// Stop mode, batched runs: the decision state of one record (epoch); the
// fields of RunState that belong to a single record, per record.
struct RecStop {
    int nbit;      // sifts applied to the record's current IMF
    int pass;      // envelope passes of the current IMF
    int imf_done;  // the record's residual has too few extrema (its decomposition ends)
    int fin;       // the record's decomposition has ended (no further IMF)
    int apply;     // subtract the mean of the last pass from this record
    int sifting;   // the record takes part in the current sift loop
    int n_imfs;    // IMFs written for the record
    int q;         // qualified directions of the last pass
    int few;       // every direction has fewer than 3 interior extrema (last pass)
    int pad;
    unsigned long long over1, over2;  // samples with sigma > sd, > sd2 in the last pass
    int sifts[64];                    // sifts per IMF
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
__device__ __forceinline__ dd fmad_(dd a, dd b, dd c) { return a * b + c; }
__device__ __forceinline__ dd mul_(dd a, dd b) { return a * b; }
__device__ __forceinline__ dd add_(dd a, dd b) { return a + b; }
__device__ __forceinline__ dd sub_(dd a, dd b) { return a - b; }
__device__ __forceinline__ dd div_(dd a, dd b) { return a / b; }
__device__ __forceinline__ double shfl_xor_(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ float shfl_xor_(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double shfl_idx_(double v, int l) { return __shfl_sync(0xffffffffu, v, l); }
__device__ __forceinline__ float shfl_idx_(float v, int l) { return __shfl_sync(0xffffffffu, v, l); }
__device__ __forceinline__ dd shfl_idx_(dd v, int l)
{
    return dd(__shfl_sync(0xffffffffu, v.hi, l), __shfl_sync(0xffffffffu, v.lo, l));
}
__device__ __forceinline__ dd shfl_xor_(dd v, int o)
{
    return dd(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
}
__device__ __forceinline__ double sqrt_(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ dd sqrt_(dd a) { return dd_sqrt(a); }
// a * t + c with a plain float t
__device__ __forceinline__ double fmat_(double a, float t, double c) { return __fma_rn(a, (double)t, c); }
__device__ __forceinline__ float fmat_(float a, float t, float c) { return __fmaf_rn(a, t, c); }
__device__ __forceinline__ dd fmat_(dd a, float t, dd c) { return dd_mulf(a, t) + c; }
// 1/a: IEEE division for double and float (the FP64 and FP32 forms keep the
// reference's arithmetic); for a double-float, the correctly rounded float
// reciprocal refined by one Newton step with an fma residual (~47 bits, a
// quarter of the instructions of the double-float division)
__device__ __forceinline__ double recip_(double a) { return __ddiv_rn(1.0, a); }
__device__ __forceinline__ float recip_(float a) { return __fdiv_rn(1.0f, a); }
__device__ __forceinline__ dd recip_(dd a)
{
    const float x0 = __frcp_rn(a.hi);
    const float e = __fmaf_rn(-a.lo, x0, __fmaf_rn(-a.hi, x0, 1.0f));  // 1 - a x0
    return dd_renorm(x0, __fmul_rn(x0, e));
}
// identity rows of the factorisation (natural end conditions, record ends)
// carry m = 1 exactly; every other row has m <= 1/3 (pivot >= 3)
__device__ __forceinline__ bool is_one(double v) { return v == 1.0; }
__device__ __forceinline__ bool is_one(float v) { return v == 1.0f; }
__device__ __forceinline__ bool is_one(dd v) { return v.hi == 1.0f && v.lo == 0.0f; }
__device__ __forceinline__ bool is_zero(double v) { return v == 0.0; }
__device__ __forceinline__ bool is_zero(float v) { return v == 0.0f; }
__device__ __forceinline__ bool is_zero(dd v) { return v.hi == 0.0f; }
// magnitude as a float (bounds only: the float may round down by 1 ulp)
__device__ __forceinline__ float magf(double v) { return (float)fabs(v); }
__device__ __forceinline__ float magf(float v) { return fabsf(v); }
__device__ __forceinline__ float magf(dd v) { return fabsf(v.hi); }

}  // namespace memd
