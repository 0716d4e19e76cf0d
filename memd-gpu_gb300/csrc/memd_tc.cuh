// memd_tc.cuh -- projection + extrema bitmasks on the tensor cores (mixed form).
//
// P[n][k] = sum_c X[n][c] dir[k][c] (reference: cublasSgemm,
// memReducedEpochs_dev.cu:1182-1184, followed by the extrema flags of
// find_extrema_shfl_max/min :77-141) as a 128-sample x N-direction tile per
// CTA on the 5th-generation tensor cores:
//
//   k_split_tf32    the working signal's high words (double-float X[n][c].x)
//                   and the directions' high words split into tf32 "big" and
//                   "small" parts, x = big + small + r with |r| <= 2^-22 |x|,
//                   stored [rows][Cp] (Cp = C rounded up to 32, zero padded)
//   k_project_tc    TMA (cp.async.bulk.tensor, 128-byte swizzle) stages the
//                   big / small tiles of 128 samples and N directions per
//                   32-channel block; one thread issues the 3xTF32 products
//                   big.big + big.small + small.big as tcgen05.mma kind::tf32
//                   (M = 128, N <= 256, K = 8 per instruction) into a TMEM
//                   accumulator; four warps read it back (tcgen05.ld, one
//                   TMEM lane = one sample per thread) and form the extremum
//                   tests with their neighbours by shuffle, the words of the
//                   bitmask by ballot.
//
// Certification (the extrema sets stay those of the FP64 projection, as in
// k_project_mx).  With S = sum_c |dh_c| max|xh_c| over the tile (and its two
// neighbour rows), the tensor-core value differs from the exact projection by
// at most
//   (4C + 8) 2^-22 S            products: the dropped small.small and
//                               remainder terms (3.01 2^-22 |x||d| each) and
//                               accumulation, counted as 2 ulp of the
//                               largest partial sum per product and step
//   + 2^-24 S + sum|dl| max|X|  the double-float low words of X and dir
// (times 1.01).  A comparison whose tensor-core margin is within twice that
// bound is redone with an FP32 fma dot product in channel order (bound
// (C+2) 2^-24 S + sum|dl| max|X|, as k_project_mx), and one still within
// twice that bound with double-float dot products (~2^-44).
//
// Every wait on an mbarrier is bounded (iterations and clock); a wait that
// runs out sets MEMD_FLAG_DEVICE_TIMEOUT in the run state, waits (bounded)
// for the copies and products already issued, frees the TMEM columns and
// returns.
#pragma once

#include <cuda.h>

#include "memd_kernels.cuh"  // kFull, df_dot, df_gt, sample_rule
#include "memd_ptx.cuh"

namespace memd {

constexpr int kTcRows = 128;        // samples per tile (MMA M)
constexpr int kTcThreads = 128;     // four warps: one TMEM lane quarter each
constexpr int kTcMaxN = 256;        // directions per tile (MMA N)
constexpr int kTcKB = 32;           // channels per K block (one 128-byte swizzled row of tf32)
constexpr long long kTcWaitClocks = 1ll << 31;  // ~1 s at 2 GHz: the limit of every wait

// Shared-memory matrix descriptor of a K-major operand in the 128-byte
// swizzled layout TMA writes: rows of 128 bytes, 8-row atoms 1024 bytes apart
// (stride byte offset), leading byte offset unused, descriptor version 1,
// layout type 2 (128-byte swizzle).  The start address moves by 32 bytes per
// K step of 8 tf32 values inside the atom.
__device__ __forceinline__ uint64_t sw128_kmajor_desc(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((1024u >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}
// Instruction descriptor: D f32, A and B tf32, both K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t tc_idesc_tf32(int n)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);
}
__device__ __forceinline__ float tf32_rna(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// ---------------------------------------------------------------------------
// Split into tf32 parts: big[r][c] = tf32(v), small[r][c] = tf32(v - big) of
// v = src(r, c) for c < C, zero for C <= c < Cp.  src is the high word of a
// double-float row-major [rows][C] array (stride 2 floats per element), or a
// plain float array (stride 1).
// ---------------------------------------------------------------------------
__global__ void k_split_tf32(const float* __restrict__ src, int elem_stride, float* __restrict__ big,
                             float* __restrict__ small, int rows, int C, int Cp)
{
    const size_t total = (size_t)rows * Cp;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / Cp;
        const int c = (int)(i - r * Cp);
        const float v = c < C ? src[(r * C + c) * elem_stride] : 0.f;
        const float b = tf32_rna(v);
        big[i] = b;
        small[i] = tf32_rna(__fsub_rn(v, b));
    }
}

struct TcMaps {
    CUtensorMap xb, xs, db, ds;
};

// Shared memory of k_project_tc for N directions per tile (bytes, with the
// slack for aligning the operand tiles to 1024 bytes).
__host__ __device__ constexpr size_t tc_smem_bytes(int n)
{
    return 1024 + 2 * (size_t)kTcRows * 128 + 2 * (size_t)n * 128  // operand tiles
           + sizeof(float) * (8 * (size_t)kTcMaxN                  // edges [4][2][N]
                              + 2 * (size_t)kTcMaxN                // halo rows [2][N]
                              + 2 * (size_t)kTcMaxN                // thresholds [2][N]
                              + 4 * 32 + 32)                       // channel maxima
           + 64;                                                   // barriers, TMEM address
}

__device__ __forceinline__ float proj_fma(const float2* __restrict__ xrow, const float* __restrict__ dh, int C)
{
    float acc = 0.f;
    for (int c = 0; c < C; ++c) acc = __fmaf_rn(xrow[c].x, dh[c], acc);
    return acc;
}

__global__ void __launch_bounds__(kTcThreads)
k_project_tc(const __grid_constant__ TcMaps maps, const float2* __restrict__ X, const float* __restrict__ dh_all,
             const float* __restrict__ dl_all, uint32_t* __restrict__ bits, Geom g, int k0, int Kc, int Cp, int nt,
             RunState* st, Epochs ep)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // operand tiles at a 1024-byte boundary (the 128-byte swizzle repeats
    // every 8 rows of 128 bytes)
    const uint32_t base = smem_u32(smem_raw);
    unsigned char* tiles = smem_raw + (((base + 1023u) & ~1023u) - base);
    float* Ab = reinterpret_cast<float*>(tiles);             // [128][32]
    float* As = Ab + kTcRows * kTcKB;                        // [128][32]
    float* Bb = As + kTcRows * kTcKB;                        // [nt][32]
    float* Bs = Bb + nt * kTcKB;                             // [nt][32]
    float* edge = Bs + nt * kTcKB;                           // [4 warps][2][kTcMaxN]: lane 0 / lane 31 values
    float* halo = edge + 8 * kTcMaxN;                        // [2][kTcMaxN]: rows n0 - 1, n0 + 128
    float* thr = halo + 2 * kTcMaxN;                         // [2][kTcMaxN]: tensor-core / FP32 thresholds
    float* cmx = thr + 2 * kTcMaxN;                          // [4][32] per-warp channel maxima
    float* mx = cmx + 4 * 32;                                // [32] channel maxima of the block
    uint64_t* bars = reinterpret_cast<uint64_t*>(mx + 32);   // [0] TMA, [1] MMA
    uint32_t* s_taddr = reinterpret_cast<uint32_t*>(bars + 2);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int C = g.C;
    const int n0 = blockIdx.x * kTcRows;
    const int kt0 = blockIdx.y * kTcMaxN;       // first direction of the tile within the chunk
    const int nk = min(nt, Kc - kt0);           // valid directions of the tile
    const uint32_t ncols = nt <= 32 ? 32u : (nt <= 64 ? 64u : (nt <= 128 ? 128u : 256u));
    const int nkb = Cp / kTcKB;

    if (warp == 0) {
        tmem_alloc(s_taddr, ncols);
        tmem_relinquish();
    }
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    for (int i = tid; i < nt; i += kTcThreads) {
        thr[i] = 0.f;
        thr[kTcMaxN + i] = 0.f;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *s_taddr;

    // halo rows n0 - 1 and n0 + 128 in FP32 (fma over the channels in order)
    for (int i = tid; i < 2 * nk; i += kTcThreads) {
        const int side = i / nk, kk = i - side * nk;
        const int n = side ? n0 + kTcRows : n0 - 1;
        float v = 0.f;
        if (n >= 0 && n < g.L) v = proj_fma(X + (size_t)n * C, dh_all + (size_t)(k0 + kt0 + kk) * C, C);
        halo[side * kTcMaxN + kk] = v;
    }

    const uint32_t idesc = tc_idesc_tf32(nt);
    const uint32_t tx_bytes = (uint32_t)(2 * kTcRows * 128 + 2 * nt * 128);
    int fail = 0, kb = 0;  // fail: 1 = a copy, 2 = the products did not complete in time
    for (; kb < nkb; ++kb) {
        if (tid == 0) {
            mbar_expect_tx(&bars[0], tx_bytes);
            tma_load_2d(Ab, &maps.xb, &bars[0], kb * kTcKB, n0);
            tma_load_2d(As, &maps.xs, &bars[0], kb * kTcKB, n0);
            tma_load_2d(Bb, &maps.db, &bars[0], kb * kTcKB, k0 + kt0);
            tma_load_2d(Bs, &maps.ds, &bars[0], kb * kTcKB, k0 + kt0);
        }
        const bool got = mbar_wait_bounded(&bars[0], (uint32_t)(kb & 1), kTcWaitClocks);
        if (__syncthreads_or(!got)) {  // the same decision in every thread
            fail = 1;
            break;
        }
        tc_fence_after();
        if (tid == 0) {
            const uint32_t ab = smem_u32(Ab), as = smem_u32(As), bb = smem_u32(Bb), bs = smem_u32(Bs);
#pragma unroll
            for (int ks = 0; ks < kTcKB / 8; ++ks) {
                const uint32_t o = (uint32_t)ks * 32u;
                mma_tf32(taddr, sw128_kmajor_desc(ab + o), sw128_kmajor_desc(bb + o), idesc, (kb | ks) ? 1u : 0u);
                mma_tf32(taddr, sw128_kmajor_desc(ab + o), sw128_kmajor_desc(bs + o), idesc, 1u);
                mma_tf32(taddr, sw128_kmajor_desc(as + o), sw128_kmajor_desc(bb + o), idesc, 1u);
            }
            mma_commit(&bars[1]);
        }
        // channel maxima of this block over the tile's rows (the big parts;
        // |x| <= |big| (1 + 2^-10)) while the products run: lane = channel,
        // warp w = rows 32w .. 32w + 31; element (r, c) of the swizzled tile
        // sits in 16-byte chunk (c / 4) ^ (r % 8) of row r
        {
            float m = 0.f;
            for (int rr = 0; rr < 32; ++rr) {
                const int r = warp * 32 + rr;
                const int chunk = (lane >> 2) ^ (r & 7);
                m = fmaxf(m, fabsf(Ab[r * kTcKB + chunk * 4 + (lane & 3)]));
            }
            cmx[warp * 32 + lane] = m;
        }
        __syncthreads();
        if (warp == 0) {
            float m = fmaxf(fmaxf(cmx[lane], cmx[32 + lane]), fmaxf(cmx[64 + lane], cmx[96 + lane]));
            const int c = kb * kTcKB + lane;
            // the halo rows' values
            if (c < C) {
                if (n0 - 1 >= 0) m = fmaxf(m, fabsf(X[(size_t)(n0 - 1) * C + c].x));
                if (n0 + kTcRows < g.L) m = fmaxf(m, fabsf(X[(size_t)(n0 + kTcRows) * C + c].x));
            }
            mx[lane] = m * 1.0009765625f;  // |big + small| <= |big| (1 + 2^-10)
        }
        __syncthreads();
        // partial bounds of this block: thr[k] += sum_c |dh| mx, thr[N + k] += sum_c |dl| mx
        for (int kk = tid; kk < nk; kk += kTcThreads) {
            const float* dh = dh_all + (size_t)(k0 + kt0 + kk) * C;
            const float* dl = dl_all + (size_t)(k0 + kt0 + kk) * C;
            float sh = thr[kk], sl = thr[kTcMaxN + kk];
            const int c1 = min(C, (kb + 1) * kTcKB);
            for (int c = kb * kTcKB; c < c1; ++c) {
                sh = __fmaf_ru(fabsf(dh[c]), mx[c - kb * kTcKB], sh);
                sl = __fmaf_ru(fabsf(dl[c]), mx[c - kb * kTcKB], sl);
            }
            thr[kk] = sh;
            thr[kTcMaxN + kk] = sl;
        }
        const bool done = mbar_wait_bounded(&bars[1], (uint32_t)(kb & 1), kTcWaitClocks);
        tc_fence_after();
        // (a barrier: the next block's copies overwrite the tiles)
        if (__syncthreads_or(!done)) {
            fail = 2;
            break;
        }
    }
    if (fail) {
        // a wait ran out: flag it, give the copies or products already issued
        // a bounded time to land, free the TMEM columns, return
        if (tid == 0) atomicOr(&st->flags, MEMD_FLAG_DEVICE_TIMEOUT);
        mbar_wait_bounded(&bars[fail - 1], (uint32_t)(kb & 1), kTcWaitClocks);
        tc_fence_before();
        __syncthreads();
        if (warp == 0) {
            tc_fence_after();
            tmem_dealloc(taddr, ncols);
        }
        return;
    }
    // thresholds: twice the error bounds, with the margin for their own rounding
    {
        const float eps_tc = (float)(4 * C + 8) * 2.384185791e-7f + 5.9604645e-8f;  // (4C + 8) 2^-22 + 2^-24
        const float eps_f = (float)(C + 2) * 5.9604645e-8f;                           // (C + 2) 2^-24
        for (int kk = tid; kk < nk; kk += kTcThreads) {
            const float sh = thr[kk], sl = thr[kTcMaxN + kk] * 1.0000002f;
            thr[kk] = 2.02f * __fmaf_ru(eps_tc, sh, sl);
            thr[kTcMaxN + kk] = 2.02f * __fmaf_ru(eps_f, sh, sl);
        }
    }
    // pass 1: every warp publishes its first and last rows for the neighbours
    const uint32_t tl = taddr + ((uint32_t)(warp * 32) << 16);
    for (int j0 = 0; j0 < nt; j0 += 32) {
        float v[32];
        __syncwarp();
        tmem_ld32(tl + (uint32_t)j0, v);
        if (lane == 0 || lane == 31) {
            float* e = edge + (warp * 2 + (lane == 31)) * kTcMaxN + j0;
#pragma unroll
            for (int j = 0; j < 32; ++j) e[j] = v[j];
        }
    }
    __syncthreads();
    // pass 2: extremum tests, ballots, one bitmask word per lane and direction
    const int r = warp * 32 + lane;
    const int n = n0 + r;
    bool inrange, endpt, interior;
    sample_rule(g, ep, n, inrange, endpt, interior);
    const int w = (n0 >> 5) + warp;
    int refined = 0, rechecked = 0;
    for (int j0 = 0; j0 < nt; j0 += 32) {
        float v[32];
        __syncwarp();  // tcgen05.ld is warp-collective
        tmem_ld32(tl + (uint32_t)j0, v);
        uint32_t my_max = 0u, my_min = 0u;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const int kk = j0 + j;
            const float p = v[j];
            float pl = __shfl_up_sync(kFull, p, 1);
            float pn = __shfl_down_sync(kFull, p, 1);
            if (lane == 0) pl = warp == 0 ? halo[kk] : edge[((warp - 1) * 2 + 1) * kTcMaxN + kk];
            if (lane == 31) pn = warp == 3 ? halo[kTcMaxN + kk] : edge[((warp + 1) * 2) * kTcMaxN + kk];
            bool mxf = p > pl && p > pn;
            bool mnf = p < pl && p < pn;
            const bool kok = kk < nk;
            if (interior && kok) {
                const float t1 = thr[kk];
                if (fabsf(__fsub_rn(p, pl)) <= t1 || fabsf(__fsub_rn(p, pn)) <= t1) {
                    // within the tensor-core bound: FP32 dot products in channel order
                    const float* dh = dh_all + (size_t)(k0 + kt0 + kk) * C;
                    const float a = proj_fma(X + (size_t)(n - 1) * C, dh, C);
                    const float b = proj_fma(X + (size_t)n * C, dh, C);
                    const float c2 = proj_fma(X + (size_t)(n + 1) * C, dh, C);
                    const float t2 = thr[kTcMaxN + kk];
                    ++rechecked;
                    if (fabsf(__fsub_rn(b, a)) <= t2 || fabsf(__fsub_rn(b, c2)) <= t2) {
                        // still within the FP32 bound: double-float
                        const float* dl = dl_all + (size_t)(k0 + kt0 + kk) * C;
                        const float2 da = df_dot(X + (size_t)(n - 1) * C, dh, dl, C);
                        const float2 db = df_dot(X + (size_t)n * C, dh, dl, C);
                        const float2 dc = df_dot(X + (size_t)(n + 1) * C, dh, dl, C);
                        mxf = df_gt(db, da) && df_gt(db, dc);
                        mnf = df_gt(da, db) && df_gt(dc, db);
                        ++refined;
                    } else {
                        mxf = b > a && b > c2;
                        mnf = b < a && b < c2;
                    }
                }
            }
            const uint32_t wmax = __ballot_sync(kFull, inrange && (endpt || (interior && mxf)));
            const uint32_t wmin = __ballot_sync(kFull, inrange && (endpt || (interior && mnf)));
            if (lane == j) {
                my_max = wmax;
                my_min = wmin;
            }
        }
        const int kk = j0 + lane;
        if (kk < nk && w < g.W) {
            bits[(size_t)(kt0 + kk) * g.W + w] = my_max;
            bits[(size_t)(Kc + kt0 + kk) * g.W + w] = my_min;
        }
    }
    refined = warp_sum(refined);
    rechecked = warp_sum(rechecked);
    if (lane == 0 && refined) atomicAdd(&st->pad[3], refined);
    if (lane == 0 && rechecked) atomicAdd(&st->rechecked, rechecked);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(taddr, ncols);
    }
}

}  // namespace memd
