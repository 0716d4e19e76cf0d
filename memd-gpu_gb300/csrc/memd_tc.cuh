// memd_tc.cuh -- projection + extrema bitmasks on the tensor cores (mixed form).
//
// The reference projects with cublasSgemm (memReducedEpochs_dev.cu:1182-1184)
// and then flags strict local extrema of every projected direction
// (find_extrema_shfl_max/min :77-141).  Here the tensor cores compute, per
// tile of 128 samples and N <= 256 directions, the projected first differences
//     D[n][k] = P[n][k] - P[n-1][k] = sum_c dir[k][c] (X[n][c] - X[n-1][c])
// and sample n is a maximum (minimum) of direction k when D[n] > 0 > D[n+1]
// (D[n] < 0 < D[n+1]): the same strict comparisons P[n] > P[n-1], P[n] >
// P[n+1] as the reference, read from the signs of the differences.
//
//   k_split_tf32    the first differences of the working signal (double-float
//                   X[n][c], differenced in double-float, rounded to float)
//                   and the (float32) directions, each split into tf32 "big"
//                   and "small" parts, v = big + small + r, |r| <= 2^-22 |v|,
//                   stored [rows][Cp] (Cp = C rounded up to 32, zero padded)
//   k_project_tc    TMA (cp.async.bulk.tensor, 128-byte swizzle) stages the
//                   big / small tiles of 128 samples and N directions per
//                   32-channel block; one thread issues the 3xTF32 products
//                   big.big + big.small + small.big as tcgen05.mma kind::tf32
//                   (M = 128, N <= 256, K = 8 per instruction) into a TMEM
//                   accumulator; four warps read it back (tcgen05.ld: one TMEM
//                   lane = one sample per thread), take D[n+1] from the next
//                   lane, warp or the tile's halo row, and form the bitmask
//                   words by ballot.
//
// Certification.  With S = sum_c |dh_c| max|dx_c| over the tile's rows and its
// halo row (dx the rounded differences, dh the float32 direction; S summed
// with upward rounding), the tensor-core D differs from the exact difference
// of the projections by at most
//   (4C + 8) 2^-22 S       the dropped small.small and remainder terms
//                          (3.01 2^-22 |dx||d| per product) and the
//                          accumulation, counted as 2 ulp of the largest
//                          partial sum per product and step
//   + 2^-24 S              the rounding of the differences to float
// (times 1.01).  A sign within that bound of zero is decided again by a
// double-float dot product of the double-float differences (~2^-44 relative),
// so the extrema sets are those of the exact projection except at ties closer
// than that.  Differencing first makes the bound scale with the signal's
// sample-to-sample change rather than its size: smooth late-IMF signals, whose
// neighbouring projections agree to many digits, stay decidable on the tensor
// cores.
//
// Every wait on an mbarrier is bounded (iterations and clock); a wait that
// runs out sets MEMD_FLAG_DEVICE_TIMEOUT in the run state, waits (bounded)
// for the copies or products already issued, frees the TMEM columns and
// returns.
#pragma once

#include <cuda.h>

#include "memd_kernels.cuh"  // kFull, sample_rule
#include "memd_ptx.cuh"

namespace memd {

constexpr int kTcRows = 128;        // samples per tile (MMA M)
constexpr int kTcThreads = 128;     // four warps: one TMEM lane quarter each
constexpr int kTcMaxN = 256;        // directions per tile at most (MMA N)
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

// First difference of the double-float signal, X[n][c] - X[n-1][c], as a
// double-float.
__device__ __forceinline__ dd xdiff(float2 a, float2 b) { return dd(a.x, a.y) - dd(b.x, b.y); }

// ---------------------------------------------------------------------------
// Split into tf32 parts: big[r][c] = tf32(v), small[r][c] = tf32(v - big) for
// c < C, zero for C <= c < Cp.
//   diff = 1: v = float(X[r][c] - X[r-1][c]) of the double-float signal X
//             ([rows][C] float2; v = 0 in row 0)
//   diff = 0: v = src[r][c] of a float array ([rows][C])
// ---------------------------------------------------------------------------
__global__ void k_split_tf32(const void* __restrict__ src, int diff, float* __restrict__ big,
                             float* __restrict__ small, int rows, int C, int Cp)
{
    const size_t total = (size_t)rows * Cp;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / Cp;
        const int c = (int)(i - r * Cp);
        float v = 0.f;
        if (c < C) {
            if (diff) {
                const float2* X = static_cast<const float2*>(src);
                if (r > 0) v = xdiff(X[r * C + c], X[(r - 1) * C + c]).hi;
            } else {
                v = static_cast<const float*>(src)[r * C + c];
            }
        }
        const float b = tf32_rna(v);
        big[i] = b;
        small[i] = tf32_rna(__fsub_rn(v, b));
    }
}

struct TcMaps {
    CUtensorMap xb, xs, db, ds;
};

// TMEM columns (and padded per-direction array length) of a tile of n
// directions: a power of two >= 32.
__host__ __device__ constexpr int tc_cols(int n) { return n <= 32 ? 32 : (n <= 64 ? 64 : (n <= 128 ? 128 : 256)); }

// Shared memory of k_project_tc for N directions per tile (bytes, with the
// slack for aligning the operand tiles to 1024 bytes): 52.5 KB at N = 64,
// four CTAs per SM.
__host__ __device__ constexpr size_t tc_smem_bytes(int n)
{
    return 1024 + 2 * (size_t)kTcRows * 128 + 2 * (size_t)n * 128  // operand tiles
           + sizeof(float) * (4 * (size_t)tc_cols(n)               // first rows of the warps [4][NP]
                              + (size_t)tc_cols(n)                 // halo row [NP]
                              + (size_t)tc_cols(n)                 // bound sums [NP]
                              + 4 * 32 + 32                        // channel maxima
                              + 32)                                // halo-row differences of a block
           + 64;                                                   // barriers, TMEM address
}

__device__ __forceinline__ int dd_sign(dd v) { return v.hi > 0.f ? 1 : (v.hi < 0.f ? -1 : (v.lo > 0.f) - (v.lo < 0.f)); }

// The sign of sum_c dir[c] (X1[c] - X0[c]) in double-float, computed by the
// whole warp: lane l takes channels l, l + 32, ... (one coalesced row load
// per operand), the lanes' double-float partial sums meet in a butterfly of
// shuffles; every lane returns lane 0's sign.  The directions are float32
// (the mixed form's input), so each term is the exact two-product of the
// direction with the double-float difference's high word plus its product
// with the low word, and the sum carries ~2^-44 relative to
// sum |dir| |X1 - X0|.
__device__ __noinline__ int warp_df_diff_sign(const float2* __restrict__ x1, const float2* __restrict__ x0,
                                                 const float* __restrict__ dh, int C, int lane)
{
    dd acc(0.f, 0.f);
    for (int c = lane; c < C; c += 32) {
        const dd v = xdiff(x1[c], x0[c]);
        const float a = dh[c];
        const float p = __fmul_rn(a, v.hi);
        float e = __fmaf_rn(a, v.hi, -p);
        e = __fmaf_rn(a, v.lo, e);
        acc = acc + dd_renorm(p, e);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = acc + shfl_xor_(acc, o);
    return __shfl_sync(kFull, dd_sign(acc), 0);
}

// Grid: (ceil(L / 128), ceil(Kc / nt)); nt = directions per tile (a multiple
// of 16 in [16, 256]; narrower tiles give more CTAs, each loading the same
// signal tile).
__global__ void __launch_bounds__(kTcThreads)
k_project_tc(const __grid_constant__ TcMaps maps, const float2* __restrict__ X, const float* __restrict__ dh_all,
             uint32_t* __restrict__ bits, Geom g, int k0, int Kc, int Cp, int nt, RunState* st, Epochs ep)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // operand tiles at a 1024-byte boundary (the 128-byte swizzle repeats
    // every 8 rows of 128 bytes)
    const uint32_t base = smem_u32(smem_raw);
    unsigned char* tiles = smem_raw + (((base + 1023u) & ~1023u) - base);
    float* Ab = reinterpret_cast<float*>(tiles);             // [128][32] big parts of the differences
    float* As = Ab + kTcRows * kTcKB;                        // [128][32] small parts
    float* Bb = As + kTcRows * kTcKB;                        // [nt][32] directions, big
    float* Bs = Bb + nt * kTcKB;                             // [nt][32] directions, small
    const uint32_t ncols = (uint32_t)tc_cols(nt);  // TMEM columns; per-direction arrays padded to this
    const int NP = (int)ncols;
    float* first = Bs + nt * kTcKB;                          // [4 warps][NP]: D of each warp's lane 0
    float* halo = first + 4 * NP;                            // [NP]: D at sample n0 + 128
    float* thr = halo + NP;                                  // [NP]: sum |dh| max|dx|, then the bound
    float* cmx = thr + NP;                                   // [4][32] per-warp channel maxima
    float* mx = cmx + 4 * 32;                                // [32] channel maxima of the block
    float* xd = mx + 32;                                     // [32] halo-row differences of the block
    uint64_t* bars = reinterpret_cast<uint64_t*>(xd + 32);   // [0] TMA, [1] MMA
    uint32_t* s_taddr = reinterpret_cast<uint32_t*>(bars + 2);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int C = g.C;
    const int n0 = blockIdx.x * kTcRows;
    const int kt0 = blockIdx.y * nt;            // first direction of the tile within the chunk
    const int nk = min(nt, Kc - kt0);           // valid directions of the tile
    const int nkb = Cp / kTcKB;
    const int nh = n0 + kTcRows;                // the halo row
    const bool has_halo = nh < g.L;

    if (warp == 0) {
        tmem_alloc(s_taddr, ncols);
        tmem_relinquish();
    }
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    // halo: D at sample n0 + 128 in FP32 from the rounded differences (the
    // same numbers the tensor cores see), its error within the same bound;
    // halo and bound summed over the channel blocks below
    for (int i = tid; i < NP; i += kTcThreads) {
        thr[i] = 0.f;
        halo[i] = 0.f;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *s_taddr;

    const uint32_t idesc = tc_idesc_tf32(nt);
    const uint32_t tx_bytes = (uint32_t)(2 * kTcRows * 128 + 2 * nt * 128);
    if (tid == 0) {  // the first block's copies, before anything else
        mbar_expect_tx(&bars[0], tx_bytes);
        tma_load_2d(Ab, &maps.xb, &bars[0], 0, n0);
        tma_load_2d(As, &maps.xs, &bars[0], 0, n0);
        tma_load_2d(Bb, &maps.db, &bars[0], 0, k0 + kt0);
        tma_load_2d(Bs, &maps.ds, &bars[0], 0, k0 + kt0);
    }

    int fail = 0, kb = 0;  // fail: 1 = a copy, 2 = the products did not complete in time
    for (; kb < nkb; ++kb) {
        if (tid == 0 && kb > 0) {
            mbar_expect_tx(&bars[0], tx_bytes);
            tma_load_2d(Ab, &maps.xb, &bars[0], kb * kTcKB, n0);
            tma_load_2d(As, &maps.xs, &bars[0], kb * kTcKB, n0);
            tma_load_2d(Bb, &maps.db, &bars[0], kb * kTcKB, k0 + kt0);
            tma_load_2d(Bs, &maps.ds, &bars[0], kb * kTcKB, k0 + kt0);
        }
        // the halo row's differences of this block (while the copies land)
        if (tid < 32) {
            const int c = kb * kTcKB + tid;
            xd[tid] = (has_halo && c < C) ? xdiff(X[(size_t)nh * C + c], X[(size_t)(nh - 1) * C + c]).hi : 0.f;
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
        // channel maxima of |dx| over the tile's rows (the big parts;
        // |big + small| <= |big| (1 + 2^-10)) while the products run: lane =
        // channel, warp w = rows 32w .. 32w + 31; element (r, c) of the
        // swizzled tile sits in 16-byte chunk (c / 4) ^ (r % 8) of row r
        {
            float m = 0.f;
#pragma unroll 8
            for (int rr = 0; rr < 32; ++rr) {
                const int r = warp * 32 + rr;
                const int chunk = (lane >> 2) ^ (r & 7);
                m = fmaxf(m, fabsf(Ab[r * kTcKB + chunk * 4 + (lane & 3)]));
            }
            cmx[warp * 32 + lane] = m;
        }
        __syncthreads();
        if (warp == 0) {
            const float m = fmaxf(fmaxf(cmx[lane], cmx[32 + lane]), fmaxf(cmx[64 + lane], cmx[96 + lane]));
            mx[lane] = fmaxf(m, fabsf(xd[lane])) * 1.0009765625f;
        }
        __syncthreads();
        // this block's part of the halo row and of the bound sum, per
        // direction: warp w takes directions w, w + 4, ...; lane = channel, so
        // each direction is one coalesced 128-byte row of the direction set
        // (L1/L2-resident), reduced by shuffles (the bound rounded up)
        {
            const int c = kb * kTcKB + lane;
            const bool cin = c < C;
            const float xdl = xd[lane], mxl = mx[lane];
            const float* drow = dh_all + (size_t)(k0 + kt0) * C + (cin ? c : 0);
            constexpr int DB = 4;  // directions per batch of loads
            for (int kb0 = warp; kb0 < nk; kb0 += 4 * DB) {
                float dv[DB];
#pragma unroll
                for (int u = 0; u < DB; ++u) {
                    const int kk = kb0 + 4 * u;
                    dv[u] = (cin && kk < nk) ? __ldg(drow + (size_t)kk * C) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < DB; ++u) {
                    const int kk = kb0 + 4 * u;
                    float h = __fmul_rn(dv[u], xdl);
                    float sh = __fmul_ru(fabsf(dv[u]), mxl);
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) {
                        h = __fadd_rn(h, __shfl_xor_sync(kFull, h, o));
                        sh = __fadd_ru(sh, __shfl_xor_sync(kFull, sh, o));
                    }
                    if (lane == 0 && kk < nk) {
                        halo[kk] = __fadd_rn(halo[kk], h);
                        thr[kk] = __fadd_ru(thr[kk], sh);
                    }
                }
            }
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
    // the bound on |D_tc - D| per direction, with the margin for its own rounding
    {
        const float eps = (float)(4 * C + 8) * 2.384185791e-7f + 5.9604645e-8f;  // (4C + 8) 2^-22 + 2^-24
        for (int kk = tid; kk < nk; kk += kTcThreads)
            thr[kk] = 1.01f * __fmul_ru(eps, thr[kk]);
    }
    // pass 1: every warp publishes its lane 0 (its first sample) for the warp before
    const uint32_t tl = taddr + ((uint32_t)(warp * 32) << 16);
    for (int j0 = 0; j0 < nt; j0 += 32) {
        float v[32];
        (void)MEMD_CHECK(j0 + 32 <= (int)ncols && j0 + 32 <= kTcMaxN);
        __syncwarp();  // tcgen05.ld is warp-collective
        tmem_ld32(tl + (uint32_t)j0, v);
        if (lane == 0) {
            float* e = first + warp * NP + j0;
#pragma unroll
            for (int j = 0; j < 32; ++j) e[j] = v[j];
        }
    }
    __syncthreads();
    // pass 2: signs of D[n] and D[n+1], ballots, one bitmask word per lane and direction
    const int n = n0 + warp * 32 + lane;
    bool inrange, endpt, interior;
    sample_rule(g, ep, n, inrange, endpt, interior);
    const int w = (n0 >> 5) + warp;
    int refined = 0;
    for (int j0 = 0; j0 < nt; j0 += 32) {
        float v[32];
        __syncwarp();
        tmem_ld32(tl + (uint32_t)j0, v);
        // bit j of each mask: direction j0 + j at this lane's sample
        uint32_t mxm = 0u, mnm = 0u, nearm = 0u;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const int kk = j0 + j;
            const float d0 = v[j];  // D[n]
            float d1 = __shfl_down_sync(kFull, d0, 1);
            if (lane == 31) d1 = warp == 3 ? halo[kk] : first[(warp + 1) * NP + kk];
            if (d0 > 0.f && d1 < 0.f) mxm |= 1u << j;
            if (d0 < 0.f && d1 > 0.f) mnm |= 1u << j;
            if (interior && kk < nk) {
                const float t = thr[kk];
                if (fabsf(d0) <= t || fabsf(d1) <= t) nearm |= 1u << j;
            }
        }
        refined += __popc(nearm);
        // signs within the bound: decided again in double-float, one
        // (direction, lane) at a time by the whole warp (lanes over channels)
        uint32_t anyj = __reduce_or_sync(kFull, nearm);
        while (anyj) {
            const int j = __ffs(anyj) - 1;
            anyj &= anyj - 1u;
            const int kk = j0 + j;
            const float* dh = dh_all + (size_t)(k0 + kt0 + kk) * C;
            uint32_t need = __ballot_sync(kFull, (nearm >> j) & 1u);
            while (need) {
                const int l = __ffs(need) - 1;
                need &= need - 1u;
                const float2* xl = X + (size_t)(n0 + warp * 32 + l) * C;
                const int s0 = warp_df_diff_sign(xl, xl - C, dh, C, lane);
                const int s1 = warp_df_diff_sign(xl + C, xl, dh, C, lane);
                if (lane == l) {
                    const uint32_t bit = 1u << j;
                    mxm = (s0 > 0 && s1 < 0) ? (mxm | bit) : (mxm & ~bit);
                    mnm = (s0 < 0 && s1 > 0) ? (mnm | bit) : (mnm & ~bit);
                }
            }
        }
        // the bitmask words: lane j keeps the ballot of direction j0 + j
        uint32_t my_max = 0u, my_min = 0u;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const uint32_t wmax = __ballot_sync(kFull, inrange && (endpt || (interior && ((mxm >> j) & 1u))));
            const uint32_t wmin = __ballot_sync(kFull, inrange && (endpt || (interior && ((mnm >> j) & 1u))));
            if (lane == j) {
                my_max = wmax;
                my_min = wmin;
            }
        }
        const int kk = j0 + lane;
        if (kk < nk && w < g.W && MEMD_CHECK(kt0 + kk < Kc)) {
            bits[(size_t)(kt0 + kk) * g.W + w] = my_max;
            bits[(size_t)(Kc + kt0 + kk) * g.W + w] = my_min;
        }
    }
    refined = warp_sum(refined);
    if (lane == 0 && refined) atomicAdd(&st->pad[3], refined);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(taddr, ncols);
    }
}

}  // namespace memd
