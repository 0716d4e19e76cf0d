// memd_kernels.cuh -- the per-sift kernels of the GB300 MEMD engine.
//
// One sift (reference loop body memReducedEpochs_dev.cu:1179-1327) is five
// launches per direction chunk, all templated on the arithmetic type:
//
//   k_project_extrema  projection P = dir . X for a tile of samples and
//                      directions, strict-extremum tests, warp ballots into
//                      one 32-bit word per (direction, 32 samples)
//                      (REF:1182-1184 + REF:77-141)
//   k_compact          per (direction, envelope): popcount prefix of the
//                      bitmask, ordered knot list, knot count, end-point clamp
//                      of the knot values, optional trace (REF:143-486, 545-584)
//   k_factor           channel-independent Thomas factorisation of the
//                      natural-spline system (REF:704-736; replaces the
//                      factorisation inside cusparse gtsv2_nopivot)
//   k_solve_fwd/bwd    forward and backward substitution for every channel,
//                      in windows of S knots with an H-knot halo (REF:1227-1241)
//   k_mean_cum         mixed form, fixed mode: the mean envelope rebuilt from
//                      per-knot impulses and per-word anchors (REF:775-864)
//   k_eval             spline coefficients per interval, envelope evaluation
//                      fused with the mean over directions and the update of
//                      the working signal (REF:775-864)
//
// Working layout in HBM (sample-major, channel-minor, so that a knot's C
// values are one contiguous row):
//   X[n][c]                         working signal (n < L, c < C)
//   bits[env][kk][w]                extrema bitmask, bit j of word w = sample 32w+j
//   wpref[env][kk][w]               knots before word w (w <= W)
//   knots[env][kk][i]               knot sample indices, i < E <= cap
//   fac[env][kk][i]                 Fac<real> per knot row
//   yv[env][kk][i][c]               knot values (end knots clamped)
//   sv[env][kk][i][c]               spline solution per knot and channel
// env 0 = maxima (upper envelope), 1 = minima (lower envelope); kk indexes the
// directions of the current chunk, counts cnt[env][k] use the global k.
#pragma once

#include "memd_device.cuh"

namespace memd {

constexpr unsigned kFull = 0xffffffffu;
// longest anchor span of the impulse-accumulation mean: 4 words = 128
// samples (its accumulators then fit four CTAs per SM, at 64 registers)
constexpr int kCumMaxWords = 4;
constexpr int kTrace = 1;

// ---------------------------------------------------------------------------
// Projection + extrema bitmasks.  CTA tile: 64 samples x 16 directions,
// 8 warps = 2 sample groups x 4 direction groups of 4 directions; warp 0 also
// computes the two halo samples (n0-1, n0+64) for all 16 directions.
// P is summed over channels in index order with fma, like the oracle.
// ---------------------------------------------------------------------------
constexpr int kProjTN = 64;
constexpr int kProjTK = 16;

template <typename real, typename XT>
__global__ void __launch_bounds__(256)
k_project_extrema(const XT* __restrict__ X, const real* __restrict__ dir,
                  uint32_t* __restrict__ bits, Geom g, int k0, int Kc, Epochs ep)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int C = g.C;
    const int ldx = C + 1;  // odd stride: lanes reading different rows hit different banks
    real* xs = reinterpret_cast<real*>(smem_raw);          // (TN + 2) x ldx
    real* ds = xs + (kProjTN + 2) * ldx;                     // TK x C
    real* ps = ds + kProjTK * C;                              // TK x (TN + 2)
    const int n0 = blockIdx.x * kProjTN;
    const int kt0 = blockIdx.y * kProjTK;
    // tile loads: rows by warp, channels by lane (no division by C)
    for (int r = threadIdx.x >> 5; r < kProjTN + 2; r += blockDim.x >> 5) {
        const int n = n0 - 1 + r;
        for (int c = threadIdx.x & 31; c < C; c += 32)
            xs[r * ldx + c] = (n >= 0 && n < g.L) ? xval<real>(X[(size_t)n * C + c]) : real(0);
    }
    for (int kk = threadIdx.x >> 5; kk < kProjTK; kk += blockDim.x >> 5) {
        const int k = kt0 + kk;
        for (int c = threadIdx.x & 31; c < C; c += 32) ds[kk * C + c] = (k < Kc) ? dir[(size_t)(k0 + k) * C + c] : real(0);
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sg = warp & 1, dg = warp >> 1;
    {
        const int r = 1 + sg * 32 + lane;
        real acc[4] = {real(0), real(0), real(0), real(0)};
        const real* xr = xs + r * ldx;
        const real* d0 = ds + (dg * 4) * C;
        for (int c = 0; c < C; ++c) {
            const real xv = xr[c];
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[j] = fmad_(xv, d0[j * C + c], acc[j]);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) ps[(dg * 4 + j) * (kProjTN + 2) + r] = acc[j];
    }
    if (warp == 0) {
        const int side = lane >> 4, kk = lane & 15;
        const int r = side ? kProjTN + 1 : 0;
        real acc = real(0);
        const real* xr = xs + r * ldx;
        const real* dd = ds + kk * C;
        for (int c = 0; c < C; ++c) acc = fmad_(xr[c], dd[c], acc);
        ps[kk * (kProjTN + 2) + r] = acc;
    }
    __syncthreads();
    const int n = n0 + sg * 32 + lane;
    const int r = 1 + sg * 32 + lane;
    bool inrange, endpt, interior;
    sample_rule(g, ep, n, inrange, endpt, interior);
    const int w = (n0 >> 5) + sg;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int kk = dg * 4 + j;
        const real* pr = ps + kk * (kProjTN + 2);
        const real p = pr[r], pl = pr[r - 1], pn = pr[r + 1];
        const bool mx = inrange && (endpt || (interior && p > pl && p > pn));
        const bool mn = inrange && (endpt || (interior && p < pl && p < pn));
        const uint32_t wmax = __ballot_sync(kFull, mx);
        const uint32_t wmin = __ballot_sync(kFull, mn);
        if (lane == 0 && kt0 + kk < Kc && w < g.W) {
            bits[(size_t)(kt0 + kk) * g.W + w] = wmax;
            bits[(size_t)(Kc + kt0 + kk) * g.W + w] = wmin;
        }
    }
}

// Knot lists.  The bitmask of each (envelope, direction) is cut into chunks of
// kCompactChunk words; CTA (chunk, slot) of 512 threads writes the knots of its
// chunk (each thread an ordered run of words, a block scan of the popcounts,
// the offset of the chunk from k_compact_count's per-chunk totals) and gathers
// their values; the last CTA of a slot to arrive (an atomic counter, no
// waiting) writes the count, the trace entry, the mirrored knots and the
// end-point clamp.  A record of up to kCompactChunk words is one chunk and
// needs no count pass.
// ---------------------------------------------------------------------------
constexpr int kCompactChunk = 4096;

struct CompactShared {
    int* ctot;                 // [2 Kc][nch] interior knots per chunk
    unsigned long long* hacc;  // [2 Kc] trace hash partial sums (zero between launches)
    int* arrive;               // [2 Kc] CTAs done (zero between launches)
};

__global__ void __launch_bounds__(512)
k_compact_count(const uint32_t* __restrict__ bits, int* __restrict__ ctot, Geom g, int nch)
{
    const int chunk = blockIdx.x, slot = blockIdx.y;
    const uint32_t* b = bits + (size_t)slot * g.W;
    const int w0 = chunk * kCompactChunk, w1 = min(g.W, w0 + kCompactChunk);
    int local = 0;
    for (int w = w0 + (int)threadIdx.x; w < w1; w += blockDim.x) local += __popc(b[w]);
    local = warp_sum(local);
    __shared__ int ws[16];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) ws[wid] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += ws[i];
        ctot[(size_t)slot * nch + chunk] = t;
    }
}

template <typename real, typename XT>
__global__ void __launch_bounds__(512)
k_compact(const uint32_t* __restrict__ bits, int* __restrict__ wpref, int* __restrict__ knots,
          int* __restrict__ cnt, real* __restrict__ yv, const XT* __restrict__ X,
          memd_trace_entry* __restrict__ trace, Geom g, int k0, int Kc, RunState* st, int trace_rows,
          real* __restrict__ yend, Epochs ep, const int* __restrict__ mir, CompactShared cs, int nch)
{
    // yend != nullptr: the knot values are not gathered; only the two end
    // knots' values (clamped) are written, to yend[env][kk][2][C], and the
    // consumers read the interior knot values from X.
    // trace_rows > 0: trace is the base of a [trace_rows][K][2] array and the
    // row of this pass is st->trace_row (stop mode); otherwise trace points at
    // this pass's [K][2] block.
    // g.mirror: the knot list is [left mirrored | interior extrema | right
    // mirrored] (mir from k_mirror); wpref and the bitmask count the interior
    // extrema only, the knot values come from the mirrored knots' source
    // samples, and the reference's end-point clamp does not apply.
    const int chunk = blockIdx.x;
    const int slot_i = blockIdx.y;
    const int env = slot_i / Kc, kk = slot_i - env * Kc;
    const size_t slot = (size_t)slot_i;
    const uint32_t* b = bits + slot * g.W;
    int* wp = wpref + slot * (g.W + 1);
    int* kn = knots + slot * g.cap;
    const int* mi = g.mirror ? mir + (size_t)(k0 + kk) * kMirWords : nullptr;
    const int nlm = mi ? mi[kMirNl + env] : 0, nrm = mi ? mi[kMirNr + env] : 0;
    const int C = g.C;
    __shared__ int wsum[16];
    __shared__ unsigned long long hsum[16];
    __shared__ int total_s, off_s, last_s;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        int o = 0;
        for (int c = 0; c < chunk; ++c) o += cs.ctot[slot * nch + c];
        off_s = o;
    }
    const int cw0 = chunk * kCompactChunk, cw1 = min(g.W, cw0 + kCompactChunk);
    const int per = (cw1 - cw0 + blockDim.x - 1) / blockDim.x;
    const int wb = cw0 + threadIdx.x * per, we = min(cw1, wb + per);
    int local = 0;
    for (int w = wb; w < we; ++w) local += __popc(b[w]);
    int incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        const int v = lane < nw ? wsum[lane] : 0;
        int iv = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, iv, o);
            if (lane >= o) iv += t;
        }
        if (lane < nw) wsum[lane] = iv - v;
        if (lane == nw - 1) total_s = iv;
    }
    __syncthreads();
    const int off = off_s;
    int run = off + wsum[wid] + incl - local;
    uint64_t h = 0;
    for (int w = wb; w < we; ++w) {
        wp[w] = run;
        uint32_t word = b[w];
        while (word) {
            const int j = __ffs(word) - 1;
            word &= word - 1u;
            const int n = w * 32 + j;
            if (nlm + run < g.cap) kn[nlm + run] = n;
            ++run;
            h += splitmix64((uint64_t)(uint32_t)n);
        }
    }
    h = warp_sum<unsigned long long>(h);
    if (lane == 0) hsum[wid] = h;
    __syncthreads();
    // values of this chunk's interior knots, every channel (contiguous per knot)
    if (!yend) {
        real* y = yv + slot * (size_t)g.cap * C;
        const int i0 = nlm + off, i1 = min(g.cap, nlm + off + total_s);
        for (int idx = threadIdx.x; idx < (i1 - i0) * C; idx += blockDim.x) {
            const int i = i0 + idx / C, c = idx % C;
            y[(size_t)i * C + c] = xval<real>(X[(size_t)kn[i] * C + c]);
        }
    }
    unsigned long long hchunk = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) hchunk += hsum[i];
    // the last CTA of the slot finishes it
    if (nch > 1) {
        if (threadIdx.x == 0) atomicAdd(&cs.hacc[slot], hchunk);
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) last_s = (atomicAdd(&cs.arrive[slot], 1) == nch - 1);
        __syncthreads();
        if (!last_s) return;  // uniform over the CTA
        __threadfence();
    }
    // from here on, knots and prefix counts written by the slot's other CTAs
    // are read through L2 (__ldcg): this CTA's L1 may hold lines it read earlier
    if (threadIdx.x == 0) {
        int Eint = total_s;
        if (nch > 1) {
            Eint = 0;
            for (int c = 0; c < nch; ++c) Eint += __ldcg(&cs.ctot[slot * nch + c]);
        }
        unsigned long long htot = hchunk;
        if (nch > 1) {
            htot = __ldcg(&cs.hacc[slot]);
            cs.hacc[slot] = 0ull;
            cs.arrive[slot] = 0;
        }
        const int E = nlm + Eint + nrm;
        wp[g.W] = Eint;
        cnt[env * g.K + k0 + kk] = E;
        if (E > g.cap) atomicOr(&st->flags, 2);
        // mirrored knots: positions, and their part of the trace hash
        if (mi) {
            for (int j = 0; j < nlm; ++j) {
                const int pos = 2 * mi[kMirLsym] - mi[kMirLsrc + 2 * env + j];
                if (j < g.cap) kn[j] = pos;
                htot += splitmix64((uint64_t)(uint32_t)pos);
            }
            for (int j = 0; j < nrm; ++j) {
                const int pos = 2 * mi[kMirRsym] - mi[kMirRsrc + 2 * env + j];
                if (nlm + Eint + j < g.cap) kn[nlm + Eint + j] = pos;
                htot += splitmix64((uint64_t)(uint32_t)pos);
            }
        }
        memd_trace_entry* tr = trace;
        if (tr && trace_rows > 0) {
            const int r = st->trace_row;
            tr = (r >= 0 && r < trace_rows) ? tr + (size_t)r * g.K * 2 : nullptr;
        }
        if (tr) {
            memd_trace_entry e;
            e.count = E;
            e.flags = 0;
            e.hash = htot;
            tr[(size_t)(k0 + kk) * 2 + env] = e;
        }
        total_s = E;
        off_s = Eint;
    }
    __syncthreads();
    const int E = total_s, Eint = off_s;
    if (E > g.cap || E < 2) return;
    const int nrec = ep.n > 0 ? ep.n : 1;
    if (ep.n > 0) {
        for (int e = threadIdx.x; e < ep.n; e += blockDim.x)
            ep.cnt[((size_t)env * g.K + k0 + kk) * ep.n + e] = __ldcg(&wp[ep.w0[e + 1]]) - __ldcg(&wp[ep.w0[e]]);
    }
    if (mi) {
        // the mirrored knots' values from their source samples
        if (!yend) {
            real* y = yv + slot * (size_t)g.cap * C;
            for (int idx = threadIdx.x; idx < (nlm + nrm) * C; idx += blockDim.x) {
                const int j = idx / C, c = idx % C;
                const int i = j < nlm ? j : nlm + Eint + (j - nlm);
                const int src = j < nlm ? mi[kMirLsrc + 2 * env + j] : mi[kMirRsrc + 2 * env + (j - nlm)];
                y[(size_t)i * C + c] = xval<real>(X[(size_t)src * C + c]);
            }
        }
        return;
    }
    // The end-point clamp of the two end knots of each record (REF:447-486
    // max, 545-584 min); the raw end values were gathered with the chunks.
    for (int idx = threadIdx.x; idx < nrec * C; idx += blockDim.x) {
        const int e = idx / C, c = idx - e * C;
        const int kb = ep.n > 0 ? __ldcg(&wp[ep.w0[e]]) : 0;
        const int ke = ep.n > 0 ? __ldcg(&wp[ep.w0[e + 1]]) : E;  // the record's knots: kb .. ke - 1
        const int Er = ke - kb;
        const int* kr = kn + kb;
        const int x0 = __ldcg(&kr[0]), xE = __ldcg(&kr[Er - 1]);
        real v0 = xval<real>(X[(size_t)x0 * C + c]);
        real vE = xval<real>(X[(size_t)xE * C + c]);
        if (Er - 1 > 4) {
            const int x1 = __ldcg(&kr[1]), x2 = __ldcg(&kr[2]);
            const int xa = __ldcg(&kr[Er - 3]), xb = __ldcg(&kr[Er - 2]);
            const real v1 = xval<real>(X[(size_t)x1 * C + c]);
            const real v2 = xval<real>(X[(size_t)x2 * C + c]);
            real slope = div_(sub_(v2, v1), real(x2 - x1));
            real t = fmad_(-slope, real(x1 - x0), v1);
            if (env == 0 ? (t > v0) : (t < v0)) v0 = t;
            const real a = xval<real>(X[(size_t)xa * C + c]);
            const real bb = xval<real>(X[(size_t)xb * C + c]);
            slope = div_(sub_(bb, a), real(xb - xa));
            t = fmad_(slope, real(xE - xb), bb);
            if (env == 0 ? (t > vE) : (t < vE)) vE = t;
        }
        if (yend) {
            real* ye = yend + ((slot * nrec) + e) * 2 * (size_t)C;
            ye[c] = v0;
            ye[C + c] = vE;
        } else {
            real* y = yv + slot * (size_t)g.cap * C;
            y[(size_t)kb * C + c] = v0;
            y[(size_t)(ke - 1) * C + c] = vE;
        }
    }
}

// ---------------------------------------------------------------------------
// Channel-independent factorisation.  One thread per (envelope, direction,
// segment of Sf rows); the pivot recurrence starts Hf rows early (exact when
// the window reaches row 0, whose pivot is 1 with cp = 0; otherwise the
// start error decays by a factor u l / (2 (l + u) - l cp)^2 <= 1/12 per row,
// cp <= 1/2, l and u the row's neighbouring spacings; identity and
// not-a-knot end rows restart it).  rtab[h] = 1/h.
// ---------------------------------------------------------------------------
template <typename real, bool NAK>
__global__ void __launch_bounds__(128)
k_factor(const int* __restrict__ knots, const int* __restrict__ cnt, const real* __restrict__ rtab,
         Fac<real>* __restrict__ fac, Geom g, int k0, int Kc, int Sf, int Hf, int* __restrict__ cumcfg,
         Epochs ep, int cum_ctas)
{
    // cumcfg != nullptr (impulse-accumulation mean): block 0 picks the mean
    // kernel's anchor span, 32 m samples (m the largest power of two <= 4 with
    // 32 m <= 2 h, h the chunk's mean knot spacing, so that rounding carried
    // across a span grows by at most ~(32m/h)^2 = 4 over a direct evaluation;
    // at the densest knots m = 1), and splits each span's (direction,
    // envelope) pairs over P <= m CTAs
    if (cumcfg && blockIdx.x == 0 && threadIdx.x < 32) {
        int q = 0;
        long long et = 0;
        for (int k = threadIdx.x; k < Kc; k += 32) {
            const int a = cnt[k0 + k], b = cnt[g.K + k0 + k];
            if (a > 3 && b > 3) {
                ++q;
                et += a + b;
            }
        }
        q = warp_sum(q);
        et = warp_sum(et);
        if (threadIdx.x == 0) {
            int m = 1;
            if (et > 0) {
                const double h = (double)g.L * (2.0 * q) / (double)et;
                while (m < kCumMaxWords && 32.0 * (2 * m) <= 2.0 * h) m *= 2;
            }
            // parts per span: the fewest (a power of two <= m) that still give
            // the launch ~cum_ctas working CTAs (2048 unless tuned); a long
            // record or a batch has enough spans on its own, and every extra
            // part costs a flush of the span's accumulators
            const long spans = (long)((g.W + m - 1) / m) * ((g.C + 31) / 32);
            int P = m;
            while (P > 1 && spans * (P / 2) >= cum_ctas) P >>= 1;
            cumcfg[0] = m;
            cumcfg[1] = P;
        }
    }
    // thread = (segment, envelope, direction), the segment slowest so that
    // whole CTAs past the systems' knots exit at once; 32-bit index
    // arithmetic (the plan keeps the launch below 2^31 threads)
    const unsigned gid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nsys = 2u * (unsigned)Kc;
    const unsigned segu = gid / nsys;
    if (segu >= (unsigned)((g.cap + Sf - 1) / Sf)) return;
    const int seg = (int)segu;
    const int sys = (int)(gid - segu * nsys);
    const int env = sys >= Kc ? 1 : 0;
    const int kk = sys - env * Kc;
    const int E = cnt[env * g.K + k0 + kk];
    if (E > g.cap) return;
    const int i0 = seg * Sf;
    if (i0 >= E) return;
    const int i1 = min(E, i0 + Sf);
    const size_t slot = (size_t)env * Kc + kk;
    const int* x = knots + slot * g.cap;
    Fac<real>* f = fac + slot * g.cap;
    const int js = (Hf < 0) ? 0 : max(0, i0 - Hf);
    real cp = real(0);
    int xl = js > 0 ? x[js - 1] : 0;
    int xi = x[js];
    constexpr int FB = 8;  // knot positions loaded per batch (independent loads)
    // FULL (compile-time): all FB rows are owned (>= i0, < i1) and have a right
    // neighbour, so no row needs a guard
    // A batch in two phases: first every row's coefficients (small integers:
    // spacings, end conditions) and the reciprocal spacing of its right piece,
    // none of which depends on the pivots, so their loads and tests overlap;
    // then the pivot recurrence itself, the only serial part.
    auto batch = [&](auto full, int base) {
        constexpr bool FULL = decltype(full)::value;
        int xs[FB];
#pragma unroll
        for (int k = 0; k < FB; ++k) {
            const int i = base + k;
            xs[k] = (FULL || (i < i1 && i < E - 1)) ? x[i + 1] : 0;
        }
        int li[FB], di[FB], ui[FB];
        [[maybe_unused]] int wn[FB], wd[FB];  // not-a-knot rows: right-hand side weighted by wn / wd (wd > 0)
        real rt[FB];
#pragma unroll
        for (int k = 0; k < FB; ++k) {
            const int i = base + k;
            const bool act = FULL || i < i1;
            const int xr = (FULL || i < E - 1) ? xs[k] : xi;
            bool end;  // natural end conditions: s = 0
            [[maybe_unused]] bool nfirst = false, nlast = false;  // not-a-knot rows: second, second-to-last knot
            if (!NAK || ep.n == 0) {
                end = record_end_knot(ep, xi, i, E);
                if constexpr (NAK) {
                    nfirst = !end && E >= 4 && i == 1;
                    nlast = !end && E >= 4 && i == E - 2;
                }
            } else {
                // batched: the record's ends are knots, so knot i is its second
                // knot when its left neighbour is the record's first sample, and
                // the record has at least four knots when then its right
                // neighbour is not the last sample (and the mirror image)
                int rf, rl;
                record_bounds(ep, xi, rf, rl);
                end = xi == rf || xi == rl;
                nfirst = !end && xl == rf && xr != rl;
                nlast = !end && xr == rl && xl != rf;
            }
            const int hl = xi - xl, hr = xr - xi;
            li[k] = end ? 0 : hl;
            ui[k] = end ? 0 : hr;
            di[k] = end ? 1 : 2 * (hl + hr);
            if constexpr (NAK) {
                wn[k] = 0;
                wd[k] = 0;
                if (nfirst) {
                    // s_0 eliminated by the not-a-knot condition d_0 = d_1
                    li[k] = 0; di[k] = hl + 2 * hr; ui[k] = hr - hl;
                    wn[k] = hr; wd[k] = hl + hr;
                } else if (nlast) {
                    // s_{E-1} eliminated by d_{E-3} = d_{E-2}
                    li[k] = hl - hr; di[k] = 2 * hl + hr; ui[k] = 0;
                    wn[k] = hl; wd[k] = hl + hr;
                }
            }
            rt[k] = (act && (FULL || i < E - 1)) ? rtab[xr - xi] : real(0);
            if (act) {
                xl = xi;
                xi = xr;
            }
        }
#pragma unroll
        for (int k = 0; k < FB; ++k) {
            const int i = base + k;
            if (FULL || i < i1) {
                const real l = real(li[k]);
                const real gp = fmad_(-l, cp, real(di[k]));
                const real m = recip_(gp);
                cp = mul_(real(ui[k]), m);
                if (FULL || i >= i0) {
                    Fac<real> o;
                    o.m = m;
                    if constexpr (NAK) {
                        if (wd[k] > 0) o.m = mul_(m, div_(real(wn[k]), real(wd[k])));
                    }
                    o.lm = mul_(l, m);
                    o.cp = cp;
                    o.ih = (FULL || i < E - 1) ? fac_ih(rt[k]) : real(0);
                    f[i] = o;
                }
            }
        }
    };
    for (int base = js; base < i1; base += FB) {
        if (base >= i0 && base + FB <= i1 && base + FB < E) batch(std::true_type{}, base);
        else batch(std::false_type{}, base);
    }
}

// ---------------------------------------------------------------------------
// Substitution, as two kernels.  A warp handles one (envelope, direction,
// segment, group of 32 channels); each lane one channel (lanes past the last
// channel compute on a copy of it and store nothing).
//   k_solve_fwd: forward sweep over [i0-H, i1), writing the eliminated right
//                -hand side d of rows [i0, i1) to dbuf (and, in place, its
//                first H rows also to hz);
//   k_solve_bwd: backward sweep from i1+H-1 down to i0, reading d of the
//                segment and of the next segment's first H rows from dbuf
//                (in place: the latter from hz), writing the solution of rows
//                [i0, i1) to sv.  In place dbuf == sv: each warp reads a row's
//                d before it writes that row's solution, and no other warp
//                reads the row, so one [2][Kc][cap][C] array serves both.
// Rows go in batches of 8: every lane loads its 8 values at once, lanes
// 0..7 load the batch's factor rows, which the sweep takes by shuffle, so a
// batch costs one memory round trip instead of one per row.
// Both recurrences contract (multipliers <= 2/3 and <= 1/2 per row), so a
// window's truncated start perturbs the segment by at most that factor to the
// power H; the rows a thread reads from the next segment are that segment's
// own converged values, so the result does not depend on the segmentation.
// H < 0 selects the exact single-window solve.  Segments hold the longest
// power of two in [Ss, S] knots that leaves the system more than 16 segments
// (more, shorter segments keep the GPU busy when the knot sets are short;
// longer ones spend less on halos).  The segment index is the
// slowest grid index, so whole CTAs past the active segments exit at once.
// bnd != nullptr: raise bnd[c] (forward: max |y| over the segment's knots) and
// bnd[C + c] (backward: max h^2 (|s_i| + |s_{i+1}|) / 4 over its pieces), float
// bits; their sum bounds |S(n)| (the linear interpolant plus h^2/8 max|S''|).
// ---------------------------------------------------------------------------
constexpr int kSolveThreads = 128;
constexpr int kSolveBatch = 8;

struct SolveItem {
    int env, kk, seg, c, i0, i1, E;
    bool ok;
};

// Segment length of a system of E knots: the longest power of two in [Ss, S]
// that still gives it more than 16 segments (H < 0: one window over all).
__device__ __forceinline__ int solve_seg_len(int E, int cap, int S, int Ss, int H)
{
    if (H < 0) return cap;
    for (int t = S; t > Ss; t >>= 1)
        if (E > 16 * t) return t;
    return Ss;
}

// The most segments solve_seg_len gives a system of at most cap knots (the
// static grid's segment rows): systems of E in (16 t, hi] knots take segments
// of t, hi the smaller bound left by the longer segments, the rest take Ss.
__host__ __device__ inline long solve_segments_max(int cap, int S, int Ss, int H)
{
    if (H < 0) return 1;
    long m = 0;
    int hi = cap;
    for (int t = S; t > Ss; t >>= 1) {
        if (hi > 16 * t) m = m > (hi + t - 1) / t ? m : (hi + t - 1) / t;
        hi = hi < 16 * t ? hi : 16 * t;
    }
    const long r = (hi + Ss - 1) / Ss;
    return m > r ? m : r;
}

// Device work queue of the substitution (optional, memd_tuning.solve_queue):
// k_solve_queue writes, per pass, the segments before each (envelope,
// direction) slot; the persistent sweeps take items (segment x channel group)
// by atomic ticket until the pass runs out.  Without it (pref == nullptr)
// warp w of the launch is item w, over every segment the capacity allows.
struct SolveQueue {
    int* pref;    // [2 Kc + 1] segments before slot s (pref[2 Kc] = all segments)
    int* total;   // [1] items: segments x channel groups
    int* ticket;  // [2] next item of the forward and of the backward sweep
};

__device__ __forceinline__ SolveItem solve_item_of(int env, int kk, int seg, int cgi, const int* cnt, const Geom& g,
                                                   int k0, int S, int Ss, int H)
{
    SolveItem it;
    it.seg = seg;
    it.env = env;
    it.kk = kk;
    it.c = cgi * 32 + (int)(threadIdx.x & 31);
    it.ok = false;
    it.E = cnt[env * g.K + k0 + kk];
    if (it.E > g.cap || it.E < 2) return it;
    const int Se = solve_seg_len(it.E, g.cap, S, Ss, H);
    it.i0 = seg * Se;
    if (it.i0 >= it.E) return it;
    it.i1 = min(it.E, it.i0 + Se);
    it.ok = true;
    return it;
}

// static mapping: warp w of the launch = item w (segments up to the capacity;
// those past a system's knots exit)
__device__ __forceinline__ SolveItem solve_item(const int* cnt, const Geom& g, int k0, int Kc, int S, int Ss, int H,
                                                int ngroups)
{
    // 32-bit index arithmetic: the plan keeps the launch below 2^31 threads
    const unsigned gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // warp = item
    const unsigned ng = (unsigned)ngroups, nsl = 2u * (unsigned)Kc;
    const unsigned item = ng == 1u ? gw : gw / ng;
    const int cgi = (int)(gw - item * ng);
    const unsigned segu = item / nsl;
    const int slot = (int)(item - segu * nsl);
    const int seg = (int)segu;
    return solve_item_of(slot / Kc, slot % Kc, seg, cgi, cnt, g, k0, S, Ss, H);
}

// queue mapping: item = segment index over all slots x channel group; the
// slot by binary search in the prefix
__device__ __forceinline__ SolveItem solve_item_queued(int item, const SolveQueue& q, const int* cnt, const Geom& g,
                                                       int k0, int Kc, int S, int Ss, int H, int ngroups)
{
    const int cgi = item % ngroups;
    const int si = item / ngroups;
    int lo = 0, hi = 2 * Kc;  // pref[lo] <= si < pref[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&q.pref[mid]) <= si) lo = mid;
        else hi = mid;
    }
    return solve_item_of(lo / Kc, lo % Kc, si - __ldg(&q.pref[lo]), cgi, cnt, g, k0, S, Ss, H);
}

// The next item of this warp: the static mapping (one item, q.pref == nullptr)
// or the queue's next ticket; false when there is none.
__device__ __forceinline__ bool solve_next(SolveItem& it, bool& first, int which, const SolveQueue& q, const int* cnt,
                                           const Geom& g, int k0, int Kc, int S, int Ss, int H, int ngroups)
{
    if (!q.pref) {
        if (!first) return false;
        first = false;
        it = solve_item(cnt, g, k0, Kc, S, Ss, H, ngroups);
        return true;
    }
    int item = 0;
    if ((threadIdx.x & 31) == 0) item = atomicAdd(&q.ticket[which], 1);
    item = __shfl_sync(kFull, item, 0);
    if (item >= __ldcg(q.total)) return false;
    it = solve_item_queued(item, q, cnt, g, k0, Kc, S, Ss, H, ngroups);
    return true;
}

// One CTA of 1024 threads: segments per slot, their exclusive prefix, the item
// count, and both tickets reset for the pass.
__global__ void __launch_bounds__(1024)
k_solve_queue(const int* __restrict__ cnt, Geom g, int k0, int Kc, int S, int Ss, int H, int ngroups, SolveQueue q)
{
    __shared__ int wsum[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int base = 0; base < 2 * Kc; base += 1024) {
        const int slot = base + (int)threadIdx.x;
        int nseg = 0;
        if (slot < 2 * Kc) {
            const int env = slot / Kc, kk = slot - env * Kc;
            const int E = cnt[env * g.K + k0 + kk];
            if (E <= g.cap && E >= 2) {
                const int Se = solve_seg_len(E, g.cap, S, Ss, H);
                nseg = (E + Se - 1) / Se;
            }
        }
        int incl = nseg;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) wsum[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            const int v = wsum[lane];
            int iv = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(kFull, iv, o);
                if (lane >= o) iv += t;
            }
            wsum[lane] = iv - v;
        }
        __syncthreads();
        const int c0 = carry;
        if (slot < 2 * Kc) q.pref[slot] = c0 + wsum[wid] + incl - nseg;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c0 + wsum[wid] + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        q.pref[2 * Kc] = carry;
        *q.total = carry * ngroups;
        q.ticket[0] = 0;
        q.ticket[1] = 0;
    }
}

template <typename real, typename XT, bool XM, bool EPB, bool NAK>
__global__ void __launch_bounds__(kSolveThreads)
k_solve_fwd(const real* __restrict__ yv, const int* __restrict__ cnt, const Fac<real>* __restrict__ fac,
            real* __restrict__ dbuf, Geom g, int k0, int Kc, int S, int Ss, int H, int ngroups,
            unsigned* __restrict__ bnd, const XT* __restrict__ X, const int* __restrict__ knots,
            const real* __restrict__ yend, Epochs ep, real* __restrict__ hz, int hsegs, SolveQueue q)
{
    // hz != nullptr (the backward sweep solves in place in dbuf): the first H
    // rows of every segment also go to hz[slot][segment][H][C], the halo the
    // backward sweep of the segment before reads while this one's rows are
    // being overwritten by their solutions
    // XM: knot values read from the working signal, y_i = X[x_i] (interior
    // knots) and yend (the clamped end knots of each record), instead of yv;
    // EPB (with XM): batched epochs, a record's end knots found by position.
    // Rows of a record's end knots are the identity rows of the
    // factorisation (lm == 0): their right-hand side is 0.
    constexpr int B = kSolveBatch;
    SolveItem it;
    bool first = true;
    while (solve_next(it, first, 0, q, cnt, g, k0, Kc, S, Ss, H, ngroups)) {
    if (!it.ok) continue;  // uniform over the warp
    const int lane = threadIdx.x & 31;
    const int C = g.C, E = it.E, i0 = it.i0, i1 = it.i1;
    const bool cok = it.c < C;
    const int cl = min(it.c, C - 1);
    const size_t slot = (size_t)it.env * Kc + it.kk;
    const Fac<real>* f = fac + slot * g.cap;
    const real* y = XM ? nullptr : yv + slot * (size_t)g.cap * C + cl;
    const int* kn = knots + slot * g.cap;
    const int nrec = EPB ? ep.n : 1;
    const real* ye = XM ? yend + slot * nrec * 2 * (size_t)C + cl : nullptr;
    // (XM) knot r at sample n: its record and whether it is the record's
    // first (1) or last (2) knot
    auto endfl = [&](int r, int n, int& e) -> int {
        if constexpr (!EPB) {
            e = 0;
            return r == 0 ? 1 : (r == E - 1 ? 2 : 0);
        } else {
            e = ep.wep[n >> 5];
            const int o = ep.off[e];
            return n == o ? 1 : (n == o + ep.len[e] - 1 ? 2 : 0);
        }
    };
    auto yx = [&](int n, int fl, int e) -> real {
        if (fl) return ye[(size_t)e * 2 * C + (fl == 2 ? C : 0)];
        return xval<real>(X[(size_t)n * C + cl]);
    };
    auto yrow = [&](int r) -> real {
        if constexpr (!XM) {
            return y[(size_t)r * C];
        } else {
            const int n = kn[r];
            int e;
            const int fl = endfl(r, n, e);
            return yx(n, fl, e);
        }
    };
    real* o = dbuf + slot * (size_t)g.cap * C + cl;
    const int is = (H < 0) ? 0 : max(0, i0 - H);
    real yi = yrow(is);
    real slope_prev = real(0);
    if (is > 0) slope_prev = mul_(sub_(yi, yrow(is - 1)), f[is - 1].ih);
    real dprev = real(0);
    float ymax = 0.0f;
    // one batch of B rows; FULL (a compile-time flag): all B rows are owned
    // (>= i0), below i1 and have a right neighbour, so no row needs a guard
    // INNER (with FULL, one record): no row of the batch is the record's
    // first or last knot, so every knot value comes from the signal
    auto batch = [&](auto full, auto inner, int base) {
        constexpr bool FULL = decltype(full)::value;
        [[maybe_unused]] constexpr bool INNER = FULL && !EPB && decltype(inner)::value;
        const int nb = FULL ? B : min(B, i1 - base);
        real fm = real(0), flm = real(0), fih = real(0);
        int fx = 0, ffl = 0, fe = 0;
        if (lane < nb) {
            const Fac<real> fr = MEMD_CHECK(base + lane < g.cap) ? f[base + lane] : Fac<real>{};
            fm = fr.m;
            flm = fr.lm;
            fih = fr.ih;
            if (XM && base + 1 + lane < E) {
                fx = kn[base + 1 + lane];
                if (EPB) ffl = endfl(base + 1 + lane, fx, fe);
            }
        }
        real yb[B];
        // batched (EPB): a full batch none of whose knots ends a record (one
        // vote over the lanes' end flags) reads every value from the signal
        bool inner_rt = false;
        if constexpr (FULL && EPB && XM) inner_rt = !__any_sync(0xffffffffu, ffl != 0);
        if (inner_rt) {
#pragma unroll
            for (int k = 0; k < B; ++k) yb[k] = xval<real>(X[(size_t)__shfl_sync(0xffffffffu, fx, k) * C + cl]);
        } else if constexpr (XM) {
#pragma unroll
            for (int k = 0; k < B; ++k) {
                const int n = __shfl_sync(0xffffffffu, fx, k);
                if constexpr (INNER) {
                    yb[k] = xval<real>(X[(size_t)n * C + cl]);
                    continue;
                }
                int fl, e;
                if constexpr (EPB) {
                    fl = __shfl_sync(0xffffffffu, ffl, k);
                    e = __shfl_sync(0xffffffffu, fe, k);
                } else {
                    fl = endfl(base + 1 + k, n, e);
                }
                yb[k] = (FULL || (k < nb && base + 1 + k < E)) ? yx(n, fl, e) : real(0);
            }
        } else {
#pragma unroll
            for (int k = 0; k < B; ++k)
                yb[k] = (FULL || (k < nb && base + 1 + k < E)) ? y[(size_t)(base + 1 + k) * C] : real(0);
        }
#pragma unroll
        for (int k = 0; k < B; ++k) {
            const real m = shfl_idx_(fm, k), lm = shfl_idx_(flm, k), ih = shfl_idx_(fih, k);
            if (FULL || k < nb) {
                const int i = base + k;
                const real ynext = yb[k];
                real slope = real(0), r = real(0);
                if (FULL || i < E - 1) slope = mul_(sub_(ynext, yi), ih);
                // identity rows (record ends) have lm = 0 and m = 1; a not-a-knot
                // row 1 also has lm = 0, so NAK tells them apart by m
                if (NAK ? !is_one(m) : !is_zero(lm)) {
                    if constexpr (kFacIh3<real>) r = sub_(slope, slope_prev);  // slopes carry the factor 3
                    else r = mul_(real(3), sub_(slope, slope_prev));
                }
                const real dcur = fmad_(-lm, dprev, mul_(m, r));
                // rows before i0 only warm the recurrence up
                if (FULL || i >= i0) {
                    if (cok && MEMD_CHECK(i >= 0 && i < g.cap)) o[(size_t)i * C] = dcur;
                    ymax = fmaxf(ymax, magf(yi));
                }
                slope_prev = slope;
                yi = ynext;
                dprev = dcur;
            }
        }
    };
    for (int base = is; base < i1; base += B) {
        const bool full = base >= i0 && base + B <= i1 && base + B < E;
        if constexpr (XM && !EPB) {
            if (full && base + B < E - 1) batch(std::true_type{}, std::true_type{}, base);
            else if (full) batch(std::true_type{}, std::false_type{}, base);
            else batch(std::false_type{}, std::false_type{}, base);
        } else {
            if (full) batch(std::true_type{}, std::false_type{}, base);
            else batch(std::false_type{}, std::false_type{}, base);
        }
    }
    if (bnd && cok) {
        if (i1 < E) ymax = fmaxf(ymax, magf(yi));  // right end of the last piece
        atomicMax(&bnd[it.c], __float_as_uint(ymax * 1.01f));
    }
    if (hz && cok && i0 > 0 && MEMD_CHECK(it.seg < hsegs)) {  // the halo of the segment before, set aside
        real* hs = hz + (((size_t)slot * hsegs + it.seg) * H) * C + cl;
        const int nh = min(H, i1 - i0);
        for (int r = 0; r < nh; ++r) hs[(size_t)r * C] = o[(size_t)(i0 + r) * C];
    }
    }  // items
}

template <typename real, bool NAK, bool INPL>
__global__ void __launch_bounds__(kSolveThreads)
k_solve_bwd(const int* __restrict__ cnt, const Fac<real>* __restrict__ fac, const real* __restrict__ dbuf,
            real* __restrict__ sv, Geom g, int k0, int Kc, int S, int Ss, int H, int ngroups,
            unsigned* __restrict__ bnd, const int* __restrict__ knots, const real* __restrict__ hz, int hsegs,
            SolveQueue q)
{
    // INPL (dbuf unused): the eliminated right-hand side is in sv,
    // each row's read by the same warp just before it writes the row's
    // solution there; the next segment's first H rows (the halo) come from
    // hz, copied there by the forward sweep, since that segment's own warp
    // overwrites them.
    // NAK (not-a-knot end conditions, g.nak), E >= 4: rows 0 and E-1 were solved as
    // identity rows; s_0 = s_1 + (h_0 / h_1)(s_1 - s_2) is applied at row 0,
    // and s_{E-1} = s_{E-2} + (h_{E-2} / h_{E-3})(s_{E-2} - s_{E-3}) by the
    // warp that owns row E-3 (its window always reaches row E-1, and row E-2
    // does not depend on s_{E-1}), which also writes row E-1.
    constexpr int B = kSolveBatch;
    SolveItem it;
    bool first = true;
    while (solve_next(it, first, 1, q, cnt, g, k0, Kc, S, Ss, H, ngroups)) {
    if (!it.ok) continue;  // uniform over the warp
    const int lane = threadIdx.x & 31;
    const int C = g.C, E = it.E, i0 = it.i0, i1 = it.i1;
    const bool cok = it.c < C;
    const int cl = min(it.c, C - 1);
    const size_t slot = (size_t)it.env * Kc + it.kk;
    const Fac<real>* f = fac + slot * g.cap;
    const real* d = (INPL ? sv : dbuf) + slot * (size_t)g.cap * C + cl;
    real* o = sv + slot * (size_t)g.cap * C + cl;
    const int* kn = knots + slot * g.cap;
    const bool nak = NAK && E >= 4;
    // the next segment's first rows, as the forward sweep left them
    const real* hzs = (INPL && hz && i1 < E && MEMD_CHECK(it.seg + 1 < hsegs))
                          ? hz + (((size_t)slot * hsegs + it.seg + 1) * H) * C + cl
                          : nullptr;
    const int ie = (H < 0) ? E : min(E, i1 + H);
    real snext = real(0), snext2 = real(0);
    float spart = 0.0f;
    // one batch of B rows from top down; FULL (a compile-time flag): all B
    // rows are owned (>= i0, < i1) and have a right neighbour
    auto batch = [&](auto full, int top) {
        constexpr bool FULL = decltype(full)::value;
        const int nb = FULL ? B : min(B, top - i0 + 1);
        real fcp = real(0), fih = real(0);
        if (lane < nb) {
            const Fac<real> fr = MEMD_CHECK(top - lane >= 0 && top - lane < g.cap) ? f[top - lane] : Fac<real>{};
            fcp = fr.cp;
            fih = fr.ih;
        }
        real db[B];
#pragma unroll
        for (int k = 0; k < B; ++k)
            db[k] = ((FULL || k < nb) && MEMD_CHECK(top - k >= 0 && top - k < g.cap))
                        ? ((hzs && top - k >= i1) ? hzs[(size_t)(top - k - i1) * C] : d[(size_t)(top - k) * C])
                        : real(0);
#pragma unroll
        for (int k = 0; k < B; ++k) {
            const real cp = shfl_idx_(fcp, k), ihr = shfl_idx_(fih, k);
            if (FULL || k < nb) {
                const int i = top - k;
                real sol = fmad_(-cp, snext, db[k]);
                if constexpr (NAK) {
                    if (nak && i == 0)
                        sol = add_(snext, div_(mul_(sub_(snext, snext2), real(kn[1] - kn[0])), real(kn[2] - kn[1])));
                }
                if (FULL || i < i1) {
                    if (cok && !(NAK && nak && i == E - 1) && MEMD_CHECK(i >= 0 && i < g.cap)) o[(size_t)i * C] = sol;
                    if (bnd && (FULL || i < E - 1)) {
                        // h^2 = 1 / ih^2 (9 / ih^2 when ih holds 3/h); the approximate
                        // division's error is inside the 1.01 margin applied at the end
                        const float ih = magf(ihr);
                        spart = fmaxf(spart, __fdividef((kFacIh3<real> ? 2.25f : 0.25f) * (magf(sol) + magf(snext)), ih * ih));
                    }
                    if constexpr (NAK) {
                        if (nak && i == E - 3) {
                            const int hb = kn[E - 1] - kn[E - 2];
                            const real sl =
                                add_(snext, div_(mul_(sub_(snext, sol), real(hb)), real(kn[E - 2] - kn[E - 3])));
                            if (cok) o[(size_t)(E - 1) * C] = sl;
                            if (bnd) spart = fmaxf(spart, 0.25f * (magf(snext) + magf(sl)) * (float)hb * (float)hb);
                        }
                    }
                }
                if constexpr (NAK) snext2 = snext;
                snext = sol;
            }
        }
    };
    for (int top = ie - 1; top >= i0; top -= B) {
        if (!NAK && top - B + 1 >= i0 && top < i1 && top < E - 1) batch(std::true_type{}, top);
        else batch(std::false_type{}, top);
    }
    if (bnd && cok) atomicMax(&bnd[C + it.c], __float_as_uint(spart * 1.01f));
    }  // items
}

// ---------------------------------------------------------------------------
// Not-a-knot ends of the records of a batched run.  The factorisation solved
// each record's first and last knot as identity rows and eliminated them from
// the record's second and second-to-last rows, so the sweeps give every other
// row; this kernel sets, per (envelope, direction, record, channel) of a
// record with at least four knots,
//     s_b   = s_b+1 + (s_b+1 - s_b+2) h_b / h_b+1          (d_b = d_b+1)
//     s_e-1 = s_e-2 + (s_e-2 - s_e-3) h_e-2 / h_e-3        (d_e-3 = d_e-2)
// (b .. e-1 the record's knots, h_i = x_i+1 - x_i) with the single-record
// backward sweep's arithmetic, and raises the mean's bound bnd[C + c] by the
// two end pieces as that sweep does.
// ---------------------------------------------------------------------------
template <typename real>
__global__ void __launch_bounds__(128)
k_nak_ends(const int* __restrict__ knots, const int* __restrict__ cnt, const int* __restrict__ wpref,
           const Fac<real>* __restrict__ fac, real* __restrict__ sv, Geom g, int k0, int Kc, Epochs ep,
           unsigned* __restrict__ bnd)
{
    const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int C = g.C;
    const long per_slot = (long)ep.n * C;
    const int slot = (int)(gid / per_slot);
    if (slot >= 2 * Kc) return;
    const long r = gid - (long)slot * per_slot;
    const int e = (int)(r / C), c = (int)(r - (long)e * C);
    const int env = slot >= Kc ? 1 : 0, kk = slot - env * Kc;
    if (cnt[env * g.K + k0 + kk] > g.cap) return;
    const int* wp = wpref + (size_t)slot * (g.W + 1);
    const int b = wp[ep.w0[e]], en = wp[ep.w0[e + 1]];  // the record's knots: b .. en - 1
    if (en - b < 4) return;
    const int* kn = knots + (size_t)slot * g.cap;
    real* s = sv + (size_t)slot * g.cap * C + c;
    const Fac<real>* f = fac + (size_t)slot * g.cap;
    const real s1 = s[(size_t)(b + 1) * C], s2 = s[(size_t)(b + 2) * C];
    const real s0 = add_(s1, div_(mul_(sub_(s1, s2), real(kn[b + 1] - kn[b])), real(kn[b + 2] - kn[b + 1])));
    const real sa = s[(size_t)(en - 3) * C], sb = s[(size_t)(en - 2) * C];
    const int hb = kn[en - 1] - kn[en - 2];
    const real sl = add_(sb, div_(mul_(sub_(sb, sa), real(hb)), real(kn[en - 2] - kn[en - 3])));
    s[(size_t)b * C] = s0;
    s[(size_t)(en - 1) * C] = sl;
    if (bnd) {
        const float ih = magf(f[b].ih);
        float v = __fdividef((kFacIh3<real> ? 2.25f : 0.25f) * (magf(s0) + magf(s1)), ih * ih);
        v = fmaxf(v, 0.25f * (magf(sb) + magf(sl)) * (float)hb * (float)hb);
        atomicMax(&bnd[C + c], __float_as_uint(v * 1.01f));
    }
}

// ---------------------------------------------------------------------------
// Envelope evaluation fused with the mean over directions and the update.
// CTA: T = (256/G)*SPT samples x G channels; thread (row, ch) owns SPT
// consecutive samples of one channel and keeps their running sum over the
// directions in registers.  Per (direction, envelope):
//   (a) the tile's knots, 1/h and bit words into shared memory,
//   (b) interval index and offset t per sample; coefficients
//       a = y_i, b = (y_{i+1}-y_i)/h - h(2 s_i + s_{i+1})/3, c = s_i,
//       d = (s_{i+1} - s_i)/(3h) per (interval, channel),
//   (c) S = fma(fma(fma(d, t, c), t, b), t, a) per (sample, channel).
// The sum over qualified directions (E_max > 3 && E_min > 3) runs in
// direction order; the last chunk applies X -= (sum/2)/Q (REF:832-864).
// ---------------------------------------------------------------------------
template <typename real, int G, int SPT>
struct EvalShape {
    static constexpr int NR = 256 / G;
    static constexpr int T = NR * SPT;
    static constexpr int MI = T / 2 + 4;
    static size_t smem_bytes(int Kc, bool mirror)
    {
        return sizeof(real) * ((size_t)MI * 4 * G + T + MI) +
               sizeof(int) * ((size_t)(MI + 1) + T + T / 32 + 8 * Kc + 4 + (mirror ? 10 * Kc : 0));
    }
};

// Mirror boundary: knots before sample n among the mirrored ones (positions
// lp0 <= lp1 left, rp0 <= rp1 right; INT_MAX where absent).  The interval of
// sample n is (this + interior knots before n) - 1, clamped to [0, E - 2].
__device__ __forceinline__ int mirror_before(int n, int lp0, int lp1, int rp0, int rp1)
{
    return (lp0 < n) + (lp1 < n) + (rp0 < n) + (rp1 < n);
}
// the mirrored knot positions of a (direction, envelope) with E knots
__device__ __forceinline__ void mirror_positions(const int* __restrict__ mi, const int* __restrict__ kn, int env, int E,
                                                 int& lp0, int& lp1, int& rp0, int& rp1)
{
    const int nl = mi[kMirNl + env], nr = mi[kMirNr + env];
    lp0 = nl > 0 ? kn[0] : INT_MAX;
    lp1 = nl > 1 ? kn[1] : INT_MAX;
    rp0 = nr > 0 ? kn[E - nr] : INT_MAX;
    rp1 = nr > 1 ? kn[E - 1] : INT_MAX;
}

template <typename real, int G, int SPT>
__global__ void __launch_bounds__(256)
k_eval(real* __restrict__ X, real* __restrict__ acc_buf, const uint32_t* __restrict__ bits,
       const int* __restrict__ wpref, const int* __restrict__ knots, const int* __restrict__ cnt,
       const Fac<real>* __restrict__ fac, const real* __restrict__ sv, const real* __restrict__ yv, Geom g,
       int k0, int Kc, int first_chunk, int last_chunk, RunState* st, real* __restrict__ M,
       real* __restrict__ part, Epochs ep, const int* __restrict__ mir)
{
    // M == nullptr: fixed mode, the last chunk updates X in place.
    // g.mirror: intervals count the mirrored knots too (mirror_before).
    // M != nullptr: stop mode, the last chunk writes the mean envelope to M and
    // every chunk writes part[cg][kk][n] = sum over this CTA's channels of
    // (U - L)^2 for the amplitude statistic.
    using Sh = EvalShape<real, G, SPT>;
    constexpr int T = Sh::T;
    constexpr int MI = Sh::MI;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    real* coef = reinterpret_cast<real*>(smem_raw);  // [MI][4][G]
    real* tts = coef + MI * 4 * G;                    // [T]
    real* ihs = tts + T;                              // [MI]
    int* kx = reinterpret_cast<int*>(ihs + MI);       // [MI + 1]
    int* lis = kx + MI + 1;                           // [T]
    uint32_t* wds = reinterpret_cast<uint32_t*>(lis + T);  // [T/32]
    int* tab = reinterpret_cast<int*>(wds + T / 32);  // [2*Kc][3]; batched: + [1] + [2*Kc] record knot bases
    int* sQ = tab + 6 * Kc;
    int* mtab = tab + 8 * Kc + 4;                      // mirror: [2*Kc][5] lp0, lp1, rp0, rp1, E

    const int n0 = blockIdx.x * T;
    const int cg = blockIdx.y;
    const int cc = threadIdx.x % G;
    const int row = threadIdx.x / G;
    const int c = cg * G + cc;
    const bool cok = c < g.C;
    // the tile's record (epoch): tiles (T | 512) never straddle two
    const int rec = ep.n > 0 ? ep.wep[n0 >> 5] : 0;
    const int rend = ep.n > 0 ? ep.off[rec] + ep.len[rec] : g.L;
    if (n0 >= rend) return;  // gap between epochs; uniform over the CTA
    const int nl = min(T, rend - n0);
    const int C = g.C;
    const real third = real(1.0 / 3.0);

    for (int idx = threadIdx.x; idx < 2 * Kc; idx += blockDim.x) {
        const int env = idx / Kc, kk = idx - env * Kc;
        const size_t slot = (size_t)env * Kc + kk;
        const int* wp = wpref + slot * (g.W + 1);
        const uint32_t* b = bits + slot * g.W;
        // pieces of the record only: kb .. ke - 2 (n at the record's first sample uses its first piece)
        const int kb = ep.n > 0 ? wp[ep.w0[rec]] : 0;
        const int cl0 = wp[n0 >> 5];
        const int nlast = n0 + nl - 1;
        const int wl = nlast >> 5, jl = nlast & 31;
        const int cll = wp[wl] + __popc(b[wl] & ((1u << jl) - 1u));
        tab[idx * 3 + 0] = max(cl0 - 1, kb);
        tab[idx * 3 + 1] = max(cll - 1, kb);
        tab[idx * 3 + 2] = cl0;
        if (ep.n > 0) tab[6 * Kc + 1 + idx] = kb;
        if (g.mirror) {
            const int E = cnt[env * g.K + k0 + kk];
            int lp0 = INT_MAX, lp1 = INT_MAX, rp0 = INT_MAX, rp1 = INT_MAX;
            if (E >= 2 && E <= g.cap) {
                mirror_positions(mir + (size_t)(k0 + kk) * kMirWords, knots + slot * g.cap, env, E, lp0, lp1, rp0, rp1);
                tab[idx * 3 + 0] = min(max(mirror_before(n0, lp0, lp1, rp0, rp1) + cl0 - 1, 0), E - 2);
                tab[idx * 3 + 1] = min(max(mirror_before(nlast, lp0, lp1, rp0, rp1) + cll - 1, 0), E - 2);
            }
            int* mt = mtab + idx * 5;
            mt[0] = lp0;
            mt[1] = lp1;
            mt[2] = rp0;
            mt[3] = rp1;
            mt[4] = E;
        }
    }
    if (threadIdx.x < 32) {
        int q = 0;
        for (int k = threadIdx.x; k < g.K; k += 32) q += dir_qualifies(g, ep, cnt, k, rec) ? 1 : 0;
        q = warp_sum(q);
        if (threadIdx.x == 0) sQ[0] = q;
    }
    real acc[SPT];
    real u[SPT];
#pragma unroll
    for (int j = 0; j < SPT; ++j) {
        const int t = row * SPT + j;
        acc[j] = real(0);
        u[j] = real(0);
        if (!first_chunk && cok && t < nl) acc[j] = acc_buf[(size_t)(n0 + t) * C + c];
    }
    __syncthreads();

    for (int kk = 0; kk < Kc; ++kk) {
        const int k = k0 + kk;
        const int Emax = cnt[k], Emin = cnt[g.K + k];
        if (!dir_qualifies(g, ep, cnt, k, rec)) continue;
        if (Emax > g.cap || Emin > g.cap) continue;
#pragma unroll
        for (int env = 0; env < 2; ++env) {
            const size_t slot = (size_t)env * Kc + kk;
            const int ia = tab[(env * Kc + kk) * 3 + 0];
            const int ib = tab[(env * Kc + kk) * 3 + 1];
            const int cl0 = tab[(env * Kc + kk) * 3 + 2];
            int m = ib - ia + 1;
            if (m > MI - 1) {
                if (threadIdx.x == 0) atomicOr(&st->flags, 2);
                m = MI - 1;
            }
            const int* kn = knots + slot * g.cap;
            const Fac<real>* fc = fac + slot * g.cap;
            const real* svs = sv + slot * (size_t)g.cap * C;
            const real* yvs = yv + slot * (size_t)g.cap * C;
            const uint32_t* b = bits + slot * g.W;
            __syncthreads();
            for (int j = threadIdx.x; j <= m; j += blockDim.x) kx[j] = kn[ia + j];
            for (int j = threadIdx.x; j < m; j += blockDim.x) ihs[j] = fc[ia + j].ih;
            if (threadIdx.x < T / 32) {
                const int w = (n0 >> 5) + threadIdx.x;
                wds[threadIdx.x] = (w < g.W) ? b[w] : 0u;
            }
            __syncthreads();
            for (int t = threadIdx.x; t < nl; t += blockDim.x) {
                const int w = t >> 5, jb = t & 31;
                int cntl = 0;
                for (int q = 0; q < w; ++q) cntl += __popc(wds[q]);
                cntl += __popc(wds[w] & ((1u << jb) - 1u));
                int iv = max(cl0 + cntl - 1, ep.n > 0 ? tab[6 * Kc + 1 + env * Kc + kk] : 0);
                if (g.mirror) {
                    const int* mt = mtab + (env * Kc + kk) * 5;
                    iv = min(max(mirror_before(n0 + t, mt[0], mt[1], mt[2], mt[3]) + cl0 + cntl - 1, 0), mt[4] - 2);
                }
                int li = iv - ia;
                li = min(li, m - 1);
                lis[t] = li;
                tts[t] = real(n0 + t - kx[li]);
            }
            for (int it = threadIdx.x; it < m * G; it += blockDim.x) {
                const int li = it / G, ch = it - li * G;
                const int cch = cg * G + ch;
                if (cch < C) {
                    const int i = ia + li;
                    const real s0 = svs[(size_t)i * C + cch], s1 = svs[(size_t)(i + 1) * C + cch];
                    const real y0 = yvs[(size_t)i * C + cch], y1 = yvs[(size_t)(i + 1) * C + cch];
                    const real h = real(kx[li + 1] - kx[li]);
                    const real ih = ihs[li];
                    const real slope = mul_(sub_(y1, y0), ih);
                    const real bq = fmad_(-mul_(h, third), fmad_(real(2), s0, s1), slope);
                    const real dq = mul_(sub_(s1, s0), mul_(ih, third));
                    real* cf = coef + (size_t)li * 4 * G + ch;
                    cf[0] = y0;
                    cf[G] = bq;
                    cf[2 * G] = s0;
                    cf[3 * G] = dq;
                }
            }
            __syncthreads();
            if (cok) {
#pragma unroll
                for (int j = 0; j < SPT; ++j) {
                    const int t = row * SPT + j;
                    if (t < nl) {
                        const int li = lis[t];
                        const real tt = tts[t];
                        const real* cf = coef + (size_t)li * 4 * G + cc;
                        const real v = fmad_(fmad_(fmad_(cf[3 * G], tt, cf[2 * G]), tt, cf[G]), tt, cf[0]);
                        if (env == 0) {
                            u[j] = v;
                        } else {
                            acc[j] = add_(acc[j], add_(u[j], v));
                            if (M) u[j] = sub_(u[j], v);  // spread U - L for the amplitude
                        }
                    }
                }
            }
            if (M && env == 1) {
                // sum of squared spreads over the G channels of each sample row
#pragma unroll
                for (int j = 0; j < SPT; ++j) {
                    const int t = row * SPT + j;
                    real d2 = (cok && t < nl) ? mul_(u[j], u[j]) : real(0);
#pragma unroll
                    for (int o = 1; o < G; o <<= 1) d2 = add_(d2, shfl_xor_(d2, o));
                    if (cc == 0 && t < nl) part[((size_t)cg * Kc + kk) * g.L + n0 + t] = d2;
                }
            }
        }
    }
    const int Q = sQ[0];
    if (!M && last_chunk && Q == 0 && (blockIdx.x == 0 || ep.n > 0) && blockIdx.y == 0 && threadIdx.x == 0)
        atomicOr(&st->flags, 1);
    if (!cok) return;
#pragma unroll
    for (int j = 0; j < SPT; ++j) {
        const int t = row * SPT + j;
        if (t < nl) {
            const size_t idx = (size_t)(n0 + t) * C + c;
            if (last_chunk) {
                const real val = mul_(acc[j], real(0.5));
                if (M) M[idx] = div_(val, real(Q));
                else X[idx] = sub_(X[idx], div_(val, real(Q)));
            } else {
                acc_buf[idx] = acc[j];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Envelope evaluation, FP32 arithmetic, one warp per direction.
// CTA: T = (32/G)*SPL samples x G channels, 8 warps; warp w handles the
// directions w, w+8, ... of the chunk on its own (no block barrier inside the
// direction loop), so the load latency of one direction is covered by the
// other warps' work.  Per (direction, envelope) a warp stages the tile's
// knots, knot values and solutions in its shared-memory slice, then every
// lane walks its SPL consecutive samples of one channel, recomputing the
// cubic's coefficients when the interval changes.  The warps' partial sums
// are added in warp order at the end (a pairwise sum over the directions).
// X is float (FP32 path) or float2 (double-float, mixed path).
// ---------------------------------------------------------------------------
template <int G, int SPL, typename R>
struct EvalWShape {
    static constexpr int NS = 32 / G;
    static constexpr int T = NS * SPL;
    static constexpr int MI = T / 2 + 4;
    static constexpr int WARPS = 8;
    static constexpr int NW = T / 32;
    // per warp: accumulator tile, (stop mode) spread tile, knots, bit words
    __host__ __device__ static constexpr size_t per_warp(bool stopm)
    {
        return (size_t)(stopm ? 2 : 1) * sizeof(R) * T * G + sizeof(int) * (MI + 1) + sizeof(uint32_t) * (NW + 1);
    }
    static size_t smem_bytes(bool stopm) { return WARPS * ((per_warp(stopm) + 15) / 16 * 16); }
};

template <int G, int SPL, typename XT, typename R, bool STOPM>
__global__ void __launch_bounds__(256)
k_eval_w(XT* __restrict__ X, R* __restrict__ acc_buf, const uint32_t* __restrict__ bits,
         const int* __restrict__ wpref, const int* __restrict__ knots, const int* __restrict__ cnt,
         const R* __restrict__ rtab, const R* __restrict__ sv, const R* __restrict__ yv, Geom g,
         int k0, int Kc, int first_chunk, int last_chunk, RunState* st, R* __restrict__ M,
         R* __restrict__ part, const int* __restrict__ mir, Epochs ep)
{
    // g.mirror: intervals count the mirrored knots too (mirror_before).
    // ep.n > 0 (batched): a tile (T | 512) lies in one record; pieces, the
    // qualified directions and Q are the record's own.
    using Sh = EvalWShape<G, SPL, R>;
    constexpr int T = Sh::T;
    constexpr int MI = Sh::MI;
    constexpr int NW = Sh::NW;
    constexpr size_t PW = (Sh::per_warp(STOPM) + 15) / 16 * 16;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int sQ;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cc = lane % G, sgrp = lane / G;
    const int n0 = blockIdx.x * T, cg = blockIdx.y;
    const int c = cg * G + cc;
    const bool cok = c < g.C;
    const int rec = ep.n > 0 ? ep.wep[n0 >> 5] : 0;
    const int rend = ep.n > 0 ? ep.off[rec] + ep.len[rec] : g.L;
    if (n0 >= rend) return;  // gap between epochs; uniform over the CTA
    const int nl = min(T, rend - n0);
    const int C = g.C;
    const int w0 = n0 >> 5;
    unsigned char* wb = smem_raw + (size_t)warp * PW;
    R* accs = reinterpret_cast<R*>(wb);                        // [T][G]
    R* us = accs + (STOPM ? T * G : 0);                        // [T][G] (stop mode)
    int* kx = reinterpret_cast<int*>(accs + (STOPM ? 2 : 1) * T * G);
    uint32_t* wd = reinterpret_cast<uint32_t*>(kx + MI + 1);
    if (warp == 0) {
        int q = 0;
        for (int k = lane; k < g.K; k += 32) q += dir_qualifies(g, ep, cnt, k, rec) ? 1 : 0;
        q = warp_sum(q);
        if (lane == 0) sQ = q;
    }
    const int s_first = sgrp * SPL;
    for (int j = 0; j < SPL; ++j) accs[(s_first + j) * G + cc] = R(0.0f);
    const R third = R(1.0 / 3.0);
    const R* yc = yv + c;
    const R* sc = sv + c;
    bool overflow = false;

    for (int kk = warp; kk < Kc; kk += Sh::WARPS) {
        const int k = k0 + kk;
        if (!dir_qualifies(g, ep, cnt, k, rec)) continue;
        if (cnt[k] > g.cap || cnt[g.K + k] > g.cap) continue;
        for (int env = 0; env < 2; ++env) {
            const size_t slot = (size_t)env * Kc + kk;
            const int* wp = wpref + slot * (g.W + 1);
            const uint32_t* b = bits + slot * g.W;
            const int cl0 = wp[w0];
            const int kb = ep.n > 0 ? wp[ep.w0[rec]] : 0;  // the record's first knot
            const uint32_t myw = (lane < NW && w0 + lane < g.W) ? b[w0 + lane] : 0u;
            const int nlast = nl - 1;
            int cnt_last = 0;
#pragma unroll
            for (int q = 0; q < NW; ++q) {
                const uint32_t w = __shfl_sync(kFull, myw, q);
                if (32 * q + 32 <= nlast) cnt_last += __popc(w);
                else if (32 * q < nlast) cnt_last += __popc(w & ((1u << (nlast - 32 * q)) - 1u));
            }
            int ia = max(cl0 - 1, kb);
            int ib = max(cl0 + cnt_last - 1, kb);
            const int Ee = cnt[env * g.K + k];
            int lp0 = INT_MAX, lp1 = INT_MAX, rp0 = INT_MAX, rp1 = INT_MAX;
            if (g.mirror) {
                mirror_positions(mir + (size_t)k * kMirWords, knots + slot * g.cap, env, Ee, lp0, lp1, rp0, rp1);
                ia = min(max(mirror_before(n0, lp0, lp1, rp0, rp1) + cl0 - 1, 0), Ee - 2);
                ib = min(max(mirror_before(n0 + nlast, lp0, lp1, rp0, rp1) + cl0 + cnt_last - 1, 0), Ee - 2);
            }
            int m = ib - ia + 1;
            if (m > MI - 1) {
                overflow = true;
                m = MI - 1;
            }
            const int* kn = knots + slot * g.cap;
            const size_t base = (slot * (size_t)g.cap + ia) * C;  // knot ia, channel 0
            __syncwarp();
            for (int j = lane; j <= m; j += 32) kx[j] = kn[ia + j];
            if (lane < NW) wd[lane] = myw;
            __syncwarp();
            int cntb = 0;
#pragma unroll
            for (int q = 0; q < NW; ++q) {
                const uint32_t w = wd[q];
                if (32 * q + 32 <= s_first) cntb += __popc(w);
                else if (32 * q < s_first) cntb += __popc(w & ((1u << (s_first - 32 * q)) - 1u));
            }
            int cur = -2, x0 = 0;  // -2: no interval loaded yet (li >= 0 never equals cur + 1)
            R ca = R(0.0f), cb = R(0.0f), c2 = R(0.0f), cd = R(0.0f);
            R ynx = R(0.0f), snx = R(0.0f);  // values at knot cur + 1
#pragma unroll 2
            for (int j = 0; j < SPL; ++j) {
                const int t = s_first + j;
                if (t < nl && cok) {
                    int iv = max(cl0 + cntb - 1, kb);
                    if (g.mirror)
                        iv = min(max(mirror_before(n0 + t, lp0, lp1, rp0, rp1) + cl0 + cntb - 1, 0), Ee - 2);
                    const int li = min(iv - ia, m - 1);
                    if (li != cur) {
                        R y0, s0;
                        if (li == cur + 1) {
                            y0 = ynx;
                            s0 = snx;
                        } else {
                            y0 = yc[base + (size_t)li * C];
                            s0 = sc[base + (size_t)li * C];
                        }
                        ynx = yc[base + (size_t)(li + 1) * C];
                        snx = sc[base + (size_t)(li + 1) * C];
                        cur = li;
                        x0 = kx[li];
                        const int h = kx[li + 1] - x0;
                        const R ih = rtab[h];
                        const R slope = mul_(sub_(ynx, y0), ih);
                        ca = y0;
                        cb = fmad_(-mul_(R(h), third), fmad_(R(2), s0, snx), slope);
                        c2 = s0;
                        cd = mul_(sub_(snx, s0), mul_(ih, third));
                    }
                    const float tt = (float)(n0 + t - x0);
                    const R v = fmat_(fmat_(fmat_(cd, tt, c2), tt, cb), tt, ca);
                    const int idx = t * G + cc;
                    if constexpr (STOPM) {
                        if (env == 0) {
                            us[idx] = v;
                        } else {
                            const R uu = us[idx];
                            accs[idx] = add_(accs[idx], add_(uu, v));
                            us[idx] = sub_(uu, v);
                        }
                    } else {
                        accs[idx] = add_(accs[idx], v);
                    }
                }
                cntb += (int)((wd[t >> 5] >> (t & 31)) & 1u);
            }
            if constexpr (STOPM) {
                if (env == 1) {
                    __syncwarp();
                    for (int j = 0; j < SPL; ++j) {
                        const int t = s_first + j;
                        R d2 = R(0.0f);
                        if (cok && t < nl) {
                            const R uu = us[t * G + cc];
                            d2 = mul_(uu, uu);
                        }
#pragma unroll
                        for (int o = 1; o < G; o <<= 1) d2 = add_(d2, shfl_xor_(d2, o));
                        if (cc == 0 && t < nl) part[((size_t)cg * Kc + kk) * g.L + n0 + t] = d2;
                    }
                }
            }
        }
    }
    if (overflow) atomicOr(&st->flags, 2);
    __syncthreads();
    const int Q = sQ;
    if (!M && last_chunk && Q == 0 && (blockIdx.x == 0 || ep.n > 0) && blockIdx.y == 0 && threadIdx.x == 0)
        atomicOr(&st->flags, 1);
    for (int idx = threadIdx.x; idx < T * G; idx += blockDim.x) {
        const int t = idx / G, ch = idx - t * G;
        const int cch = cg * G + ch;
        if (t >= nl || cch >= C) continue;
        const size_t off = (size_t)(n0 + t) * C + cch;
        R tot = first_chunk ? R(0.0f) : acc_buf[off];
#pragma unroll
        for (int w = 0; w < Sh::WARPS; ++w)
            tot = add_(tot, reinterpret_cast<const R*>(smem_raw + (size_t)w * PW)[idx]);
        if (last_chunk) {
            const R mval = div_(mul_(tot, R(0.5f)), R(Q));
            if (M) M[off] = mval;
            else X[off] = xsub(X[off], mval);
        } else {
            acc_buf[off] = tot;
        }
    }
}

// ---------------------------------------------------------------------------
// Mean envelope by impulse accumulation (mixed form, fixed mode).
//
// A natural cubic spline with knots x_j is, for n >= x_0,
//     S(n) = P_0(n) + sum_j dd_j (n - x_j)_+^3,   dd_j = d_j - d_{j-1}
// (the pieces agree in value, slope and curvature at every interior knot;
// only the cubic coefficient d jumps).  The fourth forward difference of
// (n - x)_+^3 is 1, 4, 1 at n = x-3, x-2, x-1 and zero elsewhere, so the sum
// over all envelopes M(n) = sum_e S_e(n) obeys
//     Delta^4 M(n) = I(n) = sum over interior knots of dd_j * {1,4,1}.
// Per span of 32 m samples (m = 1 .. 4 words, longer where the knots are
// sparse) the kernel anchors M at the middle sample n_a (value and the first
// three forward differences of the pieces active there, plus the impulses that
// knots at n_a+1, n_a+2 place before n_a), then rebuilds M(n) by running the
// difference recurrence forwards and backwards over the span.  Work per span:
// O(knots + envelopes) instead of O(envelopes x samples).
//
// The jumps q_j - q_{j-1} (q_j: d_j quantised), the anchor sums and the
// recurrence are integers in units of q = 2^(e - 62), 2^e > 2 Kc B_c, with B_c
// a bound on |S_e(n)| for channel c written by the solve (max |y| plus max
// h^2 (|s_i| + |s_{i+1}|) / 4 over the pieces), so the sums over directions
// are exact and independent of their order; each lane's anchor coefficients
// are summed in double-float in a fixed order before quantisation.  The
// double-float inputs carry ~48 bits, and the recurrence extrapolates each
// anchor over at most 16 m samples (one mean knot spacing where the knots are
// sparse enough for m > 1; 16 samples at the densest), which keeps the mean
// within ~1e-13 of its value relative to the signal (the direct evaluation:
// ~1e-15).  The conversions round to nearest: truncation's one-sided error
// accumulates over the sifts.
//
// CTA: one span (or one of the P parts of a span's directions) x G channels,
// 8 warps, four CTAs per SM (64 registers; the accumulators of a span of at
// most 128 samples take 33.5 KB); lane = (subgroup, channel), the (direction,
// envelope) pairs are dealt round-robin to the 8 * 32/G subgroups, which add
// each knot's jump into a per-row array in shared memory (one 64-bit integer
// atomic per knot).  The recurrence runs as four block-wide exact prefix sums
// plus the cubic that matches the anchor state, so all warps share it.
// ---------------------------------------------------------------------------
// The double-float v times 2^sh as a 64-bit two's-complement integer (|v 2^sh|
// < 2^62), rounded to nearest (ties up) from the 48-bit combined mantissa, by
// integer instructions only: the float-to-int64 conversion instructions run on
// the FP64 pipe, 1/64 of the FP32 rate on this GPU.  Rounding to nearest keeps
// the conversions unbiased: a truncation's one-sided error accumulates over
// the sifts of a decomposition.
__device__ __forceinline__ unsigned long long qfix(dd v, int sh)
{
    const unsigned uh = __float_as_uint(v.hi), ul = __float_as_uint(v.lo);
    const int eh = (int)((uh >> 23) & 0xffu), el = (int)((ul >> 23) & 0xffu);
    if (eh == 0) return 0ull;  // zero (or subnormal): below any quantum in use
    int mh = (int)((uh & 0x7fffffu) | 0x800000u);
    int ml = (el == 0) ? 0 : (int)((ul & 0x7fffffu) | 0x800000u);
    if (uh >> 31) mh = -mh;
    if (ul >> 31) ml = -ml;
    // lo in units of 2^(eh - 174): ml 2^(el - eh + 24); |lo| <= ulp(hi) gives el <= eh - 23
    const int dl = eh - el - 24;
    const int mlo = (dl < 0) ? ml * 2 : (dl == 0 ? ml : (dl < 31 ? ((ml + (1 << (dl - 1))) >> dl) : 0));
    const long long comb = (long long)mh * (1ll << 24) + (long long)mlo;  // |comb| < 2^48
    const int s = eh - 174 + sh;                                           // value 2^sh = comb 2^s
    long long r;
    if (s >= 0) r = (long long)((unsigned long long)comb << min(s, 63));
    else if (s > -63) r = (comb + (1ll << (-s - 1))) >> (-s);
    else r = 0;
    return (unsigned long long)r;
}

// the non-negative integer a (< 2^63) times 2^-sh as a float, truncated to
// 24 bits; *rest receives the bits below them
__device__ __forceinline__ float fix2f(unsigned long long a, int sh, unsigned long long* rest)
{
    if (a == 0ull) {
        *rest = 0ull;
        return 0.0f;
    }
    const int msb = 63 - __clzll((long long)a);
    const int sd = msb - 23;
    const unsigned long long top = (sd >= 0) ? (a >> sd) : (a << -sd);
    *rest = (sd > 0) ? a - (top << sd) : 0ull;
    const int be = msb - sh + 127;  // biased exponent of the result
    if (be <= 0) return 0.0f;
    return __uint_as_float(((unsigned)be << 23) | ((unsigned)top & 0x7fffffu));
}
// the non-negative integer a (< 2^40) times 2^-sh as a float, rounded to nearest
__device__ __forceinline__ float fix2f_rn(unsigned long long a, int sh)
{
    if (a == 0ull) return 0.0f;
    int msb = 63 - __clzll((long long)a);
    int sd = msb - 23;
    unsigned long long top = (sd > 0) ? ((a + (1ull << (sd - 1))) >> sd) : (a << -sd);
    if (top >> 24) {  // the rounding carried into a new leading bit
        top >>= 1;
        ++msb;
    }
    const int be = msb - sh + 127;
    if (be <= 0) return 0.0f;
    return __uint_as_float(((unsigned)be << 23) | ((unsigned)top & 0x7fffffu));
}
// the two's-complement integer v times 2^-sh as a double-float: the high word
// truncated to 24 bits, the rest rounded to nearest (~48 bits, unbiased)
__device__ __forceinline__ dd fix2dd(unsigned long long v, int sh)
{
    const bool neg = (long long)v < 0;
    const unsigned long long a = neg ? 0ull - v : v;
    unsigned long long r1;
    const float hi = fix2f(a, sh, &r1);
    const float lo = fix2f_rn(r1, sh);
    return neg ? dd(-hi, -lo) : dd(hi, lo);
}

constexpr int kCumMaxParts = 4;  // most CTAs sharing one span

// Global accumulators of the spans split over several CTAs (zero between
// launches: the CTA that finishes a span clears them).
struct CumShared {
    unsigned long long* kq;   // [W][35][C]: span si uses rows si*(32m+3) .. (si+1)*(32m+3)-1
    unsigned long long* anc;  // [W][4][C]
    int* arrive;              // [groups][W]
};

template <int G>
__global__ void __launch_bounds__(256, 4)
k_mean_cum(const float2* __restrict__ X, float2* __restrict__ Xout, dd* __restrict__ acc_buf,
           const uint32_t* __restrict__ bits,
           const int* __restrict__ wpref, const int* __restrict__ knots, const int* __restrict__ cnt,
           const dd* __restrict__ rtab, const dd* __restrict__ rtab3, const dd* __restrict__ sv,
           const dd* __restrict__ yend, const unsigned* __restrict__ bnd, unsigned* __restrict__ bnd_clear,
           const int* __restrict__ cumcfg, CumShared sh_g, Geom g, int k0, int Kc, int first_chunk, int last_chunk,
           RunState* st, Epochs ep)
{
    constexpr int SUB = 32 / G;
    constexpr int NWS = 8 * SUB;
    constexpr int NE = 256;  // (direction, envelope) pairs described per round
    constexpr int KB = 4;    // knots per batch of loads
    extern __shared__ __align__(16) unsigned long long kq[];  // [32 * kCumMaxWords + 3][G]: jump of d at row x - p0
    // The pairs' descriptions are dead once the pairs are done; the anchor
    // sums and the scan state live only after that, so the two share one
    // buffer (less shared memory per CTA leaves more of the SM's L1)
    union Shared {
        struct {
            int I[NE], J[NE], N[NE], X[NE], H[NE];
        } e;
        struct {
            unsigned long long anc[4 * G];
            unsigned long long part[NWS * G];  // per row group: totals of a scan pass
            unsigned long long pst[6 * G];     // particular solution at n_a; look-ahead jumps
        } f;
    };
    __shared__ __align__(16) Shared su;
    int *eI = su.e.I, *eJ = su.e.J, *eN = su.e.N, *eX = su.e.X, *eH = su.e.H;
    unsigned long long *anc = su.f.anc, *part = su.f.part, *pst = su.f.pst;
    __shared__ int sQ, sLast;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cc = lane % G, sub = lane / G;
    const int C = g.C;
    const int mw = min(max(cumcfg[0], 1), kCumMaxWords), P = min(max(cumcfg[1], 1), kCumMaxParts);
    // CTA b works on part b % P of span b / P (launched: W rounded up to a
    // multiple of 4 CTAs, so that every part of every span exists; P | m | 4)
    const int si = blockIdx.x / P, prt = blockIdx.x % P;
    const int w = si * mw;
    if (bnd_clear && blockIdx.x == 0 && blockIdx.y == 0)
        for (int i = threadIdx.x; i < 2 * C; i += blockDim.x) bnd_clear[i] = 0u;
    if (w >= g.W) return;  // uniform over the CTA
    // the record (epoch) of the span; spans never straddle two (epochs start at
    // multiples of kEpochAlign = 512 samples, spans are at most 128 long)
    const int rec = ep.n > 0 ? ep.wep[w] : 0;
    const int rend = ep.n > 0 ? ep.off[rec] + ep.len[rec] : g.L;  // one past the record's last sample
    const int p0 = w * 32;
    if (p0 >= rend) return;  // gap between epochs
    const int nl = min(32 * mw, rend - p0);
    const int ra = min(16 * mw, nl - 1);
    const int na = p0 + ra;
    const int c = blockIdx.y * G + cc;
    const bool cok = c < C;
    const int cl = min(c, C - 1);  // loads of lanes past the last channel stay in bounds
    for (int i = threadIdx.x; i < (nl + 3) * G; i += blockDim.x) kq[i] = 0ull;
    // quantum: |sum over the chunk's envelopes| <= 2 Kc B < 2^ex
    const float B = __uint_as_float(bnd[cl]) + __uint_as_float(bnd[C + cl]);
    const bool bad = !(B < INFINITY);
    int ex = 0;
    frexpf(__fmul_rn(B, (float)(2 * Kc)) * 1.0009765625f, &ex);
    ex = max(ex, -60);
    const int sh = 62 - ex;  // value = units * 2^-sh
    const dd third = dd(1.0 / 3.0);
    const int wa = w + (ra >> 5), ba = ra & 31;
    const int wend = min(w + mw, g.W);
    // this CTA's share of the (direction, envelope) pairs
    const int e_lo = prt * 2 * Kc / P, e_hi = (prt + 1) * 2 * Kc / P;  // 2 Kc <= 2048, P <= 4

    dd aA(0.0f, 0.0f), aB(0.0f, 0.0f), aC(0.0f, 0.0f), aD(0.0f, 0.0f);  // anchor coefficients, summed in a fixed order
    for (int base = e_lo; base < e_hi; base += NE) {
        __syncthreads();
        // (1) per (direction, envelope): anchor piece i (x_i <= n_a < x_{i+1}),
        //     first interior knot j past p0 and the number n of interior knots
        //     in (p0, p0 + nl + 2]; n = -1 marks a direction that does not count
        {
            const int ei = base + (int)threadIdx.x;
            int n = -1, i = 0, j = 0, xi = 0, hh = 1;
            if (ei < e_hi) {
                const int kk = ei >> 1, env = ei & 1, k = k0 + kk;
                const int Ex = cnt[k], En = cnt[g.K + k];
                if (Ex <= g.cap && En <= g.cap && dir_qualifies(g, ep, cnt, k, rec)) {
                    const size_t slot = (size_t)env * Kc + kk;
                    const uint32_t* bb = bits + slot * g.W;
                    const int* wp = wpref + slot * (g.W + 1);
                    // the record's knots: kb .. ke - 1 (first and last at its end samples)
                    const int kb = ep.n > 0 ? wp[ep.w0[rec]] : 0;
                    const int ke = ep.n > 0 ? wp[ep.w0[rec + 1]] : (env ? En : Ex);
                    const uint32_t bw = bb[w];
                    const uint32_t bwa = bb[wa];
                    const uint32_t le = (ba == 31) ? bwa : (bwa & ((2u << ba) - 1u));
                    i = min(wp[wa] + __popc(le) - 1, ke - 2);
                    j = max(kb + 1, wp[w] + (int)(bw & 1u));
                    int nw = wp[wend] - wp[w] - (int)(bw & 1u);  // knots in (p0, p0 + 32 m)
                    if (wend < g.W && nl == 32 * mw) nw += __popc(bb[wend] & 7u);
                    n = max(0, min(j + nw - 1, ke - 2) - j + 1);
                    const int* kn = knots + slot * g.cap;
                    xi = kn[i];
                    hh = kn[i + 1] - xi;
                }
            }
            if (threadIdx.x < NE) {
                eI[threadIdx.x] = i;
                eJ[threadIdx.x] = j;
                eN[threadIdx.x] = n;
                eX[threadIdx.x] = xi;
                eH[threadIdx.x] = hh;
            }
        }
        __syncthreads();
        const int nround = min(NE, e_hi - base);
        for (int le = warp * SUB + sub; le < nround; le += NWS) {
            const int n = eN[le];
            if (n < 0) continue;
            const int ei = base + le;
            const int kk = ei >> 1, env = ei & 1;
            const size_t slot = (size_t)env * Kc + kk;
            const int* kn = knots + slot * g.cap;
            const size_t rb = slot * (size_t)g.cap * C + cl;
            // (2) anchor: Taylor coefficients of the piece at n_a
            {
                const int i = eI[le];
                const int xi = eX[le], h = eH[le];
                // knot values: X at interior knots, the record's clamped end knots from yend
                const dd* ye = yend + (slot * (ep.n > 0 ? ep.n : 1) + rec) * 2 * (size_t)C + cl;
                const int rbeg = ep.n > 0 ? ep.off[rec] : 0;
                const dd y0 = (xi == rbeg) ? ye[0] : xval<dd>(X[(size_t)xi * C + cl]);
                const dd y1 = (xi + h == rend - 1) ? ye[C] : xval<dd>(X[(size_t)(xi + h) * C + cl]);
                const dd s0 = sv[rb + (size_t)i * C], s1 = sv[rb + (size_t)(i + 1) * C];
                const dd d = (s1 - s0) * rtab3[h];
                const dd s02(2.0f * s0.hi, 2.0f * s0.lo);  // exact
                const dd b = (y1 - y0) * rtab[h] - dd_mulf(s02 + s1, (float)h) * third;
                const float u = (float)(na - xi);
                const dd d3 = dd_mulf(d, 3.0f);
                aA = aA + (dd_mulf(dd_mulf(dd_mulf(d, u) + s0, u) + b, u) + y0);
                aB = aB + (dd_mulf(dd_mulf(d3, u) + s02, u) + b);
                aC = aC + (dd_mulf(d3, u) + s0);
                aD = aD + d;
            }
            // (3) jumps q_j - q_{j-1} at row x_j - p0 (in 1 .. nl + 2), q_j the
            //     quantised d_j = (s_{j+1} - s_j) / (3 h_j); full batches of KB
            //     knots (loads first, no predication), then the remainder
            const int j0 = eJ[le];
            if (n > 0) {
                int xj = kn[j0];
                dd sj = sv[rb + (size_t)j0 * C];
                unsigned long long qprev = qfix((sj - sv[rb + (size_t)(j0 - 1) * C]) * rtab3[xj - kn[j0 - 1]], sh);
                int t0 = 0;
                for (; t0 + KB <= n; t0 += KB) {
                    int xn[KB];
                    dd sn[KB], r3[KB];
                    const int* knp = kn + j0 + t0 + 1;
                    const dd* svp = sv + rb + (size_t)(j0 + t0 + 1) * C;
#pragma unroll
                    for (int k = 0; k < KB; ++k) {
                        xn[k] = knp[k];
                        sn[k] = svp[(size_t)k * C];
                    }
                    {
                        int xa = xj;
#pragma unroll
                        for (int k = 0; k < KB; ++k) {
                            r3[k] = rtab3[xn[k] - xa];
                            xa = xn[k];
                        }
                    }
#pragma unroll
                    for (int k = 0; k < KB; ++k) {
                        const unsigned long long qcur = qfix((sn[k] - sj) * r3[k], sh);
                        if (MEMD_CHECK(xj - p0 >= 0 && xj - p0 < nl + 3)) atomicAdd(&kq[(xj - p0) * G + cc], qcur - qprev);
                        qprev = qcur;
                        xj = xn[k];
                        sj = sn[k];
                    }
                }
                for (; t0 < n; ++t0) {
                    const int xn1 = kn[j0 + t0 + 1];
                    const dd sn1 = sv[rb + (size_t)(j0 + t0 + 1) * C];
                    const unsigned long long qcur = qfix((sn1 - sj) * rtab3[xn1 - xj], sh);
                    if (MEMD_CHECK(xj - p0 >= 0 && xj - p0 < nl + 3)) atomicAdd(&kq[(xj - p0) * G + cc], qcur - qprev);
                    qprev = qcur;
                    xj = xn1;
                    sj = sn1;
                }
            }
        }
    }
    __syncthreads();  // the descriptions are dead: anc takes their place
    for (int i = threadIdx.x; i < 4 * G; i += blockDim.x) anc[i] = 0ull;
    __syncthreads();
    atomicAdd(&anc[0 * G + cc], qfix(aA, sh));
    atomicAdd(&anc[1 * G + cc], qfix(aB, sh));
    atomicAdd(&anc[2 * G + cc], qfix(aC, sh));
    atomicAdd(&anc[3 * G + cc], qfix(aD, sh));
    __syncthreads();
    if (P > 1) {
        // a span shared by P CTAs: add this CTA's rows to the span's global
        // accumulators; the last CTA to arrive finishes the span and clears them
        const int rows = 32 * mw + 3;
        unsigned long long* gk = sh_g.kq + (size_t)si * rows * C + (size_t)blockIdx.y * G;
        unsigned long long* ga = sh_g.anc + (size_t)si * 4 * C + (size_t)blockIdx.y * G;
        for (int i = threadIdx.x; i < (nl + 3) * G; i += blockDim.x) {
            const int r = i / G, ch = i - r * G;
            const unsigned long long v = kq[i];
            if (v != 0ull && blockIdx.y * G + ch < C) atomicAdd(&gk[(size_t)r * C + ch], v);
        }
        for (int i = threadIdx.x; i < 4 * G; i += blockDim.x) {
            const int r = i / G, ch = i - r * G;
            if (blockIdx.y * G + ch < C) atomicAdd(&ga[(size_t)r * C + ch], anc[i]);
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) sLast = (atomicAdd(&sh_g.arrive[(size_t)blockIdx.y * g.W + si], 1) == P - 1);
        __syncthreads();
        if (!sLast) return;  // uniform over the CTA
        __threadfence();
        for (int i = threadIdx.x; i < (nl + 3) * G; i += blockDim.x) {
            const int r = i / G, ch = i - r * G;
            unsigned long long v = 0ull;
            if (blockIdx.y * G + ch < C) {
                v = __ldcg(&gk[(size_t)r * C + ch]);
                gk[(size_t)r * C + ch] = 0ull;
            }
            kq[i] = v;
        }
        for (int i = threadIdx.x; i < 4 * G; i += blockDim.x) {
            const int r = i / G, ch = i - r * G;
            unsigned long long v = 0ull;
            if (blockIdx.y * G + ch < C) {
                v = __ldcg(&ga[(size_t)r * C + ch]);
                ga[(size_t)r * C + ch] = 0ull;
            }
            anc[i] = v;
        }
        if (threadIdx.x == 0) sh_g.arrive[(size_t)blockIdx.y * g.W + si] = 0;
    }
    if (warp == 0) {
        int q = 0;
        for (int k = lane; k < g.K; k += 32) q += dir_qualifies(g, ep, cnt, k, rec) ? 1 : 0;
        q = warp_sum(q);
        if (lane == 0) sQ = q;
    }
    // (4) M over the span, in parallel: row group rg = warp * SUB + sub owns
    //     rows [r0, r1).  The particular solution P (zero state at row 0) is
    //     four exclusive prefix sums of the impulses I(r) = kq[r+1] + 4 kq[r+2]
    //     + kq[r+3]; M = P + H with H the cubic (Delta^4 H = 0) whose
    //     differences at n_a are the anchor state minus P's.
    const int rg = warp * SUB + sub;
    const int RB = (nl + NWS - 1) / NWS;
    const int r0 = min(nl, rg * RB), r1 = min(nl, r0 + RB);
    unsigned long long e0 = 0, e1 = 0, e2 = 0;  // rows r1 .. r1 + 2, read before they are overwritten
    __syncthreads();
    if (r0 < r1) {
        e0 = kq[r1 * G + cc];
        e1 = kq[(r1 + 1) * G + cc];
        e2 = kq[(r1 + 2) * G + cc];
    }
    if (rg == 0) {
        pst[3 * G + cc] = kq[(ra + 1) * G + cc];  // jump at n_a + 1
        pst[4 * G + cc] = kq[(ra + 2) * G + cc];  // jump at n_a + 2
    }
    __syncthreads();
    const int Q = sQ;
    if (last_chunk && Q == 0 && blockIdx.y == 0 && threadIdx.x == 0) atomicOr(&st->flags, 1);
    for (int r = r0; r < r1; ++r) {  // in place: I(r) reads rows > r only
        const unsigned long long a1 = (r + 1 < r1) ? kq[(r + 1) * G + cc] : (r + 1 == r1 ? e0 : (r + 1 == r1 + 1 ? e1 : e2));
        const unsigned long long a2 = (r + 2 < r1) ? kq[(r + 2) * G + cc] : (r + 2 == r1 ? e0 : (r + 2 == r1 + 1 ? e1 : e2));
        const unsigned long long a3 = (r + 3 < r1) ? kq[(r + 3) * G + cc] : (r + 3 == r1 ? e0 : (r + 3 == r1 + 1 ? e1 : e2));
        kq[r * G + cc] = a1 + (a2 << 2) + a3;
    }
    for (int pass = 0; pass < 4; ++pass) {
        unsigned long long run = 0;
        for (int r = r0; r < r1; ++r) {
            const unsigned long long t = kq[r * G + cc];
            kq[r * G + cc] = run;
            run += t;
        }
        part[rg * G + cc] = run;
        __syncthreads();
        unsigned long long off = 0;
        for (int q = 0; q < rg; ++q) off += part[q * G + cc];
        for (int r = r0; r < r1; ++r) kq[r * G + cc] += off;
        if (pass < 3 && ra >= r0 && ra < r1) pst[pass * G + cc] = kq[ra * G + cc];  // P's d3, d2, d1 at n_a
        __syncthreads();
    }
    if (!cok || r0 >= r1) return;
    const unsigned long long sA = anc[cc], sB = anc[G + cc], sC = anc[2 * G + cc], sD = anc[3 * G + cc];
    const unsigned long long k1 = pst[3 * G + cc], k2 = pst[4 * G + cc];
    // state at n_a: differences of the anchor polynomials plus the part of the
    // jumps at n_a + 1 and n_a + 2 that falls before n_a (Delta^4 of (n - x)_+^3
    // is 1, 4, 1 at x - 3, x - 2, x - 1), minus P's state there
    const unsigned long long h0 = sA - kq[ra * G + cc];
    const unsigned long long h1 = sB + sC + sD - pst[2 * G + cc];
    const unsigned long long h2 = 2ull * sC + 6ull * sD + k1 - pst[1 * G + cc];
    const unsigned long long h3 = 6ull * sD + 5ull * k1 + k2 - pst[cc];
    const dd qd = dd((float)Q, 0.0f);
    constexpr int XB = 4;  // rows per batch of X loads
    for (int rb0 = r0; rb0 < r1; rb0 += XB) {
        float2 xs[XB];
        dd ac[XB];
#pragma unroll
        for (int k = 0; k < XB; ++k) {
            if (rb0 + k < r1) {
                const size_t off = (size_t)(p0 + rb0 + k) * C + c;
                if (last_chunk) xs[k] = X[off];
                if (!first_chunk) ac[k] = acc_buf[off];
            }
        }
#pragma unroll
        for (int k = 0; k < XB; ++k) {
            const int r = rb0 + k;
            if (r < r1) {
                // H(n_a + t) = h0 + t h1 + C(t,2) h2 + C(t,3) h3 (Newton's form, any integer t)
                // |t| <= 128: the binomials are exact in 32-bit integers
                const int t = r - ra;
                const unsigned long long c2 = (unsigned long long)(long long)(t * (t - 1) / 2);
                const unsigned long long c3 = (unsigned long long)(long long)(t * (t - 1) * (t - 2) / 6);
                const unsigned long long val =
                    kq[r * G + cc] + h0 + (unsigned long long)(long long)t * h1 + c2 * h2 + c3 * h3;
                dd tot = fix2dd(val, sh);
                if (bad) tot = dd(__int_as_float(0x7fc00000), 0.0f);
                const size_t off = (size_t)(p0 + r) * C + c;
                if (!first_chunk) tot = tot + ac[k];
                if (last_chunk) Xout[off] = xsub(xs[k], dd_mulf(tot, 0.5f) / qd);
                else acc_buf[off] = tot;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Projection + extrema for the mixed path: P = dir . X in FP32 from the high
// words of the double-float signal, with a rigorous bound on its error
//   |P32 - P| <= (C+2) 2^-24 sum_c |dh_c| max|xh_c| + sum_c |dl_c| max|X_c|
// (dh, dl: high/low words of the direction).  A comparison whose FP32 margin
// is within twice the bound is decided again on double-float projections
// (two-product fma splitting, ~2^-44 relative), so the extrema sets are those
// of the FP64 projection except at ties closer than that.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 df_dot(const float2* __restrict__ x, const float* __restrict__ dh,
                                         const float* __restrict__ dl, int C)
{
    float hi = 0.f, lo = 0.f;
    for (int c = 0; c < C; ++c) {
        const float2 xv = x[c];
        const float a = dh[c], al = dl[c];
        const float p = __fmul_rn(a, xv.x);
        float e = __fmaf_rn(a, xv.x, -p);
        e = __fmaf_rn(a, xv.y, __fmaf_rn(al, xv.x, e));
        const float s = __fadd_rn(hi, p);
        const float bb = __fsub_rn(s, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
        lo = __fadd_rn(lo, __fadd_rn(err, e));
        hi = s;
    }
    const float sh = __fadd_rn(hi, lo);
    return make_float2(sh, __fsub_rn(lo, __fsub_rn(sh, hi)));
}

__device__ __forceinline__ bool df_gt(float2 a, float2 b) { return a.x > b.x || (a.x == b.x && a.y > b.y); }

__global__ void __launch_bounds__(256)
k_project_mx(const float2* __restrict__ X, const float* __restrict__ dh_all, const float* __restrict__ dl_all,
             uint32_t* __restrict__ bits, Geom g, int k0, int Kc, RunState* st, Epochs ep)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int C = g.C;
    const int ldx = C + 1;
    float* xs = reinterpret_cast<float*>(smem_raw);        // (TN + 2) x ldx
    float* ds = xs + (kProjTN + 2) * ldx;                  // TK x C (high words)
    float* ps = ds + kProjTK * C;                          // TK x (TN + 2)
    float* mx = ps + kProjTK * (kProjTN + 2);              // C: max |x| over the tile
    float* bnd = mx + C;                                   // TK
    float* dls = bnd + kProjTK;                            // TK x C (low words)
    const int n0 = blockIdx.x * kProjTN;
    const int kt0 = blockIdx.y * kProjTK;
    // tile loads: rows by warp, channels by lane (no division by C)
    for (int r = threadIdx.x >> 5; r < kProjTN + 2; r += blockDim.x >> 5) {
        const int n = n0 - 1 + r;
        for (int c = threadIdx.x & 31; c < C; c += 32)
            xs[r * ldx + c] = (n >= 0 && n < g.L) ? X[(size_t)n * C + c].x : 0.f;
    }
    for (int kk = threadIdx.x >> 5; kk < kProjTK; kk += blockDim.x >> 5) {
        const int k = kt0 + kk;
        for (int c = threadIdx.x & 31; c < C; c += 32) {
            ds[kk * C + c] = (k < Kc) ? dh_all[(size_t)(k0 + k) * C + c] : 0.f;
            dls[kk * C + c] = (k < Kc) ? dl_all[(size_t)(k0 + k) * C + c] : 0.f;
        }
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // max |x| per channel over the tile: warp w takes rows w, w + 8, ...
    for (int c0 = 0; c0 < C; c0 += 32) {
        const int c = c0 + lane;
        float m = 0.f;
        if (c < C)
            for (int r = warp; r < kProjTN + 2; r += 8) m = fmaxf(m, fabsf(xs[r * ldx + c]));
        ps[warp * 32 + lane] = m;  // ps is free until the projections
        __syncthreads();
        if (warp == 0 && c < C) {
            float t = ps[lane];
#pragma unroll
            for (int w8 = 1; w8 < 8; ++w8) t = fmaxf(t, ps[w8 * 32 + lane]);
            mx[c] = t;
        }
        __syncthreads();
    }
    // error bound of each projection (warp w: directions 2w, 2w + 1; lanes
    // over channels), with margin for the bound's own rounding
    for (int j = 0; j < 2; ++j) {
        const int kk = warp * 2 + j;
        float bh = 0.f, bl = 0.f;
        if (kt0 + kk < Kc)
            for (int c = lane; c < C; c += 32) {
                bh = __fmaf_ru(fabsf(ds[kk * C + c]), mx[c], bh);
                bl = __fmaf_ru(fabsf(dls[kk * C + c]), mx[c], bl);
            }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            bh = __fadd_ru(bh, __shfl_xor_sync(kFull, bh, o));
            bl = __fadd_ru(bl, __shfl_xor_sync(kFull, bl, o));
        }
        if (lane == 0) bnd[kk] = 1.01f * ((float)(C + 2) * 5.9604645e-8f * bh + 1.0000002f * bl);
    }
    const int sg = warp & 1, dg = warp >> 1;
    {
        const int r = 1 + sg * 32 + lane;
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        const float* xr = xs + r * ldx;
        const float* d0 = ds + (dg * 4) * C;
        for (int c = 0; c < C; ++c) {
            const float xv = xr[c];
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[j] = __fmaf_rn(xv, d0[j * C + c], acc[j]);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) ps[(dg * 4 + j) * (kProjTN + 2) + r] = acc[j];
    }
    if (warp == 0) {
        const int side = lane >> 4, kk = lane & 15;
        const int r = side ? kProjTN + 1 : 0;
        float acc = 0.f;
        const float* xr = xs + r * ldx;
        const float* dd = ds + kk * C;
        for (int c = 0; c < C; ++c) acc = __fmaf_rn(xr[c], dd[c], acc);
        ps[kk * (kProjTN + 2) + r] = acc;
    }
    __syncthreads();
    const int n = n0 + sg * 32 + lane;
    const int r = 1 + sg * 32 + lane;
    bool inrange, endpt, interior;
    sample_rule(g, ep, n, inrange, endpt, interior);
    const int w = (n0 >> 5) + sg;
    int refined = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int kk = dg * 4 + j;
        const float* pr = ps + kk * (kProjTN + 2);
        const float p = pr[r], pl = pr[r - 1], pn = pr[r + 1];
        bool mxf = p > pl && p > pn;
        bool mnf = p < pl && p < pn;
        const float thr = 2.f * bnd[kk];
        if (interior && kt0 + kk < Kc && (fabsf(__fsub_rn(p, pl)) <= thr || fabsf(__fsub_rn(p, pn)) <= thr)) {
            const float* dh = dh_all + (size_t)(k0 + kt0 + kk) * C;
            const float* dl = dl_all + (size_t)(k0 + kt0 + kk) * C;
            const float2 a = df_dot(X + (size_t)(n - 1) * C, dh, dl, C);
            const float2 bq = df_dot(X + (size_t)n * C, dh, dl, C);
            const float2 cq = df_dot(X + (size_t)(n + 1) * C, dh, dl, C);
            mxf = df_gt(bq, a) && df_gt(bq, cq);
            mnf = df_gt(a, bq) && df_gt(cq, bq);
            ++refined;
        }
        const bool mxb = inrange && (endpt || (interior && mxf));
        const bool mnb = inrange && (endpt || (interior && mnf));
        const uint32_t wmax = __ballot_sync(kFull, mxb);
        const uint32_t wmin = __ballot_sync(kFull, mnb);
        if (lane == 0 && kt0 + kk < Kc && w < g.W) {
            bits[(size_t)(kt0 + kk) * g.W + w] = wmax;
            bits[(size_t)(Kc + kt0 + kk) * g.W + w] = wmin;
        }
    }
    refined = warp_sum(refined);
    if (lane == 0 && refined) atomicAdd(&st->pad[3], refined);
}

// ---------------------------------------------------------------------------
// Stop mode (the sifting criterion of Rilling et al. 2003 used by Rehman &
// Mandic 2010; no counterpart in the reference, which runs max_iter sifts).
// ---------------------------------------------------------------------------
// amp[n] (+)= sum over qualified directions of the chunk of
//             sqrt(sum over channel groups of part[g][kk][n]) / 2
// ---------------------------------------------------------------------------
// Mirrored end knots (boundary mode MEMD_BOUNDARY_MIRROR; no reference
// counterpart: the mirror extension of Rilling, Flandrin & Goncalves 2003,
// two extrema per end).  One warp per direction: the first and last three
// interior maxima and minima from the bitmasks, the projection at the end
// samples and at the outermost extrema (summed like the projection kernel:
// fma over the channels in order; double-float for the mixed form), then the
// rule below, written to mir[k].
// Left end, leading maximum: if P(0) lies above the first minimum the knots
// mirror about the first maximum (maxima 2..3, minima 1..2), otherwise about
// sample 0, which joins the minima (maxima 1..2; minimum 1 and sample 0).  A
// leading minimum is the same with the roles exchanged.  If the outermost
// mirrored knot of either list stays inside the record, the symmetry point
// moves to sample 0 and the list of the symmetry extremum's kind becomes its
// first two extrema.  The right end is the mirror image.  Directions with
// fewer than two interior maxima or minima (which never enter the mean) get
// no mirrored knots.
// ---------------------------------------------------------------------------
// the first `want` (<= 3) set bits of b[0..W) in ascending order; warp-wide
__device__ __forceinline__ int warp_first_bits(const uint32_t* __restrict__ b, int W, int want, int* out)
{
    const int lane = threadIdx.x & 31;
    int found = 0;
    for (int w0 = 0; w0 < W && found < want; w0 += 32) {
        const int w = w0 + lane;
        const uint32_t v = (w < W) ? b[w] : 0u;
        const int c = __popc(v);
        int inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, inc, o);
            if (lane >= o) inc += t;
        }
        const int tot = __shfl_sync(kFull, inc, 31);
        const int exc = inc - c;
        const int take = min(want - found, tot);
        for (int r = 0; r < take; ++r) {
            const unsigned m = __ballot_sync(kFull, exc <= r && r < inc);
            const int sl = __ffs((int)m) - 1;
            int pos = 0;
            if (lane == sl) {
                uint32_t x = v;
                for (int j = exc; j < r; ++j) x &= x - 1u;
                pos = w * 32 + __ffs((int)x) - 1;
            }
            out[found + r] = __shfl_sync(kFull, pos, sl);
        }
        found += take;
    }
    return found;
}
// the last `want` (<= 3) set bits of b[0..W) in descending order; warp-wide
__device__ __forceinline__ int warp_last_bits(const uint32_t* __restrict__ b, int W, int want, int* out)
{
    const int lane = threadIdx.x & 31;
    int found = 0;
    for (int w0 = W - 1; w0 >= 0 && found < want; w0 -= 32) {
        const int w = w0 - lane;
        const uint32_t v = (w >= 0) ? b[w] : 0u;
        const int c = __popc(v);
        int inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, inc, o);
            if (lane >= o) inc += t;
        }
        const int tot = __shfl_sync(kFull, inc, 31);
        const int exc = inc - c;
        const int take = min(want - found, tot);
        for (int r = 0; r < take; ++r) {
            const unsigned m = __ballot_sync(kFull, exc <= r && r < inc);
            const int sl = __ffs((int)m) - 1;
            int pos = 0;
            if (lane == sl) {
                uint32_t x = v;
                for (int j = exc; j < r; ++j) x ^= 1u << (31 - __clz((int)x));
                pos = w * 32 + 31 - __clz((int)x);
            }
            out[found + r] = __shfl_sync(kFull, pos, sl);
        }
        found += take;
    }
    return found;
}

// projection of sample n on direction row d (summed like the projection kernels)
template <typename real, typename XT>
__device__ __forceinline__ real proj_at(const XT* __restrict__ X, const real* __restrict__ d, int n, int C)
{
    real acc = real(0);
    for (int c = 0; c < C; ++c) acc = fmad_(xval<real>(X[(size_t)n * C + c]), d[c], acc);
    return acc;
}
__device__ __forceinline__ bool mgt(double a, double b) { return a > b; }
__device__ __forceinline__ bool mgt(float a, float b) { return a > b; }
__device__ __forceinline__ bool mgt(float2 a, float2 b) { return df_gt(a, b); }

// MX: mixed form (double-float signal, float direction words dh / dl)
template <typename PT, typename real, typename XT, bool MX>
__global__ void __launch_bounds__(128)
k_mirror(const uint32_t* __restrict__ bits, const XT* __restrict__ X, const real* __restrict__ dir,
         const float* __restrict__ dh_all, const float* __restrict__ dl_all, int* __restrict__ mir, Geom g, int k0,
         int Kc)
{
    const int kk = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (kk >= Kc) return;  // uniform over the warp
    const int lane = threadIdx.x & 31;
    const int k = k0 + kk;
    int fx[3], fn[3], lx[3], ln[3];  // first (ascending) / last (descending) maxima and minima
    const int nfx = warp_first_bits(bits + (size_t)kk * g.W, g.W, 3, fx);
    const int nfn = warp_first_bits(bits + (size_t)(Kc + kk) * g.W, g.W, 3, fn);
    const int nlx = warp_last_bits(bits + (size_t)kk * g.W, g.W, 3, lx);
    const int nln = warp_last_bits(bits + (size_t)(Kc + kk) * g.W, g.W, 3, ln);
    int* out = mir + (size_t)k * kMirWords;
    if (nfx < 2 || nfn < 2) {
        if (lane < kMirWords) out[lane] = 0;
        return;
    }
    const int last = g.L - 1;
    // projections at 0, L-1, the first maximum / minimum, the last maximum / minimum
    const int smp = lane == 0 ? 0 : (lane == 1 ? last : (lane == 2 ? fx[0] : (lane == 3 ? fn[0] : (lane == 4 ? lx[0] : ln[0]))));
    PT pv{};
    if (lane < 6) {
        if constexpr (MX) pv = df_dot(X + (size_t)smp * g.C, dh_all + (size_t)k * g.C, dl_all + (size_t)k * g.C, g.C);
        else pv = proj_at<real, XT>(X, dir + (size_t)k * g.C, smp, g.C);
    }
    PT pr[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        if constexpr (MX) pr[j] = make_float2(__shfl_sync(kFull, pv.x, j), __shfl_sync(kFull, pv.y, j));
        else pr[j] = shfl_idx_(pv, j);
    }
    if (lane != 0) return;
    const PT P0 = pr[0], PL = pr[1], Pfx = pr[2], Pfn = pr[3], Plx = pr[4], Pln = pr[5];
    int nl[2], nr[2], ls[2][2], rs[2][2], lsym, rsym;
    // rev(a[from:to]) of the first extrema f (ascending, nf known)
    auto firstrev = [](const int* f, int nf, int from, int to, int* o) -> int {
        int c = 0;
        for (int i = min(to, nf) - 1; i >= from; --i) o[c++] = f[i];
        return c;
    };
    if (fx[0] < fn[0]) {
        if (mgt(P0, Pfn)) {
            nl[0] = firstrev(fx, nfx, 1, 3, ls[0]);
            nl[1] = firstrev(fn, nfn, 0, 2, ls[1]);
            lsym = fx[0];
        } else {
            nl[0] = firstrev(fx, nfx, 0, 2, ls[0]);
            nl[1] = firstrev(fn, nfn, 0, 1, ls[1]);
            ls[1][nl[1]++] = 0;
            lsym = 0;
        }
    } else {
        if (mgt(Pfx, P0)) {
            nl[0] = firstrev(fx, nfx, 0, 2, ls[0]);
            nl[1] = firstrev(fn, nfn, 1, 3, ls[1]);
            lsym = fn[0];
        } else {
            nl[0] = firstrev(fx, nfx, 0, 1, ls[0]);
            ls[0][nl[0]++] = 0;
            nl[1] = firstrev(fn, nfn, 0, 2, ls[1]);
            lsym = 0;
        }
    }
    if (2 * lsym - ls[0][0] > 0 || 2 * lsym - ls[1][0] > 0) {
        if (lsym == fx[0]) nl[0] = firstrev(fx, nfx, 0, 2, ls[0]);
        else nl[1] = firstrev(fn, nfn, 0, 2, ls[1]);
        lsym = 0;
    }
    // the last extrema l (descending): rev(a[n-2:n]) = l[0], l[1]; rev(a[n-3:n-1]) = l[1], l[2]
    auto last2 = [](const int* l, int nl_, int* o) -> int {
        const int c = min(2, nl_);
        for (int i = 0; i < c; ++i) o[i] = l[i];
        return c;
    };
    auto prev2 = [](const int* l, int nl_, int* o) -> int {
        const int c = min(2, nl_ - 1);
        for (int i = 0; i < c; ++i) o[i] = l[1 + i];
        return c;
    };
    if (lx[0] < ln[0]) {
        if (mgt(Plx, PL)) {
            nr[0] = last2(lx, nlx, rs[0]);
            nr[1] = prev2(ln, nln, rs[1]);
            rsym = ln[0];
        } else {
            rs[0][0] = last;
            rs[0][1] = lx[0];
            nr[0] = 2;
            nr[1] = last2(ln, nln, rs[1]);
            rsym = last;
        }
    } else {
        if (mgt(PL, Pln)) {
            nr[0] = prev2(lx, nlx, rs[0]);
            nr[1] = last2(ln, nln, rs[1]);
            rsym = lx[0];
        } else {
            nr[0] = last2(lx, nlx, rs[0]);
            rs[1][0] = last;
            rs[1][1] = ln[0];
            nr[1] = 2;
            rsym = last;
        }
    }
    if (2 * rsym - rs[0][nr[0] - 1] < last || 2 * rsym - rs[1][nr[1] - 1] < last) {
        if (rsym == lx[0]) nr[0] = last2(lx, nlx, rs[0]);
        else nr[1] = last2(ln, nln, rs[1]);
        rsym = last;
    }
    out[kMirLsym] = lsym;
    out[kMirRsym] = rsym;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        out[kMirNl + e] = nl[e];
        out[kMirNr + e] = nr[e];
        out[kMirLsrc + 2 * e] = ls[e][0];
        out[kMirLsrc + 2 * e + 1] = nl[e] > 1 ? ls[e][1] : 0;
        out[kMirRsrc + 2 * e] = rs[e][0];
        out[kMirRsrc + 2 * e + 1] = nr[e] > 1 ? rs[e][1] : 0;
    }
    out[14] = 0;
    out[15] = 0;
}

template <typename real>
__global__ void k_amp(const real* __restrict__ part, real* __restrict__ amp, const int* __restrict__ cnt,
                      Geom g, int k0, int Kc, int groups, int first_chunk, Epochs ep)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < g.L; n += gridDim.x * blockDim.x) {
        real a = first_chunk ? real(0) : amp[n];
        const int rec = ep.n > 0 ? ep.wep[n >> 5] : 0;  // qualification of the sample's record
        for (int kk = 0; kk < Kc; ++kk) {
            const int k = k0 + kk;
            if (!dir_qualifies(g, ep, cnt, k, rec)) continue;
            real s2 = real(0);
            for (int q = 0; q < groups; ++q) s2 = add_(s2, part[((size_t)q * Kc + kk) * g.L + n]);
            a = fmad_(sqrt_(s2), real(0.5), a);
        }
        amp[n] = a;
    }
}

// sigma(n) = ||m(n)||_2 / (amp(n) / Q); counts samples above sd and sd2.
template <typename real>
__global__ void __launch_bounds__(256)
k_stop_stats(const real* __restrict__ M, const real* __restrict__ amp, const int* __restrict__ cnt, Geom g,
             double sd, double sd2, RunState* st)
{
    __shared__ int sq;
    __shared__ unsigned long long s1, s2;
    if (threadIdx.x < 32) {
        int q = 0;
        for (int k = threadIdx.x; k < g.K; k += 32) q += (cnt[k] > 3 && cnt[g.K + k] > 3) ? 1 : 0;
        q = warp_sum(q);
        if (threadIdx.x == 0) {
            sq = q;
            s1 = 0;
            s2 = 0;
        }
    }
    __syncthreads();
    const int Q = sq;
    unsigned long long c1 = 0, c2 = 0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < g.L; n += gridDim.x * blockDim.x) {
        real m2 = real(0);
        for (int c = 0; c < g.C; ++c) {
            const real v = M[(size_t)n * g.C + c];
            m2 = fmad_(v, v, m2);
        }
        const real a = div_(amp[n], real(Q));
        real sig;
        if (a > real(0.0f)) sig = div_(sqrt_(m2), a);
        else sig = m2 > real(0.0f) ? real(INFINITY) : real(0.0f);
        c1 += (static_cast<double>(sig) > sd) ? 1 : 0;
        c2 += (static_cast<double>(sig) > sd2) ? 1 : 0;
    }
    c1 = warp_sum<unsigned long long>(c1);
    c2 = warp_sum<unsigned long long>(c2);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&s1, c1);
        atomicAdd(&s2, c2);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicAdd(&st->over1, s1);
        atomicAdd(&st->over2, s2);
    }
}

// After each pass: stop, or subtract the mean and sift again.  Before the
// first subtraction of an IMF, a residual whose every direction has fewer
// than 3 interior extrema ends the decomposition.  Drives the sift loop's
// conditional WHILE node.
__global__ void k_decide(RunState* st, const int* __restrict__ cnt, Geom g, double tol, int max_iter,
                         cudaGraphConditionalHandle h_sift, const int* __restrict__ mir)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int q = 0;
    bool few = true;
    for (int k = 0; k < g.K; ++k) {
        const int a = cnt[k], b = cnt[g.K + k];
        if (a > 3 && b > 3) ++q;
        // interior extrema: the knots less the two end samples (reference
        // boundary) or less the mirrored knots
        int ia = a - 2, ib = b - 2;
        if (g.mirror) {
            const int* mi = mir + (size_t)k * kMirWords;
            ia = a - mi[kMirNl] - mi[kMirNr];
            ib = b - mi[kMirNl + 1] - mi[kMirNr + 1];
        }
        if (ia + ib >= 3) few = false;
    }
    st->q = q;
    unsigned cont = 0;
    st->apply = 0;
    if (st->pass == 0 && few) {
        st->imf_done = 1;
    } else {
        const bool stop = (q == 0) || !(((double)st->over1 / (double)g.L > tol) || st->over2 > 0);
        if (!stop) {
            st->apply = 1;
            st->nbit += 1;
            cont = st->nbit < max_iter ? 1u : 0u;
        }
    }
    st->pass += 1;
    if (st->trace_row >= 0) st->trace_row += 1;
    st->over1 = 0;
    st->over2 = 0;
    st->pad[0] += 1;  // passes over the whole run
    st->pad[1] = (int)cont;
    if (h_sift) cudaGraphSetConditional(h_sift, cont);
}

template <typename real, typename XT>
__global__ void k_apply(XT* __restrict__ X, const real* __restrict__ M, const RunState* __restrict__ st, size_t n)
{
    if (!st->apply) return;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        X[i] = xsub(X[i], M[i]);
}

// Start of an IMF: sift counters reset, sift loop armed.
__global__ void k_imf_begin(RunState* st, int max_iter, int tracing, cudaGraphConditionalHandle h_sift)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    st->nbit = 0;
    st->pass = 0;
    st->imf_done = 0;
    st->apply = 0;
    st->over1 = 0;
    st->over2 = 0;
    st->trace_row = tracing ? st->n_imfs * (max_iter + 1) : -1;
    st->pad[1] = 1;
    if (h_sift) cudaGraphSetConditional(h_sift, 1u);
}

// IMF slot n_imfs = X (channel-major), run -= X; skipped when the residual
// ended the decomposition.
template <typename XT, typename TO>
__global__ void k_imf_out_dyn(const XT* __restrict__ X, TO* __restrict__ imf, XT* __restrict__ run,
                              const RunState* __restrict__ st, int C, int L)
{
    if (st->imf_done) return;
    __shared__ XT tile[32][33];
    TO* out = imf + (size_t)st->n_imfs * C * L;
    const int n_base = blockIdx.x * 32, c_base = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int n = n_base + r, c = c_base + threadIdx.x;
        if (c < C && n < L) {
            const size_t idx = (size_t)n * C + c;
            const XT v = X[idx];
            tile[r][threadIdx.x] = v;
            run[idx] = xsub(run[idx], v);
        }
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int c = c_base + r, n = n_base + threadIdx.x;
        if (c < C && n < L) out[(size_t)c * L + n] = xfrom<TO>(tile[threadIdx.x][r]);
    }
}

__global__ void k_imf_commit(RunState* st, int nimf, cudaGraphConditionalHandle h_imf)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned cont = 0;
    if (!st->imf_done) {
        const int i = st->n_imfs;
        if (i < 64) st->sifts[i] = st->nbit;
        st->n_imfs = i + 1;
        cont = (st->n_imfs < nimf - 1) ? 1u : 0u;
    }
    st->pad[2] = (int)cont;
    if (h_imf) cudaGraphSetConditional(h_imf, cont);
}

// Zero the IMF slots left unused when the decomposition ended early.
template <typename real>
__global__ void k_zero_unused(real* __restrict__ imf, const RunState* __restrict__ st, int nimf, size_t CL)
{
    const size_t begin = (size_t)st->n_imfs * CL, end = (size_t)(nimf - 1) * CL;
    for (size_t i = begin + (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < end; i += (size_t)gridDim.x * blockDim.x)
        imf[i] = real(0);
}

// ---------------------------------------------------------------------------
// Stop mode, batched runs: every record (epoch) takes its own decisions, with
// the single-record rules (k_decide, k_imf_commit) applied to its own counts,
// length and statistics; the graph's sift and IMF loops run while any record
// goes on, and a record that has stopped is neither updated nor written
// again.  Gap samples between records are never read or written.
// ---------------------------------------------------------------------------
// Per record: qualified directions and whether every direction has fewer
// than 3 interior extrema (one warp per record).
__global__ void k_rec_q(RecStop* __restrict__ rs, Geom g, Epochs ep)
{
    const int e = blockIdx.x, lane = threadIdx.x;
    if (e >= ep.n) return;
    int q = 0;
    bool few = true;
    for (int k = lane; k < g.K; k += 32) {
        const int a = ep.cnt[(size_t)k * ep.n + e], b = ep.cnt[((size_t)g.K + k) * ep.n + e];
        if (a > 3 && b > 3) ++q;
        if ((a - 2) + (b - 2) >= 3) few = false;  // interior extrema: the knots less the two end samples
    }
    q = warp_sum(q);
    few = __all_sync(kFull, few);
    if (lane == 0) {
        rs[e].q = q;
        rs[e].few = few ? 1 : 0;
    }
}

// sigma statistics per record: a warp's 32 consecutive samples are one
// bitmask word, which lies in one record.
template <typename real>
__global__ void __launch_bounds__(256)
k_stop_stats_b(const real* __restrict__ M, const real* __restrict__ amp, RecStop* __restrict__ rs, Geom g, Epochs ep,
               double sd, double sd2)
{
    const int lane = threadIdx.x & 31;
    const long stride = (long)gridDim.x * blockDim.x;
    for (long nw = (long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); nw < g.L; nw += stride) {
        const int n = (int)nw + lane;
        const int e = ep.wep[nw >> 5];  // the word's record (uniform over the warp)
        if (!rs[e].sifting) continue;
        const bool in = n < g.L && n - ep.off[e] < ep.len[e];
        bool o1 = false, o2 = false;
        if (in) {
            real m2 = real(0);
            for (int c = 0; c < g.C; ++c) {
                const real v = M[(size_t)n * g.C + c];
                m2 = fmad_(v, v, m2);
            }
            const real a = div_(amp[n], real(rs[e].q));
            real sig;
            if (a > real(0.0f)) sig = div_(sqrt_(m2), a);
            else sig = m2 > real(0.0f) ? real(INFINITY) : real(0.0f);
            o1 = static_cast<double>(sig) > sd;
            o2 = static_cast<double>(sig) > sd2;
        }
        const unsigned b1 = __ballot_sync(kFull, o1), b2 = __ballot_sync(kFull, o2);
        if (lane == 0) {
            if (b1) atomicAdd(&rs[e].over1, (unsigned long long)__popc(b1));
            if (b2) atomicAdd(&rs[e].over2, (unsigned long long)__popc(b2));
        }
    }
}

// One CTA: the stop test of every sifting record; the sift loop goes on
// while any record does.
__global__ void __launch_bounds__(1024)
k_decide_b(RunState* st, RecStop* __restrict__ rs, Epochs ep, double tol, int max_iter,
           cudaGraphConditionalHandle h_sift)
{
    int any = 0;
    for (int e = threadIdx.x; e < ep.n; e += blockDim.x) {
        RecStop& r = rs[e];
        r.apply = 0;
        if (!r.sifting) continue;
        int cont = 0;
        if (r.pass == 0 && r.few) {
            r.imf_done = 1;
        } else {
            const bool stop = (r.q == 0) || !(((double)r.over1 / (double)ep.len[e] > tol) || r.over2 > 0);
            if (!stop) {
                r.apply = 1;
                r.nbit += 1;
                cont = r.nbit < max_iter ? 1 : 0;
            }
        }
        r.pass += 1;
        r.over1 = 0;
        r.over2 = 0;
        r.sifting = cont;
        any |= cont;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0) {
        st->pad[0] += 1;
        st->pad[1] = any;
        if (h_sift) cudaGraphSetConditional(h_sift, any ? 1u : 0u);
    }
}

// X -= M on the samples of the records whose last pass is applied.
template <typename real, typename XT>
__global__ void k_apply_b(XT* __restrict__ X, const real* __restrict__ M, const RecStop* __restrict__ rs, Geom g,
                          Epochs ep)
{
    const size_t total = (size_t)g.L * g.C;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int n = (int)(i / g.C);
        const int e = ep.wep[n >> 5];
        if (rs[e].apply && n - ep.off[e] < ep.len[e]) X[i] = xsub(X[i], M[i]);
    }
}

// One CTA, before each IMF's sift loop: the records still decomposing sift.
__global__ void __launch_bounds__(1024)
k_imf_begin_b(RecStop* __restrict__ rs, Epochs ep, cudaGraphConditionalHandle h_sift)
{
    int any = 0;
    for (int e = threadIdx.x; e < ep.n; e += blockDim.x) {
        RecStop& r = rs[e];
        r.nbit = 0;
        r.pass = 0;
        r.imf_done = 0;
        r.apply = 0;
        r.over1 = 0;
        r.over2 = 0;
        r.sifting = r.fin ? 0 : 1;
        any |= r.sifting;
    }
    any = __syncthreads_or(any);
    if (threadIdx.x == 0 && h_sift) cudaGraphSetConditional(h_sift, any ? 1u : 0u);
}

// The IMF of each record that produced one, into the record's next slot;
// the running residual updated.  One CTA per (32-sample word, 32 channels).
template <typename XT, typename TO>
__global__ void k_imf_out_b(const XT* __restrict__ X, TO* __restrict__ imf, XT* __restrict__ run,
                            const RecStop* __restrict__ rs, Epochs ep, int C, int L)
{
    __shared__ XT tile[32][33];
    const int n_base = blockIdx.x * 32, c_base = blockIdx.y * 32;
    const int e = ep.wep[n_base >> 5];  // the word's record
    if (rs[e].fin || rs[e].imf_done) return;  // uniform over the CTA
    const int nend = ep.off[e] + ep.len[e];
    TO* out = imf + (size_t)rs[e].n_imfs * C * L;
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int n = n_base + r, c = c_base + threadIdx.x;
        if (c < C && n < nend) {
            const size_t idx = (size_t)n * C + c;
            const XT v = X[idx];
            tile[r][threadIdx.x] = v;
            run[idx] = xsub(run[idx], v);
        }
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int c = c_base + r, n = n_base + threadIdx.x;
        if (c < C && n < nend) out[(size_t)c * L + n] = xfrom<TO>(tile[threadIdx.x][r]);
    }
}

// One CTA, after each IMF's sift loop: count the IMFs; the IMF loop goes on
// while any record does (RunState.n_imfs: the most IMFs of any record).
__global__ void __launch_bounds__(1024)
k_imf_commit_b(RunState* st, RecStop* __restrict__ rs, Epochs ep, int nimf, cudaGraphConditionalHandle h_imf)
{
    int any = 0, most = 0;
    for (int e = threadIdx.x; e < ep.n; e += blockDim.x) {
        RecStop& r = rs[e];
        if (!r.fin) {
            if (!r.imf_done) {
                const int i = r.n_imfs;
                if (i < 64) r.sifts[i] = r.nbit;
                r.n_imfs = i + 1;
                if (r.n_imfs >= nimf - 1) r.fin = 1;
            } else {
                r.fin = 1;
            }
        }
        any |= r.fin ? 0 : 1;
        most = max(most, r.n_imfs);
    }
    any = __syncthreads_or(any);
    __shared__ int smost;
    if (threadIdx.x == 0) smost = 0;
    __syncthreads();
    atomicMax(&smost, most);
    __syncthreads();
    if (threadIdx.x == 0) {
        st->n_imfs = smost;
        st->pad[2] = any;
        if (h_imf) cudaGraphSetConditional(h_imf, any ? 1u : 0u);
    }
}

// Zero the IMF slots a record left unused.
template <typename real>
__global__ void k_zero_unused_b(real* __restrict__ imf, const RecStop* __restrict__ rs, Epochs ep, int nimf, int C,
                                int L)
{
    const size_t CL = (size_t)C * L, total = (size_t)(nimf - 1) * CL;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int s = (int)(i / CL);
        const int n = (int)(i % (size_t)L);
        const int e = ep.wep[n >> 5];
        if (s >= rs[e].n_imfs) imf[i] = real(0);
    }
}

// ---------------------------------------------------------------------------
// Layout transforms and IMF bookkeeping (REF:1174, 1178, 1328-1338).
// 32 x 32 tiles through shared memory; block (32, 8).
// ---------------------------------------------------------------------------
// run[n][c] = (real) y[c][n]
template <typename XT, typename tin>
__global__ void k_to_sample_major(const tin* __restrict__ y, XT* __restrict__ run, int C, int L)
{
    __shared__ XT tile[32][33];
    const int n_base = blockIdx.x * 32, c_base = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int c = c_base + r, n = n_base + threadIdx.x;
        if (c < C && n < L) tile[r][threadIdx.x] = xfrom<XT>(y[(size_t)c * L + n]);
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int n = n_base + r, c = c_base + threadIdx.x;
        if (c < C && n < L) run[(size_t)n * C + c] = tile[threadIdx.x][r];
    }
}

// Batched input: epoch e's record (C x len[e], channel-major, at y + yoff[e]
// elements) -> the concatenated working signal run[off[e] + t][c].  One CTA
// per (32-sample word, 32 channels); the gaps between epochs are left as they
// are (zeroed by the caller).
template <typename XT, typename tin>
__global__ void k_batched_in(const tin* __restrict__ y, const long long* __restrict__ yoff, XT* __restrict__ run,
                             int C, Epochs ep)
{
    __shared__ XT tile[32][33];
    const int w = blockIdx.x;
    const int e = ep.wep[w];
    const int Le = ep.len[e];
    const int t_base = w * 32 - ep.off[e], c_base = blockIdx.y * 32;
    if (t_base >= Le) return;  // gap; uniform over the CTA
    const tin* ye = y + yoff[e];
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int c = c_base + r, t = t_base + threadIdx.x;
        if (c < C && t < Le) tile[r][threadIdx.x] = xfrom<XT>(ye[(size_t)c * Le + t]);
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int t = t_base + r, c = c_base + threadIdx.x;
        if (c < C && t < Le) run[(size_t)(w * 32 + r) * C + c] = tile[threadIdx.x][r];
    }
}

// Batched output: staged IMFs imf[i][c][n] (concatenated record) -> epoch e's
// block out + nimf * yoff[e]: out[i][c][t] (nimf x C x len[e]).
template <typename T>
__global__ void k_batched_out(const T* __restrict__ imf, const long long* __restrict__ yoff, T* __restrict__ out,
                              int C, int L, int nimf, Epochs ep)
{
    const long long total = (long long)nimf * C * L;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int n = (int)(idx % L);
        const long long ic = idx / L;  // i * C + c
        const int e = ep.wep[n >> 5];
        const int t = n - ep.off[e], Le = ep.len[e];
        if (t >= Le) continue;
        const int c = (int)(ic % C), i = (int)(ic / C);
        out[(long long)nimf * yoff[e] + ((long long)i * C + c) * Le + t] = imf[idx];
    }
}

// out[c][n] = src[n][c]; when upd != nullptr also upd[n][c] -= src[n][c]
template <typename XT, typename tout>
__global__ void k_to_channel_major(const XT* __restrict__ src, tout* __restrict__ out,
                                   XT* __restrict__ upd, int C, int L)
{
    __shared__ XT tile[32][33];
    const int n_base = blockIdx.x * 32, c_base = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int n = n_base + r, c = c_base + threadIdx.x;
        if (c < C && n < L) {
            const size_t idx = (size_t)n * C + c;
            const XT v = src[idx];
            tile[r][threadIdx.x] = v;
            if (upd) upd[idx] = xsub(upd[idx], v);
        }
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int c = c_base + r, n = n_base + threadIdx.x;
        if (c < C && n < L) out[(size_t)c * L + n] = xfrom<tout>(tile[threadIdx.x][r]);
    }
}

__global__ void k_check_coords(const int32_t* __restrict__ x, int L, int* __restrict__ bad)
{
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < L; n += gridDim.x * blockDim.x)
        if (x[n] != n) atomicOr(bad, 1);
}

__global__ void k_fill_reciprocals(double* __restrict__ r64, float* __restrict__ r32, dd* __restrict__ rdd,
                                   dd* __restrict__ r3dd, int n)
{
    // r3dd (optional): 1/(3h) as a double-float
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < n; h += gridDim.x * blockDim.x) {
        const double r = h > 0 ? __ddiv_rn(1.0, (double)h) : 0.0;
        r64[h] = r;
        r32[h] = h > 0 ? __fdiv_rn(1.0f, (float)h) : 0.0f;
        rdd[h] = dd(r);
        if (r3dd) r3dd[h] = h > 0 ? dd(__ddiv_rn(1.0, 3.0 * (double)h)) : dd(0.0f, 0.0f);
    }
}

__global__ void k_set_sifts(RunState* st, int imf, int sifts)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        st->sifts[imf < 64 ? imf : 63] = sifts;
        st->n_imfs = imf + 1;
    }
}

}  // namespace memd
