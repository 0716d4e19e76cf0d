// memd_api.cu -- plan, workspace, CUDA-graph capture and the C ABI entry points.
//
// A plan owns every device buffer of the decomposition; a run copies the
// caller's record into the plan's sample-major working layout, launches the
// captured graph of the whole decomposition (all IMFs, all sifts, every
// kernel of every sift: reference loop memReducedEpochs_dev.cu:1176-1338) and
// copies the IMFs out.  Fixed-iteration runs have no data-dependent host
// control at all, so the graph is captured once per plan and relaunched.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "memd_internal.h"
#include "memd_kernels.cuh"
#include "memd_tc.cuh"

namespace memd {

static thread_local std::string g_err;

memd_status set_error(memd_status code, const char* msg)
{
    g_err = msg;
    return code;
}

memd_status set_cuda_error(const char* where, cudaError_t e)
{
    g_err = std::string(where) + ": " + cudaGetErrorString(e);
    return MEMD_ERR_CUDA;
}

static int next_pow2(int v)
{
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

}  // namespace memd

using memd::Fac;
using memd::Geom;
using memd::RunState;
using memd::dd;

struct memd_plan {
    memd_config cfg;
    Geom g;
    int prec;
    int real_bytes;  // spline arithmetic
    int xbytes;      // working-signal storage
    int tbytes;      // caller's element type
    int Kc, nchunks;
    int S, H, Sf, Hf, Ss;  // solve segments (long / short systems) and halo; factor segments and halo
    int GS, ngroups;
    int evalG, evalSPT, evalT;  // FP64 evaluation tile
    int ewG, ewSPL;             // FP32 / mixed evaluation tile
    int cum, cumG;              // mixed fixed mode: impulse-accumulation mean, channels per lane group
    int bpass;                  // (sift, chunk) passes enqueued so far in the decomposition being built
    size_t proj_smem;
    void* X;
    void* Xb;  // impulse-accumulation mean: the other working-signal buffer (the mean kernel reads X, writes Xb)
    void* run;
    void* dir;   // FP64/FP32: K x C; mixed: high words then low words
    void* acc;
    void* imf;
    void* yv;
    void* sv;
    void* yend;  // impulse-accumulation mean: clamped end-knot values [2][Kc][records][2][C] (no yv gather)
    void* dbuf;  // forward-eliminated right-hand sides [2][Kc][cap][C]
    void* fac;
    void* rtab;
    void* rtab3;  // impulse-accumulation mean: 1/(3h) as double-float
    unsigned* bnd;  // impulse-accumulation mean: [2 passes][2 parts][C] per-channel bounds (float bits)
    int* cumcfg;    // impulse-accumulation mean: anchor span (words) and CTAs per span, set by the factor kernel
    // batched runs (cfg.max_epochs > 0): epochs concatenated at multiples of
    // kEpochAlign samples; ep describes the current call's layout (n = 0: one record)
    int batched;
    int Lrec;                       // longest epoch (cfg.length)
    memd::Epochs ep;
    int* ep_dev;                    // off, len, cov [max_epochs] | w0 [max_epochs + 1] | wep [W capacity]
    long long* ep_yoff;             // [max_epochs] caller offsets of the current call
    std::vector<int64_t> ep_lens;   // lengths of the layout the graph was built for
    std::vector<int> ep_host;       // staging of ep_dev
    memd::CumShared cumsh;  // impulse-accumulation mean: accumulators of spans split over CTAs
    void* M;     // stop mode: mean envelope of the last pass [L][C]
    void* part;  // stop mode: per channel group, direction and sample sum of (U-L)^2
    void* amp;   // stop mode: amplitude statistic [L]
    void* recstop;  // stop mode, batched: RecStop per record [max_epochs]
    void* hz;       // in-place substitution: the first H rows of every segment [2][Kc][hsegs][H][C]
    int hsegs;      // segments per slot at most (solve_segments_max)
    int inplace;    // the backward sweep writes the solution over dbuf (dbuf == sv)
    int egroups; // evaluation channel groups
    uint32_t* bits;
    int* wpref;
    int* knots;
    int* cnt;
    int* mir;       // mirror boundary: [K][kMirWords] mirrored end knots per direction
    memd::CompactShared csh;  // chunked compaction: per-chunk counts, hash sums, arrival counters
    RunState* st;
    int* coord_bad;
    int* host_flag;
    memd_trace_entry* trace_dev;
    memd_trace_entry* trace_host;
    size_t trace_n;
    std::vector<void*> allocs;
    size_t bytes;
    cudaStream_t cap;
    cudaGraphExec_t exec;
    int64_t graph_launches;
    cudaEvent_t e0, e1;
    // mixed form, tensor-core projection: tf32 split of the signal and of the
    // directions ([rows][Cp], zero-padded channels) and their TMA descriptors
    int tc;          // k_project_tc replaces k_project_mx
    int Cp;          // channels rounded up to 32
    int tc_nt;       // directions per tile (MMA N)
    float* xbig;
    float* xsmall;
    float* dbig;
    float* dsmall;
    memd::TcMaps maps;
    // substitution work queue (persistent sweeps pull segments by ticket)
    int squeue;       // 1: queue, 0: one warp per possible segment
    memd::SolveQueue sq;
    int sms;          // multiprocessors of the device
    int cum_ctas;     // impulse-accumulation mean: working CTAs the split of spans over CTAs aims for
};

namespace memd {

// Element types of the three precision forms.
template <int P> struct Prec;
template <> struct Prec<MEMD_PREC_F64> { using X = double; using R = double; using T = double; };
template <> struct Prec<MEMD_PREC_F32> { using X = float;  using R = float;  using T = float; };
template <> struct Prec<MEMD_PREC_MIXED> { using X = float2; using R = dd; using T = float; };

static memd_status dev_alloc(memd_plan* p, void** ptr, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        cudaGetLastError();
        return set_error(MEMD_ERR_NOMEM, "plan: device allocation failed");
    }
    p->allocs.push_back(*ptr);
    p->bytes += bytes;
    return MEMD_OK;
}

// cuTensorMapEncodeTiled from the driver, without linking libcuda
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
    }
    return fn;
}

// TMA descriptor of a row-major float array [rows][cols] (cols a multiple of
// 32), copied in boxes of 32 columns (128 bytes) x box_rows rows into the
// 128-byte swizzled shared-memory layout; rows past the end read as zero.
static bool make_tile_map(CUtensorMap* m, void* base, uint64_t cols, uint64_t rows, uint32_t box_rows)
{
    auto enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * sizeof(float)};
    const cuuint32_t box[2] = {32u, box_rows};
    const cuuint32_t es[2] = {1u, 1u};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

// Directions per pass (the automatic direction chunk) that fit in 60% of the
// device's free memory: the [2][Kc][cap]-shaped knot, factor, knot-value and
// solution arrays and the bitmask words per direction, the record-sized
// buffers once.  Fewer passes re-run the projection, compaction and mean over
// the record fewer times (512 batched epochs of 32 x 1024..8192 samples, 64
// directions: three passes 1.80 s, one pass 1.31 s).
static int directions_that_fit(const memd_config& c, const Geom& g, int rb, int xbytes, int tbytes, bool cum,
                               bool inplace)
{
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess || fr == 0) {
        cudaGetLastError();
        return INT_MAX;
    }
    const double C = g.C, L = g.L, cap = g.cap, W = g.W;
    const bool stop = c.stop_mode == MEMD_STOP_CRITERION;
    // eliminated right-hand sides and solutions (one array in place, with a
    // quarter for the halo copies at most), knot values unless the mean reads
    // the signal
    const double arrays = (inplace ? 1.25 : 2.0) + (cum ? 0.0 : 1.0);
    const double per_dir = 2.0 * cap * (4.0 + 4.0 * rb + (double)rb * C * arrays) + 8.0 * (2.0 * W + 1.0) +
                           (stop ? (double)rb * std::ceil(C / 4.0) * L : 0.0);
    const double fixed = C * L * (3.0 * xbytes + (double)tbytes * (double)c.num_imfs + 2.0 * rb) + 8.0 * 39.0 * W * C +
                         8.0 * (C + 31.0) * L + 24.0 * (double)c.directions * C;
    const double budget = 0.6 * (double)fr - fixed;
    if (budget <= per_dir) return 1;
    return (int)std::min(1e9, std::floor(budget / per_dir));
}

// Grid of a persistent kernel: as many CTAs as can be resident at once (at
// most the static grid).
template <typename Kern>
static unsigned persistent_grid(Kern kern, int threads, int sms, unsigned nb_static)
{
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, 0) != cudaSuccess || occ < 1) occ = 1;
    return std::min<unsigned>(nb_static, (unsigned)std::max(1, sms * occ));
}

// ----- launch accounting / per-stage timing --------------------------------
// Counts every kernel launch; when a profile is requested, brackets each
// launch with CUDA events on the launching stream and waits for it.
struct Launches {
    int64_t count = 0;
    memd_profile* prof = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    cudaStream_t s = nullptr;
    // NVTX range per launch named after its stage (visible to profilers that
    // filter by range, e.g. ncu --nvtx-include "memd/solve/"; a captured graph
    // carries them only for its capture)
    void begin(int stage)
    {
        static const char* const names[MEMD_STAGES] = {"project", "compact", "factor", "solve",
                                                       "eval",    "other",   "other",  "other"};
        nvtxRangePushA(names[stage]);
        if (prof) cudaEventRecord(a, s);
    }
    void end(int stage)
    {
        ++count;
        nvtxRangePop();
        if (!prof) return;
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        prof->ms[stage] += ms;
        prof->launches[stage] += 1;
    }
};

// ----- evaluation kernels ---------------------------------------------------
#define MEMD_EVAL_CASES(X_)                                                                \
    X_(4, 2) X_(4, 4) X_(4, 8) X_(8, 2) X_(8, 4) X_(8, 8) X_(16, 2) X_(16, 4) X_(16, 8) \
    X_(32, 4) X_(32, 8)
#define MEMD_EVALW_CASES(X_) X_(4, 32) X_(8, 32) X_(16, 32) X_(32, 32) X_(4, 16) X_(8, 16) X_(16, 16)

template <int P>
static void launch_eval(memd_plan* p, cudaStream_t s, int k0, int kc, int first, int last)
{
    using R = typename Prec<P>::R;
    using XT = typename Prec<P>::X;
    const Geom& g = p->g;
    if constexpr (P == MEMD_PREC_F64) {
#define MEMD_CASE(G_, S_)                                                                                  \
    if (p->evalG == G_ && p->evalSPT == S_) {                                                              \
        using Sh = EvalShape<R, G_, S_>;                                                                   \
        dim3 grid((unsigned)((g.L + Sh::T - 1) / Sh::T), (unsigned)((g.C + G_ - 1) / G_));                 \
        k_eval<R, G_, S_><<<grid, 256, Sh::smem_bytes(p->Kc, g.mirror), s>>>(                             \
            (R*)p->X, (R*)p->acc, p->bits, p->wpref, p->knots, p->cnt, (const Fac<R>*)p->fac,            \
            (const R*)p->sv, (const R*)p->yv, g, k0, kc, first, last, p->st, (R*)p->M, (R*)p->part, p->ep, \
            p->mir);                                                                                       \
        return;                                                                                            \
    }
        MEMD_EVAL_CASES(MEMD_CASE)
#undef MEMD_CASE
    } else {
        if constexpr (P == MEMD_PREC_MIXED) {
            if (p->cum) {
                const unsigned* cur = p->bnd + (size_t)(p->bpass & 1) * 2 * g.C;
                unsigned* other = p->bnd + (size_t)((p->bpass + 1) & 1) * 2 * g.C;
#define MEMD_CASE(G_)                                                                                              \
    if (p->cumG == G_) {                                                                                           \
        dim3 grid((unsigned)((g.W + kCumMaxWords - 1) / kCumMaxWords * kCumMaxWords),                             \
                  (unsigned)((g.C + G_ - 1) / G_));                                                                \
        k_mean_cum<G_><<<grid, 256, sizeof(unsigned long long) * (32 * kCumMaxWords + 3) * G_, s>>>(               \
            (const float2*)p->X, (float2*)p->Xb, (dd*)p->acc, p->bits, p->wpref, p->knots, p->cnt,               \
                                            (const dd*)p->rtab, (const dd*)p->rtab3, (const dd*)p->sv,           \
                                            (const dd*)p->yend, cur, other, p->cumcfg, p->cumsh, g, k0, kc, first,\
                                            last, p->st, p->ep);                                                   \
        return;                                                                                                    \
    }
                MEMD_CASE(32) MEMD_CASE(16) MEMD_CASE(8)
#undef MEMD_CASE
            }
        }
        const bool stopm = p->cfg.stop_mode == MEMD_STOP_CRITERION;
#define MEMD_CASE(G_, S_)                                                                                  \
    if (p->ewG == G_ && p->ewSPL == S_) {                                                                  \
        using Sh = EvalWShape<G_, S_, R>;                                                                  \
        dim3 grid((unsigned)((g.L + Sh::T - 1) / Sh::T), (unsigned)((g.C + G_ - 1) / G_));                 \
        if (stopm)                                                                                         \
            k_eval_w<G_, S_, XT, R, true><<<grid, 256, Sh::smem_bytes(true), s>>>(                         \
                (XT*)p->X, (R*)p->acc, p->bits, p->wpref, p->knots, p->cnt, (const R*)p->rtab,             \
                (const R*)p->sv, (const R*)p->yv, g, k0, kc, first, last, p->st, (R*)p->M, (R*)p->part,   \
                p->mir, p->ep);                                                                            \
        else                                                                                               \
            k_eval_w<G_, S_, XT, R, false><<<grid, 256, Sh::smem_bytes(false), s>>>(                       \
                (XT*)p->X, (R*)p->acc, p->bits, p->wpref, p->knots, p->cnt, (const R*)p->rtab,             \
                (const R*)p->sv, (const R*)p->yv, g, k0, kc, first, last, p->st, nullptr, nullptr, p->mir,  \
                p->ep);                                                                                    \
        return;                                                                                            \
    }
        MEMD_EVALW_CASES(MEMD_CASE)
#undef MEMD_CASE
    }
}

template <int P>
static cudaError_t set_attrs(memd_plan* p)
{
    using R = typename Prec<P>::R;
    using XT = typename Prec<P>::X;
    cudaError_t e = cudaSuccess;
    if constexpr (P == MEMD_PREC_F64) {
#define MEMD_CASE(G_, S_)                                                                              \
    if (p->evalG == G_ && p->evalSPT == S_)                                                            \
        e = cudaFuncSetAttribute(k_eval<R, G_, S_>, cudaFuncAttributeMaxDynamicSharedMemorySize,       \
                                 (int)EvalShape<R, G_, S_>::smem_bytes(p->Kc, p->g.mirror));
        MEMD_EVAL_CASES(MEMD_CASE)
#undef MEMD_CASE
    } else {
#define MEMD_CASE(G_, S_)                                                                                     \
    if (p->ewG == G_ && p->ewSPL == S_) {                                                                     \
        e = cudaFuncSetAttribute(k_eval_w<G_, S_, XT, R, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                 (int)EvalWShape<G_, S_, R>::smem_bytes(true));                               \
        if (e == cudaSuccess)                                                                                 \
            e = cudaFuncSetAttribute(k_eval_w<G_, S_, XT, R, false>,                                          \
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,                             \
                                     (int)EvalWShape<G_, S_, R>::smem_bytes(false));                          \
    }
        MEMD_EVALW_CASES(MEMD_CASE)
#undef MEMD_CASE
    }
    if (e != cudaSuccess) return e;
    if constexpr (P == MEMD_PREC_MIXED) {
        const int cb[3] = {32, 16, 8};
        for (int i = 0; i < 3 && e == cudaSuccess; ++i) {
            const int bytes = (int)sizeof(unsigned long long) * (32 * kCumMaxWords + 3) * cb[i];
            if (cb[i] == 32) e = cudaFuncSetAttribute(k_mean_cum<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            if (cb[i] == 16) e = cudaFuncSetAttribute(k_mean_cum<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            if (cb[i] == 8) e = cudaFuncSetAttribute(k_mean_cum<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        }
    }
    if (e != cudaSuccess) return e;
    if constexpr (P == MEMD_PREC_MIXED) {
        e = cudaFuncSetAttribute(k_project_mx, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->proj_smem);
        if (e == cudaSuccess && p->tc)
            e = cudaFuncSetAttribute(k_project_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tc_smem_bytes(p->tc_nt));
    } else
        e = cudaFuncSetAttribute(k_project_extrema<R, XT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)p->proj_smem);
    return e;
}

// ----- one sift, all direction chunks ---------------------------------------
template <int P>
static void enqueue_sift(memd_plan* p, cudaStream_t s, memd_trace_entry* trace, Launches& lc,
                         cudaGraphConditionalHandle h_sift = 0)
{
    using R = typename Prec<P>::R;
    using XT = typename Prec<P>::X;
    const Geom& g = p->g;
    const bool stop = p->cfg.stop_mode == MEMD_STOP_CRITERION;
    const int trace_rows = stop && trace ? (int)(p->cfg.num_imfs * (p->cfg.max_iter + 1)) : 0;
    for (int ch = 0; ch < p->nchunks; ++ch) {
        const int k0 = ch * p->Kc;
        const int kc = std::min(p->Kc, g.K - k0);
        dim3 pg((unsigned)((g.L + kProjTN - 1) / kProjTN), (unsigned)((kc + kProjTK - 1) / kProjTK));
        lc.begin(MEMD_STAGE_PROJECT);
        if constexpr (P == MEMD_PREC_MIXED) {
            if (p->tc) {
                if (ch == 0) {  // tf32 split of the signal's first differences, once per sift
                    const size_t n = (size_t)g.L * p->Cp;
                    k_split_tf32<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, s>>>(
                        p->X, 1, p->xbig, p->xsmall, g.L, g.C, p->Cp);
                    lc.end(MEMD_STAGE_PROJECT);
                    lc.begin(MEMD_STAGE_PROJECT);
                }
                dim3 tg((unsigned)((g.L + kTcRows - 1) / kTcRows), (unsigned)((kc + p->tc_nt - 1) / p->tc_nt));
                k_project_tc<<<tg, kTcThreads, tc_smem_bytes(p->tc_nt), s>>>(
                    p->maps, (const float2*)p->X, (const float*)p->dir, p->bits, g, k0, kc, p->Cp, p->tc_nt, p->st,
                    p->ep);
            } else {
                k_project_mx<<<pg, 256, p->proj_smem, s>>>((const float2*)p->X, (const float*)p->dir,
                                                           (const float*)p->dir + (size_t)g.K * g.C, p->bits, g, k0, kc,
                                                           p->st, p->ep);
            }
        } else
            k_project_extrema<R, XT><<<pg, 256, p->proj_smem, s>>>((const XT*)p->X, (const R*)p->dir, p->bits, g, k0, kc,
                                                                   p->ep);
        lc.end(MEMD_STAGE_PROJECT);
        if (g.mirror) {
            const unsigned mb = (unsigned)((32L * kc + 127) / 128);
            lc.begin(MEMD_STAGE_PROJECT);
            if constexpr (P == MEMD_PREC_MIXED)
                k_mirror<float2, float, float2, true><<<mb, 128, 0, s>>>(
                    p->bits, (const float2*)p->X, nullptr, (const float*)p->dir,
                    (const float*)p->dir + (size_t)g.K * g.C, p->mir, g, k0, kc);
            else
                k_mirror<R, R, XT, false><<<mb, 128, 0, s>>>(p->bits, (const XT*)p->X, (const R*)p->dir, nullptr,
                                                              nullptr, p->mir, g, k0, kc);
            lc.end(MEMD_STAGE_PROJECT);
        }
        const int nch = (g.W + kCompactChunk - 1) / kCompactChunk;
        if (nch > 1) {
            lc.begin(MEMD_STAGE_COMPACT);
            k_compact_count<<<dim3((unsigned)nch, (unsigned)(2 * kc)), 512, 0, s>>>(p->bits, p->csh.ctot, g, nch);
            lc.end(MEMD_STAGE_COMPACT);
        }
        lc.begin(MEMD_STAGE_COMPACT);
        k_compact<R, XT><<<dim3((unsigned)nch, (unsigned)(2 * kc)), 512, 0, s>>>(
            p->bits, p->wpref, p->knots, p->cnt, (R*)p->yv, (const XT*)p->X, trace, g, k0, kc, p->st, trace_rows,
            p->cum ? (R*)p->yend : nullptr, p->ep, p->mir, p->csh, nch);
        lc.end(MEMD_STAGE_COMPACT);
        const long nsegf = (g.cap + p->Sf - 1) / p->Sf;
        const long nf = 2L * kc * nsegf;
        lc.begin(MEMD_STAGE_FACTOR);
        if (g.nak)
            k_factor<R, true><<<(unsigned)((nf + 127) / 128), 128, 0, s>>>(p->knots, p->cnt, (const R*)p->rtab,
                                                                       (Fac<R>*)p->fac, g, k0, kc, p->Sf, p->Hf,
                                                                       p->cum ? p->cumcfg : nullptr, p->ep, p->cum_ctas);
        else
            k_factor<R, false><<<(unsigned)((nf + 127) / 128), 128, 0, s>>>(p->knots, p->cnt, (const R*)p->rtab,
                                                                        (Fac<R>*)p->fac, g, k0, kc, p->Sf, p->Hf,
                                                                        p->cum ? p->cumcfg : nullptr, p->ep, p->cum_ctas);
        lc.end(MEMD_STAGE_FACTOR);
        const long nseg = solve_segments_max(g.cap, p->S, p->Ss, p->H);
        const long ns = 2L * kc * nseg * p->ngroups * 32;
        const unsigned nb = (unsigned)((ns + kSolveThreads - 1) / kSolveThreads);
        unsigned* bcur = p->cum ? p->bnd + (size_t)(p->bpass & 1) * 2 * g.C : nullptr;
        SolveQueue q{};  // null prefix: the static mapping
        if (p->squeue) {
            q = p->sq;
            lc.begin(MEMD_STAGE_SOLVE);
            k_solve_queue<<<1, 1024, 0, s>>>(p->cnt, g, k0, kc, p->S, p->Ss, p->H, p->ngroups, q);
            lc.end(MEMD_STAGE_SOLVE);
        }
        lc.begin(MEMD_STAGE_SOLVE);
        bool xm = false;
#define MEMD_FWD(XM_, EPB_, NAK_)                                                                               \
    k_solve_fwd<R, XT, XM_, EPB_, NAK_><<<p->squeue ? persistent_grid(k_solve_fwd<R, XT, XM_, EPB_, NAK_>,     \
                                                                      kSolveThreads, p->sms, nb) : nb,          \
                                          kSolveThreads, 0, s>>>(                                              \
        (const R*)p->yv, p->cnt, (const Fac<R>*)p->fac, (R*)p->dbuf, g, k0, kc, p->S, p->Ss, p->H, p->ngroups, \
        bcur, XM_ ? (const XT*)p->X : nullptr, p->knots, XM_ ? (const R*)p->yend : nullptr, p->ep,               \
        p->inplace ? (R*)p->hz : nullptr, p->hsegs, q)
        if constexpr (P == MEMD_PREC_MIXED) {
            if (p->cum) {  // knot values from the working signal (the impulse-accumulation path)
                xm = true;
                if (p->ep.n > 0) {  // batched runs: record ends found by position
                    if (g.nak) MEMD_FWD(true, true, true);
                    else MEMD_FWD(true, true, false);
                } else if (g.nak) MEMD_FWD(true, false, true);
                else MEMD_FWD(true, false, false);
            }
        }
        if (!xm) {
            if (g.nak) MEMD_FWD(false, false, true);
            else MEMD_FWD(false, false, false);
        }
#undef MEMD_FWD
        lc.end(MEMD_STAGE_SOLVE);
        lc.begin(MEMD_STAGE_SOLVE);
        // not-a-knot ends: applied in the sweep for one record, by k_nak_ends
        // per record for a batch (the sweep then keeps the identity end rows)
        const bool nak_ends = g.nak && p->ep.n > 0;
        if (g.nak && !nak_ends)  // one record: never in place (its sweep writes the last row from another warp)
            k_solve_bwd<R, true, false>
                <<<p->squeue ? persistent_grid(k_solve_bwd<R, true, false>, kSolveThreads, p->sms, nb) : nb,
                   kSolveThreads, 0, s>>>(p->cnt, (const Fac<R>*)p->fac, (const R*)p->dbuf, (R*)p->sv, g, k0, kc,
                                          p->S, p->Ss, p->H, p->ngroups, bcur, p->knots, nullptr, 0, q);
        else if (p->inplace)
            k_solve_bwd<R, false, true>
                <<<p->squeue ? persistent_grid(k_solve_bwd<R, false, true>, kSolveThreads, p->sms, nb) : nb,
                   kSolveThreads, 0, s>>>(p->cnt, (const Fac<R>*)p->fac, nullptr, (R*)p->sv, g, k0, kc, p->S,
                                          p->Ss, p->H, p->ngroups, bcur, p->knots, (const R*)p->hz, p->hsegs, q);
        else
            k_solve_bwd<R, false, false>
                <<<p->squeue ? persistent_grid(k_solve_bwd<R, false, false>, kSolveThreads, p->sms, nb) : nb,
                   kSolveThreads, 0, s>>>(p->cnt, (const Fac<R>*)p->fac, (const R*)p->dbuf, (R*)p->sv, g, k0, kc,
                                          p->S, p->Ss, p->H, p->ngroups, bcur, p->knots, nullptr, 0, q);
        lc.end(MEMD_STAGE_SOLVE);
        if (nak_ends) {
            const long nt = 2L * kc * p->ep.n * g.C;
            lc.begin(MEMD_STAGE_SOLVE);
            k_nak_ends<R><<<(unsigned)((nt + 127) / 128), 128, 0, s>>>(p->knots, p->cnt, p->wpref,
                                                                        (const Fac<R>*)p->fac, (R*)p->sv, g, k0, kc,
                                                                        p->ep, bcur);
            lc.end(MEMD_STAGE_SOLVE);
        }
        lc.begin(MEMD_STAGE_EVAL);
        launch_eval<P>(p, s, k0, kc, ch == 0, ch == p->nchunks - 1);
        lc.end(MEMD_STAGE_EVAL);
        ++p->bpass;
        if (p->cum && ch == p->nchunks - 1) std::swap(p->X, p->Xb);  // the next pass reads the updated signal
        if (stop) {
            lc.begin(MEMD_STAGE_OTHER);
            k_amp<R><<<(unsigned)((g.L + 255) / 256), 256, 0, s>>>((const R*)p->part, (R*)p->amp, p->cnt, g, k0, kc,
                                                                 p->egroups, ch == 0, p->ep);
            lc.end(MEMD_STAGE_OTHER);
        }
    }
    if (stop && p->batched) {  // every record decides for itself
        RecStop* rs = (RecStop*)p->recstop;
        lc.begin(MEMD_STAGE_OTHER);
        k_rec_q<<<(unsigned)p->ep.n, 32, 0, s>>>(rs, g, p->ep);
        lc.end(MEMD_STAGE_OTHER);
        lc.begin(MEMD_STAGE_OTHER);
        k_stop_stats_b<R><<<(unsigned)std::min<long>((g.L + 255) / 256, 1024), 256, 0, s>>>(
            (const R*)p->M, (const R*)p->amp, rs, g, p->ep, p->cfg.stop_sd, p->cfg.stop_sd2);
        lc.end(MEMD_STAGE_OTHER);
        lc.begin(MEMD_STAGE_OTHER);
        k_decide_b<<<1, 1024, 0, s>>>(p->st, rs, p->ep, p->cfg.stop_tol, (int)p->cfg.max_iter, h_sift);
        lc.end(MEMD_STAGE_OTHER);
        lc.begin(MEMD_STAGE_OTHER);
        k_apply_b<R, XT><<<(unsigned)std::min<size_t>(((size_t)g.C * g.L + 255) / 256, 4096), 256, 0, s>>>(
            (XT*)p->X, (const R*)p->M, rs, g, p->ep);
        lc.end(MEMD_STAGE_OTHER);
    } else if (stop) {
        const size_t CL = (size_t)g.C * g.L;
        lc.begin(MEMD_STAGE_OTHER);
        k_stop_stats<R><<<(unsigned)std::min<long>((g.L + 255) / 256, 1024), 256, 0, s>>>(
            (const R*)p->M, (const R*)p->amp, p->cnt, g, p->cfg.stop_sd, p->cfg.stop_sd2, p->st);
        lc.end(MEMD_STAGE_OTHER);
        lc.begin(MEMD_STAGE_OTHER);
        k_decide<<<1, 32, 0, s>>>(p->st, p->cnt, g, p->cfg.stop_tol, (int)p->cfg.max_iter, h_sift, p->mir);
        lc.end(MEMD_STAGE_OTHER);
        lc.begin(MEMD_STAGE_OTHER);
        k_apply<R, XT><<<(unsigned)std::min<size_t>((CL + 255) / 256, 4096), 256, 0, s>>>((XT*)p->X, (const R*)p->M,
                                                                                         p->st, CL);
        lc.end(MEMD_STAGE_OTHER);
    }
}

template <int P>
static void enqueue_decomposition(memd_plan* p, cudaStream_t s, Launches& lc)
{
    using XT = typename Prec<P>::X;
    using T = typename Prec<P>::T;
    const Geom& g = p->g;
    const size_t CL = (size_t)g.C * g.L;
    const int nimf = (int)p->cfg.num_imfs;
    const int maxit = (int)p->cfg.max_iter;
    dim3 tb(32, 8), tg((unsigned)((g.L + 31) / 32), (unsigned)((g.C + 31) / 32));
    p->bpass = 0;
    void* const x0 = p->X;
    if (p->cum) cudaMemsetAsync(p->bnd, 0, sizeof(unsigned) * 4 * (size_t)g.C, s);
    for (int i = 0; i + 1 < nimf; ++i) {
        nvtxRangePushA("imf");
        cudaMemcpyAsync(p->X, p->run, CL * sizeof(XT), cudaMemcpyDeviceToDevice, s);
        for (int j = 0; j < maxit; ++j) {
            memd_trace_entry* tr = p->trace_dev ? p->trace_dev + ((size_t)i * (maxit + 1) + j) * (size_t)g.K * 2 : nullptr;
            nvtxRangePushA("sift");
            enqueue_sift<P>(p, s, tr, lc);
            nvtxRangePop();
        }
        nvtxRangePop();
        lc.begin(MEMD_STAGE_OTHER);
        k_to_channel_major<XT, T><<<tg, tb, 0, s>>>((const XT*)p->X, (T*)p->imf + (size_t)i * CL, (XT*)p->run, g.C, g.L);
        lc.end(MEMD_STAGE_OTHER);
    }
    lc.begin(MEMD_STAGE_OTHER);
    k_to_channel_major<XT, T><<<tg, tb, 0, s>>>((const XT*)p->run, (T*)p->imf + (size_t)(nimf - 1) * CL, nullptr, g.C, g.L);
    lc.end(MEMD_STAGE_OTHER);
    if (p->X != x0) std::swap(p->X, p->Xb);  // the buffers' roles as at the start
}

template <int P>
static memd_status build_graph(memd_plan* p)
{
    if (p->exec) return MEMD_OK;
    cudaError_t e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return set_cuda_error("graph: begin capture", e);
    Launches lc;
    enqueue_decomposition<P>(p, p->cap, lc);
    p->graph_launches = lc.count;
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(p->cap, &graph);
    if (e != cudaSuccess) return set_cuda_error("graph: end capture", e);
    e = cudaGraphInstantiate(&p->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        p->exec = nullptr;
        return set_cuda_error("graph: instantiate", e);
    }
    return MEMD_OK;
}

// Stop mode: the IMF loop and the sift loop are conditional WHILE nodes
// (the sift loop nested in the IMF loop's body); k_decide and k_imf_commit set
// their conditions on the device, so a run needs no host round trip.
template <int P>
static memd_status build_graph_stop(memd_plan* p)
{
    using XT = typename Prec<P>::X;
    using T = typename Prec<P>::T;
    if (p->exec) return MEMD_OK;
    const Geom& g = p->g;
    const size_t CL = (size_t)g.C * g.L;
    const int nimf = (int)p->cfg.num_imfs;
    const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    dim3 tb(32, 8), tg((unsigned)((g.L + 31) / 32), (unsigned)((g.C + 31) / 32));
    cudaGraph_t top = nullptr;
    cudaError_t e = cudaGraphCreate(&top, 0);
    if (e != cudaSuccess) return set_cuda_error("graph: create", e);
    Launches lc;
    cudaGraphConditionalHandle h_imf = 0, h_sift = 0;
    cudaGraphNode_t outer = nullptr, inner = nullptr;
    cudaGraph_t obody = nullptr, ibody = nullptr;
    std::vector<cudaGraphNode_t> d1;
    do {
        e = cudaGraphConditionalHandleCreate(&h_imf, top, nimf > 1 ? 1u : 0u, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) break;
        cudaGraphNodeParams op = {};
        op.type = cudaGraphNodeTypeConditional;
        op.conditional.handle = h_imf;
        op.conditional.type = cudaGraphCondTypeWhile;
        op.conditional.size = 1;
        e = cudaGraphAddNode(&outer, top, nullptr, nullptr, 0, &op);
        if (e != cudaSuccess) break;
        obody = op.conditional.phGraph_out[0];
        e = cudaGraphConditionalHandleCreate(&h_sift, obody, 1u, 0);
        if (e != cudaSuccess) break;
        // IMF body, part 1: X = running residual, sift loop armed
        e = cudaStreamBeginCaptureToGraph(p->cap, obody, nullptr, nullptr, 0, mode);
        if (e != cudaSuccess) break;
        cudaMemcpyAsync(p->X, p->run, CL * sizeof(XT), cudaMemcpyDeviceToDevice, p->cap);
        if (p->batched)
            k_imf_begin_b<<<1, 1024, 0, p->cap>>>((RecStop*)p->recstop, p->ep, h_sift);
        else
            k_imf_begin<<<1, 32, 0, p->cap>>>(p->st, (int)p->cfg.max_iter, p->trace_dev ? 1 : 0, h_sift);
        {
            cudaStreamCaptureStatus cs;
            const cudaGraphNode_t* deps = nullptr;
            size_t nd = 0;
            e = cudaStreamGetCaptureInfo(p->cap, &cs, nullptr, nullptr, &deps, nullptr, &nd);
            if (e == cudaSuccess) d1.assign(deps, deps + nd);
        }
        cudaGraph_t tmp = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(p->cap, &tmp);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (e == cudaSuccess) e = e2;
            break;
        }
        cudaGraphNodeParams ip = {};
        ip.type = cudaGraphNodeTypeConditional;
        ip.conditional.handle = h_sift;
        ip.conditional.type = cudaGraphCondTypeWhile;
        ip.conditional.size = 1;
        e = cudaGraphAddNode(&inner, obody, d1.data(), nullptr, d1.size(), &ip);
        if (e != cudaSuccess) break;
        ibody = ip.conditional.phGraph_out[0];
        // sift body: one envelope pass + stop test + (conditional) subtraction
        e = cudaStreamBeginCaptureToGraph(p->cap, ibody, nullptr, nullptr, 0, mode);
        if (e != cudaSuccess) break;
        enqueue_sift<P>(p, p->cap, p->batched ? nullptr : p->trace_dev, lc, h_sift);
        e = cudaStreamEndCapture(p->cap, &tmp);
        if (e != cudaSuccess) break;
        // IMF body, part 2: write the IMF, update the residual, continue?
        e = cudaStreamBeginCaptureToGraph(p->cap, obody, &inner, nullptr, 1, mode);
        if (e != cudaSuccess) break;
        if (p->batched) {
            k_imf_out_b<XT, T><<<tg, tb, 0, p->cap>>>((const XT*)p->X, (T*)p->imf, (XT*)p->run,
                                                       (const RecStop*)p->recstop, p->ep, g.C, g.L);
            k_imf_commit_b<<<1, 1024, 0, p->cap>>>(p->st, (RecStop*)p->recstop, p->ep, nimf, h_imf);
        } else {
            k_imf_out_dyn<XT, T><<<tg, tb, 0, p->cap>>>((const XT*)p->X, (T*)p->imf, (XT*)p->run, p->st, g.C, g.L);
            k_imf_commit<<<1, 32, 0, p->cap>>>(p->st, nimf, h_imf);
        }
        e = cudaStreamEndCapture(p->cap, &tmp);
        if (e != cudaSuccess) break;
        // after the IMF loop: unused slots zeroed, residual into the last slot
        e = cudaStreamBeginCaptureToGraph(p->cap, top, &outer, nullptr, 1, mode);
        if (e != cudaSuccess) break;
        if (p->batched)
            k_zero_unused_b<T><<<1024, 256, 0, p->cap>>>((T*)p->imf, (const RecStop*)p->recstop, p->ep, nimf, g.C, g.L);
        else
            k_zero_unused<T><<<1024, 256, 0, p->cap>>>((T*)p->imf, p->st, nimf, CL);
        k_to_channel_major<XT, T><<<tg, tb, 0, p->cap>>>((const XT*)p->run, (T*)p->imf + (size_t)(nimf - 1) * CL,
                                                         nullptr, g.C, g.L);
        e = cudaStreamEndCapture(p->cap, &tmp);
        if (e != cudaSuccess) break;
        e = cudaGraphInstantiate(&p->exec, top, 0);
    } while (0);
    cudaGraphDestroy(top);
    if (e != cudaSuccess) {
        p->exec = nullptr;
        cudaGetLastError();
        return set_cuda_error("graph: stop-mode build", e);
    }
    p->graph_launches = lc.count;  // kernels of one sift pass (dynamic count per run)
    return MEMD_OK;
}

// tf32 big / small parts of the directions' high words for the tensor-core
// projection (the directions are constant over a run).
static void split_directions(memd_plan* p, cudaStream_t s, Launches& lc)
{
    if (!p->tc) return;
    const size_t n = (size_t)p->g.K * p->Cp;
    lc.begin(MEMD_STAGE_OTHER);
    k_split_tf32<<<(unsigned)std::min<size_t>((n + 255) / 256, 1024), 256, 0, s>>>(p->dir, 0, p->dbig, p->dsmall,
                                                                                   p->g.K, p->g.C, p->Cp);
    lc.end(MEMD_STAGE_OTHER);
}

// Bounds-checked build: the index-check failures since the last call
// (MEMD_FLAG_CHECK_FAILED), cleared; always 0 in the normal build.
static int checked_flags()
{
#ifdef MEMD_CHECKED
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_memd_check, sizeof(int)) != cudaSuccess) return 0;
    if (v) {
        const int z = 0;
        cudaMemcpyToSymbol(g_memd_check, &z, sizeof(int));
        return MEMD_FLAG_CHECK_FAILED;
    }
#endif
    return 0;
}

// Caller's record -> working layout; directions -> plan buffer.
template <int P>
static void enqueue_inputs(memd_plan* p, const typename Prec<P>::T* d_y, const typename Prec<P>::T* d_dir,
                           cudaStream_t s, Launches& lc)
{
    using XT = typename Prec<P>::X;
    using T = typename Prec<P>::T;
    const Geom& g = p->g;
    dim3 tb(32, 8), tg((unsigned)((g.L + 31) / 32), (unsigned)((g.C + 31) / 32));
    lc.begin(MEMD_STAGE_OTHER);
    k_to_sample_major<XT, T><<<tg, tb, 0, s>>>(d_y, (XT*)p->run, g.C, g.L);
    lc.end(MEMD_STAGE_OTHER);
    cudaMemcpyAsync(p->dir, d_dir, sizeof(T) * (size_t)g.K * g.C, cudaMemcpyDeviceToDevice, s);
    if constexpr (P == MEMD_PREC_MIXED) {  // float directions: the low words are zero
        cudaMemsetAsync((float*)p->dir + (size_t)g.K * g.C, 0, sizeof(float) * (size_t)g.K * g.C, s);
        split_directions(p, s, lc);
    }
}

template <int P>
static memd_status run_impl(memd_plan* p, const int32_t* d_x, const typename Prec<P>::T* d_y,
                            const typename Prec<P>::T* d_dir, typename Prec<P>::T* d_imfs, void* stream,
                            memd_stats* stats)
{
    using T = typename Prec<P>::T;
    cudaStream_t s = (cudaStream_t)stream;
    const Geom& g = p->g;
    const size_t CL = (size_t)g.C * g.L;
    cudaError_t e;
    if (d_x) {
        cudaMemsetAsync(p->coord_bad, 0, sizeof(int), s);
        k_check_coords<<<64, 256, 0, s>>>(d_x, g.L, p->coord_bad);
        cudaMemcpyAsync(p->host_flag, p->coord_bad, sizeof(int), cudaMemcpyDeviceToHost, s);
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return set_cuda_error("run: coordinate check", e);
        if (*p->host_flag) return set_error(MEMD_ERR_COORD, "run: d_x must hold 0..L-1");
    }
    const bool stopm = p->cfg.stop_mode == MEMD_STOP_CRITERION;
    memd_status st = stopm ? build_graph_stop<P>(p) : build_graph<P>(p);
    if (st != MEMD_OK) return st;
    cudaMemsetAsync(p->st, 0, sizeof(RunState), s);
    Launches lc;
    enqueue_inputs<P>(p, d_y, d_dir, s, lc);
    // the copies and clears above must have been accepted before the graph
    // runs on the buffers they fill
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error("run: inputs", e);
    cudaEventRecord(p->e0, s);
    nvtxRangePushA("memd_run");
    e = cudaGraphLaunch(p->exec, s);
    nvtxRangePop();
    if (e != cudaSuccess) return set_cuda_error("run: graph launch", e);
    cudaEventRecord(p->e1, s);
    cudaMemcpyAsync(d_imfs, p->imf, sizeof(T) * CL * (size_t)p->cfg.num_imfs, cudaMemcpyDeviceToDevice, s);
    if (p->trace_dev && p->trace_host)
        cudaMemcpyAsync(p->trace_host, p->trace_dev, sizeof(memd_trace_entry) * p->trace_n, cudaMemcpyDeviceToHost, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error("run: launch", e);
    if (stats || (p->trace_dev && p->trace_host)) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return set_cuda_error("run: synchronize", e);
    }
    if (stats) {
        RunState hs;
        e = cudaMemcpy(&hs, p->st, sizeof(RunState), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return set_cuda_error("run: read state", e);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p->e0, p->e1);
        memset(stats, 0, sizeof(*stats));
        stats->elapsed_ms = ms;
        stats->flags = hs.flags | checked_flags();
        if (stopm) {
            stats->n_imfs = hs.n_imfs;
            for (int i = 0; i < hs.n_imfs && i < 64; ++i) stats->sifts[i] = hs.sifts[i];
            // per pass: the sift kernels; per IMF: begin, out, commit; at the end: 2
            stats->launches = p->graph_launches * (int64_t)hs.pad[0] + 3LL * (hs.n_imfs + 1) + 2 + lc.count + (d_x ? 1 : 0);
        } else {
            stats->n_imfs = (int)p->cfg.num_imfs - 1;
            stats->launches = p->graph_launches + lc.count + (d_x ? 1 : 0);
            for (int i = 0; i + 1 < (int)p->cfg.num_imfs && i < 64; ++i) stats->sifts[i] = (int)p->cfg.max_iter;
        }
        stats->refined = hs.pad[3];
    }
    return MEMD_OK;
}

// Batched run: lay the epochs out at multiples of kEpochAlign samples (the
// graph is rebuilt when the set of lengths changes), scatter the records into
// the working signal, run the decomposition graph over all of them at once,
// and scatter the IMFs back to each epoch's block.
template <int P>
static memd_status batched_inputs(memd_plan* p, int n, const int64_t* lengths, const int64_t* offsets,
                                  const typename Prec<P>::T* d_y, const typename Prec<P>::T* d_dir,
                                  typename Prec<P>::T* d_imfs, cudaStream_t s)
{
    using XT = typename Prec<P>::X;
    using T = typename Prec<P>::T;
    if (!p->batched) return set_error(MEMD_ERR_UNSUPPORTED, "run_batched: the plan was created without max_epochs");
    if (n < 1 || n > p->cfg.max_epochs) return set_error(MEMD_ERR_INVALID, "run_batched: n_epochs out of range");
    if (!lengths || !offsets || !d_y || !d_dir || !d_imfs) return set_error(MEMD_ERR_INVALID, "run_batched: null argument");
    for (int e = 0; e < n; ++e) {
        if (lengths[e] < 4 || lengths[e] > p->Lrec) return set_error(MEMD_ERR_INVALID, "run_batched: epoch length out of range");
        if (offsets[e] < 0) return set_error(MEMD_ERR_INVALID, "run_batched: negative offset");
    }
    const int C = p->g.C;
    cudaError_t e;
    std::vector<int64_t> lens(lengths, lengths + n);
    if (lens != p->ep_lens || !p->exec) {
        // A run still in flight on s may be reading the epoch table (its graph
        // and k_batched_out): let it finish before the table and the graph
        // change.  Only a change of the length set takes this path.
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return set_cuda_error("run_batched: synchronize before a new layout", e);
        // layout: off[e] = sum of the earlier lengths rounded up to kEpochAlign
        const int me = (int)p->cfg.max_epochs;
        std::vector<int> off(n), cov(n), w0(n + 1);
        int64_t acc = 0;
        for (int i = 0; i < n; ++i) {
            off[i] = (int)acc;
            const int Le = (int)lens[i];
            cov[i] = p->cfg.ref_window ? 240 * ((Le + 241) / 242) : Le;
            w0[i] = (int)(acc / 32);
            acc += (Le + kEpochAlign - 1) / kEpochAlign * kEpochAlign;
        }
        const int Ltot = (int)acc, W = Ltot / 32;
        w0[n] = W;
        p->ep_host.assign(4 * (size_t)me + 1 + (size_t)W, 0);
        int* h = p->ep_host.data();
        for (int i = 0; i < n; ++i) {
            h[i] = off[i];
            h[me + i] = (int)lens[i];
            h[2 * me + i] = cov[i];
        }
        for (int i = 0; i <= n; ++i) h[3 * me + i] = w0[i];
        int* wep = h + 4 * me + 1;
        for (int i = 0; i < n; ++i)
            for (int w = w0[i]; w < w0[i + 1]; ++w) wep[w] = i;
        // stream-ordered copy on the caller's stream; the host staging vector
        // is rewritten only on the next layout change, after the synchronise
        // above
        e = cudaMemcpyAsync(p->ep_dev, h, sizeof(int) * p->ep_host.size(), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return set_cuda_error("run_batched: epoch table", e);
        p->ep.n = n;
        p->ep.off = p->ep_dev;
        p->ep.len = p->ep_dev + me;
        p->ep.cov = p->ep_dev + 2 * me;
        p->ep.w0 = p->ep_dev + 3 * me;
        p->ep.wep = p->ep_dev + 4 * me + 1;
        p->g.L = Ltot;
        p->g.W = W;
        if (p->exec) cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
        p->ep_lens = lens;
    }
    const Geom& g = p->g;
    const size_t CL = (size_t)C * g.L;
    std::vector<long long> yoff(offsets, offsets + n);
    e = cudaMemcpyAsync(p->ep_yoff, yoff.data(), sizeof(long long) * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return set_cuda_error("run_batched: offsets", e);
    cudaMemsetAsync(p->st, 0, sizeof(RunState), s);
    // the gaps between epochs stay zero in every working buffer
    cudaMemsetAsync(p->run, 0, CL * sizeof(XT), s);
    cudaMemsetAsync(p->X, 0, CL * sizeof(XT), s);
    if (p->Xb) cudaMemsetAsync(p->Xb, 0, CL * sizeof(XT), s);
    k_batched_in<XT, T><<<dim3((unsigned)g.W, (unsigned)((C + 31) / 32)), dim3(32, 8), 0, s>>>(d_y, p->ep_yoff, (XT*)p->run,
                                                                                              C, p->ep);
    cudaMemcpyAsync(p->dir, d_dir, sizeof(T) * (size_t)g.K * C, cudaMemcpyDeviceToDevice, s);
    if constexpr (P == MEMD_PREC_MIXED) {
        cudaMemsetAsync((float*)p->dir + (size_t)g.K * C, 0, sizeof(float) * (size_t)g.K * C, s);
        Launches lc;
        split_directions(p, s, lc);
    }
    // the copies and clears above must have been accepted before the graph
    // runs on the buffers they fill
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error("run_batched: inputs", e);
    return MEMD_OK;
}

template <int P>
static memd_status run_batched_impl(memd_plan* p, int n, const int64_t* lengths, const int64_t* offsets,
                                    const typename Prec<P>::T* d_y, const typename Prec<P>::T* d_dir,
                                    typename Prec<P>::T* d_imfs, void* stream, memd_stats* stats)
{
    using T = typename Prec<P>::T;
    cudaStream_t s = (cudaStream_t)stream;
    memd_status st = batched_inputs<P>(p, n, lengths, offsets, d_y, d_dir, d_imfs, s);
    if (st != MEMD_OK) return st;
    const bool stopm = p->cfg.stop_mode == MEMD_STOP_CRITERION;
    if (stopm) {
        const cudaError_t ez = cudaMemsetAsync(p->recstop, 0, sizeof(RecStop) * (size_t)n, s);
        if (ez != cudaSuccess) return set_cuda_error("run_batched: clear per-epoch state", ez);
    }
    st = stopm ? build_graph_stop<P>(p) : build_graph<P>(p);
    if (st != MEMD_OK) return st;
    const Geom& g = p->g;
    const int C = g.C;
    cudaEventRecord(p->e0, s);
    cudaError_t e = cudaGraphLaunch(p->exec, s);
    if (e != cudaSuccess) return set_cuda_error("run_batched: graph launch", e);
    cudaEventRecord(p->e1, s);
    k_batched_out<T><<<1024, 256, 0, s>>>((const T*)p->imf, p->ep_yoff, d_imfs, C, g.L, (int)p->cfg.num_imfs, p->ep);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error("run_batched: launch", e);
    if (stats) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return set_cuda_error("run_batched: synchronize", e);
        RunState hs;
        e = cudaMemcpy(&hs, p->st, sizeof(RunState), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return set_cuda_error("run_batched: read state", e);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p->e0, p->e1);
        memset(stats, 0, sizeof(*stats));
        stats->elapsed_ms = ms;
        stats->flags = hs.flags | checked_flags();
        if (stopm) {  // per-epoch counts: memd_batched_counts
            stats->n_imfs = hs.n_imfs;
            stats->launches = p->graph_launches * (int64_t)hs.pad[0] + 3LL * (hs.n_imfs + 1) + 2;
        } else {
            stats->n_imfs = (int)p->cfg.num_imfs - 1;
            stats->launches = p->graph_launches + 2;
            for (int i = 0; i + 1 < (int)p->cfg.num_imfs && i < 64; ++i) stats->sifts[i] = (int)p->cfg.max_iter;
        }
        stats->refined = hs.pad[3];
    }
    return MEMD_OK;
}

template <int P>
static memd_status profile_impl(memd_plan* p, const typename Prec<P>::T* d_y, const typename Prec<P>::T* d_dir,
                                typename Prec<P>::T* d_imfs, void* stream, memd_profile* prof)
{
    using XT = typename Prec<P>::X;
    using T = typename Prec<P>::T;
    cudaStream_t s = (cudaStream_t)stream;
    const Geom& g = p->g;
    const size_t CL = (size_t)g.C * g.L;
    memset(prof, 0, sizeof(*prof));
    Launches lc;
    lc.prof = prof;
    lc.s = s;
    cudaEventCreate(&lc.a);
    cudaEventCreate(&lc.b);
    cudaMemsetAsync(p->st, 0, sizeof(RunState), s);
    dim3 tb(32, 8), tg((unsigned)((g.L + 31) / 32), (unsigned)((g.C + 31) / 32));
    enqueue_inputs<P>(p, d_y, d_dir, s, lc);
    {
        const cudaError_t ei = cudaGetLastError();
        if (ei != cudaSuccess) {
            cudaEventDestroy(lc.a);
            cudaEventDestroy(lc.b);
            return set_cuda_error("profile: inputs", ei);
        }
    }
    memd_trace_entry* keep = p->trace_dev;
    p->trace_dev = nullptr;
    if (p->cfg.stop_mode == MEMD_STOP_CRITERION) {
        // the graph's data-dependent loops, driven from the host
        RunState hs;
        const int nimf = (int)p->cfg.num_imfs;
        for (int i = 0; i + 1 < nimf; ++i) {
            cudaMemcpyAsync(p->X, p->run, CL * sizeof(XT), cudaMemcpyDeviceToDevice, s);
            k_imf_begin<<<1, 32, 0, s>>>(p->st, (int)p->cfg.max_iter, 0, 0);
            for (;;) {
                enqueue_sift<P>(p, s, nullptr, lc, 0);
                cudaMemcpyAsync(&hs, p->st, sizeof(RunState), cudaMemcpyDeviceToHost, s);
                cudaStreamSynchronize(s);
                if (!hs.pad[1]) break;
            }
            k_imf_out_dyn<XT, T><<<tg, tb, 0, s>>>((const XT*)p->X, (T*)p->imf, (XT*)p->run, p->st, g.C, g.L);
            k_imf_commit<<<1, 32, 0, s>>>(p->st, nimf, 0);
            cudaMemcpyAsync(&hs, p->st, sizeof(RunState), cudaMemcpyDeviceToHost, s);
            cudaStreamSynchronize(s);
            if (!hs.pad[2]) break;
        }
        k_zero_unused<T><<<1024, 256, 0, s>>>((T*)p->imf, p->st, nimf, CL);
        k_to_channel_major<XT, T><<<tg, tb, 0, s>>>((const XT*)p->run, (T*)p->imf + (size_t)(nimf - 1) * CL, nullptr,
                                                    g.C, g.L);
    } else {
        enqueue_decomposition<P>(p, s, lc);
    }
    p->trace_dev = keep;
    cudaMemcpyAsync(d_imfs, p->imf, sizeof(T) * CL * (size_t)p->cfg.num_imfs, cudaMemcpyDeviceToDevice, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(lc.a);
    cudaEventDestroy(lc.b);
    if (e != cudaSuccess) return set_cuda_error("profile: run", e);
    return MEMD_OK;
}

// Batched run launched kernel by kernel, each timed (per-stage figures).
template <int P>
static memd_status profile_batched_impl(memd_plan* p, int n, const int64_t* lengths, const int64_t* offsets,
                                        const typename Prec<P>::T* d_y, const typename Prec<P>::T* d_dir,
                                        typename Prec<P>::T* d_imfs, void* stream, memd_profile* prof)
{
    using T = typename Prec<P>::T;
    cudaStream_t s = (cudaStream_t)stream;
    if (p->cfg.stop_mode == MEMD_STOP_CRITERION)
        return set_error(MEMD_ERR_UNSUPPORTED, "profile_batched: stop mode is profiled per record (memd_profile_*)");
    memd_status st = batched_inputs<P>(p, n, lengths, offsets, d_y, d_dir, d_imfs, s);
    if (st != MEMD_OK) return st;
    memset(prof, 0, sizeof(*prof));
    Launches lc;
    lc.prof = prof;
    lc.s = s;
    cudaEventCreate(&lc.a);
    cudaEventCreate(&lc.b);
    memd_trace_entry* keep = p->trace_dev;
    p->trace_dev = nullptr;
    enqueue_decomposition<P>(p, s, lc);
    p->trace_dev = keep;
    k_batched_out<T><<<1024, 256, 0, s>>>((const T*)p->imf, p->ep_yoff, d_imfs, p->g.C, p->g.L,
                                          (int)p->cfg.num_imfs, p->ep);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(lc.a);
    cudaEventDestroy(lc.b);
    if (e != cudaSuccess) return set_cuda_error("profile_batched: run", e);
    return MEMD_OK;
}

}  // namespace memd

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

void memd_default_config(memd_config* cfg)
{
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->num_imfs = 9;
    cfg->max_iter = 10;
    cfg->precision = MEMD_PREC_F64;
    cfg->stop_mode = MEMD_STOP_FIXED;
    cfg->stop_sd = 0.075;
    cfg->stop_sd2 = 0.75;
    cfg->stop_tol = 0.075;
    cfg->ref_window = 1;
}

const char* memd_last_error(void) { return memd::g_err.c_str(); }

#ifdef MEMD_CHECKED
const char* memd_version(void) { return "memd-gb300 0.2 (sm_103a, bounds-checked)"; }
#else
const char* memd_version(void) { return "memd-gb300 0.2 (sm_103a)"; }
#endif

memd_status memd_plan_destroy(memd_plan* p)
{
    if (!p) return MEMD_OK;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    for (void* a : p->allocs) cudaFree(a);
    if (p->host_flag) cudaFreeHost(p->host_flag);
    if (p->cap) cudaStreamDestroy(p->cap);
    if (p->e0) cudaEventDestroy(p->e0);
    if (p->e1) cudaEventDestroy(p->e1);
    delete p;
    return MEMD_OK;
}

size_t memd_plan_workspace_bytes(const memd_plan* p) { return p ? p->bytes : 0; }

memd_status memd_plan_create(const memd_config* cfg, memd_plan** out) { return memd_plan_create_tuned(cfg, nullptr, out); }

memd_status memd_plan_get_tuning(const memd_plan* p, memd_tuning* t)
{
    using namespace memd;
    if (!p || !t) return set_error(MEMD_ERR_INVALID, "get_tuning: null argument");
    memset(t, 0, sizeof(*t));
    t->solve_segment = p->S;
    t->solve_min_segment = p->Ss;
    t->factor_segment = p->Sf;
    t->solve_queue = p->squeue ? 1 : 2;
    t->mean_ctas = p->cum_ctas;
    t->proj_tile_n = p->tc ? p->tc_nt : 0;
    t->solve_layout = p->inplace ? 1 : 2;
    return MEMD_OK;
}

namespace memd {
static memd_status create_plan(const memd_config* cfg, const memd_tuning* tun, memd_plan** out, int kc_limit,
                               int* kc_used);
}

// A plan with the automatic direction chunk whose allocation fails is made
// again with half the directions per pass.
memd_status memd_plan_create_tuned(const memd_config* cfg, const memd_tuning* tun, memd_plan** out)
{
    using namespace memd;
    int limit = INT_MAX;
    for (;;) {
        int used = 0;
        const memd_status s = create_plan(cfg, tun, out, limit, &used);
        if (s != MEMD_ERR_NOMEM || !cfg || cfg->dir_chunk > 0 || used <= 1) return s;
        cudaGetLastError();
        limit = used / 2;
    }
}

namespace memd {
static memd_status create_plan(const memd_config* cfg, const memd_tuning* tun, memd_plan** out, int kc_limit,
                               int* kc_used)
{
    *kc_used = 0;
    if (!cfg || !out) return set_error(MEMD_ERR_INVALID, "plan: null argument");
    memd_tuning tu;
    memset(&tu, 0, sizeof(tu));
    if (tun) tu = *tun;
    auto pow2 = [](int v) { return v > 0 && (v & (v - 1)) == 0; };
    if (tu.solve_segment && (!pow2(tu.solve_segment) || tu.solve_segment < 32 || tu.solve_segment > 1024))
        return set_error(MEMD_ERR_INVALID, "tuning: solve_segment must be a power of two in [32, 1024]");
    if (tu.solve_min_segment &&
        (!pow2(tu.solve_min_segment) || tu.solve_min_segment < 16 ||
         tu.solve_min_segment > (tu.solve_segment ? tu.solve_segment : 256)))
        return set_error(MEMD_ERR_INVALID, "tuning: solve_min_segment must be a power of two in [16, solve_segment]");
    if (tu.factor_segment && (tu.factor_segment < 4 || tu.factor_segment > 256))
        return set_error(MEMD_ERR_INVALID, "tuning: factor_segment must be in [4, 256]");
    if (tu.solve_queue < 0 || tu.solve_queue > 2) return set_error(MEMD_ERR_INVALID, "tuning: solve_queue must be 0, 1 or 2");
    if (tu.mean_ctas && (tu.mean_ctas < 128 || tu.mean_ctas > 65536))
        return set_error(MEMD_ERR_INVALID, "tuning: mean_ctas must be in [128, 65536]");
    if (tu.proj_tile_n && (tu.proj_tile_n % 16 != 0 || tu.proj_tile_n < 16 || tu.proj_tile_n > kTcMaxN))
        return set_error(MEMD_ERR_INVALID, "tuning: proj_tile_n must be a multiple of 16 in [16, 256]");
    if (tu.solve_layout < 0 || tu.solve_layout > 2) return set_error(MEMD_ERR_INVALID, "tuning: solve_layout must be 0, 1 or 2");
    *out = nullptr;
    const memd_config c = *cfg;
    if (c.channels < 1 || c.channels > 256) return set_error(MEMD_ERR_INVALID, "plan: channels must be in [1, 256]");
    if (c.length < 4 || c.length > (1LL << 28)) return set_error(MEMD_ERR_INVALID, "plan: length must be in [4, 2^28]");
    if (c.directions < 1 || c.directions > 65536) return set_error(MEMD_ERR_INVALID, "plan: directions must be in [1, 65536]");
    if (c.num_imfs < 1 || c.num_imfs > 4096) return set_error(MEMD_ERR_INVALID, "plan: num_imfs must be in [1, 4096]");
    if (c.max_iter < 0 || c.max_iter > 100000) return set_error(MEMD_ERR_INVALID, "plan: max_iter must be in [0, 100000]");
    if (c.precision < MEMD_PREC_F64 || c.precision > MEMD_PREC_MIXED) return set_error(MEMD_ERR_INVALID, "plan: bad precision");
    if (c.stop_mode != MEMD_STOP_FIXED && c.stop_mode != MEMD_STOP_CRITERION)
        return set_error(MEMD_ERR_INVALID, "plan: bad stop mode");
    if (c.stop_mode == MEMD_STOP_CRITERION && (c.max_iter < 1 || !(c.stop_sd > 0) || !(c.stop_sd2 > 0) || c.stop_tol < 0))
        return set_error(MEMD_ERR_INVALID, "plan: stop criterion needs max_iter >= 1 and positive thresholds");
    if (c.max_epochs < 0 || c.max_epochs > (1 << 20)) return set_error(MEMD_ERR_INVALID, "plan: bad max_epochs");
    if (c.spline_end != MEMD_SPLINE_NATURAL && c.spline_end != MEMD_SPLINE_NOT_A_KNOT)
        return set_error(MEMD_ERR_INVALID, "plan: bad spline_end");
    if (c.boundary != MEMD_BOUNDARY_REFERENCE && c.boundary != MEMD_BOUNDARY_MIRROR)
        return set_error(MEMD_ERR_INVALID, "plan: bad boundary");
    if (c.projection != 0 && c.projection != 1) return set_error(MEMD_ERR_INVALID, "plan: projection must be 0 or 1");
    if (c.max_epochs > 0 && c.boundary != MEMD_BOUNDARY_REFERENCE)
        return set_error(MEMD_ERR_UNSUPPORTED, "plan: batched runs are built for the reference boundary");
    if (c.max_epochs > 0) {
        if ((int64_t)c.max_epochs * ((c.length + kEpochAlign - 1) / kEpochAlign * kEpochAlign) > (1LL << 28))
            return set_error(MEMD_ERR_INVALID, "plan: max_epochs x length exceeds 2^28 samples");
    }
    memd_plan* p = new memd_plan();  // value-initialised: every pointer and count starts at zero
    p->cfg = c;
    const int C = (int)c.channels, K = (int)c.directions;
    p->batched = c.max_epochs > 0;
    p->Lrec = (int)c.length;
    // batched: room for max_epochs epochs of the longest length, each padded to
    // a multiple of kEpochAlign samples
    const int L = p->batched ? (int)(c.max_epochs * ((c.length + kEpochAlign - 1) / kEpochAlign * kEpochAlign))
                             : (int)c.length;
    p->prec = c.precision;
    const bool f64 = c.precision == MEMD_PREC_F64;
    p->real_bytes = (f64 || c.precision == MEMD_PREC_MIXED) ? 8 : 4;  // double, float or double-float
    p->xbytes = f64 ? 8 : (c.precision == MEMD_PREC_MIXED ? 8 : 4);
    p->tbytes = f64 ? 8 : 4;
    p->g.C = C;
    p->g.L = L;
    p->g.K = K;
    p->g.W = (L + 31) / 32;
    p->g.cap = p->batched ? L / 2 + 5 * (int)c.max_epochs + 4 : (L + 1) / 2 + 4 + (c.boundary ? 4 : 0);
    p->g.cov = c.ref_window ? 240 * ((L + 241) / 242) : L;
    p->g.nak = c.spline_end == MEMD_SPLINE_NOT_A_KNOT;
    p->g.mirror = c.boundary == MEMD_BOUNDARY_MIRROR;
    if (c.solve_window < 0) {
        p->S = p->g.cap;
        p->Ss = p->g.cap;
        p->H = -1;
        p->Sf = p->g.cap;
        p->Hf = -1;
    } else {
        // halo lengths: the truncation error decays by <= 1/2 (solve) and
        // <= 1/12 (pivots: u l / (2 (l + u) - l cp)^2 with cp <= 1/2) per
        // knot; FP64 and double-float need ~1e-15 (double-float pivots: 16
        // rows, 12^-16 = 5e-18)
        const bool wide = f64 || c.precision == MEMD_PREC_MIXED;
        p->S = tu.solve_segment ? tu.solve_segment : 256;
        p->Ss = tu.solve_min_segment ? tu.solve_min_segment : std::min(64, p->S);
        p->H = c.solve_window > 0 ? (int)c.solve_window : (f64 ? 48 : (wide ? 32 : 24));
        // short factorisation segments (the pivot recurrence is latency-bound),
        // except for FP64, whose longer halo would dominate
        p->Sf = tu.factor_segment ? tu.factor_segment : (f64 ? 64 : 16);
        p->Hf = f64 ? 40 : (wide ? 16 : 20);
    }
    // in place (when memory limits the directions per pass): the solution
    // overwrites the eliminated right-hand side row by row (same warp, read
    // first); the halo rows a warp reads from the next segment are copied
    // aside by the forward sweep, so segments must be at least a halo long.
    // Not for one record with not-a-knot ends, whose backward sweep writes the
    // last row from another segment's warp (batched runs set their ends after
    // the sweep).
    const bool inplace_ok = (p->H < 0 || p->Ss >= p->H) && !(p->g.nak && !p->batched);
    p->Kc = (c.dir_chunk > 0) ? std::min<int>((int)c.dir_chunk, K) : K;
    bool want_inplace = tu.solve_layout == 1 && inplace_ok;
    if (c.dir_chunk <= 0 && tu.solve_layout == 0) {
        // automatic: as many directions per pass as the free memory allows,
        // with separate right-hand-side and solution arrays while all of them
        // fit (the faster layout), solving in place when that fits more
        const bool cum_cfg = c.precision == MEMD_PREC_MIXED && c.stop_mode == MEMD_STOP_FIXED &&
                             c.boundary == MEMD_BOUNDARY_REFERENCE && c.mean_eval != 1;
        const int want = std::min(K, kc_limit);
        const int fit_sep = directions_that_fit(c, p->g, p->real_bytes, p->xbytes, p->tbytes, cum_cfg, false);
        if (fit_sep >= want || !inplace_ok) {
            p->Kc = std::max(1, std::min(want, fit_sep));
        } else {
            const int fit_inp = directions_that_fit(c, p->g, p->real_bytes, p->xbytes, p->tbytes, cum_cfg, true);
            p->Kc = std::max(1, std::min(want, std::max(fit_sep, fit_inp)));
            want_inplace = fit_inp > fit_sep;
        }
    } else if (c.dir_chunk <= 0) {  // layout fixed by the tuning: the directions that fit with it
        const bool cum_cfg = c.precision == MEMD_PREC_MIXED && c.stop_mode == MEMD_STOP_FIXED &&
                             c.boundary == MEMD_BOUNDARY_REFERENCE && c.mean_eval != 1;
        const int fit = directions_that_fit(c, p->g, p->real_bytes, p->xbytes, p->tbytes, cum_cfg, want_inplace);
        p->Kc = std::max(1, std::min({K, fit, kc_limit}));
    }
    p->Kc = std::min(p->Kc, 1024);
    *kc_used = p->Kc;
    p->nchunks = (K + p->Kc - 1) / p->Kc;
    p->GS = 32;  // solve: one warp per (envelope, direction, segment, 32 channels)
    p->ngroups = (C + 31) / 32;
    {
        // the factorisation and substitution kernels index their threads in 32 bits
        const double nfac = 2.0 * p->Kc * (double)((p->g.cap + p->Sf - 1) / p->Sf);
        const double nsol = 2.0 * p->Kc * (double)solve_segments_max(p->g.cap, p->S, p->Ss, p->H) * p->ngroups * 32.0;
        if (nfac >= 2147483648.0 || nsol >= 2147483648.0) {
            delete p;
            return set_error(MEMD_ERR_UNSUPPORTED, "plan: a factorisation or substitution launch would exceed 2^31 "
                                                   "threads (fewer directions per chunk or longer segments)");
        }
    }
    // FP64 evaluation tile: G channels x T samples, enough CTAs to fill the GPU
    p->evalG = std::min(32, std::max(4, next_pow2(C)));
    {
        const int NR = 256 / p->evalG;
        const int groups = (C + p->evalG - 1) / p->evalG;
        int best = -1, bestT = 0;
        const int spts[3] = {2, 4, 8};
        for (int i = 0; i < 3; ++i) {
            const int T = NR * spts[i];
            if (T % 32 != 0 || T > 512) continue;
            const long ctas = (long)((L + T - 1) / T) * groups;
            if (best < 0) { best = spts[i]; bestT = T; }
            if (ctas >= 608) { best = spts[i]; bestT = T; }
        }
        p->evalSPT = best;
        p->evalT = bestT;
    }
    // FP32 evaluation tile: G channel lanes x 32 samples per lane; the
    // double-float (mixed) tile keeps half the samples per lane in registers
    if (c.precision == MEMD_PREC_MIXED) {
        p->ewG = std::min(16, std::max(4, next_pow2(C)));
        p->ewSPL = 16;
    } else {
        p->ewG = p->evalG;
        p->ewSPL = 32;
    }
    p->egroups = (C + (f64 ? p->evalG : p->ewG) - 1) / (f64 ? p->evalG : p->ewG);
    // mean envelope: impulse accumulation for the mixed form in fixed mode
    // (mean_eval 0 = automatic, 1 = direct evaluation, 2 = impulse accumulation)
    if (c.mean_eval < 0 || c.mean_eval > 2) {
        delete p;
        return set_error(MEMD_ERR_INVALID, "plan: mean_eval must be 0, 1 or 2");
    }
    const bool cum_ok = c.precision == MEMD_PREC_MIXED && c.stop_mode == MEMD_STOP_FIXED &&
                        c.boundary == MEMD_BOUNDARY_REFERENCE;
    if (c.mean_eval == 2 && !cum_ok) {
        delete p;
        return set_error(MEMD_ERR_UNSUPPORTED,
                         "plan: impulse-accumulation mean needs the mixed form in fixed mode with the reference boundary");
    }
    p->cum = cum_ok && c.mean_eval != 1;
    p->cumG = C >= 32 ? 32 : (C > 8 ? 16 : 8);
    const size_t rb = (size_t)p->real_bytes;
    if (c.precision == MEMD_PREC_MIXED)
        p->proj_smem = 4 * ((size_t)(kProjTN + 2) * (C + 1) + 2 * (size_t)kProjTK * C + (size_t)kProjTK * (kProjTN + 2) + C + kProjTK);
    else
        p->proj_smem = rb * ((size_t)(kProjTN + 2) * (C + 1) + (size_t)kProjTK * C + (size_t)kProjTK * (kProjTN + 2));
    const size_t CL = (size_t)C * L;
    const size_t Kc = (size_t)p->Kc;
    memd_status st = MEMD_OK;
#define ALLOC(ptr, bytes)                                              \
    do {                                                               \
        if (st == MEMD_OK) st = dev_alloc(p, (void**)&(ptr), (bytes)); \
    } while (0)
    ALLOC(p->X, (size_t)p->xbytes * CL);
    if (p->cum) ALLOC(p->Xb, (size_t)p->xbytes * CL);
    ALLOC(p->run, (size_t)p->xbytes * CL);
    ALLOC(p->dir, 8 * (size_t)K * C);
    if (p->nchunks > 1) ALLOC(p->acc, rb * CL);
    ALLOC(p->imf, (size_t)p->tbytes * CL * (size_t)c.num_imfs);
    ALLOC(p->bits, sizeof(uint32_t) * 2 * Kc * p->g.W);
    ALLOC(p->wpref, sizeof(int) * 2 * Kc * (p->g.W + 1));
    ALLOC(p->knots, sizeof(int) * 2 * Kc * p->g.cap);
    ALLOC(p->cnt, sizeof(int) * 2 * (size_t)K);
    if (p->g.mirror) ALLOC(p->mir, sizeof(int) * kMirWords * (size_t)K);
    const size_t nch_max = (size_t)(p->g.W + kCompactChunk - 1) / kCompactChunk;
    ALLOC(p->csh.ctot, sizeof(int) * 2 * Kc * nch_max);
    ALLOC(p->csh.hacc, sizeof(unsigned long long) * 2 * Kc);
    ALLOC(p->csh.arrive, sizeof(int) * 2 * Kc);
    ALLOC(p->fac, rb * 4 * 2 * Kc * p->g.cap);
    if (!p->cum) ALLOC(p->yv, rb * 2 * Kc * p->g.cap * C);
    else ALLOC(p->yend, rb * 2 * Kc * (size_t)std::max<int64_t>(1, c.max_epochs) * 2 * C);  // [2][Kc][epochs][2][C]
    ALLOC(p->sv, rb * 2 * Kc * p->g.cap * C);
    p->inplace = want_inplace;
    p->hsegs = p->H > 0 ? (int)solve_segments_max(p->g.cap, p->S, p->Ss, p->H) : 0;
    if (p->inplace) {
        p->dbuf = p->sv;
        if (p->H > 0) ALLOC(p->hz, rb * 2 * Kc * (size_t)p->hsegs * p->H * C);
    } else {
        ALLOC(p->dbuf, rb * 2 * Kc * p->g.cap * C);
    }
    // longest knot gap: a record (epoch) length; mirrored knots reach 2L - 2
    const int Lh = p->batched ? std::max(p->Lrec, kEpochAlign) : (p->g.mirror ? 2 * L : L);
    ALLOC(p->rtab, rb * (size_t)(Lh + 1));
    if (p->cum) {
        ALLOC(p->rtab3, sizeof(dd) * (size_t)(Lh + 1));
        ALLOC(p->bnd, sizeof(unsigned) * 4 * (size_t)C);
        ALLOC(p->cumcfg, sizeof(int) * 4);
        ALLOC(p->cumsh.kq, sizeof(unsigned long long) * 35 * (size_t)p->g.W * C);
        ALLOC(p->cumsh.anc, sizeof(unsigned long long) * 4 * (size_t)p->g.W * C);
        ALLOC(p->cumsh.arrive, sizeof(int) * (size_t)p->g.W * ((C + 7) / 8));
    }
    if (c.stop_mode == MEMD_STOP_CRITERION) {
        ALLOC(p->M, rb * CL);
        ALLOC(p->part, rb * (size_t)p->egroups * Kc * L);
        ALLOC(p->amp, rb * (size_t)L);
        if (p->batched) ALLOC(p->recstop, sizeof(RecStop) * (size_t)c.max_epochs);
    }
    if (p->batched) {
        const size_t me = (size_t)c.max_epochs;
        ALLOC(p->ep_dev, sizeof(int) * (4 * me + 1 + (size_t)p->g.W));
        ALLOC(p->ep_yoff, sizeof(long long) * me);
        ALLOC(p->ep.cnt, sizeof(int) * 2 * (size_t)K * me);
    }
    // mixed form: the tensor-core projection's tf32 splits
    p->Cp = (C + kTcKB - 1) / kTcKB * kTcKB;
    p->tc = c.precision == MEMD_PREC_MIXED && c.projection == 0;
    if (p->tc) {
        // directions per tile: 64 by default (more, narrower tiles keep more
        // CTAs in flight; the kernel is latency-bound, not tensor-bound)
        p->tc_nt = std::max(16, (std::min(p->Kc, tu.proj_tile_n ? tu.proj_tile_n : 64) + 15) / 16 * 16);
        ALLOC(p->xbig, sizeof(float) * (size_t)L * p->Cp);
        ALLOC(p->xsmall, sizeof(float) * (size_t)L * p->Cp);
        ALLOC(p->dbig, sizeof(float) * (size_t)K * p->Cp);
        ALLOC(p->dsmall, sizeof(float) * (size_t)K * p->Cp);
    }
    p->squeue = tu.solve_queue == 1;
    p->cum_ctas = tu.mean_ctas ? tu.mean_ctas : 2048;
    if (p->squeue) {
        ALLOC(p->sq.pref, sizeof(int) * (2 * Kc + 1));
        ALLOC(p->sq.total, sizeof(int));
        ALLOC(p->sq.ticket, sizeof(int) * 2);
    }
    ALLOC(p->st, sizeof(RunState));
    ALLOC(p->coord_bad, sizeof(int));
#undef ALLOC
    if (st != MEMD_OK) {
        memd_plan_destroy(p);
        return st;
    }
    if (p->tc) {
        const bool mok = make_tile_map(&p->maps.xb, p->xbig, (uint64_t)p->Cp, (uint64_t)L, (uint32_t)kTcRows) &&
                         make_tile_map(&p->maps.xs, p->xsmall, (uint64_t)p->Cp, (uint64_t)L, (uint32_t)kTcRows) &&
                         make_tile_map(&p->maps.db, p->dbig, (uint64_t)p->Cp, (uint64_t)K, (uint32_t)p->tc_nt) &&
                         make_tile_map(&p->maps.ds, p->dsmall, (uint64_t)p->Cp, (uint64_t)K, (uint32_t)p->tc_nt);
        if (!mok) {
            memd_plan_destroy(p);
            return set_error(MEMD_ERR_CUDA, "plan: TMA descriptors (cuTensorMapEncodeTiled) could not be made");
        }
    }
    {
        int dev = 0;
        cudaGetDevice(&dev);
        p->sms = 0;
        cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, dev);
        if (p->sms < 1) p->sms = 1;
    }
    cudaError_t e = cudaMallocHost((void**)&p->host_flag, sizeof(int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&p->e0);
    if (e == cudaSuccess) e = cudaEventCreate(&p->e1);
    if (e == cudaSuccess) {
        if (c.precision == MEMD_PREC_F64) e = set_attrs<MEMD_PREC_F64>(p);
        else if (c.precision == MEMD_PREC_F32) e = set_attrs<MEMD_PREC_F32>(p);
        else e = set_attrs<MEMD_PREC_MIXED>(p);
    }
    if (e == cudaSuccess) {
        // reciprocal table 1/h, h = 0..L (h = 0 unused)
        double* r64 = nullptr;
        float* r32 = nullptr;
        dd* rdd = nullptr;
        e = cudaMalloc((void**)&r64, sizeof(double) * (size_t)(Lh + 1));
        if (e == cudaSuccess) e = cudaMalloc((void**)&r32, sizeof(float) * (size_t)(Lh + 1));
        if (e == cudaSuccess) e = cudaMalloc((void**)&rdd, sizeof(dd) * (size_t)(Lh + 1));
        if (e == cudaSuccess) {
            k_fill_reciprocals<<<256, 256>>>(r64, r32, rdd, (dd*)p->rtab3, Lh + 1);
            const void* src = f64 ? (void*)r64 : (c.precision == MEMD_PREC_MIXED ? (void*)rdd : (void*)r32);
            e = cudaMemcpy(p->rtab, src, rb * (size_t)(Lh + 1), cudaMemcpyDeviceToDevice);
        }
        cudaFree(r64);
        cudaFree(r32);
        cudaFree(rdd);
    }
    if (e == cudaSuccess) e = cudaMemset(p->csh.hacc, 0, sizeof(unsigned long long) * 2 * (size_t)p->Kc);
    if (e == cudaSuccess) e = cudaMemset(p->csh.arrive, 0, sizeof(int) * 2 * (size_t)p->Kc);
    if (e == cudaSuccess && p->cum) {
        e = cudaMemset(p->cumsh.kq, 0, sizeof(unsigned long long) * 35 * (size_t)p->g.W * C);
        if (e == cudaSuccess) e = cudaMemset(p->cumsh.anc, 0, sizeof(unsigned long long) * 4 * (size_t)p->g.W * C);
        if (e == cudaSuccess) e = cudaMemset(p->cumsh.arrive, 0, sizeof(int) * (size_t)p->g.W * ((C + 7) / 8));
        if (e == cudaSuccess) e = cudaMemset(p->cumcfg, 0, sizeof(int) * 4);
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        memd_plan_destroy(p);
        return set_cuda_error("plan: setup", e);
    }
    *out = p;
    return MEMD_OK;
}
}  // namespace memd

memd_status memd_plan_set_trace(memd_plan* p, memd_trace_entry* host_trace)
{
    using namespace memd;
    if (!p) return set_error(MEMD_ERR_INVALID, "trace: null plan");
    if (p->exec) {
        cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
    }
    p->trace_host = host_trace;
    if (!host_trace) {
        p->trace_dev = nullptr;
        return MEMD_OK;
    }
    p->trace_n = (size_t)p->cfg.num_imfs * (size_t)(p->cfg.max_iter + 1) * (size_t)p->g.K * 2;
    if (!p->trace_dev) {
        memd_status st = dev_alloc(p, (void**)&p->trace_dev, sizeof(memd_trace_entry) * p->trace_n);
        if (st != MEMD_OK) return st;
    }
    cudaMemset(p->trace_dev, 0, sizeof(memd_trace_entry) * p->trace_n);
    return MEMD_OK;
}

memd_status memd_run_f64(memd_plan* plan, const int32_t* d_x, const double* d_y, const double* d_dir,
                         double* d_imfs, void* stream, memd_stats* stats)
{
    using namespace memd;
    if (!plan) return set_error(MEMD_ERR_INVALID, "run: null plan");
    if (!d_y || !d_dir || !d_imfs) return set_error(MEMD_ERR_INVALID, "run: null pointer");
    if (plan->prec != MEMD_PREC_F64) return set_error(MEMD_ERR_PRECISION, "run_f64: plan is not FP64");
    if (plan->batched) return set_error(MEMD_ERR_UNSUPPORTED, "run_f64: batched plan: use memd_run_batched_f64");
    return run_impl<MEMD_PREC_F64>(plan, d_x, d_y, d_dir, d_imfs, stream, stats);
}

memd_status memd_run_f32(memd_plan* plan, const int32_t* d_x, const float* d_y, const float* d_dir,
                         float* d_imfs, void* stream, memd_stats* stats)
{
    using namespace memd;
    if (!plan) return set_error(MEMD_ERR_INVALID, "run: null plan");
    if (!d_y || !d_dir || !d_imfs) return set_error(MEMD_ERR_INVALID, "run: null pointer");
    if (plan->batched) return set_error(MEMD_ERR_UNSUPPORTED, "run_f32: batched plan: use memd_run_batched_f32");
    if (plan->prec == MEMD_PREC_F32) return run_impl<MEMD_PREC_F32>(plan, d_x, d_y, d_dir, d_imfs, stream, stats);
    if (plan->prec == MEMD_PREC_MIXED) return run_impl<MEMD_PREC_MIXED>(plan, d_x, d_y, d_dir, d_imfs, stream, stats);
    return set_error(MEMD_ERR_PRECISION, "run_f32: plan is FP64");
}

memd_status memd_profile_f64(memd_plan* plan, const double* d_y, const double* d_dir, double* d_imfs,
                             void* stream, memd_profile* prof)
{
    using namespace memd;
    if (!plan || !d_y || !d_dir || !d_imfs || !prof) return set_error(MEMD_ERR_INVALID, "profile: null argument");
    if (plan->prec != MEMD_PREC_F64) return set_error(MEMD_ERR_PRECISION, "profile_f64: plan is not FP64");
    if (plan->batched) return set_error(MEMD_ERR_UNSUPPORTED, "profile: batched plans are not profiled");
    return profile_impl<MEMD_PREC_F64>(plan, d_y, d_dir, d_imfs, stream, prof);
}

memd_status memd_profile_f32(memd_plan* plan, const float* d_y, const float* d_dir, float* d_imfs,
                             void* stream, memd_profile* prof)
{
    using namespace memd;
    if (!plan || !d_y || !d_dir || !d_imfs || !prof) return set_error(MEMD_ERR_INVALID, "profile: null argument");
    if (plan->batched) return set_error(MEMD_ERR_UNSUPPORTED, "profile: batched plans are not profiled");
    if (plan->prec == MEMD_PREC_F32) return profile_impl<MEMD_PREC_F32>(plan, d_y, d_dir, d_imfs, stream, prof);
    if (plan->prec == MEMD_PREC_MIXED) return profile_impl<MEMD_PREC_MIXED>(plan, d_y, d_dir, d_imfs, stream, prof);
    return set_error(MEMD_ERR_PRECISION, "profile_f32: plan is FP64");
}

memd_status memd_profile_batched_f64(memd_plan* plan, int32_t n_epochs, const int64_t* lengths,
                                     const int64_t* offsets, const double* d_y, const double* d_dir, double* d_imfs,
                                     void* stream, memd_profile* prof)
{
    using namespace memd;
    if (!plan || !prof) return set_error(MEMD_ERR_INVALID, "profile_batched: null argument");
    if (plan->prec != MEMD_PREC_F64) return set_error(MEMD_ERR_PRECISION, "profile_batched_f64: plan is not FP64");
    return profile_batched_impl<MEMD_PREC_F64>(plan, n_epochs, lengths, offsets, d_y, d_dir, d_imfs, stream, prof);
}

memd_status memd_profile_batched_f32(memd_plan* plan, int32_t n_epochs, const int64_t* lengths,
                                     const int64_t* offsets, const float* d_y, const float* d_dir, float* d_imfs,
                                     void* stream, memd_profile* prof)
{
    using namespace memd;
    if (!plan || !prof) return set_error(MEMD_ERR_INVALID, "profile_batched: null argument");
    if (plan->prec == MEMD_PREC_MIXED)
        return profile_batched_impl<MEMD_PREC_MIXED>(plan, n_epochs, lengths, offsets, d_y, d_dir, d_imfs, stream,
                                                     prof);
    if (plan->prec == MEMD_PREC_F32)
        return profile_batched_impl<MEMD_PREC_F32>(plan, n_epochs, lengths, offsets, d_y, d_dir, d_imfs, stream,
                                                   prof);
    return set_error(MEMD_ERR_PRECISION, "profile_batched_f32: plan is FP64");
}

memd_status memd_batched_counts(const memd_plan* plan, int32_t n_epochs, int32_t* n_imfs, int32_t* sifts)
{
    using namespace memd;
    if (!plan || !n_imfs) return set_error(MEMD_ERR_INVALID, "batched_counts: null argument");
    if (!plan->batched || plan->cfg.stop_mode != MEMD_STOP_CRITERION || !plan->recstop)
        return set_error(MEMD_ERR_UNSUPPORTED, "batched_counts: the plan is not a batched stop-mode plan");
    if (n_epochs < 1 || n_epochs > plan->ep.n)
        return set_error(MEMD_ERR_INVALID, "batched_counts: n_epochs exceeds the last run's epochs");
    std::vector<RecStop> h((size_t)n_epochs);
    const cudaError_t e = cudaMemcpy(h.data(), plan->recstop, sizeof(RecStop) * h.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return set_cuda_error("batched_counts: read", e);
    for (int i = 0; i < n_epochs; ++i) {
        n_imfs[i] = h[i].n_imfs;
        if (sifts)
            for (int j = 0; j < 64; ++j) sifts[64 * (size_t)i + j] = j < h[i].n_imfs ? h[i].sifts[j] : 0;
    }
    return MEMD_OK;
}

memd_status memd_run_batched_f64(memd_plan* plan, int32_t n_epochs, const int64_t* lengths, const int64_t* offsets,
                                 const double* d_y, const double* d_dir, double* d_imfs, void* stream, memd_stats* stats)
{
    using namespace memd;
    if (!plan) return set_error(MEMD_ERR_INVALID, "run_batched: null plan");
    if (plan->prec != MEMD_PREC_F64) return set_error(MEMD_ERR_PRECISION, "run_batched_f64: plan is not FP64");
    return run_batched_impl<MEMD_PREC_F64>(plan, n_epochs, lengths, offsets, d_y, d_dir, d_imfs, stream, stats);
}

memd_status memd_run_batched_f32(memd_plan* plan, int32_t n_epochs, const int64_t* lengths, const int64_t* offsets,
                                 const float* d_y, const float* d_dir, float* d_imfs, void* stream, memd_stats* stats)
{
    using namespace memd;
    if (!plan) return set_error(MEMD_ERR_INVALID, "run_batched: null plan");
    if (plan->prec == MEMD_PREC_MIXED)
        return run_batched_impl<MEMD_PREC_MIXED>(plan, n_epochs, lengths, offsets, d_y, d_dir, d_imfs, stream, stats);
    if (plan->prec == MEMD_PREC_F32)
        return run_batched_impl<MEMD_PREC_F32>(plan, n_epochs, lengths, offsets, d_y, d_dir, d_imfs, stream, stats);
    return set_error(MEMD_ERR_PRECISION, "run_batched_f32: plan is FP64");
}

}  // extern "C"
