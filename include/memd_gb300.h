/*
 * memd_gb300.h -- C ABI of the GB300 MEMD engine (libmemd_gb300.so).
 *
 * Multivariate empirical mode decomposition (Rehman & Mandic 2010) of a
 * C-channel record of L samples with K projection directions, on one GPU.
 * The entry points replace the reference's host interface for this path
 * (reference files memReducedEpochs_dev.cu and memdMatlabCuda.cu):
 *
 *   memd_plan_create / memd_run_f64 / memd_run_f32 / memd_plan_destroy
 *       replace  template<coord_t, real_t> double memd(size_t SignalDim,
 *                size_t SignalLength, size_t NumDirVector, size_t num_IMFs,
 *                size_t max_iter, coord_t* d_x, real_t* d_y,
 *                real_t* d_DirectionVectors, real_t* d_IMFs)
 *                memReducedEpochs_dev.cu:1074-1368, which allocates and frees
 *                its workspace on every call; here the workspace belongs to
 *                the plan and a run allocates nothing.
 *   memd_directions_f64 / memd_directions_f32
 *       replace  template<T> void GenerateDirectionVector(size_t SignalDim,
 *                size_t NumDirVector, T* d_DirectionVector)
 *                memReducedEpochs_dev.cu:1029-1072 (primes == NULL), and the
 *                in-line direction set of the MEX entry
 *                memdMatlabCuda.cu:1131-1152 (primes = the caller's table).
 *   memd_run_batched_f64 / memd_run_batched_f32
 *       no single reference counterpart: the reference decomposes one record
 *       per memd() call (runBenchmark, memReducedEpochs_dev.cu:1370-1464,
 *       loops over calls); this decomposes many records of equal C and
 *       uneven L in one pass.
 *
 * Data layout (identical to the reference):
 *   d_y     C x L, channel-major (y[c*L + n])
 *   d_dir   K x C, direction-major (dir[k*C + c])
 *   d_imfs  num_imfs x C x L; slot i < num_imfs-1 is IMF i, the last slot
 *           holds the residual.
 *   d_x     the sample coordinate 0..L-1 (int32); the reference compares the
 *           sample index with these values (memReducedEpochs_dev.cu:812-826),
 *           so any other content is rejected (MEMD_ERR_COORD) when d_x is
 *           given; pass NULL to skip the check.
 *
 * All calls are stream-ordered on the given stream (cudaStream_t passed as
 * void*, NULL = legacy default stream) and return a memd_status.  A plan is
 * not thread-safe: one run at a time per plan.
 */
#ifndef MEMD_GB300_H
#define MEMD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    MEMD_OK = 0,
    MEMD_ERR_INVALID = 1,      /* bad size / argument / null pointer */
    MEMD_ERR_CUDA = 2,         /* a CUDA runtime call failed; see memd_last_error() */
    MEMD_ERR_NOMEM = 3,        /* device or host allocation failed at plan creation */
    MEMD_ERR_COORD = 4,        /* d_x is not 0..L-1 */
    MEMD_ERR_PRECISION = 5,    /* run_f64 on a plan built for f32 or the reverse */
    MEMD_ERR_UNSUPPORTED = 6   /* combination not built (e.g. stop mode + batched) */
} memd_status;

typedef enum {
    MEMD_PREC_F64 = 0,     /* plain FP64 end to end (the drop-in / parity path) */
    MEMD_PREC_F32 = 1,     /* FP32 end to end (the reference's own precision) */
    MEMD_PREC_MIXED = 2    /* FP32 storage and splines, FP64 where it matters */
} memd_precision;

typedef enum {
    MEMD_STOP_FIXED = 0,   /* exactly max_iter sifts per IMF (the reference) */
    MEMD_STOP_CRITERION = 1/* Rilling et al. 2003 thresholds (sd, sd2, tol) */
} memd_stop_mode;

typedef enum {
    MEMD_SPLINE_NATURAL = 0,   /* zero second derivative at the end knots: the
                                  reference's tridiagonal_setup
                                  (memReducedEpochs_dev.cu:704-736) */
    MEMD_SPLINE_NOT_A_KNOT = 1 /* continuous third derivative at the second and
                                  second-to-last knots (MATLAB spline, as the
                                  published MEMD uses it; the reference's unused
                                  tridiagonal_setup_nak, :738-773); envelopes
                                  with fewer than 4 knots stay natural */
} memd_spline_end;

typedef enum {
    MEMD_BOUNDARY_REFERENCE = 0, /* both end samples are knots of both
                                    envelopes, their values clamped by linear
                                    extrapolation (memReducedEpochs_dev.cu:98-103,
                                    447-486, 545-584) */
    MEMD_BOUNDARY_MIRROR = 1     /* no forced end knots: two extrema per end
                                    mirrored about the outermost extremum or the
                                    end sample (Rilling, Flandrin & Goncalves
                                    2003); no reference counterpart */
} memd_boundary;

typedef struct {
    int64_t channels;      /* C >= 1 */
    int64_t length;        /* L >= 4 (batched: maximum epoch length) */
    int64_t directions;    /* K >= 1 */
    int64_t num_imfs;      /* output slots >= 1 (IMFs + residual) */
    int64_t max_iter;      /* sifts per IMF (fixed) or cap (criterion) */
    int32_t precision;     /* memd_precision */
    int32_t stop_mode;     /* memd_stop_mode */
    double stop_sd;        /* theta1, default 0.075 */
    double stop_sd2;       /* theta2, default 0.75 */
    double stop_tol;       /* alpha, default 0.075 */
    int32_t ref_window;    /* 1: extrema tested only at interior samples
                              n <= 240*ceil(L/242), as the reference's launch
                              (memReducedEpochs_dev.cu:1191-1195) does; 0: all */
    int32_t dir_chunk;     /* directions per pass (0 = automatic: as many of the K as fit in 60% of
                              the device's free memory at plan creation; a plan whose allocation
                              still fails is made again with half as many) */
    int32_t solve_window;  /* tridiagonal halo in knots (0 = default; <0 = exact) */
    int32_t max_epochs;    /* batched runs: epochs per call (0 = single record) */
    int32_t mean_eval;     /* mean envelope: 0 = automatic (impulse accumulation
                              for the mixed form in fixed mode with the
                              reference boundary, otherwise direct evaluation),
                              1 = direct evaluation of every envelope,
                              2 = impulse accumulation (mixed form, fixed mode,
                              reference boundary only) */
    int32_t spline_end;    /* memd_spline_end: end conditions of the envelope
                              splines */
    int32_t boundary;      /* memd_boundary: how the envelopes are closed at the
                              record's ends */
    int32_t projection;    /* mixed form: 0 = automatic (tensor cores: 3xTF32
                              tcgen05.mma with TMA-staged tiles), 1 = CUDA
                              cores (FP32 fma); both certify every extremum
                              test against the FP64 projection */
    int64_t reserved[2];
} memd_config;

typedef struct {
    int32_t n_imfs;        /* IMFs extracted (excluding the residual slot) */
    int32_t flags;         /* MEMD_FLAG_* bits seen during the run */
    double elapsed_ms;     /* device time of the decomposition (CUDA events) */
    int64_t launches;      /* kernels this library launched for the run */
    int32_t sifts[64];     /* sifts per IMF (first 64 IMFs) */
    int32_t refined;       /* mixed precision: extremum tests re-decided in
                              double-float because the FP32 margin was within
                              the projection's error bound */
    int32_t reserved;
} memd_stats;

/* Per-stage device time of one eagerly launched decomposition (every kernel
 * bracketed by CUDA events on the run's stream). */
enum {
    MEMD_STAGE_PROJECT = 0,   /* projection + extrema bitmasks */
    MEMD_STAGE_COMPACT = 1,   /* knot lists, counts, end-point clamp */
    MEMD_STAGE_FACTOR = 2,    /* tridiagonal factorisation */
    MEMD_STAGE_SOLVE = 3,     /* tridiagonal substitution */
    MEMD_STAGE_EVAL = 4,      /* envelope evaluation + mean + update */
    MEMD_STAGE_OTHER = 5,     /* layout transforms, IMF bookkeeping, stop tests */
    MEMD_STAGES = 8
};
typedef struct {
    double ms[MEMD_STAGES];
    int64_t launches[MEMD_STAGES];
} memd_profile;

#define MEMD_FLAG_NO_QUALIFIED_DIRECTION 1  /* a sift had no direction with >3 maxima
                                               and >3 minima: the reference's 0/0 NaN */
#define MEMD_FLAG_KNOT_OVERFLOW 2           /* internal knot capacity exceeded */
#define MEMD_FLAG_DEVICE_TIMEOUT 4          /* a bounded device-side wait ran out (a kernel
                                               gave up on a copy or product it issued);
                                               the run's results are not valid */
#define MEMD_FLAG_CHECK_FAILED 8            /* bounds-checked build (libmemd_gb300_checked.so):
                                               an index check failed and its access was
                                               skipped */

/* One entry per (IMF, sift, direction, envelope) when a trace buffer is
 * given: the extrema index set of that projected direction. */
typedef struct {
    int32_t count;   /* knots, both end samples included */
    int32_t flags;
    uint64_t hash;   /* sum over the knot sample indices n of splitmix64(n), mod 2^64 */
} memd_trace_entry;

typedef struct memd_plan memd_plan;

/* Launch shapes of a plan's kernels (what the autotuner chooses; 0 = the
 * default).  None of them changes what is computed beyond rounding: segment
 * lengths only move where the windowed tridiagonal sweeps start (their
 * truncation is below the arithmetic's precision), the rest are grid
 * shapes and work distribution. */
typedef struct {
    int32_t solve_segment;      /* longest substitution segment in knots, a power of two in [32, 1024] (256) */
    int32_t solve_min_segment;  /* shortest substitution segment, a power of two in [16, solve_segment] (64) */
    int32_t factor_segment;     /* factorisation rows per thread, 4 .. 256 (FP64 64, otherwise 16) */
    int32_t solve_queue;        /* substitution work: 1 = device work queue pulled by a persistent grid,
                                   2 or 0 = one warp per possible segment (the default) */
    int32_t mean_ctas;          /* impulse-accumulation mean: CTAs the split of spans over CTAs aims for,
                                   128 .. 65536 (2048) */
    int32_t proj_tile_n;        /* tensor-core projection: directions per tile, a multiple of 16 in
                                   [16, 256] (64) */
    int32_t solve_layout;       /* substitution storage: 1 = the solution overwrites the eliminated
                                   right-hand side (one array, halo rows copied aside), 2 = separate
                                   arrays, 0 = separate while every direction of the pass fits in the
                                   memory budget, in place when that fits more (same results) */
    int32_t reserved[9];
} memd_tuning;

void memd_default_config(memd_config* cfg);

/* Allocates every device buffer the runs need (nothing is allocated later). */
memd_status memd_plan_create(const memd_config* cfg, memd_plan** plan);
/* memd_plan_create with explicit launch shapes (tuning may be NULL: defaults). */
memd_status memd_plan_create_tuned(const memd_config* cfg, const memd_tuning* tuning, memd_plan** plan);
/* The launch shapes a plan uses (the defaults filled in). */
memd_status memd_plan_get_tuning(const memd_plan* plan, memd_tuning* tuning);
memd_status memd_plan_destroy(memd_plan* plan);
/* Device bytes held by the plan. */
size_t memd_plan_workspace_bytes(const memd_plan* plan);

/* Optional per-sift trace: trace has num_imfs*(max_iter+1)*K*2 entries in
 * [imf][sift][direction][max=0|min=1] order (host or device memory reachable
 * by the GPU is not required: the plan copies into its own buffer and the
 * entries are written back to this host array at the end of the run). */
memd_status memd_plan_set_trace(memd_plan* plan, memd_trace_entry* host_trace);

/* Full decomposition.  stats may be NULL; when given the call waits for the
 * run to finish and fills it. */
memd_status memd_run_f64(memd_plan* plan, const int32_t* d_x, const double* d_y,
                         const double* d_dir, double* d_imfs, void* stream,
                         memd_stats* stats);
memd_status memd_run_f32(memd_plan* plan, const int32_t* d_x, const float* d_y,
                         const float* d_dir, float* d_imfs, void* stream,
                         memd_stats* stats);

/* Same decomposition as memd_run_*, launched kernel by kernel without the
 * graph, each kernel timed with CUDA events; for per-kernel roofline figures.
 * Synchronises the stream. */
memd_status memd_profile_f64(memd_plan* plan, const double* d_y, const double* d_dir, double* d_imfs,
                             void* stream, memd_profile* prof);
memd_status memd_profile_f32(memd_plan* plan, const float* d_y, const float* d_dir, float* d_imfs,
                             void* stream, memd_profile* prof);

/* Batched: n_epochs records of C channels; epoch e has length lengths[e]
 * (host array, 4 <= lengths[e] <= cfg.length) and its samples at
 * d_y + offsets[e] (C x lengths[e], channel-major); its IMFs go to
 * d_imfs + num_imfs*offsets[e] (num_imfs x C x lengths[e]).  offsets is a
 * host array of n_epochs entries in units of elements. */
memd_status memd_run_batched_f64(memd_plan* plan, int32_t n_epochs, const int64_t* lengths,
                                 const int64_t* offsets, const double* d_y, const double* d_dir,
                                 double* d_imfs, void* stream, memd_stats* stats);
memd_status memd_run_batched_f32(memd_plan* plan, int32_t n_epochs, const int64_t* lengths,
                                 const int64_t* offsets, const float* d_y, const float* d_dir,
                                 float* d_imfs, void* stream, memd_stats* stats);
/* Stop mode, batched: after a run of n_epochs epochs (and after its stream
 * has been synchronised), the IMFs of each epoch (n_imfs[e]; its unused
 * slots are zero, the residual is in the last slot, as for one record) and,
 * if sifts is not NULL, the sifts of its IMFs (sifts[64 e + i], i < 64).
 * Reads device memory synchronously. */
memd_status memd_batched_counts(const memd_plan* plan, int32_t n_epochs, int32_t* n_imfs, int32_t* sifts);

/* Batched run launched kernel by kernel without the graph, each kernel timed
 * (per-stage figures, as memd_profile_*).  Synchronises the stream.
 * memd_profile_batched_f32 takes FP32 and mixed-form plans. */
memd_status memd_profile_batched_f64(memd_plan* plan, int32_t n_epochs, const int64_t* lengths,
                                     const int64_t* offsets, const double* d_y, const double* d_dir,
                                     double* d_imfs, void* stream, memd_profile* prof);
memd_status memd_profile_batched_f32(memd_plan* plan, int32_t n_epochs, const int64_t* lengths,
                                     const int64_t* offsets, const float* d_y, const float* d_dir,
                                     float* d_imfs, void* stream, memd_profile* prof);

/* Direction set on the device.  primes == NULL: the standalone convention
 * (table {-K, 2, 3, 5, ...}); otherwise primes[0..C-1] (host memory) as the
 * MEX entry receives them.  d_dir: K x C. */
memd_status memd_directions_f64(int64_t channels, int64_t directions, const int32_t* primes,
                                double* d_dir, void* stream);
memd_status memd_directions_f32(int64_t channels, int64_t directions, const int32_t* primes,
                                float* d_dir, void* stream);

/* Same direction set as memd_directions_f64, for callers that must not
 * allocate device memory: a MATLAB MEX function whose GPU buffers have to come
 * from MATLAB's own allocator, a real-time acquisition loop that cannot
 * afford the device-wide synchronisation cudaMalloc/cudaFree may cause, or an
 * application that hands out all device memory from one arena it owns.  It
 * allocates nothing: the prime table lives in a static device array of 4096
 * entries, so channels > 4096 is rejected (MEMD_ERR_INVALID).  The array is
 * shared by all calls and keeps the last call's table: calls whose copies and
 * kernels overlap on the GPU (for example on two streams) race and must be
 * ordered by the caller.  Each call looks up the array's address in the
 * current context (cudaGetSymbolAddress, which allocates nothing), so a device
 * reset between calls is harmless.  The table is copied from host stack
 * memory with cudaMemcpyAsync on the given stream.
 * No counterpart in the reference (which always allocates its tables). */
memd_status memd_directions_noalloc_f64(int64_t channels, int64_t directions, const int32_t* primes,
                                        double* d_dir, void* stream);

/* Diagnostic: sustained fma throughput (flop/s, fma = 2 flops) of the current
 * GPU for MEMD_PREC_F64 or MEMD_PREC_F32 arithmetic; the denominator of the
 * CUDA-core roofline figures.  No reference counterpart. */
memd_status memd_diag_fma_rate(int32_t precision, double* flops_per_s);

/* Diagnostic of the device-side failure detection: one CTA waits on an
 * mbarrier that nothing completes, with the bounded wait the tensor-core
 * kernels use (limit max_clocks, 1 .. 2^32); *flags receives the run-state
 * bits the kernel set (MEMD_FLAG_DEVICE_TIMEOUT when the wait gave up).  No
 * reference counterpart (the reference has no device waits). */
memd_status memd_diag_wait_timeout(int64_t max_clocks, int32_t* flags);

/* Text of the last error on this thread. */
const char* memd_last_error(void);
/* Library version string. */
const char* memd_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MEMD_GB300_H */
