/*
 * memd_oracle.c -- CPU oracle for the MEMD hot path.
 *
 * TEST INFRASTRUCTURE ONLY: a C restatement of the reference algorithm
 * (memReducedEpochs_dev.cu, MEX variant memdMatlabCuda.cu) used as the
 * checker by tests/, __graft_entry__.smoke() and as the timed CPU baseline
 * ("port") by bench.py.  The CUDA library never links or calls it.
 *
 * Build: see oracle/build_oracle.py (gcc -O2 -fopenmp -ffp-contract=off -shared).
 *
 * Restated functions (reference file:line):
 *   directions       memReducedEpochs_dev.cu:934-1072 (MEX 900-978, 1131-1152)
 *   projection       memReducedEpochs_dev.cu:1182-1184 (cublasSgemm; summed in
 *                    channel order with fma here)
 *   extrema          memReducedEpochs_dev.cu:77-141, window quirk of the launch
 *                    at :1191-1195
 *   scan+compaction  memReducedEpochs_dev.cu:143-445 (a plain ordered walk)
 *   end-point clamp  memReducedEpochs_dev.cu:447-486, 545-584
 *   spline system    memReducedEpochs_dev.cu:704-736 (natural); the not-a-knot
 *                    option follows the intent of the unused
 *                    tridiagonal_setup_nak (memReducedEpochs_dev.cu:738-773),
 *                    with c_0 / c_{E-1} eliminated (no zero pivot at equal
 *                    spacings) and MATLAB spline's end conditions
 *   mirror option    no reference counterpart: mirrored extrema at both ends,
 *                    two per end (Rilling, Flandrin & Goncalves 2003)
 *   tridiagonal      memReducedEpochs_dev.cu:1227-1241 (Thomas instead of the
 *                    closed cusparse gtsv2_nopivot)
 *   coefficients     memReducedEpochs_dev.cu:775-793
 *   interpolation    memReducedEpochs_dev.cu:795-830
 *   mean / update    memReducedEpochs_dev.cu:832-874
 *   IMF loop         memReducedEpochs_dev.cu:1174-1338
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int32_t count;   /* knots of this direction/envelope, both end samples included */
    int32_t flags;
    uint64_t hash;   /* sum over knots n of splitmix64(n), mod 2^64 */
} memd_trace_entry;

typedef struct {
    int32_t ref_window;  /* 1: extrema only at interior n <= 240*ceil(L/242) (reference launch) */
    int32_t stop_mode;   /* 0: fixed max_iter sifts per IMF (reference); 1: stop criterion */
    double sd, sd2, tol; /* stop thresholds (theta1, theta2, alpha) */
    int32_t nthreads;
    int32_t spline_end;  /* 0: natural (reference); 1: not-a-knot (MATLAB spline) */
    int32_t boundary;    /* 0: forced end knots + clamp (reference); 1: mirrored extrema */
    int32_t reserved;
} oracle_opts;

void oracle_default_opts(oracle_opts* o)
{
    o->ref_window = 1;
    o->stop_mode = 0;
    o->sd = 0.075;
    o->sd2 = 0.75;
    o->tol = 0.075;
#ifdef _OPENMP
    o->nthreads = omp_get_max_threads();
#else
    o->nthreads = 1;
#endif
    o->spline_end = 0;
    o->boundary = 0;
    o->reserved = 0;
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Last interior sample the reference's extrema launch tests: blocks of 256
 * threads, ceil(L/242) blocks per direction, each warp covering 30 new
 * samples (REF:84-93, 1191-1193). */
int64_t oracle_window_cover(int64_t L)
{
    return 240 * ((L + 241) / 242);
}

static uint64_t oracle_splitmix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t oracle_knot_hash(const int32_t* pos, int64_t E)
{
    uint64_t h = 0;
    int64_t i;
    for (i = 0; i < E; ++i) h += oracle_splitmix64((uint64_t)(uint32_t)pos[i]);
    return h;
}

/* REF:1014-1046: table {-K, 2, 3, 5, 7, ...} of C entries. */
void oracle_prime_table(int64_t C, int64_t K, int32_t* p)
{
    int64_t cnt = 1;
    int32_t cand = 2;
    while (cnt < C) {
        int32_t d, composite = 0;
        for (d = 2; d <= cand / 2; ++d)
            if (cand % d == 0) { composite = 1; break; }
        if (!composite) p[cnt++] = cand;
        ++cand;
    }
    p[0] = -(int32_t)K;
}

/* REF:934-946: radical inverse, always in float.  nvcc contracts the
 * accumulation into an fma. */
float oracle_radical_inverse(int32_t base, uint32_t i)
{
    float digit, radical, inv;
    digit = radical = (float)(1.0 / (double)base);
    inv = 0.0f;
    while (i) {
        inv = fmaf(digit, (float)(i % (uint32_t)base), inv);
        digit *= radical;
        i /= (uint32_t)base;
    }
    return inv;
}

/* Mirrored end knots of one direction (boundary mode 1): for each envelope
 * (0 = maxima, 1 = minima) up to two source samples per end, listed in
 * ascending order of their mirrored position 2*sym - src. */
typedef struct {
    int32_t lsym, rsym;
    int32_t nl[2], nr[2];
    int32_t lsrc[2][2], rsrc[2][2];
} oracle_mirror;

/* out = a[to-1], a[to-2], ..., a[from] (from, to clamped to [0, n]); returns the count */
static int32_t oracle_take_rev(const int32_t* a, int64_t n, int64_t from, int64_t to, int32_t* out)
{
    int32_t c = 0;
    int64_t i;
    if (from < 0) from = 0;
    if (to > n) to = n;
    for (i = to - 1; i >= from; --i) out[c++] = a[i];
    return c;
}

/* ---- double instantiation ---- */
#define REAL double
#define SUFFIX f64
#define FMA fma
#define SQRT sqrt
#define ATAN2 atan2
#define SIN sin
#define COS cos
#include "memd_oracle_impl.h"
#undef REAL
#undef SUFFIX
#undef FMA
#undef SQRT
#undef ATAN2
#undef SIN
#undef COS

/* ---- float instantiation ---- */
#define REAL float
#define SUFFIX f32
#define FMA fmaf
#define SQRT sqrtf
#define ATAN2 atan2f
#define SIN sinf
#define COS cosf
#include "memd_oracle_impl.h"
#undef REAL
#undef SUFFIX
#undef FMA
#undef SQRT
#undef ATAN2
#undef SIN
#undef COS

/* Single envelope, exposed for unit tests (spline reproduces cubics etc.).
 * nak: 0 natural, 1 not-a-knot end conditions. */
int oracle_envelope_f64(const int32_t* pos, const double* val, int64_t E, int64_t L, double* out, int32_t nak)
{
    double* ws;
    if (E < 2 || L < 1) return -1;
    ws = (double*)malloc(sizeof(double) * (size_t)(5 * E));
    if (!ws) return -2;
    envelope_f64(pos, val, E, L, out, ws, nak);
    free(ws);
    return 0;
}

/* Mirrored end knots of one direction, exposed for unit tests: the source
 * samples of the left / right mirrored knots of each envelope (env 0 = maxima)
 * and the two symmetry samples.  out[0..1] = lsym, rsym; out[2..5] = counts
 * nl[0], nl[1], nr[0], nr[1]; out[6..13] = lsrc[env][j]; out[14..21] =
 * rsrc[env][j] (ascending mirrored position). */
int oracle_mirror_f64(const double* P, int64_t L, const int32_t* imax, int64_t nx, const int32_t* imin,
                      int64_t nn, int32_t* out)
{
    oracle_mirror m;
    int e, j;
    if (nx < 2 || nn < 2 || L < 4) return -1;
    mirror_f64(P, L, imax, nx, imin, nn, &m);
    out[0] = m.lsym; out[1] = m.rsym;
    out[2] = m.nl[0]; out[3] = m.nl[1]; out[4] = m.nr[0]; out[5] = m.nr[1];
    for (e = 0; e < 2; ++e)
        for (j = 0; j < 4; ++j) {
            out[6 + e * 4 + j] = j < 2 ? m.lsrc[e][j] : 0;
            out[14 + e * 4 + j] = j < 2 ? m.rsrc[e][j] : 0;
        }
    return 0;
}
