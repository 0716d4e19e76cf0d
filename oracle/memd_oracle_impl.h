/*
 * memd_oracle_impl.h -- body of the CPU oracle, included twice by memd_oracle.c
 * (REAL = double -> *_f64, REAL = float -> *_f32).
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C restatement of the reference
 * MEMD hot path (memReducedEpochs_dev.cu, "REF" below).  Only tests/,
 * __graft_entry__.smoke() and the cpu_baseline leg of bench.py load it, as the
 * checker and the timed CPU baseline; the product path never calls it.
 *
 * Arithmetic follows the reference kernels expression by expression.  The file
 * is compiled with -ffp-contract=off; the places where nvcc contracts a
 * multiply-add in the reference are written as explicit fma() calls.
 */

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SUFFIX)

/* Cubic-spline envelope of one channel through the knots (pos[0..E-1],
 * val[0..E-1], ascending; mirrored knots may lie outside 0..L-1) evaluated
 * at n = 0..L-1.
 *   - natural end conditions                        REF:704-736 tridiagonal_setup
 *     or, nak != 0 and E >= 4, not-a-knot (third derivative continuous at
 *     x_1 and x_{E-2}; the intent of the unused tridiagonal_setup_nak,
 *     REF:738-773): c_0 is eliminated with row 1, which becomes
 *       (h0 + 2 h1) c_1 + (h1 - h0) c_2 = h1 r_1 / (h0 + h1),
 *     and c_{E-1} with row E-2 (a = h_{E-3}, b = h_{E-2}):
 *       (a - b) c_{E-3} + (2a + b) c_{E-2} = a r_{E-2} / (a + b);
 *     rows 0 and E-1 stay identity rows and c_0, c_{E-1} follow from the
 *     not-a-knot conditions after the solve (REF:738-773 keeps c_0 in row 0
 *     instead, whose pivot h0^2 - h1^2 vanishes at equal spacings)
 *   - tridiagonal solve (Thomas, stands in for the
 *     closed cusparse<t>gtsv2_nopivot)              REF:1227-1241
 *   - coefficients                                  REF:775-793 spline_coefficients
 *   - evaluation, interval x_i < n <= x_{i+1}
 *     (n = 0 uses interval 0), Horner with the
 *     three FMAs nvcc forms                         REF:795-830 interpolate
 * ws must hold 5*E REALs. */
static void FN(envelope_)(const int32_t* pos, const REAL* val, int64_t E, int64_t L,
                          REAL* out, REAL* ws, int nak)
{
    REAL* lo = ws;
    REAL* mid = ws + E;
    REAL* up = ws + 2 * E;
    REAL* rhs = ws + 3 * E;
    REAL* cp = ws + 4 * E;
    int64_t i;
    /* REF:714-735: rows 0 and E-1 are identity with rhs 0; interior rows use
     * integer spacings, the rhs divides real differences by integer spacings. */
    for (i = 0; i < E; ++i) {
        if (i == 0 || i == E - 1) {
            mid[i] = 1; up[i] = 0; lo[i] = 0; rhs[i] = 0;
        } else {
            int32_t hl = pos[i] - pos[i - 1];
            int32_t hr = pos[i + 1] - pos[i];
            mid[i] = (REAL)(2 * (hl + hr));
            up[i] = (REAL)hr;
            lo[i] = (REAL)hl;
            rhs[i] = (REAL)3 * ((val[i + 1] - val[i]) / (REAL)hr - (val[i] - val[i - 1]) / (REAL)hl);
            if (nak && E >= 4 && i == 1) {
                mid[i] = (REAL)(hl + 2 * hr);
                up[i] = (REAL)(hr - hl);
                lo[i] = 0;
                rhs[i] = rhs[i] * (REAL)hr / (REAL)(hl + hr);
            } else if (nak && E >= 4 && i == E - 2) {
                mid[i] = (REAL)(2 * hl + hr);
                up[i] = 0;
                lo[i] = (REAL)(hl - hr);
                rhs[i] = rhs[i] * (REAL)hl / (REAL)(hl + hr);
            }
        }
    }
    /* Thomas elimination without pivoting; the system is strictly diagonally
     * dominant (|2(hl+hr)| > hl + hr) so no pivoting is needed. */
    cp[0] = up[0] / mid[0];
    rhs[0] = rhs[0] / mid[0];
    for (i = 1; i < E; ++i) {
        REAL w = mid[i] - lo[i] * cp[i - 1];
        cp[i] = up[i] / w;
        rhs[i] = (rhs[i] - lo[i] * rhs[i - 1]) / w;
    }
    for (i = E - 2; i >= 0; --i) rhs[i] = rhs[i] - cp[i] * rhs[i + 1];
    /* rhs now holds the solution s_i (the reference's d_solutionGtsv). */
    if (nak && E >= 4) {
        /* d_0 = d_1:       c_0 = c_1 + (h0 / h1) (c_1 - c_2)
         * d_{E-3} = d_{E-2}: c_{E-1} = c_{E-2} + (b / a) (c_{E-2} - c_{E-3}) */
        int32_t h0 = pos[1] - pos[0], h1 = pos[2] - pos[1];
        int32_t a = pos[E - 2] - pos[E - 3], b = pos[E - 1] - pos[E - 2];
        rhs[0] = rhs[1] + (rhs[1] - rhs[2]) * (REAL)h0 / (REAL)h1;
        rhs[E - 1] = rhs[E - 2] + (rhs[E - 2] - rhs[E - 3]) * (REAL)b / (REAL)a;
    }
    {
        int64_t iv = 0;
        REAL a = val[0], b = 0, c = 0, d = 0;
        int32_t x0 = pos[0];
        int have = 0;
        int64_t n;
        for (n = 0; n < L; ++n) {
            int64_t want = iv;
            while (want + 1 < E - 1 && pos[want + 1] < n) ++want;
            if (!have || want != iv) {
                /* REF:785-791 */
                REAL h = (REAL)(pos[want + 1] - pos[want]);
                REAL s0 = rhs[want], s1 = rhs[want + 1];
                iv = want;
                a = val[want];
                b = (val[want + 1] - val[want]) / h - h * ((REAL)2 * s0 + s1) / (REAL)3;
                d = (s1 - s0) / ((REAL)3 * h);
                c = s0;
                x0 = pos[want];
                have = 1;
            }
            {
                REAL t = (REAL)(int32_t)((int32_t)n - x0);
                out[n] = FMA(FMA(FMA(d, t, c), t, b), t, a);
            }
        }
    }
}

/* Knot values of channel row y at the knots, with the reference's end-point
 * clamp (REF:447-486 setBoundaryMax, REF:545-584 setBoundaryMin): when the
 * direction has E >= 6 knots (exclusive scan at L-1 > 4), each end knot value
 * is replaced by the linear extrapolation of its two inner neighbours if that
 * lies above (maxima) / below (minima) it. */
static void FN(knot_values_)(const int32_t* pos, int64_t E, const REAL* y, int is_max, REAL* val)
{
    int64_t i;
    for (i = 0; i < E; ++i) val[i] = y[pos[i]];
    if (E - 1 > 4) {
        REAL slope, t;
        slope = (val[2] - val[1]) / (REAL)(pos[2] - pos[1]);
        t = FMA(-slope, (REAL)(pos[1] - pos[0]), val[1]);
        if (is_max ? (t > val[0]) : (t < val[0])) val[0] = t;
        slope = (val[E - 2] - val[E - 3]) / (REAL)(pos[E - 2] - pos[E - 3]);
        t = FMA(slope, (REAL)(pos[E - 1] - pos[E - 2]), val[E - 2]);
        if (is_max ? (t > val[E - 1]) : (t < val[E - 1])) val[E - 1] = t;
    }
}

/* Directions (REF:934-1072, MEX:900-978).  primes == NULL selects the
 * standalone convention (prime table {-K, 2, 3, 5, ...}, REF:1033-1046);
 * otherwise primes[0..C-1] are used as the MEX entry receives them.
 * Output: dir[k*C + c]. */
int FN(oracle_directions_)(int64_t C, int64_t K, const int32_t* primes, REAL* dir)
{
    int32_t* p;
    REAL* seq;
    REAL* tht;
    int64_t k, c, j;
    if (C < 1 || K < 1 || !dir) return -1;
    p = (int32_t*)malloc(sizeof(int32_t) * (size_t)C);
    seq = (REAL*)malloc(sizeof(REAL) * (size_t)C);
    tht = (REAL*)malloc(sizeof(REAL) * (size_t)(C > 1 ? C - 1 : 1));
    if (!p || !seq || !tht) { free(p); free(seq); free(tht); return -2; }
    if (primes) {
        for (c = 0; c < C; ++c) p[c] = primes[c];
    } else {
        oracle_prime_table(C, K, p);
    }
    for (k = 0; k < K; ++k) {
        /* REF:996-1003 GenerateHammSeq: coordinate 0 = (k + 1.5) / (-p[0])
         * computed in double; coordinates c >= 1 = float radical inverse of
         * k+1 in base p[c]. */
        seq[0] = (REAL)(((double)(uint32_t)k + 1.5) / (double)(-p[0]));
        for (c = 1; c < C; ++c) seq[c] = (REAL)oracle_radical_inverse(p[c], (uint32_t)(k + 1));
        /* REF:948-990 Sequence2Vector */
        for (c = 0; c < C; ++c) seq[c] = FMA((REAL)2, seq[c], (REAL)-1);
        for (c = 0; c < C - 1; ++c) {
            REAL tem = 0;
            for (j = C - 1; j > c; --j) tem = FMA(seq[j], seq[j], tem);
            tht[c] = ATAN2(SQRT(tem), seq[c]);
        }
        for (c = 0; c < C; ++c) {
            REAL v = 1;
            if (c > 0) for (j = 0; j < c; ++j) v = v * SIN(tht[j]);
            dir[k * C + c] = v;
        }
        for (c = 0; c < C - 1; ++c) dir[k * C + c] = dir[k * C + c] * COS(tht[c]);
    }
    free(p); free(seq); free(tht);
    return 0;
}

/* Extrema of one projected direction (REF:77-141 find_extrema_shfl_max/min,
 * compaction REF:384-445): strict local maxima (minima) at interior samples
 * n <= cov, plus both end samples when ends != 0.  Returns the count. */
static int64_t FN(extrema_)(const REAL* P, int64_t L, int64_t cov, int is_max, int32_t* pos, int ends)
{
    int64_t E = 0, n, last = L - 2;
    if (cov < last) last = cov;
    if (ends) pos[E++] = 0;
    for (n = 1; n <= last; ++n) {
        REAL v = P[n], l = P[n - 1], r = P[n + 1];
        if (is_max ? (v > l && v > r) : (v < l && v < r)) pos[E++] = (int32_t)n;
    }
    if (ends && L - 1 > 0) pos[E++] = (int32_t)(L - 1);
    return E;
}

/* Mirrored end knots (boundary mode 1; no reference counterpart, the method
 * of Rilling, Flandrin & Goncalves 2003 with two extrema per end).  Inputs:
 * the interior maxima imx[0..nx-1] and minima imn[0..nn-1] (ascending,
 * nx >= 2, nn >= 2) of the projection P.
 * Left end: when the first extremum is a maximum and P[0] lies above the
 * first minimum, the knots mirror about that maximum (the next two maxima and
 * the first two minima); otherwise sample 0 acts as a minimum: the knots
 * mirror about sample 0 (the first two maxima; the first minimum and sample 0
 * itself).  The case of a leading minimum is the same with the roles
 * exchanged.  If a list's outermost mirrored knot then falls inside the
 * record (position > 0), the symmetry point moves to sample 0 and the list
 * of the symmetry extremum's kind becomes its first two extrema.  The right
 * end is the mirror image of this rule. */
static void FN(mirror_)(const REAL* P, int64_t L, const int32_t* imx, int64_t nx, const int32_t* imn, int64_t nn,
                        oracle_mirror* m)
{
    const int32_t last = (int32_t)(L - 1);
    if (imx[0] < imn[0]) {
        if (P[0] > P[imn[0]]) {
            m->nl[0] = oracle_take_rev(imx, nx, 1, 3, m->lsrc[0]);
            m->nl[1] = oracle_take_rev(imn, nn, 0, 2, m->lsrc[1]);
            m->lsym = imx[0];
        } else {
            m->nl[0] = oracle_take_rev(imx, nx, 0, 2, m->lsrc[0]);
            m->nl[1] = oracle_take_rev(imn, nn, 0, 1, m->lsrc[1]);
            m->lsrc[1][m->nl[1]++] = 0;
            m->lsym = 0;
        }
    } else {
        if (P[0] < P[imx[0]]) {
            m->nl[0] = oracle_take_rev(imx, nx, 0, 2, m->lsrc[0]);
            m->nl[1] = oracle_take_rev(imn, nn, 1, 3, m->lsrc[1]);
            m->lsym = imn[0];
        } else {
            m->nl[0] = oracle_take_rev(imx, nx, 0, 1, m->lsrc[0]);
            m->lsrc[0][m->nl[0]++] = 0;
            m->nl[1] = oracle_take_rev(imn, nn, 0, 2, m->lsrc[1]);
            m->lsym = 0;
        }
    }
    if (2 * m->lsym - m->lsrc[0][0] > 0 || 2 * m->lsym - m->lsrc[1][0] > 0) {
        if (m->lsym == imx[0]) m->nl[0] = oracle_take_rev(imx, nx, 0, 2, m->lsrc[0]);
        else m->nl[1] = oracle_take_rev(imn, nn, 0, 2, m->lsrc[1]);
        m->lsym = 0;
    }
    if (imx[nx - 1] < imn[nn - 1]) {
        if (P[last] < P[imx[nx - 1]]) {
            m->nr[0] = oracle_take_rev(imx, nx, nx - 2, nx, m->rsrc[0]);
            m->nr[1] = oracle_take_rev(imn, nn, nn - 3, nn - 1, m->rsrc[1]);
            m->rsym = imn[nn - 1];
        } else {
            m->rsrc[0][0] = last;
            m->nr[0] = 1 + oracle_take_rev(imx, nx, nx - 1, nx, m->rsrc[0] + 1);
            m->nr[1] = oracle_take_rev(imn, nn, nn - 2, nn, m->rsrc[1]);
            m->rsym = last;
        }
    } else {
        if (P[last] > P[imn[nn - 1]]) {
            m->nr[0] = oracle_take_rev(imx, nx, nx - 3, nx - 1, m->rsrc[0]);
            m->nr[1] = oracle_take_rev(imn, nn, nn - 2, nn, m->rsrc[1]);
            m->rsym = imx[nx - 1];
        } else {
            m->nr[0] = oracle_take_rev(imx, nx, nx - 2, nx, m->rsrc[0]);
            m->rsrc[1][0] = last;
            m->nr[1] = 1 + oracle_take_rev(imn, nn, nn - 1, nn, m->rsrc[1] + 1);
            m->rsym = last;
        }
    }
    if (2 * m->rsym - m->rsrc[0][m->nr[0] - 1] < last || 2 * m->rsym - m->rsrc[1][m->nr[1] - 1] < last) {
        if (m->rsym == imx[nx - 1]) m->nr[0] = oracle_take_rev(imx, nx, nx - 2, nx, m->rsrc[0]);
        else m->nr[1] = oracle_take_rev(imn, nn, nn - 2, nn, m->rsrc[1]);
        m->rsym = last;
    }
}

typedef struct {
    int32_t* pos[2];   /* per direction: knot positions (max, min), K*(L+4) each */
    int32_t* src[2];   /* per direction: the sample each knot takes its value from */
    int64_t* cnt;      /* K*2 knots */
    int64_t* nint;     /* K*2 interior extrema */
    REAL* P;           /* K*L projections */
    REAL* acc;         /* C*L running sum of mean envelopes */
    REAL* amp;         /* L (stop mode) */
    REAL* env;         /* per thread: 2*L envelopes + 2*L knot values + 5*L solver */
    int nthreads;
} FN(oracle_ws_);

/* One evaluation of the mean envelope of `cur` (C x L channel-major):
 *   projection (REF:1182, summed over c in order with fma),
 *   extrema + knots per direction,
 *   envelopes of every channel for each qualified direction
 *   (E_max > 3 && E_min > 3, REF:840, 856),
 *   acc[c,n] = sum_k (U + L)/2 in direction order (REF:846-864).
 * Returns Q, the number of qualified directions.  In stop mode also fills
 * amp[n] = sum_k ||U_k(n) - L_k(n)||_2 / 2 over the qualified directions. */
static int64_t FN(mean_envelope_)(int64_t C, int64_t L, int64_t K, const REAL* cur, const REAL* dir,
                                  const oracle_opts* o, FN(oracle_ws_)* w, int want_amp,
                                  memd_trace_entry* trace)
{
    int64_t cov = o->ref_window ? oracle_window_cover(L) : L;
    int64_t k, q = 0;
    int64_t i;
    const int64_t LS = L + 4;  /* knot stride per direction */
    for (i = 0; i < C * L; ++i) w->acc[i] = 0;
    if (want_amp) for (i = 0; i < L; ++i) w->amp[i] = 0;
#pragma omp parallel for schedule(static) num_threads(w->nthreads)
    for (k = 0; k < K; ++k) {
        REAL* P = w->P + k * L;
        int64_t n, c;
        for (n = 0; n < L; ++n) {
            REAL s = 0;
            for (c = 0; c < C; ++c) s = FMA(cur[c * L + n], dir[k * C + c], s);
            P[n] = s;
        }
        if (!o->boundary) {
            w->cnt[2 * k + 0] = FN(extrema_)(P, L, cov, 1, w->pos[0] + k * LS, 1);
            w->cnt[2 * k + 1] = FN(extrema_)(P, L, cov, 0, w->pos[1] + k * LS, 1);
            w->nint[2 * k + 0] = w->cnt[2 * k + 0] - 2;
            w->nint[2 * k + 1] = w->cnt[2 * k + 1] - 2;
        } else {
            /* interior extrema, then (qualifying directions) the mirrored
             * knots: [left mirrored | interior | right mirrored] */
            oracle_mirror m;
            int32_t* sx = w->src[0] + k * LS;
            int32_t* sn = w->src[1] + k * LS;
            int64_t ni[2];
            int e;
            ni[0] = FN(extrema_)(P, L, cov, 1, sx + 2, 0);
            ni[1] = FN(extrema_)(P, L, cov, 0, sn + 2, 0);
            memset(&m, 0, sizeof(m));
            if (ni[0] >= 2 && ni[1] >= 2) FN(mirror_)(P, L, sx + 2, ni[0], sn + 2, ni[1], &m);
            for (e = 0; e < 2; ++e) {
                int32_t* sr = e ? sn : sx;
                int32_t* ps = w->pos[e] + k * LS;
                int64_t j, E;
                memmove(sr + m.nl[e], sr + 2, sizeof(int32_t) * (size_t)ni[e]);
                for (j = 0; j < m.nl[e]; ++j) sr[j] = m.lsrc[e][j];
                for (j = 0; j < m.nr[e]; ++j) sr[m.nl[e] + ni[e] + j] = m.rsrc[e][j];
                E = m.nl[e] + ni[e] + m.nr[e];
                for (j = 0; j < E; ++j) {
                    int32_t v = sr[j];
                    if (j < m.nl[e]) v = 2 * m.lsym - v;
                    else if (j >= m.nl[e] + ni[e]) v = 2 * m.rsym - v;
                    ps[j] = v;
                }
                w->cnt[2 * k + e] = E;
                w->nint[2 * k + e] = ni[e];
            }
        }
    }
    if (trace) {
        for (k = 0; k < K; ++k) {
            int e;
            for (e = 0; e < 2; ++e) {
                trace[2 * k + e].count = (int32_t)w->cnt[2 * k + e];
                trace[2 * k + e].flags = 0;
                trace[2 * k + e].hash = oracle_knot_hash(w->pos[e] + k * LS, w->cnt[2 * k + e]);
            }
        }
    }
    for (k = 0; k < K; ++k) {
        int64_t Em = w->cnt[2 * k], En = w->cnt[2 * k + 1];
        int64_t c;
        /* REF:840, 856: E_max > 3 && E_min > 3 with both end samples counted,
         * i.e. at least two interior maxima and two interior minima (the same
         * rule in the mirror mode, which then always finds its extrema) */
        if (!(w->nint[2 * k] >= 2 && w->nint[2 * k + 1] >= 2)) continue;
        ++q;
#pragma omp parallel for schedule(static) num_threads(w->nthreads)
        for (c = 0; c < C; ++c) {
            int tid = 0;
            REAL *U, *Lo, *vm, *vn, *sws;
            int64_t n;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
            U = w->env + (size_t)tid * 9 * LS;
            Lo = U + LS; vm = Lo + LS; vn = vm + LS; sws = vn + LS;
            if (!o->boundary) {
                FN(knot_values_)(w->pos[0] + k * LS, Em, cur + c * L, 1, vm);
                FN(knot_values_)(w->pos[1] + k * LS, En, cur + c * L, 0, vn);
            } else {
                const int32_t* sx = w->src[0] + k * LS;
                const int32_t* sn = w->src[1] + k * LS;
                for (n = 0; n < Em; ++n) vm[n] = cur[c * L + sx[n]];
                for (n = 0; n < En; ++n) vn[n] = cur[c * L + sn[n]];
            }
            FN(envelope_)(w->pos[0] + k * LS, vm, Em, L, U, sws, o->spline_end);
            FN(envelope_)(w->pos[1] + k * LS, vn, En, L, Lo, sws, o->spline_end);
            for (n = 0; n < L; ++n) {
                /* REF:842 mean = (U + L) / 2.0, exact halving */
                w->acc[c * L + n] = w->acc[c * L + n] + (U[n] + Lo[n]) * (REAL)0.5;
                if (want_amp) {
                    REAL dlt = U[n] - Lo[n];
                    U[n] = dlt * dlt; /* reuse U as squared spread of channel c */
                }
            }
            if (want_amp) {
                /* stash the squared spread for the channel-norm reduction */
                REAL* dst = w->P + (size_t)c * L; /* P is free after the extrema pass */
                for (n = 0; n < L; ++n) dst[n] = U[n];
            }
        }
        if (want_amp) {
            int64_t n;
            /* requires K >= C so that P (K*L) can hold C rows: ensured by the caller */
            for (n = 0; n < L; ++n) {
                REAL s2 = 0;
                int64_t cc;
                for (cc = 0; cc < C; ++cc) s2 = s2 + w->P[cc * L + n];
                w->amp[n] = w->amp[n] + SQRT(s2) * (REAL)0.5;
            }
        }
    }
    return q;
}

int FN(oracle_memd_)(int64_t C, int64_t L, int64_t K, int64_t nimf, int64_t max_iter,
                     const REAL* y, const REAL* dir, REAL* imfs, const oracle_opts* opts,
                     memd_trace_entry* trace, int32_t* sifts_out, int32_t* nimf_out)
{
    oracle_opts o;
    FN(oracle_ws_) w;
    REAL *cur, *run;
    int64_t i, j, n, imf_done = 0;
    int stop_mode;
    int64_t prows;
    if (C < 1 || L < 4 || K < 1 || nimf < 1 || max_iter < 0 || !y || !dir || !imfs) return -1;
    if (opts) o = *opts; else oracle_default_opts(&o);
    stop_mode = o.stop_mode;
    memset(&w, 0, sizeof(w));
    w.nthreads = o.nthreads > 0 ? o.nthreads : 1;
    prows = K > C ? K : C;
    w.pos[0] = (int32_t*)malloc(sizeof(int32_t) * (size_t)(K * (L + 4)));
    w.pos[1] = (int32_t*)malloc(sizeof(int32_t) * (size_t)(K * (L + 4)));
    w.src[0] = (int32_t*)malloc(sizeof(int32_t) * (size_t)(K * (L + 4)));
    w.src[1] = (int32_t*)malloc(sizeof(int32_t) * (size_t)(K * (L + 4)));
    w.cnt = (int64_t*)malloc(sizeof(int64_t) * (size_t)(2 * K));
    w.nint = (int64_t*)malloc(sizeof(int64_t) * (size_t)(2 * K));
    w.P = (REAL*)malloc(sizeof(REAL) * (size_t)(prows * L));
    w.acc = (REAL*)malloc(sizeof(REAL) * (size_t)(C * L));
    w.amp = (REAL*)malloc(sizeof(REAL) * (size_t)L);
    w.env = (REAL*)malloc(sizeof(REAL) * (size_t)(9 * (L + 4)) * (size_t)w.nthreads);
    cur = (REAL*)malloc(sizeof(REAL) * (size_t)(C * L));
    run = (REAL*)malloc(sizeof(REAL) * (size_t)(C * L));
    if (!w.pos[0] || !w.pos[1] || !w.src[0] || !w.src[1] || !w.cnt || !w.nint || !w.P || !w.acc || !w.amp ||
        !w.env || !cur || !run) {
        free(w.pos[0]); free(w.pos[1]); free(w.src[0]); free(w.src[1]); free(w.cnt); free(w.nint);
        free(w.P); free(w.acc); free(w.amp); free(w.env);
        free(cur); free(run);
        return -2;
    }
    for (i = 0; i < C * L; ++i) run[i] = y[i];           /* REF:1174 */
    if (sifts_out) for (i = 0; i < nimf; ++i) sifts_out[i] = 0;
    for (i = 0; i + 1 < nimf; ++i) {                    /* REF:1176 */
        memd_trace_entry* trow = trace ? trace + (size_t)i * (size_t)(max_iter + 1) * (size_t)(2 * K) : NULL;
        for (n = 0; n < C * L; ++n) cur[n] = run[n];     /* REF:1178 */
        if (!stop_mode) {
            for (j = 0; j < max_iter; ++j) {             /* REF:1179 */
                int64_t q = FN(mean_envelope_)(C, L, K, cur, dir, &o, &w, 0,
                                              trow ? trow + (size_t)j * (size_t)(2 * K) : NULL);
                REAL qq = (REAL)q;
                /* REF:862: current -= value / numCompDir (0/0 = NaN when q == 0) */
                for (n = 0; n < C * L; ++n) cur[n] = cur[n] - w.acc[n] / qq;
            }
            if (sifts_out) sifts_out[i] = (int32_t)max_iter;
        } else {
            /* Stop mode (Rilling et al. 2003 criterion as used by Rehman &
             * Mandic 2010 for MEMD).  Before each IMF: stop the decomposition
             * when every direction of the residual has fewer than 3 interior
             * extrema.  Each sifting pass computes the mean envelope m(n) and
             * the mean half-spread a(n); sigma(n) = ||m(n)||_2 / a(n); sifting
             * stops when the fraction of samples with sigma > sd is at most tol
             * and no sample has sigma > sd2, or when no direction qualifies, or
             * after max_iter updates. */
            int64_t nbit = 0;
            int64_t ev = 0;
            for (;;) {
                int64_t q = FN(mean_envelope_)(C, L, K, cur, dir, &o, &w, 1,
                                              (trow && ev <= max_iter) ? trow + (size_t)ev * (size_t)(2 * K) : NULL);
                int stop = 0;
                ++ev;
                if (nbit == 0) {
                    int64_t k, few = 1;
                    for (k = 0; k < K; ++k)
                        if (w.nint[2 * k] + w.nint[2 * k + 1] >= 3) few = 0;
                    if (few) { imf_done = 1; break; }
                }
                if (q == 0) {
                    stop = 1;
                } else {
                    REAL qq = (REAL)q;
                    int64_t over1 = 0, over2 = 0;
                    for (n = 0; n < L; ++n) {
                        REAL m2 = 0, a, sig;
                        int64_t c;
                        for (c = 0; c < C; ++c) {
                            REAL mv = w.acc[c * L + n] / qq;
                            m2 = m2 + mv * mv;
                        }
                        a = w.amp[n] / qq;
                        sig = (a > 0) ? SQRT(m2) / a : (m2 > 0 ? (REAL)INFINITY : (REAL)0);
                        if (sig > (REAL)o.sd) ++over1;
                        if (sig > (REAL)o.sd2) ++over2;
                    }
                    stop = !(((double)over1 / (double)L > o.tol) || over2 > 0);
                }
                if (stop) break;
                {
                    REAL qq = (REAL)q;
                    for (n = 0; n < C * L; ++n) cur[n] = cur[n] - w.acc[n] / qq;
                }
                ++nbit;
                if (nbit >= max_iter) break;
            }
            if (imf_done) break;
            if (sifts_out) sifts_out[i] = (int32_t)nbit;
        }
        for (n = 0; n < C * L; ++n) imfs[i * C * L + n] = cur[n];          /* REF:1328 */
        for (n = 0; n < C * L; ++n) run[n] = run[n] - cur[n];               /* REF:866-874 */
    }
    if (nimf_out) *nimf_out = (int32_t)i;
    for (j = i; j + 1 < nimf; ++j)
        for (n = 0; n < C * L; ++n) imfs[j * C * L + n] = 0;
    for (n = 0; n < C * L; ++n) imfs[(nimf - 1) * C * L + n] = run[n];   /* REF:1338 */
    free(w.pos[0]); free(w.pos[1]); free(w.src[0]); free(w.src[1]); free(w.cnt); free(w.nint);
    free(w.P); free(w.acc); free(w.amp); free(w.env);
    free(cur); free(run);
    return 0;
}

#undef FN
#undef CAT
#undef CAT2
