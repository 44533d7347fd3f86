/*
 * symeig_oracle.c -- CPU restatement of SymmetricEigenProblem.jl's eigensolver hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the tests, the smoke check and
 * bench.py's CPU-baseline leg call it; the product library (libsymeig.so) never links,
 * loads or calls it.
 *
 * What is restated (file:line in the reference project):
 *   givens_algorithm    LinearAlgebra.givensAlgorithm, called by get_rotation
 *                       (src/simple_givens.jl:20-23).  Julia's stdlib port of LAPACK 3.2
 *                       DLARTG: safmn2 = 2^-485 scaling loops, sign fix when |f|>|g| and c<0.
 *                       The Julia version is unpinned by the reference (no Manifest.toml);
 *                       the DLARTG-3.2 form is the one in the Julia releases that could run
 *                       the reference's SIMDPirates dependency.
 *   rmul semantics      rmul!(A, G::Rotation2) (src/simple_givens.jl:53-65):
 *                       col_i <- c*col_i + s*col_{i+1};  col_{i+1} <- -s*col_i + c*col_{i+1}.
 *   single_shift        single_shift! (src/bulge_chasing.jl:11-144).
 *   qr flush / qr       qr_algorithm! (src/bulge_chasing.jl:146-288), including
 *                       is_offdiagonal_small (:7-8), the deflation scan (:205-222), the layer
 *                       capacity rule (:226-230), the Wilkinson shift (:239-265), the
 *                       maxiter exit (:180-182) and the bulk flush (:282).
 *   apply (layer-major) The semantics of bulk_wave_order_2x2_rmul! (src/wave.jl:62-162):
 *                       its wave order applies rotation (i,L) after (i-1,L) and (i+1,L-1),
 *                       which for every matrix element is the same sequence of rotations as
 *                       "for L in 1:k, for i in 1:n-1: rmul!(A, G[i,L])".
 *   apply (wave)        The fused 2x2 wave order itself (src/wave.jl:62-162 with the
 *                       three kernels of src/bulk_givens.jl:4-279) and its row-slab
 *                       threading (src/wave.jl:36-60).  Used as the CPU baseline and to
 *                       check that wave order equals layer-major order.
 *
 * Canonical floating-point forms.  The reference evaluates single_shift! and the rotation
 * kernels under @fastmath, so its roundings depend on what LLVM contracts.  This file fixes
 * one contraction pattern and the CUDA kernels use the same one, which makes oracle and
 * device results comparable bit for bit:
 *   rotation of a pair (x, y):   x' = fma(c, x, s*y);   y' = fma(c, y, -(s*x))
 *   chase 2x2 updates:           u*a + v*b  ->  fma(u, a, v*b)  (first product fused)
 * Code outside @fastmath (givensAlgorithm, the Wilkinson shift, is_offdiagonal_small) is
 * plain IEEE with no contraction, as Julia compiles it.  Build with -ffp-contract=off.
 *
 * Parity status: the eigenvalues are pinned against LAPACK (the reference test's own check,
 * test/runtests.jl:10) and against the README residual magnitude (README.md:65-77).  The
 * (c,s) stream and Q bits have no golden vectors in the reference (Julia is not available
 * here); they are pinned against an independent pure-Python restatement with exactly
 * rounded FMAs (tests/golden/make_golden.py and its fixtures), not against the reference's
 * own execution.
 *
 *   apply (scaled)      The device's optional scaled ("fast Givens") form of the FP64 apply
 *                       (no reference counterpart), restated so that its results can be
 *                       checked bit for bit as well.
 *   qr multishift       The device's multishift chase (chase mode 3; no reference
 *                       counterpart): batches of sweeps with the trailing square's
 *                       eigenvalues as shifts, on the reference's deflation, capacity and
 *                       placement rules.  Checked by the reference's error bounds, and by the
 *                       reference's bits where no block takes a batch.
 */
#define _POSIX_C_SOURCE 200809L
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <time.h>

/* ------------------------------------------------------------------------------------ */
/* givensAlgorithm (LinearAlgebra, DLARTG 3.2 port); call site src/simple_givens.jl:21   */
/* ------------------------------------------------------------------------------------ */

/* Julia's max propagates NaN. */
static inline double jl_max(double a, double b) { return (a > b || a != a) ? a : b; }

void oracle_givens(double f, double g, double* c_out, double* s_out, double* r_out)
{
    const double safmn2 = 0x1p-485;   /* floatmin2(Float64) */
    const double safmx2 = 0x1p+485;
    double cs, sn, r;
    if (g == 0.0) {
        cs = 1.0; sn = 0.0; r = f;
    } else if (f == 0.0) {
        cs = 0.0; sn = 1.0; r = g;
    } else {
        double f1 = f, g1 = g;
        double scale = jl_max(fabs(f1), fabs(g1));
        if (scale >= safmx2) {
            int count = 0;
            do {
                ++count;
                f1 *= safmn2; g1 *= safmn2;
                scale = jl_max(fabs(f1), fabs(g1));
            } while (scale >= safmx2 && count < 20);
            r = sqrt(f1 * f1 + g1 * g1);
            cs = f1 / r; sn = g1 / r;
            for (int i = 0; i < count; ++i) r *= safmx2;
        } else if (scale <= safmn2) {
            int count = 0;
            do {
                ++count;
                f1 *= safmx2; g1 *= safmx2;
                scale = jl_max(fabs(f1), fabs(g1));
            } while (scale <= safmn2);
            r = sqrt(f1 * f1 + g1 * g1);
            cs = f1 / r; sn = g1 / r;
            for (int i = 0; i < count; ++i) r *= safmn2;
        } else {
            r = sqrt(f1 * f1 + g1 * g1);
            cs = f1 / r; sn = g1 / r;
        }
        if (fabs(f) > fabs(g) && cs < 0.0) { cs = -cs; sn = -sn; r = -r; }
    }
    *c_out = cs; *s_out = sn; *r_out = r;
}

/* ------------------------------------------------------------------------------------ */
/* Column rotations: rmul! semantics (src/simple_givens.jl:53-65)                        */
/* ------------------------------------------------------------------------------------ */

static inline void rot_f64(double* x, double* y, double c, double s)
{
    double a = *x, b = *y;
    double sb = s * b, sa = s * a;
    *x = fma(c, a, sb);
    *y = fma(c, b, -sa);
}

static inline void rot_f32(float* x, float* y, float c, float s)
{
    float a = *x, b = *y;
    float sb = s * b, sa = s * a;
    *x = fmaf(c, a, sb);
    *y = fmaf(c, b, -sa);
}

/* Scaled ("fast Givens") form of one pass of the device apply (the GB300 kernel's optional
 * form; no reference counterpart -- the reference applies (c,s) as rmul! does).  Columns
 * c0 .. c0+nloc-1 of Q carry scale factors d (1 at the start of the pass), Q = Qt diag(d).
 * Rotation (r, L), r = 0..nloc-2 local, L = 0..63 of the pass, in layer-major order:
 *   form 1 (|c| >= |s|): k = s/c,  A = k (d[r+1]/d[r]),  B = -(k (d[r]/d[r+1])),
 *                        d[r] = c d[r],  d[r+1] = c d[r+1]
 *   form 2 (|s| >  |c|): k = c/s,  A = k (d[r]/d[r+1]),  B = -(k (d[r+1]/d[r])),
 *                        d[r] = s d[r+1],  d[r+1] = -(s d[r])
 * and on every row
 *   (u, v) = form 2 ? (y, x) : (x, y);   x = fma(A, v, u);   y = fma(B, u, v).
 * Every d is an unevaluated sum hi + lo, updated by dd_mul (an exact product to about
 * 2^-106); A and B take the hi parts, each operation rounded once (divisions correctly
 * rounded).  Layers beyond the grid's (`layers`) are padding with A = B = +0, form 1 (the
 * kernel's zeroed table slots).  At the end of the pass column c is multiplied by the hi part
 * of d[c].  place (may be NULL): layer L of rotation i is (1, 0) unless L < place[i], as for
 * the canonical apply. */
typedef struct { double hi, lo; } dd_t;

static dd_t dd_mul(dd_t a, double m)
{
    const double p = a.hi * m;
    double e = fma(a.hi, m, -p);
    e = fma(a.lo, m, e);
    const double h = p + e;
    dd_t r = {h, e - (h - p)};
    return r;
}

static void scaled_coeffs(double c, double s, dd_t dr, dd_t dr1, double* A, double* B, int* f2,
                          dd_t* nr, dd_t* nr1)
{
    if (fabs(s) > fabs(c)) {
        const double k = c / s;
        *A = k * (dr.hi / dr1.hi);
        *B = -(k * (dr1.hi / dr.hi));
        *nr = dd_mul(dr1, s);
        *nr1 = dd_mul(dr, -s);
        *f2 = 1;
    } else {
        const double k = s / c;
        *A = k * (dr1.hi / dr.hi);
        *B = -(k * (dr.hi / dr1.hi));
        *nr = dd_mul(dr, c);
        *nr1 = dd_mul(dr1, c);
        *f2 = 0;
    }
}

int oracle_apply_scaled_pass_f64(double* Q, int64_t ldq, int64_t m, const double* grid, int64_t grid_rows,
                                 const int32_t* place, int64_t c0, int64_t nloc, int64_t L0,
                                 int64_t layers)
{
    if (nloc < 2 || m <= 0) return 0;
    dd_t* d = (dd_t*)malloc(sizeof(dd_t) * nloc);
    if (!d) return -2;
    for (int64_t c = 0; c < nloc; ++c) { d[c].hi = 1.0; d[c].lo = 0.0; }
    for (int64_t L = 0; L < 64; ++L)
        for (int64_t r = 0; r + 1 < nloc; ++r) {
            double A = 0.0, B = 0.0;
            int f2 = 0;
            if (L < layers) {
                double c = 1.0, s = 0.0;
                const int64_t i = c0 + r, LL = L0 + L;
                if (place == NULL || LL < (int64_t)place[i]) {
                    c = grid[2 * (i + LL * grid_rows)];
                    s = grid[2 * (i + LL * grid_rows) + 1];
                }
                dd_t nr, nr1;
                scaled_coeffs(c, s, d[r], d[r + 1], &A, &B, &f2, &nr, &nr1);
                d[r] = nr;
                d[r + 1] = nr1;
            }
            double* x = Q + (c0 + r) * ldq;
            double* y = Q + (c0 + r + 1) * ldq;
            for (int64_t row = 0; row < m; ++row) {
                const double a = x[row], b = y[row];
                const double u = f2 ? b : a, v = f2 ? a : b;
                x[row] = fma(A, v, u);
                y[row] = fma(B, u, v);
            }
        }
    for (int64_t c = 0; c < nloc; ++c) {
        double* x = Q + (c0 + c) * ldq;
        for (int64_t row = 0; row < m; ++row) x[row] = d[c].hi * x[row];
    }
    free(d);
    return 0;
}

/* The whole bulk apply in the scaled form: passes of 64 layers over columns 0..n-1. */
int oracle_apply_scaled_f64(double* Q, int64_t ldq, int64_t m, int64_t n, const double* cs, int64_t k)
{
    for (int64_t L0 = 0; L0 < k; L0 += 64) {
        const int64_t layers = k - L0 < 64 ? k - L0 : 64;
        const int rc = oracle_apply_scaled_pass_f64(Q, ldq, m, cs, n - 1, NULL, 0, n, L0, layers);
        if (rc) return rc;
    }
    return 0;
}

/* Layer-major definition of the bulk apply: Q (m x n, column-major, leading dim ldq)
 * times every rotation of the (n-1) x k grid cs (Julia Matrix{Tuple{T,T}} layout: entry
 * (i,L), 0-based, holds c at cs[2*(i + L*(n-1))] and s right after it). */
void oracle_apply_seq_f64(double* Q, int64_t ldq, int64_t m, int64_t n, const double* cs, int64_t k)
{
    for (int64_t L = 0; L < k; ++L)
        for (int64_t i = 0; i + 1 < n; ++i) {
            double c = cs[2 * (i + L * (n - 1))], s = cs[2 * (i + L * (n - 1)) + 1];
            double* x = Q + i * ldq;
            double* y = Q + (i + 1) * ldq;
            for (int64_t r = 0; r < m; ++r) rot_f64(x + r, y + r, c, s);
        }
}

void oracle_apply_seq_f32(float* Q, int64_t ldq, int64_t m, int64_t n, const float* cs, int64_t k)
{
    for (int64_t L = 0; L < k; ++L)
        for (int64_t i = 0; i + 1 < n; ++i) {
            float c = cs[2 * (i + L * (n - 1))], s = cs[2 * (i + L * (n - 1)) + 1];
            float* x = Q + i * ldq;
            float* y = Q + (i + 1) * ldq;
            for (int64_t r = 0; r < m; ++r) rot_f32(x + r, y + r, c, s);
        }
}

/* ------------------------------------------------------------------------------------ */
/* Wave-order fused apply (src/wave.jl:62-162, src/bulk_givens.jl:4-279)                 */
/* ------------------------------------------------------------------------------------ */
/*
 * The grid is walked in waves w = 2, 4, 6, ... (1-based as in wave.jl).  Wave w holds the
 * blocks of layer pairs (j, j+1), j = 1, 3, ..., k-1, whose first column is sc = w - j - 1.
 * A block carries up to four rotations, applied in this order to the columns sc..sc+3:
 *   (sc+1, j), (sc+2, j), (sc, j+1), (sc+1, j+1).
 * Rotations outside 1..n-1 are absent (the reference's two truncated kernels); a block
 * whose present rotations all have s == 0 is skipped, as the reference does.
 * Requires k even and n - 1 odd (src/wave.jl:65-66).
 */
#define WAVE_TEMPLATE(T, ROT)                                                                  \
static void wave_block_##T(T* Q, int64_t ldq, int64_t m, int64_t n, const T* cs, int64_t k,    \
                           int64_t sc, int64_t j)                                              \
{                                                                                              \
    /* 1-based rotation indices and layers */                                                  \
    const int64_t ri[4] = {sc + 1, sc + 2, sc, sc + 1};                                        \
    const int64_t li[4] = {j, j, j + 1, j + 1};                                                \
    T c[4] = {0}, s[4] = {0}; int present[4]; int any = 0;                                     \
    for (int q = 0; q < 4; ++q) {                                                              \
        present[q] = (ri[q] >= 1 && ri[q] <= n - 1 && li[q] >= 1 && li[q] <= k);               \
        if (present[q]) {                                                                      \
            int64_t idx = (ri[q] - 1) + (li[q] - 1) * (n - 1);                                 \
            c[q] = cs[2 * idx]; s[q] = cs[2 * idx + 1];                                        \
            if (s[q] != 0) any = 1;                                                            \
        }                                                                                      \
    }                                                                                          \
    if (!any) return;                                                                          \
    /* columns sc..sc+3 (1-based) -> pointers; absent columns are never touched */             \
    T* col[4];                                                                                 \
    for (int q = 0; q < 4; ++q) {                                                              \
        int64_t cidx = sc + q;                                                                 \
        col[q] = (cidx >= 1 && cidx <= n) ? Q + (cidx - 1) * ldq : NULL;                       \
    }                                                                                          \
    /* rotation q acts on columns (ri[q], ri[q]+1) = local (ri[q]-sc, ri[q]-sc+1) */           \
    if (present[0] && present[1] && present[2] && present[3]) {                                \
        /* the full block (bulk_givens.jl:43-57): straight-line code the compiler vectorizes */ \
        T* restrict c0p = col[0]; T* restrict c1p = col[1];                                    \
        T* restrict c2p = col[2]; T* restrict c3p = col[3];                                    \
        for (int64_t r = 0; r < m; ++r) {                                                      \
            T v0 = c0p[r], v1 = c1p[r], v2 = c2p[r], v3 = c3p[r];                              \
            ROT(&v1, &v2, c[0], s[0]);                                                         \
            ROT(&v2, &v3, c[1], s[1]);                                                         \
            ROT(&v0, &v1, c[2], s[2]);                                                         \
            ROT(&v1, &v2, c[3], s[3]);                                                         \
            c0p[r] = v0; c1p[r] = v1; c2p[r] = v2; c3p[r] = v3;                                \
        }                                                                                      \
        return;                                                                                \
    }                                                                                          \
    for (int64_t r = 0; r < m; ++r) {                                                          \
        T v[4];                                                                                \
        for (int q = 0; q < 4; ++q) v[q] = col[q] ? col[q][r] : (T)0;                          \
        for (int q = 0; q < 4; ++q)                                                            \
            if (present[q]) { int64_t a = ri[q] - sc; ROT(&v[a], &v[a + 1], c[q], s[q]); }     \
        for (int q = 0; q < 4; ++q) if (col[q]) col[q][r] = v[q];                              \
    }                                                                                          \
}                                                                                              \
static void wave_apply_##T(T* Q, int64_t ldq, int64_t m, int64_t n, const T* cs, int64_t k)    \
{                                                                                              \
    int64_t wmax = (n - 1) + k + 1;                                                            \
    for (int64_t w = 2; w <= wmax; w += 2)                                                     \
        for (int64_t j = 1; j <= k - 1; j += 2) {                                              \
            int64_t sc = w - j - 1;                                                            \
            if (sc + 2 < 1 || sc > n - 1) continue;                                            \
            wave_block_##T(Q, ldq, m, n, cs, k, sc, j);                                        \
        }                                                                                      \
}

WAVE_TEMPLATE(double, rot_f64)
WAVE_TEMPLATE(float, rot_f32)

typedef struct {
    void* Q; int64_t ldq, m, n, k; const void* cs; int is_f32;
} wave_job;

static void* wave_worker(void* arg)
{
    wave_job* jb = (wave_job*)arg;
    if (jb->is_f32) wave_apply_float((float*)jb->Q, jb->ldq, jb->m, jb->n, (const float*)jb->cs, jb->k);
    else wave_apply_double((double*)jb->Q, jb->ldq, jb->m, jb->n, (const double*)jb->cs, jb->k);
    return NULL;
}

/* Row slabs of a multiple of W rows per thread, the last thread takes the remainder
 * (src/wave.jl:44-57).  Returns 0, or 1 when the reference's asserts would fail. */
static int wave_parallel(void* Q, int64_t ldq, int64_t m, int64_t n, const void* cs, int64_t k,
                         int nthreads, int is_f32)
{
    if ((n - 1) % 2 != 1 || k % 2 != 0) return 1;
    const int64_t W = 8;
    size_t esz = is_f32 ? sizeof(float) : sizeof(double);
    if (nthreads <= 1) {
        wave_job jb = {Q, ldq, m, n, k, cs, is_f32};
        wave_worker(&jb);
        return 0;
    }
    int64_t part = W * ((m / nthreads) / W);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);
    wave_job* jobs = (wave_job*)malloc(sizeof(wave_job) * nthreads);
    for (int t = 0; t < nthreads; ++t) {
        int64_t from = part * t;
        int64_t to = (t == nthreads - 1) ? m : part * (t + 1);
        jobs[t].Q = (char*)Q + from * esz; jobs[t].ldq = ldq; jobs[t].m = to - from;
        jobs[t].n = n; jobs[t].k = k; jobs[t].cs = cs; jobs[t].is_f32 = is_f32;
        pthread_create(&th[t], NULL, wave_worker, &jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th); free(jobs);
    return 0;
}

int oracle_apply_wave_f64(double* Q, int64_t ldq, int64_t m, int64_t n, const double* cs, int64_t k, int nthreads)
{ return wave_parallel(Q, ldq, m, n, cs, k, nthreads, 0); }

int oracle_apply_wave_f32(float* Q, int64_t ldq, int64_t m, int64_t n, const float* cs, int64_t k, int nthreads)
{ return wave_parallel(Q, ldq, m, n, cs, k, nthreads, 1); }

/* ------------------------------------------------------------------------------------ */
/* The eigensolver driver: single_shift! and qr_algorithm! (src/bulge_chasing.jl)      */
/* ------------------------------------------------------------------------------------ */

/* is_offdiagonal_small (src/bulge_chasing.jl:7-8); 1-based i as in the reference. */
static inline int is_small(const double* dv, const double* ev, int64_t i, double tol)
{
    return fabs(ev[i - 1]) <= tol * (fabs(dv[i - 1]) + fabs(dv[i]));
}

/* Record (c,s) of rotation i (1-based).  The reference stores it at
 * givens[i, ++layer_thickness[i]] (src/bulge_chasing.jl:61-63, 137-139): `thick` is that
 * count and drives the capacity rule.  `place` is the grid layer actually used: equal to
 * thick in reference mode, or the sweep's common layer in exact-order mode (see
 * sweep_layer). */
static inline void record(double* givens, int64_t* thick, int64_t* place, int64_t rows,
                          int64_t i, int64_t layer, double c, double s)
{
    thick[i - 1] += 1;
    if (layer <= 0) layer = thick[i - 1];
    place[i - 1] = layer;
    int64_t idx = (i - 1) + (layer - 1) * rows;
    givens[2 * idx] = c;
    givens[2 * idx + 1] = s;
}

/* Layer for every rotation of a sweep over [from, to] in exact-order mode.
 *
 * The reference applies a flush's grid in layer-major order (its wave order).  That equals
 * the order in which the chase produced the rotations only if every sweep finds the same
 * layer count on all of its indices.  When a block that had split re-merges (an
 * off-diagonal that was small stops being small because a neighbouring diagonal entry
 * changed) a sweep meets uneven counts, and the reference's Q then loses accuracy
 * (residual ~0.3 at n=257 for d, e ~ U[0,1)).  Exact-order mode puts every rotation of a
 * sweep at one layer, above everything it must follow:
 *   L = 1 + max(place[from..to-1], place[to], place[from-1] - 1)
 * (rotation to shares column to with rotation to-1 and must precede it; rotation from-1
 * shares column from and precedes it already when its layer is <= L).  Slots skipped over
 * stay (1,0).  The chase, and therefore every eigenvalue, is unchanged. */
static int64_t sweep_layer(const int64_t* place, int64_t n, int64_t from, int64_t to)
{
    int64_t L = 0;
    for (int64_t q = from; q <= to - 1; ++q) if (place[q - 1] > L) L = place[q - 1];
    if (to <= n - 1 && place[to - 1] > L) L = place[to - 1];
    if (from >= 2 && place[from - 2] - 1 > L) L = place[from - 2] - 1;
    return L + 1;
}

/* single_shift! (src/bulge_chasing.jl:11-144); dv, ev 0-based arrays, from/to 1-based.
 * layer <= 0: reference placement; layer > 0: every rotation of the sweep at that layer. */
void oracle_single_shift(double* dv, double* ev, int64_t n, int64_t from, int64_t to, double mu,
                         double* givens, int64_t rows, int64_t* thick, int64_t* place,
                         int64_t layer)
{
    double H11 = dv[from - 1], H21 = ev[from - 1];
    double c, s, nrm;
    oracle_givens(H11 - mu, H21, &c, &s, &nrm);
    double H22 = dv[from];
    double H11p = fma(c, H11, s * H21);
    double H21p = fma(c, H21, -(s * H11));
    double H12p = fma(c, H21, s * H22);
    double H22p = fma(c, H22, -(s * H21));
    double H11pp = fma(H11p, c, H12p * s);
    double H12pp = fma(H12p, c, -(H11p * s));
    double H22pp = fma(H22p, c, -(H21p * s));
    dv[from - 1] = H11pp;
    dv[from] = H22pp;
    ev[from - 1] = H12pp;
    double bulge = 0.0;
    if (from + 2 <= to) {
        double H23 = ev[from];
        bulge = s * H23;
        ev[from] = c * H23;
    }
    record(givens, thick, place, rows, from, layer, c, s);

    for (int64_t i = from + 1; i <= to - 1; ++i) {
        double p1 = ev[i - 2], p2 = bulge;
        oracle_givens(p1, p2, &c, &s, &nrm);
        ev[i - 2] = nrm;
        double B11 = dv[i - 1], B22 = dv[i], B21 = ev[i - 1];
        double B11p = fma(c, B11, s * B21);
        double B21p = fma(c, B21, -(s * B11));
        double B12p = fma(c, B21, s * B22);
        double B22p = fma(c, B22, -(s * B21));
        double B11pp = fma(B11p, c, B12p * s);
        double B12pp = fma(B12p, c, -(B11p * s));
        double B22pp = fma(B22p, c, -(B21p * s));
        dv[i - 1] = B11pp;
        dv[i] = B22pp;
        ev[i - 1] = B12pp;
        if (i + 2 <= to) {
            double B23 = ev[i];
            bulge = s * B23;
            ev[i] = c * B23;
        }
        record(givens, thick, place, rows, i, layer, c, s);
    }
}

/* Wilkinson shift (src/bulge_chasing.jl:239-265): eigenvalue of the trailing 2x2 of the
 * block closest to its last diagonal entry, computed on the scaled block.  Plain IEEE. */
double oracle_wilkinson_shift(double a, double b, double c)
{
    /* a = H[to-1,to-1], b = H[to,to], c = H[to-1,to] */
    double scale = fabs(a) + 2.0 * fabs(c) + fabs(b);
    double H11 = a / scale, H12 = c / scale, H22 = b / scale;
    double t = (H11 + H22) / 2.0;
    double p = (H11 - t) * (H22 - t);
    double q = H12 * H12;
    double d = p - q;
    double sq = sqrt(fabs(d));
    double l1 = t + sq, l2 = t - sq;
    double lam = fabs(H22 - l1) < fabs(H22 - l2) ? l1 : l2;
    return lam * scale;
}

typedef struct {
    int64_t n;
    int32_t max_layers;
    double tol;
    int64_t maxiter;
    int64_t start, last_block_ends_at, iter;
    int32_t exact_order;        /* 1: exact-order placement (see sweep_layer) */
    int32_t grid_layers;        /* layer capacity of the grid buffer */
    int64_t flush_count;
    int64_t rotations;          /* rotations written by the last flush */
    int64_t total_rotations;    /* all rotations written so far */
    int64_t early_flushes;      /* flushes ended because a sweep's layer exceeded grid_layers */
    int64_t max_place;          /* thickest grid column of the last flush */
    int64_t min_from, max_to;   /* 1-based column range of the last flush's sweeps */
    int32_t ms_bulges;          /* multishift batches: bulge cap (0: single shifts only) */
    int32_t ms_rows;            /* multishift batches: block rows per bulge */
    int32_t ms_window;          /* multishift batches: shift window, in multiples of the bulges */
    int32_t ms_min;             /* multishift batches: fewest bulges of a batch (else a single sweep) */
    int64_t batches;            /* multishift batches run */
} oracle_qr_state;

void oracle_qr_init(oracle_qr_state* st, int64_t n, int32_t max_layers, double tol, int64_t maxiter,
                    int32_t exact_order)
{
    memset(st, 0, sizeof(*st));
    st->n = n; st->max_layers = max_layers; st->tol = tol; st->maxiter = maxiter;
    st->start = 1; st->last_block_ends_at = n; st->iter = 0;
    st->exact_order = exact_order;
    st->grid_layers = exact_order ? 2 * max_layers : max_layers;
}

/* The shifts of a multishift batch of nb sweeps over the block [from, to] (1-based): nb
 * eigenvalues of the block's trailing w x w principal submatrix, w = min(window * nb, to -
 * from + 1), ascending -- those ranked about the bottom diagonal entry: with r the number of
 * the window's eigenvalues below dv[to] (a Sturm count), the ones of rank k0 .. k0 + nb - 1,
 * k0 = min(max(r - nb / 2, 0), w - nb).  With window = 1 they are all of the trailing
 * square's eigenvalues.  A window twice the batch approximates the eigenvalues that belong
 * to the bottom rows better than the square of the batch's size does (about a quarter fewer
 * sweeps at n = 16384, case A).  Eigenvalues by bisection on Sturm counts (the LDL^T pivots of
 * T - x I, a negative pivot per eigenvalue below x) down to adjacent doubles.  The device
 * computes the same eigenvalues to about 1e-16 relative to the window's norm by FP32
 * bisection and a safeguarded FP64 Newton iteration; shifts only steer convergence, so the
 * two need not agree in their last bits. */
static int oracle_sturm_count(const double* d, const double* e, int w, double x, double pivmin)
{
    int cnt = 0;
    double q = d[0] - x;
    if (q < 0.0) ++cnt;
    for (int i = 1; i < w; ++i) {
        if (fabs(q) < pivmin) q = -pivmin;
        q = (d[i] - x) - e[i - 1] * e[i - 1] / q;
        if (q < 0.0) ++cnt;
    }
    return cnt;
}

static void oracle_trailing_eigenvalues(const double* dv, const double* ev, int64_t from, int64_t to, int nb,
                                        int window, double* out)
{
    int64_t w64 = (int64_t)window * nb;
    if (w64 > to - from + 1) w64 = to - from + 1;
    const int w = (int)w64;
    const double* d = dv + (to - w);
    const double* e = ev + (to - w);
    double lo = INFINITY, hi = -INFINITY, e2max = 0.0;
    for (int i = 0; i < w; ++i) {
        const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < w - 1 ? fabs(e[i]) : 0.0);
        if (d[i] - r < lo) lo = d[i] - r;
        if (d[i] + r > hi) hi = d[i] + r;
        if (i < w - 1 && e[i] * e[i] > e2max) e2max = e[i] * e[i];
    }
    const double pivmin = DBL_MIN * (e2max > 1.0 ? e2max : 1.0);
    const double wd = hi - lo;
    lo -= 1e-12 * (wd > 0.0 ? wd : 1.0) + DBL_MIN;
    hi += 1e-12 * (wd > 0.0 ? wd : 1.0) + DBL_MIN;
    int k0 = 0;
    if (w > nb) {
        k0 = oracle_sturm_count(d, e, w, d[w - 1], pivmin) - nb / 2;
        if (k0 < 0) k0 = 0;
        if (k0 > w - nb) k0 = w - nb;
    }
    for (int j = 0; j < nb; ++j) {
        const int k = k0 + j;
        double a = lo, b = hi;
        for (int it = 0; it < 200; ++it) {
            const double mid = 0.5 * (a + b);
            if (!(mid > a && mid < b)) break;
            if (oracle_sturm_count(d, e, w, mid, pivmin) > k) b = mid;
            else a = mid;
        }
        out[j] = 0.5 * (a + b);
    }
}

/* One pass of qr_algorithm!'s outer loop up to (not including) the bulk apply
 * (src/bulge_chasing.jl:166-279).  givens: (n-1) x grid_layers (c,s) pairs; thick, place:
 * n entries.  Returns 1 when rotations were recorded (the caller applies them), 0 when the
 * matrix has converged (no rotation recorded), -1 when iter exceeded maxiter (the reference
 * returns (H, false, iter) without applying the partial flush). */
int oracle_qr_flush(oracle_qr_state* st, double* dv, double* ev, double* givens, int64_t* thick,
                    int64_t* place)
{
    const int64_t n = st->n;
    const int64_t start = st->start;
    const double tol = st->tol;
    const int64_t rows = n > 1 ? n - 1 : 1;
    for (int64_t q = 0; q < rows * (int64_t)st->grid_layers; ++q) { givens[2 * q] = 1.0; givens[2 * q + 1] = 0.0; }
    for (int64_t q = 0; q < n; ++q) { thick[q] = 0; place[q] = 0; }
    int did_a_thing = 0;
    int64_t rot_before = st->total_rotations;
    int64_t to = st->last_block_ends_at;
    st->min_from = n + 1;
    st->max_to = 0;
    for (;;) {
        if (st->iter > st->maxiter) return -1;
        int64_t from = to;
        while (from > start && !is_small(dv, ev, from - 1, tol)) from -= 1;
        if (to <= start) break;
        if (from == to) {
            ev[from - 2] = 0.0;
            if (to == st->last_block_ends_at) st->last_block_ends_at -= 1;
            to -= 1;
        } else {
            int64_t thickness = 0;
            for (int64_t q = from; q <= to; ++q) if (thick[q - 1] > thickness) thickness = thick[q - 1];
            if (thickness == st->max_layers) {
                to = from - 1;
            } else {
                int64_t layer = 0;
                if (st->exact_order) {
                    layer = sweep_layer(place, n, from, to);
                    if (layer > st->grid_layers) { st->early_flushes += 1; break; }
                }
                /* multishift (the device's chase mode 3): as many sweeps as the block's length,
                 * its layer room (the capacity rule of that many single sweeps) and maxiter
                 * allow, with the trailing submatrix's eigenvalues as shifts; the device chases
                 * them as concurrent bulges, which computes what these sweeps in sequence do */
                int64_t nbl = 1;
                if (st->ms_bulges >= 2) {
                    int64_t cap = (int64_t)st->max_layers - thickness;
                    if (st->exact_order && (int64_t)st->grid_layers - layer + 1 < cap) cap = st->grid_layers - layer + 1;
                    nbl = (to - from + 1) / st->ms_rows;
                    if (nbl > st->ms_bulges) nbl = st->ms_bulges;
                    if (nbl > cap) nbl = cap;
                    if (nbl > st->maxiter - st->iter + 1) nbl = st->maxiter - st->iter + 1;
                    if (nbl < st->ms_min) nbl = 1;
                }
                did_a_thing = 1;
                if (nbl >= 2) {
                    double shifts[128];
                    oracle_trailing_eigenvalues(dv, ev, from, to, (int)nbl, st->ms_window, shifts);
                    for (int64_t j = 0; j < nbl; ++j)
                        oracle_single_shift(dv, ev, n, from, to, shifts[j], givens, rows, thick, place,
                                            layer > 0 ? layer + j : 0);
                    st->batches += 1;
                } else {
                    double mu = oracle_wilkinson_shift(dv[to - 2], dv[to - 1], ev[to - 2]);
                    oracle_single_shift(dv, ev, n, from, to, mu, givens, rows, thick, place, layer);
                    nbl = 1;
                }
                if (from < st->min_from) st->min_from = from;
                if (to > st->max_to) st->max_to = to;
                st->total_rotations += nbl * (to - from);
                st->iter += nbl;
            }
        }
        if (to <= start) break;
    }
    st->rotations = st->total_rotations - rot_before;
    st->max_place = 0;
    for (int64_t q = 0; q < n; ++q) if (place[q] > st->max_place) st->max_place = place[q];
    if (!did_a_thing) return 0;
    st->flush_count += 1;
    return 1;
}

/* qr_algorithm!(H, Q, max_layers, tol, maxiter) (src/bulge_chasing.jl:146-288).
 * d (n), e (n-1) are overwritten (eigenvalues unsorted in d); Q (m x n, ldq) is overwritten
 * with Q * prod(G).  q_is_f32 != 0 means Q is float and every (c,s) is rounded to float
 * before the update (the FP32-Q variant; the chase stays FP64).  Returns 0 on success,
 * a positive value for bad arguments, -2 for allocation failure. */
int oracle_qr_form(double* d, double* e, int64_t n, void* Q, int64_t ldq, int64_t m, int q_is_f32,
                   int32_t max_layers, double tol, int64_t maxiter, int32_t exact_order,
                   int32_t apply_form, int32_t* converged, int64_t* iter, int64_t* flushes,
                   int64_t* rotations);

int oracle_qr(double* d, double* e, int64_t n, void* Q, int64_t ldq, int64_t m, int q_is_f32,
              int32_t max_layers, double tol, int64_t maxiter, int32_t exact_order,
              int32_t* converged, int64_t* iter, int64_t* flushes, int64_t* rotations)
{
    return oracle_qr_form(d, e, n, Q, ldq, m, q_is_f32, max_layers, tol, maxiter, exact_order, 0,
                          converged, iter, flushes, rotations);
}

/* oracle_qr with the bulk apply in the canonical form (apply_form 0) or in the device's
 * scaled form (apply_form 1, FP64 Q): each flush is applied to the columns its sweeps
 * touched, min_from-1 .. max_to-1, in passes of 64 layers (oracle_apply_scaled_pass_f64),
 * as the device applies it. */
static int oracle_qr_driver(double* d, double* e, int64_t n, void* Q, int64_t ldq, int64_t m, int q_is_f32,
                            int32_t max_layers, double tol, int64_t maxiter, int32_t exact_order,
                            int32_t apply_form, int32_t ms_bulges, int32_t ms_rows, int32_t ms_window,
                            int32_t ms_min, int32_t* converged, int64_t* iter, int64_t* flushes,
                            int64_t* rotations, int64_t* batches);

int oracle_qr_form(double* d, double* e, int64_t n, void* Q, int64_t ldq, int64_t m, int q_is_f32,
                   int32_t max_layers, double tol, int64_t maxiter, int32_t exact_order,
                   int32_t apply_form, int32_t* converged, int64_t* iter, int64_t* flushes,
                   int64_t* rotations)
{
    return oracle_qr_driver(d, e, n, Q, ldq, m, q_is_f32, max_layers, tol, maxiter, exact_order,
                            apply_form, 0, 16, 1, 2, converged, iter, flushes, rotations, NULL);
}

/* The device's multishift chase (chase mode 3; not the reference's algorithm, which is
 * oracle_qr) restated: where a block has room, a batch of up to ms_bulges sweeps
 * (min(ms_bulges, len / ms_rows), the layer room and maxiter decide; fewer than ms_min make a
 * single sweep with the reference's shift instead) with the eigenvalues of
 * a trailing window of ms_window times the batch's size as shifts (oracle_trailing_eigenvalues),
 * run as sweeps in sequence with the reference's rotations; every other decision, the apply
 * and the placement as in oracle_qr.  FP64 Q, canonical apply.  *batches receives the number
 * of batches. */
int oracle_qr_multishift(double* d, double* e, int64_t n, double* Q, int64_t ldq, int64_t m,
                         int32_t max_layers, double tol, int64_t maxiter, int32_t exact_order,
                         int32_t ms_bulges, int32_t ms_rows, int32_t ms_window, int32_t ms_min,
                         int32_t* converged, int64_t* iter, int64_t* flushes, int64_t* rotations,
                         int64_t* batches)
{
    if (ms_bulges < 2 || ms_bulges > 128 || ms_rows < 4 || ms_window < 1 || ms_window > 4) return 1;
    if (ms_min < 2 || ms_min > ms_bulges) return 1;
    return oracle_qr_driver(d, e, n, Q, ldq, m, 0, max_layers, tol, maxiter, exact_order, 0, ms_bulges,
                            ms_rows, ms_window, ms_min, converged, iter, flushes, rotations, batches);
}

static int oracle_qr_driver(double* d, double* e, int64_t n, void* Q, int64_t ldq, int64_t m, int q_is_f32,
                            int32_t max_layers, double tol, int64_t maxiter, int32_t exact_order,
                            int32_t apply_form, int32_t ms_bulges, int32_t ms_rows, int32_t ms_window,
                            int32_t ms_min, int32_t* converged, int64_t* iter, int64_t* flushes,
                            int64_t* rotations, int64_t* batches)
{
    if (apply_form != 0 && q_is_f32) return 1;
    if (n < 1 || max_layers < 1 || (Q && ldq < m)) return 1;
    oracle_qr_state st;
    oracle_qr_init(&st, n, max_layers, tol, maxiter, exact_order);
    st.ms_bulges = ms_bulges;
    st.ms_rows = ms_rows;
    st.ms_window = ms_window;
    st.ms_min = ms_min;
    int64_t nr = n > 1 ? n - 1 : 1;
    int64_t GL = st.grid_layers;
    double* givens = (double*)malloc(sizeof(double) * 2 * nr * GL);
    float* g32 = q_is_f32 ? (float*)malloc(sizeof(float) * 2 * nr * GL) : NULL;
    int64_t* thick = (int64_t*)malloc(sizeof(int64_t) * n);
    int64_t* place = (int64_t*)malloc(sizeof(int64_t) * n);
    if (!givens || !thick || !place || (q_is_f32 && !g32)) { free(givens); free(g32); free(thick); free(place); return -2; }
    int rc;
    *converged = 1;
    for (;;) {
        rc = oracle_qr_flush(&st, d, e, givens, thick, place);
        if (rc < 0) { *converged = 0; break; }
        if (rc == 0) break;
        if (Q && m > 0) {
            /* only layers up to the thickest grid column carry rotations */
            int64_t K = st.max_place;
            if (q_is_f32) {
                for (int64_t q = 0; q < 2 * (n - 1) * K; ++q) g32[q] = (float)givens[q];
                oracle_apply_seq_f32((float*)Q, ldq, m, n, g32, K);
            } else if (apply_form == 1) {
                const int64_t c_lo = st.min_from - 1, n_loc = st.max_to - c_lo;
                for (int64_t L0 = 0; L0 < K; L0 += 64) {
                    rc = oracle_apply_scaled_pass_f64((double*)Q, ldq, m, givens, nr, NULL, c_lo, n_loc,
                                                      L0, K - L0 < 64 ? K - L0 : 64);
                    if (rc) { free(givens); free(g32); free(thick); free(place); return rc; }
                }
            } else {
                oracle_apply_seq_f64((double*)Q, ldq, m, n, givens, K);
            }
        }
    }
    *iter = st.iter;
    if (flushes) *flushes = st.flush_count;
    if (rotations) *rotations = st.total_rotations;
    if (batches) *batches = st.batches;
    free(givens); free(g32); free(thick); free(place);
    return 0;
}

/* The reference's own solve path, for timing on the host (the CPU baseline of the full
 * eigensolve): qr_algorithm! exactly as src/bulge_chasing.jl:146-288 runs it -- the
 * reference's grid placement (givens[i, ++layer_thickness[i]]), a grid of (n-1) x max_layers
 * filled with (1, 0) at every flush (:169), and each flush applied as a whole by the
 * row-slab threaded wave kernel, bulk_wave_order_2x2_rmul_parallel!(Q, givens) (:282,
 * src/wave.jl:36-60), on nthreads threads.  Needs even n and even max_layers, as the
 * reference asserts (:155, src/wave.jl:65-66); returns 1 otherwise.  The chase and the applies
 * are timed separately (seconds of wall clock).  apply_every > 1 applies only every
 * apply_every-th flush (a timing sample: the chase never reads Q, and the wave kernel's cost
 * depends on the grid only, about in proportion to its rotations); *rot_applied and
 * *rot_total count the rotations of the applied flushes and of all flushes. */
static double now_seconds(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int oracle_qr_reference_path(double* d, double* e, int64_t n, double* Q, int64_t ldq, int64_t m,
                             int32_t max_layers, double tol, int64_t maxiter, int nthreads,
                             int32_t apply_every, int32_t* converged, int64_t* iter, int64_t* flushes,
                             double* chase_seconds, double* apply_seconds, int64_t* rot_applied,
                             int64_t* rot_total)
{
    if (n < 2 || n % 2 != 0 || max_layers < 2 || max_layers % 2 != 0 || (Q && ldq < m)) return 1;
    oracle_qr_state st;
    oracle_qr_init(&st, n, max_layers, tol, maxiter, 0);
    const int64_t nr = n - 1;
    double* givens = (double*)malloc(sizeof(double) * 2 * nr * max_layers);
    int64_t* thick = (int64_t*)malloc(sizeof(int64_t) * n);
    int64_t* place = (int64_t*)malloc(sizeof(int64_t) * n);
    if (!givens || !thick || !place) { free(givens); free(thick); free(place); return -2; }
    double tc = 0.0, ta = 0.0;
    int64_t ra = 0, f = 0;
    if (apply_every < 1) apply_every = 1;
    *converged = 1;
    for (;; ++f) {
        double t0 = now_seconds();
        int rc = oracle_qr_flush(&st, d, e, givens, thick, place);
        tc += now_seconds() - t0;
        if (rc < 0) { *converged = 0; break; }
        if (rc == 0) break;
        if (Q && m > 0 && f % apply_every == 0) {
            t0 = now_seconds();
            wave_parallel(Q, ldq, m, n, givens, max_layers, nthreads, 0);
            ta += now_seconds() - t0;
            ra += st.rotations;
        }
    }
    if (rot_applied) *rot_applied = ra;
    if (rot_total) *rot_total = st.total_rotations;
    *iter = st.iter;
    if (flushes) *flushes = st.flush_count;
    if (chase_seconds) *chase_seconds = tc;
    if (apply_seconds) *apply_seconds = ta;
    free(givens); free(thick); free(place);
    return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Diagnostics (tests only)                                                              */
/* ------------------------------------------------------------------------------------ */

/* The same driver, but every rotation is applied to Q the moment the chase produces it:
 * the order that defines the QR iteration mathematically.  Exact-order placement must give
 * the same Q as this, bit for bit.  *uneven_sweeps counts the sweeps that met uneven
 * reference layer counts (where the reference's grid order differs from time order). */
int oracle_qr_timeorder(double* d, double* e, int64_t n, double* Q, int64_t ldq, int64_t m,
                        int32_t max_layers, double tol, int64_t maxiter,
                        int32_t* converged, int64_t* iter, int64_t* uneven_sweeps)
{
    if (n < 1 || max_layers < 1 || (Q && ldq < m)) return 1;
    oracle_qr_state st;
    oracle_qr_init(&st, n, max_layers, tol, maxiter, 0);
    int64_t rows = n > 1 ? n - 1 : 1;
    double* givens = (double*)malloc(sizeof(double) * 2 * rows * max_layers);
    int64_t* thick = (int64_t*)malloc(sizeof(int64_t) * n);
    int64_t* place = (int64_t*)malloc(sizeof(int64_t) * n);
    int64_t uneven = 0;
    *converged = 1;
    const int64_t start = 1;
    for (;;) {
        for (int64_t q = 0; q < n; ++q) { thick[q] = 0; place[q] = 0; }
        int did = 0, stop = 0;
        int64_t to = st.last_block_ends_at;
        for (;;) {
            if (st.iter > st.maxiter) { stop = -1; break; }
            int64_t from = to;
            while (from > start && !is_small(d, e, from - 1, tol)) from -= 1;
            if (to <= start) break;
            if (from == to) {
                e[from - 2] = 0.0;
                if (to == st.last_block_ends_at) st.last_block_ends_at -= 1;
                to -= 1;
            } else {
                int64_t thickness = 0, tmin = INT64_MAX, tmax = 0;
                for (int64_t q = from; q <= to; ++q) if (thick[q - 1] > thickness) thickness = thick[q - 1];
                if (thickness == max_layers) {
                    to = from - 1;
                } else {
                    for (int64_t q = from; q <= to - 1; ++q) {
                        if (thick[q - 1] < tmin) tmin = thick[q - 1];
                        if (thick[q - 1] > tmax) tmax = thick[q - 1];
                    }
                    if (tmax != tmin) uneven += 1;
                    double mu = oracle_wilkinson_shift(d[to - 2], d[to - 1], e[to - 2]);
                    did = 1;
                    oracle_single_shift(d, e, n, from, to, mu, givens, rows, thick, place, 0);
                    if (Q && m > 0)
                        for (int64_t i = from; i <= to - 1; ++i) {
                            int64_t idx = (i - 1) + (place[i - 1] - 1) * rows;
                            double c = givens[2 * idx], s = givens[2 * idx + 1];
                            double* x = Q + (i - 1) * ldq;
                            double* y = Q + i * ldq;
                            for (int64_t r = 0; r < m; ++r) rot_f64(x + r, y + r, c, s);
                        }
                    st.iter += 1;
                }
            }
            if (to <= start) break;
        }
        if (stop < 0) { *converged = 0; break; }
        if (!did) break;
    }
    *iter = st.iter;
    *uneven_sweeps = uneven;
    free(givens); free(thick); free(place);
    return 0;
}
