/*
 * symeig.h -- C ABI of libsymeig.so, the GB300 (sm_103a) implementation of
 * SymmetricEigenProblem.jl's eigensolver hot path.
 *
 * Every entry point returns an int status: 0 = success, > 0 = argument error (nothing was
 * touched), < 0 = device error.  No C++ exception crosses this boundary.  Matrices are
 * column-major with an explicit leading dimension, exactly as Julia stores them.  A handle
 * owns one device, one CUDA stream and grow-only scratch buffers; use one handle per host
 * thread.
 *
 * Reference interfaces replaced (paths inside the SymmetricEigenProblem.jl project):
 *   symeig_qr_*            qr_algorithm!(H::SymTridiagonal, Q, max_layers, tol, maxiter)
 *                          src/bulge_chasing.jl:146  -> (H, converged, iter)
 *   symeig_apply_givens_*  bulk_wave_order_2x2_rmul!(A, givens)  src/wave.jl:62 and
 *                          bulk_wave_order_2x2_rmul_parallel!(A, givens)  src/wave.jl:36
 *   symeig_eigen_decomp_*  eigen_decomp!(H)  src/bulge_chasing.jl:290-299
 */
#ifndef SYMEIG_H
#define SYMEIG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define SYMEIG_OK                 0
#define SYMEIG_ERR_NULL           1   /* a required pointer is NULL                       */
#define SYMEIG_ERR_SIZE           2   /* n < 1, m < 0, k < 0, or a size overflows         */
#define SYMEIG_ERR_LD             3   /* leading dimension smaller than the row count     */
#define SYMEIG_ERR_LAYERS         4   /* max_layers < 1                                   */
#define SYMEIG_ERR_HANDLE         5   /* invalid handle                                   */
#define SYMEIG_ERR_CUDA          -1   /* a CUDA runtime call failed                       */
#define SYMEIG_ERR_NOMEM         -2   /* device or pinned host allocation failed          */
#define SYMEIG_ERR_TIMEOUT       -3   /* a bounded device wait ran out (kernel returned)  */
#define SYMEIG_ERR_DEVICE        -4   /* a kernel reported an internal error              */

typedef struct symeig_context* symeig_handle;

/* Statistics of the last solve or apply on a handle. */
typedef struct {
    int64_t iterations;      /* QR sweeps (the reference's iter)                          */
    int64_t flushes;         /* bulk applications of the rotation buffer                  */
    int64_t rotations;       /* non-padding rotations recorded by the chase               */
    int64_t applied_rotation_rows; /* rotations x rows of Q the apply kernels processed   */
    double  chase_ms;        /* device time of the chase kernels                          */
    double  apply_ms;        /* device time of the table-build + apply kernels            */
    double  total_ms;        /* wall time of the call                                     */
    int64_t early_flushes;   /* flushes ended early to keep exact rotation order (see below)  */
    int64_t wave_launches;   /* launches of the wave-window Givens kernel                 */
    double  wave_kernel_ms;  /* their summed device time (only with kernel timing on)     */
    int64_t device_errors;   /* nonzero if a kernel's bounded wait gave up (sticky)        */
    int64_t redone_sweeps;   /* chase sweeps run again in the reference form (see below)  */
    int64_t bulge_batches;   /* multishift batches the chase ran (chase mode 3)           */
} symeig_stats;

/* Create a handle bound to CUDA device `device`.  Replaces nothing in the reference (the
 * Julia code has no device state); the Julia binding creates one per task. */
int symeig_create(symeig_handle* out, int device);
int symeig_destroy(symeig_handle h);
/* The stream the *_dev entry points run on: a cudaStream_t, where NULL is the legacy default
 * stream.  A new handle uses a non-blocking stream of its own; symeig_get_stream returns the
 * current one (save it to restore it later). */
int symeig_set_stream(symeig_handle h, void* stream);
int symeig_get_stream(symeig_handle h, void** stream);
int symeig_get_stats(symeig_handle h, symeig_stats* out);
/* Rotation placement of the qr driver.  1 (default): every rotation of a sweep goes to one
 * grid layer, so the layer-major (wave) order of a flush is exactly the order the chase
 * produced the rotations; eigenvalues and the sweep sequence are the reference's.  0: the
 * reference's placement, grid[i, ++layer_thickness[i]] (src/bulge_chasing.jl:61-63,
 * 137-139), whose wave order differs from the chase's order when a split block re-merges
 * within a flush (Q then loses accuracy in the reference too).  No reference counterpart. */
int symeig_set_exact_order(symeig_handle h, int32_t exact_order);
/* How the chase kernel computes its rotations.  Modes 0-2 give the same bits: the reference's
 * sweep sequence and rotations.
 * 0 (default): two warps, givensAlgorithm's plain branch from FMA-only Newton steps whose
 *   rounding is proved step by step; a sweep with an unproved step is restored and run again
 *   in the reference form (counted in redone_sweeps).
 * 1: the reference form (correctly rounded division and square root) on one thread.
 * 2: as 0, but every sweep is then redone in the reference form (exercises the restore).
 * 3: multishift.  Where a block has at least 2 * 16 rows and room for several layers, the
 *   chase runs a batch of up to 64 sweeps (symeig_set_multishift) whose shifts are nb
 *   eigenvalues of the block's trailing window of 2 nb rows (those ranked about its bottom
 *   entry; FP32 bisection, then a safeguarded FP64 Newton iteration), as bulges chased
 *   concurrently on separate SMs, each a fixed number of rows behind the one before.  The
 *   deflation test, the capacity rule and the rotation placement are those of a sequence of
 *   single sweeps with those shifts; shorter blocks take the Wilkinson single sweep of mode 0.
 *   Results meet the same error bounds as the reference (eigenvalues within 10 n eps ||T||,
 *   residual and orthogonality within 10 n eps) but are not the reference's bits; the sweep
 *   count is about the reference's (1.00x at n = 16384 with d_i = i, about 1.3x on a random
 *   diagonal), the chase time far lower.  No reference counterpart. */
int symeig_set_chase_mode(symeig_handle h, int32_t mode);
/* Batch shape of chase mode 3: a batch over a block of len rows runs
 * min(max_bulges, len / rows_per_bulge) bulges (and only when that is at least 2), and each
 * bulge releases its progress to the next every release_every steps.  max_bulges in
 * [2, 128] (default 64), rows_per_bulge >= 4 (default 16), release_every a power of two in
 * [1, 64] (default 4).  No reference counterpart. */
int symeig_set_multishift(symeig_handle h, int32_t max_bulges, int32_t rows_per_bulge,
                          int32_t release_every);
/* Fewest bulges of a chase-mode-3 batch: a block with room for fewer (len / rows_per_bulge,
 * capped by max_bulges and the layer room) takes one sweep with the reference's Wilkinson
 * shift instead, which avoids a batch's launches and shift solve on short blocks.
 * min_bulges in [2, 128]; default 2.  No reference counterpart. */
int symeig_set_multishift_min(symeig_handle h, int32_t min_bulges);
/* Arithmetic form of the FP64 bulk apply (symeig_apply_givens_f64*, and the qr driver's
 * apply with FP64 Q).  0 (default): every rotation as the reference's rmul!, two products and
 * two FMAs per rotation and row; from 3072 rows of Q on, the two products are computed on the
 * integer pipes (exact round-to-nearest-even FP64 products, see symeig_mul_rn_f64_dev) and
 * only the FMAs use the FP64 pipe.  2: the same rotation with all four operations on the FP64
 * pipe; forms 0 and 2 give the same bits.  1: the scaled ("fast Givens") form: columns carry
 * scale factors within each pass of 64 layers, so a rotation costs two FMAs per row; results
 * agree with form 0 to a few ulps per rotation (not bit for bit) and with the oracle's
 * restatement of the same form bit for bit.  The FP32, left, batched and allocation-free
 * applies use form 0.  No reference counterpart. */
int symeig_set_apply_form(symeig_handle h, int32_t form);
/* Test hook for the failure path of the bounded device waits: with chunk > 0 the wave
 * kernels stop copying their rotation table from that chunk on, so their waits run out
 * (~2 s of SM clock), the kernels return without touching Q further, and the synchronous
 * entry points return SYMEIG_ERR_TIMEOUT (device_errors = 1 in the statistics).  In chase
 * mode 3 the first bulge of each batch also stops releasing its progress, so the next bulge's
 * wait runs out the same way.  Q (and, in mode 3, H) is then unspecified; the handle and the
 * context stay usable.  0 (default) turns it off. */
int symeig_set_test_stall(symeig_handle h, int32_t chunk);
/* Record CUDA events around every wave-kernel launch so symeig_get_stats can report their
 * device time (wave_kernel_ms).  Off by default.  symeig_get_stats waits for the last
 * marked launch.  No reference counterpart (the reference times with BenchmarkTools). */
int symeig_set_kernel_timing(symeig_handle h, int32_t on);
/* FMA throughput of device `device` now, in TFLOP/s (an FMA = 2 flops), FP64 when fp64 != 0
 * else FP32: the roofline denominator of the Givens kernels.  Runs ~10 ms.  No reference
 * counterpart (the README compares with LinearAlgebra.peakflops(), README.md:28-31). */
int symeig_measure_fma_peak(int device, int32_t fp64, double* tflops);
/* The FP64 tensor-core (mma.sync .f64) rate, TFLOP/s, measured the same way: the roofline
 * denominator of the adjoint and dense-reduction GEMMs.  No reference counterpart. */
int symeig_measure_dmma_peak(int device, double* tflops);
const char* symeig_status_string(int status);
/* Device properties the library tuned for (SM count, FP64/FP32 launch shapes). */
int symeig_device_info(symeig_handle h, int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor);

/* ---- qr_algorithm!  (src/bulge_chasing.jl:146-288) ---------------------------------- *
 * d[n] (diagonal) and e[n-1] (off-diagonal) are overwritten: d holds the eigenvalues,
 * unsorted, as H.dv does in the reference; e holds the deflated off-diagonal.
 * Q (m x n, column-major, leading dimension ldq >= m) is overwritten with Q * prod(G).
 * Q == NULL (with m == 0) computes eigenvalues only.  max_layers, tol and maxiter mean what
 * they mean in the reference (defaults there: 128, eps(Float64), 100n).  On return
 * *converged is 0 when iter exceeded maxiter (the reference's (H, false, iter)), and the
 * rotations of the unfinished flush are not applied to Q, as in the reference.
 * Unlike the reference, odd n is accepted (the even-n assert, src/bulge_chasing.jl:155,
 * exists only for the reference's fused kernels).
 * Host-pointer variants copy to the device and back; *_dev variants take device pointers
 * and run on the handle's stream (they return after the solve has finished). */
int symeig_qr_f64(symeig_handle h, double* d, double* e, int64_t n,
                  double* Q, int64_t ldq, int64_t m,
                  int32_t max_layers, double tol, int64_t maxiter,
                  int32_t* converged, int64_t* iter);
int symeig_qr_f64_dev(symeig_handle h, double* d, double* e, int64_t n,
                      double* Q, int64_t ldq, int64_t m,
                      int32_t max_layers, double tol, int64_t maxiter,
                      int32_t* converged, int64_t* iter);
/* FP32-Q variant: the chase is FP64, each (c,s) is rounded to float, Q is float. */
int symeig_qr_f64_q32(symeig_handle h, double* d, double* e, int64_t n,
                      float* Q, int64_t ldq, int64_t m,
                      int32_t max_layers, double tol, int64_t maxiter,
                      int32_t* converged, int64_t* iter);
int symeig_qr_f64_q32_dev(symeig_handle h, double* d, double* e, int64_t n,
                          float* Q, int64_t ldq, int64_t m,
                          int32_t max_layers, double tol, int64_t maxiter,
                          int32_t* converged, int64_t* iter);

/* ---- bulk_wave_order_2x2_rmul!  (src/wave.jl:36-162) ---------------------------------- *
 * A (m x n, column-major, lda >= m) <- A * prod of the (n-1) x k grid of rotations cs,
 * in the reference's wave order (equivalently: for L in 1:k, for i in 1:n-1,
 * rmul!(A, G[i,L]), src/simple_givens.jl:53-65).  cs uses Julia's Matrix{Tuple{T,T}}
 * layout: rotation (i,L) (0-based) has c at cs[2*(i + L*(n-1))] and s at the next slot.
 * Unlike the reference, any n >= 1 and any k >= 0 are accepted (the reference asserts odd
 * n-1 and even k, src/wave.jl:65-66, and silently needs k <= n-1). */
int symeig_apply_givens_f64(symeig_handle h, double* A, int64_t lda, int64_t m, int64_t n,
                            const double* cs, int64_t k);
int symeig_apply_givens_f32(symeig_handle h, float* A, int64_t lda, int64_t m, int64_t n,
                            const float* cs, int64_t k);
int symeig_apply_givens_f64_dev(symeig_handle h, double* A, int64_t lda, int64_t m, int64_t n,
                                const double* cs, int64_t k);
int symeig_apply_givens_f32_dev(symeig_handle h, float* A, int64_t lda, int64_t m, int64_t n,
                                const float* cs, int64_t k);

/* ---- batched qr_algorithm! ---------------------------------------------------------------- *
 * count independent solves, each exactly qr_algorithm!(SymTridiagonal(d_i, e_i), Q_i,
 * max_layers, tol, maxiter_factor * n_i) (src/bulge_chasing.jl:146; maxiter_factor <= 0
 * means the reference's 100).  Packed layout: matrix i has order n[i]; its diagonal is
 * d[sum_{j<i} n_j ...], its off-diagonal e[sum_{j<i} (n_j - 1) ...], its Q (n_i x n_i,
 * column-major, leading dimension n_i, overwritten with Q_i * prod(G)) at
 * Q[sum_{j<i} n_j^2 ...]; Q may be NULL (eigenvalues only).  n, converged and iters are host
 * arrays of count entries.  The reference has no batched entry point; this replaces a loop of
 * qr_algorithm! calls.  Matrices run one flush per round: a one-lane-per-matrix chase, then
 * a persistent wave-kernel launch over a device-built queue of (matrix, row tile) items.  Each
 * round's apply runs beside the next round's chase (double-buffered rotation grids); the
 * rounds are captured as CUDA graphs and replayed until every matrix has finished.  Device
 * scratch: the two grids take 2 * sum_i (n_i - 1) * G * 16 bytes, G = 2 * max_layers layers
 * (about 17.4 GB for 4096 matrices of n ~ U{32..1024} at max_layers = 128), plus the tables
 * and per-matrix state. */
int symeig_qr_batched_f64(symeig_handle h, int64_t count, const int64_t* n, double* d, double* e,
                          double* Q, int32_t max_layers, double tol, int64_t maxiter_factor,
                          int32_t* converged, int64_t* iters);
int symeig_qr_batched_f64_dev(symeig_handle h, int64_t count, const int64_t* n, double* d,
                              double* e, double* Q, int32_t max_layers, double tol,
                              int64_t maxiter_factor, int32_t* converged, int64_t* iters);
/* The same batched solve with an FP32 Q (the FP32-Q variant of qr_algorithm!: the chase and
 * the rotations stay FP64, each (c,s) is rounded to float and applied to the FP32 Q).  Same
 * packed layout, Q of sum n_i^2 floats.  No reference counterpart. */
int symeig_qr_batched_f64_q32(symeig_handle h, int64_t count, const int64_t* n, double* d, double* e,
                              float* Q, int32_t max_layers, double tol, int64_t maxiter_factor,
                              int32_t* converged, int64_t* iters);
int symeig_qr_batched_f64_q32_dev(symeig_handle h, int64_t count, const int64_t* n, double* d,
                                  double* e, float* Q, int32_t max_layers, double tol,
                                  int64_t maxiter_factor, int32_t* converged, int64_t* iters);
/* Autotuner of the batched apply: for each precision of Q and each size class (n <= split,
 * n > split) it times every candidate tile on a synthetic batch of that class (one 128-layer
 * flush of every matrix; orders spread over the class: 2048 matrices of n = 32 .. split, 512
 * of n = split + 1 .. 4 split) and keeps the fastest per (class, precision), process-wide.  Tiles: 0 = 16 rows x 8
 * lane groups of 8 layers, 1 = 32 rows x 4 groups of 16 layers (both 64 layers per pass),
 * 2 = 8 rows x 16 groups of 8 layers (128 layers per pass: a whole flush in one pass).  ms
 * (may be NULL) receives 12 timings, ms[(dtype * 2 + class) * 3 + tile] with dtype 0 = FP64 Q,
 * 1 = FP32 Q.  No reference counterpart. */
int symeig_batched_autotune(symeig_handle h, double* ms);
/* The same with the orders of the batch to be solved (count entries of n, host array): each
 * class is timed on those of its orders (thinned evenly to 1.5 GiB of FP64 Q), a class with
 * none on the spread above.  No reference counterpart. */
int symeig_batched_autotune_sizes(symeig_handle h, int64_t count, const int64_t* n, double* ms);
/* Read (set = 0) or write (set != 0) the tile shape of the single-matrix wave kernel for FP64
 * (fp64 != 0) or FP32: 0 = 8 lane groups of 8 layers (4 rows per warp), 1 = 4 groups of 16
 * layers (8 rows per warp); FP32 only: 2 = shape 1 and 3 = shape 0 with two rows per thread,
 * 4 = shape 1 in CTAs of 14 warps (112 rows); FP64 only: 2 = shape 0 in CTAs of 27 warps
 * (108 rows, one CTA per SM at m = 16384), 3 = 16 groups of 8 layers, passes of 128 layers
 * (2 rows per warp; canonical form, for more than 64 layers, else it runs as 0).  FP64 shape 0
 * runs as 2, and FP32 shape 2 as 4, when m >= 15000.  -1 (the default for both) chooses by the
 * launch's rows m: FP64 shape 3 below 7168 rows for more than 64 layers, else shape 0 below
 * 9728 rows and 2 from there; FP32 shape 0 below 7168, 1 below 14336 and 4 from there (the
 * fastest measured at each m).  Returns SYMEIG_ERR_SIZE for a shape the precision
 * lacks.  Process-wide.  No reference counterpart. */
int symeig_apply_tuning(int32_t fp64, int32_t* shape, int32_t set);
/* Read (set = 0) or write (set != 0) the batched tuning of FP64 Q (fp64 != 0) or FP32 Q: the
 * class split and the tile (0..2, as for the autotuner) per class.  SYMEIG_ERR_SIZE for a split
 * below 1 or a tile out of range.  Defaults: split 256, tile 0 for both classes. */
int symeig_batched_tuning_dtype(int32_t fp64, int64_t* split, int32_t* shape_small, int32_t* shape_large,
                                int32_t set);
/* symeig_batched_tuning_dtype for FP64 Q. */
int symeig_batched_tuning(int64_t* split, int32_t* shape_small, int32_t* shape_large, int32_t set);

/* ---- adjoint (reverse-mode derivative) of the eigensolve ------------------------------------ *
 * No reference counterpart (the reference has no derivatives); this is the pullback behind
 * the Julia ChainRulesCore rrule and the torch autograd Function of the host bindings.
 * For count matrices of order n (back to back): eigenvalues lam (n each, in the order the
 * solver returns them, i.e. unsorted like H.dv), eigenvectors Q (n x n column-major,
 * leading dimension n, the solver's output), loss gradients glam (n) and gQ (n x n, or NULL
 * for a loss of the eigenvalues only).  Writes dL/dd (gd, n each) and dL/de (ge, n-1 each):
 *   M = diag(glam) + F o (Q^T gQ), F_ij = 1/(lam_j - lam_i) (0 on the diagonal and where
 *   lam_i == lam_j), Abar = Q M Q^T, dL/dd_i = Abar_ii, dL/de_i = Abar_{i,i+1} + Abar_{i+1,i}.
 * Q^T gQ and Q M run on the FP64 tensor cores (mma.sync .f64) with the F-masking and the
 * (off-)diagonal extraction fused into their epilogues; Abar is never formed. */
int symeig_eig_adjoint_f64(symeig_handle h, int64_t count, int64_t n, const double* lam,
                           const double* Q, const double* glam, const double* gQ, double* gd,
                           double* ge);
int symeig_eig_adjoint_f64_dev(symeig_handle h, int64_t count, int64_t n, const double* lam,
                               const double* Q, const double* glam, const double* gQ, double* gd,
                               double* ge);

/* ---- bulk apply without any allocation -------------------------------------------------- *
 * No counterpart in the reference.  For callers that cannot allocate device memory at call
 * time (their device memory belongs to another allocator that reserved it up front, or
 * cudaMalloc's implicit synchronisation is unacceptable on their path).  Same operation and
 * arguments as symeig_apply_givens_f64_dev, but it needs no handle: A and cs are device
 * pointers, `stream` is a cudaStream_t (NULL = legacy default stream) on the current device,
 * and the call is asynchronous.  Its wave table lives in a file-scope device array of
 * SYMEIG_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until exit; n must
 * satisfy ceil((n + 71) / 9) * 10368 <= SYMEIG_NOALLOC_SCRATCH_BYTES (n <= 29053), else
 * SYMEIG_ERR_SIZE is returned and nothing runs.  The first call on a device resolves the
 * array's address (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  All calls share the array: calls whose kernels overlap on the
 * GPU race; calls on one stream are ordered and safe. */
#define SYMEIG_NOALLOC_SCRATCH_BYTES (32u << 20)
int symeig_apply_givens_f64_noalloc(double* A, int64_t lda, int64_t m, int64_t n,
                                    const double* cs, int64_t k, void* stream);
/* No counterpart in the reference.  The set-up step of symeig_apply_givens_f64_noalloc on
 * the current device, on its own: under lazy module loading (the CUDA default) the first
 * use of the entry point's module on a device loads it and claims its device array, which
 * fails with SYMEIG_ERR_CUDA if another allocator already holds the memory.  Call this once
 * per device before such an allocator reserves the device and before any stream capture;
 * it allocates nothing else and is cheap to repeat. */
int symeig_noalloc_init(void);
/* No counterpart in the reference.  The allocation-free apply is asynchronous, so its
 * return value cannot report a bounded wait that gave up inside its kernel (Q is then only
 * partly rotated).  This waits for `stream` (NULL = legacy default stream, current device),
 * reads the shared error word of the allocation-free apply on the current device, clears it,
 * and returns SYMEIG_ERR_TIMEOUT if any call since the last check gave up, else SYMEIG_OK.
 * It allocates nothing. */
int symeig_noalloc_status(void* stream);

/* ---- bulk lmul!: row rotations  (src/simple_givens.jl:38-51) --------------------------------- *
 * A (m x n, column-major, lda >= m) <- prod of the (m-1) x k grid of row rotations cs applied
 * from the left, in layer-major order: for L in 1:k, for i in 1:m-1, lmul!(G[i,L], A)
 * (rows i, i+1: a_i <- c a_i + s a_{i+1}, a_{i+1} <- -s a_i + c a_{i+1}).  The reference has
 * only the single-rotation lmul!; this is its bulk form (e.g. for applying Q^T to a block of
 * vectors).  Same cs layout as symeig_apply_givens_* with m in place of n. */
int symeig_apply_givens_left_f64(symeig_handle h, double* A, int64_t lda, int64_t m, int64_t n,
                                 const double* cs, int64_t k);
int symeig_apply_givens_left_f32(symeig_handle h, float* A, int64_t lda, int64_t m, int64_t n,
                                 const float* cs, int64_t k);
int symeig_apply_givens_left_f64_dev(symeig_handle h, double* A, int64_t lda, int64_t m,
                                     int64_t n, const double* cs, int64_t k);
int symeig_apply_givens_left_f32_dev(symeig_handle h, float* A, int64_t lda, int64_t m,
                                     int64_t n, const float* cs, int64_t k);

/* Dense symmetric -> tridiagonal, the step before qr_algorithm! (no reference counterpart:
 * the reference's callers supply a SymTridiagonal).  LAPACK dsytrd / dorgtr semantics, lower:
 * A (n x n, both triangles stored, column-major, lda) = Q T Q^T, T = SymTridiagonal(d, e);
 * on exit A's diagonal and subdiagonal hold T and the Householder vectors lie below, tau
 * (n-1) holds their scalars.  orgtr forms Q (n x n, ldq) from them.  syev is the dense
 * eigensolve: sytrd, orgtr into V, then qr_algorithm!(SymTridiagonal(lam, e), V): lam the
 * (unsorted) eigenvalues, V the eigenvectors; the device version overwrites A, the host
 * version leaves it unchanged.  Results match LAPACK within rounding (not bit for bit). */
int symeig_sytrd_f64(symeig_handle h, int64_t n, double* A, int64_t lda, double* d, double* e,
                     double* tau);
int symeig_sytrd_f64_dev(symeig_handle h, int64_t n, double* A, int64_t lda, double* d, double* e,
                         double* tau);
int symeig_orgtr_f64(symeig_handle h, int64_t n, const double* A, int64_t lda, const double* tau,
                     double* Q, int64_t ldq);
int symeig_orgtr_f64_dev(symeig_handle h, int64_t n, const double* A, int64_t lda, const double* tau,
                         double* Q, int64_t ldq);
int symeig_syev_f64(symeig_handle h, int64_t n, const double* A, int64_t lda, double* lam, double* V,
                    int64_t ldv, int32_t* converged, int64_t* iter);
int symeig_syev_f64_dev(symeig_handle h, int64_t n, double* A, int64_t lda, double* lam, double* V,
                        int64_t ldv, int32_t* converged, int64_t* iter);

/* get_rotation(f, g) -> (c, s, r) (src/simple_givens.jl:20-23, LinearAlgebra.givensAlgorithm)
 * elementwise on `count` pairs, computed on the device the way the chase computes them (the
 * proved Newton form, or the reference form when symeig_set_chase_mode(h, 1)); both give the
 * reference's bits.  Host arrays (copied) or, for _dev, device arrays on the handle's stream. */
int symeig_get_rotation_f64(symeig_handle h, int64_t count, const double* f, const double* g,
                            double* c, double* s, double* r);
int symeig_get_rotation_f64_dev(symeig_handle h, int64_t count, const double* f, const double* g,
                                double* c, double* s, double* r);
/* Elementwise FP64 products out[i] = a[i] * b[i] of device arrays on the handle's stream:
 * form 0 as the canonical bulk apply computes its rotation products (from integer
 * arithmetic on GB300's integer pipes, bit for bit the IEEE round-to-nearest product; lanes
 * with a zero, subnormal, infinite or NaN operand or an out-of-range result are recomputed on
 * the FP64 pipe), form 1 with the FP64 multiply.  A self-check of the apply's arithmetic: both
 * forms give the same bits.  No reference counterpart (the products are those of rmul!,
 * src/simple_givens.jl:53-65). */
int symeig_mul_rn_f64_dev(symeig_handle h, int64_t count, const double* a, const double* b, double* out,
                          int32_t form);
/* ---- eigen_decomp!  (src/bulge_chasing.jl:290-299) ----------------------------------- *
 * Q (n x n, ldq >= n) is set to the identity, then qr_algorithm! runs with the default
 * max_layers = 128, tol = eps, maxiter = 100n.  d/e overwritten as in symeig_qr_f64. */
int symeig_eigen_decomp_f64(symeig_handle h, double* d, double* e, int64_t n,
                            double* Q, int64_t ldq, int32_t* converged, int64_t* iter);

#ifdef __cplusplus
}
#endif

#endif /* SYMEIG_H */
