// symeig_common.cuh -- shared definitions of the libsymeig.so kernels (sm_103a).
//
// Floating-point forms are fixed with the _rn intrinsics so nvcc cannot contract or
// reassociate them; the CPU oracle uses the same forms, which lets the tests compare
// device and oracle results bit for bit:
//   rotation of a pair (x, y):   x' = fma(c, x, s*y);   y' = fma(c, y, -(s*x))
// This is rmul!(A, G::Rotation2) of the reference (src/simple_givens.jl:53-65) with the
// first product of each line fused.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace symeig {

template <typename T> struct Pair;
template <> struct Pair<double> { using type = double2; };
template <> struct Pair<float>  { using type = float2; };

__device__ __forceinline__ void rot(double& x, double& y, double c, double s)
{
    const double sy = __dmul_rn(s, y);
    const double sx = __dmul_rn(s, x);
    x = __fma_rn(c, x, sy);
    y = __fma_rn(c, y, -sx);
}

// The same rotation with the two products issued as FMAs with a -0.0 addend.  For every
// product p (including +-0, +-inf and NaN), p + (-0.0) == p bit for bit, so
// fma(s, y, -0.0) == s*y exactly; on GB300 an FP64 FMA issues at ~1.18x the rate of an FP64
// multiply (measured), and a rotation is half multiplies.  `nz` must be -0.0 supplied at run
// time (a kernel argument), so that no compiler pass folds the FMA back into a multiply.
__device__ __forceinline__ void rot_fma(double& x, double& y, double c, double s, double nz)
{
    const double sy = __fma_rn(s, y, nz);
    const double sx = __fma_rn(s, x, nz);
    x = __fma_rn(c, x, sy);
    y = __fma_rn(c, y, -sx);
}

__device__ __forceinline__ void rot(float& x, float& y, float c, float s)
{
    const float sy = __fmul_rn(s, y);
    const float sx = __fmul_rn(s, x);
    x = __fmaf_rn(c, x, sy);
    y = __fmaf_rn(c, y, -sx);
}

// ---- chase state shared by the chase kernel and the host driver -------------------------
enum ChaseStatus : int32_t {
    CHASE_RUNNING   = 0,
    CHASE_CONVERGED = 1,   // the flush recorded no rotation: the reference's `!did_a_thing && break`
    CHASE_MAXITER   = 2,   // iter > maxiter: the reference returns (H, false, iter)
    CHASE_FLUSH     = 3,   // rotations recorded; apply them, then chase again
    CHASE_BATCH     = 4,   // a multishift batch is pending: run it, then resume the flush
};

// Multishift batches (chase_mode 3): a batch over a block of len rows has at most
// min(ms_bulges, len / ms_rows) bulges (ChaseState; defaults kDefaultBulges and
// kDefaultRowsPerBulge, the fastest measured at n = 2000 and 16384), and never more than
// kMaxBulges.  A bulge releases its progress every kDefaultProgEvery steps; the host queues
// kBatchesAhead batches per round trip.
constexpr int kMaxBulges = 128;
constexpr int kDefaultBulges = 64;
constexpr int kDefaultRowsPerBulge = 16;
constexpr int kDefaultProgEvery = 4;
// A block with room for fewer than ms_min_bulges bulges takes a single sweep instead of a batch.
constexpr int kDefaultMinBulges = 2;
constexpr int kBatchesAhead = 8;

// Device scratch of a batch: the bulges' shifts and their progress words.
struct BulgeScratch {
    double shifts[kMaxBulges];
    long long prog[kMaxBulges];  // last step whose stores a bulge has released
};

struct ChaseState {
    int64_t n;
    int64_t start;               // always 1 (the reference's `start`)
    int64_t last_block_ends_at;  // 1-based, as in the reference
    int64_t iter;
    int64_t maxiter;
    double  tol;
    int32_t max_layers;
    int32_t grid_layers;         // layer capacity of the grid buffer
    int32_t exact_order;         // 1: exact-order placement, 0: the reference's placement
    int32_t status;
    // outputs of the last flush
    int64_t rotations;           // rotations recorded by the flush
    int64_t min_from;            // 1-based smallest `from` of any sweep
    int64_t max_to;              // 1-based largest `to` of any sweep
    int64_t max_thickness;       // thickest column of the rotation grid (placement layers)
    int64_t total_rotations;
    int64_t early_flushes;       // flushes ended because a sweep's layer exceeded grid_layers
    double  neg_zero;            // -0.0, supplied at run time (see mulz in givens.cuh)
    int32_t chase_mode;          // 0 Newton-form two-warp sweeps, 1 reference form on one
                                 // thread, 2 Newton form with every sweep redone (tests)
    int32_t pad0;
    int64_t redone_sweeps;       // sweeps run again in the reference form (cumulative)
    // chase_mode 3: the pending batch and the flush's loop state to resume after it
    int32_t resume;              // 1: the next chase launch continues the flush after a batch
    int32_t b_bulges;            // bulges of the pending batch
    int64_t b_from, b_to;        // 1-based block the batch sweeps
    int32_t b_layer0;            // exact-order layer of bulge 0, or 0 (the reference's placement)
    int32_t r_did;
    int64_t r_to, r_rotations, r_min_from, r_max_to, r_early;
    int64_t batches;             // batches run (cumulative)
    int32_t ms_bulges;           // bulge cap of a batch (2 .. kMaxBulges)
    int32_t ms_rows;             // rows of a block per bulge (>= 4)
    int32_t ms_prog_mask;        // a bulge releases its progress every (mask + 1) steps
    int32_t test_stall;          // test hook (symeig_set_test_stall): bulge 0 of a batch never
                                 // releases its progress, so the next bulge's wait runs out
    int32_t ms_min_bulges;       // fewest bulges of a batch; fewer make a single sweep (>= 2)
    int32_t pad1;
};

// ---- launch helpers (defined in the .cu files) ------------------------------------------
// Apply geometry of one pass of the wave-window kernel: columns [c0, c0 + n_loc) of Q and
// layers [L0, L0 + layers) of the (n-1) x * rotation grid.
// Parts of a pass that apply_pass launches: the table (with the scaled form's recurrence), the
// wave kernel over the m rows given, or both.  A table built once serves launches over
// disjoint row ranges of Q on several streams.
enum : int { kPassTable = 1, kPassWave = 2, kPassAll = 3 };

// Row blocks (and streams) of the pipelined host-pointer apply.
constexpr int kPipeBlocks = 16;

struct ApplyPass {
    int64_t c0, n_loc, L0, layers;
    int64_t rs = 1;  // stride between the kernel's rows (1: rmul!, lda: lmul! on the transpose)
    int32_t form = 0;  // 0 canonical rotations, 1 the scaled form (FP64 only; see apply.cu)
    int32_t stall = 0; // test hook: > 0 stops the table copies from that chunk on (see wave_tile)
    int32_t rec = 0;   // form 1: 1 if launch_scaled_recurrences already filled scratch slot `slot`
    int32_t slot = 0;  // form 1: the pass's scratch slot (its index within the flush)
};

// The scaled form's column-scale recurrences of all passes of [L0, L0 + layers) in one launch
// (one CTA per pass of 64 layers), into the scratch slots after the table.
cudaError_t launch_scaled_recurrences(const double* grid, int64_t grid_rows, const int32_t* place,
                                      int64_t c0, int64_t n_loc, int64_t L0, int64_t layers,
                                      void* table, cudaStream_t stream);

// Layers one pass of the wave-window kernel handles for element type T.
// Layers per pass of an apply of `layers` layers to m rows in `form` (64, or 128 where the
// 128-layer FP64 tile takes the pass).
template <typename T> int64_t apply_layers_per_pass(int64_t m, int64_t layers, int form);

// Bytes of the wave table one pass needs (for FP64 including the scaled form's scratch).
template <typename T> size_t apply_table_bytes(int64_t n_loc, int64_t layers);
// Bytes of the canonical form's table alone.
template <typename T> size_t apply_canonical_table_bytes(int64_t n_loc);

// Build the wave table of one pass from a grid of (c,s) pairs in Julia layout
// (grid_rows rows, column L = layer L).  When place != nullptr, layer L of rotation i is
// the identity unless L < place[i] (the qr flush: the reference fills unused slots with
// (1,0); here the chase writes only slots below place[i]).  Then run the wave-window
// kernel on Q.
// `err` is a device word the kernel sets to 1 if a bounded wait gave up (it never waits on
// anything but its own bulk copies).  ev_begin/ev_end (may be null) are recorded on
// `stream` around the wave kernel alone.
template <typename Tsrc, typename T>
cudaError_t apply_pass(T* Q, int64_t ldq, int64_t m, const Tsrc* grid, int64_t grid_rows,
                       const int32_t* thick, const ApplyPass& pass, void* table, int* err,
                       cudaStream_t stream, cudaEvent_t ev_begin = nullptr,
                       cudaEvent_t ev_end = nullptr, int what = kPassAll);

// A host-resident Q streamed through the device by column segments (apply_host_segmented).
struct HostStream {
    void* host;             // the caller's m x n column-major matrix (host memory)
    int64_t lda;            // its leading dimension
    cudaStream_t s_in, s_out;
    cudaEvent_t* ev_in;     // nseg events: columns of segment j copied in
    cudaEvent_t* ev_seg;    // nseg events: segment j's kernel done
    int nseg;
    void* state;            // apply_segment_state_bytes(m) bytes of device memory
};

// One pass of k <= 64 layers of the (n-1) x k grid d_cs (Julia layout, on the device) applied
// to a host-resident m x n Q through the device buffer dQ (leading dimension m), with the
// copies in, the kernels and the copies out overlapped by column segments (see apply.cu).
template <typename T>
cudaError_t apply_host_segmented(T* dQ, int64_t m, const T* d_cs, const ApplyPass& pass, void* table, int* err,
                                 cudaStream_t stream, const HostStream& io);
template <typename T> size_t apply_segment_state_bytes(int64_t m);
template <typename T> bool apply_host_segmented_supported(int64_t m);

// Tile shape of the single-matrix wave kernel per precision (see apply.cu).
void apply_set_shape(int fp64, int shape);
int apply_get_shape(int fp64);
int apply_num_shapes(int fp64);  // tile shapes available to FP64 (fp64 != 0) or FP32

// Dense symmetric -> tridiagonal (sytrd.cu).  Scratch sizes in doubles.
int64_t dense_scratch_doubles(int64_t n);
int sytrd_dev(cudaStream_t s, int64_t n, double* A, int64_t lda, double* d, double* e, double* tau,
              double* scratch);
int orgtr_dev(cudaStream_t s, int64_t n, const double* A, int64_t lda, const double* tau, double* Q,
              int64_t ldq, double* scratch);
// max |A_ij| into *out (device), and A *= scale (exact for a power of two)
cudaError_t launch_dense_maxabs(const double* A, int64_t lda, int64_t n, double* out, cudaStream_t s);
cudaError_t launch_dense_scale(double* A, int64_t lda, int64_t n, double scale, cudaStream_t s);
// d *= f, e *= f, and the diagonal / subdiagonal of A set from them
cudaError_t launch_tridiag_unscale(double* A, int64_t lda, int64_t n, double* d, double* e,
                                   double f, cudaStream_t s);
// a[i] * b[i] elementwise: form 0 the canonical apply's integer-pipe products, 1 the FP64 pipe.
cudaError_t launch_mul_rn(int64_t count, const double* a, const double* b, double* out, int32_t form,
                          cudaStream_t stream);
// givensAlgorithm elementwise on device arrays (form 0 Newton form, 1 reference form).
cudaError_t launch_get_rotation(int64_t count, const double* f, const double* g, double* c,
                                double* s, double* r, int32_t form, cudaStream_t stream);
// resume_only: run only if a multishift batch is pending resumption (else return at once).
cudaError_t launch_chase(ChaseState* state, double* d, double* e, double* grid, int32_t* thick,
                         int32_t* place, double* bak, BulgeScratch* bs, int32_t resume_only,
                         cudaStream_t stream);
// The pending multishift batch of `state`, if its status is CHASE_BATCH (else the launch
// returns at once): `bulges` (>= the batch's) CTAs of two warps in one cooperative launch,
// one bulge each.  A bounded wait that gives up sets *err.
cudaError_t launch_bulge_batch(const ChaseState* state, double* d, double* e, double* grid,
                               const int32_t* thick, BulgeScratch* bs, int* err, int32_t bulges,
                               cudaStream_t stream);

// One matrix of a batch: size and offsets into the packed arrays (elements, not bytes).
struct BatchMat {
    int64_t n;
    int64_t doff;    // diagonal (n), thick and place (n)
    int64_t eoff;    // off-diagonal (n-1)
    int64_t qoff;    // Q (n x n, leading dimension n)
    int64_t goff;    // rotation grid ((n-1) x grid_layers (c,s) pairs)
    int32_t cls;     // apply size class
    int32_t pad;
};

// One flush of every unfinished matrix of a batch, one lane per matrix, lanes in `order`.
cudaError_t launch_chase_batched(const BatchMat* mats, const int32_t* order, int32_t count,
                                 ChaseState* states, double* d, double* e, double* grids,
                                 int32_t* thick, int32_t* place, cudaStream_t stream);

// Batched solve on device pointers (batched.cu); n, converged, iters are host arrays; Q is
// FP64 or FP32 (the FP32-Q variant).
template <typename T>
int qr_batched_dev(int device, cudaStream_t stream, int64_t count, const int64_t* n, double* d,
                   double* e, T* Q, int32_t max_layers, double tol, int64_t maxiter_factor,
                   int32_t exact_order, int32_t* converged, int64_t* iters, int64_t* rounds_out,
                   double* ms_out);
int batched_autotune(int device, cudaStream_t stream, int64_t count, const int64_t* n, double* ms);
// Adjoint of the eigensolve for count matrices of order n (adjoint.cu).
int adjoint_dev(cudaStream_t s, int64_t count, int64_t n, const double* lam, const double* Q,
                const double* glam, const double* gQ, double* gd, double* ge, double* scratch);
int64_t adjoint_scratch_doubles(int64_t count, int64_t n);
void batched_set_tuning(int fp64, int64_t split, int32_t shape0, int32_t shape1);
void batched_get_tuning(int fp64, int64_t* split, int32_t* shape0, int32_t* shape1);
int batched_num_tiles();

}  // namespace symeig
