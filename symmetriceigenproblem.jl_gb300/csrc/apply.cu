// apply.cu -- the wave-window Givens kernel for one matrix: Q <- Q * prod of a grid of column
// rotations.
//
// Replaces bulk_wave_order_2x2_rmul[_parallel]! (src/wave.jl:36-162) and its fused SIMD
// kernels (src/bulk_givens.jl:4-279).  The reference streams all m rows of 4 columns per
// fused block and relies on cache for reuse across waves; here every thread owns one row of
// Q and keeps a sliding window of columns of that row in registers, so each element of Q is
// loaded once and stored once per pass of 64 layers.  The tile algorithm (wave order, layer
// groups, TMA-staged (c,s) table) is described in wave_common.cuh.
#include <algorithm>

#include "wave_common.cuh"

namespace symeig {

namespace {

using wave::Shape;
using wave::kThreads;

// Tile shapes.  Each covers 64 layers per pass, except FP64 shape 3 (128).
//   shape 0 = 8 lane groups of 8 layers: 4 rows per warp -- at m = 16384, 4096 warps, all
//             resident at <= 7 CTAs of 4 warps per SM (register budget 73), 6 or 7 warps per
//             SM sub-partition.  The FP64 shape below 9728 rows: the FP64 unit (2 FMA per SM
//             per clock on GB300) is the limit and this shape balances it best; from there
//             its CTAs of 27 warps (shape 2) even out the SMs' loads.
//   shape 1 = 4 lane groups of 16 layers: 8 rows per warp, twice the rotations per wave for
//             the same per-wave overhead (shuffle, Q load/store, address arithmetic).  For
//             FP32 the overhead per rotation matters more than the coarser balance.
//   shapes 2, 3 (FP32 only) = shapes 1, 0 with 2 rows per thread: each (c,s) pair read from
//             shared memory serves two rows, so the shared-memory pipe (2 wavefronts per
//             128-bit broadcast read of 4 or 8 distinct addresses) carries half the load per
//             rotation-row, and each thread has two independent rotation chains.  Shape 2
//             runs as shape 4 (below) from 15000 rows on.
// By default (kAutoShape) the rows of the launch choose the shape (resolve_shape).
template <typename T, int S> struct Cfg;
// MINB: CTAs per SM the launch bounds ask for; MINB_INT the same for the FP64 kernels whose
// products run on the integer pipes (int_mul.cuh: about 95 registers with one row per thread).
template <> struct Cfg<double, 0> { using Sh = Shape<double, 8, 8>; static constexpr int MINB = 7, MINB_INT = 5; static constexpr int THREADS = Sh::THREADS; };
template <> struct Cfg<double, 1> { using Sh = Shape<double, 16, 4>; static constexpr int MINB = 4, MINB_INT = 3; static constexpr int THREADS = Sh::THREADS; };
template <> struct Cfg<float, 0> { using Sh = Shape<float, 8, 8>; static constexpr int MINB = 7, MINB_INT = 7; static constexpr int THREADS = Sh::THREADS; };
template <> struct Cfg<float, 1> { using Sh = Shape<float, 16, 4>; static constexpr int MINB = 5, MINB_INT = 5; static constexpr int THREADS = Sh::THREADS; };
template <> struct Cfg<float, 2> { using Sh = Shape<float, 16, 4, 2>; static constexpr int MINB = 3, MINB_INT = 3; static constexpr int THREADS = Sh::THREADS; };
// FP64 shape 2 = shape 0 in one CTA of 27 warps (108 rows): at m = 16384 that is 152 CTAs, one
// per SM, every SM with the same rows, where 1024 CTAs of 16 rows leave 112 SMs with 7 CTAs and
// 40 with 6 (the kernel's time is the busiest SM's).  27 warps x 72 registers fit one SM.
template <> struct Cfg<double, 2> { using Sh = Shape<double, 8, 8, 1, 27>; static constexpr int MINB = 1, MINB_INT = 1; static constexpr int THREADS = Sh::THREADS; };
template <> struct Cfg<float, 3> { using Sh = Shape<float, 8, 8, 2>; static constexpr int MINB = 4, MINB_INT = 4; static constexpr int THREADS = Sh::THREADS; };
// FP32 shape 4 = shape 1 (one row per thread) in CTAs of 14 warps (112 rows): at m = 16384,
// 147 CTAs, about one per SM, 13.5 warps per SM.  FP32 shape 2 runs as shape 4 from 15000
// rows on: 27.8 TFLOP/s against 25.2 for shape 2 at 16384 x 16384, k = 64 (measured with every other FP32 shape: 8 x 8 in
// CTAs of 27 warps 25.2, 8 x 8 with two rows per thread in 14 warps 24.9, four rows per
// thread in 7 warps 24.3, 16 x 4 with two rows in 7 warps 27.6).
template <> struct Cfg<float, 4> { using Sh = Shape<float, 16, 4, 1, 14>; static constexpr int MINB = 1, MINB_INT = 1; static constexpr int THREADS = Sh::THREADS; };
// FP64 shape 3 = 16 lane groups of 8 layers: 128 layers per pass, 2 rows per warp.  A flush of
// the reference's 128-layer buffer runs as one pass instead of two: twice the lane groups per
// row (the parallelism of a short Q) and one read and write of Q instead of two.  Canonical
// form, for passes of more than 64 layers.
template <> struct Cfg<double, 3> { using Sh = Shape<double, 8, 16>; static constexpr int MINB = 5, MINB_INT = 5; static constexpr int THREADS = Sh::THREADS; };
static_assert(Cfg<float, 4>::Sh::CHUNK == Cfg<float, 1>::Sh::CHUNK, "table layout");
// the table depends on (KB, G) only, so shapes 2 and 3 share the tables of 1 and 0
static_assert(Cfg<float, 2>::Sh::CHUNK == Cfg<float, 1>::Sh::CHUNK, "table layout");
static_assert(Cfg<float, 3>::Sh::CHUNK == Cfg<float, 0>::Sh::CHUNK, "table layout");
static_assert(Cfg<double, 2>::Sh::CHUNK == Cfg<double, 0>::Sh::CHUNK, "table layout");

constexpr int kShapes[2] = {4, 5};  // shapes available to [0] FP64, [1] FP32
// FP64 shape 0 runs as shape 2 from this many rows on (about 152 SMs x 108 rows x 0.92)
constexpr int64_t kWideRows = 15000;
// The canonical FP64 form computes its products on the integer pipes from this many rows on.
// Below it the grid has too few warps to hide the integer products' longer dependency chain
// (measured, 64 layers on m x m: 556 against 642 GFLOP/s at m = 2000, 916 against 710 at
// m = 4096), and the products stay on the FP64 pipe; both give the same bits.
constexpr int64_t kIntMulRows = 3072;
// The tile shape by precision ([0] FP64, [1] FP32): a shape index, or kAutoShape (the default)
// for the shape chosen by the rows of the launch.  Measured at n = 4096, k = 64 for m = 1024 ..
// 16384 (TFLOP/s):
//   FP32  m:      2048   4096   6144   8192  12288  15000  16384
//         shape 0  8.60  15.10  18.77  19.64  19.82  21.44  23.25
//         shape 1  6.92  13.75  16.30  21.55  24.30  22.01  23.94
//         shape 4  3.32   6.62   9.95  13.26  19.86  24.25  26.31   (shape 2: within 8 % of 4)
//   FP64  shape 0  0.67   0.81   0.90   0.88   0.84   1.39*  1.51*  (* as shape 2)
//         shape 2  0.10   0.38   0.57   0.76   1.14   1.39   1.51
// The 27-warp FP64 shape runs one CTA of 108 rows per SM, so it pays once m gives it about 90
// of the 152 SMs; FP32 shape 0 wins while its 16-row CTAs are needed to fill the SMs, shape 1
// in between, and the 14-warp shape 4 from about 14000 rows.
constexpr int kAutoShape = -1;
constexpr int64_t kAutoWideRows64 = 9728;       // FP64: shape 0 below, shape 2 from here
constexpr int64_t kAutoRows32[2] = {7168, 14336};  // FP32: shape 0 below [0], 1 below [1], 4 from [1]
int g_shape[2] = {kAutoShape, kAutoShape};

// FP64: passes of more than 64 layers in the canonical form run as one 128-layer pass of
// shape 3 below this many rows (auto), where the grid is short of warps.  Measured on m x m, k =
// 128 (TFLOP/s, shape 0 as two passes against shape 3 as one): m = 1000 0.309 / 0.578, 3000
// 0.515 / 0.669, 4096 0.823 / 0.884, 6000 0.909 / 1.037, 8192 0.906 / 0.777; equal at 2000
// (0.641 / 0.650), where both leave a fifth of the SMs idle and saturate the FP64 pipes of the
// rest.  Both give the same bits.
constexpr int64_t kAutoDeepRows64 = 7168;

// The shape an m-row launch of T runs for a pass of `layers` layers in `form`: the auto choice
// above, or the tuned shape (FP64 0 runs as 2, and FP32 2 as 4, from kWideRows rows on).  The
// 128-layer FP64 shape 3 takes only passes of more than 64 layers of canonical rotations (the
// scaled form's recurrences run in passes of 64); others run as 0.
template <typename T> int resolve_shape(int64_t m, int64_t layers = 64, int form = 0)
{
    const int s = g_shape[sizeof(T) == 8 ? 0 : 1];
    if constexpr (sizeof(T) == 8) {
        const bool deep_ok = layers > 64 && form != 1;   // canonical rotations (form 0 or 2)
        if (s == kAutoShape) return (deep_ok && m < kAutoDeepRows64) ? 3 : (m < kAutoWideRows64 ? 0 : 2);
        if (s == 3) return deep_ok ? 3 : 0;
        return (s == 0 && m >= kWideRows) ? 2 : s;
    } else {
        if (s == kAutoShape) return m < kAutoRows32[0] ? 0 : (m < kAutoRows32[1] ? 1 : 4);
        return (s == 2 && m >= kWideRows) ? 4 : s;
    }
}

template <typename Tsrc, typename T, int S>
__global__ void __launch_bounds__(256)
build_table_kernel(unsigned char* __restrict__ table, int64_t n_chunks,
                   const Tsrc* __restrict__ grid, int64_t grid_rows,
                   const int32_t* __restrict__ place, int64_t c0, int64_t n_loc,
                   int64_t L0, int64_t layers)
{
    using Sh = typename Cfg<T, S>::Sh;
    constexpr int KB = Sh::KB, G = Sh::G;
    const int64_t total = n_chunks * Sh::CH * G * KB;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = idx / (G * KB);
        const int g = (int)((idx / KB) % G);
        const int l = (int)(idx % KB);
        wave::table_entry<T, Sh, Tsrc>(table, t, g, l, grid, grid_rows, place, c0, n_loc, L0, layers);
    }
}

// ---- the scaled (fast-Givens) form, FP64 -----------------------------------------------
//
// With Q = Qt diag(d) (d = 1 at the start of a pass), rotation (r, L) of the pass becomes two
// FMAs per row of Qt (wave_rotations_scaled):
//   form 1 (|c| >= |s|): k = s/c,  A = k (d[r+1]/d[r]),  B = -(k (d[r]/d[r+1])),
//                        d[r] <- c d[r],  d[r+1] <- c d[r+1];
//   form 2 (|s| >  |c|): k = c/s,  A = k (d[r]/d[r+1]),  B = -(k (d[r+1]/d[r])),
//                        d[r] <- s d[r+1],  d[r+1] <- -(s d[r]),
// each operation rounded once (divisions correctly rounded), and column c is multiplied by
// its final d[c] when it is stored.  |A B| <= 1 and every d loses at most a factor sqrt(2) per
// rotation, so 64 layers keep d within [2^-64, 1].  The recurrence carries each d as an
// unevaluated sum hi + lo (the products d <- m d exact to about 2^-106: p = RN(hi m),
// e = fma(hi, m, -p), e = fma(lo, m, e), hi' = RN(p + e), lo' = RN(e - RN(hi' - p)))
// and A, B and the final scale use hi.  With d rounded to one double at every product, the
// rounding errors of a column's scale are shared by all rows of Q (unlike the per-element
// errors of the canonical form) and add up pass after pass: ||Q^T Q - I|| of a full solve
// grew to 2.3x the canonical form's at n = 4096 and 13x at n = 16384.  With hi + lo it equals
// the canonical form's (0.0698 of 10 n eps at n = 4096, both).  Two kernels build the table:
//   scaled_recurrence_kernel: the d recurrence itself.  Only the multiplications d <- c d
//     form the chain; it runs as a wavefront (rotations r + 2L = step are independent and
//     touch disjoint columns) on one CTA of one thread per layer, and records each
//     rotation's d[r], d[r+1] before it (hi), its form, and each column's final d (hi).
//   scaled_table_kernel: A and B of every slot from those (the divisions, all independent),
//     the group's flag word and, for group G-1, the final d of the column it stores.

constexpr int kRB = 64;   // recurrence steps per staging block
constexpr int kPL = 2 * 63 + kRB;  // columns whose place[] a staging block needs

// shared memory of the recurrence: two staging blocks of (c, s) (one row of kRB pairs per
// layer) and of place[], and the ring of column scales
struct RecSmem {
    double2 cs[2][64][kRB + 1];   // rows padded by one pair: thread L reads row L
    int32_t pl[2][kPL + 2];
    double2 d[256];  // (hi, lo) of the column scales
};

// (hi, lo) * m, about 2^-106 relative: the recurrence's scale update
__device__ __forceinline__ double2 dd_mul(double2 a, double m)
{
    const double p = __dmul_rn(a.x, m);
    double e = __fma_rn(a.x, m, -p);
    e = __fma_rn(a.y, m, e);
    const double h = __dadd_rn(p, e);
    return make_double2(h, __dsub_rn(e, __dsub_rn(h, p)));
}

template <typename Tsrc>
__device__ __forceinline__ double2 grid_cs(const Tsrc* grid, int64_t grid_rows, const int32_t* place,
                                           int64_t i, int64_t L)
{
    if (place != nullptr && L >= (int64_t)place[i]) return make_double2(1.0, 0.0);
    const Tsrc* p = grid + 2 * (i + L * grid_rows);
    return make_double2((double)p[0], (double)p[1]);
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(wave::smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(wave::smem_u32(dst)), "l"(src) : "memory");
}

// Stage block `blk` (steps [blk kRB, (blk+1) kRB)): thread L copies its rotations
// r = t - 2L of those steps (layer L0+L, contiguous in the grid), all threads together the
// place[] entries of columns [blk kRB - 126, blk kRB + kRB).
__device__ __forceinline__ void rec_stage(RecSmem& sm, int buf, int64_t blk, const double* grid,
                                          int64_t grid_rows, const int32_t* place, int64_t c0,
                                          int64_t nr, int64_t L0, int64_t layers)
{
    const int L = threadIdx.x;
    const int64_t T = blk * kRB;
    if (L < layers) {
        const int64_t r0 = T - 2 * L;
        for (int k = 0; k < kRB; ++k) {
            const int64_t r = r0 + k;
            if (r >= 0 && r < nr) cp_async16(&sm.cs[buf][L][k], grid + 2 * (c0 + r + (L0 + L) * grid_rows));
        }
    }
    if (place != nullptr) {
        for (int q = L; q < kPL; q += 64) {
            const int64_t r = T - 126 + q;
            if (r >= 0 && r < nr) cp_async4(&sm.pl[buf][q], place + c0 + r);
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// The d recurrence of one pass (see the section comment); one CTA of 64 threads, thread L =
// layer L of the pass; step t treats rotation (t - 2L, L).  The grid is FP64 (the scaled
// form is FP64 only).
__host__ __device__ inline size_t scaled_pre_bytes(int64_t n_loc) { return (size_t)64 * (size_t)(n_loc - 1) * 16; }
__host__ __device__ inline size_t scaled_form_bytes(int64_t n_loc) { return ((size_t)64 * (size_t)(n_loc - 1) + 255) & ~(size_t)255; }
// one pass's scratch slot: pre (64 x (n_loc-1) double2), form (64 x (n_loc-1) bytes, padded),
// dfinal (n_loc doubles), padded to 256 bytes
__host__ __device__ inline size_t scaled_slot_bytes(int64_t n_loc)
{
    return (scaled_pre_bytes(n_loc) + scaled_form_bytes(n_loc) + (size_t)n_loc * sizeof(double) + 255) &
           ~(size_t)255;
}

// CTA b runs the recurrence of pass b of a flush: layers [L0 + 64 b, L0 + 64 b + 64) of the
// layers_total from L0 on, into scratch slot b.  The passes' recurrences are independent (d
// starts at 1 in every pass), so one launch of all of a flush's passes costs one pass.
__global__ void __launch_bounds__(64)
scaled_recurrence_kernel(const double* __restrict__ grid, int64_t grid_rows,
                         const int32_t* __restrict__ place, int64_t c0, int64_t n_loc, int64_t L0_all,
                         int64_t layers_total, unsigned char* __restrict__ scratch, size_t slot_bytes)
{
    extern __shared__ __align__(16) unsigned char rec_raw[];
    RecSmem& sm = *reinterpret_cast<RecSmem*>(rec_raw);
    const int64_t L0 = L0_all + 64 * (int64_t)blockIdx.x;
    const int64_t layers = layers_total - 64 * (int64_t)blockIdx.x < 64 ? layers_total - 64 * (int64_t)blockIdx.x : 64;
    unsigned char* slot = scratch + (size_t)blockIdx.x * slot_bytes;
    double2* __restrict__ pre = (double2*)slot;
    unsigned char* __restrict__ form = slot + scaled_pre_bytes(n_loc);
    double* __restrict__ dfinal = (double*)(form + scaled_form_bytes(n_loc));
    const int L = threadIdx.x;
    const int64_t nr = n_loc - 1;                       // rotations per layer
    const int64_t last = nr - 1 + 2 * (layers - 1);     // last step
    const int64_t nblk = last / kRB + 1;
    const bool active = L < layers;
    if (threadIdx.x == 0) sm.d[0] = make_double2(1.0, 0.0);
    rec_stage(sm, 0, 0, grid, grid_rows, place, c0, nr, L0, layers);
    for (int64_t blk = 0; blk < nblk; ++blk) {
        const int buf = (int)(blk & 1);
        if (blk + 1 < nblk) {
            rec_stage(sm, buf ^ 1, blk + 1, grid, grid_rows, place, c0, nr, L0, layers);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        const int64_t T = blk * kRB;
        for (int k = 0; k < kRB; ++k) {
            const int64_t t = T + k;
            if (t > last) break;   // uniform
            // column t+1 is first touched at step t (rotation (t, 0), thread 0)
            if (threadIdx.x == 0 && t + 1 < n_loc) sm.d[(t + 1) & 255] = make_double2(1.0, 0.0);
            const int64_t r = t - 2 * L;
            if (active && r >= 0 && r < nr) {
                double2 cs = sm.cs[buf][L][k];
                if (place != nullptr && L0 + L >= (int64_t)sm.pl[buf][r - (T - 126)]) cs = make_double2(1.0, 0.0);
                const double c = cs.x, s = cs.y;
                const double2 dr = sm.d[r & 255], dr1 = sm.d[(r + 1) & 255];
                // |s| > |c| on the integer pipe (an FP64 compare costs an FP64 issue slot)
                const uint64_t ac = (uint64_t)__double_as_longlong(c) & 0x7FFFFFFFFFFFFFFFull;
                const uint64_t as = (uint64_t)__double_as_longlong(s) & 0x7FFFFFFFFFFFFFFFull;
                const bool f2 = as > ac;
                pre[L * nr + r] = make_double2(dr.x, dr1.x);
                form[L * nr + r] = f2 ? 1 : 0;
                // form 1: (c dr, c dr1); form 2: (s dr1, -(s dr)) = (s dr1, (-s) dr)
                const double ns = __longlong_as_double(__double_as_longlong(s) ^ (long long)0x8000000000000000ull);
                const double m1 = f2 ? s : c, m2 = f2 ? ns : c;
                const double2 x1 = f2 ? dr1 : dr, x2 = f2 ? dr : dr1;
                sm.d[r & 255] = dd_mul(x1, m1);
                sm.d[(r + 1) & 255] = dd_mul(x2, m2);
            }
            __syncthreads();
            // column t - 2 (layers - 1) had its last rotation at this step (and the last
            // column with it)
            const int64_t cf = t - 2 * (layers - 1);
            if (threadIdx.x == 0 && cf >= 0 && cf < nr) {
                dfinal[cf] = sm.d[cf & 255].x;
                if (cf == nr - 1) dfinal[cf + 1] = sm.d[(cf + 1) & 255].x;
            }
        }
        __syncthreads();   // the staging buffer of this block is refilled next
    }
}

template <typename Tsrc, int S>
__global__ void __launch_bounds__(256)
scaled_table_kernel(unsigned char* __restrict__ table, int64_t n_chunks, const Tsrc* __restrict__ grid,
                    int64_t grid_rows, const int32_t* __restrict__ place, int64_t c0, int64_t n_loc,
                    int64_t L0, int64_t layers, const double2* __restrict__ pre,
                    const unsigned char* __restrict__ form, const double* __restrict__ dfinal)
{
    using Sh = typename Cfg<double, S>::Sh;
    constexpr int KB = Sh::KB, G = Sh::G, W = Sh::W;
    const int64_t nr = n_loc - 1;
    const int64_t total = n_chunks * Sh::CH * G;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = idx / G;
        const int g = (int)(idx % G);
        unsigned char* base = table + t * Sh::ITER + g * Sh::GSTRIDE;
        uint32_t flags = 0;
#pragma unroll
        for (int l = 0; l < KB; ++l) {
            const int64_t i_loc = t - (int64_t)g * W - 1 - l;
            const int64_t lay = (int64_t)g * KB + l;
            double A = 0.0, B = 0.0;
            if (i_loc >= 0 && i_loc < nr && lay < layers) {
                const double2 cs = grid_cs(grid, grid_rows, place, c0 + i_loc, L0 + lay);
                const double2 p = pre[lay * nr + i_loc];
                if (form[lay * nr + i_loc]) {
                    const double k = cs.x / cs.y;
                    A = k * (p.x / p.y);
                    B = -(k * (p.y / p.x));
                    flags |= 1u << l;
                } else {
                    const double k = cs.y / cs.x;
                    A = k * (p.y / p.x);
                    B = -(k * (p.x / p.y));
                }
            }
            *reinterpret_cast<double2*>(base + l * 16) = make_double2(A, B);
        }
        double dst = 0.0;
        const int64_t cst = t - (int64_t)(G - 1) * W - KB;   // the column group G-1 stores
        if (g == G - 1 && cst >= 0 && cst < n_loc) dst = dfinal[cst];
        *reinterpret_cast<uint32_t*>(base + KB * 16) = flags;
        *reinterpret_cast<uint32_t*>(base + KB * 16 + 4) = 0u;
        *reinterpret_cast<double*>(base + KB * 16 + 8) = dst;
    }
}

// One launch covers chunks [c_begin, c_end) of the pass (all of them unless the pass runs as
// column segments, see wave_tile); `state` holds the registers carried between segments,
// segment_state_values * THREADS values per CTA.
template <typename T, int S, bool SCALED = false, bool INT_MUL = false, bool SEG = false>
__global__ void __launch_bounds__(Cfg<T, S>::THREADS, INT_MUL ? Cfg<T, S>::MINB_INT : Cfg<T, S>::MINB)
wave_apply_kernel(T* __restrict__ Q, int64_t ldq, int64_t m, int32_t n_loc,
                  const unsigned char* __restrict__ table, int32_t n_chunks, int* __restrict__ err,
                  const T nz, int64_t rs, int32_t stall, int32_t c_begin, int32_t c_end,
                  T* __restrict__ state)
{
    using Sh = typename Cfg<T, S>::Sh;
    __shared__ __align__(128) unsigned char ring[2][Sh::CHUNK];
    __shared__ __align__(8) uint64_t bar[2];
    wave::Staging<Sh> st{ring, bar, 0, 0};
#ifdef SYMEIG_DEVICE_CHECKS
    st.check = err;
#endif
    wave::staging_init(st);
    const int64_t row0 = (int64_t)blockIdx.x * Sh::ROWS;
    T* cta_state = (SEG && state) ? state + (int64_t)blockIdx.x * (wave::segment_state_values<Sh>() * Sh::THREADS) : nullptr;
    if (!wave::wave_tile<T, Sh, SCALED, INT_MUL, SEG>(Q, ldq, m, row0, n_loc, table, n_chunks, nz, st, rs, stall,
                                                      c_begin, c_end, cta_state)) {
        if (threadIdx.x == 0) atomicOr(err, 1);
    }
}

// Elementwise products a[i] * b[i]: form 0 as the canonical FP64 apply computes them
// (integer pipes, FP64-pipe recomputation of the lanes the integer path does not cover),
// form 1 on the FP64 pipe.  A self-check of int_mul.cuh against the FP64 multiply.
__global__ void __launch_bounds__(256)
mul_rn_kernel(int64_t count, const double* __restrict__ a, const double* __restrict__ b,
              double* __restrict__ out, int32_t form, double nz)
{
    // every lane of a warp runs the same number of loop trips (the vote inside needs them all)
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t base = (int64_t)blockIdx.x * blockDim.x;
    for (int64_t i0 = base; i0 < count; i0 += stride) {
        const int64_t i = i0 + threadIdx.x;
        const bool ok = i < count;
        const double x = ok ? a[i] : 1.0, y = ok ? b[i] : 1.0;
        double p;
        if (form == 0) {
            const SplitFactor f = split_factor(x);
            bool sp = f.special;
            p = mul_rn_int(f, y, sp);
            if (__any_sync(0xffffffffu, sp)) {
                if (sp) p = fma_pair_call(x, y, y, nz).x;
            }
        } else {
            p = __dmul_rn(x, y);
        }
        if (ok) out[i] = p;
    }
}

}  // namespace

cudaError_t launch_mul_rn(int64_t count, const double* a, const double* b, double* out, int32_t form,
                          cudaStream_t stream)
{
    if (count <= 0) return cudaSuccess;
    const int64_t blocks = (count + 255) / 256 < 1216 ? (count + 255) / 256 : 1216;
    mul_rn_kernel<<<(unsigned)blocks, 256, 0, stream>>>(count, a, b, out, form, -0.0);
    return cudaGetLastError();
}

// Layers per pass of an apply of `layers` layers to m rows in `form`: 128 where the 128-layer
// FP64 shape takes it, else 64.
template <typename T> int64_t apply_layers_per_pass(int64_t m, int64_t layers, int form)
{
    if constexpr (sizeof(T) == 8)
        if (resolve_shape<T>(m, layers, form) == 3) return 128;
    return 64;
}
template int64_t apply_layers_per_pass<double>(int64_t, int64_t, int);
template int64_t apply_layers_per_pass<float>(int64_t, int64_t, int);

// bytes of the largest of the shapes' tables for passes of `layers` layers (so the tuning can
// change between calls), rounded up to 256
template <typename T> size_t table_region(int64_t n_loc, int64_t layers = 64)
{
    size_t b = (size_t)std::max(Cfg<T, 0>::Sh::table_bytes(n_loc), Cfg<T, 1>::Sh::table_bytes(n_loc));
    if constexpr (sizeof(T) == 8)
        if (layers > 64) b = std::max(b, (size_t)Cfg<T, 3>::Sh::table_bytes(n_loc));
    return (b + 255) & ~(size_t)255;
}

// FP64: the scaled form's scratch follows the table, one slot per pass of `layers`
template <typename T> size_t apply_table_bytes(int64_t n_loc, int64_t layers)
{
    size_t b = table_region<T>(n_loc, layers);
    if (sizeof(T) == 8 && n_loc >= 2) {
        const int64_t passes = layers > 64 ? (layers + 63) / 64 : 1;
        b += (size_t)passes * scaled_slot_bytes(n_loc);
    }
    return b;
}

cudaError_t launch_scaled_recurrences(const double* grid, int64_t grid_rows, const int32_t* place,
                                      int64_t c0, int64_t n_loc, int64_t L0, int64_t layers,
                                      void* table, cudaStream_t stream)
{
    if (n_loc < 2 || layers <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(scaled_recurrence_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(RecSmem));
    if (e != cudaSuccess) return e;
    const unsigned passes = (unsigned)((layers + 63) / 64);
    scaled_recurrence_kernel<<<passes, 64, sizeof(RecSmem), stream>>>(
        grid, grid_rows, place, c0, n_loc, L0, layers,
        (unsigned char*)table + table_region<double>(n_loc), scaled_slot_bytes(n_loc));
    return cudaGetLastError();
}
template size_t apply_table_bytes<double>(int64_t, int64_t);
template size_t apply_table_bytes<float>(int64_t, int64_t);

template <typename T> size_t apply_canonical_table_bytes(int64_t n_loc) { return table_region<T>(n_loc); }
template size_t apply_canonical_table_bytes<double>(int64_t);
template size_t apply_canonical_table_bytes<float>(int64_t);

// Chunk range of one launch of the wave kernel and the segment state (wave_tile).
struct Seg {
    int32_t c_begin = 0, c_end = -1;
    void* state = nullptr;
};

// The table of one pass (with the scaled form's recurrence and coefficients).
template <typename Tsrc, typename T, int S>
cudaError_t prep_pass_shape(const Tsrc* grid, int64_t grid_rows, const int32_t* place, const ApplyPass& pass,
                            void* table, cudaStream_t stream)
{
    using Sh = typename Cfg<T, S>::Sh;
    const int64_t n_chunks = Sh::chunks(pass.n_loc);
    if constexpr (sizeof(T) == 8) {
        if (pass.form == 1) {
            unsigned char* tb = (unsigned char*)table;
            unsigned char* slot = tb + table_region<T>(pass.n_loc) + (size_t)pass.slot * scaled_slot_bytes(pass.n_loc);
            double2* pre = (double2*)slot;
            unsigned char* form = slot + scaled_pre_bytes(pass.n_loc);
            double* dfinal = (double*)(form + scaled_form_bytes(pass.n_loc));
            static_assert(sizeof(Tsrc) == 8, "the scaled form reads an FP64 grid");
            if (!pass.rec) {  // else launch_scaled_recurrences filled this pass's slot
                cudaError_t e = cudaFuncSetAttribute(scaled_recurrence_kernel,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(RecSmem));
                if (e != cudaSuccess) return e;
                scaled_recurrence_kernel<<<1, 64, sizeof(RecSmem), stream>>>(
                    (const double*)grid, grid_rows, place, pass.c0, pass.n_loc, pass.L0, pass.layers, slot,
                    scaled_slot_bytes(pass.n_loc));
            }
            const int64_t total = n_chunks * Sh::CH * Sh::G;
            int64_t tb_blocks = (total + 255) / 256;
            if (tb_blocks > 152 * 16) tb_blocks = 152 * 16;
            scaled_table_kernel<Tsrc, S><<<(unsigned)tb_blocks, 256, 0, stream>>>(
                tb, n_chunks, grid, grid_rows, place, pass.c0, pass.n_loc, pass.L0, pass.layers,
                pre, form, dfinal);
            return cudaGetLastError();
        }
    }
    const int64_t total = n_chunks * Sh::CH * Sh::G * Sh::KB;
    int64_t tb_blocks = (total + 255) / 256;
    if (tb_blocks > 152 * 16) tb_blocks = 152 * 16;
    build_table_kernel<Tsrc, T, S><<<(unsigned)tb_blocks, 256, 0, stream>>>(
        (unsigned char*)table, n_chunks, grid, grid_rows, place, pass.c0, pass.n_loc, pass.L0,
        pass.layers);
    return cudaGetLastError();
}

// The wave kernel over chunks [seg.c_begin, seg.c_end) of one pass, rows [0, m).
// `int_mul_rows`: the canonical FP64 form takes the integer-pipe products from this many rows
// of the launch on.
template <typename T, int S, bool SEG>
cudaError_t launch_wave_variant(T* Q, int64_t ldq, int64_t m, const ApplyPass& pass, const void* table, int* err,
                                cudaStream_t stream, const Seg& seg, int64_t int_mul_rows)
{
    using Sh = typename Cfg<T, S>::Sh;
    const int64_t n_chunks = Sh::chunks(pass.n_loc);
    const int64_t blocks = (m + Sh::ROWS - 1) / Sh::ROWS;
    const int32_t stall = pass.stall > 0 ? pass.stall : 0x7fffffff;
    T* q = Q + pass.c0 * ldq;
    const unsigned char* tb = (const unsigned char*)table;
    if constexpr (sizeof(T) == 8) {
        if (pass.form == 1) {
            wave_apply_kernel<T, S, true, false, SEG><<<(unsigned)blocks, Sh::THREADS, 0, stream>>>(
                q, ldq, m, (int32_t)pass.n_loc, tb, (int32_t)n_chunks, err, (T)-0.0, pass.rs, stall,
                seg.c_begin, seg.c_end, (T*)seg.state);
            return cudaGetLastError();
        }
        if (pass.form == 0 && m >= int_mul_rows) {   // canonical FP64: products on the integer pipes
            wave_apply_kernel<T, S, false, true, SEG><<<(unsigned)blocks, Sh::THREADS, 0, stream>>>(
                q, ldq, m, (int32_t)pass.n_loc, tb, (int32_t)n_chunks, err, (T)-0.0, pass.rs, stall,
                seg.c_begin, seg.c_end, (T*)seg.state);
            return cudaGetLastError();
        }
    }
    wave_apply_kernel<T, S, false, false, SEG><<<(unsigned)blocks, Sh::THREADS, 0, stream>>>(
        q, ldq, m, (int32_t)pass.n_loc, tb, (int32_t)n_chunks, err, (T)-0.0, pass.rs, stall,
        seg.c_begin, seg.c_end, (T*)seg.state);
    return cudaGetLastError();
}

// The wave kernel over chunks [seg.c_begin, seg.c_end) of one pass, rows [0, m): the whole-pass
// kernel unless a segment is given.  `int_mul_rows`: the canonical FP64 form takes the
// integer-pipe products from this many rows of the launch on.
template <typename T, int S>
cudaError_t launch_wave_shape(T* Q, int64_t ldq, int64_t m, const ApplyPass& pass, const void* table, int* err,
                              cudaStream_t stream, const Seg& seg, int64_t int_mul_rows = kIntMulRows)
{
    if (seg.state != nullptr)
        return launch_wave_variant<T, S, true>(Q, ldq, m, pass, table, err, stream, seg, int_mul_rows);
    return launch_wave_variant<T, S, false>(Q, ldq, m, pass, table, err, stream, seg, int_mul_rows);
}

template <typename Tsrc, typename T, int S>
cudaError_t apply_pass_shape(T* Q, int64_t ldq, int64_t m, const Tsrc* grid, int64_t grid_rows,
                             const int32_t* place, const ApplyPass& pass, void* table, int* err,
                             cudaStream_t stream, cudaEvent_t ev_begin, cudaEvent_t ev_end, int what)
{
    if (pass.n_loc < 2 || pass.layers <= 0) return cudaSuccess;
    if (m <= 0 && what != kPassTable) return cudaSuccess;
    cudaError_t e;
    if (what & kPassTable) {
        e = prep_pass_shape<Tsrc, T, S>(grid, grid_rows, place, pass, table, stream);
        if (e != cudaSuccess) return e;
    }
    if (!(what & kPassWave)) return cudaSuccess;
    if (ev_begin) cudaEventRecord(ev_begin, stream);
    e = launch_wave_shape<T, S>(Q, ldq, m, pass, table, err, stream, Seg{});
    if (ev_end) cudaEventRecord(ev_end, stream);
    return e;
}

// The host-pointer apply of one pass of k <= 64 layers, streamed by column segments.  The
// caller's column-major Q (host memory, leading dimension lda) goes to the device buffer dQ
// (leading dimension m) in column chunks on io.s_in; the pass runs as io.nseg launches over
// consecutive chunk ranges of its table on `stream`, each waiting for the columns its chunks
// read (wave_tile: below c_end * CH + W) and carrying its registers to the next launch in
// io.state; the columns a launch finishes (below c_end * CH - (G-1) * W - KB, all of them after
// the last) go back on io.s_out as soon as it ends.  So the copies in both directions overlap
// the kernels, and every launch runs the whole m-row grid (the integer-pipe products and the
// one-CTA-per-SM shape need all rows together).  Only stream events order the three streams.
template <typename T, int S>
cudaError_t host_segmented_shape(T* dQ, int64_t m, const T* d_cs, const ApplyPass& pass, void* table, int* err,
                                 cudaStream_t stream, const HostStream& io)
{
    using Sh = typename Cfg<T, S>::Sh;
    const int64_t n = pass.n_loc;
    cudaError_t e = prep_pass_shape<T, T, S>(d_cs, n - 1, nullptr, pass, table, stream);
    if (e != cudaSuccess) return e;
    const int64_t n_chunks = Sh::chunks(n);
    const int nseg = (int)std::max<int64_t>(1, std::min<int64_t>(io.nseg, n_chunks));
    const size_t esz = sizeof(T);
    T* host = (T*)io.host;
    int64_t in_lo = 0, out_lo = 0;
    // copies in and kernels first, then the copies out: with pageable host memory a copy out
    // blocks the calling thread until it is done, and must not hold back the next copy in
    for (int j = 0; j < nseg; ++j) {
        const int64_t cb = (int64_t)j * n_chunks / nseg, ce = (int64_t)(j + 1) * n_chunks / nseg;
        const int64_t in_hi = std::min<int64_t>(n, ce * Sh::CH + Sh::W);
        if (in_hi > in_lo) {
            e = cudaMemcpy2DAsync(dQ + in_lo * m, m * esz, host + in_lo * io.lda, io.lda * esz, m * esz,
                                  in_hi - in_lo, cudaMemcpyHostToDevice, io.s_in);
            if (e != cudaSuccess) return e;
            in_lo = in_hi;
        }
        if ((e = cudaEventRecord(io.ev_in[j], io.s_in)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(stream, io.ev_in[j], 0)) != cudaSuccess) return e;
        Seg seg{(int32_t)cb, (int32_t)ce, io.state};
        e = launch_wave_shape<T, S>(dQ, m, m, pass, table, err, stream, seg, 0);
        if (e != cudaSuccess) return e;
        if ((e = cudaEventRecord(io.ev_seg[j], stream)) != cudaSuccess) return e;
    }
    for (int j = 0; j < nseg; ++j) {
        const int64_t ce = (int64_t)(j + 1) * n_chunks / nseg;
        const int64_t out_hi = (j == nseg - 1) ? n
            : std::max<int64_t>(0, std::min<int64_t>(n, ce * Sh::CH - (int64_t)(Sh::G - 1) * Sh::W - Sh::KB));
        if ((e = cudaStreamWaitEvent(io.s_out, io.ev_seg[j], 0)) != cudaSuccess) return e;
        if (out_hi > out_lo) {
            e = cudaMemcpy2DAsync(host + out_lo * io.lda, io.lda * esz, dQ + out_lo * m, m * esz, m * esz,
                                  out_hi - out_lo, cudaMemcpyDeviceToHost, io.s_out);
            if (e != cudaSuccess) return e;
            out_lo = out_hi;
        }
    }
    return cudaSuccess;
}

template <typename Tsrc, typename T>
cudaError_t apply_pass(T* Q, int64_t ldq, int64_t m, const Tsrc* grid, int64_t grid_rows,
                       const int32_t* place, const ApplyPass& pass, void* table, int* err,
                       cudaStream_t stream, cudaEvent_t ev_begin, cudaEvent_t ev_end, int what)
{
    const int s = resolve_shape<T>(m, pass.layers, pass.form);
    if constexpr (sizeof(T) == 8) {
        if (s == 2)
            return apply_pass_shape<Tsrc, T, 2>(Q, ldq, m, grid, grid_rows, place, pass, table, err,
                                                stream, ev_begin, ev_end, what);
        if (s == 3)
            return apply_pass_shape<Tsrc, T, 3>(Q, ldq, m, grid, grid_rows, place, pass, table, err,
                                                stream, ev_begin, ev_end, what);
    }
    if constexpr (sizeof(T) == 4) {
        if (s == 4)
            return apply_pass_shape<Tsrc, T, 4>(Q, ldq, m, grid, grid_rows, place, pass, table, err,
                                                stream, ev_begin, ev_end, what);
        if (s == 2)
            return apply_pass_shape<Tsrc, T, 2>(Q, ldq, m, grid, grid_rows, place, pass, table, err,
                                                stream, ev_begin, ev_end, what);
        if (s == 3)
            return apply_pass_shape<Tsrc, T, 3>(Q, ldq, m, grid, grid_rows, place, pass, table, err,
                                                stream, ev_begin, ev_end, what);
    }
    if (s == 0)
        return apply_pass_shape<Tsrc, T, 0>(Q, ldq, m, grid, grid_rows, place, pass, table, err,
                                            stream, ev_begin, ev_end, what);
    return apply_pass_shape<Tsrc, T, 1>(Q, ldq, m, grid, grid_rows, place, pass, table, err, stream,
                                        ev_begin, ev_end, what);
}

template <typename T>
cudaError_t apply_host_segmented(T* dQ, int64_t m, const T* d_cs, const ApplyPass& pass, void* table, int* err,
                                 cudaStream_t stream, const HostStream& io)
{
    if (pass.n_loc < 2 || pass.layers <= 0 || m <= 0) return cudaSuccess;
    if (pass.layers > 64 || pass.c0 != 0 || pass.L0 != 0) return cudaErrorInvalidValue;
    // segmented launches exist for FP64 shapes 0 and 2 and FP32 shapes 0, 1, 2 and 4 (every
    // shape the auto choice takes); other tunings take the unpipelined path
    const int s = resolve_shape<T>(m);
    if constexpr (sizeof(T) == 8) {
        if (s == 2) return host_segmented_shape<T, 2>(dQ, m, d_cs, pass, table, err, stream, io);
        if (s == 0) return host_segmented_shape<T, 0>(dQ, m, d_cs, pass, table, err, stream, io);
    } else {
        if (s == 4) return host_segmented_shape<T, 4>(dQ, m, d_cs, pass, table, err, stream, io);
        if (s == 2) return host_segmented_shape<T, 2>(dQ, m, d_cs, pass, table, err, stream, io);
        if (s == 1) return host_segmented_shape<T, 1>(dQ, m, d_cs, pass, table, err, stream, io);
        if (s == 0) return host_segmented_shape<T, 0>(dQ, m, d_cs, pass, table, err, stream, io);
    }
    return cudaErrorNotSupported;
}
// Whether apply_host_segmented takes the shape an m-row launch of T runs.
template <typename T> bool apply_host_segmented_supported(int64_t m)
{
    const int s = resolve_shape<T>(m);
    return sizeof(T) == 8 ? (s == 0 || s == 2) : (s != 3);
}
template bool apply_host_segmented_supported<double>(int64_t);
template bool apply_host_segmented_supported<float>(int64_t);
template cudaError_t apply_host_segmented<double>(double*, int64_t, const double*, const ApplyPass&, void*, int*,
                                                  cudaStream_t, const HostStream&);
template cudaError_t apply_host_segmented<float>(float*, int64_t, const float*, const ApplyPass&, void*, int*,
                                                 cudaStream_t, const HostStream&);

// Device memory the segment state of an m-row launch needs (the largest over the shapes).
template <typename T, int S> size_t state_bytes(int64_t m)
{
    using Sh = typename Cfg<T, S>::Sh;
    return (size_t)((m + Sh::ROWS - 1) / Sh::ROWS) * Sh::THREADS * wave::segment_state_values<Sh>() * sizeof(T);
}
template <typename T> size_t apply_segment_state_bytes(int64_t m)
{
    size_t b = std::max(state_bytes<T, 0>(m), state_bytes<T, 1>(m));
    b = std::max(b, state_bytes<T, 2>(m));
    if constexpr (sizeof(T) == 4) {
        b = std::max(b, state_bytes<T, 3>(m));
        b = std::max(b, state_bytes<T, 4>(m));
    }
    return b;
}
template size_t apply_segment_state_bytes<double>(int64_t);
template size_t apply_segment_state_bytes<float>(int64_t);

int apply_num_shapes(int fp64) { return kShapes[fp64 ? 0 : 1]; }
void apply_set_shape(int fp64, int shape)
{
    g_shape[fp64 ? 0 : 1] = (shape >= 0 && shape < apply_num_shapes(fp64)) ? shape : kAutoShape;
}
int apply_get_shape(int fp64) { return g_shape[fp64 ? 0 : 1]; }

template cudaError_t apply_pass<double, double>(double*, int64_t, int64_t, const double*, int64_t,
    const int32_t*, const ApplyPass&, void*, int*, cudaStream_t, cudaEvent_t, cudaEvent_t, int);
template cudaError_t apply_pass<float, float>(float*, int64_t, int64_t, const float*, int64_t,
    const int32_t*, const ApplyPass&, void*, int*, cudaStream_t, cudaEvent_t, cudaEvent_t, int);
template cudaError_t apply_pass<double, float>(float*, int64_t, int64_t, const double*, int64_t,
    const int32_t*, const ApplyPass&, void*, int*, cudaStream_t, cudaEvent_t, cudaEvent_t, int);

}  // namespace symeig
