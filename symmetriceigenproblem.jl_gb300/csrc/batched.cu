// batched.cu -- many independent eigensolves (qr_algorithm! on each of a batch of
// SymTridiagonal matrices of different orders) in one stream of persistent launches.
//
// The reference solves one matrix per call (src/bulge_chasing.jl:146).  A batch here runs
// in rounds; each round is one flush of every unfinished matrix:
//   1. chase: one lane per matrix runs the reference's inner loop until its rotation buffer
//      is full or it converges (chase.cu, chase_batched_kernel).  Lanes are assigned in
//      order of decreasing n so that a warp's 32 chases sweep similar lengths.
//   2. worklist (one CTA): for every matrix with rotations, the column range and layer
//      count of its flush, its number of row tiles, and exclusive prefix sums of tiles per
//      (pass, size class) -- the work queue of (matrix, row-tile) items -- and the number of
//      matrices still active.
//   3. per pass: one CTA per matrix builds the wave table; then a persistent wave kernel per
//      size class (grid = SMs x resident CTAs) pulls (matrix, row-tile) items from the
//      queue with an atomic counter and runs the wave tile of wave_common.cuh on them.
// Round r's apply (3) runs beside round r + 1's chase (1), with the rotation grids double
// buffered, and each round's work list, apply and next chase are captured once as a CUDA
// graph (one per buffer parity) that is replayed until no matrix is left.
// Q is FP64 (the canonical rotation with its products on the integer pipes) or FP32 (the
// FP32-Q variant: the chase stays FP64, each (c,s) is rounded to float).  The tile -- rows per
// tile and layers per pass (k) -- is chosen per size class and per precision of Q by the
// autotuner (symeig_batched_autotune) among three candidates.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <numeric>
#include <type_traits>
#include <vector>

#include "symeig.h"
#include "wave_common.cuh"

namespace symeig {
namespace {

using wave::Shape;
using wave::kThreads;

constexpr int kMaxPasses = 4;   // grid_layers <= 2 * 128 exact-order layers, passes of >= 64
constexpr int kClasses = 2;     // size classes: n <= split and n > split
constexpr int kTiles = 3;       // candidate tiles

// Candidate tiles (CTAs of 4 warps):
//   0: 8 lane groups of 8 layers  -- 64 layers per pass, 16 rows per tile;
//   1: 4 lane groups of 16 layers -- 64 layers per pass, 32 rows per tile;
//   2: 16 lane groups of 8 layers -- 128 layers per pass (a whole flush of the reference's
//      128-layer buffer in one pass), 8 rows per tile.
template <typename T, int S> struct TileOf;
template <typename T> struct TileOf<T, 0> { using type = Shape<T, 8, 8>; };
template <typename T> struct TileOf<T, 1> { using type = Shape<T, 16, 4>; };
template <typename T> struct TileOf<T, 2> { using type = Shape<T, 8, 16>; };

template <typename T>
__host__ __device__ inline int64_t tile_rows(int s)
{
    return s == 0 ? TileOf<T, 0>::type::ROWS : s == 1 ? TileOf<T, 1>::type::ROWS : TileOf<T, 2>::type::ROWS;
}
__host__ __device__ inline int64_t tile_layers(int s) { return s == 2 ? 128 : 64; }
template <typename T>
__host__ __device__ inline int64_t tile_table_bytes(int s, int64_t n_loc)
{
    return s == 0 ? TileOf<T, 0>::type::table_bytes(n_loc)
         : s == 1 ? TileOf<T, 1>::type::table_bytes(n_loc)
                  : TileOf<T, 2>::type::table_bytes(n_loc);
}

struct Work {
    int64_t c0;       // first column of the flush
    int64_t n_loc;    // columns of the flush
    int64_t bytes;    // table bytes of one pass
    int32_t passes;   // passes of the class's tile (64 or 128 layers)
    int32_t tiles;    // row tiles
};

struct Worklist {
    int64_t active;                              // matrices not finished after the chase
    int64_t total_tiles[kMaxPasses][kClasses];   // queue lengths
    int32_t next_tile[kMaxPasses][kClasses];     // queue heads (atomic)
};

// ---- 2. worklist -------------------------------------------------------------------------
__device__ int64_t block_exclusive_scan(int64_t v, int64_t* sh)
{
    // sh: blockDim.x entries of shared scratch; returns the exclusive prefix of v
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {
        const int64_t x = (t >= off) ? sh[t - off] : 0;
        __syncthreads();
        sh[t] += x;
        __syncthreads();
    }
    const int64_t incl = sh[t];
    __syncthreads();
    return incl - v;
}

template <typename T>
__global__ void __launch_bounds__(1024)
worklist_kernel(const BatchMat* __restrict__ mats, const ChaseState* __restrict__ states,
                int32_t count, const int32_t* __restrict__ shape_of_class,
                Work* __restrict__ work, int64_t* __restrict__ toff,
                int64_t* __restrict__ tile_prefix /* [kMaxPasses][kClasses][count+1] */,
                Worklist* __restrict__ wl)
{
    __shared__ int64_t sh[1024];
    const int t = threadIdx.x;
    const int per = (count + blockDim.x - 1) / blockDim.x;
    const int i0 = min(t * per, count), i1 = min(i0 + per, count);
    int64_t active = 0, bytes = 0;
    for (int i = i0; i < i1; ++i) {
        const ChaseState& st = states[i];
        Work w{0, 0, 0, 0, 0};
        if (st.status == CHASE_FLUSH || st.status == CHASE_RUNNING) active += 1;
        if (st.status == CHASE_FLUSH) {
            const int s = shape_of_class[mats[i].cls];
            w.c0 = st.min_from - 1;
            w.n_loc = st.max_to - w.c0;
            w.passes = (int32_t)((st.max_thickness + tile_layers(s) - 1) / tile_layers(s));
            w.tiles = (int32_t)((mats[i].n + tile_rows<T>(s) - 1) / tile_rows<T>(s));
            w.bytes = tile_table_bytes<T>(s, w.n_loc);
        }
        work[i] = w;
        bytes += w.bytes;
    }
    // table offsets (the same region serves every pass)
    int64_t off = block_exclusive_scan(bytes, sh);
    for (int i = i0; i < i1; ++i) {
        toff[i] = off;
        off += work[i].bytes;
    }
    const int64_t act = block_exclusive_scan(active, sh) + active;
    if (t == blockDim.x - 1) wl->active = act;
    // tile prefixes per (pass, class)
    for (int p = 0; p < kMaxPasses; ++p)
        for (int c = 0; c < kClasses; ++c) {
            int64_t* pre = tile_prefix + ((int64_t)p * kClasses + c) * (count + 1);
            int64_t mine = 0;
            for (int i = i0; i < i1; ++i)
                if (mats[i].cls == c && work[i].passes > p) mine += work[i].tiles;
            int64_t run = block_exclusive_scan(mine, sh);
            for (int i = i0; i < i1; ++i) {
                pre[i] = run;
                if (mats[i].cls == c && work[i].passes > p) run += work[i].tiles;
            }
            if (t == blockDim.x - 1) {
                pre[count] = run;
                wl->total_tiles[p][c] = run;
                wl->next_tile[p][c] = 0;
            }
        }
}

// ---- 3a. tables: one CTA per matrix --------------------------------------------------------
template <typename T, typename Sh>
__device__ void build_table_for(unsigned char* table, const Work& w, const double* grid,
                                int64_t grid_rows, const int32_t* place, int pass)
{
    const int64_t total = Sh::chunks(w.n_loc) * Sh::CH * Sh::G * Sh::KB;
    for (int64_t idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int64_t t = idx / (Sh::G * Sh::KB);
        const int g = (int)((idx / Sh::KB) % Sh::G);
        const int l = (int)(idx % Sh::KB);
        wave::table_entry<T, Sh, double>(table, t, g, l, grid, grid_rows, place, w.c0, w.n_loc,
                                         (int64_t)pass * Sh::LAYERS, Sh::LAYERS);
    }
}

template <typename T>
__global__ void __launch_bounds__(256)
batched_table_kernel(const BatchMat* __restrict__ mats, const Work* __restrict__ work,
                     const int64_t* __restrict__ toff, const int32_t* __restrict__ shape_of_class,
                     const double* __restrict__ grids, const int32_t* __restrict__ place,
                     unsigned char* __restrict__ tables, int pass)
{
    const int i = blockIdx.x;
    const Work w = work[i];
    if (w.passes <= pass) return;
    const BatchMat mt = mats[i];
    const int64_t rows = mt.n > 1 ? mt.n - 1 : 1;
    unsigned char* tb = tables + toff[i];
    const int s = shape_of_class[mt.cls];
    if (s == 0)
        build_table_for<T, typename TileOf<T, 0>::type>(tb, w, grids + mt.goff, rows, place + mt.doff, pass);
    else if (s == 1)
        build_table_for<T, typename TileOf<T, 1>::type>(tb, w, grids + mt.goff, rows, place + mt.doff, pass);
    else
        build_table_for<T, typename TileOf<T, 2>::type>(tb, w, grids + mt.goff, rows, place + mt.doff, pass);
}

// ---- 3b. persistent wave kernel of one (pass, class) ---------------------------------------
template <typename T, typename Sh>
__global__ void __launch_bounds__(kThreads)
batched_wave_kernel(const BatchMat* __restrict__ mats, const Work* __restrict__ work,
                    const int64_t* __restrict__ toff, const int64_t* __restrict__ prefix,
                    int32_t count, Worklist* __restrict__ wl, int pass, int cls,
                    T* __restrict__ Q, const unsigned char* __restrict__ tables,
                    int* __restrict__ err, const T nz)
{
    __shared__ __align__(128) unsigned char ring[2][Sh::CHUNK];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int32_t tile_sh;
    wave::Staging<Sh> st{ring, bar, 0, 0};
#ifdef SYMEIG_DEVICE_CHECKS
    st.check = err;
#endif
    wave::staging_init(st);
    const int64_t total = wl->total_tiles[pass][cls];
    for (;;) {
        if (threadIdx.x == 0) tile_sh = atomicAdd(&wl->next_tile[pass][cls], 1);
        __syncthreads();
        const int64_t tile = tile_sh;
        __syncthreads();
        if (tile >= total) break;
        // matrix of this tile: last i with prefix[i] <= tile
        int lo = 0, hi = count;  // prefix[lo] <= tile < prefix[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (prefix[mid] <= tile) lo = mid; else hi = mid;
        }
        const BatchMat mt = mats[lo];
        const Work w = work[lo];
        const int64_t row0 = (tile - prefix[lo]) * Sh::ROWS;
        T* q = Q + mt.qoff + w.c0 * mt.n;
        // FP64: the canonical rotation with its products on the integer pipes (int_mul.cuh)
        if (!wave::wave_tile<T, Sh, false, sizeof(T) == 8>(q, mt.n, mt.n, row0, (int32_t)w.n_loc, tables + toff[lo],
                                                           (int32_t)Sh::chunks(w.n_loc), nz, st)) {
            if (threadIdx.x == 0) atomicOr(err, 1);
            return;
        }
    }
}

int cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return SYMEIG_OK;
    if (e == cudaErrorMemoryAllocation) return SYMEIG_ERR_NOMEM;
    return SYMEIG_ERR_CUDA;
}

#define CKB(call)                                        \
    do {                                                 \
        cudaError_t _e = (call);                         \
        if (_e != cudaSuccess) { rc = cuda_status(_e); goto done; } \
    } while (0)

template <typename T, typename Sh>
int resident_ctas(int sm_count)
{
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batched_wave_kernel<T, Sh>, kThreads, 0) != cudaSuccess ||
        per < 1)
        per = 1;
    return per * sm_count;
}

// The persistent wave kernel of tile s over the queue of (pass, class).
template <typename T>
void launch_batched_wave(int s, int sms, const BatchMat* mats, const Work* work, const int64_t* toff,
                         const int64_t* pre, int32_t count, Worklist* wl, int pass, int cls, T* Q,
                         const unsigned char* tables, int* err, cudaStream_t stream)
{
    using S0 = typename TileOf<T, 0>::type;
    using S1 = typename TileOf<T, 1>::type;
    using S2 = typename TileOf<T, 2>::type;
    if (s == 0)
        batched_wave_kernel<T, S0><<<resident_ctas<T, S0>(sms), kThreads, 0, stream>>>(
            mats, work, toff, pre, count, wl, pass, cls, Q, tables, err, (T)-0.0);
    else if (s == 1)
        batched_wave_kernel<T, S1><<<resident_ctas<T, S1>(sms), kThreads, 0, stream>>>(
            mats, work, toff, pre, count, wl, pass, cls, Q, tables, err, (T)-0.0);
    else
        batched_wave_kernel<T, S2><<<resident_ctas<T, S2>(sms), kThreads, 0, stream>>>(
            mats, work, toff, pre, count, wl, pass, cls, Q, tables, err, (T)-0.0);
}

}  // namespace

// Size-class split and tile per class for the batched apply, per precision of Q ([0] FP64,
// [1] FP32); written by the autotuner.
struct BatchTuning {
    int64_t split = 256;          // class 0: n <= split, class 1: n > split
    int32_t shape[kClasses] = {0, 0};
};

static BatchTuning g_tuning[2];

void batched_set_tuning(int fp64, int64_t split, int32_t shape0, int32_t shape1)
{
    BatchTuning& t = g_tuning[fp64 ? 0 : 1];
    t.split = split;
    t.shape[0] = (shape0 >= 0 && shape0 < kTiles) ? shape0 : 0;
    t.shape[1] = (shape1 >= 0 && shape1 < kTiles) ? shape1 : 0;
}

void batched_get_tuning(int fp64, int64_t* split, int32_t* shape0, int32_t* shape1)
{
    const BatchTuning& t = g_tuning[fp64 ? 0 : 1];
    *split = t.split;
    *shape0 = t.shape[0];
    *shape1 = t.shape[1];
}

int batched_num_tiles() { return kTiles; }

// Device-pointer batched solve.  n, converged, iters are host arrays of `count` entries.
template <typename T>
int qr_batched_dev(int device, cudaStream_t stream, int64_t count, const int64_t* n, double* d,
                   double* e, T* Q, int32_t max_layers, double tol, int64_t maxiter_factor,
                   int32_t exact_order, int32_t* converged, int64_t* iters, int64_t* rounds_out,
                   double* ms_out)
{
    if (count <= 0) return SYMEIG_OK;
    if (count > (1 << 24)) return SYMEIG_ERR_SIZE;
    auto t0 = std::chrono::steady_clock::now();
    const int32_t grid_layers = exact_order ? 2 * max_layers : max_layers;
    if (grid_layers > kMaxPasses * 64) return SYMEIG_ERR_LAYERS;
    const BatchTuning tun = g_tuning[sizeof(T) == 8 ? 0 : 1];

    int rc = SYMEIG_OK;
    std::vector<BatchMat> mats(count);
    std::vector<ChaseState> states(count);
    int64_t doff = 0, eoff = 0, qoff = 0, goff = 0;
    int64_t table_cap = 0;
    for (int64_t i = 0; i < count; ++i) {
        const int64_t ni = n[i];
        if (ni < 1 || ni > (1 << 20)) return SYMEIG_ERR_SIZE;
        const int cls = ni <= tun.split ? 0 : 1;
        mats[i] = BatchMat{ni, doff, eoff, qoff, goff, cls, 0};
        doff += ni;
        eoff += ni > 1 ? ni - 1 : 0;
        qoff += ni * ni;
        goff += 2 * (ni > 1 ? ni - 1 : 1) * (int64_t)grid_layers;
        table_cap += tile_table_bytes<T>(tun.shape[cls], ni);
        ChaseState s{};
        s.n = ni;
        s.start = 1;
        s.last_block_ends_at = ni;
        s.maxiter = (maxiter_factor > 0 ? maxiter_factor : 100) * ni;
        s.tol = tol;
        s.max_layers = max_layers;
        s.grid_layers = grid_layers;
        s.exact_order = exact_order;
        s.status = CHASE_RUNNING;
        s.neg_zero = -0.0;
        states[i] = s;
    }
    // lanes in order of decreasing n (stable), so that a warp's chases have similar lengths
    std::vector<int32_t> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return n[a] > n[b]; });

    BatchMat* d_mats = nullptr;
    ChaseState* d_states = nullptr;
    int32_t* d_order = nullptr;
    int32_t* d_shape = nullptr;
    double* d_grids[2] = {nullptr, nullptr};
    int32_t* d_thick = nullptr;
    int32_t* d_place[2] = {nullptr, nullptr};
    Work* d_work = nullptr;
    int64_t* d_toff = nullptr;
    int64_t* d_prefix = nullptr;
    Worklist* d_wl = nullptr;
    unsigned char* d_tables = nullptr;
    int* d_err = nullptr;
    Worklist* h_wl = nullptr;
    cudaGraph_t graph[2] = {nullptr, nullptr};
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int64_t rounds = 0;
    const bool want_q = Q != nullptr;
    int sms = 0;
    CKB(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    CKB(cudaMalloc(&d_mats, sizeof(BatchMat) * count));
    CKB(cudaMalloc(&d_states, sizeof(ChaseState) * count));
    CKB(cudaMalloc(&d_order, sizeof(int32_t) * count));
    CKB(cudaMalloc(&d_shape, sizeof(int32_t) * kClasses));
    for (int b = 0; b < 2; ++b) {
        CKB(cudaMalloc(&d_grids[b], sizeof(double) * goff));
        CKB(cudaMalloc(&d_place[b], sizeof(int32_t) * doff));
    }
    CKB(cudaMalloc(&d_thick, sizeof(int32_t) * doff));
    CKB(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    CKB(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    CKB(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    CKB(cudaMalloc(&d_work, sizeof(Work) * count));
    CKB(cudaMalloc(&d_toff, sizeof(int64_t) * count));
    CKB(cudaMalloc(&d_prefix, sizeof(int64_t) * kMaxPasses * kClasses * (count + 1)));
    CKB(cudaMalloc(&d_wl, sizeof(Worklist)));
    CKB(cudaMalloc(&d_tables, std::max<int64_t>(table_cap, 256)));
    CKB(cudaMalloc(&d_err, sizeof(int)));
    CKB(cudaMallocHost(&h_wl, sizeof(Worklist)));
    CKB(cudaMemcpyAsync(d_mats, mats.data(), sizeof(BatchMat) * count, cudaMemcpyHostToDevice, stream));
    CKB(cudaMemcpyAsync(d_states, states.data(), sizeof(ChaseState) * count, cudaMemcpyHostToDevice, stream));
    CKB(cudaMemcpyAsync(d_order, order.data(), sizeof(int32_t) * count, cudaMemcpyHostToDevice, stream));
    CKB(cudaMemcpyAsync(d_shape, tun.shape, sizeof(int32_t) * kClasses, cudaMemcpyHostToDevice, stream));
    CKB(cudaMemsetAsync(d_err, 0, sizeof(int), stream));
    CKB(cudaStreamSynchronize(stream));

    {
        // Rounds are pipelined: round r's apply (its rotations in grid buffer r % 2) runs beside
        // round r + 1's chase (into the other buffer).  The chase never reads Q and the apply
        // never reads the chase states: the work list snapshots round r's flushes before the
        // next chase starts.  The lane-per-matrix chase is as long as the batch's largest
        // sweeps and holds few warps, the apply fills the GPU, so the two overlap well.
        // Round 0's chase runs first; graph b (b = r % 2) then runs, per round r,
        //   work list (round r) -> [ tables + wave passes on buffer b  ||  chase into buffer 1-b ]
        // and copies the number of matrices still active after chase r to the host.  The loop
        // ends at the first round with none: its chase (of converged matrices) returns at once.
        CKB(launch_chase_batched(d_mats, d_order, (int32_t)count, d_states, d, e, d_grids[0], d_thick,
                                 d_place[0], stream));
        for (int b = 0; b < 2; ++b) {
            CKB(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            worklist_kernel<T><<<1, 1024, 0, stream>>>(d_mats, d_states, (int32_t)count, d_shape, d_work,
                                                       d_toff, d_prefix, d_wl);
            cudaEventRecord(ev_fork, stream);
            cudaStreamWaitEvent(side, ev_fork, 0);
            cudaError_t ce = launch_chase_batched(d_mats, d_order, (int32_t)count, d_states, d, e,
                                                  d_grids[1 - b], d_thick, d_place[1 - b], side);
            cudaEventRecord(ev_join, side);
            if (want_q) {
                // passes of 64-layer tiles: up to kMaxPasses; of the 128-layer tile: half as many
                const int passes = std::max(tile_layers(tun.shape[0]) == 64 ? kMaxPasses : kMaxPasses / 2,
                                            tile_layers(tun.shape[1]) == 64 ? kMaxPasses : kMaxPasses / 2);
                for (int p = 0; p < passes; ++p) {
                    batched_table_kernel<T><<<(unsigned)count, 256, 0, stream>>>(
                        d_mats, d_work, d_toff, d_shape, d_grids[b], d_place[b], d_tables, p);
                    for (int c = 0; c < kClasses; ++c) {
                        if (p >= (tile_layers(tun.shape[c]) == 64 ? kMaxPasses : kMaxPasses / 2)) continue;
                        const int64_t* pre = d_prefix + ((int64_t)p * kClasses + c) * (count + 1);
                        launch_batched_wave<T>(tun.shape[c], sms, d_mats, d_work, d_toff, pre, (int32_t)count,
                                               d_wl, p, c, Q, d_tables, d_err, stream);
                    }
                }
            }
            cudaStreamWaitEvent(stream, ev_join, 0);
            cudaMemcpyAsync(h_wl, d_wl, sizeof(Worklist), cudaMemcpyDeviceToHost, stream);
            cudaError_t end = cudaStreamEndCapture(stream, &graph[b]);
            if (ce != cudaSuccess) { rc = cuda_status(ce); goto done; }
            CKB(end);
            CKB(cudaGetLastError());
            CKB(cudaGraphInstantiate(&exec[b], graph[b], 0));
        }
        for (;;) {
            CKB(cudaGraphLaunch(exec[rounds & 1], stream));
            CKB(cudaStreamSynchronize(stream));
            rounds += 1;
            if (h_wl->active == 0) break;
            if (rounds > (int64_t)1 << 24) { rc = SYMEIG_ERR_DEVICE; goto done; }
        }
        int herr = 0;
        CKB(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (herr) { rc = (herr & 2) ? SYMEIG_ERR_DEVICE : SYMEIG_ERR_TIMEOUT; goto done; }
        CKB(cudaMemcpy(states.data(), d_states, sizeof(ChaseState) * count, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < count; ++i) {
            if (converged) converged[i] = states[i].status == CHASE_MAXITER ? 0 : 1;
            if (iters) iters[i] = states[i].iter;
        }
    }
done:
    for (int b = 0; b < 2; ++b) {
        if (exec[b]) cudaGraphExecDestroy(exec[b]);
        if (graph[b]) cudaGraphDestroy(graph[b]);
        cudaFree(d_grids[b]);
        cudaFree(d_place[b]);
    }
    if (side) {
        cudaStreamSynchronize(side);
        cudaStreamDestroy(side);
    }
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    cudaFree(d_mats); cudaFree(d_states); cudaFree(d_order); cudaFree(d_shape);
    cudaFree(d_thick); cudaFree(d_work); cudaFree(d_toff);
    cudaFree(d_prefix); cudaFree(d_wl); cudaFree(d_tables); cudaFree(d_err);
    if (h_wl) cudaFreeHost(h_wl);
    if (rounds_out) *rounds_out = rounds;
    if (ms_out) *ms_out = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}
template int qr_batched_dev<double>(int, cudaStream_t, int64_t, const int64_t*, double*, double*, double*,
                                    int32_t, double, int64_t, int32_t, int32_t*, int64_t*, int64_t*, double*);
template int qr_batched_dev<float>(int, cudaStream_t, int64_t, const int64_t*, double*, double*, float*,
                                   int32_t, double, int64_t, int32_t, int32_t*, int64_t*, int64_t*, double*);

// ---- autotuner ---------------------------------------------------------------------------
namespace {

__global__ void fill_grid_kernel(double* grid, int64_t pairs, uint64_t seed)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < pairs;
         k += (int64_t)gridDim.x * blockDim.x) {
        uint64_t x = (uint64_t)k * 0x9E3779B97F4A7C15ull + seed;
        x ^= x >> 31; x *= 0xBF58476D1CE4E5B9ull; x ^= x >> 27;
        const double th = (double)(x >> 11) * 0x1p-53 * 6.283185307179586;
        grid[2 * k] = cos(th);
        grid[2 * k + 1] = sin(th);
    }
}

__global__ void fill_int_kernel(int32_t* a, int64_t n, int32_t v)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) a[k] = v;
}

// Time the batched apply of one full flush (128 layers: two passes of a 64-layer tile, one of
// the 128-layer tile; table builds included) with tile `sh` on matrices of the orders in
// `sizes`, all in class c; the best of two repetitions after one warm-up, in ms.  Returns a
// CUDA error or success.
template <typename T>
cudaError_t time_tile(int sms, cudaStream_t stream, int c, int sh, const std::vector<int64_t>& sizes, float* out)
{
    const int64_t count = (int64_t)sizes.size();
    std::vector<BatchMat> mats(count);
    std::vector<Work> work(count);
    std::vector<int64_t> toff(count), pre(kMaxPasses * kClasses * (count + 1), 0);
    Worklist wl{};
    const int64_t gl = 128;   // one 128-layer flush
    const int passes = (int)(128 / tile_layers(sh));
    int64_t tb = 0, doff = 0, qoff = 0, goff = 0;
    for (int64_t i = 0; i < count; ++i) {
        const int64_t n = sizes[i];
        mats[i] = BatchMat{n, doff, 0, qoff, goff, c, 0};
        work[i] = Work{0, n, tile_table_bytes<T>(sh, n), passes, (int32_t)((n + tile_rows<T>(sh) - 1) / tile_rows<T>(sh))};
        toff[i] = tb;
        tb += work[i].bytes;
        doff += n;
        qoff += n * n;
        goff += 2 * (n - 1) * gl;
    }
    for (int p = 0; p < passes; ++p) {
        int64_t* q = pre.data() + ((int64_t)p * kClasses + c) * (count + 1);
        for (int64_t i = 0; i < count; ++i) q[i + 1] = q[i] + work[i].tiles;
        wl.total_tiles[p][c] = q[count];
    }
    int32_t shapes[kClasses] = {sh, sh};
    BatchMat* d_mats = nullptr; Work* d_work = nullptr; int64_t* d_toff = nullptr;
    int64_t* d_pre = nullptr; Worklist* d_wl = nullptr; int32_t* d_shape = nullptr;
    double* d_grid = nullptr; int32_t* d_place = nullptr; T* d_q = nullptr;
    unsigned char* d_tab = nullptr; int* d_err = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t er = cudaSuccess;
    auto ck = [&](cudaError_t x) { if (er == cudaSuccess) er = x; };
    ck(cudaMalloc(&d_mats, sizeof(BatchMat) * count));
    ck(cudaMalloc(&d_work, sizeof(Work) * count));
    ck(cudaMalloc(&d_toff, sizeof(int64_t) * count));
    ck(cudaMalloc(&d_pre, sizeof(int64_t) * pre.size()));
    ck(cudaMalloc(&d_wl, sizeof(Worklist)));
    ck(cudaMalloc(&d_shape, sizeof(shapes)));
    ck(cudaMalloc(&d_grid, sizeof(double) * goff));
    ck(cudaMalloc(&d_place, sizeof(int32_t) * doff));
    ck(cudaMalloc(&d_q, sizeof(T) * qoff));
    ck(cudaMalloc(&d_tab, tb));
    ck(cudaMalloc(&d_err, sizeof(int)));
    ck(cudaEventCreate(&e0));
    ck(cudaEventCreate(&e1));
    float t = 1e30f;
    if (er == cudaSuccess) {
        ck(cudaMemcpyAsync(d_mats, mats.data(), sizeof(BatchMat) * count, cudaMemcpyHostToDevice, stream));
        ck(cudaMemcpyAsync(d_work, work.data(), sizeof(Work) * count, cudaMemcpyHostToDevice, stream));
        ck(cudaMemcpyAsync(d_toff, toff.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, stream));
        ck(cudaMemcpyAsync(d_pre, pre.data(), sizeof(int64_t) * pre.size(), cudaMemcpyHostToDevice, stream));
        ck(cudaMemcpyAsync(d_shape, shapes, sizeof(shapes), cudaMemcpyHostToDevice, stream));
        ck(cudaMemsetAsync(d_q, 0, sizeof(T) * qoff, stream));
        ck(cudaMemsetAsync(d_err, 0, sizeof(int), stream));
        fill_grid_kernel<<<sms * 4, 256, 0, stream>>>(d_grid, goff / 2, 1234 + c);
        fill_int_kernel<<<sms, 256, 0, stream>>>(d_place, doff, 128);
        for (int rep = 0; rep < 3 && er == cudaSuccess; ++rep) {
            ck(cudaMemcpyAsync(d_wl, &wl, sizeof(Worklist), cudaMemcpyHostToDevice, stream));
            ck(cudaEventRecord(e0, stream));
            for (int p = 0; p < passes; ++p) {
                batched_table_kernel<T><<<(unsigned)count, 256, 0, stream>>>(d_mats, d_work, d_toff, d_shape, d_grid,
                                                                            d_place, d_tab, p);
                const int64_t* q = d_pre + ((int64_t)p * kClasses + c) * (count + 1);
                launch_batched_wave<T>(sh, sms, d_mats, d_work, d_toff, q, (int32_t)count, d_wl, p, c, d_q, d_tab,
                                       d_err, stream);
            }
            ck(cudaEventRecord(e1, stream));
            ck(cudaEventSynchronize(e1));
            float x = 0.f;
            ck(cudaEventElapsedTime(&x, e0, e1));
            if (rep > 0 && x < t) t = x;
        }
        ck(cudaGetLastError());
    }
    cudaFree(d_mats); cudaFree(d_work); cudaFree(d_toff); cudaFree(d_pre); cudaFree(d_wl);
    cudaFree(d_shape); cudaFree(d_grid); cudaFree(d_place); cudaFree(d_q); cudaFree(d_tab);
    cudaFree(d_err);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    *out = t;
    return er;
}

// The matrices the autotuner times for class c: the caller's orders in that class (n, count),
// thinned evenly so that their Q stays within kTuneBytes, or, with none given, a spread of
// orders over the class (class 0: 2048 matrices, n from 32 to the split; class 1: 512
// matrices, n from split + 1 to 4 * split).
constexpr int64_t kTuneBytes = (int64_t)3 << 29;   // 1.5 GiB of FP64 Q per class

std::vector<int64_t> tune_sizes(int c, int64_t split, int64_t count, const int64_t* n)
{
    std::vector<int64_t> mine;
    for (int64_t i = 0; i < count && n; ++i)
        if (n[i] >= 2 && (c == 0 ? n[i] <= split : n[i] > split)) mine.push_back(n[i]);
    if (mine.empty()) {
        const int64_t lo = c == 0 ? std::min<int64_t>(32, split) : split + 1, hi = c == 0 ? split : 4 * split;
        const int64_t k = c == 0 ? 2048 : 512;
        for (int64_t i = 0; i < k; ++i) mine.push_back(std::max<int64_t>(2, lo + (hi - lo) * i / (k - 1)));
    }
    int64_t bytes = 0;
    for (int64_t v : mine) bytes += v * v * 8;
    if (bytes > kTuneBytes) {
        // keep every step-th matrix
        const int64_t step = (bytes + kTuneBytes - 1) / kTuneBytes;
        std::vector<int64_t> thin;
        for (size_t i = 0; i < mine.size(); i += (size_t)step) thin.push_back(mine[i]);
        mine.swap(thin);
    }
    return mine;
}

}  // namespace

// For each precision of Q and each size class, time every candidate tile on a batch of that
// class (a full 128-layer flush of every matrix) and keep the fastest: rows per tile and
// layers per pass (k) are chosen per (n, dtype).  The batch is the caller's orders (count, n;
// n may be NULL for a spread of orders over each class).  ms[(dtype * kClasses + c) * kTiles
// + s] receives the time of tile s on class c's batch, dtype 0 = FP64 Q, 1 = FP32 Q.
int batched_autotune(int device, cudaStream_t stream, int64_t count, const int64_t* n, double* ms)
{
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return SYMEIG_ERR_CUDA;
    for (int dt = 0; dt < 2; ++dt) {
        for (int c = 0; c < kClasses; ++c) {
            const std::vector<int64_t> sizes = tune_sizes(c, g_tuning[dt].split, count, n);
            float best = 1e30f;
            int best_s = 0;
            for (int sh = 0; sh < kTiles; ++sh) {
                float t = 0.f;
                const cudaError_t er = dt == 0 ? time_tile<double>(sms, stream, c, sh, sizes, &t)
                                               : time_tile<float>(sms, stream, c, sh, sizes, &t);
                if (er != cudaSuccess) return cuda_status(er);
                if (ms) ms[(dt * kClasses + c) * kTiles + sh] = t;
                if (t < best) {
                    best = t;
                    best_s = sh;
                }
            }
            g_tuning[dt].shape[c] = best_s;
        }
    }
    return SYMEIG_OK;
}

}  // namespace symeig
