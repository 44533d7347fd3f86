// batched.cu -- many independent eigensolves (qr_algorithm! on each of a batch of
// SymTridiagonal matrices of different orders) in one stream of persistent launches.
//
// The reference solves one matrix per call (src/bulge_chasing.jl:146).  A batch here runs
// in rounds; each round is one flush of every unfinished matrix and is captured once as a
// CUDA graph that is replayed until no matrix is left:
//   1. chase: one lane per matrix runs the reference's inner loop until its rotation buffer
//      is full or it converges (chase.cu, chase_batched_kernel).  Lanes are assigned in
//      order of decreasing n so that a warp's 32 chases sweep similar lengths.
//   2. worklist (one CTA): for every matrix with rotations, the column range and layer
//      count of its flush, its number of row tiles, and exclusive prefix sums of tiles per
//      (pass, size class) -- the work queue of (matrix, row-tile) items.
//   3. per pass of 64 layers: one CTA per matrix builds the wave table; then a persistent
//      wave kernel per size class (grid = SMs x resident CTAs) pulls (matrix, row-tile)
//      items from the queue with an atomic counter and runs the wave tile of
//      wave_common.cuh on them.
//   4. the number of unfinished matrices is copied to pinned host memory.
// The shape of the wave tile (rows per tile, layers per lane group) is chosen per size
// class by the autotuner (symeig_batched_autotune) among shapes with 64 layers per pass.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <numeric>
#include <vector>

#include "symeig.h"
#include "wave_common.cuh"

namespace symeig {
namespace {

using wave::Shape;
using wave::kThreads;

constexpr int kPassLayers = 64;
constexpr int kMaxPasses = 4;   // grid_layers <= 2 * 128 exact-order layers
constexpr int kClasses = 2;     // size classes: n <= split and n > split

// candidate shapes, all 64 layers per pass
using ShapeA = Shape<double, 8, 8>;    // 16 rows per tile
using ShapeB = Shape<double, 16, 4>;   // 32 rows per tile

template <int S> struct ShapeOf;
template <> struct ShapeOf<0> { using type = ShapeA; };
template <> struct ShapeOf<1> { using type = ShapeB; };

__host__ __device__ inline int64_t shape_rows(int s) { return s == 0 ? ShapeA::ROWS : ShapeB::ROWS; }
__host__ __device__ inline int64_t shape_table_bytes(int s, int64_t n_loc)
{
    return s == 0 ? ShapeA::table_bytes(n_loc) : ShapeB::table_bytes(n_loc);
}

struct Work {
    int64_t c0;       // first column of the flush
    int64_t n_loc;    // columns of the flush
    int64_t bytes;    // table bytes of one pass
    int32_t passes;   // passes of 64 layers
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
            w.passes = (int32_t)((st.max_thickness + kPassLayers - 1) / kPassLayers);
            w.tiles = (int32_t)((mats[i].n + shape_rows(s) - 1) / shape_rows(s));
            w.bytes = shape_table_bytes(s, w.n_loc);
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
template <typename Sh>
__device__ void build_table_for(unsigned char* table, const Work& w, const double* grid,
                                int64_t grid_rows, const int32_t* place, int pass)
{
    const int64_t total = Sh::chunks(w.n_loc) * Sh::CH * Sh::G * Sh::KB;
    for (int64_t idx = threadIdx.x; idx < total; idx += blockDim.x) {
        const int64_t t = idx / (Sh::G * Sh::KB);
        const int g = (int)((idx / Sh::KB) % Sh::G);
        const int l = (int)(idx % Sh::KB);
        wave::table_entry<double, Sh, double>(table, t, g, l, grid, grid_rows, place, w.c0, w.n_loc,
                                              (int64_t)pass * kPassLayers, kPassLayers);
    }
}

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
    if (shape_of_class[mt.cls] == 0)
        build_table_for<ShapeA>(tb, w, grids + mt.goff, rows, place + mt.doff, pass);
    else
        build_table_for<ShapeB>(tb, w, grids + mt.goff, rows, place + mt.doff, pass);
}

// ---- 3b. persistent wave kernel of one (pass, class) ---------------------------------------
template <typename Sh>
__global__ void __launch_bounds__(kThreads)
batched_wave_kernel(const BatchMat* __restrict__ mats, const Work* __restrict__ work,
                    const int64_t* __restrict__ toff, const int64_t* __restrict__ prefix,
                    int32_t count, Worklist* __restrict__ wl, int pass, int cls,
                    double* __restrict__ Q, const unsigned char* __restrict__ tables,
                    int* __restrict__ err, const double nz)
{
    __shared__ __align__(128) unsigned char ring[2][Sh::CHUNK];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int32_t tile_sh;
    wave::Staging<Sh> st{ring, bar, 0, 0};
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
        double* q = Q + mt.qoff + w.c0 * mt.n;
        // the canonical rotation with its products on the integer pipes (int_mul.cuh)
        if (!wave::wave_tile<double, Sh, false, true>(q, mt.n, mt.n, row0, (int32_t)w.n_loc, tables + toff[lo],
                                                      (int32_t)Sh::chunks(w.n_loc), nz, st)) {
            if (threadIdx.x == 0) atomicExch(err, 1);
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

template <typename Sh>
int resident_ctas(int sm_count)
{
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batched_wave_kernel<Sh>, kThreads, 0) != cudaSuccess || per < 1)
        per = 1;
    return per * sm_count;
}

}  // namespace

// Size-class split and tile shape per class for the batched apply; written by the autotuner.
struct BatchTuning {
    int64_t split = 256;          // class 0: n <= split, class 1: n > split
    int32_t shape[kClasses] = {0, 0};
};

static BatchTuning g_tuning;

void batched_set_tuning(int64_t split, int32_t shape0, int32_t shape1)
{
    g_tuning.split = split;
    g_tuning.shape[0] = shape0 & 1;
    g_tuning.shape[1] = shape1 & 1;
}

void batched_get_tuning(int64_t* split, int32_t* shape0, int32_t* shape1)
{
    *split = g_tuning.split;
    *shape0 = g_tuning.shape[0];
    *shape1 = g_tuning.shape[1];
}

// Device-pointer batched solve.  n, converged, iters are host arrays of `count` entries.
int qr_batched_dev(int device, cudaStream_t stream, int64_t count, const int64_t* n, double* d,
                   double* e, double* Q, int32_t max_layers, double tol, int64_t maxiter_factor,
                   int32_t exact_order, int32_t* converged, int64_t* iters, int64_t* rounds_out,
                   double* ms_out)
{
    if (count <= 0) return SYMEIG_OK;
    if (count > (1 << 24)) return SYMEIG_ERR_SIZE;
    (void)device;
    auto t0 = std::chrono::steady_clock::now();
    const int32_t grid_layers = exact_order ? 2 * max_layers : max_layers;
    if (grid_layers > kMaxPasses * kPassLayers) return SYMEIG_ERR_LAYERS;

    int rc = SYMEIG_OK;
    std::vector<BatchMat> mats(count);
    std::vector<ChaseState> states(count);
    int64_t doff = 0, eoff = 0, qoff = 0, goff = 0;
    int64_t table_cap = 0;
    for (int64_t i = 0; i < count; ++i) {
        const int64_t ni = n[i];
        if (ni < 1 || ni > (1 << 20)) return SYMEIG_ERR_SIZE;
        const int cls = ni <= g_tuning.split ? 0 : 1;
        mats[i] = BatchMat{ni, doff, eoff, qoff, goff, cls, 0};
        doff += ni;
        eoff += ni > 1 ? ni - 1 : 0;
        qoff += ni * ni;
        goff += 2 * (ni > 1 ? ni - 1 : 1) * (int64_t)grid_layers;
        table_cap += shape_table_bytes(g_tuning.shape[cls], ni);
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
    double* d_grids = nullptr;
    int32_t* d_thick = nullptr;
    int32_t* d_place = nullptr;
    Work* d_work = nullptr;
    int64_t* d_toff = nullptr;
    int64_t* d_prefix = nullptr;
    Worklist* d_wl = nullptr;
    unsigned char* d_tables = nullptr;
    int* d_err = nullptr;
    Worklist* h_wl = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t rounds = 0;
    const bool want_q = Q != nullptr;
    int sms = 0;
    CKB(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    CKB(cudaMalloc(&d_mats, sizeof(BatchMat) * count));
    CKB(cudaMalloc(&d_states, sizeof(ChaseState) * count));
    CKB(cudaMalloc(&d_order, sizeof(int32_t) * count));
    CKB(cudaMalloc(&d_shape, sizeof(int32_t) * kClasses));
    CKB(cudaMalloc(&d_grids, sizeof(double) * goff));
    CKB(cudaMalloc(&d_thick, sizeof(int32_t) * doff));
    CKB(cudaMalloc(&d_place, sizeof(int32_t) * doff));
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
    CKB(cudaMemcpyAsync(d_shape, g_tuning.shape, sizeof(int32_t) * kClasses, cudaMemcpyHostToDevice, stream));
    CKB(cudaMemsetAsync(d_err, 0, sizeof(int), stream));
    CKB(cudaStreamSynchronize(stream));

    {
        // capture one round
        const int ctasA = resident_ctas<ShapeA>(sms), ctasB = resident_ctas<ShapeB>(sms);
        CKB(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        {
            cudaError_t ce = launch_chase_batched(d_mats, d_order, (int32_t)count, d_states, d, e,
                                                  d_grids, d_thick, d_place, stream);
            worklist_kernel<<<1, 1024, 0, stream>>>(d_mats, d_states, (int32_t)count, d_shape, d_work,
                                                    d_toff, d_prefix, d_wl);
            if (want_q) {
                for (int p = 0; p < kMaxPasses; ++p) {
                    batched_table_kernel<<<(unsigned)count, 256, 0, stream>>>(
                        d_mats, d_work, d_toff, d_shape, d_grids, d_place, d_tables, p);
                    for (int c = 0; c < kClasses; ++c) {
                        const int64_t* pre = d_prefix + ((int64_t)p * kClasses + c) * (count + 1);
                        if (g_tuning.shape[c] == 0)
                            batched_wave_kernel<ShapeA><<<ctasA, kThreads, 0, stream>>>(
                                d_mats, d_work, d_toff, pre, (int32_t)count, d_wl, p, c, Q, d_tables, d_err, -0.0);
                        else
                            batched_wave_kernel<ShapeB><<<ctasB, kThreads, 0, stream>>>(
                                d_mats, d_work, d_toff, pre, (int32_t)count, d_wl, p, c, Q, d_tables, d_err, -0.0);
                    }
                }
            }
            cudaMemcpyAsync(h_wl, d_wl, sizeof(Worklist), cudaMemcpyDeviceToHost, stream);
            cudaError_t end = cudaStreamEndCapture(stream, &graph);
            if (ce != cudaSuccess) { rc = cuda_status(ce); goto done; }
            CKB(end);
            CKB(cudaGetLastError());
        }
        CKB(cudaGraphInstantiate(&exec, graph, 0));
        for (;;) {
            CKB(cudaGraphLaunch(exec, stream));
            CKB(cudaStreamSynchronize(stream));
            rounds += 1;
            if (h_wl->active == 0) break;
            if (rounds > (int64_t)1 << 24) { rc = SYMEIG_ERR_DEVICE; goto done; }
        }
        int herr = 0;
        CKB(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (herr) { rc = SYMEIG_ERR_TIMEOUT; goto done; }
        CKB(cudaMemcpy(states.data(), d_states, sizeof(ChaseState) * count, cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < count; ++i) {
            if (converged) converged[i] = states[i].status == CHASE_MAXITER ? 0 : 1;
            if (iters) iters[i] = states[i].iter;
        }
    }
done:
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaFree(d_mats); cudaFree(d_states); cudaFree(d_order); cudaFree(d_shape);
    cudaFree(d_grids); cudaFree(d_thick); cudaFree(d_place); cudaFree(d_work); cudaFree(d_toff);
    cudaFree(d_prefix); cudaFree(d_wl); cudaFree(d_tables); cudaFree(d_err);
    if (h_wl) cudaFreeHost(h_wl);
    if (rounds_out) *rounds_out = rounds;
    if (ms_out) *ms_out = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

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

}  // namespace

// Time the batched apply (table build + persistent wave kernel, 2 passes of 64 layers) of
// each candidate tile shape on a synthetic batch of each size class; keep the faster shape
// per class.  ms[c*2 + s] receives the time of shape s on class c's batch.
int batched_autotune(int device, cudaStream_t stream, double* ms)
{
    int rc = SYMEIG_OK;
    int sms = 0;
    const int64_t rep_n[kClasses] = {160, 640};
    const int64_t rep_count[kClasses] = {512, 32};
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return SYMEIG_ERR_CUDA;
    for (int c = 0; c < kClasses; ++c) {
        const int64_t n = rep_n[c], count = rep_count[c];
        double best = 1e30;
        int best_s = 0;
        for (int sh = 0; sh < 2; ++sh) {
            std::vector<BatchMat> mats(count);
            std::vector<Work> work(count);
            std::vector<int64_t> toff(count), pre(kMaxPasses * kClasses * (count + 1), 0);
            Worklist wl{};
            const int64_t gl = 256;
            int64_t tb = 0;
            for (int64_t i = 0; i < count; ++i) {
                mats[i] = BatchMat{n, i * n, i * (n - 1), i * n * n, i * 2 * (n - 1) * gl, c, 0};
                work[i] = Work{0, n, shape_table_bytes(sh, n), 2, (int32_t)((n + shape_rows(sh) - 1) / shape_rows(sh))};
                toff[i] = tb;
                tb += work[i].bytes;
            }
            for (int p = 0; p < 2; ++p) {
                int64_t* q = pre.data() + ((int64_t)p * kClasses + c) * (count + 1);
                for (int64_t i = 0; i < count; ++i) q[i + 1] = q[i] + work[i].tiles;
                wl.total_tiles[p][c] = q[count];
            }
            int32_t shapes[kClasses] = {sh, sh};
            BatchMat* d_mats = nullptr; Work* d_work = nullptr; int64_t* d_toff = nullptr;
            int64_t* d_pre = nullptr; Worklist* d_wl = nullptr; int32_t* d_shape = nullptr;
            double* d_grid = nullptr; int32_t* d_place = nullptr; double* d_q = nullptr;
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
            ck(cudaMalloc(&d_grid, sizeof(double) * count * 2 * (n - 1) * gl));
            ck(cudaMalloc(&d_place, sizeof(int32_t) * count * n));
            ck(cudaMalloc(&d_q, sizeof(double) * count * n * n));
            ck(cudaMalloc(&d_tab, tb));
            ck(cudaMalloc(&d_err, sizeof(int)));
            ck(cudaEventCreate(&e0));
            ck(cudaEventCreate(&e1));
            if (er == cudaSuccess) {
                ck(cudaMemcpyAsync(d_mats, mats.data(), sizeof(BatchMat) * count, cudaMemcpyHostToDevice, stream));
                ck(cudaMemcpyAsync(d_work, work.data(), sizeof(Work) * count, cudaMemcpyHostToDevice, stream));
                ck(cudaMemcpyAsync(d_toff, toff.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice, stream));
                ck(cudaMemcpyAsync(d_pre, pre.data(), sizeof(int64_t) * pre.size(), cudaMemcpyHostToDevice, stream));
                ck(cudaMemcpyAsync(d_shape, shapes, sizeof(shapes), cudaMemcpyHostToDevice, stream));
                ck(cudaMemsetAsync(d_q, 0, sizeof(double) * count * n * n, stream));
                ck(cudaMemsetAsync(d_err, 0, sizeof(int), stream));
                fill_grid_kernel<<<sms * 4, 256, 0, stream>>>(d_grid, count * (n - 1) * gl, 1234 + c);
                fill_int_kernel<<<sms, 256, 0, stream>>>(d_place, count * n, 128);
                const int ctas = sh == 0 ? resident_ctas<ShapeA>(sms) : resident_ctas<ShapeB>(sms);
                float t = 1e30f;
                for (int rep = 0; rep < 3 && er == cudaSuccess; ++rep) {
                    ck(cudaMemcpyAsync(d_wl, &wl, sizeof(Worklist), cudaMemcpyHostToDevice, stream));
                    ck(cudaEventRecord(e0, stream));
                    for (int p = 0; p < 2; ++p) {
                        batched_table_kernel<<<(unsigned)count, 256, 0, stream>>>(d_mats, d_work, d_toff, d_shape, d_grid, d_place, d_tab, p);
                        const int64_t* q = d_pre + ((int64_t)p * kClasses + c) * (count + 1);
                        if (sh == 0)
                            batched_wave_kernel<ShapeA><<<ctas, kThreads, 0, stream>>>(d_mats, d_work, d_toff, q, (int32_t)count, d_wl, p, c, d_q, d_tab, d_err, -0.0);
                        else
                            batched_wave_kernel<ShapeB><<<ctas, kThreads, 0, stream>>>(d_mats, d_work, d_toff, q, (int32_t)count, d_wl, p, c, d_q, d_tab, d_err, -0.0);
                    }
                    ck(cudaEventRecord(e1, stream));
                    ck(cudaEventSynchronize(e1));
                    float x = 0.f;
                    ck(cudaEventElapsedTime(&x, e0, e1));
                    if (rep > 0 && x < t) t = x;
                }
                ck(cudaGetLastError());
                if (ms) ms[c * 2 + sh] = t;
                if (t < best) { best = t; best_s = sh; }
            }
            cudaFree(d_mats); cudaFree(d_work); cudaFree(d_toff); cudaFree(d_pre); cudaFree(d_wl);
            cudaFree(d_shape); cudaFree(d_grid); cudaFree(d_place); cudaFree(d_q); cudaFree(d_tab);
            cudaFree(d_err);
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            if (er != cudaSuccess) return cuda_status(er);
        }
        g_tuning.shape[c] = best_s;
    }
    return rc;
}

}  // namespace symeig
