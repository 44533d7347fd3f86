// api.cu -- the C ABI of libsymeig.so (declared in include/symeig.h) and the host driver of
// the device eigensolver.
//
// qr driver.  The reference's outer loop (src/bulge_chasing.jl:166-284) alternates a serial
// chase that fills a (n-1) x max_layers rotation buffer with a bulk application of that
// buffer to Q.  Here the chase is a two-warp kernel on a side stream and the apply is the
// wave-window kernel on the main stream, ordered by events: chase f, apply f, chase f+1, ...
// (the rotation grid is double-buffered so that a concurrent schedule is possible; see the
// note in the flush loop for why it is not used).  After each chase the host reads its
// status (pinned memory) to learn whether to apply, stop (converged) or give up (maxiter),
// exactly the three exits of the reference.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#include "symeig.h"
#include "symeig_common.cuh"

using namespace symeig;

struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t want)
    {
        if (want <= bytes) return cudaSuccess;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&ptr, want);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release()
    {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
};

struct symeig_context {
    int device = 0;
    int sm_count = 0, cc_major = 0, cc_minor = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;       // main (apply) stream
    cudaStream_t chase_stream = nullptr; // side stream for the chase
    cudaEvent_t ev_chased[2] = {nullptr, nullptr};
    cudaEvent_t ev_consumed[2] = {nullptr, nullptr};
    cudaEvent_t ev_main = nullptr;
    // the pipelined host-pointer apply: one stream and completion event per row block, and the
    // event after the table (created on first use)
    cudaStream_t pipe[kPipeBlocks] = {};
    cudaEvent_t pipe_done[kPipeBlocks] = {};
    cudaEvent_t ev_table = nullptr;
    // the column-segment pipeline of the host-pointer apply: per segment, columns copied in and
    // kernel done
    cudaEvent_t seg_in[kPipeBlocks] = {}, seg_done[kPipeBlocks] = {};
    DevBuf grid[2], thick[2], place[2], table, state, d, e, q, cs, bak, rot, dense, dense_io, bulge, seg_state;
    int* derr = nullptr;   // device error word of the wave kernels (bounded waits)
    int32_t exact_order = 1;  // rotation placement of the qr driver
    int32_t chase_mode = 0;   // symeig_set_chase_mode
    int32_t apply_form = 0;   // symeig_set_apply_form
    int32_t test_stall = 0;   // symeig_set_test_stall
    int32_t ms_bulges = kDefaultBulges;      // symeig_set_multishift
    int32_t ms_rows = kDefaultRowsPerBulge;
    int32_t ms_prog_every = kDefaultProgEvery;
    int32_t ms_min_bulges = kDefaultMinBulges;  // symeig_set_multishift_min
    ChaseState* h_state = nullptr;  // pinned
    std::vector<cudaEvent_t> timing;  // pool of timing events
    symeig_stats stats{};
    // optional per-launch timing of the wave kernel (symeig_set_kernel_timing)
    bool kernel_timing = false;
    std::vector<cudaEvent_t> kpool;
    size_t kused = 0;
    bool kpending = false;
};

namespace {

// NVTX range over a host scope (header-only NVTX 3: a no-op unless a profiler is attached).
// The qr driver marks each flush's chase (the host waits for it inside the range, so the
// range spans its device time) and each apply enqueue; the bulk entry points mark the call.
struct NvtxRange {
    bool open = true;
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { end(); }
    void end()
    {
        if (open) nvtxRangePop();
        open = false;
    }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

int cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return SYMEIG_OK;
    if (e == cudaErrorMemoryAllocation) return SYMEIG_ERR_NOMEM;
    return SYMEIG_ERR_CUDA;
}

#define CK(call)                                        \
    do {                                                \
        cudaError_t _e = (call);                        \
        if (_e != cudaSuccess) return cuda_status(_e);  \
    } while (0)

int check_handle(symeig_handle h)
{
    if (!h) return SYMEIG_ERR_HANDLE;
    if (cudaSetDevice(h->device) != cudaSuccess) return SYMEIG_ERR_CUDA;
    return SYMEIG_OK;
}

bool mul_overflows(int64_t a, int64_t b)
{
    return a > 0 && b > 0 && a > INT64_MAX / b;
}

int validate_matrix(const void* A, int64_t lda, int64_t m, int64_t n)
{
    // the kernels index columns with 32-bit integers
    if (m < 0 || n < 0 || n > (int64_t)1 << 30) return SYMEIG_ERR_SIZE;
    if (m > 0 && n > 0 && !A) return SYMEIG_ERR_NULL;
    if (m > 0 && lda < m) return SYMEIG_ERR_LD;
    if (mul_overflows(lda, n)) return SYMEIG_ERR_SIZE;
    return SYMEIG_OK;
}

cudaEvent_t timing_event(symeig_handle h, size_t idx)
{
    while (h->timing.size() <= idx) {
        cudaEvent_t ev;
        if (cudaEventCreate(&ev) != cudaSuccess) return nullptr;
        h->timing.push_back(ev);
    }
    return h->timing[idx];
}

cudaEvent_t kernel_event(symeig_handle h)
{
    if (h->kused == h->kpool.size()) {
        cudaEvent_t ev;
        if (cudaEventCreate(&ev) != cudaSuccess) return nullptr;
        h->kpool.push_back(ev);
    }
    return h->kpool[h->kused++];
}

// Start a new call: statistics and kernel-timing marks refer to the last call only.
void begin_call(symeig_handle h)
{
    std::memset(&h->stats, 0, sizeof(h->stats));
    h->kused = 0;
    h->kpending = false;
    // the error word of the bounded waits reports on this call only
    cudaMemsetAsync(h->derr, 0, sizeof(int), h->stream);
}

// After a synchronous call: SYMEIG_ERR_TIMEOUT if a wave kernel's bounded wait gave up.
int check_device_error(symeig_handle h)
{
    int derr = 0;
    CK(cudaMemcpy(&derr, h->derr, sizeof(int), cudaMemcpyDeviceToHost));
    h->stats.device_errors = derr;
    // bit 0: a bounded wait gave up; bit 1: an index check of a checked build failed
    if (derr & 2) return SYMEIG_ERR_DEVICE;
    return derr ? SYMEIG_ERR_TIMEOUT : SYMEIG_OK;
}

// Run every pass of one bulk apply of `layers` layers of `grid` to columns [c0, c0+n_loc).
template <typename Tsrc, typename T>
int apply_grid(symeig_handle h, T* Q, int64_t ldq, int64_t m, const Tsrc* grid, int64_t grid_rows,
               const int32_t* thick, int64_t c0, int64_t n_loc, int64_t layers, cudaStream_t s,
               int64_t rs = 1)
{
    if (m <= 0 || n_loc < 2 || layers <= 0) return SYMEIG_OK;
    const int64_t per = apply_layers_per_pass<T>(m, layers, sizeof(T) == 8 ? h->apply_form : 0);
    CK(h->table.ensure(apply_table_bytes<T>(n_loc, layers)));
    // the scaled form: the column-scale recurrences of all passes at once
    bool rec_all = false;
    if constexpr (std::is_same<Tsrc, double>::value && std::is_same<T, double>::value) {
        if (h->apply_form == 1 && layers > per) {
            CK(launch_scaled_recurrences(grid, grid_rows, thick, c0, n_loc, 0, layers, h->table.ptr, s));
            rec_all = true;
        }
    }
    for (int64_t L0 = 0; L0 < layers; L0 += per) {
        ApplyPass pass{c0, n_loc, L0, std::min(per, layers - L0), rs};
        pass.form = sizeof(T) == 8 ? h->apply_form : 0;
        pass.stall = h->test_stall;
        pass.rec = rec_all ? 1 : 0;
        pass.slot = rec_all ? (int32_t)(L0 / per) : 0;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (h->kernel_timing) {
            e0 = kernel_event(h);
            e1 = kernel_event(h);
            if (!e0 || !e1) return SYMEIG_ERR_CUDA;
            h->kpending = true;
        }
        CK((apply_pass<Tsrc, T>(Q, ldq, m, grid, grid_rows, thick, pass, h->table.ptr, h->derr, s,
                                e0, e1)));
        h->stats.wave_launches += 1;
    }
    h->stats.applied_rotation_rows += (n_loc - 1) * layers * m;
    return SYMEIG_OK;
}

template <typename T>
int qr_dev(symeig_handle h, double* d, double* e, int64_t n, T* Q, int64_t ldq, int64_t m,
           int32_t max_layers, double tol, int64_t maxiter, int32_t* converged, int64_t* iter)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (!converged || !iter) return SYMEIG_ERR_NULL;
    if (n < 1) return SYMEIG_ERR_SIZE;
    if (!d || (n > 1 && !e)) return SYMEIG_ERR_NULL;
    if (max_layers < 1) return SYMEIG_ERR_LAYERS;
    if (Q == nullptr) m = 0;
    rc = validate_matrix(Q, ldq, m, n);
    if (rc) return rc;
    const int64_t rows = n > 1 ? n - 1 : 1;
    if (max_layers > (1 << 29) || mul_overflows(rows, (int64_t)max_layers * 32)) return SYMEIG_ERR_SIZE;
    // exact-order placement can need more layers than the reference's capacity rule allows
    const int32_t grid_layers = h->exact_order ? 2 * max_layers : max_layers;

    auto t0 = std::chrono::steady_clock::now();
    begin_call(h);
    const size_t grid_bytes = (size_t)rows * grid_layers * 2 * sizeof(double);
    for (int b = 0; b < 2; ++b) {
        CK(h->grid[b].ensure(grid_bytes));
        CK(h->thick[b].ensure((size_t)n * sizeof(int32_t)));
        CK(h->place[b].ensure((size_t)n * sizeof(int32_t)));
    }
    CK(h->state.ensure(sizeof(ChaseState)));
    CK(h->bak.ensure((size_t)2 * n * sizeof(double)));
    CK(h->bulge.ensure(sizeof(BulgeScratch)));

    ChaseState init{};
    init.n = n;
    init.start = 1;
    init.last_block_ends_at = n;
    init.iter = 0;
    init.maxiter = maxiter;
    init.tol = tol;
    init.max_layers = max_layers;
    init.grid_layers = grid_layers;
    init.exact_order = h->exact_order;
    init.status = CHASE_RUNNING;
    init.neg_zero = -0.0;
    init.chase_mode = h->chase_mode;
    init.ms_bulges = h->ms_bulges;
    init.ms_rows = h->ms_rows;
    init.ms_prog_mask = h->ms_prog_every - 1;
    init.ms_min_bulges = h->ms_min_bulges;
    init.test_stall = h->test_stall;
    ChaseState* dstate = (ChaseState*)h->state.ptr;

    cudaStream_t ms = h->stream, cs = h->chase_stream;
    // the chase must see whatever the caller enqueued on the main stream (d, e, Q writes)
    CK(cudaEventRecord(h->ev_main, ms));
    CK(cudaStreamWaitEvent(cs, h->ev_main, 0));
    CK(cudaMemcpyAsync(dstate, &init, sizeof(init), cudaMemcpyHostToDevice, cs));
    // the memcpy above reads a stack object: make it complete before returning from scope
    CK(cudaStreamSynchronize(cs));

    // SYMEIG_DEBUG=1 prints one line per flush to stderr.
    static const bool debug = std::getenv("SYMEIG_DEBUG") != nullptr;
    size_t tev = 0;
    double chase_ms = 0.0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> apply_marks;
    int32_t conv = 1;
    int64_t flush = 0;
    int result = SYMEIG_OK;
    for (;; ++flush) {
        const int b = (int)(flush & 1);
        // The chase of a flush starts after the previous flush's apply has finished.  Running
        // them concurrently (they touch disjoint buffers) was tried: at n = 8192 a chase that
        // overlapped a 512-CTA apply did not finish within 150 s, for a reason not yet found,
        // so the two are serialised.  The apply is ~5% of the chase time at these sizes.
        if (flush >= 1) CK(cudaStreamWaitEvent(cs, h->ev_consumed[b ^ 1], 0));
        cudaEvent_t c0 = timing_event(h, tev++), c1 = timing_event(h, tev++);
        if (!c0 || !c1) return SYMEIG_ERR_CUDA;
        NvtxRange nv_chase("symeig chase");
        CK(cudaEventRecord(c0, cs));
        BulgeScratch* bsc = (BulgeScratch*)h->bulge.ptr;
        CK(launch_chase(dstate, d, e, (double*)h->grid[b].ptr, (int32_t*)h->thick[b].ptr,
                        (int32_t*)h->place[b].ptr, (double*)h->bak.ptr, bsc, 0, cs));
        CK(cudaEventRecord(c1, cs));
        CK(cudaMemcpyAsync(h->h_state, dstate, sizeof(ChaseState), cudaMemcpyDeviceToHost, cs));
        CK(cudaEventRecord(h->ev_chased[b], cs));
        CK(cudaEventSynchronize(h->ev_chased[b]));
        // chase_mode 3: each multishift batch runs in its own cooperative launch, after which
        // the chase kernel resumes the flush.  kBatchesAhead (batch, resume) pairs are queued
        // per host round trip; those queued after the flush's last batch return at once.
        while (h->h_state->status == CHASE_BATCH) {
            for (int k = 0; k < kBatchesAhead; ++k) {
                CK(launch_bulge_batch(dstate, d, e, (double*)h->grid[b].ptr,
                                      (const int32_t*)h->thick[b].ptr, bsc, h->derr, h->ms_bulges, cs));
                CK(launch_chase(dstate, d, e, (double*)h->grid[b].ptr, (int32_t*)h->thick[b].ptr,
                                (int32_t*)h->place[b].ptr, (double*)h->bak.ptr, bsc, 1, cs));
            }
            CK(cudaEventRecord(c1, cs));
            CK(cudaMemcpyAsync(h->h_state, dstate, sizeof(ChaseState), cudaMemcpyDeviceToHost, cs));
            CK(cudaEventRecord(h->ev_chased[b], cs));
            CK(cudaEventSynchronize(h->ev_chased[b]));
        }
        nv_chase.end();
        float ms_chase = 0.f;
        CK(cudaEventElapsedTime(&ms_chase, c0, c1));
        chase_ms += ms_chase;
        const ChaseState st = *h->h_state;
        if (debug)
            fprintf(stderr, "[symeig] flush %lld: chase %.1f ms status %d rot %lld K %lld cols %lld..%lld t=%.1f ms\n",
                    (long long)flush, ms_chase, st.status, (long long)st.rotations,
                    (long long)st.max_thickness, (long long)st.min_from, (long long)st.max_to,
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
        if (st.status == CHASE_MAXITER) { conv = 0; break; }
        if (st.status == CHASE_CONVERGED) break;
        if (st.status != CHASE_FLUSH) { result = SYMEIG_ERR_DEVICE; break; }
        h->stats.flushes += 1;
        if (m > 0) {
            CK(cudaStreamWaitEvent(ms, h->ev_chased[b], 0));
            cudaEvent_t a0 = timing_event(h, tev++), a1 = timing_event(h, tev++);
            if (!a0 || !a1) return SYMEIG_ERR_CUDA;
            CK(cudaEventRecord(a0, ms));
            const int64_t c_lo = st.min_from - 1;          // 0-based first column touched
            const int64_t n_loc = st.max_to - c_lo;         // columns from..to of every sweep
            NvtxRange nv("symeig apply flush");
            rc = apply_grid<double, T>(h, Q, ldq, m, (const double*)h->grid[b].ptr, rows,
                                       (const int32_t*)h->place[b].ptr, c_lo, n_loc,
                                       st.max_thickness, ms);
            if (rc) return rc;
            CK(cudaEventRecord(a1, ms));
            apply_marks.emplace_back(a0, a1);
            CK(cudaEventRecord(h->ev_consumed[b], ms));
        } else {
            CK(cudaEventRecord(h->ev_consumed[b], cs));
        }
    }
    CK(cudaEventRecord(h->ev_main, cs));
    CK(cudaStreamWaitEvent(ms, h->ev_main, 0));
    CK(cudaStreamSynchronize(ms));
    double apply_ms = 0.0;
    for (auto& pr : apply_marks) {
        float x = 0.f;
        CK(cudaEventElapsedTime(&x, pr.first, pr.second));
        apply_ms += x;
    }
    const ChaseState fin = *h->h_state;
    *converged = conv;
    *iter = fin.iter;
    h->stats.iterations = fin.iter;
    h->stats.rotations = fin.total_rotations;
    h->stats.early_flushes = fin.early_flushes;
    h->stats.redone_sweeps = fin.redone_sweeps;
    h->stats.bulge_batches = fin.batches;
    h->stats.chase_ms = chase_ms;
    h->stats.apply_ms = apply_ms;
    h->stats.total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (result == SYMEIG_OK) result = check_device_error(h);
    return result;
}

template <typename T>
int qr_host(symeig_handle h, double* d, double* e, int64_t n, T* Q, int64_t ldq, int64_t m,
            int32_t max_layers, double tol, int64_t maxiter, int32_t* converged, int64_t* iter)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (n < 1) return SYMEIG_ERR_SIZE;
    if (!d || (n > 1 && !e) || !converged || !iter) return SYMEIG_ERR_NULL;
    if (Q == nullptr) m = 0;
    rc = validate_matrix(Q, ldq, m, n);
    if (rc) return rc;
    auto t0 = std::chrono::steady_clock::now();
    const int64_t ne = n > 1 ? n - 1 : 1;
    CK(h->d.ensure((size_t)n * sizeof(double)));
    CK(h->e.ensure((size_t)ne * sizeof(double)));
    T* dq = nullptr;
    if (m > 0) {
        CK(h->q.ensure((size_t)m * n * sizeof(T)));
        dq = (T*)h->q.ptr;
    }
    cudaStream_t s = h->stream;
    CK(cudaMemcpyAsync(h->d.ptr, d, n * sizeof(double), cudaMemcpyHostToDevice, s));
    if (n > 1) CK(cudaMemcpyAsync(h->e.ptr, e, (n - 1) * sizeof(double), cudaMemcpyHostToDevice, s));
    if (m > 0)
        CK(cudaMemcpy2DAsync(dq, m * sizeof(T), Q, ldq * sizeof(T), m * sizeof(T), n,
                             cudaMemcpyHostToDevice, s));
    rc = qr_dev<T>(h, (double*)h->d.ptr, (double*)h->e.ptr, n, dq, m, m, max_layers, tol, maxiter,
                   converged, iter);
    if (rc) return rc;
    CK(cudaMemcpyAsync(d, h->d.ptr, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (n > 1) CK(cudaMemcpyAsync(e, h->e.ptr, (n - 1) * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (m > 0)
        CK(cudaMemcpy2DAsync(Q, ldq * sizeof(T), dq, m * sizeof(T), m * sizeof(T), n,
                             cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    h->stats.total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return SYMEIG_OK;
}

template <typename T>
int apply_dev(symeig_handle h, T* A, int64_t lda, int64_t m, int64_t n, const T* cs, int64_t k)
{
    NvtxRange nv("symeig apply_givens (device pointers)");
    int rc = check_handle(h);
    if (rc) return rc;
    if (k < 0 || n < 0) return SYMEIG_ERR_SIZE;
    rc = validate_matrix(A, lda, m, n);
    if (rc) return rc;
    if (n >= 2 && k > 0 && !cs) return SYMEIG_ERR_NULL;
    if (mul_overflows(n, k * 2)) return SYMEIG_ERR_SIZE;
    begin_call(h);
    if (m == 0 || n < 2 || k == 0) return SYMEIG_OK;
    return apply_grid<T, T>(h, A, lda, m, cs, n - 1, nullptr, 0, n, k, h->stream);
}

// One pass (k <= 64 layers) with host Q, pipelined by column segments (apply_host_segmented,
// apply.cu): the columns of Q go to the device in kPipeBlocks chunks on one copy stream, the
// pass runs as kPipeBlocks launches of the whole-matrix wave kernel (each waiting only for the
// columns it reads, carrying its registers to the next in a state buffer), and the columns
// each launch finishes go back on a second copy stream right after it.  The copies in both
// directions then overlap the kernels, which run at the full-matrix rate.
template <typename T>
int apply_host_pipelined(symeig_handle h, T* A, int64_t lda, int64_t m, int64_t n, const T* cs, int64_t k)
{
    cudaStream_t s = h->stream;
    begin_call(h);
    for (int b = 0; b < 2; ++b)
        if (!h->pipe[b]) CK(cudaStreamCreateWithFlags(&h->pipe[b], cudaStreamNonBlocking));
    for (int j = 0; j < kPipeBlocks; ++j) {
        if (!h->seg_in[j]) CK(cudaEventCreateWithFlags(&h->seg_in[j], cudaEventDisableTiming));
        if (!h->seg_done[j]) CK(cudaEventCreateWithFlags(&h->seg_done[j], cudaEventDisableTiming));
    }
    if (!h->pipe_done[0]) CK(cudaEventCreateWithFlags(&h->pipe_done[0], cudaEventDisableTiming));
    CK(h->seg_state.ensure(apply_segment_state_bytes<T>(m)));
    CK(h->table.ensure(apply_table_bytes<T>(n, k)));
    // the copies start after whatever the caller queued on the main stream before this call
    CK(cudaEventRecord(h->ev_main, s));
    CK(cudaStreamWaitEvent(h->pipe[0], h->ev_main, 0));
    CK(cudaStreamWaitEvent(h->pipe[1], h->ev_main, 0));
    const size_t cs_bytes = (size_t)(n - 1) * k * 2 * sizeof(T);
    CK(cudaMemcpyAsync(h->cs.ptr, cs, cs_bytes, cudaMemcpyHostToDevice, s));
    ApplyPass pass{0, n, 0, k, 1};
    pass.form = sizeof(T) == 8 ? h->apply_form : 0;
    pass.stall = h->test_stall;
    HostStream io{A, lda, h->pipe[0], h->pipe[1], h->seg_in, h->seg_done, kPipeBlocks, h->seg_state.ptr};
    CK(apply_host_segmented<T>((T*)h->q.ptr, m, (const T*)h->cs.ptr, pass, h->table.ptr, h->derr, s, io));
    // the call ends when the last copy out has landed
    CK(cudaEventRecord(h->pipe_done[0], h->pipe[1]));
    CK(cudaStreamWaitEvent(s, h->pipe_done[0], 0));
    h->stats.wave_launches += kPipeBlocks;
    h->stats.applied_rotation_rows += (n - 1) * k * m;
    return SYMEIG_OK;
}

template <typename T>
int apply_host(symeig_handle h, T* A, int64_t lda, int64_t m, int64_t n, const T* cs, int64_t k)
{
    NvtxRange nv("symeig apply_givens (host pointers)");
    int rc = check_handle(h);
    if (rc) return rc;
    if (k < 0 || n < 0) return SYMEIG_ERR_SIZE;
    rc = validate_matrix(A, lda, m, n);
    if (rc) return rc;
    if (n >= 2 && k > 0 && !cs) return SYMEIG_ERR_NULL;
    if (m == 0 || n < 2 || k == 0) return SYMEIG_OK;
    if (mul_overflows(n, k * 2)) return SYMEIG_ERR_SIZE;
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = h->stream;
    CK(h->q.ensure((size_t)m * n * sizeof(T)));
    const size_t cs_bytes = (size_t)(n - 1) * k * 2 * sizeof(T);
    CK(h->cs.ensure(cs_bytes));
    if (k <= 64 && m >= (int64_t)kPipeBlocks * 256 && !h->kernel_timing &&
        apply_host_segmented_supported<T>(m)) {
        rc = apply_host_pipelined<T>(h, A, lda, m, n, cs, k);
        if (rc) {
            // nothing queued may still read or write the caller's buffer after the return
            for (int b = 0; b < 2; ++b)
                if (h->pipe[b]) cudaStreamSynchronize(h->pipe[b]);
            cudaStreamSynchronize(s);
            return rc;
        }
        CK(cudaStreamSynchronize(s));
        h->stats.total_ms =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return check_device_error(h);
    }
    CK(cudaMemcpyAsync(h->cs.ptr, cs, cs_bytes, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpy2DAsync(h->q.ptr, m * sizeof(T), A, lda * sizeof(T), m * sizeof(T), n,
                         cudaMemcpyHostToDevice, s));
    rc = apply_dev<T>(h, (T*)h->q.ptr, m, m, n, (const T*)h->cs.ptr, k);
    if (rc) return rc;
    CK(cudaMemcpy2DAsync(A, lda * sizeof(T), h->q.ptr, m * sizeof(T), m * sizeof(T), n,
                         cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    h->stats.total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return check_device_error(h);
}

// Row rotations (lmul!, src/simple_givens.jl:38-51) of an m x n column-major A: the wave
// kernel on the transposed view, whose rows (A's columns) are lda apart and whose columns
// (A's rows) are adjacent.  The grid is (m-1) x k.
template <typename T>
int apply_left_dev(symeig_handle h, T* A, int64_t lda, int64_t m, int64_t n, const T* cs, int64_t k)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (k < 0 || m < 0) return SYMEIG_ERR_SIZE;
    rc = validate_matrix(A, lda, m, n);
    if (rc) return rc;
    if (m > ((int64_t)1 << 30)) return SYMEIG_ERR_SIZE;
    if (m >= 2 && k > 0 && !cs) return SYMEIG_ERR_NULL;
    begin_call(h);
    if (n == 0 || m < 2 || k == 0) return SYMEIG_OK;
    return apply_grid<T, T>(h, A, 1, n, cs, m - 1, nullptr, 0, m, k, h->stream, lda);
}

template <typename T>
int apply_left_host(symeig_handle h, T* A, int64_t lda, int64_t m, int64_t n, const T* cs, int64_t k)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (k < 0 || m < 0) return SYMEIG_ERR_SIZE;
    rc = validate_matrix(A, lda, m, n);
    if (rc) return rc;
    if (m >= 2 && k > 0 && !cs) return SYMEIG_ERR_NULL;
    if (n == 0 || m < 2 || k == 0) return SYMEIG_OK;
    cudaStream_t s = h->stream;
    CK(h->q.ensure((size_t)m * n * sizeof(T)));
    const size_t cs_bytes = (size_t)(m - 1) * k * 2 * sizeof(T);
    CK(h->cs.ensure(cs_bytes));
    CK(cudaMemcpyAsync(h->cs.ptr, cs, cs_bytes, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpy2DAsync(h->q.ptr, m * sizeof(T), A, lda * sizeof(T), m * sizeof(T), n,
                         cudaMemcpyHostToDevice, s));
    rc = apply_left_dev<T>(h, (T*)h->q.ptr, m, m, n, (const T*)h->cs.ptr, k);
    if (rc) return rc;
    CK(cudaMemcpy2DAsync(A, lda * sizeof(T), h->q.ptr, m * sizeof(T), m * sizeof(T), n,
                         cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return SYMEIG_OK;
}

}  // namespace

namespace {

// sytrd with an exact power-of-two prescaling of A (see sytrd.cu on the range of the norms).
// work: dense_scratch_doubles(n) + 1 doubles on the device.
int sytrd_scaled(symeig_handle h, int64_t n, double* A, int64_t lda, double* d, double* e, double* tau,
                 double* work)
{
    cudaStream_t st = h->stream;
    double* amax_d = work + dense_scratch_doubles(n);
    CK(launch_dense_maxabs(A, lda, n, amax_d, st));
    double amax = 0.0;
    CK(cudaMemcpyAsync(&amax, amax_d, sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    int ea = 0;
    const bool scale = amax != 0.0 && std::isfinite(amax) && ((ea = std::ilogb(amax)) < -2 || ea > 2);
    if (scale) CK(launch_dense_scale(A, lda, n, std::ldexp(1.0, -ea), st));
    int rc = sytrd_dev(st, n, A, lda, d, e, tau, work);
    if (rc) return rc;
    if (scale) CK(launch_tridiag_unscale(A, lda, n, d, e, std::ldexp(1.0, ea), st));
    return SYMEIG_OK;
}

int dense_args(symeig_handle h, int64_t n, const void* A, int64_t lda)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (n < 1 || n > ((int64_t)1 << 30)) return SYMEIG_ERR_SIZE;
    if (!A) return SYMEIG_ERR_NULL;
    if (lda < n) return SYMEIG_ERR_LD;
    if (mul_overflows(lda, n)) return SYMEIG_ERR_SIZE;
    return SYMEIG_OK;
}

}  // namespace

namespace {

// Batched solve with d, e and Q on the device; Q is FP64 or FP32.
template <typename T>
int qr_batched_dev_entry(symeig_handle h, int64_t count, const int64_t* n, double* d, double* e, T* Q,
                         int32_t max_layers, double tol, int64_t maxiter_factor, int32_t* converged,
                         int64_t* iters)
{
    NvtxRange nv("symeig qr batched");
    int rc = check_handle(h);
    if (rc) return rc;
    if (count < 0) return SYMEIG_ERR_SIZE;
    if (count > 0 && (!n || !d || !e)) return SYMEIG_ERR_NULL;
    if (max_layers < 1) return SYMEIG_ERR_LAYERS;
    begin_call(h);
    auto t0 = std::chrono::steady_clock::now();
    // The rounds are captured as a CUDA graph, which needs a capturable stream (not the legacy
    // default stream): run on the handle's own stream, ordered after the caller's stream.
    CK(cudaEventRecord(h->ev_main, h->stream));
    CK(cudaStreamWaitEvent(h->own_stream, h->ev_main, 0));
    rc = qr_batched_dev<T>(h->device, h->own_stream, count, n, d, e, Q, max_layers, tol, maxiter_factor,
                           h->exact_order, converged, iters, &h->stats.flushes, nullptr);
    for (int64_t i = 0; i < count && iters; ++i) h->stats.iterations += iters[i];
    h->stats.total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

// Batched solve with host d, e and Q: copies in, the device solve, copies out.
template <typename T>
int qr_batched_host_entry(symeig_handle h, int64_t count, const int64_t* n, double* d, double* e, T* Q,
                          int32_t max_layers, double tol, int64_t maxiter_factor, int32_t* converged,
                          int64_t* iters)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (count < 0) return SYMEIG_ERR_SIZE;
    if (count == 0) return SYMEIG_OK;
    if (!n || !d || !e) return SYMEIG_ERR_NULL;
    int64_t nd = 0, ne = 0, nq = 0;
    for (int64_t i = 0; i < count; ++i) {
        if (n[i] < 1) return SYMEIG_ERR_SIZE;
        nd += n[i];
        ne += n[i] - 1;
        nq += n[i] * n[i];
    }
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = h->stream;
    CK(h->d.ensure(nd * sizeof(double)));
    CK(h->e.ensure(std::max<int64_t>(ne, 1) * sizeof(double)));
    if (Q) CK(h->q.ensure(nq * sizeof(T)));
    CK(cudaMemcpyAsync(h->d.ptr, d, nd * sizeof(double), cudaMemcpyHostToDevice, s));
    if (ne) CK(cudaMemcpyAsync(h->e.ptr, e, ne * sizeof(double), cudaMemcpyHostToDevice, s));
    if (Q) CK(cudaMemcpyAsync(h->q.ptr, Q, nq * sizeof(T), cudaMemcpyHostToDevice, s));
    rc = qr_batched_dev_entry<T>(h, count, n, (double*)h->d.ptr, (double*)h->e.ptr, Q ? (T*)h->q.ptr : nullptr,
                                 max_layers, tol, maxiter_factor, converged, iters);
    if (rc) return rc;
    CK(cudaMemcpyAsync(d, h->d.ptr, nd * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (ne) CK(cudaMemcpyAsync(e, h->e.ptr, ne * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (Q) CK(cudaMemcpyAsync(Q, h->q.ptr, nq * sizeof(T), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    h->stats.total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return SYMEIG_OK;
}

}  // namespace

extern "C" {

int symeig_apply_givens_left_f64(symeig_handle h, double* A, int64_t lda, int64_t m, int64_t n,
                                 const double* cs, int64_t k)
{
    return apply_left_host<double>(h, A, lda, m, n, cs, k);
}

int symeig_apply_givens_left_f32(symeig_handle h, float* A, int64_t lda, int64_t m, int64_t n,
                                 const float* cs, int64_t k)
{
    return apply_left_host<float>(h, A, lda, m, n, cs, k);
}

int symeig_apply_givens_left_f64_dev(symeig_handle h, double* A, int64_t lda, int64_t m,
                                     int64_t n, const double* cs, int64_t k)
{
    return apply_left_dev<double>(h, A, lda, m, n, cs, k);
}

int symeig_apply_givens_left_f32_dev(symeig_handle h, float* A, int64_t lda, int64_t m,
                                     int64_t n, const float* cs, int64_t k)
{
    return apply_left_dev<float>(h, A, lda, m, n, cs, k);
}


int symeig_create(symeig_handle* out, int device)
{
    if (!out) return SYMEIG_ERR_NULL;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
        return SYMEIG_ERR_CUDA;
    symeig_context* h = new (std::nothrow) symeig_context();
    if (!h) return SYMEIG_ERR_NOMEM;
    h->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->cc_major, cudaDevAttrComputeCapabilityMajor, device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->cc_minor, cudaDevAttrComputeCapabilityMinor, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->chase_stream, cudaStreamNonBlocking);
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
        e = cudaEventCreateWithFlags(&h->ev_chased[b], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_consumed[b], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_main, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&h->h_state, sizeof(ChaseState));
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->derr, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(h->derr, 0, sizeof(int));
    if (e != cudaSuccess) {
        symeig_destroy(h);
        return cuda_status(e);
    }
    h->stream = h->own_stream;
    *out = h;
    return SYMEIG_OK;
}

int symeig_destroy(symeig_handle h)
{
    if (!h) return SYMEIG_ERR_HANDLE;
    cudaSetDevice(h->device);
    if (h->own_stream) cudaStreamSynchronize(h->own_stream);
    if (h->chase_stream) cudaStreamSynchronize(h->chase_stream);
    if (h->stream && h->stream != h->own_stream) cudaStreamSynchronize(h->stream);
    for (int b = 0; b < 2; ++b) {
        h->grid[b].release();
        h->thick[b].release();
        h->place[b].release();
        if (h->ev_chased[b]) cudaEventDestroy(h->ev_chased[b]);
        if (h->ev_consumed[b]) cudaEventDestroy(h->ev_consumed[b]);
    }
    h->table.release(); h->state.release(); h->d.release(); h->e.release();
    h->q.release(); h->cs.release(); h->bak.release(); h->rot.release();
    h->dense.release(); h->dense_io.release(); h->bulge.release(); h->seg_state.release();
    if (h->ev_main) cudaEventDestroy(h->ev_main);
    for (int b = 0; b < kPipeBlocks; ++b) {
        if (h->pipe[b]) {
            cudaStreamSynchronize(h->pipe[b]);
            cudaStreamDestroy(h->pipe[b]);
        }
        if (h->pipe_done[b]) cudaEventDestroy(h->pipe_done[b]);
        if (h->seg_in[b]) cudaEventDestroy(h->seg_in[b]);
        if (h->seg_done[b]) cudaEventDestroy(h->seg_done[b]);
    }
    if (h->ev_table) cudaEventDestroy(h->ev_table);
    for (cudaEvent_t ev : h->timing) cudaEventDestroy(ev);
    for (cudaEvent_t ev : h->kpool) cudaEventDestroy(ev);
    if (h->h_state) cudaFreeHost(h->h_state);
    if (h->derr) cudaFree(h->derr);
    if (h->chase_stream) cudaStreamDestroy(h->chase_stream);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return SYMEIG_OK;
}

int symeig_set_stream(symeig_handle h, void* stream)
{
    int rc = check_handle(h);
    if (rc) return rc;
    h->stream = (cudaStream_t)stream;  // NULL is the legacy default stream
    return SYMEIG_OK;
}

int symeig_get_stream(symeig_handle h, void** stream)
{
    if (!h) return SYMEIG_ERR_HANDLE;
    if (!stream) return SYMEIG_ERR_NULL;
    *stream = (void*)h->stream;
    return SYMEIG_OK;
}

int symeig_set_exact_order(symeig_handle h, int32_t exact_order)
{
    if (!h) return SYMEIG_ERR_HANDLE;
    h->exact_order = exact_order ? 1 : 0;
    return SYMEIG_OK;
}

int symeig_set_chase_mode(symeig_handle h, int32_t mode)
{
    if (!h) return SYMEIG_ERR_HANDLE;
    if (mode < 0 || mode > 3) return SYMEIG_ERR_SIZE;
    h->chase_mode = mode;
    return SYMEIG_OK;
}

int symeig_set_multishift(symeig_handle h, int32_t max_bulges, int32_t rows_per_bulge,
                          int32_t release_every)
{
    if (!h) return SYMEIG_ERR_HANDLE;
    if (max_bulges < 2 || max_bulges > kMaxBulges || rows_per_bulge < 4) return SYMEIG_ERR_SIZE;
    if (release_every < 1 || release_every > 64 || (release_every & (release_every - 1))) return SYMEIG_ERR_SIZE;
    h->ms_bulges = max_bulges;
    h->ms_rows = rows_per_bulge;
    h->ms_prog_every = release_every;
    return SYMEIG_OK;
}

int symeig_set_multishift_min(symeig_handle h, int32_t min_bulges)
{
    if (!h) return SYMEIG_ERR_HANDLE;
    if (min_bulges < 2 || min_bulges > kMaxBulges) return SYMEIG_ERR_SIZE;
    h->ms_min_bulges = min_bulges;
    return SYMEIG_OK;
}

int symeig_set_apply_form(symeig_handle h, int32_t form)
{
    if (!h) return SYMEIG_ERR_HANDLE;
    if (form < 0 || form > 2) return SYMEIG_ERR_SIZE;
    h->apply_form = form;
    return SYMEIG_OK;
}

int symeig_set_test_stall(symeig_handle h, int32_t chunk)
{
    if (!h) return SYMEIG_ERR_HANDLE;
    if (chunk < 0) return SYMEIG_ERR_SIZE;
    h->test_stall = chunk;
    return SYMEIG_OK;
}

int symeig_set_kernel_timing(symeig_handle h, int32_t on)
{
    if (!h) return SYMEIG_ERR_HANDLE;
    h->kernel_timing = on != 0;
    return SYMEIG_OK;
}

int symeig_get_stats(symeig_handle h, symeig_stats* out)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (!out) return SYMEIG_ERR_NULL;
    if (h->kpending) {
        // wait for the last marked launch, then sum the wave-kernel durations of the call
        CK(cudaEventSynchronize(h->kpool[h->kused - 1]));
        double ms = 0.0;
        for (size_t i = 0; i + 1 < h->kused; i += 2) {
            float x = 0.f;
            CK(cudaEventElapsedTime(&x, h->kpool[i], h->kpool[i + 1]));
            ms += x;
        }
        h->stats.wave_kernel_ms = ms;
        h->kpending = false;
    }
    int derr = 0;
    CK(cudaMemcpy(&derr, h->derr, sizeof(int), cudaMemcpyDeviceToHost));
    h->stats.device_errors = derr;
    *out = h->stats;
    return SYMEIG_OK;
}

int symeig_device_info(symeig_handle h, int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor)
{
    if (!h) return SYMEIG_ERR_HANDLE;
    if (sm_count) *sm_count = h->sm_count;
    if (cc_major) *cc_major = h->cc_major;
    if (cc_minor) *cc_minor = h->cc_minor;
    return SYMEIG_OK;
}

const char* symeig_status_string(int status)
{
    switch (status) {
        case SYMEIG_OK: return "ok";
        case SYMEIG_ERR_NULL: return "a required pointer is NULL";
        case SYMEIG_ERR_SIZE: return "invalid size";
        case SYMEIG_ERR_LD: return "leading dimension smaller than the row count";
        case SYMEIG_ERR_LAYERS: return "max_layers must be >= 1";
        case SYMEIG_ERR_HANDLE: return "invalid handle";
        case SYMEIG_ERR_CUDA: return "CUDA runtime error";
        case SYMEIG_ERR_NOMEM: return "out of memory";
        case SYMEIG_ERR_TIMEOUT: return "bounded device wait timed out";
        case SYMEIG_ERR_DEVICE: return "device kernel reported an error";
        default: return "unknown status";
    }
}

int symeig_qr_f64(symeig_handle h, double* d, double* e, int64_t n, double* Q, int64_t ldq,
                  int64_t m, int32_t max_layers, double tol, int64_t maxiter, int32_t* converged,
                  int64_t* iter)
{
    return qr_host<double>(h, d, e, n, Q, ldq, m, max_layers, tol, maxiter, converged, iter);
}

int symeig_qr_f64_dev(symeig_handle h, double* d, double* e, int64_t n, double* Q, int64_t ldq,
                      int64_t m, int32_t max_layers, double tol, int64_t maxiter,
                      int32_t* converged, int64_t* iter)
{
    return qr_dev<double>(h, d, e, n, Q, ldq, m, max_layers, tol, maxiter, converged, iter);
}

int symeig_qr_f64_q32(symeig_handle h, double* d, double* e, int64_t n, float* Q, int64_t ldq,
                      int64_t m, int32_t max_layers, double tol, int64_t maxiter,
                      int32_t* converged, int64_t* iter)
{
    return qr_host<float>(h, d, e, n, Q, ldq, m, max_layers, tol, maxiter, converged, iter);
}

int symeig_qr_f64_q32_dev(symeig_handle h, double* d, double* e, int64_t n, float* Q,
                          int64_t ldq, int64_t m, int32_t max_layers, double tol,
                          int64_t maxiter, int32_t* converged, int64_t* iter)
{
    return qr_dev<float>(h, d, e, n, Q, ldq, m, max_layers, tol, maxiter, converged, iter);
}

int symeig_apply_givens_f64(symeig_handle h, double* A, int64_t lda, int64_t m, int64_t n,
                            const double* cs, int64_t k)
{
    return apply_host<double>(h, A, lda, m, n, cs, k);
}

int symeig_apply_givens_f32(symeig_handle h, float* A, int64_t lda, int64_t m, int64_t n,
                            const float* cs, int64_t k)
{
    return apply_host<float>(h, A, lda, m, n, cs, k);
}

int symeig_apply_givens_f64_dev(symeig_handle h, double* A, int64_t lda, int64_t m, int64_t n,
                                const double* cs, int64_t k)
{
    return apply_dev<double>(h, A, lda, m, n, cs, k);
}

int symeig_apply_givens_f32_dev(symeig_handle h, float* A, int64_t lda, int64_t m, int64_t n,
                                const float* cs, int64_t k)
{
    return apply_dev<float>(h, A, lda, m, n, cs, k);
}


int symeig_qr_batched_f64_dev(symeig_handle h, int64_t count, const int64_t* n, double* d,
                              double* e, double* Q, int32_t max_layers, double tol,
                              int64_t maxiter_factor, int32_t* converged, int64_t* iters)
{
    return qr_batched_dev_entry<double>(h, count, n, d, e, Q, max_layers, tol, maxiter_factor, converged, iters);
}

int symeig_qr_batched_f64(symeig_handle h, int64_t count, const int64_t* n, double* d, double* e,
                          double* Q, int32_t max_layers, double tol, int64_t maxiter_factor,
                          int32_t* converged, int64_t* iters)
{
    return qr_batched_host_entry<double>(h, count, n, d, e, Q, max_layers, tol, maxiter_factor, converged, iters);
}

int symeig_qr_batched_f64_q32_dev(symeig_handle h, int64_t count, const int64_t* n, double* d,
                                  double* e, float* Q, int32_t max_layers, double tol,
                                  int64_t maxiter_factor, int32_t* converged, int64_t* iters)
{
    return qr_batched_dev_entry<float>(h, count, n, d, e, Q, max_layers, tol, maxiter_factor, converged, iters);
}

int symeig_qr_batched_f64_q32(symeig_handle h, int64_t count, const int64_t* n, double* d, double* e,
                              float* Q, int32_t max_layers, double tol, int64_t maxiter_factor,
                              int32_t* converged, int64_t* iters)
{
    return qr_batched_host_entry<float>(h, count, n, d, e, Q, max_layers, tol, maxiter_factor, converged, iters);
}

int symeig_apply_tuning(int32_t fp64, int32_t* shape, int32_t set)
{
    if (!shape) return SYMEIG_ERR_NULL;
    if (set) {
        if (*shape < -1 || *shape >= apply_num_shapes(fp64)) return SYMEIG_ERR_SIZE;
        apply_set_shape(fp64, *shape);
    } else {
        *shape = apply_get_shape(fp64);
    }
    return SYMEIG_OK;
}

int symeig_batched_autotune(symeig_handle h, double* ms)
{
    int rc = check_handle(h);
    if (rc) return rc;
    return batched_autotune(h->device, h->stream, 0, nullptr, ms);
}

int symeig_batched_autotune_sizes(symeig_handle h, int64_t count, const int64_t* n, double* ms)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (count < 0) return SYMEIG_ERR_SIZE;
    if (count > 0 && !n) return SYMEIG_ERR_NULL;
    for (int64_t i = 0; i < count; ++i)
        if (n[i] < 1 || n[i] > (1 << 20)) return SYMEIG_ERR_SIZE;
    return batched_autotune(h->device, h->stream, count, n, ms);
}

int symeig_batched_tuning_dtype(int32_t fp64, int64_t* split, int32_t* shape_small, int32_t* shape_large,
                                int32_t set)
{
    if (!split || !shape_small || !shape_large) return SYMEIG_ERR_NULL;
    if (set) {
        const int nt = batched_num_tiles();
        if (*split < 1 || *shape_small < 0 || *shape_small >= nt || *shape_large < 0 || *shape_large >= nt)
            return SYMEIG_ERR_SIZE;
        batched_set_tuning(fp64, *split, *shape_small, *shape_large);
    } else {
        batched_get_tuning(fp64, split, shape_small, shape_large);
    }
    return SYMEIG_OK;
}

int symeig_batched_tuning(int64_t* split, int32_t* shape_small, int32_t* shape_large, int32_t set)
{
    return symeig_batched_tuning_dtype(1, split, shape_small, shape_large, set);
}

int symeig_eig_adjoint_f64_dev(symeig_handle h, int64_t count, int64_t n, const double* lam,
                               const double* Q, const double* glam, const double* gQ, double* gd,
                               double* ge)
{
    NvtxRange nv("symeig adjoint");
    int rc = check_handle(h);
    if (rc) return rc;
    if (count < 0 || n < 0 || (count > 0 && n > (1 << 20))) return SYMEIG_ERR_SIZE;
    if (count == 0 || n == 0) return SYMEIG_OK;
    if (!lam || !Q || !glam || !gd || (n > 1 && !ge)) return SYMEIG_ERR_NULL;
    begin_call(h);
    if (gQ) CK(h->cs.ensure((size_t)adjoint_scratch_doubles(count, n) * sizeof(double)));
    auto t0 = std::chrono::steady_clock::now();
    rc = adjoint_dev(h->stream, count, n, lam, Q, glam, gQ, gd, ge, (double*)h->cs.ptr);
    h->stats.total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

int symeig_eig_adjoint_f64(symeig_handle h, int64_t count, int64_t n, const double* lam,
                           const double* Q, const double* glam, const double* gQ, double* gd,
                           double* ge)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (count < 0 || n < 0 || (count > 0 && n > (1 << 20))) return SYMEIG_ERR_SIZE;
    if (count == 0 || n == 0) return SYMEIG_OK;
    if (!lam || !Q || !glam || !gd || (n > 1 && !ge)) return SYMEIG_ERR_NULL;
    cudaStream_t s = h->stream;
    const size_t nn = (size_t)count * n * n, nv = (size_t)count * n, ne = (size_t)count * (n - 1);
    // device staging: Q and gQ in q (2 nn), lam/glam/gd in d (3 nv), ge in e
    CK(h->q.ensure((gQ ? 2 : 1) * nn * sizeof(double)));
    CK(h->d.ensure(3 * nv * sizeof(double)));
    CK(h->e.ensure(std::max<size_t>(ne, 1) * sizeof(double)));
    double* dq = (double*)h->q.ptr;
    double* dgq = gQ ? dq + nn : nullptr;
    double* dl = (double*)h->d.ptr;
    double* dgl = dl + nv;
    double* dgd = dl + 2 * nv;
    double* dge = (double*)h->e.ptr;
    CK(cudaMemcpyAsync(dq, Q, nn * sizeof(double), cudaMemcpyHostToDevice, s));
    if (gQ) CK(cudaMemcpyAsync(dgq, gQ, nn * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dl, lam, nv * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dgl, glam, nv * sizeof(double), cudaMemcpyHostToDevice, s));
    rc = symeig_eig_adjoint_f64_dev(h, count, n, dl, dq, dgl, dgq, dgd, dge);
    if (rc) return rc;
    CK(cudaMemcpyAsync(gd, dgd, nv * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (ne) CK(cudaMemcpyAsync(ge, dge, ne * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return SYMEIG_OK;
}

int symeig_sytrd_f64_dev(symeig_handle h, int64_t n, double* A, int64_t lda, double* d, double* e,
                         double* tau)
{
    int rc = dense_args(h, n, A, lda);
    if (rc) return rc;
    if (!d || (n > 1 && (!e || !tau))) return SYMEIG_ERR_NULL;
    begin_call(h);
    CK(h->dense.ensure((size_t)(dense_scratch_doubles(n) + 1) * sizeof(double)));
    return sytrd_scaled(h, n, A, lda, d, e, tau, (double*)h->dense.ptr);
}

int symeig_orgtr_f64_dev(symeig_handle h, int64_t n, const double* A, int64_t lda, const double* tau,
                         double* Q, int64_t ldq)
{
    int rc = dense_args(h, n, A, lda);
    if (rc) return rc;
    if (!Q || (n > 1 && !tau)) return SYMEIG_ERR_NULL;
    if (ldq < n) return SYMEIG_ERR_LD;
    begin_call(h);
    CK(h->dense.ensure((size_t)(dense_scratch_doubles(n) + 1) * sizeof(double)));
    return orgtr_dev(h->stream, n, A, lda, tau, Q, ldq, (double*)h->dense.ptr);
}

int symeig_syev_f64_dev(symeig_handle h, int64_t n, double* A, int64_t lda, double* lam, double* V,
                        int64_t ldv, int32_t* converged, int64_t* iter)
{
    int rc = dense_args(h, n, A, lda);
    if (rc) return rc;
    if (!lam || !V || !converged || !iter) return SYMEIG_ERR_NULL;
    if (ldv < n) return SYMEIG_ERR_LD;
    begin_call(h);
    const size_t ws = (size_t)dense_scratch_doubles(n) + 1;
    CK(h->dense.ensure((ws + 2 * (size_t)n) * sizeof(double)));
    double* work = (double*)h->dense.ptr;
    double* e = work + ws;
    double* tau = e + n;
    rc = sytrd_scaled(h, n, A, lda, lam, e, tau, work);
    if (rc) return rc;
    rc = orgtr_dev(h->stream, n, A, lda, tau, V, ldv, work);
    if (rc) return rc;
    const double eps = 2.220446049250313e-16;
    return qr_dev<double>(h, lam, e, n, V, ldv, n, 128, eps, 100 * n, converged, iter);
}

int symeig_sytrd_f64(symeig_handle h, int64_t n, double* A, int64_t lda, double* d, double* e,
                     double* tau)
{
    int rc = dense_args(h, n, A, lda);
    if (rc) return rc;
    if (!d || (n > 1 && (!e || !tau))) return SYMEIG_ERR_NULL;
    const size_t nn = (size_t)n * n;
    CK(h->dense_io.ensure((nn + 3 * (size_t)n) * sizeof(double)));
    double* dA = (double*)h->dense_io.ptr;
    double *dd = dA + nn, *de = dd + n, *dt = de + n;
    cudaStream_t st = h->stream;
    CK(cudaMemcpy2DAsync(dA, n * sizeof(double), A, lda * sizeof(double), n * sizeof(double), n,
                         cudaMemcpyHostToDevice, st));
    rc = symeig_sytrd_f64_dev(h, n, dA, n, dd, de, dt);
    if (rc) return rc;
    CK(cudaMemcpy2DAsync(A, lda * sizeof(double), dA, n * sizeof(double), n * sizeof(double), n,
                         cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(d, dd, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (n > 1) {
        CK(cudaMemcpyAsync(e, de, (n - 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(tau, dt, (n - 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    return SYMEIG_OK;
}

int symeig_orgtr_f64(symeig_handle h, int64_t n, const double* A, int64_t lda, const double* tau,
                     double* Q, int64_t ldq)
{
    int rc = dense_args(h, n, A, lda);
    if (rc) return rc;
    if (!Q || (n > 1 && !tau)) return SYMEIG_ERR_NULL;
    if (ldq < n) return SYMEIG_ERR_LD;
    const size_t nn = (size_t)n * n;
    CK(h->dense_io.ensure((2 * nn + (size_t)n) * sizeof(double)));
    double* dA = (double*)h->dense_io.ptr;
    double *dQ = dA + nn, *dt = dQ + nn;
    cudaStream_t st = h->stream;
    CK(cudaMemcpy2DAsync(dA, n * sizeof(double), A, lda * sizeof(double), n * sizeof(double), n,
                         cudaMemcpyHostToDevice, st));
    if (n > 1) CK(cudaMemcpyAsync(dt, tau, (n - 1) * sizeof(double), cudaMemcpyHostToDevice, st));
    rc = symeig_orgtr_f64_dev(h, n, dA, n, dt, dQ, n);
    if (rc) return rc;
    CK(cudaMemcpy2DAsync(Q, ldq * sizeof(double), dQ, n * sizeof(double), n * sizeof(double), n,
                         cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return SYMEIG_OK;
}

int symeig_syev_f64(symeig_handle h, int64_t n, const double* A, int64_t lda, double* lam, double* V,
                    int64_t ldv, int32_t* converged, int64_t* iter)
{
    int rc = dense_args(h, n, A, lda);
    if (rc) return rc;
    if (!lam || !V || !converged || !iter) return SYMEIG_ERR_NULL;
    if (ldv < n) return SYMEIG_ERR_LD;
    auto t0 = std::chrono::steady_clock::now();
    const size_t nn = (size_t)n * n;
    CK(h->dense_io.ensure((2 * nn + (size_t)n) * sizeof(double)));
    double* dA = (double*)h->dense_io.ptr;
    double *dV = dA + nn, *dl = dV + nn;
    cudaStream_t st = h->stream;
    CK(cudaMemcpy2DAsync(dA, n * sizeof(double), A, lda * sizeof(double), n * sizeof(double), n,
                         cudaMemcpyHostToDevice, st));
    rc = symeig_syev_f64_dev(h, n, dA, n, dl, dV, n, converged, iter);
    if (rc) return rc;
    CK(cudaMemcpy2DAsync(V, ldv * sizeof(double), dV, n * sizeof(double), n * sizeof(double), n,
                         cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(lam, dl, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    h->stats.total_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return SYMEIG_OK;
}

int symeig_get_rotation_f64_dev(symeig_handle h, int64_t count, const double* f, const double* g,
                                double* c, double* s, double* r)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (count < 0) return SYMEIG_ERR_SIZE;
    if (count > 0 && (!f || !g || !c || !s || !r)) return SYMEIG_ERR_NULL;
    begin_call(h);
    CK(launch_get_rotation(count, f, g, c, s, r, h->chase_mode == 1 ? 1 : 0, h->stream));
    return SYMEIG_OK;
}

int symeig_mul_rn_f64_dev(symeig_handle h, int64_t count, const double* a, const double* b, double* out,
                          int32_t form)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (count < 0 || form < 0 || form > 1) return SYMEIG_ERR_SIZE;
    if (count > 0 && (!a || !b || !out)) return SYMEIG_ERR_NULL;
    begin_call(h);
    CK(launch_mul_rn(count, a, b, out, form, h->stream));
    return SYMEIG_OK;
}

int symeig_get_rotation_f64(symeig_handle h, int64_t count, const double* f, const double* g,
                            double* c, double* s, double* r)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (count < 0 || count > ((int64_t)1 << 40)) return SYMEIG_ERR_SIZE;
    if (count == 0) return SYMEIG_OK;
    if (!f || !g || !c || !s || !r) return SYMEIG_ERR_NULL;
    const size_t b = (size_t)count * sizeof(double);
    CK(h->rot.ensure(5 * b));
    double* base = (double*)h->rot.ptr;
    double *df = base, *dg = base + count, *dc = base + 2 * count, *ds = base + 3 * count,
           *dr = base + 4 * count;
    cudaStream_t st = h->stream;
    CK(cudaMemcpyAsync(df, f, b, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dg, g, b, cudaMemcpyHostToDevice, st));
    rc = symeig_get_rotation_f64_dev(h, count, df, dg, dc, ds, dr);
    if (rc) return rc;
    CK(cudaMemcpyAsync(c, dc, b, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(s, ds, b, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(r, dr, b, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return SYMEIG_OK;
}

int symeig_eigen_decomp_f64(symeig_handle h, double* d, double* e, int64_t n, double* Q,
                            int64_t ldq, int32_t* converged, int64_t* iter)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (n < 1) return SYMEIG_ERR_SIZE;
    if (!Q) return SYMEIG_ERR_NULL;
    if (ldq < n) return SYMEIG_ERR_LD;
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < n; ++i) Q[i + j * ldq] = (i == j) ? 1.0 : 0.0;
    const double eps = 2.220446049250313e-16;
    return qr_host<double>(h, d, e, n, Q, ldq, n, 128, eps, 100 * n, converged, iter);
}

}  // extern "C"
