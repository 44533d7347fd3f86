// noalloc.cu -- a bulk Givens apply that allocates nothing.
//
// Some callers of this library cannot allocate device memory at call time.  One kind owns
// the device through another allocator, such as a framework that reserved nearly all of
// HBM for its own pool up front: a cudaMalloc from this library would fail or fragment that
// pool.  Another kind cannot afford cudaMalloc's implicit device-wide synchronisation on a
// latency-critical path.  The handle-based entry points allocate
// (grow-only scratch, pinned status memory, streams), so those callers get this one instead:
// the FP64 wave-window apply with its wave table in a fixed, file-scope device array.
//
// The array costs every GPU that loads the library SYMEIG_NOALLOC_SCRATCH_BYTES of device
// memory until the process exits.  All calls share it: two calls whose kernels overlap on
// the GPU (different streams, or different host threads without ordering) race on the
// table and give wrong results; calls issued on one stream are ordered and safe.  The
// table-build kernel rewrites every table entry a pass reads before the pass runs, so the
// contents left by the previous call never need clearing.
//
// The calls are asynchronous, so a bounded wait that gave up inside a kernel (the error
// word below) cannot change their return value.  symeig_noalloc_status reads and clears
// that word after the caller's stream has drained.  Under lazy module loading (the CUDA
// default) the array is claimed when this file's module first loads on a device, i.e. at
// the first call there; symeig_noalloc_init does that step on its own, so a caller can run
// it before its own allocator takes the device's memory and before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "symeig.h"
#include "symeig_common.cuh"

namespace symeig {
namespace {

// The scratch: one pass's wave table, and the kernel's error word (set to 1 if a bounded
// wait inside the kernel gave up; read and cleared by symeig_noalloc_status).
static __device__ __align__(256) unsigned char g_noalloc_table[SYMEIG_NOALLOC_SCRATCH_BYTES];
static __device__ int g_noalloc_err;

constexpr int kMaxDevices = 64;
std::mutex g_setup_lock;
void* g_table_addr[kMaxDevices] = {};  // device address of g_noalloc_table, per device
void* g_err_addr[kMaxDevices] = {};    // device address of g_noalloc_err, per device

// Once per device, with that device current: resolve the device addresses of the arrays.
// In host code `g_noalloc_table` names a host-side stand-in, never a device address.
int table_address(void** table, int** err)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SYMEIG_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_setup_lock);
    if (!g_table_addr[dev]) {
        void* p = nullptr;
        void* q = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_table) != cudaSuccess || !p) return SYMEIG_ERR_CUDA;
        if (cudaGetSymbolAddress(&q, g_noalloc_err) != cudaSuccess || !q) return SYMEIG_ERR_CUDA;
        g_table_addr[dev] = p;
        g_err_addr[dev] = q;
    }
    *table = g_table_addr[dev];
    *err = (int*)g_err_addr[dev];
    return SYMEIG_OK;
}

}  // namespace
}  // namespace symeig

extern "C" int symeig_noalloc_init(void)
{
    void* table = nullptr;
    int* err = nullptr;
    return symeig::table_address(&table, &err);
}

extern "C" int symeig_noalloc_status(void* stream)
{
    void* table = nullptr;
    int* err = nullptr;
    int rc = symeig::table_address(&table, &err);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    int word = 0;
    if (cudaMemcpyAsync(&word, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return SYMEIG_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return SYMEIG_ERR_CUDA;
    if (word != 0) {
        if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) return SYMEIG_ERR_CUDA;
        if (cudaStreamSynchronize(s) != cudaSuccess) return SYMEIG_ERR_CUDA;
        return SYMEIG_ERR_TIMEOUT;
    }
    return SYMEIG_OK;
}

extern "C" int symeig_apply_givens_f64_noalloc(double* A, int64_t lda, int64_t m, int64_t n,
                                               const double* cs, int64_t k, void* stream)
{
    using namespace symeig;
    if (m < 0 || n < 0 || k < 0 || n > (int64_t)1 << 30) return SYMEIG_ERR_SIZE;
    if (m > 0 && n > 0 && !A) return SYMEIG_ERR_NULL;
    if (m > 0 && lda < m) return SYMEIG_ERR_LD;
    if (m == 0 || n < 2 || k == 0) return SYMEIG_OK;
    if (!cs) return SYMEIG_ERR_NULL;
    const int64_t per = 64;   // passes of the 64-layer tiles, whose tables the scratch holds
    if (apply_canonical_table_bytes<double>(n) > (size_t)SYMEIG_NOALLOC_SCRATCH_BYTES) return SYMEIG_ERR_SIZE;
    void* table = nullptr;
    int* err = nullptr;
    int rc = table_address(&table, &err);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    for (int64_t L0 = 0; L0 < k; L0 += per) {
        ApplyPass pass{0, n, L0, k - L0 < per ? k - L0 : per};
        if (apply_pass<double, double>(A, lda, m, cs, n - 1, nullptr, pass, table, err, s) != cudaSuccess)
            return SYMEIG_ERR_CUDA;
    }
    return SYMEIG_OK;
}
