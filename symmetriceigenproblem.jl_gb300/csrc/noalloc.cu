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
#include <cuda_runtime.h>

#include <mutex>

#include "symeig.h"
#include "symeig_common.cuh"

namespace symeig {
namespace {

// The scratch: one pass's wave table (sized for n + 71 waves x 64 (c,s) pairs of FP64).
static __device__ __align__(256) unsigned char g_noalloc_table[SYMEIG_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_lock;
void* g_table_addr[kMaxDevices] = {};  // device address of g_noalloc_table, per device

// Once per device, with that device current: resolve the device address of the array.  In
// host code `g_noalloc_table` names a host-side stand-in, never a device address.
int table_address(void** out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SYMEIG_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_setup_lock);
    if (!g_table_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_table) != cudaSuccess || !p) return SYMEIG_ERR_CUDA;
        g_table_addr[dev] = p;
    }
    *out = g_table_addr[dev];
    return SYMEIG_OK;
}

}  // namespace
}  // namespace symeig

extern "C" int symeig_apply_givens_f64_noalloc(double* A, int64_t lda, int64_t m, int64_t n,
                                               const double* cs, int64_t k, void* stream)
{
    using namespace symeig;
    if (m < 0 || n < 0 || k < 0) return SYMEIG_ERR_SIZE;
    if (m > 0 && n > 0 && !A) return SYMEIG_ERR_NULL;
    if (m > 0 && lda < m) return SYMEIG_ERR_LD;
    if (m == 0 || n < 2 || k == 0) return SYMEIG_OK;
    if (!cs) return SYMEIG_ERR_NULL;
    const int64_t per = apply_layers_per_pass<double>();
    if (apply_table_bytes<double>(n, per) > (size_t)SYMEIG_NOALLOC_SCRATCH_BYTES) return SYMEIG_ERR_SIZE;
    void* table = nullptr;
    int rc = table_address(&table);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    for (int64_t L0 = 0; L0 < k; L0 += per) {
        ApplyPass pass{0, n, L0, k - L0 < per ? k - L0 : per};
        if (apply_pass<double, double>(A, lda, m, cs, n - 1, nullptr, pass, table, s) != cudaSuccess)
            return SYMEIG_ERR_CUDA;
    }
    return SYMEIG_OK;
}
