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

// Tile shapes.  Both cover 64 layers per pass.
//   shape 0 = 8 lane groups of 8 layers: 4 rows per warp -- at m = 16384, 4096 warps, all
//             resident at <= 7 CTAs of 4 warps per SM (register budget 73), 6 or 7 warps per
//             SM sub-partition.  The FP64 choice: the FP64 unit (2 FMA per SM per clock on
//             GB300) is the limit and this shape balances it best.
//   shape 1 = 4 lane groups of 16 layers: 8 rows per warp, twice the rotations per wave for
//             the same per-wave overhead (shuffle, Q load/store, address arithmetic).  The
//             FP32 choice: FP32 is issue-bound, so overhead per rotation matters more than
//             the coarser balance.
template <typename T, int S> struct Cfg;
template <> struct Cfg<double, 0> { using Sh = Shape<double, 8, 8>; static constexpr int MINB = 7; };
template <> struct Cfg<double, 1> { using Sh = Shape<double, 16, 4>; static constexpr int MINB = 4; };
template <> struct Cfg<float, 0> { using Sh = Shape<float, 8, 8>; static constexpr int MINB = 7; };
template <> struct Cfg<float, 1> { using Sh = Shape<float, 16, 4>; static constexpr int MINB = 5; };

int g_shape[2] = {0, 1};  // [0] FP64, [1] FP32
template <typename T> int shape_index() { return g_shape[sizeof(T) == 8 ? 0 : 1]; }

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

template <typename T, int S>
__global__ void __launch_bounds__(kThreads, Cfg<T, S>::MINB)
wave_apply_kernel(T* __restrict__ Q, int64_t ldq, int64_t m, int32_t n_loc,
                  const unsigned char* __restrict__ table, int32_t n_chunks, int* __restrict__ err,
                  const T nz, int64_t rs)
{
    using Sh = typename Cfg<T, S>::Sh;
    __shared__ __align__(128) unsigned char ring[2][Sh::CHUNK];
    __shared__ __align__(8) uint64_t bar[2];
    wave::Staging<Sh> st{ring, bar, 0, 0};
    wave::staging_init(st);
    const int64_t row0 = (int64_t)blockIdx.x * Sh::ROWS;
    if (!wave::wave_tile<T, Sh>(Q, ldq, m, row0, n_loc, table, n_chunks, nz, st, rs)) {
        if (threadIdx.x == 0) atomicExch(err, 1);
    }
}

}  // namespace

template <typename T> int64_t apply_layers_per_pass() { return 64; }
template int64_t apply_layers_per_pass<double>();
template int64_t apply_layers_per_pass<float>();

template <typename T> size_t apply_table_bytes(int64_t n_loc, int64_t layers)
{
    (void)layers;
    // the larger of the two shapes' tables, so the tuning can change between calls
    return (size_t)std::max(Cfg<T, 0>::Sh::table_bytes(n_loc), Cfg<T, 1>::Sh::table_bytes(n_loc));
}
template size_t apply_table_bytes<double>(int64_t, int64_t);
template size_t apply_table_bytes<float>(int64_t, int64_t);

template <typename Tsrc, typename T, int S>
cudaError_t apply_pass_shape(T* Q, int64_t ldq, int64_t m, const Tsrc* grid, int64_t grid_rows,
                             const int32_t* place, const ApplyPass& pass, void* table, int* err,
                             cudaStream_t stream, cudaEvent_t ev_begin, cudaEvent_t ev_end)
{
    using Sh = typename Cfg<T, S>::Sh;
    if (m <= 0 || pass.n_loc < 2 || pass.layers <= 0) return cudaSuccess;
    const int64_t n_chunks = Sh::chunks(pass.n_loc);
    const int64_t total = n_chunks * Sh::CH * Sh::G * Sh::KB;
    int64_t tb_blocks = (total + 255) / 256;
    if (tb_blocks > 152 * 16) tb_blocks = 152 * 16;
    build_table_kernel<Tsrc, T, S><<<(unsigned)tb_blocks, 256, 0, stream>>>(
        (unsigned char*)table, n_chunks, grid, grid_rows, place, pass.c0, pass.n_loc, pass.L0,
        pass.layers);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int64_t blocks = (m + Sh::ROWS - 1) / Sh::ROWS;
    if (ev_begin) cudaEventRecord(ev_begin, stream);
    wave_apply_kernel<T, S><<<(unsigned)blocks, kThreads, 0, stream>>>(
        Q + pass.c0 * ldq, ldq, m, (int32_t)pass.n_loc, (const unsigned char*)table,
        (int32_t)n_chunks, err, (T)-0.0, pass.rs);
    e = cudaGetLastError();
    if (ev_end) cudaEventRecord(ev_end, stream);
    return e;
}

template <typename Tsrc, typename T>
cudaError_t apply_pass(T* Q, int64_t ldq, int64_t m, const Tsrc* grid, int64_t grid_rows,
                       const int32_t* place, const ApplyPass& pass, void* table, int* err,
                       cudaStream_t stream, cudaEvent_t ev_begin, cudaEvent_t ev_end)
{
    if (shape_index<T>() == 0)
        return apply_pass_shape<Tsrc, T, 0>(Q, ldq, m, grid, grid_rows, place, pass, table, err,
                                            stream, ev_begin, ev_end);
    return apply_pass_shape<Tsrc, T, 1>(Q, ldq, m, grid, grid_rows, place, pass, table, err, stream,
                                        ev_begin, ev_end);
}

void apply_set_shape(int fp64, int shape) { g_shape[fp64 ? 0 : 1] = shape ? 1 : 0; }
int apply_get_shape(int fp64) { return g_shape[fp64 ? 0 : 1]; }

template cudaError_t apply_pass<double, double>(double*, int64_t, int64_t, const double*, int64_t,
    const int32_t*, const ApplyPass&, void*, int*, cudaStream_t, cudaEvent_t, cudaEvent_t);
template cudaError_t apply_pass<float, float>(float*, int64_t, int64_t, const float*, int64_t,
    const int32_t*, const ApplyPass&, void*, int*, cudaStream_t, cudaEvent_t, cudaEvent_t);
template cudaError_t apply_pass<double, float>(float*, int64_t, int64_t, const double*, int64_t,
    const int32_t*, const ApplyPass&, void*, int*, cudaStream_t, cudaEvent_t, cudaEvent_t);

}  // namespace symeig
