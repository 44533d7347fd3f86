// apply.cu -- the wave-window Givens kernel: Q <- Q * prod of a grid of column rotations.
//
// Replaces bulk_wave_order_2x2_rmul[_parallel]! (src/wave.jl:36-162) and its fused SIMD
// kernels (src/bulk_givens.jl:4-279).  The reference streams all m rows of 4 columns per
// fused block and relies on cache for reuse across waves; here every thread owns one row of
// Q and keeps a sliding window of KB+1 columns of that row in registers, so each element
// of Q is loaded once and stored once per pass.
//
// Order of the rotations.  Rotation (i, L) acts on columns (i, i+1).  The reference's wave
// order applies (i, L) after (i-1, L) and after (i+1, L-1); per element of Q that is the
// same sequence of rotations as the layer-major loop "for L, for i".  This kernel walks
// waves t = 0, 1, 2, ... of one group of KB layers: wave t applies rotation (t-1-l, l) for
// l = 0..KB-1, i.e. the pairs of columns (t-1-l, t-l) from right to left, which respects
// both dependencies.  After wave t, column t-KB is final for the group.
//
// Layer groups.  One pass covers G groups of KB layers.  The G groups of a row run in the
// G lane groups of one warp (32/G rows per warp); group g lags group g-1 by KB+1 waves and
// receives its input columns from group g-1 through a warp shuffle, so a pass reads and
// writes Q exactly once and every warp holds G-fold more independent work than a warp of
// 32 rows would.  Group 0 loads columns of Q; group G-1 stores them.
//
// (c,s) staging.  The host-side table builder lays the rotations out per iteration: the
// G*KB pairs one warp needs in iteration t are contiguous.  Rotations outside the grid or
// above a column's layer count are stored as (1, 0), so the inner loop has no bounds logic.
#include "symeig_common.cuh"

namespace symeig {

namespace {

template <typename T> struct Cfg;
// FP64: the FP64 unit (two FP64 FMA per SM per clock on GB300) is the limit; 8 groups of 8
// layers give 4 rows per warp and enough warps to keep every SM sub-partition busy.
template <> struct Cfg<double> { static constexpr int KB = 8; static constexpr int G = 8; };
// FP32: same shape; the FP32 pipe is 64x faster, so load/issue overheads matter more.
template <> struct Cfg<float>  { static constexpr int KB = 8; static constexpr int G = 8; };

constexpr int kThreads = 128;

template <typename T>
__host__ __device__ constexpr int64_t n_iterations(int64_t n_loc, int KB, int G)
{
    // waves 0 .. n_loc+KB-1 for group 0, plus the lag of the last group
    return n_loc + KB + (int64_t)(G - 1) * (KB + 1);
}

template <typename Tsrc, typename T, int KB, int G>
__global__ void __launch_bounds__(256)
build_table_kernel(typename Pair<T>::type* __restrict__ table, int64_t n_iter,
                   const Tsrc* __restrict__ grid, int64_t grid_rows,
                   const int32_t* __restrict__ thick, int64_t c0, int64_t n_loc,
                   int64_t L0, int64_t layers)
{
    using P2 = typename Pair<T>::type;
    const int64_t total = n_iter * G * KB;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = idx / (G * KB);
        const int g = (int)((idx / KB) % G);
        const int l = (int)(idx % KB);
        const int64_t tg = t - (int64_t)g * (KB + 1);
        const int64_t i_loc = tg - 1 - l;
        const int64_t lay = (int64_t)g * KB + l;  // layer within the pass
        Tsrc c = Tsrc(1), s = Tsrc(0);
        if (i_loc >= 0 && i_loc <= n_loc - 2 && lay < layers) {
            const int64_t i = c0 + i_loc;
            const int64_t L = L0 + lay;
            if (thick == nullptr || L < (int64_t)thick[i]) {
                const Tsrc* p = grid + 2 * (i + L * grid_rows);
                c = p[0];
                s = p[1];
            }
        }
        P2 v;
        v.x = (T)c;
        v.y = (T)s;
        table[idx] = v;
    }
}

template <typename T, int KB, int G>
__global__ void __launch_bounds__(kThreads)
wave_apply_kernel(T* __restrict__ Q, int64_t ldq, int64_t m, int64_t n_loc,
                  const typename Pair<T>::type* __restrict__ table, int64_t n_iter)
{
    using P2 = typename Pair<T>::type;
    constexpr int RPW = 32 / G;  // rows per warp
    const int lane = threadIdx.x & 31;
    const int g = lane / RPW;
    const int rl = lane - g * RPW;
    const int64_t warp = ((int64_t)blockIdx.x * kThreads + threadIdx.x) >> 5;
    const int64_t row = warp * RPW + rl;
    const bool row_ok = row < m;
    T* __restrict__ qrow = Q + (row_ok ? row : 0);

    T win[KB + 1];
#pragma unroll
    for (int q = 0; q <= KB; ++q) win[q] = T(0);
    T xout = T(0);

    const P2* __restrict__ tb = table + (int64_t)g * KB;
    const int64_t tstride = (int64_t)G * KB;

    P2 cs_next[KB];
#pragma unroll
    for (int l = 0; l < KB; ++l) cs_next[l] = tb[l];
    // group 0 prefetches the next input column
    T xin_next = T(0);
    if (g == 0 && row_ok && n_loc > 0) xin_next = qrow[0];

    for (int64_t t = 0; t < n_iter; ++t) {
        P2 cs[KB];
#pragma unroll
        for (int l = 0; l < KB; ++l) cs[l] = cs_next[l];
        if (t + 1 < n_iter) {
            const P2* p = tb + (t + 1) * tstride;
#pragma unroll
            for (int l = 0; l < KB; ++l) cs_next[l] = p[l];
        }
        const int64_t tg = t - (int64_t)g * (KB + 1);

        T xin = __shfl_up_sync(0xffffffffu, xout, RPW);
        if (g == 0) {
            xin = xin_next;
            const int64_t nc = tg + 1;
            xin_next = (row_ok && nc < n_loc) ? qrow[nc * ldq] : T(0);
        }
#pragma unroll
        for (int q = 0; q < KB; ++q) win[q] = win[q + 1];
        win[KB] = xin;

#pragma unroll
        for (int l = 0; l < KB; ++l) rot(win[KB - 1 - l], win[KB - l], cs[l].x, cs[l].y);

        xout = win[0];
        if (g == G - 1) {
            const int64_t col = tg - KB;
            if (row_ok && col >= 0 && col < n_loc) qrow[col * ldq] = xout;
        }
    }
}

}  // namespace

template <typename T> int64_t apply_layers_per_pass() { return (int64_t)Cfg<T>::KB * Cfg<T>::G; }
template int64_t apply_layers_per_pass<double>();
template int64_t apply_layers_per_pass<float>();

template <typename T> size_t apply_table_bytes(int64_t n_loc, int64_t layers)
{
    (void)layers;
    constexpr int KB = Cfg<T>::KB, G = Cfg<T>::G;
    return (size_t)n_iterations<T>(n_loc, KB, G) * G * KB * sizeof(typename Pair<T>::type);
}
template size_t apply_table_bytes<double>(int64_t, int64_t);
template size_t apply_table_bytes<float>(int64_t, int64_t);

template <typename Tsrc, typename T>
cudaError_t apply_pass(T* Q, int64_t ldq, int64_t m, const Tsrc* grid, int64_t grid_rows,
                       const int32_t* thick, const ApplyPass& pass, void* table,
                       cudaStream_t stream, cudaEvent_t ev_begin, cudaEvent_t ev_end)
{
    constexpr int KB = Cfg<T>::KB, G = Cfg<T>::G;
    using P2 = typename Pair<T>::type;
    if (m <= 0 || pass.n_loc < 2 || pass.layers <= 0) return cudaSuccess;
    const int64_t n_iter = n_iterations<T>(pass.n_loc, KB, G);
    const int64_t total = n_iter * G * KB;
    int64_t tb_blocks = (total + 255) / 256;
    if (tb_blocks > 152 * 16) tb_blocks = 152 * 16;
    build_table_kernel<Tsrc, T, KB, G><<<(unsigned)tb_blocks, 256, 0, stream>>>(
        (P2*)table, n_iter, grid, grid_rows, thick, pass.c0, pass.n_loc, pass.L0, pass.layers);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    constexpr int RPW = 32 / G;
    const int64_t warps = (m + RPW - 1) / RPW;
    const int64_t blocks = (warps * 32 + kThreads - 1) / kThreads;
    if (ev_begin) cudaEventRecord(ev_begin, stream);
    wave_apply_kernel<T, KB, G><<<(unsigned)blocks, kThreads, 0, stream>>>(
        Q + pass.c0 * ldq, ldq, m, pass.n_loc, (const P2*)table, n_iter);
    err = cudaGetLastError();
    if (ev_end) cudaEventRecord(ev_end, stream);
    return err;
}

template cudaError_t apply_pass<double, double>(double*, int64_t, int64_t, const double*, int64_t,
    const int32_t*, const ApplyPass&, void*, cudaStream_t, cudaEvent_t, cudaEvent_t);
template cudaError_t apply_pass<float, float>(float*, int64_t, int64_t, const float*, int64_t,
    const int32_t*, const ApplyPass&, void*, cudaStream_t, cudaEvent_t, cudaEvent_t);
template cudaError_t apply_pass<double, float>(float*, int64_t, int64_t, const double*, int64_t,
    const int32_t*, const ApplyPass&, void*, cudaStream_t, cudaEvent_t, cudaEvent_t);

}  // namespace symeig
