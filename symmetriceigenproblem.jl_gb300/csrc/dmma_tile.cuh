// dmma_tile.cuh -- a 64 x 64 FP64 tensor-core tile product for the dense kernels (the adjoint
// GEMMs and the dense -> tridiagonal reduction).
//
// One CTA of 128 threads (4 warps, 2 x 2, each 32 x 32) computes the 64 x 64 tile
// C[i0 .. i0+63][j0 .. j0+63] of A[M x K] * B[K x N] with mma.sync.m8n8k4 .f64 (the FP64 MMA
// of sm_103a; tcgen05 has no f64 kind).  A(i, k) is read at a + i * a_si + k * a_sk and
// B(k, j) at b + k * b_sk + j * b_sj; each is staged through shared memory in the order that
// makes its global loads coalesced (the unit stride fastest).  Out-of-range elements read as 0.
// acc[x][y][h] holds the warp's 4 x 4 grid of 8 x 8 MMA tiles: element
//   row  wm + 8 x + (lane >> 2),   column  wn + 8 y + 2 (lane & 3) + h
// with wm = 32 (warp >> 1), wn = 32 (warp & 1) (tile_row / tile_col below).
#pragma once
#include <cstdint>

namespace symeig {
namespace dmma {

constexpr int BM = 64, BN = 64, BK = 16;  // CTA tile
constexpr int kThreads = 128;             // 4 warps
constexpr int SPAD = 2;                   // smem row padding (doubles)

__device__ __forceinline__ void mma(double (&c)[2], double a, double b)
{
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                 : "+d"(c[0]), "+d"(c[1]) : "d"(a), "d"(b));
}

__device__ __forceinline__ int tile_row(int x)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    return (warp >> 1) * 32 + x * 8 + (lane >> 2);
}
__device__ __forceinline__ int tile_col(int y, int h)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    return (warp & 1) * 32 + y * 8 + (lane & 3) * 2 + h;
}

struct Smem {
    double A[BM][BK + SPAD];
    double B[BN][BK + SPAD];
};

__device__ __forceinline__ void tile_gemm(const double* __restrict__ a, int64_t a_si, int64_t a_sk,
                                          const double* __restrict__ b, int64_t b_sk, int64_t b_sj,
                                          int64_t M, int64_t N, int64_t K, int64_t i0, int64_t j0,
                                          int64_t k_begin, int64_t k_end, double (&acc)[4][4][2],
                                          Smem& sm)
{
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int grp = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) acc[x][y][0] = acc[x][y][1] = 0.0;
    const bool a_kfast = (a_sk == 1);
    const bool b_kfast = (b_sk == 1);
    if (k_end > K) k_end = K;
    for (int64_t k0 = k_begin; k0 < k_end; k0 += BK) {
#pragma unroll
        for (int q = 0; q < (BM * BK) / kThreads; ++q) {
            const int e = tid + q * kThreads;
            int r, kk;
            if (a_kfast) { r = e / BK; kk = e % BK; } else { kk = e / BM; r = e % BM; }
            const int64_t gi = i0 + r, gk = k0 + kk;
            sm.A[r][kk] = (gi < M && gk < k_end) ? a[gi * a_si + gk * a_sk] : 0.0;
        }
#pragma unroll
        for (int q = 0; q < (BN * BK) / kThreads; ++q) {
            const int e = tid + q * kThreads;
            int c, kk;
            if (b_kfast) { c = e / BK; kk = e % BK; } else { kk = e / BN; c = e % BN; }
            const int64_t gj = j0 + c, gk = k0 + kk;
            sm.B[c][kk] = (gj < N && gk < k_end) ? b[gk * b_sk + gj * b_sj] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < BK; ks += 4) {
            double af[4], bf[4];
#pragma unroll
            for (int x = 0; x < 4; ++x) af[x] = sm.A[wm + x * 8 + grp][ks + tig];
#pragma unroll
            for (int y = 0; y < 4; ++y) bf[y] = sm.B[wn + y * 8 + grp][ks + tig];
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
                for (int y = 0; y < 4; ++y) mma(acc[x][y], af[x], bf[y]);
        }
        __syncthreads();
    }
}

}  // namespace dmma
}  // namespace symeig
