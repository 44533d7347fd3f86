// adjoint.cu -- reverse-mode derivative of the tridiagonal eigensolve.
//
// For T = Q diag(lam) Q^T (columns of Q the eigenvectors of the symmetric tridiagonal with
// diagonal d and off-diagonal e), a loss L(lam, Q) with gradients glam = dL/dlam and
// gQ = dL/dQ has
//     Abar = Q M Q^T,   M = diag(glam) + F o (Q^T gQ),   F_ij = 1 / (lam_j - lam_i)  (i != j),
//     dL/dd_i = Abar_ii,   dL/de_i = Abar_{i,i+1} + Abar_{i+1,i}.
// (F_ii = 0, and F_ij = 0 where lam_i == lam_j: the formula assumes separated eigenvalues.)
// The reference has no derivative; this is the pullback behind the Julia rrule and the torch
// autograd Function of the host bindings.  Q is the solver's output, so no rotation history
// is stored.
//
// Two FP64 tensor-core GEMMs (dmma_tile.cuh: mma.sync m8n8k4 .f64, the FP64 MMA of sm_103a;
// tcgen05 has no f64 kind) with fused epilogues:
//   1. G = Q^T gQ, epilogue M_ij = i == j ? glam_i : G_ij / (lam_j - lam_i), M stored.
//   2. P = Q M, epilogue: per row i the partial sums over the CTA's columns k of
//        P_ik Q_ik (-> dd_i),  P_ik Q_{i+1,k} and P_ik Q_{i-1,k} (-> de_i, de_{i-1}),
//      written per column tile; Abar itself is never stored.
//   3. a reduction over column tiles in a fixed order (deterministic).
// A batch of matrices of one order runs with blockIdx.z = matrix.
#include <cuda_runtime.h>

#include "symeig.h"
#include "symeig_common.cuh"
#include "dmma_tile.cuh"

namespace symeig {
namespace {

using dmma::BM;
using dmma::BN;
constexpr int kAdjThreads = dmma::kThreads;

// 1. M = diag(glam) + F o (Q^T gQ), M column-major with leading dimension n.
__global__ void __launch_bounds__(kAdjThreads)
adjoint_m_kernel(const double* __restrict__ Q, int64_t ldq, const double* __restrict__ gQ,
                 int64_t ldg, const double* __restrict__ lam, const double* __restrict__ glam,
                 int64_t n, double* __restrict__ Mout, int64_t strideQ, int64_t strideG,
                 int64_t strideM)
{
    __shared__ dmma::Smem sm;
    const int64_t z = blockIdx.z;
    Q += z * strideQ;
    gQ += z * strideG;
    Mout += z * strideM;
    lam += z * n;
    glam += z * n;
    const int64_t i0 = (int64_t)blockIdx.y * BM, j0 = (int64_t)blockIdx.x * BN;
    double acc[4][4][2];
    // A(i, k) = Q(k, i): k contiguous; B(k, j) = gQ(k, j): k contiguous
    dmma::tile_gemm(Q, ldq, 1, gQ, 1, ldg, n, n, n, i0, j0, 0, n, acc, sm);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int grp = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int64_t i = i0 + wm + x * 8 + grp;
                const int64_t j = j0 + wn + y * 8 + tig * 2 + h;
                if (i >= n || j >= n) continue;
                double v;
                if (i == j) {
                    v = glam[i];
                } else {
                    const double gap = lam[j] - lam[i];
                    v = gap != 0.0 ? acc[x][y][h] / gap : 0.0;
                }
                Mout[i + j * n] = v;
            }
}

// 2. P = Q M and the per-row partial sums of the CTA's columns (see the file comment).
// part: [3][n_col_tiles][n]: 0 = P_ik Q_ik, 1 = P_ik Q_{i+1,k}, 2 = P_ik Q_{i-1,k}.
__global__ void __launch_bounds__(kAdjThreads)
adjoint_p_kernel(const double* __restrict__ Q, int64_t ldq, const double* __restrict__ M,
                 int64_t n, double* __restrict__ part, int64_t strideQ, int64_t strideM,
                 int64_t stridePart)
{
    __shared__ dmma::Smem sm;
    __shared__ double red[3][2][BM];
    const int64_t z = blockIdx.z;
    Q += z * strideQ;
    M += z * strideM;
    part += z * stridePart;
    const int64_t i0 = (int64_t)blockIdx.y * BM, k0 = (int64_t)blockIdx.x * BN;
    double acc[4][4][2];
    // A(i, j) = Q(i, j): i contiguous; B(j, k) = M(j, k): j contiguous
    dmma::tile_gemm(Q, 1, ldq, M, 1, n, n, n, n, i0, k0, 0, n, acc, sm);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int grp = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        const int r = wm + x * 8 + grp;
        const int64_t i = i0 + r;
        double sd = 0.0, su = 0.0, sl = 0.0;
        if (i < n) {
#pragma unroll
            for (int y = 0; y < 4; ++y)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int64_t k = k0 + wn + y * 8 + tig * 2 + h;
                    if (k >= n) continue;
                    const double p = acc[x][y][h];
                    sd = fma(p, Q[i + k * ldq], sd);
                    if (i + 1 < n) su = fma(p, Q[i + 1 + k * ldq], su);
                    if (i >= 1) sl = fma(p, Q[i - 1 + k * ldq], sl);
                }
        }
        // the 4 lanes of a group hold the same row: sum them
#pragma unroll
        for (int o = 1; o < 4; o <<= 1) {
            sd += __shfl_xor_sync(0xffffffffu, sd, o);
            su += __shfl_xor_sync(0xffffffffu, su, o);
            sl += __shfl_xor_sync(0xffffffffu, sl, o);
        }
        if (tig == 0) {
            red[0][warp & 1][r] = sd;
            red[1][warp & 1][r] = su;
            red[2][warp & 1][r] = sl;
        }
    }
    __syncthreads();
    const int64_t tiles = (n + BN - 1) / BN;
    for (int r = threadIdx.x; r < BM; r += blockDim.x) {
        const int64_t i = i0 + r;
        if (i >= n) continue;
#pragma unroll
        for (int t = 0; t < 3; ++t)
            part[((int64_t)t * tiles + blockIdx.x) * n + i] = red[t][0][r] + red[t][1][r];
    }
}

// 3. dd_i = sum_tiles part0[i];  de_i = sum_tiles (part1[i] + part2[i+1]).
__global__ void adjoint_reduce_kernel(const double* __restrict__ part, int64_t n, double* __restrict__ gd,
                                      double* __restrict__ ge, int64_t stridePart)
{
    const int64_t z = blockIdx.y;
    part += z * stridePart;
    gd += z * n;
    ge += z * (n > 1 ? n - 1 : 0);
    const int64_t tiles = (n + BN - 1) / BN;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double sd = 0.0, se = 0.0;
        for (int64_t t = 0; t < tiles; ++t) {
            sd += part[(0 * tiles + t) * n + i];
            if (i + 1 < n) se += part[(1 * tiles + t) * n + i] + part[(2 * tiles + t) * n + i + 1];
        }
        gd[i] = sd;
        if (i + 1 < n) ge[i] = se;
    }
}

// Eigenvalue-only loss (gQ = 0): dd_i = sum_k glam_k Q_ik^2, de_i = 2 sum_k glam_k Q_ik Q_{i+1,k}.
__global__ void adjoint_lambda_only_kernel(const double* __restrict__ Q, int64_t ldq,
                                           const double* __restrict__ glam, int64_t n,
                                           double* __restrict__ gd, double* __restrict__ ge,
                                           int64_t strideQ)
{
    const int64_t z = blockIdx.y;
    Q += z * strideQ;
    glam += z * n;
    gd += z * n;
    ge += z * (n > 1 ? n - 1 : 0);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double sd = 0.0, se = 0.0;
        for (int64_t k = 0; k < n; ++k) {
            const double q = Q[i + k * ldq];
            sd = fma(glam[k] * q, q, sd);
            if (i + 1 < n) se = fma(glam[k] * q, Q[i + 1 + k * ldq], se);
        }
        gd[i] = sd;
        if (i + 1 < n) ge[i] = 2.0 * se;
    }
}

}  // namespace

// Device-pointer adjoint for `count` matrices of order n stored back to back (Q, gQ with
// leading dimension n and stride n*n; lam, glam, gd with stride n; ge with stride n-1).
// scratch: count * (n*n + 3*ceil(n/64)*n) doubles.
int adjoint_dev(cudaStream_t s, int64_t count, int64_t n, const double* lam, const double* Q,
                const double* glam, const double* gQ, double* gd, double* ge, double* scratch)
{
    if (count <= 0 || n <= 0) return SYMEIG_OK;
    const int64_t tiles = (n + BN - 1) / BN;
    const int64_t strideQ = n * n, strideM = n * n, stridePart = 3 * tiles * n;
    if (count > 65535) return SYMEIG_ERR_SIZE;
    if (!gQ) {
        adjoint_lambda_only_kernel<<<dim3((unsigned)((n + 127) / 128), (unsigned)count), 128, 0, s>>>(
            Q, n, glam, n, gd, ge, strideQ);
        return cudaGetLastError() == cudaSuccess ? SYMEIG_OK : SYMEIG_ERR_CUDA;
    }
    double* Mbuf = scratch;
    double* part = scratch + count * strideM;
    const dim3 grid((unsigned)tiles, (unsigned)((n + BM - 1) / BM), (unsigned)count);
    adjoint_m_kernel<<<grid, kAdjThreads, 0, s>>>(Q, n, gQ, n, lam, glam, n, Mbuf, strideQ, strideQ, strideM);
    adjoint_p_kernel<<<grid, kAdjThreads, 0, s>>>(Q, n, Mbuf, n, part, strideQ, strideM, stridePart);
    adjoint_reduce_kernel<<<dim3((unsigned)((n + 255) / 256), (unsigned)count), 256, 0, s>>>(part, n, gd, ge, stridePart);
    return cudaGetLastError() == cudaSuccess ? SYMEIG_OK : SYMEIG_ERR_CUDA;
}

int64_t adjoint_scratch_doubles(int64_t count, int64_t n)
{
    const int64_t tiles = (n + BN - 1) / BN;
    return count * (n * n + 3 * tiles * n);
}

}  // namespace symeig
