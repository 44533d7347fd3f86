// sytrd.cu -- dense symmetric -> tridiagonal reduction and its orthogonal factor: the step
// before qr_algorithm! when the input is a dense symmetric matrix.  The reference has none
// (its callers supply a SymTridiagonal); this follows LAPACK's dsytrd / dlatrd / dorgtr with
// UPLO = 'L'.
//
// A (n x n, column-major, both triangles stored) = Q T Q^T with T symmetric tridiagonal
// (d, e) and Q = H_0 H_1 ... H_{n-2},  H_j = I - tau_j v_j v_j^T,  v_j = (0, .., 0, 1, x_j)
// with the 1 in row j+1.  Panels of NB = 64 columns:
//   for each column j of a panel (i = j - p earlier reflectors of the panel):
//     a(j:n, j) -= V W(j, 0:i)^T + W V(j, 0:i)^T            (the panel's updates, lazily)
//     reflector of a(j+1:n, j):  beta = -sign(alpha) ||(alpha, x)||,  tau = (beta - alpha)/beta,
//       x /= alpha - beta   (dlarfg; x == 0 gives tau = 0, H = I)
//     w = tau (A22 v - W (V^T v) - V (W^T v));   w -= (tau/2) (w^T v) v
//   after the panel:  A(q:n, q:n) -= V W^T + W V^T     (q = p + pb; both triangles)
// The matrix-vector product A22 v of each column is the O(n^2) part; on GB300 it is bound by
// the FP64 pipe (one FMA per element read) and runs on all SMs.  The trailing update is one
// FP64 tensor-core GEMM (dmma_tile.cuh) of inner dimension 2 pb.  Every reduction sums in a
// fixed order, so results are deterministic.
// On exit, as in LAPACK: A's diagonal and first subdiagonal hold T, x_j lies below the
// subdiagonal of column j, tau_j in tau.
//
// orgtr forms Q by backward accumulation of the panels in compact WY form (dlarft / dlarfb):
//   Q(R, R) -= (V T) (V^T Q(R, R)),   R = rows and columns p+1 .. n-1,
// with T the pb x pb upper-triangular factor from V^T V; V^T V and V^T Q are long inner sums
// and run split over K.
//
// Range: the reflector norms are plain sums of squares, so |a_ij| must lie within 2^+-500
// (the host entry points scale A by a power of two into [2^-2, 2^2] around its largest entry).
#include <cuda_runtime.h>

#include "dmma_tile.cuh"
#include "symeig.h"
#include "symeig_common.cuh"

namespace symeig {
namespace {

constexpr int NB = 64;    // panel width
constexpr int RT = 256;   // rows per CTA in the column kernels
constexpr int GCH = 256;  // columns per CTA in the matrix-vector product
constexpr int KCH = 512;  // inner-dimension chunk of the split-K products

// sum over the CTA in a fixed order; the result is valid in thread 0
__device__ double block_sum(double v, double* sh)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[k];
    return s;
}

// a(j:n, j) -= V W(j,:)^T + W V(j,:)^T over the panel's i earlier reflectors;
// part[b] = sum over this CTA's rows r >= j+2 of a(r, j)^2.
// VW: n x 2pb, columns [0, pb) = V, [pb, 2pb) = W (leading dimension n).
__global__ void __launch_bounds__(RT)
col_update_kernel(double* __restrict__ A, int64_t lda, int64_t n, int64_t j, int i, int pb,
                  const double* __restrict__ VW, double* __restrict__ part)
{
    __shared__ double vj[NB], wj[NB], sh[32];
    for (int t = threadIdx.x; t < i; t += blockDim.x) {
        vj[t] = VW[j + (int64_t)t * n];
        wj[t] = VW[j + (int64_t)(pb + t) * n];
    }
    __syncthreads();
    const int64_t r = j + (int64_t)blockIdx.x * RT + threadIdx.x;
    double x2 = 0.0;
    if (r < n) {
        double a = A[r + j * lda];
        for (int t = 0; t < i; ++t) {
            a = fma(-VW[r + (int64_t)t * n], wj[t], a);
            a = fma(-VW[r + (int64_t)(pb + t) * n], vj[t], a);
        }
        A[r + j * lda] = a;
        if (r >= j + 2) x2 = a * a;
    }
    const double s = block_sum(x2, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// the reflector's scalars (dlarfg): d_j, e_j = beta, tau_j; sc = {tau, 1/(alpha-beta), beta}
__global__ void __launch_bounds__(RT)
reflector_kernel(const double* __restrict__ A, int64_t lda, int64_t j, const double* __restrict__ part,
                 int nparts, double* __restrict__ d, double* __restrict__ e, double* __restrict__ tau,
                 double* __restrict__ sc)
{
    __shared__ double sh[32];
    double v = 0.0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) v += part[b];
    const double s = block_sum(v, sh);
    if (threadIdx.x == 0) {
        const double alpha = A[j + 1 + j * lda];
        d[j] = A[j + j * lda];
        double t, scale, beta;
        if (s == 0.0) {
            t = 0.0;
            beta = alpha;
            scale = 0.0;
        } else {
            const double nrm = sqrt(fma(alpha, alpha, s));
            beta = alpha >= 0.0 ? -nrm : nrm;
            t = (beta - alpha) / beta;
            scale = 1.0 / (alpha - beta);
        }
        e[j] = beta;
        tau[j] = t;
        sc[0] = t;
        sc[1] = scale;
        sc[2] = beta;
    }
}

// v (rows j+1..n-1) into VW column i and WV column pb+i, x_j into A below the subdiagonal,
// e_j on the subdiagonal; dpart[b][t] = (V_t . v), dpart[b][NB+t] = (W_t . v) over the CTA.
__global__ void __launch_bounds__(RT)
make_v_kernel(double* __restrict__ A, int64_t lda, int64_t n, int64_t j, int i, int pb,
              double* __restrict__ VW, double* __restrict__ WV, const double* __restrict__ sc,
              double* __restrict__ dpart)
{
    __shared__ double sh[32];
    const double scale = sc[1], beta = sc[2];
    const int64_t r = j + 1 + (int64_t)blockIdx.x * RT + threadIdx.x;
    double v = 0.0;
    if (r < n) {
        if (r == j + 1) {
            v = 1.0;
            A[r + j * lda] = beta;
        } else {
            v = A[r + j * lda] * scale;
            A[r + j * lda] = v;
        }
        VW[r + (int64_t)i * n] = v;
        WV[r + (int64_t)(pb + i) * n] = v;
    }
    for (int t = 0; t < i; ++t) {
        const double p1 = r < n ? VW[r + (int64_t)t * n] * v : 0.0;
        const double p2 = r < n ? VW[r + (int64_t)(pb + t) * n] * v : 0.0;
        const double s1 = block_sum(p1, sh);
        const double s2 = block_sum(p2, sh);
        if (threadIdx.x == 0) {
            dpart[(int64_t)blockIdx.x * 2 * NB + t] = s1;
            dpart[(int64_t)blockIdx.x * 2 * NB + NB + t] = s2;
        }
    }
}

// ypart[c][r] = sum over the column chunk c of A(r, col) v(col), rows and columns j+1..n-1
__global__ void __launch_bounds__(RT)
symv_kernel(const double* __restrict__ A, int64_t lda, int64_t n, int64_t j,
            const double* __restrict__ v, double* __restrict__ ypart)
{
    __shared__ double vs[GCH];
    const int64_t c0 = j + 1 + (int64_t)blockIdx.y * GCH;
    const int64_t c1 = c0 + GCH < n ? c0 + GCH : n;
    for (int64_t c = c0 + threadIdx.x; c < c1; c += blockDim.x) vs[c - c0] = v[c];
    __syncthreads();
    const int64_t r = j + 1 + (int64_t)blockIdx.x * RT + threadIdx.x;
    if (r >= n) return;
    const double* col = A + r + c0 * lda;
    const int len = (int)(c1 - c0);
    double a0 = 0.0, a1 = 0.0;
    int c = 0;
    for (; c + 1 < len; c += 2) {
        a0 = fma(col[c * lda], vs[c], a0);
        a1 = fma(col[(c + 1) * lda], vs[c + 1], a1);
    }
    if (c < len) a0 = fma(col[c * lda], vs[c], a0);
    ypart[(int64_t)blockIdx.y * n + r] = a0 + a1;
}

// w = tau (A22 v - W (V^T v) - V (W^T v)) into VW column pb+i and WV column i;
// wpart[b] = (w . v) over the CTA.
__global__ void __launch_bounds__(RT)
w_kernel(int64_t n, int64_t j, int i, int pb, double* __restrict__ VW, double* __restrict__ WV,
         const double* __restrict__ ypart, int nchunks, const double* __restrict__ dpart,
         int nparts, const double* __restrict__ sc, double* __restrict__ wpart)
{
    __shared__ double c1[NB], c2[NB], sh[32];
    for (int t = threadIdx.x; t < i; t += blockDim.x) {
        double s1 = 0.0, s2 = 0.0;
        for (int b = 0; b < nparts; ++b) {
            s1 += dpart[(int64_t)b * 2 * NB + t];
            s2 += dpart[(int64_t)b * 2 * NB + NB + t];
        }
        c1[t] = s1;
        c2[t] = s2;
    }
    __syncthreads();
    const double t_ = sc[0];
    const int64_t r = j + 1 + (int64_t)blockIdx.x * RT + threadIdx.x;
    double wv = 0.0;
    if (r < n) {
        double y = 0.0;
        for (int b = 0; b < nchunks; ++b) y += ypart[(int64_t)b * n + r];
        for (int t = 0; t < i; ++t) {
            y = fma(-VW[r + (int64_t)(pb + t) * n], c1[t], y);
            y = fma(-VW[r + (int64_t)t * n], c2[t], y);
        }
        const double w = t_ * y;
        VW[r + (int64_t)(pb + i) * n] = w;
        WV[r + (int64_t)i * n] = w;
        wv = w * VW[r + (int64_t)i * n];
    }
    const double s = block_sum(wv, sh);
    if (threadIdx.x == 0) wpart[blockIdx.x] = s;
}

// w += -(tau/2) (w . v) v
__global__ void __launch_bounds__(RT)
w_fix_kernel(int64_t n, int64_t j, int i, int pb, double* __restrict__ VW, double* __restrict__ WV,
             const double* __restrict__ sc, const double* __restrict__ wpart, int nparts)
{
    __shared__ double a2;
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < nparts; ++b) s += wpart[b];
        a2 = -0.5 * sc[0] * s;
    }
    __syncthreads();
    const int64_t r = j + 1 + (int64_t)blockIdx.x * RT + threadIdx.x;
    if (r < n) {
        const double w = fma(a2, VW[r + (int64_t)i * n], VW[r + (int64_t)(pb + i) * n]);
        VW[r + (int64_t)(pb + i) * n] = w;
        WV[r + (int64_t)i * n] = w;
    }
}

// A(q:n, q:n) -= [V W] [W V]^T  (inner dimension 2 pb), both triangles
__global__ void __launch_bounds__(dmma::kThreads)
trailing_update_kernel(double* __restrict__ A, int64_t lda, int64_t n, int64_t q, int pb,
                       const double* __restrict__ VW, const double* __restrict__ WV)
{
    __shared__ dmma::Smem sm;
    const int64_t m = n - q;
    const int64_t i0 = (int64_t)blockIdx.y * dmma::BM, j0 = (int64_t)blockIdx.x * dmma::BN;
    double acc[4][4][2];
    dmma::tile_gemm(VW + q, 1, n, WV + q, n, 1, m, m, 2 * pb, i0, j0, 0, 2 * pb, acc, sm);
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int64_t ii = i0 + dmma::tile_row(x), jj = j0 + dmma::tile_col(y, h);
                if (ii < m && jj < m) A[(q + ii) + (q + jj) * lda] -= acc[x][y][h];
            }
}

__global__ void last_diag_kernel(const double* __restrict__ A, int64_t lda, int64_t n, double* __restrict__ d)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) d[n - 1] = A[(n - 1) + (n - 1) * lda];
}

// ---- orgtr ---------------------------------------------------------------------------------

__global__ void identity_kernel(double* __restrict__ Q, int64_t ldq, int64_t n)
{
    const int64_t total = n * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t % n, c = t / n;
        Q[r + c * ldq] = r == c ? 1.0 : 0.0;
    }
}

// Vp (m x pb, leading dimension m): column i is v_{p+i} on rows p+1 .. n-1
__global__ void extract_v_kernel(const double* __restrict__ A, int64_t lda, int64_t n, int64_t p,
                                 int pb, double* __restrict__ Vp)
{
    const int64_t m = n - p - 1;
    const int64_t total = m * pb;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t l = t % m, i = t / m;
        const int64_t r = p + 1 + l, jj = p + i;
        double v;
        if (r < jj + 1) v = 0.0;
        else if (r == jj + 1) v = 1.0;
        else v = A[r + jj * lda];
        Vp[l + i * m] = v;
    }
}

// split-K partial tiles of op(X)[M x K] op(Y)[K x N] for M, N <= 64 (one tile), K chunk z:
// out[z][i + 64 j]
__global__ void __launch_bounds__(dmma::kThreads)
splitk_tile_kernel(const double* __restrict__ a, int64_t a_si, int64_t a_sk,
                   const double* __restrict__ b, int64_t b_sk, int64_t b_sj, int64_t M, int64_t N,
                   int64_t K, double* __restrict__ out)
{
    __shared__ dmma::Smem sm;
    const int64_t kb = (int64_t)blockIdx.z * KCH;
    const int64_t i0 = (int64_t)blockIdx.y * dmma::BM, j0 = (int64_t)blockIdx.x * dmma::BN;
    double acc[4][4][2];
    dmma::tile_gemm(a, a_si, a_sk, b, b_sk, b_sj, M, N, K, i0, j0, kb, kb + KCH, acc, sm);
    const int64_t tiles_m = (M + dmma::BM - 1) / dmma::BM;
    double* o = out + ((int64_t)blockIdx.z * tiles_m * ((N + dmma::BN - 1) / dmma::BN) +
                       (int64_t)blockIdx.x * tiles_m + blockIdx.y) * dmma::BM * dmma::BN;
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y)
#pragma unroll
            for (int h = 0; h < 2; ++h) o[dmma::tile_row(x) + dmma::BM * dmma::tile_col(y, h)] = acc[x][y][h];
}

// Y[pb x m] (leading dimension pb) = sum over K chunks of the split-K tiles of Vp^T Q
__global__ void reduce_tiles_kernel(const double* __restrict__ part, int64_t M, int64_t N,
                                    int nk, double* __restrict__ Y, int64_t ldy)
{
    const int64_t tiles_m = (M + dmma::BM - 1) / dmma::BM, tiles_n = (N + dmma::BN - 1) / dmma::BN;
    const int64_t total = M * N;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t % M, jcol = t / M;
        const int64_t ti = i / dmma::BM, tj = jcol / dmma::BN;
        const int64_t off = (tj * tiles_m + ti) * dmma::BM * dmma::BN + (i % dmma::BM) + dmma::BM * (jcol % dmma::BN);
        double s = 0.0;
        for (int z = 0; z < nk; ++z) s += part[(int64_t)z * tiles_m * tiles_n * dmma::BM * dmma::BN + off];
        Y[i + jcol * ldy] = s;
    }
}

// T (pb x pb upper triangular, leading dimension NB) of the panel from G = V^T V and tau:
// T(i, i) = tau_i,  T(r, i) = -tau_i sum_{c = r}^{i-1} T(r, c) G(c, i)   (dlarft, forward)
__global__ void tfactor_kernel(const double* __restrict__ G, int64_t ldg, const double* __restrict__ tau,
                               int pb, double* __restrict__ T)
{
    __shared__ double Ts[NB][NB + 1];
    const int r = threadIdx.x;
    for (int i = 0; i < pb; ++i) {
        if (r < i) {
            double s = 0.0;
            for (int c = r; c < i; ++c) s = fma(Ts[r][c], G[c + i * ldg], s);
            Ts[r][i] = -tau[i] * s;
        } else if (r == i) {
            Ts[i][i] = tau[i];
        } else if (r < NB) {
            Ts[r][i] = 0.0;
        }
        __syncthreads();
    }
    for (int i = 0; i < pb; ++i)
        if (r < pb) T[r + i * NB] = Ts[r][i];
}

// VT[m x pb] = Vp T
__global__ void vt_kernel(const double* __restrict__ Vp, int64_t m, int pb, const double* __restrict__ T,
                          double* __restrict__ VT)
{
    __shared__ double Ts[NB * NB];
    for (int t = threadIdx.x; t < NB * NB; t += blockDim.x) Ts[t] = T[t];
    __syncthreads();
    const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= m) return;
    for (int i = 0; i < pb; ++i) {
        double s = 0.0;
        for (int c = 0; c <= i; ++c) s = fma(Vp[l + (int64_t)c * m], Ts[c + i * NB], s);
        VT[l + (int64_t)i * m] = s;
    }
}

// Q(R, R) -= VT Y   (R = p+1 .. n-1; inner dimension pb)
__global__ void __launch_bounds__(dmma::kThreads)
wy_update_kernel(double* __restrict__ Q, int64_t ldq, int64_t p1, int64_t m, int pb,
                 const double* __restrict__ VT, const double* __restrict__ Y)
{
    __shared__ dmma::Smem sm;
    const int64_t i0 = (int64_t)blockIdx.y * dmma::BM, j0 = (int64_t)blockIdx.x * dmma::BN;
    double acc[4][4][2];
    dmma::tile_gemm(VT, 1, m, Y, 1, pb, m, m, pb, i0, j0, 0, pb, acc, sm);
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int64_t ii = i0 + dmma::tile_row(x), jj = j0 + dmma::tile_col(y, h);
                if (ii < m && jj < m) Q[(p1 + ii) + (p1 + jj) * ldq] -= acc[x][y][h];
            }
}

__global__ void maxabs_kernel(const double* __restrict__ A, int64_t lda, int64_t n, double* __restrict__ out)
{
    __shared__ double sh[32];
    double m = 0.0;
    const int64_t total = n * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x)
        m = fmax(m, fabs(A[(t % n) + (t / n) * lda]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) r = fmax(r, sh[k]);
        // non-negative doubles order as their bit patterns
        atomicMax(reinterpret_cast<unsigned long long*>(out), (unsigned long long)__double_as_longlong(r));
    }
}

__global__ void scale_kernel(double* __restrict__ A, int64_t lda, int64_t n, double f)
{
    const int64_t total = n * n;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x)
        A[(t % n) + (t / n) * lda] *= f;
}

__global__ void tridiag_unscale_kernel(double* __restrict__ A, int64_t lda, int64_t n, double* __restrict__ d,
                                       double* __restrict__ e, double f)
{
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        d[t] *= f;
        A[t + t * lda] = d[t];
        if (t + 1 < n) {
            e[t] *= f;
            A[t + 1 + t * lda] = e[t];
        }
    }
}

inline unsigned blocks_for(int64_t rows, int per) { return (unsigned)((rows + per - 1) / per); }

}  // namespace

cudaError_t launch_dense_maxabs(const double* A, int64_t lda, int64_t n, double* out, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), s);
    if (e != cudaSuccess) return e;
    if (n <= 0) return cudaSuccess;
    maxabs_kernel<<<608, 256, 0, s>>>(A, lda, n, out);
    return cudaGetLastError();
}

cudaError_t launch_dense_scale(double* A, int64_t lda, int64_t n, double f, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    scale_kernel<<<1216, 256, 0, s>>>(A, lda, n, f);
    return cudaGetLastError();
}

cudaError_t launch_tridiag_unscale(double* A, int64_t lda, int64_t n, double* d, double* e, double f,
                                   cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    tridiag_unscale_kernel<<<(unsigned)((n + 255) / 256 < 1216 ? (n + 255) / 256 : 1216), 256, 0, s>>>(A, lda, n, d, e, f);
    return cudaGetLastError();
}

// Scratch (doubles) of sytrd_dev / orgtr_dev for order n.
int64_t dense_scratch_doubles(int64_t n)
{
    const int64_t rb = (n + RT - 1) / RT + 1, gc = (n + GCH - 1) / GCH + 1;
    const int64_t sytrd = 2 * n * 2 * NB + rb + rb * 2 * NB + gc * n + rb + 8;
    const int64_t kch = (n + KCH - 1) / KCH + 1;
    const int64_t tiles = (n + dmma::BN - 1) / dmma::BN + 1;
    const int64_t orgtr = n * NB + n * NB + NB * n + kch * tiles * dmma::BM * dmma::BN + 2 * NB * NB + 8;
    return sytrd > orgtr ? sytrd : orgtr;
}

// A (n x n, lda) -> d (n), e (n-1), tau (n-1); A overwritten as by LAPACK dsytrd('L').
int sytrd_dev(cudaStream_t s, int64_t n, double* A, int64_t lda, double* d, double* e, double* tau,
              double* scratch)
{
    if (n <= 0) return SYMEIG_OK;
    double* VW = scratch;
    double* WV = VW + n * 2 * NB;
    const int64_t rb = (n + RT - 1) / RT + 1;
    double* part = WV + n * 2 * NB;
    double* dpart = part + rb;
    double* ypart = dpart + rb * 2 * NB;
    const int64_t gc = (n + GCH - 1) / GCH + 1;
    double* wpart = ypart + gc * n;
    double* sc = wpart + rb;
    for (int64_t p = 0; p < n - 1; p += NB) {
        const int pb = (int)(n - 1 - p < NB ? n - 1 - p : NB);
        for (int i = 0; i < pb; ++i) {
            const int64_t j = p + i;
            const unsigned rows_j = blocks_for(n - j, RT);        // rows j .. n-1
            const unsigned rows_j1 = blocks_for(n - j - 1, RT);   // rows j+1 .. n-1
            const unsigned chunks = blocks_for(n - j - 1, GCH);
            col_update_kernel<<<rows_j, RT, 0, s>>>(A, lda, n, j, i, pb, VW, part);
            reflector_kernel<<<1, RT, 0, s>>>(A, lda, j, part, (int)rows_j, d, e, tau, sc);
            make_v_kernel<<<rows_j1, RT, 0, s>>>(A, lda, n, j, i, pb, VW, WV, sc, dpart);
            symv_kernel<<<dim3(rows_j1, chunks), RT, 0, s>>>(A, lda, n, j, VW + (int64_t)i * n, ypart);
            w_kernel<<<rows_j1, RT, 0, s>>>(n, j, i, pb, VW, WV, ypart, (int)chunks, dpart, (int)rows_j1, sc, wpart);
            w_fix_kernel<<<rows_j1, RT, 0, s>>>(n, j, i, pb, VW, WV, sc, wpart, (int)rows_j1);
        }
        const int64_t q = p + pb;
        if (q < n) {
            const unsigned t = blocks_for(n - q, dmma::BM);
            trailing_update_kernel<<<dim3(t, t), dmma::kThreads, 0, s>>>(A, lda, n, q, pb, VW, WV);
        }
    }
    last_diag_kernel<<<1, 32, 0, s>>>(A, lda, n, d);
    return cudaGetLastError() == cudaSuccess ? SYMEIG_OK : SYMEIG_ERR_CUDA;
}

// Q (n x n, ldq) = H_0 ... H_{n-2} from sytrd_dev's A and tau.
int orgtr_dev(cudaStream_t s, int64_t n, const double* A, int64_t lda, const double* tau, double* Q,
              int64_t ldq, double* scratch)
{
    if (n <= 0) return SYMEIG_OK;
    identity_kernel<<<1216, 256, 0, s>>>(Q, ldq, n);
    if (n == 1) return cudaGetLastError() == cudaSuccess ? SYMEIG_OK : SYMEIG_ERR_CUDA;
    double* Vp = scratch;
    double* VT = Vp + n * NB;
    double* Y = VT + n * NB;
    double* part = Y + NB * n;
    const int64_t kch = (n + KCH - 1) / KCH + 1;
    const int64_t tiles = (n + dmma::BN - 1) / dmma::BN + 1;
    double* G = part + kch * tiles * dmma::BM * dmma::BN;
    double* T = G + NB * NB;
    const int64_t last = ((n - 2) / NB) * NB;   // start of the last panel
    for (int64_t p = last; p >= 0; p -= NB) {
        const int pb = (int)(n - 1 - p < NB ? n - 1 - p : NB);
        const int64_t m = n - p - 1;
        extract_v_kernel<<<blocks_for(m * pb, 256) < 1216 ? blocks_for(m * pb, 256) : 1216, 256, 0, s>>>(A, lda, n, p, pb, Vp);
        const unsigned nk = blocks_for(m, KCH);
        // G = Vp^T Vp (pb x pb): A(i, k) = Vp(k, i), B(k, j) = Vp(k, j)
        splitk_tile_kernel<<<dim3(1, 1, nk), dmma::kThreads, 0, s>>>(Vp, m, 1, Vp, 1, m, pb, pb, m, part);
        reduce_tiles_kernel<<<16, 256, 0, s>>>(part, pb, pb, (int)nk, G, NB);
        tfactor_kernel<<<1, NB, 0, s>>>(G, NB, tau + p, pb, T);
        vt_kernel<<<blocks_for(m, 128), 128, 0, s>>>(Vp, m, pb, T, VT);
        // Y = Vp^T Q(R, R) (pb x m): B(k, j) = Q(p+1+k, p+1+j)
        const double* QR = Q + (p + 1) + (p + 1) * ldq;
        const unsigned tn = blocks_for(m, dmma::BN);
        splitk_tile_kernel<<<dim3(tn, 1, nk), dmma::kThreads, 0, s>>>(Vp, m, 1, QR, 1, ldq, pb, m, m, part);
        reduce_tiles_kernel<<<blocks_for(pb * m, 256) < 4096 ? blocks_for(pb * m, 256) : 4096, 256, 0, s>>>(part, pb, m, (int)nk, Y, pb);
        const unsigned tm = blocks_for(m, dmma::BM);
        wy_update_kernel<<<dim3(tm, tm), dmma::kThreads, 0, s>>>(Q, ldq, p + 1, m, pb, VT, Y);
    }
    return cudaGetLastError() == cudaSuccess ? SYMEIG_OK : SYMEIG_ERR_CUDA;
}

}  // namespace symeig
