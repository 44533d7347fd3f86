// wave_common.cuh -- the wave-window Givens tile shared by the single-matrix and the batched
// apply kernels.
//
// A tile is the work of one CTA of WARPS warps (4 unless a shape says otherwise): WARPS * R *
// (32/G) consecutive rows of Q (R rows per thread), all columns of the pass, all G*KB layers
// of the pass.
//
// Order of the rotations.  Rotation (i, L) acts on columns (i, i+1).  The reference's wave
// order (src/wave.jl:62-162) applies (i, L) after (i-1, L) and after (i+1, L-1); per element
// of Q that is the same sequence of rotations as the layer-major loop "for L, for i".  A
// lane group walks waves t = 0, 1, 2, ... of its KB layers: wave t applies rotation
// (t-1-l, l) for l = 0..KB-1, i.e. the column pairs (t-1-l, t-l) from right to left, which
// respects both dependencies.  After wave t, column t-KB is final for the group.
//
// Layer groups.  The G groups of a row run in the G lane groups of one warp (R * 32/G rows
// per warp).  Group g lags group g-1 by KB+1 waves and receives its input columns from group g-1
// through a warp shuffle, so a pass reads and writes each element of Q once.  All groups of a
// warp hold the same rows, so the column read issued by every lane costs one sector per
// warp; group 0 keeps it, group G-1 stores the finished column.
//
// (c,s) staging.  The table lays the rotations out per iteration: the G*KB pairs a warp needs
// in iteration t are contiguous, each group's KB pairs padded by 16 bytes so that the
// groups' pairs land in disjoint shared-memory banks.  Rotations outside the grid or above
// a column's layer count are (1, 0), so the inner loop has no bounds logic.  The table is
// cut into chunks of CH iterations that the CTA streams into a two-slot shared-memory ring
// with cp.async.bulk (the TMA engine's bulk copy; no tensor map, no multicast), completion
// tracked by one mbarrier per slot.  Every wait is bounded: after ~2 s of SM clock the tile
// gives up and reports failure, and the kernel returns without touching Q again.
//
// Scaled form (SCALED = true, FP64).  The table holds per slot (A, B) instead of (c, s), the
// group's form flags in its pad word, and in group G-1's pad the scale factor of the column
// that group stores in that iteration (see wave_rotations_scaled and apply.cu).
//
// Register window.  CH is a multiple of KB+1 and the chunk loop is fully unrolled, so column
// t always lives in window slot t mod (KB+1), a compile-time constant: the window rotates
// without register moves.  Group 0 keeps a second ring of KB+1 registers with the next
// columns of Q, read KB+1 waves ahead.
#pragma once

#include "int_mul.cuh"
#include "symeig_common.cuh"

namespace symeig {
namespace wave {

constexpr int kThreads = 128;  // 4 warps per CTA

template <typename T, int KB_, int G_, int R_ = 1, int WARPS_ = kThreads / 32>
struct Shape {
    using P2 = typename Pair<T>::type;
    static constexpr int KB = KB_, G = G_, W = KB_ + 1;
    static constexpr int R = R_;                                // rows per thread
    static constexpr int RPW = 32 / G;                          // lanes per group
    static constexpr int THREADS = 32 * WARPS_;                 // threads per CTA
    static constexpr int ROWS = R * RPW * WARPS_;               // rows per tile
    static constexpr int CH = W;                                // iterations per chunk
    static constexpr int GSTRIDE = KB * (int)sizeof(P2) + 16;   // bytes per group, padded
    static constexpr int ITER = G * GSTRIDE;                    // bytes per iteration
    static constexpr int CHUNK = CH * ITER;                     // bytes per chunk
    static constexpr int LAYERS = KB * G;                       // layers per pass
    static_assert(32 % G == 0, "groups must divide a warp");
    static_assert(KB % 2 == 0, "pairs of slots are read together");
    static_assert(CHUNK % 16 == 0 && GSTRIDE % 16 == 0, "bulk-copy alignment");
    __host__ __device__ static int64_t iterations(int64_t n_loc) { return n_loc + KB + (int64_t)(G - 1) * W; }
    __host__ __device__ static int64_t chunks(int64_t n_loc) { return (iterations(n_loc) + CH - 1) / CH; }
    __host__ __device__ static int64_t table_bytes(int64_t n_loc) { return chunks(n_loc) * (int64_t)CHUNK; }
};

// ---- mbarrier / bulk-copy helpers (PTX) -----------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return ok != 0;
}

// Wait for phase `parity` of `bar`, giving up after ~2 s of SM clock.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity)
{
    if (mbar_test(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_test(bar, parity)) {
        if (clock64() - t0 > 4000000000LL) return false;
    }
    return true;
}

// Store with a predicate, forced to a predicated instruction (no branch).
__device__ __forceinline__ void st_pred(double* p, double v, bool pred)
{
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q st.global.f64 [%0], %1;\n\t}"
                 ::"l"(p), "d"(v), "r"((unsigned)pred));
}
__device__ __forceinline__ void st_pred(float* p, float v, bool pred)
{
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q st.global.f32 [%0], %1;\n\t}"
                 ::"l"(p), "f"(v), "r"((unsigned)pred));
}

// One table entry: iteration t, group g, slot l of a pass over columns [c0, c0+n_loc) and
// layers [L0, L0+layers) of a Julia-layout grid with grid_rows rows.  place (may be null):
// layer L of rotation i is (1,0) unless L < place[i].
template <typename T, typename Sh, typename Tsrc>
__device__ __forceinline__ void table_entry(unsigned char* table, int64_t t, int g, int l,
                                            const Tsrc* grid, int64_t grid_rows,
                                            const int32_t* place, int64_t c0, int64_t n_loc,
                                            int64_t L0, int64_t layers)
{
    using P2 = typename Sh::P2;
    const int64_t tg = t - (int64_t)g * Sh::W;
    const int64_t i_loc = tg - 1 - l;
    const int64_t lay = (int64_t)g * Sh::KB + l;
    Tsrc c = Tsrc(1), s = Tsrc(0);
    if (i_loc >= 0 && i_loc <= n_loc - 2 && lay < layers) {
        const int64_t i = c0 + i_loc;
        const int64_t L = L0 + lay;
        if (place == nullptr || L < (int64_t)place[i]) {
            const Tsrc* p = grid + 2 * (i + L * grid_rows);
            c = p[0];
            s = p[1];
        }
    }
    P2 v;
    v.x = (T)c;
    v.y = (T)s;
    *(P2*)(table + t * Sh::ITER + g * Sh::GSTRIDE + l * (int)sizeof(P2)) = v;
}

// The KB rotations of one wave on the windows of the thread's R rows, (c,s) read from shared
// memory once for all R rows.  U is the wave's slot (t mod (KB+1)); callers pass a constant of
// a fully unrolled loop, so every window index folds to a constant and the windows stay in
// registers.  FP64 with INT_MUL: the products s*y and s*x of each rotation come from the
// integer pipes (int_mul.cuh), bit-identical to the FP64 products, and only the two FMAs use
// the FP64 pipe; a lane whose product the integer path does not cover (a zero, subnormal,
// infinite or NaN operand, an underflow) recomputes both products on the FP64 pipe, behind a
// warp vote so that the FP64 instructions issue only when some lane needs them.
template <typename T, int KB, int R, bool INT_MUL = false>
__device__ __forceinline__ void wave_rotations(T (&win)[R][KB + 1], const unsigned char* cs, const int U,
                                               const T nz)
{
    constexpr int W = KB + 1;
    if constexpr (sizeof(T) == 8 && INT_MUL) {
#pragma unroll
        for (int l = 0; l < KB; ++l) {
            const double2 p = *reinterpret_cast<const double2*>(cs + l * 16);
            const SplitFactor f = split_factor(p.y);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                double& x = win[r][(U - 1 - l + 2 * W) % W];
                double& y = win[r][(U - l + 2 * W) % W];
                bool sp = f.special;
                double sy = mul_rn_int(f, y, sp);
                double sx = mul_rn_int(f, x, sp);
                if (__any_sync(0xffffffffu, sp)) {
                    if (sp) {
                        const double2 q = fma_pair_call(p.y, y, x, nz);
                        sy = q.x;
                        sx = q.y;
                    }
                }
                x = __fma_rn(p.x, x, sy);
                y = __fma_rn(p.x, y, -sx);
            }
        }
    } else if constexpr (sizeof(T) == 8) {
#pragma unroll
        for (int l = 0; l < KB; ++l) {
            const double2 p = *reinterpret_cast<const double2*>(cs + l * 16);
#pragma unroll
            for (int r = 0; r < R; ++r)
                rot_fma(win[r][(U - 1 - l + 2 * W) % W], win[r][(U - l + 2 * W) % W], p.x, p.y, nz);
        }
    } else {
#pragma unroll
        for (int l = 0; l < KB; l += 2) {
            const float4 p = *reinterpret_cast<const float4*>(cs + l * 8);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                rot(win[r][(U - 1 - l + 2 * W) % W], win[r][(U - l + 2 * W) % W], p.x, p.y);
                rot(win[r][(U - 2 - l + 2 * W) % W], win[r][(U - 1 - l + 2 * W) % W], p.z, p.w);
            }
        }
    }
}

// The scaled form of the KB rotations of one wave (FP64): each slot holds (A, B) and the
// group's flag word (in the 16-byte pad after its KB pairs) selects, per slot l, form 2 (bit
// l set) or form 1.  With (u, v) = form 2 ? (y, x) : (x, y):  x = fma(A, v, u), y = fma(B, u, v)
// -- two FP64 instructions per rotation-row instead of four.  The scale factors the form
// folds out of the columns are applied once per pass when group G-1 stores a column.
template <int KB, int R>
__device__ __forceinline__ void wave_rotations_scaled(double (&win)[R][KB + 1], const unsigned char* cs,
                                                      const int U)
{
    constexpr int W = KB + 1;
    const uint32_t flags = *reinterpret_cast<const uint32_t*>(cs + KB * 16);
#pragma unroll
    for (int l = 0; l < KB; ++l) {
        const double2 p = *reinterpret_cast<const double2*>(cs + l * 16);
        const bool f2 = (flags >> l) & 1u;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            double& x = win[r][(U - 1 - l + 2 * W) % W];
            double& y = win[r][(U - l + 2 * W) % W];
            const double u = f2 ? y : x, v = f2 ? x : y;
            x = __fma_rn(p.x, v, u);
            y = __fma_rn(p.y, u, v);
        }
    }
}

// CTA-shared staging state of the tile loop: the two-slot ring and one mbarrier per slot,
// with the number of completed waits per slot (their parity is the phase to wait for next).
template <typename Sh>
struct Staging {
    unsigned char (*ring)[Sh::CHUNK];
    uint64_t* bar;
    uint32_t uses0, uses1;
    int* check = nullptr;   // checked builds: the kernel's error word (index_ok)
};

// Checked builds (-DSYMEIG_DEVICE_CHECKS, build.build_checked): every global access of a wave
// tile to Q is first checked against the pass's extent (rows [0, m), columns [0, n_loc)); an
// access outside it is skipped and sets bit 1 (value 2) of the kernel's error word, which the
// host reports as SYMEIG_ERR_DEVICE.  The default build compiles the checks away.
#ifdef SYMEIG_DEVICE_CHECKS
__device__ __forceinline__ bool index_ok(int* check, bool ok)
{
    if (!ok && check != nullptr) atomicOr(check, 2);
    return ok;
}
#define WAVE_IDX_OK(st, cond) ::symeig::wave::index_ok((st).check, (cond))
#else
#define WAVE_IDX_OK(st, cond) true
#endif

template <typename Sh>
__device__ __forceinline__ void staging_init(Staging<Sh>& st)
{
    if (threadIdx.x == 0) {
        mbar_init(&st.bar[0], 1);
        mbar_init(&st.bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    st.uses0 = st.uses1 = 0;
    __syncthreads();
}

// Values a thread carries across a segment boundary (see wave_tile): its windows, its ring of
// columns read ahead, and the column it last handed to the next lane group.
template <typename Sh> __host__ __device__ constexpr int segment_state_values() { return Sh::R * (2 * Sh::W + 1); }

// One tile: rows [row0, row0 + ROWS) of Q (m rows, columns [0, n_loc) of the pass) through
// chunks [c_begin, c_end) of the n_chunks chunks of `table` (c_end < 0: to the last).
// A pass may run as several launches over consecutive chunk ranges ("segments"): a segment
// that does not start at chunk 0 restores each thread's registers from `state` (which the
// previous segment saved there), and one that does not end at the last chunk saves them.
// Chunk c reads the columns below (c + 1) * CH + W and finishes the columns below
// (c + 1) * CH - (G - 1) * W - KB, so a segment needs only the columns its chunks read, and
// the columns it finishes are final.  `state` (segments only) points at this CTA's
// segment_state_values * THREADS values, laid out value-major so that saving and restoring
// are coalesced.  `stall` (a test hook, default never): chunks from that index on are not
// copied, so their bounded waits run out and the tile returns false.
// Element (row, col) is Q[row * rs + col * ldq]: rs = 1 for
// the column rotations of rmul! on a column-major matrix, rs = lda and ldq = 1 for the row
// rotations of lmul! (the same wave on the transposed view).  Every thread of the CTA calls
// it.  Returns false (all threads) when a bounded wait gave up.  SEG = false compiles the
// whole-pass tile (c_begin, c_end and state ignored): the segment logic in registers costs the
// whole-pass kernel about 6 % (measured at 16384^2, 71.0 against 67.1 ms).
template <typename T, typename Sh, bool SCALED = false, bool INT_MUL = false, bool SEG = false>
__device__ __forceinline__ bool wave_tile(T* __restrict__ Q, int64_t ldq, int64_t m, int64_t row0,
                                          int32_t n_loc, const unsigned char* __restrict__ table,
                                          int32_t n_chunks, const T nz, Staging<Sh>& st,
                                          int64_t rs = 1, int32_t stall = 0x7fffffff,
                                          int32_t c_begin_arg = 0, int32_t c_end_arg = -1,
                                          T* __restrict__ state = nullptr)
{
    constexpr int KB = Sh::KB, G = Sh::G, CH = Sh::CH, W = Sh::W, RPW = Sh::RPW, R = Sh::R;
    const int tid = threadIdx.x;
    const int32_t c_begin = SEG ? c_begin_arg : 0;
    const int32_t c_end = SEG ? ((c_end_arg < 0 || c_end_arg > n_chunks) ? n_chunks : c_end_arg) : n_chunks;
    if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (c_begin < c_end && c_begin < stall)
            bulk_load(st.ring[0], table + (int64_t)c_begin * Sh::CHUNK, Sh::CHUNK, &st.bar[0]);
        if (c_begin + 1 < c_end && c_begin + 1 < stall)
            bulk_load(st.ring[1], table + (int64_t)(c_begin + 1) * Sh::CHUNK, Sh::CHUNK, &st.bar[1]);
    }

    // lane rl of group g holds rows rbase + r*RPW, r < R, of the warp's R*RPW rows
    const int lane = tid & 31;
    const int g = lane / RPW;
    const int rl = lane - g * RPW;
    const int64_t rbase = row0 + (int64_t)(tid >> 5) * (R * RPW) + rl;
    T* __restrict__ qrow[R];
    bool storer[R];  // group G-1 writes Q
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int64_t row = rbase + (int64_t)r * RPW;
        const bool row_ok = row < m;
        qrow[r] = Q + (row_ok ? row : 0) * rs;
        storer[r] = (g == G - 1) && row_ok;
    }
    const int lag = g * W;  // waves this group trails group 0

    T win[R][W], ahead[R][W];
    T xout[R];
    constexpr int NT = Sh::THREADS;
    if (!SEG || c_begin == 0) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
#pragma unroll
            for (int q = 0; q < W; ++q) {
                win[r][q] = T(0);
                ahead[r][q] = (q < n_loc) ? qrow[r][(int64_t)q * ldq] : T(0);
            }
            xout[r] = T(0);
        }
    } else {
#pragma unroll
        for (int r = 0; r < R; ++r) {
#pragma unroll
            for (int q = 0; q < W; ++q) {
                win[r][q] = state[(r * (2 * W + 1) + q) * NT + tid];
                ahead[r][q] = state[(r * (2 * W + 1) + W + q) * NT + tid];
            }
            xout[r] = state[(r * (2 * W + 1) + 2 * W) * NT + tid];
        }
    }

    for (int32_t c = c_begin; c < c_end; ++c) {
        const int b = (c - c_begin) & 1;
        const uint32_t parity = ((b ? st.uses1 : st.uses0) + (uint32_t)((c - c_begin) >> 1)) & 1u;
        const bool ok = mbar_wait_bounded(&st.bar[b], parity);
        if (__syncthreads_or(!ok)) return false;
        const unsigned char* sb = st.ring[b] + g * Sh::GSTRIDE;
        const int32_t t0 = c * CH;
        // column t0 + u + W is read in iteration u; group G-1 writes column t0 + u - lag - KB
        const int32_t st0 = t0 - lag - KB;
        const bool interior = (t0 + W + CH <= n_loc) && (t0 - (G - 1) * W - KB >= 0) &&
                              (t0 - KB + CH <= n_loc);
        if (interior) {
            const T* lp[R];
            T* sp[R];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                lp[r] = qrow[r] + (int64_t)(t0 + W) * ldq;
                sp[r] = qrow[r] + (int64_t)st0 * ldq;
            }
#pragma unroll
            for (int u = 0; u < CH; ++u) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const T up = __shfl_up_sync(0xffffffffu, xout[r], RPW);
                    const T xin = (g == 0) ? ahead[r][u % W] : up;
                    ahead[r][u % W] = WAVE_IDX_OK(st, t0 + W + u < n_loc) ? *lp[r] : T(0);
                    lp[r] += ldq;
                    win[r][u % W] = xin;
                }
                if constexpr (SCALED) wave_rotations_scaled<KB, R>(win, sb + u * Sh::ITER, u % W);
                else wave_rotations<T, KB, R, INT_MUL>(win, sb + u * Sh::ITER, u % W, nz);
                T dsc = T(1);
                if constexpr (SCALED) dsc = *reinterpret_cast<const T*>(sb + u * Sh::ITER + KB * 16 + 8);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    xout[r] = win[r][(u + 1) % W];
                    const bool in = storer[r] && WAVE_IDX_OK(st, st0 + u >= 0 && st0 + u < n_loc);
                    if constexpr (SCALED) {
                        if (in) *sp[r] = xout[r] * dsc;
                    } else {
                        if (in) *sp[r] = xout[r];
                    }
                    sp[r] += ldq;
                }
            }
        } else {
            const int32_t ld_cnt = min(max(n_loc - t0 - W, 0), CH);
            const int32_t st_lo = max(-st0, 0);
            const int32_t st_hi = min(n_loc - st0, CH);
#pragma unroll
            for (int u = 0; u < CH; ++u) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const T up = __shfl_up_sync(0xffffffffu, xout[r], RPW);
                    const T xin = (g == 0) ? ahead[r][u % W] : up;
                    T nxt = T(0);
                    if (u < ld_cnt && WAVE_IDX_OK(st, t0 + W + u < n_loc)) nxt = qrow[r][(int64_t)(t0 + W + u) * ldq];
                    ahead[r][u % W] = nxt;
                    win[r][u % W] = xin;
                }
                if constexpr (SCALED) wave_rotations_scaled<KB, R>(win, sb + u * Sh::ITER, u % W);
                else wave_rotations<T, KB, R, INT_MUL>(win, sb + u * Sh::ITER, u % W, nz);
                T dsc = T(1);
                if constexpr (SCALED) dsc = *reinterpret_cast<const T*>(sb + u * Sh::ITER + KB * 16 + 8);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    xout[r] = win[r][(u + 1) % W];
                    T xs = xout[r];
                    if constexpr (SCALED) xs = xout[r] * dsc;
                    const bool in = storer[r] && u >= st_lo && u < st_hi;
                    st_pred(qrow[r] + (int64_t)(st0 + u) * ldq, xs,
                            in && WAVE_IDX_OK(st, st0 + u >= 0 && st0 + u < n_loc));
                }
            }
        }
        __syncthreads();
        if (tid == 0 && c + 2 < c_end && c + 2 < stall) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            bulk_load(st.ring[b], table + (int64_t)(c + 2) * Sh::CHUNK, Sh::CHUNK, &st.bar[b]);
        }
    }
    const int32_t used = c_end > c_begin ? c_end - c_begin : 0;
    st.uses0 += (uint32_t)((used + 1) >> 1);
    st.uses1 += (uint32_t)(used >> 1);
    if (SEG && state != nullptr && c_end < n_chunks) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
#pragma unroll
            for (int q = 0; q < W; ++q) {
                state[(r * (2 * W + 1) + q) * NT + tid] = win[r][q];
                state[(r * (2 * W + 1) + W + q) * NT + tid] = ahead[r][q];
            }
            state[(r * (2 * W + 1) + 2 * W) * NT + tid] = xout[r];
        }
    }
    return true;
}

}  // namespace wave
}  // namespace symeig
