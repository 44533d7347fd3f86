// chase.cu -- the FP64 bulge-chase kernel: one flush of qr_algorithm! on the device.
//
// Restates, on one warp, the inner loop of qr_algorithm! (src/bulge_chasing.jl:166-279):
// the deflation scan (:205-222, is_offdiagonal_small :7-8), the layer capacity rule
// (:226-230), the Wilkinson shift (:239-265) and single_shift! (:11-144) with
// get_rotation / LinearAlgebra.givensAlgorithm (src/simple_givens.jl:20-23).  The sweep is a
// strict dependency chain and runs on lane 0; the O(n) scans (deflation, thickest column)
// use all 32 lanes with ballots.  Rotations go to a Julia-layout (c,s) grid: at
// grid[i, ++thickness[i]] as the reference records them, or (the default) at the sweep's
// exact-order layer described at chase_kernel.
//
// Every floating-point operation is an explicit _rn intrinsic.  Inside single_shift! the
// reference runs under @fastmath; this kernel and the CPU oracle fuse the first product of
// each `u*a + v*b` (see symeig_common.cuh).  Outside it (givensAlgorithm, the shift, the
// deflation test) the arithmetic is plain IEEE without contraction, as Julia compiles it.
// Division and square root are the correctly rounded __ddiv_rn / __dsqrt_rn, so the kernel
// reproduces the oracle's rotation stream bit for bit.
//
// The kernel never traps and never waits on another kernel: a flush ends by itself and
// reports CHASE_FLUSH, CHASE_CONVERGED or CHASE_MAXITER in ChaseState.
#include "symeig_common.cuh"
#include "givens.cuh"

namespace symeig {

namespace {

using namespace gv;

// is_offdiagonal_small(H, j, tol), 1-based j (src/bulge_chasing.jl:7-8).
__device__ __forceinline__ bool is_small(const double* dv, const double* ev, int64_t j, double tol)
{
    return fabs(ev[j - 1]) <= __dmul_rn(tol, __dadd_rn(fabs(dv[j - 1]), fabs(dv[j])));
}

// Wilkinson shift from the trailing 2x2 block [a c; c b] (src/bulge_chasing.jl:239-265).
__device__ __forceinline__ double wilkinson_shift(double a, double b, double c)
{
    const double scale = __dadd_rn(__dadd_rn(fabs(a), __dmul_rn(2.0, fabs(c))), fabs(b));
    const double H11 = __ddiv_rn(a, scale), H12 = __ddiv_rn(c, scale), H22 = __ddiv_rn(b, scale);
    const double t = __ddiv_rn(__dadd_rn(H11, H22), 2.0);
    const double p = __dmul_rn(__dsub_rn(H11, t), __dsub_rn(H22, t));
    const double q = __dmul_rn(H12, H12);
    const double d = __dsub_rn(p, q);
    const double sq = __dsqrt_rn(fabs(d));
    const double l1 = __dadd_rn(t, sq), l2 = __dsub_rn(t, sq);
    const double lam = fabs(__dsub_rn(H22, l1)) < fabs(__dsub_rn(H22, l2)) ? l1 : l2;
    return __dmul_rn(lam, scale);
}

__device__ __forceinline__ double fsum(double u, double a, double v, double b, double nz)
{
    // u*a + v*b with the first product fused
    return __fma_rn(u, a, mulz(v, b, nz));
}

// u*a - v*b with the first product fused
__device__ __forceinline__ double fdif(double u, double a, double v, double b, double nz)
{
    return __fma_rn(u, a, neg(mulz(v, b, nz)));
}

// Record (c,s) of rotation i (1-based).  thick[i] is the reference's layer_thickness (it
// drives the capacity rule); place[i] is the grid layer used, equal to thick[i] in reference
// mode (layer <= 0) or the sweep's common layer in exact-order mode.
__device__ __forceinline__ void record(double* grid, int32_t* thick, int32_t* place, int64_t rows,
                                       int64_t i, int32_t layer, double c, double s)
{
    const int32_t t = thick[i - 1] + 1;
    thick[i - 1] = t;
    if (layer <= 0) layer = t;
    place[i - 1] = layer;
    double* p = grid + 2 * ((i - 1) + (int64_t)(layer - 1) * rows);
    p[0] = c;
    p[1] = s;
}

// single_shift!(H, from, to, mu, givens, layer_thickness) (src/bulge_chasing.jl:11-144).
// dv/ev are 0-based arrays; from/to 1-based.  Values the sweep itself produced travel in
// registers; only untouched entries are loaded.
// NR = true computes each rotation by givens_nr (proved Newton form, else the reference form).
template <bool NR>
__device__ void single_shift(double* __restrict__ dv, double* __restrict__ ev, int64_t from,
                             int64_t to, double mu, double* __restrict__ grid,
                             int32_t* __restrict__ thick, int32_t* __restrict__ place,
                             int64_t rows, int32_t layer, double nz)
{
    const double H11 = dv[from - 1], H21 = ev[from - 1], H22 = dv[from];
    double c, s, nrm;
    if (NR) givens_nr(__dsub_rn(H11, mu), H21, mulz(H21, H21, nz), c, s, nrm, nz);
    else givens_fast(__dsub_rn(H11, mu), H21, c, s, nrm, nz);
    const double H11p = fsum(c, H11, s, H21, nz);
    const double H21p = fdif(c, H21, s, H11, nz);
    const double H12p = fsum(c, H21, s, H22, nz);
    const double H22p = fdif(c, H22, s, H21, nz);
    const double H11pp = fsum(H11p, c, H12p, s, nz);
    const double H12pp = fdif(H12p, c, H11p, s, nz);
    const double H22pp = fdif(H22p, c, H21p, s, nz);
    dv[from - 1] = H11pp;
    dv[from] = H22pp;
    ev[from - 1] = H12pp;
    double bulge = 0.0;
    double e_next = 0.0;  // ev[i] (1-based) entering step i
    if (from + 2 <= to) {
        const double H23 = ev[from];
        bulge = mulz(s, H23, nz);
        e_next = mulz(c, H23, nz);
        ev[from] = e_next;
    }
    record(grid, thick, place, rows, from, layer, c, s);

    double p1 = H12pp;      // ev[i-1] (1-based) entering step i
    double B11 = H22pp;     // dv[i]   (1-based) entering step i
    // untouched entries for the first loop step
    double B22_n = (from + 1 <= to - 1) ? dv[from + 1] : 0.0;
    double B23_n = (from + 3 <= to) ? ev[from + 1] : 0.0;
    for (int64_t i = from + 1; i <= to - 1; ++i) {
        const double B22 = B22_n, B23 = B23_n;
        // prefetch for step i+1: dv[i+2], ev[i+2] (1-based)
        if (i + 1 <= to - 1) B22_n = dv[i + 1];
        if (i + 3 <= to) B23_n = ev[i + 1];
        if (NR) givens_nr(p1, bulge, mulz(bulge, bulge, nz), c, s, nrm, nz);
        else givens_fast(p1, bulge, c, s, nrm, nz);
        ev[i - 2] = nrm;
        const double B21 = e_next;
        const double B11p = fsum(c, B11, s, B21, nz);
        const double B21p = fdif(c, B21, s, B11, nz);
        const double B12p = fsum(c, B21, s, B22, nz);
        const double B22p = fdif(c, B22, s, B21, nz);
        const double B11pp = fsum(B11p, c, B12p, s, nz);
        const double B12pp = fdif(B12p, c, B11p, s, nz);
        const double B22pp = fdif(B22p, c, B21p, s, nz);
        dv[i - 1] = B11pp;
        dv[i] = B22pp;
        ev[i - 1] = B12pp;
        if (i + 2 <= to) {
            bulge = mulz(s, B23, nz);
            e_next = mulz(c, B23, nz);
            ev[i] = e_next;
        }
        record(grid, thick, place, rows, i, layer, c, s);
        p1 = B12pp;
        B11 = B22pp;
    }
}

// ---- the sweep on two warps, Newton-form rotations -------------------------------------
//
// single_shift! is one dependency chain per step: (f, g) -> r = sqrt(f^2 + g^2) -> c = f/r,
// s = g/r -> the 2x2 update -> next (f, g).  On GB300 one warp issues an FP64 instruction
// about every 64-90 cycles whatever their dependences, and the SM runs a few such warps at
// once, so the step time is set by the FP64 instructions on the warp that carries the chain.
// Here (the fastest split measured)
//   warp 0 (the chain): the rotation by givens_nr_core (14 FP64 instructions), the four
//           products of the 2x2 update that give the next f (B11', B12', B11'*s, B12'') and
//           the next bulge g = s*ev[i+1] with g*g;
//   warp 1: next B21 = c*ev[i+1] and the B21'/B22'/B22'' half of the update (-> next B11),
//           B11'', the rounding proof of warp 0's rotation, every store and the record.
// They trade values through a two-slot shared mailbox (slot = step parity) and two named
// barriers, each used producer -> consumer (bar.arrive / bar.sync) and each strictly
// alternating: warp 0 waits for B(i-1) before it arrives at CS(i), and warp 1 arrives at
// B(i) only after CS(i).
// Warp 0 does not wait for the proof.  Warp 1 records a failed proof (none was seen in 10^9
// random rotations; see givens.cuh) and the kernel then restores the sweep's entries from a
// copy taken before it and runs the sweep again in the reference form (single_shift), so the
// result is bit-identical either way.  Steps whose (f, g) are outside the Newton form's range
// take givens_fast on warp 0 and skip the proof.
enum : int { kBarCS = 1, kBarB = 2 };

struct NrMail {
    double c, s, r, x, f, g;  // warp 0 -> 1 (kBarCS); r with the sign convention applied
    int32_t slow;             // 1: (c, s, r) from givens_fast, nothing to prove
    double b22pp, e_next;     // warp 1 -> 0 (kBarB): next B11, next B21
};

__device__ __forceinline__ void nb_sync(int id)
{
    asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory");
}
__device__ __forceinline__ void nb_arrive(int id)
{
    asm volatile("bar.arrive %0, 64;" ::"r"(id) : "memory");
}

// single_shift!(H, from, to, mu, givens, layer_thickness) (src/bulge_chasing.jl:11-144) by
// both warps of the CTA.  Step i (1-based, from .. to-1) is the reference's first rotation
// for i = from and its loop body otherwise; both have the same 2x2 update.  Of the entries the
// reference writes and later overwrites within the sweep only the final ones are stored:
// dv[from-1 .. to-1] (0-based), ev[from-1 .. to-3] = the norms r of steps from+1 .. to-1 and
// ev[to-2] = the last B12''.  The grid slot of rotation i is column `layer` (exact order) or
// thick[i-1] + 1 (the reference's placement; thick is updated by the caller after the sweep).
// *fail is set when a Newton-form rotation could not be proved.
__device__ void sweep_nr_2w(double* __restrict__ dv, double* __restrict__ ev, int64_t from,
                            int64_t to, double mu, double* __restrict__ grid,
                            const int32_t* __restrict__ thick, int64_t rows, int32_t layer,
                            double nz, NrMail* mail, int32_t* fail)
{
    const int warp = threadIdx.x >> 5;
    const bool lead = (threadIdx.x & 31) == 0;
    const double H11 = dv[from - 1], H21 = ev[from - 1];
    if (warp == 0) {
        double f = __dsub_rn(H11, mu), g = H21, gg = mulz(H21, H21, nz);
        double B11 = H11, B21 = H21;
        double B22n = dv[from];                                  // dv[i+1] (1-based) for step i
        double B23n = (from + 2 <= to) ? ev[from] : 0.0;         // ev[i+1] (1-based) for step i
        for (int64_t i = from; i <= to - 1; ++i) {
            const double B22 = B22n, B23 = B23n;
            if (i + 1 <= to - 1) B22n = dv[i + 1];
            if (i + 3 <= to) B23n = ev[i + 1];
            // the Newton form whatever the range (no branch before the chain), then the
            // reference form when the inputs are out of its range
            const NrRot o = givens_nr_core(f, g, gg, nz);
            double c = o.c, s = o.s, r = o.r;
            int32_t slow = 0;
            if (!nr_in_range(f, g)) {
                givens_fast(f, g, c, s, r, nz);
                slow = 1;
            }
            if (i > from) {
                nb_sync(kBarB);
                const NrMail& pv = mail[(i - 1) & 1];
                B11 = pv.b22pp;
                B21 = pv.e_next;
            }
            NrMail& mb = mail[i & 1];
            mb.c = c; mb.s = s; mb.r = r; mb.x = o.x; mb.f = f; mb.g = g; mb.slow = slow;
            nb_arrive(kBarCS);
            const double B11p = __fma_rn(c, B11, mulz(s, B21, nz));
            const double B12p = __fma_rn(c, B21, mulz(s, B22, nz));
            f = __fma_rn(B12p, c, -mulz(B11p, s, nz));
            g = (i + 2 <= to) ? mulz(s, B23, nz) : 0.0;
            gg = mulz(g, g, nz);
        }
    } else {
        double B11 = H11, B21 = H21;
        double B22n = dv[from];
        double B23n = (from + 2 <= to) ? ev[from] : 0.0;
        int32_t thn = layer <= 0 ? thick[from - 1] : 0;
        bool bad = false;
        for (int64_t i = from; i <= to - 1; ++i) {
            const double B22 = B22n, B23 = B23n;
            const int32_t th = thn;
            if (i + 1 <= to - 1) B22n = dv[i + 1];
            if (i + 3 <= to) B23n = ev[i + 1];
            if (layer <= 0 && i + 1 <= to - 1) thn = thick[i];
            nb_sync(kBarCS);
            NrMail& mb = mail[i & 1];
            const double c = mb.c, s = mb.s, r = mb.r, x = mb.x, f = mb.f, g = mb.g;
            const int32_t slow = mb.slow;
            const double e_next = (i + 2 <= to) ? mulz(c, B23, nz) : 0.0;
            const double sB21 = mulz(s, B21, nz);
            const double B21p = __fma_rn(c, B21, -mulz(s, B11, nz));
            const double B22p = __fma_rn(c, B22, -sB21);
            const double B22pp = __fma_rn(B22p, c, -mulz(B21p, s, nz));
            if (i < to - 1) {
                mb.b22pp = B22pp;
                mb.e_next = e_next;
                nb_arrive(kBarB);
            }
            const double B11p = __fma_rn(c, B11, sB21);
            const double B12p = __fma_rn(c, B21, mulz(s, B22, nz));
            const double B11pp = __fma_rn(B11p, c, mulz(B12p, s, nz));
            if (!slow && !givens_nr_proved(f, g, x, c, s, r)) bad = true;
            if (lead) {
                dv[i - 1] = B11pp;
                if (i > from) ev[i - 2] = r;
                const int32_t L = layer > 0 ? layer : th + 1;
                *reinterpret_cast<double2*>(grid + 2 * ((i - 1) + (int64_t)(L - 1) * rows)) =
                    make_double2(c, s);
                if (i == to - 1) {
                    dv[i] = B22pp;
                    ev[i - 1] = __fma_rn(B12p, c, -mulz(B11p, s, nz));
                }
            }
            B11 = B22pp;
            B21 = e_next;
        }
        if (lead && bad) *fail = 1;
    }
}

constexpr int kScanUnroll = 8;  // chunks of 32 entries per round of the deflation scan

__device__ __forceinline__ int32_t warp_max(int32_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// ---- multishift batches (chase_mode 3) -----------------------------------------------------
//
// Shifts of a batch of nb <= kMaxBulges bulges over the block [from, to] (1-based): nb
// eigenvalues of the block's trailing w x w principal submatrix, w = min(kShiftWindow * nb,
// to - from + 1), ascending -- those ranked about the bottom diagonal entry (with r the number
// of the window's eigenvalues below dv[to], the ranks k0 .. k0 + nb - 1,
// k0 = min(max(r - nb / 2, 0), w - nb)).  A window twice the batch approximates the
// eigenvalues that belong to the bottom rows better than the square of the batch's own size
// (measured in the oracle's restatement: 0.95-1.02x the reference's sweeps for case A at
// n = 4096-8192, against 1.43-1.53x).
// The window is scaled by an exact power of two to max |entry| in [0.5, 1).  The rank r and
// a bracket of each eigenvalue come from bisection on FP32 Sturm counts; the shift itself is
// then refined in FP64 by a safeguarded Newton iteration on the characteristic polynomial
// p(x) = det(T_w - x I): one pass of the three-term recurrence gives p, p' and, from the
// signs of the leading minors p_i, the FP64 Sturm count at x, which moves an FP64 bracket
// [A, B] of the eigenvalue; a Newton step that is not finite or leaves [A, B] is replaced by
// the bracket's midpoint.  The recurrence is rescaled by exact powers of two whenever the
// exponent of p_i leaves [-600, 600]: over 128 rows of a window whose diagonal lies close to
// the shift, the unscaled p_i underflows (about 1e-362 in case A), which made every Newton
// step non-finite and left the shifts at FP32 accuracy.  Warp 0 of the controller sets up the
// window (batch_shifts_setup), then every thread of the CTA solves for its shifts
// (batch_shifts_solve); sd, se2, sea (FP32) and dd, ee2 (FP64) are
// kShiftWindow * kMaxBulges-entry shared arrays.
constexpr int kShiftWindow = 2;
constexpr int kWinMax = kShiftWindow * kMaxBulges;

// Number of the scaled window's eigenvalues below x, from the FP32 pivots of
// T - x I = L D L^T (a negative pivot per eigenvalue below x).
__device__ __forceinline__ int window_count32(const float* sd, const float* se2, int w, float x)
{
    constexpr float kPiv = 1e-30f;
    float q = sd[0] - x;
    int cnt = q < 0.0f;
    for (int i = 1; i < w; ++i) {
        if (fabsf(q) < kPiv) q = -kPiv;
        q = (sd[i] - x) - se2[i - 1] / q;
        cnt += q < 0.0f;
    }
    return cnt;
}

// p(x), p'(x) and the number of eigenvalues below x of the scaled window (dd, ee2), in FP64.
__device__ __forceinline__ void char_poly(const double* __restrict__ dd, const double* __restrict__ ee2, int w,
                                          double x, double& p, double& dp, int& below)
{
    double p0 = 1.0, p1 = dd[0] - x, q0 = 0.0, q1 = -1.0;
    int cnt = p1 < 0.0;
    for (int i = 1; i < w; ++i) {
        const double aa = dd[i] - x, bb = ee2[i - 1];
        const double t = -bb * p0, u = -bb * q0 - p1;
        const double p2 = __fma_rn(aa, p1, t);
        const double q2 = __fma_rn(aa, q1, u);
        // a sign change of the leading minors is an eigenvalue below x; an exact zero takes
        // the sign opposite to its predecessor's (the pivot convention of the FP32 counts)
        cnt += (p2 == 0.0) ? 1 : ((p2 < 0.0) != (p1 < 0.0));
        p0 = p1;
        p1 = (p2 == 0.0) ? -copysign(1e-300, p1) : p2;
        q0 = q1;
        q1 = q2;
        // keep p1 within 2^+-600 by exact power-of-two scaling of the whole recurrence state
        const int e = (int)((__double_as_longlong(p1) >> 52) & 0x7FF) - 1023;
        if ((e > 600 && e < 1024) || e < -600) {
            const double sc = __longlong_as_double((long long)(1023 - e) << 52);   // 2^-e, exact
            p0 *= sc;
            p1 *= sc;
            q0 *= sc;
            q1 *= sc;
        }
    }
    p = p1;
    dp = q1;
    below = cnt;
}

// What batch_shifts_setup leaves for batch_shifts_solve (shared memory).
struct ShiftWindow {
    int32_t w, k0, ex, trivial;
    float lo, hi;
};

// Warp 0: load and scale the window into the shared arrays, its Gershgorin interval, and the
// rank k0 of the first shift.
__device__ void batch_shifts_setup(const double* __restrict__ dv, const double* __restrict__ ev, int64_t from,
                                   int64_t to, int nb, ShiftWindow& sw, float* sd, float* se2, float* sea,
                                   double* dd, double* ee2)
{
    const int lane = threadIdx.x & 31;
    constexpr int H = kWinMax / 32;
    const int w = (int)min((int64_t)kShiftWindow * nb, to - from + 1);
    const int64_t r0 = to - w;  // 0-based first row of the window
    // lane holds entries q = lane + 32 h of the window
    double dq[H], eq[H];
    double mx = 0.0;
#pragma unroll
    for (int h = 0; h < H; ++h) {
        const int q = lane + 32 * h;
        dq[h] = q < w ? dv[r0 + q] : 0.0;
        eq[h] = q < w - 1 ? ev[r0 + q] : 0.0;
        mx = fmax(mx, fmax(fabs(dq[h]), fabs(eq[h])));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (!(mx > 0.0) || !isfinite(mx)) {
        // a zero block is already diagonal; a non-finite one is left to the sweep
        if (lane == 0) {
            sw.w = w;
            sw.trivial = 1;
        }
        __syncwarp();
        return;
    }
    int ex;
    frexp(mx, &ex);
#pragma unroll
    for (int h = 0; h < H; ++h) {
        const int q = lane + 32 * h;
        const double dsc = ldexp(dq[h], -ex), esc = ldexp(eq[h], -ex);
        const float ef = (float)esc;
        sd[q] = (float)dsc;
        se2[q] = ef * ef;
        sea[q] = fabsf(ef);
        dd[q] = dsc;
        ee2[q] = esc * esc;
    }
    __syncwarp();
    // Gershgorin interval of the window
    float lo = 3.0f, hi = -3.0f;
#pragma unroll
    for (int h = 0; h < H; ++h) {
        const int q = lane + 32 * h;
        if (q < w) {
            const float rad = (q >= 1 ? sea[q - 1] : 0.0f) + (q < w - 1 ? sea[q] : 0.0f);
            lo = fminf(lo, sd[q] - rad);
            hi = fmaxf(hi, sd[q] + rad);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    int k0 = 0;
    if (w > nb) k0 = min(max(window_count32(sd, se2, w, sd[w - 1]) - nb / 2, 0), w - nb);
    if (lane == 0) {
        sw.w = w;
        sw.k0 = k0;
        sw.ex = ex;
        sw.trivial = 0;
        sw.lo = lo - 1e-6f;
        sw.hi = hi + 1e-6f;
    }
    __syncwarp();
}

// All threads of the CTA (after a barrier that follows the setup): thread j finds shift j,
// j + blockDim.x, ...  FP32 bisection to a bracket, then the safeguarded FP64 Newton iteration.
__device__ void batch_shifts_solve(const double* __restrict__ dv, int64_t to, int nb, const ShiftWindow& sw,
                                   double* __restrict__ shifts, const float* sd, const float* se2,
                                   const double* dd, const double* ee2)
{
    if (sw.trivial) {
        for (int j = threadIdx.x; j < nb; j += blockDim.x) shifts[j] = dv[to - nb + j];
        return;
    }
    const int w = sw.w;
    for (int j = threadIdx.x; j < nb; j += blockDim.x) {
        const int k = sw.k0 + j;
        float a = sw.lo, b = sw.hi;
        for (int it = 0; it < 40; ++it) {
            const float mid = 0.5f * (a + b);
            if (!(mid > a && mid < b)) break;
            if (window_count32(sd, se2, w, mid) > k) b = mid;
            else a = mid;
        }
        // FP64 refinement inside a bracket kept by FP64 Sturm counts
        double A = (double)a - 4e-7, B = (double)b + 4e-7;
        double x = 0.5 * ((double)a + (double)b);
        for (int it = 0; it < 5; ++it) {
            double p, dp;
            int below;
            char_poly(dd, ee2, w, x, p, dp, below);
            if (below > k) B = x;
            else A = x;
            const double step = p / dp;
            // converged: a step below the last bits ends the iteration first (such a step can
            // land on the bracket's edge, which the safeguard below would turn into a jump)
            if (fabs(step) <= 4e-16 * fabs(x) + 1e-300) break;
            double xn = x - step;
            if (!(xn > A && xn < B)) xn = 0.5 * (A + B);
            x = xn;
        }
        shifts[j] = ldexp(x, sw.ex);
    }
}

// The bulges of a batch.  Bulge j (CTA j) runs the two-warp sweep of sweep_nr_2w (same split,
// mailbox and barriers) with shift shifts[j] over the batch's block, a few steps behind bulge
// j-1, reading only what bulge j-1 has stored: step k of a sweep stores dv[k-1] and ev[k-2] (0-based; its last step also
// dv[k] and ev[k-1]), so before its loads for step i+1 (dv[i+1], ev[i+1]) bulge j needs bulge
// j-1 through step min(i+3, to-1).  The helper warp's store thread releases the bulge's
// progress every (prog_mask + 1) steps and at its last step (st.release.gpu); the next bulge's
// warps read it with ld.acquire.gpu only when the value they hold is too small, and read
// dv/ev through L2 (ld.global.cg), never from a stale L1 line.  Bulge j waits only for bulge
// j-1 and the CTAs are co-resident (one cooperative launch), so the waits form one chain that
// starts at bulge 0, which waits for none.  Every wait is bounded (about 2 s of SM clock): one
// that gives up sets the device error word, and the warp carries on without waiting, so the
// two warps' barrier protocol still completes; the call then reports the error.
// The rotation is givens_nr_core (reference form out of its range) without the rounding
// proof: the batch is not the reference's sweep sequence, so there are no bits to match.
// `hold` (the test hook of symeig_set_test_stall, bulge 0 only) withholds every release, so
// the next bulge's wait runs out.

__device__ __forceinline__ long long ld_acquire_gpu(const long long* p)
{
    long long v;
    asm volatile("ld.acquire.gpu.global.s64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_gpu(long long* p, long long v)
{
    asm volatile("st.release.gpu.global.s64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Every lane polls with its own acquire load, and the warp moves on together: when all lanes
// saw the value needed (it keeps their minimum, which every lane has synchronised with, the
// progress word only growing) or when any lane's wait ran out.
struct PipeWait {
    const long long* pred;  // progress word of the bulge ahead; null for bulge 0
    int* err;
    long long known;        // the smallest value the warp's lanes last read (warp-uniform)
    __device__ __forceinline__ void until(long long need)
    {
        if (pred == nullptr || known >= need) return;
        const long long t0 = clock64();
        for (;;) {
            long long v = ld_acquire_gpu(pred);
            if (__all_sync(0xffffffffu, v >= need)) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
                known = v;
                return;
            }
            const bool give_up = *(volatile int*)err != 0 || clock64() - t0 > 4000000000LL;
            if (__any_sync(0xffffffffu, give_up)) {
                if ((threadIdx.x & 31) == 0) atomicExch(err, 1);
                known = 0x7fffffffffffffffLL;  // stop waiting for the rest of the sweep
                return;
            }
        }
    }
};

__device__ void sweep_bulge_2w(double* __restrict__ dv, double* __restrict__ ev, int64_t from,
                               int64_t to, double mu, double* __restrict__ grid,
                               const int32_t* __restrict__ thick, int64_t rows, int32_t layer,
                               int32_t jofs, double nz, NrMail* mail, PipeWait pw,
                               long long* __restrict__ my_prog, int64_t prog_mask, bool hold)
{
    const int warp = threadIdx.x >> 5;
    const bool lead = (threadIdx.x & 31) == 0;
    pw.until(min(from + 2, to - 1));
    const double H11 = __ldcg(dv + from - 1), H21 = __ldcg(ev + from - 1);
    if (warp == 0) {
        double f = __dsub_rn(H11, mu), g = H21, gg = mulz(H21, H21, nz);
        double B11 = H11, B21 = H21;
        double B22n = __ldcg(dv + from);
        double B23n = (from + 2 <= to) ? __ldcg(ev + from) : 0.0;
        for (int64_t i = from; i <= to - 1; ++i) {
            const double B22 = B22n, B23 = B23n;
            pw.until(min(i + 3, to - 1));
            if (i + 1 <= to - 1) B22n = __ldcg(dv + i + 1);
            if (i + 3 <= to) B23n = __ldcg(ev + i + 1);
            const NrRot o = givens_nr_core(f, g, gg, nz);
            double c = o.c, s = o.s, r = o.r;
            if (!nr_in_range(f, g)) givens_fast(f, g, c, s, r, nz);
            if (i > from) {
                nb_sync(kBarB);
                const NrMail& pv = mail[(i - 1) & 1];
                B11 = pv.b22pp;
                B21 = pv.e_next;
            }
            NrMail& mb = mail[i & 1];
            mb.c = c; mb.s = s; mb.r = r;
            nb_arrive(kBarCS);
            const double B11p = __fma_rn(c, B11, mulz(s, B21, nz));
            const double B12p = __fma_rn(c, B21, mulz(s, B22, nz));
            f = __fma_rn(B12p, c, -mulz(B11p, s, nz));
            g = (i + 2 <= to) ? mulz(s, B23, nz) : 0.0;
            gg = mulz(g, g, nz);
        }
    } else {
        double B11 = H11, B21 = H21;
        double B22n = __ldcg(dv + from);
        double B23n = (from + 2 <= to) ? __ldcg(ev + from) : 0.0;
        int32_t thn = layer <= 0 ? thick[from - 1] : 0;
        for (int64_t i = from; i <= to - 1; ++i) {
            const double B22 = B22n, B23 = B23n;
            const int32_t th = thn;
            pw.until(min(i + 3, to - 1));
            if (i + 1 <= to - 1) B22n = __ldcg(dv + i + 1);
            if (i + 3 <= to) B23n = __ldcg(ev + i + 1);
            if (layer <= 0 && i + 1 <= to - 1) thn = thick[i];
            nb_sync(kBarCS);
            const NrMail& mb = mail[i & 1];
            const double c = mb.c, s = mb.s, r = mb.r;
            const double e_next = (i + 2 <= to) ? mulz(c, B23, nz) : 0.0;
            const double sB21 = mulz(s, B21, nz);
            const double B21p = __fma_rn(c, B21, -mulz(s, B11, nz));
            const double B22p = __fma_rn(c, B22, -sB21);
            const double B22pp = __fma_rn(B22p, c, -mulz(B21p, s, nz));
            if (i < to - 1) {
                NrMail& mo = mail[i & 1];
                mo.b22pp = B22pp;
                mo.e_next = e_next;
                nb_arrive(kBarB);
            }
            const double B11p = __fma_rn(c, B11, sB21);
            const double B12p = __fma_rn(c, B21, mulz(s, B22, nz));
            const double B11pp = __fma_rn(B11p, c, mulz(B12p, s, nz));
            if (lead) {
                dv[i - 1] = B11pp;
                if (i > from) ev[i - 2] = r;
                const int32_t L = layer > 0 ? layer : th + 1 + jofs;
                *reinterpret_cast<double2*>(grid + 2 * ((i - 1) + (int64_t)(L - 1) * rows)) =
                    make_double2(c, s);
                if (i == to - 1) {
                    dv[i] = B22pp;
                    ev[i - 1] = __fma_rn(B12p, c, -mulz(B11p, s, nz));
                }
                if (!hold && (i == to - 1 || ((i - from) & prog_mask) == prog_mask)) st_release_gpu(my_prog, i);
            }
            B11 = B22pp;
            B21 = e_next;
        }
    }
}

// One CTA of two warps per bulge; dynamic shared memory (kBatchSmem) keeps one CTA per SM, so
// no two bulges share an SM's FP64 unit.
constexpr int kBatchSmem = 120 * 1024;

__global__ void __launch_bounds__(64, 1)
bulge_batch_kernel(const ChaseState* __restrict__ st, double* __restrict__ dv,
                   double* __restrict__ ev, double* __restrict__ grid,
                   const int32_t* __restrict__ thick, BulgeScratch* __restrict__ bs,
                   int* __restrict__ err)
{
    __shared__ NrMail mail[2];
    const int j = blockIdx.x;
    if (st->status != CHASE_BATCH) return;  // a launch queued ahead after the batches ended
    const int32_t nb = st->b_bulges;
    if (j >= nb) return;
    const int64_t n = st->n, from = st->b_from, to = st->b_to;
    const int64_t rows = n > 1 ? n - 1 : 1;
    const int32_t L0 = st->b_layer0;
    PipeWait pw{j > 0 ? &bs->prog[j - 1] : nullptr, err, -1};
    sweep_bulge_2w(dv, ev, from, to, bs->shifts[j], grid, thick, rows, L0 > 0 ? L0 + j : 0, j,
                   st->neg_zero, mail, pw, &bs->prog[j], (int64_t)st->ms_prog_mask,
                   st->test_stall != 0 && j == 0);
}

// One flush: the reference's inner loop from `to = last_block_ends_at` until the matrix is
// split into converged parts, every block has reached max_layers, or iter > maxiter.
// Warp 0 runs the control flow and the O(n) scans with ballots; each sweep runs on both
// warps (sweep_nr_2w) after both copy the entries it may change to `bak` (2n doubles).
//
// Exact-order placement (st->exact_order != 0).  The reference applies a flush's grid in
// layer-major order, which equals the order the chase made the rotations only while every
// sweep meets equal layer counts on its indices; when a split block re-merges it does not,
// and the reference's Q loses accuracy.  In exact-order mode every rotation of a sweep over
// [from, to] goes to the single layer
//     L = 1 + max(place[from..to-1], place[to], place[from-1] - 1)
// and skipped slots are set to (1,0), so the layer-major order of the grid is the chase's
// order.  The chase itself (and so every eigenvalue) is the reference's.  A sweep whose layer
// would exceed the grid's capacity ends the flush early (st->early_flushes counts these).
struct Decision {
    int64_t from, to;
    double mu;
    int32_t layer;
    int32_t action;  // 0 stop, 1 sweep, 2 no sweep this iteration, 3 multishift batch
    int32_t bulges;  // action 3: sweeps of the batch
};

__global__ void __launch_bounds__(64, 1)
chase_kernel(ChaseState* __restrict__ st, double* __restrict__ dv, double* __restrict__ ev,
             double* __restrict__ grid, int32_t* __restrict__ thick, int32_t* __restrict__ place,
             double* __restrict__ bak, BulgeScratch* __restrict__ bs, int32_t resume_only)
{
    __shared__ NrMail mail[2];
    __shared__ Decision dec;
    __shared__ int32_t fail;
    __shared__ float ms_d[kWinMax], ms_e2[kWinMax], ms_ea[kWinMax];
    __shared__ double ms_dd[kWinMax], ms_ee2[kWinMax];
    __shared__ ShiftWindow swin;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int64_t n = st->n;
    const int64_t start = st->start;
    const double tol = st->tol;
    const double nz = st->neg_zero;
    const int32_t max_layers = st->max_layers;
    const int32_t grid_layers = st->grid_layers;
    const bool exact = st->exact_order != 0;
    const int64_t maxiter = st->maxiter;
    const int32_t mode = st->chase_mode;
    const int32_t ms_bulges = min(max(st->ms_bulges, 2), kMaxBulges);
    const int32_t ms_min = min(max(st->ms_min_bulges, 2), ms_bulges);
    const int64_t ms_rows = max(st->ms_rows, 4);
    int64_t iter = st->iter;
    int64_t lbe = st->last_block_ends_at;
    const int64_t rows = n > 1 ? n - 1 : 1;
    int64_t redone = 0;

    // chase_mode 3 returns to the host for each multishift batch; the launch after the batch
    // resumes the flush where it stopped, first recording the batch in thick/place: every
    // index of its block got one layer per bulge (bulge j at layer thick + 1 + j, or at the
    // exact-order layer b_layer0 + j).
    const bool resume = st->resume != 0;
    if (resume_only && !resume) return;  // a launch queued ahead after the batches ended
    if (!resume) {
        for (int64_t q = threadIdx.x; q < n; q += 64) {
            thick[q] = 0;
            place[q] = 0;
        }
    } else {
        const int32_t nbk = st->b_bulges, L0 = st->b_layer0;
        for (int64_t q = st->b_from - 1 + threadIdx.x; q < st->b_to - 1; q += 64) {
            const int32_t t = thick[q] + nbk;
            thick[q] = t;
            place[q] = L0 > 0 ? L0 + nbk - 1 : t;
        }
    }
    if (threadIdx.x == 0) fail = 0;
    __syncthreads();

    bool did = resume && st->r_did != 0;
    int64_t rotations = resume ? st->r_rotations : 0, min_from = resume ? st->r_min_from : n + 1;
    int64_t max_to = resume ? st->r_max_to : 0, early = resume ? st->r_early : 0;
    int32_t status = CHASE_RUNNING;
    int64_t to = resume ? st->r_to : lbe;
    Decision last{};

    for (;;) {
        if (warp == 0) {
            Decision d{0, 0, 0.0, 0, 2, 1};
            if (iter > maxiter) {
                status = CHASE_MAXITER;
                d.action = 0;
            } else if (to <= start) {
                d.action = 0;
            } else {
                // from = largest j+1 with is_small(j), j in [start, to-1]; start if none.
                // kScanUnroll chunks of 32 per round: their loads are issued together, so a
                // long block costs one memory latency per 32 * kScanUnroll entries.
                int64_t from = start;
                for (int64_t base = to - 1; base >= start; base -= 32 * kScanUnroll) {
                    bool sm[kScanUnroll];
#pragma unroll
                    for (int u = 0; u < kScanUnroll; ++u) {
                        const int64_t j = base - 32 * u - lane;
                        sm[u] = (j >= start) && is_small(dv, ev, j, tol);
                    }
                    bool found = false;
#pragma unroll
                    for (int u = 0; u < kScanUnroll; ++u) {
                        const unsigned mask = __ballot_sync(0xffffffffu, sm[u]);
                        if (!found && mask) {
                            from = base - 32 * u - (__ffs(mask) - 1) + 1;
                            found = true;
                        }
                    }
                    if (found) break;
                }
                if (from == to) {
                    if (lane == 0) ev[from - 2] = 0.0;
                    if (to == lbe) lbe -= 1;
                    to -= 1;
                } else {
                    int32_t mx = 0;
#pragma unroll 8
                    for (int64_t q = from - 1 + lane; q <= to - 1; q += 32) mx = max(mx, thick[q]);
                    mx = warp_max(mx);
                    if (mx == max_layers) {
                        to = from - 1;
                    } else {
                        int32_t layer = 0;
                        bool go = true;
                        if (exact) {
                            int32_t L = 0;
#pragma unroll 8
                            for (int64_t q = from - 1 + lane; q <= to - 2; q += 32) L = max(L, place[q]);
                            L = warp_max(L);
                            if (to <= n - 1) L = max(L, place[to - 1]);
                            if (from >= 2) L = max(L, place[from - 2] - 1);
                            layer = L + 1;
                            if (layer > grid_layers) {
                                early = 1;
                                go = false;
                                d.action = 0;
                            } else {
                                // slots skipped by the jump to `layer` hold the identity
                                for (int64_t q = from - 1 + lane; q <= to - 2; q += 32)
                                    for (int32_t g = place[q] + 1; g < layer; ++g) {
                                        double* p = grid + 2 * (q + (int64_t)(g - 1) * rows);
                                        p[0] = 1.0;
                                        p[1] = 0.0;
                                    }
                            }
                        }
                        if (go) {
                            // mode 3: as many bulges as the block's length, its layer room
                            // (the capacity rule of that many single sweeps) and maxiter allow
                            int64_t nbl = 1;
                            if (mode == 3) {
                                int64_t cap = (int64_t)max_layers - mx;
                                if (exact) cap = min(cap, (int64_t)grid_layers - layer + 1);
                                nbl = min(min((int64_t)ms_bulges, (to - from + 1) / ms_rows), cap);
                                nbl = min(nbl, maxiter - iter + 1);
                                // a batch too small to repay its launches and shift solve
                                // runs as one sweep with the reference's shift
                                if (nbl < ms_min) nbl = 1;
                            }
                            if (nbl >= 2) {
                                batch_shifts_setup(dv, ev, from, to, (int)nbl, swin, ms_d, ms_e2, ms_ea, ms_dd, ms_ee2);
                                d.bulges = (int32_t)nbl;
                                d.action = 3;
                            } else {
                                d.mu = wilkinson_shift(dv[to - 2], dv[to - 1], ev[to - 2]);
                                d.action = 1;
                            }
                            d.from = from;
                            d.to = to;
                            d.layer = layer;
                            did = true;
                            iter += nbl >= 2 ? nbl : 1;
                            rotations += (nbl >= 2 ? nbl : 1) * (to - from);
                            min_from = min(min_from, from);
                            max_to = max(max_to, to);
                        }
                    }
                }
                if (d.action == 2 && to <= start) d.action = 0;
            }
            if (lane == 0) dec = d;
        }
        __syncthreads();
        const Decision d = dec;
        last = d;
        if (d.action == 3) {
            // the batch's shifts, one per thread, then the batch runs in its own launch
            batch_shifts_solve(dv, d.to, d.bulges, swin, bs->shifts, ms_d, ms_e2, ms_dd, ms_ee2);
            break;
        }
        if (d.action == 1) {
            // entries the sweep may change: dv[from-1 .. to-1], ev[from-1 .. to-2] (0-based)
            const int64_t q0 = d.from - 1, q1 = d.to - 1;
            bool redo = mode == 1;
            if (mode != 1) {
                for (int64_t q = q0 + threadIdx.x; q <= q1; q += 64) {
                    bak[q] = dv[q];
                    if (q < q1) bak[n + q] = ev[q];
                }
                __syncthreads();
                sweep_nr_2w(dv, ev, d.from, d.to, d.mu, grid, thick, rows, d.layer, nz, mail, &fail);
                __syncthreads();
                redo = fail != 0 || mode == 2;
                if (redo) {
                    for (int64_t q = q0 + threadIdx.x; q <= q1; q += 64) {
                        dv[q] = bak[q];
                        if (q < q1) ev[q] = bak[n + q];
                    }
                    ++redone;
                }
            }
            if (redo) {
                // the reference form on one thread; it updates thick/place itself
                __syncthreads();
                if (threadIdx.x == 0)
                    single_shift<false>(dv, ev, d.from, d.to, d.mu, grid, thick, place, rows, d.layer, nz);
                if (threadIdx.x == 0) fail = 0;
            } else {
                for (int64_t q = q0 + threadIdx.x; q < q1; q += 64) {
                    const int32_t t = thick[q] + 1;
                    thick[q] = t;
                    place[q] = d.layer > 0 ? d.layer : t;
                }
            }
        }
        __syncthreads();
        if (d.action == 0) break;  // both warps leave on the same decision
    }

    if (last.action == 3) {
        // hand the batch to the host: its block, its layers, and the loop state to resume
        for (int q = threadIdx.x; q < last.bulges; q += 64) bs->prog[q] = -1;
        if (threadIdx.x == 0) {
            st->status = CHASE_BATCH;
            st->resume = 1;
            st->b_bulges = last.bulges;
            st->b_from = last.from;
            st->b_to = last.to;
            st->b_layer0 = last.layer;
            st->r_did = did ? 1 : 0;
            st->r_to = to;
            st->r_rotations = rotations;
            st->r_min_from = min_from;
            st->r_max_to = max_to;
            st->r_early = early;
            st->iter = iter;
            st->last_block_ends_at = lbe;
            st->redone_sweeps += redone;
            st->batches += 1;
        }
        return;
    }
    if (warp == 0) {
        int32_t kmax = 0;
        for (int64_t q = lane; q < n; q += 32) kmax = max(kmax, place[q]);
        kmax = warp_max(kmax);
        if (lane == 0) {
            if (status == CHASE_RUNNING) status = did ? CHASE_FLUSH : CHASE_CONVERGED;
            st->status = status;
            st->iter = iter;
            st->last_block_ends_at = lbe;
            st->rotations = rotations;
            st->min_from = min_from;
            st->max_to = max_to;
            st->max_thickness = kmax;
            st->total_rotations += rotations;
            st->early_flushes += early;
            st->redone_sweeps += redone;
            st->resume = 0;
        }
    }
}

// ---- batched chase: one lane per matrix --------------------------------------------------
//
// A chase step is a chain of ~55 dependent FP64 operations, and on GB300 an FP64 instruction
// occupies its sub-partition's FP64 unit for 64 cycles whether 1 or 32 lanes are active.  So
// for many independent matrices each lane runs its own matrix's flush: 32 chases share every
// FP64 instruction.  The host sorts matrices by size so that a warp's lanes sweep similar
// lengths.  The scans (deflation, thickest column, exact-order layer) are serial per lane.

// One flush of one matrix (the same steps, in the same order, as chase_kernel).
__device__ void chase_flush_lane(ChaseState* __restrict__ st, double* __restrict__ dv,
                                 double* __restrict__ ev, double* __restrict__ grid,
                                 int32_t* __restrict__ thick, int32_t* __restrict__ place)
{
    const int64_t n = st->n;
    const int64_t start = st->start;
    const double tol = st->tol;
    const int32_t max_layers = st->max_layers;
    const int32_t grid_layers = st->grid_layers;
    const bool exact = st->exact_order != 0;
    const int64_t maxiter = st->maxiter;
    int64_t iter = st->iter;
    int64_t lbe = st->last_block_ends_at;
    const int64_t rows = n > 1 ? n - 1 : 1;

    for (int64_t q = 0; q < n; ++q) {
        thick[q] = 0;
        place[q] = 0;
    }
    bool did = false;
    int64_t rotations = 0, min_from = n + 1, max_to = 0, early = 0;
    int32_t status = CHASE_RUNNING;
    int64_t to = lbe;
    for (;;) {
        if (iter > maxiter) { status = CHASE_MAXITER; break; }
        if (to <= start) break;
        int64_t from = to;
        while (from > start && !is_small(dv, ev, from - 1, tol)) from -= 1;
        if (from == to) {
            ev[from - 2] = 0.0;
            if (to == lbe) lbe -= 1;
            to -= 1;
        } else {
            int32_t mx = 0;
            for (int64_t q = from - 1; q <= to - 1; ++q) mx = max(mx, thick[q]);
            if (mx == max_layers) {
                to = from - 1;
            } else {
                int32_t layer = 0;
                if (exact) {
                    int32_t L = 0;
                    for (int64_t q = from - 1; q <= to - 2; ++q) L = max(L, place[q]);
                    if (to <= n - 1) L = max(L, place[to - 1]);
                    if (from >= 2) L = max(L, place[from - 2] - 1);
                    layer = L + 1;
                    if (layer > grid_layers) { early = 1; break; }
                    for (int64_t q = from - 1; q <= to - 2; ++q)
                        for (int32_t g = place[q] + 1; g < layer; ++g) {
                            double* p = grid + 2 * (q + (int64_t)(g - 1) * rows);
                            p[0] = 1.0;
                            p[1] = 0.0;
                        }
                }
                const double mu = wilkinson_shift(dv[to - 2], dv[to - 1], ev[to - 2]);
                single_shift<true>(dv, ev, from, to, mu, grid, thick, place, rows, layer, st->neg_zero);
                did = true;
                iter += 1;
                rotations += to - from;
                min_from = min(min_from, from);
                max_to = max(max_to, to);
            }
        }
        if (to <= start) break;
    }
    int32_t kmax = 0;
    for (int64_t q = 0; q < n; ++q) kmax = max(kmax, place[q]);
    if (status == CHASE_RUNNING) status = did ? CHASE_FLUSH : CHASE_CONVERGED;
    st->status = status;
    st->iter = iter;
    st->last_block_ends_at = lbe;
    st->rotations = rotations;
    st->min_from = min_from;
    st->max_to = max_to;
    st->max_thickness = kmax;
    st->total_rotations += rotations;
    st->early_flushes += early;
}

__global__ void __launch_bounds__(32)
chase_batched_kernel(const BatchMat* __restrict__ mats, const int32_t* __restrict__ order,
                     int32_t count, ChaseState* __restrict__ states, double* __restrict__ d,
                     double* __restrict__ e, double* __restrict__ grids,
                     int32_t* __restrict__ thick, int32_t* __restrict__ place)
{
    const int32_t k = blockIdx.x * 32 + threadIdx.x;
    if (k >= count) return;
    const int32_t i = order[k];
    ChaseState* st = states + i;
    const int32_t s0 = st->status;
    if (s0 == CHASE_CONVERGED || s0 == CHASE_MAXITER) return;
    const BatchMat mt = mats[i];
    chase_flush_lane(st, d + mt.doff, e + mt.eoff, grids + mt.goff, thick + mt.doff, place + mt.doff);
}

// get_rotation(f, g) (src/simple_givens.jl:20-23) elementwise: form 0 the chase's Newton form
// (givens_nr), form 1 the reference form (givens).
__global__ void get_rotation_kernel(int64_t count, const double* __restrict__ f,
                                    const double* __restrict__ g, double* __restrict__ c,
                                    double* __restrict__ s, double* __restrict__ r, int32_t form,
                                    double nz)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double fi = f[i], gi = g[i];
        double ci, si, ri;
        if (form == 1) givens(fi, gi, ci, si, ri);
        else givens_nr(fi, gi, mulz(gi, gi, nz), ci, si, ri, nz);
        c[i] = ci;
        s[i] = si;
        r[i] = ri;
    }
}

}  // namespace

cudaError_t launch_get_rotation(int64_t count, const double* f, const double* g, double* c,
                                double* s, double* r, int32_t form, cudaStream_t stream)
{
    if (count <= 0) return cudaSuccess;
    const int64_t blocks = (count + 255) / 256 < 1216 ? (count + 255) / 256 : 1216;
    get_rotation_kernel<<<(unsigned)blocks, 256, 0, stream>>>(count, f, g, c, s, r, form, -0.0);
    return cudaGetLastError();
}

cudaError_t launch_chase(ChaseState* state, double* d, double* e, double* grid, int32_t* thick,
                         int32_t* place, double* bak, BulgeScratch* bs, int32_t resume_only,
                         cudaStream_t stream)
{
    chase_kernel<<<1, 64, 0, stream>>>(state, d, e, grid, thick, place, bak, bs, resume_only);
    return cudaGetLastError();
}

cudaError_t launch_bulge_batch(const ChaseState* state, double* d, double* e, double* grid,
                               const int32_t* thick, BulgeScratch* bs, int* err, int32_t bulges,
                               cudaStream_t stream)
{
    if (bulges < 2 || bulges > kMaxBulges) return cudaErrorInvalidValue;
    cudaError_t ce = cudaFuncSetAttribute(bulge_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          kBatchSmem);
    if (ce != cudaSuccess) return ce;
    void* args[] = {(void*)&state, (void*)&d, (void*)&e, (void*)&grid, (void*)&thick, (void*)&bs, (void*)&err};
    return cudaLaunchCooperativeKernel((const void*)bulge_batch_kernel, dim3((unsigned)bulges), dim3(64), args,
                                       (size_t)kBatchSmem, stream);
}

cudaError_t launch_chase_batched(const BatchMat* mats, const int32_t* order, int32_t count,
                                 ChaseState* states, double* d, double* e, double* grids,
                                 int32_t* thick, int32_t* place, cudaStream_t stream)
{
    if (count <= 0) return cudaSuccess;
    chase_batched_kernel<<<(count + 31) / 32, 32, 0, stream>>>(mats, order, count, states, d, e,
                                                               grids, thick, place);
    return cudaGetLastError();
}

}  // namespace symeig
