// givens.cuh -- LinearAlgebra.givensAlgorithm (LAPACK 3.2 DLARTG port, called by get_rotation,
// src/simple_givens.jl:20-23) on the device, in three forms that give identical bits:
//
//   givens()        the reference form, branch by branch, with __dsqrt_rn / __ddiv_rn;
//   givens_fast()   the same with its branch tests on the integer pipe;
//   givens_nr()     the plain branch (the one a bulge chase takes) from FMA-only Newton steps,
//                   each result proved correctly rounded by an exact FMA residual, and
//                   givens() for everything else.
//
// On GB300 an FP64 instruction holds its warp for ~64 cycles and FP64 compares count as FP64
// instructions, so the branch tests are done on bit patterns and the square root and the two
// divisions are replaced by 18 FMAs whose results are checked rather than trusted.
#pragma once
#include <cstdint>

namespace symeig {
namespace gv {

// ---- bit-pattern tests on the integer pipe ----------------------------------------------
__device__ __forceinline__ uint64_t bits(double x) { return (uint64_t)__double_as_longlong(x); }
__device__ __forceinline__ double from_bits(uint64_t b) { return __longlong_as_double((long long)b); }
__device__ __forceinline__ uint64_t abs_bits(double x) { return bits(x) & 0x7FFFFFFFFFFFFFFFull; }
__device__ __forceinline__ bool nan_bits(uint64_t a) { return a > 0x7FF0000000000000ull; }
__device__ __forceinline__ double neg(double x) { return from_bits(bits(x) ^ 0x8000000000000000ull); }
__device__ __forceinline__ double neg_if(double x, bool p)
{
    return from_bits(bits(x) ^ (p ? 0x8000000000000000ull : 0ull));
}
// x < 0.0
__device__ __forceinline__ bool is_negative(double x)
{
    const uint64_t b = bits(x), a = b & 0x7FFFFFFFFFFFFFFFull;
    return (b >> 63) != 0 && a != 0 && !nan_bits(a);
}
// a*b as an FMA with a -0.0 addend supplied at run time: bit-identical to the product, and an
// FP64 FMA issues faster than an FP64 multiply on GB300.
__device__ __forceinline__ double mulz(double a, double b, double nz) { return __fma_rn(a, b, nz); }

__device__ __forceinline__ double jl_max(double a, double b) { return (a > b || a != a) ? a : b; }

// Which branch of givensAlgorithm (f, g) takes: 0 g == 0, 1 f == 0, 2 scaled down,
// 3 scaled up, 4 plain (also when f or g is NaN: the NaN scale fails both range tests).
__device__ __forceinline__ int givens_case(double f, double g)
{
    const uint64_t af = abs_bits(f), ag = abs_bits(g);
    if (ag == 0) return 0;
    if (af == 0) return 1;
    if (nan_bits(af) || nan_bits(ag)) return 4;
    const uint64_t m = af > ag ? af : ag;
    if (m >= 0x5E40000000000000ull) return 2;  // max(|f|,|g|) >= 2^485
    if (m <= 0x21A0000000000000ull) return 3;  // max(|f|,|g|) <= 2^-485
    return 4;
}

// The sign convention of givensAlgorithm: flip (c, s, r) when |f| > |g| and c < 0.
__device__ __forceinline__ bool givens_flip(double f, double g, double c)
{
    const uint64_t af = abs_bits(f), ag = abs_bits(g);
    return af > ag && !nan_bits(af) && !nan_bits(ag) && is_negative(c);
}

// LinearAlgebra.givensAlgorithm, branch by branch.
__device__ __forceinline__ void givens(double f, double g, double& cs, double& sn, double& r)
{
    const double safmn2 = 0x1p-485;
    const double safmx2 = 0x1p+485;
    if (g == 0.0) {
        cs = 1.0; sn = 0.0; r = f;
    } else if (f == 0.0) {
        cs = 0.0; sn = 1.0; r = g;
    } else {
        double f1 = f, g1 = g;
        double scale = jl_max(fabs(f1), fabs(g1));
        if (scale >= safmx2) {
            int count = 0;
            do {
                ++count;
                f1 = __dmul_rn(f1, safmn2); g1 = __dmul_rn(g1, safmn2);
                scale = jl_max(fabs(f1), fabs(g1));
            } while (scale >= safmx2 && count < 20);
            r = __dsqrt_rn(__dadd_rn(__dmul_rn(f1, f1), __dmul_rn(g1, g1)));
            cs = __ddiv_rn(f1, r); sn = __ddiv_rn(g1, r);
            for (int i = 0; i < count; ++i) r = __dmul_rn(r, safmx2);
        } else if (scale <= safmn2) {
            int count = 0;
            do {
                ++count;
                f1 = __dmul_rn(f1, safmx2); g1 = __dmul_rn(g1, safmx2);
                scale = jl_max(fabs(f1), fabs(g1));
            } while (scale <= safmn2 && count < 64);  // 64 steps cover every subnormal
            r = __dsqrt_rn(__dadd_rn(__dmul_rn(f1, f1), __dmul_rn(g1, g1)));
            cs = __ddiv_rn(f1, r); sn = __ddiv_rn(g1, r);
            for (int i = 0; i < count; ++i) r = __dmul_rn(r, safmn2);
        } else {
            r = __dsqrt_rn(__dadd_rn(__dmul_rn(f1, f1), __dmul_rn(g1, g1)));
            cs = __ddiv_rn(f1, r); sn = __ddiv_rn(g1, r);
        }
        if (fabs(f) > fabs(g) && cs < 0.0) { cs = -cs; sn = -sn; r = -r; }
    }
}

// givensAlgorithm with its branch tests on the integer pipe and its products issued as FMAs.
__device__ __forceinline__ void givens_fast(double f, double g, double& cs, double& sn, double& r,
                                            double nz)
{
    if (givens_case(f, g) != 4) {
        givens(f, g, cs, sn, r);
        return;
    }
    r = __dsqrt_rn(__dadd_rn(mulz(f, f, nz), mulz(g, g, nz)));
    cs = __ddiv_rn(f, r);
    sn = __ddiv_rn(g, r);
    if (givens_flip(f, g, cs)) { cs = neg(cs); sn = neg(sn); r = neg(r); }
}

// ---- the plain branch from Newton steps -------------------------------------------------
//
// Inputs in range (nr_in_range): f, g nonzero and finite, max(|f|,|g|) in [2^-450, 2^450),
// min(|f|,|g|) >= max(|f|,|g|) * 2^-400.  Then givensAlgorithm takes its plain branch and
//   x = RN(RN(f f) + RN(g g)) in [2^-900, 2^901),  r = RN(sqrt x) in [2^-450, 2^451),
//   |c|, |s| in [2^-401, 1],
// and every residual below stays a normal number.  The method (Newton's iteration for
// 1/sqrt and the FMA remainder correction of Markstein, "IA-64 and Elementary Functions",
// 2000, ch. 8):
//   y  ~ 1/sqrt(x)                       rsqrt.approx.ftz.f64 (relative error ~2^-23)
//   g0 = x y, h0 = y/2;  d = 1/2 - g0 h0;  g1 = g0 + g0 d, h1 = h0 + h0 d     (error ~2^-44)
//   r  = g1 + (x - g1^2) h1                                                   (error ~2^-88)
//   q  = a y' + (a - (a y') r) y',  y' = 2 h1 ~ 1/r, for a = +-f and +-g      (error ~2^-88)
// Proofs of rounding (exact because each candidate is within one ulp, so each residual is a
// multiple of the product of the two ulps and fits in 53 bits):
//   r = RN(sqrt x)  iff  -r u- < x - r^2 <= r u        (u = ulp(r), u- = gap below r)
//   q = RN(a / r)   iff  -r v- / 2 < sgn(a) (a - q r) < r v / 2  (v = ulp(q), v- gap below |q|)
// (a quotient of two doubles is never a midpoint, so the strict bounds lose nothing).  A
// candidate that is off by one ulp or more fails its bound, and then givens() is used.

__device__ __forceinline__ bool nr_in_range(double f, double g)
{
    const uint64_t af = abs_bits(f), ag = abs_bits(g);
    const uint64_t mx = af > ag ? af : ag, mn = af > ag ? ag : af;
    const int emx = (int)(mx >> 52), emn = (int)(mn >> 52);
    return emx >= 1023 - 450 && emx <= 1023 + 449 && emn >= emx - 400;
}

// y/2 and 2y by exponent arithmetic (y normal, result normal)
__device__ __forceinline__ double half_of(double y) { return from_bits(bits(y) - (1ull << 52)); }
__device__ __forceinline__ double twice(double y) { return from_bits(bits(y) + (1ull << 52)); }

__device__ __forceinline__ double rsqrt_seed(double x)
{
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    return y;
}

// x - r^2 (given as rr) within (-r u-, r u]
__device__ __forceinline__ bool sqrt_proved(double r, double rr)
{
    const uint64_t rb = bits(r);
    const uint64_t er = rb >> 52;                                  // biased exponent of r
    const uint64_t up = rb + ((er - 1075ull) << 52);               // r * 2^(er-1023-52)
    const uint64_t dn = (rb & 0x000FFFFFFFFFFFFFull) == 0 ? up - (1ull << 52) : up;
    const uint64_t rrb = bits(rr), rra = rrb & 0x7FFFFFFFFFFFFFFFull;
    return (rrb >> 63) ? rra < dn : rra <= up;
}

// sgn(a) * e within (-r v- / 2, r v / 2), e = a - q r; q has the sign of a
__device__ __forceinline__ bool div_proved(double q, double r, double e, bool a_neg)
{
    const uint64_t qb = bits(q) & 0x7FFFFFFFFFFFFFFFull;
    const uint64_t eq = qb >> 52;
    const uint64_t up = bits(r) + ((eq - 1076ull) << 52);          // r * ulp(q) / 2
    const uint64_t dn = (qb & 0x000FFFFFFFFFFFFFull) == 0 ? up - (1ull << 52) : up;
    const uint64_t eb = bits(e) ^ (a_neg ? 0x8000000000000000ull : 0ull);
    const uint64_t ea = eb & 0x7FFFFFFFFFFFFFFFull;
    return (eb >> 63) ? ea < dn : ea < up;
}

// givensAlgorithm(f, g) for in-range inputs by the Newton form, sign convention applied, with
// x = RN(RN(f f) + gg) for the proof.  gg = RN(g*g).  Equal to givens() when
// givens_nr_proved() holds.  Negations are written as operand signs so that they fold into
// the FMAs.
struct NrRot {
    double c, s, r, x;
};

__device__ __forceinline__ NrRot givens_nr_core(double f, double g, double gg, double nz)
{
    const uint64_t af = abs_bits(f), ag = abs_bits(g);
    const bool flip = af > ag && (bits(f) >> 63) != 0;   // |f| > |g| and c = f/r < 0
    const double fs = neg_if(f, flip), gs = neg_if(g, flip);
    const double x = __dadd_rn(mulz(f, f, nz), gg);
    const double y = rsqrt_seed(x);
    const double g0 = mulz(x, y, nz);
    const double h0 = half_of(y);
    const double d = __fma_rn(-g0, h0, 0.5);
    const double g1 = __fma_rn(g0, d, g0);
    const double h1 = __fma_rn(h0, d, h0);
    const double e1 = __fma_rn(-g1, g1, x);
    const double r = __fma_rn(e1, h1, g1);
    const double yr = twice(h1);
    const double qc = mulz(fs, yr, nz), qs = mulz(gs, yr, nz);
    const double ec = __fma_rn(-qc, r, fs), es = __fma_rn(-qs, r, gs);
    NrRot o;
    o.c = __fma_rn(ec, yr, qc);
    o.s = __fma_rn(es, yr, qs);
    o.r = neg_if(r, flip);
    o.x = x;
    return o;
}

// Whether (c, s, r) from givens_nr_core(f, g, ...) with its x are the correctly rounded values
// (then they equal givens(f, g)); f, g in range.
__device__ __forceinline__ bool givens_nr_proved(double f, double g, double x, double c, double s,
                                                 double r_signed)
{
    const uint64_t af = abs_bits(f), ag = abs_bits(g);
    const bool flip = af > ag && (bits(f) >> 63) != 0;
    const double r = neg_if(r_signed, flip);
    const double fs = neg_if(f, flip), gs = neg_if(g, flip);
    const double rr = __fma_rn(-r, r, x);
    const double ec = __fma_rn(-c, r, fs), es = __fma_rn(-s, r, gs);
    return sqrt_proved(r, rr) && div_proved(c, r, ec, (bits(fs) >> 63) != 0) &&
           div_proved(s, r, es, (bits(gs) >> 63) != 0);
}

// givensAlgorithm(f, g) -> (c, s, r), gg = RN(g*g): the Newton form when in range and proved,
// else givens_fast().
__device__ __forceinline__ void givens_nr(double f, double g, double gg, double& cs, double& sn,
                                          double& r, double nz)
{
    if (nr_in_range(f, g)) {
        const NrRot o = givens_nr_core(f, g, gg, nz);
        if (givens_nr_proved(f, g, o.x, o.c, o.s, o.r)) {
            cs = o.c; sn = o.s; r = o.r;
            return;
        }
    }
    givens_fast(f, g, cs, sn, r, nz);
}

}  // namespace gv
}  // namespace symeig
