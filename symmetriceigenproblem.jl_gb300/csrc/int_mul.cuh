// int_mul.cuh -- correctly rounded FP64 products on the integer pipes.
//
// GB300 executes FP64 arithmetic at 2 lanes per SM per clock, about a sixtieth of its 32-bit
// integer rate.  The canonical rotation of the bulk apply, x' = fma(c, x, s*y) and
// y' = fma(c, y, -(s*x)), spends four FP64-pipe instructions per rotation and row, two of them
// on the products s*y and s*x.  Those two products are computed here from integer
// arithmetic instead, to the same bits as the FP64 multiply (IEEE 754 binary64,
// round-to-nearest-even), which leaves two FMAs per rotation-row on the FP64 pipe.
//
// Method (textbook IEEE multiplication; e.g. Muller et al., Handbook of Floating-Point
// Arithmetic, ch. 7-8): for normal operands a = (-1)^sa 2^(ea-1023) Ma / 2^52 with 53-bit
// significands Ma, Mb, the exact product is P = Ma * Mb, an integer in [2^104, 2^106).
//   * P from four 32 x 32 -> 64-bit multiply-adds on the 21-bit and 32-bit halves of Ma, Mb.
//   * H = floor(P / 2^42), a 64-bit integer in [2^62, 2^64), with every nonzero bit of
//     P mod 2^42 folded into H's bit 0 (a sticky bit: H's bits 0..8 lie below the rounding
//     position in either case, so only their being nonzero matters).
//   * The rounding position: k = 11 if H >= 2^63 (P >= 2^105) else 10.  Round to nearest even
//     (the sticky bit in H's bit 0, below the rounding position):
//     M = (H + 2^(k-1) - 1 + bit_k(H)) >> k, a 53-bit significand, or 2^53 when the rounding
//     carries out (then the exponent field below is one too small and adding M's implicit
//     bit position carries into it, which gives the right bits, up to an overflow to infinity).
//   * The biased exponent of the result is E = ea + eb - 1023 + (k - 10); the bits are
//     ((E - 1) << 52) + M with the sign sa xor sb.
// The integer path covers products of two normal numbers whose result exponent E, before
// rounding, lies in [1, 2046], and products with a zero factor and a finite other factor
// (the rotation grid's identity padding (1, 0) and the zeros of an initial Q = I are common):
// a zero factor makes P = 0 (no implicit bit) and forces the exponent field to 0, which
// yields the signed zero.  Everything else -- a subnormal, infinite or NaN operand, and
// results that underflow or overflow -- is flagged `special`, and the caller recomputes those
// lanes on the FP64 pipe (a warp-uniform branch taken only when some lane needs it).
//
// Both factors' significands enter through 32-bit halves, and the factor s of a rotation is
// shared by every row of Q, so split_factor() runs once per rotation and mul_rn_int() once per
// product.
#pragma once

#include <stdint.h>

namespace symeig {

struct SplitFactor {
    uint32_t m1;     // significand bits 32..52 with the implicit bit (21 bits); 0 for s = +-0
    uint32_t m0;     // significand bits 0..31
    uint32_t eadj;   // exponent field (in place, << 20) minus 1024 << 20, modulo 2^32
    uint32_t sign;   // sign bit (in place)
    bool zero;       // s = +-0
    bool special;    // subnormal, infinite or NaN
};

__device__ __forceinline__ SplitFactor split_factor(double s)
{
    const uint32_t hi = (uint32_t)__double2hiint(s), lo = (uint32_t)__double2loint(s);
    SplitFactor f;
    const uint32_t ef = hi & 0x7FF00000u;
    f.zero = ((hi & 0x7FFFFFFFu) | lo) == 0u;
    f.m1 = (hi & 0x000FFFFFu) | (f.zero ? 0u : 0x00100000u);
    f.m0 = lo;
    f.eadj = ef - (1024u << 20);
    f.sign = hi & 0x80000000u;
    f.special = !f.zero && (ef - 0x00100000u) >= 0x7FE00000u;   // field 0 or 2047, not zero
    return f;
}

// RN(s * y) for the factor s split by split_factor; sets `special` when the integer path does
// not apply (the returned bits are then meaningless).
__device__ __forceinline__ double mul_rn_int(const SplitFactor& f, double y, bool& special)
{
    const uint32_t yh = (uint32_t)__double2hiint(y), yl = (uint32_t)__double2loint(y);
    const uint32_t ey = yh & 0x7FF00000u;
    // the implicit bit only for a nonzero exponent field: y = +-0 gives P = 0 (a subnormal y
    // gives garbage, flagged special below)
    const uint32_t y1 = (yh & 0x000FFFFFu) | min(ey, 0x00100000u);
    const bool yzero = (y1 | yl) == 0u;   // +-0 (a subnormal y keeps mantissa bits)
    // P = t3 2^64 + t2l 2^32 + t0l
    const uint64_t t0 = (uint64_t)yl * f.m0;
    const uint64_t t1 = (uint64_t)yl * f.m1 + (t0 >> 32);
    const uint64_t t2 = (uint64_t)y1 * f.m0 + t1;
    const uint64_t t3 = (uint64_t)y1 * f.m1 + (t2 >> 32);
    const uint32_t t2l = (uint32_t)t2, t0l = (uint32_t)t0;
    const uint32_t t3l = (uint32_t)t3, t3h = (uint32_t)(t3 >> 32);
    // H = P >> 42 (hhi:hlo), with every nonzero bit of P below 2^42 folded into H's bit 0:
    // H's bits 0..9 lie below the rounding position (bit 10 or 11), so only their being
    // nonzero matters
    const uint32_t hlo = __funnelshift_r(t2l, t3l, 10) | (((t2l & 0x3FFu) | t0l) != 0u ? 1u : 0u);
    const uint32_t hhi = __funnelshift_r(t3l, t3h, 10);
    const uint32_t big = hhi >> 31;                   // P >= 2^105: round at bit 11, else 10
    const uint32_t k = 10u + big;
    // Round to nearest even: add 2^(k-1) - 1 + bit_k(H) and drop k bits.  The dropped part
    // (with the sticky bit in bit 0) carries exactly when it exceeds half an ulp, or equals it
    // with an odd kept part.  P = 0 gives M = 0.
    const uint32_t half = 0x1FFu + (big << 9);        // 2^(k-1) - 1
    const uint64_t Hs = (((uint64_t)hhi << 32) | hlo) + (uint64_t)(half + ((hlo >> k) & 1u));
    const uint32_t slo = (uint32_t)Hs, shi = (uint32_t)(Hs >> 32);
    const uint32_t mlo = __funnelshift_r(slo, shi, k);
    const uint32_t mhi = shi >> k;
    // (E - 1) << 20, modulo 2^32; 0 for a zero factor, so that the result is the signed zero
    const bool zero = f.zero || yzero;
    const uint32_t ef = zero ? 0u : ey + f.eadj + (big << 20);
    // special: a result exponent out of [1, 2046] (the unsigned compare catches E - 1 < 0 as
    // well), or y subnormal, infinite or NaN (field 0 with mantissa bits, or 2047)
    special = special || (ef > (2045u << 20)) || (!yzero && (ey - 0x00100000u) >= 0x7FE00000u);
    const uint32_t rh = ef + mhi + ((yh & 0x80000000u) ^ f.sign);
    return __hiloint2double((int)rh, (int)mlo);
}

// The fall-back of the integer products: both products of a rotation on the FP64 pipe, as an
// out-of-line call.  Written inline, the compiler evaluates the two FMAs for every lane and
// selects (or the assembler predicates them), so they would issue on every rotation and the
// FP64 pipe would carry four instructions per rotation-row again (measured: same FP64
// instruction count as the FP64-pipe form).  A call is a branch that neither can flatten, so
// the FMAs issue only in a warp where some lane needs them.
static __device__ __noinline__ double2 fma_pair_call(double s, double y, double x, double nz)
{
    return make_double2(__fma_rn(s, y, nz), __fma_rn(s, x, nz));
}

}  // namespace symeig
