// Correctly rounded FP64 division on the integer pipes.
//
// GB300 issues FP64 at 2 lanes per SM per clock -- 1/32 of its integer rate -- and an IEEE
// FP64 division built from FP64 Newton steps costs about ten FP64 instructions.  This
// routine computes the same correctly rounded quotient (round to nearest, ties to even)
// with integer multiplies instead, by the classical scheme of a Newton-Raphson refined
// fixed-point reciprocal, a quotient by multiplication, and an exact remainder that both
// corrects the quotient and decides the rounding (see Muller et al., "Handbook of
// Floating-Point Arithmetic", the chapter on division; Moller & Granlund, "Improved division
// by invariant integers", IEEE TC 2011, for the fixed-point reciprocal arithmetic):
//
//   a = ma 2^ea, b = mb 2^eb, ma, mb in [2^52, 2^53) (ma doubled when ma < mb, so that the
//   quotient mantissa lies in [1, 2));
//   X ~ 2^116 / mb: an FP32 reciprocal of mb's top 24 bits (about 23 correct bits), then two
//   Newton steps X += X (2^116 - mb X) / 2^116 in 64-bit fixed point (about 62 bits);
//   Q ~ floor(ma X / 2^64) = floor(ma 2^52 / mb) to within a few units; the exact remainder
//   R = ma 2^52 - Q mb (small, so exact modulo 2^64) moves Q to the true floor; 2R against
//   mb rounds it to nearest even.
//
// Every operand outside this fast path -- zero, subnormal, infinite or NaN divisor; a
// subnormal, infinite or NaN dividend; a quotient whose exponent leaves the normal range --
// goes to the hardware division, so the result equals `a / b` bit for bit for all inputs.
// A zero dividend over a normal divisor gives the correctly signed zero directly.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

// The arithmetic helpers compile for the device and for the host (the host build lets the
// CPU test suite run the exact kernel arithmetic against the oracle without a GPU).
#define HF_HD __host__ __device__ __forceinline__

namespace hf {

HF_HD uint64_t f64_bits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
#endif
}
HF_HD double f64_from(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x;
    std::memcpy(&x, &u, 8);
    return x;
#endif
}
HF_HD uint32_t f32_bits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return u;
#endif
}
HF_HD uint64_t umulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}
HF_HD float f32_from(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    std::memcpy(&x, &u, 4);
    return x;
#endif
}
// FP32 seeds of the Newton iterations: approximate reciprocal and reciprocal square root
// (one special-function instruction each on the device).  The iterations converge from any
// seed within a few ulp, so the host build perturbs the exact value by up to +-4 ulp to
// exercise that margin.
HF_HD float rcp_f32(float x) {
#ifdef __CUDA_ARCH__
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    volatile float one = 1.0f;
    const uint32_t b = f32_bits(one / x);
    return f32_from(b + ((b * 2654435761u) >> 29) - 4u);
#endif
}
HF_HD float rsqrt_f32(float x) {
#ifdef __CUDA_ARCH__
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    volatile float one = 1.0f;
    const uint32_t b = f32_bits(one / std::sqrt(x));
    return f32_from(b + ((b * 2654435761u) >> 29) - 4u);
#endif
}
// an integer in [2^23, 2^24) as an FP32 value, from its bits (no conversion instruction)
HF_HD float u24_float(uint32_t m) { return f32_from(0x4B000000u | (m & 0x7FFFFFu)); }
// an integer in [2^22, 2^24) as an FP32 value
HF_HD float u22_24_float(uint32_t m) {
    return (m >> 23) ? f32_from(0x4B000000u | (m & 0x7FFFFFu)) : f32_from(0x4A800000u | ((m << 1) & 0x7FFFFFu));
}
// IEEE comparisons on the integer pipes (NaN compares false, -0 equals +0).  A double's
// sign-magnitude bits map to an order-preserving signed key: key = sign ? -|x| : |x|.
constexpr uint64_t kAbs = 0x7FFFFFFFFFFFFFFFull, kInf = 0x7FF0000000000000ull;
HF_HD bool is_nan(double x) { return (f64_bits(x) & kAbs) > kInf; }
HF_HD int64_t order_key(double x) {
    const uint64_t u = f64_bits(x);
    const int64_t m = (int64_t)(u & kAbs);
    return (u >> 63) ? -m : m;
}
HF_HD bool lt(double a, double b) { return !is_nan(a) && !is_nan(b) && order_key(a) < order_key(b); }
HF_HD bool le0(double x) {            // x <= 0.0
    const uint64_t u = f64_bits(x), m = u & kAbs;
    return m == 0 || ((u >> 63) && m <= kInf);
}
HF_HD bool ge0(double x) {            // 0.0 <= x
    const uint64_t u = f64_bits(x), m = u & kAbs;
    return m == 0 || (!(u >> 63) && m <= kInf);
}
HF_HD bool gt0(double x) {            // 0.0 < x: sign clear, not zero, not NaN
    const uint64_t u = f64_bits(x);
    return u != 0 && u <= kInf;
}
// |x| <= t for a positive finite t (false for NaN)
HF_HD bool abs_le(double x, double t) { return (f64_bits(x) & kAbs) <= f64_bits(t); }

// 0.5 * x, equal to the FP64 multiplication for every x, on the integer pipe and without a
// branch: a normal x above the lowest binade has its exponent lowered by one (exact); for
// zeros, subnormals and the lowest normal binade the 53-bit significand-with-exponent-bit
// field is shifted right by one with round to nearest even (a carry into the exponent field
// gives the smallest normal, as the multiplication does); infinities and NaN are returned as
// they are.
HF_HD double half(double x) {
    const uint64_t u = f64_bits(x);
    const uint64_t sgn = u & 0x8000000000000000ull, a = u & 0x7FFFFFFFFFFFFFFFull;
    const uint32_t e = (uint32_t)(a >> 52);
    const uint64_t low = sgn | ((a >> 1) + (a & (a >> 1) & 1ull));   // e <= 1
    const uint64_t r = (e - 2u < 0x7FDu) ? u - (1ull << 52) : (e <= 1u ? low : u);
    return f64_from(r);
}

HF_HD double hw_div(double a, double b) { return a / b; }
HF_HD double hw_sqrt(double x) { return std::sqrt(x); }

// Fixed-point reciprocal X ~ 2^116 / mb of a divisor mantissa mb in (2^52, 2^53) (not a
// power of two): an FP32 seed of mb's top 24 bits, then two Newton steps.
HF_HD uint64_t recip_fixed(uint64_t mb) {
    // FP32 seed: X0 = 2^87 / dh with dh = mb >> 29 in [2^23, 2^24)
    const uint32_t dh = (uint32_t)(mb >> 29);
    const float r = rcp_f32(u24_float(dh));
    const uint32_t rb = f32_bits(r);
    const uint64_t mr = (uint64_t)((rb & 0x7FFFFFu) | 0x800000u);
    const int sh = (int)((rb >> 23) & 0xFFu) - 63;   // r = mr 2^(E-150); X0 = mr 2^(E-63)
    uint64_t X = sh >= 41 ? 0xFFFFFFFFFFFFFFFFull : (mr << sh);
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        // E = 2^116 - mb X as a signed 128-bit value (small); C = X E / 2^116
        const uint64_t plo = mb * X, phi = umulhi64(mb, X);
        const uint64_t elo = 0ull - plo;
        const uint64_t ehi = (1ull << 52) - phi - (plo != 0 ? 1ull : 0ull);
        const int64_t e52 = (int64_t)((ehi << 12) | (elo >> 52));     // E >> 52
        const uint64_t mag = e52 < 0 ? (uint64_t)(-e52) : (uint64_t)e52;
        const uint64_t c = umulhi64(X, mag);
        X = e52 < 0 ? X - c : X + c;
    }
    return X;
}

// The quotient of the fast path: a, b as in div_rn with `fast` true and a nonzero; X the
// reciprocal of b's mantissa (unused when b is a power of two).
HF_HD double quot_fast(uint64_t A, uint64_t B, uint64_t X) {
    const uint32_t ea = (uint32_t)(A >> 52) & 0x7FFu, eb = (uint32_t)(B >> 52) & 0x7FFu;
    const uint64_t sign = (A ^ B) & 0x8000000000000000ull;
    const uint64_t M52 = 0x000FFFFFFFFFFFFFull, H52 = 0x0010000000000000ull;
    int e = (int)ea - (int)eb + 1023;
    uint64_t ma = (A & M52) | H52;
    const uint64_t mb = (B & M52) | H52;
    const bool shift = ma < mb;
    e -= shift ? 1 : 0;
    if (shift) ma <<= 1;                       // ma / mb in [1, 2)
    uint64_t Q, R;
    if ((B & M52) == 0) {                      // divisor a power of two: exact
        Q = ma;                                // ma in [2^52, 2^53): no shift happened
        R = 0;
    } else {
        Q = umulhi64(ma, X);
        int64_t Rs = (int64_t)((ma << 52) - Q * mb);   // exact: |R| < 2^55
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (Rs < 0) { Q -= 1; Rs += (int64_t)mb; }
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (Rs >= (int64_t)mb) { Q += 1; Rs -= (int64_t)mb; }
        R = (uint64_t)Rs;
    }
    // round to nearest, ties to even
    const uint64_t r2 = R << 1;
    if (r2 > mb || (r2 == mb && (Q & 1ull))) Q += 1;
    if (Q == (H52 << 1)) { Q = H52; e += 1; }
    return f64_from(sign | ((uint64_t)e << 52) | (Q & M52));
}

// true when a / b takes the integer path: b normal, and a zero, or a normal with a normal
// quotient exponent
HF_HD bool div_fast(uint64_t A, uint64_t B) {
    const uint32_t ea = (uint32_t)(A >> 52) & 0x7FFu, eb = (uint32_t)(B >> 52) & 0x7FFu;
    const uint64_t M52 = 0x000FFFFFFFFFFFFFull, H52 = 0x0010000000000000ull;
    const bool a_zero = (A << 1) == 0;
    int e = (int)ea - (int)eb + 1023;
    e -= (((A & M52) | H52) < ((B & M52) | H52)) ? 1 : 0;
    return (eb - 1u < 2046u) && (a_zero || ((ea - 1u < 2046u) && e >= 1 && e <= 2045));
}

// Kept out of line: the stencils call it about 55 times per cell, and one shared copy keeps the
// kernels inside the instruction cache (measured faster than inlining every call).
static __host__ __device__ __noinline__ double div_rn(double a, double b) {
    const uint64_t A = f64_bits(a), B = f64_bits(b);
    if (!div_fast(A, B)) return hw_div(a, b);
    if ((A << 1) == 0) return f64_from((A ^ B) & 0x8000000000000000ull);
    const uint64_t M52 = 0x000FFFFFFFFFFFFFull, H52 = 0x0010000000000000ull;
    const uint64_t X = (B & M52) == 0 ? 0ull : recip_fixed((B & M52) | H52);
    return quot_fast(A, B, X);
}

}  // namespace hf

namespace hf {

// Correctly rounded FP64 square root on the integer pipes, by the same scheme: x = m 2^E
// (m doubled when E is odd so the exponent halves exactly), Y ~ 2^90 / sqrt(m) from an FP32
// reciprocal square root refined by two Newton steps Y += Y (2^180 - m Y^2) / 2^181 in
// fixed point, S ~ m Y / 2^64 = floor(sqrt(m 2^52)) corrected with the exact remainder
// R = m 2^52 - S^2, and rounded up when R > S (a square root is never a halfway case).
// Zero, negative, subnormal, infinite and NaN arguments go to the hardware sqrt.
// out of line, as div_rn
static __host__ __device__ __noinline__ double sqrt_rn(double x) {
    const uint64_t X = f64_bits(x);
    const uint32_t ex = (uint32_t)(X >> 52) & 0x7FFu;
    if ((X >> 63) != 0 || ex - 1u >= 2046u) return hw_sqrt(x);
    const uint64_t M52 = 0x000FFFFFFFFFFFFFull, H52 = 0x0010000000000000ull;
    const int E = (int)ex - 1023;
    uint64_t m = (X & M52) | H52;
    int Eh;
    if (E & 1) { m <<= 1; Eh = (E - 1) / 2; } else { Eh = E / 2; }   // m in [2^52, 2^54)
    uint64_t S;
    if (m == H52) {
        S = H52;                                   // x is an even power of two
    } else {
        const uint32_t mh = (uint32_t)(m >> 30);   // [2^22, 2^24), exact in FP32
        const float rs = rsqrt_f32(u22_24_float(mh));
        const uint32_t rb = f32_bits(rs);
        const uint64_t mr = (uint64_t)((rb & 0x7FFFFFu) | 0x800000u);
        const int sh = (int)((rb >> 23) & 0xFFu) - 75;        // Y0 = 2^75 rs = mr 2^(E_r - 75)
        uint64_t Y = sh >= 41 ? 0xFFFFFFFFFFFFFFFFull : (sh < 0 ? 0ull : (mr << sh));
#pragma unroll
        for (int it = 0; it < 2; ++it) {
            const uint64_t t = umulhi64(Y, Y);                    // ~ 2^116 / m
            const uint64_t plo = m * t, phi = umulhi64(m, t);
            const uint64_t elo = 0ull - plo;
            const uint64_t ehi = (1ull << 52) - phi - (plo != 0 ? 1ull : 0ull);
            const int64_t e52 = (int64_t)((ehi << 12) | (elo >> 52));   // (2^116 - m t) >> 52
            const uint64_t mag = e52 < 0 ? (uint64_t)(-e52) : (uint64_t)e52;
            const uint64_t c = umulhi64(Y, mag) >> 1;
            Y = e52 < 0 ? Y - c : Y + c;
        }
        S = umulhi64(m, Y);
        int64_t R = (int64_t)((m << 52) - S * S);                  // exact: |R| small
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (R < 0) { R += (int64_t)(2 * S - 1); S -= 1; }
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (R >= (int64_t)(2 * S + 1)) { R -= (int64_t)(2 * S + 1); S += 1; }
        if (R > (int64_t)S) S += 1;
    }
    int eo = Eh + 1023;
    if (S == (H52 << 1)) { S = H52; eo += 1; }
    return f64_from(((uint64_t)eo << 52) | (S & M52));
}

}  // namespace hf
