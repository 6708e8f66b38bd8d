// Device-side building blocks shared by every HyperFlow-GB300 kernel.
//
// Arithmetic parity: all kernels are compiled with --fmad=false, so a*b+c stays a
// rounded multiply followed by a rounded add, exactly as the reference's C++ (ISO
// mode, no contraction) evaluates it.  Divisions and square roots are correctly rounded
// (div_rn / sqrt_rn of hf_intdiv.cuh compute them on the integer pipes, bit-identical to
// the IEEE operations of the hardware and of libm).  Every expression below keeps the
// reference's operand order; identical sub-expressions the reference evaluates more
// than once (cons_to_prim inside cons_flux_x, prim_total_energy inside calc_U_k, ...)
// are evaluated once and reused, which changes no result because they are
// deterministic functions of the same inputs.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "hf_ctrl.h"
#include "hf_intdiv.cuh"

namespace hf {

__device__ __forceinline__ void raise_error(Ctrl* c, int code) { atomicCAS(&c->err, 0, code); }

// Checked builds (-DHF_CHECKS): a global-memory index outside its buffer sets the error word
// (HF_DEV_BOUNDS, reported by the next synchronising call) and the caller skips the access --
// no trap, no assert.  In normal builds the check compiles to `true`.
#ifdef HF_CHECKS
__device__ __forceinline__ bool hf_in(long long i, long long n, int* err) {
    if (i >= 0 && i < n) return true;
    atomicCAS(err, 0, (int)HF_DEV_BOUNDS);
    return false;
}
#else
__device__ __forceinline__ bool hf_in(long long, long long, int*) { return true; }
#endif

// ------------------------------------------------------------------------------
// std::min / std::max exactly (NaN-order semantics of the C++ library)
// ------------------------------------------------------------------------------
HF_HD double smin(double a, double b) { return lt(b, a) ? b : a; }
HF_HD double smax(double a, double b) { return lt(a, b) ? b : a; }
HF_HD double sgn(double v) { return (double)((v > 0.0) - (v < 0.0)); }

// ------------------------------------------------------------------------------
// ideal-gas model, src/fvm_2d_cart/model/euler_ideal_gas/euler_ideal_gas.cpp
// ------------------------------------------------------------------------------
struct Prim {
    double r, u, v, p;   // cons_to_prim (76-92)
    double q;            // u*u + v*v, shared by cons_to_prim and prim_total_energy
    double Et;           // prim_total_energy (40-46), recomputed from the primitives
};

// the primitives without the total energy (Et left unset)
HF_HD Prim to_prim_noE(double g1, double r, double ru, double rv, double E) {
    Prim w;
    w.r = r;
    w.u = div_rn(ru, r);
    w.v = div_rn(rv, r);
    w.q = w.u * w.u + w.v * w.v;
    w.p = g1 * (E - half(r) * w.q);
    return w;
}

// prim_total_energy (40-46) of the primitives, with prim_internal_energy (32-36)
HF_HD double prim_energy(double g1, const Prim& w) {
    double e = div_rn(w.p, w.r * g1);
    return w.r * (half(w.q) + e);
}

HF_HD Prim to_prim(double g1, double r, double ru, double rv, double E) {
    Prim w = to_prim_noE(g1, r, ru, rv, E);
    w.Et = prim_energy(g1, w);
    return w;
}

// only the primitives (no energy): what TimeStep needs
HF_HD void to_prim_short(double g1, double r, double ru, double rv, double E,
                                              double& u, double& v, double& p) {
    u = div_rn(ru, r);
    v = div_rn(rv, r);
    p = g1 * (E - half(r) * (u * u + v * v));
}

// prim_speed_of_sound (60-64)
HF_HD double sound(double g, double r, double p) { return sqrt_rn(div_rn(g * p, r)); }

// cons_flux_x / cons_flux_y (113-149): rho*u*u == (rho*u)*u etc.
template <int DIR>
HF_HD void flux(const Prim& w, double* f) {
    if (DIR == 0) {
        double ru = w.r * w.u;
        f[0] = ru;
        f[1] = ru * w.u + w.p;
        f[2] = ru * w.v;
        f[3] = w.u * (w.Et + w.p);
    } else {
        f[0] = w.r * w.v;
        f[1] = w.r * w.u * w.v;
        f[2] = f[0] * w.v + w.p;
        f[3] = w.v * (w.Et + w.p);
    }
}

// ------------------------------------------------------------------------------
// HLLC, src/fvm_2d_cart/scheme/riemann/riemann_hllc/riemann_hllc.cpp:169-212
// U*: calc_U_k (37-63); S*: calc_S_star (67-97); F*: calc_F_star (153-164).
// Only the flux the branch returns is formed; the others would be discarded.
// Returns 1 when the "should not get here" branch yields the zero flux.
// ------------------------------------------------------------------------------
template <int DIR>
HF_HD void star_flux(const double* UK, const Prim& wK, double SK, double Ss,
                                          const double* FK, double* F) {
    double velK = DIR == 0 ? wK.u : wK.v;
    double coef = wK.r * div_rn(SK - velK, SK - Ss);
    double us[4];
    us[0] = coef;
    if (DIR == 0) {
        us[1] = coef * Ss;
        us[2] = coef * wK.v;
    } else {
        us[1] = coef * wK.u;
        us[2] = coef * Ss;
    }
    us[3] = coef * (div_rn(wK.Et, wK.r) + (Ss - velK) * (Ss + div_rn(wK.p, wK.r * (SK - velK))));
#pragma unroll
    for (int i = 0; i < 4; ++i) F[i] = FK[i] + SK * (us[i] - UK[i]);
}

// The branches of riemann_hllc.cpp:179-211 in the reference's order.  After the supersonic-left
// test every branch uses one side only, so that side's state, flux and wave speed are selected
// first and one flux / one star state is formed: a warp whose faces take different branches
// runs the star-state arithmetic once, not once per branch.  LAZY forms the side's flux from its
// primitives (the MUSCL-Hancock and unstructured faces) and its total energy, which nothing else
// uses, for the selected side only (wL.Et / wR.Et are not read), after the branches have joined,
// so a warp whose faces take different branches forms one energy and one flux per face;
// otherwise FL / FR and the energies are given.
template <int DIR, bool LAZY>
HF_HD int hllc_sel(double g1, const double* UL, const Prim& wL, double aL, const double* FL,
                   const double* UR, const Prim& wR, double aR, const double* FR, double* F) {
    double velL = DIR == 0 ? wL.u : wL.v;
    double velR = DIR == 0 ? wR.u : wR.v;
    double SL = smin(velL - aL, velR - aR);
    double SR = smax(velL + aL, velR + aR);
    bool left = true, star = false;   // the side whose state and flux the result uses; star region?
    double Ss = 0.0;
    if (!ge0(SL)) {
        double num = wR.p - wL.p + wL.r * velL * (SL - velL) - wR.r * velR * (SR - velR);
        double den = wL.r * (SL - velL) - wR.r * (SR - velR);
        Ss = div_rn(num, den);
        const bool star_l = le0(SL) && ge0(Ss);
        const bool star_r = !star_l && le0(Ss) && ge0(SR);
        const bool right = !star_l && !star_r && le0(SR);
        if (!(star_l || star_r || right)) {
#pragma unroll
            for (int i = 0; i < 4; ++i) F[i] = 0.0;
            return 1;
        }
        left = star_l;
        star = !right;
    }
    Prim w;
    w.r = left ? wL.r : wR.r;
    w.u = left ? wL.u : wR.u;
    w.v = left ? wL.v : wR.v;
    w.p = left ? wL.p : wR.p;
    w.q = left ? wL.q : wR.q;
    w.Et = LAZY ? prim_energy(g1, w) : (left ? wL.Et : wR.Et);
    double FK[4];
    if (LAZY) {
        flux<DIR>(w, FK);
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i) FK[i] = left ? FL[i] : FR[i];
    }
    if (!star) {   // supersonic left (riemann_hllc.cpp:179-181) or right (203-205)
#pragma unroll
        for (int i = 0; i < 4; ++i) F[i] = FK[i];
        return 0;
    }
    double UK[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) UK[i] = left ? UL[i] : UR[i];
    star_flux<DIR>(UK, w, left ? SL : SR, Ss, FK, F);
    return 0;
}

template <int DIR>
HF_HD int hllc(const double* UL, const Prim& wL, double aL, const double* FL,
               const double* UR, const Prim& wR, double aR, const double* FR, double* F) {
    return hllc_sel<DIR, false>(0.0, UL, wL, aL, FL, UR, wR, aR, FR, F);
}

// HLLC from two conservative states (computes primitives, sound speeds, the used flux)
template <int DIR>
HF_HD int hllc_cons(double g, double g1, const double* UL, const double* UR,
                                         double* F) {
    Prim wL = to_prim_noE(g1, UL[0], UL[1], UL[2], UL[3]);
    Prim wR = to_prim_noE(g1, UR[0], UR[1], UR[2], UR[3]);
    // calc_wave_speeds_direct_min_max (127-150): sqrt(gamma * p / rho)
    double aL = sound(g, wL.r, wL.p);
    double aR = sound(g, wR.r, wR.p);
    return hllc_sel<DIR, true>(g1, UL, wL, aL, nullptr, UR, wR, aR, nullptr, F);
}

// ------------------------------------------------------------------------------
// slope limiters, src/fvm_2d_cart/scheme/limiter (omega 0, beta 1, tol 1e-6 from
// parser.cpp:230-233) and the limited slope of muscl_hancock.cpp:67-206
// ------------------------------------------------------------------------------
constexpr double kTol = 1e-6;

HF_HD double xi_right(double r) {
    // Limiter::xi_right + denom_tol (limiter.cpp:26-53): 2*beta / (1 - omega + (1 + omega) r)
    double den = 1.0 + r;   // (1.0 - 0.0) + (1.0 + 0.0) * r rounds to the same value
    if ((f64_bits(den) & kAbs) < f64_bits(kTol)) den = (den == 0.0) ? kTol : kTol * sgn(den);
    return div_rn(2.0, den);
}

template <int LIM>
HF_HD double limiter(double r) {
    if (LIM == 0) {   // MinBeeLimiter::operator() minbee.cpp:29-38
        if (le0(r)) return 0.0;
        // here r > 0 or NaN; (0 < r && r <= 1) is the unsigned bit compare with 1.0
        if (f64_bits(r) <= 0x3FF0000000000000ull) return r;
        // r > 1: 1 + r > 2, so denom_tol leaves it and 2/(1+r) <= 1 = min(1, 2/(1+r));
        // r NaN: min(1.0, NaN) is 1.0
        return is_nan(r) ? 1.0 : div_rn(2.0, 1.0 + r);
    } else {          // VanLeerLimiter::operator() vanleer.cpp:29-36
        if (le0(r)) return 0.0;
        // min(2r/(1+r), 2/(1+r)) for a finite r > 0: 1 + r > 1 keeps denom_tol out of xi_right,
        // and correct rounding is monotone, so the minimum is the first quotient when r <= 1 and
        // the second when r > 1 -- one division instead of two, the same bits.  NaN and +inf
        // take the reference's expression (2r/(1+r) is NaN there, and so is the minimum).
        const uint64_t rb = f64_bits(r);
        if (rb >= 0x7FF0000000000000ull) return smin(div_rn(2.0 * r, 1.0 + r), xi_right(r));
        return rb <= 0x3FF0000000000000ull ? div_rn(2.0 * r, 1.0 + r) : div_rn(2.0, 1.0 + r);
    }
}

// The difference clamp of calculate_slope_limiters (muscl_hancock.cpp:78-84): |d| <= tol gives
// tol for d = +-0 and tol * sgn(d) otherwise, i.e. tol with d's sign (NaN fails |d| <= tol).  On
// the bit pattern: the FP64 compares, the conversion and the multiplication of the literal form
// would all run on the FP64 pipe, and the clamp fires in every uniform region.
HF_HD double clamp_tol(double d) {
    const uint64_t b = f64_bits(d);
    if ((b & kAbs) > f64_bits(kTol)) return d;
    if ((b & kAbs) == 0) return kTol;
    return f64_from(f64_bits(kTol) | (b & ~kAbs));
}

// limited slope of one variable from the three cell averages (um, u0, up)
template <int LIM>
HF_HD double slope(double um, double u0, double up) {
    double dl = u0 - um, dr = up - u0;
    double xi = limiter<LIM>(div_rn(clamp_tol(dl), clamp_tol(dr)));
    return xi * (half(dl) + half(dr));
}

// ------------------------------------------------------------------------------
// TimeStep pieces (timestep.cpp:29-68)
// ------------------------------------------------------------------------------
// Per-cell wave-speed terms s_x = |u| + c and s_y = |v| + c.  The reference folds
// dx / s over cells with std::min; fl(dx / s) is non-increasing in s, so that fold
// equals fl(dx / max s) -- a max over s, which is exact in any order.  NaN terms are
// skipped in both.
HF_HD bool wave_terms(double g, double g1, double r, double ru, double rv,
                                           double E, double& sx, double& sy) {
    double u, v, p;
    to_prim_short(g1, r, ru, rv, E, u, v, p);
    double c = sound(g, r, p);
    sx = fabs(u) + c;
    sy = fabs(v) + c;
    return gt0(r) && gt0(p);   // the state is physical: density and pressure positive, not NaN
}

// NaN-skipping max of non-negative values
HF_HD double nmax(double m, double s) {
    // s > m for m >= +0 (never NaN): the unsigned bit order, NaN excluded
    const uint64_t us = f64_bits(s);
    return (us <= kInf && us > f64_bits(m)) ? s : m;
}

__device__ __forceinline__ unsigned long long dbits(double x) {
    return (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ double bitsd(unsigned long long x) {
    return __longlong_as_double((long long)x);
}

// dt of TimeStep call number `call` (0-based) over all blocks; blocks < new_upto take
// their interior maximum from parity `pn` (already advanced this step), the others
// from parity `po`.  CP: const Ctrl*, or const volatile Ctrl* to read values other CTAs of the
// same launch wrote (past the L1 cache).
template <class CP>
__device__ __forceinline__ double cfl_dt_t(CP c, long long call, int new_upto, int po, int pn) {
    double dtx = 1e16, dty = 1e16;
    const int nb = c->nblocks;
    for (int b = 0; b < nb; ++b) {
        int pp = b < new_upto ? pn : po;
        double mx = smax(bitsd(c->ghost_s[b][0]), bitsd(c->int_s[pp][b][0]));
        double my = smax(bitsd(c->ghost_s[b][1]), bitsd(c->int_s[pp][b][1]));
        dtx = smin(dtx, div_rn(c->dx[b], mx));   // exact, on the integer pipes
        dty = smin(dty, div_rn(c->dy[b], my));
    }
    const double cfl = c->cfl;
    double final_cfl = (call + 1 <= 10) ? 0.2 * cfl : cfl;
    return final_cfl * smin(dtx, dty);
}
__device__ __forceinline__ double cfl_dt(const Ctrl* c, long long call, int new_upto, int po, int pn) {
    return cfl_dt_t<const Ctrl*>(c, call, new_upto, po, pn);
}
__device__ __forceinline__ double cfl_dt_fresh(const Ctrl* c, long long call, int new_upto, int po, int pn) {
    return cfl_dt_t<const volatile Ctrl*>(c, call, new_upto, po, pn);
}

// block-wide max of two values, one atomicMax per CTA
template <int NT>
__device__ __forceinline__ void block_max2_atomic(double sx, double sy, unsigned long long* ax,
                                                  unsigned long long* ay) {
    __shared__ double red[2][NT / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sx = nmax(sx, __shfl_xor_sync(0xffffffffu, sx, o));
        sy = nmax(sy, __shfl_xor_sync(0xffffffffu, sy, o));
    }
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { red[0][w] = sx; red[1][w] = sy; }
    __syncthreads();
    if (w == 0) {
        sx = l < NT / 32 ? red[0][l] : 0.0;
        sy = l < NT / 32 ? red[1][l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sx = nmax(sx, __shfl_xor_sync(0xffffffffu, sx, o));
            sy = nmax(sy, __shfl_xor_sync(0xffffffffu, sy, o));
        }
        if (l == 0) {
            if (sx > 0.0) atomicMax(ax, dbits(sx));
            if (sy > 0.0) atomicMax(ay, dbits(sy));
        }
    }
}

// ------------------------------------------------------------------------------
// TMA + mbarrier (inline PTX, sm_90+ forms valid on sm_103a)
// ------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait: gives up after `limit` polls (each poll itself suspends for a
// hardware-chosen interval) and reports failure instead of hanging the GPU
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x,
                                            int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace hf
