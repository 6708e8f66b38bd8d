// Learned coarse solver: an FP32 MUSCL-Hancock + HLLC step on a coarse grid plus a per-face
// flux correction predicted by a small MLP, trained on box-filtered fine-grid FP64 runs of
// the plain solver.  C ABI in include/hyperflow_gb300_learned.h.  No counterpart in the
// reference; the plain part follows the reference's MUSCL-Hancock step
// (src/fvm_2d_cart/scheme/muscl_hancock/muscl_hancock.cpp:41-376) in FP32 on one block with
// transmissive sides (ghost cells read as mirrored interior cells).
//
// Per face (x faces between cells (i,j),(i+1,j); y faces between (i,j),(i,j+1)):
//   features: a 4x4 window of cells -- 4 along the face normal (offsets -1..2 from the
//     lower cell) by 4 along the face (offsets -1..2) -- each as (rho/rho_ref - 1,
//     u_n/c_ref, u_t/c_ref, p/p_ref - 1) with rho_ref, p_ref the mean of the two face
//     cells and c_ref = sqrt(gamma p_ref / rho_ref): 64 inputs, rounded to BF16;
//   MLP: 64 -> 64 (GELU) -> 64 (GELU) -> 4, BF16 weights and activations on the tensor
//     cores (tcgen05.mma, BF16 x BF16 -> FP32 accumulators in TMEM), FP32 biases;
//   correction: dF = rho_ref c_ref * (o0, o1 c_ref, o2 c_ref, o3 c_ref^2) in the face frame
//     (normal, tangential), rotated back to (x, y);
//   guard: a cell whose corrected update has rho <= 0, p <= 0, or (mode 0) a density / energy
//     change beyond `bound` times the plain update's, or (mode 1) a density / energy outside the
//     min / max of its 3x3 neighbourhood's old and plainly updated values, rejects the
//     corrections on all its faces (they fall back to the plain flux); a cell still violating
//     after that takes its plain update.
// Training: one-step loss L = mean_cells sum_v w_v (U^{n+1}_v - T_v)^2 against the filtered
// fine solution T; dL/dF flows only through the linear conservative update.  The backward runs
// its products on the tensor cores (weight gradients accumulated in TMEM), Adam on the CUDA
// cores.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/hyperflow_gb300_learned.h"
#include "hf_device.cuh"
#include "hf_trace.h"

namespace hf {
namespace lc {

constexpr int H = 64;          // hidden width
constexpr int NIN = 64;        // inputs
constexpr int NOUT = 4;
// packed parameter layout (floats): W1[64][64] b1[64] W2[64][64] b2[64] W3[4][64] b3[4]
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * NIN, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H,
              OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + NOUT * H, NPARAM = OFF_B3 + NOUT;

// the hardware's approximate tanh (one MUFU instruction, absolute error about 2^-11): GELU's
// epilogue cost, which bounds the MLP kernels, falls by half against the accurate tanhf
__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// GELU, tanh form: 0.5 z (1 + tanh(k (z + 0.044715 z^3))), k = sqrt(2/pi), formed as h + h t with
// h = z / 2 and t = tanh(z (k + 0.044715 k z^2)) -- half of what the MLP kernels' packed gelu2x
// computes, exactly, so the backward's recomputed activations equal the forward's -- and its
// derivative 0.5 (1 + t) + 0.5 z (1 - t^2) k (1 + 3 0.044715 z^2) from the same tanh
__device__ __forceinline__ void gelu_both(float z, float& h, float& g) {
    const float k = 0.7978845608028654f, c = 0.7978845608028654f * 0.044715f;
    const float z2 = z * z;
    const float t = tanh_fast(z * fmaf(z2, c, k));
    const float hz = z * 0.5f;
    h = fmaf(hz, t, hz);
    g = fmaf(hz * fmaf(-t, t, 1.0f), fmaf(3.0f * c, z2, k), fmaf(0.5f, t, 0.5f));
}

__device__ __forceinline__ int mir(int x, int n) {
    x = x < 0 ? -1 - x : (x >= n ? 2 * n - 1 - x : x);
    return x < 0 ? 0 : (x >= n ? n - 1 : x);
}

// ---------------------------------------------------------------------------------
// FP32 model + HLLC + limiter (the reference's formulas, single precision)
// ---------------------------------------------------------------------------------
struct PrimF { float r, u, v, p, E; };
__device__ __forceinline__ PrimF prim(float g1, const float* c) {
    PrimF w;
    w.r = c[0];
    w.u = c[1] / c[0];
    w.v = c[2] / c[0];
    const float q = w.u * w.u + w.v * w.v;
    w.p = g1 * (c[3] - 0.5f * c[0] * q);
    w.E = w.r * (0.5f * q + w.p / (w.r * g1));
    return w;
}
template <int DIR>
__device__ __forceinline__ void fluxf(const PrimF& w, float* f) {
    if (DIR == 0) { float ru = w.r * w.u; f[0] = ru; f[1] = ru * w.u + w.p; f[2] = ru * w.v; f[3] = w.u * (w.E + w.p); }
    else { f[0] = w.r * w.v; f[1] = w.r * w.u * w.v; f[2] = f[0] * w.v + w.p; f[3] = w.v * (w.E + w.p); }
}
template <int DIR>
__device__ void hllcf(float g, float g1, const float* UL, const float* UR, float* F) {
    PrimF wL = prim(g1, UL), wR = prim(g1, UR);
    const float aL = sqrtf(g * wL.p / wL.r), aR = sqrtf(g * wR.p / wR.r);
    const float vL = DIR == 0 ? wL.u : wL.v, vR = DIR == 0 ? wR.u : wR.v;
    const float SL = fminf(vL - aL, vR - aR), SR = fmaxf(vL + aL, vR + aR);
    float FL[4], FR[4];
    fluxf<DIR>(wL, FL);
    fluxf<DIR>(wR, FR);
    if (0.0f <= SL) { for (int i = 0; i < 4; ++i) F[i] = FL[i]; return; }
    if (SR <= 0.0f) { for (int i = 0; i < 4; ++i) F[i] = FR[i]; return; }
    const float Ss = (wR.p - wL.p + wL.r * vL * (SL - vL) - wR.r * vR * (SR - vR)) /
                     (wL.r * (SL - vL) - wR.r * (SR - vR));
    const bool left = 0.0f <= Ss;
    const PrimF& w = left ? wL : wR;
    const float SK = left ? SL : SR, vK = left ? vL : vR;
    const float* UK = left ? UL : UR;
    const float* FK = left ? FL : FR;
    const float coef = w.r * ((SK - vK) / (SK - Ss));
    float us[4];
    us[0] = coef;
    us[1] = DIR == 0 ? coef * Ss : coef * w.u;
    us[2] = DIR == 0 ? coef * w.v : coef * Ss;
    us[3] = coef * (w.E / w.r + (Ss - vK) * (Ss + w.p / (w.r * (SK - vK))));
    for (int i = 0; i < 4; ++i) F[i] = FK[i] + SK * (us[i] - UK[i]);
}
__device__ __forceinline__ float limf(int lim, float r) {
    if (r <= 0.0f) return 0.0f;
    const float xr = 2.0f / (1.0f + r);
    if (lim == 0) return r <= 1.0f ? r : fminf(1.0f, xr);
    return fminf(2.0f * r / (1.0f + r), xr);
}
__device__ __forceinline__ float slopef(int lim, float um, float u0, float up) {
    float dl = u0 - um, dr = up - u0;
    float dlc = fabsf(dl) <= 1e-6f ? (dl == 0.0f ? 1e-6f : copysignf(1e-6f, dl)) : dl;
    float drc = fabsf(dr) <= 1e-6f ? (dr == 0.0f ? 1e-6f : copysignf(1e-6f, dr)) : dr;
    return limf(lim, dlc / drc) * (0.5f * dl + 0.5f * dr);
}

struct Grid {
    int n;
    float dx, g, g1;
    int lim;
};

__device__ __forceinline__ void load_cell(const float* __restrict__ U, int n, int i, int j, float* c) {
    const size_t o = (size_t)mir(j, n) * n + mir(i, n), pl = (size_t)n * n;
    c[0] = U[o]; c[1] = U[pl + o]; c[2] = U[2 * pl + o]; c[3] = U[3 * pl + o];
}

// evolved face pair of cell (i, j) in direction DIR: e0 (lower face), e1 (upper face)
template <int DIR>
__device__ void evolved_pair(const float* __restrict__ U, const Grid& G, float hdt_dx, int i, int j,
                             float* e0, float* e1) {
    float cm[4], c0[4], cp[4];
    load_cell(U, G.n, i - (DIR == 0), j - (DIR == 1), cm);
    load_cell(U, G.n, i, j, c0);
    load_cell(U, G.n, i + (DIR == 0), j + (DIR == 1), cp);
    for (int v = 0; v < 4; ++v) {
        const float s = slopef(G.lim, cm[v], c0[v], cp[v]);
        e0[v] = c0[v] - 0.5f * s;
        e1[v] = c0[v] + 0.5f * s;
    }
    PrimF w0 = prim(G.g1, e0), w1 = prim(G.g1, e1);
    float f0[4], f1[4];
    fluxf<DIR>(w0, f0);
    fluxf<DIR>(w1, f1);
    for (int v = 0; v < 4; ++v) {
        const float d = hdt_dx * (f0[v] - f1[v]);
        e0[v] += d;
        e1[v] += d;
    }
}

// face index f: x faces first (f = j*(n+1) + i, face between cells i-1 and i, i in 0..n),
// then y faces (f = NX + j*n + i, between cells (i, j-1) and (i, j), j in 0..n)
__device__ __forceinline__ void face_of(int f, int n, int& dir, int& i, int& j) {
    const int nxf = (n + 1) * n;
    if (f < nxf) { dir = 0; j = f / (n + 1); i = f % (n + 1); }
    else { f -= nxf; dir = 1; j = f / n; i = f % n; }
}

// plain MUSCL-Hancock HLLC flux of face f (FP32); hdt = dt / (2 dx)
__device__ __forceinline__ void plain_face_flux(const float* __restrict__ U, const Grid& G, float hdt, int f,
                                                float* out) {
    int dir, i, j;
    face_of(f, G.n, dir, i, j);
    float a0[4], a1[4], b0[4], b1[4];
    if (dir == 0) {
        evolved_pair<0>(U, G, hdt, i - 1, j, a0, a1);
        evolved_pair<0>(U, G, hdt, i, j, b0, b1);
        hllcf<0>(G.g, G.g1, a1, b0, out);
    } else {
        evolved_pair<1>(U, G, hdt, i, j - 1, a0, a1);
        evolved_pair<1>(U, G, hdt, i, j, b0, b1);
        hllcf<1>(G.g, G.g1, a1, b0, out);
    }
}

// plain MUSCL-Hancock HLLC flux of every face (FP32)
__global__ void plain_flux_kernel(const float* __restrict__ U, Grid G, float dt, float* __restrict__ F) {
    const int nf = 2 * (G.n + 1) * G.n;
    const float hdt = 0.5f * dt / G.dx;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        float out[4];
        plain_face_flux(U, G, hdt, f, out);
        for (int v = 0; v < 4; ++v) F[(size_t)v * nf + f] = out[v];
    }
}

// primitives of every cell, formed once: each is shared by the stencils of up to 16 faces
__global__ void prims_kernel(const float* __restrict__ U, int n, float g1, float4* __restrict__ W) {
    const size_t pl = (size_t)n * n;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < pl; k += (size_t)gridDim.x * blockDim.x) {
        const float c[4] = {U[k], U[pl + k], U[2 * pl + k], U[3 * pl + k]};
        const PrimF w = prim(g1, c);
        W[k] = make_float4(w.r, w.u, w.v, w.p);
    }
}

constexpr int kFeatNT = 256;

// two FP32 values rounded to BF16 (lo in the low half)
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// the 64 features of face (dir, i, j) (face_of's indices), rounded to BF16 and packed in pairs
// (normal offset outer, tangential offset inner; per cell rho, u_n, u_t, p), and its correction
// scale (rho_ref, c_ref).  The scaled values are products with the reciprocals of rho_ref, c_ref and
// p_ref (one division each per face), and the stencil's mirrored columns and rows are formed
// once per face.
__device__ __forceinline__ void face_features(const float4* __restrict__ W, const Grid& G, int dir, int i, int j,
                                              uint32_t* pk, float& rr, float& cref) {
    const bool xface = dir == 0;
    const int n = G.n;
    // lower cell (il, jl); stencil cell (a, b), a along the normal and b along the face, both
    // -1..2, is column il + a, row jl + b on an x face and column il + b, row jl + a on a y face
    const int il = xface ? i - 1 : i, jl = xface ? j : j - 1;
    int col[4], row[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        col[k] = mir(il + k - 1, n);
        row[k] = mir(jl + k - 1, n);
    }
    const float4 wl = W[(size_t)row[1] * n + col[1]];
    const float4 wr = xface ? W[(size_t)row[1] * n + col[2]] : W[(size_t)row[2] * n + col[1]];
    rr = 0.5f * (wl.x + wr.x);
    const float pr = 0.5f * (wl.w + wr.w);
    cref = sqrtf(fmaxf(G.g * pr / rr, 1e-12f));
    const float irr = 1.0f / rr, ipr = 1.0f / pr, ic = 1.0f / cref;
    int k = 0;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int r = xface ? row[b] : row[a], c = xface ? col[a] : col[b];
            const float4 w = W[(size_t)r * n + c];
            const float un = xface ? w.y : w.z, ut = xface ? w.z : w.y;
            pk[k++] = pack2(w.x * irr - 1.0f, un * ic);
            pk[k++] = pack2(ut * ic, w.w * ipr - 1.0f);
        }
}

// features (BF16 [nf][64]) and the correction scale of every face.  Each thread forms one
// face's 64 features in registers; a CTA's 256 faces (32 KB) go out through shared memory as
// contiguous 16-byte stores (a face's row is 128 bytes, so per-element stores would touch a
// different line in every lane).
__global__ void __launch_bounds__(kFeatNT) features_kernel(const float4* __restrict__ W, Grid G,
                                                          __nv_bfloat16* __restrict__ X,
                                                          float* __restrict__ scale /* [nf][2] */) {
    __shared__ uint4 stage[kFeatNT * 8];
    const int nf = 2 * (G.n + 1) * G.n;
    for (int base = blockIdx.x * kFeatNT; base < nf; base += gridDim.x * kFeatNT) {
        const int f = base + threadIdx.x;
        uint32_t pk[32] = {};
        if (f < nf) {
            float rr, cref;
            int dir, i, j;
            face_of(f, G.n, dir, i, j);
            face_features(W, G, dir, i, j, pk, rr, cref);
            scale[2 * (size_t)f] = rr;
            scale[2 * (size_t)f + 1] = cref;
        }
        // chunk q (16 bytes) of face t sits at t * 8 + (q ^ (t & 7)): conflict-free both ways
#pragma unroll
        for (int q = 0; q < 8; ++q)
            stage[threadIdx.x * 8 + (q ^ (threadIdx.x & 7))] =
                make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
        __syncthreads();
        const int nvalid = nf - base < kFeatNT ? nf - base : kFeatNT;
        uint4* __restrict__ dst = reinterpret_cast<uint4*>(X + (size_t)base * NIN);
        for (int L = threadIdx.x; L < nvalid * 8; L += kFeatNT) {
            const int t = L >> 3, q = L & 7;
            dst[L] = stage[t * 8 + (q ^ (t & 7))];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------
// MLP on the 5th-generation tensor cores: tcgen05.mma, BF16 x BF16 -> FP32 in TMEM
// ---------------------------------------------------------------------------------
// A CTA of 256 threads is two independent groups of 128 (warps 0-3 and 4-7) that share the
// weights in shared memory.  A group takes 128 faces per tile, one face per thread and per TMEM
// lane, with its own A operand, TMEM accumulator (64 columns), mbarrier, named barrier and MMA
// issuing thread: every layer is 5 MMAs of M 128, K 16.  Decoupled, the groups of the CTAs on
// an SM overlap one another's feature loads, MMAs and epilogues.
// Operands sit in shared memory in the canonical K-major layout without swizzle: 8 x 8 BF16
// core matrices of 128 contiguous bytes, core matrices adjacent along K 128 B apart (the
// descriptor's leading-dimension offset), 8-row groups 1280 B apart (its stride offset).
// K runs to 80: columns 0..63 hold the layer's inputs, column 64 and 65 of every A row are 1
// and the same columns of the weight rows hold the bias split into two BF16 parts (hi, and
// the remainder lo), so the MMA adds the bias with FP32 accumulation; columns 66..79 are 0.
// Each layer's MMAs are issued by one thread and committed to an mbarrier; the FP32
// accumulators are read back with tcgen05.ld, passed through GELU in packed FP32x2 arithmetic,
// rounded to BF16 and stored as the next layer's A operand -- stored doubled, 2 GELU(z) =
// z + z tanh(.), with the next layer's weights halved: both scalings are exact, so the products
// equal those of GELU(z) and the unscaled weights.  The output layer runs with N = 16 (rows
// 4..15 of its weight tile are zero).
constexpr int kTcRows = 128;       // rows of an MMA tile = TMEM lanes
constexpr int kTcThreads = 256;    // threads per CTA: two groups of kTcRows
constexpr int kTcCols = 128;       // TMEM columns held by a CTA (two 64-column accumulators)
constexpr int kTcK = 80;           // operand K: 64 inputs, the bias pair, zero padding
constexpr int kTcKSteps = kTcK / 16;
constexpr uint32_t kTcWaitLimit = 1u << 16;   // polls of at most kTcSleepNs each
constexpr uint32_t kTcSleepNs = 20000;

__device__ __forceinline__ uint32_t canon_off(int r, int k) {   // bytes; K = 80 BF16 per row
    return (uint32_t)((r >> 3) * (kTcK * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}
// shared-memory matrix descriptor: start >> 4, leading offset 128 B, stride offset 1280 B,
// descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) |
           ((uint64_t)((kTcK * 16) >> 4) << 32) | (1ull << 46);
}
// bounded mbarrier wait that lets the waiting warps sleep: each poll suspends the thread until
// the phase completes or kTcSleepNs pass, so the wait costs few issue slots; gives up after
// `limit` polls
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity), "r"(kTcSleepNs)
            : "memory");
        if (ok) return true;
    }
    return false;
}
// kind::f16 instruction descriptor: D FP32, A and B BF16, both K-major, M = 128, N = n
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);
}
__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, int acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void async_smem_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive accumulator columns of this thread's TMEM lane; the wait is tied to the
// registers so no use of them moves above it
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]),
                   "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]),
                   "+r"(r[14]), "+r"(r[15])
                 :
                 : "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}



struct __align__(1024) TcSmem {
    unsigned char a[2][kTcRows * kTcK * 2];   // each group's activations (its A operand)
    unsigned char w1[64 * kTcK * 2], w2[64 * kTcK * 2], w3[16 * kTcK * 2];
    uint64_t bar[2];                          // each group's MMA completion
    uint32_t taddr;
};

// this thread's group (0 or 1) and its index in the group
__device__ __forceinline__ int grp() { return threadIdx.x >> 7; }
__device__ __forceinline__ int grp_tid() { return threadIdx.x & (kTcRows - 1); }
// the group's named barrier (ids 1 and 2, as immediates; 0 is the CTA's)
__device__ __forceinline__ void grp_sync() {
    if (grp() == 0) asm volatile("bar.sync 1, 128;" ::: "memory");
    else asm volatile("bar.sync 2, 128;" ::: "memory");
}
__device__ __forceinline__ bool grp_any(bool v) {
    uint32_t r;
    if (grp() == 0)
        asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, 1, 128, p;\n selp.u32 %0, 1, 0, q;\n}\n"
                     : "=r"(r) : "r"((uint32_t)v) : "memory");
    else
        asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, 2, 128, p;\n selp.u32 %0, 1, 0, q;\n}\n"
                     : "=r"(r) : "r"((uint32_t)v) : "memory");
    return r != 0;
}

// packed FP32x2 arithmetic (one instruction for two lanes' worth of work)
__device__ __forceinline__ uint64_t f2(float lo, float hi) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float2 f2_split(uint64_t v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
// two BF16 values packed (lo in the low half) from their bit patterns
__device__ __forceinline__ uint32_t bf16_pair(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}
// 8 BF16 weights from global memory, halved (exact) when `half`
__device__ __forceinline__ uint4 w_chunk(const __nv_bfloat16* __restrict__ w, bool half) {
    uint4 q = *reinterpret_cast<const uint4*>(w);
    if (half) {
        uint32_t* u = &q.x;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162*>(&u[k]);
            u[k] = bf16_pair(__float2bfloat16_rn(0.5f * __low2float(v)), __float2bfloat16_rn(0.5f * __high2float(v)));
        }
    }
    return q;
}
// the bias b as its BF16 part and the BF16 rounding of the remainder, in K columns 64 and 65
__device__ __forceinline__ uint4 bias_chunk(float b) {
    const __nv_bfloat16 hi = __float2bfloat16_rn(b);
    const __nv_bfloat16 lo = __float2bfloat16_rn(b - __bfloat162float(hi));
    return make_uint4(bf16_pair(hi, lo), 0u, 0u, 0u);
}

// The pieces of one CTA's MLP work.  Weights into the canonical layout (W2 and W3 halved, W3
// padded to 16 rows) with the bias pairs, the constant K columns 64..79 of the A operands, the
// mbarrier and the CTA's TMEM columns; returns with the CTA synchronised.
__device__ __forceinline__ void mlp_setup(TcSmem& S, const __nv_bfloat16* __restrict__ Wb,
                                          const float* __restrict__ P) {
    const int tid = threadIdx.x;
    const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
    for (int c = tid; c < 64 * 10; c += kTcThreads) {
        const int n = c / 10, kb = c % 10;
        uint4 q1 = zero, q2 = zero;
        if (kb < 8) {
            q1 = w_chunk(Wb + (size_t)n * NIN + kb * 8, false);
            q2 = w_chunk(Wb + H * NIN + (size_t)n * H + kb * 8, true);
        } else if (kb == 8) {
            q1 = bias_chunk(P[OFF_B1 + n]);
            q2 = bias_chunk(P[OFF_B2 + n]);
        }
        *reinterpret_cast<uint4*>(S.w1 + canon_off(n, kb * 8)) = q1;
        *reinterpret_cast<uint4*>(S.w2 + canon_off(n, kb * 8)) = q2;
    }
    for (int c = tid; c < 16 * 10; c += kTcThreads) {
        const int n = c / 10, kb = c % 10;
        uint4 q = zero;
        if (n < NOUT && kb < 8) q = w_chunk(Wb + H * NIN + H * H + (size_t)n * H + kb * 8, true);
        else if (n < NOUT && kb == 8) q = bias_chunk(P[OFF_B3 + n]);
        *reinterpret_cast<uint4*>(S.w3 + canon_off(n, kb * 8)) = q;
    }
    {   // A columns 64..79 of this thread's row: (1, 1, 0, ..., 0)
        const uint32_t one2 = bf16_pair(__float2bfloat16_rn(1.0f), __float2bfloat16_rn(1.0f));
        unsigned char* A = S.a[tid >> 7];
        *reinterpret_cast<uint4*>(A + canon_off(tid & (kTcRows - 1), 64)) = make_uint4(one2, 0u, 0u, 0u);
        *reinterpret_cast<uint4*>(A + canon_off(tid & (kTcRows - 1), 72)) = zero;
    }
    if (tid == 0) {
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
    }
    if ((tid >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.taddr)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    async_smem_fence();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
}

__device__ __forceinline__ void mlp_teardown(TcSmem& S) {
    tc_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
        tc_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(S.taddr), "r"(kTcCols) : "memory");
    }
}

// this thread's row of the tile's A operands (16-byte chunk q of 8 along K)
__device__ __forceinline__ uint4* a_chunk(TcSmem& S, int q) {
    return reinterpret_cast<uint4*>(S.a[threadIdx.x >> 7] + canon_off(threadIdx.x & (kTcRows - 1), q * 8));
}
// this thread's TMEM lane and accumulator: lane quarter warp mod 4, half warp / 4
__device__ __forceinline__ uint32_t lane_addr(const TcSmem& S) {
    const uint32_t w = threadIdx.x >> 5;
    return S.taddr + ((uint32_t)((w & 3) * 32) << 16) + (w >> 2) * 64;
}

// the group's operand made visible to the tensor cores, then one layer's MMAs (K = 5 x 16)
// issued by the group's first thread and committed to the group's mbarrier
__device__ __forceinline__ void mlp_issue(TcSmem& S, int layer) {
    async_smem_fence();
    tc_before_sync();
    grp_sync();
    if (grp_tid() == 0) {
        tc_after_sync();
        const int g = grp();
        const uint32_t wb = smem_u32(layer == 0 ? S.w1 : (layer == 1 ? S.w2 : S.w3));
        const uint32_t id = idesc_bf16(layer == 2 ? 16 : 64);
        const uint32_t sa = smem_u32(S.a[g]);
#pragma unroll
        for (int kk = 0; kk < kTcKSteps; ++kk)
            tc_mma(S.taddr + g * 64, smem_desc(sa + kk * 256), smem_desc(wb + kk * 256), id, kk);
        tc_commit(&S.bar[g]);
    }
}

// waits for the group's layer.  false, in every thread of the group, when the bounded wait gave
// up: *err is set and the group's issuing thread has waited (bounded) for its MMAs in flight, so
// the TMEM can be freed.
__device__ __forceinline__ bool mlp_wait(TcSmem& S, uint32_t& phase, int* err) {
    uint64_t* bar = &S.bar[grp()];
    const bool ok = mbar_wait_sleep(bar, phase, kTcWaitLimit);
    phase ^= 1u;
    if (grp_any(!ok)) {
        if (grp_tid() == 0) {
            atomicExch(err, 1);
            mbar_wait_sleep(bar, phase ^ 1u, kTcWaitLimit);
        }
        return false;
    }
    tc_after_sync();
    return true;
}

// GELU doubled (tanh form) of a pair: 2 GELU(z) = z + z t, t = tanh(z (k + 0.044715 k z^2)),
// k = sqrt(2/pi)
__device__ __forceinline__ uint64_t gelu2x(uint64_t z) {
    const float k = 0.7978845608028654f, c = 0.7978845608028654f * 0.044715f;
    const float2 u = f2_split(f2_mul(z, f2_fma(f2_mul(z, z), f2(c, c), f2(k, k))));
    return f2_fma(z, f2(tanh_fast(u.x), tanh_fast(u.y)), z);
}

// 16 accumulator columns of this thread's TMEM lane into r, without waiting: tc_wait16(r)
// must come before r is read (several loads may be in flight; the wait covers them all)
__device__ __forceinline__ void tc_ld16_issue(uint32_t taddr, uint32_t* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
}
__device__ __forceinline__ void tc_wait16(uint32_t* r) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
                 :
                 : "memory");
}

// a hidden layer's epilogue: this thread's accumulator row (its face, bias included) through
// GELU, doubled, into the next A operand as BF16; the pre-activations to Zs[face] when given.
// The row is read in four 16-column pieces, the next one loading while this one is processed.
__device__ __forceinline__ void mlp_hidden(TcSmem& S, uint32_t tl, float* __restrict__ Zs, int face, bool valid) {
    uint32_t ra[16], rb[16];
    tc_ld16_issue(tl, ra);
    tc_wait16(ra);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        uint32_t* cur = (q & 1) ? rb : ra;
        uint32_t* nxt = (q & 1) ? ra : rb;
        if (q < 3) tc_ld16_issue(tl + (q + 1) * 16, nxt);
        uint32_t hb[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float2 g = f2_split(gelu2x(f2(__uint_as_float(cur[2 * k]), __uint_as_float(cur[2 * k + 1]))));
            hb[k] = pack2(g.x, g.y);
        }
        if (Zs && valid) {
            float4* zo = reinterpret_cast<float4*>(Zs + (size_t)face * H + q * 16);
#pragma unroll
            for (int k = 0; k < 4; ++k)
                zo[k] = make_float4(__uint_as_float(cur[4 * k]), __uint_as_float(cur[4 * k + 1]),
                                    __uint_as_float(cur[4 * k + 2]), __uint_as_float(cur[4 * k + 3]));
        }
        *a_chunk(S, 2 * q) = make_uint4(hb[0], hb[1], hb[2], hb[3]);
        *a_chunk(S, 2 * q + 1) = make_uint4(hb[4], hb[5], hb[6], hb[7]);
        if (q < 3) tc_wait16(nxt);
    }
}

// the output layer's 4 values of this thread's face (biases included)
__device__ __forceinline__ void mlp_out(uint32_t tl, float* o) {
    float y[16];
    tc_ld16(tl, y);
#pragma unroll
    for (int k = 0; k < NOUT; ++k) o[k] = y[k];
}

// Y[nf][4] = MLP(X), 128-face tiles per group.  When Z1/Z2 are given (training), the hidden
// pre-activations are saved.
// A bounded wait that gives up sets *err, waits (bounded) for the CTA's MMAs in flight,
// frees the TMEM columns and returns.
__global__ void __launch_bounds__(kTcThreads, 3)
mlp_forward_kernel(const __nv_bfloat16* __restrict__ X, int nf, const __nv_bfloat16* __restrict__ Wb,
                   const float* __restrict__ P, float* __restrict__ Y, float* __restrict__ Z1,
                   float* __restrict__ Z2, int* __restrict__ err) {
    extern __shared__ unsigned char smem_raw[];
    TcSmem& S = *reinterpret_cast<TcSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    mlp_setup(S, Wb, P);
    const uint32_t tl = lane_addr(S);
    uint32_t phase = 0;
    bool failed = false;

    for (int base = (blockIdx.x * 2 + grp()) * kTcRows; base < nf && !failed; base += gridDim.x * 2 * kTcRows) {
        const int face = base + grp_tid();
        const bool valid = face < nf;
        {   // features -> A
            const uint4* x = reinterpret_cast<const uint4*>(X + (size_t)(valid ? face : 0) * NIN);
#pragma unroll
            for (int q = 0; q < 8; ++q) *a_chunk(S, q) = valid ? x[q] : make_uint4(0u, 0u, 0u, 0u);
        }
#pragma unroll
        for (int layer = 0; layer < 3; ++layer) {
            mlp_issue(S, layer);
            if (!mlp_wait(S, phase, err)) {
                failed = true;
                break;
            }
            if (layer < 2) {
                mlp_hidden(S, tl, layer == 0 ? Z1 : Z2, face, valid);
            } else {
                float o[NOUT];
                mlp_out(tl, o);
                if (valid) *reinterpret_cast<float4*>(Y + (size_t)face * 4) = make_float4(o[0], o[1], o[2], o[3]);
            }
        }
    }
    mlp_teardown(S);
}

// The inference path of a learned step in one kernel, per 128-face tile of a group: the features of every
// face formed straight into the MLP's first operand, the three layers on the tensor cores, and
// (FLUX) the plain MUSCL-Hancock HLLC flux computed on the CUDA cores while the first layer
// runs.  Out go the correction dF [4][nf] (the correction kernel's formula), the guard's face
// mask set to 1, the step's rejection count and maximum wave speed zeroed, and (FLUX) the plain
// flux F [4][nf].  The results equal those of features +
// mlp_forward + correction (+ plain_flux) bit for bit: the same device functions.  Failure
// handling as mlp_forward_kernel's.
template <bool FLUX>
__global__ void __launch_bounds__(kTcThreads, 3)
face_kernel(const float* __restrict__ U, const float4* __restrict__ W, Grid G, float dt,
            const __nv_bfloat16* __restrict__ Wb, const float* __restrict__ P, float* __restrict__ F,
            float* __restrict__ dF, unsigned char* __restrict__ ok, unsigned long long* __restrict__ rejected,
            float* __restrict__ maxs, int* __restrict__ err) {
    extern __shared__ unsigned char smem_raw[];
    TcSmem& S = *reinterpret_cast<TcSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    if (blockIdx.x == 0 && threadIdx.x == 0) {   // the step's counters, read by the guard and the update
        *rejected = 0ull;
        *maxs = 0.0f;
    }
    const int nf = 2 * (G.n + 1) * G.n;
    const float hdt = 0.5f * dt / G.dx;
    mlp_setup(S, Wb, P);
    const uint32_t tl = lane_addr(S);
    uint32_t phase = 0;

    for (int base = (blockIdx.x * 2 + grp()) * kTcRows; base < nf; base += gridDim.x * 2 * kTcRows) {
        const int f = base + grp_tid();
        const bool valid = f < nf;
        int dir = 0, i = 0, j = 0;
        if (valid) face_of(f, G.n, dir, i, j);
        const bool xface = dir == 0;
        float rr = 0.0f, cref = 0.0f;
        {
            uint32_t pk[32] = {};
            if (valid) face_features(W, G, dir, i, j, pk, rr, cref);
#pragma unroll
            for (int q = 0; q < 8; ++q) *a_chunk(S, q) = make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
        }
        mlp_issue(S, 0);
        if (valid) {
            if (FLUX) {   // the plain flux while the tensor cores run the first layer
                float fl[4];
                plain_face_flux(U, G, hdt, f, fl);
#pragma unroll
                for (int v = 0; v < 4; ++v) F[(size_t)v * nf + f] = fl[v];
            }
            ok[f] = 1;
        }
        if (!mlp_wait(S, phase, err)) break;
        mlp_hidden(S, tl, nullptr, f, valid);
        mlp_issue(S, 1);
        if (!mlp_wait(S, phase, err)) break;
        mlp_hidden(S, tl, nullptr, f, valid);
        mlp_issue(S, 2);
        if (!mlp_wait(S, phase, err)) break;
        float o[NOUT];
        mlp_out(tl, o);
        if (valid) {
            const float m = rr * cref;
            dF[f] = m * o[0];
            dF[(size_t)nf + f] = m * cref * (xface ? o[1] : o[2]);
            dF[2 * (size_t)nf + f] = m * cref * (xface ? o[2] : o[1]);
            dF[3 * (size_t)nf + f] = m * cref * cref * o[3];
        }
    }
    mlp_teardown(S);
}

size_t mlp_forward_smem() { return sizeof(TcSmem) + 1024; }

// ---------------------------------------------------------------------------------
// MLP backward on the tensor cores (BF16 operands, FP32 accumulation in TMEM)
// ---------------------------------------------------------------------------------
// Per tile of 128 faces (one per TMEM lane; four threads per face, 16 of the 64 units each) of a
// 512-thread CTA:
//   the tile's saved rows (pre-activations z1, z2, inputs x, output gradients dY) arrive in
//     shared memory by coalesced 16-byte asynchronous copies into rows padded by 16 bytes, so
//     that a thread reading its own face's row meets no bank conflict; the next tile's are
//     issued as soon as this one's are consumed, so the copies overlap the MMAs;
//   dz2 = (dY W3) * gelu'(z2) on the CUDA cores (K = 4);
//   dz1 = (dz2 W2) * gelu'(z1): one MMA, M 128 faces, N 64, K 64; A = dz2 read in place from the
//     weight-gradient operand below (its bytes are a K-major view of the faces' dz2 rows), B =
//     W2 transposed into K-major rows at setup;
//   the weight gradients in one MMA per tile, accumulated in TMEM over all the CTA's tiles:
//     M 128 = [dz1 | dz2] units, N 144 = [x | h1 | 1 | 0 ...], K 128 = the tile's faces, both
//     operands MN-major (a face's values contiguous): D[0:64][0:64] = sum dz1^T x = dW1,
//     D[64:128][64:128] = sum dz2^T h1 = dW2, D[:][128] = sum dz = db1, db2; the off-diagonal
//     blocks are not used;
//   dW3 = sum dY^T h2 and db3 on the CUDA cores from shared memory while that MMA runs.
// The activations h1, h2 are the forward's (BF16(gelu(z)) from the saved pre-activations).
// MN-major canonical layout without swizzle: core matrices of 8 K-rows x 8 contiguous M/N
// elements (128 B), K-adjacent core matrices 128 B apart (the descriptor's leading offset),
// M/N-adjacent ones 2048 B apart (its stride offset), so a face's 8 consecutive values are one
// 16-byte store.  Bounded waits as the forward kernel's.
constexpr int kBwTile = 128;                 // faces per tile = threads per CTA = the MMA's K
constexpr int kBwN = 144;                    // N of the weight-gradient MMA
constexpr int kBwColD1 = 192;                // TMEM column of the dz1 accumulator (64 columns)
constexpr int kBwCols = 256;                 // TMEM columns held by a CTA

__device__ __forceinline__ uint32_t mn_off(int r, int k) {   // bytes; K = 128 faces
    return (uint32_t)((r >> 3) * (kBwTile * 16) + (k >> 3) * 128 + (k & 7) * 16 + (r & 7) * 2);
}
__device__ __forceinline__ uint32_t k64_off(int r, int k) {  // bytes; K-major, K = 64
    return (uint32_t)((r >> 3) * 1024 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}
__device__ __forceinline__ uint64_t smem_desc_lbo_sbo(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}
// kind::f16 instruction descriptor, both operands MN-major
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}
constexpr int kBwParts = 4;                          // threads per face: each takes 16 of the 64 units
constexpr int kBwThreads = kBwTile * kBwParts;       // 512
constexpr int kBwU = H / kBwParts;                   // 16 units per thread

struct __align__(1024) BwSmem {
    unsigned char aw[128 * kBwTile * 2];    // [dz1 | dz2] per face, MN-major (32 KB)
    unsigned char bw[kBwN * kBwTile * 2];   // [x | h1 | 1 | 0] per face, MN-major (36 KB)
    unsigned char w2t[64 * 64 * 2];         // W2 transposed, K-major (8 KB)
    float z1[kBwTile][H + 4], z2[kBwTile][H + 4];   // the tile's saved rows, padded (68 KB)
    __nv_bfloat16 x[kBwTile][NIN + 8];              // (18 KB)
    float dyr[kBwTile][NOUT];                       // (2 KB)
    __nv_bfloat16 h2[kBwTile][H + 8];               // the tile's h2 and dY for dW3 (18 KB + 2 KB)
    float dy[kBwTile][NOUT];
    float w3[NOUT][H];
    uint64_t bar;
    uint32_t taddr;
};

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__global__ void __launch_bounds__(kBwThreads, 1)
mlp_backward_kernel(const __nv_bfloat16* __restrict__ X, int nf, const __nv_bfloat16* __restrict__ Wb,
                    const float* __restrict__ Z1, const float* __restrict__ Z2, const float* __restrict__ dY,
                    float* __restrict__ grad, int* __restrict__ err) {
    extern __shared__ unsigned char smem_raw[];
    BwSmem& S = *reinterpret_cast<BwSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x;
    const int l = tid & (kBwTile - 1), part = tid / kBwTile, u0 = part * kBwU;   // face row, its units
    // W2 transposed: B row c, K column o = W2[o][c]; W3 as FP32; the constant rows of bw
    for (int e = tid; e < H * H; e += kBwThreads) {
        const int o = e / H, c = e % H;
        *reinterpret_cast<__nv_bfloat16*>(S.w2t + k64_off(c, o)) = Wb[H * NIN + e];
    }
    for (int e = tid; e < NOUT * H; e += kBwThreads) S.w3[e / H][e % H] = __bfloat162float(Wb[H * NIN + H * H + e]);
    if (part < 2) {
        const uint32_t one = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(1.0f));
        const int r = 128 + part * 8;
        *reinterpret_cast<uint4*>(S.bw + mn_off(r, l)) = make_uint4(r == 128 ? one : 0u, 0u, 0u, 0u);
    }
    if (tid == 0) mbar_init(&S.bar, 1);
    if ((tid >> 5) == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.taddr)),
                     "r"(kBwCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    async_smem_fence();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const uint32_t tm = S.taddr;
    const uint32_t lane = tm + ((uint32_t)(((tid >> 5) & 3) * 32) << 16);   // lane quarter of row l
    uint32_t phase = 0;
    bool failed = false, first = true, ld_inflight = false;   // ld_inflight: a tile's copies issued, not waited for
    float g3 = 0.0f, gb3 = 0.0f;   // dW3 entry (tid mod 256) over half the faces; db3

    // the saved rows of the tile at base into the padded rows: coalesced 16-byte asynchronous
    // copies by all threads, one commit group (waited for before the rows are read)
    auto load_tile = [&](int base) {
        const int nv = nf - base < kBwTile ? nf - base : kBwTile;
        for (int c = tid; c < nv * (H / 4); c += kBwThreads) {
            const int r = c / (H / 4), k = (c % (H / 4)) * 4;
            cp_async16(&S.z1[r][k], Z1 + (size_t)(base + r) * H + k);
            cp_async16(&S.z2[r][k], Z2 + (size_t)(base + r) * H + k);
        }
        for (int c = tid; c < nv * (NIN / 8); c += kBwThreads) {
            const int r = c / (NIN / 8), k = (c % (NIN / 8)) * 8;
            cp_async16(&S.x[r][k], X + (size_t)(base + r) * NIN + k);
        }
        for (int c = tid; c < nv; c += kBwThreads) cp_async16(S.dyr[c], dY + (size_t)(base + c) * NOUT);
        cp_async_commit();
    };
    // publish the operands, issue MMAs (thread 0), wait; false when the bounded wait gave up
    auto run_mma = [&](int which) -> bool {
        async_smem_fence();
        tc_before_sync();
        __syncthreads();
        if (tid == 0) {
            tc_after_sync();
            if (which == 0) {   // dz1 pre-activations: dz2 (K-major view of aw's rows 64..127) x W2^T
                const uint32_t sa = smem_u32(S.aw) + 8 * (kBwTile * 16), sb = smem_u32(S.w2t);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
                    tc_mma(tm + kBwColD1, smem_desc_lbo_sbo(sa + kk * 2 * (kBwTile * 16), kBwTile * 16, 128),
                           smem_desc_lbo_sbo(sb + kk * 256, 128, 1024), idesc_bf16(64), kk);
            } else {            // weight gradients, K = the tile's 128 faces
                const uint32_t sa = smem_u32(S.aw), sb = smem_u32(S.bw);
#pragma unroll
                for (int kk = 0; kk < kBwTile / 16; ++kk)
                    tc_mma(tm, smem_desc_lbo_sbo(sa + kk * 256, 128, kBwTile * 16),
                           smem_desc_lbo_sbo(sb + kk * 256, 128, kBwTile * 16), idesc_bf16_mn(128, kBwN),
                           (first && kk == 0) ? 0 : 1);
            }
            tc_commit(&S.bar);
        }
        const bool ok = mbar_wait_sleep(&S.bar, phase, kTcWaitLimit);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicExch(err, 1);
                mbar_wait_sleep(&S.bar, phase ^ 1u, kTcWaitLimit);
            }
            return false;
        }
        tc_after_sync();
        return true;
    };

    int base = blockIdx.x * kBwTile;
    if (base < nf) {
        load_tile(base);
        ld_inflight = true;
    }
    for (; base < nf && !failed; base += gridDim.x * kBwTile) {
        const bool valid = base + l < nf;
        cp_async_wait_all();
        __syncthreads();
        ld_inflight = false;
        float dy[NOUT] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (valid) {
            const float4 d = *reinterpret_cast<const float4*>(S.dyr[l]);
            dy[0] = d.x; dy[1] = d.y; dy[2] = d.z; dy[3] = d.w;
        }
        if (part == 0)
#pragma unroll
            for (int k = 0; k < NOUT; ++k) S.dy[l][k] = dy[k];
        // this thread's 16 units: x, h1 into bw; dz2 into aw; h2 into its tile; gelu'(z1) kept
        float g1[kBwU];
#pragma unroll
        for (int q = 0; q < kBwU / 8; ++q) {
            const int ub = u0 + q * 8;
            uint4 xq = make_uint4(0u, 0u, 0u, 0u);
            float z1v[8] = {}, z2v[8] = {};
            if (valid) {
                xq = *reinterpret_cast<const uint4*>(&S.x[l][ub]);
                const float4 a = *reinterpret_cast<const float4*>(&S.z1[l][ub]);
                const float4 b = *reinterpret_cast<const float4*>(&S.z1[l][ub + 4]);
                const float4 c = *reinterpret_cast<const float4*>(&S.z2[l][ub]);
                const float4 d = *reinterpret_cast<const float4*>(&S.z2[l][ub + 4]);
                z1v[0] = a.x; z1v[1] = a.y; z1v[2] = a.z; z1v[3] = a.w; z1v[4] = b.x; z1v[5] = b.y; z1v[6] = b.z; z1v[7] = b.w;
                z2v[0] = c.x; z2v[1] = c.y; z2v[2] = c.z; z2v[3] = c.w; z2v[4] = d.x; z2v[5] = d.y; z2v[6] = d.z; z2v[7] = d.w;
            }
            uint32_t h1p[4], h2p[4], dzp[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                float dz[2], h1[2], h2[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int o = ub + 2 * k + u;
                    const float z1 = z1v[2 * k + u], z2 = z2v[2 * k + u];
                    float s = 0.0f;
#pragma unroll
                    for (int m = 0; m < NOUT; ++m) s = fmaf(dy[m], S.w3[m][o], s);
                    float hh1, gg1, hh2, gg2;
                    gelu_both(z1, hh1, gg1);
                    gelu_both(z2, hh2, gg2);
                    dz[u] = valid ? gg2 * s : 0.0f;
                    h1[u] = valid ? hh1 : 0.0f;
                    h2[u] = valid ? hh2 : 0.0f;
                    g1[q * 8 + 2 * k + u] = valid ? gg1 : 0.0f;
                }
                h1p[k] = pack2(h1[0], h1[1]);
                h2p[k] = pack2(h2[0], h2[1]);
                dzp[k] = pack2(dz[0], dz[1]);
            }
            *reinterpret_cast<uint4*>(S.bw + mn_off(ub, l)) = xq;
            *reinterpret_cast<uint4*>(S.bw + mn_off(64 + ub, l)) = make_uint4(h1p[0], h1p[1], h1p[2], h1p[3]);
            *reinterpret_cast<uint4*>(S.aw + mn_off(64 + ub, l)) = make_uint4(dzp[0], dzp[1], dzp[2], dzp[3]);
            *reinterpret_cast<uint4*>(&S.h2[l][ub]) = make_uint4(h2p[0], h2p[1], h2p[2], h2p[3]);
        }
        __syncthreads();   // the saved rows are consumed: the next tile's copies may land
        if (base + gridDim.x * kBwTile < nf) {
            load_tile(base + gridDim.x * kBwTile);
            ld_inflight = true;
        }
        if (!run_mma(0)) { failed = true; break; }
        {   // dz1 = (dz2 W2) * gelu'(z1) for this thread's 16 units, into aw's first 64 rows
            float d[16];
            tc_ld16(lane + kBwColD1 + u0, d);
            uint32_t p[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) p[k] = pack2(d[2 * k] * g1[2 * k], d[2 * k + 1] * g1[2 * k + 1]);
            *reinterpret_cast<uint4*>(S.aw + mn_off(u0, l)) = make_uint4(p[0], p[1], p[2], p[3]);
            *reinterpret_cast<uint4*>(S.aw + mn_off(u0 + 8, l)) = make_uint4(p[4], p[5], p[6], p[7]);
        }
        if (!run_mma(1)) { failed = true; break; }
        first = false;
        {   // dW3 entry tid mod 256 over this thread's half of the faces; db3
            const int e = tid & 255, o = e / H, c = e % H, g0 = (tid >> 8) * (kBwTile / 2);
            for (int g = g0; g < g0 + kBwTile / 2; ++g) g3 = fmaf(S.dy[g][o], __bfloat162float(S.h2[g][c]), g3);
            if (tid < NOUT)
                for (int g = 0; g < kBwTile; ++g) gb3 += S.dy[g][tid];
        }
        __syncthreads();
    }
    if (ld_inflight) cp_async_wait_all();   // copies still in flight land before the shared memory is given up
    if (!failed && !first) {
        // row l of the accumulated D, this thread's 16 columns of its block
        const bool l1 = l < 64;
        const int row = l1 ? l : l - 64;
        float d[16];
        tc_ld16(lane + (l1 ? 0 : 64) + u0, d);
        float* gw = grad + (l1 ? OFF_W1 + row * NIN : OFF_W2 + row * H) + u0;
#pragma unroll
        for (int k = 0; k < 16; ++k) atomicAdd(gw + k, d[k]);
        if (part == 0) {   // warp-uniform, as the collective tcgen05.ld requires
            tc_ld16(lane + 128, d);
            atomicAdd(grad + (l1 ? OFF_B1 : OFF_B2) + row, d[0]);
        }
    }
    if (!first) {
        atomicAdd(&grad[OFF_W3 + (tid & 255)], g3);
        if (tid < NOUT) atomicAdd(&grad[OFF_B3 + tid], gb3);
    }
    tc_before_sync();
    __syncthreads();
    if ((tid >> 5) == 0) {
        tc_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"(kBwCols) : "memory");
    }
}

size_t mlp_backward_smem() { return sizeof(BwSmem) + 1024; }

// Adam on the FP32 master parameters; refreshes the BF16 weight copy
__global__ void adam_kernel(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ m,
                            float* __restrict__ v, __nv_bfloat16* __restrict__ Wb, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < NPARAM; k += gridDim.x * blockDim.x) {
        const float g = G[k];
        const float mk = b1 * m[k] + (1.f - b1) * g, vk = b2 * v[k] + (1.f - b2) * g * g;
        m[k] = mk;
        v[k] = vk;
        P[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
    }
}

__global__ void to_bf16_kernel(const float* __restrict__ P, __nv_bfloat16* __restrict__ Wb) {
    // BF16 copies of W1, W2, W3 (contiguous: [W1 | W2 | W3])
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < H * NIN + H * H + NOUT * H; k += gridDim.x * blockDim.x) {
        int src = k < H * NIN ? OFF_W1 + k : (k < H * NIN + H * H ? OFF_W2 + (k - H * NIN) : OFF_W3 + (k - H * NIN - H * H));
        Wb[k] = __float2bfloat16_rn(P[src]);
    }
}

// ---------------------------------------------------------------------------------
// corrections, guarded update, loss gradient
// ---------------------------------------------------------------------------------
// dF (physical, [4][nf]) from the MLP outputs
__global__ void correction_kernel(const float* __restrict__ Y, const float* __restrict__ scale, int n,
                                  float* __restrict__ dF) {
    const int nf = 2 * (n + 1) * n;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        const float r = scale[2 * (size_t)f], c = scale[2 * (size_t)f + 1];
        const float m = r * c;
        const float o0 = Y[4 * (size_t)f], o1 = Y[4 * (size_t)f + 1], o2 = Y[4 * (size_t)f + 2], o3 = Y[4 * (size_t)f + 3];
        const bool xface = f < (n + 1) * n;
        dF[f] = m * o0;
        dF[(size_t)nf + f] = m * c * (xface ? o1 : o2);          // x momentum: normal on x faces
        dF[2 * (size_t)nf + f] = m * c * (xface ? o2 : o1);      // y momentum
        dF[3 * (size_t)nf + f] = m * c * c * o3;
    }
}

__device__ __forceinline__ int xf(int n, int i, int j) { return j * (n + 1) + i; }            // left face of (i,j)
__device__ __forceinline__ int yf(int n, int i, int j) { return (n + 1) * n + j * n + i; }    // bottom face

// update of cell (i,j) with fluxes F (+ dF on faces whose mask bit is set)
__device__ __forceinline__ void cell_update(const float* __restrict__ U, const float* __restrict__ F,
                                            const float* __restrict__ dF, const unsigned char* __restrict__ ok,
                                            int n, float r, int i, int j, float* out) {
    const int nf = 2 * (n + 1) * n;
    const int fl = xf(n, i, j), fr = xf(n, i + 1, j), fb = yf(n, i, j), ft = yf(n, i, j + 1);
    const size_t o = (size_t)j * n + i, pl = (size_t)n * n;
    for (int v = 0; v < 4; ++v) {
        float Fl = F[(size_t)v * nf + fl], Fr = F[(size_t)v * nf + fr];
        float Gb = F[(size_t)v * nf + fb], Gt = F[(size_t)v * nf + ft];
        if (dF) {
            if (!ok || ok[fl]) Fl += dF[(size_t)v * nf + fl];
            if (!ok || ok[fr]) Fr += dF[(size_t)v * nf + fr];
            if (!ok || ok[fb]) Gb += dF[(size_t)v * nf + fb];
            if (!ok || ok[ft]) Gt += dF[(size_t)v * nf + ft];
        }
        out[v] = U[v * pl + o] + r * ((Fl - Fr) + (Gb - Gt));
    }
}

__device__ __forceinline__ bool cell_bad(float g1, const float* un, const float* up, const float* u0, float bound) {
    PrimF w = prim(g1, un);
    if (!(w.r > 0.0f) || !(w.p > 0.0f)) return true;
    const float dr = fabsf(un[0] - up[0]), de = fabsf(un[3] - up[3]);
    const float sr = fabsf(up[0] - u0[0]) + 1e-6f * fabsf(u0[0]), se = fabsf(up[3] - u0[3]) + 1e-6f * fabsf(u0[3]);
    return dr > bound * sr || de > bound * se;
}

// Local-extremum guard (flux-corrected-transport bounds, Zalesak 1979): the corrected density
// and energy must stay within the minimum and maximum, over the cell and its 8 neighbours, of
// both the old state and the plain (uncorrected) update; and density and pressure positive.
__device__ __forceinline__ bool cell_bad_local(const float* __restrict__ U, const float* __restrict__ F,
                                               Grid G, float r, int i, int j, const float* un) {
    PrimF w = prim(G.g1, un);
    if (!(w.r > 0.0f) || !(w.p > 0.0f)) return true;
    const int n = G.n;
    const size_t pl = (size_t)n * n;
    float lo0 = 3.4e38f, hi0 = -3.4e38f, lo3 = 3.4e38f, hi3 = -3.4e38f;
    for (int b = -1; b <= 1; ++b)
        for (int a = -1; a <= 1; ++a) {
            const int ii = i + a, jj = j + b;
            if (ii < 0 || jj < 0 || ii >= n || jj >= n) continue;
            float up[4];
            cell_update(U, F, nullptr, nullptr, n, r, ii, jj, up);
            const size_t o = (size_t)jj * n + ii;
            lo0 = fminf(lo0, fminf(up[0], U[o]));
            hi0 = fmaxf(hi0, fmaxf(up[0], U[o]));
            lo3 = fminf(lo3, fminf(up[3], U[3 * pl + o]));
            hi3 = fmaxf(hi3, fmaxf(up[3], U[3 * pl + o]));
        }
    return un[0] < lo0 || un[0] > hi0 || un[3] < lo3 || un[3] > hi3;
}

// mode 0: the change bound of cell_bad; mode 1: the local-extremum bounds of cell_bad_local
__device__ __forceinline__ bool guard_bad(const float* __restrict__ U, const float* __restrict__ F, Grid G,
                                          float r, int i, int j, const float* un, const float* up,
                                          const float* u0, float bound, int mode) {
    return mode == 1 ? cell_bad_local(U, F, G, r, i, j, un) : cell_bad(G.g1, un, up, u0, bound);
}

// pass 1: mark faces whose correction is rejected (any adjacent cell violates); Uc (optional)
// keeps every cell's update with all its corrections for pass 2
__global__ void guard_kernel(const float* __restrict__ U, const float* __restrict__ F, const float* __restrict__ dF,
                             Grid G, float r, float bound, int mode, unsigned char* __restrict__ ok,
                             unsigned long long* __restrict__ rejected, float4* __restrict__ Uc) {
    const int n = G.n;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n * n; c += gridDim.x * blockDim.x) {
        const int i = c % n, j = c / n;
        float un[4], up[4], u0[4];
        cell_update(U, F, dF, nullptr, n, r, i, j, un);
        cell_update(U, F, nullptr, nullptr, n, r, i, j, up);
        if (Uc) Uc[c] = make_float4(un[0], un[1], un[2], un[3]);
        for (int v = 0; v < 4; ++v) u0[v] = U[(size_t)v * n * n + (size_t)j * n + i];
        if (guard_bad(U, F, G, r, i, j, un, up, u0, bound, mode)) {
            ok[xf(n, i, j)] = 0; ok[xf(n, i + 1, j)] = 0; ok[yf(n, i, j)] = 0; ok[yf(n, i, j + 1)] = 0;
            atomicAdd(rejected, 1ull);
        }
    }
}

// pass 2: the update (corrections where accepted); a cell still violating takes its plain update
// Wn (optional): the primitives of the new state, as prims_kernel forms them, for the next step's
// features.  Uc (optional, with dF and ok): pass 1's fully corrected updates -- a cell whose four
// faces all kept their corrections takes its own (the same arithmetic as recomputing it; the
// guard passed it, or a face would have been rejected), the others are recomputed.
__global__ void update_kernel(const float* __restrict__ U, const float* __restrict__ F, const float* __restrict__ dF,
                              const unsigned char* __restrict__ ok, Grid G, float r, float bound, int mode,
                              float* __restrict__ Un, float* __restrict__ maxs, float4* __restrict__ Wn,
                              const float4* __restrict__ Uc) {
    const int n = G.n;
    float m = 0.0f;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n * n; c += gridDim.x * blockDim.x) {
        const int i = c % n, j = c / n;
        float un[4], up[4], u0[4];
        if (Uc && ok[xf(n, i, j)] && ok[xf(n, i + 1, j)] && ok[yf(n, i, j)] && ok[yf(n, i, j + 1)]) {
            const float4 q = Uc[c];
            un[0] = q.x; un[1] = q.y; un[2] = q.z; un[3] = q.w;
        } else if (dF) {
            cell_update(U, F, nullptr, nullptr, n, r, i, j, up);
            cell_update(U, F, dF, ok, n, r, i, j, un);
            for (int v = 0; v < 4; ++v) u0[v] = U[(size_t)v * n * n + (size_t)j * n + i];
            if (ok && guard_bad(U, F, G, r, i, j, un, up, u0, bound, mode))
                for (int v = 0; v < 4; ++v) un[v] = up[v];
        } else {
            cell_update(U, F, nullptr, nullptr, n, r, i, j, un);
        }
        for (int v = 0; v < 4; ++v) Un[(size_t)v * n * n + (size_t)j * n + i] = un[v];
        PrimF w = prim(G.g1, un);
        if (Wn) Wn[(size_t)j * n + i] = make_float4(w.r, w.u, w.v, w.p);
        const float cs = sqrtf(G.g * w.p / w.r);
        const float s = fmaxf(fabsf(w.u), fabsf(w.v)) + cs;
        if (s > m) m = s;
    }
    // the CTA's maximum, then one atomic per CTA (non-negative floats order as their bit patterns)
    __shared__ float wmax[32];
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? wmax[threadIdx.x] : 0.0f;
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0 && m > 0.0f) atomicMax(reinterpret_cast<int*>(maxs), __float_as_int(m));
    }
}

// dL/dY for L = (1/N) sum_cells sum_v w_v (U^{n+1}_v - T_v)^2, U^{n+1} with every correction
__global__ void loss_grad_kernel(const float* __restrict__ Un, const float* __restrict__ T, const float* __restrict__ scale,
                                 int n, float r, const float* __restrict__ wv, const unsigned char* __restrict__ ok,
                                 float* __restrict__ dY, double* __restrict__ loss) {
    const int nf = 2 * (n + 1) * n;
    const float invN = 1.0f / ((float)n * n);
    double ls = 0.0;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        int dir, i, j;
        face_of(f, n, dir, i, j);
        // cells below (lower) and above (upper) the face; outside cells do not exist
        const int il = dir == 0 ? i - 1 : i, jl = dir == 0 ? j : j - 1;
        const int iu = i, ju = j;
        float gF[4];
        for (int v = 0; v < 4; ++v) {
            float gl = 0.f, gu = 0.f;
            if (il >= 0 && jl >= 0) {
                const size_t o = (size_t)v * n * n + (size_t)jl * n + il;
                gl = 2.0f * wv[v] * (Un[o] - T[o]) * invN;
            }
            if (iu < n && ju < n) {
                const size_t o = (size_t)v * n * n + (size_t)ju * n + iu;
                gu = 2.0f * wv[v] * (Un[o] - T[o]) * invN;
            }
            // U_lower gets -r*F, U_upper gets +r*F; a face whose correction the guard rejected
            // does not take part
            gF[v] = (ok && !ok[f]) ? 0.0f : r * (gu - gl);
        }
        const float rr = scale[2 * (size_t)f], c = scale[2 * (size_t)f + 1], m = rr * c;
        const bool xface = dir == 0;
        dY[4 * (size_t)f] = m * gF[0];
        dY[4 * (size_t)f + 1] = m * c * (xface ? gF[1] : gF[2]);
        dY[4 * (size_t)f + 2] = m * c * (xface ? gF[2] : gF[1]);
        dY[4 * (size_t)f + 3] = m * c * c * gF[3];
    }
    // the loss itself, over cells
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n * n; c += gridDim.x * blockDim.x)
        for (int v = 0; v < 4; ++v) {
            const float d = Un[(size_t)v * n * n + c] - T[(size_t)v * n * n + c];
            ls += (double)(wv[v] * d * d * invN);
        }
    for (int o = 16; o > 0; o >>= 1) ls += __shfl_xor_sync(0xffffffffu, ls, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, ls);
}

}  // namespace lc
}  // namespace hf

// =====================================================================================
// host side
// =====================================================================================
using namespace hf::lc;

struct hf_lc {
    int n = 0, lim = 0;
    double dx = 0, gamma = 1.4, cfl = 0.8, bound = 0.5;
    int guard_mode = 0;        // 0: change bound, 1: local-extremum bounds
    int train_guard = 0;       // training applies the guard as inference does
    int fused = 1;             // inference: 1 features + MLP + correction in face_kernel, 2 with the
                               // plain flux too, 0 the separate kernels
    int face_ctas_per_sm = 0;  // face_kernel CTAs per SM (0: as many as fit)
    int sms = 152;             // the device's SMs, and how many CTAs of each MLP kernel fit on one
    int fit_fwd = 1, fit_face[2] = {1, 1};
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;           // the plain fluxes, beside the fused face kernel
    cudaEvent_t fork = nullptr, join = nullptr;
    float *U[2] = {nullptr, nullptr}, *F = nullptr, *dF = nullptr, *scale = nullptr, *Y = nullptr;
    float *Z1 = nullptr, *Z2 = nullptr, *dY = nullptr, *T = nullptr, *wv = nullptr;
    __nv_bfloat16 *X = nullptr, *Wb = nullptr;
    float4* Wp = nullptr;      // per-cell primitives (rho, u, v, p) for the feature stencils
    bool wp_valid = false;     // Wp holds the primitives of U[cur] (written by the last step)
    float4* Uc = nullptr;      // the guard pass's fully corrected cell updates
    bool maxs_valid = false;   // maxs holds the maximum wave speed of U[cur] (the last step's update
                               // or CFL pass formed it)
    float *P = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr, *maxs = nullptr;
    unsigned char* ok = nullptr;
    unsigned long long* rejected = nullptr;
    double* loss = nullptr;
    int* derr = nullptr;       // device error word (a bounded wait gave up)
    int cur = 0;
    long long steps = 0;       // steps since time 0 (TimeStep's start-up multiplier)
    long long adam_t = 0;
    double t = 0.0;
    std::vector<void*> allocs;
    std::string err;
};

namespace {

int lfail(hf_lc* L, int code, const std::string& m) {
    if (L) L->err = m;
    return code;
}
#define LCK(call)                                                                             \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return lfail(L, HF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int alloc(hf_lc* L, T** p, size_t n) {
    LCK(cudaMalloc(p, n * sizeof(T) + 64));
    L->allocs.push_back(*p);
    LCK(cudaMemset(*p, 0, n * sizeof(T) + 64));
    return HF_OK;
}

hf::lc::Grid grid(const hf_lc* L) {
    hf::lc::Grid G;
    G.n = L->n;
    G.dx = (float)L->dx;
    G.g = (float)L->gamma;
    G.g1 = (float)(L->gamma - 1.0);
    G.lim = L->lim;
    return G;
}

int nfaces(const hf_lc* L) { return 2 * (L->n + 1) * L->n; }
int blocks_for(long long n, int t) { long long b = (n + t - 1) / t; return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b)); }

// Persistent CTAs of the MLP kernels (256 threads, two 128-face tiles at a time): per_sm per SM (0: as
// many as fit by registers, shared memory and TMEM), never more than the tiles.  The fit (formed
// once per context) comes from the kernel's attributes: registers are allocated per warp in units of 256 from
// each SM sub-partition's 16,384; each CTA holds its dynamic shared memory plus 1 KB the
// hardware reserves; 4 CTAs x 128 TMEM columns fill an SM's 512.
int mlp_fit(const void* kernel) {
    int dev = 0, smem_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess || smem_sm < 1)
        smem_sm = 233472;
    cudaFuncAttributes fa{};
    int fit = 1;
    if (cudaFuncGetAttributes(&fa, kernel) == cudaSuccess && fa.numRegs > 0) {
        const int warp_regs = ((fa.numRegs * 32 + 255) / 256) * 256;
        const int by_regs = 4 * (16384 / warp_regs) / (hf::lc::kTcThreads / 32);
        const int by_smem = smem_sm / (int)(hf::lc::mlp_forward_smem() + fa.sharedSizeBytes + 1024);
        fit = by_regs < by_smem ? by_regs : by_smem;
        fit = fit > 4 ? 4 : (fit < 1 ? 1 : fit);
    }
    return fit;
}
// the grid for nf faces with fit CTAs per SM at most (per_sm, when set and lower, instead)
int mlp_grid(const hf_lc* L, int fit, int nf, int per_sm) {
    const int per = per_sm > 0 && per_sm < fit ? per_sm : fit;
    const int tiles = (nf + hf::lc::kTcThreads - 1) / hf::lc::kTcThreads;
    return tiles < per * L->sms ? tiles : per * L->sms;
}

void launch_forward(hf_lc* L, int nf, bool save_acts) {
    const int g = mlp_grid(L, L->fit_fwd, nf, 0);
    hf::lc::mlp_forward_kernel<<<g, hf::lc::kTcThreads, hf::lc::mlp_forward_smem(), L->stream>>>(
        L->X, nf, L->Wb, L->P, L->Y, save_acts ? L->Z1 : nullptr, save_acts ? L->Z2 : nullptr, L->derr);
}

// the MLP backward: one persistent CTA per SM at most (its shared memory allows one)
void launch_backward(hf_lc* L, int nf) {
    const int sms = L->sms;
    const int tiles = (nf + hf::lc::kBwTile - 1) / hf::lc::kBwTile;
    hf::lc::mlp_backward_kernel<<<tiles < sms ? tiles : sms, hf::lc::kBwThreads, hf::lc::mlp_backward_smem(), L->stream>>>(
        L->X, nf, L->Wb, L->Z1, L->Z2, L->dY, L->grad, L->derr);
}

// the device error word: a bounded wait in a kernel gave up
int check_derr(hf_lc* L) {
    int e = 0;
    LCK(cudaMemcpy(&e, L->derr, sizeof e, cudaMemcpyDeviceToHost));
    if (e) return lfail(L, HF_ERR_DEVICE, "a bounded device wait gave up (tensor-core MLP)");
    return HF_OK;
}

// plain fluxes, and (use_mlp) features -> MLP -> corrections for state U[cur]
void launch_features(hf_lc* L) {
    hf::lc::Grid G = grid(L);
    const int nf = nfaces(L);
    prims_kernel<<<blocks_for(L->n * L->n, 256), 256, 0, L->stream>>>(L->U[L->cur], L->n, G.g1, L->Wp);
    L->wp_valid = true;
    features_kernel<<<blocks_for(nf, hf::lc::kFeatNT), hf::lc::kFeatNT, 0, L->stream>>>(L->Wp, G, L->X, L->scale);
}

// plain fluxes F, and (use_mlp) the corrections dF for state U[cur].  Inference (no saved
// activations) with the fused kernel also sets the guard's face mask and zeroes the step's
// counters; returns through *mask_set whether it did.
int fluxes(hf_lc* L, float dt, bool use_mlp, bool save_acts, bool* mask_set = nullptr) {
    hf::lc::Grid G = grid(L);
    const int nf = nfaces(L);
    if (mask_set) *mask_set = false;
    if (use_mlp && !save_acts && L->fused) {
        if (!L->wp_valid)   // else the previous step's update wrote them
            prims_kernel<<<blocks_for(L->n * L->n, 256), 256, 0, L->stream>>>(L->U[L->cur], L->n, G.g1, L->Wp);
        L->wp_valid = true;
        const size_t sm = hf::lc::mlp_forward_smem();
        const int units = nf;
        if (L->fused == 2) {
            face_kernel<true><<<mlp_grid(L, L->fit_face[1], units, L->face_ctas_per_sm),
                                hf::lc::kTcThreads, sm, L->stream>>>(L->U[L->cur], L->Wp, G, dt, L->Wb, L->P, L->F,
                                                                     L->dF, L->ok, L->rejected, L->maxs, L->derr);
        } else {
            // the plain fluxes on the side stream, running beside the face kernel (independent
            // work: the face kernel is latency-bound, the flux kernel arithmetic-bound); the face
            // kernel at 2 CTAs per SM by default leaves the flux kernel room on every SM
            LCK(cudaEventRecord(L->fork, L->stream));
            face_kernel<false><<<mlp_grid(L, L->fit_face[0], units,
                                          L->face_ctas_per_sm > 0 ? L->face_ctas_per_sm : 2),
                                 hf::lc::kTcThreads, sm, L->stream>>>(L->U[L->cur], L->Wp, G, dt, L->Wb, L->P, L->F,
                                                                      L->dF, L->ok, L->rejected, L->maxs, L->derr);
            LCK(cudaStreamWaitEvent(L->side, L->fork, 0));
            plain_flux_kernel<<<blocks_for(nf, 256), 256, 0, L->side>>>(L->U[L->cur], G, dt, L->F);
            LCK(cudaEventRecord(L->join, L->side));
            LCK(cudaStreamWaitEvent(L->stream, L->join, 0));
        }
        LCK(cudaGetLastError());
        if (mask_set) *mask_set = true;
        return HF_OK;
    }
    plain_flux_kernel<<<blocks_for(nf, 256), 256, 0, L->stream>>>(L->U[L->cur], G, dt, L->F);
    if (use_mlp) {
        launch_features(L);
        launch_forward(L, nf, save_acts);
        correction_kernel<<<blocks_for(nf, 256), 256, 0, L->stream>>>(L->Y, L->scale, L->n, L->dF);
    }
    LCK(cudaGetLastError());
    return HF_OK;
}

double max_speed(hf_lc* L) {
    float m = 0.f;
    cudaMemcpy(&m, L->maxs, sizeof m, cudaMemcpyDeviceToHost);
    return m;
}

}  // namespace

extern "C" {

int hf_lc_create(int n, double dx, double gamma, double cfl, int limiter, hf_lc** out) {
    if (!out || n < 4 || n > 8192 || dx <= 0) return HF_ERR_ARG;
    hf_lc* L = new hf_lc();
    *out = L;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return lfail(L, HF_ERR_NO_DEVICE, "no CUDA device");
    L->n = n; L->dx = dx; L->gamma = gamma; L->cfl = cfl; L->lim = limiter;
    LCK(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking));
    LCK(cudaStreamCreateWithFlags(&L->side, cudaStreamNonBlocking));
    LCK(cudaEventCreateWithFlags(&L->fork, cudaEventDisableTiming));
    LCK(cudaEventCreateWithFlags(&L->join, cudaEventDisableTiming));
    LCK(cudaFuncSetAttribute(hf::lc::face_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)hf::lc::mlp_forward_smem()));
    LCK(cudaFuncSetAttribute(hf::lc::face_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)hf::lc::mlp_forward_smem()));
    LCK(cudaFuncSetAttribute(hf::lc::mlp_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)hf::lc::mlp_forward_smem()));
    LCK(cudaFuncSetAttribute(hf::lc::mlp_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)hf::lc::mlp_backward_smem()));
    for (const void* k : {(const void*)hf::lc::face_kernel<false>, (const void*)hf::lc::face_kernel<true>,
                          (const void*)hf::lc::mlp_forward_kernel})
        LCK(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&L->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || L->sms < 1)
            L->sms = 152;
        L->fit_fwd = mlp_fit((const void*)hf::lc::mlp_forward_kernel);
        L->fit_face[0] = mlp_fit((const void*)hf::lc::face_kernel<false>);
        L->fit_face[1] = mlp_fit((const void*)hf::lc::face_kernel<true>);
    }
    const size_t cells = (size_t)n * n, nf = nfaces(L);
    int r;
    if ((r = alloc(L, &L->U[0], 4 * cells)) || (r = alloc(L, &L->U[1], 4 * cells)) || (r = alloc(L, &L->F, 4 * nf)) ||
        (r = alloc(L, &L->dF, 4 * nf)) || (r = alloc(L, &L->scale, 2 * nf)) || (r = alloc(L, &L->Y, 4 * nf)) ||
        (r = alloc(L, &L->Z1, (size_t)H * nf)) || (r = alloc(L, &L->Z2, (size_t)H * nf)) || (r = alloc(L, &L->dY, 4 * nf)) ||
        (r = alloc(L, &L->T, 4 * cells)) || (r = alloc(L, &L->wv, 4)) || (r = alloc(L, &L->X, (size_t)NIN * nf)) ||
        (r = alloc(L, &L->Wb, (size_t)(H * NIN + H * H + NOUT * H))) || (r = alloc(L, &L->P, (size_t)NPARAM)) ||
        (r = alloc(L, &L->grad, (size_t)NPARAM)) || (r = alloc(L, &L->m1, (size_t)NPARAM)) ||
        (r = alloc(L, &L->m2, (size_t)NPARAM)) || (r = alloc(L, &L->maxs, 4)) || (r = alloc(L, &L->ok, nf)) ||
        (r = alloc(L, &L->rejected, 1)) || (r = alloc(L, &L->loss, 1)) || (r = alloc(L, &L->derr, 1)) ||
        (r = alloc(L, &L->Wp, cells)) || (r = alloc(L, &L->Uc, cells)))
        return r;
    return HF_OK;
}

void hf_lc_destroy(hf_lc* L) {
    if (!L) return;
    if (L->stream) cudaStreamSynchronize(L->stream);
    if (L->side) cudaStreamSynchronize(L->side);
    for (void* p : L->allocs) cudaFree(p);
    if (L->fork) cudaEventDestroy(L->fork);
    if (L->join) cudaEventDestroy(L->join);
    if (L->side) cudaStreamDestroy(L->side);
    if (L->stream) cudaStreamDestroy(L->stream);
    delete L;
}

const char* hf_lc_last_error_message(const hf_lc* L) { return L ? L->err.c_str() : ""; }
int hf_lc_num_params(int* n) { if (!n) return HF_ERR_ARG; *n = NPARAM; return HF_OK; }

int hf_lc_set_params(hf_lc* L, const float* params) {
    if (!L || !params) return HF_ERR_ARG;
    LCK(cudaMemcpy(L->P, params, NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    to_bf16_kernel<<<16, 256, 0, L->stream>>>(L->P, L->Wb);
    LCK(cudaMemsetAsync(L->m1, 0, NPARAM * sizeof(float), L->stream));
    LCK(cudaMemsetAsync(L->m2, 0, NPARAM * sizeof(float), L->stream));
    L->adam_t = 0;
    LCK(cudaStreamSynchronize(L->stream));
    return HF_OK;
}

int hf_lc_get_params(hf_lc* L, float* params) {
    if (!L || !params) return HF_ERR_ARG;
    LCK(cudaStreamSynchronize(L->stream));
    LCK(cudaMemcpy(params, L->P, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return HF_OK;
}

int hf_lc_set_state(hf_lc* L, const float* U) {
    if (!L || !U) return HF_ERR_ARG;
    LCK(cudaStreamSynchronize(L->stream));
    LCK(cudaMemcpy(L->U[L->cur], U, (size_t)4 * L->n * L->n * sizeof(float), cudaMemcpyHostToDevice));
    L->wp_valid = false;
    L->maxs_valid = false;
    return HF_OK;
}

int hf_lc_get_state(hf_lc* L, float* U) {
    if (!L || !U) return HF_ERR_ARG;
    LCK(cudaStreamSynchronize(L->stream));
    LCK(cudaMemcpy(U, L->U[L->cur], (size_t)4 * L->n * L->n * sizeof(float), cudaMemcpyDeviceToHost));
    return HF_OK;
}

// the maximum wave speed of the current state into maxs, unless the last step's update left it
// (the same cells through the same code: the same value)
static int enqueue_max_speed(hf_lc* L) {
    if (L->maxs_valid) return HF_OK;
    // an update with zero fluxes writes U unchanged and forms its maximum
    hf::lc::Grid G = grid(L);
    LCK(cudaMemsetAsync(L->maxs, 0, 4, L->stream));
    LCK(cudaMemsetAsync(L->F, 0, (size_t)4 * nfaces(L) * sizeof(float), L->stream));
    update_kernel<<<blocks_for((long long)L->n * L->n, 256), 256, 0, L->stream>>>(
        L->U[L->cur], L->F, nullptr, nullptr, G, 0.0f, 0.0f, 0, L->U[L->cur ^ 1], L->maxs, nullptr, nullptr);
    LCK(cudaGetLastError());
    L->maxs_valid = true;
    return HF_OK;
}

int hf_lc_cfl_dt(hf_lc* L, double* dt) {
    if (!L || !dt) return HF_ERR_ARG;
    int r = enqueue_max_speed(L);
    if (r) return r;
    LCK(cudaStreamSynchronize(L->stream));
    *dt = L->cfl * L->dx / max_speed(L);
    return HF_OK;
}

// one coarse step with the given dt; use_mlp adds the guarded correction
int hf_lc_step(hf_lc* L, double dt, int use_mlp, int64_t* rejected_cells) {
    hf::TraceRange trace_("hf_lc_step");
    if (!L || dt <= 0) return HF_ERR_ARG;
    hf::lc::Grid G = grid(L);
    bool mask_set = false;
    int r = fluxes(L, (float)dt, use_mlp != 0, false, &mask_set);
    if (r) return r;
    const float rr = (float)(dt / L->dx);
    const int nf = nfaces(L);
    if (!mask_set) {   // else the fused kernel set the mask and zeroed the counters
        LCK(cudaMemsetAsync(L->maxs, 0, 4, L->stream));
        if (use_mlp) {
            LCK(cudaMemsetAsync(L->ok, 1, nf, L->stream));
            LCK(cudaMemsetAsync(L->rejected, 0, 8, L->stream));
        }
    }
    if (use_mlp)
        guard_kernel<<<blocks_for((long long)L->n * L->n, 256), 256, 0, L->stream>>>(
            L->U[L->cur], L->F, L->dF, G, rr, (float)L->bound, L->guard_mode, L->ok, L->rejected,
            L->fused ? L->Uc : nullptr);
    // an MLP step also leaves the primitives of the new state for the next one's features; with
    // the fused kernels the update takes the guard pass's corrected states where no face was
    // rejected (the separate kernels recompute them all: the same values)
    update_kernel<<<blocks_for((long long)L->n * L->n, 256), 256, 0, L->stream>>>(
        L->U[L->cur], L->F, use_mlp ? L->dF : nullptr, use_mlp ? L->ok : nullptr, G, rr, (float)L->bound,
        L->guard_mode, L->U[L->cur ^ 1], L->maxs, use_mlp ? L->Wp : nullptr, use_mlp && L->fused ? L->Uc : nullptr);
    LCK(cudaGetLastError());
    L->cur ^= 1;
    L->wp_valid = use_mlp != 0;
    L->maxs_valid = true;   // the update formed the new state's maximum wave speed
    L->t += dt;
    L->steps += 1;
    if (rejected_cells) {
        unsigned long long v = 0;
        if (use_mlp) LCK(cudaMemcpyAsync(&v, L->rejected, 8, cudaMemcpyDeviceToHost, L->stream));
        LCK(cudaStreamSynchronize(L->stream));
        *rejected_cells = (int64_t)v;
        if (use_mlp) return check_derr(L);
    }
    return HF_OK;
}

// runs until t_end with CFL dt (host loop, one sync per step for dt); returns steps
int hf_lc_run_to(hf_lc* L, double t_end, int use_mlp, int64_t* steps, int64_t* rejected_cells) {
    hf::TraceRange trace_("hf_lc_run_to");
    if (!L) return HF_ERR_ARG;
    // one wait per step: the step's wave-speed maximum (the next dt) and rejection count are read
    // together; the device error word once at the end
    int64_t k = 0, rej = 0;
    int r = enqueue_max_speed(L);
    if (r) return r;
    while (L->t < t_end) {
        float m = 0.0f;
        unsigned long long rc = 0;
        LCK(cudaMemcpyAsync(&m, L->maxs, sizeof m, cudaMemcpyDeviceToHost, L->stream));
        if (use_mlp && k > 0) LCK(cudaMemcpyAsync(&rc, L->rejected, sizeof rc, cudaMemcpyDeviceToHost, L->stream));
        LCK(cudaStreamSynchronize(L->stream));
        rej += (int64_t)rc;
        double dt = L->cfl * L->dx / (double)m;
        // the reference's TimeStep uses 0.2 x CFL for its first 10 calls; a MUSCL-Hancock
        // step makes two (step and predictor), so the first 5 steps are reduced
        if (L->steps < 5) dt *= 0.2;
        if (!(dt > 0.0) || !std::isfinite(dt))
            return lfail(L, HF_ERR_DEVICE, "coarse run stopped advancing (non-positive or non-finite dt)");
        if (L->t + dt > t_end) dt = t_end - L->t;
        r = hf_lc_step(L, dt, use_mlp, nullptr);
        if (r) return r;
        ++k;
    }
    if (use_mlp && k > 0) {
        unsigned long long rc = 0;
        LCK(cudaMemcpyAsync(&rc, L->rejected, sizeof rc, cudaMemcpyDeviceToHost, L->stream));
        LCK(cudaStreamSynchronize(L->stream));
        rej += (int64_t)rc;
    }
    LCK(cudaStreamSynchronize(L->stream));
    if (steps) *steps = k;
    if (rejected_cells) *rejected_cells = rej;
    return check_derr(L);
}

int hf_lc_set_time(hf_lc* L, double t) {
    if (!L) return HF_ERR_ARG;
    L->t = t;
    if (t == 0.0) L->steps = 0;
    return HF_OK;
}
int hf_lc_get_time(hf_lc* L, double* t) { if (!L || !t) return HF_ERR_ARG; *t = L->t; return HF_OK; }
int hf_lc_set_bound(hf_lc* L, double bound) { if (!L || bound <= 0) return HF_ERR_ARG; L->bound = bound; return HF_OK; }
int hf_lc_set_train_guard(hf_lc* L, int on) {
    if (!L) return HF_ERR_ARG;
    L->train_guard = on ? 1 : 0;
    return HF_OK;
}
int hf_lc_set_fused(hf_lc* L, int fused, int ctas_per_sm) {
    if (!L || fused < 0 || fused > 2 || ctas_per_sm < 0 || ctas_per_sm > 4) return HF_ERR_ARG;
    L->fused = fused;
    L->face_ctas_per_sm = ctas_per_sm;
    return HF_OK;
}
int hf_lc_set_guard_mode(hf_lc* L, int mode) {
    if (!L || mode < 0 || mode > 1) return HF_ERR_ARG;
    L->guard_mode = mode;
    return HF_OK;
}

// One training iteration on the pair (U0, T) with step dt: forward (plain + MLP, no guard),
// loss and dL/dY, backward, Adam.  U0/T are host arrays [4][n][n] (U0 null: the solver's
// current state, left unchanged); w = 4 variable weights.
int hf_lc_train_step(hf_lc* L, const float* U0, const float* T, const float* w, double dt, double lr,
                     double* loss) {
    if (!L || !T || !w || dt <= 0) return HF_ERR_ARG;
    L->maxs_valid = false;   // the training update forms the maximum of its prediction, not of U[cur]
    const size_t bytes = (size_t)4 * L->n * L->n * sizeof(float);
    const int nf = nfaces(L);
    hf::lc::Grid G = grid(L);
    if (U0) {
        LCK(cudaMemcpyAsync(L->U[L->cur], U0, bytes, cudaMemcpyHostToDevice, L->stream));
        L->wp_valid = false;
    }
    LCK(cudaMemcpyAsync(L->T, T, bytes, cudaMemcpyHostToDevice, L->stream));
    LCK(cudaMemcpyAsync(L->wv, w, 4 * sizeof(float), cudaMemcpyHostToDevice, L->stream));
    int r = fluxes(L, (float)dt, true, true);
    if (r) return r;
    const float rr = (float)(dt / L->dx);
    if (L->train_guard) {   // the guard of inference: rejected faces take the plain flux
        LCK(cudaMemsetAsync(L->ok, 1, nf, L->stream));
        LCK(cudaMemsetAsync(L->rejected, 0, 8, L->stream));
        guard_kernel<<<blocks_for((long long)L->n * L->n, 256), 256, 0, L->stream>>>(
            L->U[L->cur], L->F, L->dF, G, rr, (float)L->bound, L->guard_mode, L->ok, L->rejected, nullptr);
        update_kernel<<<blocks_for((long long)L->n * L->n, 256), 256, 0, L->stream>>>(
            L->U[L->cur], L->F, L->dF, L->ok, G, rr, (float)L->bound, L->guard_mode, L->U[L->cur ^ 1], L->maxs,
            nullptr, nullptr);
    } else {
        update_kernel<<<blocks_for((long long)L->n * L->n, 256), 256, 0, L->stream>>>(
            L->U[L->cur], L->F, L->dF, nullptr, G, rr, 0.0f, 0, L->U[L->cur ^ 1], L->maxs, nullptr, nullptr);
    }
    LCK(cudaMemsetAsync(L->loss, 0, 8, L->stream));
    loss_grad_kernel<<<blocks_for(nf, 256), 256, 0, L->stream>>>(L->U[L->cur ^ 1], L->T, L->scale, L->n, rr, L->wv,
                                                                  L->train_guard ? L->ok : nullptr, L->dY, L->loss);
    LCK(cudaMemsetAsync(L->grad, 0, NPARAM * sizeof(float), L->stream));
    launch_backward(L, nf);
    L->adam_t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)L->adam_t), c2 = 1.f - powf(b2, (float)L->adam_t);
    adam_kernel<<<16, 256, 0, L->stream>>>(L->P, L->grad, L->m1, L->m2, L->Wb, (float)lr, b1, b2, 1e-8f, c1, c2);
    to_bf16_kernel<<<16, 256, 0, L->stream>>>(L->P, L->Wb);
    LCK(cudaGetLastError());
    if (loss) {
        LCK(cudaMemcpyAsync(loss, L->loss, 8, cudaMemcpyDeviceToHost, L->stream));
    }
    LCK(cudaStreamSynchronize(L->stream));
    return check_derr(L);
}

// ---- test entry points: the MLP alone on given inputs ----
int hf_lc_features(hf_lc* L, uint16_t* x_bf16, float* scale) {
    if (!L || !x_bf16 || !scale) return HF_ERR_ARG;
    const size_t nf = nfaces(L);
    launch_features(L);
    LCK(cudaGetLastError());
    LCK(cudaMemcpyAsync(x_bf16, L->X, nf * NIN * 2, cudaMemcpyDeviceToHost, L->stream));
    LCK(cudaMemcpyAsync(scale, L->scale, nf * 2 * sizeof(float), cudaMemcpyDeviceToHost, L->stream));
    LCK(cudaStreamSynchronize(L->stream));
    return HF_OK;
}

int hf_lc_mlp_forward(hf_lc* L, const uint16_t* x_bf16, int nf, float* y) {
    if (!L || !x_bf16 || !y || nf < 1 || nf > nfaces(L)) return HF_ERR_ARG;
    LCK(cudaMemcpy(L->X, x_bf16, (size_t)nf * NIN * 2, cudaMemcpyHostToDevice));
    launch_forward(L, nf, true);
    LCK(cudaGetLastError());
    LCK(cudaStreamSynchronize(L->stream));
    LCK(cudaMemcpy(y, L->Y, (size_t)nf * 4 * sizeof(float), cudaMemcpyDeviceToHost));
    return check_derr(L);
}

int hf_lc_mlp_backward(hf_lc* L, const uint16_t* x_bf16, const float* dy, int nf, float* grad) {
    if (!L || !x_bf16 || !dy || !grad || nf < 1 || nf > nfaces(L)) return HF_ERR_ARG;
    LCK(cudaMemcpy(L->X, x_bf16, (size_t)nf * NIN * 2, cudaMemcpyHostToDevice));
    launch_forward(L, nf, true);
    LCK(cudaMemcpyAsync(L->dY, dy, (size_t)nf * 4 * sizeof(float), cudaMemcpyHostToDevice, L->stream));
    LCK(cudaMemsetAsync(L->grad, 0, NPARAM * sizeof(float), L->stream));
    launch_backward(L, nf);
    LCK(cudaGetLastError());
    LCK(cudaStreamSynchronize(L->stream));
    LCK(cudaMemcpy(grad, L->grad, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return check_derr(L);
}

int hf_lc_stream(hf_lc* L, void** s) { if (!L || !s) return HF_ERR_ARG; *s = (void*)L->stream; return HF_OK; }

}  // extern "C"
