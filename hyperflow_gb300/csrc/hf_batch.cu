// Batched single-block cases: hundreds of independent, all-transmissive cases of different
// sizes advanced together by one persistent cooperative kernel per run of steps, captured in a
// CUDA graph, each case with its own CFL dt.  C ABI in include/hyperflow_gb300_batch.h.
//
// Each case is the reference's single-block MUSCL-Hancock step
// (src/fvm_2d_cart/scheme/muscl_hancock/muscl_hancock.cpp:41-376 + TimeStep +
// ForwardEuler) or Godunov step (src/fvm_2d_cart/scheme/godunov/godunov.cpp:27-118 + TimeStep +
// ForwardEuler); all cases of a batch use the same scheme.  With transmissive boundaries on all
// four sides every ghost value is a mirror copy of an interior value
// (transmissive_boundary.cpp:25-104; the fill order makes corner ghosts mirror in x and in y).
// So the tile loader reads the mirrored interior cell directly and the state is stored without
// ghosts, and the CFL maximum over ghost cells equals the maximum over the interior.  A single
// small case (the 256^2 Godunov quadrant problem) runs as a batch of one: its whole run of steps
// is one launch, with no per-step launch chain.
//
// Work decomposition: every case is cut into TX x TY tiles; the tiles of all cases form
// one list that the persistent CTAs walk round-robin.  A step ends at a grid barrier
// (bounded wait; a timeout raises the error word and stops the kernel).  The CFL maxima
// rotate through three slots per case: read (this step's dt), write (the next step's, by
// the update epilogue), and cleared (for the step after).
//
// Autotuning: the tile shape, threads per CTA and the number of halo staging buffers
// (1 = load then compute; 2 = the next tile's halo is fetched with cp.async while the
// current tile computes) come from a small set of compiled configurations; the autotuner
// times each on the real batch and keeps the fastest.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/hyperflow_gb300_batch.h"
#include "hf_cart.h"
#include "hf_device.cuh"
#include "hf_trace.h"
#include "hf_godunov_tile.cuh"
#include "hf_mh_tile.cuh"

namespace hf {

struct BatchInst {
    int n;                 // cells per side
    int pitch;             // doubles per row: n rounded up to even (a TMA row stride is a multiple of 16 bytes)
    long long off;         // offset (doubles) of the case's [4][n][pitch] state
    double dx, dy;
};

struct BatchCtrl {
    double gamma, g1, cfl;
    long long calls;        // TimeStep calls made by every case so far
    long long step;         // steps completed
    int limiter;
    int scheme;             // 0 Godunov, 1 MUSCL-Hancock
    int ninst;
    int err;
    unsigned int bar_count;
    unsigned int bar_gen;
    long long hllc_errors;
    unsigned long long first_nonpos;   // least batch_key of a cell a step left with density or
                                       // pressure not positive, ~0 when none
};

// Key of a cell for the earliest non-positive record: the step (24 bits, saturating), then the
// cell's offset in the batch state (40 bits: the case's offset + j * n + i), which orders by case,
// row, column.
__device__ __forceinline__ unsigned long long batch_key(long long step, long long off) {
    const unsigned long long s = step > 0xFFFFFFll ? 0xFFFFFFull : (unsigned long long)step;
    return (s << 40) | ((unsigned long long)off & 0xFFFFFFFFFFull);
}

struct BatchDev {
    BatchCtrl* ctrl;
    const BatchInst* inst;
    const CUtensorMap* maps;       // MUSCL-Hancock: per state parity, per case, [2][ninst]
    int ninst;
    const int* tile_inst;
    const int* tile_xy;            // x0 | (y0 << 16), interior cells
    long long ntiles;
    double* U[2];
    unsigned long long* acc;       // [3][ninst][2]
    double* t;                     // [ninst]
    double* last_dt;               // [ninst]
};

__device__ __forceinline__ unsigned long long gtimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// grid-wide barrier with a bounded wait (10 s); false after a timeout
__device__ bool grid_barrier(BatchCtrl* c) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* gen = &c->bar_gen;
        const unsigned int g0 = *gen;
        __threadfence();
        const unsigned int arrived = atomicAdd(&c->bar_count, 1u) + 1u;
        if (arrived == gridDim.x) {
            c->bar_count = 0u;
            __threadfence();
            atomicAdd(&c->bar_gen, 1u);
            ok = 1;
        } else {
            ok = 0;
            const unsigned long long t0 = gtimer_ns();
            for (;;) {
                if (*gen != g0) { ok = 1; break; }
                if (c->err != 0) break;
                if (gtimer_ns() - t0 > 10000000000ull) {
                    atomicCAS(&c->err, 0, HF_DEV_TIMEOUT);
                    break;
                }
                __nanosleep(128);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

__device__ __forceinline__ int mirror(int x, int n) {
    x = x < 0 ? -1 - x : (x >= n ? 2 * n - 1 - x : x);
    return x < 0 ? 0 : (x >= n ? n - 1 : x);   // positions past the 2-cell halo are never used
}

constexpr unsigned kBatchWaitLimit = 1u << 22;   // bounded mbarrier polls before giving up

__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// shared-memory tiles of the two schemes: halo H cells, the staged state, the scratch after it
template <int SCHEME, int TX, int TY>
struct BatchTile;
template <int TX, int TY>
struct BatchTile<0, TX, TY> {   // Godunov: 1-cell halo; per-cell primitives/fluxes, face fluxes
    using T = GoTile<TX, TY>;
    static constexpr int H = 1, UX = T::UX, UY = T::UY, U_SIZE = T::U_SIZE;
    static constexpr int WORK = T::Q_SIZE + T::F_SIZE + T::G_SIZE;
};
template <int TX, int TY>
struct BatchTile<1, TX, TY> {   // MUSCL-Hancock: 2-cell halo; evolved states, face fluxes
    using T = MhTile<TX, TY>;
    static constexpr int H = 2, UX = T::UX, UY = T::UY, U_SIZE = T::U_SIZE;
    static constexpr int WORK = T::A_SIZE + T::F_SIZE + T::G_SIZE;
};

// stage tile `t`'s state + mirrored halo into sU (cp.async, one commit group)
template <int SCHEME, int TX, int TY, int NT>
__device__ __forceinline__ void stage_tile(const BatchDev& d, const double* __restrict__ U, long long t,
                                           double* sU) {
    using T = BatchTile<SCHEME, TX, TY>;
    const int inst = d.tile_inst[t];
    const int xy = d.tile_xy[t];
    const int x0 = xy & 0xffff, y0 = xy >> 16;
    const BatchInst I = d.inst[inst];
    const double* __restrict__ base = U + I.off;
    const size_t plane = (size_t)I.pitch * I.n;
    for (int k = threadIdx.x; k < T::U_SIZE; k += NT) {
        const int v = k / (T::UY * T::UX);
        const int r = k - v * (T::UY * T::UX);
        const int ly = r / T::UX, lx = r - ly * T::UX;
        const int gx = mirror(x0 + lx - T::H, I.n), gy = mirror(y0 + ly - T::H, I.n);
        cp_async8(sU + k, base + v * plane + (size_t)gy * I.pitch + gx);
    }
    cp_async_commit();
}

// MUSCL-Hancock tiles by TMA: one 3-D box (the tile and its 2-cell halo, all four variables) of
// the case's state per tile, issued by thread 0 on `bar`; positions outside the case arrive as
// zeros and mirror_halo then writes the transmissive ghosts there.  (The box's x start, x0 - 2, is
// even, as a TMA copy of FP64 needs; Godunov's 1-cell halo would start at an odd x, so Godunov
// batches keep the element-wise loader.)
template <int TX, int TY>
__device__ __forceinline__ void tma_tile(const BatchDev& d, int p, long long t, double* sU, uint64_t* bar) {
    using T = BatchTile<1, TX, TY>;
    const int inst = d.tile_inst[t];
    const int xy = d.tile_xy[t];
    const int x0 = xy & 0xffff, y0 = xy >> 16;
    // the previous tile's reads and writes of this buffer (generic proxy) come before the copy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, T::U_SIZE * 8);
    tma_load_3d(sU, &d.maps[(size_t)p * d.ninst + inst], bar, x0 - T::H, y0 - T::H, 0);
}

// The halo positions outside the case (within 2 cells of it) take the mirrored interior values,
// the transmissive ghosts (transmissive_boundary.cpp:25-104; corners mirrored in x and in y).
// Every source is an interior cell inside the same box.  Positions further out are never read.
template <int TX, int TY, int NT>
__device__ __forceinline__ void mirror_halo(double* sU, int x0, int y0, int n) {
    using T = BatchTile<1, TX, TY>;
    constexpr int H = T::H;
    if (x0 >= H && y0 >= H && x0 + TX + H <= n && y0 + TY + H <= n) return;   // the box lies inside the case
    for (int k = threadIdx.x; k < T::U_SIZE; k += NT) {
        const int v = k / (T::UY * T::UX);
        const int r = k - v * (T::UY * T::UX);
        const int ly = r / T::UX, lx = r - ly * T::UX;
        const int gx = x0 + lx - H, gy = y0 + ly - H;
        if (gx >= 0 && gx < n && gy >= 0 && gy < n) continue;
        if (gx < -H || gy < -H || gx >= n + H || gy >= n + H) continue;
        const int sx = mirror(gx, n) - x0 + H, sy = mirror(gy, n) - y0 + H;
        sU[k] = sU[(v * T::UY + sy) * T::UX + sx];
    }
}

template <int SCHEME, int TX, int TY, int NT, int STAGES, int MINB>
__global__ void __launch_bounds__(NT, MINB) batch_kernel(BatchDev d, int nsteps) {
    using BT = BatchTile<SCHEME, TX, TY>;
    constexpr int CALLS = SCHEME == 1 ? 2 : 1;   // TimeStep calls per step (+ the predictor's)
    extern __shared__ __align__(1024) double smem[];
    double* sUb[STAGES];
#pragma unroll
    for (int k = 0; k < STAGES; ++k) sUb[k] = smem + k * BT::U_SIZE;
    double* sW = smem + STAGES * BT::U_SIZE;   // MUSCL-Hancock: sA; Godunov: sQ
    double* sF = sW + (SCHEME == 1 ? MhTile<TX, TY>::A_SIZE : GoTile<TX, TY>::Q_SIZE);
    double* sG = sF + (SCHEME == 1 ? MhTile<TX, TY>::F_SIZE : GoTile<TX, TY>::F_SIZE);
    __shared__ double sdt[5];

    BatchCtrl* c = d.ctrl;
    const long long step0 = c->step, calls0 = c->calls;
    const double g = c->gamma, g1 = c->g1, cfl = c->cfl;
    const int lim = c->limiter, ninst = c->ninst;
    int herr = 0;
    // MUSCL-Hancock: one mbarrier per staging buffer for the TMA loads, and its phase
    __shared__ uint64_t tbar[2];
    uint32_t tph[2] = {0u, 0u};
    bool failed = false;
    if (SCHEME == 1) {
        if (threadIdx.x == 0) {
            mbar_init(&tbar[0], 1);
            mbar_init(&tbar[1], 1);
        }
        __syncthreads();
    }

    for (int s = 0; s < nsteps; ++s) {
        const long long step = step0 + s;
        const int p = (int)(step & 1);
        const int ar = (int)(step % 3), aw = (int)((step + 1) % 3), az = (int)((step + 2) % 3);
        const long long calls = calls0 + CALLS * s;
        const double m0 = (calls + 1 <= 10) ? 0.2 * cfl : cfl;        // step TimeStep call
        const double m1 = (calls + 2 <= 10) ? 0.2 * cfl : cfl;        // predictor call
        for (int i = blockIdx.x * NT + threadIdx.x; i < 2 * ninst; i += gridDim.x * NT)
            d.acc[(size_t)az * 2 * ninst + i] = 0ull;
        const double* __restrict__ U = d.U[p];
        double* __restrict__ Un = d.U[p ^ 1];
        long long t = blockIdx.x;
        if (STAGES == 2 && t < d.ntiles) {
            if (SCHEME == 1) {
                if (threadIdx.x == 0) tma_tile<TX, TY>(d, p, t, sUb[0], &tbar[0]);
            } else {
                stage_tile<SCHEME, TX, TY, NT>(d, U, t, sUb[0]);
            }
        }
        int buf = 0;
        for (; t < d.ntiles; t += gridDim.x) {
            double* sU = sUb[STAGES == 2 ? buf : 0];
            const int sb = STAGES == 2 ? buf : 0;   // this tile's staging buffer and mbarrier
            if (SCHEME == 1) {
                if (threadIdx.x == 0) {
                    if (STAGES == 1) tma_tile<TX, TY>(d, p, t, sU, &tbar[0]);
                    else if (t + gridDim.x < d.ntiles) tma_tile<TX, TY>(d, p, t + gridDim.x, sUb[buf ^ 1], &tbar[buf ^ 1]);
                }
                const bool ok = mbar_wait_bounded(&tbar[sb], tph[sb], kBatchWaitLimit);
                if (__syncthreads_or(!ok)) {
                    failed = true;
                    break;
                }
                tph[sb] ^= 1u;
            } else if (STAGES == 1) {
                stage_tile<SCHEME, TX, TY, NT>(d, U, t, sU);
                cp_async_wait<0>();
            } else {
                const long long tn = t + gridDim.x;
                if (tn < d.ntiles) {
                    stage_tile<SCHEME, TX, TY, NT>(d, U, tn, sUb[buf ^ 1]);
                    cp_async_wait<1>();
                } else {
                    cp_async_wait<0>();
                }
            }
            const int inst = d.tile_inst[t];
            const int xy = d.tile_xy[t];
            const int x0 = xy & 0xffff, y0 = xy >> 16;
            const BatchInst I = d.inst[inst];
            if (SCHEME == 1) mirror_halo<TX, TY, NT>(sU, x0, y0, I.n);
            __syncthreads();
            if (threadIdx.x == 0) {
                // TimeStep::operator() for this case (timestep.cpp:29-68) from last step's maxima
                const unsigned long long* a = d.acc + ((size_t)ar * ninst + inst) * 2;
                // (divisions on the integer pipes: the same correctly rounded quotients, without
                // the FP64 pipe's Newton sequences on one thread while the CTA waits)
                const double dtx = smin(1e16, div_rn(I.dx, bitsd(a[0])));
                const double dty = smin(1e16, div_rn(I.dy, bitsd(a[1])));
                sdt[0] = m0 * smin(dtx, dty);
                if (SCHEME == 1) {
                    const double dtp = m1 * smin(dtx, dty);
                    sdt[1] = div_rn(0.5 * dtp, I.dx);   // muscl_hancock.cpp:248-249
                    sdt[2] = div_rn(0.5 * dtp, I.dy);
                }
                sdt[3] = div_rn(1.0, I.dx);             // muscl_hancock.cpp:352-353, godunov.cpp:97-98
                sdt[4] = div_rn(1.0, I.dy);
            }
            __syncthreads();
            const double dt = sdt[0], hdx = sdt[1], hdy = sdt[2], one_dx = sdt[3], one_dy = sdt[4];
            if (SCHEME == 0)
                herr += go_tile_fluxes<TX, TY, NT>(sU, sW, sF, sG, g, g1, x0, y0, I.n, I.n);
            else if (lim == 0)
                herr += mh_tile_fluxes<TX, TY, NT, 0>(sU, sW, sF, sG, g, g1, hdx, hdy, x0, y0, I.n, I.n);
            else
                herr += mh_tile_fluxes<TX, TY, NT, 1>(sU, sW, sF, sG, g, g1, hdx, hdy, x0, y0, I.n, I.n);
            double mx = 0.0, my = 0.0;
            double* __restrict__ out = Un + I.off;
            const size_t plane = (size_t)I.pitch * I.n;
            for (int it = threadIdx.x; it < TX * TY; it += NT) {
                const int ox = it % TX, oy = it / TX;
                const int gx = x0 + ox, gy = y0 + oy;
                if (gx < I.n && gy < I.n) {
                    double un[4];
#pragma unroll
                    for (int v = 0; v < 4; ++v) {
                        un[v] = SCHEME == 0 ? go_update<TX, TY>(sU, sF, sG, v, ox, oy, dt, one_dx, one_dy)
                                            : mh_update<TX, TY>(sU, sF, sG, v, ox, oy, dt, one_dx, one_dy);
                        out[v * plane + (size_t)gy * I.pitch + gx] = un[v];
                    }
                    double sx, sy;
                    if (!wave_terms(g, g1, un[0], un[1], un[2], un[3], sx, sy))
                        atomicMin(&c->first_nonpos, batch_key(step, I.off + (long long)gy * I.pitch + gx));
                    mx = nmax(mx, sx);
                    my = nmax(my, sy);
                }
            }
            unsigned long long* aw_p = d.acc + ((size_t)aw * ninst + inst) * 2;
            block_max2_atomic<NT>(mx, my, aw_p, aw_p + 1);
            if (x0 == 0 && y0 == 0 && threadIdx.x == 0) {
                d.t[inst] = d.t[inst] + dt;
                d.last_dt[inst] = dt;
            }
            __syncthreads();   // smem reuse by the next tile
            buf ^= 1;
        }
        if (failed) {
            if (threadIdx.x == 0) {
                atomicCAS(&c->err, 0, (int)HF_DEV_TIMEOUT);
                // let the copies in flight land before the CTA's shared memory goes
                for (int k = 0; k < 2; ++k) mbar_wait_bounded(&tbar[k], tph[k], kBatchWaitLimit);
            }
            __syncthreads();
            break;
        }
        if (!grid_barrier(c)) break;
    }
    if (herr) atomicAdd(reinterpret_cast<unsigned long long*>(&c->hllc_errors), (unsigned long long)herr);
    if (blockIdx.x == 0 && threadIdx.x == 0 && c->err == 0) {
        c->step = step0 + nsteps;
        c->calls = calls0 + CALLS * nsteps;
    }
}

// CFL maxima of the current state, into slot step % 3 (after an upload)
template <int TX, int TY, int NT>
__global__ void __launch_bounds__(NT) batch_cfl_kernel(BatchDev d) {
    BatchCtrl* c = d.ctrl;
    const long long step = c->step;
    const int p = (int)(step & 1), ar = (int)(step % 3);
    const long long t = blockIdx.x;
    const int inst = d.tile_inst[t];
    const int xy = d.tile_xy[t];
    const int x0 = xy & 0xffff, y0 = xy >> 16;
    const BatchInst I = d.inst[inst];
    const double* U = d.U[p] + I.off;
    const size_t plane = (size_t)I.pitch * I.n;
    double mx = 0.0, my = 0.0;
    for (int it = threadIdx.x; it < TX * TY; it += NT) {
        const int gx = x0 + it % TX, gy = y0 + it / TX;
        if (gx < I.n && gy < I.n) {
            const size_t o = (size_t)gy * I.pitch + gx;
            double sx, sy;
            wave_terms(c->gamma, c->g1, U[o], U[plane + o], U[2 * plane + o], U[3 * plane + o], sx, sy);
            mx = nmax(mx, sx);
            my = nmax(my, sy);
        }
    }
    unsigned long long* a = d.acc + ((size_t)ar * c->ninst + inst) * 2;
    block_max2_atomic<NT>(mx, my, a, a + 1);
}

struct BatchConfig {
    int tx, ty, threads, stages, min_ctas_per_sm;
};

// tile shape, threads, halo staging buffers, CTAs per SM the registers are budgeted for
// (the last, 32x4 tiles of 128 threads at four CTAs per SM, is for batches too small to give
// every SM several large tiles per step, such as a single 256^2 case)
constexpr BatchConfig kConfigs[] = {{32, 14, 256, 1, 2}, {32, 14, 256, 2, 2}, {32, 16, 256, 1, 2},
                                    {32, 12, 256, 1, 3}, {32, 12, 256, 2, 2}, {32, 4, 128, 1, 4}};
constexpr int kNumConfigs = 6;

template <int SCHEME, int TX, int TY, int ST>
size_t batch_smem() {
    using T = BatchTile<SCHEME, TX, TY>;
    return (size_t)(ST * T::U_SIZE + T::WORK) * 8;
}

template <int SCHEME, int TX, int TY, int NT, int ST, int MINB>
cudaError_t launch_batch(const BatchDev& d, int nsteps, int sms, cudaStream_t s, bool cfl_only) {
    auto k = batch_kernel<SCHEME, TX, TY, NT, ST, MINB>;
    const size_t smem = batch_smem<SCHEME, TX, TY, ST>();
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (cfl_only) {
        batch_cfl_kernel<TX, TY, NT><<<(unsigned)d.ntiles, NT, 0, s>>>(d);
        return cudaGetLastError();
    }
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, NT, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    long long grid = (long long)per_sm * sms;
    if (grid > d.ntiles) grid = d.ntiles;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;   // all CTAs co-resident: the grid barrier is safe
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, d, nsteps);
}

template <int SCHEME>
cudaError_t launch_scheme_config(int k, const BatchDev& d, int nsteps, int sms, cudaStream_t s, bool cfl_only) {
    switch (k) {
        case 0: return launch_batch<SCHEME, 32, 14, 256, 1, 2>(d, nsteps, sms, s, cfl_only);
        case 1: return launch_batch<SCHEME, 32, 14, 256, 2, 2>(d, nsteps, sms, s, cfl_only);
        case 2: return launch_batch<SCHEME, 32, 16, 256, 1, 2>(d, nsteps, sms, s, cfl_only);
        case 3: return launch_batch<SCHEME, 32, 12, 256, 1, 3>(d, nsteps, sms, s, cfl_only);
        case 4: return launch_batch<SCHEME, 32, 12, 256, 2, 2>(d, nsteps, sms, s, cfl_only);
        default: return launch_batch<SCHEME, 32, 4, 128, 1, 4>(d, nsteps, sms, s, cfl_only);
    }
}

cudaError_t launch_batch_config(int k, int scheme, const BatchDev& d, int nsteps, int sms, cudaStream_t s,
                                bool cfl_only) {
    return scheme == 0 ? launch_scheme_config<0>(k, d, nsteps, sms, s, cfl_only)
                       : launch_scheme_config<1>(k, d, nsteps, sms, s, cfl_only);
}

}  // namespace hf

// =====================================================================================
// host side
// =====================================================================================
struct hf_batch {
    cudaStream_t stream = nullptr;
    int sms = 0;
    double gamma = 1.4, cfl = 0.8;
    int limiter = 0;
    int scheme = 1;             // 0 Godunov, 1 MUSCL-Hancock
    std::vector<hf::BatchInst> inst;
    long long total_cells = 0;
    long long total_doubles = 0;   // the state buffer: every case's [4][n][pitch]
    std::vector<void*> allocs;
    hf::BatchCtrl* dctrl = nullptr;
    hf::BatchInst* dinst = nullptr;
    double* U[2] = {nullptr, nullptr};
    unsigned long long* acc = nullptr;
    double* t = nullptr;
    double* last_dt = nullptr;
    // per configuration: device tile lists
    int* tile_inst[hf::kNumConfigs] = {};
    int* tile_xy[hf::kNumConfigs] = {};
    long long ntiles[hf::kNumConfigs] = {};
    CUtensorMap* maps[hf::kNumConfigs] = {};   // MUSCL-Hancock: the TMA maps of the config's tile box
    int config = 0;
    // graphs: key = (config, nsteps)
    struct G { int config; long long nsteps; cudaGraphExec_t exec; };
    std::vector<G> graphs;
    std::string err;
};

namespace {

int bfail(hf_batch* b, int code, const std::string& m) {
    if (b) b->err = m;
    return code;
}

#define BCK(call)                                                                              \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return bfail(b, HF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
    } while (0)

int ensure_tiles(hf_batch* b, int k) {
    if (b->tile_inst[k]) return HF_OK;
    const hf::BatchConfig C = hf::kConfigs[k];
    std::vector<int> ti, txy;
    for (size_t i = 0; i < b->inst.size(); ++i) {
        const int n = b->inst[i].n;
        for (int y0 = 0; y0 < n; y0 += C.ty)
            for (int x0 = 0; x0 < n; x0 += C.tx) {
                ti.push_back((int)i);
                txy.push_back(x0 | (y0 << 16));
            }
    }
    BCK(cudaMalloc(&b->tile_inst[k], ti.size() * sizeof(int)));
    BCK(cudaMalloc(&b->tile_xy[k], txy.size() * sizeof(int)));
    b->allocs.push_back(b->tile_inst[k]);
    b->allocs.push_back(b->tile_xy[k]);
    BCK(cudaMemcpy(b->tile_inst[k], ti.data(), ti.size() * sizeof(int), cudaMemcpyHostToDevice));
    BCK(cudaMemcpy(b->tile_xy[k], txy.data(), txy.size() * sizeof(int), cudaMemcpyHostToDevice));
    b->ntiles[k] = (long long)ti.size();
    return HF_OK;
}

// The TMA maps of configuration k (MUSCL-Hancock batches): per state parity and case, the case's
// [4][n][pitch] state as a 3-D tensor {n, n, 4} with the box of the config's tile and its 2-cell halo.
int ensure_maps(hf_batch* b, int k) {
    if (b->scheme != 1 || b->maps[k]) return HF_OK;
    const hf::BatchConfig C = hf::kConfigs[k];
    hf::EncodeTiledFn enc = hf::tensor_map_encoder();
    if (!enc) return bfail(b, HF_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    const size_t n = b->inst.size();
    std::vector<CUtensorMap> maps(2 * n);
    for (int par = 0; par < 2; ++par)
        for (size_t i = 0; i < n; ++i) {
            const hf::BatchInst& I = b->inst[i];
            cuuint64_t dims[3] = {(cuuint64_t)I.n, (cuuint64_t)I.n, 4};
            cuuint64_t strides[2] = {(cuuint64_t)I.pitch * 8, (cuuint64_t)I.pitch * I.n * 8};
            cuuint32_t box[3] = {(cuuint32_t)(C.tx + 4), (cuuint32_t)(C.ty + 4), 4};
            cuuint32_t es[3] = {1, 1, 1};
            CUresult r = enc(&maps[par * n + i], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, b->U[par] + I.off, dims, strides,
                             box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS)
                return bfail(b, HF_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
        }
    BCK(cudaMalloc(&b->maps[k], maps.size() * sizeof(CUtensorMap)));
    b->allocs.push_back(b->maps[k]);
    BCK(cudaMemcpy(b->maps[k], maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
    return HF_OK;
}

hf::BatchDev devview(hf_batch* b, int k) {
    hf::BatchDev d{};
    d.ctrl = b->dctrl;
    d.inst = b->dinst;
    d.maps = b->maps[k];
    d.ninst = (int)b->inst.size();
    d.tile_inst = b->tile_inst[k];
    d.tile_xy = b->tile_xy[k];
    d.ntiles = b->ntiles[k];
    d.U[0] = b->U[0];
    d.U[1] = b->U[1];
    d.acc = b->acc;
    d.t = b->t;
    d.last_dt = b->last_dt;
    return d;
}

long long read_step(hf_batch* b) {
    long long s = 0;
    cudaStreamSynchronize(b->stream);
    cudaMemcpy(&s, &b->dctrl->step, sizeof s, cudaMemcpyDeviceToHost);
    return s;
}

// refresh the read slot's CFL maxima from the current state (after an upload)
int refresh_cfl(hf_batch* b) {
    long long step = read_step(b);
    int ar = (int)(step % 3);
    BCK(cudaMemsetAsync(b->acc + (size_t)ar * 2 * b->inst.size(), 0, 2 * b->inst.size() * sizeof(unsigned long long), b->stream));
    int r = ensure_tiles(b, 0);
    if (r) return r;
    BCK(hf::launch_batch_config(0, b->scheme, devview(b, 0), 0, b->sms, b->stream, true));
    BCK(cudaStreamSynchronize(b->stream));
    return HF_OK;
}

int check_device_error(hf_batch* b) {
    int e = 0;
    BCK(cudaStreamSynchronize(b->stream));
    BCK(cudaMemcpy(&e, &b->dctrl->err, sizeof e, cudaMemcpyDeviceToHost));
    if (e) return bfail(b, HF_ERR_DEVICE, "device error word " + std::to_string(e));
    return HF_OK;
}

}  // namespace

extern "C" {

int hf_batch_create(const char* manifest, size_t len, hf_batch** out) {
    using hf::Json;
    if (!manifest || !out) return HF_ERR_ARG;
    hf_batch* b = new hf_batch();
    *out = b;
    std::vector<std::vector<double>> init;
    try {
        Json m = Json::parse(manifest, len);
        const Json& cs = m["cases"];
        if (cs.size() == 0) return bfail(b, HF_ERR_ARG, "manifest has no cases");
        for (size_t i = 0; i < cs.size(); ++i) {
            const Json& c = cs[i];
            if (c["model"]["model"].string() != "EulerIdealGas")
                return bfail(b, HF_ERR_UNSUPPORTED, "model must be EulerIdealGas");
            const Json& sch = c["scheme"];
            const std::string type = sch["type"].string();
            const int S = type == "Godunov" ? 0 : (type == "MUSCLHancock" ? 1 : -1);
            if (S < 0 || sch["riemann"].string() != "HLLCEuler" || sch["ode"].string() != "ForwardEuler")
                return bfail(b, HF_ERR_UNSUPPORTED,
                             "batched cases are Godunov or MUSCL-Hancock + HLLC + forward Euler");
            int L = 0;
            if (S == 1) {
                const std::string lim = sch["limiter"].string();
                L = lim == "MinBee" ? 0 : (lim == "VanLeer" ? 1 : -1);
                if (L < 0) return bfail(b, HF_ERR_UNSUPPORTED, "limiter '" + lim + "' not supported");
            }
            double gamma = c["model"]["gamma"].number(), cfl = c["simulation"]["cfl"].number();
            if (i == 0) { b->gamma = gamma; b->cfl = cfl; b->limiter = L; b->scheme = S; }
            else if (gamma != b->gamma || cfl != b->cfl || L != b->limiter || S != b->scheme)
                return bfail(b, HF_ERR_UNSUPPORTED, "all batched cases share scheme, gamma, cfl and limiter");
            const Json& blocks = c["mesh"]["blocks"];
            if (blocks.size() != 1) return bfail(b, HF_ERR_UNSUPPORTED, "batched cases have one block");
            const Json& blk = blocks[0];
            for (const char* side : {"bottom", "right", "top", "left"})
                if (blk["boundaries"][side]["type"].string() != "Transmissive")
                    return bfail(b, HF_ERR_UNSUPPORTED, "batched cases are transmissive on every side");
            const double cx = blk["x_cells"].number(), cy = blk["y_cells"].number();
            if (!(cx >= 4.0 && cx <= 65535.0) || cx != cy || cx != (double)(int)cx)
                return bfail(b, HF_ERR_UNSUPPORTED, "batched cases are square, 4..65535 cells per side");
            const int nx = (int)cx, ny = (int)cy;
            const Json& ex = blk["extents"];
            double xl = ex["x_left"].number(), xr = ex["x_right"].number();
            double yb = ex["y_bottom"].number(), yt = ex["y_top"].number();
            hf::BatchInst I{};
            I.n = nx;
            I.pitch = nx + (nx & 1);
            I.off = b->total_doubles;
            b->total_doubles += 4LL * I.pitch * nx;
            I.dx = (xr - xl) / nx;   // mesh_block.cpp:227-236
            I.dy = (yt - yb) / ny;
            b->inst.push_back(I);
            b->total_cells += (long long)nx * ny;
            // the centroids depend on the ghost width in floating point (mesh_block.cpp:239-257),
            // so the initial condition is sampled on the scheme's own ghost layout
            const int gh = S == 0 ? 1 : 2;
            std::vector<double> soa;
            hf::BlockGeom G{nx + 2 * gh, ny + 2 * gh, xl, yb, I.dx, I.dy};
            hf::build_initial_state(c["initial_condition"], gamma, G, gh, soa);
            std::vector<double> inner((size_t)4 * nx * ny);
            for (int v = 0; v < 4; ++v)
                for (int j = 0; j < ny; ++j)
                    std::memcpy(&inner[((size_t)v * ny + j) * nx],
                                &soa[((size_t)v * (ny + 2 * gh) + j + gh) * (nx + 2 * gh) + gh], nx * sizeof(double));
            init.push_back(std::move(inner));
        }
    } catch (const std::exception& e) {
        return bfail(b, HF_ERR_PARSE, e.what());
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return bfail(b, HF_ERR_NO_DEVICE, "no CUDA device visible");
    int dev = 0;
    BCK(cudaGetDevice(&dev));
    BCK(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev));
    BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    const size_t n = b->inst.size();
    for (int k = 0; k < 2; ++k) {
        BCK(cudaMalloc(&b->U[k], (size_t)b->total_doubles * sizeof(double)));
        BCK(cudaMemset(b->U[k], 0, (size_t)b->total_doubles * sizeof(double)));
        b->allocs.push_back(b->U[k]);
    }
    BCK(cudaMalloc(&b->acc, 3 * 2 * n * sizeof(unsigned long long)));
    BCK(cudaMalloc(&b->t, n * sizeof(double)));
    BCK(cudaMalloc(&b->last_dt, n * sizeof(double)));
    BCK(cudaMalloc(&b->dinst, n * sizeof(hf::BatchInst)));
    BCK(cudaMalloc(&b->dctrl, sizeof(hf::BatchCtrl)));
    for (void* p : {(void*)b->acc, (void*)b->t, (void*)b->last_dt, (void*)b->dinst, (void*)b->dctrl}) b->allocs.push_back(p);
    BCK(cudaMemset(b->acc, 0, 3 * 2 * n * sizeof(unsigned long long)));
    BCK(cudaMemset(b->t, 0, n * sizeof(double)));
    BCK(cudaMemset(b->last_dt, 0, n * sizeof(double)));
    BCK(cudaMemcpy(b->dinst, b->inst.data(), n * sizeof(hf::BatchInst), cudaMemcpyHostToDevice));
    hf::BatchCtrl C{};
    C.gamma = b->gamma;
    C.g1 = b->gamma - 1.0;
    C.cfl = b->cfl;
    C.limiter = b->limiter;
    C.scheme = b->scheme;
    C.ninst = (int)n;
    C.first_nonpos = ~0ull;
    BCK(cudaMemcpy(b->dctrl, &C, sizeof C, cudaMemcpyHostToDevice));
    for (size_t i = 0; i < n; ++i) {
        const hf::BatchInst& I = b->inst[i];
        BCK(cudaMemcpy2D(b->U[0] + I.off, (size_t)I.pitch * 8, init[i].data(), (size_t)I.n * 8, (size_t)I.n * 8,
                         (size_t)4 * I.n, cudaMemcpyHostToDevice));
    }
    return refresh_cfl(b);
}

void hf_batch_destroy(hf_batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
    for (void* p : b->allocs) cudaFree(p);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

const char* hf_batch_last_error_message(const hf_batch* b) { return b ? b->err.c_str() : ""; }

int hf_batch_sizes(const hf_batch* b, int* ninst, int64_t* total_cells) {
    if (!b) return HF_ERR_ARG;
    if (ninst) *ninst = (int)b->inst.size();
    if (total_cells) *total_cells = b->total_cells;
    return HF_OK;
}

int hf_batch_instance_side(const hf_batch* b, int i, int* n) {
    if (!b || !n || i < 0 || i >= (int)b->inst.size()) return HF_ERR_ARG;
    *n = b->inst[i].n;
    return HF_OK;
}

int hf_batch_num_configs(int* n) {
    if (!n) return HF_ERR_ARG;
    *n = hf::kNumConfigs;
    return HF_OK;
}

int hf_batch_config_info(int k, int* tile_x, int* tile_y, int* threads, int* stages) {
    if (k < 0 || k >= hf::kNumConfigs) return HF_ERR_ARG;
    const hf::BatchConfig C = hf::kConfigs[k];
    if (tile_x) *tile_x = C.tx;
    if (tile_y) *tile_y = C.ty;
    if (threads) *threads = C.threads;
    if (stages) *stages = C.stages;
    return HF_OK;
}

int hf_batch_set_config(hf_batch* b, int k) {
    if (!b || k < 0 || k >= hf::kNumConfigs) return HF_ERR_ARG;
    b->config = k;
    return HF_OK;
}

int hf_batch_run(hf_batch* b, int64_t nsteps, int use_graph) {
    hf::TraceRange trace_("hf_batch_run");
    if (!b || nsteps < 0 || nsteps > (1 << 30)) return HF_ERR_ARG;
    if (nsteps == 0) return HF_OK;
    int r = ensure_tiles(b, b->config);
    if (!r) r = ensure_maps(b, b->config);
    if (r) return r;
    hf::BatchDev d = devview(b, b->config);
    if (!use_graph) {
        BCK(hf::launch_batch_config(b->config, b->scheme, d, (int)nsteps, b->sms, b->stream, false));
        return HF_OK;
    }
    cudaGraphExec_t exec = nullptr;
    for (auto& g : b->graphs)
        if (g.config == b->config && g.nsteps == nsteps) exec = g.exec;
    if (!exec) {
        cudaGraph_t graph;
        BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = hf::launch_batch_config(b->config, b->scheme, d, (int)nsteps, b->sms, b->stream, false);
        cudaError_t e2 = cudaStreamEndCapture(b->stream, &graph);
        if (e != cudaSuccess) return bfail(b, HF_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
        if (e2 != cudaSuccess) return bfail(b, HF_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e2));
        BCK(cudaGraphInstantiate(&exec, graph, 0));
        cudaGraphDestroy(graph);
        b->graphs.push_back({b->config, nsteps, exec});
    }
    BCK(cudaGraphLaunch(exec, b->stream));
    return HF_OK;
}

int hf_batch_sync(hf_batch* b) {
    if (!b) return HF_ERR_ARG;
    return check_device_error(b);
}

int hf_batch_autotune(hf_batch* b, int steps_per_trial, int* best, double* ms_per_step) {
    if (!b || steps_per_trial < 1) return HF_ERR_ARG;
    // trials advance a copy: save the live state, time each configuration, restore
    const size_t bytes = (size_t)b->total_doubles * sizeof(double);
    long long step = read_step(b);
    int p = (int)(step & 1);
    double* save = nullptr;
    BCK(cudaMalloc(&save, bytes));
    std::vector<unsigned long long> acc(3 * 2 * b->inst.size());
    std::vector<double> tt(b->inst.size()), ld(b->inst.size());
    hf::BatchCtrl C;
    BCK(cudaMemcpy(save, b->U[p], bytes, cudaMemcpyDeviceToDevice));
    BCK(cudaMemcpy(acc.data(), b->acc, acc.size() * 8, cudaMemcpyDeviceToHost));
    BCK(cudaMemcpy(tt.data(), b->t, tt.size() * 8, cudaMemcpyDeviceToHost));
    BCK(cudaMemcpy(ld.data(), b->last_dt, ld.size() * 8, cudaMemcpyDeviceToHost));
    BCK(cudaMemcpy(&C, b->dctrl, sizeof C, cudaMemcpyDeviceToHost));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int bestk = -1;
    double bestms = 1e300;
    for (int k = 0; k < hf::kNumConfigs; ++k) {
        int r = ensure_tiles(b, k);
        if (!r) r = ensure_maps(b, k);
        if (r) return r;
        hf::BatchDev d = devview(b, k);
        // warm (first launch pays the shared-memory opt-in), then time
        BCK(hf::launch_batch_config(k, b->scheme, d, 1, b->sms, b->stream, false));
        cudaEventRecord(e0, b->stream);
        BCK(hf::launch_batch_config(k, b->scheme, d, steps_per_trial, b->sms, b->stream, false));
        cudaEventRecord(e1, b->stream);
        int er = check_device_error(b);
        if (er) return er;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        double per = ms / steps_per_trial;
        if (ms_per_step) ms_per_step[k] = per;
        if (per < bestms) { bestms = per; bestk = k; }
        // restore
        BCK(cudaMemcpy(b->U[p], save, bytes, cudaMemcpyDeviceToDevice));
        BCK(cudaMemcpy(b->acc, acc.data(), acc.size() * 8, cudaMemcpyHostToDevice));
        BCK(cudaMemcpy(b->t, tt.data(), tt.size() * 8, cudaMemcpyHostToDevice));
        BCK(cudaMemcpy(b->last_dt, ld.data(), ld.size() * 8, cudaMemcpyHostToDevice));
        BCK(cudaMemcpy(b->dctrl, &C, sizeof C, cudaMemcpyHostToDevice));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(save);
    b->config = bestk;
    if (best) *best = bestk;
    return HF_OK;
}

int hf_batch_get_state(hf_batch* b, int i, double* out) {
    if (!b || !out || i < 0 || i >= (int)b->inst.size()) return HF_ERR_ARG;
    long long step = read_step(b);
    const hf::BatchInst& I = b->inst[i];
    BCK(cudaMemcpy2D(out, (size_t)I.n * 8, b->U[step & 1] + I.off, (size_t)I.pitch * 8, (size_t)I.n * 8,
                     (size_t)4 * I.n, cudaMemcpyDeviceToHost));
    return HF_OK;
}

int hf_batch_set_state(hf_batch* b, int i, const double* in) {
    if (!b || !in || i < 0 || i >= (int)b->inst.size()) return HF_ERR_ARG;
    long long step = read_step(b);
    const hf::BatchInst& I = b->inst[i];
    BCK(cudaMemcpy2D(b->U[step & 1] + I.off, (size_t)I.pitch * 8, in, (size_t)I.n * 8, (size_t)I.n * 8,
                     (size_t)4 * I.n, cudaMemcpyHostToDevice));
    return refresh_cfl(b);
}

int hf_batch_instance_time(hf_batch* b, int i, double* t, double* last_dt) {
    if (!b || i < 0 || i >= (int)b->inst.size()) return HF_ERR_ARG;
    BCK(cudaStreamSynchronize(b->stream));
    if (t) BCK(cudaMemcpy(t, b->t + i, sizeof(double), cudaMemcpyDeviceToHost));
    if (last_dt) BCK(cudaMemcpy(last_dt, b->last_dt + i, sizeof(double), cudaMemcpyDeviceToHost));
    return HF_OK;
}

int hf_batch_counters(hf_batch* b, int64_t* steps, int64_t* calls, int64_t* hllc_errors) {
    if (!b) return HF_ERR_ARG;
    hf::BatchCtrl C;
    BCK(cudaStreamSynchronize(b->stream));
    BCK(cudaMemcpy(&C, b->dctrl, sizeof C, cudaMemcpyDeviceToHost));
    if (steps) *steps = C.step;
    if (calls) *calls = C.calls;
    if (hllc_errors) *hllc_errors = C.hllc_errors;
    return HF_OK;
}

int hf_batch_last_nonpositive_cell(hf_batch* b, int* instance, int* i, int* j, int64_t* step) {
    if (!b) return HF_ERR_ARG;
    unsigned long long k = ~0ull;
    BCK(cudaStreamSynchronize(b->stream));
    BCK(cudaMemcpy(&k, &b->dctrl->first_nonpos, sizeof k, cudaMemcpyDeviceToHost));
    int ci = -1, cj = -1, cx = -1;
    long long st = -1;
    if (k != ~0ull) {
        const long long off = (long long)(k & 0xFFFFFFFFFFull);
        // the case whose state holds that offset (offsets ascend with the case index)
        size_t lo = 0, hi = b->inst.size();
        while (hi - lo > 1) {
            const size_t mid = (lo + hi) / 2;
            (b->inst[mid].off <= off ? lo : hi) = mid;
        }
        const long long rem = off - b->inst[lo].off;
        cx = (int)lo;
        cj = (int)(rem / b->inst[lo].pitch);
        ci = (int)(rem % b->inst[lo].pitch);
        st = (long long)(k >> 40);
    }
    if (instance) *instance = cx;
    if (i) *i = ci;
    if (j) *j = cj;
    if (step) *step = st;
    return HF_OK;
}

int hf_batch_clear_error_cell(hf_batch* b) {
    if (!b) return HF_ERR_ARG;
    const unsigned long long none = ~0ull;
    BCK(cudaMemcpyAsync(&b->dctrl->first_nonpos, &none, sizeof none, cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return HF_OK;
}

int hf_batch_stream(hf_batch* b, void** stream) {
    if (!b || !stream) return HF_ERR_ARG;
    *stream = (void*)b->stream;
    return HF_OK;
}

}  // extern "C"
