// Cartesian time-step kernels for sm_103a.
//
//   bc_fill       ghost/halo fill, Mesh::apply_bcs (src/fvm_2d_cart/mesh/mesh/mesh.cpp:31-39)
//   ghost_cfl     TimeStep over ghost cells + the step dt (timestep.cpp:29-68)
//   interior_cfl  TimeStep terms over interior cells (after a state upload)
//   godunov       fused x/y HLLC + update, GodunovScheme (godunov.cpp:27-118) + ForwardEuler
//   muscl_hancock fused slopes/limiter/predictor/HLLC/update, MUSCLHancockScheme
//                 (muscl_hancock.cpp:41-376) + ForwardEuler, with the next step's TimeStep
//                 terms reduced in the epilogue
//
// Layout: per block, SoA FP64 [var][total_y][pitch] (x contiguous), ghosts included, two
// buffers alternating by step parity.  The stencil CTAs stage one tile plus its halo with a
// single 3-D TMA load (box = tile + 2*ghost in x and y, all four variables) into shared
// memory; halos come from the neighbouring tiles' cells in HBM, never from another CTA.
#include <cstdio>

#include "hf_cart.h"
#include "hf_device.cuh"
#include "hf_godunov_tile.cuh"
#include "hf_mh_tile.cuh"

namespace hf {

constexpr unsigned kWaitLimit = 1u << 22;   // bounded mbarrier polls before giving up

// start of a step: stop at t_end (device loop), clear this step's accumulators
__global__ void step_begin_kernel(Ctrl* __restrict__ c) {
    const int p = (int)(c->step & 1);
    int done = c->clamp && (c->t == c->t_end);
    if (c->strict && (c->first_bad != ~0ull || c->first_nonpos != ~0ull)) done = 1;   // strict mode
    // a step takes at most two frames: pause the loop while the ring lacks room for them
    if (c->clamp && c->frames && c->captured - c->drained > c->ring_slots - 2) done = 1;
    c->done = done;
    c->snap_pre = c->snap_post = 0;
    if (done) return;
    for (int b = 0; b < HF_MAXB; ++b) {
        c->ghost_s[b][0] = c->ghost_s[b][1] = 0ull;
        c->int_s[p ^ 1][b][0] = c->int_s[p ^ 1][b][1] = 0ull;
        c->step_hllc[b] = 0;
        c->step_bad[b] = c->step_nonpos[b] = ~0ull;
    }
    c->ticket = 0u;
    c->tile_ctr = 0u;
    c->bar_count = 0u;
}

// ------------------------------------------------------------------------------------
// TimeStep over the ghost cells; the last CTA forms the step dt
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void ghost_cell_ij(const BlockDev& B, int g, long long k, int& i, int& j) {
    const long long row_cells = (long long)g * B.tx;
    if (k < row_cells) {                      // bottom ghost rows
        j = (int)(k / B.tx); i = (int)(k % B.tx);
    } else if (k < 2 * row_cells) {           // top ghost rows
        k -= row_cells;
        j = B.ty - g + (int)(k / B.tx); i = (int)(k % B.tx);
    } else {                                  // left/right ghost columns of interior rows
        k -= 2 * row_cells;
        j = g + (int)(k / (2 * g));
        int c = (int)(k % (2 * g));
        i = c < g ? c : B.tx - 2 * g + c;
    }
}

constexpr int kRedThreads = 256;

__device__ void form_step_dt(Ctrl* __restrict__ c, int p);

// form_dt = 0: the ghost maxima only (for a predictor TimeStep in a step whose dt the caller gave)
__global__ void __launch_bounds__(kRedThreads) ghost_cfl_kernel(Ctrl* __restrict__ c,
                                                                const MeshDev* __restrict__ m, int form_dt) {
    if (c->done) return;
    const int p = (int)(c->step & 1);
    const double g = c->gamma, g1 = c->g1;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (int b = 0; b < m->nblocks; ++b) {
        const BlockDev& B = m->b[b];
        const size_t plane = (size_t)B.ty * B.pitch;
        const double* __restrict__ U = B.buf[p];
        double mx = 0.0, my = 0.0;
        for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < B.ghost_count;
             k += stride) {
            int i, j;
            ghost_cell_ij(B, m->ghost, k, i, j);
            size_t o = (size_t)j * B.pitch + i;
            if (!hf_in((long long)o, (long long)plane, &c->err)) continue;
            double sx, sy;
            wave_terms(g, g1, U[o], U[plane + o], U[2 * plane + o], U[3 * plane + o], sx, sy);
            mx = nmax(mx, sx);
            my = nmax(my, sy);
        }
        block_max2_atomic<kRedThreads>(mx, my, &c->ghost_s[b][0], &c->ghost_s[b][1]);
        __syncthreads();
    }
    if (form_dt) form_step_dt(c, p);
}

// The last CTA of a ghost-maxima launch to finish forms the step's dt: TimeStep call number
// `calls` over every block (timestep.cpp:29-68), then Simulation::solve's clamps and frame points.
__device__ void form_step_dt(Ctrl* __restrict__ c, int p) {
    __shared__ bool last;
    __threadfence();
    if (threadIdx.x == 0) last = (atomicAdd(&c->ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    volatile Ctrl* vc = c;
    long long call = vc->calls;
    double dt = cfl_dt_fresh(c, call, 0, p, p);
    c->dt_cfl = dt;
    const double t = c->t;
    if (c->clamp && t + dt > c->t_end) dt = c->t_end - t;        // simulation.cpp:88-90
    if (c->clamp && c->frames) {
        const double cur = c->frame_next;
        c->snap_pre = (cur == 0.0);                              // simulation.cpp:93-96
        if ((t + dt > cur) && (cur > 0.0)) dt = cur - t;         // simulation.cpp:98-102
        if (fabs(t - cur) < 1e-12) {                             // simulation.cpp:106-113
            c->snap_post = 1;
            c->frame_next = cur + c->frame_interval;
        }
        c->snap_t = t;
    }
    c->dt = dt;
    c->calls = call + 1;
    c->ticket = 0u;
}

// the block of ghost cell k of the all-blocks enumeration
__device__ __forceinline__ int ghost_block(const MeshDev* __restrict__ m, long long k) {
    int b = 0;
    while (b + 1 < m->nblocks && k >= m->b[b + 1].ghost_off) ++b;
    return b;
}

// Mesh::apply_bcs (mesh.cpp:31-39) for every block in one launch: ghost cell k takes its final
// value from the fill program (a copy of one cell's pre-fill value or of a Dirichlet side's state,
// with the reflective sides' negations: transmissive_boundary.cpp, reflective_boundary.cpp,
// dirichlet_boundary.cpp, internal_boundary.cpp replayed in the reference's order on the host),
// then its TimeStep terms feed the block's ghost maxima.
__global__ void __launch_bounds__(kRedThreads) fill_cfl_kernel(Ctrl* __restrict__ c, const MeshDev* __restrict__ m,
                                                               int form_dt) {
    if (c->done) return;
    const int p = (int)(c->step & 1);
    const double g = c->gamma, g1 = c->g1;
    const int gh = m->ghost;
    const long long total = m->total_ghost;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long k0 = (long long)blockIdx.x * blockDim.x;
    const long long k1 = (k0 + blockDim.x < total ? k0 + blockDim.x : total) - 1;
    int b = -1;
    double sx = 0.0, sy = 0.0;
    if (k < total) {
        b = ghost_block(m, k);
        const BlockDev& B = m->b[b];
        int i, j;
        ghost_cell_ij(B, gh, k - B.ghost_off, i, j);
        const FillOp op = m->fill[k];
        double u[4];
        if (op.kind == 2) {
            const BlockDev& S = m->b[op.block];
#pragma unroll
            for (int v = 0; v < 4; ++v) u[v] = S.bc_state[op.side][v];
        } else {
            const BlockDev& S = m->b[op.block];
            const size_t splane = (size_t)S.ty * S.pitch;
            const double* __restrict__ src = S.buf[op.kind == 0 ? p : p ^ 1];
            if (hf_in(op.src, (long long)splane, &c->err)) {
#pragma unroll
                for (int v = 0; v < 4; ++v) u[v] = src[v * splane + op.src];
            } else {
#pragma unroll
                for (int v = 0; v < 4; ++v) u[v] = 0.0;
            }
        }
        if (op.neg & 1) u[1] = -1.0 * u[1];
        if (op.neg & 2) u[2] = -1.0 * u[2];
        const size_t plane = (size_t)B.ty * B.pitch, o = (size_t)j * B.pitch + i;
        if (hf_in((long long)o, (long long)plane, &c->err)) {
            double* __restrict__ dst = B.buf[p];
#pragma unroll
            for (int v = 0; v < 4; ++v) dst[v * plane + o] = u[v];
        }
        double tx_, ty_;
        wave_terms(g, g1, u[0], u[1], u[2], u[3], tx_, ty_);
        sx = nmax(0.0, tx_);   // NaN terms are skipped, as TimeStep's std::min skips them
        sy = nmax(0.0, ty_);
    }
    // one atomic pair per block this CTA touched (its cells are consecutive in block order)
    const int b0 = ghost_block(m, k0), b1 = ghost_block(m, k1);
    for (int bb = b0; bb <= b1; ++bb)
        block_max2_atomic<kRedThreads>(b == bb ? sx : 0.0, b == bb ? sy : 0.0, &c->ghost_s[bb][0],
                                       &c->ghost_s[bb][1]);
    if (form_dt) form_step_dt(c, p);
}

// the current buffer's ghost cells into the other buffer (after a fill no stencil follows)
__global__ void __launch_bounds__(256) ghost_mirror_kernel(const Ctrl* __restrict__ c, const MeshDev* __restrict__ m) {
    const int p = (int)(c->step & 1);
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m->total_ghost) return;
    const int b = ghost_block(m, k);
    const BlockDev& B = m->b[b];
    int i, j;
    ghost_cell_ij(B, m->ghost, k - B.ghost_off, i, j);
    const size_t plane = (size_t)B.ty * B.pitch, o = (size_t)j * B.pitch + i;
#pragma unroll
    for (int v = 0; v < 4; ++v) B.buf[p ^ 1][v * plane + o] = B.buf[p][v * plane + o];
}

// TimeStep terms over one block's interior (after an upload of new state)
__global__ void __launch_bounds__(kRedThreads) interior_cfl_kernel(Ctrl* __restrict__ c,
                                                                   const MeshDev* __restrict__ m,
                                                                   int b, int parity) {
    const BlockDev& B = m->b[b];
    const int g = m->ghost;
    const size_t plane = (size_t)B.ty * B.pitch;
    const double* __restrict__ U = B.buf[parity];
    const double gm = c->gamma, g1 = c->g1;
    double mx = 0.0, my = 0.0;
    const long long n = (long long)B.nx * B.ny;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        int i = (int)(k % B.nx) + g, j = (int)(k / B.nx) + g;
        size_t o = (size_t)j * B.pitch + i;
        double sx, sy;
        wave_terms(gm, g1, U[o], U[plane + o], U[2 * plane + o], U[3 * plane + o], sx, sy);
        mx = nmax(mx, sx);
        my = nmax(my, sy);
    }
    block_max2_atomic<kRedThreads>(mx, my, &c->int_s[parity][b][0], &c->int_s[parity][b][1]);
}

// A block's whole state ([4][total_y][total_x], ghosts included) read from host memory the GPU
// maps (pinned), written into both buffers, with the TimeStep terms of the interior cells -- the
// upload, buffer copy and interior_cfl of a host-buffer step in one pass over the link.
__global__ void __launch_bounds__(kRedThreads) upload_kernel(Ctrl* __restrict__ c, const MeshDev* __restrict__ m,
                                                             int b, int parity, const double* __restrict__ hin) {
    const BlockDev& B = m->b[b];
    const int g = m->ghost;
    const size_t plane = (size_t)B.ty * B.pitch, hplane = (size_t)B.ty * B.tx;
    double* __restrict__ U0 = B.buf[parity];
    double* __restrict__ U1 = B.buf[parity ^ 1];
    const double gm = c->gamma, g1 = c->g1;
    double mx = 0.0, my = 0.0;
    const long long n = (long long)B.tx * B.ty;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k % B.tx), j = (int)(k / B.tx);
        const size_t o = (size_t)j * B.pitch + i;
        if (!hf_in((long long)o, (long long)plane, &c->err)) continue;
        double u[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) u[v] = __ldcs(&hin[v * hplane + (size_t)k]);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            U0[v * plane + o] = u[v];
            U1[v * plane + o] = u[v];
        }
        if (i >= g && i < B.tx - g && j >= g && j < B.ty - g) {
            double sx, sy;
            wave_terms(gm, g1, u[0], u[1], u[2], u[3], sx, sy);
            mx = nmax(mx, sx);
            my = nmax(my, sy);
        }
    }
    block_max2_atomic<kRedThreads>(mx, my, &c->int_s[parity][b][0], &c->int_s[parity][b][1]);
}

// The ghost cells filled this step into host memory the GPU maps: with the stencil's own host
// stores of the updated cells, the whole block downloaded.
__global__ void __launch_bounds__(256) ghost_store_kernel(Ctrl* __restrict__ c, const MeshDev* __restrict__ m,
                                                          int b, int parity, double* __restrict__ hout) {
    const BlockDev& B = m->b[b];
    const int g = m->ghost;
    const size_t plane = (size_t)B.ty * B.pitch, hplane = (size_t)B.ty * B.tx;
    const double* __restrict__ U = B.buf[parity];    // filled this step; the stencil copies them later
    const long long rows = (long long)g * B.tx;          // cells in the g bottom (or top) rows
    const long long n = 2 * rows + 2LL * g * B.ny;       // + g columns each side of the interior rows
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        int i, j;
        if (k < 2 * rows) {
            const long long r = k < rows ? k : k - rows;
            i = (int)(r % B.tx);
            j = (int)(r / B.tx) + (k < rows ? 0 : B.ty - g);
        } else {
            const long long r = k - 2 * rows;
            const int col = (int)(r % (2 * g));
            j = g + (int)(r / (2 * g));
            i = col < g ? col : B.tx - 2 * g + col;
        }
        const size_t o = (size_t)j * B.pitch + i, h = (size_t)j * B.tx + i;
        if (!hf_in((long long)o, (long long)plane, &c->err) || !hf_in((long long)h, (long long)hplane, &c->err))
            continue;
#pragma unroll
        for (int v = 0; v < 4; ++v) __stcs(&hout[v * hplane + h], U[v * plane + o]);
    }
}

__global__ void set_dt_kernel(Ctrl* c, double dt) { c->dt = dt; }

// Frames of this step into the device ring: the interior of every block, SoA per block,
// packed ([b][var][y][x]); the state before the update is still in buffer `step & 1` and the
// updated one in the other buffer until finalize flips the parity.
__global__ void __launch_bounds__(256) frame_copy_kernel(const Ctrl* __restrict__ c,
                                                         const MeshDev* __restrict__ m,
                                                         FrameRing ring) {
    if (c->done) return;
    const int pre = c->snap_pre, post = c->snap_post;
    if (!pre && !post) return;
    const int p = (int)(c->step & 1);
    const long long R = c->ring_slots;
    const long long slot_pre = c->captured % R, slot_post = (c->captured + pre) % R;
    const int g = m->ghost;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (int which = 0; which < 2; ++which) {
        if (which == 0 ? !pre : !post) continue;
        double* __restrict__ dst = ring.base + (which == 0 ? slot_pre : slot_post) * ring.slot_len;
        for (int b = 0; b < m->nblocks; ++b) {
            const BlockDev& B = m->b[b];
            const double* __restrict__ src = B.buf[which == 0 ? p : p ^ 1];
            const long long plane = (long long)B.nx * B.ny, n = 4 * plane;
            double* __restrict__ d = dst + ring.off[b];
            for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
                const long long v = k / plane, r = k - v * plane;
                const int j = (int)(r / B.nx), i = (int)(r - (long long)j * B.nx);
                d[k] = src[(size_t)v * B.ty * B.pitch + (size_t)(j + g) * B.pitch + (i + g)];
            }
        }
    }
}

// end of step: t += dt; the MUSCL-Hancock predictor calls advance the counter; record this
// step's frames; flip parity
__global__ void finalize_kernel(Ctrl* c) {
    if (c->done) return;
    if (c->clamp && c->frames) {
        for (int which = 0; which < 2; ++which) {
            if (which == 0 ? !c->snap_pre : !c->snap_post) continue;
            const long long slot = c->captured % c->ring_slots;
            c->ring_t[slot] = c->snap_t;
            c->ring_idx[slot] = c->frame_idx;
            c->frame_idx = c->frame_idx + 1;
            c->captured = c->captured + 1;
        }
    }
    c->t = c->t + c->dt;
    if (c->scheme == 1) c->calls = c->calls + c->nblocks;
    c->step = c->step + 1;
}

// ------------------------------------------------------------------------------------
// shared helpers for the stencils
// ------------------------------------------------------------------------------------
// issue the tile's TMA load and wait for it (bounded); false if the wait gave up
template <int NBYTES>
__device__ __forceinline__ bool load_tile(double* sU, uint64_t* bar, const CUtensorMap* tm, int x0,
                                          int y0, Ctrl* c) {
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_expect_tx(bar, NBYTES);
        tma_load_3d(sU, tm, bar, x0, y0, 0);
    }
    __syncthreads();
    bool ok = mbar_wait_bounded(bar, 0, kWaitLimit);
    int bad = __syncthreads_or(!ok);
    if (bad) {
        if (threadIdx.x == 0) {
            raise_error(c, HF_DEV_TIMEOUT);
            mbar_wait_bounded(bar, 0, kWaitLimit);   // let an in-flight copy land before exit
        }
        __syncthreads();
        return false;
    }
    return true;
}

// The ghost cells in a tile's halo (loaded after this step's fill), from shared memory into the
// step's output buffer, so the updated state carries the ghost values the reference's mesh holds
// after the step (its update leaves ghost cells as filled) and the next fill finds this fill's
// values in its other buffer.  Each ghost cell is stored by the one tile holding its nearest
// interior cell; only tiles on the block's edge hold any.  sU is [4][TY + 2G][TX + 2G].
template <int TX, int TY, int G, int NT>
__device__ __forceinline__ void store_ghosts(const double* __restrict__ sU, const BlockDev& B, int x0, int y0,
                                             double* __restrict__ out, int* err) {
    if (x0 > 0 && y0 > 0 && x0 + TX < B.nx && y0 + TY < B.ny) return;
    constexpr int UX = TX + 2 * G, UY = TY + 2 * G;
    const size_t plane = (size_t)B.ty * B.pitch;
    for (int it = threadIdx.x; it < UX * UY; it += NT) {
        const int lx = it % UX, ly = it / UX;
        const int x = x0 - G + lx, y = y0 - G + ly;   // interior coordinates
        if (x < -G || y < -G || x >= B.nx + G || y >= B.ny + G) continue;
        if (x >= 0 && y >= 0 && x < B.nx && y < B.ny) continue;
        const int cx = x < 0 ? 0 : (x >= B.nx ? B.nx - 1 : x);
        const int cy = y < 0 ? 0 : (y >= B.ny ? B.ny - 1 : y);
        if (cx < x0 || cx >= x0 + TX || cy < y0 || cy >= y0 + TY) continue;
        const size_t o = (size_t)(y + G) * B.pitch + (x + G);
        if (!hf_in((long long)o, (long long)plane, err)) continue;
#pragma unroll
        for (int v = 0; v < 4; ++v) out[v * plane + o] = sU[(v * UY + ly) * UX + lx];
    }
}

// ------------------------------------------------------------------------------------
// MUSCL-Hancock, fused
// ------------------------------------------------------------------------------------
template <int TX, int TY>
struct MhLayout {
    using T = MhTile<TX, TY>;
    static constexpr int U_OFF = 0;
    static constexpr int A_OFF = U_OFF + T::U_SIZE;
    static constexpr int F_OFF = A_OFF + T::A_SIZE;
    static constexpr int G_OFF = F_OFF + T::F_SIZE;
    static constexpr int END = G_OFF + T::G_SIZE;
    static constexpr size_t BYTES = (size_t)END * 8 + 16;   // + mbarrier
    static constexpr int TMA_BYTES = T::U_SIZE * 8;
};

template <int TX, int TY, int LIM, int NT>
// three 256-thread CTAs per SM (80 registers, 73 KB of shared memory each): 24 warps hide more
// of the integer sequences' latency than 16 (measured faster despite a few spilled registers)
__global__ void __launch_bounds__(NT, 3) mh_kernel(Ctrl* __restrict__ c, const MeshDev* __restrict__ m,
                                                int b, const __grid_constant__ CUtensorMap tm0,
                                                const __grid_constant__ CUtensorMap tm1,
                                                double* __restrict__ hout) {
    using L = MhLayout<TX, TY>;
    extern __shared__ __align__(1024) double smem[];
    double* sU = smem + L::U_OFF;
    double* sA = smem + L::A_OFF;
    double* sF = smem + L::F_OFF;
    double* sG = smem + L::G_OFF;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L::END);
    if (c->done) return;

    const BlockDev& B = m->b[b];
    const int p = (int)(c->step & 1);
    const int tiles_x = (B.nx + TX - 1) / TX;
    const int x0 = (blockIdx.x % tiles_x) * TX, y0 = (blockIdx.x / tiles_x) * TY;

    // scalars of this step, formed once per CTA by thread 0 while the tile is in flight and
    // published by the barrier in load_tile
    __shared__ double sc[5];
    const double g = c->gamma, g1 = c->g1;
    const double dt = c->dt;
    if (threadIdx.x == 0) {
        // the predictor's own TimeStep call (muscl_hancock.cpp:246): blocks < b already advanced
        const double dtp = cfl_dt(c, c->calls + b, b, p, p ^ 1);
        const double dx = c->dx[b], dy = c->dy[b];
        sc[0] = 0.5 * dtp / dx;   // 248-249
        sc[1] = 0.5 * dtp / dy;
        sc[2] = 1.0 / dx;         // 352-353
        sc[3] = 1.0 / dy;
        if (blockIdx.x == 0) c->dt_pred[b] = dtp;
    }

    if (!load_tile<L::TMA_BYTES>(sU, bar, p ? &tm1 : &tm0, x0, y0, c)) return;
    const double hdx = sc[0], hdy = sc[1], one_dx = sc[2], one_dy = sc[3];

    const int herr = mh_tile_fluxes<TX, TY, NT, LIM>(sU, sA, sF, sG, g, g1, hdx, hdy, x0, y0, B.nx, B.ny,
                                                     &c->first_bad, face_key(c->step, b, 0, 0, 0));
    // conservative update + forward Euler, and the next step's TimeStep terms
    double* __restrict__ out = B.buf[p ^ 1];
    const size_t plane = (size_t)B.ty * B.pitch;
    double mx = 0.0, my = 0.0;
    for (int it = threadIdx.x; it < TX * TY; it += NT) {
        const int ox = it % TX, oy = it / TX;
        const int gxx = x0 + ox, gyy = y0 + oy;
        if (gxx < B.nx && gyy < B.ny) {
            double un[4];
            const size_t o = (size_t)(gyy + 2) * B.pitch + (gxx + 2);
            const size_t h = (size_t)(gyy + 2) * B.tx + gxx + 2;
            if (!hf_in((long long)o, (long long)plane, &c->err) ||
                !hf_in((long long)h, (long long)B.ty * B.tx, &c->err))
                continue;
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                un[v] = mh_update<TX, TY>(sU, sF, sG, v, ox, oy, dt, one_dx, one_dy);
                out[v * plane + o] = un[v];
                if (hout) __stcs(&hout[(size_t)v * B.ty * B.tx + h], un[v]);
            }
            double sx, sy;
            if (!wave_terms(g, g1, un[0], un[1], un[2], un[3], sx, sy))
                atomicMin(&c->first_nonpos, face_key(c->step, b, 0, gyy, gxx));
            mx = nmax(mx, sx);
            my = nmax(my, sy);
        }
    }
    store_ghosts<TX, TY, 2, NT>(sU, B, x0, y0, out, &c->err);
    block_max2_atomic<NT>(mx, my, &c->int_s[p ^ 1][b][0], &c->int_s[p ^ 1][b][1]);
    if (herr) atomicAdd(reinterpret_cast<unsigned long long*>(&c->hllc_errors), (unsigned long long)herr);
}

// ------------------------------------------------------------------------------------
// MUSCL-Hancock, every block of a step in one persistent launch
// ------------------------------------------------------------------------------------
// The reference updates the blocks one after the other, and block b's half-step predictor takes
// its dt from a TimeStep call over a mesh whose blocks < b are already updated
// (muscl_hancock.cpp:246, called from simulation.cpp:106-110).  One launch per block leaves a
// partly filled last wave of CTAs at the end of every block.  Here one cooperative launch (all
// CTAs resident) walks the tiles of all blocks, in block order, from a shared counter, so one
// block's tail overlaps the next block's start, and runs every block with the predictor dt of a
// TimeStep call over the step's starting state.  For block 0 that is the reference's value.  For
// block b > 0 it is the reference's value whenever updating blocks 0..b-1 leaves the largest wave
// speed TimeStep sees unchanged, the usual case.  After all tiles, block by block: a grid barrier,
// then every CTA forms block b's true predictor dt (the reference's call: blocks < b from their
// updated state) from the same data; where its bits differ from the value used, the grid runs
// block b again with it.  A step never writes a block's input buffer, so the second run gives
// exactly the sequential result; a block's wave-speed maxima and numerical-failure records are
// kept per block and folded into the totals only when every block is final, so a discarded run
// leaves nothing behind.
// grid-wide barrier with a bounded wait (10 s of the global timer); false after a timeout or
// once another CTA raised the error word
__device__ bool step_grid_barrier(Ctrl* c) {
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
            unsigned long long t0;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
            for (;;) {
                if (*gen != g0) { ok = 1; break; }
                if (*(volatile int*)&c->err != 0) break;
                unsigned long long t1;
                asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
                if (t1 - t0 > 10000000000ull) {
                    raise_error(c, HF_DEV_TIMEOUT);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// this launch's predictor scalars per block: 0.5 dtp / dx, 0.5 dtp / dy, 1 / dx, 1 / dy, and dtp
__shared__ double s_step_sc[kStepMaxBlocks][5];

// One tile of block b (local tile index `local`): its TMA load (mbarrier phase `phase`), the
// fused fluxes with the block's predictor scalars, the update and the block's records.  False if
// the load's bounded wait gave up.  Out of line: the tile loop and the re-run loop share one copy.
template <int TX, int TY, int LIM, int NT>
__device__ __noinline__ bool mh_step_tile(Ctrl* __restrict__ c, const MeshDev* __restrict__ m,
                                          const StepPlan& plan, int b, int local, int p, uint32_t phase) {
    using L = MhLayout<TX, TY>;
    extern __shared__ __align__(1024) double smem[];
    double* sU = smem + L::U_OFF;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L::END);
    const BlockDev& B = m->b[b];
    const int x0 = (local % plan.tiles_x[b]) * TX, y0 = (local / plan.tiles_x[b]) * TY;
    if (threadIdx.x == 0) {
        // the previous tile's reads of sU (generic proxy) are ordered before this copy's writes
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(bar, L::TMA_BYTES);
        tma_load_3d(sU, &plan.tm[b][p], bar, x0, y0, 0);
    }
    const bool ok = mbar_wait_bounded(bar, phase, kWaitLimit);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) {
            raise_error(c, HF_DEV_TIMEOUT);
            mbar_wait_bounded(bar, phase, kWaitLimit);   // let an in-flight copy land before exit
        }
        __syncthreads();
        return false;
    }
    const double g = c->gamma, g1 = c->g1;
    const int herr = mh_tile_fluxes<TX, TY, NT, LIM>(sU, smem + L::A_OFF, smem + L::F_OFF, smem + L::G_OFF, g, g1,
                                                     s_step_sc[b][0], s_step_sc[b][1], x0, y0, B.nx, B.ny,
                                                     &c->step_bad[b], face_key(c->step, b, 0, 0, 0));
    const double* sF = smem + L::F_OFF;
    const double* sG = smem + L::G_OFF;
    const double dt = c->dt, one_dx = s_step_sc[b][2], one_dy = s_step_sc[b][3];
    double* __restrict__ out = B.buf[p ^ 1];
    double* __restrict__ hout = plan.hout[b];
    const size_t plane = (size_t)B.ty * B.pitch;
    double mx = 0.0, my = 0.0;
    for (int it = threadIdx.x; it < TX * TY; it += NT) {
        const int ox = it % TX, oy = it / TX;
        const int gxx = x0 + ox, gyy = y0 + oy;
        if (gxx < B.nx && gyy < B.ny) {
            double un[4];
            const size_t o = (size_t)(gyy + 2) * B.pitch + (gxx + 2);
            const size_t h = (size_t)(gyy + 2) * B.tx + gxx + 2;
            if (!hf_in((long long)o, (long long)plane, &c->err) ||
                !hf_in((long long)h, (long long)B.ty * B.tx, &c->err))
                continue;
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                un[v] = mh_update<TX, TY>(sU, sF, sG, v, ox, oy, dt, one_dx, one_dy);
                out[v * plane + o] = un[v];
                if (hout) __stcs(&hout[(size_t)v * B.ty * B.tx + h], un[v]);
            }
            double sx, sy;
            if (!wave_terms(g, g1, un[0], un[1], un[2], un[3], sx, sy))
                atomicMin(&c->step_nonpos[b], face_key(c->step, b, 0, gyy, gxx));
            mx = nmax(mx, sx);
            my = nmax(my, sy);
        }
    }
    store_ghosts<TX, TY, 2, NT>(sU, B, x0, y0, out, &c->err);
    block_max2_atomic<NT>(mx, my, &c->int_s[p ^ 1][b][0], &c->int_s[p ^ 1][b][1]);
    if (herr) atomicAdd(reinterpret_cast<unsigned long long*>(&c->step_hllc[b]), (unsigned long long)herr);
    return true;
}

// the predictor scalars of block b from its predictor dt (muscl_hancock.cpp:248-249, 352-353)
__device__ __forceinline__ void step_scalars(const Ctrl* c, int b, double dtp) {
    s_step_sc[b][0] = div_rn(0.5 * dtp, c->dx[b]);
    s_step_sc[b][1] = div_rn(0.5 * dtp, c->dy[b]);
    s_step_sc[b][2] = div_rn(1.0, c->dx[b]);
    s_step_sc[b][3] = div_rn(1.0, c->dy[b]);
    s_step_sc[b][4] = dtp;
}

template <int TX, int TY, int LIM, int NT>
__global__ void __launch_bounds__(NT, 3) mh_step_kernel(Ctrl* __restrict__ c, const MeshDev* __restrict__ m,
                                                     const __grid_constant__ StepPlan plan) {
    using L = MhLayout<TX, TY>;
    extern __shared__ __align__(1024) double smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L::END);
    if (c->done) return;   // set before this launch: every CTA leaves, no barrier is entered

    const int p = (int)(c->step & 1);
    const int nb = plan.nb;
    const long long calls = c->calls;
    __shared__ int s_tile, s_redo;
    if (threadIdx.x == 0) {
        for (int b = 0; b < nb; ++b) step_scalars(c, b, cfl_dt(c, calls + b, 0, p, p ^ 1));   // starting state
        mbar_init(bar, 1);
    }
    __syncthreads();
    uint32_t phase = 0u;
    const int total = plan.tile_start[nb];
    for (;;) {
        if (threadIdx.x == 0) s_tile = (int)atomicAdd(&c->tile_ctr, 1u);
        __syncthreads();
        const int t = s_tile;
        if (t >= total) break;
        int b = 0;
        while (t >= plan.tile_start[b + 1]) ++b;
        if (!mh_step_tile<TX, TY, LIM, NT>(c, m, plan, b, t - plan.tile_start[b], p, phase)) return;
        phase ^= 1u;
    }
    for (int b = 1; b < nb; ++b) {
        if (!step_grid_barrier(c)) return;   // blocks < b final
        if (threadIdx.x == 0) {
            const double dtp = cfl_dt_fresh(c, calls + b, b, p, p ^ 1);
            s_redo = f64_bits(dtp) != f64_bits(s_step_sc[b][4]);
            if (s_redo) {
                step_scalars(c, b, dtp);
                if (blockIdx.x == 0) {   // forget the first run's records of block b
                    c->int_s[p ^ 1][b][0] = c->int_s[p ^ 1][b][1] = 0ull;
                    c->step_hllc[b] = 0;
                    c->step_bad[b] = c->step_nonpos[b] = ~0ull;
                    c->blocks_rerun = c->blocks_rerun + 1;
                }
            }
        }
        __syncthreads();
        if (!s_redo) continue;
        if (!step_grid_barrier(c)) return;   // the cleared records are in place before the re-run
        const int ntiles = plan.tile_start[b + 1] - plan.tile_start[b];
        for (int local = blockIdx.x; local < ntiles; local += gridDim.x) {
            if (!mh_step_tile<TX, TY, LIM, NT>(c, m, plan, b, local, p, phase)) return;
            phase ^= 1u;
        }
    }
    if (!step_grid_barrier(c)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {   // every block final: fold this step's records
        const volatile Ctrl* vc = c;
        long long herr = 0;
        for (int b = 0; b < nb; ++b) {
            herr += vc->step_hllc[b];
            const unsigned long long fb = vc->step_bad[b], fn = vc->step_nonpos[b];
            if (fb < c->first_bad) c->first_bad = fb;
            if (fn < c->first_nonpos) c->first_nonpos = fn;
            c->dt_pred[b] = s_step_sc[b][4];
        }
        c->hllc_errors = c->hllc_errors + herr;
    }
}

// ------------------------------------------------------------------------------------
// Godunov, fused: per-cell primitives/fluxes once, then x/y HLLC, then update
// ------------------------------------------------------------------------------------
template <int TX, int TY>
struct GoLayout {
    using T = GoTile<TX, TY>;
    static constexpr int NC = T::NC;
    static constexpr int U_OFF = 0;
    static constexpr int Q_OFF = U_OFF + T::U_SIZE;
    static constexpr int F_OFF = Q_OFF + T::Q_SIZE;
    static constexpr int G_OFF = F_OFF + T::F_SIZE;
    static constexpr int END = G_OFF + T::G_SIZE;
    static constexpr size_t BYTES = (size_t)END * 8 + 16;   // + mbarrier
    static constexpr int TMA_BYTES = T::U_SIZE * 8;
};

// three 256-thread CTAs per SM (80 registers, 74 KB of shared memory with 32x10 tiles): measured
// 3 % faster than two CTAs of 32x14 tiles at 110 registers, and than 32x8 or 32x6 tiles
template <int TX, int TY, int NT>
__global__ void __launch_bounds__(NT, 3) godunov_kernel(Ctrl* __restrict__ c,
                                                     const MeshDev* __restrict__ m, int b,
                                                     const __grid_constant__ CUtensorMap tm0,
                                                     const __grid_constant__ CUtensorMap tm1,
                                                     double* __restrict__ hout) {
    using L = GoLayout<TX, TY>;
    extern __shared__ __align__(1024) double smem[];
    double* sU = smem + L::U_OFF;
    double* sQ = smem + L::Q_OFF;
    double* sF = smem + L::F_OFF;
    double* sG = smem + L::G_OFF;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L::END);
    if (c->done) return;

    const BlockDev& B = m->b[b];
    const int p = (int)(c->step & 1);
    const int tiles_x = (B.nx + TX - 1) / TX;
    const int x0 = (blockIdx.x % tiles_x) * TX, y0 = (blockIdx.x / tiles_x) * TY;
    const double g = c->gamma, g1 = c->g1;
    const double dt = c->dt;
    __shared__ double sc[2];
    if (threadIdx.x == 0) {
        sc[0] = 1.0 / c->dx[b];   // godunov.cpp:97-98
        sc[1] = 1.0 / c->dy[b];
    }

    if (!load_tile<L::TMA_BYTES>(sU, bar, p ? &tm1 : &tm0, x0, y0, c)) return;
    const double one_dx = sc[0], one_dy = sc[1];

    const int herr = go_tile_fluxes<TX, TY, NT>(sU, sQ, sF, sG, g, g1, x0, y0, B.nx, B.ny, &c->first_bad,
                                                face_key(c->step, b, 0, 0, 0));
    double* __restrict__ out = B.buf[p ^ 1];
    const size_t plane = (size_t)B.ty * B.pitch;
    double mx = 0.0, my = 0.0;
    for (int it = threadIdx.x; it < TX * TY; it += NT) {
        const int ox = it % TX, oy = it / TX;
        const int gxx = x0 + ox, gyy = y0 + oy;
        if (gxx < B.nx && gyy < B.ny) {
            double un[4];
            const size_t o = (size_t)(gyy + 1) * B.pitch + (gxx + 1);
            const size_t h = (size_t)(gyy + 1) * B.tx + gxx + 1;
            if (!hf_in((long long)o, (long long)plane, &c->err) ||
                !hf_in((long long)h, (long long)B.ty * B.tx, &c->err))
                continue;
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                un[v] = go_update<TX, TY>(sU, sF, sG, v, ox, oy, dt, one_dx, one_dy);
                out[v * plane + o] = un[v];
                if (hout) __stcs(&hout[(size_t)v * B.ty * B.tx + h], un[v]);
            }
            double sx, sy;
            if (!wave_terms(g, g1, un[0], un[1], un[2], un[3], sx, sy))
                atomicMin(&c->first_nonpos, face_key(c->step, b, 0, gyy, gxx));
            mx = nmax(mx, sx);
            my = nmax(my, sy);
        }
    }
    store_ghosts<TX, TY, 1, NT>(sU, B, x0, y0, out, &c->err);
    block_max2_atomic<NT>(mx, my, &c->int_s[p ^ 1][b][0], &c->int_s[p ^ 1][b][1]);
    if (herr) atomicAdd(reinterpret_cast<unsigned long long*>(&c->hllc_errors), (unsigned long long)herr);
}

// ------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------
constexpr int kMhTX = 32, kMhTY = 12, kMhNT = 256;
constexpr int kGoTX = 32, kGoTY = 10, kGoNT = 256;

StencilTiles stencil_tiles(int scheme) {
    return scheme == 0 ? StencilTiles{kGoTX + 2, kGoTY + 2} : StencilTiles{kMhTX + 4, kMhTY + 4};
}

void step_plan_tiles(StepPlan& plan, int b, int nx, int ny) {
    plan.tiles_x[b] = (nx + kMhTX - 1) / kMhTX;
    plan.tile_start[b + 1] = plan.tile_start[b] + plan.tiles_x[b] * ((ny + kMhTY - 1) / kMhTY);
}

// CTAs of the all-blocks launch: as many as are resident at once (the grid barrier needs every
// CTA running), found once per limiter and device
static int g_step_grid[2][64];

template <int LIM>
static cudaError_t launch_mh_step_lim(Ctrl* c, const MeshDev* m, const StepPlan& plan, cudaStream_t s) {
    auto k = mh_step_kernel<kMhTX, kMhTY, LIM, kMhNT>;
    const size_t smem = MhLayout<kMhTX, kMhTY>::BYTES;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    int& grid = g_step_grid[LIM][dev];
    if (grid == 0) {
        int per_sm = 0, sms = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kMhNT, smem)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorInvalidConfiguration;
        grid = per_sm * sms;
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kMhNT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;   // all CTAs resident: the grid barrier is safe
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, c, m, plan);
}

cudaError_t launch_mh_step(Ctrl* c, const MeshDev* m, const StepPlan& plan, int limiter, cudaStream_t s) {
    if (plan.nb < 1 || plan.nb > kStepMaxBlocks) return cudaErrorInvalidValue;
    return limiter == 0 ? launch_mh_step_lim<0>(c, m, plan, s) : launch_mh_step_lim<1>(c, m, plan, s);
}

cudaError_t stencil_prepare() {
    cudaError_t e;
    e = cudaFuncSetAttribute(mh_step_kernel<kMhTX, kMhTY, 0, kMhNT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)MhLayout<kMhTX, kMhTY>::BYTES);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(mh_step_kernel<kMhTX, kMhTY, 1, kMhNT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)MhLayout<kMhTX, kMhTY>::BYTES);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(mh_kernel<kMhTX, kMhTY, 0, kMhNT>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)MhLayout<kMhTX, kMhTY>::BYTES);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(mh_kernel<kMhTX, kMhTY, 1, kMhNT>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)MhLayout<kMhTX, kMhTY>::BYTES);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(godunov_kernel<kGoTX, kGoTY, kGoNT>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)GoLayout<kGoTX, kGoTY>::BYTES);
}

cudaError_t launch_step_begin(Ctrl* c, cudaStream_t s) {
    step_begin_kernel<<<1, 1, 0, s>>>(c);
    return cudaGetLastError();
}

cudaError_t launch_fill_cfl(Ctrl* c, const MeshDev* m, long long total_ghost, cudaStream_t s, int form_dt) {
    long long grid = (total_ghost + kRedThreads - 1) / kRedThreads;
    fill_cfl_kernel<<<(unsigned)(grid < 1 ? 1 : grid), kRedThreads, 0, s>>>(c, m, form_dt);
    return cudaGetLastError();
}

cudaError_t launch_ghost_mirror(Ctrl* c, const MeshDev* m, long long total_ghost, cudaStream_t s) {
    long long grid = (total_ghost + 255) / 256;
    ghost_mirror_kernel<<<(unsigned)(grid < 1 ? 1 : grid), 256, 0, s>>>(c, m);
    return cudaGetLastError();
}

cudaError_t launch_ghost_cfl(Ctrl* c, const MeshDev* m, long long total_ghost, cudaStream_t s, int form_dt) {
    long long want = (total_ghost + kRedThreads - 1) / kRedThreads;
    int grid = (int)(want < 1 ? 1 : (want > 4 * 152 ? 4 * 152 : want));
    ghost_cfl_kernel<<<grid, kRedThreads, 0, s>>>(c, m, form_dt);
    return cudaGetLastError();
}

cudaError_t launch_interior_cfl(Ctrl* c, const MeshDev* m, int b, int nx, int ny, int parity,
                                cudaStream_t s) {
    long long want = ((long long)nx * ny + kRedThreads - 1) / kRedThreads;
    int grid = (int)(want < 1 ? 1 : (want > 8 * 152 ? 8 * 152 : want));
    interior_cfl_kernel<<<grid, kRedThreads, 0, s>>>(c, m, b, parity);
    return cudaGetLastError();
}

cudaError_t launch_set_dt(Ctrl* c, double dt, cudaStream_t s) {
    set_dt_kernel<<<1, 1, 0, s>>>(c, dt);
    return cudaGetLastError();
}

// k x k box average of one block's interior in FP64, stored as FP32 [4][ny/k][nx/k]
__global__ void __launch_bounds__(256) coarsen_kernel(const Ctrl* __restrict__ c,
                                                      const MeshDev* __restrict__ m, int b, int k,
                                                      float* __restrict__ out) {
    const BlockDev& B = m->b[b];
    const double* __restrict__ U = B.buf[(int)(c->step & 1)];
    const int g = m->ghost, cx = B.nx / k, cy = B.ny / k;
    const long long n = 4LL * cx * cy;
    const double inv = 1.0 / ((double)k * (double)k);
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const int v = (int)(q / ((long long)cx * cy));
        const long long r = q - (long long)v * cx * cy;
        const int j = (int)(r / cx), i = (int)(r - (long long)j * cx);
        const double* base = U + (size_t)v * B.ty * B.pitch + (size_t)(j * k + g) * B.pitch + (i * k + g);
        double acc = 0.0;
        for (int jj = 0; jj < k; ++jj)
            for (int ii = 0; ii < k; ++ii) acc += base[(size_t)jj * B.pitch + ii];
        out[q] = (float)(acc * inv);
    }
}

cudaError_t launch_coarsen(const Ctrl* c, const MeshDev* m, int b, int k, long long n, float* out,
                           cudaStream_t s) {
    long long want = (n + 255) / 256;
    int grid = (int)(want < 1 ? 1 : (want > 8 * 152 ? 8 * 152 : want));
    coarsen_kernel<<<grid, 256, 0, s>>>(c, m, b, k, out);
    return cudaGetLastError();
}

cudaError_t launch_frame_copy(Ctrl* c, const MeshDev* m, const FrameRing& ring, cudaStream_t s) {
    frame_copy_kernel<<<4 * 152, 256, 0, s>>>(c, m, ring);
    return cudaGetLastError();
}

cudaError_t launch_finalize(Ctrl* c, cudaStream_t s) {
    finalize_kernel<<<1, 1, 0, s>>>(c);
    return cudaGetLastError();
}

cudaError_t launch_stencil(Ctrl* c, const MeshDev* m, int b, int nx, int ny, int scheme, int limiter,
                           const CUtensorMap* tm0, const CUtensorMap* tm1, cudaStream_t s, double* hout) {
    if (scheme == 0) {
        int tiles = ((nx + kGoTX - 1) / kGoTX) * ((ny + kGoTY - 1) / kGoTY);
        godunov_kernel<kGoTX, kGoTY, kGoNT>
            <<<tiles, kGoNT, GoLayout<kGoTX, kGoTY>::BYTES, s>>>(c, m, b, *tm0, *tm1, hout);
    } else {
        int tiles = ((nx + kMhTX - 1) / kMhTX) * ((ny + kMhTY - 1) / kMhTY);
        if (limiter == 0)
            mh_kernel<kMhTX, kMhTY, 0, kMhNT>
                <<<tiles, kMhNT, MhLayout<kMhTX, kMhTY>::BYTES, s>>>(c, m, b, *tm0, *tm1, hout);
        else
            mh_kernel<kMhTX, kMhTY, 1, kMhNT>
                <<<tiles, kMhNT, MhLayout<kMhTX, kMhTY>::BYTES, s>>>(c, m, b, *tm0, *tm1, hout);
    }
    return cudaGetLastError();
}

cudaError_t launch_upload(Ctrl* c, const MeshDev* m, int b, int tx, int ty, int parity, const double* hin,
                          cudaStream_t s) {
    long long want = ((long long)tx * ty + kRedThreads - 1) / kRedThreads;
    int grid = (int)(want < 1 ? 1 : (want > 8 * 152 ? 8 * 152 : want));
    upload_kernel<<<grid, kRedThreads, 0, s>>>(c, m, b, parity, hin);
    return cudaGetLastError();
}

cudaError_t launch_ghost_store(Ctrl* c, const MeshDev* m, int b, int tx, int ny, int ghost, int parity,
                               double* hout, cudaStream_t s) {
    long long n = 2LL * ghost * (tx + ny);
    int grid = (int)((n + 255) / 256);
    ghost_store_kernel<<<grid < 1 ? 1 : grid, 256, 0, s>>>(c, m, b, parity, hout);
    return cudaGetLastError();
}

}  // namespace hf
