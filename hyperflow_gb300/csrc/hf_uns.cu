// Unstructured (triangle / quadrilateral) Godunov + HLLC time step for sm_103a, and its
// C ABI (declared in include/hyperflow_gb300_uns.h).
//
// Reference: src/fvm_2d_uns -- GodunovScheme::operator() (scheme/godunov/godunov.cpp:31-77)
// walks every (cell, edge) pair in order; for each it rotates the cell state and the
// neighbour state (a cell, or a boundary state from scheme/boundary/boundary.cpp:29-69)
// into the edge's outward-normal frame (model/euler_ideal_gas/euler_ideal_gas.cpp:152-165),
// runs HLLC in x, rotates the flux back, scales by the edge length and accumulates on the
// cell; then L = -acc/area and forward Euler.  TimeStep (scheme/timestep/timestep.cpp:29-62)
// uses the incircle radius.
//
// Device layout: cells SoA FP64 [4][ncells] (two buffers alternating by step parity); the
// (cell, edge) pairs in CSR order by cell -- exactly the reference's cell_edge_indices
// order -- with per-pair neighbour index (or negative boundary code), length and the
// cos/sin of the rotation angles precomputed on the host with the same libm calls the
// reference makes every step.  One thread owns one cell and accumulates its pairs in
// order, so the sum matches the reference bit for bit.
#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "../../include/hyperflow_gb300_uns.h"
#include "hf_ctrl.h"
#include "hf_device.cuh"
#include "hf_trace.h"
#include "hf_json.hpp"

namespace hf {

struct UnsCtrl {
    double gamma, g1, cfl;
    double t, t_end, dt;
    long long calls, step;
    int clamp, done;
    unsigned long long min_dt[2];   // [parity] min over cells of r_in / (|V| + c), bit pattern
    int err;
    long long hllc_errors;
    unsigned long long first_bad;   // least uns_key of a zero-flux pair, ~0 when none
    unsigned long long first_nonpos;// least uns_key of a cell a step left with density or
                                    // pressure not positive, ~0 when none
    int strict;                     // a recorded zero flux or non-positive cell stops the loop
    // frame output with Simulation::solve's cadence (device loop only, i.e. clamp set)
    int frames, ring_slots, snap_pre, snap_post;
    double frame_next, frame_interval, snap_t;
    long long frame_idx, captured, drained;
    double ring_t[HF_MAXRING];
    long long ring_idx[HF_MAXRING];
};

struct UnsMesh {
    int ncells;
    const int* __restrict__ pair_start;   // ncells + 1
    const int* __restrict__ nbr;          // per pair: cell index, or -1 reflective, -2 transmissive, -3 inlet
    const double* __restrict__ geo;       // per pair: [5][npairs] cos a, sin a, cos(-a), sin(-a), length
    const double* __restrict__ inv_area;  // per cell 1.0 / signed area
    const double* __restrict__ rin;       // per cell incircle radius (quads: shortest edge)
    double* U[2];
    double inlet[4];
    long long npairs;
    // edge-based mode: per pair, the unique interior edge it belongs to and whether the pair
    // owns it (+1) or takes the owner's flux negated (-1); -1 for boundary pairs
    const int* __restrict__ pair_edge;
    const signed char* __restrict__ pair_sign;
    const int* __restrict__ edge_pair;      // per unique edge: the owning pair
    const int* __restrict__ edge_cell;      // per unique edge: the owning cell
    const int* __restrict__ edge_nbr;       // per unique edge: the other cell
    const double* __restrict__ edge_geo;    // [5][nedges]: the owning pair's geo, edge by edge
    double* edge_flux;                      // [4][nedges]: length x rotated-back HLLC flux
    int nedges;
    // cells are held in a locality order (Morton order of their vertex centroids); orig[i] is
    // the mesh file's index of device cell i, used in the failure records' keys
    const int* __restrict__ orig;
};

// rotate_flow_values (euler_ideal_gas.cpp:152-165) with precomputed cos/sin
__device__ __forceinline__ void rot(double c, double s, const double* f, double* o) {
    o[0] = f[0];
    o[1] = c * f[1] + s * f[2];
    o[2] = (-s) * f[1] + c * f[2];   // -1.0 * sin(..) * f[1] there; -1.0 * s is exactly -s
    o[3] = f[3];
}

// TimeStep term r_in / (|V| + c) of one cell (uns timestep.cpp:51-58)
__device__ __forceinline__ double uns_dt_term(double g, double g1, double rin, const double* u, bool& pos) {
    double uu, vv, p;
    to_prim_short(g1, u[0], u[1], u[2], u[3], uu, vv, p);
    pos = gt0(u[0]) && gt0(p);   // density and pressure positive, not NaN
    double c = sound(g, u[0], p);
    return div_rn(rin, fabs(sqrt_rn(uu * uu + vv * vv)) + c);
}

// NaN-skipping min of non-negative values
__device__ __forceinline__ double nmin(double m, double s) { return (s < m) ? s : m; }

template <int NT>
__device__ __forceinline__ void block_min_atomic(double v, unsigned long long* acc) {
    __shared__ double red[NT / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = nmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = l < NT / 32 ? red[l] : 1e16;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = nmin(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (l == 0 && v < 1e16) atomicMin(acc, dbits(v));
    }
}

constexpr int kUnsNT = 256;

// key of a cell in the error records (a zero-flux pair's cell, a non-positive cell): step (24
// bits), then cell (40 bits)
__device__ __forceinline__ unsigned long long uns_key(long long step, long long cell) {
    const unsigned long long s = step > 0xFFFFFFll ? 0xFFFFFFull : (unsigned long long)step;
    return (s << 40) | ((unsigned long long)cell & 0xFFFFFFFFFFull);
}

// length x rotated-back HLLC flux of the pair (owner cell c, neighbour cell k); in checked
// builds a pair or neighbour index outside the mesh raises the error word and gives a zero flux
__device__ __forceinline__ int pair_flux(const UnsMesh& m, const double* __restrict__ U, size_t N, double g,
                                         double g1, int e, const double* cv, double* f, int* err) {
    if (!hf_in(e, m.npairs, err) || (m.nbr[e] >= 0 && !hf_in(m.nbr[e], m.ncells, err))) {
#pragma unroll
        for (int v = 0; v < 4; ++v) f[v] = 0.0;
        return 0;
    }
    const double ca = m.geo[e], sa = m.geo[m.npairs + e];
    const double cn = m.geo[2 * m.npairs + e], sn = m.geo[3 * m.npairs + e];
    const double len = m.geo[4 * m.npairs + e];
    const int k = m.nbr[e];
    double rc[4], rn[4];
    rot(ca, sa, cv, rc);
    if (k >= 0) {
        double nb[4] = {U[k], U[N + k], U[2 * N + k], U[3 * N + k]};
        rot(ca, sa, nb, rn);
    } else if (k == -1) {   // reflective: rotate, negate normal momentum, rotate back
        double r1[4], nb[4];
        r1[0] = rc[0]; r1[1] = rc[1] * -1.0; r1[2] = rc[2]; r1[3] = rc[3];
        rot(cn, sn, r1, nb);
        rot(ca, sa, nb, rn);
    } else if (k == -2) {   // transmissive: the cell's own state
        rot(ca, sa, cv, rn);
    } else {                // inlet
        rot(ca, sa, m.inlet, rn);
    }
    double rf[4], fr[4];
    const int bad = hllc_cons<0>(g, g1, rc, rn, rf);
    rot(cn, sn, rf, fr);
#pragma unroll
    for (int v = 0; v < 4; ++v) f[v] = len * fr[v];
    return bad;
}

// pair_flux of an interior edge's owning pair from the per-edge arrays (the same arithmetic):
// the edge kernel reads its geometry once, contiguously, instead of through the pair lists
__device__ __forceinline__ int edge_flux(const UnsMesh& m, const double* __restrict__ U, size_t N, double g,
                                         double g1, int e, const double* cv, double* f, int* err) {
    const int k = m.edge_nbr[e];
    if (!hf_in(k, m.ncells, err)) {
#pragma unroll
        for (int v = 0; v < 4; ++v) f[v] = 0.0;
        return 0;
    }
    const size_t E = (size_t)m.nedges;
    const double ca = m.edge_geo[e], sa = m.edge_geo[E + e];
    const double cn = m.edge_geo[2 * E + e], sn = m.edge_geo[3 * E + e];
    const double len = m.edge_geo[4 * E + e];
    double rc[4], rn[4], nb[4] = {U[k], U[N + k], U[2 * N + k], U[3 * N + k]};
    rot(ca, sa, cv, rc);
    rot(ca, sa, nb, rn);
    double rf[4], fr[4];
    const int bad = hllc_cons<0>(g, g1, rc, rn, rf);
    rot(cn, sn, rf, fr);
#pragma unroll
    for (int v = 0; v < 4; ++v) f[v] = len * fr[v];
    return bad;
}

// edge-based mode, pass 1: one flux per unique interior edge, from its owner's side
__global__ void __launch_bounds__(kUnsNT, 3) uns_edge_flux_kernel(UnsCtrl* __restrict__ c, UnsMesh m) {
    if (c->done) return;
    const int p = (int)(c->step & 1);
    const double g = c->gamma, g1 = c->g1;
    const size_t N = (size_t)m.ncells;
    const double* __restrict__ U = m.U[p];
    int herr = 0;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m.nedges; e += gridDim.x * blockDim.x) {
        const int i = m.edge_cell[e];
        if (!hf_in(i, m.ncells, &c->err)) continue;
        double cv[4] = {U[i], U[N + i], U[2 * N + i], U[3 * N + i]}, f[4];
        if (edge_flux(m, U, N, g, g1, e, cv, f, &c->err)) {
            ++herr;
            atomicMin(&c->first_bad, uns_key(c->step, m.orig[i]));
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) m.edge_flux[(size_t)v * m.nedges + e] = f[v];
    }
    if (herr) atomicAdd(reinterpret_cast<unsigned long long*>(&c->hllc_errors), (unsigned long long)herr);
}

__global__ void __launch_bounds__(kUnsNT) uns_cfl_kernel(UnsCtrl* __restrict__ c, UnsMesh m, int parity) {
    double mn = 1e16;
    const double* U = m.U[parity];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m.ncells; i += gridDim.x * blockDim.x) {
        double u[4] = {U[i], U[m.ncells + i], U[2 * (size_t)m.ncells + i], U[3 * (size_t)m.ncells + i]};
        bool pos;
        mn = nmin(mn, uns_dt_term(c->gamma, c->g1, m.rin[i], u, pos));
    }
    block_min_atomic<kUnsNT>(mn, &c->min_dt[parity]);
}

// start of a device-loop step: stop at t_end, form dt (TimeStep call), reset the accumulator
__global__ void uns_prep_kernel(UnsCtrl* c) {
    int p = (int)(c->step & 1);
    c->snap_pre = c->snap_post = 0;
    if (c->clamp && c->t == c->t_end) { c->done = 1; return; }
    if (c->strict && (c->first_bad != ~0ull || c->first_nonpos != ~0ull)) { c->done = 1; return; }   // strict mode
    // a step takes at most two frames: pause the loop while the ring lacks room for them
    if (c->clamp && c->frames && c->captured - c->drained > c->ring_slots - 2) { c->done = 1; return; }
    c->done = 0;
    double dtr = smin(1e16, bitsd(c->min_dt[p]));
    double final_cfl = (c->calls + 1 <= 10) ? 0.2 * c->cfl : c->cfl;
    double dt = final_cfl * dtr;
    const double t = c->t;
    if (c->clamp && t + dt > c->t_end) dt = c->t_end - t;        // simulation.cpp:85-88
    if (c->clamp && c->frames) {
        const double cur = c->frame_next;
        c->snap_pre = (cur == 0.0);                              // simulation.cpp:91-94
        if ((t + dt > cur) && (cur > 0.0)) dt = cur - t;         // simulation.cpp:96-100
        if (fabs(t - cur) < 1e-12) {                             // simulation.cpp:107-113
            c->snap_post = 1;
            c->frame_next = cur + c->frame_interval;
        }
        c->snap_t = t;
    }
    c->dt = dt;
    c->calls = c->calls + 1;
    c->min_dt[p ^ 1] = dbits(1e16);
}

__global__ void uns_set_dt_kernel(UnsCtrl* c, double dt) {
    c->done = 0;
    c->dt = dt;
    c->min_dt[(c->step & 1) ^ 1] = dbits(1e16);
}

// this step's frames into the ring (cell states SoA [4][ncells]); the state before the
// update is in buffer `step & 1`, the updated one in the other buffer
__global__ void __launch_bounds__(256) uns_frame_copy_kernel(const UnsCtrl* __restrict__ c,
                                                             UnsMesh m, double* __restrict__ ring) {
    if (c->done) return;
    const int pre = c->snap_pre, post = c->snap_post;
    if (!pre && !post) return;
    const int p = (int)(c->step & 1);
    const long long R = c->ring_slots, len = 4LL * m.ncells;
    for (int which = 0; which < 2; ++which) {
        if (which == 0 ? !pre : !post) continue;
        const long long slot = (c->captured + (which == 0 ? 0 : pre)) % R;
        const double* __restrict__ src = m.U[which == 0 ? p : p ^ 1];
        double* __restrict__ dst = ring + slot * len;
        for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < len;
             k += (long long)gridDim.x * blockDim.x)
            dst[k] = src[k];
    }
}

__global__ void uns_finalize_kernel(UnsCtrl* c) {
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
    c->step = c->step + 1;
}

// MINB: CTAs per SM the registers are budgeted for -- three in edge mode (the per-cell work is a
// gather of precomputed edge fluxes, and more warps hide its latency), two in the per-pair mode
// (its HLLC needs the registers: 128 per thread; at 148 only one CTA fits and it runs 27 % slower)
template <int MINB>
__global__ void __launch_bounds__(kUnsNT, MINB) uns_step_kernel(UnsCtrl* __restrict__ c, UnsMesh m) {
    if (c->done) return;
    const int p = (int)(c->step & 1);
    const double g = c->gamma, g1 = c->g1, dt = c->dt;
    const size_t N = (size_t)m.ncells;
    const double* __restrict__ U = m.U[p];
    double* __restrict__ Un = m.U[p ^ 1];
    double mn = 1e16;
    int herr = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m.ncells; i += gridDim.x * blockDim.x) {
        double cv[4] = {U[i], U[N + i], U[2 * N + i], U[3 * N + i]};
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        const int e0 = m.pair_start[i], e1 = m.pair_start[i + 1];
        for (int e = e0; e < e1; ++e) {
            double f[4];
            const int ed = m.pair_edge && hf_in(e, m.npairs, &c->err) ? m.pair_edge[e] : -1;
            if (ed >= 0 && hf_in(ed, m.nedges, &c->err)) {   // edge-based mode: the owner's flux, negated on the other side
                // (a sign flip, not a multiplication by -1.0: the same value, off the FP64 pipe)
                const bool neg = m.pair_sign[e] < 0;
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const double x = m.edge_flux[(size_t)v * m.nedges + ed];
                    f[v] = neg ? -x : x;
                }
            } else if (pair_flux(m, U, N, g, g1, e, cv, f, &c->err)) {
                ++herr;
                atomicMin(&c->first_bad, uns_key(c->step, m.orig[i]));
            }
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[v] = acc[v] + f[v];
        }
        const double inv = m.inv_area[i];
        double un[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const double L = -(inv * acc[v]);   // -1.0 * (...) of godunov.cpp, exactly
            un[v] = dt * L + cv[v];
            Un[v * N + i] = un[v];
        }
        bool pos;
        mn = nmin(mn, uns_dt_term(g, g1, m.rin[i], un, pos));
        if (!pos) atomicMin(&c->first_nonpos, uns_key(c->step, m.orig[i]));
    }
    block_min_atomic<kUnsNT>(mn, &c->min_dt[p ^ 1]);
    if (herr) atomicAdd(reinterpret_cast<unsigned long long*>(&c->hllc_errors), (unsigned long long)herr);
}

}  // namespace hf

// =====================================================================================
// host side
// =====================================================================================
using hf::Json;

struct hf_uns {
    cudaStream_t stream = nullptr;
    double gamma = 1.4, cfl = 0.5, t_start = 0.0, t_end = 0.0;
    double inlet[4] = {0, 0, 0, 0};
    int ncells = 0;
    std::vector<int> nverts;
    std::vector<double> verts;          // per cell vertex, x y
    std::vector<int> codes;             // per pair boundary code from the mesh file
    std::vector<int> pair_start, nbr;
    // the device holds cells in a locality order: perm[d] = file index of device cell d,
    // iperm[f] = device index of file cell f; stage: a [4][ncells] host buffer for reordering
    std::vector<int> perm, iperm;
    std::vector<double> stage;
    long long unmatched = 0;            // pairs with a cell-index code (0: interior) and no match
    long long first_unmatched = -1;     // the first of them, or -1
    std::vector<double> angle, length, area, rin;
    std::vector<double> init;           // initial SoA state
    hf::UnsMesh dm{};
    hf::UnsCtrl* dctrl = nullptr;
    std::vector<void*> allocs;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    bool edge_mode = false;
    int strict = 0;                     // hf_uns_set_strict
    bool has_anim = false;
    double anim_duration = 0.0, anim_fps = 0.0;
    double* ring = nullptr;             // device frame ring
    int ring_slots = 0;
    long long drained = 0;
    int* d_pair_edge = nullptr;
    signed char* d_pair_sign = nullptr;
    std::string err;
};

namespace {

int ufail(hf_uns* u, int code, const std::string& m) {
    if (u) u->err = m;
    return code;
}

#define UCK(call)                                                                              \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return ufail(u, HF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
    } while (0)

void prim_to_cons(double gamma, const double* w, double* c) {
    double rho = w[0], uu = w[1], v = w[2], p = w[3];
    c[0] = rho;
    c[1] = rho * uu;
    c[2] = rho * v;
    c[3] = p / (gamma - 1.0) + 0.5 * rho * (uu * uu + v * v);
}

// The boundary codes of the mesh file must be one per (cell, edge) pair, and each a boundary
// type of src/fvm_2d_uns/scheme/boundary/boundary.h:12 (-1 reflective, -2 transmissive,
// -3 inlet) or a cell index (0 marks an interior edge; an unmatched pair takes its code as its
// neighbour, mesh_structured.cpp:96-109).  The reference reads past its vectors (or prints
// "not supported" and continues with an empty state) otherwise; here such a mesh is refused
// before any device work.
int validate_codes(hf_uns* u, const std::vector<long>* raw = nullptr) {
    int64_t np = 0;
    for (int v : u->nverts) np += v;
    const size_t nc = raw ? raw->size() : u->codes.size();
    if ((int64_t)nc != np)
        return ufail(u, HF_ERR_PARSE, "mesh: " + std::to_string(nc) + " boundary codes for " + std::to_string(np) +
                                          " (cell, edge) pairs");
    for (size_t q = 0; q < nc; ++q) {
        const long k = raw ? (*raw)[q] : (long)u->codes[q];
        if (k < -3 || k >= (long)u->ncells)
            return ufail(u, HF_ERR_PARSE, "mesh: boundary code " + std::to_string(k) + " of pair " +
                                              std::to_string(q) + " is neither -1, -2, -3 nor a cell index");
    }
    return HF_OK;
}

// the mesh text format of generate_block_mesh.py:217-246, cells of 3 or 4 vertices; parsed in
// place, line by line
int parse_mesh(hf_uns* u, const std::string& text) {
    const char* p = text.c_str();
    const char* const end = p + text.size();
    // the next line as [b, e), without its newline; false at the end of the text
    auto next_line = [&](const char*& b, const char*& e) {
        if (p >= end) return false;
        b = p;
        const char* nl = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
        e = nl ? nl : end;
        p = nl ? nl + 1 : end;
        return true;
    };
    const char *b, *e;
    if (!next_line(b, e) || e - b < 5 || std::strncmp(b, "CELLS", 5) != 0)
        return ufail(u, HF_ERR_PARSE, "mesh: expected CELLS header");
    if (!next_line(b, e)) return ufail(u, HF_ERR_PARSE, "mesh: missing cell count");
    const long n = std::strtol(b, nullptr, 0);
    if (n < 0 || n > INT32_MAX / 4) return ufail(u, HF_ERR_PARSE, "mesh: bad cell count");
    u->nverts.reserve(n);
    u->verts.reserve((size_t)n * 8);
    bool edges = false;
    while (next_line(b, e)) {
        if (e - b >= 5 && std::strncmp(b, "EDGES", 5) == 0) {
            edges = true;
            break;
        }
        // std::from_chars rounds correctly, as strtod does, and is several times faster
        const char* s = b;
        double v[8];
        int k = 0;
        while (k < 8) {
            while (s < e && (*s == ' ' || *s == '\t' || *s == '\r')) ++s;
            if (s < e && *s == '+') ++s;
            if (s >= e) break;
            double x;
            const std::from_chars_result r = std::from_chars(s, e, x);
            if (r.ec != std::errc()) break;
            v[k++] = x;
            s = r.ptr;
        }
        if (k != 6 && k != 8) return ufail(u, HF_ERR_PARSE, "mesh: a cell needs 3 or 4 vertices");
        u->nverts.push_back(k / 2);
        for (int i = 0; i < k; ++i) u->verts.push_back(v[i]);
    }
    if ((long)u->nverts.size() != n) return ufail(u, HF_ERR_PARSE, "mesh: cell count mismatch");
    if (!edges || !next_line(b, e)) return ufail(u, HF_ERR_PARSE, "mesh: missing edge count");
    const long ne = std::strtol(b, nullptr, 0);
    std::vector<long> raw;
    if (ne >= 0 && ne <= 4 * n) raw.reserve(ne);
    while (next_line(b, e)) {
        const char* s = b;
        while (s < e && (*s == ' ' || *s == '\t' || *s == '\r')) ++s;
        if (s == e) continue;
        raw.push_back(std::strtol(s, nullptr, 0));
    }
    if ((long)raw.size() != ne) return ufail(u, HF_ERR_PARSE, "mesh: edge count mismatch");
    u->ncells = (int)n;
    const int r = validate_codes(u, &raw);
    if (r != HF_OK) return r;
    u->codes.assign(raw.begin(), raw.end());
    return HF_OK;
}

// The binary mesh format: the text format's content in a fixed little-endian layout, read
// without number parsing.
//   bytes 0..7    "HFMESHB1"
//   bytes 8..15   ncells, int64
//   bytes 16..23  npairs (the cells' vertex counts summed: one (cell, edge) pair per vertex), int64
//   ncells int32  vertices per cell, 3 or 4
//   npairs int32  boundary code per pair, in the text format's EDGES order
//   zero padding to a multiple of 8 bytes
//   npairs x 2 float64  the cells' vertices (x, y) in order
constexpr char kMeshMagic[8] = {'H', 'F', 'M', 'E', 'S', 'H', 'B', '1'};

bool is_binary_mesh(const std::string& data) {
    return data.size() >= 8 && std::memcmp(data.data(), kMeshMagic, 8) == 0;
}

int parse_mesh_binary(hf_uns* u, const std::string& data) {
    const size_t size = data.size();
    if (size < 24) return ufail(u, HF_ERR_PARSE, "binary mesh: truncated header");
    int64_t n = 0, np = 0;
    std::memcpy(&n, data.data() + 8, 8);
    std::memcpy(&np, data.data() + 16, 8);
    if (n < 1 || n > INT32_MAX / 4 || np < 3 * n || np > 4 * n)
        return ufail(u, HF_ERR_PARSE, "binary mesh: bad cell or pair count");
    const size_t ints = 24 + 4 * (size_t)(n + np);
    const size_t vo = (ints + 7) / 8 * 8;
    if (size != vo + 16 * (size_t)np) return ufail(u, HF_ERR_PARSE, "binary mesh: size does not match the counts");
    u->nverts.resize(n);
    std::memcpy(u->nverts.data(), data.data() + 24, 4 * (size_t)n);
    int64_t sum = 0;
    for (int v : u->nverts) {
        if (v != 3 && v != 4) return ufail(u, HF_ERR_PARSE, "binary mesh: a cell needs 3 or 4 vertices");
        sum += v;
    }
    if (sum != np) return ufail(u, HF_ERR_PARSE, "binary mesh: vertex counts do not sum to the pair count");
    u->codes.resize(np);
    std::memcpy(u->codes.data(), data.data() + 24 + 4 * (size_t)n, 4 * (size_t)np);
    u->verts.resize(2 * (size_t)np);
    std::memcpy(u->verts.data(), data.data() + vo, 16 * (size_t)np);
    u->ncells = (int)n;
    return validate_codes(u);
}

// 64-bit finaliser of MurmurHash3 (Appleby): every input bit affects every output bit
inline uint64_t fmix64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xFF51AFD7ED558CCDull;
    x ^= x >> 33;
    x *= 0xC4CEB9FE1A85EC53ull;
    x ^= x >> 33;
    return x;
}

// The tolerance of Edge::opposite_edges_equal: the Edge constructor's default _tol
// (src/fvm_2d_uns/geometry/edge/edge.h:21), which the loader's cells use.
constexpr double kEdgeTol = 1e-12;

// Grid key of one coordinate for the neighbour search: floor(x * 2^30), i.e. grid cells of
// 2^-30 (9.3e-10, far wider than the tolerance), for |x| < 2^32, where the product is exact and
// the key fits in 62 bits.  Beyond 2^32 one ulp exceeds 1e-12, so two coordinates within the
// tolerance are equal and the key is the bit pattern (tagged so it cannot meet a grid key).
// -0.0 and +0.0 both give key 0.
inline int64_t grid_key(double x) {
    if (std::fabs(x) < 4294967296.0) return (int64_t)std::floor(x * 1073741824.0);
    uint64_t b;
    std::memcpy(&b, &x, 8);
    return (int64_t)((b >> 2) | 0x8000000000000000ull) - 1;   // below every grid key
}

// Grid keys a coordinate within the tolerance of x can have: [lo, hi], one or two keys.
// The margin of 4 tolerances covers the rounding of x -/+ 4e-12 and of the test's own
// difference; the exact test below decides.
inline void grid_range(double x, int64_t& lo, int64_t& hi) {
    if (std::fabs(x) < 4294967296.0) {
        lo = grid_key(x - 4 * kEdgeTol);
        hi = grid_key(x + 4 * kEdgeTol);
        if (lo > hi || hi - lo > 2) lo = hi = grid_key(x);   // cannot happen below 2^32
    } else {
        lo = hi = grid_key(x);
    }
}

// Neighbour search of LoadStructuredMesh (mesh_structured.cpp:92-114): for pair q (the edge
// from vertex A to vertex B of its cell) every pair r of the mesh is tested with
// Edge::opposite_edges_equal (edge.cpp:59-71) -- |start_r - B| < 1e-12 and |end_r - A| < 1e-12,
// coordinate by coordinate, as fabs of the difference -- and the last matching r in the scan
// order (cell by cell, edge by edge: the pair index) gives the neighbour cell; a pair with no
// match keeps its code from the mesh file (a boundary type, or a cell index -- 0 for an interior
// edge, so an unmatched interior pair reads cell 0 exactly as in the reference; such pairs are
// counted and reported).  Instead of the O(E^2) scan, pairs are bucketed by the grid keys of
// their start vertex, and a query visits only the buckets a start within the tolerance of B can
// fall in (one, or two near a grid line per axis); every candidate there is tested with the
// reference's own comparison, so the result is the reference's, including the last-match rule,
// self-matches of degenerate edges and coordinates that differ in their last bits between two
// cells.  Non-finite coordinates never compare as within the tolerance and are not bucketed.
// Pair p runs from vertex p to vertex nxt[p] (the cells' vertices are stored pair by pair).
void build_pairs(hf_uns* u) {
    const int n = u->ncells;
    u->pair_start.assign(n + 1, 0);
    for (int c = 0; c < n; ++c) u->pair_start[c + 1] = u->pair_start[c] + u->nverts[c];
    const size_t np = (size_t)u->pair_start[n];
    const double* V = u->verts.data();
    std::vector<int> nxt(np), cell(np);
    for (int c = 0; c < n; ++c) {
        const int s = u->pair_start[c], e = u->pair_start[c + 1];
        for (int q = s; q < e; ++q) {
            nxt[q] = (q == e - 1) ? s : q + 1;
            cell[q] = c;
        }
    }
    // buckets: open-addressed over distinct (kx, ky) start keys; each holds the head of a chain
    // through chain[] in decreasing pair order (pairs are inserted in increasing order)
    size_t cap = 16;
    while (cap < 2 * np) cap <<= 1;
    const size_t mask = cap - 1;
    std::vector<int64_t> kxs(cap), kys(cap);
    std::vector<int> head(cap, -1), chain(np, -1);
    auto bucket_hash = [](int64_t kx, int64_t ky) {
        return fmix64((uint64_t)kx ^ fmix64((uint64_t)ky + 0x9E3779B97F4A7C15ull));
    };
    for (size_t r = 0; r < np; ++r) {
        const double x = V[2 * r], y = V[2 * r + 1];
        if (!std::isfinite(x) || !std::isfinite(y)) continue;
        const int64_t kx = grid_key(x), ky = grid_key(y);
        for (size_t i = bucket_hash(kx, ky) & mask;; i = (i + 1) & mask) {
            if (head[i] < 0) {
                kxs[i] = kx;
                kys[i] = ky;
                head[i] = (int)r;
                break;
            }
            if (kxs[i] == kx && kys[i] == ky) {
                chain[r] = head[i];
                head[i] = (int)r;
                break;
            }
        }
    }
    auto find_bucket = [&](int64_t kx, int64_t ky) {
        for (size_t i = bucket_hash(kx, ky) & mask;; i = (i + 1) & mask) {
            if (head[i] < 0) return -1;
            if (kxs[i] == kx && kys[i] == ky) return head[i];
        }
    };
    u->nbr.resize(np);
    u->unmatched = 0;
    u->first_unmatched = -1;
    for (size_t q = 0; q < np; ++q) {
        const double ax = V[2 * q], ay = V[2 * q + 1];              // this edge's start
        const double bx = V[2 * nxt[q]], by = V[2 * nxt[q] + 1];    // and end
        long long best = -1;
        if (std::isfinite(bx) && std::isfinite(by)) {
            int64_t xlo, xhi, ylo, yhi;
            grid_range(bx, xlo, xhi);
            grid_range(by, ylo, yhi);
            for (int64_t kx = xlo; kx <= xhi; ++kx)
                for (int64_t ky = ylo; ky <= yhi; ++ky)
                    for (int r = find_bucket(kx, ky); r > best; r = chain[r]) {
                        // rhs = pair r, this = pair q, as in edge.cpp:65-68
                        const double rsx = V[2 * (size_t)r], rsy = V[2 * (size_t)r + 1];
                        const double rex = V[2 * (size_t)nxt[r]], rey = V[2 * (size_t)nxt[r] + 1];
                        if ((std::fabs(rsx - bx) < kEdgeTol) && (std::fabs(rsy - by) < kEdgeTol) &&
                            (std::fabs(rex - ax) < kEdgeTol) && (std::fabs(rey - ay) < kEdgeTol)) {
                            best = r;   // the chain runs in decreasing order: the bucket's last match
                            break;
                        }
                    }
        }
        if (best >= 0) {
            u->nbr[q] = cell[best];
        } else {
            u->nbr[q] = u->codes[q];
            if (u->codes[q] >= 0) {
                if (u->unmatched == 0) u->first_unmatched = (long long)q;
                ++u->unmatched;
            }
        }
    }
}

// geometry exactly as the reference: Edge (edge.cpp:165-218), Polygon (polygon.cpp:72-212)
void build_geometry(hf_uns* u) {
    int n = u->ncells;
    size_t np = u->pair_start[n];
    u->angle.resize(np);
    u->length.resize(np);
    u->area.resize(n);
    u->rin.resize(n);
    size_t vo = 0;
    for (int c = 0; c < n; ++c) {
        int nv = u->nverts[c];
        const double* V = &u->verts[2 * vo];
        double el[4];
        for (int k = 0; k < nv; ++k) {
            int k1 = (k == nv - 1) ? 0 : k + 1;
            double p0 = V[2 * k1] - V[2 * k], p1 = V[2 * k1 + 1] - V[2 * k + 1];
            double n0 = p1, n1 = -1.0 * p0;
            double nl = std::sqrt(n0 * n0 + n1 * n1);
            n0 /= nl;
            n1 /= nl;
            size_t pr = u->pair_start[c] + k;
            u->angle[pr] = std::atan2(n1, n0) * 180.0 / M_PI;
            double d = 0.0;
            d += p0 * p0;
            d += p1 * p1;
            u->length[pr] = std::sqrt(d);
            el[k] = u->length[pr];
        }
        double vol = 0.0;
        for (int k = 0; k < nv; ++k) {
            int k1 = (k == nv - 1) ? 0 : k + 1;
            vol += (V[2 * k] * V[2 * k1 + 1] - V[2 * k1] * V[2 * k + 1]);
        }
        vol *= 0.5;
        u->area[c] = vol;
        if (nv == 3) {
            double a = el[0], b = el[1], cc = el[2];
            double s = (a + b + cc) / 2.0;
            double num = s * (s - a) * (s - b) * (s - cc);
            u->rin[c] = std::sqrt(num) / s;
        } else {
            double sh = 1e16;
            for (int k = 0; k < nv; ++k) sh = (sh < el[k]) ? sh : el[k];
            u->rin[c] = sh;
        }
        vo += nv;
    }
}

// a [4][ncells] state in the mesh file's cell order into u->stage in device order, and back
void to_device_order(hf_uns* u, const double* cons) {
    const size_t n = (size_t)u->ncells;
    for (int v = 0; v < 4; ++v)
        for (size_t d = 0; d < n; ++d) u->stage[v * n + d] = cons[v * n + (size_t)u->perm[d]];
}
void to_file_order(const hf_uns* u, double* cons) {
    const size_t n = (size_t)u->ncells;
    for (int v = 0; v < 4; ++v)
        for (size_t d = 0; d < n; ++d) cons[v * n + (size_t)u->perm[d]] = u->stage[v * n + d];
}

template <class T>
int upload(hf_uns* u, T** dst, const std::vector<T>& src) {
    UCK(cudaMalloc(dst, src.size() * sizeof(T) + 16));
    u->allocs.push_back(*dst);
    UCK(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
    return HF_OK;
}

int read_step(hf_uns* u, long long* s) {
    UCK(cudaStreamSynchronize(u->stream));
    UCK(cudaMemcpy(s, &u->dctrl->step, sizeof *s, cudaMemcpyDeviceToHost));
    return HF_OK;
}

int finish_create(hf_uns* u, const Json& cfg) {
    const Json& ic = cfg["initial_condition"];
    const std::string type = ic["type"].string();
    double w[4], c4[4];
    if (type != "Constant") return ufail(u, HF_ERR_UNSUPPORTED, "unstructured IC must be Constant");
    for (int k = 0; k < 4; ++k) w[k] = ic["init_state"][k].number();
    prim_to_cons(u->gamma, w, c4);   // parser.cpp always converts the constant state
    build_pairs(u);
    build_geometry(u);
    int n = u->ncells;
    u->init.assign((size_t)4 * n, 0.0);
    for (int v = 0; v < 4; ++v)
        for (int c = 0; c < n; ++c) u->init[(size_t)v * n + c] = c4[v];
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return ufail(u, HF_ERR_NO_DEVICE, "no CUDA device visible");
    UCK(cudaStreamCreateWithFlags(&u->stream, cudaStreamNonBlocking));
    size_t np = u->pair_start[n];
    // Device cell order: the Morton (Z-order) code of each cell's vertex mean on a 2^16 x 2^16
    // grid over the mesh's bounding box, ties in file order.  Neighbouring cells then sit close
    // in memory, so the flux kernels' gathers of neighbour states and edge fluxes hit the caches.
    // The arithmetic is unchanged: each cell still sums its own pairs in the file's order.
    {
        std::vector<double> cx(n), cy(n);
        double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
        size_t vo = 0;
        for (int c = 0; c < n; ++c) {
            double sx = 0.0, sy = 0.0;
            for (int k = 0; k < u->nverts[c]; ++k) {
                sx += u->verts[2 * (vo + k)];
                sy += u->verts[2 * (vo + k) + 1];
            }
            vo += u->nverts[c];
            cx[c] = std::isfinite(sx) ? sx / u->nverts[c] : 0.0;
            cy[c] = std::isfinite(sy) ? sy / u->nverts[c] : 0.0;
            x0 = std::min(x0, cx[c]); x1 = std::max(x1, cx[c]);
            y0 = std::min(y0, cy[c]); y1 = std::max(y1, cy[c]);
        }
        auto spread = [](uint32_t v) {   // the 16 bits of v to the even bit positions
            v &= 0xFFFFu;
            v = (v | (v << 8)) & 0x00FF00FFu;
            v = (v | (v << 4)) & 0x0F0F0F0Fu;
            v = (v | (v << 2)) & 0x33333333u;
            v = (v | (v << 1)) & 0x55555555u;
            return v;
        };
        const double sxr = x1 > x0 ? 65535.0 / (x1 - x0) : 0.0, syr = y1 > y0 ? 65535.0 / (y1 - y0) : 0.0;
        std::vector<uint64_t> key(n);
        for (int c = 0; c < n; ++c) {
            const uint32_t qx = (uint32_t)((cx[c] - x0) * sxr), qy = (uint32_t)((cy[c] - y0) * syr);
            key[c] = ((uint64_t)(spread(qx) | (spread(qy) << 1)) << 32) | (uint32_t)c;
        }
        std::sort(key.begin(), key.end());
        u->perm.resize(n);
        u->iperm.resize(n);
        for (int d = 0; d < n; ++d) {
            u->perm[d] = (int)(key[d] & 0xFFFFFFFFu);
            u->iperm[u->perm[d]] = d;
        }
        u->stage.resize((size_t)4 * n);
    }
    const std::vector<int>& perm = u->perm;
    const std::vector<int>& iperm = u->iperm;
    // pairs in device order: device cell d holds the pairs of file cell perm[d], in their order
    std::vector<int> dps(n + 1, 0), qmap(np);   // qmap[device pair] = file pair
    for (int d = 0; d < n; ++d) {
        const int f = perm[d];
        dps[d + 1] = dps[d] + u->nverts[f];
        for (int k = 0; k < u->nverts[f]; ++k) qmap[(size_t)dps[d] + k] = u->pair_start[f] + k;
    }
    std::vector<int> dnbr(np);
    std::vector<double> geo(5 * np), inv(n), drin(n);
    for (size_t e = 0; e < np; ++e) {
        const size_t q = (size_t)qmap[e];
        const int k = u->nbr[q];
        dnbr[e] = k >= 0 ? iperm[k] : k;
        double a = u->angle[q] * (M_PI / 180.0);
        double an = (-1.0 * u->angle[q]) * (M_PI / 180.0);
        geo[e] = std::cos(a);
        geo[np + e] = std::sin(a);
        geo[2 * np + e] = std::cos(an);
        geo[3 * np + e] = std::sin(an);
        geo[4 * np + e] = u->length[q];
    }
    for (int d = 0; d < n; ++d) {
        inv[d] = 1.0 / u->area[perm[d]];
        drin[d] = u->rin[perm[d]];
    }
    int r;
    int* ps; int* nb; double* g; double* ia; double* ri; int* org;
    if ((r = upload(u, &ps, dps)) || (r = upload(u, &nb, dnbr)) || (r = upload(u, &g, geo)) ||
        (r = upload(u, &ia, inv)) || (r = upload(u, &ri, drin)) || (r = upload(u, &org, perm)))
        return r;
    // unique interior edges (edge-based mode), owned by the cell with the lower file index, listed
    // in device order of their owners; each with its owner pair's geometry, contiguous by edge
    {
        std::vector<int> pe(np, -1), ep, ec, en;
        std::vector<signed char> sg(np, 0);
        for (int d = 0; d < n; ++d)
            for (int q = dps[d]; q < dps[d + 1]; ++q) {
                const int k = dnbr[q];
                if (k < 0) continue;
                if (perm[d] < perm[k]) {
                    pe[q] = (int)ep.size();
                    sg[q] = 1;
                    ep.push_back(q);
                    ec.push_back(d);
                    en.push_back(k);
                }
            }
        // the partner side: the owner cell's pair facing this cell (its last such pair, should a
        // degenerate mesh hold two)
        for (int d = 0; d < n; ++d)
            for (int q = dps[d]; q < dps[d + 1]; ++q) {
                const int k = dnbr[q];
                if (k < 0 || perm[d] < perm[k]) continue;
                int own = -1;
                for (int o = dps[k + 1] - 1; o >= dps[k] && own < 0; --o)
                    if (dnbr[o] == d) own = o;
                if (own < 0) continue;                  // unmatched: keep the per-side flux
                pe[q] = pe[own];
                sg[q] = -1;
            }
        const size_t ne = ep.size();
        std::vector<double> eg(5 * ne);
        for (size_t e = 0; e < ne; ++e)
            for (int j = 0; j < 5; ++j) eg[j * ne + e] = geo[(size_t)j * np + ep[e]];
        int* d_pe; signed char* d_sg; int* d_ep; int* d_ec; int* d_en; double* d_eg; double* d_ef;
        if ((r = upload(u, &d_pe, pe)) || (r = upload(u, &d_sg, sg)) || (r = upload(u, &d_ep, ep)) ||
            (r = upload(u, &d_ec, ec)) || (r = upload(u, &d_en, en)) || (r = upload(u, &d_eg, eg)))
            return r;
        UCK(cudaMalloc(&d_ef, 4 * (ne + 1) * sizeof(double)));
        u->allocs.push_back(d_ef);
        u->d_pair_edge = d_pe;
        u->d_pair_sign = d_sg;
        u->dm.edge_pair = d_ep;
        u->dm.edge_cell = d_ec;
        u->dm.edge_nbr = d_en;
        u->dm.edge_geo = d_eg;
        u->dm.edge_flux = d_ef;
        u->dm.nedges = (int)ne;
    }
    u->dm.orig = org;
    u->dm.ncells = n;
    u->dm.pair_start = ps;
    u->dm.nbr = nb;
    u->dm.geo = g;
    u->dm.inv_area = ia;
    u->dm.rin = ri;
    u->dm.npairs = (long long)np;
    for (int k = 0; k < 4; ++k) u->dm.inlet[k] = u->inlet[k];
    for (int k = 0; k < 2; ++k) {
        double* p;
        UCK(cudaMalloc(&p, (size_t)4 * n * sizeof(double)));
        u->allocs.push_back(p);
        u->dm.U[k] = p;
    }
    hf::UnsCtrl C{};
    C.gamma = u->gamma;
    C.g1 = u->gamma - 1.0;
    C.cfl = u->cfl;
    C.t = u->t_start;
    C.t_end = u->t_end;
    C.first_bad = ~0ull;
    C.first_nonpos = ~0ull;
    UCK(cudaMalloc(&u->dctrl, sizeof C));
    UCK(cudaMemcpy(u->dctrl, &C, sizeof C, cudaMemcpyHostToDevice));
    return hf_uns_set_state(u, u->init.data());
}

int enqueue_uns_step(hf_uns* u, bool prep) {
    int grid = (u->ncells + hf::kUnsNT - 1) / hf::kUnsNT;
    if (prep) hf::uns_prep_kernel<<<1, 1, 0, u->stream>>>(u->dctrl);
    hf::UnsMesh m = u->dm;
    if (u->edge_mode) {
        m.pair_edge = u->d_pair_edge;
        m.pair_sign = u->d_pair_sign;
        int eg = (m.nedges + hf::kUnsNT - 1) / hf::kUnsNT;
        hf::uns_edge_flux_kernel<<<eg < 1 ? 1 : eg, hf::kUnsNT, 0, u->stream>>>(u->dctrl, m);
    } else {
        m.pair_edge = nullptr;
    }
    if (u->edge_mode)
        hf::uns_step_kernel<3><<<grid, hf::kUnsNT, 0, u->stream>>>(u->dctrl, m);
    else
        hf::uns_step_kernel<2><<<grid, hf::kUnsNT, 0, u->stream>>>(u->dctrl, m);
    if (u->ring_slots > 0) hf::uns_frame_copy_kernel<<<4 * 152, 256, 0, u->stream>>>(u->dctrl, m, u->ring);
    hf::uns_finalize_kernel<<<1, 1, 0, u->stream>>>(u->dctrl);
    UCK(cudaGetLastError());
    return HF_OK;
}

int create_common(const char* case_json, size_t len, const std::string* mesh_text, hf_uns** out) {
    if (!case_json || !out) return HF_ERR_ARG;
    hf_uns* u = new hf_uns();
    *out = u;
    try {
        Json cfg = Json::parse(case_json, len);
        if (cfg["model"]["model"].string() != "EulerIdealGas")
            return ufail(u, HF_ERR_UNSUPPORTED, "model must be EulerIdealGas");
        u->gamma = cfg["model"]["gamma"].number();
        if (cfg["scheme"]["type"].string() != "Godunov")
            return ufail(u, HF_ERR_UNSUPPORTED, "the unstructured solver is Godunov only");
        if (cfg["scheme"]["riemann"].string() != "HLLCEuler")
            return ufail(u, HF_ERR_UNSUPPORTED, "Riemann solver must be HLLCEuler");
        u->cfl = cfg["simulation"]["cfl"].number();
        u->t_start = cfg["simulation"]["t_start"].number();
        u->t_end = cfg["simulation"]["t_end"].number();
        if (cfg["simulation"].has("animation")) {
            u->has_anim = true;
            u->anim_duration = cfg["simulation"]["animation"]["duration"].number();
            u->anim_fps = cfg["simulation"]["animation"]["fps"].number();
        }
        double w[4];
        for (int k = 0; k < 4; ++k) w[k] = cfg["mesh"]["boundaries"]["inlet"][k].number();
        prim_to_cons(u->gamma, w, u->inlet);   // parser.cpp:211-217
        const std::string mt = cfg["mesh"]["type"].string();
        if (mt != "hyperflow_structured" && mt != "hyperflow_unstructured")
            return ufail(u, HF_ERR_UNSUPPORTED, "mesh type '" + mt + "' not supported");
        std::string text;
        if (mesh_text) {
            text = *mesh_text;
        } else {
            std::ifstream f(cfg["mesh"]["file"].string(), std::ios::binary | std::ios::ate);
            if (!f) return ufail(u, HF_ERR_ARG, "unable to open mesh file " + cfg["mesh"]["file"].string());
            const std::streamoff size = f.tellg();
            text.resize(size > 0 ? (size_t)size : 0);
            f.seekg(0);
            if (size > 0 && !f.read(&text[0], size))
                return ufail(u, HF_ERR_ARG, "unable to read mesh file " + cfg["mesh"]["file"].string());
        }
        int r = is_binary_mesh(text) ? parse_mesh_binary(u, text) : parse_mesh(u, text);
        if (r != HF_OK) return r;
        return finish_create(u, cfg);
    } catch (const std::exception& e) {
        return ufail(u, HF_ERR_PARSE, e.what());
    }
}

}  // namespace

extern "C" {

int hf_uns_create(const char* case_json, size_t len, hf_uns** out) {
    return create_common(case_json, len, nullptr, out);
}

int hf_uns_create_mesh(const char* case_json, size_t len, const char* mesh_text, size_t mesh_len,
                       hf_uns** out) {
    if (!mesh_text) return HF_ERR_ARG;
    std::string t(mesh_text, mesh_len);
    return create_common(case_json, len, &t, out);
}

void hf_uns_destroy(hf_uns* u) {
    if (!u) return;
    if (u->stream) cudaStreamSynchronize(u->stream);
    for (int k = 0; k < 2; ++k)
        if (u->graph[k]) cudaGraphExecDestroy(u->graph[k]);
    for (void* p : u->allocs) cudaFree(p);
    if (u->ring) cudaFree(u->ring);
    if (u->dctrl) cudaFree(u->dctrl);
    if (u->stream) cudaStreamDestroy(u->stream);
    delete u;
}

const char* hf_uns_last_error_message(const hf_uns* u) { return u ? u->err.c_str() : ""; }

int hf_uns_sizes(const hf_uns* u, int64_t* ncells, int64_t* npairs) {
    if (!u) return HF_ERR_ARG;
    if (ncells) *ncells = u->ncells;
    if (npairs) *npairs = u->pair_start.empty() ? 0 : u->pair_start.back();
    return HF_OK;
}

int hf_uns_unmatched_pairs(const hf_uns* u, int64_t* count, int64_t* first_pair) {
    if (!u) return HF_ERR_ARG;
    if (count) *count = u->unmatched;
    if (first_pair) *first_pair = u->first_unmatched;
    return HF_OK;
}

int hf_uns_mesh_neighbours(const char* mesh, size_t mesh_len, int64_t* ncells, int64_t* npairs,
                           int32_t* nbr, int64_t max_pairs, int64_t* unmatched, int64_t* first_unmatched) {
    if (!mesh) return HF_ERR_ARG;
    hf_uns u;
    try {
        const std::string text(mesh, mesh_len);
        const int r = is_binary_mesh(text) ? parse_mesh_binary(&u, text) : parse_mesh(&u, text);
        if (r != HF_OK) return r;
        build_pairs(&u);
    } catch (const std::exception&) {
        return HF_ERR_PARSE;
    }
    const int64_t np = u.pair_start.back();
    if (ncells) *ncells = u.ncells;
    if (npairs) *npairs = np;
    if (unmatched) *unmatched = u.unmatched;
    if (first_unmatched) *first_unmatched = u.first_unmatched;
    if (nbr) {
        if (max_pairs < np) return HF_ERR_ARG;
        std::memcpy(nbr, u.nbr.data(), (size_t)np * sizeof(int32_t));
    }
    return HF_OK;
}

int hf_uns_mesh_arrays(const hf_uns* u, int32_t* pair_start, int32_t* nbr, double* angle,
                       double* length, double* area, double* rin) {
    if (!u) return HF_ERR_ARG;
    size_t n = u->ncells, np = u->pair_start.empty() ? 0 : u->pair_start.back();
    if (pair_start) std::memcpy(pair_start, u->pair_start.data(), (n + 1) * sizeof(int));
    if (nbr) std::memcpy(nbr, u->nbr.data(), np * sizeof(int));
    if (angle) std::memcpy(angle, u->angle.data(), np * sizeof(double));
    if (length) std::memcpy(length, u->length.data(), np * sizeof(double));
    if (area) std::memcpy(area, u->area.data(), n * sizeof(double));
    if (rin) std::memcpy(rin, u->rin.data(), n * sizeof(double));
    return HF_OK;
}

// Polygon::calculate_centroid (src/fvm_2d_uns/geometry/polygon/polygon.cpp:188-212) over the
// signed area the reference divides by
int hf_uns_centroids(const hf_uns* u, double* xy) {
    if (!u || !xy) return HF_ERR_ARG;
    const size_t n = u->ncells;
    size_t vo = 0;
    for (size_t c = 0; c < n; ++c) {
        const int nv = u->nverts[c];
        const double* V = u->verts.data() + 2 * vo;
        double cx = 0.0, cy = 0.0;
        for (int i = 0; i < nv; ++i) {
            const int j = (i == nv - 1) ? 0 : i + 1;
            const double second = (V[2 * i] * V[2 * j + 1] - V[2 * j] * V[2 * i + 1]);
            cx += ((V[2 * i] + V[2 * j]) * second);
            cy += ((V[2 * i + 1] + V[2 * j + 1]) * second);
        }
        cx /= (6.0 * u->area[c]);
        cy /= (6.0 * u->area[c]);
        xy[c] = cx;
        xy[n + c] = cy;
        vo += nv;
    }
    return HF_OK;
}

int hf_uns_set_state(hf_uns* u, const double* cons) {
    if (!u || !cons || !u->dctrl) return HF_ERR_ARG;
    long long s;
    int r = read_step(u, &s);
    if (r) return r;
    int p = (int)(s & 1);
    size_t bytes = (size_t)4 * u->ncells * sizeof(double);
    to_device_order(u, cons);
    UCK(cudaMemcpyAsync(u->dm.U[p], u->stage.data(), bytes, cudaMemcpyHostToDevice, u->stream));
    unsigned long long init = 0;
    double big = 1e16;
    std::memcpy(&init, &big, 8);
    UCK(cudaMemcpyAsync(&u->dctrl->min_dt[p], &init, 8, cudaMemcpyHostToDevice, u->stream));
    int grid = (u->ncells + hf::kUnsNT - 1) / hf::kUnsNT;
    if (grid > 8 * 152) grid = 8 * 152;
    hf::uns_cfl_kernel<<<grid, hf::kUnsNT, 0, u->stream>>>(u->dctrl, u->dm, p);
    UCK(cudaGetLastError());
    UCK(cudaStreamSynchronize(u->stream));
    return HF_OK;
}

int hf_uns_get_state(hf_uns* u, double* cons) {
    if (!u || !cons || !u->dctrl) return HF_ERR_ARG;
    long long s;
    int r = read_step(u, &s);
    if (r) return r;
    UCK(cudaMemcpy(u->stage.data(), u->dm.U[s & 1], (size_t)4 * u->ncells * sizeof(double), cudaMemcpyDeviceToHost));
    to_file_order(u, cons);
    return HF_OK;
}

// strict mode, after a synchronisation: HF_ERR_NUMERIC once a zero-flux pair or a non-positive
// cell is recorded (the record of the earlier step; a zero flux first within one step)
static int uns_strict_check(hf_uns* u) {
    if (!u->strict) return HF_OK;
    unsigned long long k[2] = {~0ull, ~0ull};
    UCK(cudaMemcpy(&k[0], &u->dctrl->first_bad, sizeof k[0], cudaMemcpyDeviceToHost));
    UCK(cudaMemcpy(&k[1], &u->dctrl->first_nonpos, sizeof k[1], cudaMemcpyDeviceToHost));
    auto at = [](unsigned long long x) {
        return "step " + std::to_string(x >> 40) + ", cell " + std::to_string(x & 0xFFFFFFFFFFull);
    };
    if (k[0] != ~0ull && (k[0] >> 40) <= (k[1] >> 40))
        return ufail(u, HF_ERR_NUMERIC, "HLLC zero flux (all wave-speed branches failed) at " + at(k[0]));
    if (k[1] != ~0ull) return ufail(u, HF_ERR_NUMERIC, "non-positive density or pressure at " + at(k[1]));
    return HF_OK;
}

int hf_uns_sync(hf_uns* u) {
    if (!u || !u->dctrl) return HF_ERR_ARG;
    UCK(cudaStreamSynchronize(u->stream));
    int e = 0;
    UCK(cudaMemcpy(&e, &u->dctrl->err, sizeof e, cudaMemcpyDeviceToHost));
    if (e != 0) return ufail(u, HF_ERR_DEVICE, "device error word " + std::to_string(e));
    return uns_strict_check(u);
}

int hf_uns_set_strict(hf_uns* u, int on) {
    if (!u || !u->dctrl) return HF_ERR_ARG;
    u->strict = on ? 1 : 0;
    UCK(cudaMemcpyAsync(&u->dctrl->strict, &u->strict, sizeof(int), cudaMemcpyHostToDevice, u->stream));
    UCK(cudaStreamSynchronize(u->stream));
    return HF_OK;
}

int hf_uns_last_error_cell(hf_uns* u, int64_t* cell, int64_t* step) {
    if (!u || !u->dctrl) return HF_ERR_ARG;
    unsigned long long k = ~0ull;
    UCK(cudaStreamSynchronize(u->stream));
    UCK(cudaMemcpy(&k, &u->dctrl->first_bad, sizeof k, cudaMemcpyDeviceToHost));
    const bool none = k == ~0ull;
    if (cell) *cell = none ? -1 : (int64_t)(k & 0xFFFFFFFFFFull);
    if (step) *step = none ? -1 : (int64_t)(k >> 40);
    return HF_OK;
}

int hf_uns_last_nonpositive_cell(hf_uns* u, int64_t* cell, int64_t* step) {
    if (!u || !u->dctrl) return HF_ERR_ARG;
    unsigned long long k = ~0ull;
    UCK(cudaStreamSynchronize(u->stream));
    UCK(cudaMemcpy(&k, &u->dctrl->first_nonpos, sizeof k, cudaMemcpyDeviceToHost));
    const bool none = k == ~0ull;
    if (cell) *cell = none ? -1 : (int64_t)(k & 0xFFFFFFFFFFull);
    if (step) *step = none ? -1 : (int64_t)(k >> 40);
    return HF_OK;
}

int hf_uns_clear_error_cell(hf_uns* u) {
    if (!u || !u->dctrl) return HF_ERR_ARG;
    const unsigned long long none = ~0ull;
    UCK(cudaMemcpyAsync(&u->dctrl->first_bad, &none, sizeof none, cudaMemcpyHostToDevice, u->stream));
    UCK(cudaMemcpyAsync(&u->dctrl->first_nonpos, &none, sizeof none, cudaMemcpyHostToDevice, u->stream));
    UCK(cudaStreamSynchronize(u->stream));
    return HF_OK;
}

int hf_uns_time_step(hf_uns* u, double* dt) {
    hf::TraceRange trace_("hf_uns_time_step");
    if (!u || !u->dctrl) return HF_ERR_ARG;
    int clamp = 0;
    UCK(cudaMemcpyAsync(&u->dctrl->clamp, &clamp, sizeof clamp, cudaMemcpyHostToDevice, u->stream));
    hf::uns_prep_kernel<<<1, 1, 0, u->stream>>>(u->dctrl);
    UCK(cudaGetLastError());
    if (dt) {
        UCK(cudaMemcpyAsync(dt, &u->dctrl->dt, sizeof(double), cudaMemcpyDeviceToHost, u->stream));
        UCK(cudaStreamSynchronize(u->stream));
        return uns_strict_check(u);
    }
    return HF_OK;
}

int hf_uns_advance(hf_uns* u, double dt) {
    hf::TraceRange trace_("hf_uns_advance");
    if (!u || !u->dctrl) return HF_ERR_ARG;
    hf::uns_set_dt_kernel<<<1, 1, 0, u->stream>>>(u->dctrl, dt);
    return enqueue_uns_step(u, false);
}

int hf_uns_run(hf_uns* u, int64_t n, int clamp_t_end, int use_graph, int64_t* steps_done) {
    hf::TraceRange trace_("hf_uns_run");
    if (!u || !u->dctrl || n < 0) return HF_ERR_ARG;
    long long s0 = 0;
    int r = read_step(u, &s0);
    if (r) return r;
    int clamp = clamp_t_end ? 1 : 0;
    UCK(cudaMemcpyAsync(&u->dctrl->clamp, &clamp, sizeof clamp, cudaMemcpyHostToDevice, u->stream));
    if (use_graph) {
        if (!u->graph[clamp]) {
            cudaGraph_t g;
            UCK(cudaStreamBeginCapture(u->stream, cudaStreamCaptureModeThreadLocal));
            r = enqueue_uns_step(u, true);
            cudaError_t e = cudaStreamEndCapture(u->stream, &g);
            if (r) return r;
            if (e != cudaSuccess) return ufail(u, HF_ERR_CUDA, cudaGetErrorString(e));
            UCK(cudaGraphInstantiate(&u->graph[clamp], g, 0));
            cudaGraphDestroy(g);
        }
        for (int64_t k = 0; k < n; ++k) UCK(cudaGraphLaunch(u->graph[clamp], u->stream));
    } else {
        for (int64_t k = 0; k < n; ++k)
            if ((r = enqueue_uns_step(u, true))) return r;
    }
    long long s1;
    if ((r = read_step(u, &s1))) return r;
    if (steps_done) *steps_done = s1 - s0;
    return uns_strict_check(u);
}

int hf_uns_frames_enable(hf_uns* u, int ring_slots) {
    if (!u || !u->dctrl || ring_slots < 0 || ring_slots == 1 || ring_slots > HF_MAXRING)
        return HF_ERR_ARG;
    if (ring_slots > 0 && !u->has_anim)
        return ufail(u, HF_ERR_ARG, "the case has no simulation.animation {duration, fps}");
    UCK(cudaStreamSynchronize(u->stream));
    for (int k = 0; k < 2; ++k)
        if (u->graph[k]) { cudaGraphExecDestroy(u->graph[k]); u->graph[k] = nullptr; }
    if (u->ring) { UCK(cudaFree(u->ring)); u->ring = nullptr; }
    u->ring_slots = 0;
    if (ring_slots > 0) {
        UCK(cudaMalloc(&u->ring, (size_t)ring_slots * 4 * u->ncells * sizeof(double)));
        u->ring_slots = ring_slots;
    }
    // the interval exactly as simulation.cpp:57 forms it
    const double interval = ring_slots > 0 ? u->t_end / (u->anim_duration * u->anim_fps) : 0.0;
    hf::UnsCtrl C;
    UCK(cudaMemcpy(&C, u->dctrl, sizeof C, cudaMemcpyDeviceToHost));
    C.frames = ring_slots > 0 ? 1 : 0;
    C.ring_slots = ring_slots;
    C.frame_interval = interval;
    C.captured = C.drained = 0;
    u->drained = 0;
    UCK(cudaMemcpy(u->dctrl, &C, sizeof C, cudaMemcpyHostToDevice));
    return HF_OK;
}

int hf_uns_frames_pending(hf_uns* u, int64_t* n) {
    if (!u || !u->dctrl || !n) return HF_ERR_ARG;
    long long cap = 0;
    UCK(cudaStreamSynchronize(u->stream));
    UCK(cudaMemcpy(&cap, &u->dctrl->captured, sizeof cap, cudaMemcpyDeviceToHost));
    *n = u->ring_slots > 0 ? cap - u->drained : 0;
    return HF_OK;
}

// ---- checkpoint / restart ----
namespace {
struct UnsCkptHeader {
    char magic[8];
    uint32_t version, ctrl_bytes;
    int64_t ncells, npairs;
    uint64_t mesh_hash;
    double gamma, cfl, t_end;
};

// FNV-1a over the mesh connectivity and cell areas: a checkpoint of another mesh with the
// same cell and pair counts is refused too
uint64_t uns_mesh_hash(const hf_uns* u) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; ++i) {
            h ^= b[i];
            h *= 1099511628211ull;
        }
    };
    mix(u->pair_start.data(), u->pair_start.size() * sizeof(int));
    mix(u->nbr.data(), u->nbr.size() * sizeof(int));
    mix(u->area.data(), u->area.size() * sizeof(double));
    return h;
}
const char kUnsCkptMagic[8] = {'H', 'F', 'U', 'C', 'K', 'P', '0', '1'};

UnsCkptHeader uns_ckpt_header(const hf_uns* u) {
    UnsCkptHeader h;
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, kUnsCkptMagic, 8);
    h.version = 1;
    h.ctrl_bytes = (uint32_t)sizeof(hf::UnsCtrl);
    h.ncells = u->ncells;
    h.npairs = u->pair_start.empty() ? 0 : u->pair_start.back();
    h.mesh_hash = uns_mesh_hash(u);
    h.gamma = u->gamma;
    h.cfl = u->cfl;
    h.t_end = u->t_end;
    return h;
}
}  // namespace

int hf_uns_checkpoint_size(const hf_uns* u, size_t* bytes) {
    if (!u || !bytes) return HF_ERR_ARG;
    *bytes = sizeof(UnsCkptHeader) + sizeof(hf::UnsCtrl) + 2 * (size_t)4 * u->ncells * sizeof(double);
    return HF_OK;
}

int hf_uns_checkpoint_save(hf_uns* u, void* buf, size_t bytes) {
    if (!u || !u->dctrl || !buf) return HF_ERR_ARG;
    size_t need = 0;
    hf_uns_checkpoint_size(u, &need);
    if (bytes < need) return ufail(u, HF_ERR_ARG, "checkpoint buffer too small");
    hf::UnsCtrl C;
    UCK(cudaStreamSynchronize(u->stream));
    UCK(cudaMemcpy(&C, u->dctrl, sizeof C, cudaMemcpyDeviceToHost));
    if (u->ring_slots > 0 && C.captured != u->drained)
        return ufail(u, HF_ERR_STATE, "pop the pending frames before a checkpoint");
    const UnsCkptHeader h = uns_ckpt_header(u);
    char* p = static_cast<char*>(buf);
    std::memcpy(p, &h, sizeof h);
    p += sizeof h;
    std::memcpy(p, &C, sizeof C);
    p += sizeof C;
    const size_t n = (size_t)4 * u->ncells * sizeof(double);
    for (int k = 0; k < 2; ++k) {
        UCK(cudaMemcpy(p, u->dm.U[k], n, cudaMemcpyDeviceToHost));
        p += n;
    }
    return HF_OK;
}

int hf_uns_checkpoint_load(hf_uns* u, const void* buf, size_t bytes) {
    if (!u || !u->dctrl || !buf) return HF_ERR_ARG;
    size_t need = 0;
    hf_uns_checkpoint_size(u, &need);
    if (bytes < need) return ufail(u, HF_ERR_ARG, "checkpoint too short for this mesh");
    UnsCkptHeader got;
    std::memcpy(&got, buf, sizeof got);
    const UnsCkptHeader want = uns_ckpt_header(u);
    if (std::memcmp(got.magic, kUnsCkptMagic, 8) != 0 || got.version != want.version)
        return ufail(u, HF_ERR_PARSE, "not an unstructured checkpoint of this format version");
    if (std::memcmp(&got, &want, sizeof got) != 0)
        return ufail(u, HF_ERR_ARG, "checkpoint was taken from a different case, mesh or build");
    const char* p = static_cast<const char*>(buf) + sizeof got;
    hf::UnsCtrl C, cur;
    std::memcpy(&C, p, sizeof C);
    p += sizeof C;
    UCK(cudaStreamSynchronize(u->stream));
    UCK(cudaMemcpy(&cur, u->dctrl, sizeof cur, cudaMemcpyDeviceToHost));
    // the frame ring belongs to this context: keep its configuration, start it empty
    C.frames = cur.frames;
    C.ring_slots = cur.ring_slots;
    C.frame_interval = cur.frame_interval;
    C.captured = C.drained = 0;
    C.clamp = 0;
    C.done = 0;
    C.err = 0;
    C.strict = cur.strict;
    u->drained = 0;
    const size_t n = (size_t)4 * u->ncells * sizeof(double);
    for (int k = 0; k < 2; ++k) {
        UCK(cudaMemcpy(u->dm.U[k], p, n, cudaMemcpyHostToDevice));
        p += n;
    }
    UCK(cudaMemcpy(u->dctrl, &C, sizeof C, cudaMemcpyHostToDevice));
    return HF_OK;
}

int hf_uns_frame_pop(hf_uns* u, double* cons, double* t, int64_t* index) {
    if (!u || !u->dctrl) return HF_ERR_ARG;
    if (u->ring_slots == 0) return ufail(u, HF_ERR_STATE, "frames are not enabled");
    hf::UnsCtrl C;
    UCK(cudaStreamSynchronize(u->stream));
    UCK(cudaMemcpy(&C, u->dctrl, sizeof C, cudaMemcpyDeviceToHost));
    if (C.captured == u->drained) return ufail(u, HF_ERR_STATE, "no frame pending");
    const long long slot = u->drained % u->ring_slots, len = 4LL * u->ncells;
    if (cons) {
        UCK(cudaMemcpy(u->stage.data(), u->ring + slot * len, (size_t)len * sizeof(double), cudaMemcpyDeviceToHost));
        to_file_order(u, cons);
    }
    if (t) *t = C.ring_t[slot];
    if (index) *index = C.ring_idx[slot];
    u->drained += 1;
    long long d = u->drained;
    UCK(cudaMemcpy(&u->dctrl->drained, &d, sizeof d, cudaMemcpyHostToDevice));
    return HF_OK;
}

int hf_uns_get_time(hf_uns* u, double* t, int64_t* calls, double* last_dt) {
    if (!u || !u->dctrl) return HF_ERR_ARG;
    hf::UnsCtrl C;
    UCK(cudaStreamSynchronize(u->stream));
    UCK(cudaMemcpy(&C, u->dctrl, sizeof C, cudaMemcpyDeviceToHost));
    if (t) *t = C.t;
    if (calls) *calls = C.calls;
    if (last_dt) *last_dt = C.dt;
    return HF_OK;
}

int hf_uns_hllc_errors(hf_uns* u, int64_t* count) {
    if (!u || !u->dctrl || !count) return HF_ERR_ARG;
    long long v;
    UCK(cudaStreamSynchronize(u->stream));
    UCK(cudaMemcpy(&v, &u->dctrl->hllc_errors, sizeof v, cudaMemcpyDeviceToHost));
    *count = v;
    return HF_OK;
}

int hf_uns_set_edge_mode(hf_uns* u, int edge_based) {
    if (!u || !u->dctrl) return HF_ERR_ARG;
    UCK(cudaStreamSynchronize(u->stream));
    u->edge_mode = edge_based != 0;
    for (int k = 0; k < 2; ++k)
        if (u->graph[k]) { cudaGraphExecDestroy(u->graph[k]); u->graph[k] = nullptr; }
    return HF_OK;
}

int hf_uns_stream(hf_uns* u, void** stream) {
    if (!u || !stream) return HF_ERR_ARG;
    *stream = (void*)u->stream;
    return HF_OK;
}

}  // extern "C"
