// The MUSCL-Hancock tile computation shared by the per-block stencil (hf_cart.cu) and the
// batched persistent kernel (hf_batch.cu).
//
// Input: sU, the tile's conservative state plus a 2-cell halo in shared memory,
// [4][TY+4][TX+4].  Output: sF / sG, the HLLC fluxes of the tile's x faces
// [4][TY][TX+1] and y faces [4][TY+1][TX]; sA is scratch for the evolved face states.
// The reference steps restated here: calculate_slope_limiters_{x,y} + calculate_slopes_{x,y}
// (muscl_hancock.cpp:67-206), calculate_boundary_extrapolations (209-240),
// evolve_boundary_reconstruction (243-281), calculate_fluxes_{x,y} (284-345).
#pragma once

#include "hf_device.cuh"

namespace hf {

template <int TX, int TY>
struct MhTile {
    static constexpr int UX = TX + 4, UY = TY + 4;
    static constexpr int AXN = (TX + 2) * TY, AYN = TX * (TY + 2);
    static constexpr int AN = AXN > AYN ? AXN : AYN;
    static constexpr int U_SIZE = 4 * UY * UX;        // doubles
    static constexpr int A_SIZE = 8 * AN;
    static constexpr int F_SIZE = 4 * TY * (TX + 1);
    static constexpr int G_SIZE = 4 * (TY + 1) * TX;
};

// A face on a tile edge is formed by both tiles that share it, and partial tiles form
// faces past the block.  Only the owner counts an HLLC zero-flux fallback, so the count
// equals the reference's: face index gf (0..n along the normal) of row gr, local index lf.
__device__ __forceinline__ bool owned_face(int gf, int lf, int T, int n, int gr, int nr) {
    return gr < nr && gf <= n && (lf < T || gf == n);
}

// One cell of the half-step predictor along DIR: limited slopes of the four variables from the
// cell and its two neighbours (u points at the cell's variable 0; plane and stride step to the
// next variable and the next cell along DIR), the extrapolated face states, their fluxes and the
// evolved states.  The minus-side state goes to lo[v * los], the plus-side one to hi[v * his].
template <int DIR, int LIM>
__device__ __forceinline__ void mh_predict(const double* __restrict__ u, int plane, int stride, double g1,
                                           double h, double* __restrict__ lo, int los,
                                           double* __restrict__ hi, int his) {
    double e0[4], e1[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const double* q = u + v * plane;
        const double u0 = q[0];
        const double s = slope<LIM>(q[-stride], u0, q[stride]);
        const double hs = half(s);
        e0[v] = u0 - hs;
        e1[v] = u0 + hs;
    }
    Prim w0 = to_prim(g1, e0[0], e0[1], e0[2], e0[3]);
    Prim w1 = to_prim(g1, e1[0], e1[1], e1[2], e1[3]);
    double f0[4], f1[4];
    flux<DIR>(w0, f0);
    flux<DIR>(w1, f1);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const double d = h * (f0[v] - f1[v]);
        lo[v * los] = e0[v] + d;
        hi[v * his] = e1[v] + d;
    }
}

// One face along DIR: HLLC between the evolved states l[v * ls] (minus side) and r[v * rs];
// the flux goes to f[v * fs].  Returns 1 for the zero-flux fallback.
template <int DIR>
__device__ __forceinline__ int mh_face(const double* __restrict__ l, int ls, const double* __restrict__ r,
                                       int rs, double g, double g1, double* __restrict__ f, int fs) {
    double UL[4], UR[4], F[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        UL[v] = l[v * ls];
        UR[v] = r[v * rs];
    }
    const int bad = hllc_cons<DIR>(g, g1, UL, UR, F);
#pragma unroll
    for (int v = 0; v < 4; ++v) f[v * fs] = F[v];
    return bad;
}

// Computes sF and sG from sU.  Ends with __syncthreads().  Returns the number of owned
// faces whose HLLC took the zero-flux branch (tile origin x0, y0 in interior cells); with
// first_bad, each such face's face_key (key_base: its step and block bits) is min-reduced there.
template <int TX, int TY, int NT, int LIM>
__device__ __forceinline__ int mh_tile_fluxes(const double* __restrict__ sU, double* __restrict__ sA,
                                              double* __restrict__ sF, double* __restrict__ sG,
                                              double g, double g1, double hdx, double hdy, int x0,
                                              int y0, int nx, int ny, unsigned long long* first_bad = nullptr,
                                              unsigned long long key_base = 0) {
    using L = MhTile<TX, TY>;
    constexpr int PL = L::UY * L::UX;
    int herr = 0;
    // Items past the block (cells beyond the first ghost layer, faces beyond the last face) are
    // skipped: no in-block cell reads them, and their zero-filled states would only take the
    // slow special-operand division paths.
    // x phase: slopes, extrapolation, half-step predictor of the x face pair, cells -1..TX
    for (int it = threadIdx.x; it < L::AXN; it += NT) {
        const int lx = it % (TX + 2), ly = it / (TX + 2);
        if (x0 - 1 + lx > nx || y0 + ly >= ny) continue;
        mh_predict<0, LIM>(sU + (ly + 2) * L::UX + lx + 1, PL, 1, g1, hdx, sA + it, L::AN,
                           sA + 4 * L::AN + it, L::AN);
    }
    __syncthreads();
    // x faces 0..TX of each tile row (face f is the left face of output cell f)
    for (int it = threadIdx.x; it < (TX + 1) * TY; it += NT) {
        const int fx = it % (TX + 1), fy = it / (TX + 1);
        if (x0 + fx > nx || y0 + fy >= ny) continue;
        const int al = fy * (TX + 2) + fx;
        const int bad = mh_face<0>(sA + 4 * L::AN + al, L::AN, sA + al + 1, L::AN, g, g1,
                                   sF + fy * (TX + 1) + fx, TY * (TX + 1));
        if (bad && owned_face(x0 + fx, fx, TX, nx, y0 + fy, ny)) {
            ++herr;
            if (first_bad) atomicMin(first_bad, key_base | face_key(0, 0, 0, y0 + fy, x0 + fx));
        }
    }
    __syncthreads();
    // y phase, cells -1..TY of each tile column
    for (int it = threadIdx.x; it < L::AYN; it += NT) {
        const int lx = it % TX, ly = it / TX;
        if (x0 + lx >= nx || y0 - 1 + ly > ny) continue;
        mh_predict<1, LIM>(sU + (ly + 1) * L::UX + lx + 2, PL, L::UX, g1, hdy, sA + it, L::AN,
                           sA + 4 * L::AN + it, L::AN);
    }
    __syncthreads();
    // y faces 0..TY of each tile column
    for (int it = threadIdx.x; it < TX * (TY + 1); it += NT) {
        const int gx = it % TX, gy = it / TX;
        if (x0 + gx >= nx || y0 + gy > ny) continue;
        const int bad = mh_face<1>(sA + 4 * L::AN + gy * TX + gx, L::AN, sA + (gy + 1) * TX + gx, L::AN, g, g1,
                                   sG + gy * TX + gx, (TY + 1) * TX);
        if (bad && owned_face(y0 + gy, gy, TY, ny, x0 + gx, nx)) {
            ++herr;
            if (first_bad) atomicMin(first_bad, key_base | face_key(0, 0, 1, y0 + gy, x0 + gx));
        }
    }
    __syncthreads();
    return herr;
}

// Conservative update + forward Euler of output cell (ox, oy) of the tile, variable v
// (calculate_spatial_update, muscl_hancock.cpp:348-376; forward_euler.cpp:19-29)
template <int TX, int TY>
__device__ __forceinline__ double mh_update(const double* __restrict__ sU, const double* __restrict__ sF,
                                            const double* __restrict__ sG, int v, int ox, int oy,
                                            double dt, double one_dx, double one_dy) {
    using L = MhTile<TX, TY>;
    const double Lv = (one_dx * (sF[(v * TY + oy) * (TX + 1) + ox] - sF[(v * TY + oy) * (TX + 1) + ox + 1])) +
                      (one_dy * (sG[(v * (TY + 1) + oy) * TX + ox] - sG[(v * (TY + 1) + oy + 1) * TX + ox]));
    return dt * Lv + sU[(v * L::UY + oy + 2) * L::UX + ox + 2];
}

}  // namespace hf
