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

// Computes sF and sG from sU.  Ends with __syncthreads().  Returns the number of owned
// faces whose HLLC took the zero-flux branch (tile origin x0, y0 in interior cells).
template <int TX, int TY, int NT, int LIM>
__device__ __forceinline__ int mh_tile_fluxes(const double* __restrict__ sU, double* __restrict__ sA,
                                              double* __restrict__ sF, double* __restrict__ sG,
                                              double g, double g1, double hdx, double hdy, int x0,
                                              int y0, int nx, int ny) {
    using L = MhTile<TX, TY>;
    int herr = 0;
    // x phase: slopes, extrapolation, half-step predictor of the x face pair, cells -1..TX
    for (int it = threadIdx.x; it < L::AXN; it += NT) {
        const int lx = it % (TX + 2), ly = it / (TX + 2);
        const int sx = lx + 1, sy = ly + 2;
        double e0[4], e1[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const double* row = sU + (v * L::UY + sy) * L::UX;
            const double u0 = row[sx];
            const double s = slope<LIM>(row[sx - 1], u0, row[sx + 1]);
            const double hs = half(s);
            e0[v] = u0 - hs;
            e1[v] = u0 + hs;
        }
        Prim w0 = to_prim(g1, e0[0], e0[1], e0[2], e0[3]);
        Prim w1 = to_prim(g1, e1[0], e1[1], e1[2], e1[3]);
        double f0[4], f1[4];
        flux<0>(w0, f0);
        flux<0>(w1, f1);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const double d = hdx * (f0[v] - f1[v]);
            sA[(0 * 4 + v) * L::AN + it] = e0[v] + d;
            sA[(1 * 4 + v) * L::AN + it] = e1[v] + d;
        }
    }
    __syncthreads();
    // x faces 0..TX of each tile row (face f is the left face of output cell f)
    for (int it = threadIdx.x; it < (TX + 1) * TY; it += NT) {
        const int fx = it % (TX + 1), fy = it / (TX + 1);
        const int al = fy * (TX + 2) + fx;
        double UL[4], UR[4], F[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            UL[v] = sA[(1 * 4 + v) * L::AN + al];
            UR[v] = sA[(0 * 4 + v) * L::AN + al + 1];
        }
        const int bad = hllc_cons<0>(g, g1, UL, UR, F);
        herr += bad && owned_face(x0 + fx, fx, TX, nx, y0 + fy, ny);
#pragma unroll
        for (int v = 0; v < 4; ++v) sF[(v * TY + fy) * (TX + 1) + fx] = F[v];
    }
    __syncthreads();
    // y phase, cells -1..TY of each tile column
    for (int it = threadIdx.x; it < L::AYN; it += NT) {
        const int lx = it % TX, ly = it / TX;
        const int sx = lx + 2, sy = ly + 1;
        double e2[4], e3[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const double* col = sU + (v * L::UY + sy) * L::UX + sx;
            const double u0 = col[0];
            const double s = slope<LIM>(col[-L::UX], u0, col[L::UX]);
            const double hs = half(s);
            e2[v] = u0 - hs;
            e3[v] = u0 + hs;
        }
        Prim w2 = to_prim(g1, e2[0], e2[1], e2[2], e2[3]);
        Prim w3 = to_prim(g1, e3[0], e3[1], e3[2], e3[3]);
        double f2[4], f3[4];
        flux<1>(w2, f2);
        flux<1>(w3, f3);
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const double d = hdy * (f2[v] - f3[v]);
            sA[(0 * 4 + v) * L::AN + it] = e2[v] + d;
            sA[(1 * 4 + v) * L::AN + it] = e3[v] + d;
        }
    }
    __syncthreads();
    // y faces 0..TY of each tile column
    for (int it = threadIdx.x; it < TX * (TY + 1); it += NT) {
        const int gx = it % TX, gy = it / TX;
        double UB[4], UT[4], F[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            UB[v] = sA[(1 * 4 + v) * L::AN + gy * TX + gx];
            UT[v] = sA[(0 * 4 + v) * L::AN + (gy + 1) * TX + gx];
        }
        const int bad = hllc_cons<1>(g, g1, UB, UT, F);
        herr += bad && owned_face(y0 + gy, gy, TY, ny, x0 + gx, nx);
#pragma unroll
        for (int v = 0; v < 4; ++v) sG[(v * (TY + 1) + gy) * TX + gx] = F[v];
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
