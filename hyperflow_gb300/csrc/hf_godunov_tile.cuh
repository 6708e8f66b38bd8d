// The first-order Godunov tile computation shared by the per-block stencil (hf_cart.cu) and the
// batched persistent kernel (hf_batch.cu): GodunovScheme::calculate_fluxes_{x,y} +
// calculate_spatial_update (src/fvm_2d_cart/scheme/godunov/godunov.cpp:27-118) with the
// forward-Euler update (forward_euler.cpp:19-29).
//
// Input: sU, the tile's conservative state plus a 1-cell halo in shared memory,
// [4][TY+2][TX+2].  Each cell's primitives, sound speed and x/y fluxes are formed once (sQ) and
// shared by the two faces that use them.  Output: sF / sG, the HLLC fluxes of the tile's x faces
// [4][TY][TX+1] and y faces [4][TY+1][TX].
#pragma once

#include "hf_ctrl.h"
#include "hf_device.cuh"
#include "hf_mh_tile.cuh"   // owned_face

namespace hf {

template <int TX, int TY>
struct GoTile {
    static constexpr int UX = TX + 2, UY = TY + 2, NC = UX * UY;
    static constexpr int NQ = 12;   // u v p Et a fx0 fx1 fx2 fx3 fy0 fy2 fy3 (fy1 == fx2)
    static constexpr int U_SIZE = 4 * NC;
    static constexpr int Q_SIZE = NQ * NC;
    static constexpr int F_SIZE = 4 * TY * (TX + 1);
    static constexpr int G_SIZE = 4 * (TY + 1) * TX;
};

// Computes sF and sG from sU (tile origin x0, y0 in interior cells of an nx x ny block).  Ends
// with __syncthreads().  Returns the number of owned faces whose HLLC took the zero-flux branch;
// with first_bad, each such face's face_key (key_base: its step and block bits) is min-reduced
// there.  Cells beyond the first ghost layer and faces beyond the last face are skipped: no
// in-block cell reads them, and zero-filled states would only take the slow division paths.
template <int TX, int TY, int NT>
__device__ __forceinline__ int go_tile_fluxes(const double* __restrict__ sU, double* __restrict__ sQ,
                                              double* __restrict__ sF, double* __restrict__ sG, double g,
                                              double g1, int x0, int y0, int nx, int ny,
                                              unsigned long long* first_bad = nullptr,
                                              unsigned long long key_base = 0) {
    using L = GoTile<TX, TY>;
#define Q(k, cell) sQ[(k) * L::NC + (cell)]
    for (int cell = threadIdx.x; cell < L::NC; cell += NT) {
        if (x0 - 1 + cell % L::UX > nx || y0 - 1 + cell / L::UX > ny) continue;
        Prim w = to_prim(g1, sU[cell], sU[L::NC + cell], sU[2 * L::NC + cell], sU[3 * L::NC + cell]);
        double fx[4], fy[4];
        flux<0>(w, fx);
        flux<1>(w, fy);
        Q(0, cell) = w.u; Q(1, cell) = w.v; Q(2, cell) = w.p; Q(3, cell) = w.Et;
        Q(4, cell) = sound(g, w.r, w.p);
        Q(5, cell) = fx[0]; Q(6, cell) = fx[1]; Q(7, cell) = fx[2]; Q(8, cell) = fx[3];
        Q(9, cell) = fy[0]; Q(10, cell) = fy[2]; Q(11, cell) = fy[3];
    }
    __syncthreads();
    int herr = 0;
    auto load = [&](int cell, double* U, Prim& w, double& a, double* fx, double* fy) {
#pragma unroll
        for (int v = 0; v < 4; ++v) U[v] = sU[v * L::NC + cell];
        w.r = U[0]; w.u = Q(0, cell); w.v = Q(1, cell); w.p = Q(2, cell); w.Et = Q(3, cell); w.q = 0.0;
        a = Q(4, cell);
        if (fx) { fx[0] = Q(5, cell); fx[1] = Q(6, cell); fx[2] = Q(7, cell); fx[3] = Q(8, cell); }
        if (fy) { fy[0] = Q(9, cell); fy[1] = Q(7, cell); fy[2] = Q(10, cell); fy[3] = Q(11, cell); }
    };
    // x faces: face f of row r sits between tile cells (f-1, r) and (f, r)
    for (int it = threadIdx.x; it < (TX + 1) * TY; it += NT) {
        const int fx = it % (TX + 1), fy = it / (TX + 1);
        if (x0 + fx > nx || y0 + fy >= ny) continue;
        const int cl = (fy + 1) * L::UX + fx, cr = cl + 1;
        double UL[4], UR[4], FL[4], FR[4], F[4], aL, aR;
        Prim wL, wR;
        load(cl, UL, wL, aL, FL, nullptr);
        load(cr, UR, wR, aR, FR, nullptr);
        const int bad = hllc<0>(UL, wL, aL, FL, UR, wR, aR, FR, F);
        if (bad && owned_face(x0 + fx, fx, TX, nx, y0 + fy, ny)) {
            ++herr;
            if (first_bad) atomicMin(first_bad, key_base | face_key(0, 0, 0, y0 + fy, x0 + fx));
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) sF[(v * TY + fy) * (TX + 1) + fx] = F[v];
    }
    for (int it = threadIdx.x; it < TX * (TY + 1); it += NT) {
        const int gx = it % TX, gy = it / TX;
        if (x0 + gx >= nx || y0 + gy > ny) continue;
        const int cb = gy * L::UX + gx + 1, ct = cb + L::UX;
        double UB[4], UT[4], FB[4], FT[4], F[4], aB, aT;
        Prim wB, wT;
        load(cb, UB, wB, aB, nullptr, FB);
        load(ct, UT, wT, aT, nullptr, FT);
        const int bad = hllc<1>(UB, wB, aB, FB, UT, wT, aT, FT, F);
        if (bad && owned_face(y0 + gy, gy, TY, ny, x0 + gx, nx)) {
            ++herr;
            if (first_bad) atomicMin(first_bad, key_base | face_key(0, 0, 1, y0 + gy, x0 + gx));
        }
#pragma unroll
        for (int v = 0; v < 4; ++v) sG[(v * (TY + 1) + gy) * TX + gx] = F[v];
    }
#undef Q
    __syncthreads();
    return herr;
}

// Conservative update + forward Euler of output cell (ox, oy) of the tile, variable v
// (godunov.cpp:97-113; forward_euler.cpp:19-29)
template <int TX, int TY>
__device__ __forceinline__ double go_update(const double* __restrict__ sU, const double* __restrict__ sF,
                                            const double* __restrict__ sG, int v, int ox, int oy, double dt,
                                            double one_dx, double one_dy) {
    using L = GoTile<TX, TY>;
    const double Lv = (one_dx * (sF[(v * TY + oy) * (TX + 1) + ox] - sF[(v * TY + oy) * (TX + 1) + ox + 1])) +
                      (one_dy * (sG[(v * (TY + 1) + oy) * TX + ox] - sG[(v * (TY + 1) + oy + 1) * TX + ox]));
    return dt * Lv + sU[v * L::NC + (oy + 1) * L::UX + ox + 1];
}

}  // namespace hf
