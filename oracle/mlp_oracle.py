"""Test infrastructure only -- CPU oracle of the learned solver's MLP.

Restates the network the CUDA kernels of the learned coarse solver evaluate:
64 -> 64 (GELU, tanh form) -> 64 (GELU) -> 4, y = W x + b, with the inputs, the weights
and the two hidden activations rounded to BF16 (round to nearest even) exactly where the
tensor-core kernels round them, and every product and sum in float64.  The backward gives
dL/dparams for a given dL/dy through that same forward (weights and activations as BF16
values), packed like the parameters: W1[64][64] b1[64] W2[64][64] b2[64] W3[4][64] b3[4].
The kernels add each bias inside the MMA as two BF16 parts (its rounding and the rounded
remainder), within about 2^-17 of the bias; the oracle adds the bias itself.
"""
from __future__ import annotations

import numpy as np

H, NIN, NOUT = 64, 64, 4
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * NIN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + NOUT * H
NPARAM = OFF_B3 + NOUT


def bf16_bits(x) -> np.ndarray:
    """float32 -> BF16 bit patterns, round to nearest even (NaN kept quiet)."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    out = ((u + rounding) >> 16).astype(np.uint16)
    nan = np.isnan(f)
    out[nan] = ((u[nan] >> 16) | 0x40).astype(np.uint16)
    return out


def bf16_value(bits: np.ndarray) -> np.ndarray:
    return (bits.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def round_bf16(x) -> np.ndarray:
    return bf16_value(bf16_bits(np.asarray(x, dtype=np.float32)))


def gelu(z):
    k = np.sqrt(2.0 / np.pi)
    return 0.5 * z * (1.0 + np.tanh(k * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    k = np.sqrt(2.0 / np.pi)
    u = k * (z + 0.044715 * z ** 3)
    t = np.tanh(u)
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * k * (1.0 + 3 * 0.044715 * z * z)


def forward(params, x_bits, rounding: bool = True):
    """rounding=False evaluates the same network without BF16 rounding (float64 weights
    and activations): the function whose derivative the backward formulas are."""
    W1, b1, W2, b2, W3, b3 = unpack(params) if rounding else \
        (np.asarray(a, np.float64) for a in unpack(np.asarray(params, np.float64)))
    x = bf16_value(x_bits)
    rnd = round_bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    w1, w2, w3 = rnd(W1), rnd(W2), rnd(W3)
    z1 = x @ w1.T + np.asarray(b1, np.float64)
    h1 = rnd(gelu(z1))
    z2 = h1 @ w2.T + np.asarray(b2, np.float64)
    h2 = rnd(gelu(z2))
    y = h2 @ w3.T + np.asarray(b3, np.float64)
    return y, (x, z1, h1, z2, h2, w2, w3)


def unpack(params):
    p = np.asarray(params)
    W1 = p[OFF_W1:OFF_B1].reshape(H, NIN)
    b1 = p[OFF_B1:OFF_W2]
    W2 = p[OFF_W2:OFF_B2].reshape(H, H)
    b2 = p[OFF_B2:OFF_W3]
    W3 = p[OFF_W3:OFF_B3].reshape(NOUT, H)
    b3 = p[OFF_B3:NPARAM]
    return W1, b1, W2, b2, W3, b3


def backward(params, x_bits, dy, rounding: bool = True):
    y, (x, z1, h1, z2, h2, w2, w3) = forward(params, x_bits, rounding)
    dy = np.asarray(dy, dtype=np.float64)
    g = np.zeros(NPARAM)
    g[OFF_W3:OFF_B3] = (dy.T @ h2).ravel()
    g[OFF_B3:NPARAM] = dy.sum(0)
    dz2 = (dy @ w3) * gelu_grad(z2)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    dz1 = (dz2 @ w2) * gelu_grad(z1)
    g[OFF_W1:OFF_B1] = (dz1.T @ x).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    return g


def features(U, gamma: float):
    """The MLP's inputs for every face, restating hf_learned.cu's feature kernel in float32
    (same operations, same order, IEEE float32 rounding): faces x first ([n][n+1], face i of
    row j between cells i-1 and i), then y; per face the 4x4 primitive stencil (normal offsets
    -1..2 outer, tangential -1..2 inner; cells mirrored past the edges) as rho (1/rho_ref) - 1,
    u_n (1/c_ref), u_t (1/c_ref), p (1/p_ref) - 1 with rho_ref, p_ref the two face cells' means,
    c_ref = sqrt(max(gamma p_ref / rho_ref, 1e-12)) and each reciprocal a rounded float32
    division.  Returns (BF16 bits [nf][64], scale [nf][2] = rho_ref, c_ref)."""
    U = np.asarray(U, np.float32)
    n = U.shape[1]
    g = np.float32(gamma)
    g1 = np.float32(gamma - 1.0)
    r, ru, rv, E = U[0], U[1], U[2], U[3]
    with np.errstate(all="ignore"):
        u = ru / r
        v = rv / r
        q = u * u + v * v
        p = g1 * (E - np.float32(0.5) * r * q)
    idx = np.arange(-3, n + 3)
    m = np.where(idx < 0, -1 - idx, np.where(idx >= n, 2 * n - 1 - idx, idx))
    m = np.clip(m, 0, n - 1)

    def at(a, jj, ii):   # a[mir(j)][mir(i)] for index arrays
        return a[m[jj + 3], m[ii + 3]]

    out_x, out_s = [], []
    for d in (0, 1):
        if d == 0:
            jj, ii = np.meshgrid(np.arange(n), np.arange(n + 1), indexing="ij")
            il, jl = ii - 1, jj
        else:
            jj, ii = np.meshgrid(np.arange(n + 1), np.arange(n), indexing="ij")
            il, jl = ii, jj - 1
        il, jl = il.ravel(), jl.ravel()
        ni, nj = (1, 0) if d == 0 else (0, 1)
        ti, tj = (0, 1) if d == 0 else (1, 0)
        with np.errstate(all="ignore"):
            rr = np.float32(0.5) * (at(r, jl, il) + at(r, jl + nj, il + ni))
            pr = np.float32(0.5) * (at(p, jl, il) + at(p, jl + nj, il + ni))
            cref = np.sqrt(np.maximum(g * pr / rr, np.float32(1e-12)))
            one = np.float32(1.0)
            irr, ipr, ic = one / rr, one / pr, one / cref
            cols = []
            for a in (-1, 0, 1, 2):
                for b in (-1, 0, 1, 2):
                    ci, cj = il + a * ni + b * ti, jl + a * nj + b * tj
                    wr, wu, wv, wp = at(r, cj, ci), at(u, cj, ci), at(v, cj, ci), at(p, cj, ci)
                    un, ut = (wu, wv) if d == 0 else (wv, wu)
                    cols += [wr * irr - one, un * ic, ut * ic, wp * ipr - one]
        out_x.append(np.stack(cols, axis=1))
        out_s.append(np.stack([rr, cref], axis=1))
    x = np.concatenate(out_x).astype(np.float32)
    return bf16_bits(x), np.concatenate(out_s).astype(np.float32)
