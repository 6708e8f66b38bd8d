/* Test infrastructure only -- the oracle (see hf_oracle.h).
 *
 * Every function restates one reference function and names it (path:line within the
 * reference project).  Expressions keep the reference's operand order, which C
 * evaluates left to right exactly as the C++ does; std::min / std::max are restated
 * as the comparisons the standard library performs, so NaN propagation matches.
 */
#include "hf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846 /* the value glibc's <math.h> gives M_PI */
#endif

#define TOL 1e-6  /* MUSCLHancockScheme::tol (muscl_hancock.cpp:32), Limiter tol (parser.cpp:231) */

/* std::min(a, b) == (b < a) ? b : a ; std::max(a, b) == (a < b) ? b : a */
static inline double smin(double a, double b) { return (b < a) ? b : a; }
static inline double smax(double a, double b) { return (a < b) ? b : a; }

/* sign() of muscl_hancock.cpp:8-11 */
static inline double sgn(double v) { return (double)((v > 0) - (v < 0)); }

/* ---------------- model: src/fvm_2d_cart/model/euler_ideal_gas/euler_ideal_gas.cpp ------- */

/* cons_to_prim, euler_ideal_gas.cpp:76-92 */
void hfo_cons_to_prim(double g, const double *c, double *w) {
    double rho = c[0], rho_u = c[1], rho_v = c[2], E = c[3];
    double u = rho_u / rho;
    double v = rho_v / rho;
    w[0] = rho;
    w[1] = u;
    w[2] = v;
    w[3] = (g - 1.0) * (E - 0.5 * rho * (u * u + v * v));
}

/* prim_to_cons, euler_ideal_gas.cpp:96-109 */
void hfo_prim_to_cons(double g, const double *w, double *c) {
    double rho = w[0], u = w[1], v = w[2], p = w[3];
    c[0] = rho;
    c[1] = rho * u;
    c[2] = rho * v;
    c[3] = p / (g - 1.0) + 0.5 * rho * (u * u + v * v);
}

/* prim_internal_energy + prim_total_energy, euler_ideal_gas.cpp:32-46 */
static inline double prim_total_energy(double g, const double *w) {
    double e = w[3] / (w[0] * (g - 1.0));
    return w[0] * (0.5 * (w[1] * w[1] + w[2] * w[2]) + e);
}

/* prim_speed_of_sound, euler_ideal_gas.cpp:60-64 */
static inline double sound_speed(double g, const double *w) { return sqrt(g * w[3] / w[0]); }

/* cons_flux_x / cons_flux_y, euler_ideal_gas.cpp:113-149 */
void hfo_cons_flux(double g, const double *c, int dir, double *f) {
    double w[4];
    hfo_cons_to_prim(g, c, w);
    double E = prim_total_energy(g, w);
    double rho = w[0], u = w[1], v = w[2], p = w[3];
    if (dir == 0) {
        f[0] = rho * u;
        f[1] = rho * u * u + p;
        f[2] = rho * u * v;
        f[3] = u * (E + p);
    } else {
        f[0] = rho * v;
        f[1] = rho * u * v;
        f[2] = rho * v * v + p;
        f[3] = v * (E + p);
    }
}

/* ---------------- HLLC: src/fvm_2d_cart/scheme/riemann/riemann_hllc/riemann_hllc.cpp ------- */

/* calc_U_k, riemann_hllc.cpp:37-63 */
static void calc_U_k(double g, const double *wK, double SK, double Ss, int dir, double *UK) {
    double dK = wK[0], uK = wK[1], vK = wK[2], pK = wK[3];
    double EK = prim_total_energy(g, wK);
    if (dir == 0) {
        double coef = dK * ((SK - uK) / (SK - Ss));
        UK[0] = coef;
        UK[1] = coef * Ss;
        UK[2] = coef * vK;
        UK[3] = coef * (EK / dK + (Ss - uK) * (Ss + (pK / (dK * (SK - uK)))));
    } else {
        double coef = dK * ((SK - vK) / (SK - Ss));
        UK[0] = coef;
        UK[1] = coef * uK;
        UK[2] = coef * Ss;
        UK[3] = coef * (EK / dK + (Ss - vK) * (Ss + (pK / (dK * (SK - vK)))));
    }
}

/* calc_hllc_flux, riemann_hllc.cpp:169-212 (with calc_wave_speeds_direct_min_max 127-150,
 * calc_S_star 67-97, calc_F_star 153-164).  Returns 1 when the "should not get here"
 * branch (199-211) produced the zero flux. */
int hfo_hllc(double g, const double *UL, const double *UR, int dir, double *F) {
    double wL[4], wR[4];
    hfo_cons_to_prim(g, UL, wL);
    hfo_cons_to_prim(g, UR, wR);
    double aL = sqrt(g * wL[3] / wL[0]);
    double aR = sqrt(g * wR[3] / wR[0]);
    double velL = dir == 0 ? wL[1] : wL[2];
    double velR = dir == 0 ? wR[1] : wR[2];
    double SL = smin(velL - aL, velR - aR);
    double SR = smax(velL + aL, velR + aR);
    double FL[4], FR[4];
    hfo_cons_flux(g, UL, dir, FL);
    hfo_cons_flux(g, UR, dir, FR);
    double dL = wL[0], pL = wL[3], dR = wR[0], pR = wR[3];
    double num = pR - pL + dL * velL * (SL - velL) - dR * velR * (SR - velR);
    double den = dL * (SL - velL) - dR * (SR - velR);
    double Ss = num / den;
    double ULs[4], URs[4];
    calc_U_k(g, wL, SL, Ss, dir, ULs);
    calc_U_k(g, wR, SR, Ss, dir, URs);
    if (0.0 <= SL) {
        memcpy(F, FL, sizeof FL);
    } else if (SL <= 0.0 && 0.0 <= Ss) {
        for (int i = 0; i < 4; ++i) F[i] = FL[i] + SL * (ULs[i] - UL[i]);
    } else if (Ss <= 0.0 && 0.0 <= SR) {
        for (int i = 0; i < 4; ++i) F[i] = FR[i] + SR * (URs[i] - UR[i]);
    } else if (0.0 >= SR) {
        memcpy(F, FR, sizeof FR);
    } else {
        for (int i = 0; i < 4; ++i) F[i] = 0.0;
        return 1;
    }
    return 0;
}

/* ---------------- limiters: src/fvm_2d_cart/scheme/limiter ---------------------------- */

/* Limiter::denom_tol + xi_right with omega = 0, beta = 1 (limiter.cpp:26-53, parser.cpp:231) */
static inline double xi_right(double r) {
    double num = 2.0 * 1.0;
    double den = 1.0 - 0.0 + (1.0 + 0.0) * r;
    if (fabs(den) < TOL) den = (den == 0.0) ? TOL : TOL * sgn(den);
    return num / den;
}

/* MinBeeLimiter::operator() minbee.cpp:29-38 ; VanLeerLimiter::operator() vanleer.cpp:29-36 */
double hfo_limiter(int kind, double r) {
    if (kind == 0) {
        if (r <= 0.0) return 0.0;
        if ((0.0 < r) && (r <= 1.0)) return r;
        return smin(1.0, xi_right(r));
    }
    if (r <= 0.0) return 0.0;
    return smin((2.0 * r) / (1.0 + r), xi_right(r));
}

/* ---------------- mesh: src/fvm_2d_cart/mesh/mesh_block/mesh_block.cpp ---------------- */

static inline int tot_x(const hfo_mesh *m, int b) { return m->nx[b] + 2 * m->ghost; }
static inline int tot_y(const hfo_mesh *m, int b) { return m->ny[b] + 2 * m->ghost; }
/* calculate_dx / calculate_dy, mesh_block.cpp:227-236 */
static inline double blk_dx(const hfo_mesh *m, int b) { return (m->xr[b] - m->xl[b]) / m->nx[b]; }
static inline double blk_dy(const hfo_mesh *m, int b) { return (m->yt[b] - m->yb[b]) / m->ny[b]; }

#define AT(m, b, v, i, j) ((m)->U[b][((size_t)(v) * tot_y(m, b) + (size_t)(j)) * tot_x(m, b) + (size_t)(i)])

/* cell-centroid sampling: calculate_centroids (mesh_block.cpp:239-257) and
 * initialise_field_values over the interior (mesh_block.cpp:215-224) */
typedef void (*ic_fn)(const void *ctx, double x, double y, double *out);

static void init_ic(hfo_mesh *m, int b, ic_fn fn, const void *ctx) {
    int g = m->ghost, tx = tot_x(m, b), ty = tot_y(m, b);
    double dx = blk_dx(m, b), dy = blk_dy(m, b);
    double sx = m->xl[b] - ((double)g - 0.5) * dx;
    double sy = m->yb[b] - ((double)g - 0.5) * dy;
    for (int i = g; i < tx - g; ++i)
        for (int j = g; j < ty - g; ++j) {
            double x = sx + (double)i * dx, y = sy + (double)j * dy, s[4];
            fn(ctx, x, y, s);
            for (int v = 0; v < 4; ++v) AT(m, b, v, i, j) = s[v];
        }
}

typedef struct { double xi, yi; const double *ne, *nw, *sw, *se; } quad_ctx;
/* QuadRiemannProblemInitialCondition::field_func_dim, quadrp.cpp:49-64 */
static void quad_fn(const void *p, double x, double y, double *o) {
    const quad_ctx *c = (const quad_ctx *)p;
    const double *s;
    if ((x <= c->xi) && (y <= c->yi)) s = c->sw;
    else if ((x <= c->xi) && (y > c->yi)) s = c->nw;
    else if ((x > c->xi) && (y <= c->yi)) s = c->se;
    else s = c->ne;
    memcpy(o, s, 4 * sizeof(double));
}
void hfo_init_quadrant(hfo_mesh *m, int b, double xi, double yi, const double *ne,
                       const double *nw, const double *sw, const double *se) {
    quad_ctx c = {xi, yi, ne, nw, sw, se};
    init_ic(m, b, quad_fn, &c);
}

/* ConstantInitialCondition, constant.cpp:34-40 */
static void const_fn(const void *p, double x, double y, double *o) {
    (void)x; (void)y;
    memcpy(o, p, 4 * sizeof(double));
}
void hfo_init_constant(hfo_mesh *m, int b, const double *state) { init_ic(m, b, const_fn, state); }

typedef struct { double xlm, xmr; const double *l, *mid, *r; } dbl_ctx;
/* DoubleRiemannProblemInitialCondition, doublerp.cpp:42-55 */
static void dbl_fn(const void *p, double x, double y, double *o) {
    const dbl_ctx *c = (const dbl_ctx *)p;
    (void)y;
    const double *s;
    if (x <= c->xlm) s = c->l;
    else if ((x > c->xlm) && (x <= c->xmr)) s = c->mid;
    else s = c->r;
    memcpy(o, s, 4 * sizeof(double));
}
void hfo_init_double(hfo_mesh *m, int b, double xlm, double xmr, const double *l,
                     const double *mid, const double *r) {
    dbl_ctx c = {xlm, xmr, l, mid, r};
    init_ic(m, b, dbl_fn, &c);
}

typedef struct { double rad, xo, yo; const double *in, *out; } sph_ctx;
/* SphericalRiemannProblemInitialCondition, sphericalrp.cpp:62-72 */
static void sph_fn(const void *p, double x, double y, double *o) {
    const sph_ctx *c = (const sph_ctx *)p;
    const double *s = (((x - c->xo) * (x - c->xo) + (y - c->yo) * (y - c->yo)) <= (c->rad * c->rad))
                          ? c->in : c->out;
    memcpy(o, s, 4 * sizeof(double));
}
void hfo_init_sphere(hfo_mesh *m, int b, double radius, double xo, double yo,
                     const double *in, const double *out) {
    sph_ctx c = {radius, xo, yo, in, out};
    init_ic(m, b, sph_fn, &c);
}

typedef struct { double sx, bx, by, r; const double *post, *bub, *amb; } sb_ctx;
static void sb_fn(const void *p, double x, double y, double *o) {
    const sb_ctx *c = (const sb_ctx *)p;
    const double *s;
    if (x <= c->sx) s = c->post;
    else if (((x - c->bx) * (x - c->bx) + (y - c->by) * (y - c->by)) <= (c->r * c->r)) s = c->bub;
    else s = c->amb;
    memcpy(o, s, 4 * sizeof(double));
}
void hfo_init_shock_bubble(hfo_mesh *m, int b, double shock_x, double bx, double by, double r,
                           const double *post, const double *bubble, const double *ambient) {
    sb_ctx c = {shock_x, bx, by, r, post, bubble, ambient};
    init_ic(m, b, sb_fn, &c);
}

/* ---------------- boundaries: src/fvm_2d_cart/scheme/boundary ------------------------ */

static inline void copy_cell(hfo_mesh *m, int bd, int id, int jd, int bs, int is, int js) {
    for (int v = 0; v < 4; ++v) AT(m, bd, v, id, jd) = AT(m, bs, v, is, js);
}
static inline void set_cell(hfo_mesh *m, int b, int i, int j, const double *s) {
    for (int v = 0; v < 4; ++v) AT(m, b, v, i, j) = s[v];
}
static inline void neg(hfo_mesh *m, int b, int v, int i, int j) {
    AT(m, b, v, i, j) = -1.0 * AT(m, b, v, i, j);
}

/* one side of one block: transmissive_boundary.cpp:25-104, reflective_boundary.cpp:25-120,
 * dirichlet_boundary.cpp:25-104, internal_boundary.cpp:27-108 */
static void apply_side(hfo_mesh *m, int b, int side) {
    int g = m->ghost, tx = tot_x(m, b), ty = tot_y(m, b);
    int kind = m->bc_type[b][side];
    const double *st = m->bc_state[b][side];
    int e = m->bc_block[b][side];
    if (side == HFO_LEFT) {
        for (int j = 0; j < ty; ++j) {
            if (kind == HFO_DIRICHLET) {
                for (int k = 0; k < g; ++k) set_cell(m, b, g - 1 - k, j, st);
            } else if (kind == HFO_INTERNAL) {
                int etx = tot_x(m, e);
                if (g == 1) copy_cell(m, b, 0, j, e, etx - 2, j);
                else { copy_cell(m, b, 1, j, e, etx - 3, j); copy_cell(m, b, 0, j, e, etx - 4, j); }
            } else {
                if (g == 1) copy_cell(m, b, 0, j, b, 1, j);
                else { copy_cell(m, b, 1, j, b, 2, j); copy_cell(m, b, 0, j, b, 3, j); }
                if (kind == HFO_REFLECTIVE) {
                    if (g == 1) neg(m, b, 1, 0, j);
                    else { neg(m, b, 1, 1, j); neg(m, b, 1, 0, j); }
                }
            }
        }
    } else if (side == HFO_RIGHT) {
        for (int j = 0; j < ty; ++j) {
            if (kind == HFO_DIRICHLET) {
                for (int k = 0; k < g; ++k) set_cell(m, b, tx - g + k, j, st);
            } else if (kind == HFO_INTERNAL) {
                if (g == 1) copy_cell(m, b, tx - 1, j, e, 1, j);
                else { copy_cell(m, b, tx - 1, j, e, 3, j); copy_cell(m, b, tx - 2, j, e, 2, j); }
            } else {
                if (g == 1) copy_cell(m, b, tx - 1, j, b, tx - 2, j);
                else { copy_cell(m, b, tx - 2, j, b, tx - 3, j); copy_cell(m, b, tx - 1, j, b, tx - 4, j); }
                if (kind == HFO_REFLECTIVE) {
                    if (g == 1) neg(m, b, 1, tx - 1, j);
                    else { neg(m, b, 1, tx - 2, j); neg(m, b, 1, tx - 1, j); }
                }
            }
        }
    } else if (side == HFO_BOTTOM) {
        for (int i = 0; i < tx; ++i) {
            if (kind == HFO_DIRICHLET) {
                for (int k = 0; k < g; ++k) set_cell(m, b, i, g - 1 - k, st);
            } else if (kind == HFO_INTERNAL) {
                int ety = tot_y(m, e);
                if (g == 1) copy_cell(m, b, i, 0, e, i, ety - 2);
                else { copy_cell(m, b, i, 1, e, i, ety - 3); copy_cell(m, b, i, 0, e, i, ety - 4); }
            } else {
                if (g == 1) copy_cell(m, b, i, 0, b, i, 1);
                else { copy_cell(m, b, i, 1, b, i, 2); copy_cell(m, b, i, 0, b, i, 3); }
                if (kind == HFO_REFLECTIVE) {
                    if (g == 1) neg(m, b, 2, i, 0);
                    else { neg(m, b, 2, i, 1); neg(m, b, 2, i, 0); }
                }
            }
        }
    } else { /* top */
        for (int i = 0; i < tx; ++i) {
            if (kind == HFO_DIRICHLET) {
                for (int k = 0; k < g; ++k) set_cell(m, b, i, ty - g + k, st);
            } else if (kind == HFO_INTERNAL) {
                if (g == 1) copy_cell(m, b, i, ty - 1, e, i, 1);
                else { copy_cell(m, b, i, ty - 1, e, i, 3); copy_cell(m, b, i, ty - 2, e, i, 2); }
            } else {
                if (g == 1) copy_cell(m, b, i, ty - 1, b, i, ty - 2);
                else { copy_cell(m, b, i, ty - 2, b, i, ty - 3); copy_cell(m, b, i, ty - 1, b, i, ty - 4); }
                if (kind == HFO_REFLECTIVE) {
                    if (g == 1) neg(m, b, 2, i, ty - 1);
                    else { neg(m, b, 2, i, ty - 2); neg(m, b, 2, i, ty - 1); }
                }
            }
        }
    }
}

/* Mesh::apply_bcs, mesh.cpp:31-39: per block in order, bottom, right, top, left */
void hfo_apply_bcs(hfo_mesh *m) {
    for (int b = 0; b < m->nblocks; ++b)
        for (int s = 0; s < 4; ++s) apply_side(m, b, s);
}

/* ---------------- TimeStep::operator(), timestep.cpp:29-68 ----------------------------- */

double hfo_time_step(hfo_mesh *m) {
    double dtx = 1e16, dty = 1e16;
    for (int b = 0; b < m->nblocks; ++b) {
        double dx = blk_dx(m, b), dy = blk_dy(m, b);
        int tx = tot_x(m, b), ty = tot_y(m, b);
        /* min is order independent (NaN terms never replace the accumulator), so a
         * per-thread fold followed by a fold of the partials equals the serial loop */
#pragma omp parallel num_threads(m->nthreads > 0 ? m->nthreads : 1)
        {
            double lx = 1e16, ly = 1e16;
#pragma omp for schedule(static)
            for (int j = 0; j < ty; ++j)
                for (int i = 0; i < tx; ++i) {
                    double c4[4], w[4];
                    for (int v = 0; v < 4; ++v) c4[v] = AT(m, b, v, i, j);
                    hfo_cons_to_prim(m->gamma, c4, w);
                    double c = sound_speed(m->gamma, w);
                    lx = smin(lx, dx / (fabs(w[1]) + c));
                    ly = smin(ly, dy / (fabs(w[2]) + c));
                }
#pragma omp critical
            {
                dtx = smin(dtx, lx);
                dty = smin(dty, ly);
            }
        }
    }
    double final_cfl = (m->calls + 1 <= 10) ? 0.2 * m->cfl : m->cfl;
    m->calls++;
    return final_cfl * smin(dtx, dty);
}

/* The earliest zero-flux face as a key ordered by step, block, direction (0: x face i between
 * interior cells (i-1, j) and (i, j); 1: y face j between (i, j-1) and (i, j)), j, i; fields
 * saturate at 22, 4, 1, 18 and 19 bits.  Not in the reference, which prints a message
 * (riemann_hllc.cpp:199-211); the GPU records the same key. */
static uint64_t err_key(const hfo_mesh *m, int b, int dir, int j, int i) {
    uint64_t s = m->steps > 0x3FFFFF ? 0x3FFFFFu : (uint64_t)m->steps;
    uint64_t jj = j > 0x3FFFF ? 0x3FFFFu : (uint64_t)j, ii = i > 0x7FFFF ? 0x7FFFFu : (uint64_t)i;
    return (s << 42) | ((uint64_t)(b & 0xF) << 38) | ((uint64_t)(dir & 1) << 37) | (jj << 19) | ii;
}

static void note_bad(hfo_mesh *m, int b, int dir, int j, int i) {
    uint64_t k = err_key(m, b, dir, j, i);
#pragma omp critical(hfo_first_bad)
    if (k < m->first_bad) m->first_bad = k;
}

/* density and pressure (cons_to_prim) both positive; false for zero, negative and NaN.  Not in
 * the reference, which carries such a state on; the GPU records the earliest cell that fails it. */
static int physical(double g, const double *c) {
    double w[4];
    hfo_cons_to_prim(g, c, w);
    return c[0] > 0.0 && w[3] > 0.0;
}

/* the earliest interior cell of block b's new state (layout of m->U[b]) that is not physical */
static void note_nonpos(hfo_mesh *m, int b, const double *Unew) {
    int tx = tot_x(m, b), ty = tot_y(m, b), gh = m->ghost;
    size_t plane = (size_t)tx * ty;
    for (int j = 0; j < m->ny[b]; ++j)
        for (int i = 0; i < m->nx[b]; ++i) {
            size_t o = (size_t)(j + gh) * tx + (i + gh);
            double c[4] = {Unew[o], Unew[plane + o], Unew[2 * plane + o], Unew[3 * plane + o]};
            if (!physical(m->gamma, c)) {
                uint64_t k = err_key(m, b, 0, j, i);
                if (k < m->first_nonpos) m->first_nonpos = k;
                return;   /* row-major scan: the first one found is the least */
            }
        }
}

/* ---------------- Godunov block update, src/fvm_2d_cart/scheme/godunov/godunov.cpp:27-118,
 * fused with ForwardEulerODESolver (forward_euler.cpp:15-33) ---------------------------- */

static void godunov_block(hfo_mesh *m, int b, double dt, double *Unew) {
    int tx = tot_x(m, b), ty = tot_y(m, b), nx = m->nx[b], ny = m->ny[b];
    double one_dx = 1.0 / blk_dx(m, b), one_dy = 1.0 / blk_dy(m, b);
    size_t fxn = (size_t)(nx + 1) * ty, fyn = (size_t)tx * (ny + 1);
    double *FX = (double *)malloc(4 * fxn * sizeof(double));
    double *FY = (double *)malloc(4 * fyn * sizeof(double));
    int64_t err = 0;
    int nt = m->nthreads > 0 ? m->nthreads : 1;
    /* x fluxes: faces i in [0, nx], rows j in [1, ty-1) (the ghost rows' fluxes are unused) */
#pragma omp parallel for num_threads(nt) reduction(+ : err) schedule(static)
    for (int j = 1; j < ty - 1; ++j)
        for (int i = 0; i <= nx; ++i) {
            double a[4], c[4], f[4];
            for (int v = 0; v < 4; ++v) { a[v] = AT(m, b, v, i, j); c[v] = AT(m, b, v, i + 1, j); }
            int bad = hfo_hllc(m->gamma, a, c, 0, f);
            err += bad;
            if (bad && j <= ny) note_bad(m, b, 0, j - 1, i);
            for (int v = 0; v < 4; ++v) FX[((size_t)v * ty + j) * (nx + 1) + i] = f[v];
        }
#pragma omp parallel for num_threads(nt) reduction(+ : err) schedule(static)
    for (int j = 0; j <= ny; ++j)
        for (int i = 1; i < tx - 1; ++i) {
            double a[4], c[4], f[4];
            for (int v = 0; v < 4; ++v) { a[v] = AT(m, b, v, i, j); c[v] = AT(m, b, v, i, j + 1); }
            int bad = hfo_hllc(m->gamma, a, c, 1, f);
            err += bad;
            if (bad && i <= nx) note_bad(m, b, 1, j, i - 1);
            for (int v = 0; v < 4; ++v) FY[((size_t)v * (ny + 1) + j) * tx + i] = f[v];
        }
    m->hllc_errors += err;
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int j = 0; j < ty; ++j)
        for (int i = 0; i < tx; ++i)
            for (int v = 0; v < 4; ++v) {
                double L = 0.0;
                if (i >= 1 && i < tx - 1 && j >= 1 && j < ty - 1) {
                    L = (one_dx * (FX[((size_t)v * ty + j) * (nx + 1) + (i - 1)] -
                                   FX[((size_t)v * ty + j) * (nx + 1) + i])) +
                        (one_dy * (FY[((size_t)v * (ny + 1) + (j - 1)) * tx + i] -
                                   FY[((size_t)v * (ny + 1) + j) * tx + i]));
                }
                Unew[((size_t)v * ty + j) * tx + i] = dt * L + AT(m, b, v, i, j);
            }
    free(FX);
    free(FY);
}

/* ---------------- MUSCL-Hancock block update, muscl_hancock.cpp:41-376 ------------------ */

/* calculate_slope_limiters_{x,y} (67-134) + calculate_slopes_{x,y} (137-206), one variable */
static inline double mh_slope(int lim, double um, double u0, double up) {
    double dl = u0 - um, dr = up - u0;
    double dlc = dl, drc = dr;
    if (fabs(dlc) <= TOL) dlc = (dlc == 0.0) ? TOL : TOL * sgn(dlc);
    if (fabs(drc) <= TOL) drc = (drc == 0.0) ? TOL : TOL * sgn(drc);
    double r = dlc / drc;
    double xi = hfo_limiter(lim, r);
    return xi * (0.5 * (1.0 + 0.0) * dl + 0.5 * (1.0 - 0.0) * dr);
}

static void mh_block(hfo_mesh *m, int b, double dt, double dt_pred, double *Unew) {
    int tx = tot_x(m, b), ty = tot_y(m, b), nx = m->nx[b], ny = m->ny[b];
    double dx = blk_dx(m, b), dy = blk_dy(m, b);
    double hdx = 0.5 * dt_pred / dx, hdy = 0.5 * dt_pred / dy;   /* 248-249 */
    double one_dx = 1.0 / dx, one_dy = 1.0 / dy;                 /* 352-353 */
    size_t nc = (size_t)tx * ty;
    /* REC[f][v][cell]: f = 0 left, 1 right, 2 bottom, 3 top  (Vec4D of 217) */
    double *REC = (double *)calloc(16 * nc, sizeof(double));
    size_t fxn = (size_t)(nx + 1) * ny, fyn = (size_t)nx * (ny + 1);
    double *FX = (double *)malloc(4 * fxn * sizeof(double));
    double *FY = (double *)malloc(4 * fyn * sizeof(double));
    int nt = m->nthreads > 0 ? m->nthreads : 1;
    int lim = m->limiter;
    double g = m->gamma;
#define R(f, v, c) REC[((size_t)(f) * 4 + (v)) * nc + (c)]
    /* slopes, extrapolations (209-240) and the half-step predictor (243-281) */
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int j = 1; j < ty - 1; ++j)
        for (int i = 1; i < tx - 1; ++i) {
            size_t c = (size_t)j * tx + i;
            double e[4][4];
            for (int v = 0; v < 4; ++v) {
                double u0 = AT(m, b, v, i, j);
                double sx = mh_slope(lim, AT(m, b, v, i - 1, j), u0, AT(m, b, v, i + 1, j));
                double sy = mh_slope(lim, AT(m, b, v, i, j - 1), u0, AT(m, b, v, i, j + 1));
                e[0][v] = u0 - 0.5 * sx;
                e[1][v] = u0 + 0.5 * sx;
                e[2][v] = u0 - 0.5 * sy;
                e[3][v] = u0 + 0.5 * sy;
            }
            double fl[4], fr[4], fb[4], ft[4];
            hfo_cons_flux(g, e[0], 0, fl);
            hfo_cons_flux(g, e[1], 0, fr);
            hfo_cons_flux(g, e[2], 1, fb);
            hfo_cons_flux(g, e[3], 1, ft);
            for (int v = 0; v < 4; ++v) {
                R(0, v, c) = e[0][v] + hdx * (fl[v] - fr[v]);
                R(1, v, c) = e[1][v] + hdx * (fl[v] - fr[v]);
                R(2, v, c) = e[2][v] + hdy * (fb[v] - ft[v]);
                R(3, v, c) = e[3][v] + hdy * (fb[v] - ft[v]);
            }
        }
    int64_t err = 0;
    /* calculate_fluxes_x (284-313): face i between total cells i+1 and i+2, interior row j+2 */
#pragma omp parallel for num_threads(nt) reduction(+ : err) schedule(static)
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i <= nx; ++i) {
            size_t cl = (size_t)(j + 2) * tx + (i + 1), cr = (size_t)(j + 2) * tx + (i + 2);
            double a[4], c4[4], f[4];
            for (int v = 0; v < 4; ++v) { a[v] = R(1, v, cl); c4[v] = R(0, v, cr); }
            int bad = hfo_hllc(g, a, c4, 0, f);
            err += bad;
            if (bad) note_bad(m, b, 0, j, i);
            for (int v = 0; v < 4; ++v) FX[((size_t)v * ny + j) * (nx + 1) + i] = f[v];
        }
    /* calculate_fluxes_y (316-345) */
#pragma omp parallel for num_threads(nt) reduction(+ : err) schedule(static)
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i < nx; ++i) {
            size_t cb = (size_t)(j + 1) * tx + (i + 2), ct = (size_t)(j + 2) * tx + (i + 2);
            double a[4], c4[4], f[4];
            for (int v = 0; v < 4; ++v) { a[v] = R(3, v, cb); c4[v] = R(2, v, ct); }
            int bad = hfo_hllc(g, a, c4, 1, f);
            err += bad;
            if (bad) note_bad(m, b, 1, j, i);
            for (int v = 0; v < 4; ++v) FY[((size_t)v * (ny + 1) + j) * nx + i] = f[v];
        }
    m->hllc_errors += err;
#undef R
    /* calculate_spatial_update (348-376) + forward Euler (forward_euler.cpp:19-29) */
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int j = 0; j < ty; ++j)
        for (int i = 0; i < tx; ++i)
            for (int v = 0; v < 4; ++v) {
                double L = 0.0;
                if (i >= 2 && i < nx + 2 && j >= 2 && j < ny + 2) {
                    int ii = i - 2, jj = j - 2;
                    L = (one_dx * (FX[((size_t)v * ny + jj) * (nx + 1) + ii] -
                                   FX[((size_t)v * ny + jj) * (nx + 1) + ii + 1])) +
                        (one_dy * (FY[((size_t)v * (ny + 1) + jj) * nx + ii] -
                                   FY[((size_t)v * (ny + 1) + jj + 1) * nx + ii]));
                }
                Unew[((size_t)v * ty + j) * tx + i] = dt * L + AT(m, b, v, i, j);
            }
    free(REC);
    free(FX);
    free(FY);
}

/* the per-block loop of Simulation::solve (simulation.cpp:106-110): block b is advanced
 * and stored before block b+1 is computed; the MUSCL-Hancock predictor makes its own
 * TimeStep call on that partly advanced mesh (muscl_hancock.cpp:246) */
void hfo_advance(hfo_mesh *m, double dt) {
    for (int b = 0; b < m->nblocks; ++b) {
        size_t n = (size_t)4 * tot_x(m, b) * tot_y(m, b);
        double *Unew = (double *)malloc(n * sizeof(double));
        if (m->scheme == 0) {
            godunov_block(m, b, dt, Unew);
        } else {
            double dtp = hfo_time_step(m);
            mh_block(m, b, dt, dtp, Unew);
        }
        note_nonpos(m, b, Unew);
        memcpy(m->U[b], Unew, n * sizeof(double));
        free(Unew);
    }
    m->steps++;
}

/* Simulation::solve body (simulation.cpp:81-120) without the frame-output clamps */
int hfo_run(hfo_mesh *m, int n, int clamp_t_end, double *dts) {
    int taken = 0;
    for (int s = 0; s < n; ++s) {
        if (clamp_t_end && m->t == m->t_end) break;
        hfo_apply_bcs(m);
        double dt = hfo_time_step(m);
        if (clamp_t_end && m->t + dt > m->t_end) dt = m->t_end - m->t;
        hfo_advance(m, dt);
        if (dts) dts[taken] = dt;
        m->t += dt;
        ++taken;
    }
    return taken;
}

/* copies the interior of every block, SoA per block ([var][y][x]), into out */
static void frame_copy(const hfo_mesh *m, double *out) {
    size_t o = 0;
    for (int b = 0; b < m->nblocks; ++b)
        for (int v = 0; v < 4; ++v)
            for (int j = 0; j < m->ny[b]; ++j)
                for (int i = 0; i < m->nx[b]; ++i)
                    out[o++] = AT(m, b, v, i + m->ghost, j + m->ghost);
}

/* Simulation::solve (simulation.cpp:51-124) with its output cadence: the t_end clamp
 * (88-90), the frame clamp (98-102), a frame before the first update (93-96), a frame after
 * every update that starts within 1e-12 of the frame time, labelled with the time before
 * that update (106-113), and a last frame after the loop (122).  interval is
 * t_end / (duration * fps).  Frames beyond max_frames are counted but not stored; dts
 * beyond max_dts likewise.  Returns the steps taken. */
int64_t hfo_solve(hfo_mesh *m, double interval, int64_t max_steps, double *dts, int64_t max_dts,
                  double *frames, double *frame_t, int64_t max_frames, int64_t *nframes) {
    size_t fcells = 0;
    for (int b = 0; b < m->nblocks; ++b) fcells += (size_t)4 * m->nx[b] * m->ny[b];
    double cur = 0.0;
    int64_t nf = 0, taken = 0;
#define HFO_FRAME(label)                                                     \
    do {                                                                     \
        if (nf < max_frames) {                                               \
            if (frames) frame_copy(m, frames + (size_t)nf * fcells);         \
            if (frame_t) frame_t[nf] = (label);                              \
        }                                                                    \
        ++nf;                                                                \
    } while (0)
    for (int64_t n = 1; n < 1000000000 && taken < max_steps; ++n) {
        if (m->t == m->t_end) break;
        hfo_apply_bcs(m);
        double dt = hfo_time_step(m);
        if (m->t + dt > m->t_end) dt = m->t_end - m->t;
        if (cur == 0.0) HFO_FRAME(m->t);
        if ((m->t + dt > cur) && (cur > 0.0)) dt = cur - m->t;
        hfo_advance(m, dt);
        if (fabs(m->t - cur) < 1e-12) {
            HFO_FRAME(m->t);
            cur += interval;
        }
        if (dts && taken < max_dts) dts[taken] = dt;
        m->t += dt;
        ++taken;
    }
    if (m->t == m->t_end) HFO_FRAME(m->t);
#undef HFO_FRAME
    if (nframes) *nframes = nf;
    return taken;
}

/* ---------------- unstructured: src/fvm_2d_uns ------------------------------------------ */

/* Edge::calculate_outward_unit_normal + calculate_outward_normal_angle (edge.cpp:189-218),
 * Edge::get_length (edge.cpp:98-101 via Tensor1D::l2_norm), Polygon::calculate_volume
 * (polygon.cpp:172-186), Polygon::radius_incircle (polygon.cpp:72-94) */
void hfo_uns_geometry(int ncells, const int *nverts, const double *verts, double *angle,
                      double *length, double *area, double *rin) {
    size_t vo = 0, pair = 0;
    for (int c = 0; c < ncells; ++c) {
        int nv = nverts[c];
        const double *V = verts + 2 * vo;
        double el[4];
        for (int k = 0; k < nv; ++k) {
            int k1 = (k == nv - 1) ? 0 : k + 1;
            double p0 = V[2 * k1] - V[2 * k], p1 = V[2 * k1 + 1] - V[2 * k + 1];
            double n0 = p1, n1 = -1.0 * p0;
            double nl = sqrt(n0 * n0 + n1 * n1);
            n0 /= nl;
            n1 /= nl;
            angle[pair] = atan2(n1, n0) * 180.0 / M_PI;
            double d = 0.0;
            d += p0 * p0;
            d += p1 * p1;
            length[pair] = sqrt(d);
            el[k] = length[pair];
            ++pair;
        }
        double vol = 0.0;
        for (int k = 0; k < nv; ++k) {
            int k1 = (k == nv - 1) ? 0 : k + 1;
            vol += (V[2 * k] * V[2 * k1 + 1] - V[2 * k1] * V[2 * k + 1]);
        }
        vol *= 0.5;
        area[c] = vol;
        if (nv == 3) {
            double a = el[0], bb = el[1], cc = el[2];
            double s = (a + bb + cc) / 2.0;
            double num = s * (s - a) * (s - bb) * (s - cc);
            rin[c] = sqrt(num) / s;
        } else {
            double sh = 1e16;
            for (int k = 0; k < nv; ++k) sh = smin(el[k], sh);
            rin[c] = sh;
        }
        vo += nv;
    }
}

/* EulerIdealGasModel::rotate_flow_values, src/fvm_2d_uns/model/euler_ideal_gas/euler_ideal_gas.cpp:152-165 */
static inline void rotate(double deg, const double *f, double *o) {
    double a = deg * (M_PI / 180.0);
    o[0] = f[0];
    o[1] = cos(a) * f[1] + sin(a) * f[2];
    o[2] = -1.0 * sin(a) * f[1] + cos(a) * f[2];
    o[3] = f[3];
}

/* GodunovScheme::operator() (src/fvm_2d_uns/scheme/godunov/godunov.cpp:31-77) with
 * BoundaryConditions (src/fvm_2d_uns/scheme/boundary/boundary.cpp:29-69), the uns
 * TimeStep (src/fvm_2d_uns/scheme/timestep/timestep.cpp:29-62) and forward Euler. */
/* the unstructured TimeStep (uns timestep.cpp:29-62): dt for the next step; advances calls */
static double uns_dt(double g, double cfl, int64_t *calls, int ncells, const double *rin,
                     const double *U, int nt) {
    size_t N = (size_t)ncells;
    double dtr = 1e16;
#pragma omp parallel num_threads(nt)
    {
        double l = 1e16;
#pragma omp for schedule(static)
        for (int c = 0; c < ncells; ++c) {
            double c4[4] = {U[c], U[N + c], U[2 * N + c], U[3 * N + c]}, w[4];
            hfo_cons_to_prim(g, c4, w);
            double u = w[1], v = w[2], cs = sound_speed(g, w);
            l = smin(l, rin[c] / (fabs(sqrt(u * u + v * v)) + cs));
        }
#pragma omp critical
        dtr = smin(dtr, l);
    }
    double final_cfl = (*calls + 1 <= 10) ? 0.2 * cfl : cfl;
    (*calls)++;
    return final_cfl * dtr;
}

/* ODESolver(GodunovScheme) + set_cells_flow_values (godunov.cpp:31-77) with dt; U -> Un */
static void uns_update(double g, int ncells, const int *pair_start, const int *pair_nbr,
                       const double *angle, const double *length, const double *area,
                       const double *inlet, const double *U, double *Un, double dt, int nt) {
    size_t N = (size_t)ncells;
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int c = 0; c < ncells; ++c) {
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        double cv[4] = {U[c], U[N + c], U[2 * N + c], U[3 * N + c]};
        for (int p = pair_start[c]; p < pair_start[c + 1]; ++p) {
            double ang = angle[p], nb[4];
            int k = pair_nbr[p];
            if (k >= 0) {
                for (int v = 0; v < 4; ++v) nb[v] = U[v * N + k];
            } else if (k == -1) {            /* Reflective */
                double r[4];
                rotate(ang, cv, r);
                r[1] *= -1.0;
                rotate(-1.0 * ang, r, nb);
            } else if (k == -2) {            /* Transmissive */
                memcpy(nb, cv, sizeof nb);
            } else {                         /* Inlet */
                memcpy(nb, inlet, sizeof nb);
            }
            double rc[4], rn[4], rf[4], f[4];
            rotate(ang, cv, rc);
            rotate(ang, nb, rn);
            hfo_hllc(g, rc, rn, 0, rf);
            rotate(-1.0 * ang, rf, f);
            for (int v = 0; v < 4; ++v) acc[v] += length[p] * f[v];
        }
        double inv = 1.0 / area[c];
        for (int v = 0; v < 4; ++v) {
            double L = -1.0 * (inv * acc[v]);
            Un[v * N + c] = dt * L + cv[v];
        }
    }
}

/* the least cell of an unstructured state [4][ncells] whose density or pressure is not
 * positive (or NaN), -1 when none; the GPU records it per step */
int64_t hfo_uns_first_nonpositive(double g, int ncells, const double *U) {
    size_t N = (size_t)ncells;
    for (int c = 0; c < ncells; ++c) {
        double c4[4] = {U[c], U[N + c], U[2 * N + c], U[3 * N + c]};
        if (!physical(g, c4)) return c;
    }
    return -1;
}

int hfo_uns_run(double g, double cfl, int64_t *calls, int ncells, const int *pair_start,
                const int *pair_nbr, const double *angle, const double *length,
                const double *area, const double *rin, const double *inlet, double *U,
                int n, double *dts, int nthreads) {
    size_t N = (size_t)ncells;
    double *Un = (double *)malloc(4 * N * sizeof(double));
    int nt = nthreads > 0 ? nthreads : 1;
    for (int s = 0; s < n; ++s) {
        double dt = uns_dt(g, cfl, calls, ncells, rin, U, nt);
        uns_update(g, ncells, pair_start, pair_nbr, angle, length, area, inlet, U, Un, dt, nt);
        memcpy(U, Un, 4 * N * sizeof(double));
        if (dts) dts[s] = dt;
    }
    free(Un);
    return n;
}

/* the unstructured Simulation::solve (uns simulation.cpp:51-120) from t = t_start with the
 * t_end clamp, the frame dt clamp and the frame cadence of the Cartesian hfo_solve; frames
 * are the cell states [4][ncells].  Returns the steps taken. */
int64_t hfo_uns_solve(double g, double cfl, int64_t *calls, int ncells, const int *pair_start,
                      const int *pair_nbr, const double *angle, const double *length,
                      const double *area, const double *rin, const double *inlet, double *U,
                      double t_start, double t_end, double interval, double *t_out,
                      double *frames, double *frame_t, int64_t max_frames, int64_t *nframes,
                      int nthreads) {
    size_t N = (size_t)ncells;
    double *Un = (double *)malloc(4 * N * sizeof(double));
    int nt = nthreads > 0 ? nthreads : 1;
    double t = t_start, cur = 0.0;
    int64_t nf = 0, taken = 0;
#define HFO_UFRAME(src, label)                                                              \
    do {                                                                                    \
        if (nf < max_frames) {                                                              \
            if (frames) memcpy(frames + (size_t)nf * 4 * N, (src), 4 * N * sizeof(double)); \
            if (frame_t) frame_t[nf] = (label);                                             \
        }                                                                                   \
        ++nf;                                                                               \
    } while (0)
    for (int64_t n = 1; n < 1000000000; ++n) {
        if (t == t_end) break;
        double dt = uns_dt(g, cfl, calls, ncells, rin, U, nt);
        if (t + dt > t_end) dt = t_end - t;
        if (cur == 0.0) HFO_UFRAME(U, t);
        if ((t + dt > cur) && (cur > 0.0)) dt = cur - t;
        uns_update(g, ncells, pair_start, pair_nbr, angle, length, area, inlet, U, Un, dt, nt);
        memcpy(U, Un, 4 * N * sizeof(double));
        if (fabs(t - cur) < 1e-12) {
            HFO_UFRAME(U, t);
            cur += interval;
        }
        t += dt;
        ++taken;
    }
    HFO_UFRAME(U, t);
#undef HFO_UFRAME
    free(Un);
    if (t_out) *t_out = t;
    if (nframes) *nframes = nf;
    return taken;
}
