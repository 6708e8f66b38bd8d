/* Test infrastructure only -- the oracle.
 *
 * A plain-C, CPU restatement of the reference solver's time step (qcrm/HyperFlow,
 * src/fvm_2d_cart and src/fvm_2d_uns), written to reproduce the reference's
 * floating-point results bit for bit: same operations, same evaluation order, no
 * FMA contraction (built with -ffp-contract=off).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it, and only to check results or as the timed
 * CPU baseline.  The product never calls it.
 *
 * Parity of this restatement is pinned against the reference itself: the reference's
 * own sources, compiled in place by oracle/Makefile into oracle/_ref/, generate the
 * golden fixtures under tests/golden/, and tests/test_oracle_vs_reference.py compares
 * the two whenever oracle/_ref/ has been built.
 */
#ifndef HF_ORACLE_H
#define HF_ORACLE_H

#include <stdint.h>

#define HFO_MAXB 16

/* boundary kinds of src/fvm_2d_cart/simulation/parser/parser.cpp:441-463 */
enum { HFO_TRANSMISSIVE = 0, HFO_REFLECTIVE = 1, HFO_DIRICHLET = 2, HFO_INTERNAL = 3 };
/* sides in the order Mesh::apply_bcs visits them (mesh.cpp:33-38) */
enum { HFO_BOTTOM = 0, HFO_RIGHT = 1, HFO_TOP = 2, HFO_LEFT = 3 };

typedef struct {
    int scheme;             /* 0 Godunov (ghost 1), 1 MUSCL-Hancock (ghost 2) */
    int limiter;            /* 0 MinBee, 1 Van Leer */
    int nblocks;
    int ghost;
    double gamma, cfl;
    int64_t calls;          /* TimeStep calls made so far (timestep.cpp 'steps' - 1) */
    double t, t_end;
    int nx[HFO_MAXB], ny[HFO_MAXB];
    double xl[HFO_MAXB], xr[HFO_MAXB], yb[HFO_MAXB], yt[HFO_MAXB];
    int bc_type[HFO_MAXB][4];
    int bc_block[HFO_MAXB][4];
    double bc_state[HFO_MAXB][4][4];   /* Dirichlet conservative state per side */
    double *U[HFO_MAXB];               /* SoA [var][y][x] incl. ghosts, x fastest */
    int nthreads;
    int64_t hllc_errors;               /* times the HLLC "should not get here" branch ran */
    int64_t steps;                     /* hfo_advance calls completed */
    uint64_t first_bad;                /* least key (step, block, direction, j, i) of such a face */
    uint64_t first_nonpos;             /* least key (step, block, 0, j, i) of an interior cell a step
                                          left with density or pressure not positive (or NaN) */
} hfo_mesh;

#ifdef __cplusplus
extern "C" {
#endif

/* unit-level functions */
void hfo_cons_to_prim(double gamma, const double *u, double *w);
void hfo_prim_to_cons(double gamma, const double *w, double *u);
void hfo_cons_flux(double gamma, const double *u, int dir, double *f);
int hfo_hllc(double gamma, const double *ul, const double *ur, int dir, double *flux);
double hfo_limiter(int kind, double r);

/* initial conditions (conservative states), evaluated at cell centroids over the interior */
void hfo_init_quadrant(hfo_mesh *m, int b, double xi, double yi, const double *ne,
                       const double *nw, const double *sw, const double *se);
void hfo_init_constant(hfo_mesh *m, int b, const double *state);
void hfo_init_double(hfo_mesh *m, int b, double xlm, double xmr, const double *l,
                     const double *mid, const double *r);
void hfo_init_sphere(hfo_mesh *m, int b, double radius, double xo, double yo,
                     const double *in, const double *out);
/* shock-bubble (no reference counterpart): post-shock state for x <= shock_x, else the
 * bubble state inside the circle, else the ambient state */
void hfo_init_shock_bubble(hfo_mesh *m, int b, double shock_x, double bx, double by, double r,
                           const double *post, const double *bubble, const double *ambient);

/* the step pieces */
void hfo_apply_bcs(hfo_mesh *m);
double hfo_time_step(hfo_mesh *m);
void hfo_advance(hfo_mesh *m, double dt);
/* runs n steps (apply_bcs, dt, optional t_end clamp, blocks in order); writes each dt */
int hfo_run(hfo_mesh *m, int n, int clamp_t_end, double *dts);
/* Simulation::solve with its t_end and frame-output clamps and its frame cadence; frames are
 * every block's interior, SoA per block, with the reference's time labels */
int64_t hfo_solve(hfo_mesh *m, double interval, int64_t max_steps, double *dts, int64_t max_dts,
                  double *frames, double *frame_t, int64_t max_frames, int64_t *nframes);

/* unstructured Godunov (src/fvm_2d_uns): cells in order, their (cell, edge) pairs
 * contiguous in pair order; verts holds each cell's vertices, 2 doubles each */
void hfo_uns_geometry(int ncells, const int *nverts, const double *verts,
                      double *angle, double *length, double *area, double *rin);
int hfo_uns_run(double gamma, double cfl, int64_t *calls, int ncells, const int *pair_start,
                const int *pair_nbr, const double *angle, const double *length,
                const double *area, const double *rin, const double *inlet,
                double *U, int n, double *dts, int nthreads);
/* the least cell of a state [4][ncells] whose density or pressure is not positive, or -1 */
int64_t hfo_uns_first_nonpositive(double gamma, int ncells, const double *U);
/* the unstructured Simulation::solve with its t_end and frame clamps and frame cadence */
int64_t hfo_uns_solve(double g, double cfl, int64_t *calls, int ncells, const int *pair_start,
                      const int *pair_nbr, const double *angle, const double *length,
                      const double *area, const double *rin, const double *inlet, double *U,
                      double t_start, double t_end, double interval, double *t_out,
                      double *frames, double *frame_t, int64_t max_frames, int64_t *nframes,
                      int nthreads);

#ifdef __cplusplus
}
#endif
#endif
