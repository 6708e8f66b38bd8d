/* HyperFlow-GB300 -- C ABI of the learned coarse solver.
 *
 * No counterpart in the reference.  An FP32 MUSCL-Hancock + HLLC step (the reference's
 * scheme, src/fvm_2d_cart/scheme/muscl_hancock/muscl_hancock.cpp:41-376, in single precision
 * on one n x n block with transmissive sides) whose face fluxes receive a correction from a
 * small MLP (64 -> 64 -> 64 -> 4, GELU; BF16 weights on the tensor cores, FP32 accumulation)
 * so that the coarse grid reproduces a box-filtered fine-grid solution.  Corrections that
 * break density/pressure positivity or exceed a per-cell bound fall back to the plain flux.
 * Training (one-step loss against filtered fine states, hand-written backward and Adam) runs
 * on the device.  States are SoA FP32 [4][n][n] (rho, rho u, rho v, E).
 */
#ifndef HYPERFLOW_GB300_LEARNED_H
#define HYPERFLOW_GB300_LEARNED_H

#include <stddef.h>
#include <stdint.h>

#include "hyperflow_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hf_lc hf_lc;

/* n x n cells of spacing dx; limiter 0 = MinBee, 1 = Van Leer */
int hf_lc_create(int n, double dx, double gamma, double cfl, int limiter, hf_lc** out);
void hf_lc_destroy(hf_lc* L);
const char* hf_lc_last_error_message(const hf_lc* L);

/* packed FP32 parameters: W1[64][64] b1[64] W2[64][64] b2[64] W3[4][64] b3[4] (y = W x + b) */
int hf_lc_num_params(int* n);
int hf_lc_set_params(hf_lc* L, const float* params);   /* also resets the Adam moments */
int hf_lc_get_params(hf_lc* L, float* params);
/* the guard's per-cell bound: a corrected density or energy change larger than bound x the
 * plain update's change rejects the correction */
int hf_lc_set_bound(hf_lc* L, double bound);
/* guard mode 0 (default): the change bound above; 1: local-extremum bounds (flux-corrected
 * transport, Zalesak 1979) -- the corrected density and energy must stay within the min and max,
 * over the cell and its 8 neighbours, of the old state and of the plain update.  Both reject
 * non-positive density or pressure. */
int hf_lc_set_guard_mode(hf_lc* L, int mode);
/* on != 0: training steps apply the guard as inference does (rejected faces take the plain
 * flux and pass no gradient); default off */
int hf_lc_set_train_guard(hf_lc* L, int on);
/* How an inference step runs.  fused 1 (default): the features, the MLP and the corrections
 * in one kernel per 256-face tile (face_kernel), the plain fluxes in their own kernel; 2: the
 * plain fluxes inside face_kernel as well; 0: separate kernels (plain flux, features, MLP
 * forward, correction).  All three give the same results bit for bit.  ctas_per_sm (0..4, 0 = as
 * many as fit) sets face_kernel's launch shape. */
int hf_lc_set_fused(hf_lc* L, int fused, int ctas_per_sm);

int hf_lc_set_state(hf_lc* L, const float* U);
int hf_lc_get_state(hf_lc* L, float* U);
int hf_lc_set_time(hf_lc* L, double t);
int hf_lc_get_time(hf_lc* L, double* t);

/* CFL dt of the current state: cfl * dx / max(max(|u|,|v|) + c) */
int hf_lc_cfl_dt(hf_lc* L, double* dt);
/* one step with dt; use_mlp != 0 applies the guarded correction; rejected_cells (optional)
 * counts cells whose faces' corrections were rejected -- given, the call waits for the step and
 * reports a device error; null, the step is only enqueued on the solver's stream */
int hf_lc_step(hf_lc* L, double dt, int use_mlp, int64_t* rejected_cells);
/* steps with the CFL dt until t_end (dt clamped to reach it) */
int hf_lc_run_to(hf_lc* L, double t_end, int use_mlp, int64_t* steps, int64_t* rejected_cells);

/* one Adam iteration on the pair (U0 -> T over dt) with variable weights w[4]; loss written.
 * U0 null trains from the solver's current state (e.g. after its own steps), which stays. */
int hf_lc_train_step(hf_lc* L, const float* U0, const float* T, const float* w, double dt, double lr,
                     double* loss);

/* the MLP alone (for checking it): y[nf][4] = MLP(x) with x BF16 bit patterns [nf][64];
 * backward gives dL/dparams for dL/dy = dy (packed like the parameters) */
/* the MLP's inputs of every face for the current state (BF16 bits [nf][64], faces x first) and
 * the correction scale [nf][2] (rho_ref, c_ref): what the step feeds the network */
int hf_lc_features(hf_lc* L, uint16_t* x_bf16, float* scale);
int hf_lc_mlp_forward(hf_lc* L, const uint16_t* x_bf16, int nf, float* y);
int hf_lc_mlp_backward(hf_lc* L, const uint16_t* x_bf16, const float* dy, int nf, float* grad);
int hf_lc_stream(hf_lc* L, void** stream);

#ifdef __cplusplus
}
#endif
#endif
