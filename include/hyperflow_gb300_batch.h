/* HyperFlow-GB300 -- C ABI of the batched single-block step.
 *
 * Many independent single-block cases advance together: the reference's MUSCL-Hancock step
 * (src/fvm_2d_cart/scheme/muscl_hancock/muscl_hancock.cpp:41-376) or Godunov step
 * (src/fvm_2d_cart/scheme/godunov/godunov.cpp:27-118), with TimeStep
 * (src/fvm_2d_cart/scheme/timestep/timestep.cpp:29-68) and ForwardEuler (forward_euler.cpp:15-33),
 * applied to every case with its own CFL dt, in one persistent cooperative kernel launch per
 * run of steps (optionally captured in a CUDA graph).  Each case's results equal what the
 * reference computes for that case alone, bit for bit.  A batch of one runs a small case's
 * whole loop in one launch.  Status codes are the HF_* codes of hyperflow_gb300.h.  States are
 * interior-only SoA [4][n][n].
 */
#ifndef HYPERFLOW_GB300_BATCH_H
#define HYPERFLOW_GB300_BATCH_H

#include <stddef.h>
#include <stdint.h>

#include "hyperflow_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hf_batch hf_batch;

/* manifest: {"cases": [case, case, ...]}, each a case file of the reference's schema
 * (src/fvm_2d_cart/simulation/parser/parser.cpp) with one square block, Transmissive on all
 * sides, Godunov or MUSCLHancock + HLLCEuler + ForwardEuler; all cases share the scheme, gamma,
 * cfl and limiter.
 * Replaces one JSONParser + Simulation per case.  On failure *out may be set; destroy it. */
int hf_batch_create(const char* manifest_json, size_t len, hf_batch** out);
void hf_batch_destroy(hf_batch* b);
const char* hf_batch_last_error_message(const hf_batch* b);

int hf_batch_sizes(const hf_batch* b, int* ninstances, int64_t* total_cells);
int hf_batch_instance_side(const hf_batch* b, int i, int* n);

/* compiled launch configurations: tile shape, threads per CTA, halo staging buffers */
int hf_batch_num_configs(int* n);
int hf_batch_config_info(int k, int* tile_x, int* tile_y, int* threads, int* stages);
int hf_batch_set_config(hf_batch* b, int k);
/* times every configuration for steps_per_trial steps on the live batch (the state is saved
 * and restored around the trials), selects the fastest; ms_per_step (optional, one entry per
 * configuration) receives the timings */
int hf_batch_autotune(hf_batch* b, int steps_per_trial, int* best, double* ms_per_step);

/* nsteps steps of every case in one persistent launch; use_graph replays a captured graph of
 * that launch (captured once per (configuration, nsteps)) */
int hf_batch_run(hf_batch* b, int64_t nsteps, int use_graph);
int hf_batch_sync(hf_batch* b);

/* one case's state (Mesh block fields without ghosts, mesh_block.cpp:155-164) */
int hf_batch_get_state(hf_batch* b, int i, double* out);
int hf_batch_set_state(hf_batch* b, int i, const double* in);
int hf_batch_instance_time(hf_batch* b, int i, double* t, double* last_dt);
int hf_batch_counters(hf_batch* b, int64_t* steps, int64_t* calls, int64_t* hllc_errors);
/* the earliest cell a step left with a density or pressure (cons_to_prim) that is not positive --
 * zero, negative or NaN -- since creation or hf_batch_clear_error_cell: the least (step, case,
 * j, i), step counting the steps completed before it; all -1 when there is none.  The run
 * continues, as the reference's does; there is no strict mode in a batch. */
int hf_batch_last_nonpositive_cell(hf_batch* b, int* instance, int* i, int* j, int64_t* step);
int hf_batch_clear_error_cell(hf_batch* b);
int hf_batch_stream(hf_batch* b, void** stream);

#ifdef __cplusplus
}
#endif
#endif
