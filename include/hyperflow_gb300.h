/* HyperFlow-GB300 -- C ABI of the GPU time step.
 *
 * This is the drop-in boundary for the reference solver's per-step update
 * (qcrm/HyperFlow).  The reference's step is the triple
 *     Mesh::apply_bcs()                     src/fvm_2d_cart/mesh/mesh/mesh.cpp:31-39
 *     Scheme::calculate_time_step(mesh)     src/fvm_2d_cart/scheme/scheme/scheme.h:23
 *     ODESolver::operator()(Scheme(block))  src/fvm_2d_cart/scheme/ode/ode/ode.h:22-24
 * driven block by block by Simulation::solve (simulation.cpp:85-120).  Each entry point
 * below replaces one of those calls (cited beside it) with device work on FP64 state
 * resident in HBM; results match the reference bit for bit.
 *
 * Conventions: every call returns an HF_* status (never throws).  The caller owns host
 * buffers; the context owns device memory and one CUDA stream.  A context is not
 * thread-safe; distinct contexts are independent.
 */
#ifndef HYPERFLOW_GB300_H
#define HYPERFLOW_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hf_ctx hf_ctx;

enum {
    HF_OK = 0,
    HF_ERR_ARG = 1,          /* bad argument (null pointer, index out of range, bad layout) */
    HF_ERR_PARSE = 2,        /* case file is not valid JSON or misses a key the reference reads */
    HF_ERR_UNSUPPORTED = 3,  /* a model/scheme/boundary the reference does not provide */
    HF_ERR_CUDA = 4,         /* a CUDA runtime call failed (see hf_last_error_message) */
    HF_ERR_DEVICE = 5,       /* a kernel raised its error word (bounded wait timed out, ...) */
    HF_ERR_STATE = 6,        /* call out of order (e.g. advancing block 2 before block 1) */
    HF_ERR_NO_DEVICE = 7,    /* no CUDA device is visible */
    HF_ERR_TOO_LARGE = 8,    /* the problem exceeds a fixed-size working area */
    HF_ERR_NUMERIC = 9       /* strict mode: an HLLC zero-flux fallback (hf_last_error_cell) or a
                                non-positive density or pressure (hf_last_nonpositive_cell) occurred */
};

/* state layouts for hf_set_state / hf_get_state */
enum {
    HF_LAYOUT_SOA = 0,       /* [var][y][x], x fastest, ghosts included (the device layout) */
    HF_LAYOUT_AOS_XY = 1     /* [x][y][var], ghosts included: MeshBlock::fields order,
                                src/fvm_2d_cart/mesh/mesh_block/mesh_block.cpp:35 */
};

/* Parses a case file (the JSON read by src/fvm_2d_cart/simulation/parser/parser.cpp:13-488,
 * same keys and meaning), allocates device state, and initialises the interior from the
 * initial condition exactly as Simulation::Simulation does (simulation.cpp:43).
 * Replaces: JSONParser + generate_* + Simulation construction (src/fvm_2d_cart/main.cpp:33-86).
 * Supported: EulerIdealGas, Godunov or MUSCLHancock (MinBee / VanLeer), HLLCEuler, ForwardEuler,
 * up to 16 blocks, each at least 2 x ghost cells wide along both axes (2 for Godunov, 4 for
 * MUSCL-Hancock; narrower blocks would mirror ghost cells into ghost cells): anything else
 * returns HF_ERR_UNSUPPORTED with the reason in hf_last_error_message. */
int hf_create(const char* case_json, size_t len, hf_ctx** out);
void hf_destroy(hf_ctx* ctx);

/* number of mesh blocks; dims = {total_x, total_y, ghost, x_cells, y_cells} of block b
 * (MeshBlock::get_total_x_cells etc., mesh_block.cpp:70-97) */
int hf_num_blocks(const hf_ctx* ctx, int* nblocks);
int hf_block_dims(const hf_ctx* ctx, int block, int dims[5]);

/* copy a block's conservative state (ghosts included) in / out.
 * Replaces MeshBlock::set_fields / get_fields (mesh_block.cpp:155-164). */
int hf_set_state(hf_ctx* ctx, int block, const double* cons, int layout);
int hf_get_state(hf_ctx* ctx, int block, double* cons, int layout);

/* Mesh::apply_bcs (mesh.cpp:31-39): ghost fill, blocks in order, bottom/right/top/left */
int hf_apply_bcs(hf_ctx* ctx);

/* TimeStep::operator() (src/fvm_2d_cart/scheme/timestep/timestep.cpp:29-68) as called by
 * Scheme::calculate_time_step: CFL dt over all cells incl. ghosts; advances the call counter.
 * It starts the step (its wave-speed accumulators), so it follows either hf_apply_bcs or
 * uploads of fields whose ghosts the caller filled on the host. */
int hf_time_step(hf_ctx* ctx, double* dt);

/* ODESolver(Scheme(block b)) + set_fields for one block (simulation.cpp:106-110, fused
 * forward Euler of forward_euler.cpp:15-33).  Blocks must be advanced in order 0..B-1 within
 * a step; MUSCL-Hancock's predictor TimeStep call (muscl_hancock.cpp:246) happens on the
 * device against the partly advanced mesh, as in the reference -- over all cells, ghosts
 * included, also when the caller gives dt without calling hf_time_step in that step. */
int hf_advance_block(hf_ctx* ctx, int block, double dt);
/* all blocks in order with the same dt, then t += dt */
int hf_advance(hf_ctx* ctx, double dt);

/* one whole step with no clamps: apply_bcs, dt, advance; dt written if non-null */
int hf_step(hf_ctx* ctx, double* dt);

/* One step with the state in host memory, for callers that keep the fields on the host
 * between steps (the reference's own per-step set_fields / get_fields pattern,
 * simulation.cpp:106-110): uploads every block (in[b], SoA [4][total_y][total_x] with ghosts,
 * as hf_set_state), runs one step without the t_end clamp (hf_step), and downloads every block's
 * new state into out[b].  in and out may be the same arrays.  dt (optional) receives the step's
 * dt.  When every array is pinned host memory (hf_host_mapped), the kernels read and write it
 * directly: one pass per block uploads it, and each stencil stores its updated cells to the host
 * as it computes them, so no download trails the last block's update.  Otherwise the arrays are
 * copied, each block's download starting as soon as its update is done. */
int hf_step_io(hf_ctx* ctx, const double* const* in, double* const* out, double* dt);
/* *mapped = 1 when p is 8-byte aligned host memory that the kernels address directly (pinned by
 * cudaHostAlloc / cudaHostRegister), i.e. hf_step_io's direct path applies to it. */
int hf_host_mapped(const void* p, int* mapped);

/* Simulation::solve's loop body (simulation.cpp:81-120, frame clamps excluded) run n times
 * on the device with no host round trip per step: dt stays on the device.  clamp_t_end != 0
 * applies the t_end clamp and stops at t_end like the reference.  use_graph != 0 replays a
 * captured CUDA graph of one step.  steps_done (optional) = steps actually taken. */
int hf_run(hf_ctx* ctx, int64_t n, int clamp_t_end, int use_graph, int64_t* steps_done);

/* simulation time, TimeStep call count, and the dt applied by the last step */
int hf_get_time(hf_ctx* ctx, double* t, int64_t* calls, double* last_dt);

/* number of HLLC zero-flux fallbacks (riemann_hllc.cpp:207-211) seen so far */
int hf_hllc_errors(hf_ctx* ctx, int64_t* count);

/* waits for the context's stream; returns HF_ERR_DEVICE if a kernel raised its error word
 * (and HF_ERR_NUMERIC in strict mode once a zero-flux face or a non-positive cell is recorded) */
int hf_sync(hf_ctx* ctx);

/* Faces whose HLLC takes none of its four branches (riemann_hllc.cpp:199-211: NaN wave speeds,
 * e.g. a negative pressure) get the zero flux and the run continues, as in the reference, which
 * prints a message there; hf_hllc_errors counts them.  hf_last_error_cell gives the earliest such
 * face since the context was created or hf_clear_error_cell: the least (step, block, direction,
 * j, i), where direction 0 is the x face i between interior cells (i-1, j) and (i, j) and 1 the
 * y face j between (i, j-1) and (i, j); step counts the steps completed before it.  All outputs
 * are -1 when there is none; any pointer may be null.
 * hf_last_nonpositive_cell gives, the same way, the earliest (step, block, j, i) interior cell
 * that a step left with a density or pressure (EulerIdealGasModel::cons_to_prim,
 * euler_ideal_gas.cpp:76-92) that is not positive -- zero, negative or NaN.  The reference has no
 * such check and carries the state on; so does this library outside strict mode.
 * hf_set_strict(ctx, 1): once either is recorded the step completes, later steps do
 * nothing, and hf_step / hf_run (with steps_done) / hf_step_io / hf_sync return HF_ERR_NUMERIC
 * with the face or cell in hf_last_error_message.  hf_clear_error_cell clears both records and
 * lets the run go on. */
int hf_set_strict(hf_ctx* ctx, int on);
int hf_last_error_cell(hf_ctx* ctx, int* block, int* i, int* j, int* dir, int64_t* step);
int hf_last_nonpositive_cell(hf_ctx* ctx, int* block, int* i, int* j, int64_t* step);
int hf_clear_error_cell(hf_ctx* ctx);

/* the context's CUDA stream (a cudaStream_t), for callers that time or order work on it */
int hf_stream(hf_ctx* ctx, void** stream);

/* How a step's MUSCL-Hancock block updates are launched.  No counterpart in the reference,
 * whose Simulation::solve updates the blocks in order (simulation.cpp:106-110).  By default a
 * mesh of 2 to 4 blocks (or one block of at least 1024 tiles of 32 x 12 cells) is updated by one
 * cooperative launch that takes the blocks' tiles in
 * order from one counter (no partly filled last wave per block) and runs every block with the
 * predictor dt of a TimeStep call over the step's starting state; each block b > 0 is then
 * checked against the predictor dt the reference forms (muscl_hancock.cpp:246: blocks < b
 * already updated) and run again where the two differ, so results are the reference's bit for
 * bit either way.  per_block = 1 selects one launch per block in order instead (also used for
 * Godunov, for meshes of more blocks and by hf_advance_block).  hf_blocks_rerun counts the
 * block runs redone since creation. */
int hf_set_block_launches(hf_ctx* ctx, int per_block);
int hf_blocks_rerun(hf_ctx* ctx, int64_t* count);

/* per-kernel timing: when enabled, every step's stencil launches are bracketed by CUDA events on
 * the context's stream; hf_kernel_time returns the summed milliseconds and the number of
 * bracketed steps since the last reset.  kind 0 = stencil (Godunov/MUSCL-Hancock), 1 = ghost
 * fill + CFL. */
int hf_profile(hf_ctx* ctx, int enable);
int hf_kernel_time(hf_ctx* ctx, int kind, double* ms, int64_t* launches);

/* Frame output with the cadence of Simulation::solve (src/fvm_2d_cart/simulation/simulation/
 * simulation.cpp:57-122), replacing the per-frame EulerIdealGasDataOutput::to_file call
 * (src/fvm_2d_cart/simulation/output/euler_data_output/euler_data_output.cpp:37-84) with
 * full-precision device snapshots.  With frames enabled, hf_run(clamp_t_end = 1) also applies
 * the reference's frame dt clamp (dt = cur_frame_out - t, simulation.cpp:98-102, interval =
 * t_end / (animation.duration * animation.fps)) and copies, on the device, the interior of
 * every block into a ring of ring_slots frames (2..32): before the first update, and after
 * every update that starts within 1e-12 of a frame time, labelled with the time before that
 * update -- the reference's own points and labels.  The last frame the reference writes after
 * its loop is the state at t_end (hf_get_state).  The loop pauses (hf_run returns fewer
 * steps than asked, t < t_end) while the ring lacks room for two frames; hf_frame_pop frees
 * a slot.  ring_slots = 0 disables frames.  HF_ERR_ARG when the case has no
 * simulation.animation.  The cadence (next frame time, frame count) belongs to the
 * simulation state and is kept by checkpoints; the ring does not. */
int hf_frames_enable(hf_ctx* ctx, int ring_slots);
/* doubles in one frame: sum over blocks of 4 * nx * ny (interior cells, SoA per block,
 * [block][var][y][x], x fastest) */
int hf_frame_len(const hf_ctx* ctx, int64_t* n);
/* frames in the ring not yet popped (synchronises the context's stream) */
int hf_frames_pending(hf_ctx* ctx, int64_t* n);
/* copies the oldest pending frame to cons (hf_frame_len doubles; NULL skips the copy), its
 * time label and frame index (the reference's frame_idx, the n of results_%06d); HF_ERR_STATE
 * when none is pending */
int hf_frame_pop(hf_ctx* ctx, double* cons, double* t, int64_t* index);

/* factor x factor box average of block b's interior cells (FP64 sums) as FP32
 * [4][ny/factor][nx/factor], written to out (host).  No counterpart in the reference: it makes
 * the training data of the learned coarse solver from the solver's own fine runs without
 * copying the fine state off the device.  nx and ny must be multiples of factor. */
int hf_coarsen(hf_ctx* ctx, int block, int factor, float* out);

/* Checkpoint / restart of the whole simulation state: both state buffers of every block
 * (ghosts included) and the control block (t, TimeStep call count, step parity, interior
 * wave-speed maxima, frame cadence).  No counterpart in the reference, whose only output is
 * the 6-digit CSV frame.  A run restored into a context created from the same case continues
 * bit for bit as the run that saved it.  hf_checkpoint_save needs the pending frames popped
 * (HF_ERR_STATE otherwise); hf_checkpoint_load rejects a blob of another case, scheme, block
 * layout or build (HF_ERR_ARG / HF_ERR_PARSE).  Both synchronise the context's stream. */
int hf_checkpoint_size(const hf_ctx* ctx, size_t* bytes);
int hf_checkpoint_save(hf_ctx* ctx, void* buf, size_t bytes);
int hf_checkpoint_load(hf_ctx* ctx, const void* buf, size_t bytes);

/* The CFL time step of one block for callers that cannot allocate device memory (a
 * pool-managed application, a no-allocation time loop).  No counterpart in the reference:
 * it computes what TimeStep::operator() computes, over all total_x * total_y cells of one
 * block given as SoA FP64 [4][total_y][pitch] in device memory, for TimeStep call number
 * call_index (0-based; the first 10 calls use 0.2 * cfl), and writes dt to the device word
 * d_dt on `stream` (a cudaStream_t; 0 = default stream).  It allocates nothing: its only
 * working memory is a 64 KiB static device array, so it handles at most 16,777,216 cells
 * (larger blocks return HF_ERR_TOO_LARGE).  Calls that overlap on the GPU share that array
 * and race.  The first call on each device looks up the array's address (kept once found;
 * a failed lookup returns HF_ERR_CUDA and the next call retries it); make it before any
 * stream capture. */
int hf_time_step_noalloc(const double* d_cons, int total_x, int total_y, int pitch, double dx,
                         double dy, double gamma, double cfl, int64_t call_index, double* d_dt,
                         void* stream);

const char* hf_status_string(int status);
const char* hf_last_error_message(const hf_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif
