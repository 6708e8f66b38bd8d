/* HyperFlow-GB300 -- C ABI of the unstructured (triangle / quadrilateral) GPU time step.
 *
 * Drop-in for the reference's unstructured solver step (qcrm/HyperFlow, src/fvm_2d_uns):
 *     TimeStep::operator()(mesh)            src/fvm_2d_uns/scheme/timestep/timestep.cpp:29-62
 *     ODESolver(GodunovScheme::operator())  src/fvm_2d_uns/scheme/godunov/godunov.cpp:31-77,
 *                                           src/fvm_2d_uns/scheme/ode/forward_euler/forward_euler.cpp
 * as driven by Simulation::solve (src/fvm_2d_uns/simulation/simulation/simulation.cpp:61-120).
 * Status codes are the HF_* codes of hyperflow_gb300.h.  Cell states are SoA [4][ncells]
 * (rho, rho*u, rho*v, E) in the mesh file's cell order.
 */
#ifndef HYPERFLOW_GB300_UNS_H
#define HYPERFLOW_GB300_UNS_H

#include <stddef.h>
#include <stdint.h>

#include "hyperflow_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hf_uns hf_uns;

/* Parses the unstructured case file (keys of src/fvm_2d_uns/simulation/parser/parser.cpp:
 * model, mesh.{type,file,boundaries.inlet}, initial_condition, scheme, simulation) and loads
 * mesh.file.  Replaces JSONParser::generate_mesh + LoadStructuredMesh
 * (src/fvm_2d_uns/mesh/mesh_structured/mesh_structured.cpp:23-122): same text format, cells
 * of 3 or 4 vertices, and the same neighbours -- a pair's neighbour is the cell of the last
 * pair (in cell, edge order) whose edge equals it reversed within 1e-12 per coordinate
 * (Edge::opposite_edges_equal, src/fvm_2d_uns/geometry/edge/edge.cpp:59-71), else the pair's
 * code -- found through a grid hash of the edge start points in O(E) instead of the O(E^2) scan.
 * A mesh whose code count differs from its (cell, edge) pair count, or with a code that is
 * neither -1, -2, -3 nor a cell index, is refused with HF_ERR_PARSE before any device work.
 * mesh.file may instead hold the binary format, recognised by its first 8 bytes "HFMESHB1":
 * int64 cell count, int64 pair count (the vertex counts summed), int32 vertices per cell,
 * int32 boundary code per (cell, edge) pair, zero padding to a multiple of 8 bytes, then
 * float64 (x, y) per vertex, cell by cell, all little-endian -- the text format's content,
 * read without number parsing.
 * On failure *out may still be set (for hf_uns_last_error_message); destroy it. */
int hf_uns_create(const char* case_json, size_t len, hf_uns** out);
/* same, with the mesh (text or binary format) passed in memory instead of read from mesh.file */
int hf_uns_create_mesh(const char* case_json, size_t len, const char* mesh_text, size_t mesh_len,
                       hf_uns** out);
void hf_uns_destroy(hf_uns* u);
const char* hf_uns_last_error_message(const hf_uns* u);

/* cell and (cell, edge)-pair counts (Mesh::get_cells / get_cell_edge_indices, mesh.cpp) */
int hf_uns_sizes(const hf_uns* u, int64_t* ncells, int64_t* npairs);
/* host copies of the loaded mesh: CSR pair starts, neighbour per pair (cell index or the
 * negative BoundaryCondition code of src/fvm_2d_uns/scheme/boundary/boundary.h:12), and
 * the reference's geometry (Edge outward-normal angle in degrees and length, edge.cpp:98-218;
 * Polygon signed area and incircle radius, polygon.cpp:72-186).  Null outputs are skipped. */
int hf_uns_mesh_arrays(const hf_uns* u, int32_t* pair_start, int32_t* nbr, double* angle,
                       double* length, double* area, double* rin);

/* Pairs whose code names a cell (0 for an interior edge) but that match no pair of the mesh.
 * The reference then takes the code itself as the neighbour -- an interior edge reads cell 0 --
 * without a message (mesh_structured.cpp:96-109); this library does the same for parity and
 * counts them here: the count and the first such pair index (-1 when none).  No counterpart in
 * the reference. */
int hf_uns_unmatched_pairs(const hf_uns* u, int64_t* count, int64_t* first_pair);

/* The mesh loader alone, on the host: parses a mesh (text or binary format), validates its
 * codes and runs the neighbour search of hf_uns_create, with no device work and no case file --
 * for tools that inspect meshes and for checking the search on machines without a GPU.  Gives
 * the cell and pair counts, the neighbour of every pair (as hf_uns_mesh_arrays; skipped when
 * nbr is null, HF_ERR_ARG when max_pairs is below the pair count) and the unmatched-pair
 * diagnostics of hf_uns_unmatched_pairs.  Replaces LoadStructuredMesh::load_structured_mesh
 * (mesh_structured.cpp:23-122) up to its cell_edge_indices. */
int hf_uns_mesh_neighbours(const char* mesh, size_t mesh_len, int64_t* ncells, int64_t* npairs,
                           int32_t* nbr, int64_t max_pairs, int64_t* unmatched,
                           int64_t* first_unmatched);

/* cell centroids [2][ncells] as Polygon::calculate_centroid computes them
 * (src/fvm_2d_uns/geometry/polygon/polygon.cpp:188-212); host-side, no device work */
int hf_uns_centroids(const hf_uns* u, double* xy);

/* Mesh::set_cells_flow_values / get_cells_flow_values (src/fvm_2d_uns/mesh/mesh/mesh.cpp:153-168) */
int hf_uns_set_state(hf_uns* u, const double* cons);
int hf_uns_get_state(hf_uns* u, double* cons);

/* TimeStep::operator() (uns timestep.cpp:29-62): advances the call counter */
int hf_uns_time_step(hf_uns* u, double* dt);
/* ODESolver(Scheme()) + set_cells_flow_values with the given dt (simulation.cpp:103-105) */
int hf_uns_advance(hf_uns* u, double dt);
/* n steps of the loop body on the device (dt stays on the device); clamp_t_end stops at t_end */
int hf_uns_run(hf_uns* u, int64_t n, int clamp_t_end, int use_graph, int64_t* steps_done);

/* Flux evaluation mode.  0 (default, the parity path): every (cell, edge) pair evaluates its
 * own HLLC flux in its own rotated frame, exactly as GodunovScheme::operator() does -- results
 * equal the reference bit for bit, and every interior edge is evaluated twice.  1: edge-based --
 * one flux per unique interior edge, evaluated from the lower-indexed cell's side (bit-equal
 * for that cell) and applied negated to the other cell; half the HLLC work, and the other cell's
 * flux differs from the reference's own evaluation by rounding only. */
int hf_uns_set_edge_mode(hf_uns* u, int edge_based);

/* Frame output with the cadence of the unstructured Simulation::solve
 * (src/fvm_2d_uns/simulation/simulation/simulation.cpp:57-120), replacing its per-frame
 * EulerIdealGasDataOutput::to_file (src/fvm_2d_uns/simulation/output/euler_data_output/
 * euler_data_output.cpp:37-82) with full-precision device snapshots -- the same contract as
 * hf_frames_enable / hf_frames_pending / hf_frame_pop of hyperflow_gb300.h: with frames
 * enabled, hf_uns_run(clamp_t_end = 1) applies the frame dt clamp and copies the cell states
 * (SoA [4][ncells]) into a device ring of ring_slots (2..32) frames, pausing while the ring
 * lacks room for two; hf_uns_frame_pop returns the oldest with its time label and index. */
int hf_uns_frames_enable(hf_uns* u, int ring_slots);
int hf_uns_frames_pending(hf_uns* u, int64_t* n);
int hf_uns_frame_pop(hf_uns* u, double* cons, double* t, int64_t* index);

/* Pairs whose HLLC takes the zero flux (NaN wave speeds) are counted by hf_uns_hllc_errors and
 * the run continues, as in the reference.  hf_uns_last_error_cell gives the earliest one since
 * creation or hf_uns_clear_error_cell: the least (step, cell) -- in edge-based mode the edge's
 * owner cell -- or -1.  hf_uns_last_nonpositive_cell gives the least (step, cell) of a cell that
 * a step left with a density or pressure (cons_to_prim) that is not positive -- zero, negative or
 * NaN -- or -1; the reference carries such a state on, and so does this library outside strict
 * mode.  Strict mode (hf_uns_set_strict(u, 1)): once either is recorded the step
 * completes, later device-loop steps do nothing, and hf_uns_run / hf_uns_time_step return
 * HF_ERR_NUMERIC with the cell in hf_uns_last_error_message.  hf_uns_clear_error_cell clears
 * both records. */
/* waits for the context's stream; HF_ERR_DEVICE if a kernel raised the error word (in the
 * bounds-checked build: an index outside the mesh), HF_ERR_NUMERIC as hf_uns_run in strict mode */
int hf_uns_sync(hf_uns* u);
int hf_uns_set_strict(hf_uns* u, int on);
int hf_uns_last_error_cell(hf_uns* u, int64_t* cell, int64_t* step);
int hf_uns_last_nonpositive_cell(hf_uns* u, int64_t* cell, int64_t* step);
int hf_uns_clear_error_cell(hf_uns* u);

/* Checkpoint / restart of the whole unstructured simulation state (both cell-state buffers and
 * the control block: t, TimeStep call count, step parity, the CFL minimum, frame cadence), as
 * hf_checkpoint_* of hyperflow_gb300.h.  No counterpart in the reference.  A run restored into a
 * context created from the same case and mesh continues bit for bit; a blob of another case,
 * mesh or build is refused (HF_ERR_ARG / HF_ERR_PARSE). */
int hf_uns_checkpoint_size(const hf_uns* u, size_t* bytes);
int hf_uns_checkpoint_save(hf_uns* u, void* buf, size_t bytes);
int hf_uns_checkpoint_load(hf_uns* u, const void* buf, size_t bytes);

int hf_uns_get_time(hf_uns* u, double* t, int64_t* calls, double* last_dt);
int hf_uns_hllc_errors(hf_uns* u, int64_t* count);
int hf_uns_stream(hf_uns* u, void** stream);

#ifdef __cplusplus
}
#endif
#endif
