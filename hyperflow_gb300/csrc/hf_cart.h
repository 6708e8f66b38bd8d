// Internal interface between the C-ABI layer (hf_api.cpp) and the Cartesian kernels
// (hf_cart.cu).  Not part of the public ABI.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <vector>

#include "hf_ctrl.h"
#include "hf_json.hpp"

namespace hf {

enum { BC_TRANSMISSIVE = 0, BC_REFLECTIVE = 1, BC_DIRICHLET = 2, BC_INTERNAL = 3 };
enum { SIDE_BOTTOM = 0, SIDE_RIGHT = 1, SIDE_TOP = 2, SIDE_LEFT = 3 };

// One mesh block on the device: SoA FP64 [var][total_y][pitch], x contiguous, rows
// padded to `pitch` doubles (a multiple of 32 = 256 bytes), two buffers that
// alternate each step (the stencil reads one and writes the other).
struct BlockDev {
    int tx, ty, nx, ny, pitch;
    double* buf[2];
    int bc_type[4];
    int bc_block[4];
    double bc_state[4][4];
    long long ghost_off;   // first index of this block in the all-blocks ghost-cell enumeration
    int ghost_count;
};

// One ghost cell's value after the whole ghost fill of Mesh::apply_bcs (all blocks, all sides, in
// the reference's order), found by replaying that fill on the host once: a copy of one cell's
// value from before the fill, or of a side's Dirichlet state, with the reflective sides' sign
// changes.  Cells are listed in the ghost-cell enumeration of the CFL pass (ghost_off order).
struct FillOp {
    long long src;          // kinds 0, 1: offset of the source cell in its block's buffer plane
    int block;              // kinds 0, 1: the source block; kind 2: the block whose side is used
    unsigned char kind;     // 0: an interior cell (current buffer); 1: a ghost cell's value before
                            // the fill (held by the other buffer); 2: a Dirichlet side's state
    unsigned char neg;      // bit 0: negate rho*u, bit 1: negate rho*v
    unsigned char side;     // kind 2: the side
    unsigned char pad;
};

struct MeshDev {
    int nblocks, ghost;
    long long total_ghost;
    BlockDev b[HF_MAXB];
    const FillOp* fill;     // total_ghost entries
};

// the device frame ring: slots of slot_len doubles; block b's interior at off[b] in a slot
struct FrameRing {
    double* base;
    long long slot_len;
    long long off[HF_MAXB];
};

struct StencilTiles {
    int box_x, box_y;   // the stencil's TMA box per variable plane (tile + halo)
};

// launchers (all asynchronous on `s`)
// The ghost fill of every block in one launch from the fill program (m->fill), written into the
// current buffer only, with the ghost cells' TimeStep terms; with form_dt the last CTA forms the
// step's dt (a TimeStep call: counter, clamps, frame points).  Its ghost-cell sources are read
// from the other buffer, whose ghost cells equal the current buffer's before the fill: every
// stencil stores the ghost cells it loaded into its output buffer, and launch_ghost_mirror does
// the same after a fill that no stencil follows.  Launch after launch_step_begin.
cudaError_t launch_fill_cfl(Ctrl* c, const MeshDev* m, long long total_ghost, cudaStream_t s, int form_dt = 1);
// the current buffer's ghost cells into the other buffer
cudaError_t launch_ghost_mirror(Ctrl* c, const MeshDev* m, long long total_ghost, cudaStream_t s);
// start of a step (before its ghost fill, or before a TimeStep call when the caller filled the
// ghosts): stop flags; the ghost and next-state maxima, the reduction ticket and the all-blocks
// launch's counters and records reset
cudaError_t launch_step_begin(Ctrl* c, cudaStream_t s);
// wave-speed maxima over the ghost cells; with form_dt the last CTA forms the step's dt (a
// TimeStep call: counter, clamps, frame points)
cudaError_t launch_ghost_cfl(Ctrl* c, const MeshDev* m, long long total_ghost, cudaStream_t s,
                             int form_dt = 1);
cudaError_t launch_interior_cfl(Ctrl* c, const MeshDev* m, int b, int nx, int ny, int parity,
                                cudaStream_t s);
cudaError_t launch_set_dt(Ctrl* c, double dt, cudaStream_t s);
cudaError_t launch_finalize(Ctrl* c, cudaStream_t s);
// k x k box average of block b's interior (FP64 sums) as FP32 [4][ny/k][nx/k]; n = its length
cudaError_t launch_coarsen(const Ctrl* c, const MeshDev* m, int b, int k, long long n, float* out,
                           cudaStream_t s);
// this step's frames (if any) into the ring; between the stencils and launch_finalize
cudaError_t launch_frame_copy(Ctrl* c, const MeshDev* m, const FrameRing& ring, cudaStream_t s);
// hout (optional): host memory the GPU maps, [4][total_y][total_x]; the stencil also stores its
// updated interior cells there
cudaError_t launch_stencil(Ctrl* c, const MeshDev* m, int b, int nx, int ny, int scheme, int limiter,
                           const CUtensorMap* tm0, const CUtensorMap* tm1, cudaStream_t s,
                           double* hout = nullptr);
// host-buffer steps over mapped host memory: block b's state [4][total_y][total_x] into both
// buffers with the interior TimeStep terms (int_s[parity][b] zeroed before), and, after the
// ghost fill, the updated buffer's ghost cells back out
cudaError_t launch_upload(Ctrl* c, const MeshDev* m, int b, int tx, int ty, int parity, const double* hin,
                          cudaStream_t s);
cudaError_t launch_ghost_store(Ctrl* c, const MeshDev* m, int b, int tx, int ny, int ghost, int parity,
                               double* hout, cudaStream_t s);
// Every block of a MUSCL-Hancock step in one cooperative launch (mh_step_kernel in hf_cart.cu:
// the blocks' tiles from one counter, each block's predictor dt verified against the reference's
// TimeStep call and the block run again where it differs), for meshes of at most
// kStepMaxBlocks blocks.
constexpr int kStepMaxBlocks = 4;
struct StepPlan {
    CUtensorMap tm[kStepMaxBlocks][2];   // per block, per state parity
    double* hout[kStepMaxBlocks];        // host-buffer stores of the updated cells, or null
    int tiles_x[kStepMaxBlocks];
    int tile_start[kStepMaxBlocks + 1];  // prefix sums of the blocks' tile counts
    int nb;
};
// the tile grid of block b (nx x ny interior cells) in the plan
void step_plan_tiles(StepPlan& plan, int b, int nx, int ny);
cudaError_t launch_mh_step(Ctrl* c, const MeshDev* m, const StepPlan& plan, int limiter, cudaStream_t s);

// the driver's cuTensorMapEncodeTiled, or null where the driver lacks it
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn tensor_map_encoder();

// TMA box of the stencil for the scheme
StencilTiles stencil_tiles(int scheme);
cudaError_t stencil_prepare();   // sets the large dynamic shared-memory opt-ins once

// geometry of one block as the initial condition needs it
struct BlockGeom {
    int tx, ty;          // total cells incl. ghosts
    double xl, yb;       // lower-left corner of the interior
    double dx, dy;
};
// The case's initial condition on one block's interior (MeshBlock::calculate_centroids +
// initialise_field_values, mesh_block.cpp:215-257; the IC classes of
// src/fvm_2d_cart/simulation/initcon; the parser's prim->cons conversions).  SoA
// [4][ty][tx] with zero ghosts.  Throws std::invalid_argument for an unknown IC type.
void build_initial_state(const Json& ic, double gamma, const BlockGeom& B, int ghost,
                         std::vector<double>& soa);

}  // namespace hf
