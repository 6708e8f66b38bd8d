// The per-context control block shared by host and device code (plain data only).
#pragma once

#define HF_MAXB 16
#define HF_MAXRING 32

namespace hf {

// the per-context control block, resident in device memory
struct Ctrl {
    // static (set once at context creation)
    int nblocks, scheme, limiter, ghost;
    double gamma, g1, cfl;                 // g1 = gamma - 1.0, as the reference recomputes it
    double dx[HF_MAXB], dy[HF_MAXB];
    // dynamic
    double t, t_end;
    double dt;                              // dt applied by the current step
    double dt_cfl;                          // last step-call CFL dt before clamping
    double dt_pred[HF_MAXB];                // MUSCL-Hancock predictor dt per block, last step
    long long calls;                        // TimeStep calls made so far
    long long step;                         // steps completed; parity selects the state buffer
    int clamp;                              // device loop clamps dt to t_end and stops there
    int done;                               // t == t_end reached (device loop)
    unsigned long long ghost_s[HF_MAXB][2]; // max |u|+c, |v|+c over ghost cells (bit patterns)
    unsigned long long int_s[2][HF_MAXB][2];// [parity][block] same over interior cells
    unsigned int ticket;
    int err;                                // first error code raised on the device
    long long hllc_errors;                  // HLLC "should not get here" zero fluxes
    unsigned long long first_bad;           // least face_key of such a face, ~0 when none
    unsigned long long first_nonpos;        // least face_key (direction 0) of an updated interior cell
                                            // whose density or pressure is not positive, ~0 when none
    int strict;                             // a recorded zero flux or non-positive cell stops the loop
    // frame output with Simulation::solve's cadence (device loop only, i.e. clamp set)
    int frames;                             // frame clamp and capture on
    int ring_slots;                         // depth of the device frame ring
    int snap_pre, snap_post;                // this step takes a frame before / after its update
    double frame_next;                      // the time of the next frame (cur_frame_out)
    double frame_interval;                  // t_end / (duration * fps)
    double snap_t;                          // time label of this step's frames
    long long frame_idx;                    // frames taken so far, the final one excluded
    long long captured, drained;            // frames put into / taken out of the ring
    double ring_t[HF_MAXRING];              // time label per ring slot
    long long ring_idx[HF_MAXRING];         // frame index per ring slot
    // the all-blocks MUSCL-Hancock step launch (mh_step_kernel): its tile counter and grid
    // barrier, and this step's per-block records, folded into the totals above when the step's
    // blocks are final (a block run again discards its first run's records)
    unsigned int tile_ctr;
    unsigned int bar_count, bar_gen;
    long long step_hllc[HF_MAXB];
    unsigned long long step_bad[HF_MAXB], step_nonpos[HF_MAXB];
    long long blocks_rerun;                 // blocks run again because their predictor dt changed
};

enum : int {
    HF_DEV_OK = 0,
    HF_DEV_TIMEOUT = 1,   // a bounded wait gave up
    HF_DEV_BOUNDS = 2,    // a checked index fell outside its buffer
};

// Key of a Cartesian face for the earliest zero-flux record: ordered by step, block, direction
// (0: x face i between interior cells (i-1, j) and (i, j); 1: y face j between (i, j-1) and
// (i, j)), row, column.  Fields saturate at their widths.
#if defined(__CUDACC__)
__host__ __device__
#endif
inline unsigned long long face_key(long long step, int block, int dir, int j, int i) {
    const unsigned long long s = step < 0 ? 0ull : (step > 0x3FFFFFll ? 0x3FFFFFull : (unsigned long long)step);
    const unsigned long long jj = j < 0 ? 0ull : (j > 0x3FFFF ? 0x3FFFFull : (unsigned long long)j);
    const unsigned long long ii = i < 0 ? 0ull : (i > 0x7FFFF ? 0x7FFFFull : (unsigned long long)i);
    return (s << 42) | ((unsigned long long)(block & 0xF) << 38) | ((unsigned long long)(dir & 1) << 37) |
           (jj << 19) | ii;
}

}  // namespace hf
