// C ABI of the Cartesian GPU time step (declared in include/hyperflow_gb300.h).
//
// Host side: parses the reference's case file, builds the initial state exactly as
// the reference does (setup only), owns the device buffers, the TMA descriptors and the
// CUDA stream, and orders the kernels of one step:
//     bc_fill -> ghost_cfl (dt) -> stencil(block 0) ... stencil(block B-1) -> finalize
// which is the reference's apply_bcs -> calculate_time_step -> per-block ODE sequence
// (src/fvm_2d_cart/simulation/simulation/simulation.cpp:85-120).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/hyperflow_gb300.h"
#include "hf_cart.h"
#include "hf_trace.h"
#include "hf_json.hpp"

namespace {

using hf::Json;

typedef hf::EncodeTiledFn PFN_encodeTiled;
PFN_encodeTiled get_encode() { return hf::tensor_map_encoder(); }

struct BlockHost {
    int nx, ny, tx, ty, pitch;
    double xl, xr, yb, yt, dx, dy;
    int bc_type[4];
    int bc_block[4];
    double bc_state[4][4];
};

// prim_to_cons, src/fvm_2d_cart/model/euler_ideal_gas/euler_ideal_gas.cpp:96-109
void prim_to_cons(double gamma, const double* w, double* c) {
    double rho = w[0], u = w[1], v = w[2], p = w[3];
    c[0] = rho;
    c[1] = rho * u;
    c[2] = rho * v;
    c[3] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v);
}

std::vector<double> read_vec4(const Json& a) {
    if (a.kind != Json::Array || a.size() != 4) throw std::runtime_error("state must have 4 entries");
    std::vector<double> v(4);
    for (int k = 0; k < 4; ++k) v[k] = a[k].number();
    return v;
}

}  // namespace

struct hf_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;   // downloads of hf_step_io, created on first use
    cudaEvent_t block_done[HF_MAXB] = {};
    int scheme = 0, limiter = 0, ghost = 1, nblocks = 0;
    double gamma = 1.4, cfl = 0.5, t_start = 0.0, t_end = 0.0;
    std::vector<BlockHost> blocks;
    hf::MeshDev hmesh{};
    hf::MeshDev* dmesh = nullptr;
    hf::Ctrl* dctrl = nullptr;
    CUtensorMap tmap[HF_MAXB][2];
    hf::StepPlan plan{};        // the all-blocks MUSCL-Hancock launch (plan.nb = 0: not usable)
    bool block_launches = false;   // hf_set_block_launches: one stencil launch per block instead
    std::vector<double*> allocs;
    double* pinned = nullptr;   // staging for layout conversion
    size_t pinned_n = 0;
    // frame output: simulation.animation of the case and the device frame ring
    bool has_anim = false;
    double anim_duration = 0.0, anim_fps = 0.0;
    hf::FrameRing ring{};
    int ring_slots = 0;
    long long drained = 0;      // host count of frames popped from the ring
    float* coarse = nullptr;    // device scratch of hf_coarsen
    size_t coarse_n = 0;
    int next_block = 0;         // next block hf_advance_block expects
    // graphs of one step (index = clamp flag)
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int strict = 0;             // hf_set_strict: a zero-flux face stops the loop
    // piecewise steps: has this step been started (accumulators reset) and are the ghost
    // maxima those of the current fields (a TimeStep call since the last fill or upload)?
    bool step_started = false;
    bool ghost_fresh = false;
    // profiling
    bool profile = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[2];
    size_t ev_used[2] = {0, 0};
    std::string err;
};

namespace {

int fail(hf_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            return fail(ctx, HF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

// Shock-bubble states (no counterpart in the reference).  Keys: shock_x, mach,
// bubble_x, bubble_y, bubble_radius, bubble_density, ambient_state (primitive rho,u,v,p).
// The post-shock state follows the Rankine-Hugoniot relations for a shock of Mach number M
// moving into the ambient gas: p2 = p1 (1 + 2g/(g+1) (M^2 - 1)),
// rho2 = rho1 (g+1) M^2 / ((g-1) M^2 + 2), u2 = u1 + M c1 (1 - rho1/rho2), c1 = sqrt(g p1/rho1).
// Outputs: positions (shock_x, bubble_x, bubble_y, radius) and conservative states
// (post-shock, bubble, ambient).
namespace {
void shock_bubble_states(const hf::Json& ic, double g, double& shock_x, double& bx, double& by,
                         double& r, std::vector<double>& post, std::vector<double>& bub,
                         std::vector<double>& amb) {
    shock_x = ic["shock_x"].number();
    const double M = ic["mach"].number();
    bx = ic["bubble_x"].number();
    by = ic["bubble_y"].number();
    r = ic["bubble_radius"].number();
    const double rb = ic["bubble_density"].number();
    std::vector<double> a = read_vec4(ic["ambient_state"]);
    const double rho1 = a[0], u1 = a[1], v1 = a[2], p1 = a[3];
    const double c1 = std::sqrt(g * p1 / rho1);
    const double p2 = p1 * (1.0 + 2.0 * g / (g + 1.0) * (M * M - 1.0));
    const double rho2 = rho1 * ((g + 1.0) * M * M / ((g - 1.0) * M * M + 2.0));
    const double u2 = u1 + M * c1 * (1.0 - rho1 / rho2);
    const double wpost[4] = {rho2, u2, v1, p2}, wbub[4] = {rb, u1, v1, p1}, wamb[4] = {rho1, u1, v1, p1};
    post.assign(4, 0.0);
    bub.assign(4, 0.0);
    amb.assign(4, 0.0);
    prim_to_cons(g, wpost, post.data());
    prim_to_cons(g, wbub, bub.data());
    prim_to_cons(g, wamb, amb.data());
}
}  // namespace

// ---- initial conditions (setup only; same formulas as the reference) --------------
// MeshBlock::calculate_centroids (mesh_block.cpp:239-257) + initialise_field_values
// (215-224); the per-type field functions of quadrp.cpp:49-64, doublerp.cpp:42-55,
// sphericalrp.cpp:62-72, constant.cpp:34-40; the parser's prim->cons conversions
// (parser.cpp:311-428).
void hf::build_initial_state(const Json& ic, double gamma, const BlockGeom& B, int g,
                             std::vector<double>& soa) {
    soa.assign((size_t)4 * B.ty * B.tx, 0.0);
    const std::string type = ic["type"].string();
    const bool prim = ic.has("variables") && ic["variables"].string() == "Primitive";
    auto cons = [&](const Json& a, bool convert) {
        std::vector<double> s = read_vec4(a), c(4);
        if (!convert) return s;
        prim_to_cons(gamma, s.data(), c.data());
        return c;
    };
    std::vector<double> s0, s1, s2, s3;
    double p0 = 0, p1 = 0, p2 = 0, p3 = 0;
    int kind;
    if (type == "Constant") {
        kind = 0;
        s0 = cons(ic["init_state"], true);
    } else if (type == "DoubleRiemannProblem") {
        kind = 1;
        p0 = ic["x_lm_interface"].number();
        p1 = ic["x_mr_interface"].number();
        s0 = cons(ic["init_left_state"], prim);
        s1 = cons(ic["init_middle_state"], prim);
        s2 = cons(ic["init_right_state"], prim);
    } else if (type == "QuadRiemannProblem") {
        kind = 2;
        p0 = ic["x_interface"].number();
        p1 = ic["y_interface"].number();
        s0 = cons(ic["init_ne_state"], prim);
        s1 = cons(ic["init_nw_state"], prim);
        s2 = cons(ic["init_sw_state"], prim);
        s3 = cons(ic["init_se_state"], prim);
    } else if (type == "SphericalRiemannProblem") {
        kind = 3;
        p0 = ic["radius"].number();
        p1 = ic["x_origin"].number();
        p2 = ic["y_origin"].number();
        s0 = cons(ic["init_sphere_state"], true);
        s1 = cons(ic["init_ext_state"], true);
    } else if (type == "ShockBubble") {
        // a planar shock of Mach number `mach` moving in +x into the ambient state, and a
        // circular bubble of another density at the ambient pressure and velocity
        kind = 4;
        shock_bubble_states(ic, gamma, p0, p1, p2, p3, s0, s1, s2);
    } else {
        throw std::invalid_argument("initial condition '" + type + "' not supported");
    }
    const double sx = B.xl - (static_cast<double>(g) - 0.5) * B.dx;
    const double sy = B.yb - (static_cast<double>(g) - 0.5) * B.dy;
    for (int i = g; i < B.tx - g; ++i)
        for (int j = g; j < B.ty - g; ++j) {
            const double x = sx + static_cast<double>(i) * B.dx;
            const double y = sy + static_cast<double>(j) * B.dy;
            const double* s;
            switch (kind) {
                case 0: s = s0.data(); break;
                case 1:
                    if (x <= p0) s = s0.data();
                    else if ((x > p0) && (x <= p1)) s = s1.data();
                    else s = s2.data();
                    break;
                case 2:
                    if ((x <= p0) && (y <= p1)) s = s2.data();          // SW
                    else if ((x <= p0) && (y > p1)) s = s1.data();      // NW
                    else if ((x > p0) && (y <= p1)) s = s3.data();      // SE
                    else s = s0.data();                                  // NE
                    break;
                case 3:
                    s = (((x - p1) * (x - p1) + (y - p2) * (y - p2)) <= (p0 * p0)) ? s0.data()
                                                                                 : s1.data();
                    break;
                default:   // shock-bubble: post-shock left of the shock, then bubble, then ambient
                    if (x <= p0) s = s0.data();
                    else if (((x - p1) * (x - p1) + (y - p2) * (y - p2)) <= (p3 * p3)) s = s1.data();
                    else s = s2.data();
            }
            for (int v = 0; v < 4; ++v) soa[((size_t)v * B.ty + j) * B.tx + i] = s[v];
        }
}

namespace {

int parse_case(hf_ctx* ctx, const Json& cfg) {
    const Json& model = cfg["model"];
    if (model["model"].string() != "EulerIdealGas")
        return fail(ctx, HF_ERR_UNSUPPORTED, "model must be EulerIdealGas");
    ctx->gamma = model["gamma"].number();
    const Json& sch = cfg["scheme"];
    const std::string st = sch["type"].string();
    if (st == "Godunov") {
        ctx->scheme = 0;
        ctx->ghost = 1;
    } else if (st == "MUSCLHancock") {
        ctx->scheme = 1;
        ctx->ghost = 2;
        const std::string lim = sch["limiter"].string();
        if (lim == "MinBee") ctx->limiter = 0;
        else if (lim == "VanLeer") ctx->limiter = 1;
        else return fail(ctx, HF_ERR_UNSUPPORTED, "limiter '" + lim + "' not supported");
    } else {
        return fail(ctx, HF_ERR_UNSUPPORTED, "scheme '" + st + "' not supported");
    }
    if (sch["riemann"].string() != "HLLCEuler")
        return fail(ctx, HF_ERR_UNSUPPORTED, "Riemann solver must be HLLCEuler");
    if (sch["ode"].string() != "ForwardEuler")
        return fail(ctx, HF_ERR_UNSUPPORTED, "ODE solver must be ForwardEuler");
    const Json& sim = cfg["simulation"];
    ctx->cfl = sim["cfl"].number();
    ctx->t_start = sim["t_start"].number();
    ctx->t_end = sim["t_end"].number();
    if (sim.has("animation")) {
        ctx->has_anim = true;
        ctx->anim_duration = sim["animation"]["duration"].number();
        ctx->anim_fps = sim["animation"]["fps"].number();
    }
    const Json& blocks = cfg["mesh"]["blocks"];
    ctx->nblocks = (int)blocks.size();
    if (ctx->nblocks < 1 || ctx->nblocks > HF_MAXB)
        return fail(ctx, HF_ERR_UNSUPPORTED, "between 1 and 16 mesh blocks are supported");
    static const char* sides[4] = {"bottom", "right", "top", "left"};
    for (int b = 0; b < ctx->nblocks; ++b) {
        const Json& jb = blocks[b];
        BlockHost B{};
        const Json& ex = jb["extents"];
        B.xl = ex["x_left"].number();
        B.xr = ex["x_right"].number();
        B.yb = ex["y_bottom"].number();
        B.yt = ex["y_top"].number();
        const double cx = jb["x_cells"].number(), cy = jb["y_cells"].number();
        // cell counts are whole numbers; above 2^24 per side no state fits in device memory
        if (!(cx >= 0.0 && cx <= 16777216.0 && cy >= 0.0 && cy <= 16777216.0) || cx != (double)(long long)cx ||
            cy != (double)(long long)cy)
            return fail(ctx, HF_ERR_UNSUPPORTED, "x_cells and y_cells must be whole numbers up to 2^24");
        B.nx = (int)cx;
        B.ny = (int)cy;
        if (B.nx < 2 * ctx->ghost || B.ny < 2 * ctx->ghost)
            return fail(ctx, HF_ERR_UNSUPPORTED, "a block needs at least 2*ghost cells per axis");
        B.tx = B.nx + 2 * ctx->ghost;
        B.ty = B.ny + 2 * ctx->ghost;
        B.pitch = (B.tx + 31) / 32 * 32;
        B.dx = (B.xr - B.xl) / B.nx;   // mesh_block.cpp:227-236
        B.dy = (B.yt - B.yb) / B.ny;
        for (int s = 0; s < 4; ++s) {
            const Json& bc = jb["boundaries"][sides[s]];
            const std::string kind = bc["type"].string();
            if (kind == "Transmissive") B.bc_type[s] = hf::BC_TRANSMISSIVE;
            else if (kind == "Reflective") B.bc_type[s] = hf::BC_REFLECTIVE;
            else if (kind == "Dirichlet") {
                B.bc_type[s] = hf::BC_DIRICHLET;
                std::vector<double> st4 = read_vec4(bc["flow_state"]);
                if (bc["variables"].string() == "Primitive") {
                    double c4[4];
                    prim_to_cons(ctx->gamma, st4.data(), c4);
                    for (int v = 0; v < 4; ++v) B.bc_state[s][v] = c4[v];
                } else {
                    for (int v = 0; v < 4; ++v) B.bc_state[s][v] = st4[v];
                }
            } else if (kind == "Internal") {
                B.bc_type[s] = hf::BC_INTERNAL;
                const double nb = bc["block"].number();   // a block index: checked below
                B.bc_block[s] = (nb >= 0.0 && nb < (double)HF_MAXB && nb == (double)(int)nb) ? (int)nb : -1;
            } else {
                return fail(ctx, HF_ERR_UNSUPPORTED, "boundary '" + kind + "' not recognised");
            }
        }
        ctx->blocks.push_back(B);
    }
    // an Internal side copies whole rows/columns of its neighbour: the extents along the
    // shared side must agree (the reference indexes the neighbour with the same index)
    for (int b = 0; b < ctx->nblocks; ++b)
        for (int s = 0; s < 4; ++s) {
            const BlockHost& B = ctx->blocks[b];
            if (B.bc_type[s] != hf::BC_INTERNAL) continue;
            int e = B.bc_block[s];
            if (e < 0 || e >= ctx->nblocks)
                return fail(ctx, HF_ERR_ARG, "Internal boundary names a missing block");
            const BlockHost& E = ctx->blocks[e];
            bool along_x = (s == 0 || s == 2);
            if (along_x ? (E.tx != B.tx) : (E.ty != B.ty))
                return fail(ctx, HF_ERR_UNSUPPORTED, "Internal boundary between blocks of unequal extent");
        }
    return HF_OK;
}

// Mesh::apply_bcs (mesh.cpp:31-39) replayed on the host in the reference's order -- blocks in
// case order; per block the bottom, right, top and left sides; per side position by position,
// layer by layer (transmissive_boundary.cpp, reflective_boundary.cpp: the normal momentum negated,
// dirichlet_boundary.cpp, internal_boundary.cpp: the neighbour block's cells) -- tracking, for
// every ghost cell written, where its value comes from: a cell's value before the fill (an
// interior cell, or a ghost cell not yet written in this fill, whose value is the previous
// fill's) or a Dirichlet side's state, with the sign changes of the reflective sides met on the
// way.  The result is one FillOp per ghost cell, in the ghost enumeration of the CFL pass; the
// device applies them all at once.  Every ghost cell is written by some side.
int build_fill_program(hf_ctx* ctx, std::vector<hf::FillOp>& ops) {
    const int g = ctx->ghost;
    const hf::MeshDev& M = ctx->hmesh;
    auto key = [](int b, long long off) { return ((long long)b << 44) | off; };
    std::unordered_map<long long, hf::FillOp> cur;   // ghost cells written so far: their values
    cur.reserve((size_t)M.total_ghost * 2);
    auto is_ghost = [g](const hf::BlockDev& B, int i, int j) {
        return i < g || i >= B.tx - g || j < g || j >= B.ty - g;
    };
    for (int b = 0; b < M.nblocks; ++b) {
        const hf::BlockDev& B = M.b[b];
        for (int side = 0; side < 4; ++side) {
            const int kind = B.bc_type[side];
            const int eb = kind == hf::BC_INTERNAL ? B.bc_block[side] : b;
            if (eb < 0 || eb >= M.nblocks) return fail(ctx, HF_ERR_PARSE, "internal boundary names no block");
            const hf::BlockDev& E = M.b[eb];
            const bool along_x = (side == hf::SIDE_BOTTOM || side == hf::SIDE_TOP);
            const int n = along_x ? B.tx : B.ty;
            const unsigned char neg = along_x ? 2 : 1;   // reflective: rho*v across y sides, rho*u across x
            for (int pos = 0; pos < n; ++pos)
                for (int k = 0; k < g; ++k) {
                    int di, dj, si = 0, sj = 0;
                    switch (side) {
                        case hf::SIDE_BOTTOM:
                            di = pos; dj = g - 1 - k;
                            si = pos; sj = kind == hf::BC_INTERNAL ? E.ty - g - 1 - k : g + k;
                            break;
                        case hf::SIDE_TOP:
                            di = pos; dj = B.ty - g + k;
                            si = pos; sj = kind == hf::BC_INTERNAL ? g + k : B.ty - g - 1 - k;
                            break;
                        case hf::SIDE_LEFT:
                            dj = pos; di = g - 1 - k;
                            sj = pos; si = kind == hf::BC_INTERNAL ? E.tx - g - 1 - k : g + k;
                            break;
                        default:  // right
                            dj = pos; di = B.tx - g + k;
                            sj = pos; si = kind == hf::BC_INTERNAL ? g + k : B.tx - g - 1 - k;
                            break;
                    }
                    hf::FillOp v{};
                    if (kind == hf::BC_DIRICHLET) {
                        v.kind = 2;
                        v.block = b;
                        v.side = (unsigned char)side;
                    } else {
                        if (si < 0 || si >= E.tx || sj < 0 || sj >= E.ty)
                            return fail(ctx, HF_ERR_UNSUPPORTED, "a ghost fill source lies outside its block");
                        const long long so = (long long)sj * E.pitch + si;
                        auto it = cur.find(key(eb, so));
                        if (it != cur.end()) {
                            v = it->second;
                        } else {
                            v.kind = is_ghost(E, si, sj) ? 1 : 0;
                            v.block = eb;
                            v.src = so;
                        }
                        if (kind == hf::BC_REFLECTIVE) v.neg ^= neg;
                    }
                    cur[key(b, (long long)dj * B.pitch + di)] = v;
                }
        }
    }
    ops.resize((size_t)M.total_ghost);
    for (int b = 0; b < M.nblocks; ++b) {
        const hf::BlockDev& B = M.b[b];
        const long long rows = (long long)g * B.tx;
        for (long long k = 0; k < B.ghost_count; ++k) {
            int i, j;   // the ghost enumeration of the CFL pass (hf_cart.cu ghost_cell_ij)
            if (k < rows) {
                j = (int)(k / B.tx); i = (int)(k % B.tx);
            } else if (k < 2 * rows) {
                j = B.ty - g + (int)((k - rows) / B.tx); i = (int)((k - rows) % B.tx);
            } else {
                const long long r = k - 2 * rows;
                j = g + (int)(r / (2 * g));
                const int c = (int)(r % (2 * g));
                i = c < g ? c : B.tx - 2 * g + c;
            }
            auto it = cur.find(key(b, (long long)j * B.pitch + i));
            if (it == cur.end()) return fail(ctx, HF_ERR_UNSUPPORTED, "a ghost cell no side fills");
            ops[(size_t)(B.ghost_off + k)] = it->second;
        }
    }
    return HF_OK;
}

// every block of a MUSCL-Hancock step in one launch, where the mesh has few enough blocks
bool step_kernel(const hf_ctx* ctx) { return ctx->scheme == 1 && ctx->plan.nb > 0 && !ctx->block_launches; }

// The all-blocks launch pays a grid barrier per block and the start-up of every resident CTA; a
// mesh of one block gains nothing from it unless the block fills many waves (measured: a 264^2
// block 341 Mcell-updates/s against 448 with one launch per block, 1010^2 999 against 986, 4096^2
// 1173 against 1163).
constexpr int kStepMinTilesOneBlock = 1024;

void make_plan(hf_ctx* ctx) {
    ctx->plan = hf::StepPlan{};
    if (ctx->scheme != 1 || ctx->nblocks > hf::kStepMaxBlocks) return;
    hf::StepPlan plan{};
    for (int b = 0; b < ctx->nblocks; ++b) {
        plan.tm[b][0] = ctx->tmap[b][0];
        plan.tm[b][1] = ctx->tmap[b][1];
        hf::step_plan_tiles(plan, b, ctx->blocks[b].nx, ctx->blocks[b].ny);
    }
    plan.nb = ctx->nblocks;
    if (ctx->nblocks == 1 && plan.tile_start[1] < kStepMinTilesOneBlock) return;
    ctx->plan = plan;
}

int make_tmaps(hf_ctx* ctx) {
    PFN_encodeTiled enc = get_encode();
    if (!enc) return fail(ctx, HF_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    hf::StencilTiles t = hf::stencil_tiles(ctx->scheme);
    for (int b = 0; b < ctx->nblocks; ++b) {
        const BlockHost& B = ctx->blocks[b];
        for (int k = 0; k < 2; ++k) {
            cuuint64_t dims[3] = {(cuuint64_t)B.tx, (cuuint64_t)B.ty, 4};
            cuuint64_t strides[2] = {(cuuint64_t)B.pitch * 8, (cuuint64_t)B.pitch * B.ty * 8};
            cuuint32_t box[3] = {(cuuint32_t)t.box_x, (cuuint32_t)t.box_y, 4};
            cuuint32_t es[3] = {1, 1, 1};
            CUresult r = enc(&ctx->tmap[b][k], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
                             ctx->hmesh.b[b].buf[k], dims, strides, box, es,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS)
                return fail(ctx, HF_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
        }
    }
    return HF_OK;
}

long long read_step(hf_ctx* ctx) {
    long long s = 0;
    cudaStreamSynchronize(ctx->stream);
    cudaMemcpy(&s, &ctx->dctrl->step, sizeof s, cudaMemcpyDeviceToHost);
    return s;
}

double* staging(hf_ctx* ctx, size_t n) {
    if (ctx->pinned_n < n) {
        if (ctx->pinned) cudaFreeHost(ctx->pinned);
        ctx->pinned = nullptr;
        ctx->pinned_n = 0;
        if (cudaMallocHost(&ctx->pinned, n * sizeof(double)) != cudaSuccess) return nullptr;
        ctx->pinned_n = n;
    }
    return ctx->pinned;
}

void ev_record(hf_ctx* ctx, int kind, bool start) {
    auto& v = ctx->ev[kind];
    size_t& used = ctx->ev_used[kind];
    if (start) {
        if (used == v.size()) {
            cudaEvent_t a, b;
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            v.push_back({a, b});
        }
        cudaEventRecord(v[used].first, ctx->stream);
    } else {
        cudaEventRecord(v[used].second, ctx->stream);
        ++used;
    }
}

// one step's kernels after the ghost fill: dt, then every block, then finalize
int enqueue_step(hf_ctx* ctx, bool profiled) {
    if (profiled) ev_record(ctx, 1, true);
    {
        hf::TraceRange trace_("ghost fill + dt");
        CK(hf::launch_step_begin(ctx->dctrl, ctx->stream));
        CK(hf::launch_fill_cfl(ctx->dctrl, ctx->dmesh, ctx->hmesh.total_ghost, ctx->stream));
    }
    if (profiled) { ev_record(ctx, 1, false); ev_record(ctx, 0, true); }
    {
        hf::TraceRange trace_("block stencils");
        if (step_kernel(ctx)) {
            CK(hf::launch_mh_step(ctx->dctrl, ctx->dmesh, ctx->plan, ctx->limiter, ctx->stream));
        } else {
            for (int b = 0; b < ctx->nblocks; ++b)
                CK(hf::launch_stencil(ctx->dctrl, ctx->dmesh, b, ctx->blocks[b].nx, ctx->blocks[b].ny,
                                      ctx->scheme, ctx->limiter, &ctx->tmap[b][0], &ctx->tmap[b][1],
                                      ctx->stream));
        }
    }
    if (profiled) ev_record(ctx, 0, false);
    if (ctx->ring_slots > 0) CK(hf::launch_frame_copy(ctx->dctrl, ctx->dmesh, ctx->ring, ctx->stream));
    CK(hf::launch_finalize(ctx->dctrl, ctx->stream));
    ctx->step_started = ctx->ghost_fresh = false;
    return HF_OK;
}

int set_clamp(hf_ctx* ctx, int clamp) {
    if (clamp == 0)   // the common case needs no host memory
        CK(cudaMemsetAsync(&ctx->dctrl->clamp, 0, sizeof(int), ctx->stream));
    else
        CK(cudaMemcpyAsync(&ctx->dctrl->clamp, &clamp, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    return HF_OK;
}

}  // namespace

extern "C" {

const char* hf_status_string(int s) {
    switch (s) {
        case HF_OK: return "ok";
        case HF_ERR_ARG: return "bad argument";
        case HF_ERR_PARSE: return "case file parse error";
        case HF_ERR_UNSUPPORTED: return "unsupported case";
        case HF_ERR_CUDA: return "CUDA error";
        case HF_ERR_DEVICE: return "device error word raised";
        case HF_ERR_STATE: return "call out of order";
        case HF_ERR_NO_DEVICE: return "no CUDA device";
        case HF_ERR_TOO_LARGE: return "problem exceeds the fixed-size working area";
        case HF_ERR_NUMERIC: return "strict mode: an HLLC zero-flux fallback occurred";
        default: return "unknown status";
    }
}

const char* hf_last_error_message(const hf_ctx* ctx) { return ctx ? ctx->err.c_str() : ""; }

int hf_create(const char* case_json, size_t len, hf_ctx** out) {
    if (!case_json || !out) return HF_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<hf_ctx> holder(new hf_ctx());
    hf_ctx* ctx = holder.get();
    Json cfg;
    try {
        cfg = Json::parse(case_json, len);
        int r = parse_case(ctx, cfg);
        if (r != HF_OK) { *out = holder.release(); return r; }
    } catch (const std::exception& e) {
        ctx->err = e.what();
        *out = holder.release();
        return HF_ERR_PARSE;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        ctx->err = "no CUDA device visible";
        *out = holder.release();
        return HF_ERR_NO_DEVICE;
    }
    *out = holder.release();
    CK(cudaGetDevice(&ctx->device));
    CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    CK(hf::stencil_prepare());
    // device state
    hf::MeshDev& M = ctx->hmesh;
    M.nblocks = ctx->nblocks;
    M.ghost = ctx->ghost;
    long long goff = 0;
    for (int b = 0; b < ctx->nblocks; ++b) {
        const BlockHost& B = ctx->blocks[b];
        hf::BlockDev& D = M.b[b];
        D.tx = B.tx; D.ty = B.ty; D.nx = B.nx; D.ny = B.ny; D.pitch = B.pitch;
        for (int s = 0; s < 4; ++s) {
            D.bc_type[s] = B.bc_type[s];
            D.bc_block[s] = B.bc_block[s];
            for (int v = 0; v < 4; ++v) D.bc_state[s][v] = B.bc_state[s][v];
        }
        size_t n = (size_t)4 * B.ty * B.pitch;
        for (int k = 0; k < 2; ++k) {
            double* p = nullptr;
            CK(cudaMalloc(&p, n * sizeof(double)));
            ctx->allocs.push_back(p);
            CK(cudaMemsetAsync(p, 0, n * sizeof(double), ctx->stream));
            D.buf[k] = p;
        }
        D.ghost_off = goff;
        D.ghost_count = B.tx * B.ty - B.nx * B.ny;
        goff += D.ghost_count;
    }
    M.total_ghost = goff;
    {
        std::vector<hf::FillOp> ops;
        int r = build_fill_program(ctx, ops);
        if (r != HF_OK) return r;
        hf::FillOp* d = nullptr;
        CK(cudaMalloc(&d, ops.size() * sizeof(hf::FillOp)));
        ctx->allocs.push_back(reinterpret_cast<double*>(d));
        CK(cudaMemcpyAsync(d, ops.data(), ops.size() * sizeof(hf::FillOp), cudaMemcpyHostToDevice, ctx->stream));
        M.fill = d;
    }
    CK(cudaMalloc(&ctx->dmesh, sizeof(hf::MeshDev)));
    CK(cudaMemcpyAsync(ctx->dmesh, &M, sizeof M, cudaMemcpyHostToDevice, ctx->stream));
    hf::Ctrl C{};
    C.nblocks = ctx->nblocks;
    C.scheme = ctx->scheme;
    C.limiter = ctx->limiter;
    C.ghost = ctx->ghost;
    C.gamma = ctx->gamma;
    C.g1 = ctx->gamma - 1.0;
    C.cfl = ctx->cfl;
    for (int b = 0; b < ctx->nblocks; ++b) {
        C.dx[b] = ctx->blocks[b].dx;
        C.dy[b] = ctx->blocks[b].dy;
    }
    C.t = ctx->t_start;
    C.t_end = ctx->t_end;
    C.first_bad = ~0ull;
    C.first_nonpos = ~0ull;
    CK(cudaMalloc(&ctx->dctrl, sizeof(hf::Ctrl)));
    CK(cudaMemcpyAsync(ctx->dctrl, &C, sizeof C, cudaMemcpyHostToDevice, ctx->stream));
    int r = make_tmaps(ctx);
    if (r != HF_OK) return r;
    make_plan(ctx);
    // initial condition, uploaded into both buffers (ghosts zero until the first fill)
    try {
        for (int b = 0; b < ctx->nblocks; ++b) {
            std::vector<double> soa;
            hf::BlockGeom G{ctx->blocks[b].tx, ctx->blocks[b].ty, ctx->blocks[b].xl, ctx->blocks[b].yb,
                            ctx->blocks[b].dx, ctx->blocks[b].dy};
            hf::build_initial_state(cfg["initial_condition"], ctx->gamma, G, ctx->ghost, soa);
            r = hf_set_state(ctx, b, soa.data(), HF_LAYOUT_SOA);
            if (r != HF_OK) return r;
        }
    } catch (const std::exception& e) {
        return fail(ctx, HF_ERR_UNSUPPORTED, e.what());
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return HF_OK;
}

void hf_destroy(hf_ctx* ctx) {
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (int k = 0; k < 2; ++k) {
        if (ctx->graph[k]) cudaGraphExecDestroy(ctx->graph[k]);
        for (auto& pr : ctx->ev[k]) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
    }
    for (double* p : ctx->allocs) cudaFree(p);
    if (ctx->ring.base) cudaFree(ctx->ring.base);
    if (ctx->coarse) cudaFree(ctx->coarse);
    if (ctx->dmesh) cudaFree(ctx->dmesh);
    if (ctx->dctrl) cudaFree(ctx->dctrl);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    for (int b = 0; b < HF_MAXB; ++b)
        if (ctx->block_done[b]) cudaEventDestroy(ctx->block_done[b]);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int hf_num_blocks(const hf_ctx* ctx, int* n) {
    if (!ctx || !n) return HF_ERR_ARG;
    *n = ctx->nblocks;
    return HF_OK;
}

int hf_block_dims(const hf_ctx* ctx, int b, int dims[5]) {
    if (!ctx || !dims || b < 0 || b >= ctx->nblocks) return HF_ERR_ARG;
    const BlockHost& B = ctx->blocks[b];
    dims[0] = B.tx; dims[1] = B.ty; dims[2] = ctx->ghost; dims[3] = B.nx; dims[4] = B.ny;
    return HF_OK;
}

int hf_set_state(hf_ctx* ctx, int b, const double* cons, int layout) {
    hf::TraceRange trace_("hf_set_state");
    if (!ctx || !cons || b < 0 || b >= ctx->nblocks) return HF_ERR_ARG;
    if (layout != HF_LAYOUT_SOA && layout != HF_LAYOUT_AOS_XY) return HF_ERR_ARG;
    if (ctx->next_block != 0) return fail(ctx, HF_ERR_STATE, "state upload in the middle of a step");
    const BlockHost& B = ctx->blocks[b];
    const hf::BlockDev& D = ctx->hmesh.b[b];
    size_t n = (size_t)4 * B.ty * B.tx;
    const double* st = cons;   // SoA uploads go straight from the caller's buffer
    if (layout == HF_LAYOUT_AOS_XY) {
        double* tmp = staging(ctx, n);
        if (!tmp) return fail(ctx, HF_ERR_CUDA, "pinned staging allocation failed");
        for (int i = 0; i < B.tx; ++i)
            for (int j = 0; j < B.ty; ++j)
                for (int v = 0; v < 4; ++v)
                    tmp[((size_t)v * B.ty + j) * B.tx + i] = cons[((size_t)i * B.ty + j) * 4 + v];
        st = tmp;
    }
    long long step = read_step(ctx);
    int p = (int)(step & 1);
    // into the current buffer, then a device copy into the other (the ghost fill relies on
    // both holding the same values)
    CK(cudaMemcpy2DAsync(D.buf[p], (size_t)B.pitch * 8, st, (size_t)B.tx * 8, (size_t)B.tx * 8,
                         (size_t)4 * B.ty, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(D.buf[p ^ 1], D.buf[p], (size_t)4 * B.ty * B.pitch * 8, cudaMemcpyDeviceToDevice,
                       ctx->stream));
    // TimeStep terms of the uploaded interior
    unsigned long long zero[2] = {0ull, 0ull};
    CK(cudaMemcpyAsync(&ctx->dctrl->int_s[p][b][0], zero, sizeof zero, cudaMemcpyHostToDevice, ctx->stream));
    CK(hf::launch_interior_cfl(ctx->dctrl, ctx->dmesh, b, B.nx, B.ny, p, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->ghost_fresh = false;
    return HF_OK;
}

int hf_get_state(hf_ctx* ctx, int b, double* cons, int layout) {
    hf::TraceRange trace_("hf_get_state");
    if (!ctx || !cons || b < 0 || b >= ctx->nblocks) return HF_ERR_ARG;
    if (layout != HF_LAYOUT_SOA && layout != HF_LAYOUT_AOS_XY) return HF_ERR_ARG;
    const BlockHost& B = ctx->blocks[b];
    const hf::BlockDev& D = ctx->hmesh.b[b];
    long long step = read_step(ctx);
    int p = (int)(step & 1);
    // a block already advanced in the step in progress lives in the other buffer
    if (ctx->next_block > b) p ^= 1;
    size_t n = (size_t)4 * B.ty * B.tx;
    double* st = layout == HF_LAYOUT_SOA ? cons : staging(ctx, n);
    if (!st) return fail(ctx, HF_ERR_CUDA, "pinned staging allocation failed");
    CK(cudaMemcpy2DAsync(st, (size_t)B.tx * 8, D.buf[p], (size_t)B.pitch * 8, (size_t)B.tx * 8,
                         (size_t)4 * B.ty, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (layout == HF_LAYOUT_AOS_XY) {
        for (int i = 0; i < B.tx; ++i)
            for (int j = 0; j < B.ty; ++j)
                for (int v = 0; v < 4; ++v)
                    cons[((size_t)i * B.ty + j) * 4 + v] = st[((size_t)v * B.ty + j) * B.tx + i];
    }
    return HF_OK;
}

int hf_apply_bcs(hf_ctx* ctx) {
    hf::TraceRange trace_("hf_apply_bcs");
    if (!ctx) return HF_ERR_ARG;
    if (ctx->next_block != 0) return fail(ctx, HF_ERR_STATE, "apply_bcs in the middle of a step");
    CK(hf::launch_step_begin(ctx->dctrl, ctx->stream));
    CK(hf::launch_fill_cfl(ctx->dctrl, ctx->dmesh, ctx->hmesh.total_ghost, ctx->stream, 0));
    CK(hf::launch_ghost_mirror(ctx->dctrl, ctx->dmesh, ctx->hmesh.total_ghost, ctx->stream));
    ctx->step_started = true;
    ctx->ghost_fresh = false;
    return HF_OK;
}

int hf_time_step(hf_ctx* ctx, double* dt) {
    hf::TraceRange trace_("hf_time_step");
    if (!ctx) return HF_ERR_ARG;
    int r = set_clamp(ctx, 0);
    if (r != HF_OK) return r;
    // a step's accumulators start from zero whether or not the ghost fill ran on the device
    // (a caller that fills the ghosts on the host uploads them and calls this directly)
    CK(hf::launch_step_begin(ctx->dctrl, ctx->stream));
    CK(hf::launch_ghost_cfl(ctx->dctrl, ctx->dmesh, ctx->hmesh.total_ghost, ctx->stream));
    ctx->step_started = true;
    ctx->ghost_fresh = true;
    if (dt) {
        CK(cudaMemcpyAsync(dt, &ctx->dctrl->dt_cfl, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return HF_OK;
}

int hf_advance_block(hf_ctx* ctx, int b, double dt) {
    hf::TraceRange trace_("hf_advance_block");
    if (!ctx || b < 0 || b >= ctx->nblocks) return HF_ERR_ARG;
    if (b != ctx->next_block) return fail(ctx, HF_ERR_STATE, "blocks must be advanced in order");
    if (b == 0) {
        // a caller that gives dt itself may have skipped hf_time_step: start the step, and give
        // the MUSCL-Hancock predictor's TimeStep call the ghost maxima of the current fields
        if (!ctx->step_started) CK(hf::launch_step_begin(ctx->dctrl, ctx->stream));
        if (ctx->scheme == 1 && !ctx->ghost_fresh)
            CK(hf::launch_ghost_cfl(ctx->dctrl, ctx->dmesh, ctx->hmesh.total_ghost, ctx->stream, 0));
        CK(hf::launch_set_dt(ctx->dctrl, dt, ctx->stream));
    }
    CK(hf::launch_stencil(ctx->dctrl, ctx->dmesh, b, ctx->blocks[b].nx, ctx->blocks[b].ny,
                          ctx->scheme, ctx->limiter, &ctx->tmap[b][0], &ctx->tmap[b][1], ctx->stream));
    if (b == ctx->nblocks - 1) {
        CK(hf::launch_finalize(ctx->dctrl, ctx->stream));
        ctx->next_block = 0;
        ctx->step_started = ctx->ghost_fresh = false;
    } else {
        ctx->next_block = b + 1;
    }
    return HF_OK;
}

int hf_advance(hf_ctx* ctx, double dt) {
    if (!ctx) return HF_ERR_ARG;
    for (int b = 0; b < ctx->nblocks; ++b) {
        int r = hf_advance_block(ctx, b, dt);
        if (r != HF_OK) return r;
    }
    return HF_OK;
}

// the (step, block, direction, j, i) fields of a face_key
static std::string key_text(unsigned long long k, bool face) {
    const long long step = (long long)(k >> 42);
    const int b = (int)((k >> 38) & 0xF), dir = (int)((k >> 37) & 1);
    const int j = (int)((k >> 19) & 0x3FFFF), i = (int)(k & 0x7FFFF);
    return "step " + std::to_string(step) + ", block " + std::to_string(b) + ", " +
           (face ? std::string(dir ? "y face" : "x face") : std::string("cell")) + " (i " + std::to_string(i) +
           ", j " + std::to_string(j) + ")";
}

// strict mode, after a synchronisation: HF_ERR_NUMERIC once a zero-flux face or a non-positive
// cell is recorded
static int strict_check(hf_ctx* ctx) {
    if (!ctx->strict) return HF_OK;
    unsigned long long k[2] = {~0ull, ~0ull};
    CK(cudaMemcpy(&k[0], &ctx->dctrl->first_bad, sizeof k[0], cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&k[1], &ctx->dctrl->first_nonpos, sizeof k[1], cudaMemcpyDeviceToHost));
    // the record of the earlier step (a zero flux first within one step)
    if (k[0] != ~0ull && (k[0] >> 42) <= (k[1] >> 42))
        return fail(ctx, HF_ERR_NUMERIC, "HLLC zero flux (all wave-speed branches failed) at " + key_text(k[0], true));
    if (k[1] != ~0ull)
        return fail(ctx, HF_ERR_NUMERIC, "non-positive density or pressure at " + key_text(k[1], false));
    return HF_OK;
}

// true when every pointer is 8-byte aligned host memory that kernels may address as it is
// (pinned by cudaHostAlloc / cudaHostRegister: the device pointer is the host pointer)
static bool host_mapped(const double* const* p, int n) {
    for (int b = 0; b < n; ++b) {
        if (reinterpret_cast<uintptr_t>(p[b]) % 8 != 0) return false;
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, p[b]) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (a.type != cudaMemoryTypeHost || a.devicePointer != static_cast<const void*>(p[b])) return false;
    }
    return true;
}

int hf_host_mapped(const void* p, int* mapped) {
    if (!mapped) return HF_ERR_ARG;
    const double* q = static_cast<const double*>(p);
    *mapped = p && host_mapped(&q, 1) ? 1 : 0;
    return HF_OK;
}

// One step with the state in host memory: every block uploaded (into both buffers, with the
// interior TimeStep terms, as hf_set_state), one step (as hf_step), every block downloaded --
// each block's download on a second stream as soon as its own update is done, so it overlaps
// the updates of the blocks after it.  No synchronisation between the pieces.
int hf_step_io(hf_ctx* ctx, const double* const* in, double* const* out, double* dt) {
    hf::TraceRange trace_("hf_step_io");
    if (!ctx || !in || !out) return HF_ERR_ARG;
    for (int b = 0; b < ctx->nblocks; ++b)
        if (!in[b] || !out[b]) return HF_ERR_ARG;
    if (ctx->next_block != 0) return fail(ctx, HF_ERR_STATE, "step in the middle of a step");
    if (!ctx->copy_stream) {
        CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        for (int b = 0; b < ctx->nblocks; ++b)
            CK(cudaEventCreateWithFlags(&ctx->block_done[b], cudaEventDisableTiming));
    }
    const long long step = read_step(ctx);
    const int p = (int)(step & 1);
    if (host_mapped(in, ctx->nblocks) && host_mapped((const double* const*)out, ctx->nblocks)) {
        // pinned host memory: the kernels read and write it over the link themselves -- one
        // pass uploads each block into both buffers with its TimeStep terms, and every stencil
        // stores its updated cells to the host as it goes, so no download trails the last
        // block's update
        // every block's interior TimeStep maxima (int_s[p][b], contiguous over b) start at 0
        CK(cudaMemsetAsync(&ctx->dctrl->int_s[p][0][0], 0, (size_t)ctx->nblocks * 2 * sizeof(unsigned long long),
                           ctx->stream));
        for (int b = 0; b < ctx->nblocks; ++b) {
            const BlockHost& B = ctx->blocks[b];
            CK(hf::launch_upload(ctx->dctrl, ctx->dmesh, b, B.tx, B.ty, p, in[b], ctx->stream));
        }
        int r = set_clamp(ctx, 0);
        if (r != HF_OK) return r;
        CK(hf::launch_step_begin(ctx->dctrl, ctx->stream));
        CK(hf::launch_fill_cfl(ctx->dctrl, ctx->dmesh, ctx->hmesh.total_ghost, ctx->stream));
        for (int b = 0; b < ctx->nblocks; ++b)
            CK(hf::launch_ghost_store(ctx->dctrl, ctx->dmesh, b, ctx->blocks[b].tx, ctx->blocks[b].ny, ctx->ghost,
                                      p, out[b], ctx->stream));
        if (step_kernel(ctx)) {
            hf::StepPlan plan = ctx->plan;
            for (int b = 0; b < ctx->nblocks; ++b) plan.hout[b] = out[b];
            CK(hf::launch_mh_step(ctx->dctrl, ctx->dmesh, plan, ctx->limiter, ctx->stream));
        } else {
            for (int b = 0; b < ctx->nblocks; ++b) {
                const BlockHost& B = ctx->blocks[b];
                CK(hf::launch_stencil(ctx->dctrl, ctx->dmesh, b, B.nx, B.ny, ctx->scheme, ctx->limiter,
                                      &ctx->tmap[b][0], &ctx->tmap[b][1], ctx->stream, out[b]));
            }
        }
        CK(hf::launch_finalize(ctx->dctrl, ctx->stream));
        ctx->step_started = ctx->ghost_fresh = false;
        if (dt) CK(cudaMemcpyAsync(dt, &ctx->dctrl->dt, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        return strict_check(ctx);
    }
    for (int b = 0; b < ctx->nblocks; ++b) {
        const BlockHost& B = ctx->blocks[b];
        const hf::BlockDev& D = ctx->hmesh.b[b];
        CK(cudaMemcpy2DAsync(D.buf[p], (size_t)B.pitch * 8, in[b], (size_t)B.tx * 8, (size_t)B.tx * 8,
                             (size_t)4 * B.ty, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync(D.buf[p ^ 1], D.buf[p], (size_t)4 * B.ty * B.pitch * 8, cudaMemcpyDeviceToDevice,
                           ctx->stream));
        CK(cudaMemsetAsync(&ctx->dctrl->int_s[p][b][0], 0, 2 * sizeof(unsigned long long), ctx->stream));
        CK(hf::launch_interior_cfl(ctx->dctrl, ctx->dmesh, b, B.nx, B.ny, p, ctx->stream));
    }
    int r = set_clamp(ctx, 0);
    if (r != HF_OK) return r;
    CK(hf::launch_step_begin(ctx->dctrl, ctx->stream));
    CK(hf::launch_fill_cfl(ctx->dctrl, ctx->dmesh, ctx->hmesh.total_ghost, ctx->stream));
    for (int b = 0; b < ctx->nblocks; ++b) {
        const BlockHost& B = ctx->blocks[b];
        CK(hf::launch_stencil(ctx->dctrl, ctx->dmesh, b, B.nx, B.ny, ctx->scheme, ctx->limiter,
                              &ctx->tmap[b][0], &ctx->tmap[b][1], ctx->stream));
        CK(cudaEventRecord(ctx->block_done[b], ctx->stream));
        CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->block_done[b], 0));
        CK(cudaMemcpy2DAsync(out[b], (size_t)B.tx * 8, ctx->hmesh.b[b].buf[p ^ 1], (size_t)B.pitch * 8,
                             (size_t)B.tx * 8, (size_t)4 * B.ty, cudaMemcpyDeviceToHost, ctx->copy_stream));
    }
    CK(hf::launch_finalize(ctx->dctrl, ctx->stream));
    ctx->step_started = ctx->ghost_fresh = false;
    if (dt) CK(cudaMemcpyAsync(dt, &ctx->dctrl->dt, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaStreamSynchronize(ctx->copy_stream));
    return strict_check(ctx);
}

int hf_step(hf_ctx* ctx, double* dt) {
    hf::TraceRange trace_("hf_step");
    if (!ctx) return HF_ERR_ARG;
    if (ctx->next_block != 0) return fail(ctx, HF_ERR_STATE, "step in the middle of a step");
    int r = set_clamp(ctx, 0);
    if (r != HF_OK) return r;
    r = enqueue_step(ctx, ctx->profile);
    if (r != HF_OK) return r;
    if (dt) {
        CK(cudaMemcpyAsync(dt, &ctx->dctrl->dt, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        return strict_check(ctx);
    }
    return HF_OK;
}

int hf_run(hf_ctx* ctx, int64_t n, int clamp_t_end, int use_graph, int64_t* steps_done) {
    hf::TraceRange trace_("hf_run");
    if (!ctx || n < 0) return HF_ERR_ARG;
    if (ctx->next_block != 0) return fail(ctx, HF_ERR_STATE, "run in the middle of a step");
    long long s0 = steps_done ? read_step(ctx) : 0;
    int clamp = clamp_t_end ? 1 : 0;
    int r = set_clamp(ctx, clamp);
    if (r != HF_OK) return r;
    if (use_graph && !ctx->profile) {
        if (!ctx->graph[clamp]) {
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            r = enqueue_step(ctx, false);
            cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
            if (r != HF_OK) return r;
            if (e != cudaSuccess) return fail(ctx, HF_ERR_CUDA, cudaGetErrorString(e));
            CK(cudaGraphInstantiate(&ctx->graph[clamp], g, 0));
            cudaGraphDestroy(g);
        }
        for (int64_t k = 0; k < n; ++k) CK(cudaGraphLaunch(ctx->graph[clamp], ctx->stream));
    } else {
        for (int64_t k = 0; k < n; ++k) {
            r = enqueue_step(ctx, ctx->profile);
            if (r != HF_OK) return r;
        }
    }
    if (steps_done) {
        *steps_done = read_step(ctx) - s0;
        return strict_check(ctx);
    }
    return HF_OK;
}

int hf_get_time(hf_ctx* ctx, double* t, int64_t* calls, double* last_dt) {
    if (!ctx) return HF_ERR_ARG;
    hf::Ctrl C;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&C, ctx->dctrl, sizeof C, cudaMemcpyDeviceToHost));
    if (t) *t = C.t;
    if (calls) *calls = C.calls;
    if (last_dt) *last_dt = C.dt;
    return HF_OK;
}

int hf_hllc_errors(hf_ctx* ctx, int64_t* count) {
    if (!ctx || !count) return HF_ERR_ARG;
    long long v = 0;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&v, &ctx->dctrl->hllc_errors, sizeof v, cudaMemcpyDeviceToHost));
    *count = v;
    return HF_OK;
}

int hf_sync(hf_ctx* ctx) {
    if (!ctx) return HF_ERR_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    int e = 0;
    CK(cudaMemcpy(&e, &ctx->dctrl->err, sizeof e, cudaMemcpyDeviceToHost));
    if (e != 0) return fail(ctx, HF_ERR_DEVICE, "device error word " + std::to_string(e));
    return strict_check(ctx);
}

int hf_set_strict(hf_ctx* ctx, int on) {
    if (!ctx) return HF_ERR_ARG;
    ctx->strict = on ? 1 : 0;
    CK(cudaMemcpyAsync(&ctx->dctrl->strict, &ctx->strict, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return HF_OK;
}

int hf_last_error_cell(hf_ctx* ctx, int* block, int* i, int* j, int* dir, int64_t* step) {
    if (!ctx) return HF_ERR_ARG;
    unsigned long long k = ~0ull;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&k, &ctx->dctrl->first_bad, sizeof k, cudaMemcpyDeviceToHost));
    const bool none = k == ~0ull;
    if (block) *block = none ? -1 : (int)((k >> 38) & 0xF);
    if (dir) *dir = none ? -1 : (int)((k >> 37) & 1);
    if (j) *j = none ? -1 : (int)((k >> 19) & 0x3FFFF);
    if (i) *i = none ? -1 : (int)(k & 0x7FFFF);
    if (step) *step = none ? -1 : (int64_t)(k >> 42);
    return HF_OK;
}

int hf_last_nonpositive_cell(hf_ctx* ctx, int* block, int* i, int* j, int64_t* step) {
    if (!ctx) return HF_ERR_ARG;
    unsigned long long k = ~0ull;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&k, &ctx->dctrl->first_nonpos, sizeof k, cudaMemcpyDeviceToHost));
    const bool none = k == ~0ull;
    if (block) *block = none ? -1 : (int)((k >> 38) & 0xF);
    if (j) *j = none ? -1 : (int)((k >> 19) & 0x3FFFF);
    if (i) *i = none ? -1 : (int)(k & 0x7FFFF);
    if (step) *step = none ? -1 : (int64_t)(k >> 42);
    return HF_OK;
}

int hf_clear_error_cell(hf_ctx* ctx) {
    if (!ctx) return HF_ERR_ARG;
    const unsigned long long none = ~0ull;
    CK(cudaMemcpyAsync(&ctx->dctrl->first_bad, &none, sizeof none, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(&ctx->dctrl->first_nonpos, &none, sizeof none, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return HF_OK;
}

int hf_stream(hf_ctx* ctx, void** stream) {
    if (!ctx || !stream) return HF_ERR_ARG;
    *stream = (void*)ctx->stream;
    return HF_OK;
}

int hf_profile(hf_ctx* ctx, int enable) {
    if (!ctx) return HF_ERR_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->profile = enable != 0;
    ctx->ev_used[0] = ctx->ev_used[1] = 0;
    return HF_OK;
}

// ---- frame output (Simulation::solve's cadence, simulation.cpp:57-122) ----

int hf_frames_enable(hf_ctx* ctx, int ring_slots) {
    if (!ctx || ring_slots < 0 || ring_slots == 1 || ring_slots > HF_MAXRING) return HF_ERR_ARG;
    if (ring_slots > 0 && !ctx->has_anim)
        return fail(ctx, HF_ERR_ARG, "the case has no simulation.animation {duration, fps}");
    if (ctx->next_block != 0) return fail(ctx, HF_ERR_STATE, "frames_enable in the middle of a step");
    CK(cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < 2; ++k)
        if (ctx->graph[k]) { cudaGraphExecDestroy(ctx->graph[k]); ctx->graph[k] = nullptr; }
    if (ctx->ring.base) { CK(cudaFree(ctx->ring.base)); ctx->ring.base = nullptr; }
    ctx->ring_slots = 0;
    long long len = 0;
    for (int b = 0; b < ctx->nblocks; ++b) {
        ctx->ring.off[b] = len;
        len += 4LL * ctx->blocks[b].nx * ctx->blocks[b].ny;
    }
    ctx->ring.slot_len = len;
    if (ring_slots > 0) {
        CK(cudaMalloc(&ctx->ring.base, (size_t)ring_slots * len * sizeof(double)));
        ctx->ring_slots = ring_slots;
    }
    // the interval exactly as simulation.cpp:57 forms it
    const double interval = ring_slots > 0 ? ctx->t_end / (ctx->anim_duration * ctx->anim_fps) : 0.0;
    hf::Ctrl C;
    CK(cudaMemcpy(&C, ctx->dctrl, sizeof C, cudaMemcpyDeviceToHost));
    C.frames = ring_slots > 0 ? 1 : 0;
    C.ring_slots = ring_slots;
    C.frame_interval = interval;
    C.captured = C.drained = 0;
    ctx->drained = 0;
    CK(cudaMemcpy(ctx->dctrl, &C, sizeof C, cudaMemcpyHostToDevice));
    return HF_OK;
}

int hf_frame_len(const hf_ctx* ctx, int64_t* n) {
    if (!ctx || !n) return HF_ERR_ARG;
    long long len = 0;
    for (int b = 0; b < ctx->nblocks; ++b) len += 4LL * ctx->blocks[b].nx * ctx->blocks[b].ny;
    *n = len;
    return HF_OK;
}

int hf_frames_pending(hf_ctx* ctx, int64_t* n) {
    if (!ctx || !n) return HF_ERR_ARG;
    long long cap = 0;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&cap, &ctx->dctrl->captured, sizeof cap, cudaMemcpyDeviceToHost));
    *n = ctx->ring_slots > 0 ? cap - ctx->drained : 0;
    return HF_OK;
}

int hf_frame_pop(hf_ctx* ctx, double* cons, double* t, int64_t* index) {
    if (!ctx) return HF_ERR_ARG;
    if (ctx->ring_slots == 0) return fail(ctx, HF_ERR_STATE, "frames are not enabled");
    hf::Ctrl C;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&C, ctx->dctrl, sizeof C, cudaMemcpyDeviceToHost));
    if (C.captured == ctx->drained) return fail(ctx, HF_ERR_STATE, "no frame pending");
    const long long slot = ctx->drained % ctx->ring_slots;
    if (cons)
        CK(cudaMemcpy(cons, ctx->ring.base + slot * ctx->ring.slot_len,
                      (size_t)ctx->ring.slot_len * sizeof(double), cudaMemcpyDeviceToHost));
    if (t) *t = C.ring_t[slot];
    if (index) *index = C.ring_idx[slot];
    ctx->drained += 1;
    long long d = ctx->drained;
    CK(cudaMemcpy(&ctx->dctrl->drained, &d, sizeof d, cudaMemcpyHostToDevice));
    return HF_OK;
}

// ---- coarse copies of the state (training data of the learned coarse solver) ----

int hf_coarsen(hf_ctx* ctx, int b, int factor, float* out) {
    if (!ctx || !out || b < 0 || b >= ctx->nblocks || factor < 1) return HF_ERR_ARG;
    const BlockHost& B = ctx->blocks[b];
    if (B.nx % factor != 0 || B.ny % factor != 0)
        return fail(ctx, HF_ERR_ARG, "block sides must be multiples of the coarsening factor");
    if (ctx->next_block != 0) return fail(ctx, HF_ERR_STATE, "coarsen in the middle of a step");
    const size_t n = (size_t)4 * (B.nx / factor) * (B.ny / factor);
    if (ctx->coarse_n < n) {
        if (ctx->coarse) CK(cudaFree(ctx->coarse));
        ctx->coarse = nullptr;
        ctx->coarse_n = 0;
        CK(cudaMalloc(&ctx->coarse, n * sizeof(float)));
        ctx->coarse_n = n;
    }
    CK(hf::launch_coarsen(ctx->dctrl, ctx->dmesh, b, factor, (long long)n, ctx->coarse, ctx->stream));
    CK(cudaMemcpyAsync(out, ctx->coarse, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return HF_OK;
}

// ---- checkpoint / restart ----

namespace {
struct CkptHeader {
    char magic[8];
    uint32_t version, ctrl_bytes;
    int32_t nblocks, scheme, limiter, ghost;
    double gamma, cfl, t_end;
    int32_t tx[HF_MAXB], ty[HF_MAXB], pitch[HF_MAXB];
    uint64_t state_bytes;
};
const char kCkptMagic[8] = {'H', 'F', 'C', 'K', 'P', 'T', '0', '1'};

CkptHeader ckpt_header(const hf_ctx* ctx) {
    CkptHeader h;
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, kCkptMagic, 8);
    h.version = 1;
    h.ctrl_bytes = (uint32_t)sizeof(hf::Ctrl);
    h.nblocks = ctx->nblocks;
    h.scheme = ctx->scheme;
    h.limiter = ctx->limiter;
    h.ghost = ctx->ghost;
    h.gamma = ctx->gamma;
    h.cfl = ctx->cfl;
    h.t_end = ctx->t_end;
    uint64_t n = 0;
    for (int b = 0; b < ctx->nblocks; ++b) {
        h.tx[b] = ctx->blocks[b].tx;
        h.ty[b] = ctx->blocks[b].ty;
        h.pitch[b] = ctx->blocks[b].pitch;
        n += 2ull * 4 * ctx->blocks[b].ty * ctx->blocks[b].pitch * sizeof(double);
    }
    h.state_bytes = n;
    return h;
}
}  // namespace

int hf_checkpoint_size(const hf_ctx* ctx, size_t* bytes) {
    if (!ctx || !bytes) return HF_ERR_ARG;
    CkptHeader h = ckpt_header(ctx);
    *bytes = sizeof h + sizeof(hf::Ctrl) + (size_t)h.state_bytes;
    return HF_OK;
}

int hf_checkpoint_save(hf_ctx* ctx, void* buf, size_t bytes) {
    if (!ctx || !buf) return HF_ERR_ARG;
    size_t need = 0;
    hf_checkpoint_size(ctx, &need);
    if (bytes < need) return fail(ctx, HF_ERR_ARG, "checkpoint buffer too small");
    if (ctx->next_block != 0) return fail(ctx, HF_ERR_STATE, "checkpoint in the middle of a step");
    CkptHeader h = ckpt_header(ctx);
    hf::Ctrl C;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&C, ctx->dctrl, sizeof C, cudaMemcpyDeviceToHost));
    if (ctx->ring_slots > 0 && C.captured != ctx->drained)
        return fail(ctx, HF_ERR_STATE, "pop the pending frames before a checkpoint");
    char* p = static_cast<char*>(buf);
    std::memcpy(p, &h, sizeof h);
    p += sizeof h;
    std::memcpy(p, &C, sizeof C);
    p += sizeof C;
    for (int b = 0; b < ctx->nblocks; ++b)
        for (int k = 0; k < 2; ++k) {
            size_t n = (size_t)4 * ctx->blocks[b].ty * ctx->blocks[b].pitch * sizeof(double);
            CK(cudaMemcpy(p, ctx->hmesh.b[b].buf[k], n, cudaMemcpyDeviceToHost));
            p += n;
        }
    return HF_OK;
}

int hf_checkpoint_load(hf_ctx* ctx, const void* buf, size_t bytes) {
    if (!ctx || !buf) return HF_ERR_ARG;
    if (ctx->next_block != 0) return fail(ctx, HF_ERR_STATE, "restore in the middle of a step");
    size_t need = 0;
    hf_checkpoint_size(ctx, &need);
    if (bytes < need) return fail(ctx, HF_ERR_ARG, "checkpoint too short for this case");
    CkptHeader want = ckpt_header(ctx), got;
    std::memcpy(&got, buf, sizeof got);
    if (std::memcmp(got.magic, kCkptMagic, 8) != 0 || got.version != want.version)
        return fail(ctx, HF_ERR_PARSE, "not a checkpoint of this format version");
    if (std::memcmp(&got, &want, sizeof got) != 0)
        return fail(ctx, HF_ERR_ARG, "checkpoint was taken from a different case or build");
    const char* p = static_cast<const char*>(buf) + sizeof got;
    hf::Ctrl C, cur;
    std::memcpy(&C, p, sizeof C);
    p += sizeof C;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&cur, ctx->dctrl, sizeof cur, cudaMemcpyDeviceToHost));
    // the ring belongs to this context: keep its configuration, start it empty
    C.frames = cur.frames;
    C.ring_slots = cur.ring_slots;
    C.frame_interval = cur.frame_interval;
    C.captured = C.drained = 0;
    C.clamp = 0;
    C.done = 0;
    C.err = 0;
    C.strict = cur.strict;
    ctx->drained = 0;
    ctx->step_started = ctx->ghost_fresh = false;
    for (int b = 0; b < ctx->nblocks; ++b)
        for (int k = 0; k < 2; ++k) {
            size_t n = (size_t)4 * ctx->blocks[b].ty * ctx->blocks[b].pitch * sizeof(double);
            CK(cudaMemcpy(ctx->hmesh.b[b].buf[k], p, n, cudaMemcpyHostToDevice));
            p += n;
        }
    CK(cudaMemcpy(ctx->dctrl, &C, sizeof C, cudaMemcpyHostToDevice));
    return HF_OK;
}

int hf_set_block_launches(hf_ctx* ctx, int per_block) {
    if (!ctx) return HF_ERR_ARG;
    if (ctx->next_block != 0) return fail(ctx, HF_ERR_STATE, "launch mode changed in the middle of a step");
    if (ctx->block_launches != (per_block != 0)) {
        CK(cudaStreamSynchronize(ctx->stream));
        for (int k = 0; k < 2; ++k)   // the captured steps hold the other launch mode
            if (ctx->graph[k]) {
                cudaGraphExecDestroy(ctx->graph[k]);
                ctx->graph[k] = nullptr;
            }
    }
    ctx->block_launches = per_block != 0;
    return HF_OK;
}

int hf_blocks_rerun(hf_ctx* ctx, int64_t* count) {
    if (!ctx || !count) return HF_ERR_ARG;
    long long n = 0;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&n, &ctx->dctrl->blocks_rerun, sizeof n, cudaMemcpyDeviceToHost));
    *count = n;
    return HF_OK;
}

int hf_kernel_time(hf_ctx* ctx, int kind, double* ms, int64_t* launches) {
    if (!ctx || kind < 0 || kind > 1) return HF_ERR_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    double tot = 0.0;
    for (size_t i = 0; i < ctx->ev_used[kind]; ++i) {
        float f = 0.f;
        CK(cudaEventElapsedTime(&f, ctx->ev[kind][i].first, ctx->ev[kind][i].second));
        tot += f;
    }
    if (ms) *ms = tot;
    if (launches) *launches = (int64_t)ctx->ev_used[kind];
    return HF_OK;
}

}  // extern "C"

namespace hf {
EncodeTiledFn tensor_map_encoder() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}
}  // namespace hf
