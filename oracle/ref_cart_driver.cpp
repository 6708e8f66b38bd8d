// Test infrastructure only: a fixed-step driver that links the reference's own
// Cartesian solver sources (compiled in place from the reference tree by
// oracle/Makefile) and exposes them through a tiny C ABI for the parity tests and
// the golden-fixture generator.  Nothing in the product links or loads this file.
//
// The driver builds every object exactly as src/fvm_2d_cart/main.cpp:24-71 does
// (JSONParser -> model -> mesh -> initial condition -> Riemann -> TimeStep ->
// scheme -> ODE), initialises the fields as Simulation::Simulation does
// (src/fvm_2d_cart/simulation/simulation/simulation.cpp:43), and then runs the
// body of Simulation::solve (simulation.cpp:85-120) for exactly N steps:
//   apply_bcs -> calculate_time_step -> optional t_end clamp -> per-block
//   ODE(Scheme) + set_fields, in block order -> t += dt.
// hfref_cart_run leaves the frame-output clamps (simulation.cpp:93-102) out;
// hfref_cart_solve runs the reference's own Simulation::solve, frames and all.
#include <unistd.h>

#include <cstring>
#include <functional>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include <nlohmann/json.hpp>

#include "simulation/parser/parser.h"
#include "simulation/simulation/simulation.h"
#include "scheme/riemann/riemann_hllc/riemann_hllc.h"
#include "scheme/limiter/minbee/minbee.h"
#include "scheme/limiter/vanleer/vanleer.h"

using json = nlohmann::json;
using namespace HyperFlow;

namespace {

// Records every TimeStep call (the step dt and the MUSCL-Hancock predictor dt
// of muscl_hancock.cpp:246) so the parity tests can compare the whole dt stream.
class RecordingTimeStep : public TimeStep {
  public:
    RecordingTimeStep(const std::shared_ptr<Model>& m, double cfl) : TimeStep(m, cfl) {}
    double operator()(const std::shared_ptr<Mesh>& mesh) override {
        double dt = TimeStep::operator()(mesh);
        calls.push_back(dt);
        return dt;
    }
    std::vector<double> calls;
};

struct RefCart {
    json config;
    std::unique_ptr<JSONParser> parser;
    std::shared_ptr<Model> model;
    std::shared_ptr<Mesh> mesh;
    std::shared_ptr<InitialCondition> initcon;
    std::shared_ptr<RiemannSolver> riemann;
    std::shared_ptr<RecordingTimeStep> time_step;
    std::shared_ptr<Scheme> scheme;
    std::shared_ptr<ODESolver> ode;
    double t = 0.0;
    double t_end = 0.0;
    std::vector<double> step_dts;
};

}  // namespace

extern "C" {

void* hfref_cart_create(const char* case_json) {
    RefCart* r = new RefCart();
    r->config = json::parse(case_json);
    r->parser.reset(new JSONParser(r->config));
    double cfl = r->parser->get_cfl();
    r->t = r->parser->get_t_start();
    r->t_end = r->parser->get_t_end();
    r->model = r->parser->generate_model();
    r->mesh = r->parser->generate_mesh();
    r->initcon = r->parser->generate_initial_condition();
    r->riemann = r->parser->generate_riemann_solver();
    r->time_step = std::make_shared<RecordingTimeStep>(r->model, cfl);
    r->scheme = r->parser->generate_spatial_scheme(r->model, r->riemann, r->time_step, r->mesh);
    r->ode = r->parser->generate_ode_solver();
    r->mesh->initialise_field_values(r->initcon);
    return r;
}

void hfref_cart_destroy(void* h) { delete static_cast<RefCart*>(h); }

int hfref_cart_num_blocks(void* h) {
    return (int)static_cast<RefCart*>(h)->mesh->get_mesh_blocks().size();
}

// dims[0..2] = total_x, total_y, ghost
void hfref_cart_block_dims(void* h, int b, int* dims) {
    auto blk = static_cast<RefCart*>(h)->mesh->get_mesh_blocks()[b];
    dims[0] = (int)blk->get_total_x_cells();
    dims[1] = (int)blk->get_total_y_cells();
    dims[2] = (int)blk->get_ghost_cells();
}

// Runs n steps.  clamp_t_end != 0 applies simulation.cpp:81-90 (stop at t_end,
// clamp dt); otherwise exactly n steps run.  Returns the number of steps taken.
int hfref_cart_run(void* h, int n, int clamp_t_end) {
    RefCart* r = static_cast<RefCart*>(h);
    auto& blocks = r->mesh->get_mesh_blocks();
    int taken = 0;
    for (int s = 0; s < n; ++s) {
        if (clamp_t_end && r->t == r->t_end) break;
        r->mesh->apply_bcs();
        double dt = r->scheme->calculate_time_step(r->mesh);
        if (clamp_t_end && r->t + dt > r->t_end) dt = r->t_end - r->t;
        for (unsigned b = 0; b < blocks.size(); ++b) {
            auto f = std::bind(&Scheme::operator(), r->scheme, blocks[b]);
            Vec3D nf = r->ode->operator()(f, blocks[b]->get_fields(), dt);
            blocks[b]->set_fields(nf);
        }
        r->step_dts.push_back(dt);
        r->t += dt;
        ++taken;
    }
    return taken;
}

// The reference's own Simulation::solve (simulation.cpp:51-124) on this context's objects,
// as main.cpp:73-88 runs it, inside `outdir` (the CSV frames results_%06d.csv land there).
// Returns 0, or -1 when outdir cannot be entered.
int hfref_cart_solve(void* h, const char* outdir) {
    RefCart* r = static_cast<RefCart*>(h);
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd) || chdir(outdir) != 0) return -1;
    auto out = r->parser->generate_data_output();
    auto sim = std::make_shared<Simulation>(r->model, out, r->mesh, r->initcon, r->ode, r->scheme,
                                            r->riemann, r->time_step, r->parser->get_cfl(),
                                            r->parser->get_t_start(), r->parser->get_t_end(),
                                            r->parser->get_anim_duration(),
                                            r->parser->get_anim_fps());
    sim->solve();
    r->t = r->parser->get_t_end();
    return chdir(cwd) == 0 ? 0 : -1;
}

// Applies only the ghost fill (mesh.cpp:31-39).
void hfref_cart_apply_bcs(void* h) { static_cast<RefCart*>(h)->mesh->apply_bcs(); }

double hfref_cart_time(void* h) { return static_cast<RefCart*>(h)->t; }

int hfref_cart_num_calls(void* h) { return (int)static_cast<RefCart*>(h)->time_step->calls.size(); }
void hfref_cart_calls(void* h, double* out) {
    auto& c = static_cast<RefCart*>(h)->time_step->calls;
    std::memcpy(out, c.data(), c.size() * sizeof(double));
}
int hfref_cart_num_steps(void* h) { return (int)static_cast<RefCart*>(h)->step_dts.size(); }
void hfref_cart_step_dts(void* h, double* out) {
    auto& c = static_cast<RefCart*>(h)->step_dts;
    std::memcpy(out, c.data(), c.size() * sizeof(double));
}

// Block state in SoA order [var][y][x] including ghosts (the device layout).
void hfref_cart_get_state(void* h, int b, double* out) {
    auto blk = static_cast<RefCart*>(h)->mesh->get_mesh_blocks()[b];
    unsigned tx = blk->get_total_x_cells(), ty = blk->get_total_y_cells();
    for (unsigned v = 0; v < 4; ++v)
        for (unsigned j = 0; j < ty; ++j)
            for (unsigned i = 0; i < tx; ++i)
                out[((size_t)v * ty + j) * tx + i] = blk->get_flow_values(i, j)[v];
}

void hfref_cart_set_state(void* h, int b, const double* in) {
    auto blk = static_cast<RefCart*>(h)->mesh->get_mesh_blocks()[b];
    unsigned tx = blk->get_total_x_cells(), ty = blk->get_total_y_cells();
    for (unsigned j = 0; j < ty; ++j)
        for (unsigned i = 0; i < tx; ++i) {
            Vec1D v(4);
            for (unsigned k = 0; k < 4; ++k) v[k] = in[((size_t)k * ty + j) * tx + i];
            blk->set_flow_values(i, j, v);
        }
}

// ---- unit-level entry points: the reference's own functions on given inputs ----

// riemann_hllc.cpp:178-184 -> calc_hllc_flux (322-365)
void hfref_hllc(double gamma, const double* ul, const double* ur, int dir, double* flux) {
    auto model = std::make_shared<EulerIdealGasModel>(gamma);
    HLLCEulerRiemannSolver rs(model);
    Vec1D a(4), b(4);
    for (int k = 0; k < 4; ++k) { a[k] = ul[k]; b[k] = ur[k]; }
    Vec1D f = rs(a, b, dir == 0 ? Direction::x : Direction::y);
    for (int k = 0; k < 4; ++k) flux[k] = f[k];
}

// minbee.cpp:29-38 / vanleer.cpp:29-36 with the parser's parameters (parser.cpp:230-233)
double hfref_limiter(int kind, double r) {
    if (kind == 0) { MinBeeLimiter l(0.0, 1.0, 1.0, 1e-6); return l(r); }
    VanLeerLimiter l(0.0, 1.0, 1.0, 1e-6);
    return l(r);
}

// euler_ideal_gas.cpp:76-92 and 113-149
void hfref_cons_to_prim(double gamma, const double* u, double* w) {
    EulerIdealGasModel m(gamma);
    Vec1D a(4);
    for (int k = 0; k < 4; ++k) a[k] = u[k];
    Vec1D p = m.cons_to_prim(a);
    for (int k = 0; k < 4; ++k) w[k] = p[k];
}

void hfref_cons_flux(double gamma, const double* u, int dir, double* f) {
    EulerIdealGasModel m(gamma);
    Vec1D a(4);
    for (int k = 0; k < 4; ++k) a[k] = u[k];
    Vec1D r = dir == 0 ? m.cons_flux_x(a) : m.cons_flux_y(a);
    for (int k = 0; k < 4; ++k) f[k] = r[k];
}

}  // extern "C"
