// Test infrastructure only: builds the reference's own Simulation from a case file with the
// GPU adaptor (hyperflow_gb300/adaptor/gpu_scheme.h) in place of its scheme and ODE solver,
// compiled against the reference's headers and sources where they lie (oracle/Makefile
// target `adaptor`).  With a GPU it runs Simulation::solve-style steps on both the reference
// CPU objects and the adaptor and compares the fields bit for bit; without one, creating the
// GPU context reports the missing device and the check exits 3, which shows the adaptor
// compiles and links against the reference's real interfaces (the reference objects are built
// first, so that part runs everywhere).
//
// With a third argument (a directory), the check instead runs the reference's own, unmodified
// Simulation::solve (simulation.cpp:51-124) twice to the case's t_end, once with the
// reference's scheme and ODE solver and once with GpuScheme / GpuForwardEuler in their place,
// each writing its CSV frames (results_%06d.csv, euler_data_output.cpp:37-84) into its own
// subdirectory, and compares the two runs' frames byte for byte.
#include <unistd.h>
#include <sys/stat.h>

#include <cstdio>
#include <fstream>
#include <functional>
#include <memory>
#include <sstream>
#include <string>

#include <nlohmann/json.hpp>

#include "gpu_scheme.h"
#include "simulation/parser/parser.h"
#include "simulation/simulation/simulation.h"

using json = nlohmann::json;
using namespace HyperFlow;

namespace {

std::string slurp(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    std::stringstream ss;
    ss << in.rdbuf();
    return ss.str();
}

// Simulation::solve with the given scheme / ODE solver, run inside `dir`
void solve_in(const std::string& dir, JSONParser& p, const std::shared_ptr<Model>& model,
              const std::shared_ptr<Mesh>& mesh, const std::shared_ptr<Scheme>& scheme,
              const std::shared_ptr<ODESolver>& ode, const std::shared_ptr<RiemannSolver>& riemann,
              const std::shared_ptr<TimeStep>& ts) {
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd) || chdir(dir.c_str()) != 0) throw std::runtime_error("cannot enter " + dir);
    auto out = p.generate_data_output();
    auto ic = p.generate_initial_condition();
    Simulation sim(model, out, mesh, ic, ode, scheme, riemann, ts, p.get_cfl(), p.get_t_start(), p.get_t_end(),
                   p.get_anim_duration(), p.get_anim_fps());
    sim.solve();
    if (chdir(cwd) != 0) throw std::runtime_error("cannot return to " + std::string(cwd));
}

int solve_mode(const std::string& text, const std::string& dir) {
    json config = json::parse(text);
    const std::string dref = dir + "/reference", dgpu = dir + "/gpu";
    mkdir(dref.c_str(), 0755);
    mkdir(dgpu.c_str(), 0755);
    JSONParser p_ref(config), p_gpu(config);
    auto model = p_ref.generate_model();
    auto model_g = p_gpu.generate_model();
    auto mesh_ref = p_ref.generate_mesh(), mesh_gpu = p_gpu.generate_mesh();
    auto riemann = p_ref.generate_riemann_solver();
    auto ts = p_ref.generate_time_step();
    auto scheme = p_ref.generate_spatial_scheme(model, riemann, ts, mesh_ref);
    auto ode = p_ref.generate_ode_solver();
    std::shared_ptr<GpuContext> gpu;
    try {
        gpu = std::make_shared<GpuContext>(text);
    } catch (const std::exception& e) {
        std::printf("reference objects built; no GPU context: %s\n", e.what());
        return 3;
    }
    auto gscheme = std::make_shared<GpuScheme>(gpu);
    auto gode = std::make_shared<GpuForwardEuler>(gpu);
    // stdout carries Simulation::solve's per-step lines; the verdict goes to stderr as well
    solve_in(dref, p_ref, model, mesh_ref, scheme, ode, riemann, ts);
    solve_in(dgpu, p_gpu, model_g, mesh_gpu, gscheme, gode, p_gpu.generate_riemann_solver(),
             p_gpu.generate_time_step());
    int frames = 0, differ = 0;
    for (;; ++frames) {
        char name[32];
        std::snprintf(name, sizeof name, "/results_%06d.csv", frames);
        std::ifstream a(dref + name), b(dgpu + name);
        if (!a || !b) {
            if ((bool)a != (bool)b) ++differ;   // one run wrote a frame the other did not
            break;
        }
        if (slurp(dref + name) != slurp(dgpu + name)) ++differ;
    }
    std::printf("Simulation::solve: %d frames, %d differing frames\n", frames, differ);
    std::fprintf(stderr, "Simulation::solve: %d frames, %d differing frames\n", frames, differ);
    return (differ == 0 && frames > 0) ? 0 : 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: adaptor_check case.json steps [solve_dir]\n");
        return 2;
    }
    const std::string text = slurp(argv[1]);
    if (argc > 3) return solve_mode(text, argv[3]);
    const int steps = std::atoi(argv[2]);
    json config = json::parse(text);
    // the reference's objects, twice: one mesh stepped by its own scheme, one through the adaptor
    JSONParser p_ref(config), p_gpu(config);
    auto model = p_ref.generate_model();
    p_gpu.generate_model();   // the parser's Dirichlet states are converted with its own model
    auto mesh_ref = p_ref.generate_mesh(), mesh_gpu = p_gpu.generate_mesh();
    auto ic = p_ref.generate_initial_condition();
    mesh_ref->initialise_field_values(ic);
    mesh_gpu->initialise_field_values(ic);
    auto riemann = p_ref.generate_riemann_solver();
    auto ts = std::make_shared<TimeStep>(model, p_ref.get_cfl());
    auto scheme = p_ref.generate_spatial_scheme(model, riemann, ts, mesh_ref);
    auto ode = p_ref.generate_ode_solver();
    std::shared_ptr<GpuContext> gpu;
    try {
        gpu = std::make_shared<GpuContext>(text);
    } catch (const std::exception& e) {
        std::printf("reference objects built; no GPU context: %s\n", e.what());
        return 3;
    }
    auto gscheme = std::make_shared<GpuScheme>(gpu);
    auto gode = std::make_shared<GpuForwardEuler>(gpu);
    for (int s = 0; s < steps; ++s) {   // Simulation::solve's body (simulation.cpp:85-110)
        for (auto pair : {std::make_pair(mesh_ref, std::static_pointer_cast<Scheme>(scheme)),
                          std::make_pair(mesh_gpu, std::static_pointer_cast<Scheme>(gscheme))}) {
            auto& mesh = pair.first;
            auto& sch = pair.second;
            std::shared_ptr<ODESolver> o = sch == scheme ? ode : std::static_pointer_cast<ODESolver>(gode);
            mesh->apply_bcs();
            const double dt = sch->calculate_time_step(mesh);
            for (auto& blk : mesh->get_mesh_blocks()) {
                auto f = std::bind(&Scheme::operator(), sch, blk);
                blk->set_fields((*o)(f, blk->get_fields(), dt));
            }
        }
    }
    long long diff = 0, cells = 0;
    auto& a = mesh_ref->get_mesh_blocks();
    auto& b = mesh_gpu->get_mesh_blocks();
    for (size_t k = 0; k < a.size(); ++k)
        for (unsigned i = 0; i < a[k]->get_total_x_cells(); ++i)
            for (unsigned j = 0; j < a[k]->get_total_y_cells(); ++j, ++cells)
                for (unsigned v = 0; v < 4; ++v) {
                    const double x = a[k]->get_flow_values(i, j)[v], y = b[k]->get_flow_values(i, j)[v];
                    if (!(x == y || (x != x && y != y))) ++diff;
                }
    std::printf("%d steps, %lld cells, %lld differing values\n", steps, cells, diff);
    return diff == 0 ? 0 : 1;
}
