// Test infrastructure only: the unstructured counterpart of adaptor_check.cpp.  Builds the
// reference's own uns objects from a case file (its parser and O(E^2) mesh loader), and steps
// them beside the GPU adaptor (hyperflow_gb300/adaptor/gpu_uns_scheme.h) with the body of
// Simulation::solve (simulation.cpp:85-105), comparing the cell values bit for bit.  Without a
// GPU, the reference objects are built and creating the context reports the missing device;
// the check exits 3.
//
// With a third argument (a directory), the check runs the reference's own, unmodified
// uns Simulation::solve (simulation.cpp:51-120) to the case's t_end twice -- with the
// reference's Godunov scheme and ODE solver, and with GpuUnsScheme / GpuUnsForwardEuler in their
// place (dt from Simulation::solve's own local TimeStep) -- each writing its CSV frames into its
// own subdirectory, and compares the frames byte for byte.
#include <unistd.h>
#include <sys/stat.h>

#include <cstdio>
#include <fstream>
#include <functional>
#include <memory>
#include <sstream>
#include <string>

#include <nlohmann/json.hpp>

#include "gpu_uns_scheme.h"
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

int solve_mode(const std::string& text, const std::string& dir) {
    json config = json::parse(text);
    const std::string dref = dir + "/reference", dgpu = dir + "/gpu";
    mkdir(dref.c_str(), 0755);
    mkdir(dgpu.c_str(), 0755);
    std::shared_ptr<GpuUnsContext> gpu;
    int frames = 0, differ = 0;
    for (int side = 0; side < 2; ++side) {
        JSONParser p(config);
        auto model = p.generate_model();
        auto mesh = p.generate_mesh();
        auto ic = p.generate_initial_condition();
        auto riemann = p.generate_riemann_solver();
        auto ts = p.generate_time_step();
        std::shared_ptr<Scheme> scheme;
        std::shared_ptr<ODESolver> ode;
        if (side == 0) {
            scheme = p.generate_spatial_scheme(model, riemann, ts, mesh);
            ode = p.generate_ode_solver();
        } else {
            try {
                gpu = std::make_shared<GpuUnsContext>(text);
            } catch (const std::exception& e) {
                std::printf("reference objects built; no GPU context: %s\n", e.what());
                return 3;
            }
            scheme = std::make_shared<GpuUnsScheme>();
            ode = std::make_shared<GpuUnsForwardEuler>(gpu);
        }
        char cwd[4096];
        const std::string& d = side == 0 ? dref : dgpu;
        if (!getcwd(cwd, sizeof cwd) || chdir(d.c_str()) != 0) return 2;
        auto out = p.generate_data_output();
        Simulation sim(model, out, mesh, ic, ode, scheme, riemann, ts, p.get_cfl(), p.get_t_start(),
                       p.get_t_end(), p.get_anim_duration(), p.get_anim_fps());
        sim.solve();
        if (chdir(cwd) != 0) return 2;
    }
    for (;; ++frames) {
        char name[32];
        std::snprintf(name, sizeof name, "/results_%06d.csv", frames);
        std::ifstream a(dref + name), b(dgpu + name);
        if (!a || !b) {
            if ((bool)a != (bool)b) ++differ;
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
        std::fprintf(stderr, "usage: adaptor_uns_check case.json steps [solve_dir]\n");
        return 2;
    }
    const std::string text = slurp(argv[1]);
    if (argc > 3) return solve_mode(text, argv[3]);
    const int steps = std::atoi(argv[2]);
    json config = json::parse(text);
    JSONParser p(config);
    auto model = p.generate_model();
    auto mesh_ref = p.generate_mesh(), mesh_gpu = p.generate_mesh();
    auto ic = p.generate_initial_condition();
    mesh_ref->initialise_field_values(ic);
    mesh_gpu->initialise_field_values(ic);
    auto riemann = p.generate_riemann_solver();
    std::shared_ptr<TimeStep> unused = p.generate_time_step();
    auto scheme = p.generate_spatial_scheme(model, riemann, unused, mesh_ref);
    auto ode = p.generate_ode_solver();
    TimeStep ts(model, p.get_cfl());
    std::shared_ptr<GpuUnsContext> gpu;
    try {
        gpu = std::make_shared<GpuUnsContext>(text);
    } catch (const std::exception& e) {
        std::printf("reference objects built; no GPU context: %s\n", e.what());
        return 3;
    }
    auto gscheme = std::make_shared<GpuUnsScheme>();
    GpuUnsForwardEuler gode(gpu);
    GpuUnsTimeStep gts(gpu);
    for (int s = 0; s < steps; ++s) {   // Simulation::solve's body (simulation.cpp:85-105)
        const double dt = ts(mesh_ref);
        auto f = std::bind(&Scheme::operator(), scheme);
        mesh_ref->set_cells_flow_values((*ode)(f, mesh_ref->get_cells_flow_values(), dt));
        const double gdt = gts(mesh_gpu);
        auto gf = std::bind(&Scheme::operator(), gscheme);
        mesh_gpu->set_cells_flow_values(gode(gf, mesh_gpu->get_cells_flow_values(), gdt));
        if (gdt != dt) {
            std::printf("step %d: dt %.17g on the GPU, %.17g in the reference\n", s, gdt, dt);
            return 1;
        }
    }
    const Vec2D a = mesh_ref->get_cells_flow_values(), b = mesh_gpu->get_cells_flow_values();
    long long diff = 0;
    for (size_t c = 0; c < a.size(); ++c)
        for (unsigned v = 0; v < 4; ++v)
            if (!(a[c][v] == b[c][v] || (a[c][v] != a[c][v] && b[c][v] != b[c][v]))) ++diff;
    std::printf("%d steps, %zu cells, %lld differing values\n", steps, a.size(), diff);
    return diff == 0 ? 0 : 1;
}
