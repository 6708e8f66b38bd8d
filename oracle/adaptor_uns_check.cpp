// Test infrastructure only: the unstructured counterpart of adaptor_check.cpp.  Builds the
// reference's own uns objects from a case file (its parser and O(E^2) mesh loader), and steps
// them beside the GPU adaptor (hyperflow_gb300/adaptor/gpu_uns_scheme.h) with the body of
// Simulation::solve (simulation.cpp:85-105), comparing the cell values bit for bit.  Without a
// GPU, the reference objects are built and creating the context reports the missing device;
// the check exits 3.
#include <cstdio>
#include <fstream>
#include <functional>
#include <memory>
#include <sstream>
#include <string>

#include <nlohmann/json.hpp>

#include "gpu_uns_scheme.h"
#include "simulation/parser/parser.h"

using json = nlohmann::json;
using namespace HyperFlow;

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: adaptor_uns_check case.json steps\n");
        return 2;
    }
    std::ifstream in(argv[1]);
    std::stringstream ss;
    ss << in.rdbuf();
    const std::string text = ss.str();
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
