// Test infrastructure only: builds the reference's own Simulation from a case file with the
// GPU adaptor (hyperflow_gb300/adaptor/gpu_scheme.h) in place of its scheme and ODE solver,
// compiled against the reference's headers and sources where they lie (oracle/Makefile
// target `adaptor`).  With a GPU it runs Simulation::solve-style steps on both the reference
// CPU objects and the adaptor and compares the fields bit for bit; without one, creating the
// GPU context reports the missing device and the check exits 3, which shows the adaptor
// compiles and links against the reference's real interfaces (the reference objects are built
// first, so that part runs everywhere).
#include <cstdio>
#include <fstream>
#include <functional>
#include <memory>
#include <sstream>
#include <string>

#include <nlohmann/json.hpp>

#include "gpu_scheme.h"
#include "simulation/parser/parser.h"

using json = nlohmann::json;
using namespace HyperFlow;

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: adaptor_check case.json steps\n");
        return 2;
    }
    std::ifstream in(argv[1]);
    std::stringstream ss;
    ss << in.rdbuf();
    const std::string text = ss.str();
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
