// Reference-side adaptor for the unstructured solver: the GPU step behind the reference's own
// uns Scheme, ODESolver and TimeStep interfaces (src/fvm_2d_uns/scheme/scheme/scheme.h:20,
// scheme/ode/ode/ode.h:22, scheme/timestep/timestep.h:28), for its Simulation::solve
// (src/fvm_2d_uns/simulation/simulation/simulation.cpp:51-120).
//
// A maintainer copies this header into the reference tree (e.g. src/fvm_2d_uns/scheme/gpu/),
// compiles with -I src/fvm_2d_uns -I <this repo>/include, links libhyperflow_gb300.so, and has
// the parser return GpuUnsScheme / GpuUnsForwardEuler / GpuUnsTimeStep sharing one
// GpuUnsContext.  Simulation::solve builds a local TimeStep (simulation.cpp:61); with that one
// line made the injected time step, per step:
//   * GpuUnsTimeStep uploads the cells' values (Mesh::get_cells_flow_values) and returns
//     TimeStep's dt computed on the device, counter included;
//   * GpuUnsForwardEuler advances every cell on the device and returns the new values, which
//     Simulation::solve stores with set_cells_flow_values.
// Left unmodified, Simulation::solve forms dt with its local (CPU) TimeStep and the ODE adaptor
// uploads the values it is handed before advancing them; the results are the same.
// The GPU context reads the same case file and mesh file (its loader keeps the reference's cell
// and edge order), so cell i is the same cell on both sides.  Results equal the reference's bit
// for bit (per-(cell, edge) flux mode, the default).
#ifndef HYPERFLOW_GB300_GPU_UNS_SCHEME_H
#define HYPERFLOW_GB300_GPU_UNS_SCHEME_H

#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "hyperflow_gb300_uns.h"
#include "mesh/mesh/mesh.h"
#include "scheme/ode/ode/ode.h"
#include "scheme/scheme/scheme.h"
#include "scheme/timestep/timestep.h"

namespace HyperFlow {

class GpuUnsContext {
  public:
    explicit GpuUnsContext(const std::string& case_json) {
        const int s = hf_uns_create(case_json.data(), case_json.size(), &u);
        if (s != HF_OK) {
            const std::string why = std::string(hf_status_string(s)) + ": " + hf_uns_last_error_message(u);
            hf_uns_destroy(u);
            u = nullptr;
            throw std::runtime_error(why);
        }
        int64_t npairs = 0;
        hf_uns_sizes(u, &ncells, &npairs);
        soa.resize((size_t)4 * ncells);
    }
    ~GpuUnsContext() { hf_uns_destroy(u); }
    GpuUnsContext(const GpuUnsContext&) = delete;
    GpuUnsContext& operator=(const GpuUnsContext&) = delete;

    void check(int status) const {
        if (status != HF_OK)
            throw std::runtime_error(std::string(hf_status_string(status)) + ": " + hf_uns_last_error_message(u));
    }

    // the cells' values into the device state
    void upload(const Vec2D& vals) {
        const size_t n = (size_t)ncells;
        for (size_t c = 0; c < n; ++c)
            for (unsigned v = 0; v < 4; ++v) soa[v * n + c] = vals[c][v];
        check(hf_uns_set_state(u, soa.data()));
        uploaded = true;
    }

    hf_uns* u = nullptr;
    int64_t ncells = 0;
    std::vector<double> soa;   // [4][ncells] staging
    bool uploaded = false;     // the device holds the values of this step
};

class GpuUnsTimeStep : public TimeStep {   // replaces the local TimeStep of Simulation::solve
  public:
    explicit GpuUnsTimeStep(std::shared_ptr<GpuUnsContext> g) : gpu(std::move(g)) {}

    double operator()(const std::shared_ptr<Mesh>& mesh) override {
        gpu->upload(mesh->get_cells_flow_values());
        double dt = 0.0;
        gpu->check(hf_uns_time_step(gpu->u, &dt));   // TimeStep::operator(), counter advanced
        return dt;
    }

  private:
    std::shared_ptr<GpuUnsContext> gpu;
};

class GpuUnsScheme : public Scheme {   // replaces GodunovScheme
  public:
    Vec2D operator()() override { return Vec2D(); }   // not formed: the ODE adaptor returns U^{n+1}
};

class GpuUnsForwardEuler : public ODESolver {   // replaces ForwardEulerODESolver
  public:
    explicit GpuUnsForwardEuler(std::shared_ptr<GpuUnsContext> g) : gpu(std::move(g)) {}

    // `values` are the cells' values Simulation::solve passes (get_cells_flow_values): uploaded
    // here unless GpuUnsTimeStep did so this step, so the adaptor also runs under the
    // reference's unmodified Simulation::solve, whose own TimeStep then forms dt on the host
    Vec2D operator()(const std::function<Vec2D()>&, const Vec2D& values, const double dt) override {
        if (!gpu->uploaded) gpu->upload(values);
        gpu->uploaded = false;
        gpu->check(hf_uns_advance(gpu->u, dt));
        gpu->check(hf_uns_get_state(gpu->u, gpu->soa.data()));
        const size_t n = (size_t)gpu->ncells;
        Vec2D out(n, Vec1D(4));
        for (size_t c = 0; c < n; ++c)
            for (unsigned v = 0; v < 4; ++v) out[c][v] = gpu->soa[v * n + c];
        return out;
    }

  private:
    std::shared_ptr<GpuUnsContext> gpu;
};

}  // namespace HyperFlow

#endif
