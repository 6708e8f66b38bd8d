// Reference-side adaptor: the GPU time step behind the reference's own Scheme and ODESolver
// interfaces (src/fvm_2d_cart/scheme/scheme/scheme.h:9-25, src/fvm_2d_cart/scheme/ode/ode/ode.h:10-26),
// so that its unmodified Simulation::solve (simulation.cpp:51-124) runs on the GPU.
//
// A maintainer copies this header into the reference tree (e.g. src/fvm_2d_cart/scheme/gpu/),
// compiles with -I src/fvm_2d_cart -I <this repo>/include, links libhyperflow_gb300.so, and has
// JSONParser::generate_spatial_scheme / generate_ode_solver return GpuScheme / GpuForwardEuler
// sharing one GpuContext.  Per step, Simulation::solve then:
//   * applies the boundary conditions on the host fields (Mesh::apply_bcs, unchanged);
//   * calls GpuScheme::calculate_time_step, which uploads every block's fields (ghosts
//     included) and returns TimeStep's dt computed on the device, counter included;
//   * calls GpuForwardEuler once per block, which advances that block on the device (the
//     MUSCL-Hancock predictor's own TimeStep call happens there) and returns U^{n+1}.
// The scheme's L(U) is not formed: U^{n+1} does not round-trip bit for bit through L(U), so the
// ODE adaptor ignores `func` and returns the device's U^{n+1}.  Results equal the reference's
// bit for bit.
#ifndef HYPERFLOW_GB300_GPU_SCHEME_H
#define HYPERFLOW_GB300_GPU_SCHEME_H

#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "hyperflow_gb300.h"
#include "mesh/mesh/mesh.h"
#include "scheme/ode/ode/ode.h"
#include "scheme/scheme/scheme.h"

namespace HyperFlow {

// One GPU context per simulation, created from the same case file the reference parsed.
class GpuContext {
  public:
    explicit GpuContext(const std::string& case_json) {
        const int s = hf_create(case_json.data(), case_json.size(), &ctx);
        if (s != HF_OK) {
            const std::string why = std::string(hf_status_string(s)) + ": " + hf_last_error_message(ctx);
            hf_destroy(ctx);
            ctx = nullptr;
            throw std::runtime_error(why);
        }
        hf_num_blocks(ctx, &nblocks);
    }
    ~GpuContext() { hf_destroy(ctx); }
    GpuContext(const GpuContext&) = delete;
    GpuContext& operator=(const GpuContext&) = delete;

    void check(int status) const {
        if (status != HF_OK)
            throw std::runtime_error(std::string(hf_status_string(status)) + ": " + hf_last_error_message(ctx));
    }

    hf_ctx* ctx = nullptr;
    int nblocks = 0;
    int next_block = 0;   // the block the next ODE call advances (Simulation::solve's order)
};

// MeshBlock fields <-> the C ABI's MeshBlock-order layout [x][y][var], ghosts included
inline std::vector<double> gpu_pack(const MeshBlock& blk) {
    const unsigned tx = blk.get_total_x_cells(), ty = blk.get_total_y_cells();
    std::vector<double> aos((size_t)tx * ty * 4);
    for (unsigned i = 0; i < tx; ++i)
        for (unsigned j = 0; j < ty; ++j) {
            const Vec1D& w = blk.get_flow_values(i, j);
            for (unsigned v = 0; v < 4; ++v) aos[((size_t)i * ty + j) * 4 + v] = w[v];
        }
    return aos;
}

class GpuScheme : public Scheme {   // replaces GodunovScheme / MUSCLHancockScheme
  public:
    explicit GpuScheme(std::shared_ptr<GpuContext> g) : gpu(std::move(g)) {}

    Vec3D operator()(const std::shared_ptr<MeshBlock>&) override { return Vec3D(); }   // not formed

    double calculate_time_step(const std::shared_ptr<Mesh>& mesh) override {
        auto& blocks = mesh->get_mesh_blocks();
        for (unsigned b = 0; b < blocks.size(); ++b) {
            const std::vector<double> aos = gpu_pack(*blocks[b]);
            gpu->check(hf_set_state(gpu->ctx, (int)b, aos.data(), HF_LAYOUT_AOS_XY));
        }
        double dt = 0.0;
        gpu->check(hf_time_step(gpu->ctx, &dt));   // TimeStep::operator(), counter advanced
        gpu->next_block = 0;
        return dt;
    }

  private:
    std::shared_ptr<GpuContext> gpu;
};

class GpuForwardEuler : public ODESolver {   // replaces ForwardEulerODESolver
  public:
    explicit GpuForwardEuler(std::shared_ptr<GpuContext> g) : gpu(std::move(g)) {}

    Vec3D operator()(const std::function<Vec3D()>&, const Vec3D& fields, const double dt) override {
        const int b = gpu->next_block;
        gpu->check(hf_advance_block(gpu->ctx, b, dt));
        const unsigned tx = (unsigned)fields.size(), ty = (unsigned)fields[0].size();
        std::vector<double> aos((size_t)tx * ty * 4);
        gpu->check(hf_get_state(gpu->ctx, b, aos.data(), HF_LAYOUT_AOS_XY));
        Vec3D out(tx, Vec2D(ty, Vec1D(4)));
        for (unsigned i = 0; i < tx; ++i)
            for (unsigned j = 0; j < ty; ++j)
                for (unsigned v = 0; v < 4; ++v) out[i][j][v] = aos[((size_t)i * ty + j) * 4 + v];
        gpu->next_block = (b + 1) % gpu->nblocks;
        return out;
    }

  private:
    std::shared_ptr<GpuContext> gpu;
};

}  // namespace HyperFlow

#endif
