// Test infrastructure only: a fixed-step driver over the reference's own
// unstructured solver sources (compiled in place by oracle/Makefile).
//
// The reference loads meshes only through LoadStructuredMesh
// (src/fvm_2d_uns/mesh/mesh_structured/mesh_structured.cpp:23-122), which reads
// quadrilaterals and matches neighbours in O(E^2); hfref_uns_create_file runs exactly that
// on a mesh file, for quadrilateral meshes small enough for its scan.  For triangle meshes,
// which that loader cannot read, hfref_uns_create builds
// Mesh(edges, cells, cell_edge_indices) directly (src/fvm_2d_uns/mesh/mesh/mesh.cpp:17-24)
// with the same cell_edge_indices layout as mesh_structured.cpp:93-115:
//   one entry per (cell, own edge) in cell order, [cell, neighbour-or-bc, pair index],
// and the edge vector holding each cell's own Edge object in the same order.
// The caller supplies the neighbour of each pair (a cell index, or the negative
// BoundaryCondition code of src/fvm_2d_uns/scheme/boundary/boundary.h:12).
// Everything else -- Godunov, HLLC, rotation, boundary states, TimeStep, ODE --
// is the reference's own code, driven as Simulation::solve does
// (src/fvm_2d_uns/simulation/simulation/simulation.cpp:61-120) for exactly N steps.
#include <unistd.h>

#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include <nlohmann/json.hpp>

#include "simulation/parser/parser.h"
#include "simulation/simulation/simulation.h"

using json = nlohmann::json;
using namespace HyperFlow;

namespace {

struct RefUns {
    json config;
    std::unique_ptr<JSONParser> parser;
    std::shared_ptr<Model> model;
    std::shared_ptr<Mesh> mesh;
    std::shared_ptr<InitialCondition> initcon;
    std::shared_ptr<RiemannSolver> riemann;
    std::shared_ptr<Scheme> scheme;
    std::shared_ptr<ODESolver> ode;
    std::unique_ptr<TimeStep> time_step;
    double t = 0.0;
    std::vector<double> dts;
};

// the objects JSONParser makes after the mesh, as Simulation's caller does (main.cpp)
void finish_setup(RefUns* r) {
    r->initcon = r->parser->generate_initial_condition();
    r->riemann = r->parser->generate_riemann_solver();
    std::shared_ptr<TimeStep> unused = r->parser->generate_time_step();
    r->scheme = r->parser->generate_spatial_scheme(r->model, r->riemann, unused, r->mesh);
    r->ode = r->parser->generate_ode_solver();
    r->mesh->initialise_field_values(r->initcon);
    r->time_step.reset(new TimeStep(r->model, r->parser->get_cfl()));
}

}  // namespace

extern "C" {

// The reference's own loader end to end: JSONParser::generate_mesh (parser.cpp:141-158) with
// LoadStructuredMesh on the case's mesh.file (mesh_structured.cpp:23-122: quadrilaterals, the
// O(E^2) neighbour search with Edge::opposite_edges_equal), then the solver objects.
void* hfref_uns_create_file(const char* case_json) {
    RefUns* r = new RefUns();
    r->config = json::parse(case_json);
    r->parser.reset(new JSONParser(r->config));
    r->t = r->parser->get_t_start();
    r->model = r->parser->generate_model();
    r->mesh = r->parser->generate_mesh();
    if (!r->mesh) {
        delete r;
        return nullptr;
    }
    finish_setup(r);
    return r;
}

// the mesh's cell_edge_indices (mesh.h:43), [npairs][3] = (cell, neighbour or code, edge index);
// returns the pair count (the rows written only when it is at most cap)
long hfref_uns_cell_edge_indices(void* h, int* out, long cap) {
    auto& cei = static_cast<RefUns*>(h)->mesh->get_cell_edge_indices();
    const long n = (long)cei.size();
    if (out && n <= cap)
        for (long k = 0; k < n; ++k)
            for (int j = 0; j < 3; ++j) out[3 * k + j] = cei[k][j];
    return n;
}

void* hfref_uns_create(const char* case_json, int ncells, const int* nverts,
                       const double* verts, const int* pair_nbr) {
    RefUns* r = new RefUns();
    r->config = json::parse(case_json);
    r->parser.reset(new JSONParser(r->config));
    r->t = r->parser->get_t_start();
    r->model = r->parser->generate_model();

    CellVec1D cells;
    cells.reserve(ncells);
    size_t vo = 0;
    for (int c = 0; c < ncells; ++c) {
        Vec2D vs;
        for (int k = 0; k < nverts[c]; ++k) {
            Vec1D v = {verts[2 * (vo + k)], verts[2 * (vo + k) + 1]};
            vs.push_back(v);
        }
        vo += nverts[c];
        cells.push_back(Cell(vs));
    }
    std::vector<std::vector<int> > cei;
    EdgeVec1D edges;
    int pair = 0;
    for (int c = 0; c < ncells; ++c) {
        unsigned ne = cells[c].get_edges().size();
        for (unsigned e = 0; e < ne; ++e) {
            std::vector<int> idx = {c, pair_nbr[pair], pair};
            cei.push_back(idx);
            edges.push_back(cells[c].get_edges()[e]);
            ++pair;
        }
    }
    r->mesh = std::make_shared<Mesh>(edges, cells, cei);
    finish_setup(r);
    return r;
}

void hfref_uns_destroy(void* h) { delete static_cast<RefUns*>(h); }

int hfref_uns_run(void* h, int n) {
    RefUns* r = static_cast<RefUns*>(h);
    for (int s = 0; s < n; ++s) {
        double dt = (*r->time_step)(r->mesh);
        auto f = std::bind(&Scheme::operator(), r->scheme);
        Vec2D upd = r->ode->operator()(f, r->mesh->get_cells_flow_values(), dt);
        r->mesh->set_cells_flow_values(upd);
        r->dts.push_back(dt);
        r->t += dt;
    }
    return n;
}

// The reference's own Simulation::solve (simulation.cpp:51-120) on this context's mesh,
// inside `outdir` (its CSV frames results_%06d.csv land there).  Simulation re-applies the
// initial condition (simulation.cpp:43) and builds its own TimeStep.  0, or -1 when
// outdir cannot be entered.
int hfref_uns_solve(void* h, const char* outdir) {
    RefUns* r = static_cast<RefUns*>(h);
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd) || chdir(outdir) != 0) return -1;
    auto out = r->parser->generate_data_output();
    std::shared_ptr<TimeStep> ts = r->parser->generate_time_step();
    auto sim = std::make_shared<Simulation>(r->model, out, r->mesh, r->initcon, r->ode, r->scheme,
                                            r->riemann, ts, r->parser->get_cfl(),
                                            r->parser->get_t_start(), r->parser->get_t_end(),
                                            r->parser->get_anim_duration(),
                                            r->parser->get_anim_fps());
    sim->solve();
    r->t = r->parser->get_t_end();
    return chdir(cwd) == 0 ? 0 : -1;
}

// cell centroids as the reference computes them (Polygon::calculate_centroid,
// polygon.cpp:188-212), [2][ncells]
void hfref_uns_centroids(void* h, double* out) {
    auto& cells = static_cast<RefUns*>(h)->mesh->get_cells();
    size_t n = cells.size();
    for (size_t c = 0; c < n; ++c) {
        Vec1D& x = cells[c].get_centroid();
        out[c] = x[0];
        out[n + c] = x[1];
    }
}

void hfref_uns_dts(void* h, double* out) {
    auto& d = static_cast<RefUns*>(h)->dts;
    std::memcpy(out, d.data(), d.size() * sizeof(double));
}

// SoA [var][cell]
void hfref_uns_get_state(void* h, double* out) {
    auto& cells = static_cast<RefUns*>(h)->mesh->get_cells();
    size_t n = cells.size();
    for (size_t c = 0; c < n; ++c)
        for (int k = 0; k < 4; ++k) out[k * n + c] = cells[c].get_flow_values()[k];
}

void hfref_uns_set_state(void* h, const double* in) {
    auto& cells = static_cast<RefUns*>(h)->mesh->get_cells();
    size_t n = cells.size();
    for (size_t c = 0; c < n; ++c) {
        Vec1D v(4);
        for (int k = 0; k < 4; ++k) v[k] = in[k * n + c];
        cells[c].set_flow_values(v);
    }
}

// Geometry exactly as the reference computes it: per pair the outward normal
// angle in degrees (edge.cpp:215-218) and length (edge.cpp:98-101); per cell the
// signed area (polygon.cpp:172-186) and incircle radius (polygon.cpp:72-94).
void hfref_uns_geometry(void* h, double* angle, double* length, double* area, double* rin) {
    RefUns* r = static_cast<RefUns*>(h);
    auto& edges = r->mesh->get_edges();
    for (size_t e = 0; e < edges.size(); ++e) {
        angle[e] = edges[e].get_outward_normal_angle();
        length[e] = edges[e].get_length();
    }
    auto& cells = r->mesh->get_cells();
    for (size_t c = 0; c < cells.size(); ++c) {
        area[c] = cells[c].get_volume();
        rin[c] = cells[c].radius_incircle();
    }
}

}  // extern "C"
