// fHSL.h -- DOLFIN-free drop-in for eQ's src/fHSL.h over the eqfield C ABI.
//
// Put this directory ahead of eQ's src/ on the include path and Simulation
// (src/simulation.h:9 includes "fHSL.h") builds against it unchanged: it declares
// class fenicsInterface, the implementation of the plugin eQ::diffusionSolver
// (src/eQ.h:302-330), with the public members Simulation reads and writes
// (src/fHSL.h:333-449; src/simulation.cpp:207-313, 475-505, 536-546, 578, 583-602):
//
//   shell->mesh->num_vertices(), shell->mesh_coords, shell->dof_from_vertex
//   solution_vector (DOF order), totalBoundaryFlux, D11 / D22 / D12,
//   topChannelData / bottomChannelData, setBoundaryValues(), writeDataFiles()
//
// and the few DOLFIN names simulation.cpp calls (dolfin_version, ufc_signature,
// git_commit_hash, SubSystemsManager::singleton().finalize; src/simulation.cpp:57-59,
// 696).  The layer's solve runs on the GPU through include/eqfield.h; the step
// semantics are those of fenicsInterface::stepDiffusion (src/fHSL.cpp:98-161):
// solution_vector (with the controller's deposits) is the step's u0, the new field
// comes back in solution_vector, the flow channels are stepped, and
// totalBoundaryFlux = D dt (-int grad u . n ds).
//
// Wall conditions are decoded from eQ::data::parameters as createHSL does
// (src/fHSL.cpp:367-573, rates of setRobinBoundaryConditions 331-364):
// boundaryType MICROFLUIDIC_TRAP with parameters["boundaries"] (Dirichlet values,
// homogeneous Neumann, Robin at the flow-derived rates, flow channels for a
// Dirichlet value of -1 on the top / bottom walls), DIRICHLET_UPDATE (every wall at
// the compartment value set by setBoundaryValues), DIRICHLET_0 with trapType
// (NOWALLED, THREEWALLED, TWOWALLED, ONEWALLED), NEUMANN_3WALLED_TEST, else all
// walls at zero.  The anisotropic tensor D11 / D22 / D12 (grid order, as
// AnisotropicDiffusionTensor samples it, src/Expressions.h:112-118) is pushed to the
// device whenever the caller changed it.
//
// DOF order: DOLFIN numbers a P1 space's DOFs with its own graph reordering, which
// this library does not reproduce; any permutation serves Simulation, which builds
// its lookup table from mesh_coords and dof_from_vertex (src/simulation.cpp:363-386).
// The default is the identity (DOF = vertex = grid index j + i*nodesW);
// eqfield::dof_shuffle_seed selects a seeded random permutation instead (to check
// a caller's use of the map).  eqfield::precision selects the solve's arithmetic
// (the plain FP64 form by default, as the reference's direct solve).
//
// The data-recording instance (the constructor taking params, create_DataGrid,
// src/simulation.cpp:553-568) records nothing: cell-data grids are output, not part
// of the field step.
#ifndef FENICS_H
#define FENICS_H

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <initializer_list>
#include <iostream>
#include <memory>
#include <random>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "eQ.h"
#include "eqfield.h"

// The DOLFIN names Simulation calls outside the solver (version banner, shutdown).
namespace dolfin {
inline std::string dolfin_version() { return "none (eqfield GPU solver)"; }
inline std::string ufc_signature() { return "none"; }
inline std::string git_commit_hash() { return "none"; }
class SubSystemsManager {
 public:
  static SubSystemsManager& singleton() {
    static SubSystemsManager s;
    return s;
  }
  void finalize() {}
};
}  // namespace dolfin

namespace eqfield {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc, const eqf_batch* h) {
  if (rc != EQF_OK) throw Error(rc, eqf_last_error(h));
}

// Solve arithmetic of new instances: EQF_PREC_FP64 or EQF_PREC_FP32_IR.
inline int precision = EQF_PREC_FP64;
// 0: DOF = grid index; otherwise the seed of a random DOF permutation.
inline unsigned dof_shuffle_seed = 0;

// The mesh as Simulation sees it (a vertex count and the vertex coordinates).
class Mesh {
 public:
  std::size_t num_vertices() const { return coords_.size() / 2; }
  const std::vector<double>& coordinates() const { return coords_; }
  std::vector<double> coords_;
};

// Parameter lookups on eQ::data::parameters (a JSON object).
template <class J>
inline bool has(J& p, const char* key) {
  return p.count(key) > 0;
}
template <class J>
inline std::string str_param(J& p, const char* key, const char* dflt) {
  return has(p, key) ? p[key].template get<std::string>() : std::string(dflt);
}
template <class J>
inline double num_param(J& p, const char* key, double dflt) {
  return has(p, key) ? p[key].template get<double>() : dflt;
}

}  // namespace eqfield

// The part of the reference's fenicsShell Simulation touches (src/fHSL.h:60-127).
class fenicsShell {
 public:
  typedef std::shared_ptr<eQ::gridFunction<size_t>> HSLgrid;
  virtual ~fenicsShell() = default;

  std::shared_ptr<eqfield::Mesh> mesh;
  std::vector<double> mesh_coords;      // (x, y) per vertex, vertex order
  std::vector<size_t> vertex_from_dof;  // dof_to_vertex_map
  std::vector<int> dof_from_vertex;     // vertex_to_dof_map
  HSLgrid dofLookupTable;

  // The layer's own (iy, jx) -> DOF table (createGridCoordinatesToDofMapping,
  // src/fHSL.h:89-114): lattice point of each vertex's coordinates.
  void createGridCoordinatesToDofMapping(size_t nodesH, size_t nodesW, double npm) {
    dofLookupTable = std::make_shared<eQ::gridFunction<size_t>>(nodesH, nodesW);
    for (size_t v = 0; v < mesh_coords.size() / 2; ++v) {
      const auto ij = eQ::data::ij_from_xy(mesh_coords[2 * v], mesh_coords[2 * v + 1], npm);
      (*dofLookupTable)[ij] = size_t(dof_from_vertex[v]);
    }
  }
};

class fenicsInterface : public eQ::diffusionSolver {
 public:
  fenicsInterface() : shell(std::make_shared<fenicsShell>()) {}
  // data-recording instance (create_DataGrid): holds its parameters, records nothing
  explicit fenicsInterface(const eQ::diffusionSolver::params& p)
      : myParams(p), shell(std::make_shared<fenicsShell>()), isDataRecordingNode_(true) {}
  ~fenicsInterface() { release(); }
  fenicsInterface(const fenicsInterface&) = delete;
  fenicsInterface& operator=(const fenicsInterface&) = delete;

  eQ::diffusionSolver::params myParams{};
  std::shared_ptr<fenicsShell> shell;

  bool isFenicsRootNode = true;
  int myRankMPI = 0, numFenicsPEs = 1;
  size_t nodesChannel = 0;
  double wellScaling = 0.0;
  size_t nodesH = 0, nodesW = 0;
  std::vector<std::pair<double, double>> coords;

  std::vector<double> solution_vector;  // DOF order
  std::vector<double> solution_vectorTopChannel, solution_vectorBottomChannel;
  std::vector<double> topChannelData, bottomChannelData;  // grid order along x
  std::vector<double> fluxTopChannel, fluxBottomChannel;
  double totalBoundaryFlux = 0.0;
  std::shared_ptr<std::vector<double>> D11, D22, D12;

  // fenicsInterface::initDiffusion (src/fHSL.cpp:37-53) -> fenicsClassInit (195-328)
  void initDiffusion(eQ::diffusionSolver::params& p) override {
    release();
    myParams = p;
    auto& P = eQ::data::parameters;
    // squares as fenicsClassInit counts them (src/fHSL.cpp:242-243); nodes are one more
    const int32_t nx = (int32_t)std::ceil(p.trapWidthMicrons * p.nodesPerMicron);
    const int32_t ny = (int32_t)std::ceil(p.trapHeightMicrons * p.nodesPerMicron);
    nodesW = (size_t)nx + 1;
    nodesH = (size_t)ny + 1;
    nodesChannel = nodesW;
    const size_t n = nodesW * nodesH;
    eqf_trap_params t{};
    t.width = p.trapWidthMicrons;
    t.height = p.trapHeightMicrons;
    t.nx = nx;
    t.ny = ny;
    t.D = p.D_HSL;
    t.dt = p.dt;
    t.adv_len = 1.0;
    eqf_solver_opts o;
    eqfield::check(eqf_default_opts(eqfield::precision, &o), nullptr);
    o.use_graph = 1;
    eqfield::check(eqf_create(1, &t, &o, &h_), nullptr);
    const Walls w = decode_boundaries(P, myParams.D_HSL, myParams.nodesPerMicron);
    channels_ = w.channels;
    well_walls_ = w.well;
    eqfield::check(eqf_set_boundaries(h_, 0, &w.bc), h_);
    // vertices in RectangleMesh order (x fastest), the DOF map, the shell's tables
    shell->mesh = std::make_shared<eqfield::Mesh>();
    shell->mesh->coords_.resize(2 * n);
    coords.resize(n);
    for (size_t i = 0; i < nodesH; ++i)
      for (size_t j = 0; j < nodesW; ++j) {
        const size_t v = j + i * nodesW;
        const double x = p.trapWidthMicrons * (double)j / nx;
        const double y = p.trapHeightMicrons * (double)i / ny;
        shell->mesh->coords_[2 * v] = x;
        shell->mesh->coords_[2 * v + 1] = y;
        coords[v] = {x, y};
      }
    shell->mesh_coords = shell->mesh->coords_;
    shell->dof_from_vertex.resize(n);
    for (size_t v = 0; v < n; ++v) shell->dof_from_vertex[v] = (int)v;
    if (eqfield::dof_shuffle_seed) {
      std::mt19937 rng(eqfield::dof_shuffle_seed);
      std::shuffle(shell->dof_from_vertex.begin(), shell->dof_from_vertex.end(), rng);
    }
    shell->vertex_from_dof.resize(n);
    for (size_t v = 0; v < n; ++v) shell->vertex_from_dof[(size_t)shell->dof_from_vertex[v]] = v;
    shell->createGridCoordinatesToDofMapping(nodesH, nodesW, p.nodesPerMicron);
    solution_vector.assign(n, 0.0);
    pushed_ = solution_vector;
    // isotropic tensor (1, 1, 0), as fenicsClassInit initialises it (src/fHSL.cpp:317-323)
    D11 = std::make_shared<std::vector<double>>(n, 1.0);
    D22 = std::make_shared<std::vector<double>>(n, 1.0);
    D12 = std::make_shared<std::vector<double>>(n, 0.0);
    isotropic_ = true;
    t11_.clear();
    // channel buffers (src/fHSL.cpp:418-427) and the flux buffers (src/fHSL.cpp:50-51)
    solution_vectorTopChannel.assign(nodesChannel, 0.0);
    solution_vectorBottomChannel.assign(nodesChannel, 0.0);
    topChannelData.assign(nodesChannel, 0.0);
    bottomChannelData.assign(nodesChannel, 0.0);
    fluxTopChannel.assign(nodesW, 0.0);
    fluxBottomChannel.assign(nodesW, 0.0);
    // h and wellScaling as initDiffusion computes them (src/fHSL.cpp:43-47)
    const double npm = eqfield::num_param(P, "nodesPerMicronSignaling", p.nodesPerMicron);
    wellScaling = 10.0 * (25.0 / eqfield::num_param(P, "lengthScaling", 1.0)) / npm;
    if (!myParams.filePath.empty()) {
      eqfield::check(eqf_vtk_open(myParams.filePath.c_str(), &vtk_), h_);
      if (channels_) {
        if (!myParams.filePathTopChannel.empty())
          eqfield::check(eqf_vtk_open(myParams.filePathTopChannel.c_str(), &vtk_top_), h_);
        if (!myParams.filePathBottomChannel.empty())
          eqfield::check(eqf_vtk_open(myParams.filePathBottomChannel.c_str(), &vtk_bottom_), h_);
      }
    }
  }

  // fenicsInterface::stepDiffusion (src/fHSL.cpp:98-161)
  void stepDiffusion() override {
    if (!h_) throw eqfield::Error(EQF_ERR_INVALID, "stepDiffusion before initDiffusion");
    push_tensor();
    const int32_t* dof = shell->dof_from_vertex.data();
    if (solution_vector != pushed_)
      eqfield::check(eqf_set_nodal_dof(h_, 0, dof, solution_vector.data()), h_);
    eqfield::check(eqf_step(h_, 1), h_);
    eqfield::check(eqf_read_nodal_dof(h_, 0, dof, solution_vector.data()), h_);
    pushed_ = solution_vector;
    if (channels_) {
      eqfield::check(eqf_read_channels(h_, 0, bottomChannelData.data(), topChannelData.data()),
                     h_);
      solution_vectorTopChannel = topChannelData;  // the channels' DOF order is the grid's
      solution_vectorBottomChannel = bottomChannelData;
    }
    eqfield::check(eqf_boundary_flux(h_, 0, &totalBoundaryFlux), h_);
  }

  eQ::data::parametersType getBoundaryFlux(void) override {
    eQ::data::parametersType j;
    j["totalFlux"] = totalBoundaryFlux;
    return j;
  }

  // dolfin File << u (src/fHSL.cpp:606-632): .pvd series of the layer (and channels)
  void writeDiffusionFiles(double timestamp) override {
    if (!h_) return;
    if (vtk_) eqfield::check(eqf_vtk_write(vtk_, h_, 0, timestamp), h_);
    if (vtk_top_)
      eqfield::check(eqf_vtk_write_channel(vtk_top_, h_, 0, EQF_SIDE_TOP, timestamp), h_);
    if (vtk_bottom_)
      eqfield::check(eqf_vtk_write_channel(vtk_bottom_, h_, 0, EQF_SIDE_BOTTOM, timestamp), h_);
  }

  void finalize(void) override {}

  // DIRICHLET_UPDATE: every wall takes the compartment value (src/fHSL.cpp:601-604)
  void setBoundaryValues(const double bval) {
    if (h_ && well_walls_) eqfield::check(eqf_set_well_concentration(h_, 0, bval), h_);
  }

  // cell-data recording (src/fHSL.cpp:637-654): not part of the field step
  void writeDataFiles(double) {}

  // Wall conditions of the layer from eQ::data::parameters, as createHSL decodes them
  // (src/fHSL.cpp:367-573) with the Robin rates of setRobinBoundaryConditions
  // (src/fHSL.cpp:331-364).  D is the layer's diffusion constant, npm its nodes per
  // micron (when parameters has no nodesPerMicronSignaling).
  struct Walls {
    eqf_boundaries bc;
    bool channels, well;
  };
  template <class J>
  static Walls decode_boundaries(J& P, double D, double npm_default) {
    Walls out{};
    eqf_boundaries& bc = out.bc;
    for (int w = 0; w < 4; ++w) bc.wall[w].kind = EQF_BC_NEUMANN;
    bc.channel_substeps = 1;
    bc.well_scaling = 1.0;
    const std::string type = eqfield::str_param(P, "boundaryType", "DIRICHLET_0");
    const std::string trap = eqfield::str_param(P, "trapType", "THREEWALLED");
    auto dirichlet0 = [&](std::initializer_list<int> sides) {
      for (int s : sides) bc.wall[s] = eqf_wall{EQF_BC_DIRICHLET, 0.0, 0.0};
    };
    if (type == "MICROFLUIDIC_TRAP") {
      const double v = eqfield::num_param(P, "simulationFlowRate", 0.0);
      const double lenL = eqfield::num_param(P, "simulationChannelLengthLeft", 1.0);
      const double lenR = eqfield::num_param(P, "simulationChannelLengthRight", 1.0);
      double rl, rr;
      if (v > 1.0e-6) {
        rl = v * (1.0 / (1.0 - std::exp(-(lenL * v) / D)));
        rr = v * (1.0 / (std::exp((lenR * v) / D) - 1.0));
      } else {
        rl = D / lenL;
        rr = D / lenR;
      }
      const double chan_rl = rl, chan_rr = rr;  // the channels keep the flow-derived rates
      const bool htrap = trap == "H_TRAP";
      if (htrap) rl = rr = v;
      auto side = [&](const char* name) {
        return P["boundaries"][name][1].template get<std::vector<double>>();
      };
      auto lr = [&](const std::vector<double>& d, int s, double rate) {
        if (d[0] == 0.0)
          bc.wall[s] = eqf_wall{EQF_BC_DIRICHLET, d[2], 0.0};
        else if (d[1] == 0.0)
          bc.wall[s] = eqf_wall{EQF_BC_NEUMANN, 0.0, 0.0};  // homogeneous only
        else
          bc.wall[s] = eqf_wall{EQF_BC_ROBIN, 0.0, rate};  // external value 0
      };
      lr(side("left"), EQF_SIDE_LEFT, rl);
      lr(side("right"), EQF_SIDE_RIGHT, rr);
      auto tb = [&](const std::vector<double>& d, int s) {
        if (d[0] != 0.0) return;  // Neumann: nothing
        if (d[2] == -1.0 && !htrap) {  // the flow channel (not stepped for an H-trap)
          bc.wall[s] = eqf_wall{EQF_BC_CHANNEL, 0.0, 0.0};
          out.channels = true;
        } else {
          bc.wall[s] = eqf_wall{EQF_BC_DIRICHLET, d[2] == -1.0 ? 0.0 : d[2], 0.0};
        }
      };
      tb(side("top"), EQF_SIDE_TOP);
      tb(side("bottom"), EQF_SIDE_BOTTOM);
      if (out.channels) {
        bc.channel_velocity = v;
        bc.channel_D = D;
        bc.channel_rate[0] = chan_rl;
        bc.channel_rate[1] = chan_rr;
        bc.channel_substeps =
            (int32_t)std::max(1.0, eqfield::num_param(P, "channelSolverNumberIterations", 1.0));
        const double npm = eqfield::num_param(P, "nodesPerMicronSignaling", npm_default);
        bc.well_scaling = 10.0 * (25.0 / eqfield::num_param(P, "lengthScaling", 1.0)) / npm;
      }
    } else if (type == "DIRICHLET_UPDATE") {
      for (int s = 0; s < 4; ++s) bc.wall[s] = eqf_wall{EQF_BC_WELL, 0.0, 0.0};
      out.well = true;
    } else if (type == "DIRICHLET_0") {
      if (trap == "NOWALLED")
        dirichlet0({EQF_SIDE_BOTTOM, EQF_SIDE_TOP, EQF_SIDE_LEFT, EQF_SIDE_RIGHT});
      else if (trap == "THREEWALLED")
        dirichlet0({EQF_SIDE_BOTTOM});
      else if (trap == "TWOWALLED")
        dirichlet0({EQF_SIDE_BOTTOM, EQF_SIDE_TOP});
      else if (trap == "ONEWALLED")
        dirichlet0({EQF_SIDE_BOTTOM, EQF_SIDE_LEFT, EQF_SIDE_RIGHT});
    } else if (type == "NEUMANN_3WALLED_TEST") {
      dirichlet0({EQF_SIDE_BOTTOM, EQF_SIDE_LEFT, EQF_SIDE_RIGHT});
    } else {
      dirichlet0({EQF_SIDE_BOTTOM, EQF_SIDE_TOP, EQF_SIDE_LEFT, EQF_SIDE_RIGHT});
    }
    return out;
  }

  eqf_batch* handle() const { return h_; }
  bool isDataRecordingNode() const { return isDataRecordingNode_; }

 private:
  // the caller's tensor grids, pushed when they changed since the last step
  void push_tensor() {
    const size_t n = nodesW * nodesH;
    auto grid = [&](const std::shared_ptr<std::vector<double>>& d, double test,
                    std::vector<double>& out) {
      out.resize(n);
      for (size_t k = 0; k < n; ++k) out[k] = (d && k < d->size()) ? (*d)[k] : test;
    };
    std::vector<double> a, b, c;
    grid(D11, 1.0, a);
    grid(D22, 1.0, b);
    grid(D12, 0.0, c);
    if (a == t11_ && b == t22_ && c == t12_) return;
    bool iso = true;
    for (size_t k = 0; k < n && iso; ++k) iso = a[k] == 1.0 && b[k] == 1.0 && c[k] == 0.0;
    if (iso) {
      if (!isotropic_) eqfield::check(eqf_set_tensor(h_, 0, nullptr, nullptr, nullptr), h_);
    } else {
      eqfield::check(eqf_set_tensor(h_, 0, a.data(), b.data(), c.data()), h_);
    }
    isotropic_ = iso;
    t11_ = std::move(a);
    t22_ = std::move(b);
    t12_ = std::move(c);
  }

  void release() {
    if (vtk_) eqf_vtk_close(vtk_);
    if (vtk_top_) eqf_vtk_close(vtk_top_);
    if (vtk_bottom_) eqf_vtk_close(vtk_bottom_);
    vtk_ = vtk_top_ = vtk_bottom_ = nullptr;
    if (h_) eqf_destroy(h_);
    h_ = nullptr;
  }

  bool isDataRecordingNode_ = false;
  bool channels_ = false, well_walls_ = false, isotropic_ = true;
  eqf_batch* h_ = nullptr;
  eqf_vtk *vtk_ = nullptr, *vtk_top_ = nullptr, *vtk_bottom_ = nullptr;
  std::vector<double> pushed_, t11_, t22_, t12_;
};

#endif  // FENICS_H
