// GpuFieldSolver — eQ's HSL-layer solver interface over the eqfield C ABI.
//
// Drop-in for fenicsInterface (src/fHSL.h:333-449), the implementation of the
// plugin eQ::diffusionSolver (src/eQ.h:302-330).  It keeps the public members that
// Simulation reads and writes (src/simulation.cpp:207-313, 475-505, 536-546,
// 583-602): solution_vector (grid order; the DOLFIN DOF map is the identity here,
// so shell-style mesh_coords / dof_from_vertex are provided for the DOF-table
// exchange of create_HSLgrid), totalBoundaryFlux, and the tensor grids D11/D22/D12.
//
// Inside eQ, define EQFIELD_WITH_EQ before including this header (after eQ.h) and
// the class derives from eQ::diffusionSolver; stand-alone it only needs
// include/eqfield.h and libeqfield.so.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <fstream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "eqfield.h"

namespace eqfield {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc, const eqf_batch* h) {
  if (rc != EQF_OK) throw Error(rc, eqf_last_error(h));
}

#ifdef EQFIELD_WITH_EQ
#define EQFIELD_BASE : public eQ::diffusionSolver
#define EQFIELD_OVERRIDE override
#else
#define EQFIELD_BASE
#define EQFIELD_OVERRIDE
#endif

class GpuFieldSolver EQFIELD_BASE {
 public:
  // Wall set of the trap (the reference decodes trapType under DIRICHLET_0,
  // src/fHSL.cpp:557-569): THREEWALLED = bottom wall open (Dirichlet).
  explicit GpuFieldSolver(uint32_t walls = EQF_WALL_BOTTOM, double decay = 0.0,
                          int precision = EQF_PREC_FP64)
      : walls_(walls), decay_(decay), precision_(precision) {}
  ~GpuFieldSolver() { finalize(); }
  GpuFieldSolver(const GpuFieldSolver&) = delete;
  GpuFieldSolver& operator=(const GpuFieldSolver&) = delete;

  // Accepts eQ::diffusionSolver::params or any struct with the same fields
  // (dt, D_HSL, trapWidthMicrons, trapHeightMicrons, nodesPerMicron, filePath).
  template <class Params>
  void initDiffusion_(const Params& p) {
    finalize();
    dt_ = p.dt;
    D_ = p.D_HSL;
    filePath_ = p.filePath;
    // squares as in fenicsClassInit (src/fHSL.cpp:242-243)
    nx_ = (int32_t)std::ceil(p.trapWidthMicrons * p.nodesPerMicron);
    ny_ = (int32_t)std::ceil(p.trapHeightMicrons * p.nodesPerMicron);
    eqf_trap_params t{};
    t.width = p.trapWidthMicrons;
    t.height = p.trapHeightMicrons;
    t.nx = nx_;
    t.ny = ny_;
    t.D = p.D_HSL;
    t.dt = p.dt;
    t.decay = decay_;
    t.adv_u = 0.0;
    t.adv_len = 1.0;
    t.walls = walls_;
    eqf_solver_opts o;
    check(eqf_default_opts(precision_, &o), nullptr);
    o.use_graph = 1;
    check(eqf_create(1, &t, &o, &h_), nullptr);
    nodesW = (size_t)nx_ + 1;
    nodesH = (size_t)ny_ + 1;
    const size_t n = nodesW * nodesH;
    solution_vector.assign(n, 0.0);
    pushed_ = solution_vector;
    D11 = std::make_shared<std::vector<double>>(n, 1.0);
    D22 = std::make_shared<std::vector<double>>(n, 1.0);
    D12 = std::make_shared<std::vector<double>>(n, 0.0);
    // grid-order coordinates and the identity DOF map (fenicsShell, src/fHSL.h:116-118)
    mesh_coords.resize(2 * n);
    dof_from_vertex.resize(n);
    for (size_t i = 0; i < nodesH; ++i)
      for (size_t j = 0; j < nodesW; ++j) {
        const size_t k = j + i * nodesW;
        mesh_coords[2 * k] = p.trapWidthMicrons * (double)j / nx_;
        mesh_coords[2 * k + 1] = p.trapHeightMicrons * (double)i / ny_;
        dof_from_vertex[k] = (int)k;
      }
  }

#ifdef EQFIELD_WITH_EQ
  void initDiffusion(eQ::diffusionSolver::params& p) override { initDiffusion_(p); }
#else
  template <class Params>
  void initDiffusion(Params& p) {
    initDiffusion_(p);
  }
#endif

  // One backward-Euler step (fenicsInterface::stepDiffusion, src/fHSL.cpp:98-161):
  // the caller's edits of solution_vector (deposits) are pushed, the new field is
  // pulled back and totalBoundaryFlux is refreshed.
  void stepDiffusion() EQFIELD_OVERRIDE {
    if (solution_vector != pushed_) check(eqf_set_nodal(h_, 0, solution_vector.data()), h_);
    check(eqf_step(h_, 1), h_);
    check(eqf_read_nodal(h_, 0, solution_vector.data()), h_);
    pushed_ = solution_vector;
    check(eqf_boundary_flux(h_, 0, &totalBoundaryFlux), h_);
  }

#ifdef EQFIELD_WITH_EQ
  eQ::data::parametersType getBoundaryFlux(void) override {
    eQ::data::parametersType j;
    j["totalFlux"] = totalBoundaryFlux;
    return j;
  }
#else
  std::map<std::string, double> getBoundaryFlux() { return {{"totalFlux", totalBoundaryFlux}}; }
#endif

  // The reference writes DOLFIN .pvd files; this writes the nodal field in grid
  // order as a JSON frame like the reference main program's externalHSL record
  // (src/main.cpp:148-162).
  void writeDiffusionFiles(double timestamp) EQFIELD_OVERRIDE {
    if (filePath_.empty()) return;
    std::ofstream f(filePath_ + "_" + std::to_string(timestamp) + ".json");
    f << "{\"time\": " << timestamp << ", \"nodesW\": " << nodesW << ", \"nodesH\": " << nodesH
      << ", \"externalHSL\": [";
    for (size_t k = 0; k < solution_vector.size(); ++k) f << (k ? "," : "") << solution_vector[k];
    f << "]}\n";
  }

  void finalize() EQFIELD_OVERRIDE {
    if (h_) eqf_destroy(h_);
    h_ = nullptr;
  }

  eqf_batch* handle() const { return h_; }

  // data plane read/written by Simulation
  std::vector<double> solution_vector;
  double totalBoundaryFlux = 0.0;
  std::shared_ptr<std::vector<double>> D11, D22, D12;
  std::vector<double> mesh_coords;
  std::vector<int> dof_from_vertex;
  size_t nodesW = 0, nodesH = 0;

 private:
  uint32_t walls_;
  double decay_;
  int precision_;
  double dt_ = 0.0, D_ = 0.0;
  int32_t nx_ = 0, ny_ = 0;
  std::string filePath_;
  eqf_batch* h_ = nullptr;
  std::vector<double> pushed_;
};

}  // namespace eqfield
