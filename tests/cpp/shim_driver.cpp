// Test driver of the drop-in fHSL.h: plays the controller's side of
// Simulation::create_HSLgrid / stepSimulation (src/simulation.cpp:181-394, 414-510)
// in one process -- the lookup table from shell->mesh_coords and
// shell->dof_from_vertex, deposits added into solution_vector through it, the
// tensor grids written into D11/D22/D12, setBoundaryValues -- and writes what it
// read back.  Builds against eQ's own src/eQ.h or the stand-in in tests/cpp.
// Test infrastructure only.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fHSL.h"

eQ::data::parametersType eQ::data::parameters;

#ifndef EQ_TEST_STANDIN
// eQ.h declares the insertion of an encoded boundaryCondition into the parameters as
// a friend; eQ's main program defines it.  This one stores the encoded walls.
namespace eQ {
data::parametersType& operator<<(data::parametersType& os, const boundaryCondition& bc) {
  os["boundaries"] = bc._bcs;
  return os;
}
}  // namespace eQ
#endif

static void set_side(const char* side, const char* kind, double a, double b, double v) {
#ifdef EQ_TEST_STANDIN
  eQ::data::parameters["boundaries"][side] =
      eqmock::Json::array({eqmock::Json(kind), eqmock::Json(std::vector<double>{a, b, v})});
#else
  eQ::data::parameters["boundaries"][side] = {kind, {a, b, v}};
#endif
}

// the encodings of eQ::boundaryCondition (src/eQ.h:391-421)
static void dirichlet(const char* side, double v) { set_side(side, "Dirichlet", 0.0, 1.0, v); }
static void neumann(const char* side) { set_side(side, "Neumann", 1.0, 0.0, 0.0); }
static void robin(const char* side) { set_side(side, "Robin", 1.0, 1.0, 0.0); }

static void print_walls(const char* name) {
  const auto w = fenicsInterface::decode_boundaries(eQ::data::parameters, 490.0, 4.0);
  std::printf("%s", name);
  for (int s = 0; s < 4; ++s)
    std::printf(" %d:%.17g:%.17g", w.bc.wall[s].kind, w.bc.wall[s].value, w.bc.wall[s].rate);
  std::printf(" ch=%d well=%d v=%.17g D=%.17g r=%.17g,%.17g sub=%d ws=%.17g\n", w.channels ? 1 : 0,
              w.well ? 1 : 0, w.bc.channel_velocity, w.bc.channel_D, w.bc.channel_rate[0],
              w.bc.channel_rate[1], w.bc.channel_substeps, w.bc.well_scaling);
}

// parameters["..."] = value, the same on both JSON types
template <class T>
static void setp(const char* key, T value) {
  eQ::data::parameters[key] = value;
}

static void microfluidic_parameters() {
  setp("boundaryType", "MICROFLUIDIC_TRAP");
  setp("trapType", "TWOWALLED");
  setp("simulationFlowRate", 40.0);
  setp("simulationChannelLengthLeft", 10.0);
  setp("simulationChannelLengthRight", 12.0);
  setp("channelSolverNumberIterations", 6.0);
  setp("lengthScaling", 1.0);
  setp("nodesPerMicronSignaling", 4.0);
  robin("left");
  robin("right");
  dirichlet("top", -1.0);  // CHANNELUPDATE
  dirichlet("bottom", -1.0);
}

static int decode_cases() {
  setp("boundaryType", "DIRICHLET_0");
  for (const char* t : {"NOWALLED", "THREEWALLED", "TWOWALLED", "ONEWALLED"}) {
    setp("trapType", t);
    print_walls(t);
  }
  setp("boundaryType", "DIRICHLET_UPDATE");
  print_walls("DIRICHLET_UPDATE");
  setp("boundaryType", "NEUMANN_3WALLED_TEST");
  print_walls("NEUMANN_3WALLED_TEST");
  microfluidic_parameters();
  print_walls("MICROFLUIDIC_TRAP");
  dirichlet("left", 0.7);
  neumann("right");
  dirichlet("bottom", 0.3);
  print_walls("MICROFLUIDIC_VALUES");
  setp("simulationFlowRate", 0.0);
  print_walls("MICROFLUIDIC_NOFLOW");
  setp("trapType", "H_TRAP");
  setp("simulationFlowRate", 40.0);
  robin("left");
  robin("right");
  dirichlet("bottom", -1.0);
  print_walls("H_TRAP");
#ifndef EQ_TEST_STANDIN
  // the reference's own encoder: CHANNELUPDATE on top/bottom, ROBIN on left/right
  eQ::boundaryCondition bc;
  bc << eQ::boundaryCondition::type::CHANNELUPDATE << eQ::boundaryCondition::wall::TOP
     << eQ::boundaryCondition::wall::BOTTOM << eQ::boundaryCondition::type::ROBIN
     << eQ::boundaryCondition::wall::LEFT << eQ::boundaryCondition::wall::RIGHT;
  eQ::data::parameters << bc;
  setp("trapType", "TWOWALLED");
  print_walls("ENCODED");
#endif
  return 0;
}

int main(int argc, char** argv) {
  const std::string mode = argc > 1 ? argv[1] : "decode";
  if (mode == "decode") return decode_cases();
  const std::string out = argc > 2 ? argv[2] : "shim_out.bin";
  eQ::diffusionSolver::params p{};
  p.dt = 0.1;
  p.D_HSL = 49.0;
  p.trapWidthMicrons = 20.0;
  p.trapHeightMicrons = 10.0;
  p.nodesPerMicron = 4.0;
  p.filePath = argc > 3 ? argv[3] : "";
  if (mode == "aniso") {
    setp("boundaryType", "DIRICHLET_0");
    setp("trapType", "THREEWALLED");
  } else if (mode == "microfluidic") {
    microfluidic_parameters();
    p.D_HSL = 490.0;
  } else if (mode == "update") {
    setp("boundaryType", "DIRICHLET_UPDATE");
  } else {
    std::printf("unknown mode\n");
    return 2;
  }
  eqfield::dof_shuffle_seed = 7;  // a DOF order that is not the grid order
  auto solver = std::make_shared<fenicsInterface>();
  try {
    solver->initDiffusion(p);
  } catch (const eqfield::Error& e) {
    std::printf("init-error %d %s\n", e.code, e.what());
    return 3;
  }
  // Simulation::create_HSLgrid's check and lookup table (src/simulation.cpp:298-301, 363-386)
  const size_t nh = solver->nodesH, nw = solver->nodesW, n = nh * nw;
  if (solver->shell->mesh->num_vertices() != n) {
    std::printf("vertex count mismatch\n");
    return 4;
  }
  const double npm = p.nodesPerMicron;
  eQ::gridFunction<size_t> table(nh, nw);
  for (size_t v = 0; v < n; ++v) {
    const auto ij = eQ::data::ij_from_xy(solver->shell->mesh_coords[2 * v],
                                         solver->shell->mesh_coords[2 * v + 1], npm);
    table[ij] = size_t(solver->shell->dof_from_vertex[v]);
  }
  FILE* f = std::fopen(out.c_str(), "wb");
  const int steps = 6;
  for (int s = 0; s < steps; ++s) {
    // deposits into the nodal vector through the lookup table (writeHSL)
    solver->solution_vector[table[{20, 30}]] += 1.0 + s;
    solver->solution_vector[table[{12, 61}]] += 0.5;
    solver->solution_vector[table[{33, 7}]] += 0.25 * s;
    if (mode == "aniso" && (s == 0 || s == 3)) {  // the controller's tensor grids
      const double turn = s == 0 ? 0.0 : 0.9;
      for (size_t i = 0; i < nh; ++i)
        for (size_t j = 0; j < nw; ++j) {
          const double th = turn + 0.6 * std::sin(6.283185307179586 * j / (nw - 1)) +
                            0.4 * double(i) / (nh - 1);
          const double c = std::cos(th), sn = std::sin(th), dx = 2.0, dy = 0.5;
          (*solver->D11)[i * nw + j] = dx * c * c + dy * sn * sn;
          (*solver->D22)[i * nw + j] = dx * sn * sn + dy * c * c;
          (*solver->D12)[i * nw + j] = (dx - dy) * sn * c;
        }
    }
    if (mode == "update") solver->setBoundaryValues(0.2 * (s + 1));
    solver->stepDiffusion();
    if (!p.filePath.empty()) solver->writeDiffusionFiles(0.1 * (s + 1));
    // the field in grid order, read through the table
    std::vector<double> grid(n);
    for (size_t i = 0; i < nh; ++i)
      for (size_t j = 0; j < nw; ++j) grid[i * nw + j] = solver->solution_vector[table[{i, j}]];
    std::fwrite(grid.data(), sizeof(double), n, f);
    std::fwrite(&solver->totalBoundaryFlux, sizeof(double), 1, f);
    std::fwrite(solver->bottomChannelData.data(), sizeof(double), solver->bottomChannelData.size(), f);
    std::fwrite(solver->topChannelData.data(), sizeof(double), solver->topChannelData.size(), f);
  }
  std::fclose(f);
  const auto flux = solver->getBoundaryFlux();
  (void)flux;
  dolfin::SubSystemsManager::singleton().finalize();
  std::printf("ok %zu %zu\n", nh, nw);
  return 0;
}
