"""The C++ drop-in (eq_gb300/cpp/gpu_field_solver.hpp): it compiles stand-alone and
against a stand-in of eQ's plugin base class, and on a GPU it reproduces the oracle
for the reference's own step semantics (deposits added into solution_vector, then
stepDiffusion)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from eq_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r'''
#include <cstdio>
#include <cstring>
#include <string>
#include "gpu_field_solver.hpp"
struct Params {  // the fields of eQ::diffusionSolver::params the solver reads
  double dt, D_HSL, trapHeightMicrons, trapWidthMicrons, nodesPerMicron;
  std::string filePath;
};
int main(int argc, char** argv) {
  Params p{0.1, 490.0, 20.0, 40.0, 4.0, ""};
  eqfield::GpuFieldSolver s;  // THREEWALLED, no decay, FP64
  try {
    s.initDiffusion(p);
  } catch (const eqfield::Error& e) {
    std::printf("init-error %d\n", e.code);
    return 0;
  }
  // reference semantics (src/abm/eQabm.cpp:347-358): deposits are added into the
  // nodal vector, then the layer is stepped
  const size_t n = s.solution_vector.size();
  for (int step = 0; step < 5; ++step) {
    s.solution_vector[(size_t)(40 + 161 * 30)] += 1.0;
    s.solution_vector[(size_t)(100 + 161 * 60)] += 0.5 * (step + 1);
    s.stepDiffusion();
  }
  FILE* f = std::fopen(argv[1], "wb");
  std::fwrite(s.solution_vector.data(), sizeof(double), n, f);
  std::fclose(f);
  std::printf("ok %zu %.17g\n", n, s.getBoundaryFlux()["totalFlux"]);
  return 0;
}
'''

MOCK_EQ = r'''
#include <map>
#include <memory>
#include <string>
#include <vector>
// stand-in for the parts of src/eQ.h the adapter binds to (the plugin interface)
namespace eQ {
namespace data {
struct parametersType {
  std::map<std::string, double> v;
  double& operator[](const std::string& k) { return v[k]; }
};
}  // namespace data
class diffusionSolver {
 public:
  struct params {
    int argc; char** argv; size_t uniqueID; int comm; double dt; double D_HSL;
    std::string filePath, filePathTopChannel, filePathBottomChannel;
    std::shared_ptr<int> dataFiles;
    double trapHeightMicrons, trapWidthMicrons, nodesPerMicron, trapChannelVelocity;
  };
  virtual void initDiffusion(eQ::diffusionSolver::params&) = 0;
  virtual void stepDiffusion() {}
  virtual eQ::data::parametersType getBoundaryFlux(void) { return {}; }
  virtual void writeDiffusionFiles(double timestamp) = 0;
  virtual void finalize(void) {}
  virtual ~diffusionSolver() = default;
};
}  // namespace eQ
#define EQFIELD_WITH_EQ
#include "gpu_field_solver.hpp"
int main() {
  std::shared_ptr<eQ::diffusionSolver> s = std::make_shared<eqfield::GpuFieldSolver>();
  (void)s;
  return 0;
}
'''


def _compile(src_text, exe, extra=()):
    with tempfile.NamedTemporaryFile("w", suffix=".cpp", delete=False) as f:
        f.write(src_text)
        src = f.name
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "eq_gb300", "cpp"), src, "-o", exe,
           "-L", os.path.dirname(_lib.LIB_PATH), "-leqfield",
           "-Wl,-rpath," + os.path.dirname(_lib.LIB_PATH)] + list(extra)
    subprocess.run(cmd, check=True)
    os.unlink(src)


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    build.build()
    exe = str(tmp_path_factory.mktemp("cpp") / "driver")
    _compile(DRIVER, exe)
    return exe


def test_adapter_compiles_against_the_plugin_interface(tmp_path):
    build.build()
    _compile(MOCK_EQ, str(tmp_path / "mock"))


def test_adapter_runs_or_reports_missing_device(driver, tmp_path):
    out = subprocess.run([driver, str(tmp_path / "u.bin")], capture_output=True, text=True,
                         check=True).stdout
    assert out.startswith("ok") or out.startswith("init-error")


@pytest.mark.gpu
def test_adapter_matches_oracle_with_reference_deposits(driver, tmp_path):
    from oracle import hsld
    path = str(tmp_path / "u.bin")
    out = subprocess.run([driver, path], capture_output=True, text=True, check=True).stdout
    assert out.startswith("ok"), out
    u_gpu = np.fromfile(path, dtype=np.float64)
    o = hsld.HsldOracle(40.0, 20.0, 160, 80, 490.0, 0.1, 0.0, walls=1)
    u = np.zeros(o.mesh.n_nodes)
    for step in range(5):
        u[40 + 161 * 30] += 1.0
        u[100 + 161 * 60] += 0.5 * (step + 1)
        u = o.step(u)
    assert np.linalg.norm(u_gpu - u) / np.linalg.norm(u) <= 1e-9
    flux = float(out.split()[2])
    assert abs(flux - o.boundary_flux(u)) <= 1e-9 * abs(o.boundary_flux(u))
