"""The C++ host object (host/PatchMHDMF.hpp): a program that configures it
through the reference's setter names (main/MHDAM.cpp:771-1046) compiles
against the header, links libmfgpu.so and reports the state count and ghost
layers of EqSysMHDMF / PatchMHDAM::numGhostCells without touching the GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ms-flukss-multifluid_gb300")

PROGRAM = r"""
#include "PatchMHDMF.hpp"
#include <cstdio>
int main() {
  mfgpu::PatchMHDMF a(3, 4);
  a.setDivergenceCleaning(5, 0.5, 1.0);
  a.setTimeApproximation(mfgpu::PatchMHDMF::TA_RK2);
  std::printf("%d %d\n", a.numStates(), a.numGhostCells());
  const double u[3] = {-1.0, 0.0, 0.0};
  a.setTrackingSurfaces(1, MF_LIM_MC, true, u);
  a.setTimeApproximation(mfgpu::PatchMHDMF::TA_Hancock);
  std::printf("%d %d %d %d %g\n", a.numStates(), a.numGhostCells(), a.params().limiter_ls,
              a.params().region_tracer, a.params().lism_u[0]);
  mfgpu::PatchMHDMF b(2, 1);
  b.setTrackingSurfaces(2, MF_LIM_MINMOD);
  std::printf("%d\n", b.numStates());
  return 0;
}
"""


def test_host_object_configures_like_the_reference(gpulib, tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "t.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "t"
    lib = os.path.join(PKG, "mfgpu")
    subprocess.run(["g++", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(PKG, "host"), str(src), "-L" + lib, "-lmfgpu",
                    "-Wl,-rpath," + lib, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    # plasma + psi + 3 neutrals = 24 states, RK2: 4 ghosts; one more state
    # with the region tracer, Hancock: 3 ghosts; MHD alone + 2 surfaces: 10
    assert out == ["24", "4", "25", "3", "4", "1", "-1", "10"]
