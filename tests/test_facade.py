"""The C++ facade (include/lpm_gb300.hpp) compiles against the header and
links against the shared library like a reference-side host would; without a
GPU, creating a context throws std::runtime_error (LPM_REQUIRE style), and the
host-only entry points work."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

PROGRAM = r'''
#include <cstdio>
#include <stdexcept>
#include <vector>
#include "lpm_gb300.hpp"
int main() {
  int64_t nv = 0, nf = 0;
  lpm_gb300::require(lpm_mesh_sizes(LPM_MESH_ICOS_TRI, 3, &nv, &nf), "mesh sizes");
  std::vector<double> vx(3 * nv), fx(3 * nf), fa(nf);
  std::vector<uint8_t> fm(nf);
  lpm_gb300::require(lpm_mesh_build(LPM_MESH_ICOS_TRI, 3, 1.0, vx.data(), fx.data(), fa.data(),
                                    fm.data()), "mesh");
  int64_t st[9];
  lpm_gb300::require(lpm_octree_stats(fx.data(), nf, vx.data(), nv, 64, st), "octree");
  std::printf("mesh %lld %lld octree_errors %lld\n", (long long)nv, (long long)nf, (long long)st[8]);
  try {
    lpm_gb300::Context ctx(0, LPM_FP32C);
    std::printf("context ok\n");
  } catch (const std::runtime_error& e) {
    std::printf("context error: %s\n", e.what());
  }
  return 0;
}
'''


def test_cpp_facade_builds_links_and_runs(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    from lpm_gb300 import build as B

    lib = B.build()
    src = tmp_path / "host.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "host"
    cuda_inc = "/usr/local/cuda/include"
    cmd = ["g++", "-std=c++17", f"-I{ROOT / 'include'}", f"-I{cuda_inc}", str(src), "-o", str(exe),
           f"-L{lib.parent}", "-llpm_gb300", f"-Wl,-rpath,{lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    env = dict(os.environ)
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "mesh 642 1700 octree_errors 0" in r.stdout
    assert "context ok" in r.stdout or "context error" in r.stdout
