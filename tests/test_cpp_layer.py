"""The C++ layer (include/mps_system.hpp): compiles and links against libmps_gb300.so on the CPU;
on the GPU the example program's state after 20 frames equals the Python API's bit for bit."""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def compile_example(out: Path) -> Path:
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    lib = ROOT / "mps_cuda_gb300"
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", f"-I{cuda / 'include'}",
           str(ROOT / "tests/cpp/system_example.cpp"), f"-L{lib}", "-lmps_gb300", f"-Wl,-rpath,{lib}",
           f"-L{cuda / 'lib64'}", "-lcudart", f"-Wl,-rpath,{cuda / 'lib64'}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_cpp_layer_compiles_and_links(mps, tmp_path):
    exe = compile_example(tmp_path / "system_example")
    assert exe.exists()


def test_cpp_material_semantics(mps, tmp_path):
    """SPHMaterial defaults and SetRadius as the reference computes them (MPSSPHMaterial.cpp)."""
    src = tmp_path / "mat.cpp"
    src.write_text('''#include <cstdio>
#include "mps_system.hpp"
int main() { mps::SPHMaterial m; m.SetRadius(0.4);
  std::printf("%.17g %.17g %.17g %.17g %.17g %.17g\\n", m.GetRadius(), m.GetVolume(), m.GetMass(), m.GetViscosity(),
              m.GetXSPH(), m.GetSurfaceTension()); return 0; }''')
    cxx = shutil.which("g++") or pytest.skip("no C++ compiler")
    exe = tmp_path / "mat"
    r = subprocess.run([cxx, "-std=c++17", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    vals = [float(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    h = 0.4
    assert vals == [h, h ** 3 / 48.0 * 3.141592, h ** 3 / 48.0 * 3.141592 * 1.0, 0.025, 0.1, 100.0]


@pytest.mark.gpu
def test_cpp_example_matches_python_api(mps, tmp_path):
    from mps_cuda_gb300 import Simulation, scenes
    exe = compile_example(tmp_path / "system_example")
    out = tmp_path / "state.bin"
    r = subprocess.run([str(exe), str(out), "20"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "frames 20 steps 20" in r.stdout
    data = np.fromfile(out, np.float32).reshape(2, -1, 4)
    sim = Simulation.from_scene(scenes.dam_break_small(10, seed=0))
    sim.step(20)
    p, v = sim.get_fluid()
    assert np.array_equal(data[0], p) and np.array_equal(data[1], v)
    # the same frames through the phase functions (the reference's OnUpdate call sequence)
    out2 = tmp_path / "state_phases.bin"
    r = subprocess.run([str(exe), str(out2), "20", "phases"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "frames 20 steps 20" in r.stdout
    data2 = np.fromfile(out2, np.float32).reshape(2, -1, 4)
    assert np.array_equal(data2, data)
