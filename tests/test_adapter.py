"""The C++ FluidSimulation adapter (dcgrid_gb300/adapter/fluid_simulation_gb300.h).

* CPU: it compiles against the reference's unmodified interface headers
  (src/fluid_simulation.h, src/data/sim_params.h) when the reference's source
  tree is present, and against the restated interface always.
* GPU: a C++ program drives the reference's frame order through the adapter
  and checks it against dcg_step bit for bit, and the adapter's render() into
  a CUDA surface against dcg_render.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(ROOT, "dcgrid_gb300", "adapter")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _reference_src():
    import __graft_entry__ as g
    src = os.path.join(g.REFERENCE_TREE, "src")
    return src if os.path.isfile(os.path.join(src, "fluid_simulation.h")) else None


def _compile(extra, out=None, src=None, tmp=None):
    cxx = shutil.which("g++")
    if not cxx or not os.path.isdir(os.path.join(CUDA, "include")):
        pytest.skip("g++ or the CUDA headers missing")
    cmd = [cxx, "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I", ADAPTER,
           "-I", os.path.join(CUDA, "include")] + extra
    if out is None:
        unit = os.path.join(str(tmp), "unit.cpp")
        with open(unit, "w") as f:
            f.write('#include "fluid_simulation_gb300.h"\n')
        cmd += ["-fsyntax-only", "-H", unit]
    else:
        cmd += [src, "-o", out, "-L", os.path.join(ROOT, "dcgrid_gb300"), "-ldcgrid_gb300",
                "-L", os.path.join(CUDA, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(ROOT, "dcgrid_gb300")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return r.stderr


def test_adapter_compiles_against_the_reference_interface(tmp_path):
    src = _reference_src()
    if src is None:
        pytest.skip("the reference's source tree is not present")
    headers = _compile(["-I", src], tmp=tmp_path)
    # the reference's own interface headers were the ones included
    assert os.path.join(src, "fluid_simulation.h") in headers
    assert os.path.join(src, "data", "sim_params.h") in headers
    assert "reference_interface.h" not in headers


def test_adapter_compiles_against_the_restated_interface(tmp_path):
    assert "reference_interface.h" in _compile([], tmp=tmp_path)


@pytest.mark.gpu
@pytest.mark.usefixtures("cuda_ok", "dcg_lib")
def test_adapter_runs_the_reference_frame_order(tmp_path):
    exe = str(tmp_path / "adapter_frame_order")
    _compile([], out=exe, src=os.path.join(ROOT, "tests", "cpp", "adapter_frame_order.cpp"))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stderr
    assert "adapter ok" in r.stdout
