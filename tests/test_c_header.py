"""The C ABI from plain C and C++: include/dcg.h compiles as C99 and as C++11
under -Wall -Wextra -pedantic -Werror, and a program linked against
libdcgrid_gb300.so runs the calls that need no GPU (defaults, struct sizes,
the memory planner, null-handle rejection) with the same results as the
Python mirror."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from dcgrid_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include "dcg.h"

int main(void) {
  dcg_params p;
  int64_t bytes = 0, blocks = 0;
  int rc;
  dcg_default_params(&p, 64, 128, 64, 3000);
  printf("sizes %zu %zu %zu %zu %zu\n", dcg_sizeof_params(), dcg_sizeof_info(), dcg_sizeof_stats(),
         dcg_sizeof_tuning(), dcg_sizeof_render_params());
  printf("defaults %g %g %d %d\n", (double)p.dt, (double)p.dx, (int)p.jacobi_iters, (int)p.init_adapt_passes);
  rc = dcg_plan_bytes(&p, DCG_MODE_ADAPTIVE, &bytes);
  printf("plan %d %lld\n", rc, (long long)bytes);
  rc = dcg_blocks_for_budget(&p, (int64_t)1 << 30, &blocks);
  printf("budget %d %lld\n", rc, (long long)blocks);
  printf("null %d %d\n", dcg_step(NULL, 1), dcg_set_heightmap(NULL, NULL, 0, 0, DCG_HOST));
  return 0;
}
"""


@pytest.fixture(scope="module")
def c_program(dcg_lib, tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("c_abi")
    src, exe = d / "prog.c", d / "prog"
    src.write_text(PROGRAM)
    libdir = os.path.join(ROOT, "dcgrid_gb300")
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
           str(src), "-o", str(exe), "-L", libdir, "-ldcgrid_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    return dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())


def test_struct_sizes_match_the_python_mirror(c_program):
    sizes = [int(x) for x in c_program["sizes"].split()]
    assert sizes == [C.sizeof(capi.DcgParams), C.sizeof(capi.DcgInfo), C.sizeof(capi.DcgStats),
                     C.sizeof(capi.DcgTuning), C.sizeof(capi.DcgRenderParams)]


def test_defaults_and_planner_match_the_python_mirror(c_program, dcg_lib):
    p = capi.default_params(64, 128, 64, 3000)
    dt, dx, iters, passes = c_program["defaults"].split()
    assert (float(dt), float(dx), int(iters), int(passes)) == pytest.approx(
        (p.dt, p.dx, p.jacobi_iters, p.init_adapt_passes))
    rc, nbytes = (int(x) for x in c_program["plan"].split())
    want = C.c_int64()
    assert rc == capi.DCG_OK
    assert dcg_lib.dcg_plan_bytes(C.byref(p), capi.MODE_ADAPTIVE, C.byref(want)) == capi.DCG_OK
    assert nbytes == want.value > 0
    rc, blocks = (int(x) for x in c_program["budget"].split())
    assert rc == capi.DCG_OK and blocks >= 3000


def test_null_handles_from_c(c_program):
    assert [int(x) for x in c_program["null"].split()] == [capi.DCG_E_INVALID, capi.DCG_E_INVALID]


def test_header_compiles_as_cpp(tmp_path, dcg_lib):
    """The reference's side is C++: the header also compiles as C++11 under
    -pedantic -Werror, and its extern "C" names link."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "prog.cpp"
    src.write_text(PROGRAM.replace("#include <stdio.h>", "#include <cstdio>"))
    libdir = os.path.join(ROOT, "dcgrid_gb300")
    cmd = [cxx, "-std=c++11", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
           str(src), "-o", str(tmp_path / "prog"), "-L", libdir, "-ldcgrid_gb300", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(tmp_path / "prog")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "plan 0 " in r.stdout, r.stdout + r.stderr
