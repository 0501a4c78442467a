"""CPU checks of the C-ABI library: it loads, exports every function
include/dcg.h declares, the ctypes struct mirrors match the C layouts, and
the Python default parameters equal dcg_default_params. No compute calls."""
import ctypes as C
import os
import re

import pytest

from dcgrid_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(dcg_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_library_exports_every_declared_symbol(dcg_lib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(dcg_lib, n)]
    assert not missing, missing


def test_struct_layouts(dcg_lib):
    assert dcg_lib.dcg_sizeof_params() == C.sizeof(capi.DcgParams)
    assert dcg_lib.dcg_sizeof_info() == C.sizeof(capi.DcgInfo)
    assert dcg_lib.dcg_sizeof_stats() == C.sizeof(capi.DcgStats)
    dcg_lib.dcg_sizeof_tuning.restype = C.c_size_t
    assert dcg_lib.dcg_sizeof_tuning() == C.sizeof(capi.DcgTuning)
    assert dcg_lib.dcg_sizeof_render_params() == C.sizeof(capi.DcgRenderParams)


def test_python_defaults_match_c_defaults(dcg_lib):
    from dcgrid_gb300 import sim
    a = sim.default_params(256, 256, 256, 40000)
    b = capi.default_params(256, 256, 256, 40000)
    assert capi.params_to_dict(a) == pytest.approx(capi.params_to_dict(b))


def test_null_handles_are_rejected(dcg_lib):
    assert dcg_lib.dcg_step(None, 1) == capi.DCG_E_INVALID
    assert dcg_lib.dcg_destroy(None) == capi.DCG_E_INVALID
    assert dcg_lib.dcg_create(None, 0, None) == capi.DCG_E_INVALID
    assert dcg_lib.dcg_batch_step(None, 1) == capi.DCG_E_INVALID
    assert dcg_lib.dcg_batch_destroy(None) == capi.DCG_E_INVALID
    assert dcg_lib.dcg_batch_create(0, None, None) == capi.DCG_E_INVALID


def test_oracle_exports(oracle_lib):
    for n in ["dcgo_create", "dcgo_step", "dcgo_get_field", "dcgo_apron_mismatches", "dcgo_adapt_replay"]:
        assert hasattr(oracle_lib, n)


def test_tuning_dict_round_trip():
    from dcgrid_gb300 import capi
    t = capi.DcgTuning()
    t.tile[0], t.tile[3], t.solve_cache, t.solve_ctas_per_sm, t.solve_barrier = 1, 8, 19, 3, 2
    t.round_ctas_per_sm[2], t.round_cache[2], t.round_barrier[2] = -4, 18, 1
    d = capi.tuning_to_dict(t)
    back = capi.tuning_to_dict(capi.tuning_from_dict(d))
    assert back == d


def declared_arities():
    """{function: parameter count} from include/dcg.h."""
    txt = open(os.path.join(ROOT, "include", "dcg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for name, args in re.findall(r"\b(dcg_[a-z0-9_]+)\s*\(([^()]*)\)\s*;", txt):
        args = args.strip()
        out[name] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_python_bindings_match_the_header_arities(dcg_lib):
    arity = declared_arities()
    assert len(arity) >= 60
    checked = 0
    for name, n in arity.items():
        fn = getattr(dcg_lib, name)
        if fn.argtypes is not None:
            assert len(fn.argtypes) == n, f"{name}: header has {n} parameters, binding {len(fn.argtypes)}"
            checked += 1
    assert checked == len(arity)  # every declared function has its argument types bound
