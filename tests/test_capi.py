"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/vardyn_gb300.h declares (no GPU needed: no compute calls)."""
import ctypes
import os
import re

import pytest

from vardyn_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "vardyn_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vd_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from vardyn_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("vd_qg1l_plan_create", "vd_qg1l_step", "vd_qg1l_step_tgl", "vd_qg1l_step_adj",
              "vd_qg1l_pv2h", "vd_obs_misfit", "vd_obs_adjoint", "vd_sumsq_f64"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_header():
    from vardyn_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES), \
        set(declared_symbols()) - set(_lib.SIGNATURES)


def test_version_string(lib):
    assert b"sm_103a" in lib.vd_version()


def test_null_arguments_are_rejected_without_gpu(lib):
    # argument validation happens before any CUDA call
    assert lib.vd_qg1l_plan_create(None, None) == 1
    assert lib.vd_obs_misfit(7, 1, None, 0, None, None, None, None, None, None, None) == 1
    d = _lib.VdQgtracDesc()
    d.ntrac, d.time_scheme = 1, _lib.VD_RK2
    # no plan, an unknown scheme, a tracer model without relaxation weights
    assert lib.vd_qgtrac_workspace_bytes(None, ctypes.byref(d), 1) == 0
    assert lib.vd_qgtrac_step(None, ctypes.byref(d), 1, None, None, None, None, 1, None, None, None, 0, None) == 1
    # npix out of range, non-positive spacing
    assert lib.vd_obs_knn_excl(1, None, None, 4, 4, 1.0, 1.0, 5, 2.0, None, None, None, None) == 1
    assert lib.vd_obs_knn_excl(1, None, None, 4, 4, 0.0, 1.0, 4, 2.0, None, None, None, None) == 1
    assert lib.vd_obs_knn_excl(0, None, None, 4, 4, 1.0, 1.0, 4, 2.0, None, None, None, None) == 0
    assert lib.vd_qg1l_workspace_bytes(None, 4) == 0
