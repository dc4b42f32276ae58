"""The C ABI library without a GPU: it loads, exports every entry point that
include/agb.h declares, and its host-only parts (synthetic inputs, option
defaults, argument checks) behave.  No kernel is launched here."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "agb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(agb_[a-z0-9_]+)\s*\(", src)))


def test_header_lists_match_python_binding(agb):
    from alamo_gb300 import _lib
    assert sorted(_lib.EXPORTS) == declared_symbols()


def test_library_exports_every_declared_symbol(agb):
    lib = agb.lib()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", agb.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (agb_[a-z0-9_]+)", out))
    assert set(declared_symbols()) <= exported


def test_default_opts_mirror_reference_defaults(agb):
    o = agb.default_opts()
    assert (o.pre_smooth, o.post_smooth, o.final_smooth, o.bottom_smooth) == (2, 2, 8, 0)
    assert abs(o.omega - 2.0 / 3.0) < 1e-15
    assert o.bottom_tol_rel == 1e-4 and o.max_iter == 200 and o.max_coarsening_level == -1


def test_status_strings(agb):
    from alamo_gb300 import _lib
    assert _lib.status_string(_lib.AGB_NOT_CONVERGED) == "AGB_NOT_CONVERGED"
    assert _lib.status_string(99) == "AGB_UNKNOWN"


def test_create_rejects_bad_arguments(agb):
    from alamo_gb300 import _lib
    h = ctypes.c_void_p()
    dx = (ctypes.c_double * 3)(1, 1, 1)
    assert agb.lib().agb_elastic_create(ctypes.byref(h), 2, 5, 5, dx, 0, None) == _lib.AGB_BAD_ARG
    assert agb.lib().agb_elastic_create(ctypes.byref(h), 5, 5, 5, dx, 7, None) == _lib.AGB_BAD_ARG
    bad = (ctypes.c_double * 3)(1, -1, 1)
    assert agb.lib().agb_elastic_create(ctypes.byref(h), 5, 5, 5, bad, 0, None) == _lib.AGB_BAD_ARG
    assert agb.lib().agb_elastic_create(None, 5, 5, 5, dx, 0, None) == _lib.AGB_BAD_ARG
    assert agb.lib().agb_elastic_destroy(None) == _lib.AGB_OK


def test_synthetic_inputs_are_deterministic(agb):
    from alamo_gb300 import synth
    a = synth.uniform(20261203, (3, 9, 9, 9))
    b = synth.uniform(20261203, (3, 9, 9, 9))
    assert np.array_equal(a, b) and a.min() >= -1 and a.max() < 1
    C1, dx = synth.voronoi_cubic(17, 8, seed=4)
    C2, _ = synth.voronoi_cubic(17, 8, seed=4)
    assert np.array_equal(C1, C2) and C1.shape == (17, 17, 17, 21)
    C, F0, dx, placed = synth.spheres_iso(33, 20, seed=2)
    assert placed == 20 and set(np.unique(C[..., 0])) <= {1.0, 10.0} and F0.max() <= 0.02


def test_cubic_matches_oracle(agb, oracle):
    from alamo_gb300 import synth
    rng = np.random.default_rng(3)
    for _ in range(4):
        R, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        assert np.array_equal(synth.cubic_stiffness(1.68, 1.21, 0.75, R), oracle.cubic(1.68, 1.21, 0.75, R))


def test_inclusion_config(agb):
    from alamo_gb300 import synth
    C, F0, dx = synth.inclusion_iso(33)
    x = np.arange(33) * dx
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    inside = np.sqrt((X - .5) ** 2 + (Y - .5) ** 2 + (Z - .5) ** 2) < 0.25
    assert np.array_equal(C[..., 0] == 10.0, inside) and np.array_equal(F0 == 0.01, inside)
