"""The C-ABI library loads and exports every entry point include/hexopt_gpu.h declares; host-only
entry points (aabb.h value types, argument validation without a device) behave.  No GPU needed."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    import build as b
    b.build()
    from hexopt import _lib
    return _lib


def header_functions():
    s = open(os.path.join(ROOT, "include", "hexopt_gpu.h")).read()
    s = re.sub(r"/\*.*?\*/", "", s, flags=re.S)
    return set(re.findall(r"\b(hexopt_[a-z_0-9]+)\s*\(", s))


def test_every_declared_symbol_is_exported(lib):
    out = subprocess.run(["nm", "-D", lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    declared = header_functions()
    assert declared, "no declarations parsed"
    assert declared <= exported, f"declared but not exported: {sorted(declared - exported)}"
    assert {e for e in exported if not e.startswith("hexopt_")} == set(), "library exports non-ABI symbols"


def test_binding_covers_the_header(lib):
    assert header_functions() == set(lib.SIGNATURES)
    L = lib.load()
    for name in lib.SIGNATURES:
        assert getattr(L, name) is not None


def test_aabb_value_types(lib):
    L = lib.load()
    a = lib.AABB((0, 0, 0), (1, 2, 3))
    b = lib.AABB((-1, 0.5, 0), (0.5, 1, 4))
    assert L.hexopt_aabb_largest_axis(C.byref(a)) == 2
    assert L.hexopt_aabb_surface_area(C.byref(a)) == pytest.approx(2 * (2 + 6 + 3))
    p = (C.c_double * 3)(2, 1, -1)
    assert L.hexopt_aabb_squared_distance(C.byref(a), p) == pytest.approx(1 + 0 + 1)
    L.hexopt_aabb_merge(C.byref(a), C.byref(b))
    assert list(a.min) == [-1, 0, 0] and list(a.max) == [1, 2, 4]
    r = lib.Ray((-5, 0.5, 0.5), (1, 0, 0), (1, float("inf"), float("inf")), 0.0, 1e30)
    n, f = C.c_double(), C.c_double()
    assert L.hexopt_aabb_ray_intersect(C.byref(a), C.byref(r), C.byref(n), C.byref(f)) == 1
    assert (n.value, f.value) == (4.0, 6.0)
    r2 = lib.Ray((-5, 5.5, 0.5), (1, 0, 0), (1, float("inf"), float("inf")), 0.0, 1e30)
    assert L.hexopt_aabb_ray_intersect(C.byref(a), C.byref(r2), None, None) == 0


def test_create_without_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    L = lib.load()
    h = C.c_void_p()
    assert L.hexopt_create(C.byref(h), 0) != 0
    assert not h.value
