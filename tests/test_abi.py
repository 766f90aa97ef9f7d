"""The C-ABI library loads and exports every entry point include/hexopt_gpu.h declares; host-only
entry points (aabb.h value types, argument validation without a device) behave.  No GPU needed."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
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


def test_hex_mesh_files_round_trip(tmp_path):
    """MEDIT .mesh written as the reference writes it (6 significant digits, 1-based ids) reads
    back; the .vtk carries the hexes as VTK_HEXAHEDRON cells and the boundary flags."""
    import hexopt
    from hexopt import meshgen
    V, H = meshgen.grid_hex(3, 2, 2, hi=(1.5, 1.0, 0.5))
    b = meshgen.grid_boundary_mask(3, 2, 2)
    p = str(tmp_path / "m.mesh")
    hexopt.write_hex_mesh(p, V, H)
    V2, H2 = hexopt.read_hex_mesh(p)
    assert np.array_equal(H2, H)
    np.testing.assert_allclose(V2, V, rtol=1e-6)
    txt = open(p).read().split("\n")
    assert txt[0] == "MeshVersionFormatted 1" and txt[2] == f"Vertices {len(V)}" and txt[-1] == "End"
    q = str(tmp_path / "m.vtk")
    hexopt.write_hex_mesh(q, V, H, fmt="vtk", boundary=b)
    t = open(q).read()
    assert f"CELLS {len(H)} {9 * len(H)}" in t and t.count("\n12\n") + t.count("\n12") >= len(H)
    pd = t.split("LOOKUP_TABLE default\n")[1].split()
    assert [int(x) for x in pd] == b.astype(int).tolist()
