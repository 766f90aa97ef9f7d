"""The drop-in C++ shim (shim/hexopt_reference_shim.cpp: the reference's own entry-point
signatures over the C ABI) against the reference's headers and callers.

It has to compile with the reference's own headers, and the reference's callers of those entry
points (optimization.cpp, global_functions.cpp, global_types.cpp) have to link against it --
with the shim in place of slim_m.cpp and metro_hausdorff.cpp and the CPU scaled_jacobian made
local, as a maintainer removing it would -- leaving no symbol unresolved that the CPU build
resolves.  A shim whose signature drifts leaves the callers' reference unresolved, which the
negative case shows.  Needs the reference tree (and its objects from oracle/Makefile's `ref`
target); skipped where it is absent.  Nothing here runs GPU code.
"""
import os
import shutil
import subprocess

import pytest

from conftest import PKG, ROOT

def _ref_tree():
    """The reference tree oracle/Makefile reads (its REF: $HEXOPT_REFERENCE_TREE or its default)."""
    try:
        r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "print-ref"], capture_output=True,
                           text=True, timeout=60)
        return r.stdout.strip()
    except (OSError, subprocess.SubprocessError):
        return ""


REF = _ref_tree()
OBJ = os.path.join(ROOT, "oracle", "_ref")
SHIM = os.path.join(PKG, "shim", "hexopt_reference_shim.cpp")
CPU_SJ = "_Z15scaled_jacobianR4MeshR12Mesh_Quality"

pytestmark = pytest.mark.skipif(not REF or not os.path.isdir(REF) or shutil.which("g++") is None
                                or shutil.which("objcopy") is None,
                                reason="reference tree or host toolchain absent")


def _inc():
    ext = os.path.join(REF, "extern")
    return [f"-I{REF}", f"-I{ext}/eigen", f"-I{ext}/libigl/include", f"-I{ext}/geogram/src/lib",
            f"-I{ext}/tbb/include", f"-I{ext}/vcg", f"-I{ext}/libigl/external/embree/include",
            f"-I{os.path.join(ROOT, 'include')}", f"-I{os.path.join(PKG, 'shim')}"]


def _compile(out, extra=()):
    cmd = ["g++", "-std=c++14", "-O1", "-w", "-fopenmp", "-DNOMINMAX", "-ffp-contract=off", "-fPIC",
           "-DHEXOPT_SHIM_SCALED_JACOBIAN", *extra, *_inc(), "-c", SHIM, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def _unresolved(objs, libs=()):
    r = subprocess.run(["g++", "-shared", "-fopenmp", "-Wl,--no-undefined", "-o", os.devnull, *objs, *libs],
                       capture_output=True, text=True)
    return {line.split("undefined reference to", 1)[1].strip() for line in r.stderr.splitlines()
            if "undefined reference to" in line}


@pytest.fixture(scope="module")
def objs(tmp_path_factory):
    need = ["slim_m", "metro_hausdorff", "optimization", "global_types", "global_functions", "geo_stub"]
    if not all(os.path.exists(os.path.join(OBJ, n + ".o")) for n in need):
        subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
    import build
    lib = build.build()
    d = tmp_path_factory.mktemp("shim")
    gf = str(d / "global_functions_local.o")
    subprocess.run(["objcopy", f"--localize-symbol={CPU_SJ}", os.path.join(OBJ, "global_functions.o"), gf], check=True)
    o = {n: os.path.join(OBJ, n + ".o") for n in need}
    o["gf_local"] = gf
    o["dir"] = d
    o["lib"] = [f"-L{os.path.dirname(lib)}", "-lhexopt_gpu"]
    return o


def test_shim_defines_the_reference_entry_points(objs):
    out = str(objs["dir"] / "shim.o")
    _compile(out)
    r = subprocess.run(["nm", "-C", "--defined-only", out], capture_output=True, text=True, check=True)
    want = ["slim_precompute(Eigen::Matrix<double, -1, -1, 0, -1, -1>&, Eigen::Matrix<int, -1, -1, 0, -1, -1>&, "
            "Eigen::Matrix<double, -1, -1, 0, -1, -1>&, SLIMData&, SLIM_ENERGY, Tetralize_Set)",
            "slim_solve2(SLIMData&, int, int, bool)", "slim_solve(SLIMData&, int, int, bool)",
            "compute(Mesh&, Mesh&, double&, double&)", "compute(Mesh&, Mesh&, double&, double&, double&)",
            "compute(Mesh const&, Mesh const&, double&, double&, double&)",
            "scaled_jacobian(Mesh&, Mesh_Quality&)"]
    for w in want:
        assert w in r.stdout, w


def test_reference_callers_link_against_the_shim(objs):
    shim = str(objs["dir"] / "shim.o")
    if not os.path.exists(shim):
        _compile(shim)
    common = [objs["optimization"], objs["global_types"], objs["geo_stub"]]
    cpu = _unresolved([objs["slim_m"], objs["metro_hausdorff"], objs["global_functions"], *common])
    gpu = _unresolved([shim, objs["gf_local"], *common], objs["lib"])
    # the CPU build's own leftovers are libraries outside these objects (io, tbb, embree)
    assert gpu <= cpu, sorted(gpu - cpu)


def test_signature_drift_is_caught(objs):
    bad = str(objs["dir"] / "shim_bad.o")
    _compile(bad, ["-Dslim_solve2=slim_solve2_renamed"])
    common = [objs["optimization"], objs["global_types"], objs["geo_stub"]]
    cpu = _unresolved([objs["slim_m"], objs["metro_hausdorff"], objs["global_functions"], *common])
    gpu = _unresolved([bad, objs["gf_local"], *common], objs["lib"])
    assert any("slim_solve2" in s for s in gpu - cpu)


def test_shim_compiles_with_slim_opt_igl(objs):
    """With HEXOPT_SHIM_SLIM_OPT_IGL the shim also defines optimization::slim_opt_igl (for a build
    that drops the CPU definition from optimization.cpp)."""
    out = str(objs["dir"] / "shim_igl.o")
    _compile(out, extra=["-DHEXOPT_SHIM_SLIM_OPT_IGL"])
    r = subprocess.run(["nm", "-C", "--defined-only", out], capture_output=True, text=True, check=True)
    assert "optimization::slim_opt_igl(Tetralize_Set&, unsigned int)" in r.stdout
