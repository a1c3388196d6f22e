"""The C++ plugins (include/gbompl_ompl.hpp) compiled against OMPL's own headers and objects. Needs
the OMPL source tree (it is not present on every machine); with a GPU the plugins are compared with
OMPL's DiscreteMotionValidator / NearestNeighborsLinear, without one the error path is checked."""
import glob
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("OMPL_SOURCE_TREE", "")  # the OMPL source tree; the tests skip without one


def test_plugins_compile_and_run_against_ompl(tmp_path):
    if not os.path.isdir(os.path.join(REF, "src", "ompl")):
        pytest.skip("OMPL source tree not available")
    lib = os.path.join(ROOT, "ompl_gb300", "libgbompl.so")
    if not os.path.exists(lib):
        pytest.skip("libgbompl.so not built")
    from oracle.oracle import build_reference
    build_reference(REF)
    objs = [o for o in glob.glob(os.path.join(ROOT, "oracle", "_ref", "obj", "*.o"))
            if not o.endswith(("ref_api.o",))]
    exe = str(tmp_path / "plugin_check")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-w", "-I", os.path.join(ROOT, "oracle", "ref", "shim"),
           "-I", os.path.join(REF, "src"), "-I", os.path.join(ROOT, "include"), "-include", "cstring", "-include",
           "vector", "-include", "array", os.path.join(ROOT, "tests", "cpp", "plugin_check.cpp"), *objs, lib,
           f"-Wl,-rpath,{os.path.dirname(lib)}", "-lpthread", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith(("MATCH", "NO_DEVICE")), r.stdout


def test_metric_guard_rejects_a_foreign_distance_function(tmp_path):
    """GpuNearestNeighbors' distance function check (gbompl::MetricGuard), which needs no device."""
    if not os.path.isdir(os.path.join(REF, "src", "ompl")):
        pytest.skip("OMPL source tree not available")
    lib = os.path.join(ROOT, "ompl_gb300", "libgbompl.so")
    if not os.path.exists(lib):
        pytest.skip("libgbompl.so not built")
    from oracle.oracle import build_reference
    build_reference(REF)
    objs = [o for o in glob.glob(os.path.join(ROOT, "oracle", "_ref", "obj", "*.o"))
            if not o.endswith(("ref_api.o",))]
    exe = str(tmp_path / "metric_check")
    cmd = ["g++", "-std=c++17", "-O2", "-w", "-I", os.path.join(ROOT, "oracle", "ref", "shim"),
           "-I", os.path.join(REF, "src"), "-I", os.path.join(ROOT, "include"), "-include", "cstring", "-include",
           "vector", "-include", "array", os.path.join(ROOT, "tests", "cpp", "metric_check.cpp"), *objs, lib,
           f"-Wl,-rpath,{os.path.dirname(lib)}", "-lpthread", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
