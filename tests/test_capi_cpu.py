"""C-ABI library checks that need no GPU: it loads, exports every declared entry point, and validates
arguments with OMPL's error behaviour before touching a device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "ompl_gb300", "libgbompl.so")
HDR = os.path.join(ROOT, "include", "gbompl.h")


def declared():
    txt = open(HDR).read()
    return sorted(set(re.findall(r"^\s*(?:gbo_status|const char \*|uint64_t)\s*(gbo_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        pytest.skip("libgbompl.so not built")
    from ompl_gb300 import capi
    return capi.lib()


def test_header_declares_entry_points():
    names = declared()
    assert "gbo_check_motion" in names and "gbo_nn_nearest_k" in names and len(names) >= 30


def test_every_declared_symbol_is_exported(lib):
    for name in declared():
        assert hasattr(lib, name), name


def test_signature_table_matches_header(lib):
    from ompl_gb300 import capi
    assert sorted(capi.SIGNATURES) == declared()


def test_space_argument_errors_match_ompl(lib):
    from ompl_gb300 import capi
    h = C.c_void_p()
    lo = np.zeros(2)
    hi = np.ones(2)
    dp = C.POINTER(C.c_double)
    # StateSpace::setLongestValidSegmentFraction rejects fractions outside (eps, 1-eps) (StateSpace.cpp:828-834)
    assert lib.gbo_space_create(0, 2, lo.ctypes.data_as(dp), hi.ctypes.data_as(dp), 0.0, -1.0, 0.0, 1,
                                C.byref(h)) == capi.ERR_INVALID_ARGUMENT
    assert b"fraction" in lib.gbo_last_error()
    # setValidSegmentCountFactor(0) throws (StateSpace.cpp:820-826)
    assert lib.gbo_space_create(0, 2, lo.ctypes.data_as(dp), hi.ctypes.data_as(dp), 0.0, -1.0, 0.01, 0,
                                C.byref(h)) == capi.ERR_INVALID_ARGUMENT
    assert lib.gbo_space_create(1, 2, None, None, 0.0, -1.0, 0.01, 1, C.byref(h)) == capi.ERR_INVALID_ARGUMENT
    assert lib.gbo_space_create(0, 17, lo.ctypes.data_as(dp), hi.ctypes.data_as(dp), 0.0, -1.0, 0.01, 1,
                                C.byref(h)) == capi.ERR_UNSUPPORTED
    # a valid space needs no device: extent and segment length as StateSpace::setup computes them
    assert lib.gbo_space_create(0, 2, lo.ctypes.data_as(dp), hi.ctypes.data_as(dp), 0.0, -1.0, 0.01, 1,
                                C.byref(h)) == capi.OK
    e, l_ = C.c_double(), C.c_double()
    assert lib.gbo_space_info(h, C.byref(e), C.byref(l_)) == capi.OK
    assert e.value == np.sqrt(2.0) and l_.value == np.sqrt(2.0) * 0.01
    lib.gbo_space_destroy(h)


def test_space_extent_and_lvs_match_oracle(lib, port):
    from oracle.oracle import SpaceDesc
    from ompl_gb300 import capi
    dp = C.POINTER(C.c_double)
    for kind, dim, link in ((0, 7, 0.0), (1, 1, 0.0), (2, 10, 0.1), (3, 7, 0.0)):
        lo = np.linspace(-3, -1, dim)
        hi = np.linspace(1, 4, dim)
        h = C.c_void_p()
        assert lib.gbo_space_create(kind, dim, lo.ctypes.data_as(dp), hi.ctypes.data_as(dp), link, -1.0, 0.003, 1,
                                    C.byref(h)) == capi.OK
        e, l_ = C.c_double(), C.c_double()
        lib.gbo_space_info(h, C.byref(e), C.byref(l_))
        sp = SpaceDesc(kind, dim, lo, hi, link, 0.003, 1)
        assert e.value == port.extent(sp) and l_.value == port.lvs(sp)
        lib.gbo_space_destroy(h)


def test_device_calls_fail_cleanly_without_gpu(lib):
    from ompl_gb300 import capi
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    sm = C.c_int()
    assert lib.gbo_device_check(C.byref(sm), None, None) == capi.ERR_NO_DEVICE
    h = C.c_void_p()
    lo = np.zeros(2)
    hi = np.ones(2)
    dp = C.POINTER(C.c_double)
    lib.gbo_space_create(0, 2, lo.ctypes.data_as(dp), hi.ctypes.data_as(dp), 0.0, -1.0, 0.01, 1, C.byref(h))
    ck = C.c_void_p()
    w = np.zeros((1, 3))
    assert lib.gbo_checker_create(h, 1, w.ctypes.data_as(dp), 1, None, 0, 0, 0.0, C.byref(ck)) == capi.ERR_NO_DEVICE
    lib.gbo_space_destroy(h)


def test_bounded_wait_selftest_rejects_bad_limits():
    import ctypes as C
    from ompl_gb300 import capi
    lib = capi.lib()
    el = C.c_double()
    assert lib.gbo_selftest_bounded_wait(0, C.byref(el)) == capi.ERR_INVALID_ARGUMENT
    assert lib.gbo_selftest_bounded_wait(3_000_000_000, C.byref(el)) == capi.ERR_INVALID_ARGUMENT
