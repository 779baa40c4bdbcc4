"""The C-ABI library builds for sm_103a, loads, exports every entry point declared in
include/*.h, and validates arguments on the host (no device compute here)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(smob_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from spheresimulator_gb300 import _native
    L = _native.lib()
    decl = declared_functions()
    assert len(decl) >= 25
    missing = [n for n in decl if not hasattr(L, n)]
    assert not missing, missing
    raw = ctypes.CDLL(_native.library_path())
    for n in decl:
        getattr(raw, n)


def test_library_is_sm103a():
    from spheresimulator_gb300 import _build
    assert "arch=compute_103a,code=sm_103a" in " ".join(_build.ARCH)
    assert os.path.exists(_build.build())


def test_argument_validation_on_host():
    from spheresimulator_gb300 import _native as N
    L = N.lib()
    h = ctypes.c_void_p()
    assert L.smob_create(ctypes.byref(h), None, 0) == N.SMOB_ERR_ARG
    c = np.zeros((1, 3))
    r = np.ones(1)
    o = np.full(1, 8, np.int32)
    geo = N.Geometry(0, N.dptr(c), N.dptr(r), None, N.iptr(o), None, 1.0)
    assert L.smob_create(ctypes.byref(h), ctypes.byref(geo), 0) == N.SMOB_ERR_ARG
    assert b"n_spheres" in L.smob_last_error()
    geo = N.Geometry(1, N.dptr(c), N.dptr(r), None, N.iptr(o), None, -1.0)
    assert L.smob_create(ctypes.byref(h), ctypes.byref(geo), 0) == N.SMOB_ERR_ARG
    assert L.smob_destroy(None) == N.SMOB_OK
    major, minor = ctypes.c_int(), ctypes.c_int()
    assert L.smob_version(ctypes.byref(major), ctypes.byref(minor)) == N.SMOB_OK


def test_no_device_is_reported_not_faked():
    """Without a GPU the library refuses to run instead of falling back to the CPU."""
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    from spheresimulator_gb300 import SphereSTKSHOperator, SmobError
    with pytest.raises(SmobError) as e:
        SphereSTKSHOperator([[0, 0, 0]], [1.0], [8])
    assert e.value.code == 7


def test_structures_match_header():
    """ctypes mirrors of smob_geometry / smob_solve_opts / smob_problem_stats have the C layout."""
    from spheresimulator_gb300 import _native as N
    assert ctypes.sizeof(N.Geometry) == 56
    assert ctypes.sizeof(N.SolveOpts) == 40
    assert ctypes.sizeof(N.ProblemStats) == 40
    assert ctypes.sizeof(N.ServerOpts) == 48  # ... inner_tol, graphs (+4 padding)
    assert ctypes.sizeof(N.RequestInfo) == 96  # ... stats, t_ctx, route (+4 padding)


def test_warm_start_codes():
    """warm_start maps to smob_warm_start: False 0, True 1 (previous solution), "recycle" 2."""
    from spheresimulator_gb300 import WARM_LAST, WARM_NONE, WARM_RECYCLE, solve_opts
    assert (WARM_NONE, WARM_LAST, WARM_RECYCLE) == (0, 1, 2)
    assert solve_opts(warm_start=False).warm_start == 0
    assert solve_opts(warm_start=True).warm_start == 1
    assert solve_opts(warm_start="recycle").warm_start == 2
    with pytest.raises(ValueError):
        solve_opts(warm_start="sometimes")
    hdr = open(os.path.join(ROOT, "include", "smob.h")).read()
    for name, v in (("SMOB_WARM_NONE", 0), ("SMOB_WARM_LAST", 1), ("SMOB_WARM_RECYCLE", 2)):
        assert re.search(r"%s\s*=\s*%d" % (name, v), hdr)
    from spheresimulator_gb300 import _native as N
    L = N.lib()
    k = ctypes.c_int()
    assert L.smob_recycle_info(None, ctypes.byref(k), None) == N.SMOB_ERR_ARG
    assert L.smob_recycle_clear(None) == N.SMOB_ERR_ARG


def test_warm_orders_is_host_only():
    """smob_warm_orders builds the per-order host tables without a device and checks its orders."""
    from spheresimulator_gb300 import SmobError, warm_orders
    warm_orders([8, 12])
    warm_orders([])
    with pytest.raises(SmobError):
        warm_orders([33])


def test_server_options_are_checked_on_host():
    """smob_server_create rejects bad options before it touches a device."""
    from spheresimulator_gb300 import _native as N
    L = N.lib()
    srv = ctypes.c_void_p()
    assert L.smob_server_create(ctypes.byref(srv), None) == N.SMOB_ERR_ARG
    o = N.ServerOpts(device=0, max_slots=2, hbm_budget_bytes=0.0, restart=50, max_iters=200, precision=0,
                     inner_tol=0.0, graphs=3)
    assert L.smob_server_create(ctypes.byref(srv), ctypes.byref(o)) == N.SMOB_ERR_ARG
    assert b"graphs" in L.smob_last_error()
    o.graphs, o.max_slots = 0, 0
    assert L.smob_server_create(ctypes.byref(srv), ctypes.byref(o)) == N.SMOB_ERR_ARG
    assert not srv.value
