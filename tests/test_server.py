"""Host logic of the serving loop (no device work): admission footprint, request validation,
budget rejection, and that a missing GPU surfaces as an error instead of a CPU fallback."""
import numpy as np
import pytest

from spheresimulator_gb300 import SmobError, SolveServer, configs, request_bytes


def test_request_bytes_monotone():
    a = request_bytes([8] * 4)
    assert a > request_bytes([8] * 2) and request_bytes([16] * 4) > a
    assert request_bytes([8] * 4, restart=100) > request_bytes([8] * 4, restart=10)
    # the largest cfg5 request (2048 spheres, p = 24) fits a GB300 many times over
    assert 1e9 < request_bytes([24] * 2048) < 20e9


def test_submit_validation_and_budget():
    srv = SolveServer(max_slots=1, hbm_budget_bytes=1e6)
    c = configs.cfg1()
    with pytest.raises(SmobError) as e:
        srv.submit(c["centers"], c["radii"], c["orders"], c["force"], tol=1e-8)  # ~9 MB > 1 MB budget
    assert e.value.code == 3
    with pytest.raises(SmobError):
        srv.submit(c["centers"], c["radii"], c["orders"], c["force"], tol=-1.0)
    srv.close()


def test_no_gpu_is_an_error_not_a_fallback():
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    srv = SolveServer(max_slots=2)
    c = configs.cfg1()
    rid = srv.submit(c["centers"], c["radii"], c["orders"], c["force"], tol=1e-8)
    with pytest.raises(SmobError) as e:
        srv.wait(rid, timeout=60)
    assert e.value.code == 7
    st = srv.stats()
    assert st["completed"] == 1 and st["running"] == 0 and st["bytes_in_use"] == 0
    srv.close()


def test_cfg5_stream_properties():
    s = configs.cfg5_stream(seed=5, n_requests=40, rate=2.0)
    t = np.array([r["arrival"] for r in s])
    assert np.all(np.diff(t) > 0)
    n = np.array([len(r["radii"]) for r in s])
    assert n.min() >= 4 and n.max() <= 2048
    assert {int(r["orders"][0]) for r in s} <= {8, 12, 16, 24}
    assert {r["tol"] for r in s} == {1e-6, 1e-8}
    for r in s[:8]:
        c, a = r["centers"], r["radii"]
        d = np.linalg.norm(c[:, None] - c[None], axis=2) - a[:, None] - a[None]
        np.fill_diagonal(d, 1e9)
        assert d.min() >= 0.05 - 1e-12
