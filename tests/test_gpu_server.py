"""Continuous batching: requests solved concurrently by the server give the same results as the
same requests solved alone (bitwise: each request runs its own deterministic kernels)."""
import numpy as np
import pytest

from spheresimulator_gb300 import PREC_MIXED, SolveServer, SphereSTKMobMat, configs

pytestmark = pytest.mark.gpu


def test_server_results_equal_solo_solves():
    rng = np.random.default_rng(3)
    reqs = []
    for k, (n, p) in enumerate([(3, 6), (12, 8), (5, 10), (30, 6), (2, 12), (8, 8)]):
        r = configs.small_cluster(seed=40 + k, n=n, p=p, gap=0.08, quats=bool(k % 2))
        r["tol"] = 1e-8 if k % 2 else 1e-6
        reqs.append(r)
    with SolveServer(max_slots=4, precision=PREC_MIXED) as srv:
        ids = [srv.submit(r["centers"], r["radii"], r["orders"], r["force"], tol=r["tol"], quats=r["quats"])
               for r in reqs]
        out = [srv.wait(i, timeout=600) for i in ids]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["peak_running"] >= 2
    for r, (vel, info) in zip(reqs, out):
        assert info["status"] == 0 and info["t_submit"] <= info["t_admit"] <= info["t_done"]
        assert info["stats"]["relres"] < r["tol"]
        solo = SphereSTKMobMat(r["centers"], r["radii"], r["orders"], quats=r["quats"])
        v = solo.solveMob(r["force"], tol=r["tol"], restart=50, max_iters=2000, precision=PREC_MIXED)
        assert np.array_equal(vel, v)


def test_concurrent_first_use_of_an_order():
    """Four requests of one order that no earlier context used (p = 13) start together, so the
    workers build that order's host tables and near maps concurrently; every result equals its solo
    solve bit for bit."""
    reqs = [configs.small_cluster(seed=70 + k, n=5, p=13, gap=0.15, quats=True) for k in range(4)]
    with SolveServer(max_slots=4, precision=PREC_MIXED) as srv:
        ids = [srv.submit(r["centers"], r["radii"], r["orders"], r["force"], tol=1e-8, quats=r["quats"])
               for r in reqs]
        out = [srv.wait(i, timeout=600) for i in ids]
    for r, (vel, info) in zip(reqs, out):
        assert info["status"] == 0
        solo = SphereSTKMobMat(r["centers"], r["radii"], r["orders"], quats=r["quats"])
        assert np.array_equal(vel, solo.solveMob(r["force"], tol=1e-8, restart=50, max_iters=2000,
                                                  precision=PREC_MIXED))


def test_server_admission_respects_budget():
    """With a budget that fits one request at a time, requests run one after another."""
    from spheresimulator_gb300 import request_bytes
    reqs = [configs.small_cluster(seed=60 + k, n=6, p=8, gap=0.2) for k in range(3)]
    budget = 1.5 * request_bytes(reqs[0]["orders"])
    with SolveServer(max_slots=3, hbm_budget_bytes=budget, precision=PREC_MIXED) as srv:
        ids = [srv.submit(r["centers"], r["radii"], r["orders"], r["force"]) for r in reqs]
        infos = [srv.wait(i, timeout=600)[1] for i in ids]
        st = srv.stats()
    assert st["peak_running"] == 1 and st["peak_bytes"] <= budget
    spans = sorted((x["t_admit"], x["t_done"]) for x in infos)
    for (a0, d0), (a1, d1) in zip(spans, spans[1:]):
        assert a1 >= d0 - 1e-3


def test_partitioned_server_results_equal_solo_solves():
    """With the SMs split into green contexts (small requests on a reserved partition while a big one
    runs, big requests on the rest), every result still equals its solo solve bit for bit (the kernels
    are deterministic on any number of SMs), the partition has the requested size rounded to the
    device's granularity, and the server cannot be re-partitioned while it has work."""
    big = configs.cfg2()  # 36,992 points: above the 1e9-pair line of a small request
    smalls = [configs.small_cluster(seed=80 + k, n=n, p=8, gap=0.1, quats=True) for k, n in enumerate((4, 9, 6))]
    with SolveServer(max_slots=4, precision=PREC_MIXED, small_sms=12) as srv:
        a, b = srv.partition_info()
        assert a == 16 and a + b <= 152 and b >= 128  # 12 rounded up to the 8-SM granularity
        ids = [srv.submit(big["centers"], big["radii"], big["orders"], big["force"], tol=1e-8)]
        ids += [srv.submit(r["centers"], r["radii"], r["orders"], r["force"], tol=1e-8, quats=r["quats"])
                for r in smalls]
        from spheresimulator_gb300 import SmobError
        with pytest.raises(SmobError):
            srv.partition(0)  # requests are queued or running
        out = [srv.wait(i, timeout=600) for i in ids]
    for r, (vel, info) in zip([big] + smalls, out):
        assert info["status"] == 0
        solo = SphereSTKMobMat(r["centers"], r["radii"], r["orders"], quats=r.get("quats"))
        assert np.array_equal(vel, solo.solveMob(r["force"], tol=1e-8, restart=50, max_iters=2000,
                                                  precision=PREC_MIXED))
