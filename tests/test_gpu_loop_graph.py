"""The graph-driven restart loop against the host-driven loop.

With the loop graph on, a solve's restart cycles run as one CUDA graph launch whose decisions (per
problem stop tests, the Arnoldi step sequence, the residual kind, the next cycle) are taken by device
kernels steering conditional graph nodes. The host-driven loop takes the same decisions on the host
(BIE/SphereSTKMobMat.cpp:209-241 is the Belos solve loop both replace). Both must give the same bits
and the same per-problem statistics, in every precision, for batches, several right-hand sides,
restarts, iteration limits, warm starts and the preconditioner; the graph-driven loop must issue far
fewer launches from the host.
"""
import os

import numpy as np
import pytest

from spheresimulator_gb300 import PREC_FLOAT_FLOAT, PREC_FP64, PREC_MIXED, SphereSTKMobMat, configs

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STAT_KEYS = ("status", "iterations", "refinements", "operator_passes_fp64", "operator_passes_fp32", "bnorm", "relres")


def make(cfg):
    return SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg.get("quats"),
                           problem=cfg.get("problem"))


def both_loops(mob, run):
    """run() with the loop graph (twice: built, then replayed) and with the host loop"""
    mob.set_loop_graph(True)
    a = run()
    sa = [dict(s) for s in mob.last_stats]
    assert mob.loop_graph_info() == (True, True)
    a2 = run()
    mob.set_loop_graph(False)
    b = run()
    sb = [dict(s) for s in mob.last_stats]
    return a, a2, sa, b, sb


def assert_same(a, a2, sa, b, sb):
    assert np.array_equal(a, b) and np.array_equal(a2, b)
    assert len(sa) == len(sb)
    for x, y in zip(sa, sb):
        for k in STAT_KEYS:
            assert x[k] == y[k], (k, x[k], y[k])


@pytest.mark.parametrize("prec", [PREC_MIXED, PREC_FP64, PREC_FLOAT_FLOAT])
def test_loop_graph_matches_host_loop(prec):
    cfg = configs.small_cluster(seed=31, n=6, p=8, gap=0.2, quats=True)
    mob = make(cfg)
    assert_same(*both_loops(mob, lambda: mob.solveMob(cfg["force"], tol=1e-10, precision=prec)))


def test_loop_graph_uneven_batch():
    g = dict(np.load(os.path.join(GOLDEN, "golden_batch6.npz")))
    mob = make(g)
    assert mob.n_problems == 6
    assert_same(*both_loops(mob, lambda: mob.solveMob(g["force"], tol=1e-8, restart=50, max_iters=2000,
                                                       precision=PREC_MIXED)))


def test_loop_graph_restarts_and_iteration_limit():
    cfg = configs.small_cluster(seed=32, n=8, p=8, gap=0.15, quats=True)
    mob = make(cfg)
    # restart 4: many cycles, the last step index of a cycle reached every time
    assert_same(*both_loops(mob, lambda: mob.solveMob(cfg["force"], tol=1e-10, restart=4, max_iters=500,
                                                       precision=PREC_FP64)))
    assert mob.last_stats[0]["refinements"] > 3
    # an iteration limit inside a cycle: the problem stops unconverged in both loops
    run = lambda: mob.solveMob(cfg["force"], tol=1e-13, restart=30, max_iters=7, precision=PREC_MIXED,
                               raise_on_not_converged=False)
    a, a2, sa, b, sb = both_loops(mob, run)
    assert_same(a, a2, sa, b, sb)
    assert sa[0]["iterations"] == 7 and sa[0]["status"] != 0


def test_loop_graph_preconditioned_warm_and_several_columns():
    cfg = configs.small_cluster(seed=33, n=6, p=8, gap=0.2, quats=True)
    mob = make(cfg)
    assert_same(*both_loops(mob, lambda: mob.solveMob(cfg["force"], tol=1e-10, precision=PREC_MIXED, precond=1)))
    f2 = np.random.default_rng(3).standard_normal(cfg["force"].shape)

    def warm():  # a cold solve sets the previous solution, the next one starts from it
        mob.solveMob(cfg["force"], tol=1e-10, precision=PREC_MIXED)
        return mob.solveMob(f2, tol=1e-10, precision=PREC_MIXED, warm_start=True)
    assert_same(*both_loops(mob, warm))
    cols = np.stack([cfg["force"], f2, cfg["force"] - 0.5 * f2])
    mob.set_loop_graph(True)
    a = mob.solveMobMulti(cols, tol=1e-10, precision=PREC_MIXED)
    mob.set_loop_graph(False)
    b = mob.solveMobMulti(cols, tol=1e-10, precision=PREC_MIXED)
    assert np.array_equal(a, b)


def test_loop_graph_cuts_host_launches():
    cfg = configs.small_cluster(seed=34, n=12, p=8, gap=0.2, quats=True)
    mob = make(cfg)
    counts = {}
    for on in (True, False):
        mob.set_loop_graph(on)
        mob.solveMob(cfg["force"], tol=1e-8, precision=PREC_MIXED)  # builds the graphs
        k0, h0 = mob.launch_stats()
        mob.solveMob(cfg["force"], tol=1e-8, precision=PREC_MIXED)
        k1, h1 = mob.launch_stats()
        counts[on] = (k1 - k0, h1 - h0)
    kg, hg = counts[True]
    kh, hh = counts[False]
    # the device loop runs no more kernels (the host loop's blocks also run steps after the last stop);
    # from the host: the set-up and final-velocity kernels and one graph launch, against those plus a
    # graph launch per 4-step block and the cycle kernels
    assert 0 < kg <= kh
    assert hg * 2 < hh and hg <= 32, counts


def test_loop_graph_zero_and_mixed_batch_forces():
    """A problem with zero forcing is converged at once (zero density correction,
    BIE/SphereSTKMobMat.cpp:217) while its batch partner iterates: the device-side set-up takes the same
    decisions as the host's."""
    a = configs.small_cluster(seed=35, n=4, p=8, gap=0.2, quats=True)
    b = configs.small_cluster(seed=36, n=5, p=8, gap=0.2, quats=True)
    cfg = dict(centers=np.vstack([a["centers"], b["centers"] + 100.0]), radii=np.concatenate([a["radii"], b["radii"]]),
               orders=np.concatenate([a["orders"], b["orders"]]), quats=np.vstack([a["quats"], b["quats"]]),
               problem=np.array([0] * 4 + [1] * 5, dtype=np.int32))
    F = np.concatenate([np.zeros(24), b["force"]])
    mob = make(cfg)
    a_, a2, sa, b_, sb = both_loops(mob, lambda: mob.solveMob(F, tol=1e-10, precision=PREC_MIXED))
    assert_same(a_, a2, sa, b_, sb)
    assert sa[0]["iterations"] == 0 and sa[0]["status"] == 0 and np.all(a_[:24] == 0)
    assert sa[1]["iterations"] > 0 and sa[1]["status"] == 0


def test_loop_graph_non_finite_force_through_device_api():
    """Device-pointer forces are not screened on the host: a non-finite one stops its problem in the
    set-up (device-side decision in the graph) with SMOB_ERR_NONFINITE, its batch partner converges."""
    import ctypes

    from spheresimulator_gb300 import _native as N
    from spheresimulator_gb300 import solve_opts
    a = configs.small_cluster(seed=37, n=4, p=8, gap=0.2, quats=True)
    b = configs.small_cluster(seed=38, n=4, p=8, gap=0.2, quats=True)
    cfg = dict(centers=np.vstack([a["centers"], b["centers"] + 100.0]), radii=np.concatenate([a["radii"], b["radii"]]),
               orders=np.concatenate([a["orders"], b["orders"]]), quats=np.vstack([a["quats"], b["quats"]]),
               problem=np.array([0] * 4 + [1] * 4, dtype=np.int32))
    F = np.concatenate([a["force"], b["force"]])
    F[3] = np.nan
    mob = make(cfg)
    L, h = N.lib(), mob.handle
    d_f, d_v = ctypes.c_void_p(), ctypes.c_void_p()
    N.check(L.smob_device_alloc(h, 8 * 48, ctypes.byref(d_f)))
    N.check(L.smob_device_alloc(h, 8 * 48, ctypes.byref(d_v)))
    try:
        N.check(L.smob_memcpy_h2d(h, d_f, F.ctypes.data_as(ctypes.c_void_p), 8 * 48))
        out = {}
        for on in (True, False):
            mob.set_loop_graph(on)
            stats = (N.ProblemStats * 2)()
            o = solve_opts(1e-10, 50, 500, PREC_MIXED)
            code = L.smob_solve_mob_device(h, d_f, d_v, None, ctypes.byref(o), stats)
            out[on] = (code, [s.as_dict() for s in stats])
        assert out[True][0] == out[False][0] == N.SMOB_ERR_NONFINITE
        for x, y in zip(out[True][1], out[False][1]):
            assert x["status"] == y["status"] and x["iterations"] == y["iterations"]
        assert out[True][1][0]["status"] == N.SMOB_ERR_NONFINITE and out[True][1][1]["status"] == 0
    finally:
        L.smob_device_free(h, d_f)
        L.smob_device_free(h, d_v)
