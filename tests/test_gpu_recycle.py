"""Recycled solutions (warm_start="recycle"): a sequence of mobility solves on one geometry, as the
collision solver issues them (the reference keeps its Krylov solver between solves for this,
BIE/SphereSTKMobMat.cpp:232). Each solve starts from the combination of earlier solutions that fits
its force best (exact for a force in their span); results equal cold solves to the tolerance."""
import numpy as np
import pytest

from spheresimulator_gb300 import PREC_FP64, PREC_MIXED, SmobError, SphereSTKMobMat, configs

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _mob(seed=5, n=6, p=8, **kw):
    cfg = configs.small_cluster(seed=seed, n=n, p=p, gap=0.1, quats=True, **kw)
    return cfg, SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg["quats"])


def test_repeated_force_starts_converged_fp64():
    cfg, g = _mob()
    assert g.recycle_info() == (0, 16)
    v1 = g.solveMob(cfg["force"], tol=1e-10, precision=PREC_FP64, warm_start="recycle")
    it1 = g.last_stats[0]["iterations"]
    assert g.recycle_info()[0] == 1 and it1 > 5
    v2 = g.solveMob(cfg["force"], tol=1e-10, precision=PREC_FP64, warm_start="recycle")
    assert g.last_stats[0]["iterations"] == 0
    assert g.last_stats[0]["relres"] < 1e-10
    assert _rel(v2, v1) < 1e-12
    # the repeated right-hand side adds no new column
    assert g.recycle_info()[0] == 1


def test_linear_combination_of_earlier_forces_fp64():
    cfg, g = _mob(seed=6)
    rng = np.random.default_rng(1)
    F1, F2 = cfg["force"], rng.standard_normal(cfg["force"].shape)
    v1 = g.solveMob(F1, tol=1e-11, precision=PREC_FP64, warm_start="recycle")
    v2 = g.solveMob(F2, tol=1e-11, precision=PREC_FP64, warm_start="recycle")
    v3 = g.solveMob(0.3 * F1 - 1.7 * F2, tol=1e-10, precision=PREC_FP64, warm_start="recycle")
    assert g.last_stats[0]["iterations"] == 0
    assert _rel(v3, 0.3 * v1 - 1.7 * v2) < 1e-9


def _contact_forces(centers, n_contacts, n_solves, seed):
    """Forces of a collision solver's iterations on one configuration: F = D gamma, the columns of D
    equal and opposite unit forces along the centre line of the n_contacts closest sphere pairs,
    gamma >= 0 changing every iteration."""
    c = np.asarray(centers)
    n = len(c)
    d = np.linalg.norm(c[:, None] - c[None], axis=-1) + np.eye(n) * 1e9
    pairs = sorted(((d[i, j], i, j) for i in range(n) for j in range(i + 1, n)))[:n_contacts]
    D = np.zeros((6 * n, n_contacts))
    for k, (_, i, j) in enumerate(pairs):
        e = (c[j] - c[i]) / np.linalg.norm(c[j] - c[i])
        D[6 * i:6 * i + 3, k] = -e
        D[6 * j:6 * j + 3, k] = e
    g = np.random.default_rng(seed).uniform(0.0, 1.0, (n_solves, n_contacts))
    return [D @ gk for gk in g]


def test_mixed_contact_sequence_equals_cold_solves_with_fewer_iterations():
    """Once the forces of earlier solves span the contact directions, each new solve starts close to
    its solution: far fewer iterations than cold solves, the same results to the tolerance."""
    cfg, g = _mob(seed=7, n=8)
    cold = SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg["quats"])
    it_rec, it_cold = [], []
    for F in _contact_forces(cfg["centers"], 4, 10, seed=2):
        v = g.solveMob(F, tol=1e-10, precision=PREC_MIXED, warm_start="recycle")
        st = g.last_stats[0]
        assert st["status"] == 0 and st["relres"] < 1e-10
        it_rec.append(st["iterations"])
        vc = cold.solveMob(F, tol=1e-10, precision=PREC_MIXED)
        it_cold.append(cold.last_stats[0]["iterations"])
        assert _rel(v, vc) < 1e-8
    assert g.recycle_info()[0] == 4
    assert sum(it_rec[4:]) < 0.4 * sum(it_cold[4:])


def test_fp64_contact_sequence_starts_at_the_tolerance():
    cfg, g = _mob(seed=14, n=8)
    its = []
    for k, F in enumerate(_contact_forces(cfg["centers"], 3, 7, seed=3)):
        v = g.solveMob(F, tol=1e-10, precision=PREC_FP64, warm_start="recycle")
        its.append(g.last_stats[0]["iterations"])
    # the combination of the earlier solutions' residuals (each below the tolerance) is left
    assert max(its[3:]) <= 5 and max(its[3:]) < min(its[:3]) // 3
    fresh = SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg["quats"])
    assert _rel(v, fresh.solveMob(F, tol=1e-10, precision=PREC_FP64)) < 1e-8


def test_drifting_forces_equal_cold_solves():
    """Forces with a new random part every solve: the recycled start is no worse than the previous
    solution's, and the results equal cold solves."""
    cfg, g = _mob(seed=15, n=6)
    cold = SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg["quats"])
    rng = np.random.default_rng(5)
    F = cfg["force"].copy()
    for k in range(4):
        F = F + 0.05 * np.linalg.norm(F) / np.sqrt(F.size) * rng.standard_normal(F.shape)
        v = g.solveMob(F, tol=1e-10, precision=PREC_MIXED, warm_start="recycle")
        assert _rel(v, cold.solveMob(F, tol=1e-10, precision=PREC_MIXED)) < 1e-8
    assert g.recycle_info()[0] == 4


def test_mixed_force_in_the_span_needs_no_high_precision_pass():
    """A repeated force and a combination of earlier forces: the combined residual and single layer
    of the stored MIXED states stand in for the float-float pass."""
    cfg, g = _mob(seed=8)
    rng = np.random.default_rng(6)
    F1, F2 = cfg["force"], rng.standard_normal(cfg["force"].shape)
    v1 = g.solveMob(F1, tol=1e-8, precision=PREC_MIXED, warm_start="recycle")
    s1 = g.last_stats[0]
    assert s1["operator_passes_fp64"] >= 1
    v2 = g.solveMob(F1, tol=1e-8, precision=PREC_MIXED, warm_start="recycle")
    s2 = g.last_stats[0]
    assert s2["status"] == 0 and s2["relres"] < 1e-8 and s2["iterations"] == 0
    assert s2["operator_passes_fp64"] == 0
    assert _rel(v2, v1) < 1e-12
    w2 = g.solveMob(F2, tol=1e-8, precision=PREC_MIXED, warm_start="recycle")
    F3 = 0.6 * F1 + 1.3 * F2
    v3 = g.solveMob(F3, tol=1e-8, precision=PREC_MIXED, warm_start="recycle")
    s3 = g.last_stats[0]
    assert s3["status"] == 0 and s3["relres"] < 1e-8 and s3["operator_passes_fp64"] == 0
    assert s3["iterations"] <= 6
    cold = SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg["quats"])
    ref = cold.solveMob(F3, tol=1e-11, precision=PREC_FP64)
    assert _rel(v3, ref) < 1e-7 and _rel(v3, 0.6 * v1 + 1.3 * w2) < 1e-7


def test_geometry_update_empties_the_space():
    cfg, g = _mob(seed=9)
    g.solveMob(cfg["force"], tol=1e-10, precision=PREC_FP64, warm_start="recycle")
    assert g.recycle_info()[0] == 1
    c2 = cfg["centers"] + 0.01
    g.set_geometry(c2)
    assert g.recycle_info()[0] == 0
    v = g.solveMob(cfg["force"], tol=1e-10, precision=PREC_FP64, warm_start="recycle")
    fresh = SphereSTKMobMat(c2, cfg["radii"], cfg["orders"], quats=cfg["quats"])
    assert _rel(v, fresh.solveMob(cfg["force"], tol=1e-10, precision=PREC_FP64)) < 1e-8
    g.recycle_clear()
    assert g.recycle_info()[0] == 0
    # the previous solution is forgotten as well: a warm start from it is a cold solve
    g.solveMob(cfg["force"], tol=1e-10, precision=PREC_FP64, warm_start=True)
    assert g.last_stats[0]["iterations"] == fresh.last_stats[0]["iterations"]


def test_capacity_restarts_from_the_newest_pair():
    cfg, g = _mob(seed=10, n=4, p=4)  # 24 force components: 17 random forces are independent
    rng = np.random.default_rng(3)
    for k in range(17):
        g.solveMob(rng.standard_normal(cfg["force"].shape), tol=1e-10, precision=PREC_FP64, warm_start="recycle")
        assert g.recycle_info()[0] == (k % 16) + 1
    # the 17th pair started a new space, which still reproduces its own solve exactly
    F = rng.standard_normal(cfg["force"].shape)
    v = g.solveMob(F, tol=1e-10, precision=PREC_FP64, warm_start="recycle")
    assert g.recycle_info()[0] == 2
    v2 = g.solveMob(F, tol=1e-10, precision=PREC_FP64, warm_start="recycle")
    assert g.last_stats[0]["iterations"] == 0 and _rel(v2, v) < 1e-12
    assert _rel(g.solveMob(F, tol=1e-10, precision=PREC_FP64), v) < 1e-8


def test_batched_problems_recycle_per_problem():
    """Two independent problems in one context: problem 0 repeats its force, problem 1 gets a new one.
    Problem 0 starts converged, problem 1 iterates; both equal their cold solves."""
    a = configs.small_cluster(seed=11, n=4, p=6, gap=0.1)
    b = configs.small_cluster(seed=12, n=5, p=6, gap=0.1)
    centers = np.vstack([a["centers"], b["centers"] + 100.0])
    radii = np.concatenate([a["radii"], b["radii"]])
    orders = np.concatenate([a["orders"], b["orders"]])
    prob = np.array([0] * 4 + [1] * 5, dtype=np.int32)
    g = SphereSTKMobMat(centers, radii, orders, problem=prob)
    cold = SphereSTKMobMat(centers, radii, orders, problem=prob)
    F = np.concatenate([a["force"], b["force"]])
    g.solveMob(F, tol=1e-10, precision=PREC_FP64, warm_start="recycle")
    F2 = F.copy()
    F2[24:] = np.random.default_rng(4).standard_normal(30)
    v = g.solveMob(F2, tol=1e-10, precision=PREC_FP64, warm_start="recycle")
    st = g.last_stats
    assert st[0]["iterations"] == 0 and st[1]["iterations"] > 5
    vc = cold.solveMob(F2, tol=1e-10, precision=PREC_FP64)
    assert _rel(v[:24], vc[:24]) < 1e-8 and _rel(v[24:], vc[24:]) < 1e-8


def test_unknown_warm_start_is_rejected():
    cfg, g = _mob(seed=13, n=2, p=4)
    with pytest.raises(SmobError):
        g.solveMob(cfg["force"], tol=1e-8, warm_start=3)
    with pytest.raises(ValueError):
        g.solveMob(cfg["force"], tol=1e-8, warm_start="always")
