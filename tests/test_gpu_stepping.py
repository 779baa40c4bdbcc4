"""Time stepping (Sphere::stepEuler, Sphere/Sphere.cpp:367-373): after smob_step_euler /
smob_set_geometry the context equals, bit for bit, a context created from the new geometry (grid,
near pairs, operator, solve); overlapping moves are rejected without changing the context; the
previous solution warm-starts the next solve."""
import numpy as np
import pytest

from spheresimulator_gb300 import PREC_FP64, PREC_MIXED, SmobError, SphereSTKMobMat, SphereSTKSHOperator, configs

pytestmark = pytest.mark.gpu


def fresh(mob, cls=SphereSTKSHOperator):
    c, q = mob.geometry()
    return cls(c, mob.radii, mob.orders, quats=q, viscosity=mob.viscosity)


def quat_step(q, w, dt):
    """q <- (cos(|w|dt/2), sin(|w|dt/2) w/|w|) q, normalised (independent restatement)."""
    wn = np.linalg.norm(w)
    if wn * abs(dt) == 0:
        return q
    h = 0.5 * wn * dt
    a0, a = np.cos(h), np.sin(h) * w / wn
    r = np.array([a0 * q[0] - a @ q[1:], *(a0 * q[1:] + q[0] * a + np.cross(a, q[1:]))])
    return r / np.linalg.norm(r)


def same_operator(a, b, n_points, seed=0):
    x = np.random.default_rng(seed).standard_normal(3 * n_points)
    for prec in (PREC_FP64, PREC_MIXED):
        assert np.array_equal(a.apply(x, precision=prec), b.apply(x, precision=prec))


def test_step_euler_equals_fresh_context():
    cfg = configs.small_cluster(seed=31, n=7, p=8, gap=0.3, quats=True)
    mob = SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg["quats"])
    v = mob.solveMob(cfg["force"], tol=1e-10)
    c0, q0 = mob.geometry()
    dt = 0.2
    mob.step_euler(v, dt)
    c1, q1 = mob.geometry()
    V = v.reshape(-1, 6)
    assert np.array_equal(c1, c0 + V[:, :3] * dt)
    for i in range(len(q0)):
        assert np.allclose(q1[i], quat_step(q0[i], V[i, 3:], dt), rtol=0, atol=1e-14)
    f = fresh(mob, SphereSTKMobMat)
    for k in range(3):
        assert np.array_equal(mob._grid()[k], f._grid()[k])
    t, s = mob.near_pairs()
    tf, sf = f.near_pairs()
    assert np.array_equal(t, tf) and np.array_equal(s, sf)
    same_operator(mob, f, mob.n_points)
    for prec in (PREC_FP64, PREC_MIXED):
        assert np.array_equal(mob.solveMob(cfg["force"], tol=1e-10, precision=prec),
                              f.solveMob(cfg["force"], tol=1e-10, precision=prec))


def test_set_geometry_new_near_pairs_and_orders():
    """Moving a sphere of an order that had no near partner next to another builds its near maps."""
    centers = np.array([[0.0, 0, 0], [2.6, 0, 0], [30.0, 0, 0]])
    radii = np.array([1.0, 1.0, 0.9])
    orders = np.array([6, 6, 10])
    op = SphereSTKSHOperator(centers, radii, orders)
    n0 = op.n_near_pairs
    moved = centers.copy()
    moved[2] = [0.0, 2.5, 0.3]
    rng = np.random.default_rng(2)
    q = rng.standard_normal((3, 4))
    op.set_geometry(moved, q)
    assert op.n_near_pairs > n0
    f = fresh(op)
    t, s = op.near_pairs()
    tf, sf = f.near_pairs()
    assert np.array_equal(t, tf) and np.array_equal(s, sf) and 2 in s
    same_operator(op, f, op.n_points, seed=4)


def test_overlapping_move_is_rejected():
    cfg = configs.small_cluster(seed=32, n=4, p=6, gap=0.3, quats=True)
    op = SphereSTKSHOperator(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg["quats"])
    x = np.random.default_rng(5).standard_normal(3 * op.n_points)
    before = op.apply(x)
    c, q = op.geometry()
    bad = c.copy()
    bad[1] = bad[0] + 0.5 * (cfg["radii"][0] + cfg["radii"][1]) * np.array([1.0, 0, 0])
    with pytest.raises(SmobError):
        op.set_geometry(bad)
    c2, q2 = op.geometry()
    assert np.array_equal(c, c2) and np.array_equal(q, q2)
    assert np.array_equal(op.apply(x), before)


def test_time_loop_with_warm_start_and_several_columns():
    cfg = configs.small_cluster(seed=33, n=6, p=8, gap=0.4, quats=True)
    mob = SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg["quats"])
    F = cfg["force"]
    v = mob.solveMob(F, tol=1e-10, precision=PREC_MIXED)
    for _ in range(3):
        mob.step_euler(v, 0.02)
        v = mob.solveMob(F, tol=1e-10, precision=PREC_MIXED, warm_start=True)
        warm = mob.last_stats[0]
        cold = fresh(mob, SphereSTKMobMat)
        vc = cold.solveMob(F, tol=1e-10, precision=PREC_MIXED)
        assert warm["status"] == 0 and warm["iterations"] <= cold.last_stats[0]["iterations"]
        assert np.linalg.norm(v - vc) / np.linalg.norm(vc) < 1e-8
    # several columns: each the same bits as its single solve with the one-target tile, the coarse
    # targets off and every float-float pair summed (what the several-column kernels evaluate)
    mob.set_far_tile(1)
    mob.set_far_coarse_targets(False)
    mob.set_far_compression(1e-5, 0)
    G = np.random.default_rng(6).standard_normal((3, 6 * mob.n_spheres))
    V = mob.solveMobMulti(G, tol=1e-10, precision=PREC_MIXED)
    for j in range(3):
        assert np.array_equal(V[j], mob.solveMob(G[j], tol=1e-10, precision=PREC_MIXED))
