"""Mobility solves of the CUDA path against the FP64 oracle at the benchmark configurations' scale.

The oracle's answers are committed fixtures (tests/golden/golden_{cfg2_solve,poly48,batch6,p24,seq12}.npz,
written by `tests/golden/make_golden.py --scale` from oracle solves at relative residual 1e-12, so
they stand for the exact solution of the discretised problem); the oracle takes tens of seconds per
solve at these sizes, the GPU solves here take milliseconds.

Tolerance: a solve to relative residual 1e-8 (FP64, or MIXED: FP32 operator inside high-precision
iterative refinement) must give velocities within 1e-6 relative of the oracle's; tighter solves are
held to tighter bounds where stated. The cases:
  * Cfg 2 itself (64 spheres, p = 16): the benchmark's headline solve;
  * Cfg 3 in small: 48 spheres, radii U[0.8, 1.2], gap 0.05, p = 16, near-singular pairs;
  * Cfg 4 in small: a batch of 6 independent problems, N 6..24, p in {8, 12, 16};
  * a Cfg 5 request: 20 spheres, p = 24, through the serving loop at its own tolerance;
  * several right-hand sides (one call, three columns), a recycled solve (force in the span of
    earlier ones) and a solve after an Euler time step (SphereSTKMobMat::solveMob, apply and
    Sphere::stepEuler: BIE/SphereSTKMobMat.cpp:98-286, Sphere/Sphere.cpp:367-373).
"""
import os

import numpy as np
import pytest

from spheresimulator_gb300 import PREC_FP64, PREC_MIXED, SolveServer, SphereSTKMobMat

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-8
BOUND = 1e-6  # velocities of a 1e-8 solve against the oracle


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def mob_of(g, quats=None, problem=None):
    return SphereSTKMobMat(g["centers"], g["radii"], g["orders"], quats=quats, problem=problem)


def near_singular_pairs(centers, radii):
    d = np.linalg.norm(centers[:, None] - centers[None], axis=-1)
    gap = d - radii[:, None] - radii[None]
    off = ~np.eye(len(radii), dtype=bool)
    return int(((gap < 0.1 * np.minimum(radii[:, None], radii[None])) & off).sum())


def test_cfg2_headline_solve_matches_oracle():
    g = load("golden_cfg2_solve.npz")
    mob = mob_of(g)
    assert mob.n_spheres == 64 and mob.n_points == 36992
    for prec in (PREC_MIXED, PREC_FP64):
        v = mob.solveMob(g["force"], tol=TOL, restart=50, max_iters=1000, precision=prec)
        st = mob.last_stats[0]
        assert st["status"] == 0 and st["relres"] < TOL
        assert rel(v, g["vel"]) < BOUND, (prec, rel(v, g["vel"]))
    # a tight FP64 solve reproduces the oracle's velocities to 1e-8 (only the summation order differs)
    v = mob.solveMob(g["force"], tol=1e-11, restart=50, max_iters=1000, precision=PREC_FP64)
    assert rel(v, g["vel"]) < 1e-8


def test_polydisperse_near_singular_solve_matches_oracle():
    g = load("golden_poly48.npz")
    assert near_singular_pairs(g["centers"], g["radii"]) >= 4  # gap < 0.1 a: FP64 near-singular quadrature
    mob = mob_of(g)
    assert mob.n_near_pairs == 82
    for prec in (PREC_MIXED, PREC_FP64):
        v = mob.solveMob(g["force"], tol=TOL, restart=50, max_iters=2000, precision=prec)
        assert mob.last_stats[0]["status"] == 0
        assert rel(v, g["vel"]) < BOUND, (prec, rel(v, g["vel"]))


def test_uneven_batch_matches_oracle_per_problem():
    g = load("golden_batch6.npz")
    mob = mob_of(g, problem=g["problem"])
    assert mob.n_problems == 6 and len(set(g["orders"])) == 3
    v = mob.solveMob(g["force"], tol=TOL, restart=50, max_iters=2000, precision=PREC_MIXED)
    for k in range(6):
        m6 = np.repeat(g["problem"] == k, 6)
        assert mob.last_stats[k]["status"] == 0
        assert rel(v[m6], g["vel"][m6]) < BOUND, (k, rel(v[m6], g["vel"][m6]))


def test_p24_request_served_and_solved_matches_oracle():
    g = load("golden_p24.npz")
    assert int(g["orders"][0]) == 24
    # through the serving loop at the request's own tolerance (1e-6): within 1e-5 of the oracle
    with SolveServer(device=0, max_slots=2, precision=PREC_MIXED) as srv:
        rid = srv.submit(g["centers"], g["radii"], g["orders"], g["force"], tol=1e-6)
        v, info = srv.wait(rid)
        assert info["status"] == 0
        assert rel(v, g["vel"]) < 1e-5, rel(v, g["vel"])
    mob = mob_of(g)
    for prec in (PREC_MIXED, PREC_FP64):
        v = mob.solveMob(g["force"], tol=TOL, restart=50, max_iters=2000, precision=prec)
        assert rel(v, g["vel"]) < BOUND, (prec, rel(v, g["vel"]))


def test_several_right_hand_sides_match_oracle():
    g = load("golden_seq12.npz")
    mob = mob_of(g, quats=g["quats"])
    v = mob.solveMobMulti(g["cols"], tol=TOL, restart=50, max_iters=1000, precision=PREC_MIXED)
    for j in range(3):
        assert rel(v[j], g["v_cols"][j]) < BOUND, (j, rel(v[j], g["v_cols"][j]))
    # the mobility-matrix apply with several columns (SphereSTKMobMat::apply) solves them the same way
    Y = mob.apply(g["cols"], tol=TOL, precision=PREC_MIXED)
    for j in range(3):
        assert rel(Y[j], g["v_cols"][j]) < BOUND


def test_recycled_solve_matches_oracle():
    g = load("golden_seq12.npz")
    mob = mob_of(g, quats=g["quats"])
    kw = dict(tol=TOL, restart=50, max_iters=1000, precision=PREC_MIXED, warm_start="recycle")
    for j in range(3):
        assert rel(mob.solveMob(g["cols"][j], **kw), g["v_cols"][j]) < BOUND
    assert mob.recycle_info()[0] == 3
    cold_iters = mob.last_stats[0]["iterations"]
    # a force in the span of the three: the recycled guess already meets the tolerance
    v = mob.solveMob(g["in_span"], **kw)
    assert mob.last_stats[0]["iterations"] < max(cold_iters, 1)
    assert rel(v, g["v_span"]) < BOUND, rel(v, g["v_span"])
    # a new force: least-squares guess, then GMRES
    v = mob.solveMob(g["fresh"], **kw)
    assert rel(v, g["v_fresh"]) < BOUND, rel(v, g["v_fresh"])


def test_solve_after_euler_step_matches_oracle():
    g = load("golden_seq12.npz")
    mob = mob_of(g, quats=g["quats"])
    mob.solveMob(g["cols"][1], tol=TOL, precision=PREC_MIXED)
    mob.step_euler(g["vstep"], float(g["dt"]))
    c1, q1 = mob.geometry()
    assert np.array_equal(c1, g["centers_moved"])
    assert np.abs(q1 - g["quats_moved"]).max() < 1e-14
    for prec in (PREC_MIXED, PREC_FP64):
        # warm start from the previous solution (the reference's xLast), on the moved geometry
        v = mob.solveMob(g["cols"][0], tol=TOL, restart=50, max_iters=1000, precision=prec, warm_start=True)
        assert rel(v, g["v_moved"]) < BOUND, (prec, rel(v, g["v_moved"]))
