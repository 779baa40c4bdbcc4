"""The near-pair neighbour list, built on the GPU (nbrlist.cu), against the oracle's host evaluation of
the reference's rule (MPI/NearInteraction.txx:430-447 with Rad = 1.5 a, BIE/SphereSTKSHOperator.cpp:547):
ordered pairs (t, s) of one problem with 0 < |c_s - c_t|^2 < (1.5 a_s + 1.5 a_t)^2. The lists must be
identical, pair for pair, including spheres exactly at the cut-off distance, after geometry updates that
create and remove pairs, and within batches of independent problems. The device overlap check rejects a
move that makes spheres touch and leaves the context unchanged."""
import os

import numpy as np
import pytest

from spheresimulator_gb300 import PREC_FP64, SmobError, SphereSTKMobMat, SphereSTKSHOperator, configs

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def same_pairs(op, oracle, centers, radii):
    t, s = op.near_pairs()
    to, so = oracle.near_pairs(centers, radii)
    return np.array_equal(t, to) and np.array_equal(s, so)


def test_pairs_at_the_cut_off_are_decided_as_on_the_host(oracle):
    # pairs 10 apart from each other, every distance exact in binary: unit spheres at distance exactly
    # 3 (= 1.5 (1 + 1): not near, the rule is strict), one ulp below 3 (near), 2.5 (near), 3 + 2^-40
    # (not near); radii 1 and 0.5 at exactly 2.25 = 1.5 (1 + 0.5) (not near)
    below = np.nextafter(3.0, 0.0)
    centers = np.array([[0.0, 0, 0], [3.0, 0, 0], [0, 10.0, 0], [below, 10.0, 0], [0, 20.0, 0], [2.5, 20.0, 0],
                        [0, 30.0, 0], [3.0 + 2.0 ** -40, 30.0, 0], [0, 40.0, 0], [2.25, 40.0, 0]])
    radii = np.array([1.0] * 9 + [0.5])
    op = SphereSTKSHOperator(centers, radii, np.full(10, 4))
    assert same_pairs(op, oracle, centers, radii)
    t, s = op.near_pairs()
    assert sorted(zip(t.tolist(), s.tolist())) == [(2, 3), (3, 2), (4, 5), (5, 4)]


@pytest.mark.parametrize("name", ["golden_poly48.npz", "golden_p24.npz"])
def test_pairs_match_oracle_on_packed_geometries(oracle, name):
    g = dict(np.load(os.path.join(GOLDEN, name)))
    op = SphereSTKSHOperator(g["centers"], g["radii"], g["orders"])
    assert op.n_near_pairs > 0 and same_pairs(op, oracle, g["centers"], g["radii"])


def test_pairs_per_problem_in_a_batch(oracle):
    b = configs.cfg4(seed=41, n_problems=6, nmax=24)
    # the problems' boxes overlap in space: pairs must never cross problems
    op = SphereSTKSHOperator(b["centers"], b["radii"], b["orders"], problem=b["problem"])
    t, s = op.near_pairs()
    assert np.all(b["problem"][t] == b["problem"][s])
    tt, ss = [], []
    for k in range(6):
        idx = np.flatnonzero(b["problem"] == k)
        to, so = oracle.near_pairs(b["centers"][idx], b["radii"][idx])
        tt.append(idx[to])
        ss.append(idx[so])
    assert np.array_equal(t, np.concatenate(tt)) and np.array_equal(s, np.concatenate(ss))


def test_pairs_follow_geometry_updates(oracle):
    cfg = configs.small_cluster(seed=51, n=10, p=6, gap=0.3, quats=True)
    mob = SphereSTKMobMat(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg["quats"])
    assert same_pairs(mob, oracle, cfg["centers"], cfg["radii"])
    rng = np.random.default_rng(51)
    c = cfg["centers"].copy()
    n0 = mob.n_near_pairs
    for step in range(6):
        # spread the cluster out, then pull it in again: pairs disappear and reappear
        c = c * (1.15 if step < 3 else 1 / 1.15) + rng.uniform(-0.01, 0.01, c.shape)
        mob.set_geometry(c)
        assert same_pairs(mob, oracle, c, cfg["radii"]), step
    assert mob.n_near_pairs > 0 and n0 > 0
    F = rng.standard_normal(6 * 10)
    v = mob.solveMob(F, tol=1e-11, precision=PREC_FP64)
    o = oracle.Operator(c, cfg["radii"], cfg["orders"], quats=cfg["quats"]).solve_mob(F, tol=1e-12)
    assert np.linalg.norm(v - o["vel"]) / np.linalg.norm(o["vel"]) < 1e-8


def test_touching_move_is_rejected_on_the_device():
    centers = np.array([[0.0, 0, 0], [2.5, 0, 0], [0, 5.0, 0]])
    radii = np.array([1.0, 1.0, 1.0])
    op = SphereSTKSHOperator(centers, radii, np.full(3, 4))
    before = op.near_pairs()
    moved = centers.copy()
    moved[2] = [2.5, 2.0, 0]  # touches sphere 1 exactly (distance 2 = 1 + 1)
    with pytest.raises(SmobError, match="spheres 1 and 2 overlap or touch"):
        op.set_geometry(moved)
    after = op.near_pairs()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    assert np.array_equal(op.geometry()[0], centers)
