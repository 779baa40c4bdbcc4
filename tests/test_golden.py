"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from the FP64 oracle on
seeded inputs): the oracle still reproduces them (CPU), and the CUDA path matches them (GPU)."""
import os

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(HERE, name)))


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b)


def test_oracle_reproduces_golden(oracle):
    g = load("golden_cfg1.npz")
    r = oracle.Operator(g["centers"], g["radii"], g["orders"]).solve_mob(g["force"], tol=1e-12)
    assert rel(r["vel"], g["vel"]) < 1e-12 and abs(r["iters"] - int(g["iters"])) <= 1
    c = load("golden_cluster.npz")
    op = oracle.Operator(c["centers"], c["radii"], c["orders"], quats=c["quats"])
    t, s = op.pairs()
    assert np.array_equal(t, c["pairs_t"]) and np.array_equal(s, c["pairs_s"])
    assert rel(op.apply_p2p(c["x"], 0.5, 0.0, 1.0), c["p2p_trac"]) < 1e-12
    assert rel(op.apply_p2p(c["x"], 0.0, 1.0, 0.0), c["p2p_sl"]) < 1e-12
    assert rel(op.apply(c["x"]), c["apply"]) < 1e-12
    h = load("golden_shexp.npz")
    p, a, q = int(h["p"]), float(h["radius"]), h["quat"]
    assert np.abs(oracle.sh_g2s(p, h["grid"], q) - h["coeff"]).max() < 1e-13
    u, tr = oracle.sh_eval_exterior(p, h["coeff"], h["targets"], h["normals"], radius=a, quat=q)
    assert rel(u, h["sl"]) < 1e-12 and rel(tr, h["trac"]) < 1e-12


def test_golden_physics():
    """Sanity of the fixtures themselves: Cfg 1 spheres move roughly with the Stokes drag of their
    own force (they are 3 radii apart) and the cluster's velocities are finite."""
    g = load("golden_cfg1.npz")
    F = g["force"].reshape(2, 6)
    V = g["vel"].reshape(2, 6)
    drag = F[:, :3] / (6 * np.pi)
    assert np.linalg.norm(V[:, :3] - drag) < 0.6 * np.linalg.norm(drag)
    assert np.all(np.isfinite(load("golden_cluster.npz")["vel"]))


@pytest.mark.gpu
def test_cuda_matches_golden():
    from spheresimulator_gb300 import PREC_FP64, SphereSTKMobMat, SphereSTKSHOperator
    g = load("golden_cfg1.npz")
    mob = SphereSTKMobMat(g["centers"], g["radii"], g["orders"])
    assert rel(mob.solveMob(g["force"], tol=1e-12), g["vel"]) < 1e-9
    c = load("golden_cluster.npz")
    op = SphereSTKSHOperator(c["centers"], c["radii"], c["orders"], quats=c["quats"])
    t, s = op.near_pairs()
    assert np.array_equal(t, c["pairs_t"]) and np.array_equal(s, c["pairs_s"])
    assert rel(op.applyP2POP(c["x"], None, 0.5, 0.0, 1.0, PREC_FP64), c["p2p_trac"]) < 1e-11
    assert rel(op.applyP2POP(c["x"], None, 0.0, 1.0, 0.0, PREC_FP64), c["p2p_sl"]) < 1e-11
    assert rel(op.applyLOP(c["x"]), c["lop"]) < 1e-13
    assert rel(op.apply(c["x"]), c["apply"]) < 1e-11
    mob = SphereSTKMobMat(c["centers"], c["radii"], c["orders"], quats=c["quats"])
    assert rel(mob.solveMob(c["force"], tol=1e-12), c["vel"]) < 1e-9
