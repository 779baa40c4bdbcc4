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


def test_scale_fixtures_match_their_generators():
    """The at-scale solve fixtures (tests/golden/make_golden.py --scale) hold the inputs that the
    seeded generators still produce, and their oracle answers are finite and physically sized."""
    import sys
    sys.path.insert(0, HERE)
    import make_golden as M
    from spheresimulator_gb300 import configs
    c2 = load("golden_cfg2_solve.npz")
    ref = configs.cfg2()
    assert np.array_equal(c2["centers"], ref["centers"]) and np.array_equal(c2["force"], ref["force"])
    c3 = load("golden_poly48.npz")
    ref = configs.cfg3(seed=38, n=48, box=14.0)
    assert np.array_equal(c3["centers"], ref["centers"]) and np.array_equal(c3["radii"], ref["radii"])
    b = load("golden_batch6.npz")
    ref = configs.cfg4(seed=41, n_problems=6, nmax=24)
    assert np.array_equal(b["centers"], ref["centers"]) and np.array_equal(b["problem"], ref["problem"])
    q = load("golden_p24.npz")
    ref = configs.cfg5_request(np.random.default_rng(24), nmin=20, nmax=20, orders=(24,))
    assert np.array_equal(q["centers"], ref["centers"]) and np.array_equal(q["force"], ref["force"])
    s = load("golden_seq12.npz")
    cl, cols, in_span, fresh, vstep, dt, c1, q1 = M.seq12()
    assert np.array_equal(s["cols"], cols) and np.array_equal(s["centers_moved"], c1)
    assert np.array_equal(s["quats_moved"], q1)
    # linearity of the oracle's solutions: the in-span force's velocity is the same combination
    combo = 0.6 * s["v_cols"][0] - 1.3 * s["v_cols"][1] + 0.25 * s["v_cols"][2]
    assert rel(combo, s["v_span"]) < 1e-10
    for f in (c2, c3, b, q):
        V = f["vel"].reshape(-1, 6)
        F = f["force"].reshape(-1, 6)
        assert np.all(np.isfinite(V))
        # dissipation: the mobility matrix is positive definite, F . V > 0
        assert float((F * V).sum()) > 0
