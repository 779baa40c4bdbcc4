"""Generate the golden fixtures (seeded inputs and FP64 oracle outputs) used by the tests.

The reference ships no golden vectors (Sphere/Shexp_test.cpp draws from random_device), so the
fixtures are produced by the FP64 CPU restatement in oracle/ on seeded inputs and committed:

  golden_cfg1.npz     Cfg 1 (2 spheres, p=8): forces, velocities, density, iterations at tol 1e-12
  golden_cluster.npz  5-sphere cluster with near pairs and random orientations (p=7): an input
                      density and the outputs of applyP2POP(traction), applyP2POP(single layer),
                      applyLOP, apply, and a mobility solve
  golden_shexp.npz    one sphere (p=12, radius 1.7, random orientation): grid density, its
                      coefficients, self single layer / traction PV, exterior SL and traction at
                      targets 1.2a..4a

Mobility solves at the benchmark configurations' scale (oracle at tol 1e-12, the "exact" answer the
GPU solves at 1e-8 / 1e-6 are checked against), written by --scale:

  golden_cfg2_solve.npz  Cfg 2 itself (64 spheres, p=16, 36,992 points): force, velocities
  golden_poly48.npz      Cfg 3 in small: 48 spheres a ~ U[0.8,1.2], RSA gap 0.05 in a box of side 14,
                         p=16, 82 near pairs of which 4 are near-singular (gap < 0.1 a)
  golden_batch6.npz      Cfg 4 in small: 6 independent problems, N 6..24, p in {8,12,16}; one oracle
                         solve per problem
  golden_p24.npz         a Cfg 5 request: 20 spheres a ~ U[0.9,1.1], gap 0.05, p=24
  golden_seq12.npz       12 spheres p=12 with random orientations: three force columns (several
                         right-hand sides), a force in their span and a new one (recycling), and a
                         time step (prescribed v, omega, dt) with the oracle solve on the moved geometry

Run:  python tests/golden/make_golden.py [--scale [cfg2 poly48 batch6 p24 seq12]]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from spheresimulator_gb300 import configs  # noqa: E402


def main():
    c1 = configs.cfg1()
    op = O.Operator(c1["centers"], c1["radii"], c1["orders"])
    r = op.solve_mob(c1["force"], tol=1e-12)
    np.savez_compressed(os.path.join(HERE, "golden_cfg1.npz"), centers=c1["centers"], radii=c1["radii"],
                        orders=c1["orders"], force=c1["force"], vel=r["vel"], density=r["density"],
                        iters=r["iters"])

    cl = configs.small_cluster(seed=7, n=5, p=7, gap=0.2, quats=True)
    op = O.Operator(cl["centers"], cl["radii"], cl["orders"], quats=cl["quats"])
    x = np.random.default_rng(7).standard_normal(3 * op.m)
    r = op.solve_mob(cl["force"], tol=1e-12)
    np.savez_compressed(os.path.join(HERE, "golden_cluster.npz"), centers=cl["centers"], radii=cl["radii"],
                        orders=cl["orders"], quats=cl["quats"], force=cl["force"], x=x,
                        p2p_trac=op.apply_p2p(x, 0.5, 0.0, 1.0), p2p_sl=op.apply_p2p(x, 0.0, 1.0, 0.0),
                        lop=op.apply_lop(x, 1.0), apply=op.apply(x), vel=r["vel"], density=r["density"],
                        pairs_t=op.pairs()[0], pairs_s=op.pairs()[1])

    rng = np.random.default_rng(12)
    p, a = 12, 1.7
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    g = O.sh_s2g(p, O.sh_g2s(p, rng.uniform(-1, 1, (O.grid_number(p), 3)), q), q)
    co = O.sh_g2s(p, g, q)
    X = rng.standard_normal((64, 3))
    X = X / np.linalg.norm(X, axis=1)[:, None] * rng.uniform(1.2 * a, 4 * a, 64)[:, None]
    Nr = rng.standard_normal((64, 3))
    Nr /= np.linalg.norm(Nr, axis=1)[:, None]
    u, t = O.sh_eval_exterior(p, co, X, Nr, radius=a, quat=q)
    np.savez_compressed(os.path.join(HERE, "golden_shexp.npz"), p=p, radius=a, quat=q, grid=g, coeff=co,
                        self_sl=O.sh_self(p, co, O.SELF_SL, a, q), self_pv=O.sh_self(p, co, O.SELF_TRAC_PV, a, q),
                        targets=X, normals=Nr, sl=u, trac=t)
    print("wrote golden fixtures to", HERE)


def quat_step(q, w, dt):
    """Orientation after a step: rotation by |w| dt about w composed on the left, normalised."""
    wn = np.linalg.norm(w)
    if wn * abs(dt) == 0:
        return np.array(q, dtype=float)
    h = 0.5 * wn * dt
    a0, a = np.cos(h), np.sin(h) * w / wn
    r = np.array([a0 * q[0] - a @ q[1:], *(a0 * q[1:] + q[0] * a + np.cross(a, q[1:]))])
    return r / np.linalg.norm(r)


def seq12():
    """Geometry, forces and the moved geometry of golden_seq12.npz (also used by the GPU tests)."""
    cl = configs.small_cluster(seed=12, n=12, p=12, gap=0.2, quats=True)
    rng = np.random.default_rng(1212)
    cols = rng.standard_normal((3, 6 * 12))
    in_span = 0.6 * cols[0] - 1.3 * cols[1] + 0.25 * cols[2]
    fresh = rng.standard_normal(6 * 12)
    vstep = 0.1 * rng.standard_normal((12, 6))
    dt = 0.25
    c1 = cl["centers"] + vstep[:, :3] * dt
    d = np.linalg.norm(c1[:, None] - c1[None], axis=-1) - cl["radii"][:, None] - cl["radii"][None]
    assert d[~np.eye(12, dtype=bool)].min() > 0.1, "the step brings two spheres within 0.1 of each other"
    q1 = np.array([quat_step(cl["quats"][i], vstep[i, 3:], dt) for i in range(12)])
    return cl, cols, in_span, fresh, vstep, dt, c1, q1


def scale(only=None):
    """Writes the at-scale solve fixtures (all, or those named in `only`)."""
    def want(name):
        return not only or name in only

    def solve(centers, radii, orders, force, quats=None):
        op = O.Operator(centers, radii, orders, quats=quats)
        r = op.solve_mob(force, tol=1e-12, restart=50, maxit=2000)
        assert r["status"] == 0 and r["relres"] < 1e-12, (r["status"], r["relres"])
        return r

    if want("cfg2"):
        c2 = configs.cfg2()
        r = solve(c2["centers"], c2["radii"], c2["orders"], c2["force"])
        np.savez_compressed(os.path.join(HERE, "golden_cfg2_solve.npz"), centers=c2["centers"], radii=c2["radii"],
                            orders=c2["orders"], force=c2["force"], vel=r["vel"], iters=r["iters"])
        print("cfg2", r["iters"], r["relres"], flush=True)

    if want("poly48"):
        c3 = configs.cfg3(seed=38, n=48, box=14.0)
        r = solve(c3["centers"], c3["radii"], c3["orders"], c3["force"])
        np.savez_compressed(os.path.join(HERE, "golden_poly48.npz"), centers=c3["centers"], radii=c3["radii"],
                            orders=c3["orders"], force=c3["force"], vel=r["vel"], iters=r["iters"])
        print("poly48", r["iters"], r["relres"], flush=True)

    if want("batch6"):
        b = configs.cfg4(seed=41, n_problems=6, nmax=24)
        vel = np.zeros_like(b["force"])
        for k in range(6):
            m = b["problem"] == k
            m6 = np.repeat(m, 6)
            vel[m6] = solve(b["centers"][m], b["radii"][m], b["orders"][m], b["force"][m6])["vel"]
        np.savez_compressed(os.path.join(HERE, "golden_batch6.npz"), centers=b["centers"], radii=b["radii"],
                            orders=b["orders"], problem=b["problem"], force=b["force"], vel=vel)
        print("batch6", flush=True)

    if want("p24"):
        q = configs.cfg5_request(np.random.default_rng(24), nmin=20, nmax=20, orders=(24,))
        r = solve(q["centers"], q["radii"], q["orders"], q["force"])
        np.savez_compressed(os.path.join(HERE, "golden_p24.npz"), centers=q["centers"], radii=q["radii"],
                            orders=q["orders"], force=q["force"], vel=r["vel"], iters=r["iters"])
        print("p24", r["iters"], r["relres"], flush=True)

    if want("seq12"):
        cl, cols, in_span, fresh, vstep, dt, c1, q1 = seq12()
        v_cols = np.stack([solve(cl["centers"], cl["radii"], cl["orders"], f, cl["quats"])["vel"] for f in cols])
        v_span = solve(cl["centers"], cl["radii"], cl["orders"], in_span, cl["quats"])["vel"]
        v_fresh = solve(cl["centers"], cl["radii"], cl["orders"], fresh, cl["quats"])["vel"]
        v_moved = solve(c1, cl["radii"], cl["orders"], cols[0], q1)["vel"]
        np.savez_compressed(os.path.join(HERE, "golden_seq12.npz"), centers=cl["centers"], radii=cl["radii"],
                            orders=cl["orders"], quats=cl["quats"], cols=cols, v_cols=v_cols, in_span=in_span,
                            v_span=v_span, fresh=fresh, v_fresh=v_fresh, vstep=vstep, dt=dt, centers_moved=c1,
                            quats_moved=q1, v_moved=v_moved)
        print("seq12", flush=True)


if __name__ == "__main__":
    if "--scale" in sys.argv:
        scale([a for a in sys.argv[1:] if not a.startswith("--")])
    else:
        main()
