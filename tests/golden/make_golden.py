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

Run:  python tests/golden/make_golden.py
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


if __name__ == "__main__":
    main()
