"""Pins of the FP64 CPU oracle against the reference's own numerical tests and known answers.

The reference's only numerical tests of this path are in Sphere/Shexp_test.cpp: the G2S/S2G
round trip (testSTKConvert :77-107) and spectral single layer / traction against a direct
grid quadrature at far targets (testSTKSL :109-200, testTrac :301-411, testTracSelf :413-524),
at order 12, radius in [0.2, 5], random orientation, tolerance 1e-7 (:14). They are seeded
here (the reference draws from random_device). Known answers added: isolated-sphere Stokes
drag, reciprocity of the two-sphere mobility matrix, the near-pair rule, and the self
operators against the off-surface evaluator.
"""
import numpy as np
import pytest

P12 = 12
EBAR = 1e-7  # Sphere/Shexp_test.cpp:14


def random_quat(rng):
    q = rng.standard_normal(4)
    return q / np.linalg.norm(q)


def rot(q, v):
    w, x, y, z = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    return v @ R.T


def random_fill(O, p, q, seed=0):
    """Shexp::randomFill (Sphere/Shexp.cpp:482-501): decaying random coefficients, then
    S2G -> G2S -> S2G to drop the non-representable parts."""
    rng = np.random.default_rng(seed)
    nc2 = (p + 1) * (p + 2)
    co = np.concatenate([rng.uniform(-2, 2, nc2) * 0.8 ** np.arange(nc2) for _ in range(3)])
    g = O.sh_s2g(p, co, q)
    g = O.sh_s2g(p, O.sh_g2s(p, g, q), q)
    return g


def direct(pts, w, dens, X, Nrm=None):
    f = dens * w[:, None]
    u = np.zeros_like(X)
    t = np.zeros_like(X)
    for i in range(len(X)):
        r = X[i] - pts
        r2 = (r * r).sum(1)
        ri = 1 / np.sqrt(r2)
        rf = (r * f).sum(1)
        u[i] = ((f * ri[:, None]).sum(0) + ((rf * ri ** 3)[:, None] * r).sum(0)) / (8 * np.pi)
        if Nrm is not None:
            t[i] = -3 / (4 * np.pi) * ((rf * (r @ Nrm[i]) * ri ** 5)[:, None] * r).sum(0)
    return u, t


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_gauss_legendre(oracle):
    for n in (1, 2, 5, 9, 13, 17, 25, 33):
        x, w = oracle.gauss_legendre(n)
        xr, wr = np.polynomial.legendre.leggauss(n)
        assert np.abs(x - xr).max() < 1e-14 and np.abs(w - wr).max() < 1e-14


def test_grid_layout(oracle):
    """Shexp::getGridWithPole (Sphere/Shexp.cpp:206-271) with the poles removed."""
    rng = np.random.default_rng(3)
    p, a = 7, 1.7
    q = random_quat(rng)
    c0 = np.array([0.3, -2.0, 5.0])
    c, n, w = oracle.sh_grid(p, a, q, c0)
    x, wg = np.polynomial.legendre.leggauss(p + 1)
    ref = []
    wref = []
    for j in range(p + 1):
        ct = x[p - j]
        st = np.sqrt(1 - ct * ct)
        for k in range(2 * p + 2):
            ph = 2 * np.pi * k / (2 * p + 2)
            ref.append([st * np.cos(ph), st * np.sin(ph), ct])
            wref.append(a * a * 2 * np.pi / (2 * p + 2) * wg[p - j])
    ref = rot(q, np.array(ref))
    assert np.abs(n - ref).max() < 1e-14
    assert np.abs(c - (a * ref + c0)).max() < 1e-13
    assert np.abs(w - np.array(wref)).max() < 1e-14
    assert abs(w.sum() - 4 * np.pi * a * a) < 1e-12


def test_convert_idempotent(oracle):
    """testSTKConvert (Sphere/Shexp_test.cpp:77-107)."""
    rng = np.random.default_rng(11)
    q = random_quat(rng)
    g0 = rng.uniform(-2, 2, (oracle.grid_number(P12), 3))
    g = oracle.sh_s2g(P12, oracle.sh_g2s(P12, g0, q), q)
    ref = g.copy()
    for _ in range(50):
        g = oracle.sh_s2g(P12, oracle.sh_g2s(P12, g, q), q)
    assert np.abs(g - ref).max() < EBAR * np.abs(ref).max()
    # coefficient round trip is exact on the band-limited space
    co = oracle.sh_g2s(P12, ref, q)
    assert np.abs(oracle.sh_g2s(P12, oracle.sh_s2g(P12, co, q), q) - co).max() < 1e-12


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_spectral_vs_direct_far(oracle, seed):
    """testSTKSL / testTrac / testTracSelf exterior cases (Sphere/Shexp_test.cpp:109-524)."""
    rng = np.random.default_rng(100 + seed)
    a = rng.uniform(0.2, 5.0)
    q = random_quat(rng)
    dens = random_fill(oracle, P12, q, seed)
    pts, _, w = oracle.sh_grid(P12, a, q)
    co = oracle.sh_g2s(P12, dens, q)
    X = rng.standard_normal((300, 3))
    X = 4 * a * X / np.linalg.norm(X, axis=1)[:, None]
    Nr = rng.standard_normal((300, 3))
    Nr /= np.linalg.norm(Nr, axis=1)[:, None]
    u, t = oracle.sh_eval_exterior(P12, co, X, Nr, radius=a, quat=q)
    ud, td = direct(pts, w, dens, X, Nr)
    assert rel(u, ud) < EBAR
    assert rel(t, td) < EBAR
    # TracSelf: targets with radial normals
    Nself = X / np.linalg.norm(X, axis=1)[:, None]
    _, ts = oracle.sh_eval_exterior(P12, co, X, Nself, radius=a, quat=q, sl=False)
    _, tsd = direct(pts, w, dens, X, Nself)
    assert rel(ts, tsd) < EBAR


def test_self_operators_vs_evaluator(oracle):
    """On-surface self terms (multipliers) equal the off-surface evaluator's exterior limit at r=a;
    PV = exterior + f/2, interior = exterior + f (traction jump of the single layer)."""
    rng = np.random.default_rng(5)
    p, a = 10, 1.3
    q = random_quat(rng)
    dens = oracle.sh_s2g(p, oracle.sh_g2s(p, rng.uniform(-1, 1, (oracle.grid_number(p), 3)), q), q)
    co = oracle.sh_g2s(p, dens, q)
    pts, nrm, _ = oracle.sh_grid(p, a, q)
    u_e, t_e = oracle.sh_eval_exterior(p, co, pts, nrm, radius=a, quat=q)
    sl = oracle.sh_self(p, co, oracle.SELF_SL, a, q)
    ext = oracle.sh_self(p, co, oracle.SELF_TRAC_EXT, a, q)
    pv = oracle.sh_self(p, co, oracle.SELF_TRAC_PV, a, q)
    inn = oracle.sh_self(p, co, oracle.SELF_TRAC_INT, a, q)
    scale = np.abs(t_e).max()
    assert np.abs(sl - u_e).max() < 1e-12 * np.abs(u_e).max()
    assert np.abs(ext - t_e).max() < 1e-12 * scale
    assert np.abs(pv - (t_e + 0.5 * dens)).max() < 1e-12 * scale
    assert np.abs(inn - (t_e + dens)).max() < 1e-12 * scale


def test_near_evaluator_vs_fine_quadrature(oracle):
    """Near-singular targets (0.15a..0.6a off the surface): the spectral evaluator agrees with a
    direct quadrature of the same band-limited density on a much finer grid."""
    rng = np.random.default_rng(9)
    p, pf, a = 8, 80, 1.0
    q = random_quat(rng)
    dens = oracle.sh_s2g(p, oracle.sh_g2s(p, rng.uniform(-1, 1, (oracle.grid_number(p), 3)), q), q)
    co = oracle.sh_g2s(p, dens, q)
    # pad the coefficients into the order-pf layout and synthesise on the fine grid
    ncp, ncf = (p + 1) * (p + 2) // 2, (pf + 1) * (pf + 2) // 2
    cf = np.zeros(3 * 2 * ncf)
    for b in range(3):
        cf[b * 2 * ncf:b * 2 * ncf + 2 * ncp] = co[b * 2 * ncp:(b + 1) * 2 * ncp]
    dens_f = oracle.sh_s2g(pf, cf, q)
    pts_f, _, w_f = oracle.sh_grid(pf, a, q)
    X = rng.standard_normal((40, 3))
    X = X / np.linalg.norm(X, axis=1)[:, None] * rng.uniform(1.15, 1.6, 40)[:, None]
    Nr = rng.standard_normal((40, 3))
    Nr /= np.linalg.norm(Nr, axis=1)[:, None]
    u, t = oracle.sh_eval_exterior(p, co, X, Nr, radius=a, quat=q)
    ud, td = direct(pts_f, w_f, dens_f, X, Nr)
    # the fine quadrature converges geometrically to the spectral value (1e-11 / 1e-9 at order 80)
    assert rel(u, ud) < 1e-9
    assert rel(t, td) < 1e-8


@pytest.mark.parametrize("a,visc", [(1.0, 1.0), (0.7, 2.5), (1.9, 0.3)])
def test_isolated_sphere_drag(oracle, a, visc):
    """One sphere: V = F/(6 pi mu a), Omega = T/(8 pi mu a^3) (SRC/SphereSystem.cpp:261-262)."""
    rng = np.random.default_rng(int(a * 10))
    q = random_quat(rng)
    op = oracle.Operator([[0.3, -1, 2]], [a], [8], quats=q, viscosity=visc)
    F = rng.standard_normal(6)
    r = op.solve_mob(F, tol=1e-12)
    assert np.allclose(r["vel"][:3], F[:3] / (6 * np.pi * visc * a), rtol=1e-12, atol=1e-14)
    assert np.allclose(r["vel"][3:], F[3:] / (8 * np.pi * visc * a ** 3), rtol=1e-12, atol=1e-14)


def test_two_sphere_mobility_reciprocal(oracle):
    """Cfg 1 geometry: the 12x12 mobility matrix is symmetric positive definite."""
    op = oracle.Operator([[0, 0, 0], [3, 0, 0]], [1, 1], [8, 8])
    M = np.zeros((12, 12))
    for k in range(12):
        e = np.zeros(12)
        e[k] = 1
        M[:, k] = op.solve_mob(e, tol=1e-12)["vel"]
    assert np.abs(M - M.T).max() < 1e-7 * np.abs(M).max()
    assert np.linalg.eigvalsh(0.5 * (M + M.T)).min() > 0
    # far-apart limit: self mobility close to the Stokes drag
    assert abs(M[0, 0] * 6 * np.pi - 1) < 0.1


def test_near_pair_rule(oracle):
    """MPI/NearInteraction.txx:430-447 with Rad = 1.5 a (BIE/SphereSTKSHOperator.cpp:547):
    strict inequality, no self pairs; Cfg 1 (distance exactly 3) has no pairs."""
    t, s = oracle.near_pairs(np.array([[0, 0, 0], [3.0, 0, 0]]), np.ones(2))
    assert len(t) == 0
    c = np.array([[0, 0, 0], [2.9, 0, 0], [0, 2.5, 0], [10, 0, 0]])
    r = np.array([1.0, 1.0, 0.8, 1.0])
    t, s = oracle.near_pairs(c, r)
    pairs = set(zip(t.tolist(), s.tolist()))
    expect = set()
    for i in range(4):
        for j in range(4):
            d2 = ((c[i] - c[j]) ** 2).sum()
            if d2 > 0 and d2 < (1.5 * r[i] + 1.5 * r[j]) ** 2:
                expect.add((i, j))
    assert pairs == expect and (0, 1) in pairs and (1, 0) in pairs
    assert list(zip(t, s)) == sorted(zip(t, s))


def test_rotation_changes_only_discretisation(oracle):
    """Random layer quaternions (SRC/SphereSystem.cpp:56-57) rotate the grids; the velocities
    agree with identity orientations to discretisation accuracy."""
    rng = np.random.default_rng(21)
    c = np.array([[0, 0, 0], [2.6, 0.4, 0.0], [0.5, 2.7, 0.3]])
    r = np.array([1.0, 0.9, 1.1])
    F = rng.standard_normal(18)
    v0 = oracle.Operator(c, r, [10] * 3).solve_mob(F, tol=1e-12)["vel"]
    q = np.array([random_quat(rng) for _ in range(3)])
    v1 = oracle.Operator(c, r, [10] * 3, quats=q).solve_mob(F, tol=1e-12)["vel"]
    assert np.abs(v1 - v0).max() < 2e-3 * np.abs(v0).max()


def test_zero_force_shortcut(oracle):
    """|b| < 1e-5 -> mu = 0 (BIE/SphereSTKMobMat.cpp:217-218)."""
    op = oracle.Operator([[0, 0, 0], [2.5, 0, 0]], [1, 1], [6, 6])
    r = op.solve_mob(np.zeros(12))
    assert r["iters"] == 0 and np.all(r["vel"] == 0)
