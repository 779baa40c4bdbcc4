"""Parity of the CUDA path (through the C ABI) with the FP64 CPU oracle.

Tolerances: FP64 kernels agree with the oracle to 1e-11 relative (summation order only);
FP32 kernels to 2e-5 relative (single-precision pair sums); FP64 solves to 1e-8 relative in
the velocities at tol 1e-12; mixed-precision solves to 1e-6 relative at tol 1e-10.
"""
import numpy as np
import pytest

from spheresimulator_gb300 import (PREC_FLOAT_FLOAT, PREC_FP64, PREC_MIXED, SmobError, SphereSTKMobMat,
                                   SphereSTKSHOperator, configs)

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def cluster(seed=0, n=5, p=6, quats=True, gap=0.25):
    return configs.small_cluster(seed=seed, n=n, p=p, gap=gap, quats=quats)


def make(cfg, cls=SphereSTKSHOperator, **kw):
    return cls(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg.get("quats"), problem=cfg.get("problem"), **kw)


def oracle_op(oracle, cfg, **kw):
    return oracle.Operator(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg.get("quats"), **kw)


def test_grid_matches_oracle(oracle):
    cfg = cluster(1)
    g = make(cfg)
    o = oracle_op(oracle, cfg)
    c, n, w = o.grid()
    assert np.abs(g.getGridCoords() - c).max() < 1e-13
    assert np.abs(g.getGridNorms() - n).max() < 1e-14
    assert np.abs(g.getGridWeights() - w).max() < 1e-14
    t, s = g.near_pairs()
    to, so = o.pairs()
    assert len(t) > 0 and np.array_equal(t, to) and np.array_equal(s, so)


@pytest.mark.parametrize("seed", [0, 1])
def test_far_field(oracle, seed):
    cfg = cluster(seed)
    g = make(cfg)
    o = oracle_op(oracle, cfg)
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(3 * g.n_points)
    for c_sl, c_tr in ((0.0, 1.0), (1.0, 0.0), (0.7, -1.3)):
        ref = o.far_traction(x, c_tr, excl_near=True) + o.far_sl(x, c_sl, excl_near=True)
        assert rel(g.far_field(x, cSL=c_sl, cTrac=c_tr, precision=PREC_FP64), ref) < 1e-11
        assert rel(g.far_field(x, cSL=c_sl, cTrac=c_tr, precision=PREC_MIXED), ref) < 2e-5
        # float-float (hi+lo float pairs): ~48 significant bits
        assert rel(g.far_field(x, cSL=c_sl, cTrac=c_tr, precision=PREC_FLOAT_FLOAT), ref) < 1e-12


def test_far_tile_variants(oracle):
    """Each FP32 far-field variant (1, 2 or 4 targets per thread, scalar or packed FP32x2) matches the
    oracle; forcing one replaces the autotuner's choice."""
    cfg = cluster(3, n=7, p=8)
    g = make(cfg)
    g.set_far_coarse_targets(False)  # the FP32 passes run the grid kernels
    o = oracle_op(oracle, cfg)
    x = np.random.default_rng(3).standard_normal(3 * g.n_points)
    ref = o.far_traction(x, 1.0, excl_near=True) + o.far_sl(x, 0.5, excl_near=True)
    outs = []
    for tpt in (1, 2, 4):
        g.set_far_tile(tpt)
        assert g.tuning()[0] == tpt
        outs.append(g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_MIXED))
        assert rel(outs[-1], ref) < 2e-5
    assert rel(outs[1], outs[2]) < 1e-6
    with pytest.raises(SmobError):
        g.set_far_tile(3)


def test_transforms(oracle):
    cfg = cluster(2, n=3, p=9)
    g = make(cfg)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((g.n_points, 3))
    co = g.sh_g2s(x.reshape(-1))
    off = g.coeff_offsets()
    gi = g.getGridNumberIndex()
    for i in range(g.n_spheres):
        p = int(cfg["orders"][i])
        ng = (p + 1) * (2 * p + 2)
        ref = oracle.sh_g2s(p, x[gi[i]:gi[i] + ng], cfg["quats"][i])
        assert np.abs(co[off[i]:off[i + 1]] - ref).max() < 1e-12 * np.abs(ref).max()
    back = g.sh_s2g(co).reshape(-1, 3)
    for i in range(g.n_spheres):
        p = int(cfg["orders"][i])
        ng = (p + 1) * (2 * p + 2)
        ref = oracle.sh_s2g(p, co[off[i]:off[i + 1]], cfg["quats"][i])
        assert np.abs(back[gi[i]:gi[i] + ng] - ref).max() < 1e-12 * np.abs(ref).max()
    proj = g.projectNullSpace(x.reshape(-1))
    assert np.abs(proj - back.reshape(-1)).max() < 1e-13 * np.abs(back).max()


@pytest.mark.parametrize("coefs", [(0.5, 0.0, 1.0), (-0.5, 0.0, -1.0), (0.0, 1.0, 0.0), (0.2, 0.8, -0.4)])
def test_apply_p2p(oracle, coefs):
    cfg = cluster(3, n=5, p=7)
    g = make(cfg)
    o = oracle_op(oracle, cfg)
    rng = np.random.default_rng(4)
    x = rng.standard_normal(3 * g.n_points)
    y0 = rng.standard_normal(3 * g.n_points)
    ref = o.apply_p2p(x, *coefs, out=y0)
    out = g.applyP2POP(x, y0, *coefs, precision=PREC_FP64)
    assert rel(out - y0, ref - y0) < 1e-11
    out32 = g.applyP2POP(x, y0, *coefs, precision=PREC_MIXED)
    assert rel(out32 - y0, ref - y0) < 2e-5
    outdf = g.applyP2POP(x, y0, *coefs, precision=PREC_FLOAT_FLOAT)
    assert rel(outdf - y0, ref - y0) < 1e-12


def test_near_field_is_spectral_part(oracle):
    """far(excluding near spheres) + near(spectral) equals the reference decomposition
    far(all other spheres) + near(spectral - direct)."""
    cfg = cluster(5, n=6, p=8)
    g = make(cfg)
    o = oracle_op(oracle, cfg)
    assert g.n_near_pairs > 0
    x = np.random.default_rng(5).standard_normal(3 * g.n_points)
    mine = g.far_field(x, 0.3, 1.0) + g.near_field(x, 0.3, 1.0)
    ref = o.far_traction(x, 1.0) + o.far_sl(x, 0.3) + o.near_correction(x, 0.3, 1.0)
    assert rel(mine, ref) < 1e-11


def test_apply_lop_and_apply(oracle):
    cfg = cluster(6, n=4, p=6)
    g = make(cfg)
    o = oracle_op(oracle, cfg)
    rng = np.random.default_rng(6)
    x = rng.standard_normal(3 * g.n_points)
    assert rel(g.applyLOP(x, cLOP=1.7), o.apply_lop(x, 1.7)) < 1e-13
    y = rng.standard_normal(3 * g.n_points)
    assert rel(g.apply(x, y, alpha=0.7, beta=-0.3), o.apply(x, y, 0.7, -0.3)) < 1e-11
    X = rng.standard_normal((3, 3 * g.n_points))
    Y = g.apply(X)
    for k in range(3):
        assert rel(Y[k], o.apply(X[k])) < 1e-11


def test_apply_cfg2_scale(oracle):
    """Cfg 2 geometry (64 spheres, p=16): one operator application against the oracle."""
    cfg = configs.cfg2()
    g = make(cfg)
    o = oracle_op(oracle, cfg)
    x = np.random.default_rng(7).standard_normal(3 * g.n_points)
    ref = o.apply(x)
    assert rel(g.apply(x), ref) < 1e-11
    assert rel(g.apply(x, precision=PREC_MIXED), ref) < 2e-5


def test_high_orders(oracle):
    """Orders up to the library maximum p = 32 (Cfg 5 draws p = 24) with near pairs between spheres of
    different orders: the operator and a solve match the oracle."""
    rng = np.random.default_rng(23)
    q = rng.standard_normal((3, 4))
    cfg = dict(centers=np.array([[0.0, 0, 0], [2.2, 0, 0], [4.4, 0.4, 0]]), radii=np.array([1.0, 1.0, 0.9]),
               orders=np.array([24, 32, 20]), quats=q / np.linalg.norm(q, axis=1)[:, None],
               force=rng.standard_normal(18))
    g = make(cfg)
    assert g.n_near_pairs > 0
    o = oracle_op(oracle, cfg)
    x = np.random.default_rng(23).standard_normal(3 * g.n_points)
    ref = o.apply(x)
    assert rel(g.apply(x), ref) < 1e-11
    assert rel(g.apply(x, precision=PREC_MIXED), ref) < 2e-5
    mob = make(cfg, SphereSTKMobMat)
    vel = mob.solveMob(cfg["force"], tol=1e-11)
    assert rel(vel, o.solve_mob(cfg["force"], tol=1e-12)["vel"]) < 1e-8


def test_mobility_properties_cfg2_scale():
    """Cfg 2 (64 spheres, p=16, the bench workload) through size-independent properties of the
    mobility matrix M: reciprocity F1.M F2 = F2.M F1 (M is symmetric), positive dissipation F.M F > 0,
    and linearity M(a F1 + b F2) = a M F1 + b M F2, all to the solve tolerance, mixed precision; the
    several-column solve gives the single solves' columns."""
    cfg = configs.cfg2()
    mob = make(cfg, SphereSTKMobMat)
    rng = np.random.default_rng(5)
    F1, F2 = rng.standard_normal((2, 6 * mob.n_spheres))
    kw = dict(tol=1e-10, precision=PREC_MIXED, want_density=False)
    V1, V2 = mob.solveMob(F1, **kw), mob.solveMob(F2, **kw)
    assert abs(F1 @ V2 - F2 @ V1) < 1e-8 * np.linalg.norm(F1) * np.linalg.norm(V2)
    assert F1 @ V1 > 0 and F2 @ V2 > 0
    V12 = mob.solveMob(0.3 * F1 - 1.7 * F2, **kw)
    assert rel(V12, 0.3 * V1 - 1.7 * V2) < 1e-8
    Vm = mob.solveMobMulti(np.stack([F1, F2]), tol=1e-10, precision=PREC_MIXED)
    assert rel(Vm[0], V1) < 1e-8 and rel(Vm[1], V2) < 1e-8


@pytest.mark.parametrize("which", ["cfg1", "cluster"])
def test_solve_mob_fp64(oracle, which):
    cfg = configs.cfg1() if which == "cfg1" else cluster(8, n=6, p=8)
    g = make(cfg, SphereSTKMobMat)
    o = oracle_op(oracle, cfg)
    ref = o.solve_mob(cfg["force"], tol=1e-12, restart=50, maxit=500)
    vel = g.solveMob(cfg["force"], tol=1e-12, restart=50, max_iters=500)
    assert rel(vel, ref["vel"]) < 1e-8
    assert rel(g.getDensitySolution(), ref["density"]) < 1e-8
    st = g.last_stats[0]
    assert st["status"] == 0 and st["relres"] < 1e-12
    assert abs(st["iterations"] - ref["iters"]) <= 1


def test_solve_mob_mixed(oracle):
    cfg = cluster(9, n=6, p=8)
    g = make(cfg, SphereSTKMobMat)
    o = oracle_op(oracle, cfg)
    ref = o.solve_mob(cfg["force"], tol=1e-12)
    vel = g.solveMob(cfg["force"], tol=1e-10, precision=PREC_MIXED)
    st = g.last_stats[0]
    assert st["status"] == 0 and st["relres"] < 1e-10
    assert st["operator_passes_fp32"] > 0
    # b in FP32, then fused high-precision residual + single-layer passes only where refinement needs them
    assert 1 <= st["operator_passes_fp64"] <= st["refinements"]
    assert rel(vel, ref["vel"]) < 1e-6


def test_restart_small(oracle):
    """GMRES(5) with restarts reaches the same solution."""
    cfg = cluster(10, n=5, p=6)
    g = make(cfg, SphereSTKMobMat)
    o = oracle_op(oracle, cfg)
    ref = o.solve_mob(cfg["force"], tol=1e-11, restart=5, maxit=400)
    vel = g.solveMob(cfg["force"], tol=1e-11, restart=5, max_iters=400)
    assert rel(vel, ref["vel"]) < 1e-8
    assert g.last_stats[0]["refinements"] > 1


def test_batched_equals_alone():
    """Problems solved together give bitwise the same result as each solved alone (problems of a
    batch may overlap in space: they never interact)."""
    a = cluster(11, n=4, p=6)
    b = cluster(12, n=7, p=8)
    cat = dict(centers=np.concatenate([a["centers"], b["centers"]]), radii=np.concatenate([a["radii"], b["radii"]]),
               orders=np.concatenate([a["orders"], b["orders"]]), quats=np.concatenate([a["quats"], b["quats"]]),
               problem=np.concatenate([np.zeros(4, np.int32), np.ones(7, np.int32)]))
    F = np.concatenate([a["force"], b["force"]])
    for prec in (PREC_FP64, PREC_MIXED):
        va = make(a, SphereSTKMobMat).solveMob(a["force"], tol=1e-10, precision=prec)
        vb = make(b, SphereSTKMobMat).solveMob(b["force"], tol=1e-10, precision=prec)
        gb = make(cat, SphereSTKMobMat)
        v = gb.solveMob(F, tol=1e-10, precision=prec)
        assert np.array_equal(v[:24], va) and np.array_equal(v[24:], vb)
        assert len(gb.last_stats) == 2


@pytest.mark.parametrize("k", [2, 5])
def test_multi_rhs_batch_equals_single_solves(k):
    """K right-hand sides solved together as a batch of copies (the default) give bit for bit each
    column's single solve with the context's own settings (coarse sources and targets, float-float
    compression, tensor-core kernels), in both precisions."""
    rng = np.random.default_rng(23)
    radii = rng.uniform(0.8, 1.2, 14)
    cfg = dict(centers=configs.rsa(rng, 14, radii, 26.0, 0.1), radii=radii, orders=np.full(14, 10))
    mob = make(cfg, SphereSTKMobMat)
    assert mob.far_compression_info()[2] > 0 and mob.far_compression_info(hp=True)[2] > 0
    F = np.random.default_rng(k + 30).standard_normal((k, 6 * mob.n_spheres))
    for prec in (PREC_MIXED, PREC_FP64):
        V = mob.solveMobMulti(F, tol=1e-9, precision=prec)
        for j in range(k):
            assert np.array_equal(V[j], mob.solveMob(F[j], tol=1e-9, precision=prec)), (prec, j)


@pytest.mark.parametrize("k", [2, 3, 6])
def test_multi_rhs_equals_single_solves(k):
    """K right-hand sides solved together with the shared-pair kernels (smob_set_multi_shared_pairs:
    the FP32 far field evaluates each pair's geometry once for all columns) give bit for bit the
    solves of each column alone with the one-target-per-thread FP32 kernel, with and without coarse
    equivalent sources in the FP32 passes (the several-column float-float pass sums every grid-point
    pair and the several-column FP32 kernel evaluates the grid targets of every far pair, so the single
    solves' float-float set and coarse targets are off here); the Tpetra-style apply with K columns
    uses the same path."""
    rng = np.random.default_rng(19)
    radii = rng.uniform(0.8, 1.2, 12)
    cfg = dict(centers=configs.rsa(rng, 12, radii, 24.0, 0.1), radii=radii, orders=np.full(12, 10))
    mob = make(cfg, SphereSTKMobMat)
    mob.set_multi_shared_pairs(True)
    mob.set_far_tile(1)
    mob.set_far_compression(1e-7, 0)
    mob.set_far_coarse_targets(False)
    assert mob.far_compression_info()[2] > 0
    F = np.random.default_rng(k).standard_normal((k, 6 * mob.n_spheres))
    for prec in (PREC_MIXED, PREC_FP64):
        V = mob.solveMobMulti(F, tol=1e-10, precision=prec, want_density=True)
        stats, dens = mob.last_stats, mob.getDensitySolution()
        assert len(stats) == k and all(s["status"] == 0 for s in stats)
        for j in range(k):
            v = mob.solveMob(F[j], tol=1e-10, precision=prec)
            assert np.array_equal(V[j], v)
            assert np.array_equal(dens[j], mob.getDensitySolution())
            assert stats[j]["iterations"] == mob.last_stats[0]["iterations"]
    mob.set_far_compression(0, 0)
    V = mob.solveMobMulti(F, tol=1e-10, precision=PREC_MIXED)
    for j in range(k):
        assert np.array_equal(V[j], mob.solveMob(F[j], tol=1e-10, precision=PREC_MIXED))
    Y0 = np.random.default_rng(1).standard_normal(F.shape)
    Y = mob.apply(F, Y0, alpha=2.0, beta=0.5, tol=1e-10, precision=PREC_MIXED)
    assert np.allclose(Y, 0.5 * Y0 + 2.0 * mob.solveMobMulti(F, tol=1e-10, precision=PREC_MIXED), rtol=0, atol=1e-14)


def test_block_diagonal_preconditioner(oracle):
    """precond=1 (each sphere's own I/2 + K_PV + L inverted, right preconditioning) reaches the same
    solution with fewer iterations; its reported residual is the true residual of A mu = b; a batch
    gives bit for bit the problems solved alone."""
    cfg = cluster(20, n=8, p=8, gap=0.1)
    mob = make(cfg, SphereSTKMobMat)
    op = make(cfg)
    ref = oracle_op(oracle, cfg).solve_mob(cfg["force"], tol=1e-12)
    for prec in (PREC_FP64, PREC_MIXED):
        v0 = mob.solveMob(cfg["force"], tol=1e-10, precision=prec)
        it0 = mob.last_stats[0]["iterations"]
        v1 = mob.solveMob(cfg["force"], tol=1e-10, precision=prec, precond=1)
        st = mob.last_stats[0]
        assert st["status"] == 0 and st["iterations"] < it0
        assert rel(v1, ref["vel"]) < 1e-8 and rel(v1, v0) < 1e-8
        rho = rigid_density(op, cfg)
        mu = mob.getDensitySolution() - rho
        b = op.applyP2POP(rho, cId=-0.5, cSL=0.0, cTrac=-1.0)
        true = np.linalg.norm(b - op.apply(mu)) / np.linalg.norm(b)
        # MIXED: the last residual may be updated with the FP32 operator (r <- r - A32 d once r is below
        # 1e-4 |b|), whose relative error (~3e-6, 3xTF32 near contraction) bounds the difference
        assert true < 1e-10 and abs(true - st["relres"]) < 3e-11
    a = cluster(11, n=4, p=6)
    bb = cluster(12, n=7, p=8)
    cat = dict(centers=np.concatenate([a["centers"], bb["centers"]]), radii=np.concatenate([a["radii"], bb["radii"]]),
               orders=np.concatenate([a["orders"], bb["orders"]]), quats=np.concatenate([a["quats"], bb["quats"]]),
               problem=np.concatenate([np.zeros(4, np.int32), np.ones(7, np.int32)]))
    va = make(a, SphereSTKMobMat).solveMob(a["force"], tol=1e-10, precision=PREC_MIXED, precond=1)
    vb = make(bb, SphereSTKMobMat).solveMob(bb["force"], tol=1e-10, precision=PREC_MIXED, precond=1)
    v = make(cat, SphereSTKMobMat).solveMob(np.concatenate([a["force"], bb["force"]]), tol=1e-10,
                                            precision=PREC_MIXED, precond=1)
    assert np.array_equal(v[:24], va) and np.array_equal(v[24:], vb)


def test_multi_rhs_needs_one_problem():
    a = cluster(11, n=3, p=5)
    b = cluster(12, n=3, p=5)
    cat = dict(centers=np.concatenate([a["centers"], b["centers"]]), radii=np.concatenate([a["radii"], b["radii"]]),
               orders=np.concatenate([a["orders"], b["orders"]]), problem=np.array([0, 0, 0, 1, 1, 1], np.int32))
    with pytest.raises(SmobError):
        make(cat, SphereSTKMobMat).solveMobMulti(np.zeros((2, 36)))


def test_graphs_match_eager():
    """Captured Arnoldi blocks replay exactly the kernels the eager path launches."""
    cfg = cluster(16, n=5, p=7)
    for prec in (PREC_FP64, PREC_MIXED):
        g = make(cfg, SphereSTKMobMat)
        v_graph = g.solveMob(cfg["force"], tol=1e-10, precision=prec)
        v_graph2 = g.solveMob(cfg["force"], tol=1e-10, precision=prec)  # replay of the cached graphs
        g.set_graphs(False)
        v_eager = g.solveMob(cfg["force"], tol=1e-10, precision=prec)
        assert np.array_equal(v_graph, v_eager) and np.array_equal(v_graph2, v_eager)


def test_float_float_solve(oracle):
    """Restarted GMRES with the float-float far field throughout is FP64-accurate."""
    cfg = cluster(17, n=6, p=8)
    g = make(cfg, SphereSTKMobMat)
    ref = oracle_op(oracle, cfg).solve_mob(cfg["force"], tol=1e-12)
    vel = g.solveMob(cfg["force"], tol=1e-12, precision=PREC_FLOAT_FLOAT)
    assert g.last_stats[0]["status"] == 0 and g.last_stats[0]["operator_passes_fp32"] == 0
    assert rel(vel, ref["vel"]) < 1e-9


def test_mixed_with_near_singular_pairs(oracle):
    """Pairs closer than 0.1 radius are evaluated in FP64 inside the FP32 operator."""
    cfg = configs.small_cluster(seed=21, n=6, p=8, gap=0.05, quats=True)
    g = make(cfg, SphereSTKMobMat)
    t, s = g.near_pairs()
    gaps = np.linalg.norm(cfg["centers"][t] - cfg["centers"][s], axis=1) - cfg["radii"][t] - cfg["radii"][s]
    assert np.any(gaps < 0.1 * np.minimum(cfg["radii"][t], cfg["radii"][s]))
    o = oracle_op(oracle, cfg)
    x = np.random.default_rng(3).standard_normal(3 * g.n_points)
    assert rel(make(cfg).apply(x, precision=PREC_MIXED), o.apply(x)) < 2e-5
    ref = o.solve_mob(cfg["force"], tol=1e-12)
    vel = g.solveMob(cfg["force"], tol=1e-10, precision=PREC_MIXED)
    assert g.last_stats[0]["status"] == 0 and rel(vel, ref["vel"]) < 1e-6


def rigid_density(op, cfg):
    """rho = F/(4 pi a^2) + 3/(8 pi a^4) T x (a n) on every grid point (BIE/SphereSTKMobMat.cpp:174-192)."""
    n = op.getGridNorms()
    sid = np.repeat(np.arange(op.n_spheres), [(p + 1) * (2 * p + 2) for p in cfg["orders"]])
    a = np.asarray(cfg["radii"])[sid][:, None]
    F = np.asarray(cfg["force"]).reshape(-1, 6)[sid]
    return (F[:, :3] / (4 * np.pi * a * a) + 3 / (8 * np.pi * a ** 4) * np.cross(F[:, 3:], a * n)).reshape(-1)


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_reported_residual_is_true_residual(prec):
    """|b - A mu|/|b| recomputed independently with the FP64 operator matches the solver's report."""
    cfg = cluster(18, n=6, p=8, gap=0.1)
    mob = make(cfg, SphereSTKMobMat)
    op = make(cfg)
    mob.solveMob(cfg["force"], tol=1e-10, precision=prec)
    st = mob.last_stats[0]
    rho = rigid_density(op, cfg)
    mu = mob.getDensitySolution() - rho
    b = op.applyP2POP(rho, cId=-0.5, cSL=0.0, cTrac=-1.0)
    true = np.linalg.norm(b - op.apply(mu)) / np.linalg.norm(b)
    assert st["status"] == 0 and true < 1e-10
    assert abs(true - st["relres"]) < 3e-11  # the FP32-updated last residual (see the preconditioner test)


def test_isolated_sphere_drag_gpu():
    rng = np.random.default_rng(13)
    q = rng.standard_normal(4)
    g = SphereSTKMobMat([[1.0, 2.0, -3.0]], [0.8], [10], quats=q / np.linalg.norm(q), viscosity=1.7)
    F = rng.standard_normal(6)
    v = g.solveMob(F)
    assert np.allclose(v[:3], F[:3] / (6 * np.pi * 1.7 * 0.8), rtol=1e-11)
    assert np.allclose(v[3:], F[3:] / (8 * np.pi * 1.7 * 0.8 ** 3), rtol=1e-11)
    assert g.last_stats[0]["iterations"] == 0


def test_determinism_and_warm_start():
    cfg = cluster(14, n=5, p=7)
    g = make(cfg, SphereSTKMobMat)
    v1 = g.solveMob(cfg["force"], tol=1e-10)
    it1 = g.last_stats[0]["iterations"]
    v2 = make(cfg, SphereSTKMobMat).solveMob(cfg["force"], tol=1e-10)
    assert np.array_equal(v1, v2)
    v3 = g.solveMob(cfg["force"], tol=1e-10, warm_start=True)
    assert g.last_stats[0]["iterations"] < it1
    assert rel(v3, v1) < 1e-9


def test_error_paths():
    cfg = cluster(15, n=3, p=5)
    g = make(cfg, SphereSTKMobMat)
    f = cfg["force"].copy()
    f[2] = np.nan
    with pytest.raises(SmobError) as e:
        g.solveMob(f)
    assert e.value.code == 5
    with pytest.raises(SmobError) as e:
        SphereSTKSHOperator([[0, 0, 0], [1.5, 0, 0]], [1, 1], [6, 6])
    assert e.value.code == 1
    v = g.solveMob(np.zeros(18))
    assert np.all(v == 0) and g.last_stats[0]["iterations"] == 0
    v = g.solveMob(cfg["force"], tol=1e-14, max_iters=3, raise_on_not_converged=False)
    assert g.last_stats[0]["status"] == 4 and g.last_stats[0]["iterations"] == 3


@pytest.mark.parametrize("orders", [(8, 8, 8, 8, 8), (6, 12, 16, 24, 32)])
def test_near_field_tensor_cores(oracle, orders):
    """The FP32 near field as a tcgen05 TF32 GEMM (3xTF32 split) against the oracle's spectral near
    field (FP32 tolerance 2e-5) and against the SIMT FP32 kernel (same contraction, FP32 multiply-adds),
    traction and single layer, with near pairs between spheres of different orders (different K per
    source, padded chunks) and random orientations."""
    cfg = configs.small_cluster(seed=41, n=5, p=8, gap=0.15, quats=True)
    cfg["orders"] = np.asarray(orders)
    g = make(cfg)
    assert g.n_near_pairs >= 4
    o = oracle_op(oracle, cfg)
    x = np.random.default_rng(41).standard_normal(3 * g.n_points)
    for c_sl, c_tr in ((0.0, 1.0), (1.0, 0.0), (0.4, -1.1)):
        ref = g.near_field(x, c_sl, c_tr, precision=PREC_FP64)
        far = o.far_traction(x, c_tr) + o.far_sl(x, c_sl) + o.near_correction(x, c_sl, c_tr)
        assert rel(g.far_field(x, c_sl, c_tr, precision=PREC_FP64) + ref, far) < 1e-11
        tc = g.near_field(x, c_sl, c_tr, precision=PREC_MIXED)
        g.set_near_tc(False)
        simt = g.near_field(x, c_sl, c_tr, precision=PREC_MIXED)
        g.set_near_tc(True)
        assert rel(tc, ref) < 2e-5 and rel(simt, ref) < 2e-5, (rel(tc, ref), rel(simt, ref))
        assert rel(tc, simt) < 2e-5
        # deterministic: the same call gives the same bits
        assert np.array_equal(tc, g.near_field(x, c_sl, c_tr, precision=PREC_MIXED))


def test_near_tensor_cores_in_batches_and_solves(oracle):
    """Batched problems (every target point has near pairs, many CTAs) and a mixed solve with the
    tensor-core near field: each problem equals its solve alone bit for bit, and the solve matches the
    oracle."""
    a = configs.small_cluster(seed=43, n=6, p=10, gap=0.2, quats=True)
    b = configs.small_cluster(seed=44, n=4, p=12, gap=0.2, quats=True)
    centers = np.vstack([a["centers"], b["centers"] + 100.0])
    radii = np.concatenate([a["radii"], b["radii"]])
    orders = np.concatenate([a["orders"], b["orders"]])
    quats = np.vstack([a["quats"], b["quats"]])
    prob = np.array([0] * 6 + [1] * 4, dtype=np.int32)
    F = np.concatenate([a["force"], b["force"]])
    mob = SphereSTKMobMat(centers, radii, orders, quats=quats, problem=prob)
    v = mob.solveMob(F, tol=1e-10, precision=PREC_MIXED)
    alone = SphereSTKMobMat(a["centers"], a["radii"], a["orders"], quats=a["quats"])
    assert np.array_equal(alone.solveMob(a["force"], tol=1e-10, precision=PREC_MIXED), v[:36])
    ref = oracle_op(oracle, a).solve_mob(a["force"], tol=1e-12)
    assert rel(v[:36], ref["vel"]) < 1e-8
    mob.set_near_tc(False)
    assert rel(mob.solveMob(F, tol=1e-10, precision=PREC_MIXED), v) < 1e-8


@pytest.mark.parametrize("orders", [(8, 8, 8, 8, 8), (6, 12, 16, 24, 32)])
def test_sphere_operator_tensor_cores(oracle, orders):
    """The FP32 sphere operator with its Legendre stage as tcgen05 TF32 GEMMs (forward, self multipliers,
    inverse per order and m) against the oracle (FP32 tolerance 2e-5) and against the SIMT FP32 kernel,
    for the traction (principal value), the single layer and the identity / L terms, orders up to 32."""
    cfg = configs.small_cluster(seed=45, n=5, p=8, gap=0.3, quats=True)
    cfg["orders"] = np.asarray(orders)
    g = make(cfg)
    o = oracle_op(oracle, cfg)
    x = np.random.default_rng(45).standard_normal(3 * g.n_points)
    assert not g.sphere_tc()  # the SIMT operator is the default (faster at these sizes)
    for coefs in ((0.5, 0.0, 1.0), (0.0, 1.0, 0.0), (0.2, 0.8, -0.4)):
        ref = o.apply_p2p(x, *coefs)
        g.set_sphere_tc(True)
        tc = g.applyP2POP(x, None, *coefs, precision=PREC_MIXED)
        g.set_sphere_tc(False)
        simt = g.applyP2POP(x, None, *coefs, precision=PREC_MIXED)
        assert rel(tc, ref) < 2e-5 and rel(simt, ref) < 2e-5, (coefs, rel(tc, ref), rel(simt, ref))
        assert rel(tc, simt) < 2e-5
    g.set_sphere_tc(True)
    assert rel(g.apply(x, precision=PREC_MIXED), o.apply(x)) < 2e-5


def test_sphere_tensor_cores_several_tiles():
    """Cfg 2 (64 spheres of one order: four tiles of up to 21 spheres): the FP32 operator with the
    tensor-core Legendre stage equals the SIMT one to FP32 rounding, and a mixed solve with the block
    preconditioner (the third self operator) matches the FP64 solve."""
    cfg = configs.cfg2()
    g = make(cfg, SphereSTKMobMat)
    x = np.random.default_rng(46).standard_normal(3 * g.n_points)
    ref = g.apply(x, precision=PREC_FP64)
    simt = g.apply(x, precision=PREC_MIXED)
    g.set_sphere_tc(True)
    tc = g.apply(x, precision=PREC_MIXED)
    assert rel(tc, ref) < 2e-5 and rel(tc, simt) < 1e-5
    v = g.solveMob(cfg["force"], tol=1e-10, precision=PREC_MIXED, precond=1)
    assert g.last_stats[0]["status"] == 0
    assert rel(v, g.solveMob(cfg["force"], tol=1e-11, precision=PREC_FP64)) < 1e-8


@pytest.mark.parametrize("orders", [(8, 8, 8, 8, 8), (6, 12, 16, 24, 32)])
def test_near_field_float_float(oracle, orders):
    """The near field of the high-precision passes in float-float on the FP32 pipes (k_near_eval_df:
    recurrence and contraction as float pairs, FP64 frame and assembly) against the FP64 kernel and the
    oracle's decomposition, traction and single layer, orders up to 32 (sets staged or read from L2)."""
    cfg = configs.small_cluster(seed=47, n=5, p=8, gap=0.05, quats=True)
    cfg["orders"] = np.asarray(orders)
    g = make(cfg)
    g.set_far_compression(1e-5, 1e-10)  # the far-field part of the 1e-11 bound below
    o = oracle_op(oracle, cfg)
    x = np.random.default_rng(47).standard_normal(3 * g.n_points)
    for c_sl, c_tr in ((0.0, 1.0), (1.0, 0.0), (0.3, -0.9)):
        ref = g.near_field(x, c_sl, c_tr, precision=PREC_FP64)
        df = g.near_field(x, c_sl, c_tr, precision=PREC_FLOAT_FLOAT)
        assert rel(df, ref) < 1e-12, rel(df, ref)
        full = o.far_traction(x, c_tr) + o.far_sl(x, c_sl) + o.near_correction(x, c_sl, c_tr)
        assert rel(g.far_field(x, c_sl, c_tr, precision=PREC_FLOAT_FLOAT) + df, full) < 1e-11
