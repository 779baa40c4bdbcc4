"""FP32 far field from coarse equivalent sources for well-separated sphere pairs: accuracy against
the direct sum and the FP64 oracle, tolerance control, solves that equal the direct-sum solves to
the tolerance, and batches and geometry updates."""
import numpy as np
import pytest

from spheresimulator_gb300 import PREC_FLOAT_FLOAT, PREC_FP64, PREC_MIXED, SphereSTKMobMat, SphereSTKSHOperator, configs

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _spread(seed=0, n=24, p=12, box=22.0):
    """Spheres spread in a box, so most pairs are well separated."""
    rng = np.random.default_rng(seed)
    radii = rng.uniform(0.8, 1.2, n)
    return dict(centers=configs.rsa(rng, n, radii, box, 0.3), radii=radii, orders=np.full(n, p))


def test_far_field_matches_direct_sum():
    c = _spread()
    g = SphereSTKSHOperator(c["centers"], c["radii"], c["orders"])
    eps, pts, ent = g.far_compression_info()
    assert eps == 1e-5 and ent > 0 and pts > 0
    x = np.random.default_rng(1).standard_normal(3 * g.n_points)
    fp64 = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_FP64)
    comp = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_MIXED)
    g.set_far_compression(0)
    assert g.far_compression_info()[1:] == (0, 0) and g.far_compression_info(hp=True)[2] > 0
    direct = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_MIXED)
    # the compression error stays a few times the FP32 rounding level, well below the 1e-5 the
    # inner solves stop at
    assert _rel(direct, fp64) < 2e-5
    assert _rel(comp, fp64) < 2e-5
    assert _rel(comp, direct) < 1e-5


def test_float_float_far_field_with_coarse_sources():
    """The float-float set (tolerance 1e-10) against the direct float-float sum and the FP64 sum."""
    c = _spread(seed=9, n=24, p=12, box=26.0)
    g = SphereSTKSHOperator(c["centers"], c["radii"], c["orders"])
    eps_hp, pts, ent = g.far_compression_info(hp=True)
    assert eps_hp == 1e-9 and ent > 0 and pts > 0  # the default set
    x = np.random.default_rng(9).standard_normal(3 * g.n_points)
    fp64 = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_FP64)
    assert _rel(g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_FLOAT_FLOAT), fp64) < 1e-9
    g.set_far_compression(1e-5, 1e-10)  # the bounds below are those of a 1e-10 set
    comp = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_FLOAT_FLOAT)
    g.set_far_compression(1e-7, 0)
    assert g.far_compression_info(hp=True)[1:] == (0, 0)
    direct = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_FLOAT_FLOAT)
    # float-float sums carry ~1e-12 relative rounding on this size; the coarse sources add below 1e-10
    assert _rel(direct, fp64) < 1e-11
    assert _rel(comp, fp64) < 1e-10 and _rel(comp, direct) < 1e-10
    g.set_far_compression(1e-6, 1e-12)
    assert _rel(g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_FLOAT_FLOAT), direct) < 2e-11


def test_tolerance_controls_the_error():
    c = _spread(seed=2)
    g = SphereSTKSHOperator(c["centers"], c["radii"], c["orders"])
    x = np.random.default_rng(2).standard_normal(3 * g.n_points)
    ref = g.far_field(x, cTrac=1.0, precision=PREC_FP64)
    errs = []
    for eps in (1e-3 * 0.99, 1e-5, 1e-8):
        g.set_far_compression(eps)
        assert g.far_compression_info()[2] > 0
        errs.append(_rel(g.far_field(x, cTrac=1.0, precision=PREC_MIXED), ref))
    # the loose tolerance shows; the tight one is at the FP32 rounding level of the direct sum
    assert errs[0] > 3 * errs[2] and errs[0] < 1e-3 and errs[2] < 2e-6


@pytest.mark.parametrize("precond", [0, 1])
def test_mixed_solve_equals_direct_sum_solve(precond):
    c = _spread(seed=3, n=20, p=10, box=16.0)
    F = np.random.default_rng(3).standard_normal(6 * 20)
    g = SphereSTKMobMat(c["centers"], c["radii"], c["orders"])
    assert g.far_compression_info()[2] > 0
    v = g.solveMob(F, tol=1e-10, precision=PREC_MIXED, precond=precond)
    s = g.last_stats[0]
    d = SphereSTKMobMat(c["centers"], c["radii"], c["orders"])
    d.set_far_compression(0, 0)
    vd = d.solveMob(F, tol=1e-10, precision=PREC_MIXED, precond=precond)
    ref = d.solveMob(F, tol=1e-11, precision=PREC_FP64)
    assert s["status"] == 0 and s["relres"] < 1e-10
    assert _rel(v, vd) < 1e-9 and _rel(v, ref) < 1e-9
    assert s["iterations"] <= d.last_stats[0]["iterations"] + 2


def test_batch_equals_problems_alone_and_update_equals_fresh():
    a, b = _spread(seed=4, n=10, p=8, box=14.0), _spread(seed=5, n=14, p=8, box=16.0)
    centers = np.vstack([a["centers"], b["centers"] + 200.0])
    radii = np.concatenate([a["radii"], b["radii"]])
    orders = np.concatenate([a["orders"], b["orders"]])
    prob = np.array([0] * 10 + [1] * 14, dtype=np.int32)
    F = np.random.default_rng(6).standard_normal(6 * 24)
    g = SphereSTKMobMat(centers, radii, orders, problem=prob)
    v = g.solveMob(F, tol=1e-10, precision=PREC_MIXED)
    for sl, pts, cc, rr, oo in ((slice(0, 60), slice(0, 10), a["centers"], a["radii"], a["orders"]),
                                (slice(60, 144), slice(10, 24), b["centers"] + 200.0, b["radii"], b["orders"])):
        alone = SphereSTKMobMat(cc, rr, oo)
        assert np.array_equal(alone.solveMob(F[sl], tol=1e-10, precision=PREC_MIXED), v[sl])
    moved = centers + np.random.default_rng(7).uniform(-0.05, 0.05, centers.shape)
    g.set_geometry(moved)
    fresh = SphereSTKMobMat(moved, radii, orders, problem=prob)
    assert g.far_compression_info() == fresh.far_compression_info()
    assert np.array_equal(g.solveMob(F, tol=1e-10, precision=PREC_MIXED),
                          fresh.solveMob(F, tol=1e-10, precision=PREC_MIXED))


def test_invalid_tolerance_is_rejected():
    c = _spread(seed=8, n=3, p=4)
    g = SphereSTKSHOperator(c["centers"], c["radii"], c["orders"])
    from spheresimulator_gb300 import SmobError
    with pytest.raises(SmobError):
        g.set_far_compression(0.1)
    with pytest.raises(SmobError):
        g.set_far_compression(float("nan"))
    with pytest.raises(SmobError):
        g.set_far_compression(1e-7, 1e-8)


def test_high_orders_use_fine_coarse_levels():
    """Orders up to 32 spread apart: coarse orders up to 28 (several shared-memory tiles per coarse
    sphere, the largest maps); the far field and a mixed solve match the direct sum and the FP64 solve."""
    rng = np.random.default_rng(21)
    centers = np.array([[0.0, 0, 0], [9.0, 0, 0], [0, 11.0, 0], [0, 0, 13.0], [8.0, 9.0, 7.0]])
    radii = np.array([1.0, 1.1, 0.9, 1.0, 1.2])
    orders = np.array([32, 24, 20, 16, 28])
    g = SphereSTKMobMat(centers, radii, orders)
    assert g.far_compression_info()[2] > 0 and g.far_compression_info(hp=True)[2] > 0
    x = rng.standard_normal(3 * g.n_points)
    fp64 = g.far_field(x, cSL=0.4, cTrac=1.0, precision=PREC_FP64)
    assert _rel(g.far_field(x, cSL=0.4, cTrac=1.0, precision=PREC_MIXED), fp64) < 2e-5
    assert _rel(g.far_field(x, cSL=0.4, cTrac=1.0, precision=PREC_FLOAT_FLOAT), fp64) < 1e-10
    F = rng.standard_normal(30)
    v = g.solveMob(F, tol=1e-10, precision=PREC_MIXED)
    assert g.last_stats[0]["status"] == 0
    assert _rel(v, g.solveMob(F, tol=1e-12, precision=PREC_FP64)) < 1e-9


def test_far_pairs_replay():
    """The host replay of the kernels' per-CTA choices: the direct count is every far pair, the
    evaluated count drops with coarse sources and equals the direct count without them."""
    c = _spread(seed=12, n=16, p=10, box=18.0)
    g = SphereSTKSHOperator(c["centers"], c["radii"], c["orders"])
    ng = (c["orders"] + 1) * (2 * c["orders"] + 2)
    t, s = g.near_pairs()
    direct = int(ng.sum() ** 2 - (ng ** 2).sum() - (ng[t] * ng[s]).sum())
    d, e, macs = g.far_pairs()
    assert d == direct and 0 < e < d and macs > 0
    # the fused float-float pass's set: the same direct pairs, at most as many evaluated
    dh, eh, mh = g.far_pairs(hp=True)
    assert dh == direct and 0 < eh <= dh
    g.set_far_compression(0, 0)
    d0, e0, m0 = g.far_pairs()
    assert d0 == direct and e0 == direct and m0 == 0
    assert g.far_pairs(hp=True)[:2] == (direct, direct)


def test_coarse_targets_match_direct_sum():
    """Coarse targets (far fields at a target sphere's coarse nodes, interpolated to its grid) on a
    spread geometry: fewer evaluated pairs, the same accuracy class as the sources alone, and at a
    tight tolerance the FP32 rounding level of the direct sum."""
    c = _spread(seed=31, n=40, p=14, box=40.0)
    g = SphereSTKSHOperator(c["centers"], c["radii"], c["orders"])
    x = np.random.default_rng(31).standard_normal(3 * g.n_points)
    fp64 = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_FP64)
    d_on, e_on, _ = g.far_pairs()
    on = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_MIXED)
    g.set_far_coarse_targets(False)
    d_off, e_off, _ = g.far_pairs()
    off = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_MIXED)
    assert d_on == d_off and e_on < 0.7 * e_off
    assert _rel(off, fp64) < 2e-5 and _rel(on, fp64) < 2e-5
    for trac, sl in ((1.0, 0.0), (0.0, 1.0)):
        ref = g.far_field(x, cSL=sl, cTrac=trac, precision=PREC_FP64)
        g.set_far_coarse_targets(True)
        g.set_far_compression(1e-8)
        assert _rel(g.far_field(x, cSL=sl, cTrac=trac, precision=PREC_MIXED), ref) < 2e-6
        g.set_far_compression(1e-5)
        assert _rel(g.far_field(x, cSL=sl, cTrac=trac, precision=PREC_MIXED), ref) < 2e-5
        g.set_far_coarse_targets(False)


def test_coarse_targets_in_batches_and_mixed_solves():
    """Coarse targets inside a batch of two problems: each problem's solve equals its solve alone bit
    for bit, and equals the solve without coarse targets to the solve tolerance."""
    a, b = _spread(seed=32, n=16, p=10, box=30.0), _spread(seed=33, n=12, p=12, box=30.0)
    centers = np.vstack([a["centers"], b["centers"] + 300.0])
    radii = np.concatenate([a["radii"], b["radii"]])
    orders = np.concatenate([a["orders"], b["orders"]])
    prob = np.array([0] * 16 + [1] * 12, dtype=np.int32)
    F = np.random.default_rng(34).standard_normal(6 * 28)
    g = SphereSTKMobMat(centers, radii, orders, problem=prob)
    v = g.solveMob(F, tol=1e-10, precision=PREC_MIXED)
    assert all(s["status"] == 0 for s in g.last_stats)
    alone = SphereSTKMobMat(a["centers"], a["radii"], a["orders"])
    assert np.array_equal(alone.solveMob(F[:96], tol=1e-10, precision=PREC_MIXED), v[:96])
    g.set_far_coarse_targets(False)
    assert _rel(g.solveMob(F, tol=1e-10, precision=PREC_MIXED), v) < 1e-9


def test_float_float_coarse_targets():
    """The fused float-float pass with coarse targets (its 1e-10 set): against the same pass with grid
    targets and the FP64 sum, and a mixed solve against the FP64 solve."""
    c = _spread(seed=35, n=16, p=16, box=60.0)
    g = SphereSTKMobMat(c["centers"], c["radii"], c["orders"])
    g.set_far_compression(1e-5, 1e-10)
    x = np.random.default_rng(35).standard_normal(3 * g.n_points)
    fp64 = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_FP64)
    on = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_FLOAT_FLOAT)
    F = np.random.default_rng(36).standard_normal(6 * 16)
    v_on = g.solveMob(F, tol=1e-10, precision=PREC_MIXED)
    assert g.last_stats[0]["status"] == 0
    g.set_far_coarse_targets(False)
    off = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_FLOAT_FLOAT)
    assert _rel(off, fp64) < 1e-10 and _rel(on, fp64) < 1e-10 and _rel(on, off) < 1e-10
    ref = g.solveMob(F, tol=1e-12, precision=PREC_FP64)
    assert _rel(v_on, ref) < 1e-9


def test_coarse_strengths_on_tensor_cores():
    """The FP32 coarse strengths and coarse-target interpolation as 3xTF32 GEMMs on the tensor cores
    (k_coarse_src_tc, k_ct_interp_tc) against the SIMT GEMMs and the FP64 sum: FP32 accuracy; a batch's
    problems equal the problems alone bit for bit."""
    c = _spread(seed=51, n=40, p=12, box=40.0)
    g = SphereSTKSHOperator(c["centers"], c["radii"], c["orders"])
    assert g.coarse_tc() and g.far_compression_info()[2] > 0
    x = np.random.default_rng(51).standard_normal(3 * g.n_points)
    fp64 = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_FP64)
    tc = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_MIXED)
    g.set_coarse_tc(False)
    simt = g.far_field(x, cSL=0.5, cTrac=1.0, precision=PREC_MIXED)
    e_tc, e_simt = _rel(tc, fp64), _rel(simt, fp64)
    print("coarse strengths: tensor cores %.3g, SIMT %.3g against FP64; between them %.3g" % (e_tc, e_simt,
                                                                                           _rel(tc, simt)))
    assert e_tc < 2e-5 and e_simt < 2e-5
    # 3xTF32 products (2^-22 relative each) instead of FP32 ones (2^-24): the same order as the
    # compression's own error here
    assert e_tc < max(2 * e_simt, 2e-6) and _rel(tc, simt) < 5e-6
    # batched with a second problem: the first problem's solve is the same bits as alone
    b = _spread(seed=52, n=20, p=16, box=30.0)
    centers = np.vstack([c["centers"], b["centers"] + 500.0])
    radii = np.concatenate([c["radii"], b["radii"]])
    orders = np.concatenate([c["orders"], b["orders"]])
    prob = np.array([0] * 40 + [1] * 20, dtype=np.int32)
    F = np.random.default_rng(53).standard_normal(6 * 60)
    both = SphereSTKMobMat(centers, radii, orders, problem=prob)
    alone = SphereSTKMobMat(c["centers"], c["radii"], c["orders"])
    v = both.solveMob(F, tol=1e-8, precision=PREC_MIXED)
    assert np.array_equal(alone.solveMob(F[:240], tol=1e-8, precision=PREC_MIXED), v[:240])


def test_batch_of_compressed_and_uncompressed_problems():
    """A problem without well-separated pairs (no coarse level anywhere) batched with one that has
    them: it is solved alone and in the batch with the same far-field kernels and gives the same bits
    (the coarse-target machinery is built whenever it is on, whatever the data)."""
    # three spheres whose pairs are all far pairs (centres 3.2 and 4.5 apart, beyond 1.5 (a_s + a_t))
    # but too close for any coarse order below p = 8
    tight = dict(centers=np.array([[0.0, 0.0, 0.0], [3.2, 0.0, 0.0], [0.0, 3.2, 0.0]]), radii=np.ones(3),
                 orders=np.full(3, 8))
    far = _spread(seed=62, n=16, p=12, box=36.0)
    alone = SphereSTKMobMat(tight["centers"], tight["radii"], tight["orders"])
    assert alone.far_compression_info()[2] == 0  # no coarse entry
    centers = np.vstack([tight["centers"], far["centers"] + 400.0])
    radii = np.concatenate([tight["radii"], far["radii"]])
    orders = np.concatenate([tight["orders"], far["orders"]])
    prob = np.array([0] * 3 + [1] * 16, dtype=np.int32)
    both = SphereSTKMobMat(centers, radii, orders, problem=prob)
    assert both.far_compression_info()[2] > 0
    F = np.random.default_rng(63).standard_normal(6 * 19)
    for prec in (PREC_MIXED, PREC_FLOAT_FLOAT):
        v = both.solveMob(F, tol=1e-10, precision=prec)
        assert np.array_equal(alone.solveMob(F[:18], tol=1e-10, precision=prec), v[:18]), prec
