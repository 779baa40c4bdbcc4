"""The mathematics of the coarse equivalent sources and coarse targets, restated in numpy (CPU): for
a sphere's grid sources f_j, equivalent sources f_e = W_pe K_pe f on the order-pe grid of the same
sphere, with K_pe(k, j) = sum_{n <= pe} (2n+1)/(4 pi) P_n(nu_k . nu_j), reproduce the sphere's Stokes
single-layer and traction far fields to ~(a / r_min)^(pe+1) relative; the library's level rule
pe >= log(eps) / log(a / r_min) + 1 keeps the error near eps (below 3.4 eps over p = 8-24,
a / r_min = 0.05-0.4, both kernels and eps = 1e-5-1e-10; below eps with a margin of 2). On the target
side the transposed map interpolates a field sampled at a sphere's order-pt nodes to its grid, exact
for degree <= pt; with the target rule's margin of 2 both sides together stay within 10 eps."""
import numpy as np
from numpy.polynomial.legendre import leggauss, legval


def grid(p):
    x, w = leggauss(p + 1)
    x, w = x[::-1], w[::-1]  # rings north to south, as the sphere grids
    nphi = 2 * p + 2
    phi = 2 * np.pi * np.arange(nphi) / nphi
    ct = np.repeat(x, nphi)
    st = np.sqrt(1 - ct ** 2)
    ph = np.tile(phi, p + 1)
    return np.stack([st * np.cos(ph), st * np.sin(ph), ct], 1), np.repeat(w * 2 * np.pi / nphi, nphi)


def coarse_map(p, pe):
    nf, _ = grid(p)
    nc, wc = grid(pe)
    kern = legval(np.clip(nc @ nf.T, -1, 1), [(2 * n + 1) / (4 * np.pi) for n in range(pe + 1)])
    return wc[:, None] * kern


def far(trg, nrm, src, f, trac):
    r = trg[:, None, :] - src[None, :, :]
    ri = 1 / np.sqrt((r ** 2).sum(-1))
    rf = (r * f[None]).sum(-1)
    if trac:
        rn = (r * nrm[:, None, :]).sum(-1)
        return ((rf * rn * ri ** 5)[..., None] * r).sum(1)
    return (f[None] * ri[..., None] + (rf * ri ** 3)[..., None] * r).sum(1)


def test_map_reproduces_low_degrees_exactly():
    """A constant density maps to the coarse quadrature weights (total strength kept), and the map is
    exact on fields of degree <= pe (the coarse samples of a degree-1 field)."""
    p, pe = 10, 5
    nf, wf = grid(p)
    nc, wc = grid(pe)
    M = coarse_map(p, pe)
    assert np.allclose(M @ wf, wc, rtol=0, atol=1e-14)
    lin = nf @ np.array([0.3, -1.2, 0.7])  # degree 1
    assert np.allclose(M @ (wf * lin), wc * (nc @ np.array([0.3, -1.2, 0.7])), atol=1e-13)


def test_far_field_error_follows_the_level_rule():
    rng = np.random.default_rng(0)
    p = 12
    nf, wf = grid(p)
    f = wf[:, None] * rng.standard_normal((len(nf), 3))
    tg, _ = grid(4)
    for trac in (True, False):
        for R, eps in ((5.0, 1e-5), (8.0, 1e-7), (12.0, 1e-9)):
            d = rng.standard_normal(3)
            d /= np.linalg.norm(d)
            trg = R * d + tg
            ref = far(trg, tg, nf, f, trac)
            ratio = 1.0 / (R - 1.0)
            pe = int(np.ceil(np.log(eps) / np.log(ratio) + 1))
            if pe >= p:
                continue
            nc, _ = grid(pe)
            val = far(trg, tg, nc, coarse_map(p, pe) @ f, trac)
            err = np.abs(val - ref).max() / np.abs(ref).max()
            assert err < 4 * eps, (trac, R, pe, err)
            # three orders coarser is worse, so the rule does not overshoot by orders
            if pe > 3:
                nc2, _ = grid(pe - 3)
                worse = np.abs(far(trg, tg, nc2, coarse_map(p, pe - 3) @ f, trac) - ref).max() / np.abs(ref).max()
                assert worse > err


def test_target_interpolation_is_exact_to_degree_pe():
    """The transposed map interpolates a field sampled at the order-pe nodes to the order-p grid:
    u(nu_j) = sum_k w_k K_pe(nu_j . nu_k) u(nu_k), exact for degree <= pe."""
    p, pe = 12, 5
    nf, _ = grid(p)
    nc, _ = grid(pe)
    M = coarse_map(p, pe)
    for field in (lambda n: n @ np.array([0.3, -1.2, 0.7]),
                  lambda n: n[:, 0] * n[:, 1] * n[:, 2] ** 3 - 0.4 * n[:, 2] ** 5):  # degrees 1 and 5
        assert np.allclose(M.T @ field(nc), field(nf), atol=1e-13)


def test_coarse_targets_and_sources_follow_the_level_rules():
    """Both sides compressed: the far field of the source sphere's coarse sources (level from
    a_s / (d - a_t), margin 1) at the target sphere's coarse nodes (level from a_t / (d - a_s),
    margin 2: the traction's target normal adds a degree), interpolated to the target grid, stays
    within 10 eps of the direct sum relative to the pair's largest value."""
    rng = np.random.default_rng(5)
    ladder = (3, 4, 5, 6, 8, 10, 12, 14)

    def level(ratio, eps, p, margin):
        need = np.log(eps) / np.log(ratio) + margin
        for pe in ladder:
            if pe >= p:
                return None
            if pe >= need:
                return pe
        return None

    p = 16
    nf, wf = grid(p)
    checked = 0
    for _ in range(12):
        at, a_s = rng.uniform(0.8, 1.2, 2)
        d = rng.uniform(1.5 * (at + a_s), 14.0)
        u = rng.standard_normal(3)
        u /= np.linalg.norm(u)
        f = (wf * a_s ** 2)[:, None] * rng.standard_normal((len(nf), 3))
        for eps in (1e-5, 1e-10):
            lt = level(at / (d - a_s), eps, p, 2.0)
            if lt is None:
                continue
            ls = level(a_s / (d - at), eps, p, 1.0)
            src, fs = (d * u + a_s * nf, f) if ls is None else (d * u + a_s * grid(ls)[0], coarse_map(p, ls) @ f)
            nc, _ = grid(lt)
            for trac in (True, False):
                ref = far(at * nf, nf, d * u + a_s * nf, f, trac)
                val = coarse_map(p, lt).T @ far(at * nc, nc, src, fs, trac)
                assert np.abs(val - ref).max() / np.abs(ref).max() < 10 * eps, (trac, d, eps, lt, ls)
                checked += 1
    assert checked > 10
