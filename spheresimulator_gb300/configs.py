"""Seeded synthetic workloads for the five benchmark configurations of the mobility solve.

The reference ships no datasets; these generators produce sphere packings with the stated
sizes and distributions (random sequential addition, RSA) and N(0,1) forces/torques.

  cfg1  2 spheres, a=1, centres (0,0,0),(3,0,0), p=8, identity orientations, GMRES to 1e-10
  cfg2  64 spheres, a=1, RSA in a box of side 20 (min surface gap 0.1), p=16, GMRES(50) to 1e-10
  cfg3  1024 spheres, a ~ U[0.8,1.2], RSA in a box of side 40 (min gap 0.05), p=16, 1e-8
  cfg4  256 independent problems, N ~ U{2..128}, p ~ U{8,12,16}, a=1, box side 4 N^(1/3), gap 0.1
  cfg5  request stream: N log-uniform in [4,2048], p ~ U{8,12,16,24}, a ~ U[0.9,1.1], gap 0.05,
        box side 4 N^(1/3), tolerance 1e-6 or 1e-8 (50/50), Poisson arrivals at rate lam
"""
import numpy as np


def rsa(rng, n, radii, box, min_gap, max_tries=2000000):
    """Random sequential addition of spheres with the given radii inside [0, box]^3 (sphere fully
    inside the box); a proposal is rejected if any surface gap to a placed sphere is < min_gap."""
    radii = np.asarray(radii, dtype=np.float64)
    centers = np.zeros((n, 3))
    placed = 0
    tries = 0
    while placed < n:
        if tries > max_tries:
            raise RuntimeError("RSA could not place %d spheres in box %.3g" % (n, box))
        a = radii[placed]
        c = rng.uniform(a, box - a, size=3)
        tries += 1
        if placed:
            d = np.sqrt(((centers[:placed] - c) ** 2).sum(1))
            if np.any(d - radii[:placed] - a < min_gap):
                continue
        centers[placed] = c
        placed += 1
    return centers


def forces(rng, n):
    return rng.standard_normal(6 * n)


def cfg1(seed=1):
    rng = np.random.default_rng(seed)
    return dict(name="cfg1", centers=np.array([[0.0, 0, 0], [3.0, 0, 0]]), radii=np.ones(2), orders=np.full(2, 8),
                quats=None, force=forces(rng, 2), tol=1e-10, restart=50)


def cfg2(seed=2, p=16, n=64, box=20.0, gap=0.1):
    rng = np.random.default_rng(seed)
    radii = np.ones(n)
    c = rsa(rng, n, radii, box, gap)
    return dict(name="cfg2", centers=c, radii=radii, orders=np.full(n, p), quats=None, force=forces(rng, n),
                tol=1e-10, restart=50)


def cfg3(seed=3, p=16, n=1024, box=40.0, gap=0.05):
    rng = np.random.default_rng(seed)
    radii = rng.uniform(0.8, 1.2, n)
    c = rsa(rng, n, radii, box, gap)
    return dict(name="cfg3", centers=c, radii=radii, orders=np.full(n, p), quats=None, force=forces(rng, n),
                tol=1e-8, restart=50)


def _problem(rng, n, p, radii, gap):
    box = 4.0 * n ** (1.0 / 3.0)
    c = rsa(rng, n, radii, box, gap)
    return c


def cfg4(seed=4, n_problems=256, nmin=2, nmax=128, orders=(8, 12, 16), gap=0.1):
    """Batch of independent problems, concatenated with a problem id per sphere."""
    rng = np.random.default_rng(seed)
    cs, rs, ps, pid, fs = [], [], [], [], []
    for k in range(n_problems):
        n = int(rng.integers(nmin, nmax + 1))
        p = int(rng.choice(orders))
        r = np.ones(n)
        cs.append(_problem(rng, n, p, r, gap))
        rs.append(r)
        ps.append(np.full(n, p))
        pid.append(np.full(n, k))
        fs.append(forces(rng, n))
    return dict(name="cfg4", centers=np.concatenate(cs), radii=np.concatenate(rs), orders=np.concatenate(ps),
                problem=np.concatenate(pid), quats=None, force=np.concatenate(fs), tol=1e-8, restart=50)


def cfg5_request(rng, nmin=4, nmax=2048, orders=(8, 12, 16, 24), gap=0.05):
    n = int(np.round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
    p = int(rng.choice(orders))
    r = rng.uniform(0.9, 1.1, n)
    c = _problem(rng, n, p, r, gap)
    tol = 1e-6 if rng.random() < 0.5 else 1e-8
    return dict(centers=c, radii=r, orders=np.full(n, p), force=forces(rng, n), tol=tol, box=4.0 * n ** (1 / 3))


def cfg5_stream(seed=5, n_requests=64, rate=2.0, **kw):
    """Poisson arrivals (exponential inter-arrival times, mean 1/rate seconds)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate)
        req = cfg5_request(rng, **kw)
        req["arrival"] = t
        req["id"] = i
        out.append(req)
    return out


def small_cluster(seed=0, n=4, p=6, gap=0.3, radius_range=(0.8, 1.2), quats=False):
    """A small test cluster with near pairs (centre distance < 1.5 (a_s + a_t))."""
    rng = np.random.default_rng(seed)
    radii = rng.uniform(*radius_range, n)
    box = 2.2 * n ** (1 / 3) * radii.max() + 2
    c = rsa(rng, n, radii, box, gap)
    q = None
    if quats:
        q = rng.standard_normal((n, 4))
        q /= np.linalg.norm(q, axis=1)[:, None]
    return dict(name="cluster", centers=c, radii=radii, orders=np.full(n, p), quats=q, force=forces(rng, n),
                tol=1e-10, restart=50)
