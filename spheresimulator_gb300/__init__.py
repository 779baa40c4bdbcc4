"""spheresimulator_gb300 — GB300-native sphere mobility operator and mobility solve.

Host-side mirror of the reference's operator interface over the C ABI of libsmob.so
(include/smob.h). The names follow the reference classes:

  SphereSTKSHOperator  (BIE/SphereSTKSHOperator.hpp:112-231): A = 0.5 I + K + L on the
                       spheres' grid densities; apply / applyP2POP / applyLOP / projectNullSpace
  SphereSTKMobMat      (BIE/SphereSTKMobMat.hpp:26-79): mobility matrix 6N -> 6N through a
                       GMRES boundary-integral solve; solveMob / apply / getDensitySolution

Every computation runs in the CUDA library; there is no CPU path.
"""
import ctypes

import numpy as np

from . import _native as N
from ._native import PREC_FLOAT_FLOAT, PREC_FP64, PREC_MIXED, SmobError

__all__ = ["SphereSTKSHOperator", "SphereSTKMobMat", "SmobError", "PREC_FP64", "PREC_MIXED", "PREC_FLOAT_FLOAT", "solve_opts",
           "grid_number", "spectral_dof", "warm_orders", "request_bytes", "SolveServer"]


def grid_number(p):
    """(p+1)(2p+2) grid points per sphere (Sphere/Shexp.hpp:65)."""
    return (p + 1) * (2 * p + 2)


def spectral_dof(p):
    """3(p+1)(p+2) doubles of spectral coefficients per sphere (Sphere/Shexp.hpp:66)."""
    return 3 * (p + 1) * (p + 2)


WARM_NONE, WARM_LAST, WARM_RECYCLE = 0, 1, 2


def _warm_code(warm_start):
    if isinstance(warm_start, str):
        if warm_start != "recycle":
            raise ValueError("warm_start: False, True (previous solution) or 'recycle'")
        return WARM_RECYCLE
    if isinstance(warm_start, (bool, np.bool_)):
        return WARM_LAST if warm_start else WARM_NONE
    return int(warm_start)


def solve_opts(tol=1e-10, restart=50, max_iters=500, precision=PREC_FP64, warm_start=False, inner_tol=0.0,
               precond=0):
    """GMRES settings (mobilitySolver.yaml:3-16 names: Convergence Tolerance, Num Blocks, Maximum Iterations);
    warm_start: False (zero), True (previous solution, SphereSTKMobMat.cpp:222) or "recycle" (the closest
    combination of earlier solutions on this geometry, which the solve then joins);
    precond=1 adds the block-diagonal right preconditioner (each sphere's own operator inverted)."""
    return N.SolveOpts(float(tol), int(restart), int(max_iters), int(precision), _warm_code(warm_start),
                       float(inner_tol), int(precond))


class _Context:
    def __init__(self, centers, radii, orders, quats=None, problem=None, viscosity=1.0, device=0):
        self._L = N.lib()
        self.centers = N.f64(centers).reshape(-1, 3)
        self.radii = N.f64(radii).reshape(-1)
        self.orders = N.i32(orders).reshape(-1)
        self.quats = None if quats is None else N.f64(quats).reshape(-1, 4)
        self.problem = None if problem is None else N.i32(problem).reshape(-1)
        n = len(self.radii)
        if self.centers.shape[0] != n or self.orders.shape[0] != n:
            raise ValueError("centers, radii and orders must describe the same number of spheres")
        geo = N.Geometry(n, N.dptr(self.centers), N.dptr(self.radii), N.dptr(self.quats), N.iptr(self.orders),
                         N.iptr(self.problem), float(viscosity))
        h = ctypes.c_void_p()
        N.check(self._L.smob_create(ctypes.byref(h), ctypes.byref(geo), int(device)))
        self._h = h
        ns, npt, npb, nnp = (ctypes.c_int() for _ in range(4))
        N.check(self._L.smob_get_sizes(h, ctypes.byref(ns), ctypes.byref(npt), ctypes.byref(npb), ctypes.byref(nnp)))
        self.n_spheres, self.n_points, self.n_problems, self.n_near_pairs = ns.value, npt.value, npb.value, nnp.value
        self.viscosity = float(viscosity)

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            self._L.smob_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- time stepping (Sphere::stepEuler, Sphere/Sphere.cpp:367-373): the context is rebuilt in place
    def _refresh(self):
        c = np.zeros((self.n_spheres, 3))
        q = np.zeros((self.n_spheres, 4))
        N.check(self._L.smob_get_geometry(self._h, N.dptr(c), N.dptr(q)))
        self.centers, self.quats = c, q
        nnp = ctypes.c_int()
        N.check(self._L.smob_get_sizes(self._h, None, None, None, ctypes.byref(nnp)))
        self.n_near_pairs = nnp.value

    def geometry(self):
        """(centres [N,3], unit quaternions [N,4]) of the current geometry, as the library holds it."""
        c = np.zeros((self.n_spheres, 3))
        q = np.zeros((self.n_spheres, 4))
        N.check(self._L.smob_get_geometry(self._h, N.dptr(c), N.dptr(q)))
        return c, q

    def step_euler(self, vel, dt):
        """Advance every sphere by its velocity/angular velocity (6N, as solveMob returns) over dt."""
        v = N.f64(vel).reshape(-1)
        if v.shape[0] != 6 * self.n_spheres:
            raise ValueError("expected 6N velocities")
        N.check(self._L.smob_step_euler(self._h, N.dptr(v), float(dt)))
        self._refresh()

    def set_geometry(self, centers, quats=None):
        """New centres (and orientations) for the same spheres."""
        c = N.f64(centers).reshape(-1)
        q = None if quats is None else N.f64(quats).reshape(-1)
        if c.shape[0] != 3 * self.n_spheres or (q is not None and q.shape[0] != 4 * self.n_spheres):
            raise ValueError("expected 3N centres and 4N quaternions")
        N.check(self._L.smob_set_geometry(self._h, N.dptr(c), N.dptr(q)))
        self._refresh()

    # ---- output files (Sphere::writeVTU/writePVTU, SphereSystem::writeXYZ)
    def writeVTU(self, prefix, postfix, density, name="stkmob"):
        """Density (3M) on every sphere's grid with poles: <prefix>Sphere_<name>_r0_<postfix>.vtu + .pvtu."""
        d = N.f64(density).reshape(-1)
        if d.shape[0] != 3 * self.n_points:
            raise ValueError("expected 3M density values")
        N.check(self._L.smob_write_vtu(self._h, str(prefix).encode(), str(postfix).encode(), str(name).encode(),
                                       N.dptr(d)))

    def writeXYZ(self, path, time=0.0, gids=None):
        """Sphere centres and radii, one 'S gid radius x y z' line per sphere."""
        g = None if gids is None else N.i32(gids).reshape(-1)
        N.check(self._L.smob_write_xyz(self._h, str(path).encode(), N.iptr(g), float(time)))

    # grid getters (SphereSTKSHOperator.hpp:218-223)
    def _grid(self):
        c = np.zeros((self.n_points, 3))
        nn = np.zeros((self.n_points, 3))
        w = np.zeros(self.n_points)
        N.check(self._L.smob_get_grid(self._h, N.dptr(c), N.dptr(nn), N.dptr(w)))
        return c, nn, w

    def getGridCoords(self):
        return self._grid()[0]

    def getGridNorms(self):
        return self._grid()[1]

    def getGridWeights(self):
        return self._grid()[2]

    def getGridNumberIndex(self):
        lens = np.array([grid_number(p) for p in self.orders])
        return np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)

    def near_pairs(self):
        t = np.zeros(max(self.n_near_pairs, 1), np.int32)
        s = np.zeros(max(self.n_near_pairs, 1), np.int32)
        N.check(self._L.smob_get_near_pairs(self._h, N.iptr(t), N.iptr(s)))
        return t[:self.n_near_pairs], s[:self.n_near_pairs]

    def launch_count(self):
        v = ctypes.c_longlong()
        N.check(self._L.smob_launch_count(self._h, ctypes.byref(v)))
        return v.value

    def set_graphs(self, on=True):
        """CUDA graphs for the solves (on by default)."""
        N.check(self._L.smob_set_graphs(self._h, int(on)))

    def set_loop_graph(self, on=True):
        """The whole restart-cycle loop as one graph launch with device-side decisions (with graphs on);
        off: the host drives the cycles and replays captured blocks of Arnoldi steps."""
        N.check(self._L.smob_set_loop_graph(self._h, int(on)))

    def loop_graph_info(self):
        """(selected, available): the loop graph is selected; building one has not failed here."""
        on, ok = ctypes.c_int(), ctypes.c_int()
        N.check(self._L.smob_loop_graph_info(self._h, ctypes.byref(on), ctypes.byref(ok)))
        return bool(on.value), bool(ok.value)

    def launch_stats(self):
        """(kernels run, host launch calls) on this context since creation."""
        k, h = ctypes.c_longlong(), ctypes.c_longlong()
        N.check(self._L.smob_launch_stats(self._h, ctypes.byref(k), ctypes.byref(h)))
        return k.value, h.value

    def near_tc(self):
        """True if the FP32 near field runs on the tensor cores"""
        v = ctypes.c_int()
        N.check(self._L.smob_tc_info(self._h, ctypes.byref(v), None))
        return bool(v.value)

    def sphere_tc(self):
        """True if the FP32 sphere operator runs its Legendre stage on the tensor cores"""
        v = ctypes.c_int()
        N.check(self._L.smob_tc_info(self._h, None, ctypes.byref(v)))
        return bool(v.value)

    def set_sphere_tc(self, on=True):
        """FP32 sphere operator with its Legendre stage on the tensor cores or the SIMT kernel (default)"""
        N.check(self._L.smob_set_sphere_tc(self._h, int(bool(on))))

    def coarse_tc(self):
        """Mode of the FP32 coarse GEMMs: 1 both on the tensor cores, 0 both SIMT, 2 only the strengths,
        3 only the coarse-target interpolation on the tensor cores"""
        v = ctypes.c_int()
        N.check(self._L.smob_coarse_tc_info(self._h, ctypes.byref(v)))
        return v.value

    def set_multi_shared_pairs(self, on=True):
        """Several right-hand sides with the shared-pair kernels (each grid-point pair once for all
        columns) instead of a batch of copies (the default)."""
        N.check(self._L.smob_set_multi_shared_pairs(self._h, int(bool(on))))

    def set_coarse_tc(self, mode=1):
        """FP32 coarse equivalent-source strengths and coarse-target interpolation on the tensor cores
        (mode 1, default; True) or as SIMT GEMMs (0, False); 2 only the strengths, 3 only the
        interpolation on the tensor cores"""
        N.check(self._L.smob_set_coarse_tc(self._h, int(mode)))

    def set_near_tc(self, on=True):
        """FP32 near field on the tensor cores (default) or on the SIMT pipes"""
        N.check(self._L.smob_set_near_tc(self._h, int(bool(on))))

    def set_far_tile(self, targets_per_thread):
        """Force the FP32 far-field variant (1, 2 or 4 targets per thread) over the autotuner's choice."""
        N.check(self._L.smob_set_far_tile(self._h, int(targets_per_thread)))

    def set_far_compression(self, eps, eps_hp=None):
        """Tolerances of the far field's coarse equivalent sources for well-separated sphere pairs
        (relative to each source sphere's contribution): eps for the FP32 passes, eps_hp for the
        float-float passes (None: unchanged); <= 0 evaluates every pair directly."""
        if eps_hp is None:
            eps_hp = self.far_compression_info(hp=True)[0]
        N.check(self._L.smob_set_far_compression(self._h, float(eps), float(eps_hp)))

    def set_far_coarse_targets(self, on):
        """Coarse targets of the FP32 set (default on): the far field of a well-separated source sphere
        evaluated at a coarse grid of the target sphere and interpolated to its grid."""
        N.check(self._L.smob_set_far_coarse_targets(self._h, int(bool(on))))

    def far_compression_info(self, hp=False):
        """(eps, coarse points held, (sphere, level) entries) of the FP32 set, or of the float-float set"""
        e, pts, ent = ctypes.c_double(), ctypes.c_int(), ctypes.c_int()
        N.check(self._L.smob_far_compression_info(self._h, int(bool(hp)), ctypes.byref(e), ctypes.byref(pts),
                                                  ctypes.byref(ent)))
        return e.value, pts.value, ent.value

    def far_pairs(self, hp=False):
        """(direct-sum pairs, evaluated pairs, coarse multiply-adds: strengths and target interpolation) of one
        FP32 far-field pass, or (hp=True) of one fused float-float pass"""
        d, e, m = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        N.check(self._L.smob_far_pairs_set(self._h, int(bool(hp)), ctypes.byref(d), ctypes.byref(e),
                                           ctypes.byref(m)))
        return d.value, e.value, m.value

    def recycle_info(self):
        """(recycled solutions held, capacity) for warm_start="recycle"."""
        k, cap = ctypes.c_int(), ctypes.c_int()
        N.check(self._L.smob_recycle_info(self._h, ctypes.byref(k), ctypes.byref(cap)))
        return k.value, cap.value

    def recycle_clear(self):
        N.check(self._L.smob_recycle_clear(self._h))

    def tuning(self):
        """(targets per thread in use, measured ms of the 1/2/4 variants, whether the choice was cached)"""
        t, c = ctypes.c_int(), ctypes.c_int()
        ms = np.zeros(3)
        N.check(self._L.smob_tuning(self._h, ctypes.byref(t), N.dptr(ms), ctypes.byref(c)))
        return t.value, ms, bool(c.value)

    def profile(self, on=True):
        N.check(self._L.smob_profile_enable(self._h, int(on)))

    def profile_reset(self):
        N.check(self._L.smob_profile_reset(self._h))

    def profile_table(self):
        n = ctypes.c_int()
        N.check(self._L.smob_profile_count(self._h, ctypes.byref(n)))
        out = {}
        for i in range(n.value):
            name = ctypes.create_string_buffer(64)
            la = ctypes.c_longlong()
            ms = ctypes.c_double()
            N.check(self._L.smob_profile_get(self._h, i, name, 64, ctypes.byref(la), ctypes.byref(ms)))
            out[name.value.decode()] = (la.value, ms.value)
        return out


class SphereSTKSHOperator(_Context):
    """A = 0.5 I + K + L (the operator SphereSTKMobMat builds with cId=0.5, cSL=0, cTrac=1, cLOP=1,
    BIE/SphereSTKMobMat.cpp:17), applied on the GPU."""

    def _vec(self, x):
        x = N.f64(x).reshape(-1)
        if x.shape[0] != 3 * self.n_points:
            raise ValueError("expected a vector of length 3M = %d" % (3 * self.n_points))
        return x

    def apply(self, X, Y=None, alpha=1.0, beta=0.0, precision=PREC_FP64):
        """Y = alpha*A*X + beta*Y (Tpetra::Operator::apply, BIE/SphereSTKSHOperator.cpp:153-236);
        X may have shape (3M,) or (ncol, 3M)."""
        X = N.f64(X)
        one = X.ndim == 1
        X2 = X.reshape(1, -1) if one else X
        if X2.shape[1] != 3 * self.n_points:
            raise ValueError("expected columns of length 3M")
        Y2 = np.zeros_like(X2) if Y is None else N.f64(Y).reshape(X2.shape).copy()
        N.check(self._L.smob_apply(self._h, N.dptr(X2), N.dptr(Y2), X2.shape[0], float(alpha), float(beta),
                                   int(precision)))
        return Y2.reshape(-1) if one else Y2

    def applyP2POP(self, inp, out=None, cId=0.0, cSL=0.0, cTrac=0.0, precision=PREC_FP64):
        """out += cId*in + cSL*S[in] + cTrac*K[in] (BIE/SphereSTKSHOperator.cpp:262-485)."""
        inp = self._vec(inp)
        out = np.zeros(3 * self.n_points) if out is None else self._vec(out).copy()
        N.check(self._L.smob_apply_p2p(self._h, N.dptr(inp), N.dptr(out), float(cId), float(cSL), float(cTrac),
                                       int(precision)))
        return out

    def applyLOP(self, inp, out=None, cLOP=1.0):
        """out += cLOP * L[in] (BIE/SphereSTKSHOperator.cpp:487-521)."""
        inp = self._vec(inp)
        out = np.zeros(3 * self.n_points) if out is None else self._vec(out).copy()
        N.check(self._L.smob_apply_lop(self._h, N.dptr(inp), N.dptr(out), float(cLOP)))
        return out

    def projectNullSpace(self, x):
        """Projection onto each sphere's band-limited space (BIE/SphereSTKSHOperator.cpp:239-260)."""
        x = self._vec(x).copy()
        N.check(self._L.smob_project_null_space(self._h, N.dptr(x)))
        return x

    def far_field(self, inp, cSL=0.0, cTrac=0.0, precision=PREC_FP64):
        inp = self._vec(inp)
        out = np.zeros(3 * self.n_points)
        N.check(self._L.smob_far_field(self._h, N.dptr(inp), N.dptr(out), float(cSL), float(cTrac), int(precision)))
        return out

    def near_field(self, inp, cSL=0.0, cTrac=0.0, precision=PREC_FP64):
        inp = self._vec(inp)
        out = np.zeros(3 * self.n_points)
        N.check(self._L.smob_near_field(self._h, N.dptr(inp), N.dptr(out), float(cSL), float(cTrac), int(precision)))
        return out

    def coeff_offsets(self):
        off = np.zeros(self.n_spheres + 1, np.int32)
        N.check(self._L.smob_coeff_offsets(self._h, N.iptr(off)))
        return off

    def sh_g2s(self, grid):
        grid = self._vec(grid)
        out = np.zeros(int(self.coeff_offsets()[-1]))
        N.check(self._L.smob_sh_g2s(self._h, N.dptr(grid), N.dptr(out)))
        return out

    def sh_s2g(self, coeff):
        coeff = N.f64(coeff).reshape(-1)
        out = np.zeros(3 * self.n_points)
        N.check(self._L.smob_sh_s2g(self._h, N.dptr(coeff), N.dptr(out)))
        return out


def warm_orders(orders):
    """Build the per-order host tables of these orders now (smob_warm_orders), so that the first
    context of each order does not pay for them."""
    o = N.i32(orders).reshape(-1)
    N.check(N.lib().smob_warm_orders(N.iptr(o), len(o)))


def request_bytes(orders, restart=50):
    """Device-memory footprint the server uses to admit a request (host arithmetic only)."""
    o = N.i32(orders).reshape(-1)
    return int(N.lib().smob_request_bytes(len(o), N.iptr(o), int(restart)))


class SolveServer:
    """Request loop with continuous batching of mobility solves on one GPU (smob_server_*)."""

    def __init__(self, device=0, max_slots=8, hbm_budget_bytes=0.0, restart=50, max_iters=2000,
                 precision=PREC_MIXED, inner_tol=0.0, small_sms=0, graphs=False):
        """small_sms > 0: SMs reserved (green context) for small requests while big ones run;
        graphs: CUDA graphs in the request contexts: False/0 none (each solves once), True/1 all, 2 big
        requests only"""
        self._L = N.lib()
        opts = N.ServerOpts(int(device), int(max_slots), float(hbm_budget_bytes), int(restart), int(max_iters),
                            int(precision), float(inner_tol), int(graphs))
        h = ctypes.c_void_p()
        N.check(self._L.smob_server_create(ctypes.byref(h), ctypes.byref(opts)))
        self._h = h
        self._n = {}
        if small_sms:
            self.partition(small_sms)

    def partition(self, small_sms):
        """Split the device's SMs: small_sms for small requests while big ones run (0: no split)."""
        N.check(self._L.smob_server_partition(self._h, int(small_sms)))

    def partition_info(self):
        """(SMs of the small partition, SMs of the big partition); (0, 0) without a partition."""
        a, b = ctypes.c_int(), ctypes.c_int()
        N.check(self._L.smob_server_partition_info(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def submit(self, centers, radii, orders, force, tol=1e-8, quats=None, viscosity=1.0):
        c = N.f64(centers).reshape(-1, 3)
        r = N.f64(radii).reshape(-1)
        o = N.i32(orders).reshape(-1)
        q = None if quats is None else N.f64(quats).reshape(-1, 4)
        f = N.f64(force).reshape(-1)
        geo = N.Geometry(len(r), N.dptr(c), N.dptr(r), N.dptr(q), N.iptr(o), None, float(viscosity))
        rid = ctypes.c_longlong()
        N.check(self._L.smob_server_submit(self._h, ctypes.byref(geo), N.dptr(f), float(tol), ctypes.byref(rid)))
        self._n[rid.value] = len(r)
        return rid.value

    def poll(self, rid):
        vel = np.zeros(6 * self._n[rid])
        info = N.RequestInfo()
        done = ctypes.c_int()
        N.check(self._L.smob_server_poll(self._h, rid, N.dptr(vel), ctypes.byref(info), ctypes.byref(done)))
        return (vel if done.value else None), self._info(info)

    def wait(self, rid, timeout=0.0):
        vel = np.zeros(6 * self._n[rid])
        info = N.RequestInfo()
        code = self._L.smob_server_wait(self._h, rid, float(timeout), N.dptr(vel), ctypes.byref(info))
        N.check(code, allow=(N.SMOB_ERR_NOT_CONVERGED,))
        return vel, self._info(info)

    def release(self, rid):
        N.check(self._L.smob_server_release(self._h, rid))
        self._n.pop(rid, None)

    def stats(self):
        s = N.ServerInfo()
        N.check(self._L.smob_server_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    @staticmethod
    def _info(i):
        return {"state": i.state, "status": i.status, "t_submit": i.t_submit, "t_admit": i.t_admit,
                "t_ctx": i.t_ctx, "t_done": i.t_done, "route": i.route, "bytes": i.bytes, "stats": i.stats.as_dict()}

    def close(self):
        if getattr(self, "_h", None):
            self._L.smob_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SphereSTKMobMat(SphereSTKSHOperator):
    """Mobility matrix force/torque (6N) -> velocity/angular velocity (6N)
    (BIE/SphereSTKMobMat.cpp:98-286). One context may hold several independent problems
    (``problem`` ids per sphere); they are solved together, each with its own Krylov space."""

    def __init__(self, *args, **kw):
        super().__init__(*args, **kw)
        self._density = None
        self.last_stats = None

    def solveMob(self, force, tol=1e-10, restart=50, max_iters=500, precision=PREC_FP64, warm_start=False,
                 inner_tol=0.0, want_density=True, raise_on_not_converged=True, precond=0):
        """force (6N) -> velocity (6N); also keeps rho+mu (getDensitySolution)."""
        force = N.f64(force).reshape(-1)
        if force.shape[0] != 6 * self.n_spheres:
            raise ValueError("expected 6N forces/torques")
        vel = np.zeros(6 * self.n_spheres)
        dens = np.zeros(3 * self.n_points) if want_density else None
        stats = (N.ProblemStats * self.n_problems)()
        opts = solve_opts(tol, restart, max_iters, precision, warm_start, inner_tol, precond)
        code = self._L.smob_solve_mob(self._h, N.dptr(force), N.dptr(vel), N.dptr(dens), ctypes.byref(opts), stats)
        allow = () if raise_on_not_converged else (N.SMOB_ERR_NOT_CONVERGED,)
        N.check(code, allow)
        self._density = dens
        self.last_stats = [s.as_dict() for s in stats]
        return vel

    def solveMobMulti(self, forces, tol=1e-10, restart=50, max_iters=500, precision=PREC_FP64, warm_start=False,
                      inner_tol=0.0, want_density=False, raise_on_not_converged=True, precond=0):
        """forces [K][6N] -> velocities [K][6N]: K right-hand sides on this geometry solved together
        (the columns SphereSTKMobMat::apply solves one by one, BIE/SphereSTKMobMat.cpp:129-143)."""
        F = np.ascontiguousarray(N.f64(forces).reshape(-1, 6 * self.n_spheres))
        k = F.shape[0]
        vel = np.zeros_like(F)
        dens = np.zeros((k, 3 * self.n_points)) if want_density else None
        stats = (N.ProblemStats * k)()
        opts = solve_opts(tol, restart, max_iters, precision, warm_start, inner_tol, precond)
        code = self._L.smob_solve_mob_multi(self._h, k, N.dptr(F), N.dptr(vel), N.dptr(dens), ctypes.byref(opts),
                                            stats)
        allow = () if raise_on_not_converged else (N.SMOB_ERR_NOT_CONVERGED,)
        N.check(code, allow)
        self.last_stats = [s.as_dict() for s in stats]
        if want_density:
            self._density = dens
        return vel

    def getDensitySolution(self):
        """rho + mu from the last solve (BIE/SphereSTKMobMat.hpp:76)."""
        return self._density

    def apply(self, X, Y=None, alpha=1.0, beta=0.0, tol=1e-10, restart=50, max_iters=500, precision=PREC_FP64):
        """Y = alpha*M X + beta*Y for the mobility matrix M (BIE/SphereSTKMobMat.cpp:98-144)."""
        X = N.f64(X)
        one = X.ndim == 1
        X2 = X.reshape(1, -1) if one else X
        Y2 = np.zeros_like(X2) if Y is None else N.f64(Y).reshape(X2.shape).copy()
        opts = solve_opts(tol, restart, max_iters, precision)
        N.check(self._L.smob_mob_apply(self._h, N.dptr(X2), N.dptr(Y2), X2.shape[0], float(alpha), float(beta),
                                       ctypes.byref(opts)))
        return Y2.reshape(-1) if one else Y2
