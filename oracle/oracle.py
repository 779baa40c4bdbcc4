"""ctypes binding of the FP64 CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this module; the
product path (spheresimulator_gb300) never imports it.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        vp = ctypes.c_void_p
        sig = {
            "orc_grid_number": (ctypes.c_int, [ctypes.c_int]),
            "orc_spectral_dof": (ctypes.c_int, [ctypes.c_int]),
            "orc_gauss_legendre": (None, [ctypes.c_int, dp, dp]),
            "orc_sh_grid": (None, [ctypes.c_int, ctypes.c_double, dp, dp, dp, dp, dp]),
            "orc_sh_g2s": (None, [ctypes.c_int, dp, dp, dp]),
            "orc_sh_s2g": (None, [ctypes.c_int, dp, dp, dp]),
            "orc_sh_self": (None, [ctypes.c_int, ctypes.c_double, dp, dp, ctypes.c_int, dp]),
            "orc_sh_eval_exterior": (None, [ctypes.c_int, ctypes.c_double, dp, dp, ctypes.c_int, dp, dp, dp, dp]),
            "orc_create": (vp, [ctypes.c_int, dp, dp, dp, ip, ctypes.c_double]),
            "orc_destroy": (None, [vp]),
            "orc_num_points": (ctypes.c_int, [vp]),
            "orc_num_pairs": (ctypes.c_int, [vp]),
            "orc_get_pairs": (None, [vp, ip, ip]),
            "orc_get_grid": (None, [vp, dp, dp, dp]),
            "orc_apply_p2p": (None, [vp, dp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
            "orc_apply_lop": (None, [vp, dp, dp, ctypes.c_double]),
            "orc_apply": (None, [vp, dp, dp, ctypes.c_double, ctypes.c_double]),
            "orc_far_traction": (None, [vp, dp, dp, ctypes.c_double, ctypes.c_int]),
            "orc_far_sl": (None, [vp, dp, dp, ctypes.c_double, ctypes.c_int]),
            "orc_near_correction": (None, [vp, dp, dp, ctypes.c_double, ctypes.c_double]),
            "orc_solve_mob": (ctypes.c_int, [vp, dp, dp, dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ip, dp]),
            "orc_set_threads": (None, [ctypes.c_int]),
            "orc_near_pairs": (ctypes.c_int, [ctypes.c_int, dp, dp, ctypes.c_int, ip, ip]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _d(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _arr(x, dtype=np.float64):
    return None if x is None else np.ascontiguousarray(x, dtype=dtype)


def set_threads(n):
    lib().orc_set_threads(int(n))


def gauss_legendre(n):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().orc_gauss_legendre(n, _d(x), _d(w))
    return x, w


def grid_number(p):
    return (p + 1) * (2 * p + 2)


def spectral_dof(p):
    return 3 * (p + 1) * (p + 2)


def sh_grid(p, radius=1.0, quat=None, center=None):
    ng = grid_number(p)
    c = np.zeros((ng, 3))
    n = np.zeros((ng, 3))
    w = np.zeros(ng)
    quat = _arr(quat)
    center = _arr(center)
    lib().orc_sh_grid(p, radius, _d(quat), _d(center), _d(c), _d(n), _d(w))
    return c, n, w


def sh_g2s(p, grid3, quat=None):
    grid3 = _arr(grid3)
    out = np.zeros(spectral_dof(p))
    quat = _arr(quat)
    lib().orc_sh_g2s(p, _d(quat), _d(grid3), _d(out))
    return out


def sh_s2g(p, coeff, quat=None):
    coeff = _arr(coeff)
    out = np.zeros((grid_number(p), 3))
    quat = _arr(quat)
    lib().orc_sh_s2g(p, _d(quat), _d(coeff), _d(out))
    return out


SELF_SL, SELF_TRAC_EXT, SELF_TRAC_INT, SELF_TRAC_PV = 0, 1, 2, 3


def sh_self(p, coeff, kind, radius=1.0, quat=None):
    coeff = _arr(coeff)
    out = np.zeros((grid_number(p), 3))
    quat = _arr(quat)
    lib().orc_sh_self(p, radius, _d(quat), _d(coeff), kind, _d(out))
    return out


def sh_eval_exterior(p, coeff, trg_rel, trg_norm=None, radius=1.0, quat=None, sl=True, trac=True):
    coeff = _arr(coeff)
    trg_rel = _arr(trg_rel)
    nt = trg_rel.shape[0]
    trg_norm = _arr(trg_norm)
    u = np.zeros((nt, 3)) if sl else None
    t = np.zeros((nt, 3)) if trac else None
    quat = _arr(quat)
    lib().orc_sh_eval_exterior(p, radius, _d(quat), _d(coeff), nt, _d(trg_rel), _d(trg_norm), _d(u), _d(t))
    return u, t


def near_pairs(centers, radii):
    centers = _arr(centers)
    radii = _arr(radii)
    n = len(radii)
    cnt = lib().orc_near_pairs(n, _d(centers), _d(radii), 0, None, None)
    t = np.zeros(max(cnt, 1), dtype=np.int32)
    s = np.zeros(max(cnt, 1), dtype=np.int32)
    lib().orc_near_pairs(n, _d(centers), _d(radii), cnt, _i(t), _i(s))
    return t[:cnt], s[:cnt]


class Operator:
    """Oracle counterpart of SphereSTKSHOperator / SphereSTKMobMat on one set of spheres."""

    def __init__(self, centers, radii, orders, quats=None, viscosity=1.0):
        self.centers = _arr(centers).reshape(-1, 3)
        self.radii = _arr(radii)
        self.orders = _arr(orders, np.int32)
        self.quats = _arr(quats)
        self.n = len(self.radii)
        self.h = lib().orc_create(self.n, _d(self.centers), _d(self.radii), _d(self.quats), _i(self.orders),
                                  float(viscosity))
        self.m = lib().orc_num_points(self.h)

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def grid(self):
        c = np.zeros((self.m, 3))
        n = np.zeros((self.m, 3))
        w = np.zeros(self.m)
        lib().orc_get_grid(self.h, _d(c), _d(n), _d(w))
        return c, n, w

    def pairs(self):
        k = lib().orc_num_pairs(self.h)
        t = np.zeros(max(k, 1), dtype=np.int32)
        s = np.zeros(max(k, 1), dtype=np.int32)
        lib().orc_get_pairs(self.h, _i(t), _i(s))
        return t[:k], s[:k]

    def _io(self, x, out):
        x = _arr(x).reshape(-1)
        out = np.zeros(3 * self.m) if out is None else _arr(out).reshape(-1).copy()
        return x, out

    def apply_p2p(self, x, c_id, c_sl, c_trac, out=None):
        x, out = self._io(x, out)
        lib().orc_apply_p2p(self.h, _d(x), _d(out), c_id, c_sl, c_trac)
        return out

    def apply_lop(self, x, c_lop, out=None):
        x, out = self._io(x, out)
        lib().orc_apply_lop(self.h, _d(x), _d(out), c_lop)
        return out

    def apply(self, x, y=None, alpha=1.0, beta=0.0):
        x, y = self._io(x, y)
        lib().orc_apply(self.h, _d(x), _d(y), alpha, beta)
        return y

    def far_traction(self, x, c=1.0, excl_near=False):
        x, out = self._io(x, None)
        lib().orc_far_traction(self.h, _d(x), _d(out), c, int(excl_near))
        return out

    def far_sl(self, x, c=1.0, excl_near=False):
        x, out = self._io(x, None)
        lib().orc_far_sl(self.h, _d(x), _d(out), c, int(excl_near))
        return out

    def near_correction(self, x, c_sl, c_trac):
        x, out = self._io(x, None)
        lib().orc_near_correction(self.h, _d(x), _d(out), c_sl, c_trac)
        return out

    def solve_mob(self, force, tol=1e-10, restart=50, maxit=500):
        force = _arr(force).reshape(-1)
        vel = np.zeros(6 * self.n)
        dens = np.zeros(3 * self.m)
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0)
        st = lib().orc_solve_mob(self.h, _d(force), _d(vel), _d(dens), tol, restart, maxit, ctypes.byref(it),
                                 ctypes.byref(rr))
        return dict(vel=vel, density=dens, iters=it.value, relres=rr.value, status=st)
