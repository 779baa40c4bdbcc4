"""smob_far_traction_noalloc: the traction far field for callers that cannot allocate device
memory (their memory is reserved by another allocator, or they sit in a loop where cudaMalloc /
cudaFree would stall the device). It must give the same result as the context entry point
smob_far_field, call after call, although its scratch lives in one shared __device__ array.

This file is collected last so that a stopped run has already run every other test."""
import ctypes

import numpy as np
import pytest

from spheresimulator_gb300 import PREC_FP64, SphereSTKSHOperator
from spheresimulator_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _cudart():
    """The CUDA runtime that libsmob already loaded (found through this process's mappings)."""
    for line in open("/proc/self/maps"):
        if "libcudart" in line:
            return ctypes.CDLL(line.split()[-1])
    raise RuntimeError("libcudart is not loaded")


def _lattice(orders):
    # 8 spheres on a cube of side 4: centre distances >= 4 > 1.5 (a_s + a_t), so no near pairs and
    # the context entry point sums over exactly the same sources
    rng = np.random.default_rng(77)
    centers = np.array([[i, j, k] for i in (0, 4.0) for j in (0, 4.0) for k in (0, 4.0)])
    radii = rng.uniform(0.9, 1.1, 8)
    quats = rng.standard_normal((8, 4))
    quats /= np.linalg.norm(quats, axis=1)[:, None]
    return centers, radii, np.asarray(orders), quats


# equal orders: 1152 points (9 whole tiles of 128 targets, 8 equal source chunks); mixed orders:
# 1510 points, a partial last tile (102 targets) and source chunks of unequal length
@pytest.mark.parametrize("orders,caller_stream", [([8] * 8, False), ([8, 9, 10, 7, 8, 11, 7, 9], True)])
def test_far_traction_noalloc_matches_context_entry_point(orders, caller_stream):
    centers, radii, orders, quats = _lattice(orders)
    op = SphereSTKSHOperator(centers, radii, orders, quats=quats)
    assert op.n_near_pairs == 0
    L = N.lib()
    h = op.handle
    n = op.n_points
    coords, norms, weights = op._grid()
    sphere = np.repeat(np.arange(8, dtype=np.int32), [(p + 1) * (2 * p + 2) for p in orders])

    # the test allocates the caller's buffers; the entry point itself allocates nothing
    def dev(arr):
        arr = np.ascontiguousarray(arr)
        p = ctypes.c_void_p()
        N.check(L.smob_device_alloc(h, arr.nbytes, ctypes.byref(p)))
        N.check(L.smob_memcpy_h2d(h, p, arr.ctypes.data_as(ctypes.c_void_p), arr.nbytes))
        return p

    d_coords, d_norms, d_w, d_sid = dev(coords), dev(norms), dev(weights), dev(sphere)
    d_dens = dev(np.zeros(3 * n))
    d_out = dev(np.zeros(3 * n))
    rng = np.random.default_rng(5)
    cudart = _cudart()
    stream = ctypes.c_void_p()
    if caller_stream:
        # a non-blocking stream of the caller (cudaStreamNonBlocking = 1)
        assert cudart.cudaStreamCreateWithFlags(ctypes.byref(stream), 1) == 0
    try:
        for call, c in enumerate((1.0, -0.7)):
            dens = rng.standard_normal(3 * n)
            start = rng.standard_normal(3 * n) if call else np.zeros(3 * n)
            N.check(L.smob_memcpy_h2d(h, d_dens, dens.ctypes.data_as(ctypes.c_void_p), dens.nbytes))
            N.check(L.smob_memcpy_h2d(h, d_out, start.ctypes.data_as(ctypes.c_void_p), start.nbytes))
            # stream NULL: the legacy default stream, which the context's non-blocking stream does
            # not wait for, so the whole device is synchronized before the copy back; a caller
            # stream is synchronized by itself
            N.check(L.smob_far_traction_noalloc(d_coords, d_norms, d_w, d_dens, d_sid, n, c, d_out,
                                                stream if caller_stream else None))
            if caller_stream:
                assert cudart.cudaStreamSynchronize(stream) == 0
            else:
                assert cudart.cudaDeviceSynchronize() == 0
            out = np.zeros(3 * n)
            N.check(L.smob_memcpy_d2h(h, out.ctypes.data_as(ctypes.c_void_p), d_out, out.nbytes))
            ref = op.far_field(dens, cSL=0.0, cTrac=c, precision=PREC_FP64)
            got = out - start
            # FP64 on both sides; only the summation order differs
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-11, call
        # beyond the fixed scratch size the call is refused before any device work
        assert L.smob_far_traction_noalloc(d_coords, d_norms, d_w, d_dens, d_sid, 40961, 1.0, d_out, None) == N.SMOB_ERR_ARG
        assert b"40960" in L.smob_last_error()
    finally:
        if caller_stream:
            cudart.cudaStreamDestroy(stream)
        for p in (d_coords, d_norms, d_w, d_sid, d_dens, d_out):
            L.smob_device_free(h, p)
