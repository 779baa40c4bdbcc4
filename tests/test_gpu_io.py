"""Output files in the reference's formats: the per-sphere VTU of a density (grid with poles, pole
values from the spectral expansion, the reference's cell layout and file names) and the XYZ of the
sphere centres (Sphere/Sphere.cpp:322-365, Sphere/Shexp.cpp:96-339, SRC/SphereSystem.cpp:158-179)."""
import base64
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from spheresimulator_gb300 import SmobError, SphereSTKSHOperator, configs

pytestmark = pytest.mark.gpu

DT = {"Float64": np.float64, "Int32": np.int32, "UInt8": np.uint8}


def decode(el):
    raw = base64.b64decode(el.text.strip())
    n = int(np.frombuffer(raw[:8], np.uint64)[0])
    assert len(raw) == 8 + n
    a = np.frombuffer(raw[8:], DT[el.get("type")])
    return a.reshape(-1, int(el.get("NumberOfComponents", "1")))


def qrot(q, v):
    w, u = q[0], q[1:]
    t = 2 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def reference_cells(p):
    """The reference's cell list (getGridWithPoleCellConnect), restated with ring/column indices."""
    nphi = 2 * p + 2
    south = (p + 1) * nphi + 1
    idx = lambda j, k: 1 + j * nphi + k % nphi  # noqa: E731
    cells = [[0, idx(0, k), idx(0, k + 1)] for k in range(nphi)]
    cells += [[idx(j, k), idx(j, k + 1), idx(j - 1, k + 1), idx(j - 1, k)] for j in range(1, p + 1) for k in range(nphi)]
    cells += [[south, idx(p, nphi - 1), idx(p, 0)]]
    cells += [[south, idx(p, k + 1), idx(p, k)] for k in range(nphi - 2, -1, -1)]
    return cells


def test_vtu_of_a_linear_density(tmp_path):
    cfg = configs.small_cluster(seed=41, n=4, p=5, gap=0.4, quats=True)
    cfg["orders"] = np.array([5, 6, 5, 7])
    op = SphereSTKSHOperator(cfg["centers"], cfg["radii"], cfg["orders"], quats=cfg["quats"])
    rng = np.random.default_rng(1)
    A, b = rng.standard_normal((3, 3)), rng.standard_normal(3)
    n = op.getGridNorms()
    dens = (n @ A.T + b).reshape(-1)  # degree <= 2 in every component: exactly band-limited
    prefix = str(tmp_path) + os.sep
    op.writeVTU(prefix, "12", dens, name="stkmob")
    head = ET.parse(prefix + "Sphere_stkmob_12.pvtu").getroot()
    assert head.get("type") == "PUnstructuredGrid"
    assert head.find("PUnstructuredGrid/Piece").get("Source") == "Sphere_stkmob_r0_12.vtu"
    root = ET.parse(prefix + "Sphere_stkmob_r0_12.vtu").getroot()
    assert root.get("header_type") == "UInt64" and root.get("byte_order") == "LittleEndian"
    pieces = root.findall("UnstructuredGrid/Piece")
    assert len(pieces) == 4
    coords, w = op.getGridCoords(), op.getGridWeights()
    c, q = op.geometry()
    g0 = op.getGridNumberIndex()
    for i, pc in enumerate(pieces):
        p = int(cfg["orders"][i])
        ng = (p + 1) * (2 * p + 2)
        assert int(pc.get("NumberOfPoints")) == ng + 2 and int(pc.get("NumberOfCells")) == (2 * p + 2) * (p + 2)
        arr = {e.get("Name"): decode(e) for e in pc.iter("DataArray")}
        pts, val, wt = arr["points"], arr["stkmob"], arr["weights"].ravel()
        sl = slice(g0[i], g0[i] + ng)
        assert np.array_equal(pts[1:-1], coords[sl]) and np.array_equal(wt[1:-1], w[sl])
        assert wt[0] == 0 and wt[-1] == 0
        assert np.array_equal(val[1:-1], dens.reshape(-1, 3)[sl])
        z = qrot(q[i], np.array([0.0, 0, 1]))
        a = cfg["radii"][i]
        assert np.allclose(pts[0], c[i] + a * z, atol=1e-13) and np.allclose(pts[-1], c[i] - a * z, atol=1e-13)
        # the pole values are the expansion at theta = 1e-6 from the pole: A n + b up to that offset
        assert np.allclose(val[0], A @ z + b, atol=2e-5) and np.allclose(val[-1], -A @ z + b, atol=2e-5)
        conn, offs, types = arr["connectivity"].ravel(), arr["offsets"].ravel(), arr["types"].ravel()
        cells = reference_cells(p)
        assert np.array_equal(conn, np.concatenate(cells))
        assert np.array_equal(offs, np.cumsum([len(cl) for cl in cells]))
        assert np.array_equal(types, [5 if len(cl) == 3 else 9 for cl in cells])
    with pytest.raises(ValueError):
        op.writeVTU(prefix, "1", dens[:-3])
    with pytest.raises(SmobError):
        op.writeVTU(str(tmp_path / "missing_dir") + os.sep, "1", dens)


def test_xyz(tmp_path):
    cfg = configs.small_cluster(seed=42, n=3, p=4, gap=0.4)
    op = SphereSTKSHOperator(cfg["centers"], cfg["radii"], cfg["orders"])
    path = str(tmp_path / "SphereXYZ_r0_3.xyz")
    op.writeXYZ(path, time=0.25, gids=[7, 8, 9])
    lines = open(path).read().splitlines()
    assert lines[0] == "3" and lines[1] == "SphereNumber: 3, time: 0.250000"
    for i, ln in enumerate(lines[2:]):
        f = ln.split("\t")
        assert f[0] == "S" and int(f[1]) == 7 + i
        assert np.allclose([float(v) for v in f[2:]], [cfg["radii"][i], *cfg["centers"][i]], rtol=1e-13)
