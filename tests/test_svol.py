"""The ".svol" rest-SDF files of solid-solid contact, on the host.

The scene writer's narrow band (eulersf_gb300/svol.py) is read back by the
Python reader and by the library's C reader (esf_svol_read, no device
needed) to the same lattice; the reference's shipped sphere volume, where a
copy of the reference is at hand, reads the same way through both and agrees
with the distance to its sphere; malformed files are refused with
ESF_ERR_IO.
"""
import ctypes as C
import os

import numpy as np
import pytest

from eulersf_gb300 import svol

REFERENCE = os.environ.get("EULERSF_REFERENCE", "/root/reference")
SHIPPED = os.path.join(REFERENCE, "meshes", "sphere", "sphere.svol")


def _c_read(lib, path):
    lo, n = (C.c_int * 3)(), (C.c_int * 3)()
    dx, tr, cs = C.c_double(), (C.c_double * 3)(), (C.c_double * 2)()
    st = lib.esf_svol_read(path.encode(), lo, n, C.byref(dx), tr, cs, None, None, 0)
    if st != 0:
        return st, None
    tot = n[0] * n[1] * n[2]
    v, c = np.zeros(tot, np.float32), np.zeros(tot, np.int8)
    assert lib.esf_svol_read(path.encode(), lo, n, C.byref(dx), tr, cs, v.ctypes.data, c.ctypes.data, tot) == 0
    shape = (n[2], n[1], n[0])
    return 0, {"lo": list(lo), "n": list(n), "dx": dx.value, "translation": list(tr),
               "inside": cs[0], "outside": cs[1],
               "values": v.reshape(shape).transpose(2, 1, 0), "code": c.reshape(shape).transpose(2, 1, 0)}


def _same(a, b):
    assert list(a["lo"]) == list(b["lo"]) and list(a["n"]) == list(b["n"])
    assert a["dx"] == b["dx"] and np.array_equal(a["translation"], b["translation"])
    assert a["inside"] == b["inside"] and a["outside"] == b["outside"]
    assert np.array_equal(a["values"], b["values"]) and np.array_equal(a["code"], b["code"])


@pytest.fixture(scope="module")
def lib():
    import eulersf_gb300 as E
    return E.load(build_if_missing=True)


def test_written_sphere_reads_back(lib, tmp_path):
    path = str(tmp_path / "ball.svol")
    r = 0.12
    svol.sphere_svol(path, r)
    py = svol.read_svol(path)
    st, cr = _c_read(lib, path)
    assert st == 0
    _same(py, cr)
    band = py["code"] == 1
    idx = np.argwhere(band) + py["lo"]
    p = idx * py["dx"] + py["translation"]
    d = np.linalg.norm(p, axis=1) - r
    assert np.abs(py["values"][band] - d).max() <= 1e-6  # float32 values of the exact distance
    gamma = svol.BAND_CELLS * py["dx"]
    assert np.abs(py["values"][band]).max() < gamma
    # the interior beyond the band reads as the inside constant, the rest outside
    inside = py["code"] == -1
    assert inside.any()
    q = (np.argwhere(inside) + py["lo"]) * py["dx"] + py["translation"]
    assert (np.linalg.norm(q, axis=1) < r).all()


@pytest.mark.skipif(not os.path.exists(SHIPPED), reason="no copy of the reference's meshes")
def test_shipped_sphere_volume_reads_the_same(lib):
    py = svol.read_svol(SHIPPED)
    st, cr = _c_read(lib, SHIPPED)
    assert st == 0
    _same(py, cr)
    assert py["dx"] == 0.00241982
    band = py["code"] == 1
    p = (np.argwhere(band) + py["lo"]) * py["dx"] + py["translation"]
    # the shipped mesh is a sphere of radius ~0.0995: the band's values are
    # its distance to a fifth of a lattice step
    assert np.abs(py["values"][band] - (np.linalg.norm(p, axis=1) - 0.0995)).max() < 0.25 * py["dx"]


def test_malformed_volumes_are_refused(lib, tmp_path):
    good = str(tmp_path / "ball.svol")
    svol.sphere_svol(good, 0.1)
    raw = open(good, "rb").read()
    cases = {"header": b"XTG v1.0  " + raw[10:], "truncated": raw[: len(raw) // 2],
             "no_values": raw[: raw.index(b"Constant outsideConstant")]}
    for name, data in cases.items():
        p = str(tmp_path / f"{name}.svol")
        open(p, "wb").write(data)
        st, _ = _c_read(lib, p)
        assert st == 5, (name, st)  # ESF_ERR_IO
    st, _ = _c_read(lib, str(tmp_path / "missing.svol"))
    assert st == 5
