"""Rest-pose signed distance volumes in the DT-Grid ".svol" format.

Scenes with more than one solid need each solid's rest SDF for solid-solid
contact (DEFOR_SOLID_3D::loadRestSDF, DEFOR_SOLID_3D.cpp:210-214). The
reference ships one for its sphere mesh; synthetic scenes get one written
here: the exact signed distance of a sphere of the solid's rest radius on a
narrow band, in the file layout DTGrid::loadSparseVolume reads
(SvolLoader_DTTop1.0.h):

* text: ``DTG v1.0  `` and the index/int/real sizes and endianness;
* binary: the bounding box (6 index ints), translation and rotation (3 reals
  each), then per level (x, then y per x, then z per (x, y)) the count and the
  run bounds (pairs of index ints) and the count and the per-element offsets
  into the next level's run array (the run-start sums are rebuilt on load);
* text: the auxiliary field header and the constants dx, gamma, beta,
  insideConstant, outsideConstant; binary: the band values, z fastest.

Lattice point (x, y, z) sits at ``translation + (x, y, z) * dx``.
"""
from __future__ import annotations

import struct

import numpy as np

# band half-width and lattice step of the shipped sphere (meshes/sphere/sphere.svol:
# radius 0.1, dx 0.00241982, gamma 20 dx)
DX_PER_RADIUS = 0.0241982
BAND_CELLS = 20


def _runs(mask: np.ndarray) -> list[tuple[int, int]]:
    """Inclusive (start, end) of the True runs of a 1-D mask."""
    if not mask.any():
        return []
    m = np.concatenate([[False], mask, [False]]).astype(np.int8)
    d = np.diff(m)
    starts = np.flatnonzero(d == 1)
    ends = np.flatnonzero(d == -1) - 1
    return list(zip(starts.tolist(), ends.tolist()))


def write_svol(path: str, values: np.ndarray, band: np.ndarray, lo, dx: float, translation,
               gamma: float, beta: float, inside: float, outside: float) -> None:
    """Write a narrow band: values/band are [x, y, z] arrays over lattice
    indices lo + (i, j, k); band marks the stored points."""
    values = np.asarray(values, dtype=np.float32)
    band = np.asarray(band, dtype=bool)
    lo = [int(v) for v in lo]
    xs = _runs(band.any(axis=(1, 2)))
    x_idx, va1, y_idx, va2, z_idx, vals = [], [], [], [], [], []
    for xa, xb in xs:
        x_idx += [xa + lo[0], xb + lo[0]]
        for x in range(xa, xb + 1):
            va1.append(len(y_idx))
            plane = band[x]
            for ya, yb in _runs(plane.any(axis=1)):
                y_idx += [ya + lo[1], yb + lo[1]]
                for y in range(ya, yb + 1):
                    va2.append(len(z_idx))
                    for za, zb in _runs(plane[y]):
                        z_idx += [za + lo[2], zb + lo[2]]
                        vals.append(values[x, y, za:zb + 1])
    vals = np.concatenate(vals) if vals else np.zeros(0, np.float32)
    bbox = [min(x_idx), max(x_idx), min(y_idx), max(y_idx), min(z_idx), max(z_idx)]
    with open(path, "wb") as f:
        f.write(b"DTG v1.0  IndexTypeTextDescription short\nIndexTypeSizeInBytes 2\n"
                b"IntTypeTextDescription int\nIntTypeSizeInBytes 4\n"
                b"RealTypeTextDescription float\nRealTypeSizeInBytes 4\nEndian LittleEndian\n")
        f.write(struct.pack("<6h", *bbox))
        f.write(struct.pack("<3f", *[float(t) for t in translation]))
        f.write(struct.pack("<3f", 0.0, 0.0, 0.0))
        for idx, va in ((x_idx, va1), (y_idx, va2), (z_idx, None)):
            f.write(struct.pack("<I", len(idx)))
            f.write(np.asarray(idx, dtype="<i2").tobytes())
            n = len(va) if va is not None else len(vals)
            f.write(struct.pack("<I", n))
            if va is not None:
                f.write(np.asarray(va, dtype="<u4").tobytes())
        f.write(b"Auxiliary Fields v1.0\nNumberOfScalarFields 1\n"
                b"Header DTGridTopology Auxiliary Field v1.0\n"
                b"DataTextDescription SignedDistanceField\nEndian LittleEndian\n"
                b"DataTypeTextDescription float\nDataTypeSizeInBytes 4\n")
        f.write(f"NumberOfDataItems {len(vals)}\nNumberOfConstants 5\n".encode())
        for name, v in (("dx", dx), ("gamma", gamma), ("beta", beta), ("insideConstant", inside),
                        ("outsideConstant", outside)):
            f.write(f"Constant {name} {v!r}\n".encode())
        f.write(vals.astype("<f4").tobytes())


def sphere_svol(path: str, radius: float) -> None:
    """The rest SDF of a sphere of `radius` about the origin: lattice step
    radius * DX_PER_RADIUS, band |d| < BAND_CELLS steps, the inside and
    outside constants -/+ that half-width."""
    dx = float(np.float32(radius * DX_PER_RADIUS))
    gamma = BAND_CELLS * dx
    half = int(np.ceil((radius + gamma) / dx)) + 2
    n = 2 * half + 1
    t = float(np.float32(-half * dx))
    c = t + np.arange(n) * dx
    d = np.sqrt(c[:, None, None] ** 2 + c[None, :, None] ** 2 + c[None, None, :] ** 2) - radius
    band = np.abs(d) < gamma
    write_svol(path, d.astype(np.float32), band, (0, 0, 0), dx, (t, t, t), gamma, gamma / 2,
               -gamma, gamma)


def read_svol(path: str) -> dict:
    """Parse a ".svol" file (the layout above) into its dense lattice:
    {"lo", "n", "dx", "translation", "inside", "outside", "values"[x, y, z],
    "code"[x, y, z]} with code 1 at band points, -1 where the DT-Grid returns
    its inside constant (a gap between two z-runs whose next run starts
    negative) and 0 elsewhere (outside constant)."""
    raw = open(path, "rb").read()
    if raw[:10] != b"DTG v1.0  ":
        raise ValueError("not a DT-Grid v1.0 file")
    pos = 10

    def line():
        nonlocal pos
        e = raw.index(b"\n", pos)
        out = raw[pos:e].decode()
        pos = e + 1
        return out

    head = dict(line().split(" ", 1) for _ in range(7))
    isz, csz, rsz = (int(head[k]) for k in ("IndexTypeSizeInBytes", "IntTypeSizeInBytes",
                                            "RealTypeSizeInBytes"))
    if head["Endian"] != "LittleEndian":
        raise ValueError("big-endian volumes are not read here")
    idt = {1: "<i1", 2: "<i2", 4: "<i4", 8: "<i8"}[isz]
    cdt = {4: "<u4", 8: "<u8"}[csz]
    rdt = {4: "<f4", 8: "<f8"}[rsz]

    def take(dt, n):
        nonlocal pos
        a = np.frombuffer(raw, dtype=dt, count=n, offset=pos)
        pos += a.nbytes
        return a.astype(np.int64) if dt[1] in "iu" else a.astype(np.float64)

    take(idt, 6)
    tr = take(rdt, 3)
    take(rdt, 3)
    levels = []
    for lev in range(3):
        n = int(take(cdt, 1)[0])
        idx = take(idt, n)
        nva = int(take(cdt, 1)[0])
        va = take(cdt, nva) if lev < 2 else None
        levels.append((idx, va, nva))
    aux = {}
    while True:
        k, _, v = line().partition(" ")
        aux[k] = v
        if k == "NumberOfConstants":
            break
    consts = {}
    for _ in range(int(aux["NumberOfConstants"])):
        _, name, v = line().split()
        consts[name] = float(v)
    vdt = {4: "<f4", 8: "<f8"}[int(aux["DataTypeSizeInBytes"])]
    vals = np.frombuffer(raw, dtype=vdt, count=levels[2][2], offset=pos).astype(np.float64)
    (xi, va1, _), (yi, va2, _), (zi, _, _) = levels

    def aa(idx):
        lens = idx[1::2] - idx[0::2] + 1
        return np.concatenate([[0], np.cumsum(lens)])

    aa1, aa2, aa3 = aa(xi), aa(yi), aa(zi)
    lo = np.array([xi.min(), yi.min(), zi.min()]) - 1
    n = np.array([xi.max(), yi.max(), zi.max()]) - lo + 2
    values = np.zeros(n, np.float32)
    code = np.zeros(n, np.int8)
    for r in range(len(xi) // 2):
        for x in range(xi[2 * r], xi[2 * r + 1] + 1):
            i1 = aa1[r] + x - xi[2 * r]
            ya, yb = va1[i1], va1[i1 + 1] if i1 + 1 < len(va1) else len(yi)
            for ry in range(ya, yb, 2):
                for y in range(yi[ry], yi[ry + 1] + 1):
                    i2 = aa2[ry // 2] + y - yi[ry]
                    za, zb = va2[i2], va2[i2 + 1] if i2 + 1 < len(va2) else len(zi)
                    for rz in range(za, zb, 2):
                        z0, z1 = zi[rz], zi[rz + 1]
                        v = vals[aa3[rz // 2]:aa3[rz // 2] + z1 - z0 + 1]
                        X, Y = x - lo[0], y - lo[1]
                        values[X, Y, z0 - lo[2]:z1 - lo[2] + 1] = v
                        code[X, Y, z0 - lo[2]:z1 - lo[2] + 1] = 1
                        if rz + 2 < zb:
                            nz = zi[rz + 2]
                            code[X, Y, z1 + 1 - lo[2]:nz - lo[2]] = -1 if vals[aa3[(rz + 2) // 2]] < 0 else 0
    return {"lo": lo, "n": n, "dx": consts["dx"], "translation": tr,
            "inside": consts.get("insideConstant", 0.0), "outside": consts.get("outsideConstant", 0.0),
            "values": values, "code": code}
