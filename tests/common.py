"""Shared helpers of the test suite: golden fixtures, scenes, comparisons."""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

from eulersf_gb300.scene import SceneDesc, SolidDesc  # noqa: E402

GOLDEN_SCENES = ["ball16", "ball20_vort", "wall20", "plastic20", "rot20", "shipped20"]


def register_shipped_sphere():
    """The reference's shipped sphere mesh with the rest mass its own
    rasterizeSolid tool baked (tests/golden/sphere_mass.npz) as the rest
    assets "shipped_sphere"."""
    from eulersf_gb300.scene import register_assets
    z = np.load(os.path.join(GOLDEN, "sphere_mass.npz"))
    res = [int(v) for v in z["res"]]
    n = res[0] * res[1] * res[2]
    data = np.unpackbits(z["solid"])[:n].astype(np.float64) * float(z["density"])
    register_assets("shipped_sphere", (res, float(z["dh"]), z["origin"].astype(np.float64),
                                       data.reshape(res[2], res[1], res[0])), z["vertices"], z["triangles"])

# bit-exact integer/flag fields (the reference's DOF maps, cell flags, boxes)
EXACT = ["gridIdxToSolutionIdx", "gridIdxToSolidIdx", "solid0.valid", "solid0.boxes"]
# floating-point fields compared at a relative (max-norm) tolerance
FLOAT = ["velocity", "intensity", "solidMass", "nodeSolidVolumeFraction", "lambda1",
         "solid0.mass", "solid0.phi", "solid0.u", "solid0.X", "solid0.velocity",
         "solid0.particles", "solid0.meshVertices", "solid0.detFInv", "nzMassVecInv",
         "JMInvJTDiag", "b1", "velocityAtDt0", "solidUnitForce", "dampedSolidMassVec",
         "solidVelocityAtDt0", "solid0.FpInv", "solid0.FpInvGrid"]

# golden name -> integrator field name (abi.FIELDS)
NAME = {n: n.replace("solid0.", "solid.") for n in EXACT + FLOAT}


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["scene"]))
    log = json.loads(str(z["log"]))
    solids = [SolidDesc(center=tuple(s["center"]), radius=s["radius"], density=s["density"],
                        E=s["E"], nu=s["nu"], velocity=tuple(s["velocity"]),
                        plastic_yield=s.get("plastic_yield", -1.0),
                        rotation=tuple(s.get("rotation", (0.0, 0.0, 0.0))),
                        scaling=tuple(s.get("scaling", (1.0, 1.0, 1.0))),
                        rotation_matrix=s.get("rotation_matrix"),
                        asset=s.get("asset", "")) for s in meta["solids"]]
    if any(s.asset == "shipped_sphere" for s in solids):
        register_shipped_sphere()
    desc = SceneDesc(N=meta["N"], mass_sample_dh=meta["mass_sample_dh"],
                     vorticity_eps=meta["vorticity_eps"], buoyancy=meta["buoyancy"],
                     noise_seed=meta["noise_seed"], flow_rate=meta.get("flow_rate", 0.5),
                     solids=solids)
    return desc, z, log


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    scale = np.abs(b).max() if b.size else 0.0
    if scale == 0:
        return float(np.abs(a - b).max()) if a.size else 0.0
    return float(np.abs(a - b).max() / scale)


def csr_to_blocks(indptr, indices, data, sdof, X, Y):
    """The reference's _systemMatrix (CSR over 3S rows) as per-solid-node
    27-neighbour 3x3 blocks and a structural mask (bit j = block present)."""
    S = len(indptr) // 3
    node_of = np.empty(S, dtype=np.int64)
    idx = np.nonzero(sdof >= 0)[0]
    node_of[sdof[idx]] = idx
    blocks = np.zeros((S, 27, 3, 3))
    mask = np.zeros(S, dtype=np.int64)
    for r in range(3 * S):
        a = r // 3
        na = node_of[a]
        ax, ay, az = na % X, (na // X) % Y, na // (X * Y)
        for e in range(indptr[r], indptr[r + 1]):
            c = indices[e]
            nb = node_of[c // 3]
            bx, by, bz = nb % X, (nb // X) % Y, nb // (X * Y)
            j = (bx - ax + 1) + 3 * (by - ay + 1) + 9 * (bz - az + 1)
            blocks[a, j, r % 3, c % 3] = data[e]
            mask[a] |= 1 << j
    return blocks, mask.astype(np.int32)


def compare_to_golden(get, z, step, tol, fields=None, skip=()):
    """Compare an integrator's state (get(name) -> array) with the golden
    state after `step` (0 = after init). Returns a list of failure strings."""
    fails = []
    pre = f"s{step}."
    for g in EXACT:
        if g in skip or pre + g not in z.files:
            continue
        mine = np.asarray(get(NAME[g])).reshape(-1)
        ref = z[pre + g].reshape(-1)
        if mine.shape != ref.shape or not np.array_equal(mine, ref.astype(mine.dtype)):
            bad = np.count_nonzero(mine != ref) if mine.shape == ref.shape else "shape"
            fails.append(f"{pre}{g}: not bit-exact ({bad})")
    for g in (fields or FLOAT):
        if g in skip or pre + g not in z.files:
            continue
        ref = z[pre + g]
        mine = np.asarray(get(NAME[g]))
        if mine.size != ref.size:
            fails.append(f"{pre}{g}: size {mine.size} != {ref.size}")
            continue
        if g == "solid0.particles":
            # positions, velocities, rest positions, mass
            e = rel_err(mine.reshape(-1, 10)[:, :9], ref.reshape(-1, 10)[:, :9])
        else:
            e = rel_err(mine, ref)
        if not e <= tol:
            fails.append(f"{pre}{g}: rel err {e:.3e} > {tol:.1e}")
    return fails


# ------------------------------------------- benchmark-sized (compact) fixtures
BIG_SCENES = ["config1_64", "config2_128"]
# fixture name -> integrator field name
BIG_NAME = {"velocity": "velocity", "lambda1": "lambda1", "intensity": "intensity",
            "nodeSolidVolumeFraction": "nodeSolidVolumeFraction", "solid0.u": "solid.u",
            "solid0.velocity": "solid.velocity", "solid0.mass": "solid.mass",
            "solid0.meshVertices": "solid.meshVertices"}


def load_big(name):
    """A compact fixture of tests/golden/make_golden.py --big: (desc, z, log, meta)."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["scene"]))
    log = json.loads(str(z["log"]))
    solids = [SolidDesc(center=tuple(s["center"]), radius=s["radius"], density=s["density"],
                        E=s["E"], nu=s["nu"], velocity=tuple(s["velocity"])) for s in meta["solids"]]
    desc = SceneDesc(N=meta["N"], mass_sample_dh=meta["mass_sample_dh"],
                     vorticity_eps=meta["vorticity_eps"], buoyancy=meta["buoyancy"],
                     noise_seed=meta["noise_seed"], solids=solids)
    return desc, z, log, meta


def compare_big(get, z, step, tol):
    """Compare an integrator's state after `step` with a compact fixture.
    Integer maps/flags bit-exact; each floating-point field's max |.| and
    L2 norm within `tol` relative; at the stored steps, the sampled nodes and
    cells and the solid nodes within `tol` of the field's max |.| (the
    max-norm relative error of the full fields, restricted to those points).
    Returns (failures, {field: worst relative error})."""
    fails, worst = [], {}
    pre = f"s{step}."
    exact = ["gridIdxToSolidIdx", "solid0.valid", "solid0.boxes"]
    if step == 0:
        exact.append("gridIdxToSolutionIdx")
    for f in exact:
        mine = np.asarray(get(NAME[f])).reshape(-1)
        ref = z[pre + f].reshape(-1)
        if mine.shape != ref.shape or not np.array_equal(mine, ref.astype(mine.dtype)):
            bad = np.count_nonzero(mine != ref) if mine.shape == ref.shape else "shape"
            fails.append(f"{pre}{f}: not bit-exact ({bad})")
    sdof = z[pre + "gridIdxToSolidIdx"].reshape(-1)
    nodes, cells = z["sample.nodes"], z["sample.cells"]
    for f, name in BIG_NAME.items():
        if pre + f + ".stats" not in z.files:
            continue
        a = np.asarray(get(name), dtype=np.float64)
        ref_max, _, ref_sq = z[pre + f + ".stats"]
        mine_max, mine_sq = float(np.abs(a).max()), float((a.reshape(-1) ** 2).sum())
        scale = ref_max if ref_max > 0 else 1.0
        errs = [abs(mine_max - ref_max) / scale,
                abs(np.sqrt(mine_sq) - np.sqrt(ref_sq)) / (np.sqrt(ref_sq) or 1.0)]
        # node fields: one row per grid node; lambda1: one value per cell
        comp = a.reshape(-1) if f in ("lambda1", "solid0.meshVertices") else a.reshape(len(sdof), -1)
        if pre + f + ".sample" in z.files:
            pts = cells if f == "lambda1" else nodes
            errs.append(float(np.abs(comp[pts].reshape(-1) - z[pre + f + ".sample"].reshape(-1)).max()) / scale)
        if pre + f + ".solid" in z.files:
            errs.append(float(np.abs(comp[sdof >= 0].reshape(-1) - z[pre + f + ".solid"].reshape(-1)).max()) / scale)
        if pre + f in z.files:
            errs.append(float(np.abs(a.reshape(-1) - z[pre + f].reshape(-1)).max()) / scale)
        worst[f] = max(errs)
        if not worst[f] <= tol:
            fails.append(f"{pre}{f}: rel err {worst[f]:.3e} > {tol:.1e}")
    return fails, worst
