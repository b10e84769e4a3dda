"""Generate the golden fixtures of tests/golden/ by running the reference's own
CPU implementation (oracle/_ref/ref_harness, built by oracle/Makefile from
the unmodified EULERSF sources) on small synthetic scenes.

    make -C oracle REF=/path/to/EULERSF && python tests/golden/make_golden.py [scene ...]

Each scene is written as <name>.npz holding the initial state (s0.*) and the
state after every step (s<k>.*) for the fields listed below, plus the step
log (iterations per solve, dt, energy) as JSON text.

The benchmark-sized scenes (64^3 for 20 steps, 128^3 for a 2-step prefix)
run the reference's OpenMP build (``make -C oracle omp``) and are stored in a
compact form (``compact()``): the DOF maps and cell flags of every step in
full, per-step statistics of the floating-point fields, and at a few steps
the grid fields at a fixed seeded sample of nodes and cells and the solid's
fields at every solid node:

    python tests/golden/make_golden.py --big config1_64 config2_128 [--keep DIR]

and the reference's own frame files with a restart from them (``run_frame``),
and its offline mass baking of the shipped sphere (``run_mass``,
``make -C oracle rasterize`` first):

    python tests/golden/make_golden.py --frame
    python tests/golden/make_golden.py --mass

and a two-ball scene with solid-solid contact (``run_contact``):

    python tests/golden/make_golden.py --contact

``--keep DIR`` keeps the harness's raw dumps there and reuses a completed run.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from eulersf_gb300.scene import SceneDesc, SolidDesc, write_scene  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
HARNESS_OMP = os.path.join(ROOT, "oracle", "_ref", "ref_harness_omp")


def scenes():
    """name -> (SceneDesc, frames)."""
    out = {}
    out["ball16"] = (SceneDesc(N=16, mass_sample_dh=(1 / 16) / 4), 3)
    # vorticity confinement and buoyancy on (the benchmark scenes turn both off)
    out["ball20_vort"] = (SceneDesc(N=20, mass_sample_dh=(1 / 20) / 4, vorticity_eps=1.5,
                                    buoyancy=0.1, noise_seed=3), 2)
    # ball resting one cell above the floor, moving down: CFL factor 0.6 and
    # wall-contact impulses in gridToParticle
    out["wall20"] = (SceneDesc(N=20, mass_sample_dh=(1 / 20) / 4, noise_seed=5,
                               solids=[SolidDesc(center=(0.5, 0.2, 0.45), radius=0.14,
                                                 velocity=(0.0, -0.6, 0.0))]), 2)
    # plastic ball hitting the floor: stress above the yield, FpInv updated
    out["plastic20"] = (SceneDesc(N=20, mass_sample_dh=(1 / 20) / 4, noise_seed=7, flow_rate=0.5,
                                  solids=[SolidDesc(center=(0.5, 0.2, 0.45), radius=0.14,
                                                    velocity=(0.0, -0.6, 0.0), plastic_yield=40.0)]), 2)
    # rotated, non-uniformly scaled (pre-stretched) ball: setInitialState's
    # transform of X and of the mesh
    out["rot20"] = (SceneDesc(N=20, mass_sample_dh=(1 / 20) / 4, noise_seed=4,
                              solids=[SolidDesc(center=(0.5, 0.55, 0.5), radius=0.12,
                                                rotation=(0.1, 0.25, 0.4),
                                                scaling=(1.05, 0.95, 1.0))]), 2)
    # the reference's shipped sphere (meshes/sphere/sphere.obj) with the rest
    # mass its own rasterizeSolid tool baked (sphere_mass.npz, made by --mass)
    out["shipped20"] = (SceneDesc(N=20, mass_sample_dh=(1 / 20) / 4, noise_seed=2,
                                  solids=[SolidDesc(center=(0.5, 0.6, 0.5), radius=0.0995,
                                                    asset="shipped_sphere")]), 2)
    return out


def register_shipped_sphere():
    """The shipped sphere's mesh and tool-baked mass (sphere_mass.npz) as the
    rest assets "shipped_sphere"."""
    from eulersf_gb300.scene import register_assets
    z = np.load(os.path.join(HERE, "sphere_mass.npz"))
    res = [int(v) for v in z["res"]]
    n = res[0] * res[1] * res[2]
    data = np.unpackbits(z["solid"])[:n].astype(np.float64) * float(z["density"])
    register_assets("shipped_sphere", (res, float(z["dh"]), z["origin"].astype(np.float64),
                                       data.reshape(res[2], res[1], res[0])), z["vertices"], z["triangles"])


INIT_FIELDS = ["gridIdxToSolutionIdx", "gridIdxToSolidIdx", "velocity", "intensity", "solidMass",
               "nodeSolidVolumeFraction", "solid0.valid", "solid0.boxes", "solid0.mass",
               "solid0.phi", "solid0.u", "solid0.X", "solid0.particles", "solid0.meshVertices",
               "solid0.detFInv"]
STEP_FIELDS = ["gridIdxToSolidIdx", "velocity", "intensity", "lambda1",
               "nodeSolidVolumeFraction", "solid0.valid", "solid0.boxes", "solid0.mass",
               "solid0.phi", "solid0.u", "solid0.velocity", "solid0.meshVertices", "nzMassVecInv",
               "JMInvJTDiag", "b1", "velocityAtDt0", "solidUnitForce", "dampedSolidMassVec",
               "solidVelocityAtDt0", "systemMatrix.indptr", "systemMatrix.indices",
               "systemMatrix.data"]
LAST_STEP_FIELDS = ["solid0.particles"]
PLASTIC_FIELDS = ["solid0.FpInv", "solid0.FpInvGrid"]


def run(name, desc, frames, out_dir):
    tmp = tempfile.mkdtemp(prefix="esf_golden_")
    try:
        cfg = write_scene(desc, os.path.join(tmp, "scene"))
        dump = os.path.join(tmp, "dump")
        subprocess.run([HARNESS, cfg, dump, str(frames), "--noise",
                        os.path.join(tmp, "scene", "noise.f64")], check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        arrays = {}
        for f in INIT_FIELDS + PLASTIC_FIELDS:
            p = os.path.join(dump, f"s0.{f}.npy")
            if os.path.exists(p):
                arrays["s0." + f] = np.load(p)
        log = [json.loads(l) for l in open(os.path.join(dump, "log.jsonl"))][1:]
        for k in range(1, len(log) + 1):
            for f in STEP_FIELDS + PLASTIC_FIELDS + (LAST_STEP_FIELDS if k == len(log) else []):
                p = os.path.join(dump, f"s{k}.{f}.npy")
                if os.path.exists(p):
                    arrays[f"s{k}.{f}"] = np.load(p)
        for l in log:
            l.pop("seconds", None)
        arrays["log"] = np.array(json.dumps(log))
        solids = [dict(sd.__dict__) for sd in desc.solids]
        for i, sd in enumerate(solids):
            p = os.path.join(dump, f"s0.solid{i}.rotation.npy")
            if os.path.exists(p):  # the reference's own rotation matrix
                sd["rotation_matrix"] = [float(x) for x in np.load(p).reshape(-1)]
        arrays["scene"] = np.array(json.dumps({
            "N": desc.N, "mass_sample_dh": desc.mass_sample_dh, "vorticity_eps": desc.vorticity_eps,
            "buoyancy": desc.buoyancy, "noise_seed": desc.noise_seed, "frames": frames,
            "flow_rate": desc.flow_rate, "solids": solids}))
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **arrays)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


# Frame files: the reference writes its state after the last step
# (writeFrame, frame 0, debug), a second integrator reads them back (readFrame)
# and writes them again as frame 1, and takes one step. The fixture holds the
# frame files as written (gz bytes, OBJ text), the warm start the step used
# (the last solve's lambda1, a function-local static the frame does not
# carry) and the state after the read (r0.*) and after the step (r1.*).
FRAME_SCENE = ("frame16", SceneDesc(N=16, mass_sample_dh=(1 / 16) / 4, noise_seed=6), 2)
RESTART_FIELDS = ["gridIdxToSolidIdx", "velocity", "intensity", "lambda1", "solid0.valid", "solid0.boxes",
                  "solid0.mass", "solid0.phi", "solid0.u", "solid0.velocity", "solid0.meshVertices",
                  "solid0.particles", "nodeSolidVolumeFraction"]


def run_frame(out_dir):
    name, desc, frames = FRAME_SCENE
    tmp = tempfile.mkdtemp(prefix="esf_golden_")
    try:
        cfg = write_scene(desc, os.path.join(tmp, "scene"))
        dump, fdir = os.path.join(tmp, "dump"), os.path.join(tmp, "frames")
        subprocess.run([HARNESS, cfg, dump, str(frames), "--noise", os.path.join(tmp, "scene", "noise.f64"),
                        "--no-dump", "--frame-restart", fdir], check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        arrays = {}
        for f in sorted(os.listdir(fdir)):
            if f.endswith(".pbrt"):
                continue  # render export, not state
            with open(os.path.join(fdir, f), "rb") as fh:
                arrays["file." + f] = np.frombuffer(fh.read(), dtype=np.uint8)
        for pre in ("r0.", "r1."):
            for f in RESTART_FIELDS:
                p = os.path.join(dump, f"{pre}{f}.npy")
                if os.path.exists(p):
                    arrays[pre + f] = np.load(p)
        log = [json.loads(l) for l in open(os.path.join(dump, "log.jsonl"))][1:]
        for l in log:
            l.pop("seconds", None)
        arrays["log"] = np.array(json.dumps(log))
        arrays["log_restart"] = np.array(json.dumps(
            [json.loads(l) for l in open(os.path.join(dump, "log_restart.jsonl"))]))
        solids = [dict(sd.__dict__) for sd in desc.solids]
        arrays["scene"] = np.array(json.dumps({
            "N": desc.N, "mass_sample_dh": desc.mass_sample_dh, "vorticity_eps": desc.vorticity_eps,
            "buoyancy": desc.buoyancy, "noise_seed": desc.noise_seed, "frames": frames,
            "flow_rate": desc.flow_rate, "solids": solids}))
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **arrays)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


# Solid-solid contact: two balls moving towards each other, one grid cell
# apart, so that particles of each come within the contact distance of the
# other's rest SDF (the scene writer's ".svol" files, read by the reference
# through SPARSE_SDF) in the first steps. The fixture holds the state of both
# solids, the system matrix the two assemble together, and the contact query
# SPARSE_SDF::signedDistAndCurrentNormal alone at seeded rest points around
# each surface (after init).
CONTACT_SCENE = ("contact20", SceneDesc(
    N=20, mass_sample_dh=(1 / 20) / 4, noise_seed=8,
    solids=[SolidDesc(center=(0.335, 0.5, 0.5), radius=0.15, velocity=(0.8, 0.0, 0.0)),
            SolidDesc(center=(0.665, 0.52, 0.5), radius=0.15, velocity=(-0.8, 0.0, 0.0))]), 3)
CONTACT_STEP_FIELDS = ["gridIdxToSolidIdx", "velocity", "lambda1", "solidMass", "solidUnitForce",
                       "dampedSolidMassVec", "solidVelocityAtDt0", "systemMatrix.indptr",
                       "systemMatrix.indices", "systemMatrix.data"]
CONTACT_SOLID_FIELDS = ["valid", "boxes", "mass", "phi", "u", "velocity", "meshVertices"]


def contact_query_points(radius, count=4096, seed=5):
    """Rest points around a sphere's surface: seeded directions at distances
    within +-0.2 radius of it (the contact band and beyond), then 64 deep
    inside (below the band) and 64 far outside (beyond the volume's box)."""
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((count + 128, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    r = np.concatenate([radius * (1 + rng.uniform(-0.2, 0.2, count)),
                        radius * rng.uniform(0.0, 0.5, 64), radius * rng.uniform(2.0, 3.0, 64)])
    return d * r[:, None]


def run_contact(out_dir):
    name, desc, frames = CONTACT_SCENE
    tmp = tempfile.mkdtemp(prefix="esf_golden_")
    try:
        cfg = write_scene(desc, os.path.join(tmp, "scene"))
        dump = os.path.join(tmp, "dump")
        pts = contact_query_points(desc.solids[0].radius)
        qfile = os.path.join(tmp, "query.f64")
        pts.astype("<f8").tofile(qfile)
        safe = 0.5 * desc.dh  # "contact safe distance" default
        subprocess.run([HARNESS, cfg, dump, str(frames), "--noise", os.path.join(tmp, "scene", "noise.f64"),
                        "--sdf-query", qfile, repr(safe)], check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        arrays = {"sdfq.points": pts, "sdfq.safe": np.array(safe)}
        for i in range(len(desc.solids)):
            arrays[f"sdfq.solid{i}"] = np.load(os.path.join(dump, f"sdfq.solid{i}.npy"))
        log = [json.loads(l) for l in open(os.path.join(dump, "log.jsonl"))][1:]
        solids = [f"solid{i}." for i in range(len(desc.solids))]
        for k in range(0, len(log) + 1):
            step_fields = [f for f in CONTACT_STEP_FIELDS if k == 1 or not f.startswith("systemMatrix")]
            fields = (INIT_FIELDS if k == 0 else step_fields) + \
                [sp + f for sp in solids for f in CONTACT_SOLID_FIELDS + (["particles"] if k in (0, len(log)) else [])]
            for f in fields:
                p = os.path.join(dump, f"s{k}.{f}.npy")
                if os.path.exists(p):
                    arrays[f"s{k}.{f}"] = np.load(p)
        for l in log:
            l.pop("seconds", None)
        arrays["log"] = np.array(json.dumps(log))
        arrays["scene"] = np.array(json.dumps({
            "N": desc.N, "mass_sample_dh": desc.mass_sample_dh, "vorticity_eps": desc.vorticity_eps,
            "buoyancy": desc.buoyancy, "noise_seed": desc.noise_seed, "frames": frames,
            "flow_rate": desc.flow_rate, "solids": [dict(sd.__dict__) for sd in desc.solids]}))
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **arrays)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


# Mass baking: the reference's rasterizeSolid tool on its shipped sphere
# (meshes/sphere/sphere.obj and its DT-Grid SDF sphere.svol, cfg/sphere.cfg's
# mass dh 0.001 and density 1000). The fixture holds the mesh (vertices,
# 0-based triangles) and the baked grid (resolution, dh, origin, density and
# the nodes that carry mass as a bit mask).
RASTERIZE = os.path.join(ROOT, "oracle", "_ref", "rasterize_solid")


def read_obj(path):
    """Vertices and 0-based triangles of an OBJ ("f a/b/c ..." entries)."""
    verts, tris = [], []
    for line in open(path):
        t = line.split()
        if not t:
            continue
        if t[0] == "v":
            verts.append([float(x) for x in t[1:4]])
        elif t[0] == "f":
            tris.append([int(x.split("/")[0]) - 1 for x in t[1:4]])
    return np.array(verts, dtype=np.float64), np.array(tris, dtype=np.int32)


def run_mass(out_dir):
    from eulersf_gb300.scene import read_field_gz
    ref = os.environ.get("EULERSF_REFERENCE", "/root/reference")
    obj, svol = os.path.join(ref, "meshes/sphere/sphere.obj"), os.path.join(ref, "meshes/sphere/sphere.svol")
    tmp = tempfile.mkdtemp(prefix="esf_golden_")
    try:
        cfg = os.path.join(tmp, "sphere.cfg")
        with open(cfg, "w") as f:
            f.write(f"mesh file name = {obj}\nsdf file name = {svol}\n"
                    f"mass file name = {tmp}/sphere.mass\nsolid mass density = 1000\nmass dh = 0.001\n")
        subprocess.run([RASTERIZE, cfg], check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        res, dh, origin, data = read_field_gz(os.path.join(tmp, "sphere.mass"))
        verts, tris = read_obj(obj)
        np.savez_compressed(os.path.join(out_dir, "sphere_mass.npz"), vertices=verts, triangles=tris,
                            res=np.array(res), dh=np.array(dh), origin=np.array(origin), density=np.array(1000.0),
                            solid=np.packbits(data.reshape(-1) > 0), total=np.array(float(data.sum()) * dh ** 3))
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def big_scenes():
    """The rubber-ball scene at the benchmark's 64^3 and 128^3 sizes; the
    fluid-noise seed is 0 for both. The mass sample spacing divides dh by a
    power of two, so the reference's integer sample count per axis
    (DEFOR_SOLID_3D.cpp:583) is exact: dh/8 at 64^3 and dh/4 at 128^3, where
    dh/8 would make every subsample's mass (rest density 1000 x spacing^3 =
    9.3e-7) fall under the reference's fixed 1e-6 threshold and leave the
    solid massless.
    name -> (SceneDesc, steps, steps whose fields are stored, nodes sampled)."""
    return {
        "config1_64": (SceneDesc(N=64, mass_sample_dh=(1 / 64) / 8, noise_seed=0), 20,
                       (1, 5, 10, 15, 20), 1 << 14),
        "config2_128": (SceneDesc(N=128, mass_sample_dh=(1 / 128) / 4, noise_seed=0), 2, (1, 2), 1 << 15),
    }


# fields of the compact fixtures: integer maps/flags kept whole at every step;
# floating-point fields as whole-field statistics at every step and, at the
# stored steps, at a fixed seeded sample of nodes/cells (grid fields) or at
# every solid node (the solid's fields, which live on and near the solid)
BIG_EXACT = ["gridIdxToSolidIdx", "solid0.valid", "solid0.boxes"]
BIG_FLOAT = ["velocity", "lambda1", "solid0.u", "solid0.velocity", "solid0.mass", "intensity",
             "nodeSolidVolumeFraction", "solid0.meshVertices"]
NODE_FIELDS = ["velocity", "intensity", "nodeSolidVolumeFraction"]
CELL_FIELDS = ["lambda1"]
SOLID_FIELDS = ["solid0.u", "solid0.velocity", "solid0.mass"]


def field_stats(a):
    """max |a|, sum a, sum a^2 in FP64."""
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    return np.array([np.abs(a).max() if a.size else 0.0, a.sum(), (a * a).sum()])


def sample_indices(n, count, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, size=min(count, n), replace=False)).astype(np.int64)


def compact(dump, desc, steps, stored, sample):
    """The compact fixture of a benchmark-sized run (see the module docstring)."""
    arrays = {}
    X = desc.res
    nodes = sample_indices(X ** 3, sample, 1234)
    cells = sample_indices(desc.N ** 3, sample, 4321)
    arrays["sample.nodes"], arrays["sample.cells"] = nodes, cells
    for k in range(0, steps + 1):
        pre = f"s{k}."
        load = lambda f: np.load(os.path.join(dump, f"{pre}{f}.npy"))
        for f in BIG_EXACT + (["gridIdxToSolutionIdx"] if k == 0 else []):
            arrays[pre + f] = load(f)
        sdof = load("gridIdxToSolidIdx")
        for f in BIG_FLOAT:
            if not os.path.exists(os.path.join(dump, f"{pre}{f}.npy")):
                continue
            a = load(f)
            arrays[pre + f + ".stats"] = field_stats(a)
            if k not in stored:
                continue
            if f in NODE_FIELDS:
                arrays[pre + f + ".sample"] = a.reshape(X ** 3, -1)[nodes]
            elif f in CELL_FIELDS:
                arrays[pre + f + ".sample"] = a.reshape(-1)[cells]
            elif f in SOLID_FIELDS:
                arrays[pre + f + ".solid"] = a.reshape(X ** 3, -1)[sdof >= 0]
            else:
                arrays[pre + f] = a
    return arrays


def run_big(name, desc, steps, stored, sample, out_dir, keep=None):
    tmp = os.path.join(keep, name) if keep else tempfile.mkdtemp(prefix="esf_golden_")
    try:
        dump = os.path.join(tmp, "dump")
        log_path = os.path.join(dump, "log.jsonl")
        done = os.path.exists(log_path) and sum(1 for _ in open(log_path)) >= steps + 1
        if not done:
            cfg = write_scene(desc, os.path.join(tmp, "scene"))
            subprocess.run([HARNESS_OMP, cfg, dump, str(steps), "--noise",
                            os.path.join(tmp, "scene", "noise.f64"), "--full-every", "1000000"],
                           check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        log = [json.loads(l) for l in open(log_path)][1:]
        if len(log) != steps:
            raise RuntimeError(f"{name}: {len(log)} steps in {steps} frames (substeps)")
        arrays = compact(dump, desc, steps, stored, sample)
        seconds = [l.pop("seconds", None) for l in log]
        arrays["log"] = np.array(json.dumps(log))
        solids = [dict(sd.__dict__) for sd in desc.solids]
        arrays["scene"] = np.array(json.dumps({
            "N": desc.N, "mass_sample_dh": desc.mass_sample_dh, "vorticity_eps": desc.vorticity_eps,
            "buoyancy": desc.buoyancy, "noise_seed": desc.noise_seed, "frames": steps,
            "flow_rate": desc.flow_rate, "solids": solids, "stored_steps": list(stored),
            "sample": sample, "reference_seconds_per_step": seconds,
            "reference_threads": os.cpu_count()}))
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **arrays)
    finally:
        if not keep:
            shutil.rmtree(tmp, ignore_errors=True)


def main():
    args = sys.argv[1:]
    register_shipped_sphere()
    if args and args[0] == "--contact":
        run_contact(HERE)
        print(CONTACT_SCENE[0], os.path.getsize(os.path.join(HERE, CONTACT_SCENE[0] + ".npz")), "bytes")
        return
    if args and args[0] == "--big":
        keep = None
        if "--keep" in args:
            i = args.index("--keep")
            keep = args[i + 1]
            del args[i:i + 2]
        if not os.path.exists(HARNESS_OMP):
            sys.exit(f"{HARNESS_OMP} missing: build it with make -C oracle omp")
        only = args[1:]
        for name, (desc, steps, full, sample) in big_scenes().items():
            if only and name not in only:
                continue
            run_big(name, desc, steps, full, sample, HERE, keep)
            print(name, os.path.getsize(os.path.join(HERE, name + ".npz")), "bytes")
        return
    if not os.path.exists(HARNESS):
        sys.exit(f"{HARNESS} missing: build it with make -C oracle")
    if args == ["--mass"]:
        run_mass(HERE)
        print("sphere_mass", os.path.getsize(os.path.join(HERE, "sphere_mass.npz")), "bytes")
        return
    if args == ["--frame"]:
        run_frame(HERE)
        print(FRAME_SCENE[0], os.path.getsize(os.path.join(HERE, FRAME_SCENE[0] + ".npz")), "bytes")
        return
    only = args  # optional scene names
    for name, (desc, frames) in scenes().items():
        if only and name not in only:
            continue
        run(name, desc, frames, HERE)
        print(name, os.path.getsize(os.path.join(HERE, name + ".npz")), "bytes")


if __name__ == "__main__":
    main()
