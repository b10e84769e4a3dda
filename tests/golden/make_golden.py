"""Generate the golden fixtures of tests/golden/ by running the reference's own
CPU implementation (oracle/_ref/ref_harness, built by oracle/Makefile from
the unmodified EULERSF sources) on small synthetic scenes.

    make -C oracle REF=/path/to/EULERSF && python tests/golden/make_golden.py [scene ...]

Each scene is written as <name>.npz holding the initial state (s0.*) and the
state after every step (s<k>.*) for the fields listed below, plus the step
log (iterations per solve, dt, energy) as JSON text.
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
    return out


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


def main():
    if not os.path.exists(HARNESS):
        sys.exit(f"{HARNESS} missing: build it with make -C oracle")
    only = sys.argv[1:]  # optional scene names
    for name, (desc, frames) in scenes().items():
        if only and name not in only:
            continue
        run(name, desc, frames, HERE)
        print(name, os.path.getsize(os.path.join(HERE, name + ".npz")), "bytes")


if __name__ == "__main__":
    main()
