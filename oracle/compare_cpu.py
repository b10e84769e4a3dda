"""Times one coupled step of the same synthetic scene with the reference's
own OpenMP build (oracle/_ref/ref_harness_omp, from `make -C oracle omp`)
and with the oracle port (oracle/esf_oracle.c), on this machine's cores.
TEST INFRASTRUCTURE ONLY: it calibrates the CPU baseline that bench.py
measures with the port (the reference's build does not exist on the GPU
host), and is never part of the product.

    OMP_NUM_THREADS=8 python oracle/compare_cpu.py [N]
"""
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.dirname(HERE), HERE]

from eulersf_gb300.scene import SceneDesc, write_scene  # noqa: E402

import oracle  # noqa: E402


def main(N=48):
    desc = SceneDesc(N=N, mass_sample_dh=(1.0 / N) / 4, noise_seed=7)
    tmp = tempfile.mkdtemp(prefix="esf_cpu_")
    cfg = write_scene(desc, os.path.join(tmp, "scene"))
    harness = os.path.join(HERE, "_ref", "ref_harness_omp")
    subprocess.run([harness, cfg, os.path.join(tmp, "dump"), "1", "--noise",
                    os.path.join(tmp, "scene", "noise.f64"), "--no-dump"], check=True,
                   stdout=subprocess.DEVNULL)
    log = [json.loads(l) for l in open(os.path.join(tmp, "dump", "log.jsonl"))][1:]
    O = oracle.scene(desc)
    t0 = time.perf_counter()
    r = O.stepImplicit()
    port = time.perf_counter() - t0
    ref = log[0]
    print(json.dumps({"N": N, "threads": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count())),
                      "reference_step_s": ref["seconds"], "reference_iterations":
                      ref["solid_iters"][:1] + ref["pressure_iters"] + ref["solid_iters"][1:],
                      "port_step_s": port, "port_iterations": r["iterations"],
                      "port_over_reference_speed": ref["seconds"] / port}))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 48)
