"""The multi-scene server (esf_server_*): each request's result is the same,
bit for bit, whether it runs alone or concurrently with others, with its
inner solves batched with the other scenes' of its grid shape (continuous
batching) or run on its own stream; admission holds a request back until the
memory budget has room; a request larger than the budget is refused."""
import ctypes as C

import numpy as np
import pytest

from eulersf_gb300 import abi
from eulersf_gb300.scene import SceneDesc

pytestmark = pytest.mark.gpu


def _descs():
    return [SceneDesc(N=16, mass_sample_dh=(1.0 / 16) / 4, noise_seed=1),
            SceneDesc(N=20, mass_sample_dh=(1.0 / 20) / 4, noise_seed=2),
            SceneDesc(N=16, mass_sample_dh=(1.0 / 16) / 4, noise_seed=3, fluid_height=0.25)]


def test_concurrent_requests_equal_solo_runs(gpu_lib):
    import eulersf_gb300 as E
    from eulersf_gb300.serve import ESF_REQ_DONE, Server
    descs, steps = _descs(), 2
    with Server(max_active=3) as srv:
        tickets = [srv.submit(d, steps, abi.ESF_MIXED) for d in descs]
        got = []
        for d, t in zip(descs, tickets):
            st = srv.wait(t)
            assert st["state"] == ESF_REQ_DONE and st["steps_done"] == steps, st
            got.append((srv.get(t, "velocity", d.res ** 3 * 3), srv.get(t, "lambda1", d.N ** 3),
                         st["last"]["iterations"]))
            srv.release(t)
        stats = srv.batch_stats()
    # the two 16^3 scenes' inner solves went through the batcher
    assert stats["inner_solves"] > 0 and stats["launches"] > 0, stats
    for d, (vel, lam, its) in zip(descs, got):
        G = E.make_scene(d, precision=abi.ESF_MIXED)
        for _ in range(steps):
            r = G.stepImplicit()
        assert its == r["iterations"]
        assert np.array_equal(vel, G.get("velocity")), d
        assert np.array_equal(lam, G.get("lambda1")), d
        G.close()


def test_admission_waits_for_budget_and_refuses_oversize(gpu_lib):
    from eulersf_gb300.serve import Server, request_for
    d = _descs()[0]
    q, keep = request_for(d, 1)
    one = gpu_lib.esf_scene_footprint(C.byref(q.grid), C.byref(q.params), q.num_solids, q.solids)
    assert one > 0
    with Server(hbm_budget_bytes=int(one * 1.5), max_active=4) as srv:
        a, b = srv.submit(d, 1), srv.submit(d, 1)
        sa = srv.wait(a)
        assert sa["state"] == 2
        assert srv.poll(b)["state"] == 0  # still queued: a holds the budget until released
        srv.release(a)
        sb = srv.wait(b)
        assert sb["state"] == 2 and sb["steps_done"] == 1
        srv.release(b)
        with pytest.raises(abi.EsfError) as e:
            srv.submit(SceneDesc(N=64), 1)
        assert e.value.status == 4  # ESF_ERR_OOM


def test_batched_and_unbatched_serving_agree(gpu_lib):
    """The same requests through a server without batching (each scene's
    inner solves on its own stream): the same bits as batched."""
    from eulersf_gb300.serve import Server
    descs, steps = _descs(), 2
    out = {}
    for batching in (True, False):
        with Server(max_active=3, batching=batching) as srv:
            tickets = [srv.submit(d, steps, abi.ESF_MIXED) for d in descs]
            res = []
            for d, t in zip(descs, tickets):
                st = srv.wait(t)
                assert st["state"] == 2, st
                res.append((srv.get(t, "velocity", d.res ** 3 * 3), st["last"]["iterations"]))
                srv.release(t)
            if not batching:
                assert srv.batch_stats()["launches"] == 0
        out[batching] = res
    for (va, ia), (vb, ib) in zip(out[True], out[False]):
        assert ia == ib
        assert np.array_equal(va, vb)


def test_two_solid_request_equals_solo_run(gpu_lib):
    """A served scene with two solids (each with its rest SDF path in the
    request) gives the same bits as the same scene stepped alone; a
    two-solid request without rest SDF paths is refused at submit."""
    import eulersf_gb300 as E
    from common import load_golden
    from eulersf_gb300.serve import ESF_REQ_DONE, Server, request_for
    desc, _, _ = load_golden("contact20")
    steps = 2
    with Server(max_active=2) as srv:
        t = srv.submit(desc, steps, abi.ESF_FP64)
        st = srv.wait(t)
        assert st["state"] == ESF_REQ_DONE and st["steps_done"] == steps, st
        vel = srv.get(t, "velocity", desc.res ** 3 * 3)
        srv.release(t)
        q, keep = request_for(desc, steps, abi.ESF_FP64)
        q.rest_sdf_paths = None
        tk = C.c_uint64()
        assert srv._lib.esf_server_submit(srv._h, C.byref(q), C.byref(tk)) == 1  # ESF_ERR_INVALID_ARG
        del keep
    G = E.make_scene(desc)
    for _ in range(steps):
        G.stepImplicit()
    assert np.array_equal(vel, G.get("velocity"))
    G.close()
