"""The scene server (demsph_server_*): many scenes on one GPU, admitted by a
device-memory budget and advanced together.  Each scene's result is the same,
bit for bit, alone and in the mix; the budget is never exceeded; requests
that arrive while others run are admitted as memory frees up."""
import time

import numpy as np
import pytest

MIX = (("tiny_coupled", 60), ("tiny_granular", 45), ("tiny_dam_break", 30), ("tiny_escape", 50),
       ("tiny_coupled", 23))


def _alone(ds, sc, steps):
    eng = ds.Engine(sc)
    eng.initialize()
    eng.update(sc.time_step, 1, steps, sc.fluid_integrate_gap, use_graph=True)
    f = eng.download_fluids() if sc.n_fluid else None
    s = eng.download_solids() if sc.n_solid else None
    return f, s


def _same(res, f, s):
    if f is not None:
        assert np.array_equal(res["fluid_pos"], f[0])
        assert np.array_equal(res["fluid_vel"], f[1])
        assert np.array_equal(res["fluid_drho"], f[3])
    if s is not None:
        assert np.array_equal(res["solid_pos"], s["pos"])
        assert np.array_equal(res["solid_vel"], s["vel"])
        assert np.array_equal(res["solid_angvel"], s["angvel"])


def test_server_reports_failure_without_a_gpu(ds, scenes):
    """No GPU here: an admitted scene fails with the engine's status, its memory
    is released and the server stays usable (the host-side failure path)."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    _, sc = ds.build_scene(scenes.tiny_coupled())
    srv = ds.Server(workers=2)
    try:
        rid = srv.submit(sc, 5)
        with pytest.raises(ds.DemSphError) as e:
            srv.wait(rid, 30.0)
        assert e.value.status == 4  # DEMSPH_ERR_NO_DEVICE
        st = srv.stats()
        assert st["failed"] == 1 and st["bytes_in_use"] == 0
        assert srv.info(rid)["state"] == "failed"
        srv.release(rid)
        with pytest.raises(ds.DemSphError):
            srv.info(rid)
    finally:
        srv.close()


def test_server_rejects_an_unknown_graph_mode(ds):
    for bad in (2, -2):
        with pytest.raises(ds.DemSphError) as e:
            ds.Server(workers=1, graphs=bad)
        assert e.value.status == 1  # DEMSPH_ERR_ARGUMENT


def test_server_rejects_a_scene_over_the_budget(ds, scenes):
    _, sc = ds.build_scene(scenes.tiny_coupled())
    srv = ds.Server(workers=1, hbm_budget_bytes=ds.estimate_bytes(sc) // 2)
    try:
        with pytest.raises(ds.DemSphError) as e:
            srv.submit(sc, 5)
        assert e.value.status == 5  # DEMSPH_ERR_CAPACITY
    finally:
        srv.close()


@pytest.mark.gpu
@pytest.mark.parametrize("graphs", [0, 1, -1])
def test_mix_equals_alone(ds, scenes, graphs):
    """In the mix, scenes launch directly (graphs 0: several are active; -1)
    or replay graphs (1); each result has the bits of the scene run alone
    from graphs."""
    built = [(ds.build_scene(getattr(scenes, name)()), steps) for name, steps in MIX]
    srv = ds.Server(workers=4, chunk_steps=7, graphs=graphs)
    try:
        ids = [srv.submit(sc, steps) for (_, sc), steps in built]
        srv.wait(-1, 600.0)
        st = srv.stats()
        assert st["completed"] == len(MIX) and st["failed"] == 0
        assert st["steps"] == sum(steps for _, steps in MIX)
        assert st["p99_step_ms"] >= st["p50_step_ms"] > 0
        for rid, ((_, sc), steps) in zip(ids, built):
            _same(srv.fetch(rid), *_alone(ds, sc, steps))
    finally:
        srv.close()


@pytest.mark.gpu
def test_budget_admits_in_order_and_is_never_exceeded(ds, scenes):
    built = [ds.build_scene(scenes.tiny_coupled(seed=k)) for k in range(4)]
    one = max(int(ds.estimate_bytes(sc) * 1.25) + 1 for _, sc in built)
    srv = ds.Server(workers=4, hbm_budget_bytes=int(one * 1.5))  # room for one scene at a time
    try:
        ids = [srv.submit(sc, 40) for _, sc in built]
        srv.wait(-1, 600.0)
        st = srv.stats()
        assert st["completed"] == 4 and st["peak_bytes"] <= int(one * 1.5)
        infos = [srv.info(i) for i in ids]
        assert infos[-1]["queued_s"] > 0.0  # waited for memory
        for rid, (_, sc) in zip(ids, built):
            _same(srv.fetch(rid), *_alone(ds, sc, 40))
    finally:
        srv.close()


@pytest.mark.gpu
def test_late_arrivals_join_running_scenes(ds, scenes):
    """Continuous batching: requests submitted while others are on the GPU are
    admitted and finish with the same results as alone."""
    _, big = ds.build_scene(scenes.tiny_coupled())
    late = [ds.build_scene(scenes.tiny_granular(seed=k)) for k in range(3)]
    srv = ds.Server(workers=4, chunk_steps=10)
    try:
        first = srv.submit(big, 400)
        while srv.info(first)["steps_done"] == 0:
            time.sleep(0.01)
        ids = [srv.submit(sc, 30) for _, sc in late]
        srv.wait(-1, 600.0)
        assert srv.info(first)["state"] == "done"
        for rid, (_, sc) in zip(ids, late):
            assert srv.info(rid)["state"] == "done"
            _same(srv.fetch(rid), *_alone(ds, sc, 30))
    finally:
        srv.close()


@pytest.mark.gpu
def test_autotune_choice_is_used_bit_for_bit(ds, scenes):
    """demsph_autotune picks the threads per fluid particle; an engine created
    with that choice follows the autotuned one bit for bit."""
    _, sc = ds.build_scene(scenes.tiny_coupled())
    a = ds.Engine(sc)
    a.initialize()
    lanes = a.autotune()
    assert lanes in (1, 2, 4, 8)
    b = ds.Engine(sc, fluid_lanes=lanes)
    b.initialize()
    for e in (a, b):
        e.update(sc.time_step, 1, 40, sc.fluid_integrate_gap)
    for x, y in zip(a.download_fluids(), b.download_fluids()):
        assert np.array_equal(x, y)


@pytest.mark.gpu
def test_autotuning_server_completes_the_mix(ds, scenes):
    built = [(ds.build_scene(getattr(scenes, name)()), steps) for name, steps in MIX]
    srv = ds.Server(workers=4, chunk_steps=9, autotune=True)
    try:
        ids = [srv.submit(sc, steps) for (_, sc), steps in built]
        srv.wait(-1, 600.0)
        assert srv.stats()["completed"] == len(MIX)
        for rid, ((_, sc), steps) in zip(ids, built):
            got = srv.fetch(rid)
            f, s = _alone(ds, sc, steps)
            if f is not None:  # the lane count may differ from the default: same physics to rounding
                assert np.allclose(got["fluid_pos"], f[0], rtol=0, atol=1e-9)
            if s is not None:
                assert np.allclose(got["solid_pos"], s["pos"], rtol=0, atol=1e-9)
    finally:
        srv.close()
