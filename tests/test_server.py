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


def test_batch_needs_a_gpu(ds):
    """No GPU here: creating a batch reports DEMSPH_ERR_NO_DEVICE."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(ds.DemSphError) as e:
        ds.Batch(0)
    assert e.value.status == 4


@pytest.mark.gpu
@pytest.mark.parametrize("graphs,batch", [(0, False), (1, False), (-1, False), (0, True)])
def test_mix_equals_alone(ds, scenes, graphs, batch):
    """In the mix, scenes launch directly (graphs 0: several are active; -1),
    replay graphs (1), or advance together in one graph launch per round
    (batch); each result has the bits of the scene run alone from graphs."""
    built = [(ds.build_scene(getattr(scenes, name)()), steps) for name, steps in MIX]
    srv = ds.Server(workers=4, chunk_steps=7, graphs=graphs, batch=batch, batch_round_steps=10)
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


def _batched(ds, built, rounds, **opts):
    """Engines of `built` [(scene, steps)] advanced by a Batch in rounds of
    (at most) the given lengths, cycling; returns the engines and the batch."""
    engines = [ds.Engine(sc, **opts) for sc, _ in built]
    for e in engines:
        e.initialize()
    b = ds.Batch(0)
    nxt = [1] * len(built)
    r = 0
    while any(n <= steps for n, (_, steps) in zip(nxt, built)):
        live = [k for k, (sc, steps) in enumerate(built) if nxt[k] <= steps]
        ln = [min(rounds[r % len(rounds)], built[k][1] - nxt[k] + 1) for k in live]
        st = b.update([engines[k] for k in live], [nxt[k] for k in live], ln,
                      [built[k][0].time_step for k in live], [built[k][0].fluid_integrate_gap for k in live])
        assert st == [0] * len(live)
        for k, n in zip(live, ln):
            nxt[k] += n
        r += 1
    return engines, b


def _state(eng, sc):
    f = eng.download_fluids() if sc.n_fluid else None
    s = eng.download_solids() if sc.n_solid else None
    return f, s


def _equal(a, b):
    (fa, sa), (fb, sb) = a, b
    if fa is not None:
        for x, y in zip(fa, fb):
            assert np.array_equal(x, y)
    if sa is not None:
        for k in ("pos", "vel", "angvel", "acc", "torque"):
            assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.gpu
def test_batch_rounds_equal_alone(ds, scenes):
    """demsph_batch_update over scenes of different kinds and gaps, rounds of
    odd and even lengths, from step 1: every state equals the scene run alone,
    bit for bit."""
    built = [(sc, steps) for ((_, sc), steps) in [(ds.build_scene(getattr(scenes, n)()), st) for n, st in MIX]]
    engines, b = _batched(ds, built, [7, 10, 3, 30])
    for e, (sc, steps) in zip(engines, built):
        alone = ds.Engine(sc)
        alone.initialize()
        alone.update(sc.time_step, 1, steps, sc.fluid_integrate_gap, use_graph=True)
        _equal(_state(e, sc), _state(alone, sc))
    assert b.info()["launches"] > 0


@pytest.mark.gpu
def test_batch_reuses_its_graph_for_repeating_rounds(ds, scenes):
    """Rounds that are whole Shepard periods of even length repeat: after the
    first rounds the same executable graph is launched again."""
    _, a = ds.build_scene(scenes.tiny_dam_break())
    _, c = ds.build_scene(scenes.tiny_granular())
    built = [(a, 1 + 8 * 10), (c, 1 + 8 * 10)]
    engines = [ds.Engine(sc) for sc, _ in built]
    for e, (sc, _) in zip(engines, built):
        e.initialize()
        e.update(sc.time_step, 1, 1, sc.fluid_integrate_gap)
    b = ds.Batch(0)
    for r in range(8):
        st = b.update(engines, [2 + 10 * r] * 2, [10, 10], [a.time_step, c.time_step],
                      [a.fluid_integrate_gap, c.fluid_integrate_gap])
        assert st == [0, 0]
    with pytest.raises(ds.DemSphError) as e:  # an engine twice in one launch
        b.update([engines[0], engines[0]], [82, 82], [2, 2], [a.time_step] * 2, [a.fluid_integrate_gap] * 2)
    assert e.value.status == 1
    info = b.info()
    # a list growth in the first rounds drops the member's graphs (a rebuild)
    assert info["launches"] == 8 and info["graph_builds"] <= 3 and info["members"] == 2


@pytest.mark.gpu
def test_batch_member_overflow_grows_and_matches(ds, scenes):
    """Lists too small for the scene: members overflow inside the batched
    round, grow their lists, finish the round alone and end bit for bit where
    the same engine options end alone."""
    opts = dict(fluid_neighbors_max=8, fluid_solids_max=2, solid_contacts_per_particle=1)
    built = [(ds.build_scene(scenes.tiny_coupled())[1], 40), (ds.build_scene(scenes.tiny_granular())[1], 40)]
    engines, _ = _batched(ds, built, [20], **opts)
    grown = 0
    for e, (sc, steps) in zip(engines, built):
        grown += e.run_stats()["list_growths"]
        alone = ds.Engine(sc, **opts)
        alone.initialize()
        alone.update(sc.time_step, 1, steps, sc.fluid_integrate_gap, use_graph=True)
        _equal(_state(e, sc), _state(alone, sc))
    assert grown > 0
