"""Binary frame files (demsph_frame_writer_*): the reference's fluid_,
solid_ and fluid2Solid_NNNN.vtu (core/solverBase.cpp:69-333) written by a
background thread.  Each array must equal the engine's own FP64 state
(downloads and the fluid2Solid export) rounded once to FP32, for frames taken
while later steps are already enqueued."""
import numpy as np
import pytest

from vtu import read_vtu

pytestmark = pytest.mark.gpu


def _state(eng, sc):
    fp, fv, _, fd = eng.download_fluids()
    s = eng.download_solids()
    pairs = eng.fluid_solid_pairs()
    return fp, fv, fd, s, pairs


def _check_frame(tmp, frame, step, time, sc, st):
    fp, fv, fd, s, pairs = st
    n = sc.n_fluid
    rho0 = np.ctypeslib.as_array(sc.fluid_rho0, shape=(n,))
    c = np.ctypeslib.as_array(sc.fluid_sound_speed, shape=(n,))
    h = np.ctypeslib.as_array(sc.fluid_smoothing_length, shape=(n,))
    f = read_vtu(tmp / f"fluid_{frame:04d}.vtu")
    assert f["STEP"] == step and abs(f["TIME"] - time) <= 1e-9 * max(1.0, abs(time))
    assert np.array_equal(f["Points"], fp.astype(np.float32))
    assert np.array_equal(f["velocity"], fv.astype(np.float32))
    assert np.array_equal(f["smooth length"], h.astype(np.float32))
    np.testing.assert_allclose(f["density"], (rho0 + fd).astype(np.float32), rtol=3e-7)
    np.testing.assert_allclose(f["pressure"], fd * c * c, rtol=1e-6, atol=1e-6 * np.abs(fd * c * c).max())
    assert np.array_equal(f["connectivity"], np.arange(n)) and np.array_equal(f["offsets"], np.arange(1, n + 1))
    assert np.all(f["types"] == 1)
    ns = sc.n_solid
    g = read_vtu(tmp / f"solid_{frame:04d}.vtu")
    assert np.array_equal(g["Points"], s["pos"].astype(np.float32))
    assert np.array_equal(g["velocity"], s["vel"].astype(np.float32))
    assert np.array_equal(g["angularVelocity"], s["angvel"].astype(np.float32))
    assert np.array_equal(g["normal"], s["normal"].astype(np.float32))
    assert np.array_equal(g["radius"], np.ctypeslib.as_array(sc.solid_radius, shape=(ns,)).astype(np.float32))
    assert np.array_equal(g["clusterID"], np.ctypeslib.as_array(sc.solid_cluster, shape=(ns,)))
    assert np.array_equal(g["clumpID"], np.ctypeslib.as_array(sc.solid_clump, shape=(ns,)))
    p = read_vtu(tmp / f"fluid2Solid_{frame:04d}.vtu")
    a, b = pairs["pointed"], pairs["pointing"]
    assert len(a) > 0
    mid = 0.5 * (fp[a] + s["pos"][b])
    assert np.array_equal(p["Points"], mid.astype(np.float32))
    assert np.array_equal(p["force"], pairs["force"].astype(np.float32))


def test_binary_frames_equal_the_engine_state(ds, scenes, tmp_path):
    b, sc = ds.build_scene(scenes.tiny_coupled())
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    eng = ds.Engine(sc, debug=1)  # keeps the per-pair coupling forces
    eng.initialize()
    states = []
    with ds.FrameWriter(eng, tmp_path) as fw:
        step = 0
        for frame in range(4):
            fw.write(ds.FRAME_ALL, frame, step, step * dt)
            states.append((frame, step, step * dt, _state(eng, sc)))
            # the steps run while the writer thread copies and writes the frame
            eng.update(dt, step + 1, 2 * gap, gap, use_graph=True)
            step += 2 * gap
        fw.flush()
    for frame, step, t, st in states:
        _check_frame(tmp_path, frame, step, t, sc, st)
    eng.close()


def test_writer_errors_are_reported(ds, scenes, tmp_path):
    b, sc = ds.build_scene(scenes.tiny_coupled())
    eng = ds.Engine(sc)
    eng.initialize()
    blocker = tmp_path / "file"
    blocker.write_text("x")
    with pytest.raises(ds.DemSphError):
        ds.FrameWriter(eng, blocker / "sub")  # a directory below a file cannot be made
    fw = ds.FrameWriter(eng, tmp_path / "out")
    with pytest.raises(ds.DemSphError):
        fw.write(8, 0, 0, 0.0)  # no such kind
    fw.write(ds.FRAME_FLUID, 0, 0, 0.0)
    fw.close()
    assert (tmp_path / "out" / "fluid_0000.vtu").exists()
    eng.close()
