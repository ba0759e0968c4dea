"""The FP64 oracle against the reference's own solver.

The golden fixtures (tests/golden/*.npz) hold the reference's arrays after
initialisation and after 1, 2, 5 and 10 update() calls on three seeded scenes
(a dam break, a Hertz-Mindlin settle with clumps and walls, a coupled scene
with bonds and a fluid sub-cycling gap of 3).  They were produced by the
reference's own kernels compiled for the CPU (tests/golden/make_golden.py).
The oracle must reproduce every integer artefact exactly and every float to
1e-12 relative (the bound allows only libm last-bit differences between
machines).
"""
import os

import numpy as np
import pytest

from golden.make_golden import SCENES, load, scene_digest

HERE = os.path.dirname(os.path.abspath(__file__))
FLOAT_TOL = 1.0e-12


def _oracle(ds, scenes, name):
    from oracle.oracle import OracleSolver
    recipe = getattr(scenes, name)()
    b, sc = ds.build_scene(recipe)
    return b, sc, OracleSolver(sc)


def _compare(snap, orc, tag):
    for k, ref in snap.items():
        got = orc.get(k)
        assert got.shape == ref.shape, f"{tag} {k}: shape {got.shape} vs {ref.shape}"
        if ref.dtype.kind == "i":
            assert np.array_equal(got, ref), f"{tag} {k}: integer artefact differs"
        elif ref.size:
            scale = np.max(np.abs(ref))
            err = np.max(np.abs(got - ref)) / scale if scale > 0 else np.max(np.abs(got))
            assert err <= FLOAT_TOL, f"{tag} {k}: relative error {err:.3e}"


@pytest.mark.parametrize("name", SCENES)
def test_oracle_matches_reference_fixture(ds, scenes, name):
    snaps, meta = load(os.path.join(HERE, "golden", f"{name}.npz"))
    b, sc, orc = _oracle(ds, scenes, name)
    assert scene_digest(sc) == str(meta["digest"]), "scene generator no longer reproduces the fixture's inputs"
    dt, gap = float(meta["time_step"]), int(meta["gap"])
    assert dt == sc.time_step and gap == sc.fluid_integrate_gap
    orc.initialize()
    step = 0
    for t in sorted(snaps):
        while step < t:
            step += 1
            orc.update(dt, step, 1, gap)
        _compare(snaps[t], orc, f"{name} step {t}")


def test_fixture_scenes_exercise_the_path(ds, scenes):
    """The fixtures cover live contacts, bonds, walls, clumps and fluid-solid pairs."""
    g = load(os.path.join(HERE, "golden", "tiny_granular.npz"))[0][10]
    assert (np.linalg.norm(g["ss.force"], axis=1) > 0).sum() > 20
    assert (np.linalg.norm(g["ss.sliding"], axis=1) > 0).sum() > 20
    c = load(os.path.join(HERE, "golden", "tiny_coupled.npz"))[0][10]
    assert len(c["bond.pointed"]) > 50 and c["fs.pointed"].size > 1000
    assert np.abs(c["bond.normalForce"]).max() > 0
    d = load(os.path.join(HERE, "golden", "tiny_dam_break.npz"))[0][10]
    assert d["ff.pointed"].size > 1000 and np.abs(d["fluid.dRho"]).max() > 0


refrun = pytest.importorskip("oracle.refrun")


@pytest.mark.skipif(not refrun.available(), reason="reference not compiled here (needs its sources)")
@pytest.mark.parametrize("name", SCENES)
def test_oracle_matches_reference_live(ds, scenes, name):
    """Where the reference compiles (its sources present), step both for 25
    updates and compare everything after each."""
    recipe = getattr(scenes, name)()
    ref = refrun.RefSolver()
    recipe.apply(ref)
    ref.initialize()
    b, sc, orc = _oracle(ds, scenes, name)
    orc.initialize()
    dt, gap = ref.time_step, ref.gap
    for s in range(1, 26):
        ref.update()
        orc.update(dt, s, 1, gap)
        _compare({k: ref.get(k) for k in refrun.FIELDS}, orc, f"{name} step {s}")


@pytest.mark.skipif(not refrun.available(), reason="reference not compiled here (needs its sources)")
def test_reference_continuity_race_is_order_dependent(ds, scenes):
    """The reference's continuity kernel updates dRho in place while neighbours
    read it (core/integrate.cu:55-161).  Run in index order (as a single
    thread would) it differs from the pass-start reading the GPU gives when
    the whole grid is resident - which is what the oracle and the engine do."""
    recipe = scenes.tiny_dam_break()
    out = []
    for jacobi in (True, False):  # the hook mode is process-wide: run one solver at a time
        r = refrun.RefSolver(jacobi_continuity=jacobi)
        recipe.apply(r)
        r.initialize()
        for _ in range(3):
            r.update()
        out.append(r.get("fluid.dRho"))
    refrun.RefSolver(jacobi_continuity=True)  # restore the default mode for later tests
    da, db = out
    assert np.max(np.abs(da - db)) > 1e-6 * np.max(np.abs(da))


def test_fixed_modes_change_the_oracle(ds, scenes):
    """The two switchable reference behaviours matter on the fixture scenes:
    checking every wall changes the granular scene (spheres pressed into a
    side wall while clear of the floor), and integrating clump orientations
    changes the spinning anisotropic clumps of the tumbling scene, within ten
    steps (so the GPU tests of these modes compare something)."""
    from oracle.oracle import OracleSolver
    for name, fix, field in (("tiny_granular", ds.FIX_WALL_LOOP, "solid.vel"),
                             ("tiny_tumbling", ds.FIX_CLUMP_ROTATION, "clump.angvel")):
        b, sc = ds.build_scene(getattr(scenes, name)())
        out = []
        for fixes in (0, fix):
            o = OracleSolver(sc, fixes=fixes)
            o.initialize()
            o.update(sc.time_step, 1, 10, sc.fluid_integrate_gap)
            out.append(o.get(field))
        assert not np.array_equal(out[0], out[1]), name
