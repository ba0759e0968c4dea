"""demsph_append: particles added while a simulation runs (dataBase::addFluid,
addCluster, addSolid after the start; core/dataBase.cpp:226-268, 83-113,
307-343), against the oracle's restatement (oracle_append): integer
artefacts (lists, hashes, bonds) identical right after the append and after
the steps that follow; floating point within the multi-step drift
tolerance."""
import numpy as np
import pytest

from parity import DRIFT_TOL, check_step, compare_integer_artefacts, oracle_for

pytestmark = pytest.mark.gpu


def _additions(ds, scenes):
    add_r, whole_r = scenes.tiny_additions()
    _, add = ds.build_scene(add_r)
    _, whole = ds.build_scene(whole_r)
    ns0 = whole.n_solid - add.n_solid
    cl = np.ctypeslib.as_array(add.solid_cluster, shape=(add.n_solid,))
    cl[:] = np.ctypeslib.as_array(whole.solid_cluster, shape=(whole.n_solid,))[ns0:]
    return add, whole


def test_append_matches_the_oracle(ds, scenes):
    recipe = scenes.tiny_coupled()
    _, sc = ds.build_scene(recipe)
    add, whole = _additions(ds, scenes)
    eng = ds.Engine(sc)
    orc = oracle_for(sc)
    eng.initialize()
    orc.initialize()
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    eng.update(dt, 1, 9, gap, use_graph=True)
    orc.update(dt, 1, 9, gap)
    eng.append(sc, add)
    eng.scene = whole  # the static arrays of the whole scene, for the comparisons
    orc.append(add)
    bad, art = compare_integer_artefacts(eng, orc)
    assert bad == [], f"after the append: {bad}"
    ns0 = sc.n_solid
    assert (art["bond.pointed"][-12:] >= ns0).all() and len(art["bond.pointed"]) == len(orc.get("bond.pointed"))
    assert not eng.download_solids()["normal"][ns0:].any()
    eng.update(dt, 10, 9, gap, use_graph=True)
    orc.update(dt, 10, 9, gap)
    bad, _ = compare_integer_artefacts(eng, orc)
    assert bad == [], f"step 18: {bad}"
    check_step(eng, orc, whole, recipe.meta["dx"], 18, dt, DRIFT_TOL, 1e-8)


def test_append_refuses_walls_and_clumps(ds, scenes):
    _, sc = ds.build_scene(scenes.tiny_coupled())
    eng = ds.Engine(sc)
    eng.initialize()
    eng.update(sc.time_step, 1, 3, sc.fluid_integrate_gap)
    with pytest.raises(ds.DemSphError) as e:
        eng.append(sc, sc)  # holds a clump and a wall
    assert e.value.status == 1
    eng.update(sc.time_step, 4, 3, sc.fluid_integrate_gap)  # the engine is unchanged and usable


def test_frame_writer_refuses_after_an_append(ds, scenes, tmp_path):
    """A writer sized for the counts at its opening refuses frames once
    particles were added (its slots would be too small); a new writer works."""
    _, sc = ds.build_scene(scenes.tiny_coupled())
    add, whole = _additions(ds, scenes)
    eng = ds.Engine(sc)
    eng.initialize()
    eng.update(sc.time_step, 1, 3, sc.fluid_integrate_gap)
    fw = ds.FrameWriter(eng, tmp_path / "a")
    fw.write(ds.FRAME_ALL, 0, 3, 0.0)
    fw.flush()
    eng.append(sc, add)
    eng.scene = whole
    with pytest.raises(ds.DemSphError) as e:
        fw.write(ds.FRAME_ALL, 1, 3, 0.0)
    assert e.value.status == 2
    fw.close()
    with ds.FrameWriter(eng, tmp_path / "b") as fw2:
        fw2.write(ds.FRAME_ALL, 1, 3, 0.0)
    from vtu import read_vtu
    assert read_vtu(tmp_path / "b" / "fluid_0001.vtu")["Points"].shape[0] == whole.n_fluid
