"""Particles added while a simulation runs (oracle_append, the oracle's
restatement of dataBase::addFluidData / addSolidData after the start,
core/dataBase.cpp:226-268, with addCluster's bonds, :83-113 and :307-343):
the new particles follow the old ones, contact springs carry over, wall
springs start again from zero, new solids have zero normals, only the new
cluster is bonded, and new fluids get Shepard reference sums."""
import numpy as np
import pytest

from oracle.oracle import OracleSolver


def _additions(ds, scenes):
    add_r, whole_r = scenes.tiny_additions()
    _, add = ds.build_scene(add_r)
    _, whole = ds.build_scene(whole_r)
    ns0 = whole.n_solid - add.n_solid
    # the new cluster's id as addCluster numbers it (one above the largest)
    cl = np.ctypeslib.as_array(add.solid_cluster, shape=(add.n_solid,))
    cl[:] = np.ctypeslib.as_array(whole.solid_cluster, shape=(whole.n_solid,))[ns0:]
    return add, whole


def _pairs(o):
    a, b = o.get("ss.pointed"), o.get("ss.pointing")
    return {(int(x), int(y)): k for k, (x, y) in enumerate(zip(a, b))}


def test_append_keeps_history_and_bonds_only_the_new_cluster(ds, scenes):
    _, sc = ds.build_scene(scenes.tiny_coupled())
    add, whole = _additions(ds, scenes)
    o = OracleSolver(sc)
    o.initialize()
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    o.update(dt, 1, 9, gap)
    nf0, ns0 = sc.n_fluid, sc.n_solid
    before = _pairs(o)
    springs = {k: o.get("ss.sliding")[i] for k, i in before.items()}
    bonds = {k: o.get("bond." + k).copy() for k in ("pointed", "pointing", "normalForce", "shearForce")}
    normals = o.get("solid.normal").copy()
    o.append(add)
    assert o.get("fluid.pos").shape[0] == nf0 + add.n_fluid
    assert o.get("solid.pos").shape[0] == ns0 + add.n_solid
    assert np.array_equal(o.get("solid.normal")[:ns0], normals)
    assert not o.get("solid.normal")[ns0:].any()
    nb0 = len(bonds["pointed"])
    for k, v in bonds.items():
        assert np.array_equal(o.get("bond." + k)[:nb0], v)
    pa, pb = o.get("bond.pointed")[nb0:], o.get("bond.pointing")[nb0:]
    assert len(pa) == 12  # the face neighbours of a 2x2x2 lattice of touching spheres
    assert (pa >= ns0).all() and (pb >= ns0).all()
    after = _pairs(o)
    kept = [k for k in before if k in after]
    assert kept
    for k in kept:
        assert np.array_equal(o.get("ss.sliding")[after[k]], springs[k])
    assert (o.get("fluid.sumW0")[nf0:] > 0).all()
    o.update(dt, 10, 9, gap)
    for f in ("fluid.pos", "solid.pos", "fluid.dRho"):
        assert np.isfinite(o.get(f)).all()


def test_append_refuses_walls_and_clumps(ds, scenes):
    _, sc = ds.build_scene(scenes.tiny_coupled())
    o = OracleSolver(sc)
    o.initialize()
    _, with_clump = ds.build_scene(scenes.tiny_coupled())  # holds a clump and a wall
    with pytest.raises(ValueError):
        o.append(with_clump)
