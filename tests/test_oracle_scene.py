"""The oracle's own scene assembly (oracle/scene.py, the reference's setup
calls of core/dataBase.cpp:3-177 restated in numpy) gives the same arrays,
bit for bit, as the product's scene builder (dem-sphsource_gb300/host/
sceneBuilder.cpp) for every workload and test scene: so the CPU baseline and
the reference arm of bench.py can build their scenes without loading the
product library, and still see the inputs the engine sees."""
import numpy as np
import pytest

from oracle.scene import build_scene as oracle_build, scene_arrays

SMALL = ("tiny_dam_break", "tiny_granular", "tiny_coupled", "tiny_escape", "tiny_two_fluids", "tiny_converging",
         "tiny_linear", "tiny_tumbling")


def _same(ds, recipe):
    _, prod = ds.build_scene(recipe)
    _, orc = oracle_build(recipe)
    a, b = scene_arrays(prod), scene_arrays(orc)
    assert set(a) == set(b)
    bad = [k for k in a if a[k].shape != b[k].shape or a[k].tobytes() != b[k].tobytes()]
    assert bad == [], f"{recipe.name}: arrays differ: {bad}"


@pytest.mark.parametrize("name", SMALL)
def test_small_scenes_assemble_identically(ds, scenes, name):
    if not ds.library_available():
        pytest.skip("product library not built")
    _same(ds, getattr(scenes, name)())


@pytest.mark.parametrize("config", ("dam_break", "granular_settle", "coupled_dam_break"))
def test_workload_scenes_assemble_identically(ds, scenes, config):
    """The three single-scene workloads at their full sizes."""
    if not ds.library_available():
        pytest.skip("product library not built")
    _same(ds, getattr(scenes, config)())


def test_batched_and_serving_recipes_assemble_identically(ds, scenes):
    if not ds.library_available():
        pytest.skip("product library not built")
    for r in scenes.batch_mix(n_scenes=6, n_range=(2000, 6000)):
        _same(ds, r)
    _same(ds, scenes.make_request("dem", 3000, 10, 5))


def test_rejected_calls_leave_the_scene_unchanged(ds, scenes):
    """A material index past the table, or mismatched array lengths, are
    refused by both (the reference prints and returns)."""
    if not ds.library_available():
        pytest.skip("product library not built")
    r = scenes.tiny_granular()
    r.calls = [c for c in r.calls]
    from oracle.scene import OracleScene
    o = OracleScene()
    r.apply(o)
    n0 = o.scene().n_solid
    o.addSolid(np.zeros((2, 3)), (0, 0, 0), 1e-3, 2500.0, 10)
    o.addCluster(np.zeros((2, 3)), np.ones(3), np.ones(2), (0, 0, 0), 0)
    assert o.scene().n_solid == n0
