"""GPU engine against the FP64 oracle on the benchmark workloads themselves, at
their full sizes, through the C ABI:

* the 48k-fluid dam break, one step;
* the 1.0M-fluid coupled dam break, one step and one whole fluid period
  (28 update() calls through the CUDA-graph path the benchmark times);
* the 200k-sphere settle, one step from a contact-dense bed (the settle run
  on the GPU first, then the engine and the oracle restarted from that state).

Integer artefacts (cell keys, sorted order, cell spans, fluid-fluid,
fluid-solid and solid contact lists, bonds, spring-history remap) must be
identical; floating point within the tolerances of tests/parity.py: FORCE_TOL
for one step from the same state, DRIFT_TOL after a fluid period.
"""
import importlib.util
import os

import numpy as np
import pytest

from parity import DRIFT_TOL, FORCE_TOL, POS_TOL, check_step, compare_integer_artefacts, oracle_for

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_for_configs", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _pair(ds, recipe):
    b, sc = ds.build_scene(recipe)
    eng = ds.Engine(sc)
    orc = oracle_for(sc)
    eng.initialize()
    orc.initialize()
    return b, sc, eng, orc


def test_dam_break_48k_one_step(ds, scenes):
    recipe = scenes.dam_break()
    b, sc, eng, orc = _pair(ds, recipe)
    bad, _ = compare_integer_artefacts(eng, orc)
    assert bad == [], f"after initialize: {bad}"
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    eng.update(dt, 1, 1, gap, use_graph=True)
    orc.update(dt, 1, 1, gap)
    bad, _ = compare_integer_artefacts(eng, orc)
    assert bad == [], f"step 1: {bad}"
    check_step(eng, orc, sc, recipe.meta["dx"], 1, dt, FORCE_TOL, POS_TOL)


def test_coupled_1M_one_step_and_one_fluid_period(ds, scenes):
    """Step 1 (a DEM step: contacts, bonds, coupling forces from the initial
    fluid) within FORCE_TOL; then steps 2..28 through the graph path, step 28
    being the fluid step (lists rebuilt, continuity, momentum): artefacts
    identical, state within DRIFT_TOL."""
    recipe = scenes.coupled_dam_break()
    b, sc, eng, orc = _pair(ds, recipe)
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    assert gap == 28
    bad, _ = compare_integer_artefacts(eng, orc)
    assert bad == [], f"after initialize: {bad}"
    eng.update(dt, 1, 1, gap, use_graph=True)
    orc.update(dt, 1, 1, gap)
    bad, _ = compare_integer_artefacts(eng, orc, skip_fluid_hash=True)
    assert bad == [], f"step 1: {bad}"
    check_step(eng, orc, sc, recipe.meta["dx"], 1, dt, FORCE_TOL, POS_TOL)
    eng.update(dt, 2, gap - 1, gap, use_graph=True)
    orc.update(dt, 2, gap - 1, gap)
    bad, art = compare_integer_artefacts(eng, orc)
    assert bad == [], f"step {gap}: {bad}"
    assert len(art["ff.pointed"]) > 10_000_000 and len(art["ss.pointed"]) > 50_000
    assert int(art["bond.isBonded"].sum()) > 50_000
    check_step(eng, orc, sc, recipe.meta["dx"], gap, dt, DRIFT_TOL, 1e-8)


def test_granular_200k_one_step_from_a_contact_dense_bed(ds, scenes):
    """The settle runs on the GPU until the bed is dense; the engine and the
    oracle then restart from that state (springs zero for both) and take one
    step: the contact list (several contacts per sphere) is identical and
    every contact force, torque and spring is within FORCE_TOL."""
    bench = _bench()
    recipe = bench.make_recipe(1)  # the benchmark's settle: floor wall, sides of fixed spheres
    b, sc = ds.build_scene(recipe)
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    settle = ds.Engine(sc)
    settle.initialize()
    n_settle = bench.SETTLE_STEPS[1]
    settle.update(dt, 1, n_settle, gap, use_graph=True)
    state = bench.engine_state(settle)
    settle.close()
    bench.restart_scene(sc, state)
    eng = ds.Engine(sc)
    orc = oracle_for(sc)
    eng.initialize()
    orc.initialize()
    bad, _ = compare_integer_artefacts(eng, orc)
    assert bad == [], f"after initialize: {bad}"
    first = n_settle + 1
    eng.update(dt, first, 1, gap, use_graph=True)
    orc.update(dt, first, 1, gap)
    bad, art = compare_integer_artefacts(eng, orc)
    assert bad == [], f"step {first}: {bad}"
    _, n_mobile, _ = bench.mobile_counts(sc)
    live = int((np.linalg.norm(art["ss.force"], axis=1) > 0).sum())
    print(f"contacts listed {len(art['ss.pointed'])}, with force {live}, per mobile solid {live / n_mobile:.2f}")
    assert live > n_mobile, "the bed is not contact-dense"
    check_step(eng, orc, sc, 2.5e-3, 1, dt, FORCE_TOL, POS_TOL)
