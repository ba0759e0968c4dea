"""GPU engine against the FP64 oracle on the same scenes, through the C ABI.

Integer artefacts must be identical; floating-point results must agree within
the tolerances stated in tests/parity.py.  The oracle itself is pinned to the
reference's own kernels (tests/test_oracle_golden.py).
"""
import numpy as np
import pytest

from parity import (DRIFT_TOL, FORCE_TOL, POS_TOL, check_step, compare_integer_artefacts, engine_artefacts,
                    oracle_for, state_errors)

pytestmark = pytest.mark.gpu

SCENES = ("tiny_dam_break", "tiny_granular", "tiny_coupled", "tiny_escape", "tiny_two_fluids", "tiny_linear",
          "tiny_tumbling")
# solid contact candidates: default margin, one so small that candidates are
# rebuilt nearly every step, and none (the 27-cell walk every step)
SKINS = (0.0, 1.0e-9, -1.0)


def _setup(ds, scenes, name, **opts):
    recipe = getattr(scenes, name)()
    b, sc = ds.build_scene(recipe)
    eng = ds.Engine(sc, **opts)
    orc = oracle_for(sc, fixes=opts.get("fixes", 0))
    return recipe, b, sc, eng, orc


def _spacing(recipe):
    return recipe.meta.get("dx", 2.0e-3)


@pytest.mark.parametrize("name", SCENES)
def test_initialize_artefacts_identical(ds, scenes, name):
    recipe, b, sc, eng, orc = _setup(ds, scenes, name)
    eng.initialize()
    orc.initialize()
    bad, art = compare_integer_artefacts(eng, orc)
    assert bad == [], f"integer artefacts differ after initialize: {bad}"
    if eng.ns:
        s = eng.download_solids()
        assert np.max(np.abs(s["normal"] - orc.get("solid.normal"))) < 1e-5
        if len(art["bond.pointed"]):
            assert np.allclose(art["bond.contactNormal"], orc.get("bond.contactNormal"), atol=1e-6)
            assert np.allclose(art["bond.contactPoint"], orc.get("bond.contactPoint"), atol=1e-9)


@pytest.mark.parametrize("name", SCENES)
def test_one_step_within_force_tolerance(ds, scenes, name):
    """One update() from the same initial state: every force, torque, spring,
    density and state within the per-step tolerance, integer artefacts equal."""
    recipe, b, sc, eng, orc = _setup(ds, scenes, name)
    eng.initialize()
    orc.initialize()
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    eng.step(dt, 1, gap)
    orc.update(dt, 1, 1, gap)
    bad, _ = compare_integer_artefacts(eng, orc, skip_fluid_hash=(1 % gap != 0))
    assert bad == [], f"integer artefacts differ: {bad}"
    check_step(eng, orc, sc, _spacing(recipe), 1, dt, FORCE_TOL, POS_TOL)


# (solid candidate margin, threads per fluid particle, fluid candidate margin,
# membership bits): the defaults (list kernels), the solid margin variants,
# one thread per fluid particle (what large scenes use), fluid candidates
# rebuilt every fluid step, the fluid walk, and the fluid lists kept as
# membership bits (DEMSPH_FLUID_TILES=1) with two solid margins
VARIANTS = [(s, 0, 0.0, "0") for s in SKINS] + [(0.0, 1, 0.0, "0"), (0.0, 0, 1.0e-9, "0"), (0.0, 0, -1.0, "0"),
                                                 (0.0, 0, 0.0, "1"), (1.0e-9, 0, 0.0, "1")]


@pytest.mark.parametrize("skin,lanes,fskin,tiles", VARIANTS)
@pytest.mark.parametrize("name", SCENES)
def test_ten_steps_artefacts_equal_drift_bounded(ds, scenes, name, skin, lanes, fskin, tiles, monkeypatch):
    """Ten update() calls through the five stage calls: integer artefacts equal
    after every step; floating-point drift within DRIFT_TOL."""
    monkeypatch.setenv("DEMSPH_FLUID_TILES", tiles)
    recipe, b, sc, eng, orc = _setup(ds, scenes, name, solid_verlet_skin=skin, fluid_lanes=lanes,
                                     fluid_verlet_skin=fskin)
    eng.initialize()
    orc.initialize()
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for step in range(1, 11):
        eng.step(dt, step, gap)
        orc.update(dt, step, 1, gap)
        bad, _ = compare_integer_artefacts(eng, orc, skip_fluid_hash=(step % gap != 0))
        assert bad == [], f"step {step}: integer artefacts differ: {bad}"
        check_step(eng, orc, sc, _spacing(recipe), step, dt, DRIFT_TOL, 1e-8)


@pytest.mark.parametrize("name", SCENES)
def test_graph_batch_equals_staged_calls(ds, scenes, name):
    """demsph_update (CUDA graph over whole periods) gives the same bits as the
    five stage calls per step."""
    recipe, b, sc, e1, _ = _setup(ds, scenes, name)
    e2 = ds.Engine(sc)
    e1.initialize()
    e2.initialize()
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    n = 10 * gap * 2 + 3
    for s in range(1, n + 1):
        e1.step(dt, s, gap)
    e2.update(dt, 1, n, gap, use_graph=True)
    if e1.nf:
        for a, c in zip(e1.download_fluids(), e2.download_fluids()):
            assert np.array_equal(a, c)
    if e1.ns:
        s1, s2 = e1.download_solids(), e2.download_solids()
        for k in s1:
            assert np.array_equal(s1[k], s2[k]), k


@pytest.mark.parametrize("name", ("tiny_coupled", "tiny_granular", "tiny_dam_break"))
def test_update_io_equals_separate_transfers(ds, scenes, name):
    """demsph_update_io (upload, steps, download, one synchronisation) gives the
    bits of demsph_upload_* + demsph_update + demsph_download_*."""
    recipe, b, sc, e1, _ = _setup(ds, scenes, name)
    e2 = ds.Engine(sc)
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for e in (e1, e2):
        e.initialize()
        e.update(dt, 1, 3, gap)
    nf, ns = sc.n_fluid, sc.n_solid
    f1 = tuple(np.zeros(s) for s in ((nf, 3), (nf, 3), (nf,))) if nf else None
    s1 = tuple(np.zeros((ns, 3)) for _ in range(3)) if ns else None
    f2 = tuple(a.copy() for a in f1) if nf else None
    s2 = tuple(a.copy() for a in s1) if ns else None
    if nf:
        e1.download_fluids(out=(f1[0], f1[1], None, f1[2]))
        e2.download_fluids(out=(f2[0], f2[1], None, f2[2]))
    if ns:
        e1.download_solids(out={"pos": s1[0], "vel": s1[1], "angvel": s1[2]})
        e2.download_solids(out={"pos": s2[0], "vel": s2[1], "angvel": s2[2]})
    for step in range(4, 10):
        if ns:
            e1.upload_solids(*s1)
        if nf:
            e1.upload_fluids(*f1)
        e1.update(dt, step, 1, gap)
        if ns:
            e1.download_solids(out={"pos": s1[0], "vel": s1[1], "angvel": s1[2]})
        if nf:
            e1.download_fluids(out=(f1[0], f1[1], None, f1[2]))
        e2.update_io(dt, step, 1, gap, fluid_in=f2, solid_in=s2, fluid_out=f2, solid_out=s2)
        for a, c in zip(f1 or (), f2 or ()):
            assert np.array_equal(a, c)
        for a, c in zip(s1 or (), s2 or ()):
            assert np.array_equal(a, c)


@pytest.mark.parametrize("name", SCENES)
def test_deterministic(ds, scenes, name):
    recipe, b, sc, e1, _ = _setup(ds, scenes, name)
    e2 = ds.Engine(sc)
    for e in (e1, e2):
        e.initialize()
        e.update(sc.time_step, 1, 12, sc.fluid_integrate_gap, use_graph=False)
    if e1.nf:
        assert all(np.array_equal(a, c) for a, c in zip(e1.download_fluids(), e2.download_fluids()))
    if e1.ns:
        s1, s2 = e1.download_solids(), e2.download_solids()
        assert all(np.array_equal(s1[k], s2[k]) for k in s1)


def test_list_overflow_grows_and_matches(ds, scenes):
    """With lists far too small the engine grows them and re-runs; the result is
    the same as with ample lists."""
    recipe = scenes.tiny_coupled()
    b, sc = ds.build_scene(recipe)
    small = ds.Engine(sc, fluid_neighbors_max=4, fluid_solids_max=2, solid_contacts_per_particle=1)
    big = ds.Engine(sc)
    for e in (small, big):
        e.initialize()
        e.update(sc.time_step, 1, 30, sc.fluid_integrate_gap, use_graph=True)
    for a, c in zip(small.download_fluids(), big.download_fluids()):
        assert np.array_equal(a, c)
    s1, s2 = small.download_solids(), big.download_solids()
    assert all(np.array_equal(s1[k], s2[k]) for k in s1)


@pytest.mark.parametrize("name", ("tiny_granular", "tiny_coupled"))
def test_contact_candidates_do_not_change_results(ds, scenes, name):
    """The candidate margin only changes how often contact candidates are
    rebuilt: sixty steps with the default margin, a margin of 1 nm (rebuilt
    nearly every step) and the 27-cell walk every step give the same contact
    lists and the same state, bit for bit (lists are kept in index order, so
    every per-solid force sum adds the same terms in the same order)."""
    recipe = getattr(scenes, name)()
    b, sc = ds.build_scene(recipe)
    engines = [ds.Engine(sc, solid_verlet_skin=s) for s in SKINS]
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for e in engines:
        e.initialize()
        e.update(dt, 1, 60, gap)
    ref = engines[0].solid_pairs()
    s0 = engines[0].download_solids()
    for e in engines[1:]:
        got = e.solid_pairs()
        for k in ref:
            assert np.array_equal(got[k], ref[k]), k
        s1 = e.download_solids()
        for k in s0:
            assert np.array_equal(s1[k], s0[k]), k


@pytest.mark.parametrize("name", ("tiny_granular", "tiny_coupled"))
def test_contact_rows_per_warp_do_not_change_results(ds, scenes, name):
    """The contact kernels hand a warp's (row, contact) items to its lanes
    whatever the rows per warp: 4, 32 and the adaptive choice (re-made after
    every update call) give the same contact lists and state, bit for bit."""
    recipe = getattr(scenes, name)()
    b, sc = ds.build_scene(recipe)
    engines = [ds.Engine(sc, contact_rows_per_warp=r) for r in (32, 4, 0)]
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for e in engines:
        e.initialize()
        for k in range(6):
            e.update(dt, 1 + 10 * k, 10, gap, use_graph=True)
    ref = engines[0].solid_pairs()
    s0 = engines[0].download_solids()
    for e in engines[1:]:
        got = e.solid_pairs()
        for k in ref:
            assert np.array_equal(got[k], ref[k]), k
        s1 = e.download_solids()
        for k in s0:
            assert np.array_equal(s1[k], s0[k]), k


@pytest.mark.parametrize("cells,lo,hi", [(200_000, 4096, 524_288), (1_000_000, 524_288, 2_500_000)])
def test_large_grids_sort_like_the_oracle(ds, scenes, cells, lo, hi):
    """The sort by cell scans the cell counts in one block up to 524,288
    cells and in three launches beyond: a granular scene in a widened domain
    gives the oracle's cell spans, sorted order and contact lists at
    initialisation and after every one of ten steps (the candidates are
    rebuilt, and the solids re-sorted, along the way)."""
    recipe = scenes.tiny_granular_wide(cells)
    b, sc = ds.build_scene(recipe)
    eng = ds.Engine(sc, solid_verlet_skin=1.0e-9)  # rebuild (and sort) nearly every step
    orc = oracle_for(sc)
    eng.initialize()
    orc.initialize()
    assert lo < eng.counts().grid_cells <= hi
    bad, _ = compare_integer_artefacts(eng, orc)
    assert bad == [], f"integer artefacts differ after initialize: {bad}"
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for step in range(1, 11):
        eng.step(dt, step, gap)
        orc.update(dt, step, 1, gap)
        bad, _ = compare_integer_artefacts(eng, orc, skip_fluid_hash=(step % gap != 0))
        assert bad == [], f"step {step}: integer artefacts differ: {bad}"
        check_step(eng, orc, sc, _spacing(recipe), step, dt, DRIFT_TOL, 1e-8)


@pytest.mark.parametrize("name", ("tiny_granular", "tiny_coupled", "tiny_dam_break"))
def test_cooperative_sorts_equal_launch_per_phase_sorts(ds, scenes, name, monkeypatch):
    """The one-launch cooperative sorts (solid sort by cell; fluid hash and
    reorder) give the same bits as the launch-per-phase sorts they replace
    (DEMSPH_COOPERATIVE_SORT=0, read when an engine is created), over forty
    steps with candidates rebuilt, and so sorts run, nearly every step."""
    recipe = getattr(scenes, name)()
    b, sc = ds.build_scene(recipe)
    engines = []
    for flag in ("1", "0"):
        monkeypatch.setenv("DEMSPH_COOPERATIVE_SORT", flag)
        engines.append(ds.Engine(sc, solid_verlet_skin=1.0e-9, fluid_verlet_skin=1.0e-9))
    monkeypatch.delenv("DEMSPH_COOPERATIVE_SORT")
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for e in engines:
        e.initialize()
        e.update(dt, 1, 40, gap, use_graph=True)
    if sc.n_fluid:
        for a, c in zip(engines[0].download_fluids(), engines[1].download_fluids()):
            assert np.array_equal(a, c)
    if sc.n_solid:
        s0, s1 = engines[0].download_solids(), engines[1].download_solids()
        for k in s0:
            assert np.array_equal(s0[k], s1[k]), k


def _dry_granular(scenes):
    return scenes.tiny_granular(with_probe_fluid=False)


def _same_state_and_lists(e0, e1):
    if e0.nf:
        for a, c in zip(e0.download_fluids(), e1.download_fluids()):
            assert np.array_equal(a, c)
    if e0.ns:
        s0, s1 = e0.download_solids(), e1.download_solids()
        for k in s0:
            assert np.array_equal(s0[k], s1[k]), k
        p0, p1 = e0.solid_pairs(), e1.solid_pairs()
        for k in p0:
            assert np.array_equal(p0[k], p1[k]), k


@pytest.mark.parametrize("name,skin", [("tiny_converging", 0.0), ("dry_granular", 0.0), ("dry_granular", 1.0e-9),
                                       ("tiny_coupled", 0.0)])
def test_fused_integration_equals_separate_passes(ds, scenes, name, skin, monkeypatch):
    """Graphs of plain DEM steps close each step and open the next in one
    integration pass, with the neighbour search in between reading the
    end-of-step offsets, and (without bonds) build the contact list of an
    opened step in the launch of its contact forces; forty steps give the
    bits of the two separate passes (DEMSPH_FUSE_INTEGRATION=0), of the fused
    pass with two contact launches (DEMSPH_MERGE_CONTACTS=0; both read when an
    engine is created) and of the staged calls; with a 1 nm candidate margin
    the opened steps also rebuild their candidates in that launch."""
    recipe = _dry_granular(scenes) if name == "dry_granular" else getattr(scenes, name)()
    b, sc = ds.build_scene(recipe)
    engines = []
    for fuse, merge in (("1", "1"), ("0", "1"), ("1", "0")):
        monkeypatch.setenv("DEMSPH_FUSE_INTEGRATION", fuse)
        monkeypatch.setenv("DEMSPH_MERGE_CONTACTS", merge)
        engines.append(ds.Engine(sc, solid_verlet_skin=skin))
    monkeypatch.delenv("DEMSPH_FUSE_INTEGRATION")
    monkeypatch.delenv("DEMSPH_MERGE_CONTACTS")
    staged = ds.Engine(sc, solid_verlet_skin=skin)
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for e in engines + [staged]:
        e.initialize()
    for e in engines:
        e.update(dt, 1, 40, gap, use_graph=True)
    for s in range(1, 41):
        staged.step(dt, s, gap)
    assert engines[0].run_stats()["fused_passes"] > 0
    assert engines[1].run_stats()["fused_passes"] == 0
    for e in engines[1:] + [staged]:
        _same_state_and_lists(engines[0], e)


@pytest.mark.parametrize("name", ("dry_granular", "tiny_coupled", "tiny_converging"))
def test_profiled_update_runs_the_graph_bodies(ds, scenes, name):
    """With stage timing on, demsph_update issues the launches its graphs
    hold (fused runs included) one by one, each stage timed: forty steps give
    the bits and lists of the graph replay, and the fused integration pass has
    its own timed launches."""
    recipe = _dry_granular(scenes) if name == "dry_granular" else getattr(scenes, name)()
    b, sc = ds.build_scene(recipe)
    opts = dict(solid_contacts_per_particle=1) if name == "tiny_converging" else {}
    timed, plain = ds.Engine(sc, **opts), ds.Engine(sc, **opts)
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for e in (timed, plain):
        e.initialize()
    timed.set_profiling(True)
    timed.profile_report()
    timed.update(dt, 1, 40, gap, use_graph=True)
    stages = timed.profile_report()
    timed.set_profiling(False)
    plain.update(dt, 1, 40, gap, use_graph=True)
    assert timed.run_stats()["fused_passes"] == plain.run_stats()["fused_passes"] > 0
    assert timed.run_stats()["resumed_steps"] == plain.run_stats()["resumed_steps"]
    # every step sums its solids' forces: after its pair forces, or in the one
    # launch that also builds the list of a step a fused pass opened
    sums = sum(stages.get(k, (0, 0.0))[0] for k in ("solid_forces", "contact_forces"))
    assert stages["integrate_after"][0] >= 40 and sums >= 40, stages
    _same_state_and_lists(timed, plain)


@pytest.mark.parametrize("name", ("coupled_without_clump", "tiny_converging", "tiny_escape"))
def test_folded_integration_equals_the_separate_pass(ds, scenes, name, monkeypatch):
    """Where the integrated solids are exactly the contact rows (no clumps,
    no moving dummy particles) the per-solid force sums run the solids'
    integration pass in the same launch: forty steps from graphs give the bits
    and lists of the separate pass (DEMSPH_FOLD_INTEGRATION=0, read when an
    engine is created) and of the staged calls, with fewer launches."""
    recipe = scenes.tiny_coupled(with_clump=False) if name == "coupled_without_clump" else getattr(scenes, name)()
    b, sc = ds.build_scene(recipe)
    engines = []
    for fold in ("1", "0"):
        monkeypatch.setenv("DEMSPH_FOLD_INTEGRATION", fold)
        engines.append(ds.Engine(sc))
    monkeypatch.delenv("DEMSPH_FOLD_INTEGRATION")
    staged = ds.Engine(sc)
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for e in engines + [staged]:
        e.initialize()
    launches = []
    for e in engines:
        before = e.kernel_launches()
        e.update(dt, 1, 40, gap, use_graph=True)
        launches.append(e.kernel_launches() - before)
    for s in range(1, 41):
        staged.step(dt, s, gap)
    assert launches[0] < launches[1], launches
    _same_state_and_lists(engines[0], engines[1])
    _same_state_and_lists(engines[0], staged)


def test_walk_mode_splits_the_merged_contact_launch(ds, scenes):
    """Two solids start above the domain, so the lists come from the walk:
    the first step a fused pass opens finds the one-launch contact list
    unusable, raises its status before writing anything, and is resumed from
    its midpoint with two launches (as every later step is).  Thirty steps give
    the bits of the staged calls."""
    b, sc = ds.build_scene(scenes.tiny_escape(with_probe_fluid=False))
    e, staged = ds.Engine(sc), ds.Engine(sc)
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for x in (e, staged):
        x.initialize()
    e.update(dt, 1, 30, gap, use_graph=True)
    for s in range(1, 31):
        staged.step(dt, s, gap)
    assert e.run_stats()["resumed_steps"] >= 1
    _same_state_and_lists(e, staged)


def test_overflow_inside_a_fused_run_resumes_the_opened_step(ds, scenes):
    """In the converging lattice every sphere gains three forward contacts
    at step 15, inside the graph of steps 12-21; with one contact slot per row
    that step's search overflows after the fused pass has opened it.  The
    engine grows the rows and resumes the step from its midpoint (no second
    opening half step): the result equals a run with ample rows, bit for bit."""
    b, sc = ds.build_scene(scenes.tiny_converging())
    small = ds.Engine(sc, solid_contacts_per_particle=1)
    big = ds.Engine(sc)
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for e in (small, big):
        e.initialize()
        e.update(dt, 1, 40, gap, use_graph=True)
    st = small.run_stats()
    assert st["resumed_steps"] >= 1 and st["list_growths"] >= 1, st
    assert big.run_stats()["list_growths"] == 0
    _same_state_and_lists(small, big)


def test_drift_bounded_over_run(ds, scenes):
    """Forty steps of the coupled scene: the engine stays within bounded
    distance of the FP64 oracle (no systematic FP32 drift)."""
    recipe, b, sc, eng, orc = _setup(ds, scenes, "tiny_coupled")
    eng.initialize()
    orc.initialize()
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    eng.update(dt, 1, 40, gap)
    orc.update(dt, 1, 40, gap)
    err = state_errors(eng, orc, recipe.meta["dx"], 40, dt)
    assert err["fluid.pos"] < 1e-7, err
    assert err["solid.pos"] < 1e-7, err
    assert err["fluid.dRho"] < 1e-5, err


@pytest.mark.parametrize("name", ("tiny_coupled", "tiny_granular"))
def test_audit_matches_the_state(ds, scenes, name):
    """demsph_audit's FP64 sums on the GPU equal the same sums formed on the
    host from the downloaded state and the scene's masses."""
    recipe, b, sc, eng, _ = _setup(ds, scenes, name)
    eng.initialize()
    eng.update(sc.time_step, 1, 20, sc.fluid_integrate_gap)
    a = eng.audit()
    arr = lambda p, n, w=1: np.ctypeslib.as_array(p, shape=(n * w,)).reshape(n, w) if w > 1 else \
        np.ctypeslib.as_array(p, shape=(n,))
    o = np.array(sc.domain_origin[:])
    g = np.array(sc.gravity[:])
    mass = px = ke = rot = pe = rho = 0.0
    px = np.zeros(3)
    if sc.n_fluid:
        pos, vel, _, drho = eng.download_fluids()
        m = (arr(sc.fluid_smoothing_length, sc.n_fluid) / 1.3) ** 3 * arr(sc.fluid_rho0, sc.n_fluid)
        mass += m.sum()
        px += (m[:, None] * vel).sum(0)
        ke += 0.5 * (m * (vel * vel).sum(1)).sum()
        pe -= (m * ((pos - o) @ g)).sum()
        rho += (arr(sc.fluid_rho0, sc.n_fluid) + drho).sum()
    s = eng.download_solids()
    im = arr(sc.solid_inverse_mass, sc.n_solid)
    clump = arr(sc.solid_clump, sc.n_solid)
    free = (im > 0) & (clump < 0)
    m = 1.0 / im[free]
    mass += m.sum()
    px += (m[:, None] * s["vel"][free]).sum(0)
    ke += 0.5 * (m * (s["vel"][free] ** 2).sum(1)).sum()
    r = arr(sc.solid_radius, sc.n_solid)[free]
    rot += (0.5 * 0.4 * m * r * r * (s["angvel"][free] ** 2).sum(1)).sum()
    pe -= (m * ((s["pos"][free] - o) @ g)).sum()
    if sc.n_clump:
        c = eng.download_clumps()
        cim = arr(sc.clump_inverse_mass, sc.n_clump)
        cm = 1.0 / cim[cim > 0]
        mass += cm.sum()
        px += (cm[:, None] * c["vel"][cim > 0]).sum(0)
        ke += 0.5 * (cm * (c["vel"][cim > 0] ** 2).sum(1)).sum()
        pe -= (cm * ((c["centroid"][cim > 0] - o) @ g)).sum()
    rel = lambda x, y: abs(x - y) / max(abs(y), 1e-30)
    assert rel(a["mass"], mass) < 1e-7  # fluid masses are stored in FP32
    assert np.allclose(a["momentum"], px, rtol=1e-6, atol=1e-12 * mass)
    assert rel(a["kinetic_energy"], ke) < 1e-6
    assert rel(a["rotational_energy"], rot) < 1e-6 or rot == 0.0
    assert rel(a["potential_energy"], pe) < 1e-6
    if sc.n_fluid:
        assert rel(a["fluid_density_sum"], rho) < 1e-7


@pytest.mark.parametrize("name", ("tiny_granular", "tiny_coupled", "tiny_linear", "tiny_tumbling"))
def test_fixed_modes_match_the_oracle(ds, scenes, name):
    """With DEMSPH_FIX_WALL_LOOP | DEMSPH_FIX_CLUMP_ROTATION (every wall
    checked; clump orientation integrated in FP64) the engine follows the
    oracle run with the same flags: artefacts identical after each of ten
    steps, one step within FORCE_TOL, drift within DRIFT_TOL.  The reference
    has no code for either mode, so the oracle alone pins them
    (tests/test_oracle_golden.py shows the modes change its result)."""
    fixes = ds.FIX_WALL_LOOP | ds.FIX_CLUMP_ROTATION
    recipe, b, sc, eng, orc = _setup(ds, scenes, name, fixes=fixes)
    eng.initialize()
    orc.initialize()
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for step in range(1, 11):
        eng.step(dt, step, gap)
        orc.update(dt, step, 1, gap)
        bad, _ = compare_integer_artefacts(eng, orc, skip_fluid_hash=(step % gap != 0))
        assert bad == [], f"step {step}: integer artefacts differ: {bad}"
        # with every wall checked, grains pressed into the side walls at the
        # start fly off: positions are held to 1e-7 of the spacing after step 1
        check_step(eng, orc, sc, _spacing(recipe), step, dt, FORCE_TOL if step == 1 else DRIFT_TOL,
                   POS_TOL if step == 1 else 1e-7)
    if name == "tiny_tumbling":  # its clumps spin from the start
        q = eng.download_clumps()["orientation"]
        assert np.abs(q[:, 1:]).max() > 0, "clump orientations were not integrated"
        assert np.allclose(q, orc.get("clump.orientation"), rtol=0, atol=1e-9)


@pytest.mark.parametrize("name", ("tiny_dam_break", "tiny_coupled"))
def test_tile_and_list_pair_loops_agree(ds, scenes, name, monkeypatch):
    """The fluid lists kept as membership bits with the pair loops over them
    (DEMSPH_FLUID_TILES=1, read when an engine is created) and the list
    kernels (the default) over twenty steps: the same fluid-fluid and
    fluid-solid lists bit for bit (the bits written out as lists), and states
    within the per-step force tolerance of each other (the sums add the same
    terms in another order)."""
    b, sc = ds.build_scene(getattr(scenes, name)())
    engines = []
    for flag in ("1", "0"):
        monkeypatch.setenv("DEMSPH_FLUID_TILES", flag)
        engines.append(ds.Engine(sc))
    monkeypatch.delenv("DEMSPH_FLUID_TILES")
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    for e in engines:
        e.initialize()
        e.update(dt, 1, 20, gap, use_graph=True)
    a, c = engines[0].fluid_pairs(), engines[1].fluid_pairs()
    for k in a:
        assert np.array_equal(a[k], c[k]), k
    a, c = engines[0].fluid_solid_pairs(), engines[1].fluid_solid_pairs()
    for k in ("prefix", "pointed", "pointing"):
        assert np.array_equal(a[k], c[k]), k
    (p0, v0, a0, r0), (p1, v1, a1, r1) = engines[0].download_fluids(), engines[1].download_fluids()
    assert np.max(np.linalg.norm(a0 - a1, axis=1) / np.maximum(np.linalg.norm(a1, axis=1), 9.81)) <= FORCE_TOL
    assert np.max(np.abs(r0 - r1)) <= 1e-6 * 1000.0
    assert np.max(np.abs(p0 - p1)) <= 1e-9


def test_dummies_given_a_velocity_move_and_stop(ds, scenes):
    """An upload that gives dummy particles a velocity puts them in the
    integration (the device finds that their motion changed): they drift by
    v t while the other dummy particles stay put; an upload that sets the
    velocity back to zero stops them, through graphs and staged calls alike."""
    b, sc = ds.build_scene(scenes.tiny_dam_break())
    moving = np.array([i for i in range(sc.n_solid) if sc.solid_is_dummy[i]][:10])
    assert len(moving) == 10
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    e = ds.Engine(sc)
    e.initialize()
    e.update(dt, 1, 2, gap)
    s0 = e.download_solids()
    pos, vel, w = s0["pos"].copy(), s0["vel"].copy(), s0["angvel"].copy()
    vel[moving] = (0.01, -0.02, 0.0)
    e.upload_solids(pos, vel, w)
    e.update(dt, 3, 5, gap, use_graph=True)
    for s in range(8, 10):
        e.step(dt, s, gap)
    s1 = e.download_solids()
    t = 7 * dt
    assert np.allclose(s1["pos"][moving], pos[moving] + t * vel[moving], rtol=0, atol=1e-12)
    others = np.setdiff1d(np.arange(sc.n_solid), moving)
    assert np.array_equal(s1["pos"][others], pos[others])
    assert np.allclose(s1["vel"][moving], vel[moving], rtol=1e-14, atol=0)  # kept as double-float
    vel[moving] = 0.0
    e.upload_solids(s1["pos"], vel, s1["angvel"])
    e.update(dt, 10, 4, gap, use_graph=True)
    s2 = e.download_solids()
    assert np.array_equal(s2["pos"], s1["pos"])


def test_moving_dummies_keep_the_fluid_candidates_fresh(ds, scenes):
    """The tank's dummy particles given a velocity that carries them past half
    the fluid candidates' margin within a few steps: the candidates are rebuilt
    as the walls move, so the fluid forces follow those of the reference's
    walk every fluid step (fluid_verlet_skin < 0) within a rounding-level
    bound."""
    b, sc = ds.build_scene(scenes.tiny_dam_break())
    dummies = np.array([i for i in range(sc.n_solid) if sc.solid_is_dummy[i]])
    dt, gap = sc.time_step, sc.fluid_integrate_gap
    cand, walk = ds.Engine(sc), ds.Engine(sc, fluid_verlet_skin=-1.0)
    for e in (cand, walk):
        e.initialize()
        e.update(dt, 1, 2, gap)
        s = e.download_solids()
        vel = s["vel"].copy()
        vel[dummies] = (2.0, 0.0, 0.0)
        e.upload_solids(s["pos"], vel, s["angvel"])
        e.update(dt, 3, 14, gap, use_graph=True)
    fc, fw = cand.download_fluids(), walk.download_fluids()
    moved = cand.download_solids()["pos"][dummies, 0] - walk.download_solids()["pos"][dummies, 0]
    assert np.abs(moved).max() == 0.0
    scale = max(np.abs(fw[2]).max(), 9.81)
    assert np.abs(fc[2] - fw[2]).max() <= 1e-4 * scale
    assert np.abs(fc[0] - fw[0]).max() <= 1e-9
