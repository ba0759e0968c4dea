"""Helpers shared by the parity tests: run the GPU engine and the FP64 oracle
side by side on the same scene and compare them.

Tolerances (stated once, used by every test):

* integer artefacts (cell keys, sorted order, cell spans, pair lists, bond
  endpoints and states): identical;
* positions: |x - x64| <= POS_TOL * (largest particle spacing in the scene);
* fluid acceleration: |a - a64| <= FORCE_TOL * max(|a64|, |g|) per particle
  (|g| is the physical scale of the net force per unit mass in a fluid near
  hydrostatic balance; a per-particle |a64| alone is ill-posed where pressure
  forces cancel);
* density change: |dRho - dRho64| <= DRHO_TOL * rho0;
* contact forces, torques and springs per pair, and the accelerations,
  torques and spins of solids: |f - f64| <= FORCE_TOL * (|f64| + S) with
  S = max(1e-3 max|f64|, floor); the floor is the physical scale of the
  quantity (weight m g of the lightest grain for forces, m g r for torques,
  1e-6 r for springs, g dt n / r for spins), so that a field that is still
  ~0 everywhere is not measured by its rounding noise.  A quantity that is
  ~0 for one particle or pair because its terms cancel (a head-on contact:
  no tangential motion, no torque) is measured against the sum of its terms
  instead: a solid's acceleration against sum_j |F_ij| / m_i (a grain at
  rest in a bed), its torque against r_i sum_j |F_ij|, its spin against what
  that torque turns in the steps, a pair's torque against min(r) |F_pair|,
  and its springs against the relative motion at the contact times n dt;
* velocities: |v - v64| <= FORCE_TOL * max(|v64|, g dt n) after n steps.

These bounds hold for ONE step from the same state (the per-step force
tolerance).  Over several steps the trajectories of FP32 and FP64 separate -
granular contact dynamics amplify any difference - so multi-step comparisons
use DRIFT_TOL for quantities that integrate state (springs, bond forces,
torques of sliding contacts) and position bounds for the run.
"""
from __future__ import annotations

import numpy as np

FORCE_TOL = 1.0e-5
DRIFT_TOL = 1.0e-4
POS_TOL = 1.0e-9
DRHO_TOL = 1.0e-6
G = 9.81


def oracle_for(scene, fixes=0):
    from oracle.oracle import OracleSolver
    o = OracleSolver(scene, fixes=fixes)
    return o


def engine_artefacts(eng):
    out = {}
    if eng.nf:
        h = eng.cell_hash(0)
        out["fluid.hash.value"], out["fluid.hash.index"] = h["value"], h["index"]
        out["grid.cellStartFluid"], out["grid.cellEndFluid"] = h["start"], h["end"]
        ff = eng.fluid_pairs()
        out["fluid.ffPrefix"], out["ff.pointed"], out["ff.pointing"] = ff["prefix"], ff["pointed"], ff["pointing"]
        fs = eng.fluid_solid_pairs()
        out["fluid.fsPrefix"], out["fs.pointed"], out["fs.pointing"] = fs["prefix"], fs["pointed"], fs["pointing"]
    if eng.ns:
        h = eng.cell_hash(1)
        out["solid.hash.value"], out["solid.hash.index"] = h["value"], h["index"]
        out["grid.cellStartSolid"], out["grid.cellEndSolid"] = h["start"], h["end"]
        ss = eng.solid_pairs()
        out["solid.ssPrefix"], out["ss.pointed"], out["ss.pointing"] = ss["prefix"], ss["pointed"], ss["pointing"]
        for k in ("force", "torque", "sliding", "rolling", "torsion"):
            out["ss." + k] = ss[k]
        b = eng.bonds()
        for k in ("pointed", "pointing", "isBonded", "normalForce", "torsionTorque", "shearForce", "bendingTorque",
                  "contactNormal", "contactPoint"):
            out["bond." + k] = b[k]
    return out


INT_FIELDS = ("fluid.hash.value", "fluid.hash.index", "grid.cellStartFluid", "grid.cellEndFluid", "fluid.ffPrefix",
              "ff.pointed", "ff.pointing", "fluid.fsPrefix", "fs.pointed", "fs.pointing", "solid.hash.value",
              "solid.hash.index", "grid.cellStartSolid", "grid.cellEndSolid", "solid.ssPrefix", "ss.pointed",
              "ss.pointing", "bond.pointed", "bond.pointing", "bond.isBonded")


def compare_integer_artefacts(eng, orc, skip_fluid_hash=False):
    """Returns a list of mismatching field names (empty when identical)."""
    art = engine_artefacts(eng)
    bad = []
    for k in INT_FIELDS:
        if k not in art:
            continue
        if skip_fluid_hash and k.startswith(("fluid.hash", "grid.cellStartFluid", "grid.cellEndFluid")):
            continue
        a, o = art[k], orc.get(k)
        if a.shape != o.shape or not np.array_equal(a, o):
            bad.append(k)
    return bad, art


def rel_pair_error(a, o, floor=0.0):
    """max |a - o| / (|o| + max(1e-3 max|o|, floor)) over rows (vector norm per row)."""
    if len(o) == 0:
        return 0.0
    no = np.linalg.norm(o, axis=1) if o.ndim == 2 else np.abs(o)
    na = np.linalg.norm(a - o, axis=1) if o.ndim == 2 else np.abs(a - o)
    scale = no + max(1.0e-3 * no.max(), floor, 1e-300)
    return float(np.max(na / scale))


def rel_rows_scaled(a, o, floor, scale):
    """rel_pair_error with a per-row scale added to the floor: max over rows of
    |a - o| / (|o| + max(1e-3 max|o|, floor, scale_row))."""
    if len(o) == 0:
        return 0.0
    no = np.linalg.norm(o, axis=1)
    na = np.linalg.norm(a - o, axis=1)
    den = no + np.maximum(max(1.0e-3 * no.max(), floor, 1e-300), scale)
    return float(np.max(na / den))


def solid_scales(scene):
    """Lightest massive grain's mass and the smallest radius of the scene."""
    ns = scene.n_solid
    if ns == 0:
        return 1.0, 1.0
    im = np.ctypeslib.as_array(scene.solid_inverse_mass, shape=(ns,))
    r = np.ctypeslib.as_array(scene.solid_radius, shape=(ns,))
    dummy = np.ctypeslib.as_array(scene.solid_is_dummy, shape=(ns,))
    live = (im > 0) & (dummy == 0)
    if not live.any():
        return 1.0, float(r.min())
    return float(1.0 / im[live].max()), float(r[live].min())


def pair_floors(scene, dt, steps):
    m, r = solid_scales(scene)
    return {"force": m * G, "torque": m * G * r, "spring": 1e-6 * r, "spin": G * dt * max(steps, 1) / r,
            "acc": G}


def contact_scales(orc, ns):
    """Per solid: the sum of the magnitudes of its pair contact forces in the
    oracle's list (both sides), the "sum of pair terms" scale of a net
    quantity that cancels (a torque whose contacts push through the centre)."""
    s = np.zeros(ns)
    f = orc.get("ss.force")
    if len(f):
        m = np.linalg.norm(f, axis=1)
        np.add.at(s, orc.get("ss.pointed"), m)
        np.add.at(s, orc.get("ss.pointing"), m)
    return s


def state_errors(eng, orc, dx, steps_done, dt, rho0=1000.0):
    """Per-quantity normalised errors of the engine against the oracle.

    Torques and spins of a solid are scaled by at least the sum of its pair
    terms: r_i sum_j |F_ij| for the torque (the lever times the contact forces
    it balances) and steps dt r_i sum_j |F_ij| / I_i for the spin, so that a
    torque the FP64 oracle gives as rounding noise (a head-on contact) is
    measured against the forces acting, not against its own zero."""
    e = {}
    if eng.nf:
        pos, vel, acc, drho = eng.download_fluids()
        e["fluid.pos"] = float(np.max(np.abs(pos - orc.get("fluid.pos")))) / dx
        v64 = orc.get("fluid.vel")
        vs = max(np.abs(v64).max(), G * dt * max(steps_done, 1))
        e["fluid.vel"] = float(np.max(np.abs(vel - v64))) / vs
        a64 = orc.get("fluid.acc")
        e["fluid.acc"] = float(np.max(np.linalg.norm(acc - a64, axis=1) /
                                      np.maximum(np.linalg.norm(a64, axis=1), G)))
        e["fluid.dRho"] = float(np.max(np.abs(drho - orc.get("fluid.dRho")))) / rho0
    if eng.ns:
        s = eng.download_solids()
        e["solid.pos"] = float(np.max(np.abs(s["pos"] - orc.get("solid.pos")))) / dx
        v64 = orc.get("solid.vel")
        vs = max(np.abs(v64).max(), G * dt * max(steps_done, 1))
        e["solid.vel"] = float(np.max(np.abs(s["vel"] - v64))) / vs
        fl = pair_floors(eng.scene, dt, steps_done)
        ns = eng.ns
        r = np.ctypeslib.as_array(eng.scene.solid_radius, shape=(ns,))
        im = np.ctypeslib.as_array(eng.scene.solid_inverse_mass, shape=(ns,))
        fsum = contact_scales(orc, ns)
        # a grain at rest in a bed: its contact forces (many weights deep in the
        # bed) cancel to ~0 net, so the net acceleration is measured against
        # sum_j |F_ij| / m_i as well as g
        e["solid.acc"] = rel_rows_scaled(s["acc"], orc.get("solid.acc"), fl["acc"], fsum * im)
        tscale = r * fsum
        # spin change the summed contact torques give over the steps: dt n r F / (0.4 m r^2)
        wscale = np.where(im > 0, max(steps_done, 1) * dt * fsum * im / np.maximum(0.4 * r, 1e-300), 0.0)
        e["solid.torque"] = rel_rows_scaled(s["torque"], orc.get("solid.torque"), fl["torque"], tscale)
        e["solid.angvel"] = rel_rows_scaled(s["angvel"], orc.get("solid.angvel"), fl["spin"], wscale)
        e["solid.normal"] = float(np.max(np.abs(s["normal"] - orc.get("solid.normal"))))
    return e


def check_step(eng, orc, sc, dx, step, dt, tol_force, tol_pos):
    """Asserts the engine's state, per-pair contact forces, torques, springs
    and bond forces are within tolerance of the oracle's after `step` steps."""
    err = state_errors(eng, orc, dx, step, dt)
    for k, v in err.items():
        tol = {"fluid.pos": tol_pos, "solid.pos": tol_pos, "fluid.dRho": DRHO_TOL, "solid.normal": 1e-5}.get(k, tol_force)
        assert v <= tol, f"step {step}: {k} error {v:.3e} > {tol:.1e}"
    art = engine_artefacts(eng)
    fl = pair_floors(sc, dt, step)
    if eng.ns and len(art["ss.pointed"]):
        # per-pair scales (the "sum of pair terms" of a quantity that can cancel
        # to ~0, e.g. in a head-on contact): the pair torque against the lever
        # times the pair force; a spring against what the relative motion at
        # the contact adds to it over the steps
        a, b = orc.get("ss.pointed"), orc.get("ss.pointing")
        r = np.ctypeslib.as_array(sc.solid_radius, shape=(sc.n_solid,))
        v, w = orc.get("solid.vel"), orc.get("solid.angvel")
        f64 = orc.get("ss.force")
        tscale = np.minimum(r[a], r[b]) * np.linalg.norm(f64, axis=1)
        rel_motion = (np.linalg.norm(v[a] - v[b], axis=1) + 2.0 * (r[a] * np.linalg.norm(w[a], axis=1) +
                                                                      r[b] * np.linalg.norm(w[b], axis=1)))
        sscale = max(step, 1) * dt * rel_motion
        assert rel_pair_error(art["ss.force"], f64, fl["force"]) <= tol_force
        assert rel_rows_scaled(art["ss.torque"], orc.get("ss.torque"), fl["torque"], tscale) <= tol_force
        for k in ("sliding", "rolling", "torsion"):
            e = rel_rows_scaled(art["ss." + k], orc.get("ss." + k), fl["spring"], sscale)
            assert e <= tol_force, f"step {step}: ss.{k} error {e:.3e} > {tol_force:.1e}"
    if eng.ns and len(art["bond.pointed"]):
        assert rel_pair_error(art["bond.normalForce"], orc.get("bond.normalForce"), fl["force"]) <= tol_force
        assert rel_pair_error(art["bond.shearForce"], orc.get("bond.shearForce"), fl["force"]) <= tol_force
    return err
