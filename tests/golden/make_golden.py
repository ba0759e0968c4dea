"""Generates the golden fixtures in tests/golden/ by running the REFERENCE'S OWN
solver (core/*.cu, core/*.cpp compiled for the CPU by oracle/build_ref.sh)
on the small seeded scenes of dem-sphsource_gb300/scenes.py.

Run where the reference sources exist:

    sh oracle/build_ref.sh && python tests/golden/make_golden.py

Each fixture stores, after initialisation and after selected update() calls,
every array the reference keeps on the device for the step (positions,
velocities, densities, forces, springs, bonds, cell hashes, pair lists, ...),
plus a digest of the scene inputs so a test can tell if the generator
drifted.  The continuity pass runs with every thread reading the pass-start
densities (see oracle/ref_harness.cpp).
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import conftest  # noqa: E402  (loads the package)

from oracle.refrun import FIELDS, RefSolver  # noqa: E402

SNAP_STEPS = (0, 1, 2, 5, 10)
SCENES = ("tiny_dam_break", "tiny_granular", "tiny_coupled", "tiny_escape", "tiny_two_fluids", "tiny_linear",
          "tiny_tumbling")


def scene_digest(scene):
    """sha256 over the builder's input arrays (what every solver receives)."""
    h = hashlib.sha256()
    n = {"fluid": scene.n_fluid, "solid": scene.n_solid, "clump": scene.n_clump, "wall": scene.n_wall}
    for name, cnt, comp in (("fluid_position", n["fluid"], 3), ("fluid_smoothing_length", n["fluid"], 1),
                            ("solid_position", n["solid"], 3), ("solid_radius", n["solid"], 1),
                            ("solid_inverse_mass", n["solid"], 1), ("clump_centroid", n["clump"], 3),
                            ("wall_point", n["wall"], 3)):
        ptr = getattr(scene, name)
        if cnt and ptr:
            h.update(np.ctypeslib.as_array(ptr, shape=(cnt * comp,)).tobytes())
    h.update(np.array([scene.time_step, scene.fluid_integrate_gap], dtype=np.float64).tobytes())
    return h.hexdigest()


def load(path):
    """Returns {step: {field: array}} with de-duplicated snapshots resolved."""
    z = np.load(path)
    snaps = {int(t): {} for t in z["snap_steps"]}
    for key in z.files:
        if "/" not in key:
            continue
        tag, field = key.split("/", 1)
        t = int(tag[1:])
        if field.endswith("@"):
            continue
        snaps[t][field] = z[key]
    for key in z.files:
        if "/" in key and key.endswith("@"):
            tag, field = key[:-1].split("/", 1)
            snaps[int(tag[1:])][field] = snaps[int(z[key])][field]
    meta = {k: z[k] for k in ("digest", "time_step", "gap")}
    return snaps, meta


def make(name):
    ds = conftest.load_package()
    import dem_sphsource_gb300.scenes as scenes

    recipe = getattr(scenes, name)()
    _, sc = ds.build_scene(recipe)
    ref = RefSolver(jacobi_continuity=True)
    recipe.apply(ref)
    ref.initialize()
    out = {"digest": np.array(scene_digest(sc)), "time_step": np.array(ref.time_step), "gap": np.array(ref.gap),
           "snap_steps": np.array(SNAP_STEPS)}
    step = 0
    last = {}
    for target in SNAP_STEPS:
        while step < target:
            ref.update()
            step += 1
        for k in FIELDS:
            a = ref.get(k)
            # an array identical to its previous snapshot is stored once
            if k in last and last[k][1].shape == a.shape and np.array_equal(last[k][1], a):
                out[f"s{target}/{k}@"] = np.array(last[k][0])
                continue
            out[f"s{target}/{k}"] = a
            last[k] = (target, a)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    return path


if __name__ == "__main__":
    for n in SCENES:
        p = make(n)
        print(p, os.path.getsize(p), "bytes")
