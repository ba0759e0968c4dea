"""bench.py's two arms measure the same workload, and the reference arm never
touches the product: its scene comes from the oracle's own assembly and the
product library is not loaded in its process."""
import importlib.util
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Args:
    gpus = 1


@pytest.mark.parametrize("config", (0, 2))
def test_both_arms_print_the_same_config(ds, config):
    """workload_config from the product's scene and from the oracle's scene
    (same recipe) are equal, key for key."""
    if not ds.library_available():
        pytest.skip("product library not built")
    b = _bench()
    recipe = b.make_recipe(config)
    _, prod = ds.build_scene(recipe)
    _, orc = b.oracle_scene(recipe)
    assert b.workload_config(config, prod, _Args, 0) == b.workload_config(config, orc, _Args, 0)


def test_bench_step_is_one_fluid_period():
    """One bench step of the coupled workload is one fluid period: its updates
    count the fluid once and the mobile solids gap times."""
    b = _bench()
    recipe = b.make_recipe(2)
    _, sc = b.oracle_scene(recipe)
    gap = sc.fluid_integrate_gap
    assert gap > 1
    nf, nm, _ = b.mobile_counts(sc)
    cfg = b.workload_config(2, sc, _Args, 0)
    assert cfg["updates_per_step"] == nf + gap * nm
    # any gap-aligned window of K bench steps holds K fluid steps
    assert b.updates_for(1 + 3 * gap, 5 * gap, gap, nf, nm) == 5 * (nf + gap * nm)


def test_reference_arm_does_not_load_the_product_library(tmp_path):
    """The reference arm, run as the driver runs it, maps no file of the
    product package: only the oracle's library."""
    code = (
        "import sys, runpy\n"
        f"sys.argv = ['bench.py', '--impl', 'reference', '--config', '0', '--steps', '1', '--warmup', '1']\n"
        f"runpy.run_path({os.path.join(ROOT, 'bench.py')!r}, run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('PRODUCT_LOADED' if 'libdemsph_gb300' in maps else 'PRODUCT_NOT_LOADED')\n"
        "print('ORACLE_LOADED' if 'liboracle_demsph' in maps else 'ORACLE_NOT_LOADED')\n")
    if not os.path.exists(os.path.join(ROOT, "oracle", "liboracle_demsph.so")):
        pytest.skip("oracle not built")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=str(tmp_path), timeout=600)
    assert r.returncode == 0, r.stderr
    assert "PRODUCT_NOT_LOADED" in r.stdout and "ORACLE_LOADED" in r.stdout, r.stdout
    assert '"impl": "reference"' in r.stdout


def test_every_timed_stage_has_algorithmic_bytes():
    """Each stage the engine times (its TIMED tags) has an algorithmic-bytes
    formula in bench.py, so the roofline of whichever stage dominates a line
    is defined (the clump force only where clumps exist is included too)."""
    import re
    src = ""
    for name in ("engine.cu",):
        with open(os.path.join(ROOT, "dem-sphsource_gb300", "csrc", name)) as f:
            src += f.read()
    stages = sorted(set(re.findall(r'TIMED\("([a-z_]+)"\)', src)))
    assert "continuity" in stages and "pair_forces" in stages and "contact_forces" in stages
    counts = {"solid_pairs": 10, "n_solid_active": 5, "n_fluid": 7, "bonds": 3, "n_solid": 9, "fluid_partners": 60.0,
              "fluid_solid_partners": 2.0, "coupling_pairs": 4, "n_pebbles": 2}
    b = _bench()
    missing = [s for s in stages if not b.stage_bytes(s, counts)]
    assert missing == []
