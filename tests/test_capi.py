"""The C ABI library: it loads, exports every function include/demsph_gb300.h
declares, and its scene builder follows the reference's setup semantics
(core/dataBase.h:33-219, core/dataBase.cpp:3-177).  No GPU needed: nothing
here launches a kernel."""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "demsph_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^DEMSPH_API\s+[\w\s\*]*?\b(demsph_\w+)\s*\(", text, flags=re.M)))


def test_library_loads_and_exports_every_declared_symbol(ds):
    lib = ds.load_library()
    names = declared_functions()
    assert len(names) >= 45
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []
    assert b"sm_103a" in lib.demsph_version()


def test_status_strings(ds):
    lib = ds.load_library()
    assert lib.demsph_status_string(0) == b"ok"
    assert lib.demsph_status_string(5) == b"list capacity exceeded"
    assert lib.demsph_status_string(99) == b"unknown status"


def test_create_rejects_bad_arguments_without_touching_a_gpu(ds):
    lib = ds.load_library()
    h = C.c_void_p()
    assert lib.demsph_create(None, None, C.byref(h)) == 1
    assert lib.demsph_destroy(None) == 1
    assert lib.demsph_initialize(None) == 1


def _view(arr_ptr, n, comp=1, dtype=np.float64):
    return np.ctypeslib.as_array(arr_ptr, shape=(n * comp,)).reshape(n, comp) if n else np.zeros((0, comp))


def test_builder_derived_quantities_follow_the_reference(ds):
    b = ds.Builder()
    p = np.array([[0.1, 0.2, 0.3], [0.4, 0.5, 0.6]])
    b.addFluid(p, (1, 2, 3), 0.013, 1000.0, 20.0, 1e-6)
    b.addDummyParticleWall(p + 1, 0.005)
    b.addSolid(p + 2, (0, 0, -1), 0.002, 2500.0, 3)
    b.addCluster(p + 3, [0.001, 0.0015], [2000.0, 0.0], (0, 0, 0), 1)
    b.addCluster(p + 4, [0.001, 0.001], [2000.0, 2000.0], (0, 0, 0), 1)
    I = (2e-6, 3e-6, 4e-6, 0.0, 0.0, 0.0)
    b.addClump(p + 5, [0.001, 0.002], (5.25, 5.35, 5.45), (1, 0, 0), (0, 0, 10.0), 0.05, I, 2)
    s = b.scene()
    assert (s.n_fluid, s.n_solid, s.n_clump) == (2, 10, 1)
    h = _view(s.fluid_smoothing_length, 2)[:, 0]
    assert np.all(h == 0.013)
    eff = _view(s.solid_effective_radius, 10)[:, 0]
    rad = _view(s.solid_radius, 10)[:, 0]
    im = _view(s.solid_inverse_mass, 10)[:, 0]
    dummy = _view(s.solid_is_dummy, 10, dtype=np.int32)[:, 0]
    cluster = _view(s.solid_cluster, 10, dtype=np.int32)[:, 0]
    clump = _view(s.solid_clump, 10, dtype=np.int32)[:, 0]
    # dummy walls: search radius 2.6 r, fixed, dummy flag (dataBase.cpp:19-31)
    assert np.allclose(eff[:2], 2.6 * 0.005) and np.all(im[:2] == 0) and np.all(dummy[:2] == 1)
    # solids: 1.1 r, inverse mass of a sphere (dataBase.cpp:33-53)
    assert np.allclose(eff[2:4], 1.1 * 0.002)
    assert im[2] == 1.0 / (4.0 / 3.0 * 0.002 ** 3 * math.pi * 2500.0)
    # clusters get consecutive ids; zero density means infinite mass (dataBase.cpp:84-118)
    assert list(cluster[4:8]) == [0, 0, 1, 1] and im[5] == 0.0 and im[4] > 0
    # clump pebbles share the clump's mass by (2r)^3 volume (dataBase.cpp:120-177)
    vol = (2 * 0.001) ** 3 + (2 * 0.002) ** 3
    assert np.isclose(im[8], 1.0 / ((2 * 0.001) ** 3 * 0.05 / vol))
    assert list(clump[8:]) == [0, 0]
    vel = _view(s.solid_velocity, 10, 3)
    r8 = (p + 5)[0] - np.array([5.25, 5.35, 5.45])
    assert np.allclose(vel[8], np.array([1, 0, 0]) + np.cross([0, 0, 10.0], r8))
    assert _view(s.clump_pebble_start, 1, dtype=np.int32)[0, 0] == 8
    assert _view(s.clump_pebble_end, 1, dtype=np.int32)[0, 0] == 10
    invI = _view(s.clump_inverse_inertia, 1, 6)[0]
    assert np.allclose(invI[:3], [1 / 2e-6, 1 / 3e-6, 1 / 4e-6])


def test_builder_validation_messages(ds):
    b = ds.Builder()
    with pytest.raises(ds.DemSphError, match="material index exceeds"):
        b.addSolid([[0, 0, 0]], (0, 0, 0), 0.001, 1000.0, 10)
    with pytest.raises(ds.DemSphError, match="material index exceeds"):
        b.setHertzianContactModel(3, 10, 1, 1, 1, 0, 0, 0, 0, 0)
    with pytest.raises(ds.DemSphError, match="time step"):
        b.setSimulationParameterTimeStep(-1.0)
    with pytest.raises(ds.DemSphError, match="at least 1"):
        b.setFluidIntegrateGap(0)
    with pytest.raises(ds.DemSphError, match="domain size"):
        b.setDomain((0, 0, 0), (1, 0, 1))
    with pytest.raises(ds.DemSphError, match="must be the same"):
        b.addCluster([[0, 0, 0], [1, 1, 1]], [0.001], [1000.0, 1000.0], (0, 0, 0), 0)


def test_contact_table_layout(ds):
    b = ds.Builder(n_material=4)
    b.setHertzianContactModel(2, 1, 1.5, 2.5, 0.7, 0.1, 0.2, 0.3, 0.4, 0.5)
    b.setBondedContactModel(3, 3, 9.0, 2.5, 1.0, 1e6, 2e6, 0.3)
    s = b.scene()
    nslot = 4 * 5 // 2
    hz = _view(s.hertzian, nslot, 8)
    bd = _view(s.bonded, nslot, 6)
    # getCombinedIndex(1, 2) = 1 * (2*4 - 1 + 1) / 2 + 2 - 1 = 5 (core/hostStructs.h:369-384)
    assert np.allclose(hz[5], [1.5, 2.5, 0.7, 0.1, 0.2, 0.3, 0.4, 0.5])
    assert np.all(hz[0][2] == 1.0)  # default restitution 1
    assert np.allclose(bd[9], [1.0, 9.0, 2.5, 1e6, 2e6, 0.3])
    assert np.allclose(bd[0], [1.0, 0.0, 2.0, 0.0, 0.0, 0.0])  # defaults gamma 1, k_n/k_s 2
