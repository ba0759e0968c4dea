"""ctypes driver for oracle/_ref/libref_demsph.so - the reference's own solver
compiled for the CPU by oracle/build_ref.sh.

Test infrastructure: replays a scene recipe through the reference's dataBase
API, steps solverBase::update(), and reads any device array back.  Used only by
tests/golden/make_golden.py (which needs the reference sources, so it runs
where they are) and by CPU tests that skip when the library is absent.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libref_demsph.so")

_D = C.c_double
_I = C.c_int
_P = C.c_void_p
_DP = C.POINTER(C.c_double)

# name -> (dtype, components)
FIELDS = {
    "grid.gridSize": (np.int32, 1), "grid.minBound": (np.float64, 1), "grid.maxBound": (np.float64, 1),
    "grid.cellSize": (np.float64, 1),
    "grid.cellStartFluid": (np.int32, 1), "grid.cellEndFluid": (np.int32, 1),
    "grid.cellStartSolid": (np.int32, 1), "grid.cellEndSolid": (np.int32, 1),
    "fluid.pos": (np.float64, 3), "fluid.vel": (np.float64, 3), "fluid.acc": (np.float64, 3),
    "fluid.h": (np.float64, 1), "fluid.dRho": (np.float64, 1), "fluid.sumW0": (np.float64, 1),
    "fluid.hash.value": (np.int32, 1), "fluid.hash.index": (np.int32, 1),
    "fluid.ffPrefix": (np.int32, 1), "fluid.fsPrefix": (np.int32, 1),
    "fluid.fluidRange.start": (np.int32, 1), "fluid.fluidRange.end": (np.int32, 1),
    "solid.pos": (np.float64, 3), "solid.vel": (np.float64, 3), "solid.acc": (np.float64, 3),
    "solid.angvel": (np.float64, 3), "solid.torque": (np.float64, 3), "solid.normal": (np.float64, 3),
    "solid.radius": (np.float64, 1), "solid.effRadius": (np.float64, 1), "solid.invMass": (np.float64, 1),
    "solid.hash.value": (np.int32, 1), "solid.hash.index": (np.int32, 1), "solid.ssPrefix": (np.int32, 1),
    "solid.solidRange.start": (np.int32, 1), "solid.solidRange.end": (np.int32, 1),
    "solid.fluidSolidRange.start": (np.int32, 1), "solid.fluidSolidRange.end": (np.int32, 1),
    "clump.centroid": (np.float64, 3), "clump.vel": (np.float64, 3), "clump.acc": (np.float64, 3),
    "clump.angvel": (np.float64, 3), "clump.torque": (np.float64, 3),
    "ff.pointed": (np.int32, 1), "ff.pointing": (np.int32, 1), "ff.hash.index": (np.int32, 1),
    "fs.pointed": (np.int32, 1), "fs.pointing": (np.int32, 1), "fs.force": (np.float64, 3),
    "fs.hash.index": (np.int32, 1),
    "ss.pointed": (np.int32, 1), "ss.pointing": (np.int32, 1), "ss.force": (np.float64, 3),
    "ss.torque": (np.float64, 3), "ss.sliding": (np.float64, 3), "ss.rolling": (np.float64, 3),
    "ss.torsion": (np.float64, 3), "ss.hash.index": (np.int32, 1),
    "bond.pointed": (np.int32, 1), "bond.pointing": (np.int32, 1), "bond.isBonded": (np.int32, 1),
    "bond.normalForce": (np.float64, 1), "bond.torsionTorque": (np.float64, 1),
    "bond.shearForce": (np.float64, 3), "bond.bendingTorque": (np.float64, 3),
    "bond.contactNormal": (np.float64, 3), "bond.contactPoint": (np.float64, 3),
}


def available():
    return os.path.exists(LIB_PATH)


def _load():
    lib = C.CDLL(LIB_PATH)
    lib.ref_new.restype = _P
    lib.ref_get.restype = C.c_long
    lib.ref_get.argtypes = [_P, C.c_char_p, _P, C.c_long]
    lib.ref_time_step.restype = _D
    for name in ("ref_free", "ref_initialize", "ref_update"):
        getattr(lib, name).argtypes = [_P]
    for name in ("ref_istep", "ref_num_steps", "ref_gap"):
        getattr(lib, name).argtypes = [_P]
        getattr(lib, name).restype = _I
    lib.ref_time_step.argtypes = [_P]
    return lib


def _ptr(a):
    return a.ctypes.data_as(_DP)


class RefSolver:
    """The reference's solverBase, built from a recipe and stepped one update() at a time."""

    def __init__(self, jacobi_continuity=True):
        self.lib = _load()
        self.lib.ref_set_jacobi(_I(1 if jacobi_continuity else 0))
        self.h = self.lib.ref_new()

    def __del__(self):
        try:
            self.lib.ref_free(self.h)
        except Exception:
            pass

    # --- recipe target: the reference's setup calls ---
    def setDomain(self, o, s):
        self.lib.ref_set_domain(_P(self.h), *map(_D, o), *map(_D, s))

    def setGravity(self, g):
        self.lib.ref_set_gravity(_P(self.h), *map(_D, g))

    def setSimulationParameterTimeStep(self, dt):
        self.lib.ref_set_time_step(_P(self.h), _D(dt))

    def setSimulationParameterMaximumTime(self, t):
        self.lib.ref_set_maximum_time(_P(self.h), _D(t))

    def setSimulationParameterNumFrames(self, n):
        self.lib.ref_set_num_frames(_P(self.h), _I(n))

    def setFluidIntegrateGap(self, g):
        self.lib.ref_set_fluid_integrate_gap(_P(self.h), _I(g))

    def setHertzianContactModel(self, mi, mj, *v):
        self.lib.ref_set_hertzian(_P(self.h), _I(mi), _I(mj), *map(_D, v))

    def setLinearContactModel(self, mi, mj, *v):
        self.lib.ref_set_linear(_P(self.h), _I(mi), _I(mj), *map(_D, v))

    def setBondedContactModel(self, mi, mj, *v):
        self.lib.ref_set_bonded(_P(self.h), _I(mi), _I(mj), *map(_D, v))

    def addFluid(self, p, v, sl, rho, c, nu):
        p = np.ascontiguousarray(p, dtype=np.float64)
        self.lib.ref_add_fluid(_P(self.h), _I(len(p)), _ptr(p), *map(_D, v), _D(sl), _D(rho), _D(c), _D(nu))

    def addDummyParticleWall(self, p, spacing):
        p = np.ascontiguousarray(p, dtype=np.float64)
        self.lib.ref_add_dummy_wall(_P(self.h), _I(len(p)), _ptr(p), _D(spacing))

    def addSolid(self, p, v, r, rho, mat):
        p = np.ascontiguousarray(p, dtype=np.float64)
        self.lib.ref_add_solid(_P(self.h), _I(len(p)), _ptr(p), *map(_D, v), _D(r), _D(rho), _I(mat))

    def addInfiniteWall(self, p, n, mat):
        self.lib.ref_add_infinite_wall(_P(self.h), *map(_D, p), *map(_D, n), _I(mat))

    def addCluster(self, p, r, rho, v, mat):
        p = np.ascontiguousarray(p, dtype=np.float64)
        r = np.ascontiguousarray(r, dtype=np.float64)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        self.lib.ref_add_cluster(_P(self.h), _I(len(p)), _ptr(p), _ptr(r), _ptr(rho), *map(_D, v), _I(mat))

    def addClump(self, p, r, c, v, w, mass, I6, mat):
        p = np.ascontiguousarray(p, dtype=np.float64)
        r = np.ascontiguousarray(r, dtype=np.float64)
        I6 = np.ascontiguousarray(I6, dtype=np.float64)
        self.lib.ref_add_clump(_P(self.h), _I(len(p)), _ptr(p), _ptr(r), *map(_D, c), *map(_D, v), *map(_D, w),
                               _D(mass), _ptr(I6), _I(mat))

    # --- run ---
    def initialize(self):
        self.lib.ref_initialize(_P(self.h))

    def update(self):
        self.lib.ref_update(_P(self.h))

    @property
    def istep(self):
        return self.lib.ref_istep(_P(self.h))

    @property
    def gap(self):
        return self.lib.ref_gap(_P(self.h))

    @property
    def time_step(self):
        return self.lib.ref_time_step(_P(self.h))

    def get(self, name):
        dt, comp = FIELDS[name]
        n = self.lib.ref_get(_P(self.h), name.encode(), None, 0)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n * comp, dtype=dt)
        self.lib.ref_get(_P(self.h), name.encode(), out.ctypes.data_as(_P), n * comp)
        return out.reshape(n, comp) if comp == 3 else out

    def snapshot(self, names=None):
        return {k: self.get(k) for k in (names or FIELDS)}
