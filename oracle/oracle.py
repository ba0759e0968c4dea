"""ctypes driver for oracle/liboracle_demsph.so - the FP64 CPU oracle.

TEST INFRASTRUCTURE: the reference side of the GPU engine's parity tests, the CPU
baseline leg of bench.py, and nothing else.  The product never loads it.

The oracle takes the same ``demsph_scene`` the engine takes (built by the
package's scene builder) and exposes the reference's arrays under the same
names as oracle/refrun.py, so the two can be compared field by field.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .refrun import FIELDS as REF_FIELDS

# the reference's arrays plus what only the oracle keeps (the clump
# orientation: the reference never integrates it)
FIELDS = dict(REF_FIELDS, **{"clump.orientation": (np.float64, 4)})

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_demsph.so")

_P = C.c_void_p
_D = C.c_double
_I = C.c_int

_lib = None


def available():
    return os.path.exists(LIB_PATH)


def load():
    global _lib
    if _lib is None:
        lib = C.CDLL(LIB_PATH)
        lib.oracle_create.restype = _P
        lib.oracle_create.argtypes = [_P, _I]
        lib.oracle_get.restype = C.c_long
        lib.oracle_get.argtypes = [_P, C.c_char_p, _P, C.c_long]
        for n in ("oracle_destroy", "oracle_initialize"):
            getattr(lib, n).argtypes = [_P]
        lib.oracle_neighbor_search.argtypes = [_P, _I, _I]
        lib.oracle_append.argtypes = [_P, _P]
        lib.oracle_append.restype = _I
        lib.oracle_solid_integrate_before_contact.argtypes = [_P, _D]
        lib.oracle_fluid_integrate.argtypes = [_P, _D, _I, _I]
        lib.oracle_solid_contact_after_fluid_integrate.argtypes = [_P, _D]
        lib.oracle_solid_integrate_after_contact.argtypes = [_P, _D]
        lib.oracle_update.argtypes = [_P, _D, _I, _I, _I]
        lib.oracle_set_threads.argtypes = [_I]
        lib.oracle_max_threads.restype = _I
        _lib = lib
    return _lib


def set_threads(n):
    load().oracle_set_threads(int(n))


def max_threads():
    return load().oracle_max_threads()


class OracleSolver:
    """The reference's step restated in FP64 on the CPU."""

    def __init__(self, scene, fixes=0):
        self.lib = load()
        self.scene = scene
        self.h = self.lib.oracle_create(C.cast(C.byref(scene), _P), _I(fixes))
        if not self.h:
            raise RuntimeError("oracle_create failed")

    def __del__(self):
        try:
            self.lib.oracle_destroy(self.h)
        except Exception:
            pass

    def initialize(self):
        self.lib.oracle_initialize(self.h)

    def neighbor_search(self, i_step, gap):
        self.lib.oracle_neighbor_search(self.h, i_step, gap)

    def append(self, additions):
        """Particles of the scene `additions` added after the start (oracle_append)."""
        if self.lib.oracle_append(self.h, C.cast(C.byref(additions), _P)) != 0:
            raise ValueError("oracle_append: walls and clumps cannot be added after the start")
        self._keep = getattr(self, "_keep", []) + [additions]

    def solid_integrate_before_contact(self, dt):
        self.lib.oracle_solid_integrate_before_contact(self.h, dt)

    def fluid_integrate(self, dt, i_step, gap):
        self.lib.oracle_fluid_integrate(self.h, dt, i_step, gap)

    def solid_contact_after_fluid_integrate(self, dt):
        self.lib.oracle_solid_contact_after_fluid_integrate(self.h, dt)

    def solid_integrate_after_contact(self, dt):
        self.lib.oracle_solid_integrate_after_contact(self.h, dt)

    def update(self, dt, first_step, n_steps, gap):
        self.lib.oracle_update(self.h, dt, first_step, n_steps, gap)

    def get(self, name):
        dt, comp = FIELDS[name]
        n = self.lib.oracle_get(self.h, name.encode(), None, 0)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n * comp, dtype=dt)
        self.lib.oracle_get(self.h, name.encode(), out.ctypes.data_as(_P), n * comp)
        return out.reshape(n, comp) if comp > 1 else out
