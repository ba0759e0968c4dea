"""GB300-native coupled DEM-SPH step - Python binding of the C ABI.

The product is ``libdemsph_gb300.so`` (CUDA kernels for sm_103a plus the host
API, include/demsph_gb300.h).  This module is a thin ctypes layer over it so
Python code (tests, benchmarks, notebooks) can build a scene with the
reference's setup calls and drive the step:

    import dem_sphsource_gb300 as ds
    b = ds.Builder()
    b.setDomain(...); b.addFluid(...); ...          # the reference's dataBase calls
    eng = ds.Engine(b.scene())                       # DeviceData::copy + buildDeviceData
    eng.initialize()                                 # neighborSearch(0,1), bonds, normals
    eng.update(dt, first_step=1, n_steps=100, gap=1) # 100 x solverBase::update()
    pos, vel, acc, drho = eng.download_fluids()

There is no CPU fallback: if the library is missing or no sm_103a GPU is
present, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdemsph_gb300.so")

DEMSPH_OK = 0
DEMSPH_ERR_CAPACITY = 5
FIX_WALL_LOOP = 1
FIX_CLUMP_ROTATION = 2

_D = C.c_double
_I = C.c_int
_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)


class Scene(C.Structure):
    """ctypes mirror of ``demsph_scene`` (include/demsph_gb300.h)."""

    _fields_ = [
        ("domain_origin", _D * 3), ("domain_size", _D * 3), ("gravity", _D * 3), ("time_step", _D),
        ("fluid_integrate_gap", _I), ("maximum_time", _D), ("num_frames", _I),
        ("n_fluid", _I), ("fluid_position", _DP), ("fluid_velocity", _DP), ("fluid_acceleration", _DP),
        ("fluid_smoothing_length", _DP), ("fluid_rho0", _DP), ("fluid_drho", _DP), ("fluid_sound_speed", _DP),
        ("fluid_nu", _DP),
        ("n_solid", _I), ("solid_position", _DP), ("solid_velocity", _DP), ("solid_acceleration", _DP),
        ("solid_normal", _DP), ("solid_torque", _DP), ("solid_angular_velocity", _DP),
        ("solid_effective_radius", _DP), ("solid_radius", _DP), ("solid_inverse_mass", _DP),
        ("solid_material", _IP), ("solid_cluster", _IP), ("solid_clump", _IP), ("solid_is_dummy", _IP),
        ("n_clump", _I), ("clump_centroid", _DP), ("clump_velocity", _DP), ("clump_acceleration", _DP),
        ("clump_angular_velocity", _DP), ("clump_torque", _DP), ("clump_orientation", _DP),
        ("clump_inverse_inertia", _DP), ("clump_inverse_mass", _DP), ("clump_pebble_start", _IP),
        ("clump_pebble_end", _IP),
        ("n_wall", _I), ("wall_point", _DP), ("wall_normal", _DP), ("wall_material", _IP),
        ("n_material", _I), ("hertzian", _DP), ("linear", _DP), ("bonded", _DP),
    ]


class Options(C.Structure):
    """ctypes mirror of ``demsph_options``."""

    _fields_ = [("device", _I), ("fluid_neighbors_max", _I), ("fluid_solids_max", _I),
                ("solid_contacts_per_particle", _I), ("fixes", _I), ("debug", _I), ("solid_verlet_skin", _D),
                ("fluid_lanes", _I), ("fluid_verlet_skin", _D), ("contact_rows_per_warp", _I)]


def _options(device=0, **opts):
    """Options from keyword arguments (the field names; missing ones 0)."""
    o = Options()
    o.device = int(device)
    for name, typ in Options._fields_:
        if name in opts and name != "device":
            setattr(o, name, float(opts[name]) if typ is _D else int(opts[name]))
    return o


class Counts(C.Structure):
    _fields_ = [("fluid_pairs", C.c_longlong), ("fluid_solid_pairs", C.c_longlong), ("solid_pairs", C.c_longlong),
                ("bonds", C.c_longlong), ("bonds_intact", C.c_longlong), ("grid_cells", _I), ("grid_size", _I * 3),
                ("cell_size", _D * 3)]


class LaunchShapes(C.Structure):
    _fields_ = [("fluid_lanes", _I), ("clump_lanes", _I), ("contact_force_rows", _I), ("fluid_bit_lists", _I),
                ("fluid_bit_words", _I)]


class RunStats(C.Structure):
    _fields_ = [("list_growths", C.c_longlong), ("resumed_steps", C.c_longlong), ("fused_passes", C.c_longlong)]


class AuditValues(C.Structure):
    _fields_ = [("mass", _D), ("momentum", _D * 3), ("kinetic_energy", _D), ("rotational_energy", _D),
                ("potential_energy", _D), ("fluid_density_sum", _D)]


class ServerConfig(C.Structure):
    """ctypes mirror of ``demsph_server_config``."""

    _fields_ = [("device", _I), ("workers", _I), ("chunk_steps", _I), ("hbm_budget_bytes", C.c_longlong),
                ("autotune", _I), ("graphs", _I), ("batch", _I), ("batch_round_steps", _I)]


class ServerSummary(C.Structure):
    _fields_ = [(k, C.c_longlong) for k in ("submitted", "admitted", "completed", "failed", "pending", "steps",
                                             "particle_updates", "chunks", "bytes_in_use", "peak_bytes")] + \
               [(k, _D) for k in ("busy_s", "updates_per_s", "p50_step_ms", "p99_step_ms", "create_s", "step_s",
                                  "download_s")] + \
               [(k, C.c_longlong) for k in ("batch_rounds", "batch_graph_builds")] + \
               [(k, _D) for k in ("batch_capture_s", "batch_instantiate_s", "batch_launch_s")]


class RequestInfo(C.Structure):
    _fields_ = [("state", _I), ("steps_done", _I), ("reserved_bytes", C.c_longlong), ("queued_s", _D),
                ("run_s", _D)]


class DemSphError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{message} (status {status})")
        self.status = status


_lib = None


def library_available():
    return os.path.exists(LIB_PATH)


def load_library():
    """Loads libdemsph_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                           "(dem-sphsource_gb300/build.py); there is no CPU fallback")
    lib = C.CDLL(LIB_PATH)
    lib.demsph_status_string.restype = C.c_char_p
    lib.demsph_last_error.restype = C.c_char_p
    lib.demsph_last_error.argtypes = [_P]
    lib.demsph_version.restype = C.c_char_p
    lib.demsph_builder_new.restype = _P
    lib.demsph_builder_last_error.restype = C.c_char_p
    lib.demsph_builder_last_error.argtypes = [_P]
    lib.demsph_stream.restype = _P
    lib.demsph_stream.argtypes = [_P]
    lib.demsph_kernel_launches.restype = C.c_longlong
    lib.demsph_kernel_launches.argtypes = [_P]
    lib.demsph_batch_create.argtypes = [_I, C.POINTER(_P)]
    lib.demsph_batch_destroy.argtypes = [_P]
    lib.demsph_batch_update.argtypes = [_P, C.POINTER(_P), _I, C.POINTER(_I), C.POINTER(_I), C.POINTER(_D),
                                        C.POINTER(_I), C.POINTER(_I)]
    lib.demsph_batch_get_info.argtypes = [_P, _P]
    lib.demsph_batch_last_error.argtypes = [_P]
    lib.demsph_batch_last_error.restype = C.c_char_p
    lib.demsph_frame_writer_open.argtypes = [_P, _P, C.c_char_p, C.POINTER(_P)]
    lib.demsph_frame_writer_write.argtypes = [_P, C.c_int, C.c_int, C.c_int, C.c_double]
    lib.demsph_frame_writer_flush.argtypes = [_P]
    lib.demsph_frame_writer_close.argtypes = [_P]
    lib.demsph_device_bytes.restype = C.c_longlong
    lib.demsph_device_bytes.argtypes = [_P]
    lib.demsph_estimate_bytes.restype = C.c_longlong
    lib.demsph_estimate_bytes.argtypes = [_P, _P]
    _lib = lib
    return lib


def _ptr(a, t=_DP):
    return a.ctypes.data_as(t)


def _v3(v):
    return (_D * 3)(*map(float, v))


class Builder:
    """The reference's setup API (class dataBase, core/dataBase.h:33-219) over
    the C ABI scene builder.  Method names and arguments are the reference's."""

    def __init__(self, n_material=10):
        self.lib = load_library()
        self.h = self.lib.demsph_builder_new(_I(n_material))
        if not self.h:
            raise DemSphError(1, "demsph_builder_new failed")
        self._keep = []

    def __del__(self):
        try:
            self.lib.demsph_builder_free(_P(self.h))
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc != DEMSPH_OK:
            msg = self.lib.demsph_builder_last_error(_P(self.h)).decode()
            raise DemSphError(rc, f"{what}: {msg}")

    def setDomain(self, o, s):
        self._chk(self.lib.demsph_builder_set_domain(_P(self.h), _v3(o), _v3(s)), "setDomain")

    def setGravity(self, g):
        self._chk(self.lib.demsph_builder_set_gravity(_P(self.h), _v3(g)), "setGravity")

    def setSimulationParameterTimeStep(self, dt):
        self._chk(self.lib.demsph_builder_set_time_step(_P(self.h), _D(dt)), "setSimulationParameterTimeStep")

    def setSimulationParameterMaximumTime(self, t):
        self._chk(self.lib.demsph_builder_set_maximum_time(_P(self.h), _D(t)), "setSimulationParameterMaximumTime")

    def setSimulationParameterNumFrames(self, n):
        self._chk(self.lib.demsph_builder_set_num_frames(_P(self.h), _I(n)), "setSimulationParameterNumFrames")

    def setFluidIntegrateGap(self, g):
        self._chk(self.lib.demsph_builder_set_fluid_integrate_gap(_P(self.h), _I(g)), "setFluidIntegrateGap")

    def setHertzianContactModel(self, mi, mj, *v):
        self._chk(self.lib.demsph_builder_set_hertzian(_P(self.h), _I(mi), _I(mj), *map(_D, v)),
                  "setHertzianContactModel")

    def setLinearContactModel(self, mi, mj, *v):
        self._chk(self.lib.demsph_builder_set_linear(_P(self.h), _I(mi), _I(mj), *map(_D, v)),
                  "setLinearContactModel")

    def setBondedContactModel(self, mi, mj, *v):
        self._chk(self.lib.demsph_builder_set_bonded(_P(self.h), _I(mi), _I(mj), *map(_D, v)),
                  "setBondedContactModel")

    def addFluid(self, p, v, sl, rho, c, nu):
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        self._chk(self.lib.demsph_builder_add_fluid(_P(self.h), _I(len(p)), _ptr(p), _v3(v), _D(sl), _D(rho), _D(c),
                                                    _D(nu)), "addFluid")

    def addDummyParticleWall(self, p, spacing):
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        self._chk(self.lib.demsph_builder_add_dummy_wall(_P(self.h), _I(len(p)), _ptr(p), _D(spacing)),
                  "addDummyParticleWall")

    def addSolid(self, p, v, r, rho, mat):
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        self._chk(self.lib.demsph_builder_add_solid(_P(self.h), _I(len(p)), _ptr(p), _v3(v), _D(r), _D(rho),
                                                    _I(mat)), "addSolid")

    def addInfiniteWall(self, p, n, mat):
        self._chk(self.lib.demsph_builder_add_infinite_wall(_P(self.h), _v3(p), _v3(n), _I(mat)), "addInfiniteWall")

    def addCylinderWall(self, p, axis, w, r, mat):
        self._chk(self.lib.demsph_builder_add_cylinder_wall(_P(self.h), _v3(p), _v3(axis), _v3(w), _D(r), _I(mat)),
                  "addCylinderWall")

    def addCluster(self, p, r, rho, v, mat):
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(r, dtype=np.float64).ravel()
        rho = np.ascontiguousarray(rho, dtype=np.float64).ravel()
        if len(r) != len(p) or len(rho) != len(p):  # the C call takes one count for all three arrays
            raise DemSphError(1, "addCluster: Error: the size of position, velocity, and radius vectors must be "
                                 "the same when adding a cluster.")
        self._chk(self.lib.demsph_builder_add_cluster(_P(self.h), _I(len(p)), _ptr(p), _ptr(r), _ptr(rho), _v3(v),
                                                      _I(mat)), "addCluster")

    def addClump(self, p, r, c, v, w, mass, I6, mat):
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(r, dtype=np.float64).ravel()
        if len(r) != len(p):
            raise DemSphError(1, "addClump: Error: the size of position and radius vectors must be the same when "
                                 "adding a clump.")
        I6 = (_D * 6)(*map(float, I6))
        self._chk(self.lib.demsph_builder_add_clump(_P(self.h), _I(len(p)), _ptr(p), _ptr(r), _v3(c), _v3(v), _v3(w),
                                                    _D(mass), I6, _I(mat)), "addClump")

    def scene(self):
        """The C view of the builder's arrays (valid while the builder lives and is unchanged)."""
        s = Scene()
        self._chk(self.lib.demsph_builder_scene(_P(self.h), C.byref(s)), "scene")
        s._builder = self  # keep the arrays alive
        return s


def build_scene(recipe, n_material=10):
    """Replays a scenes.Recipe on a new Builder; returns (builder, scene)."""
    b = Builder(n_material)
    recipe.apply(b)
    return b, b.scene()


FRAME_FLUID, FRAME_SOLID, FRAME_FLUID2SOLID, FRAME_ALL = 1, 2, 4, 7


class FrameWriter:
    """The frame files of class solverBase (fluid_NNNN.vtu, solid_NNNN.vtu,
    fluid2Solid_NNNN.vtu in `directory`) of one engine as binary VTU, written
    by a background thread (demsph_frame_writer_*).  Close it before the
    engine."""

    def __init__(self, engine, directory):
        self.engine = engine
        self.lib = engine.lib
        h = _P()
        engine._chk(self.lib.demsph_frame_writer_open(engine.h, C.addressof(engine.scene), str(directory).encode(),
                                                      C.byref(h)), "demsph_frame_writer_open")
        self.h = h

    def write(self, what, frame, step, time):
        """Enqueues the files of the kinds in `what` (FRAME_* bits); returns at once."""
        self.engine._chk(self.lib.demsph_frame_writer_write(self.h, what, frame, step, time),
                         "demsph_frame_writer_write")

    def flush(self):
        self.engine._chk(self.lib.demsph_frame_writer_flush(self.h), "demsph_frame_writer_flush")

    def close(self):
        if getattr(self, "h", None):
            h, self.h = self.h, None
            self.engine._chk(self.lib.demsph_frame_writer_close(h), "demsph_frame_writer_close")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Engine:
    """One scene on one GPU (the C ABI engine)."""

    def __init__(self, scene, device=0, **opts):
        """Keyword options are the fields of ``demsph_options`` (0 = default):
        fluid_neighbors_max, fluid_solids_max, solid_contacts_per_particle,
        fixes, debug, solid_verlet_skin (margin (m) of the solid contact
        candidates; < 0 = the 27-cell walk every step), fluid_lanes,
        fluid_verlet_skin, contact_rows_per_warp."""
        unknown = set(opts) - {n for n, _ in Options._fields_}
        if unknown:
            raise TypeError(f"unknown engine options: {sorted(unknown)}")
        self.lib = load_library()
        self.scene = scene
        opts = _options(device, **opts)
        h = _P()
        rc = self.lib.demsph_create(C.byref(scene), C.byref(opts), C.byref(h))
        self.h = h
        if rc != DEMSPH_OK:
            msg = self.lib.demsph_last_error(h).decode() if h else ""
            if h:
                self.lib.demsph_destroy(h)
                self.h = None
            raise DemSphError(rc, f"demsph_create: {msg}")
        self.nf, self.ns, self.nc = scene.n_fluid, scene.n_solid, scene.n_clump

    def close(self):
        if getattr(self, "h", None):
            self.lib.demsph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc != DEMSPH_OK:
            msg = self.lib.demsph_last_error(self.h).decode()
            raise DemSphError(rc, f"{what}: {msg}")

    # ---- life cycle and the five stages ----
    def initialize(self):
        self._chk(self.lib.demsph_initialize(self.h), "demsph_initialize")

    def neighbor_search(self, i_step, gap):
        self._chk(self.lib.demsph_neighbor_search(self.h, _I(i_step), _I(gap)), "demsph_neighbor_search")

    def append(self, current, additions):
        """Adds the particles of scene `additions` while the simulation runs
        (demsph_append); `current` is the scene as it stands (its parameters
        and tables; the state is the engine's).  Returns the new counts."""
        self._chk(self.lib.demsph_append(self.h, C.byref(current), C.byref(additions)), "demsph_append")
        self.nf += additions.n_fluid
        self.ns += additions.n_solid
        return self.nf, self.ns

    def solid_integrate_before_contact(self, dt):
        self._chk(self.lib.demsph_solid_integrate_before_contact(self.h, _D(dt)), "before_contact")

    def fluid_integrate(self, dt, i_step, gap):
        self._chk(self.lib.demsph_fluid_integrate(self.h, _D(dt), _I(i_step), _I(gap)), "fluid_integrate")

    def solid_contact_after_fluid_integrate(self, dt):
        self._chk(self.lib.demsph_solid_contact_after_fluid_integrate(self.h, _D(dt)), "contact")

    def solid_integrate_after_contact(self, dt):
        self._chk(self.lib.demsph_solid_integrate_after_contact(self.h, _D(dt)), "after_contact")

    def step(self, dt, i_step, gap):
        """One solverBase::update() through the five stage calls."""
        self.neighbor_search(i_step, gap)
        self.solid_integrate_before_contact(dt)
        self.fluid_integrate(dt, i_step, gap)
        self.solid_contact_after_fluid_integrate(dt)
        self.solid_integrate_after_contact(dt)

    def update(self, dt, first_step, n_steps, gap, use_graph=True):
        self._chk(self.lib.demsph_update(self.h, _D(dt), _I(first_step), _I(n_steps), _I(gap), _I(1 if use_graph else 0)),
                  "demsph_update")

    def update_io(self, dt, first_step, n_steps, gap, use_graph=True, fluid_in=None, solid_in=None,
                  fluid_out=None, solid_out=None):
        """demsph_update_io: uploads ``fluid_in`` (pos, vel, drho) and ``solid_in``
        (pos, vel, angvel) (any entry may be None), advances the steps and
        downloads into ``fluid_out`` / ``solid_out`` (same tuples), with one
        synchronisation."""
        def ptrs(t, k):
            t = t if t is not None else (None,) * k
            return [None if a is None else _ptr(a) for a in t]
        args = ptrs(fluid_in, 3) + ptrs(solid_in, 3) + ptrs(fluid_out, 3) + ptrs(solid_out, 3)
        self._chk(self.lib.demsph_update_io(self.h, _D(dt), _I(first_step), _I(n_steps), _I(gap),
                                            _I(1 if use_graph else 0), *args), "demsph_update_io")

    def synchronize(self):
        self._chk(self.lib.demsph_synchronize(self.h), "demsph_synchronize")

    # ---- timing ----
    def stream_ptr(self):
        """Address of the engine's cudaStream_t (for CUDA events around its work)."""
        return int(self.lib.demsph_stream(self.h) or 0)

    def kernel_launches(self):
        return int(self.lib.demsph_kernel_launches(self.h))

    def set_profiling(self, on):
        self._chk(self.lib.demsph_set_profiling(self.h, _I(1 if on else 0)), "set_profiling")

    def profile_report(self):
        """{stage: (launches, total_ms)} since the last report."""
        buf = C.create_string_buffer(1 << 16)
        self._chk(self.lib.demsph_profile_report(self.h, buf, _I(len(buf))), "profile_report")
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms = line.split()
            out[name] = (int(n), float(ms))
        return out

    # ---- state ----
    def download_fluids(self, out=None):
        """(pos, vel, acc, dRho) in original order; ``out`` may supply the four arrays."""
        n = self.nf
        pos, vel, acc, drho = out if out is not None else (np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3)),
                                                           np.zeros(n))
        self._chk(self.lib.demsph_download_fluids(self.h, *[None if a is None else _ptr(a) for a in (pos, vel, acc,
                                                                                                    drho)]),
                  "download_fluids")
        return pos, vel, acc, drho

    def download_solids(self, out=None):
        """dict of pos, vel, acc, normal, torque, angvel; ``out`` may supply (some of) the six arrays."""
        n = self.ns
        keys = ("pos", "vel", "acc", "normal", "torque", "angvel")
        arrs = [out.get(k) for k in keys] if out is not None else [np.zeros((n, 3)) for _ in range(6)]
        self._chk(self.lib.demsph_download_solids(self.h, *[None if a is None else _ptr(a) for a in arrs]),
                  "download_solids")
        return dict(zip(keys, arrs))

    def download_clumps(self):
        n = self.nc
        out = [np.zeros((n, 3)) for _ in range(5)] + [np.zeros((n, 4))]
        self._chk(self.lib.demsph_download_clumps(self.h, *[_ptr(a) for a in out]), "download_clumps")
        return dict(zip(("centroid", "vel", "acc", "angvel", "torque", "orientation"), out))

    def upload_fluids(self, pos=None, vel=None, drho=None):
        a = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (pos, vel, drho)]
        self._chk(self.lib.demsph_upload_fluids(self.h, *[None if x is None else _ptr(x) for x in a]), "upload_fluids")

    def upload_solids(self, pos=None, vel=None, angvel=None):
        a = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (pos, vel, angvel)]
        self._chk(self.lib.demsph_upload_solids(self.h, *[None if x is None else _ptr(x) for x in a]), "upload_solids")

    def set_gravity(self, g):
        self._chk(self.lib.demsph_set_gravity(self.h, _v3(g)), "set_gravity")

    def set_clump_velocity(self, c, v):
        self._chk(self.lib.demsph_set_clump_velocity(self.h, _I(c), _v3(v)), "set_clump_velocity")

    def add_external_force(self, i, f):
        self._chk(self.lib.demsph_add_external_force(self.h, _I(i), _v3(f)), "add_external_force")

    def add_global_damping(self, i, cd):
        self._chk(self.lib.demsph_add_global_damping(self.h, _I(i), _D(cd)), "add_global_damping")

    # ---- artefacts in the reference's index space ----
    def counts(self):
        c = Counts()
        self._chk(self.lib.demsph_get_counts(self.h, C.byref(c)), "get_counts")
        return c

    def cell_hash(self, which):
        n = self.nf if which == 0 else self.ns
        ng = self.counts().grid_cells
        value, index = np.zeros(n, np.int32), np.zeros(n, np.int32)
        start, end = np.zeros(ng, np.int32), np.zeros(ng, np.int32)
        self._chk(self.lib.demsph_export_cell_hash(self.h, _I(which), _ptr(value, _IP), _ptr(index, _IP),
                                                   _ptr(start, _IP), _ptr(end, _IP)), "export_cell_hash")
        return {"value": value, "index": index, "start": start, "end": end}

    def fluid_pairs(self):
        prefix = np.zeros(self.nf, np.int32)
        self._chk(self.lib.demsph_export_fluid_pairs(self.h, _ptr(prefix, _IP), None, None, C.c_longlong(0)), "ff")
        m = int(prefix[-1]) if self.nf else 0
        a, b = np.zeros(m, np.int32), np.zeros(m, np.int32)
        self._chk(self.lib.demsph_export_fluid_pairs(self.h, _ptr(prefix, _IP), _ptr(a, _IP), _ptr(b, _IP),
                                                     C.c_longlong(m)), "ff")
        return {"prefix": prefix, "pointed": a, "pointing": b}

    def fluid_solid_pairs(self):
        prefix = np.zeros(self.nf, np.int32)
        self._chk(self.lib.demsph_export_fluid_solid_pairs(self.h, _ptr(prefix, _IP), None, None, None,
                                                           C.c_longlong(0)), "fs")
        m = int(prefix[-1]) if self.nf else 0
        a, b, f = np.zeros(m, np.int32), np.zeros(m, np.int32), np.zeros((m, 3))
        self._chk(self.lib.demsph_export_fluid_solid_pairs(self.h, _ptr(prefix, _IP), _ptr(a, _IP), _ptr(b, _IP),
                                                           _ptr(f), C.c_longlong(m)), "fs")
        return {"prefix": prefix, "pointed": a, "pointing": b, "force": f}

    def audit(self):
        """FP64 sums over the scene: mass, momentum, kinetic / rotational /
        potential energy, fluid density sum (demsph_audit)."""
        a = AuditValues()
        self._chk(self.lib.demsph_audit(self.h, C.byref(a)), "audit")
        return {"mass": a.mass, "momentum": np.array(a.momentum[:]), "kinetic_energy": a.kinetic_energy,
                "rotational_energy": a.rotational_energy, "potential_energy": a.potential_energy,
                "fluid_density_sum": a.fluid_density_sum}

    def autotune(self):
        """Times the fluid pair loop with 1, 2, 4 and 8 threads per particle and
        keeps the fastest (demsph_autotune); returns the choice."""
        lanes = _I()
        self._chk(self.lib.demsph_autotune(self.h, C.byref(lanes)), "autotune")
        return lanes.value

    def launch_shapes(self):
        """{fluid_lanes, clump_lanes, contact_force_rows, fluid_bit_lists, fluid_bit_words} in use
        (the last two 0 when the fluid lists are lists, not membership bits)."""
        v = LaunchShapes()
        self._chk(self.lib.demsph_get_launch_shapes(self.h, C.byref(v)), "launch_shapes")
        return {n: getattr(v, n) for n, _ in LaunchShapes._fields_}

    def run_stats(self):
        """{list_growths, resumed_steps, fused_passes} of the update runs so far."""
        v = RunStats()
        self._chk(self.lib.demsph_get_run_stats(self.h, C.byref(v)), "run_stats")
        return {n: getattr(v, n) for n, _ in RunStats._fields_}

    def solid_pairs(self):
        prefix = np.zeros(self.ns, np.int32)
        self._chk(self.lib.demsph_export_solid_pairs(self.h, _ptr(prefix, _IP), *([None] * 7), C.c_longlong(0)), "ss")
        m = int(prefix[-1]) if self.ns else 0
        a, b = np.zeros(m, np.int32), np.zeros(m, np.int32)
        F, T, S, R, Q = (np.zeros((m, 3)) for _ in range(5))
        self._chk(self.lib.demsph_export_solid_pairs(self.h, _ptr(prefix, _IP), _ptr(a, _IP), _ptr(b, _IP), _ptr(F),
                                                     _ptr(T), _ptr(S), _ptr(R), _ptr(Q), C.c_longlong(m)), "ss")
        return {"prefix": prefix, "pointed": a, "pointing": b, "force": F, "torque": T, "sliding": S, "rolling": R,
                "torsion": Q}

    def bonds(self):
        m = self.counts().bonds
        a, b, on = np.zeros(m, np.int32), np.zeros(m, np.int32), np.zeros(m, np.int32)
        fn, tt = np.zeros(m), np.zeros(m)
        fs, tb, n, p = (np.zeros((m, 3)) for _ in range(4))
        self._chk(self.lib.demsph_export_bonds(self.h, _ptr(a, _IP), _ptr(b, _IP), _ptr(on, _IP), _ptr(fn), _ptr(tt),
                                               _ptr(fs), _ptr(tb), _ptr(n), _ptr(p), C.c_longlong(m)), "bonds")
        return {"pointed": a, "pointing": b, "isBonded": on, "normalForce": fn, "torsionTorque": tt,
                "shearForce": fs, "bendingTorque": tb, "contactNormal": n, "contactPoint": p}

    def sumw0(self):
        out = np.zeros(self.nf)
        self._chk(self.lib.demsph_export_fluid_sumw0(self.h, _ptr(out)), "sumw0")
        return out


def selftest_barrier(device=0, missing=1):
    """Runs the grid-barrier self-test (demsph_selftest_barrier); returns the
    device status bits (128 when the barrier wait ran out)."""
    lib = load_library()
    st = _I()
    rc = lib.demsph_selftest_barrier(_I(device), _I(missing), C.byref(st))
    if rc != DEMSPH_OK:
        raise DemSphError(rc, "demsph_selftest_barrier")
    return st.value


def estimate_bytes(scene, **opts):
    """Device memory demsph_create will allocate for the scene (an estimate)."""
    lib = load_library()
    o = _options(0, **opts)
    return int(lib.demsph_estimate_bytes(C.byref(scene), C.byref(o)))


class BatchInfo(C.Structure):
    _fields_ = [(k, C.c_longlong) for k in ("launches", "graph_builds", "members", "nodes")] + \
               [(k, _D) for k in ("capture_s", "instantiate_s", "launch_s")]


class Batch:
    """Many engines advanced in one CUDA graph launch (demsph_batch_*)."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = _P()
        rc = self.lib.demsph_batch_create(device, C.byref(h))
        if rc != DEMSPH_OK:
            raise DemSphError(rc, "demsph_batch_create")
        self.h = h

    def update(self, engines, first_steps, n_steps, dts, gaps):
        """Advances engines[k] by n_steps[k] steps from first_steps[k]; returns
        the per-engine status list (raises if the launch itself failed)."""
        k = len(engines)
        arr = (_P * k)(*[e.h.value for e in engines])
        st = (_I * k)()
        rc = self.lib.demsph_batch_update(self.h, arr, k, (_I * k)(*first_steps), (_I * k)(*n_steps),
                                          (_D * k)(*dts), (_I * k)(*gaps), st)
        if rc != DEMSPH_OK:
            raise DemSphError(rc, "demsph_batch_update: " + self.lib.demsph_batch_last_error(self.h).decode())
        return list(st)

    def info(self):
        i = BatchInfo()
        self.lib.demsph_batch_get_info(self.h, C.addressof(i))
        return {k: getattr(i, k) for k, _ in BatchInfo._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.demsph_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Many scenes on one GPU (demsph_server_*): submit, wait, fetch."""

    STATES = ("pending", "running", "done", "failed")

    def __init__(self, device=0, workers=0, chunk_steps=0, hbm_budget_bytes=0, autotune=False, graphs=0,
                 batch=False, batch_round_steps=0):
        """graphs: CUDA graphs for a scene's turns - 0 only while it is the
        only active scene, 1 always, -1 never.  batch: every active scene
        advances in one graph launch per round (demsph_batch_update), rounds
        of about batch_round_steps steps."""
        self.lib = load_library()
        cfg = ServerConfig(device, workers, chunk_steps, int(hbm_budget_bytes), 1 if autotune else 0, int(graphs),
                           1 if batch else 0, int(batch_round_steps))
        h = _P()
        rc = self.lib.demsph_server_create(C.byref(cfg), C.byref(h))
        if rc != DEMSPH_OK:
            raise DemSphError(rc, "demsph_server_create")
        self.h = h
        self._sizes = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.demsph_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, scene, n_steps, **opts):
        o = _options(0, **opts)
        rid = C.c_longlong()
        rc = self.lib.demsph_server_submit(self.h, C.byref(scene), C.byref(o), _I(n_steps), C.byref(rid))
        if rc != DEMSPH_OK:
            raise DemSphError(rc, "demsph_server_submit")
        self._sizes[rid.value] = (scene.n_fluid, scene.n_solid)
        return rid.value

    def wait(self, request_id=-1, timeout=-1.0):
        rc = self.lib.demsph_server_wait(self.h, C.c_longlong(request_id), _D(timeout))
        if rc != DEMSPH_OK:
            raise DemSphError(rc, f"request {request_id}")

    def fetch(self, request_id):
        nf, ns = self._sizes[request_id]
        out = {"fluid_pos": np.zeros((nf, 3)), "fluid_vel": np.zeros((nf, 3)), "fluid_drho": np.zeros(nf),
               "solid_pos": np.zeros((ns, 3)), "solid_vel": np.zeros((ns, 3)), "solid_angvel": np.zeros((ns, 3))}
        rc = self.lib.demsph_server_fetch(self.h, C.c_longlong(request_id),
                                          *[_ptr(out[k]) for k in ("fluid_pos", "fluid_vel", "fluid_drho",
                                                                    "solid_pos", "solid_vel", "solid_angvel")])
        if rc != DEMSPH_OK:
            raise DemSphError(rc, f"fetch {request_id}")
        return out

    def release(self, request_id):
        rc = self.lib.demsph_server_release(self.h, C.c_longlong(request_id))
        if rc != DEMSPH_OK:
            raise DemSphError(rc, f"release {request_id}")
        self._sizes.pop(request_id, None)

    def info(self, request_id):
        i = RequestInfo()
        rc = self.lib.demsph_server_request_info(self.h, C.c_longlong(request_id), C.byref(i))
        if rc != DEMSPH_OK:
            raise DemSphError(rc, f"info {request_id}")
        return {"state": self.STATES[i.state], "steps_done": i.steps_done, "reserved_bytes": i.reserved_bytes,
                "queued_s": i.queued_s, "run_s": i.run_s}

    def stats(self):
        st = ServerSummary()
        rc = self.lib.demsph_server_stats(self.h, C.byref(st))
        if rc != DEMSPH_OK:
            raise DemSphError(rc, "stats")
        return {k: getattr(st, k) for k, _ in ServerSummary._fields_}
