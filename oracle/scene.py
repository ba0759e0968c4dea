"""Scene assembly for the FP64 oracle, independent of the product library.

TEST INFRASTRUCTURE: used by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg and reference arm, never by the product.

:class:`OracleScene` takes the reference's setup calls (the method names of
class dataBase, core/dataBase.h:33-219, as a scenes.Recipe replays them) and
forms the arrays those calls leave in HostData (core/hostStructs.h), with the
reference's derived quantities restated in numpy:

* addFluid            core/dataBase.cpp:3-17      h, rho0, c, nu per particle
* addDummyParticleWall core/dataBase.cpp:19-31    radius = spacing, search radius 2.6 r, dummy flag
* addSolid            core/dataBase.cpp:33-53     search radius 1.1 r, 1 / (4/3 r^3 pi rho)
* addCluster          core/dataBase.cpp:84-118    one new cluster id per call
* addClump            core/dataBase.cpp:120-177   mass spread by (2r)^3, pebble v = v + w x (p - c),
                                                  inverse inertia (core/myMat.h:129-142)
* addInfiniteWall     core/dataBase.cpp:55-67
* set*ContactModel    core/dataBase.h:111-167     pair slot getCombinedIndex (core/hostStructs.h:369-384)
* defaults            core/dataBase.h:9-24, core/hostStructs.h (cluster / clump ids -1, res 1,
                      bond gamma 1 and k_n/k_s 2, orientation (1, 0, 0, 0))

Every power is taken with the C library's pow (``math.pow``) and every
expression keeps the reference's operand order, so the arrays equal the
reference's bit for bit (tests/test_oracle_scene.py compares them with the
product's scene builder array by array).  The scene is handed to the oracle
as a ``demsph_scene`` (include/demsph_gb300.h), mirrored here with ctypes.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

_D = C.c_double
_I = C.c_int
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)

PI = 3.1415926535897931  # pi() of core/myVec.h:10-13


class SceneStruct(C.Structure):
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


# (struct field, array name, columns, dtype): every array of the scene
ARRAYS = (
    ("fluid_position", "f_pos", 3, np.float64), ("fluid_velocity", "f_vel", 3, np.float64),
    ("fluid_acceleration", "f_acc", 3, np.float64), ("fluid_smoothing_length", "f_h", 1, np.float64),
    ("fluid_rho0", "f_rho0", 1, np.float64), ("fluid_drho", "f_drho", 1, np.float64),
    ("fluid_sound_speed", "f_c", 1, np.float64), ("fluid_nu", "f_nu", 1, np.float64),
    ("solid_position", "s_pos", 3, np.float64), ("solid_velocity", "s_vel", 3, np.float64),
    ("solid_acceleration", "s_acc", 3, np.float64), ("solid_normal", "s_normal", 3, np.float64),
    ("solid_torque", "s_torque", 3, np.float64), ("solid_angular_velocity", "s_w", 3, np.float64),
    ("solid_effective_radius", "s_eff", 1, np.float64), ("solid_radius", "s_r", 1, np.float64),
    ("solid_inverse_mass", "s_invm", 1, np.float64), ("solid_material", "s_mat", 1, np.int32),
    ("solid_cluster", "s_cluster", 1, np.int32), ("solid_clump", "s_clump", 1, np.int32),
    ("solid_is_dummy", "s_dummy", 1, np.int32),
    ("clump_centroid", "c_pos", 3, np.float64), ("clump_velocity", "c_vel", 3, np.float64),
    ("clump_acceleration", "c_acc", 3, np.float64), ("clump_angular_velocity", "c_w", 3, np.float64),
    ("clump_torque", "c_torque", 3, np.float64), ("clump_orientation", "c_q", 4, np.float64),
    ("clump_inverse_inertia", "c_invI", 6, np.float64), ("clump_inverse_mass", "c_invm", 1, np.float64),
    ("clump_pebble_start", "c_start", 1, np.int32), ("clump_pebble_end", "c_end", 1, np.int32),
    ("wall_point", "w_p", 3, np.float64), ("wall_normal", "w_n", 3, np.float64),
    ("wall_material", "w_mat", 1, np.int32),
)
COUNTS = {"f": "n_fluid", "s": "n_solid", "c": "n_clump", "w": "n_wall"}


def _pow3(a):
    """a**3 element by element through the C library's pow (the reference's pow(x, 3))."""
    return np.array([math.pow(float(x), 3) for x in np.asarray(a, dtype=np.float64).ravel()], dtype=np.float64)


def _v3(v):
    return np.array([float(v[0]), float(v[1]), float(v[2])], dtype=np.float64)


def _inverse6(I6):
    """inverse(symMatrix) of core/myMat.h:129-142 on (xx, yy, zz, xy, xz, yz)."""
    xx, yy, zz, xy, xz, yz = map(float, I6)
    det = 1. / (xx * (yy * zz - yz * yz) + xy * (yz * xz - xy * zz) + xz * (xy * yz - yy * xz))
    return (
        (yy * zz - yz * yz) * det,
        (xx * zz - xz * xz) * det,
        (xx * yy - xy * xy) * det,
        -(xy * zz - xz * yz) * det,
        (xy * yz - xz * yy) * det,
        -(xx * yz - xz * xy) * det,
    )


class OracleScene:
    """The reference's dataBase setup calls, forming the arrays of HostData."""

    def __init__(self, n_material=10):
        # dataBase() defaults (core/dataBase.h:9-24)
        self.domain_origin = (0.0, 0.0, 0.0)
        self.domain_size = (1.0, 1.0, 1.0)
        self.gravity = (0.0, 0.0, -9.81)
        self.time_step = 1.0
        self.maximum_time = 1.0
        self.num_frames = 1
        self.fluid_integrate_gap = 1
        self.n_material = int(n_material)
        nslot = n_material * (n_material + 1) // 2
        # HostSolidContactModel(n) defaults (core/hostStructs.h:291-349)
        self.hertzian = np.zeros((nslot, 8))
        self.hertzian[:, 2] = 1.0                                 # res
        self.linear = np.zeros((nslot, 11))
        self.bonded = np.zeros((nslot, 6))
        self.bonded[:, 0] = 1.0                                   # gamma
        self.bonded[:, 2] = 2.0                                   # k_n / k_s
        self._parts = {k: [] for k in ("f", "s", "c", "w")}
        self._n = {k: 0 for k in ("f", "s", "c", "w")}
        self._max_cluster = None
        self._struct = None

    # ---- setters (core/dataBase.h:38-167) ----
    def setDomain(self, origin, size):
        self.domain_origin, self.domain_size = tuple(map(float, origin)), tuple(map(float, size))

    def setGravity(self, g):
        self.gravity = tuple(map(float, g))

    def setSimulationParameterTimeStep(self, dt):
        if dt > 0.:
            self.time_step = float(dt)

    def setSimulationParameterMaximumTime(self, t):
        if t > 0.:
            self.maximum_time = float(t)

    def setSimulationParameterNumFrames(self, n):
        if n >= 1:
            self.num_frames = int(n)

    def setFluidIntegrateGap(self, gap):
        if gap >= 1:
            self.fluid_integrate_gap = int(gap)

    def _slot(self, mi, mj):
        if mi >= self.n_material or mj >= self.n_material:
            return -1
        i, j = (mi, mj) if mi <= mj else (mj, mi)
        return (i * (2 * self.n_material - i + 1)) // 2 + j - i

    def setHertzianContactModel(self, mi, mj, *v):
        c = self._slot(mi, mj)
        if c >= 0:
            self.hertzian[c] = v

    def setLinearContactModel(self, mi, mj, *v):
        c = self._slot(mi, mj)
        if c >= 0:
            self.linear[c] = v

    def setBondedContactModel(self, mi, mj, E, k_n_k_s, gamma, sigma_s, Cc, mu):
        c = self._slot(mi, mj)
        if c >= 0:
            # slot layout of demsph_scene.bonded: gamma E k_n_k_s sigma_s C mu
            self.bonded[c] = (gamma, E, k_n_k_s, sigma_s, Cc, mu)

    # ---- particles (core/dataBase.cpp:3-177) ----
    def _add(self, kind, **arrays):
        n = len(next(iter(arrays.values())))
        self._parts[kind].append(arrays)
        self._n[kind] += n
        self._struct = None

    def _solids(self, p, v, eff, r, invm, mat, cluster, clump, dummy, w=None):
        n = len(p)
        self._add("s", s_pos=p, s_vel=v, s_acc=np.zeros((n, 3)), s_normal=np.zeros((n, 3)),
                  s_torque=np.zeros((n, 3)), s_w=np.zeros((n, 3)) if w is None else w, s_eff=eff, s_r=r,
                  s_invm=invm, s_mat=np.full(n, mat, np.int32), s_cluster=np.asarray(cluster, np.int32),
                  s_clump=np.asarray(clump, np.int32), s_dummy=np.full(n, dummy, np.int32))
        c = np.asarray(cluster).max() if n else -1
        self._max_cluster = c if self._max_cluster is None else max(self._max_cluster, c)

    def addFluid(self, p, velocity, smoothLength, density, soundSpeed, kinematicViscosity):
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        n = len(p)
        self._add("f", f_pos=p.copy(), f_vel=np.tile(_v3(velocity), (n, 1)), f_acc=np.zeros((n, 3)),
                  f_h=np.full(n, float(smoothLength)), f_rho0=np.full(n, float(density)), f_drho=np.zeros(n),
                  f_c=np.full(n, float(soundSpeed)), f_nu=np.full(n, float(kinematicViscosity)))

    def addDummyParticleWall(self, p, radius):
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        n = len(p)
        self._solids(p.copy(), np.zeros((n, 3)), np.full(n, 2.6 * float(radius)), np.full(n, float(radius)),
                     np.zeros(n), 0, np.full(n, -1), np.full(n, -1), 1)

    def _sphere_invm(self, r, rho):
        """1 / (4/3 pow(r, 3) pi rho) where rho > 0, else 0."""
        r = np.asarray(r, dtype=np.float64).ravel()
        rho = np.asarray(rho, dtype=np.float64).ravel()
        out = np.zeros(len(r))
        live = rho > 0
        out[live] = 1. / ((4. / 3.) * _pow3(r[live]) * PI * rho[live])
        return out

    def addSolid(self, p, velocity, radius, density, materialID):
        if materialID >= self.n_material:
            return
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        n = len(p)
        r = np.full(n, float(radius))
        self._solids(p.copy(), np.tile(_v3(velocity), (n, 1)), 1.1 * r, r, self._sphere_invm(r, np.full(n, density)),
                     materialID, np.full(n, -1), np.full(n, -1), 0)

    def addInfiniteWall(self, p, normal, materialID):
        self._add("w", w_p=_v3(p)[None, :], w_n=_v3(normal)[None, :], w_mat=np.array([materialID], np.int32))

    def addCluster(self, p, radius, density, velocity, materialID):
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        r = np.asarray(radius, dtype=np.float64).ravel()
        rho = np.asarray(density, dtype=np.float64).ravel()
        if len(r) != len(p) or len(rho) != len(p) or materialID >= self.n_material:
            return
        cid = 0 if self._n["s"] == 0 else int(self._max_cluster) + 1
        n = len(p)
        self._solids(p.copy(), np.tile(_v3(velocity), (n, 1)), 1.1 * r, r.copy(), self._sphere_invm(r, rho),
                     materialID, np.full(n, cid), np.full(n, -1), 0)

    def addClump(self, p, radius, centroidPosition, velocity, angularVelocity, mass, inertia6, materialID):
        p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
        r = np.asarray(radius, dtype=np.float64).ravel()
        if len(r) != len(p) or materialID >= self.n_material:
            return
        cid = self._n["c"]
        c, v, w = _v3(centroidPosition), _v3(velocity), _v3(angularVelocity)
        start = self._n["s"]
        volume = 0.0
        for x in r:
            volume += math.pow(2. * float(x), 3)
        dens = mass / volume if volume > 0. else 0.
        n = len(p)
        pv = np.empty((n, 3))
        invm = np.zeros(n)
        for k in range(n):
            d = p[k] - c
            # v + cross(w, p - c), core/myVec.h:73-79
            pv[k] = (v[0] + (w[1] * d[2] - w[2] * d[1]), v[1] + (w[2] * d[0] - w[0] * d[2]),
                     v[2] + (w[0] * d[1] - w[1] * d[0]))
            if dens > 0. and r[k] > 0:
                invm[k] = 1. / (math.pow(2. * float(r[k]), 3) * dens)
        self._solids(p.copy(), pv, 1.1 * r, r.copy(), invm, materialID, np.full(n, -1), np.full(n, cid), 0,
                     w=np.tile(w, (n, 1)))
        self._add("c", c_pos=c[None, :], c_vel=v[None, :], c_acc=np.zeros((1, 3)), c_w=w[None, :],
                  c_torque=np.zeros((1, 3)), c_q=np.array([[1.0, 0.0, 0.0, 0.0]]),
                  c_invI=np.array([_inverse6(inertia6)]), c_invm=np.array([1. / mass if mass > 0. else 0.]),
                  c_start=np.array([start], np.int32), c_end=np.array([self._n["s"]], np.int32))

    # ---- the C view ----
    def arrays(self):
        """{array name: contiguous numpy array} of the whole scene."""
        out = {}
        for field, name, cols, dt in ARRAYS:
            kind = name.split("_")[0]
            parts = [a[name] for a in self._parts[kind]]
            n = self._n[kind]
            if parts:
                a = np.concatenate([np.asarray(x, dtype=dt).reshape(-1, cols) if cols > 1 else
                                    np.asarray(x, dtype=dt).ravel() for x in parts])
            else:
                a = np.zeros((0, cols) if cols > 1 else 0, dtype=dt)
            assert len(a) == n, (name, len(a), n)
            out[name] = np.ascontiguousarray(a)
        return out

    def scene(self):
        """The scene as a ``demsph_scene`` (valid while this object lives)."""
        s = SceneStruct()
        s.domain_origin = (_D * 3)(*self.domain_origin)
        s.domain_size = (_D * 3)(*self.domain_size)
        s.gravity = (_D * 3)(*self.gravity)
        s.time_step = self.time_step
        s.fluid_integrate_gap = self.fluid_integrate_gap
        s.maximum_time = self.maximum_time
        s.num_frames = self.num_frames
        self._arr = self.arrays()
        for kind, cnt in COUNTS.items():
            setattr(s, cnt, self._n[kind])
        for field, name, cols, dt in ARRAYS:
            a = self._arr[name]
            setattr(s, field, a.ctypes.data_as(_IP if dt == np.int32 else _DP) if len(a) else None)
        self._tables = [np.ascontiguousarray(t.ravel()) for t in (self.hertzian, self.linear, self.bonded)]
        s.n_material = self.n_material
        s.hertzian, s.linear, s.bonded = (t.ctypes.data_as(_DP) for t in self._tables)
        s._owner = self  # keeps the arrays alive
        return s


def build_scene(recipe, n_material=10):
    """Replays a scenes.Recipe on an OracleScene; returns (assembly, scene)."""
    o = OracleScene(n_material)
    recipe.apply(o)
    return o, o.scene()


def scene_arrays(scene):
    """Every array of a ``demsph_scene`` (either ctypes mirror) as numpy, plus
    the scalars and material tables: {name: array}.  Used to compare scenes."""
    out = {}
    n = {"f": scene.n_fluid, "s": scene.n_solid, "c": scene.n_clump, "w": scene.n_wall}
    for field, name, cols, dt in ARRAYS:
        cnt = n[name.split("_")[0]]
        ptr = getattr(scene, field)
        if cnt and ptr:
            a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_int32 if dt == np.int32 else C.c_double)),
                                      shape=(cnt * cols,))
            out[field] = np.array(a, dtype=dt)
        else:
            out[field] = np.zeros(cnt * cols, dtype=dt)
    nslot = scene.n_material * (scene.n_material + 1) // 2
    for field, w in (("hertzian", 8), ("linear", 11), ("bonded", 6)):
        out[field] = np.array(np.ctypeslib.as_array(C.cast(getattr(scene, field), C.POINTER(C.c_double)),
                                                    shape=(nslot * w,)))
    out["scalars"] = np.array(list(scene.domain_origin) + list(scene.domain_size) + list(scene.gravity) +
                              [scene.time_step, scene.fluid_integrate_gap, scene.maximum_time, scene.num_frames,
                               scene.n_fluid, scene.n_solid, scene.n_clump, scene.n_wall, scene.n_material],
                              dtype=np.float64)
    return out
