"""Seeded synthetic scenes, written as recipes of the reference's setup calls.

A scene is a :class:`Recipe`: an ordered list of the calls a case driver makes
on the reference's ``dataBase`` API (core/dataBase.h:33-219), e.g. ``addFluid``,
``addDummyParticleWall``, ``addCluster``, ``setHertzianContactModel``.  The same
recipe can be replayed on

* this package's scene builder (the C-ABI mirror of that API),
* the FP64 oracle (which takes the builder's arrays), and
* the reference itself compiled for the CPU (``oracle/_ref``),

so all three see bit-identical inputs.

Workloads (the reference publishes no data; every input is generated here from
a seed with the sizes and value distributions below):

* ``dam_break``        - WCSPH dam break: water column on a jittered cubic
  lattice in a tank of three layers of dummy wall particles (the layout of
  driver/cases/damBreak.cpp).  The 48k-fluid case is tank 1.6x0.4x0.6 m, column
  0.4x0.4x0.3 m, dx = 0.01 m, rho0 = 1000, c0 = 20, h = 1.3 dx, dt = 0.2 h / c0.
* ``granular_settle``  - dry Hertz-Mindlin settle of lognormal spheres plus
  4-pebble clumps with uniformly random orientations, on a floor wall.
* ``coupled_dam_break`` - dam break striking bonded cubes of 8^3 spheres.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# Call names follow the reference's dataBase API one for one.
CALLS = (
    "setDomain", "setGravity", "setSimulationParameterTimeStep", "setSimulationParameterMaximumTime",
    "setSimulationParameterNumFrames", "setFluidIntegrateGap", "setHertzianContactModel",
    "setLinearContactModel", "setBondedContactModel", "addFluid", "addDummyParticleWall", "addSolid",
    "addInfiniteWall", "addCluster", "addClump",
)


@dataclass
class Recipe:
    """An ordered list of reference setup calls plus bookkeeping."""

    name: str
    calls: list = field(default_factory=list)
    meta: dict = field(default_factory=dict)

    def _add(self, fn, *args):
        assert fn in CALLS, fn
        self.calls.append((fn, args))
        return self

    # --- the reference's setters (core/dataBase.h) ---
    def setDomain(self, origin, size):
        return self._add("setDomain", tuple(map(float, origin)), tuple(map(float, size)))

    def setGravity(self, g):
        return self._add("setGravity", tuple(map(float, g)))

    def setSimulationParameterTimeStep(self, dt):
        return self._add("setSimulationParameterTimeStep", float(dt))

    def setSimulationParameterMaximumTime(self, t):
        return self._add("setSimulationParameterMaximumTime", float(t))

    def setSimulationParameterNumFrames(self, n):
        return self._add("setSimulationParameterNumFrames", int(n))

    def setFluidIntegrateGap(self, gap):
        return self._add("setFluidIntegrateGap", int(gap))

    def setHertzianContactModel(self, mi, mj, E, G, res, k_r_k_s, k_t_k_s, mu_s, mu_r, mu_t):
        return self._add("setHertzianContactModel", int(mi), int(mj), *map(float, (E, G, res, k_r_k_s, k_t_k_s,
                                                                                   mu_s, mu_r, mu_t)))

    def setLinearContactModel(self, mi, mj, k_n, k_s, k_r, k_t, d_n, d_s, d_r, d_t, mu_s, mu_r, mu_t):
        return self._add("setLinearContactModel", int(mi), int(mj),
                         *map(float, (k_n, k_s, k_r, k_t, d_n, d_s, d_r, d_t, mu_s, mu_r, mu_t)))

    def setBondedContactModel(self, mi, mj, E, k_n_k_s, gamma, sigma_s, C, mu):
        return self._add("setBondedContactModel", int(mi), int(mj), *map(float, (E, k_n_k_s, gamma, sigma_s, C, mu)))

    def addFluid(self, p, velocity, smoothLength, density, soundSpeed, kinematicViscosity):
        return self._add("addFluid", _pts(p), tuple(map(float, velocity)), float(smoothLength), float(density),
                         float(soundSpeed), float(kinematicViscosity))

    def addDummyParticleWall(self, p, spacing):
        return self._add("addDummyParticleWall", _pts(p), float(spacing))

    def addSolid(self, p, velocity, radius, density, materialID):
        return self._add("addSolid", _pts(p), tuple(map(float, velocity)), float(radius), float(density),
                         int(materialID))

    def addInfiniteWall(self, p, normal, materialID):
        return self._add("addInfiniteWall", tuple(map(float, p)), tuple(map(float, normal)), int(materialID))

    def addCluster(self, p, radius, density, velocity, materialID):
        p = _pts(p)
        return self._add("addCluster", p, np.ascontiguousarray(radius, dtype=np.float64),
                         np.ascontiguousarray(density, dtype=np.float64), tuple(map(float, velocity)),
                         int(materialID))

    def addClump(self, p, radius, centroidPosition, velocity, angularVelocity, mass, inertia6, materialID):
        return self._add("addClump", _pts(p), np.ascontiguousarray(radius, dtype=np.float64),
                         tuple(map(float, centroidPosition)), tuple(map(float, velocity)),
                         tuple(map(float, angularVelocity)), float(mass), tuple(map(float, inertia6)),
                         int(materialID))

    def apply(self, target):
        """Replays every call on ``target`` (anything with the same method names)."""
        for fn, args in self.calls:
            getattr(target, fn)(*args)
        return target

    # --- counts ---
    def counts(self):
        nf = sum(len(a[0]) for fn, a in self.calls if fn == "addFluid")
        nw = sum(len(a[0]) for fn, a in self.calls if fn == "addDummyParticleWall")
        ns = sum(len(a[0]) for fn, a in self.calls if fn in ("addSolid", "addCluster", "addClump"))
        nc = sum(1 for fn, a in self.calls if fn == "addClump")
        return {"fluid": nf, "dummy": nw, "solid": ns, "clump": nc}


def _pts(p):
    a = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)
    return a


def regular_packed_points(origin, size, spacing):
    """Same lattice as the reference's getRegularPackedPoints (core/generatePoints.h:4-33):
    cell-centred points, x outermost, z innermost."""
    n = [int((size[k] + 1.0e-10) / spacing) for k in range(3)]
    if min(n) == 0:
        return np.array([[origin[k] + 0.5 * size[k] for k in range(3)]], dtype=np.float64)
    d = [size[k] / float(n[k]) for k in range(3)]
    ax = [origin[k] + d[k] * (np.arange(1, n[k] + 1, dtype=np.float64) - 0.5) for k in range(3)]
    X, Y, Z = np.meshgrid(ax[0], ax[1], ax[2], indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)


def _tank_walls(dx, tank, layers=3):
    """Dummy wall particles: the lattice of the tank grown by ``layers`` spacings on
    every side, minus the tank's inside, open at the top (driver/cases/damBreak.cpp:23-29)."""
    m = layers * dx
    sp0 = regular_packed_points((-m, -m, -m), (tank[0] + 2 * m, tank[1] + 2 * m, tank[2] + 2 * m), dx)
    keep = (sp0[:, 0] < 0) | (sp0[:, 1] < 0) | (sp0[:, 2] < 0) | (sp0[:, 0] > tank[0]) | (sp0[:, 1] > tank[1])
    return sp0[keep]


def dam_break(dx=0.01, tank=(1.6, 0.4, 0.6), column=(0.4, 0.4, 0.3), rho0=1000.0, c0=20.0, nu=1.0e-6,
              cfl=0.2, steps=2000, jitter=0.01, seed=0, name=None):
    """WCSPH dam break (the 48k-fluid plain case at the defaults)."""
    rng = np.random.default_rng(seed)
    h = 1.3 * dx
    m = 3 * dx
    r = Recipe(name or f"dam_break_dx{dx:g}")
    r.setDomain((-m, -m, -m), (tank[0] + 2 * m, tank[1] + 2 * m, tank[2] + 2 * m))
    fp = regular_packed_points((0.0, 0.0, 0.0), column, dx)
    fp = fp + rng.uniform(-jitter * dx, jitter * dx, size=fp.shape)
    r.addFluid(fp, (0, 0, 0), h, rho0, c0, nu)
    r.addDummyParticleWall(_tank_walls(dx, tank), 0.5 * dx)
    dt = cfl * h / c0
    r.setSimulationParameterTimeStep(dt)
    r.setFluidIntegrateGap(1)
    r.setSimulationParameterMaximumTime((steps - 0.5) * dt)
    r.setSimulationParameterNumFrames(1)
    r.meta.update(dt=dt, steps=steps, dx=dx, h=h, gap=1)
    return r


def hertz_from_E_nu(E, nu):
    """Effective moduli for two identical spheres: E* = E / (2 (1 - nu^2)), G* = E / (4 (2 - nu)(1 + nu))."""
    return E / (2.0 * (1.0 - nu * nu)), E / (4.0 * (2.0 - nu) * (1.0 + nu))


def _random_rotations(rng, n):
    """Rotation matrices from uniformly distributed unit quaternions (Shoemake's method)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)], axis=1)
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z); R[:, 0, 1] = 2 * (x * y - z * w); R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w); R[:, 1, 1] = 1 - 2 * (x * x + z * z); R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w); R[:, 2, 1] = 2 * (y * z + x * w); R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def clump_inertia(pebbles, radii, centroid, mass):
    """Inertia tensor (xx, yy, zz, xy, xz, yz) of a clump: point masses at the pebbles
    (mass shared by pebble volume) plus each pebble's own solid-sphere inertia."""
    v = radii ** 3
    mp = mass * v / v.sum()
    d = pebbles - centroid
    I = np.zeros((3, 3))
    for k in range(len(radii)):
        I += mp[k] * (np.dot(d[k], d[k]) * np.eye(3) - np.outer(d[k], d[k]))
        I += 0.4 * mp[k] * radii[k] ** 2 * np.eye(3)
    return (I[0, 0], I[1, 1], I[2, 2], I[0, 1], I[0, 2], I[1, 2])


def granular_settle(n_spheres=200_000, n_clumps=5_000, box=(0.1, 0.1), spacing=2.5e-3, r_median=1.0e-3,
                    sigma=0.2, r_clip=(0.6e-3, 1.2e-3), E=1.0e8, poisson=0.3, res=0.5, mu_s=0.4, density=2500.0,
                    steps=20_000, jitter=0.05, seed=1, z0=None, velocity=(0, 0, 0), name=None,
                    side_walls="infinite"):
    """Dry Hertz-Mindlin settle: lognormal spheres on a jittered lattice plus 4-pebble
    clumps (tetrahedral, uniformly random orientation) above them, on a floor wall.

    side_walls: "infinite" adds four infinite walls after the floor; "spheres"
    lines the four sides with fixed spheres (density 0, radius 1 mm, touching
    on a square lattice) instead.  The reference's wall loop stops at the first
    wall a particle does not touch (core/integrate.cu:540), so infinite side
    walls after the floor hold only particles that touch the floor: a settling
    column leaks through them; walls of fixed spheres contain it under the
    reference's own rules."""
    rng = np.random.default_rng(seed)
    r = Recipe(name or f"granular_settle_{n_spheres}_{n_clumps}")
    nx, ny = int(round(box[0] / spacing)), int(round(box[1] / spacing))
    layers = int(math.ceil(n_spheres / (nx * ny)))
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(layers), indexing="ij")
    zoff = 0.5 * spacing if z0 is None else z0
    lat = np.stack([(ii.ravel(order="F") + 0.5) * spacing, (jj.ravel(order="F") + 0.5) * spacing,
                    kk.ravel(order="F") * spacing + zoff], axis=1)[:n_spheres]
    radii = np.clip(np.exp(np.log(r_median) + sigma * rng.standard_normal(n_spheres)), *r_clip)
    lat = lat + rng.uniform(-jitter, jitter, size=lat.shape) * (spacing - 2 * radii[:, None]).clip(0) * 0.5
    top = layers * spacing
    # clumps: 4 pebbles of radius r_p at the vertices of a tetrahedron of circumradius a
    r_p, a = 1.0e-3, 0.8e-3
    csp = 2 * (a + r_p) * 1.05
    cnx, cny = max(1, int(box[0] / csp)), max(1, int(box[1] / csp))
    clayers = int(math.ceil(n_clumps / (cnx * cny))) if n_clumps else 0
    height = top + clayers * csp
    m = 3 * spacing
    r.setDomain((-m, -m, -m), (box[0] + 2 * m, box[1] + 2 * m, height + 2 * m))
    Es, Gs = hertz_from_E_nu(E, poisson)
    r.setHertzianContactModel(0, 0, Es, Gs, res, 0.0, 0.0, mu_s, 0.0, 0.0)
    r.setHertzianContactModel(0, 1, Es, Gs, res, 0.0, 0.0, mu_s, 0.0, 0.0)
    r.setHertzianContactModel(1, 1, Es, Gs, res, 0.0, 0.0, mu_s, 0.0, 0.0)
    # One addCluster call per sphere would give every sphere its own cluster id; a single
    # call with zero bond modulus gives unbonded spheres with individual radii.
    r.addCluster(lat, radii, np.full(n_spheres, density), velocity, 0)
    tet = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=np.float64) / math.sqrt(3.0) * a
    Rs = _random_rotations(rng, n_clumps)
    vol = 0.0
    for k in range(n_clumps):
        cz, rem = divmod(k, cnx * cny)
        cy, cx = divmod(rem, cnx)
        c = np.array([(cx + 0.5) * csp, (cy + 0.5) * csp, top + (cz + 0.5) * csp])
        peb = c + tet @ Rs[k].T
        pr = np.full(4, r_p)
        mass = density * 4.0 / 3.0 * math.pi * r_p ** 3 * 4 * 0.8  # overlapping pebbles: ~80% of 4 spheres
        r.addClump(peb, pr, c, (0, 0, 0), (0, 0, 0), mass, clump_inertia(peb, pr, c, mass), 1)
    r.addInfiniteWall((0, 0, 0), (0, 0, 1), 0)
    if side_walls == "infinite":
        for p, n in (((0, 0, 0), (1, 0, 0)), ((box[0], 0, 0), (-1, 0, 0)), ((0, 0, 0), (0, 1, 0)),
                     ((0, box[1], 0), (0, -1, 0))):
            r.addInfiniteWall(p, n, 0)
    else:
        rw = 1.0e-3
        zs = np.arange(rw, height + rw, 2 * rw)
        ys = np.arange(-rw, box[1] + 2 * rw, 2 * rw)
        xs = np.arange(rw, box[0], 2 * rw)
        Y, Z = np.meshgrid(ys, zs, indexing="ij")
        X, Z2 = np.meshgrid(xs, zs, indexing="ij")
        walls = [np.stack([np.full(Y.size, -rw), Y.ravel(), Z.ravel()], 1),
                 np.stack([np.full(Y.size, box[0] + rw), Y.ravel(), Z.ravel()], 1),
                 np.stack([X.ravel(), np.full(X.size, -rw), Z2.ravel()], 1),
                 np.stack([X.ravel(), np.full(X.size, box[1] + rw), Z2.ravel()], 1)]
        r.addSolid(np.concatenate(walls), (0, 0, 0), rw, 0.0, 0)
    rmin = float(radii.min())
    G = E / (2 * (1 + poisson))
    t_r = math.pi * rmin * math.sqrt(density / G) / (0.1631 * poisson + 0.8766)
    dt = 0.1 * t_r
    r.setSimulationParameterTimeStep(dt)
    r.setSimulationParameterMaximumTime((steps - 0.5) * dt)
    r.setSimulationParameterNumFrames(1)
    r.meta.update(dt=dt, steps=steps, gap=1, rayleigh=t_r)
    return r


def coupled_dam_break(dx=0.004, tank=(1.6, 0.4, 0.6), column=(0.4, 0.4, 0.4), n_cubes=64, cube_n=8,
                      sphere_r=2.0e-3, kn=1.0e6, ks=4.0e5, sigma_range=(0.5e6, 2.0e6), n_strength_levels=9,
                      E=1.0e8, poisson=0.3, res=0.5, mu_s=0.4, density=2500.0, rho0=1000.0, c0=20.0, nu=1.0e-6,
                      cfl=0.2, steps=5000, jitter=0.01, seed=2, name=None):
    """Coupled DEM-SPH: the dam break of :func:`dam_break` at ``dx`` striking
    ``n_cubes`` bonded cubes of ``cube_n``^3 spheres placed uniformly on the floor.

    Bond tensile strength is keyed by material pair in the reference
    (core/hostStructs.h:334-349, 10 materials), so the uniform per-bond draw is
    made per cube from ``n_strength_levels`` equally spaced levels (materials 1..9)."""
    rng = np.random.default_rng(seed)
    h = 1.3 * dx
    m = 3 * dx
    r = Recipe(name or f"coupled_dam_break_dx{dx:g}_{n_cubes}")
    r.setDomain((-m, -m, -m), (tank[0] + 2 * m, tank[1] + 2 * m, tank[2] + 2 * m))
    fp = regular_packed_points((0.0, 0.0, 0.0), column, dx)
    fp = fp + rng.uniform(-jitter * dx, jitter * dx, size=fp.shape)
    r.addFluid(fp, (0, 0, 0), h, rho0, c0, nu)
    r.addDummyParticleWall(_tank_walls(dx, tank), 0.5 * dx)
    Es, Gs = hertz_from_E_nu(E, poisson)
    bondE = 2.0 * kn / (math.pi * sphere_r)      # k_n = E * pi r^2 / (2 r) for gamma = 1
    levels = np.linspace(sigma_range[0], sigma_range[1], n_strength_levels)
    for a in range(10):
        for b in range(a, 10):
            r.setHertzianContactModel(a, b, Es, Gs, res, 0.0, 0.0, mu_s, 0.0, 0.0)
    for k, s in enumerate(levels):
        r.setBondedContactModel(k + 1, k + 1, bondE, kn / ks, 1.0, s, 0.0, 0.0)
    side = cube_n * 2 * sphere_r
    x0 = column[0] + 0.05
    placed = []
    while len(placed) < n_cubes:
        c = (rng.uniform(x0, tank[0] - side), rng.uniform(0.0, tank[1] - side))
        if all(abs(c[0] - q[0]) >= side * 1.05 or abs(c[1] - q[1]) >= side * 1.05 for q in placed):
            placed.append(c)
    for k, (cx, cy) in enumerate(placed):
        pts = regular_packed_points((cx, cy, 0.0), (side, side, side), 2 * sphere_r)
        mat = 1 + int(rng.integers(0, n_strength_levels))
        r.addCluster(pts, np.full(len(pts), sphere_r), np.full(len(pts), density), (0, 0, 0), mat)
    r.addInfiniteWall((0, 0, 0), (0, 0, 1), 0)
    mass = density * 4.0 / 3.0 * math.pi * sphere_r ** 3
    dt = 0.2 * math.sqrt(mass / kn)
    dt_f = cfl * h / c0
    gap = max(1, int(dt_f / dt))
    r.setSimulationParameterTimeStep(dt)
    r.setFluidIntegrateGap(gap)
    r.setSimulationParameterMaximumTime((steps - 0.5) * dt)
    r.setSimulationParameterNumFrames(1)
    r.meta.update(dt=dt, steps=steps, gap=gap, dx=dx, h=h)
    return r


# ---------------------------------------------------------------------------
# Many scenes: the batched mix and the serving stream.
# ---------------------------------------------------------------------------

def sized_dam_break(n_fluid, column_height=0.3, steps=1000, seed=0):
    """:func:`dam_break` with dx chosen so that a 0.4 x 0.4 x column_height
    column holds about n_fluid particles."""
    dx = (0.16 * column_height / n_fluid) ** (1.0 / 3.0)
    return dam_break(dx=dx, column=(0.4, 0.4, column_height), steps=steps, seed=seed,
                     name=f"dam_break_{n_fluid}")


def sized_coupled(n_fluid, column_height=0.4, steps=1000, seed=0):
    """:func:`coupled_dam_break` with dx for about n_fluid fluid particles and
    the cube count scaled from 64 cubes per million fluid particles (at least one)."""
    dx = (0.16 * column_height / n_fluid) ** (1.0 / 3.0)
    cubes = max(1, int(round(64 * n_fluid / 1.0e6)))
    return coupled_dam_break(dx=dx, column=(0.4, 0.4, column_height), n_cubes=cubes, steps=steps, seed=seed,
                             name=f"coupled_{n_fluid}_{cubes}")


def sized_granular(n_particles, steps=1000, seed=0):
    """:func:`granular_settle` with about n_particles spheres and pebbles (one
    four-pebble clump per 40 spheres)."""
    n_clumps = max(1, n_particles // 44)
    return granular_settle(n_spheres=n_particles - 4 * n_clumps, n_clumps=n_clumps, steps=steps, seed=seed,
                           name=f"granular_{n_particles}", side_walls="spheres")


def batch_mix(n_scenes=256, n_range=(2000, 60000), sph_fraction=0.6, height_range=(0.2, 0.5), steps=1000,
              seed=7):
    """The batched workload: independent scenes, sph_fraction of them SPH dam
    breaks and the rest coupled dam breaks, fluid counts log-uniform in
    n_range, column heights uniform in height_range.  Returns recipes."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        hgt = float(rng.uniform(*height_range))
        if rng.random() < sph_fraction:
            out.append(sized_dam_break(n, hgt, steps, seed=seed * 1000 + k))
        else:
            out.append(sized_coupled(n, hgt, steps, seed=seed * 1000 + k))
    return out


def serving_stream(rate=20.0, duration=300.0, n_range=(5000, 500000), step_range=(200, 5000), seed=11):
    """The serving workload: (arrival time s, kind, particle count, steps, seed)
    tuples of a Poisson process of `rate` requests per second over `duration`
    seconds; kinds SPH, DEM and coupled in equal shares, sizes log-uniform in
    n_range, step counts uniform in step_range.  Scenes are built with
    :func:`make_request` when they arrive."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        kind = ("sph", "dem", "coupled")[int(rng.integers(0, 3))]
        out.append((t, kind, n, int(rng.integers(step_range[0], step_range[1] + 1)), int(rng.integers(1 << 30))))


def make_request(kind, n, steps, seed):
    if kind == "sph":
        return sized_dam_break(n, 0.3, steps, seed)
    if kind == "dem":
        return sized_granular(n, steps, seed)
    return sized_coupled(n, 0.4, steps, seed)


# ---------------------------------------------------------------------------
# Small scenes for parity tests and the smoke run (seconds on one CPU core).
# ---------------------------------------------------------------------------

def tiny_dam_break(seed=0):
    """180 fluid particles in a 3-layer dummy-wall tank."""
    return dam_break(dx=0.02, tank=(0.3, 0.12, 0.2), column=(0.12, 0.12, 0.1), steps=20, seed=seed,
                     name="tiny_dam_break")


def tiny_granular(seed=3, with_probe_fluid=True):
    """~300 lognormal spheres and 8 tetrahedral clumps settling on a floor
    wall with four side walls (the reference returns from its wall loop at
    the first wall not touched, core/integrate.cu:540).

    The reference's solver dereferences the largest fluid smoothing length
    when it computes wall normals (core/dataBase.cpp:359) and so needs at
    least one fluid particle; with ``with_probe_fluid`` one is placed far from
    the grains, where it only falls."""
    # 2.3 mm spacing with radii up to 1.2 mm: some neighbours start overlapping,
    # and the bottom layer starts pressed into the floor, so contacts are live at once
    r = granular_settle(n_spheres=288, n_clumps=8, box=(0.02, 0.02), spacing=2.3e-3, steps=50, seed=seed,
                        z0=1.0e-3, velocity=(0.05, -0.03, -0.2), name="tiny_granular")
    if with_probe_fluid:
        calls = r.calls
        idx = next(k for k, (fn, _) in enumerate(calls) if fn == "setDomain")
        o, s = calls[idx][1]
        p = np.array([[o[0] + s[0] - 1e-3, o[1] + s[1] - 1e-3, o[2] + s[2] - 1e-3]])
        r.addFluid(p, (0, 0, 0), 5.0e-4, 1000.0, 20.0, 1.0e-6)
    return r


def tiny_linear(seed=8):
    """:func:`tiny_granular` with the linear spring-dashpot law
    (setLinearContactModel, core/SPHKernelDEMContactModel.h:214-268) between
    material 0 (spheres and walls) and both materials, with rolling and
    torsion springs and viscous damping; the clumps (material 1) keep the
    Hertz-Mindlin law among themselves.  The reference picks the linear law
    for a material pair whose k_n is set (core/integrate.cu:463-484, and
    :559-580 for walls), so both laws run in one scene."""
    r = tiny_granular(seed=seed)
    r.name = "tiny_linear"
    for mi, mj in ((0, 0), (0, 1)):
        r.setLinearContactModel(mi, mj, 2.0e3, 1.0e3, 4.0e2, 3.0e2, 0.3, 0.2, 0.1, 0.1, 0.4, 0.05, 0.05)
    return r


def tiny_tumbling(seed=9, n_clumps=12, n_spheres=30, steps=50):
    """Spinning clumps of four pebbles in an irregular shape (three in a row
    and one off the line: an anisotropic inertia tensor), with random
    orientations and spins, dropped so that their lowest pebble starts just
    pressed into the floor, among loose spheres, with side walls; rolling and
    torsion springs on.  The orientation of a spinning anisotropic clump
    changes its world inverse inertia (core/myMat.h:102-127), so this scene
    tells the reference's never-integrated orientation (core/integrate.cu:919)
    from DEMSPH_FIX_CLUMP_ROTATION."""
    rng = np.random.default_rng(seed)
    box = 0.03
    r = Recipe("tiny_tumbling")
    m = 0.006
    r.setDomain((-m, -m, -m), (box + 2 * m, box + 2 * m, 0.02 + 2 * m))
    Es, Gs = hertz_from_E_nu(1.0e8, 0.3)
    for a in range(2):
        for b in range(a, 2):
            r.setHertzianContactModel(a, b, Es, Gs, 0.5, 0.2, 0.2, 0.4, 0.05, 0.05)
    rp = 1.0e-3
    shape = np.array([[-1.5, 0.0, 0.0], [0.0, 0.0, 0.0], [1.5, 0.0, 0.0], [0.2, 1.3, 0.0]]) * 1.0e-3
    shape -= shape.mean(axis=0)
    Rs = _random_rotations(rng, n_clumps)
    density = 2500.0
    for k in range(n_clumps):
        gx, gy = k % 4, k // 4
        peb = shape @ Rs[k].T
        c = np.array([0.004 + gx * 0.0065, 0.004 + gy * 0.009, 0.0])
        c[2] = rp - 2.0e-5 - peb[:, 2].min()
        peb = peb + c
        pr = np.full(4, rp)
        mass = density * 4.0 / 3.0 * math.pi * rp ** 3 * 4 * 0.9
        w = tuple(rng.uniform(-60.0, 60.0, 3))
        r.addClump(peb, pr, c, (0.0, 0.0, -0.2), w, mass, clump_inertia(peb, pr, c, mass), 1)
    sp = np.column_stack([rng.uniform(0.002, box - 0.002, n_spheres), rng.uniform(0.002, box - 0.002, n_spheres),
                          rng.uniform(0.004, 0.012, n_spheres)])
    r.addCluster(sp, rng.uniform(0.6e-3, 1.0e-3, n_spheres), np.full(n_spheres, density), (0.0, 0.0, -0.3), 0)
    r.addInfiniteWall((0, 0, 0), (0, 0, 1), 0)
    for p, n in (((0, 0, 0), (1, 0, 0)), ((box, 0, 0), (-1, 0, 0)), ((0, 0, 0), (0, 1, 0)),
                 ((0, box, 0), (0, -1, 0))):
        r.addInfiniteWall(p, n, 0)
    G = 1.0e8 / (2 * 1.3)
    t_r = math.pi * 0.6e-3 * math.sqrt(density / G) / (0.1631 * 0.3 + 0.8766)
    dt = 0.1 * t_r
    r.setSimulationParameterTimeStep(dt)
    r.setSimulationParameterMaximumTime((steps - 0.5) * dt)
    r.setSimulationParameterNumFrames(1)
    # the reference's wall normals need a fluid smoothing length (core/dataBase.cpp:359)
    r.addFluid(np.array([[box + m - 1e-3, box + m - 1e-3, 0.02 + m - 1e-3]]), (0, 0, 0), 5.0e-4, 1000.0, 20.0,
               1.0e-6)
    r.meta.update(dt=dt, steps=steps, gap=1, dx=2.0e-3)
    return r


def tiny_granular_wide(cells=700_000, seed=3):
    """:func:`tiny_granular` in a domain widened (empty cells around the grains)
    to about ``cells`` grid cells, so the sort by cell scans long cell arrays:
    one block up to 524,288 cells, three launches beyond."""
    r = tiny_granular(seed)
    idx = next(k for k, (fn, _) in enumerate(r.calls) if fn == "setDomain")
    o, s = r.calls[idx][1]
    base = s[0] * s[1] * s[2]
    # cells of 2 x the largest effective radius (1.2 mm + margin): scale x and y
    cell = 2.4e-3
    k = max(1.0, float(np.sqrt(cells * cell ** 3 / base)))
    r.calls[idx] = ("setDomain", (o, (s[0] * k, s[1] * k, s[2])))
    r.name = f"tiny_granular_wide_{cells}"
    return r


def tiny_two_fluids(seed=6):
    """:func:`tiny_dam_break` with a second, denser column beside the first
    (its own rest density, sound speed and smoothing length)."""
    r = tiny_dam_break(seed)
    rng = np.random.default_rng(seed)
    dx = 0.02
    fp = regular_packed_points((0.16, 0.0, 0.0), (0.08, 0.12, 0.08), dx)
    fp = fp + rng.uniform(-0.01 * dx, 0.01 * dx, size=fp.shape)
    r.addFluid(fp, (0, 0, 0), 1.2 * dx, 1500.0, 25.0, 2.0e-6)
    r.name = "tiny_two_fluids"
    return r


def tiny_escape(seed=5, with_probe_fluid=True):
    """64 spheres on a floor wall (no side walls) and two touching spheres
    above the domain: the reference hashes those to its overflow cell
    (core/neighborSearch.h:44-53) and finds their contact only because that
    cell's key is one of the keys its 27-cell walk visits from the corner cell
    below them, so the lists must come from that walk.  The probe fluid
    particle is there for the reference's wall normals (see
    :func:`tiny_granular`)."""
    r = granular_settle(n_spheres=64, n_clumps=0, box=(0.01, 0.01), spacing=2.3e-3, steps=50, seed=seed,
                        z0=1.0e-3, velocity=(0.05, -0.03, -0.2), name="tiny_escape")
    r.calls = [c for c in r.calls if not (c[0] == "addInfiniteWall" and tuple(c[1][1]) != (0.0, 0.0, 1.0))]
    o, sz = next(args for fn, args in r.calls if fn == "setDomain")
    top = o[2] + sz[2]
    p = np.array([[o[0] + 1.0e-3, o[1] + 1.0e-3, top + 0.9e-3], [o[0] + 2.4e-3, o[1] + 1.0e-3, top + 0.9e-3]])
    r.addSolid(p, (0, 0, -0.3), 8.0e-4, 2500.0, 0)
    if with_probe_fluid:
        r.addFluid(np.array([[o[0] + sz[0] - 1e-3, o[1] + sz[1] - 1e-3, o[2] + 1e-3]]), (0, 0, 0), 5.0e-4, 1000.0,
                   20.0, 1.0e-6)
    return r


def tiny_coupled(seed=4, gap=3, with_clump=True):
    """Dam break of 600 fluid particles onto two bonded 3x3x3 clusters and a
    4-pebble clump (left out when ``with_clump`` is false), with walls; the
    fluid is integrated every ``gap`` steps."""
    rng = np.random.default_rng(seed)
    dx = 0.01
    tank = (0.2, 0.08, 0.12)
    m = 3 * dx
    r = Recipe("tiny_coupled")
    r.setDomain((-m, -m, -m), (tank[0] + 2 * m, tank[1] + 2 * m, tank[2] + 2 * m))
    fp = regular_packed_points((0.0, 0.0, 0.0), (0.06, 0.08, 0.08), dx)
    fp = fp + rng.uniform(-0.01 * dx, 0.01 * dx, size=fp.shape)
    r.addFluid(fp, (0, 0, 0), 1.3 * dx, 1000.0, 20.0, 1.0e-6)
    r.addDummyParticleWall(_tank_walls(dx, tank), 0.5 * dx)
    sr = 2.0e-3
    Es, Gs = hertz_from_E_nu(1.0e7, 0.3)
    for a in range(3):
        for b in range(a, 3):
            r.setHertzianContactModel(a, b, Es, Gs, 0.5, 0.1, 0.1, 0.4, 0.05, 0.05)
    r.setBondedContactModel(1, 1, 2.0 * 1.0e4 / (math.pi * sr), 2.5, 1.0, 0.5e6, 0.3e6, 0.2)
    for k, x0 in enumerate((0.09, 0.14)):
        pts = regular_packed_points((x0, 0.03, 0.0), (6 * sr, 6 * sr, 6 * sr), 2 * sr)
        r.addCluster(pts, np.full(len(pts), sr), np.full(len(pts), 2500.0), (0, 0, 0), 1)
    tet = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=np.float64) / math.sqrt(3.0) * 1.5e-3
    c = np.array([0.12, 0.06, 0.01])
    peb = c + tet
    pr = np.full(4, 1.5e-3)
    mass = 2500.0 * 4.0 / 3.0 * math.pi * 1.5e-3 ** 3 * 3.2
    if with_clump:
        r.addClump(peb, pr, c, (0, 0, 0), (0, 0, 0), mass, clump_inertia(peb, pr, c, mass), 2)
    r.addInfiniteWall((0, 0, 0), (0, 0, 1), 0)
    mass1 = 2500.0 * 4.0 / 3.0 * math.pi * sr ** 3
    dt = 0.2 * math.sqrt(mass1 / 1.0e4)
    r.setSimulationParameterTimeStep(dt)
    r.setFluidIntegrateGap(gap)
    r.setSimulationParameterMaximumTime(40 * dt)
    r.setSimulationParameterNumFrames(1)
    r.meta.update(dt=dt, steps=40, gap=gap, dx=dx)
    return r


def tiny_additions(base=None):
    """Particles added to tiny_coupled while it runs (dataBase::addFluid,
    addCluster and addSolid after the start): a 3x3x3 block of fluid over the
    dry end of the tank, a bonded 2x2x2 cluster on the floor and a single
    sphere above the clump.  Returns (additions, whole): the additions alone
    (the base's domain and contact models with the new particles only) and
    the base with them added in the same order."""
    base = base or tiny_coupled()
    dx = base.meta["dx"]
    blocks = Recipe("blocks")
    fp = regular_packed_points((0.16, 0.02, 0.05), (0.03, 0.03, 0.03), dx)
    blocks.addFluid(fp, (0, 0, 0), 1.3 * dx, 1000.0, 20.0, 1.0e-6)
    sr = 2.0e-3
    pts = regular_packed_points((0.17, 0.05, 0.0), (4 * sr, 4 * sr, 4 * sr), 2 * sr)
    blocks.addCluster(pts, np.full(len(pts), sr), np.full(len(pts), 2500.0), (0, 0, 0), 1)
    blocks.addSolid(np.array([[0.12, 0.06, 0.02]]), (0, 0, 0), sr, 2500.0, 0)
    setters = [c for c in base.calls if not c[0].startswith("add")]
    add = Recipe(base.name + "_additions", setters + blocks.calls, dict(base.meta))
    whole = Recipe(base.name + "_whole", base.calls + blocks.calls, dict(base.meta))
    return add, whole


def tiny_converging(n=4, spacing=2.3e-3, radius=1.0e-3, rate=1200.0, steps=40):
    """An n x n x n lattice of equal spheres with 0.3 mm gaps whose velocities
    point at the lattice centre (v = -rate (x - centre)), no gravity, no walls,
    no fluid: every sphere meets its lattice neighbours within a few steps of
    the others, so the contact rows fill from empty in the middle of a run."""
    r = Recipe("tiny_converging")
    ax = (np.arange(n) + 0.5) * spacing
    p = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), axis=-1).reshape(-1, 3)
    c = 0.5 * n * spacing
    m = 3 * spacing
    r.setDomain((-m, -m, -m), (n * spacing + 2 * m,) * 3)
    r.setGravity((0.0, 0.0, 0.0))
    Es, Gs = hertz_from_E_nu(1.0e8, 0.3)
    r.setHertzianContactModel(0, 0, Es, Gs, 0.5, 0.0, 0.0, 0.4, 0.0, 0.0)
    density = 2500.0
    for k in range(len(p)):
        r.addSolid(p[k:k + 1], tuple(-rate * (p[k] - c)), radius, density, 0)
    G = 1.0e8 / (2 * 1.3)
    t_r = math.pi * radius * math.sqrt(density / G) / (0.1631 * 0.3 + 0.8766)
    dt = 0.1 * t_r
    r.setSimulationParameterTimeStep(dt)
    r.setSimulationParameterMaximumTime((steps - 0.5) * dt)
    r.setSimulationParameterNumFrames(1)
    r.meta.update(dt=dt, steps=steps, gap=1, dx=spacing)
    return r
