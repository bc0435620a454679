"""Seeded synthetic scenes (host-side numpy), identical for the CUDA path and
any checker.  Each builder returns a ``Scene``: parameters plus particle,
constraint and body arrays in the layout of the C ABI.

Randomness comes from splitmix64 streams keyed by the seed, so every
consumer gets bit-identical inputs.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

PHASE_FLUID, PHASE_GAS, PHASE_CLOTH, PHASE_SOLID, PHASE_RIGID = 0, 1, 2, 3, 4
FLAG_TWOD = 1
FLAG_DENSITY_NEIGHBOR_MASS = 1 << 1
FLAG_KERNEL_UNITS = 1 << 4
FLAG_SKIP_FIXED_NEIGHBORS = 1 << 5
FLAG_DELTA_OVER_COUNT = 1 << 6
FLAG_CPU_CONTACTS = 1 << 7


def splitmix64(seed: int, count: int) -> np.ndarray:
    """count uint64 outputs of the splitmix64 generator started at seed."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, shape, lo: float, hi: float) -> np.ndarray:
    n = int(np.prod(shape))
    u = (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return (lo + (hi - lo) * u).reshape(shape)


def next_pow2(v: float) -> int:
    return 1 << max(0, math.ceil(math.log2(max(1.0, v))))


@dataclass
class Scene:
    name: str
    params: dict
    pos_w: np.ndarray                      # (N, 4) float32: xyz, inverse mass
    phase: np.ndarray                      # (N,) int32
    vel: np.ndarray | None = None          # (N, 4) float32
    rest_density: np.ndarray | None = None  # (N,) float32
    pairs: np.ndarray | None = None        # (M, 2) uint32
    rest: np.ndarray | None = None         # (M,) float32
    stiffness: np.ndarray | None = None    # (M,) float32
    pins: np.ndarray | None = None         # (P,) uint32
    pin_points: np.ndarray | None = None   # (P, 3) float32
    bodies: list = field(default_factory=list)  # (first, count, stiffness)
    open_gas: list = field(default_factory=list)  # (first, count) ranges of open gas
    sdf: list = field(default_factory=list)  # per body (same order): (count, 4) sdf data or None
    dt: float = 1.0 / 60.0
    info: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.pos_w.shape[0])


def poly6_rest_density(spacing: float, h: float, mass: float = 1.0) -> float:
    """Sum of poly6 over a cubic lattice (self included), FP64: the rest
    density at which a perfect lattice of that spacing has C = 0."""
    c = 315.0 / (64.0 * math.pi * h ** 9)
    k = int(math.ceil(h / spacing)) + 1
    rng = np.arange(-k, k + 1)
    ox, oy, oz = np.meshgrid(rng, rng, rng, indexing="ij")
    r2 = (ox ** 2 + oy ** 2 + oz ** 2).astype(np.float64) * spacing * spacing
    r2 = r2[r2 < h * h]
    return float(mass * np.sum(c * (h * h - r2) ** 3))


def dam_break(nx: int = 128, ny: int = 128, nz: int = 64, h: float = 0.1, seed: int = 2024,
              iterations: int = 4, xsph: float = 0.01, cell_div: int = 1) -> Scene:
    """3-D PBF dam break: an nx*ny*nz fluid block, lattice spacing h/2,
    jitter U(-0.01h, 0.01h), in the corner of a box four block-widths long
    in x and twice the block height; cell size h / cell_div, power-of-two
    grid covering the box's length and depth and the block's height.

    Unit mass, rest density = the lattice's poly6 sum; s_corr k = 0.1,
    n = 4, dq = 0.2 h and relaxation 1 in kernel-radius units
    (FLAG_KERNEL_UNITS: 100 m^-2 at h = 0.1).  The reference's literal
    relaxation 0.01 lets particles with few neighbours take lambda ~ 80
    and the block explodes within one step at this length scale."""
    s = 0.5 * h
    r = 0.5 * s
    ext = np.array([4 * nx * s, 2 * ny * s, nz * s])
    cell = h / cell_div
    # the grid spans the box in x and z and the block's height in y; rare
    # particles splashing higher wrap onto lower cells (the reference's
    # power-of-two wrap), where the distance test rejects them
    grid = [next_pow2(ext[0] / cell), next_pow2(ny * s / cell), next_pow2(ext[2] / cell)]
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    # particle order: x fastest, then y, then z (the reference's lattice loops)
    lat = np.stack([ii.transpose(2, 1, 0).ravel(), jj.transpose(2, 1, 0).ravel(), kk.transpose(2, 1, 0).ravel()], 1)
    pos = (lat + 0.5) * s + uniform(seed, lat.shape, -0.01 * h, 0.01 * h)
    n = pos.shape[0]
    pos_w = np.empty((n, 4), np.float32)
    pos_w[:, :3] = pos
    pos_w[:, 3] = 1.0
    rho0 = poly6_rest_density(s, h)
    params = dict(particle_radius=r, kernel_radius=h, cell_size=cell, grid_size=grid,
                  world_origin=[0.0, 0.0, 0.0], gravity=[0.0, -9.8, 0.0], box_min=[0.0, 0.0, 0.0],
                  box_max=[float(v) for v in ext], iterations=iterations, relaxation=1.0, scorr_k=0.1,
                  scorr_n=4.0, scorr_dq=0.2, xsph_c=xsph, max_dt=0.05, max_neighbors=500,
                  flags=FLAG_KERNEL_UNITS)
    return Scene("dam_break", params, pos_w, np.zeros(n, np.int32),
                 rest_density=np.full(n, rho0, np.float32), dt=1.0 / 120.0,
                 info=dict(nx=nx, ny=ny, nz=nz, spacing=s, rho0=rho0, seed=seed))


def reference_scene_params(radius=0.25, grid=(64, 64, 64), min_bounds=(-50, 0, -50), max_bounds=(50, 200, 50),
                           iterations=5) -> dict:
    """The reference ParticleSystem constants (particleapp.cpp:23-38,
    particlesystem.cpp:52-66, integration_kernel.cuh:20-42)."""
    return dict(particle_radius=radius, kernel_radius=2.0, cell_size=2.0 * radius, grid_size=list(grid),
                world_origin=[0.0, 0.0, 0.0], gravity=[0.0, -9.8, 0.0], box_min=[float(v) for v in min_bounds],
                box_max=[float(v) for v in max_bounds], iterations=iterations, relaxation=0.01, scorr_k=0.1,
                scorr_n=4.0, scorr_dq=0.2, xsph_c=0.0, max_dt=0.05, max_neighbors=500,
                contact_static_friction=0.005, contact_kinetic_friction=0.0002,
                wall_static_friction=0.005, wall_kinetic_friction=0.0002)


def reference_fluid(ll=(-4, 0, -4), ur=(4, 6, 4), radius=0.25, density=1.0, mass=1.0, seed=7,
                    grid=(64, 64, 64), min_bounds=(-50, 0, -50), max_bounds=(50, 200, 50), jitter=0.01,
                    iterations=5) -> Scene:
    """The reference addFluid lattice (spacing 2.5 r, particlesystem.cpp:
    357-405) with seeded jitter, reference constants (h = 2)."""
    d = radius * 2.5
    cnt = [int(float(int(math.ceil(ur[k] - ll[k]))) / d) for k in range(3)]
    zz, yy, xx = np.meshgrid(np.arange(cnt[2]), np.arange(cnt[1]), np.arange(cnt[0]), indexing="ij")
    lat = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], 1).astype(np.float64)
    pos = np.array(ll, np.float64) + lat * d + uniform(seed, lat.shape, -1.0, 1.0) * (radius * jitter)
    n = pos.shape[0]
    pos_w = np.empty((n, 4), np.float32)
    pos_w[:, :3] = pos
    pos_w[:, 3] = 1.0 / mass
    params = reference_scene_params(radius, grid, min_bounds, max_bounds, iterations)
    return Scene("reference_fluid", params, pos_w, np.zeros(n, np.int32),
                 rest_density=np.full(n, density, np.float32), dt=1.0 / 60.0)


def reference_granular(ll=(-3, 0, -3), ur=(3, 8, 3), radius=0.25, mass=1.0, seed=11, jitter=0.05,
                       grid=(64, 64, 64), min_bounds=(-50, 0, -50), max_bounds=(50, 200, 50),
                       iterations=5, spacing_scale=1.95) -> Scene:
    """A solid-particle stack (addParticleGrid, particlesystem.cpp:408-458)
    packed slightly tighter than contact distance so contacts are active."""
    d = radius * spacing_scale
    cnt = [int(float(int(math.ceil(ur[k] - ll[k]))) / d) for k in range(3)]
    zz, yy, xx = np.meshgrid(np.arange(cnt[2]), np.arange(cnt[1]), np.arange(cnt[0]), indexing="ij")
    lat = np.stack([xx.ravel(), yy.ravel(), zz.ravel()], 1).astype(np.float64)
    pos = np.array(ll, np.float64) + lat * d + uniform(seed, lat.shape, -1.0, 1.0) * (radius * jitter)
    pos[:, 1] += radius
    n = pos.shape[0]
    pos_w = np.empty((n, 4), np.float32)
    pos_w[:, :3] = pos
    pos_w[:, 3] = 1.0 / mass
    params = reference_scene_params(radius, grid, min_bounds, max_bounds, iterations)
    return Scene("reference_granular", params, pos_w, np.full(n, PHASE_SOLID, np.int32), dt=1.0 / 60.0)


def rope_and_cloth(radius=0.25, seed=3, iterations=5, cloth=(12, 10), ropes=4, links=16) -> Scene:
    """Ropes and a cloth as the reference builds them (addRope,
    addHorizCloth; particlesystem.cpp:461-616): object phases RIGID + id,
    axis distance constraints, pinned starts / one pinned cloth edge.  The
    constrained particles come first so the reference's segment indexing
    (solver.cu:227-230) is harmless and the reference can be compared."""
    params = reference_scene_params(radius, iterations=iterations)
    pos, ph, pairs, rest, pins, pts = [], [], [], [], [], []
    obj = 0
    n0 = 0
    for r in range(ropes):
        start = np.array([-6.0 + 3.0 * r, 20.0, 0.5 * r])
        spacing = np.array([0.45, -0.12, 0.05 * (r + 1)])
        for i in range(links + 1):
            pos.append([*(start + i * spacing), 1.0])
            ph.append(PHASE_RIGID + obj)
            if i:
                pairs.append([n0 + i - 1, n0 + i])
                rest.append(0.4)
        pins.append(n0)
        pts.append(start)
        n0 += links + 1
        obj += 1
    cx, cz = cloth
    for z in range(cz):
        for x in range(cx):
            p = n0 + z * cx + x
            pos.append([5.0 + 0.5 * x, 7.0, -3.0 + 0.5 * z, 1.0 / 3.0])
            ph.append(PHASE_RIGID + obj)
            if x > 0:
                pairs.append([p - 1, p])
                rest.append(0.3)
            else:
                pins.append(p)
                pts.append(pos[-1][:3])
            if z > 0:
                pairs.append([p - cx, p])
                rest.append(0.3)
    pos_w = np.asarray(pos, np.float32)
    jit = uniform(seed, (pos_w.shape[0], 3), -0.01, 0.01)
    pos_w[:, :3] += jit.astype(np.float32)
    pts = np.asarray(pts, np.float32)
    pin_idx = np.asarray(pins, np.uint32)
    pts = pos_w[pin_idx, :3].copy()
    return Scene("rope_and_cloth", params, pos_w, np.asarray(ph, np.int32), pairs=np.asarray(pairs, np.uint32),
                 rest=np.asarray(rest, np.float32), pins=pin_idx, pin_points=pts, dt=1.0 / 60.0)


def random_quaternions(seed: int, count: int) -> np.ndarray:
    """Uniform random unit quaternions (Shoemake's method), (count, 4) xyzw."""
    u = uniform(seed, (count, 3), 0.0, 1.0)
    a, b, c = u[:, 0], u[:, 1], u[:, 2]
    q = np.stack([np.sqrt(1 - a) * np.sin(2 * np.pi * b), np.sqrt(1 - a) * np.cos(2 * np.pi * b),
                  np.sqrt(a) * np.sin(2 * np.pi * c), np.sqrt(a) * np.cos(2 * np.pi * c)], 1)
    return q


def quat_rotate(q: np.ndarray, v: np.ndarray) -> np.ndarray:
    x, y, z, w = q[..., 0:1], q[..., 1:2], q[..., 2:3], q[..., 3:4]
    u = np.concatenate([x, y, z], -1)
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def box_sdf(dims, radius: float) -> np.ndarray:
    """Signed-distance data of a box of particles on a lattice of spacing
    2 r, in the lattice order of np.meshgrid(..., indexing="ij") over dims
    (2 or 3 axes): (N, 4) outward normal xyz and depth.  The reference's
    SDF boxes (simulation.cpp:666-672) generalised: the normal is the
    normalised sum of the outward axes whose faces are nearest, the depth
    that face distance times sqrt(number of such axes) -- r on a face, r
    sqrt(2) on an edge, r sqrt(3) at a corner; a particle whose nearest
    faces cancel (the centre of an odd axis) points up."""
    dims = list(dims)
    idx = np.stack(np.meshgrid(*[np.arange(k) for k in dims], indexing="ij"), -1).reshape(-1, len(dims))
    n = np.asarray(dims)
    face = (np.minimum(idx, n - 1 - idx) * 2 + 1) * radius  # distance to the nearer face, per axis
    dmin = face.min(1, keepdims=True)
    near = np.isclose(face, dmin)
    side = np.where(idx < n - 1 - idx, -1.0, np.where(idx > n - 1 - idx, 1.0, 0.0))
    g = np.zeros((idx.shape[0], 3))
    g[:, :len(dims)] = np.where(near, side, 0.0)
    t = near.sum(1)
    ln = np.linalg.norm(g, axis=1)
    g[ln == 0.0] = [0.0, 1.0, 0.0]
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    out = np.empty((idx.shape[0], 4))
    out[:, :3] = g
    out[:, 3] = dmin[:, 0] * np.sqrt(t)
    return out


def rigid_boxes(count=8, side=4, radius=0.25, seed=5, iterations=4, drop_height=6.0, stiffness=1.0,
                sdf: bool = False) -> Scene:
    """count shape-matched side^3 boxes at seeded random orientations above
    the floor, as separate objects (phase RIGID + id); with sdf, each body
    carries box_sdf data in its rest frame (the frame it was added in)."""
    params = reference_scene_params(radius, iterations=iterations)
    d = 2.0 * radius
    g = (np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3) - (side - 1) / 2.0) * d
    qs = random_quaternions(seed, count)
    centers = np.stack([(np.arange(count) % 4) * (side * d * 2.0) - 4.0,
                        drop_height + (np.arange(count) // 4) * side * d * 2.0,
                        uniform(seed + 1, (count,), -1.0, 1.0)], 1)
    pos, ph, bodies, sdfs = [], [], [], []
    lattice_sdf = box_sdf([side] * 3, radius) if sdf else None
    for b in range(count):
        qb = np.broadcast_to(qs[b], (g.shape[0], 4))
        pts = quat_rotate(qb, g) + centers[b]
        bodies.append((len(pos), g.shape[0], stiffness))
        if sdf:
            e = lattice_sdf.copy()
            e[:, :3] = quat_rotate(qb, lattice_sdf[:, :3])
            sdfs.append(e.astype(np.float32))
        for p in pts:
            pos.append([*p, 1.0])
            ph.append(PHASE_RIGID + b)
    return Scene("rigid_boxes", params, np.asarray(pos, np.float32), np.asarray(ph, np.int32), bodies=bodies,
                 sdf=sdfs, dt=1.0 / 60.0)


def sdf_contact_pairs(pairs: int = 24, radius: float = 0.25, seed: int = 9) -> dict:
    """2-D pinning case of the signed-distance rigid contact: `pairs` pairs
    of 2 x 2 boxes (spacing 2 r, the reference's SDF corners: normal
    (+-1, +-1) / sqrt(2), depth r sqrt(2)), each body rotated by a seeded
    angle, the second box of a pair placed so that exactly one corner of
    each touches (centre distance U(1.5 r, 1.95 r)) while every other pair
    of particles of different bodies stays beyond 2.05 r; estimates =
    start + U(-0.05 r, 0.05 r).  Pairs are 10 apart along x.  Returns the
    lattice-frame positions (rest shape), start and estimate positions
    (n, 2), inverse masses U(0.5, 2), body of each particle, lattice-frame
    sdf (n, 4), body angles and the touching particle pairs (i1 < i2)."""
    d = 2.0 * radius
    lat = (np.array([[0, 0], [0, 1], [1, 0], [1, 1]], float) - 0.5) * d
    corner_sdf = np.zeros((4, 4))
    corner_sdf[:, :2] = np.sign(lat) / np.sqrt(2.0)
    corner_sdf[:, 3] = radius * np.sqrt(2.0)
    rot = lambda a, v: np.stack([np.cos(a) * v[:, 0] - np.sin(a) * v[:, 1],  # noqa: E731
                                 np.sin(a) * v[:, 0] + np.cos(a) * v[:, 1]], 1)
    rng_seed = seed
    start, angles, body, touching = [], [], [], []
    k = 0
    while len(touching) < pairs:
        u = uniform(rng_seed, (6,), 0.0, 1.0)
        rng_seed += 1
        a_ang, b_ang = u[0] * 2 * np.pi, u[1] * 2 * np.pi
        base = np.array([10.0 * len(touching), 5.0])
        pa = rot(a_ang, lat) + base
        ca = int(u[2] * 4) % 4
        cb = int(u[3] * 4) % 4
        dirn = pa[ca] - pa.mean(0)
        dirn = rot((u[4] - 0.5) * 0.8, (dirn / np.linalg.norm(dirn))[None])[0]
        gap = (1.5 + 0.45 * u[5]) * radius
        lb = rot(b_ang, lat)
        pb = lb - lb[cb] + pa[ca] + gap * dirn
        dist = np.linalg.norm(pa[:, None, :] - pb[None, :, :], axis=2)
        close = dist < 2.05 * radius
        if close.sum() != 1 or not close[ca, cb]:
            continue
        first = 8 * len(touching)
        start += [pa, pb]
        angles += [a_ang, b_ang]
        body += [2 * len(touching)] * 4 + [2 * len(touching) + 1] * 4
        touching.append((first + ca, first + 4 + cb))
        k += 1
    start = np.concatenate(start)
    n = start.shape[0]
    est = start + uniform(seed + 1000, (n, 2), -0.05 * radius, 0.05 * radius)
    return dict(lattice=np.tile(lat, (2 * pairs, 1)), start=start, estimate=est,
                imass=uniform(seed + 2000, (n,), 0.5, 2.0), body=np.asarray(body, np.int32),
                sdf=np.tile(corner_sdf, (2 * pairs, 1)), angles=np.asarray(angles),
                pairs=np.asarray(touching, np.int32))


def apply_to(scene: Scene, system, params=None):
    """Load a Scene into anything with the C ABI's add_* methods (the CUDA
    ParticleSystem, or a checker with the same surface)."""
    system.add_particles(scene.pos_w, scene.vel, scene.phase, scene.rest_density)
    if scene.pairs is not None and len(scene.pairs):
        system.add_distance_constraints(scene.pairs, scene.rest, scene.stiffness)
    if scene.pins is not None and len(scene.pins):
        system.add_point_constraints(scene.pins, scene.pin_points)
    for k, (first, count, st) in enumerate(scene.bodies):
        b = system.add_rigid_body(first, count, st)
        if k < len(scene.sdf) and scene.sdf[k] is not None:
            system.set_rigid_sdf(b, scene.sdf[k])
    for first, count in scene.open_gas:
        system.set_gas_open(first, count, True)
    return system


def mixed_scene(cloth: int = 256, ropes: int = 2000, rope_particles: int = 64, bodies: int = 10000,
                side: int = 4, radius: float = 0.25, seed: int = 77, iterations: int = 4,
                rope_lift: float = 3.0, layer_gap: float = 1.0, body_lift: float | None = None) -> Scene:
    """Mixed rigid/rope/cloth scene: a cloth x cloth sheet with stretch
    (axis neighbours), shear (diagonals) and bend (skip-one) distance
    constraints and pinned edges; `ropes` free ropes of `rope_particles`
    particles in layers above it; and `bodies` shape-matched side^3 boxes at
    seeded uniform-random orientations above the ropes.  Spacing 2 r;
    every object has its own phase (RIGID + id), so no self-collisions.
    Heights: cloth at 10, the first rope layer rope_lift above it, rope
    layers layer_gap apart, box centres from body_lift (default 2 side r)
    above the last rope layer, box layers 4 side r apart.
    The defaults give 65,536 + 128,000 + 640,000 = 833,536 particles."""
    d = 2.0 * radius
    ext = cloth * d  # sheet edge length
    pos, phase, pairs, rest, pins = [], [], [], [], []
    obj = 0
    # cloth, particle (x, z) at index x + cloth * z, height 10
    cx, cz = np.meshgrid(np.arange(cloth), np.arange(cloth), indexing="xy")
    cloth_pos = np.stack([cx.ravel() * d, np.full(cloth * cloth, 10.0), cz.ravel() * d], 1)
    pos.append(cloth_pos)
    phase.append(np.full(cloth * cloth, PHASE_RIGID + obj, np.int32))
    obj += 1
    idx = np.arange(cloth * cloth).reshape(cloth, cloth)  # [z, x]
    for (a, b, rl) in ((idx[:, :-1], idx[:, 1:], d), (idx[:-1, :], idx[1:, :], d),            # stretch
                       (idx[:-1, :-1], idx[1:, 1:], d * math.sqrt(2)), (idx[:-1, 1:], idx[1:, :-1], d * math.sqrt(2)),  # shear
                       (idx[:, :-2], idx[:, 2:], 2 * d), (idx[:-2, :], idx[2:, :], 2 * d)):     # bend
        pairs.append(np.stack([a.ravel(), b.ravel()], 1))
        rest.append(np.full(a.size, rl))
    edge = np.unique(np.concatenate([idx[0, :], idx[-1, :], idx[:, 0], idx[:, -1]]))
    pins.append(edge)
    n0 = cloth * cloth
    # ropes along x in layers above the sheet
    per_row = max(1, int(ext // (rope_particles * d)))
    rows_per_layer = max(1, int(ext // 1.0))
    for r in range(ropes):
        layer, rr = divmod(r, per_row * rows_per_layer)
        row, k = divmod(rr, per_row)
        start = np.array([k * rope_particles * d, 10.0 + rope_lift + layer_gap * layer,
                          (row + 0.5) * (ext / rows_per_layer)])
        rp = start + np.arange(rope_particles)[:, None] * np.array([d, 0.0, 0.0])
        pos.append(rp)
        phase.append(np.full(rope_particles, PHASE_RIGID + obj, np.int32))
        obj += 1
        ids = n0 + np.arange(rope_particles)
        pairs.append(np.stack([ids[:-1], ids[1:]], 1))
        rest.append(np.full(rope_particles - 1, d))
        n0 += rope_particles
    rope_layers = -(-ropes // (per_row * rows_per_layer))
    top = 10.0 + rope_lift + layer_gap * max(0, rope_layers - 1) + (side * d if body_lift is None else body_lift)
    # boxes above, on a lattice of 2 side spacing, random orientations
    g = (np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3) - (side - 1) / 2.0) * d
    qs = random_quaternions(seed, bodies)
    pitch = 2.0 * side * d
    per_axis = max(1, int(ext // pitch))
    body_list = []
    for b in range(bodies):
        layer, rr = divmod(b, per_axis * per_axis)
        ix, iz = divmod(rr, per_axis)
        c = np.array([(ix + 0.5) * pitch, top + layer * pitch, (iz + 0.5) * pitch])
        pts = quat_rotate(np.broadcast_to(qs[b], (g.shape[0], 4)), g) + c
        body_list.append((n0, g.shape[0], 1.0))
        pos.append(pts)
        phase.append(np.full(g.shape[0], PHASE_RIGID + obj, np.int32))
        obj += 1
        n0 += g.shape[0]
    pos = np.concatenate(pos)
    n = pos.shape[0]
    pos_w = np.empty((n, 4), np.float32)
    pos_w[:, :3] = pos + uniform(seed + 1, (n, 3), -0.01 * radius, 0.01 * radius)
    pos_w[:, 3] = 1.0
    pins = np.concatenate(pins).astype(np.uint32)
    height = float(top + (bodies // (per_axis * per_axis) + 1) * pitch + 2.0)
    cell = 2.002 * radius
    # the wrapping hash lets x and z spill a few cells past the grid's span
    grid = [next_pow2(ext / cell), next_pow2(height / cell), next_pow2(ext / cell)]
    params = dict(particle_radius=radius, kernel_radius=2.0 * radius, cell_size=cell, grid_size=grid,
                  world_origin=[-1.0, 0.0, -1.0], gravity=[0.0, -9.8, 0.0], box_min=[-1.0, 0.0, -1.0],
                  box_max=[ext + 1.0, height, ext + 1.0], iterations=iterations, relaxation=0.01, scorr_k=0.1,
                  scorr_n=4.0, scorr_dq=0.2, xsph_c=0.0, max_dt=0.05, max_neighbors=500,
                  contact_static_friction=0.005, contact_kinetic_friction=0.0002,
                  wall_static_friction=0.005, wall_kinetic_friction=0.0002)
    return Scene("mixed", params, pos_w, np.concatenate(phase), pairs=np.concatenate(pairs).astype(np.uint32),
                 rest=np.concatenate(rest).astype(np.float32), pins=pins, pin_points=pos_w[pins, :3].copy(),
                 bodies=body_list, dt=1.0 / 60.0,
                 info=dict(cloth=cloth, ropes=ropes, bodies=bodies, constraints=int(sum(len(r) for r in rest))))


_RHO0_CACHE: dict = {}


def pbf_block(count: int, h: float = 0.1, seed: int = 2024, iterations: int = 4, xsph: float = 0.01,
              cell_div: int = 1, max_dt: float = 1.0 / 120.0) -> Scene:
    """A PBF block of exactly `count` fluid particles on the dam-break
    lattice (spacing h/2, jitter U(-0.01h, 0.01h)): footprint nx = 2 nz
    columns, filled from the floor up (x fastest, then z, then y; the top
    layer may be partial), in the corner of a box four block-widths long
    and twice the block height.  Parameters as dam_break; max_dt = 1/120
    so that a 1/60 step of a mixed batch gives the dam break's 1/120."""
    s = 0.5 * h
    nz = max(1, int(round((count / 4.0) ** (1.0 / 3.0))))
    nx = 2 * nz
    ny = -(-count // (nx * nz))
    k = np.arange(count)
    lat = np.stack([k % nx, k // (nx * nz), (k // nx) % nz], 1)
    pos = (lat + 0.5) * s + uniform(seed, lat.shape, -0.01 * h, 0.01 * h)
    ext = np.array([4 * nx * s, 2 * ny * s, nz * s])
    cell = h / cell_div
    grid = [next_pow2(ext[0] / cell), next_pow2(ny * s / cell), next_pow2(ext[2] / cell)]
    pos_w = np.empty((count, 4), np.float32)
    pos_w[:, :3] = pos
    pos_w[:, 3] = 1.0
    key = (s, h)
    if key not in _RHO0_CACHE:
        _RHO0_CACHE[key] = poly6_rest_density(s, h)
    rho0 = _RHO0_CACHE[key]
    params = dict(particle_radius=0.5 * s, kernel_radius=h, cell_size=cell, grid_size=grid,
                  world_origin=[0.0, 0.0, 0.0], gravity=[0.0, -9.8, 0.0], box_min=[0.0, 0.0, 0.0],
                  box_max=[float(v) for v in ext], iterations=iterations, relaxation=1.0, scorr_k=0.1,
                  scorr_n=4.0, scorr_dq=0.2, xsph_c=xsph, max_dt=max_dt, max_neighbors=500,
                  flags=FLAG_KERNEL_UNITS)
    return Scene("pbf_block", params, pos_w, np.zeros(count, np.int32),
                 rest_density=np.full(count, rho0, np.float32), dt=1.0 / 120.0,
                 info=dict(nx=nx, ny=ny, nz=nz, rho0=rho0, seed=seed))


def granular_column(count: int = 1600, width: int | None = None, radius: float = 0.25, seed: int = 1600,
                    iterations: int = 3, static_friction: float = 0.5, kinetic_friction: float = 0.3,
                    cpu_contacts: bool = False) -> Scene:
    """2-D granular column collapse: `count` solid particles (unit inverse
    mass) on a lattice of spacing 2r, `width` columns (default round(sqrt
    (count)), 40 for 1,600), rows from y = r up, the top row possibly
    partial, jitter U(-0.01r, 0.01r) in x and y; centred in a box as wide as
    twice the column, friction mu_s / mu_k on contacts and walls, z pinned
    to 0 (FLAG_TWOD), 3 iterations, dt = 1/60.  Cell 2r as the reference;
    the grid covers the box's width and the column's height and is one cell
    deep (in 2-D the particles share one z layer and the stencils walk only
    that layer).  cpu_contacts: the CPU reference's contact and boundary
    projectors (PBD_FLAG_CPU_CONTACTS) and its open-topped box (walls at
    x = +-half and y = 0; the top at 1e6), as its sand pile runs them."""
    d = 2.0 * radius
    width = int(width or max(1, round(math.sqrt(count))))
    rows = -(-count // width)
    k = np.arange(count)
    pos = np.zeros((count, 3))
    pos[:, 0] = (k % width - (width - 1) / 2.0) * d
    pos[:, 1] = radius + (k // width) * d
    pos[:, :2] += uniform(seed, (count, 2), -0.01 * radius, 0.01 * radius)
    half = width * d
    height = rows * d
    cell = d
    grid = [next_pow2(2 * half / cell), next_pow2(height / cell), 1]
    pos_w = np.empty((count, 4), np.float32)
    pos_w[:, :3] = pos
    pos_w[:, 3] = 1.0
    params = dict(particle_radius=radius, kernel_radius=2.0 * d, cell_size=cell, grid_size=grid,
                  world_origin=[-half, 0.0, -2.0 * cell], gravity=[0.0, -9.8, 0.0],
                  box_min=[-half, 0.0, -1.0], box_max=[half, 2.0 * height + 10.0, 1.0], iterations=iterations,
                  relaxation=0.01, scorr_k=0.1, scorr_n=4.0, scorr_dq=0.2, xsph_c=0.0, max_dt=1.0 / 60.0,
                  max_neighbors=500, contact_static_friction=static_friction,
                  contact_kinetic_friction=kinetic_friction, wall_static_friction=static_friction,
                  wall_kinetic_friction=kinetic_friction, twod_z=0.0, flags=FLAG_TWOD)
    if cpu_contacts:
        params["flags"] = FLAG_TWOD | FLAG_CPU_CONTACTS
        params["box_max"] = [half, 1e6, 1.0]
    return Scene("granular_column", params, pos_w, np.full(count, PHASE_SOLID, np.int32), dt=1.0 / 60.0,
                 info=dict(width=width, rows=rows, seed=seed, cpu_contacts=cpu_contacts))


def smoke_box(spacing: float = 0.63, half: float = 4.0, twod: bool = False, density: float | None = None,
              open_gas: bool = True, seed: int = 1096, iterations: int = 3, solid_floor: bool = False) -> Scene:
    """The CPU reference's smoke scene (initSmokeOpen / initSmokeClosed,
    cpu/src/simulation.cpp:1096-1134) in 3-D, or in 2-D with twod: gas
    particles of unit mass on a lattice of spacing 0.63 over [-4, 4)^d,
    jitter 0.2 U(-0.5, 0.5) per axis (the reference's .2 (frand() - .5),
    seeded), one gas, open or closed, of rest density 1.5 in 2-D (the
    reference's value, about the 2-D lattice's poly6 sum) and the lattice's
    poly6 sum in 3-D unless `density` is given; h = 2, cell h,
    relaxation 0.01 and the gas constants of gasconstraint.h (the
    pbd_params defaults), gravity -9.8 (x ALPHA = -0.2 on gas: it rises),
    3 iterations, dt 1/60, box x (and z) in [-6, 6], y in [-4, 200].  With
    solid_floor, a fixed solid plate (w = 0) of the same spacing lies below
    the gas, and a layer of movable solid grains on it, so gas particles
    have solid neighbours (weighted S_SOLID) and fixed ones (ignored)."""
    axis = np.arange(-half, half - 1e-9, spacing)
    dims = 2 if twod else 3
    if density is None:
        density = 1.5 if twod else poly6_rest_density(spacing, 2.0)
    grids = np.meshgrid(*([axis] * dims), indexing="ij")
    lat = np.stack([g.ravel() for g in grids], 1)
    n = lat.shape[0]
    pos = np.zeros((n, 3))
    pos[:, 0] = lat[:, 0]
    pos[:, 1] = lat[:, 1]
    if not twod:
        pos[:, 2] = lat[:, 2]
    pos[:, :dims] += 0.2 * uniform(seed, (n, dims), -0.5, 0.5)
    pos_w = np.empty((n, 4), np.float32)
    pos_w[:, :3] = pos
    pos_w[:, 3] = 1.0
    phase = np.full(n, PHASE_GAS, np.int32)
    rho0 = np.full(n, density, np.float32)
    if solid_floor:
        plane = np.meshgrid(*([axis] * (dims - 1)), indexing="ij")
        flat = np.stack([g.ravel() for g in plane], 1)
        m = flat.shape[0]
        extra = []
        for y, w in ((-half - 1.2, 0.0), (-half - 0.6, 1.0)):  # fixed plate, then grains
            q = np.zeros((m, 4), np.float32)
            q[:, 0] = flat[:, 0]
            q[:, 1] = y
            if not twod:
                q[:, 2] = flat[:, 1]
            q[:, 3] = w
            extra.append(q)
        pos_w = np.concatenate([pos_w] + extra)
        phase = np.concatenate([phase, np.full(2 * m, PHASE_SOLID, np.int32)])
        rho0 = np.concatenate([rho0, np.ones(2 * m, np.float32)])
    h = 2.0
    cell = h
    box_lo, box_hi = [-6.0, -4.0 - (2.0 if solid_floor else 0.0), -6.0], [6.0, 200.0, 6.0]
    grid = [next_pow2((box_hi[0] - box_lo[0]) / cell), next_pow2((box_hi[1] - box_lo[1]) / cell),
            1 if twod else next_pow2((box_hi[2] - box_lo[2]) / cell)]
    origin = [box_lo[0], box_lo[1], -2.0 * cell if twod else box_lo[2]]
    params = dict(particle_radius=0.25, kernel_radius=h, cell_size=cell, grid_size=grid, world_origin=origin,
                  gravity=[0.0, -9.8, 0.0], box_min=[box_lo[0], box_lo[1], -1.0 if twod else box_lo[2]],
                  box_max=[box_hi[0], box_hi[1], 1.0 if twod else box_hi[2]], iterations=iterations,
                  relaxation=0.01, scorr_k=0.1, scorr_n=4.0, scorr_dq=0.2, xsph_c=0.0, max_dt=1.0 / 60.0,
                  max_neighbors=500, twod_z=0.0, flags=FLAG_TWOD if twod else 0)
    return Scene("smoke_box", params, pos_w, phase, rest_density=rho0,
                 open_gas=[(0, n)] if open_gas else [], dt=1.0 / 60.0,
                 info=dict(gas=n, solids=int(pos_w.shape[0] - n), seed=seed, open=open_gas))


def cpu_fluid_box(spacing: float = 0.7, seed: int = 890, density: float = 1.75, solid_floor: bool = True,
                  iterations: int = 3) -> Scene:
    """The CPU reference's 2-D fluid scene (initFluid, cpu/src/simulation.cpp:
    894-913): fluid particles of unit mass on a lattice of spacing 0.7 over
    [-4, 4) x [-4, 2), jitter 0.2 U(-0.5, 0.5) per axis (the reference's .2
    (frand() - .5), seeded), rest density 1.75 (its second fluid's), h = 2,
    cell h.  With solid_floor, a fixed solid plate (w = 0) of the same
    spacing below the fluid and a layer of movable solid grains on it, so
    fluid particles have solid neighbours and fixed ones.  The flags select
    the CPU reference's fluid formulas (TotalFluidConstraint::project,
    totalfluidconstraint.cpp:41-116): neighbour masses in the density,
    fixed particles left out, the correction over rho0 (n + 1); and
    solid_density_weight 0 (S_SOLID, totalfluidconstraint.h:30).  2-D
    mode, no neighbour cap in effect (the reference has none)."""
    xs = np.arange(-4.0, 4.0 - 1e-9, spacing)
    ys = np.arange(-4.0, 2.0 - 1e-9, spacing)
    gx, gy = np.meshgrid(xs, ys, indexing="ij")
    n = gx.size
    pos = np.zeros((n, 3))
    pos[:, 0] = gx.ravel()
    pos[:, 1] = gy.ravel()
    pos[:, :2] += 0.2 * uniform(seed, (n, 2), -0.5, 0.5)
    pos_w = np.empty((n, 4), np.float32)
    pos_w[:, :3] = pos
    pos_w[:, 3] = 1.0
    phase = np.full(n, PHASE_FLUID, np.int32)
    rho0 = np.full(n, density, np.float32)
    if solid_floor:
        m = xs.size
        extra = []
        for y, w in ((-4.0 - 1.4, 0.0), (-4.0 - spacing, 1.0)):  # fixed plate, then grains
            q = np.zeros((m, 4), np.float32)
            q[:, 0] = xs
            q[:, 1] = y
            q[:, 3] = w
            extra.append(q)
        pos_w = np.concatenate([pos_w] + extra)
        phase = np.concatenate([phase, np.full(2 * m, PHASE_SOLID, np.int32)])
        rho0 = np.concatenate([rho0, np.ones(2 * m, np.float32)])
    h = 2.0
    box_lo, box_hi = [-8.0, -8.0, -1.0], [8.0, 40.0, 1.0]
    grid = [next_pow2((box_hi[0] - box_lo[0]) / h), next_pow2((box_hi[1] - box_lo[1]) / h), 1]
    params = dict(particle_radius=0.25, kernel_radius=h, cell_size=h, grid_size=grid,
                  world_origin=[box_lo[0], box_lo[1], -2.0 * h], gravity=[0.0, -9.8, 0.0], box_min=box_lo,
                  box_max=box_hi, iterations=iterations, relaxation=0.01, scorr_k=0.1, scorr_n=4.0, scorr_dq=0.2,
                  xsph_c=0.0, max_dt=1.0 / 60.0, max_neighbors=100000, twod_z=0.0, solid_density_weight=0.0,
                  flags=FLAG_TWOD | FLAG_DENSITY_NEIGHBOR_MASS | FLAG_SKIP_FIXED_NEIGHBORS | FLAG_DELTA_OVER_COUNT)
    return Scene("cpu_fluid_box", params, pos_w, phase, rest_density=rho0, dt=1.0 / 60.0,
                 info=dict(fluid=n, solids=int(pos_w.shape[0] - n), seed=seed))


CPU_CONTACT_BOX = (-20.0, 400.0, 0.0, 50.0)  # xmin, xmax, ymin, ymax of the contact pinning case


def cpu_contact_case(pairs: int = 24, fluid_pairs: int = 12, walls: int = 16, radius: float = 0.25,
                     seed: int = 31) -> dict:
    """2-D pinning case of the CPU reference's contact projectors, each
    particle in exactly one constraint (so the reference's sequential
    projection and a Jacobi pass coincide): `pairs` pairs of solid grains
    touching at a centre distance U(1.5 r, 1.95 r) in a seeded direction,
    `fluid_pairs` grains each touching one fluid particle the same way, and
    `walls` grains each past one wall of the box CPU_CONTACT_BOX by U(0.1 r,
    0.8 r) (lower and upper x, lower and upper y in turn; at most 17 so
    that no grain is past two walls).  Objects stand 10 apart along x at
    heights 3 + U(0, 4) (the masses are height-scaled); estimates = start +
    U(-0.08 r, 0.08 r); inverse masses U(0.5, 2).  Returns the start and
    estimate positions (n, 2), inverse masses, solid flags, the touching
    pairs (i1 < i2) and the walls (idx, is_x, lower)."""
    xmin, xmax, ymin, ymax = CPU_CONTACT_BOX
    start, solid, plist, wlist = [], [], [], []
    u = uniform(seed, (pairs + fluid_pairs, 4), 0.0, 1.0)
    for k in range(pairs + fluid_pairs):
        base = np.array([10.0 * k, 3.0 + 4.0 * u[k, 0]])
        ang = 2.0 * np.pi * u[k, 1]
        gap = (1.5 + 0.45 * u[k, 2]) * radius
        i = len(start)
        start += [base, base + gap * np.array([np.cos(ang), np.sin(ang)])]
        solid += [1, 1 if k < pairs else 0]
        plist.append((i, i + 1))
    wu = uniform(seed + 1, (walls, 2), 0.0, 1.0)
    for k in range(walls):
        side = k % 4
        depth = (0.1 + 0.7 * wu[k, 0]) * radius
        along = 10.0 + 4.0 * (k // 4) + wu[k, 1]  # walls' grains 3 or more apart
        if side == 0:
            q, is_x, lower = (xmin + radius - depth, along), 1, 1
        elif side == 1:
            q, is_x, lower = (xmax - radius + depth, along), 1, 0
        elif side == 2:
            q, is_x, lower = (40.0 + 20.0 * k, ymin + radius - depth), 0, 1
        else:
            q, is_x, lower = (40.0 + 20.0 * k, ymax - radius + depth), 0, 0
        wlist.append((len(start), is_x, lower))
        start.append(np.array(q))
        solid.append(1)
    start = np.asarray(start)
    n = start.shape[0]
    est = start + uniform(seed + 2, (n, 2), -0.08 * radius, 0.08 * radius)
    return dict(start=start, estimate=est, imass=uniform(seed + 3, (n,), 0.5, 2.0),
                solid=np.asarray(solid, np.int32), pairs=np.asarray(plist, np.int32),
                walls=np.asarray(wlist, np.int32))


def batched_scenes(count: int = 512, seed: int = 512, lo: int = 1024, hi: int = 65536) -> list:
    """`count` independent scenes with particle counts round(exp(U(ln lo,
    ln hi))), each a PBF block or a granular column by a seeded coin flip."""
    sizes = np.rint(np.exp(uniform(seed, (count,), math.log(lo), math.log(hi)))).astype(np.int64)
    coin = uniform(seed + 1, (count,), 0.0, 1.0) < 0.5
    out = []
    for k in range(count):
        n = int(sizes[k])
        out.append(pbf_block(n, seed=seed * 1000 + k) if coin[k] else granular_column(n, seed=seed * 1000 + k))
    return out


def cloth_ropes_grains(cloth: int = 64, ropes: int = 8, rope_particles: int = 32, grains: int = 200,
                       radius: float = 0.25, seed: int = 5, iterations: int = 4, drop: float = 3.0,
                       stiffness_seed: int | None = None) -> Scene:
    """A cloth x cloth sheet (spacing 2r, stretch constraints between axis
    neighbours, the two edges x = 0 and x = max pinned) at height 6; `ropes`
    ropes of `rope_particles` particles lying across it 0.6 above (first
    particle pinned); `grains` solid grains seeded uniformly in a slab
    `drop` above the sheet with downward velocities U(-2, -1) and small
    sideways ones.  Stiffness U(0.2, 1) per constraint when stiffness_seed
    is given (else 1).  The defaults give 4,096 + 256 + 200 = 4,552
    particles."""
    d = 2.0 * radius
    ext = cloth * d
    pos, vel, phase, pairs, pins = [], [], [], [], []
    obj = 0
    cx, cz = np.meshgrid(np.arange(cloth), np.arange(cloth), indexing="xy")
    pos.append(np.stack([cx.ravel() * d, np.full(cloth * cloth, 6.0), cz.ravel() * d], 1))
    phase.append(np.full(cloth * cloth, PHASE_RIGID + obj, np.int32))
    obj += 1
    idx = np.arange(cloth * cloth).reshape(cloth, cloth)  # [z, x]
    pairs += [np.stack([idx[:, :-1].ravel(), idx[:, 1:].ravel()], 1),
              np.stack([idx[:-1, :].ravel(), idx[1:, :].ravel()], 1)]
    pins.append(np.concatenate([idx[:, 0], idx[:, -1]]))
    n0 = cloth * cloth
    for r in range(ropes):
        z = (r + 0.5) * ext / ropes
        rp = np.stack([0.5 * d + np.arange(rope_particles) * d * min(1.0, (cloth - 1) / rope_particles),
                       np.full(rope_particles, 6.6), np.full(rope_particles, z)], 1)
        pos.append(rp)
        phase.append(np.full(rope_particles, PHASE_RIGID + obj, np.int32))
        obj += 1
        ids = n0 + np.arange(rope_particles)
        pairs.append(np.stack([ids[:-1], ids[1:]], 1))
        pins.append(ids[:1])
        n0 += rope_particles
    g = np.stack([uniform(seed, (grains,), 0.1 * ext, 0.9 * ext), uniform(seed + 1, (grains,), 7.2, 7.2 + drop),
                  uniform(seed + 2, (grains,), 0.1 * ext, 0.9 * ext)], 1)
    pos.append(g)
    phase.append(np.full(grains, PHASE_SOLID, np.int32))
    pos = np.concatenate(pos)
    n = pos.shape[0]
    pos_w = np.empty((n, 4), np.float32)
    pos_w[:, :3] = pos
    pos_w[:, 3] = 1.0
    vel = np.zeros((n, 4), np.float32)
    vel[n - grains:, 0] = uniform(seed + 3, (grains,), -0.3, 0.3)
    vel[n - grains:, 1] = uniform(seed + 4, (grains,), -2.0, -1.0)
    vel[n - grains:, 2] = uniform(seed + 5, (grains,), -0.3, 0.3)
    pairs = np.concatenate(pairs).astype(np.uint32)
    rest = np.linalg.norm(pos_w[pairs[:, 0], :3].astype(np.float64) - pos_w[pairs[:, 1], :3], axis=1)
    stiff = (np.ones(len(pairs), np.float32) if stiffness_seed is None
             else uniform(stiffness_seed, (len(pairs),), 0.2, 1.0).astype(np.float32))
    pins = np.concatenate(pins).astype(np.uint32)
    cell = 2.002 * radius
    height = 7.2 + drop + 2.0
    grid = [next_pow2(ext / cell), next_pow2(height / cell), next_pow2(ext / cell)]
    params = dict(particle_radius=radius, kernel_radius=2.0 * radius, cell_size=cell, grid_size=grid,
                  world_origin=[-1.0, 0.0, -1.0], gravity=[0.0, -9.8, 0.0], box_min=[-1.0, 0.0, -1.0],
                  box_max=[ext + 1.0, 60.0, ext + 1.0], iterations=iterations, relaxation=0.01, scorr_k=0.1,
                  scorr_n=4.0, scorr_dq=0.2, xsph_c=0.0, max_dt=1.0 / 60.0, max_neighbors=500,
                  contact_static_friction=0.1, contact_kinetic_friction=0.05,
                  wall_static_friction=0.1, wall_kinetic_friction=0.05)
    return Scene("cloth_ropes_grains", params, pos_w, np.concatenate(phase), vel=vel, pairs=pairs,
                 rest=rest.astype(np.float32), stiffness=stiff, pins=pins, pin_points=pos_w[pins, :3].copy(),
                 dt=1.0 / 60.0, info=dict(cloth=cloth, ropes=ropes, grains=grains))


def differentiation_scenes(count: int = 64, seed: int = 64, **kw) -> list:
    """`count` cloth / rope / grain scenes (cloth_ropes_grains), each with
    its own grain cloud and hidden per-constraint stiffness U(0.2, 1)."""
    return [cloth_ropes_grains(seed=seed * 1000 + 10 * k, stiffness_seed=seed * 1000 + 10 * k + 7, **kw)
            for k in range(count)]
