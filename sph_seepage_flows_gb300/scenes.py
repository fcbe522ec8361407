"""Seeded synthetic scenes of the benchmark workloads.

The reference builds its scenes with host emitters
(seepage_flows_cuda/src/kiri_pbs_cuda/emitter/*.cpp). Its box emitter jitters
with an unseeded ``std::random_device`` (cuda_volume_emitter.cpp:86-99) and its
app scene needs a bunny asset that is not distributed, so every scene here is
generated from a seed: lattice blocks with uniform +-1% jitter per axis, the
world-boundary shell of ``CudaBoundaryEmitter::BuildWorldBoundary``
(cuda_boundary_emitter.cpp:12-80, restated in float32 by
:func:`world_boundary`) and the reference parameters of main.cpp:40-83.

Workloads (sizes in metres):

* ``plain_small``: 8,000 sand (r = 0.01) + 32,000 water (pitch 0.02) in a
  1 x 1 x 1 box (the 1.0 x 0.5 x 0.5 box of the spec cannot hold a 40 x 40
  water column at 0.02 pitch; the counts are kept and the box grown).
* ``plain_large``: ~500k sand (r = 0.005) in a trapezoidal embankment 0.4 high
  with 1V:2H slopes + ~500k water (pitch 0.01) in a reservoir to 0.35, box
  4.0 x 0.6 x 1.0, h = 0.02.
* ``batched``: independent sand-block + water-column scenes with log-uniform
  counts and per-scene friction / capillary / permeability scales.
* ``adjoint``: 10k-sand column (32 x 32 x 10) + ~10k water at its base.
* ``tiny``: a few thousand particles for parity fixtures.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .params import (SF_LABEL_SAND, SF_LABEL_WATER, SF_TYPE_MULTI_SF, SfBoundaryParams, SfParams,
                     SfSolverParams, boundary_params, reference_params, solver_params, tan_deg)

WATER_COLOR = (np.array([127.0, 205.0, 255.0], dtype=np.float32) / np.float32(255.0))


@dataclass
class Scene:
    name: str
    params: SfParams
    bparams: SfBoundaryParams
    sparams: SfSolverParams
    pos: np.ndarray
    vel: np.ndarray
    col: np.ndarray
    label: np.ndarray
    mass: np.ndarray
    radius: np.ndarray
    cda0asat: np.ndarray
    amcamcp: np.ndarray
    bpos: np.ndarray
    blabel: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    @property
    def nb(self) -> int:
        return int(self.bpos.shape[0])

    @property
    def n_sand(self) -> int:
        return int((self.label == SF_LABEL_SAND).sum())

    @property
    def n_water(self) -> int:
        return int((self.label == SF_LABEL_WATER).sum())


def world_boundary(lowest, highest, particle_radius: float):
    """CudaBoundaryEmitter::BuildWorldBoundary (cuda_boundary_emitter.cpp:12-80)
    in float32: six lattice planes at pitch 2r (bottom, top, back, front,
    left, right), label 0, edges repeated as the reference repeats them."""
    lo = np.asarray(lowest, dtype=np.float32)
    hi = np.asarray(highest, dtype=np.float32)
    spacing = np.float32(particle_radius) * np.float32(2.0)
    sides = (hi - lo) / spacing

    def count(s):  # for (size_t i = 0; i <= s; ++i) with the float comparison
        return int(math.floor(float(s))) + 1 if s >= 0 else 0

    def coords(base, k):
        return (base + np.arange(k, dtype=np.float32) * spacing).astype(np.float32)

    nx, ny, nz = count(sides[0]), count(sides[1]), count(sides[2])
    X, Y, Z = coords(lo[0], nx), coords(lo[1], ny), coords(lo[2], nz)
    planes = []

    def plane(a, b, fn):
        A, Bv = np.meshgrid(a, b, indexing="ij")
        planes.append(fn(A.ravel(), Bv.ravel()))

    full = lambda v, k: np.full(k, v, dtype=np.float32)  # noqa: E731
    plane(X, Z, lambda a, b: np.stack([a, full(lo[1], a.size), b], 1))   # ZX bottom
    plane(X, Z, lambda a, b: np.stack([a, full(hi[1], a.size), b], 1))   # ZX top
    plane(X, Y, lambda a, b: np.stack([a, b, full(lo[2], a.size)], 1))   # XY back
    plane(X, Y, lambda a, b: np.stack([a, b, full(hi[2], a.size)], 1))   # XY front
    plane(Y, Z, lambda a, b: np.stack([full(lo[0], a.size), a, b], 1))   # YZ left
    plane(Y, Z, lambda a, b: np.stack([full(hi[0], a.size), a, b], 1))   # YZ right
    pos = np.concatenate(planes).astype(np.float32)
    return pos, np.zeros(pos.shape[0], dtype=np.int32)


def _lattice(origin, counts, pitch, rng, jitter_frac):
    o = np.asarray(origin, dtype=np.float64)
    idx = np.stack(np.meshgrid(*[np.arange(c) for c in counts], indexing="ij"), -1).reshape(-1, 3)
    p = o + idx * pitch
    if jitter_frac > 0:
        p = p + rng.uniform(-jitter_frac * pitch, jitter_frac * pitch, size=p.shape)
    return p.astype(np.float32)


def _assemble(name, params, bparams, sparams, sand_pos, water_pos, sand_radius, water_radius,
              cda0asat=None, amcamcp=None, meta=None) -> Scene:
    ns, nw = sand_pos.shape[0], water_pos.shape[0]
    pos = np.concatenate([sand_pos, water_pos]).astype(np.float32)
    label = np.concatenate([np.full(ns, SF_LABEL_SAND, np.int32), np.full(nw, SF_LABEL_WATER, np.int32)])
    sand_mass = np.float32(params.dem_density) * (np.float32(4.0) / np.float32(3.0) * np.float32(math.pi)
                                                  * np.float32(sand_radius) ** np.float32(3))
    mass = np.concatenate([np.full(ns, sand_mass, np.float32), np.full(nw, params.sph_mass, np.float32)])
    radius = np.concatenate([np.full(ns, sand_radius, np.float32), np.full(nw, water_radius, np.float32)])
    dry = np.asarray(params.sf_dry_sand_color[:], dtype=np.float32)
    col = np.concatenate([np.tile(dry, (ns, 1)), np.tile(WATER_COLOR, (nw, 1))]).astype(np.float32)
    if cda0asat is None:
        cda0asat = np.array([params.sf_cd, params.sf_a0, params.sf_asat], dtype=np.float32)
    if amcamcp is None:
        amcamcp = np.array([params.sf_amc, params.sf_amc_p], dtype=np.float32)
    # per-material arrays are set for sand only; water keeps the zero fill of
    # the reference's cleared arrays (AddSphParticles never writes them)
    cda = np.zeros((ns + nw, 3), np.float32)
    cda[:ns] = cda0asat
    amc = np.zeros((ns + nw, 2), np.float32)
    amc[:ns] = amcamcp
    lo = np.asarray(bparams.lowest_point[:], np.float32)
    hi = np.asarray(bparams.highest_point[:], np.float32)
    bpos, blabel = world_boundary(lo, hi, params.sph_particle_radius)
    return Scene(name=name, params=params, bparams=bparams, sparams=sparams, pos=pos,
                 vel=np.zeros_like(pos), col=col, label=label, mass=mass, radius=radius,
                 cda0asat=cda, amcamcp=amc, bpos=bpos, blabel=blabel, meta=meta or {})


def block_scene(name, box, sand_counts, water_counts, pitch, seed, sand_origin=None, water_origin=None,
                jitter_frac=0.01, tan_phi=None, cap_scale=1.0, perm_scale=1.0, dem_density=2650.0,
                gravity_y=-9.81) -> Scene:
    """A sand lattice block resting on the floor at the +x end of the box and
    a water lattice column at the -x end (the plain-small layout)."""
    r = pitch / 2.0
    params = reference_params(sph_radius=r, dem_radius=r, dem_density=dem_density, gravity_y=gravity_y)
    if tan_phi is not None:
        params.dem_tan_friction_angle = float(np.float32(tan_phi))
    params.sf_c0 = float(np.float32(params.sf_c0 * cap_scale))
    params.sf_cmc = float(np.float32(params.sf_cmc * cap_scale))
    params.sf_csat = float(np.float32(params.sf_csat * cap_scale))
    params.sf_cd = float(np.float32(params.sf_cd * perm_scale))
    h = params.sph_kernel_radius
    bparams = boundary_params((0.0, 0.0, 0.0), box, h)
    sparams = solver_params()
    rng = np.random.default_rng(seed)
    rij = 2.0 * r  # sand radius + water radius: the DEM world-wall contact distance
    sx, sy, sz = sand_counts
    if sand_origin is None:
        sand_origin = (box[0] - rij - (sx - 1) * pitch, rij, 0.5 * box[2] - 0.5 * (sz - 1) * pitch)
    if water_origin is None:
        water_origin = (2.0 * r, 2.0 * r, 2.0 * r)
    sand = _lattice(sand_origin, sand_counts, pitch, rng, jitter_frac)
    water = _lattice(water_origin, water_counts, pitch, rng, jitter_frac)
    meta = {"seed": seed, "pitch": pitch, "box": list(box), "sand_counts": list(sand_counts),
            "water_counts": list(water_counts), "tan_phi": params.dem_tan_friction_angle,
            "cap_scale": cap_scale, "perm_scale": perm_scale}
    return _assemble(name, params, bparams, sparams, sand, water, r, r, meta=meta)


def plain_small(seed: int = 1234) -> Scene:
    """8,000 sand spheres (20^3, r = 0.01) on the floor at x in [0.6, 1.0] and
    a 20 x 40 x 40 water column at pitch 0.02 at x in [0, 0.4], 1 m box."""
    return block_scene("plain_small", (1.0, 1.0, 1.0), (20, 20, 20), (20, 40, 40), 0.02, seed,
                       sand_origin=(0.6, 0.02, 0.31), water_origin=(0.02, 0.02, 0.1))


def tiny(seed: int = 7, sand=(10, 8, 10), water=(8, 12, 10)) -> Scene:
    """A few-thousand-particle version of plain_small for parity fixtures:
    a sand block and a water column that touch, in a 0.4 x 0.4 x 0.4 box."""
    pitch = 0.02
    return block_scene("tiny", (0.4, 0.4, 0.4), sand, water, pitch, seed,
                       sand_origin=(0.4 - 0.02 - (sand[0] - 1) * pitch, 0.02, 0.06),
                       water_origin=(0.4 - 0.02 - (sand[0] - 1 + water[0]) * pitch, 0.02, 0.06))


def add_shape_boundary(scene: Scene, points) -> Scene:
    """Appends shape boundary particles (label 1), as
    CudaBoundaryEmitter::BuildBoundaryShapeVolume does with the points of a
    shape file (cuda_boundary_emitter.cpp:82-92): sand collides with them
    (DEM) and water is pushed out of them at the end of every substep."""
    pts = np.asarray(points, np.float32).reshape(-1, 3)
    scene.bpos = np.concatenate([scene.bpos, pts]).astype(np.float32)
    scene.blabel = np.concatenate([scene.blabel, np.ones(len(pts), np.int32)])
    return scene


def tiny_with_plate(seed: int = 21) -> Scene:
    """tiny() standing on a shape-boundary plate (label 1) at z = 0.055, 5 mm
    below the lowest particle layer: the sand block rests on it through DEM
    contacts and the water above it is pushed out of its 2r shell."""
    sc = tiny(seed=seed)
    xs = np.arange(0.03, 0.39, 0.01, dtype=np.float32)
    ys = np.arange(0.01, 0.39, 0.01, dtype=np.float32)
    gx, gy = np.meshgrid(xs, ys, indexing="ij")
    plate = np.stack([gx.ravel(), gy.ravel(), np.full(gx.size, 0.055, np.float32)], axis=1)
    sc.name = "tiny_plate"
    return add_shape_boundary(sc, plate)


def _axis(start, stop, pitch):
    """Lattice coordinates start + k*pitch <= stop (k = 0, 1, ...)."""
    if stop < start:
        return np.zeros(0)
    return start + pitch * np.arange(int(np.floor((stop - start) / pitch + 1e-9)) + 1)


def _embankment_rows(toe, crest, height, pitch, y0):
    """(y, x-coordinates) rows of a trapezoid with 1V:2H slopes on the floor."""
    base = crest + 4.0 * height
    xs = _axis(toe, toe + base, pitch)
    rows = []
    for y in _axis(y0, height, pitch):
        rows.append((y, xs[(xs >= toe + 2.0 * y) & (xs <= toe + base - 2.0 * y)]))
    return rows


def _reservoir_rows(x0, toe, level, pitch, y0, gap):
    """(y, x-coordinates) rows of water from x0 up to the upstream slope."""
    xs = _axis(x0, toe + 2.0 * level, pitch)
    return [(y, xs[xs < toe + 2.0 * y - gap]) for y in _axis(y0, level, pitch)]


def _rows_count(rows, nz):
    return sum(len(x) for _, x in rows) * nz


def _rows_points(rows, zs):
    pts = []
    for y, xs in rows:
        if len(xs) == 0:
            continue
        X, Z = np.meshgrid(xs, zs, indexing="ij")
        pts.append(np.stack([X.ravel(), np.full(X.size, y), Z.ravel()], 1))
    return np.concatenate(pts) if pts else np.zeros((0, 3))


def plain_large(seed: int = 2024, target_sand: int = 500_000, target_water: int = 500_000) -> Scene:
    """1M particles: sand embankment (0.4 high, 1V:2H slopes, crest solved so
    the sand count is within 0.5% of target) and the upstream reservoir to
    0.35 (length solved likewise) in a 4.0 x 0.6 x 1.0 box, h = 0.02."""
    pitch, r = 0.01, 0.005
    box = (4.0, 0.6, 1.0)
    params = reference_params(sph_radius=r, dem_radius=r, dem_density=2650.0)
    bparams = boundary_params((0.0, 0.0, 0.0), box, params.sph_kernel_radius)
    rng = np.random.default_rng(seed)
    zs_s = _axis(2.0 * 2.0 * r, box[2] - 2.0 * r, pitch)     # the z-min wall tests 2 * rij
    zs_w = _axis(2.0 * r, box[2] - 2.0 * r, pitch)
    y0 = 2.0 * r
    height, level = 0.4, 0.35
    x0 = 2.0 * r
    lo_L, hi_L = 0.1, 3.0
    for _ in range(50):
        mid = 0.5 * (lo_L + hi_L)
        if _rows_count(_reservoir_rows(x0, x0 + mid, level, pitch, y0, pitch), len(zs_w)) < target_water:
            lo_L = mid
        else:
            hi_L = mid
    L = hi_L
    toe = x0 + L
    lo_c, hi_c = 0.0, 2.0
    for _ in range(50):
        mid = 0.5 * (lo_c + hi_c)
        if _rows_count(_embankment_rows(toe, mid, height, pitch, y0), len(zs_s)) < target_sand:
            lo_c = mid
        else:
            hi_c = mid
    crest = hi_c
    sand = _rows_points(_embankment_rows(toe, crest, height, pitch, y0), zs_s)
    water = _rows_points(_reservoir_rows(x0, toe, level, pitch, y0, pitch), zs_w)
    sand = (sand + rng.uniform(-0.01 * pitch, 0.01 * pitch, size=sand.shape)).astype(np.float32)
    water = (water + rng.uniform(-0.01 * pitch, 0.01 * pitch, size=water.shape)).astype(np.float32)
    meta = {"seed": seed, "crest": crest, "reservoir_length": L, "toe": toe,
            "n_sand": int(sand.shape[0]), "n_water": int(water.shape[0])}
    return _assemble("plain_large", params, bparams, solver_params(), sand, water, r, r, meta=meta)


def batched(n_scenes: int = 64, seed: int = 99, n_min: int = 2000, n_max: int = 60000):
    """Independent scenes: counts log-uniform in [n_min, n_max], sand fraction
    U[0.3, 0.7], friction angle U[25, 40] deg, capillary and permeability
    scales U[0.5, 2]; each a sand block + water column in a cubic box scaled
    to N^(1/3)."""
    rng = np.random.default_rng(seed)
    scenes = []
    pitch = 0.02
    for s in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        frac = rng.uniform(0.3, 0.7)
        phi = rng.uniform(25.0, 40.0)
        cap = rng.uniform(0.5, 2.0)
        perm = rng.uniform(0.5, 2.0)
        ns = max(8, int(round(n * frac)))
        nw = max(8, n - ns)
        side_s = max(2, int(round(ns ** (1.0 / 3.0))))
        sand_counts = (side_s, max(2, int(round(ns / side_s / side_s))), side_s)
        side_w = max(2, int(round((nw / 2.0) ** (1.0 / 3.0))))
        water_counts = (side_w, max(2, int(round(nw / side_w / side_w))), side_w)
        ext = max(sand_counts[0] + water_counts[0] + 4, sand_counts[1] + 4, water_counts[1] + 4,
                  sand_counts[2] + 4, water_counts[2] + 4)
        L = float(np.float32(ext * pitch + 0.04))
        box = (L, L, L)
        scenes.append(block_scene(f"batched_{s:02d}", box, sand_counts, water_counts, pitch,
                                  seed * 1000 + s,
                                  sand_origin=(L - 0.02 - (sand_counts[0] - 1) * pitch, 0.02,
                                               0.04 + 0.5 * (L - 0.08 - (sand_counts[2] - 1) * pitch)),
                                  water_origin=(0.02, 0.02, 0.04 + 0.5 * (L - 0.08 - (water_counts[2] - 1) * pitch)),
                                  tan_phi=tan_deg(phi), cap_scale=cap, perm_scale=perm))
    return scenes


def adjoint_column(seed: int = 5) -> Scene:
    """10,240 sand (32 x 10 x 32, r = 0.01, 0.2 m tall) with ~10k water at
    pitch 0.02 around the column base."""
    pitch = 0.02
    box = (1.2, 0.6, 1.2)
    sand_counts = (32, 10, 32)
    water_counts = (50, 4, 50)
    return block_scene("adjoint", box, sand_counts, water_counts, pitch, seed,
                       sand_origin=(0.29, 0.02, 0.29), water_origin=(0.1, 0.02, 0.1))


def column_scene(name: str, n_sand: int, n_water: int, seed: int, pitch: float = 0.02) -> Scene:
    """Column collapse: a sand column (height twice its width) in the middle
    of a square box whose base is flooded by a water layer three particles
    deep, the lattices offset by half a pitch (the adjoint-column geometry at
    another size)."""
    r = pitch / 2.0
    params = reference_params(sph_radius=r, dem_radius=r)
    s = max(2, int(round((n_sand / 2.0) ** (1.0 / 3.0))))
    sand_counts = (s, max(2, int(round(n_sand / (s * s)))), s)
    w = max(2, int(round(math.sqrt(n_water / 3.0))))
    water_counts = (w, 3, w)
    side = (max(w, s) + 4) * pitch
    height = (sand_counts[1] + 4) * pitch
    box = (float(np.float32(side)), float(np.float32(height)), float(np.float32(side)))
    bparams = boundary_params((0.0, 0.0, 0.0), box, params.sph_kernel_radius)
    rng = np.random.default_rng(seed)
    sand = _lattice((0.5 * side - 0.5 * (s - 1) * pitch, pitch, 0.5 * side - 0.5 * (s - 1) * pitch), sand_counts,
                    pitch, rng, 0.01)
    wo = 0.5 * side - 0.5 * (w - 1) * pitch + 0.5 * pitch
    water = _lattice((wo, pitch, wo), water_counts, pitch, rng, 0.01)
    return _assemble(name, params, bparams, solver_params(), sand, water, r, r,
                     meta={"seed": seed, "geometry": "column", "sand_counts": list(sand_counts),
                           "water_counts": list(water_counts)})


def embankment_scene(name: str, n_sand: int, n_water: int, seed: int, pitch: float = 0.02) -> Scene:
    """Embankment seepage: a sand trapezoid (1V:2H slopes, 10 layers high)
    with the reservoir behind it to 80% of its height, the depth (z extent)
    chosen for the sand count and the reservoir length for the water count."""
    r = pitch / 2.0
    params = reference_params(sph_radius=r, dem_radius=r)
    height = 10 * pitch
    level = 0.8 * height
    y0 = 2.0 * r
    crest = 4 * pitch
    toe_rel = lambda L: 2.0 * r + L  # noqa: E731
    per_z = _rows_count(_embankment_rows(0.0, crest, height, pitch, y0), 1)
    nz = max(2, int(round(n_sand / per_z)))
    lo_L, hi_L = 0.0, 20.0
    for _ in range(50):
        mid = 0.5 * (lo_L + hi_L)
        if _rows_count(_reservoir_rows(2.0 * r, toe_rel(mid), level, pitch, y0, pitch), nz) < n_water:
            lo_L = mid
        else:
            hi_L = mid
    toe = toe_rel(hi_L)
    length = toe + crest + 4.0 * height + 4.0 * pitch
    depth = (nz + 3) * pitch
    box = (float(np.float32(length)), float(np.float32(height + 4 * pitch)), float(np.float32(depth)))
    bparams = boundary_params((0.0, 0.0, 0.0), box, params.sph_kernel_radius)
    zs_s = _axis(2.0 * 2.0 * r, 2.0 * 2.0 * r + (nz - 1) * pitch, pitch)   # the z-min wall tests 2 * rij
    zs_w = zs_s
    rng = np.random.default_rng(seed)
    sand = _rows_points(_embankment_rows(toe, crest, height, pitch, y0), zs_s)
    water = _rows_points(_reservoir_rows(2.0 * r, toe, level, pitch, y0, pitch), zs_w)
    sand = (sand + rng.uniform(-0.01 * pitch, 0.01 * pitch, size=sand.shape)).astype(np.float32)
    water = (water + rng.uniform(-0.01 * pitch, 0.01 * pitch, size=water.shape)).astype(np.float32)
    return _assemble(name, params, bparams, solver_params(), sand, water, r, r,
                     meta={"seed": seed, "geometry": "embankment", "toe": toe, "depth_layers": nz})


def calibration_scenes(n_scenes: int = 32, seed: int = 77, n_min: int = 10_000, n_max: int = 50_000):
    """Scenes of the batched calibration: sizes log-uniform in [n_min, n_max],
    sand fraction U[0.4, 0.6], alternating column-collapse and
    embankment-seepage geometries."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        frac = rng.uniform(0.4, 0.6)
        ns, nw = int(round(n * frac)), n - int(round(n * frac))
        make = column_scene if s % 2 == 0 else embankment_scene
        out.append(make(f"calib_{s:02d}", ns, nw, seed * 1000 + s))
    return out


def capillary_rupture(r: float) -> float:
    """Liquid-bridge rupture distance of two sand spheres of radius r
    (ComputeDemCapillaryForces, cuda_dem_solver_common_gpu.cuh:63-65)."""
    contact_angle = 30.0 / 180.0 * math.pi
    vlb = 4.0 / 3.0 * math.pi * r ** 3 * 0.01 * 0.01
    return (1.0 + 0.5 * contact_angle) * (vlb ** (1.0 / 3.0) + 0.1 * vlb ** (2.0 / 3.0))


def adjoint_probe(seed: int = 11, sand_counts=(5, 3, 5), water_counts=(5, 6, 8), gap: float = 0.012,
                  sand_velocity=(0.05, 0.0, 0.03), water_pitch: float = 0.019, water_speed: float = 0.01,
                  margin: float = 5e-4, sand_overlap: float = 0.0, sand_speed: float = 0.0) -> Scene:
    """A small scene whose short-horizon trajectory stays away from the
    model's value discontinuities, for gradient checks against finite
    differences: sand at pitch 2r + s_rupture / 2 (every lattice pair inside
    the liquid-bridge band, no sand-sand contact), its bottom layer pressed
    1e-4 into the floor and sliding at sand_velocity (friction at the cap), a
    slightly compressed water block (positive pressure) beside it at the
    given gap, moving at random velocities up to water_speed (so no pair
    sits on the viscosity switch dv . d = 0), no sand-water pair within margin
    of h / 2 or h (the ends of the adhesion spline) and no sand whose nearest
    water lies within margin of h (voidage onset). With sand_overlap > 0 the
    sand pitch is 2r - sand_overlap instead (every lattice pair in DEM
    contact, no liquid bridges) and sand_speed adds random sand velocities
    (sliding contacts at the friction cap)."""
    r = 0.01
    params = reference_params(sph_radius=r, dem_radius=r)
    h = params.sph_kernel_radius
    box = (0.36, 0.24, 0.36)
    bparams = boundary_params((0.0, 0.0, 0.0), box, h)
    sparams = solver_params()
    rng = np.random.default_rng(seed)
    srupt = capillary_rupture(r)
    ps = 2.0 * r + 0.5 * srupt if sand_overlap <= 0.0 else 2.0 * r - sand_overlap
    sx, sy, sz = sand_counts
    idx = np.stack(np.meshgrid(*[np.arange(c) for c in sand_counts], indexing="ij"), -1).reshape(-1, 3)
    sand = np.array([0.20, 0.0199, 0.5 * box[2] - 0.5 * (sz - 1) * ps]) + idx * ps
    jit = 0.1 * srupt if sand_overlap <= 0.0 else 0.05 * sand_overlap
    sand = sand + rng.uniform(-jit, jit, size=sand.shape) * np.array([1.0, 0.2, 1.0])
    wx, wy, wz = water_counts
    widx = np.stack(np.meshgrid(*[np.arange(c) for c in water_counts], indexing="ij"), -1).reshape(-1, 3)
    wp = water_pitch
    zc = 0.5 * box[2] - 0.5 * (wz - 1) * wp
    water = np.array([0.20 - gap - (wx - 1) * wp, 0.035, zc]) + widx * wp
    water = water + rng.uniform(-2e-4, 2e-4, size=water.shape)
    wvel = rng.uniform(-water_speed, water_speed, size=water.shape)
    # drop water in the singular windows of the adhesion spline
    d = np.linalg.norm(water[:, None, :] - sand[None, :, :], axis=2)
    bad = (np.abs(d - 0.5 * h) < margin).any(1) | (np.abs(d - h) < margin).any(1)
    water = water[~bad]
    wvel = wvel[~bad]
    d = d[~bad]
    nearest = d.min(0)
    if np.any(np.abs(nearest - h) < margin):
        raise ValueError("a sand particle's nearest water lies at the kernel radius; pick another seed")
    sc = _assemble("adjoint_probe", params, bparams, sparams, sand.astype(np.float32), water.astype(np.float32),
                   r, r, meta={"seed": seed, "sand_pitch": ps, "gap": gap})
    sc.vel[: sand.shape[0]] = np.asarray(sand_velocity, dtype=np.float32)
    if sand_speed > 0.0:
        sc.vel[: sand.shape[0]] += rng.uniform(-sand_speed, sand_speed, size=(sand.shape[0], 3)).astype(np.float32)
    sc.vel[sand.shape[0]:] = wvel.astype(np.float32)
    return sc


def remove_overlaps(scene: Scene, min_dist: float) -> Scene:
    """Drop water particles closer than min_dist to a sand particle (used
    where a water lattice is laid over a sand block)."""
    sand = scene.pos[scene.label == SF_LABEL_SAND].astype(np.float64)
    water_idx = np.nonzero(scene.label == SF_LABEL_WATER)[0]
    if sand.size == 0 or water_idx.size == 0:
        return scene
    cell = min_dist
    keys = {}
    for k, p in enumerate(np.floor(sand / cell).astype(np.int64)):
        keys.setdefault(tuple(p), []).append(k)
    keep = np.ones(scene.n, dtype=bool)
    wp = scene.pos[water_idx].astype(np.float64)
    wc = np.floor(wp / cell).astype(np.int64)
    for a, (p, c) in enumerate(zip(wp, wc)):
        hit = False
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for k in keys.get((c[0] + dx, c[1] + dy, c[2] + dz), ()):
                        if np.sum((sand[k] - p) ** 2) < min_dist * min_dist:
                            hit = True
                            break
        if hit:
            keep[water_idx[a]] = False
    for name in ("pos", "vel", "col", "label", "mass", "radius", "cda0asat", "amcamcp"):
        setattr(scene, name, getattr(scene, name)[keep])
    return scene


WORKLOADS = {
    "plain_small": plain_small,
    "plain_large": plain_large,
    "tiny": tiny,
    "adjoint": adjoint_column,
}
