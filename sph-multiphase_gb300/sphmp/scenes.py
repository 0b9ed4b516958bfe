"""Seeded synthetic scenes for the multiphase SPH step.

The reference has no public benchmark or dataset; these builders stand in for
its scene files with the particle counts, spacings, phase layouts and
densities of the workloads this library is measured on:

* ``dam_break_2phase``  — 32x32x32 liquid block (d = 0.01 m, h = 0.02 m) with a gas
  sphere (r = 0.06 m at (0.16, 0.10, 0.16)) in a 0.64 m open box;
* ``blobs_3phase``      — 1,048,576 liquid particles on a 128 x 64 x 128 lattice (x, y, z;
  d = 0.005 m, h = 0.01 m) in a 1.28 x 0.64 x 0.64 m open box, phases from 64 random
  spherical blobs (radii 0.02-0.08 m);
* ``small_block``       — parameterised small scenes for parity tests.

Particles are generated with the library's own reference-equivalent generators
(sphmp_add_fluid_volume / sphmp_add_open_box) and the phase of each liquid
particle is then set from the blob layout. Boundary walls are two lattice
layers at the fluid spacing. The builders that take ``gen`` accept another set of
generator functions with the same signatures (the CPU oracle's, for runs that must
not load the CUDA library).
"""
from dataclasses import dataclass
from types import SimpleNamespace

import numpy as np

from . import abi
from . import add_fluid_volume, add_open_box, params_default, record_arrays, setup_constants, setup_grid

# the library's generators (the default of every builder's `gen`)
LIBRARY = SimpleNamespace(params_default=params_default, setup_constants=setup_constants, setup_grid=setup_grid,
                          record_arrays=record_arrays, add_fluid_volume=add_fluid_volume, add_open_box=add_open_box)


@dataclass
class Scene:
    params: abi.Params
    disp: np.ndarray
    calc: np.ndarray
    n_fluid: int
    n_boundary: int
    name: str = ""

    @property
    def n(self):
        return len(self.disp)


def make_params(*, h, d, dt, box_min, box_max, nphase, dens, visc, simscale=1.0, gravity=(0.0, -9.81, 0.0),
                eos=abi.EOS_LINEAR, eos_k=3.0, multiphase=1, headroom=None, bvisc=100.0, wall_layers=2, gen=LIBRARY):
    """Parameters for a box [box_min, box_max] (sim units) with `wall_layers` boundary layers at spacing d.
    Masses are rest density times (d * simscale)^3, the physical volume of a lattice site."""
    p = gen.params_default()
    p.smoothradius = h
    p.simscale = simscale
    p.dt = dt
    for a in range(3):
        p.gravity[a] = gravity[a]
    p.nphase = nphase
    p.multiphase = multiphase
    p.eos = eos
    p.eos_stiffness = eos_k
    for k in range(3):
        kk = min(k, nphase - 1)
        p.densArr[k] = dens[kk]
        p.viscArr[k] = visc[kk]
        p.massArr[k] = np.float32(dens[kk]) * np.float32(d * simscale) ** 3
    p.restdensity = dens[0]
    p.viscosity = visc[0]
    p.mass = p.massArr[0]
    p.bRestdensity = 1000.0
    p.bmass = np.float32(1000.0) * np.float32(d * simscale) ** 3
    p.bvisc = bvisc
    gen.setup_constants(p)
    # grid: walls (thickness t) plus two cells of padding; extra headroom above the box
    t = (wall_layers - 0.5) * d
    pad = t + 2.0 * p.cellsize / simscale
    hr = (box_max[1] - box_min[1]) * 0.5 if headroom is None else headroom
    for a in range(3):
        p.volmin[a] = box_min[a] - pad
        p.volmax[a] = box_max[a] + pad + (hr if a == 1 else 0.0)
    gen.setup_grid(p)
    return p


def _block(p, disp, calc, count, corner, counts, d, jitter, seed, phase=0, gen=LIBRARY):
    vmin = [corner[a] + 0.5 * d for a in range(3)]
    vmax = [vmin[a] + (counts[a] - 0.5) * d for a in range(3)]
    return gen.add_fluid_volume(p, disp, calc, count, vmin, vmax, d, phase=phase, jitter=jitter * d, seed=seed)


def _walls(p, disp, calc, count, box_min, box_max, d, layers=2, gen=LIBRARY):
    return gen.add_open_box(p, disp, calc, count, box_min, box_max, (layers - 0.5) * d)


def _assign_phase(p, calc, sel, phase):
    calc["restdens"][sel] = p.densArr[phase]
    calc["mass"][sel] = p.massArr[phase]
    calc["visc"][sel] = p.viscArr[phase]


def _finish(p, disp, calc, count, n_fluid, name):
    disp = disp[:count].copy()
    calc = calc[:count].copy()
    p.num = count
    p.maxNum = count
    return Scene(params=p, disp=disp, calc=calc, n_fluid=n_fluid, n_boundary=count - n_fluid, name=name)


def dam_break_2phase(seed=1, n_side=32, d=0.01, h=0.02, box=0.64, dt=2e-4, eos=abi.EOS_LINEAR, eos_k=3.0,
                     gas_center=(0.16, 0.10, 0.16), gas_radius=0.06, multiphase=1, walls=True, gen=LIBRARY):
    """32^3 liquid block with a gas sphere in a `box`-metre open box (liquid 1000, gas 1.2 kg/m^3)."""
    bmin, bmax = (0.0, 0.0, 0.0), (box, box, box)
    p = make_params(h=h, d=d, dt=dt, box_min=bmin, box_max=bmax, nphase=2, dens=(1000.0, 1.2), visc=(0.2, 0.2),
                    eos=eos, eos_k=eos_k, multiphase=multiphase, gen=gen)
    cap = n_side ** 3 + (int(6 * (box / d + 4) ** 2 * 2.2) if walls else 0)
    disp, calc = gen.record_arrays(cap)
    count = _block(p, disp, calc, 0, bmin, (n_side,) * 3, d, 0.1, seed, gen=gen)
    n_fluid = count
    pos = disp["pos"][:count]
    gas = np.sum((pos - np.asarray(gas_center, np.float32)) ** 2, axis=1) < gas_radius ** 2
    _assign_phase(p, calc, np.nonzero(gas)[0], 1)
    if walls:
        count = _walls(p, disp, calc, count, bmin, bmax, d, gen=gen)
    return _finish(p, disp, calc, count, n_fluid, f"dam_break_2phase_{n_side}")


def blobs_3phase(seed=2, lattice=(128, 64, 128), d=0.005, h=0.01, box=(1.28, 0.64, 0.64), dt=1e-4,
                 eos=abi.EOS_LINEAR, eos_k=3.0, n_blobs=64, rmin=0.02, rmax=0.08, multiphase=1, walls=True,
                 gen=LIBRARY):
    """A lattice block in the low-x corner of the box; phases 0/1/2 (1000/800/1.2 kg/m^3) from
    random blobs (the last blob containing a particle wins, phase 0 elsewhere)."""
    bmin, bmax = (0.0, 0.0, 0.0), tuple(box)
    p = make_params(h=h, d=d, dt=dt, box_min=bmin, box_max=bmax, nphase=3, dens=(1000.0, 800.0, 1.2),
                    visc=(0.2, 0.2, 0.2), eos=eos, eos_k=eos_k, multiphase=multiphase, gen=gen)
    wall_est = 0
    if walls:
        nx, ny, nz = [int(b / d) + 8 for b in box]
        wall_est = 2 * (nx * nz + 2 * nx * ny + 2 * nz * ny) + 4096
    cap = int(np.prod(lattice)) + wall_est
    disp, calc = gen.record_arrays(cap)
    count = _block(p, disp, calc, 0, bmin, lattice, d, 0.1, seed, gen=gen)
    n_fluid = count
    rng = np.random.default_rng(seed)
    ext = np.asarray(lattice, np.float32) * np.float32(d)
    centers = (rng.uniform(0.0, 1.0, size=(n_blobs, 3)) * ext).astype(np.float32)
    radii = rng.uniform(rmin, rmax, size=n_blobs).astype(np.float32)
    phases = rng.integers(0, 3, size=n_blobs)
    pos = disp["pos"][:count]
    phase = np.zeros(count, np.int64)
    for c, r, ph in zip(centers, radii, phases):  # the last blob containing a particle wins
        inside = np.sum((pos - c) ** 2, axis=1) < r * r
        phase[inside] = ph
    for k in range(3):
        _assign_phase(p, calc, np.nonzero(phase == k)[0], k)
    if walls:
        count = _walls(p, disp, calc, count, bmin, bmax, d, gen=gen)
    name = "blobs_3phase_" + "x".join(str(v) for v in lattice)
    return _finish(p, disp, calc, count, n_fluid, name)


def small_block(seed=3, n=(12, 10, 8), d=0.01, h=0.02, box=None, dt=2e-4, nphase=2, eos=abi.EOS_TAIT,
                dens=(1000.0, 1.2, 800.0), visc=(0.2, 0.05, 0.1), jitter=0.1, phase_frac=0.3, multiphase=1,
                walls=True, simscale=1.0, velocity_scale=0.0):
    """A small jittered block with random phases and (optionally) random velocities, for parity tests."""
    if box is None:
        box = tuple(max(n[a] * d * 1.5, 4 * h) for a in range(3))
    bmin, bmax = (0.0, 0.0, 0.0), tuple(box)
    p = make_params(h=h, d=d, dt=dt, box_min=bmin, box_max=bmax, nphase=nphase, dens=dens[:nphase],
                    visc=visc[:nphase], eos=eos, multiphase=multiphase, simscale=simscale)
    cap = int(np.prod(n)) + (int(2 * 2 * sum(box[a] * box[b] for a in range(3) for b in range(a + 1, 3))
                                 / d ** 2 * 1.6) + 2048 if walls else 0)
    disp, calc = record_arrays(cap)
    count = _block(p, disp, calc, 0, bmin, n, d, jitter, seed)
    n_fluid = count
    rng = np.random.default_rng(seed)
    if nphase > 1:
        ph = np.where(rng.random(count) < phase_frac, rng.integers(1, nphase, size=count), 0)
        for k in range(nphase):
            _assign_phase(p, calc, np.nonzero(ph == k)[0], k)
    if velocity_scale:
        calc["vel"][:count] = rng.normal(0, velocity_scale, size=(count, 3)).astype(np.float32)
        calc["veleval"][:count] = calc["vel"][:count]
    if walls:
        count = _walls(p, disp, calc, count, bmin, bmax, d)
    return _finish(p, disp, calc, count, n_fluid, "small_block")


def bubble_scene(seed, n_particles, d=0.01, h=0.02, dt=2e-4, eos=abi.EOS_LINEAR, eos_k=3.0, jitter=0.05,
                 multiphase=1):
    """One scene of the batched configuration: a near-cubic liquid lattice of about `n_particles` sites at
    spacing d with +-jitter*d jitter, 1-4 gas bubbles of radius U(3h, 8h) (liquid 1000, gas 1.2 kg/m^3),
    in an open box 1.5x the block."""
    rng = np.random.default_rng(seed)
    side = n_particles ** (1.0 / 3.0)
    nx = max(4, int(round(side)))
    nz = max(4, int(round(side)))
    ny = max(4, int(round(n_particles / (nx * nz))))
    box = tuple(max(c * d * 1.5, 4 * h) for c in (nx, ny, nz))
    bmin, bmax = (0.0, 0.0, 0.0), box
    p = make_params(h=h, d=d, dt=dt, box_min=bmin, box_max=bmax, nphase=2, dens=(1000.0, 1.2), visc=(0.2, 0.2),
                    eos=eos, eos_k=eos_k, multiphase=multiphase)
    cap = nx * ny * nz + int(2 * 2 * sum(box[a] * box[b] for a in range(3) for b in range(a + 1, 3)) / d ** 2 * 1.6) \
        + 2048
    disp, calc = record_arrays(cap)
    count = _block(p, disp, calc, 0, bmin, (nx, ny, nz), d, jitter, seed)
    n_fluid = count
    ext = np.array([nx, ny, nz], np.float32) * np.float32(d)
    pos = disp["pos"][:count]
    gas = np.zeros(count, bool)
    for _ in range(int(rng.integers(1, 5))):
        c = (rng.uniform(0.2, 0.8, 3) * ext).astype(np.float32)
        r = np.float32(rng.uniform(3 * h, 8 * h))
        gas |= np.sum((pos - c) ** 2, axis=1) < r * r
    _assign_phase(p, calc, np.nonzero(gas)[0], 1)
    count = _walls(p, disp, calc, count, bmin, bmax, d)
    return _finish(p, disp, calc, count, n_fluid, f"bubbles_{nx}x{ny}x{nz}")


def rollout_bubbles(seed=9, lattice=(256, 128, 128), d=0.005, h=0.01, dt=1e-4, n_bubbles=256, liquid_only=False,
                    eos=abi.EOS_LINEAR, eos_k=3.0):
    """The learned-corrector rollout scene: a lattice block (x, y, z sites at spacing d, +-0.05 d jitter) in
    the low corner of an open box 4h longer in x and z and 1.25x taller than the block, two phases
    (liquid 1000, gas 1.2 kg/m^3) with `n_bubbles` gas spheres of radius U(2h, 10h) centred uniformly in
    the block; `liquid_only` keeps every particle liquid (same lattice, no bubbles)."""
    rng = np.random.default_rng(seed)
    ext = np.asarray(lattice, np.float64) * d
    box = (float(ext[0] + 4 * h), float(ext[1] * 1.25), float(ext[2] + 4 * h))
    bmin = (0.0, 0.0, 0.0)
    p = make_params(h=h, d=d, dt=dt, box_min=bmin, box_max=box, nphase=2, dens=(1000.0, 1.2), visc=(0.2, 0.2),
                    eos=eos, eos_k=eos_k, multiphase=1)
    nx, ny, nz = [int(b / d) + 8 for b in box]
    cap = int(np.prod(lattice)) + 2 * (nx * nz + 2 * nx * ny + 2 * nz * ny) + 4096
    disp, calc = record_arrays(cap)
    count = _block(p, disp, calc, 0, bmin, lattice, d, 0.05, seed)
    n_fluid = count
    if not liquid_only:
        pos = disp["pos"][:count]
        gas = np.zeros(count, bool)
        centres = (rng.uniform(0.0, 1.0, size=(n_bubbles, 3)) * ext).astype(np.float32)
        radii = rng.uniform(2 * h, 10 * h, size=n_bubbles).astype(np.float32)
        for c, r in zip(centres, radii):
            gas |= np.sum((pos - c) ** 2, axis=1) < r * r
        _assign_phase(p, calc, np.nonzero(gas)[0], 1)
    count = _walls(p, disp, calc, count, bmin, box, d)
    name = ("liquid_" if liquid_only else "bubbles_") + "x".join(str(v) for v in lattice)
    return _finish(p, disp, calc, count, n_fluid, name)


def tile(scene_list, gap_cells=2):
    """Independent scenes in one domain, so that every pass covers all of them in one launch: each scene
    is moved into its own tile of a 3D arrangement (x fastest, then z, then y), tiles separated by
    `gap_cells` empty grid cells, all offsets whole multiples of the cell size. Every scene keeps its
    own grid padding (two cells outside its walls), so no particle of one scene is ever within h of
    another's. The scenes must share their physics (h, dt, phases, EOS, simscale); the combined grid
    covers every tile. One difference from running a scene alone: a particle that leaves its walls
    stays in the combined grid instead of reaching that scene's grid border. Returns the combined
    Scene and, per scene, (first record, record count, offset)."""
    p0 = scene_list[0].params
    cell = float(p0.cellsize) / float(p0.simscale)
    ext = np.array([[s.params.volmax[a] - s.params.volmin[a] for a in range(3)] for s in scene_list], np.float64)
    pitch = np.ceil(ext.max(axis=0) / cell) * cell + gap_cells * cell
    k = len(scene_list)
    nx = int(np.ceil(k ** (1.0 / 3.0) - 1e-9))
    nz = nx
    disp_all, calc_all, layout = [], [], []
    first = 0
    n_fluid = 0
    for i, s in enumerate(scene_list):
        ix, iz, iy = i % nx, (i // nx) % nz, i // (nx * nz)
        corner = np.array([ix, iy, iz], np.float64) * pitch
        off = (corner - np.array([s.params.volmin[a] for a in range(3)], np.float64))
        off = (np.round(off / cell) * cell).astype(np.float32)
        d = s.disp.copy()
        c = s.calc.copy()
        d["pos"] += off
        c["bornid"] += first
        disp_all.append(d)
        calc_all.append(c)
        layout.append((first, len(d), off))
        first += len(d)
        n_fluid += s.n_fluid
    disp = np.concatenate(disp_all)
    calc = np.concatenate(calc_all)
    p = p0.copy()
    lo = np.min([np.array([s.params.volmin[a] for a in range(3)]) + o for s, (_, _, o) in zip(scene_list, layout)],
                axis=0)
    hi = np.max([np.array([s.params.volmax[a] for a in range(3)]) + o for s, (_, _, o) in zip(scene_list, layout)],
                axis=0)
    for a in range(3):
        p.volmin[a] = lo[a]
        p.volmax[a] = hi[a]
    setup_grid(p)
    p.num = len(disp)
    p.maxNum = len(disp)
    return Scene(params=p, disp=disp, calc=calc, n_fluid=n_fluid, n_boundary=len(disp) - n_fluid,
                 name=f"tiled_{k}"), layout
