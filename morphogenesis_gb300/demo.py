"""Seeded synthetic tissue blocks in the reference buffer layouts (the role of the
reference's SetupAddVolumeMorphogenesis2 + WriteDemoSimParams, fluid_system.cpp:1037-1167 and
fileCL_IO.cpp:636-740).

A block is an n x n x n jittered cubic lattice with elastic bonds to its six lattice
neighbours, 16 morphogen concentrations and 16 gene states per particle, inside a walled box
four times the block extent.  Two parameterisations share positions, grid and memory traffic:

* ``"L"`` (literal): simulation scale 0.005, smoothing radius h = 0.01, spacing 0.5 h.
* ``"R"`` (reference-consistent): simulation scale 1, smoothing radius 2.0, spacing 1.0 --
  the same world-unit geometry with the scale the reference's own demos use
  (src/demo/SpecificationFile.txt), so that the kernels' mixed world/simulation-unit
  comparisons (computePressure r2, computeForce dsq < 1) see neighbours.  computeDiffusion
  weights each neighbour by (r2 - dsq) * simscale^2 (cuda:3053), so with simscale 1 the
  diffusion rate is rescaled by 0.005^2 to keep the literal configuration's per-step
  exchange (a rate of 0.1 with weights of order 1 over ~30 neighbours is an unstable
  explicit scheme and overflows within 60 steps).

The grid cell is 2h with a 27-cell (gsrch = 3) search window; the grid volume extends two
cells beyond the walls on every side, as SetupSpacing places the walls (fluid_system.cpp:2536-2541).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _abi as A

PURPOSE_JITTER, PURPOSE_CONC, PURPOSE_GENES, PURPOSE_TABLE = 0, 1, 2, 3


@dataclass
class Demo:
    n_side: int | tuple
    params: A.FParams
    genome: A.Genome
    arrays: dict = field(default_factory=dict)  # buffer id -> numpy array (reference layout)
    n_particles: int = 0

    @property
    def n(self) -> int:
        return self.n_particles


def dims_of(n_side) -> tuple:
    """(nx, ny, nz) of a block given as an edge length or a triple."""
    if isinstance(n_side, (tuple, list)):
        return tuple(int(v) for v in n_side)
    return (int(n_side),) * 3


def rng(seed: int, purpose: int) -> np.random.Generator:
    return np.random.default_rng([int(seed), int(purpose)])


def make_params(n_side: int, parameterisation: str = "R", *, dt: float = 1e-3,
                intstiff: float = 1.0) -> A.FParams:
    if parameterisation == "L":
        ss, sr = 0.005, 0.01
    elif parameterisation == "R":
        ss, sr = 1.0, 2.0
    else:
        raise ValueError("parameterisation must be 'L' or 'R'")
    spacing = 1.0                       # world units in both
    cell_world = 2.0 * (sr / ss)        # grid cell 2h
    extent = max(dims_of(n_side)) * spacing
    box = 4.0 * extent                  # cubic box, four times the largest block extent
    p = A.FParams()
    p.psimscale = ss
    p.psmoothradius = sr
    p.pradius = 0.015                   # SetupDefaultParams (fluid_system.cpp:2183)
    p.pmass = 2.0543e-4
    p.prest_dens = 600.0
    p.pextstiff = 50000.0
    p.pintstiff = intstiff
    p.pvisc = 0.2
    p.psurface_t = 0.1
    p.pdamp = 100.0
    p.pforce_min = 0.0
    p.pforce_max = 0.0
    p.pforce_freq = 16.0
    p.pground_slope = 0.0
    p.pgravity[:] = (0.0, -9.8, 0.0)
    p.paccel_limit = 150.0
    p.pvel_limit = 3.0
    p.actuation_factor = 0.0
    p.actuation_period = 1.0
    p.pboundmin[:] = (0.0, 0.0, 0.0)
    p.pboundmax[:] = (box, box, box)
    vmin = (A.C.c_float * 3)(*(-2 * cell_world,) * 3)
    vmax = (A.C.c_float * 3)(*(box + 2 * cell_world,) * 3)
    p.dt = dt
    p.time = 0.0
    p.freeze = 0
    # SetupGrid with the cell size in simulation units; gsrch = 3 through FluidSetupCL's gsrch
    setup_grid(p, vmin, vmax, cell_world * ss, 3)
    return p


def setup_grid(p: A.FParams, vmin, vmax, cell_size: float, gsrch: int) -> None:
    """SetupGrid (fluid_system.cpp:2073-2131) in float32, as mg_setup_grid computes it."""
    f = np.float32
    ss = f(p.psimscale)
    world = f(cell_size) / ss
    total = 1
    for k in range(3):
        p.grid_min[k] = vmin[k]
        p.grid_max[k] = vmax[k]
        size = f(vmax[k]) - f(vmin[k])
        res = int(np.ceil(size / world))
        p.grid_res[k] = res
        gsize = f(res) * f(cell_size) / ss
        p.grid_size[k] = gsize
        p.grid_delta[k] = f(res) / f(gsize)
        total *= res
    p.grid_total = total
    srch = int(np.floor(f(2.0) * (f(p.psmoothradius) / ss) / world) + 1.0)
    p.grid_srch = gsrch if gsrch > 0 else max(srch, 2)


def diffusion_rate(parameterisation: str, rate: float = 0.1) -> float:
    """Genome diffusability giving the literal configuration's per-step exchange."""
    return rate if parameterisation == "L" else rate * 0.005 * 0.005


def make_genome(seed: int = 1, diffusion: float = 0.1, decay: float = 0.01,
                secretion: float = 0.004, density: float = 0.25) -> A.Genome:
    """Signed 16x16 regulatory table (25 % nonzero, U[-1,1]); gene g secretes species g."""
    g = A.Genome()
    r = rng(seed, PURPOSE_TABLE)
    mask = r.random((A.NUM_GENES, A.NUM_TF)) < density
    w = r.uniform(-1.0, 1.0, (A.NUM_GENES, A.NUM_TF)).astype(np.float32)
    table = np.where(mask, w, np.float32(0.0)).astype(np.float32)
    for a in range(A.NUM_GENES):
        for t in range(A.NUM_TF):
            g.sensitivity[a][t] = float(table[a, t])
        g.secrete[a][0] = float(a)
        g.secrete[a][1] = secretion
        g.secrete[a][2 * A.NUM_TF] = 1.0
        g.activate[a][2 * A.NUM_GENES] = 0.0
        g.delay[a] = 0
    for t in range(A.NUM_TF):
        g.tf_diffusability[t] = diffusion
        g.tf_breakdown_rate[t] = 1.0 - decay
    # bond parameters for re-formed bonds: [elastLim, rest length, modulus, damping] at 8..11
    for k in range(3):
        g.param[k][8] = 1.5
        g.param[k][9] = 1.0
        g.param[k][10] = 1000.0
        g.param[k][11] = 10.0
    # computeBondChanges' shifted tanh per bond type (elastin, collagen, apatite):
    # rest length *= l_a + l_b tanh(l_c strain - l_d), modulus *= s_a + s_b tanh(s_c strain^2 - s_d)
    for k, (lb, lc, ld, sb, sc, sd) in enumerate(((0.01, 10.0, 0.7, 0.02, 5.0, 0.5),
                                                  (0.005, 8.0, 1.0, 0.03, 4.0, 0.25),
                                                  (0.002, 6.0, 2.0, 0.01, 3.0, 1.0))):
        g.tanh_param[k][:] = [1.0, lb, lc, ld, 1.0, sb, sc, sd]
    return g


def make_block(n_side: int, parameterisation: str = "R", seed: int = 0, *,
               breakable: bool = False, genome: A.Genome | None = None,
               intstiff: float = 1.0, max_points: int | None = None) -> Demo:
    """A jittered n^3 lattice centred in its box, in the reference buffer layouts.

    Bonds get rest length = initial distance, modulus 1e3, damping 10 and an elastic limit of
    1.5 x rest length when ``breakable`` (bonds break at strain > 0.5), else 1e30.
    """
    p = make_params(n_side, parameterisation, intstiff=intstiff)
    g = genome if genome is not None else make_genome(seed=1, diffusion=diffusion_rate(parameterisation))
    nx, ny, nz = dims_of(n_side)
    n = nx * ny * nz
    cap = max_points or n
    spacing = np.float32(1.0)
    box = float(p.pboundmax[0])
    ix = np.arange(n, dtype=np.int64)
    x, y, z = ix % nx, (ix // nx) % ny, ix // (nx * ny)
    jit = rng(seed, PURPOSE_JITTER).uniform(-0.05, 0.05, (n, 3)).astype(np.float32) * spacing
    pos = np.zeros((cap, 4), np.float32)
    for k, (c, m) in enumerate(((x, nx), (y, ny), (z, nz))):
        origin = np.float32(box / 2 - (m - 1) * 0.5 * spacing)
        pos[:n, k] = origin + c.astype(np.float32) * spacing + jit[:, k]
    if cap > n:  # unused slots parked outside the grid like the reference's null points
        pos[n:, 0] = p.pboundmin[0]
        pos[n:, 1] = p.pboundmin[1]
        pos[n:, 2] = np.float32(p.pboundmin[2]) - np.float32(2 * p.grid_res[2])

    pid = np.full(cap, A.NO_PARTNER, np.uint32)
    pid[:n] = (ix + 1).astype(np.uint32)
    # bonds: slot a -> neighbour in direction a (+x,-x,+y,-y,+z,-z); partner's incoming slot a^1
    el = np.zeros((cap, 6, 9), np.uint32)
    elf = el.view(np.float32)
    el[:, :, 0] = A.NO_PARTNER
    el[:, :, 5] = A.NO_PARTNER
    pidx = np.full((cap, 12), A.NO_PARTNER, np.uint32)
    coords = np.stack([x, y, z], 1)
    dirs = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    for a, d in enumerate(dirs):
        nb = coords + np.array(d)
        ok = np.all((nb >= 0) & (nb < np.array([nx, ny, nz])), axis=1)
        i = ix[ok]
        j = (nb[ok, 0] + nx * (nb[ok, 1] + ny * nb[ok, 2])).astype(np.int64)
        d3 = pos[i, :3] - pos[j, :3]
        L0 = np.sqrt((d3.astype(np.float32) ** 2).sum(1)).astype(np.float32)
        el[i, a, 0] = j.astype(np.uint32)
        elf[i, a, 1] = (np.float32(1.5) * L0) if breakable else np.float32(1e30)
        elf[i, a, 2] = L0
        elf[i, a, 3] = np.float32(1000.0)
        elf[i, a, 4] = np.float32(10.0)
        el[i, a, 5] = pid[j]
        elf[i, a, 6] = 0.0
        elf[i, a, 7] = 0.0
        el[i, a, 8] = 0
        pidx[j, 2 * (a ^ 1)] = i.astype(np.uint32)
        pidx[j, 2 * (a ^ 1) + 1] = a
    conc = np.zeros((cap, A.NUM_TF), np.float32)
    conc[:n] = rng(seed, PURPOSE_CONC).random((n, A.NUM_TF), dtype=np.float32)
    bits = rng(seed, PURPOSE_GENES).random((A.NUM_GENES, n)) < 0.5
    epigen = np.zeros((A.NUM_GENES, cap), np.uint32)
    epigen[:, :n] = np.where(bits, np.uint32(A.EPIGEN_ACTIVE), np.uint32(0))
    mr = np.uint32((int(np.float32(p.pmass) * 255 * 255) << 16) | int(np.float32(p.pradius) * 255 * 255))
    arrays = {
        A.FPOS: pos,
        A.FVEL: np.zeros((cap, 4), np.float32),
        A.FVEVAL: np.zeros((cap, 4), np.float32),
        A.FELASTIDX: el.reshape(cap, A.BOND_DATA),
        A.FPARTICLEIDX: pidx,
        A.FCONC: conc,
        A.FEPIGEN: epigen,
        A.FPARTICLE_ID: pid,
        A.FAGE: np.zeros(cap, np.uint32),
        A.FCOLOR: np.full(cap, 0xFF3366CC, np.uint32),
        A.FMASS_RADIUS: np.where(np.arange(cap) < n, mr, np.uint32(0)).astype(np.uint32),
        A.FNERVEIDX: np.where(pid % 10 == 0, pid // 10, 0).astype(np.uint32),
    }
    return Demo(n_side=n_side, params=p, genome=g, arrays=arrays, n_particles=cap)
