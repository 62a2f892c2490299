"""Scene builders shared by the tests (reference buffer layouts)."""
from __future__ import annotations

import numpy as np

from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo


def scene(positions, n_side_box: int = 8, *, bonds=(), conc=None, genes=None, vel=None,
          param: str = "R", genome=None, max_points=None):
    """Particles at `positions` (world units) inside the box of an n_side_box block.

    bonds: iterable of (i, a, j, L0, modulus, damping, elastlim); the incoming table of j gets
    (i, a) in slot a ^ 1.
    """
    pos_in = np.asarray(positions, np.float32).reshape(-1, 3)
    n = len(pos_in)
    cap = max_points or n
    p = demo.make_params(n_side_box, param)
    g = genome if genome is not None else demo.make_genome(seed=1)
    pos = np.zeros((cap, 4), np.float32)
    pos[:n, :3] = pos_in
    if cap > n:
        pos[n:, 0] = p.pboundmin[0]
        pos[n:, 1] = p.pboundmin[1]
        pos[n:, 2] = np.float32(p.pboundmin[2]) - np.float32(2 * p.grid_res[2])
    el = np.zeros((cap, 6, 9), np.uint32)
    elf = el.view(np.float32)
    el[:, :, 0] = A.NO_PARTNER
    el[:, :, 5] = A.NO_PARTNER
    pidx = np.full((cap, 12), A.NO_PARTNER, np.uint32)
    for (i, a, j, L0, mod, damp, lim) in bonds:
        el[i, a, 0] = j
        elf[i, a, 1] = lim
        elf[i, a, 2] = L0
        elf[i, a, 3] = mod
        elf[i, a, 4] = damp
        el[i, a, 5] = j + 1
        pidx[j, 2 * (a ^ 1)] = i
        pidx[j, 2 * (a ^ 1) + 1] = a
    c = np.zeros((cap, A.NUM_TF), np.float32)
    if conc is not None:
        c[:n] = np.asarray(conc, np.float32).reshape(n, A.NUM_TF)
    ep = np.zeros((A.NUM_GENES, cap), np.uint32)
    if genes is not None:
        for k, bits in enumerate(genes):
            for gg in range(A.NUM_GENES):
                if (bits >> gg) & 1:
                    ep[gg, k] = A.EPIGEN_ACTIVE
    v = np.zeros((cap, 4), np.float32)
    if vel is not None:
        v[:n, :3] = np.asarray(vel, np.float32).reshape(n, 3)
    arrays = {A.FPOS: pos, A.FVEL: v, A.FVEVAL: v.copy(), A.FELASTIDX: el.reshape(cap, 54),
              A.FPARTICLEIDX: pidx, A.FCONC: c, A.FEPIGEN: ep,
              A.FPARTICLE_ID: np.where(np.arange(cap) < n, np.arange(cap) + 1, A.NO_PARTNER).astype(np.uint32)}
    return demo.Demo(n_side=n_side_box, params=p, genome=g, arrays=arrays, n_particles=cap), cap


def box_centre(n_side_box: int = 8) -> float:
    return float(demo.make_params(n_side_box, "R").pboundmax[0]) / 2
