"""Stage sequence shared by the reference-pin fixture generator and its tests.

`run_stages` drives one scene through bin, scan, sort, pressure, force, diffusion and advance
on any implementation with the stage methods (the reference harness, the oracle, the GPU
façade) and returns, per stage, the SHA-256 of each bit-exact output buffer and the FFORCE
array (compared within tolerance).  `run` maps a stage name to a call on the implementation;
`download(buf)` reads a buffer in the reference layout; `set_force(arr)` makes the
integration start from the given forces.
"""
from __future__ import annotations

import hashlib

import numpy as np

from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo

def pin_genome():
    """The regulatory genome of the demos with integer diffusability 1 and breakdown rate 1:
    the reference's genome fields are integers (fluid.h FGenome)."""
    return demo.make_genome(seed=1, diffusion=1.0, decay=0.0)


def scene(kind: str, side: int = 16):
    """Blocks of side^3 particles: 'R', 'L' (the two parameterisations), and 'R-strained'
    (extra jitter of +-0.35 spacing so that some bonds exceed 1.5 x rest length and break,
    random velocities for the damping and velocity-limit terms, block moved against the low
    walls so the wall terms act)."""
    param = "L" if kind == "L" else "R"
    d = demo.make_block(side, param, seed=3 if kind == "R-strained" else 0, breakable=True,
                        genome=pin_genome())
    if kind == "R-strained":
        r = np.random.default_rng(7)
        pos = d.arrays[A.FPOS]
        pos[:, :3] += r.uniform(-0.35, 0.35, (d.n, 3)).astype(np.float32)
        lo = np.float32(d.params.pboundmin[0]) + np.float32(0.005)
        pos[:, :3] -= pos[:, :3].min(0) - lo
        v = r.uniform(-2.0, 2.0, (d.n, 4)).astype(np.float32)
        v[:, 3] = 0
        d.arrays[A.FVEL] = v
        d.arrays[A.FVEVAL] = (v * np.float32(0.9)).astype(np.float32)
    return d


STAGE_BUFS = {
    "insert": (A.FGCELL, A.FGNDX, A.FBIN_COUNT),
    "scan": (A.FBIN_OFFSET,),
    "sort": (A.FPOS, A.FVEL, A.FVEVAL, A.FGCELL, A.FGNDX, A.FPARTICLE_ID, A.FMASS_RADIUS,
             A.FNERVEIDX, A.FAGE, A.FCOLOR, A.FCONC, A.FEPIGEN, A.FPARTICLEIDX, A.FELASTIDX),
    "pressure": (A.FPRESS, A.FDENSITY),
    "force": (A.FELASTIDX,),
    "diffusion": (A.FCONC,),
    "advance": (A.FPOS, A.FVEL, A.FVEVAL),
}
ORDER = ("insert", "scan", "sort", "pressure", "force", "diffusion", "advance")


def canonical(buf: int, a: np.ndarray) -> np.ndarray:
    """Bits of a buffer with the reference's "no partner" 65535 written as 0xFFFFFFFF (bond
    partners, incoming-bond entries) and the float4 padding word of positions and velocities
    cleared."""
    a = np.array(a, copy=True)
    if a.dtype == np.float32:
        a = a.view(np.uint32)
    if buf == A.FPARTICLEIDX:
        a[a == 65535] = A.NO_PARTNER
    if buf == A.FELASTIDX:
        e = a.reshape(-1, 6, 9)
        w0 = e[:, :, 0]
        w0[w0 == 65535] = A.NO_PARTNER
    if buf in (A.FPOS, A.FVEL, A.FVEVAL, A.FFORCE):
        a.reshape(-1, 4)[:, 3] = 0
    return a


def digest(buf: int, a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(canonical(buf, a)).tobytes()).hexdigest()


def run_stages(run, download, set_force, advance_force) -> dict:
    """Runs the stages in ORDER; before "advance", set_force(advance_force) gives the
    integration the canonical forces (the oracle's gathered sums, D2), so that every
    implementation integrates from the same input."""
    out = {}
    for st in ORDER:
        if st == "advance":
            set_force(advance_force)
        run(st)
        rec = {str(b): digest(b, download(b)) for b in STAGE_BUFS[st]}
        if st == "force":
            rec["FFORCE"] = np.array(download(A.FFORCE), np.float32)[:, :3].copy()
        out[st] = rec
    return out
