"""Random sequences of operations on small tissues, the CUDA path (through the C-ABI) against
the oracle after every operation, bit for bit.

Each sequence starts from a seeded block (5-8 particles a side, breakable bonds in half of
them) and applies eight operations drawn from: whole steps with a random flag set (physics,
genes, both, frozen bonds, remodelling), the stages one by one in the reference's order
(insertParticles, prefixSum, countingSortFull, computePressure, computeForce,
computeDiffusion, advanceParticles), an upload of FPOS that nudges some particles, drops some
out of the grid or gives parked slots positions again, an upload of FCONC, and on the GPU side
only a new re-origin period or a run of the autotuner (neither may change a result).
"""
import numpy as np
import pytest

import oracle as orc
from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo

pytestmark = pytest.mark.gpu

BUFS = [A.FPOS, A.FVEL, A.FVEVAL, A.FFORCE, A.FPRESS, A.FDENSITY, A.FCONC, A.FELASTIDX,
        A.FPARTICLEIDX, A.FPARTICLE_ID, A.FEPIGEN, A.FAGE, A.FCOLOR, A.FMASS_RADIUS, A.FNERVEIDX,
        A.FGCELL, A.FGNDX]
FLAGS = [A.STEP_DEFAULT, A.STEP_PHYSICS, A.STEP_GENES, A.STEP_DEFAULT | A.STEP_FREEZE,
         A.STEP_DEFAULT | A.STEP_REMODEL]


def bits(a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        a = np.where(np.isnan(a), np.float32(np.nan), a)  # one NaN pattern
        return a.view(np.uint32)
    return a


def check(g, o, what):
    for b in BUFS:
        x, y = bits(g.download(b)), bits(o.download(b))
        assert np.array_equal(x, y), f"{what}: buffer {b} differs in {np.count_nonzero(x != y)} words"
    assert g.counts()[0] == o.counts()[0], what


@pytest.mark.parametrize("seed", range(6))
def test_random_operation_sequences(built, seed):
    import morphogenesis_gb300 as mg

    r = np.random.default_rng(1000 + seed)
    side = int(r.integers(5, 9))
    d = demo.make_block(side, "R", seed=seed, breakable=bool(seed % 2))
    g = mg.FluidSystem(d.params, d.genome, d.n)
    o = orc.Oracle(d.params, d.genome, d.n)
    g.TransferToCL(d.arrays)
    o.upload_all(d.arrays)
    box = float(d.params.pboundmax[0])
    sorted_once = False
    log = []
    for k in range(8):
        op = int(r.integers(0, 8))
        if op in (0, 1, 2) or not sorted_once:
            n, fl = int(r.integers(1, 4)), FLAGS[int(r.integers(0, len(FLAGS)))]
            g.Run(n, fl)
            o.step(n, fl)
            sorted_once = True
            log.append(f"run {n} flags {fl}")
        elif op == 3:
            for gs, os_ in ((g.InsertParticlesCL, o.insert), (g.PrefixSumCellsCL, o.prefix_sum),
                            (g.CountingSortFullCL, o.sort), (g.ComputePressureCL, o.pressure),
                            (g.ComputeForceCL, o.force), (g.ComputeDiffusionCL, o.diffusion),
                            (g.AdvanceCL, o.advance)):
                gs()
                os_()
            log.append("stages")
        elif op == 4:
            pos = g.download(A.FPOS)
            nact = g.counts()[0]
            kind = int(r.integers(0, 3))
            if kind == 0:  # nudge a few
                sel = r.random(len(pos)) < 0.2
                pos[sel, :3] += r.uniform(-0.3, 0.3, (int(sel.sum()), 3)).astype(np.float32)
            elif kind == 1:  # drop a few out of the grid
                sel = r.random(len(pos)) < 0.1
                pos[sel, 0] = np.float32(-1e4)
            elif nact < len(pos):  # give parked slots positions again
                m = len(pos) - nact
                pos[nact:, :3] = pos[:m, :3] + np.float32(0.41)
            g.upload(A.FPOS, pos)
            o.upload(A.FPOS, pos)
            log.append(f"upload FPOS kind {kind}")
        elif op == 5:
            c = r.random((d.n, 16)).astype(np.float32)
            g.upload(A.FCONC, c)
            o.upload(A.FCONC, c)
            log.append("upload FCONC")
        elif op == 6:
            g.set_option(A.OPT_REORIGIN_PERIOD, int(r.choice([0, 1, 2, 64])))
            log.append("re-origin period")
        else:
            g.autotune(2)
            log.append("autotune")
        check(g, o, f"seed {seed}, after " + "; ".join(log))
        assert np.isfinite(g.download(A.FPOS)[: g.counts()[0], :3]).all() or box <= 0
    g.close()
    o.close()
