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


CHANGE_BUFS = [A.FBIN_COUNT_CHANGES, A.FBIN_OFFSET_CHANGES, A.FDENSE_LIST_LENGTHS_CHANGES,
               A.FDENSE_LISTS_CHANGES]


def moving_tissue(seed):
    """A breakable, moving block, mostly living, with tissue genes (tendon, muscle, bone,
    elastic ligament) at random."""
    d = demo.make_block(7, "R", seed=seed, breakable=True)
    r = np.random.default_rng(seed)
    v = r.uniform(-30, 30, (d.n, 4)).astype(np.float32)
    v[:, 3] = 0
    d.arrays[A.FVEL] = v
    d.arrays[A.FVEVAL] = v.copy()
    ep = d.arrays[A.FEPIGEN]
    ep[2] = np.where(r.random(d.n) < 0.8, A.EPIGEN_ACTIVE, 0)
    for gene, share in ((6, 0.2), (7, 0.2), (9, 0.2), (10, 0.1)):
        ep[gene] = np.where(r.random(d.n) < share, A.EPIGEN_ACTIVE, 0)
    return d


@pytest.mark.parametrize("seed", range(4))
def test_random_sequences_with_remodelling(built, seed):
    """Remodelling tissues: steps with bond changes and heal, the Run2 loop's pieces
    (PhysicalSort, InnerPhysicalLoop, GeneAction, Remodelling), uploads of FELASTIDX that break
    or remove bonds, of FEPIGEN with countdowns (the full epigenetic state), ZeroVel; every
    buffer and the change lists against the oracle after each operation."""
    import morphogenesis_gb300 as mg

    r = np.random.default_rng(2000 + seed)
    d = moving_tissue(seed)
    g = mg.FluidSystem(d.params, d.genome, d.n)
    o = orc.Oracle(d.params, d.genome, d.n)
    g.TransferToCL(d.arrays)
    o.upload_all(d.arrays)
    log = []
    g.Run(1)
    o.step(1)
    for k in range(8):
        op = int(r.integers(0, 7))
        if op == 0:
            n = int(r.integers(1, 4))
            fl = [A.STEP_DEFAULT | A.STEP_BOND_CHANGES, A.STEP_DEFAULT | A.STEP_REMODEL,
                  A.STEP_PHYSICS | A.STEP_REMODEL][int(r.integers(0, 3))]
            g.Run(n, fl)
            o.step(n, fl)
            log.append(f"run {n} flags {fl}")
        elif op == 1:
            inner = int(r.integers(1, 4))
            g.Run2PhysicalSort()
            o.insert(); o.prefix_sum(); o.sort()
            for _ in range(inner):
                g.Run2InnerPhysicalLoop()
                o.pressure(); o.force(); o.advance()
            g.Run2GeneAction()
            o.diffusion(); o.genes()
            g.Run2Remodelling(inner)
            o.bond_changes(inner); o.remodel()
            log.append(f"run2 cycle {inner}")
        elif op == 2:
            e0 = g.download(A.FELASTIDX)
            e = e0.reshape(-1, 6, 9)  # a view of e0: [particle][bond][word]
            pick = r.random(e.shape[:2])
            e[pick < 0.05, 2] = np.float32(0).view(np.uint32)        # rest length 0: broken
            e[(pick >= 0.05) & (pick < 0.08), 0] = A.NO_PARTNER       # no partner
            g.upload(A.FELASTIDX, e0)
            o.upload(A.FELASTIDX, e0)
            log.append("upload FELASTIDX")
        elif op == 3:
            ep = g.download(A.FEPIGEN)
            pick = r.random(ep.shape)
            ep[pick < 0.05] = r.integers(1, 6, ep.shape)[pick < 0.05].astype(np.uint32)
            g.upload(A.FEPIGEN, ep)
            o.upload(A.FEPIGEN, ep)
            log.append("upload FEPIGEN")
        elif op == 4:
            g.ZeroVelCL()
            z = np.zeros((d.n, 4), np.float32)
            o.upload(A.FVEL, z)
            o.upload(A.FVEVAL, z)
            log.append("zero velocities")
        elif op == 5:
            g.Run(2)
            o.step(2)
            log.append("run 2")
        else:
            g.set_option(A.OPT_REORIGIN_PERIOD, int(r.choice([0, 1, 3])))
            log.append("re-origin period")
        what = f"seed {seed}, after " + "; ".join(log)
        check(g, o, what)
        for b in CHANGE_BUFS:
            assert np.array_equal(g.download(b), o.download(b)), f"{what}: change buffer {b}"
    g.close()
    o.close()


@pytest.mark.parametrize("seed", range(3))
def test_random_sequences_packed_instances(built, seed):
    """Packed instances against the same tissues as systems of their own under random steps
    (physics, genes only, both, frozen bonds), position nudges and drops applied to both, and
    re-origin periods: every instance's sorted segment bit for bit equal to its own system's
    active particles after each operation."""
    import morphogenesis_gb300 as mg

    r = np.random.default_rng(3000 + seed)
    ds = []
    for k in range(4):
        side = int(r.integers(4, 9))
        g0 = demo.make_genome(seed=40 + k, diffusion=demo.diffusion_rate("R", float(r.uniform(0.05, 0.2))))
        ds.append(demo.make_block(side, "R", seed=seed * 10 + k, genome=g0,
                                  intstiff=float(r.uniform(0.5, 2.0)), breakable=bool(k % 2)))
    pk = mg.Packed([d.params for d in ds], [d.genome for d in ds], [d.n for d in ds])
    pk.TransferToCL(pk.concat([d.arrays for d in ds]))
    alone = []
    for d in ds:
        fs = mg.FluidSystem(d.params, d.genome, d.n)
        fs.TransferToCL(d.arrays)
        alone.append(fs)
    bufs = (A.FPOS, A.FVEL, A.FVEVAL, A.FFORCE, A.FPRESS, A.FDENSITY, A.FCONC, A.FELASTIDX,
            A.FPARTICLEIDX, A.FPARTICLE_ID, A.FEPIGEN)
    log = []
    pk.Run(1)
    for fs in alone:
        fs.Run(1)
    for step in range(6):
        op = int(r.integers(0, 4))
        if op <= 1:
            n = int(r.integers(1, 4))
            fl = FLAGS[int(r.integers(0, 4))]
            pk.Run(n, fl)
            for fs in alone:
                fs.Run(n, fl)
            log.append(f"run {n} flags {fl}")
        elif op == 2:
            drop = bool(r.integers(0, 2))
            ppos = pk.download(A.FPOS)
            for (f, c), fs in zip(pk.ranges(), alone):
                apos = fs.download(A.FPOS)
                sel = np.nonzero(r.random(c) < (0.08 if drop else 0.2))[0]
                if drop:
                    apos[sel, 0] = np.float32(-1e4)
                else:
                    apos[sel, :3] += r.uniform(-0.2, 0.2, (len(sel), 3)).astype(np.float32)
                ppos[f + sel] = apos[sel]
                fs.upload(A.FPOS, apos)
            pk.upload(A.FPOS, ppos)
            log.append("drop" if drop else "nudge")
        else:
            period = int(r.choice([0, 1, 64]))
            pk.set_option(A.OPT_REORIGIN_PERIOD, period)
            for fs in alone:
                fs.set_option(A.OPT_REORIGIN_PERIOD, int(r.choice([0, 1, 64])))
            log.append("re-origin periods")
        what = f"seed {seed}, after " + "; ".join(log)
        ranges = pk.ranges()
        for b in bufs:
            parts = pk.split(b)
            for k, fs in enumerate(alone):
                x, y = bits(parts[k]), bits(fs.download(b))
                c = ranges[k][1]
                assert fs.counts()[0] == c, f"{what}: instance {k} holds {fs.counts()[0]} particles alone, {c} packed"
                y = y[:, :c] if b == A.FEPIGEN else y[:c]
                assert np.array_equal(x, y), f"{what}: instance {k}, buffer {b}"
    pk.close()
    for fs in alone:
        fs.close()
