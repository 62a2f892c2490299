"""Batched instances: one graph launch per step advances several independent systems of
different sizes, parameters and genomes; each must end bit-for-bit where it ends when stepped
alone."""
import numpy as np
import pytest

import morphogenesis_gb300 as mg
from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo

pytestmark = pytest.mark.gpu

BUFS = (A.FPOS, A.FVEL, A.FVEVAL, A.FCONC, A.FELASTIDX, A.FPARTICLEIDX, A.FPARTICLE_ID, A.FEPIGEN)


def instance(k):
    r = np.random.default_rng(100 + k)
    side = int(r.integers(6, 14))
    g = demo.make_genome(seed=10 + k, diffusion=demo.diffusion_rate("R", float(r.uniform(0.05, 0.2))))
    return demo.make_block(side, "R", seed=k, genome=g, intstiff=float(r.uniform(0.5, 2.0)),
                           breakable=bool(k % 2))


def test_batch_equals_members_stepped_alone(built):
    ds = [instance(k) for k in range(5)]
    alone, batched = [], []
    for d in ds:
        for lst in (alone, batched):
            fs = mg.FluidSystem(d.params, d.genome, d.n)
            fs.TransferToCL(d.arrays)
            lst.append(fs)
    batched[2].Run(1)  # members need not be in the same buffer state
    alone[2].Run(1)
    b = mg.Batch(batched)
    flags = A.STEP_DEFAULT | A.STEP_REMODEL
    b.Run(7, flags)
    b.Run(5)
    for fs in alone:
        fs.Run(7, flags)
        fs.Run(5)
    for k, (x, y) in enumerate(zip(alone, batched)):
        for buf in BUFS:
            assert np.array_equal(x.download(buf).view(np.uint32), y.download(buf).view(np.uint32)), \
                f"instance {k} buffer {buf}"
    ms = b.time_steps(3)
    assert ms > 0
    batched[0].Run(1)  # a member's own stream is ordered after the batch
    b.close()


def test_batch_follows_member_changes(built):
    """Members whose genome, parameters or options change between batch steps: the batch steps
    them with the new values (its steps are captured anew), bit-equal to twins stepped alone
    with the same changes."""
    ds = [instance(k) for k in range(4)]
    alone, batched = [], []
    for d in ds:
        for lst in (alone, batched):
            fs = mg.FluidSystem(d.params, d.genome, d.n)
            fs.TransferToCL(d.arrays)
            lst.append(fs)
    b = mg.Batch(batched)
    b.Run(4)
    for fs in alone:
        fs.Run(4)
    g = demo.make_genome(seed=77, diffusion=demo.diffusion_rate("R", 0.15))
    p = ds[1].params
    p.pintstiff = 1.7
    for group in (alone, batched):
        group[0].UpdateGenome(g)
        group[1].UpdateParams(p)
        group[2].set_option(A.OPT_NEIGHBOR_SEARCH, 0)
        group[3].SetParam(A.PVISC, 0.35)
    b.Run(6)
    for fs in alone:
        fs.Run(6)
    for k, (x, y) in enumerate(zip(alone, batched)):
        for buf in BUFS:
            assert np.array_equal(x.download(buf).view(np.uint32), y.download(buf).view(np.uint32)), \
                f"instance {k} buffer {buf} after a change between batch steps"
    b.Run(2)  # no change since: the recaptured graphs are reused
    b.close()


def test_batch_rejects_duplicates(built):
    d = instance(0)
    fs = mg.FluidSystem(d.params, d.genome, d.n)
    with pytest.raises(A.MgError):
        mg.Batch([fs, fs])
