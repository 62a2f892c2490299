"""Packed instances (mg_create_packed): several tissues of different sizes, stiffnesses and
genomes advanced as one system, one kernel launch per stage, must each end bit for bit where
the same tissue ends as a system of its own (every instance keeps its own frame and grid)."""
import numpy as np
import pytest

import morphogenesis_gb300 as mg
from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo

pytestmark = pytest.mark.gpu

BUFS = (A.FPOS, A.FVEL, A.FVEVAL, A.FFORCE, A.FPRESS, A.FDENSITY, A.FCONC, A.FELASTIDX,
        A.FPARTICLEIDX, A.FPARTICLE_ID, A.FEPIGEN)


def instance(k):
    r = np.random.default_rng(200 + k)
    side = int(r.integers(5, 15))
    g = demo.make_genome(seed=20 + k, diffusion=demo.diffusion_rate("R", float(r.uniform(0.05, 0.2))))
    return demo.make_block(side, "R", seed=k, genome=g, intstiff=float(r.uniform(0.5, 2.0)),
                           breakable=bool(k % 2))


def test_packed_equals_instances_alone(built):
    ds = [instance(k) for k in range(6)]
    pk = mg.Packed([d.params for d in ds], [d.genome for d in ds], [d.n for d in ds])
    pk.TransferToCL(pk.concat([d.arrays for d in ds]))
    alone = []
    for d in ds:
        fs = mg.FluidSystem(d.params, d.genome, d.n)
        fs.TransferToCL(d.arrays)
        alone.append(fs)
    for flags, n in ((A.STEP_DEFAULT, 9), (A.STEP_DEFAULT | A.STEP_FREEZE, 2), (A.STEP_PHYSICS, 3),
                     (A.STEP_DEFAULT, 6)):
        pk.Run(n, flags)
        for fs in alone:
            fs.Run(n, flags)
    assert [c for _, c in pk.ranges()] == [d.n for d in ds]
    for b in BUFS:
        parts = pk.split(b)
        for k, fs in enumerate(alone):
            x, y = parts[k], fs.download(b)
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), f"instance {k}, buffer {b}"
    ms = pk.time_steps(3)
    assert ms > 0
    pk.close()


def test_packed_rejects_single_system_features(built):
    ds = [instance(k) for k in range(2)]
    pk = mg.Packed([d.params for d in ds], [d.genome for d in ds], [d.n for d in ds])
    pk.TransferToCL(pk.concat([d.arrays for d in ds]))
    for flags in (A.STEP_DEFAULT | A.STEP_REMODEL, A.STEP_DEFAULT | A.STEP_SURROGATE):
        with pytest.raises(A.MgError):
            pk.Run(1, flags)
    with pytest.raises(A.MgError):
        pk.set_option(A.OPT_NEIGHBOR_SEARCH, 0)
    with pytest.raises(A.MgError):
        pk.UpdateGenome(ds[1].genome)
    pk.close()


def test_packed_needs_equal_shared_parameters(built):
    ds = [instance(k) for k in range(2)]
    p1 = ds[1].params
    p1.pvisc = 0.3
    with pytest.raises(A.MgError):
        mg.Packed([ds[0].params, p1], [d.genome for d in ds], [d.n for d in ds])
