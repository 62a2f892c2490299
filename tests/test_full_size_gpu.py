"""The configurations' full sizes on the GPU: 1,048,576 particles (128x64x128 lattice) bitwise
against the oracle over two full steps, and 16,777,216 particles (256^3) through properties
that do not depend on size (every particle kept once, cells in order, counts and offsets
consistent, bond tables reciprocal)."""
import numpy as np
import pytest

import oracle as orc
from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo
from test_parity_gpu import compare, pair

pytestmark = pytest.mark.gpu


def test_config1_two_steps_match_oracle(built):
    d = demo.make_block((128, 64, 128), "R", seed=0)
    assert d.n == 1_048_576
    g, o = pair(d, d.n)
    g.Run(2)
    o.step(2)
    assert g.counts() == o.counts()
    assert compare(g, o), "1,048,576 particles: two steps are not bitwise equal to the oracle"
    g.close()
    o.close()


def test_config4_size_properties(built):
    import morphogenesis_gb300 as mg

    d = demo.make_block(256, "R", seed=4)
    n = d.n
    assert n == 16_777_216
    fs = mg.FluidSystem(d.params, d.genome, n)
    fs.TransferToCL(d.arrays)
    del d
    fs.Run(2, A.STEP_DEFAULT | A.STEP_REMODEL)
    total, active = fs.counts()
    assert total == n and active == n
    pid = fs.download(A.FPARTICLE_ID)
    assert np.array_equal(np.sort(pid), np.arange(1, n + 1, dtype=np.uint32)), "particles lost or duplicated"
    cell = fs.download(A.FGCELL)
    assert np.all(cell[1:] >= cell[:-1]), "sorted particles are not in cell order"
    cnt = fs.download(A.FBIN_COUNT).astype(np.int64)
    off = fs.download(A.FBIN_OFFSET).astype(np.int64)
    assert cnt.sum() == n
    assert np.array_equal(off[1:], np.cumsum(cnt)[:-1]) and off[0] == 0
    assert np.array_equal(np.bincount(cell, minlength=len(cnt)), cnt)
    # every bond's partner lists it in its incoming table (sampled particles)
    el = fs.download(A.FELASTIDX).reshape(n, 6, 9)
    pidx = fs.download(A.FPARTICLEIDX).reshape(n, 6, 2)
    rs = np.random.default_rng(4).choice(n, 200_000, replace=False)
    part = el[rs, :, 0]
    for a in range(6):
        ok = part[:, a] < n
        p, j = rs[ok], part[ok, a].astype(np.int64)
        inc = pidx[j]
        found = np.any((inc[:, :, 0] == p[:, None]) & (inc[:, :, 1] == a), axis=1)
        assert found.all(), f"slot {a}: {np.count_nonzero(~found)} bonds missing from their partner's table"
    fs.close()
