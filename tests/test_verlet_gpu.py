"""Verlet neighbour lists of the density pass (MG_OPT_VERLET) against searching every step.

The lists must give the same bits as the search on every step: they hold every particle within
the search radius plus a skin at the last build, and are rebuilt once any particle has moved
half the skin.  Each case runs twin handles, lists on and off, and compares every state buffer
bitwise; the oracle comparisons of test_parity_gpu.py run with the lists on (the default).
"""
import numpy as np
import pytest

import morphogenesis_gb300 as mg
from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo

pytestmark = pytest.mark.gpu

BUFS = (A.FPOS, A.FVEL, A.FVEVAL, A.FFORCE, A.FPRESS, A.FDENSITY, A.FCONC, A.FELASTIDX,
        A.FPARTICLEIDX, A.FPARTICLE_ID, A.FGCELL)


def twins(d, skin=None):
    on = mg.FluidSystem(d.params, d.genome, d.n)
    off = mg.FluidSystem(d.params, d.genome, d.n)
    off.set_option(A.OPT_VERLET, 0)
    if skin is not None:
        on.set_option(A.OPT_VERLET_SKIN, skin)
    for fs in (on, off):
        fs.TransferToCL(d.arrays)
    return on, off


def same(on, off, what):
    for b in BUFS:
        x, y = on.download(b), off.download(b)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), f"{what}: buffer {b} differs"


def moving(side=12, seed=2):
    """A breakable block with random velocities near the velocity limit."""
    d = demo.make_block(side, "R", seed=seed, breakable=True)
    r = np.random.default_rng(seed)
    v = r.uniform(-2.5, 2.5, (d.n, 4)).astype(np.float32)
    v[:, 3] = 0
    d.arrays[A.FVEL] = v
    d.arrays[A.FVEVAL] = v.copy()
    return d


@pytest.mark.parametrize("param", ["R", "L"])
def test_lists_equal_search_100_steps(built, param):
    d = demo.make_block(16, param, seed=1)
    on, off = twins(d)
    on.Run(100)
    off.Run(100)
    same(on, off, f"{param}, 100 steps")
    assert on.neighbor_list_builds() >= 1
    assert off.neighbor_list_builds() == 0


def test_rebuilds_keep_results(built):
    """A small skin and fast particles: the lists are rebuilt many times."""
    d = moving()
    on, off = twins(d, skin=5)  # skin 0.5% of the radius: a rebuild every few steps
    flags = A.STEP_DEFAULT | A.STEP_REMODEL
    for _ in range(4):
        on.Run(15, flags)
        off.Run(15, flags)
        same(on, off, "breaking, moving block")
    assert on.neighbor_list_builds() >= 5, on.neighbor_list_builds()


def test_exchange_round_trip_keeps_lists(built):
    """Positions written back unchanged every step (the host exchange cycle) keep the lists;
    a changed position makes the next step rebuild them."""
    d = demo.make_block(12, "R", seed=3)
    on, off = twins(d)
    on.Run(2)
    off.Run(2)
    bufs = (A.FPOS, A.FVEL, A.FVEVAL, A.FCONC)
    host = {b: mg.pinned_empty(*mg._shape(b, d.n, int(d.params.grid_total))[::-1]) for b in bufs}
    host2 = {b: mg.pinned_empty(*mg._shape(b, d.n, int(d.params.grid_total))[::-1]) for b in bufs}
    for b in bufs:
        on.download(b, host[b])
        off.download(b, host2[b])
    b0 = on.neighbor_list_builds()
    for _ in range(10):
        on.step_io(host, 1, A.STEP_DEFAULT, host)
        off.step_io(host2, 1, A.STEP_DEFAULT, host2)
    same(on, off, "exchange round trip")
    assert on.neighbor_list_builds() == b0, "unchanged positions forced a rebuild"
    pos = on.download(A.FPOS)
    pos[5, 0] += np.float32(0.5)
    on.upload(A.FPOS, pos)
    off.upload(A.FPOS, pos)
    on.Run(3)
    off.Run(3)
    same(on, off, "after a moved particle")
    assert on.neighbor_list_builds() == b0 + 1


def test_inner_steps_without_sort(built):
    """Run2 inner steps (positions move without a sort) and a sort after them."""
    d = moving(10, seed=4)
    on, off = twins(d, skin=20)
    for fs in (on, off):
        fs.Run2PhysicalSort()
        for _ in range(4):
            fs.Run2InnerPhysicalLoop()
        fs.Run2GeneAction()
        fs.Run(5)
    same(on, off, "Run2 cycle")
