"""GPU pipeline vs the CPU oracle through the C-ABI (parity tests proper).

Integer outputs (cells, ranks, counts, offsets, sorted order, bond remap, gene bits) must be
bit-exact.  Float fields are compared with an explicit tolerance: FP_RTOL relative plus
FP_ATOL absolute scaled by the field's magnitude.  The kernels evaluate the reference
expressions in the oracle's order without fused multiply-adds, so the observed difference is
zero; the tolerance is the contract, the bitwise check is reported.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle as orc
from helpers import box_centre, scene
from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo

pytestmark = pytest.mark.gpu

FP_RTOL = 1e-5
FP_ATOL = 1e-6
KATS = json.loads((Path(__file__).parent / "golden" / "kats.json").read_text())
C0 = box_centre()

INT_BUFS = [A.FGCELL, A.FGNDX, A.FBIN, A.FPARTICLE_ID, A.FPARTICLEIDX, A.FEPIGEN, A.FAGE,
            A.FCOLOR, A.FMASS_RADIUS, A.FNERVEIDX, A.FBIN_COUNT, A.FBIN_OFFSET]
FLOAT_BUFS = [A.FPOS, A.FVEL, A.FVEVAL, A.FFORCE, A.FPRESS, A.FDENSITY, A.FCONC]


def pair(d, n, bits=32):
    import morphogenesis_gb300 as mg

    g = mg.FluidSystem(d.params, d.genome, n)
    o = orc.Oracle(d.params, d.genome, n, bits)
    g.TransferToCL(d.arrays)
    o.upload_all(d.arrays)
    return g, o


def close(a, b, what=""):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(1.0, float(np.nanmax(np.abs(b))) if b.size else 1.0)
    ok = np.isclose(a, b, rtol=FP_RTOL, atol=FP_ATOL * scale, equal_nan=True)
    assert ok.all(), f"{what}: {np.count_nonzero(~ok)} of {a.size} differ, max |d| {np.nanmax(np.abs(a - b))}"


def compare(g, o, bufs_int=INT_BUFS, bufs_float=FLOAT_BUFS, elast=True):
    for b in bufs_int:
        x, y = g.download(b), o.download(b)
        assert np.array_equal(x, y), f"integer buffer {b}: {np.count_nonzero(x != y)} words differ"
    bitwise = True
    for b in bufs_float:
        x, y = g.download(b), o.download(b)
        close(x, y, f"float buffer {b}")
        bitwise &= same_bits(x, y)
    if elast:
        x, y = g.download(A.FELASTIDX).reshape(-1, 6, 9), o.download(A.FELASTIDX).reshape(-1, 6, 9)
        for w in (0, 5, 8):
            assert np.array_equal(x[:, :, w], y[:, :, w]), f"FELASTIDX word {w}"
        for w in (1, 2, 3, 4, 6, 7):
            close(x[:, :, w].view(np.float32), y[:, :, w].view(np.float32), f"FELASTIDX word {w}")
        bitwise &= same_bits(x.view(np.float32), y.view(np.float32))
    return bitwise


def same_bits(x, y):
    """Bitwise equality with every NaN mapped to one pattern (NaN payloads differ by ISA)."""
    x = np.where(np.isnan(x), np.float32(np.nan), x).view(np.uint32)
    y = np.where(np.isnan(y), np.float32(np.nan), y).view(np.uint32)
    return np.array_equal(x, y)


@pytest.fixture(scope="module")
def cfg0():
    return demo.make_block(16, "R", seed=0)


def test_stage_by_stage_config0(built, cfg0):
    g, o = pair(cfg0, cfg0.n)
    g.InsertParticlesCL(); o.insert()
    compare(g, o, [A.FGCELL, A.FGNDX, A.FBIN_COUNT], [], elast=False)
    g.PrefixSumCellsCL(); o.prefix_sum()
    compare(g, o, [A.FBIN_OFFSET], [], elast=False)
    assert g.counts() == o.counts()
    g.CountingSortFullCL(); o.sort()
    compare(g, o, bufs_float=[A.FPOS, A.FVEL, A.FVEVAL, A.FCONC])
    g.ComputePressureCL(); o.pressure()
    compare(g, o, [], [A.FPRESS, A.FDENSITY], elast=False)
    g.ComputeForceCL(); o.force()
    compare(g, o, [], [A.FFORCE])
    g.ComputeDiffusionCL(); o.diffusion()
    compare(g, o, [], [A.FCONC], elast=False)
    g.ComputeGenesCL(); o.genes()
    compare(g, o, [A.FEPIGEN], [A.FCONC], elast=False)
    g.AdvanceCL(); o.advance()
    assert compare(g, o), "expected bitwise equality with the oracle"


@pytest.mark.parametrize("param", ["R", "L"])
def test_full_step_1_and_100_steps(built, param):
    d = demo.make_block(16, param, seed=1)
    g, o = pair(d, d.n)
    g.Run(1); o.step(1)
    assert compare(g, o)
    g.Run(99); o.step(99)
    assert compare(g, o), "100-step trajectories should stay bit-identical"
    assert g.counts() == o.counts()


def test_flags_physics_only_and_genes_only(built, cfg0):
    for flags in (A.STEP_PHYSICS, A.STEP_GENES, A.STEP_PHYSICS | A.STEP_GENES | A.STEP_FREEZE):
        g, o = pair(cfg0, cfg0.n)
        g.Run(3, flags); o.step(3, flags)
        compare(g, o)


def test_breakable_bonds_break_identically(built):
    d = demo.make_block(10, "R", seed=4, breakable=True)
    v = np.random.default_rng(4).uniform(-30, 30, (d.n, 4)).astype(np.float32)
    v[:, 3] = 0
    d.arrays[A.FVEL] = v
    d.arrays[A.FVEVAL] = v.copy()
    g, o = pair(d, d.n)
    g.Run(30); o.step(30)
    compare(g, o)
    el = o.download(A.FELASTIDX).reshape(-1, 6, 9)
    broken = (el[:, :, 0] != A.NO_PARTNER) & (el[:, :, 2] == 0)
    assert broken.any(), "scenario should break some bonds"


def test_kat_scenes_on_gpu(built):
    k = KATS["bond_spring"]
    d, n = scene([[C0, C0, C0], [C0 + k["d"], C0, C0]],
                 bonds=[(0, 0, 1, k["L0"], k["modulus"], k["damping"], 1e30)])
    g, o = pair(d, n)
    g.Run2PhysicalSort(); g.ComputePressureCL(); g.ComputeForceCL()
    f = g.download(A.FFORCE)[np.argsort(g.download(A.FPARTICLE_ID))]
    np.testing.assert_allclose(f[:, 0], [k["force_owner_x"], k["force_partner_x"]], rtol=2e-6)
    k = KATS["pair_density"]
    d, n = scene([[C0, C0, C0], [C0 + k["r"], C0, C0]])
    g, o = pair(d, n)
    g.Run2PhysicalSort(); g.ComputePressureCL()
    np.testing.assert_allclose(g.download(A.FPRESS), [k["press"]] * 2, rtol=2e-6)
    np.testing.assert_allclose(g.download(A.FDENSITY), [k["invdens"]] * 2, rtol=2e-6)


def test_stable_sort_hand_case_gpu(built):
    cw = 4.0
    x0, x1 = C0 + 0.5, C0 - cw + 0.5
    d, n = scene([[x0, C0, C0], [x1, C0, C0], [x0 + 0.25, C0, C0], [x1 + 0.25, C0, C0]])
    g, _ = pair(d, n)
    g.InsertParticlesCL()
    assert list(g.download(A.FGNDX)) == [0, 0, 1, 1]
    g.PrefixSumCellsCL(); g.CountingSortFullCL()
    assert list(g.download(A.FPARTICLE_ID)) == [2, 4, 1, 3]
    assert list(g.download(A.FGNDX)) == [0, 1, 0, 1]


def test_edge_empty_ragged_and_dropped(built):
    # every particle outside the grid window
    d, n = scene([[-1e6, 0, 0], [np.nan, 1, 1], [C0, -5.0, C0]])
    g, o = pair(d, n)
    g.Run(2); o.step(2)
    assert g.counts()[0] == 0
    compare(g, o)
    # ragged: capacity larger than the particle count, spare slots parked outside the grid
    d = demo.make_block(6, "R", seed=5, max_points=6 ** 3 + 37)
    g, o = pair(d, 6 ** 3 + 37)
    g.Run(3); o.step(3)
    assert g.counts()[0] == 6 ** 3
    compare(g, o)
    # particles pushed out of the window mid-run are dropped identically
    d = demo.make_block(6, "R", seed=6)
    pos = d.arrays[A.FPOS]
    pos[::7, 0] = -3.0
    g, o = pair(d, d.n)
    g.Run(2); o.step(2)
    compare(g, o)
    # parked slots given in-grid positions again by an upload of FPOS come back without bonds
    # (their records were dropped with them) and step identically; every re-origin period
    d = demo.make_block(6, "R", seed=7)
    d.arrays[A.FPOS][::7, 0] = -1e4
    g, o = pair(d, d.n)
    g.Run(2); o.step(2)
    nact = g.counts()[0]
    assert nact < d.n
    back = g.download(A.FPOS)
    live = back[:nact, :3]
    back[nact:, :3] = live[: d.n - nact] + np.float32(0.37)
    for period in (0, 1, 64):
        g2, o2 = pair(d, d.n)
        g2.set_option(A.OPT_REORIGIN_PERIOD, period)
        g2.Run(2); o2.step(2)
        g2.upload(A.FPOS, back); o2.upload(A.FPOS, back)
        g2.Run(3); o2.step(3)
        assert g2.counts()[0] == o2.counts()[0] > nact
        compare(g2, o2)
        g2.close(); o2.close()


@pytest.mark.parametrize("count", [300, 9000])
def test_crowded_cell_orders(built, count):
    """Cells above the warp tier (256) and above the block tier (8192) keep the stable order."""
    rs = np.random.default_rng(count)
    pts = C0 + rs.uniform(0.1, 3.9, (count, 3))
    pts = np.concatenate([pts, C0 + 6 + rs.uniform(0, 8, (200, 3))])
    d, n = scene(pts)
    g, o = pair(d, n)
    g.Run(1, A.STEP_GENES); o.step(1, A.STEP_GENES)
    compare(g, o, bufs_float=[A.FPOS, A.FCONC])
    # a full step: every particle of the crowded cell overflows its list and is walked by its
    # warp (density, diffusion and the fluid-force list)
    g1, o1 = pair(d, n)
    g1.Run(1, A.STEP_DEFAULT); o1.step(1, A.STEP_DEFAULT)
    assert compare(g1, o1), "crowded cell: full step differs from the oracle"
    # the per-lane sub-cell search scans such cells whole
    g2, _ = pair(d, n)
    g2.set_option(A.OPT_NEIGHBOR_SEARCH, 2)
    g2.Run(1, A.STEP_GENES)
    assert same_bits(g2.download(A.FCONC), o.download(A.FCONC))


def test_dense_gene_lists(built, cfg0):
    g, o = pair(cfg0, cfg0.n)
    g.Run(2); o.step(2)
    for b in (A.FBIN_COUNT_ACTIVE_GENES, A.FBIN_OFFSET_ACTIVE_GENES, A.FDENSE_LIST_LENGTHS,
              A.FDENSE_LISTS):
        assert np.array_equal(g.download(b), o.download(b)), f"dense-list buffer {b}"


def test_rejects_what_it_cannot_hold(built, cfg0):
    import morphogenesis_gb300 as mg

    g = mg.FluidSystem(cfg0.params, cfg0.genome, cfg0.n)
    with pytest.raises(mg.MgError):
        g.ComputePressureCL()  # no sort yet
    with pytest.raises(ValueError):
        g.upload(A.FPOS, cfg0.arrays[A.FPOS][:10])


def epigenetic_scene(seed):
    """A block whose FEPIGEN words hold countdowns and whose genome has delays and activation
    lists (the full epigenetic state of computeGeneAction)."""
    d = demo.make_block(8, "R", seed=seed)
    r = np.random.default_rng(seed)
    ep = d.arrays[A.FEPIGEN].copy()
    pick = r.random(ep.shape)
    ep[pick < 0.15] = r.integers(1, 6, ep.shape)[pick < 0.15].astype(np.uint32)
    ep[2, :] = np.where(r.random(ep.shape[1]) < 0.8, np.uint32(A.EPIGEN_ACTIVE), ep[2, :])  # mostly living
    d.arrays[A.FEPIGEN] = ep
    g = d.genome
    for a in range(A.NUM_GENES):
        g.delay[a] = int(r.integers(1, 5))
        na = int(r.integers(0, 3))
        for k in range(na):
            g.activate[a][2 * k] = float(r.integers(0, A.NUM_GENES))
            g.activate[a][2 * k + 1] = float(r.uniform(-0.2, 0.2))
        g.activate[a][2 * A.NUM_GENES] = float(na)
    return d


def test_full_epigenetic_state_matches_oracle(built):
    d = epigenetic_scene(5)
    gsys, o = pair(d, d.n)
    gsys.Run(12)
    o.step(12)
    assert compare(gsys, o), "full epigenetic steps are not bitwise equal to the oracle"
    ep = gsys.download(A.FEPIGEN)
    assert ((ep != 0) & (ep != A.EPIGEN_ACTIVE)).any(), "countdowns should remain in the state"
    # the surrogate step needs binary gene states
    import morphogenesis_gb300 as mg
    from morphogenesis_gb300 import surrogate as S
    S.attach(gsys, S.Mlp(seed=1), 0, 0, 1e-3)
    with pytest.raises(mg.MgError):
        gsys.Run(1, A.STEP_DEFAULT | A.STEP_SURROGATE)


def test_deterministic_rerun(built):
    d = demo.make_block(12, "R", seed=7)
    outs = []
    for _ in range(2):
        g, _o = pair(d, d.n)
        g.Run(5)
        outs.append({b: g.download(b) for b in (A.FPOS, A.FCONC, A.FPARTICLE_ID, A.FELASTIDX)})
    for b in outs[0]:
        assert np.array_equal(outs[0][b], outs[1][b])


def test_graph_cache_alternates_buffers(built, cfg0):
    """Odd and even step counts, mixed with stage calls, give the oracle's result."""
    g, o = pair(cfg0, cfg0.n)
    g.Run(1); o.step(1)
    g.Run2PhysicalSort(); o.insert(); o.prefix_sum(); o.sort()
    g.Run2InnerPhysicalLoop(); o.pressure(); o.force(); o.advance()
    g.Run2GeneAction(); o.diffusion(); o.genes()
    g.Run(3); o.step(3)
    compare(g, o)


@pytest.mark.parametrize("param", ["R", "L"])
def test_warp_search_equals_direct_walk(built, param):
    """The warp-cooperative neighbour search gives the direct walk's bits."""
    import morphogenesis_gb300 as mg

    d = demo.make_block((20, 12, 16), param, seed=8)
    outs = []
    for mode in (0, 1, 2):
        g = mg.FluidSystem(d.params, d.genome, d.n)
        g.set_option(A.OPT_NEIGHBOR_SEARCH, mode)
        g.TransferToCL(d.arrays)
        g.Run(20)
        outs.append({b: g.download(b) for b in (A.FPOS, A.FVEL, A.FCONC, A.FPRESS, A.FDENSITY,
                                                 A.FFORCE, A.FELASTIDX, A.FPARTICLE_ID)})
    for b in outs[0]:
        for m in (1, 2):
            assert same_bits(outs[0][b].view(np.float32), outs[m][b].view(np.float32)), f"buffer {b} mode {m}"


def test_remodelling_reforms_identically(built):
    d = demo.make_block(10, "R", seed=4, breakable=True)
    v = np.random.default_rng(4).uniform(-30, 30, (d.n, 4)).astype(np.float32)
    v[:, 3] = 0
    d.arrays[A.FVEL] = v
    d.arrays[A.FVEVAL] = v.copy()
    g, o = pair(d, d.n)
    flags = A.STEP_DEFAULT | A.STEP_REMODEL
    g.Run(40, flags)
    o.step(40, flags)
    assert compare(g, o), "remodelling run is not bitwise equal to the oracle"
    plain = orc.Oracle(d.params, d.genome, d.n)
    plain.upload_all(d.arrays)
    plain.step(40)

    def broken(x):
        el = x.download(A.FELASTIDX).reshape(-1, 6, 9)
        return int(((el[:, :, 0] != A.NO_PARTNER) & (el[:, :, 2] == 0)).sum())

    assert broken(o) < broken(plain), "re-forming should leave fewer broken bonds"
    plain.close()


def test_remodelling_stage_matches_oracle(built):
    q, p1, p2 = [C0, C0, C0], [C0 + 1.0, C0, C0], [C0 - 1.2, C0, C0]
    rs = [[C0, C0 + 3.0, C0], [C0, C0 - 3.0, C0], [C0, C0, C0 + 3.0], [C0, C0, C0 - 3.0],
          [C0, C0 + 2.2, C0 + 2.2]]
    bonds = [(1, 0, 2, 0.0, 1000.0, 10.0, 5.0), (2, 0, 1, 0.0, 1000.0, 10.0, 5.0)]
    bonds += [(3 + k, 0, 0, 3.0, 1000.0, 10.0, 9.0) for k in range(5)]
    d, n = scene([q, p1, p2] + rs, bonds=bonds)
    pidx = d.arrays[A.FPARTICLEIDX]
    pidx[0, :] = A.NO_PARTNER
    for k in range(5):
        pidx[0, 2 * k] = 3 + k
        pidx[0, 2 * k + 1] = 0
    g, o = pair(d, n)
    for _ in range(2):
        g.Run2PhysicalSort()
        g.Run2Remodelling()
        o.insert(); o.prefix_sum(); o.sort(); o.remodel()
        for b in (A.FELASTIDX, A.FPARTICLEIDX, A.FPARTICLE_ID):
            assert np.array_equal(g.download(b), o.download(b)), f"buffer {b}"


CHANGE_BUFS = [A.FBIN_COUNT_CHANGES, A.FBIN_OFFSET_CHANGES, A.FDENSE_LIST_LENGTHS_CHANGES,
               A.FDENSE_LISTS_CHANGES]


def bond_change_block(seed):
    """A breakable 10^3 block, moving, 80 % living, tissue genes (tendon, muscle, bone,
    elastic ligament) at random, genome with the shifted-tanh remodel parameters."""
    d = demo.make_block(10, "R", seed=seed, breakable=True)
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


def test_bond_changes_step_matches_oracle(built):
    """computeBondChanges + heal of the flagged slots inside the step, both heal-parameter
    modes: bitwise equal to the oracle, change lists equal."""
    for heal_params in (0, 1):
        d = bond_change_block(7)
        g, o = pair(d, d.n)
        g.set_option(A.OPT_HEAL_PARAMS, heal_params)
        o.set_heal_params(heal_params)
        flags = A.STEP_DEFAULT | A.STEP_BOND_CHANGES
        g.Run(30, flags)
        o.step(30, flags)
        assert compare(g, o), f"bond-change run (heal parameters {heal_params}) is not bitwise equal"
        for b in CHANGE_BUFS:
            x, y = g.download(b), o.download(b)
            assert np.array_equal(x, y), f"change buffer {b}"
        assert g.download(A.FDENSE_LIST_LENGTHS_CHANGES)[0] > 0, "no slot flagged for heal"
        g.close()
        o.close()


def test_run2_remodelling_matches_oracle(built):
    """The reference's Run2 loop: sort, 4 inner physical steps, Run2Remodelling(4)."""
    d = bond_change_block(8)
    g, o = pair(d, d.n)
    for _ in range(3):
        g.Run2PhysicalSort()
        o.insert(); o.prefix_sum(); o.sort()
        for _ in range(4):
            g.Run2InnerPhysicalLoop()
            o.pressure(); o.force(); o.advance()
        g.Run2Remodelling(4)
        o.bond_changes(4)
        o.remodel()
        assert compare(g, o), "Run2Remodelling(4) is not bitwise equal to the oracle"
        for b in CHANGE_BUFS:
            assert np.array_equal(g.download(b), o.download(b)), f"change buffer {b}"
    g.close()
    o.close()


def test_drifted_positions_between_sorts(built):
    """The reference's Run2 loop sorts once per several inner steps, so positions move away from
    the cells they were binned in (here about an eighth of a cell per step).  The neighbour
    searches then must not skip window cells by their geometric box: pressure, force, diffusion
    and the re-forming search stay bitwise equal to the oracle, which walks all 27 cells."""
    d = demo.make_block(10, "R", seed=12, breakable=True)
    d.params.pvel_limit = 1000.0
    d.params.paccel_limit = 1e6
    r = np.random.default_rng(12)
    v = r.uniform(-500, 500, (d.n, 4)).astype(np.float32)
    v[:, 3] = 0
    d.arrays[A.FVEL] = v
    d.arrays[A.FVEVAL] = v.copy()
    g, o = pair(d, d.n)
    for _ in range(3):
        g.Run2PhysicalSort()
        o.insert(); o.prefix_sum(); o.sort()
        for _ in range(4):
            g.Run2InnerPhysicalLoop()
            o.pressure(); o.force(); o.advance()
        g.Run2GeneAction()
        o.diffusion(); o.genes()
        g.Run2Remodelling()
        o.remodel()
        assert compare(g, o), "drifted positions: not bitwise equal to the oracle"
    g.close()
    o.close()


def test_time_and_zero_vel(built, cfg0):
    """m_Time advances by dt per integrating step (AdvanceTime) and is kept across SetParam;
    ZeroVelCL clears the velocities of every particle."""
    import morphogenesis_gb300 as mg

    fs = mg.FluidSystem(cfg0.params, cfg0.genome, cfg0.n)
    o = orc.Oracle(cfg0.params, cfg0.genome, cfg0.n)
    fs.TransferToCL(cfg0.arrays)
    o.upload_all(cfg0.arrays)
    fs.Run(5)
    o.step(5)
    assert fs.time() == o.time()
    fs.SetParam(A.PFREEZE, 1.0)
    assert fs.time() == o.time(), "SetParam must not rewind m_Time"
    fs.Run(1, A.STEP_GENES)  # no integration: time unchanged
    assert fs.time() == o.time()
    fs.ZeroVelCL()
    assert not fs.download(A.FVEL).any() and not fs.download(A.FVEVAL).any()
    fs.close()
    o.close()


def test_launch_shapes_give_identical_results(built):
    d = demo.make_block((24, 12, 24), "R", seed=6)
    import morphogenesis_gb300 as mg

    ref = mg.FluidSystem(d.params, d.genome, d.n)
    ref.TransferToCL(d.arrays)
    ref.Run(30)
    want = {b: ref.download(b).view(np.uint32) for b in (A.FPOS, A.FVEL, A.FCONC, A.FELASTIDX, A.FPARTICLE_ID)}
    for shape in ((4, 1, 1, 1), (8, 1, 2, 1), (4, 0, 2, 1), (8, 0, 1, 1), (8, 0, 1, 2), (4, 0, 1, 2)):
        fs = mg.FluidSystem(d.params, d.genome, d.n)
        fs.TransferToCL(d.arrays)
        fs.set_tuning(*shape)
        fs.Run(30)
        for b, w in want.items():
            assert np.array_equal(fs.download(b).view(np.uint32), w), f"shape {shape} buffer {b}"
        fs.close()
    # re-origin periods (bond records and cold fields renumbered to the sorted order): never,
    # every step, every third step
    for period in (0, 1, 3):
        fs = mg.FluidSystem(d.params, d.genome, d.n)
        fs.TransferToCL(d.arrays)
        fs.set_option(A.OPT_REORIGIN_PERIOD, period)
        fs.Run(30)
        for b, w in want.items():
            assert np.array_equal(fs.download(b).view(np.uint32), w), f"re-origin period {period} buffer {b}"
        for b in (A.FAGE, A.FCOLOR, A.FPARTICLE_ID, A.FMASS_RADIUS, A.FNERVEIDX):
            assert np.array_equal(fs.download(b), ref.download(b)), f"re-origin period {period} buffer {b}"
        fs.close()
    # block sizes of the force, gather and advance passes
    for threads in ((128, 512, 128), (512, 128, 512)):
        fs = mg.FluidSystem(d.params, d.genome, d.n)
        fs.TransferToCL(d.arrays)
        fs.set_block_sizes(*threads)
        assert fs.block_sizes() == threads
        fs.Run(30)
        for b, w in want.items():
            assert np.array_equal(fs.download(b).view(np.uint32), w), f"block sizes {threads} buffer {b}"
        with pytest.raises(A.MgError):
            fs.set_block_sizes(64, 256, 256)
        fs.close()
    # the autotuner restores the state it tunes on
    fs = mg.FluidSystem(d.params, d.genome, d.n)
    fs.TransferToCL(d.arrays)
    fs.Run(10)
    before = fs.download(A.FPOS).copy()
    res = fs.autotune(3)
    assert fs.tuning() == (res["dens_warps"], res["group_mode"], res["sub_bits"], res["search"])
    assert fs.block_sizes() == (res["force_threads"], res["gather_threads"], res["advance_threads"])
    assert np.array_equal(fs.download(A.FPOS), before)
    fs.Run(20)
    for b, w in want.items():
        assert np.array_equal(fs.download(b).view(np.uint32), w), f"after autotune, buffer {b}"


def test_step_io_equals_separate_calls(built, cfg0):
    import morphogenesis_gb300 as mg

    bufs = (A.FPOS, A.FVEL, A.FVEVAL, A.FCONC, A.FELASTIDX)
    a = mg.FluidSystem(cfg0.params, cfg0.genome, cfg0.n)
    b = mg.FluidSystem(cfg0.params, cfg0.genome, cfg0.n)
    for fs in (a, b):
        fs.TransferToCL(cfg0.arrays)
        fs.Run(3)
    host = {k: a.download(k) for k in bufs}
    host[A.FVEL] = (host[A.FVEL] * np.float32(0.5)).astype(np.float32)  # the host edits state
    out_a = {k: np.empty_like(v) for k, v in host.items()}
    for k, v in host.items():
        b.upload(k, v)
    b.Run(2)
    a.step_io(host, 2, A.STEP_DEFAULT, out_a)
    for k in bufs:
        assert np.array_equal(out_a[k].view(np.uint32), b.download(k).view(np.uint32)), f"buffer {k}"


def test_step_io_overlapped_exchange(built, cfg0):
    """Page-locked plain-copy buffers take the graph path (uploads and downloads captured with
    the first and last step, FCONC downloaded under the force pass): same results as uploads,
    steps and downloads issued one after another."""
    import morphogenesis_gb300 as mg

    cases = [((A.FPOS, A.FVEL, A.FVEVAL, A.FCONC), 1, A.STEP_DEFAULT),
             ((A.FPOS, A.FVEL, A.FVEVAL, A.FCONC), 3, A.STEP_DEFAULT | A.STEP_REMODEL),
             ((A.FPOS, A.FVEL, A.FVEVAL, A.FCONC), 2, A.STEP_GENES),
             # no concentrations: the gather's motion part alone waits for its uploads
             ((A.FPOS, A.FVEL, A.FPARTICLEIDX), 2, A.STEP_DEFAULT),
             ((A.FVEVAL, A.FCONC), 1, A.STEP_DEFAULT)]
    for bufs, nsteps, flags in cases:
        a = mg.FluidSystem(cfg0.params, cfg0.genome, cfg0.n)
        b = mg.FluidSystem(cfg0.params, cfg0.genome, cfg0.n)
        for fs in (a, b):
            fs.TransferToCL(cfg0.arrays)
            fs.Run(2)
        host = {k: mg.pinned_empty(*_shape_of(a, k)) for k in bufs}
        outs = {k: mg.pinned_empty(*_shape_of(a, k)) for k in bufs}
        for k in bufs:
            host[k][...] = a.download(k)
        if A.FVEL in host:
            host[A.FVEL][...] = host[A.FVEL] * np.float32(0.5)
        for rep in range(2):  # the second call replays the cached exchange graphs
            for k in bufs:
                b.upload(k, np.ascontiguousarray(host[k]))
            b.Run(nsteps, flags)
            a.step_io(host, nsteps, flags, outs)
            for k in bufs:
                assert np.array_equal(outs[k].view(np.uint32), b.download(k).view(np.uint32)), (bufs, nsteps, flags, k)
            for k in (A.FPOS, A.FVEL, A.FVEVAL, A.FCONC, A.FPARTICLEIDX):  # the whole state agrees
                assert np.array_equal(a.download(k).view(np.uint32), b.download(k).view(np.uint32)), (bufs, k)
            for k in bufs:
                host[k][...] = outs[k]
        a.close()
        b.close()


def _shape_of(fs, buf):
    import morphogenesis_gb300 as mg
    dt, shape = mg._shape(buf, fs.max_points, fs.cells)
    return shape, dt


def test_eight_cell_window_matches_oracle(built):
    """gsrch 2 (the reference's own grid-search formula for a cell of 2h: offsets -1..0 per
    axis): the warp search and the direct walk give the oracle's bits."""
    d = demo.make_block(12, "R", seed=4)
    d.params.grid_srch = 2
    for mode in (1, 0):
        g, o = pair(d, d.n)
        g.set_option(A.OPT_NEIGHBOR_SEARCH, mode)
        g.Run(5)
        o.step(5)
        assert compare(g, o), f"gsrch 2, search mode {mode}: not bitwise equal to the oracle"


def test_special_particles_match_oracle(built):
    d = demo.make_block(10, "R", seed=9)
    d.params.actuation_factor = 0.05
    d.params.actuation_period = 10.0
    g, o = pair(d, d.n)
    flags = A.STEP_DEFAULT | A.STEP_SPECIAL
    g.Run(20, flags)
    o.step(20, flags)
    assert compare(g, o), "special-particle steps are not bitwise equal to the oracle"
    # gene 11 particles keep their initial position; gene 12 (not 11) particles move in z only
    ids = g.download(A.FPARTICLE_ID).astype(np.int64) - 1
    pos = g.download(A.FPOS)
    ep = d.arrays[A.FEPIGEN]
    p0 = d.arrays[A.FPOS]
    fixed = ep[11, ids] != 0
    act = (ep[12, ids] != 0) & ~fixed
    assert fixed.any() and act.any()
    assert np.array_equal(pos[fixed, :3], p0[ids[fixed], :3])
    assert np.array_equal(pos[act, :2], p0[ids[act], :2])
    assert not np.array_equal(pos[act, 2], p0[ids[act], 2])
