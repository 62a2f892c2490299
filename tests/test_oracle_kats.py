"""The CPU oracle against the hand-derived known-answer vectors (tests/golden/kats.json) and
the integer properties of the reference's sort.  No GPU needed."""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle as orc
from helpers import box_centre, scene
from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo

KATS = json.loads((Path(__file__).parent / "golden" / "kats.json").read_text())
C0 = box_centre()


def run_stages(o, stages):
    for s in stages:
        getattr(o, s)()


def by_pid(o, buf):
    pid = o.download(A.FPARTICLE_ID)
    arr = o.download(buf)
    if arr.ndim == 2 and arr.shape[0] == A.NUM_GENES and buf == A.FEPIGEN:
        arr = arr.T
    order = np.argsort(pid, kind="stable")
    return arr[order]


@pytest.fixture(params=[32, 64], ids=["f32", "f64"])
def bits(request, built):
    return request.param


def tol(bits):
    # the f64 twin takes float32 parameters (mass, pi literal), hence 1e-7 rather than 1e-15
    return dict(rtol=2e-6, atol=0) if bits == 32 else dict(rtol=1e-7, atol=0)


def test_derived_params(built):
    d = demo.make_block(4, "R")
    o = orc.Oracle(d.params, d.genome, d.n)
    dv = o.derived()
    p = d.params
    assert dv.r2 == np.float32(p.psmoothradius) * np.float32(p.psmoothradius)
    assert dv.wendlandC2kern == np.float32(21) / (np.float32(2) * np.float32(3.141592))
    assert dv.gridAdjCnt == 27
    res = list(p.grid_res)
    assert list(dv.gridScanMax) == [r - 3 for r in res]
    expect = [(y * res[2] + z) * res[0] + x for y in range(3) for z in range(3) for x in range(3)]
    assert list(dv.gridAdj)[:27] == expect
    assert dv.nadj == (res[2] + 1) * res[0] + 1


def test_pair_density(bits):
    k = KATS["pair_density"]
    d, n = scene([[C0, C0, C0], [C0 + k["r"], C0, C0]])
    o = orc.Oracle(d.params, d.genome, n, bits)
    o.upload_all(d.arrays)
    run_stages(o, ["insert", "prefix_sum", "sort", "pressure"])
    np.testing.assert_allclose(o.download_f64(A.FPRESS), [k["press"]] * 2, **tol(bits))
    np.testing.assert_allclose(o.download_f64(A.FDENSITY), [k["invdens"]] * 2, **tol(bits))


def test_lone_density(bits):
    k = KATS["lone_density"]
    d, n = scene([[C0, C0, C0]])
    o = orc.Oracle(d.params, d.genome, n, bits)
    o.upload_all(d.arrays)
    run_stages(o, ["insert", "prefix_sum", "sort", "pressure"])
    assert o.download_f64(A.FPRESS)[0] == k["press"]
    assert o.download_f64(A.FDENSITY)[0] == k["invdens"]


def test_bond_spring(bits):
    k = KATS["bond_spring"]
    d, n = scene([[C0, C0, C0], [C0 + k["d"], C0, C0]],
                 bonds=[(0, 0, 1, k["L0"], k["modulus"], k["damping"], 1e30)])
    o = orc.Oracle(d.params, d.genome, n, bits)
    o.upload_all(d.arrays)
    run_stages(o, ["insert", "prefix_sum", "sort", "pressure", "force"])
    f = by_pid(o, A.FFORCE) if bits == 32 else None
    pid = o.download(A.FPARTICLE_ID)
    f64 = o.download_f64(A.FFORCE).reshape(-1, 4)[np.argsort(pid)]
    np.testing.assert_allclose(f64[0, 0], k["force_owner_x"], **tol(bits))
    np.testing.assert_allclose(f64[1, 0], k["force_partner_x"], **tol(bits))
    assert np.all(f64[:, 1:3] == 0)
    el = o.download_f64(A.FELASTIDX).reshape(-1, 6, 9)[np.argsort(pid)]
    np.testing.assert_allclose(el[0, 0, 6], k["strain_sq"], **tol(bits))
    np.testing.assert_allclose(el[0, 0, 7], k["strain"], **tol(bits))
    if f is not None:
        assert f[0, 0] == -f[1, 0]  # equal and opposite, bit for bit


def test_pair_diffusion(bits):
    k = KATS["pair_diffusion"]
    conc = np.zeros((2, 16), np.float32)
    conc[0, 0], conc[1, 0] = k["ci"], k["cj"]
    g = demo.make_genome(seed=1, diffusion=k["rate"], decay=1 - k["breakdown"])
    d, n = scene([[C0, C0, C0], [C0 + k["d"], C0, C0]], conc=conc, genome=g)
    o = orc.Oracle(d.params, d.genome, n, bits)
    o.upload_all(d.arrays)
    run_stages(o, ["insert", "prefix_sum", "sort", "diffusion"])
    pid = o.download(A.FPARTICLE_ID)
    c = o.download_f64(A.FCONC).reshape(-1, 16)[np.argsort(pid)]
    np.testing.assert_allclose(c[:, 0], [k["new_i"], k["new_j"]], rtol=1e-6 if bits == 32 else 1e-7)


@pytest.mark.parametrize("case", ["advance_free", "advance_clamp"])
def test_advance(bits, case):
    k = KATS[case]
    vel = k.get("vel", [0.0, 0.0, 0.0])
    d, n = scene([[C0, C0, C0]], vel=[vel])
    o = orc.Oracle(d.params, d.genome, n, bits)
    o.upload_all(d.arrays)
    run_stages(o, ["insert", "prefix_sum", "sort"])
    f = np.zeros((1, 4), np.float32)
    f[0, :3] = k["force"]
    o.upload(A.FFORCE, f)
    o.advance()
    np.testing.assert_allclose(o.download_f64(A.FVEL)[0, :3], k["vel_new"], rtol=1e-5 if bits == 32 else 1e-7)
    assert abs(o.time() - np.float32(1e-3)) < 1e-9


def test_gene_reaction(bits):
    k = KATS["gene_reaction"]
    g = demo.make_genome(seed=1, secretion=0.1)
    for a in range(16):
        for t in range(16):
            g.sensitivity[a][t] = 0.0
    g.sensitivity[0][1] = 0.5
    g.sensitivity[0][3] = -0.25
    g.sensitivity[2][0] = 1.0
    d, n = scene([[C0, C0, C0]], conc=[k["conc"]], genes=[0b101], genome=g)
    o = orc.Oracle(d.params, d.genome, n, bits)
    o.upload_all(d.arrays)
    run_stages(o, ["insert", "prefix_sum", "sort", "genes"])
    np.testing.assert_allclose(o.download_f64(A.FCONC)[0], k["conc_new"], rtol=1e-6 if bits == 32 else 1e-7)
    # not living (gene 2 off): no secretion is tallied
    d, n = scene([[C0, C0, C0]], conc=[k["conc"]], genes=[0b001], genome=g)
    o = orc.Oracle(d.params, d.genome, n, bits)
    o.upload_all(d.arrays)
    run_stages(o, ["insert", "prefix_sum", "sort", "genes"])
    np.testing.assert_allclose(o.download_f64(A.FCONC)[0], k["conc"], rtol=1e-7)


def test_stable_sort_hand_case(built):
    """Particles A(cell X) B(cell Y<X) C(cell X) D(cell Y): sorted B, D, A, C; ranks A0 B0 C1 D1."""
    cw = 4.0
    x0, x1 = C0 + 0.5, C0 - cw + 0.5  # x1 is one cell lower in x
    d, n = scene([[x0, C0, C0], [x1, C0, C0], [x0 + 0.25, C0, C0], [x1 + 0.25, C0, C0]])
    o = orc.Oracle(d.params, d.genome, n)
    o.upload_all(d.arrays)
    o.insert()
    assert list(o.download(A.FGNDX)) == [0, 0, 1, 1]
    cells = o.download(A.FGCELL)
    assert cells[0] == cells[2] and cells[1] == cells[3] and cells[1] == cells[0] - 1
    o.prefix_sum()
    o.sort()
    assert list(o.download(A.FPARTICLE_ID)) == [2, 4, 1, 3]
    assert list(o.download(A.FGNDX)) == [0, 1, 0, 1]


def test_sort_properties_config0(built):
    """Sortedness, stable ranks, permutation and bond-remap consistency at 4096 particles."""
    d = demo.make_block(16, "R", seed=3)
    o = orc.Oracle(d.params, d.genome, d.n)
    o.upload_all(d.arrays)
    o.insert()
    pre_cells = o.download(A.FGCELL)
    pre_ndx = o.download(A.FGNDX)
    # D1: rank = number of earlier particles in the same cell
    seen = {}
    for i, c in enumerate(pre_cells):
        assert pre_ndx[i] == seen.get(c, 0)
        seen[c] = seen.get(c, 0) + 1
    o.prefix_sum()
    cnt, off = o.download(A.FBIN_COUNT), o.download(A.FBIN_OFFSET)
    assert np.array_equal(off, np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.uint32))
    o.sort()
    cells = o.download(A.FGCELL)
    assert np.all(np.diff(cells.astype(np.int64)) >= 0)
    pid = o.download(A.FPARTICLE_ID)
    assert sorted(pid.tolist()) == list(range(1, d.n + 1))
    el = o.download(A.FELASTIDX).reshape(-1, 6, 9)
    pidx = o.download(A.FPARTICLEIDX).reshape(-1, 6, 2)
    for i in range(0, d.n, 97):
        for a in range(6):
            j = el[i, a, 0]
            if j == A.NO_PARTNER:
                continue
            assert el[i, a, 5] == pid[j]               # partner ID follows the remap
            assert pidx[j, a ^ 1, 0] == i and pidx[j, a ^ 1, 1] == a


def test_out_of_grid_particles_are_dropped(built):
    d, n = scene([[C0, C0, C0], [-1000.0, C0, C0], [C0 + 1, C0, C0], [C0, 1e9, C0]])
    o = orc.Oracle(d.params, d.genome, n)
    o.upload_all(d.arrays)
    o.step(1)
    assert o.counts()[0] == 2
    pid = o.download(A.FPARTICLE_ID)
    assert list(pid[:2]) == [1, 3] and list(pid[2:]) == [A.NO_PARTNER] * 2
    pos = o.download(A.FPOS)
    assert np.all(pos[2:, 2] == np.float32(d.params.pboundmin[2]) - 2 * d.params.grid_res[2])


def test_f32_f64_one_step_close(built):
    d = demo.make_block(8, "R")
    o32 = orc.Oracle(d.params, d.genome, d.n, 32)
    o64 = orc.Oracle(d.params, d.genome, d.n, 64)
    for o in (o32, o64):
        o.upload_all(d.arrays)
        o.step(1)
    assert np.array_equal(o32.download(A.FPARTICLE_ID), o64.download(A.FPARTICLE_ID))
    np.testing.assert_allclose(o32.download(A.FCONC), o64.download_f64(A.FCONC), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(o32.download(A.FPOS), o64.download_f64(A.FPOS), rtol=1e-5, atol=1e-4)
