"""computeBondChanges on the CPU oracle: the deterministic tanh, the shifted-tanh remodel of rest
length and modulus with integrator averaging, the heal flag that ends a particle's loop, the
change lists, and heal of the flagged slots."""
import math

import numpy as np

import oracle as orc
from helpers import box_centre, scene
from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo

C0 = box_centre()
f32 = np.float32


def test_tanh_within_two_ulp():
    orc.build()
    L = orc.lib(32)
    xs = np.concatenate([np.linspace(-12, 12, 40001, dtype=np.float32),
                         np.float32(np.logspace(-9, 1.2, 4000)), -np.float32(np.logspace(-9, 1.2, 4000)),
                         np.float32([0.0, -0.0, 0.5, -0.5, 9.0, -9.0, np.nextafter(f32(0.5), f32(0))])])
    worst = 0.0
    for x in xs:
        got = L.mgo_tanh_cw(float(x))
        want = math.tanh(float(x))
        ulp = float(np.spacing(f32(abs(want)))) if want != 0 else float(np.spacing(f32(0)))
        worst = max(worst, abs(got - want) / ulp)
        assert got == -L.mgo_tanh_cw(float(-x)), "odd function"
    assert worst <= 2.0, f"tanh off by {worst} ulp"
    assert math.isnan(L.mgo_tanh_cw(float("nan")))
    assert L.mgo_tanh_cw(30.0) == 1.0 and L.mgo_tanh_cw(-30.0) == -1.0


def tanh32(x):
    return f32(orc.lib(32).mgo_tanh_cw(float(f32(x))))


def remodel_factor(T, s):
    """a + b tanh(c s - d) in the kernel's float operations."""
    return f32(f32(T[0]) + f32(f32(T[1]) * tanh32(f32(f32(T[2]) * f32(s)) - f32(T[3]))))


def kat_scene():
    # A (0): living tendon; bonds: slot 0 -> B (collagen), slot 1 -> C (elastin), slot 2 empty
    # (heal), slot 3 -> B (after the heal flag: untouched).  B (1) is not living.  D (3) is
    # the nearest free particle for A's heal.  Only A is living (a living particle without
    # bonds would flag its empty slot 0).
    pos = [[C0, C0, C0], [C0 + 1.0, C0, C0], [C0, C0 + 1.2, C0], [C0, C0, C0 + 1.5]]
    bonds = [(0, 0, 1, 1.0, 1000.0, 10.0, 1.5), (0, 1, 2, 1.2, 800.0, 8.0, 1.8),
             (0, 3, 1, 0.9, 500.0, 5.0, 1.4), (1, 0, 0, 1.0, 1000.0, 10.0, 1.5)]
    genes = [(1 << 2) | (1 << 6), 0, 0, 0]
    d, n = scene(pos, bonds=bonds, genes=genes)
    el = d.arrays[A.FELASTIDX].reshape(n, 6, 9)
    elf = el.view(np.float32)
    for a, (sq, si) in {0: (0.5, 0.8), 1: (0.2, 0.4), 3: (0.3, 0.6)}.items():
        elf[0, a, 6], elf[0, a, 7] = sq, si
    elf[1, 0, 6], elf[1, 0, 7] = 0.7, 0.9
    el[0, 3, 8] = 0
    return d, n


def by_id(o, buf):
    ids = o.download(A.FPARTICLE_ID).astype(np.int64) - 1
    order = np.argsort(ids)
    return o.download(buf)[order], ids


def test_bond_changes_known_answer():
    d, n = kat_scene()
    orc.build()
    o = orc.Oracle(d.params, d.genome, n)
    o.upload_all(d.arrays)
    o.insert(); o.prefix_sum(); o.sort()
    o.bond_changes(4)
    el, ids = by_id(o, A.FELASTIDX)
    el = el.reshape(n, 6, 9)
    elf = el.view(np.float32)
    G = d.genome
    collagen, elastin = list(G.tanh_param[1]), list(G.tanh_param[0])
    # slot 0: collagen; integrators averaged over 4 steps (0.8 / 4, 0.5 / 4) and zeroed
    assert elf[0, 0, 2] == f32(1.0) * remodel_factor(collagen[0:4], f32(0.8) / f32(4))
    assert elf[0, 0, 3] == f32(1000.0) * remodel_factor(collagen[4:8], f32(0.5) / f32(4))
    want = 1.0 * (collagen[0] + collagen[1] * math.tanh(collagen[2] * 0.2 - collagen[3]))
    assert abs(float(elf[0, 0, 2]) - want) < 4e-7
    assert elf[0, 0, 6] == 0 and elf[0, 0, 7] == 0
    # slot 1: elastin (a tendon's bonds 1-5 are elastin)
    assert elf[0, 1, 2] == f32(1.2) * remodel_factor(elastin[0:4], f32(0.4) / f32(4))
    assert elf[0, 1, 3] == f32(800.0) * remodel_factor(elastin[4:8], f32(0.2) / f32(4))
    # slot 2 (no partner) is flagged for heal and ends the loop: slot 3 keeps its values
    assert list(el[0, :3, 8]) == [0, 0, 1]
    assert elf[0, 3, 2] == f32(0.9) and elf[0, 3, 6] == f32(0.3) and elf[0, 3, 7] == f32(0.6)
    # B is not living: untouched
    assert elf[1, 0, 2] == f32(1.0) and elf[1, 0, 6] == f32(0.7)
    # change list 0 holds (A, slot 2); lists 1-8 are empty
    lens = o.download(A.FDENSE_LIST_LENGTHS_CHANGES)
    assert list(lens) == [1] + [0] * 8
    lists = o.download(A.FDENSE_LISTS_CHANGES)
    a_sorted = int(np.nonzero(ids == 0)[0][0])
    assert lists[0, 0, 0] == a_sorted and lists[0, 1, 0] == 2
    counts = o.download(A.FBIN_COUNT_CHANGES)
    assert counts.sum() == 1 and counts[1:].sum() == 0
    o.close()


def test_heal_of_flagged_slot_with_genome_defaults():
    d, n = kat_scene()
    o = orc.Oracle(d.params, d.genome, n)
    o.upload_all(d.arrays)
    o.insert(); o.prefix_sum(); o.sort()
    o.set_heal_params(1)
    o.bond_changes(4)
    o.remodel()
    el, ids = by_id(o, A.FELASTIDX)
    el = el.reshape(n, 6, 9)
    elf = el.view(np.float32)
    partner = int(ids[el[0, 2, 0]])
    assert partner == 3, "healed to the nearest particle that is not a partner"
    E = list(d.genome.param[0])
    assert (elf[0, 2, 1], elf[0, 2, 2], elf[0, 2, 3], elf[0, 2, 4]) == (f32(E[8]), f32(E[9]), f32(E[10]), f32(E[11]))
    assert el[0, 2, 5] == 4 and el[0, 2, 8] == 0
    # a second heal call leaves the new bond alone
    o.remodel()
    el2, _ = by_id(o, A.FELASTIDX)
    assert np.array_equal(el2.reshape(n, 6, 9)[0], el[0])
    o.close()


def test_zero_tanh_parameters_break_living_bonds():
    """With a genome whose tanh parameters are 0 the multiplier is 0: the first visited bond's
    rest length becomes 0, so it is flagged for heal and ends the loop (as in the reference)."""
    d, n = kat_scene()
    g = demo.make_genome(seed=1)
    for k in range(3):
        g.tanh_param[k][:] = [0.0] * 8
    o = orc.Oracle(d.params, g, n)
    o.upload_all(d.arrays)
    o.insert(); o.prefix_sum(); o.sort()
    o.bond_changes(1)
    el, _ = by_id(o, A.FELASTIDX)
    elf = el.reshape(n, 6, 9).view(np.float32)
    assert elf[0, 0, 2] == 0 and elf[0, 1, 2] == f32(1.2) and elf[0, 3, 2] == f32(0.9)
    assert list(el.reshape(n, 6, 9)[0, :, 8]) == [1, 0, 0, 0, 0, 0]
    o.close()
