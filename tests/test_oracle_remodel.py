"""Known-answer cases of the deterministic bond re-forming rule (D5) on the CPU oracle:
nearest eligible particle within h, existing partners excluded, proposals accepted in
(distance, index) order into free incoming slots."""
import numpy as np

import oracle as orc
from helpers import box_centre, scene
from morphogenesis_gb300 import _abi as A

C0 = box_centre()


def sorted_view(o):
    """FELASTIDX / FPARTICLEIDX indexed by particle id - 1 (the scene's input order)."""
    ids = o.download(A.FPARTICLE_ID).astype(np.int64) - 1
    order = np.argsort(ids)
    el = o.download(A.FELASTIDX).reshape(-1, 6, 9)
    pidx = o.download(A.FPARTICLEIDX).reshape(-1, 12)
    to_input = lambda j: int(ids[j]) if j < len(ids) else j
    return el[order], pidx[order], to_input


def resort(o):
    o.insert(); o.prefix_sum(); o.sort()


def test_reforms_to_nearest_eligible_particle():
    # A (0) has a broken bond to B (1); C (2) at distance 1.0 and D (3) at 1.5 are eligible
    pos = [[C0, C0, C0], [C0 + 1.9, C0, C0], [C0, C0 + 1.0, C0], [C0, C0, C0 + 1.5]]
    d, n = scene(pos, bonds=[(0, 0, 1, 0.0, 1000.0, 10.0, 3.0)])
    orc.build()
    o = orc.Oracle(d.params, d.genome, n)
    o.upload_all(d.arrays)
    resort(o)
    o.remodel()
    el, pidx, back = sorted_view(o)
    elf = el.view(np.float32)
    assert back(el[0, 0, 0]) == 2, "re-formed to the nearest eligible particle"
    assert elf[0, 0, 2] == np.float32(1.0) and elf[0, 0, 1] == np.float32(1.5)
    assert elf[0, 0, 3] == np.float32(1000.0) and elf[0, 0, 4] == np.float32(10.0)
    assert el[0, 0, 5] == 3  # particle id of the partner
    # C's first free incoming slot (slot 0) now holds (A, 0)
    assert back(pidx[2, 0]) == 0 and pidx[2, 1] == 0
    o.close()


def test_free_slots_are_taken_in_distance_order():
    q = [C0, C0, C0]
    p1 = [C0 + 1.0, C0, C0]   # closer to Q
    p2 = [C0 - 1.2, C0, C0]
    rs = [[C0, C0 + 3.0, C0], [C0, C0 - 3.0, C0], [C0, C0, C0 + 3.0], [C0, C0, C0 - 3.0],
          [C0, C0 + 2.2, C0 + 2.2]]
    pos = [q, p1, p2] + rs
    bonds = [(1, 0, 2, 0.0, 1000.0, 10.0, 5.0), (2, 0, 1, 0.0, 1000.0, 10.0, 5.0)]
    bonds += [(3 + k, 0, 0, 3.0, 1000.0, 10.0, 9.0) for k in range(5)]
    d, n = scene(pos, bonds=bonds)
    pidx = d.arrays[A.FPARTICLEIDX]
    pidx[0, :] = A.NO_PARTNER
    for k in range(5):  # Q's incoming slots 0..4 hold the five live bonds, slot 5 is free
        pidx[0, 2 * k] = 3 + k
        pidx[0, 2 * k + 1] = 0
    orc.build()
    o = orc.Oracle(d.params, d.genome, n)
    o.upload_all(d.arrays)
    resort(o)
    o.remodel()
    el, pidx, back = sorted_view(o)
    assert back(el[1, 0, 0]) == 0, "the closer proposer takes Q's last free slot"
    assert el.view(np.float32)[2, 0, 2] == 0.0, "the farther proposer stays broken"
    assert back(pidx[0, 10]) == 1 and pidx[0, 11] == 0
    resort(o)
    o.remodel()  # Q is full now and nothing else is within h of P2
    el, _, _ = sorted_view(o)
    assert el.view(np.float32)[2, 0, 2] == 0.0
    o.close()
