"""Generates tests/golden/kats.json: known-answer vectors for the oracle.

The reference ships no tests or golden vectors, so these cases are derived by hand from the
reference kernel formulas (Morphogenesis src/fluid_system_cuda.cu) and evaluated here in
float64 with plain Python arithmetic, independently of the oracle's C code:

* pair_density    - contributePressure/computePressure (cuda:620-712) for two particles
* lone_density    - an isolated particle: sum == 0 -> density 1 (cuda:697)
* bond_spring     - one stretched bond, no fluid contact (computeForce, cuda:3263-3313)
* pair_diffusion  - contributeDiffusion/computeDiffusion for two particles (cuda:3026-3105)
* advance_free    - advanceParticles leap-frog with walls out of reach (cuda:3470-3614)
* advance_clamp   - the same with the acceleration limit AL active
* gene_reaction   - computeGeneAction + tally for one living particle (cuda:714-772)
* scan            - exclusive prefix sum (cuda:147-183, zero_offsets = 1)
Run: python tests/golden/gen_kats.py
"""
from __future__ import annotations

import json
import math
from pathlib import Path

OUT = Path(__file__).with_name("kats.json")

MASS, REST, ISTIFF = 2.0543e-4, 600.0, 1.0
WC2 = 21.0 / (2 * 3.141592)


def wendland_pair(r, sr):
    q = r / sr
    b = (1 - q) ** 4
    return b * (4 * q + 1)


def main():
    kats = {}
    # two particles at distance 1.0, smoothing radius 2 (simulation scale 1)
    s = wendland_pair(1.0, 2.0)
    rho = s * MASS * WC2
    kats["pair_density"] = {"sr": 2.0, "ss": 1.0, "r": 1.0,
                            "press": (rho - REST) * ISTIFF, "invdens": 1.0 / rho}
    kats["lone_density"] = {"press": (1.0 - REST) * ISTIFF, "invdens": 1.0}
    # bond: rest length 1.0, stretched to 1.25 along x (dsq > 1: no fluid term)
    L0, d, mod, damp = 1.0, 1.25, 1000.0, 10.0
    strain = (d - L0) / L0
    # owner i at x, partner j at x + d: dist = pos_i - pos_j = -d, unit -1, no relative velocity;
    # eterm = (unit * strain * modulus) / mass; owner gets -eterm, partner +eterm
    e = (-1.0 * strain * mod) / MASS
    kats["bond_spring"] = {"L0": L0, "d": d, "modulus": mod, "damping": damp,
                           "force_owner_x": -e, "force_partner_x": e,
                           "strain_sq": strain * strain, "strain": strain}
    # diffusion between two particles at distance 1.5, sr = 2, ss = 1, rate 0.1, decay 0.01
    r2 = (2.0 * 2.0) / (1.0 * 1.0)
    c = (r2 - 1.5 * 1.5) * 1.0
    ci, cj, dif, brk = 0.25, 0.75, 0.1, 0.99
    kats["pair_diffusion"] = {"ci": ci, "cj": cj, "d": 1.5, "rate": dif, "breakdown": brk,
                              "new_i": brk * (ci + dif * c * (cj - ci)),
                              "new_j": brk * (cj + dif * c * (ci - cj))}
    # leap-frog with accel (1, 2, -3) + gravity (0,-9.8,0), v = (0.5, 0, 0), dt = 1e-3
    a = [1.0, 2.0 - 9.8, -3.0]
    v = [0.5, 0.0, 0.0]
    dt = 1e-3
    vn = [a[k] * dt + v[k] for k in range(3)]
    kats["advance_free"] = {"force": [1.0, 2.0, -3.0], "vel": v, "dt": dt,
                            "vel_new": vn, "veval_new": [(v[k] + vn[k]) * 0.5 for k in range(3)],
                            "dpos": [vn[k] * dt for k in range(3)]}
    big = [300.0, 400.0, 0.0]
    ag = [big[0], big[1] - 9.8, big[2]]
    sp = math.sqrt(sum(x * x for x in ag))
    ac = [x * 150.0 / sp for x in ag]
    kats["advance_clamp"] = {"force": big, "AL": 150.0, "dt": dt,
                             "vel_new": [ac[k] * dt for k in range(3)]}
    # gene reaction: genes 0 and 2 active (2 = living), sens[0] = (0.5 on tf 1, -0.25 on tf 3),
    # sens[2] = (1.0 on tf 0); gene g secretes tf g at rate 0.1
    conc = [0.2, 0.4, 0.6, 0.8] + [0.0] * 12
    act0 = 0.5 * conc[1] + (-0.25) * conc[3]
    act2 = 1.0 * conc[0]
    out = list(conc)
    out[0] += 0.1 * act0
    out[2] += 0.1 * act2
    kats["gene_reaction"] = {"conc": conc, "conc_new": out, "act0": act0, "act2": act2}
    arr = [3, 0, 5, 1, 0, 0, 7, 2]
    pre, run = [], 0
    for x in arr:
        pre.append(run)
        run += x
    kats["scan"] = {"in": arr, "out": pre, "total": run}
    OUT.write_text(json.dumps(kats, indent=1, sort_keys=True) + "\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
