"""Writes tests/golden/ref_pins.json: outputs of the reference's own kernels (the harness
oracle/ref_harness.cpp, built from the reference sources by `make -C oracle ref`) on three
scenes of 8^3 particles, stage by stage (see pin_stages.py).

    python tests/golden/gen_ref_pins.py

Per scene: the SHA-256 of every bit-exact output of insertParticles, the cell scan,
countingSortFull, computePressure, computeForce (bond words), computeDiffusion and
advanceParticles; the reference's FFORCE (float32, base64) for the within-tolerance check; and
the forces the integration starts from (the oracle's gathered sums, D2), so that every
implementation integrates from the same input.  Needs the reference sources; the tests that
read the file do not.
"""
from __future__ import annotations

import base64
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
for p in (ROOT, ROOT / "oracle", ROOT / "tests"):
    sys.path.insert(0, str(p))

import oracle as orc  # noqa: E402
from golden.pin_stages import ORDER, run_stages, scene  # noqa: E402
from morphogenesis_gb300 import _abi as A  # noqa: E402

SIDE = 8
KINDS = ("R", "L", "R-strained")


def b64(a: np.ndarray) -> str:
    return base64.b64encode(np.ascontiguousarray(a, np.float32).tobytes()).decode()


def oracle_force(d) -> np.ndarray:
    o = orc.Oracle(d.params, d.genome, d.n)
    o.upload_all(d.arrays)
    for st in ("insert", "prefix_sum", "sort", "pressure", "force"):
        getattr(o, st)()
    f = o.download(A.FFORCE)
    o.close()
    return f


def main() -> None:
    orc.build()
    if not orc.build_ref():
        raise SystemExit("the reference sources are needed to build oracle/_ref")
    out = {"side": SIDE, "stages": list(ORDER), "scenes": {}}
    for kind in KINDS:
        d = scene(kind, SIDE)
        adv = oracle_force(d)
        r = orc.RefKernels(d.params, d.genome, d.n)
        r.upload_all(d.arrays)
        t0 = float(d.params.time)
        calls = {"insert": r.insert, "scan": r.prefix_sum, "sort": r.sort, "pressure": r.pressure,
                 "force": r.force, "diffusion": r.diffusion, "advance": lambda: r.advance(t0)}
        rec = run_stages(lambda st: calls[st](), r.download, lambda f: r.upload(A.FFORCE, f), adv)
        ref_force = rec["force"].pop("FFORCE")
        out["scenes"][kind] = {"n": d.n, "digests": rec, "ref_force": b64(ref_force),
                               "advance_force": b64(adv)}
    (HERE / "ref_pins.json").write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", HERE / "ref_pins.json")


if __name__ == "__main__":
    main()
