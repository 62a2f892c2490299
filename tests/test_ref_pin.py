"""The oracle against the reference's own kernels (no GPU).

oracle/_ref/libmg_ref.so is the reference's insertParticles, countingSortFull, computePressure,
computeForce, computeDiffusion and advanceParticles (fluid_system_cuda.cu:53-100, 196-296,
620-712, 3167-3358, 3026-3105, 3470-3614) compiled as host C++ from the reference sources
(oracle/ref_harness.cpp, oracle/Makefile `ref`) and run one thread at a time.  Each stage runs
on both sides from the same state and the outputs are compared:

* bit-exact: cells, ranks, counts, offsets, the sorted order and every moved word, bond and
  incoming-bond remap (the reference's "no partner" 65535 read as the oracle's 0xFFFFFFFF),
  pressure and 1/density, diffusion, the strain integrators and break flags of the force
  pass, and integration;
* within FORCE_RTOL: FFORCE, because the reference adds bond reactions to the partner with
  atomicAdd in thread order while the oracle gathers them in slot order (D2), and evaluates
  (sr - r)^3 with pow (D10: t*t*t).

Between stages the reference side takes the oracle's state for the buffers a stage may write
differently within tolerance (FFORCE before advance), so every comparison starts from equal
inputs.  The reference genome holds integers, so the scenes use diffusability 1 and breakdown
rate 1.  When the reference sources are absent (oracle/_ref not built) the tests are skipped;
tests/test_ref_pin_golden.py checks the oracle against vectors this harness produced.
"""
import numpy as np
import pytest

import oracle as orc
from golden.pin_stages import scene
from morphogenesis_gb300 import _abi as A

FORCE_RTOL = 2e-5

pytestmark = pytest.mark.skipif(not orc.build_ref(), reason="reference sources not present")


def norm_partner(x):
    x = np.array(x, np.uint32, copy=True)
    x[x == 65535] = A.NO_PARTNER
    return x


def bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def same(o, r, buf, what):
    x, y = o.download(buf), r.download(buf)
    if buf in (A.FPARTICLEIDX,):
        x, y = norm_partner(x), norm_partner(y)
    assert np.array_equal(bits(x), bits(y)), f"{what}: {buf} differs in {np.count_nonzero(bits(x) != bits(y))} words"


def pair(d):
    o = orc.Oracle(d.params, d.genome, d.n)
    r = orc.RefKernels(d.params, d.genome, d.n)
    o.upload_all(d.arrays)
    r.upload_all(d.arrays)
    return o, r


@pytest.mark.parametrize("kind", ["R", "L", "R-strained"])
def test_stages_match_reference_kernels(built, kind):
    d = scene(kind)
    o, r = pair(d)

    o.insert(); r.insert()
    for b in (A.FGCELL, A.FGNDX, A.FBIN_COUNT):
        same(o, r, b, "insertParticles")
    o.prefix_sum(); r.prefix_sum()
    same(o, r, A.FBIN_OFFSET, "cell offsets")

    o.sort(); r.sort()
    for b in (A.FPOS, A.FVEL, A.FVEVAL, A.FGCELL, A.FGNDX, A.FPARTICLE_ID, A.FMASS_RADIUS,
              A.FNERVEIDX, A.FAGE, A.FCOLOR, A.FCONC, A.FEPIGEN, A.FPARTICLEIDX):
        same(o, r, b, "countingSortFull")
    eo = o.download(A.FELASTIDX).reshape(-1, 6, 9)
    er = r.download(A.FELASTIDX).reshape(-1, 6, 9)
    assert np.array_equal(norm_partner(eo[:, :, 0]), norm_partner(er[:, :, 0])), "bond partner remap"
    for w in range(1, 9):
        assert np.array_equal(eo[:, :, w], er[:, :, w]), f"countingSortFull: FELASTIDX word {w}"

    o.pressure(); r.pressure()
    same(o, r, A.FPRESS, "computePressure")
    same(o, r, A.FDENSITY, "computePressure")

    o.force(); r.force()
    fo, fr = o.download(A.FFORCE)[:, :3], r.download(A.FFORCE)[:, :3]
    scale = float(np.abs(fr).max())
    assert np.allclose(fo, fr, rtol=FORCE_RTOL, atol=FORCE_RTOL * scale), \
        f"computeForce: max |d| {np.abs(fo - fr).max()} (scale {scale})"
    eo = o.download(A.FELASTIDX).reshape(-1, 6, 9)
    er = r.download(A.FELASTIDX).reshape(-1, 6, 9)
    for w in (2, 6, 7):  # rest length (0 when broken), strain^2 and strain integrators
        assert np.array_equal(eo[:, :, w], er[:, :, w]), f"computeForce: FELASTIDX word {w}"
    if kind == "R-strained":
        broken = np.count_nonzero(eo[:, :, 2].view(np.float32) == 0)
        assert broken > 0, "the strained scene should break bonds"

    o.diffusion(); r.diffusion()
    same(o, r, A.FCONC, "computeDiffusion")

    r.upload(A.FFORCE, o.download(A.FFORCE))  # advance from equal forces
    t = o.time()
    o.advance(); r.advance(t)
    for b in (A.FPOS, A.FVEL, A.FVEVAL):
        same(o, r, b, "advanceParticles")
    o.close()
