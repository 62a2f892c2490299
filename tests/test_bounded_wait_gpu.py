"""Failure detection without a GPU fault: each bounded device-side wait is made to run out
against a flag that nothing sets, and the library must report MG_ERR_DEVICE_TIMEOUT promptly
with the CUDA context still usable (a plain step afterwards matches the oracle).

* The prefix sum's decoupled look-back (the scan kernel of mg_prefix_sum_cells and of every
  step): a scan whose first tile is never launched, so the other tiles wait on a status word
  that is never published.
* The surrogate inference's tensor-core completion wait: an inference CTA whose MMAs are
  withheld, so its mbarrier is never arrived on; the CTA frees its tensor memory and returns.
* The training GEMM's completion wait, the same way (a GEMM CTA with its MMAs withheld).
"""
import time

import numpy as np
import pytest

import oracle as orc
from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1, 2], ids=["scan-look-back", "mlp-completion", "gemm-completion"])
def test_wait_gives_up_and_reports_timeout(built, which):
    lib = A.load()
    t0 = time.perf_counter()
    st = lib.mg_selftest_bounded_wait(which, 1000)
    dt = time.perf_counter() - t0
    assert st == A.MG_ERR_DEVICE_TIMEOUT, f"status {st}: {lib.mg_last_error(None)}"
    assert dt < 10.0, f"the bounded wait took {dt:.1f} s"
    assert lib.mg_selftest_bounded_wait(which, 0) == A.MG_ERR_INVALID_ARG


def test_context_usable_after_timeouts(built):
    import morphogenesis_gb300 as mg

    lib = A.load()
    for which in (0, 1, 2):
        assert lib.mg_selftest_bounded_wait(which, 200) == A.MG_ERR_DEVICE_TIMEOUT
    d = demo.make_block(8, "R", seed=0)
    g = mg.FluidSystem(d.params, d.genome, d.n)
    o = orc.Oracle(d.params, d.genome, d.n)
    g.TransferToCL(d.arrays)
    o.upload_all(d.arrays)
    g.Run(2)
    o.step(2)
    for buf in (A.FPOS, A.FCONC, A.FGCELL):
        assert np.array_equal(g.download(buf).view(np.uint32), o.download(buf).view(np.uint32))
    g.close()
    o.close()
