"""mg_prefix_sum_noalloc: the allocation-free prefix sum over caller-owned device arrays,
checked against the handle-based mg_prefix_sum_cells on the same cell counts (bit-exact:
integer work), on two calls in a row.  Device buffers come from torch; the entry point itself
allocates nothing.  Collected last so it also runs after every other GPU test."""
import ctypes as C

import numpy as np
import pytest

import morphogenesis_gb300 as mg
from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo

pytestmark = pytest.mark.gpu

MAX = 67108864  # MG_NOALLOC_SCAN_MAX


def _dev(torch, host_u32):
    return torch.from_numpy(np.ascontiguousarray(host_u32).view(np.int32)).cuda()


def _scan(lib, torch, counts, out, total, err):
    stream = torch.cuda.current_stream().cuda_stream
    return lib.mg_prefix_sum_noalloc(C.c_void_p(counts.data_ptr()), C.c_void_p(out.data_ptr()),
                                     counts.numel(), C.c_void_p(total.data_ptr()),
                                     C.c_void_p(err.data_ptr()), C.c_void_p(stream))


def _u32(t):
    return t.cpu().numpy().view(np.uint32)


def test_noalloc_scan_matches_prefix_sum_cells(built):
    torch = pytest.importorskip("torch")
    lib = A.load()
    d = demo.make_block(32, "R", seed=5)
    fs = mg.FluidSystem(d.params, d.genome, d.n)
    fs.TransferToCL(d.arrays)
    fs.InsertParticlesCL()
    fs.PrefixSumCellsCL()
    counts = fs.download(A.FBIN_COUNT)
    want = fs.download(A.FBIN_OFFSET)
    fs.close()
    assert counts.size > 4 * 4096 and counts.sum() == d.n  # several scan tiles
    dc = _dev(torch, counts)
    outs = [torch.full_like(dc, -1) for _ in range(2)]
    totals = [torch.full((1,), -1, dtype=torch.int32, device="cuda") for _ in range(2)]
    errs = [torch.zeros(1, dtype=torch.int32, device="cuda") for _ in range(2)]
    for k in range(2):  # back to back on one stream, no synchronisation between them
        rc = _scan(lib, torch, dc, outs[k], totals[k], errs[k])
        assert rc == 0, lib.mg_last_error(None)
    torch.cuda.synchronize()
    for k in range(2):
        assert np.array_equal(_u32(outs[k]), want), f"call {k + 1} differs from mg_prefix_sum_cells"
        assert int(_u32(totals[k])[0]) == int(counts.sum())
        assert int(errs[k].item()) == 0


@pytest.mark.parametrize("n", [1, 4095, 4096, 4097, 3 * 4096 + 17, 2_299_968])
def test_noalloc_scan_ragged_sizes(built, n):
    torch = pytest.importorskip("torch")
    lib = A.load()
    r = np.random.default_rng(n)
    counts = r.integers(0, 9, n, dtype=np.uint32)
    want = np.zeros(n, np.uint64)
    want[1:] = np.cumsum(counts[:-1].astype(np.uint64))
    dc = _dev(torch, counts)
    for _ in range(2):
        out = torch.full_like(dc, -1)
        total = torch.full((1,), -1, dtype=torch.int32, device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        assert _scan(lib, torch, dc, out, total, err) == 0, lib.mg_last_error(None)
        torch.cuda.synchronize()
        assert np.array_equal(_u32(out), (want & 0xFFFFFFFF).astype(np.uint32))
        assert int(_u32(total)[0]) == int(counts.astype(np.uint64).sum() & 0xFFFFFFFF)
        assert int(err.item()) == 0


def test_noalloc_scan_allocates_nothing(built):
    """Free device memory is the same before and after repeated calls (buffers made first)."""
    torch = pytest.importorskip("torch")
    lib = A.load()
    n = 3 * 4096 + 5
    counts = np.arange(n, dtype=np.uint32) % 7
    dc = _dev(torch, counts)
    out = torch.empty_like(dc)
    total = torch.zeros(1, dtype=torch.int32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert _scan(lib, torch, dc, out, total, err) == 0  # warm-up: the device code is loaded
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(8):
        assert _scan(lib, torch, dc, out, total, err) == 0, lib.mg_last_error(None)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"


def test_noalloc_scan_limits(built):
    torch = pytest.importorskip("torch")
    lib = A.load()
    dummy = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    # beyond the fixed scratch: rejected before anything is enqueued
    assert lib.mg_prefix_sum_noalloc(p, p, MAX + 1, None, None, stream) == 1
    assert b"maximum" in lib.mg_last_error(None)
    # no arrays with n > 0
    assert lib.mg_prefix_sum_noalloc(None, None, 5, None, None, stream) == 1
    # n == 0 writes a zero total
    total = torch.full((1,), 7, dtype=torch.int32, device="cuda")
    assert lib.mg_prefix_sum_noalloc(None, None, 0, C.c_void_p(total.data_ptr()), None, stream) == 0
    torch.cuda.synchronize()
    assert int(total.item()) == 0
