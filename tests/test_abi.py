"""C-ABI library: loads, exports every declared symbol, host-only helpers, and fails loudly
without a GPU.  No GPU needed (no compute calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo

HEADER = Path(__file__).resolve().parent.parent / "include" / "mg_abi.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(mg_\w+)\s*\(", text, re.M)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("mg_create", "mg_destroy", "mg_upload", "mg_download", "mg_step",
                     "mg_insert_particles", "mg_prefix_sum_cells", "mg_counting_sort_full",
                     "mg_compute_pressure", "mg_compute_force", "mg_compute_diffusion",
                     "mg_compute_genes", "mg_advance", "mg_run_physical_sort"):
        assert required in names


def test_library_exports_every_declared_symbol(built):
    lib = C.CDLL(str(A.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared in mg_abi.h but not exported: {missing}"
    assert {n for n, _, _ in A.SIGNATURES} <= set(declared_functions())


def test_struct_sizes_match_header_layout(built):
    # mg_fparams: 27 floats/ints before grid_res ... checked field by field against offsets
    assert C.sizeof(A.FParams) == 4 * (5 + 3 + 3 + 9 + 3 + 4 + 3 + 1 + 3 * 4 + 1 + 4)
    assert C.sizeof(A.Genome) == 4 * (16 + 16 + 256 + 16 + 16 + 16 * 33 * 2 + 24 + 36)


def test_setup_grid_matches_reference_formula(built):
    lib = A.load()
    for param in ("R", "L"):
        ref = demo.make_params(16, param)
        p = A.FParams()
        p.psimscale = ref.psimscale
        p.psmoothradius = ref.psmoothradius
        vmin = (C.c_float * 3)(*ref.grid_min)
        vmax = (C.c_float * 3)(*ref.grid_max)
        cell = float(np.float32(2.0) * np.float32(ref.psmoothradius))  # grid cell 2h (sim units)
        assert lib.mg_setup_grid(C.byref(p), vmin, vmax, cell, 3) == 0
        assert list(p.grid_res) == list(ref.grid_res)
        assert p.grid_total == ref.grid_total
        assert list(p.grid_delta) == list(ref.grid_delta)
        assert p.grid_srch == 3
        # without the override SetupGrid's own formula applies: floor(2*(sr/ss)/cell)+1 = 2
        assert lib.mg_setup_grid(C.byref(p), vmin, vmax, cell, 0) == 0
        assert p.grid_srch == 2


def test_version_and_bad_arguments(built):
    lib = A.load()
    assert b"sm_103a" in lib.mg_version()
    h = C.c_void_p()
    p = demo.make_params(4, "R")
    p.grid_srch = 9
    st = lib.mg_create(C.byref(p), C.byref(demo.make_genome()), 64, C.byref(h))
    assert st == 1 and b"grid_srch" in lib.mg_last_error(None)


def test_create_fails_loudly_without_a_gpu(built):
    """The product path has no CPU fallback: without a device mg_create reports a CUDA error."""
    lib = A.load()
    d = demo.make_block(4, "R")
    h = C.c_void_p()
    st = lib.mg_create(C.byref(d.params), C.byref(d.genome), d.n, C.byref(h))
    if st == 0:
        lib.mg_destroy(h)
        pytest.skip("a GPU is present")
    assert st == 6
    assert lib.mg_last_error(None)
    import morphogenesis_gb300 as mg

    with pytest.raises(mg.MgError):
        mg.FluidSystem(d.params, d.genome, d.n)


def test_demo_block_bond_tables_are_consistent():
    d = demo.make_block(6, "R", seed=2, breakable=True)
    el = d.arrays[A.FELASTIDX].reshape(-1, 6, 9)
    elf = el.view(np.float32)
    pidx = d.arrays[A.FPARTICLEIDX].reshape(-1, 6, 2)
    pid = d.arrays[A.FPARTICLE_ID]
    nbonds = 0
    for i in range(d.n):
        for a in range(6):
            j = el[i, a, 0]
            if j == A.NO_PARTNER:
                continue
            nbonds += 1
            assert pidx[j, a ^ 1, 0] == i and pidx[j, a ^ 1, 1] == a
            assert el[i, a, 5] == pid[j]
            assert elf[i, a, 1] == np.float32(1.5) * elf[i, a, 2]
    assert nbonds == 6 * 6 * 6 * 6 - 6 * 6 * 6  # 6 directions x (n^3 - n^2 boundary faces)
    assert np.isin(d.arrays[A.FEPIGEN], [0, A.EPIGEN_ACTIVE]).all()
