"""The bounds-checking build: MG_BOUNDS_CHECK=1 checks every data-dependent index of the sort's
gather (the permutation, the origins), the density pass (the processing order, window cells,
candidates, list entries) and the force pass (the origin, the recorded fluid neighbours)
against its buffer; an index past it sets ERR_INDEX, is replaced by one inside the buffer and
turns the step's status into MG_ERR_CUDA.  This stands in for a memory checker, which is not
available where the GPU runs.

The variant is built into morphogenesis_gb300/_build_check and loaded by a child pytest
(MG_BUILD_DIR), which runs the random operation sequences, the edge cases (empty, ragged,
dropped, revived particles), the remodelling tests and a full-size step; any index error fails
them.
"""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


def test_bounds_checking_build_records_no_index_error(built):
    env = dict(os.environ, MG_NVCC_EXTRA="-DMG_BOUNDS_CHECK=1", MG_BUILD_DIR="_build_check")
    cmd = [sys.executable, "-m", "pytest", "-q", "-m", "gpu", "-x", "-p", "no:cacheprovider",
           "tests/test_random_ops_gpu.py",
           "tests/test_parity_gpu.py::test_edge_empty_ragged_and_dropped",
           "tests/test_parity_gpu.py::test_remodelling_reforms_identically",
           "tests/test_parity_gpu.py::test_crowded_cell_orders",
           "tests/test_full_size_gpu.py"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=1800)
    tail = (r.stdout + r.stderr)[-3000:]
    assert r.returncode == 0, f"bounds-checking build failed its runs:\n{tail}"
    # the child loaded the variant, not the product library
    assert (ROOT / "morphogenesis_gb300" / "_build_check" / "libmg_gb300.so").exists()
