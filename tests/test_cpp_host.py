"""A compiled C++ host on the boundary: tests/abi_host.cpp, built with g++ against
include/mg_fluid_system.hpp (the FluidSystem-style C++ façade) and include/mg_abi.h, linked to
the CUDA library.  The compile check needs no GPU; the run (GPU) drives the reference's calling
sequence (FluidSetupCL, FluidParamCL, UpdateGenome, AllocateParticles, TransferToCL, one Run2
cycle, legacy steps, TransferFromCL) with FCONC species-major, as the reference host keeps it,
and must give the same bits as the same sequence through the Python binding."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo

ROOT = Path(__file__).resolve().parent.parent
IDS = (A.FPOS, A.FVEL, A.FVEVAL, A.FELASTIDX, A.FPARTICLEIDX, A.FPARTICLE_ID, A.FCONC, A.FEPIGEN)


def compile_host(out: Path) -> Path:
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = out / "abi_host"
    lib = A.LIB_PATH.parent
    cmd = [gxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "abi_host.cpp"), "-o", str(exe), f"-L{lib}", "-lmg_gb300",
           f"-Wl,-rpath,{lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_cpp_host_compiles(built, tmp_path):
    compile_host(tmp_path)


@pytest.mark.gpu
def test_cpp_host_matches_python_binding(built, tmp_path):
    import morphogenesis_gb300 as mg

    exe = compile_host(tmp_path)
    d = demo.make_block(8, "R", seed=0)
    n, steps = d.n, 5
    (tmp_path / "params.bin").write_bytes(bytes(d.params))
    (tmp_path / "genome.bin").write_bytes(bytes(d.genome))
    (tmp_path / "n.txt").write_text(str(n))
    for b in IDS:
        a = d.arrays[b]
        if b == A.FCONC:
            a = np.ascontiguousarray(a.T)  # getConc's species-major layout
        (tmp_path / f"in_{b}.bin").write_bytes(np.ascontiguousarray(a).tobytes())
    r = subprocess.run([str(exe), str(tmp_path), str(steps)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr

    fs = mg.FluidSystem(d.params, d.genome, n)
    fs.TransferToCL({b: d.arrays[b] for b in IDS})
    fs.Run2PhysicalSort()
    fs.Run2InnerPhysicalLoop()
    fs.Run2GeneAction()
    fs.Run(steps)
    for b in IDS:
        want = fs.download(b)
        if b == A.FCONC:
            want = np.ascontiguousarray(want.T)
        got = np.frombuffer((tmp_path / f"out_{b}.bin").read_bytes(), dtype=want.dtype).reshape(want.shape)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"buffer {b} differs"
    fs.close()


@pytest.mark.gpu
def test_species_major_conc_round_trip(built):
    """MG_OPT_CONC_LAYOUT 1: FCONC is exchanged as [16][N] and steps give the same bits."""
    import morphogenesis_gb300 as mg

    d = demo.make_block(10, "R", seed=2)
    a = mg.FluidSystem(d.params, d.genome, d.n)
    b = mg.FluidSystem(d.params, d.genome, d.n)
    b.set_option(A.OPT_CONC_LAYOUT, 1)
    a.TransferToCL(d.arrays)
    b.TransferToCL({**d.arrays, A.FCONC: np.ascontiguousarray(d.arrays[A.FCONC].T)})
    assert np.array_equal(b.download(A.FCONC), a.download(A.FCONC).T)
    a.Run(3)
    b.Run(3)
    assert np.array_equal(b.download(A.FCONC).view(np.uint32), a.download(A.FCONC).T.view(np.uint32))
    a.close()
    b.close()
