"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, and
only as the checker or the timed CPU reference.  Parity status: pinned by the reference's own
kernels.  RefKernels runs the reference's insertParticles, countingSortFull, computePressure,
computeForce, computeDiffusion and advanceParticles compiled as host C++ from the reference
sources (oracle/ref_harness.cpp); tests/test_ref_pin.py compares the oracle with them stage by
stage, and tests/golden/ref_pins.json holds their outputs for machines without the sources.
The gene reaction (D3) and the remodelling decisions (D5, D12) are pinned by the hand-derived
known-answer tests in tests/golden/ only.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
ROOT = HERE.parent

import sys  # noqa: E402

if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
from morphogenesis_gb300 import _abi as A  # noqa: E402  (struct layouts of include/mg_abi.h)


class Derived(C.Structure):
    _fields_ = [("r2", C.c_float), ("H", C.c_float), ("d2", C.c_float), ("rd2", C.c_float),
                ("wendlandC2kern", C.c_float), ("AL2", C.c_float), ("VL2", C.c_float),
                ("pdist", C.c_float), ("gridScanMax", C.c_int32 * 3), ("gridAdjCnt", C.c_int32),
                ("gridAdj", C.c_int32 * 64), ("nadj", C.c_int32)]


def build() -> None:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


_libs: dict[int, C.CDLL] = {}


def lib(bits: int = 32) -> C.CDLL:
    if bits in _libs:
        return _libs[bits]
    path = BUILD / f"liboracle_f{bits}.so"
    if not path.exists():
        build()
    L = C.CDLL(str(path))
    H = C.c_void_p
    sig = {
        "mgo_precision_bits": (C.c_int, []),
        "mgo_create": (H, [C.POINTER(A.FParams), C.POINTER(A.Genome), C.c_uint32]),
        "mgo_destroy": (None, [H]),
        "mgo_update_params": (C.c_int, [H, C.POINTER(A.FParams)]),
        "mgo_update_genome": (C.c_int, [H, C.POINTER(A.Genome)]),
        "mgo_get_derived": (None, [H, C.POINTER(Derived)]),
        "mgo_get_time": (C.c_float, [H]),
        "mgo_import": (C.c_int, [H, C.c_int32, C.c_void_p, C.c_size_t]),
        "mgo_export": (C.c_int, [H, C.c_int32, C.c_void_p, C.c_size_t]),
        "mgo_export_f64": (C.c_int, [H, C.c_int32, C.c_void_p, C.c_size_t]),
        "mgo_get_counts": (None, [H, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
        "mgo_insert_particles": (None, [H]),
        "mgo_prefix_sum_cells": (None, [H]),
        "mgo_counting_sort_full": (None, [H]),
        "mgo_compute_pressure": (None, [H]),
        "mgo_compute_force": (None, [H]),
        "mgo_compute_diffusion": (None, [H]),
        "mgo_compute_genes": (None, [H]),
        "mgo_advance": (None, [H]),
        "mgo_remodel": (None, [H]),
        "mgo_compute_bond_changes": (None, [H, C.c_uint32]),
        "mgo_set_heal_params": (None, [H, C.c_int]),
        "mgo_tanh_cw": (C.c_float, [C.c_float]),
        "mgo_step": (None, [H, C.c_uint32, C.c_uint32]),
        "mgo_set_threads": (C.c_int, [C.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _libs[bits] = L
    return L


def buffer_shape(buf: int, n: int, cells: int):
    """numpy (dtype, shape) of a buffer id in the reference layout."""
    f32, u32 = np.float32, np.uint32
    table = {
        A.FPOS: (f32, (n, 4)), A.FVEL: (f32, (n, 4)), A.FVEVAL: (f32, (n, 4)),
        A.FFORCE: (f32, (n, 4)), A.FPRESS: (f32, (n,)), A.FDENSITY: (f32, (n,)),
        A.FAGE: (u32, (n,)), A.FCOLOR: (u32, (n,)), A.FGCELL: (u32, (n,)), A.FGNDX: (u32, (n,)),
        A.FBIN: (u32, (n,)), A.FPARTICLE_ID: (u32, (n,)), A.FMASS_RADIUS: (u32, (n,)),
        A.FNERVEIDX: (u32, (n,)), A.FELASTIDX: (u32, (n, A.BOND_DATA)),
        A.FPARTICLEIDX: (u32, (n, 12)), A.FCONC: (f32, (n, A.NUM_TF)),
        A.FEPIGEN: (u32, (A.NUM_GENES, n)), A.FBIN_COUNT: (u32, (cells,)),
        A.FBIN_OFFSET: (u32, (cells,)), A.FBIN_COUNT_ACTIVE_GENES: (u32, (A.NUM_GENES, cells)),
        A.FBIN_OFFSET_ACTIVE_GENES: (u32, (A.NUM_GENES, cells)),
        A.FDENSE_LIST_LENGTHS: (u32, (A.NUM_GENES,)), A.FDENSE_LISTS: (u32, (A.NUM_GENES, n)),
        A.FBIN_COUNT_CHANGES: (u32, (A.NUM_CHANGES, cells)), A.FBIN_OFFSET_CHANGES: (u32, (A.NUM_CHANGES, cells)),
        A.FDENSE_LIST_LENGTHS_CHANGES: (u32, (A.NUM_CHANGES,)),
        A.FDENSE_LISTS_CHANGES: (u32, (A.NUM_CHANGES, 2, n)),
    }
    return table[buf]


class Oracle:
    """CPU restatement of the reference step, buffers exchanged in the reference layouts."""

    def __init__(self, params: A.FParams, genome: A.Genome, max_points: int, bits: int = 32):
        self.L = lib(bits)
        self.bits = bits
        self.n = max_points
        self.cells = params.grid_total
        self.h = self.L.mgo_create(C.byref(params), C.byref(genome), max_points)
        if not self.h:
            raise RuntimeError("mgo_create failed")

    def close(self):
        if self.h:
            self.L.mgo_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def upload(self, buf: int, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr)
        rc = self.L.mgo_import(self.h, buf, a.ctypes.data, a.nbytes)
        if rc:
            raise RuntimeError(f"mgo_import({buf}) failed: {rc}")

    def upload_all(self, arrays: dict) -> None:
        for k, v in arrays.items():
            self.upload(k, v)

    def download(self, buf: int) -> np.ndarray:
        dt, shape = buffer_shape(buf, self.n, self.cells)
        out = np.empty(shape, dt)
        rc = self.L.mgo_export(self.h, buf, out.ctypes.data, out.nbytes)
        if rc:
            raise RuntimeError(f"mgo_export({buf}) failed: {rc}")
        return out

    def download_f64(self, buf: int) -> np.ndarray:
        dt, shape = buffer_shape(buf, self.n, self.cells)
        out = np.empty(shape, np.float64)
        rc = self.L.mgo_export_f64(self.h, buf, out.ctypes.data, out.size)
        if rc:
            raise RuntimeError(f"mgo_export_f64({buf}) failed: {rc}")
        return out

    def derived(self) -> Derived:
        d = Derived()
        self.L.mgo_get_derived(self.h, C.byref(d))
        return d

    def counts(self):
        a, b = C.c_uint32(), C.c_uint32()
        self.L.mgo_get_counts(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def time(self) -> float:
        return float(self.L.mgo_get_time(self.h))

    def insert(self): self.L.mgo_insert_particles(self.h)
    def prefix_sum(self): self.L.mgo_prefix_sum_cells(self.h)
    def sort(self): self.L.mgo_counting_sort_full(self.h)
    def pressure(self): self.L.mgo_compute_pressure(self.h)
    def force(self): self.L.mgo_compute_force(self.h)
    def diffusion(self): self.L.mgo_compute_diffusion(self.h)
    def genes(self): self.L.mgo_compute_genes(self.h)
    def advance(self): self.L.mgo_advance(self.h)
    def remodel(self): self.L.mgo_remodel(self.h)
    def bond_changes(self, steps: int = 1): self.L.mgo_compute_bond_changes(self.h, int(steps))
    def update_params(self, params: A.FParams):
        if self.L.mgo_update_params(self.h, C.byref(params)):
            raise RuntimeError("mgo_update_params failed")
    def set_heal_params(self, mode: int): self.L.mgo_set_heal_params(self.h, int(mode))

    def step(self, nsteps: int = 1, flags: int = A.STEP_DEFAULT) -> None:
        self.L.mgo_step(self.h, nsteps, flags)


def set_threads(n: int, bits: int = 32) -> int:
    return lib(bits).mgo_set_threads(n)


FP64_FIELDS = {"FPOS": A.FPOS, "FVEL": A.FVEL, "FVEVAL": A.FVEVAL, "FFORCE": A.FFORCE,
               "FPRESS": A.FPRESS, "FDENSITY": A.FDENSITY, "FCONC": A.FCONC}


def fp64_error_report(download, o64: "Oracle") -> dict:
    """Per-field error of an FP32 result against the FP64 oracle run of the same steps.

    `download(buf)` returns the FP32 result's buffer in the reference layout (GPU or FP32
    oracle); `o64` is an Oracle built with bits=64 that ran the same steps from the same
    inputs.  Particles are matched by FPARTICLE_ID, so a particle binned differently in double
    precision is still compared with itself.  Per field (fields written by computePressure,
    computeForce and advanceParticles, fluid_system_cuda.cu:620-712, 3167-3358, 3470-3614, and
    FCONC by computeDiffusion/computeGeneAction): rel_l2 = |x - y|_2 / |y|_2, rel_max =
    max|x - y| / max|y|, rel_median = median |x - y| / (|y| + 1e-6 max|y|).  The w word of the
    float4 fields is not compared.
    """
    ida = np.asarray(download(A.FPARTICLE_ID))
    idb = o64.download(A.FPARTICLE_ID)
    pa = np.argsort(ida, kind="stable")
    pb = np.argsort(idb, kind="stable")
    if not np.array_equal(ida[pa], idb[pb]):
        raise AssertionError("the FP32 result and the FP64 oracle hold different particles")
    out = {}
    for name, buf in FP64_FIELDS.items():
        x = np.asarray(download(buf), np.float64)[pa]
        y = o64.download_f64(buf)[pb]
        if x.ndim == 2 and x.shape[1] == 4:
            x, y = x[:, :3], y[:, :3]
        d = np.abs(x - y)
        s = float(np.abs(y).max()) if y.size else 0.0
        ny = float(np.linalg.norm(y))
        out[name] = {"rel_l2": float(np.linalg.norm(x - y) / ny) if ny > 0 else float(np.linalg.norm(x - y)),
                     "rel_max": float(d.max() / s) if s > 0 else float(d.max()),
                     "rel_median": float(np.median(d / (np.abs(y) + 1e-6 * s))) if s > 0 else float(np.median(d))}
    return out


REF_LIB = HERE / "_ref" / "libmg_ref.so"
REF_SRC = Path("/root/reference/Morphogenesis/src")


def build_ref() -> bool:
    """Builds the pinning harness (the reference's kernels as host C++, oracle/ref_harness.cpp)
    when the reference sources are present; returns whether the library exists."""
    if (REF_SRC / "fluid_system_cuda.cu").exists():
        r = subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF_SRC={REF_SRC}"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference harness build failed:\n" + r.stdout + r.stderr)
    return REF_LIB.exists()


class RefKernels:
    """The reference's own insertParticles, countingSortFull, computePressure, computeForce,
    computeDiffusion and advanceParticles run serially on the host (oracle/ref_harness.cpp),
    with the buffer exchange of Oracle.  One instance at a time (the kernels use globals)."""

    _lib = None

    def __init__(self, params: A.FParams, genome: A.Genome, max_points: int):
        if RefKernels._lib is None:
            L = C.CDLL(str(REF_LIB))
            for name, res, args in (
                    ("mgr_create", C.c_int, [C.POINTER(A.FParams), C.POINTER(A.Genome), C.c_uint32]),
                    ("mgr_import", C.c_int, [C.c_int32, C.c_void_p, C.c_size_t]),
                    ("mgr_export", C.c_int, [C.c_int32, C.c_void_p, C.c_size_t]),
                    ("mgr_insert", None, []), ("mgr_scan", None, []), ("mgr_sort", None, []),
                    ("mgr_pressure", None, []), ("mgr_force", None, [C.c_int]),
                    ("mgr_diffusion", None, []),
                    ("mgr_advance", None, [C.c_float, C.c_float, C.c_float])):
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            RefKernels._lib = L
        self.L = RefKernels._lib
        self.n = max_points
        self.cells = params.grid_total
        self.params = params
        self.L.mgr_create(C.byref(params), C.byref(genome), max_points)

    def upload(self, buf: int, arr: np.ndarray) -> None:
        a = np.ascontiguousarray(arr)
        if self.L.mgr_import(buf, a.ctypes.data, a.nbytes):
            raise RuntimeError(f"mgr_import({buf}) failed")

    def upload_all(self, arrays: dict) -> None:
        for k, v in arrays.items():
            self.upload(k, v)

    def download(self, buf: int) -> np.ndarray:
        dt, shape = buffer_shape(buf, self.n, self.cells)
        out = np.empty(shape, dt)
        if self.L.mgr_export(buf, out.ctypes.data, out.nbytes):
            raise RuntimeError(f"mgr_export({buf}) failed")
        return out

    def insert(self): self.L.mgr_insert()
    def prefix_sum(self): self.L.mgr_scan()
    def sort(self): self.L.mgr_sort()
    def pressure(self): self.L.mgr_pressure()
    def force(self, freeze: bool = False): self.L.mgr_force(int(freeze))
    def diffusion(self): self.L.mgr_diffusion()

    def advance(self, time: float):
        p = self.params
        self.L.mgr_advance(time, p.dt, p.psimscale)
