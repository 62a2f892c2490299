"""The reference's files: SimParams.txt, genome.csv, the particle CSV of SavePointsCSV2,
SpecificationFile.txt, results.csv and the VTP frames of SavePointsVTP2 (C++ readers and writers
in the library, include/mg_abi.h).

    sp = read_simparams("demo/SimParams.txt"); params = fparams_from_simparams(sp)
    genome = read_genome("demo/genome.csv")
    arrays = read_points_csv("demo/particles_pos_vel_color100001.csv")   # {buffer id: array}
    fs = FluidSystem(params, genome, len(arrays[A.FPOS])); fs.TransferToCL(arrays)
    write_points_csv("out", frame, fs)
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi as A
from ._abi import MgError, load


def _check(lib, st, what):
    if st != A.MG_OK:
        raise MgError(st, f"{what}: {(lib.mg_last_error(None) or b'').decode()}")


def read_simparams(path: str | os.PathLike) -> A.SimParams:
    lib = load()
    sp = A.SimParams()
    _check(lib, lib.mg_read_simparams(os.fsencode(path), C.byref(sp)), "read_simparams")
    return sp


def write_simparams(directory: str | os.PathLike, sp: A.SimParams) -> None:
    lib = load()
    _check(lib, lib.mg_write_simparams(os.fsencode(directory), C.byref(sp)), "write_simparams")


def fparams_from_simparams(sp: A.SimParams, gsrch: int = 0) -> A.FParams:
    lib = load()
    p = A.FParams()
    _check(lib, lib.mg_fparams_from_simparams(C.byref(sp), gsrch, C.byref(p)), "fparams_from_simparams")
    return p


def read_genome(path: str | os.PathLike) -> A.Genome:
    lib = load()
    g = A.Genome()
    _check(lib, lib.mg_read_genome(os.fsencode(path), C.byref(g)), "read_genome")
    return g


def write_genome(directory: str | os.PathLike, g: A.Genome, integer_fields: bool = False) -> None:
    lib = load()
    _check(lib, lib.mg_write_genome(os.fsencode(directory), C.byref(g), 1 if integer_fields else 0),
           "write_genome")


_POINT_BUFS = [(A.FPOS, "pos", (4,), np.float32), (A.FVEL, "vel", (4,), np.float32),
               (A.FAGE, "age", (), np.uint32), (A.FCOLOR, "color", (), np.uint32),
               (A.FELASTIDX, "elastidx", (54,), np.uint32), (A.FPARTICLE_ID, "particle_id", (), np.uint32),
               (A.FMASS_RADIUS, "mass_radius", (), np.uint32), (A.FNERVEIDX, "nerve", (), np.uint32),
               (A.FPARTICLEIDX, "pidx", (12,), np.uint32), (A.FCONC, "conc", (16,), np.float32)]


def _points(arrays: dict, n: int) -> A.Points:
    pts = A.Points()
    pts.n = n
    for b, name, tail, dt in _POINT_BUFS:
        x = arrays[b]
        if x.dtype != dt or x.shape != (n, *tail) or not x.flags["C_CONTIGUOUS"]:
            raise ValueError(f"buffer {b}: want a C-contiguous {np.dtype(dt).name} array of shape {(n, *tail)}")
        setattr(pts, name, x.ctypes.data)
    ep = arrays[A.FEPIGEN]
    if ep.dtype != np.uint32 or ep.shape != (16, n) or not ep.flags["C_CONTIGUOUS"]:
        raise ValueError("FEPIGEN: want a C-contiguous uint32 array of shape (16, n)")
    pts.epigen = ep.ctypes.data
    return pts


def read_points_csv(path: str | os.PathLike) -> dict:
    """{buffer id: array} in the mg_upload layouts (FVEVAL is a copy of FVEL, as the reference's
    AddParticleMorphogenesis2 sets it)."""
    lib = load()
    n = C.c_uint32()
    _check(lib, lib.mg_count_points_csv(os.fsencode(path), C.byref(n)), "count_points_csv")
    n = n.value
    arrays = {b: np.zeros((n, *tail), dt) for b, _, tail, dt in _POINT_BUFS}
    arrays[A.FEPIGEN] = np.zeros((16, n), np.uint32)
    pts = _points(arrays, n)
    _check(lib, lib.mg_read_points_csv(os.fsencode(path), C.byref(pts)), "read_points_csv")
    arrays[A.FVEVAL] = arrays[A.FVEL].copy()
    return arrays


def write_points_csv(directory: str | os.PathLike, frame: int, source) -> None:
    """source: {buffer id: array} in the mg_download layouts, or a FluidSystem (downloaded)."""
    lib = load()
    if hasattr(source, "download"):
        arrays = {b: source.download(b) for b, *_ in _POINT_BUFS}
        arrays[A.FEPIGEN] = source.download(A.FEPIGEN)
        n = len(arrays[A.FPOS])
    else:
        arrays = source
        n = len(arrays[A.FPOS])
    pts = _points(arrays, n)
    _check(lib, lib.mg_write_points_csv(os.fsencode(directory), int(frame), C.byref(pts)), "write_points_csv")


def read_specification(directory: str | os.PathLike) -> A.Spec:
    """directory/SpecificationFile.txt (ReadSpecificationFile)."""
    lib = load()
    sp = A.Spec()
    _check(lib, lib.mg_read_specification(os.fsencode(directory), C.byref(sp)), "read_specification")
    return sp


def write_specification(directory: str | os.PathLike, spec: A.Spec) -> None:
    lib = load()
    _check(lib, lib.mg_write_specification(os.fsencode(directory), C.byref(spec)), "write_specification")


def write_results_csv(input_folder: str, output_folder: str | os.PathLike, spec: A.Spec,
                      num_particles_start: int, num_particles_end: int, elastidx: np.ndarray,
                      num_bonds_start: int = 65535) -> None:
    """output_folder/results.csv (WriteResultsCSV); bonds with rest length > 0 are counted from
    elastidx (FELASTIDX layout).  65535 is the reference's marker for the unknown start count."""
    lib = load()
    el = np.ascontiguousarray(elastidx, np.uint32).reshape(-1, A.BOND_DATA)
    _check(lib, lib.mg_write_results_csv(os.fsencode(input_folder), os.fsencode(output_folder), C.byref(spec),
                                         int(num_particles_start), int(num_particles_end), int(num_bonds_start),
                                         el.ctypes.data, len(el)), "write_results_csv")


def write_points_vtp(directory: str | os.PathLike, frame: int, source, volmin, volmax,
                     active: int | None = None) -> None:
    """directory/particles_pos_vel_color{frame+100000}.vtp (SavePointsVTP2's content, VTK XML).
    source: a FluidSystem (downloaded; active = its active count) or {buffer id: array} with the
    point buffers plus FVEVAL, FFORCE, FPRESS, FDENSITY."""
    lib = load()
    bufs = [b for b, *_ in _POINT_BUFS] + [A.FEPIGEN, A.FVEVAL, A.FFORCE, A.FPRESS, A.FDENSITY]
    if hasattr(source, "download"):
        arrays = {b: source.download(b) for b in bufs}
        if active is None:
            active = source.counts()[1]
    else:
        arrays = source
    n = len(arrays[A.FPOS])
    active = n if active is None else int(active)
    pts = _points(arrays, n)
    extra = [np.ascontiguousarray(arrays[b], np.float32) for b in (A.FVEVAL, A.FFORCE, A.FPRESS, A.FDENSITY)]
    lo = (C.c_float * 3)(*volmin)
    hi = (C.c_float * 3)(*volmax)
    _check(lib, lib.mg_write_points_vtp(os.fsencode(directory), int(frame), C.byref(pts), active,
                                        *[e.ctypes.data for e in extra], lo, hi), "write_points_vtp")
