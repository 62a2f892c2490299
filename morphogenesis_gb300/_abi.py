"""ctypes mirror of include/mg_abi.h (structs, ids, flags) and the library loader."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
# MG_BUILD_DIR: load a variant built there (morphogenesis_gb300/build.py), else the product build
LIB_PATH = PKG / os.environ.get("MG_BUILD_DIR", "_build") / "libmg_gb300.so"

BONDS_PER_PARTICLE = 6
DATA_PER_BOND = 9
BOND_DATA = BONDS_PER_PARTICLE * DATA_PER_BOND
NUM_TF = 16
NUM_GENES = 16
GRID_UNDEF = 0xFFFFFFFF
NO_PARTNER = 0xFFFFFFFF
EPIGEN_ACTIVE = 2147483647

# buffer ids (fluid.h:138-206)
FPOS, FVEL, FVEVAL, FFORCE, FPRESS, FDENSITY, FAGE, FCOLOR, FGCELL, FGNDX = range(10)
FELASTIDX, FNERVEIDX, FCONC, FEPIGEN, FBIN, FBIN_COUNT, FBIN_OFFSET = 14, 15, 16, 17, 18, 19, 20
FPARTICLEIDX, FPARTICLE_ID, FMASS_RADIUS = 29, 30, 31
FBIN_COUNT_ACTIVE_GENES, FBIN_OFFSET_ACTIVE_GENES, FDENSE_LIST_LENGTHS, FDENSE_LISTS = 32, 33, 34, 35
FBIN_OFFSET_CHANGES, FBIN_COUNT_CHANGES, FDENSE_LIST_LENGTHS_CHANGES, FDENSE_LISTS_CHANGES = 37, 38, 39, 40
NUM_CHANGES = 9

# m_Param ids (fluid_system.h:77-103) + run controls
PSIMSCALE, PVISC, PRESTDENSITY, PMASS, PRADIUS = 4, 7, 8, 9, 10
PSMOOTHRADIUS, PINTSTIFF, PEXTSTIFF, PEXTDAMP, PACCEL_LIMIT, PVEL_LIMIT = 12, 13, 14, 15, 16, 17
PGROUND_SLOPE, PFORCE_MIN, PFORCE_MAX, PFORCE_FREQ, PSURFACE_TENSION = 19, 20, 21, 23, 24
PACTUATION_FACTOR, PACTUATION_PERIOD, PDT, PTIME, PFREEZE = 25, 26, 100, 101, 102

STEP_PHYSICS, STEP_GENES, STEP_REMODEL, STEP_FREEZE, STEP_SURROGATE, STEP_SPECIAL = 1, 2, 4, 8, 16, 32
STEP_BOND_CHANGES = 64
STEP_DEFAULT = STEP_PHYSICS | STEP_GENES

OPT_NEIGHBOR_SEARCH = 1
OPT_HEAL_PARAMS = 2
OPT_CONC_LAYOUT = 3
OPT_REORIGIN_PERIOD = 4
MLP_IN, MLP_H, MLP_OUT = 48, 128, 16
P_W1 = 0
P_B1 = P_W1 + MLP_H * MLP_IN
P_W2 = P_B1 + MLP_H
P_B2 = P_W2 + MLP_H * MLP_H
P_W3 = P_B2 + MLP_H
P_B3 = P_W3 + MLP_OUT * MLP_H
P_COUNT = P_B3 + MLP_OUT
NORM_COUNT = 2 * MLP_IN + 2 * MLP_OUT

MG_OK = 0
MG_OK, MG_ERR_INVALID_ARG, MG_ERR_OOM, MG_ERR_GRID_OVERFLOW, MG_ERR_LIST_OVERFLOW = 0, 1, 2, 3, 4
MG_ERR_DEVICE_TIMEOUT, MG_ERR_CUDA, MG_ERR_UNSUPPORTED, MG_ERR_INCONSISTENT = 5, 6, 7, 8
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "GRID_OVERFLOW", 4: "LIST_OVERFLOW",
                5: "DEVICE_TIMEOUT", 6: "CUDA_ERROR", 7: "UNSUPPORTED", 8: "INCONSISTENT"}

F3 = C.c_float * 3
I3 = C.c_int32 * 3


class FParams(C.Structure):
    _fields_ = [
        ("psimscale", C.c_float), ("psmoothradius", C.c_float), ("pradius", C.c_float),
        ("pmass", C.c_float), ("prest_dens", C.c_float), ("pboundmin", F3), ("pboundmax", F3),
        ("pextstiff", C.c_float), ("pintstiff", C.c_float), ("pvisc", C.c_float),
        ("psurface_t", C.c_float), ("pdamp", C.c_float), ("pforce_min", C.c_float),
        ("pforce_max", C.c_float), ("pforce_freq", C.c_float), ("pground_slope", C.c_float),
        ("pgravity", F3), ("paccel_limit", C.c_float), ("pvel_limit", C.c_float),
        ("actuation_factor", C.c_float), ("actuation_period", C.c_float),
        ("grid_res", I3), ("grid_srch", C.c_int32), ("grid_size", F3), ("grid_delta", F3),
        ("grid_min", F3), ("grid_max", F3), ("grid_total", C.c_int32), ("dt", C.c_float),
        ("time", C.c_float), ("freeze", C.c_int32), ("debug", C.c_int32),
    ]


class Genome(C.Structure):
    _fields_ = [
        ("mutability", C.c_uint32 * NUM_GENES), ("delay", C.c_uint32 * NUM_GENES),
        ("sensitivity", (C.c_float * NUM_TF) * NUM_GENES),
        ("tf_diffusability", C.c_float * NUM_TF), ("tf_breakdown_rate", C.c_float * NUM_TF),
        ("secrete", (C.c_float * (2 * NUM_TF + 1)) * NUM_GENES),
        ("activate", (C.c_float * (2 * NUM_GENES + 1)) * NUM_GENES),
        ("tanh_param", (C.c_float * 8) * 3), ("param", (C.c_float * 12) * 3),
    ]


class MgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class SimParams(C.Structure):
    """mg_simparams: the fields of SimParams.txt."""
    _fields_ = [(n, C.c_float) for n in (
        "time", "dt", "simscale", "grid_density", "visc", "surface_tension", "rest_density", "spacing",
        "mass", "radius", "dist", "smooth_radius", "intstiff", "extstiff", "extdamp", "accel_limit",
        "vel_limit", "grav", "ground_slope", "force_min", "force_max", "force_freq")] + [
        ("plane_grav_dir", C.c_float * 3), ("grid_size", C.c_float), ("volmin", C.c_float * 3),
        ("volmax", C.c_float * 3), ("initmin", C.c_float * 3), ("initmax", C.c_float * 3)]


class Spec(C.Structure):
    """mg_spec: the fields of SpecificationFile.txt."""
    _fields_ = [(n, C.c_uint32) for n in ("num_particles", "demo_type", "sim_space")] + [
        (n, C.c_float) for n in (
            "time", "dt", "gridsize", "spacing", "simscale", "smooth_radius", "visc", "surface_tension",
            "mass", "radius", "intstiff", "extstiff", "extdamp", "accel_limit", "vel_limit", "grav",
            "ground_slope", "force_min", "force_max", "force_freq")] + [
        (n, C.c_float * 3) for n in ("dim", "pos", "volmin", "volmax", "initmin", "initmax")] + [
        (n, C.c_char * 256) for n in ("params_path", "points_path", "genome_path", "out_path")] + [
        (n, C.c_uint32) for n in ("num_files", "steps_per_inner_loop", "steps_per_file", "freeze_steps",
                                  "debug", "file_num")] + [
        (n, C.c_char) for n in ("save_ply", "save_csv", "save_vtp", "gene_activity", "remodelling",
                                "read_genome")] + [
        ("actuation_factor", C.c_float), ("actuation_period", C.c_float)]


class Points(C.Structure):
    """mg_points: host arrays of a particle CSV."""
    _fields_ = [("n", C.c_uint32), ("pos", C.c_void_p), ("vel", C.c_void_p), ("age", C.c_void_p),
                ("color", C.c_void_p), ("elastidx", C.c_void_p), ("particle_id", C.c_void_p),
                ("mass_radius", C.c_void_p), ("nerve", C.c_void_p), ("pidx", C.c_void_p),
                ("conc", C.c_void_p), ("epigen", C.c_void_p), ("conc_species_major", C.c_uint32)]


class IO(C.Structure):
    """mg_io: one buffer of an mg_step_io exchange."""
    _fields_ = [("buf_id", C.c_int32), ("host", C.c_void_p), ("bytes", C.c_size_t)]


# (name, restype, argtypes) of every entry point declared in include/mg_abi.h
H = C.c_void_p
SIGNATURES = [
    ("mg_setup_grid", C.c_int, [C.POINTER(FParams), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float, C.c_int32]),
    ("mg_version", C.c_char_p, []),
    ("mg_last_error", C.c_char_p, [H]),
    ("mg_create", C.c_int, [C.POINTER(FParams), C.POINTER(Genome), C.c_uint32, C.POINTER(H)]),
    ("mg_destroy", C.c_int, [H]),
    ("mg_update_params", C.c_int, [H, C.POINTER(FParams)]),
    ("mg_update_genome", C.c_int, [H, C.POINTER(Genome)]),
    ("mg_set_param", C.c_int, [H, C.c_int32, C.c_float]),
    ("mg_get_params", C.c_int, [H, C.POINTER(FParams)]),
    ("mg_buffer_bytes", C.c_int, [H, C.c_int32, C.POINTER(C.c_size_t)]),
    ("mg_upload", C.c_int, [H, C.c_int32, C.c_void_p, C.c_size_t]),
    ("mg_download", C.c_int, [H, C.c_int32, C.c_void_p, C.c_size_t]),
    ("mg_host_alloc", C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    ("mg_host_free", C.c_int, [C.c_void_p]),
    ("mg_get_counts", C.c_int, [H, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    ("mg_insert_particles", C.c_int, [H]),
    ("mg_prefix_sum_cells", C.c_int, [H]),
    ("mg_counting_sort_full", C.c_int, [H]),
    ("mg_compute_pressure", C.c_int, [H]),
    ("mg_compute_force", C.c_int, [H]),
    ("mg_compute_diffusion", C.c_int, [H]),
    ("mg_compute_genes", C.c_int, [H]),
    ("mg_advance", C.c_int, [H]),
    ("mg_run_physical_sort", C.c_int, [H]),
    ("mg_run_inner_physical_loop", C.c_int, [H]),
    ("mg_run_gene_action", C.c_int, [H]),
    ("mg_step", C.c_int, [H, C.c_uint32, C.c_uint32]),
    ("mg_synchronize", C.c_int, [H]),
    ("mg_time_steps", C.c_int, [H, C.c_uint32, C.c_uint32, C.POINTER(C.c_float)]),
    ("mg_set_option", C.c_int, [H, C.c_int32, C.c_int32]),
    ("mg_mlp_create", C.c_int, [C.c_uint64, C.POINTER(H)]),
    ("mg_mlp_destroy", C.c_int, [H]),
    ("mg_mlp_sizes", C.c_int, [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    ("mg_mlp_get_params", C.c_int, [H, C.c_void_p, C.c_size_t]),
    ("mg_mlp_set_params", C.c_int, [H, C.c_void_p, C.c_size_t]),
    ("mg_mlp_get_norm", C.c_int, [H, C.c_void_p, C.c_size_t]),
    ("mg_mlp_set_norm", C.c_int, [H, C.c_void_p, C.c_size_t]),
    ("mg_mlp_gradients", C.c_int, [H, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_double)]),
    ("mg_mlp_infer", C.c_int, [H, C.c_void_p, C.c_uint32, C.c_void_p]),
    ("mg_mlp_fit_normalization", C.c_int, [H, H]),
    ("mg_mlp_train", C.c_int, [H, H, C.c_uint32, C.c_uint32, C.c_float, C.c_uint64, C.c_void_p]),
    ("mg_dataset_create", C.c_int, [C.c_uint64, C.POINTER(H)]),
    ("mg_dataset_destroy", C.c_int, [H]),
    ("mg_dataset_capture", C.c_int, [H, H, C.c_uint32]),
    ("mg_dataset_size", C.c_int, [H, C.POINTER(C.c_uint64)]),
    ("mg_dataset_read", C.c_int, [H, C.c_uint64, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("mg_set_surrogate", C.c_int, [H, H, C.c_uint32, C.c_uint32, C.c_float]),
    ("mg_surrogate_stats", C.c_int, [H, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_float), C.c_int32]),
    ("mg_profile_enable", C.c_int, [H, C.c_int32]),
    ("mg_profile_read", C.c_int, [H, C.c_int32, C.c_char_p, C.POINTER(C.c_uint32),
                                  C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    ("mg_algorithmic_bytes", C.c_int, [H, C.c_char_p, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("mg_kernel_launches", C.c_uint64, [H]),
    ("mg_run_remodelling", C.c_int, [H]),
    ("mg_compute_bond_changes", C.c_int, [H, C.c_uint32]),
    ("mg_run_remodelling_steps", C.c_int, [H, C.c_uint32]),
    ("mg_zero_vel", C.c_int, [H]),
    ("mg_get_time", C.c_int, [H, C.POINTER(C.c_float)]),
    ("mg_read_simparams", C.c_int, [C.c_char_p, C.POINTER(SimParams)]),
    ("mg_write_simparams", C.c_int, [C.c_char_p, C.POINTER(SimParams)]),
    ("mg_fparams_from_simparams", C.c_int, [C.POINTER(SimParams), C.c_int32, C.POINTER(FParams)]),
    ("mg_read_genome", C.c_int, [C.c_char_p, C.POINTER(Genome)]),
    ("mg_write_genome", C.c_int, [C.c_char_p, C.POINTER(Genome), C.c_int32]),
    ("mg_count_points_csv", C.c_int, [C.c_char_p, C.POINTER(C.c_uint32)]),
    ("mg_read_points_csv", C.c_int, [C.c_char_p, C.POINTER(Points)]),
    ("mg_write_points_csv", C.c_int, [C.c_char_p, C.c_int32, C.POINTER(Points)]),
    ("mg_read_specification", C.c_int, [C.c_char_p, C.POINTER(Spec)]),
    ("mg_write_specification", C.c_int, [C.c_char_p, C.POINTER(Spec)]),
    ("mg_write_results_csv", C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(Spec), C.c_uint32, C.c_uint32,
                                       C.c_uint32, C.c_void_p, C.c_uint32]),
    ("mg_write_points_vtp", C.c_int, [C.c_char_p, C.c_int32, C.POINTER(Points), C.c_uint32, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_float),
                                      C.POINTER(C.c_float)]),
    ("mg_step_io", C.c_int, [H, C.POINTER(IO), C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(IO), C.c_uint32]),
    ("mg_device_bytes", C.c_int, [H, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    ("mg_get_tuning", C.c_int, [H, C.POINTER(C.c_int32)]),
    ("mg_set_tuning", C.c_int, [H, C.POINTER(C.c_int32)]),
    ("mg_get_block_sizes", C.c_int, [H, C.POINTER(C.c_int32)]),
    ("mg_set_block_sizes", C.c_int, [H, C.POINTER(C.c_int32)]),
    ("mg_autotune", C.c_int, [H, C.c_uint32, C.c_uint32, C.POINTER(C.c_int32), C.POINTER(C.c_float)]),
    ("mg_batch_create", C.c_int, [C.POINTER(H), C.c_uint32, C.POINTER(H)]),
    ("mg_batch_destroy", C.c_int, [H]),
    ("mg_batch_step", C.c_int, [H, C.c_uint32, C.c_uint32]),
    ("mg_batch_time_steps", C.c_int, [H, C.c_uint32, C.c_uint32, C.POINTER(C.c_float)]),
    ("mg_prefix_sum_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("mg_selftest_bounded_wait", C.c_int, [C.c_int32, C.c_uint32]),
    ("mg_create_packed", C.c_int, [C.POINTER(FParams), C.POINTER(Genome), C.POINTER(C.c_uint32), C.c_uint32,
                                   C.POINTER(H)]),
    ("mg_instance_ranges", C.c_int, [H, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
]

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads the CUDA extension; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"CUDA extension {p} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
