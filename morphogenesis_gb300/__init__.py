"""GB300-native per-timestep particle pipeline of the Morphogenesis simulator.

``FluidSystem`` mirrors the reference's host API names (src/fluid_system.h) over the C-ABI
of ``include/mg_abi.h``; every stage runs as a hand-written sm_103a kernel of the in-tree
library ``_build/libmg_gb300.so``.  There is no CPU fallback: constructing a FluidSystem
without the built library or without a GPU raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from ._abi import MgError, load  # noqa: F401

__all__ = ["FluidSystem", "MgError", "load", "A", "pinned_empty"]


class _Pinned:
    """Owner of one page-locked host allocation (freed with the last numpy view)."""

    def __init__(self, nbytes: int):
        self.lib = load()
        self.ptr = C.c_void_p()
        st = self.lib.mg_host_alloc(nbytes, C.byref(self.ptr))
        if st != A.MG_OK:
            raise MgError(st, (self.lib.mg_last_error(None) or b"").decode())
        self.nbytes = nbytes

    def __del__(self):
        if self.ptr:
            self.lib.mg_host_free(self.ptr)
            self.ptr = None


def pinned_empty(shape, dtype) -> np.ndarray:
    """numpy array in page-locked host memory (for full-bandwidth transfers)."""
    dt = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dt.itemsize
    owner = _Pinned(max(nbytes, 1))
    buf = (C.c_char * nbytes).from_address(owner.ptr.value)
    arr = np.frombuffer(buf, dtype=dt).reshape(shape)
    return _PinnedArray(arr, owner)


class _PinnedArray(np.ndarray):
    def __new__(cls, arr, owner):
        obj = arr.view(cls)
        obj._owner = owner
        return obj

    def __array_finalize__(self, obj):
        if obj is not None:
            self._owner = getattr(obj, "_owner", None)


def _shape(buf: int, n: int, cells: int):
    f32, u32 = np.float32, np.uint32
    if buf in (A.FPOS, A.FVEL, A.FVEVAL, A.FFORCE):
        return f32, (n, 4)
    if buf in (A.FPRESS, A.FDENSITY):
        return f32, (n,)
    if buf in (A.FAGE, A.FCOLOR, A.FGCELL, A.FGNDX, A.FBIN, A.FPARTICLE_ID, A.FMASS_RADIUS,
               A.FNERVEIDX):
        return u32, (n,)
    if buf == A.FELASTIDX:
        return u32, (n, A.BOND_DATA)
    if buf == A.FPARTICLEIDX:
        return u32, (n, 12)
    if buf == A.FCONC:
        return f32, (n, A.NUM_TF)
    if buf == A.FEPIGEN:
        return u32, (A.NUM_GENES, n)
    if buf in (A.FBIN_COUNT, A.FBIN_OFFSET):
        return u32, (cells,)
    if buf in (A.FBIN_COUNT_ACTIVE_GENES, A.FBIN_OFFSET_ACTIVE_GENES):
        return u32, (A.NUM_GENES, cells)
    if buf == A.FDENSE_LIST_LENGTHS:
        return u32, (A.NUM_GENES,)
    if buf == A.FDENSE_LISTS:
        return u32, (A.NUM_GENES, n)
    if buf in (A.FBIN_COUNT_CHANGES, A.FBIN_OFFSET_CHANGES):
        return u32, (A.NUM_CHANGES, cells)
    if buf == A.FDENSE_LIST_LENGTHS_CHANGES:
        return u32, (A.NUM_CHANGES,)
    if buf == A.FDENSE_LISTS_CHANGES:
        return u32, (A.NUM_CHANGES, 2, n)
    raise ValueError(f"buffer id {buf} is not exchanged")


class FluidSystem:
    """Host object of one simulation (reference: class FluidSystem, fluid_system.h:357-766).

    Setup mirrors FluidSetupCL + FluidParamCL + UpdateGenome + AllocateParticles/AllocateGrid;
    TransferToCL/TransferFromCL move buffers in the reference layouts; the *CL stage methods
    and Run2* loops launch the GPU kernels.
    """

    def __init__(self, params: A.FParams, genome: A.Genome, max_points: int):
        self.lib = load()
        self.params = params
        self.genome = genome
        self.max_points = int(max_points)
        self.cells = int(params.grid_total)
        h = C.c_void_p()
        self._check(self.lib.mg_create(C.byref(params), C.byref(genome), self.max_points, C.byref(h)), None)
        self.h = h

    # -- lifetime -----------------------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.mg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, status: int, h=...) -> None:
        if status != A.MG_OK:
            handle = self.h if h is ... else h
            msg = self.lib.mg_last_error(handle)
            raise MgError(status, (msg or b"").decode())

    # -- parameters -----------------------------------------------------------------------------
    def UpdateParams(self, params: A.FParams | None = None) -> None:
        if params is not None:
            self.params = params
        self._check(self.lib.mg_update_params(self.h, C.byref(self.params)))

    def UpdateGenome(self, genome: A.Genome | None = None) -> None:
        if genome is not None:
            self.genome = genome
        self._check(self.lib.mg_update_genome(self.h, C.byref(self.genome)))

    def SetParam(self, param_id: int, value: float) -> None:
        self._check(self.lib.mg_set_param(self.h, param_id, float(value)))

    def GetParams(self) -> A.FParams:
        p = A.FParams()
        self._check(self.lib.mg_get_params(self.h, C.byref(p)))
        return p

    # -- transfer -------------------------------------------------------------------------------
    def _buf_shape(self, buf: int):
        dt, shape = _shape(buf, self.max_points, self.cells)
        if buf == A.FCONC and getattr(self, "conc_species_major", False):
            shape = (A.NUM_TF, self.max_points)  # getConc's layout (MG_OPT_CONC_LAYOUT 1)
        return dt, shape

    def upload(self, buf: int, arr: np.ndarray) -> None:
        dt, shape = self._buf_shape(buf)
        a = np.ascontiguousarray(arr, dtype=dt)
        if a.shape != shape:
            raise ValueError(f"buffer {buf}: expected shape {shape}, got {a.shape}")
        self._check(self.lib.mg_upload(self.h, buf, a.ctypes.data, a.nbytes))

    def download(self, buf: int, out: np.ndarray | None = None) -> np.ndarray:
        dt, shape = self._buf_shape(buf)
        if out is None:
            out = np.empty(shape, dt)
        self._check(self.lib.mg_download(self.h, buf, out.ctypes.data, out.nbytes))
        return out

    def TransferToCL(self, arrays: dict) -> None:
        for buf, arr in arrays.items():
            self.upload(buf, arr)

    def TransferFromCL(self, bufs=(A.FPOS, A.FVEL, A.FVEVAL, A.FFORCE, A.FPRESS, A.FDENSITY,
                                   A.FELASTIDX, A.FPARTICLEIDX, A.FCONC, A.FEPIGEN,
                                   A.FPARTICLE_ID)) -> dict:
        return {b: self.download(b) for b in bufs}

    def getPos(self) -> np.ndarray:
        return self.download(A.FPOS)

    def getVel(self) -> np.ndarray:
        return self.download(A.FVEL)

    def getElastIdx(self) -> np.ndarray:
        return self.download(A.FELASTIDX)

    def getParticle_Idx(self) -> np.ndarray:
        return self.download(A.FPARTICLEIDX)

    def getConc(self) -> np.ndarray:
        return self.download(A.FCONC)

    def getEpiGen(self) -> np.ndarray:
        return self.download(A.FEPIGEN)

    def counts(self) -> tuple[int, int]:
        """(mNumPoints, mActivePoints) after the last sort."""
        a, b = C.c_uint32(), C.c_uint32()
        self._check(self.lib.mg_get_counts(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    # -- stages (host_CL.cpp *CL wrappers) --------------------------------------------------------
    def InsertParticlesCL(self) -> None: self._check(self.lib.mg_insert_particles(self.h))
    def PrefixSumCellsCL(self) -> None: self._check(self.lib.mg_prefix_sum_cells(self.h))
    def CountingSortFullCL(self) -> None: self._check(self.lib.mg_counting_sort_full(self.h))
    def ComputePressureCL(self) -> None: self._check(self.lib.mg_compute_pressure(self.h))
    def ComputeForceCL(self) -> None: self._check(self.lib.mg_compute_force(self.h))
    def ComputeDiffusionCL(self) -> None: self._check(self.lib.mg_compute_diffusion(self.h))
    def ComputeGenesCL(self) -> None: self._check(self.lib.mg_compute_genes(self.h))
    def AdvanceCL(self) -> None: self._check(self.lib.mg_advance(self.h))
    def ComputeBondChangesCL(self, steps_per_InnerPhysicalLoop: int = 1) -> None:
        self._check(self.lib.mg_compute_bond_changes(self.h, int(steps_per_InnerPhysicalLoop)))
    def ComputeParticleChangesCL(self) -> None: self._check(self.lib.mg_run_remodelling(self.h))
    def ZeroVelCL(self) -> None: self._check(self.lib.mg_zero_vel(self.h))

    def time(self) -> float:
        """m_Time after the steps issued so far."""
        t = C.c_float()
        self._check(self.lib.mg_get_time(self.h, C.byref(t)))
        return t.value

    # -- run loop (fluid_system.cpp Run2*) --------------------------------------------------------
    def Run2PhysicalSort(self) -> None: self._check(self.lib.mg_run_physical_sort(self.h))
    def Run2InnerPhysicalLoop(self) -> None: self._check(self.lib.mg_run_inner_physical_loop(self.h))
    def Run2GeneAction(self) -> None: self._check(self.lib.mg_run_gene_action(self.h))
    def Run2Remodelling(self, steps_per_InnerPhysicalLoop: int | None = None) -> None:
        """With a step count: computeBondChanges over that many inner-loop steps, then heal of
        the slots it flagged (the reference's Run2Remodelling).  Without: heal only (D5 rule)."""
        if steps_per_InnerPhysicalLoop is None:
            self._check(self.lib.mg_run_remodelling(self.h))
        else:
            self._check(self.lib.mg_run_remodelling_steps(self.h, int(steps_per_InnerPhysicalLoop)))

    def Run(self, nsteps: int = 1, flags: int = A.STEP_DEFAULT) -> None:
        """nsteps steps in the legacy Run() order (one sort per step), graph-captured."""
        self._check(self.lib.mg_step(self.h, int(nsteps), int(flags)))

    def step_io(self, inputs: dict, nsteps: int = 1, flags: int = A.STEP_DEFAULT,
                outputs: dict | None = None) -> None:
        """Uploads `inputs` ({buffer id: array}), runs nsteps steps and downloads into `outputs`
        ({buffer id: array}) with one synchronisation (mg_step_io).  Arrays must be C-contiguous
        with the buffer's exact byte size; pinned arrays (pinned_empty) transfer fastest."""
        outputs = outputs or {}
        def pack(d):
            arr = (A.IO * max(1, len(d)))()
            for k, (b, x) in enumerate(d.items()):
                if not x.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"buffer {b}: array must be C-contiguous")
                arr[k].buf_id = int(b)
                arr[k].host = x.ctypes.data
                arr[k].bytes = x.nbytes
            return arr
        i, o = pack(inputs), pack(outputs)
        self._check(self.lib.mg_step_io(self.h, i, len(inputs), nsteps, flags, o, len(outputs)))

    def time_steps(self, nsteps: int, flags: int = A.STEP_DEFAULT) -> float:
        ms = C.c_float()
        self._check(self.lib.mg_time_steps(self.h, int(nsteps), int(flags), C.byref(ms)))
        return float(ms.value)

    def synchronize(self) -> None:
        self._check(self.lib.mg_synchronize(self.h))

    def set_option(self, option: int, value: int) -> None:
        self._check(self.lib.mg_set_option(self.h, int(option), int(value)))
        if option == A.OPT_CONC_LAYOUT:
            self.conc_species_major = bool(value)

    def autotune(self, steps: int = 5, flags: int = A.STEP_DEFAULT) -> dict:
        """Times the density pass's launch shapes, then the force, gather and advance block
        sizes, on the current state (restored after each trial) and keeps the fastest;
        returns the choice and its ms per step."""
        ch = (C.c_int32 * 4)()
        ms = C.c_float()
        self._check(self.lib.mg_autotune(self.h, steps, flags, ch, C.byref(ms)))
        f, g, a = self.block_sizes()
        return {"dens_warps": ch[0], "group_mode": ch[1], "sub_bits": ch[2], "search": ch[3],
                "force_threads": f, "gather_threads": g, "advance_threads": a,
                "ms_per_step": ms.value}

    def block_sizes(self) -> tuple[int, int, int]:
        """Threads per block of the (force, gather, advance) passes."""
        t = (C.c_int32 * 3)()
        self._check(self.lib.mg_get_block_sizes(self.h, t))
        return tuple(t)

    def set_block_sizes(self, force: int, gather: int, advance: int) -> None:
        t = (C.c_int32 * 3)(force, gather, advance)
        self._check(self.lib.mg_set_block_sizes(self.h, t))

    def device_bytes(self) -> tuple[int, int]:
        """(arena bytes, all device bytes the handle holds now)."""
        a, t = C.c_size_t(), C.c_size_t()
        self._check(self.lib.mg_device_bytes(self.h, C.byref(a), C.byref(t)))
        return a.value, t.value

    def tuning(self) -> tuple[int, int, int, int]:
        """(warps per block, search groups, sub-cell bits, neighbour search) of the density pass."""
        ch = (C.c_int32 * 4)()
        self._check(self.lib.mg_get_tuning(self.h, ch))
        return tuple(ch)

    def set_tuning(self, dens_warps: int, group_mode: int, sub_bits: int, search: int = 1) -> None:
        ch = (C.c_int32 * 4)(dens_warps, group_mode, sub_bits, search)
        self._check(self.lib.mg_set_tuning(self.h, ch))

    def profile(self, enable: bool = True) -> None:
        self._check(self.lib.mg_profile_enable(self.h, 1 if enable else 0))

    def profile_read(self) -> dict:
        n = C.c_int32()
        self._check(self.lib.mg_profile_read(self.h, 0, None, None, None, C.byref(n)))
        k = n.value
        names = C.create_string_buffer(32 * max(k, 1))
        launches = (C.c_uint32 * max(k, 1))()
        ms = (C.c_double * max(k, 1))()
        self._check(self.lib.mg_profile_read(self.h, k, names, launches, ms, C.byref(n)))
        out = {}
        for i in range(k):
            nm = names.raw[32 * i:32 * i + 32].split(b"\0", 1)[0].decode()
            out[nm] = (int(launches[i]), float(ms[i]))
        return out

    def algorithmic_bytes(self, kernel: str | None = None, flags: int = A.STEP_DEFAULT):
        bp, bc = C.c_double(), C.c_double()
        self._check(self.lib.mg_algorithmic_bytes(self.h, kernel.encode() if kernel else None,
                                                  flags, C.byref(bp), C.byref(bc)))
        return bp.value, bc.value

    def kernel_launches(self) -> int:
        return int(self.lib.mg_kernel_launches(self.h))


class Batch:
    """Independent systems stepped together: one graph launch per step advances every member
    (parameter sweeps over tissue instances of different sizes, parameters and genomes)."""

    def __init__(self, members):
        self.lib = A.load()
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.h for m in self.members])
        h = C.c_void_p()
        st = self.lib.mg_batch_create(arr, len(self.members), C.byref(h))
        if st != A.MG_OK:
            raise A.MgError(st, (self.lib.mg_last_error(None) or b"").decode())
        self.h = h

    def _check(self, st):
        if st != A.MG_OK:
            raise A.MgError(st, (self.lib.mg_last_error(None) or b"").decode())

    def Run(self, nsteps: int = 1, flags: int = A.STEP_DEFAULT) -> None:
        self._check(self.lib.mg_batch_step(self.h, nsteps, flags))

    def step_io(self, inputs: dict, nsteps: int = 1, flags: int = A.STEP_DEFAULT,
                outputs: dict | None = None) -> None:
        """Uploads `inputs` ({buffer id: array}), runs nsteps steps and downloads into `outputs`
        ({buffer id: array}) with one synchronisation (mg_step_io).  Arrays must be C-contiguous
        with the buffer's exact byte size; pinned arrays (pinned_empty) transfer fastest."""
        outputs = outputs or {}
        def pack(d):
            arr = (A.IO * max(1, len(d)))()
            for k, (b, x) in enumerate(d.items()):
                if not x.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"buffer {b}: array must be C-contiguous")
                arr[k].buf_id = int(b)
                arr[k].host = x.ctypes.data
                arr[k].bytes = x.nbytes
            return arr
        i, o = pack(inputs), pack(outputs)
        self._check(self.lib.mg_step_io(self.h, i, len(inputs), nsteps, flags, o, len(outputs)))

    def time_steps(self, nsteps: int, flags: int = A.STEP_DEFAULT) -> float:
        ms = C.c_float()
        self._check(self.lib.mg_batch_time_steps(self.h, nsteps, flags, C.byref(ms)))
        return ms.value

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.mg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass



# buffers whose entries are particle indices of the same system (shifted when instances are packed)
_INDEX_WORDS = {A.FELASTIDX: (A.BOND_DATA, (0,), 9), A.FPARTICLEIDX: (12, (0,), 2)}


class Packed(FluidSystem):
    """Independent tissues advanced as one system (mg_create_packed): every stage is one kernel
    launch over all instances' particles, each instance keeping its own box, grid, stiffness,
    genome and coordinate frame (so it computes exactly what it computes alone).  Buffers are
    exchanged as one system of sum(counts) particles, instance 0's first (`concat` builds them
    from per-instance arrays, `split` cuts a downloaded buffer back into instances).  The
    reference runs such a sweep as separate jobs (src/slurm/Morphogenesis_param_sweep.slurm)."""

    def __init__(self, params_list, genome_list, counts):
        self.lib = load()
        k = len(params_list)
        if k == 0 or len(genome_list) != k or len(counts) != k:
            raise ValueError("one parameter set, genome and particle count per instance")
        self.counts = [int(c) for c in counts]
        self.offsets = np.concatenate([[0], np.cumsum(self.counts)]).astype(np.int64)
        self.params = params_list[0]
        self.genome = genome_list[0]
        self.max_points = int(self.offsets[-1])
        P = (A.FParams * k)(*params_list)
        G = (A.Genome * k)(*genome_list)
        cnt = (C.c_uint32 * k)(*self.counts)
        h = C.c_void_p()
        self._check(self.lib.mg_create_packed(P, G, cnt, k, C.byref(h)), None)
        self.h = h
        self.cells = int(self.GetParams().grid_total)

    def concat(self, arrays_list) -> dict:
        """Per-instance arrays in the reference layouts -> one dict for TransferToCL: rows
        stacked in instance order (FEPIGEN along its particle axis), bond partners and incoming
        entries shifted by the instance's first slot (no-partner values kept)."""
        out = {}
        for buf in arrays_list[0]:
            parts = []
            for j, arrs in enumerate(arrays_list):
                a = np.array(arrs[buf], copy=True)
                if buf in _INDEX_WORDS:
                    width, cols, stride = _INDEX_WORDS[buf]
                    v = a.reshape(self.counts[j], -1)
                    for c0 in cols:
                        col = v[:, c0::stride]
                        valid = col < self.counts[j]
                        col[valid] += np.uint32(self.offsets[j])
                        col[~valid] = A.NO_PARTNER
                        v[:, c0::stride] = col
                parts.append(a)
            axis = 1 if buf == A.FEPIGEN else 0
            out[buf] = np.ascontiguousarray(np.concatenate(parts, axis=axis))
        return out

    def ranges(self):
        """Sorted-index segment (first, count) of every instance after the last sort."""
        k = len(self.counts)
        first, count = (C.c_uint32 * k)(), (C.c_uint32 * k)()
        self._check(self.lib.mg_instance_ranges(self.h, first, count))
        return [(int(first[j]), int(count[j])) for j in range(k)]

    def split(self, buf: int, arr: np.ndarray | None = None) -> list:
        """A downloaded buffer cut into the instances' sorted segments, indices made local."""
        a = self.download(buf) if arr is None else arr
        out = []
        for (f, c) in self.ranges():
            part = np.array(a[:, f:f + c] if buf == A.FEPIGEN else a[f:f + c], copy=True)
            if buf in _INDEX_WORDS:
                width, cols, stride = _INDEX_WORDS[buf]
                v = part.reshape(c, -1)
                for c0 in cols:
                    col = v[:, c0::stride]
                    inside = (col >= f) & (col < f + c)
                    col[inside] -= np.uint32(f)
                    v[:, c0::stride] = col
            out.append(part)
        return out
