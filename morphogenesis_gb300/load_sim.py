"""The reference's load_sim driver on the GPU (load_sim.cpp:99-182 with the loop of
Run2Simulation, fluid_system.cpp:2596-2700): reads SpecificationFile.txt from a folder, the
SimParams.txt, genome.csv and particle CSV it names, and runs

    sort; save frame file_num + 90
    freeze phase (bonds do not break), files up to freeze_steps * 100:
        steps_per_file x [steps_per_InnerPhysicalLoop x Run2InnerPhysicalLoop,
                          Run2GeneAction if gene_activity, Run2Remodelling(k) if remodelling,
                          Run2PhysicalSort, ZeroVelCL]
    normal phase up to num_files: the same without ZeroVelCL, frames saved per file
    SimParams.txt, genome.csv, SpecificationFile.txt and results.csv written to outPath

    python -m morphogenesis_gb300.load_sim SPEC_DIR [--out DIR] [--gsrch 3]

Paths in the specification are relative to the working directory, as in the reference.
"""
from __future__ import annotations

import argparse
import os
import time

from . import FluidSystem
from . import _abi as A
from . import files as F


def _save(fs, spec, out, frame, volmin, volmax):
    if spec.save_csv == b"y":
        F.write_points_csv(out, frame, fs)
    if spec.save_vtp == b"y":
        F.write_points_vtp(out, frame, fs, volmin, volmax)


def run(spec_dir: str, out: str | None = None, gsrch: int = 0, verbose: bool = True,
        keep_state: bool = False) -> dict:
    """Runs the specification; returns counts and wall time (and, with keep_state, the final
    buffers {buffer id: array})."""
    spec = F.read_specification(spec_dir)
    sp = F.read_simparams(spec.params_path.decode())
    params = F.fparams_from_simparams(sp, gsrch)
    genome = F.read_genome(spec.genome_path.decode())
    arrays = F.read_points_csv(spec.points_path.decode())
    out = out or spec.out_path.decode()
    os.makedirs(out, exist_ok=True)
    n = len(arrays[A.FPOS])
    volmin, volmax = list(sp.volmin), list(sp.volmax)
    inner, per_file = spec.steps_per_inner_loop, spec.steps_per_file
    t0 = time.perf_counter()
    with FluidSystem(params, genome, n) as fs:
        fs.TransferToCL(arrays)
        file_num = spec.file_num
        fs.SetParam(A.PFREEZE, 1.0)
        fs.Run2PhysicalSort()
        n_start = fs.counts()[1]
        _save(fs, spec, out, file_num + 90, volmin, volmax)
        file_num += 100

        def cycle(zero_vel: bool):
            for _ in range(per_file):
                for _ in range(inner):
                    fs.Run2InnerPhysicalLoop()
                if spec.gene_activity == b"y":
                    fs.Run2GeneAction()
                if spec.remodelling == b"y":
                    fs.Run2Remodelling(inner)
                fs.Run2PhysicalSort()
                if zero_vel:
                    fs.ZeroVelCL()

        while file_num <= spec.freeze_steps * 100:
            cycle(True)
            file_num += 100
        fs.SetParam(A.PFREEZE, 0.0)
        while file_num < spec.num_files:
            cycle(False)
            _save(fs, spec, out, file_num + 90, volmin, volmax)
            if verbose:
                print(f"File# {file_num}.", flush=True)
            file_num += 100
        fs.synchronize()
        n_end = fs.counts()[1]
        sp.time = fs.time()
        F.write_simparams(out, sp)
        F.write_genome(out, genome, integer_fields=False)
        F.write_specification(out, spec)
        F.write_results_csv(spec_dir, out, spec, n_start, n_end, fs.download(A.FELASTIDX))
        state = fs.TransferFromCL() if keep_state else None
    res = {"particles": n, "active_start": n_start, "active_end": n_end,
           "seconds": time.perf_counter() - t0}
    if keep_state:
        res["state"] = state
    return res


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("spec_dir")
    ap.add_argument("--out", default=None)
    ap.add_argument("--gsrch", type=int, default=0)
    a = ap.parse_args(argv)
    print(run(a.spec_dir, a.out, a.gsrch))


if __name__ == "__main__":
    main()
