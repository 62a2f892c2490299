"""The load_sim driver (SpecificationFile.txt -> SimParams, genome, particle CSV -> the Run2 loop
with its freeze phase, gene action and remodelling -> CSV / VTP frames and results.csv) against
the oracle running the same stage sequence: the final state is bitwise equal."""
import copy
import os

import numpy as np
import pytest

import oracle as orc
from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo
from morphogenesis_gb300 import files as F
from morphogenesis_gb300 import load_sim

pytestmark = pytest.mark.gpu


def write_inputs(tmp_path):
    d = demo.make_block(8, "R", seed=2, breakable=True)
    p = d.params
    sp = A.SimParams()
    for k, v in dict(time=0.0, dt=p.dt, simscale=p.psimscale, grid_density=1.0, visc=p.pvisc,
                     surface_tension=p.psurface_t, rest_density=p.prest_dens, spacing=1.0, mass=p.pmass,
                     radius=p.pradius, dist=1.0, smooth_radius=p.psmoothradius, intstiff=p.pintstiff,
                     extstiff=p.pextstiff, extdamp=p.pdamp, accel_limit=p.paccel_limit,
                     vel_limit=p.pvel_limit, grav=9.8, ground_slope=p.pground_slope, force_min=0.0,
                     force_max=0.0, force_freq=p.pforce_freq, grid_size=0.0).items():
        setattr(sp, k, v)
    sp.plane_grav_dir[:] = (0, -1, 0)
    sp.volmin[:] = list(p.pboundmin)
    sp.volmax[:] = list(p.pboundmax)
    sp.initmin[:] = list(p.pboundmin)
    sp.initmax[:] = list(p.pboundmax)
    inp = tmp_path / "in"
    inp.mkdir()
    F.write_simparams(inp, sp)
    F.write_genome(inp, d.genome)
    arrays = dict(d.arrays)
    for b in (A.FAGE, A.FCOLOR, A.FMASS_RADIUS, A.FNERVEIDX):
        arrays[b] = np.zeros(d.n, np.uint32)
    F.write_points_csv(inp, 1, arrays)
    spec = A.Spec()
    spec.num_particles = d.n
    spec.dt, spec.simscale, spec.smooth_radius = p.dt, p.psimscale, p.psmoothradius
    spec.params_path = str(inp / "SimParams.txt").encode()
    spec.genome_path = str(inp / "genome.csv").encode()
    spec.points_path = str(inp / "particles_pos_vel_color100001.csv").encode()
    spec.out_path = str(tmp_path / "out").encode()
    spec.num_files, spec.steps_per_inner_loop, spec.steps_per_file, spec.freeze_steps = 400, 2, 2, 1
    spec.save_ply, spec.save_csv, spec.save_vtp = b"n", b"y", b"y"
    spec.gene_activity, spec.remodelling, spec.read_genome = b"y", b"y", b"y"
    F.write_specification(inp, spec)
    return inp, spec


def test_load_sim_matches_oracle(built, tmp_path):
    inp, spec = write_inputs(tmp_path)
    res = load_sim.run(str(inp), gsrch=3, verbose=False, keep_state=True)
    out = tmp_path / "out"
    for f in ("particles_pos_vel_color100090.csv", "particles_pos_vel_color100390.vtp", "results.csv",
              "SimParams.txt", "genome.csv", "SpecificationFile.txt"):
        assert (out / f).exists(), f
    assert "timesteps=,16," in (out / "results.csv").read_text()
    # the oracle runs the same sequence from the same files
    sp = F.read_simparams(inp / "SimParams.txt")
    params = F.fparams_from_simparams(sp, 3)
    genome = F.read_genome(inp / "genome.csv")
    arrays = F.read_points_csv(inp / "particles_pos_vel_color100001.csv")
    n = len(arrays[A.FPOS])
    o = orc.Oracle(params, genome, n)
    o.upload_all(arrays)
    frozen = copy.copy(params)
    frozen.freeze = 1
    frozen.time = o.time()
    o.update_params(frozen)
    o.insert(); o.prefix_sum(); o.sort()
    zeros = np.zeros((n, 4), np.float32)
    for cyc in range(3):
        if cyc == 1:
            thawed = copy.copy(params)
            thawed.freeze = 0
            thawed.time = o.time()  # SetParam keeps m_Time
            o.update_params(thawed)
        for _ in range(2):
            for _ in range(2):
                o.pressure(); o.force(); o.advance()
            o.diffusion(); o.genes()
            o.bond_changes(2); o.remodel()
            o.insert(); o.prefix_sum(); o.sort()
            if cyc == 0:
                o.upload(A.FVEL, zeros); o.upload(A.FVEVAL, zeros)
    st = res["state"]
    for b in (A.FPOS, A.FVEL, A.FVEVAL, A.FCONC, A.FELASTIDX, A.FPARTICLEIDX, A.FEPIGEN, A.FPARTICLE_ID):
        x, y = st[b], o.download(b)
        if x.dtype == np.float32:
            x = np.where(np.isnan(x), np.float32(np.nan), x)
            y = np.where(np.isnan(y), np.float32(np.nan), y)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), f"buffer {b}"
    assert res["active_end"] == o.counts()[1]
    o.close()
