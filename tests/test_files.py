"""The reference's text formats (SimParams.txt, genome.csv, particle CSV): round trips, the
reference's line layouts, and the set-up ReadPointsCSV2 derives from SimParams.  Host code only,
no GPU needed."""
import numpy as np
import pytest

from morphogenesis_gb300 import _abi as A
from morphogenesis_gb300 import demo
from morphogenesis_gb300 import files as F


def simparams():
    sp = A.SimParams()
    vals = dict(time=0.5, dt=0.001, simscale=1.0, grid_density=1.0, visc=0.25, surface_tension=0.125,
                rest_density=600.0, spacing=0.0, mass=0.000205, radius=0.5, dist=0.0625, smooth_radius=2.0,
                intstiff=1.0, extstiff=10000.0, extdamp=256.0, accel_limit=100.0, vel_limit=50.0, grav=9.8125,
                ground_slope=0.0, force_min=0.0, force_max=0.0, force_freq=8.0, grid_size=4.0)
    for k, v in vals.items():
        setattr(sp, k, v)
    for k, v in (("plane_grav_dir", (0, -1, 0)), ("volmin", (0, 0, 0)), ("volmax", (64, 64, 64)),
                 ("initmin", (8, 8, 8)), ("initmax", (24, 24, 24))):
        getattr(sp, k)[:] = v
    return sp


def test_simparams_round_trip_and_layout(built, tmp_path):
    sp = simparams()
    F.write_simparams(tmp_path, sp)
    text = (tmp_path / "SimParams.txt").read_text()
    assert text.startswith(" m_Time = 0.500000\n m_DT = 0.001000\n m_Param [ PSIMSCALE ] = 1.000000\n")
    assert " m_Vec [ PPLANE_GRAV_DIR ].Set ( 0.000000, -1.000000, 0.000000 )\n // Default sim config\n" in text
    back = F.read_simparams(tmp_path / "SimParams.txt")
    for name, _ in A.SimParams._fields_:
        a, b = getattr(sp, name), getattr(back, name)
        if isinstance(a, float):
            assert b == pytest.approx(a, abs=5e-7), name
        else:
            assert list(b) == pytest.approx(list(a), abs=5e-7), name


def test_simparams_give_the_reference_setup(built):
    sp = simparams()
    p = F.fparams_from_simparams(sp, 3)
    # grid cell 2 * 2 / 1 = 4, SetupGrid over [0, 64]^3, bounds 2 cells in from the volume
    assert list(p.grid_res) == [16, 16, 16] and p.grid_total == 4096
    assert p.grid_srch == 3
    assert list(p.pboundmin) == [8.0, 8.0, 8.0] and list(p.pboundmax) == [56.0, 56.0, 56.0]
    assert list(p.pgravity) == pytest.approx([0.0, -9.8125, 0.0])
    assert p.prest_dens == 600.0 and p.psmoothradius == 2.0 and p.pmass == pytest.approx(0.000205)
    # with a spacing the rest density follows from it (SetupSpacing)
    sp.spacing = 1.0
    p2 = F.fparams_from_simparams(sp, 3)
    dist = np.float32(1.0) * np.float32(1.0) / np.float32(0.87)
    assert p2.prest_dens == pytest.approx(float(np.float32(0.000205) / dist ** 3), rel=1e-6)


def test_genome_round_trip(built, tmp_path):
    g = demo.make_genome(seed=3)
    F.write_genome(tmp_path, g)
    back = F.read_genome(tmp_path / "genome.csv")
    assert bytes(back) == bytes(g), "float genome does not survive a round trip"
    text = (tmp_path / "genome.csv").read_text()
    assert text.startswith("num genes = 16,\tnum transcription factors = 16 \nmutability, delay,\tsensitivity[NUM_GENES]")
    assert "\nTranscription Factors (tf_difusibility,tf_breakdown_rate) \n" in text
    # the reference's integer fields
    gi = A.Genome()
    for i in range(16):
        for j in range(16):
            gi.sensitivity[i][j] = float((i * 7 + j) % 5 - 2)
        gi.secrete[i][0], gi.secrete[i][1], gi.secrete[i][32] = float(i), 3.0, 1.0
        gi.tf_diffusability[i], gi.tf_breakdown_rate[i] = 1.0, 99.0
    F.write_genome(tmp_path, gi, integer_fields=True)
    text = (tmp_path / "genome.csv").read_text()
    row = text.splitlines()[2]
    assert row.startswith("0,\t0,\t\t-2,\t-1,\t0,\t1,\t2,\t-2,")
    assert bytes(F.read_genome(tmp_path / "genome.csv")) == bytes(gi)


def test_points_csv_round_trip(built, tmp_path):
    d = demo.make_block(4, "R", seed=1)
    arrays = {b: np.ascontiguousarray(v) for b, v in d.arrays.items()}
    for b in (A.FAGE, A.FCOLOR, A.FMASS_RADIUS, A.FNERVEIDX):
        arrays.setdefault(b, np.zeros(d.n, np.uint32))
        arrays[b] = np.arange(d.n, dtype=np.uint32) * (b + 1)
    F.write_points_csv(tmp_path, 1, arrays)
    path = tmp_path / "particles_pos_vel_color100001.csv"
    header = path.read_text().splitlines()[0]
    assert header.startswith("i,, x coord, y coord, z coord\t\t x vel, y vel, z vel\t\t age,  color\t\t FELASTIDX[6*9]")
    back = F.read_points_csv(path)
    for b in (A.FPOS, A.FVEL, A.FCONC):
        np.testing.assert_allclose(back[b], arrays[b], atol=6e-7, err_msg=f"buffer {b}")
    for b in (A.FPARTICLEIDX, A.FPARTICLE_ID, A.FEPIGEN, A.FAGE, A.FCOLOR, A.FNERVEIDX):
        assert np.array_equal(back[b], arrays[b]), f"buffer {b}"
    mr = arrays[A.FMASS_RADIUS]
    assert np.array_equal(back[A.FMASS_RADIUS], (mr & 0xFFFF) + ((mr >> 16) << 16))
    el, eb = arrays[A.FELASTIDX].reshape(-1, 6, 9), back[A.FELASTIDX].reshape(-1, 6, 9)
    for w in (0, 5, 8):
        assert np.array_equal(el[:, :, w], eb[:, :, w]), f"bond word {w}"
    for w in (1, 2, 3, 4, 6, 7):
        np.testing.assert_allclose(eb[:, :, w].view(np.float32), el[:, :, w].view(np.float32), atol=6e-7)


def test_points_csv_species_major_concentrations(built, tmp_path):
    """conc_species_major reads and writes FCONC as [16][n] (the reference host's getConc layout):
    the file is the same as from the [n][16] layout."""
    import ctypes as C
    d = demo.make_block(4, "R", seed=2)
    arrays = {b: np.ascontiguousarray(v) for b, v in d.arrays.items()}
    for b in (A.FAGE, A.FCOLOR, A.FMASS_RADIUS, A.FNERVEIDX):
        arrays[b] = np.arange(d.n, dtype=np.uint32)
    lib = A.load()
    (tmp_path / "pm").mkdir()
    (tmp_path / "sm").mkdir()
    pts = F._points(arrays, d.n)
    assert lib.mg_write_points_csv(str(tmp_path / "pm").encode(), 0, C.byref(pts)) == 0
    species_major = np.ascontiguousarray(arrays[A.FCONC].T)
    pts.conc = species_major.ctypes.data
    pts.conc_species_major = 1
    assert lib.mg_write_points_csv(str(tmp_path / "sm").encode(), 0, C.byref(pts)) == 0
    name = "particles_pos_vel_color100000.csv"
    assert (tmp_path / "pm" / name).read_text() == (tmp_path / "sm" / name).read_text()
    back = np.zeros_like(species_major)
    pts.conc = back.ctypes.data
    assert lib.mg_read_points_csv(str(tmp_path / "pm" / name).encode(), C.byref(pts)) == 0
    np.testing.assert_allclose(back, species_major, atol=6e-7)


def test_file_errors_are_returned(built, tmp_path):
    (tmp_path / "bad.txt").write_text("not a simparams file\n")
    with pytest.raises(A.MgError):
        F.read_simparams(tmp_path / "bad.txt")
    with pytest.raises(A.MgError):
        F.read_genome(tmp_path / "missing.csv")


def make_spec():
    s = A.Spec()
    s.num_particles, s.demo_type, s.sim_space = 4096, 1, 0
    for k, v in dict(time=0.0, dt=0.001, gridsize=64.0, spacing=1.0, simscale=1.0, smooth_radius=2.0, visc=0.1,
                     surface_tension=0.25, mass=0.0005, radius=0.5, intstiff=1.0, extstiff=10000.0,
                     extdamp=256.0, accel_limit=100.0, vel_limit=50.0, grav=9.8, ground_slope=0.0,
                     force_min=0.0, force_max=0.0, force_freq=8.0, actuation_factor=0.5,
                     actuation_period=400.0).items():
        setattr(s, k, v)
    for k, v in (("dim", (16, 16, 16)), ("pos", (8, 8, 8)), ("volmin", (0, 0, 0)), ("volmax", (64, 64, 64)),
                 ("initmin", (8, 8, 8)), ("initmax", (24, 24, 24))):
        getattr(s, k)[:] = v
    s.params_path, s.points_path = b"demo/SimParams.txt", b"demo/particles_pos_vel_color100001.csv"
    s.genome_path, s.out_path = b"demo/genome.csv", b"out"
    s.num_files, s.steps_per_inner_loop, s.steps_per_file, s.freeze_steps = 400, 3, 6, 1
    s.debug, s.file_num = 0, 0
    s.save_ply, s.save_csv, s.save_vtp = b"n", b"y", b"y"
    s.gene_activity, s.remodelling, s.read_genome = b"y", b"y", b"n"
    return s


def test_specification_round_trip_and_layout(built, tmp_path):
    s = make_spec()
    F.write_specification(tmp_path, s)
    text = (tmp_path / "SpecificationFile.txt").read_text()
    assert text.startswith("num_particles = 4096\n demoType = 1\n simSpace = 0\n \nm_Time = 0.000000\n m_DT = 0.001000\n")
    assert " \nvolmin_x = 0.000000\n volmin_y = 0.000000\n" in text
    assert "steps_per_InnerPhysicalLoop = 3\n" in text and "remodelling = y\n" in text
    back = F.read_specification(tmp_path)
    for name, _ in A.Spec._fields_:
        a, b = getattr(s, name), getattr(back, name)
        if isinstance(a, float):
            assert b == pytest.approx(a, abs=5e-7), name
        elif isinstance(a, (int, bytes)):
            assert a == b, name
        else:
            assert list(b) == pytest.approx(list(a), abs=5e-7), name


def test_results_csv(built, tmp_path):
    d = demo.make_block(4, "R", seed=1)
    el = d.arrays[A.FELASTIDX].reshape(-1, 6, 9).copy()
    rest = el.view(np.float32)[:, :, 2]
    bonds = int((rest > 0).sum())
    F.write_results_csv("in", tmp_path, make_spec(), d.n, d.n - 3, el)
    text = (tmp_path / "results.csv").read_text()
    # timesteps = (num_files / 100) * steps_per_InnerPhysicalLoop * steps_per_file = 4 * 3 * 6
    assert text == (f"input_folder=,in,\toutput_folder=,{tmp_path},\tfreeze_steps=,1,\ttimesteps=,72,\t"
                    f"num_particles_start=,{d.n},\tnum_particles_end=,{d.n - 3},\tnum_bonds_start=,65535,\t"
                    f"num_bonds_end=,{bonds},\t\n")


def test_points_vtp(built, tmp_path):
    import xml.etree.ElementTree as ET
    d = demo.make_block(4, "R", seed=3)
    n = d.n
    arrays = {b: np.ascontiguousarray(v) for b, v in d.arrays.items()}
    for b in (A.FAGE, A.FCOLOR, A.FMASS_RADIUS, A.FNERVEIDX):
        arrays[b] = np.arange(n, dtype=np.uint32)
    arrays[A.FFORCE] = np.ones((n, 4), np.float32)
    arrays[A.FPRESS] = np.full(n, 2.0, np.float32)
    arrays[A.FDENSITY] = np.full(n, 0.25, np.float32)
    el = arrays[A.FELASTIDX].reshape(n, 6, 9)
    el.view(np.float32)[0, 1, 2] = 0.0  # a broken bond is drawn to the particle itself
    p = d.params
    F.write_points_vtp(tmp_path, 3, arrays, p.pboundmin, p.pboundmax, active=n)
    root = ET.parse(tmp_path / "particles_pos_vel_color100003.vtp").getroot()
    piece = root.find("PolyData/Piece")
    assert int(piece.get("NumberOfPoints")) == n + 8 and int(piece.get("NumberOfLines")) == 6 * (n + 8)

    def arr(parent, name):
        for a in piece.find(parent):
            if a.get("Name") == name:
                return np.array(a.text.split(), np.float64)
        raise KeyError(name)

    pts = arr("Points", "Points").reshape(-1, 3)
    assert np.allclose(pts[:n], arrays[A.FPOS][:, :3]) and np.allclose(pts[n], list(p.pboundmin))
    assert np.allclose(pts[n + 7], list(p.pboundmax))
    conn = arr("Lines", "connectivity").astype(np.int64).reshape(-1, 6, 2)
    partners = el[:, :, 0].astype(np.int64)
    rest = el.view(np.float32)[:, :, 2]
    want = np.where((rest >= 1e-6) & (partners < n), partners, np.arange(n)[:, None])
    assert np.array_equal(conn[:n, :, 1], want) and conn[0, 1, 1] == 0
    assert np.array_equal(conn[n:, :, 0], conn[n:, :, 1])
    assert len(arr("CellData", "restlength")) == 6 * (n + 8)
    assert np.allclose(arr("CellData", "restlength")[: 6 * n], rest.ravel())
    dens = arr("PointData", "FDENSITY,(1/density,density)").reshape(-1, 2)
    assert np.allclose(dens[:n], [0.25, 4.0]) and np.allclose(dens[n:], 0)
    assert np.allclose(arr("PointData", "FCONC_5")[:n], arrays[A.FCONC][:, 5], atol=1e-6)
    tissue = arr("PointData", "F_TISSUE_TYPE")[:n]
    ep = arrays[A.FEPIGEN] > 0
    want_t = np.select([ep[9], ep[6], ep[7], ep[10], ep[8]], [9, 6, 7, 10, 8], 0)
    assert np.array_equal(tissue, want_t)
