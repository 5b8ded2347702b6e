"""The C++ host (2d_dvm_microflows_gb300/host/dvm_host.cpp): it reads the reference's deck
format and drives the C ABI the way solve() drives the reference kernels."""
import importlib
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
DECKS = os.path.join(HERE, "decks")


@pytest.fixture(scope="module")
def host(pkg):
    exe = os.path.join(os.path.dirname(pkg.LIB_PATH), "dvm_host")
    if not os.path.exists(exe):
        importlib.import_module("2d_dvm_microflows_gb300.build").build()
    return exe


def _check(exe, deck):
    r = subprocess.run([exe, deck, "--check"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    tok = r.stdout.split()
    return {tok[i]: tok[i + 1] for i in range(0, len(tok) - 1, 2)}


def test_deck_reading(host, pkg):
    ph = pkg.physics
    d = _check(host, os.path.join(DECKS, "relax0d.inp"))
    assert d["geometry"] == "0" and d["cells"] == "1" and d["nv"] == str(12 ** 3)
    assert d["coll"] == "3" and d["samples_mode"] == "1" and d["samples"] == "20000"
    mol = ph.molecule("Ar", ph.CSECTION_HS)
    assert float(d["sigma"]) == pytest.approx(ph.cross_section(mol, ph.CSECTION_BIRD), rel=1e-15)
    assert abs(float(d["mass"]) - 1.0) < 1e-13
    d = _check(host, os.path.join(DECKS, "shock1d.inp"))
    assert d["geometry"] == "1" and d["cells"] == "10" and d["conv"] == "1"
    assert float(d["omega"]) == 0.81


def test_bad_deck_reports_error(host, tmp_path):
    p = tmp_path / "bad.inp"
    p.write_text("species_codes = 'Kr'\n")
    r = subprocess.run([host, str(p), "--check"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "unsupported species" in r.stderr


REF_TRUNK = "/root/reference/software/trunk"


def _run(exe, deck, *args):
    return subprocess.run([exe, str(deck)] + list(args), capture_output=True, text=True,
                          timeout=120)


@pytest.mark.skipif(not os.path.isdir(REF_TRUNK), reason="the reference's decks are not here")
def test_reference_shipped_decks(host):
    """The decks the reference ships: the 2-D input of its bin/ directory, and the two
    decks of its test suite, written for the earlier reader (nspace, per-zone entries).
    Those two take the right wall's state under InitC = 2, whose density is 0, so the
    reference starts them from an empty gas (initial_conditions.f90:456-469) and so does
    this host, with a warning."""
    d = _check(host, os.path.join(REF_TRUNK, "bin", "velocity_refined.inp"))
    assert d["geometry"] == "2" and d["cells"] == "100" and d["conv"] == "1"
    assert abs(float(d["mass"]) - 100.0) < 1e-9
    for name in ("maxwell_relax.inp", "bkw_relax.inp"):
        path = os.path.join(REF_TRUNK, "test", "input_files", name)
        r = _run(host, path, "--check")
        assert r.returncode == 0, r.stderr
        tok = r.stdout.split()
        d = {tok[i]: tok[i + 1] for i in range(0, len(tok) - 1, 2)}
        assert d["nv"] == str(11 ** 3) and d["cells"] == "1" and d["omega"] == "1"
        assert float(d["mass"]) == 0.0 and "empty" in r.stderr


def _deck(tmp_path, name, body):
    p = tmp_path / name
    p.write_text(body)
    return p


BASE = """[species]
species_codes = 'Ar'
[csection_model]
csection_method = 2
csection_coeff = 1
[time_stepping]
deltat = 0.05d0
ntstep = 4
[vel_grid]
num_points_x = '9 11'
num_points_y = '9 11'
num_points_z = '9 11'
xv_min = '-4.0d0 -3.5d0'
xv_max = '4.0d0 3.5d0'
yv_min = '-4.0d0'
yv_max = '4.0d0'
zv_min = '-4.0d0'
zv_max = '4.0d0'
[collision]
iColl = 3
samples_per_step = 5000
"""


def test_legacy_keys_and_refusals(host, tmp_path):
    # the earlier reader's nspace; several entries per key: the first (species / zone 1)
    d = _check(host, _deck(tmp_path, "a.inp", BASE + "[phy_grid]\nnspace = '3'\n"
                           "num_zones = '1'\n[boundary]\nInitC = '5'\n"))
    assert d["cells"] == "3" and d["nv"] == str(9 ** 3)
    r = _run(host, _deck(tmp_path, "b.inp", BASE + "[phy_grid]\nnum_zones = 2\n"), "--check")
    assert r.returncode == 1 and "num_zones" in r.stderr
    # a state that cannot be formed: positive density at zero temperature
    r = _run(host, _deck(tmp_path, "c.inp", BASE + "[boundary]\nInitC = 5\n"
                         "dens_init = 1.0d0\ntr_temp_init = 0.0d0\n"), "--check")
    assert r.returncode == 1 and "not finite" in r.stderr
    r = _run(host, _deck(tmp_path, "d.inp", BASE + "[boundary]\nInitC = 4\n"), "--check")
    assert r.returncode == 1 and "InitC 4" in r.stderr


@pytest.mark.parametrize("initdf", [1, 2, 3, 4])
def test_initial_distributions(host, pkg, tmp_path, initdf):
    """InitDF 1-4 of initialize_dist_func, each scaled to the density: the Maxwellian and
    the BKW state equal the package's (physics.maxwellian, physics.bkw at t = 0); the delta
    function sits on one node; the exactly integrated Gaussian is close to the Maxwellian."""
    ph = pkg.physics
    deck = _deck(tmp_path, "s.inp", BASE + "[boundary]\nInitC = 5\nInitDF = %d\n"
                 "dens_init = 1.3d0\nx_vel_init = 0.4d0\ntr_temp_init = 1.2d0\n"
                 "x_delta_loc = 1.0d0\ny_delta_loc = 0.0d0\nz_delta_loc = -2.0d0\n" % initdf)
    out = tmp_path / "f0.bin"
    r = _run(host, deck, "--check", "--dump-f", str(out))
    assert r.returncode == 0, r.stderr
    f = np.fromfile(str(out), dtype=np.float64)
    g = ph.VelocityGrid.uniform(9, -4.0, 4.0)
    assert abs(f.sum() - 1.3) < 1e-14
    if initdf == 1:
        m = ph.maxwellian(g, 1.3, 0.4, 0.0, 0.0, 1.2)
        assert np.abs(f - m).max() <= 1e-14 * m.max()
    elif initdf == 4:
        # compute_exact_gaussian (dist_func.f90:345-372): the Maxwellian integrated between
        # the midpoints to each neighbour (beyond the ends, half a node volume out)
        import math
        a, b = g.x, g.bx
        lo = np.concatenate(([a[0] - b[0]], a[:-1]))
        hi = np.concatenate((a[1:], [a[-1] + b[-1]]))
        sq = math.sqrt(1.0 / 1.2)
        erf = np.vectorize(math.erf)
        vel = (0.4, 0.0, 0.0)
        C = [erf(sq * (a + 0.5 * (hi - a) - u)) - erf(sq * (lo + 0.5 * (a - lo) - u)) for u in vel]
        X, Y, Z, B3 = g.mesh()
        n = len(a)
        Cx = np.tile(C[0], n * n)
        Cy = np.tile(np.repeat(C[1], n), n)
        Cz = np.repeat(C[2], n * n)
        ref = Cx * Cy * Cz * B3
        ref = 1.3 * ref / ref.sum()
        assert np.abs(f - ref).max() <= 1e-13 * ref.max()
        m = ph.maxwellian(g, 1.3, 0.4, 0.0, 0.0, 1.2)
        assert np.abs(f - m).max() <= 0.25 * m.max()  # the same gas, integrated over cells
    elif initdf == 2:
        b = ph.bkw(g, 1.3, 1.2, 0.0, u=0.4)
        assert np.abs(f - b).max() <= 1e-14 * np.abs(b).max()
        assert f.min() < 0.0 or np.isclose(f.min(), 0.0)  # K = 3/5: a hole at the drift
    else:
        X, Y, Z, _ = g.mesh()
        hit = (X == 1.0) & (Y == 0.0) & (Z == -2.0)
        assert hit.sum() == 1 and f[hit][0] == pytest.approx(1.3) and f[~hit].max() == 0.0


def _python_solver(pkg, deck):
    ph = pkg.physics
    if deck == "relax0d.inp":
        g = ph.VelocityGrid.uniform(12, -5.0, 5.0)
        mol = ph.molecule("Ar", ph.CSECTION_HS)
        cfg = pkg.DVMConfig(deltat=0.02, Kn=1.0, mass=1.0, omega=mol["omega"], alpha=mol["alpha"],
                            sigma=ph.cross_section(mol, ph.CSECTION_BIRD), iColl=pkg.DVM_COLL_VR,
                            samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=20000, seed=5,
                            ColnRMS=0.001, cdf_tolerance=0.01)
        return cfg, g, ph.bimodal(g)[None, :], 3
    g = ph.VelocityGrid.uniform(10, -7.0, 7.0)
    mol = ph.molecule("Ar", ph.CSECTION_VHS)
    f0, up, dn = ph.shock_profile(g, 10, 0.5, 2.0, 1.5)
    walls = ((dn["n"], dn["u"], 0, 0, dn["T"]), (up["n"], up["u"], 0, 0, up["T"]),
             (1, 0, 0, 0, 1), (1, 0, 0, 0, 1))
    cfg = pkg.DVMConfig(geometry=pkg.DVM_GEOM_1D, nx_space=10, dx=0.5, deltat=0.03, Kn=1.0,
                        omega=mol["omega"], alpha=mol["alpha"],
                        sigma=ph.cross_section(mol, ph.CSECTION_BIRD), iColl=pkg.DVM_COLL_VR,
                        iConv=pkg.DVM_CONV_UPWIND1, samples_mode=pkg.DVM_SAMPLES_FIXED,
                        samples_per_step=3000, seed=9, walls=walls,
                        bc=(pkg.DVM_BC1D_INOUT, pkg.DVM_BC1D_INOUT, 1, 1))
    return cfg, g, f0, 2


@pytest.mark.gpu
@pytest.mark.parametrize("deck", ["relax0d.inp", "shock1d.inp"])
def test_host_matches_python_host(gpulib, host, pkg, tmp_path, deck):
    out = tmp_path / "f.bin"
    r = subprocess.run([host, os.path.join(DECKS, deck), "--dump-f", str(out)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    f_host = np.fromfile(str(out), dtype=np.float64)
    cfg, g, f0, steps = _python_solver(pkg, deck)
    s = pkg.DVMSolver(cfg, g)
    s.initialize_dist_func(f0)
    s.solve(steps)
    f_py = s.phi().ravel()
    assert np.abs(f_host - f_py).max() <= 1e-12 * np.abs(f_py).max()


@pytest.mark.gpu
def test_host_restart_continues_the_run(gpulib, host, tmp_path):
    """restart.f90's role: a run stopped after 1 step and restarted for 2 ends where the
    straight 3-step run ends; the Tecplot file has one zone per output time."""
    base = open(os.path.join(DECKS, "shock1d.inp")).read()
    dat = tmp_path / "props"
    vis_deck = tmp_path / "shock_vis.inp"
    vis_deck.write_text(base.replace("ntstep = 2", "ntstep = 3") +
                        "\n[vis]\nenable_properties_vis = 1\nproperties_vis_filename = %s\n"
                        "properties_vis_dump_freq = 1\nwrite_dens = 1\nwrite_x_vel = 1\n"
                        "write_tr_temp = 1\n" % dat)
    deck = os.path.join(DECKS, "shock1d.inp")
    straight, part, resumed = tmp_path / "a.bin", tmp_path / "ck.bin", tmp_path / "b.bin"
    r = subprocess.run([host, str(vis_deck), "--steps", "3", "--dump-f", str(straight)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([host, deck, "--steps", "1", "--restart-out", str(part)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([host, deck, "--steps", "2", "--restart-in", str(part), "--dump-f",
                        str(resumed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    a = np.fromfile(str(straight), dtype=np.float64)
    b = np.fromfile(str(resumed), dtype=np.float64)
    assert np.abs(a - b).max() <= 1e-13 * np.abs(a).max()
    lines = open(str(dat) + ".dat").read().splitlines()
    assert lines[0].startswith("title") and lines[1].startswith("variables")
    assert sum(1 for l in lines if l.startswith("zone")) == 4  # times 0, 1, 2, 3
    assert len(lines) == 2 + 4 * 11


@pytest.mark.gpu
def test_host_output_equals_package_output(gpulib, host, pkg, tmp_path):
    """The C++ host's Tecplot files from a deck equal, byte for byte, what the package's
    TecplotOutput writes from the same run (convection and moments only, which are
    deterministic): both go through dvm_vis_* with f downloaded at each output time."""
    base = open(os.path.join(DECKS, "shock1d.inp")).read().replace("iColl = 3", "iColl = 0")
    out = tmp_path / "h"
    keys = ("write_dens", "write_x_vel", "write_tr_temp", "write_temp_x", "write_entropy",
            "write_heat_flux_x", "write_pressure")
    deck = tmp_path / "v.inp"
    deck.write_text(base + "\n[vis]\nenable_properties_vis = 1\nproperties_vis_filename = %s\n"
                    "properties_vis_dump_freq = 1\nwrite_stress = 2\nstress_directions = '11 12'\n"
                    % out + "".join("%s = 1\n" % k for k in keys))
    r = subprocess.run([host, str(deck)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    f0_host = tmp_path / "f0.bin"
    r = subprocess.run([host, str(deck), "--check", "--dump-f", str(f0_host)],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    cfg, g, _, steps = _python_solver(pkg, "shock1d.inp")
    f0 = np.fromfile(str(f0_host), dtype=np.float64).reshape(cfg.nx_space, g.nv)
    cfg.iColl = pkg.DVM_COLL_NONE
    s = pkg.DVMSolver(cfg, g)
    s.initialize_dist_func(f0)
    py = str(tmp_path / "p")
    vis = pkg.TecplotOutput(cfg.nx_space, 1, cfg.dx, cfg.dy, mass=cfg.mass, omega=cfg.omega,
                            end_time=steps, properties_filename=py, properties=keys,
                            stress=(11, 12), right_wall_dens=cfg.walls[1][0])
    vis.write_headers()
    vis.write_properties(0.0, f=s.phi(), grid=g)
    for n in range(1, steps + 1):
        s.solve(1)
        vis.write_properties(n * cfg.deltat, f=s.phi(), grid=g)
    for suffix in (".dat", "_1.dat"):
        assert open(str(out) + suffix).read() == open(py + suffix).read()
