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
    deck = os.path.join(DECKS, "shock1d.inp")
    straight, part, resumed = tmp_path / "a.bin", tmp_path / "ck.bin", tmp_path / "b.bin"
    dat = tmp_path / "props.dat"
    r = subprocess.run([host, deck, "--steps", "3", "--dump-f", str(straight), "--props-dat",
                        str(dat)], capture_output=True, text=True, timeout=300)
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
    lines = dat.read_text().splitlines()
    assert lines[0].startswith("title") and lines[1].startswith("variables")
    assert sum(1 for l in lines if l.startswith("zone")) == 4  # times 0, 1, 2, 3
    assert len(lines) == 2 + 4 * 11
