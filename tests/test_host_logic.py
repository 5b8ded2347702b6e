"""Host-side set-up (grids, constants, initial states, shock end states) and the CPU
restatement's physical invariants. Runs without a GPU."""
import math

import numpy as np
import pytest


def test_uniform_axis_and_node_volumes(pkg):
    ph = pkg.physics
    x = ph.uniform_axis(24, -5.0, 5.0)
    assert x[0] == -5.0 and abs(x[-1] - 5.0) < 1e-15
    b = ph.node_volumes(x)
    h = 10.0 / 23.0
    assert abs(b[0] - h) < 1e-14 and abs(b[-1] - h) < 1e-14  # full spacing at the ends
    assert np.allclose(b[1:-1], h, rtol=1e-13)


def test_gamma_and_cross_section(pkg):
    ph = pkg.physics
    assert abs(ph.gamma_reference(2.0, pi_mode=1) - 1.0) < 1e-13
    assert abs(ph.gamma_reference(0.5, pi_mode=1) - math.sqrt(math.pi)) < 1e-12
    # the reference pi shifts Gamma(2) away from 1
    assert abs(ph.gamma_reference(2.0, pi_mode=0) - 1.0) > 1e-4
    hs = ph.molecule("Ar", ph.CSECTION_HS)
    assert hs["omega"] == 0.5 and hs["alpha"] == 1.0 and hs["mass"] == 1.0
    assert ph.cross_section(hs, ph.CSECTION_CLARKE) == 1.0
    vhs = ph.molecule("Ar", ph.CSECTION_VHS)
    assert vhs["omega"] == 0.81 and vhs["alpha"] == 1.0


def test_maxwellian_and_bimodal_moments(pkg):
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(24, -5.0, 5.0)
    X, Y, Z, B3 = g.mesh()
    f = ph.maxwellian(g, 2.0, 0.3, 0.0, 0.0, 1.5, pi_mode=1)
    n = f.sum()
    u = (f * X).sum() / n
    T = 2.0 * ((X - u) ** 2 + Y ** 2 + Z ** 2) @ f / (3.0 * n)
    assert abs(n - 2.0) < 1e-13 and abs(u - 0.3) < 1e-6 and abs(T - 1.5) < 1e-3
    fb = ph.bimodal(g)
    assert abs(fb.sum() - 1.0) < 1e-13


@pytest.mark.parametrize("mach", [1.5, 3.0])
def test_rankine_hugoniot(pkg, mach):
    ph = pkg.physics
    up, dn = ph.normal_shock(mach)
    g = 5.0 / 3.0
    # mass, momentum and energy fluxes agree across the jump (nondimensional: p = n T / 2)
    m1, m2 = up["n"] * up["u"], dn["n"] * dn["u"]
    p1, p2 = 0.5 * up["n"] * up["T"], 0.5 * dn["n"] * dn["T"]
    assert abs(m1 - m2) < 1e-12 * abs(m1)
    assert abs((m1 * up["u"] + p1) - (m2 * dn["u"] + p2)) < 1e-12
    h1 = g / (g - 1) * p1 / up["n"] + 0.5 * up["u"] ** 2
    h2 = g / (g - 1) * p2 / dn["n"] + 0.5 * dn["u"] ** 2
    assert abs(h1 - h2) < 1e-12
    assert up["u"] < 0 and dn["n"] > up["n"]


def test_shock_profile_ends(pkg):
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(12, -8.0, 8.0)
    f, up, dn = ph.shock_profile(g, 40, 1.0, 2.0, 3.0)
    assert f.shape == (40, g.nv)
    assert abs(f[0].sum() - dn["n"]) < 1e-4 and abs(f[-1].sum() - up["n"]) < 1e-4


def _solver(pkg, oracle, g, **kw):
    cfg = pkg.DVMConfig(**kw)
    return oracle.OracleSolver(cfg, g)


@pytest.mark.parametrize("method", ["VR", "FMC"])
def test_oracle_collisions_conserve(pkg, oracle, method):
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(10, -5.0, 5.0)
    coll = pkg.DVM_COLL_VR if method == "VR" else pkg.DVM_COLL_FMC
    s = _solver(pkg, oracle, g, iColl=coll, samples_mode=pkg.DVM_SAMPLES_FIXED,
                samples_per_step=5000, seed=4)
    s.initialize_dist_func(ph.bimodal(g))
    p0 = s.properties()[0]
    s.solve(3)
    p1 = s.properties()[0]
    assert abs(p1[0] - p0[0]) < 1e-12
    assert np.allclose(p1[1:4], p0[1:4], atol=1e-12)
    assert abs(p1[4] - p0[4]) < 1e-11
    assert s.error_word() == 0
    assert s.collision_count() == 5000


def test_oracle_vr_near_equilibrium(pkg, oracle):
    """Variance reduction samples only the deviation from the cell's Maxwellian: on a
    discrete Maxwellian the update is far smaller than on the bimodal state."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(16, -6.0, 6.0)
    changes = []
    for f0 in (ph.maxwellian(g, 1.0, 0.2, 0.0, 0.0, 1.3), ph.bimodal(g)):
        s = _solver(pkg, oracle, g, iColl=pkg.DVM_COLL_VR, samples_mode=pkg.DVM_SAMPLES_FIXED,
                    samples_per_step=4000, seed=2)
        s.initialize_dist_func(f0)
        s.compute_collision_integral(step=0)
        changes.append(np.abs(s.phi()[0] - f0).sum())
        ce, cd, kin, _, _ = s.cell_cdf_vr(0)
        assert abs(ce[-1] - 1.0) < 1e-2  # n_eq ~ n
    assert changes[0] < 0.05 * changes[1]


def test_oracle_cavity_conserves_mass_with_diffuse_walls(pkg, oracle):
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(8, -4.0, 4.0)
    nxs, nys = 6, 5
    f0 = np.stack([ph.maxwellian(g, 1.0 + 0.03 * c, 0.0, 0.0, 0.0, 1.0) for c in range(nxs * nys)])
    walls = ((1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0.3, 0, 0, 1.0))
    s = _solver(pkg, oracle, g, geometry=pkg.DVM_GEOM_2D, nx_space=nxs, ny_space=nys, dx=0.5,
                dy=0.5, deltat=0.05, iColl=pkg.DVM_COLL_NONE, iConv=pkg.DVM_CONV_UPWIND1,
                acc_coeff=1.0, walls=walls)
    s.initialize_dist_func(f0)
    m0 = f0.sum()
    for _ in range(4):
        s.compute_convection()
    assert abs(s.phi().sum() - m0) < 1e-12 * m0


def test_pair_constants_in_the_kernels():
    """The hi + lo float pairs written as hex literals in the device code are the pair
    splits of the constants they stand for: hi the float nearest the value, |lo| at most
    half an ulp of hi, hi + lo within 2^-48 of the value."""
    import math
    import os
    import re
    from fractions import Fraction

    import numpy as np

    root = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..",
                        "2d_dvm_microflows_gb300", "csrc")
    src = open(os.path.join(root, "dfloat.cuh")).read() + open(
        os.path.join(root, "dvm_kernels.cu")).read()
    pair = re.compile(r"dfl_make\((-?0x[0-9a-f.]+p[-+]?\d+)f, (-?0x[0-9a-f.]+p[-+]?\d+)f\)")
    found = {}
    for name, value in (("c3 ", 1 / 3), ("c5 ", 1 / 5), ("c7 ", 1 / 7), ("inv_ln2", 1 / math.log(2)),
                        ("u ln 2", math.log(2)), ("v^3/6", 1 / 6), ("one_sixth", 1 / 6)):
        line = next(ln for ln in src.splitlines() if name in ln and "dfl_make(0x" in ln)
        hi_s, lo_s = pair.search(line).groups()
        hi, lo = float.fromhex(hi_s), float.fromhex(lo_s)
        found[name] = (hi, lo)
        assert np.float32(hi) == hi and np.float32(lo) == lo  # both are floats
        assert float(np.float32(value)) == hi  # hi rounds the value to nearest
        assert abs(lo) <= float(np.spacing(np.float32(abs(hi)))) / 2
        assert abs(Fraction(hi) + Fraction(lo) - Fraction(value)) <= Fraction(value) * Fraction(1, 2 ** 48)
    assert len(found) == 7
