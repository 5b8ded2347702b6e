"""Precision form (DVM_PREC_FP32): FP32 sampling and scatter, FP64 conservation projection,
FP64 moments. Checked against the FP64 plain method on the same Philox stream: moments
within the specification's bar of 1e-3 relative (per moment field), and mass, momentum
and energy conserved by every collision step to FP64 round-off."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MOMENT_BAR = 1.0e-3


def _scales(p):
    n, T = np.abs(p[:, 0]).max(), np.abs(p[:, 4]).max()
    pr = 0.5 * n * T
    return np.array([n, np.sqrt(T), np.sqrt(T), np.sqrt(T), T, T, np.sqrt(T), pr] +
                    [n * T ** 1.5] * 3 + [pr] * 6)


def moment_errors(p32, p64):
    """Per moment field: max over cells of |FP32 - FP64| / the field's physical scale."""
    return np.abs(p32[:, :17] - p64[:, :17]).max(0) / _scales(p64)


def _pair(pkg, g, f0, steps, **kw):
    out = []
    for prec in (pkg.DVM_PREC_FP64, pkg.DVM_PREC_FP32):
        s = pkg.DVMSolver(pkg.DVMConfig(precision=prec, **kw), g)
        s.initialize_dist_func(f0)
        s.solve(steps)
        out.append((s.properties(), s.phi(), s.error_word()))
    return out


def test_relaxation_fp32_vs_fp64(gpulib, pkg):
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(24, -5.0, 5.0)
    (p64, f64, e64), (p32, f32, e32) = _pair(
        pkg, g, ph.bimodal(g), 20, iColl=pkg.DVM_COLL_VR, samples_mode=pkg.DVM_SAMPLES_FIXED,
        samples_per_step=100000, deltat=0.01, seed=3)
    err = moment_errors(p32, p64)
    assert err.max() <= MOMENT_BAR, dict(zip(pkg.PROP_NAMES, err))
    assert e32 == 0 and e64 == 0


def test_fp32_steps_conserve(gpulib, pkg):
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(24, -5.0, 5.0)
    s = pkg.DVMSolver(pkg.DVMConfig(precision=pkg.DVM_PREC_FP32, iColl=pkg.DVM_COLL_VR,
                                    samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=100000,
                                    deltat=0.01, seed=4), g)
    s.initialize_dist_func(ph.bimodal(g))
    p0 = s.properties()[0]
    for _ in range(10):
        s.solve(1)
        p1 = s.properties()[0]
        assert abs(p1[0] - p0[0]) <= 1e-12
        assert np.abs(p1[0] * p1[1:4] - p0[0] * p0[1:4]).max() <= 1e-12
        e0 = p0[0] * (1.5 * p0[4] + (p0[1:4] ** 2).sum())
        e1 = p1[0] * (1.5 * p1[4] + (p1[1:4] ** 2).sum())
        assert abs(e1 - e0) <= 1e-11 * e0
    assert s.error_word() == 0


def test_cavity_fp32_vs_fp64(gpulib, pkg):
    """2-D cavity with a moving lid: collisions, diffuse walls, several steps. The FP32 and
    FP64 runs share the Philox stream, but their f differ by FP32 rounding, so a few partner
    picks differ and the Monte Carlo realisations drift apart; the seed-to-seed spread of
    two FP64 runs is printed beside the FP32-vs-FP64 difference as the yardstick."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(12, -5.0, 5.0)
    nxs = nys = 6
    f0 = np.stack([ph.maxwellian(g, 1.0, 0.0, 0.0, 0.0, 1.0) for _ in range(nxs * nys)])
    walls = ((1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0.3, 0, 0, 1.0))
    kw = dict(geometry=pkg.DVM_GEOM_2D, nx_space=nxs, ny_space=nys, dx=0.5, dy=0.5,
              deltat=0.03, Kn=0.1, iColl=pkg.DVM_COLL_VR, iConv=pkg.DVM_CONV_UPWIND1,
              samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=100000, walls=walls)
    (p64, _, _), (p32, _, e32) = _pair(pkg, g, f0, 10, seed=8, **kw)
    (q64, _, _), _ = _pair(pkg, g, f0, 10, seed=9, **kw)
    err = moment_errors(p32, p64)
    noise = moment_errors(q64, p64)
    report = {n: "%.2e (seed spread %.2e)" % (e, z) for n, e, z in zip(pkg.PROP_NAMES, err, noise)}
    print(report)
    assert err.max() <= MOMENT_BAR, report
    assert e32 == 0


def test_fp32_pairlist_close_to_restatement(gpulib, pkg, oracle):
    """Same recorded list: the FP32 increment, once projected, differs from the FP64
    restatement only at FP32 rounding level."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(12, -5.0, 5.0)
    f0 = ph.bimodal(g)
    rng = np.random.default_rng(12)
    subs = [{"count": n, "num_repl": 1, "glA": rng.integers(0, g.nv, n).astype(np.int32),
             "glB": rng.integers(0, g.nv, n).astype(np.int32), "r_phi": rng.random(n),
             "r_cos": rng.random(n)} for n in (3000, 2000, 1000)]
    cfg32 = pkg.DVMConfig(iColl=pkg.DVM_COLL_VR, deltat=0.05, precision=pkg.DVM_PREC_FP32)
    cfg64 = pkg.DVMConfig(iColl=pkg.DVM_COLL_VR, deltat=0.05)
    gpu = pkg.DVMSolver(cfg32, g)
    cpu = oracle.OracleSolver(cfg64, g)
    gpu.initialize_dist_func(f0)
    cpu.initialize_dist_func(f0)
    gpu.compute_collision_integral(0, pkg.PairList(subs))
    cpu.compute_collision_integral(0, pkg.PairList(subs))
    d32, d64 = gpu.phi()[0] - f0, cpu.phi()[0] - f0
    assert np.abs(d32 - d64).max() <= 1e-4 * np.abs(d64).max()


def test_cavity_fp32_one_step_error(gpulib, pkg):
    """The precision form's own error on the cavity: one step of each form from the same
    state with the same Philox words differs only by FP32 rounding (far below the bar)."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(12, -5.0, 5.0)
    nxs = nys = 6
    f0 = np.stack([ph.maxwellian(g, 1.0, 0.1 * (c % 3), 0.0, 0.0, 1.0 + 0.05 * (c % 5))
                   for c in range(nxs * nys)])
    walls = ((1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0.3, 0, 0, 1.0))
    kw = dict(geometry=pkg.DVM_GEOM_2D, nx_space=nxs, ny_space=nys, dx=0.5, dy=0.5,
              deltat=0.03, Kn=0.1, iColl=pkg.DVM_COLL_VR, iConv=pkg.DVM_CONV_UPWIND1,
              samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=20000, walls=walls, seed=5)
    (p64, _, _), (p32, _, e32) = _pair(pkg, g, f0, 1, **kw)
    err = moment_errors(p32, p64)
    assert err.max() <= 1e-6, dict(zip(pkg.PROP_NAMES, err))
    assert e32 == 0


@pytest.mark.parametrize("n", [16, 40])
def test_fp32_one_step_error_grid_sizes(gpulib, pkg, n):
    """One step of the FP32 form on a small and a large grid (tables in shared memory and
    the g-table through L1): within FP32 rounding of the FP64 step, conservative."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(n, -5.0, 5.0)
    f0 = ph.bimodal(g)
    kw = dict(iColl=pkg.DVM_COLL_VR, samples_mode=pkg.DVM_SAMPLES_FIXED,
              samples_per_step=50000, deltat=0.02, seed=6)
    (p64, _, _), (p32, _, e32) = _pair(pkg, g, f0, 1, **kw)
    err = moment_errors(p32, p64)
    assert err.max() <= 1e-6, dict(zip(pkg.PROP_NAMES, err))
    assert abs(p32[0, 0] - p64[0, 0]) <= 1e-12 and e32 == 0


def test_fp32_scatter_count_matches_fp64(gpulib, pkg):
    """Both forms draw the same partners from the same Philox words, so the kernels' own
    counts of their adds agree (the FP32 stencil can differ only for a velocity within FP32
    rounding of a node midpoint)."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(16, -5.0, 5.0)
    counts = []
    for prec in (pkg.DVM_PREC_FP64, pkg.DVM_PREC_FP32):
        s = pkg.DVMSolver(pkg.DVMConfig(precision=prec, iColl=pkg.DVM_COLL_VR,
                                        samples_mode=pkg.DVM_SAMPLES_FIXED,
                                        samples_per_step=50000, deltat=0.01, seed=8), g)
        s.initialize_dist_func(ph.bimodal(g))
        s.solve(1)
        n = s.collision_count()
        counts.append(s.scatter_count())
        assert 2 * n < counts[-1] <= 16 * n
    assert abs(counts[0] - counts[1]) <= 1e-3 * counts[0]
