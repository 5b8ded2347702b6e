"""Checkpoint and restart (the reference's restart files, input_output/restart.f90:93-250):
a context restored from a checkpoint continues the run as the saved one does, including a
cached equilibrium that the next steps reuse; a checkpoint of another shape is refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cavity(pkg):
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(12, -5.0, 5.0)
    walls = ((1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0.3, 0, 0, 1.0))
    cfg = pkg.DVMConfig(geometry=pkg.DVM_GEOM_2D, nx_space=5, ny_space=4, dx=0.2, dy=0.25,
                        deltat=0.01, Kn=0.3, iColl=pkg.DVM_COLL_VR, iConv=pkg.DVM_CONV_UPWIND1,
                        samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=5000, walls=walls,
                        seed=21)
    f0 = np.tile(ph.maxwellian(g, 1.0, 0.0, 0.0, 0.0, 1.0), (20, 1))
    return cfg, g, f0


def _drifting_relaxation(pkg):
    """0-D, drift +0.5: the moments are conserved, so the equilibrium cache hits every step
    after the first and the cached equilibrium CDF is reused."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(14, -5.0, 6.0)
    cfg = pkg.DVMConfig(iColl=pkg.DVM_COLL_VR, samples_mode=pkg.DVM_SAMPLES_FIXED,
                        samples_per_step=30000, deltat=0.05, seed=4)
    f0 = ph.bimodal(g, u1=1.5, u2=-0.5)[None, :]
    return cfg, g, f0


@pytest.mark.parametrize("case", ["cavity", "relaxation"])
def test_restart_continues_exactly(gpulib, pkg, case):
    cfg, g, f0 = (_cavity if case == "cavity" else _drifting_relaxation)(pkg)
    a = pkg.DVMSolver(cfg, g)
    a.initialize_dist_func(f0)
    a.solve(3)
    ck = a.checkpoint()
    a.solve(4)
    b = pkg.DVMSolver(cfg, g)
    b.initialize_dist_func(np.zeros_like(f0))
    b.restore(ck)
    assert b.ntime == 3
    b.solve(4)
    fa, fb = a.phi(), b.phi()
    assert np.abs(fa - fb).max() <= 1e-13 * np.abs(fa).max()
    assert np.abs(a.properties()[:, :17] - b.properties()[:, :17]).max() <= 1e-12
    assert a.error_word() == 0 and b.error_word() == 0


def test_restart_refuses_other_shapes(gpulib, pkg):
    cfg, g, f0 = _drifting_relaxation(pkg)
    a = pkg.DVMSolver(cfg, g)
    a.initialize_dist_func(f0)
    ck = a.checkpoint()
    other = pkg.DVMSolver(cfg, pkg.physics.VelocityGrid.uniform(12, -5.0, 6.0))
    with pytest.raises(pkg.DVMError):
        other.restore(ck)
    with pytest.raises(pkg.DVMError):
        a.restore(b"not a checkpoint" * 100)


def test_bounded_wait_reports_and_context_survives(gpulib, pkg):
    """Failure detection without a fault: a device wait on a barrier that nothing completes
    gives up after its bound and sets DVM_EW_WAIT; the context then steps normally."""
    cfg, g, f0 = _drifting_relaxation(pkg)
    s = pkg.DVMSolver(cfg, g)
    s.initialize_dist_func(f0)
    assert s.error_word() == 0
    _ok = s.lib.dvm_wait_selftest(s.ctx)
    assert _ok == 0
    assert s.error_word() == pkg.DVM_EW_WAIT
    s.solve(2)
    assert s.error_word() == 0
    assert np.isfinite(s.properties()[:, :17]).all()
