"""dvm_step is the composition of the three calls of solve()'s loop
(dvm_compute_collision_integral, dvm_compute_convection, dvm_calculate_physical_properties:
solver/dvm_solver.f90:299-357): its f, properties and residual equal theirs on 2-D grids with
walls, Couette ends and open ends, and the moments come out of every CTA width the column
count picks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _config(pkg, bc, lid, coll):
    walls = ((1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.2), (1, 0, 0, 0, 0.9), (1, lid, 0, 0, 1.0))
    return pkg.DVMConfig(geometry=pkg.DVM_GEOM_2D, nx_space=6, ny_space=5, dx=0.2, dy=0.25,
                         deltat=0.01, Kn=0.3, iColl=coll, iConv=pkg.DVM_CONV_UPWIND1,
                         samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=4000, bc=bc,
                         walls=walls, seed=5)


def _start(pkg, g, ncells):
    ph = pkg.physics
    rng = np.random.default_rng(9)
    f0 = np.stack([ph.maxwellian(g, 1.0 + 0.1 * rng.random(), 0.2 * rng.random() - 0.1,
                                 0.1 * rng.random(), 0.0, 1.0 + 0.2 * rng.random())
                   for _ in range(ncells)])
    return f0


def _bc(pkg, kind):
    W, C, I = pkg.DVM_BC2D_WALL, pkg.DVM_BC2D_COUETTE, pkg.DVM_BC2D_INOUT
    if kind == "cavity":
        return (W, W, W, W)
    if kind == "couette":
        return (C, C, W, W)
    return (I, I, W, W)


@pytest.mark.parametrize("kind", ["cavity", "couette", "open"])
def test_step_bitwise_without_collisions(gpulib, pkg, kind):
    g = pkg.physics.VelocityGrid.uniform(10, -5.0, 5.0)
    cfg = _config(pkg, _bc(pkg, kind), 0.4, pkg.DVM_COLL_NONE)
    f0 = _start(pkg, g, cfg.nx_space * cfg.ny_space)
    a, b = pkg.DVMSolver(cfg, g), pkg.DVMSolver(cfg, g)
    a.initialize_dist_func(f0)
    b.initialize_dist_func(f0)
    for _ in range(3):
        a.solve(1)
        b.compute_collision_integral()
        b.compute_convection()
        b.calculate_physical_properties()
        b.ntime += 1
        assert np.array_equal(a.phi(), b.phi())
        assert np.array_equal(a.properties(), b.properties())
        assert a.residual() == b.residual()
    assert a.error_word() == 0 and b.error_word() == 0


def test_step_with_collisions(gpulib, pkg):
    """With collisions the FP64 atomic order differs between two contexts, so the two
    paths agree to the rounding of a sum rather than bit for bit."""
    g = pkg.physics.VelocityGrid.uniform(10, -5.0, 5.0)
    cfg = _config(pkg, _bc(pkg, "cavity"), 0.4, pkg.DVM_COLL_VR)
    f0 = _start(pkg, g, cfg.nx_space * cfg.ny_space)
    a, b = pkg.DVMSolver(cfg, g), pkg.DVMSolver(cfg, g)
    a.initialize_dist_func(f0)
    b.initialize_dist_func(f0)
    for _ in range(3):
        a.solve(1)
        b.compute_collision_integral()
        b.compute_convection()
        b.calculate_physical_properties()
        b.ntime += 1
    fa, fb = a.phi(), b.phi()
    assert np.abs(fa - fb).max() <= 1e-13 * np.abs(fa).max()
    assert np.abs(a.properties()[:, :17] - b.properties()[:, :17]).max() <= 1e-12


@pytest.mark.parametrize("pinned", [True, False])
def test_step_host_equals_upload_step_download(gpulib, pkg, pinned):
    """dvm_step_host (host f in, steps, host f out in one call) gives what dvm_upload_f,
    dvm_step and dvm_download_f give: with page-locked buffers the device reads and writes
    them in its moments passes, with pageable ones through copies. Same Philox steps, so the
    results agree to the FP64 atomics' ordering (1e-12), moments included, and the buffer
    may be both input and output."""
    import torch

    ph = pkg.physics
    g = ph.VelocityGrid.uniform(14, -6.0, 6.0)
    f0, up, dn = ph.shock_profile(g, 12, 0.5, 2.0, 2.0)
    walls = ((dn["n"], dn["u"], 0.0, 0.0, dn["T"]), (up["n"], up["u"], 0.0, 0.0, up["T"]),
             (1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0))
    cfg = pkg.DVMConfig(geometry=pkg.DVM_GEOM_1D, nx_space=12, dx=0.5, deltat=0.05,
                        iColl=pkg.DVM_COLL_VR, iConv=pkg.DVM_CONV_UPWIND1,
                        samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=5000,
                        bc=(pkg.DVM_BC1D_INOUT, pkg.DVM_BC1D_INOUT, 0, 0), walls=walls, seed=3)
    ref = pkg.DVMSolver(cfg, g)
    ref.initialize_dist_func(f0)
    ref.solve(3)
    fr, pr = ref.phi(), ref.properties()
    ref.close()
    if pinned:
        buf = torch.empty(f0.shape, dtype=torch.float64, pin_memory=True).numpy()
    else:
        buf = np.empty_like(f0)
    buf[:] = f0
    s = pkg.DVMSolver(cfg, g)
    s.step_host(buf, 3, f_out=buf)
    ps = s.properties()
    assert s.error_word() == 0
    s.close()
    assert np.abs(buf - fr).max() <= 1e-12 * np.abs(fr).max()
    assert np.abs(ps[:, :17] - pr[:, :17]).max() <= 1e-11 * max(1.0, np.abs(pr).max())
