"""Edge cases of the collision step against the CPU restatement (through the C ABI): the
smallest grid, extreme axis shapes, the largest replica count, no samples, negative node
values. The same bar as the parity tests: f within 1e-12 of max|f|, identical sample and
add counts, identical error words."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1.0e-12


def _pair(pkg, oracle, g, f0, steps, **kw):
    cfg = pkg.DVMConfig(**kw)
    gpu = pkg.DVMSolver(cfg, g)
    cpu = oracle.OracleSolver(cfg, g)
    gpu.initialize_dist_func(f0)
    cpu.initialize_dist_func(f0)
    for _ in range(steps):
        gpu.solve(1)
        cpu.solve(1)
        a, b = gpu.phi(), cpu.phi()
        assert np.abs(a - b).max() <= REL * max(np.abs(b).max(), 1e-300)
        assert gpu.collision_count() == cpu.collision_count()
        assert gpu.scatter_count() == cpu.scatter_count()
    assert gpu.error_word() == cpu.error_word()
    out = gpu.phi()
    gpu.close()
    return out


@pytest.mark.parametrize("method", ["VR", "FMC"])
def test_smallest_grid(gpulib, pkg, oracle, method):
    """3 x 3 x 3 nodes, the smallest grid accepted: most remap stencils reach the grid's edge
    (boundary stencils, and samples whose velocity has no exterior node, which both sides
    skip and flag the same way)."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(3, -2.0, 2.0)
    f0 = ph.bimodal(g, u1=0.5, u2=-0.5, T2=2.0)
    coll = pkg.DVM_COLL_VR if method == "VR" else pkg.DVM_COLL_FMC
    _pair(pkg, oracle, g, f0, 2, iColl=coll, samples_mode=pkg.DVM_SAMPLES_FIXED,
          samples_per_step=4000, deltat=0.02, seed=2)


def test_extreme_axis_shapes(gpulib, pkg, oracle):
    """3, 5 and 128 nodes on the three axes over different ranges (no velocity table; the
    longest axis allowed beside the shortest)."""
    ph = pkg.physics
    g = ph.VelocityGrid(np.linspace(-3.0, 3.0, 3), np.linspace(-4.0, 4.0, 5),
                        np.linspace(-5.0, 5.0, 128))
    f0 = ph.maxwellian(g, 1.0, 0.2, 0.0, -0.3, 1.2) + 0.3 * ph.maxwellian(g, 1.0, 0.0, 0.5, 0.8, 0.6)
    _pair(pkg, oracle, g, f0, 2, iColl=pkg.DVM_COLL_VR, samples_mode=pkg.DVM_SAMPLES_FIXED,
          samples_per_step=20000, deltat=0.02, seed=4)


def test_largest_replica_count(gpulib, pkg, oracle):
    """NRepl = 16, the most the library accepts: every sample replenishes sixteen times with
    its own angles (replenishing_collisions.f90:134-354)."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(10, -5.0, 5.0)
    _pair(pkg, oracle, g, ph.bimodal(g), 2, iColl=pkg.DVM_COLL_VR,
          samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=3000, NRepl=16, deltat=0.02,
          seed=6)


def test_no_samples_leaves_f(gpulib, pkg, oracle):
    """A step with no samples drawn changes nothing in a 0-D cell."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(8, -4.0, 4.0)
    f0 = ph.bimodal(g)
    f = _pair(pkg, oracle, g, f0, 2, iColl=pkg.DVM_COLL_VR, samples_mode=pkg.DVM_SAMPLES_FIXED,
              samples_per_step=0, deltat=0.02)
    assert np.array_equal(f[0], f0)


@pytest.mark.parametrize("method", ["VR", "FMC"])
def test_negative_node_values(gpulib, pkg, oracle, method):
    """A state with negative values at some nodes (as Monte Carlo noise leaves in the tails):
    the signs of the deviation (VR) and of f (FMC) enter the depletion factors the same way
    on both sides."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(12, -5.0, 5.0)
    rng = np.random.default_rng(8)
    f0 = ph.bimodal(g)
    idx = rng.choice(g.nv, g.nv // 20, replace=False)
    f0[idx] = -1e-3 * f0.max() * rng.random(len(idx))
    coll = pkg.DVM_COLL_VR if method == "VR" else pkg.DVM_COLL_FMC
    _pair(pkg, oracle, g, f0, 2, iColl=coll, samples_mode=pkg.DVM_SAMPLES_FIXED,
          samples_per_step=20000, deltat=0.02, seed=10)
