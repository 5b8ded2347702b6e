"""Where the reference's own rounding decides a Monte Carlo partner.

The reference forms the equilibrium value of node l as the difference of its FP64 running
sum, phi_eq = eq_df(l) - eq_df(l-1) (variance_reduction.f90:400), so each value carries the
running sum's rounding, up to half an ulp of the cell density (about 2e-16 n), and the
deviation f - phi_eq of a cell near equilibrium inherits it. In the benchmarked shock the
deviation is about 2e-3 of the density in every cell, so that rounding shifts the
boundaries of the deviation CDF by a measurable fraction of the CDF: about one partner
draw in 1e7 lands on the other side of a boundary than it would with the exact node
values. The GPU kernels form the node values from the Maxwellian directly (as exact
fixed-point terms), so they share the outcome of every draw with the reference except
those few.

These CPU tests pin that statement on the oracle alone: the restatement with the
reference's formation and the restatement with directly formed node values
(OracleSolver.set_eq_node_mode(True)) agree to 1e-12 in every cell but a handful, and in
those the difference is a few whole samples that conserve mass, momentum and energy. The
GPU tests then show the GPU equal to the direct formation to 1e-12 on the whole benchmark,
and equal to the reference's formation outside the same few events.
"""
import importlib.util
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
THREADS = max(1, min(16, os.cpu_count() or 1))


def bench_module():
    spec = importlib.util.spec_from_file_location("bench_cfg",
                                                  os.path.join(os.path.dirname(HERE), "bench.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def collision_step(oracle, cfg, g, f0, direct):
    s = oracle.OracleSolver(cfg, g, threads=THREADS)
    s.set_eq_node_mode(direct)
    s.initialize_dist_func(f0)
    s.compute_collision_integral(0)
    out = s.phi(), s.collision_count(), s.scatter_count()
    s.close()
    return out


def event_cells(a, b, tol=1e-12):
    """Cells whose largest difference exceeds tol of the cell's own max|f|."""
    err = np.abs(a - b).max(axis=1) / np.maximum(np.abs(b).max(axis=1), 1e-300)
    return np.nonzero(err > tol)[0], err


def check_sample_events(g, a, b, cells, max_cells, samples_per_event=32, max_events=3):
    """In each event cell the difference is confined to a few samples' nodes (two partner
    nodes and at most two seven-node stencils per sample, in either run) and conserves
    mass, momentum and energy as every sample does."""
    assert 1 <= len(cells) <= max_cells
    X, Y, Z, _ = g.mesh()
    weights = (np.ones_like(X), X, Y, Z, X * X + Y * Y + Z * Z)
    for c in cells:
        d = a[c] - b[c]
        scale = np.abs(b[c]).max()
        assert (np.abs(d) > 1e-12 * scale).sum() <= samples_per_event * max_events
        assert np.abs(d).max() <= 1e-5 * scale  # a few samples out of 2e5
        for w in weights:
            assert abs((d * w).sum()) <= 1e-5 * np.abs(d * w).sum() + \
                1e-12 * np.abs(b[c] * w).sum()


def test_running_sum_rounding_decides_a_few_partners(pkg, oracle):
    """Benchmark shock (200 cells x 32^3, 2e5 samples per cell-step), first collision step:
    the reference's formation of the equilibrium node values and the direct formation draw
    the same partners for all but a few samples, in a few near-equilibrium cells."""
    bench = bench_module()
    cfg, g, f0 = bench.workload_config(pkg)
    ref, n_ref, s_ref = collision_step(oracle, cfg, g, f0, direct=False)
    dirn, n_dir, s_dir = collision_step(oracle, cfg, g, f0, direct=True)
    assert n_ref == n_dir == 200 * 200000
    cells, err = event_cells(dirn, ref)
    check_sample_events(g, dirn, ref, cells, max_cells=12)
    rest = np.setdiff1d(np.arange(ref.shape[0]), cells)
    assert err[rest].max() <= 1e-12


def test_far_from_equilibrium_no_events(pkg, oracle):
    """With a deviation of the order of the density (a bimodal relaxation on 24^3, 1e5
    samples) the two formations agree everywhere within 1e-12: the running sum's rounding
    is far below the deviation CDF's resolution there."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(24, -5.0, 5.0)
    cfg = pkg.DVMConfig(iColl=pkg.DVM_COLL_VR, samples_mode=pkg.DVM_SAMPLES_FIXED,
                        samples_per_step=100000, deltat=0.01, seed=1)
    f0 = ph.bimodal(g)[None, :]
    ref, _, _ = collision_step(oracle, cfg, g, f0, direct=False)
    dirn, _, _ = collision_step(oracle, cfg, g, f0, direct=True)
    cells, _ = event_cells(dirn, ref)
    assert len(cells) == 0
