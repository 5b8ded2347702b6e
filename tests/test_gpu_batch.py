"""Batched homogeneous relaxations (dvm_batch_*): instances on several velocity grids, one
CUDA-graph replay per step, autotuned persistent launches. Each instance must evolve exactly
as it does in a plain multi-cell 0-D context holding its grid's instances (same kernels, same
Philox counters), the autotuner must leave the state untouched, and the FP32 form must stay
within 1e-3 of FP64 per moment field."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instances(ph, grids, ninst, seed):
    rng = np.random.default_rng(seed)
    gid = rng.integers(0, len(grids), ninst).astype(np.int32)
    f0 = []
    for i in range(ninst):
        g = grids[gid[i]]
        tr = rng.uniform(1.0, 4.0)
        u = rng.uniform(0.0, 1.5)
        f0.append(0.5 * ph.maxwellian(g, 1.0, u, 0.0, 0.0, 1.0) +
                  0.5 * ph.maxwellian(g, 1.0, -u, 0.0, 0.0, tr))
    return gid, f0


def _cfg(pkg, prec, seed=5):
    return pkg.DVMConfig(iColl=pkg.DVM_COLL_VR, deltat=0.01, seed=seed, precision=prec)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_batch_matches_grouped_contexts(gpulib, pkg, prec):
    ph = pkg.physics
    prec = pkg.DVM_PREC_FP64 if prec == "fp64" else pkg.DVM_PREC_FP32
    grids = [ph.VelocityGrid.uniform(12, -5.0, 5.0), ph.VelocityGrid.uniform(16, -5.0, 5.0)]
    samples = [20000, 40000]
    gid, f0 = _instances(ph, grids, 9, 1)
    batch = pkg.DVMBatch(_cfg(pkg, prec), grids, gid, samples)
    for i, f in enumerate(f0):
        batch.upload_f(i, f)
    # FP32 atomics round in arrival order, so two runs differ at FP32 rounding after one step;
    # from the second step on such differences can move a sample across a CDF boundary and
    # the runs decorrelate, so the FP32 form is compared after one step
    nsteps = 3 if prec == pkg.DVM_PREC_FP64 else 1
    batch.step(nsteps)
    pb = batch.properties()
    for q, g in enumerate(grids):
        members = np.flatnonzero(gid == q)
        cfg = _cfg(pkg, prec)
        cfg.nx_space = len(members)
        cfg.samples_mode = pkg.DVM_SAMPLES_FIXED
        cfg.samples_per_step = samples[q]
        s = pkg.DVMSolver(cfg, g)
        s.initialize_dist_func(np.stack([f0[i] for i in members]))
        s.solve(nsteps)
        ps, fs = s.properties(), s.phi()
        # FP64 scatters in FP64 atomics (order effects at round-off); the FP32 form's FP32
        # atomics round in arrival order, so two runs agree to FP32 rounding of the increment
        ftol, ptol = (1e-12, 1e-11) if prec == pkg.DVM_PREC_FP64 else (1e-5, 1e-6)
        for c, i in enumerate(members):
            fb = batch.download_f(i)
            assert np.abs(fb - fs[c]).max() <= ftol * np.abs(fs[c]).max(), (q, i)
            assert np.abs(pb[i, :17] - ps[c, :17]).max() <= ptol * max(1.0, np.abs(ps[c]).max())


def _batch_props(pkg, grids, gid, samples, f0, prec, seed, steps):
    b = pkg.DVMBatch(_cfg(pkg, prec, seed=seed), grids, gid, samples)
    for i, f in enumerate(f0):
        b.upload_f(i, f)
    b.step(steps)
    p = b.properties()
    b.close()
    return p


def _scale(p64):
    n, T = p64[:, 0:1], p64[:, 4:5]
    return np.concatenate([n, np.sqrt(T).repeat(3, 1), T.repeat(2, 1), np.sqrt(T),
                           0.5 * n * T, (n * T ** 1.5).repeat(3, 1), (0.5 * n * T).repeat(6, 1)],
                          axis=1)


def test_batch_fp32_one_step_error(gpulib, pkg):
    """The precision form's own error: one FP32 step and one FP64 step from the same state
    and the same Philox words (so the same partners) differ only by FP32 rounding."""
    ph = pkg.physics
    grids = [ph.VelocityGrid.uniform(n, -5.0, 5.0) for n in (16, 24)]
    samples = [int(1e5 * (n / 24.0) ** 3) for n in (16, 24)]
    gid, f0 = _instances(ph, grids, 12, 2)
    p64 = _batch_props(pkg, grids, gid, samples, f0, pkg.DVM_PREC_FP64, 11, 1)
    p32 = _batch_props(pkg, grids, gid, samples, f0, pkg.DVM_PREC_FP32, 11, 1)
    err = (np.abs(p32[:, :17] - p64[:, :17]) / _scale(p64)).max(0)
    assert err.max() <= 1e-6, dict(zip(pkg.PROP_NAMES, err))
    assert np.abs(p32[:, 0] - p64[:, 0]).max() <= 1e-12  # mass conserved by both


def test_batch_fp32_ensemble_within_bar(gpulib, pkg):
    """Over ten steps the FP32 and FP64 Monte Carlo realisations decorrelate, so the forms
    are compared as ensembles over seeds: the mean moments agree within three standard
    errors and within the 1e-3 bar."""
    ph = pkg.physics
    grids = [ph.VelocityGrid.uniform(n, -5.0, 5.0) for n in (16, 24)]
    samples = [int(1e5 * (n / 24.0) ** 3) for n in (16, 24)]
    gid, f0 = _instances(ph, grids, 12, 2)
    runs = {}
    for prec in (pkg.DVM_PREC_FP64, pkg.DVM_PREC_FP32):
        runs[prec] = np.stack([_batch_props(pkg, grids, gid, samples, f0, prec, 100 + k, 10)
                               for k in range(6)])
    a, b = runs[pkg.DVM_PREC_FP32], runs[pkg.DVM_PREC_FP64]
    sc = _scale(b.mean(0))
    diff = np.abs(a.mean(0)[:, :17] - b.mean(0)[:, :17]) / sc
    se = np.sqrt(a.var(0, ddof=1) / len(a) + b.var(0, ddof=1) / len(b))[:, :17] / sc
    assert (diff <= 3.0 * se + 1e-12).mean() >= 0.95, (diff.max(), se.max())
    assert diff.max() <= 1e-3, diff.max()


def test_batch_rejects_bad_instances(gpulib, pkg):
    ph = pkg.physics
    grids = [ph.VelocityGrid.uniform(8, -4.0, 4.0)]
    with pytest.raises(pkg.DVMError):
        pkg.DVMBatch(_cfg(pkg, pkg.DVM_PREC_FP64), grids, [0, 1], [1000])
    b = pkg.DVMBatch(_cfg(pkg, pkg.DVM_PREC_FP64), grids, [0, 0], [1000])
    f = np.zeros(grids[0].nv)
    ptr = f.ctypes.data_as(pkg._abi.C.POINTER(pkg._abi.C.c_double))
    assert b.lib.dvm_batch_upload_f(b.b, 2, ptr) == pkg.DVM_ERR_PARAM
    assert b.lib.dvm_batch_step(b.b, -1) == pkg.DVM_ERR_PARAM


def test_batch_one_launch_per_kernel_over_grids(gpulib, pkg):
    """Instances on ten velocity grids (more than one grouped launch holds) step exactly as
    plain multi-cell contexts of each grid's instances do, with one launch of each kernel per
    block of up to eight grids: CDF, plan, collide and moments, then the step counter."""
    ph = pkg.physics
    sizes = list(range(6, 16))
    grids = [ph.VelocityGrid.uniform(n, -4.5, 4.5) for n in sizes]
    samples = [3000 + 500 * q for q in range(len(grids))]
    rng = np.random.default_rng(3)
    gid = np.concatenate([np.arange(len(grids)), rng.integers(0, len(grids), 8)]).astype(np.int32)
    f0 = []
    for i in range(len(gid)):
        g = grids[gid[i]]
        u = rng.uniform(0.0, 1.0)
        f0.append(0.5 * ph.maxwellian(g, 1.0, u, 0.0, 0.0, 1.0) +
                  0.5 * ph.maxwellian(g, 1.0, -u, 0.0, 0.0, 2.0))
    batch = pkg.DVMBatch(_cfg(pkg, pkg.DVM_PREC_FP64), grids, gid, samples)
    for i, f in enumerate(f0):
        batch.upload_f(i, f)
    batch.step(2)
    shape = batch.launch_shape()
    assert shape["launches_per_step"] == 2 * 4 + 1, shape
    assert shape["cdf_threads"] in (256, 512, 1024) and 1 <= shape["collide_ctas_per_sm"] <= 4
    pb = batch.properties()
    for q, g in enumerate(grids):
        members = np.flatnonzero(gid == q)
        cfg = _cfg(pkg, pkg.DVM_PREC_FP64)
        cfg.nx_space = len(members)
        cfg.samples_mode = pkg.DVM_SAMPLES_FIXED
        cfg.samples_per_step = samples[q]
        s = pkg.DVMSolver(cfg, g)
        s.initialize_dist_func(np.stack([f0[i] for i in members]))
        s.solve(2)
        ps, fs = s.properties(), s.phi()
        s.close()
        for c, i in enumerate(members):
            fb = batch.download_f(i)
            assert np.abs(fb - fs[c]).max() <= 1e-12 * np.abs(fs[c]).max(), (q, i)
            assert np.abs(pb[i, :17] - ps[c, :17]).max() <= 1e-11 * max(1.0, np.abs(ps[c]).max())
    batch.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_batch_configuration4_grids_single_grouped_launch(gpulib, pkg, prec):
    """The four grids of configuration 4 (16^3, 24^3, 32^3, 40^3: the two largest read their
    velocity table through L1, the others stage it in shared memory) advance in one grouped
    launch of each kernel; FP64 equals the per-grid contexts to 1e-12 after two steps."""
    ph = pkg.physics
    prec = pkg.DVM_PREC_FP64 if prec == "fp64" else pkg.DVM_PREC_FP32
    grids = [ph.VelocityGrid.uniform(n, -5.0, 5.0) for n in (16, 24, 32, 40)]
    samples = [int(2e4 * (n / 24.0) ** 3) for n in (16, 24, 32, 40)]
    gid, f0 = _instances(ph, grids, 10, 4)
    batch = pkg.DVMBatch(_cfg(pkg, prec), grids, gid, samples)
    for i, f in enumerate(f0):
        batch.upload_f(i, f)
    nsteps = 2 if prec == pkg.DVM_PREC_FP64 else 1
    batch.step(nsteps)
    assert batch.launch_shape()["launches_per_step"] == (4 if prec == pkg.DVM_PREC_FP64 else 5) + 1
    for q, g in enumerate(grids):
        members = np.flatnonzero(gid == q)
        if len(members) == 0:
            continue
        cfg = _cfg(pkg, prec)
        cfg.nx_space = len(members)
        cfg.samples_mode = pkg.DVM_SAMPLES_FIXED
        cfg.samples_per_step = samples[q]
        s = pkg.DVMSolver(cfg, g)
        s.initialize_dist_func(np.stack([f0[i] for i in members]))
        s.solve(nsteps)
        fs = s.phi()
        s.close()
        ftol = 1e-12 if prec == pkg.DVM_PREC_FP64 else 1e-5
        for c, i in enumerate(members):
            fb = batch.download_f(i)
            assert np.abs(fb - fs[c]).max() <= ftol * np.abs(fs[c]).max(), (q, i)
    batch.close()


def _row_states(ph, g, rows, nxs, seed):
    rng = np.random.default_rng(seed)
    out = []
    for r in range(rows):
        f, _, _ = ph.shock_profile(g, nxs, 0.5, 1.6 + 0.3 * r, 1.5)
        out.append(f * (1.0 + 0.05 * rng.random(f.shape)))
    return out


@pytest.mark.parametrize("bc", [("INOUT", "INOUT"), ("DIFFUSE", "SPECULAR"),
                                ("ZEROGRAD", "DIFFUSE")])
def test_1d_rows_equal_single_row_contexts(gpulib, pkg, bc):
    """A 1-D context of several rows (ny_space > 1) is that many independent 1-D domains,
    each with both end conditions: three convection steps of a three-row context equal three
    single-row contexts to 1e-12 (partial accommodation, so the diffuse end's specular remap
    runs too)."""
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(10, -5.0, 5.0)
    nxs, rows = 6, 3
    f0 = _row_states(ph, g, rows, nxs, 1)
    code = {"INOUT": pkg.DVM_BC1D_INOUT, "DIFFUSE": pkg.DVM_BC1D_DIFFUSE,
            "SPECULAR": pkg.DVM_BC1D_SPECULAR, "ZEROGRAD": pkg.DVM_BC1D_ZEROGRAD}
    walls = ((1.5, -0.8, 0.0, 0.0, 1.4), (1.0, -1.6, 0.0, 0.0, 1.0), (1, 0, 0, 0, 1.0),
             (1, 0, 0, 0, 1.0))

    def cfg(ny):
        return pkg.DVMConfig(geometry=pkg.DVM_GEOM_1D, nx_space=nxs, ny_space=ny, dx=0.5,
                             deltat=0.05, iColl=pkg.DVM_COLL_NONE, iConv=pkg.DVM_CONV_UPWIND1,
                             bc=(code[bc[0]], code[bc[1]], 0, 0), walls=walls, acc_coeff=0.7)

    multi = pkg.DVMSolver(cfg(rows), g)
    multi.initialize_dist_func(np.concatenate(f0))
    multi.solve(3)
    fm, pm = multi.phi(), multi.properties()
    assert multi.error_word() == 0
    for r in range(rows):
        s = pkg.DVMSolver(cfg(1), g)
        s.initialize_dist_func(f0[r])
        s.solve(3)
        fs, ps = s.phi(), s.properties()
        s.close()
        rr = slice(r * nxs, (r + 1) * nxs)
        assert np.abs(fm[rr] - fs).max() <= 1e-12 * np.abs(fs).max(), r
        assert np.abs(pm[rr, :17] - ps[:, :17]).max() <= 1e-11 * max(1.0, np.abs(ps).max())
    multi.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_batch_1d_instances(gpulib, pkg, prec):
    """1-D instances join the batch: five 8-cell shock instances on two grids (inflow ends,
    VR collisions), one grouped launch of each collision kernel plus the convection of each
    grid per step. Three steps (both placements of f, so both of the batch's graphs) equal
    the multi-row contexts of each grid's instances: FP64 to 1e-12; FP32 one step to the
    FP32 rounding of the increment."""
    ph = pkg.physics
    prec = pkg.DVM_PREC_FP64 if prec == "fp64" else pkg.DVM_PREC_FP32
    grids = [ph.VelocityGrid.uniform(12, -6.0, 6.0), ph.VelocityGrid.uniform(14, -6.0, 6.0)]
    samples = [3000, 4000]
    gid = np.array([0, 1, 0, 1, 1], dtype=np.int32)
    nxs = 8
    f0 = [_row_states(ph, grids[q], 1, nxs, 10 + i)[0] for i, q in enumerate(gid)]
    _, up, dn = ph.shock_profile(grids[0], nxs, 0.5, 1.6, 1.5)
    walls = ((dn["n"], dn["u"], 0.0, 0.0, dn["T"]), (up["n"], up["u"], 0.0, 0.0, up["T"]),
             (1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0))

    def cfg(ny=1, fixed=None):
        c = pkg.DVMConfig(geometry=pkg.DVM_GEOM_1D, nx_space=nxs, ny_space=ny, dx=0.5,
                          deltat=0.05, iColl=pkg.DVM_COLL_VR, iConv=pkg.DVM_CONV_UPWIND1,
                          bc=(pkg.DVM_BC1D_INOUT, pkg.DVM_BC1D_INOUT, 0, 0), walls=walls,
                          seed=21, precision=prec)
        if fixed is not None:
            c.samples_mode = pkg.DVM_SAMPLES_FIXED
            c.samples_per_step = fixed
        return c

    batch = pkg.DVMBatch(cfg(), grids, gid, samples)
    for i, f in enumerate(f0):
        batch.upload_f(i, f)
    nsteps = 3 if prec == pkg.DVM_PREC_FP64 else 1
    batch.step(nsteps)
    shape = batch.launch_shape()
    assert shape["launches_per_step"] == (4 if prec == pkg.DVM_PREC_FP64 else 5) + 2 * 2 + 1
    pb = batch.properties()
    assert pb.shape == (len(gid), nxs, pkg.DVM_NPROP)
    for q, g in enumerate(grids):
        members = np.flatnonzero(gid == q)
        s = pkg.DVMSolver(cfg(len(members), samples[q]), g)
        s.initialize_dist_func(np.concatenate([f0[i] for i in members]))
        s.solve(nsteps)
        fs, ps = s.phi(), s.properties()
        assert s.error_word() == 0
        s.close()
        ftol = 1e-12 if prec == pkg.DVM_PREC_FP64 else 1e-5
        for c, i in enumerate(members):
            rr = slice(c * nxs, (c + 1) * nxs)
            fb = batch.download_f(i)
            assert fb.shape == (nxs, g.nv)
            assert np.abs(fb - fs[rr]).max() <= ftol * np.abs(fs[rr]).max(), (q, i)
            if prec == pkg.DVM_PREC_FP64:
                assert np.abs(pb[i, :, :17] - ps[rr, :17]).max() <= 1e-11 * max(1.0, np.abs(ps).max())
    batch.close()
