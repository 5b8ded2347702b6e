"""Request server (dvm_server_*): continuous batching of independent solves admitted by HBM
footprint. Each result must be the same alone and in a mix (FP64: to 1e-12 relative, the
bar of the recorded-list parity; FP32: within the 1e-3 moment bar), and the same as the
plain solver running the same steps; admission must respect the footprint budget."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _shock(pkg, ph, cells, n, mach, seed, prec):
    g = ph.VelocityGrid.uniform(n, -6.0, 6.0)
    mol = ph.molecule("Ar", ph.CSECTION_VHS)
    f0, up, dn = ph.shock_profile(g, cells, 0.5, mach, 3.0)
    walls = ((dn["n"], dn["u"], 0.0, 0.0, dn["T"]), (up["n"], up["u"], 0.0, 0.0, up["T"]),
             (1.0, 0.0, 0.0, 0.0, 1.0), (1.0, 0.0, 0.0, 0.0, 1.0))
    cfg = pkg.DVMConfig(geometry=pkg.DVM_GEOM_1D, nx_space=cells, dx=0.5, deltat=0.05,
                        Kn=1.0, mass=mol["mass"], omega=mol["omega"], alpha=mol["alpha"],
                        sigma=ph.cross_section(mol, ph.CSECTION_BIRD), iColl=pkg.DVM_COLL_VR,
                        iConv=pkg.DVM_CONV_UPWIND1, samples_mode=pkg.DVM_SAMPLES_FIXED,
                        samples_per_step=4000, bc=(pkg.DVM_BC1D_INOUT, pkg.DVM_BC1D_INOUT, 0, 0),
                        walls=walls, seed=seed,
                        precision=prec)
    return cfg, g, f0


def _cavity(pkg, ph, nside, n, kn, seed, prec):
    g = ph.VelocityGrid.uniform(n, -5.0, 5.0)
    f0 = np.tile(ph.maxwellian(g, 1.0, 0.0, 0.0, 0.0, 1.0), (nside * nside, 1))
    walls = ((1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0, 0, 0, 1.0), (1, 0.3, 0, 0, 1.0))
    cfg = pkg.DVMConfig(geometry=pkg.DVM_GEOM_2D, nx_space=nside, ny_space=nside,
                        dx=1.0 / nside, dy=1.0 / nside, deltat=0.01, Kn=kn,
                        iColl=pkg.DVM_COLL_VR, iConv=pkg.DVM_CONV_UPWIND1,
                        samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=3000, walls=walls,
                        seed=seed, precision=prec)
    return cfg, g, f0


def _relax(pkg, ph, n, seed, prec):
    g = ph.VelocityGrid.uniform(n, -5.0, 5.0)
    cfg = pkg.DVMConfig(iColl=pkg.DVM_COLL_VR, deltat=0.05, samples_mode=pkg.DVM_SAMPLES_FIXED,
                        samples_per_step=20000, seed=seed, precision=prec)
    return cfg, g, ph.bimodal(g)[None, :]


def _requests(pkg, prec):
    ph = pkg.physics
    return [(_shock(pkg, ph, 12, 12, 2.0, 1, prec), 7),
            (_cavity(pkg, ph, 5, 10, 0.1, 2, prec), 6),
            (_relax(pkg, ph, 14, 3, prec), 5),
            (_shock(pkg, ph, 9, 10, 3.0, 4, prec), 8),
            (_cavity(pkg, ph, 4, 12, 1.0, 5, prec), 4)]


def _serve(pkg, reqs, max_active, budget=8 << 30, turn=2):
    out = []
    with pkg.DVMServer(budget, max_active=max_active, steps_per_turn=turn) as sv:
        ids = [sv.submit(cfg, g, f0, steps) for (cfg, g, f0), steps in reqs]
        for rid in ids:
            info = sv.wait(rid)
            props, f = sv.result(rid)
            out.append((info, props, f))
        stats = sv.stats()
    return out, stats


def test_footprint_matches_allocation(gpulib, pkg):
    for (cfg, g, f0), steps in _requests(pkg, pkg.DVM_PREC_FP32) + _requests(pkg, pkg.DVM_PREC_FP64)[:2]:
        res, _ = _serve(pkg, [((cfg, g, f0), 1)], 1)
        assert res[0][0]["status"] == 0
        assert res[0][0]["device_bytes"] == pkg.footprint_bytes(cfg, g)


def test_fp64_alone_equals_mix_equals_plain(gpulib, pkg):
    reqs = _requests(pkg, pkg.DVM_PREC_FP64)
    mix, stats = _serve(pkg, reqs, max_active=len(reqs))
    assert stats["completed"] == len(reqs) and stats["peak_active"] >= 2
    for q, ((cfg, g, f0), steps) in enumerate(reqs):
        alone, _ = _serve(pkg, [((cfg, g, f0), steps)], 1, turn=3)
        s = pkg.DVMSolver(cfg, g)
        s.initialize_dist_func(f0)
        s.solve(steps)
        fp = s.phi()
        for info, props, f in (mix[q], alone[0]):
            assert info["status"] == 0 and info["steps"] == steps
            assert np.abs(f - fp).max() <= 1e-12 * np.abs(fp).max(), q
        assert mix[q][0]["collisions"] > 0


def test_fp32_alone_equals_mix(gpulib, pkg):
    reqs = _requests(pkg, pkg.DVM_PREC_FP32)
    mix, _ = _serve(pkg, reqs, max_active=len(reqs))
    for q, req in enumerate(reqs):
        alone, _ = _serve(pkg, [req], 1)
        pa, pm = alone[0][1], mix[q][1]
        n, T = np.abs(pa[:, 0]).max(), np.abs(pa[:, 4]).max()
        scale = np.array([n] + [T ** 0.5] * 3 + [T, T, T ** 0.5, 0.5 * n * T] +
                         [n * T ** 1.5] * 3 + [0.5 * n * T] * 6)
        err = (np.abs(pm[:, :17] - pa[:, :17]) / scale).max()
        assert err <= 1e-3, (q, err)


def test_admission_respects_budget(gpulib, pkg):
    reqs = _requests(pkg, pkg.DVM_PREC_FP64)
    sizes = [pkg.footprint_bytes(cfg, g) + 12 for (cfg, g, _), _ in reqs]
    budget = max(sizes) + min(sizes)  # never room for more than a couple at once
    res, stats = _serve(pkg, reqs, max_active=8, budget=budget)
    assert all(r[0]["status"] == 0 for r in res)
    assert stats["peak_bytes"] <= budget
    assert stats["completed"] == len(reqs)
    with pkg.DVMServer(min(sizes) - 1, max_active=2) as sv:
        (cfg, g, f0), _ = reqs[0]
        with pytest.raises(pkg.DVMError) as e:
            sv.submit(cfg, g, f0, 2)
        assert e.value.status == pkg.DVM_ERR_TOO_LARGE


def test_residual_ends_a_relaxation(gpulib, pkg):
    """A homogeneous relaxation stops once its per-step change falls below the tolerance."""
    ph = pkg.physics
    (cfg, g, f0) = _relax(pkg, ph, 14, 7, pkg.DVM_PREC_FP64)
    with pkg.DVMServer(1 << 30, max_active=2) as sv:
        rid = sv.submit(cfg, g, f0, 400, residual_tol=2e-3)
        info = sv.wait(rid)
        sv.result(rid)
    assert info["status"] == 0 and info["converged"] == 1
    assert info["steps"] < 400 and info["residual"] <= 2e-3


def test_preemption_resumes_exactly(gpulib, pkg):
    """Round-robin through the checkpoint: one slot and preemption after every turn, so the
    requests take turns and each is checkpointed to host memory and resumed several times.
    Every result equals its uninterrupted run (FP64: 1e-12 relative), with the same steps
    and collision count."""
    reqs = _requests(pkg, pkg.DVM_PREC_FP64)
    with pkg.DVMServer(8 << 30, max_active=1, steps_per_turn=2, preempt_turns=1) as sv:
        ids = [sv.submit(cfg, g, f0, steps) for (cfg, g, f0), steps in reqs]
        res = []
        for rid in ids:
            info = sv.wait(rid)
            props, f = sv.result(rid)
            res.append((info, props, f))
        assert sv.stats()["completed"] == len(reqs)
    assert sum(info["preempted"] for info, _, _ in res) >= len(reqs) - 1
    for ((cfg, g, f0), steps), (info, props, f) in zip(reqs, res):
        alone, _ = _serve(pkg, [((cfg, g, f0), steps)], 1)
        ainfo, aprops, af = alone[0]
        assert info["status"] == 0 and info["steps"] == steps == ainfo["steps"]
        assert info["collisions"] == ainfo["collisions"]
        assert np.abs(f - af).max() <= 1e-12 * np.abs(af).max()
        assert np.abs(props[:, :17] - aprops[:, :17]).max() <= 1e-11


def test_preemption_off_by_default(gpulib, pkg):
    reqs = _requests(pkg, pkg.DVM_PREC_FP64)[:3]
    res, _ = _serve(pkg, reqs, max_active=1)
    assert all(info["preempted"] == 0 for info, _, _ in res)


def test_served_mix_ensemble_accuracy(gpulib, pkg):
    """The accuracy bar of the served precision form, at matched ensembles: a mix of shock
    and cavity requests served in FP32 (continuous batching, several in flight) under 8
    independent seeds, against the same requests run plainly in FP64 under 8 other seeds.
    After 12 steps the ensemble means of every moment field agree within 1e-3 of the field's
    scale in every cell."""
    import dataclasses

    ph = pkg.physics
    kinds = [lambda prec, seed: _shock(pkg, ph, 24, 14, 2.0, seed, prec),
             lambda prec, seed: _cavity(pkg, ph, 8, 12, 0.1, seed, prec)]
    K, steps = 8, 12
    for make in kinds:
        reqs = [(make(pkg.DVM_PREC_FP32, 100 + k), steps) for k in range(K)]
        reqs = [((dataclasses.replace(c, samples_per_step=40000), g, f0), n)
                for (c, g, f0), n in reqs]
        res, _ = _serve(pkg, reqs, max_active=4)
        served = np.array([props[:, :17] for _, props, _ in res])
        plain = []
        for k in range(K):
            c, g, f0 = make(pkg.DVM_PREC_FP64, 500 + k)
            s = pkg.DVMSolver(dataclasses.replace(c, samples_per_step=40000), g)
            s.initialize_dist_func(f0)
            s.solve(steps)
            plain.append(s.properties()[:, :17])
            s.close()
        plain = np.array(plain)
        m32, m64 = served.mean(0), plain.mean(0)
        n, T = np.abs(m64[:, 0]).max(), np.abs(m64[:, 4]).max()
        pr = 0.5 * n * T
        sc = np.array([n, T ** 0.5, T ** 0.5, T ** 0.5, T, T, T ** 0.5, pr] +
                      [n * T ** 1.5] * 3 + [pr] * 6)
        assert (np.abs(m32 - m64).max(0) / sc).max() <= 1e-3
