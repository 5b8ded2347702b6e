"""dvm_collide_noalloc: the collision integral for callers that cannot allocate device
memory (a host that owns all device memory, a pool held at a fixed budget, a real-time
loop that must stay out of the allocator). The caller hands over its own device buffers
for f and the cell properties; the library's fixed scratch array holds everything else.

The check: two calls in a row give the same distributions, within the FP64 parity bar of
the other GPU tests, as the context entry point dvm_compute_collision_integral -- on a
cubic grid whose velocity table is staged in shared memory, on one whose table is read
through L1, and on a stretched grid with no table. The size limit stated in the header is
exact, and an error of a call that did not wait is reported by the next call that does.
This file is named to be collected last, and passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1.0e-12


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def _stretched(n, vmax, beta):
    s = np.linspace(-1.0, 1.0, n)
    return vmax * np.tanh(beta * s) / np.tanh(beta)


def _grid(ph, kind):
    if kind == "cubic16":      # (g, g^(2-2w)) table staged in shared memory
        return ph.VelocityGrid.uniform(16, -5.0, 5.0)
    if kind == "cubic32":      # table too large to stage: read through L1
        return ph.VelocityGrid.uniform(32, -6.0, 6.0)
    return ph.VelocityGrid(_stretched(12, 5.0, 1.5), _stretched(11, 5.0, 1.2),
                           _stretched(13, 5.5, 1.4))  # no table, remap tables per axis


def _noalloc(lib, pkg, params, vg, fd, pd, ncells, step, collisions):
    ref = C.byref(collisions) if collisions is not None else None
    return lib.dvm_collide_noalloc(C.byref(params), C.byref(vg), C.c_void_p(fd.data_ptr()),
                                   C.c_void_p(pd.data_ptr()), ncells, step, None, ref)


@pytest.mark.parametrize("kind,method", [("cubic16", "VR"), ("cubic16", "FMC"),
                                         ("cubic32", "VR"), ("stretched", "VR"),
                                         ("stretched", "FMC")])
def test_noalloc_matches_context_entry_point(gpulib, pkg, kind, method):
    import torch

    ph = pkg.physics
    g = _grid(ph, kind)
    ncells = 6 if kind != "cubic32" else 3
    f0 = np.stack([ph.bimodal(g, u1=0.5 + 0.1 * c, T2=1.5 + 0.3 * c) for c in range(ncells)])
    coll = pkg.DVM_COLL_VR if method == "VR" else pkg.DVM_COLL_FMC
    cfg = pkg.DVMConfig(nx_space=ncells, iColl=coll, samples_mode=pkg.DVM_SAMPLES_FIXED,
                        samples_per_step=30000, deltat=0.02, omega=0.81, cdf_tolerance=0.0,
                        seed=17)
    # the existing entry point, on a context
    s = pkg.DVMSolver(cfg, g)
    s.initialize_dist_func(f0)
    props = s.properties()
    s.compute_collision_integral(step=0)
    f1_ctx = s.phi()
    s.compute_collision_integral(step=1)
    f2_ctx = s.phi()
    s.close()

    # the no-allocation entry point on caller-owned device buffers
    fd = torch.tensor(f0, dtype=torch.float64, device="cuda")
    pd = torch.tensor(props, dtype=torch.float64, device="cuda")
    params = cfg.to_params()
    vg = pkg.make_vgrid(g)
    n = C.c_int64(-1)
    torch.cuda.synchronize()
    for step, want in ((0, f1_ctx), (1, f2_ctx)):
        st = _noalloc(gpulib, pkg, params, vg, fd, pd, ncells, step, n)
        assert st == pkg.DVM_OK, gpulib.dvm_strerror(st)
        assert n.value == ncells * 30000
        assert _rel(fd.cpu().numpy(), want) <= REL


@pytest.mark.parametrize("n,most", [(24, 141), (32, 61)])
def test_noalloc_size_limit_is_exact(gpulib, pkg, n, most):
    """The documented limit (141 cells of 24^3, 61 of 32^3) runs; one cell more is refused
    before anything touches the buffers."""
    import torch

    ph = pkg.physics
    g = ph.VelocityGrid.uniform(n, -5.0, 5.0)
    vg = pkg.make_vgrid(g)
    over = pkg.DVMConfig(nx_space=most + 1, iColl=pkg.DVM_COLL_VR,
                         samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=10).to_params()
    dummy = C.c_void_p(1)  # never dereferenced: the size check comes first
    st = gpulib.dvm_collide_noalloc(C.byref(over), C.byref(vg), dummy, dummy, most + 1, 0, None,
                                    None)
    assert st == pkg.DVM_ERR_TOO_LARGE
    assert b"32 MiB" in gpulib.dvm_strerror(st)

    cfg = pkg.DVMConfig(nx_space=most, iColl=pkg.DVM_COLL_VR, samples_mode=pkg.DVM_SAMPLES_FIXED,
                        samples_per_step=500, deltat=0.02, seed=5)
    f0 = np.tile(ph.bimodal(g), (most, 1))
    s = pkg.DVMSolver(cfg, g)
    s.initialize_dist_func(f0)
    props = s.properties()
    s.compute_collision_integral(step=0)
    want = s.phi()
    s.close()
    fd = torch.tensor(f0, dtype=torch.float64, device="cuda")
    pd = torch.tensor(props, dtype=torch.float64, device="cuda")
    cnt = C.c_int64(-1)
    torch.cuda.synchronize()
    st = _noalloc(gpulib, pkg, cfg.to_params(), vg, fd, pd, most, 0, cnt)
    assert st == pkg.DVM_OK, gpulib.dvm_strerror(st)
    assert cnt.value == most * 500
    assert _rel(fd.cpu().numpy(), want) <= REL


def test_noalloc_error_of_a_call_that_did_not_wait(gpulib, pkg):
    """A non-finite node in a host-prepared f (the properties are those of the clean f) is
    caught by the CDF build. A call made without `collisions` does not wait, so the next call
    that does reports it (DVM_ERR_NUMERIC); the call after that, on clean data, is OK."""
    import torch

    ph = pkg.physics
    g = ph.VelocityGrid.uniform(12, -5.0, 5.0)
    cfg = pkg.DVMConfig(nx_space=2, iColl=pkg.DVM_COLL_VR, samples_mode=pkg.DVM_SAMPLES_FIXED,
                        samples_per_step=2000, deltat=0.02, seed=9)
    f0 = np.stack([ph.bimodal(g), ph.bimodal(g, u1=0.4)])
    s = pkg.DVMSolver(cfg, g)
    s.initialize_dist_func(f0)
    props = s.properties()
    s.close()
    params, vg = cfg.to_params(), pkg.make_vgrid(g)
    pd = torch.tensor(props, dtype=torch.float64, device="cuda")
    bad = f0.copy()
    bad[1, g.nv // 2] = np.nan
    fbad = torch.tensor(bad, dtype=torch.float64, device="cuda")
    cnt = C.c_int64(-1)
    torch.cuda.synchronize()
    assert _noalloc(gpulib, pkg, params, vg, fbad, pd, 2, 0, None) == pkg.DVM_OK
    fok = torch.tensor(f0, dtype=torch.float64, device="cuda")
    assert _noalloc(gpulib, pkg, params, vg, fok, pd, 2, 0, cnt) == pkg.DVM_ERR_NUMERIC
    fok = torch.tensor(f0, dtype=torch.float64, device="cuda")
    assert _noalloc(gpulib, pkg, params, vg, fok, pd, 2, 0, cnt) == pkg.DVM_OK
    assert cnt.value == 2 * 2000
