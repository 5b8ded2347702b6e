"""dvm_collide_noalloc: the collision integral for callers that cannot allocate device
memory (a host that owns all device memory, a pool held at a fixed budget, a real-time
loop that must stay out of the allocator). The caller hands over its own device buffers
for f and the cell properties; the library's fixed scratch array holds everything else.

The check: two calls in a row give the same distributions, within the FP64 parity bar of
the other GPU tests, as the context entry point dvm_compute_collision_integral. This file
is named to be collected last, and passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1.0e-12


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("method", ["VR", "FMC"])
def test_noalloc_matches_context_entry_point(gpulib, pkg, method):
    import torch

    ph = pkg.physics
    g = ph.VelocityGrid.uniform(16, -5.0, 5.0)
    ncells = 6
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
        st = gpulib.dvm_collide_noalloc(C.byref(params), C.byref(vg), C.c_void_p(fd.data_ptr()),
                                        C.c_void_p(pd.data_ptr()), ncells, step, None,
                                        C.byref(n))
        assert st == pkg.DVM_OK, gpulib.dvm_strerror(st)
        assert n.value == ncells * 30000
        assert _rel(fd.cpu().numpy(), want) <= REL


def test_noalloc_rejects_problems_beyond_its_scratch(gpulib, pkg):
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(32, -5.0, 5.0)
    params = pkg.DVMConfig(nx_space=200, iColl=pkg.DVM_COLL_VR,
                           samples_mode=pkg.DVM_SAMPLES_FIXED, samples_per_step=10).to_params()
    vg = pkg.make_vgrid(g)
    dummy = C.c_void_p(1)  # never dereferenced: the size check comes first
    st = gpulib.dvm_collide_noalloc(C.byref(params), C.byref(vg), dummy, dummy, 200, 0, None,
                                    None)
    assert st == pkg.DVM_ERR_TOO_LARGE
    assert b"32 MiB" in gpulib.dvm_strerror(st)
