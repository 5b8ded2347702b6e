"""The C-ABI library: it loads, exports every entry point the header declares, its structs
match the ctypes mirror, and it validates parameters before touching a device.
No compute call is made here (no GPU needed)."""
import ctypes as C
import importlib
import os
import re
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
HEADER = os.path.join(REPO, "include", "dvm_gpu.h")


@pytest.fixture(scope="module")
def lib(pkg):
    if not os.path.exists(pkg.LIB_PATH):
        importlib.import_module("2d_dvm_microflows_gb300.build").build()
    return pkg.load_library()


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(dvm_\w+)\s*\(", text, re.M)))


def test_exports_every_declared_symbol(lib, pkg):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(pkg._abi.ENTRY_POINTS), set(names) ^ set(pkg._abi.ENTRY_POINTS)
    out = subprocess.run(["nm", "-D", "--defined-only", pkg.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r" T (dvm_\w+)", out))
    assert set(names) <= exported


def test_struct_layout_matches_header(tmp_path, pkg):
    src = tmp_path / "sz.c"
    src.write_text(r'''
#include <stdio.h>
#include <stddef.h>
#include "dvm_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(dvm_params), sizeof(dvm_vgrid),
         sizeof(dvm_pairlist), offsetof(dvm_params, samples_per_step),
         offsetof(dvm_params, dx), offsetof(dvm_params, wall), offsetof(dvm_pairlist, r_cos),
         offsetof(dvm_params, precision), sizeof(dvm_request_info),
         offsetof(dvm_request_info, collisions));
  return 0;
}''')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True,
                                          text=True).stdout.split()]
    a = pkg._abi
    want = [C.sizeof(a.dvm_params), C.sizeof(a.dvm_vgrid), C.sizeof(a.dvm_pairlist),
            a.dvm_params.samples_per_step.offset, a.dvm_params.dx.offset,
            a.dvm_params.wall.offset, a.dvm_pairlist.r_cos.offset,
            a.dvm_params.precision.offset, C.sizeof(a.dvm_request_info),
            a.dvm_request_info.collisions.offset]
    assert got == want


def test_abi_version_and_strings(lib, pkg):
    assert lib.dvm_abi_version() == pkg._abi.DVM_ABI_VERSION
    assert lib.dvm_strerror(0) == b"ok"
    assert lib.dvm_strerror(1) == b"invalid parameter"
    assert lib.dvm_kernel_name(2) == b"collide"


def _params(pkg, **kw):
    cfg = pkg.DVMConfig(**kw)
    return cfg.to_params()


def test_create_rejects_bad_parameters(lib, pkg):
    ph = pkg.physics
    g = ph.VelocityGrid.uniform(8, -3.0, 3.0)
    vg = pkg.make_vgrid(g)
    ctx = C.c_void_p()
    bad = [dict(NRepl=0), dict(deltat=0.0), dict(iColl=1), dict(Kn=-1.0),
           dict(geometry=pkg.DVM_GEOM_0D, iConv=pkg.DVM_CONV_UPWIND1),
           dict(geometry=pkg.DVM_GEOM_1D, nx_space=2, iConv=pkg.DVM_CONV_UPWIND1,
                bc=(3, 3, 0, 0)),
           dict(geometry=pkg.DVM_GEOM_1D, nx_space=5, iConv=pkg.DVM_CONV_UPWIND1,
                bc=(9, 3, 0, 0))]
    for kw in bad:
        p = _params(pkg, **kw)
        assert lib.dvm_create(C.byref(p), C.byref(vg), C.byref(ctx)) == pkg.DVM_ERR_PARAM, kw
    # a non-increasing axis
    g2 = ph.VelocityGrid(np.array([0.0, 1.0, 1.0]))
    vg2 = pkg.make_vgrid(g2)
    p = _params(pkg)
    assert lib.dvm_create(C.byref(p), C.byref(vg2), C.byref(ctx)) == pkg.DVM_ERR_PARAM


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="a GPU is present")
def test_create_without_device_reports_nodevice(lib, pkg):
    g = pkg.physics.VelocityGrid.uniform(8, -3.0, 3.0)
    vg = pkg.make_vgrid(g)
    p = _params(pkg)
    ctx = C.c_void_p()
    assert lib.dvm_create(C.byref(p), C.byref(vg), C.byref(ctx)) == pkg.DVM_ERR_NODEVICE


def test_product_path_has_no_cpu_fallback(pkg, tmp_path):
    """Without the library the host raises instead of computing anything."""
    with pytest.raises(RuntimeError):
        pkg.load_library(str(tmp_path / "missing.so"))
