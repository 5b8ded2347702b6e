"""ctypes binding of the CPU restatement (oracle/dvm_oracle.c). TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, as
the checker or as the timed CPU baseline; the product path never imports it.
`OracleSolver` exposes the same calls as the GPU host mirror `DVMSolver`, so a parity test
runs the same sequence on both and compares.
"""
import ctypes as C
import importlib
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libdvm_oracle.so")

pkg = importlib.import_module("2d_dvm_microflows_gb300")
abi = pkg._abi

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        P, D, I = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)
        sig = {
            "orc_create": (P, [C.POINTER(abi.dvm_params), C.POINTER(abi.dvm_vgrid)]),
            "orc_destroy": (None, [P]),
            "orc_set_threads": (None, [P, C.c_int]),
            "orc_max_threads": (C.c_int, []),
            "orc_set_f": (None, [P, D]),
            "orc_get_f": (None, [P, D]),
            "orc_get_props": (None, [P, D]),
            "orc_set_props": (None, [P, D]),
            "orc_calculate_physical_properties": (None, [P]),
            "orc_compute_collision_integral": (C.c_int, [P, C.c_uint64, C.POINTER(abi.dvm_pairlist)]),
            "orc_compute_convection": (C.c_int, [P]),
            "orc_step": (C.c_int, [P, C.c_uint64, C.c_int]),
            "orc_last_collision_count": (C.c_int64, [P]),
            "orc_last_scatter_count": (C.c_int64, [P]),
            "orc_error_word": (C.c_uint32, [P]),
            "orc_grid_info": (None, [P, D, I]),
            "orc_remap_grid": (C.c_int, [C.POINTER(abi.dvm_vgrid), C.c_double, C.c_double,
                                         C.c_double, C.c_double, I, D]),
            "orc_center_of_mass_velocity": (None, [D, D, D, D, D]),
            "orc_philox4x32_10": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                         C.POINTER(C.c_uint32)]),
            "orc_philox_uniform2": (None, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                           C.c_uint32, C.c_uint32, D]),
            "orc_referenced_search": (C.c_int, [D, I, C.c_int, C.c_double]),
            "orc_build_ref_table": (None, [D, C.c_int, I]),
            "orc_wall_ghost_2d": (C.c_int, [P, C.c_int, C.c_int, C.c_int, D]),
            "orc_cell_cdf_vr": (C.c_int, [P, C.c_int, D, D, D, I, I]),
            "orc_set_eq_node_mode": (C.c_int, [P, C.c_int]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


class OracleSolver:
    """CPU restatement with DVMSolver's interface."""

    def __init__(self, config, grid, threads=1):
        self.L = lib()
        self.config = config
        self.grid = grid
        self._params = config.to_params()
        vg = pkg.make_vgrid(grid)
        self.ctx = self.L.orc_create(C.byref(self._params), C.byref(vg))
        if not self.ctx:
            raise ValueError("oracle rejected the grid")
        self.L.orc_set_threads(self.ctx, int(threads))
        self.ncells = config.nx_space * config.ny_space
        self.nv = grid.nv
        self.ntime = 0

    def set_eq_node_mode(self, direct):
        """Test aid: True forms the equilibrium node values directly (as the GPU kernels do)
        instead of as differences of the reference's running sum; see orc_set_eq_node_mode."""
        if self.L.orc_set_eq_node_mode(self.ctx, 1 if direct else 0):
            raise RuntimeError("oracle: cannot set the equilibrium node mode")

    def close(self):
        if getattr(self, "ctx", None):
            self.L.orc_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize_dist_func(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(self.ncells, self.nv)
        self.L.orc_set_f(self.ctx, _d(f))
        self.L.orc_calculate_physical_properties(self.ctx)

    def phi(self):
        out = np.empty((self.ncells, self.nv))
        self.L.orc_get_f(self.ctx, _d(out))
        return out

    def properties(self):
        out = np.empty((self.ncells, abi.DVM_NPROP))
        self.L.orc_get_props(self.ctx, _d(out))
        return out

    def set_properties(self, props):
        props = np.ascontiguousarray(props, dtype=np.float64).reshape(self.ncells, abi.DVM_NPROP)
        self.L.orc_set_props(self.ctx, _d(props))

    def compute_collision_integral(self, step=None, pairs=None):
        step = self.ntime if step is None else step
        ref = pairs.ref() if pairs is not None else None
        st = self.L.orc_compute_collision_integral(self.ctx, C.c_uint64(step), ref)
        if st:
            raise RuntimeError("oracle collision status %d" % st)

    def compute_convection(self):
        st = self.L.orc_compute_convection(self.ctx)
        if st:
            raise RuntimeError("oracle convection status %d" % st)

    def calculate_physical_properties(self):
        self.L.orc_calculate_physical_properties(self.ctx)

    def solve(self, nsteps):
        st = self.L.orc_step(self.ctx, C.c_uint64(self.ntime), int(nsteps))
        if st:
            raise RuntimeError("oracle step status %d" % st)
        self.ntime += nsteps

    def collision_count(self):
        return int(self.L.orc_last_collision_count(self.ctx))

    def scatter_count(self):
        """Adds into f by the last collision call: 2 depletions per sample plus the stencil
        nodes of each replenishment."""
        return int(self.L.orc_last_scatter_count(self.ctx))

    def error_word(self):
        return int(self.L.orc_error_word(self.ctx))

    def grid_info(self):
        b3 = C.c_double()
        zi = np.zeros(8, dtype=np.int32)
        self.L.orc_grid_info(self.ctx, C.byref(b3), _i(zi))
        return b3.value, zi

    def wall_ghost_2d(self, cx, cy, side):
        out = np.zeros(self.nv)
        bad = self.L.orc_wall_ghost_2d(self.ctx, cx, cy, side, _d(out))
        return out, bad

    def cell_cdf_vr(self, cell):
        n = self.nv + 1
        ce, cd, kin = np.zeros(n), np.zeros(n), np.zeros(n)
        re, rd = np.zeros(2000, np.int32), np.zeros(2000, np.int32)
        self.L.orc_cell_cdf_vr(self.ctx, cell, _d(ce), _d(cd), _d(kin), _i(re), _i(rd))
        return ce, cd, kin, re.reshape(1000, 2), rd.reshape(1000, 2)


def remap(grid, u, v, w, f_off=1.0):
    """compute_remapping_quantities on a grid: (stencil[7], mass[7], status)."""
    st = np.zeros(7, dtype=np.int32)
    ms = np.zeros(7)
    vg = pkg.make_vgrid(grid)
    r = lib().orc_remap_grid(C.byref(vg), u, v, w, f_off, _i(st), _d(ms))
    return st, ms, r


def center_of_mass_velocity(x, y, z, mass):
    x, y, z, m = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z, mass))
    out = np.zeros(3)
    lib().orc_center_of_mass_velocity(_d(x), _d(y), _d(z), _d(m), _d(out))
    return out


def philox4x32_10(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return list(o)


def philox_uniform2(seed, sample, cell, step, sub, call):
    out = np.zeros(2)
    lib().orc_philox_uniform2(seed, sample, cell, step, sub, call, _d(out))
    return out


def build_ref_table(cum):
    cum = np.ascontiguousarray(cum, dtype=np.float64)
    ref = np.zeros(2000, dtype=np.int32)
    lib().orc_build_ref_table(_d(cum), len(cum) - 1, _i(ref))
    return ref.reshape(1000, 2)


def referenced_search(cum, ref, R):
    cum = np.ascontiguousarray(cum, dtype=np.float64)
    ref = np.ascontiguousarray(ref, dtype=np.int32).reshape(-1)
    return int(lib().orc_referenced_search(_d(cum), _i(ref), len(cum) - 1, R))
