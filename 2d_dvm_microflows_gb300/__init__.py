"""GB300 (sm_103a) DVM time step behind a C ABI, and a Python host that drives it.

The package loads libdvm_gpu.so (built in-tree by build.py) through ctypes; there is no
CPU fallback: without the library every call raises. `DVMSolver` mirrors the reference
driver's time step (solver/dvm_solver.f90:231-369 in aarthisekaran11/2D_DVM_microflows):
compute_collision_integral, compute_convection (with the boundary conditions) and
calculate_physical_properties, with the reference's input-deck parameter names.
"""
import ctypes as C
import dataclasses
import os

import numpy as np

from . import _abi
from ._abi import *  # noqa: F401,F403  (constants and structs of include/dvm_gpu.h)
from . import physics

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdvm_gpu.so")

_LIB = None


class DVMError(RuntimeError):
    """A non-zero status from the C ABI (the reference prints and stops on these)."""

    def __init__(self, status, where):
        self.status = status
        msg = _LIB.dvm_strerror(status).decode() if _LIB is not None else str(status)
        super().__init__("%s: %s (status %d)" % (where, msg, status))


def load_library(path=None):
    """Loads the GPU library; raises if it is missing (no fallback path exists)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libdvm_gpu.so is not built (%s); run "
                           "`python 2d_dvm_microflows_gb300/build.py`" % p)
    lib = _abi.bind(C.CDLL(p))
    if lib.dvm_abi_version() != _abi.DVM_ABI_VERSION:
        raise RuntimeError("ABI version mismatch")
    if path is None:
        _LIB = lib
    return lib


def _check(st, where):
    if st != DVM_OK:
        raise DVMError(st, where)


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


@dataclasses.dataclass
class DVMConfig:
    """Input-deck keys of the time step (input_output/read_input_2D.f90:75-777)."""
    geometry: int = DVM_GEOM_0D
    nx_space: int = 1
    ny_space: int = 1
    dx: float = 1.0
    dy: float = 1.0
    deltat: float = 0.01
    Kn: float = 1.0
    mass: float = 1.0
    omega: float = 0.5
    alpha: float = 1.0
    sigma: float = 1.0
    iColl: int = DVM_COLL_VR
    iConv: int = DVM_CONV_NONE
    ColnRMS: float = 0.001
    NRepl: int = 1
    cdf_tolerance: float = 0.01
    samples_mode: int = DVM_SAMPLES_FORMULA
    samples_per_step: int = 0
    bc: tuple = (DVM_BC2D_WALL, DVM_BC2D_WALL, DVM_BC2D_WALL, DVM_BC2D_WALL)
    acc_coeff: float = 1.0
    # per wall (left, right, bottom, top): density, u, v, w, temperature
    walls: tuple = ((1.0, 0.0, 0.0, 0.0, 1.0),) * 4
    pi_mode: int = DVM_PI_REFERENCE
    seed: int = 0
    precision: int = DVM_PREC_FP64

    def to_params(self):
        p = dvm_params()
        p.geometry = self.geometry
        p.nx_space, p.ny_space = self.nx_space, self.ny_space
        p.coll_method, p.conv_method = self.iColl, self.iConv
        p.num_repl = self.NRepl
        p.samples_mode = self.samples_mode
        p.pi_mode = self.pi_mode
        for i in range(4):
            p.bc[i] = int(self.bc[i])
            for q in range(5):
                p.wall[i][q] = float(self.walls[i][q])
        p.samples_per_step = int(self.samples_per_step)
        p.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        p.dx, p.dy, p.dt, p.Kn = self.dx, self.dy, self.deltat, self.Kn
        p.mass, p.omega, p.alpha, p.sigma = self.mass, self.omega, self.alpha, self.sigma
        p.coln_rms, p.cdf_tolerance = self.ColnRMS, self.cdf_tolerance
        p.acc_coeff = self.acc_coeff
        p.precision = self.precision
        return p


def make_vgrid(grid):
    """dvm_vgrid view of a physics.VelocityGrid (the arrays must outlive the call)."""
    vg = dvm_vgrid()
    vg.nx, vg.ny, vg.nz = grid.nx, grid.ny, grid.nz
    vg.x, vg.y, vg.z = _dptr(grid.x), _dptr(grid.y), _dptr(grid.z)
    return vg


class PairList:
    """A recorded collision list (dvm_pairlist) built from numpy arrays.

    subs[q] = dict(glA=int32[n] or None, glB=..., rA=float64[n] or None, rB=...,
                   r_phi=float64[n*NRepl], r_cos=float64[n*NRepl])
    """

    def __init__(self, subs):
        self._keep = []
        self.s = dvm_pairlist()
        for q in range(3):
            d = subs[q] if q < len(subs) else None
            if d is None:
                self.s.count[q] = 0
                continue
            n = len(d["r_phi"]) // max(1, d.get("num_repl", 1))
            n = int(d.get("count", n))
            self.s.count[q] = n
            for key, conv, dt in (("glA", _iptr, np.int32), ("glB", _iptr, np.int32),
                                  ("rA", _dptr, np.float64), ("rB", _dptr, np.float64),
                                  ("r_phi", _dptr, np.float64), ("r_cos", _dptr, np.float64)):
                arr = d.get(key)
                if arr is None:
                    continue
                arr = np.ascontiguousarray(arr, dtype=dt)
                self._keep.append(arr)
                getattr(self.s, key)[q] = conv(arr)

    def ref(self):
        return C.byref(self.s)


class DVMSolver:
    """Host mirror of the reference time step, running on the GPU through the C ABI."""

    def __init__(self, config, grid, lib=None):
        self.lib = lib or load_library()
        self.config = config
        self.grid = grid
        self._params = config.to_params()
        vg = make_vgrid(grid)
        ctx = C.c_void_p()
        _check(self.lib.dvm_create(C.byref(self._params), C.byref(vg), C.byref(ctx)), "dvm_create")
        self.ctx = ctx
        self.ncells = config.nx_space * config.ny_space
        self.nv = grid.nv
        self.ntime = 0

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.dvm_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- state ---------------------------------------------------------------------------
    def initialize_dist_func(self, f):
        """Uploads f[cells, nv] (phi and delta_phi) and computes its properties."""
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(self.ncells, self.nv)
        _check(self.lib.dvm_upload_f(self.ctx, _dptr(f)), "dvm_upload_f")

    def phi(self):
        out = np.empty((self.ncells, self.nv))
        _check(self.lib.dvm_download_f(self.ctx, _dptr(out)), "dvm_download_f")
        return out

    def properties(self):
        out = np.empty((self.ncells, DVM_NPROP))
        _check(self.lib.dvm_get_properties(self.ctx, _dptr(out)), "dvm_get_properties")
        return out

    def set_properties(self, props):
        props = np.ascontiguousarray(props, dtype=np.float64).reshape(self.ncells, DVM_NPROP)
        _check(self.lib.dvm_set_properties(self.ctx, _dptr(props)), "dvm_set_properties")

    # -- the time step -------------------------------------------------------------------
    def compute_collision_integral(self, step=None, pairs=None):
        step = self.ntime if step is None else step
        ref = pairs.ref() if pairs is not None else None
        _check(self.lib.dvm_compute_collision_integral(self.ctx, C.c_uint64(step), ref),
               "dvm_compute_collision_integral")

    def compute_convection(self):
        _check(self.lib.dvm_compute_convection(self.ctx), "dvm_compute_convection")

    def calculate_physical_properties(self):
        _check(self.lib.dvm_calculate_physical_properties(self.ctx),
               "dvm_calculate_physical_properties")

    def solve(self, nsteps):
        """nsteps iterations of solve()'s loop (dvm_solver.f90:299-357)."""
        _check(self.lib.dvm_step(self.ctx, C.c_uint64(self.ntime), int(nsteps)), "dvm_step")
        self.ntime += nsteps

    def step_host(self, f_in, nsteps=1, f_out=None):
        """dvm_step_host: f_in (host, [cells, nv]) in, nsteps steps, f out (into f_out, which
        may be f_in itself; a new array if None). Page-locked buffers move by the kernels."""
        f_in = np.ascontiguousarray(f_in, dtype=np.float64)
        if f_out is None:
            f_out = np.empty_like(f_in)
        if f_out.dtype != np.float64 or not f_out.flags["C_CONTIGUOUS"]:
            raise ValueError("f_out must be a contiguous float64 array")
        _check(self.lib.dvm_step_host(self.ctx, C.c_uint64(self.ntime), int(nsteps),
                                      _dptr(f_in), _dptr(f_out)), "dvm_step_host")
        self.ntime += nsteps
        return f_out

    def collision_count(self):
        v = C.c_int64()
        _check(self.lib.dvm_last_collision_count(self.ctx, C.byref(v)), "dvm_last_collision_count")
        return v.value

    def scatter_count(self):
        """Adds into f counted by the last collision launch (dvm_last_scatter_count)."""
        v = C.c_int64()
        _check(self.lib.dvm_last_scatter_count(self.ctx, C.byref(v)), "dvm_last_scatter_count")
        return v.value

    def error_word(self):
        v = C.c_uint32()
        _check(self.lib.dvm_get_error_word(self.ctx, C.byref(v)), "dvm_get_error_word")
        return v.value

    def synchronize(self):
        _check(self.lib.dvm_synchronize(self.ctx), "dvm_synchronize")

    def checkpoint(self):
        """The context's state as bytes (restart.f90's ntime + phi, plus the cached
        equilibrium the next step may reuse)."""
        n = C.c_uint64()
        _check(self.lib.dvm_checkpoint_size(self.ctx, C.byref(n)), "dvm_checkpoint_size")
        buf = C.create_string_buffer(n.value)
        _check(self.lib.dvm_checkpoint_save(self.ctx, C.c_uint64(self.ntime), buf, n.value),
               "dvm_checkpoint_save")
        return buf.raw

    def restore(self, data):
        """Loads a checkpoint of a context of the same shape; the run continues from it."""
        buf = C.create_string_buffer(bytes(data), len(data))
        nt = C.c_uint64()
        _check(self.lib.dvm_checkpoint_load(self.ctx, buf, len(data), C.byref(nt)),
               "dvm_checkpoint_load")
        self.ntime = nt.value

    def residual(self):
        """Largest relative change of the moments in the last step (dvm_get_residual)."""
        v = C.c_double()
        _check(self.lib.dvm_get_residual(self.ctx, C.byref(v)), "dvm_get_residual")
        return v.value

    # -- instrumentation -----------------------------------------------------------------
    def profile(self, enable=True):
        _check(self.lib.dvm_profile_enable(self.ctx, int(enable)), "dvm_profile_enable")

    def profile_reset(self):
        _check(self.lib.dvm_profile_reset(self.ctx), "dvm_profile_reset")

    def profile_read(self):
        out = {}
        for k in range(DVM_K_COUNT):
            ms, n = C.c_double(), C.c_int64()
            _check(self.lib.dvm_profile_read(self.ctx, k, C.byref(ms), C.byref(n)),
                   "dvm_profile_read")
            out[KERNEL_NAMES[k]] = (ms.value, n.value)
        return out

    def launch_count(self):
        v = C.c_int64()
        _check(self.lib.dvm_launch_count(self.ctx, C.byref(v)), "dvm_launch_count")
        return v.value

    def time_steps(self, nsteps):
        ms = C.c_double()
        _check(self.lib.dvm_time_steps(self.ctx, C.c_uint64(self.ntime), int(nsteps),
                                       C.byref(ms)), "dvm_time_steps")
        self.ntime += nsteps
        return ms.value

    def flush_l2(self):
        _check(self.lib.dvm_flush_l2(self.ctx), "dvm_flush_l2")

    def atomic_rate(self, window_bytes):
        """Measured FP64 atomic adds per second over a window of device memory."""
        v = C.c_double()
        _check(self.lib.dvm_atomic_rate(self.ctx, C.c_uint64(int(window_bytes)), C.byref(v)),
               "dvm_atomic_rate")
        return v.value


class DVMBatch:
    """Many independent solves stepped together (dvm_batch_*): 0-D relaxations, or 1-D
    instances of config.nx_space cells sharing the config's end conditions. Instances on the
    same velocity grid share one context, one step of all of them is one CUDA-graph replay
    (one launch of each kernel over all grids), and the launch shape is autotuned."""

    def __init__(self, config, grids, instance_grid, samples_per_grid, lib=None):
        self.lib = lib or load_library()
        self.config = config
        self.grids = list(grids)
        self.instance_grid = np.ascontiguousarray(instance_grid, dtype=np.int32)
        self.samples = np.ascontiguousarray(samples_per_grid, dtype=np.int64)
        if len(self.samples) != len(self.grids):
            raise ValueError("one sample count per grid")
        self._params = config.to_params()
        vgs = (dvm_vgrid * len(self.grids))()
        for i, g in enumerate(self.grids):
            vgs[i] = make_vgrid(g)
        b = C.c_void_p()
        _check(self.lib.dvm_batch_create(
            C.byref(self._params), vgs, len(self.grids),
            self.instance_grid.ctypes.data_as(C.POINTER(C.c_int32)), len(self.instance_grid),
            self.samples.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(b)), "dvm_batch_create")
        self.b = b
        self.ninstances = len(self.instance_grid)
        self.cells = config.nx_space if config.geometry == DVM_GEOM_1D else 1

    def close(self):
        if getattr(self, "b", None):
            self.lib.dvm_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload_f(self, instance, f):
        g = self.grids[self.instance_grid[instance]]
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(self.cells * g.nv)
        _check(self.lib.dvm_batch_upload_f(self.b, int(instance), _dptr(f)), "dvm_batch_upload_f")

    def download_f(self, instance):
        """f of one instance: [nv] (0-D) or [cells, nv] (1-D)."""
        g = self.grids[self.instance_grid[instance]]
        out = np.empty((self.cells, g.nv)) if self.cells > 1 else np.empty(g.nv)
        _check(self.lib.dvm_batch_download_f(self.b, int(instance), _dptr(out)),
               "dvm_batch_download_f")
        return out

    def step(self, nsteps=1):
        _check(self.lib.dvm_batch_step(self.b, int(nsteps)), "dvm_batch_step")

    def properties(self):
        """[instances, DVM_NPROP] (0-D) or [instances, cells, DVM_NPROP] (1-D)."""
        out = np.empty((self.ninstances, self.cells, DVM_NPROP))
        _check(self.lib.dvm_batch_get_properties(self.b, _dptr(out)), "dvm_batch_get_properties")
        return out if self.cells > 1 else out[:, 0, :]

    def time_steps(self, nsteps):
        ms, n = C.c_double(), C.c_int64()
        _check(self.lib.dvm_batch_time_steps(self.b, int(nsteps), C.byref(ms), C.byref(n)),
               "dvm_batch_time_steps")
        return ms.value, n.value

    def launch_shape(self):
        """The autotuned shape: CDF threads per CTA, collision CTAs per SM, launches per step."""
        t, b, n = C.c_int(), C.c_int(), C.c_int()
        _check(self.lib.dvm_batch_launch_shape(self.b, C.byref(t), C.byref(b), C.byref(n)),
               "dvm_batch_launch_shape")
        return {"cdf_threads": t.value, "collide_ctas_per_sm": b.value,
                "launches_per_step": n.value}


def footprint_bytes(config, grid, lib=None):
    """Device bytes a context for (config, grid) allocates (dvm_footprint_bytes)."""
    lib = lib or load_library()
    p = config.to_params()
    vg = make_vgrid(grid)
    v = C.c_uint64()
    _check(lib.dvm_footprint_bytes(C.byref(p), C.byref(vg), C.byref(v)), "dvm_footprint_bytes")
    return v.value


class DVMServer:
    """Continuous-batching request server (dvm_server_*): submit solves of any geometry and
    grid; native host threads admit them by HBM footprint, keep their state on the
    device and advance them concurrently until each reaches its residual or step limit."""

    def __init__(self, hbm_budget_bytes, max_active=16, steps_per_turn=2, preempt_turns=0,
                 lib=None):
        self.lib = lib or load_library()
        sv = C.c_void_p()
        _check(self.lib.dvm_server_create(C.c_uint64(int(hbm_budget_bytes)), int(max_active),
                                          int(steps_per_turn), C.byref(sv)), "dvm_server_create")
        self.sv = sv
        self._shape = {}
        if preempt_turns:
            _check(self.lib.dvm_server_set_preemption(self.sv, int(preempt_turns)),
                   "dvm_server_set_preemption")

    def close(self):
        if getattr(self, "sv", None):
            self.lib.dvm_server_destroy(self.sv)
            self.sv = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, config, grid, f0, max_steps, residual_tol=0.0):
        p = config.to_params()
        vg = make_vgrid(grid)
        cells = config.nx_space * config.ny_space
        f0 = np.ascontiguousarray(f0, dtype=np.float64).reshape(cells, grid.nv)
        rid = C.c_int64()
        _check(self.lib.dvm_server_submit(self.sv, C.byref(p), C.byref(vg), _dptr(f0),
                                          int(max_steps), float(residual_tol), C.byref(rid)),
               "dvm_server_submit")
        self._shape[rid.value] = (cells, grid.nv)
        return rid.value

    def wait(self, rid):
        info = dvm_request_info()
        _check(self.lib.dvm_server_wait(self.sv, C.c_int64(rid), C.byref(info)), "dvm_server_wait")
        return {k: getattr(info, k) for k, _ in dvm_request_info._fields_}

    def result(self, rid):
        """(properties[cells, DVM_NPROP], f[cells, nv]) of a finished request."""
        cells, nv = self._shape.pop(rid)
        props = np.empty((cells, DVM_NPROP))
        f = np.empty((cells, nv))
        _check(self.lib.dvm_server_result(self.sv, C.c_int64(rid), _dptr(props), _dptr(f)),
               "dvm_server_result")
        return props, f

    def stats(self):
        n, a, b = C.c_int64(), C.c_int32(), C.c_uint64()
        _check(self.lib.dvm_server_stats(self.sv, C.byref(n), C.byref(a), C.byref(b)),
               "dvm_server_stats")
        return {"completed": n.value, "peak_active": a.value, "peak_bytes": b.value}


# Tecplot output: the reference's visualization module (input_output/visualization.f90),
# written by the library's host code (dvm_vis_* in the C ABI) so that this host and the
# C++ one write the same bytes.
VIS_PROPERTY_KEYS = ("write_dens", "write_x_vel", "write_y_vel", "write_z_vel", "write_speed",
                     "write_mach", "write_tr_temp", "write_rot_temp", "write_vib_temp",
                     "write_tot_temp", "write_temp_x", "write_temp_y", "write_temp_z",
                     "write_tr_energy", "write_rot_energy", "write_vib_energy",
                     "write_tot_energy", "write_entropy", "write_heat_flux_x",
                     "write_heat_flux_y", "write_heat_flux_z", "write_rot_dof",
                     "write_vib_dof", "write_rot_temp_relax", "write_vib_temp_relax",
                     "write_kin_temp_relax", "write_pressure")


class TecplotOutput:
    """The reference's output files for one monatomic species: `write_headers`, then
    `write_properties` and `write_df` at each output time (write_vis_data,
    visualization.f90:870-918, calls them at ntime % dump_freq == 0 and at the last step).

    `properties` holds the deck's write_* flags by name (VIS_PROPERTY_KEYS, the order of the
    reference's property_names); `stress` the stress_directions (11, 22, 33, 12, 13, 23);
    `moments` the moment_numbers (written to the species file, zero in the mixture file);
    `df_locations` the 1-based (x, y) cells of the distribution-function files."""

    def __init__(self, nx_space, ny_space, dx, dy, mass=1.0, omega=0.5, end_time=0,
                 properties_filename=None, properties=(), properties_dump_freq=1,
                 stress=(), moments=(), df_filename=None, df_locations=(), df_dimension=1,
                 enable_vel_df=True, rot_levels=0, vib_levels=0, pi_mode=DVM_PI_REFERENCE,
                 right_wall_dens=1.0, cZr=0.0, cZv=0.0, right_wall_temp_rot=0.0,
                 right_wall_temp_vib=0.0, lib=None):
        self.lib = lib or load_library()
        v = dvm_vis()
        if properties_filename:
            v.properties_filename = properties_filename.encode()
            v.enable_properties = 1
        for key in properties:
            v.properties_to_output[VIS_PROPERTY_KEYS.index(key)] = 1
        if len(stress) > 6:
            raise ValueError("at most six stress components")
        v.write_stress = len(stress)
        for i, d in enumerate(stress):
            v.stress_directions[i] = int(d)
        if len(moments) > 6:
            raise ValueError("at most six moment columns")
        v.write_moment = len(moments)
        for i, d in enumerate(moments):
            v.moment_numbers[i] = int(d)
        v.nx_space, v.ny_space, v.dx, v.dy = nx_space, ny_space, dx, dy
        v.end_time, v.properties_dump_freq = int(end_time), int(properties_dump_freq)
        if df_filename:
            if not 1 <= len(df_locations) <= 16:
                raise ValueError("1 to 16 distribution-function locations")
            v.df_filename = df_filename.encode()
            v.enable_vel_df = 1 if enable_vel_df else 0
            v.enable_rot_df = 1 if rot_levels else 0
            v.enable_vib_df = 1 if vib_levels else 0
            v.df_dimension = int(df_dimension)
            v.num_locations = len(df_locations)
            for i, (x, y) in enumerate(df_locations):
                v.x_locations[i], v.y_locations[i] = int(x), int(y)
        v.rot_levels, v.vib_levels, v.pi_mode = int(rot_levels), int(vib_levels), int(pi_mode)
        v.mass, v.omega, v.cZr, v.cZv = mass, omega, cZr, cZv
        v.right_wall_dens = right_wall_dens
        v.right_wall_temp_rot, v.right_wall_temp_vib = right_wall_temp_rot, right_wall_temp_vib
        self.vis = v

    def write_headers(self):
        _check(self.lib.dvm_vis_write_headers(C.byref(self.vis)), "dvm_vis_write_headers")

    def write_properties(self, time, props=None, f=None, grid=None):
        """props[cells, DVM_NPROP] (device moments) and/or f[cells, Nv]; with f every column
        is formed from it the way the reference forms it."""
        pp = fp = None
        keep = []
        if props is not None:
            props = np.ascontiguousarray(props, dtype=np.float64)
            keep.append(props)
            pp = _dptr(props)
        vg = None
        if f is not None:
            f = np.ascontiguousarray(f, dtype=np.float64)
            keep.append(f)
            fp = _dptr(f)
            vg = C.byref(make_vgrid(grid))
        _check(self.lib.dvm_vis_write_properties(C.byref(self.vis), float(time), pp, fp, vg),
               "dvm_vis_write_properties")

    def write_df(self, time, f, grid):
        f = np.ascontiguousarray(f, dtype=np.float64)
        _check(self.lib.dvm_vis_write_df(C.byref(self.vis), float(time), _dptr(f),
                                         C.byref(make_vgrid(grid))), "dvm_vis_write_df")


def fortran_e(x, w, d, lib=None):
    """One Ew.d field as the reference's format statements write it."""
    lib = lib or load_library()
    buf = C.create_string_buffer(w + 1)
    _check(lib.dvm_vis_format_e(float(x), w, d, buf, w + 1), "dvm_vis_format_e")
    return buf.value.decode()
