"""ctypes mirror of include/dvm_gpu.h (the C ABI of the GPU time step).

The structs and constants here must match the header field for field; tests check the
sizes against the compiled library (dvm_abi_version) and the header text.
"""
import ctypes as C

DVM_ABI_VERSION = 2

# status codes
DVM_OK, DVM_ERR_PARAM, DVM_ERR_OOM, DVM_ERR_CUDA, DVM_ERR_NUMERIC, DVM_ERR_TIMEOUT, \
    DVM_ERR_NODEVICE, DVM_ERR_TOO_LARGE, DVM_ERR_IO = range(9)

# device error word bits
DVM_EW_SEARCH, DVM_EW_REMAP, DVM_EW_NONFINITE, DVM_EW_NEGDENS, DVM_EW_WAIT = 1, 2, 4, 8, 16

# iColl / iConv / geometry
DVM_COLL_NONE, DVM_COLL_FMC, DVM_COLL_VR = 0, 2, 3
DVM_CONV_NONE, DVM_CONV_UPWIND1 = 0, 1
DVM_GEOM_0D, DVM_GEOM_1D, DVM_GEOM_2D = 0, 1, 2
# 2-D wall numbering (trunk) and 1-D end numbering (grid_ref)
DVM_BC2D_WALL, DVM_BC2D_INOUT, DVM_BC2D_ZEROGRAD, DVM_BC2D_COUETTE = 1, 2, 3, 4
DVM_BC1D_SPECULAR, DVM_BC1D_DIFFUSE, DVM_BC1D_INOUT, DVM_BC1D_ZEROGRAD = 1, 2, 3, 4
DVM_PI_REFERENCE, DVM_PI_EXACT = 0, 1
DVM_SAMPLES_FORMULA, DVM_SAMPLES_FIXED = 0, 1
DVM_PREC_FP64, DVM_PREC_FP32 = 0, 1
DVM_WALL_LEFT, DVM_WALL_RIGHT, DVM_WALL_BOTTOM, DVM_WALL_TOP = 0, 1, 2, 3
DVM_WP_DENS, DVM_WP_U, DVM_WP_V, DVM_WP_W, DVM_WP_TEMP = 0, 1, 2, 3, 4

# property record
PROP_NAMES = ["dens", "u", "v", "w", "temp", "species_temp", "avg_speed", "pressure",
              "qx", "qy", "qz", "txx", "tyy", "tzz", "txy", "txz", "tyz"]
DVM_P = {n: i for i, n in enumerate(PROP_NAMES)}
(DVM_P_DENS, DVM_P_U, DVM_P_V, DVM_P_W, DVM_P_TEMP, DVM_P_SPECIES_TEMP, DVM_P_AVG_SPEED,
 DVM_P_PRESSURE, DVM_P_QX, DVM_P_QY, DVM_P_QZ, DVM_P_TXX, DVM_P_TYY, DVM_P_TZZ, DVM_P_TXY,
 DVM_P_TXZ, DVM_P_TYZ) = range(17)
DVM_NPROP = 20

# kernel ids for instrumentation
KERNEL_NAMES = ["cdf_build", "collide_plan", "collide", "wall_flux", "wall_ghost",
                "convect", "bc_1d", "moments", "project"]
DVM_K_COUNT = len(KERNEL_NAMES)


class dvm_vgrid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("x", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)),
                ("z", C.POINTER(C.c_double))]


class dvm_params(C.Structure):
    _fields_ = [("geometry", C.c_int32), ("nx_space", C.c_int32), ("ny_space", C.c_int32),
                ("coll_method", C.c_int32), ("conv_method", C.c_int32),
                ("num_repl", C.c_int32), ("samples_mode", C.c_int32), ("pi_mode", C.c_int32),
                ("bc", C.c_int32 * 4), ("samples_per_step", C.c_int64), ("seed", C.c_uint64),
                ("dx", C.c_double), ("dy", C.c_double), ("dt", C.c_double),
                ("Kn", C.c_double), ("mass", C.c_double), ("omega", C.c_double),
                ("alpha", C.c_double), ("sigma", C.c_double), ("coln_rms", C.c_double),
                ("cdf_tolerance", C.c_double), ("acc_coeff", C.c_double),
                ("wall", (C.c_double * 5) * 4), ("precision", C.c_int32),
                ("reserved", C.c_int32)]


class dvm_pairlist(C.Structure):
    _fields_ = [("count", C.c_int64 * 3),
                ("glA", C.POINTER(C.c_int32) * 3), ("glB", C.POINTER(C.c_int32) * 3),
                ("rA", C.POINTER(C.c_double) * 3), ("rB", C.POINTER(C.c_double) * 3),
                ("r_phi", C.POINTER(C.c_double) * 3), ("r_cos", C.POINTER(C.c_double) * 3)]


class dvm_request_info(C.Structure):
    _fields_ = [("status", C.c_int32), ("converged", C.c_int32), ("steps", C.c_int32),
                ("preempted", C.c_int32), ("residual", C.c_double), ("queue_ms", C.c_double),
                ("latency_ms", C.c_double), ("collisions", C.c_int64),
                ("device_bytes", C.c_uint64)]


# Tecplot output settings (visualization.f90); see dvm_vis in the header
DVM_VIS_NPROP = 27
DVM_VIS_DF_1D, DVM_VIS_DF_2D, DVM_VIS_DF_3D = 1, 2, 3


class dvm_vis(C.Structure):
    _fields_ = [("properties_filename", C.c_char * 128), ("df_filename", C.c_char * 128),
                ("enable_properties", C.c_int32),
                ("properties_to_output", C.c_int32 * DVM_VIS_NPROP),
                ("write_stress", C.c_int32), ("stress_directions", C.c_int32 * 6),
                ("write_moment", C.c_int32), ("moment_numbers", C.c_int32 * 6),
                ("nx_space", C.c_int32), ("ny_space", C.c_int32),
                ("dx", C.c_double), ("dy", C.c_double),
                ("end_time", C.c_int32), ("properties_dump_freq", C.c_int32),
                ("enable_vel_df", C.c_int32), ("enable_rot_df", C.c_int32),
                ("enable_vib_df", C.c_int32), ("df_dimension", C.c_int32),
                ("num_locations", C.c_int32), ("x_locations", C.c_int32 * 16),
                ("y_locations", C.c_int32 * 16), ("rot_levels", C.c_int32),
                ("vib_levels", C.c_int32), ("pi_mode", C.c_int32),
                ("mass", C.c_double), ("omega", C.c_double),
                ("cZr", C.c_double), ("cZv", C.c_double), ("right_wall_dens", C.c_double),
                ("right_wall_temp_rot", C.c_double), ("right_wall_temp_vib", C.c_double)]


# Entry points declared in include/dvm_gpu.h: name -> (restype, argtypes)
_P = C.c_void_p
ENTRY_POINTS = {
    "dvm_create": (C.c_int, [C.POINTER(dvm_params), C.POINTER(dvm_vgrid), C.POINTER(_P)]),
    "dvm_destroy": (C.c_int, [_P]),
    "dvm_strerror": (C.c_char_p, [C.c_int]),
    "dvm_abi_version": (C.c_int, []),
    "dvm_upload_f": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "dvm_download_f": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "dvm_num_velocity_points": (C.c_int, [_P]),
    "dvm_num_cells": (C.c_int, [_P]),
    "dvm_compute_collision_integral": (C.c_int, [_P, C.c_uint64, C.POINTER(dvm_pairlist)]),
    "dvm_compute_convection": (C.c_int, [_P]),
    "dvm_calculate_physical_properties": (C.c_int, [_P]),
    "dvm_get_properties": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "dvm_set_properties": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "dvm_step": (C.c_int, [_P, C.c_uint64, C.c_int]),
    "dvm_last_collision_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "dvm_last_scatter_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "dvm_synchronize": (C.c_int, [_P]),
    "dvm_get_error_word": (C.c_int, [_P, C.POINTER(C.c_uint32)]),
    "dvm_profile_enable": (C.c_int, [_P, C.c_int]),
    "dvm_kernel_name": (C.c_char_p, [C.c_int]),
    "dvm_profile_read": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "dvm_profile_reset": (C.c_int, [_P]),
    "dvm_launch_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "dvm_time_steps": (C.c_int, [_P, C.c_uint64, C.c_int, C.POINTER(C.c_double)]),
    "dvm_flush_l2": (C.c_int, [_P]),
    "dvm_get_residual": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "dvm_wait_selftest": (C.c_int, [_P]),
    "dvm_atomic_rate": (C.c_int, [_P, C.c_uint64, C.POINTER(C.c_double)]),
    "dvm_checkpoint_size": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "dvm_checkpoint_save": (C.c_int, [_P, C.c_uint64, C.c_void_p, C.c_uint64]),
    "dvm_checkpoint_load": (C.c_int, [_P, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "dvm_step_host": (C.c_int, [_P, C.c_uint64, C.c_int, C.POINTER(C.c_double),
                                C.POINTER(C.c_double)]),
    "dvm_batch_create": (C.c_int, [C.POINTER(dvm_params), C.POINTER(dvm_vgrid), C.c_int,
                                   C.POINTER(C.c_int32), C.c_int, C.POINTER(C.c_int64),
                                   C.POINTER(_P)]),
    "dvm_batch_destroy": (C.c_int, [_P]),
    "dvm_batch_upload_f": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double)]),
    "dvm_batch_download_f": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double)]),
    "dvm_batch_step": (C.c_int, [_P, C.c_int]),
    "dvm_batch_get_properties": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "dvm_batch_time_steps": (C.c_int, [_P, C.c_int, C.POINTER(C.c_double),
                                       C.POINTER(C.c_int64)]),
    "dvm_batch_launch_shape": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                         C.POINTER(C.c_int)]),
    "dvm_footprint_bytes": (C.c_int, [C.POINTER(dvm_params), C.POINTER(dvm_vgrid),
                                      C.POINTER(C.c_uint64)]),
    "dvm_server_create": (C.c_int, [C.c_uint64, C.c_int, C.c_int, C.POINTER(_P)]),
    "dvm_server_destroy": (C.c_int, [_P]),
    "dvm_server_submit": (C.c_int, [_P, C.POINTER(dvm_params), C.POINTER(dvm_vgrid),
                                    C.POINTER(C.c_double), C.c_int32, C.c_double,
                                    C.POINTER(C.c_int64)]),
    "dvm_server_wait": (C.c_int, [_P, C.c_int64, C.POINTER(dvm_request_info)]),
    "dvm_server_result": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_double),
                                    C.POINTER(C.c_double)]),
    "dvm_server_stats": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                   C.POINTER(C.c_uint64)]),
    "dvm_server_set_preemption": (C.c_int, [_P, C.c_int32]),
    "dvm_collide_noalloc": (C.c_int, [C.POINTER(dvm_params), C.POINTER(dvm_vgrid), _P, _P,
                                      C.c_int, C.c_uint64, _P, C.POINTER(C.c_int64)]),
    "dvm_vis_write_headers": (C.c_int, [C.POINTER(dvm_vis)]),
    "dvm_vis_write_properties": (C.c_int, [C.POINTER(dvm_vis), C.c_double,
                                           C.POINTER(C.c_double), C.POINTER(C.c_double),
                                           C.POINTER(dvm_vgrid)]),
    "dvm_vis_write_df": (C.c_int, [C.POINTER(dvm_vis), C.c_double, C.POINTER(C.c_double),
                                   C.POINTER(dvm_vgrid)]),
    "dvm_vis_format_e": (C.c_int, [C.c_double, C.c_int, C.c_int, C.c_char_p, C.c_int]),
}


def bind(lib):
    """Attach restype/argtypes for every entry point to a loaded CDLL."""
    for name, (res, args) in ENTRY_POINTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
