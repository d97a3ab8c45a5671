"""Loads libsif_gb300.so (built in-tree by sif_gb300/build.py) and declares
its C signatures (include/sif_gb300.h). There is no fallback: a missing
library is an ImportError-like failure the caller sees.
"""
import ctypes as C
import os

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsif_gb300.so")

class DeviceMesh(C.Structure):
    """sifg_device_mesh_t: a chain mesh's device columns."""
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("offsets", C.c_void_p), ("w", C.c_void_p), ("cell_w", C.c_void_p),
                ("total_weight", C.c_double), ("n_particles", C.c_uint64),
                ("n_cells", C.c_uint32)]


_lib = None


class RungStat(C.Structure):
    _fields_ = [("radius", C.c_float), ("r_search", C.c_float),
                ("n_candidates", C.c_uint64), ("n_survivors", C.c_uint64),
                ("n_accepted", C.c_uint64), ("rounds", C.c_uint64),
                ("n_rescale_fail", C.c_uint64), ("n_overflow", C.c_uint64),
                ("rung_ms", C.c_double), ("count_wait_ms", C.c_double),
                ("sort_ms", C.c_double), ("commit_ms", C.c_double),
                ("growth_particles", C.c_uint64), ("growth_cells", C.c_uint64),
                ("cand_wait_ms", C.c_double), ("from_list", C.c_uint64),
                ("n_witness", C.c_uint64), ("n_displaced", C.c_uint64)]


class Timings(C.Structure):
    _fields_ = [("wall_ms", C.c_double), ("growth_ms", C.c_double), ("growth_launches", C.c_int),
                ("filter_ms", C.c_double), ("filter_launches", C.c_int),
                ("cic_ms", C.c_double), ("cic_launches", C.c_int),
                ("mesh_ms", C.c_double), ("mesh_launches", C.c_int),
                ("growth_particles", C.c_uint64), ("growth_cells", C.c_uint64),
                ("witness_ms", C.c_double), ("witness_launches", C.c_int),
                ("commit_ms", C.c_double), ("commit_launches", C.c_int),
                ("cic_stage_ms", C.c_double)]


class TraceEvent(C.Structure):
    """sifg_trace_event_t: one span of the last run's timeline."""
    _fields_ = [("kind", C.c_int32), ("start_ms", C.c_float), ("end_ms", C.c_float)]


EXPORTED = [
    # sif's API
    "sif_system_init", "sif_system_finalise", "sif_error_message", "sif_error_status",
    "sif_field_alloc", "sif_field_free", "sif_field_assign_positions",
    "sif_field_assign_weights", "sif_field_reserve_weights",
    "sif_grid_alloc", "sif_grid_free", "sif_grid_assign_cic", "sif_grid_to_density_contrast",
    "sif_chain_mesh_alloc", "sif_chain_mesh_alloc_consume", "sif_chain_mesh_free",
    "sif_catalogue_free", "sif_finder_exodus_preset", "sif_finder_exodus_variant_name",
    "sif_finder_exodus_variant_from_name", "sif_finder_exodus", "sif_finder_exodus_raw",
    "sif_finder_grid_cells_from_size", "sif_finder_exodus_checkpoint_read",
    "sif_finder_exodus_survey", "sif_finder_exodus_survey_raw", "sif_finder_exodus_survey_box",
    "sifg_exodus_survey_device",
    # device-resident additions
    "sifg_cic_device", "sifg_contrast_device", "sifg_mesh_device", "sifg_smooth_device",
    "sifg_exodus_device", "sifg_box_device", "sifg_last_rung_stats", "sifg_last_timings", "sifg_last_trace",
    "sifg_set_window", "sifg_set_growth_mode", "sifg_set_shell_list", "sifg_set_commit_mode", "sifg_set_scan_mode", "sifg_set_witness", "sifg_set_factor_tables", "sifg_set_halt_after",
    "sifg_set_host_mirrors", "sifg_host_mirrors", "sifg_host_modified", "sifg_copy_bytes", "sifg_candidate_ranks", "sifg_stream", "sifg_launch_count",
    "sifg_mesh_device_noalloc",
    # the FP64 form
    "sifg_cic_device_f64", "sifg_contrast_device_f64", "sifg_mesh_device_f64",
    "sifg_smooth_device_f64", "sifg_exodus_device_f64", "sifg_box_device_f64",
    # weighted meshes
    "sifg_cic_weighted_device", "sifg_cic_weighted_device_f64", "sifg_mesh_weights_device",
    "sifg_mesh_weights_device_f64", "sifg_exodus_weighted_device",
    "sifg_exodus_weighted_device_f64",
    # the adjoint
    "sifg_contrast_vjp_device", "sifg_contrast_vjp_device_f64",
    # the batched form
    "sifg_box_batch_device", "sifg_box_batch_autotune",
]


class BoxJob(C.Structure):
    """sifg_box_job_t (include/sif_gb300.h)."""
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("n_particles", C.c_uint64), ("n_grid", C.c_uint32), ("box", C.c_float),
                ("mesh_cells", C.c_uint32), ("radii", C.c_void_p), ("n_radii", C.c_uint32),
                ("threshold", C.c_float), ("overlap", C.c_float), ("options", C.c_uint32),
                ("cx", C.c_void_p), ("cy", C.c_void_p), ("cz", C.c_void_p), ("r", C.c_void_p),
                ("capacity", C.c_uint64), ("n_voids", C.c_uint64), ("status", C.c_int),
                ("wall_ms", C.c_double)]


def load():
    """The library, loaded once; raises OSError when it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError(f"{LIB_PATH} is not built; run sif_gb300/build.py "
                      "(or __graft_entry__.build())")
    lib = C.CDLL(LIB_PATH)
    abi.bind_sif_api(lib)
    vp, u32, u64, f32, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_int
    f64 = C.c_double
    sigs = {
        "sifg_cic_device": (i32, [vp, vp, vp, u64, u32, f32, vp]),
        "sifg_contrast_device": (i32, [vp, u64, C.POINTER(C.c_double)]),
        "sifg_mesh_device": (i32, [vp, vp, vp, u64, u32, f32, vp, vp, vp, vp, vp]),
        "sifg_smooth_device": (i32, [vp, u32, f32, f32, i32, i32, vp]),
        "sifg_exodus_device": (i32, [vp, u32, f32, vp, vp, vp, vp, u64, u32, vp, u32, f32, f32,
                                     u32, vp, vp, u64, vp, vp, vp, vp, u64, C.POINTER(u64)]),
        "sifg_box_device": (i32, [vp, vp, vp, u64, u32, f32, u32, vp, u32, f32, f32, u32,
                                  vp, vp, vp, vp, u64, C.POINTER(u64)]),
        "sifg_last_rung_stats": (u32, [C.POINTER(RungStat), u32]),
        "sifg_last_timings": (None, [C.POINTER(Timings)]),
        "sifg_last_trace": (u32, [C.POINTER(TraceEvent), u32]),
        "sifg_set_window": (None, [i32]),
        "sifg_set_growth_mode": (None, [i32]),
        "sifg_set_shell_list": (None, [i32]),
        "sifg_set_commit_mode": (None, [i32]),
        "sifg_set_scan_mode": (None, [i32]),
        "sifg_set_witness": (None, [i32]),
        "sifg_set_factor_tables": (None, [i32]),
        "sifg_set_halt_after": (None, [u32]),
        "sifg_exodus_survey_device": (i32, [vp, vp, u32, f32, C.POINTER(DeviceMesh),
                                            C.POINTER(DeviceMesh), vp, u32, f32, f32, u32, vp,
                                            vp, u64, vp, vp, vp, vp, vp, vp, u64,
                                            C.POINTER(u64)]),
        "sifg_set_host_mirrors": (None, [i32]),
        "sifg_host_mirrors": (i32, []),
        "sifg_host_modified": (None, [vp]),
        "sifg_copy_bytes": (None, [C.POINTER(u64), C.POINTER(u64)]),
        "sifg_stream": (u64, []),
        "sifg_launch_count": (u64, []),
        "sifg_mesh_device_noalloc": (i32, [vp, vp, vp, u64, u32, f32, vp, vp, vp, vp, vp]),
        "sifg_candidate_ranks": (None, [vp, u32, vp]),
        "sifg_cic_device_f64": (i32, [vp, vp, vp, u64, u32, f64, vp]),
        "sifg_contrast_device_f64": (i32, [vp, u64, C.POINTER(C.c_double)]),
        "sifg_mesh_device_f64": (i32, [vp, vp, vp, u64, u32, f64, vp, vp, vp, vp, vp]),
        "sifg_smooth_device_f64": (i32, [vp, u32, f64, f64, i32, i32, vp]),
        "sifg_exodus_device_f64": (i32, [vp, u32, f64, vp, vp, vp, vp, u64, u32, vp, u32, f64,
                                         f64, u32, vp, vp, u64, vp, vp, vp, vp, u64, C.POINTER(u64)]),
        "sifg_box_device_f64": (i32, [vp, vp, vp, u64, u32, f64, u32, vp, u32, f64, f64, u32,
                                      vp, vp, vp, vp, u64, C.POINTER(u64)]),
        "sifg_cic_weighted_device": (i32, [vp, vp, vp, vp, u64, u32, f32, vp]),
        "sifg_cic_weighted_device_f64": (i32, [vp, vp, vp, vp, u64, u32, f64, vp]),
        "sifg_mesh_weights_device": (i32, [vp, vp, u64, vp, u32, vp, vp, C.POINTER(f64)]),
        "sifg_mesh_weights_device_f64": (i32, [vp, vp, u64, vp, u32, vp, vp, C.POINTER(f64)]),
        "sifg_exodus_weighted_device": (i32, [vp, u32, f32, vp, vp, vp, vp, vp, vp, f64, u64, u32,
                                              vp, u32, f32, f32, u32, vp, vp, u64, vp, vp, vp,
                                              vp, u64, C.POINTER(u64)]),
        "sifg_exodus_weighted_device_f64": (i32, [vp, u32, f64, vp, vp, vp, vp, vp, vp, f64, u64,
                                                  u32, vp, u32, f64, f64, u32, vp, vp, u64, vp,
                                                  vp, vp, vp, u64, C.POINTER(u64)]),
        "sifg_contrast_vjp_device": (i32, [vp, vp, vp, u64, u32, f32, vp, vp, vp, vp]),
        "sifg_contrast_vjp_device_f64": (i32, [vp, vp, vp, u64, u32, f64, vp, vp, vp, vp]),
        "sifg_box_batch_device": (i32, [C.POINTER(BoxJob), u32, u32, C.POINTER(u32)]),
        "sifg_box_batch_autotune": (i32, [C.POINTER(BoxJob), u32, C.POINTER(u32)]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_error(lib, status, what):
    """The exception pysif raises for a sif status (python/src/py_common.h)."""
    msg = lib.sif_error_message()
    text = f"{what}: {msg.decode() if msg else status}"
    if status == abi.SIF_ERR_UNINITIALISED:
        return RuntimeError(text)
    if status == abi.SIF_ERR_ALLOC:
        return MemoryError(text)
    if status == abi.SIF_ERR_UNSUPPORTED:
        return NotImplementedError(text)
    return ValueError(text)
