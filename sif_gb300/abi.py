"""ctypes mirrors of sif's public C structs and constants.

The GB300 library exports sif's own C API, so it takes and returns the same
structs as the reference; these are their layouts, field for field, for the
single-precision build (``sif_real`` = float):

- ``sif_field_t``       include/sif/structures/field.h:90-133
- ``sif_grid_t``        include/sif/structures/grid.h:86-128
- ``sif_chain_mesh_t``  include/sif/structures/chain_mesh.h:40-108
- ``sif_catalogue_t``   include/sif/structures/catalogue.h:38-93
- ``sif_config_t``      include/sif/core/system.h:61-100
- ``sif_finder_exodus_extras_t``  include/sif/finder/exodus_finder.h:40-106

The option bits and status codes are sif's (include/sif/core/macros.h).
"""
import ctypes as C

sif_real = C.c_float
P_real = C.POINTER(sif_real)
P_u64 = C.POINTER(C.c_uint64)

# Status codes, include/sif/core/macros.h:690-707.
SIF_OK = 0
SIF_ERR_ALLOC = -1
SIF_ERR_INVALID = -2
SIF_ERR_RANGE = -3
SIF_ERR_IO = -4
SIF_ERR_UNSUPPORTED = -5
SIF_ERR_UNINITIALISED = -6

# Finder options, include/sif/core/macros.h:73-292.
SIF_FINDER_ALIASING_WINDOW = 1 << 8
SIF_FINDER_SEEDS_CELLS = 0
SIF_FINDER_SEEDS_MINIMA = 1 << 9
SIF_FINDER_NO_CHECKPOINT = 1 << 11
SIF_FINDER_SEARCH_1_50 = 0 << 12
SIF_FINDER_SEARCH_1_25 = 1 << 12
SIF_FINDER_SEARCH_1_75 = 2 << 12
SIF_FINDER_SEARCH_2_00 = 3 << 12
SIF__FINDER_SEARCH_MASK = 3 << 12
SIF_FINDER_KEEP_CIC_WINDOW = 1 << 14
SIF_FINDER_CONSUME_GRID = 1 << 15
SIF_MESH_DROP_INDICES = 1 << 16
SIF_MESH_NO_CANONICAL = 1 << 17
SIF_FINDER_LAGRANGIAN_OVERLAP = 1 << 18
SIF_FINDER_REFINE_NONE = 0 << 19
SIF_FINDER_REFINE_GAUSSIAN = 1 << 19
SIF_FINDER_REFINE_TRACERS = 2 << 19
SIF_FINDER_REFINE_HILL = 3 << 19
SIF__FINDER_REFINE_MASK = 3 << 19
SIF_FINDER_EXTEND_REACH = 1 << 21
SIF_FINDER_DISPLACE = 1 << 22

# Search factors by encoding, include/sif/core/macros.h:123-126.
SEARCH_FACTORS = (1.5, 1.25, 1.75, 2.0)

# Variants, include/sif/finder/exodus_finder.h:124-133.
SIF_EXODUS_EXCURSION_SET = 0
SIF_EXODUS_EXCURSION_PEAK = 1
SIF_EXODUS_LAGRANGIAN_OVERLAP = 2

# Grid content / assignment tags, include/sif/structures/grid.h:32-71.
SIF_GRID_EMPTY = 0
SIF_GRID_DENSITY = 1
SIF_GRID_DENSITY_CONTRAST = 2
SIF_ASSIGNMENT_CIC = 2

# Log levels, include/sif/core/macros.h:772-777.
SIF_LOG_LEVEL_TRACE = 0
SIF_LOG_LEVEL_INFO = 2
SIF_LOG_LEVEL_WARNING = 3
SIF_LOG_LEVEL_ERROR = 4
SIF_LOG_LEVEL_NONE = 5


class sif_fft_config_t(C.Structure):
    _fields_ = [("skip_tuning", C.c_bool)]


class sif_omp_config_t(C.Structure):
    _fields_ = [("n_threads", C.c_uint32)]


class sif_setting_t(C.Structure):
    _fields_ = [("key", C.c_char_p), ("value", C.c_char_p)]


class sif_config_t(C.Structure):
    _fields_ = [
        ("fft_config", C.POINTER(sif_fft_config_t)),
        ("omp_config", C.POINTER(sif_omp_config_t)),
        ("log_level", C.c_uint8),
        ("settings", C.POINTER(sif_setting_t)),
        ("n_settings", C.c_size_t),
    ]


class sif_finder_exodus_checkpoint_t(C.Structure):
    """The exodus checkpoint's 192-byte header (include/sif/finder/
    exodus_finder.h:427-507)."""
    _fields_ = [
        ("magic", C.c_char * 4), ("version", C.c_uint32), ("byte_order", C.c_uint32),
        ("is_double", C.c_uint32), ("is_survey", C.c_uint32), ("is_weighted", C.c_uint32),
        ("options", C.c_uint32), ("n_radii", C.c_uint32), ("next_rung", C.c_uint32),
        ("grid_n_cells", C.c_uint32), ("box_length", C.c_double), ("threshold", C.c_double),
        ("overlap_fraction", C.c_double), ("n_particles", C.c_uint64),
        ("total_weight", C.c_double), ("random_n_particles", C.c_uint64),
        ("random_total_weight", C.c_double), ("offset", C.c_double * 3),
        ("n_prior", C.c_uint64), ("prior_crc32", C.c_uint32), ("crc32", C.c_uint32),
        ("n_voids", C.c_uint64), ("n_mismatched", C.c_uint64), ("assignment", C.c_uint32),
        ("reserved", C.c_char * 36),
    ]


def make_structs(real):
    """The reference's public structs with sif_real = `real` (C.c_float for
    the float build, C.c_double for its SIF_USE_DOUBLE build, whose struct
    layouts differ where a sif_real field sits before a pointer)."""
    sif_real = real
    P_real = C.POINTER(real)

    class sif_field_t(C.Structure):
        _fields_ = [
            ("_position_block", P_real),
            ("_velocity_block", P_real),
            ("x", P_real), ("y", P_real), ("z", P_real),
            ("vx", P_real), ("vy", P_real), ("vz", P_real),
            ("weights", P_real),
            ("original_indices", P_u64),
            ("min_p", sif_real * 3),
            ("max_p", sif_real * 3),
            ("centre", sif_real * 3),
            ("half_span", sif_real),
            ("state_flags", C.c_uint32),
            ("n_particles", C.c_uint64),
            ("units", C.c_int),
        ]


    class sif_grid_t(C.Structure):
        _fields_ = [
            ("values", P_real),
            ("content", C.c_int),
            ("assignment", C.c_int),
            ("interlaced", C.c_uint32),
            ("n_cells", C.c_uint32),
            ("total_cells", C.c_uint64),
            ("box_length", sif_real),
            ("cell_length", sif_real),
            ("p2_mask", C.c_uint32),
            ("p2_shift", C.c_uint32),
        ]


    class sif_chain_mesh_t(C.Structure):
        _fields_ = [
            ("n_cells", C.c_uint32),
            ("total_cells", C.c_uint64),
            ("box_length", sif_real),
            ("cell_length", sif_real),
            ("_position_block", P_real),
            ("_velocity_block", P_real),
            ("x", P_real), ("y", P_real), ("z", P_real),
            ("vx", P_real), ("vy", P_real), ("vz", P_real),
            ("weights", P_real),
            ("total_weight", C.c_double),
            ("cell_weights", P_real),
            ("original_indices", P_u64),
            ("n_particles", C.c_uint64),
            ("cell_offsets", P_u64),
        ]


    class sif_catalogue_t(C.Structure):
        _fields_ = [
            ("_block", P_real),
            ("cx", P_real), ("cy", P_real), ("cz", P_real), ("radii", P_real),
            ("_footprint_block", P_real),
            ("footprint", P_real),
            ("footprint_shell", P_real),
            ("units", C.c_int),
            ("_meta", C.c_void_p),
            ("_n_meta", C.c_uint32),
            ("n_voids", C.c_uint64),
            ("capacity", C.c_uint64),
        ]


    class sif_finder_exodus_extras_t(C.Structure):
        _fields_ = [
            ("checkpoint", C.c_char_p),
            ("prior", C.POINTER(sif_catalogue_t)),
            ("keep_checkpoint", C.c_int),
            ("save_memory", C.c_int),
        ]

    return sif_field_t, sif_grid_t, sif_chain_mesh_t, sif_catalogue_t, sif_finder_exodus_extras_t


(sif_field_t, sif_grid_t, sif_chain_mesh_t, sif_catalogue_t,
 sif_finder_exodus_extras_t) = make_structs(C.c_float)
STRUCTS_F64 = make_structs(C.c_double)


def bind_sif_api(lib, real=C.c_float):
    """Declares the signatures of sif's public C API on a loaded library.

    Used for both the reference build and the GB300 library, which export the
    same entry points; real = C.c_double for the reference's double build.
    """
    field_t, grid_t, mesh_t, cat_t, extras_t = (
        (sif_field_t, sif_grid_t, sif_chain_mesh_t, sif_catalogue_t, sif_finder_exodus_extras_t)
        if real is C.c_float else STRUCTS_F64)
    sif_real = real
    P_real = C.POINTER(real)
    P_field = C.POINTER(field_t)
    P_grid = C.POINTER(grid_t)
    P_mesh = C.POINTER(mesh_t)
    P_cat = C.POINTER(cat_t)
    sigs = {
        "sif_system_init": (C.c_int, [C.POINTER(sif_config_t)]),
        "sif_system_finalise": (None, []),
        "sif_error_status": (C.c_int, []),
        "sif_error_message": (C.c_char_p, []),
        "sif_field_alloc": (P_field, [C.c_uint64]),
        "sif_field_free": (None, [P_field]),
        "sif_field_assign_positions": (C.c_int, [P_field, P_real, P_real, P_real]),
        "sif_field_assign_weights": (C.c_int, [P_field, P_real]),
        "sif_field_reserve_weights": (C.c_int, [P_field]),
        "sif_grid_alloc": (P_grid, [C.c_uint32, sif_real]),
        "sif_grid_free": (None, [P_grid]),
        "sif_grid_assign_cic": (C.c_int, [P_grid, P_field]),
        "sif_grid_to_density_contrast": (C.c_int, [P_grid]),
        "sif_chain_mesh_alloc": (P_mesh, [C.c_uint32, sif_real, P_field, C.c_uint32]),
        "sif_chain_mesh_alloc_consume": (P_mesh, [C.c_uint32, sif_real, P_field, C.c_uint32]),
        "sif_chain_mesh_free": (None, [P_mesh]),
        "sif_catalogue_free": (None, [P_cat]),
        "sif_finder_exodus": (P_cat, [P_grid, P_mesh, P_real, C.c_uint32, sif_real,
                                      C.c_int, C.POINTER(extras_t)]),
        "sif_finder_exodus_raw": (P_cat, [P_grid, P_mesh, P_real, C.c_uint32, sif_real,
                                          sif_real, C.c_uint32, C.POINTER(extras_t)]),
        "sif_finder_exodus_preset": (C.c_int, [C.c_int, P_real, C.POINTER(C.c_uint32)]),
        "sif_finder_exodus_variant_name": (C.c_char_p, [C.c_int]),
        "sif_finder_exodus_variant_from_name": (C.c_int, [C.c_char_p, C.POINTER(C.c_int)]),
        "sif_finder_grid_cells_from_size": (C.c_uint32, [C.c_uint64, sif_real, sif_real,
                                                         C.c_int, sif_real]),
        "sif_finder_exodus_checkpoint_read": (P_cat, [C.c_char_p,
                                                      C.POINTER(sif_finder_exodus_checkpoint_t)]),
        "sif_finder_exodus_survey": (P_cat, [P_grid, P_grid, P_mesh, P_mesh, P_real, P_real,
                                             C.c_uint32, sif_real, C.c_int,
                                             C.POINTER(extras_t)]),
        "sif_finder_exodus_survey_raw": (P_cat, [P_grid, P_grid, P_mesh, P_mesh, P_real, P_real,
                                                 C.c_uint32, sif_real, sif_real, C.c_uint32,
                                                 C.POINTER(extras_t)]),
        "sif_finder_exodus_survey_box": (C.c_int, [P_field, P_field, P_real, C.c_uint32,
                                                   C.c_uint32, P_real, P_real]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib
