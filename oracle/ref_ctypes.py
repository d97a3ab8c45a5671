"""Drives the reference sif library (oracle/_ref) through its public C API.

TEST INFRASTRUCTURE ONLY: used by the CPU tests in this container, by the
fixture generator under tests/golden/, and by nothing on the product path.
The library is the reference compiled from its own sources by oracle/Makefile
(``make ref``); it is absent wherever the reference checkout is, and callers
skip then.

The calls are the ones a C user of sif makes (docs/examples/run_exodus.md):
sif_system_init, sif_field_alloc + sif_field_assign_positions,
sif_grid_alloc + sif_grid_assign_cic + sif_grid_to_density_contrast,
sif_chain_mesh_alloc, sif_finder_exodus_raw, sif_catalogue_free.
"""
import ctypes as C
import os

import numpy as np

from sif_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
VARIANTS = {
    "strict": "libsif_ref.so",
    "f64": "libsif_ref_f64.so",
    "fast": "libsif_ref_fast.so",
}

_LIBS = {}


def available(variant="strict"):
    return os.path.exists(os.path.join(HERE, "_ref", VARIANTS[variant]))


def load(variant="strict", n_threads=0, log_level=abi.SIF_LOG_LEVEL_ERROR):
    if variant in _LIBS:
        return _LIBS[variant]
    path = os.path.join(HERE, "_ref", VARIANTS[variant])
    lib = C.CDLL(path, mode=C.RTLD_LOCAL)
    abi.bind_sif_api(lib, real_of(variant))
    field_t, grid_t, mesh_t, _, extras_t = (
        abi.STRUCTS_F64 if variant == "f64" else
        (abi.sif_field_t, abi.sif_grid_t, abi.sif_chain_mesh_t, abi.sif_catalogue_t,
         abi.sif_finder_exodus_extras_t))
    lib.sif_finder_exodus_raw.argtypes = [
        C.POINTER(grid_t), C.POINTER(mesh_t), C.c_void_p,
        C.c_uint32, real_of(variant), real_of(variant), C.c_uint32, C.POINTER(extras_t)]
    lib.sif_grid_alloc.argtypes = [C.c_uint32, real_of(variant)]
    lib.sif_chain_mesh_alloc.argtypes = [C.c_uint32, real_of(variant),
                                         C.POINTER(field_t), C.c_uint32]
    lib.sif_field_assign_positions.argtypes = [C.POINTER(field_t),
                                               C.c_void_p, C.c_void_p, C.c_void_p]
    lib.sif_field_assign_weights.argtypes = [C.POINTER(field_t), C.c_void_p]
    lib.orc_hook_inject.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32]
    lib.orc_hook_capture.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32]
    lib.orc_hook_calls.restype = C.c_uint32
    fft = abi.sif_fft_config_t(skip_tuning=True)
    omp = abi.sif_omp_config_t(n_threads=n_threads)
    cfg = abi.sif_config_t(C.pointer(fft), C.pointer(omp), log_level, None, 0)
    st = lib.sif_system_init(C.byref(cfg))
    if st != abi.SIF_OK:
        raise RuntimeError(f"sif_system_init: {st}")
    _LIBS[variant] = lib
    return lib


def real_of(variant):
    return C.c_double if variant == "f64" else C.c_float


def np_real(variant):
    return np.float64 if variant == "f64" else np.float32


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _check(lib, ok, what):
    if not ok:
        msg = lib.sif_error_message()
        raise RuntimeError(f"{what}: {msg.decode() if msg else lib.sif_error_status()}")


class RefField:
    def __init__(self, lib, x, y, z, variant="strict", weights=None):
        t = np_real(variant)
        self.lib = lib
        self.x, self.y, self.z = (np.ascontiguousarray(a, dtype=t) for a in (x, y, z))
        self.ptr = lib.sif_field_alloc(len(self.x))
        _check(lib, bool(self.ptr), "sif_field_alloc")
        st = lib.sif_field_assign_positions(self.ptr, _ptr(self.x), _ptr(self.y), _ptr(self.z))
        _check(lib, st == 0, "sif_field_assign_positions")
        if weights is not None:
            self.w = np.ascontiguousarray(weights, dtype=t)
            st = lib.sif_field_assign_weights(self.ptr, _ptr(self.w))
            _check(lib, st == 0, "sif_field_assign_weights")

    def free(self):
        if self.ptr:
            self.lib.sif_field_free(self.ptr)
            self.ptr = None


class RefGrid:
    def __init__(self, lib, n, box, variant="strict"):
        self.lib, self.n, self.variant = lib, n, variant
        self.ptr = lib.sif_grid_alloc(n, box)
        _check(lib, bool(self.ptr), "sif_grid_alloc")

    def assign_cic(self, field):
        st = self.lib.sif_grid_assign_cic(self.ptr, field.ptr)
        _check(self.lib, st == 0, "sif_grid_assign_cic")

    def to_contrast(self):
        st = self.lib.sif_grid_to_density_contrast(self.ptr)
        _check(self.lib, st == 0, "sif_grid_to_density_contrast")

    def values(self):
        g = self.ptr.contents
        t = np_real(self.variant)
        buf = C.cast(g.values, C.POINTER(C.c_double if t == np.float64 else C.c_float))
        return np.ctypeslib.as_array(buf, shape=(g.total_cells,)).copy()

    def set_values(self, v, content=abi.SIF_GRID_DENSITY_CONTRAST):
        g = self.ptr.contents
        t = np_real(self.variant)
        v = np.ascontiguousarray(v, dtype=t).reshape(-1)
        assert v.size == g.total_cells
        C.memmove(g.values, _ptr(v), v.nbytes)
        g.content = content
        g.assignment = abi.SIF_ASSIGNMENT_CIC

    def free(self):
        if self.ptr:
            self.lib.sif_grid_free(self.ptr)
            self.ptr = None


class RefMesh:
    def __init__(self, lib, n_cells, box, field, opt=0):
        self.lib = lib
        self.ptr = lib.sif_chain_mesh_alloc(n_cells, box, field.ptr, opt)
        _check(lib, bool(self.ptr), "sif_chain_mesh_alloc")

    def arrays(self, variant="strict"):
        m = self.ptr.contents
        n = m.n_particles
        ct = C.c_double if variant == "f64" else C.c_float

        def col(p):
            return np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(n,)).copy()

        offs = np.ctypeslib.as_array(m.cell_offsets, shape=(m.total_cells + 1,)).copy()
        idx = None
        if m.original_indices:
            idx = np.ctypeslib.as_array(m.original_indices, shape=(n,)).copy()
        return col(m.x), col(m.y), col(m.z), offs, idx

    def weights(self, variant="strict"):
        """(weights in mesh order, per-cell sums, total), or None unweighted."""
        m = self.ptr.contents
        if not m.weights:
            return None
        ct = C.c_double if variant == "f64" else C.c_float
        w = np.ctypeslib.as_array(C.cast(m.weights, C.POINTER(ct)), shape=(m.n_particles,)).copy()
        cw = np.ctypeslib.as_array(C.cast(m.cell_weights, C.POINTER(ct)),
                                   shape=(m.total_cells,)).copy()
        return w, cw, float(m.total_weight)

    def free(self):
        if self.ptr:
            self.lib.sif_chain_mesh_free(self.ptr)
            self.ptr = None


def catalogue_arrays(lib, cat_ptr, variant="strict"):
    cat = cat_ptr.contents
    n = cat.n_voids
    ct = C.c_double if variant == "f64" else C.c_float
    out = []
    for p in (cat.cx, cat.cy, cat.cz, cat.radii):
        if n == 0:
            out.append(np.zeros(0, dtype=np_real(variant)))
        else:
            out.append(np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(n,)).copy())
    lib.sif_catalogue_free(cat_ptr)
    return tuple(out)


def exodus_raw(lib, grid, mesh, radii, threshold, overlap=0.0, opt=0, variant="strict",
               inject=None, capture=None, prior=None, calls=None):
    """Runs sif_finder_exodus_raw; returns (cx, cy, cz, r).

    inject: (n_rungs, cells) array of smoothed fields that replace the
    reference's own, rung by rung; capture: an array of the same shape that
    receives the fields the reference computed; prior: (cx, cy, cz, r), the
    voids to start from (sif_finder_exodus_extras_t::prior); calls: a list
    that receives the number of backward transforms the run made.
    """
    t = np_real(variant)
    radii = np.ascontiguousarray(radii, dtype=t)
    cells = grid.ptr.contents.total_cells
    keep = []
    extras = None
    if prior is not None:
        Cat, Extras = ((abi.STRUCTS_F64[3], abi.STRUCTS_F64[4]) if variant == "f64" else
                       (abi.sif_catalogue_t, abi.sif_finder_exodus_extras_t))
        cols = [np.ascontiguousarray(c, dtype=t) for c in prior]
        keep.extend(cols)
        P = C.POINTER(real_of(variant))
        cat = Cat()
        cat.cx, cat.cy, cat.cz, cat.radii = (c.ctypes.data_as(P) for c in cols)
        cat.units = 0
        cat.n_voids = cat.capacity = len(cols[0])
        keep.append(cat)
        extras = Extras(None, C.pointer(cat), 0, 0)
        keep.append(extras)
    if inject is not None:
        inj = np.ascontiguousarray(inject, dtype=t)
        keep.append(inj)
        lib.orc_hook_inject(_ptr(inj), cells, inj.shape[0])
    if capture is not None:
        assert capture.dtype == t and capture.flags.c_contiguous
        lib.orc_hook_capture(_ptr(capture), cells, capture.shape[0])
    try:
        cat = lib.sif_finder_exodus_raw(grid.ptr, mesh.ptr, _ptr(radii), len(radii),
                                        threshold, overlap, opt | abi.SIF_FINDER_NO_CHECKPOINT,
                                        C.byref(extras) if extras is not None else None)
    finally:
        if calls is not None:
            calls.append(lib.orc_hook_calls())
        lib.orc_hook_inject(None, 0, 0)
        lib.orc_hook_capture(None, 0, 0)
    _check(lib, bool(cat), "sif_finder_exodus_raw")
    return catalogue_arrays(lib, cat, variant)


def pipeline(x, y, z, n_grid, box, mesh_cells, radii, threshold, overlap=0.0, opt=0,
             variant="strict", n_threads=0, inject=None, capture=None, want_grid=False):
    """CIC -> contrast -> chain mesh -> exodus, all through the reference."""
    lib = load(variant, n_threads)
    f = RefField(lib, x, y, z, variant)
    g = RefGrid(lib, n_grid, box, variant)
    try:
        g.assign_cic(f)
        g.to_contrast()
        grid_vals = g.values() if want_grid else None
        m = RefMesh(lib, mesh_cells, box, f)
        try:
            cat = exodus_raw(lib, g, m, radii, threshold, overlap, opt, variant,
                             inject, capture)
        finally:
            m.free()
    finally:
        g.free()
        f.free()
    return (cat, grid_vals) if want_grid else cat


def _bind_survey(lib, variant):
    if getattr(lib, "_survey_bound", False):
        return
    field_t, grid_t, mesh_t, cat_t, extras_t = (
        abi.STRUCTS_F64 if variant == "f64" else
        (abi.sif_field_t, abi.sif_grid_t, abi.sif_chain_mesh_t, abi.sif_catalogue_t,
         abi.sif_finder_exodus_extras_t))
    real = real_of(variant)
    lib.sif_finder_exodus_survey_raw.argtypes = [
        C.POINTER(grid_t), C.POINTER(grid_t), C.POINTER(mesh_t), C.POINTER(mesh_t), C.c_void_p,
        C.c_void_p, C.c_uint32, real, real, C.c_uint32, C.POINTER(extras_t)]
    lib.sif_finder_exodus_survey_raw.restype = C.POINTER(cat_t)
    lib.sif_finder_exodus_survey_box.argtypes = [
        C.POINTER(field_t), C.POINTER(field_t), C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
        C.POINTER(real)]
    lib.sif_finder_exodus_survey_box.restype = C.c_int
    lib._survey_bound = True


def survey_box(lib, data, randoms, radii, opt=0, variant="strict"):
    """sif_finder_exodus_survey_box: (offset (3,), box length)."""
    _bind_survey(lib, variant)
    t = np_real(variant)
    r = np.ascontiguousarray(radii, dtype=t)
    off = np.zeros(3, t)
    L = real_of(variant)(0)
    st = lib.sif_finder_exodus_survey_box(data.ptr, randoms.ptr, _ptr(r), len(r), opt, _ptr(off),
                                          C.byref(L))
    _check(lib, st == 0, "sif_finder_exodus_survey_box")
    return off, float(L.value)


def exodus_survey_raw(lib, dgrid, rgrid, dmesh, rmesh, radii, threshold, overlap=0.0, opt=0,
                      offset=None, variant="strict", capture=None, calls=None):
    """Runs sif_finder_exodus_survey_raw on CIC density grids (as
    sif_grid_assign_cic leaves them) and the two meshes; returns (cx, cy, cz,
    r, footprint, footprint_shell). capture: (2 n_radii + 2, cells) receives
    the fields the run's backward transforms return, in order (per rung the
    data's top-hat, then the randoms'; the two restores last)."""
    _bind_survey(lib, variant)
    t = np_real(variant)
    radii = np.ascontiguousarray(radii, dtype=t)
    cells = dgrid.ptr.contents.total_cells
    off = None if offset is None else np.ascontiguousarray(offset, dtype=t)
    if capture is not None:
        assert capture.dtype == t and capture.flags.c_contiguous
        lib.orc_hook_capture(_ptr(capture), cells, capture.shape[0])
    try:
        cat = lib.sif_finder_exodus_survey_raw(
            dgrid.ptr, rgrid.ptr, dmesh.ptr, rmesh.ptr, _ptr(off) if off is not None else None,
            _ptr(radii), len(radii), threshold, overlap, opt | abi.SIF_FINDER_NO_CHECKPOINT, None)
    finally:
        if calls is not None:
            calls.append(lib.orc_hook_calls())
        lib.orc_hook_capture(None, 0, 0)
    _check(lib, bool(cat), "sif_finder_exodus_survey_raw")
    c = cat.contents
    n = c.n_voids
    ct = C.c_double if variant == "f64" else C.c_float
    cols = []
    for p in (c.cx, c.cy, c.cz, c.radii, c.footprint, c.footprint_shell):
        cols.append(np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(n,)).copy() if n and p
                    else np.zeros(0, t))
    lib.sif_catalogue_free(cat)
    return tuple(cols)
