"""ctypes wrapper of liboracle.so, this project's C restatement of sif's exodus
path (exodus_oracle.c). TEST INFRASTRUCTURE ONLY: imported by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg, as the checker;
never by the product path.

``build()`` compiles it with the Makefile beside this file (gcc + OpenMP),
which works on both the x86 build machine and the Arm GPU machines.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
FAST_PATH = os.path.join(HERE, "liboracle_fast.so")

_lib = None
_fast = None


def build(quiet=True):
    out = subprocess.run(["make", "-s", "-C", HERE, "oracle"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


class Mesh(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("offsets", C.c_void_p), ("n_particles", C.c_uint64),
                ("n_cells", C.c_uint32), ("box_length", C.c_float),
                ("cell_length", C.c_float), ("w", C.c_void_p), ("cell_w", C.c_void_p),
                ("total_weight", C.c_double)]


class Template(C.Structure):
    _fields_ = [("dx", C.c_void_p), ("dy", C.c_void_p), ("dz", C.c_void_p),
                ("type", C.c_void_p), ("min_d2", C.c_void_p), ("max_d2", C.c_void_p),
                ("count", C.c_uint32)]


class RungStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "n_candidates", "rejected_masked", "rejected_proxy", "rejected_overlap",
        "rejected_rescale", "rejected_proxy_recheck", "rejected_exact",
        "rejected_witness", "accepted", "n_rescaled")]


class Params(C.Structure):
    _fields_ = [("grid_n", C.c_uint32), ("box_length", C.c_float),
                ("threshold", C.c_float), ("overlap_fraction", C.c_float),
                ("options", C.c_uint32), ("n_threads", C.c_int), ("window", C.c_int),
                ("smoothing_mode", C.c_int), ("inject", C.c_void_p),
                ("prior_cx", C.c_void_p), ("prior_cy", C.c_void_p), ("prior_cz", C.c_void_p),
                ("prior_r", C.c_void_p), ("n_prior", C.c_uint64),
                ("random_mesh", C.c_void_p), ("random_grid", C.c_void_p)]


class Catalogue(C.Structure):
    _fields_ = [("cx", C.POINTER(C.c_float)), ("cy", C.POINTER(C.c_float)),
                ("cz", C.POINTER(C.c_float)), ("r", C.POINTER(C.c_float)),
                ("n_voids", C.c_uint64), ("footprint", C.POINTER(C.c_float)),
                ("footprint_shell", C.POINTER(C.c_float))]


def lib(fast=False):
    """The strict build (the checker), or with fast=True the release-flags
    build the CPU baseline is timed with."""
    global _lib, _fast
    if fast:
        if _fast is None:
            if not os.path.exists(FAST_PATH):
                build()
            _fast = _declare(C.CDLL(FAST_PATH))
        return _fast
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = _declare(C.CDLL(LIB_PATH))
    return _lib


def _declare(L):
    vp, u64, u32, f32 = C.c_void_p, C.c_uint64, C.c_uint32, C.c_float
    L.orc_chain_mesh.argtypes = [vp, vp, vp, u64, u32, f32, vp, vp, vp, vp, vp]
    L.orc_cic_f64.argtypes = [vp, vp, vp, u64, u32, f32, vp]
    L.orc_cic_float.argtypes = [vp, vp, vp, u64, u32, f32, vp]
    L.orc_cic_f64_w.argtypes = [vp, vp, vp, vp, u64, u32, f32, vp]
    L.orc_cic_float_w.argtypes = [vp, vp, vp, vp, u64, u32, f32, vp]
    L.orc_mesh_weights.argtypes = [vp, vp, u64, vp, u32, vp, vp, C.POINTER(C.c_double)]
    L.orc_density_contrast.argtypes = [vp, u64]
    L.orc_density_contrast_f64.argtypes = [vp, u64]
    L.orc_spectrum_new_f64.argtypes = [vp, u32, f32, C.c_int]
    L.orc_spectrum_new_f64.restype = vp
    L.orc_spectrum_new.argtypes = [vp, u32, f32, C.c_int, C.c_int]
    L.orc_spectrum_new.restype = vp
    L.orc_spectrum_smooth.argtypes = [vp, C.c_int, f32, f32, vp, vp]
    L.orc_spectrum_free.argtypes = [vp]
    L.orc_sort_candidates.argtypes = [vp, u64]
    L.orc_template_build.argtypes = [C.POINTER(Template), u32, f32, f32, f32]
    L.orc_template_free.argtypes = [C.POINTER(Template)]
    L.orc_find_radius.argtypes = [C.POINTER(Mesh), C.POINTER(Template), f32, f32, f32,
                                  f32, f32, f32, f32, u32, C.POINTER(C.c_uint8),
                                  C.POINTER(u64), C.POINTER(u64)]
    L.orc_find_radius.restype = f32
    L.orc_find_radius_weighted.argtypes = [C.POINTER(Mesh), C.POINTER(Template), f32, f32, f32,
                                           f32, f32, f32, f32, f32, u32, C.POINTER(C.c_uint8),
                                           C.POINTER(u64), C.POINTER(u64)]
    L.orc_find_radius_weighted.restype = f32
    L.orc_brute_force_radius.argtypes = [vp, vp, vp, u64, f32, C.c_double, C.c_double,
                                         C.c_double, C.c_double, C.c_double, C.c_double]
    L.orc_brute_force_radius.restype = C.c_double
    L.orc_exodus.argtypes = [vp, C.POINTER(Mesh), vp, u32, C.POINTER(Params),
                             C.POINTER(Catalogue), vp]
    L.orc_catalogue_free.argtypes = [C.POINTER(Catalogue)]
    L.orc_survey_occupancy.argtypes = [C.POINTER(Mesh), u32, f32, vp, C.POINTER(C.c_int32)]
    L.orc_survey_occupancy.restype = u64
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


CANDIDATE_DTYPE = np.dtype([("delta", np.float32), ("refined", np.uint32), ("flat", np.uint64)])


class OracleMesh:
    """A chain mesh built by the oracle; keeps its arrays alive. weights:
    per-particle weights in the field's order (a weighted mesh), or None."""

    def __init__(self, x, y, z, n_cells, box, weights=None):
        n = len(x)
        self.x = np.empty(n, np.float32)
        self.y = np.empty(n, np.float32)
        self.z = np.empty(n, np.float32)
        self.offsets = np.empty(n_cells ** 3 + 1, np.uint64)
        self.orig = np.empty(n, np.uint64)
        xs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z)]
        st = lib().orc_chain_mesh(_p(xs[0]), _p(xs[1]), _p(xs[2]), n, n_cells, box,
                                  _p(self.x), _p(self.y), _p(self.z), _p(self.offsets),
                                  _p(self.orig))
        if st != 0:
            raise ValueError(f"orc_chain_mesh: {st}")
        self.n_cells = n_cells
        self.box = np.float32(box)
        self.cell_length = np.float32(np.float32(box) / np.float32(n_cells))
        self.w = self.cell_w = None
        self.total_weight = float(n)
        if weights is not None:
            fw = np.ascontiguousarray(weights, np.float32)
            assert fw.shape == (n,)
            self.w = np.empty(n, np.float32)
            self.cell_w = np.empty(n_cells ** 3, np.float32)
            tot = C.c_double()
            lib().orc_mesh_weights(_p(fw), _p(self.orig), n, _p(self.offsets), n_cells,
                                   _p(self.w), _p(self.cell_w), C.byref(tot))
            self.total_weight = tot.value
        self._make_struct()

    def _make_struct(self):
        self.struct = Mesh(_p(self.x), _p(self.y), _p(self.z), _p(self.offsets), len(self.x),
                           self.n_cells, float(self.box), float(self.cell_length),
                           _p(self.w) if self.w is not None else None,
                           _p(self.cell_w) if self.cell_w is not None else None,
                           self.total_weight)

    @classmethod
    def from_arrays(cls, x, y, z, offsets, n_cells, box, w=None, cell_w=None, total_weight=None):
        """A mesh from its columns (another build's), weighted when w is given
        (with the per-cell sums and the total)."""
        self = cls.__new__(cls)
        self.x, self.y, self.z = (np.ascontiguousarray(a, np.float32) for a in (x, y, z))
        self.offsets = np.ascontiguousarray(offsets, np.uint64)
        self.orig = None
        self.n_cells = n_cells
        self.box = np.float32(box)
        self.cell_length = np.float32(np.float32(box) / np.float32(n_cells))
        self.w = None if w is None else np.ascontiguousarray(w, np.float32)
        self.cell_w = None if cell_w is None else np.ascontiguousarray(cell_w, np.float32)
        self.total_weight = float(len(self.x)) if total_weight is None else float(total_weight)
        self._make_struct()
        return self


def _weights_arg(w, n):
    if w is None:
        return None, None
    a = np.ascontiguousarray(w, dtype=np.float32)
    assert a.shape == (n,)
    return a, _p(a)


def cic_f64(x, y, z, n_grid, box, weights=None):
    out = np.empty(n_grid ** 3, np.float64)
    xs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z)]
    keep, wp = _weights_arg(weights, len(xs[0]))
    lib().orc_cic_f64_w(_p(xs[0]), _p(xs[1]), _p(xs[2]), wp, len(xs[0]), n_grid, box, _p(out))
    return out


def cic_float(x, y, z, n_grid, box, weights=None):
    """The reference's float CIC deposit (its slab and chunk order)."""
    out = np.empty(n_grid ** 3, np.float32)
    xs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z)]
    keep, wp = _weights_arg(weights, len(xs[0]))
    lib().orc_cic_float_w(_p(xs[0]), _p(xs[1]), _p(xs[2]), wp, len(xs[0]), n_grid, box, _p(out))
    return out


def density_contrast(v):
    v = np.ascontiguousarray(v, dtype=np.float32).copy()
    st = lib().orc_density_contrast(_p(v), v.size)
    if st != 0:
        raise ValueError(f"orc_density_contrast: {st}")
    return v


def density_contrast_f64(v, inplace=False):
    """The contrast of an FP64 density, in double (in v itself with inplace,
    for a contiguous float64 v)."""
    v = v if inplace else np.ascontiguousarray(v, dtype=np.float64).copy()
    st = lib().orc_density_contrast_f64(_p(v), v.size)
    if st != 0:
        raise ValueError(f"orc_density_contrast_f64: {st}")
    return v


def smooth(delta, n_grid, box, radii, filter=1, sigma=0.0, window_mode=1, mode=0,
           want="f32"):
    """Per-radius smoothed fields, (len(radii), n^3), float32 or float64. A
    float64 delta takes the whole chain in double (mode 0)."""
    if np.asarray(delta).dtype == np.float64:
        d = np.ascontiguousarray(delta)
        s = lib().orc_spectrum_new_f64(_p(d), n_grid, box, window_mode)
    else:
        d = np.ascontiguousarray(delta, dtype=np.float32)
        s = lib().orc_spectrum_new(_p(d), n_grid, box, window_mode, mode)
    try:
        out = np.empty((len(radii), n_grid ** 3), np.float64 if want == "f64" else np.float32)
        for i, r in enumerate(radii):
            row = out[i]
            if want == "f64":
                lib().orc_spectrum_smooth(s, filter, float(r), float(sigma), None, _p(row))
            else:
                lib().orc_spectrum_smooth(s, filter, float(r), float(sigma), _p(row), None)
        return out
    finally:
        lib().orc_spectrum_free(s)


def sort_candidates(records):
    a = np.ascontiguousarray(records, dtype=CANDIDATE_DTYPE).copy()
    lib().orc_sort_candidates(_p(a), len(a))
    return a


def find_radius(mesh, cx, cy, cz, radius, r_search, threshold, vol_factor, window=8):
    t = Template()
    st = lib().orc_template_build(C.byref(t), mesh.n_cells, float(mesh.cell_length),
                                  float(radius), float(r_search))
    if st != 0:
        raise ValueError("template wider than the mesh")
    try:
        reason = C.c_uint8(0)
        ss, sc = C.c_uint64(0), C.c_uint64(0)
        r = lib().orc_find_radius(C.byref(mesh.struct), C.byref(t), cx, cy, cz, r_search,
                                  threshold, vol_factor, radius, window, C.byref(reason),
                                  C.byref(ss), C.byref(sc))
        return r, reason.value
    finally:
        lib().orc_template_free(C.byref(t))


def brute_force_radius(x, y, z, box, c, rung, r_search, threshold):
    xs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z)]
    return lib().orc_brute_force_radius(_p(xs[0]), _p(xs[1]), _p(xs[2]), len(xs[0]), box,
                                        float(c[0]), float(c[1]), float(c[2]), rung,
                                        r_search, threshold)


def exodus(delta, mesh, radii, n_grid, box, threshold, overlap=0.0, options=0, n_threads=1,
           window=0, smoothing_mode=1, inject=None, with_stats=False, prior=None,
           survey=None):
    """The oracle finder; returns (cx, cy, cz, r) float32 arrays. prior:
    (cx, cy, cz, r), voids to start from. survey: (random_mesh,
    random_density) for a survey run -- delta is then the data's CIC density,
    injected fields come two a rung (data, randoms), and the footprint columns
    follow the four (cx, cy, cz, r, footprint, footprint_shell)."""
    d = np.ascontiguousarray(delta, dtype=np.float32)
    radii = np.ascontiguousarray(radii, dtype=np.float32)
    inj = None
    if inject is not None:
        # As the run's transforms return them; under the Gaussian refinement
        # up to two a rung (padded, so a short list is never read past), in a
        # survey two a rung.
        inj = np.ascontiguousarray(inject, dtype=np.float32).reshape(-1, n_grid ** 3)
        assert inj.shape[0] >= len(radii)
        want = 2 * len(radii) if (options & (3 << 19) or survey is not None) else len(radii)
        if inj.shape[0] < want:
            assert survey is None, "a survey takes both fields of every rung"
            inj = np.concatenate([inj, np.zeros((want - inj.shape[0], n_grid ** 3), np.float32)])
    pri = [np.ascontiguousarray(c, dtype=np.float32) for c in prior] if prior is not None else None
    rmesh = rgrid = None
    if survey is not None:
        rmesh = survey[0]
        rgrid = np.ascontiguousarray(survey[1], dtype=np.float32)
    p = Params(n_grid, box, threshold, overlap, options, n_threads, window, smoothing_mode,
               _p(inj) if inj is not None else None,
               *([_p(c) for c in pri] if pri else [None] * 4), len(pri[0]) if pri else 0,
               C.cast(C.pointer(rmesh.struct), C.c_void_p) if rmesh is not None else None,
               _p(rgrid) if rgrid is not None else None)
    cat = Catalogue()
    stats = (RungStats * len(radii))()
    st = lib().orc_exodus(_p(d), C.byref(mesh.struct), _p(radii), len(radii), C.byref(p),
                          C.byref(cat), stats)
    if st != 0:
        raise ValueError(f"orc_exodus: {st}")
    n = cat.n_voids
    cols = ("cx", "cy", "cz", "r") + (("footprint", "footprint_shell") if survey is not None else ())
    out = tuple(np.ctypeslib.as_array(getattr(cat, k), shape=(n,)).copy() if n else
                np.zeros(0, np.float32) for k in cols)
    lib().orc_catalogue_free(C.byref(cat))
    if with_stats:
        return out, [{k: getattr(s, k) for k, _ in RungStats._fields_} for s in stats]
    return out


def pipeline(x, y, z, n_grid, box, mesh_cells, radii, threshold, n_threads, fast=False):
    """The whole path through the restatement, as the reference's caller runs
    it (sif_grid_assign_cic, sif_grid_to_density_contrast,
    sif_chain_mesh_alloc, sif_finder_exodus_raw with its own smoothing and
    the final restore of the grid): (catalogue, seconds per stage). fast: the
    release-flags build, for timing."""
    import time

    L = lib(fast)
    xs = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z)]
    n = len(xs[0])
    t = {}
    t0 = time.perf_counter()
    grid = np.empty(n_grid ** 3, np.float32)
    L.orc_cic_float(_p(xs[0]), _p(xs[1]), _p(xs[2]), n, n_grid, box, _p(grid))
    t["cic"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    if L.orc_density_contrast(_p(grid), grid.size) != 0:
        raise ValueError("orc_density_contrast")
    t["contrast"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    mx, my, mz = (np.empty(n, np.float32) for _ in range(3))
    offs = np.empty(mesh_cells ** 3 + 1, np.uint64)
    if L.orc_chain_mesh(_p(xs[0]), _p(xs[1]), _p(xs[2]), n, mesh_cells, box, _p(mx), _p(my),
                        _p(mz), _p(offs), None) != 0:
        raise ValueError("orc_chain_mesh")
    t["mesh"] = time.perf_counter() - t0
    mesh = Mesh(_p(mx), _p(my), _p(mz), _p(offs), n, mesh_cells, float(np.float32(box)),
                float(np.float32(np.float32(box) / np.float32(mesh_cells))))
    r = np.ascontiguousarray(radii, dtype=np.float32)
    p = Params(n_grid, box, threshold, 0.0, 0, n_threads, 0, 1, None, None, None, None, None, 0,
               None, None)
    cat = Catalogue()
    t0 = time.perf_counter()
    st = L.orc_exodus(_p(grid), C.byref(mesh), _p(r), len(r), C.byref(p), C.byref(cat), None)
    t["finder"] = time.perf_counter() - t0
    if st != 0:
        raise ValueError(f"orc_exodus: {st}")
    nv = cat.n_voids
    out = tuple(np.ctypeslib.as_array(getattr(cat, k), shape=(nv,)).copy() if nv else
                np.zeros(0, np.float32) for k in ("cx", "cy", "cz", "r"))
    L.orc_catalogue_free(C.byref(cat))
    return out, t


def smoothing_seconds(delta, n_grid, box, radii, fast=False):
    """The transforms the finder runs on its own (the forward once, the
    filter and backward per rung, the unfiltered restore), timed alone: the
    part of the finder's time that is the FFT stage."""
    import time

    L = lib(fast)
    d = np.ascontiguousarray(delta, dtype=np.float32)
    out = np.empty(n_grid ** 3, np.float32)
    t0 = time.perf_counter()
    s = L.orc_spectrum_new(_p(d), n_grid, box, 1, 1)
    for r in radii:
        L.orc_spectrum_smooth(s, 1, float(r), 0.0, _p(out), None)
    L.orc_spectrum_smooth(s, 0, 0.0, 0.0, _p(out), None)
    L.orc_spectrum_free(s)
    return time.perf_counter() - t0


class Spectrum:
    """An FP64 spectrum of a double contrast, kept to smooth at several radii
    one at a time (each smoothing returns one n^3 float64 field)."""

    def __init__(self, delta64, n_grid, box, window_mode=1):
        d = np.ascontiguousarray(delta64, dtype=np.float64)
        self.n = n_grid
        self.ptr = lib().orc_spectrum_new_f64(_p(d), n_grid, box, window_mode)

    def smooth(self, r, filter=1):
        out = np.empty(self.n ** 3, np.float64)
        lib().orc_spectrum_smooth(self.ptr, filter, float(r), 0.0, None, _p(out))
        return out

    def free(self):
        if self.ptr:
            lib().orc_spectrum_free(self.ptr)
            self.ptr = None


def survey_occupancy(random_mesh, n_grid, box):
    """The observed nodes of a survey's grid, as a bool array (n^3,), and the
    closing's k."""
    words = np.zeros((n_grid ** 3 + 63) // 64, np.uint64)
    k = C.c_int32(0)
    lib().orc_survey_occupancy(C.byref(random_mesh.struct), n_grid, box, _p(words), C.byref(k))
    bits = np.unpackbits(words.view(np.uint8), bitorder="little")[: n_grid ** 3]
    return bits.astype(bool), k.value
