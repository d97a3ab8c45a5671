"""The pysif interface for the exodus path, over the GB300 library.

Mirrors the names and argument meanings of pysif (python/pysif/__init__.pyi,
finders.pyi:37-140; python/src/finders/py_finders.c:362-477;
python/src/structures/py_grid.c:49-122) so scripts written against pysif's
exodus path run unchanged: ``system_init``, ``Field``, ``Grid.assign_cic``,
``Grid.to_density_contrast``, ``ChainMesh``, ``finders.exodus`` and
``finders.exodus_raw``. Each call goes through sif's C API as the GB300
library exports it; the work runs on the GPU.
"""
import ctypes as C
import types

import numpy as np

from . import _lib, abi


def _P(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _check(status, what):
    if status != abi.SIF_OK:
        raise _lib.status_error(_lib.load(), status, what)


def system_init(n_threads=0, log_level="warning", skip_tuning=True):
    """pysif.system_init: selects the GPU; n_threads sizes the host team."""
    lib = _lib.load()
    levels = {"trace": 0, "debug": 1, "info": 2, "warning": 3, "error": 4, "none": 5}
    fft = abi.sif_fft_config_t(skip_tuning=skip_tuning)
    omp = abi.sif_omp_config_t(n_threads=n_threads)
    cfg = abi.sif_config_t(C.pointer(fft), C.pointer(omp), levels[log_level], None, 0)
    _check(lib.sif_system_init(C.byref(cfg)), "system_init")


def system_finalise():
    _lib.load().sif_system_finalise()


def set_host_mirrors(on):
    """Keep device copies of the structs' host arrays between calls
    (sifg_set_host_mirrors): a pipeline then copies each array up once. With
    mirrors on, writes through a struct's arrays (Grid.values) must be
    declared with host_modified before the next call reads them."""
    _lib.load().sifg_set_host_mirrors(1 if on else 0)


def host_modified(obj=None):
    """Declares writes through a struct's host arrays (sifg_host_modified):
    a Grid, a Field, a ChainMesh, or None for every mirror."""
    lib = _lib.load()
    if obj is None:
        lib.sifg_host_modified(None)
        return
    c = obj._ptr.contents
    ptr = c.values if isinstance(obj, Grid) else c.x
    lib.sifg_host_modified(C.cast(ptr, C.c_void_p))
    if isinstance(obj, (Field, ChainMesh)) and c.weights:
        lib.sifg_host_modified(C.cast(c.weights, C.c_void_p))
    if isinstance(obj, ChainMesh):
        lib.sifg_host_modified(C.cast(c.cell_offsets, C.c_void_p))
        if c.cell_weights:
            lib.sifg_host_modified(C.cast(c.cell_weights, C.c_void_p))


def copy_bytes():
    """(host->device, device->host) bytes the C API has copied so far."""
    h2d, d2h = C.c_uint64(0), C.c_uint64(0)
    _lib.load().sifg_copy_bytes(C.byref(h2d), C.byref(d2h))
    return h2d.value, d2h.value


class Field:
    """Particle positions (float32, in [0, box)) and, optionally, per-particle
    weights (a mass, a luminosity, a selection weight; None: every particle
    counts 1), which the CIC deposit, the mesh and the finder all use."""

    def __init__(self, x, y, z, weights=None):
        lib = _lib.load()
        x, y, z = (np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z))
        if not (len(x) == len(y) == len(z)):
            raise ValueError("positions: x, y and z differ in length")
        self._ptr = lib.sif_field_alloc(len(x))
        if not self._ptr:
            raise MemoryError("field")
        _check(lib.sif_field_assign_positions(self._ptr, _P(x), _P(y), _P(z)), "Field")
        if weights is not None:
            w = np.ascontiguousarray(weights, dtype=np.float32)
            if w.shape != x.shape:
                raise ValueError("weights: not one per particle")
            _check(lib.sif_field_assign_weights(self._ptr, _P(w)), "Field")

    @property
    def n_particles(self):
        return self._ptr.contents.n_particles if self._ptr else 0

    @property
    def has_weights(self):
        return bool(self._ptr and self._ptr.contents.weights)

    @property
    def weights(self):
        """The weights (a copy), or None for an unweighted field."""
        if not self.has_weights:
            return None
        f = self._ptr.contents
        return np.ctypeslib.as_array(f.weights, shape=(f.n_particles,)).copy()

    def __del__(self):
        if getattr(self, "_ptr", None):
            _lib.load().sif_field_free(self._ptr)
            self._ptr = None


def field_from_numpy(x, y, z, *, weights=None):
    """pysif.field_from_numpy for Cartesian positions: a new Field with its
    particles (and weights, if given) copied out of the arrays."""
    return Field(x, y, z, weights=weights)


class Grid:
    """A cubic grid of n_cells^3 float32 cells over [0, box)^3."""

    def __init__(self, n_cells, box_length):
        lib = _lib.load()
        self._ptr = lib.sif_grid_alloc(n_cells, box_length)
        if not self._ptr:
            raise _lib.status_error(lib, lib.sif_error_status(), "Grid")

    @property
    def n_cells(self):
        return self._ptr.contents.n_cells

    @property
    def box_length(self):
        return self._ptr.contents.box_length

    @property
    def values(self):
        """A view of the cells, (n, n, n), x slowest."""
        g = self._ptr.contents
        return np.ctypeslib.as_array(g.values, shape=(g.n_cells,) * 3)

    def assign_cic(self, field):
        _check(_lib.load().sif_grid_assign_cic(self._ptr, field._ptr), "assign_cic")

    def to_density_contrast(self):
        _check(_lib.load().sif_grid_to_density_contrast(self._ptr), "to_density_contrast")

    def __del__(self):
        if getattr(self, "_ptr", None):
            _lib.load().sif_grid_free(self._ptr)
            self._ptr = None


class ChainMesh:
    """Particles grouped by cell (sif_chain_mesh_alloc)."""

    def __init__(self, n_cells, box_length, field, drop_indices=False, consume=False):
        lib = _lib.load()
        opt = abi.SIF_MESH_DROP_INDICES if drop_indices else 0
        fn = lib.sif_chain_mesh_alloc_consume if consume else lib.sif_chain_mesh_alloc
        self._ptr = fn(n_cells, box_length, field._ptr, opt)
        if not self._ptr:
            raise _lib.status_error(lib, lib.sif_error_status(), "ChainMesh")

    def arrays(self):
        m = self._ptr.contents
        n = m.n_particles

        def col(p):
            return np.ctypeslib.as_array(p, shape=(n,)).copy()

        offs = np.ctypeslib.as_array(m.cell_offsets, shape=(m.total_cells + 1,)).copy()
        idx = np.ctypeslib.as_array(m.original_indices, shape=(n,)).copy() \
            if m.original_indices else None
        return col(m.x), col(m.y), col(m.z), offs, idx

    @property
    def weights(self):
        """Per-particle weights in mesh order (a copy), or None unweighted."""
        m = self._ptr.contents
        return (np.ctypeslib.as_array(m.weights, shape=(m.n_particles,)).copy()
                if m.weights else None)

    @property
    def cell_weights(self):
        """Each cell's total weight (a copy), or None unweighted."""
        m = self._ptr.contents
        return (np.ctypeslib.as_array(m.cell_weights, shape=(m.total_cells,)).copy()
                if m.cell_weights else None)

    @property
    def total_weight(self):
        """The mesh's total weight (its tracer count when unweighted)."""
        return float(self._ptr.contents.total_weight)

    def __del__(self):
        if getattr(self, "_ptr", None):
            _lib.load().sif_chain_mesh_free(self._ptr)
            self._ptr = None


class Catalogue:
    """Void centres and radii (float32 arrays); a survey's also the observed
    fractions of each sphere and of its shell to twice the radius."""

    def __init__(self, cx, cy, cz, radii, footprint=None, footprint_shell=None):
        self.cx, self.cy, self.cz, self.radii = cx, cy, cz, radii
        self.footprint, self.footprint_shell = footprint, footprint_shell

    def __len__(self):
        return len(self.radii)

    def as_tuple(self):
        return self.cx, self.cy, self.cz, self.radii


def _take_catalogue(lib, ptr, what):
    if not ptr:
        raise _lib.status_error(lib, lib.sif_error_status(), what)
    cat = ptr.contents
    n = cat.n_voids
    cols = [np.ctypeslib.as_array(p, shape=(n,)).copy() if n else np.zeros(0, np.float32)
            for p in (cat.cx, cat.cy, cat.cz, cat.radii)]
    if cat.footprint:
        cols += [np.ctypeslib.as_array(p, shape=(n,)).copy() if n else np.zeros(0, np.float32)
                 for p in (cat.footprint, cat.footprint_shell)]
    lib.sif_catalogue_free(ptr)
    return Catalogue(*cols)


_VARIANTS = {"excursion-set": 0, "excursion-peak": 1, "lagrangian-overlap": 2}
_SEARCH = {1.5: abi.SIF_FINDER_SEARCH_1_50, 1.25: abi.SIF_FINDER_SEARCH_1_25,
           1.75: abi.SIF_FINDER_SEARCH_1_75, 2.0: abi.SIF_FINDER_SEARCH_2_00}


def _extras(checkpoint, prior, keep_checkpoint, save_memory, raw):
    """exodus_extras (python/src/finders/py_finders.c:222-270): checkpoint=
    None for a name of the run's own, a path, or False for none (the raw
    entry point only; a variant always checkpoints). Returns (extras or None,
    extra option bits, objects to keep alive)."""
    import os

    keep, opt, path = [], 0, None
    if checkpoint is False and raw:
        opt = abi.SIF_FINDER_NO_CHECKPOINT
    elif checkpoint is False:
        raise ValueError("checkpoint: False (expected a path, or None for a name of the run's "
                         "own: a variant always checkpoints; exodus_raw() runs without)")
    elif checkpoint is True:
        raise ValueError("checkpoint: True (expected a path, None for a name of the run's own, "
                         "or False for none)")
    elif checkpoint is not None:
        path = os.fsencode(checkpoint)
        keep.append(path)
    cat = None
    if prior is not None:
        cols = [np.ascontiguousarray(c, dtype=np.float32) for c in
                (prior.as_tuple() if isinstance(prior, Catalogue) else prior)]
        keep.extend(cols)
        cat = abi.sif_catalogue_t()
        cat.cx, cat.cy, cat.cz, cat.radii = (_P(c) for c in cols)
        cat.units = 0
        cat.n_voids = cat.capacity = len(cols[0])
        keep.append(cat)
    if path is None and cat is None and not keep_checkpoint and not save_memory:
        return None, opt, keep
    extras = abi.sif_finder_exodus_extras_t(path, C.pointer(cat) if cat is not None else None,
                                            int(bool(keep_checkpoint)), int(bool(save_memory)))
    return extras, opt, keep


def _exodus(grid, mesh, radii, threshold, variant="excursion-set", *, checkpoint=None,
            prior=None, keep_checkpoint=False, save_memory=False):
    """finders.exodus (python/pysif/finders.pyi:37-140): a variant, which
    checkpoints after every rung (to the named file, which it resumes if it
    exists, or to a name of its own, removed when the run succeeds)."""
    lib = _lib.load()
    if variant not in _VARIANTS:
        raise ValueError(f"variant: {variant!r}")
    radii = np.ascontiguousarray(radii, dtype=np.float32)
    extras, _, keep = _extras(checkpoint, prior, keep_checkpoint, save_memory, raw=False)
    ptr = lib.sif_finder_exodus(grid._ptr, mesh._ptr, _P(radii), len(radii), threshold,
                                _VARIANTS[variant], C.byref(extras) if extras is not None else None)
    del keep
    return _take_catalogue(lib, ptr, "exodus")


def _exodus_raw(grid, mesh, radii, threshold, overlap_fraction=0.0, *, overlap_type="eulerian",
                search_factor=1.5, deconvolution="full", consume_grid=False, seeds="cells",
                refine_centres="none", extend_reach=False, displace=False, checkpoint=False,
                prior=None, keep_checkpoint=False, save_memory=False):
    """finders.exodus_raw, for the options the GPU finder runs; checkpoint=
    False (the default here) runs without one."""
    lib = _lib.load()
    radii = np.ascontiguousarray(radii, dtype=np.float32)
    extras, opt, keep = _extras(checkpoint, prior, keep_checkpoint, save_memory, raw=True)
    opt |= _SEARCH[float(search_factor)]
    if overlap_type == "lagrangian":
        opt |= abi.SIF_FINDER_LAGRANGIAN_OVERLAP
    if deconvolution == "none":
        opt |= abi.SIF_FINDER_KEEP_CIC_WINDOW
    elif deconvolution == "aliasing":
        opt |= abi.SIF_FINDER_ALIASING_WINDOW
    if consume_grid:
        opt |= abi.SIF_FINDER_CONSUME_GRID
    if seeds == "minima":
        opt |= abi.SIF_FINDER_SEEDS_MINIMA
    elif seeds != "cells":
        raise ValueError(f"seeds must be 'cells' or 'minima', not {seeds!r}")
    refine = {None: 0, "none": 0, "gaussian": abi.SIF_FINDER_REFINE_GAUSSIAN,
              "tracers": abi.SIF_FINDER_REFINE_TRACERS, "hill": abi.SIF_FINDER_REFINE_HILL}
    if refine_centres not in refine:
        raise ValueError("refine_centres must be 'none', 'gaussian', 'tracers' or 'hill', "
                         f"not {refine_centres!r}")
    opt |= refine[refine_centres]
    if extend_reach:
        opt |= abi.SIF_FINDER_EXTEND_REACH
    if displace:
        opt |= abi.SIF_FINDER_DISPLACE
    ptr = lib.sif_finder_exodus_raw(grid._ptr, mesh._ptr, _P(radii), len(radii), threshold,
                                    overlap_fraction, opt,
                                    C.byref(extras) if extras is not None else None)
    del keep
    return _take_catalogue(lib, ptr, "exodus_raw")


def checkpoint_read(path):
    """sif_finder_exodus_checkpoint_read: (Catalogue, header fields as a dict)."""
    import os

    lib = _lib.load()
    h = abi.sif_finder_exodus_checkpoint_t()
    ptr = lib.sif_finder_exodus_checkpoint_read(os.fsencode(path), C.byref(h))
    cat = _take_catalogue(lib, ptr, "checkpoint_read")
    return cat, {f: getattr(h, f) for f, _ in abi.sif_finder_exodus_checkpoint_t._fields_
                 if f not in ("magic", "reserved", "offset")}


def _suggest_mesh_cells(n_particles, box_length, max_radius=0.0, volume=0.0):
    """pysif.finders.suggest_mesh_cells: sif_finder_suggest_mesh_cells
    (include/sif/finder/exodus_finder.h:653-683), the same rule: about 30
    tracers per cell, no coarser than the widest search stencil, 8..1024."""
    import math

    if n_particles <= 0 or not (box_length > 0) or not math.isfinite(box_length) or \
            not (volume >= 0) or not math.isfinite(volume):
        return 0
    whole = n_particles * box_length ** 3 / volume if volume > 0 else float(n_particles)
    cells = (whole / 30.0) ** (1.0 / 3.0)
    if max_radius > 0:
        if 2.0 * max_radius >= box_length:
            return 0
        cells = max(cells, box_length / (box_length - 2.0 * max_radius) + 1.0)
    return int(min(max(cells, 8.0), 1024.0))


def _survey_opt(overlap_type, search_factor, deconvolution):
    opt = _SEARCH[float(search_factor)]
    if overlap_type == "lagrangian":
        opt |= abi.SIF_FINDER_LAGRANGIAN_OVERLAP
    if deconvolution == "none":
        opt |= abi.SIF_FINDER_KEEP_CIC_WINDOW
    elif deconvolution == "aliasing":
        opt |= abi.SIF_FINDER_ALIASING_WINDOW
    return opt


def _offset_arg(offset):
    if offset is None:
        return None, None
    o = np.ascontiguousarray(offset, dtype=np.float32)
    assert o.shape == (3,)
    return o, _P(o)


def _exodus_survey_raw(data_grid, random_grid, data_mesh, random_mesh, radii, threshold,
                       overlap_fraction=0.0, *, offset=None, overlap_type="eulerian",
                       search_factor=1.5, deconvolution="full", checkpoint=False, prior=None,
                       keep_checkpoint=False):
    """finders.exodus_survey_raw (sif_finder_exodus_survey_raw): grids hold
    the CIC densities of data and randoms; offset what the survey was moved
    into the box by. The catalogue comes back in the caller's frame with its
    footprint columns."""
    lib = _lib.load()
    radii = np.ascontiguousarray(radii, dtype=np.float32)
    extras, opt, keep = _extras(checkpoint, prior, keep_checkpoint, False, raw=True)
    opt |= _survey_opt(overlap_type, search_factor, deconvolution)
    o, op = _offset_arg(offset)
    ptr = lib.sif_finder_exodus_survey_raw(data_grid._ptr, random_grid._ptr, data_mesh._ptr,
                                           random_mesh._ptr, op, _P(radii), len(radii), threshold,
                                           overlap_fraction, opt,
                                           C.byref(extras) if extras is not None else None)
    del keep, o
    return _take_catalogue(lib, ptr, "exodus_survey_raw")


def _exodus_survey(data_grid, random_grid, data_mesh, random_mesh, radii, threshold,
                   variant="excursion-set", *, offset=None, checkpoint=None, prior=None,
                   keep_checkpoint=False):
    """finders.exodus_survey (sif_finder_exodus_survey): a variant."""
    lib = _lib.load()
    if variant not in _VARIANTS:
        raise ValueError(f"variant: {variant!r}")
    radii = np.ascontiguousarray(radii, dtype=np.float32)
    extras, _, keep = _extras(checkpoint, prior, keep_checkpoint, False, raw=False)
    o, op = _offset_arg(offset)
    ptr = lib.sif_finder_exodus_survey(data_grid._ptr, random_grid._ptr, data_mesh._ptr,
                                       random_mesh._ptr, op, _P(radii), len(radii), threshold,
                                       _VARIANTS[variant],
                                       C.byref(extras) if extras is not None else None)
    del keep, o
    return _take_catalogue(lib, ptr, "exodus_survey")


def _survey_box(data, randoms, radii, search_factor=1.5):
    """finders.survey_box (sif_finder_exodus_survey_box): (offset, box_length)
    for Fields in the survey's own frame."""
    lib = _lib.load()
    radii = np.ascontiguousarray(radii, dtype=np.float32)
    off = np.zeros(3, np.float32)
    L = C.c_float(0.0)
    _check(lib.sif_finder_exodus_survey_box(data._ptr, randoms._ptr, _P(radii), len(radii),
                                            _SEARCH[float(search_factor)], _P(off), C.byref(L)),
           "survey_box")
    return off, float(L.value)


finders = types.SimpleNamespace(exodus=_exodus, exodus_raw=_exodus_raw,
                                exodus_survey=_exodus_survey, exodus_survey_raw=_exodus_survey_raw,
                                survey_box=_survey_box, suggest_mesh_cells=_suggest_mesh_cells,
                                checkpoint_read=checkpoint_read)


def smoothed_contrast(x, y, z, n_grid, box, radius, filter="gaussian", window="full"):
    """The CIC density contrast of torch CUDA positions smoothed at `radius`,
    differentiable with respect to the positions (a torch.autograd.Function,
    sif_gb300.autograd.SmoothedContrast). Not in the reference's pysif, which
    has no gradients; an addition beside its names."""
    from . import autograd

    return autograd.smoothed_contrast(x, y, z, n_grid, box, radius, filter, window)
