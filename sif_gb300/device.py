"""Device-resident entry points over torch CUDA tensors.

torch only allocates and holds the device memory here; every stage is a call
into libsif_gb300.so (include/sif_gb300.h, part 2) with raw device pointers.
float64 inputs select the FP64 form (the `_f64` entry points, the reference's
SIF_USE_DOUBLE arithmetic); float32 inputs the float form.

The library runs on its own streams and returns once its results are
complete; before each call the torch stream that produced the inputs is
drained, since nothing else orders the library's reads after torch's writes.
"""
import ctypes as C
import threading

import numpy as np

from . import _lib, abi


def _ptr(t):
    if t is None:
        return None
    assert t.is_cuda and t.is_contiguous(), "expected a contiguous CUDA tensor"
    return C.c_void_p(t.data_ptr())


def _form(t):
    """(entry-point suffix, torch dtype, numpy dtype) of a tensor's form."""
    import torch

    if t.dtype == torch.float64:
        return "_f64", torch.float64, np.float64
    assert t.dtype == torch.float32, f"expected float32 or float64, got {t.dtype}"
    return "", torch.float32, np.float32


def _fn(name, t):
    """The entry point for t's form, once torch's work on t's device is done."""
    import torch

    if t.is_cuda:
        torch.cuda.current_stream(t.device).synchronize()
    return getattr(_lib.load(), name + _form(t)[0])


def _check(status, what):
    if status != abi.SIF_OK:
        raise _lib.status_error(_lib.load(), status, what)


def cic(x, y, z, n_grid, box):
    import torch

    grid = torch.empty(n_grid ** 3, dtype=_form(x)[1], device=x.device)
    _check(_fn("sifg_cic_device", x)(_ptr(x), _ptr(y), _ptr(z), x.numel(), n_grid, box,
                                     _ptr(grid)), "cic")
    return grid


def density_contrast(grid):
    mean = C.c_double(0.0)
    _check(_fn("sifg_contrast_device", grid)(_ptr(grid), grid.numel(), C.byref(mean)), "contrast")
    return mean.value


def chain_mesh(x, y, z, n_cells, box, with_indices=True):
    import torch

    n = x.numel()
    dev = x.device
    mx = torch.empty(n, dtype=_form(x)[1], device=dev)
    my = torch.empty_like(mx)
    mz = torch.empty_like(mx)
    offs = torch.empty(n_cells ** 3 + 1, dtype=torch.int32, device=dev)
    orig = torch.empty(n, dtype=torch.int32, device=dev) if with_indices else None
    _check(_fn("sifg_mesh_device", x)(_ptr(x), _ptr(y), _ptr(z), n, n_cells, box, _ptr(mx),
                                      _ptr(my), _ptr(mz), _ptr(offs), _ptr(orig)), "chain_mesh")
    return mx, my, mz, offs, orig


def cic_weighted(x, y, z, w, n_grid, box):
    """The CIC density of weighted device particles (one weight each)."""
    import torch

    grid = torch.empty(n_grid ** 3, dtype=_form(x)[1], device=x.device)
    _check(_fn("sifg_cic_weighted_device", x)(_ptr(x), _ptr(y), _ptr(z), _ptr(w), x.numel(),
                                              n_grid, box, _ptr(grid)), "cic_weighted")
    return grid


def mesh_weights(field_w, mesh, n_cells):
    """A mesh's weight columns from the field's weights: (w in mesh order,
    per-cell sums, total). mesh = chain_mesh(..., with_indices=True)."""
    import torch

    offs, orig = mesh[3], mesh[4]
    w = torch.empty_like(field_w)
    cw = torch.empty(n_cells ** 3, dtype=field_w.dtype, device=field_w.device)
    tot = C.c_double(0.0)
    _check(_fn("sifg_mesh_weights_device", field_w)(_ptr(field_w), _ptr(orig), field_w.numel(),
                                                    _ptr(offs), n_cells, _ptr(w), _ptr(cw),
                                                    C.byref(tot)), "mesh_weights")
    return w, cw, tot.value


def contrast_vjp(x, y, z, n_grid, box, g):
    """dL/dx, dL/dy, dL/dz for g = dL/d(delta), delta the CIC density contrast."""
    import torch

    gx, gy, gz = (torch.empty_like(x) for _ in range(3))
    _check(_fn("sifg_contrast_vjp_device", x)(_ptr(x), _ptr(y), _ptr(z), x.numel(), n_grid, box,
                                              _ptr(g), _ptr(gx), _ptr(gy), _ptr(gz)),
           "contrast_vjp")
    return gx, gy, gz


def smooth(delta, n_grid, box, radius, filter="top-hat", window="full"):
    import torch

    out = torch.empty(n_grid ** 3, dtype=_form(delta)[1], device=delta.device)
    f = {"top-hat": 1, "gaussian": 2}[filter]
    w = {"none": 0, "full": 1, "aliasing": 2}[window]
    _check(_fn("sifg_smooth_device", delta)(_ptr(delta), n_grid, box, radius, f, w, _ptr(out)),
           "smooth")
    return out


_scratch = threading.local()


def _catalogue_arrays(cap, dtype=np.float32):
    """Four output columns for the library to fill; kept per thread between
    calls (callers get copies): fresh arrays of this size cost more in page
    faults than the run's own host work."""
    key = (cap, np.dtype(dtype).str)
    cols = getattr(_scratch, "cols", {}).get(key)
    if cols is None:
        cols = [np.empty(cap, dtype) for _ in range(4)]
        _scratch.cols = {key: cols}
    return cols


def exodus(delta, n_grid, box, mesh, mesh_cells, radii, threshold, overlap=0.0, options=0,
           inject=None, capacity=1 << 22, prior=None, weights=None):
    """The finder on device data. mesh = (mx, my, mz, offsets, ...);
    prior: (cx, cy, cz, r) host arrays, voids to start from; weights: a
    weighted mesh's (w, cell_w, total_weight), as mesh_weights gives them."""
    _, _, nt = _form(delta)
    radii = np.ascontiguousarray(radii, dtype=nt)
    cols = _catalogue_arrays(capacity, nt)
    n = C.c_uint64(0)
    mx, my, mz, offs = mesh[:4]
    packed = np.ascontiguousarray(np.concatenate([np.asarray(c, nt) for c in prior])) \
        if prior is not None else None
    n_prior = len(prior[0]) if prior is not None else 0
    tail = (radii.ctypes.data_as(C.c_void_p), len(radii), threshold, overlap, options,
            _ptr(inject), packed.ctypes.data_as(C.c_void_p) if packed is not None else None,
            n_prior, *[c.ctypes.data_as(C.c_void_p) for c in cols], capacity, C.byref(n))
    if weights is None:
        st = _fn("sifg_exodus_device", delta)(_ptr(delta), n_grid, box, _ptr(mx), _ptr(my),
                                              _ptr(mz), _ptr(offs), mx.numel(), mesh_cells, *tail)
    else:
        w, cw, tot = weights
        st = _fn("sifg_exodus_weighted_device", delta)(
            _ptr(delta), n_grid, box, _ptr(mx), _ptr(my), _ptr(mz), _ptr(offs), _ptr(w), _ptr(cw),
            float(tot), mx.numel(), mesh_cells, *tail)
    _check(st, "exodus")
    return tuple(c[: n.value].copy() for c in cols)


def exodus_survey(data_density, random_density, n_grid, box, data_mesh, random_mesh, radii,
                  threshold, overlap=0.0, options=0, inject=None, capacity=1 << 20, prior=None):
    """The survey finder on device data (sifg_exodus_survey_device), in the
    box's frame. data_mesh / random_mesh: (mx, my, mz, offsets, mesh_cells,
    total_weight) or with (w, cell_w) after them for a weighted mesh;
    inject: 2 fields a rung (data, randoms). Returns (cx, cy, cz, r,
    footprint, footprint_shell)."""
    radii = np.ascontiguousarray(radii, dtype=np.float32)
    cols = tuple(_catalogue_arrays(capacity, np.float32)) + \
        (np.empty(capacity, np.float32), np.empty(capacity, np.float32))
    n = C.c_uint64(0)

    def addr(t):
        if t is None:
            return None
        assert t.is_cuda and t.is_contiguous(), "expected a contiguous CUDA tensor"
        return t.data_ptr()

    def dmesh(m):
        mx, my, mz, offs, cells, tot = m[:6]
        w = m[6] if len(m) > 6 else None
        cw = m[7] if len(m) > 7 else None
        return _lib.DeviceMesh(addr(mx), addr(my), addr(mz), addr(offs), addr(w), addr(cw),
                               float(tot), mx.numel(), cells)

    dm, rm = dmesh(data_mesh), dmesh(random_mesh)
    packed = np.ascontiguousarray(np.concatenate([np.asarray(c, np.float32) for c in prior])) \
        if prior is not None else None
    st = _lib.load().sifg_exodus_survey_device(
        _ptr(data_density), _ptr(random_density), n_grid, box, C.byref(dm), C.byref(rm),
        radii.ctypes.data_as(C.c_void_p), len(radii), threshold, overlap, options, _ptr(inject),
        packed.ctypes.data_as(C.c_void_p) if packed is not None else None,
        len(prior[0]) if prior is not None else 0, *[c.ctypes.data_as(C.c_void_p) for c in cols],
        capacity, C.byref(n))
    _check(st, "exodus_survey")
    return tuple(c[: n.value].copy() for c in cols)


def box(x, y, z, n_grid, box_length, mesh_cells, radii, threshold, overlap=0.0, options=0,
        capacity=1 << 22):
    """The whole path on device particles: CIC, contrast, mesh, finder."""
    _, _, nt = _form(x)
    radii = np.ascontiguousarray(radii, dtype=nt)
    cols = _catalogue_arrays(capacity, nt)
    n = C.c_uint64(0)
    st = _fn("sifg_box_device", x)(_ptr(x), _ptr(y), _ptr(z), x.numel(), n_grid, box_length, mesh_cells,
                             radii.ctypes.data_as(C.c_void_p), len(radii), threshold, overlap,
                             options, *[c.ctypes.data_as(C.c_void_p) for c in cols], capacity,
                             C.byref(n))
    _check(st, "box")
    return tuple(c[: n.value].copy() for c in cols)


def last_rung_stats():
    lib = _lib.load()
    arr = (_lib.RungStat * 256)()
    k = lib.sifg_last_rung_stats(arr, 256)
    return [{f: getattr(arr[i], f) for f, _ in _lib.RungStat._fields_} for i in range(min(k, 256))]


def last_timings():
    t = _lib.Timings()
    _lib.load().sifg_last_timings(C.byref(t))
    return {f: getattr(t, f) for f, _ in _lib.Timings._fields_}


TRACE_KINDS = ("growth", "filter", "cic", "mesh", "witness", "commit", "smoothing", "rung",
               "cic_stage")


def last_trace():
    """The last run's timeline (sifg_last_trace): (kind, start_ms, end_ms)
    spans after the run's first event, kind by kind in the order recorded."""
    lib = _lib.load()
    n = lib.sifg_last_trace(None, 0)
    buf = (_lib.TraceEvent * max(n, 1))()
    n = min(n, lib.sifg_last_trace(buf, n))
    return [(TRACE_KINDS[e.kind], e.start_ms, e.end_ms) for e in buf[:n]]


def stream():
    """The library's CUDA stream as a torch stream, for events on it."""
    import torch

    return torch.cuda.ExternalStream(_lib.load().sifg_stream())


def launch_count():
    return int(_lib.load().sifg_launch_count())


def set_growth_mode(mode):
    """0 by survivor count, 1 a CTA per survivor, 2 a warp per survivor."""
    _lib.load().sifg_set_growth_mode(int(mode))


def set_shell_list(entries):
    """The warp growth's shell list: -1 sized per rung, 0 none, n entries."""
    _lib.load().sifg_set_shell_list(int(entries))


def set_commit_mode(mode):
    """0 the commit's rounds in one cooperative launch, 1 a launch per round."""
    _lib.load().sifg_set_commit_mode(int(mode))


def set_scan_mode(mode):
    """0 the candidates from the smoothing's below-threshold list where it
    makes one, 1 a scan of the whole field every rung."""
    _lib.load().sifg_set_scan_mode(int(mode))


def set_witness(on):
    """1 the collision witness refuses doomed survivors before growth, 0 (the
    default) every survivor is grown; the catalogue is the same."""
    _lib.load().sifg_set_witness(int(on))


def set_factor_tables(on):
    """1 the 512^3 filter pass reads per-smoothing factor tables, 0 it
    evaluates the factors; the same bits either way."""
    _lib.load().sifg_set_factor_tables(int(on))


def set_window(bins):
    _lib.load().sifg_set_window(int(bins))


def box_batch(boxes, engines=0, capacity=1 << 20, check=True):
    """The batched form: boxes = [dict(x, y, z, n_grid, box, radii, threshold,
    mesh_cells=0, overlap=0.0, options=0)], particles as float32 CUDA tensors.
    Returns (catalogues, engines used); each catalogue is what box() returns
    for that box alone."""
    import torch

    lib = _lib.load()
    if boxes and boxes[0]["x"].is_cuda:
        torch.cuda.current_stream(boxes[0]["x"].device).synchronize()
    jobs = (_lib.BoxJob * len(boxes))()
    keep = []
    for j, b in zip(jobs, boxes):
        radii = np.ascontiguousarray(b["radii"], dtype=np.float32)
        cols = [np.empty(capacity, np.float32) for _ in range(4)]  # one set per job
        keep.append((radii, cols))
        j.x, j.y, j.z = (b[k].data_ptr() for k in ("x", "y", "z"))
        j.n_particles = b["x"].numel()
        j.n_grid, j.box = b["n_grid"], b["box"]
        j.mesh_cells = b.get("mesh_cells", 0)
        j.radii, j.n_radii = radii.ctypes.data, len(radii)
        j.threshold, j.overlap, j.options = b["threshold"], b.get("overlap", 0.0), b.get("options", 0)
        j.cx, j.cy, j.cz, j.r = (c.ctypes.data for c in cols)
        j.capacity = capacity
    used = C.c_uint32(0)
    st = lib.sifg_box_batch_device(jobs, len(boxes), engines, C.byref(used))
    if check:
        _check(st, "box_batch")
    cats = [tuple(c[: min(j.n_voids, capacity)].copy() for c in cols)
            for j, (_, cols) in zip(jobs, keep)]
    if not check:
        return cats, used.value, [j.status for j in jobs]
    return cats, used.value
