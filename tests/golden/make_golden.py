"""Generates the golden vectors under tests/golden/ from the reference itself.

Run in a checkout where the reference sif is compiled (``make -C oracle ref``,
which needs the reference sources); the GPU machines only read the .npz
files this writes.

golden_box32.npz -- a 32^3 Zel'dovich box (side 128, rms displacement 4,
  seed 11), ladder(8, 24, 0.1), threshold -0.7, a mesh of 8^3 cells:
  the positions; the reference's CIC density and density contrast
  (sif_grid_assign_cic, sif_grid_to_density_contrast); its chain mesh
  (positions, offsets, source indices); the 12 per-rung smoothed fields its
  own run produced (captured from sif__fft_grid_backward); and its catalogue
  for several option sets (SIF_FINDER_SEEDS_MINIMA among them), each run on
  exactly those fields.

golden_box32_f64.npz -- the same box through the reference's SIF_USE_DOUBLE
  build (sif_real = double): the float positions moved by a seeded jitter of
  up to 1e-4 so that they need double precision, and the same records in
  double (density, contrast, mesh, 12 captured fields, catalogues).

golden_box32_displace.npz, golden_box32_displace_f64.npz -- the same
  positions (the f64 file with the same jitter) at threshold -0.3 and
  ladder(3, 6, 0.1) (8 rungs), where SIF_FINDER_DISPLACE changes the
  catalogue: the excursion-peak preset (minima seeds, extended reach,
  displacement, overlap fraction 1), the same less its displacement, and
  displacement with cell seeds (overlap 0 and 0.5), with minima at 0.5 and
  with the Lagrangian overlap. The contrast, the mesh, the 8 fields the
  reference's own run smoothed, and its catalogues on them.

golden_workload_a.npz -- workload A itself: 128^3 particles (synth.workload_particles
  ("A"): box 500, rms displacement 4, seed 1001), grid 128^3, mesh 50^3,
  ladder(5, 30, 0.10) (19 rungs), threshold -0.8. The reference's whole path
  on its own (CIC in float, contrast, mesh, the shim's FFT), and its
  catalogue; the positions are not stored (25 MB), only the SHA-256 of their
  float32 bytes, so that a test regenerating them on another machine fails
  loudly where the generator does not give the same bits there.

golden_box32_extend.npz, golden_box32_extend_f64.npz -- the same positions
  (the f64 file with the same jitter) at a shallow threshold, -0.3, and the
  ladder(4, 8, 0.1) (8 rungs), where SIF_FINDER_EXTEND_REACH changes the
  catalogue: with minima seeds and an overlap fraction of 1 (the
  excursion-peak preset less its displacement) it changes 61 of 355 radii.
  The contrast, the mesh, the 8 fields the reference's own run smoothed, and
  its catalogues with and without the extended reach.
golden_box32_weighted.npz, golden_box32_weighted_f64.npz -- weighted meshes
  (sif_field_assign_weights on both the grid's field and the mesh's). Two
  sets, each through the reference's whole path at threshold -0.7 and
  ladder(8, 24, 0.15) (8 rungs): "rand", BOX32's positions (the f64 file
  with its jitter) with seeded weights, a fifth of them 0 and the rest
  uniform in [0.5, 1.5) as float32; "holes" (float file only), 32^3
  uniform positions whose weights are 0 inside three spheres and 1
  elsewhere, so that the voids exist only in the weights. Per set: the
  positions and weights, the weighted contrast, the mesh with its weight
  columns (weights in mesh order, per-cell sums, total), the 8 fields the
  reference's own run smoothed, and its catalogues for several option sets
  on them. The generator also checks that weights of 1 and of 4 give the
  unweighted catalogue bit for bit, as the reference's own test does.
golden_box32_refine.npz, golden_box32_refine_f64.npz -- SIF_FINDER_REFINE_GAUSSIAN
  on BOX32's positions (the f64 file with its jitter), threshold -0.7 and
  ladder(8, 24, 0.1) (12 rungs): the rungs' top-hat fields and the
  refinement's fields (the top-hat times a Gaussian of 0.15 of the rung) the
  reference's own runs returned, and for each option set the refinement
  takes (three in the f64 file) which rungs ran the refinement's transform
  (those with candidates) and its catalogue on those fields.
golden_survey.npz -- the survey finder (sif_finder_exodus_survey_raw) on
  synth.survey's footprint (a ball of radius 140 inside a box of 400, less a
  stripe, four holes carved into the data, one cut by the edge): 60,000 data
  and 600,000 randoms (180,000 in "sparse", whose footprint needs its chance
  holes closed), under a selection falling along z ("flat": none), grid 64^3,
  meshes of 20^3. Cases by threshold and ladder: [30, 24, 19, 15] at -0.8;
  ladder(10, 30, 0.1) at -0.5 (also weighted -- data weights uniform in
  [0.5, 1.5), a fifth 0, randoms 2 each -- and with the Lagrangian overlap);
  ladder(8, 24, 0.1) at -0.3; and "offset", the survey moved to its own frame
  and placed by sif_finder_exodus_survey_box (grid 64^3 over the box it
  gives). Per case the reference's catalogue with its footprint columns,
  from its whole path (float CIC of both sets, the shim's transforms); the
  positions are not stored, only the SHA-256 of their float32 bytes.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from sif_gb300 import abi, synth  # noqa: E402

import ref_ctypes as R  # noqa: E402

sys.path.insert(0, os.path.join(ROOT, "tests"))
from survey_cases import (SURVEY_CASES, SURVEY_GRID, SURVEY_MESH, survey_inputs,  # noqa: E402
                          survey_sha256)

# Option sets the catalogue is recorded for: (name, overlap_fraction, options).
OPTION_SETS = [
    ("default", 0.0, 0),
    ("search_2_00", 0.0, abi.SIF_FINDER_SEARCH_2_00),
    ("search_1_25", 0.0, abi.SIF_FINDER_SEARCH_1_25),
    ("lagrangian", 0.0, abi.SIF_FINDER_LAGRANGIAN_OVERLAP),
    ("overlap_0_5", 0.5, 0),
    ("minima", 0.0, abi.SIF_FINDER_SEEDS_MINIMA),
]

BOX32 = dict(n=32, box=128.0, rms_disp=4.0, seed=11, r0=8.0, threshold=-0.7, mesh=8)


def make_box32(path):
    p = BOX32
    x, y, z = synth.zeldovich(p["n"], p["box"], p["rms_disp"], p["seed"])
    radii = synth.ladder(p["r0"], 3 * p["r0"], 0.1).astype(np.float32)
    lib = R.load("strict", 4, abi.SIF_LOG_LEVEL_ERROR)
    f = R.RefField(lib, x, y, z)
    g = R.RefGrid(lib, p["n"], p["box"])
    g.assign_cic(f)
    density = g.values()
    g.to_contrast()
    delta = g.values()
    m = R.RefMesh(lib, p["mesh"], p["box"], f)
    mx, my, mz, offs, idx = m.arrays()
    fields = np.zeros((len(radii), p["n"] ** 3), np.float32)
    cat = R.exodus_raw(lib, g, m, radii, p["threshold"], capture=fields)
    out = dict(x=x, y=y, z=z, radii=radii, density=density, delta=delta, mesh_x=mx, mesh_y=my,
               mesh_z=mz, mesh_offsets=offs, mesh_index=idx, fields=fields,
               params=np.array([p["n"], p["box"], p["rms_disp"], p["seed"], p["r0"],
                                p["threshold"], p["mesh"]], np.float64))
    for name, overlap, opt in OPTION_SETS:
        c = R.exodus_raw(lib, g, m, radii, p["threshold"], overlap, opt, inject=fields)
        for k, col in zip(("cx", "cy", "cz", "r"), c):
            out[f"cat_{name}_{k}"] = col
        out[f"cat_{name}_opt"] = np.array([overlap, opt], np.float64)
    # The default run on its own fields is the run that captured them.
    assert all(np.array_equal(a, out[f"cat_default_{k}"]) for a, k in zip(cat, "cx cy cz r".split()))
    # A prior catalogue (sif_finder_exodus_extras_t::prior): the ten largest
    # voids of the search-2.0 run, given to a default run, which returns them
    # first and adds what respects them.
    order = np.argsort(-out["cat_search_2_00_r"], kind="stable")[:10]
    prior = tuple(out[f"cat_search_2_00_{k}"][order] for k in ("cx", "cy", "cz", "r"))
    c = R.exodus_raw(lib, g, m, radii, p["threshold"], inject=fields, prior=prior)
    for k, col, pc in zip(("cx", "cy", "cz", "r"), c, prior):
        out[f"prior_{k}"] = pc
        out[f"cat_prior_{k}"] = col
    m.free()
    g.free()
    f.free()
    np.savez_compressed(path, **out)
    print(f"{path}: {len(cat[0])} voids over {len(radii)} rungs; with the prior {len(c[0])}")


def make_box32_f64(path):
    p = BOX32
    x32, y32, z32 = synth.zeldovich(p["n"], p["box"], p["rms_disp"], p["seed"])
    rng = np.random.default_rng(p["seed"] + 1000)

    def jitter(a):
        v = a.astype(np.float64) + rng.uniform(-1e-4, 1e-4, a.shape)
        v = np.where(v < 0.0, v + p["box"], v)
        return np.where(v >= p["box"], v - p["box"], v)

    x, y, z = jitter(x32), jitter(y32), jitter(z32)
    radii = synth.ladder(p["r0"], 3 * p["r0"], 0.1).astype(np.float64)
    v = "f64"
    lib = R.load(v, 4, abi.SIF_LOG_LEVEL_ERROR)
    f = R.RefField(lib, x, y, z, variant=v)
    g = R.RefGrid(lib, p["n"], p["box"], variant=v)
    g.assign_cic(f)
    density = g.values()
    g.to_contrast()
    delta = g.values()
    m = R.RefMesh(lib, p["mesh"], p["box"], f)
    mx, my, mz, offs, idx = m.arrays(variant=v)
    fields = np.zeros((len(radii), p["n"] ** 3), np.float64)
    cat = R.exodus_raw(lib, g, m, radii, p["threshold"], variant=v, capture=fields)
    out = dict(x=x, y=y, z=z, radii=radii, density=density, delta=delta, mesh_x=mx, mesh_y=my,
               mesh_z=mz, mesh_offsets=offs, mesh_index=idx, fields=fields,
               params=np.array([p["n"], p["box"], p["rms_disp"], p["seed"], p["r0"],
                                p["threshold"], p["mesh"]], np.float64))
    for name, overlap, opt in OPTION_SETS:
        c = R.exodus_raw(lib, g, m, radii, p["threshold"], overlap, opt, variant=v, inject=fields)
        for k, col in zip(("cx", "cy", "cz", "r"), c):
            out[f"cat_{name}_{k}"] = col
        out[f"cat_{name}_opt"] = np.array([overlap, opt], np.float64)
    assert all(np.array_equal(a, out[f"cat_default_{k}"]) for a, k in zip(cat, "cx cy cz r".split()))
    m.free()
    g.free()
    f.free()
    np.savez_compressed(path, **out)
    print(f"{path}: {len(cat[0])} voids over {len(radii)} rungs")


# The extended reach's box: BOX32's positions at a shallow threshold and a
# short ladder, and the option sets that differ by SIF_FINDER_EXTEND_REACH.
EXTEND = dict(BOX32, threshold=-0.3, r0=4.0, top=2.0)
EXTEND_SETS = [
    ("minima_f1", 1.0, abi.SIF_FINDER_SEEDS_MINIMA),
    ("extend_minima_f1", 1.0, abi.SIF_FINDER_SEEDS_MINIMA | abi.SIF_FINDER_EXTEND_REACH),
    ("extend_f1", 1.0, abi.SIF_FINDER_EXTEND_REACH),
    ("extend", 0.0, abi.SIF_FINDER_EXTEND_REACH),
]


def make_box32_extend(path, v="strict"):
    p = EXTEND
    x, y, z = synth.zeldovich(p["n"], p["box"], p["rms_disp"], p["seed"])
    real = np.float32
    if v == "f64":
        rng = np.random.default_rng(p["seed"] + 1000)  # BOX32's f64 jitter

        def jitter(a):
            w = a.astype(np.float64) + rng.uniform(-1e-4, 1e-4, a.shape)
            w = np.where(w < 0.0, w + p["box"], w)
            return np.where(w >= p["box"], w - p["box"], w)

        x, y, z = jitter(x), jitter(y), jitter(z)
        real = np.float64
    radii = synth.ladder(p["r0"], p["top"] * p["r0"], 0.1).astype(real)
    lib = R.load(v, 4, abi.SIF_LOG_LEVEL_ERROR)
    kw = dict(variant=v) if v == "f64" else {}
    f = R.RefField(lib, x, y, z, **kw)
    g = R.RefGrid(lib, p["n"], p["box"], **kw)
    g.assign_cic(f)
    g.to_contrast()
    delta = g.values()
    m = R.RefMesh(lib, p["mesh"], p["box"], f)
    mx, my, mz, offs, idx = m.arrays(**kw)
    fields = np.zeros((len(radii), p["n"] ** 3), real)
    R.exodus_raw(lib, g, m, radii, p["threshold"], capture=fields, **kw)
    out = dict(x=x, y=y, z=z, radii=radii, delta=delta, mesh_x=mx, mesh_y=my, mesh_z=mz,
               mesh_offsets=offs, mesh_index=idx, fields=fields,
               params=np.array([p["n"], p["box"], p["rms_disp"], p["seed"], p["r0"],
                                p["threshold"], p["mesh"]], np.float64))
    for name, overlap, opt in EXTEND_SETS:
        c = R.exodus_raw(lib, g, m, radii, p["threshold"], overlap, opt, inject=fields, **kw)
        for k, col in zip(("cx", "cy", "cz", "r"), c):
            out[f"cat_{name}_{k}"] = col
        out[f"cat_{name}_opt"] = np.array([overlap, opt], np.float64)
    a, b = out["cat_minima_f1_r"], out["cat_extend_minima_f1_r"]
    assert len(a) != len(b) or not np.array_equal(a, b), "the extended reach changes nothing here"
    m.free()
    g.free()
    f.free()
    np.savez_compressed(path, **out)
    print(f"{path}: " + ", ".join(f"{n} {len(out[f'cat_{n}_r'])}" for n, _, _ in EXTEND_SETS))


DISPLACE = dict(BOX32, threshold=-0.3, r0=3.0, top=2.0)
DISPLACE_SETS = [
    ("peak", 1.0, abi.SIF_FINDER_SEEDS_MINIMA | abi.SIF_FINDER_EXTEND_REACH | abi.SIF_FINDER_DISPLACE),
    ("peak_no_displace", 1.0, abi.SIF_FINDER_SEEDS_MINIMA | abi.SIF_FINDER_EXTEND_REACH),
    ("cells_f0", 0.0, abi.SIF_FINDER_DISPLACE),
    ("cells_f05", 0.5, abi.SIF_FINDER_DISPLACE),
    ("minima_f05", 0.5, abi.SIF_FINDER_SEEDS_MINIMA | abi.SIF_FINDER_DISPLACE),
    ("lagrangian", 0.0, abi.SIF_FINDER_LAGRANGIAN_OVERLAP | abi.SIF_FINDER_DISPLACE),
]


def make_box32_displace(path, v="strict"):
    p = DISPLACE
    x, y, z = synth.zeldovich(p["n"], p["box"], p["rms_disp"], p["seed"])
    real = np.float32
    if v == "f64":
        rng = np.random.default_rng(p["seed"] + 1000)  # BOX32's f64 jitter

        def jitter(a):
            w = a.astype(np.float64) + rng.uniform(-1e-4, 1e-4, a.shape)
            w = np.where(w < 0.0, w + p["box"], w)
            return np.where(w >= p["box"], w - p["box"], w)

        x, y, z = jitter(x), jitter(y), jitter(z)
        real = np.float64
    radii = synth.ladder(p["r0"], p["top"] * p["r0"], 0.1).astype(real)
    lib = R.load(v, 4, abi.SIF_LOG_LEVEL_ERROR)
    kw = dict(variant=v) if v == "f64" else {}
    f = R.RefField(lib, x, y, z, **kw)
    g = R.RefGrid(lib, p["n"], p["box"], **kw)
    g.assign_cic(f)
    g.to_contrast()
    delta = g.values()
    m = R.RefMesh(lib, p["mesh"], p["box"], f)
    mx, my, mz, offs, idx = m.arrays(**kw)
    fields = np.zeros((len(radii), p["n"] ** 3), real)
    R.exodus_raw(lib, g, m, radii, p["threshold"], capture=fields, **kw)
    out = dict(x=x, y=y, z=z, radii=radii, delta=delta, mesh_x=mx, mesh_y=my, mesh_z=mz,
               mesh_offsets=offs, mesh_index=idx, fields=fields,
               params=np.array([p["n"], p["box"], p["rms_disp"], p["seed"], p["r0"],
                                p["threshold"], p["mesh"]], np.float64))
    for name, overlap, opt in DISPLACE_SETS:
        c = R.exodus_raw(lib, g, m, radii, p["threshold"], overlap, opt, inject=fields, **kw)
        for k, col in zip(("cx", "cy", "cz", "r"), c):
            out[f"cat_{name}_{k}"] = col
        out[f"cat_{name}_opt"] = np.array([overlap, opt], np.float64)
    a, b = out["cat_peak_r"], out["cat_peak_no_displace_r"]
    assert len(a) != len(b) or not np.array_equal(a, b), "displacement changes nothing here"
    m.free()
    g.free()
    f.free()
    np.savez_compressed(path, **out)
    print(f"{path}: " + ", ".join(f"{n} {len(out[f'cat_{n}_r'])}" for n, _, _ in DISPLACE_SETS))


WEIGHTED = dict(BOX32, r0=8.0, top=3.0, step=0.15)
WEIGHTED_SETS = [
    ("default", 0.0, 0),
    ("minima", 0.0, abi.SIF_FINDER_SEEDS_MINIMA),
    ("extend_minima_f1", 1.0, abi.SIF_FINDER_SEEDS_MINIMA | abi.SIF_FINDER_EXTEND_REACH),
    ("peak", 1.0, abi.SIF_FINDER_SEEDS_MINIMA | abi.SIF_FINDER_EXTEND_REACH | abi.SIF_FINDER_DISPLACE),
    ("lagrangian", 0.0, abi.SIF_FINDER_LAGRANGIAN_OVERLAP),
]
HOLES = [((32.0, 32.0, 32.0), 18.0), ((90.0, 70.0, 40.0), 14.0), ((60.0, 100.0, 96.0), 20.0)]


def weighted_inputs(name, v="strict"):
    """Positions and weights of a weighted set (see the module docstring)."""
    p = WEIGHTED
    n3 = p["n"] ** 3
    if name == "rand":
        x, y, z = synth.zeldovich(p["n"], p["box"], p["rms_disp"], p["seed"])
        rng = np.random.default_rng(p["seed"] + 2000)
        w = rng.uniform(0.5, 1.5, n3).astype(np.float32)
        w[rng.random(n3) < 0.2] = 0.0
        if v == "f64":
            jr = np.random.default_rng(p["seed"] + 1000)  # BOX32's f64 jitter

            def jitter(a):
                u = a.astype(np.float64) + jr.uniform(-1e-4, 1e-4, a.shape)
                u = np.where(u < 0.0, u + p["box"], u)
                return np.where(u >= p["box"], u - p["box"], u)

            x, y, z = jitter(x), jitter(y), jitter(z)
        return x, y, z, w
    rng = np.random.default_rng(p["seed"] + 3000)
    pos = (rng.random((3, n3)) * p["box"]).astype(np.float32)
    pos = np.where(pos >= np.float32(p["box"]), np.float32(0.0), pos)
    w = np.ones(n3, np.float32)
    for c, r in HOLES:
        d = pos.astype(np.float64) - np.array(c)[:, None]
        d -= p["box"] * np.round(d / p["box"])
        w[(d ** 2).sum(0) < r * r] = 0.0
    return pos[0], pos[1], pos[2], w


def _ref_run(lib, x, y, z, w, radii, kw):
    p = WEIGHTED
    f = R.RefField(lib, x, y, z, weights=w, **kw)
    g = R.RefGrid(lib, p["n"], p["box"], **kw)
    g.assign_cic(f)
    g.to_contrast()
    m = R.RefMesh(lib, p["mesh"], p["box"], f)
    return f, g, m


def make_box32_weighted(path, v="strict"):
    p = WEIGHTED
    real = np.float64 if v == "f64" else np.float32
    kw = dict(variant=v) if v == "f64" else {}
    radii = synth.ladder(p["r0"], p["top"] * p["r0"], p["step"]).astype(real)
    lib = R.load(v, 4, abi.SIF_LOG_LEVEL_ERROR)
    out = dict(radii=radii, params=np.array([p["n"], p["box"], p["rms_disp"], p["seed"], p["r0"],
                                             p["threshold"], p["mesh"]], np.float64))
    for name in (("rand", "holes") if v == "strict" else ("rand",)):
        x, y, z, w = weighted_inputs(name, v)
        f, g, m = _ref_run(lib, x, y, z, w, radii, kw)
        mx, my, mz, offs, idx = m.arrays(**kw)
        mw, cw, tot = m.weights(**kw)
        delta = g.values()  # before the run smooths the grid in place and restores it
        fields = np.zeros((len(radii), p["n"] ** 3), real)
        R.exodus_raw(lib, g, m, radii, p["threshold"], capture=fields, **kw)
        out.update({f"{name}_{k}": a for k, a in dict(
            x=x, y=y, z=z, w=w, delta=delta, mesh_x=mx, mesh_y=my, mesh_z=mz,
            mesh_offsets=offs, mesh_index=idx, mesh_w=mw, mesh_cell_w=cw, fields=fields).items()})
        out[f"{name}_total_weight"] = np.array(tot)
        for oname, overlap, opt in WEIGHTED_SETS:
            c = R.exodus_raw(lib, g, m, radii, p["threshold"], overlap, opt, inject=fields, **kw)
            for k, col in zip(("cx", "cy", "cz", "r"), c):
                out[f"{name}_cat_{oname}_{k}"] = col
            out[f"{name}_cat_{oname}_opt"] = np.array([overlap, opt], np.float64)
        m.free()
        g.free()
        f.free()
        print(f"{path} {name}: " + ", ".join(
            f"{o} {len(out[f'{name}_cat_{o}_r'])}" for o, _, _ in WEIGHTED_SETS))
    # Weights of 1 and of 4 change nothing, bit for bit (the grid through the
    # CIC deposit, the rescaling through the mesh).
    x, y, z, _ = weighted_inputs("rand", v)
    cats = []
    for w in (None, np.ones(len(x), np.float32), np.full(len(x), 4.0, np.float32)):
        f, g, m = _ref_run(lib, x, y, z, w, radii, kw)
        cats.append(R.exodus_raw(lib, g, m, radii, p["threshold"], **kw))
        m.free()
        g.free()
        f.free()
    for c in cats[1:]:
        assert all(np.array_equal(a, b) for a, b in zip(c, cats[0])), "uniform weights changed the run"
    np.savez_compressed(path, **out)


REFINE = dict(BOX32)
REFINE_SETS = [
    ("cells", 0.0, abi.SIF_FINDER_REFINE_GAUSSIAN),
    ("minima", 0.0, abi.SIF_FINDER_SEEDS_MINIMA | abi.SIF_FINDER_REFINE_GAUSSIAN),
    ("minima_f05", 0.5, abi.SIF_FINDER_SEEDS_MINIMA | abi.SIF_FINDER_REFINE_GAUSSIAN),
    ("peak", 1.0, abi.SIF_FINDER_SEEDS_MINIMA | abi.SIF_FINDER_REFINE_GAUSSIAN |
     abi.SIF_FINDER_EXTEND_REACH | abi.SIF_FINDER_DISPLACE),
    ("lagrangian", 0.0, abi.SIF_FINDER_REFINE_GAUSSIAN | abi.SIF_FINDER_LAGRANGIAN_OVERLAP),
]


def make_box32_refine(path, v="strict"):
    p = REFINE
    x, y, z = synth.zeldovich(p["n"], p["box"], p["rms_disp"], p["seed"])
    real = np.float32
    kw = {}
    if v == "f64":
        rng = np.random.default_rng(p["seed"] + 1000)  # BOX32's f64 jitter

        def jitter(a):
            w = a.astype(np.float64) + rng.uniform(-1e-4, 1e-4, a.shape)
            w = np.where(w < 0.0, w + p["box"], w)
            return np.where(w >= p["box"], w - p["box"], w)

        x, y, z = jitter(x), jitter(y), jitter(z)
        real = np.float64
        kw = dict(variant=v)
    radii = synth.ladder(p["r0"], 3 * p["r0"], 0.1).astype(real)
    lib = R.load(v, 4, abi.SIF_LOG_LEVEL_ERROR)
    f = R.RefField(lib, x, y, z, **kw)
    g = R.RefGrid(lib, p["n"], p["box"], **kw)
    g.assign_cic(f)
    g.to_contrast()
    delta = g.values()
    m = R.RefMesh(lib, p["mesh"], p["box"], f)
    mx, my, mz, offs, idx = m.arrays(**kw)
    out = dict(radii=radii, delta=delta, mesh_x=mx, mesh_y=my, mesh_z=mz, mesh_offsets=offs,
               params=np.array([p["n"], p["box"], p["rms_disp"], p["seed"], p["r0"],
                                p["threshold"], p["mesh"]], np.float64))
    # The rungs' top-hat fields, from an unrefined run of the same contrast.
    n_r = len(radii)
    tophat = np.zeros((n_r + 1, p["n"] ** 3), real)
    R.exodus_raw(lib, g, m, radii, p["threshold"], capture=tophat, **kw)
    tophat = tophat[:n_r]
    gauss = np.zeros((n_r, p["n"] ** 3), real)
    have = np.zeros(n_r, bool)
    sets = REFINE_SETS if v == "strict" else [s_ for s_ in REFINE_SETS if s_[0] in ("cells", "minima", "peak")]
    for name, overlap, opt in sets:
        # Each run from the same contrast (a run hands its grid back restored
        # through a transform, not bit for bit).
        g.set_values(delta)
        cap = np.zeros((2 * n_r + 1, p["n"] ** 3), real)
        calls = []
        c0 = R.exodus_raw(lib, g, m, radii, p["threshold"], overlap, opt, capture=cap,
                          calls=calls, **kw)
        seq = cap[: calls[0] - 1]  # the last call is the grid's restore
        # Which rungs ran the refinement's transform: after rung i's top-hat
        # comes either rung i+1's top-hat or rung i's refinement field.
        k, used = 0, np.zeros(n_r, bool)
        for i in range(n_r):
            assert np.array_equal(seq[k], tophat[i])
            k += 1
            if k < len(seq) and (i + 1 == n_r or not np.array_equal(seq[k], tophat[i + 1])):
                assert not have[i] or np.array_equal(gauss[i], seq[k])
                gauss[i], have[i], used[i] = seq[k], True, True
                k += 1
        assert k == len(seq)
        g.set_values(delta)
        c = R.exodus_raw(lib, g, m, radii, p["threshold"], overlap, opt, inject=seq, **kw)
        # The run on its own fields is the run that returned them.
        assert all(np.array_equal(a, b) for a, b in zip(c, c0))
        out[f"{name}_refined_rungs"] = used
        for k_, col in zip(("cx", "cy", "cz", "r"), c):
            out[f"cat_{name}_{k_}"] = col
        out[f"cat_{name}_opt"] = np.array([overlap, opt], np.float64)
        g.set_values(delta)
        base = R.exodus_raw(lib, g, m, radii, p["threshold"], overlap,
                            opt & ~abi.SIF_FINDER_REFINE_GAUSSIAN, **kw)
        print(f"{path} {name}: {len(c[0])} voids ({len(base[0])} unrefined), "
              f"{int(used.sum())} rungs refined")
    out["tophat"] = tophat
    out["gauss_rungs"] = np.flatnonzero(have)
    out["gauss"] = gauss[have]
    m.free()
    g.free()
    f.free()
    np.savez_compressed(path, **out)


def positions_sha256(x, y, z):
    import hashlib

    h = hashlib.sha256()
    for a in (x, y, z):
        h.update(np.ascontiguousarray(a, np.float32).tobytes())
    return h.hexdigest()


def make_workload_a(path):
    w = synth.WORKLOADS["A"]
    x, y, z = synth.workload_particles("A")
    radii = synth.workload_radii("A")
    mesh = int(round(w["box"] / w["mesh_cell"]))
    cat = R.pipeline(x, y, z, w["n"], w["box"], mesh, radii, w["threshold"], n_threads=0)
    out = {f"cat_{k}": c for k, c in zip(("cx", "cy", "cz", "r"), cat)}
    out.update(radii=radii, positions_sha256=np.array(positions_sha256(x, y, z)),
               params=np.array([w["n"], w["box"], w["rms_disp"], w["seed"], w["n"], mesh,
                                w["threshold"]], np.float64))
    np.savez_compressed(path, **out)
    print(f"{path}: {len(cat[0])} voids over {len(radii)} rungs")


def make_survey(path):
    lib = R.load()
    out = {}
    for case in SURVEY_CASES:
        name, sel, n_r, thr, lad, weighted, opt, moved = case
        data, rand, wd, wr, radii = survey_inputs(case)
        fd = R.RefField(lib, *data, weights=wd)
        fr = R.RefField(lib, *rand, weights=wr)
        offset = None
        box = synth.SURVEY["box"]
        if moved:
            offset, box = R.survey_box(lib, fd, fr, radii, opt)
            fd.free()
            fr.free()
            data = tuple(np.float32(a + o) for a, o in zip(data, offset))
            rand = tuple(np.float32(a + o) for a, o in zip(rand, offset))
            fd = R.RefField(lib, *data, weights=wd)
            fr = R.RefField(lib, *rand, weights=wr)
        gd, gr = R.RefGrid(lib, SURVEY_GRID, box), R.RefGrid(lib, SURVEY_GRID, box)
        gd.assign_cic(fd)
        gr.assign_cic(fr)
        md = R.RefMesh(lib, SURVEY_MESH, box, fd, abi.SIF_MESH_DROP_INDICES)
        mr = R.RefMesh(lib, SURVEY_MESH, box, fr, abi.SIF_MESH_DROP_INDICES)
        cat = R.exodus_survey_raw(lib, gd, gr, md, mr, radii, thr, 0.0, opt, offset=offset)
        for k, c in zip(("cx", "cy", "cz", "r", "foot", "shell"), cat):
            out[f"{name}_{k}"] = c
        out[f"{name}_sha256"] = np.array(survey_sha256(*survey_inputs(case)[:4]))
        out[f"{name}_box"] = np.array([box] + (list(offset) if moved else [0.0, 0.0, 0.0]),
                                      np.float32)
        print(f"{path}: {name}: {len(cat[0])} voids over {len(radii)} rungs")
        for o in (md, mr, gd, gr, fd, fr):
            o.free()
    np.savez_compressed(path, **out)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "survey":
        make_survey(os.path.join(HERE, "golden_survey.npz"))
        sys.exit(0)
    if len(sys.argv) > 1 and sys.argv[1] == "workload_a":
        make_workload_a(os.path.join(HERE, "golden_workload_a.npz"))
        sys.exit(0)
    if len(sys.argv) > 1 and sys.argv[1] == "refine":
        make_box32_refine(os.path.join(HERE, "golden_box32_refine.npz"))
        make_box32_refine(os.path.join(HERE, "golden_box32_refine_f64.npz"), "f64")
        sys.exit(0)
    if len(sys.argv) > 1 and sys.argv[1] == "weighted":
        make_box32_weighted(os.path.join(HERE, "golden_box32_weighted.npz"))
        make_box32_weighted(os.path.join(HERE, "golden_box32_weighted_f64.npz"), "f64")
        sys.exit(0)
    if len(sys.argv) > 1 and sys.argv[1] == "displace":
        make_box32_displace(os.path.join(HERE, "golden_box32_displace.npz"))
        make_box32_displace(os.path.join(HERE, "golden_box32_displace_f64.npz"), "f64")
        sys.exit(0)
    make_box32(os.path.join(HERE, "golden_box32.npz"))
    make_box32_f64(os.path.join(HERE, "golden_box32_f64.npz"))
    make_box32_extend(os.path.join(HERE, "golden_box32_extend.npz"))
    make_box32_extend(os.path.join(HERE, "golden_box32_extend_f64.npz"), "f64")
    make_box32_displace(os.path.join(HERE, "golden_box32_displace.npz"))
    make_box32_displace(os.path.join(HERE, "golden_box32_displace_f64.npz"), "f64")
    make_box32_weighted(os.path.join(HERE, "golden_box32_weighted.npz"))
    make_box32_weighted(os.path.join(HERE, "golden_box32_weighted_f64.npz"), "f64")
    make_box32_refine(os.path.join(HERE, "golden_box32_refine.npz"))
    make_box32_refine(os.path.join(HERE, "golden_box32_refine_f64.npz"), "f64")
    make_workload_a(os.path.join(HERE, "golden_workload_a.npz"))
    make_survey(os.path.join(HERE, "golden_survey.npz"))
