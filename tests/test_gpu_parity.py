"""Parity of the GPU path with the oracle and the reference's golden vectors.

Every stage is called through the C ABI (libsif_gb300.so), on device data
for the stage tests and through sif's own API for the end-to-end ones.
Bars: the chain mesh and the catalogue bit for bit (integer and index work,
and the finder's float tests replayed op for op); the CIC grid and the
smoothed field against FP64 within 1e-6 relative L2 (the tolerance the
workloads state), 1e-5 max-norm over the field rms.
"""
import numpy as np
import pytest

from conftest import same_bits, same_catalogue
from sif_gb300 import abi, synth

pytestmark = pytest.mark.gpu

FIELD_L2_TOL = 1e-6
FIELD_MAX_TOL = 1e-5


def _cuda(*arrays):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrays]


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    rms = np.sqrt((b * b).mean())
    return np.sqrt(((a - b) ** 2).mean()) / rms, np.abs(a - b).max() / rms


@pytest.fixture(scope="module")
def dev(gpu_lib):
    from sif_gb300 import device

    return device


def test_cic_against_fp64(dev, oracle):
    x, y, z = synth.zeldovich(64, 250.0, 4.0, 5)
    g = dev.cic(*_cuda(x, y, z), 64, 250.0).cpu().numpy()
    want = oracle.cic_f64(x, y, z, 64, 250.0)
    l2, mx = _rel(g, want)
    assert l2 <= FIELD_L2_TOL and mx <= FIELD_MAX_TOL, (l2, mx)
    cl = 250.0 / 64
    assert abs(g.astype(np.float64).sum() * cl ** 3 - len(x)) <= 1e-5 * len(x)


def test_cic_is_independent_of_particle_order(dev):
    x, y, z = synth.zeldovich(48, 200.0, 4.0, 6)
    perm = np.random.default_rng(1).permutation(len(x))
    a = dev.cic(*_cuda(x, y, z), 48, 200.0).cpu().numpy()
    b = dev.cic(*_cuda(x[perm], y[perm], z[perm]), 48, 200.0).cpu().numpy()
    assert same_bits(a, b)


@pytest.mark.parametrize("n_grid", [37, 64, 100])
def test_cic_non_tile_multiple_grids(dev, oracle, n_grid):
    x, y, z = synth.zeldovich(40, 180.0, 4.0, n_grid)
    g = dev.cic(*_cuda(x, y, z), n_grid, 180.0).cpu().numpy()
    l2, mx = _rel(g, oracle.cic_f64(x, y, z, n_grid, 180.0))
    assert l2 <= FIELD_L2_TOL and mx <= FIELD_MAX_TOL, (l2, mx)


def test_cic_edge_coordinates(dev, oracle):
    """Coordinates on and within rounding of the faces fold as the
    reference's do (src/structures/field_internal.h:58-64)."""
    box = np.float32(100.0)
    v = np.array([0.0, np.nextafter(box, 0), 99.99999, 50.0, 0.0, 1e-30], np.float32)
    x, y, z = v, v[::-1].copy(), np.roll(v, 2)
    g = dev.cic(*_cuda(x, y, z), 16, 100.0).cpu().numpy()
    l2, mx = _rel(g, oracle.cic_f64(x, y, z, 16, 100.0))
    assert mx <= 1e-5


def test_contrast_matches_oracle(dev, oracle, golden_box32):
    import torch

    d = torch.from_numpy(golden_box32["density"].copy()).cuda()
    dev.density_contrast(d)
    assert same_bits(d.cpu().numpy(), golden_box32["delta"])


def test_mesh_matches_reference_golden(dev, golden_box32):
    g = golden_box32
    mx, my, mz, offs, orig = dev.chain_mesh(*_cuda(g["x"], g["y"], g["z"]), int(g["params"][6]),
                                            float(g["params"][1]))
    assert same_bits(mx.cpu().numpy(), g["mesh_x"])
    assert same_bits(my.cpu().numpy(), g["mesh_y"])
    assert same_bits(mz.cpu().numpy(), g["mesh_z"])
    assert np.array_equal(offs.cpu().numpy().astype(np.uint64), g["mesh_offsets"])
    assert np.array_equal(orig.cpu().numpy().astype(np.uint64), g["mesh_index"])


@pytest.mark.parametrize("n_cells", [7, 25, 64])
def test_mesh_matches_oracle(dev, oracle, n_cells):
    x, y, z = synth.zeldovich(50, 300.0, 6.0, n_cells)
    # Clustered duplicates exercise the large-cell path of the canonical sort.
    x[:3000] = x[0]
    y[:3000] = y[0]
    z[:3000] = z[0]
    mx, my, mz, offs, orig = dev.chain_mesh(*_cuda(x, y, z), n_cells, 300.0)
    m = oracle.OracleMesh(x, y, z, n_cells, 300.0)
    assert same_bits(mx.cpu().numpy(), m.x) and same_bits(mz.cpu().numpy(), m.z)
    assert np.array_equal(offs.cpu().numpy().astype(np.uint64), m.offsets)
    assert np.array_equal(orig.cpu().numpy().astype(np.uint64), m.orig)


@pytest.mark.parametrize("n_cells", [1626, 1 << 22])
def test_mesh_refuses_a_side_past_32_bit_offsets(gpu_lib, n_cells):
    """The GPU mesh keeps 32-bit cell ids and offsets: a side whose cube
    (plus the end offset) passes 2^32, or whose cube wraps in 64 bits, is
    refused with SIF_ERR_RANGE before anything is cubed or allocated."""
    import ctypes as C

    import torch

    from sif_gb300 import _lib

    lib = _lib.load()
    xs = [torch.zeros(16, dtype=torch.float32, device="cuda") for _ in range(3)]
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    st = lib.sifg_mesh_device(p(xs[0]), p(xs[1]), p(xs[2]), 16, n_cells, 100.0, p(xs[0]),
                              p(xs[1]), p(xs[2]), p(xs[0]), p(xs[1]))
    assert st == abi.SIF_ERR_RANGE
    assert b"cells a side" in lib.sif_error_message()


@pytest.mark.parametrize("window", ["full", "aliasing", "none"])
def test_smoothing_against_fp64(dev, oracle, golden_box32, window):
    g = golden_box32
    n, box = int(g["params"][0]), float(g["params"][1])
    (delta,) = _cuda(g["delta"])
    radii = np.sort(g["radii"])[::-1]
    mode = {"none": 0, "full": 1, "aliasing": 2}[window]
    want = oracle.smooth(g["delta"], n, box, radii, window_mode=mode, mode=0, want="f64")
    for i, r in enumerate(radii):
        got = dev.smooth(delta, n, box, float(r), window=window).cpu().numpy()
        l2, mx = _rel(got, want[i])
        assert l2 <= FIELD_L2_TOL and mx <= FIELD_MAX_TOL, (r, l2, mx)


@pytest.mark.parametrize("n", [27, 30])
def test_smoothing_odd_and_non_power_grids(dev, oracle, n):
    """Grids whose mode count n^2 (n/2+1) is odd (27) or not a power of two (30)."""
    rng = np.random.default_rng(n)
    delta = rng.standard_normal(n ** 3).astype(np.float32)
    box = 3.0 * n
    want = oracle.smooth(delta, n, box, [5.0, 9.0], mode=0, want="f64")
    (d,) = _cuda(delta)
    for i, r in enumerate([5.0, 9.0]):
        got = dev.smooth(d, n, box, r).cpu().numpy()
        l2, mx = _rel(got, want[i])
        assert l2 <= FIELD_L2_TOL and mx <= FIELD_MAX_TOL, (n, r, l2, mx)


@pytest.mark.parametrize("window", ["full", "aliasing", "none"])
def test_smoothing_512_against_the_fp64_form(dev, window):
    """n = 512, the bench's grid, where the float form runs its own three-pass
    inverse transform (filter + kx, ky, kz C2R): against the FP64 form's
    (cuFFT D2Z/Z2D, pinned to the oracle on smaller grids) on the same
    contrast, for top-hat and Gaussian filters."""
    import torch

    n, box = 512, 1000.0
    x, y, z = synth.zeldovich(128, box, 5.0, 22)
    xs = _cuda(x, y, z)
    grid = dev.cic(*xs, n, box)
    dev.density_contrast(grid)
    g64 = grid.double()
    for r, filt in ((4.0, "top-hat"), (20.0, "top-hat"), (6.0, "gaussian")):
        a = dev.smooth(grid, n, box, r, filter=filt, window=window).double()
        b = dev.smooth(g64, n, box, r, filter=filt, window=window)
        rms = torch.sqrt((b * b).mean())
        l2 = float(torch.sqrt(((a - b) ** 2).mean()) / rms)
        mx = float((a - b).abs().max() / rms)
        assert l2 <= FIELD_L2_TOL and mx <= FIELD_MAX_TOL, (r, filt, l2, mx)


def test_factor_tables_change_no_bit(dev):
    """At 512^3 the filter pass reads each smoothing's factor table; the
    fields are bit for bit those of the pass that evaluates the factors, for
    both filters and every window, and a table reused on a second smoothing
    at the same radius gives the same bits again."""
    import torch

    n, box = 512, 1000.0
    x, y, z = synth.zeldovich(128, box, 5.0, 23)
    grid = dev.cic(*_cuda(x, y, z), n, box)
    dev.density_contrast(grid)
    for window in ("full", "aliasing", "none"):
        for r, filt in ((4.0, "top-hat"), (17.3, "top-hat"), (6.0, "gaussian")):
            a = dev.smooth(grid, n, box, r, filter=filt, window=window)
            b = dev.smooth(grid, n, box, r, filter=filt, window=window)
            dev.set_factor_tables(0)
            try:
                c = dev.smooth(grid, n, box, r, filter=filt, window=window)
            finally:
                dev.set_factor_tables(1)
            assert torch.equal(a.view(torch.int32), c.view(torch.int32)), (window, r, filt)
            assert torch.equal(a.view(torch.int32), b.view(torch.int32))


def test_gaussian_smoothing_against_fp64(dev, oracle, golden_box32):
    g = golden_box32
    n, box = int(g["params"][0]), float(g["params"][1])
    (delta,) = _cuda(g["delta"])
    want = oracle.smooth(g["delta"], n, box, [6.0], filter=2, mode=0, want="f64")[0]
    got = dev.smooth(delta, n, box, 6.0, filter="gaussian").cpu().numpy()
    l2, mx = _rel(got, want)
    assert l2 <= FIELD_L2_TOL and mx <= FIELD_MAX_TOL


def _golden_mesh(g):
    return _cuda(g["mesh_x"], g["mesh_y"], g["mesh_z"], g["mesh_offsets"].astype(np.int32))


@pytest.mark.parametrize("name", ["default", "search_2_00", "search_1_25", "lagrangian", "minima",
                                  "overlap_0_5"])
def test_catalogue_matches_reference_golden(dev, golden_box32, name):
    """The reference's own catalogue, on the fields its own run smoothed."""
    g = golden_box32
    n, box, thr, n_mesh = int(g["params"][0]), float(g["params"][1]), float(g["params"][5]), int(g["params"][6])
    overlap, opt = g[f"cat_{name}_opt"]
    delta, fields = _cuda(g["delta"], g["fields"].reshape(-1))
    cat = dev.exodus(delta, n, box, _golden_mesh(g), n_mesh, g["radii"], thr, float(overlap),
                     int(opt), inject=fields)
    want = tuple(g[f"cat_{name}_{k}"] for k in ("cx", "cy", "cz", "r"))
    assert len(cat[0]) == len(want[0])
    assert same_catalogue(cat, want)


@pytest.mark.parametrize("mode", [1, 2], ids=["cta", "warp"])
def test_catalogue_with_prior_matches_reference_golden(dev, golden_box32, mode):
    """Ten voids to start from (sif_finder_exodus_extras_t::prior): accepted
    before the first rung, returned first, and respected by every rung after;
    the reference's catalogue on its own fields, by each growth kernel."""
    g = golden_box32
    n, box, thr, n_mesh = int(g["params"][0]), float(g["params"][1]), float(g["params"][5]), int(g["params"][6])
    delta, fields = _cuda(g["delta"], g["fields"].reshape(-1))
    prior = tuple(g[f"prior_{k}"] for k in ("cx", "cy", "cz", "r"))
    dev.set_growth_mode(mode)
    try:
        cat = dev.exodus(delta, n, box, _golden_mesh(g), n_mesh, g["radii"], thr, inject=fields,
                         prior=prior)
    finally:
        dev.set_growth_mode(0)
    want = tuple(g[f"cat_prior_{k}"] for k in ("cx", "cy", "cz", "r"))
    assert len(cat[0]) == len(want[0])
    assert same_catalogue(cat, want)


@pytest.mark.parametrize("bad", ["radius_zero", "radius_nan", "centre_outside", "centre_negative"])
def test_prior_checked_as_the_reference_checks_it(dev, golden_box32, bad):
    """sif__exodus_check_extras (src/finder/exodus_finder.c:1163-1197): a radius
    that is not positive and finite, or a centre outside [0, box), is refused."""
    g = golden_box32
    n, box, thr, n_mesh = int(g["params"][0]), float(g["params"][1]), float(g["params"][5]), int(g["params"][6])
    delta, fields = _cuda(g["delta"], g["fields"].reshape(-1))
    cx, cy, cz, r = (g[f"prior_{k}"].copy() for k in ("cx", "cy", "cz", "r"))
    if bad == "radius_zero":
        r[3] = 0.0
    elif bad == "radius_nan":
        r[3] = np.nan
    elif bad == "centre_outside":
        cy[2] = box
    else:
        cz[1] = -1e-3
    with pytest.raises(Exception, match="prior"):
        dev.exodus(delta, n, box, _golden_mesh(g), n_mesh, g["radii"], thr, inject=fields,
                   prior=(cx, cy, cz, r))


def test_pysif_exodus_with_prior_and_save_memory(gpu_lib):
    """finders.exodus(prior=..., save_memory=True) through sif's C API: the
    prior voids come back first and unchanged; save_memory changes nothing."""
    from test_oracle import _holes_field

    pysif = gpu_lib
    x, y, z, holes = _holes_field()
    f = pysif.Field(x, y, z)
    g = pysif.Grid(32, 200.0)
    g.assign_cic(f)
    g.to_density_contrast()
    m = pysif.ChainMesh(8, 200.0, f, drop_indices=True)
    radii = np.array([30, 25, 20, 16, 13, 10], np.float32)
    plain = pysif.finders.exodus(g, m, radii, -0.7).as_tuple()
    prior = tuple(np.asarray(c[:2], np.float32) for c in plain)
    cat = pysif.finders.exodus(g, m, radii, -0.7, prior=prior, save_memory=True).as_tuple()
    assert all(np.array_equal(a[:2], b) for a, b in zip(cat, prior))
    assert same_catalogue(pysif.finders.exodus(g, m, radii, -0.7, save_memory=True).as_tuple(), plain)


EXTEND_SETS = ["minima_f1", "extend_minima_f1", "extend_f1", "extend"]


@pytest.mark.parametrize("mode", [0, 1, 2], ids=["auto", "cta", "warp"])
@pytest.mark.parametrize("name", EXTEND_SETS)
def test_catalogue_matches_reference_golden_extended_reach(dev, golden_box32_extend, name, mode):
    """SIF_FINDER_EXTEND_REACH: a crossing past the rung's reach measured at
    the levels of an extended reach, by each growth kernel; the reference's
    catalogues, with and without it, on its own fields."""
    dev.set_growth_mode(mode)
    try:
        test_catalogue_matches_reference_golden(dev, golden_box32_extend, name)
    finally:
        dev.set_growth_mode(0)


DISPLACE_SETS = ["peak", "peak_no_displace", "cells_f0", "cells_f05", "minima_f05", "lagrangian"]


@pytest.mark.parametrize("mode", [0, 1, 2], ids=["auto", "cta", "warp"])
@pytest.mark.parametrize("name", DISPLACE_SETS)
def test_catalogue_matches_reference_golden_displacement(dev, golden_box32_displace, name, mode):
    """SIF_FINDER_DISPLACE on the GPU: every candidate grown, then the
    survivors one at a time in rank order, displacing the smaller voids they
    collide with; the reference's catalogues (the excursion-peak preset among
    them) on its own fields, by each growth kernel."""
    dev.set_growth_mode(mode)
    try:
        test_catalogue_matches_reference_golden(dev, golden_box32_displace, name)
    finally:
        dev.set_growth_mode(0)


@pytest.fixture(params=[1, 2], ids=["cta", "warp"])
def growth_mode(request, dev):
    """Each sphere-growth kernel forced in turn; back to automatic after."""
    dev.set_growth_mode(request.param)
    yield request.param
    dev.set_growth_mode(0)


@pytest.mark.parametrize("name", ["default", "search_2_00", "lagrangian", "minima", "overlap_0_5"])
def test_catalogue_matches_reference_golden_either_growth_kernel(dev, golden_box32, growth_mode,
                                                                 name):
    test_catalogue_matches_reference_golden(dev, golden_box32, name)


@pytest.fixture(params=[-1, 0, 64, 512], ids=["list_auto", "list_none", "list_64", "list_512"])
def shell_list(request, dev):
    """The warp growth's shell list sized per rung, absent, small (most
    survivors walk again), and at its largest; back to automatic after."""
    dev.set_growth_mode(2)
    dev.set_shell_list(request.param)
    yield request.param
    dev.set_shell_list(-1)
    dev.set_growth_mode(0)


@pytest.mark.parametrize("name", ["default", "search_2_00", "lagrangian", "overlap_0_5"])
def test_catalogue_matches_reference_golden_any_shell_list(dev, golden_box32, shell_list, name):
    """A window's distances from the shell list or from a walk over the
    cells: the same catalogue, bit for bit."""
    test_catalogue_matches_reference_golden(dev, golden_box32, name)


@pytest.mark.parametrize("name", ["default", "search_2_00", "lagrangian", "minima", "overlap_0_5"])
def test_catalogue_matches_reference_golden_with_the_witness(dev, golden_box32, name):
    """The collision witness only refuses survivors the commit would refuse:
    switched on, the reference's catalogue all the same."""
    dev.set_witness(1)
    try:
        test_catalogue_matches_reference_golden(dev, golden_box32, name)
    finally:
        dev.set_witness(0)


@pytest.mark.parametrize("name", EXTEND_SETS)
def test_extended_reach_golden_with_the_witness(dev, golden_box32_extend, name):
    dev.set_witness(1)
    try:
        test_catalogue_matches_reference_golden(dev, golden_box32_extend, name)
    finally:
        dev.set_witness(0)


@pytest.fixture(params=[0, 1], ids=["one_launch", "launch_per_round"])
def commit_mode(request, dev):
    """The commit's rounds in one cooperative launch, then a launch per round."""
    dev.set_commit_mode(request.param)
    yield request.param
    dev.set_commit_mode(0)


@pytest.mark.parametrize("name", ["default", "lagrangian", "minima", "overlap_0_5"])
def test_catalogue_matches_reference_golden_either_commit_form(dev, golden_box32, commit_mode,
                                                               name):
    test_catalogue_matches_reference_golden(dev, golden_box32, name)


@pytest.mark.parametrize("window", [1, 5, 64])
def test_catalogue_independent_of_resolve_window(dev, golden_box32, window):
    g = golden_box32
    n, box, thr = int(g["params"][0]), float(g["params"][1]), float(g["params"][5])
    delta, fields = _cuda(g["delta"], g["fields"].reshape(-1))
    dev.set_window(window)
    try:
        cat = dev.exodus(delta, n, box, _golden_mesh(g), int(g["params"][6]), g["radii"], thr,
                         inject=fields)
    finally:
        dev.set_window(8)
    want = tuple(g[f"cat_default_{k}"] for k in ("cx", "cy", "cz", "r"))
    assert same_catalogue(cat, want)


BOXES = [
    # n, box, rms, seed, grid, mesh, r0, threshold, options, overlap
    (64, 250.0, 4.0, 31, 64, 25, 5.0, -0.8, 0, 0.0),
    (60, 240.0, 5.0, 32, 60, 20, 6.0, -0.75, abi.SIF_FINDER_SEARCH_2_00, 0.0),
    (72, 300.0, 5.0, 33, 96, 24, 6.5, -0.7, abi.SIF_FINDER_LAGRANGIAN_OVERLAP, 0.0),
    (64, 200.0, 3.0, 34, 64, 16, 4.0, -0.8, abi.SIF_FINDER_SEARCH_1_75, 0.25),
]


@pytest.mark.parametrize("case", BOXES, ids=[f"box{i}" for i in range(len(BOXES))])
def test_catalogue_matches_oracle_on_shared_fields(dev, oracle, case):
    """The GPU's own smoothed fields, handed to the oracle: every candidate,
    radius and commit decision must then agree bit for bit."""
    import torch

    n, box, rms, seed, ng, nm, r0, thr, opt, ov = case
    x, y, z = synth.zeldovich(n, box, rms, seed)
    xs = _cuda(x, y, z)
    grid = dev.cic(*xs, ng, box)
    dev.density_contrast(grid)
    mesh = dev.chain_mesh(*xs, nm, box)
    radii = synth.ladder(r0, 4 * r0, 0.1).astype(np.float32)
    fields = torch.stack([dev.smooth(grid, ng, box, float(r)) for r in np.sort(radii)[::-1]])
    got = dev.exodus(grid, ng, box, mesh, nm, radii, thr, ov, opt, inject=fields.reshape(-1))
    m = oracle.OracleMesh(x, y, z, nm, box)
    want = oracle.exodus(grid.cpu().numpy(), m, radii, ng, box, thr, ov, opt, n_threads=4,
                         inject=fields.cpu().numpy())
    assert len(want[0]) > 10
    assert len(got[0]) == len(want[0]) and same_catalogue(got, want)
    # The GPU's own run (smoothing inside the finder) is the same run.
    own = dev.exodus(grid, ng, box, mesh, nm, radii, thr, ov, opt)
    assert same_catalogue(own, want)
    # And so is each sphere-growth kernel forced, and the commit a launch per round.
    for mode in (1, 2):
        dev.set_growth_mode(mode)
        try:
            forced = dev.exodus(grid, ng, box, mesh, nm, radii, thr, ov, opt, inject=fields.reshape(-1))
        finally:
            dev.set_growth_mode(0)
        assert same_catalogue(forced, want), mode
    dev.set_commit_mode(1)
    try:
        per_round = dev.exodus(grid, ng, box, mesh, nm, radii, thr, ov, opt, inject=fields.reshape(-1))
    finally:
        dev.set_commit_mode(0)
    assert same_catalogue(per_round, want)


def test_four_holes_and_brute_force_radii(gpu_lib, oracle):
    """tests/test_finders.c:117-164, 433-538 on the GPU path, through sif's
    C API: the four evacuated holes, and each radius equal to the O(N)
    brute-force radius in double to 1e-5."""
    from test_oracle import _check_holes, _holes_field

    pysif = gpu_lib
    x, y, z, holes = _holes_field()
    f = pysif.Field(x, y, z)
    g = pysif.Grid(32, 200.0)
    g.assign_cic(f)
    g.to_density_contrast()
    m = pysif.ChainMesh(8, 200.0, f, drop_indices=True)
    radii = np.array([30, 25, 20, 16, 13, 10], np.float32)
    before = g.values.copy()
    cat = pysif.finders.exodus(g, m, radii, -0.7)
    _check_holes(cat.as_tuple(), holes, 200.0 / 32)
    assert same_bits(g.values, before)  # restored exactly
    for rung, factor in [(16.0, 1.5), (20.0, 2.0), (13.0, 1.25)]:
        c = pysif.finders.exodus_raw(g, m, [rung], -0.7, search_factor=factor)
        assert len(c) > 0
        r_search = rung + max((factor - 1.0) * rung, 3.0 * 200.0 / 32)
        for i in range(len(c)):
            want = oracle.brute_force_radius(x, y, z, 200.0, (c.cx[i], c.cy[i], c.cz[i]), rung,
                                             r_search, -0.7)
            assert want > 0 and abs(c.radii[i] - want) <= 1e-5 * want


def test_c_api_end_to_end_and_errors(gpu_lib, oracle):
    pysif = gpu_lib
    x, y, z = synth.zeldovich(48, 220.0, 5.0, 41)
    f = pysif.Field(x, y, z)
    g = pysif.Grid(48, 220.0)
    g.assign_cic(f)
    l2, mx = _rel(g.values.reshape(-1), oracle.cic_f64(x, y, z, 48, 220.0))
    assert l2 <= FIELD_L2_TOL
    g.to_density_contrast()
    with pytest.raises(ValueError):
        g.to_density_contrast()  # already a contrast
    m = pysif.ChainMesh(11, 220.0, f)
    om = oracle.OracleMesh(x, y, z, 11, 220.0)
    mx_, my_, mz_, offs, idx = m.arrays()
    assert same_bits(mx_, om.x) and np.array_equal(offs, om.offsets) and np.array_equal(idx, om.orig)
    radii = synth.ladder(7.0, 21.0, 0.1)
    cat = pysif.finders.exodus(g, m, radii, -0.75)
    assert len(cat) > 0
    with pytest.raises(ValueError):
        pysif.finders.exodus(g, m, radii, 0.5)  # threshold out of (-1, 0)
    with pytest.raises(ValueError):
        pysif.finders.exodus(g, m, [-1.0], -0.7)
    # The excursion-peak preset (minima seeds, extended reach, displacement)
    # runs through sif's C API, and agrees with the oracle on the GPU's field.
    peak = pysif.finders.exodus(g, m, radii, -0.75, variant="excursion-peak").as_tuple()
    assert len(peak[0]) > 0
    wrong = pysif.Grid(48, 221.0)
    with pytest.raises(ValueError):
        pysif.finders.exodus(wrong, m, radii, -0.7)
    bad = pysif.Field(np.array([1.0, 300.0], np.float32), np.zeros(2, np.float32),
                      np.zeros(2, np.float32))
    with pytest.raises(ValueError):
        pysif.Grid(8, 220.0).assign_cic(bad)  # a particle outside the box
    # CONSUME_GRID leaves the last rung's smoothing in the grid.
    g2 = pysif.Grid(48, 220.0)
    g2.assign_cic(f)
    g2.to_density_contrast()
    pysif.finders.exodus_raw(g2, m, radii, -0.75, consume_grid=True)
    assert not same_bits(g2.values, g.values)


def test_consumed_grid_at_512_is_the_last_smoothing(gpu_lib, dev):
    """At a 512^3 grid the rungs' candidates come from the smoothing's lists
    and the fields themselves are not written -- but the last rung's is, for
    SIF_FINDER_CONSUME_GRID: the grid handed back is that rung's smoothing,
    bit for bit the transform's own."""
    import torch

    pysif = gpu_lib
    x, y, z = synth.zeldovich(128, 1000.0, 5.0, 31)
    f = pysif.Field(x, y, z)
    g = pysif.Grid(512, 1000.0)
    g.assign_cic(f)
    g.to_density_contrast()
    contrast = torch.from_numpy(g.values.reshape(-1).copy()).cuda()
    m = pysif.ChainMesh(50, 1000.0, f, drop_indices=True)
    radii = synth.ladder(16.0, 40.0, 0.2).astype(np.float32)
    cat = pysif.finders.exodus_raw(g, m, radii, -0.6, consume_grid=True)
    assert len(cat) > 0
    want = dev.smooth(contrast, 512, 1000.0, float(radii.min())).cpu().numpy()
    assert same_bits(g.values.reshape(-1), want)


@pytest.mark.parametrize("options,overlap", [(0, 0.0), (abi.SIF_FINDER_LAGRANGIAN_OVERLAP, 0.0),
                                             (0, 0.5)], ids=["default", "lagrangian", "overlap_0_5"])
def test_box_candidates_from_the_smoothing_list(dev, options, overlap):
    """At a 512^3 grid the float form's smoothing lists the cells at or below
    the threshold as it writes the field, and the rung's candidates are that
    list less the masked cells: the same catalogue, bit for bit, as a scan of
    the whole field every rung (which the oracle tests pin)."""
    import torch

    x, y, z = synth.zeldovich(256, 500.0, 5.0, 1205, backend="torch")
    xs = [torch.from_numpy(a).cuda() for a in (x, y, z)]
    radii = synth.ladder(4.0, 16.0, 0.1).astype(np.float32)
    cats, listed = [], []
    for mode in (0, 1):
        dev.set_scan_mode(mode)
        try:
            cats.append(dev.box(*xs, 512, 500.0, 62, radii, -0.8, overlap, options))
            listed.append([r["from_list"] for r in dev.last_rung_stats()])
        finally:
            dev.set_scan_mode(0)
    assert all(listed[0]) and not any(listed[1])
    assert len(cats[0][0]) > 100
    assert len(cats[0][0]) == len(cats[1][0]) and same_catalogue(cats[0], cats[1])


def test_last_run_timeline(dev):
    """sifg_last_trace after a box run: a span per rung on the run's stream,
    in order and not overlapping, a smoothing span per rung, and as many
    growth and commit spans as the run's timings count, each after its
    rung's start."""
    import torch

    x, y, z = synth.zeldovich(64, 250.0, 4.0, 31, backend="torch")
    xs = [torch.from_numpy(a).cuda() for a in (x, y, z)]
    radii = synth.ladder(5.0, 20.0, 0.1).astype(np.float32)
    cat = dev.box(*xs, 64, 250.0, 25, radii, -0.75)
    assert len(cat[0]) > 0
    trace = dev.last_trace()
    tm = dev.last_timings()
    by = {k: [(a, b) for kk, a, b in trace if kk == k] for k in dev.TRACE_KINDS}
    assert all(0.0 <= a <= b for _, a, b in trace)
    rungs = by["rung"]
    assert len(rungs) == len(radii) == len(by["smoothing"])
    assert all(b0 <= a1 for (_, b0), (a1, _) in zip(rungs, rungs[1:]))
    assert len(by["growth"]) == tm["growth_launches"] > 0
    assert len(by["commit"]) == tm["commit_launches"] > 0
    assert len(by["cic"]) == 1 and len(by["mesh"]) == 1 and len(by["cic_stage"]) == 1
    stage = by["cic_stage"][0]
    assert stage[0] <= by["cic"][0][0] and by["cic"][0][1] <= stage[1] <= rungs[0][0]
    assert abs(tm["cic_stage_ms"] - (stage[1] - stage[0])) < 1e-3
    assert all(any(a >= r0 and b <= r1 for r0, r1 in rungs) for a, b in by["growth"])
