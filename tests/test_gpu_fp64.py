"""The FP64 form (the `_f64` entry points) against the reference's
SIF_USE_DOUBLE build, through the C ABI on device data.

Bars: the chain mesh and the catalogue (on the reference's own double
fields) bit for bit; the deposit within the 2^-40-per-particle quantum
(relative 1e-11 of a cell); the contrast and the smoothing against double
references within 1e-12 relative.
"""
import numpy as np
import pytest

from conftest import same_bits64, same_catalogue64
from sif_gb300 import synth

pytestmark = pytest.mark.gpu

NAMES = ["default", "search_2_00", "search_1_25", "lagrangian", "overlap_0_5", "minima"]


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


def _params(g):
    p = g["params"]
    return int(p[0]), float(p[1]), float(p[5]), int(p[6])


def test_fp64_mesh_matches_reference(dev, golden_box32_f64):
    g = golden_box32_f64
    n, box, _, n_mesh = _params(g)
    mx, my, mz, offs, orig = dev.chain_mesh(*_cuda(g["x"], g["y"], g["z"]), n_mesh, box)
    assert mx.dtype.itemsize == 8
    assert same_bits64(mx.cpu().numpy(), g["mesh_x"])
    assert same_bits64(my.cpu().numpy(), g["mesh_y"])
    assert same_bits64(mz.cpu().numpy(), g["mesh_z"])
    assert np.array_equal(offs.cpu().numpy().astype(np.uint64), g["mesh_offsets"])
    assert np.array_equal(orig.cpu().numpy().astype(np.uint64), g["mesh_index"])


def test_fp64_deposit_matches_reference(dev, golden_box32_f64):
    g = golden_box32_f64
    n, box, _, _ = _params(g)
    got = dev.cic(*_cuda(g["x"], g["y"], g["z"]), n, box).cpu().numpy()
    assert got.dtype == np.float64
    l2, mx = _rel(got, g["density"])
    assert l2 <= 1e-11 and mx <= 1e-11, (l2, mx)
    # Mass: exactly one particle per particle, to the quantum.
    cell = box / n
    assert abs(got.sum() * cell ** 3 - len(g["x"])) <= 1e-6


def test_fp64_contrast_matches_reference(dev, golden_box32_f64):
    g = golden_box32_f64
    (grid,) = _cuda(g["density"])
    dev.density_contrast(grid)
    l2, mx = _rel(grid.cpu().numpy(), g["delta"])
    assert l2 <= 1e-14 and mx <= 1e-13, (l2, mx)


@pytest.mark.parametrize("name", NAMES)
def test_fp64_catalogue_matches_reference(dev, golden_box32_f64, name):
    """The SIF_USE_DOUBLE build's catalogue, on the double fields its run smoothed."""
    g = golden_box32_f64
    n, box, thr, n_mesh = _params(g)
    overlap, opt = g[f"cat_{name}_opt"]
    mesh = _cuda(g["mesh_x"], g["mesh_y"], g["mesh_z"], g["mesh_offsets"].astype(np.int32))
    delta, fields = _cuda(g["delta"], g["fields"].reshape(-1))
    got = dev.exodus(delta, n, box, mesh, n_mesh, g["radii"], thr, overlap=float(overlap),
                     options=int(opt), inject=fields)
    want = tuple(g[f"cat_{name}_{k}"] for k in ("cx", "cy", "cz", "r"))
    assert got[0].dtype == np.float64
    assert len(got[0]) == len(want[0]) and same_catalogue64(got, want), (len(got[0]), len(want[0]))


@pytest.mark.parametrize("mode", [1, 2], ids=["cta", "warp"])
def test_fp64_catalogue_either_growth_kernel(dev, golden_box32_f64, mode):
    dev.set_growth_mode(mode)
    try:
        for name in ("default", "minima"):
            test_fp64_catalogue_matches_reference(dev, golden_box32_f64, name)
    finally:
        dev.set_growth_mode(0)


@pytest.mark.parametrize("mode", [0, 1, 2], ids=["auto", "cta", "warp"])
@pytest.mark.parametrize("name", ["minima_f1", "extend_minima_f1", "extend_f1", "extend"])
def test_fp64_catalogue_extended_reach(dev, golden_box32_extend_f64, name, mode):
    """SIF_FINDER_EXTEND_REACH in the FP64 form: the reference's
    SIF_USE_DOUBLE catalogues, with and without it, on its own fields."""
    dev.set_growth_mode(mode)
    try:
        test_fp64_catalogue_matches_reference(dev, golden_box32_extend_f64, name)
    finally:
        dev.set_growth_mode(0)


@pytest.mark.parametrize("mode", [0, 1, 2], ids=["auto", "cta", "warp"])
@pytest.mark.parametrize("name", ["peak", "peak_no_displace", "cells_f0", "cells_f05",
                                  "minima_f05", "lagrangian"])
def test_fp64_catalogue_displacement(dev, golden_box32_displace_f64, name, mode):
    """SIF_FINDER_DISPLACE in the FP64 form: the reference's SIF_USE_DOUBLE
    catalogues (the excursion-peak preset among them) on its own fields."""
    dev.set_growth_mode(mode)
    try:
        test_fp64_catalogue_matches_reference(dev, golden_box32_displace_f64, name)
    finally:
        dev.set_growth_mode(0)


@pytest.mark.parametrize("window", ["full", "aliasing", "none"])
def test_fp64_smoothing_against_oracle(dev, oracle, golden_box32_f64, window):
    g = golden_box32_f64
    n, box, _, _ = _params(g)
    mode = {"none": 0, "full": 1, "aliasing": 2}[window]
    # The oracle's double smoothing takes a float grid and float radii: give
    # both the same.
    radii = np.sort(g["radii"])[::-1][:4].astype(np.float32).astype(np.float64)
    d32 = g["delta"].astype(np.float32)
    want = oracle.smooth(d32, n, box, radii, window_mode=mode, mode=0, want="f64")
    (delta,) = _cuda(d32.astype(np.float64))
    for i, r in enumerate(radii):
        got = dev.smooth(delta, n, box, float(r), window=window).cpu().numpy()
        l2, mx = _rel(got, want[i])
        assert l2 <= 1e-12 and mx <= 1e-11, (r, l2, mx)


def test_fp64_box_path_is_its_stages(dev):
    """sifg_box_device_f64 = CIC, contrast, mesh and the finder called one by one."""
    x, y, z = synth.zeldovich(48, 200.0, 4.0, 77)
    xs = _cuda(*(a.astype(np.float64) for a in (x, y, z)))
    radii = synth.ladder(5.0, 15.0, 0.1).astype(np.float64)
    whole = dev.box(*xs, 48, 200.0, 12, radii, -0.75)
    grid = dev.cic(*xs, 48, 200.0)
    dev.density_contrast(grid)
    mesh = dev.chain_mesh(*xs, 12, 200.0)
    staged = dev.exodus(grid, 48, 200.0, mesh, 12, radii, -0.75)
    assert len(whole[0]) > 0 and same_catalogue64(whole, staged)
    # The float form on the same particles finds nearly the same voids.
    f32 = dev.box(*_cuda(x, y, z), 48, 200.0, 12, radii.astype(np.float32), -0.75)
    assert abs(len(f32[0]) - len(whole[0])) <= max(2, len(whole[0]) // 10)
