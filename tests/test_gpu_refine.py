"""SIF_FINDER_REFINE_GAUSSIAN on the GPU (sif__finder_scan_refined,
src/finder/utils.c:406-552; candidate_centre and masked_overlap,
src/finder/exodus_finder.c:371-452), against the reference's own refined runs
(tests/golden/golden_box32_refine*.npz): on the fields its transforms
returned, in order, the catalogue bit for bit under cell and minima seeds, an
overlap fraction, the excursion-peak preset and the Lagrangian scale, in the
float form and the FP64 form; and the refinement through sif's C API
(pysif's refine_centres='gaussian'), where the GPU smooths on its own.
"""
import numpy as np
import pytest

from conftest import refine_fields, same_catalogue, same_catalogue64

pytestmark = pytest.mark.gpu

REFINE_SETS = ["cells", "minima", "minima_f05", "peak", "lagrangian"]


def _cuda(*arrays):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrays]


@pytest.fixture(scope="module")
def dev(gpu_lib):
    from sif_gb300 import device

    return device


def _params(g):
    return int(g["params"][0]), float(g["params"][1]), float(g["params"][5]), int(g["params"][6])


def _run(dev, g, name):
    n, box, thr, n_mesh = _params(g)
    overlap, opt = g[f"cat_{name}_opt"]
    mesh = _cuda(g["mesh_x"], g["mesh_y"], g["mesh_z"], g["mesh_offsets"].astype(np.int32))
    delta, fields = _cuda(g["delta"], refine_fields(g, name).reshape(-1))
    return dev.exodus(delta, n, box, mesh, n_mesh, g["radii"], thr, float(overlap), int(opt),
                      inject=fields)


@pytest.mark.parametrize("name", REFINE_SETS)
def test_refined_catalogue_is_the_reference(dev, golden_box32_refine, name):
    g = golden_box32_refine
    cat = _run(dev, g, name)
    want = tuple(g[f"cat_{name}_{k}"] for k in ("cx", "cy", "cz", "r"))
    assert len(cat[0]) == len(want[0])
    assert same_catalogue(cat, want)


@pytest.mark.parametrize("mode", [1, 2], ids=["cta", "warp"])
def test_refined_catalogue_either_growth_kernel(dev, golden_box32_refine, mode):
    dev.set_growth_mode(mode)
    try:
        for name in ("cells", "minima"):
            test_refined_catalogue_is_the_reference(dev, golden_box32_refine, name)
    finally:
        dev.set_growth_mode(0)


@pytest.mark.parametrize("name", ["cells", "minima", "peak"])
def test_refined_catalogue_fp64_is_the_reference(dev, golden_box32_refine_f64, name):
    g = golden_box32_refine_f64
    cat = _run(dev, g, name)
    want = tuple(g[f"cat_{name}_{k}"] for k in ("cx", "cy", "cz", "r"))
    assert cat[0].dtype == np.float64
    assert len(cat[0]) == len(want[0])
    assert same_catalogue64(cat, want)


def test_refinement_through_the_c_api(gpu_lib):
    """refine_centres='gaussian' through sif_finder_exodus_raw: the GPU's own
    smoothing of both fields; the refined run is not the unrefined one, and
    some centres sit between the nodes."""
    from sif_gb300 import synth

    pysif = gpu_lib
    x, y, z = synth.zeldovich(48, 200.0, 4.0, 21)
    f = pysif.Field(x, y, z)
    g = pysif.Grid(48, 200.0)
    g.assign_cic(f)
    g.to_density_contrast()
    m = pysif.ChainMesh(10, 200.0, f, drop_indices=True)
    radii = synth.ladder(6.0, 18.0, 0.1)
    plain = pysif.finders.exodus_raw(g, m, radii, -0.7, seeds="minima").as_tuple()
    refined = pysif.finders.exodus_raw(g, m, radii, -0.7, seeds="minima",
                                       refine_centres="gaussian").as_tuple()
    assert len(refined[0]) > 0
    cell = np.float32(200.0 / 48)
    off_node = [np.abs(c / cell - np.round(c / cell)) > 1e-3 for c in refined[:3]]
    assert np.any(off_node[0] | off_node[1] | off_node[2])
    assert not same_catalogue(plain, refined)
    with pytest.raises(NotImplementedError):
        pysif.finders.exodus_raw(g, m, radii, -0.7, refine_centres="hill")
