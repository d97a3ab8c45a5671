"""Weighted meshes on the GPU (sif_field_assign_weights; the weighted CIC,
grid.c:635-639; the mesh's weight columns, chain_mesh.c:624-672, 800-801;
sif__exodus_find_radius_weighted, exodus_rescale.c:642-1037; the weight
checks, exodus_finder.c:1076-1106), against the reference's own weighted
runs (tests/golden/golden_box32_weighted*.npz) and its test_finders.c weight
cases: weights of 1 and of 4 change nothing, voids that exist only in the
weights are found, negative and non-finite weights are refused.

Bars: the mesh's weight columns and the catalogue bit for bit (the weights
here are float32 values whose double sums are exact, where the GPU's
fixed-point sums give the reference's doubles); the weighted CIC against its
FP64 restatement within 1e-6 relative L2.
"""
import numpy as np
import pytest

from conftest import same_bits, same_bits64, same_catalogue, same_catalogue64
from sif_gb300 import synth

pytestmark = pytest.mark.gpu

WEIGHTED_SETS = ["default", "minima", "extend_minima_f1", "peak", "lagrangian"]


def _cuda(*arrays):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrays]


@pytest.fixture(scope="module")
def dev(gpu_lib):
    from sif_gb300 import device

    return device


def _params(g):
    return int(g["params"][0]), float(g["params"][1]), float(g["params"][5]), int(g["params"][6])


@pytest.mark.parametrize("which", ["rand", "holes"])
def test_weighted_mesh_columns_are_the_reference(dev, golden_box32_weighted, which):
    g = golden_box32_weighted
    n, box, _, n_mesh = _params(g)
    x, y, z, w = _cuda(*(g[f"{which}_{k}"] for k in "xyzw"))
    mesh = dev.chain_mesh(x, y, z, n_mesh, box, with_indices=True)
    assert np.array_equal(mesh[4].cpu().numpy().astype(np.uint64), g[f"{which}_mesh_index"])
    mw, cw, tot = dev.mesh_weights(w, mesh, n_mesh)
    assert same_bits(mw.cpu().numpy(), g[f"{which}_mesh_w"])
    assert same_bits(cw.cpu().numpy(), g[f"{which}_mesh_cell_w"])
    assert tot == float(g[f"{which}_total_weight"])


@pytest.mark.parametrize("which,name", [("rand", s) for s in WEIGHTED_SETS] + [("holes", "default")])
def test_weighted_catalogue_is_the_reference(dev, golden_box32_weighted, which, name):
    """On the fields the reference's own weighted run smoothed, with its
    mesh and weight columns: its catalogue bit for bit, under every option set
    recorded (the excursion-peak preset's displacement among them)."""
    g = golden_box32_weighted
    n, box, thr, n_mesh = _params(g)
    overlap, opt = g[f"{which}_cat_{name}_opt"]
    mesh = _cuda(g[f"{which}_mesh_x"], g[f"{which}_mesh_y"], g[f"{which}_mesh_z"],
                 g[f"{which}_mesh_offsets"].astype(np.int32))
    mw, cw = _cuda(g[f"{which}_mesh_w"], g[f"{which}_mesh_cell_w"])
    delta, fields = _cuda(g[f"{which}_delta"], g[f"{which}_fields"].reshape(-1))
    cat = dev.exodus(delta, n, box, mesh, n_mesh, g["radii"], thr, float(overlap), int(opt),
                     inject=fields, weights=(mw, cw, float(g[f"{which}_total_weight"])))
    want = tuple(g[f"{which}_cat_{name}_{k}"] for k in ("cx", "cy", "cz", "r"))
    assert len(cat[0]) == len(want[0])
    assert same_catalogue(cat, want)


@pytest.mark.parametrize("name", ["default", "extend_minima_f1", "peak"])
def test_weighted_catalogue_fp64_is_the_reference(dev, golden_box32_weighted_f64, name):
    """The FP64 form against the reference's SIF_USE_DOUBLE build: its mesh
    weight columns and its catalogue, bit for bit."""
    g = golden_box32_weighted_f64
    n, box, thr, n_mesh = _params(g)
    x, y, z, w = _cuda(*(np.asarray(g[f"rand_{k}"], np.float64) for k in "xyzw"))
    mesh = dev.chain_mesh(x, y, z, n_mesh, box, with_indices=True)
    mw, cw, tot = dev.mesh_weights(w, mesh, n_mesh)
    assert same_bits64(mw.cpu().numpy(), g["rand_mesh_w"])
    assert same_bits64(cw.cpu().numpy(), g["rand_mesh_cell_w"])
    assert tot == float(g["rand_total_weight"])
    overlap, opt = g[f"rand_cat_{name}_opt"]
    delta, fields = _cuda(g["rand_delta"], g["rand_fields"].reshape(-1))
    cat = dev.exodus(delta, n, box, mesh, n_mesh, g["radii"], thr, float(overlap), int(opt),
                     inject=fields, weights=(mw, cw, tot))
    want = tuple(g[f"rand_cat_{name}_{k}"] for k in ("cx", "cy", "cz", "r"))
    assert len(cat[0]) == len(want[0])
    assert same_catalogue64(cat, want)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_weighted_cic_against_fp64(dev, oracle, dtype):
    x, y, z = synth.zeldovich(64, 250.0, 4.0, 7)
    rng = np.random.default_rng(7)
    w = rng.uniform(0.0, 3.0, len(x)).astype(np.float32)
    w[rng.random(len(x)) < 0.1] = 0.0
    args = _cuda(*(np.asarray(a, dtype) for a in (x, y, z, w)))
    got = dev.cic_weighted(*args, 64, 250.0).cpu().numpy().astype(np.float64)
    want = oracle.cic_f64(x, y, z, 64, 250.0, weights=w)
    rms = np.sqrt((want * want).mean())
    assert np.sqrt(((got - want) ** 2).mean()) / rms < 1e-6


def _pipeline(pysif, x, y, z, w, n, box, n_mesh, radii, thr):
    f = pysif.Field(x, y, z, weights=w)
    g = pysif.Grid(n, box)
    g.assign_cic(f)
    dens = g.values.copy()
    g.to_density_contrast()
    m = pysif.ChainMesh(n_mesh, box, f, drop_indices=True)
    cat = pysif.finders.exodus_raw(g, m, radii, thr, checkpoint=False).as_tuple()
    return dens, g.values.copy(), cat


def test_uniform_weights_change_nothing(gpu_lib, golden_box32_weighted):
    """tests/test_finders.c:335-356 through the C API: weights of 1 give the
    unweighted density, contrast and catalogue bit for bit; weights of 4 four
    times the density and the same contrast and catalogue."""
    pysif = gpu_lib
    g = golden_box32_weighted
    n, box, thr, n_mesh = _params(g)
    x, y, z = (g[f"rand_{k}"] for k in "xyz")
    d0, c0, cat0 = _pipeline(pysif, x, y, z, None, n, box, n_mesh, g["radii"], thr)
    d1, c1, cat1 = _pipeline(pysif, x, y, z, np.ones(len(x), np.float32), n, box, n_mesh,
                             g["radii"], thr)
    d4, c4, cat4 = _pipeline(pysif, x, y, z, np.full(len(x), 4.0, np.float32), n, box, n_mesh,
                             g["radii"], thr)
    assert same_bits(d1, d0) and same_bits(c1, c0) and same_catalogue(cat1, cat0)
    assert same_bits(d4, 4.0 * d0) and same_bits(c4, c0) and same_catalogue(cat4, cat0)
    assert len(cat0[0]) > 0


def test_voids_only_in_the_weights(gpu_lib, golden_box32_weighted):
    """tests/test_finders.c:360-381: uniform tracers whose weights are 0
    inside three spheres; through the whole C API path the three voids are
    found, within a grid cell of the reference's centres and a few per cent
    of its radii (the GPU's deposit sums exactly where the reference's float
    sums round, so the fields differ in their last bits)."""
    pysif = gpu_lib
    g = golden_box32_weighted
    n, box, thr, n_mesh = _params(g)
    x, y, z, w = (g[f"holes_{k}"] for k in "xyzw")
    _, _, cat = _pipeline(pysif, x, y, z, w, n, box, n_mesh, g["radii"], thr)
    want = tuple(g[f"holes_cat_default_{k}"] for k in ("cx", "cy", "cz", "r"))
    assert len(cat[0]) == len(want[0]) == 3
    cell = box / n
    for i in range(3):
        assert max(abs(cat[k][i] - want[k][i]) for k in range(3)) <= cell
        assert abs(cat[3][i] / want[3][i] - 1.0) < 0.03


def test_bad_weights_are_refused(gpu_lib, golden_box32_weighted):
    """exodus_finder.c:1076-1106 and grid.c:1223-1230 (tests/test_finders.c:
    383-407): a negative weight refuses the finder; a NaN weight leaves a grid
    that does not normalise and a mesh the finder refuses; a negative zero
    passes."""
    pysif = gpu_lib
    g = golden_box32_weighted
    n, box, thr, n_mesh = _params(g)
    x, y, z, w = (g[f"rand_{k}"] for k in "xyzw")
    radii = g["radii"][:3]
    clean = pysif.Field(x, y, z, weights=w)
    grid = pysif.Grid(n, box)
    grid.assign_cic(clean)
    grid.to_density_contrast()
    for bad in (-1.0, np.nan, np.inf):
        wb = w.copy()
        wb[len(wb) // 2] = bad
        m = pysif.ChainMesh(n_mesh, box, pysif.Field(x, y, z, weights=wb), drop_indices=True)
        with pytest.raises(ValueError, match="finite and non-negative"):
            pysif.finders.exodus_raw(grid, m, radii, thr, checkpoint=False)
    wz = w.copy()
    wz[len(wz) // 2] = -0.0
    m = pysif.ChainMesh(n_mesh, box, pysif.Field(x, y, z, weights=wz), drop_indices=True)
    pysif.finders.exodus_raw(grid, m, radii, thr, checkpoint=False)
    wn = w.copy()
    wn[len(wn) // 2] = np.nan
    gn = pysif.Grid(n, box)
    gn.assign_cic(pysif.Field(x, y, z, weights=wn))
    with pytest.raises(ValueError, match="mean density"):
        gn.to_density_contrast()
