"""The batched form (sifg_box_batch_device): every box's catalogue is the
one sifg_box_device gives for it alone, whatever the number of engines run
at once, and a failing box fails alone."""
import numpy as np
import pytest

from conftest import same_catalogue
from sif_gb300 import abi, synth

pytestmark = pytest.mark.gpu

SPECS = [(48, 200.0, 12, 31), (24, 150.0, 8, 32), (40, 300.0, 10, 33), (32, 100.0, 9, 34),
         (56, 250.0, 12, 35)]


def _boxes():
    import torch

    out = []
    for n, box, mesh, seed in SPECS:
        x, y, z = synth.zeldovich(n, box, 4.0, seed)
        r0 = 2.0 * box / n
        out.append(dict(x=torch.from_numpy(x).cuda(), y=torch.from_numpy(y).cuda(),
                        z=torch.from_numpy(z).cuda(), n_grid=n, box=box, mesh_cells=mesh,
                        radii=synth.ladder(r0, 6 * r0, 0.1).astype(np.float32), threshold=-0.8))
    return out


@pytest.fixture(scope="module")
def dev(gpu_lib):
    from sif_gb300 import device

    return device


def test_batch_equals_boxes_run_alone(dev):
    boxes = _boxes()
    alone = [dev.box(b["x"], b["y"], b["z"], b["n_grid"], b["box"], b["mesh_cells"], b["radii"],
                     b["threshold"]) for b in boxes]
    assert sum(len(c[0]) for c in alone) > 0
    for engines in (1, 3, 0):
        cats, used = dev.box_batch(boxes, engines=engines)
        assert used >= 1
        for got, want in zip(cats, alone):
            assert len(got[0]) == len(want[0]) and same_catalogue(got, want), engines


def test_batch_suggested_mesh_gives_the_same_catalogue(dev):
    """mesh_cells 0 picks sif_finder_suggest_mesh_cells; the catalogue does
    not depend on the mesh."""
    boxes = _boxes()[:3]
    want, _ = dev.box_batch(boxes, engines=2)
    for b in boxes:
        b["mesh_cells"] = 0
    got, _ = dev.box_batch(boxes, engines=2)
    for g, w in zip(got, want):
        assert same_catalogue(g, w)


def test_a_failing_box_fails_alone(dev):
    boxes = _boxes()[:3]
    bad = boxes[1]["x"].clone()
    bad[5] = 2.0 * boxes[1]["box"]
    boxes[1]["x"] = bad
    cats, _, status = dev.box_batch(boxes, engines=2, check=False)
    assert status[1] == abi.SIF_ERR_RANGE
    assert status[0] == abi.SIF_OK and status[2] == abi.SIF_OK
    assert len(cats[1][0]) == 0 and len(cats[0][0]) > 0
