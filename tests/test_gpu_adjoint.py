"""The adjoint of deposit + smoothing (sif_gb300.autograd) against central
finite differences of the FP64 forward, and the float form's gradient
against the FP64 form's.

The loss is the workload's: the sum of the squared smoothed contrast over the
cells within 2R of fixed void centres. A CIC weight is linear within a cell,
so the loss is quadratic in a particle's coordinate there and a central
difference is exact but for rounding -- except across a cell face, where the
weight has a kink; a few such particles are allowed to differ.
"""
import numpy as np
import pytest

from sif_gb300 import synth

pytestmark = pytest.mark.gpu

N, BOX, R = 32, 128.0, 6.0


def _setup(dtype, seed=3):
    import torch

    x, y, z = synth.zeldovich(N, BOX, 4.0, seed)
    xs = [torch.from_numpy(a.astype(dtype)).cuda() for a in (x, y, z)]
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0, BOX, (3, 3))
    q = (np.arange(N) + 0.0) * (BOX / N)
    gx, gy, gz = np.meshgrid(q, q, q, indexing="ij")
    mask = np.zeros((N, N, N), bool)
    for c in centres:
        d = [np.abs(g - ci) for g, ci in zip((gx, gy, gz), c)]
        d = [np.minimum(a, BOX - a) for a in d]
        mask |= d[0] ** 2 + d[1] ** 2 + d[2] ** 2 <= (2 * R) ** 2
    return xs, torch.from_numpy(mask.reshape(-1)).cuda()


def _loss(xs, mask, filt):
    from sif_gb300 import autograd

    s = autograd.smoothed_contrast(*xs, N, BOX, R, filter=filt)
    return (s[mask] ** 2).sum()


def _grad(xs, mask, filt):
    xs = [a.clone().requires_grad_(True) for a in xs]
    _loss(xs, mask, filt).backward()
    return [a.grad.cpu().numpy() for a in xs]


@pytest.mark.parametrize("filt", ["gaussian", "top-hat"])
def test_adjoint_matches_fp64_central_differences(gpu_lib, filt):
    import torch

    xs, mask = _setup(np.float64)
    grads = _grad(xs, mask, filt)
    rng = np.random.default_rng(11)
    h = 1e-3
    errs = []
    for p in rng.choice(N ** 3, 40, replace=False):
        for a in range(3):
            vals = []
            for sgn in (1.0, -1.0):
                moved = [t.clone() for t in xs]
                v = float(moved[a][p]) + sgn * h
                moved[a][p] = v - BOX if v >= BOX else (v + BOX if v < 0 else v)
                with torch.no_grad():
                    vals.append(float(_loss(moved, mask, filt)))
            fd = (vals[0] - vals[1]) / (2 * h)
            g = grads[a][p]
            errs.append(abs(fd - g) / max(abs(fd), abs(g), 1e-3))
    errs = np.array(errs)
    assert np.median(errs) < 1e-6, np.median(errs)
    assert (errs < 1e-4).mean() >= 0.95, np.sort(errs)[-10:]


def test_float_gradient_matches_fp64(gpu_lib):
    xs64, mask = _setup(np.float64)
    xs32 = [a.float() for a in xs64]
    g64 = np.concatenate(_grad(xs64, mask, "gaussian"))
    g32 = np.concatenate(_grad(xs32, mask, "gaussian")).astype(np.float64)
    rel = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
    assert rel < 1e-5, rel


def test_adjoint_is_the_transpose_of_the_forward(gpu_lib):
    """<J^T g, v> = <g, J v> with J v from a central difference along v."""
    import torch

    from sif_gb300 import autograd

    xs, _ = _setup(np.float64, seed=8)
    rng = np.random.default_rng(2)
    g = torch.from_numpy(rng.standard_normal(N ** 3)).cuda()
    v = [torch.from_numpy(rng.standard_normal(N ** 3) * 1e-4).cuda() for _ in range(3)]
    xg = [a.clone().requires_grad_(True) for a in xs]
    (autograd.smoothed_contrast(*xg, N, BOX, R) * g).sum().backward()
    lhs = sum(float((a.grad * b).sum()) for a, b in zip(xg, v))
    with torch.no_grad():
        fp = autograd.smoothed_contrast(*[(a + b) % BOX for a, b in zip(xs, v)], N, BOX, R)
        fm = autograd.smoothed_contrast(*[(a - b) % BOX for a, b in zip(xs, v)], N, BOX, R)
    rhs = float(((fp - fm) * 0.5 * g).sum())
    assert abs(lhs - rhs) <= 1e-3 * abs(lhs), (lhs, rhs)
