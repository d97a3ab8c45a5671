"""The allocation-free chain-mesh build (sifg_mesh_device_noalloc), for callers
that cannot let the library allocate device memory -- a process whose
framework already reserved the GPU's memory in its own pool, a pipeline that
cannot wait on cudaFree. Called through the C ABI, its mesh must equal the
allocating build's bit for bit, two calls in a row, and inputs past its fixed
scratch must be refused with SIF_ERR_RANGE."""
import ctypes as C

import numpy as np
import pytest

from sif_gb300 import abi, synth

pytestmark = pytest.mark.gpu


def _mesh_noalloc(lib, xs, n_cells, box):
    import torch

    n = xs[0].numel()
    out = [torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(3)]
    offs = torch.empty(n_cells ** 3 + 1, dtype=torch.int32, device="cuda")
    orig = torch.empty(n, dtype=torch.int32, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    st = lib.sifg_mesh_device_noalloc(p(xs[0]), p(xs[1]), p(xs[2]), n, n_cells, box,
                                      p(out[0]), p(out[1]), p(out[2]), p(offs), p(orig))
    return st, out + [offs, orig]


def test_noalloc_mesh_matches_the_allocating_build(gpu_lib):
    import torch

    from sif_gb300 import _lib, device

    lib = _lib.load()
    # Two calls in a row, then one at the limits: 100^3 = 1,000,000 particles
    # in 64^3 cells, whose offsets take the scan's multi-block path and the
    # static scratch's chunk totals to their last slots.
    cases = [(48, 200.0, 5.0, 51, 20), (40, 150.0, 4.0, 52, 13), (100, 400.0, 5.0, 53, 64)]
    for n, box, rms, seed, n_cells in cases:
        x, y, z = synth.zeldovich(n, box, rms, seed)
        xs = [torch.from_numpy(a).cuda() for a in (x, y, z)]
        st, got = _mesh_noalloc(lib, xs, n_cells, box)
        assert st == abi.SIF_OK, lib.sif_error_message()
        want = device.chain_mesh(*xs, n_cells, box)
        for a, b in zip(got, want):
            assert torch.equal(a, b)


def test_noalloc_mesh_refuses_inputs_past_its_scratch(gpu_lib):
    import torch

    from sif_gb300 import _lib

    lib = _lib.load()
    xs = [torch.zeros(16, dtype=torch.float32, device="cuda") for _ in range(3)]
    st, _ = _mesh_noalloc(lib, xs, 65, 100.0)  # 65^3 cells > 2^18
    assert st == abi.SIF_ERR_RANGE
    assert b"fixed scratch" in lib.sif_error_message()


def test_noalloc_mesh_refuses_a_side_that_would_wrap_when_cubed(gpu_lib):
    """2^22 cells a side: its cube wraps to 0 in 64 bits, so the side itself
    is bounded before it is cubed."""
    import torch

    from sif_gb300 import _lib

    lib = _lib.load()
    xs = [torch.zeros(16, dtype=torch.float32, device="cuda") for _ in range(3)]
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    st = lib.sifg_mesh_device_noalloc(p(xs[0]), p(xs[1]), p(xs[2]), 16, 1 << 22, 100.0,
                                      p(xs[0]), p(xs[1]), p(xs[2]), p(xs[0]), p(xs[1]))
    assert st == abi.SIF_ERR_RANGE
    assert b"fixed scratch" in lib.sif_error_message()


@pytest.mark.parametrize("bad", ["past_the_face", "nan"])
def test_noalloc_mesh_checks_the_box(gpu_lib, bad):
    """sif__field_check_in_box: a coordinate further than 4 float epsilons of
    the box past a face, or not a number, is refused with SIF_ERR_RANGE; one
    within that tolerance is folded and accepted."""
    import torch

    from sif_gb300 import _lib, device

    lib = _lib.load()
    box = np.float32(100.0)
    x, y, z = synth.zeldovich(16, float(box), 2.0, 54)
    tol = float(box) * 4.0 * float(np.finfo(np.float32).eps)
    x = x.copy()
    x[7] = np.nextafter(np.float32(float(box) + tol), np.float32(1e9))
    if bad == "nan":
        x[7] = np.float32(np.nan)
    xs = [torch.from_numpy(a).cuda() for a in (x, y, z)]
    st, _ = _mesh_noalloc(lib, xs, 8, float(box))
    assert st == abi.SIF_ERR_RANGE
    assert b"outside the box" in lib.sif_error_message()
    # Within the tolerance: folded, and the same mesh as the allocating build.
    x[7] = np.float32(float(box))
    xs = [torch.from_numpy(a).cuda() for a in (x, y, z)]
    st, got = _mesh_noalloc(lib, xs, 8, float(box))
    assert st == abi.SIF_OK, lib.sif_error_message()
    for a, b in zip(got, device.chain_mesh(*xs, 8, float(box))):
        assert torch.equal(a, b)
