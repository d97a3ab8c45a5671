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
    cases = [(48, 200.0, 5.0, 51, 20), (40, 150.0, 4.0, 52, 13)]  # two calls in a row
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
