"""Exodus checkpoints through sif's C API on the GPU (the XCKP v3 file,
include/sif/finder/exodus_finder.h:409-507; run_start, checkpoint_rung and
checkpoint_finish, src/finder/exodus_finder.c:1384-1574).

As the reference's tests/test_finders.c:673-745 and
tests/python/test_checkpoint.py do: a run stopped after some rungs (the halt
hook) keeps its checkpoint; resumed from it, it returns the catalogue of a
run never stopped, bit for bit; a checkpoint of another run is refused; a
finished run removes its checkpoint unless asked to keep it.
"""
import os
import struct
import zlib

import numpy as np
import pytest

from conftest import same_catalogue

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def box(gpu_lib):
    from test_oracle import _holes_field

    pysif = gpu_lib
    x, y, z, _ = _holes_field()
    f = pysif.Field(x, y, z)
    g = pysif.Grid(32, 200.0)
    g.assign_cic(f)
    g.to_density_contrast()
    m = pysif.ChainMesh(8, 200.0, f, drop_indices=True)
    return pysif, g, m, np.array([30, 25, 20, 16, 13, 10, 8, 6.5], np.float32)


def _halt(pysif, n):
    from sif_gb300 import _lib

    _lib.load().sifg_set_halt_after(n)


def test_halted_run_resumes_to_the_uninterrupted_catalogue(box, tmp_path):
    pysif, g, m, radii = box
    whole = pysif.finders.exodus(g, m, radii, -0.7, checkpoint=str(tmp_path / "none.ckpt")).as_tuple()
    assert not os.path.exists(tmp_path / "none.ckpt")  # removed on success
    path = str(tmp_path / "run.ckpt")
    for halt in (3, 6):
        if os.path.exists(path):
            os.remove(path)
        _halt(pysif, halt)
        try:
            with pytest.raises(ValueError, match="halted"):
                pysif.finders.exodus(g, m, radii, -0.7, checkpoint=path)
        finally:
            _halt(pysif, 0)
        assert os.path.exists(path)
        cat, h = pysif.finders.checkpoint_read(path)
        assert h["next_rung"] == halt and h["n_radii"] == len(radii) and h["version"] == 3
        assert h["threshold"] == np.float32(-0.7) and h["grid_n_cells"] == 32
        # The catalogue so far is the uninterrupted run's first voids.
        part = cat.as_tuple()
        assert all(np.array_equal(a, b[: len(a)]) for a, b in zip(part, whole))
        # The file's CRC-32 (zlib's) over the header with its crc field zero
        # and everything after it.
        raw = bytearray(open(path, "rb").read())
        assert raw[:4] == b"XCKP"
        crc = struct.unpack_from("<I", raw, 132)[0]
        raw[132:136] = b"\0\0\0\0"
        assert zlib.crc32(bytes(raw)) == crc
        resumed = pysif.finders.exodus(g, m, radii, -0.7, checkpoint=path,
                                       keep_checkpoint=True).as_tuple()
        assert same_catalogue(resumed, whole)
        assert os.path.exists(path)  # kept, as asked
        _, h2 = pysif.finders.checkpoint_read(path)
        assert h2["next_rung"] == len(radii) and h2["n_voids"] == len(whole[0])


def test_checkpoint_of_another_run_is_refused(box, tmp_path):
    pysif, g, m, radii = box
    path = str(tmp_path / "other.ckpt")
    _halt(pysif, 2)
    try:
        with pytest.raises(ValueError):
            pysif.finders.exodus(g, m, radii, -0.7, checkpoint=path)
    finally:
        _halt(pysif, 0)
    with pytest.raises(ValueError, match="not this run"):
        pysif.finders.exodus(g, m, radii, -0.75, checkpoint=path)  # another threshold
    with pytest.raises(ValueError, match="not this run"):
        pysif.finders.exodus(g, m, radii[:-1], -0.7, checkpoint=path)  # another ladder
    # Damaged: refused before any rung runs.
    raw = bytearray(open(path, "rb").read())
    raw[-1] ^= 1
    open(path, "wb").write(bytes(raw))
    with pytest.raises(ValueError, match="checksum"):
        pysif.finders.exodus(g, m, radii, -0.7, checkpoint=path)


def test_default_checkpoint_is_written_and_removed(box, tmp_path, monkeypatch):
    """A variant without a named checkpoint writes exodus-<hex>.ckpt in the
    working directory and removes it when the run succeeds; exodus_raw with
    checkpoint=False writes none."""
    pysif, g, m, radii = box
    monkeypatch.chdir(tmp_path)
    pysif.finders.exodus(g, m, radii, -0.7)
    pysif.finders.exodus_raw(g, m, radii, -0.7)
    assert os.listdir(tmp_path) == []
    _halt(pysif, 4)
    try:
        with pytest.raises(ValueError):
            pysif.finders.exodus(g, m, radii, -0.7)
    finally:
        _halt(pysif, 0)
    left = os.listdir(tmp_path)
    assert len(left) == 1 and left[0].startswith("exodus-") and left[0].endswith(".ckpt")
