"""Device mirrors of the structs' host arrays (sifg_set_host_mirrors): the
C API pipeline (CIC, contrast, chain mesh, finder) gives the same density,
contrast, mesh and catalogue bits with mirrors on as with every array copied
on every call, while copying the positions up once and the grid and the mesh
not at all; and what the header promises for arrays the caller writes:
declared writes (sifg_host_modified) and the library's own writes are seen,
undeclared wholesale writes are caught by the sampled words, an undeclared
write that misses every sampled word is not.
"""
import numpy as np
import pytest

from conftest import same_bits, same_catalogue
from sif_gb300 import synth

pytestmark = pytest.mark.gpu

N, BOX, GRID, MESH, THR = 64, 250.0, 64, 25, -0.75


@pytest.fixture(scope="module")
def sif(gpu_lib):
    yield gpu_lib
    gpu_lib.set_host_mirrors(False)


@pytest.fixture(scope="module")
def particles():
    return synth.zeldovich(N, BOX, 4.0, 31)


def _radii():
    return synth.ladder(5.0, 20.0, 0.1)


def _pipeline(sif, field, grid):
    grid._ptr.contents.content = 0  # SIF_GRID_EMPTY: assign again
    before = sif.copy_bytes()
    grid.assign_cic(field)
    dens = grid.values.copy()
    grid.to_density_contrast()
    contrast = grid.values.copy()
    mesh = sif.ChainMesh(MESH, BOX, field, drop_indices=True)
    c = mesh._ptr.contents
    n = c.n_particles
    mesh_cols = [np.ctypeslib.as_array(a, shape=(n,)).copy() for a in (c.x, c.y, c.z)]
    cat = sif.finders.exodus_raw(grid, mesh, _radii(), THR, checkpoint=False).as_tuple()
    after = sif.copy_bytes()
    return dens, contrast, mesh_cols, cat, (after[0] - before[0], after[1] - before[1])


def test_pipeline_bits_and_copies(sif, particles):
    x, y, z = particles
    n = len(x)
    field = sif.Field(x, y, z)
    grid = sif.Grid(GRID, BOX)
    sif.set_host_mirrors(False)
    plain = _pipeline(sif, field, grid)
    sif.set_host_mirrors(True)
    try:
        first = _pipeline(sif, field, grid)
        again = _pipeline(sif, field, grid)
    finally:
        sif.set_host_mirrors(False)
    for run in (first, again):
        assert same_bits(run[0], plain[0]) and same_bits(run[1], plain[1])
        assert all(same_bits(a, b) for a, b in zip(run[2], plain[2]))
        assert same_catalogue(run[3], plain[3]) and len(plain[3][0]) > 0
    cells, mcells = GRID ** 3, MESH ** 3 + 1
    # Without mirrors: positions twice, the grid twice, the mesh (positions
    # and 64-bit offsets) once.
    assert plain[4][0] == 2 * 12 * n + 2 * 4 * cells + 12 * n + 8 * mcells
    # With them: the positions once on the first run, nothing after.
    assert first[4][0] == 12 * n
    assert again[4][0] == 0
    # What comes down is the same either way.
    assert first[4][1] == again[4][1] == plain[4][1]


def test_declared_and_library_writes_are_seen(sif, particles):
    x, y, z = particles
    field = sif.Field(x, y, z)
    grid = sif.Grid(GRID, BOX)
    sif.set_host_mirrors(True)
    try:
        grid.assign_cic(field)
        # One cell changed and declared: the contrast sees it.
        grid.values[0, 0, 1] += 3.0
        want = grid.values.copy()
        sif.host_modified(grid)
        grid.to_density_contrast()
        got = grid.values.copy()
        # New positions through the API: the next deposit sees them.
        x2 = np.ascontiguousarray(np.roll(x, 1) * 0.5, np.float32)
        field2 = sif.Field(x2, y, z)
        lib = sif._lib.load()
        assert lib.sif_field_assign_positions(field._ptr, sif._P(x2), sif._P(y), sif._P(z)) == 0
        grid._ptr.contents.content = 0
        grid.assign_cic(field)
        dens_new = grid.values.copy()
    finally:
        sif.set_host_mirrors(False)
    ref = sif.Grid(GRID, BOX)
    ref.values[...] = want
    ref._ptr.contents.content = 1  # SIF_GRID_DENSITY
    ref.to_density_contrast()
    assert same_bits(got, ref.values)
    ref2 = sif.Grid(GRID, BOX)
    ref2.assign_cic(field2)
    assert same_bits(dens_new, ref2.values)


def test_undeclared_writes(sif, particles):
    """A wholesale write is caught by the sampled words; a single word that
    no sample covers is read stale, as the header says, until declared."""
    x, y, z = particles
    field = sif.Field(x, y, z)
    grid = sif.Grid(GRID, BOX)
    sif.set_host_mirrors(True)
    try:
        grid.assign_cic(field)
        dens = grid.values.copy()
        grid.values[...] *= 2.0  # every word changes
        grid.to_density_contrast()
        scaled = grid.values.copy()
        grid._ptr.contents.content = 0
        grid.assign_cic(field)
        # Word 1 of the grid: samples fall on words (n - 1) k / 1023, so only
        # word 0 lies below word (n - 1) / 1023.
        grid.values.reshape(-1)[1] += 5.0
        grid.to_density_contrast()
        stale = grid.values.copy()
    finally:
        sif.set_host_mirrors(False)
    ref = sif.Grid(GRID, BOX)
    ref.values[...] = 2.0 * dens
    ref._ptr.contents.content = 1
    ref.to_density_contrast()
    assert same_bits(scaled, ref.values)
    ref.values[...] = dens
    ref._ptr.contents.content = 1
    ref.to_density_contrast()
    assert same_bits(stale, ref.values)


def test_freed_blocks_forget_their_mirrors(sif, particles):
    """A mesh freed and another built from other particles in the block the
    pool hands back: the finder reads the new mesh, not the old mirror."""
    x, y, z = particles
    sif.set_host_mirrors(True)
    try:
        f1 = sif.Field(x, y, z)
        m1 = sif.ChainMesh(MESH, BOX, f1, drop_indices=True)
        del m1
        rng = np.random.default_rng(5)
        xs = [np.ascontiguousarray(rng.uniform(0, BOX, len(x)), np.float32) for _ in range(3)]
        f2 = sif.Field(*xs)
        m2 = sif.ChainMesh(MESH, BOX, f2, drop_indices=True)
        grid = sif.Grid(GRID, BOX)
        grid.assign_cic(f2)
        grid.to_density_contrast()
        got = sif.finders.exodus_raw(grid, m2, _radii(), THR, checkpoint=False).as_tuple()
    finally:
        sif.set_host_mirrors(False)
    grid = sif.Grid(GRID, BOX)
    grid.assign_cic(f2)
    grid.to_density_contrast()
    m3 = sif.ChainMesh(MESH, BOX, f2, drop_indices=True)
    want = sif.finders.exodus_raw(grid, m3, _radii(), THR, checkpoint=False).as_tuple()
    assert same_catalogue(got, want)
