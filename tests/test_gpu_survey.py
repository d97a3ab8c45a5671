"""The survey finder on the GPU (sif_finder_exodus_survey_raw,
src/finder/exodus_survey.c; the survey branches of exodus_finder.c;
sif__exodus_find_radius_survey, exodus_rescale.c:2154-2317).

- On the fields the GPU smooths (data and randoms, every rung), injected into
  both: the GPU's catalogue and footprint columns are the oracle's, bit for
  bit, for the golden cases (selection, sparse randoms whose footprint needs
  closing, weights on both sides, the Lagrangian overlap, 527 voids).
- Through sif's C API end to end (CIC of both sets, both meshes, the survey
  finder with its own smoothing, a survey placed by survey_box and moved
  back): against the reference's own catalogue (tests/golden/
  golden_survey.npz), which ran the same path on its own float CIC and
  transforms: every reference void found within a grid cell and 1% of its
  radius, with its footprint within 0.01, on the cases with well-separated
  voids; at least 90% so matched where hundreds of voids crowd.
- The refusals the reference makes (exodus_survey.c:401-545, exodus_finder.c:
  1114-1137): box-only options, a contrast grid, a survey too close to the
  box's faces.
- A survey checkpoint (is_survey, the randoms, the offset in its header),
  halted and resumed to the same catalogue.
"""
import numpy as np
import pytest

import survey_cases as S
from conftest import same_bits
from sif_gb300 import abi, synth

pytestmark = pytest.mark.gpu

PARITY_CASES = ["sel", "sparse", "weighted", "lagrangian", "many"]


def _case(name):
    return next(c for c in S.SURVEY_CASES if c[0] == name)


def _cuda(*arrays):
    import torch

    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrays]


@pytest.fixture(scope="module")
def dev(gpu_lib):
    from sif_gb300 import device

    return device


def _gpu_inputs(dev, case, golden):
    """Positions in the box, the GPU's density grids and canonical meshes
    (with weight columns), and the case's radii."""
    spec = _case(case)
    data, rand, wd, wr, radii = S.survey_inputs(spec)
    box = float(golden[f"{case}_box"][0])
    if spec[7]:
        off = golden[f"{case}_box"][1:]
        data = tuple(np.float32(a + o) for a, o in zip(data, off))
        rand = tuple(np.float32(a + o) for a, o in zip(rand, off))
    n, nm = S.SURVEY_GRID, S.SURVEY_MESH
    out = []
    for pos, w in ((data, wd), (rand, wr)):
        xs = _cuda(*pos)
        if w is None:
            grid = dev.cic(*xs, n, box)
        else:
            (wt,) = _cuda(w)
            grid = dev.cic_weighted(*xs, wt, n, box)
        mesh = dev.chain_mesh(*xs, nm, box, with_indices=True)
        desc = list(mesh[:4]) + [nm, float(len(pos[0]))]
        if w is not None:
            mw, cw, tot = dev.mesh_weights(wt, mesh, nm)
            desc = list(mesh[:4]) + [nm, tot, mw, cw]
        out.append((grid, desc))
    return spec, data, rand, wd, wr, radii, box, out


@pytest.mark.parametrize("case", PARITY_CASES)
def test_survey_catalogue_is_the_oracle_on_gpu_fields(dev, oracle, golden_survey, case):
    import torch

    spec, data, rand, wd, wr, radii, box, ((dg, dmesh), (rg, rmesh)) = _gpu_inputs(
        dev, case, golden_survey)
    n = S.SURVEY_GRID
    fields = []
    for r in sorted(radii, reverse=True):
        fields.append(dev.smooth(dg, n, box, float(r)))
        fields.append(dev.smooth(rg, n, box, float(r)))
    inject = torch.cat(fields)
    got = dev.exodus_survey(dg, rg, n, box, dmesh, rmesh, radii, spec[3], 0.0, spec[6],
                            inject=inject)
    dm = oracle.OracleMesh(*data, S.SURVEY_MESH, box, weights=wd)
    rm = oracle.OracleMesh(*rand, S.SURVEY_MESH, box, weights=wr)
    for mesh, desc in ((dm, dmesh), (rm, rmesh)):
        assert np.array_equal(desc[0].cpu().numpy(), mesh.x)
        assert np.array_equal(desc[3].cpu().numpy().astype(np.uint64), mesh.offsets)
    want = oracle.exodus(dg.cpu().numpy(), dm, radii, n, box, spec[3], 0.0, spec[6], n_threads=8,
                         inject=inject.cpu().numpy(), survey=(rm, rg.cpu().numpy()))
    assert len(got[0]) == len(want[0]) > 0
    assert all(same_bits(a, b) for a, b in zip(got, want))


def _api_run(sif, case, golden, checkpoint=False, extras=None):
    spec = _case(case)
    data, rand, wd, wr, radii = S.survey_inputs(spec)
    fd = sif.Field(*data, weights=wd)
    fr = sif.Field(*rand, weights=wr)
    offset = None
    box = synth.SURVEY["box"]
    if spec[7]:
        offset, box = sif.finders.survey_box(fd, fr, radii)
        assert np.allclose(offset, golden[f"{case}_box"][1:]) and box == float(golden[f"{case}_box"][0])
        fd = sif.Field(*[np.float32(a + o) for a, o in zip(data, offset)], weights=wd)
        fr = sif.Field(*[np.float32(a + o) for a, o in zip(rand, offset)], weights=wr)
    gd, gr = sif.Grid(S.SURVEY_GRID, box), sif.Grid(S.SURVEY_GRID, box)
    gd.assign_cic(fd)
    gr.assign_cic(fr)
    md = sif.ChainMesh(S.SURVEY_MESH, box, fd, drop_indices=True)
    mr = sif.ChainMesh(S.SURVEY_MESH, box, fr, drop_indices=True)
    overlap = "lagrangian" if spec[6] & abi.SIF_FINDER_LAGRANGIAN_OVERLAP else "eulerian"
    cat = sif.finders.exodus_survey_raw(gd, gr, md, mr, radii, spec[3], offset=offset,
                                        overlap_type=overlap, checkpoint=checkpoint, **(extras or {}))
    return cat, (gd, gr, md, mr, radii, spec, offset)


def _matched(got, want, cell):
    """How many of want's voids have one of got's within a cell, 1% of the
    radius and 0.01 of both footprints."""
    k = 0
    for i in range(len(want[0])):
        d = np.sqrt((got[0] - want[0][i]) ** 2 + (got[1] - want[1][i]) ** 2 +
                    (got[2] - want[2][i]) ** 2)
        ok = (d <= cell) & (np.abs(got[3] / want[3][i] - 1.0) < 0.01) & \
             (np.abs(got[4] - want[4][i]) <= 0.01) & (np.abs(got[5] - want[5][i]) <= 0.01)
        k += bool(ok.any())
    return k


@pytest.mark.parametrize("case", [c[0] for c in S.SURVEY_CASES])
def test_survey_through_the_c_api_against_the_reference(gpu_lib, golden_survey, case):
    cat, (gd, *_rest) = _api_run(gpu_lib, case, golden_survey)
    got = (cat.cx, cat.cy, cat.cz, cat.radii, cat.footprint, cat.footprint_shell)
    want = [golden_survey[f"{case}_{k}"] for k in ("cx", "cy", "cz", "r", "foot", "shell")]
    cell = float(golden_survey[f"{case}_box"][0]) / S.SURVEY_GRID
    m = _matched(got, want, cell)
    print(f"{case}: {len(got[0])} voids against the reference's {len(want[0])}, {m} matched")
    if len(want[0]) <= 10:
        assert len(got[0]) == len(want[0]) == m
    else:
        assert m >= 0.9 * len(want[0]) and abs(len(got[0]) - len(want[0])) <= 0.1 * len(want[0])
    assert gd.values.min() >= 0.0  # the data grid handed back as it was given: a density


def test_survey_refusals(gpu_lib, golden_survey):
    sif = gpu_lib
    cat, (gd, gr, md, mr, radii, spec, _) = _api_run(sif, "sel", golden_survey)
    lib = sif._lib.load()
    r = np.ascontiguousarray(radii, np.float32)
    for opt in (abi.SIF_FINDER_SEEDS_MINIMA, abi.SIF_FINDER_REFINE_GAUSSIAN,
                abi.SIF_FINDER_EXTEND_REACH, abi.SIF_FINDER_DISPLACE):
        ptr = lib.sif_finder_exodus_survey_raw(gd._ptr, gr._ptr, md._ptr, mr._ptr, None, sif._P(r),
                                               len(r), -0.8, 0.0, opt | abi.SIF_FINDER_NO_CHECKPOINT,
                                               None)
        assert not ptr and lib.sif_error_status() == abi.SIF_ERR_INVALID
        assert b"a survey" in lib.sif_error_message()
    with pytest.raises(Exception):
        sif.finders.exodus_survey(gd, gr, md, mr, radii, -0.8, "excursion-peak")
    # A grid already turned into a contrast against the box mean.
    gc = sif.Grid(S.SURVEY_GRID, synth.SURVEY["box"])
    data, rand, *_ = S.survey_inputs(_case("sel"))
    gc.assign_cic(sif.Field(*data))
    gc.to_density_contrast()
    with pytest.raises(ValueError, match="density contrast"):
        sif.finders.exodus_survey_raw(gc, gr, md, mr, radii, -0.8)
    # A survey too close to the faces: the data moved 50 toward one.
    moved = [np.float32(a - 50.0) if k == 0 else a for k, a in enumerate(data)]
    fm = sif.Field(*moved)
    gm = sif.Grid(S.SURVEY_GRID, synth.SURVEY["box"])
    gm.assign_cic(fm)
    mm = sif.ChainMesh(S.SURVEY_MESH, synth.SURVEY["box"], fm, drop_indices=True)
    with pytest.raises(ValueError, match="padding"):
        sif.finders.exodus_survey_raw(gm, gr, mm, mr, radii, -0.8)


def test_survey_checkpoint_resumes(gpu_lib, golden_survey, tmp_path):
    sif = gpu_lib
    path = str(tmp_path / "survey.ckpt")
    full, _ = _api_run(sif, "offset", golden_survey)
    lib = sif._lib.load()
    lib.sifg_set_halt_after(5)
    try:
        with pytest.raises(Exception):
            _api_run(sif, "offset", golden_survey, checkpoint=path)
    finally:
        lib.sifg_set_halt_after(0)
    saved, header = sif.finders.checkpoint_read(path)
    assert header["is_survey"] == 1 and header["next_rung"] == 5
    assert header["random_n_particles"] == _case("offset")[2]
    resumed, _ = _api_run(sif, "offset", golden_survey, checkpoint=path)
    for a, b in zip((resumed.cx, resumed.cy, resumed.cz, resumed.radii, resumed.footprint,
                     resumed.footprint_shell),
                    (full.cx, full.cy, full.cz, full.radii, full.footprint, full.footprint_shell)):
        assert same_bits(a, b)
    # The saved voids, read back, in the caller's frame: the resumed run's first ones.
    k = len(saved.cx)
    assert k > 0 and same_bits(saved.radii, full.radii[:k])
    assert np.allclose(saved.cx, full.cx[:k], atol=1e-3)
