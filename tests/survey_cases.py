"""The survey finder's test cases: the inputs the golden generator ran the
reference on (tests/golden/golden_survey.npz) and the tests regenerate,
checked against the SHA-256 stored beside each catalogue."""
import numpy as np

from sif_gb300 import abi, synth

# Survey cases: (name, selection, n_randoms, threshold, ladder, weighted,
# options, moved).
SURVEY_CASES = [
    ("sel", True, 600000, -0.8, (30.0, 24.0, 19.0, 15.0), False, 0, False),
    ("flat", False, 600000, -0.8, (30.0, 24.0, 19.0, 15.0), False, 0, False),
    ("sparse", True, 180000, -0.8, (30.0, 24.0, 19.0, 15.0), False, 0, False),
    ("shallow", True, 600000, -0.5, "10,30", False, 0, False),
    ("weighted", True, 600000, -0.5, "10,30", True, 0, False),
    ("lagrangian", True, 600000, -0.5, "10,30", False, abi.SIF_FINDER_LAGRANGIAN_OVERLAP, False),
    ("many", True, 600000, -0.3, "8,24", False, 0, False),
    ("offset", True, 600000, -0.5, "10,30", False, 0, True),
]
SURVEY_SEED, SURVEY_DATA, SURVEY_GRID, SURVEY_MESH = 7, 60000, 64, 20
SURVEY_MOVE = (-530.25, 311.5, 1207.0)


def survey_inputs(case):
    """The case's (data, randoms, data weights, random weights, radii) as the
    generator and the tests both make them: positions in the survey's own
    frame (moved away from the box for the "offset" case), weights None
    where the case has none."""
    name, sel, n_r, thr, lad, weighted, opt, moved = case
    data, rand = synth.survey(SURVEY_DATA, n_r, SURVEY_SEED, selection=sel)
    radii = (np.array(lad, np.float32) if not isinstance(lad, str) else
             synth.ladder(*[float(v) for v in lad.split(",")], 0.1).astype(np.float32))
    wd = wr = None
    if weighted:
        rng = np.random.default_rng(SURVEY_SEED + 1)
        wd = rng.uniform(0.5, 1.5, len(data[0])).astype(np.float32)
        wd[rng.random(len(wd)) < 0.2] = 0.0
        wr = np.full(len(rand[0]), 2.0, np.float32)
    if moved:
        data = tuple(np.float32(a + np.float32(m)) for a, m in zip(data, SURVEY_MOVE))
        rand = tuple(np.float32(a + np.float32(m)) for a, m in zip(rand, SURVEY_MOVE))
    return data, rand, wd, wr, radii


def survey_sha256(data, rand, wd, wr):
    import hashlib

    h = hashlib.sha256()
    for a in tuple(data) + tuple(rand) + ((wd,) if wd is not None else ()) + \
            ((wr,) if wr is not None else ()):
        h.update(np.ascontiguousarray(a, np.float32).tobytes())
    return h.hexdigest()


