import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

GOLDEN = os.path.join(ROOT, "tests", "golden")


def reference_dir():
    """The reference's source checkout, where one is present: the directory
    SIF_REFERENCE_DIR names, else a checkout named `reference` beside this
    repository; None where there is neither (the GPU machines)."""
    for cand in (os.environ.get("SIF_REFERENCE_DIR"), os.path.join(ROOT, "..", "reference")):
        if cand and os.path.isfile(os.path.join(cand, "include", "sif", "finder", "exodus_finder.h")):
            return os.path.abspath(cand)
    return None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: a full-size workload")


@pytest.fixture(scope="session")
def oracle():
    import oracle_ctypes as O

    O.build()
    return O


@pytest.fixture(scope="session")
def golden_box32():
    return dict(np.load(os.path.join(GOLDEN, "golden_box32.npz")))


@pytest.fixture(scope="session")
def golden_box32_f64():
    """The same box through the reference's SIF_USE_DOUBLE build."""
    return dict(np.load(os.path.join(GOLDEN, "golden_box32_f64.npz")))


@pytest.fixture(scope="session")
def golden_box32_extend():
    """The same positions at threshold -0.3 and ladder(4, 8): catalogues with
    and without SIF_FINDER_EXTEND_REACH."""
    return dict(np.load(os.path.join(GOLDEN, "golden_box32_extend.npz")))


@pytest.fixture(scope="session")
def golden_box32_extend_f64():
    """The extended-reach box through the reference's SIF_USE_DOUBLE build."""
    return dict(np.load(os.path.join(GOLDEN, "golden_box32_extend_f64.npz")))


@pytest.fixture(scope="session")
def golden_box32_displace():
    """The same positions at threshold -0.3 and ladder(3, 6): catalogues under
    SIF_FINDER_DISPLACE (the excursion-peak preset among them)."""
    return dict(np.load(os.path.join(GOLDEN, "golden_box32_displace.npz")))


@pytest.fixture(scope="session")
def golden_box32_weighted():
    """Weighted meshes through the reference: the "rand" and "holes" sets
    (positions, weights, weighted contrast, mesh with its weight columns,
    captured fields, catalogues)."""
    return dict(np.load(os.path.join(GOLDEN, "golden_box32_weighted.npz")))


@pytest.fixture(scope="session")
def golden_box32_weighted_f64():
    """The "rand" weighted set through the reference's SIF_USE_DOUBLE build."""
    return dict(np.load(os.path.join(GOLDEN, "golden_box32_weighted_f64.npz")))


@pytest.fixture(scope="session")
def golden_survey():
    return np.load(os.path.join(GOLDEN, "golden_survey.npz"))


@pytest.fixture(scope="session")
def golden_box32_refine():
    """SIF_FINDER_REFINE_GAUSSIAN through the reference: the rungs' top-hat
    and refinement fields, and per option set the rungs refined and the
    catalogue."""
    return dict(np.load(os.path.join(GOLDEN, "golden_box32_refine.npz")))


@pytest.fixture(scope="session")
def golden_box32_refine_f64():
    """The refinement through the reference's SIF_USE_DOUBLE build."""
    return dict(np.load(os.path.join(GOLDEN, "golden_box32_refine_f64.npz")))


def refine_fields(g, name):
    """The fields a refined run's transforms returned, in order: per rung the
    top-hat and, where the rung ran it, the refinement's own."""
    where = {int(r): k for k, r in enumerate(g["gauss_rungs"])}
    seq = []
    for i, th in enumerate(g["tophat"]):
        seq.append(th)
        if g[f"{name}_refined_rungs"][i]:
            seq.append(g["gauss"][where[i]])
    return np.stack(seq)


@pytest.fixture(scope="session")
def golden_box32_displace_f64():
    """The displacement box through the reference's SIF_USE_DOUBLE build."""
    return dict(np.load(os.path.join(GOLDEN, "golden_box32_displace_f64.npz")))


@pytest.fixture(scope="session")
def gpu_lib():
    """The built GB300 library, initialised on the GPU."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sif_gb300 import build, pysif

    build.build()
    pysif.system_init(log_level="error")
    return pysif


def same_bits(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def same_catalogue(c1, c2):
    return all(same_bits(a, b) for a, b in zip(c1, c2))


def same_bits64(a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def same_catalogue64(c1, c2):
    return all(same_bits64(a, b) for a, b in zip(c1, c2))
