"""The C ABI: the library builds, loads, and exports every entry point
include/sif_gb300.h declares; the host-side logic that needs no GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from sif_gb300 import _lib, build

    build.build()
    return _lib.load()


def _declared():
    """The header's functions the library must export (static inline ones,
    which a caller compiles from the header, excepted)."""
    text = open(os.path.join(ROOT, "include", "sif_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    inline = set(re.findall(r"static inline [^(]*?\b((?:sif|sifg)_[a-z0-9_]+)\s*\(", text))
    return sorted(set(re.findall(r"\b((?:sif|sifg)_[a-z0-9_]+)\s*\(", text)) - inline)


def test_suggest_mesh_cells_is_the_reference_rule():
    """sif_finder_suggest_mesh_cells (exodus_finder.h:653-683), compiled from
    the header, against the rule restated here: 30 tracers per cell,
    a floor from the widest stencil, clamped to [8, 1024]."""
    import subprocess
    import tempfile

    src = ('#include "sif_gb300.h"\n#include <stdio.h>\nint main(void) {\n'
           '  printf("%u %u %u %u %u %u\\n", sif_finder_suggest_mesh_cells(134217728ull, 1000.f, 24.f, 0.f),\n'
           '         sif_finder_suggest_mesh_cells(2097152ull, 500.f, 30.f, 0.f),\n'
           '         sif_finder_suggest_mesh_cells(1000ull, 100.f, 45.f, 0.f),\n'
           '         sif_finder_suggest_mesh_cells(64ull * 64 * 64, 200.f, 8.f, 8e6f),\n'
           '         sif_finder_suggest_mesh_cells(0ull, 100.f, 5.f, 0.f),\n'
           '         sif_finder_suggest_mesh_cells(1ull << 40, 1000.f, 5.f, 0.f));\n  return 0;\n}\n')
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-O2", "-I", os.path.join(ROOT, "include"), c, "-o", exe, "-lm"],
                       check=True)
        got = [int(v) for v in subprocess.run([exe], capture_output=True, text=True).stdout.split()]

    def rule(n, L, rmax, vol):
        whole = n * L ** 3 / vol if vol > 0 else n
        cells = (whole / 30.0) ** (1 / 3)
        if rmax > 0:
            if 2 * rmax >= L:
                return 0
            cells = max(cells, L / (L - 2 * rmax) + 1)
        return int(min(max(cells, 8.0), 1024.0)) if n else 0

    want = [rule(134217728, 1000, 24, 0), rule(2097152, 500, 30, 0), rule(1000, 100, 45, 0),
            rule(64 ** 3, 200, 8, 8e6), 0, rule(1 << 40, 1000, 5, 0)]
    assert got == want, (got, want)


def test_header_declares_the_reference_entry_points():
    names = _declared()
    for n in ["sif_grid_assign_cic", "sif_grid_to_density_contrast", "sif_chain_mesh_alloc",
              "sif_chain_mesh_alloc_consume", "sif_finder_exodus", "sif_finder_exodus_raw",
              "sif_system_init", "sif_error_message"]:
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    from sif_gb300 import _lib

    for name in _declared():
        assert hasattr(lib, name), name
    assert set(_declared()) == set(_lib.EXPORTED)


_PROBE_HEADERS = {
    "reference": ["sif/structures/field.h", "sif/structures/grid.h", "sif/structures/chain_mesh.h",
                  "sif/structures/catalogue.h", "sif/finder/exodus_finder.h", "sif/core/system.h"],
    "gb300": ["sif_gb300.h"],
}


def _layout_probe(include_dir, headers, structs, defines=()):
    """Compiles a C program against `headers` that prints sizeof of each
    struct and offsetof of each of its fields (the ctypes field names), and
    returns {struct: [size, offset, ...]}."""
    import subprocess
    import tempfile

    lines = ["#include <stddef.h>", "#include <stdio.h>"]
    lines += [f'#include "{h}"' for h in headers]
    lines.append("int main(void) {")
    for name, cls in structs.items():
        args = [f"sizeof({name})"] + [f"offsetof({name}, {f})" for f, _ in cls._fields_]
        lines.append(f'  printf("{name}' + " %zu" * len(args) + '\\n", ' + ", ".join(args) + ");")
    lines.append("  return 0;\n}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        open(c, "w").write("\n".join(lines) + "\n")
        exe = os.path.join(d, "probe")
        subprocess.run(["gcc", "-std=gnu99", "-I", include_dir, *[f"-D{x}" for x in defines], c,
                        "-o", exe, "-lm"], check=True, capture_output=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    return {ln.split()[0]: [int(v) for v in ln.split()[1:]] for ln in out.strip().splitlines()}


def _ctypes_layout(structs):
    return {name: [C.sizeof(cls)] + [getattr(cls, f).offset for f, _ in cls._fields_]
            for name, cls in structs.items()}


def _structs(real):
    from sif_gb300 import abi

    field, grid, mesh, cat, extras = (
        (abi.sif_field_t, abi.sif_grid_t, abi.sif_chain_mesh_t, abi.sif_catalogue_t,
         abi.sif_finder_exodus_extras_t) if real == "float" else abi.STRUCTS_F64)
    return {"sif_field_t": field, "sif_grid_t": grid, "sif_chain_mesh_t": mesh,
            "sif_catalogue_t": cat, "sif_finder_exodus_extras_t": extras,
            "sif_config_t": abi.sif_config_t}


def test_header_struct_layouts_match_the_ctypes_mirror():
    """include/sif_gb300.h compiled: every struct's size and every field's
    offset equal the ctypes structs pysif's mirror and the tests use."""
    structs = _structs("float")
    got = _layout_probe(os.path.join(ROOT, "include"), _PROBE_HEADERS["gb300"], structs)
    assert got == _ctypes_layout(structs)


@pytest.mark.parametrize("real", ["float", "double"])
def test_struct_layouts_match_the_reference_headers(real):
    """The reference's own headers compiled (its float build, and its
    SIF_USE_DOUBLE build whose layouts the _f64 entry points' callers use):
    sizeof and offsetof of every field of the boundary's structs equal the
    ctypes mirror, and, for the float build, this library's header."""
    from conftest import reference_dir

    ref = reference_dir()
    if ref is None:
        pytest.skip("no reference checkout (SIF_REFERENCE_DIR)")
    structs = _structs(real)
    want = _layout_probe(os.path.join(ref, "include"), _PROBE_HEADERS["reference"], structs,
                         ("SIF_USE_DOUBLE",) if real == "double" else ())
    assert _ctypes_layout(structs) == want
    if real == "float":
        assert _layout_probe(os.path.join(ROOT, "include"), _PROBE_HEADERS["gb300"], structs) == want


def _host_ranks_vs_oracle(lib, oracle, d):
    m = len(d)
    rank = np.empty(m, np.uint32)
    if m:
        lib.sifg_candidate_ranks(d.ctypes.data, m, rank.ctypes.data)
    rec = np.zeros(m, oracle.CANDIDATE_DTYPE)
    rec["delta"] = d
    rec["flat"] = np.arange(m)
    s = oracle.sort_candidates(rec)
    want = np.empty(m, np.int64)
    want[s["flat"].astype(np.int64)] = np.arange(m)
    assert np.array_equal(rank.astype(np.int64), want), m


def test_host_rank_replay_matches_oracle_sort(lib, oracle):
    rng = np.random.default_rng(9)
    for m in [0, 1, 7, 4095, 4096, 4097, 32769, 70000, 200000]:
        d = (rng.integers(0, 64, m) * np.float32(-0.002) - np.float32(0.8)).astype(np.float32)
        _host_ranks_vs_oracle(lib, oracle, d)


def test_host_rank_replay_shapes(lib, oracle):
    """Continuous keys with scattered ties, already ordered and reversed
    inputs, one key throughout, and a million keys over a few hundred values."""
    rng = np.random.default_rng(10)
    d = rng.uniform(-1.0, -0.8, 150000).astype(np.float32)
    d[rng.integers(0, len(d), 20000)] = d[rng.integers(0, len(d), 20000)]
    for case in [d, np.sort(d), np.sort(d)[::-1].copy(), np.full(50000, -0.9, np.float32),
                 (rng.integers(0, 300, 1000000) * np.float32(-0.0005)).astype(np.float32)]:
        _host_ranks_vs_oracle(lib, oracle, np.ascontiguousarray(case))


def test_host_rank_replay_with_ties_on_the_pivot(lib, oracle):
    """Segments large enough to be partitioned on every thread, with keys
    equal to the first pivot (the middle element) scattered through them:
    the queue of equal keys, rotated by the smaller keys examined between
    them, must come out as the sequential partition leaves it."""
    rng = np.random.default_rng(12)
    for m, copies in [(100000, 2), (100000, 50), (120001, 2000), (70000, 300)]:
        d = rng.uniform(-1.0, -0.8, m).astype(np.float32)
        piv = d[(m - 1) // 2]
        d[rng.choice(m, copies, replace=False)] = piv
        d[rng.integers(0, m, 3000)] = d[rng.integers(0, m, 3000)]  # ties elsewhere too
        _host_ranks_vs_oracle(lib, oracle, d)
        # The pivot's twins bunched at either end.
        e = d.copy()
        e[:copies // 2] = piv
        e[-(copies - copies // 2):] = piv
        _host_ranks_vs_oracle(lib, oracle, e)


def test_variants_and_argument_errors_without_a_gpu(lib):
    from sif_gb300 import abi

    ov = C.c_float(-1)
    opt = C.c_uint32(0)
    assert lib.sif_finder_exodus_preset(1, C.byref(ov), C.byref(opt)) == 0
    assert ov.value == 1.0 and opt.value == (abi.SIF_FINDER_SEEDS_MINIMA |
                                             abi.SIF_FINDER_EXTEND_REACH | abi.SIF_FINDER_DISPLACE)
    assert lib.sif_finder_exodus_preset(7, None, None) == abi.SIF_ERR_INVALID
    assert lib.sif_finder_exodus_variant_name(2) == b"lagrangian-overlap"
    v = C.c_int(-1)
    assert lib.sif_finder_exodus_variant_from_name(b"excursion-peak", C.byref(v)) == 0 and v.value == 1
    assert lib.sif_finder_grid_cells_from_size(0, 256.0, 1.0, 0, 0.0) == 256
    g = lib.sif_grid_alloc(0, 100.0)
    assert not g and lib.sif_error_status() == abi.SIF_ERR_INVALID


def test_init_without_a_gpu_fails_loudly(lib):
    """No silent CPU path: without a CUDA device the library refuses."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from sif_gb300 import abi

    cfg = abi.sif_config_t(None, None, abi.SIF_LOG_LEVEL_NONE, None, 0)
    assert lib.sif_system_init(C.byref(cfg)) == abi.SIF_ERR_UNSUPPORTED
    assert b"GPU" in lib.sif_error_message()


def _ref_checkpoint(tmp_path, halt=9):
    """A checkpoint the reference writes: the golden box's run stopped after
    `halt` rungs by its own test hook (sif__exodus_halt_after_set)."""
    import numpy as np

    import ref_ctypes as R
    from sif_gb300 import synth

    lib = R.load("strict", 4, abi_mod().SIF_LOG_LEVEL_NONE)
    x, y, z = synth.zeldovich(32, 128.0, 4.0, 11)
    f = R.RefField(lib, x, y, z)
    g = R.RefGrid(lib, 32, 128.0)
    g.assign_cic(f)
    g.to_contrast()
    m = R.RefMesh(lib, 8, 128.0, f)
    radii = synth.ladder(8.0, 24.0, 0.1).astype(np.float32)
    path = str(tmp_path / "ref.ckpt")
    extras = abi_mod().sif_finder_exodus_extras_t(path.encode(), None, 1, 0)
    lib.sif__exodus_halt_after_set.argtypes = [C.c_uint32]
    lib.sif__exodus_halt_after_set(halt)
    try:
        cat = lib.sif_finder_exodus_raw(g.ptr, m.ptr, radii.ctypes.data, len(radii), -0.7, 0.0, 0,
                                        C.byref(extras))
    finally:
        lib.sif__exodus_halt_after_set(0)
    assert not cat  # halted: the run fails, the checkpoint stays
    h = abi_mod().sif_finder_exodus_checkpoint_t()
    want = lib.sif_finder_exodus_checkpoint_read(path.encode(), C.byref(h))
    assert want
    cols = R.catalogue_arrays(lib, want)
    m.free()
    g.free()
    f.free()
    return path, h, cols


def abi_mod():
    from sif_gb300 import abi

    return abi


@pytest.mark.skipif("not __import__('ref_ctypes').available()")
def test_reads_the_reference_checkpoint(lib, tmp_path):
    """The XCKP v3 file (include/sif/finder/exodus_finder.h:409-507) the
    reference writes is read by this library as the reference reads it: the
    same header, the same voids; its CRC-32 is zlib's; a corrupted byte or a
    truncated file is refused."""
    import zlib

    import numpy as np

    from sif_gb300 import abi

    path, want_h, want = _ref_checkpoint(tmp_path)
    h = abi.sif_finder_exodus_checkpoint_t()
    got = lib.sif_finder_exodus_checkpoint_read(path.encode(), C.byref(h))
    assert got
    c = got.contents
    cols = [np.ctypeslib.as_array(p, shape=(c.n_voids,)).copy() for p in (c.cx, c.cy, c.cz, c.radii)]
    lib.sif_catalogue_free(got)
    assert bytes(h) == bytes(want_h)
    assert h.next_rung == 9 and h.n_voids == len(want[0]) > 0
    assert all(np.array_equal(a, b) for a, b in zip(cols, want))
    raw = bytearray(open(path, "rb").read())
    body = bytearray(raw)
    body[132:136] = b"\0\0\0\0"  # the header's crc32 field, zeroed
    assert zlib.crc32(bytes(body)) == h.crc32
    bad = tmp_path / "bad.ckpt"
    raw[-3] ^= 0x40
    bad.write_bytes(bytes(raw))
    assert not lib.sif_finder_exodus_checkpoint_read(str(bad).encode(), None)
    assert b"checksum" in lib.sif_error_message()
    bad.write_bytes(bytes(raw[:-4]))
    assert not lib.sif_finder_exodus_checkpoint_read(str(bad).encode(), None)
    assert b"bytes" in lib.sif_error_message()


def test_host_mirror_switch_without_a_gpu(lib):
    """The mirrors' switch and the copy counters answer without a device;
    declaring a write to an address the library never mirrored is harmless."""
    import ctypes as C

    lib.sifg_set_host_mirrors(1)
    assert lib.sifg_host_mirrors() == 1
    buf = (C.c_float * 16)()
    lib.sifg_host_modified(C.cast(buf, C.c_void_p))
    lib.sifg_host_modified(None)
    lib.sifg_set_host_mirrors(0)
    assert lib.sifg_host_mirrors() == 0
    h2d, d2h = C.c_uint64(1), C.c_uint64(1)
    lib.sifg_copy_bytes(C.byref(h2d), C.byref(d2h))
    assert h2d.value == 0 and d2h.value == 0
