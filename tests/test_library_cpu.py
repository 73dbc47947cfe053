"""Checks that need no GPU: the C-ABI library builds, loads and exports every
entry point declared in include/mdmc.h, and the Marching Cubes case tables
built into it (and into the oracle) equal the reference's tables."""
import ctypes
import hashlib
import json
import re

import numpy as np
import pytest

from _support import GOLDEN_DIR, ROOT, oracle

import manifolddmc_gb300 as mdmc


def _declared_functions():
    text = (ROOT / "include" / "mdmc.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mdmc_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(mdmc.build()))
    names = _declared_functions()
    assert len(names) >= 14
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def _digest():
    return json.loads((GOLDEN_DIR / "mc_tables_digest.json").read_text())


def test_library_case_tables_match_reference():
    words, amb = mdmc.case_tables()
    d = _digest()
    assert hashlib.sha256(words.astype("<u8").tobytes()).hexdigest() == d["contour_words_sha256"]
    assert hashlib.sha256(amb.astype(np.uint8).tobytes()).hexdigest() == d["ambiguous_sha256"]
    assert int(amb.sum()) == d["num_ambiguous"] == 128


def test_oracle_case_tables_match_reference():
    text = (ROOT / "oracle" / "mc_contour_table_oracle.h").read_text()
    words = [int(w, 16) for w in re.findall(r"0x([0-9a-f]{16})ULL", text)]
    assert len(words) == 256
    d = _digest()
    assert hashlib.sha256(b"".join(w.to_bytes(8, "little") for w in words)).hexdigest() == d["contour_words_sha256"]
    lib = oracle()
    lib.mdmc_oracle_case_ambiguous.argtypes = [ctypes.c_int]
    amb = bytes(lib.mdmc_oracle_case_ambiguous(c) for c in range(256))
    assert hashlib.sha256(amb).hexdigest() == d["ambiguous_sha256"]


def test_default_options_mirror_reference_defaults():
    # DualMarchingCubes.cu:110-133, ManifoldSplitter.cu:84
    o = mdmc.Options()
    mdmc.library().mdmc_default_options(ctypes.byref(o))
    assert (o.enable_surface_to_vertex_iteration, o.simplify_p3x3y_color, o.simplify_p3x3y_old, o.simplify_p3333,
            o.split_non_manifold_halfedges, o.detect_non_manifold_vertices, o.splitting_step) == (1, 0, 0, 0, 1, 1, 100)


def test_read_bin_matches_oracle_reader(tmp_path):
    from _support import golden_grid, reference_goldens
    import struct
    g = reference_goldens()["1-Edge"]
    path = tmp_path / "g.bin"
    path.write_bytes(struct.pack("3i", *g["dims"]) + struct.pack("3f", *g["spacing"]) +
                     struct.pack("%dH" % len(g["samples"]), *g["samples"]))
    samples, dims, sp, org = mdmc.read_bin(path)
    s2, d2, o2, sp2, _ = golden_grid("1-Edge")
    assert dims == d2
    assert np.array_equal(samples.reshape(-1), s2)
    assert np.array_equal(org, o2) and np.array_equal(sp, sp2)


def test_create_without_device_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(mdmc.MDMCError):
        mdmc.DualMarchingCubes()
