"""A seeded sweep of grid shapes, value fields, iso-values, refinement,
padding and flags through the C ABI against the oracle, every output array
bit-exact (the same comparison as tests/test_gpu_parity.py).  The cases mix
thin grids (2 samples along an axis), uneven dims, values with ties at the
iso-value, negative and large-magnitude fields, and every flag combination
the reference exposes, so that index arithmetic, boundary handling and the
repair paths meet inputs the hand-written cases do not."""
import zlib

import numpy as np
import pytest

from test_gpu_parity import assert_parity, gpu_run, oracle_for

pytestmark = pytest.mark.gpu


def _field(rng, kind, dims):
    X, Y, Z = dims
    z, y, x = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    if kind == "noise":
        return rng.random((Z, Y, X), dtype=np.float32)
    if kind == "quantised":  # many samples exactly at the iso-value
        return (rng.integers(0, 5, (Z, Y, X)) * 0.25).astype(np.float32)
    if kind == "blobs":
        v = np.zeros((Z, Y, X))
        for _ in range(rng.integers(1, 5)):
            c = rng.uniform(0, [X - 1, Y - 1, Z - 1])
            s = rng.uniform(1.0, 4.0)
            v += np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
        return v.astype(np.float32)
    if kind == "sdf":  # signed distance, negative inside, scaled up
        c = np.array([X - 1, Y - 1, Z - 1]) / 2.0
        r = 0.35 * min(X, Y, Z) + 0.3
        return (1000.0 * (np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) - r)).astype(np.float32)
    raise ValueError(kind)


def _cases(n=160, seed=20261203):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        kind = ["noise", "quantised", "blobs", "sdf"][i % 4]
        dims = [int(rng.integers(2, 19 if i < 120 else 31)) for _ in range(3)]
        if i % 9 == 0:
            dims[int(rng.integers(0, 3))] = 2
        refinement = int(rng.choice([0, 0, 1, 2, 3]))
        pad = bool(rng.integers(0, 2))
        opts = {"surface_iteration": int(rng.integers(0, 2)), "split_non_manifold": int(rng.integers(0, 2)),
                "detect_non_manifold_vertices": int(rng.integers(0, 2))}
        if i % 6 == 5:
            opts.update(simplify_3x3y_color=int(rng.integers(0, 2)), simplify_3x3y_old=int(rng.integers(0, 2)),
                        simplify_3333=int(rng.integers(0, 2)))
        if i % 7 == 3:
            opts["splitting_step"] = int(rng.choice([0, 1, 2, 3, 4, 5, 6, 100]))
        iso = {"noise": 0.5, "quantised": 0.5, "blobs": float(rng.uniform(0.2, 0.7)), "sdf": 0.0}[kind]
        out.append(("%02d_%s_%dx%dx%d_r%d%s" % (i, kind, dims[0], dims[1], dims[2], refinement, "_pad" if pad else ""),
                    kind, dims, int(rng.integers(0, 2**31)), iso, refinement, pad, opts))
    return out


CASES = _cases()


@pytest.mark.parametrize("name,kind,dims,seed,iso,refinement,pad,opts", CASES, ids=[c[0] for c in CASES])
def test_sweep_bit_exact(name, kind, dims, seed, iso, refinement, pad, opts):
    vol = _field(np.random.default_rng(seed), kind, dims)
    origin = np.array([0.25, -3.0, 1.5], np.float32)
    spacing = np.array([0.5, 1.25, 0.75], np.float32)
    dmc, m, _ = gpu_run(vol.reshape(-1), dims, origin, spacing, iso, refinement, pad, **opts)
    ref, _ = oracle_for(vol.reshape(-1), dims, origin, spacing, iso, refinement, pad, **opts)
    assert_parity(dmc, m, ref)


# Larger noise grids: several splitter iterations, the local edge-bucket
# refresh of the later ones, the decider table on many ambiguous cells, and
# detection after the splitter with and without the vertex pass's fan degrees
# (a simplification before the splitter renumbers vertices and turns them off).
NOISE_CASES = [
    ("noise48_iso045", 48, 0.45, {}),
    ("noise56_iso055_nodetect", 56, 0.55, {"detect_non_manifold_vertices": 0}),
    ("noise64_iso05", 64, 0.5, {}),
    ("noise64_iso03_nosurf", 64, 0.3, {"surface_iteration": 0}),
    ("noise40_iso05_simplify", 40, 0.5, {"simplify_3333": 1}),
    ("noise44_iso06_steps", 44, 0.6, {"splitting_step": 5}),
]


@pytest.mark.parametrize("name,n,iso,opts", NOISE_CASES, ids=[c[0] for c in NOISE_CASES])
def test_noise_repair_bit_exact(name, n, iso, opts):
    vol = np.random.default_rng(zlib.crc32(name.encode())).random((n, n + 3, n - 2), dtype=np.float32)
    dims = [n - 2, n + 3, n]
    origin = np.zeros(3, np.float32)
    spacing = np.ones(3, np.float32)
    dmc, m, _ = gpu_run(vol.reshape(-1), dims, origin, spacing, iso, **opts)
    ref, _ = oracle_for(vol.reshape(-1), dims, origin, spacing, iso, **opts)
    assert_parity(dmc, m, ref)
