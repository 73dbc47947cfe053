"""mdmc_count_cells_noalloc, the allocation-free count pass, through the C ABI.

Its totals must equal the counts mdmc_run reports for the same grid and
iso-value (integers: exactly), on consecutive calls that share the entry
point's fixed scratch, and grids beyond that scratch must be rejected before
any work.  Collected last on purpose: it must pass alone in a fresh process
(where its first call sets up the scratch) and after every other test.
"""
import ctypes

import numpy as np
import pytest

import manifolddmc_gb300 as mdmc

pytestmark = pytest.mark.gpu

MDMC_OK = 0
MDMC_ERROR_LIMIT = 4


def _entry():
    lib = mdmc.library()
    f = lib.mdmc_count_cells_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
    return f


def _count(grid, iso, totals):
    msg = ctypes.create_string_buffer(256)
    st = _entry()(ctypes.addressof(grid.grid), iso, totals.data_ptr(), None, msg, len(msg))
    return st, msg.value.decode()


def _blobs(n, count, seed):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    v = np.zeros((n, n, n), np.float64)
    for _ in range(count):
        c = rng.uniform(0, n - 1, 3)
        s = rng.uniform(2.0, 6.0)
        v += np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) / (2 * s * s))
    return v.astype(np.float32)


CASES = [
    # name, volume, iso, refinement, pad
    ("noise40", lambda: np.random.default_rng(41).random((40, 40, 40), dtype=np.float32), 0.5, 0, False),
    ("blobs33_refine3", lambda: _blobs(33, 8, 42), 0.4, 3, False),
    ("noise24_pad", lambda: np.random.default_rng(43).random((24, 31, 17), dtype=np.float32), 0.5, 0, True),
    ("blobs21_refine1_pad", lambda: _blobs(21, 5, 44), 0.45, 1, True),
]


def test_noalloc_count_matches_run_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    grids = []
    for name, factory, iso, r, pad in CASES:
        vol = factory()
        dims = [vol.shape[2], vol.shape[1], vol.shape[0]]
        grid = mdmc.UniformGrid(vol, dims, (0.5, -1.0, 2.0), (0.25, 0.5, 1.0), r, pad)
        dmc = mdmc.DualMarchingCubes()
        dmc.run(iso, grid)
        expect = (int(dmc.stats.num_active_cells), int(dmc.stats.num_dmc_quads))
        assert expect[0] > 0 and expect[1] > 0, name
        grids.append((name, grid, iso, expect))
    torch.cuda.synchronize()
    totals = torch.full((2,), -7, dtype=torch.int64, device="cuda")
    # two calls in a row on every grid, then the first grid again after the
    # others have left their contents in the shared scratch
    order = [g for g in grids for _ in range(2)] + [grids[0]]
    for name, grid, iso, expect in order:
        st, msg = _count(grid, iso, totals)
        assert st == MDMC_OK, (name, msg)
        torch.cuda.synchronize()
        assert tuple(int(t) for t in totals.cpu()) == expect, name
        totals.fill_(-7)


def _smooth_field(dims, torch):
    """A smooth field on the device with many iso-crossings (dims x, y, z)."""
    X, Y, Z = dims
    z = torch.arange(Z, device="cuda", dtype=torch.float32).view(Z, 1, 1)
    y = torch.arange(Y, device="cuda", dtype=torch.float32).view(1, Y, 1)
    x = torch.arange(X, device="cuda", dtype=torch.float32).view(1, 1, X)
    return (torch.sin(0.21 * x + 0.3) * torch.cos(0.17 * y) + torch.sin(0.13 * z + 0.05 * x)).contiguous()


def test_noalloc_count_at_exactly_its_limits():
    """Grids at exactly the scratch's limits are accepted and count like mdmc_run.

    The refined limit case ends its last row of coarse cells on the last word
    of the bit mask, where the row walker also loads the word after it."""
    torch = pytest.importorskip("torch")
    totals = torch.full((2,), -7, dtype=torch.int64, device="cuda")
    cases = [
        # (512 * 512) = 2^18 x-rows of cells, dense
        ("rows_2^18", [3, 513, 513], 0, False),
        # 256^3 = 2^24 coarse cells, padded on demand (259^3 samples)
        ("coarse_2^24_pad", [257, 257, 257], 0, True),
        # 2^24 coarse cells refined x2 (coarse 257^3, 513^3 samples)
        ("coarse_2^24_refine1", [257, 257, 257], 1, False),
    ]
    for name, cdims, r, pad in cases:
        field = _smooth_field(cdims, torch)
        grid = mdmc.UniformGrid(field, cdims, refinement=r, add_zero_boundary=pad)
        dmc = mdmc.DualMarchingCubes(split_non_manifold_halfedges=False, detect_non_manifold_vertices=False)
        dmc.run(0.1, grid)
        expect = (int(dmc.stats.num_active_cells), int(dmc.stats.num_dmc_quads))
        assert expect[0] > 0 and expect[1] > 0, name
        del dmc
        for _ in range(2):
            st, msg = _count(grid, 0.1, totals)
            assert st == MDMC_OK, (name, msg)
            torch.cuda.synchronize()
            assert tuple(int(t) for t in totals.cpu()) == expect, name
            totals.fill_(-7)


def test_noalloc_count_rejects_grids_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    totals = torch.full((2,), -7, dtype=torch.int64, device="cuda")
    # (1026-1) * (258-1) x-rows of cells > 2^18 (samples really allocated)
    dense = torch.rand(258, 1026, 2, device="cuda")
    grid = mdmc.UniformGrid(dense, [2, 1026, 258])
    st, msg = _count(grid, 0.5, totals)
    assert st == MDMC_ERROR_LIMIT and "x-rows" in msg
    # padded grid over 257^3 > 2^24 coarse cells
    coarse = torch.rand(258, 258, 258, device="cuda")
    grid = mdmc.UniformGrid(coarse, [258, 258, 258], refinement=0, add_zero_boundary=True)
    st, msg = _count(grid, 0.5, totals)
    assert st == MDMC_ERROR_LIMIT and "coarse cells" in msg
    torch.cuda.synchronize()
    assert totals.cpu().tolist() == [-7, -7]
