"""Seeded synthetic grids for the benchmark configurations.

No public dataset is involved: every grid is generated from a numpy
default_rng seed with the shapes and value distributions of the benchmark
configurations (sums of isotropic Gaussian blobs, or iid uniform noise).
"""
import numpy as np


def gaussian_blobs(n, count, sigma_range, seed, amplitude=1.0):
    """Sum of `count` isotropic Gaussians on an n^3 grid (x fastest in memory),
    centres uniform in [0, n-1]^3, sigma uniform in sigma_range (cells)."""
    rng = np.random.default_rng(seed)
    ax = np.arange(n, dtype=np.float64)
    out = np.zeros((n, n, n), np.float64)
    for _ in range(count):
        c = rng.uniform(0.0, n - 1.0, 3)
        s = rng.uniform(sigma_range[0], sigma_range[1])
        g = [np.exp(-((ax - c[k]) ** 2) / (2.0 * s * s)) for k in range(3)]
        out += amplitude * (g[2][:, None, None] * g[1][None, :, None] * g[0][None, None, :])
    return out.astype(np.float32)


def gaussian_blobs_xyz(dims, count, sigma_range, seed, amplitude=1.0):
    """Sum of `count` isotropic Gaussians on a grid of dims (X, Y, Z), array [Z, Y, X]."""
    rng = np.random.default_rng(seed)
    axes = [np.arange(d, dtype=np.float64) for d in dims]
    out = np.zeros((dims[2], dims[1], dims[0]), np.float64)
    for _ in range(count):
        c = [rng.uniform(0.0, d - 1.0) for d in dims]
        s = rng.uniform(sigma_range[0], sigma_range[1])
        g = [np.exp(-((axes[k] - c[k]) ** 2) / (2.0 * s * s)) for k in range(3)]
        out += amplitude * (g[2][:, None, None] * g[1][None, :, None] * g[0][None, None, :])
    return out.astype(np.float32)


def batch_grids(count=96, seed=4, dim_range=(24, 192)):
    """The batched workload: `count` grids with dims drawn per axis uniformly
    from dim_range, values 4-32 Gaussian blobs (sigma 2-8 cells) or iid
    uniform noise (50/50), iso-values uniform in [0.3, 0.7].  Returns a list
    of (array [Z, Y, X] float32, iso)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        dims = [int(x) for x in rng.integers(dim_range[0], dim_range[1] + 1, 3)]
        iso = float(np.float32(rng.uniform(0.3, 0.7)))
        sub = int(rng.integers(0, 2**31))
        if rng.random() < 0.5:
            vol = gaussian_blobs_xyz(dims, int(rng.integers(4, 33)), (2.0, 8.0), sub)
        else:
            vol = np.random.default_rng(sub).random((dims[2], dims[1], dims[0]), dtype=np.float32)
        out.append((vol, iso))
    return out


def uniform_noise(n, seed):
    return np.random.default_rng(seed).random((n, n, n), dtype=np.float32)


def sphere_sdf(n, radius, seed=0):
    """Signed distance (cells) to a sphere of `radius` centred in an n^3 grid;
    `seed` is unused (the field is deterministic)."""
    ax = np.arange(n, dtype=np.float64) - (n - 1) / 2.0
    d = np.sqrt(ax[None, None, :] ** 2 + ax[None, :, None] ** 2 + ax[:, None, None] ** 2)
    return (d - radius).astype(np.float32)


def torus_points(count, major, minor, centre, seed):
    """`count` points uniform in area on a torus (radii in cells) around the z
    axis through `centre`, by rejection sampling of the tube angle."""
    rng = np.random.default_rng(seed)
    pts = []
    need = count
    while need > 0:
        u = rng.uniform(0, 2 * np.pi, 2 * need)
        v = rng.uniform(0, 2 * np.pi, 2 * need)
        keep = rng.uniform(0, 1, 2 * need) < (major + minor * np.cos(v)) / (major + minor)
        u, v = u[keep][:need], v[keep][:need]
        r = major + minor * np.cos(v)
        pts.append(np.stack([r * np.cos(u), r * np.sin(u), minor * np.sin(v)], 1))
        need -= len(u)
    return (np.concatenate(pts)[:count] + np.asarray(centre)).astype(np.float32)


# name: (description, generator, iso, refinement, pad)
CONFIGS = {
    "blobs64_pad": ("64^3 fp32 grid, 8 Gaussian blobs (sigma 4-10), padded by 1, iso 0.5",
                    lambda seed=0: gaussian_blobs(64, 8, (4.0, 10.0), seed), 0.5, 0, True),
    "noise128": ("128^3 fp32 iid uniform[0,1] noise, iso 0.5 (the noise workload at 1/8 size, for profiling)",
                 lambda seed=1: uniform_noise(128, seed), 0.5, 0, False),
    "noise256": ("256^3 fp32 iid uniform[0,1] noise, iso 0.5",
                 lambda seed=1: uniform_noise(256, seed), 0.5, 0, False),
    "blobs129_refine4": ("129^3 fp32 grid, 64 Gaussian blobs (sigma 3-12), trilinearly refined x4 "
                         "to 513^3 samples = 512^3 cells, iso 0.4",
                         lambda seed=2: gaussian_blobs(129, 64, (3.0, 12.0), seed), 0.4, 3, False),
    "blobs65_refine4": ("65^3 fp32 grid, 16 Gaussian blobs (sigma 3-12), trilinearly refined x4 to 257^3 samples = "
                        "256^3 cells, iso 0.4 (the refined workload at 1/8 size, for profiling)",
                        lambda seed=2: gaussian_blobs(65, 16, (3.0, 12.0), seed), 0.4, 3, False),
    "noise513": ("513^3 fp32 iid uniform[0,1] noise (512^3 cells), iso 0.5: the noise grid at the headline size",
                 lambda seed=5: uniform_noise(513, seed), 0.5, 0, False),
    "sphere128_sdf": ("128^3 fp32 signed distance to a sphere of radius 40 cells, iso 0, surface iteration off "
                      "(the differentiable form)",
                      lambda seed=0: sphere_sdf(128, 40.0, seed), 0.0, 0, False),
}
