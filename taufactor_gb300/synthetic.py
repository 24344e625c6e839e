"""Seeded synthetic microstructures for tests and benchmarks.

The reference benchmarks its solvers on generated structures (taufactor/utils.py:101-221,
taufactor/benchmark.py:28-34). The throughput workloads here are blurred Gaussian noise
thresholded at a porosity quantile: ``gaussian_filter(rng.standard_normal(shape), sigma) <
quantile(., porosity)`` with numpy's default_rng seeds fixed per volume.
"""
from __future__ import annotations

import concurrent.futures as cf

import numpy as np
from scipy.ndimage import gaussian_filter


def blurred_noise(shape, sigma: float, porosity: float, seed: int) -> np.ndarray:
    """uint8 volume, 1 = conductive, with the given conductive fraction."""
    f = gaussian_filter(np.random.default_rng(seed).standard_normal(shape, dtype=np.float32), sigma)
    thr = np.quantile(f, porosity)
    return (f < thr).astype(np.uint8)


def batch_256(n: int = 16, side: int = 256, sigma: float = 2.0, workers: int = 8, first: int = 0) -> np.ndarray:
    """Volumes first..first+n-1 of one sequence, each side^3: volume i from default_rng(1000+i),
    porosity_i ~ U[0.35,0.70] (the i-th draw of default_rng(999)). A rank of a multi-GPU run takes
    its own slice (first = rank * n)."""
    por = np.random.default_rng(999).uniform(0.35, 0.70, first + n)
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        vols = list(ex.map(lambda i: blurred_noise((side,) * 3, sigma, por[i], 1000 + i), range(first, first + n)))
    return np.stack(vols)


def _uneven_draws(n: int, sides):
    rng = np.random.default_rng(2000)
    shapes = [tuple(int(s) for s in rng.choice(sides, 3)) for _ in range(n)]
    por = rng.uniform(0.35, 0.70, n)
    return shapes, por


def uneven_volumes(n: int = 64, sides=(64, 96, 128, 192, 256), sigma: float = 2.0, workers: int = 8):
    """n volumes with independently drawn sides (default_rng(2000)); volume i from default_rng(2001+i)."""
    shapes, por = _uneven_draws(n, sides)
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        vols = list(ex.map(lambda i: blurred_noise(shapes[i], sigma, por[i], 2001 + i), range(n)))
    return vols


def uneven_volume(i: int, n: int = 64, sides=(64, 96, 128, 192, 256), sigma: float = 2.0) -> np.ndarray:
    """Volume i of ``uneven_volumes(n, sides, sigma)`` alone (same draws, same seed)."""
    shapes, por = _uneven_draws(n, sides)
    return blurred_noise(shapes[i], sigma, por[i], 2001 + i)


def three_phase(side: int = 320, sigma: float = 3.0) -> np.ndarray:
    """Labels 0,1,2 = argmax of three blurred noise fields (default_rng(3000..3002))."""
    fields = [gaussian_filter(np.random.default_rng(3000 + k).standard_normal((side,) * 3, dtype=np.float32), sigma)
              for k in range(3)]
    return np.argmax(np.stack(fields), axis=0).astype(np.uint8)
