"""Deterministic inputs of the golden cases.

The solver cases restate the known-answer tests of the reference
(tldr-group/taufactor v1.2.1, tests/test_taufactor.py; line numbers cited per case) plus the
100^3 Bernoulli(0.5) workload and a few small random volumes whose field after a fixed number of
half-sweeps is stored bit for bit. ``make_golden.py`` runs the reference on each input and writes
``reference_outputs.npz``; the tests rebuild the same inputs from here.
"""
from __future__ import annotations

import numpy as np


def _slanted(n=20):
    img = np.zeros((n, n + 1, n + 1))
    for i in range(n):
        img[i, i:i + 2, i:i + 2] = 1
    return img


def _blocks(shape):
    img = np.ones(shape)
    img[:, 0] = 0
    return img


def _non_percolating(n=20):
    img = np.zeros((n, n, n))
    img[:2] = 1
    return img


def _strip(n=20, t=10):
    img = np.zeros((n, n, n))
    img[:, 0:t, 0:t] = 1
    return img


def _deadend():
    img = np.zeros((10, 50, 50))
    img[:8, 25, 25] = 1
    return img


def _strip12():
    img = np.zeros((20, 20, 20))
    img[:, 0:10, 0:10] = 1
    img[:, 0:10, 10:20] = 2
    return img


def _strip123():
    img = np.ones((20, 20, 20))
    img[:, 0:10, 0:10] = 2
    img[:, 0:10, 10:20] = 3
    return img


def _label0_conductive():
    img = np.zeros((20, 20, 20))
    img[:, :2] = 1
    return img


def _batched_mp():
    a = np.ones((16, 16, 16))
    b = np.ones((16, 16, 16))
    b[:, :, :8] = 2
    return np.stack([a, b], axis=0)


def bernoulli_100():
    """100^3 iid Bernoulli(0.5) voxels from seed 0 (1 = conductive)."""
    return (np.random.default_rng(0).random((100, 100, 100)) < 0.5).astype(np.uint8)


def random_binary(shape, seed, p=0.6):
    return (np.random.default_rng(seed).random(shape) < p).astype(np.uint8)


def random_labels(shape, seed, n=3):
    return np.random.default_rng(seed).integers(0, n, shape).astype(np.uint8)


def _blur_labels(shape, seed):
    """Three labels from the argmax of three blurred noise fields (sigma 1.5)."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    f = np.stack([gaussian_filter(rng.standard_normal(shape), 1.5) for _ in range(3)])
    return np.argmax(f, axis=0).astype(np.uint8)


# name -> (kind, input builder, constructor kwargs, solve kwargs, reference test it restates)
SOLVE_CASES = {
    "blocks_cube": ("binary", lambda: _blocks((20, 20, 20)), {}, {}, "test_taufactor.py:12-19"),
    "blocks_long_x": ("binary", lambda: _blocks((40, 20, 20)), {}, {}, "test_taufactor.py:21-28"),
    "blocks_long_z": ("binary", lambda: _blocks((20, 20, 40)), {}, {}, "test_taufactor.py:30-37"),
    "nonperc": ("binary", _non_percolating, {}, {"iter_limit": 1000}, "test_taufactor.py:39-46"),
    "strip": ("binary", _strip, {}, {}, "test_taufactor.py:48-56"),
    "slanted": ("binary", _slanted, {}, {}, "test_taufactor.py:58-66"),
    "deadend": ("binary", _deadend, {}, {}, "test_taufactor.py:68-76"),
    "p_blocks": ("periodic", lambda: _blocks((20, 20, 20)), {}, {}, "test_taufactor.py:80-87"),
    "p_nonperc": ("periodic", _non_percolating, {}, {"iter_limit": 1000}, "test_taufactor.py:89-96"),
    "p_strip": ("periodic", _strip, {}, {}, "test_taufactor.py:98-106"),
    "p_slanted": ("periodic", _slanted, {}, {"iter_limit": 1000}, "test_taufactor.py:234-247"),
    "mp_nonperc": ("multiphase", _non_percolating, {}, {"iter_limit": 1000}, "test_taufactor.py:110-117"),
    "mp_ones": ("multiphase", lambda: np.ones((20, 20, 20)), {}, {"iter_limit": 1000},
                "test_taufactor.py:119-125"),
    "mp_halves": ("multiphase", lambda: np.ones((20, 20, 20)), {"diffusivities": {1: 0.5}},
                  {"iter_limit": 1000}, "test_taufactor.py:127-134"),
    "mp_strip": ("multiphase", _strip, {}, {}, "test_taufactor.py:136-144"),
    "mp_strip12": ("multiphase", _strip12, {"diffusivities": {0: 0, 1: 1, 2: 0.5}}, {},
                   "test_taufactor.py:146-156"),
    "mp_strip123": ("multiphase", _strip123, {"diffusivities": {0: 0, 1: 1, 2: 0.5, 3: 2}}, {},
                    "test_taufactor.py:158-168"),
    "mp_label0": ("multiphase", _label0_conductive, {"diffusivities": {0: 1.0, 1: 0.0}},
                  {"iter_limit": 1000}, "test_taufactor.py:180-187"),
    "mp_slanted": ("multiphase", _slanted, {}, {"iter_limit": 1000}, "test_taufactor.py:195-205"),
    "mp_batched": ("multiphase", _batched_mp, {"diffusivities": {0: 0.0, 1: 1.0, 2: 0.5}},
                   {"iter_limit": 1000}, "test_taufactor.py:207-224"),
    "pmp_ones": ("periodic_multiphase", lambda: np.ones((20, 20, 20)), {"diffusivities": {1: 1.0}},
                 {"iter_limit": 1000}, "test_taufactor.py:226-232"),
    "pmp_slanted": ("periodic_multiphase", _slanted, {"diffusivities": {0: 0.0, 1: 1.0}},
                    {"iter_limit": 1000}, "test_taufactor.py:234-247"),
    "aniso_slanted": ("anisotropic", _slanted, {"spacing": (1.0, 1.5, 0.8)}, {}, "taufactor.py:422-478"),
    "bernoulli100": ("binary", bernoulli_100, {}, {"conv_crit": 2e-2}, "100^3 Bernoulli(0.5), seed 0"),
    "bernoulli100_periodic": ("periodic", bernoulli_100, {}, {"conv_crit": 2e-2},
                              "100^3 Bernoulli(0.5), seed 0, periodic y/z"),
    # the reference has no test of its electrode solvers (taufactor/electrode.py:13-157); these
    # cases are its own outputs on seeded label volumes (1 = conductive, 0 = reactive, 2 = inert)
    "el_labels": ("electrode", lambda: random_labels((20, 12, 14), 5), {}, {"conv_crit": 1e-3},
                  "electrode.py:13-125"),
    "el_batch": ("electrode", lambda: random_labels((2, 11, 9, 13), 7), {}, {"conv_crit": 1e-3},
                 "electrode.py:13-125"),
    "el_blur": ("electrode", lambda: _blur_labels((24, 16, 16), 8), {}, {"conv_crit": 1e-3},
                "electrode.py:13-125"),
    "pel_batch": ("periodic_electrode", lambda: random_labels((2, 16, 10, 12), 6), {}, {"conv_crit": 1e-3},
                  "electrode.py:128-157"),
}

# name -> (kind, input builder, constructor kwargs, number of half-sweeps)
SWEEP_CASES = {
    "sw_binary": ("binary", lambda: random_binary((13, 10, 12), 11), {}, 57),
    "sw_binary_batch": ("binary", lambda: random_binary((3, 9, 8, 11), 12), {}, 40),
    "sw_periodic_even": ("periodic", lambda: random_binary((11, 10, 12), 13), {}, 57),
    "sw_periodic_odd": ("periodic", lambda: random_binary((10, 9, 11), 14), {}, 57),
    "sw_aniso": ("anisotropic", lambda: random_binary((12, 9, 10), 15), {"spacing": (1.0, 1.3, 0.7)}, 41),
    "sw_multiphase": ("multiphase", lambda: random_labels((12, 10, 9), 16),
                      {"diffusivities": {0: 0.0, 1: 1.0, 2: 0.1}}, 57),
    "sw_periodic_multiphase": ("periodic_multiphase", lambda: random_labels((10, 9, 11), 17),
                               {"diffusivities": {0: 0.3, 1: 1.0, 2: 0.1}}, 57),
    "sw_electrode": ("electrode", lambda: random_labels((2, 13, 10, 12), 18), {}, 57),
    "sw_periodic_electrode": ("periodic_electrode", lambda: random_labels((12, 10, 14), 19), {}, 57),
}


def _imp_deadend(n=100):
    img = np.zeros((n, n))
    img[:75, 45:55] = 1
    return img


def _imp_throughpore(n=100):
    img = np.zeros((n, n))
    img[:, 45:55] = 1
    return img


def _imp_blob(shape, seed, porosity=0.5, inert=0.0, sigma=1.5):
    """Label 1 (pore) where a blurred noise field is in its top `porosity` quantile, label 0
    (solid) elsewhere; with `inert` > 0 a second blurred field turns that fraction of the solid
    into label 2 (neither conductive nor reactive)."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    f = gaussian_filter(rng.standard_normal(shape), sigma)
    img = (f > np.quantile(f, 1 - porosity)).astype(np.uint8)
    if inert:
        g = gaussian_filter(rng.standard_normal(shape), sigma)
        img[(g > np.quantile(g, 1 - inert)) & (img == 0)] = 2
    return img


# name -> (periodic y/z, input builder, constructor kwargs, solve kwargs, reference code or test)
IMPEDANCE_CASES = {
    "imp_deadend": (False, _imp_deadend, {}, {}, "tests/test_taufactor.py:253-259"),
    "imp_throughpore": (False, _imp_throughpore, {}, {}, "tests/test_taufactor.py:261-267"),
    "imp_blob": (False, lambda: _imp_blob((20, 14, 12), 1), {}, {}, "electrode.py:160-351"),
    "imp_blob3": (False, lambda: _imp_blob((20, 14, 12), 2, inert=0.3), {}, {}, "electrode.py:160-351"),
    "imp_swap": (False, lambda: _imp_blob((18, 12, 14), 3),
                 {"conductive_label": 0, "reactive_label": 1, "spacing": 0.5}, {}, "electrode.py:167-176"),
    "imp_limit": (False, lambda: _imp_blob((18, 12, 10), 7), {}, {"iter_limit": 150}, "electrode.py:302-314"),
    "imp_nyquist": (False, lambda: _imp_blob((8, 6, 6), 4), {"mode": "nyquist"}, {}, "electrode.py:192-197"),
    "pimp_blob": (True, lambda: _imp_blob((16, 12, 10), 5), {}, {}, "electrode.py:369-402"),
    "pimp_odd": (True, lambda: _imp_blob((14, 9, 11), 6, inert=0.2), {}, {}, "electrode.py:369-402"),
}


# Full-size cases of the benchmark configurations, solved by the reference itself on the host
# (``make_golden.py fullsize``; minutes each). name -> (kind, input builder, constructor kwargs,
# solve kwargs, what it is). Only scalars and the [Nx-1] layer flux are stored; the GPU tests
# regenerate the volumes from their seeds.
def c2_volume0():
    from taufactor_gb300.synthetic import batch_256

    return batch_256(n=1, workers=1)[0]


def c3_volume15():
    from taufactor_gb300.synthetic import uneven_volume

    return uneven_volume(15)  # 256 x 256 x 192, the largest PeriodicSolver volume of the batch


def c4_crop128():
    from taufactor_gb300.synthetic import three_phase

    return three_phase(320)[:128, :128, :128]


def blur64():
    from taufactor_gb300.synthetic import blurred_noise

    return blurred_noise((64, 64, 64), 2.0, 0.5, 77)


FULLSIZE_CASES = {
    "c2_v0_cc2": ("binary", c2_volume0, {}, {"conv_crit": 1e-2}, "16 x 256^3 workload, volume 0"),
    "c2_v0_cc4": ("binary", c2_volume0, {}, {"conv_crit": 1e-4}, "16 x 256^3 workload, volume 0"),
    "c3_v15_periodic": ("periodic", c3_volume15, {}, {"conv_crit": 1e-4}, "uneven batch, volume 15"),
    "c4_crop128": ("multiphase", c4_crop128, {"diffusivities": {0: 0.0, 1: 1.0, 2: 0.1}},
                   {"conv_crit": 1e-4}, "three-label 320^3 volume, first 128^3"),
}

# The reference's precision argument (taufactor.py:24, :33): float64 sweeps.
# name -> (kind, input builder, solve kwargs)
DOUBLE_CASES = {
    "f64_bernoulli100": ("binary", bernoulli_100, {"conv_crit": 2e-2}),
    "f64_blur64": ("binary", blur64, {"conv_crit": 1e-4}),
    "f64_blur64_periodic": ("periodic", blur64, {"conv_crit": 1e-4}),
}
