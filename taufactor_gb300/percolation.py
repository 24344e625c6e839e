"""Spanning-path test behind the zero-flux branch of the convergence check.

The reference (taufactor/taufactor.py:318-327) calls
``extract_through_feature(mask, 1, 'x')`` (taufactor/metrics/connectivity.py:138-213) on the
host whenever a layer flux of a batch element is exactly zero: face-connected labelling and a
check whether any cluster touches both x-faces, without periodic wrap. This module keeps that
host-side step (it is outside the sweep loop and runs only on that branch) with the same
labelling rule.
"""
from __future__ import annotations

import numpy as np
from scipy.ndimage import generate_binary_structure, label


def spans_x(mask: np.ndarray) -> bool:
    """True if a 6-connected cluster of ``mask`` [X,Y,Z] touches both x = 0 and x = X-1."""
    mask = np.asarray(mask, dtype=bool)
    if not mask.any():
        return False
    lab, _ = label(mask, structure=generate_binary_structure(3, 1))
    first = np.unique(lab[0])
    last = np.unique(lab[-1])
    common = np.intersect1d(first[first > 0], last[last > 0])
    return common.size > 0
