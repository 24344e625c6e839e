"""Spanning-cluster test used by the reference's zero-flux fallback (test infrastructure only).

Restates ``extract_through_feature(mask, 1, 'x')`` (taufactor/metrics/connectivity.py:138-213)
as called from ``ThroughTransportSolver.compute_metrics`` (taufactor/taufactor.py:318-327):
6-connected labelling (``scipy.ndimage.label`` with the connectivity-1 structure, as the
reference uses), then "does any label occur on both the first and the last x-slice"
(``find_spanning_labels``, connectivity.py:81-113). The reference labels without periodic
wrap even for the periodic solvers; so does this.
"""
from __future__ import annotations

import numpy as np
from scipy.ndimage import generate_binary_structure, label


def spans_axis0(mask: np.ndarray) -> bool:
    """True if a face-connected cluster of ``mask`` touches both x = 0 and x = Nx-1."""
    mask = np.asarray(mask, dtype=bool)
    if not mask.any():
        return False
    lab, _ = label(mask, structure=generate_binary_structure(3, 1))
    front = set(np.unique(lab[0])) - {0}
    back = set(np.unique(lab[-1])) - {0}
    return bool(front & back)
