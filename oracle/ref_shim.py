"""Import the reference package from its source tree (test infrastructure only).

The reference (tldr-group/taufactor v1.2.1) imports IPython, matplotlib and scikit-image (and
psutil) at module level for plotting and surface metrics; none of them is used on the solve path
unless ``verbose='plot'|'debug'``. Stub modules stand in for them (psutil only where it is not
installed). Bytecode writing is disabled so the
read-only source tree is left untouched.

The golden-vector generator and the CPU oracle tests use this where the source tree exists
(``TAUFACTOR_REFERENCE`` names it, or else a directory ``reference`` beside the repository's own
directory is used); the benchmark's reference arm uses it on an installed copy of the reference
(``baseline/_ref``), which is what travels to the GPU machine.
"""
from __future__ import annotations

import importlib.util
import os
import sys
import types

# a checkout of the reference beside this repository: <parent>/reference next to <parent>/<repo>
DEFAULT_REFERENCE = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                                 "reference")


def reference_root() -> str | None:
    root = os.environ.get("TAUFACTOR_REFERENCE", DEFAULT_REFERENCE)
    return root if os.path.isdir(os.path.join(root, "taufactor")) else None


def import_reference(root: str | None = None):
    """Return the reference ``taufactor`` module, or None if its source tree is absent.

    ``root``: a directory holding the ``taufactor`` package (a source checkout, or an installed
    copy such as the benchmark's ``baseline/_ref``); default: ``reference_root()``."""
    root = root if root is not None else reference_root()
    if root is None or not os.path.isdir(os.path.join(root, "taufactor")):
        return None
    sys.dont_write_bytecode = True
    for name in ("IPython", "IPython.display", "matplotlib", "matplotlib.pyplot",
                 "skimage", "skimage.measure"):
        if name not in sys.modules:
            sys.modules[name] = types.ModuleType(name)
    # psutil: only the surface metrics' memory checks use it (taufactor/metrics/surfaces.py:253,
    # :335); a stub where it is not installed
    if "psutil" not in sys.modules and importlib.util.find_spec("psutil") is None:
        sys.modules["psutil"] = types.ModuleType("psutil")
    sys.modules["IPython.display"].clear_output = lambda *a, **k: None
    sys.modules["IPython"].display = sys.modules["IPython.display"]
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    sys.modules["skimage"].measure = sys.modules["skimage.measure"]
    if root not in sys.path:
        sys.path.insert(0, root)
    import taufactor  # noqa: E402

    return taufactor
