"""Import shim for the reference's CPU solver (fixture generation only).

ORACLE — test infrastructure.  Used only by ``tests/golden/make_golden.py`` in a
container where the S-PGO sources are mounted; nothing at test or bench time
reads the reference.

The reference CPU path (``PythonUtils/Optimizer.py``) imports ``pypose``,
``cv2`` and ``matplotlib``, none of which are installed.  Only ``cv2.Rodrigues``
is used on the solver path (``PythonUtils/LieUtils.py:22-33``); it is replaced
by the oracle's numpy Rodrigues.  ``Optimizer.update_depths`` calls
``float()`` on a shape-(1,) array, which numpy 2 rejects (``Optimizer.py:665``);
it is replaced by an equivalent that takes the scalar first.
"""
from __future__ import annotations

import sys
import types

import numpy as np

from . import lie


def _rodrigues(x):
    x = np.asarray(x, dtype=np.float64)
    if x.size == 3:
        return lie.exp_so3(x.reshape(3)), None
    return lie.log_so3(x.reshape(3, 3)).reshape(3, 1), None


def install(reference_root: str):
    """Stub the missing modules and put the reference on sys.path."""
    sys.dont_write_bytecode = True
    cv2 = types.ModuleType("cv2")
    cv2.Rodrigues = _rodrigues
    sys.modules.setdefault("cv2", cv2)
    sys.modules.setdefault("pypose", types.ModuleType("pypose"))
    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    backends = types.ModuleType("matplotlib.backends")
    agg = types.ModuleType("matplotlib.backends.backend_agg")
    agg.FigureCanvasAgg = object
    mpl.pyplot = plt
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", plt)
    sys.modules.setdefault("matplotlib.backends", backends)
    sys.modules.setdefault("matplotlib.backends.backend_agg", agg)
    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
    from PythonUtils import Optimizer as opt_mod  # noqa: E402

    def update_depths(self, delta_alpha):
        delta_alpha = np.asarray(delta_alpha).reshape(-1)
        for idx in range(self.number_of_landmarks):
            val = float(self.estimated_inverse_depths[idx]) + float(delta_alpha[idx])
            self.estimated_inverse_depths[idx] = max(self.min_alpha, min(val, self.max_alpha))

    opt_mod.Optimizer.update_depths = update_depths
    return opt_mod
