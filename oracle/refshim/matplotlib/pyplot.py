"""``matplotlib.pyplot`` stand-in for the oracle harness.

The reference does ``from matplotlib.pyplot import *`` and then uses ``np``,
``math`` and ``sys`` without importing them (radon_tgv_primal_dual_3d.py:861, 1226,
1238); real pyplot re-exports those names, so this stub does too.  Plot calls are
no-ops: the harness always passes ``plott=[0, ...]``.
"""
import math  # noqa: F401
import sys  # noqa: F401

import numpy as np  # noqa: F401


def _noop(*_a, **_k):
    return None


figure = imshow = title = draw = pause = close = _noop


def fignum_exists(*_a, **_k):
    return False


class _CM:
    gray = None


cm = _CM()
