"""CPU checks of the C ABI library: it builds, loads without a GPU and
exports every function include/regot_gb300.h declares."""
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(REPO, "include", "regot_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(regot_[a-z0-9_]+)\s*\(", src)))


def test_header_lists_all_exports():
    from regot import _lib

    assert sorted(_lib.EXPORTS) == _declared()


def test_library_exports_every_declared_symbol():
    import build as regot_build

    path = regot_build.build()
    import ctypes

    lib = ctypes.CDLL(path)
    missing = [s for s in _declared() if not hasattr(lib, s)]
    assert not missing, missing


def test_no_device_raises_loudly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np

    import regot

    with pytest.raises(RuntimeError):
        regot.sinkhorn_bcd(np.ones((2, 2)), [0.5, 0.5], [0.5, 0.5], 0.1)
