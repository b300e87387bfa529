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


def test_autotune_cache_roundtrip(tmp_path):
    """The autotuner's cache file (host-only logic): load a table, list it,
    save it elsewhere and load it back unchanged; malformed lines are
    skipped."""
    from regot import _lib

    lib = _lib.load()
    src = tmp_path / "tune.tsv"
    src.write_text(
        "NVIDIA GB300 sm152\tmixed\t3\t26\t1\t61.720\t48.100\n"
        "NVIDIA GB300 sm152\tfp64\t0\t26\t0\t2329.140\t2401.000\n"
        "a line without enough fields\n"
        "NVIDIA GB300 sm152\tmixed\t99\t26\t1\t1.0\t2.0\n")
    lib.regot_autotune_clear()
    assert lib.regot_autotune_load(str(src).encode()) == 2
    rows = _lib.autotune_entries()
    assert len(rows) == 2
    assert ["NVIDIA GB300 sm152", "mixed", "3", "26", "1", "61.720", "48.100"] in rows
    dst = tmp_path / "out.tsv"
    assert lib.regot_autotune_save(str(dst).encode()) == 2
    lib.regot_autotune_clear()
    assert _lib.autotune_entries() == []
    assert lib.regot_autotune_load(str(dst).encode()) == 2
    assert sorted(_lib.autotune_entries()) == sorted(rows)
    lib.regot_autotune_clear()
    assert lib.regot_force_pass_config(1) == -1
    assert lib.regot_force_pass_config(-1) == 1
