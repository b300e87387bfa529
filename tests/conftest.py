import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("regot-python_gb300", "oracle", "tests"):
    p = os.path.join(REPO, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the compiled library")


QROT_CG_PATHS = {"bitmask": 1, "lists": 2, "lists-global": 3}


@pytest.fixture(params=list(QROT_CG_PATHS))
def qrot_cg_path(request):
    """Runs a test with the QROT Schur CG on the sigma bitmask, on the index
    lists built from it (vectors exchanged through distributed shared
    memory), and on the lists with the global-memory exchange (the forced
    choices of regot_force_qrot_cg_path), restoring the size-based choice
    afterwards."""
    from regot import _lib

    lib = _lib.load()
    old = lib.regot_force_qrot_cg_path(QROT_CG_PATHS[request.param])
    try:
        yield request.param
    finally:
        lib.regot_force_qrot_cg_path(old)
