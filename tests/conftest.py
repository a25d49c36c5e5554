"""Shared fixtures: build the library and the oracle once per session.

Markers: ``gpu`` (needs a CUDA device; run with ``-m gpu``) and ``slow``
(long CPU oracle runs; skipped unless FS_SLOW=1)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

REFERENCE = "/root/reference"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU")
    config.addinivalue_line("markers", "slow: long CPU run, enabled with FS_SLOW=1")


def pytest_collection_modifyitems(config, items):
    if os.environ.get("FS_SLOW") == "1":
        return
    skip = pytest.mark.skip(reason="slow: set FS_SLOW=1")
    for it in items:
        if "slow" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def fslib():
    from factsieve_gb300 import build as fsbuild
    import factsieve_gb300 as fs
    if not os.path.exists(fs.LIB_PATH):
        fsbuild.build()
    return fs


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def refmath():
    """The reference's own verifyprime.c, when the reference tree is on this machine."""
    import oracle
    if os.path.isdir(REFERENCE):
        try:
            oracle.build_ref(REFERENCE)
        except Exception:
            pass
    r = oracle.ref()
    if r is None:
        pytest.skip("reference tree not present: verifyprime.c checker not built")
    return r


@pytest.fixture(scope="session")
def ctx(fslib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = fslib.Context(0)
    yield c
    c.close()
