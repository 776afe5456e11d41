import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (HERE, ROOT, os.path.join(ROOT, "octree-cuda_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the native library on the device")
    config.addinivalue_line("markers", "slow: full-size cases")


def pytest_sessionstart(session):
    # build the native libraries and the oracle once per test session
    import __graft_entry__

    __graft_entry__.build()
