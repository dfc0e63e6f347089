import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _library_stale(lib_path, src_dirs):
    if not os.path.exists(lib_path):
        return True
    built = os.path.getmtime(lib_path)
    for d in src_dirs:
        for name in os.listdir(d):
            if name.endswith((".cu", ".cuh", ".cpp", ".h")) and os.path.getmtime(os.path.join(d, name)) > built:
                return True
    return False


def pytest_sessionstart(session):
    """The tests exercise the compiled library (there is no fallback to run
    instead): build it once when this checkout has no up-to-date build."""
    from tealeaf_cuda_gb300 import LIB_PATH, make_lib
    if _library_stale(LIB_PATH, [os.path.join(ROOT, "tealeaf_cuda_gb300", "csrc"), os.path.join(ROOT, "include")]):
        make_lib.build()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")
