"""Test configuration: repo root on sys.path and the `gpu` marker.

`-m "not gpu"` runs the oracle pins, the host logic and the ABI checks (no
GPU); `-m gpu` runs the parity tests through the C ABI on a GB300.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the CUDA library")
