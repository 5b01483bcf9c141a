"""pytest configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a GB300 and the built libgb300blas (``__graft_entry__.build()``); the rest
run on any CPU host.  Run ``pytest -m "not gpu"`` here and ``pytest -m gpu`` on the GPU machine.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built libgb300blas")
