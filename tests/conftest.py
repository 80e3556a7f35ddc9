"""Test configuration: the gpu marker and import paths.

Tests marked ``gpu`` need a CUDA device and the built library; everything else
runs on the CPU (oracle against the golden vectors, host logic, ABI exports).
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "worldline-flux-tube-lattice_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")
