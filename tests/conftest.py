"""Test configuration: the `gpu` marker and import paths.

`-m "not gpu"` runs the oracle pins, host logic and ABI-export checks on
CPU; `-m gpu` runs the CUDA parity tests through the C ABI.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "cfmultigrid.jl_gb300"), os.path.join(ROOT, "oracle"), os.path.dirname(__file__),
          os.path.join(os.path.dirname(__file__), "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: large CPU oracle cases")
