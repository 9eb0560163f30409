"""Shared test setup: import paths and the `gpu` marker.

`-m "not gpu"` runs the oracle against the reference's golden vectors, the
host-side logic and the C-ABI load/export checks; `-m gpu` runs the CUDA
path against the oracle on a GB300.
"""

import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "blademaster-lab_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
