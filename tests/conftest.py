import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# Checkout of the reference (formura/formura): read as text by the CPU tests
# that compile its programs and drivers; those tests skip without it.
REFERENCE = os.environ.get("FORMURA_REFERENCE", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the CUDA library")


def bits_equal(a, b) -> bool:
    """Bit-for-bit equality of two arrays (so +0 and -0 differ, unlike ==)."""
    import numpy as np
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and a.tobytes() == b.tobytes()
