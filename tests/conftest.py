import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, 'bsam-in-matlab_gb300'), os.path.join(ROOT, 'oracle'), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a GB300 (sm_103) GPU and the CUDA library')
    config.addinivalue_line('markers', 'slow: several seconds of CPU work')
