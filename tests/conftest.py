import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


GOLDEN = os.path.join(REPO, "tests", "golden")


def golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def parse_param_text(text):
    """Key=value lines as in the reference's input files (first occurrence wins)."""
    d = {}
    for line in str(text).splitlines():
        if "=" in line:
            k, v = line.split("=", 1)
            d.setdefault(k, v.strip())
    return d
