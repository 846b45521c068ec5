import json
import math
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "compound-prism-designer_gb300")
for p in (ROOT, PKG_DIR, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")

# Build (or refresh) the product library and the oracle before any test imports them.
import build_ext  # noqa: E402  (compound-prism-designer_gb300/build_ext.py)

build_ext.build()
import oracle as _oracle  # noqa: E402

_oracle.build()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def f1_design_dict():
    """The reference's known design (src/fitness.rs:153-257) as the flat dict the
    oracle and the product builders share, with the detector auto-positioned by the
    oracle's own positioning."""
    import oracle as O

    g = load_golden("f1_known_design.json")["design"]
    d = dict(g)
    d["angles"] = [math.radians(a) for a in g["angles_deg"]]
    d["max_incident_angle"] = math.radians(g["max_incident_angle_deg"])
    e, pos, fl = O.position_detector(d, g["acceptance"])
    assert e == O.OK
    d["det_position"] = pos
    d["det_flipped"] = fl
    return d


@pytest.fixture(scope="session")
def f1():
    return f1_design_dict()
