"""Shared fixtures.  The oracle (oracle/) is the checker; the product is the
CUDA library behind helioselene_gb300."""

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

import oracle  # noqa: E402  (checker)

GOLDEN = ROOT / "tests" / "golden" / "vectors.json"
CURVES = {"helios": 0, "selene": 1}


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300)")


@pytest.fixture(scope="session")
def golden():
    return json.loads(GOLDEN.read_text())


@pytest.fixture(scope="session")
def ctx():
    import helioselene_gb300 as hs
    c = hs.Context(0)
    yield c
    c.close()


def oracle_inputs(curve: int, n: int, seed: int, edge_fraction: float = 0.0):
    """Seeded scalars + affine bases; bases come from the oracle's SWU map."""
    from helioselene_gb300.workload import make_workload
    w = make_workload(curve, n, seed, edge_fraction)
    pts = oracle.map_to_curve(curve, w.u.reshape(-1)).reshape(n, 64)
    return w.scalars.copy(), pts, w
