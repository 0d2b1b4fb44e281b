"""Shared fixtures.  Tests marked ``gpu`` need a GB300; the rest run on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden" / "ref_scenarios.npz"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def pbf():
    import __graft_entry__ as ge

    return ge.load_package()


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


def golden_scenarios(g) -> list[str]:
    return sorted({k.split("/")[0] for k in g})


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle

    return oracle


def oracle_config(oracle, values):
    fields = ["x_min", "x_max", "y_min", "y_max", "z_min", "z_max", "x_n", "y_n", "z_n",
              "timestep_length", "rest_density"]
    cfg = oracle.Config()
    for f, v in zip(fields, values):
        setattr(cfg, f, float(v))
    return cfg


def pbf_params_from_config(pbf, values, mode):
    """pbf_params carrying the .par values of a golden config."""
    p = pbf.default_params(mode)
    (p.x_min, p.x_max, p.y_min, p.y_max, p.z_min, p.z_max, p.x_n, p.y_n, p.z_n,
     p.time_step_length, p.rest_density) = [float(v) for v in values]
    return p
