import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built library")


def _load(name):
    with np.load(os.path.join(GOLDEN, name)) as d:
        return {k: d[k] for k in d.files}


@pytest.fixture(scope="session")
def explicit():
    """The reference's known-answer data (tests/pimc/explicit_data of the reference)."""
    return _load("explicit_example.npz")


@pytest.fixture(scope="session")
def runs():
    """Outputs of the reference engine itself on seeded models (make_golden.py)."""
    return _load("reference_runs.npz")


def case_of(runs, name):
    pre = name + "/"
    return {k[len(pre):]: v for k, v in runs.items() if k.startswith(pre)}


def prepared_from_case(c, P, K=None):
    from pibronic_gb300 import vibronic_io
    from pibronic_gb300.plan import PreparedModels
    vib = vibronic_io.model_from_text(str(c["vib_json"]))
    rho = vibronic_io.model_from_text(str(c["rho_json"]), diagonal=True)
    db = float(c["delta_beta"])
    return PreparedModels(vib, rho, P, beta=float(c["beta"]), delta_beta=db if db > 0 else None, K=K)


def oracle_box_from_case(c, P, X=None, B=None):
    from oracle import pimc_oracle as po
    vib = po.model_from_text(str(c["vib_json"]))
    rho = po.model_from_text(str(c["rho_json"]), diagonal=True)
    X = X if X is not None else c["q"].shape[0]
    T = 1.0 / (float(c["beta"]) * po.KB_EV)
    db = float(c["delta_beta"])
    return po.OracleBox(vib, rho, X, B or X, P, T, delta_beta=db if db > 0 else None,
                        draw_sources=False)
