"""Shared test setup: import paths, the `gpu` marker, oracle fixtures."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "biofem-ia_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); run with -m gpu")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle.pyoracle import Oracle
    return Oracle()


def golden_case(path):
    """(workload, meta, arrays) of a golden fixture made by tests/golden/make_golden.py."""
    import json
    import numpy as np
    from biofem import configs
    d = np.load(path)
    meta = json.loads(str(d["meta"]))
    opt = {k: meta[k] for k in ("dead_load", "iso_act") if k in meta}
    if meta.get("kind") == "sphere":
        keys = ("name", "freq", "index", "n_qp", "c33_iters", "pressure", "lambda_a", "jitter", "disp_rel")
        return configs.SphereWorkload(**{k: meta[k] for k in keys}, **opt), meta, d
    if meta.get("kind") == "cone":
        keys = ("name", "valence", "rings", "index", "n_qp", "c33_iters", "pressure", "z_sigma", "disp_rel")
        return configs.ConeWorkload(**{k: meta[k] for k in keys}, **opt), meta, d
    if meta.get("kind") == "capped":
        keys = ("name", "n_phi", "n_theta", "apex_vertex", "clamp", "index", "n_qp", "c33_iters", "pressure",
                "jitter", "disp_rel")
        return configs.CappedLVWorkload(**{k: meta[k] for k in keys}, **opt), meta, d
    if meta.get("kind") == "lv":
        keys = ("name", "freq", "index", "n_qp", "c33_iters", "pressure", "lambda_a", "nflip", "jitter")
        return configs.LVWorkload(**{k: meta[k] for k in keys}, **opt), meta, d
    keys = ("name", "nx", "ny", "n_qp", "c33_iters", "pressure", "z_sigma", "activation",
            "lambda_a", "disp_rel", "index")
    return configs.Workload(**{k: meta[k] for k in keys}, **opt), meta, d
