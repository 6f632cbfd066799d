"""Philox4x32-10 of this repository (numpy host version used by the model
builders, the oracle's C version, a plain-Python version) against vectors
from cuRAND's host generator (tests/golden/philox_curand.json)."""
import json
import os

import numpy as np

from oracle import models as om
from tests.test_oracle_models import philox as py_philox

HERE = os.path.dirname(os.path.abspath(__file__))


def vectors():
    with open(os.path.join(HERE, "golden", "philox_curand.json")) as f:
        return json.load(f)["vectors"]


def test_oracle_c_philox():
    for v in vectors():
        for b in v["blocks"]:
            assert list(om.philox(*b["counter"], v["seed"])) == b["out"]


def test_python_philox():
    for v in vectors():
        for b in v["blocks"]:
            assert py_philox(b["counter"], v["seed"]) == b["out"]


def test_numpy_philox_of_the_model_builders():
    from vahana_gb300 import philox
    for v in vectors():
        ks = np.arange(16, dtype=np.uint64)
        w = philox.philox4x32_10(np.zeros(16, np.uint64), np.zeros(16, np.uint64), ks,
                                 np.zeros(16, np.uint64), v["seed"])
        for k, b in enumerate(v["blocks"]):
            assert [int(w[i][k]) for i in range(4)] == b["out"]
