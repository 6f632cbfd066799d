"""Philox4x32-10 of this repository (numpy host version used by the model
builders, the oracle's C version, a plain-Python version) against vectors
from cuRAND's host generator (tests/golden/philox_curand.json)."""
import json
import os

import numpy as np
import pytest

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


def test_unit_bits_match_the_double_conversion(tmp_path):
    """u64_to_unit_bits (vahana.jl_gb300/csrc/vg_philox.cuh), the integer
    construction behind unit_below, gives the bit pattern of u64_to_unit on
    powers of two, their neighbours and 2 * 10^6 random inputs."""
    import os
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "unit_bits.cpp"
    src.write_text(r"""
#include "vg_philox.cuh"
#include <cstdio>
#include <cstring>
#include <random>
int main() {
  std::mt19937_64 g(7);
  long bad = 0;
  auto chk = [&](uint64_t x) {
    double u = vg::u64_to_unit(x);
    uint64_t b;
    std::memcpy(&b, &u, 8);
    bad += b != vg::u64_to_unit_bits(x);
    bad += vg::unit_below(x, u);  // never below itself
  };
  for (int s = 0; s < 64; s++) { chk(1ull << s); chk((1ull << s) - 1); chk(~0ull >> s); }
  chk(0);
  for (int i = 0; i < 1000000; i++) { uint64_t x = g(); chk(x); chk(x >> (i % 64)); }
  std::printf("%ld\n", bad);
  return bad != 0;
}
""")
    exe = tmp_path / "unit_bits"
    subprocess.run(["g++", "-O2", "-I", os.path.join(root, "vahana.jl_gb300", "csrc"), str(src),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "0"

