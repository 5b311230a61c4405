"""Calibration on the device (SetData): the SQ8U affine / symmetric ranges and SQ4U's 1%/99% quantile
range equal the oracle's calibrator (quant/utils.hpp:31-40 semantics) bit for bit, on data with
negative values, signed zeros, heavy ties, outliers and sizes whose 10% / 1% cut-offs round."""

import os
import tempfile

import numpy as np
import pytest

from tests.helpers import write_glass

pytestmark = pytest.mark.gpu


def datasets():
    rng = np.random.default_rng(7)
    a = rng.standard_normal((300_001, 37)).astype(np.float32) * 3.0 - 1.0
    b = np.rint(rng.uniform(0, 255, (100_000, 128))).astype(np.float32)  # ties everywhere
    c = np.array([[0.0, -0.0, 5.0, -7.5, 1e30], [2.0, 2.0, -0.0, 0.0, -1e-30], [3.0, 1.0, 1.0, 1.0, 1.0]],
                 np.float32)
    d = rng.standard_normal((50_000, 96)).astype(np.float32)
    d[::997] *= 1e6  # outliers in the trimmed tails
    return {"normal37": a, "ties128": b, "tiny": c, "outliers96": d}


@pytest.fixture(scope="module")
def tiny_graph():
    path = os.path.join(tempfile.mkdtemp(), "g2.glass")
    write_glass(path, np.array([[1, -1], [0, -1]], np.int32), [0])
    return path


@pytest.mark.parametrize("name", ["normal37", "ties128", "tiny", "outliers96"])
@pytest.mark.parametrize("quant,metric", [("SQ8U", "L2"), ("SQ8U", "IP"), ("SQ4U", "L2"), ("SQ4U", "IP"), ("SQ2U", "L2"), ("SQ4UA", "L2")])
def test_device_calibration_matches_oracle(gpu, oracle, tiny_graph, name, quant, metric):
    x = datasets()[name]
    s = gpu.Searcher(gpu.Graph(tiny_graph), x, metric, quant)
    _, params = s.calibration()
    want = oracle.Quant(quant, metric, x).params
    np.testing.assert_array_equal(np.array(params, np.float32), want)
