"""DQ map parity, pinned to the reference: tests/golden/dq.npz holds the
int16 DQ bits that the reference's own `_resident_dq_map_python`
(src/glass/engine/resident_cuda.py:3110-3297) computed on seeded maps with
non-finite values, zero / negative weights, coverage at the 0.5 edge and
geometric coverage at the partial-coverage edge (tests/golden/make_golden.py
`make_dq`).  The oracle and the library's host routine (gg_dq_map_i16) must
equal it bit for bit; the device DQ written by the integrator is checked
against the oracle in test_gpu_integrate.py."""

from __future__ import annotations

import numpy as np
import pytest

from oracle.integration import dq_map

from .conftest import GOLDEN


@pytest.fixture(scope="module")
def golden_dq():
    return np.load(GOLDEN / "dq.npz", allow_pickle=False)


def _cases(g):
    for name in (str(n) for n in g["_names"]):
        maps = {k: (g[f"{name}/{k}"] if f"{name}/{k}" in g.files else None)
                for k in ("coverage", "low", "high", "geometric")}
        yield name, g[f"{name}/master"], g[f"{name}/weight"], maps, int(g[f"{name}/active"]), g[f"{name}/dq"]


def test_oracle_dq_matches_reference_golden(golden_dq):
    n = 0
    for name, master, weight, maps, active, expected in _cases(golden_dq):
        got = dq_map(master, weight, maps["coverage"], maps["low"], maps["high"], maps["geometric"], active)
        np.testing.assert_array_equal(got, expected, err_msg=name)
        n += 1
    assert n == 12


def test_library_dq_map_matches_reference_golden(built_library, golden_dq):
    from glass_gb300 import _glass_cuda_native as native

    for name, master, weight, maps, active, expected in _cases(golden_dq):
        got = native.resident_dq_map_count_maps_i16(master, weight, maps["coverage"], maps["low"], maps["high"],
                                                    maps["geometric"], active)
        np.testing.assert_array_equal(got, expected, err_msg=name)
