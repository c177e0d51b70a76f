"""The Lanczos3 tap-weight polynomials of csrc/sampling.cuh: the table in the
header is the one glass_gb300/lanczos_poly.py fits, and evaluated in float32
as the kernel does (Horner with fused multiply-adds, pairs E +- O) it stays
within 1.5e-7 of sinc(d) sinc(d/3) in float64 (t = 0 included) and sums to the exact weight
sum within 5e-7 over t in [0, 1)."""

from __future__ import annotations

import re
from pathlib import Path

import numpy as np

from glass_gb300.lanczos_poly import fit, lanczos3

HEADER = Path(__file__).resolve().parent.parent / "glass_gb300" / "csrc" / "sampling.cuh"


def _header_table() -> dict:
    """{"EA": c0..c5, "OA": ...} from the l3_even_* / l3_odd_* Horner functions."""
    text = HEADER.read_text()
    table = {}
    for parity, pair, body in re.findall(r"float l3_(even|odd)_([abc])\(float x\) \{(.*?)\n\}", text, re.S):
        lits = [float(v) for v in re.findall(r"(-?\d\.\d+e[+-]\d+)f", body)]
        table[("E" if parity == "even" else "O") + pair.upper()] = np.array(lits[::-1], dtype=np.float32)
    assert len(table) == 6
    return table


def test_header_table_is_the_fit():
    table = _header_table()
    for pair, center in (("A", 0.5), ("B", 1.5), ("C", 2.5)):
        e, o, err = fit(center)
        assert err < 3e-10
        np.testing.assert_array_equal(table["E" + pair], e.astype(np.float32))
        np.testing.assert_array_equal(table["O" + pair], o.astype(np.float32))


def _fma(a, b, c):
    return np.float32(np.float64(a) * np.float64(b) + np.float64(c))


def test_float32_weights_match_lanczos3():
    table = _header_table()
    f32 = np.float32
    ts = np.linspace(0.0, 1.0, 4001, endpoint=False).astype(np.float32)
    worst, worst_sum = 0.0, 0.0
    for t in ts:
        u = f32(t - f32(0.5))
        x = f32(u * u)

        def poly(c):
            p = c[5]
            for k in (4, 3, 2, 1, 0):
                p = _fma(p, x, c[k])
            return p

        ea, oa = poly(table["EA"]), f32(u * poly(table["OA"]))
        eb, ob = poly(table["EB"]), f32(u * poly(table["OB"]))
        ec, oc = poly(table["EC"]), f32(u * poly(table["OC"]))
        w = [f32(ec + oc), f32(eb + ob), f32(ea + oa), f32(ea - oa), f32(eb - ob), f32(ec - oc)]
        exact = lanczos3(float(t) - np.arange(-2, 4, dtype=np.float64))
        worst = max(worst, float(np.abs(np.asarray(w, np.float64) - exact).max()))
        worst_sum = max(worst_sum, abs(float(np.sum(np.asarray(w, np.float64))) - float(exact.sum())))
    assert worst < 1.5e-7
    assert worst_sum < 5e-7
