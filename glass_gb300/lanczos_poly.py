"""Coefficients of the Lanczos3 tap weights used by the CUDA warps.

For a sample at fractional offset t in [0, 1) the six taps k = -2..3 weigh
L(t - k) with L(d) = sinc(d) sinc(d / 3) (zero for |d| >= 3).  With
u = t - 1/2 the taps pair up as L(c + u) and L(c - u) for c = 1/2, 3/2, 5/2
(L is even), so each pair is E_c(u) +- O_c(u) with E_c even and O_c odd in
u.  This script fits E_c(u) = sum_j e_j u^(2j) and O_c(u) = u sum_j o_j u^(2j)
(j = 0..5) by float64 least squares on u in [0, 1/2] and prints the C table
pasted into csrc/sampling.cuh; the fit error is below 3e-10, far under
float32 rounding.  Run: python -m glass_gb300.lanczos_poly
"""

from __future__ import annotations

import numpy as np

DEGREE = 5


def lanczos3(d: np.ndarray) -> np.ndarray:
    d = np.asarray(d, dtype=np.float64)
    out = np.sinc(d) * np.sinc(d / 3.0)
    out[np.abs(d) >= 3.0] = 0.0
    return out


def fit(center: float, samples: int = 20001):
    u = np.linspace(0.0, 0.5, samples)
    even = 0.5 * (lanczos3(center + u) + lanczos3(center - u))
    odd = 0.5 * (lanczos3(center + u) - lanczos3(center - u))
    basis = np.vander(u * u, DEGREE + 1, increasing=True)
    e, *_ = np.linalg.lstsq(basis, even, rcond=None)
    o, *_ = np.linalg.lstsq(u[:, None] * basis, odd, rcond=None)
    err = max(np.abs(basis @ e - even).max(), np.abs((u[:, None] * basis) @ o - odd).max())
    return e, o, err


def main() -> None:
    for name, center in (("A", 0.5), ("B", 1.5), ("C", 2.5)):
        e, o, err = fit(center)
        print(f"// pair {name} (c = {center}): max fit error {err:.1e}")
        print(f"__device__ constexpr float kL3E{name}[6] = {{" + ", ".join(f"{v:.9e}f" for v in e) + "};")
        print(f"__device__ constexpr float kL3O{name}[6] = {{" + ", ".join(f"{v:.9e}f" for v in o) + "};")


if __name__ == "__main__":
    main()
