"""Coefficients of the Lanczos3 tap weights used by the CUDA warps.

For a sample at fractional offset t in [0, 1) the six taps k = -2..3 weigh
L(t - k) with L(d) = sinc(d) sinc(d / 3) (zero for |d| >= 3).  With
u = t - 1/2 the taps pair up as L(c + u) and L(c - u) for c = 1/2, 3/2, 5/2
(L is even), so each pair is E_c(u) +- O_c(u) with E_c even and O_c odd in
u.  This script fits E_c(u) = sum_j e_j u^(2j) and O_c(u) = u sum_j o_j u^(2j)
(j = 0..5) by float64 least squares on u in [0, 1/2] and prints the six
Horner evaluations, with the coefficients as float literals (immediate
operands of the fused multiply-adds), pasted into csrc/sampling.cuh; the fit
error is below 3e-10, far under float32 rounding.  It also prints the
derivatives d/dx of those float32 polynomials (coefficients j * c_j, degree
4), pasted into csrc/adjoint.cuh: the Gauss-Newton refinement differentiates
exactly the weights the warp samples with.
Run: python -m glass_gb300.lanczos_poly
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


def horner_source(name: str, coefs) -> str:
    c = [f"{float(v):.9e}f" for v in coefs]
    body = f"  float p = {c[5]};\n"
    for j in (4, 3, 2, 1):
        body += f"  p = __fmaf_rn(p, x, {c[j]});\n"
    body += f"  return __fmaf_rn(p, x, {c[0]});\n"
    return f"__device__ __forceinline__ float l3_{name}(float x) {{\n{body}}}"


def derivative_source(name: str, coefs32) -> str:
    """d/dx of the float32 polynomial sum_j c_j x^j (degree 4, Horner)."""
    d = [float(j) * float(coefs32[j]) for j in range(1, DEGREE + 1)]
    c = [f"{float(np.float32(v)):.9e}f" for v in d]
    body = f"  float p = {c[4]};\n"
    for j in (3, 2, 1):
        body += f"  p = __fmaf_rn(p, x, {c[j]});\n"
    body += f"  return __fmaf_rn(p, x, {c[0]});\n"
    return f"__device__ __forceinline__ float l3_{name}_dx(float x) {{\n{body}}}"


def main(derivatives: bool = False) -> None:
    for name, center in (("a", 0.5), ("b", 1.5), ("c", 2.5)):
        e, o, err = fit(center)
        if derivatives:
            print(derivative_source("even_" + name, e.astype(np.float32)))
            print(derivative_source("odd_" + name, o.astype(np.float32)))
            continue
        print(f"// pair {name.upper()} (c = {center}): max fit error {err:.1e}")
        print(horner_source("even_" + name, e.astype(np.float32)))
        print(horner_source("odd_" + name, o.astype(np.float32)))


if __name__ == "__main__":
    import sys

    main(derivatives="--derivatives" in sys.argv[1:])
