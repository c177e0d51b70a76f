"""Differentiable affine warp and gradient-based sub-pixel registration.

``AffineWarp`` is a ``torch.autograd.Function`` whose forward is the device
warp ``gg_warp_affine_f32_device`` (bilinear or Lanczos3 sampling with the
semantics of src/glass/engine/warp.py:99-152, no overshoot clamp) and whose
backward is the hand-written adjoint ``gg_warp_affine_backward_f32_device``:
gradients with respect to the source image and to the six parameters of the
inverse (output -> source) affine map, sx = t0 x + t1 y + t2,
sy = t3 x + t4 y + t5.

``refine_affine`` improves a registration matrix (moving -> reference, the
convention of the reference's warps) by maximising the masked normalised
cross-correlation (or minimising the masked, photometrically matched SSD)
between the reference frame and the warped moving frame over the similarity /
affine / translation parameters by trust-region Newton steps (autograd
gradients through the adjoint, the Hessian from forward differences of the
gradient, Levenberg damping, capped steps).  The mask keeps pixels where
both frames and the sample are finite and drops single-frame outliers
(cosmic rays, hot pixels): a pixel whose residual after a linear photometric
match exceeds ``clip_sigma`` noise sigmas plus what a ``mask_shift_px``
misregistration of the smoother structure could explain is excluded, and so
is one whose moving-frame gradient exceeds twice the scaled reference
gradient plus three sigmas (structure the reference lacks).  The
reference's own refinement is a grid search over translations
(src/glass/engine/registration_metrics.py); this is the gradient path that
replaces it when the parameters are continuous.

The tensors are torch CUDA tensors (device memory and streams come from
PyTorch); the arithmetic is in libglass_gb300.so.  There is no CPU path: the
library must be loaded and a CUDA device present.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from glass_gb300 import _lib

_INTERP = {"bilinear": _lib.GG_INTERP_BILINEAR, "lanczos3": _lib.GG_INTERP_LANCZOS3}


def _interp_code(interpolation: str | int) -> int:
    if isinstance(interpolation, str):
        try:
            return _INTERP[interpolation]
        except KeyError:
            raise ValueError(f"interpolation must be one of {sorted(_INTERP)}") from None
    if int(interpolation) not in _INTERP.values():
        raise ValueError("interpolation must be bilinear or lanczos3")
    return int(interpolation)


def _theta_host(theta: torch.Tensor) -> np.ndarray:
    t = np.ascontiguousarray(theta.detach().to("cpu", torch.float64).numpy().reshape(-1))
    if t.size != 6:
        raise ValueError("theta must hold 6 affine parameters")
    if not np.all(np.isfinite(t)):
        raise ValueError("theta must be finite")
    return t


def _check_image(src: torch.Tensor) -> None:
    if not isinstance(src, torch.Tensor) or not src.is_cuda:
        raise ValueError("source must be a CUDA tensor")
    if src.dtype != torch.float32 or src.dim() != 2:
        raise ValueError("source must be a 2-D float32 tensor")


class AffineWarp(torch.autograd.Function):
    """out = warp(src; theta) with gradients for src and theta (float64)."""

    @staticmethod
    def forward(ctx, src: torch.Tensor, theta: torch.Tensor, interpolation: int = _lib.GG_INTERP_LANCZOS3,
                fill: float = float("nan"), src_all_finite: bool = False) -> torch.Tensor:
        _check_image(src)
        src = src.contiguous()
        t = _theta_host(theta)
        h, w = src.shape
        out = torch.empty_like(src)
        stream = torch.cuda.current_stream(src.device).cuda_stream
        _lib.call("gg_warp_affine_f32_device", ctypes.c_void_p(src.data_ptr()), h, w, t.ctypes.data,
                  int(interpolation), float(fill), int(bool(src_all_finite)), ctypes.c_void_p(out.data_ptr()),
                  ctypes.c_void_p(stream))
        ctx.save_for_backward(src)
        ctx.theta_host = t
        ctx.theta_meta = (theta.device, theta.dtype)
        ctx.interpolation = int(interpolation)
        return out

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        (src,) = ctx.saved_tensors
        grad_out = grad_out.contiguous().to(torch.float32)
        h, w = src.shape
        stream = torch.cuda.current_stream(src.device).cuda_stream
        grad_src = torch.zeros_like(src) if ctx.needs_input_grad[0] else None
        grad_theta_dev = torch.empty(6, dtype=torch.float64, device=src.device) if ctx.needs_input_grad[1] else None
        if grad_src is None and grad_theta_dev is None:
            return None, None, None, None, None
        _lib.call("gg_warp_affine_backward_f32_device", ctypes.c_void_p(src.data_ptr()), h, w,
                  ctx.theta_host.ctypes.data, ctx.interpolation, ctypes.c_void_p(grad_out.data_ptr()),
                  ctypes.c_void_p(grad_src.data_ptr() if grad_src is not None else 0),
                  ctypes.c_void_p(grad_theta_dev.data_ptr() if grad_theta_dev is not None else 0),
                  ctypes.c_void_p(stream))
        grad_theta = None
        if grad_theta_dev is not None:
            device, dtype = ctx.theta_meta
            grad_theta = grad_theta_dev.to(device=device, dtype=dtype)
        return grad_src, grad_theta, None, None, None


def warp_affine(src: torch.Tensor, theta: torch.Tensor, interpolation: str | int = "lanczos3",
                fill: float = float("nan"), src_all_finite: bool = False) -> torch.Tensor:
    """Differentiable warp of ``src`` by the inverse affine parameters ``theta``."""
    return AffineWarp.apply(src, theta, _interp_code(interpolation), fill, src_all_finite)


def theta_from_matrix(matrix) -> np.ndarray:
    """Inverse-map parameters of an affine moving -> reference matrix."""
    m = np.asarray(matrix, dtype=np.float64).reshape(3, 3)
    if not np.allclose(m[2], (0.0, 0.0, 1.0), rtol=0.0, atol=1e-12):
        raise ValueError("matrix must be affine (last row 0, 0, 1)")
    inv = np.linalg.inv(m)
    return np.array([inv[0, 0], inv[0, 1], inv[0, 2], inv[1, 0], inv[1, 1], inv[1, 2]], dtype=np.float64)


def matrix_from_theta(theta) -> np.ndarray:
    t = np.asarray(theta, dtype=np.float64).reshape(6)
    inv = np.array([[t[0], t[1], t[2]], [t[3], t[4], t[5]], [0.0, 0.0, 1.0]])
    m = np.linalg.inv(inv)
    m[2] = (0.0, 0.0, 1.0)
    return m


def _basis(model: str, height: int, width: int) -> np.ndarray:
    """Columns map unit steps of the free parameters to theta changes of about
    one pixel at the image edge, about the image centre."""
    cx, cy, r = (width - 1) / 2.0, (height - 1) / 2.0, max(height, width) / 2.0
    lin = lambda a, b, c, d: np.array([a / r, b / r, -(a * cx + b * cy) / r, c / r, d / r, -(c * cx + d * cy) / r])
    shift_x = np.array([0.0, 0.0, 1.0, 0.0, 0.0, 0.0])
    shift_y = np.array([0.0, 0.0, 0.0, 0.0, 0.0, 1.0])
    if model == "translation":
        cols = [shift_x, shift_y]
    elif model == "similarity":
        cols = [shift_x, shift_y, lin(1, 0, 0, 1), lin(0, -1, 1, 0)]
    elif model == "affine":
        cols = [shift_x, shift_y, lin(1, 0, 0, 0), lin(0, 1, 0, 0), lin(0, 0, 1, 0), lin(0, 0, 0, 1)]
    else:
        raise ValueError("model must be translation, similarity or affine")
    return np.stack(cols, axis=1)


@dataclass
class RefineConfig:
    model: str = "similarity"
    # "ssd": photometrically matched sum of squares (default); "ncc": 1 - NCC,
    # whose normalisation by the warped frame's variance favours positions
    # where interpolation smooths the noise (half-pixel shifts)
    loss: str = "ssd"
    interpolation: str = "lanczos3"
    rounds: int = 2  # mask re-estimations
    iterations: int = 6  # trust-region Newton steps per round
    max_step_px: float = 0.5  # trust radius (parameter units: about 1 px at the image edge)
    tolerance_px: float = 1.0e-3
    clip_sigma: float = 5.0
    mask_shift_px: float = 1.0
    border_px: int = 4


@dataclass
class RefineOutcome:
    matrix: np.ndarray
    theta: np.ndarray
    ncc_before: float
    ncc_after: float
    masked_fraction: float
    evaluations: int
    history: list[float] = field(default_factory=list)


def _gradient_mag(img: torch.Tensor) -> torch.Tensor:
    """Largest absolute central difference along x and y (0 on the border)."""
    g = torch.zeros_like(img)
    gx = (img[1:-1, 2:] - img[1:-1, :-2]).abs() * 0.5
    gy = (img[2:, 1:-1] - img[:-2, 1:-1]).abs() * 0.5
    g[1:-1, 1:-1] = torch.maximum(gx, gy)
    return g


def _outlier_mask(ref: torch.Tensor, warped: torch.Tensor, valid: torch.Tensor, cfg: RefineConfig):
    """(mask, alpha, beta, sigma): valid pixels that are not single-frame outliers."""
    a = ref[valid].double()
    b = warped[valid].double()
    if a.numel() < 16:
        raise ValueError("too few overlapping pixels to refine")
    am, bm = a.mean(), b.mean()
    var_a = ((a - am) ** 2).mean()
    alpha = (((a - am) * (b - bm)).mean() / var_a) if var_a > 0 else torch.zeros((), dtype=torch.float64,
                                                                                        device=a.device)
    beta = bm - alpha * am
    r = b - (alpha * a + beta)
    med = r.median()
    sigma = 1.4826 * (r - med).abs().median()
    sigma = torch.clamp(sigma, min=1e-12)
    # misregistration allowance from the smoother of the two frames
    ga = _gradient_mag(torch.where(valid, ref, torch.zeros_like(ref)))[valid].double() * alpha.abs()
    gb = _gradient_mag(torch.where(valid, warped, torch.zeros_like(warped)))[valid].double()
    allow = cfg.clip_sigma * sigma + cfg.mask_shift_px * torch.minimum(ga, gb)
    # structure the reference lacks (cosmic-ray interpolation ringing) fails
    # the gradient-consistency test
    keep = ((r - med).abs() <= allow) & (gb <= 2.0 * ga + 3.0 * sigma)
    mask = torch.zeros_like(valid)
    mask[valid] = keep
    return mask, float(alpha), float(beta), float(sigma)


def _matched_ssd(a: torch.Tensor, b: torch.Tensor, m: torch.Tensor) -> torch.Tensor:
    """Mean of (b - alpha a - beta)^2 over the mask with (alpha, beta) the
    least-squares photometric match, computed in the graph (the gradient of
    the minimum is the partial gradient at the minimiser)."""
    n = m.sum()
    am = (a * m).sum() / n
    bm = (b * m).sum() / n
    da, db = (a - am) * m, (b - bm) * m
    alpha = (da * db).sum() / (da * da).sum()
    r = db - alpha * da
    return (r * r).sum() / n


def _masked_ncc(a: torch.Tensor, b: torch.Tensor, m: torch.Tensor) -> torch.Tensor:
    n = m.sum()
    am = (a * m).sum() / n
    bm = (b * m).sum() / n
    da, db = (a - am) * m, (b - bm) * m
    return (da * db).sum() / torch.sqrt((da * da).sum() * (db * db).sum())


def refine_affine(reference: torch.Tensor, moving: torch.Tensor, matrix, config: RefineConfig | None = None,
                  ) -> RefineOutcome:
    """Gradient refinement of ``matrix`` (moving -> reference) on two device frames."""
    cfg = config or RefineConfig()
    _check_image(reference)
    _check_image(moving)
    if reference.shape != moving.shape:
        raise ValueError("reference and moving frames must have the same shape")
    if cfg.loss not in ("ncc", "ssd"):
        raise ValueError("loss must be ncc or ssd")
    interp = _interp_code(cfg.interpolation)
    h, w = reference.shape
    theta0 = torch.from_numpy(theta_from_matrix(matrix))
    basis = torch.from_numpy(_basis(cfg.model, h, w))
    u = torch.zeros(basis.shape[1], dtype=torch.float64, requires_grad=True)
    moving_finite = bool(torch.isfinite(moving).all())
    ref_finite = torch.isfinite(reference)
    inner = torch.zeros_like(ref_finite)
    bp = max(0, int(cfg.border_px))
    inner[bp:h - bp, bp:w - bp] = True
    ref0 = torch.where(ref_finite, reference, torch.zeros_like(reference)).double()
    evaluations = 0
    history: list[float] = []

    def theta_of(uu):
        return theta0 + basis @ uu

    def current_mask(theta):
        with torch.no_grad():
            warped = AffineWarp.apply(moving, theta, interp, float("nan"), moving_finite)
            valid = ref_finite & torch.isfinite(warped) & inner
            return (valid, *_outlier_mask(reference, warped, valid, cfg))

    with torch.no_grad():
        valid0, mask0, _, _, _ = current_mask(theta0)
        w0 = AffineWarp.apply(moving, theta0, interp, float("nan"), moving_finite)
        ncc_before = float(_masked_ncc(ref0, torch.where(mask0, w0, torch.zeros_like(w0)).double(),
                                       mask0.double()))
    valid, mask = valid0, mask0
    for _ in range(max(1, cfg.rounds)):
        with torch.no_grad():
            valid, mask, alpha, beta, sigma = current_mask(theta_of(u.detach()))
        mf = mask.double()

        def loss_at(uu, grad: bool):
            nonlocal evaluations
            p = uu.detach().clone().requires_grad_(grad)
            warped = AffineWarp.apply(moving, theta_of(p), interp, float("nan"), moving_finite)
            b = torch.where(mask, warped, torch.zeros_like(warped)).double()
            if cfg.loss == "ncc":
                loss = 1.0 - _masked_ncc(ref0, b, mf)
            else:
                loss = _matched_ssd(ref0, b, mf) / (sigma * sigma)
            evaluations += 1
            history.append(float(loss.detach()))
            if not grad:
                return float(loss.detach()), None
            loss.backward()
            return float(loss.detach()), p.grad.detach().clone()

        # trust-region Newton: autograd gradients, the Hessian from forward
        # differences of the gradient (steps of 0.01 px), Levenberg damping,
        # steps capped to the trust radius (parameter units ~ px at the edge)
        radius = cfg.max_step_px
        k = u.numel()
        f0, g0 = loss_at(u, True)
        for _ in range(max(1, cfg.iterations)):
            eps = 1.0e-2
            hess = torch.empty((k, k), dtype=torch.float64)
            for i in range(k):
                e = torch.zeros_like(u)
                e[i] = eps
                _, gi = loss_at(u.detach() + e, True)
                hess[:, i] = (gi - g0) / eps
            hess = 0.5 * (hess + hess.T)
            lam = 0.0
            evals = torch.linalg.eigvalsh(hess)
            if float(evals.min()) <= 0.0:
                lam = 1.0e-6 * float(evals.abs().max()) - float(evals.min())
            step = -torch.linalg.solve(hess + lam * torch.eye(k, dtype=torch.float64), g0)
            big = float(step.abs().max())
            if big > radius:
                step = step * (radius / big)
            f1, g1 = loss_at(u.detach() + step, True)
            if f1 < f0:
                with torch.no_grad():
                    u += step
                f0, g0 = f1, g1
                radius = min(2.0 * radius, cfg.max_step_px)
                if float(step.abs().max()) < cfg.tolerance_px:
                    break
            else:
                radius *= 0.25
                if radius < cfg.tolerance_px:
                    break
    theta = theta_of(u.detach()).numpy()
    with torch.no_grad():
        wf = AffineWarp.apply(moving, torch.from_numpy(theta), interp, float("nan"), moving_finite)
        ncc_after = float(_masked_ncc(ref0, torch.where(mask, wf, torch.zeros_like(wf)).double(), mask.double()))
    masked_fraction = 1.0 - float(mask.sum()) / max(1, int(valid.sum()))
    return RefineOutcome(matrix_from_theta(theta), theta, ncc_before, ncc_after, masked_fraction, evaluations,
                         history)


@dataclass
class LbfgsConfig:
    """Gradient refinement on the masked NCC of star regions by L-BFGS."""
    model: str = "affine"
    interpolation: str = "lanczos3"
    iterations: int = 20  # loss / gradient evaluations (forward + adjoint), at most
    star_sigma: float = 5.0  # reference pixels above median + star_sigma * 1.4826 MAD are star pixels
    star_radius_px: int = 3  # dilation of the star pixels
    border_px: int = 6
    history: int = 10


def star_region_mask(reference: torch.Tensor, star_sigma: float = 5.0, radius_px: int = 3,
                     border_px: int = 6) -> torch.Tensor:
    """Pixels within `radius_px` of a reference pixel brighter than the median
    plus `star_sigma` robust sigmas (1.4826 MAD), away from the border: the
    loss is taken where the frames carry structure, so that the smoothing of
    the moving frame's noise by the interpolation (smallest at half-pixel
    offsets) cannot pull the optimum off the registration."""
    finite = torch.isfinite(reference)
    vals = reference[finite]
    if vals.numel() == 0:
        raise ValueError("reference frame has no finite pixels")
    med = vals.median()
    mad = (vals - med).abs().median() * 1.4826
    star = (torch.where(finite, reference, med) > med + star_sigma * mad).float()[None, None]
    r = max(0, int(radius_px))
    mask = torch.nn.functional.max_pool2d(star, 2 * r + 1, 1, r)[0, 0] > 0 if r else star[0, 0] > 0
    b = max(0, int(border_px))
    if b:
        mask[:b] = False
        mask[-b:] = False
        mask[:, :b] = False
        mask[:, -b:] = False
    return mask & finite


def refine_affine_lbfgs(reference: torch.Tensor, moving: torch.Tensor, matrix, config: LbfgsConfig | None = None,
                        mask: torch.Tensor | None = None, warp_fn=None) -> RefineOutcome:
    """Refines ``matrix`` (moving -> reference) by L-BFGS (strong Wolfe line
    search) on 1 - NCC over the reference's star regions, every loss gradient
    coming from the hand-written warp adjoint through ``AffineWarp``.  The
    free parameters are the basis coordinates of ``_basis(model)`` (about one
    pixel of motion at the image edge per unit).  ``warp_fn(src, theta)``
    replaces the device warp (tests run the float64 PyTorch restatement)."""
    cfg = config or LbfgsConfig()
    if reference.shape != moving.shape:
        raise ValueError("reference and moving frames must have the same shape")
    h, w = reference.shape
    if warp_fn is None:
        _check_image(reference)
        _check_image(moving)
        interp = _interp_code(cfg.interpolation)
        moving_finite = bool(torch.isfinite(moving).all())

        def warp_fn(src, theta):
            return AffineWarp.apply(src, theta, interp, float("nan"), moving_finite)
    if mask is None:
        mask = star_region_mask(reference, cfg.star_sigma, cfg.star_radius_px, cfg.border_px)
    if int(mask.sum()) < 16:
        raise ValueError("too few star pixels to refine")
    theta0 = torch.from_numpy(theta_from_matrix(matrix))
    basis = torch.from_numpy(_basis(cfg.model, h, w))
    # the loss reads only the star pixels: gathered once from the reference,
    # and from each warped frame (whose gradient scatters back to them)
    star_idx = mask.reshape(-1).nonzero().squeeze(1)
    ref_stars = reference.reshape(-1)[star_idx].double()
    u = torch.zeros(basis.shape[1], dtype=torch.float64, requires_grad=True)
    history: list[float] = []

    def loss_of(uu):
        warped = warp_fn(moving, theta0 + basis @ uu).reshape(-1)[star_idx]
        m = torch.isfinite(warped)
        md = m.double()
        n = md.sum()
        a = ref_stars * md
        b = torch.where(m, warped, torch.zeros_like(warped)).double()
        am, bm = a.sum() / n, b.sum() / n
        da, db = (a - am) * md, (b - bm) * md
        return 1.0 - (da * db).sum() / torch.sqrt((da * da).sum() * (db * db).sum())

    with torch.no_grad():
        ncc_before = 1.0 - float(loss_of(u))
    opt = torch.optim.LBFGS([u], lr=1.0, max_iter=max(1, cfg.iterations), max_eval=max(1, cfg.iterations),
                            history_size=cfg.history, tolerance_grad=1e-12, tolerance_change=1e-15,
                            line_search_fn="strong_wolfe")

    def closure():
        opt.zero_grad()
        loss = loss_of(u)
        loss.backward()
        history.append(float(loss.detach()))
        return loss

    opt.step(closure)
    # L-BFGS may end on a line-search trial: keep the best point seen
    theta = (theta0 + basis @ u.detach()).numpy()
    with torch.no_grad():
        ncc_after = 1.0 - float(loss_of(u.detach()))
    if ncc_after < ncc_before:
        theta, ncc_after = theta0.numpy(), ncc_before
    return RefineOutcome(matrix_from_theta(theta), theta, ncc_before, ncc_after,
                         1.0 - float(mask.double().mean()), len(history), history)


def registration_rms_px(estimated, truth, height: int, width: int, grid: int = 16) -> float | None:
    """RMS over a grid of reference pixels of the distance between the source
    positions that two moving -> reference matrices sample (None for no
    matrices)."""
    if len(estimated) == 0:
        return None
    ys, xs = np.meshgrid(np.linspace(0, height - 1, grid), np.linspace(0, width - 1, grid), indexing="ij")
    pts = np.stack([xs.ravel(), ys.ravel(), np.ones(xs.size)])
    sq = []
    for est, tru in zip(estimated, truth):
        pe = np.linalg.inv(np.asarray(est, dtype=np.float64)) @ pts
        pt = np.linalg.inv(np.asarray(tru, dtype=np.float64)) @ pts
        pe = pe[:2] / pe[2]
        pt = pt[:2] / pt[2]
        sq.append(((pe - pt) ** 2).sum(axis=0))
    return float(np.sqrt(np.mean(np.concatenate(sq))))
