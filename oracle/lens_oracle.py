"""PyTorch-CPU restatement of the GIGA-Lens forward model and likelihood.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Every function states
the reference file:line it restates.  Arithmetic follows the reference's op
order; the precision is chosen by the dtype of the inputs (float64 = the error
reference "same method in FP64", float32 = the reference's own float32 CPU
arithmetic, used as the timed CPU baseline).

Layout: parameters are tensors of shape ``(bs,)``; images are ``(bs, H, W)``
(the reference keeps the batch axis last on its coordinate grids,
``tf/simulator.py:33-38``; the arithmetic per element is identical).
"""
import math
from typing import Dict, List, Sequence, Tuple

import numpy as np
import torch
import torch.nn.functional as Fnn

LOG_2PI = math.log(2.0 * math.pi)


# --------------------------------------------------------------------------
# coordinate grid
# --------------------------------------------------------------------------
def get_coords(supersample: int, num_pix: int, transform_pix2angle) -> Tuple[float, float, np.ndarray, np.ndarray]:
    """Zero-mean supersampled pixel grid, ``gigalens/simulator.py:91-125``.

    ``transform_pix2angle`` is the *fine* pixel-to-angle matrix, which the
    reference holds as a float32 tensor already divided by the supersampling
    factor (``tf/simulator.py:27-32``).  ``lo = min(arange(S) - mean)`` and the
    origin ``T @ [lo, lo]`` are float32; the grid itself is evaluated in
    float64 (lenstronomy ``PixelGrid``: x = T00*col + T01*row + x0,
    y = T10*col + T11*row + y0) and rounded to float32.
    """
    S = supersample * num_pix
    T = np.asarray(transform_pix2angle, dtype=np.float32)
    lo = np.arange(0, S, dtype=np.float32)
    lo = np.float32(np.min(lo - np.mean(lo)))
    ra0, dec0 = (T @ np.array([lo, lo], dtype=np.float32)).astype(np.float32)
    Td = T.astype(np.float64)
    cols, rows = np.meshgrid(np.arange(S, dtype=np.float64), np.arange(S, dtype=np.float64))
    x = Td[0, 0] * cols + Td[0, 1] * rows + np.float64(ra0)
    y = Td[1, 0] * cols + Td[1, 1] * rows + np.float64(dec0)
    return float(ra0), float(dec0), x.astype(np.float32), y.astype(np.float32)


# --------------------------------------------------------------------------
# mass profiles
# --------------------------------------------------------------------------
def _t(v, like):
    return torch.as_tensor(v, dtype=like.dtype, device=like.device)


def epl_term_count(e1, e2, niter_cap: int) -> int:
    """Number of EPL series iterations the reference executes.

    ``tf/profiles/mass/epl.py:41,51-56``: ``niter = log(1e-12)/log(max_b f) + 2``
    evaluated in float32 over the whole batch; the loop counter starts at 1 and
    runs while ``i < niter``, at most ``niter_cap`` times.
    """
    e1 = torch.as_tensor(e1).detach().to(torch.float32).reshape(-1)
    e2 = torch.as_tensor(e2).detach().to(torch.float32).reshape(-1)
    c = torch.clamp(torch.sqrt(e1 ** 2 + e2 ** 2), 0, 1)
    q = (1 - c) / (1 + c)
    f = (1 - q) / (1 + q)
    niter = float(torch.log(torch.tensor(1e-12, dtype=torch.float32)) / torch.log(torch.max(f)) + 2)
    k = 0
    i = 1.0
    while k < niter_cap and i < niter:   # NaN compares false -> 0 iterations
        k += 1
        i += 1.0
    return k


def epl_deriv(x, y, theta_E, gamma, e1, e2, center_x, center_y, n_terms: int):
    """EPL deflection by the iterative series, ``tf/profiles/mass/epl.py:23-68``."""
    phi = torch.atan2(e2, e1) / 2
    c = torch.clamp(torch.sqrt(e1 ** 2 + e2 ** 2), 0, 1)
    q = (1 - c) / (1 + c)
    theta_E_conv = theta_E / torch.sqrt((1.0 + q ** 2) / (2.0 * q))
    b = theta_E_conv * torch.sqrt((1 + q ** 2) / 2)
    t = gamma - 1
    x, y = x - center_x, y - center_y
    x, y = _rotate(x, y, phi)
    R = torch.clamp(torch.sqrt((q * x) ** 2 + y ** 2), 1e-10, 1e10)
    angle = torch.atan2(y, q * x)
    f = (1 - q) / (1 + q)
    Cs, Ss = torch.cos(angle), torch.sin(angle)
    Cs2, Ss2 = torch.cos(2 * angle), torch.sin(2 * angle)
    last_x, last_y, fx, fy = Cs, Ss, Cs, Ss
    n = 1.0
    for _ in range(n_terms):
        prefac = -f * (2 * n - (2 - t)) / (2 * n + (2 - t))
        last_x, last_y = prefac * (Cs2 * last_x - Ss2 * last_y), prefac * (Ss2 * last_x + Cs2 * last_y)
        fx, fy = fx + last_x, fy + last_y
        n += 1.0
    prefac = (2 * b) / (1 + q) * torch.pow(b / R, t - 1)
    fx, fy = fx * prefac, fy * prefac
    return _rotate(fx, fy, -phi)


def _rotate(x, y, phi):
    """``tf/profiles/mass/epl.py:63-68``."""
    cos_phi, sin_phi = torch.cos(phi), torch.sin(phi)
    return x * cos_phi + y * sin_phi, -x * sin_phi + y * cos_phi


def shear_deriv(x, y, gamma1, gamma2):
    """``tf/profiles/mass/shear.py:12-14``."""
    return gamma1 * x + gamma2 * y, gamma2 * x - gamma1 * y


def sis_deriv(x, y, theta_E, center_x, center_y):
    """``tf/profiles/mass/sis.py:13-18``."""
    dx, dy = x - center_x, y - center_y
    R = torch.sqrt(dx ** 2 + dy ** 2)
    a = torch.where(R == 0, torch.zeros_like(R), theta_E / R)
    return a * dx, a * dy


def sie_deriv(x, y, theta_E, e1, e2, center_x, center_y):
    """``tf/profiles/mass/sie.py:14-43`` (s_scale = 0 as in the reference)."""
    phi = torch.atan2(e2, e1) / 2
    c = torch.clamp(torch.sqrt(e1 ** 2 + e2 ** 2), max=0.9999)
    q = (1 - c) / (1 + c)
    theta_E_conv = theta_E / torch.sqrt((1.0 + q ** 2) / (2.0 * q))
    b = theta_E_conv * torch.sqrt((1 + q ** 2) / 2)
    s = 0.0 * torch.sqrt((1 + q ** 2) / (2 * q ** 2))
    x, y = x - center_x, y - center_y
    x, y = _rotate(x, y, phi)
    psi = torch.sqrt(q ** 2 * (s ** 2 + x ** 2) + y ** 2)
    sq = torch.sqrt(1.0 - q ** 2)
    fx = b / sq * torch.atan(sq * x / (psi + s))
    fy = b / sq * torch.atanh(sq * y / (psi + q ** 2 * s))
    return _rotate(fx, fy, -phi)


def tnfw_F(x):
    """NFW F(x), ``tf/profiles/mass/tnfw.py:40-58``: atanh branch below 1, atan
    branch above, exactly 1 at x == 1 (each branch evaluated only where taken,
    as the reference's gather/scatter does)."""
    lo, hi = x < 1, x > 1
    x_lo = torch.where(lo, x, torch.full_like(x, 0.5))
    x_hi = torch.where(hi, x, torch.full_like(x, 2.0))
    s_lo = torch.sqrt(1 - x_lo ** 2)
    s_hi = torch.sqrt(x_hi ** 2 - 1)
    return torch.where(lo, torch.atanh(s_lo) / s_lo, torch.where(hi, torch.atan(s_hi) / s_hi, torch.ones_like(x)))


def tnfw_deriv(x, y, Rs, alpha_Rs, r_trunc, center_x, center_y):
    """``tf/profiles/mass/tnfw.py:14-38``."""
    rho0 = alpha_Rs / (4.0 * Rs ** 2 * (1.0 + math.log(0.5)))
    dx, dy = x - center_x, y - center_y
    R = torch.sqrt(dx ** 2 + dy ** 2)
    R = torch.maximum(R, 0.001 * Rs)
    X = R / Rs
    tau = r_trunc / Rs
    L = torch.log(X / (tau + torch.sqrt(tau ** 2 + X ** 2)))
    F = tnfw_F(X)
    gx = (tau ** 2 / (tau ** 2 + 1) ** 2
          * ((tau ** 2 + 1 + 2 * (X ** 2 - 1)) * F + tau * math.pi + (tau ** 2 - 1) * torch.log(tau)
             + torch.sqrt(tau ** 2 + X ** 2) * (-math.pi + L * (tau ** 2 - 1) / tau)))
    a = 4 * rho0 * Rs * gx / X ** 2
    return a * dx, a * dy


# --------------------------------------------------------------------------
# light profiles
# --------------------------------------------------------------------------
def sersic_distance(x, y, cx, cy, e1=None, e2=None):
    """``tf/profiles/light/sersic.py:33-59``."""
    if e1 is None:
        e1 = torch.zeros_like(cx)
    if e2 is None:
        e2 = torch.zeros_like(cx)
    phi = torch.atan2(e2, e1) / 2
    c = torch.sqrt(e1 ** 2 + e2 ** 2)
    q = (1 - c) / (1 + c)
    dx, dy = x - cx, y - cy
    cos_phi, sin_phi = torch.cos(phi), torch.sin(phi)
    xt1 = (cos_phi * dx + sin_phi * dy) * torch.sqrt(q)
    xt2 = (-sin_phi * dx + cos_phi * dy) / torch.sqrt(q)
    return torch.sqrt(xt1 ** 2 + xt2 ** 2)


def sersic_ellipse_light(x, y, R_sersic, n_sersic, e1, e2, center_x, center_y, Ie):
    """``tf/profiles/light/sersic.py:66-72``; pass ``Ie=1`` for the lstsq basis."""
    R = sersic_distance(x, y, center_x, center_y, e1, e2)
    bn = 1.9992 * n_sersic - 0.3271
    return Ie * torch.exp(-bn * ((R / R_sersic) ** (1 / n_sersic) - 1.0))


def sersic_light(x, y, R_sersic, n_sersic, center_x, center_y, Ie):
    """Spherical Sersic, ``tf/profiles/light/sersic.py:25-31``."""
    R = sersic_distance(x, y, center_x, center_y)
    bn = 1.9992 * n_sersic - 0.3271
    return Ie * torch.exp(-bn * ((R / R_sersic) ** (1 / n_sersic) - 1.0))


def core_sersic_light(x, y, R_sersic, n_sersic, Rb, alpha, gamma, e1, e2, center_x, center_y, Ie):
    """``tf/profiles/light/sersic.py:88-121`` as written, quirks included: the
    ``- 1.0`` sits inside the exponential but outside the ``-bn * (...)``
    product, the scaled radius is divided by ``alpha * n`` instead of raised to
    ``1/(alpha n)``, and ``R_sersic ** alpha ** 1.0`` is ``R_sersic ** alpha``."""
    R = sersic_distance(x, y, center_x, center_y, e1, e2)
    bn = 1.9992 * n_sersic - 0.3271
    return (Ie * (1 + (Rb / R) ** alpha) ** (gamma / alpha)
            * torch.exp(-bn * ((R ** alpha + Rb ** alpha) / R_sersic ** alpha ** 1.0 / (alpha * n_sersic)) - 1.0))


def shapelet_orders(n_max: int) -> Tuple[List[int], List[int]]:
    """(n1, n2) order of the basis, ``tf/profiles/light/shapelets.py:26-46``."""
    n_layers = (n_max + 1) * (n_max + 2) // 2
    N1, N2 = [], []
    n1 = n2 = 0
    for _ in range(n_layers):
        N1.append(n1)
        N2.append(n2)
        if n1 == 0:
            n1 = n2 + 1
            n2 = 0
        else:
            n1 -= 1
            n2 += 1
    return N1, N2


def shapelet_phi_n(u, n_max: int):
    """Normalised Hermite functions without the Gaussian,
    ``tf/profiles/light/shapelets.py:47-48,77-85``: ``H_n(u) / sqrt(2^n sqrt(pi) n!)``."""
    H = [torch.ones_like(u), 2 * u]
    for i in range(2, n_max + 1):
        H.append(2 * (u * H[-1] - (i - 1) * H[-2]))
    out = []
    for n in range(n_max + 1):
        pref = 1.0 / math.sqrt(2 ** n * math.sqrt(math.pi) * math.exp(math.lgamma(n + 1)))
        out.append(H[n] * pref)
    return out


SHAPELET_TABLE_N = 6000
SHAPELET_TABLE_LO, SHAPELET_TABLE_HI = -5.0, 5.0


def shapelet_table(n_max: int) -> np.ndarray:
    """The reference's tabulated 1-D shapelet functions
    (``tf/profiles/light/shapelets.py:37-38``: lenstronomy's
    ``phi_n(n, linspace(-5, 5, 6000))`` stored as float32).  lenstronomy is
    not installed; its ``phi_n`` is the published 1-D shapelet function
    ``H_n(t) exp(-t^2/2) / sqrt(2^n sqrt(pi) n!)`` (Refregier 2003), evaluated
    here in float64 from the Hermite recursion and rounded to float32."""
    t = np.linspace(SHAPELET_TABLE_LO, SHAPELET_TABLE_HI, SHAPELET_TABLE_N)
    H = [np.ones_like(t), 2 * t]
    for i in range(2, n_max + 1):
        H.append(2 * (t * H[-1] - (i - 1) * H[-2]))
    rows = [H[n] * np.exp(-t ** 2 / 2) / math.sqrt(2 ** n * math.sqrt(math.pi) * math.factorial(n))
            for n in range(n_max + 1)]
    return np.asarray(rows).astype(np.float32)


def interp_regular_1d(x, table_row):
    """``tfp.math.interp_regular_1d_grid(x, -5, 5, row, fill_value_below=0,
    fill_value_above=0)`` (``tf/profiles/light/shapelets.py:57-60``): the
    fractional index ``(x - lo) / (hi - lo) (N - 1)`` clipped to the grid, the
    bracket below it (the last bracket for the top point), ``w y1 + (1 - w) y0``;
    0 outside [lo, hi], NaN for NaN x.  Differentiable in x (the bracket's
    slope), as TensorFlow's gradient of that interpolation."""
    y = torch.as_tensor(table_row, dtype=x.dtype)
    n = y.numel()
    fi = (x - SHAPELET_TABLE_LO) / (SHAPELET_TABLE_HI - SHAPELET_TABLE_LO) * (n - 1)
    fi = torch.nan_to_num(fi, nan=0.0).clamp(0, n - 1)
    ib = torch.floor(fi.detach())
    ia = torch.clamp(ib + 1, max=n - 1)
    ib = torch.clamp(ia - 1, min=0)
    w = fi - ib
    out = w * y[ia.long()] + (1 - w) * y[ib.long()]
    out = torch.where((x < SHAPELET_TABLE_LO) | (x > SHAPELET_TABLE_HI), torch.zeros_like(out), out)
    return torch.where(torch.isnan(x), x, out)


def shapelets_basis(x, y, center_x, center_y, beta, n_max: int, interpolate: bool = False):
    """Unit-amplitude basis stack ``(D, ...)``, ``tf/profiles/light/shapelets.py:53-72``;
    ``interpolate``: products of the tabulated 1-D functions."""
    u = (x - center_x) / beta
    v = (y - center_y) / beta
    N1, N2 = shapelet_orders(n_max)
    if interpolate:
        tab = shapelet_table(n_max)
        TU = [interp_regular_1d(u, tab[n]) for n in range(n_max + 1)]
        TV = [interp_regular_1d(v, tab[n]) for n in range(n_max + 1)]
        return torch.stack([TU[a] * TV[b] for a, b in zip(N1, N2)], dim=0)
    XX, YY = shapelet_phi_n(u, n_max), shapelet_phi_n(v, n_max)
    fac = torch.exp(-(u ** 2 + v ** 2) / 2)
    return torch.stack([fac * XX[a] * YY[b] for a, b in zip(N1, N2)], dim=0)


def shapelets_light(x, y, center_x, center_y, beta, amps: Sequence, n_max: int, interpolate: bool = False):
    """Amplitude-weighted sum, ``tf/profiles/light/shapelets.py:61-64,73-75``."""
    basis = shapelets_basis(x, y, center_x, center_y, beta, n_max, interpolate)
    out = torch.zeros_like(basis[0])
    for k, a in enumerate(amps):
        out = out + a * basis[k]
    return out


# --------------------------------------------------------------------------
# model spec: a tiny description of a PhysicalModel for the oracle
# --------------------------------------------------------------------------
# A model is dict(lenses=[(type, kwargs)], lens_light=[...], source_light=[...])
# with type in {"EPL", "SHEAR", "SIS", "SIE", "SERSIC", "SERSIC_ELLIPSE",
# "SHAPELETS"}; kwargs hold constructor arguments (niter, n_max).

def _mass(kind, opts, x, y, p, n_terms):
    if kind == "EPL":
        return epl_deriv(x, y, p["theta_E"], p["gamma"], p["e1"], p["e2"], p["center_x"], p["center_y"], n_terms)
    if kind == "SHEAR":
        return shear_deriv(x, y, p["gamma1"], p["gamma2"])
    if kind == "SIS":
        return sis_deriv(x, y, p["theta_E"], p["center_x"], p["center_y"])
    if kind == "SIE":
        return sie_deriv(x, y, p["theta_E"], p["e1"], p["e2"], p["center_x"], p["center_y"])
    if kind == "TNFW":
        return tnfw_deriv(x, y, p["Rs"], p["alpha_Rs"], p["r_trunc"], p["center_x"], p["center_y"])
    raise ValueError(kind)


def _light(kind, opts, x, y, p, lstsq=False):
    if kind == "SERSIC_ELLIPSE":
        Ie = torch.ones_like(p["R_sersic"]) if lstsq else p["Ie"]
        out = sersic_ellipse_light(x, y, p["R_sersic"], p["n_sersic"], p["e1"], p["e2"], p["center_x"], p["center_y"], Ie)
        return out[None] if lstsq else out
    if kind == "SERSIC":
        Ie = torch.ones_like(p["R_sersic"]) if lstsq else p["Ie"]
        out = sersic_light(x, y, p["R_sersic"], p["n_sersic"], p["center_x"], p["center_y"], Ie)
        return out[None] if lstsq else out
    if kind == "CORE_SERSIC":
        Ie = torch.ones_like(p["R_sersic"]) if lstsq else p["Ie"]
        out = core_sersic_light(x, y, p["R_sersic"], p["n_sersic"], p["Rb"], p["alpha"], p["gamma"], p["e1"],
                                p["e2"], p["center_x"], p["center_y"], Ie)
        return out[None] if lstsq else out
    if kind == "SHAPELETS":
        n_max = opts["n_max"]
        interp = bool(opts.get("interpolate", False))
        if lstsq:
            return shapelets_basis(x, y, p["center_x"], p["center_y"], p["beta"], n_max, interp)
        D = (n_max + 1) * (n_max + 2) // 2
        width = len(str(D))
        amps = [p[f"amp{str(i).zfill(width)}"] for i in range(D)]
        return shapelets_light(x, y, p["center_x"], p["center_y"], p["beta"], amps, n_max, interp)
    raise ValueError(kind)


def _expand(p: Dict, dtype):
    return {k: torch.as_tensor(v, dtype=dtype).reshape(-1, 1, 1) for k, v in p.items()}


def epl_terms_for(model, lens_params):
    """Term count per EPL lens for one batch (``tf/profiles/mass/epl.py:41``)."""
    out = []
    for (kind, opts), p in zip(model["lenses"], lens_params):
        if kind == "EPL":
            out.append(epl_term_count(p["e1"], p["e2"], opts.get("niter", 50)))
        else:
            out.append(0)
    return out


def beta(model, lens_params, x, y, dtype):
    """Ray shooting, ``tf/simulator.py:57-63``."""
    terms = epl_terms_for(model, lens_params)
    bx, by = x, y
    for (kind, opts), p, k in zip(model["lenses"], lens_params, terms):
        fx, fy = _mass(kind, opts, x, y, _expand(p, dtype), k)
        bx, by = bx - fx, by - fy
    return bx, by


class SimConfig:
    """Camera settings: ``SimulatorConfig`` (``gigalens/simulator.py:11-28``) with
    the PSF given already supersampled (the output of the reference's
    ``subgrid_kernel``, unflipped)."""

    def __init__(self, delta_pix, num_pix, supersample=1, kernel_sub=None, transform_pix2angle=None):
        self.delta_pix = float(delta_pix)
        self.num_pix = int(num_pix)
        self.supersample = int(supersample)
        self.kernel_sub = None if kernel_sub is None else np.asarray(kernel_sub, dtype=np.float64)
        # tf/simulator.py:19-29: float32 transform, det before the division by ss
        T = (np.eye(2, dtype=np.float32) * np.float32(delta_pix) if transform_pix2angle is None
             else np.asarray(transform_pix2angle, np.float32))
        self.T = T
        Td = T.astype(np.float64)
        self.conversion_factor = float(np.float32(Td[0, 0] * Td[1, 1] - Td[0, 1] * Td[1, 0]))
        _, _, self.img_x, self.img_y = get_coords(self.supersample, self.num_pix,
                                                  T / np.float32(self.supersample))


def _split(model, params):
    """``tf/simulator.py:67-72``."""
    if len(model["lens_light"]) > 0:
        return params[0], params[1], params[2]
    return params[0], [], params[1]


def _psf_pool(img, cfg: SimConfig, dtype):
    """PSF (true convolution, zero 'SAME' padding) then average pooling,
    ``tf/simulator.py:82-96``.  ``img`` is ``(B, C, S, S)``."""
    if cfg.kernel_sub is not None:
        k = cfg.kernel_sub.shape[0]
        flat = torch.as_tensor(cfg.kernel_sub[::-1, ::-1].copy(), dtype=dtype)
        C = img.shape[1]
        w = flat[None, None].repeat(C, 1, 1, 1)
        img = Fnn.conv2d(img, w, padding=(k - 1) // 2, groups=C)
    if cfg.supersample != 1:
        img = Fnn.avg_pool2d(img, cfg.supersample)
    return img


def simulate(model, cfg: SimConfig, params, dtype=torch.float64, no_deflection=False, ray_dtype=None):
    """``LensSimulator.simulate``, ``tf/simulator.py:65-97``.  Returns (bs, N, N).

    ``ray_dtype``: precision of the ray shooting alone (``tf/simulator.py:57-63``),
    the rest in ``dtype``; float32 here with float64 elsewhere isolates the
    image error that float32 deflections cause (the lensed source's profile
    amplifies the deflection's rounding)."""
    lens_p, ll_p, src_p = _split(model, params)
    x = torch.as_tensor(cfg.img_x, dtype=dtype)[None]
    y = torch.as_tensor(cfg.img_y, dtype=dtype)[None]
    if ray_dtype is None or ray_dtype == dtype:
        bx, by = beta(model, lens_p, x, y, dtype)
    else:
        lp = [{k: torch.as_tensor(v).to(ray_dtype) for k, v in p.items()} for p in lens_p]
        bx, by = beta(model, lp, x.to(ray_dtype), y.to(ray_dtype), ray_dtype)
        bx, by = bx.to(dtype), by.to(dtype)
    if no_deflection:
        bx, by = x, y
    img = 0
    for (kind, opts), p in zip(model["lens_light"], ll_p):
        img = img + _light(kind, opts, x, y, _expand(p, dtype))
    for (kind, opts), p in zip(model["source_light"], src_p):
        img = img + _light(kind, opts, bx, by, _expand(p, dtype))
    img = torch.where(torch.isnan(img), torch.zeros_like(img), img)
    out = _psf_pool(img[:, None], cfg, dtype)[:, 0]
    return out * cfg.conversion_factor


def supersampled_image(model, cfg: SimConfig, params, dtype=torch.float64):
    """The supersampled light image before the PSF (``tf/simulator.py:73-81``)."""
    lens_p, ll_p, src_p = _split(model, params)
    x = torch.as_tensor(cfg.img_x, dtype=dtype)[None]
    y = torch.as_tensor(cfg.img_y, dtype=dtype)[None]
    bx, by = beta(model, lens_p, x, y, dtype)
    img = 0
    for (kind, opts), p in zip(model["lens_light"], ll_p):
        img = img + _light(kind, opts, x, y, _expand(p, dtype))
    for (kind, opts), p in zip(model["source_light"], src_p):
        img = img + _light(kind, opts, bx, by, _expand(p, dtype))
    return torch.where(torch.isnan(img), torch.zeros_like(img), img)


def lstsq_basis(model, cfg: SimConfig, params, dtype=torch.float64):
    """PSF-convolved, binned basis stack ``(bs, N, N, D)``, ``tf/simulator.py:109-153``."""
    lens_p, ll_p, src_p = _split(model, params)
    x = torch.as_tensor(cfg.img_x, dtype=dtype)[None]
    y = torch.as_tensor(cfg.img_y, dtype=dtype)[None]
    bx, by = beta(model, lens_p, x, y, dtype)
    comps = []
    for (kind, opts), p in zip(model["lens_light"], ll_p):
        comps.append(_light(kind, opts, x, y, _expand(p, dtype), lstsq=True))
    for (kind, opts), p in zip(model["source_light"], src_p):
        comps.append(_light(kind, opts, bx, by, _expand(p, dtype), lstsq=True))
    img = torch.cat(comps, dim=0)               # (D, bs, S, S)
    img = torch.where(torch.isnan(img), torch.zeros_like(img), img)
    img = img.permute(1, 0, 2, 3)                # (bs, D, S, S)
    ret = _psf_pool(img, cfg, dtype)
    ret = torch.where(torch.isnan(ret), torch.zeros_like(ret), ret)
    return ret.permute(0, 2, 3, 1)               # (bs, N, N, D)


def lstsq_simulate(model, cfg: SimConfig, params, observed_image, err_map, dtype=torch.float64,
                   return_coeffs=False):
    """``LensSimulator.lstsq_simulate``, ``tf/simulator.py:99-165`` (pinv, rcond=1e-6;
    no conversion factor, as in the reference)."""
    ret = lstsq_basis(model, cfg, params, dtype)
    bs, N, _, D = ret.shape
    W = (1 / torch.as_tensor(err_map, dtype=dtype))[..., None]
    Y = (torch.as_tensor(observed_image, dtype=dtype) * W[..., 0]).reshape(1, -1, 1)
    X = (ret * W).reshape(bs, -1, D)
    Xt = X.transpose(1, 2)
    coeffs = (torch.linalg.pinv(Xt @ X, rtol=1e-6) @ Xt @ Y)[..., 0]
    if return_coeffs:
        return coeffs
    return (ret * coeffs[:, None, None, :]).sum(-1)


def log_likelihood(im_sim, observed, background_rms, exp_time):
    """Gaussian log-likelihood with model-based noise and chi^2,
    ``tf/model.py:77-86``.  Returns (logL (bs,), chi2 (bs,))."""
    obs = torch.as_tensor(observed, dtype=im_sim.dtype)
    err = torch.sqrt(background_rms ** 2 + torch.clamp(im_sim, 0, float("inf")) / exp_time)
    z = (obs - im_sim) / err
    logL = (-0.5 * z ** 2 - torch.log(err) - 0.5 * LOG_2PI).sum(dim=(-2, -1))
    chi2 = (((im_sim - obs) / err) ** 2).mean(dim=(-2, -1))
    return logL, chi2


def backward_log_likelihood(im_sim, observed, err_map):
    """``BackwardProbModel`` likelihood (data-based noise), ``tf/model.py:157-163``."""
    obs = torch.as_tensor(observed, dtype=im_sim.dtype)
    err = torch.as_tensor(err_map, dtype=im_sim.dtype)
    z = (im_sim - obs) / err
    logL = (-0.5 * z ** 2 - torch.log(err) - 0.5 * LOG_2PI).sum(dim=(-2, -1))
    chi2 = (z ** 2).mean(dim=(-2, -1))
    return logL, chi2


# --------------------------------------------------------------------------
# flat parameter vectors in the reference's packing order
# --------------------------------------------------------------------------
PARAM_NAMES = {
    "EPL": ["theta_E", "gamma", "e1", "e2", "center_x", "center_y"],
    "SHEAR": ["gamma1", "gamma2"],
    "SIS": ["theta_E", "center_x", "center_y"],
    "SIE": ["theta_E", "e1", "e2", "center_x", "center_y"],
    "SERSIC": ["R_sersic", "n_sersic", "center_x", "center_y", "Ie"],
    "SERSIC_ELLIPSE": ["R_sersic", "n_sersic", "e1", "e2", "center_x", "center_y", "Ie"],
    "TNFW": ["Rs", "alpha_Rs", "r_trunc", "center_x", "center_y"],
    "CORE_SERSIC": ["R_sersic", "n_sersic", "Rb", "alpha", "gamma", "e1", "e2", "center_x", "center_y", "Ie"],
}


def flat_layout(model, lstsq=False):
    """Leaf order of a flattened parameter structure: groups in order, profiles in
    order, keys sorted (``tf.nest.flatten`` order, ``tf/model.py:42-49``)."""
    groups = [model["lenses"]]
    if len(model["lens_light"]) > 0:
        groups.append(model["lens_light"])
    groups.append(model["source_light"])
    layout = []
    for gi, g in enumerate(groups):
        for pi, (kind, opts) in enumerate(g):
            if kind == "SHAPELETS":
                names = ["beta", "center_x", "center_y"]
                if not (lstsq or opts.get("use_lstsq", False)):
                    D = (opts["n_max"] + 1) * (opts["n_max"] + 2) // 2
                    names += [f"amp{str(i).zfill(len(str(D)))}" for i in range(D)]
            else:
                names = list(PARAM_NAMES[kind])
            if lstsq and "Ie" in names:
                names.remove("Ie")
            for k in sorted(names):
                layout.append((gi, pi, k))
    return layout


def unflatten(model, xflat, lstsq=False):
    """(bs, d) -> nested list-of-dicts structure in reference order."""
    layout = flat_layout(model, lstsq)
    groups = [model["lenses"]]
    if len(model["lens_light"]) > 0:
        groups.append(model["lens_light"])
    groups.append(model["source_light"])
    out = [[{} for _ in g] for g in groups]
    for col, (gi, pi, k) in enumerate(layout):
        out[gi][pi][k] = xflat[:, col]
    return out


def forward_log_likelihood_flat(model, cfg, xflat, observed, background_rms, exp_time, dtype=torch.float64):
    """x (bs, d) physical -> (logL, chi2); autograd-capable."""
    params = unflatten(model, xflat)
    im = simulate(model, cfg, params, dtype)
    if im.dim() == 2:
        im = im[None]
    return log_likelihood(im, observed, background_rms, exp_time)
