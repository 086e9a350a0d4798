"""Simulator configuration and interface, restating ``gigalens/simulator.py:11-125``.

``get_coords`` restates the grid that the reference obtains from
lenstronomy's ``PixelGrid`` (lenstronomy 1.9.3, not a dependency here): pixel
(row, col) of the supersampled grid sits at ``T @ [col, row] + T @ [lo, lo]``
with ``lo = -(S-1)/2``, T the fine pixel-to-angle matrix.  The orientation is
pinned by the reference's own demo fixture (``assets/demo.npy``): the
chi^2 of the notebook's true parameters is ~1 on this grid and >9 on its
mirror images.

``supersample_kernel`` restates the published behaviour of lenstronomy's
``kernel_util.subgrid_kernel(kernel, supersample, odd=True)`` (lenstronomy
1.9.3, called by ``tf/simulator.py:48-50``), written here from its
description: interpolate the base-scale PSF onto the finer grid, then
iterate so that re-binning the fine kernel to the base grid reproduces the
input PSF.  lenstronomy is not installed here, so its numerics are not
pinned against it ("parity unpinned"); pass
``SimulatorConfig.kernel_supersampled`` to supply the supersampled kernel
directly.
"""
from abc import ABC, abstractmethod
from dataclasses import dataclass
from typing import Any, Dict, List, Optional, Tuple

import numpy as np


@dataclass
class SimulatorConfig:
    """Camera settings (``gigalens/simulator.py:11-28``).

    Attributes:
        delta_pix: pixel scale (arcsec per base pixel)
        num_pix: image side in base pixels
        supersample: supersampling factor
        kernel: base-scale PSF (optional)
        transform_pix2angle: base-scale pixel-to-angle matrix (default delta_pix * I)
        kernel_supersampled: the PSF already on the supersampled grid (odd side);
            when given it is used as-is instead of resampling ``kernel``
    """

    delta_pix: float
    num_pix: int
    supersample: Optional[int] = 1
    kernel: Optional[Any] = None
    transform_pix2angle: Optional[np.ndarray] = None
    kernel_supersampled: Optional[Any] = None


def base_transform(sim_config: SimulatorConfig) -> np.ndarray:
    """Base-scale transform as float32, ``tf/simulator.py:19-23``."""
    if sim_config.transform_pix2angle is None:
        return np.eye(2, dtype=np.float32) * np.float32(sim_config.delta_pix)
    return np.asarray(sim_config.transform_pix2angle, dtype=np.float32).reshape(2, 2)


def _resize_matrix(n_in: int, n_out: int) -> np.ndarray:
    """Bilinear resampling along one axis, as a matrix (n_out x n_in).

    Both grids tile the same extent: input pixel i is centred at
    (i + 1/2) / n_in of it, output pixel j at (j + 1/2) / n_out.  Output
    centres outside the outermost input centres take the edge value."""
    t = ((np.arange(n_out) + 0.5) / n_out) * n_in - 0.5
    t = np.clip(t, 0.0, n_in - 1.0)
    i0 = np.minimum(np.floor(t).astype(np.int64), max(n_in - 2, 0))
    w = t - i0
    R = np.zeros((n_out, n_in))
    R[np.arange(n_out), i0] = 1.0 - w
    if n_in > 1:
        R[np.arange(n_out), i0 + 1] += w
    return R


def _rebin_matrix(n_low: int, n_high: int, ss: int) -> np.ndarray:
    """Re-binning of a fine axis to the base axis, as a matrix (n_low x n_high).

    n_high = ss * n_low: plain sums of ss fine pixels.  n_high = ss * n_low - 1
    (even ss with an odd output side): base pixel I takes fine pixels
    ss*I .. ss*I + ss - 2 whole and half of each fine pixel on its borders
    (ss*I - 1 and ss*I + ss - 1), which it shares with its neighbours.  Every
    fine pixel's weights sum to 1, so the re-binned kernel keeps the sum."""
    B = np.zeros((n_low, n_high))
    if n_high == ss * n_low:
        for i in range(n_low):
            B[i, ss * i: ss * i + ss] = 1.0
        return B
    for i in range(n_low):
        B[i, ss * i: ss * i + ss - 1] = 1.0
        if i > 0:
            B[i, ss * i - 1] = 0.5
        if i < n_low - 1:
            B[i, ss * i + ss - 1] = 0.5
    return B


def supersample_kernel(kernel, supersample: int, num_iter: int = 100) -> np.ndarray:
    """Supersampled PSF from a base-scale one (odd side), the published
    behaviour of lenstronomy's ``subgrid_kernel(kernel, ss, odd=True)``.

    The fine kernel has ``ss * k0`` pixels per side, one fewer when that is
    even, and tiles the same extent as the input (``_resize_matrix``).
    Starting from the normalised input ``u = k``, each of ``num_iter`` steps
    interpolates ``u`` onto the fine grid (bilinear), normalises it to unit
    sum, re-bins it to the base grid (``_rebin_matrix``) and adds the
    difference to the input PSF onto ``u``.  After 100 steps the re-binned
    result reproduces the input to ~1e-12 (the TinyTim PSF of the
    reference's demo).  float64 throughout, returned as float32 with unit
    sum.  ``supersample == 1`` returns the normalised input.
    """
    k = np.asarray(kernel, dtype=np.float64)
    if k.ndim != 2 or k.shape[0] != k.shape[1] or k.shape[0] % 2 == 0:
        raise ValueError("kernel must be square with odd side, got %s" % (k.shape,))
    k = k / k.sum()
    ss = int(supersample)
    if ss == 1:
        return k.astype(np.float32)
    n_in = k.shape[0]
    n_out = ss * n_in - (1 if (ss * n_in) % 2 == 0 else 0)
    R = _resize_matrix(n_in, n_out)
    B = _rebin_matrix(n_in, n_out, ss)

    def fine(u):
        f = R @ u @ R.T
        return f / f.sum()

    u = k.copy()
    sub = fine(u)
    for _ in range(max(int(num_iter), 1)):
        u = u + (k - B @ sub @ B.T)
        sub = fine(u)
    return (sub / sub.sum()).astype(np.float32)


def rebin_kernel(kernel_supersampled, supersample: int) -> np.ndarray:
    """The base-scale kernel a supersampled one re-bins to (the inverse
    direction of ``supersample_kernel``), float64."""
    f = np.asarray(kernel_supersampled, dtype=np.float64)
    ss = int(supersample)
    n_out = f.shape[0]
    n_in = (n_out + 1) // ss if n_out % ss else n_out // ss
    B = _rebin_matrix(n_in, n_out, ss)
    return B @ f @ B.T


def resolved_kernel(sim_config: SimulatorConfig) -> Optional[np.ndarray]:
    """The supersampled PSF the simulator convolves with (unflipped), or None."""
    if sim_config.kernel_supersampled is not None:
        k = np.asarray(sim_config.kernel_supersampled, dtype=np.float32)
        if k.ndim != 2 or k.shape[0] != k.shape[1] or k.shape[0] % 2 == 0:
            raise ValueError("kernel_supersampled must be square with odd side")
        return k
    if sim_config.kernel is None:
        return None
    return supersample_kernel(sim_config.kernel, int(sim_config.supersample))


class LensSimulatorInterface(ABC):
    """Simulates batches of lenses (``gigalens/simulator.py:31-89``)."""

    def __init__(self, phys_model, sim_config: SimulatorConfig, bs: int):
        self.phys_model = phys_model
        self.sim_config = sim_config
        self.bs = bs

    @abstractmethod
    def simulate(self, params: Tuple[List[Dict], List[Dict], List[Dict]]):
        """Simulated images for physical parameters ``params``."""

    @abstractmethod
    def lstsq_simulate(self, params, observed_image, err_map):
        """Simulated images with linear amplitudes solved by weighted least squares."""

    @staticmethod
    def get_coords(supersample: int, num_pix: int, transform_pix2angle) -> Tuple[float, float, np.ndarray, np.ndarray]:
        """RA/DEC of pixel (0, 0) and the supersampled coordinate grids.

        ``transform_pix2angle`` is the fine matrix (base divided by ``supersample``).
        """
        S = int(supersample) * int(num_pix)
        T = np.asarray(transform_pix2angle, dtype=np.float32).reshape(2, 2)
        lo = np.arange(0, S, dtype=np.float32)
        lo = np.float32(np.min(lo - np.mean(lo)))
        ra0, dec0 = (T @ np.array([lo, lo], dtype=np.float32)).astype(np.float32)
        Td = T.astype(np.float64)
        cols, rows = np.meshgrid(np.arange(S, dtype=np.float64), np.arange(S, dtype=np.float64))
        x = Td[0, 0] * cols + Td[0, 1] * rows + np.float64(ra0)
        y = Td[1, 0] * cols + Td[1, 1] * rows + np.float64(dec0)
        return float(ra0), float(dec0), x.astype(np.float32), y.astype(np.float32)
