"""Simulator configuration and interface, restating ``gigalens/simulator.py:11-125``.

``get_coords`` restates the grid that the reference obtains from
lenstronomy's ``PixelGrid`` (lenstronomy 1.9.3, not a dependency here): pixel
(row, col) of the supersampled grid sits at ``T @ [col, row] + T @ [lo, lo]``
with ``lo = -(S-1)/2``, T the fine pixel-to-angle matrix.  The orientation is
pinned by the reference's own demo fixture (``assets/demo.npy``): the
chi^2 of the notebook's true parameters is ~1 on this grid and >9 on its
mirror images.

``supersample_kernel`` stands in for lenstronomy's ``subgrid_kernel`` (used by
``tf/simulator.py:48-50``): a project-written resampling of the base-scale PSF
onto the supersampled grid.  Its numerics are not pinned against lenstronomy;
pass ``SimulatorConfig.kernel_supersampled`` to supply the supersampled kernel
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


def supersample_kernel(kernel, supersample: int) -> np.ndarray:
    """Resample a base-scale PSF onto the supersampled grid (odd side).

    The output has side ``ss*k0 - (ss-1)`` (odd for odd ``k0``); its pixel
    centres are at multiples of ``1/ss`` base pixels spanning the same extent
    as the input.  Values come from a bicubic spline through the input
    samples, negatives are clipped and the result is normalised to unit sum.
    ``supersample == 1`` returns the normalised input.
    """
    k = np.asarray(kernel, dtype=np.float64)
    if k.ndim != 2 or k.shape[0] != k.shape[1] or k.shape[0] % 2 == 0:
        raise ValueError("kernel must be square with odd side, got %s" % (k.shape,))
    ss = int(supersample)
    if ss == 1:
        return (k / k.sum()).astype(np.float32)
    from scipy.interpolate import RectBivariateSpline

    k0 = k.shape[0]
    c = (k0 - 1) / 2.0
    n = ss * k0 - (ss - 1)
    pos = (np.arange(n) - (n - 1) / 2.0) / ss
    spline = RectBivariateSpline(np.arange(k0) - c, np.arange(k0) - c, k, kx=3, ky=3)
    out = np.clip(spline(pos, pos), 0.0, None)
    return (out / out.sum()).astype(np.float32)


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
