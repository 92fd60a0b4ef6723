"""Speed-of-sound estimation on the differentiable delay-and-sum (no
counterpart in the reference).

A slowness model -- a global speed of sound c plus a coarse per-region
slowness map, bilinearly upsampled to the pixel grid -- feeds
``SyntheticBeamformer.differentiable``; the loss is the negative mean
lag-1 short-lag spatial coherence of the per-element images plus an image
sharpness term, so gradients reach c, the map and the channel data through
the hand-written adjoint kernels.

The coherence follows the lag-1 term of the SLSC of
examples/advanced_beamforming.ipynb (cell 2, calc_lagn_coherence), written
with torch ops so that it is differentiable: per pixel, for each pair of
adjacent elements that both accept the pixel, the normalised correlation
sum(a b) / sqrt(sum(a^2) sum(b^2)) of their axial kernels, averaged over the
pairs.  Unlike the notebook (and TabbedSLSCBeamformer) it does not subtract
the kernels' means and takes an element by its mask at the pixel itself, not
over the whole kernel: a smooth objective for optimisation, not the display
quantity.
"""
from __future__ import annotations

import torch
import torch.nn.functional as F

__all__ = ["SlownessModel", "slsc_lag1", "sharpness", "sos_loss"]


class SlownessModel(torch.nn.Module):
    """s(pixel) = 1/c + upsample(dmap): a global speed and a coarse map.

    grid_shape (nx, nz) with z fastest in the pixel order (the order of
    helpers.pixel_grid); map_shape the coarse map's (nx, nz).
    """

    def __init__(self, grid_shape, map_shape=(32, 64), c_init=1540.0, device="cuda"):
        super().__init__()
        self.grid_shape = tuple(grid_shape)
        self.c = torch.nn.Parameter(torch.tensor(float(c_init), device=device))
        self.dmap = torch.nn.Parameter(torch.zeros(tuple(map_shape), device=device))

    def forward(self) -> torch.Tensor:
        up = F.interpolate(self.dmap[None, None], size=self.grid_shape, mode="bilinear",
                           align_corners=True)[0, 0]
        return (1.0 / self.c + up).reshape(-1)


def _axial_sum(v: torch.Tensor, nkern: int) -> torch.Tensor:
    """Sum over the axial window [iz - nkern, iz + nkern] (clipped), v (..., nx, nz)."""
    if nkern == 0:
        return v
    shp = v.shape
    flat = v.reshape(-1, 1, shp[-1])
    k = torch.ones((1, 1, 2 * nkern + 1), dtype=v.dtype, device=v.device)
    return F.conv1d(flat, k, padding=nkern).reshape(shp)


def slsc_lag1(img_rx: torch.Tensor, rx_mask: torch.Tensor, grid_shape, nkern: int = 2,
              eps: float = 1e-20) -> torch.Tensor:
    """Lag-1 coherence per pixel, (nx, nz).

    img_rx: (nrx, nx*nz) transmit-summed per-element images; rx_mask
    (nrx, nx*nz) 1 where the element accepts the pixel.
    """
    nrx = img_rx.shape[0]
    nx, nz = grid_shape
    u = img_rx.reshape(nrx, nx, nz)
    m = rx_mask.reshape(nrx, nx, nz).to(u.dtype)
    a, b = u[:-1], u[1:]
    num = _axial_sum(a * b, nkern)
    den = torch.sqrt(_axial_sum(a * a, nkern) * _axial_sum(b * b, nkern) + eps)
    pair = m[:-1] * m[1:]
    r = pair * num / den
    return r.sum(0) / pair.sum(0).clamp(min=1.0)


def sharpness(img: torch.Tensor) -> torch.Tensor:
    """Normalised fourth moment of the image intensity (1 for a flat image)."""
    p = img * img
    return p.numel() * (p * p).sum() / (p.sum() ** 2 + 1e-30)


def sos_loss(img_rx: torch.Tensor, rx_mask: torch.Tensor, grid_shape, nkern: int = 2,
             weight: float = 1e-3) -> torch.Tensor:
    """-mean lag-1 coherence - weight * sharpness of the delay-and-sum image."""
    coh = slsc_lag1(img_rx, rx_mask, grid_shape, nkern)
    return -coh.mean() - weight * sharpness(img_rx.sum(0))
