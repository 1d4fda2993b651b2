"""Configuration-design helper (reference: python/cpm/parameters.py:37-55).

``phi = sum(V_c) / N_sites`` is always derived from a run, never set; this
helper inverts it to suggest a cell count before a `CPM` is built. Pure
arithmetic: nothing here reaches the engine.
"""

from __future__ import annotations

import math
import warnings

from .warnings import CPMLowResolutionWarning

_MIN_CELL_RADIUS_SITES = 5.0


def _radius(target_volume: float, dimensionality: int) -> float:
    # radius of the disc (2D) or ball (3D) with the given volume
    if dimensionality == 2:
        return math.sqrt(target_volume / math.pi)
    if dimensionality == 3:
        return (3.0 * target_volume / (4.0 * math.pi)) ** (1.0 / 3.0)
    raise ValueError(
        "grid must have length 2 or 3 (dimensionality is inferred from it); "
        f"got length {dimensionality}"
    )


def cells_for_density(grid: tuple[int, ...], target_volume: float, phi: float) -> int:
    """Cell count ``n = round(phi * N_sites / target_volume)``; warns with
    :class:`CPMLowResolutionWarning` when the implied radius is under ~5 sites."""
    n_sites = math.prod(grid)
    radius = _radius(target_volume, len(grid))
    if radius < _MIN_CELL_RADIUS_SITES:
        warnings.warn(
            f"implied cell radius {radius:.2f} sites (from target_volume={target_volume}) is below "
            f"{_MIN_CELL_RADIUS_SITES:.0f} sites; lattice discretisation will start dominating the "
            "morphology readouts at this density",
            CPMLowResolutionWarning,
            stacklevel=2,
        )
    return round(phi * n_sites / target_volume)
