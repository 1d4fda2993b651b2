"""The user-facing builder (reference: python/cpm/model.py:22-182).

Configuration calls go straight to the compiled builder (`_cpm.CPM`, a C-ABI
shim over libcpm_gpu.so). Only `run`/`run_batch` execute anything, one whole
trajectory (or batch) per call; they also own the warning policy: when the
engine reports that the default scatter-and-grow placement was used, a
`CPMInitializationWarning` is raised here, in Python, next to the `warnings`
machinery that filters it.
"""

from __future__ import annotations

import warnings
from typing import Any

from . import _cpm
from .warnings import CPMInitializationWarning

_SINGLE = (
    "default (scatter-and-grow) initial placement used; call initialize(lattice=...) for an explicit "
    "placement, or initialize(warn_on_default_init=False) to silence this"
)
_BATCH = (
    "default (scatter-and-grow) initial placement used in at least one batch member; call "
    "initialize(lattice=...) for an explicit placement, or initialize(warn_on_default_init=False) to "
    "silence this"
)


class CPM:
    """One Cellular Potts simulation: configure with the constructor and the
    builder calls, then call :meth:`run` (or :meth:`run_batch`)."""

    def __init__(
        self,
        grid: tuple[int, ...],
        boundary: str,
        seed: int,
        copy_neighborhood: str = "von_neumann",
        energy_neighborhood: str | None = None,
        connectivity_neighborhood: str = "von_neumann",
        acceptance: str | None = None,
        proposal: str | None = None,
        active_terms: dict[str, bool] | None = None,
    ) -> None:
        self._raw = _cpm.CPM(
            grid=list(grid),
            boundary=boundary,
            seed=seed,
            copy_neighborhood=copy_neighborhood,
            energy_neighborhood=energy_neighborhood,
            connectivity_neighborhood=connectivity_neighborhood,
            acceptance=acceptance,
            proposal=proposal,
            active_terms=active_terms,
        )
        self._warn_on_default_init = True

    def register_cell_type(self, name: str, target_volume: int, target_interface: int, lambda_volume: float,
                           lambda_interface: float, lambda_act: float = 0.0, max_act: int = 0) -> None:
        self._raw.register_cell_type(name, target_volume, target_interface, lambda_volume, lambda_interface,
                                     lambda_act, max_act)

    def add_cells(self, cell_type: str, n: int) -> None:
        self._raw.add_cells(cell_type, n)

    def set_adhesion(self, matrix: Any) -> None:
        """Symmetric ``(n_types + 1) x (n_types + 1)`` matrix, row/column 0 =
        medium; any nested iterable of numbers (e.g. a NumPy array)."""
        self._raw.set_adhesion([list(row) for row in matrix])

    def initialize(self, lattice: Any | None = None, cell_type_of: Any | None = None,
                   warn_on_default_init: bool = True) -> None:
        """Selects the initial placement (nothing runs yet): an explicit
        row-major lattice with ``cell_type_of``, or, when ``lattice`` is
        omitted, the default scatter-and-grow."""
        self._warn_on_default_init = warn_on_default_init
        self._raw.initialize(
            list(lattice) if lattice is not None else None,
            list(cell_type_of) if cell_type_of is not None else None,
            warn_on_default_init,
        )

    def run(self, burn_in_mcs: int, readout_mcs: int, sampling_interval_mcs: int, include_lattice: bool = False):
        """Runs the whole trajectory on the GPU in one call and returns the
        run result (``.metadata``, ``.status``, ``.samples``, ...)."""
        used_default, result = self._raw.run(burn_in_mcs, readout_mcs, sampling_interval_mcs, include_lattice)
        if used_default and self._warn_on_default_init:
            warnings.warn(_SINGLE, CPMInitializationWarning, stacklevel=2)
        return result

    def theta_names(self) -> list[str]:
        """Canonical names of the theta vector, in order."""
        return self._raw.theta_names()

    def extract_theta(self) -> list[float]:
        """The current configuration's theta, in canonical order."""
        return self._raw.extract_theta()

    def run_batch(self, thetas: Any, burn_in_mcs: int, readout_mcs: int, sampling_interval_mcs: int,
                  master_seed: int, include_lattice: bool = False) -> list[Any]:
        """One independent trajectory per theta, all resident on the GPU in
        one persistent launch; per-simulation seeds are derived from
        ``(master_seed, index)``. At most one warning for the whole batch."""
        any_used_default, results = self._raw.run_batch(
            [list(t) for t in thetas], burn_in_mcs, readout_mcs, sampling_interval_mcs, master_seed, include_lattice
        )
        if any_used_default and self._warn_on_default_init:
            warnings.warn(_BATCH, CPMInitializationWarning, stacklevel=2)
        return results


def run_many(sims: list[CPM], burn_in_mcs: int, readout_mcs: int, sampling_interval_mcs: int,
             include_lattice: bool = False, topology: bool = True) -> list[Any]:
    """Runs many independent simulations, each with its own grid, parameters
    and seed, in one persistent device launch (an extension: the reference's
    ``run_batch`` shares one grid). ``topology=False`` skips the contact graph
    and labelling readouts. At most one warning for the whole set."""
    results = _cpm.run_many([s._raw for s in sims], burn_in_mcs, readout_mcs, sampling_interval_mcs,
                            include_lattice=include_lattice, topology=topology)
    if any(r.used_default and s._warn_on_default_init for s, r in zip(sims, results)):
        warnings.warn(_BATCH, CPMInitializationWarning, stacklevel=2)
    return results


class Server:
    """A serving loop on the GPU: :meth:`submit` a configured :class:`CPM`
    with its run window at any time and collect the result with
    :meth:`wait` or :meth:`poll`. Simulations share the device by continuous
    batching (admitted as slots and ``hbm_budget_bytes`` allow, run side by
    side with their lattices resident until read back, freed when done);
    each result equals :meth:`CPM.run` for the same simulation (an
    extension: the reference has no serving API)."""

    def __init__(self, hbm_budget_bytes: int = 0, max_active: int = 0, placement_threads: int = 0,
                 tiled_grid_cap: int = 0) -> None:
        self._s = _cpm.Server(hbm_budget_bytes, max_active, placement_threads, tiled_grid_cap)

    def submit(self, sim: CPM, burn_in_mcs: int, readout_mcs: int, sampling_interval_mcs: int,
               include_lattice: bool = False, topology: bool = True) -> int:
        return self._s.submit(sim._raw, burn_in_mcs, readout_mcs, sampling_interval_mcs, include_lattice, topology)

    def poll(self, ticket: int):
        return self._s.poll(ticket)

    def wait(self, ticket: int, timeout: float | None = None):
        return self._s.wait(ticket, timeout)

    def cancel(self, ticket: int) -> None:
        self._s.cancel(ticket)

    def stats(self) -> dict:
        return self._s.stats()

    def close(self) -> None:
        self._s.close()

    def __enter__(self) -> "Server":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

