"""The resident sweep's active-block skip on sparse lattices (the device form
of the reference's EdgeList proposal, edge_list.rs:1-16: the Uniform chain
without its null attempts).

Blocks of 8 x 8 (2D) or 4 x 4 x 4 (3D) sites whose sites all have copy
neighbours of their own cell hold only null attempts; a chunk whose active
blocks are few visits only their sites. Every run here is compared with the
same run forced through the plain build (CPM_GPU_NO_SKIP): lattice, cell
state and counters must be identical, and volumes and interfaces must equal
a recount. The cases are sparse by design (a few small cells in a large
medium), so the skip path is the one that runs.
"""

import numpy as np
import pytest

from helpers import Model

pytestmark = pytest.mark.gpu

CASES = {
    # the reference's proposal-mode case (notebooks/performance_demo.ipynb cell 5)
    "2d_150_periodic": lambda: Model((150, 150), "periodic", [("a", 30, 40, 1.0, 0.2)], [[0, 3], [3, 1]], [10], seed=1),
    "2d_fixed": lambda: Model((120, 96), "fixed", [("a", 30, 40, 1.0, 0.2)], [[0, 3], [3, 1]], [8], seed=2),
    "2d_odd_periodic": lambda: Model((151, 149), "periodic", [("a", 30, 40, 1.0, 0.2)], [[0, 3], [3, 1]], [10],
                                     seed=3),
    "2d_von_neumann_energy": lambda: Model((130, 140), "periodic", [("a", 30, 40, 1.0, 0.2)], [[0, 3], [3, 1]],
                                           [12], energy="von_neumann", seed=4),
    "3d_periodic": lambda: Model((40, 40, 40), "periodic", [("a", 27, 90, 1.0, 0.2)], [[0, 3], [3, 1]], [10],
                                 energy="twenty_six", seed=5),
    "2d_metropolis_hastings": lambda: Model((150, 150), "periodic", [("a", 30, 40, 1.0, 0.2)], [[0, 3], [3, 1]],
                                            [10], seed=6, acceptance="metropolis_hastings"),
}


@pytest.mark.parametrize("name", list(CASES))
def test_active_block_skip_leaves_the_trajectory_unchanged(name, cuda_required, monkeypatch):
    from cpm import _cpm

    model = CASES[name]()
    n = 300 if model.D == 2 else 60
    monkeypatch.delenv("CPM_GPU_NO_SKIP", raising=False)
    skip = _cpm.Engine(model.builder(warn=False))
    assert skip.run_mcs(n) is None
    skip.synchronize()
    monkeypatch.setenv("CPM_GPU_NO_SKIP", "1")
    plain = _cpm.Engine(model.builder(warn=False))
    plain.run_mcs(n)
    plain.synchronize()
    assert np.array_equal(skip.padded(), plain.padded())
    for a, b in zip(skip.cells(), plain.cells()):
        assert np.array_equal(a, b)
    sa, sb = skip.stats(), plain.stats()
    for k in ("attempts", "nonnull", "topology_rejected", "guard_rejected", "evaluated", "accepted"):
        assert sa[k] == sb[k], (k, sa[k], sb[k])
    assert sa["accepted"] > 0
    assert skip.recount_check()[0]
