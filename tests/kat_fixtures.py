"""The reference's own known-answer fixtures, restated as data.

* FROZEN_2D: crates/cpm-core/tests/dimension_consistency.rs:40-131 and its
  Python twin tests/python/test_reproducibility.py:38-84 — 30x30 periodic,
  two explicit 2x2 cells, seed 20260915, 500 MCS.
* DERIVED_SEEDS_42: notebooks/batch_execution_demo.ipynb cell 7 output
  (`result.metadata.seed` for master_seed=42, indices 0..4).
"""

import numpy as np

GRID = 30
FROZEN_SEED = 20260915
FROZEN_MCS = 500
FROZEN_VOLUME = [7, 9]
FROZEN_INTERFACE = [28, 32]
FROZEN_ENERGY_BITS = 4638468362461406824
FROZEN_MODEL_HASH = "60ec713de9d698ca55697ff41339081739dfbd506b6117049acaeb7ccbc1d390"
FROZEN_TYPES = [("a", 12, 24, 1.0, 0.2), ("b", 12, 24, 1.2, 0.15)]
FROZEN_ADHESION = [[0.0, 1.0, 1.5], [1.0, 0.5, 2.0], [1.5, 2.0, 0.5]]

DERIVED_SEEDS_42 = [
    6806512004122731638,
    6015650834741855962,
    9699228670906389705,
    4448572121917619020,
    12782757592126568335,
]


def frozen_lattice():
    lat = np.zeros((GRID, GRID), dtype=np.uint32)
    for r, c in [(6, 8), (6, 9), (7, 8), (7, 9)]:
        lat[r, c] = 1
    for r, c in [(18, 20), (18, 21), (19, 20), (19, 21)]:
        lat[r, c] = 2
    return lat
