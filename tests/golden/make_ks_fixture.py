"""Generates the oracle side of the distributional (KS) parity test.

Runs the CPU oracle (restated cpm-core run path, pinned by the reference's
frozen trajectory) for seeds 1..N of the quickstart configuration
(README.md:47-83 / tests/python/test_builder.py:11-28: 30x30 periodic, one
type V*=50 I*=75 lambda_V=10 lambda_I=2, 5 cells, J=[[0,5],[5,2]], default
placement, 5000 burn-in + 5000 readout MCS) and stores the last sample's
per-cell volume, interface, squared radius of gyration and kappa^2 plus the
final energy. Usage: python tests/golden/make_ks_fixture.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402

N_SEEDS = 256
BURN_IN, READOUT = 5000, 5000


def c1_spec():
    return O.ModelSpec((30, 30), True, [(50, 75, 10.0, 2.0)], [[0, 5], [5, 2]], cell_counts=[5])


def main():
    seeds = np.arange(1, N_SEEDS + 1, dtype=np.uint64)
    failed, cells, energy, n = O.run_many(c1_spec(), seeds, BURN_IN, READOUT, threads=0, local_halo=True)
    assert failed == 0 and np.all(n == 5)
    np.savez_compressed(
        os.path.join(HERE, "c1_oracle_summary.npz"),
        seeds=seeds,
        volume=cells["volume"].astype(np.uint32),
        interface=cells["interface"].astype(np.uint32),
        rg2=cells["rg2"],
        kappa2=cells["kappa2"],
        energy=energy,
    )
    print("wrote", os.path.join(HERE, "c1_oracle_summary.npz"))


if __name__ == "__main__":
    main()
