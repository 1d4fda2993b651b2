"""Exact Boltzmann check of the device chain (tests/exact_boltzmann.rs).

The same harness the oracle passes (tests/test_oracle_boltzmann.py), run by
the device: Metropolis-Hastings acceptance (monte_carlo.rs:168-196), the
connectivity check off (the harness's `attempt(cpm, false)`; the engine's
test switch CPM_GPU_TEST_NO_CONNECTIVITY, honoured by the global-memory
sweep), conservative terms only. The device chain visits each site once per
MCS in colour-class passes, each pass applied as a sequence in priority
order; every single-site update with the n_A / n_B proposal ratio is
reversible with respect to exp(-H), so any such composition keeps exp(-H)/Z
stationary and the visit histogram must match g(H) exp(-H)/Z on the exactly
enumerated 5x5 single-cell and 4x4 two-cell lattices.

Samples are the lattices of many independent simulations (one
`cpm.run_many` launch), thinned by 40 MCS (one cell) and 200 MCS (two
cells) as the harness thins, and pooled. The statistic and its bars are the
harness's: chi-squared below 8 df after pooling bins with expected count
below 20, no bin with expected count >= 20 unvisited, a floor on distinct
bins.
"""

import numpy as np
import pytest

from helpers import Model
from test_oracle_boltzmann import MIN_EXPECTED, _exact, _spec, _start, chi_squared, energy, valid

pytestmark = pytest.mark.gpu

# (simulations, burn-in MCS, samples per simulation, MCS between samples,
#  floor on distinct energy bins visited)
RUNS = {"single": (512, 2000, 200, 40, 25), "two": (512, 2000, 100, 200, 150)}

TYPES = {
    "single": [("a", 8, 20, 0.15, 0.05)],
    "two": [("a", 5, 14, 0.05, 0.01), ("b", 5, 14, 0.05, 0.01)],
}
ADHESION = {
    "single": [[0.0, 0.0], [0.0, 0.0]],
    "two": [[0.0, 0.5, 0.5], [0.5, 0.2, 0.8], [0.5, 0.8, 0.2]],
}


def device_samples(case, run_many):
    """Thinned lattices of the device chain, shape (n, rows, cols)."""
    n_sims, burn, n_samples, thin, _ = RUNS[case]
    start = _start(case)
    k = int(start.max())
    grid = start.shape
    model = Model(grid, "fixed", TYPES[case], ADHESION[case], [1] * k, energy="moore",
                  acceptance="metropolis_hastings")
    builders = [model.builder(seed=1000 + s, lattice=start, cell_type_of=list(range(k)), warn=False)
                for s in range(n_sims)]
    results = run_many(builders, burn, n_samples * thin, thin, include_lattice=True, topology=False)
    lats = [np.asarray(smp.lattice).reshape(grid) for r in results for smp in r.samples]
    assert len(lats) == n_sims * n_samples
    return np.stack(lats)


@pytest.mark.parametrize("case", ["single", "two"])
def test_device_chain_matches_exact_boltzmann(case, cuda_required, monkeypatch):
    from cpm import _cpm

    monkeypatch.setenv("CPM_GPU_TEST_NO_CONNECTIVITY", "1")
    counter, keys, g, h = _exact(case)
    _, p = _spec(case, "metropolis_hastings")
    lats = device_samples(case, _cpm.run_many)
    skeys = counter.keys_of(lats)
    assert np.all(valid(counter, skeys))
    chi2, df, distinct, empty = chi_squared(h, g, energy(counter, skeys, **p))
    print(f"device {case}: chi2 {chi2:.1f} df {df} distinct bins {distinct}")
    assert df >= 1
    assert empty == 0, f"{empty} bins with expected count >= {MIN_EXPECTED} never visited"
    assert distinct >= RUNS[case][4], distinct
    assert chi2 < 8.0 * df, (chi2, df)
