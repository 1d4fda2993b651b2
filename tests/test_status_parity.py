"""Run-status parity on the CPU: the product's status rule (the one
`cpm_builder_run` applies to its samples, exported as `cpm_run_status`)
against the oracle's independent restatement of output.rs:456-522, on
crafted readouts that reach every kind (Ok, NotEquilibrated, Fragmented,
CellLost, Degenerate) and their priority, and on random readouts.

No GPU: both rules are host code over given energy traces and samples.
"""

import numpy as np
import pytest

import oracle as O

MCS = np.arange(1, 11, dtype=np.uint64) * 100  # ten samples, every 100 MCS


def both(trace, volumes, frag=None, pairs=(), mcs=MCS, floor=1):
    from cpm import _cpm

    got = _cpm.run_status(trace, mcs, volumes, frag, pairs, floor)
    want = O.run_status(trace, mcs, volumes, frag, pairs, floor)
    assert got == want, (got, want)
    return got


def healthy(n_cells=4, n=len(MCS)):
    return np.full((n, n_cells), 30, np.uint32)


FLAT = [5.0, 5.2, 4.9, 5.1, 5.0, 4.8, 5.2]  # no trend against its noise
TREND = [10.0, 9.0, 8.1, 7.0, 6.2, 5.0, 4.1]  # drift far above the residual


def chain(n_cells):
    """Contact pairs joining cells 1..n in a path, plus medium contacts."""
    return [(k, k + 1) for k in range(1, n_cells)] + [(0, k) for k in range(1, n_cells + 1)]


def test_ok_without_and_with_topology():
    assert both(FLAT, healthy())[0] == "Ok"
    assert both(FLAT, healthy(), frag=np.zeros(len(MCS)), pairs=[(1, 2), (0, 3)])[0] == "Ok"


def test_not_equilibrated_takes_precedence_over_everything():
    v = healthy()
    v[5:, 2] = 1  # a lost cell
    frag = np.zeros(len(MCS), np.uint32)
    frag[3] = 2
    assert both(TREND, v, frag, chain(4)) == ("NotEquilibrated", 0, 0)


def test_fragmented_reports_the_first_sample_and_its_first_id():
    v = healthy()
    v[5:, 2] = 1
    frag = np.zeros(len(MCS), np.uint32)
    frag[3], frag[6] = 4, 1
    assert both(FLAT, v, frag, chain(4)) == ("Fragmented", 4, 400)


def test_cell_lost_over_the_trailing_half_of_the_samples():
    v = healthy()
    v[5:, 2] = 1  # samples 6..10 = the trailing ceil(10 / 2)
    assert both(FLAT, v) == ("CellLost", 3, 600)
    v = healthy()
    v[6:, 2] = 1  # only the last four: not lost
    v[5:, 3] = 0
    assert both(FLAT, v) == ("CellLost", 4, 600)
    v = healthy()
    v[6:, 2] = 1
    assert both(FLAT, v)[0] == "Ok"
    # the floor is the configured minimum volume
    v = healthy()
    v[5:, 1] = 3
    assert both(FLAT, v, floor=3) == ("CellLost", 2, 600)
    assert both(FLAT, v, floor=2)[0] == "Ok"
    # an odd number of samples rounds the window up
    m = MCS[:7]
    v = healthy(n=7)
    v[3:, 0] = 1
    assert both(FLAT, v, mcs=m) == ("CellLost", 1, 400)
    v = healthy(n=7)
    v[4:, 0] = 1
    assert both(FLAT, v, mcs=m)[0] == "Ok"


def test_cell_lost_before_degenerate():
    v = healthy()
    v[5:, 0] = 1
    assert both(FLAT, v, np.zeros(len(MCS)), chain(4)) == ("CellLost", 1, 600)


def test_degenerate_needs_every_cell_in_one_cell_cluster():
    z = np.zeros(len(MCS), np.uint32)
    assert both(FLAT, healthy(), z, chain(4))[0] == "Degenerate"
    # medium contacts do not join cells
    assert both(FLAT, healthy(), z, [(0, 1), (0, 2), (0, 3), (0, 4), (1, 2), (3, 4)])[0] == "Ok"
    # an isolated cell breaks it
    assert both(FLAT, healthy(5), z, chain(4))[0] == "Ok"
    # a single cell is never degenerate
    assert both(FLAT, healthy(1), z, [(0, 1)])[0] == "Ok"
    # without topology readouts neither Fragmented nor Degenerate is reached
    frag = z.copy()
    frag[0] = 2
    assert both(FLAT, healthy(), frag, chain(4))[0] == "Fragmented"
    assert both(FLAT, healthy(), None, chain(4))[0] == "Ok"


def test_trace_edge_cases():
    v = healthy()
    assert both([], v)[0] == "Ok"
    assert both([1.0, 100.0], v)[0] == "Ok"  # fewer than three points: never flagged
    assert both([3.0, 3.0, 3.0, 3.0], v)[0] == "Ok"  # flat, no noise
    assert both([1.0, 2.0, 3.0, 4.0], v)[0] == "NotEquilibrated"  # exact line: drift with no noise
    assert both([], healthy(n=0), mcs=np.zeros(0, np.uint64))[0] == "Ok"  # no samples


@pytest.mark.parametrize("seed", range(4))
def test_random_readouts_agree(seed):
    rng = np.random.default_rng(seed)
    for _ in range(500):
        n_cells = int(rng.integers(1, 7))
        n_s = int(rng.integers(0, 9))
        mcs = np.cumsum(rng.integers(1, 50, n_s)).astype(np.uint64)
        tn = int(rng.integers(0, 9))
        trace = rng.normal(0, 1, tn) + rng.choice([0.0, 0.3, 3.0]) * np.arange(tn)
        vol = rng.integers(0, 4, (n_s, n_cells)).astype(np.uint32)
        frag = None
        if rng.random() < 0.7:
            frag = np.where(rng.random(n_s) < 0.15, rng.integers(1, n_cells + 1, n_s), 0).astype(np.uint32)
        pairs = [(int(a), int(b)) for a, b in rng.integers(0, n_cells + 1, (int(rng.integers(0, 8)), 2)) if a < b]
        both(trace, vol, frag, pairs, mcs=mcs, floor=int(rng.integers(0, 3)))
