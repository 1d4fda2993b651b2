"""The loop's other modes on the device: Metropolis-Hastings acceptance
(monte_carlo.rs:168-196) and the Act term (energy.rs:329-471), run by the
resident sweep when the lattice fits in shared memory and by the
global-memory sweep otherwise.

* Per move: for states the oracle reached (its acquisition MCS included) the
  device decides every proposed move as the oracle does, with the same
  integer interface deltas; delta-H agrees to the bit without the Act term
  and to 1e-12 with it (its geometric mean uses pow, CUDA's and the host
  library's within an ulp).
* Bookkeeping: applying the same accepted moves sets the same acquisition
  MCS, and the incremental V/I equal a recount after a run.
* Distribution: per-seed summaries of 160 runs against the oracle's
  (fixture tests/golden/modes_oracle_summary.npz), two-sample KS p > 0.01.
"""

import os
import zlib

import numpy as np
import pytest

from helpers import Model, organoid_model, padded_cells, random_interior_targets

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIELDS = ("losing", "gaining", "null_move", "topology_ok", "volume_guard_ok", "evaluated",
          "delta_i_losing", "delta_i_gaining", "accepted")

TWO = ([("a", 20, 24, 2.0, 0.5), ("b", 20, 24, 1.5, 0.4)], [[0, 4, 4], [4, 1, 6], [4, 6, 1]])

MODELS = {
    "mh_2d": lambda: Model((40, 36), "periodic", *TWO, [12, 12], acceptance="metropolis_hastings", seed=11),
    "act_2d": lambda: Model((40, 36), "periodic", *TWO, [12, 12], act=[(30.0, 15), (20.0, 25)], seed=12),
    "act_2d_fixed": lambda: Model((34, 30), "fixed", *TWO, [10, 10], act=[(25.0, 20), (0.0, 0)], seed=13),
    "act_mh_2d_vn": lambda: Model((36, 36), "periodic", *TWO, [10, 10], energy="von_neumann",
                                  acceptance="metropolis_hastings", act=[(15.0, 30), (40.0, 10)], seed=14),
    "act_3d": lambda: _act_3d(),
}


def _act_3d():
    m = organoid_model(side=14, counts=(5, 5), seed=15)
    m.act = [(20.0, 15), (10.0, 25)]
    return m


def _device_copy(model, sim):
    from cpm import _cpm

    eng = _cpm.Engine(model.builder(warn=False))
    v, i, sp, so = padded_cells(sim)
    eng.write_state(sim.padded(), v, i, sp, so)
    eng.write_act_state(sim.birth() if model.act is not None else None, sim.mcs)
    return eng


@pytest.mark.parametrize("name", list(MODELS))
def test_per_move_parity(name, cuda_required):
    model = MODELS[name]()
    sim = model.oracle()
    sim.run_mcs(25 if model.D == 2 else 4)
    eng = _device_copy(model, sim)
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    t = random_interior_targets(sim, 20000, rng)
    k = rng.integers(0, 2 * model.D, t.size).astype(np.int32)
    u = rng.random(t.size)
    got, want = eng.evaluate_moves(t, k, u), sim.evaluate_moves(t, k, u)
    for f in FIELDS:
        bad = np.flatnonzero(got[f] != want[f])
        assert bad.size == 0, f"{f} differs at {bad[:5]}: got {got[f][bad[:5]]} want {want[f][bad[:5]]}"
    assert np.array_equal(got["accepted_sweep"], got["accepted"])
    ev = want["evaluated"] != 0
    assert ev.sum() > 200
    if model.act is None:
        assert np.array_equal(got["delta_h"].view(np.uint64), want["delta_h"].view(np.uint64))
    else:
        gd, wd = got["delta_h"][ev], want["delta_h"][ev]
        same_nan = np.isnan(gd) & np.isnan(wd)
        assert np.all(same_nan | (np.abs(gd - wd) <= 1e-12 * np.maximum(1.0, np.abs(wd)))), (gd, wd)
        # the Act term contributed: the oracle's conservative part alone differs somewhere
        assert np.any(np.abs(wd) > 0)


@pytest.mark.parametrize("name", ["act_2d", "act_3d"])
def test_commit_sets_acquisition_mcs(name, cuda_required):
    model = MODELS[name]()
    sim = model.oracle()
    sim.run_mcs(10 if model.D == 2 else 3)
    eng = _device_copy(model, sim)
    rng = np.random.default_rng(5)
    pad = sim.padded()
    step = sim.strides()[model.D - 1]
    # distinct targets, none the source of another, each copying a different
    # cell from its neighbour along the last axis
    t = np.unique(random_interior_targets(sim, 600, rng))
    t = t[~np.isin(t + step, t) & ~np.isin(t - step, t)]
    g = pad[t + step].astype(np.uint32)
    keep = g != pad[t]
    t, g = t[keep][:200], g[keep][:200]
    assert t.size > 20
    for q in range(t.size):
        sim.commit(int(t[q]), int(pad[t[q]]), int(g[q]), 0.0)
    eng.commit_moves(t, g)
    assert np.array_equal(eng.read_birth(), sim.birth())


@pytest.mark.parametrize("sweep", ["auto", "global"])
@pytest.mark.parametrize("name", ["mh_2d", "act_2d", "act_3d"])
def test_runs_keep_exact_state(name, sweep, cuda_required, monkeypatch):
    """Both sweeps that run these modes (resident for lattices that fit in
    shared memory, the global-memory sweep for larger ones) keep exact V/I
    and set acquisition MCS no later than the current MCS."""
    from cpm import _cpm

    if sweep == "global":
        monkeypatch.setenv("CPM_GPU_FORCE_GLOBAL", "1")
    model = MODELS[name]()
    eng = _cpm.Engine(model.builder(warn=False))
    eng.run_mcs(30 if model.D == 2 else 6)
    eng.synchronize()
    ok, _, _ = eng.recount_check()
    assert ok
    st = eng.stats()
    assert st["accepted"] > 0
    if model.act is not None:
        b = eng.read_birth()
        assert b.max() <= eng.mcs() and b.max() > 0


@pytest.mark.parametrize("mode", ["mh", "act"])
def test_mode_distributions_match_oracle(mode, cuda_required):
    from scipy.stats import ks_2samp

    from cpm import _cpm

    ref = np.load(os.path.join(HERE, "golden", "modes_oracle_summary.npz"))
    kw = {"mh": dict(acceptance="metropolis_hastings"), "act": dict(act=[(20.0, 20)])}[mode]
    builders = [Model((40, 40), "periodic", [("a", 40, 30, 3.0, 0.6)], [[0, 6.5], [6.5, 2.2]], [20], seed=int(s),
                      **kw).builder(warn=False) for s in ref["seeds"]]
    results = _cpm.run_many(builders, 1000, 500, 500, topology=False)
    last = [r.samples[-1] for r in results]
    v = np.stack([s.volume for s in last]).astype(np.float64)
    i = np.stack([s.interface for s in last]).astype(np.float64)
    gpu = {"energy": np.array([s.conservative_energy for s in last]), "mean_volume": v.mean(1),
           "volume_std": v.std(1), "mean_interface": i.mean(1)}
    pvals = {k: ks_2samp(np.asarray(ref[f"{mode}_{k}"]), gpu[k]).pvalue for k in gpu}
    print(mode, "KS p-values:", pvals)
    for k, p in pvals.items():
        assert p > 0.01, (k, pvals)


def test_edge_list_proposal_runs_the_uniform_chain(cuda_required):
    """proposal = "edge_list" (monte_carlo.rs:336-352) is the Uniform chain
    with its null attempts removed (edge_list.rs:1-16); the device sweep
    runs the same chain for both, so the samples are identical and only the
    convention hash records the choice."""
    import cpm

    def sim(proposal):
        s = cpm.CPM(grid=(40, 40), boundary="periodic", seed=9, proposal=proposal)
        s.register_cell_type("a", 40, 30, 3.0, 0.6)
        s.add_cells("a", 12)
        s.set_adhesion([[0, 6.5], [6.5, 2.2]])
        s.initialize(warn_on_default_init=False)
        return s.run(200, 200, 100)

    u, e = sim("uniform"), sim("edge_list")
    assert len(u.samples) == len(e.samples) == 2
    for a, b in zip(u.samples, e.samples):
        assert np.array_equal(a.volume, b.volume) and np.array_equal(a.interface, b.interface)
        assert a.conservative_energy == b.conservative_energy
    assert u.metadata.convention_hash != e.metadata.convention_hash
