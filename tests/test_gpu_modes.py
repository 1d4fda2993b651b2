"""The loop's other modes on the device: Metropolis-Hastings acceptance
(monte_carlo.rs:168-196) and the Act term (energy.rs:329-471), run by the
resident sweep when the lattice fits in shared memory, by the tiled sweep for
larger lattices, and by the global-memory sweep where neither applies.

* Per move: for states the oracle reached (its acquisition MCS included) the
  device decides every proposed move as the oracle does, with the same
  integer interface deltas; delta-H agrees to the bit without the Act term
  and to 1e-12 with it (its geometric mean uses pow, CUDA's and the host
  library's within an ulp).
* Bookkeeping: applying the same accepted moves sets the same acquisition
  MCS, and the incremental V/I equal a recount after a run.
* Distribution: per-seed summaries of 160 runs against the oracle's
  (fixture tests/golden/modes_oracle_summary.npz), two-sample KS p > 0.01;
  and of 128 runs on a 96x96 lattice the tiled sweep cuts into 6x6 tiles
  (modes_tiled_oracle_summary.npz).
* Tiled sweep: exact V/I after runs on even, odd and fixed 2D and 3D
  lattices, acquisition MCS within the run, the same trajectory for any
  number of tiles per CTA and when a run is split, and with lambda_act = 0
  the Metropolis trajectory of the plain kernels, move for move.
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


def _mode_summaries(fixture, mode, grid, n_cells, burn_in, readout):
    """KS p-values of per-seed summaries (energy, mean and spread of the
    volumes, mean interface) of device runs against the oracle fixture."""
    from scipy.stats import ks_2samp

    from cpm import _cpm

    ref = np.load(os.path.join(HERE, "golden", fixture))
    kw = {"mh": dict(acceptance="metropolis_hastings"), "act": dict(act=[(20.0, 20)])}[mode]
    builders = [Model(grid, "periodic", [("a", 40, 30, 3.0, 0.6)], [[0, 6.5], [6.5, 2.2]], [n_cells], seed=int(s),
                      **kw).builder(warn=False) for s in ref["seeds"]]
    results = _cpm.run_many(builders, burn_in, readout, readout, topology=False)
    last = [r.samples[-1] for r in results]
    v = np.stack([s.volume for s in last]).astype(np.float64)
    i = np.stack([s.interface for s in last]).astype(np.float64)
    gpu = {"energy": np.array([s.conservative_energy for s in last]), "mean_volume": v.mean(1),
           "volume_std": v.std(1), "mean_interface": i.mean(1)}
    return {k: ks_2samp(np.asarray(ref[f"{mode}_{k}"]), gpu[k]).pvalue for k in gpu}


@pytest.mark.parametrize("mode", ["mh", "act"])
def test_mode_distributions_match_oracle(mode, cuda_required):
    pvals = _mode_summaries("modes_oracle_summary.npz", mode, (40, 40), 20, 1000, 500)
    print(mode, "KS p-values:", pvals)
    for k, p in pvals.items():
        assert p > 0.01, (k, pvals)


@pytest.mark.parametrize("mode", ["mh", "act"])
def test_tiled_mode_distributions_match_oracle(mode, cuda_required, monkeypatch):
    """The tiled sweep forced on 96x96: 6x6 tiles, 9 of each colour in a
    sub-phase, so cells reach into several tiles and the claims decide which
    tile moves them."""
    monkeypatch.setenv("CPM_GPU_FORCE_TILED", "1")
    pvals = _mode_summaries("modes_tiled_oracle_summary.npz", mode, (96, 96), 115, 2000, 1000)
    print(mode, "tiled 96x96 KS p-values:", pvals)
    for k, p in pvals.items():
        assert p > 0.01, (k, pvals)


TILED = {
    "mh_2d": lambda: Model((96, 84), "periodic", *TWO, [40, 40], acceptance="metropolis_hastings", seed=21),
    "act_2d": lambda: Model((96, 84), "periodic", *TWO, [40, 40], act=[(30.0, 15), (20.0, 25)], seed=22),
    "act_2d_fixed": lambda: Model((70, 64), "fixed", *TWO, [30, 30], act=[(25.0, 20), (0.0, 0)], seed=23),
    "act_mh_2d_odd": lambda: Model((65, 63), "periodic", *TWO, [25, 25], energy="von_neumann",
                                   acceptance="metropolis_hastings", act=[(15.0, 30), (40.0, 10)], seed=24),
    "act_3d": lambda: _with_act(organoid_model(side=32, counts=(30, 30), seed=25), [(20.0, 15), (10.0, 25)]),
    "mh_3d_odd": lambda: Model((33, 31, 35), "periodic", [("a", 60, 90, 2.0, 0.5), ("b", 60, 90, 2.0, 0.5)],
                                     [[0, 16, 16], [16, 4, 9], [16, 9, 5]], [30, 30], energy="twenty_six",
                                     acceptance="metropolis_hastings", seed=26),
}


def _with_act(model, act):
    model.act = act
    return model


def _tiled_engine(model):
    from cpm import _cpm

    return _cpm.Engine(model.builder(warn=False))


@pytest.mark.parametrize("name", sorted(TILED))
def test_tiled_sweep_runs_the_modes_exactly(name, cuda_required, monkeypatch):
    """The tiled sweep (lattices too large for one SM) under MH and Act:
    exact V/I after the run, acquisition MCS set during it, deterministic,
    and the same trajectory with three tiles per CTA and with the run split
    in two launches."""
    monkeypatch.setenv("CPM_GPU_FORCE_TILED", "1")
    model = TILED[name]()
    n = 40 if model.D == 2 else 8
    eng = _tiled_engine(model)
    eng.run_mcs(n)
    eng.synchronize()
    ok, _, _ = eng.recount_check()
    assert ok
    st = eng.stats()
    info = eng.info[0]
    assert st["attempts"] == n * int(info.n_sites), st
    assert st["accepted"] > 0 and st["spin_timeouts"] == 0
    if model.act is not None:
        b = eng.read_birth()
        assert 0 < b.max() <= n - 1 and eng.mcs() == n
    lat = eng.lattice()
    pdims = [int(info.padded_dims[d]) for d in range(model.D)]
    mode = "wrap" if model.boundary == "periodic" else "constant"
    assert np.array_equal(eng.padded().reshape(pdims), np.pad(lat, 1, mode=mode))
    split = _tiled_engine(model)
    split.run_mcs(n // 2)
    split.run_mcs(n - n // 2)
    split.synchronize()
    assert np.array_equal(split.lattice(), lat)
    monkeypatch.setenv("CPM_GPU_TILED_GRID", "3")
    narrow = _tiled_engine(model)
    narrow.run_mcs(n)
    narrow.synchronize()
    assert np.array_equal(narrow.lattice(), lat)
    for k in ("attempts", "nonnull", "accepted", "evaluated", "deferred"):
        assert narrow.stats()[k] == st[k], k
    if model.act is not None:
        assert np.array_equal(narrow.read_birth(), eng.read_birth())


@pytest.mark.parametrize("D", [2, 3])
def test_tiled_act_with_zero_lambda_is_the_metropolis_chain(D, cuda_required, monkeypatch):
    """With lambda_act = 0 every Act delta is zero, so the modes kernels
    (the whole decision in FP64, acquisition MCS written) must make every
    decision the plain Metropolis kernels make (float bracket and FP64
    fallback): the same lattice, counts and position sums after the run."""
    monkeypatch.setenv("CPM_GPU_FORCE_TILED", "1")
    if D == 2:
        plain = Model((96, 84), "periodic", *TWO, [40, 40], seed=31)
    else:
        plain = organoid_model(side=32, counts=(30, 30), seed=32)
    act = Model(plain.grid, plain.boundary, plain.types, plain.adhesion, plain.counts, energy=plain.energy,
                seed=plain.seed, act=[(0.0, 20)] * len(plain.types))
    n = 40 if D == 2 else 8
    engines = [_tiled_engine(m) for m in (plain, act)]
    for e in engines:
        e.run_mcs(n)
        e.synchronize()
    a, b = engines
    assert np.array_equal(a.lattice(), b.lattice())
    for k in ("attempts", "nonnull", "accepted", "evaluated", "deferred"):
        assert a.stats()[k] == b.stats()[k], k
    assert np.array_equal(a.cells()[2], b.cells()[2])
    assert 0 < b.read_birth().max() <= n - 1


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
