"""Per-move and bookkeeping parity of the GB300 kernels against the oracle.

Per move: for any lattice state and proposed move, the connectivity
verdict, the volume guard, the integer interface deltas and the FP64
Delta-H bits are identical to the reference's (oracle: restated
crates/cpm-core/src/monte_carlo.rs:52-145, connectivity.rs:42-65,
energy.rs:92-264). Exact state: the device's incremental V/I always equal a
full recount. All compare through the C ABI (libcpm_gpu.so).
"""

import numpy as np
import pytest

from helpers import Model, c1_model, organoid_model, padded_cells, random_interior_targets, sorting_model

pytestmark = pytest.mark.gpu

FIELDS = ("losing", "gaining", "null_move", "topology_ok", "volume_guard_ok", "evaluated",
          "delta_i_losing", "delta_i_gaining", "accepted")


def _engine(model, **kw):
    from cpm import _cpm

    return _cpm.Engine(model.builder(**kw))


def _compare(got, want):
    for f in FIELDS:
        bad = np.flatnonzero(got[f] != want[f])
        assert bad.size == 0, f"{f} differs at {bad[:5]}: got {got[f][bad[:5]]} want {want[f][bad[:5]]}"
    gb = got["delta_h"].view(np.uint64)
    wb = want["delta_h"].view(np.uint64)
    bad = np.flatnonzero(gb != wb)
    assert bad.size == 0, f"delta_h bits differ at {bad[:5]}: {got['delta_h'][bad[:5]]} vs {want['delta_h'][bad[:5]]}"
    # the sweeps' float pre-decision (with its FP64 fallback) on the same u
    bad = np.flatnonzero(got["accepted_sweep"] != got["accepted"])
    assert bad.size == 0, f"sweep decision differs at {bad[:5]}: dh {got['delta_h'][bad[:5]]}"


MODELS = {
    "c1_periodic": lambda: c1_model(seed=1),
    "c1_fixed": lambda: Model((30, 30), "fixed", [("e", 50, 75, 10.0, 2.0)], [[0, 5], [5, 2]], [5], seed=2),
    "sorting_moore": lambda: sorting_model(side=48, seed=4),
    "sorting_vn_energy": lambda: Model((40, 40), "periodic", [("a", 40, 30, 3.0, 1.0), ("b", 40, 30, 2.0, 0.7)],
                                       [[0, 9.5, 7.25], [9.5, 2.125, 6.3], [7.25, 6.3, 3.7]], [8, 8],
                                       energy="von_neumann", seed=5),
    "odd_periodic": lambda: Model((31, 29), "periodic", [("a", 30, 40, 4.0, 0.9)], [[0, 6.1], [6.1, 1.3]], [6], seed=6),
    "3d_26": lambda: organoid_model(side=20, energy="twenty_six"),
    "3d_18_fixed": lambda: organoid_model(side=18, energy="eighteen", boundary="fixed", counts=(6, 6)),
    "3d_vn": lambda: organoid_model(side=17, energy="von_neumann", counts=(5, 5)),
}


@pytest.mark.parametrize("name", sorted(MODELS))
def test_per_move_parity_along_oracle_trajectory(name, cuda_required):
    model = MODELS[name]()
    sim = model.oracle()
    eng = _engine(model)
    rng = np.random.default_rng(hash(name) & 0xFFFF)
    n_eval = 0
    for _ in range(4):
        sim.run_mcs(25 if model.D == 2 else 3)
        v, i, sp, so = padded_cells(sim)
        eng.write_state(sim.padded(), v, i, sp, so)
        t = random_interior_targets(sim, 20000, rng)
        k = rng.integers(0, 2 * model.D, t.size)
        u = rng.random(t.size)
        got = eng.evaluate_moves(t, k, u)
        want = sim.evaluate_moves(t, k, u)
        _compare(got, want)
        n_eval += int(want["evaluated"].sum())
    assert n_eval > 500, n_eval


# relative offsets of u from exp(-dh): inside, at and beyond the float
# pre-decision's uncertainty band (3e-5), down to 1e-12 (far above the 1-ulp
# difference between two correctly implemented FP64 exponentials)
NEAR = np.array([-1e-3, -1e-4, -3.5e-5, -3e-5, -2e-5, -1e-5, -1e-6, -1e-9, -1e-12,
                 1e-12, 1e-9, 1e-6, 1e-5, 2e-5, 3e-5, 3.5e-5, 1e-4, 1e-3])


# weak couplings, so that many uphill moves have dh of order 1
SOFT = {
    "soft_2d": lambda: Model((48, 48), "periodic", [("a", 40, 30, 0.02, 0.01), ("b", 40, 30, 0.03, 0.015)],
                             [[0, 0.8, 0.7], [0.8, 0.3, 0.55], [0.7, 0.55, 0.35]], [10, 10], seed=8),
    "soft_3d_26": lambda: Model((16, 16, 16), "periodic", [("a", 60, 90, 0.004, 0.0015)],
                                [[0, 0.11], [0.11, 0.043]], [8], energy="twenty_six", seed=9),
}


@pytest.mark.parametrize("name", sorted(SOFT))
def test_sweep_decision_at_the_metropolis_threshold(name, cuda_required):
    """u placed just below / above exp(-dh): the bounded float decision and
    its FP64 fallback give the reference's `u < exp(-dh)` every time."""
    model = SOFT[name]()
    sim = model.oracle()
    eng = _engine(model)
    rng = np.random.default_rng(7)
    checked = 0
    for _ in range(3):
        sim.run_mcs(20 if model.D == 2 else 3)
        v, i, sp, so = padded_cells(sim)
        eng.write_state(sim.padded(), v, i, sp, so)
        t = random_interior_targets(sim, 20000, rng)
        k = rng.integers(0, 2 * model.D, t.size)
        first = sim.evaluate_moves(t, k, np.full(t.size, 0.5))
        # dh < 8 keeps exp(-dh) > 3.3e-4, where the 2^-53 grid of u is finer
        # than the smallest offset
        up = np.flatnonzero((first["evaluated"] == 1) & (first["delta_h"] > 0) & (first["delta_h"] < 8))
        assert up.size > 20, up.size
        up = up[:400]
        tt = np.repeat(t[up], NEAR.size)
        kk = np.repeat(k[up], NEAR.size)
        e = np.exp(-np.repeat(first["delta_h"][up], NEAR.size))
        u = e * (1.0 + np.tile(NEAR, up.size))
        u = np.floor(np.minimum(u, 1 - 2.0**-53) * 2.0**53) * 2.0**-53  # on the 53-bit grid of gen::<f64>
        got = eng.evaluate_moves(tt, kk, u)
        want = sim.evaluate_moves(tt, kk, u)
        _compare(got, want)
        assert np.array_equal(got["accepted"], (u < e).astype(np.int32))
        checked += tt.size
    assert checked > 1000


# leaves of very different magnitude in one delta-H: adhesion energies of
# order 1e6 whose sum cancels to order 1 beside volume/interface terms of
# order 1e-6 (close calls: the float sum's rounding error is far larger than
# the result, and the error bound must send every such decision to the FP64
# fallback), and huge volume/interface couplings beside tiny adhesion
MIXED = {
    "mixed_huge_J_2d": lambda: Model((40, 40), "periodic", [("a", 40, 30, 1e-6, 3e-6), ("b", 40, 30, 2e-6, 1e-6)],
                                     [[0, 1e6, 1e6 + 1.5], [1e6, 7e5, 1e6 - 0.25], [1e6 + 1.5, 1e6 - 0.25, 7e5]],
                                     [10, 10], seed=42),
    "mixed_huge_J_3d_26": lambda: Model((16, 16, 16), "periodic", [("a", 60, 90, 1e-6, 2e-6), ("b", 60, 90, 3e-6, 1e-6)],
                                        [[0, 1e6, 1e6 + 0.75], [1e6, 6e5, 1e6 - 0.5],
                                         [1e6 + 0.75, 1e6 - 0.5, 6e5 + 0.125]], [8, 8], energy="twenty_six", seed=43),
    "mixed_huge_lambda_2d": lambda: Model((40, 40), "periodic", [("a", 40, 30, 1e6, 3e5), ("b", 41, 29, 1e6, 2.5e5)],
                                          [[0, 1e-6, 2e-6], [1e-6, 3e-6, 5e-7], [2e-6, 5e-7, 1e-6]], [10, 10],
                                          seed=41),
}


def test_sweep_decision_with_mixed_magnitudes(cuda_required):
    """delta-H summed from terms of magnitude 1e6 and 1e-6 (either way
    round): the sweeps' float decision with its FP64 fallback equals
    `u < exp(-dh)` of the reference for random u and for u placed at
    relative offsets 1e-12 ... 1e-3 from exp(-dh)."""
    near_checked = 0
    for name in sorted(MIXED):
        model = MIXED[name]()
        sim = model.oracle()
        eng = _engine(model)
        rng = np.random.default_rng(17)
        for _ in range(3):
            sim.run_mcs(5 if model.D == 2 else 2)
            v, i, sp, so = padded_cells(sim)
            eng.write_state(sim.padded(), v, i, sp, so)
            t = random_interior_targets(sim, 20000, rng)
            k = rng.integers(0, 2 * model.D, t.size)
            u = rng.random(t.size)
            got = eng.evaluate_moves(t, k, u)
            want = sim.evaluate_moves(t, k, u)
            _compare(got, want)
            assert want["evaluated"].sum() > 100
            # close calls wherever exp(-dh) is a normal double
            up = np.flatnonzero((want["evaluated"] == 1) & (want["delta_h"] > 0) & (want["delta_h"] < 700))
            up = up[:300]
            if up.size == 0:
                continue
            tt = np.repeat(t[up], NEAR.size)
            kk = np.repeat(k[up], NEAR.size)
            e = np.exp(-np.repeat(want["delta_h"][up], NEAR.size))
            uu = np.minimum(e * (1.0 + np.tile(NEAR, up.size)), 1 - 2.0**-53)
            got = eng.evaluate_moves(tt, kk, uu)
            want2 = sim.evaluate_moves(tt, kk, uu)
            _compare(got, want2)
            near_checked += tt.size
    assert near_checked > 1000, near_checked


def test_sweep_decision_for_zero_delta_h(cuda_required):
    """dh == 0 (the float bracket straddles zero) accepts for every u, up to
    the largest u below 1; small non-zero dh keep the reference's rule."""
    model = MODELS["sorting_moore"]()
    sim = model.oracle()
    eng = _engine(model)
    rng = np.random.default_rng(11)
    n_zero = 0
    for _ in range(3):
        sim.run_mcs(30)
        v, i, sp, so = padded_cells(sim)
        eng.write_state(sim.padded(), v, i, sp, so)
        t = random_interior_targets(sim, 40000, rng)
        k = rng.integers(0, 4, t.size)
        first = sim.evaluate_moves(t, k, np.full(t.size, 0.5))
        sel = np.flatnonzero((first["evaluated"] == 1) & (np.abs(first["delta_h"]) < 0.5))
        n_zero += int((first["delta_h"][sel] == 0).sum())
        us = np.array([0.0, 0.5, 0.999, 1 - 1e-6, 1 - 3 * 2.0**-53, 1 - 2 * 2.0**-53, 1 - 2.0**-53])
        tt = np.repeat(t[sel], us.size)
        kk = np.repeat(k[sel], us.size)
        u = np.tile(us, sel.size)
        got = eng.evaluate_moves(tt, kk, u)
        want = sim.evaluate_moves(tt, kk, u)
        _compare(got, want)
    assert n_zero > 10, n_zero


@pytest.mark.parametrize("D", [2, 3])
def test_topology_verdicts_on_random_patterns(D, cuda_required):
    """Random ids on the lattice give arbitrary 8/26-bit neighbourhood patterns."""
    side = 24 if D == 2 else 12
    model = Model((side,) * D, "periodic", [("a", 5, 10, 1.0, 1.0), ("b", 5, 10, 1.0, 1.0)],
                  [[0, 1, 2], [1, 0.5, 3], [2, 3, 0.25]], [1, 1],
                  energy="moore" if D == 2 else "twenty_six")
    rng = np.random.default_rng(100 + D)
    lat = np.zeros((side,) * D, dtype=np.uint32)
    lat.flat[0] = 1
    lat.flat[-1] = 2
    sim = model.oracle(lattice=lat, cell_type_of=[0, 1])
    eng = _engine(model, lattice=lat, cell_type_of=[0, 1])
    for rep in range(3):
        noise = rng.integers(0, 3, size=lat.shape).astype(np.uint32)
        ref = model.oracle(lattice=lat, cell_type_of=[0, 1])
        # write an arbitrary (not necessarily connected) state on both sides
        pad = np.zeros_like(ref.padded())
        st = ref.strides()
        idx = np.indices(noise.shape).reshape(D, -1)
        flat = sum((idx[d] + 1) * st[d] for d in range(D))
        pad[flat] = noise.ravel()
        # periodic halo: copy opposite faces
        pdims = [g + 2 for g in model.grid]
        full = pad.reshape(pdims)
        inner = noise
        full[...] = np.pad(inner, 1, mode="wrap")
        pad = full.ravel().copy()
        vol = np.array([0, 1000, 1000], dtype=np.uint32)
        itf = np.array([0, 500, 500], dtype=np.uint32)
        sim.set_state(pad, vol[1:], itf[1:])
        eng.write_state(pad, vol, itf)
        t = random_interior_targets(sim, 30000, rng)
        k = rng.integers(0, 2 * D, t.size)
        u = rng.random(t.size)
        _compare(eng.evaluate_moves(t, k, u), sim.evaluate_moves(t, k, u))


@pytest.mark.parametrize("name", ["c1_periodic", "c1_fixed", "odd_periodic", "3d_26", "3d_18_fixed"])
def test_commit_bookkeeping_parity(name, cuda_required):
    """The device commit (dynamics.rs:23-183: sigma + halo, V, I, unwrapped
    position sums) applies the same accepted moves to the same effect."""
    model = MODELS[name]()
    sim = model.oracle()
    sim.run_mcs(10 if model.D == 2 else 2)
    eng = _engine(model)
    v, i, sp, so = padded_cells(sim)
    eng.write_state(sim.padded(), v, i, sp, so)
    rng = np.random.default_rng(9)
    applied = 0
    for _ in range(40):
        t = random_interior_targets(sim, 4000, rng)
        k = rng.integers(0, 2 * model.D, t.size)
        rec = sim.evaluate_moves(t, k, np.zeros(t.size))
        ok = np.flatnonzero((rec["evaluated"] == 1) & (rec["losing"] != 0) | (rec["evaluated"] == 1) & (rec["gaining"] != 0))
        if ok.size == 0:
            continue
        j = ok[0]
        sim.commit(rec["target_flat"][j], rec["losing"][j], rec["gaining"][j], rec["delta_h"][j])
        eng.commit_moves([rec["target_flat"][j]], [rec["gaining"][j]])
        applied += 1
    assert applied > 20
    gv, gi, gsp, gso = eng.cells()
    v, i, sp, so = padded_cells(sim)
    assert np.array_equal(eng.padded(), sim.padded())
    assert np.array_equal(gv, v) and np.array_equal(gi, i)
    assert np.array_equal(gsp, sp) and np.array_equal(gso, so)


@pytest.mark.parametrize("name", ["c1_periodic", "c1_fixed", "sorting_moore", "odd_periodic", "3d_26", "3d_18_fixed",
                                  "3d_vn", "sorting_vn_energy"])
def test_sweep_keeps_exact_state(name, cuda_required):
    """After device sweeps, V and I equal a full recount (checker.rs:36-83),
    the periodic halo mirrors the interior, position sums agree with the
    lattice modulo the box, and the device energy equals the oracle's global
    energy of the same lattice."""
    model = MODELS[name]()
    eng = _engine(model)
    n = 60 if model.D == 2 else 8
    eng.run_mcs(n)
    eng.synchronize()
    ok, rv, ri = eng.recount_check()
    assert ok
    st = eng.stats()
    info = eng.info[0]
    assert st["attempts"] == n * int(info.n_sites)
    assert st["accepted"] > 0 and st["evaluated"] >= st["accepted"]
    lat = eng.lattice()
    pad = eng.padded()
    pdims = [int(info.padded_dims[d]) for d in range(model.D)]
    if model.boundary == "periodic":
        assert np.array_equal(pad.reshape(pdims), np.pad(lat, 1, mode="wrap"))
    else:
        assert np.array_equal(pad.reshape(pdims), np.pad(lat, 1, mode="constant"))
    v, i, sp, so = eng.cells()
    coords = np.indices(lat.shape)
    for cid in range(1, int(info.n_cells) + 1):
        mask = lat == cid
        for d in range(model.D):
            assert (int(sp[cid, d]) - int(coords[d][mask].sum())) % model.grid[d] == 0
    # energy: oracle global energy over the device's state
    ref = model.oracle(lattice=lat, cell_type_of=np.asarray(model.oracle().type_of()))
    e_dev = eng.energy()
    e_ref = ref.global_energy()
    assert abs(e_dev - e_ref) <= 1e-9 * max(1.0, abs(e_ref))


def test_sweep_is_deterministic(cuda_required):
    model = sorting_model(side=40, seed=8)
    a = _engine(model)
    b = _engine(model)
    a.run_mcs(30)
    b.run_mcs(15)
    b.run_mcs(15)
    a.synchronize()
    b.synchronize()
    assert np.array_equal(a.lattice(), b.lattice())
    assert a.energy() == b.energy()


def test_batch_engine_matches_single_engines(cuda_required):
    """A simulation gives the same trajectory alone and among others of
    different sizes and dimensionality (counter-based RNG, one CTA each)."""
    from cpm import _cpm

    models = [c1_model(seed=3), sorting_model(side=40, seed=9), organoid_model(side=14, counts=(4, 4)),
              Model((31, 29), "periodic", [("a", 30, 40, 4.0, 0.9)], [[0, 6.1], [6.1, 1.3]], [6], seed=6)]
    many = _cpm.Engine([m.builder() for m in models])
    many.run_mcs(20)
    many.synchronize()
    for i, m in enumerate(models):
        one = _engine(m)
        one.run_mcs(20)
        one.synchronize()
        assert np.array_equal(one.lattice(), many.lattice(i)), i


@pytest.mark.parametrize("name", ["c1_periodic", "sorting_moore", "3d_26"])
def test_global_memory_sweep_keeps_exact_state(name, cuda_required, monkeypatch):
    """The global-memory sweep (used for lattices too large for shared
    memory) keeps the same invariants as the resident sweep."""
    monkeypatch.setenv("CPM_GPU_FORCE_GLOBAL", "1")
    model = MODELS[name]()
    eng = _engine(model)
    eng.run_mcs(20 if model.D == 2 else 4)
    eng.synchronize()
    ok, _, _ = eng.recount_check()
    assert ok
    st = eng.stats()
    assert st["accepted"] > 0


TILED_MODELS = {
    "tiled_2d_periodic": lambda: sorting_model(side=64, seed=12),
    "tiled_2d_fixed": lambda: Model((64, 64), "fixed", [("a", 50, 30, 5.0, 1.0), ("b", 50, 30, 5.0, 1.0)],
                                    [[0, 16, 16], [16, 3.3, 9.1], [16, 9.1, 2.7]], [25, 25], seed=13),
    "tiled_3d_periodic": lambda: organoid_model(side=32, counts=(30, 30), seed=14),
    "tiled_3d_fixed": lambda: organoid_model(side=32, boundary="fixed", energy="eighteen", counts=(20, 20), seed=15),
    # odd periodic sides: a third site colour for the last coordinate of each odd axis
    "tiled_2d_odd_periodic": lambda: Model((65, 63), "periodic", [("a", 50, 30, 5.0, 1.0), ("b", 50, 30, 5.0, 1.0)],
                                           [[0, 16, 16], [16, 3.3, 9.1], [16, 9.1, 2.7]], [25, 25], seed=18),
    "tiled_3d_odd_periodic": lambda: Model((33, 31, 35), "periodic", [("a", 60, 90, 2.0, 0.5), ("b", 60, 90, 2.0, 0.5)],
                                           [[0, 16, 16], [16, 4, 9], [16, 9, 5]], [30, 30], energy="twenty_six",
                                           seed=19),
    # the headline shapes at full size: the 512x512 sorting lattice (24x24
    # tiles, 4196 cells) and a 96^3 organoid (10^3 tiles)
    "tiled_2d_512_sorting": lambda: sorting_model(side=512, seed=22),
    "tiled_3d_96_organoid": lambda: organoid_model(side=96, counts=(400, 400), vol=100, seed=23),
}


@pytest.mark.parametrize("name", sorted(TILED_MODELS))
def test_tiled_sweep_keeps_exact_state(name, cuda_required, monkeypatch):
    """The tiled cooperative sweep (large lattices): exact V/I, consistent
    halo and position sums, device energy = oracle energy, deterministic."""
    monkeypatch.setenv("CPM_GPU_FORCE_TILED", "1")
    model = TILED_MODELS[name]()
    eng = _engine(model)
    n = 30 if model.D == 2 else 6
    eng.run_mcs(n)
    eng.synchronize()
    ok, _, _ = eng.recount_check()
    assert ok
    st = eng.stats()
    info = eng.info[0]
    assert st["attempts"] == n * int(info.n_sites), st
    assert st["accepted"] > 0
    assert st["spin_timeouts"] == 0
    assert st["deferred"] <= 0.001 * st["nonnull"], st
    lat = eng.lattice()
    pdims = [int(info.padded_dims[d]) for d in range(model.D)]
    mode = "wrap" if model.boundary == "periodic" else "constant"
    assert np.array_equal(eng.padded().reshape(pdims), np.pad(lat, 1, mode=mode))
    v, i, sp, so = eng.cells()
    coords = np.indices(lat.shape)
    for cid in range(1, int(info.n_cells) + 1):
        mask = lat == cid
        for d in range(model.D):
            assert (int(sp[cid, d]) - int(coords[d][mask].sum())) % model.grid[d] == 0
    ref = model.oracle(lattice=lat, cell_type_of=np.asarray(model.oracle().type_of()))
    assert abs(eng.energy() - ref.global_energy()) <= 1e-9 * max(1.0, abs(ref.global_energy()))
    again = _engine(model)
    again.run_mcs(n // 2)
    again.run_mcs(n - n // 2)
    again.synchronize()
    assert np.array_equal(again.lattice(), lat)


@pytest.mark.parametrize("D", [2, 3, "2odd"])
def test_tiled_sweep_independent_of_grid(D, cuda_required, monkeypatch):
    """Tiles, claims and priorities are functions of (seed, MCS, tile id): a
    grid with several tiles per CTA gives the same trajectory as one tile
    per CTA."""
    monkeypatch.setenv("CPM_GPU_FORCE_TILED", "1")
    if D == "2odd":
        model = Model((129, 127), "periodic", [("a", 50, 30, 5.0, 1.0)], [[0, 12], [12, 3]], [200], seed=20)
    else:
        model = sorting_model(side=128, seed=16) if D == 2 else organoid_model(side=64, counts=(60, 60), seed=17)
    n = 3 if D == 3 else 12
    wide = _engine(model)
    wide.run_mcs(n)
    wide.synchronize()
    monkeypatch.setenv("CPM_GPU_TILED_GRID", "3")
    narrow = _engine(model)
    narrow.run_mcs(n)
    narrow.synchronize()
    assert np.array_equal(wide.lattice(), narrow.lattice())
    a, b = wide.stats(), narrow.stats()
    for k in ("attempts", "nonnull", "accepted", "evaluated", "deferred", "rounds"):
        assert a[k] == b[k], (k, a[k], b[k])
    ok, _, _ = narrow.recount_check()
    assert ok
    assert np.array_equal(wide.cells()[2], narrow.cells()[2])



def test_grid_tuner_trials_leave_the_trajectory_unchanged(cuda_required, monkeypatch):
    """The tiled sweep's grid tuner times its candidate grids on the run's own
    first MCS (short trial launches, each candidate twice) and keeps the
    fastest: the run equals one with the grid fixed, and one with tuning off.
    The 132x120 shape is used by no other test, so this process has not tuned
    it yet."""
    from cpm import _cpm

    monkeypatch.setenv("CPM_GPU_FORCE_TILED", "1")
    model = sorting_model(side=64, seed=21)
    model = Model((132, 120), "periodic", model.types, model.adhesion, [60] * 4, seed=21)
    n = 100
    tuned = _engine(model)
    tuned.run_mcs(n)
    tuned.synchronize()
    rep = [e for e in _cpm.tuning_report() if e["dim"] == 2 and e["done"] and e["tiles_per_axis"][:2] == [8, 8]
           and len(e["candidates"]) > 1]
    assert rep, _cpm.tuning_report()
    grid = rep[0]["grid"]
    assert grid in [c[0] for c in rep[0]["candidates"]]
    assert all(c[1] > 0 for c in rep[0]["candidates"])
    others = []
    monkeypatch.setenv("CPM_GPU_NO_TUNE", "1")
    others.append(_engine(model))
    monkeypatch.setenv("CPM_GPU_TILED_GRID", "5")
    others.append(_engine(model))
    for e in others:
        e.run_mcs(n)
        e.synchronize()
        assert np.array_equal(tuned.lattice(), e.lattice())
        a, b = tuned.stats(), e.stats()
        for k in ("attempts", "nonnull", "accepted", "evaluated", "deferred"):
            assert a[k] == b[k], (k, a[k], b[k])
        assert np.array_equal(tuned.cells()[2], e.cells()[2])
    assert tuned.recount_check()[0]


def test_tiled_barrier_timeout_is_reported_and_the_context_survives(cuda_required, monkeypatch):
    """The grid barrier's bounded wait: with a barrier that waits for one CTA
    more than the grid has (test hook), every CTA gives up after its time
    limit, the kernel records the timeout and returns, the host reports
    CPM_E_TIMEOUT, and the next launch on the same context runs normally."""
    from cpm import _cpm

    monkeypatch.setenv("CPM_GPU_FORCE_TILED", "1")
    model = sorting_model(side=64, seed=12)
    monkeypatch.setenv("CPM_GPU_TEST_BARRIER_TIMEOUT", "1")
    bad = _engine(model)
    bad.run_mcs(1)
    with pytest.raises(_cpm.CPMRuntimeError, match="timed out"):
        bad.synchronize()
    assert bad.stats()["spin_timeouts"] >= 1
    monkeypatch.delenv("CPM_GPU_TEST_BARRIER_TIMEOUT")
    good = _engine(model)
    good.run_mcs(5)
    good.synchronize()
    assert good.stats()["spin_timeouts"] == 0
    assert good.recount_check()[0]


def test_tiled_sweep_with_more_cells_than_16_bits(cuda_required):
    """The tiled sweep stages box-local cell slots, so a lattice may hold any
    number of cells: 70,000 on 1024 x 1024 (beyond 16-bit ids) run exactly
    (V/I recount, position sums against the lattice, adhesion energy
    against a direct count)."""
    model = Model((1024, 1024), "periodic", [("a", 12, 14, 2.0, 0.5)], [[0, 6], [6, 2]], [70000], seed=21)
    eng = _engine(model, warn=False)
    assert eng.info[0].n_cells == 70000
    eng.run_mcs(4)
    eng.synchronize()
    ok, _, _ = eng.recount_check()
    assert ok
    st = eng.stats()
    assert st["attempts"] == 4 * 1024 * 1024 and st["accepted"] > 0 and st["spin_timeouts"] == 0
    lat = eng.lattice()
    v, i, sp, so = eng.cells()
    ids = lat.ravel().astype(np.int64)
    coords = np.indices(lat.shape).reshape(2, -1)
    for d in range(2):
        sums = np.bincount(ids, weights=coords[d], minlength=70001)
        assert np.all((sp[1:, d].astype(np.int64) - sums[1:].astype(np.int64)) % 1024 == 0)
    # global energy: volume and interface terms from the recounted V/I, plus
    # J over each unordered pair of Moore neighbours with different owners
    e_vi = np.sum(2.0 * (v[1:].astype(np.float64) - 12) ** 2 + 0.5 * (i[1:].astype(np.float64) - 14) ** 2)
    e_adh = 0.0
    for dr, dc in ((0, 1), (1, -1), (1, 0), (1, 1)):
        nb = np.roll(np.roll(lat, -dr, axis=0), -dc, axis=1)
        diff = lat != nb
        both = diff & (lat != 0) & (nb != 0)
        e_adh += 2.0 * both.sum() + 6.0 * (diff & ~both).sum()
    assert abs(eng.energy() - (e_vi + e_adh)) <= 1e-9 * (e_vi + e_adh)
