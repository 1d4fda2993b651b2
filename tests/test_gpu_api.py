"""The reference's Python-level behaviour (tests/python/test_builder.py,
test_batch.py, test_warnings.py, test_reproducibility.py) on the GB300
engine, through the drop-in `cpm` package.

The reference's frozen-trajectory check (test_reproducibility.py:72-83)
pins its CPU random stream; the GPU sweep draws from Philox on its own
chain, so that fixture is pinned against the oracle instead
(tests/test_oracle_kat.py) and here the same run is checked for
determinism, seed sensitivity and shape.
"""

import warnings

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATUSES = {"Ok", "CellLost", "Fragmented", "NotEquilibrated", "Degenerate"}


def _confluent(seed=1):
    import cpm

    sim = cpm.CPM(grid=(30, 30), boundary="periodic", seed=seed, copy_neighborhood="von_neumann",
                  connectivity_neighborhood="von_neumann")
    sim.register_cell_type(name="epithelial", target_volume=50, target_interface=75, lambda_volume=10.0,
                           lambda_interface=2.0)
    sim.add_cells(cell_type="epithelial", n=5)
    sim.set_adhesion([[0.0, 5.0], [5.0, 2.0]])
    return sim


def _two_types(seed=1):
    import cpm

    sim = cpm.CPM(grid=(20, 20), boundary="periodic", seed=seed)
    sim.register_cell_type(name="a", target_volume=9, target_interface=20, lambda_volume=1.0, lambda_interface=0.2)
    sim.register_cell_type(name="b", target_volume=9, target_interface=20, lambda_volume=1.5, lambda_interface=0.3)
    sim.add_cells("a", 2)
    sim.add_cells("b", 2)
    sim.set_adhesion([[0.0, 3.0, 3.0], [3.0, 1.0, 5.0], [3.0, 5.0, 1.0]])
    return sim


def test_run_shapes_dtypes_and_upper_triangular_contact(cuda_required):
    from cpm.warnings import CPMInitializationWarning

    with pytest.warns(CPMInitializationWarning):
        res = _confluent().run(burn_in_mcs=20, readout_mcs=50, sampling_interval_mcs=10)
    assert len(res.samples) == 5
    assert res.status.kind in STATUSES
    assert 0.0 < res.metadata.derived_phi <= 1.0
    assert isinstance(res.metadata.convention_hash, str) and len(res.metadata.convention_hash) == 64
    s = res.samples[-1]
    n = len(s.ids)
    assert n <= 5
    assert s.centroid.shape == (n, 2) and s.eigenvalues.shape == (n, 2)
    assert s.volume.dtype == np.uint32 and s.interface.dtype == np.uint32
    assert s.contact.shape == (n + 1, n + 1) and s.contact.dtype == np.uint32
    assert not np.tril(s.contact).any()
    assert [x.mcs for x in res.samples] == [30, 40, 50, 60, 70]


def test_lattice_snapshot_is_off_by_default_and_agrees_with_volumes(cuda_required):
    from cpm.warnings import CPMInitializationWarning

    with pytest.warns(CPMInitializationWarning):
        plain = _confluent().run(burn_in_mcs=5, readout_mcs=10, sampling_interval_mcs=5)
    assert plain.samples[0].lattice is None
    with pytest.warns(CPMInitializationWarning):
        snap = _confluent().run(burn_in_mcs=5, readout_mcs=10, sampling_interval_mcs=5, include_lattice=True)
    s = snap.samples[-1]
    assert s.lattice.shape == (30, 30) and s.lattice.dtype == np.uint32
    for cid, vol in zip(s.ids, s.volume):
        assert int((s.lattice == cid).sum()) == int(vol)
    # contact counts agree with the snapshot (von Neumann pairs seen once)
    assert int(s.contact.sum()) > 0


def test_cell_type_labels(cuda_required):
    import cpm
    from cpm.warnings import CPMInitializationWarning

    sim = cpm.CPM(grid=(30, 30), boundary="periodic", seed=3)
    for name in ("epithelial", "stem"):
        sim.register_cell_type(name=name, target_volume=30, target_interface=60, lambda_volume=1.0,
                               lambda_interface=1.0)
    sim.add_cells(cell_type="epithelial", n=3)
    sim.add_cells(cell_type="stem", n=2)
    sim.set_adhesion([[0.0, 1.0, 1.0], [1.0, 0.5, 1.0], [1.0, 1.0, 0.5]])
    with pytest.warns(CPMInitializationWarning):
        res = sim.run(burn_in_mcs=5, readout_mcs=5, sampling_interval_mcs=5)
    assert res.cell_type_names == ["epithelial", "stem"]
    assert sorted(np.asarray(res.cell_type_index).tolist()) == [0, 0, 0, 1, 1]


def test_same_seed_same_run_and_other_seed_diverges(cuda_required):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        a = _confluent(seed=7).run(burn_in_mcs=10, readout_mcs=10, sampling_interval_mcs=10)
        b = _confluent(seed=7).run(burn_in_mcs=10, readout_mcs=10, sampling_interval_mcs=10)
        c = _confluent(seed=8).run(burn_in_mcs=10, readout_mcs=10, sampling_interval_mcs=10)
    assert a.samples[0].conservative_energy == b.samples[0].conservative_energy
    assert np.array_equal(a.samples[0].volume, b.samples[0].volume)
    assert np.array_equal(a.samples[0].centroid, b.samples[0].centroid)
    assert a.metadata.model_hash == b.metadata.model_hash
    assert a.samples[0].conservative_energy != c.samples[0].conservative_energy


def test_explicit_fixture_run_is_reproducible(cuda_required):
    """The reference's reproducibility fixture (explicit 2x2 blocks, seed
    20260915, one 500-MCS readout chunk) run twice on the device."""
    import cpm

    def run(seed):
        lat = [0] * 900
        for r, c in [(6, 8), (6, 9), (7, 8), (7, 9)]:
            lat[r * 30 + c] = 1
        for r, c in [(18, 20), (18, 21), (19, 20), (19, 21)]:
            lat[r * 30 + c] = 2
        sim = cpm.CPM(grid=(30, 30), boundary="periodic", seed=seed, acceptance="metropolis")
        sim.register_cell_type("a", target_volume=12, target_interface=24, lambda_volume=1.0, lambda_interface=0.2)
        sim.register_cell_type("b", target_volume=12, target_interface=24, lambda_volume=1.2, lambda_interface=0.15)
        sim.add_cells("a", 1)
        sim.add_cells("b", 1)
        sim.set_adhesion([[0.0, 1.0, 1.5], [1.0, 0.5, 2.0], [1.5, 2.0, 0.5]])
        sim.initialize(lattice=lat, cell_type_of=[0, 1])
        return sim.run(burn_in_mcs=0, readout_mcs=500, sampling_interval_mcs=500)

    a, b, c = run(20260915), run(20260915), run(1)
    assert len(a.samples) == 1 and a.samples[0].mcs == 500
    assert list(a.samples[0].ids) == [1, 2]
    assert a.samples[0].conservative_energy == b.samples[0].conservative_energy
    assert np.array_equal(a.samples[0].volume, b.samples[0].volume)
    assert a.samples[0].conservative_energy != c.samples[0].conservative_energy


def test_run_batch_order_warning_hashes_and_seeds(cuda_required):
    from cpm import _cpm
    from cpm.warnings import CPMInitializationWarning

    sim = _two_types()
    base = sim.extract_theta()
    thetas = [base, [v * 1.1 for v in base], [v * 0.9 for v in base], base, base]
    with pytest.warns(CPMInitializationWarning) as rec:
        results = sim.run_batch(thetas, burn_in_mcs=5, readout_mcs=5, sampling_interval_mcs=5, master_seed=42)
    assert len([w for w in rec if issubclass(w.category, CPMInitializationWarning)]) == 1
    assert len(results) == len(thetas)
    assert all(r.status.kind in STATUSES for r in results)
    assert len({r.metadata.convention_hash for r in results}) == 1
    assert [r.metadata.seed for r in results] == [_cpm.derive_seed_u64(42, i) for i in range(len(thetas))]
    # identical theta, different seeds: different trajectories (placements)
    assert not np.array_equal(results[3].samples[0].centroid, results[4].samples[0].centroid)


def test_run_batch_member_equals_a_single_run_with_its_seed(cuda_required):
    """Member i of run_batch is the run of theta_i with seed
    derive_seed_u64(master_seed, i) (batch.rs:110-153)."""
    from cpm import _cpm

    sim = _two_types()
    sim.initialize(warn_on_default_init=False)
    base = sim.extract_theta()
    thetas = [base, [v * 1.25 for v in base]]
    batch = sim.run_batch(thetas, burn_in_mcs=20, readout_mcs=20, sampling_interval_mcs=10, master_seed=9)
    for i, th in enumerate(thetas):
        one = _cpm.CPM(grid=[20, 20], boundary="periodic", seed=_cpm.derive_seed_u64(9, i))
        one.register_cell_type("a", 9, 20, th[0], th[2])
        one.register_cell_type("b", 9, 20, th[1], th[3])
        one.add_cells("a", 2)
        one.add_cells("b", 2)
        one.set_adhesion([[th[4], th[5], th[6]], [th[5], th[7], th[8]], [th[6], th[8], th[9]]])
        one.initialize(warn_on_default_init=False)
        _, r = one.run(20, 20, 10)
        for sa, sb in zip(batch[i].samples, r.samples):
            assert sa.conservative_energy == sb.conservative_energy
            assert np.array_equal(sa.volume, sb.volume)
            assert np.array_equal(sa.centroid, sb.centroid)


def test_run_batch_warning_can_be_silenced(cuda_required):
    from cpm.warnings import CPMInitializationWarning

    sim = _two_types()
    sim.initialize(warn_on_default_init=False)
    base = sim.extract_theta()
    with warnings.catch_warnings():
        warnings.simplefilter("error", CPMInitializationWarning)
        sim.run_batch([base, base], burn_in_mcs=5, readout_mcs=5, sampling_interval_mcs=5, master_seed=1)


def test_default_placement_warning_policy(cuda_required):
    import cpm
    from cpm.warnings import CPMInitializationWarning

    def sim():
        s = cpm.CPM(grid=(20, 20), boundary="periodic", seed=1)
        s.register_cell_type(name="a", target_volume=20, target_interface=50, lambda_volume=1.0, lambda_interface=1.0)
        s.add_cells(cell_type="a", n=2)
        s.set_adhesion([[0.0, 1.0], [1.0, 0.5]])
        return s

    with pytest.warns(CPMInitializationWarning):
        sim().run(burn_in_mcs=1, readout_mcs=1, sampling_interval_mcs=1)
    quiet = sim()
    quiet.initialize(warn_on_default_init=False)
    with warnings.catch_warnings(record=True) as caught:
        warnings.simplefilter("always")
        quiet.run(burn_in_mcs=1, readout_mcs=1, sampling_interval_mcs=1)
    assert not any(issubclass(w.category, CPMInitializationWarning) for w in caught)
    explicit = cpm.CPM(grid=(4, 4), boundary="fixed", seed=1)
    explicit.register_cell_type(name="a", target_volume=1, target_interface=4, lambda_volume=1.0,
                                lambda_interface=1.0)
    explicit.set_adhesion([[0.0, 1.0], [1.0, 0.0]])
    lat = [0] * 16
    lat[5] = 1
    explicit.initialize(lattice=lat, cell_type_of=[0])
    with warnings.catch_warnings(record=True) as caught:
        warnings.simplefilter("always")
        res = explicit.run(burn_in_mcs=0, readout_mcs=1, sampling_interval_mcs=1)
    assert not any(issubclass(w.category, CPMInitializationWarning) for w in caught)
    assert len(res.samples) == 1


@pytest.mark.parametrize("name", ["2d_periodic", "2d_fixed", "3d_periodic"])
def test_topology_readouts_match_an_independent_count_and_the_oracle(name, cuda_required):
    """Contact graph (independent count over the snapshot), fragmented cells
    and medium components (the oracle's labelling of the same state)."""
    from helpers import Model, contact_reference, energy_offsets, organoid_model, sorting_model

    model = {"2d_periodic": lambda: sorting_model(side=40, seed=31),
             "2d_fixed": lambda: Model((36, 30), "fixed", [("a", 40, 30, 3.0, 0.6)], [[0, 6.5], [6.5, 2.2]], [12],
                                       seed=32),
             "3d_periodic": lambda: organoid_model(side=14, counts=(5, 5), seed=33)}[name]()
    from cpm import _cpm

    _, res = model.builder(warn=False).run(20, 40, 20, 1)
    sim = model.oracle()
    offsets = [tuple(int(v) for v in o) for o in energy_offsets(model)]
    for s in res.samples:
        lat = np.asarray(s.lattice)
        ref = contact_reference(lat, model.boundary == "periodic", offsets)
        a, b, n = s.contact_pairs
        got = {(int(x), int(y)): int(z) for x, y, z in zip(a, b, n)}
        assert got == dict(ref)
        mode = "wrap" if model.boundary == "periodic" else "constant"
        v = np.concatenate([[0], s.volume]).astype(np.uint32)
        i = np.concatenate([[0], s.interface]).astype(np.uint32)
        sim.set_state(np.pad(lat, 1, mode=mode).ravel(), v, i)
        want = sim.take_sample()
        assert list(s.fragmented_cells) == list(want["fragmented"])
        assert list(s.medium_component_volumes) == list(want["medium_volumes"])
        assert list(s.medium_component_touches_boundary) == list(want["medium_touches"])
