"""The serving loop (cpm_serve_*): continuous batching of whole simulations.

Each result must equal `CPM.run` for the same simulation and window, bit
for bit, whether the request ran alone or in a mix of others admitted and
retired around it; admission respects the slot and HBM limits; cancelled
and invalid requests are reported, not run.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("volume", "interface", "centroid", "eigenvalues", "radius_of_gyration_sq", "kappa_sq",
          "fragmented_cells", "medium_component_volumes", "medium_component_touches_boundary")


def _sim(kind, seed):
    import cpm

    if kind == "2d_small":
        s = cpm.CPM(grid=(48, 40), boundary="periodic", seed=seed)
        s.register_cell_type("a", 40, 30, 4.0, 0.8)
        s.add_cells("a", 12)
        s.set_adhesion([[0, 9.5], [9.5, 2.25]])
    elif kind == "2d_two_types":
        s = cpm.CPM(grid=(96, 96), boundary="fixed", seed=seed)
        s.register_cell_type("a", 50, 75, 6.0, 1.2)
        s.register_cell_type("b", 50, 75, 3.0, 0.7)
        s.add_cells("a", 40)
        s.add_cells("b", 40)
        s.set_adhesion([[0, 12, 14], [12, 3.3, 9.1], [14, 9.1, 2.7]])
    elif kind == "2d_large":  # beyond one SM's shared memory: the tiled sweep
        s = cpm.CPM(grid=(320, 320), boundary="periodic", seed=seed)
        s.register_cell_type("a", 50, 30, 5.0, 1.0)
        s.add_cells("a", 900)
        s.set_adhesion([[0, 16], [16, 5.5]])
    elif kind == "3d_small":
        s = cpm.CPM(grid=(20, 20, 20), boundary="periodic", seed=seed, energy_neighborhood="twenty_six")
        s.register_cell_type("a", 60, 90, 2.0, 0.5)
        s.add_cells("a", 20)
        s.set_adhesion([[0, 16], [16, 4.0]])
    else:
        raise KeyError(kind)
    s.initialize(warn_on_default_init=False)
    return s


WINDOWS = {"2d_small": (200, 300, 100), "2d_two_types": (100, 200, 50), "2d_large": (40, 60, 20),
           "3d_small": (20, 30, 10)}


def _same(a, b):
    assert len(a.samples) == len(b.samples)
    assert a.status.kind == b.status.kind
    assert a.metadata.model_hash == b.metadata.model_hash
    for sa, sb in zip(a.samples, b.samples):
        assert sa.mcs == sb.mcs
        assert np.float64(sa.conservative_energy).tobytes() == np.float64(sb.conservative_energy).tobytes()
        for f in FIELDS:
            x, y = np.asarray(getattr(sa, f)), np.asarray(getattr(sb, f))
            assert x.shape == y.shape and x.tobytes() == y.tobytes(), f
        assert np.array_equal(sa.contact, sb.contact)


def test_serve_results_equal_run_alone_and_in_a_mix(cuda_required):
    import cpm

    kinds = list(WINDOWS)
    want = {k: _sim(k, 5).run(*WINDOWS[k]) for k in kinds}
    # alone: one request at a time
    with cpm.Server() as srv:
        for k in kinds:
            t = srv.submit(_sim(k, 5), *WINDOWS[k])
            state, res, times = srv.wait(t)
            assert state == "done"
            _same(res, want[k])
            assert times["finished_s"] >= times["device_done_s"] >= times["admitted_s"] >= times["submitted_s"]
    # in a mix: extra requests interleaved, submitted while others run
    with cpm.Server(max_active=4) as srv:
        tickets = {}
        for i, k in enumerate(kinds * 2):
            seed = 5 if i < len(kinds) else 100 + i
            tickets[(k, seed)] = srv.submit(_sim(k, seed), *WINDOWS[k])
        for (k, seed), t in tickets.items():
            state, res, _ = srv.wait(t)
            assert state == "done"
            if seed == 5:
                _same(res, want[k])
        st = srv.stats()
        assert st["completed"] == 2 * len(kinds)
        assert 1 <= st["peak_active"] <= 4
        assert st["bytes_in_use"] == 0


def test_serve_admission_respects_the_hbm_budget(cuda_required):
    import cpm

    with cpm.Server(hbm_budget_bytes=1) as srv:  # below any request: one at a time
        ts = [srv.submit(_sim("2d_small", 20 + i), 0, 100, 50) for i in range(4)]
        for t in ts:
            state, _, times = srv.wait(t)
            assert state == "done"
        st = srv.stats()
        assert st["peak_active"] == 1
        assert st["completed"] == 4


def test_serve_cancel_and_errors(cuda_required):
    import cpm

    with cpm.Server(max_active=1) as srv:
        first = srv.submit(_sim("2d_two_types", 1), 2000, 2000, 100)
        second = srv.submit(_sim("2d_small", 2), 0, 100, 100)
        srv.cancel(first)
        state, res, _ = srv.wait(first)
        assert state == "cancelled" and res is None
        state, res, _ = srv.wait(second)
        assert state == "done"
        with pytest.raises(ValueError):
            srv.submit(_sim("2d_small", 3), 0, 100, 0)  # sampling interval must be positive
        with pytest.raises(ValueError):
            srv.poll(987654)
