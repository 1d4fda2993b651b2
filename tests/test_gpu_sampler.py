"""Same-state parity of the sampler: a state the oracle reached is written
into an engine, `cpm_engine_take_sample` reads it out, and every per-cell
readout of output.rs:147-231 / 289-302 (id, volume, interface, centroid
Sigma x / V, the sorted eigenvalues of the gyration tensor, R_g^2 and
kappa^2) must equal the oracle's `take_sample` of the same state to 1e-12
relative; the sample's energy is the global energy of that state.

The oracle's position sums carry the reference's bookkeeping quirk (a lost
site is removed at its raw coordinate, a gained one added at its nearest
periodic image), so periodic runs also cover shifted sums and gyration
tensors far from a cell's true shape.
"""

import numpy as np
import pytest

from helpers import Model, organoid_model, padded_cells, sorting_model

pytestmark = pytest.mark.gpu

CASES = {
    "2d_periodic_sorting": (lambda: sorting_model(side=64, seed=41), 300),
    "2d_fixed": (lambda: Model((36, 30), "fixed", [("a", 40, 30, 3.0, 0.6)], [[0, 6.5], [6.5, 2.2]], [12],
                               seed=42), 400),
    "2d_periodic_few_large": (lambda: Model((40, 40), "periodic", [("a", 300, 80, 2.0, 0.5)], [[0, 4], [4, 9]],
                                            [3], seed=43), 2000),
    "3d_periodic": (lambda: organoid_model(side=16, counts=(6, 6), seed=44), 200),
    "3d_fixed": (lambda: organoid_model(side=14, counts=(4, 4), seed=45, boundary="fixed"), 200),
}


def _close(got, want, what):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    scale = max(1.0, float(np.max(np.abs(want))) if want.size else 1.0)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12 * scale, err_msg=what)


@pytest.mark.parametrize("name", list(CASES))
def test_take_sample_equals_the_oracle_on_the_same_state(name, cuda_required):
    from cpm import _cpm

    make, mcs = CASES[name]
    model = make()
    sim = model.oracle()
    sim.run_mcs(mcs)
    D = model.D
    v, i, sp, so = padded_cells(sim)
    eng = _cpm.Engine(model.builder(warn=False))
    eng.write_state(sim.padded(), v, i, sp, so)
    got = eng.take_sample()
    want = sim.take_sample()
    cells = want["cells"]
    n = len(cells)
    assert list(got.ids) == list(cells["id"])
    assert np.array_equal(np.asarray(got.volume), cells["volume"])
    assert np.array_equal(np.asarray(got.interface), cells["interface"])
    _close(np.asarray(got.centroid).reshape(n, D), cells["centroid"][:, :D], "centroid")
    _close(np.asarray(got.eigenvalues).reshape(n, D), cells["eigenvalues"][:, :D], "eigenvalues")
    _close(got.radius_of_gyration_sq, cells["rg2"], "radius_of_gyration_sq")
    _close(got.kappa_sq, cells["kappa2"], "kappa_sq")
    e = sim.global_energy()
    assert abs(got.conservative_energy - e) <= 1e-9 * max(1.0, abs(e))


def test_take_sample_on_shifted_position_sums(cuda_required):
    """Position sums shifted by a whole box on one axis (what the reference's
    quirk produces once a cell crosses the seam): the readouts still follow
    the formulas on those sums, as the oracle's do."""
    import oracle as O

    from cpm import _cpm

    model = Model((24, 24), "periodic", [("a", 30, 30, 1.0, 0.5)], [[0, 4], [4, 9]], [2], seed=46)
    sim = model.oracle()
    sim.run_mcs(50)
    v, i, sp, so = padded_cells(sim)
    # as if one site of cell 1 at x = 5 had been added at its image x = 29
    sp2, so2 = sp.copy(), so.copy()
    sp2[1, 0] += 24
    so2[1, 0, 0] += 29 * 29 - 5 * 5
    so2[1, 0, 1] += 24 * 7
    so2[1, 1, 0] += 24 * 7
    eng = _cpm.Engine(model.builder(warn=False))
    eng.write_state(sim.padded(), v, i, sp2, so2)
    got = eng.take_sample()
    D = 2
    for k in range(len(v) - 1):
        cen = sp2[k + 1] / float(v[k + 1])
        eig, rg2, kap = O.shape_descriptors(D, so2[k + 1], int(v[k + 1]), cen)
        _close(np.asarray(got.centroid).reshape(-1, D)[k], cen, "centroid")
        _close(np.asarray(got.eigenvalues).reshape(-1, D)[k], eig[:D], "eigenvalues")
        _close([got.radius_of_gyration_sq[k]], [rg2], "rg2")
        _close([got.kappa_sq[k]], [kap], "kappa2")
