"""Device topology readouts (cpm_readout.cu) on arbitrary states.

`Engine.take_sample` reads one sample of whatever state `write_state` put on
the device; its contact graph must equal an independent count over the
lattice, and its fragmented cells and medium components (count, order,
volumes, fixed-boundary contact) the oracle's labelling of the same state
(labelling.rs:70-154 as output.rs:304-337 reads it). Random lattices fragment
almost every cell and cut the medium into many components; the structured
cases hold enclosed lumens, a split cell and boundary-touching medium.
"""

import zlib

import numpy as np
import pytest

from helpers import Model, contact_reference, energy_offsets

pytestmark = pytest.mark.gpu


def _model(grid, boundary, n, energy=None):
    # tiny targets so that the default placement of n cells always succeeds
    return Model(grid, boundary, [("a", 2, 4, 1.0, 0.5)], [[0, 3], [3, 1]], [n], energy=energy, seed=3)


def _padded(model, lat):
    return np.pad(lat, 1, mode="wrap" if model.boundary == "periodic" else "constant").ravel().astype(np.uint32)


def _check(model, lat):
    from cpm import _cpm

    lat = np.asarray(lat, dtype=np.uint32)
    n = model.counts[0]
    pad = _padded(model, lat)
    v = np.bincount(lat.ravel(), minlength=n + 1).astype(np.uint32)
    v[0] = 0
    i = np.zeros(n + 1, np.uint32)
    eng = _cpm.Engine(model.builder(warn=False))
    eng.write_state(pad, v, i)
    s = eng.take_sample(0, include_lattice=True)
    assert np.array_equal(np.asarray(s.lattice), lat)
    assert np.array_equal(np.asarray(s.volume), v[1:])
    offsets = [tuple(int(x) for x in o) for o in energy_offsets(model)]
    want = contact_reference(lat, model.boundary == "periodic", offsets)
    a, b, c = s.contact_pairs
    got = [(int(x), int(y), int(z)) for x, y, z in zip(a, b, c)]
    assert got == sorted((p, q, k) for (p, q), k in want.items())  # ascending (a, b)
    sim = model.oracle()
    sim.set_state(pad, v[1:], i[1:])
    ref = sim.take_sample()
    assert list(s.fragmented_cells) == list(ref["fragmented"])
    assert list(s.medium_component_volumes) == list(ref["medium_volumes"])
    assert list(s.medium_component_touches_boundary) == list(ref["medium_touches"])
    return s


CASES = {
    "random_2d_periodic": ((37, 29), "periodic", 40, None),
    "random_2d_fixed": ((31, 23), "fixed", 30, None),
    "random_2d_fixed_vn": ((26, 17), "fixed", 12, "von_neumann"),
    "random_3d_periodic_26": ((9, 7, 11), "periodic", 20, "twenty_six"),
    "random_3d_fixed_18": ((8, 10, 6), "fixed", 16, "eighteen"),
    "random_3d_periodic_vn": ((6, 5, 7), "periodic", 9, "von_neumann"),
    "small_periodic_2d": ((3, 4), "periodic", 2, None),
    "small_periodic_3d": ((3, 3, 4), "periodic", 3, "twenty_six"),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("density", [0.3, 0.8])
def test_random_states(name, density, cuda_required):
    grid, boundary, n, energy = CASES[name]
    model = _model(grid, boundary, n, energy)
    rng = np.random.default_rng(zlib.crc32(f"{name}/{density}".encode()))
    lat = rng.integers(1, n + 1, size=grid) * (rng.random(grid) < density)
    s = _check(model, lat)
    if density > 0.5 and min(grid) > 4:
        assert len(s.fragmented_cells) > 0


@pytest.mark.parametrize("boundary", ["periodic", "fixed"])
def test_lumens_split_cell_and_boundary_medium(boundary, cuda_required):
    model = _model((24, 20), boundary, 3)
    lat = np.zeros((24, 20), np.uint32)
    lat[2:12, 2:12] = 1  # a ring of cell 1 around two lumens
    lat[4:6, 4:6] = 0
    lat[7:10, 6:10] = 0
    lat[14:17, 3:6] = 2  # cell 2 in two pieces
    lat[19:22, 14:18] = 2
    lat[0:24, 16] = 3  # cell 3 cuts the medium into two bands (periodic: one with the wrap)
    s = _check(model, lat)
    assert list(s.fragmented_cells) == [2]
    vols, touches = list(s.medium_component_volumes), list(s.medium_component_touches_boundary)
    assert vols[-2:] == [4, 12] and touches[-2:] == [False, False]  # the lumens, in scan order
    if boundary == "fixed":
        assert len(vols) == 4 and touches[:2] == [True, True]  # the two bands on either side of cell 3
    else:
        assert len(vols) == 3 and not any(touches)  # the bands join across the periodic edge


def test_three_d_cavity(cuda_required):
    model = _model((10, 9, 8), "fixed", 2, "twenty_six")
    lat = np.zeros((10, 9, 8), np.uint32)
    lat[1:8, 1:8, 1:7] = 1  # a shell with a closed cavity
    lat[3:6, 3:6, 3:5] = 0
    lat[8:10, 0:3, 0:2] = 2
    s = _check(model, lat)
    vols = list(s.medium_component_volumes)
    touches = list(s.medium_component_touches_boundary)
    assert 18 in vols and touches[vols.index(18)] is False


@pytest.mark.parametrize("boundary", ["periodic", "fixed"])
def test_edge_states(boundary, cuda_required):
    """All medium (one component, no contacts); single-site cells on a
    checkerboard (every cell alone, the medium cut into diagonal pieces
    under von Neumann but one piece under the full stencil); a lattice full
    of cells (no medium component at all)."""
    n = 12
    model = _model((8, 6), boundary, n)
    s = _check(model, np.zeros((8, 6), np.uint32))
    assert list(s.fragmented_cells) == [] and len(s.medium_component_volumes) == 1
    lat = np.zeros((8, 6), np.uint32)
    ids = iter(range(1, n + 1))
    for r in range(0, 8, 2):
        for c in range(0, 6, 2):
            lat[r, c] = next(ids)
    _check(model, lat)
    full = (np.arange(48).reshape(8, 6) % n + 1).astype(np.uint32)
    s = _check(model, full)
    assert len(s.medium_component_volumes) == 0
