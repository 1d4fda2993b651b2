"""Initial state on the device (initialization.rs:61-137 and 396-436).

* Explicit placement: the lattice questions of place_explicit (an id beyond
  the cell count, a cell without a site, a cell whose sites are not
  connected under the von Neumann connectivity neighbourhood) answered on
  the device give the host restatement's verdict and message, in the
  reference's order of checks: on the reference's own error cases, on
  wrap-around connectivity, and on random lattices with planted faults.
  CPM_GPU_INIT_DEVICE_MIN_SITES picks the path (0: every explicit lattice
  on the device; a huge value: the host).
* Derived state: the volume, interface and position sums the device sums
  from each uploaded lattice equal the oracle's initial state, for default
  and explicit placements, 2D and 3D, periodic and fixed, alone and in a
  set of simulations.
"""

import numpy as np
import pytest

from helpers import Model, c1_model, organoid_model, padded_cells, sorting_model

pytestmark = pytest.mark.gpu

ON_DEVICE, ON_HOST = "0", str(2**62)


def _verdict(model, lattice, cell_type_of, monkeypatch, where):
    """(lattice, cell_type_of) accepted, or the error message."""
    monkeypatch.setenv("CPM_GPU_INIT_DEVICE_MIN_SITES", where)
    try:
        lat, cto, used = model.builder(lattice=lattice, cell_type_of=cell_type_of, warn=False).initial_state()
    except ValueError as e:
        return str(e)
    assert not used
    return (lat.copy(), cto.copy())


def _same_verdict(model, lattice, cell_type_of, monkeypatch):
    dev = _verdict(model, lattice, cell_type_of, monkeypatch, ON_DEVICE)
    host = _verdict(model, lattice, cell_type_of, monkeypatch, ON_HOST)
    if isinstance(host, str):
        assert dev == host, (dev, host)
    else:
        assert not isinstance(dev, str), dev
        assert np.array_equal(dev[0], host[0]) and np.array_equal(dev[1], host[1])
    return host


def test_reference_error_cases_on_the_device(cuda_required, monkeypatch):
    m = c1_model()
    lat = np.zeros((30, 30), dtype=np.uint32)
    lat[0, 0] = 1
    lat[5, 5] = 1
    assert "cell 1 is not connected under connectivity_neighborhood" in _same_verdict(m, lat, [0], monkeypatch)
    zero = np.zeros((30, 30), np.uint32)
    assert _same_verdict(m, zero, [0], monkeypatch) == "cell 1 has zero volume in the supplied lattice"
    bad = np.zeros((30, 30), np.uint32)
    bad[3, 4] = 2
    assert (_same_verdict(m, bad, [0], monkeypatch) ==
            "lattice references cell id 2, but cell_type_of only covers 1 cells")


def test_order_of_the_checks(cuda_required, monkeypatch):
    """The reference checks every id's range first (the first offending site
    in lattice order), then zero volumes (lowest id), then connectivity
    (lowest id)."""
    m = Model((40, 36), "periodic", [("a", 20, 20, 1.0, 1.0)], [[0, 1], [1, 1]], [8])
    lat = np.zeros((40, 36), np.uint32)
    for c in range(1, 9):
        lat[4 * c:4 * c + 3, 2:6] = c
    # cells 3 and 7 split, cell 5 missing, ids 9 then 12 out of range later in the scan
    split = lat.copy()
    split[30, 20] = 7
    split[12, 30] = 3
    assert "cell 3 is not connected" in _same_verdict(m, split, [0] * 8, monkeypatch)
    gone = split.copy()
    gone[gone == 5] = 0
    assert _same_verdict(m, gone, [0] * 8, monkeypatch) == "cell 5 has zero volume in the supplied lattice"
    far = gone.copy()
    far[39, 35] = 12
    far[38, 1] = 9
    assert (_same_verdict(m, far, [0] * 8, monkeypatch) ==
            "lattice references cell id 9, but cell_type_of only covers 8 cells")
    ok = _same_verdict(m, lat, [0] * 8, monkeypatch)
    assert not isinstance(ok, str)


@pytest.mark.parametrize("boundary", ["periodic", "fixed"])
def test_wrap_around_connectivity(boundary, cuda_required, monkeypatch):
    """A cell that touches itself only across the lattice edge is connected
    on a periodic lattice and not on a fixed one (2D and 3D)."""
    m2 = Model((30, 30), boundary, [("a", 20, 20, 1.0, 1.0)], [[0, 1], [1, 1]], [1])
    lat = np.zeros((30, 30), np.uint32)
    lat[10, 0] = lat[10, 29] = lat[11, 29] = 1
    v2 = _same_verdict(m2, lat, [0], monkeypatch)
    m3 = organoid_model(side=12, boundary=boundary, counts=(1, 1))
    lat3 = np.zeros((12, 12, 12), np.uint32)
    lat3[0, 5, 5] = lat3[11, 5, 5] = lat3[11, 6, 5] = 1
    lat3[6:8, 6:8, 6:8] = 2
    v3 = _same_verdict(m3, lat3, [0, 1], monkeypatch)
    for v in (v2, v3):
        if boundary == "periodic":
            assert not isinstance(v, str), v
        else:
            assert "cell 1 is not connected" in v


@pytest.mark.parametrize("D", [2, 3])
def test_random_lattices_with_planted_faults(D, cuda_required, monkeypatch):
    """Random box-shaped cells (connected), then one planted fault or none:
    a stray site of a cell, a removed cell, an id beyond the count, a cell
    cut in two; the device and host verdicts agree case by case."""
    rng = np.random.default_rng(31 + D)
    side = 48 if D == 2 else 20
    seen = set()
    for case in range(40):
        boundary = "periodic" if case % 2 == 0 else "fixed"
        shape = (side,) * D
        lat = np.zeros(shape, np.uint32)
        n = 0
        for _ in range(60 if D == 2 else 40):
            lo = rng.integers(0, side - 4, D)
            ext = rng.integers(1, 5, D)
            sl = tuple(slice(int(a), int(a + e)) for a, e in zip(lo, ext))
            if np.any(lat[sl]):
                continue
            n += 1
            lat[sl] = n
        kind = case % 5
        if kind == 1:
            free = np.argwhere(lat == 0)
            lat[tuple(free[rng.integers(len(free))])] = rng.integers(1, n + 1)
        elif kind == 2:
            lat[lat == rng.integers(1, n + 1)] = 0
        elif kind == 3:
            free = np.argwhere(lat == 0)
            lat[tuple(free[rng.integers(len(free))])] = n + 1 + rng.integers(0, 3)
        elif kind == 4:
            c = int(rng.integers(1, n + 1))
            pts = np.argwhere(lat == c)
            cut = pts[:, 0] == pts[:, 0].min() + (pts[:, 0].max() - pts[:, 0].min()) // 2
            if pts[:, 0].max() - pts[:, 0].min() >= 2:
                lat[tuple(pts[cut].T)] = 0
        m = Model(shape, boundary, [("a", 20, 20, 1.0, 1.0)], [[0, 1], [1, 1]], [n],
                  energy="eighteen" if D == 3 else None)
        v = _same_verdict(m, lat, [0] * n, monkeypatch)
        seen.add("ok" if not isinstance(v, str) else v.split(" ")[0] + v.split(" ")[-1])
    assert len(seen) >= 3, seen


DERIVED = {
    "c1_default": lambda: (c1_model(seed=3), None),
    "fixed_2d_default": lambda: (Model((30, 34), "fixed", [("e", 50, 75, 10.0, 2.0)], [[0, 5], [5, 2]], [5], seed=2),
                                 None),
    "sorting_64": lambda: (sorting_model(side=64, seed=4), None),
    "sorting_odd": lambda: (Model((65, 63), "periodic", [("a", 50, 30, 5.0, 1.0), ("b", 50, 30, 5.0, 1.0)],
                                  [[0, 16, 16], [16, 3.3, 9.1], [16, 9.1, 2.7]], [25, 25], seed=18), None),
    "organoid_26": lambda: (organoid_model(side=20, seed=5), None),
    "organoid_fixed_18": lambda: (organoid_model(side=15, boundary="fixed", energy="eighteen", counts=(4, 3)), None),
    "explicit_3d_vn": lambda: (organoid_model(side=16, energy="von_neumann", counts=(2, 2)), "blocks"),
}


def _blocks(model):
    """Explicit lattice: one box per cell on a grid (all connected)."""
    lat = np.zeros(model.grid, np.uint32)
    n = sum(model.counts)
    for c in range(n):
        lo = [(c * 5) % (model.grid[0] - 4), ((c * 5) // (model.grid[0] - 4)) * 5 % (model.grid[1] - 4)] + \
             [2] * (model.D - 2)
        lat[tuple(slice(a, a + 3) for a in lo)] = c + 1
    return lat, [t for t, k in enumerate(model.counts) for _ in range(k)]


@pytest.mark.parametrize("name", sorted(DERIVED))
def test_derived_state_equals_the_oracles(name, cuda_required):
    from cpm import _cpm

    model, kind = DERIVED[name]()
    if kind == "blocks":
        lat, cto = _blocks(model)
        ref = model.oracle(lattice=lat, cell_type_of=cto)
        eng = _cpm.Engine(model.builder(lattice=lat, cell_type_of=cto, warn=False))
    else:
        ref = model.oracle()
        eng = _cpm.Engine(model.builder(warn=False))
    got = eng.cells()
    want = padded_cells(ref)
    for g, w, what in zip(got, want, ("volume", "interface", "sum_position", "sum_outer")):
        assert np.array_equal(np.asarray(g), np.asarray(w).reshape(np.asarray(g).shape)), what
    ok, _, _ = eng.recount_check()
    assert ok


def test_derived_state_of_a_set_of_simulations(cuda_required):
    """One launch sums every member of a set of different sizes: each equals
    its oracle initial state."""
    from cpm import _cpm

    models = [c1_model(seed=s) for s in (1, 2)] + [sorting_model(side=48, seed=7), organoid_model(side=14, seed=8)]
    eng = _cpm.Engine([m.builder(warn=False) for m in models])
    for i, m in enumerate(models):
        got = eng.cells(i)
        want = padded_cells(m.oracle())
        for g, w in zip(got, want):
            assert np.array_equal(np.asarray(g), np.asarray(w).reshape(np.asarray(g).shape))
