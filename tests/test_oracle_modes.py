"""The oracle's restatement of the loop's other modes, checked on the CPU.

* The Act term (energy.rs:329-471): the scenarios of the reference's own
  unit tests (energy.rs:955-1300: two cells on a 6x6 grid, hand-set
  acquisition MCS, MCS = 20, lambda_act = [2, 3], max_act = [10, 20]) against
  an independent coordinate-space formula, as those tests do
  (`reference_act_delta`, energy.rs:1031-1098).
* Metropolis-Hastings acceptance (monte_carlo.rs:168-196): the oracle's
  decisions with given draws against the formula evaluated here from the
  lattice (copy-neighbour counts of the losing and gaining cells).
"""

import math

import numpy as np
import pytest

import oracle as O

GRID = 6
LAMBDA_ACT = [2.0, 3.0]
MAX_ACT = [10, 20]
MCS = 20


def _two_type_spec(periodic, act=True, acceptance="metropolis"):
    return O.ModelSpec((GRID, GRID), periodic, [(3, 8, 1.0, 0.5), (3, 8, 1.0, 0.5)], [[0, 2, 2], [2, 1, 3], [2, 3, 1]],
                       cell_counts=[1, 1], energy="moore", acceptance=acceptance,
                       act=list(zip(LAMBDA_ACT, MAX_ACT)) if act else None)


def _sim(periodic, cells, types=(0, 1), **kw):
    """cells: {id: [(r, c), ...]} placed explicitly."""
    spec = _two_type_spec(periodic, **kw)
    spec.cell_counts = [0, 0]
    sim = O.OracleSim(spec, 1)
    lat = np.zeros((GRID, GRID), np.uint32)
    for cid, sites in cells.items():
        for r, c in sites:
            lat[r, c] = cid
    sim.init_explicit(lat, list(types))
    return sim, lat


def _pflat(r, c):
    return (r + 1) * (GRID + 2) + (c + 1)


def _reference_act_delta(lat, periodic, births, mcs, target, source, type_of):
    """The independent formula of energy.rs:1031-1098, in coordinates."""
    losing, gaining = int(lat[target]), int(lat[source])
    if gaining == 0:
        return 0.0
    ty = type_of[gaining - 1]
    mx, lam = MAX_ACT[ty], LAMBDA_ACT[ty]

    def owner_birth(rc):
        return int(lat[rc]), births.get(rc, 0)

    def gm(site, relevant):
        members = [owner_birth(site)]
        for dr, dc in ((-1, 0), (1, 0), (0, -1), (0, 1)):
            r, c = site[0] + dr, site[1] + dc
            if periodic:
                members.append(owner_birth((r % GRID, c % GRID)))
            elif r < 0 or r >= GRID or c < 0 or c >= GRID:
                members.append((0, 0))
            else:
                members.append(owner_birth((r, c)))
        prod, cnt = 1.0, 0
        for owner, birth in members:
            if owner != relevant:
                continue
            prod *= float(max(0, mx - max(0, mcs - birth)))
            cnt += 1
        return 0.0 if cnt == 0 else prod ** (1.0 / cnt)

    return -(lam / mx) * (gm(source, gaining) - gm(target, losing))


def _set_births(sim, births, periodic):
    b = np.zeros((GRID + 2) ** 2, np.uint32)
    for (r, c), v in births.items():
        b[_pflat(r, c)] = v
    sim.set_act_state(b, MCS)


TWO_CELLS = {1: [(1, 1), (1, 2), (2, 1)], 2: [(2, 2), (2, 3), (3, 2)]}


@pytest.mark.parametrize("periodic", [False, True])
def test_act_hand_built_matches_the_independent_formula(periodic):
    sim, lat = _sim(periodic, TWO_CELLS)
    births = {(2, 1): 15, (1, 1): 12, (2, 2): 18, (3, 2): 10, (2, 3): 19}
    _set_births(sim, births, periodic)
    got = sim.act_delta(_pflat(2, 1), _pflat(2, 2))
    want = _reference_act_delta(lat, periodic, births, MCS, (2, 1), (2, 2), [0, 1])
    assert abs(got - want) < 1e-9 and abs(got) > 1e-6


def test_act_zero_activity_zeroes_the_mean_and_gaining_medium_zeroes_delta():
    sim, lat = _sim(False, TWO_CELLS)
    births = {(2, 2): 18, (3, 2): 0, (2, 3): 19}  # (3,2) fully decayed: elapsed 20 >= max_act 20
    _set_births(sim, births, False)
    got = sim.act_delta(_pflat(2, 1), _pflat(2, 2))
    want = _reference_act_delta(lat, False, births, MCS, (2, 1), (2, 2), [0, 1])
    assert abs(got - want) < 1e-9
    assert sim.act_delta(_pflat(1, 1), _pflat(0, 1)) == 0.0  # the medium invades: no Act term


def test_act_losing_medium_uses_decayed_medium_activity():
    sim, lat = _sim(False, {1: [(2, 3)]}, types=(0,))
    births = {(2, 2): 18, (1, 2): 17, (3, 2): 16, (2, 1): 15}
    _set_births(sim, births, False)
    got = sim.act_delta(_pflat(2, 2), _pflat(2, 3))
    want = _reference_act_delta(lat, False, births, MCS, (2, 2), (2, 3), [0])
    assert abs(got - want) < 1e-9 and got != 0.0


def test_act_periodic_reads_the_interior_through_the_halo():
    cells = {1: [(0, 1), (1, 1), (5, 1)], 2: [(0, 2), (1, 2), (0, 3)]}
    sim, lat = _sim(True, cells)
    births = {(0, 1): 14, (1, 1): 11, (5, 1): 17, (0, 2): 19, (1, 2): 13, (0, 3): 16}
    _set_births(sim, births, True)
    for target, source in (((0, 1), (0, 2)), ((0, 2), (0, 1))):
        got = sim.act_delta(_pflat(*target), _pflat(*source))
        want = _reference_act_delta(lat, True, births, MCS, target, source, [0, 1])
        assert abs(got - want) < 1e-9


def test_act_commit_sets_the_acquisition_mcs():
    sim, lat = _sim(False, TWO_CELLS)
    _set_births(sim, {}, False)
    tf, sf = _pflat(2, 1), _pflat(2, 2)
    sim.commit(tf, 1, 2, 0.0)
    assert sim.birth()[tf] == MCS


def test_metropolis_hastings_decisions_follow_the_formula():
    rng = np.random.default_rng(7)
    spec = O.ModelSpec((20, 20), True, [(12, 20, 1.0, 0.3), (12, 20, 1.5, 0.2)], [[0, 3, 3], [3, 1, 4], [3, 4, 1]],
                       cell_counts=[8, 8], acceptance="metropolis_hastings")
    sim = O.OracleSim(spec, 3)
    sim.set_local_halo(True)
    sim.init_default()
    sim.run_mcs(20)
    pad = sim.padded()
    st = sim.strides()
    copy = [st[0], -st[0], st[1], -st[1]]
    n = 4000
    t = ((rng.integers(0, 20, n) + 1) * st[0] + (rng.integers(0, 20, n) + 1) * st[1]).astype(np.int64)
    k = rng.integers(0, 4, n).astype(np.int32)
    u = rng.random(n)
    out = sim.evaluate_moves(t, k, u)
    checked = 0
    for i in range(n):
        o = out[i]
        if not o["evaluated"]:
            continue
        L, G = int(o["losing"]), int(o["gaining"])
        na = sum(int(pad[t[i] + c]) == L for c in copy)
        nb = sum(int(pad[t[i] + c]) == G for c in copy)
        if na == 0:
            want = False
        else:
            want = u[i] < min((na / nb) * math.exp(-float(o["delta_h"])), 1.0)
        assert bool(o["accepted"]) == want
        checked += 1
    assert checked > 100
