"""Exact Boltzmann check of the oracle's chain (tests/exact_boltzmann.rs).

With Metropolis-Hastings acceptance (monte_carlo.rs:168-196), the
connectivity check of each attempt off (the harness calls
`attempt(cpm, false)`) and only conservative terms, the chain is reversible
with respect to exp(-H)/Z.  On lattices small enough to enumerate every
configuration, the visit histogram binned by the exact value of H must match
g(H) exp(-H)/Z, with g(H) the exactly enumerated degeneracy.  H here comes
from an independent count: Moore neighbourhood, fixed boundary, out-of-grid
slots counted as medium for both interface and adhesion (the harness's
`h_single_cell` / `h_two_cell`), no use of the oracle's energy code.

The two cases of the reference's harness, at its parameters:

* one cell on a 5x5 grid (2^25 - 1 configurations): lambda_V 0.15, V* 8,
  lambda_I 0.05, I* 20, no adhesion;
* two cells on a 4x4 grid (3^16 - 2^17 + 1 configurations with both cells
  present): lambda_V 0.05, V* 5, lambda_I 0.01, I* 14, J(cell, medium) 0.5,
  J(a, b) 0.8, and the harness's stiffer case with every coefficient doubled.

The statistic follows the harness: bins with expected count below 20 are
pooled into one tail bin, chi-squared against a blunt 8 df envelope (thinned
samples stay slightly autocorrelated), no bin with expected count >= 20 left
unvisited, and a floor on the number of distinct bins visited.  The sample
counts are smaller than the harness's (it runs 1-2M thinned samples per case,
marked ignored); four independent chains per case, pooled.  The thinned
samples also meet the independent-sample bound df + 6 sqrt(2 df), which is
asserted too.

A planted mistake shows the statistic has power: the same chain with plain
Metropolis acceptance (no n_A / n_B proposal ratio) is not reversible with
respect to exp(-H) and fails the envelope.
"""

from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import oracle as O

MIN_EXPECTED = 20.0

# Moore stencil (energy neighbourhood of the 2D harness)
MOORE = [(-1, -1), (-1, 0), (-1, 1), (0, -1), (0, 1), (1, -1), (1, 0), (1, 1)]


class Counter:
    """Counts of one configuration of `k` cells (owners 0..k, 0 = medium)
    on a rows x cols fixed-boundary grid, as an additive mixed-radix key:
    per cell its volume and its medium-or-wall contact slots, and for two
    cells the cell-cell contacts.  Built from per-row and row-pair tables so
    that 3^16 configurations enumerate in seconds."""

    def __init__(self, rows, cols, k):
        self.rows, self.cols, self.k = rows, cols, k
        sites = rows * cols
        # fields: V_1..V_k, W_1..W_k (cell-medium/wall pairs), N12
        self.radix = [sites + 1] * k + [8 * sites + 1] * k + ([8 * sites + 1] if k == 2 else [])
        self.mult = np.cumprod([1] + self.radix[:-1]).astype(np.int64)
        b = k + 1
        self.n_row = b ** cols
        self.digits = np.array([[(code // b ** x) % b for x in range(cols)] for code in range(self.n_row)], np.int64)
        self.row_key = np.stack([self._row_keys(y) for y in range(rows)])
        self.pair_key = self._pair_keys()

    def _pair(self, a, b):
        """Key increment of one unordered neighbouring pair with owners a, b
        (vectorised; 0 where a == b)."""
        k, m = self.k, self.mult
        inc = np.zeros(np.broadcast(a, b).shape, np.int64)
        diff = a != b
        for c in range(1, k + 1):
            inc += np.where(diff & (a == 0) & (b == c), m[k + c - 1], 0)
            inc += np.where(diff & (b == 0) & (a == c), m[k + c - 1], 0)
        if k == 2:
            inc += np.where(diff & (a != 0) & (b != 0), m[2 * k], 0)
        return inc

    def _row_keys(self, y):
        d, k, m = self.digits, self.k, self.mult
        key = np.zeros(self.n_row, np.int64)
        for c in range(1, k + 1):
            key += (d == c).sum(1) * m[c - 1]
        for x in range(self.cols - 1):
            key += self._pair(d[:, x], d[:, x + 1])
        for x in range(self.cols):
            in_grid = sum(1 for dy, dx in MOORE if 0 <= y + dy < self.rows and 0 <= x + dx < self.cols)
            for c in range(1, k + 1):
                key += np.where(d[:, x] == c, (8 - in_grid) * m[k + c - 1], 0)
        return key

    def _pair_keys(self):
        top, bot = self.digits[:, None, :], self.digits[None, :, :]
        key = np.zeros((self.n_row, self.n_row), np.int64)
        for x in range(self.cols):
            key += self._pair(top[..., x], bot[..., x])
            if x + 1 < self.cols:
                key += self._pair(top[..., x], bot[..., x + 1])
                key += self._pair(top[..., x + 1], bot[..., x])
        return key

    def keys_of(self, lattices):
        """Keys of configurations given as (n, rows, cols) owner arrays."""
        b = self.k + 1
        codes = (lattices.astype(np.int64) * (b ** np.arange(self.cols))).sum(2)
        key = self.row_key[np.arange(self.rows), codes].sum(1)
        for y in range(self.rows - 1):
            key += self.pair_key[codes[:, y], codes[:, y + 1]]
        return key

    def fields(self, key):
        return [(key // m) % r for m, r in zip(self.mult, self.radix)]

    def degeneracy(self):
        """(key, number of configurations) over every configuration."""
        keys, counts = [], []
        for r0 in range(self.n_row):
            acc = self.row_key[0, r0] + np.zeros(1, np.int64)
            last = np.array([r0])
            for y in range(1, self.rows):
                acc = (acc[:, None] + self.pair_key[last][:, :] + self.row_key[y][None, :]).ravel()
                last = np.tile(np.arange(self.n_row), acc.size // self.n_row)
            u, c = np.unique(acc, return_counts=True)
            keys.append(u)
            counts.append(c)
        u, inv = np.unique(np.concatenate(keys), return_inverse=True)
        return u, np.bincount(inv, weights=np.concatenate(counts)).astype(np.int64)


def energy(counter, key, lam_v, v_star, lam_i, i_star, j_medium, j_cells):
    """H of the configurations with these keys: adhesion over unordered
    neighbouring pairs (out-of-grid slots as medium) plus the volume and
    interface terms of every cell."""
    f = counter.fields(key)
    k = counter.k
    n12 = f[2 * k] if k == 2 else 0
    h = j_cells * n12 if k == 2 else np.zeros(key.shape)
    for c in range(k):
        h = h + j_medium[c] * f[k + c]
    for c in range(k):
        v, i = f[c], f[k + c] + n12
        h = h + lam_v[c] * (v - v_star[c]) ** 2 + lam_i[c] * (i - i_star[c]) ** 2
    return h


def valid(counter, key):
    f = counter.fields(key)
    return np.all([f[c] >= 1 for c in range(counter.k)], axis=0)


def chi_squared(exact_h, exact_g, sample_h):
    """The harness's statistic: (chi2, df, distinct bins visited, bins with
    expected >= 20 never visited)."""
    bins, inv = np.unique(exact_h.view(np.uint64), return_inverse=True)
    g = np.bincount(inv, weights=exact_g.astype(np.float64))
    hb = bins.view(np.float64)
    lw = np.log(g) - hb
    p = np.exp(lw - lw.max())
    p /= p.sum()
    n = sample_h.size
    expected = p * n
    sb, sc = np.unique(sample_h.view(np.uint64), return_counts=True)
    assert np.all(np.isin(sb, bins)), "a sampled energy is not an energy of any configuration"
    observed = np.zeros(bins.size)
    observed[np.searchsorted(bins, sb)] = sc
    big = expected >= MIN_EXPECTED
    chi2 = float((((observed - expected) ** 2) / np.where(big, expected, 1.0))[big].sum())
    df = int(big.sum())
    pe, po = expected[~big].sum(), observed[~big].sum()
    if pe >= MIN_EXPECTED:
        chi2 += (po - pe) ** 2 / pe
        df += 1
    df -= 1
    empty = int((big & (observed == 0)).sum())
    return chi2, df, int(sb.size), empty


def _chain(spec, lattice, seed, burn_in, n_samples, thin):
    sim = O.OracleSim(spec, seed)
    spec_cells = int(lattice.max())
    sim.init_explicit(lattice, list(range(spec_cells)))
    sim.set_check_topology(False)
    return sim.sample_attempts(burn_in, n_samples, thin)


def _sample(spec, lattice, seeds, burn_in, n_samples, thin):
    O.lib()
    with ThreadPoolExecutor(len(seeds)) as ex:
        parts = list(ex.map(lambda s: _chain(spec, lattice, s, burn_in, n_samples, thin), seeds))
    return np.concatenate(parts)


SINGLE = dict(lam_v=[0.15], v_star=[8.0], lam_i=[0.05], i_star=[20.0], j_medium=[0.0], j_cells=0.0)


def two_cell_params(scale):
    """The harness's two-cell parameters with lambda_V, lambda_I and every
    adhesion coefficient multiplied by `scale` (targets unchanged)."""
    return dict(lam_v=[0.05 * scale] * 2, v_star=[5.0, 5.0], lam_i=[0.01 * scale] * 2, i_star=[14.0, 14.0],
                j_medium=[0.5 * scale] * 2, j_cells=0.8 * scale)


def _spec(case, acceptance):
    p = SINGLE if case == "single" else two_cell_params(float(case.split("@")[1]) if "@" in case else 1.0)
    k = len(p["lam_v"])
    types = [(int(round(p["v_star"][c])), int(round(p["i_star"][c])), p["lam_v"][c], p["lam_i"][c]) for c in range(k)]
    if k == 1:
        adh = [[0.0, 0.0], [0.0, 0.0]]
    else:
        jm, jc, js = p["j_medium"][0], p["j_cells"], 0.2 * p["j_cells"] / 0.8
        adh = [[0.0, jm, jm], [jm, js, jc], [jm, jc, js]]
    grid = (5, 5) if k == 1 else (4, 4)
    return O.ModelSpec(grid, False, types, adh, cell_counts=[0] * k, energy="moore", acceptance=acceptance), p


def _start(case):
    if case == "single":
        lat = np.zeros((5, 5), np.uint32)
        lat[2, 2] = 1
    else:
        lat = np.zeros((4, 4), np.uint32)
        lat[1, 1], lat[2, 2] = 1, 2
    return lat


_EXACT = {}


def _exact(case):
    if case not in _EXACT:
        spec, p = _spec(case, "metropolis_hastings")
        counter = Counter(*spec.grid, len(p["lam_v"]))
        keys, g = counter.degeneracy()
        ok = valid(counter, keys)
        keys, g = keys[ok], g[ok]
        _EXACT[case] = (counter, keys, g, energy(counter, keys, **p))
    return _EXACT[case]


# (burn-in attempts, thinned samples per chain, attempts between samples,
#  floor on distinct energy bins visited)
RUNS = {"single": (200_000, 50_000, 40 * 25, 25), "two": (400_000, 20_000, 200 * 16, 250),
        "two@2.0": (400_000, 20_000, 200 * 16, 25)}
SEEDS = [1, 2, 3, 4]


def test_counter_matches_direct_count():
    """The table-built counts equal a direct per-site count (interface of
    each cell = its Moore slots holding another owner or outside the grid;
    adhesion over unordered pairs, wall pairs at J(cell, medium))."""
    rng = np.random.default_rng(3)
    for case in ("single", "two"):
        spec, p = _spec(case, "metropolis_hastings")
        k = len(p["lam_v"])
        R, C = spec.grid
        counter = Counter(R, C, k)
        lats = rng.integers(0, k + 1, (300, R, C))
        got = energy(counter, counter.keys_of(lats), **p)
        for n in range(lats.shape[0]):
            lat = lats[n]
            vol, itf, adh = [0] * k, [0] * k, 0.0
            jm = lambda a, b: 0.0 if a == b else (p["j_cells"] if a and b else p["j_medium"][max(a, b) - 1])
            for y in range(R):
                for x in range(C):
                    o = lat[y, x]
                    if o:
                        vol[o - 1] += 1
                    for dy, dx in MOORE:
                        yy, xx = y + dy, x + dx
                        inside = 0 <= yy < R and 0 <= xx < C
                        q = lat[yy, xx] if inside else 0
                        if o and q != o:
                            itf[o - 1] += 1
                        if q != o:
                            # pairs inside the grid are seen from both sides
                            adh += jm(o, q) * (0.5 if inside else 1.0)
            want = adh + sum(p["lam_v"][c] * (vol[c] - p["v_star"][c]) ** 2
                             + p["lam_i"][c] * (itf[c] - p["i_star"][c]) ** 2 for c in range(k))
            assert abs(got[n] - want) <= 1e-9 * max(1.0, abs(want)), (case, n, got[n], want)


@pytest.mark.parametrize("case", ["single", "two", "two@2.0"])
def test_oracle_energy_matches_independent_count(case):
    """Along a chain free to reshape (connectivity check off, so cells break
    into pieces), the oracle's running energy (initial energy plus every
    accepted delta-H) and its from-scratch global energy both equal H of the
    independent count, and its incremental V/I equal a recount."""
    spec, p = _spec(case, "metropolis_hastings")
    counter = Counter(*spec.grid, len(p["lam_v"]))
    sim = O.OracleSim(spec, 7)
    lat = _start(case)
    sim.init_explicit(lat, list(range(int(lat.max()))))
    sim.set_check_topology(False)
    pieces = 0
    for _ in range(200):
        cur = sim.sample_attempts(0, 1, 97)
        want = float(energy(counter, counter.keys_of(cur), **p)[0])
        assert abs(sim.energy - want) <= 1e-9 * max(1.0, abs(want)), (sim.energy, want)
        assert abs(sim.global_energy() - want) <= 1e-12 * max(1.0, abs(want)), (sim.global_energy(), want)
        bad, _ = sim.check()
        assert bad == 0
        pieces += int(_disconnected(cur[0]))
    assert pieces > 0  # the chain did visit disconnected shapes


def test_hand_built_two_cell_energies():
    """exact_boltzmann.rs:889-925: two diagonal singletons in opposite
    corners, two face-adjacent singletons, a 2x2 block beside a 2x1 block;
    the oracle's energy after placement equals the independent H."""
    spec, p = _spec("two", "metropolis_hastings")
    counter = Counter(4, 4, 2)
    a = np.zeros((4, 4), np.uint32)
    a[0, 0], a[3, 3] = 1, 2
    b = np.zeros((4, 4), np.uint32)
    b[1, 1], b[1, 2] = 1, 2
    c = np.zeros((4, 4), np.uint32)
    c[0:2, 0:2], c[0:2, 2] = 1, 2
    for lat in (a, b, c):
        sim = O.OracleSim(spec, 1)
        sim.init_explicit(lat, [0, 1])
        want = float(energy(counter, counter.keys_of(lat[None]), **p)[0])
        assert abs(sim.energy - want) < 1e-9 and abs(sim.global_energy() - want) < 1e-9, (lat, sim.energy, want)


def _disconnected(lat):
    """Some cell of the configuration has more than one von Neumann
    component."""
    R, C = lat.shape
    for c in range(1, int(lat.max()) + 1):
        sites = list(zip(*np.nonzero(lat == c)))
        if not sites:
            continue
        seen, stack = {sites[0]}, [sites[0]]
        while stack:
            y, x = stack.pop()
            for dy, dx in ((-1, 0), (1, 0), (0, -1), (0, 1)):
                q = (y + dy, x + dx)
                if 0 <= q[0] < R and 0 <= q[1] < C and lat[q] == c and q not in seen:
                    seen.add(q)
                    stack.append(q)
        if len(seen) != len(sites):
            return True
    return False


def test_degeneracy_totals():
    """Every configuration is counted once: 2^25 - 1 single-cell patterns,
    3^16 - 2 * 2^16 + 1 with both cells present."""
    _, _, g1, _ = _exact("single")
    assert int(g1.sum()) == 2 ** 25 - 1
    _, _, g2, _ = _exact("two")
    assert int(g2.sum()) == 3 ** 16 - 2 * 2 ** 16 + 1


@pytest.mark.parametrize("case", ["single", "two", "two@2.0"])
def test_chain_matches_exact_boltzmann(case):
    counter, keys, g, h = _exact(case)
    spec, p = _spec(case, "metropolis_hastings")
    burn, n, thin, floor = RUNS[case]
    lats = _sample(spec, _start(case), SEEDS, burn, n, thin)
    skeys = counter.keys_of(lats)
    assert np.all(valid(counter, skeys))
    chi2, df, distinct, empty = chi_squared(h, g, energy(counter, skeys, **p))
    print(f"{case}: chi2 {chi2:.1f} df {df} distinct bins {distinct}")
    assert df >= 1
    assert empty == 0, f"{empty} bins with expected count >= {MIN_EXPECTED} never visited"
    assert distinct >= floor, distinct
    assert chi2 < 8.0 * df, (chi2, df)
    assert chi2 < df + 6.0 * np.sqrt(2.0 * df), (chi2, df)


def test_plain_metropolis_fails_the_exact_check():
    """Planted mistake: plain Metropolis acceptance (no proposal ratio) on
    the same chain is not reversible with respect to exp(-H)/Z; the statistic
    rejects it."""
    counter, keys, g, h = _exact("single")
    spec, p = _spec("single", "metropolis")
    burn, n, thin, _ = RUNS["single"]
    lats = _sample(spec, _start("single"), SEEDS, burn, n, thin)
    chi2, df, _, _ = chi_squared(h, g, energy(counter, counter.keys_of(lats), **p))
    print(f"plain Metropolis: chi2 {chi2:.1f} df {df}")
    assert chi2 > 8.0 * df, (chi2, df)


def test_two_cell_chain_survives_very_stiff_parameters():
    """exact_boltzmann.rs:764-794: at four times the two-cell coefficients the
    chain is trapped (too few bins for chi-squared), but 500,000 attempts keep
    both cells at volume >= 1 and a finite energy."""
    spec, p = _spec("two@4.0", "metropolis_hastings")
    sim = O.OracleSim(spec, 2)
    lat = _start("two")
    sim.init_explicit(lat, [0, 1])
    sim.set_check_topology(False)
    last = sim.sample_attempts(500_000, 1, 0)
    assert sim.volume().min() >= 1
    counter = Counter(4, 4, 2)
    h = energy(counter, counter.keys_of(last), **p)
    assert np.all(np.isfinite(h)) and np.isfinite(sim.energy)
