"""Shared builders for the tests: the same model as an oracle simulation and
as a GB300 builder, so both sides start from identical inputs."""

from __future__ import annotations

import numpy as np

import oracle as O

NBH_DEFAULT = {2: "moore", 3: "eighteen"}


class Model:
    """A model description both engines can be built from."""

    def __init__(self, grid, boundary, types, adhesion, counts=None, energy=None, seed=1, acceptance="metropolis",
                 act=None):
        self.acceptance = acceptance  # "metropolis" or "metropolis_hastings"
        self.act = [tuple(a) for a in act] if act is not None else None  # per type (lambda_act, max_act)
        self.grid = tuple(int(g) for g in grid)
        self.D = len(self.grid)
        self.boundary = boundary
        self.types = [tuple(t) for t in types]  # (name, V*, I*, lambda_V, lambda_I)
        self.adhesion = [list(map(float, r)) for r in adhesion]
        self.counts = list(counts) if counts is not None else [0] * len(self.types)
        self.energy = energy
        self.seed = seed

    def spec(self):
        return O.ModelSpec(self.grid, self.boundary == "periodic", [t[1:] for t in self.types], self.adhesion,
                           cell_counts=self.counts, energy=self.energy or NBH_DEFAULT[self.D],
                           acceptance=self.acceptance, act=self.act)

    def oracle(self, seed=None, lattice=None, cell_type_of=None, local_halo=True):
        sim = O.OracleSim(self.spec(), self.seed if seed is None else seed)
        sim.set_local_halo(local_halo)
        if lattice is not None:
            sim.init_explicit(lattice, cell_type_of)
        else:
            sim.init_default()
        return sim

    def builder(self, seed=None, lattice=None, cell_type_of=None, warn=True):
        from cpm import _cpm

        b = _cpm.CPM(grid=list(self.grid), boundary=self.boundary, seed=self.seed if seed is None else seed,
                     energy_neighborhood=self.energy,
                     acceptance=None if self.acceptance == "metropolis" else self.acceptance,
                     active_terms={"act": True} if self.act is not None else None)
        for k, t in enumerate(self.types):
            if self.act is not None:
                b.register_cell_type(*t, lambda_act=float(self.act[k][0]), max_act=int(self.act[k][1]))
            else:
                b.register_cell_type(*t)
        for t, n in zip(self.types, self.counts):
            b.add_cells(t[0], n)
        b.set_adhesion(self.adhesion)
        if lattice is not None:
            b.initialize(lattice=np.asarray(lattice).ravel().tolist(), cell_type_of=list(cell_type_of))
        else:
            b.initialize(warn_on_default_init=warn)
        return b


def c1_model(seed=1):
    """Config 1: 30x30 periodic, one type (V*=50, I*=75, 10, 2), 5 cells, J=[[0,5],[5,2]]."""
    return Model((30, 30), "periodic", [("epithelial", 50, 75, 10.0, 2.0)], [[0, 5], [5, 2]], [5], seed=seed)


def sorting_model(side=64, seed=3, types=4, phi=0.8, jseed=11):
    """Config 2 shape on a smaller grid: 4 types, V*=50, I*=30, lambdas 5/1,
    medium row 16, type-type J uniform in [2, 14]."""
    rng = np.random.default_rng(jseed)
    n = types
    J = np.zeros((n + 1, n + 1))
    J[0, 1:] = J[1:, 0] = 16.0
    tt = rng.uniform(2, 14, size=(n, n))
    tt = np.triu(tt) + np.triu(tt, 1).T
    J[1:, 1:] = tt
    per = round(phi / types * side * side / 50)
    return Model((side, side), "periodic", [(f"t{i}", 50, 30, 5.0, 1.0) for i in range(n)], J.tolist(),
                 [per] * n, seed=seed)


def organoid_model(side=24, seed=5, energy="twenty_six", boundary="periodic", vol=60, counts=(10, 10)):
    """3D: 2 types, 26-neighbour energy (the 3D mapping of config 3)."""
    J = [[0, 16, 16], [16, 4, 9], [16, 9, 5]]
    return Model((side, side, side), boundary, [("a", vol, 90, 2.0, 0.5), ("b", vol, 90, 2.0, 0.5)], J,
                 list(counts), energy=energy, seed=seed)


def padded_cells(sim: O.OracleSim):
    """Oracle per-cell arrays re-indexed by id (entry 0 = medium)."""
    D = sim.spec.D
    v = np.concatenate([[0], sim.volume()]).astype(np.uint32)
    i = np.concatenate([[0], sim.interface()]).astype(np.uint32)
    sp = np.concatenate([np.zeros((1, D), np.int64), sim.sum_position()]).astype(np.int64)
    so = np.concatenate([np.zeros((1, D, D), np.int64), sim.sum_outer()]).astype(np.int64)
    return v, i, sp, so


def random_interior_targets(sim: O.OracleSim, n, rng):
    st = sim.strides()
    grid = sim.spec.grid
    flat = np.zeros(n, dtype=np.int64)
    for d in range(sim.spec.D):
        flat += (rng.integers(0, grid[d], n) + 1) * st[d]
    return flat


def contact_reference(lat, periodic, offsets):
    """Independent count of the contact graph: unordered pairs of neighbouring
    sites of different cells (each pair once), and for a fixed boundary each
    (site, outward offset) of a cell as a contact with the medium."""
    from collections import Counter

    lat = np.asarray(lat)
    D = lat.ndim
    cnt = Counter()
    idx = np.indices(lat.shape).reshape(D, -1).T
    flat = lat.ravel()
    shape = np.array(lat.shape)
    for off in offsets:
        nb = idx + np.asarray(off)
        if periodic:
            nb = nb % shape
            inside = np.ones(len(idx), bool)
        else:
            inside = np.all((nb >= 0) & (nb < shape), axis=1)
        src = np.ravel_multi_index(idx.T, lat.shape)
        for k in np.flatnonzero(inside):
            j = np.ravel_multi_index(nb[k], lat.shape)
            if j <= src[k]:
                continue
            a, b = flat[src[k]], flat[j]
            if a != b:
                cnt[(min(a, b), max(a, b))] += 1
        if not periodic:
            for k in np.flatnonzero(~inside):
                a = flat[src[k]]
                if a != 0:
                    cnt[(0, a)] += 1
    return cnt


def energy_offsets(model):
    """The energy stencil as coordinate offsets (neighborhood.rs order)."""
    import itertools

    D = model.D
    full = [o for o in itertools.product((-1, 0, 1), repeat=D) if any(o)]
    kind = model.energy or NBH_DEFAULT[D]
    if kind == "von_neumann":
        return [o for o in full if sum(map(abs, o)) == 1]
    if kind == "eighteen":
        return [o for o in full if sum(map(abs, o)) <= 2]
    return full
