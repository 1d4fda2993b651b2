"""ctypes wrapper over the CPU oracle (``oracle/cpm_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: the oracle is what the GB300 engine is compared
against. Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py`` (its CPU-baseline leg and ``--impl reference`` arm) may load it;
the ``cpm`` package never does.

The oracle restates DebajyotiS/cpm-rust ``cpm-core`` (see the C++ file header
for the per-function citations) and is pinned by the reference's frozen
trajectory, its calibrated target interfaces (a second trajectory, fixed
boundary) and derived-seed vectors (``tests/test_oracle_kat.py``), and by
the exact-Boltzmann harness (``tests/test_oracle_boltzmann.py``).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

NBH = {
    "von_neumann": 0,
    "moore": 1,
    "eighteen": 2,
    "twenty_six": 3,
    "twenty_six_weighted": 4,
}

_lock = threading.Lock()
_lib = None


class Move(ctypes.Structure):
    _fields_ = [
        ("target_flat", ctypes.c_int64),
        ("source_flat", ctypes.c_int64),
        ("losing", ctypes.c_uint32),
        ("gaining", ctypes.c_uint32),
        ("null_move", ctypes.c_int32),
        ("topology_ok", ctypes.c_int32),
        ("volume_guard_ok", ctypes.c_int32),
        ("evaluated", ctypes.c_int32),
        ("delta_i_losing", ctypes.c_int32),
        ("delta_i_gaining", ctypes.c_int32),
        ("delta_h", ctypes.c_double),
        ("accepted", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


MOVE_DTYPE = np.dtype(
    [
        ("target_flat", np.int64),
        ("source_flat", np.int64),
        ("losing", np.uint32),
        ("gaining", np.uint32),
        ("null_move", np.int32),
        ("topology_ok", np.int32),
        ("volume_guard_ok", np.int32),
        ("evaluated", np.int32),
        ("delta_i_losing", np.int32),
        ("delta_i_gaining", np.int32),
        ("delta_h", np.float64),
        ("accepted", np.int32),
        ("pad", np.int32),
    ]
)

CELL_SAMPLE_DTYPE = np.dtype(
    [
        ("id", np.uint32),
        ("volume", np.uint32),
        ("interface", np.uint32),
        ("pad", np.uint32),
        ("centroid", np.float64, (3,)),
        ("eigenvalues", np.float64, (3,)),
        ("rg2", np.float64),
        ("kappa2", np.float64),
    ]
)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (idempotent)."""
    src = os.path.join(HERE, "cpm_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            P = ctypes.c_void_p
            L.orc_new.restype = P
            L.orc_new.argtypes = [
                ctypes.c_int, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                ctypes.c_int, P, P, P, P, P, P, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_int,
            ]
            L.orc_free.argtypes = [P]
            L.orc_set_modes.argtypes = [P, ctypes.c_int, P, P]
            L.orc_set_act_state.argtypes = [P, P, ctypes.c_uint64]
            L.orc_get_birth.argtypes = [P, P]
            L.orc_act_delta.argtypes = [P, ctypes.c_int64, ctypes.c_int64]
            L.orc_act_delta.restype = ctypes.c_double
            L.orc_set_local_halo.argtypes = [P, ctypes.c_int]
            L.orc_set_check_topology.argtypes = [P, ctypes.c_int]
            L.orc_attempts_checked.argtypes = [P, ctypes.c_uint64, P, P]
            L.orc_attempts_checked.restype = ctypes.c_int64
            L.orc_sample_attempts.argtypes = [P, ctypes.c_uint64, ctypes.c_int64, ctypes.c_uint64, P]
            L.orc_init_explicit.argtypes = [P, P, ctypes.c_int64, P, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
            L.orc_init_default.argtypes = [P, ctypes.c_char_p, ctypes.c_int]
            L.orc_run_mcs.argtypes = [P, ctypes.c_uint64]
            L.orc_n_cells.argtypes = [P]
            L.orc_n_sites.argtypes = [P]
            L.orc_n_sites.restype = ctypes.c_int64
            L.orc_n_padded.argtypes = [P]
            L.orc_n_padded.restype = ctypes.c_int64
            L.orc_mcs.argtypes = [P]
            L.orc_mcs.restype = ctypes.c_uint64
            L.orc_energy.argtypes = [P]
            L.orc_energy.restype = ctypes.c_double
            L.orc_global_energy.argtypes = [P]
            L.orc_global_energy.restype = ctypes.c_double
            for name in ("orc_get_volume", "orc_get_interface", "orc_get_type_of", "orc_get_sum_position",
                         "orc_get_sum_outer", "orc_get_contact", "orc_get_padded", "orc_get_lattice",
                         "orc_get_strides"):
                getattr(L, name).argtypes = [P, P]
            L.orc_get_offsets.argtypes = [P, ctypes.c_int, P]
            L.orc_check.argtypes = [P, P]
            L.orc_set_state.argtypes = [P, P, P, P]
            L.orc_evaluate_moves.argtypes = [P, ctypes.c_int64, P, P, P, P]
            L.orc_commit.argtypes = [P, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double]
            L.orc_is_simple.argtypes = [ctypes.c_int, ctypes.c_uint32]
            L.orc_slow_is_simple.argtypes = [ctypes.c_int, ctypes.c_uint32]
            L.orc_table_3d.argtypes = [P]
            L.orc_blake3.argtypes = [P, ctypes.c_uint64, P]
            L.orc_derive_seed_u64.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
            L.orc_derive_seed_u64.restype = ctypes.c_uint64
            L.orc_xoshiro_stream.argtypes = [ctypes.c_uint64, ctypes.c_int, P]
            L.orc_gen_range_stream.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, P]
            L.orc_take_sample.argtypes = [P, P, P, P, P, P, P, ctypes.c_int]
            L.orc_not_equilibrated.argtypes = [P, ctypes.c_int]
            L.orc_shape_descriptors.argtypes = [ctypes.c_int, P, ctypes.c_uint32, P, P, P, P]
            L.orc_run_many.argtypes = [
                ctypes.c_int, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                ctypes.c_int, P, P, P, P, P, P, P, P, ctypes.c_int,
                ctypes.c_int, P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                ctypes.c_int, P, P, P, ctypes.c_int, P, P,
            ]
            L.orc_run_status.argtypes = [P, ctypes.c_size_t, ctypes.c_size_t, P, ctypes.c_uint32, P, P, P,
                                         ctypes.c_size_t, ctypes.c_uint32, P, P, P]
            L.orc_run_many_checkpoints.argtypes = [
                ctypes.c_int, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                ctypes.c_int, P, P, P, P, P, P, P, P, ctypes.c_int,
                ctypes.c_int, P, ctypes.c_int, P, ctypes.c_int, ctypes.c_int, P, P, P, P,
            ]
            _lib = L
        return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class ModelSpec:
    """Plain description of one model configuration (the oracle's input)."""

    def __init__(self, grid, periodic, types, adhesion, cell_counts=None, copy="von_neumann",
                 energy=None, connectivity="von_neumann", min_cell_volume=1, acceptance="metropolis", act=None):
        self.grid = [int(g) for g in grid]
        self.D = len(self.grid)
        self.periodic = bool(periodic)
        # types: list of (target_volume, target_interface, lambda_volume, lambda_interface)
        self.types = [tuple(t) for t in types]
        self.adhesion = np.ascontiguousarray(np.asarray(adhesion, dtype=np.float64))
        self.cell_counts = list(cell_counts) if cell_counts is not None else [0] * len(self.types)
        self.copy = copy
        self.energy = energy if energy is not None else ("moore" if self.D == 2 else "eighteen")
        self.connectivity = connectivity
        self.min_cell_volume = int(min_cell_volume)
        # monte_carlo.rs:147-196: "metropolis" or "metropolis_hastings"
        self.acceptance = acceptance
        # energy.rs:329-471: None (off) or per type (lambda_act, max_act)
        self.act = [tuple(a) for a in act] if act is not None else None

    def mode_args(self):
        """(acceptance code, lambda_act array or None, max_act array or None)."""
        acc = {"metropolis": 0, "metropolis_hastings": 1}[self.acceptance]
        if self.act is None:
            return acc, None, None
        return (acc, np.ascontiguousarray([a[0] for a in self.act], dtype=np.float64),
                np.ascontiguousarray([a[1] for a in self.act], dtype=np.uint32))

    def arrays(self):
        n = len(self.types)
        tv = np.array([t[0] for t in self.types], dtype=np.uint32)
        ti = np.array([t[1] for t in self.types], dtype=np.uint32)
        lv = np.array([t[2] for t in self.types], dtype=np.float64)
        li = np.array([t[3] for t in self.types], dtype=np.float64)
        cc = np.array(self.cell_counts, dtype=np.uint64)
        grid = np.array(self.grid + [1] * (3 - self.D), dtype=np.int32)
        adh = np.ascontiguousarray(self.adhesion.reshape(n + 1, n + 1))
        return grid, tv, ti, lv, li, cc, adh


class OracleSim:
    """One reference-semantics simulation on the CPU."""

    def __init__(self, spec: ModelSpec, seed: int):
        self.spec = spec
        L = lib()
        grid, tv, ti, lv, li, cc, adh = spec.arrays()
        self._keep = (grid, tv, ti, lv, li, cc, adh)
        err = ctypes.create_string_buffer(512)
        h = L.orc_new(spec.D, _ptr(grid), int(spec.periodic), NBH[spec.copy], NBH[spec.energy],
                      NBH[spec.connectivity], len(spec.types), _ptr(tv), _ptr(ti), _ptr(lv), _ptr(li),
                      _ptr(cc), _ptr(adh), ctypes.c_uint64(seed & (2**64 - 1)), spec.min_cell_volume, err, 512)
        if not h:
            raise ValueError(err.value.decode())
        self.h = ctypes.c_void_p(h)
        acc, la, ma = spec.mode_args()
        if acc or la is not None:
            self._modes = (la, ma)
            L.orc_set_modes(self.h, acc, _ptr(la) if la is not None else None, _ptr(ma) if ma is not None else None)

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and _lib is not None:
            _lib.orc_free(h)
            self.h = None

    def set_act_state(self, birth=None, mcs=0):
        b = np.ascontiguousarray(birth, dtype=np.uint32) if birth is not None else None
        lib().orc_set_act_state(self.h, _ptr(b) if b is not None else None, int(mcs))

    def birth(self):
        out = np.zeros(self.n_padded, np.uint32)
        lib().orc_get_birth(self.h, _ptr(out))
        return out

    def act_delta(self, target_flat, source_flat):
        return lib().orc_act_delta(self.h, int(target_flat), int(source_flat))

    def set_local_halo(self, on: bool):
        lib().orc_set_local_halo(self.h, int(on))

    def set_check_topology(self, on: bool):
        """Connectivity check of each attempt; off only for the exact-Boltzmann
        harness (tests/exact_boltzmann.rs calls attempt(cpm, false))."""
        lib().orc_set_check_topology(self.h, int(on))

    def attempts_checked(self, n: int):
        """`n` single attempts with the brute-force check after every accepted
        one: (index of the first failing attempt or -1, mismatch bits,
        accepted moves)."""
        acc, bad = ctypes.c_uint64(0), ctypes.c_int(0)
        first = lib().orc_attempts_checked(self.h, int(n), ctypes.byref(acc), ctypes.byref(bad))
        return first, bad.value, acc.value

    def sample_attempts(self, burn_in: int, n_samples: int, thin: int) -> np.ndarray:
        """`burn_in` single attempts, then `n_samples` interior lattices, each
        after `thin` more attempts; shape (n_samples, *grid)."""
        out = np.zeros((int(n_samples), *self.spec.grid), np.uint32)
        lib().orc_sample_attempts(self.h, int(burn_in), int(n_samples), int(thin), _ptr(out))
        return out

    def init_explicit(self, lattice, cell_type_of):
        lat = np.ascontiguousarray(np.asarray(lattice, dtype=np.uint32).ravel())
        cto = np.ascontiguousarray(np.asarray(cell_type_of, dtype=np.uint32))
        err = ctypes.create_string_buffer(512)
        if lib().orc_init_explicit(self.h, _ptr(lat), lat.size, _ptr(cto), cto.size, err, 512) != 0:
            raise ValueError(err.value.decode())

    def init_default(self):
        err = ctypes.create_string_buffer(512)
        if lib().orc_init_default(self.h, err, 512) != 0:
            raise ValueError(err.value.decode())

    def run_mcs(self, n: int):
        lib().orc_run_mcs(self.h, n)

    @property
    def n_cells(self):
        return lib().orc_n_cells(self.h)

    @property
    def n_padded(self):
        return lib().orc_n_padded(self.h)

    @property
    def mcs(self):
        return lib().orc_mcs(self.h)

    @property
    def energy(self):
        return lib().orc_energy(self.h)

    def global_energy(self):
        return lib().orc_global_energy(self.h)

    def _get(self, name, n, dtype):
        a = np.zeros(n, dtype=dtype)
        getattr(lib(), name)(self.h, _ptr(a))
        return a

    def volume(self):
        return self._get("orc_get_volume", self.n_cells, np.uint32)

    def interface(self):
        return self._get("orc_get_interface", self.n_cells, np.uint32)

    def type_of(self):
        return self._get("orc_get_type_of", self.n_cells, np.uint32)

    def sum_position(self):
        return self._get("orc_get_sum_position", self.n_cells * self.spec.D, np.int64).reshape(self.n_cells, self.spec.D)

    def sum_outer(self):
        D = self.spec.D
        return self._get("orc_get_sum_outer", self.n_cells * D * D, np.int64).reshape(self.n_cells, D, D)

    def contact(self):
        n1 = self.n_cells + 1
        return self._get("orc_get_contact", n1 * n1, np.uint32).reshape(n1, n1)

    def padded(self):
        return self._get("orc_get_padded", self.n_padded, np.uint32)

    def lattice(self):
        return self._get("orc_get_lattice", int(np.prod(self.spec.grid)), np.uint32).reshape(self.spec.grid)

    def strides(self):
        return self._get("orc_get_strides", 3, np.int64)

    def offsets(self, which: str):
        w = {"copy": 0, "energy": 1, "connectivity": 2, "topology": 3}[which]
        n = lib().orc_get_offsets(self.h, w, None)
        a = np.zeros(n, dtype=np.int64)
        lib().orc_get_offsets(self.h, w, _ptr(a))
        return a

    def check(self):
        rel = ctypes.c_double(0.0)
        bad = lib().orc_check(self.h, ctypes.byref(rel))
        return bad, rel.value

    def set_state(self, padded, volume, interface):
        p = np.ascontiguousarray(padded, dtype=np.uint32)
        v = np.ascontiguousarray(volume, dtype=np.uint32)
        i = np.ascontiguousarray(interface, dtype=np.uint32)
        lib().orc_set_state(self.h, _ptr(p), _ptr(v), _ptr(i))

    def evaluate_moves(self, target, k, u):
        t = np.ascontiguousarray(target, dtype=np.int64)
        kk = np.ascontiguousarray(k, dtype=np.int32)
        uu = np.ascontiguousarray(u, dtype=np.float64)
        out = np.zeros(t.size, dtype=MOVE_DTYPE)
        lib().orc_evaluate_moves(self.h, t.size, _ptr(t), _ptr(kk), _ptr(uu), _ptr(out))
        return out

    def commit(self, target_flat, losing, gaining, delta_h):
        lib().orc_commit(self.h, int(target_flat), int(losing), int(gaining), float(delta_h))

    def take_sample(self, max_medium=100000):
        n = self.n_cells
        cells = np.zeros(n, dtype=CELL_SAMPLE_DTYPE)
        energy = ctypes.c_double(0.0)
        frag = np.zeros(max(n, 1), dtype=np.uint32)
        nfrag = ctypes.c_int(0)
        mv = np.zeros(max_medium, dtype=np.uint32)
        mt = np.zeros(max_medium, dtype=np.uint8)
        nm = lib().orc_take_sample(self.h, _ptr(cells), ctypes.byref(energy), _ptr(frag), ctypes.byref(nfrag),
                                   _ptr(mv), _ptr(mt), max_medium)
        nm = min(nm, max_medium)
        return {
            "cells": cells,
            "energy": energy.value,
            "fragmented": frag[: nfrag.value].copy(),
            "medium_volumes": mv[:nm].copy(),
            "medium_touches": mt[:nm].astype(bool),
        }


def derive_seed_u64(master: int, index: int) -> int:
    return int(lib().orc_derive_seed_u64(master, index))


def blake3(data: bytes) -> bytes:
    buf = (ctypes.c_uint8 * max(len(data), 1)).from_buffer_copy(data if data else b"\0")
    out = (ctypes.c_uint8 * 32)()
    lib().orc_blake3(buf, len(data), out)
    return bytes(out)


def xoshiro_stream(seed: int, n: int) -> np.ndarray:
    a = np.zeros(n, dtype=np.uint64)
    lib().orc_xoshiro_stream(seed, n, _ptr(a))
    return a


def gen_range_stream(seed: int, hi: int, n: int) -> np.ndarray:
    a = np.zeros(n, dtype=np.uint64)
    lib().orc_gen_range_stream(seed, hi, n, _ptr(a))
    return a


def is_simple(D: int, pattern: int) -> bool:
    return bool(lib().orc_is_simple(D, pattern))


def slow_is_simple(D: int, pattern: int) -> bool:
    return bool(lib().orc_slow_is_simple(D, pattern))


def table_3d() -> np.ndarray:
    words = np.zeros((1 << 26) // 64, dtype=np.uint64)
    lib().orc_table_3d(_ptr(words))
    return words


def shape_descriptors(D: int, sum_outer, volume: int, centroid):
    """output.rs:147-231 for one cell: (sorted eigenvalues (3), R_g^2, kappa^2)
    of the gyration tensor sum_outer / V - c c^T."""
    so = np.ascontiguousarray(np.asarray(sum_outer, dtype=np.int64).ravel())
    c = np.zeros(3)
    c[:D] = np.asarray(centroid, dtype=np.float64)[:D]
    eig = np.zeros(3)
    rg2, kap = ctypes.c_double(0.0), ctypes.c_double(0.0)
    lib().orc_shape_descriptors(D, _ptr(so), int(volume), _ptr(c), _ptr(eig), ctypes.byref(rg2), ctypes.byref(kap))
    return eig, rg2.value, kap.value


def not_equilibrated(trace) -> bool:
    t = np.ascontiguousarray(trace, dtype=np.float64)
    return bool(lib().orc_not_equilibrated(_ptr(t), t.size))


STATUS_KINDS = ("Ok", "NotEquilibrated", "Fragmented", "CellLost", "Degenerate")


def run_status(trace, sample_mcs, volumes, first_fragmented=None, last_pairs=(), min_cell_volume=1):
    """output.rs:456-522 on given readouts: (kind, cell_id, at_mcs).
    volumes: (samples, cells) by id; first_fragmented: per sample the first
    fragmented id (0 none) or None (no topology readouts); last_pairs: the
    last sample's contact pairs (a, b) with a positive count."""
    t = np.ascontiguousarray(trace, dtype=np.float64)
    m = np.ascontiguousarray(sample_mcs, dtype=np.uint64)
    v = np.ascontiguousarray(volumes, dtype=np.uint32)
    assert v.ndim == 2 and v.shape[0] == m.size, "volumes: one row of cell volumes per sample"
    f = None if first_fragmented is None else np.ascontiguousarray(first_fragmented, dtype=np.uint32)
    p = np.ascontiguousarray(np.asarray(last_pairs, dtype=np.uint32).reshape(-1, 2))
    kind, cid, at = ctypes.c_int32(0), ctypes.c_uint32(0), ctypes.c_uint64(0)
    lib().orc_run_status(_ptr(t), t.size, m.size, _ptr(m), v.shape[1], _ptr(v), _ptr(f) if f is not None else None,
                         _ptr(p), len(p), int(min_cell_volume), ctypes.byref(kind), ctypes.byref(cid),
                         ctypes.byref(at))
    return STATUS_KINDS[kind.value], cid.value, at.value


def run_many(spec: ModelSpec, seeds, burn_in: int, readout: int, threads: int = 0, local_halo: bool = True,
             explicit=None, max_cells=None):
    """Independent runs of ``spec`` (default init unless ``explicit`` =
    (lattice, cell_type_of)); returns per-run last-sample cell summaries."""
    L = lib()
    grid, tv, ti, lv, li, cc, adh = spec.arrays()
    acc, la, ma = spec.mode_args()
    seeds = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64))
    if max_cells is None:
        max_cells = int(sum(spec.cell_counts)) if explicit is None else len(explicit[1])
    out_cells = np.zeros(seeds.size * max_cells, dtype=CELL_SAMPLE_DTYPE)
    out_energy = np.zeros(seeds.size, dtype=np.float64)
    out_n = np.zeros(seeds.size, dtype=np.int32)
    if explicit is not None:
        el = np.ascontiguousarray(np.asarray(explicit[0], dtype=np.uint32).ravel())
        et = np.ascontiguousarray(np.asarray(explicit[1], dtype=np.uint32))
        elp, etp, en = _ptr(el), _ptr(et), et.size
    else:
        elp, etp, en = None, None, 0
    failed = L.orc_run_many(spec.D, _ptr(grid), int(spec.periodic), NBH[spec.copy], NBH[spec.energy],
                            NBH[spec.connectivity], len(spec.types), _ptr(tv), _ptr(ti), _ptr(lv), _ptr(li),
                            _ptr(cc), _ptr(adh), elp, etp, en, seeds.size, _ptr(seeds), burn_in, readout,
                            threads, int(local_halo), max_cells, _ptr(out_cells), _ptr(out_energy), _ptr(out_n),
                            acc, _ptr(la) if la is not None else None, _ptr(ma) if ma is not None else None)
    return failed, out_cells.reshape(seeds.size, max_cells), out_energy, out_n


def run_many_checkpoints(spec: ModelSpec, seeds, checkpoints, threads: int = 0, explicit=None):
    """Independent runs of ``spec`` (default init unless ``explicit`` =
    (lattice, cell_type_of)), each read at the cumulative MCS counts
    ``checkpoints`` along one trajectory. Returns (failed, volume, interface,
    energy, n_cells): volume and interface of shape (runs, checkpoints,
    cells), energy (runs, checkpoints)."""
    L = lib()
    grid, tv, ti, lv, li, cc, adh = spec.arrays()
    seeds = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64))
    ck = np.ascontiguousarray(np.asarray(checkpoints, dtype=np.uint64))
    assert np.all(np.diff(ck.astype(np.int64)) > 0)
    max_cells = int(sum(spec.cell_counts)) if explicit is None else len(explicit[1])
    vol = np.zeros((seeds.size, ck.size, max_cells), dtype=np.uint32)
    itf = np.zeros_like(vol)
    energy = np.zeros((seeds.size, ck.size), dtype=np.float64)
    n = np.zeros(seeds.size, dtype=np.int32)
    if explicit is not None:
        el = np.ascontiguousarray(np.asarray(explicit[0], dtype=np.uint32).ravel())
        et = np.ascontiguousarray(np.asarray(explicit[1], dtype=np.uint32))
        elp, etp, en = _ptr(el), _ptr(et), et.size
    else:
        elp, etp, en = None, None, 0
    failed = L.orc_run_many_checkpoints(spec.D, _ptr(grid), int(spec.periodic), NBH[spec.copy], NBH[spec.energy],
                                        NBH[spec.connectivity], len(spec.types), _ptr(tv), _ptr(ti), _ptr(lv),
                                        _ptr(li), _ptr(cc), _ptr(adh), elp, etp, en, seeds.size, _ptr(seeds),
                                        ck.size, _ptr(ck), threads, max_cells, _ptr(vol), _ptr(itf), _ptr(energy),
                                        _ptr(n))
    return failed, vol, itf, energy, n
