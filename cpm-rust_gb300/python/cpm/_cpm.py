"""Compiled-surface shim: the GB300 engine's ``_cpm`` module.

Stands in for the reference's PyO3 extension ``cpm._cpm``
(crates/cpm-py/src/lib.rs:85-94): the same ``CPM`` builder class with the
same keyword arguments and return tuples (crates/cpm-py/src/builder.rs:
104-401), and result objects with the reference's attribute names and dtypes
(crates/cpm-py/src/convert.rs:27-256). Every call goes through the C ABI of
``libcpm_gpu.so`` (include/cpm_gpu.h); ctypes releases the GIL for the
duration of each foreign call, so a whole trajectory or batch runs without
the GIL, as in the reference (builder.rs:452, 509-511).

There is no CPU fallback: if the library is missing this module fails to
import, and running without a CUDA device raises.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

__version__ = "0.2.0+gb300"

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.dirname(os.path.dirname(_HERE))
_LIB_PATH = os.environ.get("CPM_GPU_LIB", os.path.join(_PKG, "lib", "libcpm_gpu.so"))

CPM_OK = 0
CPM_E_CONFIG = 1
CPM_E_INIT = 2
CPM_E_THETA = 3
CPM_E_CUDA = 4
CPM_E_TIMEOUT = 5
CPM_E_BUDGET = 6
CPM_E_ARG = 7
CPM_E_UNSUPPORTED = 8

STAT_NAMES = (
    "attempts",
    "nonnull",
    "topology_rejected",
    "guard_rejected",
    "evaluated",
    "accepted",
    "rounds",
    "passes",
    "spin_timeouts",
    "fixpoint_iterations",
    "h2d_bytes",
    "d2h_bytes",
    "deferred",
    "cycles_passes",
    "cycles_stage",
    "cycles_sync",
    "cycles_build",
    "cycles_eval",
    "cycles_fixpoint",
    "cycles_apply",
    "wide_passes",
    "cycles_lower",
    "cycles_claim",
    "cycles_barrier_claim",
    "cycles_barrier_write",
    "exact_decisions",
    "host_prep_us",
    "device_us",
    "host_read_us",
    "cycles_res_build",
    "cycles_res_resolve",
    "host_place_us",
)


class CPMRuntimeError(RuntimeError):
    """A device-side failure (CUDA error, timeout) reported by the engine."""


class ResultInfo(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("n_types", ctypes.c_int32),
        ("grid", ctypes.c_int64 * 3),
        ("n_cells", ctypes.c_uint64),
        ("n_samples", ctypes.c_uint64),
        ("used_default", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


class MetadataC(ctypes.Structure):
    _fields_ = [
        ("cpm_version", ctypes.c_char * 32),
        ("convention_hash", ctypes.c_char * 65),
        ("model_hash", ctypes.c_char * 65),
        ("seed_policy", ctypes.c_char * 32),
        ("convention_version", ctypes.c_uint32),
        ("theta_layout_version", ctypes.c_uint32),
        ("seed", ctypes.c_uint64),
        ("derived_phi", ctypes.c_double),
    ]


class StatusC(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_char * 24),
        ("has_cell", ctypes.c_int32),
        ("cell_id", ctypes.c_uint32),
        ("at_mcs", ctypes.c_uint64),
    ]


class SampleSizes(ctypes.Structure):
    _fields_ = [
        ("n_contact", ctypes.c_uint64),
        ("n_fragmented", ctypes.c_uint64),
        ("n_medium", ctypes.c_uint64),
        ("has_lattice", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ]


_P = ctypes.c_void_p


class SampleOut(ctypes.Structure):
    _fields_ = [(name, _P) for name in (
        "mcs", "conservative_energy", "ids", "volume", "interface", "centroid", "eigenvalues",
        "radius_of_gyration_sq", "kappa_sq", "contact_a", "contact_b", "contact_count", "fragmented_cells",
        "medium_component_volumes", "medium_component_touches_boundary", "lattice",
    )]


class SimInfo(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("periodic", ctypes.c_int32),
        ("dims", ctypes.c_int64 * 3),
        ("padded_dims", ctypes.c_int64 * 3),
        ("strides", ctypes.c_int64 * 3),
        ("n_sites", ctypes.c_uint64),
        ("n_padded", ctypes.c_uint64),
        ("n_cells", ctypes.c_uint64),
        ("n_energy", ctypes.c_int32),
        ("n_colors", ctypes.c_int32),
    ]


MOVE_DTYPE = np.dtype([
    ("target_flat", np.int64), ("source_flat", np.int64), ("losing", np.uint32), ("gaining", np.uint32),
    ("null_move", np.int32), ("topology_ok", np.int32), ("volume_guard_ok", np.int32), ("evaluated", np.int32),
    ("delta_i_losing", np.int32), ("delta_i_gaining", np.int32), ("delta_h", np.float64), ("accepted", np.int32),
    ("accepted_sweep", np.int32),
])

# Every symbol include/cpm_gpu.h declares (checked by the CPU test suite).
EXPORTED_SYMBOLS = (
    "cpm_last_error", "cpm_version",
    "cpm_builder_new", "cpm_builder_register_cell_type", "cpm_builder_add_cells", "cpm_builder_set_adhesion",
    "cpm_builder_initialize", "cpm_builder_run", "cpm_builder_run_batch", "cpm_builder_theta_len",
    "cpm_builder_extract_theta", "cpm_builder_theta_name", "cpm_builder_free",
    "cpm_result_info_get", "cpm_result_metadata_get", "cpm_result_status_get", "cpm_result_cell_type_index",
    "cpm_result_cell_type_name", "cpm_result_sample_sizes", "cpm_result_sample_read", "cpm_result_stats",
    "cpm_result_free",
    "cpm_engine_create", "cpm_engine_size", "cpm_engine_sim_info", "cpm_engine_run_mcs", "cpm_engine_synchronize",
    "cpm_engine_mcs", "cpm_engine_read_lattice", "cpm_engine_read_padded", "cpm_engine_read_cells",
    "cpm_engine_energy", "cpm_engine_recount_check", "cpm_engine_stats", "cpm_engine_write_state",
    "cpm_engine_evaluate_moves", "cpm_engine_commit_moves", "cpm_engine_take_sample", "cpm_engine_write_act_state",
    "cpm_engine_read_birth", "cpm_engine_destroy",
    "cpm_run_many",
    "cpm_builder_initial_state", "cpm_builder_hashes", "cpm_derive_seed_u64", "cpm_run_status", "cpm_tuning_report",
    "cpm_run_mcs_noalloc",
    "cpm_serve_start", "cpm_serve_submit", "cpm_serve_poll", "cpm_serve_wait", "cpm_serve_cancel",
    "cpm_serve_stats_get", "cpm_serve_stop", "cpm_result_samples_sizes", "cpm_result_samples_read",
    "cpm_results_samples_read",
)


def _load():
    if not os.path.exists(_LIB_PATH):
        raise ImportError(
            f"libcpm_gpu.so not found at {_LIB_PATH}: build it with `python cpm-rust_gb300/build.py` "
            "(the GB300 engine has no CPU fallback)"
        )
    L = ctypes.CDLL(_LIB_PATH)
    I32, U32, U64, SZ, D = ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t, ctypes.c_double
    L.cpm_last_error.restype = ctypes.c_char_p
    L.cpm_last_error.argtypes = []
    L.cpm_version.restype = ctypes.c_char_p
    L.cpm_builder_new.argtypes = [_P, SZ, ctypes.c_char_p, U64, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                  ctypes.c_char_p, ctypes.c_char_p, _P, _P, SZ, ctypes.POINTER(_P)]
    L.cpm_builder_register_cell_type.argtypes = [_P, ctypes.c_char_p, U32, U32, D, D, D, U32]
    L.cpm_builder_add_cells.argtypes = [_P, ctypes.c_char_p, U64]
    L.cpm_builder_set_adhesion.argtypes = [_P, _P, _P, SZ]
    L.cpm_builder_initialize.argtypes = [_P, _P, SZ, _P, SZ, I32, I32]
    L.cpm_builder_run.argtypes = [_P, U64, U64, U64, I32, ctypes.POINTER(I32), ctypes.POINTER(_P)]
    L.cpm_builder_run_batch.argtypes = [_P, _P, _P, SZ, U64, U64, U64, U64, I32, ctypes.POINTER(I32), _P]
    L.cpm_builder_theta_len.argtypes = [_P, ctypes.POINTER(SZ)]
    L.cpm_builder_extract_theta.argtypes = [_P, _P, SZ]
    L.cpm_builder_theta_name.argtypes = [_P, SZ, ctypes.c_char_p, SZ]
    L.cpm_builder_free.argtypes = [_P]
    L.cpm_builder_free.restype = None
    L.cpm_result_info_get.argtypes = [_P, ctypes.POINTER(ResultInfo)]
    L.cpm_result_metadata_get.argtypes = [_P, ctypes.POINTER(MetadataC)]
    L.cpm_result_status_get.argtypes = [_P, ctypes.POINTER(StatusC)]
    L.cpm_result_cell_type_index.argtypes = [_P, _P]
    L.cpm_result_cell_type_name.argtypes = [_P, SZ, ctypes.c_char_p, SZ]
    L.cpm_result_sample_sizes.argtypes = [_P, SZ, ctypes.POINTER(SampleSizes)]
    L.cpm_result_sample_read.argtypes = [_P, SZ, ctypes.POINTER(SampleOut)]
    L.cpm_result_stats.argtypes = [_P, _P]
    L.cpm_result_free.argtypes = [_P]
    L.cpm_result_free.restype = None
    L.cpm_engine_create.argtypes = [_P, SZ, _P, ctypes.POINTER(_P)]
    L.cpm_engine_size.argtypes = [_P, ctypes.POINTER(SZ)]
    L.cpm_engine_sim_info.argtypes = [_P, SZ, ctypes.POINTER(SimInfo)]
    L.cpm_engine_run_mcs.argtypes = [_P, U64]
    L.cpm_engine_synchronize.argtypes = [_P]
    L.cpm_engine_mcs.argtypes = [_P, SZ, ctypes.POINTER(U64)]
    L.cpm_engine_read_lattice.argtypes = [_P, SZ, _P]
    L.cpm_engine_read_padded.argtypes = [_P, SZ, _P]
    L.cpm_engine_read_cells.argtypes = [_P, SZ, _P, _P, _P, _P]
    L.cpm_engine_energy.argtypes = [_P, SZ, ctypes.POINTER(D)]
    L.cpm_engine_recount_check.argtypes = [_P, SZ, ctypes.POINTER(I32), _P, _P]
    L.cpm_engine_stats.argtypes = [_P, SZ, _P]
    L.cpm_engine_take_sample.argtypes = [_P, SZ, I32, ctypes.POINTER(_P)]
    L.cpm_engine_write_act_state.argtypes = [_P, SZ, _P, U64]
    L.cpm_engine_read_birth.argtypes = [_P, SZ, _P]
    L.cpm_engine_write_state.argtypes = [_P, SZ, _P, _P, _P, _P, _P]
    L.cpm_engine_evaluate_moves.argtypes = [_P, SZ, SZ, _P, _P, _P, _P]
    L.cpm_engine_commit_moves.argtypes = [_P, SZ, SZ, _P, _P]
    L.cpm_engine_destroy.argtypes = [_P]
    L.cpm_engine_destroy.restype = None
    L.cpm_run_many.argtypes = [_P, SZ, U64, U64, U64, I32, I32, _P]
    L.cpm_builder_initial_state.argtypes = [_P, _P, SZ, _P, ctypes.POINTER(SZ), ctypes.POINTER(I32)]
    L.cpm_builder_hashes.argtypes = [_P, U64, U64, U64, _P, SZ, _P, SZ, ctypes.c_char_p, ctypes.c_char_p]
    L.cpm_derive_seed_u64.argtypes = [U64, U64]
    L.cpm_derive_seed_u64.restype = U64
    L.cpm_tuning_report.argtypes = [ctypes.c_char_p, SZ, ctypes.POINTER(SZ)]
    L.cpm_run_status.argtypes = [_P, SZ, SZ, _P, ctypes.c_uint32, _P, _P, _P, SZ, ctypes.c_uint32, _P, _P, _P]
    L.cpm_result_samples_sizes.argtypes = [_P, _P]
    L.cpm_result_samples_read.argtypes = [_P, _P]
    L.cpm_results_samples_read.argtypes = [_P, SZ, _P]
    L.cpm_serve_start.argtypes = [_P, ctypes.POINTER(_P)]
    L.cpm_serve_submit.argtypes = [_P, _P, U64, U64, U64, I32, I32, ctypes.POINTER(U64)]
    L.cpm_serve_poll.argtypes = [_P, U64, ctypes.POINTER(I32), ctypes.POINTER(_P), _P]
    L.cpm_serve_wait.argtypes = [_P, U64, D, ctypes.POINTER(I32), ctypes.POINTER(_P), _P]
    L.cpm_serve_cancel.argtypes = [_P, U64]
    L.cpm_serve_stats_get.argtypes = [_P, _P]
    L.cpm_serve_stop.argtypes = [_P]
    return L


_lib = _load()
LIB_PATH = _LIB_PATH


def lib():
    return _lib


def _check(rc: int):
    if rc == CPM_OK:
        return
    msg = (_lib.cpm_last_error() or b"").decode("utf-8", "replace")
    if rc in (CPM_E_CONFIG, CPM_E_INIT, CPM_E_THETA, CPM_E_ARG, CPM_E_UNSUPPORTED, CPM_E_BUDGET):
        raise ValueError(msg)
    raise CPMRuntimeError(msg)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


def _u64(x, name):
    x = int(x)
    if x < 0 or x >= 2**64:
        raise OverflowError(f"{name}: can't convert {x} to an unsigned 64-bit integer")
    return x


def _u32(x, name):
    x = int(x)
    if x < 0 or x >= 2**32:
        raise OverflowError(f"{name}: can't convert {x} to an unsigned 32-bit integer")
    return x


def _enc(s):
    return None if s is None else str(s).encode("utf-8")


# ----------------------------------------------------------------- results
class RunMetadata:
    """PyRunMetadata (convert.rs:27-38)."""

    __slots__ = ("cpm_version", "convention_version", "convention_hash", "model_hash", "seed", "seed_policy",
                 "derived_phi", "theta_layout_version")

    def __repr__(self):
        return f"RunMetadata(seed={self.seed}, convention_hash={self.convention_hash!r})"


class Status:
    """PyStatus (convert.rs:40-52): kind plus cell_id/at_mcs for CellLost/Fragmented."""

    __slots__ = ("kind", "cell_id", "at_mcs")

    def __repr__(self):
        return f"Status(kind={self.kind!r}, cell_id={self.cell_id}, at_mcs={self.at_mcs})"


class Sample:
    """PySample (convert.rs:54-95): one sample of a run. Its fields are views
    into the arrays its result was read into, made on access. ``contact`` is
    the dense ``(n_cells+1, n_cells+1)`` upper-triangular uint32 matrix,
    built from the engine's sparse pairs on first access."""

    __slots__ = ("_a", "_s", "_lat", "_x", "_contact")

    def __init__(self, arrays, s, lattice, lists):
        # arrays: the result's per-field arrays; lists: (contact offsets,
        # fragmented offsets, medium offsets, fragmented ids, medium volumes,
        # medium boundary flags, mcs, energies) as Python lists
        self._a, self._s, self._lat, self._x, self._contact = arrays, s, lattice, lists, None

    @property
    def mcs(self):
        return self._x[6][self._s]

    @property
    def conservative_energy(self):
        return self._x[7][self._s]

    @property
    def ids(self):
        return self._a["ids"][self._s]

    @property
    def volume(self):
        return self._a["volume"][self._s]

    @property
    def interface(self):
        return self._a["interface"][self._s]

    @property
    def centroid(self):
        return self._a["centroid"][self._s]

    @property
    def eigenvalues(self):
        return self._a["eigenvalues"][self._s]

    @property
    def radius_of_gyration_sq(self):
        return self._a["radius_of_gyration_sq"][self._s]

    @property
    def kappa_sq(self):
        return self._a["kappa_sq"][self._s]

    @property
    def fragmented_cells(self):
        fo = self._x[1]
        return self._x[3][fo[self._s]:fo[self._s + 1]]

    @property
    def medium_component_volumes(self):
        mo = self._x[2]
        return self._x[4][mo[self._s]:mo[self._s + 1]]

    @property
    def medium_component_touches_boundary(self):
        mo = self._x[2]
        return self._x[5][mo[self._s]:mo[self._s + 1]]

    @property
    def lattice(self):
        return self._lat[self._s] if self._lat is not None else None

    @property
    def contact_pairs(self):
        """Sparse form of ``contact``: (a, b, count) arrays with a < b."""
        co = self._x[0]
        c0, c1 = co[self._s], co[self._s + 1]
        return (self._a["contact_a"][c0:c1], self._a["contact_b"][c0:c1], self._a["contact_count"][c0:c1])

    @property
    def contact(self):
        if self._contact is None:
            a, b, n = self.contact_pairs
            m = np.zeros((len(self.ids) + 1, len(self.ids) + 1), dtype=np.uint32)
            m[a.astype(np.int64), b.astype(np.int64)] = n
            self._contact = m
        return self._contact


class RunResult:
    """PyRunResult (convert.rs:97-115)."""

    __slots__ = ("metadata", "status", "samples", "cell_type_index", "cell_type_names", "stats", "used_default")


class SamplesSizesC(ctypes.Structure):
    _fields_ = [("n_samples", ctypes.c_uint64), ("n_cells", ctypes.c_uint64), ("total_contact", ctypes.c_uint64),
                ("total_fragmented", ctypes.c_uint64), ("total_medium", ctypes.c_uint64),
                ("has_lattice", ctypes.c_int32), ("pad", ctypes.c_int32)]


class SamplesOutC(ctypes.Structure):
    _fields_ = [(name, _P) for name in (
        "mcs", "conservative_energy", "ids", "volume", "interface", "centroid", "eigenvalues",
        "radius_of_gyration_sq", "kappa_sq", "contact_offsets", "contact_a", "contact_b", "contact_count",
        "fragmented_offsets", "fragmented_cells", "medium_offsets", "medium_component_volumes",
        "medium_component_touches_boundary", "lattice",
    )]


# cpm_samples_out fields: (name, dtype, extent) with extent "s" = samples,
# "s1" = samples + 1 offsets, "sn" = samples x cells, "snD" = samples x cells
# x D, "c"/"f"/"m" = the concatenated contact / fragmented / medium lists.
_SAMPLE_FIELDS = (
    ("mcs", np.uint64, "s"), ("conservative_energy", np.float64, "s"), ("ids", np.uint32, "sn"),
    ("volume", np.uint32, "sn"), ("interface", np.uint32, "sn"), ("centroid", np.float64, "snD"),
    ("eigenvalues", np.float64, "snD"), ("radius_of_gyration_sq", np.float64, "sn"), ("kappa_sq", np.float64, "sn"),
    ("contact_offsets", np.uint64, "s1"), ("contact_a", np.uint32, "c"), ("contact_b", np.uint32, "c"),
    ("contact_count", np.uint32, "c"), ("fragmented_offsets", np.uint64, "s1"), ("fragmented_cells", np.uint32, "f"),
    ("medium_offsets", np.uint64, "s1"), ("medium_component_volumes", np.uint32, "m"),
    ("medium_component_touches_boundary", np.uint8, "m"),
)


def _read_samples_many(hs, dims):
    """The samples of many results: one array per field for all of them,
    filled by one cpm_results_samples_read call (spread over the host's
    cores); every Sample's arrays are views into those arrays."""
    N = len(hs)
    sizes = []
    for h, (ns, _, _, _) in zip(hs, dims):
        sz = SamplesSizesC()
        if ns:
            _check(_lib.cpm_result_samples_sizes(h, ctypes.byref(sz)))
        sizes.append(sz)
    counts = []
    for (ns, n, D, _), sz in zip(dims, sizes):
        counts.append({"s": ns, "s1": ns + 1 if ns else 0, "sn": ns * n, "snD": ns * n * D,
                       "c": int(sz.total_contact), "f": int(sz.total_fragmented), "m": int(sz.total_medium)})
    big, starts = {}, {}
    for name, dt, ext in _SAMPLE_FIELDS:
        st, t = [], 0
        for c in counts:
            st.append(t)
            t += c[ext]
        big[name], starts[name] = np.zeros(t, dt), st
    lat_n = [ns * int(np.prod(grid)) if sz.has_lattice else 0 for (ns, _, _, grid), sz in zip(dims, sizes)]
    lat_start = np.concatenate([[0], np.cumsum(lat_n)]).astype(np.int64).tolist()
    big_lat = np.zeros(lat_start[-1], np.uint32)
    outs = (SamplesOutC * max(N, 1))()
    for k in range(N):
        o = outs[k]
        for name, dt, ext in _SAMPLE_FIELDS:
            if counts[k][ext]:
                setattr(o, name, big[name].ctypes.data + starts[name][k] * big[name].itemsize)
        if lat_n[k]:
            o.lattice = big_lat.ctypes.data + lat_start[k] * 4
    if N:
        harr = (_P * N)(*hs)
        _check(_lib.cpm_results_samples_read(ctypes.cast(harr, _P), N, ctypes.cast(outs, _P)))
    result = []
    for k, ((ns, n, D, grid), c) in enumerate(zip(dims, counts)):
        if ns == 0:
            result.append([])
            continue
        a = {name: big[name][starts[name][k]:starts[name][k] + c[ext]] for name, _, ext in _SAMPLE_FIELDS}
        for name in ("ids", "volume", "interface", "radius_of_gyration_sq", "kappa_sq"):
            a[name] = a[name].reshape(ns, n)
        for name in ("centroid", "eigenvalues"):
            a[name] = a[name].reshape(ns, n, D)
        lat = big_lat[lat_start[k]:lat_start[k + 1]].reshape((ns,) + tuple(grid)) if lat_n[k] else None
        lists = (a["contact_offsets"].tolist(), a["fragmented_offsets"].tolist(), a["medium_offsets"].tolist(),
                 a["fragmented_cells"].tolist(), a["medium_component_volumes"].tolist(),
                 [bool(x) for x in a["medium_component_touches_boundary"]], a["mcs"].tolist(),
                 a["conservative_energy"].tolist())
        out = [Sample(a, s, lat, lists) for s in range(ns)]
        result.append(out)
    return result


def _result_head(h):
    """Everything of a result but its samples, and the samples' dimensions."""
    info = ResultInfo()
    _check(_lib.cpm_result_info_get(h, ctypes.byref(info)))
    D, n = info.dim, int(info.n_cells)
    grid = tuple(int(info.grid[d]) for d in range(D))
    md = MetadataC()
    _check(_lib.cpm_result_metadata_get(h, ctypes.byref(md)))
    meta = RunMetadata()
    meta.cpm_version = md.cpm_version.decode()
    meta.convention_version = int(md.convention_version)
    meta.convention_hash = md.convention_hash.decode()
    meta.model_hash = md.model_hash.decode()
    meta.seed = int(md.seed)
    meta.seed_policy = md.seed_policy.decode()
    meta.derived_phi = float(md.derived_phi)
    meta.theta_layout_version = int(md.theta_layout_version)
    st = StatusC()
    _check(_lib.cpm_result_status_get(h, ctypes.byref(st)))
    status = Status()
    status.kind = st.kind.decode()
    status.cell_id = int(st.cell_id) if st.has_cell else None
    status.at_mcs = int(st.at_mcs) if st.has_cell else None
    cti = np.zeros(n, dtype=np.uint32)
    _check(_lib.cpm_result_cell_type_index(h, _ptr(cti)))
    names = []
    buf = ctypes.create_string_buffer(4096)
    for t in range(info.n_types):
        _check(_lib.cpm_result_cell_type_name(h, t, buf, 4096))
        names.append(buf.value.decode("utf-8"))
    stats = np.zeros(32, dtype=np.uint64)
    _check(_lib.cpm_result_stats(h, _ptr(stats)))
    r = RunResult()
    r.metadata, r.status, r.samples = meta, status, []
    r.cell_type_index, r.cell_type_names = cti, names
    r.used_default = bool(info.used_default)
    r.stats = {name: int(v) for name, v in zip(STAT_NAMES, stats.tolist())}
    return r, (int(info.n_samples), n, D, grid)


def _results_from_handles(hs) -> list:
    """Python results of result handles (freed here, also on errors)."""
    try:
        heads = [_result_head(h) for h in hs]
        for (r, _), smp in zip(heads, _read_samples_many(hs, [d for _, d in heads])):
            r.samples = smp
        return [r for r, _ in heads]
    finally:
        for h in hs:
            _lib.cpm_result_free(h)


def _result_from_handle(h) -> RunResult:
    return _results_from_handles([h])[0]


# ----------------------------------------------------------------- builder
class CPM:
    """The compiled builder (builder.rs:104-401), backed by libcpm_gpu.so."""

    def __init__(self, grid, boundary, seed, copy_neighborhood="von_neumann", energy_neighborhood=None,
                 connectivity_neighborhood="von_neumann", acceptance=None, proposal=None, active_terms=None):
        g = np.ascontiguousarray([_u64(x, "grid") for x in grid], dtype=np.uint64)
        keys, vals = [], []
        for k, v in (active_terms or {}).items():
            keys.append(str(k).encode("utf-8"))
            vals.append(1 if v else 0)
        karr = (ctypes.c_char_p * max(len(keys), 1))(*keys) if keys else None
        varr = np.ascontiguousarray(vals, dtype=np.int32) if vals else None
        h = _P()
        self._h = None
        _check(_lib.cpm_builder_new(
            _ptr(g) if g.size else None, g.size, _enc(boundary), _u64(seed, "seed"), _enc(copy_neighborhood),
            _enc(energy_neighborhood), _enc(connectivity_neighborhood), _enc(acceptance), _enc(proposal),
            ctypes.cast(karr, _P) if karr is not None else None, _ptr(varr) if varr is not None else None,
            len(keys), ctypes.byref(h)))
        self._h = h
        self._grid = tuple(int(x) for x in grid)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.cpm_builder_free(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def register_cell_type(self, name, target_volume, target_interface, lambda_volume, lambda_interface,
                           lambda_act=0.0, max_act=0):
        _check(_lib.cpm_builder_register_cell_type(
            self._h, _enc(name), _u32(target_volume, "target_volume"), _u32(target_interface, "target_interface"),
            float(lambda_volume), float(lambda_interface), float(lambda_act), _u32(max_act, "max_act")))

    def add_cells(self, cell_type, n):
        _check(_lib.cpm_builder_add_cells(self._h, _enc(cell_type), _u64(n, "n")))

    def set_adhesion(self, matrix):
        rows = [[float(x) for x in row] for row in matrix]
        lens = np.ascontiguousarray([len(r) for r in rows], dtype=np.uintp)
        vals = np.ascontiguousarray([x for r in rows for x in r], dtype=np.float64)
        _check(_lib.cpm_builder_set_adhesion(self._h, _ptr(vals) if vals.size else None,
                                             _ptr(lens) if lens.size else None, len(rows)))

    def initialize(self, lattice=None, cell_type_of=None, warn_on_default_init=True):
        if lattice is not None:
            lat = np.ascontiguousarray([_u32(x, "lattice") for x in lattice], dtype=np.uint32)
            has = cell_type_of is not None
            cto = np.ascontiguousarray([_u64(x, "cell_type_of") for x in (cell_type_of or [])], dtype=np.uint64)
            _check(_lib.cpm_builder_initialize(self._h, _ptr(lat) if lat.size else _ptr(np.zeros(1, np.uint32)),
                                               lat.size, _ptr(cto) if cto.size else None, cto.size, int(has),
                                               int(bool(warn_on_default_init))))
        else:
            _check(_lib.cpm_builder_initialize(self._h, None, 0, None, 0, 0, int(bool(warn_on_default_init))))

    def run(self, burn_in_mcs, readout_mcs, sampling_interval_mcs, include_lattice=False):
        used = ctypes.c_int32(0)
        h = _P()
        _check(_lib.cpm_builder_run(self._h, _u64(burn_in_mcs, "burn_in_mcs"), _u64(readout_mcs, "readout_mcs"),
                                    _u64(sampling_interval_mcs, "sampling_interval_mcs"), int(bool(include_lattice)),
                                    ctypes.byref(used), ctypes.byref(h)))
        return bool(used.value), _result_from_handle(h)

    def run_batch(self, thetas, burn_in_mcs, readout_mcs, sampling_interval_mcs, master_seed, include_lattice=False):
        rows = [[float(x) for x in th] for th in thetas]
        lens = np.ascontiguousarray([len(r) for r in rows], dtype=np.uintp)
        vals = np.ascontiguousarray([x for r in rows for x in r], dtype=np.float64)
        out = (_P * max(len(rows), 1))()
        anyd = ctypes.c_int32(0)
        _check(_lib.cpm_builder_run_batch(
            self._h, _ptr(vals) if vals.size else None, _ptr(lens) if lens.size else None, len(rows),
            _u64(burn_in_mcs, "burn_in_mcs"), _u64(readout_mcs, "readout_mcs"),
            _u64(sampling_interval_mcs, "sampling_interval_mcs"), _u64(master_seed, "master_seed"),
            int(bool(include_lattice)), ctypes.byref(anyd), ctypes.cast(out, _P)))
        return bool(anyd.value), _results_from_handles([_P(out[i]) for i in range(len(rows))])

    def initial_state(self):
        """Placement without a simulation: (lattice, cell_type_of, used_default).
        An explicit lattice of 65,536 sites or more (CPM_GPU_INIT_DEVICE_MIN_SITES)
        is checked on the device when the process has one."""
        n_sites = int(np.prod(self._grid))
        lat = np.zeros(n_sites, dtype=np.uint32)
        # every cell holds at least one site, so n_sites bounds the cell count:
        # one placement fills both buffers
        cto = np.zeros(max(n_sites, 1), dtype=np.uint32)
        n = ctypes.c_size_t(cto.size)
        used = ctypes.c_int32(0)
        _check(_lib.cpm_builder_initial_state(self._h, _ptr(lat), n_sites, _ptr(cto), ctypes.byref(n),
                                              ctypes.byref(used)))
        return lat.reshape(self._grid), cto[: n.value].copy(), bool(used.value)

    def hashes(self, burn_in_mcs, readout_mcs, sampling_interval_mcs, lattice, cell_type_of):
        """(convention_hash, model_hash) for the given windows and lattice."""
        lat = np.ascontiguousarray(np.asarray(lattice, dtype=np.uint32).ravel())
        cto = np.ascontiguousarray(np.asarray(cell_type_of, dtype=np.uint32))
        ch = ctypes.create_string_buffer(65)
        mh = ctypes.create_string_buffer(65)
        _check(_lib.cpm_builder_hashes(self._h, burn_in_mcs, readout_mcs, sampling_interval_mcs, _ptr(lat), lat.size,
                                       _ptr(cto) if cto.size else None, cto.size, ch, mh))
        return ch.value.decode(), mh.value.decode()

    def theta_names(self):
        n = ctypes.c_size_t(0)
        _check(_lib.cpm_builder_theta_len(self._h, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(4096)
        names = []
        for i in range(n.value):
            _check(_lib.cpm_builder_theta_name(self._h, i, buf, 4096))
            names.append(buf.value.decode("utf-8"))
        return names

    def extract_theta(self):
        n = ctypes.c_size_t(0)
        _check(_lib.cpm_builder_theta_len(self._h, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=np.float64)
        _check(_lib.cpm_builder_extract_theta(self._h, _ptr(out), n.value))
        return out.tolist()


def derive_seed_u64(master_seed: int, index: int) -> int:
    return int(_lib.cpm_derive_seed_u64(_u64(master_seed, "master_seed"), _u64(index, "index")))


STATUS_KINDS = ("Ok", "NotEquilibrated", "Fragmented", "CellLost", "Degenerate")


def tuning_report():
    """The tiled sweep's grid tuner table (``cpm_tuning_report``), parsed."""
    import json

    need = ctypes.c_size_t(0)
    _check(_lib.cpm_tuning_report(None, 0, ctypes.byref(need)))
    buf = ctypes.create_string_buffer(int(need.value) + 1)
    _check(_lib.cpm_tuning_report(buf, len(buf), ctypes.byref(need)))
    return json.loads(buf.value.decode())


def run_status(trace, sample_mcs, volumes, first_fragmented=None, last_pairs=(), min_cell_volume=1):
    """The status rule ``run`` applies (output.rs:456-522) on given readouts;
    see ``cpm_run_status``. Returns (kind, cell_id, at_mcs)."""
    t = np.ascontiguousarray(trace, dtype=np.float64)
    m = np.ascontiguousarray(sample_mcs, dtype=np.uint64)
    v = np.ascontiguousarray(volumes, dtype=np.uint32)
    if v.ndim != 2 or v.shape[0] != m.size:
        raise ValueError("volumes: one row of cell volumes per sample")
    f = None if first_fragmented is None else np.ascontiguousarray(first_fragmented, dtype=np.uint32)
    p = np.ascontiguousarray(np.asarray(last_pairs, dtype=np.uint32).reshape(-1, 2))
    kind, cid, at = ctypes.c_int32(0), ctypes.c_uint32(0), ctypes.c_uint64(0)
    _check(_lib.cpm_run_status(_ptr(t), t.size, m.size, _ptr(m), v.shape[1], _ptr(v),
                               _ptr(f) if f is not None else None, _ptr(p), len(p), int(min_cell_volume),
                               ctypes.byref(kind), ctypes.byref(cid), ctypes.byref(at)))
    return STATUS_KINDS[kind.value], cid.value, at.value


def run_many(builders, burn_in_mcs, readout_mcs, sampling_interval_mcs, include_lattice=False, topology=True):
    """Runs one simulation per builder (each with its own grid, parameters and
    seed) in one persistent device launch; see ``cpm_run_many``."""
    hs = (_P * max(len(builders), 1))(*[b.handle for b in builders])
    out = (_P * max(len(builders), 1))()
    _check(_lib.cpm_run_many(ctypes.cast(hs, _P), len(builders), _u64(burn_in_mcs, "burn_in_mcs"),
                             _u64(readout_mcs, "readout_mcs"), _u64(sampling_interval_mcs, "sampling_interval_mcs"),
                             int(bool(include_lattice)), int(bool(topology)), ctypes.cast(out, _P)))
    return _results_from_handles([_P(out[i]) for i in range(len(builders))])


class Engine:
    """Device-resident simulations driven MCS by MCS (the run_mcs seam)."""

    def __init__(self, builders, stream=None):
        if isinstance(builders, CPM):
            builders = [builders]
        self._builders = list(builders)
        hs = (_P * len(self._builders))(*[b.handle for b in self._builders])
        h = _P()
        self._h = None
        _check(_lib.cpm_engine_create(ctypes.cast(hs, _P), len(self._builders),
                                      _P(stream) if stream else None, ctypes.byref(h)))
        self._h = h
        self.info = []
        for i in range(len(self._builders)):
            si = SimInfo()
            _check(_lib.cpm_engine_sim_info(self._h, i, ctypes.byref(si)))
            self.info.append(si)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.cpm_engine_destroy(h)
            self._h = None

    def __len__(self):
        return len(self.info)

    def run_mcs(self, n: int):
        _check(_lib.cpm_engine_run_mcs(self._h, _u64(n, "n")))

    def synchronize(self):
        _check(_lib.cpm_engine_synchronize(self._h))

    def mcs(self, i=0):
        v = ctypes.c_uint64(0)
        _check(_lib.cpm_engine_mcs(self._h, i, ctypes.byref(v)))
        return v.value

    def lattice(self, i=0):
        si = self.info[i]
        out = np.zeros(int(si.n_sites), dtype=np.uint32)
        _check(_lib.cpm_engine_read_lattice(self._h, i, _ptr(out)))
        return out.reshape([int(si.dims[d]) for d in range(si.dim)])

    def padded(self, i=0):
        out = np.zeros(int(self.info[i].n_padded), dtype=np.uint32)
        _check(_lib.cpm_engine_read_padded(self._h, i, _ptr(out)))
        return out

    def cells(self, i=0):
        si = self.info[i]
        n1, D = int(si.n_cells) + 1, si.dim
        v = np.zeros(n1, np.uint32)
        it = np.zeros(n1, np.uint32)
        sp = np.zeros(n1 * D, np.int64)
        so = np.zeros(n1 * D * D, np.int64)
        _check(_lib.cpm_engine_read_cells(self._h, i, _ptr(v), _ptr(it), _ptr(sp), _ptr(so)))
        return v, it, sp.reshape(n1, D), so.reshape(n1, D, D)

    def energy(self, i=0):
        e = ctypes.c_double(0.0)
        _check(_lib.cpm_engine_energy(self._h, i, ctypes.byref(e)))
        return e.value

    def recount_check(self, i=0):
        n1 = int(self.info[i].n_cells) + 1
        okv = ctypes.c_int32(0)
        v = np.zeros(n1, np.uint32)
        it = np.zeros(n1, np.uint32)
        _check(_lib.cpm_engine_recount_check(self._h, i, ctypes.byref(okv), _ptr(v), _ptr(it)))
        return bool(okv.value), v, it

    def stats(self, i=0):
        s = np.zeros(32, np.uint64)
        _check(_lib.cpm_engine_stats(self._h, i, _ptr(s)))
        return {name: int(s[k]) for k, name in enumerate(STAT_NAMES)}

    def write_act_state(self, birth=None, mcs=0, i=0):
        """Act term harness: per-site acquisition MCS (padded indexing; None
        keeps it) and the completed-MCS counter (energy.rs:329-471)."""
        b = np.ascontiguousarray(birth, dtype=np.uint32) if birth is not None else None
        _check(_lib.cpm_engine_write_act_state(self._h, i, _ptr(b) if b is not None else None, int(mcs)))

    def read_birth(self, i=0):
        out = np.zeros(int(self.info[i].n_padded), np.uint32)
        _check(_lib.cpm_engine_read_birth(self._h, i, _ptr(out)))
        return out

    def take_sample(self, i=0, include_lattice=False):
        """One Sample of the current state (output.rs:304-337), every readout
        computed on the device; its energy is the global energy of the state."""
        h = _P()
        _check(_lib.cpm_engine_take_sample(self._h, i, 1 if include_lattice else 0, ctypes.byref(h)))
        return _result_from_handle(h).samples[0]

    def write_state(self, padded, volume, interface, sum_position=None, sum_outer=None, i=0):
        p = np.ascontiguousarray(padded, dtype=np.uint32)
        v = np.ascontiguousarray(volume, dtype=np.uint32)
        it = np.ascontiguousarray(interface, dtype=np.uint32)
        sp = np.ascontiguousarray(sum_position, dtype=np.int64) if sum_position is not None else None
        so = np.ascontiguousarray(sum_outer, dtype=np.int64) if sum_outer is not None else None
        _check(_lib.cpm_engine_write_state(self._h, i, _ptr(p), _ptr(v), _ptr(it),
                                           _ptr(sp) if sp is not None else None,
                                           _ptr(so) if so is not None else None))

    def evaluate_moves(self, target, k, u, i=0):
        t = np.ascontiguousarray(target, dtype=np.int64)
        kk = np.ascontiguousarray(k, dtype=np.int32)
        uu = np.ascontiguousarray(u, dtype=np.float64)
        out = np.zeros(t.size, dtype=MOVE_DTYPE)
        _check(_lib.cpm_engine_evaluate_moves(self._h, i, t.size, _ptr(t), _ptr(kk), _ptr(uu), _ptr(out)))
        return out

    def commit_moves(self, target, gaining, i=0):
        t = np.ascontiguousarray(target, dtype=np.int64)
        g = np.ascontiguousarray(gaining, dtype=np.uint32)
        _check(_lib.cpm_engine_commit_moves(self._h, i, t.size, _ptr(t), _ptr(g)))


# ------------------------------------------------------------- serving ----
class ServeOptionsC(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_active", ctypes.c_int32),
                ("placement_threads", ctypes.c_int32), ("tiled_grid_cap", ctypes.c_int32), ("pad", ctypes.c_int32)]


class RequestTimes(ctypes.Structure):
    _fields_ = [("submitted_s", ctypes.c_double), ("admitted_s", ctypes.c_double), ("device_done_s", ctypes.c_double),
                ("finished_s", ctypes.c_double), ("device_bytes", ctypes.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServeStatsC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "failed", "cancelled", "launched", "active",
                                               "queued", "peak_active", "bytes_in_use", "peak_bytes")] + \
               [("busy_seconds", ctypes.c_double)]


REQ_STATES = ("placing", "queued", "running", "done", "failed", "cancelled")


class Server:
    """The serving loop (``cpm_serve_*``): submit simulations at any time;
    they share the device by continuous batching and each result equals the
    one ``CPM.run`` gives for the same builder and window."""

    def __init__(self, hbm_budget_bytes=0, max_active=0, placement_threads=0, tiled_grid_cap=0):
        o = ServeOptionsC(int(hbm_budget_bytes), int(max_active), int(placement_threads), int(tiled_grid_cap), 0)
        h = _P()
        self._h = None
        _check(_lib.cpm_serve_start(ctypes.byref(o), ctypes.byref(h)))
        self._h = h

    def submit(self, builder, burn_in_mcs, readout_mcs, sampling_interval_mcs, include_lattice=False,
               topology=True) -> int:
        t = ctypes.c_uint64(0)
        _check(_lib.cpm_serve_submit(self._h, builder.handle, _u64(burn_in_mcs, "burn_in_mcs"),
                                     _u64(readout_mcs, "readout_mcs"),
                                     _u64(sampling_interval_mcs, "sampling_interval_mcs"), int(bool(include_lattice)),
                                     int(bool(topology)), ctypes.byref(t)))
        return int(t.value)

    def poll(self, ticket):
        """(state, result or None, times): non-blocking; a done result is
        handed over once."""
        st = ctypes.c_int32(0)
        out = _P()
        tm = RequestTimes()
        _check(_lib.cpm_serve_poll(self._h, int(ticket), ctypes.byref(st), ctypes.byref(out), ctypes.byref(tm)))
        res = _result_from_handle(out) if out.value else None
        return REQ_STATES[st.value], res, tm.as_dict()

    def wait(self, ticket, timeout=None):
        """(state, result or None, times) once the request has finished (or
        the timeout, in seconds, passed)."""
        st = ctypes.c_int32(0)
        out = _P()
        tm = RequestTimes()
        _check(_lib.cpm_serve_wait(self._h, int(ticket), -1.0 if timeout is None else float(timeout),
                                   ctypes.byref(st), ctypes.byref(out), ctypes.byref(tm)))
        res = _result_from_handle(out) if out.value else None
        return REQ_STATES[st.value], res, tm.as_dict()

    def cancel(self, ticket):
        _check(_lib.cpm_serve_cancel(self._h, int(ticket)))

    def stats(self):
        s = ServeStatsC()
        _check(_lib.cpm_serve_stats_get(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def close(self):
        if self._h:
            h, self._h = self._h, None
            _lib.cpm_serve_stop(h)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

