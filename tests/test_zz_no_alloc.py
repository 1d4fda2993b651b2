"""The allocation-free sweep entry point, checked against the engine.

Some callers cannot call cudaMalloc while they run (a host framework that
owns all device memory through its own pool, or a service that reserves all
memory up front and treats later allocations as failures). For them
`cpm_run_mcs_noalloc` advances a simulation whose buffers the caller already
holds on the device, with the engine's scratch in a static 1 MiB device array
instead of fresh allocations. Here the caller's buffers are torch tensors;
two calls in a row must leave exactly the state (lattice, volumes,
interfaces, position sums, counters) that `cpm_engine_run_mcs` produces for
the same simulation — the sweep is deterministic, so the tolerance is zero.
This file sorts last so a run that stops at the first failure has already
run every other test.
"""

import ctypes

import numpy as np
import pytest

from helpers import sorting_model

pytestmark = pytest.mark.gpu


class DeviceSim(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("periodic", ctypes.c_int32),
        ("dims", ctypes.c_int64 * 3),
        ("energy_neighborhood", ctypes.c_int32),
        ("n_types", ctypes.c_int32),
        ("n_cells", ctypes.c_uint32),
        ("min_cell_volume", ctypes.c_uint32),
        ("seed", ctypes.c_uint64),
        ("mcs", ctypes.c_uint64),
        ("sigma", ctypes.c_void_p),
        ("type_plus_one", ctypes.c_void_p),
        ("volume", ctypes.c_void_p),
        ("interface", ctypes.c_void_p),
        ("sum_position", ctypes.c_void_p),
        ("sum_position_outer", ctypes.c_void_p),
        ("adhesion", ctypes.c_void_p),
        ("lambda_volume", ctypes.c_void_p),
        ("lambda_interface", ctypes.c_void_p),
        ("target_volume", ctypes.c_void_p),
        ("target_interface", ctypes.c_void_p),
        ("stats", ctypes.c_void_p),
    ]


def _lib():
    from cpm import _cpm

    lib = ctypes.CDLL(_cpm.LIB_PATH)
    lib.cpm_run_mcs_noalloc.argtypes = [ctypes.POINTER(DeviceSim), ctypes.c_uint64, ctypes.c_void_p]
    lib.cpm_run_mcs_noalloc.restype = ctypes.c_int
    lib.cpm_last_error.restype = ctypes.c_char_p
    return lib


def _check_two_calls(model, builder, cto, mcs, with_stats=True):
    """Two calls of the no-allocation entry point against the engine on the
    same simulation (the engine built from `builder`); `with_stats` False
    passes no counters (the static scratch then holds them)."""
    import torch

    from cpm import _cpm

    torch.cuda.set_device(0)
    eng = _cpm.Engine(builder)
    info = eng.info[0]
    n1 = int(info.n_cells) + 1

    # caller-owned device buffers, initialised with the engine's starting state
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    sigma = dev(eng.padded().view(np.int32))
    v0, i0, sp0, so0 = eng.cells()
    vol = dev(v0.view(np.int32))
    itf = dev(i0.view(np.int32))
    sp = dev(sp0.ravel())
    so = dev(so0.ravel())
    tp1 = dev(np.concatenate([[0], np.asarray(cto, np.int64) + 1]).astype(np.int16))
    adh = dev(np.asarray(model.adhesion, np.float64).ravel())
    lam_v = dev(np.array([t[3] for t in model.types], np.float64))
    lam_i = dev(np.array([t[4] for t in model.types], np.float64))
    tv = dev(np.array([t[1] for t in model.types], np.int32))
    ti = dev(np.array([t[2] for t in model.types], np.int32))
    stats = torch.zeros(32, dtype=torch.int64, device="cuda") if with_stats else None  # CPM_STAT_COUNT counters
    torch.cuda.synchronize()

    ds = DeviceSim()
    ds.dim, ds.periodic = 2, 1
    ds.dims[0], ds.dims[1], ds.dims[2] = model.grid[0], model.grid[1], 1
    ds.energy_neighborhood = 1  # Moore
    ds.n_types, ds.n_cells, ds.min_cell_volume = len(model.types), n1 - 1, 1
    ds.seed, ds.mcs = model.seed, 0
    for name, t in (("sigma", sigma), ("type_plus_one", tp1), ("volume", vol), ("interface", itf),
                    ("sum_position", sp), ("sum_position_outer", so), ("adhesion", adh), ("lambda_volume", lam_v),
                    ("lambda_interface", lam_i), ("target_volume", tv), ("target_interface", ti), ("stats", stats)):
        setattr(ds, name, t.data_ptr() if t is not None else None)

    lib = _lib()
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        rc = lib.cpm_run_mcs_noalloc(ctypes.byref(ds), mcs, ctypes.c_void_p(stream))
        assert rc == 0, lib.cpm_last_error().decode()
        torch.cuda.synchronize()
        assert ds.mcs == mcs * (call + 1)
        eng.run_mcs(mcs)
        eng.synchronize()
        ev, ei, esp, eso = eng.cells()
        assert np.array_equal(sigma.cpu().numpy().view(np.uint32), eng.padded())
        assert np.array_equal(vol.cpu().numpy().view(np.uint32), ev)
        assert np.array_equal(itf.cpu().numpy().view(np.uint32), ei)
        assert np.array_equal(sp.cpu().numpy(), esp.ravel())
        assert np.array_equal(so.cpu().numpy(), eso.ravel())
        st = eng.stats()
        assert st["attempts"] == mcs * (call + 1) * int(info.n_sites)
        if with_stats:
            got = stats.cpu().numpy()
            assert got[0] == st["attempts"]
            assert got[5] == st["accepted"]
    assert eng.recount_check()[0]


def test_noalloc_sweep_matches_engine_on_two_calls(cuda_required):
    model = sorting_model(side=48, seed=4)
    _, cto, _ = model.builder().initial_state()
    _check_two_calls(model, model.builder(), cto, 10)


def test_noalloc_without_counters_matches_engine(cuda_required):
    """No counters passed: the sweep keeps them in the static scratch, and
    the state after two calls is still the engine's."""
    model = sorting_model(side=40, seed=6)
    _, cto, _ = model.builder().initial_state()
    _check_two_calls(model, model.builder(), cto, 7, with_stats=False)


def test_noalloc_above_the_resident_size_runs_the_global_sweep(cuda_required, monkeypatch):
    """A 320x320 lattice does not fit one SM: the entry point runs the
    one-CTA global-memory sweep, which is the engine's chain when the
    engine is forced onto that sweep."""
    monkeypatch.setenv("CPM_GPU_FORCE_GLOBAL", "1")
    model = sorting_model(side=320, seed=8)
    _, cto, _ = model.builder().initial_state()
    _check_two_calls(model, model.builder(), cto, 2)


def test_noalloc_many_cells_keep_their_slots_in_the_static_scratch(cuda_required, monkeypatch):
    """28,900 cells (2x2 blocks filling a 340x340 lattice) exceed what the
    global-memory sweep keeps in shared memory, so their conflict slots live
    in the static scratch array; the state still equals the engine's on the
    same sweep."""
    from helpers import Model

    monkeypatch.setenv("CPM_GPU_FORCE_GLOBAL", "1")
    side = 340
    r = np.arange(side) // 2
    lat = (r[:, None] * (side // 2) + r[None, :] + 1).astype(np.uint32)
    n = (side // 2) ** 2
    cto = [k % 2 for k in range(n)]
    model = Model((side, side), "periodic", [("a", 4, 8, 2.0, 0.5), ("b", 4, 8, 2.0, 0.5)],
                  [[0, 10, 10], [10, 3, 6], [10, 6, 4]], [0, 0], seed=9)
    _check_two_calls(model, model.builder(lattice=lat, cell_type_of=cto), cto, 2)


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda_required):
    lib = _lib()
    ds = DeviceSim()
    ds.dim, ds.periodic = 2, 1
    ds.dims[0], ds.dims[1] = 1024, 1024
    ds.energy_neighborhood, ds.n_types, ds.n_cells, ds.min_cell_volume = 1, 1, 200000, 1
    for name in ("sigma", "type_plus_one", "volume", "interface", "sum_position", "sum_position_outer", "adhesion",
                 "lambda_volume", "lambda_interface", "target_volume", "target_interface"):
        setattr(ds, name, 16)  # never dereferenced: the size check comes first
    rc = lib.cpm_run_mcs_noalloc(ctypes.byref(ds), 1, None)
    assert rc == 6  # CPM_E_BUDGET
    assert "exceed the scratch limit of 130559 cells" in lib.cpm_last_error().decode()
    ds.dim = 3
    assert lib.cpm_run_mcs_noalloc(ctypes.byref(ds), 1, None) == 8  # CPM_E_UNSUPPORTED
