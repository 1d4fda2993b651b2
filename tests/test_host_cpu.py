"""Host-side logic of the GB300 engine, checked on the CPU (no device work).

* libcpm_gpu.so loads and exports every symbol include/cpm_gpu.h declares;
* default placement (scatter-and-grow) equals the oracle's, site for site,
  so a device run starts from the reference's own initial lattice;
* derived seeds and the model hash reproduce the reference's known answers;
* configuration errors surface as ValueError with the reference's messages
  (tests/python/test_errors.py:8-51) and theta has the canonical layout
  (tests/python/test_batch.py:26-37);
* the C ABI answers null buffers with CPM_E_ARG.
"""

import ctypes
import re
import warnings

import numpy as np
import pytest

from helpers import Model, c1_model, organoid_model, sorting_model
from kat_fixtures import DERIVED_SEEDS_42, FROZEN_ADHESION, FROZEN_MCS, FROZEN_MODEL_HASH, FROZEN_SEED, FROZEN_TYPES, frozen_lattice


def test_library_exports_every_declared_symbol():
    from cpm import _cpm

    header = open(_cpm.__file__.replace("cpm-rust_gb300/python/cpm/_cpm.py", "include/cpm_gpu.h")).read()
    declared = set(re.findall(r"\b(cpm_[a-z0-9_]+)\s*\(", header))
    assert declared == set(_cpm.EXPORTED_SYMBOLS)
    lib = ctypes.CDLL(_cpm.LIB_PATH)
    for name in declared:
        assert hasattr(lib, name), name


@pytest.mark.parametrize("model_fn", [
    lambda: c1_model(seed=1),
    lambda: c1_model(seed=77),
    lambda: Model((30, 30), "fixed", [("e", 50, 75, 10.0, 2.0)], [[0, 5], [5, 2]], [5], seed=2),
    lambda: sorting_model(side=64, seed=4),
    lambda: organoid_model(side=20),
    lambda: organoid_model(side=15, boundary="fixed", counts=(4, 3)),
])
def test_default_placement_matches_oracle(model_fn):
    m = model_fn()
    lat, cto, used = m.builder().initial_state()
    ref = m.oracle()
    assert used
    assert np.array_equal(lat, ref.lattice())
    assert np.array_equal(cto, ref.type_of())


def test_explicit_placement_errors_match_reference():
    m = c1_model()
    lat = np.zeros((30, 30), dtype=np.uint32)
    lat[0, 0] = 1
    lat[5, 5] = 1  # disconnected
    with pytest.raises(ValueError, match="is not connected"):
        m.builder(lattice=lat, cell_type_of=[0]).initial_state()
    with pytest.raises(ValueError, match="has zero volume"):
        m.builder(lattice=np.zeros((30, 30), np.uint32), cell_type_of=[0]).initial_state()
    with pytest.raises(ValueError, match="expected N_sites = 900"):
        m.builder(lattice=np.zeros(10, np.uint32), cell_type_of=[0]).initial_state()


def test_explicit_placement_errors_on_a_large_lattice_without_a_gpu():
    """Explicit lattices of 65,536 sites or more are checked on the device
    when the process has one, else on the host (as here, without a GPU);
    either way the reference's messages in its order (range, zero volume,
    connectivity; tests/test_gpu_init.py compares the two paths)."""
    m = Model((256, 256), "periodic", [("a", 50, 75, 10.0, 2.0)], [[0, 5], [5, 2]], [3])
    lat = np.zeros((256, 256), dtype=np.uint32)
    lat[10:14, 10:14] = 1
    lat[100:104, 100:104] = 2
    lat[200, 200] = 2  # cell 2 split
    lat[0:3, 250:256] = 3
    lat[0:3, 0:2] = 3  # cell 3 joined across the periodic edge
    with pytest.raises(ValueError, match="^cell 2 is not connected under connectivity_neighborhood"):
        m.builder(lattice=lat, cell_type_of=[0, 0, 0]).initial_state()
    lat[200, 200] = 0
    lat2, cto, used = m.builder(lattice=lat, cell_type_of=[0, 0, 0]).initial_state()
    assert not used and np.array_equal(lat2, lat)
    lat[100:104, 100:104] = 0
    with pytest.raises(ValueError, match="^cell 2 has zero volume in the supplied lattice$"):
        m.builder(lattice=lat, cell_type_of=[0, 0, 0]).initial_state()
    lat[255, 255] = 7
    with pytest.raises(ValueError, match="^lattice references cell id 7, but cell_type_of only covers 3 cells$"):
        m.builder(lattice=lat, cell_type_of=[0, 0, 0]).initial_state()


def test_crowded_scatter_reports_reference_error():
    m = Model((10, 10), "periodic", [("a", 50, 75, 1.0, 1.0)], [[0, 1], [1, 1]], [20])
    with pytest.raises(ValueError, match="could not place all 20 seed points"):
        m.builder().initial_state()


def test_derived_seeds_match_published_values():
    from cpm import _cpm

    assert [_cpm.derive_seed_u64(42, i) for i in range(5)] == DERIVED_SEEDS_42


def test_model_hash_known_answer():
    import oracle as O

    m = Model((30, 30), "periodic", FROZEN_TYPES, FROZEN_ADHESION, [1, 1], seed=FROZEN_SEED)
    sim = m.oracle(lattice=frozen_lattice(), cell_type_of=[0, 1], local_halo=False)
    sim.run_mcs(FROZEN_MCS)
    b = m.builder(lattice=frozen_lattice(), cell_type_of=[0, 1])
    _, mh = b.hashes(0, 1, 1, sim.lattice(), [0, 1])
    assert mh == FROZEN_MODEL_HASH


def test_convention_hash_is_theta_independent():
    m = c1_model()
    b1 = m.builder()
    lat, cto, _ = b1.initial_state()
    m2 = Model((30, 30), "periodic", [("epithelial", 50, 75, 3.0, 9.0)], [[0, 1], [1, 7]], [5])
    b2 = m2.builder()
    assert b1.hashes(5, 5, 5, lat, cto)[0] == b2.hashes(5, 5, 5, lat, cto)[0]
    assert b1.hashes(5, 5, 5, lat, cto)[0] != b1.hashes(6, 5, 5, lat, cto)[0]


# ---- reference Python tests that need no device (tests/python/test_errors.py)
def test_unsupported_grid_length_raises_value_error():
    import cpm

    with pytest.raises(ValueError, match="length 2 or 3"):
        cpm.CPM(grid=(1, 2, 3, 4), boundary="periodic", seed=1)


def test_unknown_neighborhood_string_raises_value_error():
    import cpm

    with pytest.raises(ValueError, match="unknown neighbourhood"):
        cpm.CPM(grid=(10, 10), boundary="periodic", seed=1, copy_neighborhood="hexagonal")


def test_unknown_boundary_string_raises_value_error():
    import cpm

    with pytest.raises(ValueError, match="unknown boundary"):
        cpm.CPM(grid=(10, 10), boundary="squishy", seed=1)


def test_positive_lambda_act_with_zero_max_act_raises_immediately():
    import cpm

    sim = cpm.CPM(grid=(10, 10), boundary="periodic", seed=1)
    with pytest.raises(ValueError, match="max_act"):
        sim.register_cell_type(name="a", target_volume=20, target_interface=50, lambda_volume=1.0,
                               lambda_interface=1.0, lambda_act=1.0, max_act=0)


def test_unknown_cell_type_in_add_cells_raises_value_error():
    import cpm

    sim = cpm.CPM(grid=(10, 10), boundary="periodic", seed=1)
    with pytest.raises(ValueError, match="unknown cell type"):
        sim.add_cells(cell_type="ghost", n=1)


def test_negative_lambda_message_matches_reference():
    import cpm

    sim = cpm.CPM(grid=(10, 10), boundary="periodic", seed=1)
    with pytest.raises(ValueError, match=r"^lambda_volume must be finite and non-negative, got -1$"):
        sim.register_cell_type("bad", 20, 50, -1.0, 1.0)


def test_non_square_adhesion_matrix_is_rejected_before_any_device_work():
    import cpm

    sim = cpm.CPM(grid=(10, 10), boundary="periodic", seed=1)
    sim.register_cell_type(name="a", target_volume=20, target_interface=50, lambda_volume=1.0, lambda_interface=1.0)
    sim.add_cells(cell_type="a", n=1)
    sim.set_adhesion([[0.0, 1.0], [1.0, 0.0], [0.0, 0.0]])
    with pytest.raises(ValueError, match="adhesion matrix"):
        sim.run(burn_in_mcs=1, readout_mcs=1, sampling_interval_mcs=1)


def test_literal_config2_and_config3_neighbourhoods_are_rejected():
    """Moore / 26-neighbour *copy* is not a subset of the von Neumann
    connectivity stencil (config.rs:305-323): rejected as the reference does."""
    import cpm

    for grid, copy in (((32, 32), "moore"), ((8, 8, 8), "twenty_six")):
        sim = cpm.CPM(grid=grid, boundary="periodic", seed=1, copy_neighborhood=copy)
        sim.register_cell_type("a", 20, 30, 1.0, 1.0)
        sim.add_cells("a", 1)
        sim.set_adhesion([[0, 1], [1, 1]])
        with pytest.raises(ValueError, match="must be a subset of connectivity_neighborhood"):
            sim.run(1, 1, 1)


def test_theta_names_and_extract_theta_match_canonical_layout():
    import cpm

    sim = cpm.CPM(grid=(20, 20), boundary="periodic", seed=1)
    sim.register_cell_type(name="a", target_volume=9, target_interface=20, lambda_volume=1.0, lambda_interface=0.2)
    sim.register_cell_type(name="b", target_volume=9, target_interface=20, lambda_volume=1.5, lambda_interface=0.3)
    sim.add_cells("a", 2)
    sim.add_cells("b", 2)
    sim.set_adhesion([[0.0, 3.0, 3.0], [3.0, 1.0, 5.0], [3.0, 5.0, 1.0]])
    names = sim.theta_names()
    theta = sim.extract_theta()
    assert len(names) == len(theta) == 14
    assert names[:4] == ["lambda_volume[a]", "lambda_volume[b]", "lambda_interface[a]", "lambda_interface[b]"]
    assert theta[:4] == [1.0, 1.5, 0.2, 0.3]
    assert names[4:10] == ["J[medium][medium]", "J[medium][a]", "J[medium][b]", "J[a][a]", "J[a][b]", "J[b][b]"]


def test_wrong_length_theta_raises_a_clean_error():
    import cpm

    sim = cpm.CPM(grid=(20, 20), boundary="periodic", seed=1)
    sim.register_cell_type("a", 9, 20, 1.0, 0.2)
    sim.add_cells("a", 2)
    sim.set_adhesion([[0.0, 3.0], [3.0, 1.0]])
    base = sim.extract_theta()
    with pytest.raises(ValueError, match="theta at index 1 has length"):
        sim.run_batch([base, base[:-1]], burn_in_mcs=5, readout_mcs=5, sampling_interval_mcs=5, master_seed=1)


@pytest.mark.parametrize("bad", [-1.0, float("nan"), float("inf"), 2.0 ** 33])
def test_unrepresentable_max_act_in_theta_is_rejected(bad):
    """theta.rs:93-117, 232-266: a Max_Act entry that does not round into
    [0, u32::MAX] is rejected (not saturated), before any simulation runs."""
    import cpm

    sim = cpm.CPM(grid=(20, 20), boundary="periodic", seed=1)
    sim.register_cell_type("a", 9, 20, 1.0, 0.2)
    sim.add_cells("a", 2)
    sim.set_adhesion([[0.0, 3.0], [3.0, 1.0]])
    theta = list(sim.extract_theta())
    theta[-1] = bad
    with pytest.raises(ValueError, match=r"max_act\[a\] = .* does not round to a value representable as u32"):
        sim.run_batch([sim.extract_theta(), theta], burn_in_mcs=5, readout_mcs=5, sampling_interval_mcs=5,
                      master_seed=1)


@pytest.mark.parametrize("index, value, message", [
    (0, -1.0, "lambda_volume must be finite and non-negative, got -1"),
    (2, float("nan"), r"adhesion\[0\]\[0\] = NaN is not finite"),
])
def test_theta_that_fails_validation_is_a_value_error(index, value, message):
    """batch.rs:126-135: an injected theta goes through the same validation as
    a configuration (CPM::new), before any simulation runs."""
    import cpm

    sim = cpm.CPM(grid=(20, 20), boundary="periodic", seed=1)
    sim.register_cell_type("a", 9, 20, 1.0, 0.2)
    sim.add_cells("a", 2)
    sim.set_adhesion([[0.0, 3.0], [3.0, 1.0]])
    theta = list(sim.extract_theta())
    theta[index] = value
    with pytest.raises(ValueError, match=message):
        sim.run_batch([theta], burn_in_mcs=5, readout_mcs=5, sampling_interval_mcs=5, master_seed=1)


def test_warning_classes_are_user_warnings():
    """tests/python/test_warnings.py:8-22: both warning classes are
    UserWarnings, raisable, catchable and silenced by a filter."""
    import cpm
    from cpm.warnings import CPMInitializationWarning, CPMLowResolutionWarning

    assert cpm.CPMInitializationWarning is CPMInitializationWarning
    for cls in (CPMInitializationWarning, CPMLowResolutionWarning):
        assert issubclass(cls, UserWarning)
        with pytest.warns(cls):
            warnings.warn("x", cls, stacklevel=2)
        with warnings.catch_warnings(record=True) as caught:
            warnings.simplefilter("ignore", cls)
            warnings.warn("x", cls, stacklevel=2)
        assert not caught


def test_cells_for_density_matches_reference_helper():
    import cpm
    from cpm.warnings import CPMLowResolutionWarning

    n = cpm.cells_for_density(grid=(64, 64), target_volume=100, phi=0.8)
    assert n * 100 / 4096 == pytest.approx(0.8, abs=0.02)
    with pytest.warns(CPMLowResolutionWarning):
        cpm.cells_for_density(grid=(64, 64), target_volume=4, phi=0.8)
    with warnings.catch_warnings():
        warnings.simplefilter("error", CPMLowResolutionWarning)
        cpm.cells_for_density(grid=(64, 64), target_volume=1000, phi=0.8)
    # the cell counts of the 512x512 sorting and 128^3 organoid workloads
    assert cpm.cells_for_density((512, 512), 50, 0.2) == 1049
    assert cpm.cells_for_density((128, 128, 128), 1048, 0.8 / 3) == 534


def test_batch_workload_theta_round_trip():
    """The batch benchmark's members carry exactly their theta (theta.rs
    layout): extract_theta() of each built simulation returns it."""
    import bench

    sides, thetas = bench.batch_thetas(12)
    for side, th in zip(sides, thetas):
        sim = bench.batch_sim(side, th, seed=3)
        assert sim.extract_theta() == th
        assert len(th) == len(sim.theta_names()) == 14


def _tile_classes(L, g0, tc, periodic):
    """The tiled sweep's site colours along one axis of a tile (the
    arithmetic of the kernel's site-colour passes, restated): for each
    colour, the local offsets it visits."""
    ncls = 3 if periodic and L % 2 else 2
    out = []
    for want in range(ncls):
        if ncls == 2:
            first = (want - (g0 & 1)) & 1
            cnt = (tc - first + 1) // 2 if tc > first else 0
            out.append([first + 2 * i for i in range(cnt)])
            continue
        w = L - g0
        if want == 2:
            out.append([w - 1] if w - 1 < tc else [])
            continue
        end_a = w - 1 if w - 1 < tc else tc
        first = (want - (g0 & 1)) & 1
        cnt_a = (end_a - first + 1) // 2 if end_a > first else 0
        base_b = w + want
        cnt_b = (tc - base_b + 1) // 2 if tc > base_b else 0
        out.append([first + 2 * i for i in range(cnt_a)] + [base_b + 2 * i for i in range(cnt_b)])
    return out


def test_tiled_site_colours_partition_the_tile_into_non_adjacent_sets():
    """Every site of a tile is visited once per MCS, and no two sites of one
    colour are neighbours, across the periodic wrap included (odd sides: the
    last coordinate takes a third colour)."""
    for L in list(range(3, 40)) + [127, 129]:
        for periodic in (True, False):
            for tc in range(1, L):
                for g0 in range(L if periodic else 1):
                    classes = _tile_classes(L, g0, tc, periodic)
                    seen = sorted(i for c in classes for i in c)
                    assert seen == list(range(tc)), (L, g0, tc, classes)
                    for c in classes:
                        gl = {(g0 + i) % L for i in c}
                        for x in gl:
                            assert (x + 1) % L not in gl or L == 1, (L, g0, tc, c)


def test_samples_are_views_into_their_results_arrays():
    """Sample fields (convert.rs:54-95) read from the arrays a result was
    read into: per-sample rows, the variable-length lists by their offsets,
    the dense upper-triangular contact matrix built from the sparse pairs."""
    import numpy as np

    from cpm._cpm import Sample

    ns, n = 2, 3
    a = {
        "ids": np.array([[1, 2, 3], [1, 2, 3]], np.uint32),
        "volume": np.array([[5, 6, 7], [8, 9, 10]], np.uint32),
        "interface": np.zeros((ns, n), np.uint32), "radius_of_gyration_sq": np.zeros((ns, n)),
        "kappa_sq": np.zeros((ns, n)), "centroid": np.zeros((ns, n, 2)), "eigenvalues": np.zeros((ns, n, 2)),
        "contact_a": np.array([0, 1, 0], np.uint32), "contact_b": np.array([2, 3, 1], np.uint32),
        "contact_count": np.array([4, 5, 6], np.uint32),
    }
    lists = ([0, 2, 3], [0, 1, 1], [0, 0, 2], [3], [7, 1], [True, False], [100, 200], [1.5, 2.5])
    s0, s1 = Sample(a, 0, None, lists), Sample(a, 1, None, lists)
    assert s0.mcs == 100 and s1.conservative_energy == 2.5
    assert list(s1.volume) == [8, 9, 10]
    assert s0.fragmented_cells == [3] and s1.fragmented_cells == []
    assert s0.medium_component_volumes == [] and s1.medium_component_volumes == [7, 1]
    assert s1.medium_component_touches_boundary == [True, False]
    pa, pb, pc = s0.contact_pairs
    assert list(pa) == [0, 1] and list(pb) == [2, 3] and list(pc) == [4, 5]
    m = s0.contact
    assert m.shape == (4, 4) and m[0, 2] == 4 and m[1, 3] == 5 and m.sum() == 9
    assert s1.contact[0, 1] == 6 and s0.lattice is None


def test_c_abi_rejects_null_pointers_with_an_argument_error():
    """Host-only entry points return CPM_E_ARG ("null argument") for null
    buffers whose sizes say they hold data, instead of reading them."""
    from cpm import _cpm

    lib = ctypes.CDLL(_cpm.LIB_PATH)
    lib.cpm_last_error.restype = ctypes.c_char_p
    E_ARG = 7  # CPM_E_ARG
    P = ctypes.c_void_p
    out = P()
    grid = (ctypes.c_uint64 * 2)(10, 10)
    new = lib.cpm_builder_new
    new.argtypes = [P, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_uint64, ctypes.c_char_p, ctypes.c_char_p,
                    ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, P, P, ctypes.c_size_t, P]
    args = [ctypes.cast(grid, P), 2, b"periodic", 1, b"von_neumann", None, b"von_neumann", None, None]
    # active-term keys announced but not passed
    assert new(*args, None, None, 1, ctypes.byref(out)) == E_ARG
    assert lib.cpm_last_error() == b"null argument"
    assert new(*args, None, None, 0, ctypes.byref(out)) == 0
    b = out
    try:
        lib.cpm_builder_set_adhesion.argtypes = [P, P, P, ctypes.c_size_t]
        lens = (ctypes.c_size_t * 2)(2, 2)
        assert lib.cpm_builder_set_adhesion(b, None, ctypes.cast(lens, P), 2) == E_ARG
        assert lib.cpm_builder_set_adhesion(b, None, None, 2) == E_ARG
        lib.cpm_builder_initialize.argtypes = [P, P, ctypes.c_size_t, P, ctypes.c_size_t, ctypes.c_int32,
                                               ctypes.c_int32]
        lat = (ctypes.c_uint32 * 100)()
        assert lib.cpm_builder_initialize(b, ctypes.cast(lat, P), 100, None, 1, 1, 0) == E_ARG
        lib.cpm_builder_register_cell_type.argtypes = [P, ctypes.c_char_p, ctypes.c_uint32, ctypes.c_uint32,
                                                       ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                                       ctypes.c_uint32]
        assert lib.cpm_builder_register_cell_type(b, b"a", 20, 20, 1.0, 1.0, 0.0, 0) == 0
        adh = (ctypes.c_double * 4)(0, 1, 1, 0)
        assert lib.cpm_builder_set_adhesion(b, ctypes.cast(adh, P), ctypes.cast(lens, P), 2) == 0
        lib.cpm_builder_run_batch.argtypes = [P, P, P, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_uint64,
                                              ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32, P, P]
        tl = (ctypes.c_size_t * 1)(5)
        res = (P * 1)()
        assert lib.cpm_builder_run_batch(b, None, ctypes.cast(tl, P), 1, 1, 1, 1, 0, 0, None,
                                         ctypes.cast(res, P)) == E_ARG
    finally:
        lib.cpm_builder_free.argtypes = [P]
        lib.cpm_builder_free(b)


def test_c99_client_compiles_links_and_runs(tmp_path):
    """include/cpm_gpu.h is a C99 header and the library serves a plain C
    caller: builder calls, the reference's duplicate-type error text, theta
    length and the published derived seed for (42, 0)."""
    import shutil
    import subprocess

    from cpm import _cpm

    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    root = _cpm.__file__.replace("cpm-rust_gb300/python/cpm/_cpm.py", "")
    libdir = root + "cpm-rust_gb300/lib"
    exe = str(tmp_path / "c_abi_client")
    subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-I", root + "include", root + "tests/c_abi_client.c",
                    "-L", libdir, "-lcpm_gpu", "-Wl,-rpath," + libdir, "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    assert 'cell type "a" has already been added' in out
    assert "seed=6806512004122731638" in out
