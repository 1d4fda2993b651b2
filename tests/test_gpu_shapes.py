"""Distributional parity on the headline workloads' shapes, on lattices the
tiled sweep cuts into tiles (and, for comparison, on the resident sweep):

* sorting: the 512x512 differential-adhesion case's model on 128x128
  periodic (4 types, V*=50, I*=30, lambda 5/1, Moore energy, phi=0.8,
  medium J 16, type-type J uniform in [2, 14]), scatter-and-grow placement;
* organoid: the 128^3 case's model on 40^3 periodic (3 types, V*=1048,
  I*=600, lambda 2/0.5, 26-neighbour energy, phi=0.8, medium J 16,
  type-type J uniform in [1, 12]), nested-layer placement.

Per seed (128 seeds; the oracle side is tests/golden/shapes_oracle_summary.npz
from tests/golden/make_ks_fixture.py --shapes) the energy, the mean and
spread of the cell volumes and the mean interface are read at several MCS
along each trajectory and compared by two-sample KS tests, p > 0.01:
sorting at 300 MCS (coarsening under way) and 3000 MCS; organoid at
200 MCS (the cells have grown to their frozen size). The organoid's first
25 MCS (the growth burst) are reported, not asserted: there the colour-pass
chain is measurably ahead of the reference's random-sequential chain.
The test prints the relaxation curve (oracle mean energy, GPU minus oracle
with its standard error) at every checkpoint both sides share.
"""

import os

import numpy as np
import pytest

from helpers import Model

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
STATS = ("energy", "mean_volume", "volume_std", "mean_interface")


def _fixture():
    return np.load(os.path.join(HERE, "golden", "shapes_oracle_summary.npz"))


def _sorting_model(seed):
    import make_ks_fixture as F

    spec = F.sorting_shape_spec()
    return Model((128, 128), "periodic", [(f"t{i}", 50, 30, 5.0, 1.0) for i in range(4)], spec.adhesion.tolist(),
                 [66] * 4, seed=seed)


def _organoid_model(seed):
    import make_ks_fixture as F

    return Model((40, 40, 40), "periodic", [(f"t{i}", 1048, 600, 2.0, 0.5) for i in range(3)],
                 F.organoid_shape_adhesion().tolist(), [16] * 3, energy="twenty_six", seed=seed)


def _gpu_run(builders, checkpoints):
    from cpm import _cpm

    eng = _cpm.Engine(builders)
    n = len(builders)
    out = {k: np.zeros((n, len(checkpoints))) for k in STATS}
    done = 0
    for c, m in enumerate(checkpoints):
        eng.run_mcs(int(m) - done)
        done = int(m)
        eng.synchronize()
        for i in range(n):
            v, it, _, _ = eng.cells(i)
            v = v[1:].astype(np.float64)
            it = it[1:].astype(np.float64)
            out["energy"][i, c] = eng.energy(i)
            out["mean_volume"][i, c] = v.mean()
            out["volume_std"][i, c] = v.std()
            out["mean_interface"][i, c] = it.mean()
    st = eng.stats(0)
    for i in range(n):
        assert eng.recount_check(i)[0]
    return out, st


def _compare(name, ref, prefix, gpu, checkpoints, asserted):
    from scipy.stats import ks_2samp

    all_ck = list(ref[f"{prefix}_ckpt"])
    print(f"\n{name}: MCS | oracle mean energy | GPU - oracle (SE) | KS p: " + ", ".join(STATS))
    failures = []
    for c, m in enumerate(checkpoints):
        j = all_ck.index(m)
        eo = ref[f"{prefix}_energy"][:, j]
        eg = gpu["energy"][:, c]
        se = np.sqrt(eo.var(ddof=1) / eo.size + eg.var(ddof=1) / eg.size)
        p = {k: ks_2samp(np.asarray(ref[f"{prefix}_{k}"][:, j]), gpu[k][:, c]).pvalue for k in STATS}
        print(f"  {m:6d} | {eo.mean():14.1f} | {eg.mean() - eo.mean():+10.1f} ({se:.1f}) | " +
              ", ".join(f"{p[k]:.3f}" for k in STATS))
        if m in asserted:
            failures += [(m, k, p[k]) for k in STATS if p[k] <= 0.01]
    assert not failures, failures


@pytest.mark.parametrize("path", ["tiled", "resident"])
def test_sorting_shape_matches_oracle(path, cuda_required, monkeypatch):
    if path == "tiled":
        monkeypatch.setenv("CPM_GPU_FORCE_TILED", "1")
    ref = _fixture()
    checkpoints = (100, 300, 1000, 3000)
    builders = [_sorting_model(int(s)).builder(warn=False) for s in ref["seeds"]]
    gpu, st = _gpu_run(builders, checkpoints)
    if path == "tiled":
        assert st["passes"] > 0 and st["spin_timeouts"] == 0
        assert st["deferred"] <= 0.001 * st["nonnull"]
    _compare(f"sorting 128x128 ({path})", ref, "sorting", gpu, checkpoints, asserted=(300, 3000))


@pytest.mark.parametrize("path", ["tiled", "resident"])
def test_organoid_shape_matches_oracle(path, cuda_required, monkeypatch):
    import make_ks_fixture as F

    if path == "tiled":
        monkeypatch.setenv("CPM_GPU_FORCE_TILED", "1")
    ref = _fixture()
    checkpoints = (25, 50, 100, 200)
    lat, types = F.organoid_shape_placement()
    builders = [_organoid_model(int(s)).builder(lattice=lat, cell_type_of=types.tolist(), warn=False)
                for s in ref["seeds"]]
    gpu, st = _gpu_run(builders, checkpoints)
    if path == "tiled":
        assert st["passes"] > 0 and st["spin_timeouts"] == 0
        assert st["deferred"] <= 0.001 * st["nonnull"]
    _compare(f"organoid 40^3 ({path})", ref, "organoid", gpu, checkpoints, asserted=(200,))
