"""Generates the oracle side of the distributional (KS) parity test.

Runs the CPU oracle (restated cpm-core run path, pinned by the reference's
frozen trajectory) for seeds 1..N of the quickstart configuration
(README.md:47-83 / tests/python/test_builder.py:11-28: 30x30 periodic, one
type V*=50 I*=75 lambda_V=10 lambda_I=2, 5 cells, J=[[0,5],[5,2]], default
placement, 5000 burn-in + 5000 readout MCS) and stores the last sample's
per-cell volume, interface, squared radius of gyration and kappa^2 plus the
final energy; and (`fluct_oracle_summary.npz`) the per-seed summaries of a
second configuration sized for the tiled sweep — 84x84 periodic, one type
V*=40 I*=30 lambda_V=3 lambda_I=0.6, 80 cells, J=[[0,6.5],[6.5,2.2]],
2000 burn-in + 1000 readout MCS, seeds 1..160 — whose state is stationary
well before the sample; and (`modes_oracle_summary.npz`, `--modes`) the
same summaries for the loop's other modes on a 40x40 periodic lattice with
one type (V*=40, I*=30, lambda_V=3, lambda_I=0.6, 20 cells,
J=[[0,6.5],[6.5,2.2]], 1000 burn-in + 500 readout MCS, seeds 1..160): with
Metropolis-Hastings acceptance (monte_carlo.rs:168-196) and with the Act
term (energy.rs:329-471; lambda_act = 20, max_act = 20).
And (`odd_oracle_summary.npz`, `--odd`) a lattice with odd periodic sides,
31x29, one type (V*=50, I*=75, lambda_V=10, lambda_I=2, 5 cells) whose cells
repel (J=[[0,3],[3,12]]), so the state is stationary by the sample with no
slow aggregation (2000 burn-in + 2000 readout MCS, seeds 1..96).
And (`shapes_oracle_summary.npz`, `--shapes`) the headline shapes on
lattices the tiled sweep cuts, read at several MCS along each trajectory
(per seed: energy, mean and spread of the volumes, mean interface):
  * sorting (the 512x512 differential-adhesion case's shape on 128x128
    periodic): 4 types V*=50 I*=30 lambda_V=5 lambda_I=1, 66 cells per type
    (phi=0.8), Moore energy, medium row of J 16 and type-type J uniform in
    [2, 14] from default_rng(1), scatter-and-grow placement; seeds 1..128,
    read at 100, 300, 1000, 3000 and 10000 MCS;
  * organoid (the 128^3 case's shape on 40^3 periodic): 3 types V*=1048
    I*=600 lambda_V=2 lambda_I=0.5, 16 cells per type (phi=0.8), 26-neighbour
    energy, medium row 16 and type-type J uniform in [1, 12] from
    default_rng(1), nested-layer placement (one 2x2x2 seed per cell, types
    from the centre out); seeds 1..128, read at 25, 50, 100, 200 and 500 MCS.
And (`modes_tiled_oracle_summary.npz`, `--modes-tiled`) the loop's other
modes on a lattice the tiled sweep cuts into 6x6 tiles: 96x96 periodic, one
type (V*=40, I*=30, lambda_V=3, lambda_I=0.6, 115 cells, phi=0.5),
J=[[0,6.5],[6.5,2.2]], 2000 burn-in + 1000 readout MCS, seeds 1..128, with
Metropolis-Hastings acceptance and with the Act term (lambda_act = 20,
max_act = 20).
Usage: python tests/golden/make_ks_fixture.py [--fluct | --modes | --modes-tiled | --odd | --shapes]
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402

N_SEEDS = 256
BURN_IN, READOUT = 5000, 5000


def c1_spec():
    return O.ModelSpec((30, 30), True, [(50, 75, 10.0, 2.0)], [[0, 5], [5, 2]], cell_counts=[5])


FLUCT_SEEDS = 160
FLUCT_BURN_IN, FLUCT_READOUT = 2000, 1000


def fluct_spec():
    return O.ModelSpec((84, 84), True, [(40, 30, 3.0, 0.6)], [[0, 6.5], [6.5, 2.2]], cell_counts=[80])


def fluct_main():
    seeds = np.arange(1, FLUCT_SEEDS + 1, dtype=np.uint64)
    failed, cells, energy, n = O.run_many(fluct_spec(), seeds, FLUCT_BURN_IN, FLUCT_READOUT, threads=0,
                                          local_halo=True)
    assert failed == 0 and np.all(n == 80)
    v = cells["volume"].astype(np.float64)
    i = cells["interface"].astype(np.float64)
    np.savez_compressed(
        os.path.join(HERE, "fluct_oracle_summary.npz"),
        seeds=seeds,
        energy=energy,
        mean_volume=v.mean(1),
        volume_std=v.std(1),
        mean_interface=i.mean(1),
    )
    print("wrote", os.path.join(HERE, "fluct_oracle_summary.npz"))


MODES_SEEDS = 160
MODES_BURN_IN, MODES_READOUT = 1000, 500
MODES = {"mh": dict(acceptance="metropolis_hastings"), "act": dict(act=[(20.0, 20)])}


def modes_spec(mode):
    return O.ModelSpec((40, 40), True, [(40, 30, 3.0, 0.6)], [[0, 6.5], [6.5, 2.2]], cell_counts=[20], **MODES[mode])


def modes_main():
    seeds = np.arange(1, MODES_SEEDS + 1, dtype=np.uint64)
    out = {"seeds": seeds}
    for mode in MODES:
        failed, cells, energy, n = O.run_many(modes_spec(mode), seeds, MODES_BURN_IN, MODES_READOUT, threads=0,
                                              local_halo=True)
        assert failed == 0 and np.all(n == 20)
        v = cells["volume"].astype(np.float64)
        i = cells["interface"].astype(np.float64)
        out[f"{mode}_energy"] = energy
        out[f"{mode}_mean_volume"] = v.mean(1)
        out[f"{mode}_volume_std"] = v.std(1)
        out[f"{mode}_mean_interface"] = i.mean(1)
    np.savez_compressed(os.path.join(HERE, "modes_oracle_summary.npz"), **out)
    print("wrote", os.path.join(HERE, "modes_oracle_summary.npz"))


MODES_TILED_SEEDS = 128
MODES_TILED_BURN_IN, MODES_TILED_READOUT = 2000, 1000


def modes_tiled_spec(mode):
    return O.ModelSpec((96, 96), True, [(40, 30, 3.0, 0.6)], [[0, 6.5], [6.5, 2.2]], cell_counts=[115], **MODES[mode])


def modes_tiled_main():
    seeds = np.arange(1, MODES_TILED_SEEDS + 1, dtype=np.uint64)
    out = {"seeds": seeds}
    for mode in MODES:
        failed, cells, energy, n = O.run_many(modes_tiled_spec(mode), seeds, MODES_TILED_BURN_IN, MODES_TILED_READOUT,
                                              threads=0, local_halo=True)
        assert failed == 0 and np.all(n == 115)
        v = cells["volume"].astype(np.float64)
        i = cells["interface"].astype(np.float64)
        out[f"{mode}_energy"] = energy
        out[f"{mode}_mean_volume"] = v.mean(1)
        out[f"{mode}_volume_std"] = v.std(1)
        out[f"{mode}_mean_interface"] = i.mean(1)
    np.savez_compressed(os.path.join(HERE, "modes_tiled_oracle_summary.npz"), **out)
    print("wrote", os.path.join(HERE, "modes_tiled_oracle_summary.npz"))


ODD_SEEDS = 96
ODD_BURN_IN, ODD_READOUT = 2000, 2000


def odd_spec():
    return O.ModelSpec((31, 29), True, [(50, 75, 10.0, 2.0)], [[0, 3], [3, 12]], cell_counts=[5])


def odd_main():
    seeds = np.arange(1, ODD_SEEDS + 1, dtype=np.uint64)
    failed, cells, energy, n = O.run_many(odd_spec(), seeds, ODD_BURN_IN, ODD_READOUT, threads=0, local_halo=True)
    assert failed == 0 and np.all(n == 5)
    v = cells["volume"].astype(np.float64)
    i = cells["interface"].astype(np.float64)
    np.savez_compressed(os.path.join(HERE, "odd_oracle_summary.npz"), seeds=seeds, energy=energy,
                        mean_volume=v.mean(1), volume_std=v.std(1), mean_interface=i.mean(1))
    print("wrote", os.path.join(HERE, "odd_oracle_summary.npz"))


SHAPE_SEEDS = 128
SORTING_CKPT = (100, 300, 1000, 3000, 10000)
ORGANOID_CKPT = (25, 50, 100, 200, 500)


def sorting_shape_spec():
    rng = np.random.default_rng(1)
    J = np.zeros((5, 5))
    J[0, 1:] = J[1:, 0] = 16.0
    tt = rng.uniform(2, 14, size=(4, 4))
    J[1:, 1:] = np.triu(tt) + np.triu(tt, 1).T
    return O.ModelSpec((128, 128), True, [(50, 30, 5.0, 1.0)] * 4, J, cell_counts=[66] * 4)


def organoid_shape_adhesion():
    rng = np.random.default_rng(1)
    J = np.zeros((4, 4))
    J[0, 1:] = J[1:, 0] = 16.0
    tt = rng.uniform(1, 12, size=(3, 3))
    J[1:, 1:] = np.triu(tt) + np.triu(tt, 1).T
    return J


def organoid_shape_placement(side=40, per_type=(16, 16, 16)):
    """One 2x2x2 seed per cell on a cubic grid, the seeds nearest the centre
    first, types in order from the centre outwards."""
    k = int(sum(per_type))
    g = max(2, int((side ** 3 / max(k, 1)) ** (1.0 / 3.0)))
    while True:
        ax = np.arange(g // 2, side - 1, g)
        pts = np.stack(np.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
        if len(pts) >= k or g == 2:
            break
        g -= 1
    c = (side - 1) / 2.0
    order = np.lexsort((np.arange(len(pts)), ((pts - c) ** 2).sum(1)))
    pts = pts[order[:k]]
    lat = np.zeros((side, side, side), dtype=np.uint32)
    for i, (x, y, z) in enumerate(pts):
        lat[x:x + 2, y:y + 2, z:z + 2] = i + 1
    return lat.ravel(), np.repeat(np.arange(len(per_type)), per_type)


def organoid_shape_spec():
    return O.ModelSpec((40, 40, 40), True, [(1048, 600, 2.0, 0.5)] * 3, organoid_shape_adhesion(),
                       cell_counts=[16] * 3, energy="twenty_six")


def _summaries(vol, itf, energy):
    v = vol.astype(np.float64)
    i = itf.astype(np.float64)
    return {"energy": energy, "mean_volume": v.mean(2), "volume_std": v.std(2), "mean_interface": i.mean(2)}


def shapes_main():
    seeds = np.arange(1, SHAPE_SEEDS + 1, dtype=np.uint64)
    out = {"seeds": seeds, "sorting_ckpt": np.array(SORTING_CKPT), "organoid_ckpt": np.array(ORGANOID_CKPT)}
    failed, vol, itf, energy, n = O.run_many_checkpoints(sorting_shape_spec(), seeds, SORTING_CKPT)
    assert failed == 0 and np.all(n == 264)
    out.update({f"sorting_{k}": v for k, v in _summaries(vol, itf, energy).items()})
    failed, vol, itf, energy, n = O.run_many_checkpoints(organoid_shape_spec(), seeds, ORGANOID_CKPT,
                                                         explicit=organoid_shape_placement())
    assert failed == 0 and np.all(n == 48)
    out.update({f"organoid_{k}": v for k, v in _summaries(vol, itf, energy).items()})
    np.savez_compressed(os.path.join(HERE, "shapes_oracle_summary.npz"), **out)
    print("wrote", os.path.join(HERE, "shapes_oracle_summary.npz"))


def main():
    seeds = np.arange(1, N_SEEDS + 1, dtype=np.uint64)
    failed, cells, energy, n = O.run_many(c1_spec(), seeds, BURN_IN, READOUT, threads=0, local_halo=True)
    assert failed == 0 and np.all(n == 5)
    np.savez_compressed(
        os.path.join(HERE, "c1_oracle_summary.npz"),
        seeds=seeds,
        volume=cells["volume"].astype(np.uint32),
        interface=cells["interface"].astype(np.uint32),
        rg2=cells["rg2"],
        kappa2=cells["kappa2"],
        energy=energy,
    )
    print("wrote", os.path.join(HERE, "c1_oracle_summary.npz"))


if __name__ == "__main__":
    if "--fluct" in sys.argv:
        fluct_main()
    elif "--modes-tiled" in sys.argv:
        modes_tiled_main()
    elif "--modes" in sys.argv:
        modes_main()
    elif "--odd" in sys.argv:
        odd_main()
    elif "--shapes" in sys.argv:
        shapes_main()
    else:
        main()
        fluct_main()
        modes_main()
        modes_tiled_main()
        odd_main()
        shapes_main()
