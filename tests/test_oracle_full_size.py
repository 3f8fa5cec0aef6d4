"""The bond families of the benchmark workloads at their full sizes, on the
CPU: the oracle's cell-list search gives the bond counts the engine reports
on the GPU (tests/test_gpu_full_size.py asserts the same counts there), every
row fits the reference's row cap MN, and sampled rows equal a brute-force
search over all nodes with the reference's test |x_j - x_i|^2 < delta^2,
j != i (Neighbor.cu:42-80), in ascending order."""
import numpy as np
import pytest

import oracle as orc
from pd_gpu1_gb300 import presets
from pd_gpu1_gb300._abi import PD_MODEL_BOND


def _family(p, coords):
    m = orc.Model(p, *coords)
    widest = m.find_neighbor(brute=False)
    return m, widest


def _brute_rows(p, coords, m, rows):
    rp = m.rowptr()
    NL = m.rows(m.NL)
    pts = np.stack([np.asarray(c, dtype=np.float64) for c in coords], axis=1)
    d2max = p.delta * p.delta
    for i in rows:
        diff = pts - pts[i]
        d2 = diff[:, 0] * diff[:, 0] + diff[:, 1] * diff[:, 1]
        if pts.shape[1] == 3:
            d2 = d2 + diff[:, 2] * diff[:, 2]
        want = np.nonzero(d2 < d2max)[0]
        want = want[want != i]
        np.testing.assert_array_equal(NL[rp[i]:rp[i + 1]], want, err_msg=f"row {i}")


@pytest.mark.parametrize("name", ["crack_branching", "kalthoff_winkler_bond", "warm_start"])
def test_full_size_family(name):
    if name == "crack_branching":
        p, _, _ = presets.build_crack_branching(derive=orc.derive_params)
        coords = orc.plate_coords(p)
        n, bonds, interior_bonds = 1_600_000, 44_699_236, 44_699_236
    elif name == "kalthoff_winkler_bond":
        p, _, meta = presets.build_kalthoff_winkler(model=PD_MODEL_BOND, derive=orc.derive_params,
                                                    coord_fn=orc.coord_kw)
        coords = meta["coords"]
        n, bonds, interior_bonds = 180_873, 18_809_054, 18_809_054
    else:
        p, _, _ = presets.build_warm_start_plate(derive=orc.derive_params)
        coords = orc.plate_crack_coords(p)
        n, bonds, interior_bonds = 1_006_000, 28_095_820, 27_964_000
    assert p.N == n
    m, widest = _family(p, coords)
    assert widest <= p.MN
    assert int(m.NN.sum()) == bonds
    assert int(m.NN[: p.N_int].sum()) == interior_bonds
    rng = np.random.default_rng(3)
    sample = np.concatenate([[0, p.N - 1, p.N_int - 1], rng.integers(0, p.N, 60)])
    _brute_rows(p, coords, m, sample)
