"""Learned ADR warm start: load increments solved to a 1e-6 relative
residual from the plain start (previous solution) and from the learned
start (trained network shipped in pd_gpu1_gb300/data), on a 0.02 m version
of the warm-start plate (41,200 nodes, geometrically similar to the 1M-node
one; the network was trained on 100k-250k-node plates of the same set-up).

Bars: the learned start needs at most a third of the plain start's ADR
iterations over the increments after the first (the first has no history);
every start it uses has a residual no larger than the plain start's; the
converged displacements agree with the plain run's to 1e-2 relative (both
stop at the same absolute residual); a network whose predictions are far
off is never used (the plain start is kept)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def W():
    from pd_gpu1_gb300 import engine, warm

    engine.lib()
    return warm


def _run(W, mode, n, net=None):
    from pd_gpu1_gb300 import presets
    from pd_gpu1_gb300.engine import Engine

    p, setup, meta = presets.build_warm_start_plate(scale=0.2)
    with Engine(p) as eng:
        setup(eng)
        st = W.run_increments(eng, meta, n, mode=mode, net=net)
        return st, eng.get("UY")[: p.N_int].copy()


def test_learned_start_gains(W):
    net = W.Net.load()
    n = 8
    plain, up = _run(W, "plain", n)
    learned, ul = _run(W, "learned", n, net)
    it_p = sum(s["iters"] for s in plain[1:])
    it_l = sum(s["iters"] for s in learned[1:])
    assert it_l * 3 <= it_p, (it_l, it_p)
    for s in learned:
        assert s["r_start"] <= s["r_plain"]
        assert s["r_final"] <= 1e-6 * s["r_plain"]
    assert all(s["warm_used"] > 0 for s in learned[1:])
    assert np.linalg.norm(ul - up) <= 1e-2 * np.linalg.norm(up)


def test_bad_prediction_falls_back_to_plain(W):
    rng = np.random.default_rng(0)
    p = W.init_params(1)
    p[-258:] = rng.standard_normal(258).astype(np.float32) * 50.0  # output layer: large, wrong corrections
    bad = W.Net(65536, p)
    st, _ = _run(W, "network", 3, bad)
    for s in st[1:]:
        assert s["warm_used"] == 0 and s["r_start"] == s["r_plain"]


def test_smoothing_lowers_the_network_start_residual(W):
    """pd_warm_predict's family averaging of the network's correction removes
    the node-to-node rounding noise that the residual amplifies: the
    network's starting residual falls several-fold; the skip-term candidate
    is unchanged."""
    from pd_gpu1_gb300 import presets
    from pd_gpu1_gb300.engine import Engine

    net = W.Net.load()
    p, setup, meta = presets.build_warm_start_plate(scale=0.2)
    ratios = {}
    for sm in (0, 64):
        with Engine(p) as eng:
            setup(eng)
            st = W.run_increments(eng, meta, 4, mode="network", net=net, smooth=sm)
            assert all(s["warm_used"] == 1 for s in st[1:])  # admissible: used
            ratios[sm] = [s["r_start"] / s["r_plain"] for s in st[1:]]
    for a, b in zip(ratios[0], ratios[64]):
        assert b < 0.2 * a, (ratios[0], ratios[64])
    import torch

    L = W.lib()
    with Engine(p) as eng:
        setup(eng)
        W.run_increments(eng, meta, 2, mode="plain")
        eng.damage()
        ni = p.N_int
        U, nnref = 2 * meta["delta"], W.nn_reference(eng)
        outs = []
        for sm in (0, 16):
            du = torch.zeros(4 * ni, dtype=torch.float64, device="cuda")
            W.check(L.pd_warm_predict(eng.ctx, net.h, U, meta["delta"], nnref, sm, du.data_ptr(), eng.stream),
                    eng.ctx, "pd_warm_predict")
            outs.append(du.cpu().numpy())
        np.testing.assert_array_equal(outs[0][2 * ni:], outs[1][2 * ni:])  # the skip term
        assert not np.array_equal(outs[0][: 2 * ni], outs[1][: 2 * ni])
