"""Learned ADR warm start: load increments solved to a 1e-6 relative
residual from the plain start (previous solution), from the skip term alone
(the proportional, secant, increment) and from the learned start (the trained
network shipped in pd_gpu1_gb300/data offered beside the skip term), on
0.02 m versions of the warm-start plate (41,200 nodes) with a pre-crack of a
length the network was not trained on (22 % of the width; training used 15,
18, 20 and 25 %).

Bars:
  * the learned start needs at most a third of the plain start's ADR
    iterations over the increments after the first, every start it uses has
    a residual no larger than the plain start's, and the converged
    displacements agree with the plain run's to 1e-2 (all stop at the same
    residual);
  * over 40 increments that take the crack through its first advances, the
    learned start needs at most 0.8 of the skip term's iterations, and the
    network's start is the one used on most increments;
  * a network whose predictions are far off is never used (plain start).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FRAC = 0.22  # pre-crack length over the plate width, not among the training runs


@pytest.fixture(scope="module")
def W():
    from pd_gpu1_gb300 import engine, warm

    engine.lib()
    return warm


def _run(W, mode, n, net=None, smooth=None):
    from pd_gpu1_gb300 import presets
    from pd_gpu1_gb300.engine import Engine

    p, setup, meta = presets.build_warm_start_plate(scale=0.2, crack_frac=FRAC)
    with Engine(p) as eng:
        setup(eng)
        kw = {} if smooth is None else {"smooth": smooth}
        st = W.run_increments(eng, meta, n, mode=mode, net=net, **kw)
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


def test_network_beats_the_skip_term_through_crack_advances(W):
    net = W.Net.load()
    n = 40
    skip, _ = _run(W, "secant", n, net)
    learned, _ = _run(W, "learned", n, net)
    assert sum(s["advanced"] > 0 for s in learned) >= 2  # the crack advanced within the window
    it_s = sum(s["iters"] for s in skip[1:])
    it_l = sum(s["iters"] for s in learned[1:])
    assert it_l <= 0.8 * it_s, (it_l, it_s)
    used = [s["start"] for s in learned[1:]]
    assert used.count("network") > len(used) / 2, used


def test_bad_prediction_falls_back_to_plain(W):
    rng = np.random.default_rng(0)
    p = W.init_params(1)
    # output layer: large, wrong corrections (outputs ~1e7, i.e. ~100 U per
    # node after the 2^-16 history scale, against an increment of U / k)
    p[-258:] = rng.standard_normal(258).astype(np.float32) * 1e6
    bad = W.Net(65536, p)
    st, _ = _run(W, "network", 3, bad, smooth=0)
    for s in st[1:]:
        assert s["warm_used"] == 0 and s["r_start"] == s["r_plain"]


def test_smoothing_keeps_the_skip_candidate_and_changes_the_network_one(W):
    """pd_warm_predict's family averaging acts on the network's correction
    only: with and without it the skip-term candidate is bit for bit the same,
    the network candidate differs, and both network candidates stay within a
    small fraction of the increment of each other."""
    import torch

    from pd_gpu1_gb300 import presets
    from pd_gpu1_gb300.engine import Engine

    net = W.Net.load()
    L = W.lib()
    p, setup, meta = presets.build_warm_start_plate(scale=0.2, crack_frac=FRAC)
    with Engine(p) as eng:
        setup(eng)
        W.run_increments(eng, meta, 3, mode="plain")  # two increments of history
        eng.damage()
        ni = p.N_int
        U = 3 * meta["delta"]
        outs = []
        for sm in (0, 16):
            du = torch.zeros(4 * ni, dtype=torch.float64, device="cuda")
            W.check(L.pd_warm_predict(eng.ctx, net.h, U, meta["delta"], sm, du.data_ptr(), eng.stream), eng.ctx,
                    "pd_warm_predict")
            outs.append(du.cpu().numpy())
        np.testing.assert_array_equal(outs[0][2 * ni:], outs[1][2 * ni:])  # the skip term
        assert not np.array_equal(outs[0][: 2 * ni], outs[1][: 2 * ni])
        assert np.linalg.norm(outs[0][: 2 * ni] - outs[1][: 2 * ni]) <= 0.05 * np.linalg.norm(outs[0][: 2 * ni])
