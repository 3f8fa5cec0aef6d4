"""Snapshots (checkpoint / resume), the text writers fed from a context and
the crack-tip position.

Bars: a run resumed from a snapshot repeats the saved run bit for bit; the
crack tip of the engine and of the oracle agree within one horizon after
crack growth (and with a direct scan of the damage field exactly)."""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

STATE = ["UX", "UY", "UZ", "VX", "VY", "VZ", "AX", "AY", "AZ", "FAIL", "DMG"]


@pytest.fixture(scope="module")
def E():
    from pd_gpu1_gb300 import engine

    engine.lib()
    return engine


def _resume_matches(E, build, run, tmp_path, name):
    p, setup, meta = build()
    a, b = E.Engine(p), E.Engine(p)
    setup(a)
    setup(b)
    run(a, 0)
    path = tmp_path / f"{name}.snap"
    a.snapshot_save(path)
    run(a, 1)
    b.snapshot_load(path)
    run(b, 1)
    for f in STATE:
        np.testing.assert_array_equal(a.get(f), b.get(f), err_msg=f"{name} {f}")
    if p.dim == 3 and meta.get("cylinder") is not None:
        ca, cb = a.cylinder(), b.cylinder()
        assert list(ca.disp) == list(cb.disp) and list(ca.vel) == list(cb.vel)
    a.close()
    b.close()


def test_snapshot_resume_explicit_with_breakage(E, tmp_path):
    from pd_gpu1_gb300 import presets

    def run(eng, k):
        eng.run_explicit(60, dmg_every=30)

    _resume_matches(E, lambda: presets.build_crack_branching(scale=0.05, nt=120), run, tmp_path, "branch")


def test_snapshot_resume_adr(E, tmp_path):
    from pd_gpu1_gb300 import presets

    def run(eng, k):
        eng.run_adr(40 * k, 40, load=2.7e-8)

    _resume_matches(E, lambda: presets.build_plate_tensile(scale=0.3), run, tmp_path, "adr")


def test_snapshot_resume_kw_contact(E, tmp_path):
    from pd_gpu1_gb300 import presets

    def run(eng, k):
        eng.run_explicit(15)

    _resume_matches(E, lambda: presets.build_kalthoff_winkler(scale=0.3, nt=30), run, tmp_path, "kw")


def test_snapshot_rejects_other_problem(E, tmp_path):
    from pd_gpu1_gb300 import presets
    from pd_gpu1_gb300.engine import PDError

    p, setup, _ = presets.build_plate_tensile(scale=0.3)
    q, setup_q, _ = presets.build_plate_tensile(scale=0.2)
    a, b = E.Engine(p), E.Engine(q)
    setup(a)
    setup_q(b)
    a.snapshot_save(tmp_path / "a.snap")
    with pytest.raises(PDError):
        b.snapshot_load(tmp_path / "a.snap")
    a.close()
    b.close()


def test_crack_tip_and_writers(E, tmp_path):
    """Crack branching (small plate, 150 steps): the tip of the engine's damage
    field against the oracle's, and the context writers' files."""
    from pd_gpu1_gb300 import presets

    p, setup, meta = presets.build_crack_branching(scale=0.05, nt=150)
    eng = E.Engine(p)
    setup(eng)
    x, y = eng.get("X"), eng.get("Y")
    m = orc.Model(p, x, y)
    m.find_neighbor()
    m.surface_correct()
    m.set_crack_2d(p.length / 2.0, -p.length / 4.0, 0.0, 0.0)
    m.by[:] = eng.get("BY")
    eng.run_explicit(meta["nt"])
    for _ in range(meta["nt"]):
        m.explicit_step()
    m.damage()
    eng.damage()
    dmg = eng.get("DMG")[: p.N_int]
    tx, ty = eng.crack_tip(0.38)
    # direct scan of the damage field
    hot = np.nonzero(dmg > 0.38)[0]
    assert len(hot) > 0
    k = hot[np.argmax(x[hot])]
    assert (tx, ty) == (x[k], y[k])
    # against the oracle's damage field: within one horizon
    dm = m.dmg[: p.N_int]
    ho = np.nonzero(dm > 0.38)[0]
    ko = ho[np.argmax(x[ho])]
    assert abs(x[ko] - tx) <= p.delta and abs(y[ko] - ty) <= p.delta
    # writers
    f = tmp_path / "disp.txt"
    eng.save_disp(f)
    lines = f.read_text().splitlines()
    assert len(lines) == p.N_int
    ux, uy = eng.get("UX"), eng.get("UY")
    assert lines[7] == "%g %g %g" % (ux[7], uy[7], dmg[7])
    eng.close()
