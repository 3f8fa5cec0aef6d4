"""Batches of specimens (pd_batch_create / pd_batch_run_adr) against the same
plates set up and run alone, and the launch-shape controls.

Bars:
  - family, bond coefficients, surface-correction factors, pre-crack flags,
    forces at a given displacement and the first ADR step: bit-identical to
    the standalone plate (every specimen keeps its own coordinate frame);
  - ADR over 40 steps: 1e-9 norm-relative (the per-specimen damping sum is
    added in a different order than the single-plate grid reduction, and the
    ADR damping rule amplifies last-bit differences);
  - any launch shape of the bond kernel: bit-identical batch results.
"""
import math

import numpy as np
import pytest

import oracle as orc
from helpers import assert_close_norm

pytestmark = pytest.mark.gpu

SPECS = [
    dict(nx=17, ny=23, emod=72.0e9, critical_s=2.0e-3, crack_len=4.0e-3, crack_theta=0.3, load_scale=1.0),
    dict(nx=32, ny=32, emod=192.0e9, critical_s=1.0e-4, crack_len=0.0, crack_theta=0.0, load_scale=2.0),
    dict(nx=40, ny=12, emod=150.0e9, critical_s=5.0e-3, crack_len=6.0e-3, crack_theta=math.pi / 2, load_scale=0.5),
    dict(nx=25, ny=25, emod=90.0e9, critical_s=3.0e-3, crack_len=3.0e-3, crack_theta=0.0, load_scale=1.0),
]
NODE_FIELDS = ["FNCST_X", "FNCST_Y"]
BOND_FIELDS = ["IDIST", "FAC", "SCR", "FAIL"]


@pytest.fixture(scope="module")
def E():
    from pd_gpu1_gb300 import engine

    engine.lib()
    return engine


@pytest.fixture(scope="module")
def base():
    from pd_gpu1_gb300 import presets

    b, _, meta = presets.build_batch(count=1)
    return b, meta["load"]


def standalone(E, base, sp):
    from pd_gpu1_gb300 import presets

    p, setup = presets.build_specimen(base, sp)
    eng = E.Engine(p)
    setup(eng)
    return eng


def bonds_of(eng, rows, remap=None):
    """Per-bond arrays and neighbour lists of the given rows, in row order."""
    rp, NL = eng.csr()
    idx = np.concatenate([np.arange(rp[r], rp[r + 1]) for r in rows])
    nl = NL[idx] if remap is None else remap[NL[idx]]
    return idx, nl


def test_batch_setup_is_the_standalone_setup(E, base):
    b, load = base
    bat = E.Batch(b, SPECS)
    assert bat.count == len(SPECS)
    assert np.all(bat.interior[:-1] % 32 == 0)
    for k, sp in enumerate(SPECS):
        one = standalone(E, b, sp)
        rows = bat.rows(k)
        # standalone node j -> batch node rows[j]
        ib, nlb = bonds_of(bat, rows)
        io, nlo = bonds_of(one, np.arange(one.p.N), remap=rows)
        np.testing.assert_array_equal(bat.get("NN")[rows], one.get("NN"), err_msg=f"NN {k}")
        np.testing.assert_array_equal(nlb, nlo, err_msg=f"NL {k}")
        for f in BOND_FIELDS:
            np.testing.assert_array_equal(bat.get(f)[ib], one.get(f)[io], err_msg=f"{f} {k}")
        for f in NODE_FIELDS:
            np.testing.assert_array_equal(bat.specimen_field(f, k), one.get(f), err_msg=f"{f} {k}")
        assert (one.get("FAIL") == 0).any() == (sp["crack_len"] > 0.0)
        one.close()
    # padding rows have no bonds
    nn = bat.get("NN")
    for k, sp in enumerate(SPECS):
        assert np.all(nn[bat.interior[k] + sp["nx"] * sp["ny"]: bat.interior[k + 1]] == 0)
    bat.close()


def test_batch_forces_bitwise(E, base):
    b, _ = base
    bat = E.Batch(b, SPECS)
    rng = np.random.default_rng(5)
    ux, uy = np.zeros(bat.p.N), np.zeros(bat.p.N)
    ones = []
    for k, sp in enumerate(SPECS):
        one = standalone(E, b, sp)
        # strains up to ~4e-3: some bonds of the low-s0 specimens break
        vx = rng.standard_normal(one.p.N) * 2.0e-6
        vy = rng.standard_normal(one.p.N) * 2.0e-6
        one.set("UX", vx)
        one.set("UY", vy)
        ux[bat.rows(k)] = vx
        uy[bat.rows(k)] = vy
        ones.append(one)
    bat.set("UX", ux)
    bat.set("UY", uy)
    for _ in range(2):  # the second pass sees the bonds the first one broke
        bat.bond_force_gpu()
        for one in ones:
            one.bond_force_gpu()
    fx, fy = bat.get("FX"), bat.get("FY")
    for k, one in enumerate(ones):
        r = bat.rows(k)
        np.testing.assert_array_equal(fx[r], one.get("FX"), err_msg=f"fx {k}")
        np.testing.assert_array_equal(fy[r], one.get("FY"), err_msg=f"fy {k}")
        ib, _ = bonds_of(bat, r)
        io, _ = bonds_of(one, np.arange(one.p.N))
        np.testing.assert_array_equal(bat.get("FAIL")[ib], one.get("FAIL")[io], err_msg=f"fail {k}")
        one.close()
    bat.close()


def test_batch_adr_matches_standalone_runs(E, base):
    b, load = base
    bat = E.Batch(b, SPECS)
    ones = [standalone(E, b, sp) for sp in SPECS]
    bat.run_adr(0, 1, load)
    for one, sp in zip(ones, SPECS):
        one.run_adr(0, 1, load * sp["load_scale"])
    ux, uy = bat.get("UX"), bat.get("UY")
    cn = bat.cn()
    for k, one in enumerate(ones):
        r = bat.rows(k)
        np.testing.assert_array_equal(ux[r], one.get("UX"), err_msg=f"ux step 1, {k}")
        np.testing.assert_array_equal(uy[r], one.get("UY"), err_msg=f"uy step 1, {k}")
        assert cn[k] == pytest.approx(one.adr_cn(), rel=1e-12, abs=0.0)
    bat.run_adr(1, 39, load)
    for one, sp in zip(ones, SPECS):
        one.run_adr(1, 39, load * sp["load_scale"])
    ux, uy, cn = bat.get("UX"), bat.get("UY"), bat.cn()
    broke = 0
    for k, one in enumerate(ones):
        r = bat.rows(k)
        assert_close_norm(ux[r], one.get("UX"), 1e-9, f"ux {k}")
        assert_close_norm(uy[r], one.get("UY"), 1e-9, f"uy {k}")
        assert cn[k] == pytest.approx(one.adr_cn(), rel=1e-9)
        ib, _ = bonds_of(bat, r)
        io, _ = bonds_of(one, np.arange(one.p.N))
        fb, fo = bat.get("FAIL")[ib], one.get("FAIL")[io]
        assert (fb != fo).sum() <= 0.001 * len(fo)
        broke += int((fo == 0).sum())
        one.close()
    assert broke > 0
    bat.close()


def test_batch_specimen_matches_oracle(E, base):
    """A batch specimen against the oracle's ADR restatement (40 steps)."""
    b, load = base
    sp = SPECS[0]
    bat = E.Batch(b, [SPECS[1], sp])
    one = standalone(E, b, sp)
    m = orc.Model(one.p, one.get("X"), one.get("Y"))
    m.find_neighbor()
    m.surface_correct()
    m.set_crack_2d(sp["crack_len"], 0.0, 0.0, sp["crack_theta"])
    one.close()
    bat.run_adr(0, 40, load)
    for ct in range(40):
        m.quick_load(load)
        m.adr_step(ct)
    r = bat.rows(1)
    n = sp["nx"] * sp["ny"]
    assert_close_norm(bat.get("UX")[r][:n], m.ux[:n], 1e-9, "ux")
    assert_close_norm(bat.get("UY")[r][:n], m.uy[:n], 1e-9, "uy")
    assert bat.cn()[1] == pytest.approx(m.cn, rel=1e-9)
    bat.close()


@pytest.mark.parametrize("shape", [(128, 1, 2, 1), (512, 0, 4, 1), (256, 1, 1, 1), (128, 0, 1, 2), (256, 0, 2, 4),
                                   (512, 0, 1, 8)])
def test_launch_shapes_bitwise(E, base, shape):
    b, load = base
    ref = E.Batch(b, SPECS)
    alt = E.Batch(b, SPECS)
    alt.set_launch(*shape)
    assert alt.launch() == shape
    ref.run_adr(0, 30, load)
    alt.run_adr(0, 30, load)
    for f in ["UX", "UY", "VHX", "VHY", "FX", "FY", "FAIL"]:
        np.testing.assert_array_equal(alt.get(f), ref.get(f), err_msg=f)
    np.testing.assert_array_equal(alt.cn(), ref.cn())
    ref.close()
    alt.close()


def test_launch_shape_explicit_bitwise(E):
    from pd_gpu1_gb300 import presets

    p, setup, meta = presets.build_crack_branching(scale=0.05, nt=40)
    a, c = E.Engine(p), E.Engine(p)
    setup(a)
    setup(c)
    c.set_launch(512, 1, 2)
    d = E.Engine(p)
    setup(d)
    d.set_launch(256, 0, 1, 4)  # four warps per slice
    a.run_explicit(40)
    c.run_explicit(40)
    d.run_explicit(40)
    for f in ["UX", "UY", "VX", "VY", "FAIL"]:
        np.testing.assert_array_equal(a.get(f), c.get(f), err_msg=f)
        np.testing.assert_array_equal(a.get(f), d.get(f), err_msg="split " + f)
    a.close()
    c.close()
    d.close()


def test_autotune_leaves_the_run_unchanged(E, base):
    b, load = base
    ref = E.Batch(b, SPECS)
    tun = E.Batch(b, SPECS)
    ref.run_adr(0, 40, load)
    tun.run_adr(0, 20, load)
    block, chunked, waves, split, ms = tun.autotune(reps=3)
    assert block in (128, 256, 512) and chunked in (0, 1) and waves in (1, 2, 4, 8) and split in (1, 2, 4)
    assert ms > 0.0
    tun.run_adr(20, 20, load)
    for f in ["UX", "UY", "FAIL"]:
        np.testing.assert_array_equal(tun.get(f), ref.get(f), err_msg=f)
    ref.close()
    tun.close()


def test_batch_refuses_single_plate_loops(E, base):
    import ctypes as C

    from pd_gpu1_gb300._abi import PD_ERR_ARG, PD_ERR_STATE, PD_ERR_UNSUPPORTED

    b, load = base
    bat = E.Batch(b, SPECS[:2])
    lib = bat._lib
    assert lib.pd_run_adr(bat.ctx, 0, 1, load, None) == PD_ERR_UNSUPPORTED
    assert lib.pd_run_explicit(bat.ctx, 1, 0.0, 0, None) == PD_ERR_UNSUPPORTED
    one = standalone(E, b, SPECS[0])
    assert lib.pd_batch_run_adr(one.ctx, 0, 1, load, None) == PD_ERR_STATE
    assert lib.pd_set_launch(one.ctx, 64, 0, 1, 1) != 0
    assert lib.pd_set_launch(one.ctx, 128, 1, 1, 2) != 0  # a split slice needs the strided order
    q = bat.params()
    q.dt = 2.0 * q.dt
    assert lib.pd_set_params(bat.ctx, C.byref(q)) == PD_ERR_ARG  # per-node coefficients hold the batch's dt
    one.close()
    bat.close()


def test_full_seeded_batch_first_step(E):
    """The 256-specimen benchmark batch (6.25M nodes): one ADR step, then the
    smallest, median and largest specimens against their standalone runs."""
    from pd_gpu1_gb300 import presets

    b, specs, meta = presets.build_batch()
    bat = E.Batch(b, specs)
    assert bat.p.N_int >= sum(s["nx"] * s["ny"] for s in specs)
    bat.run_adr(0, 2, meta["load"])
    bat.check_finite()
    sizes = np.array([s["nx"] * s["ny"] for s in specs])
    order = np.argsort(sizes, kind="stable")
    ux = bat.get("UY")
    for k in (order[0], order[len(order) // 2], order[-1]):
        one = standalone(E, b, specs[k])
        one.run_adr(0, 2, meta["load"])
        assert_close_norm(ux[bat.rows(k)], one.get("UY"), 1e-12, f"uy specimen {k}")
        one.close()
    bat.close()
