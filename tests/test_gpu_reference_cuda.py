"""The engine against the reference's own CUDA kernels on the same GPU.

oracle/_ref/ref_kernels.cubin holds the reference's kernels compiled from its
sources (built where the sources are, carried to the GPU with the repository
snapshot); oracle/ref_gpu.py runs them through the CUDA driver API on the same
inputs.  Bars: forces 1e-12 norm-relative, intact flags bit-exact, explicit
runs 1e-9 and at most 0.1 % of the flags different after breakage starts.
"""
import numpy as np
import pytest

import ref_gpu
from helpers import assert_close_norm, check_per_node_2d, params_from_golden

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_gpu.available(), reason="reference cubin not built (make -C oracle ref)")]


@pytest.fixture(scope="module")
def E():
    from pd_gpu1_gb300 import engine

    engine.lib()
    return engine


def test_forces_and_breakage_match_reference_kernels(E, golden):
    g = golden("plate_tensile_bond")
    p = params_from_golden(g)
    with E.Engine(p) as eng:
        eng.set_coords(g["x"], g["y"])
        eng.find_neighbor_gpu()
        eng.surface_correct_gpu()
        eng.initial_state()
        eng.set("UX", g["f_ux"])
        eng.set("UY", g["f_uy"])
        fail0 = eng.get("FAIL")
        eng.bond_force_gpu()
        fx, fy = eng.get("FX"), eng.get("FY")
        for variant in (ref_gpu.RefGPU.PARTICLE, ref_gpu.RefGPU.WARP):
            eng.initial_state()
            r, NN = ref_gpu.from_engine(eng, p)
            r.set_disp(g["f_ux"], g["f_uy"])
            r.force(variant)
            out = r.get(NN)
            assert_close_norm(fx, out["fx"], 1e-12, f"fx variant {variant}")
            assert_close_norm(fy, out["fy"], 1e-12, f"fy variant {variant}")
            rep = check_per_node_2d(eng, fx, fy, out["fx"], out["fy"], g["f_ux"], g["f_uy"], fail0,
                                    what=f"variant {variant}")
            print("per-node forces:", rep)
            r.free()
        # breakage at a lowered critical stretch: identical intact flags
        q = eng.params()
        q.critical_s = float(g["b_s0"])
        eng.set_params(q)
        eng.initial_state()
        r, NN = ref_gpu.from_engine(eng, q)
        eng.set("UX", g["f_ux"])
        eng.set("UY", g["f_uy"])
        r.set_disp(g["f_ux"], g["f_uy"])
        for _ in range(2):
            eng.bond_force_gpu()
            r.force(ref_gpu.RefGPU.PARTICLE)
        out = r.get(NN)
        np.testing.assert_array_equal(eng.get("FAIL"), out["fail"])
        assert_close_norm(eng.get("FX"), out["fx"], 1e-12, "fx after breaks")
        r.free()


def test_explicit_crack_branching_matches_reference_kernels(E):
    from pd_gpu1_gb300 import presets

    p, setup, meta = presets.build_crack_branching(scale=0.05, nt=150)
    with E.Engine(p) as eng:
        setup(eng)
        r, NN = ref_gpu.from_engine(eng, p)
        eng.run_explicit(150)
        r.run(ref_gpu.RefGPU.PARTICLE, 150)
        out = r.get(NN)
        assert_close_norm(eng.get("UY"), out["uy"], 1e-9, "uy")
        assert_close_norm(eng.get("VY"), out["vy"], 1e-9, "vy")
        fail_e, fail_r = eng.get("FAIL"), out["fail"]
        assert (fail_e != fail_r).sum() <= 0.001 * len(fail_r)
        r.free()


def test_bond_force_3d_matches_reference_kernel(E, golden):
    """kernel_bond_force_3D (4 warps per node, the KW y >= -0.04 breaking guard)
    against the engine's 3-D bond kernel: forces 1e-12, intact flags exact."""
    g = golden("kalthoff_winkler_bond")
    p = params_from_golden(g)
    p.critical_s = float(g["f_s0"])  # low enough that bonds break
    with E.Engine(p) as eng:
        eng.set_coords(g["x"], g["y"], g["z"])
        eng.find_neighbor_gpu()
        eng.surface_correct_gpu()
        eng.initial_state()
        eng.set_crack_kw(float(g["rad"]))
        cut = int((eng.get("FAIL") == 0).sum())  # the notch cuts
        r, NN = ref_gpu.from_engine(eng, p)
        u = {k: g["f_" + k] for k in ("ux", "uy", "uz")}
        for k, v in u.items():
            eng.set(k.upper(), v)
        r.set_disp(u["ux"], u["uy"])
        r.set_disp_z(u["uz"])
        for _ in range(2):  # the second pass sees the bonds the first one broke
            eng.bond_force_gpu()
            r.force3()
        out, oz = r.get(NN), r.get_z()
        for k, ref in (("FX", out["fx"]), ("FY", out["fy"]), ("FZ", oz["fz"])):
            assert_close_norm(eng.get(k), ref, 1e-12, k)
        np.testing.assert_array_equal(eng.get("FAIL"), out["fail"])
        assert (out["fail"] == 0).sum() > cut  # bonds broke beyond the notch cuts
        r.free()


def test_kalthoff_winkler_bond_matches_reference_loop(E):
    """The impact driver's loop (Solve_Kalthoff_Winkler.cu:406-430) on the
    reference's kernels against the engine's fused steps: 100 steps with the
    impactor in contact from the start.  Displacements 1e-9 and the
    impactor's velocity 1e-9; node velocities 1e-7, because contact sets a
    projected node's velocity to (u_new - u_old) / dt (:159-161), which turns
    a displacement difference at the 1e-12 m level into 1e-5 m/s at dt = 1e-7
    s (measured: 1.1e-8 of the largest velocity after 100 steps)."""
    from pd_gpu1_gb300._abi import PD_MODEL_BOND
    from pd_gpu1_gb300 import presets

    p, setup, meta = presets.build_kalthoff_winkler(scale=0.3, dx=2e-3, nt=100, model=PD_MODEL_BOND)
    c = meta["cylinder"]
    c.y -= 0.3 * p.dx  # start 0.3 dx into the slab: contact from the first step
    with E.Engine(p) as eng:
        setup(eng)  # starts the impactor of meta["cylinder"]
        r, NN = ref_gpu.from_engine(eng, p, cyl=c)
        eng.run_explicit(100)
        r.run_kw(100)
        out, oz = r.get(NN), r.get_z()
        assert_close_norm(eng.get("UX"), out["ux"], 1e-9, "ux")
        assert_close_norm(eng.get("UY"), out["uy"], 1e-9, "uy")
        assert_close_norm(eng.get("UZ"), oz["uz"], 1e-9, "uz")
        assert_close_norm(eng.get("VY"), out["vy"], 1e-7, "vy")
        assert_close_norm(eng.get("VZ"), oz["vz"], 1e-7, "vz")
        assert np.abs(out["uy"]).max() > 0.0
        assert eng.cylinder().vel[1] == pytest.approx(oz["cyl_vel"][1], rel=1e-9)
        assert oz["cyl_vel"][1] != -32.0  # the slab pushed back
        np.testing.assert_array_equal(eng.get("FAIL"), out["fail"])
        r.free()


def test_state_force_2d_matches_reference_kernels(E):
    """kernel_cal_theta_2D + kernel_state_force_2D against the engine's
    state-based passes on a cracked plate with boundary rows: forces 1e-12,
    intact flags exact, at strains around s0 (0.04472)."""
    from pd_gpu1_gb300 import presets

    p, setup, meta = presets.build_crack_grow(scale=0.2, nt=10)
    with E.Engine(p) as eng:
        setup(eng)
        cut = int((eng.get("FAIL") == 0).sum())
        r, NN = ref_gpu.from_engine(eng, p)
        rng = np.random.default_rng(11)
        u = rng.standard_normal((2, p.N)) * 2.5e-6  # dx = 1e-4: bond strains of a few percent
        for eng_k, k in (("UX", 0), ("UY", 1)):
            eng.set(eng_k, u[k])
        r.set_disp(u[0], u[1])
        for _ in range(2):  # the second pass sees the bonds the first one broke
            eng.state_force_gpu()
            r.force_state()
        out = r.get(NN)
        assert_close_norm(eng.get("FX")[: p.N_int], out["fx"][: p.N_int], 1e-12, "fx")
        assert_close_norm(eng.get("FY")[: p.N_int], out["fy"][: p.N_int], 1e-12, "fy")
        np.testing.assert_array_equal(eng.get("FAIL"), out["fail"])
        assert (out["fail"] == 0).sum() > cut  # bonds broke beyond the pre-crack
        r.free()


def test_crack_grow_matches_reference_loop(E):
    """The crack-grow driver's state-based loop (Solve_Plate_Crack_Grow.cu:126-149)
    on the reference's kernels against the engine's steps: 40 steps with the
    boundary rows moving; displacements and velocities 1e-9, flags equal."""
    from pd_gpu1_gb300 import presets

    p, setup, meta = presets.build_crack_grow(scale=0.2, nt=40)
    with E.Engine(p) as eng:
        setup(eng)
        r, NN = ref_gpu.from_engine(eng, p)
        eng.run_explicit(40, load=meta["load"])
        r.run_state(40, meta["load"])
        out = r.get(NN)
        assert_close_norm(eng.get("UY"), out["uy"], 1e-9, "uy")
        assert_close_norm(eng.get("UX"), out["ux"], 1e-9, "ux")
        assert_close_norm(eng.get("VY"), out["vy"], 1e-9, "vy")
        assert np.abs(out["uy"][: p.N_int]).max() > 0.0
        np.testing.assert_array_equal(eng.get("FAIL"), out["fail"])
        r.free()


def test_explicit_1000_steps_before_breakage_match_reference_kernels(E):
    """Before any bond breaks: 1,000 explicit Verlet steps of the traction-loaded
    crack-branching plate (critical stretch raised so that no bond breaks)
    on the engine and on the reference's particle-force loop; displacements
    and velocities 1e-9 norm-relative, intact flags identical (the pre-crack
    only)."""
    from pd_gpu1_gb300 import presets

    p, setup, meta = presets.build_crack_branching(scale=0.05, nt=1000)
    p.critical_s = 1.0  # no bond stretches by 100 %
    with E.Engine(p) as eng:
        setup(eng)
        cut = eng.get("FAIL").copy()
        r, NN = ref_gpu.from_engine(eng, p)
        eng.run_explicit(1000)
        r.run(ref_gpu.RefGPU.PARTICLE, 1000)
        out = r.get(NN)
        for k, ref in (("UX", out["ux"]), ("UY", out["uy"]), ("VY", out["vy"])):
            assert_close_norm(eng.get(k), ref, 1e-9, k)
        assert np.abs(out["uy"]).max() > 0.0
        np.testing.assert_array_equal(eng.get("FAIL"), cut)
        np.testing.assert_array_equal(out["fail"], cut)
        r.free()


def test_state_force_3d_matches_reference_kernel(E):
    """kernel_state_force_3D (Force_State.cu:242-306), the 3-D ordinary
    state-based force, against the engine's 3-D state-based passes on a small
    notched slab of the impact layout (1,750 nodes, an even count so that the
    reference kernel's barrier, inside "if (i < N_int)" with two nodes per
    block, is reached by whole blocks).  The reference's own
    kernel_initial_weight_3D supplies m and w (checked against the engine's to
    1e-13).  kernel_cal_theta_3D is not launched (its barrier sits in a branch
    on each bond's intact flag): the dilatation theta and the per-bond
    extension e come from the oracle's restatement of it, evaluated on the
    reference's own intact flags.  Two evaluations at a lowered critical
    stretch, the second seeing the bonds the first broke: forces 1e-12, intact
    flags identical."""
    import oracle as orc
    from pd_gpu1_gb300 import presets
    from pd_gpu1_gb300._abi import PD_MODEL_STATE

    p, setup, meta = presets.build_kalthoff_winkler(scale=0.25, dx=2e-3, nt=10, model=PD_MODEL_STATE)
    assert p.N == p.N_int == 1750 and p.MN == 128
    rng = np.random.default_rng(17)
    u = rng.standard_normal((3, p.N)) * 5e-6  # dx = 2e-3: bond strains around s0 (4.0e-3)
    with E.Engine(p) as eng:
        setup(eng)
        cut = int((eng.get("FAIL") == 0).sum())  # the notch cuts
        r, NN = ref_gpu.from_engine(eng, p)
        try:
            r.setup_state3(eng.get("M"), eng.get("W"))
            r.initial_weight3()
            m_ref, w_ref = r.get_state3()
            mask = (np.arange(p.MN)[None, :] < NN[:, None]).reshape(-1)
            assert_close_norm(eng.get("M"), m_ref, 1e-13, "m")
            assert_close_norm(eng.get("W"), w_ref[mask], 1e-13, "w")
            for k, key in enumerate(("UX", "UY", "UZ")):
                eng.set(key, u[k])
            r.set_disp(u[0], u[1])
            r.set_disp_z(u[2])
            # the oracle's view of the same problem, in the reference's layout
            om = orc.Model(p, eng.get("X"), eng.get("Y"), eng.get("Z"))
            om.NN[:] = NN
            om.NL[:] = r.arrays["NL"]
            om.idist[:] = r.arrays["idist"]
            om.fac[:] = r.arrays["fac"]
            om.w[:] = w_ref
            om.m[:] = m_ref
            om.ux[:], om.uy[:], om.uz[:] = u
            for _ in range(2):  # the second pass sees the bonds the first one broke
                eng.state_force_gpu()
                om.fail[:] = r.get_fail()
                orc.lib().or_state_theta(orc.C.byref(p), *[orc._d(a) for a in (om.x, om.y, om.z, om.ux, om.uy,
                                                                                 om.uz)],
                                         orc._i(om.NN), orc._i(om.NL), orc._d(om.idist), orc._d(om.fac),
                                         orc._d(om.w), orc._d(om.m), orc._i(om.fail), orc._d(om.e),
                                         orc._d(om.theta))
                r.set_theta_e(om.theta, om.e)
                r.force_state3()
            out, oz = r.get(NN), r.get_z()
        finally:
            r.free()
        for k, ref in (("FX", out["fx"]), ("FY", out["fy"]), ("FZ", oz["fz"])):
            assert_close_norm(eng.get(k), ref, 1e-12, k)
        np.testing.assert_array_equal(eng.get("FAIL"), out["fail"])
        assert (out["fail"] == 0).sum() > cut + 1000  # bonds broke beyond the notch cuts
