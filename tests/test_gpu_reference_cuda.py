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
from helpers import assert_close_norm, params_from_golden

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
