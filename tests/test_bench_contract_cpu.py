"""The reference arm of bench.py (the oracle's OpenMP loops on the host
cores; no GPU) prints one JSON line with the keys its consumers read: the
metric and unit of the GPU arm, the CPU baseline that describes the run, and
an end-to-end entry with no host-device traffic."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                         check=True, capture_output=True, text=True, cwd=ROOT, timeout=600)
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


def test_reference_arm_line():
    d = _run("--steps", "1", "--warmup", "3")
    assert d["impl"] == "reference"
    assert d["metric"] == "bond-updates/s" and d["unit"] == "bond-updates/s"
    assert d["higher_is_better"] is True and d["scaling"] == "weak" and d["vs_baseline"] is None
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 3
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"] == "crack_branching_2d_pmb_verlet"
    assert d["config"]["nodes"] == 1_600_000 and d["config"]["bonds"] == 44_699_236
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_without_a_counterpart_says_so():
    d = _run("--workload", "warm_start", "--steps", "1", "--warmup", "3")
    assert d["impl"] == "reference" and d["unavailable"]


def test_damage_parity_of_a_short_precracked_run():
    """bench.damage_parity on a run shorter than the damage interval: the
    pre-cracked plate (the headline workload's layout, 16,000 nodes) after 20
    explicit steps on the oracle, its damage computed once after the last
    step as the bench now asks of the reference's kernels.  The pre-crack
    alone damages nodes, so both sides count damaged nodes and agree."""
    import numpy as np

    sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]
    import bench
    import oracle as orc
    from pd_gpu1_gb300 import presets

    p, setup, meta = presets.build_crack_branching(scale=0.1, derive=orc.derive_params)
    x, y = orc.plate_coords(p)
    m = orc.Model(p, x, y)
    m.find_neighbor()
    m.surface_correct()
    m.set_crack_2d(p.length / 2.0, -p.length / 4.0, 0.0, 0.0)
    m.by[:] = presets.traction_field(p, meta["sigma"])
    for _ in range(20):
        m.explicit_step()
    m.damage()
    d = m.dmg[: p.N_int].copy()
    rep = bench.damage_parity(d, d, x[: p.N_int], None, p.delta, 20)
    assert rep["damaged_nodes"] > 0 and rep["damaged_nodes"] == rep["damaged_nodes_engine"]
    assert rep["damage_nodes_equal"] == 1.0 and rep["damage_max_abs_diff"] == 0.0
    assert rep["crack_tip_x"]["engine"] == rep["crack_tip_x"]["reference"] is not None
    # a reference field that was never computed (all zero) is reported as a mismatch
    bad = bench.damage_parity(d, np.zeros_like(d), x[: p.N_int], None, p.delta, 20)
    assert bad["damaged_nodes"] == 0 and bad["damage_nodes_equal"] < 1.0


def test_roofline_tables_cover_the_step_workloads():
    """The ncu-derived tables behind the bench line's roofline: every explicit
    workload has a DRAM-traffic and an FP64-count entry, each at least the
    bond loop's own count (kernel source) and within a sane range, and the
    FP64 block takes the ncu count (per-node work included) where there is
    one."""
    sys.path[:0] = [ROOT]
    import bench

    for w in ["crack_branching_2d_pmb_verlet", "kalthoff_winkler_3d_pmb_verlet", "plate_crack_grow_2d_state_verlet",
              "kalthoff_winkler_3d_state_verlet"]:
        assert w in bench.TRAFFIC and w in bench.FP64_NCU_PER_BOND, w
        per_bond, per_node, src = bench.TRAFFIC[w]
        assert 12.125 <= per_bond <= 200.0 and per_node >= 0.0 and src
    loop = {"crack_branching_2d_pmb_verlet": (1, 2), "kalthoff_winkler_3d_pmb_verlet": (1, 3),
            "plate_crack_grow_2d_state_verlet": (2, 2), "kalthoff_winkler_3d_state_verlet": (2, 3)}
    for w, (model, dim) in loop.items():
        n_ncu, src = bench.FP64_NCU_PER_BOND[w]
        assert bench.FP64_EXEC_PER_BOND[(model, dim)] <= n_ncu <= 2.0 * bench.FP64_EXEC_PER_BOND[(model, dim)], w
        blk = bench.fp64_block(model, dim, 1_000_000, 1.0, 500.0, w)
        assert blk["executed_per_bond_ncu"] == n_ncu
        assert abs(blk["achieved_ginst_s"] - n_ncu) < 1e-9  # 1e6 bonds in 1 ms: n per ns
        assert abs(blk["frac"] - n_ncu / 500.0) < 1e-12
    blk = bench.fp64_block(1, 2, 1_000_000, 1.0, 500.0, "batch_plate_adr_2d_pmb")  # no ncu count
    assert "executed_per_bond_ncu" not in blk and blk["executed_per_bond"] == 4
