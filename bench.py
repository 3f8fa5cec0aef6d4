"""Benchmark: bond-updates/s of the peridynamics step loop on GB300.

Default workload: the 1.6M-node dynamic crack-branching plate (2-D PMB,
explicit Verlet, FP64, damage field every 100 steps).  A "step" is one time
step (force + breakage + Verlet) over the whole plate; the metric is
B_initial * steps / loop time, where B_initial is the number of directed bonds
of the force-computed nodes (broken bonds still count: both implementations
visit them).  Setup (neighbour build, surface correction) is timed separately.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload crack_branching|plate_tensile|kalthoff_winkler|kalthoff_winkler_bond|
                              crack_grow|batch|warm_start]

--workload batch: 256 seeded uneven plates (6.25M interior nodes) solved
together by ADR (1000 steps), against the same plates run one after another
(the engine's single-plate loop, and the reference's own kernels).
--workload warm_start: ADR wall-time to a 1e-6 relative residual per load
increment of the 1M-node plate, learned start against the plain start.
--workload kalthoff_winkler_bond: the reference's own impact driver (3-D
bond-based with the rigid impactor); kalthoff_winkler is the state-based
version of the same slab.

Where the reference's kernels were compiled here (oracle/_ref/ref_kernels.cubin)
the line also carries a `reference_cuda` key: the reference's own step loop
for the workload timed on the same GPU, and the damage field after the whole
run compared node by node with the engine's.

--impl reference times the oracle's OpenMP host loop (the reference's
formulas, its padded-ELL layout) on all host cores, on a bounded sample of the
same workload.  Under torchrun (N > 1) every rank runs an independent replica
(the workload does not shard); value is the sum over ranks, timed as the max.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ALG_BYTES_PER_BOND_2D = 12.125  # int32 neighbour + one FP64 coefficient + one fail bit
ALG_BYTES_PER_NODE_2D = 48.0    # read x, y, ux, uy; write fx, fy
ALG_BYTES_PER_BOND_3D = 12.125
ALG_BYTES_PER_NODE_3D = 72.0
# FP64 instructions the force kernels execute per bond in their bond loops,
# counted in the kernel source (csrc/force.cu): the bond vector's FP64
# subtractions with the reference's roundings, two per component (bond_offset),
# plus in the state-based passes the dilatation-order vector of the theta pass
# (the 3-D force pass takes its length's z term from the theta pass).  Bonds
# within two float ulps of their break threshold add one; per-node epilogue
# instructions are not counted.
FP64_EXEC_PER_BOND = {(1, 2): 4, (1, 3): 6, (2, 2): 8, (2, 3): 12}  # (model, dim), compact layouts
# FP64 instructions per bond of the step's force launches with their per-node
# work (epilogues, theta, divisions) included: ncu's FP64 pipe use of one
# capture per workload (sm__inst_executed_pipe_fp64 percentage of peak x 2
# instructions per cycle per SM x active cycles x 152 SMs), over the capture's
# bonds (kernels and case below)
FP64_NCU_PER_BOND = {
    "crack_branching_2d_pmb_verlet": (4.97, "k_bond_compact<1>, 400k-node quarter-size plate, 2026-12-04"),
    "kalthoff_winkler_3d_pmb_verlet": (7.05, "k_bond_compact3<EPI_NONE>, full slab, 2026-12-04"),
    "plate_crack_grow_2d_state_verlet": (10.55, "k_theta_compact 4.52 + k_state_compact<1> 6.03, full plate, "
                                                "2026-12-04"),
    "kalthoff_winkler_3d_state_verlet": (12.60, "k_theta_compact3 6.20 + k_state_compact3<0> 6.40, full slab, "
                                                "2026-12-04")}
# DRAM bytes per bond and per node of the step kernel: ncu dram__bytes_read.sum +
# dram__bytes_write.sum of one capture per workload (kernel, case, date below),
# scaled to the timed launch's bonds and nodes; a zero per-node figure means the
# node traffic is folded into the per-bond one
TRAFFIC = {
    "crack_branching_2d_pmb_verlet": (21.1, 0.0, "k_bond_compact<1>, 400k-node quarter-size plate (node traffic folded "
                                                 "into the per-bond figure), 2026-12-04"),
    "batch_plate_adr_2d_pmb": (22.5, 0.0, "k_bond_compact<2>, 64-plate batch (node traffic folded in), 2026-12-04"),
    "kalthoff_winkler_3d_pmb_verlet": (17.5, 0.0, "k_bond_compact3<EPI_NONE>, full slab (the Verlet and contact "
                                                  "epilogue's node traffic not included), 2026-12-04"),
    "plate_crack_grow_2d_state_verlet": (42.5, 0.0, "k_theta_compact + k_state_compact<1>, full plate, 2026-12-04"),
    "kalthoff_winkler_3d_state_verlet": (67.5, 0.0, "k_theta_compact3 + k_state_compact3<0> (z offset carried), full "
                                                    "slab, 2026-12-04")}


def layout_info(model, dim, layout, epi):
    """(kernel names of the step's force launches, per-slot bytes the step
    reads and writes in them) for the force layout in use."""
    compact = layout == "compact"
    if model == 1:
        if dim == 2:
            return ("k_bond_compact<%s>" % epi, 16) if compact else ("k_bond_force<2, %s>" % epi, 48)
        return ("k_bond_compact3<%s>" % epi, 16) if compact else \
            ("k_bond_force<3, %s> / k_bond_split3 (the autotuner's pick)" % epi, 48)
    if dim == 2:
        # dilatation: 16-byte record + e written; force: 8-byte record + e read
        return ("k_theta_compact + k_state_compact<%s>" % epi, 16 + 8 + 8 + 8) if compact else \
            ("k_theta<2> + k_state_force<2, %s>" % epi, 64 + 8 + 64 + 8)
    return ("k_theta_compact3 + k_state_compact3<EPI_NONE>", 8 + 16 + 8 + 8 + 8 + 8) if compact else \
        ("k_theta<3> + k_state_force3_phased<4>", 64 + 8 + 64 + 8)


def traffic_of(workload, bonds, nodes):
    """(bytes per launch, description of the capture) from TRAFFIC, or (None, None)."""
    tr = TRAFFIC.get(workload)
    if not tr:
        return None, None
    return tr[0] * bonds + tr[1] * nodes, (f"ncu DRAM bytes of {tr[2]}: {tr[0]} B per bond + {tr[1]} B per node, "
                                           f"scaled to this launch")


def fp64_block(model, dim, bonds, kern_ms, gfma, workload=None):
    """FP64 pipe use of the step's force launches: executed FP64 instructions
    per second against the measured FP64 instruction rate (pd_probe_fp64,
    eight independent DFMA chains per thread).  With an ncu count for the
    workload (FP64_NCU_PER_BOND: per-node work included) that count sets the
    fraction; otherwise the bond loop's count from the kernel source does."""
    n = FP64_EXEC_PER_BOND[(model, dim)]
    rate = n * bonds / (kern_ms * 1e-3) / 1e9
    out = {"executed_per_bond": n, "achieved_ginst_s": rate, "peak_ginst_s": gfma, "frac": rate / gfma,
           "counted": "FP64 instructions of the bond loop, from the kernel source; per-node work not counted",
           "peak_source": "pd_probe_fp64 (independent DFMA chains, all SMs)"}
    if workload in FP64_NCU_PER_BOND:
        m, src = FP64_NCU_PER_BOND[workload]
        rate = m * bonds / (kern_ms * 1e-3) / 1e9
        out.update({"executed_per_bond_ncu": m, "achieved_ginst_s": rate, "frac": rate / gfma,
                    "counted": f"FP64 instructions per bond with the per-node work, ncu FP64 pipe use of {src}; "
                               f"the bond loop alone executes {n} per bond (kernel source)"})
    return out


def rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class NvmlSampler:
    """SM clock and clock-event reasons of the GPU, read through NVML (ctypes on
    the driver's libnvidia-ml) every ~2 ms in a thread while the timed region
    runs: a region of a few milliseconds still gets samples.  Reads only."""

    SW_POWER_CAP, HW_SLOWDOWN, SW_THERMAL, HW_THERMAL = 0x4, 0x8, 0x20, 0x40

    def __init__(self, props):
        import ctypes as C

        self.C = C
        self.nv = C.CDLL("libnvidia-ml.so.1")
        if self.nv.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = C.c_void_p()
        uuid = str(props.uuid)
        uuid = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
        bus = "%08x:%02x:%02x.0" % (props.pci_domain_id, props.pci_bus_id, props.pci_device_id)
        if self.nv.nvmlDeviceGetHandleByUUID(uuid.encode(), C.byref(self.h)) != 0 and \
                self.nv.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), C.byref(self.h)) != 0:
            raise OSError("no NVML handle for " + uuid)
        self.reasons_fn = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = C.c_uint()
        self.nv.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(mx))
        self.max_mhz = float(mx.value)
        self.samples, self.stop_flag, self.t = [], False, None

    def _poll(self):
        C = self.C
        mhz, rs = C.c_uint(), C.c_ulonglong()
        while not self.stop_flag:
            if self.nv.nvmlDeviceGetClockInfo(self.h, 1, C.byref(mhz)) == 0 and \
                    self.reasons_fn(self.h, C.byref(rs)) == 0:
                self.samples.append((float(mhz.value), int(rs.value)))
            time.sleep(0.002)

    def start(self):
        self.stop_flag = False
        self.t = threading.Thread(target=self._poll, daemon=True)
        self.t.start()

    def stop(self):
        self.stop_flag = True
        if self.t is not None:
            self.t.join(timeout=2)
        names = {self.HW_SLOWDOWN: "hw_slowdown", self.HW_THERMAL: "hw_thermal_slowdown",
                 self.SW_THERMAL: "sw_thermal_slowdown", self.SW_POWER_CAP: "sw_power_cap"}
        reasons = sorted({nm for _, r in self.samples for bit, nm in names.items() if r & bit})
        sm = [m for m, _ in self.samples]
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": self.max_mhz, "reasons": reasons,
                "samples": len(sm), "source": "NVML, every ~2 ms during the timed region"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region
    (NVML polling where the driver's library loads; nvidia-smi at 200 ms
    otherwise)."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.nvml = None
        try:
            import torch

            self.nvml = NvmlSampler(torch.cuda.get_device_properties(gpu_index))
        except Exception:
            self.nvml = None

    def start(self):
        if self.nvml is not None:
            self.nvml.start()
            return
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.nvml is not None:
            return self.nvml.stop()
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi, every 200 ms"}


def aggregate_replicas(elapsed_s, work, dist=None, device="cpu"):
    """Replicas only: every rank times its own copy of the workload.  Returns
    (max elapsed over ranks, total work over ranks); the job's throughput is
    total work / max elapsed."""
    if dist is None:
        return elapsed_s, work
    import torch

    t = torch.tensor([elapsed_s], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    w = torch.tensor([float(work)], dtype=torch.float64, device=device)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return float(t.item()), float(w.item())


def build_workload(name, scale, host_only=False):
    """Parameters, engine set-up and metadata of a named workload.  With
    host_only the parameters come from the oracle's derivation (bit-identical,
    pinned by tests) so the CPU arm never loads the CUDA library."""
    from pd_gpu1_gb300 import presets

    kw = {}
    if host_only:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc

        kw = {"derive": orc.derive_params}
    if name == "crack_branching":
        return presets.build_crack_branching(scale=scale, **kw)
    if name == "plate_tensile":
        return presets.build_plate_tensile(scale=scale, **kw)
    if name in ("kalthoff_winkler", "kalthoff_winkler_bond"):
        from pd_gpu1_gb300._abi import PD_MODEL_BOND

        if host_only:
            kw["coord_fn"] = orc.coord_kw
        if name == "kalthoff_winkler_bond":  # the reference's own impact driver is bond-based
            kw["model"] = PD_MODEL_BOND
        return presets.build_kalthoff_winkler(scale=scale, **kw)
    if name == "crack_grow":
        return presets.build_crack_grow(scale=scale, **kw)
    raise SystemExit(f"unknown workload {name}")


def run_steps(eng, meta, k, ct0=0):
    if meta["workload"].startswith("plate_tensile"):
        eng.run_adr(ct0, k, load=meta["load"])
    else:
        eng.run_explicit(k, load=meta["load"], dmg_every=meta.get("dmg_every", 0))


# ----------------------------------------------------------------------------------------------
def cpu_reference(p, meta, eng_coords, max_seconds, max_steps, threads):
    """The oracle on the host cores: setup, then timed steps until max_seconds
    or max_steps.  Returns (bond-updates/s, steps, seconds, bonds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    orc.set_threads(threads)
    x, y, z = eng_coords
    m = orc.Model(p, x, y, z)
    m.find_neighbor(brute=False)
    w = meta["workload"]
    if w.startswith("crack_branching"):
        m.surface_correct()
        m.set_crack_2d(p.length / 2.0, -p.length / 4.0, 0.0, 0.0)
        from pd_gpu1_gb300.presets import traction_field

        m.by[:] = traction_field(p, meta["sigma"])
    elif w.startswith("plate_tensile"):
        m.surface_correct()
    elif w.startswith("kalthoff"):
        if p.model == 1:
            m.surface_correct()
        else:
            m.vol_corr()
            m.initial_weight()
        m.set_crack_kw(meta["rad"])
    else:
        m.set_crack_2d(0.01 * p.length / 0.05, 0.0, 0.0, 0.0)
        m.vol_corr()
        m.initial_weight()
    bonds = int(m.NN[: p.N_int].sum())
    cyl = None
    if w.startswith("kalthoff"):
        c = meta["cylinder"]
        cyl = orc.new_cylinder(c.rad, c.mass, c.height, c.v, c.x, c.y, c.z)
    t0 = time.perf_counter()
    n = 0
    while n < max_steps:
        if w.startswith("plate_tensile"):
            m.quick_load(meta["load"])
            m.adr_step(n)
        else:
            m.explicit_step(load=meta["load"], cyl=cyl)
            if meta.get("dmg_every") and (n + 1) % meta["dmg_every"] == 0:
                m.damage()
        n += 1
        if time.perf_counter() - t0 > max_seconds:
            break
    dt = time.perf_counter() - t0
    return bonds * n / dt, n, dt, bonds


def reference_arm(args):
    rank, world, _ = rank_info()
    if rank != 0:
        return 0
    p, setup, meta = build_workload(args.workload, args.scale, host_only=True)
    coords = host_coords(p, meta)
    threads = os.cpu_count() or 1
    # warm-up: a short sample; then the timed sample bounded to ~60 s
    rate, steps, secs, bonds = cpu_reference(p, meta, coords, max_seconds=min(60.0, 2.0 + 4.0 * args.steps),
                                             max_steps=args.warmup + args.steps, threads=threads)
    line = {
        "impl": "reference", "metric": "bond-updates/s", "value": rate, "unit": "bond-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (deterministic lattice)",
        "config": {"workload": meta["workload"], "nodes": p.N, "bonds": bonds, "dx": p.dx},
        "cpu_baseline": {"value": rate, "unit": "bond-updates/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} time steps of the full {meta['workload']} plate ({p.N} nodes), "
                                   f"{secs:.1f} s; OpenMP restatement of the reference's loops"},
        "e2e": {"value": rate, "unit": "bond-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def reference_cuda_kw(eng, p, setup, meta, args, value, B):
    """The reference's impact-driver loop (kernel_bond_force_3D, kernel_contact,
    the 3-D Verlet halves and the cylinder kernels, compiled from its sources)
    on the same slab and GPU: its rate, and the intact flags and damage after
    the whole run against the engine's, both from the same initial state (the
    reference run twice: its contact reaction is summed by atomicAdd, so two of
    its runs need not agree to the last bit)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_gpu

    if not ref_gpu.available():
        return None
    cyl = meta["cylinder"]
    setup(eng)
    r, NN = ref_gpu.from_engine(eng, p, cyl=cyl)
    kref = min(args.steps, 300)
    r.run_kw(args.warmup)
    ms_ref = r.run_kw(kref)
    rate = B * kref / (ms_ref * 1e-3)
    runs = []
    for _ in range(2):
        setup(eng)
        r.free()
        r, NN = ref_gpu.from_engine(eng, p, cyl=cyl)
        r.run_kw(args.steps)
        out = r.get(NN)
        out.update(r.get_z())
        runs.append(out)
    r.free()
    # the engine twice: its tuned launch shape and another one (the impactor's
    # reaction is then summed in another block order)
    shape = eng.launch()
    alt = (256, 0, 1, 1) if tuple(shape) != (256, 0, 1, 1) else (128, 0, 1, 4)
    eng.set_launch(*alt)
    setup(eng)
    run_steps(eng, meta, args.steps)
    fe1, uy1 = eng.get("FAIL"), eng.get("UY")
    eng.set_launch(*shape)
    setup(eng)
    cut = int((eng.get("FAIL") == 0).sum())  # the notch cuts
    run_steps(eng, meta, args.steps)
    fac = eng.get("FAC")
    fe = eng.get("FAIL")
    de = ref_gpu.damage_from_flags(NN, fe, fac, p.vol)[: p.N_int]
    de1 = ref_gpu.damage_from_flags(NN, fe1, fac, p.vol)[: p.N_int]
    dr = [ref_gpu.damage_from_flags(NN, o["fail"], fac, p.vol)[: p.N_int] for o in runs]
    uy = eng.get("UY")

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    return {"unit": "bond-updates/s", "steps": kref, "kernel_bond_force_3D_loop": rate, "best": rate,
            "engine_over_best": value / rate,
            "what": "the reference's impact-driver loop (integrate_3D_1, cy_integrate_1, bond_force_3D, contact, "
                    "integrate_3D_2, cy_integrate_2; compiled from its sources, FP64), kernel_integrate_3D_1 "
                    "given its arrays by declared name",
            "damage_after_steps": args.steps,
            "damage_nodes_equal": float(np.mean(np.abs(de - dr[0]) <= 1e-12)),
            "damage_max_abs_diff": float(np.abs(de - dr[0]).max()),
            "bonds_broken": {"engine": int((fe == 0).sum()), "reference": int((runs[0]["fail"] == 0).sum()),
                             "notch_cuts": cut},
            "intact_flags_equal": float(np.mean(fe == runs[0]["fail"])),
            "damaged_nodes": int((dr[0] > 0).sum()),
            "uy_rel_diff": rel(uy, runs[0]["uy"]),
            "impactor_vel_y": {"engine": float(eng.cylinder().vel[1]), "reference": float(runs[0]["cyl_vel"][1])},
            "reference_runs_between_themselves": {
                "damage_nodes_equal": float(np.mean(np.abs(dr[1] - dr[0]) <= 1e-12)),
                "uy_rel_diff": rel(runs[1]["uy"], runs[0]["uy"])},
            "engine_runs_between_launch_shapes": {
                "shapes": [list(shape), list(alt)],
                "damage_nodes_equal": float(np.mean(np.abs(de1 - de) <= 1e-12)),
                "uy_rel_diff": rel(uy1, uy)}}


def reference_cuda_state(eng, p, setup, meta, args, value, B):
    """The reference's crack-grow loop (kernel_cal_theta_2D, kernel_state_force_2D,
    the Verlet halves and the boundary motion, compiled from its sources) on
    the same plate and GPU: its rate, and the damage field after the whole
    run against the engine's, both from the same initial state."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_gpu

    if not ref_gpu.available():
        return None
    setup(eng)
    r, NN = ref_gpu.from_engine(eng, p)
    kref = min(args.steps, 300)
    r.run_state(args.warmup, meta["load"])
    ms_ref = r.run_state(kref, meta["load"])
    rate = B * kref / (ms_ref * 1e-3)
    r.free()
    setup(eng)
    r, NN = ref_gpu.from_engine(eng, p)
    r.run_state(args.steps, meta["load"], dmg_every=args.steps)  # kernel_cal_dmg_2D after the last step
    out = r.get(NN)
    r.free()
    setup(eng)
    run_steps(eng, meta, args.steps)
    eng.damage()
    de, dr = eng.get("DMG")[: p.N_int], out["dmg"][: p.N_int]
    xs = eng.get("X")[: p.N_int]
    tip_e = eng.crack_tip(0.38)[0]
    return {"unit": "bond-updates/s", "steps": kref, "kernel_state_force_2D_loop": rate, "best": rate,
            "engine_over_best": value / rate,
            "what": "the reference's crack-grow loop (quick_load, integrate_2D_1, cal_theta_2D, state_force_2D, "
                    "integrate_2D_2; compiled from its sources, FP64)",
            **damage_parity(de, dr, xs, tip_e, p.delta, args.steps),
            "intact_flags_equal": float(np.mean(eng.get("FAIL") == out["fail"]))}


def crack_tip_x(d, xs, threshold=0.38):
    """x of the rightmost node whose damage exceeds the threshold (None: none
    does), the row scan the reference's crack-grow driver carries in a comment
    (Solve_Plate_Crack_Grow.cu:150-162)."""
    hot = np.nonzero(d > threshold)[0]
    return float(xs[hot].max()) if len(hot) else None


def damage_parity(de, dr, xs, tip_e, horizon, steps):
    """Damage fields of two runs from the same initial state compared node by
    node: the fraction of nodes equal to 1e-12, the largest difference, the
    damaged nodes on each side and the crack tips (tip_e: the engine's own
    pd_crack_tip, else taken from de)."""
    tip_a = crack_tip_x(de, xs) if tip_e is None or tip_e != tip_e else float(tip_e)
    return {"damage_after_steps": steps,
            "damage_nodes_equal": float(np.mean(np.abs(de - dr) <= 1e-12)),
            "damage_max_abs_diff": float(np.abs(de - dr).max()) if len(de) else 0.0,
            "damaged_nodes": int((dr > 0).sum()), "damaged_nodes_engine": int((de > 0).sum()),
            "crack_tip_x": {"engine": tip_a, "reference": crack_tip_x(dr, xs), "horizon": horizon}}


def r_inputs(eng, p):
    """The engine context's problem in the argument order of RefGPU.setup."""
    return (eng.get("X"), eng.get("Y"), eng.get("NN"), eng.get("ROWPTR"), eng.get("NL"), eng.get("IDIST"),
            eng.get("SCR"), eng.get("FAC"), eng.get("FAIL"), eng.get("BX"), eng.get("BY"))


def host_coords(p, meta):
    """Node coordinates of the workload, computed on the host (same formulas as the engine)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    w = meta["workload"]
    if w.startswith("crack_branching"):
        x, y = orc.plate_coords(p)
        return x, y, None
    if w.startswith("plate_tensile") or w.startswith("plate_crack"):
        x, y = orc.plate_crack_coords(p)
        return x, y, None
    return meta["coords"]


# ---- batch of plates -------------------------------------------------------------------------
ALG_BYTES_PER_NODE_2D_ADR = 88.0  # P (x+u: 16) ... as 2-D + vh, fo (32) + ADR mass (8) for the damping sums


def batch_host_specimen(base, sp):
    """Host-only parameters and coordinates of one batch specimen (oracle
    derivation, bit-identical to the engine's, pinned by tests)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from pd_gpu1_gb300 import presets

    p, _ = presets.build_specimen(base, sp, derive=orc.derive_params)
    x, y = orc.plate_crack_coords(p)
    return p, x, y


def batch_cpu_reference(base, specs, load, max_seconds, steps_each, threads):
    """The oracle's ADR loop on the host cores over the specimens in order,
    steps_each steps per specimen, until max_seconds.  Returns (bond-updates/s,
    specimens, steps, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    orc.set_threads(threads)
    work = secs = 0.0
    done = steps = nodes = 0
    for sp in specs:
        p, x, y = batch_host_specimen(base, sp)
        m = orc.Model(p, x, y)
        m.find_neighbor(brute=False)
        m.surface_correct()
        if sp["crack_len"] > 0.0:
            m.set_crack_2d(sp["crack_len"], 0.0, 0.0, sp["crack_theta"])
        bonds = int(m.NN[: p.N_int].sum())
        nodes += p.N_int
        t0 = time.perf_counter()
        for ct in range(steps_each):
            m.quick_load(load * sp["load_scale"])
            m.adr_step(ct)
        secs += time.perf_counter() - t0
        work += bonds * steps_each
        done += 1
        steps += steps_each
        if secs > max_seconds:
            break
    # time one step of the whole batch would take at this rate (bonds per node of the sample)
    total_nodes = sum(int(sp["nx"]) * int(sp["ny"]) for sp in specs)
    ms_batch_step = (work / steps_each) / nodes * total_nodes / (work / secs) * 1e3
    return work / secs, done, steps, secs, ms_batch_step


def batch_reference_arm(args, base, specs, meta):
    threads = os.cpu_count() or 1
    rate, done, steps, secs, ms_step = batch_cpu_reference(base, specs, meta["load"],
                                                           min(60.0, 2.0 + 4.0 * args.steps), max(args.warmup, 5),
                                                           threads)
    line = {
        "impl": "reference", "metric": "bond-updates/s", "value": rate, "unit": "bond-updates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": f"synthetic (seeded specimens, seed "
                                                                       f"{meta['seed']})",
        "config": {"workload": meta["workload"], "specimens": len(specs), "dx": base.dx},
        "cpu_baseline": {"value": rate, "unit": "bond-updates/s", "cores": threads, "kind": "port",
                         "sample": f"{done} specimens of the batch in order, {steps // max(done, 1)} ADR steps "
                                   f"each ({secs:.1f} s); OpenMP restatement of the reference's loops, one plate "
                                   f"after another"},
        "e2e": {"value": rate, "unit": "bond-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def batch_arm(args):
    import ctypes as C

    import torch

    from pd_gpu1_gb300 import presets

    rank, world, local = rank_info()
    if args.impl == "reference":
        if rank != 0:
            return 0
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as orc

        base, specs, meta = presets.build_batch(count=args.count, nt=args.steps, derive=orc.derive_params)
        return batch_reference_arm(args, base, specs, meta)
    base, specs, meta = presets.build_batch(count=args.count, nt=args.steps)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from pd_gpu1_gb300 import engine as E
    from pd_gpu1_gb300._abi import FIELD
    from pd_gpu1_gb300._lib import lib

    L = lib()
    load = meta["load"]
    stream = torch.cuda.Stream()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        bat = E.Batch(base, specs, stream=stream.cuda_stream)
        bat.sync()
    setup_s = time.perf_counter() - t0
    p = bat.p
    rp = bat.get("ROWPTR")
    B = int(rp[p.N_int])
    fail0 = bat.get("FAIL")
    zeros = np.zeros(p.N)

    def reset():
        for k in ["UX", "UY", "VX", "VY", "VHX", "VHY", "FOX", "FOY", "FX", "FY"]:
            bat.set(k, zeros)
        bat.set("FAIL", fail0)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    # launch shape: the autotuner times the ADR force kernel at the initial state
    # (or the fixed shape of --launch)
    if args.launch:
        bat.set_launch(*(int(v) for v in args.launch.split(",")))
        tuned = bat.launch() + (None,)
    else:
        with torch.cuda.stream(stream):
            tuned = bat.autotune(reps=5)
    # warm-up, then the timed steps
    with torch.cuda.stream(stream):
        bat.run_adr(0, args.warmup, load)
    barrier()
    launches0 = bat.kernel_launches
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    ev0.record(stream)
    with torch.cuda.stream(stream):
        bat.run_adr(args.warmup, args.steps, load)
    ev1.record(stream)
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    launches = bat.kernel_launches - launches0
    secs_max, work = aggregate_replicas(ms * 1e-3, B * args.steps, dist, "cuda")
    value = work / secs_max
    broken = float((bat.get("FAIL") == 0).mean())

    # the force kernel (ADR epilogue with per-slice damping sums) inside the
    # step loop: CUDA events on the launch stream around each step's launch
    with torch.cuda.stream(stream):
        kern_ms, step_ms = bat.profile_steps(0, args.warmup + args.steps, min(50, args.steps), load)
    layout = bat.force_layout()
    torch.cuda.synchronize()
    alg_bytes = ALG_BYTES_PER_NODE_2D_ADR * p.N_int + ALG_BYTES_PER_BOND_2D * B
    peaks, peak_kind = measured_peaks()
    achieved = alg_bytes / (kern_ms * 1e-3) / 1e9
    traffic, traffic_src = traffic_of(meta["workload"], B, p.N_int)

    # end to end through the C ABI with host buffers: the initial state goes up
    # from pinned host memory, the displacement field comes back every 100 steps
    n = p.N
    reset()
    names_up = ["UX", "UY", "VHX", "VHY", "FOX", "FOY"]
    pin = {k: torch.zeros(n, dtype=torch.float64).pin_memory() for k in names_up}
    barrier()
    h2d = d2h = 0
    t0 = time.perf_counter()
    for k in names_up:
        bat._c(L.pd_set_field(bat.ctx, FIELD[k], pin[k].data_ptr(), n, bat.stream), "pd_set_field")
        h2d += n * 8
    done = 0
    while done < args.steps:
        k_run = min(100, args.steps - done)
        bat.run_adr(done, k_run, load)
        done += k_run
        for k in ["UX", "UY"]:
            bat._c(L.pd_get_field(bat.ctx, FIELD[k], pin[k].data_ptr(), n, bat.stream), "pd_get_field")
            d2h += n * 8
    e2e_s, e2e_work = aggregate_replicas(time.perf_counter() - t0, B * args.steps, dist, "cuda")
    e2e = {"value": e2e_work / e2e_s, "unit": "bond-updates/s", "h2d_bytes_per_step": h2d / args.steps,
           "d2h_bytes_per_step": d2h / args.steps}
    bat.close()
    # the FP64 instruction rate, after the timed runs (the probe saturates the
    # FP64 pipe of every SM for ~60 ms)
    gfma = C.c_double()
    L.pd_probe_fp64(C.byref(gfma))

    sequential = ref_cuda = cpu = None
    if rank == 0 and world == 1:
        # the same plates one after another through the engine's single-plate loop
        k_seq = min(args.steps, args.seq_steps)
        engines, bonds = [], []
        for sp in specs:
            q, setup = presets.build_specimen(base, sp)
            e = E.Engine(q, stream=stream.cuda_stream)
            with torch.cuda.stream(stream):
                setup(e)
            engines.append(e)
            bonds.append(int(e.get("ROWPTR")[q.N_int]))
        with torch.cuda.stream(stream):
            for e, sp in zip(engines, specs):
                e.run_adr(0, 3, load * sp["load_scale"])
        barrier()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        with torch.cuda.stream(stream):
            for e, sp in zip(engines, specs):
                e.run_adr(3, k_seq, load * sp["load_scale"])
        s1.record(stream)
        barrier()
        seq_ms = s0.elapsed_time(s1)
        sequential = {"value": sum(bonds) * k_seq / (seq_ms * 1e-3), "unit": "bond-updates/s", "steps_each": k_seq,
                      "what": "the same specimens one after another, pd_run_adr per plate (CUDA graphs)"}
        # the reference's own kernels, one plate after another
        if not args.no_ref_cuda:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import ref_gpu

            if ref_gpu.available():
                k_ref = min(args.steps, args.seq_steps)
                tot_ms, tot_work = 0.0, 0.0
                for e, sp, b in zip(engines, specs, bonds):
                    r, _ = ref_gpu.from_engine(e, e.p)
                    r.run_adr(0, 3, load * sp["load_scale"])
                    ms_r, _ = r.run_adr(3, k_ref, load * sp["load_scale"])
                    tot_ms += ms_r
                    tot_work += b * k_ref
                    r.free()
                best = tot_work / (tot_ms * 1e-3)
                ref_cuda = {"unit": "bond-updates/s", "steps_each": k_ref, "best": best,
                            "engine_over_best": value / best,
                            "what": "the reference's kernels (compiled from its sources, FP64), its ADR loop "
                                    "(particle force, kernel_cnn, two host-read sums, kernel_integrate) per plate, "
                                    "one plate after another; loop time summed over plates"}
        for e in engines:
            e.close()
        if not args.no_cpu:
            rate, ndone, steps, secs, _ = batch_cpu_reference(base, specs, load, args.cpu_seconds, 100,
                                                              os.cpu_count() or 1)
            cpu = {"value": rate, "unit": "bond-updates/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"{ndone} specimens of the batch in order, 100 ADR steps each ({secs:.1f} s of "
                             f"host time), the oracle's OpenMP loops"}

    if rank == 0:
        kname, slot_bytes = layout_info(1, 2, layout, "EPI_ADR")
        line = {
            "metric": "bond-updates/s", "value": value, "unit": "bond-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs_max * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": f"synthetic (seeded specimen table, seed {meta['seed']})",
            "config": {"workload": meta["workload"], "specimens": len(specs), "nodes": p.N, "interior": p.N_int,
                       "bonds": B, "dx": p.dx, "dt": p.dt, "parallelism": "replicas" if world > 1 else "single",
                       "launch": {"block": tuned[0], "chunked": tuned[1], "waves": tuned[2], "split": tuned[3]},
                       "force_layout": layout,
                       "l2": "inputs larger than L2: per-slot records %.2f GB read per step" % (B * slot_bytes / 1e9),
                       "setup_s": setup_s, "broken_bond_fraction": broken},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved / peaks["hbm_gbs"], "traffic": traffic, "traffic_source": traffic_src,
                         "peak_source": peak_kind,
                         "kernel": kname, "kernel_ms": kern_ms,
                         "kernel_share_of_step": kern_ms / step_ms, "autotune_ms": tuned[4],
                         "alg_bytes_per_launch": alg_bytes,
                         "fp64": fp64_block(1, 2, B, kern_ms, gfma.value)},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk, "sequential": sequential,
            "reference_cuda": ref_cuda,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---- learned ADR warm start ---------------------------------------------------------------------
def warm_measure(scale, K, smooth, n_plain=1, e2e=True, with_clocks=True):
    """ADR wall-time per load increment to a 1e-6 relative residual on the
    warm-start plate (1M nodes at scale 1).  Increment 0 (no displacement yet,
    so no proportional start) is solved first, untimed, and its converged
    state kept (a snapshot).  From that state each start then solves its own
    chain of increments 1..K, timed: the learned start (network shipped in
    pd_gpu1_gb300/data, offered beside the skip term; the smaller starting
    residual wins; every solved increment without crack advance becomes the
    next prediction's history) and the skip term alone (proportional, secant,
    increment).  A chain is the fair comparison: the state an increment
    converges to seeds the next prediction, so each start inherits its own
    earlier stopping error.  The plain start (previous solution) needs the
    same ~23k ADR steps on every increment; n_plain of them are timed from
    the same state.  Returns the dict of the JSON line (without the common
    keys)."""
    import os
    import tempfile

    import torch

    from pd_gpu1_gb300 import engine as E
    from pd_gpu1_gb300 import presets, warm
    from pd_gpu1_gb300._abi import FIELD
    from pd_gpu1_gb300._lib import lib

    L = lib()
    p, setup, meta = presets.build_warm_start_plate(scale=scale)
    net = warm.Net.load()
    snap_dir = tempfile.mkdtemp()
    snap = os.path.join(snap_dir, "state.snap")
    clocks = ClockSampler(torch.cuda.current_device()) if with_clocks else None
    delta = meta["delta"]
    with E.Engine(p) as eng:
        setup(eng)
        B = int(eng.get("ROWPTR")[p.N_int])
        tuned = eng.autotune(reps=5)  # the bond kernel's launch shape, at the initial state
        first = warm.run_increments(eng, meta, 1, mode="plain")[0]  # increment 0; clears the history
        eng.snapshot_save(snap)
        if clocks:
            clocks.start()
        l0 = eng.kernel_launches
        learned = warm.run_increments(eng, meta, K, mode="learned", net=net, start=1, smooth=smooth)
        learned_launches = eng.kernel_launches - l0
        eng.snapshot_load(snap)
        warm.clear_history(eng, delta)
        skip = warm.run_increments(eng, meta, K, mode="secant", net=net, start=1, record=False)
        plain = []
        for _ in range(n_plain):
            eng.snapshot_load(snap)
            plain += warm.run_increments(eng, meta, 1, mode="plain", start=1, record=False)
        clk = clocks.stop() if clocks else None
        # the network's forward pass alone (four tcgen05 products with their
        # epilogues) on the features of the state, then the whole prediction
        # (features, forward pass, smoothing passes, candidates)
        du = torch.zeros(4 * p.N_int, dtype=torch.float64, device="cuda")
        Xf = torch.zeros((p.N_int, 16), dtype=torch.bfloat16, device="cuda")
        Yf = torch.zeros((p.N_int, 2), dtype=torch.float32, device="cuda")
        eng.damage()
        U = 1 * delta
        L.pd_warm_features(eng.ctx, U, delta, Xf.data_ptr(), None)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(5):
            L.pd_mlp_forward(net.h, Xf.data_ptr(), p.N_int, Yf.data_ptr(), None)
        e1.record()
        torch.cuda.synchronize()
        infer_ms = e0.elapsed_time(e1) / 5
        e0.record()
        for _ in range(5):
            L.pd_warm_predict(eng.ctx, net.h, U, delta, smooth, du.data_ptr(), None)
        e1.record()
        torch.cuda.synchronize()
        predict_ms = e0.elapsed_time(e1) / 5
        e2e_ms = None
        if e2e:
            # the learned chain again, from the same state, through the C ABI
            # with the displacement field read back to pinned host memory after
            # each increment (an increment's input is its load step)
            eng.snapshot_load(snap)
            warm.clear_history(eng, delta)
            n = p.N
            pin = torch.zeros(n, dtype=torch.float64).pin_memory()
            t0 = time.perf_counter()
            for j in range(K):
                warm.run_increments(eng, meta, 1, mode="learned", net=net, start=1 + j, smooth=smooth)
                eng._c(L.pd_get_field(eng.ctx, FIELD["UY"], pin.data_ptr(), n, None), "pd_get_field")
            e2e_ms = (time.perf_counter() - t0) * 1e3 / K
    os.remove(snap)
    os.rmdir(snap_dir)
    # per increment: the prediction (features, network, smoothing, candidates),
    # the solve and the history record (run_increments' ms_total)
    plain_ms = float(np.mean([s["ms_total"] for s in plain]))
    skip_ms = float(np.sum([s["ms_total"] for s in skip]))
    learned_ms = float(np.sum([s["ms_total"] for s in learned]))
    flops = 2.0 * p.N_int * (16 * 128 + 2 * 128 * 128 + 128 * 16)
    peaks, peak_kind = measured_peaks()
    return {
        "value": learned_ms / K, "unit": "ms", "steps": K, "warmup": 1,
        "config": {"workload": meta["workload"], "nodes": p.N, "bonds": B, "dx": p.dx, "increment_m": delta,
                   "tol": 1e-6, "timed_increments": list(range(1, K + 1)), "smooth_passes": smooth,
                   "untimed": "increment 0 (plain start, %d ADR steps); every chain starts from its state"
                              % first["iters"],
                   "launch": {"block": tuned[0], "chunked": tuned[1], "waves": tuned[2], "split": tuned[3]}},
        "plain": {"ms_per_increment": plain_ms, "iters": [s["iters"] for s in plain],
                  "what": "increment 1 from the previous solution"},
        "skip_only": {"ms_per_increment": skip_ms / K, "iters": [s["iters"] for s in skip],
                      "total_iters": int(sum(s["iters"] for s in skip)),
                      "what": "the proportional (secant) increment alone, against the plain start, increments 1..%d"
                              % K},
        "learned": {"ms_per_increment": learned_ms / K, "iters": [s["iters"] for s in learned],
                    "total_iters": int(sum(s["iters"] for s in learned)),
                    "start_used": [s["start"] for s in learned],
                    "starts": "plain: the previous solution; network: skip term + history + network correction; "
                              "skip: the skip term alone (the only candidate offered without a history: "
                              "increment 1 and the one after a crack advance)",
                    "r_start_over_r_plain": [s["r_start"] / s["r_plain"] for s in learned],
                    "bonds_broken": [s["advanced"] for s in learned]},
        "speedup_vs_plain": plain_ms / (learned_ms / K),
        "speedup_vs_skip_only": skip_ms / learned_ms,
        "roofline": {"bound": "tensor", "kernel": "k_mlp_fused (the network's forward pass: four layers per 128-row tile, TMA-fed)",
                     "achieved": flops / (infer_ms * 1e-3) / 1e12, "peak": peaks.get("bf16_tflops"),
                     "unit": "TFLOP/s", "frac": flops / (infer_ms * 1e-3) / 1e12 / peaks.get("bf16_tflops", 1.0),
                     "traffic": None, "peak_source": peak_kind, "forward_ms": infer_ms,
                     "predict_ms": predict_ms,
                     "note": "predict_ms: features, forward pass, smoothing passes and candidates, %.1f %% of a "
                             "learned increment; an increment is bound by the ADR force kernel"
                             % (100.0 * predict_ms / max(learned_ms / K, 1e-9))},
        "e2e": None if e2e_ms is None else {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": p.N * 8},
        "gpu_launches": learned_launches // max(K, 1),
        "gpu_launches_what": "per timed increment (ADR steps in CUDA graphs, features, network, candidates)",
        "clocks": clk,
    }


def warm_arm(args):
    """--workload warm_start: warm_measure on the 1M-node plate as its own line."""
    import torch

    rank, world, local = rank_info()
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no load stepping, residual or "
                              "learned start (it runs a fixed number of ADR steps); its ADR step loop is timed by "
                              "--workload plate_tensile and batch"}), flush=True)
        return 0
    torch.cuda.set_device(local)
    m = warm_measure(args.scale, args.increments, args.smooth, n_plain=args.plain_increments)
    line = {"metric": "ADR wall-time to a 1e-6 relative residual per load increment, learned start",
            "value": m.pop("value"), "unit": m.pop("unit"), "n_gpus": world, "steps": m.pop("steps"),
            "warmup": m.pop("warmup"), "ms_per_step": None, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (solver); bf16 x bf16 -> f32 (network)",
            "data": "synthetic (deterministic lattice)", "cpu_baseline": None}
    line["ms_per_step"] = line["value"]
    line.update(m)
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def batch_block(steps, warmup, count=256):
    """The batch workload (256 seeded uneven plates, ADR) as a block
    of the default line: set-up, the autotuned launch shape, warmup + steps
    ADR steps timed with CUDA events on the launch stream (batch_arm gives the
    full line with its comparisons)."""
    import torch

    from pd_gpu1_gb300 import engine as E
    from pd_gpu1_gb300 import presets

    base, specs, meta = presets.build_batch(count=count, nt=steps)
    stream = torch.cuda.Stream()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        bat = E.Batch(base, specs, stream=stream.cuda_stream)
        bat.sync()
    setup_s = time.perf_counter() - t0
    p = bat.p
    B = int(bat.get("ROWPTR")[p.N_int])
    with torch.cuda.stream(stream):
        tuned = bat.autotune(reps=5)
        bat.run_adr(0, warmup, meta["load"])
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    with torch.cuda.stream(stream):
        bat.run_adr(warmup, steps, meta["load"])
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    with torch.cuda.stream(stream):
        kern_ms, step_ms = bat.profile_steps(0, warmup + steps, min(50, steps), meta["load"])
    torch.cuda.synchronize()
    layout = bat.force_layout()
    bat.close()
    return {"metric": "bond-updates/s", "value": B * steps / (ms * 1e-3), "unit": "bond-updates/s",
            "steps": steps, "warmup": warmup, "ms_per_step": ms / steps,
            "config": {"workload": meta["workload"], "specimens": len(specs), "seed": meta["seed"], "nodes": p.N,
                       "bonds": B, "setup_s": setup_s, "force_layout": layout,
                       "launch": {"block": tuned[0], "chunked": tuned[1], "waves": tuned[2], "split": tuned[3]}},
            "kernel": "k_bond_compact<EPI_ADR>" if layout == "compact" else "k_bond_force<2, EPI_ADR>",
            "kernel_ms": kern_ms, "kernel_share_of_step": kern_ms / step_ms,
            "what": "bench.py --workload batch gives this workload's own line with the one-plate-after-another "
                    "and reference-kernel comparisons"}


# ----------------------------------------------------------------------------------------------
def gb300_arm(args):
    import ctypes as C

    import torch

    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from pd_gpu1_gb300 import engine as E
    from pd_gpu1_gb300._lib import lib

    p, setup, meta = build_workload(args.workload, args.scale)
    stream = torch.cuda.Stream()
    eng = E.Engine(p, stream=stream.cuda_stream)
    eng.set_force_layout(args.layout)
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        setup(eng)
        eng.sync()
    setup_s = time.perf_counter() - t0
    B = int(eng.get("ROWPTR")[p.N_int])
    is3d = p.dim == 3
    # the initial state, restored before the end-to-end runs without rebuilding
    # the family (a rebuild drops the step graphs the timed runs captured)
    import tempfile

    snap_dir = tempfile.mkdtemp()
    snap0 = os.path.join(snap_dir, "initial.snap")
    eng.snapshot_save(snap0)
    tuned = None
    if args.launch:
        tuned = tuple(int(v) for v in args.launch.split(","))
        eng.set_launch(*tuned)
    elif p.model == 1 and not args.no_tune:
        # launch shape of the bond kernel: the library's autotuner at the initial state
        with torch.cuda.stream(stream):
            tuned = eng.autotune(reps=5)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    # warm-up
    with torch.cuda.stream(stream):
        run_steps(eng, meta, args.warmup)
    barrier()
    launches0 = eng.kernel_launches
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    ev0.record(stream)
    with torch.cuda.stream(stream):
        run_steps(eng, meta, args.steps, ct0=args.warmup)
    ev1.record(stream)
    barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    launches = eng.kernel_launches - launches0
    secs_max, work = aggregate_replicas(ms * 1e-3, B * args.steps, dist, "cuda")
    ms_max = secs_max * 1e3
    value = work / secs_max

    # the dominant kernel inside the step loop: CUDA events on the launch stream
    # around every step's force launch(es), over further real steps
    kern_steps = min(100, max(10, args.steps))
    kind = 0 if meta["workload"].startswith("plate_tensile") else 1
    with torch.cuda.stream(stream):
        kern_ms, step_ms = eng.profile_steps(kind, args.warmup + args.steps, kern_steps, meta["load"])
    layout = eng.force_layout()
    kname, slot_bytes = layout_info(p.model, p.dim, layout, "EPI_ADR" if kind == 0 else "EPI_VERLET")
    torch.cuda.synchronize()
    state = p.model == 2
    if state:  # dilatation + force passes (the 3-D state-based byte model; 2-D by the same count)
        alg_bytes = (88.0 if is3d else 64.0) * p.N_int + 16.125 * B
    else:
        alg_bytes = (ALG_BYTES_PER_NODE_3D if is3d else ALG_BYTES_PER_NODE_2D) * p.N_int + \
            (ALG_BYTES_PER_BOND_3D if is3d else ALG_BYTES_PER_BOND_2D) * B
    peaks, peak_kind = measured_peaks()
    achieved = alg_bytes / (kern_ms * 1e-3) / 1e9
    # DRAM bytes per launch from one ncu capture of the same kernel (the case
    # and date are carried in the line), scaled by bonds and nodes
    traffic, traffic_src = traffic_of(meta["workload"], B, p.N_int)

    # end to end through the C ABI with host buffers: the initial state and the
    # loading go up from pinned host memory, the damage field comes back at
    # every dump and the displacement field at the end, all inside the timed
    # region (pd_set_field / pd_get_field, which block on their copies)
    L = lib()
    from pd_gpu1_gb300._abi import FIELD

    n = p.N
    names_up = ["UX", "UY", "VX", "VY", "BX", "BY"] + (["UZ", "VZ", "BZ"] if is3d else [])
    eng.snapshot_load(snap0)  # the workload's initial state (family, corrections, cracks, loads, impactor)
    pin = {k: torch.from_numpy(eng.get(k)).pin_memory() for k in names_up}
    # results land in buffers of their own: the inputs stay the initial state
    # for every run
    names_down = ["UX", "UY"] + (["UZ"] if is3d else [])
    pout = {k: torch.zeros(n, dtype=torch.float64).pin_memory() for k in names_down + ["DMG"]}

    def e2e_run():
        """The job from the initial state: inputs uploaded from pinned host
        memory, the steps, the damage dumps and the final displacement read
        back; returns (seconds, bytes up, bytes down, phase seconds: uploads,
        steps with the dumps, final downloads)."""
        eng.snapshot_load(snap0)
        barrier()
        up = down = 0
        t0 = time.perf_counter()
        for k in names_up:
            eng._c(L.pd_set_field(eng.ctx, FIELD[k], pin[k].data_ptr(), n, eng.stream), "pd_set_field")
            up += n * 8
        t1 = time.perf_counter()
        every = meta.get("dmg_every") or args.steps
        done = 0
        while done < args.steps:
            k_run = min(every, args.steps - done)
            run_steps(eng, meta, k_run, ct0=done)
            done += k_run
            if meta.get("dmg_every"):
                eng._c(L.pd_get_field(eng.ctx, FIELD["DMG"], pout["DMG"].data_ptr(), n, eng.stream), "pd_get_field")
                down += n * 8
        eng.sync()
        t2 = time.perf_counter()
        for k in names_down:
            eng._c(L.pd_get_field(eng.ctx, FIELD[k], pout[k].data_ptr(), n, eng.stream), "pd_get_field")
            down += n * 8
        t3 = time.perf_counter()
        return t3 - t0, up, down, (t1 - t0, t2 - t1, t3 - t2)

    with torch.cuda.stream(stream):
        e2e_run()  # warm-up, as for the device-timed steps: the step graphs of this run's chunks
        first = {k: pout[k].numpy().copy() for k in names_down}
        e2e_clocks = ClockSampler(torch.cuda.current_device())
        e2e_clocks.start()
        secs, h2d, d2h, phases = e2e_run()
        e2e_clk = e2e_clocks.stop()
    # the timed run solved the same job: its result equals the warm-up run's bit for bit
    e2e_same = all(np.array_equal(first[k], pout[k].numpy()) for k in names_down)
    e2e_s, e2e_work = aggregate_replicas(secs, B * args.steps, dist, "cuda")
    os.remove(snap0)
    os.rmdir(snap_dir)
    e2e = {"value": e2e_work / e2e_s, "unit": "bond-updates/s",
           "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
           "phases_ms": {"upload": phases[0] * 1e3, "steps_and_dumps": phases[1] * 1e3,
                         "download": phases[2] * 1e3},
           "clocks": e2e_clk, "same_result_as_untimed_run": e2e_same}
    # the FP64 instruction rate, after the timed runs (the probe saturates the
    # FP64 pipe of every SM for ~60 ms)
    gfma = C.c_double()
    lib().pd_probe_fp64(C.byref(gfma))

    # the reference's own CUDA kernels on the same GPU and plate, when their
    # cubin was built (oracle/_ref/ref_kernels.cubin, from the reference sources)
    ref_cuda = None
    if rank == 0 and not args.no_ref_cuda and p.dim == 2 and p.model == 1 and meta["workload"].startswith("crack"):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import ref_gpu

        if ref_gpu.available():
            setup(eng)
            r, _ = ref_gpu.from_engine(eng, p)
            kref = min(args.steps, 300)
            rates = {}
            for name, variant in (("kernel_particle_force_2D", ref_gpu.RefGPU.PARTICLE),
                                  ("kernel_bond_force_2D", ref_gpu.RefGPU.WARP)):
                r.setup(p, *r_inputs(eng, p))
                r.run(variant, args.warmup, meta.get("dmg_every", 0))
                ms_ref = r.run(variant, kref, meta.get("dmg_every", 0))
                rates[name] = B * kref / (ms_ref * 1e-3)
            # the damage field after the whole run, both implementations from the
            # same initial state: nodes whose damage agrees, and the crack tips.
            # The reference's kernel_cal_dmg_2D runs once after its last step
            # (the damage field does not feed back into these steps), whatever
            # the step count: a run shorter than the dump interval still compares
            # two computed fields
            setup(eng)
            dref = {}
            for name, variant in (("particle", ref_gpu.RefGPU.PARTICLE), ("warp", ref_gpu.RefGPU.WARP)):
                r.setup(p, *r_inputs(eng, p))
                r.run(variant, args.steps, args.steps)
                dref[name] = r.get()["dmg"][: p.N_int]
            r.free()
            run_steps(eng, meta, args.steps)
            eng.damage()
            de, dr = eng.get("DMG")[: p.N_int], dref["particle"]
            xs = eng.get("X")[: p.N_int]
            tip_e = eng.crack_tip(0.38)[0]
            best = max(rates.values())
            ref_cuda = {"unit": "bond-updates/s", "steps": kref, **rates, "best": best,
                        "engine_over_best": value / best,
                        "what": "the reference's kernels (compiled from its sources, FP64) in its step loop: "
                                "integrate_2D_1, force, integrate_2D_2, damage every 100 steps",
                        **damage_parity(de, dr, xs, tip_e, p.delta, args.steps),
                        "reference_kernels_between_themselves": {
                            **damage_parity(dref["warp"], dr, xs, None, p.delta, args.steps),
                            "what": "kernel_bond_force_2D against kernel_particle_force_2D (same formulas, "
                                    "different summation order)"}}

    if rank == 0 and not args.no_ref_cuda and p.dim == 3 and p.model == 1 and meta["workload"].startswith("kalthoff"):
        ref_cuda = reference_cuda_kw(eng, p, setup, meta, args, value, B)
    if rank == 0 and not args.no_ref_cuda and p.dim == 2 and p.model == 2 and meta["workload"].startswith("plate_crack"):
        ref_cuda = reference_cuda_state(eng, p, setup, meta, args, value, B)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, steps, secs, bonds = cpu_reference(p, meta, host_coords(p, meta), max_seconds=args.cpu_seconds,
                                                 max_steps=100000, threads=os.cpu_count() or 1)
        cpu = {"value": rate, "unit": "bond-updates/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{steps} time steps of the same {p.N}-node plate ({secs:.1f} s of host time), "
                         f"the oracle's OpenMP loops"}

    # the other two workloads of the headline metric, as blocks of the same line:
    # the second half of the metric (ADR wall-time to a 1e-6 residual, learned
    # start against plain and skip-only starts) and the batch of uneven plates
    extras = {}
    if rank == 0 and world == 1 and not args.no_extras and meta["workload"].startswith("crack_branching"):
        eng.close()
        eng = None
        extras["adr_warm_start"] = warm_measure(1.0, 10, args.smooth, e2e=False)
        extras["batch"] = batch_block(200, 5)

    if rank == 0:
        line = {
            "metric": "bond-updates/s", "value": value, "unit": "bond-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (deterministic lattice, seeded nothing: the geometry fixes every input)",
            "config": {"workload": meta["workload"], "nodes": p.N, "bonds": B, "dx": p.dx, "dt": p.dt,
                       "parallelism": "replicas" if world > 1 else "single",
                       "force_layout": layout,
                       "l2": "inputs larger than L2: per-slot records %.2f GB read per step" % (B * slot_bytes / 1e9),
                       "setup_s": setup_s,
                       "launch": None if tuned is None else {"block": tuned[0], "chunked": tuned[1],
                                                             "waves": tuned[2], "split": tuned[3]}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved / peaks["hbm_gbs"], "traffic": traffic, "traffic_source": traffic_src,
                         "peak_source": peak_kind,
                         "kernel": kname,
                         "kernel_ms": kern_ms, "kernel_share_of_step": kern_ms / step_ms,
                         "alg_bytes_per_launch": alg_bytes,
                         "fp64": fp64_block(p.model, p.dim, B, kern_ms, gfma.value, meta["workload"])},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk, "reference_cuda": ref_cuda,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    if eng is not None:
        eng.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="time steps (default: the workload's nt)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="crack_branching")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ref-cuda", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape of the bond kernel")
    ap.add_argument("--launch", default=None, help="fixed launch shape of the bond kernel, block,chunked,waves,split "
                                                    "(instead of the autotuner)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--count", type=int, default=256, help="batch workload: number of specimens")
    ap.add_argument("--seq-steps", type=int, default=100, help="batch workload: steps per plate when run one "
                                                                "after another")
    ap.add_argument("--increments", type=int, default=10, help="warm_start workload: chained load increments "
                                                                "timed per start")
    ap.add_argument("--smooth", type=int, default=None, help="warm_start workload: family-averaging passes of the "
                                                           "network's correction")
    ap.add_argument("--plain-increments", type=int, default=1, help="warm_start workload: plain-start increments "
                                                                     "timed (each ~23k ADR steps at 1M nodes)")
    ap.add_argument("--layout", default="auto", choices=["auto", "compact", "records"],
                    help="force layout of the bond kernels (auto: compact where it fits)")
    ap.add_argument("--no-extras", action="store_true", help="default workload: leave out the batch and "
                                                                  "learned-warm-start blocks of the line")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.smooth is None:
        from pd_gpu1_gb300.warm import SMOOTH_PASSES

        args.smooth = SMOOTH_PASSES
    if args.steps is None:
        args.steps = {"crack_branching": 1800, "plate_tensile": 1000, "kalthoff_winkler": 1350,
                      "kalthoff_winkler_bond": 1350,
                      "crack_grow": 1250, "batch": 1000, "warm_start": 3}.get(args.workload, 1800)
    if args.workload == "batch":
        return batch_arm(args)
    if args.workload == "warm_start":
        return warm_arm(args)
    if args.impl == "reference":
        return reference_arm(args)
    return gb300_arm(args)


if __name__ == "__main__":
    sys.exit(main())
