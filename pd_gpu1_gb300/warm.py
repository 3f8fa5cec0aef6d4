"""Learned ADR warm start: quasi-static load stepping, training data from the
solver's own converged states, training and inference of the per-node MLP on
the tensor cores (``pd_mlp_*`` / ``pd_warm_*`` in include/pd.h).

A load increment moves the boundary rows by +-delta and is solved by ADR to
``|F + b| <= tol * |F + b|_plain`` (``pd_load_step``).  The plain start is the
previous converged solution; the learned start adds the network's predicted
increment ``delta * net(features)`` and is kept only when its residual is
not larger than the plain start's, so the converged answer is the plain
method's.  Features (``pd_warm_features``) and targets are normalised:
features use the accumulated boundary displacement U of the previous
increment and the history of the increment before (its departure from
proportionality and the damage it added, ``pd_warm_record``).  The
prediction is ``u * delta / U + U * net(features)``: a
skip term, the proportional (secant) increment, plus the network's output
scaled by U (optionally smoothed over the bond family, ``smooth``), so the
target of training is ``(du - u * delta / U) / U`` -- the departure from
proportionality per unit of load, which the bonds' geometric nonlinearity
keeps nearly constant along the loading (u = a U + b U^2 departs by
b U delta per increment); consecutive increments depart alike away from a
growing crack, which the history feature carries.  Training uses every
increment of each run, crack advances included; the residual rule decides
between the starts: pd_load_step receives two
candidates, the network's prediction and the skip term alone; a candidate
whose starting residual exceeds the plain start's is dropped, and of two
admissible ones the start with the smaller residual is used (``probe`` > 0
instead runs each for that many ADR steps and keeps the lower residual after
them).

No reference counterpart: the reference runs a fixed number of ADR steps
(Solve_Plate_Tensile.cu:106-131).

  python -m pd_gpu1_gb300.warm train [--out PATH]   # generate data, train, save
"""
import argparse
import ctypes as C
import json
import math
import os
import time

import numpy as np

from . import presets
from ._lib import check, lib
from .engine import Engine

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "data", "warm_mlp_params.f32")
N_PARAMS = 34434
# family-averaging passes applied to the network's correction before it is
# offered as a start (0: none).  The BF16 network's node-to-node rounding noise
# is what the residual, a stiffness-weighted norm, amplifies most.  Measured on
# two unseen plates over 50 increments through crack advances (41k and 80k
# nodes): 0 passes 24,100 / 34,700 ADR steps, 16 passes 22,000 / 31,600, 32
# passes 24,600 / 40,200 (the skip term alone 41,300 / 38,300).
SMOOTH_PASSES = 16


def init_params(seed=0):
    """He-normal hidden weights, zero output layer (the prediction starts at
    the skip term), zero biases, in the flat order of pd_mlp_set_params."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_out, fan_in in ((128, 8), (128, 128), (128, 128), (2, 128)):
        scale = 0.0 if fan_out == 2 else math.sqrt(2.0 / fan_in)
        parts.append(rng.standard_normal(fan_out * fan_in) * scale)
        parts.append(np.zeros(fan_out))
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == N_PARAMS
    return p


class Net:
    """A pd_mlp handle (parameters, optimizer state, activation buffers)."""

    def __init__(self, max_rows=65536, params=None):
        self.L = lib()
        st = C.c_int()
        self.h = self.L.pd_mlp_create(max_rows, C.byref(st))
        if not self.h:
            check(st.value, None, "pd_mlp_create")
        self.max_rows = max_rows
        self.set_params(init_params() if params is None else params)

    def close(self):
        if getattr(self, "h", None):
            self.L.pd_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(self.L.pd_mlp_set_params(self.h, p.ctypes.data, p.size), None, "pd_mlp_set_params")

    def params(self):
        p = np.zeros(N_PARAMS, dtype=np.float32)
        check(self.L.pd_mlp_get_params(self.h, p.ctypes.data, p.size), None, "pd_mlp_get_params")
        return p

    def save(self, path=WEIGHTS):
        os.makedirs(os.path.dirname(path), exist_ok=True)
        self.params().tofile(path)

    @classmethod
    def load(cls, path=WEIGHTS, max_rows=65536):
        p = np.fromfile(path, dtype=np.float32)
        if p.size != N_PARAMS:
            raise ValueError(f"{path}: {p.size} parameters, expected {N_PARAMS}")
        return cls(max_rows, p)

    def train_step(self, x_ptr, t_ptr, rows, lr, stream=None):
        loss = C.c_float()
        check(self.L.pd_mlp_train_step(self.h, x_ptr, t_ptr, rows, C.c_float(lr), C.byref(loss), stream), None,
              "pd_mlp_train_step")
        return loss.value


def run_increments(eng, meta, n_inc, mode="plain", net=None, collect=None, tol=1e-6, max_iters=400000,
                   check_every=100, keep=0.25, seed=0, start=0, probe=0, smooth=SMOOTH_PASSES, record=True,
                   last=None):
    """Solve n_inc load increments on a set-up engine.

    mode: "plain" (previous solution); "learned" (the two candidates of
    pd_warm_predict, network + skip term and skip term alone, against the
    plain start; the admissible one with the smaller residual is used; net
    required); "network" / "secant" (one of the two alone, for ablations);
    "extrapolate" (previous solution plus the previous increment).  Every
    solved increment is recorded as the history of the next prediction
    (pd_warm_record).  smooth: passes of family averaging applied to the
    network's correction (pd_warm_predict).  collect: a list that receives
    (features, targets) device tensors of a random ``keep`` fraction of the
    free nodes of every increment with U > 0 and no crack advance.
    record=False leaves the context's history as it was (a comparison run
    from a snapshot that another run continues from); last: a dict that
    receives the state before the last increment (u0, d0, U: device tensors
    and a float), from which restore_history rebuilds that increment's
    history after a snapshot load.
    Returns the per-increment statistics of pd_load_step, with "start" (the
    start used), "advanced" (bonds broken in the increment) and "ms_total"
    (wall time of the prediction, the solve and the history record; the
    bookkeeping copies of this function are outside it)."""
    import torch

    L = lib()
    ni = eng.p.N_int
    delta = meta["delta"]
    rng = np.random.default_rng(seed)
    du = torch.zeros(4 * ni, dtype=torch.float64, device="cuda")  # two candidates
    X = torch.zeros((ni, 16), dtype=torch.bfloat16, device="cuda") if collect is not None else None
    ux, uy, dmg = eng.device_view("UX", ni), eng.device_view("UY", ni), eng.device_view("DMG", ni)
    u0 = torch.empty(2 * ni, dtype=torch.float64, device="cuda")
    d0 = torch.empty(ni, dtype=torch.float64, device="cuda")
    prev = None
    out = []
    for k in range(start, start + n_inc):
        U = k * delta  # accumulated boundary displacement before this increment
        ptr = None
        eng.damage()
        eng.sync()
        # the state before the increment, kept on the device
        u0[:ni].copy_(ux)
        u0[ni:].copy_(uy)
        d0.copy_(dmg)
        if U > 0.0 and collect is not None:
            check(L.pd_warm_features(eng.ctx, U, delta, X.data_ptr(), eng.stream), eng.ctx, "pd_warm_features")
        broken0 = eng.count_broken()
        hist_set = getattr(eng, "has_history", False)
        hist = getattr(eng, "warm_history", None) if collect is not None else None
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ncand = 1
        if mode in ("learned", "network", "secant") and U > 0.0:
            check(L.pd_warm_predict(eng.ctx, net.h, U, delta, smooth, du.data_ptr(), eng.stream), eng.ctx,
                  "pd_warm_predict")
            ptr = du.data_ptr()  # "network": the network's start against the plain start
            if mode == "learned":  # both candidates
                ncand = 2
            if mode == "secant" or (mode == "learned" and not hist_set and record):
                # the skip term alone; the learned start too when there is no
                # history (the first increments, and the one after a crack advance)
                ptr = du.data_ptr() + 2 * ni * 8
                ncand = 1
        elif mode == "extrapolate" and prev is not None:
            du[: 2 * ni].copy_(prev)
            ptr = du.data_ptr()
        offered = ("plain",) if ptr is None else ("network", "skip") if ncand == 2 else \
            ("skip",) if (mode == "secant" or ptr != du.data_ptr()) else (mode,)
        st = eng.load_step(delta, ptr, tol, max_iters, check_every, ncand, probe if ncand > 1 else 0)
        advanced = eng.count_broken() - broken0  # bonds broken in the increment
        # this increment is the history of the next prediction, unless the crack
        # advanced in it (its departure is that jump, which the next increment does
        # not repeat) or it has no proportional reference (U = 0)
        recordable = U > 0.0 and advanced == 0
        if record:
            if recordable:
                record_history(eng, U, delta, u0, d0, host=collect is not None)
            else:
                clear_history(eng, delta)
        eng.sync()
        st["ms_total"] = (time.perf_counter() - t0) * 1e3
        st["start"] = "plain" if st["warm_used"] == 0 else offered[st["warm_used"] - 1]
        st["increment"] = k
        st["advanced"] = advanced
        u1 = torch.cat([ux, uy])
        prev = u1 - u0
        if collect is not None and U > 0.0 and advanced == 0:
            # target: the change of the departure from proportionality from the
            # recorded history (the network corrects the history term); increments
            # in which the crack advanced are left out (their jump is not
            # predictable from the state)
            tt = ((prev - u0 * (delta / U)) / U).cpu().numpy()
            dt = tt - hist if hist is not None else tt
            st["max_target"] = float(np.abs(dt).max())
            idx = np.sort(rng.choice(ni, max(1, int(keep * ni)), replace=False))
            t = np.stack([dt[idx], dt[ni + idx]], axis=1).astype(np.float32)
            ii = torch.from_numpy(idx).cuda()
            collect.append((X.index_select(0, ii).clone(), torch.from_numpy(t).cuda()))
        if last is not None:
            last.update(u0=u0.clone(), d0=d0.clone(), U=U if recordable else 0.0)
        out.append(st)
    return out


def record_history(eng, U_prev, delta, u_prev, dmg_prev, host=False):
    """pd_warm_record: the increment that led from (u_prev, dmg_prev) at
    accumulated boundary displacement U_prev to the context's current state
    (u_prev, dmg_prev: device tensors, or host arrays that are uploaded).
    host=True also keeps a host copy of the recorded departure on the engine
    (``warm_history``, for training targets)."""
    import torch

    up = u_prev if torch.is_tensor(u_prev) else torch.from_numpy(np.ascontiguousarray(u_prev, np.float64)).cuda()
    dp = dmg_prev if torch.is_tensor(dmg_prev) else \
        torch.from_numpy(np.ascontiguousarray(dmg_prev, np.float64)).cuda()
    check(lib().pd_warm_record(eng.ctx, U_prev, delta, up.data_ptr(), dp.data_ptr(), eng.stream), eng.ctx,
          "pd_warm_record")
    eng.has_history = True
    if host:
        eng.sync()
        ni = eng.p.N_int
        u = torch.cat([eng.device_view("UX", ni), eng.device_view("UY", ni)])
        eng.warm_history = (((u - up) - up * (delta / U_prev)) / U_prev).cpu().numpy()
    else:
        eng.warm_history = None


def clear_history(eng, delta):
    check(lib().pd_warm_record(eng.ctx, 0.0, delta, None, None, eng.stream), eng.ctx, "pd_warm_record")
    eng.has_history = False
    eng.warm_history = None


def restore_history(eng, meta, last):
    """The history of the increment described by ``last`` (run_increments),
    for a context whose state was just restored to the end of that increment
    (none when that increment recorded none)."""
    if last["U"] > 0.0:
        record_history(eng, last["U"], meta["delta"], last["u0"], last["d0"])
    else:
        clear_history(eng, meta["delta"])


def train(X, T, steps=3000, batch=16384, lr=2e-3, seed=0, log=None):
    """Adam on the mean squared error over (X, T) device tensors (BF16 [S][16],
    FP32 [S][2]); cosine learning-rate decay.  Returns the trained Net."""
    import torch

    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    net = Net(batch, init_params(seed))
    S = X.shape[0]
    for k in range(steps):
        idx = torch.randint(0, S, (batch,), device="cuda", generator=g)
        xb = X.index_select(0, idx).contiguous()
        tb = T.index_select(0, idx).contiguous()
        a = lr * 0.5 * (1.0 + math.cos(math.pi * k / steps))
        loss = net.train_step(xb.data_ptr(), tb.data_ptr(), batch, a)
        if log is not None and (k % 250 == 0 or k == steps - 1):
            log.append((k, loss))
    return net


# (scale, crack fraction, seed): 41k-104k-node plates of the same set-up,
# loaded through their first crack advances within 60 increments
TRAIN_RUNS = [
    (0.2, 0.15, 1), (0.2, 0.18, 2), (0.2, 0.25, 3), (0.25, 0.2, 4), (0.32, 0.2, 5),
]
# the network's outputs and history features are the departure per unit load
# times this factor (kHistScale of csrc/mlp.cu)
OUT_SCALE = 65536.0


def generate(runs=TRAIN_RUNS, n_inc=60, keep=0.25, tol=1e-8, log=print):
    """Converged states of seeded load-stepping runs -> (X, T) device tensors.
    Every increment starts from the previous solution (the plain method) and
    runs ADR to tol, through the crack's advances, so the targets are the
    plain method's converged increments: the change of the departure from
    proportionality from the recorded history (run_increments).  The features
    carry the history that pd_warm_record keeps."""
    import torch

    data = []
    for scale, frac, seed in runs:
        p, setup, meta = presets.build_warm_start_plate(scale=scale, crack_frac=frac)
        with Engine(p) as eng:
            setup(eng)
            t0 = time.perf_counter()
            n0 = len(data)
            st = run_increments(eng, meta, n_inc, mode="plain", collect=data, keep=keep, seed=seed, tol=tol)
            broken = int((eng.get("FAIL") == 0).sum())
        T = torch.cat([d[1] for d in data[n0:]])
        Xh = torch.cat([d[0][:, 5:7].float() for d in data[n0:]])
        log(json.dumps({"run": [scale, frac, seed], "nodes": p.N, "increments": n_inc,
                        "iters": int(sum(s["iters"] for s in st)), "max_iters": int(max(s["iters"] for s in st)),
                        "seconds": round(time.perf_counter() - t0, 1), "broken_bonds": broken,
                        "advances": [(s["increment"], s["iters"], s["advanced"]) for s in st if s["advanced"] > 0],
                        "target_std": float(T.std()) * OUT_SCALE, "history_std": float(Xh.std())}))
    X = torch.cat([d[0] for d in data])
    T = torch.cat([d[1] for d in data]) * OUT_SCALE
    return X, T


# (scale, crack fraction): plates the training runs do not include
EVAL_PLATES = [(0.2, 0.22), (0.28, 0.18)]


def evaluate(net, scale, frac, n_inc=50, smooths=(0, 16, 32), tol=1e-6):
    """Chained load increments on one plate, each start method on its own
    chain from rest: plain, the skip term alone, skip + history without the
    network (a zero output layer) and the learned start at each smoothing
    count.  Returns {method: per-increment ADR steps, candidates used, bonds
    broken, seconds}."""
    p, setup, meta = presets.build_warm_start_plate(scale=scale, crack_frac=frac)
    zero = Net(65536, init_params(0))
    runs = [("plain", "plain", 0, net), ("skip", "secant", 0, net), ("history", "learned", 0, zero)]
    runs += [("learned_s%d" % sm, "learned", sm, net) for sm in smooths]
    res = {}
    for name, mode, sm, nt in runs:
        with Engine(p) as eng:
            setup(eng)
            t0 = time.perf_counter()
            st = run_increments(eng, meta, n_inc, mode=mode, net=nt, smooth=sm, tol=tol)
        res[name] = {"seconds": round(time.perf_counter() - t0, 2), "iters": [s["iters"] for s in st],
                     "used": [s["start"] for s in st], "bonds_broken": [s["advanced"] for s in st],
                     "total_iters": int(sum(s["iters"] for s in st[1:]))}
    zero.close()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("cmd", choices=["train", "evaluate"])
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--increments", type=int, default=60)
    ap.add_argument("--tol", type=float, default=1e-8, help="ADR tolerance of the training runs")
    args = ap.parse_args()
    if args.cmd == "evaluate":
        # the shipped (or --out) weights against the skip term and the history
        # alone, 50 chained increments on each plate of EVAL_PLATES
        net = Net.load(args.out)
        for scale, frac in EVAL_PLATES:
            r = evaluate(net, scale, frac)
            print(json.dumps({"plate": [scale, frac], "results": r}), flush=True)
        return
    t0 = time.perf_counter()
    X, T = generate(n_inc=args.increments, tol=args.tol)
    print(json.dumps({"samples": int(X.shape[0]), "seconds": round(time.perf_counter() - t0, 1)}), flush=True)
    log = []
    net = train(X, T, steps=args.steps, log=log)
    net.save(args.out)
    print(json.dumps({"loss": log, "out": args.out}), flush=True)


if __name__ == "__main__":
    main()
