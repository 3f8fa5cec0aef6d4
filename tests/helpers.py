"""Shared test helpers: build parameter blocks and oracle models from golden fixtures,
and the norm-relative comparison used for floating-point parity."""
import numpy as np

import oracle as orc
from pd_gpu1_gb300._abi import PDParams

DKEYS = ["pi", "dx", "emod", "dens", "pratio", "bc", "delta", "critical_s", "vol", "dt", "mass", "K", "G",
         "thick", "sedload"]
IKEYS = ["N", "MN", "N_int", "nx", "ny", "nz", "nt"]


def params_from_golden(g, prefix=""):
    """Parameter block exactly as the reference derived it (stored in the fixture)."""
    dim = int(g[prefix + "in_dim"])
    bs = int(g[prefix + "in_bs"])
    mode = int(g[prefix + "in_mode"])
    p = orc.derive_params(dim, bs, mode, float(g[prefix + "in_dt"]), float(g[prefix + "in_nt"]),
                          float(g[prefix + "in_dx"]), float(g[prefix + "in_load"]), float(g[prefix + "in_thick"]),
                          float(g[prefix + "in_length"]), float(g[prefix + "in_height"]),
                          float(g[prefix + "in_width"]), float(g[prefix + "in_emod"]), float(g[prefix + "in_pratio"]),
                          float(g[prefix + "in_dens"]), float(g[prefix + "in_s0"]))
    for k in IKEYS:
        if k == "nt":
            continue
        setattr(p, k, int(g[prefix + "p_" + k]))
    for k in DKEYS:
        if k in ("thick", "sedload"):
            continue
        setattr(p, k, float(g[prefix + "p_" + k]))
    return p


def ell(values, NN, MN, fill=0):
    """Scatter CSR-ordered bond values into the reference's padded N*MN layout."""
    N = len(NN)
    out = np.full(N * MN, fill, dtype=values.dtype)
    mask = (np.arange(MN)[None, :] < NN[:, None]).reshape(-1)
    out[mask] = values
    return out


def model_from_golden(g, with_family=True):
    p = params_from_golden(g)
    m = orc.Model(p, g["x"], g["y"], g.get("z"))
    if with_family:
        m.NN[:] = g["NN"]
        m.NL[:] = ell(g["NL"].astype(np.int32), g["NN"], p.MN)
        m.idist[:] = ell(g["idist"], g["NN"], p.MN)
        m.fac[:] = ell(g["fac"], g["NN"], p.MN)
        if "scr" in g:
            m.scr[:] = ell(g["scr"], g["NN"], p.MN)
    return m


def assert_close_norm(actual, expected, rtol, what=""):
    """|a - e| <= rtol * max|e| elementwise (norm-relative: interior peridynamic
    forces are sums that cancel to near zero, so a per-element relative test
    would measure rounding noise, not disagreement)."""
    actual = np.asarray(actual, dtype=np.float64)
    expected = np.asarray(expected, dtype=np.float64)
    assert actual.shape == expected.shape, (what, actual.shape, expected.shape)
    scale = float(np.max(np.abs(expected))) if expected.size else 0.0
    err = float(np.max(np.abs(actual - expected))) if expected.size else 0.0
    assert err <= rtol * scale + 1e-300, f"{what}: max err {err:.3e} > {rtol:.1e} * {scale:.3e}"
    return err / scale if scale else 0.0


def exact_bond_forces_2d(x, y, ux, uy, rowptr, NL, idist, fac, scr, fail, vol, bc, nodes):
    """Node forces of the 2-D PMB kernels (Force_Bond.cu:52-85) on the given
    nodes, evaluated in extended precision (numpy longdouble: 64 or 113
    significant bits) from the reference's own FP64 bond vector
    d = ((x_c + u_c) - x_i) - u_i, which both implementations form with the
    same roundings.  Everything after d (length, stretch, force) is carried
    beyond FP64, so the result stands for the exact value of the reference's
    formula: the yardstick that separates an implementation's error from the
    reference's own FP64 rounding."""
    ld = np.longdouble
    nodes = np.asarray(nodes, dtype=np.int64)
    rp = np.asarray(rowptr, dtype=np.int64)
    cnt = rp[nodes + 1] - rp[nodes]
    own = np.repeat(np.arange(len(nodes)), cnt)
    idx = np.concatenate([np.arange(rp[n], rp[n + 1]) for n in nodes]) if len(nodes) else np.zeros(0, np.int64)
    i = nodes[own]
    c = np.asarray(NL, dtype=np.int64)[idx]
    alive = np.asarray(fail)[idx] == 1
    dx = ((x[c] + ux[c]) - x[i]) - ux[i]
    dy = ((y[c] + uy[c]) - y[i]) - uy[i]
    dxl, dyl = dx.astype(ld), dy.astype(ld)
    L = np.sqrt(dxl * dxl + dyl * dyl)
    l0 = np.asarray(idist)[idx].astype(ld)
    k = ld(vol) * np.asarray(fac)[idx].astype(ld) * ld(bc) * np.asarray(scr)[idx].astype(ld) * ((L - l0) / l0) / L
    k = np.where(alive, k, ld(0))
    fx = np.zeros(len(nodes), dtype=ld)
    fy = np.zeros(len(nodes), dtype=ld)
    np.add.at(fx, own, k * dxl)
    np.add.at(fy, own, k * dyl)
    return fx, fy


def per_node_errors(fx, fy, fx_ref, fy_ref):
    """Per-node relative difference |f - f_ref| / |f_ref| of 2-D force vectors."""
    fx_ref = np.asarray(fx_ref, dtype=np.float64)
    fy_ref = np.asarray(fy_ref, dtype=np.float64)
    mag = np.hypot(fx_ref, fy_ref)
    d = np.hypot(np.asarray(fx, dtype=np.float64) - fx_ref, np.asarray(fy, dtype=np.float64) - fy_ref)
    return d / np.maximum(mag, 1e-300)


def significant_nodes(fx, fy, frac=1e-3, cap=None, seed=0):
    """Nodes whose force magnitude is at least frac of the largest (edge rows,
    crack faces, the stretched field), optionally a seeded sample of cap of
    them that always keeps the 1,000 largest."""
    mag = np.hypot(fx, fy)
    sel = np.nonzero(mag >= frac * mag.max())[0]
    if cap is not None and len(sel) > cap:
        top = sel[np.argsort(mag[sel])[-1000:]]
        rest = np.setdiff1d(sel, top)
        rng = np.random.default_rng(seed)
        sel = np.union1d(top, rng.choice(rest, cap - len(top), replace=False))
    return sel


def check_per_node_2d(eng, fx, fy, ref_fx, ref_fy, ux, uy, fail, nodes_limit=None, bars=((1e-3, 1e-11), (1e-2, 1e-12)),
                      what=""):
    """Per-node relative force check of a 2-D bond-based evaluation.

    The engine's forces (``fx``, ``fy``, from the context ``eng`` whose family
    and coefficients they used, with the CSR intact flags ``fail`` the pass
    started from) and the reference's (``ref_fx``, ``ref_fy``) are each
    compared, node by node, with the extended-precision value of the
    reference's formula (exact_bond_forces_2d) on the nodes whose force is at
    least a fraction of the largest (a seeded sample of ``nodes_limit`` of
    them when given).  ``bars``: (fraction, bound) pairs; on the nodes above
    each fraction the engine must lie within the bound of that value.  The
    reference's own distance from it, and the engine-reference difference,
    are reported beside (the reference forms the stretch
    (|xi + eta| - |xi|) / |xi| in FP64, which cancels, and its node forces lie
    up to ~1e-10 off where bond forces cancel).  Returns the report."""
    p = eng.params()
    N = p.N_int
    fx, fy = np.asarray(fx)[:N], np.asarray(fy)[:N]
    ref_fx, ref_fy = np.asarray(ref_fx)[:N], np.asarray(ref_fy)[:N]
    lo = min(f for f, _ in bars)
    sel = significant_nodes(ref_fx, ref_fy, lo, cap=nodes_limit)
    ex, ey = exact_bond_forces_2d(eng.get("X"), eng.get("Y"), ux, uy, eng.get("ROWPTR"), eng.get("NL"),
                                  eng.get("IDIST"), eng.get("FAC"), eng.get("SCR"), fail, p.vol, p.bc, sel)
    e_eng = per_node_errors(fx[sel], fy[sel], ex, ey)
    e_ref = per_node_errors(ref_fx[sel], ref_fy[sel], ex, ey)
    e_er = per_node_errors(fx[sel], fy[sel], ref_fx[sel], ref_fy[sel])
    mag = np.hypot(ref_fx[sel], ref_fy[sel])
    top = float(np.hypot(ref_fx, ref_fy).max())
    rep = {"what": what, "nodes": int(len(sel))}
    ok = True
    for frac, bound in bars:
        m = mag >= frac * top
        w = int(np.argmax(np.where(m, e_eng, -1.0)))
        r = {"nodes": int(m.sum()), "bound": bound,
             "engine_vs_exact": {"max": float(e_eng[m].max()), "p99": float(np.quantile(e_eng[m], 0.99)),
                                 "worst_node": int(sel[w]), "worst_node_force_over_max": float(mag[w] / top)},
             "reference_vs_exact": {"max": float(e_ref[m].max()), "p99": float(np.quantile(e_ref[m], 0.99))},
             "engine_vs_reference": {"max": float(e_er[m].max()), "p99": float(np.quantile(e_er[m], 0.99))}}
        rep[f"force_ge_{frac:g}_of_max"] = r
        ok = ok and e_eng[m].max() <= bound
    assert ok, (what, rep)
    return rep
