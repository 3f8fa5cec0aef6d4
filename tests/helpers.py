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
