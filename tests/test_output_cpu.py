"""CPU checks of the text writers (host-only entry points of the C ABI):
save_disp's line format (Save.cu:27-34) and save_kw's grid order with the
notch cells (Save.cu:77-101), against a direct Python restatement of the
reference's iostream output (default formatting = %g, 6 digits)."""
import ctypes as C
import math

import numpy as np

from pd_gpu1_gb300._lib import lib


def _p(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data


def g(v):
    return "%g" % v


def test_disp_txt_2d_and_3d(tmp_path):
    rng = np.random.default_rng(1)
    n = 57
    ux, uy, uz = (rng.standard_normal(n) * 10.0 ** rng.integers(-12, 3, n) for _ in range(3))
    dmg = rng.uniform(0, 1, n)
    dmg[:3] = [0.0, 1.0, -0.0]
    keep = [ux, uy, uz, dmg]
    f2 = tmp_path / "d2.txt"
    assert lib().pd_write_disp_txt(str(f2).encode(), n, _p(ux), _p(uy), None, _p(dmg)) == 0
    want = "".join(f"{g(a)} {g(b)} {g(d)}\n" for a, b, d in zip(ux, uy, dmg))
    assert f2.read_text() == want
    f3 = tmp_path / "d3.txt"
    assert lib().pd_write_disp_txt(str(f3).encode(), n, _p(ux), _p(uy), _p(uz), _p(dmg)) == 0
    want = "".join(f"{g(a)} {g(b)} {g(c)} {g(d)}\n" for a, b, c, d in zip(ux, uy, uz, dmg))
    assert f3.read_text() == want
    del keep


def test_kw_txt_notch_rows(tmp_path):
    from pd_gpu1_gb300 import presets
    import oracle as orc

    p, setup, meta = presets.build_kalthoff_winkler(scale=0.25, derive=orc.derive_params, coord_fn=orc.coord_kw)
    x, y, z = meta["coords"]
    rad = meta["rad"]
    n = len(x)
    vals = [np.arange(n) * 1.0, -np.arange(n) * 1.0, np.arange(n) * 0.5, np.linspace(0, 1, n)]
    f = tmp_path / "kw.txt"
    assert lib().pd_write_kw_txt(str(f).encode(), C.byref(p), rad, n, *[_p(v) for v in vals]) == 0
    lines = f.read_text().splitlines()
    assert len(lines) == p.nx * p.ny
    num = 0
    for j in range(p.ny):
        for i in range(p.nx):
            tx = (-(p.nx - 1) / 2.0 + i) * p.dx
            ty = (-(p.ny - 1) / 2.0 + j) * p.dx
            notch = (-rad - 1.1 * p.dx < tx < -rad + 0.1 * p.dx) or (rad - 0.1 * p.dx < tx < rad + 1.1 * p.dx)
            line = lines[j * p.nx + i]
            if notch and ty >= -1e-10:
                assert line == "nan nan 0 nan"
            else:
                assert line == " ".join(g(v[num]) for v in vals)
                # the node written is the first z layer's node at (tx, ty)
                assert math.isclose(x[num], tx, abs_tol=1e-12) and math.isclose(y[num], ty, abs_tol=1e-12)
                num += 1


def test_writer_rejects_bad_path():
    z = np.zeros(3)
    assert lib().pd_write_disp_txt(b"/nonexistent-dir/x.txt", 3, _p(z), _p(z), None, _p(z)) != 0
