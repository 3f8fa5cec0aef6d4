"""CPU checks of the C ABI: the library loads without a GPU, exports every
entry point include/pd.h declares, and its host-only entry points (parameter
derivation, notched-slab coordinates) agree bit for bit with the oracle and
the reference's derivation recorded in the golden fixtures."""
import ctypes as C
import math
import os
import re

import numpy as np

import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "pd.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pd_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from pd_gpu1_gb300._lib import LIB_PATH, exported_symbols

    assert os.path.exists(LIB_PATH), "build the library first (__graft_entry__.build())"
    handle = C.CDLL(LIB_PATH)
    decl = declared_symbols()
    assert len(decl) > 40
    missing = [s for s in decl if not hasattr(handle, s)]
    assert not missing, missing
    # the Python binding covers the same set
    assert sorted(exported_symbols()) == decl


def test_status_strings():
    from pd_gpu1_gb300._lib import lib

    L = lib()
    for code, name in [(0, b"PD_OK"), (-1, b"PD_ERR_ARG"), (-4, b"PD_ERR_FAMILY"), (-5, b"PD_ERR_NONFINITE")]:
        assert L.pd_status_string(code) == name


def test_param_derivation_matches_oracle_and_reference(golden):
    from pd_gpu1_gb300.engine import derive_params

    cases = [
        (2, 1, 1, 1.0, 1000, 0.01, 1.0, 0.01, 1.0, 0.5, 0.0, 200e9, 1 / 3, 7850, 1.0, 0),
        (2, 2, 2, 1.3367e-8, 1250, 1e-4, 1.0, 1e-4, 0.05, 0.05, 0.0, 192e9, 0.3, 7850, 0.04472, 0),
        (3, 1, 2, 8.7e-8, 0, 1e-3, 1.0, 1e-3, 0.2, 0.1, 0.009, 191e9, 0.25, 8000, 0.01, 0),
        (3, 2, 2, 1e-7, 1350, 1e-3, 1.0, 1e-3, 0.2, 0.1, 0.009, 190e9, 0.25, 8000, 0.01, 1),
        (2, 1, 2, 2.5e-8, 1800, 5e-5, 0.0, 5e-5, 0.1, 0.04, 0.0, 72e9, 1 / 3, 2440, 7e-4, 0),
    ]
    for c in cases:
        a = derive_params(*c)
        b = orc.derive_params(*c)
        for name, _ in a._fields_:
            assert getattr(a, name) == getattr(b, name), (c, name)
    g = golden("plate_tensile_bond")
    a = derive_params(2, 1, 1, 1.0, 1000, 0.01, 1.0, 0.01, 0.2, 0.1, 0.0, 200e9, 1 / 3, 7850, 1.0)
    for k in ["bc", "delta", "vol", "mass"]:
        assert getattr(a, k) == float(g["p_" + k]), k


def test_coord_kw_matches_oracle_and_reference(golden):
    from pd_gpu1_gb300.engine import coord_kw, derive_params

    g = golden("kalthoff_winkler_bond")
    p = derive_params(3, 1, 2, 8.7e-8, 0, 0.003, 1.0, 0.003, 0.06, 0.1, 0.009, 191e9, 0.25, 8000, 0.01)
    p.nx += 1
    p.ny += 1
    p.N = p.nx * p.ny * p.nz
    x, y, z = coord_kw(p, float(g["rad"]))
    np.testing.assert_array_equal(x, g["x"])
    np.testing.assert_array_equal(y, g["y"])
    np.testing.assert_array_equal(z, g["z"])
    xo, yo, zo = orc.coord_kw(p, float(g["rad"]))
    np.testing.assert_array_equal(x, xo)


def test_full_size_kalthoff_winkler_node_count():
    """coord_KW at the reference's own size gives 180,873 nodes."""
    from pd_gpu1_gb300.engine import coord_kw, derive_params

    p = derive_params(3, 1, 2, 8.7e-8, 0, 1e-3, 1.0, 1e-3, 0.2, 0.1, 0.009, 191e9, 0.25, 8000, 0.01)
    p.nx += 1
    p.ny += 1
    x, _, _ = coord_kw(p, 0.025)
    assert len(x) == 180873


def _header_fields(struct):
    txt = open(os.path.join(ROOT, "include", "pd.h")).read()
    body = txt[txt.index(f"typedef struct {struct} {{"): txt.index(f"}} {struct};")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = []
    for decl in re.findall(r"(?:double|int32_t)\s+([^;]+);", body):
        names += [n.strip() for n in decl.split(",")]
    return names


def test_abi_struct_layout_matches_header():
    """The ctypes mirrors of pd_params and pd_specimen have the C layout
    (field order; all members naturally aligned, no padding)."""
    from pd_gpu1_gb300._abi import PDParams, PDSpecimen

    assert _header_fields("pd_params") == [f for f, _ in PDParams._fields_]
    assert C.sizeof(PDParams) % 8 == 0
    assert _header_fields("pd_specimen") == [f for f, _ in PDSpecimen._fields_]
    assert C.sizeof(PDSpecimen) == 2 * 4 + 5 * 8


def test_batch_specimen_table_is_seeded():
    """The batch workload: 256 seeded specimens of about 6.25M interior nodes,
    s0 from G0 by the 2-D closed form, cracks within 30 % of the width."""
    from pd_gpu1_gb300 import presets

    a = presets.batch_specimens()
    b = presets.batch_specimens()
    assert a == b and len(a) == 256
    n = sum(s["nx"] * s["ny"] for s in a)
    assert 5.5e6 < n < 7.0e6
    for s in a:
        assert 50 <= s["nx"] <= 300 and s["nx"] == s["ny"]
        assert 70e9 <= s["emod"] <= 210e9 and 2400 <= s["dens"] <= 8000
        assert s["critical_s"] == presets.s0_2d(s["G0"], s["emod"], 3.015 * 5e-4)
        assert 0.0 <= s["crack_len"] <= 0.3 * s["nx"] * 5e-4 and 0.0 <= s["crack_theta"] < math.pi / 2


def test_header_serves_a_plain_c_caller(tmp_path):
    """include/pd.h compiles as pedantic C99 (a foreign-function caller binds
    it as C), links against libpd_gb300.so, and its host-only entry points
    run without a GPU: the parameter derivation of the crack-branching plate
    at 5 % scale agrees with the oracle's."""
    import shutil
    import subprocess

    from pd_gpu1_gb300._lib import LIB_PATH

    gcc = shutil.which("gcc")
    if gcc is None:
        import pytest

        pytest.skip("no C compiler")
    src = tmp_path / "caller.c"
    src.write_text(
        '#include "pd.h"\n#include <stdio.h>\n'
        "int main(void) {\n"
        "    pd_params p;\n"
        "    int st = pd_params_derive(&p, 2, PD_MODEL_BOND, PD_MODE_DYNAMIC, 1e-8, 10, 5e-5, 0.0, 5e-5,\n"
        "                              0.005, 0.002, 0.0, 72e9, 1.0 / 3.0, 2440.0, 7e-4, 0);\n"
        '    printf("%s %lld %.17g %.17g\\n", pd_status_string(st), (long long)p.N, p.bc, p.mass);\n'
        "    return st;\n"
        "}\n")
    exe = tmp_path / "caller"
    libdir = os.path.dirname(LIB_PATH)
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                    os.path.join(ROOT, "include"), str(src), "-L", libdir, "-lpd_gb300",
                    "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    q = orc.derive_params(2, 1, 2, 1e-8, 10, 5e-5, 0.0, 5e-5, 0.005, 0.002, 0.0, 72e9, 1 / 3, 2440.0, 7e-4)
    assert out[0] == "PD_OK" and int(out[1]) == q.N
    assert float(out[2]) == q.bc and float(out[3]) == q.mass
