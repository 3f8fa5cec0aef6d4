"""The extended-precision yardstick of the per-node force checks.

helpers.exact_bond_forces_2d evaluates the reference's 2-D bond-force formula
beyond FP64 from the reference's own FP64 bond vector.  Checked here against
the oracle (the formula in FP64) on a 16,000-node piece of the crack-branching
plate under the compressive field of the full-size GPU test: norm-relative
they agree to 1e-12, while node by node, on the nodes carrying at least 1e-3
of the largest force, the FP64 evaluation is up to ~6e-11 off.  That is the
reference formula's own rounding (its stretch (|xi + eta| - |xi|) / |xi|
cancels), and the reason the GPU per-node checks measure both
implementations against this yardstick instead of against each other."""
import numpy as np

import oracle as orc
from helpers import exact_bond_forces_2d, per_node_errors, significant_nodes
from pd_gpu1_gb300 import presets


def test_yardstick_against_fp64_formula():
    p, setup, meta = presets.build_crack_branching(scale=0.1, derive=orc.derive_params)
    x, y = orc.plate_coords(p)
    m = orc.Model(p, x, y)
    m.find_neighbor()
    m.surface_correct()
    m.set_crack_2d(p.length / 2.0, -p.length / 4.0, 0.0, 0.0)
    ux = -4.0e-4 * x + 1.0e-3 * x * y
    uy = -4.0e-4 * y + 5.0e-4 * x * x
    m.ux[:], m.uy[:] = ux, uy
    fail0 = m.rows(m.fail).copy()
    m.bond_force()
    N = p.N_int
    allnodes = np.arange(N)
    ex, ey = exact_bond_forces_2d(x, y, ux, uy, m.rowptr(), m.rows(m.NL), m.rows(m.idist), m.rows(m.fac),
                                  m.rows(m.scr), fail0, p.vol, p.bc, allnodes)
    scale = float(np.abs(np.concatenate([ex, ey])).max())
    norm_rel = max(np.abs(m.fx[:N] - ex).max(), np.abs(m.fy[:N] - ey).max()) / scale
    assert norm_rel < 1e-12
    sel = significant_nodes(m.fx[:N], m.fy[:N], 1e-3)
    e = per_node_errors(m.fx[sel], m.fy[sel], ex[sel], ey[sel])
    assert 1e-11 < e.max() < 1e-9  # the FP64 formula's own per-node error
    assert np.median(e) < 1e-12
