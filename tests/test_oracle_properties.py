"""Physical invariants of the bond-based (PMB) force that any faithful
implementation keeps (CPU only, on the oracle).  They complement the golden
vectors: the goldens pin the oracle to the reference's own outputs on a few
inputs; these hold on any input.

* Rigid translation: a uniform displacement field stretches no bond, so every
  force vanishes up to the rounding of x_c + u - x_i - u.
* Momentum: the pair forces are equal and opposite (the surface and volume
  corrections are symmetric in the two ends), so on a plate whose nodes all
  carry forces the volume-weighted sum of the force densities vanishes.
* Mirror symmetry: the crack-branching plate and its pre-crack are symmetric
  about y = 0, so a mirror-symmetric displacement field gives mirror-symmetric
  forces.
* Small strains: the force is linear in the displacement to first order in
  the strain.
The ordinary state-based force keeps the first two as well (a state-based
plate without boundary rows).
"""
import numpy as np
import pytest

import oracle as orc
from pd_gpu1_gb300 import presets


@pytest.fixture(scope="module")
def plate():
    """The crack-branching set-up at 5 % scale (100 x 40 nodes), pre-cracked."""
    p, _, meta = presets.build_crack_branching(scale=0.05, derive=orc.derive_params)
    x, y = orc.plate_coords(p)
    m = orc.Model(p, x, y)
    m.find_neighbor()
    m.surface_correct()
    m.set_crack_2d(p.length / 2.0, -p.length / 4.0, 0.0, 0.0)
    return p, x, y, m


def _forces(m, ux, uy):
    m.ux[:] = ux
    m.uy[:] = uy
    m.bond_force()
    return m.fx.copy(), m.fy.copy()


def _strain_field(x, y, eps=1e-4):
    """A smooth, non-uniform field with strains of order eps (below s0)."""
    return eps * (x + 20.0 * x * y), eps * (-0.3 * y + 10.0 * x * x)


def test_rigid_translation_gives_no_force(plate):
    p, x, y, m = plate
    fx0, fy0 = _forces(m, *_strain_field(x, y))
    scale = max(np.abs(fx0).max(), np.abs(fy0).max())
    fx, fy = _forces(m, np.full(p.N, 3.7e-6), np.full(p.N, -1.9e-6))
    assert max(np.abs(fx).max(), np.abs(fy).max()) < 1e-9 * scale


def test_pair_forces_conserve_momentum(plate):
    p, x, y, m = plate
    assert p.N == p.N_int  # every node carries a force (no boundary rows)
    fx, fy = _forces(m, *_strain_field(x, y))
    tot = np.abs(fx).sum() + np.abs(fy).sum()
    # rounding of 4,000 node sums that cancel leaves ~2e-12 of the total;
    # an asymmetric pair force would leave O(1)
    assert abs(fx.sum()) < 1e-10 * tot
    assert abs(fy.sum()) < 1e-10 * tot


def test_momentum_check_sees_one_asymmetric_pair():
    """Negative control, planted in the oracle: one directed bond's surface
    correction 1 % off breaks the balance far beyond the bar above."""
    p, _, _ = presets.build_crack_branching(scale=0.05, derive=orc.derive_params)
    x, y = orc.plate_coords(p)
    m = orc.Model(p, x, y)
    m.find_neighbor()
    m.surface_correct()
    i = p.N // 2 + 17
    m.scr[i * p.MN] *= 1.01  # the first bond of node i, in the i -> j direction only
    fx, fy = _forces(m, *_strain_field(x, y))
    tot = np.abs(fx).sum() + np.abs(fy).sum()
    assert max(abs(fx.sum()), abs(fy.sum())) > 1e-6 * tot


def test_mirror_symmetry_about_the_crack_line(plate):
    p, x, y, m = plate
    # the node at (x, -y) for every node (x, y): the lattice (coordinates at
    # half-integer multiples of dx) is symmetric
    def k(a, b):
        return int(np.floor(2.0 * a / p.dx + 0.5)), int(np.floor(2.0 * b / p.dx + 0.5))

    key = {k(a, b): i for i, (a, b) in enumerate(zip(x, y))}
    mirror = np.array([key[k(a, -b)] for a, b in zip(x, y)])
    assert len(set(mirror.tolist())) == p.N
    ux, uy = _strain_field(x, y)
    ux = 0.5 * (ux + ux[mirror])  # ux even in y, uy odd
    uy = 0.5 * (uy - uy[mirror])
    fx, fy = _forces(m, ux, uy)
    scale = max(np.abs(fx).max(), np.abs(fy).max())
    assert np.abs(fx - fx[mirror]).max() < 1e-12 * scale
    assert np.abs(fy + fy[mirror]).max() < 1e-12 * scale


def test_force_is_linear_at_small_strains(plate):
    p, x, y, m = plate
    ux, uy = _strain_field(x, y, eps=1e-6)
    fx1, fy1 = _forces(m, ux, uy)
    fx2, fy2 = _forces(m, 2.0 * ux, 2.0 * uy)
    scale = max(np.abs(fx2).max(), np.abs(fy2).max())
    # geometric nonlinearity: relative size ~ strain (1e-6)
    assert np.abs(fx2 - 2.0 * fx1).max() < 1e-4 * scale
    assert np.abs(fy2 - 2.0 * fy1).max() < 1e-4 * scale


@pytest.fixture(scope="module")
def state_plate():
    """An ordinary state-based plate (80 x 60 nodes, dx = 1e-4, the crack-grow
    material) whose nodes all carry forces: no boundary rows."""
    p = orc.derive_params(2, 2, 2, 1.3367e-8, 10, 1e-4, 1.0, 1e-4, 0.008, 0.006, 0.0, 192e9, 0.3, 7850.0, 0.04472)
    x, y = orc.plate_coords(p)
    m = orc.Model(p, x, y)
    m.find_neighbor()
    m.vol_corr()
    m.initial_weight()
    return p, x, y, m


def _state_forces(m, ux, uy):
    m.ux[:] = ux
    m.uy[:] = uy
    m.state_force()
    return m.fx.copy(), m.fy.copy()


def test_state_based_rigid_translation_gives_no_force(state_plate):
    p, x, y, m = state_plate
    fx0, fy0 = _state_forces(m, *_strain_field(x, y))
    scale = max(np.abs(fx0).max(), np.abs(fy0).max())
    fx, fy = _state_forces(m, np.full(p.N, 3.7e-6), np.full(p.N, -1.9e-6))
    assert max(np.abs(fx).max(), np.abs(fy).max()) < 1e-9 * scale
    assert np.abs(m.theta).max() < 1e-9  # no dilatation either


def test_state_based_pair_forces_conserve_momentum(state_plate):
    """t_i + t_j is symmetric in the two ends and the bond direction is not,
    so the state-based pair forces balance as the bond-based ones do."""
    p, x, y, m = state_plate
    assert p.N == p.N_int
    fx, fy = _state_forces(m, *_strain_field(x, y))
    tot = np.abs(fx).sum() + np.abs(fy).sum()
    assert abs(fx.sum()) < 1e-10 * tot
    assert abs(fy.sum()) < 1e-10 * tot
