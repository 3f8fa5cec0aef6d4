"""Properties of the reference's algorithms that set how parity can be tested
(CPU only, on the oracle)."""
import numpy as np

import oracle as orc
from pd_gpu1_gb300 import presets


def test_adr_damping_is_chaotic():
    """The ADR damping coefficient (cal_cn, Integrate.cu:108-129) is a ratio of
    sums over force differences with a sign test, so last-bit changes grow:
    scaling u_y by 1 +- 1e-15 at step 5 changes cn by more than 1e-3 (relative)
    within 300 steps, while the first 10 steps stay at rounding level.  Any
    two implementations that round differently therefore agree tightly only
    over a short horizon."""
    p, _, meta = presets.build_plate_tensile(scale=0.3, derive=orc.derive_params)
    x, y = orc.plate_crack_coords(p)

    def run(eps):
        m = orc.Model(p, x, y)
        m.find_neighbor()
        m.surface_correct()
        cns = []
        for ct in range(300):
            m.quick_load(meta["load"])
            m.adr_step(ct)
            if ct == 5 and eps:
                sign = np.sign(np.sin(np.arange(p.N_int) + 0.5))
                m.uy[: p.N_int] = m.uy[: p.N_int] * (1 + eps * sign)
            cns.append(m.cn)
        return np.array(cns)

    a, b = run(0.0), run(1e-15)
    early = np.abs(a[6:11] - b[6:11]) / np.abs(a[6:11])
    assert early.max() < 1e-14
    late = np.abs(a[100:] - b[100:]) / np.maximum(np.abs(a[100:]), 1e-300)
    assert late.max() > 1e-3


def test_configured_time_step_is_unstable_on_the_fine_grid():
    """Crack-branching plate: the analytic explicit limit is 1.03e-8 s; at
    2.5e-8 s most bonds break within 2.5 us, at 1.0e-8 s almost none do."""
    p, _, meta = presets.build_crack_branching(scale=0.1, derive=orc.derive_params, dt=1.0e-8)
    assert abs(presets.critical_dt_2d(p) - 1.034e-8) < 1e-10

    def alive_after(dt):
        q = p.copy()
        q.dt = dt
        x, y = orc.plate_coords(q)
        m = orc.Model(q, x, y)
        m.find_neighbor()
        m.surface_correct()
        m.set_crack_2d(q.length / 2, -q.length / 4, 0.0, 0.0)
        m.by[:] = presets.traction_field(q, meta["sigma"])
        for _ in range(int(round(2.5e-6 / dt))):
            m.explicit_step()
        return m.rows(m.fail).mean()

    # the pre-crack alone cuts about 2.7 % of the bonds of this small plate
    assert alive_after(2.5e-8) < 0.5
    assert alive_after(1.0e-8) > 0.96
