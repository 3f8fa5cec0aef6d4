"""Named workloads: the benchmark configurations as engine set-ups.

Each ``build_*`` function returns ``(params, setup)`` where ``setup(engine)``
performs the set-up sequence of the matching reference driver on an
:class:`~pd_gpu1_gb300.engine.Engine` created from ``params``.  ``scale``
shrinks the plate (same dx) for quick tests.

Critical stretch from fracture energy G0 (the reference has no such formula,
so one published closed form is fixed here and used on every side):
  2-D bond-based, plane stress (Ha & Bobaru 2010):  s0 = sqrt(4 pi G0 / (9 E delta))
  3-D (Silling & Askari 2005):                      s0 = sqrt(5 G0 / (9 K delta)), K = E / (3 (1 - 2 nu))
"""
import math

import numpy as np

from ._abi import PD_MODE_DYNAMIC, PD_MODE_STATIC, PD_MODEL_BOND, PD_MODEL_STATE, PDCylinder


def _derive(derive):
    if derive is not None:
        return derive
    from .engine import derive_params

    return derive_params


def _coord_kw(fn):
    if fn is not None:
        return fn
    from .engine import coord_kw

    return coord_kw


def s0_2d(G0, E, delta):
    return math.sqrt(4.0 * math.pi * G0 / (9.0 * E * delta))


def s0_3d(G0, E, nu, delta):
    K = E / (3.0 * (1.0 - 2.0 * nu))
    return math.sqrt(5.0 * G0 / (9.0 * K * delta))


# ---- plate tensile, 2-D PMB, ADR (1000 steps) ---------------------------------------
def build_plate_tensile(scale=1.0, dx=5e-4, nt=1000, derive=None):
    """0.05 x 0.05 m plate, dx = 5e-4 (100 x 100 nodes) plus 3 boundary rows above
    and below (the crack-plate layout, Coord.cu:34-45), E = 192 GPa, nu = 1/3,
    rho = 8000, s0 = 0.04472, thickness dx, surface correction on, ADR with
    dt = 1; the boundary rows move +-2.7e-8 m per step."""
    L = 0.05 * scale
    p = _derive(derive)(2, PD_MODEL_BOND, PD_MODE_STATIC, 1.0, nt, dx, 0.0, dx, L, L, 0.0, 192.0e9, 1.0 / 3.0, 8000.0,
                      0.04472)
    p.N = p.N_int + 6 * p.nx
    load = 2.7e-8 / p.dt  # kernel_quick_load moves rows by load*dt per step

    def setup(eng):
        eng.coord_plate_crack()
        eng.find_neighbor_gpu()
        eng.surface_correct_gpu()
        eng.initial_state()
        eng.prepare()

    return p, setup, dict(load=load, nt=nt, workload="plate_tensile_2d_pmb_adr")


# ---- dynamic crack branching, 2-D PMB, Verlet (1800 steps, headline) ------------------
def critical_dt_2d(p):
    """Explicit stability limit of 2-D PMB on a regular lattice with horizon
    3.015 dx: dt_c = sqrt(2 rho / sum_j V_j c / |xi_j|) (Silling & Askari 2005),
    the sum running over the 28 interior family members."""
    dists = [1.0] * 4 + [math.sqrt(2.0)] * 4 + [2.0] * 4 + [math.sqrt(5.0)] * 8 + [math.sqrt(8.0)] * 4 + [3.0] * 4
    return math.sqrt(2.0 * p.dens / sum(p.vol * p.bc / (r * p.dx) for r in dists))


def build_crack_branching(scale=1.0, dx=5e-5, nt=1800, derive=None, dt=1.0e-8):
    """0.1 x 0.04 m glass plate, dx = 5e-5 (2000 x 800 = 1.6M nodes),
    E = 72 GPa, nu = 1/3, rho = 2440, G0 = 3.8 J/m^2, pre-crack 0.05 m along
    the mid-line from the left edge, 12 MPa traction on the top and bottom rows
    as body force sigma/dx, damage every 100 steps.

    Time step: 2.5e-8 s is the usual step of this benchmark on a grid four to
    five times coarser; on this grid the explicit limit is 1.03e-8 s
    (critical_dt_2d) and at 2.5e-8 s the plate shatters numerically within 50
    steps (83 % of bonds broken), after which both implementations skip most
    bonds.  The default is therefore 1.0e-8 s, so that every step does the full
    bond work; pass dt=2.5e-8 to run the unstable setting."""
    Lx, Ly = 0.1 * scale, 0.04 * scale
    E, nu, rho, G0 = 72.0e9, 1.0 / 3.0, 2440.0, 3.8
    delta = 3.015 * dx
    s0 = s0_2d(G0, E, delta)
    p = _derive(derive)(2, PD_MODEL_BOND, PD_MODE_DYNAMIC, dt, nt, dx, 0.0, dx, Lx, Ly, 0.0, E, nu, rho, s0)
    sigma = 12.0e6

    def setup(eng):
        eng.coord_plate()
        eng.find_neighbor_gpu()
        eng.surface_correct_gpu()
        eng.initial_state()
        # pre-crack: half the plate length, from the left edge along y = 0
        eng.set_crack_2d(Lx / 2.0, -Lx / 4.0, 0.0, 0.0)
        eng.set("BY", traction_field(p, sigma))
        eng.prepare()

    return p, setup, dict(load=0.0, nt=nt, dmg_every=100, workload="crack_branching_2d_pmb_verlet", s0=s0,
                          sigma=sigma)


def traction_field(p, sigma):
    """Body force sigma/dx on the top row (+y) and bottom row (-y) of a plate
    laid out row by row, as load_plate_tensile applies its edge load
    (Solve_Plate_Tensile.cu:12)."""
    by = np.zeros(p.N)
    by[(p.ny - 1) * p.nx: p.ny * p.nx] = sigma / p.dx
    by[0: p.nx] = -sigma / p.dx
    return by


# ---- Kalthoff-Winkler impact, 3-D state-based, Verlet (1350 steps) -------------------
def build_kalthoff_winkler(scale=1.0, dx=1e-3, nt=1350, model=PD_MODEL_STATE, derive=None, coord_fn=None):
    """Notched slab of coord_KW (Coord.cu:77-129): 0.2 x 0.1 x 0.009 m, dx = 1e-3
    (201 x 101 x 9 grid points minus the two notch strips at x = +-0.025 in the
    upper half), E = 190 GPa, nu = 0.25, rho = 8000, G0 = 22170 J/m^2, rigid
    cylindrical impactor (mass 1.57 kg, radius 0.025 m, height 0.05 m) at 32 m/s,
    dt = 1e-7.  Bulk modulus K = E / (3 (1 - 2 nu)) (the reference's 3-D
    formula at Base.cuh:175 divides by (1 - 2G) instead)."""
    L, H, W = 0.2 * scale, 0.1 * scale, 0.009
    E, nu, rho, G0 = 190.0e9, 0.25, 8000.0, 22170.0
    delta = 3.015 * dx
    s0 = s0_3d(G0, E, nu, delta)
    p = _derive(derive)(3, model, PD_MODE_DYNAMIC, 1.0e-7, nt, dx, 1.0, dx, L, H, W, E, nu, rho, s0, fix_k3d=1)
    p.nx += 1
    p.ny += 1
    rad = 0.025 * scale
    x, y, z = _coord_kw(coord_fn)(p, rad)
    p.N = p.N_int = len(x)
    cyl = PDCylinder()
    cyl.rad, cyl.mass, cyl.height, cyl.v = rad, 1.57, 0.05 * scale, -32.0
    cyl.x, cyl.y, cyl.z = 0.0, H / 2.0 + cyl.height / 2.0 + 0.1 * dx, 0.0
    cyl.vel[1] = cyl.v

    def setup(eng):
        eng.set_coords(x, y, z)
        eng.find_neighbor_gpu()
        if model == PD_MODEL_BOND:
            eng.surface_correct_gpu()
        else:
            eng.initial_weight()  # vol_Corr's idist and fac in the same family pass
        eng.initial_state()
        eng.set_crack_kw(rad)
        eng.cylinder_init(cyl)
        eng.prepare()

    name = "kalthoff_winkler_3d_pmb_verlet" if model == PD_MODEL_BOND else "kalthoff_winkler_3d_state_verlet"
    return p, setup, dict(load=0.0, nt=nt, workload=name, cylinder=cyl, s0=s0, rad=rad, coords=(x, y, z))


# ---- crack growth, 2-D state-based, Verlet (the reference crack-grow driver) ---------
def build_crack_grow(scale=1.0, dx=1e-4, nt=1250, derive=None):
    """Solve_Plate_Crack_Grow.cu:177-179: 0.05 x 0.05 m plate, dx = 1e-4,
    state-based, E = 192 GPa, nu = 0.3, rho = 7850, s0 = 0.04472, boundary rows
    moving +-20*dt per step, centre crack 0.01 m."""
    L = 0.05 * scale
    p = _derive(derive)(2, PD_MODEL_STATE, PD_MODE_DYNAMIC, 1.3367e-8, nt, dx, 1.0, dx, L, L, 0.0, 192.0e9, 0.3, 7850.0,
                      0.04472)
    p.N = p.N_int + 6 * p.nx

    def setup(eng):
        eng.coord_plate_crack()
        eng.find_neighbor_gpu()
        eng.initial_state()
        eng.set_crack_2d(0.01 * scale, 0.0, 0.0, 0.0)
        eng.initial_weight()  # vol_Corr's idist and fac in the same family pass
        eng.prepare()

    return p, setup, dict(load=20.0, nt=nt, workload="plate_crack_grow_2d_state_verlet")


# ---- batch of uneven plates, 2-D PMB, ADR (256 specimens x 1000 steps) -------------
def batch_specimens(count=256, seed=20240607, dx=5e-4, side=(50, 300), max_nodes=None):
    """Seeded specimen table: side ~ log-uniform[50, 300] nodes (square
    plates), E ~ U[70, 210] GPa, rho ~ U[2400, 8000] (drawn for the record;
    ADR uses its fictitious mass, not rho), G0 ~ U[4, 22000] J/m^2 -> s0 by
    the 2-D closed form, centred pre-crack of length U[0, 0.3] x width at an
    angle U[0, 90) degrees.  ``max_nodes`` caps the side (quick tests)."""
    rng = np.random.default_rng(seed)
    delta = 3.015 * dx
    out = []
    for _ in range(count):
        n = int(round(math.exp(rng.uniform(math.log(side[0]), math.log(side[1])))))
        if max_nodes:
            n = min(n, max_nodes)
        E = rng.uniform(70.0e9, 210.0e9)
        rho = rng.uniform(2400.0, 8000.0)
        G0 = rng.uniform(4.0, 22000.0)
        frac = rng.uniform(0.0, 0.3)
        theta = rng.uniform(0.0, math.pi / 2.0)
        out.append(dict(nx=n, ny=n, emod=E, dens=rho, G0=G0, critical_s=s0_2d(G0, E, delta),
                        crack_len=frac * n * dx, crack_theta=theta, load_scale=1.0))
    return out


def build_batch(count=256, seed=20240607, dx=5e-4, nt=1000, derive=None, max_nodes=None):
    """The plate-tensile ADR pipeline on a seeded batch of uneven plates
    (batch_specimens): shared dx = 5e-4, thickness dx, nu = 1/3, ADR dt = 1,
    boundary rows moving +-2.7e-8 m per step.  Returns (base params,
    specimens, meta)."""
    base = _derive(derive)(2, PD_MODEL_BOND, PD_MODE_STATIC, 1.0, nt, dx, 0.0, dx, 0.05, 0.05, 0.0, 192.0e9,
                           1.0 / 3.0, 8000.0, 0.04472)
    specs = batch_specimens(count, seed, dx, max_nodes=max_nodes)
    return base, specs, dict(load=2.7e-8 / base.dt, nt=nt, workload="batch_plate_adr_2d_pmb", seed=seed,
                             count=count)


def build_specimen(base, sp, derive=None):
    """One batch specimen set up alone, as the batch sets it up: the plate
    of the crack-plate layout with the specimen's size, modulus, s0 and
    pre-crack.  Returns (params, setup)."""
    nx, ny = int(sp["nx"]), int(sp["ny"])
    p = _derive(derive)(2, PD_MODEL_BOND, base.mode, base.dt, base.nt, base.dx, base.load, base.thick, nx * base.dx,
                        ny * base.dx, 0.0, float(sp["emod"]), base.pratio, base.dens, float(sp["critical_s"]))
    p.nx, p.ny = nx, ny
    p.N_int = nx * ny
    p.N = p.N_int + 6 * nx

    def setup(eng):
        eng.coord_plate_crack()
        eng.find_neighbor_gpu()
        eng.surface_correct_gpu()
        eng.initial_state()
        if sp.get("crack_len", 0.0) > 0.0:
            eng.set_crack_2d(float(sp["crack_len"]), 0.0, 0.0, float(sp.get("crack_theta", 0.0)))
        eng.prepare()

    return p, setup


# ---- quasi-static crack-growth plate for the learned ADR warm start ----------------
def build_warm_start_plate(scale=1.0, dx=1e-4, E=192.0e9, G0=2.65e3, crack_frac=0.2, derive=None):
    """0.1 x 0.1 m plate, dx = 1e-4 (1000 x 1000 nodes) plus 3 boundary rows
    above and below (the crack-plate layout, Coord.cu:34-45), 2-D PMB,
    thickness dx, nu = 1/3, s0 from G0 by the 2-D closed form, an edge
    pre-crack 0.02 m long from the left edge along the mid-line, surface
    correction on, ADR with dt = 1.  Loaded in 200 equal increments of the
    boundary rows to 1e-4 m (each increment moves the rows by +-5e-7 m).
    ``scale`` shrinks the plate and the crack together (same dx).  G0 is
    chosen so that the pre-crack starts to grow within the loading (bond
    stretch at the tip ~ 8x the nominal strain; s0 = 8e-3)."""
    L = 0.1 * scale
    delta = 3.015 * dx
    s0 = s0_2d(G0, E, delta)
    p = _derive(derive)(2, PD_MODEL_BOND, PD_MODE_STATIC, 1.0, 200, dx, 0.0, dx, L, L, 0.0, E, 1.0 / 3.0, 8000.0,
                        s0)
    p.N = p.N_int + 6 * p.nx
    crack = crack_frac * L

    def setup(eng):
        eng.coord_plate_crack()
        eng.find_neighbor_gpu()
        eng.surface_correct_gpu()
        eng.initial_state()
        eng.set_crack_2d(crack, -L / 2.0 + crack / 2.0, 0.0, 0.0)
        eng.prepare()

    return p, setup, dict(increments=200, delta=1e-4 / 200, tol=1e-6, workload="warm_start_plate_adr_2d_pmb",
                          s0=s0, crack=crack)
