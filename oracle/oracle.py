"""TEST INFRASTRUCTURE ONLY: numpy front end of the oracle (oracle/pd_oracle.c).

The oracle restates the reference's (XiaoMmingW/PD_Gpu1) algorithms on the CPU.
It is the checker of the GPU engine and the timed CPU baseline; only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU legs use it.  The product
(``pd_gpu1_gb300``) never imports this module.

Storage follows the reference: node arrays of length N, bond arrays of N*MN
slots in padded ELL (row i = slots [i*MN, i*MN+NN[i])).
"""
import ctypes as C
import os

import numpy as np

from pd_gpu1_gb300._abi import PDCylinder, PDParams, PD_MODEL_BOND, PD_MODEL_STATE

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpd_oracle.so")

_lib = None

D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)


def build():
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    import subprocess

    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _lib.or_params_derive.argtypes = [C.POINTER(PDParams), C.c_int, C.c_int, C.c_int] + [C.c_double] * 12 + [C.c_int]
        _lib.or_find_neighbor_bf.restype = C.c_int
        _lib.or_find_neighbor_cells.restype = C.c_int
        _lib.or_coord_kw.restype = C.c_int64
        _lib.or_coord_kw.argtypes = [C.POINTER(PDParams), C.c_double, D, D, D, C.c_int64]
        _lib.or_adr_cn.restype = C.c_double
        _lib.or_set_crack_2d.argtypes = [C.POINTER(PDParams), C.c_double, C.c_double, C.c_double, C.c_double, I, I, D, D, I]
        _lib.or_set_crack_kw.argtypes = [C.POINTER(PDParams), C.c_double, I, I, D, D, I]
        _lib.or_quick_load.argtypes = [C.POINTER(PDParams), C.c_double, D]
        _lib.or_adr_update.argtypes = [C.POINTER(PDParams), C.c_int, C.c_double] + [D] * 18
        _lib.or_bond_force.argtypes = [C.POINTER(PDParams), C.c_int64] + [D] * 6 + [I, I, D, D, D, I, D, D, D]
    return _lib


def set_threads(n):
    lib().or_set_threads(int(n))


def num_threads():
    return lib().or_num_threads()


def _d(a):
    if a is None:
        return C.cast(None, D)
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(D)


def _i(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(I)


def derive_params(dim, model, mode, dt, nt, dx, load=0.0, thick=0.0, length=0.05, height=0.05,
                  width=0.0, emod=192.0e9, pratio=1.0 / 3.0, dens=8000.0, critical_s=0.04472,
                  fix_k3d=0):
    """BaseModel_Parameter (Base.cuh:72-184) defaults and derivation."""
    p = PDParams()
    rc = lib().or_params_derive(C.byref(p), dim, model, mode, dt, nt, dx, load, thick, length,
                                height, width, emod, pratio, dens, critical_s, fix_k3d)
    assert rc == 0, rc
    return p


class Model:
    """Node and bond arrays of one specimen in the reference's layout."""

    def __init__(self, p, x, y, z=None):
        self.p = p
        N = p.N
        self.N = N
        self.MN = p.MN
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.y = np.ascontiguousarray(y, dtype=np.float64)
        self.z = np.ascontiguousarray(z if z is not None else np.zeros(N), dtype=np.float64)
        z0 = lambda: np.zeros(N, dtype=np.float64)
        self.ux, self.uy, self.uz = z0(), z0(), z0()
        self.vx, self.vy, self.vz = z0(), z0(), z0()
        self.ax, self.ay, self.az = z0(), z0(), z0()
        self.fx, self.fy, self.fz = z0(), z0(), z0()
        self.bx, self.by, self.bz = z0(), z0(), z0()
        self.vhx, self.vhy, self.vhz = z0(), z0(), z0()
        self.fox, self.foy, self.foz = z0(), z0(), z0()
        self.dmg = z0()
        self.m = z0()
        self.theta = z0()
        self.fncst = [z0(), z0(), z0()]
        self.NN = np.zeros(N, dtype=np.int32)
        S = N * self.MN
        self.NL = np.zeros(S, dtype=np.int32)
        self.idist = np.zeros(S)
        self.fac = np.zeros(S)
        self.scr = np.ones(S)
        self.w = np.zeros(S)
        self.e = np.zeros(S)
        self.fail = np.ones(S, dtype=np.int32)  # kernel_initial_fail (Initial.cu:6-14)
        self.cn = 0.0

    # ---- setup -------------------------------------------------------
    def find_neighbor(self, brute=None):
        if brute is None:
            brute = self.N <= 20000
        f = lib().or_find_neighbor_bf if brute else lib().or_find_neighbor_cells
        mx = f(C.byref(self.p), _d(self.x), _d(self.y), _d(self.z), _i(self.NN), _i(self.NL))
        if mx > self.MN:
            raise ValueError(f"family of {mx} exceeds MN={self.MN}")
        return mx

    def vol_corr(self):
        lib().or_vol_corr(C.byref(self.p), _i(self.NN), _i(self.NL), _d(self.x), _d(self.y), _d(self.z),
                          _d(self.idist), _d(self.fac))

    def surface_correct(self):
        lib().or_surface_correct(C.byref(self.p), _i(self.NN), _i(self.NL), _d(self.x), _d(self.y),
                                 _d(self.z), _d(self.idist), _d(self.fac), _d(self.fncst[0]),
                                 _d(self.fncst[1]), _d(self.fncst[2]), _d(self.scr))

    def initial_weight(self):
        lib().or_initial_weight(C.byref(self.p), _i(self.NN), _d(self.idist), _d(self.fac), _d(self.w), _d(self.m))

    def set_crack_2d(self, clength, loc_x, loc_y, theta):
        lib().or_set_crack_2d(C.byref(self.p), clength, loc_x, loc_y, theta, _i(self.NN), _i(self.NL),
                              _d(self.x), _d(self.y), _i(self.fail))

    def set_crack_kw(self, rad):
        lib().or_set_crack_kw(C.byref(self.p), rad, _i(self.NN), _i(self.NL), _d(self.x), _d(self.y), _i(self.fail))

    def load_plate_tensile(self):
        lib().or_load_plate_tensile(C.byref(self.p), _d(self.bx))

    def quick_load(self, load):
        lib().or_quick_load(C.byref(self.p), load, _d(self.uy))

    # ---- per step ----------------------------------------------------
    def bond_force(self, n_nodes=None):
        n = self.p.N_int if n_nodes is None else n_nodes
        lib().or_bond_force(C.byref(self.p), n, _d(self.x), _d(self.y), _d(self.z), _d(self.ux), _d(self.uy),
                            _d(self.uz), _i(self.NN), _i(self.NL), _d(self.idist), _d(self.scr), _d(self.fac),
                            _i(self.fail), _d(self.fx), _d(self.fy), _d(self.fz))

    def state_force(self):
        args = (C.byref(self.p), _d(self.x), _d(self.y), _d(self.z), _d(self.ux), _d(self.uy), _d(self.uz),
                _i(self.NN), _i(self.NL), _d(self.idist), _d(self.fac), _d(self.w), _d(self.m))
        lib().or_state_theta(*args, _i(self.fail), _d(self.e), _d(self.theta))
        lib().or_state_force(*args, _d(self.theta), _d(self.e), _i(self.fail), _d(self.fx), _d(self.fy), _d(self.fz))

    def force(self):
        if self.p.model == PD_MODEL_BOND:
            self.bond_force()
        else:
            self.state_force()

    def adr_step(self, ct):
        """Per-step body of solve_plate_tensile (Solve_Plate_Tensile.cu:109-129)."""
        self.force()
        self.cn = lib().or_adr_cn(C.byref(self.p), _d(self.fx), _d(self.fy), _d(self.fz), _d(self.fox), _d(self.foy),
                                  _d(self.foz), _d(self.vhx), _d(self.vhy), _d(self.vhz), _d(self.ux),
                                  _d(self.uy), _d(self.uz))
        lib().or_adr_update(C.byref(self.p), int(ct), self.cn, _d(self.fx), _d(self.fy), _d(self.fz), _d(self.bx),
                            _d(self.by), _d(self.bz), _d(self.vhx), _d(self.vhy), _d(self.vhz), _d(self.vx),
                            _d(self.vy), _d(self.vz), _d(self.ux), _d(self.uy), _d(self.uz), _d(self.fox),
                            _d(self.foy), _d(self.foz))

    def verlet1(self):
        lib().or_verlet1(C.byref(self.p), _d(self.vx), _d(self.vy), _d(self.vz), _d(self.ax), _d(self.ay),
                         _d(self.az), _d(self.ux), _d(self.uy), _d(self.uz))

    def verlet2(self):
        lib().or_verlet2(C.byref(self.p), _d(self.vx), _d(self.vy), _d(self.vz), _d(self.ax), _d(self.ay),
                         _d(self.az), _d(self.fx), _d(self.fy), _d(self.fz), _d(self.bx), _d(self.by), _d(self.bz))

    def explicit_step(self, load=0.0, cyl=None):
        """Per-step body of the explicit drivers (Solve_Plate_Crack_Grow.cu:127-148,
        Solve_Kalthoff_Winkler.cu:408-429)."""
        if load:
            self.quick_load(load)
        self.verlet1()
        if cyl is not None:
            lib().or_cy_integrate1(C.byref(self.p), C.byref(cyl))
        self.force()
        if cyl is not None:
            lib().or_contact(C.byref(self.p), C.byref(cyl), _d(self.dmg), _d(self.x), _d(self.y), _d(self.z),
                             _d(self.ux), _d(self.uy), _d(self.uz), _d(self.vx), _d(self.vy), _d(self.vz),
                             cyl.force)
        self.verlet2()
        if cyl is not None:
            lib().or_cy_integrate2(C.byref(self.p), C.byref(cyl))

    def damage(self):
        lib().or_damage(C.byref(self.p), _i(self.NN), _i(self.fail), _d(self.fac), _d(self.dmg))

    # ---- views -------------------------------------------------------
    def rows(self, arr):
        """Concatenate the used slots of a bond array in CSR order."""
        a = arr.reshape(self.N, self.MN)
        mask = np.arange(self.MN)[None, :] < self.NN[:, None]
        return a[mask]

    def rowptr(self):
        rp = np.zeros(self.N + 1, dtype=np.int64)
        np.cumsum(self.NN, out=rp[1:])
        return rp


def coord_kw(p, rad):
    cap = p.nx * p.ny * max(p.nz, 1)
    x = np.zeros(cap)
    y = np.zeros(cap)
    z = np.zeros(cap)
    n = lib().or_coord_kw(C.byref(p), rad, _d(x), _d(y), _d(z), cap)
    return x[:n].copy(), y[:n].copy(), z[:n].copy()


def plate_coords(p):
    x = np.zeros(p.N)
    y = np.zeros(p.N)
    lib().or_coord_plate(C.byref(p), _d(x), _d(y))
    return x, y


def plate_crack_coords(p):
    x = np.zeros(p.N)
    y = np.zeros(p.N)
    lib().or_coord_plate_crack(C.byref(p), _d(x), _d(y))
    return x, y


def new_cylinder(rad, mass, height, v, x, y, z):
    """kernel_initial_cylinder (Solve_Kalthoff_Winkler.cu:9-22): vel[1] = v."""
    c = PDCylinder()
    c.rad, c.mass, c.height, c.v, c.x, c.y, c.z = rad, mass, height, v, x, y, z
    c.vel[1] = v
    return c
