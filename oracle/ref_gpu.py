"""TEST/MEASUREMENT INFRASTRUCTURE ONLY: the reference's own CUDA kernels on the GPU.

oracle/_ref/ref_kernels.cubin is compiled from the reference sources (make -C
oracle ref, in a container that has them) and loaded through the CUDA driver
API by oracle/_build/libref_gpu_runner.so.  The caller supplies the problem in
the reference's layout; :func:`from_engine` converts an engine context's CSR
family into the reference's padded ELL arrays.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ref_kernels.cubin")
LIB = os.path.join(HERE, "_build", "libref_gpu_runner.so")

D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)


def available():
    return os.path.exists(CUBIN)


def _d(a):
    return a.ctypes.data_as(D)


def _i(a):
    return a.ctypes.data_as(I)


class RefGPU:
    PARTICLE = 0  # kernel_particle_force_2D, thread per node (the tensile driver's choice)
    WARP = 1      # kernel_bond_force_2D, warp per node

    def __init__(self):
        if not os.path.exists(LIB):
            subprocess.run(["make", "-s", "-C", HERE, "_build/libref_gpu_runner.so"], check=True)
        self.lib = C.CDLL(LIB)
        self.lib.rr_error.restype = C.c_char_p
        self.lib.rr_run.argtypes = [C.c_int, C.c_int, C.c_int, D]
        self.lib.rr_run_adr.argtypes = [C.c_int, C.c_int, C.c_double, D, D]
        self.lib.rr_run_kw.argtypes = [C.c_int, D]
        self.lib.rr_run_state.argtypes = [C.c_int, C.c_double, C.c_int, D]
        self._check(self.lib.rr_init(CUBIN.encode()), "rr_init")
        self.N = self.MN = 0

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: {self.lib.rr_error().decode()}")

    def setup(self, p, x, y, NN, rowptr, NL, idist, scr, fac, fail, bx, by):
        """p: PDParams; bond arrays in CSR order (rowptr over N rows)."""
        N, MN = p.N, p.MN
        self.N, self.MN = N, MN
        mask = (np.arange(MN)[None, :] < NN[:, None]).reshape(-1)

        def ell(v, dtype, fill):
            out = np.full(N * MN, fill, dtype=dtype)
            out[mask] = v
            return out

        self.ell = ell
        self.arrays = dict(NL=ell(NL, np.int32, 0), idist=ell(idist, np.float64, 1.0), scr=ell(scr, np.float64, 0.0),
                           fac=ell(fac, np.float64, 0.0), fail=ell(fail, np.int32, 1))
        dv = np.array([p.pi, p.dx, p.emod, p.dens, p.pratio, p.bc, p.delta, p.critical_s, p.vol, p.dt, p.mass, p.K,
                       p.G])
        iv = np.array([p.N, p.MN, p.N_int, p.nx, p.ny, p.nz, p.nt], dtype=np.int32)
        a = self.arrays
        self.keep = [np.ascontiguousarray(v, dtype=np.float64) for v in (x, y, bx, by)]
        self.NNc = np.ascontiguousarray(NN, dtype=np.int32)
        self._check(self.lib.rr_setup(_d(dv), _i(iv), _d(self.keep[0]), _d(self.keep[1]), _i(self.NNc), _i(a["NL"]),
                                      _d(a["idist"]), _d(a["scr"]), _d(a["fac"]), _i(a["fail"]), _d(self.keep[2]),
                                      _d(self.keep[3])), "rr_setup")

    def setup_z(self, z, bz, cyl):
        """Third component and impactor (cyl: rad mass height v x y z) of a 3-D
        problem set up by :meth:`setup`; starts the cylinder as the impact
        driver does."""
        self.keep_z = [np.ascontiguousarray(v, dtype=np.float64) for v in (z, bz)]
        c = np.ascontiguousarray(cyl, dtype=np.float64)
        self._check(self.lib.rr_setup_z(_d(self.keep_z[0]), _d(self.keep_z[1]), _d(c)), "rr_setup_z")

    def set_disp_z(self, uz):
        uz = np.ascontiguousarray(uz, dtype=np.float64)
        self._check(self.lib.rr_set_disp_z(_d(uz)), "rr_set_disp_z")

    def setup_state(self, m, w):
        """Weighted volume m (N) and influence weights w (CSR order) of a 2-D
        state-based problem set up by :meth:`setup`."""
        self.m = np.ascontiguousarray(m, dtype=np.float64)
        self.w = self.ell(w, np.float64, 0.0)
        self._check(self.lib.rr_setup_state(_d(self.m), _d(self.w)), "rr_setup_state")

    def force_state(self):
        self._check(self.lib.rr_force_state(), "rr_force_state")

    def run_state(self, nsteps, load, dmg_every=0):
        """nsteps of the crack-grow driver's loop; returns the elapsed ms."""
        ms = C.c_double()
        self._check(self.lib.rr_run_state(nsteps, load, dmg_every, C.byref(ms)), "rr_run_state")
        return ms.value

    def force3(self):
        self._check(self.lib.rr_force3(), "rr_force3")

    def setup_state3(self, m, w):
        """Weighted volume m (N) and influence weights w (CSR order) of a 3-D
        state-based problem set up by :meth:`setup` and :meth:`setup_z`."""
        self.m = np.ascontiguousarray(m, dtype=np.float64)
        self.w = self.ell(w, np.float64, 0.0)
        self._check(self.lib.rr_setup_state3(_d(self.m), _d(self.w)), "rr_setup_state3")

    def initial_weight3(self):
        """kernel_initial_weight_3D (N must be even)."""
        self._check(self.lib.rr_initial_weight3(), "rr_initial_weight3")

    def get_state3(self):
        """(m, w) of the 3-D state-based arrays; w in the padded N*MN layout."""
        m = np.zeros(self.N)
        w = np.zeros(self.N * self.MN)
        self._check(self.lib.rr_get_state3(_d(m), _d(w)), "rr_get_state3")
        return m, w

    def set_theta_e(self, theta, e):
        """Dilatation (N) and per-bond extension (padded N*MN layout) for
        kernel_state_force_3D."""
        self.theta_h = np.ascontiguousarray(theta, dtype=np.float64)
        self.e_h = np.ascontiguousarray(e, dtype=np.float64)
        self._check(self.lib.rr_set_theta_e(_d(self.theta_h), _d(self.e_h)), "rr_set_theta_e")

    def force_state3(self):
        """One kernel_state_force_3D evaluation (N_int must be even)."""
        self._check(self.lib.rr_force_state3(), "rr_force_state3")

    def get_fail(self):
        """The N*MN intact flags in the padded layout."""
        fail = np.zeros(self.N * self.MN, dtype=np.int32)
        self._check(self.lib.rr_get(None, None, None, None, None, _i(fail), None), "rr_get")
        return fail

    def run_kw(self, nsteps):
        """nsteps of the impact driver's loop; returns the elapsed ms."""
        ms = C.c_double()
        self._check(self.lib.rr_run_kw(nsteps, C.byref(ms)), "rr_run_kw")
        return ms.value

    def get_z(self):
        """uz, vz, fz and the impactor state (acc, disp, vel, force)."""
        out = {k: np.zeros(self.N) for k in ("uz", "vz", "fz")}
        cyl = np.zeros(12)
        self._check(self.lib.rr_get_z(_d(out["uz"]), _d(out["vz"]), _d(out["fz"]), _d(cyl)), "rr_get_z")
        out.update(cyl_acc=cyl[0:3], cyl_disp=cyl[3:6], cyl_vel=cyl[6:9], cyl_force=cyl[9:12])
        return out

    def set_disp(self, ux, uy):
        ux = np.ascontiguousarray(ux, dtype=np.float64)
        uy = np.ascontiguousarray(uy, dtype=np.float64)
        self._check(self.lib.rr_set_disp(_d(ux), _d(uy)), "rr_set_disp")

    def force(self, variant):
        self._check(self.lib.rr_force(variant), "rr_force")

    def run(self, variant, nsteps, dmg_every=0):
        ms = C.c_double()
        self._check(self.lib.rr_run(variant, nsteps, dmg_every, C.byref(ms)), "rr_run")
        return ms.value

    def run_adr(self, ct0, nsteps, load):
        """solve_plate_tensile's ADR loop with moving boundary rows; returns
        (elapsed ms, last damping coefficient)."""
        ms, cn = C.c_double(), C.c_double()
        self._check(self.lib.rr_run_adr(ct0, nsteps, load, C.byref(ms), C.byref(cn)), "rr_run_adr")
        return ms.value, cn.value

    def get(self, NN=None):
        N, MN = self.N, self.MN
        out = {k: np.zeros(N) for k in ("ux", "uy", "fx", "fy", "vy", "dmg")}
        fail = np.zeros(N * MN, dtype=np.int32)
        self._check(self.lib.rr_get(_d(out["ux"]), _d(out["uy"]), _d(out["fx"]), _d(out["fy"]), _d(out["vy"]),
                                    _i(fail), _d(out["dmg"])), "rr_get")
        if NN is not None:
            mask = (np.arange(MN)[None, :] < NN[:, None]).reshape(-1)
            out["fail"] = fail[mask]
        return out

    def free(self):
        self.lib.rr_free()


def from_engine(eng, p, cyl=None):
    """A RefGPU loaded with the engine context's current problem (family,
    coefficients, fail flags, body forces; in 3-D also z and the impactor
    ``cyl``, an object with rad, mass, height, v, x, y, z)."""
    r = RefGPU()
    NN = eng.get("NN")
    r.setup(p, eng.get("X"), eng.get("Y"), NN, eng.get("ROWPTR"), eng.get("NL"), eng.get("IDIST"), eng.get("SCR"),
            eng.get("FAC"), eng.get("FAIL"), eng.get("BX"), eng.get("BY"))
    if p.dim == 3:
        c = [0.0] * 7 if cyl is None else [cyl.rad, cyl.mass, cyl.height, cyl.v, cyl.x, cyl.y, cyl.z]
        r.setup_z(eng.get("Z"), eng.get("BZ"), c)
    if p.model == 2 and p.dim == 2:
        r.setup_state(eng.get("M"), eng.get("W"))
    return r, NN


def damage_from_flags(NN, fail, fac, vol=1.0):
    """Node damage 1 - sum(fail vol fac) / sum(vol fac) over each row's bonds
    (kernel_cal_dmg_2D/3D, Base_Function.cu:149-217), from CSR-ordered flags
    and volume-correction factors; rows without bonds get 0."""
    NN = np.asarray(NN, dtype=np.int64)
    row = np.repeat(np.arange(len(NN)), NN)
    fac = np.asarray(fac, dtype=np.float64)
    num = np.bincount(row, weights=np.asarray(fail, dtype=np.float64) * vol * fac, minlength=len(NN))
    den = np.bincount(row, weights=vol * fac, minlength=len(NN))
    den[NN == 0] = 1.0
    num[NN == 0] = 1.0
    return 1.0 - num / den
