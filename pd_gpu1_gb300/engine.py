"""Host-side front end of the GB300 engine over the C ABI.

:class:`Engine` owns one ``pd_ctx`` and exposes the operators under the names
of the reference's host launchers (XiaoMmingW/PD_Gpu1): ``find_neighbor_gpu``
(Neighbor.cuh:8), ``surface_correct_gpu`` (Surf_Corr.cuh:8),
``bond_force_gpu`` (Force_Bond.cuh:9-10), ``state_force_gpu``
(Force_State.cuh), ``static_integrate_gpu`` (Integrate.cuh:12), ``sum``
(Reduce.cuh:8) and the drivers ``solve_plate_tensile`` /
``solve_plate_crack_grow`` / ``solve_kalthoff_winkler`` (Solve_*.cuh:17-19).
Errors raise :class:`PDError` carrying the C status code instead of exiting.
"""
import ctypes as C

import numpy as np

from ._abi import FIELD, FIELD_DTYPE, PDCylinder, PDLoadStepStats, PDParams, PDResult, PDSpecimen
from ._lib import PDError, check, lib

__all__ = ["Engine", "Batch", "derive_params", "coord_kw", "solve_plate_tensile", "solve_plate_crack_grow",
           "solve_kalthoff_winkler", "PDError"]


def _stream(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, "cuda_stream", stream))


def derive_params(dim, model, mode, dt, nt, dx, load=0.0, thick=0.0, length=0.05, height=0.05, width=0.0,
                  emod=192.0e9, pratio=1.0 / 3.0, dens=8000.0, critical_s=0.04472, fix_k3d=0):
    """BaseModel_Parameter (Base.cuh:72-184) with its default arguments."""
    p = PDParams()
    check(lib().pd_params_derive(C.byref(p), dim, model, mode, dt, nt, dx, load, thick, length, height, width,
                                 emod, pratio, dens, critical_s, fix_k3d), what="pd_params_derive")
    return p


def coord_kw(p, rad):
    """coord_KW (Coord.cu:77-129): notched-slab coordinates."""
    cap = p.nx * p.ny * max(p.nz, 1)
    x, y, z = (np.zeros(cap) for _ in range(3))
    n = C.c_int64()
    dp = C.POINTER(C.c_double)
    check(lib().pd_coord_kw(C.byref(p), rad, x.ctypes.data_as(dp), y.ctypes.data_as(dp), z.ctypes.data_as(dp), cap,
                            C.byref(n)), what="pd_coord_kw")
    n = n.value
    return x[:n].copy(), y[:n].copy(), z[:n].copy()


class Engine:
    """One specimen on the GPU (a ``pd_ctx``)."""

    def __init__(self, params, stream=None):
        self._lib = lib()
        st = C.c_int(0)
        self.p = params.copy()
        self.ctx = self._lib.pd_create(C.byref(self.p), C.byref(st))
        if not self.ctx:
            check(st.value, None, "pd_create")
        self.stream = _stream(stream)

    # ---- lifetime ---------------------------------------------------------
    def close(self):
        if getattr(self, "ctx", None):
            self._lib.pd_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _c(self, status, what):
        return check(status, self.ctx, what)

    # ---- fields -----------------------------------------------------------
    def field_count(self, name):
        ptr = C.c_void_p()
        n = C.c_size_t()
        self._c(self._lib.pd_field_ptr(self.ctx, FIELD[name], C.byref(ptr), C.byref(n)), "pd_field_ptr")
        return n.value

    def get(self, name):
        n = self.field_count(name) if name not in ("X", "Y", "Z", "UX", "UY", "UZ") else self.p.N
        out = np.empty(n, dtype=FIELD_DTYPE[name])
        self._c(self._lib.pd_get_field(self.ctx, FIELD[name], out.ctypes.data, n, self.stream), "pd_get_field " + name)
        return out

    def set(self, name, values):
        arr = np.ascontiguousarray(values, dtype=FIELD_DTYPE[name])
        self._c(self._lib.pd_set_field(self.ctx, FIELD[name], arr.ctypes.data, arr.size, self.stream),
                "pd_set_field " + name)

    def device_ptr(self, name):
        ptr = C.c_void_p()
        n = C.c_size_t()
        self._c(self._lib.pd_field_ptr(self.ctx, FIELD[name], C.byref(ptr), C.byref(n)), "pd_field_ptr")
        return ptr.value, n.value

    def count_broken(self):
        """Broken bonds over the whole family (pd_count_broken: counted on the
        device, one integer copied back)."""
        v = C.c_int64()
        self._c(self._lib.pd_count_broken(self.ctx, C.byref(v), self.stream), "pd_count_broken")
        return v.value

    def device_view(self, name, count=None):
        """A torch tensor on the field's device memory (no copy); count
        elements from the start (all by default)."""
        import torch

        ptr, n = self.device_ptr(name)
        n = n if count is None else count
        dt = {np.dtype(np.float64): "<f8", np.dtype(np.int32): "<i4"}[np.dtype(FIELD_DTYPE[name])]

        class _View:
            __cuda_array_interface__ = {"shape": (n,), "typestr": dt, "data": (ptr, False), "version": 2}

        return torch.as_tensor(_View(), device="cuda")

    @property
    def num_bonds(self):
        return self._lib.pd_num_bonds(self.ctx)

    @property
    def kernel_launches(self):
        return self._lib.pd_kernel_launches(self.ctx)

    def sync(self):
        self._c(self._lib.pd_sync(self.ctx, self.stream), "pd_sync")

    def params(self):
        q = PDParams()
        self._c(self._lib.pd_get_params(self.ctx, C.byref(q)), "pd_get_params")
        return q

    def set_params(self, p):
        self._c(self._lib.pd_set_params(self.ctx, C.byref(p)), "pd_set_params")
        self.p = p.copy()

    # ---- setup (reference launcher names) -------------------------------------
    def coord_plate(self):
        self._c(self._lib.pd_coord_plate(self.ctx, self.stream), "pd_coord_plate")

    def coord_plate_crack(self):
        self._c(self._lib.pd_coord_plate_crack(self.ctx, self.stream), "pd_coord_plate_crack")

    def set_coords(self, x, y, z=None):
        self.set("X", x)
        self.set("Y", y)
        if z is not None:
            self.set("Z", z)

    def find_neighbor_gpu(self):
        self._c(self._lib.pd_find_neighbor(self.ctx, self.stream), "pd_find_neighbor")

    def vol_corr(self):
        self._c(self._lib.pd_vol_corr(self.ctx, self.stream), "pd_vol_corr")

    def surface_correct_gpu(self):
        self._c(self._lib.pd_surface_correct(self.ctx, self.stream), "pd_surface_correct")

    def initial_weight(self):
        self._c(self._lib.pd_initial_weight(self.ctx, self.stream), "pd_initial_weight")

    def set_crack_2d(self, clength, loc_x, loc_y, theta):
        self._c(self._lib.pd_set_crack_2d(self.ctx, clength, loc_x, loc_y, theta, self.stream), "pd_set_crack_2d")

    def set_crack_kw(self, rad):
        self._c(self._lib.pd_set_crack_kw(self.ctx, rad, self.stream), "pd_set_crack_kw")

    def initial_state(self):
        self._c(self._lib.pd_initial_state(self.ctx, self.stream), "pd_initial_state")

    def prepare(self):
        self._c(self._lib.pd_prepare(self.ctx, self.stream), "pd_prepare")

    def load_plate_tensile(self):
        self._c(self._lib.pd_load_plate_tensile(self.ctx, self.stream), "pd_load_plate_tensile")

    def quick_load(self, load):
        self._c(self._lib.pd_quick_load(self.ctx, load, self.stream), "pd_quick_load")

    # ---- per-step operators --------------------------------------------------
    def bond_force_gpu(self):
        self._c(self._lib.pd_bond_force(self.ctx, self.stream), "pd_bond_force")

    def state_force_gpu(self):
        self._c(self._lib.pd_state_force(self.ctx, self.stream), "pd_state_force")

    def force(self):
        if self.p.model == 1:
            self.bond_force_gpu()
        else:
            self.state_force_gpu()

    def static_integrate_gpu(self, ct):
        self._c(self._lib.pd_integrate_adr(self.ctx, ct, self.stream), "pd_integrate_adr")

    def adr_cn(self):
        v = C.c_double()
        self._c(self._lib.pd_get_adr_cn(self.ctx, C.byref(v), self.stream), "pd_get_adr_cn")
        return v.value

    def integrate_verlet1(self):
        self._c(self._lib.pd_integrate_verlet1(self.ctx, self.stream), "pd_integrate_verlet1")

    def integrate_verlet2(self):
        self._c(self._lib.pd_integrate_verlet2(self.ctx, self.stream), "pd_integrate_verlet2")

    def sum(self, name, n=None):
        ptr, count = self.device_ptr(name)
        out = C.c_double()
        self._c(self._lib.pd_reduce_sum(self.ctx, ptr, count if n is None else n, C.byref(out), self.stream),
                "pd_reduce_sum")
        return out.value

    def damage(self):
        self._c(self._lib.pd_damage(self.ctx, self.stream), "pd_damage")

    def cylinder_init(self, cyl):
        self._c(self._lib.pd_cylinder_init(self.ctx, C.byref(cyl), self.stream), "pd_cylinder_init")

    def cylinder(self):
        c = PDCylinder()
        self._c(self._lib.pd_cylinder_get(self.ctx, C.byref(c), self.stream), "pd_cylinder_get")
        return c

    def cylinder_integrate1(self):
        self._c(self._lib.pd_cylinder_integrate1(self.ctx, self.stream), "pd_cylinder_integrate1")

    def cylinder_integrate2(self):
        self._c(self._lib.pd_cylinder_integrate2(self.ctx, self.stream), "pd_cylinder_integrate2")

    def contact(self):
        self._c(self._lib.pd_contact(self.ctx, self.stream), "pd_contact")

    # ---- fused loops -------------------------------------------------------
    def run_adr(self, ct0, nsteps, load=0.0):
        self._c(self._lib.pd_run_adr(self.ctx, ct0, nsteps, load, self.stream), "pd_run_adr")

    def run_explicit(self, nsteps, load=0.0, dmg_every=0):
        self._c(self._lib.pd_run_explicit(self.ctx, nsteps, load, dmg_every, self.stream), "pd_run_explicit")

    # ---- quasi-static load stepping -----------------------------------------
    def residual(self):
        """|F + b| over the free nodes at the current displacement."""
        r = C.c_double()
        self._c(self._lib.pd_residual(self.ctx, C.byref(r), self.stream), "pd_residual")
        return r.value

    def adr_solve(self, ct0, max_iters, check_every, tol):
        it, r = C.c_int(), C.c_double()
        self._c(self._lib.pd_adr_solve(self.ctx, ct0, max_iters, check_every, tol, C.byref(it), C.byref(r),
                                       self.stream), "pd_adr_solve")
        return it.value, r.value

    def load_step(self, delta, du_ptr=None, tol_rel=1e-6, max_iters=200000, check_every=100, ncand=1,
                  probe_iters=0):
        """One load increment solved by ADR to tol_rel; du_ptr: device pointer
        to ncand candidate increments (2*N_int doubles each) or None; probe_iters:
        ADR steps of the probe that chooses among admissible candidates.
        Returns the stats."""
        st = PDLoadStepStats()
        self._c(self._lib.pd_load_step(self.ctx, delta, du_ptr, ncand if du_ptr else 0, probe_iters, tol_rel,
                                       max_iters, check_every, C.byref(st), self.stream), "pd_load_step")
        return st.as_dict()

    def check_finite(self):
        self._c(self._lib.pd_check_finite(self.ctx, self.stream), "pd_check_finite")

    def profile_steps(self, kind, ct0, nsteps, load=0.0):
        """(force ms, step ms) per step over nsteps real steps (kind 0 ADR,
        1 explicit), timed with CUDA events on the launch stream."""
        f, st = C.c_double(), C.c_double()
        self._c(self._lib.pd_profile_steps(self.ctx, kind, ct0, nsteps, load, C.byref(f), C.byref(st), self.stream),
                "pd_profile_steps")
        return f.value, st.value

    # ---- launch shape of the bond-force kernel ------------------------------
    def set_launch(self, block=256, chunked=0, waves=1, split=1):
        self._c(self._lib.pd_set_launch(self.ctx, block, chunked, waves, split), "pd_set_launch")

    def launch(self):
        b, k, w, p = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self._c(self._lib.pd_get_launch(self.ctx, C.byref(b), C.byref(k), C.byref(w), C.byref(p)),
                "pd_get_launch")
        return b.value, k.value, w.value, p.value

    LAYOUTS = {"auto": 0, "records": 1, "compact": 2}

    def set_force_layout(self, layout="auto"):
        """Per-bond storage of the bond-based kernels: "records" (48 bytes per
        slot), "compact" (16-byte records on offset-class templates, 2-D) or
        "auto" (compact where it fits); takes effect at the next prepare."""
        self._c(self._lib.pd_set_force_layout(self.ctx, self.LAYOUTS[layout]), "pd_set_force_layout")

    def force_layout(self):
        v = C.c_int()
        self._c(self._lib.pd_get_force_layout(self.ctx, C.byref(v)), "pd_get_force_layout")
        return {0: None, 1: "records", 2: "compact"}[v.value]

    def autotune(self, reps=5):
        """Times the launch shapes at the current state and keeps the fastest;
        returns (block, chunked, waves, split, ms per launch)."""
        ms = C.c_double()
        self._c(self._lib.pd_autotune(self.ctx, reps, C.byref(ms), self.stream), "pd_autotune")
        return self.launch() + (ms.value,)

    # ---- output ------------------------------------------------------------
    def save_disp(self, path="disp.txt"):
        """save_disp_gpu (Save.cu:6-36): ux uy [uz] dmg per interior node."""
        self._c(self._lib.pd_save_disp(self.ctx, str(path).encode(), self.stream), "pd_save_disp")

    def save_kw(self, rad, path="disp.txt"):
        """save_kw_gpu (Save.cu:62-101)."""
        self._c(self._lib.pd_save_kw(self.ctx, rad, str(path).encode(), self.stream), "pd_save_kw")

    def snapshot_save(self, path):
        self._c(self._lib.pd_snapshot_save(self.ctx, str(path).encode(), self.stream), "pd_snapshot_save")

    def snapshot_load(self, path):
        self._c(self._lib.pd_snapshot_load(self.ctx, str(path).encode(), self.stream), "pd_snapshot_load")

    def crack_tip(self, threshold=0.38):
        xy = (C.c_double * 2)()
        self._c(self._lib.pd_crack_tip(self.ctx, threshold, xy, self.stream), "pd_crack_tip")
        return xy[0], xy[1]

    # ---- views -------------------------------------------------------------
    def csr(self):
        """(rowptr, NL) of the bond family."""
        return self.get("ROWPTR"), self.get("NL")


class Batch(Engine):
    """Many 2-D bond-based plates in one context (``pd_batch_create``).

    ``specimens`` is a sequence of dicts (or :class:`PDSpecimen`) with keys
    nx, ny, emod, critical_s and optionally crack_len, crack_theta,
    load_scale; ``base`` carries the shared parameters (dx, dt, thickness,
    Poisson ratio, horizon, MN)."""

    def __init__(self, base, specimens, stream=None):
        self._lib = lib()
        n = len(specimens)
        arr = (PDSpecimen * n)()
        for k, sp in enumerate(specimens):
            if isinstance(sp, PDSpecimen):
                arr[k] = sp
                continue
            a = arr[k]
            a.nx, a.ny = int(sp["nx"]), int(sp["ny"])
            a.emod, a.critical_s = float(sp["emod"]), float(sp["critical_s"])
            a.crack_len = float(sp.get("crack_len", 0.0))
            a.crack_theta = float(sp.get("crack_theta", 0.0))
            a.load_scale = float(sp.get("load_scale", 1.0))
        self.specimens = arr
        st = C.c_int(0)
        b = base.copy()
        self.ctx = self._lib.pd_batch_create(C.byref(b), arr, n, C.byref(st))
        if not self.ctx:
            check(st.value, None, "pd_batch_create")
        self.stream = _stream(stream)
        self.p = self.params()
        cnt = C.c_int()
        self.interior = np.zeros(n + 1, dtype=np.int64)
        self.boundary = np.zeros(n + 1, dtype=np.int64)
        self._c(self._lib.pd_batch_info(self.ctx, C.byref(cnt), self.interior.ctypes.data_as(C.POINTER(C.c_int64)),
                                        self.boundary.ctypes.data_as(C.POINTER(C.c_int64))), "pd_batch_info")
        self.count = cnt.value

    def run_adr(self, ct0, nsteps, load=0.0):
        self._c(self._lib.pd_batch_run_adr(self.ctx, ct0, nsteps, load, self.stream), "pd_batch_run_adr")

    def cn(self):
        out = np.zeros(self.count)
        self._c(self._lib.pd_batch_get_cn(self.ctx, out.ctypes.data_as(C.POINTER(C.c_double)), self.stream),
                "pd_batch_get_cn")
        return out

    def rows(self, k):
        """Node indices of specimen k in the standalone order: interior rows,
        then its 6 nx boundary rows."""
        sp = self.specimens[k]
        a = np.arange(self.interior[k], self.interior[k] + sp.nx * sp.ny)
        b = self.p.N_int + np.arange(self.boundary[k], self.boundary[k + 1])
        return np.concatenate([a, b])

    def specimen_field(self, name, k, values=None):
        """Field ``name`` of specimen k (node fields), in standalone order."""
        v = self.get(name) if values is None else values
        return v[self.rows(k)]


def solve_plate_tensile(dx=0.0, nt=1000):
    """solve_plate_tensile (Solve_Plate_Tensile.cu:30-138); returns (ux, uy, dmg, result)."""
    f_dx = dx if dx > 1e-8 else 0.01
    p = derive_params(2, 1, 1, 1.0, nt, f_dx, 1.0, 0.01, 1.0, 0.5, 0.0, 200.0e9, 1.0 / 3.0, 7850, 1.0)
    n = p.N_int
    ux, uy, dmg = np.zeros(n), np.zeros(n), np.zeros(n)
    res = PDResult()
    dp = C.POINTER(C.c_double)
    check(lib().pd_solve_plate_tensile(dx, nt, ux.ctypes.data_as(dp), uy.ctypes.data_as(dp), dmg.ctypes.data_as(dp),
                                       C.byref(res)), what="pd_solve_plate_tensile")
    return ux, uy, dmg, res


def solve_plate_crack_grow(dx=0.0, nt=1250):
    """solve_plate_crack_grow (Solve_Plate_Crack_Grow.cu:167-308); returns (ux, uy, dmg, result)."""
    f_dx = dx if dx > 1e-8 else 0.0001
    p = derive_params(2, 2, 2, 1.3367e-8, nt, f_dx, 1.0, 0.0001, 0.05, 0.05, 0.0, 192.0e9, 0.3, 7850, 0.04472)
    n = p.N_int
    ux, uy, dmg = np.zeros(n), np.zeros(n), np.zeros(n)
    res = PDResult()
    dp = C.POINTER(C.c_double)
    check(lib().pd_solve_plate_crack_grow(dx, nt, ux.ctypes.data_as(dp), uy.ctypes.data_as(dp),
                                          dmg.ctypes.data_as(dp), C.byref(res)), what="pd_solve_plate_crack_grow")
    return ux, uy, dmg, res


def solve_kalthoff_winkler(dx=0.0, nt=0):
    """solve_kalthoff_winkler (Solve_Kalthoff_Winkler.cu:268-441); returns (ux, uy, uz, dmg, result)."""
    f_dx = dx if dx > 1e-8 else 0.001
    p = derive_params(3, 1, 2, 8.7e-8, nt, f_dx, 1.0, 0.001, 0.2, 0.1, 0.009, 191.0e9, 0.25, 8000, 0.01)
    cap = (p.nx + 1) * (p.ny + 1) * p.nz
    ux, uy, uz, dmg = (np.zeros(cap) for _ in range(4))
    res = PDResult()
    dp = C.POINTER(C.c_double)
    check(lib().pd_solve_kalthoff_winkler(dx, nt, ux.ctypes.data_as(dp), uy.ctypes.data_as(dp),
                                          uz.ctypes.data_as(dp), dmg.ctypes.data_as(dp), cap, C.byref(res)),
          what="pd_solve_kalthoff_winkler")
    n = res.N
    return ux[:n], uy[:n], uz[:n], dmg[:n], res
