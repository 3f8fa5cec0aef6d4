"""Generate golden vectors from the reference's own CPU functions.

Run in a container that has the reference sources (they are not needed at test
time):

    make -C oracle ref            # builds oracle/_ref/libpdref.so from the reference .cu files
    python tests/golden/gen_golden.py

The shim (oracle/ref_harness.cu) compiles XiaoMmingW/PD_Gpu1's sources with
-DDOUBLE_PRECISION and calls its host-side functions unmodified; this script
records their inputs and outputs as compressed .npz fixtures beside it.  Every
fixture stores the parameter block the reference derived
(BaseModel_Parameter, Base.cuh:72-184) so the tests can check the derivation
too.  Bond arrays are stored in CSR order (the used slots of each ELL row).

Semantics the reference's CPU functions do not share with its GPU kernels are
avoided here rather than recorded: the 2-D state-based dilatation is only
recorded with every bond intact (Force_State.cu:345 vs :65), and the ADR
update with a damping coefficient only for one integrated node
(Integrate.cu:375-376 assigns instead of accumulating; with one node both agree).
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref", "libpdref.so")

D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)
NULL_D = C.cast(None, D)

lib = C.CDLL(REF)
lib.ref_derive_params.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_double] * 12 + [D, I]
lib.ref_set_p.argtypes = [C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int] + [C.c_double] * 9 + [
    C.c_int, C.c_double, C.c_double, C.c_double]
lib.ref_set_cylinder.argtypes = [C.c_double] * 7
lib.ref_coord_kw.restype = C.c_int
lib.ref_cal_cn.restype = C.c_double
lib.ref_set_crack_2d.argtypes = [C.c_double] * 4 + [I, I, I, D, D]
lib.ref_quick_load.argtypes = [C.c_double, D]

DKEYS = ["pi", "dx", "emod", "dens", "pratio", "bc", "delta", "critical_s", "vol", "dt", "mass", "K", "G",
         "thick", "sedload"]
IKEYS = ["N", "MN", "N_int", "nx", "ny", "nz", "nt"]


def d(a):
    return a.ctypes.data_as(D)


def i(a):
    return a.ctypes.data_as(I)


def derive(dim, bs, mode, dt, nt, dx, load, thick, length, height, width, emod, pratio, dens, s0):
    dv = np.zeros(15)
    iv = np.zeros(7, dtype=np.int32)
    lib.ref_derive_params(dim, bs, mode, dt, nt, dx, load, thick, length, height, width, emod, pratio, dens, s0,
                          d(dv), i(iv))
    prm = dict(zip(DKEYS, dv.tolist()))
    prm.update(dict(zip(IKEYS, iv.tolist())))
    prm["inputs"] = dict(dim=dim, bs=bs, mode=mode, dt=dt, nt=nt, dx=dx, load=load, thick=thick, length=length,
                         height=height, width=width, emod=emod, pratio=pratio, dens=dens, s0=s0)
    return prm


def set_p(prm):
    lib.ref_set_p(prm["pi"], prm["N"], prm["MN"], prm["N_int"], prm["nx"], prm["ny"], prm["nz"], prm["dx"],
                  prm["emod"], prm["dens"], prm["pratio"], prm["bc"], prm["delta"], prm["critical_s"], prm["vol"],
                  prm["dt"], prm["nt"], prm["mass"], prm["K"], prm["G"])


def csr(arr, NN, MN):
    a = arr.reshape(len(NN), MN)
    return a[np.arange(MN)[None, :] < NN[:, None]]


def pack_params(prm):
    out = {}
    for k in DKEYS:
        out["p_" + k] = np.float64(prm[k])
    for k in IKEYS:
        out["p_" + k] = np.int64(prm[k])
    for k, v in prm["inputs"].items():
        out["in_" + k] = np.float64(v)
    return out


def zeros(n):
    return np.zeros(n, dtype=np.float64)


def plate_tensile_bond():
    """2-D PMB plate, the tensile driver's setup (Solve_Plate_Tensile.cu:40-41) scaled down."""
    prm = derive(2, 1, 1, 1.0, 1000, 0.01, 1.0, 0.01, 0.2, 0.1, 0.0, 200.0e9, 1.0 / 3.0, 7850, 1.0)
    set_p(prm)
    N, MN = prm["N"], prm["MN"]
    x, y = zeros(N), zeros(N)
    lib.ref_coord_plate(d(x), d(y))
    NN = np.zeros(N, dtype=np.int32)
    NL = np.zeros(N * MN, dtype=np.int32)
    lib.ref_find_neighbor_2d(d(x), d(y), i(NN), i(NL))
    idist, fac, scr = zeros(N * MN), zeros(N * MN), zeros(N * MN)
    ux, uy = zeros(N), zeros(N)
    lib.ref_surface_correct(2, i(NN), i(NL), d(x), d(y), NULL_D, d(ux), d(uy), NULL_D, d(idist), d(fac), d(scr))
    out = pack_params(prm)
    out.update(x=x, y=y, NN=NN, NL=csr(NL, NN, MN), idist=csr(idist, NN, MN), fac=csr(fac, NN, MN),
               scr=csr(scr, NN, MN))
    # body-force loading of the tensile driver (Solve_Plate_Tensile.cu:19-26)
    bx = zeros(N)
    lib.ref_load_plate_tensile(d(bx))
    out["bx"] = bx
    # forces for a seeded displacement field: uniform stretch + noise
    rng = np.random.default_rng(1234)
    ux = (2e-3 * x + 1e-5 * rng.standard_normal(N) * prm["dx"]).astype(np.float64)
    uy = (-1e-3 * y + 1e-5 * rng.standard_normal(N) * prm["dx"]).astype(np.float64)
    fail = np.ones(N * MN, dtype=np.int32)
    fx, fy = zeros(N), zeros(N)
    lib.ref_bond_force(d(x), d(ux), d(fx), d(y), d(uy), d(fy), i(NN), i(NL), d(idist), d(scr), i(fail), d(fac),
                       NULL_D, NULL_D, NULL_D)
    out.update(f_ux=ux, f_uy=uy, f_fx=fx, f_fy=fy, f_fail=csr(fail, NN, MN))
    # breakage: critical stretch lowered so that part of the family breaks
    prm_b = dict(prm)
    prm_b["critical_s"] = 1.5e-3
    set_p(prm_b)
    fail = np.ones(N * MN, dtype=np.int32)
    fx2, fy2 = zeros(N), zeros(N)
    lib.ref_bond_force(d(x), d(ux), d(fx2), d(y), d(uy), d(fy2), i(NN), i(NL), d(idist), d(scr), i(fail), d(fac),
                       NULL_D, NULL_D, NULL_D)
    fx3, fy3 = zeros(N), zeros(N)
    lib.ref_bond_force(d(x), d(ux), d(fx3), d(y), d(uy), d(fy3), i(NN), i(NL), d(idist), d(scr), i(fail), d(fac),
                       NULL_D, NULL_D, NULL_D)
    out.update(b_s0=np.float64(1.5e-3), b_fx1=fx2, b_fy1=fy2, b_fx2=fx3, b_fy2=fy3, b_fail=csr(fail, NN, MN))
    dmg = zeros(N)
    lib.ref_cal_dmg(i(NN), d(dmg), i(fail), d(fac))
    out["b_dmg"] = dmg
    set_p(prm)
    # ADR: damping coefficient (cal_cn_cpu, Integrate.cu:269-307) on a seeded state
    vhx = 1e-9 * rng.standard_normal(N)
    vhy = 1e-9 * rng.standard_normal(N)
    vhy[::7] = 0.0  # exercises the velhalfold == 0 guard
    fox = fx * (1 + 1e-3 * rng.standard_normal(N))
    foy = fy * (1 + 1e-3 * rng.standard_normal(N))
    cn = lib.ref_cal_cn(d(fx), d(vhx), d(ux), d(fox), d(fy), d(vhy), d(uy), d(foy), NULL_D, NULL_D, NULL_D, NULL_D)
    out.update(a_vhx=vhx, a_vhy=vhy, a_fox=fox, a_foy=foy, a_cn=np.float64(cn))
    # ADR update at ct = 0 over all nodes (static_integrate_cpu, Integrate.cu:362-445)
    st = dict(vh=[zeros(N), zeros(N)], v=[zeros(N), zeros(N)], u=[ux.copy(), uy.copy()], fo=[zeros(N), zeros(N)])
    vhn = [zeros(N), zeros(N)]
    lib.ref_static_integrate(0, d(fx), d(vhn[0]), d(bx), d(st["v"][0]), d(st["vh"][0]), d(st["u"][0]),
                             d(st["fo"][0]), d(fy), d(vhn[1]), d(zeros(N)), d(st["v"][1]), d(st["vh"][1]),
                             d(st["u"][1]), d(st["fo"][1]))
    out.update(a0_ux=st["u"][0], a0_uy=st["u"][1], a0_vx=st["v"][0], a0_vy=st["v"][1], a0_vhx=st["vh"][0],
               a0_vhy=st["vh"][1], a0_fox=st["fo"][0], a0_foy=st["fo"][1])
    # ADR update at ct = 5 restricted to one integrated node, where the CPU
    # damping sum equals the GPU one.
    prm1 = dict(prm)
    prm1["N_int"] = 1
    set_p(prm1)
    n1 = {k: v[:1].copy() for k, v in dict(fx=fx, fy=fy, bx=bx, ux=ux, uy=uy, vhx=vhx, vhy=vhy, fox=fox,
                                            foy=foy).items()}
    n1["vhy"][0] = 3e-9
    vh1 = [zeros(1), zeros(1)]
    v1 = [zeros(1), zeros(1)]
    u1 = [n1["ux"].copy(), n1["uy"].copy()]
    vho1 = [n1["vhx"].copy(), n1["vhy"].copy()]
    fo1 = [n1["fox"].copy(), n1["foy"].copy()]
    lib.ref_static_integrate(5, d(n1["fx"]), d(vh1[0]), d(n1["bx"]), d(v1[0]), d(vho1[0]), d(u1[0]), d(fo1[0]),
                             d(n1["fy"]), d(vh1[1]), d(zeros(1)), d(v1[1]), d(vho1[1]), d(u1[1]), d(fo1[1]))
    out.update(a1_vhy_in=np.float64(3e-9), a1_ux=u1[0], a1_uy=u1[1], a1_vx=v1[0], a1_vy=v1[1], a1_vhx=vho1[0],
               a1_vhy=vho1[1])
    set_p(prm)
    return out


def plate_crack_state():
    """2-D state-based plate with boundary rows, the crack-grow driver's setup
    (Solve_Plate_Crack_Grow.cu:177-179) scaled down."""
    prm = derive(2, 2, 2, 1.3367e-8, 1250, 1e-4, 1.0, 1e-4, 0.002, 0.002, 0.0, 192.0e9, 0.3, 7850, 0.04472)
    prm["N"] += 6 * prm["nx"]
    set_p(prm)
    N, MN, N_int = prm["N"], prm["MN"], prm["N_int"]
    x, y = zeros(N), zeros(N)
    lib.ref_coord_plate_crack(d(x), d(y))
    NN = np.zeros(N, dtype=np.int32)
    NL = np.zeros(N * MN, dtype=np.int32)
    lib.ref_find_neighbor_2d(d(x), d(y), i(NN), i(NL))
    idist, fac = zeros(N * MN), zeros(N * MN)
    lib.ref_vol_corr(i(NN), i(NL), d(x), d(y), NULL_D, d(idist), d(fac))
    w, m = zeros(N * MN), zeros(N)
    lib.ref_initial_weight(d(m), i(NN), d(w), d(idist), d(fac))
    out = pack_params(prm)
    out.update(x=x, y=y, NN=NN, NL=csr(NL, NN, MN), idist=csr(idist, NN, MN), fac=csr(fac, NN, MN),
               w=csr(w, NN, MN), m=m)
    # pre-cracks (kernel_set_crack_2D / set_crack_2D_cpu, Base_Function.cu:39-123)
    for name, (cl, lx, ly, th) in dict(c0=(0.001, 0.0, 0.0, 0.0), c90=(0.0008, 0.0, 1e-5, np.pi / 2),
                                        c30=(0.0012, -2e-4, 1e-4, np.pi / 6)).items():
        fail = np.ones(N_int * MN, dtype=np.int32)
        lib.ref_set_crack_2d(cl, lx, ly, th, i(NN), i(fail), i(NL), d(x), d(y))
        out[name + "_fail"] = csr(fail, NN[:N_int], MN)
        out[name + "_args"] = np.array([cl, lx, ly, th])
        dmg = zeros(N_int)
        lib.ref_cal_dmg(i(NN), d(dmg), i(fail), d(fac))
        out[name + "_dmg"] = dmg
    # explicit steps with every bond intact: quick_load + Verlet + state force
    ux, uy, vx, vy, ax, ay, fx, fy, bx, by = (zeros(N) for _ in range(10))
    theta = zeros(N)
    e = zeros(N * MN)
    # state_force_2D_cpu reads fail[i*MN+j] for every node i < N (Force_State.cu:345)
    fail = np.ones(N * MN, dtype=np.int32)
    for step in range(12):
        lib.ref_quick_load(20.0, d(uy))
        lib.ref_integrate_1(d(vx), d(ax), d(ux), d(vy), d(ay), d(uy), NULL_D, NULL_D, NULL_D)
        lib.ref_state_force_2d(i(NN), d(m), d(theta), i(fail), i(NL), d(e), d(w), d(idist), d(fac), d(x), d(ux),
                               d(fx), d(y), d(uy), d(fy))
        lib.ref_integrate_2(d(vx), d(ax), d(fx), d(bx), d(vy), d(ay), d(fy), d(by), NULL_D, NULL_D, NULL_D, NULL_D)
    out.update(s_steps=np.int64(12), s_load=np.float64(20.0), s_ux=ux, s_uy=uy, s_vx=vx, s_vy=vy, s_ax=ax, s_ay=ay,
               s_fx=fx, s_fy=fy, s_theta=theta.copy(), s_e=csr(e, NN, MN))
    # one state-force evaluation on a stretched field (larger forces, breaks at lowered s0)
    rng = np.random.default_rng(99)
    ux2 = 3e-3 * x + 2e-6 * prm["dx"] * rng.standard_normal(N)
    uy2 = 1e-3 * y + 2e-6 * prm["dx"] * rng.standard_normal(N)
    prm_b = dict(prm)
    prm_b["critical_s"] = 2.5e-3
    set_p(prm_b)
    fx2, fy2 = zeros(N), zeros(N)
    fail2 = np.ones(N * MN, dtype=np.int32)
    lib.ref_state_force_2d(i(NN), d(m), d(theta), i(fail2), i(NL), d(e), d(w), d(idist), d(fac), d(x), d(ux2),
                           d(fx2), d(y), d(uy2), d(fy2))
    out.update(t_s0=np.float64(2.5e-3), t_ux=ux2, t_uy=uy2, t_fx=fx2, t_fy=fy2, t_theta=theta.copy(),
               t_fail=csr(fail2[:N_int * MN], NN[:N_int], MN))
    set_p(prm)
    return out


def kalthoff_winkler_bond():
    """3-D PMB notched slab, the Kalthoff-Winkler driver's setup
    (Solve_Kalthoff_Winkler.cu:280-296) scaled down; notches at x = +-rad."""
    rad = 0.015
    prm = derive(3, 1, 2, 8.7e-8, 0, 0.003, 1.0, 0.003, 0.06, 0.1, 0.009, 191.0e9, 0.25, 8000, 0.01)
    prm["nx"] += 1
    prm["ny"] += 1
    prm["N"] = prm["nx"] * prm["ny"] * prm["nz"]
    cyl = dict(rad=rad, mass=1.57, height=0.05, v=-32.0, x=0.0, y=0.1 / 2.0 + 0.05 / 2.0 + 0.1 * prm["dx"], z=0.0)
    lib.ref_set_cylinder(cyl["rad"], cyl["mass"], cyl["height"], cyl["v"], cyl["x"], cyl["y"], cyl["z"])
    set_p(prm)
    cap = prm["N"]
    x, y, z = zeros(cap), zeros(cap), zeros(cap)
    n = lib.ref_coord_kw(d(x), d(y), d(z))
    prm["N"] = prm["N_int"] = n
    set_p(prm)
    x, y, z = x[:n].copy(), y[:n].copy(), z[:n].copy()
    N, MN = n, prm["MN"]
    NN = np.zeros(N, dtype=np.int32)
    NL = np.zeros(N * MN, dtype=np.int32)
    lib.ref_find_neighbor_3d(d(x), d(y), d(z), i(NN), i(NL))
    idist, fac, scr = zeros(N * MN), zeros(N * MN), zeros(N * MN)
    ux, uy, uz = zeros(N), zeros(N), zeros(N)
    lib.ref_surface_correct(3, i(NN), i(NL), d(x), d(y), d(z), d(ux), d(uy), d(uz), d(idist), d(fac), d(scr))
    w, m = zeros(N * MN), zeros(N)
    lib.ref_initial_weight(d(m), i(NN), d(w), d(idist), d(fac))
    out = pack_params(prm)
    out.update(rad=np.float64(rad), x=x, y=y, z=z, NN=NN, NL=csr(NL, NN, MN), idist=csr(idist, NN, MN),
               fac=csr(fac, NN, MN), scr=csr(scr, NN, MN), w=csr(w, NN, MN), m=m)
    for k, v in cyl.items():
        out["cyl_" + k] = np.float64(v)
    fail = np.ones(N * MN, dtype=np.int32)
    lib.ref_set_crack_kw(i(NN), i(NL), i(fail), d(x), d(y))
    out["kw_fail"] = csr(fail, NN, MN)
    # 3-D bond forces on a seeded field, lowered s0 so the y >= -0.04 guard matters
    rng = np.random.default_rng(7)
    ux = 1e-3 * x + 1e-6 * prm["dx"] * rng.standard_normal(N)
    uy = 4e-3 * y + 1e-6 * prm["dx"] * rng.standard_normal(N)
    uz = -1e-3 * z + 1e-6 * prm["dx"] * rng.standard_normal(N)
    prm_b = dict(prm)
    prm_b["critical_s"] = 3.0e-3
    set_p(prm_b)
    fx, fy, fz = zeros(N), zeros(N), zeros(N)
    fail_b = fail.copy()
    lib.ref_bond_force(d(x), d(ux), d(fx), d(y), d(uy), d(fy), i(NN), i(NL), d(idist), d(scr), i(fail_b), d(fac),
                       d(z), d(uz), d(fz))
    out.update(f_s0=np.float64(3.0e-3), f_ux=ux, f_uy=uy, f_uz=uz, f_fx=fx, f_fy=fy, f_fz=fz,
               f_fail=csr(fail_b, NN, MN))
    dmg = zeros(N)
    lib.ref_cal_dmg(i(NN), d(dmg), i(fail_b), d(fac))
    out["f_dmg"] = dmg
    set_p(prm)
    # contact with the rigid cylinder pushed into the top edge, then cylinder integration
    dmg0 = zeros(N)
    cux, cuy, cuz = zeros(N), zeros(N), zeros(N)
    cvx, cvy, cvz = zeros(N), zeros(N), zeros(N)
    cvy[:] = 1e-3
    force = zeros(3)
    cdisp = np.array([0.0, -0.1 * prm["dx"] - 1.0e-3, 0.0])
    lib.ref_contact(d(dmg0), d(x), d(cux), d(cvx), d(y), d(cuy), d(cvy), d(z), d(cuz), d(cvz), d(force), d(cdisp))
    out.update(c_cdisp=cdisp, c_ux=cux, c_uy=cuy, c_uz=cuz, c_vx=cvx, c_vy=cvy, c_vz=cvz, c_force=force.copy())
    cvel = np.array([0.0, -32.0, 0.0])
    cacc = np.array([0.0, 1.0, 0.0])
    cdisp2 = cdisp.copy()
    lib.ref_cy_integrate_2(d(cvel), d(cacc), d(force))
    lib.ref_cy_integrate_1(d(cvel), d(cdisp2), d(cacc))
    out.update(cy_vel=cvel, cy_acc=cacc, cy_disp=cdisp2, cy_force=force)
    # Verlet halves in 3-D (integrate_1/2, Integrate.cu:447-481)
    vx, vy, vz = (1e-3 * rng.standard_normal(N) for _ in range(3))
    ax, ay, az = (1e3 * rng.standard_normal(N) for _ in range(3))
    out.update(v_vx0=vx.copy(), v_vy0=vy.copy(), v_vz0=vz.copy(), v_ax0=ax.copy(), v_ay0=ay.copy(), v_az0=az.copy())
    uxv, uyv, uzv = zeros(N), zeros(N), zeros(N)
    lib.ref_integrate_1(d(vx), d(ax), d(uxv), d(vy), d(ay), d(uyv), d(vz), d(az), d(uzv))
    lib.ref_integrate_2(d(vx), d(ax), d(fx), d(zeros(N)), d(vy), d(ay), d(fy), d(zeros(N)), d(vz), d(az), d(fz),
                        d(zeros(N)))
    out.update(v_ux=uxv, v_uy=uyv, v_uz=uzv, v_vx=vx, v_vy=vy, v_vz=vz, v_ax=ax, v_ay=ay, v_az=az)
    return out


def neighbor_medium():
    """A larger 2-D family (9,600 nodes) and a 3-D one, brute force."""
    prm = derive(2, 1, 1, 1.0, 1, 0.01, 1.0, 0.01, 1.2, 0.8, 0.0, 200.0e9, 1.0 / 3.0, 7850, 1.0)
    set_p(prm)
    N, MN = prm["N"], prm["MN"]
    x, y = zeros(N), zeros(N)
    lib.ref_coord_plate(d(x), d(y))
    NN = np.zeros(N, dtype=np.int32)
    NL = np.zeros(N * MN, dtype=np.int32)
    lib.ref_find_neighbor_2d(d(x), d(y), i(NN), i(NL))
    out = {("n2_" + k): v for k, v in pack_params(prm).items()}
    out.update(n2_NN=NN, n2_NL=csr(NL, NN, MN))
    prm3 = derive(3, 1, 2, 1e-7, 1, 0.001, 1.0, 0.001, 0.016, 0.012, 0.009, 191.0e9, 0.25, 8000, 0.01)
    set_p(prm3)
    N3, MN3 = prm3["N"], prm3["MN"]
    x3, y3, z3 = zeros(N3), zeros(N3), zeros(N3)
    nx, ny, nz = prm3["nx"], prm3["ny"], prm3["nz"]
    k = 0
    for kz in range(nz):
        for jy in range(ny):
            for ix in range(nx):
                x3[k] = (-nx / 2.0 + 0.5 + ix) * prm3["dx"]
                y3[k] = (-ny / 2.0 + 0.5 + jy) * prm3["dx"]
                z3[k] = (-nz / 2.0 + 0.5 + kz) * prm3["dx"]
                k += 1
    NN3 = np.zeros(N3, dtype=np.int32)
    NL3 = np.zeros(N3 * MN3, dtype=np.int32)
    lib.ref_find_neighbor_3d(d(x3), d(y3), d(z3), i(NN3), i(NL3))
    out.update({("n3_" + k): v for k, v in pack_params(prm3).items()})
    out.update(n3_x=x3, n3_y=y3, n3_z=z3, n3_NN=NN3, n3_NL=csr(NL3, NN3, MN3))
    return out


def main():
    cases = dict(plate_tensile_bond=plate_tensile_bond, plate_crack_state=plate_crack_state,
                 kalthoff_winkler_bond=kalthoff_winkler_bond, neighbor_medium=neighbor_medium)
    only = sys.argv[1:]
    for name, fn in cases.items():
        if only and name not in only:
            continue
        out = fn()
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **out)
        print(f"{name}: {len(out)} arrays -> {os.path.getsize(path) / 1024:.1f} KiB")


if __name__ == "__main__":
    main()
