// Test infrastructure only: a C-ABI shim over the reference's own CPU functions.
//
// This translation unit compiles the reference sources where they lie (the
// recipe in oracle/Makefile passes their directory with -I and builds with
// -DDOUBLE_PRECISION), so every function called below is the reference's code,
// unmodified.  It defines the four globals the reference's main.cu defines
// (main.cu:6-9) and wraps the host-side functions so that
// tests/golden/gen_golden.py can drive them through ctypes and record golden
// vectors.  Nothing in the product links or loads this file.
#include "Base.cuh"
#include "Coord.cu"
#include "Memory.cu"
#include "Neighbor.cu"
#include "Base_Function.cu"
#include "Surf_Corr.cu"
#include "Integrate.cu"
#include "Reduce.cu"
#include "Initial.cu"
#include "Save.cu"
#include "Force_Bond.cu"
#include "Force_State.cu"
#include "Solve_Plate_Tensile.cu"
#include "Solve_Plate_Crack_Grow.cu"
#include "Solve_Kalthoff_Winkler.cu"

__constant__ device_parameter dp;
__constant__ Cylinder_Parameter dcyp;
device_parameter p;
Cylinder_Parameter cyp;

extern "C" {

// BaseModel_Parameter (Base.cuh:72-184) + initialil_parameter (Base_Function.cu:14-36).
// dparams: pi dx emod dens pratio bc delta critical_s vol dt mass K G thick sedload
// iparams: N MN N_int nx ny nz nt
int ref_derive_params(int dim, int bs, int mode, double dt, double nt, double dx, double load,
                      double thick, double length, double height, double width, double emod,
                      double pratio, double dens, double s0, double* dparams, int* iparams) {
    Dselect d{1, dim, bs, mode};
    BaseModel_Parameter bp(d, dt, nt, dx, load, thick, length, height, width, emod, pratio, dens, s0);
    device_parameter q;
    initialil_parameter(q, bp);
    double dv[15] = {q.pi, q.dx, q.emod, q.dens, q.pratio, q.bc, q.delta, q.critical_s, q.vol,
                     q.dt, q.mass, q.K, q.G, bp.thick, bp.sedload};
    for (int k = 0; k < 15; ++k) dparams[k] = dv[k];
    int iv[7] = {q.N, q.MN, q.N_int, q.nx, q.ny, q.nz, q.nt};
    for (int k = 0; k < 7; ++k) iparams[k] = iv[k];
    return 0;
}

// Installs the device_parameter the reference CPU functions read through `p`.
void ref_set_p(double pi, int N, int MN, int N_int, int nx, int ny, int nz, double dx, double emod,
               double dens, double pratio, double bc, double delta, double critical_s, double vol,
               double dt, int nt, double mass, double K, double G) {
    p.pi = pi; p.N = N; p.MN = MN; p.N_int = N_int; p.nx = nx; p.ny = ny; p.nz = nz;
    p.dx = dx; p.emod = emod; p.dens = dens; p.pratio = pratio; p.bc = bc; p.delta = delta;
    p.critical_s = critical_s; p.vol = vol; p.dt = dt; p.nt = nt; p.mass = mass; p.K = K; p.G = G;
}

void ref_set_cylinder(double rad, double mass, double height, double v, double x, double y, double z) {
    cyp.rad = rad; cyp.mass = mass; cyp.height = height; cyp.v = v; cyp.x = x; cyp.y = y; cyp.z = z;
}

void ref_coord_plate(double* x, double* y) { Initial_coord_plate_cpu(x, y); }
void ref_coord_plate_crack(double* x, double* y) { coord_plate_crack_cpu(x, y); }
int ref_coord_kw(double* x, double* y, double* z) { return (int)coord_KW(x, y, z) + 1; }

void ref_find_neighbor_2d(const double* x, const double* y, int* NN, int* NL) { find_neighbor_2D(x, y, NN, NL); }
void ref_find_neighbor_3d(const double* x, const double* y, const double* z, int* NN, int* NL) {
    find_neighbor_3D(x, y, z, NN, NL);
}

void ref_vol_corr(int* NN, int* NL, double* x, double* y, double* z, double* idist, double* fac) {
    vol_Corr(NN, NL, x, idist, fac, y, z);
}

// surface_correct_cpu (Surf_Corr.cu:465-524); disp_* are scratch the reference overwrites.
void ref_surface_correct(int dim, int* NN, int* NL, double* x, double* y, double* z, double* dx_,
                         double* dy_, double* dz_, double* idist, double* fac, double* scr) {
    Dselect d{1, dim, 1, 1};
    BAtom ba{};
    BBond bb{};
    ba.NN = NN; ba.x = x; ba.y = y; ba.z = z; ba.disp_x = dx_; ba.disp_y = dy_; ba.disp_z = dz_;
    bb.NL = NL; bb.idist = idist; bb.fac = fac; bb.scr = scr;
    surface_correct_cpu(d, ba, bb);
}

void ref_bond_force(double* x, double* ux, double* fx, double* y, double* uy, double* fy, int* NN,
                    int* NL, double* idist, double* scr, int* fail, double* fac, double* z,
                    double* uz, double* fz) {
    bond_force_cpu(x, ux, fx, y, uy, fy, NN, NL, idist, scr, fail, fac, z, uz, fz);
}

void ref_initial_weight(double* m, int* NN, double* w, double* idist, double* fac) {
    initial_weight_cpu(m, NN, w, idist, fac);
}

void ref_state_force_2d(int* NN, double* m, double* theta, int* fail, int* NL, double* e, double* w,
                        double* idist, double* fac, double* x, double* ux, double* fx, double* y,
                        double* uy, double* fy) {
    state_force_2D_cpu(NN, m, theta, fail, NL, e, w, idist, fac, x, ux, fx, y, uy, fy);
}

double ref_cal_cn(double* fx, double* vhx, double* ux, double* fox, double* fy, double* vhy,
                  double* uy, double* foy, double* fz, double* vhz, double* uz, double* foz) {
    return cal_cn_cpu(fx, vhx, ux, fox, fy, vhy, uy, foy, fz, vhz, uz, foz);
}

void ref_static_integrate(int ct, double* fx, double* vhx, double* bx, double* vx, double* vhox,
                          double* ux, double* fox, double* fy, double* vhy, double* by, double* vy,
                          double* vhoy, double* uy, double* foy) {
    static_integrate_cpu(ct, fx, vhx, bx, vx, vhox, ux, fox, fy, vhy, by, vy, vhoy, uy, foy);
}

void ref_integrate_1(double* vx, double* ax, double* ux, double* vy, double* ay, double* uy,
                     double* vz, double* az, double* uz) {
    integrate_1(vx, ax, ux, vy, ay, uy, vz, az, uz);
}
void ref_integrate_2(double* vx, double* ax, double* fx, double* bx, double* vy, double* ay,
                     double* fy, double* by, double* vz, double* az, double* fz, double* bz) {
    integrate_2(vx, ax, fx, bx, vy, ay, fy, by, vz, az, fz, bz);
}

void ref_cal_dmg(int* NN, double* dmg, int* fail, double* fac) { cal_dmg_cpu(NN, dmg, fail, fac); }

void ref_set_crack_2d(double clength, double loc_x, double loc_y, double theta, int* NN, int* fail,
                      int* NL, double* x, double* y) {
    set_crack_2D_cpu(clength, loc_x, loc_y, theta, NN, fail, NL, x, y);
}
// Notch cut of the Kalthoff-Winkler driver (Solve_Kalthoff_Winkler.cu:65-87).
void ref_set_crack_kw(int* NN, int* NL, int* fail, double* x, double* y) { set_crack_cpu(NN, NL, fail, x, y); }

void ref_quick_load(double load, double* uy) { quick_load_cpu(load, uy); }
void ref_load_plate_tensile(double* bx) { load_plate_tensile_cpu(bx); }

void ref_contact(double* dmg, double* x, double* ux, double* vx, double* y, double* uy, double* vy,
                 double* z, double* uz, double* vz, double* force, double* cdisp) {
    contact(0, dmg, x, ux, vx, y, uy, vy, z, uz, vz, force, cdisp);
}
void ref_cy_integrate_1(double* vel, double* disp, double* acc) { cy_integrate_1(vel, disp, acc); }
void ref_cy_integrate_2(double* vel, double* acc, double* force) { cy_integrate_2(vel, acc, force); }

}  // extern "C"
