/*
 * pd_oracle.h — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's (XiaoMmingW/PD_Gpu1) peridynamics
 * algorithms, used as the checker for the GPU engine and as the timed CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may
 * load it.  The product (libpd_gb300.so) never links or calls it.
 *
 * Semantics follow the reference's GPU kernels wherever its CPU twins differ
 * (Integrate.cu:375-376 assigns instead of accumulating the damping sums;
 * Force_State.cu:345 skips broken bonds in the 2-D dilatation where the GPU
 * kernel at :65 does not).  Storage mirrors the reference: padded ELL bond
 * arrays of N*MN slots (BBond, Base.cuh:248-259) and SoA node arrays.
 * Arithmetic is written operation for operation like the reference's
 * expressions and compiled with -ffp-contract=off, so results do not depend
 * on the host's FMA contraction.  Loops over nodes run under OpenMP; each
 * node's sum runs in ascending slot order, so results do not depend on the
 * thread count.
 */
#ifndef PD_ORACLE_H
#define PD_ORACLE_H
#include <stdint.h>
#include "pd.h"

#ifdef __cplusplus
extern "C" {
#endif

int or_params_derive(pd_params* p, int dim, int model, int mode, double dt, double nt, double dx,
                     double load, double thick, double length, double height, double width,
                     double emod, double pratio, double dens, double critical_s, int fix_k3d);
int or_num_threads(void);
void or_set_threads(int n);

void or_coord_plate(const pd_params* p, double* x, double* y);
void or_coord_plate_crack(const pd_params* p, double* x, double* y);
int64_t or_coord_kw(const pd_params* p, double rad, double* x, double* y, double* z, int64_t cap);

/* Brute-force O(N^2) family, ascending rows (Neighbor.cu:42-80). Returns the
 * largest family size; rows longer than MN are truncated (counted in NN). */
int or_find_neighbor_bf(const pd_params* p, const double* x, const double* y, const double* z,
                        int* NN, int* NL);
/* Same family through a uniform cell grid (for large N); identical output. */
int or_find_neighbor_cells(const pd_params* p, const double* x, const double* y, const double* z,
                           int* NN, int* NL);

void or_vol_corr(const pd_params* p, const int* NN, const int* NL, const double* x, const double* y,
                 const double* z, double* idist, double* fac);
void or_surface_correct(const pd_params* p, const int* NN, const int* NL, const double* x,
                        const double* y, const double* z, double* idist, double* fac,
                        double* fncst_x, double* fncst_y, double* fncst_z, double* scr);

void or_bond_force(const pd_params* p, int64_t n_nodes, const double* x, const double* y,
                   const double* z, const double* ux, const double* uy, const double* uz,
                   const int* NN, const int* NL, const double* idist, const double* scr,
                   const double* fac, int* fail, double* fx, double* fy, double* fz);

void or_initial_weight(const pd_params* p, const int* NN, const double* idist, const double* fac,
                       double* w, double* m);
void or_state_theta(const pd_params* p, const double* x, const double* y, const double* z,
                    const double* ux, const double* uy, const double* uz, const int* NN,
                    const int* NL, const double* idist, const double* fac, const double* w,
                    const double* m, const int* fail, double* e, double* theta);
void or_state_force(const pd_params* p, const double* x, const double* y, const double* z,
                    const double* ux, const double* uy, const double* uz, const int* NN,
                    const int* NL, const double* idist, const double* fac, const double* w,
                    const double* m, const double* theta, const double* e, int* fail, double* fx,
                    double* fy, double* fz);

double or_adr_cn(const pd_params* p, const double* fx, const double* fy, const double* fz,
                 const double* fox, const double* foy, const double* foz, const double* vhx,
                 const double* vhy, const double* vhz, const double* ux, const double* uy,
                 const double* uz);
void or_adr_update(const pd_params* p, int ct, double cn, const double* fx, const double* fy,
                   const double* fz, const double* bx, const double* by, const double* bz,
                   double* vhx, double* vhy, double* vhz, double* vx, double* vy, double* vz,
                   double* ux, double* uy, double* uz, double* fox, double* foy, double* foz);

void or_verlet1(const pd_params* p, double* vx, double* vy, double* vz, const double* ax,
                const double* ay, const double* az, double* ux, double* uy, double* uz);
void or_verlet2(const pd_params* p, double* vx, double* vy, double* vz, double* ax, double* ay,
                double* az, const double* fx, const double* fy, const double* fz, const double* bx,
                const double* by, const double* bz);

void or_damage(const pd_params* p, const int* NN, const int* fail, const double* fac, double* dmg);
void or_set_crack_2d(const pd_params* p, double clength, double loc_x, double loc_y, double theta,
                     const int* NN, const int* NL, const double* x, const double* y, int* fail);
void or_set_crack_kw(const pd_params* p, double rad, const int* NN, const int* NL, const double* x,
                     const double* y, int* fail);
void or_quick_load(const pd_params* p, double load, double* uy);
void or_load_plate_tensile(const pd_params* p, double* bx);

void or_contact(const pd_params* p, const pd_cylinder* cyl, const double* dmg, const double* x,
                const double* y, const double* z, double* ux, double* uy, double* uz, double* vx,
                double* vy, double* vz, double* force);
void or_cy_integrate1(const pd_params* p, pd_cylinder* cyl);
void or_cy_integrate2(const pd_params* p, pd_cylinder* cyl);

#ifdef __cplusplus
}
#endif
#endif
