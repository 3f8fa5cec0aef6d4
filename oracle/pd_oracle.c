/*
 * pd_oracle.c — TEST INFRASTRUCTURE ONLY (the oracle; see pd_oracle.h).
 *
 * Plain-C restatement of the reference's peridynamics algorithms
 * (XiaoMmingW/PD_Gpu1).  Each function cites the reference lines it follows.
 * Expressions keep the reference's operand order so that, with
 * -ffp-contract=off, every rounding step is the reference's; where the
 * reference sums with warp shuffles or atomics, the oracle sums in ascending
 * slot order.
 */
#include "pd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline double sq(double v) { return v * v; }

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* BaseModel_Parameter::cal_parameter (Base.cuh:114-183) and
 * initialil_parameter (Base_Function.cu:14-36). */
int or_params_derive(pd_params* p, int dim, int model, int mode, double dt, double nt, double dx,
                     double load, double thick, double length, double height, double width,
                     double emod, double pratio, double dens, double critical_s, int fix_k3d) {
    if (!p || (dim != 2 && dim != 3) || (model != PD_MODEL_BOND && model != PD_MODEL_STATE)) return PD_ERR_ARG;
    memset(p, 0, sizeof(*p));
    const double pi = acos(-1.0); /* Base.cuh:31 */
    p->pi = pi;
    p->dim = dim;
    p->model = model;
    p->mode = mode;
    p->dt = dt;
    p->nt = (int32_t)nt;
    p->dx = dx;
    p->load = load;
    p->length = length;
    p->height = height;
    p->width = width;
    p->emod = emod;
    p->pratio = pratio;
    p->dens = dens;
    p->critical_s = critical_s;
    p->delta = 3.015 * dx;
    p->nx = (int32_t)((length - dx / 2.0) / dx + 1);
    p->ny = (int32_t)((height - dx / 2.0) / dx + 1);
    p->nz = dim == 3 ? (int32_t)((width - dx / 2.0) / dx + 1) : 0;
    p->MN = dim == 2 ? 32 : 128; /* MN_2D, MN_3D (Base.cuh:27-29) */
    p->N = p->N_int = dim == 2 ? p->nx * p->ny : p->nx * p->ny * p->nz;
    p->break_ymin = dim == 3 ? -0.04 : -1e300;
    p->sedload = dim == 3 ? 0.6 * emod * 1.0e-6 : 0.5 * emod / (1.0 - pratio * pratio) * 1.0e-6;
    const double delta = p->delta;
    if (model == PD_MODEL_BOND) {
        p->thick = thick;
        if (dim == 2) {
            p->vol = dx * dx * thick;
            p->bc = 6.0 * emod / (pi * thick * (delta * delta * delta) * (1.0 - pratio));
        } else {
            p->vol = dx * dx * dx;
            p->bc = 6.0 * emod / (pi * delta * (delta * delta * delta) * (1.0 - 2.0 * pratio));
        }
        p->mass = 0.25 * dt * dt * (pi * delta * delta * thick) * (p->bc) / dx * 5.0;
    } else {
        p->G = 0.5 * emod / (1 + pratio);
        if (dim == 2) {
            p->thick = dx; /* Base.cuh:166 overrides the thickness */
            p->vol = dx * dx * p->thick;
            p->K = 0.5 * emod / (1 - pratio);
        } else {
            p->thick = thick;
            p->K = fix_k3d ? emod / (3.0 * (1.0 - 2.0 * pratio)) : emod / 3.0 / (1 - 2.0 * p->G);
            p->vol = dx * dx * dx;
        }
        p->mass = 0.0;
    }
    return PD_OK;
}

/* Initial_coord_plate_cpu (Coord.cu:19-28). */
void or_coord_plate(const pd_params* p, double* x, double* y) {
    for (int i = 0; i < p->ny; i++)
        for (int j = 0; j < p->nx; j++) {
            x[i * p->nx + j] = (-p->nx / 2.0 + 0.5 + j) * p->dx;
            y[i * p->nx + j] = (-p->ny / 2.0 + 0.5 + i) * p->dx;
        }
}

/* kernel_coord_plate_crack (Coord.cu:34-45): interior, 3 rows above, 3 below. */
void or_coord_plate_crack(const pd_params* p, double* x, double* y) {
    const int64_t top = (int64_t)p->N_int + 3 * (int64_t)p->nx;
    for (int64_t idx = 0; idx < p->N; idx++) {
        x[idx] = (-p->nx / 2.0 + 0.5 + (double)(idx % p->nx)) * p->dx;
        if (idx < top)
            y[idx] = (-p->ny / 2.0 + 0.5 + (double)(idx / p->nx)) * p->dx;
        else
            y[idx] = (-p->ny / 2.0 - 0.5 - (double)((idx - p->N_int - 3 * (int64_t)p->nx) / p->nx)) * p->dx;
    }
}

/* coord_KW (Coord.cu:77-129): regular slab minus two notch strips at x=+-rad
 * in the upper half.  Returns the node count (the reference returns count-1). */
int64_t or_coord_kw(const pd_params* p, double rad, double* x, double* y, double* z, int64_t cap) {
    int64_t num = 0;
    for (int k = 0; k < p->nz; k++)
        for (int j = 0; j < p->ny; j++)
            for (int i = 0; i < p->nx; i++) {
                const double tx = (-(p->nx - 1) / 2.0 + i) * p->dx;
                const double ty = (-(p->ny - 1) / 2.0 + j) * p->dx;
                const double tz = (-p->nz / 2.0 + 0.5 + k) * p->dx;
                int keep;
                if (tx > (-rad - 1.1 * p->dx) && tx < (-rad + 0.1 * p->dx))
                    keep = ty < -1.0e-10;
                else if (tx > (rad - 0.1 * p->dx) && tx < (rad + 1.1 * p->dx))
                    keep = ty < -1.0e-10;
                else
                    keep = 1;
                if (keep) {
                    if (num < cap) {
                        x[num] = tx;
                        y[num] = ty;
                        z[num] = tz;
                    }
                    num++;
                }
            }
    return num;
}

/* The family predicate of find_neighbor_2D/3D (Neighbor.cu:51, :72).
 * (b-a)^2 == (a-b)^2 exactly, so the test is symmetric in i and j. */
static inline int in_family(const pd_params* p, const double* x, const double* y, const double* z,
                            int64_t i, int64_t j) {
    if (p->dim == 2) return sq(x[j] - x[i]) + sq(y[j] - y[i]) < p->delta * p->delta;
    return sq(x[j] - x[i]) + sq(y[j] - y[i]) + sq(z[j] - z[i]) < p->delta * p->delta;
}

/* find_neighbor_2D/3D (Neighbor.cu:42-80): row i lists every j != i in
 * ascending order, which is the order the reference's serial double loop
 * produces.  Rows are computed independently (one per thread). */
int or_find_neighbor_bf(const pd_params* p, const double* x, const double* y, const double* z,
                        int* NN, int* NL) {
    const int64_t N = p->N;
    const int MN = p->MN;
    int maxnn = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(max : maxnn)
    for (int64_t i = 0; i < N; i++) {
        int c = 0;
        for (int64_t j = 0; j < N; j++) {
            if (j == i) continue;
            if (in_family(p, x, y, z, i, j)) {
                if (c < MN) NL[i * MN + c] = (int)j;
                c++;
            }
        }
        NN[i] = c;
        if (c > maxnn) maxnn = c;
    }
    return maxnn;
}

static int cmp_int(const void* a, const void* b) {
    const int u = *(const int*)a, v = *(const int*)b;
    return (u > v) - (u < v);
}

/* Cell-grid variant of the same family (same predicate, same sorted rows). */
int or_find_neighbor_cells(const pd_params* p, const double* x, const double* y, const double* z,
                           int* NN, int* NL) {
    const int64_t N = p->N;
    const int MN = p->MN;
    const int dim = p->dim;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = 0; i < N; i++) {
        const double c[3] = {x[i], y[i], dim == 3 ? z[i] : 0.0};
        for (int a = 0; a < 3; a++) {
            if (c[a] < lo[a]) lo[a] = c[a];
            if (c[a] > hi[a]) hi[a] = c[a];
        }
    }
    const double h = p->delta * 1.0001; /* cell edge >= horizon */
    int64_t nc[3];
    for (int a = 0; a < 3; a++) nc[a] = (a < dim) ? (int64_t)floor((hi[a] - lo[a]) / h) + 1 : 1;
    const int64_t ncell = nc[0] * nc[1] * nc[2];
    int64_t* start = (int64_t*)calloc((size_t)ncell + 1, sizeof(int64_t));
    int64_t* cellof = (int64_t*)malloc((size_t)N * sizeof(int64_t));
    int64_t* order = (int64_t*)malloc((size_t)N * sizeof(int64_t));
    for (int64_t i = 0; i < N; i++) {
        const double c[3] = {x[i], y[i], dim == 3 ? z[i] : 0.0};
        int64_t k[3];
        for (int a = 0; a < 3; a++) {
            k[a] = (a < dim) ? (int64_t)floor((c[a] - lo[a]) / h) : 0;
            if (k[a] >= nc[a]) k[a] = nc[a] - 1;
        }
        cellof[i] = (k[2] * nc[1] + k[1]) * nc[0] + k[0];
        start[cellof[i] + 1]++;
    }
    for (int64_t c = 0; c < ncell; c++) start[c + 1] += start[c];
    {
        int64_t* fill = (int64_t*)malloc((size_t)ncell * sizeof(int64_t));
        memcpy(fill, start, (size_t)ncell * sizeof(int64_t));
        for (int64_t i = 0; i < N; i++) order[fill[cellof[i]]++] = i;
        free(fill);
    }
    int maxnn = 0;
#pragma omp parallel reduction(max : maxnn)
    {
        int cap = 4 * MN;
        int* buf = (int*)malloc((size_t)cap * sizeof(int));
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < N; i++) {
            const int64_t ci = cellof[i];
            const int64_t k0 = ci % nc[0], k1 = (ci / nc[0]) % nc[1], k2 = ci / (nc[0] * nc[1]);
            int c = 0;
            for (int64_t d2 = -1; d2 <= 1; d2++)
                for (int64_t d1 = -1; d1 <= 1; d1++)
                    for (int64_t d0 = -1; d0 <= 1; d0++) {
                        const int64_t a0 = k0 + d0, a1 = k1 + d1, a2 = k2 + d2;
                        if (a0 < 0 || a1 < 0 || a2 < 0 || a0 >= nc[0] || a1 >= nc[1] || a2 >= nc[2]) continue;
                        const int64_t cc = (a2 * nc[1] + a1) * nc[0] + a0;
                        for (int64_t t = start[cc]; t < start[cc + 1]; t++) {
                            const int64_t j = order[t];
                            if (j == i || !in_family(p, x, y, z, i, j)) continue;
                            if (c == cap) {
                                cap *= 2;
                                buf = (int*)realloc(buf, (size_t)cap * sizeof(int));
                            }
                            buf[c++] = (int)j;
                        }
                    }
            qsort(buf, (size_t)c, sizeof(int), cmp_int);
            for (int t = 0; t < c && t < MN; t++) NL[i * MN + t] = buf[t];
            NN[i] = c;
            if (c > maxnn) maxnn = c;
        }
        free(buf);
    }
    free(start);
    free(cellof);
    free(order);
    return maxnn;
}

/* kernel_vol_Corr (Surf_Corr.cu:7-35). */
void or_vol_corr(const pd_params* p, const int* NN, const int* NL, const double* x, const double* y,
                 const double* z, double* idist, double* fac) {
    const int MN = p->MN;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p->N; i++)
        for (int j = 0; j < NN[i]; j++) {
            const int64_t idx = i * MN + j;
            const int64_t c = NL[idx];
            if (p->dim == 2)
                idist[idx] = sqrt(sq(x[c] - x[i]) + sq(y[c] - y[i]));
            else
                idist[idx] = sqrt(sq(x[c] - x[i]) + sq(y[c] - y[i]) + sq(z[c] - z[i]));
            if (idist[idx] <= p->delta - p->dx / 2.0)
                fac[idx] = 1.0;
            else if (idist[idx] <= p->delta + p->dx / 2.0)
                fac[idx] = (p->delta + p->dx / 2.0 - idist[idx]) / p->dx;
            else
                fac[idx] = 0.0;
        }
}

/* kernel_surface_F / kernel_surface_F_3D (Surf_Corr.cu:53-158) for the test
 * field u_axis = 0.001*coord_axis (kernel_Disp, :38-50), other components 0. */
static void surface_factor(const pd_params* p, int axis, const int* NN, const int* NL, const double* x,
                           const double* y, const double* z, const double* idist, const double* fac,
                           double* fncst) {
    const int MN = p->MN;
    const double sedload = p->dim == 3 ? 0.6 * p->emod * 1.0e-6
                                       : 0.5 * p->emod / (1.0 - p->pratio * p->pratio) * 1.0e-6;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p->N; i++) {
        const double uxi = axis == 0 ? 0.001 * x[i] : 0.0;
        const double uyi = axis == 1 ? 0.001 * y[i] : 0.0;
        const double uzi = (axis == 2) ? 0.001 * z[i] : 0.0;
        double st = 0.0;
        for (int j = 0; j < NN[i]; j++) {
            const int64_t idx = i * MN + j;
            const int64_t c = NL[idx];
            const double uxc = axis == 0 ? 0.001 * x[c] : 0.0;
            const double uyc = axis == 1 ? 0.001 * y[c] : 0.0;
            double L;
            if (p->dim == 2) {
                L = sqrt(sq(x[c] + uxc - x[i] - uxi) + sq(y[c] + uyc - y[i] - uyi));
            } else {
                const double uzc = axis == 2 ? 0.001 * z[c] : 0.0;
                L = sqrt(sq(x[c] + uxc - x[i] - uxi) + sq(y[c] + uyc - y[i] - uyi) +
                         sq(z[c] + uzc - z[i] - uzi));
            }
            st += 0.25 * p->bc * (L - idist[idx]) * (L - idist[idx]) / idist[idx] * p->vol * fac[idx];
        }
        fncst[i] = sedload / st;
    }
}

/* surface_correct_gpu (Surf_Corr.cu:235-310): vol_Corr, fncst per axis, then
 * kernel_cal_surf_coff_F (:160-232) per bond. */
void or_surface_correct(const pd_params* p, const int* NN, const int* NL, const double* x,
                        const double* y, const double* z, double* idist, double* fac,
                        double* fncst_x, double* fncst_y, double* fncst_z, double* scr) {
    const int MN = p->MN;
    const double pi = p->pi;
    or_vol_corr(p, NN, NL, x, y, z, idist, fac);
    surface_factor(p, 0, NN, NL, x, y, z, idist, fac, fncst_x);
    surface_factor(p, 1, NN, NL, x, y, z, idist, fac, fncst_y);
    if (p->dim == 3) surface_factor(p, 2, NN, NL, x, y, z, idist, fac, fncst_z);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p->N; i++)
        for (int j = 0; j < NN[i]; j++) {
            const int64_t idx = i * MN + j;
            const int64_t c = NL[idx];
            if (p->dim == 2) {
                double theta;
                if (fabs(y[c] - y[i]) <= 1.0e-10)
                    theta = 0.0;
                else if (fabs(x[c] - x[i]) <= 1.0e-10)
                    theta = 90.0 * pi / 180.0;
                else
                    theta = atan(fabs(y[c] - y[i]) / fabs(x[c] - x[i]));
                const double scx = (fncst_x[i] + fncst_x[c]) / 2.0;
                const double scy = (fncst_y[i] + fncst_y[c]) / 2.0;
                scr[idx] = sqrt(1.0 / (cos(theta) * cos(theta) / (scx * scx) + sin(theta) * sin(theta) / (scy * scy)));
            } else {
                if (fabs(z[c] - z[i]) < 1.0e-10) {
                    double theta;
                    if (fabs(y[c] - y[i]) < 1.0e-10)
                        theta = 0.0;
                    else if (fabs(x[c] - x[i]) < 1.0e-10)
                        theta = 90.0 * pi / 180.0;
                    else
                        theta = atan(fabs(y[c] - y[i]) / fabs(x[c] - x[i]));
                    const double phi = 90.0 * pi / 180.0;
                    const double scx = (fncst_x[i] + fncst_x[c]) / 2.0;
                    const double scy = (fncst_y[i] + fncst_y[c]) / 2.0;
                    const double scz = (fncst_z[i] + fncst_z[c]) / 2.0;
                    scr[idx] = sqrt(1.0 / (cos(theta) * cos(theta) / (scx * scx) + sin(theta) * sin(theta) / (scy * scy) +
                                           cos(phi) * cos(phi) / (scz * scz)));
                } else if (fabs(x[c] - x[i]) < 1.0e-10 && fabs(y[c] - y[i]) < 1.0e-10) {
                    scr[idx] = (fncst_z[i] + fncst_z[c]) / 2.0;
                } else {
                    const double theta = atan(fabs(y[c] - y[i]) / fabs(x[c] - x[i]));
                    const double phi = acos(fabs(z[c] - z[i]) / idist[idx]);
                    const double scx = (fncst_x[i] + fncst_x[c]) / 2.0;
                    const double scy = (fncst_y[i] + fncst_y[c]) / 2.0;
                    const double scz = (fncst_z[i] + fncst_z[c]) / 2.0;
                    scr[idx] = sqrt(1.0 / (cos(theta) * cos(theta) / (scx * scx) + sin(theta) * sin(theta) / (scy * scy) +
                                           cos(phi) * cos(phi) / (scz * scz)));
                }
            }
        }
}

/* kernel_particle_force_2D (Force_Bond.cu:52-85) and kernel_bond_force_3D
 * (:87-141): PMB force density, then break when s > s0 (3-D: only when both
 * ends have y >= -0.04, :117).  The bond contributes in the step it breaks. */
void or_bond_force(const pd_params* p, int64_t n_nodes, const double* x, const double* y,
                   const double* z, const double* ux, const double* uy, const double* uz,
                   const int* NN, const int* NL, const double* idist, const double* scr,
                   const double* fac, int* fail, double* fx, double* fy, double* fz) {
    const int MN = p->MN;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n_nodes; i++) {
        double force_x = 0.0, force_y = 0.0, force_z = 0.0;
        for (int j = 0; j < NN[i]; j++) {
            const int64_t idx = i * MN + j;
            if (fail[idx] != 1) continue;
            const int64_t c = NL[idx];
            if (p->dim == 2) {
                const double L = sqrt(sq(x[c] + ux[c] - x[i] - ux[i]) + sq(y[c] + uy[c] - y[i] - uy[i]));
                const double s = (L - idist[idx]) / idist[idx];
                force_x += p->vol * fac[idx] * p->bc * scr[idx] * s * (x[c] + ux[c] - x[i] - ux[i]) / L;
                force_y += p->vol * fac[idx] * p->bc * scr[idx] * s * (y[c] + uy[c] - y[i] - uy[i]) / L;
                if (s > p->critical_s) fail[idx] = 0;
            } else {
                const double L = sqrt(sq(x[c] + ux[c] - x[i] - ux[i]) + sq(y[c] + uy[c] - y[i] - uy[i]) +
                                      sq(z[c] + uz[c] - z[i] - uz[i]));
                const double s = (L - idist[idx]) / idist[idx];
                force_x += p->vol * fac[idx] * p->bc * scr[idx] * s * (x[c] + ux[c] - x[i] - ux[i]) / L;
                force_y += p->vol * fac[idx] * p->bc * scr[idx] * s * (y[c] + uy[c] - y[i] - uy[i]) / L;
                force_z += p->vol * fac[idx] * p->bc * scr[idx] * s * (z[c] + uz[c] - z[i] - uz[i]) / L;
                if (s > p->critical_s && y[i] >= p->break_ymin && y[c] >= p->break_ymin) fail[idx] = 0;
            }
        }
        fx[i] = force_x;
        fy[i] = force_y;
        if (p->dim == 3) fz[i] = force_z;
    }
}

/* kernel_initial_weight_2D/3D (Force_State.cu:8-54). */
void or_initial_weight(const pd_params* p, const int* NN, const double* idist, const double* fac,
                       double* w, double* m) {
    const int MN = p->MN;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p->N; i++) {
        double mm = 0.0;
        for (int j = 0; j < NN[i]; j++) {
            const int64_t idx = i * MN + j;
            w[idx] = exp(-sq(idist[idx]) / sq(p->delta));
            mm += w[idx] * sq(idist[idx]) * p->vol * fac[idx];
        }
        m[i] = mm;
    }
}

/* kernel_cal_theta_2D (Force_State.cu:56-85): every bond counts, intact or
 * not (the fail test is commented out at :65); kernel_cal_theta_3D
 * (:203-239): intact bonds only.  Runs over all N nodes and stores e. */
void or_state_theta(const pd_params* p, const double* x, const double* y, const double* z,
                    const double* ux, const double* uy, const double* uz, const int* NN,
                    const int* NL, const double* idist, const double* fac, const double* w,
                    const double* m, const int* fail, double* e, double* theta) {
    const int MN = p->MN;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p->N; i++) {
        double th = 0.0;
        for (int j = 0; j < NN[i]; j++) {
            const int64_t idx = i * MN + j;
            const int64_t c = NL[idx];
            if (p->dim == 2) {
                e[idx] = sqrt(sq(x[c] - x[i] + ux[c] - ux[i]) + sq(y[c] - y[i] + uy[c] - uy[i])) - idist[idx];
                th += 2.0 * (2.0 * p->pratio - 1.0) / (p->pratio - 1.0) / m[i] * w[idx] * idist[idx] * e[idx] *
                      fac[idx] * p->vol;
            } else {
                const int intact = (i < p->N_int) ? fail[idx] == 1 : 1;
                if (!intact) continue;
                e[idx] = sqrt(sq(x[c] - x[i] + ux[c] - ux[i]) + sq(y[c] - y[i] + uy[c] - uy[i]) +
                              sq(z[c] - z[i] + uz[c] - uz[i])) - idist[idx];
                th += 3.0 / m[i] * w[idx] * idist[idx] * e[idx] * fac[idx] * p->vol;
            }
        }
        theta[i] = th;
    }
}

/* kernel_state_force_2D (Force_State.cu:88-134) / kernel_state_force_3D
 * (:242-306) on nodes [0, N_int). */
void or_state_force(const pd_params* p, const double* x, const double* y, const double* z,
                    const double* ux, const double* uy, const double* uz, const int* NN,
                    const int* NL, const double* idist, const double* fac, const double* w,
                    const double* m, const double* theta, const double* e, int* fail, double* fx,
                    double* fy, double* fz) {
    const int MN = p->MN;
    const double pr = p->pratio, K = p->K, G = p->G, vol = p->vol;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p->N_int; i++) {
        double force_x = 0.0, force_y = 0.0, force_z = 0.0;
        for (int j = 0; j < NN[i]; j++) {
            const int64_t idx = i * MN + j;
            if (fail[idx] != 1) continue;
            const int64_t c = NL[idx];
            if (p->dim == 2) {
                const double L = sqrt(sq(x[c] + ux[c] - x[i] - ux[i]) + sq(y[c] + uy[c] - y[i] - uy[i]));
                const double s = (L - idist[idx]) / idist[idx];
                const double ti = (2.0 * pr - 1.0) / (pr - 1.0) * (2.0 * K - 32.0 * G / 9.0) * theta[i] * w[idx] *
                                      idist[idx] / m[i] +
                                  8.0 * G / m[i] * w[idx] * e[idx];
                const double tj = (2.0 * pr - 1.0) / (pr - 1.0) * (2.0 * K - 32.0 * G / 9.0) * theta[c] * w[idx] *
                                      idist[idx] / m[c] +
                                  8.0 * G / m[c] * w[idx] * e[idx];
                force_x += (ti * vol + tj * vol) * fac[idx] * (x[c] + ux[c] - x[i] - ux[i]) / L;
                force_y += (ti * vol + tj * vol) * fac[idx] * (y[c] + uy[c] - y[i] - uy[i]) / L;
                if (s > p->critical_s) fail[idx] = 0;
            } else {
                /* the z term of the length uses the dilatation pass's operand order (:272) */
                const double L = sqrt(sq(x[c] + ux[c] - x[i] - ux[i]) + sq(y[c] + uy[c] - y[i] - uy[i]) +
                                      sq(z[c] - z[i] + uz[c] - uz[i]));
                const double s = (L - idist[idx]) / idist[idx];
                const double ti = 3.0 * K * theta[i] * w[idx] * idist[idx] / m[i] +
                                  15.0 * G / m[i] * w[idx] * (e[idx] - theta[i] * idist[idx] / 3.0);
                const double tj = 3.0 * K * theta[c] * w[idx] * idist[idx] / m[c] +
                                  15.0 * G / m[c] * w[idx] * (e[idx] - theta[c] * idist[idx] / 3.0);
                force_x += (ti * vol + tj * vol) * fac[idx] * (x[c] + ux[c] - x[i] - ux[i]) / L;
                force_y += (ti * vol + tj * vol) * fac[idx] * (y[c] + uy[c] - y[i] - uy[i]) / L;
                force_z += (ti * vol + tj * vol) * fac[idx] * (z[c] + uz[c] - z[i] - uz[i]) / L;
                if (s > p->critical_s && y[i] >= p->break_ymin && y[c] >= p->break_ymin) fail[idx] = 0;
            }
        }
        fx[i] = force_x;
        fy[i] = force_y;
        if (p->dim == 3) fz[i] = force_z;
    }
}

/* kernel_cnn (Integrate.cu:7-49) + cal_cn (:108-129): damping coefficient.
 * The two sums run in ascending node order. */
double or_adr_cn(const pd_params* p, const double* fx, const double* fy, const double* fz,
                 const double* fox, const double* foy, const double* foz, const double* vhx,
                 const double* vhy, const double* vhz, const double* ux, const double* uy,
                 const double* uz) {
    double cn1 = 0.0, cn2 = 0.0;
    const double mass = p->mass, dt = p->dt;
    for (int64_t i = 0; i < p->N_int; i++) {
        double cn = 0.0, disp;
        if (vhx[i] != 0.0) cn = -1.0 * ux[i] * ux[i] * (fx[i] / mass - fox[i] / mass) / (dt * vhx[i]);
        disp = ux[i] * ux[i];
        if (vhy[i] != 0.0) cn -= 1.0 * uy[i] * uy[i] * (fy[i] / mass - foy[i] / mass) / (dt * vhy[i]);
        disp += uy[i] * uy[i];
        if (p->dim == 3) {
            if (vhz[i] != 0.0) cn -= 1.0 * uz[i] * uz[i] * (fz[i] / mass - foz[i] / mass) / (dt * vhz[i]);
            disp += uz[i] * uz[i];
        }
        cn1 += cn;
        cn2 += disp;
    }
    double cn = 0.0;
    if (cn2 != 0.0) {
        if (cn1 / cn2 > 0.0)
            cn = 2.0 * sqrt(cn1 / cn2);
        else
            cn = 0.0;
    }
    if (cn > 2.0) cn = 1.9;
    return cn;
}

/* kernel_integrate (Integrate.cu:54-106). */
void or_adr_update(const pd_params* p, int ct, double cn, const double* fx, const double* fy,
                   const double* fz, const double* bx, const double* by, const double* bz,
                   double* vhx, double* vhy, double* vhz, double* vx, double* vy, double* vz,
                   double* ux, double* uy, double* uz, double* fox, double* foy, double* foz) {
    const double dt = p->dt, mass = p->mass;
    const int nd = p->dim;
    double* vh[3] = {vhx, vhy, vhz};
    double* v[3] = {vx, vy, vz};
    double* u[3] = {ux, uy, uz};
    double* fo[3] = {fox, foy, foz};
    const double* f[3] = {fx, fy, fz};
    const double* b[3] = {bx, by, bz};
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p->N_int; i++)
        for (int a = 0; a < nd; a++) {
            const double vho = vh[a][i];
            double vhn;
            if (ct == 0)
                vhn = 1.0 * dt / mass * (f[a][i] + b[a][i]) / 2.0;
            else
                vhn = ((2.0 - cn * dt) * vho + 2.0 * dt / mass * (f[a][i] + b[a][i])) / (2.0 + cn * dt);
            v[a][i] = 0.5 * (vho + vhn);
            u[a][i] += vhn * dt;
            vh[a][i] = vhn;
            fo[a][i] = f[a][i];
        }
}

/* kernel_integrate_2D_1 / 3D_1 (Integrate.cu:174-202) on [0, N_int). */
void or_verlet1(const pd_params* p, double* vx, double* vy, double* vz, const double* ax,
                const double* ay, const double* az, double* ux, double* uy, double* uz) {
    const double dt = p->dt;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p->N_int; i++) {
        vx[i] += (dt / 2.0) * ax[i];
        vy[i] += (dt / 2.0) * ay[i];
        if (p->dim == 3) vz[i] += (dt / 2.0) * az[i];
        ux[i] += vx[i] * dt;
        uy[i] += vy[i] * dt;
        if (p->dim == 3) uz[i] += vz[i] * dt;
    }
}

/* kernel_integrate_2D_2 / 3D_2 (Integrate.cu:218-249) on [0, N_int). */
void or_verlet2(const pd_params* p, double* vx, double* vy, double* vz, double* ax, double* ay,
                double* az, const double* fx, const double* fy, const double* fz, const double* bx,
                const double* by, const double* bz) {
    const double dt = p->dt, dens = p->dens;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p->N_int; i++) {
        ax[i] = (fx[i] + bx[i]) / dens;
        ay[i] = (fy[i] + by[i]) / dens;
        if (p->dim == 3) az[i] = (fz[i] + bz[i]) / dens;
        vx[i] += (dt / 2.0) * ax[i];
        vy[i] += (dt / 2.0) * ay[i];
        if (p->dim == 3) vz[i] += (dt / 2.0) * az[i];
    }
}

/* kernel_cal_dmg_2D/3D (Base_Function.cu:149-217). */
void or_damage(const pd_params* p, const int* NN, const int* fail, const double* fac, double* dmg) {
    const int MN = p->MN;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p->N_int; i++) {
        double d1 = 0.0, d2 = 0.0;
        for (int j = 0; j < NN[i]; j++) {
            const int64_t idx = i * MN + j;
            d1 += fail[idx] * p->vol * fac[idx];
            d2 += p->vol * fac[idx];
        }
        dmg[i] = 1.0 - d1 / d2;
    }
}

/* kernel_set_crack_2D (Base_Function.cu:39-81). */
void or_set_crack_2d(const pd_params* p, double clength, double loc_x, double loc_y, double theta,
                     const int* NN, const int* NL, const double* x, const double* y, int* fail) {
    const int MN = p->MN;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p->N_int; i++)
        for (int j = 0; j < NN[i]; j++) {
            const int64_t idx = i * MN + j;
            const int64_t c = NL[idx];
            if (fabs(theta - p->pi / 2.0) < 0.0001) {
                if (fabs(y[c] - loc_y) < clength * sin(theta) / 2.0 && fabs(y[i] - loc_y) < clength * sin(theta) / 2.0)
                    if ((x[c] - loc_x) * (x[i] - loc_x) < 0.0) fail[idx] = 0;
            } else {
                const double t = tan(theta);
                const double dist_c = sq(y[c] - loc_y) + sq(x[c] - loc_x);
                const double dist_i = sq(y[i] - loc_y) + sq(x[i] - loc_x);
                const double vert_c = sq((t * x[c] - y[c] - loc_x * t + loc_y) / sqrt(1 + t * t));
                const double vert_i = sq((t * x[i] - y[i] - loc_x * t + loc_y) / sqrt(1 + t * t));
                const double len_c = sqrt(dist_c - vert_c);
                const double len_i = sqrt(dist_i - vert_i);
                if (len_c < clength / 2.0 && len_i < clength / 2.0) {
                    const double bcn = t * x[c] - loc_x * t + loc_y - y[c];
                    const double bi = t * x[i] - loc_x * t + loc_y - y[i];
                    if (bcn * bi <= 0) fail[idx] = 0;
                }
            }
        }
}

/* kernel_set_crack (Solve_Kalthoff_Winkler.cu:40-63): bonds crossing the
 * planes x = -rad or x = +rad with an end in the upper half are cut. */
void or_set_crack_kw(const pd_params* p, double rad, const int* NN, const int* NL, const double* x,
                     const double* y, int* fail) {
    const int MN = p->MN;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < p->N_int; i++)
        for (int j = 0; j < NN[i]; j++) {
            const int64_t idx = i * MN + j;
            const int64_t c = NL[idx];
            if ((x[c] > -rad && x[i] < -rad) | (x[i] > -rad && x[c] < -rad))
                if ((y[c] >= -1.0e-10) | (y[i] >= -1.0e-10)) fail[idx] = 0;
            if ((x[c] > rad && x[i] < rad) | (x[i] > rad && x[c] < rad))
                if ((y[c] >= -1.0e-10) | (y[i] >= -1.0e-10)) fail[idx] = 0;
        }
}

/* kernel_quick_load (Solve_Plate_Crack_Grow.cu:8-19). */
void or_quick_load(const pd_params* p, double load, double* uy) {
    for (int64_t i = 0; i < 3 * (int64_t)p->nx; i++) uy[p->N_int + i] += load * p->dt;
    for (int64_t i = 3 * (int64_t)p->nx; i < 6 * (int64_t)p->nx; i++) uy[p->N_int + i] -= load * p->dt;
}

/* load_plate_tensile_gpu (Solve_Plate_Tensile.cu:7-17). */
void or_load_plate_tensile(const pd_params* p, double* bx) {
    for (int i = 0; i < p->ny; i++) {
        bx[(int64_t)i * p->nx] = -0.001 * p->emod / p->dx;
        bx[(int64_t)i * p->nx + p->nx - 1] = 0.001 * p->emod / p->dx;
    }
}

/* kernel_contact (Solve_Kalthoff_Winkler.cu:112-175); reaction force summed
 * in ascending node order into force[3]. */
void or_contact(const pd_params* p, const pd_cylinder* cy, const double* dmg, const double* x,
                const double* y, const double* z, double* ux, double* uy, double* uz, double* vx,
                double* vy, double* vz, double* force) {
    const double dt = p->dt;
    for (int64_t i = 0; i < p->N_int; i++) {
        if (!(dmg[i] < 1.0)) continue;
        const double dpenx = x[i] + ux[i] - cy->x - cy->disp[0];
        const double dpeny = y[i] + uy[i] - cy->y - cy->disp[1];
        const double dpenz = z[i] + uz[i] - cy->z - cy->disp[2];
        const double dpend = sqrt(dpenx * dpenx + dpenz * dpenz);
        if (dpend <= cy->rad && fabs(dpeny) <= (cy->height / 2.0)) {
            double dprx, dpry, dprz;
            if (cy->rad - dpend <= cy->height / 2.0 - fabs(dpeny)) {
                dprx = dpenx / dpend * cy->rad;
                dpry = dpeny;
                dprz = dpenz / dpend * cy->rad;
            } else if (dpeny >= 0.0) {
                dprx = dpenx;
                dpry = cy->height / 2.0;
                dprz = dpenz;
            } else {
                dprx = dpenx;
                dpry = -cy->height / 2.0;
                dprz = dpenz;
            }
            const double oux = ux[i], ouy = uy[i], ouz = uz[i];
            const double ovx = vx[i], ovy = vy[i], ovz = vz[i];
            ux[i] = cy->x + cy->disp[0] + dprx - x[i];
            uy[i] = cy->y + cy->disp[1] + dpry - y[i];
            uz[i] = cy->z + cy->disp[2] + dprz - z[i];
            vx[i] = (ux[i] - oux) / dt;
            vy[i] = (uy[i] - ouy) / dt;
            vz[i] = (uz[i] - ouz) / dt;
            force[0] += -p->dens * (vx[i] - ovx) / dt * p->vol;
            force[1] += -p->dens * (vy[i] - ovy) / dt * p->vol;
            force[2] += -p->dens * (vz[i] - ovz) / dt * p->vol;
        }
    }
}

/* kernel_cy_integrate_1 (Solve_Kalthoff_Winkler.cu:89-99). */
void or_cy_integrate1(const pd_params* p, pd_cylinder* cy) {
    for (int a = 0; a < 3; a++) {
        cy->vel[a] += (p->dt / 2.0) * cy->acc[a];
        cy->disp[a] += cy->vel[a] * p->dt;
    }
}

/* kernel_cy_integrate_2 (Solve_Kalthoff_Winkler.cu:242-253). */
void or_cy_integrate2(const pd_params* p, pd_cylinder* cy) {
    for (int a = 0; a < 3; a++) {
        cy->acc[a] = cy->force[a] / cy->mass;
        cy->vel[a] += p->dt / 2.0 * cy->acc[a];
        cy->force[a] = 0.0;
    }
}
