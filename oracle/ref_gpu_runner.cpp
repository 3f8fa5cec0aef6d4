// Test/measurement infrastructure only: runs the reference's own CUDA kernels
// (oracle/_ref/ref_kernels.cubin, compiled from the reference sources) through
// the CUDA driver API, on inputs the caller provides in the reference's
// layout (SoA node arrays, N*MN padded ELL bond arrays).  Used by the GPU
// parity tests (the reference's GPU kernels as the oracle) and by bench.py to
// time the reference's step loop on the same GPU.  Nothing in the product
// links or loads it.
//
// Launch shapes follow the reference's drivers: kernel_particle_force_2D over
// N threads (Solve_Plate_Tensile.cu:109), kernel_bond_force_2D over N*MN
// threads (Force_Bond.cu:143-147), the Verlet halves over N_int threads
// (Integrate.cu:204-209, :251-256), kernel_cal_dmg_2D over N_int*MN threads
// (Solve_Plate_Crack_Grow.cu:301).
#include <cuda.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

namespace {

// The reference's parameter block (Base.cuh:46-68) with real = double.
struct device_parameter {
    double pi;
    int N, MN, N_int, nx, ny, nz;
    double dx, emod, dens, pratio, bc, delta, critical_s, vol, dt;
    int nt;
    double mass, K, G;
};

struct Runner {
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUfunction f_particle = nullptr, f_bond = nullptr, f_int1 = nullptr, f_int2 = nullptr, f_dmg = nullptr;
    CUfunction f_cnn = nullptr, f_adr = nullptr, f_reduce = nullptr, f_qload = nullptr;
    CUdeviceptr static_y = 0;  // Reduce.cu's block partial array
    CUstream stream = nullptr;
    device_parameter p{};
    // device arrays
    CUdeviceptr x = 0, y = 0, ux = 0, uy = 0, vx = 0, vy = 0, ax = 0, ay = 0, fx = 0, fy = 0, bx = 0, by = 0,
                dmg = 0, NN = 0, NL = 0, idist = 0, scr = 0, fac = 0, fail = 0;
    // ADR arrays (velhalf, velhalfold, pforceold per axis; kernel_cnn's outputs)
    CUdeviceptr vhx = 0, vhy = 0, vhox = 0, vhoy = 0, fox = 0, foy = 0, cn_xy = 0, disp_xy = 0;
    bool ready = false;
};

Runner R;
char g_err[256] = "";

int fail_with(CUresult r, const char* what) {
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    std::snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "?");
    return -1;
}

#define RR_TRY(call, what)               \
    do {                                 \
        CUresult _r = (call);            \
        if (_r != CUDA_SUCCESS) return fail_with(_r, what); \
    } while (0)

void free_all() {
    CUdeviceptr* all[] = {&R.x,     &R.y,   &R.ux,   &R.uy,   &R.vx,   &R.vy,    &R.ax,   &R.ay,
                          &R.fx,    &R.fy,  &R.bx,   &R.by,   &R.dmg,  &R.NN,    &R.NL,   &R.idist,
                          &R.scr,   &R.fac, &R.fail, &R.vhx,  &R.vhy,  &R.vhox,  &R.vhoy, &R.fox,
                          &R.foy,   &R.cn_xy, &R.disp_xy};
    for (CUdeviceptr* d : all)
        if (*d) {
            cuMemFree(*d);
            *d = 0;
        }
}

int launch(CUfunction f, unsigned grid, void** args) {
    RR_TRY(cuLaunchKernel(f, grid, 1, 1, 256, 1, 1, 0, R.stream, args, nullptr), "launch");
    return 0;
}

}  // namespace

extern "C" {

const char* rr_error(void) { return g_err; }

// Load the cubin into the primary context of device 0.
int rr_init(const char* cubin) {
    if (R.mod) return 0;
    RR_TRY(cuInit(0), "cuInit");
    CUdevice dev;
    RR_TRY(cuDeviceGet(&dev, 0), "cuDeviceGet");
    RR_TRY(cuDevicePrimaryCtxRetain(&R.ctx, dev), "primary context");
    RR_TRY(cuCtxSetCurrent(R.ctx), "set context");
    RR_TRY(cuModuleLoad(&R.mod, cubin), "cuModuleLoad");
    RR_TRY(cuModuleGetFunction(&R.f_particle, R.mod, "_Z24kernel_particle_force_2DPdS_S_S_S_S_PiS0_S_S_S0_S_"),
           "kernel_particle_force_2D");
    RR_TRY(cuModuleGetFunction(&R.f_bond, R.mod, "_Z20kernel_bond_force_2DPdS_S_S_S_S_PiS0_S_S_S0_S_"),
           "kernel_bond_force_2D");
    RR_TRY(cuModuleGetFunction(&R.f_int1, R.mod, "_Z21kernel_integrate_2D_1PdS_S_S_S_S_"), "kernel_integrate_2D_1");
    RR_TRY(cuModuleGetFunction(&R.f_int2, R.mod, "_Z21kernel_integrate_2D_2PdS_S_S_S_S_S_S_"),
           "kernel_integrate_2D_2");
    RR_TRY(cuModuleGetFunction(&R.f_dmg, R.mod, "_Z17kernel_cal_dmg_2DPiPdS_S0_"), "kernel_cal_dmg_2D");
    RR_TRY(cuModuleGetFunction(&R.f_cnn, R.mod, "_Z10kernel_cnnPdS_S_S_S_S_S_S_S_S_S_S_S_S_"), "kernel_cnn");
    RR_TRY(cuModuleGetFunction(&R.f_adr, R.mod, "_Z16kernel_integrateidPdS_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_S_"),
           "kernel_integrate");
    RR_TRY(cuModuleGetFunction(&R.f_reduce, R.mod, "_Z9reduce_cpPKdPdi"), "reduce_cp");
    RR_TRY(cuModuleGetFunction(&R.f_qload, R.mod, "harness_quick_load"), "harness_quick_load");
    size_t ys = 0;
    RR_TRY(cuModuleGetGlobal(&R.static_y, &ys, R.mod, "static_y"), "static_y");
    if (ys != 256 * sizeof(double)) return fail_with(CUDA_ERROR_INVALID_VALUE, "static_y size");
    RR_TRY(cuStreamCreate(&R.stream, CU_STREAM_NON_BLOCKING), "stream");
    return 0;
}

// Upload a 2-D bond-based problem.  dparams: pi dx emod dens pratio bc delta
// critical_s vol dt mass K G; iparams: N MN N_int nx ny nz nt.  Bond arrays are
// N*MN padded ELL; fail has N*MN entries (1 intact).
int rr_setup(const double* dparams, const int* iparams, const double* x, const double* y, const int* NN,
             const int* NL, const double* idist, const double* scr, const double* fac, const int* fail,
             const double* bx, const double* by) {
    if (!R.mod) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_init first");
    RR_TRY(cuCtxSetCurrent(R.ctx), "set context");
    free_all();
    device_parameter& p = R.p;
    p.pi = dparams[0];
    p.dx = dparams[1];
    p.emod = dparams[2];
    p.dens = dparams[3];
    p.pratio = dparams[4];
    p.bc = dparams[5];
    p.delta = dparams[6];
    p.critical_s = dparams[7];
    p.vol = dparams[8];
    p.dt = dparams[9];
    p.mass = dparams[10];
    p.K = dparams[11];
    p.G = dparams[12];
    p.N = iparams[0];
    p.MN = iparams[1];
    p.N_int = iparams[2];
    p.nx = iparams[3];
    p.ny = iparams[4];
    p.nz = iparams[5];
    p.nt = iparams[6];
    const size_t N = (size_t)p.N, S = (size_t)p.N * p.MN;
    CUdeviceptr dpp;
    size_t dps;
    RR_TRY(cuModuleGetGlobal(&dpp, &dps, R.mod, "dp"), "dp symbol");
    if (dps != sizeof(device_parameter)) return fail_with(CUDA_ERROR_INVALID_VALUE, "dp size");
    RR_TRY(cuMemcpyHtoD(dpp, &p, sizeof(p)), "dp copy");
    CUdeviceptr* nodes[] = {&R.x,   &R.y,    &R.ux,   &R.uy,  &R.vx,  &R.vy,    &R.ax,      &R.ay,   &R.fx,
                            &R.fy,  &R.bx,   &R.by,   &R.dmg, &R.vhx, &R.vhy,   &R.vhox,    &R.vhoy, &R.fox,
                            &R.foy, &R.cn_xy, &R.disp_xy};
    for (CUdeviceptr* d : nodes) {
        RR_TRY(cuMemAlloc(d, N * 8), "node alloc");
        RR_TRY(cuMemsetD8(*d, 0, N * 8), "node zero");
    }
    RR_TRY(cuMemAlloc(&R.NN, N * 4), "NN");
    RR_TRY(cuMemAlloc(&R.NL, S * 4), "NL");
    RR_TRY(cuMemAlloc(&R.idist, S * 8), "idist");
    RR_TRY(cuMemAlloc(&R.scr, S * 8), "scr");
    RR_TRY(cuMemAlloc(&R.fac, S * 8), "fac");
    RR_TRY(cuMemAlloc(&R.fail, S * 4), "fail");
    RR_TRY(cuMemcpyHtoD(R.x, x, N * 8), "x");
    RR_TRY(cuMemcpyHtoD(R.y, y, N * 8), "y");
    RR_TRY(cuMemcpyHtoD(R.bx, bx, N * 8), "bx");
    RR_TRY(cuMemcpyHtoD(R.by, by, N * 8), "by");
    RR_TRY(cuMemcpyHtoD(R.NN, NN, N * 4), "NN");
    RR_TRY(cuMemcpyHtoD(R.NL, NL, S * 4), "NL");
    RR_TRY(cuMemcpyHtoD(R.idist, idist, S * 8), "idist");
    RR_TRY(cuMemcpyHtoD(R.scr, scr, S * 8), "scr");
    RR_TRY(cuMemcpyHtoD(R.fac, fac, S * 8), "fac");
    RR_TRY(cuMemcpyHtoD(R.fail, fail, S * 4), "fail");
    R.ready = true;
    return 0;
}

// Set the displacement field (N doubles each); velocities and accelerations
// are left as they are.
int rr_set_disp(const double* ux, const double* uy) {
    if (!R.ready) return -1;
    RR_TRY(cuMemcpyHtoD(R.ux, ux, (size_t)R.p.N * 8), "ux");
    RR_TRY(cuMemcpyHtoD(R.uy, uy, (size_t)R.p.N * 8), "uy");
    return 0;
}

// One force evaluation: variant 0 kernel_particle_force_2D, 1 kernel_bond_force_2D.
int rr_force(int variant) {
    if (!R.ready) return -1;
    void* a[] = {&R.x, &R.ux, &R.fx, &R.y, &R.uy, &R.fy, &R.NN, &R.NL, &R.idist, &R.scr, &R.fail, &R.fac};
    const unsigned gN = (unsigned)((R.p.N - 1) / 256 + 1);
    const unsigned gS = (unsigned)(((int64_t)R.p.N * R.p.MN - 1) / 256 + 1);
    if (launch(variant == 0 ? R.f_particle : R.f_bond, variant == 0 ? gN : gS, a)) return -1;
    RR_TRY(cuStreamSynchronize(R.stream), "force");
    return 0;
}

// nsteps explicit Verlet steps (integrate_2D_1, force, integrate_2D_2), the
// damage pass every dmg_every steps (0: never).  Returns the elapsed time of
// the loop in *ms (CUDA events around it).
int rr_run(int variant, int nsteps, int dmg_every, double* ms) {
    if (!R.ready) return -1;
    void* a1[] = {&R.vx, &R.ax, &R.ux, &R.vy, &R.ay, &R.uy};
    void* af[] = {&R.x, &R.ux, &R.fx, &R.y, &R.uy, &R.fy, &R.NN, &R.NL, &R.idist, &R.scr, &R.fail, &R.fac};
    void* a2[] = {&R.vx, &R.ax, &R.fx, &R.bx, &R.vy, &R.ay, &R.fy, &R.by};
    void* ad[] = {&R.NN, &R.dmg, &R.fail, &R.fac};
    const unsigned g3 = (unsigned)((R.p.N_int - 1) / 256 + 1);
    const unsigned gN = (unsigned)((R.p.N - 1) / 256 + 1);
    const unsigned gS = (unsigned)(((int64_t)R.p.N * R.p.MN - 1) / 256 + 1);
    const unsigned g4 = (unsigned)(((int64_t)R.p.N_int * R.p.MN - 1) / 256 + 1);
    CUevent e0, e1;
    RR_TRY(cuEventCreate(&e0, CU_EVENT_DEFAULT), "event");
    RR_TRY(cuEventCreate(&e1, CU_EVENT_DEFAULT), "event");
    RR_TRY(cuEventRecord(e0, R.stream), "record");
    for (int s = 0; s < nsteps; s++) {
        if (launch(R.f_int1, g3, a1)) return -1;
        if (launch(variant == 0 ? R.f_particle : R.f_bond, variant == 0 ? gN : gS, af)) return -1;
        if (launch(R.f_int2, g3, a2)) return -1;
        if (dmg_every > 0 && (s + 1) % dmg_every == 0 && launch(R.f_dmg, g4, ad)) return -1;
    }
    RR_TRY(cuEventRecord(e1, R.stream), "record");
    RR_TRY(cuEventSynchronize(e1), "sync");
    float t = 0.f;
    RR_TRY(cuEventElapsedTime(&t, e0, e1), "elapsed");
    *ms = t;
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    return 0;
}

namespace {

// sum (Reduce.cu:52-65): two reduce_cp launches into static_y, then a
// blocking read of the result.
int ref_sum(int n, CUdeviceptr x, double* out) {
    int nn = n, nb = 256;
    void* a1[] = {&x, &R.static_y, &nn};
    void* a2[] = {&R.static_y, &R.static_y, &nb};
    RR_TRY(cuLaunchKernel(R.f_reduce, 256, 1, 1, 256, 1, 1, 256 * 8, R.stream, a1, nullptr), "reduce_cp");
    RR_TRY(cuLaunchKernel(R.f_reduce, 1, 1, 1, 256, 1, 1, 256 * 8, R.stream, a2, nullptr), "reduce_cp");
    RR_TRY(cuMemcpyDtoHAsync(out, R.static_y, sizeof(double), R.stream), "sum read");
    RR_TRY(cuStreamSynchronize(R.stream), "sum sync");
    return 0;
}

}  // namespace

// nsteps ADR steps of solve_plate_tensile's loop (Solve_Plate_Tensile.cu:106-131)
// with the crack-plate driver's moving boundary rows before each step:
// quick_load, kernel_particle_force_2D, kernel_cnn, cal_cn (two sums, each
// read back by the host), kernel_integrate.  Step indices ct0.. ; the
// elapsed time of the loop goes to *ms, the last damping coefficient to *cn.
int rr_run_adr(int ct0, int nsteps, double load, double* ms, double* cn_out) {
    if (!R.ready) return -1;
    CUdeviceptr null = 0;
    void* af[] = {&R.x, &R.ux, &R.fx, &R.y, &R.uy, &R.fy, &R.NN, &R.NL, &R.idist, &R.scr, &R.fail, &R.fac};
    void* ac[] = {&R.cn_xy, &R.fx, &R.fox, &R.vhox, &R.ux, &R.disp_xy, &R.fy, &R.foy, &R.vhoy, &R.uy,
                  &null,    &null, &null,  &null};
    void* aq[] = {&load, &R.uy};
    const unsigned gN = (unsigned)((R.p.N - 1) / 256 + 1);
    const unsigned gQ = (unsigned)((6 * R.p.nx - 1) / 256 + 1);
    CUevent e0, e1;
    RR_TRY(cuEventCreate(&e0, CU_EVENT_DEFAULT), "event");
    RR_TRY(cuEventCreate(&e1, CU_EVENT_DEFAULT), "event");
    RR_TRY(cuEventRecord(e0, R.stream), "record");
    double cn = 0.0;
    for (int s = 0; s < nsteps; s++) {
        int ct = ct0 + s;
        if (load != 0.0 && launch(R.f_qload, gQ, aq)) return -1;
        if (launch(R.f_particle, gN, af)) return -1;
        if (launch(R.f_cnn, gN, ac)) return -1;
        double cn1 = 0.0, cn2 = 0.0;
        if (ref_sum(R.p.N_int, R.cn_xy, &cn1) || ref_sum(R.p.N_int, R.disp_xy, &cn2)) return -1;
        cn = 0.0;  // cal_cn (Integrate.cu:108-129)
        if (cn2 != 0.0) {
            if (cn1 / cn2 > 0.0)
                cn = 2.0 * std::sqrt(cn1 / cn2);
            else
                cn = 0.0;
        }
        if (cn > 2.0) cn = 1.9;
        void* ai[] = {&ct,    &cn,   &R.fx,  &R.vhx, &R.bx, &R.vx,  &R.vhox, &R.ux,
                      &R.fox, &R.fy, &R.vhy, &R.by,  &R.vy, &R.vhoy, &R.uy,  &R.foy,
                      &null,  &null, &null,  &null,  &null, &null,  &null};
        if (launch(R.f_adr, gN, ai)) return -1;
    }
    RR_TRY(cuEventRecord(e1, R.stream), "record");
    RR_TRY(cuEventSynchronize(e1), "sync");
    float t = 0.f;
    RR_TRY(cuEventElapsedTime(&t, e0, e1), "elapsed");
    *ms = t;
    if (cn_out) *cn_out = cn;
    cuEventDestroy(e0);
    cuEventDestroy(e1);
    return 0;
}

// Read back node fields (N doubles each; NULL skips), the N*MN fail flags and
// the damage field (written by kernel_cal_dmg_2D at the damage steps of rr_run).
int rr_get(double* ux, double* uy, double* fx, double* fy, double* vy, int* fail, double* dmg) {
    if (!R.ready) return -1;
    const size_t N = (size_t)R.p.N;
    RR_TRY(cuStreamSynchronize(R.stream), "sync");
    if (ux) RR_TRY(cuMemcpyDtoH(ux, R.ux, N * 8), "ux");
    if (uy) RR_TRY(cuMemcpyDtoH(uy, R.uy, N * 8), "uy");
    if (fx) RR_TRY(cuMemcpyDtoH(fx, R.fx, N * 8), "fx");
    if (fy) RR_TRY(cuMemcpyDtoH(fy, R.fy, N * 8), "fy");
    if (vy) RR_TRY(cuMemcpyDtoH(vy, R.vy, N * 8), "vy");
    if (fail) RR_TRY(cuMemcpyDtoH(fail, R.fail, N * (size_t)R.p.MN * 4), "fail");
    if (dmg) RR_TRY(cuMemcpyDtoH(dmg, R.dmg, N * 8), "dmg");
    return 0;
}

int rr_free(void) {
    free_all();
    R.ready = false;
    return 0;
}

}  // extern "C"
