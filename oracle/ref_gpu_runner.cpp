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
// (Solve_Plate_Crack_Grow.cu:301); the impact driver's loop as written at
// Solve_Kalthoff_Winkler.cu:406-430 (kernel_bond_force_3D over N*MN threads
// with 3*256 doubles of shared memory, kernel_contact over N threads, the
// cylinder kernels on one warp); the crack-grow driver's state-based loop as
// written at Solve_Plate_Crack_Grow.cu:126-149 (kernel_cal_theta_2D over N*MN
// threads, kernel_state_force_2D over N_int*MN threads).
//
// Two deviations from the reference's own calls, both for defined behaviour:
//  * kernel_integrate_3D_1 declares its z parameters as (disp_z, vel_z, acc_z)
//    (Integrate.cu:188-191, Integrate.cuh:35-36) while the impact driver passes
//    (vel_z, acc_z, disp_z) (Solve_Kalthoff_Winkler.cu:408-410), which would
//    add dt/2 * disp_z to acc_z and never advance disp_z.  The runner passes
//    the arrays by the declared names: the update of the reference's host twin
//    integrate_1 (Integrate.cu:447-462).
//  * kernel_cal_dmg_3D holds __syncthreads inside "if (i < N_int)"
//    (Base_Function.cu:185-207), a divergent barrier in the last block when
//    N_int*MN is not a multiple of the block; it is not launched.  The damage
//    of a 3-D run is computed by the caller from the intact flags.
// The 3-D state-based kernels (Force_State.cu:29-54, :242-306) put two nodes in
// each 256-thread block (MN = 128) and hold __syncthreads inside "if (i < N)"
// (kernel_initial_weight_3D) and "if (i < N_int)" (kernel_state_force_3D):
// the runner launches them only when N (resp. N_int) is even, so that no block
// straddles the bound and every barrier is reached by the whole block.
// kernel_cal_theta_3D is never launched: it reads fail[idx] before its bounds
// test and holds its barrier inside "if (fail[idx] == 1)", a divergent branch
// once any bond of a block is broken (Force_State.cu:214-234); the caller
// supplies theta and e instead (rr_set_theta_e).
// kernel_bond_force_3D stores the node sums of thread j == 0 without a bound
// test (Force_Bond.cu:133-139), so the tail of the last block writes element
// N of the force arrays; node arrays are allocated with kNodePad spare
// elements to keep that store inside the allocation.
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

constexpr size_t kNodePad = 256;

// Cylinder_Parameter (Base.cuh:227-236) with real = double.
struct cylinder_parameter {
    double rad, mass, height, v, x, y, z;
};

struct Runner {
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    CUfunction f_particle = nullptr, f_bond = nullptr, f_int1 = nullptr, f_int2 = nullptr, f_dmg = nullptr;
    CUfunction f_cnn = nullptr, f_adr = nullptr, f_reduce = nullptr, f_qload = nullptr;
    CUfunction f_bond3 = nullptr, f_int31 = nullptr, f_int32 = nullptr, f_contact = nullptr, f_cy1 = nullptr,
               f_cy2 = nullptr, f_cyinit = nullptr, f_theta2 = nullptr, f_state2 = nullptr, f_weight3 = nullptr,
               f_state3 = nullptr;
    CUdeviceptr static_y = 0;  // Reduce.cu's block partial array
    CUstream stream = nullptr;
    device_parameter p{};
    // device arrays
    CUdeviceptr x = 0, y = 0, ux = 0, uy = 0, vx = 0, vy = 0, ax = 0, ay = 0, fx = 0, fy = 0, bx = 0, by = 0,
                dmg = 0, NN = 0, NL = 0, idist = 0, scr = 0, fac = 0, fail = 0;
    // ADR arrays (velhalf, velhalfold, pforceold per axis; kernel_cnn's outputs)
    CUdeviceptr vhx = 0, vhy = 0, vhox = 0, vhoy = 0, fox = 0, foy = 0, cn_xy = 0, disp_xy = 0;
    // third component and the impactor (Cylinder: acc, disp, vel, force, 3 doubles each)
    CUdeviceptr z = 0, uz = 0, vz = 0, az = 0, fz = 0, bz = 0, cacc = 0, cdisp = 0, cvel = 0, cforce = 0;
    // state-based: weighted volume m and dilatation theta per node, influence w and extension e per bond
    CUdeviceptr m = 0, theta = 0, w = 0, e = 0;
    bool ready = false, has_z = false, has_state = false, has_state3 = false;
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
                          &R.foy,   &R.cn_xy, &R.disp_xy, &R.z,   &R.uz,    &R.vz,   &R.az,
                          &R.fz,    &R.bz,  &R.cacc, &R.cdisp, &R.cvel, &R.cforce, &R.m, &R.theta,
                          &R.w,     &R.e};
    for (CUdeviceptr* d : all)
        if (*d) {
            cuMemFree(*d);
            *d = 0;
        }
}

int launch(CUfunction f, unsigned grid, void** args, unsigned block = 256, unsigned smem = 0) {
    RR_TRY(cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, R.stream, args, nullptr), "launch");
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
    RR_TRY(cuModuleGetFunction(&R.f_bond3, R.mod, "_Z20kernel_bond_force_3DPdS_S_S_S_S_S_S_S_PiS0_S_S_S0_S_"),
           "kernel_bond_force_3D");
    RR_TRY(cuModuleGetFunction(&R.f_int31, R.mod, "_Z21kernel_integrate_3D_1PdS_S_S_S_S_S_S_S_"),
           "kernel_integrate_3D_1");
    RR_TRY(cuModuleGetFunction(&R.f_int32, R.mod, "_Z21kernel_integrate_3D_2PdS_S_S_S_S_S_S_S_S_S_S_"),
           "kernel_integrate_3D_2");
    RR_TRY(cuModuleGetFunction(&R.f_contact, R.mod, "_Z14kernel_contactiPdS_S_S_S_S_S_S_S_S_S_S_"),
           "kernel_contact");
    RR_TRY(cuModuleGetFunction(&R.f_cy1, R.mod, "_Z21kernel_cy_integrate_1PdS_S_"), "kernel_cy_integrate_1");
    RR_TRY(cuModuleGetFunction(&R.f_cy2, R.mod, "_Z21kernel_cy_integrate_2PdS_S_"), "kernel_cy_integrate_2");
    RR_TRY(cuModuleGetFunction(&R.f_cyinit, R.mod, "_Z23kernel_initial_cylinderPdS_S_S_"),
           "kernel_initial_cylinder");
    RR_TRY(cuModuleGetFunction(&R.f_theta2, R.mod, "_Z19kernel_cal_theta_2DPiPdS0_S_S0_S_S0_S0_S0_S0_S0_S0_S0_"),
           "kernel_cal_theta_2D");
    RR_TRY(cuModuleGetFunction(&R.f_state2, R.mod, "_Z21kernel_state_force_2DPiPdS0_S_S_S0_S0_S0_S0_S0_S0_S0_S0_S0_S0_"),
           "kernel_state_force_2D");
    RR_TRY(cuModuleGetFunction(&R.f_weight3, R.mod, "_Z24kernel_initial_weight_3DPdPiS_S_S_"),
           "kernel_initial_weight_3D");
    RR_TRY(cuModuleGetFunction(&R.f_state3, R.mod,
                               "_Z21kernel_state_force_3DPiPdS0_S_S_S0_S0_S0_S0_S0_S0_S0_S0_S0_S0_S0_S0_S0_"),
           "kernel_state_force_3D");
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
        RR_TRY(cuMemAlloc(d, (N + kNodePad) * 8), "node alloc");
        RR_TRY(cuMemsetD8(*d, 0, (N + kNodePad) * 8), "node zero");
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
    R.has_z = false;
    R.has_state = false;
    R.has_state3 = false;
    return 0;
}

// State-based arrays of a 2-D problem set up by rr_setup: m (N doubles, the
// weighted volume) and w (N*MN padded ELL influence weights).
int rr_setup_state(const double* m, const double* w) {
    if (!R.ready) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup first");
    const size_t N = (size_t)R.p.N, S = (size_t)R.p.N * R.p.MN;
    RR_TRY(cuMemAlloc(&R.m, (N + kNodePad) * 8), "m");
    RR_TRY(cuMemAlloc(&R.theta, (N + kNodePad) * 8), "theta");
    RR_TRY(cuMemsetD8(R.theta, 0, (N + kNodePad) * 8), "theta zero");
    RR_TRY(cuMemAlloc(&R.w, S * 8), "w");
    RR_TRY(cuMemAlloc(&R.e, S * 8), "e");
    RR_TRY(cuMemsetD8(R.e, 0, S * 8), "e zero");
    RR_TRY(cuMemcpyHtoD(R.m, m, N * 8), "m copy");
    RR_TRY(cuMemcpyHtoD(R.w, w, S * 8), "w copy");
    R.has_state = true;
    return 0;
}

// Third component and impactor of a 3-D problem set up by rr_setup: z, bz (N
// doubles each); cyl: rad mass height v x y z (Cylinder_Parameter), copied to
// the reference's dcyp, then kernel_initial_cylinder as the impact driver
// launches it (Solve_Kalthoff_Winkler.cu:403).
int rr_setup_z(const double* z, const double* bz, const double* cyl) {
    if (!R.ready) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup first");
    const size_t N = (size_t)R.p.N;
    CUdeviceptr* nodes[] = {&R.z, &R.uz, &R.vz, &R.az, &R.fz, &R.bz};
    for (CUdeviceptr* d : nodes) {
        RR_TRY(cuMemAlloc(d, (N + kNodePad) * 8), "node alloc");
        RR_TRY(cuMemsetD8(*d, 0, (N + kNodePad) * 8), "node zero");
    }
    RR_TRY(cuMemcpyHtoD(R.z, z, N * 8), "z");
    RR_TRY(cuMemcpyHtoD(R.bz, bz, N * 8), "bz");
    CUdeviceptr* cy[] = {&R.cacc, &R.cdisp, &R.cvel, &R.cforce};
    for (CUdeviceptr* d : cy) {
        RR_TRY(cuMemAlloc(d, 4 * 8), "cylinder alloc");
        RR_TRY(cuMemsetD8(*d, 0, 4 * 8), "cylinder zero");
    }
    cylinder_parameter c{cyl[0], cyl[1], cyl[2], cyl[3], cyl[4], cyl[5], cyl[6]};
    CUdeviceptr cpp;
    size_t cps;
    RR_TRY(cuModuleGetGlobal(&cpp, &cps, R.mod, "dcyp"), "dcyp symbol");
    if (cps != sizeof(cylinder_parameter)) return fail_with(CUDA_ERROR_INVALID_VALUE, "dcyp size");
    RR_TRY(cuMemcpyHtoD(cpp, &c, sizeof(c)), "dcyp copy");
    void* a[] = {&R.cvel, &R.cdisp, &R.cacc, &R.cforce};
    if (launch(R.f_cyinit, 1, a, 32)) return -1;
    RR_TRY(cuStreamSynchronize(R.stream), "cylinder init");
    R.has_z = true;
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

namespace {

int launch_state2(void) {
    void* at[] = {&R.NN, &R.m, &R.theta, &R.NL, &R.w, &R.fail, &R.e, &R.idist, &R.fac, &R.x, &R.ux, &R.y, &R.uy};
    void* as[] = {&R.NN, &R.m, &R.theta, &R.fail, &R.NL, &R.e,  &R.w, &R.idist,
                  &R.fac, &R.x, &R.ux, &R.fx, &R.y, &R.uy, &R.fy};
    const unsigned g2 = (unsigned)(((int64_t)R.p.N * R.p.MN - 1) / 256 + 1);
    const unsigned g4 = (unsigned)(((int64_t)R.p.N_int * R.p.MN - 1) / 256 + 1);
    if (launch(R.f_theta2, g2, at)) return -1;
    return launch(R.f_state2, g4, as);
}

}  // namespace

// One state-based force evaluation: kernel_cal_theta_2D, kernel_state_force_2D.
int rr_force_state(void) {
    if (!R.ready || !R.has_state) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup_state first");
    if (launch_state2()) return -1;
    RR_TRY(cuStreamSynchronize(R.stream), "force state");
    return 0;
}

// nsteps of the crack-grow driver's loop (Solve_Plate_Crack_Grow.cu:126-149):
// boundary motion, integrate_2D_1, cal_theta_2D, state_force_2D,
// integrate_2D_2; kernel_cal_dmg_2D every dmg_every steps (0: never).
int rr_run_state(int nsteps, double load, int dmg_every, double* ms) {
    if (!R.ready || !R.has_state) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup_state first");
    void* aq[] = {&load, &R.uy};
    void* a1[] = {&R.vx, &R.ax, &R.ux, &R.vy, &R.ay, &R.uy};
    void* a2[] = {&R.vx, &R.ax, &R.fx, &R.bx, &R.vy, &R.ay, &R.fy, &R.by};
    void* ad[] = {&R.NN, &R.dmg, &R.fail, &R.fac};
    const unsigned gQ = (unsigned)((6 * R.p.nx - 1) / 256 + 1);
    const unsigned g3 = (unsigned)((R.p.N_int - 1) / 256 + 1);
    const unsigned g4 = (unsigned)(((int64_t)R.p.N_int * R.p.MN - 1) / 256 + 1);
    CUevent e0, e1;
    RR_TRY(cuEventCreate(&e0, CU_EVENT_DEFAULT), "event");
    RR_TRY(cuEventCreate(&e1, CU_EVENT_DEFAULT), "event");
    RR_TRY(cuEventRecord(e0, R.stream), "record");
    for (int s = 0; s < nsteps; s++) {
        if (load != 0.0 && launch(R.f_qload, gQ, aq)) return -1;
        if (launch(R.f_int1, g3, a1)) return -1;
        if (launch_state2()) return -1;
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

// Set the third displacement component (N doubles).
int rr_set_disp_z(const double* uz) {
    if (!R.ready || !R.has_z) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup_z first");
    RR_TRY(cuMemcpyHtoD(R.uz, uz, (size_t)R.p.N * 8), "uz");
    return 0;
}

// One kernel_bond_force_3D evaluation (rr_setup_z first).
int rr_force3(void) {
    if (!R.ready || !R.has_z) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup_z first");
    void* a[] = {&R.x, &R.ux, &R.fx, &R.y, &R.uy, &R.fy, &R.z, &R.uz, &R.fz, &R.NN, &R.NL, &R.idist, &R.scr,
                 &R.fail, &R.fac};
    const unsigned gS = (unsigned)(((int64_t)R.p.N * R.p.MN - 1) / 256 + 1);
    if (launch(R.f_bond3, gS, a, 256, 3 * 256 * sizeof(double))) return -1;
    RR_TRY(cuStreamSynchronize(R.stream), "force3");
    return 0;
}

// nsteps of the impact driver's loop (Solve_Kalthoff_Winkler.cu:406-430):
// integrate_3D_1, cy_integrate_1, bond_force_3D, contact, integrate_3D_2,
// cy_integrate_2.  Elapsed time of the loop (CUDA events) in *ms.
int rr_run_kw(int nsteps, double* ms) {
    if (!R.ready || !R.has_z) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup_z first");
    int loc_begin = R.p.N_int - R.p.nx * R.p.ny;  // unused by kernel_contact (its use is commented out)
    void* a1[] = {&R.vx, &R.ax, &R.ux, &R.vy, &R.ay, &R.uy, &R.uz, &R.vz, &R.az};  // declared order, see above
    void* ac1[] = {&R.cvel, &R.cdisp, &R.cacc};
    void* af[] = {&R.x, &R.ux, &R.fx, &R.y, &R.uy, &R.fy, &R.z, &R.uz, &R.fz, &R.NN, &R.NL, &R.idist, &R.scr,
                  &R.fail, &R.fac};
    void* ak[] = {&loc_begin, &R.dmg, &R.x, &R.ux, &R.vx, &R.y, &R.uy, &R.vy, &R.z, &R.uz, &R.vz, &R.cforce,
                  &R.cdisp};
    void* a2[] = {&R.vx, &R.ax, &R.fx, &R.bx, &R.vy, &R.ay, &R.fy, &R.by, &R.vz, &R.az, &R.fz, &R.bz};
    void* ac2[] = {&R.cvel, &R.cacc, &R.cforce};
    const unsigned g1 = (unsigned)((R.p.N - 1) / 256 + 1);
    const unsigned g2 = (unsigned)(((int64_t)R.p.N * R.p.MN - 1) / 256 + 1);
    const unsigned g3 = (unsigned)((R.p.N_int - 1) / 256 + 1);
    CUevent e0, e1;
    RR_TRY(cuEventCreate(&e0, CU_EVENT_DEFAULT), "event");
    RR_TRY(cuEventCreate(&e1, CU_EVENT_DEFAULT), "event");
    RR_TRY(cuEventRecord(e0, R.stream), "record");
    for (int s = 0; s < nsteps; s++) {
        if (launch(R.f_int31, g3, a1)) return -1;
        if (launch(R.f_cy1, 1, ac1, 32)) return -1;
        if (launch(R.f_bond3, g2, af, 256, 3 * 256 * sizeof(double))) return -1;
        if (launch(R.f_contact, g1, ak)) return -1;
        if (launch(R.f_int32, g3, a2)) return -1;
        if (launch(R.f_cy2, 1, ac2, 32)) return -1;
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

// Third-component node fields (N doubles each; NULL skips) and the impactor
// state cyl[12] = acc, disp, vel, force (3 each; NULL skips).
int rr_get_z(double* uz, double* vz, double* fz, double* cyl) {
    if (!R.ready || !R.has_z) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup_z first");
    const size_t N = (size_t)R.p.N;
    RR_TRY(cuStreamSynchronize(R.stream), "sync");
    if (uz) RR_TRY(cuMemcpyDtoH(uz, R.uz, N * 8), "uz");
    if (vz) RR_TRY(cuMemcpyDtoH(vz, R.vz, N * 8), "vz");
    if (fz) RR_TRY(cuMemcpyDtoH(fz, R.fz, N * 8), "fz");
    if (cyl) {
        RR_TRY(cuMemcpyDtoH(cyl, R.cacc, 24), "cylinder acc");
        RR_TRY(cuMemcpyDtoH(cyl + 3, R.cdisp, 24), "cylinder disp");
        RR_TRY(cuMemcpyDtoH(cyl + 6, R.cvel, 24), "cylinder vel");
        RR_TRY(cuMemcpyDtoH(cyl + 9, R.cforce, 24), "cylinder force");
    }
    return 0;
}

// State-based arrays of a 3-D problem set up by rr_setup and rr_setup_z: m (N
// doubles) and w (N*MN padded ELL); theta (N) and e (N*MN) start at zero.
int rr_setup_state3(const double* m, const double* w) {
    if (!R.ready || !R.has_z) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup_z first");
    const size_t N = (size_t)R.p.N, S = (size_t)R.p.N * R.p.MN;
    CUdeviceptr* arrs[] = {&R.m, &R.theta, &R.w, &R.e};
    const size_t bytes[] = {(N + kNodePad) * 8, (N + kNodePad) * 8, S * 8, S * 8};
    for (int k = 0; k < 4; k++) {
        if (*arrs[k]) {
            cuMemFree(*arrs[k]);
            *arrs[k] = 0;
        }
        RR_TRY(cuMemAlloc(arrs[k], bytes[k]), "state3 alloc");
        RR_TRY(cuMemsetD8(*arrs[k], 0, bytes[k]), "state3 zero");
    }
    RR_TRY(cuMemcpyHtoD(R.m, m, N * 8), "m copy");
    RR_TRY(cuMemcpyHtoD(R.w, w, S * 8), "w copy");
    R.has_state3 = true;
    return 0;
}

// kernel_initial_weight_3D over N*MN threads with 256 doubles of shared
// memory (the driver's commented launch, Solve_Kalthoff_Winkler.cu:400-401):
// overwrites m and w.  Refused for odd N (see the note at the top).
int rr_initial_weight3(void) {
    if (!R.has_state3) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup_state3 first");
    if (R.p.N % 2 != 0 || R.p.MN != 128) return fail_with(CUDA_ERROR_INVALID_VALUE, "N odd or MN != 128");
    void* a[] = {&R.m, &R.NN, &R.w, &R.idist, &R.fac};
    const unsigned g = (unsigned)(((int64_t)R.p.N * R.p.MN - 1) / 256 + 1);
    if (launch(R.f_weight3, g, a, 256, 256 * sizeof(double))) return -1;
    RR_TRY(cuStreamSynchronize(R.stream), "initial weight 3D");
    return 0;
}

// Dilatation theta (N doubles) and per-bond extension e (N*MN padded ELL), the
// inputs kernel_cal_theta_3D would have written.
int rr_set_theta_e(const double* theta, const double* e) {
    if (!R.has_state3) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup_state3 first");
    RR_TRY(cuMemcpyHtoD(R.theta, theta, (size_t)R.p.N * 8), "theta copy");
    RR_TRY(cuMemcpyHtoD(R.e, e, (size_t)R.p.N * R.p.MN * 8), "e copy");
    return 0;
}

// One kernel_state_force_3D evaluation over N_int*MN threads with 3*256
// doubles of shared memory (Solve_Kalthoff_Winkler.cu:420-422).  Refused for
// odd N_int (see the note at the top).
int rr_force_state3(void) {
    if (!R.has_state3) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup_state3 first");
    if (R.p.N_int % 2 != 0 || R.p.MN != 128) return fail_with(CUDA_ERROR_INVALID_VALUE, "N_int odd or MN != 128");
    void* a[] = {&R.NN, &R.m, &R.theta, &R.fail, &R.NL, &R.e, &R.w, &R.idist, &R.fac,
                 &R.x,  &R.ux, &R.fx,   &R.y,    &R.uy, &R.fy, &R.z, &R.uz,    &R.fz};
    const unsigned g = (unsigned)(((int64_t)R.p.N_int * R.p.MN - 1) / 256 + 1);
    if (launch(R.f_state3, g, a, 256, 3 * 256 * sizeof(double))) return -1;
    RR_TRY(cuStreamSynchronize(R.stream), "state force 3D");
    return 0;
}

// m (N doubles) and w (N*MN) of the 3-D state-based arrays.
int rr_get_state3(double* m, double* w) {
    if (!R.has_state3) return fail_with(CUDA_ERROR_NOT_INITIALIZED, "rr_setup_state3 first");
    RR_TRY(cuStreamSynchronize(R.stream), "sync");
    if (m) RR_TRY(cuMemcpyDtoH(m, R.m, (size_t)R.p.N * 8), "m");
    if (w) RR_TRY(cuMemcpyDtoH(w, R.w, (size_t)R.p.N * R.p.MN * 8), "w");
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
    R.has_z = false;
    R.has_state = false;
    R.has_state3 = false;
    return 0;
}

}  // extern "C"
