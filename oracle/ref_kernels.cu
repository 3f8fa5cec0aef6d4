// Test/measurement infrastructure only: the reference's GPU kernels, compiled
// from the reference sources where they lie (the recipe in oracle/Makefile
// passes their directory with -I) into a cubin for sm_103a.  Device code does
// not depend on the host architecture, so the cubin built on any host can be
// loaded on an Arm or x86 GPU host by oracle/ref_gpu_runner.cpp through the CUDA driver API and
// timed beside the engine.  The kernels are the reference's, unmodified; this
// file only defines the constant-memory parameter blocks that main.cu defines
// (main.cu:6-7) and one harness kernel (below).  Solve_Kalthoff_Winkler.cu is
// included for the impact driver's own kernels (cylinder start and halves,
// contact); its host function is parsed but not part of the cubin.
#include "Base.cuh"
#include "Neighbor.cu"
#include "Force_Bond.cu"
#include "Force_State.cu"
#include "Integrate.cu"
#include "Base_Function.cu"
#include "Reduce.cu"
#include "Solve_Kalthoff_Winkler.cu"

__constant__ device_parameter dp;
__constant__ Cylinder_Parameter dcyp;

// Harness kernel, not the reference's: the moving boundary rows of the
// crack-plate driver (kernel_quick_load, Solve_Plate_Crack_Grow.cu:8-19) are a
// file-static kernel of that driver, so the runner launches this restatement
// of its two statements instead (rows N_int.. move up 3 nx, then down 3 nx).
extern "C" __global__ void harness_quick_load(double load, double* disp_y) {
    unsigned int i = threadIdx.x + blockDim.x * blockIdx.x;
    if (i < 3 * dp.nx)
        disp_y[dp.N_int + i] += load * dp.dt;
    else if (i < 6 * dp.nx)
        disp_y[dp.N_int + i] -= load * dp.dt;
}
