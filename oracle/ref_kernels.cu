// Test/measurement infrastructure only: the reference's GPU kernels, compiled
// from the reference sources where they lie (the recipe in oracle/Makefile
// passes their directory with -I) into a cubin for sm_103a.  Device code does
// not depend on the host architecture, so the cubin built here can be loaded
// on the GPU machine by oracle/ref_gpu_runner.cpp through the CUDA driver API and
// timed beside the engine.  The kernels are the reference's, unmodified; this
// file only defines the constant-memory parameter blocks that main.cu defines
// (main.cu:6-7).
#include "Base.cuh"
#include "Neighbor.cu"
#include "Force_Bond.cu"
#include "Force_State.cu"
#include "Integrate.cu"
#include "Base_Function.cu"

__constant__ device_parameter dp;
__constant__ Cylinder_Parameter dcyp;
