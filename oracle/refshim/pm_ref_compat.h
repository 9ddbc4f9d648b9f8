// Forced include for compiling the reference's PatchMatchCuda.cu unmodified
// with CUDA 13: cudaThreadSynchronize was removed (same semantics as
// cudaDeviceSynchronize), and its unused printDevProp reads cudaDeviceProp
// fields that CUDA 13 dropped, so that one type gains them here.
#pragma once
#include <cuda_runtime.h>
struct pm_ref_devprop : public cudaDeviceProp {
    int clockRate;
    int deviceOverlap;
    int kernelExecTimeoutEnabled;
};
#define cudaDeviceProp pm_ref_devprop
#define cudaThreadSynchronize cudaDeviceSynchronize
