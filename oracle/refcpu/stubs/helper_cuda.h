// Stand-in for the reference's vendored helper_cuda.h (which uses
// cudaDeviceProp fields removed in CUDA 13): only checkCudaErrors is used by
// the headers the CPU build includes.
#pragma once
#include <cuda_runtime.h>
#define checkCudaErrors(val) (val)
