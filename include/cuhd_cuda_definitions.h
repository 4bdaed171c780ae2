// CUDA error macro of the reference API (include/cuhd_cuda_definitions.h:21-28):
// on a pending CUDA error, print it and exit(1).
#ifndef CUHD_CUDA_DEFINITIONS_
#define CUHD_CUDA_DEFINITIONS_

#include <cstdlib>
#include <iostream>

#include <cuda_runtime.h>

#define CUERR                                                                    \
    {                                                                            \
        cudaError_t cuhd_err_ = cudaGetLastError();                              \
        if (cuhd_err_ != cudaSuccess) {                                          \
            std::cout << "CUDA error: " << cudaGetErrorString(cuhd_err_) << " : " \
                      << __FILE__ << ", line " << __LINE__ << std::endl;         \
            std::exit(1);                                                        \
        }                                                                        \
    }

#endif
