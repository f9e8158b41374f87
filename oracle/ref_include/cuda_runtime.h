/* Host stand-in for <cuda_runtime.h>, used only to compile the reference's
 * kernel sections as plain C++ for the CPU oracle (oracle/_ref). */
#ifndef BDREF_CUDA_RUNTIME_STUB_H
#define BDREF_CUDA_RUNTIME_STUB_H
#include "../ref_stub.h"
#endif
