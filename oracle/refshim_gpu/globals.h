/*
 * ORACLE build shim -- utils/include/globals.h for building the reference's
 * dedispersion/msosm/msosm_gpu_batch.cpp on the host: the planning shim's
 * declarations plus the CUDA complex type the processor's header uses
 * (globals.h:29, Complex = cufftComplex).
 */
#pragma once
#include "../refshim/globals.h"

#include <cuda_runtime.h>
#include <cufft.h>

typedef cufftComplex Complex;
