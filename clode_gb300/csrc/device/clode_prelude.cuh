// First part of every ensemble program: precision, OpenCL-C shim, argument
// block and RNG, then the forward declaration of the user's right-hand side
// (signature of clode/cpp/steppers.cl:50).  The host appends the user's
// model source after this header and clode_engine.cuh after that.
#pragma once
#include "clode_shim.cuh"
#include "clode_args.h"

#include "clode_rng.cuh"

static __device__ __forceinline__ void getRHS(const realtype t, const realtype x_[], const realtype p_[],
                                              realtype dx_[], realtype aux_[], const realtype w_[]);
