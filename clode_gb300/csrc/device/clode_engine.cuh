// Second part of every ensemble program, included after the user's model
// source: steppers, observers and the kernel entry points.
#pragma once
#include "clode_steppers.cuh"
#include "clode_observers.cuh"
#include "clode_kernels.cuh"
