// device_launch_parameters.h -- empty stand-in for the host emulation of the reference engine
// (test infrastructure; see cuda_runtime.h in this directory).  The engine
// includes this header but uses nothing from it.
#pragma once
#include "cuda_runtime.h"
