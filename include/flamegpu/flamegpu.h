#ifndef INCLUDE_FLAMEGPU_FLAMEGPU_H_
#define INCLUDE_FLAMEGPU_FLAMEGPU_H_
// Umbrella header for model code: the same include the reference's models use.
#include "flamegpu/defines.h"
#include "flamegpu/exception/FLAMEGPUException.h"
#include "flamegpu/runtime/DeviceAPI.cuh"
#include "flamegpu/runtime/AgentFunction.cuh"
#include "flamegpu/model/ModelDescription.h"
#include "flamegpu/simulation/AgentVector.h"
#include "flamegpu/simulation/CUDASimulation.h"
#include "flamegpu/simulation/CUDAEnsemble.h"
#include "flamegpu/simulation/SimulationServer.h"
#ifdef __CUDACC__
#include "flamegpu/runtime/HostReductions.cuh"
#endif
#endif  // INCLUDE_FLAMEGPU_FLAMEGPU_H_
