// Allocation-free cell macros (implementation and rationale: noalloc.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "device_common.cuh"

namespace dugks {

// Largest cell count dugks_macros_noalloc accepts (its static scratch holds
// 5 doubles per cell).
constexpr int kNoAllocMaxCells = 262144;

int macros_noalloc(const StepArgs& a, int device, cudaStream_t s, const double* g, const double* h, double* rho,
                   double* U, double* T, double* q, std::string& err);

}  // namespace dugks
