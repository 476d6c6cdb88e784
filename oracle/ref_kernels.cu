// Compiles the reference's OWN kernels (CosmosCuda.cuh of
// tugrul512bit/CosmosSimulationWithCuda, unmodified) to PTX -- TEST
// INFRASTRUCTURE for the oracle harness (oracle/ref_runner.cpp).
//
// The reference fixes N, dt and the gravity multiplier at compile time
// (Constants, CosmosCuda.cuh:29-74, with the __OVERRIDE_CONSTANTS__ hook it
// provides for exactly this), so oracle/ref_build.py compiles this file once
// per (REF_N, REF_DT, REF_G).  The header is included from the reference tree
// (-I <reference root>); nothing of it is copied here.  Only the kernel
// templates are instantiated; the Universe host class is not used.
#include <cfloat>
#include <condition_variable>
#include <ctime>
#include <thread>

#define __OVERRIDE_CONSTANTS__
namespace OVERRIDE_CONSTANTS {
constexpr int THREADS = 768;
constexpr int NUM_CUDA_DEVICES = 1;
constexpr int N = REF_N;
constexpr float dt = REF_DT;
constexpr float gravityMultiplier = REF_G;
constexpr int MAX_FRAMES_BUFFERED = 4;
constexpr int BLUR_R = 3;
}  // namespace OVERRIDE_CONSTANTS

#include "CosmosCuda.cuh"

// The step kernels (CosmosCuda.cuh:89-612) for lattice size REF_N.
template __global__ void Kernels::k_generateFilterLattice<REF_N>(ComplexVar*, bool);
template __global__ void Kernels::k_generateMassAssignmentKernel<REF_N>(ComplexVar*, bool);
template __global__ void Kernels::k_applyPhaseShift<REF_N>(ComplexVar*, float, float);
template __global__ void Kernels::k_clearAccumulator<REF_N>(float* const);
template __global__ void Kernels::k_scatterMassOnAccumulator<REF_N>(float* const, const float4* const,
                                                                    const float4* const, const float4* const,
                                                                    const int, bool);
template __global__ void Kernels::k_copyAccumulatorIntoLattice<REF_N>(float* const, ComplexVar* const);
template __global__ void Kernels::k_getRealComponentOfLattice<REF_N>(ComplexVar*, float*);
template __global__ void Kernels::k_multElementwiseLatticeFilter<REF_N>(ComplexVar*, ComplexVar*);
template __global__ void Kernels::k_divElementwiseLatticeFilter<REF_N>(ComplexVar*, ComplexVar*);
template __global__ void Kernels::k_shiftLattice<REF_N>(ComplexVar*, float*, bool);
template __global__ void Kernels::k_calcGradientLattice<REF_N>(const float* const, float2* const);
template __global__ void Kernels::k_forceMultiSampling<REF_N>(const float2* const, float* const, float* const,
                                                              float* const, float* const, const int, const bool);

// The render chain (CosmosCuda.cuh:613-828, launched at :1250-1255).
template __global__ void Kernels::k_calcBlurConvolution<3, REF_N>(const float* const __restrict__,
                                                                 float* const __restrict__);
template __global__ void Kernels::k_calcMinMax<REF_N>(float*);
template __global__ void Kernels::k_scaleWithMinMax<REF_N>(float*, float*);
