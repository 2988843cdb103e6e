// Host-callable launchers of the kernels in ncgb_kernels.cu.
#ifndef NCGB_LAUNCH_HH
#define NCGB_LAUNCH_HH

#include <cstdint>
#include <cuda_runtime.h>
#include "ncgb_tables.h"

namespace ncgb {

  // Fused cross-section + scatter; neutron i uses stream index i+index_offset.
  cudaError_t launchXSScatter( const ncgb_material_view& m, const double* ekin, uint64_t n,
                               uint64_t seed, uint32_t callseq, uint32_t stream, uint32_t index_offset,
                               double* xs, double* ef, double* mu, int32_t* status,
                               unsigned long long* nfail, cudaStream_t s );
  cudaError_t launchXSScatterF32( const ncgb_material_view& m, const float* ekin, uint64_t n,
                                  uint64_t seed, uint32_t callseq, uint32_t stream, uint32_t index_offset,
                                  float* xs, float* ef, float* mu, int32_t* status,
                                  unsigned long long* nfail, cudaStream_t s );
  cudaError_t launchXS( const ncgb_material_view& m, const double* ekin, uint64_t n_ekin, uint64_t repeat,
                        double* out, cudaStream_t s );
  cudaError_t launchXSF32( const ncgb_material_view& m, const float* ekin, uint64_t n_ekin,
                           float* out, cudaStream_t s );
  // mode 0: (E', mu); mode 1: (acos(mu), E'-E).
  cudaError_t launchScatterMany( const ncgb_material_view& m, const double* ekin, uint64_t n_ekin, uint64_t n_out,
                                 uint64_t seed, uint32_t callseq, uint32_t stream, int mode,
                                 double* out_a, double* out_b, unsigned long long* nfail, cudaStream_t s );
}

#endif
