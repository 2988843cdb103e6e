// CUDA kernels of the batched non-oriented scattering path (sm_103a).
//
// One thread per output element.  The material's flat table view (~5 KB) is
// passed by value as a __grid_constant__ kernel parameter, so its scalars sit
// in the constant bank and every warp reads them with broadcast loads; the
// tables themselves stay in HBM / L2.  Inputs and outputs are contiguous
// arrays (structure of arrays), read and written once, coalesced.
#include <cuda_runtime.h>
#include <cstdint>

#include "ncgb_device.cuh"
#include "ncgb_launch.hh"

namespace {

  template<class T> __device__ __forceinline__ double toD( T v ) { return static_cast<double>(v); }
  template<class T> __device__ __forceinline__ T fromD( double v ) { return static_cast<T>(v); }

  // Fused: xs + one scatter per neutron, neutron index = i.
  template<class InT, class OutT>
  __global__ void __launch_bounds__(256)
  k_xs_scatter( const __grid_constant__ ncgb_material_view m,
                const InT* __restrict__ ekin, uint64_t n,
                uint64_t seed, uint32_t callseq, uint32_t stream, uint32_t index_offset,
                OutT* __restrict__ out_xs, OutT* __restrict__ out_ef, OutT* __restrict__ out_mu,
                int32_t* __restrict__ out_status, unsigned long long* __restrict__ nfail )
  {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for ( uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride ) {
      const double e = toD( ekin[i] );
      ncgb_rng rng;
      ncgb_rng_init( &rng, seed, (uint32_t)i + index_offset, callseq, stream );
      double xs, ef, mu;
      const int st = ncgb_dev::evalNeutron<true,true>( m, rng, e, xs, ef, mu );
      if ( out_xs ) out_xs[i] = fromD<OutT>( xs );
      if ( out_ef ) out_ef[i] = fromD<OutT>( ef );
      if ( out_mu ) out_mu[i] = fromD<OutT>( mu );
      if ( out_status ) out_status[i] = st;
      if ( st != NCGB_ST_OK ) atomicAdd( nfail, 1ull );
    }
  }

  // Cross-sections only: results[r*n_ekin+i] = xs(ekin[i]) for r < repeat
  // (ncrystal.cc:1107-1141 writes the same value for every repeat).
  template<class InT, class OutT>
  __global__ void __launch_bounds__(256)
  k_xs( const __grid_constant__ ncgb_material_view m,
        const InT* __restrict__ ekin, uint64_t n_ekin, uint64_t repeat,
        OutT* __restrict__ out )
  {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for ( uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_ekin; i += stride ) {
      ncgb_rng dummy;
      double xs, ef, mu;
      ncgb_dev::evalNeutron<true,false>( m, dummy, toD( ekin[i] ), xs, ef, mu );
      for ( uint64_t r = 0; r < repeat; ++r )
        out[r * n_ekin + i] = fromD<OutT>( xs );
    }
  }

  // Scatters for the _many calls: output index o = irepeat*n_ekin + i, energy
  // ekin[i], stream neutron index o.  mode 0: (E', mu); mode 1: (acos(mu),
  // E'-E) as ncrystal_genscatter_nonoriented_many.
  __global__ void __launch_bounds__(256)
  k_scatter_many( const __grid_constant__ ncgb_material_view m,
                  const double* __restrict__ ekin, uint64_t n_ekin, uint64_t n_out,
                  uint64_t seed, uint32_t callseq, uint32_t stream, int mode,
                  double* __restrict__ out_a, double* __restrict__ out_b,
                  unsigned long long* __restrict__ nfail )
  {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for ( uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; o < n_out; o += stride ) {
      const uint64_t i = o % n_ekin;
      const double e = ekin[i];
      ncgb_rng rng;
      ncgb_rng_init( &rng, seed, (uint32_t)o, callseq, stream );
      double xs, ef, mu;
      const int st = ncgb_dev::evalNeutron<false,true>( m, rng, e, xs, ef, mu );
      if ( st != NCGB_ST_OK ) {
        atomicAdd( nfail, 1ull );
        if ( mode == 1 )
          continue; // genscatter: outputs for failed neutrons are left untouched
      }
      if ( mode == 0 ) {
        out_a[o] = ef;
        out_b[o] = mu;
      } else {
        out_a[o] = acos( mu );
        out_b[o] = ef - e;
      }
    }
  }

  int gridFor( uint64_t n, int block )
  {
    static int nsm = 0;
    if ( !nsm ) {
      int dev = 0;
      cudaGetDevice( &dev );
      cudaDeviceGetAttribute( &nsm, cudaDevAttrMultiProcessorCount, dev );
      if ( nsm <= 0 ) nsm = 1;
    }
    uint64_t want = ( n + block - 1 ) / block;
    uint64_t cap = (uint64_t)nsm * 16; // grid-stride beyond 16 resident blocks per SM
    if ( want > cap ) want = cap;
    if ( want < 1 ) want = 1;
    return (int)want;
  }
}

namespace ncgb {

  cudaError_t launchXSScatter( const ncgb_material_view& m, const double* ekin, uint64_t n,
                               uint64_t seed, uint32_t callseq, uint32_t stream, uint32_t index_offset,
                               double* xs, double* ef, double* mu, int32_t* status,
                               unsigned long long* nfail, cudaStream_t s )
  {
    if ( n == 0 ) return cudaSuccess;
    k_xs_scatter<double,double><<<gridFor(n,256),256,0,s>>>( m, ekin, n, seed, callseq, stream, index_offset,
                                                             xs, ef, mu, status, nfail );
    return cudaGetLastError();
  }

  cudaError_t launchXSScatterF32( const ncgb_material_view& m, const float* ekin, uint64_t n,
                                  uint64_t seed, uint32_t callseq, uint32_t stream, uint32_t index_offset,
                                  float* xs, float* ef, float* mu, int32_t* status,
                                  unsigned long long* nfail, cudaStream_t s )
  {
    if ( n == 0 ) return cudaSuccess;
    k_xs_scatter<float,float><<<gridFor(n,256),256,0,s>>>( m, ekin, n, seed, callseq, stream, index_offset,
                                                           xs, ef, mu, status, nfail );
    return cudaGetLastError();
  }

  cudaError_t launchXS( const ncgb_material_view& m, const double* ekin, uint64_t n_ekin, uint64_t repeat,
                        double* out, cudaStream_t s )
  {
    if ( n_ekin == 0 || repeat == 0 ) return cudaSuccess;
    k_xs<double,double><<<gridFor(n_ekin,256),256,0,s>>>( m, ekin, n_ekin, repeat, out );
    return cudaGetLastError();
  }

  cudaError_t launchXSF32( const ncgb_material_view& m, const float* ekin, uint64_t n_ekin,
                           float* out, cudaStream_t s )
  {
    if ( n_ekin == 0 ) return cudaSuccess;
    k_xs<float,float><<<gridFor(n_ekin,256),256,0,s>>>( m, ekin, n_ekin, 1, out );
    return cudaGetLastError();
  }

  cudaError_t launchScatterMany( const ncgb_material_view& m, const double* ekin, uint64_t n_ekin, uint64_t n_out,
                                 uint64_t seed, uint32_t callseq, uint32_t stream, int mode,
                                 double* out_a, double* out_b, unsigned long long* nfail, cudaStream_t s )
  {
    if ( n_out == 0 ) return cudaSuccess;
    k_scatter_many<<<gridFor(n_out,256),256,0,s>>>( m, ekin, n_ekin, n_out, seed, callseq, stream, mode,
                                                    out_a, out_b, nfail );
    return cudaGetLastError();
  }
}
