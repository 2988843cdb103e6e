// ncgb_scatter_device_noalloc: the fused cross-section + scatter batch on
// device arrays, with its working memory taken from a fixed array that is part
// of the library image instead of from cudaMalloc.
//
// Who needs this: a caller whose process reserves all device memory up front
// through its own pool (a transport code embedded in a larger framework that
// forbids other allocations), or one that cannot afford the device-wide
// synchronisation a cudaMalloc/cudaFree can cause in the middle of its
// transport loop.  The other device entry points grow per-thread working
// buffers with cudaMalloc on demand; this one never allocates.
//
// The working memory (the S(alpha,beta) queue and the batch counters) is the
// file-scope array below: 256 bytes of counters plus 16 bytes per neutron for
// at most NCGB_NOALLOC_MAX_NEUTRONS neutrons (16 MiB in all).  Every GPU that
// loads the library holds it until the process exits.  Every call shares it:
// calls whose kernels overlap on the GPU (e.g. on two streams without an
// ordering between them) race on it and give wrong results.  The counters are
// cleared at the start of every call; the queue needs no clearing.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address with cudaGetSymbolAddress (host code cannot use the
// array's name as a device address).  Make that first call before any stream
// capture.  The address is kept for the life of the device's primary context:
// after cudaDeviceReset (or after the primary context is released and
// created anew) the cached address is stale, so such a caller must not call
// this entry point again in the same process.
//
// Like ncgb_scatter_device it computes in the handle's arithmetic mode with
// the handle's sampler (the learned proposal needs no extra working memory),
// and an empty call or a refused call consumes no call sequence number, so a
// handle draws from the same random streams as with ncgb_scatter_device.  The
// library's optional phase timing (ncgb_phase_timing) creates CUDA events; it
// is never applied to this entry point's launches.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>

#include "ncgb_launch.hh"
#include "ncrystal_gb300.h"

namespace ncgb {
  void handleBatchInfo( ncrystal_scatter_t sc, const char* fct, ncgb_material_view* view, int* device,
                        uint64_t* seed, uint32_t* streamidx, int* fast, int* learned );
  uint32_t handleNextCall( ncrystal_scatter_t sc, const char* fct );
  void reportError( const std::exception& e );
  void reportError( const char* type, const std::string& msg );
}

namespace {

  constexpr std::size_t kCounterBytes = 256;
  constexpr std::size_t kScratchBytes = kCounterBytes + sizeof(ncgb::QEntry) * (std::size_t)NCGB_NOALLOC_MAX_NEUTRONS;
  static_assert( sizeof(ncgb::Work) <= kCounterBytes, "counters do not fit" );
  static_assert( sizeof(ncgb::QEntry) == 16, "queue entry layout" );

  static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

  constexpr int kMaxDevices = 64;
  std::mutex g_mtx;
  void* g_addr[kMaxDevices] = {};

  // Device address of the scratch array on the current device (looked up once
  // per device).
  void* scratchAddress( int device )
  {
    if ( device < 0 || device >= kMaxDevices )
      throw std::runtime_error( "device index out of range" );
    std::lock_guard<std::mutex> lock( g_mtx );
    if ( !g_addr[device] ) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress( &p, g_noalloc_scratch );
      if ( e != cudaSuccess || !p )
        throw std::runtime_error( std::string( "cudaGetSymbolAddress of the fixed scratch array failed: " )
                                  + cudaGetErrorString( e ) );
      g_addr[device] = p;
    }
    return g_addr[device];
  }
}

extern "C"
int ncgb_scatter_device_noalloc( ncrystal_scatter_t sc, const double* d_ekin, unsigned long n,
                                 double* d_xs, double* d_ef, double* d_mu, int32_t* d_status, void* stream )
{
  try {
    if ( n > NCGB_NOALLOC_MAX_NEUTRONS ) {
      ncgb::reportError( "BadInput", "ncgb_scatter_device_noalloc: " + std::to_string( n )
                         + " neutrons requested, but its fixed working memory holds at most "
                         + std::to_string( (unsigned long)NCGB_NOALLOC_MAX_NEUTRONS )
                         + " per call (split the batch, or use ncgb_scatter_device)" );
      return 1;
    }
    static const char* kFct = "ncgb_scatter_device_noalloc";
    ncgb_material_view view;
    int matdev = -1, fast = 0, learned = 0;
    uint64_t seed = 0;
    uint32_t streamidx = 0;
    ncgb::handleBatchInfo( sc, kFct, &view, &matdev, &seed, &streamidx, &fast, &learned );
    if ( n == 0 )
      return 0;
    int cur = -1;
    cudaError_t e = cudaGetDevice( &cur );
    if ( e != cudaSuccess )
      throw std::runtime_error( std::string( "cudaGetDevice: " ) + cudaGetErrorString( e ) );
    if ( cur != matdev ) {
      ncgb::reportError( "BadInput", "ncgb_scatter_device_noalloc: the current CUDA device is not the one"
                         " holding the material's tables" );
      return 1;
    }
    unsigned char* base = static_cast<unsigned char*>( scratchAddress( cur ) );
    cudaStream_t st = static_cast<cudaStream_t>( stream );
    e = cudaMemsetAsync( base, 0, sizeof(ncgb::Work), st );
    if ( e != cudaSuccess )
      throw std::runtime_error( std::string( "clearing the batch counters: " ) + cudaGetErrorString( e ) );
    ncgb::Batch b;
    std::memset( &b, 0, sizeof(b) );
    b.ekin = d_ekin;
    b.n_ekin = b.n_out = n;
    b.seed = seed;
    b.callseq = ncgb::handleNextCall( sc, kFct );
    b.stream = streamidx;
    b.fast = fast;
    b.learned = learned;
    b.untimed = 1;
    b.out_xs = d_xs;
    b.out_a = d_ef;
    b.out_b = d_mu;
    b.status = d_status;
    b.work = reinterpret_cast<ncgb::Work*>( base );
    b.queue = reinterpret_cast<ncgb::QEntry*>( base + kCounterBytes );
    e = ncgb::launchScatter( view, b, st );
    if ( e != cudaSuccess )
      throw std::runtime_error( std::string( "scatter kernels: " ) + cudaGetErrorString( e ) );
    return 0;
  } catch ( std::exception& ex ) {
    ncgb::reportError( ex );
  }
  return 1;
}
