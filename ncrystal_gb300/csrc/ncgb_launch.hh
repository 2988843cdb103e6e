// Host-callable launchers of the kernels in ncgb_kernels.cu.
#ifndef NCGB_LAUNCH_HH
#define NCGB_LAUNCH_HH

#include <cstdint>
#include <cuda_runtime.h>
#include "ncgb_tables.h"

namespace ncgb {

  // Device-side counters.  launchScatter zeroes the queue counters at the
  // start of every batch; the caller zeroes nfail when it wants a new count.
  struct Work {
    unsigned long long nfail;  // neutrons with a non-OK status
    unsigned int qcount;       // SAB queue length
    unsigned int qnext;        // next queue entry to claim
  };

  // A neutron queued for S(alpha,beta) sampling: 16 bytes.
  struct QEntry {
    double ekin;
    uint32_t idx;     // output index o (stream neutron index o + index_offset)
    uint16_t comp;    // SAB component
    uint16_t ndraws;  // random numbers already drawn (the component pick)
  };

  // One batch: neutron o (< n_out) has energy ekin[o % n_ekin] and draws
  // from stream (seed, o + index_offset, callseq, stream).
  struct Batch {
    const void* ekin;
    int in_f32;
    int out_f32;
    uint64_t n_ekin, n_out;
    uint64_t seed;
    uint32_t callseq, stream, index_offset;
    int mode;          // 0: out_a = E', out_b = mu;  1: out_a = acos(mu), out_b = E'-E
    void* out_xs;      // may be null
    void* out_a;       // may be null
    void* out_b;       // may be null
    int32_t* status;   // may be null
    Work* work;        // scratch, sizeof(Work)
    QEntry* queue;     // scratch, n_out entries
  };

  cudaError_t launchScatter( const ncgb_material_view& m, const Batch& b, cudaStream_t s );
  cudaError_t launchXS( const ncgb_material_view& m, const Batch& b, uint64_t repeat, cudaStream_t s );
  int scatterLaunchesPerBatch();
  void setPhaseTiming( bool on );
  int takePhaseTimes( double* ms_pick, double* ms_sab, unsigned long* nbatches );
}

#endif
