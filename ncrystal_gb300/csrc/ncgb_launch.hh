// Host-callable launchers of the kernels in ncgb_kernels.cu.
#ifndef NCGB_LAUNCH_HH
#define NCGB_LAUNCH_HH

#include <cstdint>
#include <cuda_runtime.h>
#include "ncgb_tables.h"

namespace ncgb {

  // Device-side counters.  launchScatter zeroes the queue counters at the
  // start of every batch; the caller zeroes nfail when it wants a new count.
  // The S(alpha,beta) queue holds one or two lists in one buffer of n_out
  // entries (two for one material, either for a ragged batch):
  // the main list from the front (entries 0 .. qcount-1), and from the back
  // (entries n_out-1, n_out-2, ...) the rare list: neutrons of free-gas
  // components and neutrons above a component's energy grid, which the
  // free-gas sampler and extender serve.  A neutron is in at most one list.
  struct Work {
    unsigned long long nfail;  // neutrons with a non-OK status
    unsigned int qcount;       // main list length
    unsigned int qnext;        // next main entry to claim
    unsigned int rcount;       // rare list length
    unsigned int rnext;        // next rare entry to claim
  };

  // A neutron queued for S(alpha,beta) sampling: 16 bytes.
  struct QEntry {
    double ekin;
    uint32_t idx;     // output index o
    uint16_t mat;     // material of a multi-material batch (0 otherwise)
    uint8_t comp;     // SAB component
    uint8_t ndraws;   // random numbers already drawn (the component pick)
  };

  // One material of a multi-material batch, in device memory.
  struct MatSlot {
    ncgb_material_view view;
    uint64_t seed;
    uint32_t stream;
    uint32_t pad;
  };

  // Launch shape (autotuned for multi-material batches): threads per block of
  // the pick pass (128/256/512), resident blocks per SM of the persistent
  // S(alpha,beta) pass (0 = as many as fit).
  struct LaunchCfg {
    int pick_block = 256;
    int sab_blocks_per_sm = 0;
    int split_lists = 0;   // ragged batches: main and rare lists (1) or one list (0)
  };

  // One batch: neutron o (< n_out) has energy ekin[o % n_ekin] and draws
  // from stream (seed, o + index_offset, callseq, stream); in multi-material
  // launches index_offset is the global index of the launch's first neutron.
  struct Batch {
    const void* ekin;
    int in_f32;
    int out_f32;
    uint64_t n_ekin, n_out;
    uint64_t seed;
    uint32_t callseq, stream, index_offset;
    int mode;          // 0: out_a = E', out_b = mu;  1: out_a = acos(mu), out_b = E'-E
    int fast;          // mixed-precision mode (FP32 transcendentals outside the
                       // beta-CDF inversion and the kinematics)
    int learned;       // learned beta proposal where a component has one attached
    void* out_xs;      // may be null
    void* out_a;       // may be null
    void* out_b;       // may be null
    void* out_xs_abs;      // absorption cross-sections (AbsOOV) beside the scattering ones, or null
    const double* dir_in;  // [n_ekin][3] incoming directions (sampleScatter with directions), or null
    double* dir_out;       // [n_out][3] outgoing directions, or null
    int32_t* status;   // may be null
    const uint32_t* rng_index;   // if set (with directions only): neutron o draws from stream
                                 // (seed, rng_index[o], callseq, stream) instead
    int untimed;       // never record phase-timing events for this batch
    int reorder;       // the pick pass may visit each tile's neutrons in energy order
                       // (materials with PowderBragg components; never where the
                       // kernels read and write host memory directly)
    unsigned long long* phase_cycles;  // non-null (single material, no directions): run the
                                       // S(alpha,beta) pass with phase clocks, summing the
                                       // lanes' cycles per phase and their Alg.1 attempts here
                                       // (ncgb_dev::PH_N + 1 counters)
    Work* work;        // scratch, sizeof(Work)
    QEntry* queue;     // scratch, n_out entries
  };

  // pickDone (optional) is recorded on s between the two passes: the
  // cross-sections are final from then on.
  cudaError_t launchScatter( const ncgb_material_view& m, const Batch& b, cudaStream_t s,
                             cudaEvent_t pickDone = nullptr );
  // Ragged multi-material batch: neutrons [d_offsets[k], d_offsets[k+1]) use
  // material k, drawing from stream (seed_k, o - d_offsets[k], callseq, stream_k).
  cudaError_t launchScatterMulti( const MatSlot* d_slots, const int64_t* d_offsets, int nmat,
                                  const Batch& b, const LaunchCfg& cfg, cudaStream_t s,
                                  cudaEvent_t pickDone = nullptr );
  int maxSabBlocksPerSM();
  // (alpha, beta) of component 'comp' per neutron: out_a = alpha, out_b = beta;
  // neutron i uses stream (seed, index_offset + i, callseq, stream); failures
  // counted in work->nfail.
  cudaError_t launchSabAB( const ncgb_material_view& m, int comp, const Batch& b, cudaStream_t s );
  // Absorption cross-sections c/sqrt(E) (AbsOOV) into out_xs, repeat layout as launchXS.
  cudaError_t launchAbsXS( double abs_c, const Batch& b, uint64_t repeat, cudaStream_t s );
  cudaError_t launchXS( const ncgb_material_view& m, const Batch& b, uint64_t repeat, cudaStream_t s );
  int scatterLaunchesPerBatch();
  void setPhaseTiming( bool on );
  bool phaseTiming();
  int takePhaseTimes( double* ms_pick, double* ms_sab, unsigned long* nbatches );
}

#endif
