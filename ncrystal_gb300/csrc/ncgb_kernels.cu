// CUDA kernels of the batched non-oriented scattering path (sm_103a).
//
// A batch of neutrons is scattered in two launches:
//
//   k_pick   one thread per neutron: composition cross-section, component
//            pick, and the short samplers (PowderBragg, ElIncScatter) done in
//            place.  Neutrons that picked an S(alpha,beta) component are
//            appended to a queue (warp-aggregated atomics, 16 B per entry).
//   k_sab    persistent warps over the queue: each lane runs the SAB
//            sampler's flattened rejection loops one Alg.1 attempt per step
//            and takes the next queued neutron as soon as its own finishes,
//            so warps stay full while neutrons need different numbers of
//            attempts.
//
// Both are templated on where the material comes from:
//   SingleSrc  one material; its flat table view (~5 KB) is a
//              __grid_constant__ parameter, so its scalars sit in the constant
//              bank and warps read them with broadcast loads.
//   MultiSrc   a ragged batch of materials: a device array of views (with each
//              material's seed and stream index) and the offsets of each
//              material's neutrons; a neutron finds its material by a binary
//              search over the offsets.
// The tables themselves stay in HBM / L2.  Inputs and outputs are contiguous
// arrays, read and written once.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdlib>
#include <mutex>
#include <type_traits>
#include <vector>

#include "ncgb_device.cuh"
#include "ncgb_launch.hh"

namespace {

  using namespace ncgb_dev;

  struct SingleSrc {
    ncgb_material_view m;
    uint64_t seed;
    uint32_t stream, index_offset;
    int lean;                 // S(alpha,beta) and incoherent elastic components only (set by the host)
    int pad;
    __device__ __forceinline__ int find( uint64_t ) const { return 0; }
    __device__ __forceinline__ const ncgb_material_view& mat( int ) const { return m; }
    __device__ __forceinline__ void rngFor( ncgb_rng& r, int, uint64_t o, uint32_t callseq ) const
    {
      ncgb_rng_init( &r, seed, (uint32_t)o + index_offset, callseq, stream );
    }
    // A lane's stream before its first neutron: the launch's key and counters.
    __device__ __forceinline__ void rngIdle( ncgb_rng& r, uint32_t callseq ) const
    {
      ncgb_rng_init( &r, seed, index_offset, callseq, stream );
    }
    // main and rare lists in the S(alpha,beta) queue (see ncgb::Work)
    __device__ __forceinline__ bool splitLists() const { return true; }
  };

  // One material; neutron o's stream index read from a per-neutron array
  // (callers whose neutrons keep their streams while they move between
  // batches, such as the MiniMC engine).
  struct MappedSrc {
    ncgb_material_view m;
    uint64_t seed;
    uint32_t stream, pad;
    const uint32_t* index;
    int lean;                 // S(alpha,beta) and incoherent elastic components only (set by the host)
    int pad2;
    __device__ __forceinline__ int find( uint64_t ) const { return 0; }
    __device__ __forceinline__ const ncgb_material_view& mat( int ) const { return m; }
    __device__ __forceinline__ void rngFor( ncgb_rng& r, int, uint64_t o, uint32_t callseq ) const
    {
      ncgb_rng_init( &r, seed, __ldg( index + o ), callseq, stream );
    }
    __device__ __forceinline__ void rngIdle( ncgb_rng& r, uint32_t callseq ) const
    {
      ncgb_rng_init( &r, seed, 0, callseq, stream );
    }
    __device__ __forceinline__ bool splitLists() const { return true; }
  };

  struct MultiSrc {
    const ncgb::MatSlot* slots;
    const int64_t* offsets;   // [nmat+1]
    int nmat;
    int split;                // main and rare lists, or one list (chosen per batch by the autotuner)
    int64_t base;             // global index of this launch's first neutron (chunked host calls)
    // last k with offsets[k] <= g
    __device__ __forceinline__ int search( int64_t g ) const
    {
      int lo = 0, hi = nmat - 1;
      while ( lo < hi ) {
        const int mid = ( lo + hi + 1 ) >> 1;
        if ( __ldg( offsets + mid ) <= g ) lo = mid; else hi = mid - 1;
      }
      return lo;
    }
    // The material of neutron o.  Called by all active lanes of a warp
    // together: the first one searches, and a lane inside the same material
    // ([offsets[k], offsets[k+1]), neutrons are grouped by material) takes
    // its answer -- no later material starts at or below g, so it is the
    // same k -- and only the others search.
    __device__ __forceinline__ int find( uint64_t o ) const
    {
      const int64_t g = base + (int64_t)o;
      const unsigned m = __activemask();
      const int leader = __ffs( m ) - 1;
      int k = 0;
      if ( (int)( threadIdx.x & 31 ) == leader )
        k = search( g );
      k = __shfl_sync( m, k, leader );
      if ( __ldg( offsets + k ) <= g && g < __ldg( offsets + k + 1 ) )
        return k;
      return search( g );
    }
    __device__ __forceinline__ const ncgb_material_view& mat( int k ) const { return slots[k].view; }
    __device__ __forceinline__ void rngFor( ncgb_rng& r, int k, uint64_t o, uint32_t callseq ) const
    {
      const uint64_t local = (uint64_t)base + o - (uint64_t)__ldg( offsets + k );
      ncgb_rng_init( &r, slots[k].seed, (uint32_t)local, callseq, slots[k].stream );
    }
    // (key and stream differ between materials)
    __device__ __forceinline__ void rngIdle( ncgb_rng& r, uint32_t ) const
    {
      ncgb_rng_init( &r, 0, 0, 0, 0 );
    }
    __device__ __forceinline__ bool splitLists() const { return split != 0; }
  };

  __device__ __forceinline__ double loadE( const ncgb::Batch& b, uint64_t i )
  {
    return b.in_f32 ? (double)__ldg( static_cast<const float*>( b.ekin ) + i )
                    : __ldg( static_cast<const double*>( b.ekin ) + i );
  }

  __device__ __forceinline__ void store( void* p, int f32, uint64_t o, double v )
  {
    if ( !p ) return;
    if ( f32 ) static_cast<float*>( p )[o] = (float)v;
    else static_cast<double*>( p )[o] = v;
  }

  // Write one neutron's scatter result (mode 0: E', mu; mode 1: acos(mu), E'-E).
  // With directions (dir_out): the outgoing direction, sampled from the
  // neutron's stream after its scatter (ScatterIsotropicMat::sampleScatter,
  // NCProcImpl.cc:29-37); 'scattered' is false outside the material's domain,
  // where the direction is returned unchanged (NCProcImpl.cc:364-377).
  // (out of line: only calls with directions pay for it in registers)
  __device__ __noinline__ int writeDir( const ncgb::Batch& b, uint64_t o, int st, double mu, ncgb_rng& rng,
                                        bool scattered )
  {
    const uint64_t i = ( b.n_out == b.n_ekin ) ? o : o % b.n_ekin;
    const double* in = b.dir_in + 3 * i;
    double* out = b.dir_out + 3 * o;
    if ( st == NCGB_ST_OK && scattered )
      st = randDirGivenMu( rng, mu, in, out );
    else if ( st == NCGB_ST_OK ) {
      out[0] = in[0]; out[1] = in[1]; out[2] = in[2];
    }
    if ( st != NCGB_ST_OK ) {
      out[0] = 0.0; out[1] = 0.0; out[2] = 0.0;
    }
    return st;
  }

  template<bool Dir>
  __device__ __forceinline__ void writeScatter( const ncgb::Batch& b, uint64_t o, double e, int st,
                                                double ef, double mu, ncgb_rng& rng, bool scattered = true )
  {
    if ( Dir && b.dir_out ) {
      // a copy: the neutron's stream is not used after its result is written,
      // and the caller's state can stay in registers
      ncgb_rng r2 = rng;
      st = writeDir( b, o, st, mu, r2, scattered );
    }
    if ( b.status ) b.status[o] = st;
    if ( st != NCGB_ST_OK ) {
      atomicAdd( &b.work->nfail, 1ull );
      if ( b.mode == 1 )
        return; // genscatter: failed neutrons keep their outputs
      ef = -1.0;
      mu = -999.0;
    }
    if ( b.mode == 0 ) {
      store( b.out_a, b.out_f32, o, ef );
      store( b.out_b, b.out_f32, o, mu );
    } else {
      store( b.out_a, b.out_f32, o, acos( mu ) );
      store( b.out_b, b.out_f32, o, ef - e );
    }
  }

  // ---- phase 1: cross-section, pick, short samplers, SAB queue ----------------
  // One neutron of the pick pass (o: its output index; all lanes of the warp
  // that have a neutron call this together): cross-section, component pick,
  // the short samplers in place, or a warp-aggregated append to the
  // S(alpha,beta) queue.
  template<class Src, bool Fast, bool Dir, bool Lean = false>
  __device__ __forceinline__ void pickOne( const Src& src, const ncgb::Batch& b, uint64_t o )
  {
    {
      const uint64_t i = ( b.n_out == b.n_ekin ) ? o : o % b.n_ekin;
      const double e = loadE( b, i );
      const int k = src.find( o );
      const ncgb_material_view& m = src.mat( k );
      ncgb_rng rng;
      src.rngFor( rng, k, o, b.callseq );
      bool queue = false, rare = false;
      int qcomp = 0;
      if ( b.out_xs_abs )
        store( b.out_xs_abs, b.out_f32, o, absXS( m.abs_c, e ) );
      if ( !contains( m.dom_elow, m.dom_ehigh, e ) ) {
        // ProcComposition outside its domain: xs 0, neutron unchanged (NCProcImpl.cc:353-389)
        store( b.out_xs, b.out_f32, o, 0.0 );
        writeScatter<Dir>( b, o, e, NCGB_ST_OK, e, 1.0, rng, false );
      } else {
        const XSPick p = xsAndPick<true, Fast, Lean>( m, e, rng );
        store( b.out_xs, b.out_f32, o, p.xs );
        const ncgb_comp_view& c = m.comp[p.comp];
        int st = NCGB_ST_OK;
        double ef = e, mu = 1.0;
        switch ( c.type ) {
          case NCGB_COMP_BRAGG: {
            // PowderBragg::sampleScatterIsotropic, NCPowderBragg.cc:202-216
            if constexpr ( !Lean ) {
              int64_t idx;
              braggXS( c.bragg, e, idx );
              if ( c.bragg.n && e >= c.bragg.threshold && finited(e) )
                mu = braggMu( c.bragg, rng, e, idx );
            }
            break;
          }
          case NCGB_COMP_ELINC:
          {
            // a copy in and out: the neutron's stream stays in registers
            // (measured: the pick pass 0.73 vs 0.78 ms on polyethylene)
            ncgb_rng r2 = rng;
            mu = elincMu<Fast>( c.elinc, r2, e, st );
            rng = r2;
          }
            break;
          case NCGB_COMP_SAB:
            // sampled by k_sab's refilled lanes; with split lists, those
            // above the energy grid (the extender's path) go on the rare
            // list.  The sampler's grid search (egridUpper, an upper bound
            // over the sorted grid) returns ne exactly when e >= egrid[ne-1]:
            // for non-negative doubles the bit patterns order as the values,
            // a negative e gives 0 both ways and a NaN ne both ways.
            queue = true;
            rare = src.splitLists() && !( bits( e ) < ldgbits( c.sab.egrid + c.sab.ne - 1 ) );
            qcomp = p.comp;
            break;
          case NCGB_COMP_FREEGAS:
            queue = true;
            rare = src.splitLists();
            qcomp = p.comp;
            break;
          default:
            break;
        }
        if ( !queue )
          writeScatter<Dir>( b, o, e, st, ef, mu, rng );
      }
      // warp-aggregated appends to the two lists of the SAB queue
      const unsigned active = __activemask();
      const unsigned want = __ballot_sync( active, queue );
      if ( want ) {
        const unsigned wrare = src.splitLists() ? __ballot_sync( active, queue && rare ) : 0u;
        const unsigned wmain = want & ~wrare;
        const int lane = threadIdx.x & 31;
        const unsigned mine = ( 1u << lane ) - 1u;
        unsigned base = 0, rbase = 0;
        if ( wmain && lane == __ffs( wmain ) - 1 )
          base = atomicAdd( &b.work->qcount, (unsigned)__popc( wmain ) );
        if ( wrare && lane == __ffs( wrare ) - 1 )
          rbase = atomicAdd( &b.work->rcount, (unsigned)__popc( wrare ) );
        if ( wmain )
          base = __shfl_sync( active, base, __ffs( wmain ) - 1 );
        if ( wrare )
          rbase = __shfl_sync( active, rbase, __ffs( wrare ) - 1 );
        if ( queue ) {
          const uint64_t pos = rare ? b.n_out - 1 - ( rbase + __popc( wrare & mine ) )
                                    : base + __popc( wmain & mine );
          ncgb::QEntry q;
          q.ekin = e;
          q.idx = (uint32_t)o;
          q.mat = (uint16_t)k;
          q.comp = (uint8_t)qcomp;
          q.ndraws = (uint8_t)ncgb_rng_ndoubles( &rng );
          b.queue[pos] = q;
        }
      }
    }
  }

  template<class Src, bool Fast, bool Dir, bool Lean = false>
  __global__ void __launch_bounds__(512, 4)
  k_pick( const __grid_constant__ Src src, const ncgb::Batch b )
  {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for ( uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; o < b.n_out; o += stride )
      pickOne<Src, Fast, Dir, Lean>( src, b, o );
  }

  // The pick pass over tiles of kTile consecutive neutrons, each tile visited
  // in order of energy buckets (four per octave, counting-sorted in shared
  // memory), so that a warp's lanes evaluate neighbouring energies: the same
  // energy-grid and Bragg-plane entries, the same branches.  Every neutron
  // keeps its own index, random stream and output slot; only the order in
  // which the block visits them changes (and with it the queue's order).
  constexpr int kTileReps = 8;            // tile = 8 x blockDim neutrons
  constexpr int kPickBuckets = 128;       // 4 per octave from 2^-26 eV
  __device__ __forceinline__ int energyBucket( double e )
  {
    const long long k = ( bits( e ) >> 50 ) - ( ( 1023LL - 26 ) << 2 );
    return k < 0 ? 0 : ( k >= kPickBuckets ? kPickBuckets - 1 : (int)k );
  }

  template<class Src, bool Fast, bool Dir>
  __global__ void __launch_bounds__(512, 4)
  k_pick_tiles( const __grid_constant__ Src src, const ncgb::Batch b, int reps )
  {
    __shared__ unsigned s_hist[kPickBuckets];
    __shared__ uint16_t s_perm[512 * kTileReps];
    const int nthr = blockDim.x, tid = threadIdx.x;
    const uint64_t tile = (uint64_t)nthr * reps;   // reps <= kTileReps
    // block-uniform loop (every thread reaches the barriers)
    for ( uint64_t t0 = (uint64_t)blockIdx.x * tile; t0 < b.n_out; t0 += (uint64_t)gridDim.x * tile ) {
      const int nt = (int)( ( b.n_out - t0 ) < tile ? ( b.n_out - t0 ) : tile );
      for ( int i = tid; i < kPickBuckets; i += nthr )
        s_hist[i] = 0;
      __syncthreads();
      uint32_t slot[kTileReps];   // bucket << 16 | rank within the bucket
#pragma unroll
      for ( int r = 0; r < kTileReps; ++r ) {
        const int j = tid + r * nthr;
        slot[r] = 0;
        if ( j < nt ) {
          const uint64_t o = t0 + j;
          const int kb = energyBucket( loadE( b, ( b.n_out == b.n_ekin ) ? o : o % b.n_ekin ) );
          slot[r] = ( (uint32_t)kb << 16 ) | atomicAdd( &s_hist[kb], 1u );
        }
      }
      __syncthreads();
      // exclusive prefix sum of the bucket counts (one warp, 4 buckets a lane)
      if ( tid < 32 ) {
        unsigned c[4], run = 0;
#pragma unroll
        for ( int q = 0; q < 4; ++q ) { c[q] = s_hist[4 * tid + q]; run += c[q]; }
        unsigned incl = run;
#pragma unroll
        for ( int d = 1; d < 32; d <<= 1 ) {
          const unsigned v = __shfl_up_sync( 0xffffffffu, incl, d );
          if ( tid >= d ) incl += v;
        }
        unsigned base = incl - run;
#pragma unroll
        for ( int q = 0; q < 4; ++q ) { s_hist[4 * tid + q] = base; base += c[q]; }
      }
      __syncthreads();
#pragma unroll
      for ( int r = 0; r < kTileReps; ++r ) {
        const int j = tid + r * nthr;
        if ( j < nt )
          s_perm[s_hist[slot[r] >> 16] + ( slot[r] & 0xffffu )] = (uint16_t)j;
      }
      __syncthreads();
      for ( int r = 0; r < kTileReps; ++r ) {
        const int j = tid + r * nthr;
        if ( j < nt )
          pickOne<Src, Fast, Dir>( src, b, t0 + s_perm[j] );
      }
      __syncthreads();   // the shared arrays are reused by the next tile
    }
  }

  // ---- phase 2: persistent S(alpha,beta) sampling ---------------------------
  // The pass over one list of the queue (RareList: the rare one), shared by
  // k_sab and its phase-profiling copy (Ph: NoPhases, whose marks compile to
  // nothing, or PhaseClock).  Full: with the free-gas sampler and the
  // extender above the energy grid; a lean pass (the main list of split
  // lists) has neither, nor their out-of-line calls, and inlines the first
  // beta bin's sampler, so that its loop makes no call (measured: k_sab
  // 1.30 -> 1.21 ms on polyethylene).  A neutron's results do not depend on
  // the list it is on.
  template<class Src, bool Fast, bool Learned, bool Dir, bool RareList, bool Full, class Ph>
  __device__ __forceinline__ void sabPass( const Src& src, const ncgb::Batch& b, Ph& ph )
  {
    constexpr bool kClocked = !std::is_same<Ph, NoPhases>::value;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned qcount = RareList ? *(volatile unsigned*)&b.work->rcount : *(volatile unsigned*)&b.work->qcount;
    unsigned* qnext = RareList ? &b.work->rnext : &b.work->qnext;
    bool has = false, done = false;
    ncgb::QEntry q;
    q.ekin = 0.0; q.idx = 0; q.mat = 0; q.comp = 0; q.ndraws = 0;
    SABLane L;
    ncgb_rng rng;
    src.rngIdle( rng, b.callseq );
    // Bounded: every claimed neutron finishes within 100 x 100 Alg.1 attempts
    // (each with at most 1000 learned-proposal draws), and claims stop at qcount.
    for (;;) {
      const unsigned need = __ballot_sync( FULL, !has && !done );
      if ( need ) {
        const int leader = __ffs( need ) - 1;
        unsigned base = 0;
        if ( lane == leader )
          base = atomicAdd( qnext, (unsigned)__popc( need ) );
        base = __shfl_sync( FULL, base, leader );
        if ( !has && !done ) {
          const unsigned slot = base + __popc( need & ( ( 1u << lane ) - 1u ) );
          if ( slot < qcount ) {
            q = b.queue[RareList ? b.n_out - 1 - slot : slot];
            src.rngFor( rng, q.mat, q.idx, b.callseq );
            for ( int k = 0; k < q.ndraws; ++k )
              rand01( rng );
            const ncgb_material_view& m = src.mat( q.mat );
            const ncgb_comp_view& c = m.comp[q.comp];
            if ( c.type == NCGB_COMP_FREEGAS ) {
              // FreeGas component: sampled to completion here (never on the
              // list of a lean pass)
              double ef = q.ekin, mu = 1.0;
              int st = NCGB_ST_CALCERROR;
              if constexpr ( Full )
                st = freeGasScatter( c.fg, m.fg_erfc_table, rng, q.ekin, ef, mu );
              writeScatter<Dir>( b, q.idx, q.ekin, st, ef, mu, rng );
            } else {
              const int st = sabBegin<Full>( c.sab, m.fg_erfc_table, q.ekin, rng, L );
              if ( st != NCGB_ST_OK )
                writeScatter<Dir>( b, q.idx, q.ekin, st, q.ekin, 1.0, rng );
              else
                has = true;
            }
          } else {
            done = true;
          }
        }
      }
      if constexpr ( kClocked ) {
        if ( done && !has )
          ph.template end<PH_IDLE>();
        else
          ph.template end<PH_CLAIM>();
      }
      if ( __all_sync( FULL, done && !has ) )
        break;
      if ( has ) {
        double ef = 0.0, mu = 0.0;
        const int st = sabStep<Fast, Learned, Full>( src.mat( q.mat ).comp[q.comp].sab, L, rng, ef, mu, ph );
        if ( st >= 0 ) {
          writeScatter<Dir>( b, q.idx, L.ekin, st, ef, mu, rng );
          has = false;
          if constexpr ( kClocked )
            ph.template end<PH_CONVERT>();
        } else if constexpr ( kClocked ) {
          ph.template end<PH_ACCEPT>();
        }
      }
    }
  }

  // Full occupancy (8 blocks of 256 per SM, 32 registers): the sampler waits
  // on table gathers, and more resident warps hide that latency better than
  // registers avoid spills (measured: 4 blocks 1.64 ms, 6 blocks 1.48 ms,
  // 8 blocks 1.39 ms per 2^24-neutron polyethylene batch, mixed mode).
  // The rare list, out of line: its samplers' calls stay out of the main
  // list's loop.
  template<class Src, bool Fast, bool Learned, bool Dir>
  __device__ __noinline__ void sabRareList( const Src& src, const ncgb::Batch& b )
  {
    NoPhases ph;
    sabPass<Src, Fast, Learned, Dir, true, true>( src, b, ph );
  }

  // Each warp takes the rare list once the main list has no neutron left for
  // it (both lists are complete before this pass starts).  Measured against
  // taking it first: polyethylene k_sab 1.188 vs 1.196 ms, the crystal batch
  // the same either way.
  template<class Src, bool Fast, bool Learned, bool Dir>
  __device__ __forceinline__ void sabRareTail( const Src& src, const ncgb::Batch& b )
  {
    if ( *(volatile unsigned*)&b.work->rcount )   // the same for every lane of the warp
      sabRareList<Src, Fast, Learned, Dir>( src, b );
  }

  // Split: a lean pass over the main list, then the rare list.  Otherwise one
  // list and the full sampler (ragged batches whose autotuner found that
  // faster: the mixed batch's pass measured 1.69 ms split against 1.51 ms
  // with one list, the crystal batch's 0.66 against 0.71 ms).
  template<class Src, bool Fast, bool Learned, bool Dir, bool Split>
  __global__ void __launch_bounds__(256, 8)
  k_sab( const __grid_constant__ Src src, const __grid_constant__ ncgb::Batch b )
  {
    NoPhases ph;
    if constexpr ( Split ) {
      sabPass<Src, Fast, Learned, Dir, false, false>( src, b, ph );
      sabRareTail<Src, Fast, Learned, Dir>( src, b );
    } else {
      sabPass<Src, Fast, Learned, Dir, false, true>( src, b, ph );
    }
  }

  // The same pass with per-lane phase clocks (a measurement instrument,
  // launched by ncgb_sab_phase_profile only): the lanes' SM-clock cycles per
  // phase and their Alg.1 attempts, summed into b.phase_cycles[PH_N + 1].
  template<bool Fast, bool Learned>
  __global__ void __launch_bounds__(256, 8)
  k_sab_phases( const __grid_constant__ SingleSrc src, const __grid_constant__ ncgb::Batch b )
  {
    PhaseClock ph;
    ph.start();
    sabPass<SingleSrc, Fast, Learned, false, false, false>( src, b, ph );
    sabRareTail<SingleSrc, Fast, Learned, false>( src, b );   // not clocked
    const int lane = threadIdx.x & 31;
    for ( int i = 0; i <= PH_N; ++i ) {
      const unsigned v = __reduce_add_sync( 0xffffffffu, i < PH_N ? ph.acc[i] : ph.attempts );
      if ( lane == 0 )
        atomicAdd( b.phase_cycles + i, (unsigned long long)v );
    }
  }

  // ---- (alpha, beta) of one S(alpha,beta) component ----------------------------
  // SABSampler::sampleAlphaBeta (NCSABSampler.cc:158-227) per neutron, for the
  // proposal's training set and its tests: out_a = alpha, out_b = beta.
  template<bool Fast, bool Learned>
  __global__ void __launch_bounds__(256)
  k_sab_ab( const __grid_constant__ ncgb_material_view m, int comp, const ncgb::Batch b )
  {
    const ncgb_comp_view& c = m.comp[comp];
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for ( uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n_ekin; i += stride ) {
      const double e = loadE( b, i );
      ncgb_rng rng;
      ncgb_rng_init( &rng, b.seed, (uint32_t)( b.index_offset + i ), b.callseq, b.stream );
      double alpha = 0.0, beta = 0.0;
      SABLane L;
      int st = sabBegin( c.sab, m.fg_erfc_table, e, rng, L );
      if ( st == NCGB_ST_OK ) {
        do {
          st = sabStepAB<Fast, Learned>( c.sab, L, rng, alpha, beta );
        } while ( st < 0 );
      }
      static_cast<double*>( b.out_a )[i] = alpha;
      static_cast<double*>( b.out_b )[i] = beta;
      if ( b.status )
        b.status[i] = st;
      if ( st != NCGB_ST_OK )
        atomicAdd( &b.work->nfail, 1ull );
    }
  }

  // ---- absorption cross-sections (AbsOOV) ---------------------------------------
  __global__ void __launch_bounds__(256)
  k_absxs( double abs_c, const ncgb::Batch b, uint64_t repeat )
  {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for ( uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n_ekin; i += stride ) {
      const double xs = absXS( abs_c, loadE( b, i ) );
      for ( uint64_t r = 0; r < repeat; ++r )
        store( b.out_xs, b.out_f32, r * b.n_ekin + i, xs );
    }
  }

  // ---- cross-sections only ------------------------------------------------------
  // results[r*n_ekin+i] = xs(ekin[i]) for r < repeat (ncrystal.cc:1107-1141
  // writes the same value for every repeat).
  template<bool Fast>
  __global__ void __launch_bounds__(256)
  k_xs( const __grid_constant__ ncgb_material_view m, const ncgb::Batch b, uint64_t repeat )
  {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for ( uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n_ekin; i += stride ) {
      const double e = loadE( b, i );
      double xs = 0.0;
      if ( contains( m.dom_elow, m.dom_ehigh, e ) ) {
        ncgb_rng dummy;
        ncgb_rng_init( &dummy, 0, 0, 0, 0 );
        xs = xsAndPick<false, Fast>( m, e, dummy ).xs;
      }
      for ( uint64_t r = 0; r < repeat; ++r )
        store( b.out_xs, b.out_f32, r * b.n_ekin + i, xs );
    }
  }

  int numSMs()
  {
    static int nsm = 0;
    if ( !nsm ) {
      int dev = 0;
      cudaGetDevice( &dev );
      cudaDeviceGetAttribute( &nsm, cudaDevAttrMultiProcessorCount, dev );
      if ( nsm <= 0 ) nsm = 1;
    }
    return nsm;
  }

  template<class Src>
  int sabBlocksPerSM()
  {
    static int bps = 0;
    if ( !bps ) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor( &bps, k_sab<Src, false, false, std::is_same<Src, MappedSrc>::value, true>,
                                                     256, 0 );
      if ( bps <= 0 ) bps = 1;
    }
    return bps;
  }

  int gridFor( uint64_t n, int block )
  {
    uint64_t want = ( n + block - 1 ) / block;
    uint64_t cap = (uint64_t)numSMs() * ( 8192 / block ); // grid-stride beyond this
    if ( want > cap ) want = cap;
    if ( want < 1 ) want = 1;
    return (int)want;
  }

  // Optional CUDA-event timing of the two phases, on the launching stream
  // (enabled by ncgb_phase_timing; used by the benchmark's roofline).
  struct PhaseEvents { cudaEvent_t a, b, c; };
  bool g_timing = false;
  std::vector<PhaseEvents> g_events;
  std::mutex g_evmtx;

  // The energy-ordered tiles pay where the pick pass searches the Bragg
  // planes (measured: Al2O3 pick pass 0.96 -> 0.87 ms, crystal batch 0.59 ->
  // 0.54 ms, mixed batch 0.81 -> 0.71 ms, and their S(alpha,beta) passes
  // faster too); for polyethylene, with no Bragg component, the reordering
  // costs more than it saves (0.78 -> 0.85 ms), and with outputs in host
  // memory its scattered writes cross the link as partial lines.
  template<class Src, bool Dir>
  void launchPick( const Src& src, const ncgb::Batch& b, int pb, cudaStream_t s )
  {
    if ( b.reorder ) {
      // tiles of up to kTileReps x pb neutrons, shorter for small batches so
      // that every SM still gets its blocks (4 of pb threads each)
      const uint64_t perSlot = b.n_out / ( (uint64_t)numSMs() * 4 * (uint64_t)pb );
      const int reps = perSlot >= (uint64_t)kTileReps ? kTileReps : ( perSlot < 1 ? 1 : (int)perSlot );
      const uint64_t tiles = ( b.n_out + (uint64_t)pb * reps - 1 ) / ( (uint64_t)pb * reps );
      const int g = (int)( tiles < (uint64_t)gridFor( b.n_out, pb ) ? tiles : (uint64_t)gridFor( b.n_out, pb ) );
      if ( b.fast )
        k_pick_tiles<Src, true, Dir><<<g, pb, 0, s>>>( src, b, reps );
      else
        k_pick_tiles<Src, false, Dir><<<g, pb, 0, s>>>( src, b, reps );
      return;
    }
    if constexpr ( !std::is_same<Src, MultiSrc>::value ) {
      if ( src.lean ) {
        if ( b.fast )
          k_pick<Src, true, Dir, true><<<gridFor( b.n_out, pb ), pb, 0, s>>>( src, b );
        else
          k_pick<Src, false, Dir, true><<<gridFor( b.n_out, pb ), pb, 0, s>>>( src, b );
        return;
      }
    }
    if ( b.fast )
      k_pick<Src, true, Dir><<<gridFor( b.n_out, pb ), pb, 0, s>>>( src, b );
    else
      k_pick<Src, false, Dir><<<gridFor( b.n_out, pb ), pb, 0, s>>>( src, b );
  }

  template<class Src, bool Dir, bool Split>
  void launchSabT( const Src& src, const ncgb::Batch& b, int grid, cudaStream_t s )
  {
    if ( b.fast ) {
      if ( b.learned )
        k_sab<Src, true, true, Dir, Split><<<grid, 256, 0, s>>>( src, b );
      else
        k_sab<Src, true, false, Dir, Split><<<grid, 256, 0, s>>>( src, b );
    } else {
      if ( b.learned )
        k_sab<Src, false, true, Dir, Split><<<grid, 256, 0, s>>>( src, b );
      else
        k_sab<Src, false, false, Dir, Split><<<grid, 256, 0, s>>>( src, b );
    }
  }

  template<class Src, bool Dir>
  void launchSab( const Src& src, const ncgb::Batch& b, int grid, cudaStream_t s )
  {
    if constexpr ( std::is_same<Src, SingleSrc>::value && !Dir ) {
      if ( b.phase_cycles ) {
        if ( b.fast ) {
          if ( b.learned )
            k_sab_phases<true, true><<<grid, 256, 0, s>>>( src, b );
          else
            k_sab_phases<true, false><<<grid, 256, 0, s>>>( src, b );
        } else {
          if ( b.learned )
            k_sab_phases<false, true><<<grid, 256, 0, s>>>( src, b );
          else
            k_sab_phases<false, false><<<grid, 256, 0, s>>>( src, b );
        }
        return;
      }
    }
    if constexpr ( std::is_same<Src, MultiSrc>::value ) {
      if ( !src.split ) {
        launchSabT<Src, Dir, false>( src, b, grid, s );
        return;
      }
    }
    launchSabT<Src, Dir, true>( src, b, grid, s );
  }

  template<class Src>
  cudaError_t launchBoth( const Src& src, const ncgb::Batch& b, const ncgb::LaunchCfg& cfg, cudaStream_t s,
                          cudaEvent_t pickDone = nullptr )
  {
    if ( b.n_out == 0 )
      return cudaSuccess;
    cudaError_t e = cudaMemsetAsync( &b.work->qcount, 0, 4 * sizeof(unsigned int), s );
    if ( e != cudaSuccess )
      return e;
    PhaseEvents ev{ nullptr, nullptr, nullptr };
    const bool timing = g_timing && !b.untimed;
    if ( timing ) {
      cudaEventCreate( &ev.a );
      cudaEventCreate( &ev.b );
      cudaEventCreate( &ev.c );
      cudaEventRecord( ev.a, s );
    }
    const int pb = ( cfg.pick_block == 128 || cfg.pick_block == 512 ) ? cfg.pick_block : 256;
    constexpr bool kMulti = std::is_same<Src, MultiSrc>::value;
    constexpr bool kMapped = std::is_same<Src, MappedSrc>::value;
    if ( b.dir_out ) {
      if constexpr ( !kMulti )
        launchPick<Src, true>( src, b, pb, s );
      else
        return cudaErrorInvalidValue;   // directions: single-material calls only
    } else {
      if constexpr ( !kMapped )
        launchPick<Src, false>( src, b, pb, s );
      else
        return cudaErrorInvalidValue;   // stream index arrays: with directions only
    }
    e = cudaGetLastError();
    if ( e != cudaSuccess )
      return e;
    if ( pickDone ) {
      e = cudaEventRecord( pickDone, s );
      if ( e != cudaSuccess )
        return e;
    }
    if ( timing )
      cudaEventRecord( ev.b, s );
    const int maxb = sabBlocksPerSM<Src>();
    const int mult = ( cfg.sab_blocks_per_sm > 0 && cfg.sab_blocks_per_sm < maxb ) ? cfg.sab_blocks_per_sm : maxb;
    const int grid = numSMs() * mult;
    if ( b.dir_out ) {
      if constexpr ( !kMulti )
        launchSab<Src, true>( src, b, grid, s );
    } else {
      if constexpr ( !kMapped )
        launchSab<Src, false>( src, b, grid, s );
    }
    e = cudaGetLastError();
    if ( timing ) {
      cudaEventRecord( ev.c, s );
      std::lock_guard<std::mutex> lock( g_evmtx );
      g_events.push_back( ev );
    }
    return e;
  }
}

namespace ncgb {

  // A material whose components are S(alpha,beta) and incoherent elastic
  // only: its pick pass runs without the other types' code (measured on
  // polyethylene: 0.780 -> 0.724 ms).
  static int leanMaterial( const ncgb_material_view& m )
  {
    for ( int i = 0; i < m.ncomp && i < NCGB_MAX_COMP; ++i )
      if ( m.comp[i].type != NCGB_COMP_SAB && m.comp[i].type != NCGB_COMP_ELINC )
        return 0;
    return 1;
  }

  cudaError_t launchScatter( const ncgb_material_view& m, const Batch& b, cudaStream_t s, cudaEvent_t pickDone )
  {
    if ( b.rng_index ) {
      MappedSrc src;
      src.m = m;
      src.seed = b.seed;
      src.stream = b.stream;
      src.pad = 0;
      src.index = b.rng_index;
      src.lean = leanMaterial( m );
      src.pad2 = 0;
      return launchBoth( src, b, LaunchCfg(), s );
    }
    SingleSrc src;
    src.m = m;
    src.seed = b.seed;
    src.stream = b.stream;
    src.index_offset = b.index_offset;
    src.lean = leanMaterial( m );
    src.pad = 0;
    return launchBoth( src, b, LaunchCfg(), s, pickDone );
  }

  cudaError_t launchScatterMulti( const MatSlot* d_slots, const int64_t* d_offsets, int nmat,
                                  const Batch& b, const LaunchCfg& cfg, cudaStream_t s, cudaEvent_t pickDone )
  {
    MultiSrc src;
    src.slots = d_slots;
    src.offsets = d_offsets;
    src.nmat = nmat;
    src.split = cfg.split_lists;
    src.base = (int64_t)b.index_offset;
    return launchBoth( src, b, cfg, s, pickDone );
  }

  int maxSabBlocksPerSM() { return sabBlocksPerSM<MultiSrc>(); }

  cudaError_t launchXS( const ncgb_material_view& m, const Batch& b, uint64_t repeat, cudaStream_t s )
  {
    if ( b.n_ekin == 0 || repeat == 0 )
      return cudaSuccess;
    if ( b.fast )
      k_xs<true><<<gridFor( b.n_ekin, 256 ), 256, 0, s>>>( m, b, repeat );
    else
      k_xs<false><<<gridFor( b.n_ekin, 256 ), 256, 0, s>>>( m, b, repeat );
    return cudaGetLastError();
  }

  cudaError_t launchAbsXS( double abs_c, const Batch& b, uint64_t repeat, cudaStream_t s )
  {
    if ( b.n_ekin == 0 || repeat == 0 )
      return cudaSuccess;
    k_absxs<<<gridFor( b.n_ekin, 256 ), 256, 0, s>>>( abs_c, b, repeat );
    return cudaGetLastError();
  }

  cudaError_t launchSabAB( const ncgb_material_view& m, int comp, const Batch& b, cudaStream_t s )
  {
    if ( b.n_ekin == 0 )
      return cudaSuccess;
    const int grid = gridFor( b.n_ekin, 256 );
    if ( b.fast ) {
      if ( b.learned )
        k_sab_ab<true, true><<<grid, 256, 0, s>>>( m, comp, b );
      else
        k_sab_ab<true, false><<<grid, 256, 0, s>>>( m, comp, b );
    } else {
      if ( b.learned )
        k_sab_ab<false, true><<<grid, 256, 0, s>>>( m, comp, b );
      else
        k_sab_ab<false, false><<<grid, 256, 0, s>>>( m, comp, b );
    }
    return cudaGetLastError();
  }

  int scatterLaunchesPerBatch() { return 2; }

  bool phaseTiming() { return g_timing; }

  void setPhaseTiming( bool on )
  {
    std::lock_guard<std::mutex> lock( g_evmtx );
    g_timing = on;
  }

  // Sums the recorded phase times (waits for them) and forgets them.
  int takePhaseTimes( double* ms_pick, double* ms_sab, unsigned long* nbatches )
  {
    std::lock_guard<std::mutex> lock( g_evmtx );
    double tp = 0.0, ts = 0.0;
    for ( auto& ev : g_events ) {
      float a = 0.f, c = 0.f;
      if ( cudaEventSynchronize( ev.c ) != cudaSuccess )
        return 1;
      cudaEventElapsedTime( &a, ev.a, ev.b );
      cudaEventElapsedTime( &c, ev.b, ev.c );
      tp += a;
      ts += c;
      cudaEventDestroy( ev.a );
      cudaEventDestroy( ev.b );
      cudaEventDestroy( ev.c );
    }
    *ms_pick = tp;
    *ms_sab = ts;
    *nbatches = static_cast<unsigned long>( g_events.size() );
    g_events.clear();
    return 0;
  }
}
