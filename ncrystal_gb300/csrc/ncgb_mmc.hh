// MiniMC on the device: the reference's standard simulation engine
// (NCMMC_SimEngine.cc:170-440) with its geometries (NCMMC_Sphere.hh,
// NCMMC_Box.hh, NCMMC_Slab.hh, NCMMC_Cyl.hh), sources (NCMMC_Source.cc:433-800)
// and standard histogram tallies (NCMMC_StdTallies.cc), driving the batched
// scattering kernels of this library for every collision.
//
// The neutron population stays in device memory for the whole run.  One
// engine step is
//   k_mmc_emit       new source neutrons (propagated to the volume; misses
//                    tallied) appended to population A,
//   k_mmc_transport  over A: finish the previous step's scatter, distance to
//                    exit, absorption and scattering cross-sections, forced
//                    collision with roulette; the transmitted part is tallied
//                    and the part that scatters is appended to population B,
//   k_pick + k_sab   the library's scatter with directions over B,
// and A and B swap.  Random streams are keyed by (source index, step), so a
// neutron's history does not depend on where it sits in the arrays.
#ifndef NCGB_MMC_HH
#define NCGB_MMC_HH

#include <cstdint>
#include <string>
#include <cuda_runtime.h>
#include "ncgb_tables.h"

namespace ncgb {
  namespace mmc {

    enum GeomKind : int32_t { GEOM_SPHERE = 0, GEOM_BOX = 1, GEOM_SLAB = 2, GEOM_CYL = 3 };

    // One convex volume around the origin (NCMMC_Geom.cc:92-130).  Lengths
    // in metres; dy = 0 for a cylinder means infinitely long.
    struct Geom {
      int32_t kind;
      int32_t unbounded;   // distances to exit may be infinite (slab, infinite cylinder)
      double r, dx, dy, dz;
    };

    enum SrcKind : int32_t { SRC_CONSTANT = 0, SRC_CIRCULAR = 1, SRC_ISOTROPIC = 2 };
    enum EKind : int32_t { E_FIXED = 0, E_UNIFORM = 1, E_LOGNORMAL = 2, E_MAXWELL = 3 };

    // Source (NCMMC_Source.cc:433-800); energies per EParsed
    // (NCMMC_ParseCfg.hh:333-431).  Uniform and log-normal ranges are in eV or
    // in Aa (e_is_wl), then converted to energy.
    struct Source {
      int32_t kind, ekind, e_is_wl, might_be_outside;
      double x, y, z;          // position (circular: beam centre)
      double ux, uy, uz;       // direction (constant, circular)
      double r;                // circular: beam radius; isotropic: start at -r along the direction
      double ea, eb;           // fixed: E, -; uniform: low, high; lognormal: mu_n, sigma_n; maxwell: kT/2, -
      double ax, ay, az;       // circular: basis vectors orthogonal to the direction, times r
      double bx, by, bz;
    };

    // Engine options (NCMMC_EngineOpts.cc:56-67, NCMMC_SimEngine.cc:133-149).
    struct Engine {
      double macro;            // 100 x number density [1/(barn m)] (NCMMC_Utils.hh:103-105)
      double abs_c;            // absorption xs = abs_c/sqrt(E) (AbsOOV), used when has_abs
      double psurv, wthr, boost;   // roulette: survival probability, weight threshold, 1/psurv
      int32_t nscatthr;        // roulette applies from this many scatterings on
      int32_t nscatlimit;      // <0: none
      int32_t has_abs, has_scat;
      int32_t fast;            // cross-sections in the mixed-precision mode
      int32_t ignore_miss;
      uint64_t seed;           // of the engine's own random streams
    };

    // Tallies (NCMMC_StdTallies.cc).  Histogram k has 6 groups (total and
    // the five breakdowns NOSCAT, SINGLESCAT_ELAS, SINGLESCAT_INELAS,
    // MULTISCAT_PUREELAS, MULTISCAT_OTHER), each with running statistics
    // [sum w, sum w x, sum w x^2, min key, max key] (keys: doubles mapped to
    // order-preserving int64) and nbins+2 bins (underflow first, overflow
    // last) of [content, error^2].  The buffer holds all statistics first
    // (nstat doubles), then all bins, so that kernels can keep the statistics
    // in shared memory even when the bins do not fit there.
    enum TallyKind : int32_t { T_THETA = 0, T_MU, T_NSCAT, T_NSCAT_UW, T_W, T_E, T_L, T_DE, T_Q, T_N };
    constexpr int kGroups = 6;
    constexpr int kStats = 5;

    struct TallyHist {
      int32_t enabled, nbins;
      double xmin, xmax, inv_delta;
      int64_t off;             // first double of this histogram's bins in the tally buffer
      int64_t soff;            // first double of its statistics (< nstat)
    };

    struct Tally {
      TallyHist h[T_N];
      int32_t breakdown;
      int32_t fixed_dir;       // use (d0x, d0y, d0z) as the incoming direction
      int32_t fixed_e;         // use e0 as the incoming energy
      int32_t pad;
      double d0x, d0y, d0z, e0;
      int64_t nstat;           // doubles of statistics at the start of the buffer
      int64_t nbuf;            // doubles in the tally buffer
      double* buf;             // device
      // per launch: fixed-point scales (powers of two) of the block-local
      // bins in shared memory, for contents and errors^2
      double cscale, escale;
      // per tally: the statistics accumulate sums of w (x - shift) and
      // w (x - shift)^2, shift = the value of an unscattered source neutron
      // where that is fixed (delta-like groups keep their rms at ~0)
      double shift[T_N];
    };

    // Population of neutrons (structure of arrays; directions [n][3]).
    struct Pop {
      double* pos;             // [n][3]
      double* dir;             // [n][3]
      double* e;
      double* w;
      double* xs;              // cached macroscopic scattering xs (<0: evaluate)
      int32_t* nscat;
      int32_t* ninel;
      uint32_t* id;            // source index: the key of the neutron's random streams
      double* e0;              // [n] initial energy (per-neutron tally reference)
      double* d0;              // [n][3] initial direction (per-neutron tally reference)
      double* e_new;           // scatter results of the previous step
      double* dir_new;         // [n][3]
      int32_t* st;             // scatter status; kNoScatter: nothing pending
    };
    constexpr int32_t kNoScatter = -1;

    // Device counters of a run.
    struct Counters {
      unsigned long long n_b;          // neutrons appended to population B this step
      unsigned long long n_a;          // neutrons appended to population A by the source
      unsigned long long tallied;      // tallied neutrons (count)
      unsigned long long miss;         // source neutrons that missed the volume
      unsigned long long nfail;        // scatters with a non-OK status
      unsigned long long pad;
      double tallied_w, miss_w;
    };

    // What the host engine reads from a scatter handle (ncgb_capi.cc).
    struct HandleInfo {
      ncgb_material_view view;
      int device = 0, mode = 0, sampler = 0;
      uint64_t seed = 0;
      uint32_t streamidx = 0;
      double numdens = -1.0;           // atoms per Aa^3
      double temperature = -1.0;       // K, -1: none
      double bragg_threshold = -1.0;   // Aa, -1: none
      double abs_c = -1.0;             // AbsOOV constant, <0: not in the bundle
      std::string cfg;
    };

    // Launchers (ncgb_mmc.cu).  Streams: the engine's draws of neutron 'id'
    // in step 'step' come from Philox (seed, id, step, kStreamEngine); the
    // source's from (seed, id, 0, kStreamSource).
    constexpr uint32_t kStreamEngine = 0x4d4d4301u;
    constexpr uint32_t kStreamSource = 0x4d4d4302u;

    // Source neutrons first_id .. first_id+count-1, appended to a from index
    // base on (counted in c->n_a).
    cudaError_t launchEmit( const Source& src, const Geom& g, const Engine& eng, const Tally& t, Pop a,
                            uint64_t base, uint64_t first_id, uint64_t count, Counters* c, int numSMs,
                            cudaStream_t s );
    // One step over a[0, n_a): survivors appended to b (counted in c->n_b).
    cudaError_t launchTransport( const ncgb_material_view& m, const Geom& g, const Engine& eng, const Tally& t,
                                 Pop a, uint64_t n_a, Pop b, uint32_t step, Counters* c, int numSMs,
                                 cudaStream_t s );
  }
}

#endif
