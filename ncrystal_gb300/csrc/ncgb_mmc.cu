// Device kernels of the MiniMC engine: source emission and the transport
// step (forced collision, roulette, tallies).  The collisions themselves are
// the library's scatter kernels (ncgb_kernels.cu), launched by the host
// engine (ncgb_mmc.cc) between two transport steps.
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdlib>
#include <algorithm>
#include <cmath>

#include "ncgb_device.cuh"
#include "ncgb_mmc.hh"

namespace {

  using namespace ncgb_dev;
  using namespace ncgb::mmc;

  constexpr double kPi = 3.14159265358979323846;
  constexpr double kToDeg = 57.2957795130823208767981548141051703324054725;   // 180/pi (NCDefs.hh:124)
  constexpr double kWl2Ekin = 0.081804209605330899;                            // E[eV] = kWl2Ekin / wl[Aa]^2
  constexpr double kEkin2Ksq = 4.0 * kPi * kPi / kWl2Ekin;                     // ekin2ksq(1.0) (NCDefs.hh:872)
  constexpr double kDblMax = 1.7976931348623157e308;

  // ---- geometry ----------------------------------------------------------------

  __device__ __forceinline__ double slabExit( double x, double ux, double d )
  {
    // NCMMC_Utils.cc:516-537
    if ( ux > 0.0 )
      return ( d - x ) / ux;
    if ( ux < 0.0 )
      return -( d + x ) / ux;
    return infd();
  }

  // Distance to the volume's surface from a point inside it
  // (distToVolumeExit of NCMMC_Sphere.hh:170-216, NCMMC_Box.hh:213-226,
  // NCMMC_Slab.hh, NCMMC_Cyl.hh); may be infinite for unbounded volumes.
  __device__ double distExit( const Geom& g, const double* p, const double* u )
  {
    switch ( g.kind ) {
      case GEOM_SPHERE: {
        const double c = g.r * g.r - ( p[0] * p[0] + p[1] * p[1] + p[2] * p[2] );
        const double pd = p[0] * u[0] + p[1] * u[1] + p[2] * u[2];
        return maxd( 0.0, sqrt( maxd( 0.0, c + pd * pd ) ) - pd );
      }
      case GEOM_BOX:
        return fmin( slabExit( p[0], u[0], g.dx ), fmin( slabExit( p[1], u[1], g.dy ), slabExit( p[2], u[2], g.dz ) ) );
      case GEOM_SLAB:
        return slabExit( p[2], u[2], g.dz );
      default: {
        // cylinder around y: radial exit (larger root), then the end caps
        const double a = u[0] * u[0] + u[2] * u[2];
        double t = infd();
        if ( a > 0.0 ) {
          const double b = p[0] * u[0] + p[2] * u[2];
          const double c = p[0] * p[0] + p[2] * p[2] - g.r * g.r;
          t = maxd( 0.0, ( -b + sqrt( maxd( 0.0, b * b - a * c ) ) ) / a );
        }
        if ( g.dy > 0.0 )
          t = fmin( t, slabExit( p[1], u[1], g.dy ) );
        return t;
      }
    }
  }

  // Intersection of the ray with the slab |x| <= d as a parameter interval.
  __device__ __forceinline__ bool slabInterval( double x, double ux, double d, double& t1, double& t2 )
  {
    if ( ux != 0.0 ) {
      const double inv = 1.0 / ux;
      const double a = ( d - x ) * inv, b = ( -d - x ) * inv;
      t1 = fmax( t1, fmin( a, b ) );
      t2 = fmin( t2, fmax( a, b ) );
      return true;
    }
    return fabs( x ) <= d;
  }

  // Distance along the ray to the volume (distToVolumeEntry): 0 inside (or on
  // the surface pointing in), -1 when the ray misses it (NCMMC_Sphere.hh:
  // 110-160, NCMMC_Box.hh:112-205, NCMMC_Utils.cc:539-590).
  __device__ double distEntry( const Geom& g, const double* p, const double* u )
  {
    if ( g.kind == GEOM_SPHERE ) {
      const double pd = p[0] * u[0] + p[1] * u[1] + p[2] * u[2];
      const double c = p[0] * p[0] + p[1] * p[1] + p[2] * p[2] - g.r * g.r;
      if ( c <= 0.0 )
        return fmin( c, pd ) < 0.0 ? 0.0 : -1.0;
      const double D = pd * pd - c;
      if ( D < 0.0 )
        return -1.0;
      const double t = -( sqrt( D ) + pd );
      return t >= 0.0 ? t : -1.0;
    }
    if ( g.kind == GEOM_SLAB ) {
      const double a = fabs( p[2] ) - g.dz;
      const double xu = p[2] * u[2];
      if ( a <= 0.0 )
        return ( a != 0.0 || !( xu > 0.0 ) ) ? 0.0 : -1.0;
      return xu >= 0.0 ? -1.0 : a / fabs( u[2] );
    }
    double t1 = -infd(), t2 = infd();
    bool hit;
    if ( g.kind == GEOM_BOX ) {
      hit = slabInterval( p[0], u[0], g.dx, t1, t2 ) && slabInterval( p[1], u[1], g.dy, t1, t2 )
            && slabInterval( p[2], u[2], g.dz, t1, t2 );
    } else {
      // cylinder: radial interval, then the caps
      const double a = u[0] * u[0] + u[2] * u[2];
      const double b = p[0] * u[0] + p[2] * u[2];
      const double c = p[0] * p[0] + p[2] * p[2] - g.r * g.r;
      if ( a > 0.0 ) {
        const double D = b * b - a * c;
        hit = D >= 0.0;
        if ( hit ) {
          const double sd = sqrt( D );
          t1 = ( -b - sd ) / a;
          t2 = ( -b + sd ) / a;
        }
      } else {
        hit = c <= 0.0;
      }
      if ( hit && g.dy > 0.0 )
        hit = slabInterval( p[1], u[1], g.dy, t1, t2 );
    }
    if ( !hit || t1 >= t2 || t2 <= 0.0 )
      return -1.0;
    return maxd( 0.0, t1 );
  }

  // ---- random numbers ------------------------------------------------------------

  // Standard normal deviate (Box-Muller on two uniforms in (0,1]).
  __device__ __forceinline__ double randNormal( ncgb_rng& rng )
  {
    const double u1 = rand01( rng ), u2 = rand01( rng );
    return sqrt( -2.0 * log( u1 ) ) * cospi( 2.0 * u2 );
  }

  // randIsotropicDirection (NCRandUtils.cc:25-50, Marsaglia 1972) with the
  // reference's roundings (no contraction), so that |u|^2 - 1 is distributed
  // the same way: tallies of unscattered neutrons put mu = u.u0 at the edge
  // of the last bin.  The rejection loop is capped (acceptance pi/4).
  __device__ void randIsotropic( ncgb_rng& rng, double* u )
  {
    double x0 = 0.0, x1 = 0.0, s = 0.0;
    for ( int it = 0; it < 1000; ++it ) {
      x0 = __dsub_rn( 2.0 * rand01( rng ), 1.0 );
      x1 = __dsub_rn( 2.0 * rand01( rng ), 1.0 );
      s = __dadd_rn( __dmul_rn( x0, x0 ), __dmul_rn( x1, x1 ) );
      if ( s < 1.0 )
        break;
    }
    if ( !( s < 1.0 ) ) { x0 = 0.0; x1 = 0.0; s = 0.0; }
    const double t = 2.0 * sqrt( __dsub_rn( 1.0, s ) );
    u[0] = __dmul_rn( x0, t );
    u[1] = __dmul_rn( x1, t );
    u[2] = __dsub_rn( 1.0, 2.0 * s );
  }

  __device__ __forceinline__ double wl2ekin( double wl )
  {
    // convertBufWl2E, NCMMC_Source.cc:98-112
    const double wl2 = wl * wl;
    return kWl2Ekin / maxd( 4.9406564584124654e-324, wl2 );
  }

  // setEnergy (NCMMC_Source.cc:115-375)
  __device__ double sourceEnergy( const Source& s, ncgb_rng& rng )
  {
    switch ( s.ekind ) {
      case E_FIXED:
        return s.ea;
      case E_UNIFORM: {
        const double v = fmin( s.eb, s.ea + rand01( rng ) * ( s.eb - s.ea ) );
        return s.e_is_wl ? wl2ekin( v ) : v;
      }
      case E_LOGNORMAL: {
        const double v = exp( s.ea + s.eb * randNormal( rng ) );
        return s.e_is_wl ? wl2ekin( v ) : v;
      }
      default: {
        const double n1 = randNormal( rng ), n2 = randNormal( rng ), n3 = randNormal( rng );
        return s.ea * ( n1 * n1 + n2 * n2 + n3 * n3 );
      }
    }
  }

  // ---- tallies -----------------------------------------------------------------

  __device__ __forceinline__ long long orderKey( double x )
  {
    long long k = __double_as_longlong( x );
    return k < 0 ? ( k ^ 0x7FFFFFFFFFFFFFFFLL ) : k;
  }

  constexpr unsigned kFull = 0xffffffffu;

  // Bin of x (HistBinData1D::valueToBin with under/overflow recording,
  // NCHists.hh:376-400): 0 underflow, 1..nbins, nbins+1 overflow; x == xmax
  // goes to the last bin, and values that round up to nbins bins above xmin
  // to the overflow, as in the reference.
  __device__ __forceinline__ int binOf( const TallyHist& h, double x )
  {
    if ( x < h.xmin )
      return 0;
    if ( x >= h.xmax )
      return ( x == h.xmax ) ? h.nbins : h.nbins + 1;
    const double f = h.inv_delta * ( x - h.xmin );
    return 1 + ( f >= (double)h.nbins ? h.nbins : (int)f );
  }

  // Where a kernel's tally updates go: the warp's private statistics
  // (shared memory) and the block's bins, in shared memory as 64-bit
  // fixed-point integers (native integer atomics; FP64 atomics on shared
  // memory are compare-and-swap loops that contending lanes retry on the
  // narrow FP64 pipe) or, when they do not fit, the global FP64 buffer.
  // Indices are the global buffer's offsets (bins: minus nstat in shared
  // memory).
  struct TallyDst {
    double* stats;
    unsigned long long* ubins;
    double* gbins;
  };

  __device__ __forceinline__ void addBins( const TallyDst& d, const Tally& t, const TallyHist& h, int g, int bin,
                                           double wt, bool f )
  {
    if ( !f )
      return;
    const int64_t i = h.off + ( (int64_t)g * ( h.nbins + 2 ) + bin ) * 2;
    if ( d.ubins ) {
      unsigned long long* b = d.ubins + ( i - t.nstat );
      atomicAdd( b, __double2ull_rn( wt * t.cscale ) );
      atomicAdd( b + 1, __double2ull_rn( wt * wt * t.escale ) );
    } else {
      atomicAdd( d.gbins + i, wt );
      atomicAdd( d.gbins + i + 1, wt * wt );
    }
  }

  // Warp reduction of one group's running statistics (RunningStats1D,
  // NCHists.hh:613-650): sums of w, w x, w x^2 (FP64) and the extreme keys,
  // added by lane 0 to the warp's private slots.  Called by all 32 lanes; f
  // selects the contributing ones.
  __device__ __forceinline__ void addStats( double* st, double x, double xs, double wt, bool f )
  {
    double s0 = f ? wt : 0.0, s1 = f ? wt * xs : 0.0, s2 = f ? wt * xs * xs : 0.0;
    const long long k = orderKey( x );
    long long kmin = f ? k : 0x7FFFFFFFFFFFFFFFLL, kmax = f ? k : (long long)0x8000000000000000ULL;
#pragma unroll
    for ( int o = 16; o > 0; o >>= 1 ) {
      s0 += __shfl_xor_sync( kFull, s0, o );
      s1 += __shfl_xor_sync( kFull, s1, o );
      s2 += __shfl_xor_sync( kFull, s2, o );
      const long long a = __shfl_xor_sync( kFull, kmin, o ), b = __shfl_xor_sync( kFull, kmax, o );
      kmin = a < kmin ? a : kmin;
      kmax = b > kmax ? b : kmax;
    }
    if ( ( threadIdx.x & 31 ) == 0 ) {
      // the warp's private slots: one writer, no atomics
      st[0] += s0;
      st[1] += s1;
      st[2] += s2;
      long long* sk = reinterpret_cast<long long*>( st );
      if ( kmin < sk[3] ) sk[3] = kmin;
      if ( kmax > sk[4] ) sk[4] = kmax;
    }
    __syncwarp();
  }

  // Hist1D::fill (NCHists.hh:303-345, :525-530) of histogram h for the warp:
  // the total and, with breakdowns, the group of each lane's category.
  // Weighted fills skip weights <= 0; unweighted fills count 1.
  // One reduce-scatter step over the warp: lanes whose 'bit' is clear keep
  // the lower half of v, the others the upper half, each adding its
  // partner's copy of the kept half (n values in, n/2 out, n/2 adds).
  template<int N, class T, class Op>
  __device__ __forceinline__ void rsStep( T* v, int bit, Op op )
  {
    const bool upper = ( threadIdx.x >> bit ) & 1;
#pragma unroll
    for ( int j = 0; j < N / 2; ++j ) {
      const T send = upper ? v[j] : v[j + N / 2];
      const T keep = upper ? v[j + N / 2] : v[j];
      v[j] = op( keep, __shfl_xor_sync( kFull, send, 1 << bit ) );
    }
  }

  // Statistics of the five category groups in one warp reduce-scatter:
  // 15 sums (w, w x, w x^2 per category; 16 slots) end up one per lane pair
  // (lane l holds slot l >> 1) after 8+4+2+1+1 additions per lane, instead of
  // a 5-step butterfly of 3 sums for every category present; the extreme
  // keys (10 values, 2 x 8 slots) likewise on the integer pipe.  The lane
  // holding a slot adds it to the warp's private statistics.  Called by all
  // 32 lanes.
  __device__ __forceinline__ void addStatsCats( double* st, double x, double xs, double wt, bool f, int cat )
  {
    double v[16];
#pragma unroll
    for ( int c = 0; c < 5; ++c ) {
      const bool mine = f && cat == c;
      v[3 * c] = mine ? wt : 0.0;
      v[3 * c + 1] = mine ? wt * xs : 0.0;
      v[3 * c + 2] = mine ? wt * xs * xs : 0.0;
    }
    v[15] = 0.0;
    auto add = []( double a, double b ) { return a + b; };
    rsStep<16>( v, 4, add );
    rsStep<8>( v, 3, add );
    rsStep<4>( v, 2, add );
    rsStep<2>( v, 1, add );
    v[0] += __shfl_xor_sync( kFull, v[0], 1 );
    const int lane = threadIdx.x & 31;
    const int slot = lane >> 1;
    if ( ( lane & 1 ) == 0 && slot < 15 && v[0] != 0.0 )
      st[( 1 + slot / 3 ) * kStats + slot % 3] += v[0];
    // extremes: 8 slots of minima (5 used) and 8 of maxima
    const long long k = orderKey( x );
    long long mn[8], mx[8];
#pragma unroll
    for ( int c = 0; c < 8; ++c ) {
      const bool mine = f && cat == c;
      mn[c] = mine ? k : 0x7FFFFFFFFFFFFFFFLL;
      mx[c] = mine ? k : (long long)0x8000000000000000ULL;
    }
    auto lo = []( long long a, long long b ) { return a < b ? a : b; };
    auto hi = []( long long a, long long b ) { return a > b ? a : b; };
    rsStep<8>( mn, 4, lo );
    rsStep<8>( mx, 4, hi );
    rsStep<4>( mn, 3, lo );
    rsStep<4>( mx, 3, hi );
    rsStep<2>( mn, 2, lo );
    rsStep<2>( mx, 2, hi );
    mn[0] = lo( mn[0], __shfl_xor_sync( kFull, mn[0], 2 ) );
    mx[0] = hi( mx[0], __shfl_xor_sync( kFull, mx[0], 2 ) );
    mn[0] = lo( mn[0], __shfl_xor_sync( kFull, mn[0], 1 ) );
    mx[0] = hi( mx[0], __shfl_xor_sync( kFull, mx[0], 1 ) );
    const int ks = lane >> 2;
    if ( ( lane & 3 ) == 0 && ks < 5 ) {
      long long* sk = reinterpret_cast<long long*>( st + ( 1 + ks ) * kStats );
      if ( mn[0] < sk[3] ) sk[3] = mn[0];
      if ( mx[0] > sk[4] ) sk[4] = mx[0];
    }
    __syncwarp();
  }

  // With breakdowns only the five category groups are filled: the host
  // forms the total as their sum (bins, sums) and extremes.
  __device__ void histFillWarp( const TallyDst& d, const Tally& t, int kind, int cat, double x, double w,
                                bool weighted, bool on )
  {
    const TallyHist& h = t.h[kind];
    const bool f = on && ( !weighted || w > 0.0 );
    if ( !__any_sync( kFull, f ) )
      return;
    const double wt = weighted ? w : 1.0;
    const int bin = f ? binOf( h, x ) : 0;
    const double xs = x - t.shift[kind];
    if ( !t.breakdown ) {
      addBins( d, t, h, 0, bin, wt, f );
      addStats( d.stats + h.soff, x, xs, wt, f );
      return;
    }
    addBins( d, t, h, 1 + cat, bin, wt, f );
    addStatsCats( d.stats + h.soff, x, xs, wt, f, cat );
  }

  // tallyRecord (NCMMC_StdTallies.cc:430-660) for the warp's neutrons ('on'
  // lanes).  Called by all 32 lanes.
  template<bool Fast>
  __device__ void tallyWarp( const TallyDst& buf, const Tally& t, bool on, double e, const double* u, double w,
                             int nscat, int ninel, double e0, const double* d0 )
  {
    // init_dethistidvect, NCMMC_StdTallies.cc:288-308
    const int cat = nscat > 1 ? ( ninel ? 4 : 3 ) : ( nscat == 1 ? ( ninel ? 2 : 1 ) : 0 );
    if ( t.h[T_THETA].enabled | t.h[T_MU].enabled | t.h[T_Q].enabled ) {
      // the reference's roundings (NCMMC_StdTallies.cc:530-560): unscattered
      // neutrons sit at mu = 1 up to the last bits, on the last bin's edge
      double mu;
      if ( t.fixed_dir && t.d0z == 1.0 )
        mu = u[2];
      else if ( t.fixed_dir )
        mu = __dadd_rn( __dadd_rn( __dmul_rn( t.d0x, u[0] ), __dmul_rn( t.d0y, u[1] ) ), __dmul_rn( t.d0z, u[2] ) );
      else
        mu = __dadd_rn( __dadd_rn( __dmul_rn( d0[0], u[0] ), __dmul_rn( d0[1], u[1] ) ), __dmul_rn( d0[2], u[2] ) );
      mu = clampd( mu, -1.0, 1.0 );
      if ( t.h[T_MU].enabled )
        histFillWarp( buf, t, T_MU, cat, mu, w, true, on );
      if ( t.h[T_Q].enabled ) {
        const double ei = t.fixed_e ? t.e0 : e0;
        const double q2 = __dmul_rn( __dadd_rn( __dadd_rn( __dmul_rn( __dmul_rn( sqrt( __dmul_rn( e, ei ) ), mu ), -2.0 ),
                                                           ei ), e ), kEkin2Ksq );
        histFillWarp( buf, t, T_Q, cat, sqrt( maxd( 0.0, q2 ) ), w, true, on );
      }
      if ( t.h[T_THETA].enabled )
        histFillWarp( buf, t, T_THETA, cat, Fast ? (double)( acosf( (float)mu ) * (float)kToDeg ) : acos( mu ) * kToDeg,
                      w, true, on );
    }
    if ( t.h[T_E].enabled )
      histFillWarp( buf, t, T_E, cat, e, w, true, on );
    if ( t.h[T_DE].enabled )
      histFillWarp( buf, t, T_DE, cat, ( t.fixed_e ? t.e0 : e0 ) - e, w, true, on );
    if ( t.h[T_L].enabled )
      histFillWarp( buf, t, T_L, cat, sqrt( kWl2Ekin ) * sqrt( 1.0 / maxd( 4.9406564584124654e-324, e ) ), w,
                    true, on );
    if ( t.h[T_NSCAT].enabled )
      histFillWarp( buf, t, T_NSCAT, cat, (double)nscat, w, true, on );
    if ( t.h[T_NSCAT_UW].enabled )
      histFillWarp( buf, t, T_NSCAT_UW, cat, (double)nscat, w, false, on );
    if ( t.h[T_W].enabled )
      histFillWarp( buf, t, T_W, cat, w, w, false, on );
  }

  constexpr int kBlock = 256;
  constexpr int kWarps = kBlock / 32;

  // Block-local tallies in shared memory: kWarps private copies of the
  // statistics, then (when 'bins') the bins as fixed-point integers.  Min/max
  // keys start at the empty values, everything else at zero.
  __device__ TallyDst tallyInitShared( double* sh, const Tally& t, bool bins )
  {
    const int64_t ns = (int64_t)kWarps * t.nstat;
    const int64_t n = ns + ( bins ? t.nbuf - t.nstat : 0 );
    for ( int64_t i = threadIdx.x; i < n; i += blockDim.x ) {
      long long v = 0;
      if ( i < ns ) {
        const int j = (int)( ( i % t.nstat ) % kStats );
        if ( j == 3 ) v = 0x7FFFFFFFFFFFFFFFLL;
        if ( j == 4 ) v = (long long)0x8000000000000000ULL;
      }
      sh[i] = __longlong_as_double( v );
    }
    __syncthreads();
    TallyDst d;
    d.stats = sh + ( threadIdx.x >> 5 ) * t.nstat;
    d.ubins = bins ? reinterpret_cast<unsigned long long*>( sh + ns ) : nullptr;
    d.gbins = t.buf;
    return d;
  }

  __device__ void tallyFlushShared( const double* sh, const Tally& t, bool bins )
  {
    __syncthreads();
    for ( int64_t i = threadIdx.x; i < t.nstat; i += blockDim.x ) {
      const int j = (int)( i % kStats );
      if ( j < 3 ) {
        double v = 0.0;
        for ( int w = 0; w < kWarps; ++w )
          v += sh[w * t.nstat + i];
        if ( v != 0.0 )
          atomicAdd( t.buf + i, v );
      } else {
        long long kv = j == 3 ? 0x7FFFFFFFFFFFFFFFLL : (long long)0x8000000000000000ULL;
        for ( int w = 0; w < kWarps; ++w ) {
          const long long x = __double_as_longlong( sh[w * t.nstat + i] );
          kv = j == 3 ? ( x < kv ? x : kv ) : ( x > kv ? x : kv );
        }
        long long* dst = reinterpret_cast<long long*>( t.buf + i );
        if ( j == 3 && kv != 0x7FFFFFFFFFFFFFFFLL )
          atomicMin( dst, kv );
        if ( j == 4 && kv != (long long)0x8000000000000000ULL )
          atomicMax( dst, kv );
      }
    }
    if ( bins ) {
      const unsigned long long* ub = reinterpret_cast<const unsigned long long*>( sh + (int64_t)kWarps * t.nstat );
      const double ic = 1.0 / t.cscale, ie = 1.0 / t.escale;
      for ( int64_t i = threadIdx.x; i < t.nbuf - t.nstat; i += blockDim.x ) {
        const unsigned long long v = ub[i];
        if ( v )
          atomicAdd( t.buf + t.nstat + i, (double)v * ( ( i & 1 ) ? ie : ic ) );
      }
    }
  }

  // Warp-aggregated append: slot of this lane among the lanes with 'want'.
  __device__ __forceinline__ unsigned long long appendSlot( unsigned long long* counter, bool want )
  {
    const unsigned active = __activemask();
    const unsigned mask = __ballot_sync( active, want );
    unsigned long long base = 0;
    const int lane = threadIdx.x & 31;
    if ( mask ) {
      const int leader = __ffs( mask ) - 1;
      if ( lane == leader )
        base = atomicAdd( counter, (unsigned long long)__popc( mask ) );
      base = __shfl_sync( active, base, leader );
    }
    return base + __popc( mask & ( ( 1u << lane ) - 1u ) );
  }

  // Warp sums of the tallied (or missed) counts, added to block totals in
  // shared memory.  Called by all 32 lanes.
  struct BlockSums {
    unsigned long long n;
    double w;
  };

  __device__ __forceinline__ void addCount( BlockSums* bs, bool on, double w )
  {
    const unsigned m = __ballot_sync( kFull, on );
    double s = on ? w : 0.0;
#pragma unroll
    for ( int o = 16; o > 0; o >>= 1 )
      s += __shfl_xor_sync( kFull, s, o );
    if ( m && ( threadIdx.x & 31 ) == 0 ) {
      atomicAdd( &bs->n, (unsigned long long)__popc( m ) );
      atomicAdd( &bs->w, s );
    }
  }

  // Source neutrons first_id .. first_id+count-1: fillBasket of the source
  // (NCMMC_Source.cc) and BasketSrcFiller::propagateToVolume
  // (NCMMC_BasketSrcFiller.hh:120-178): neutrons that miss the volume are
  // tallied with nscat = -1 (NCMMC_Baskets.cc:81) unless ignoremiss, and
  // counted; the rest are moved onto the volume and appended to population a.
  // Warp-uniform loop (all lanes iterate together for the warp collectives).
  __global__ void __launch_bounds__(kBlock)
  k_mmc_emit( const Source src, const Geom g, const Engine eng, const Tally t, Pop a, uint64_t base,
              uint64_t first_id, uint64_t count, Counters* c, int bins_smem )
  {
    extern __shared__ double sh[];
    __shared__ BlockSums miss, tal;
    const TallyDst tb = tallyInitShared( sh, t, bins_smem );
    if ( threadIdx.x == 0 ) { miss.n = 0; miss.w = 0.0; tal.n = 0; tal.w = 0.0; }
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for ( uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < count; i0 += stride ) {
      const uint64_t i = i0 + threadIdx.x;
      const bool on = i < count;
      const uint64_t id = first_id + i;
      ncgb_rng rng;
      ncgb_rng_init( &rng, eng.seed, (uint32_t)id, 0u, kStreamSource );
      double p[3] = { src.x, src.y, src.z };
      double u[3] = { src.ux, src.uy, src.uz };
      double e = 0.0;
      if ( on ) {
        if ( src.kind == SRC_CIRCULAR && src.r > 0.0 ) {
          // uniform point in the unit disk (polar form of randPointInUnitCircle)
          const double rad = sqrt( rand01( rng ) ), phi = 2.0 * rand01( rng );
          const double a0 = rad * cospi( phi ), b0 = rad * sinpi( phi );
          p[0] += src.ax * a0 + src.bx * b0;
          p[1] += src.ay * a0 + src.by * b0;
          p[2] += src.az * a0 + src.bz * b0;
        } else if ( src.kind == SRC_ISOTROPIC ) {
          randIsotropic( rng, u );
          if ( src.r != 0.0 ) {
            p[0] -= u[0] * src.r;
            p[1] -= u[1] * src.r;
            p[2] -= u[2] * src.r;
          }
        }
        e = sourceEnergy( src, rng );
      }
      bool keep = on, missed = false;
      if ( on && src.might_be_outside ) {
        const double d = distEntry( g, p, u );
        if ( d < 0.0 ) {
          keep = false;
          missed = true;
        } else {
          p[0] += d * u[0];
          p[1] += d * u[1];
          p[2] += d * u[2];
        }
      }
      addCount( &miss, missed, 1.0 );
      const bool tally_miss = missed && !eng.ignore_miss;
      if ( __any_sync( kFull, tally_miss ) ) {
        tallyWarp<false>( tb, t, tally_miss, e, u, 1.0, -1, 0, e, u );
        addCount( &tal, tally_miss, 1.0 );
      }
      const unsigned long long slot = appendSlot( &c->n_a, keep );
      if ( keep ) {
        const uint64_t j = base + slot;
        a.pos[3 * j] = p[0]; a.pos[3 * j + 1] = p[1]; a.pos[3 * j + 2] = p[2];
        a.dir[3 * j] = u[0]; a.dir[3 * j + 1] = u[1]; a.dir[3 * j + 2] = u[2];
        a.e[j] = e;
        a.w[j] = 1.0;
        a.xs[j] = -1.0;
        a.nscat[j] = 0;
        a.ninel[j] = 0;
        a.id[j] = (uint32_t)id;
        a.e0[j] = e;
        a.d0[3 * j] = u[0]; a.d0[3 * j + 1] = u[1]; a.d0[3 * j + 2] = u[2];
        a.st[j] = kNoScatter;
      }
    }
    tallyFlushShared( sh, t, bins_smem );
    __syncthreads();
    if ( threadIdx.x == 0 ) {
      if ( miss.n ) {
        atomicAdd( &c->miss, miss.n );
        atomicAdd( &c->miss_w, miss.w );
      }
      if ( tal.n ) {
        atomicAdd( &c->tallied, tal.n );
        atomicAdd( &c->tallied_w, tal.w );
      }
    }
  }

  // One engine step over population a (StdSimEngine::processBasket,
  // NCMMC_SimEngine.cc:170-440).  Warp-uniform loop, as k_mmc_emit.
  template<bool Fast>
  __global__ void __launch_bounds__(kBlock)
  k_mmc_transport( const __grid_constant__ ncgb_material_view m, const Geom g, const Engine eng, const Tally t,
                   const Pop a, uint64_t n_a, const Pop b, uint32_t step, Counters* c, int bins_smem )
  {
    extern __shared__ double sh[];
    __shared__ BlockSums tal;
    const TallyDst tb = tallyInitShared( sh, t, bins_smem );
    if ( threadIdx.x == 0 ) { tal.n = 0; tal.w = 0.0; }
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for ( uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < n_a; i0 += stride ) {
      const uint64_t i = i0 + threadIdx.x;
      bool on = i < n_a;
      double p[3] = { 0.0, 0.0, 0.0 }, u[3] = { 0.0, 0.0, 1.0 }, d0[3] = { 0.0, 0.0, 1.0 };
      double e = 0.0, w = 0.0, xs = 0.0, e0 = 0.0;
      int nscat = 0, ninel = 0;
      uint32_t id = 0;
      if ( on ) {
        p[0] = a.pos[3 * i]; p[1] = a.pos[3 * i + 1]; p[2] = a.pos[3 * i + 2];
        e = a.e[i]; w = a.w[i]; xs = a.xs[i];
        nscat = a.nscat[i]; ninel = a.ninel[i];
        id = a.id[i];
        e0 = a.e0[i];
        d0[0] = a.d0[3 * i]; d0[1] = a.d0[3 * i + 1]; d0[2] = a.d0[3 * i + 2];
        const int pst = a.st[i];
        if ( pst == kNoScatter ) {
          u[0] = a.dir[3 * i]; u[1] = a.dir[3 * i + 1]; u[2] = a.dir[3 * i + 2];
        } else if ( pst == NCGB_ST_OK ) {
          // the scatter of the previous step (NCMMC_SimEngine.cc:390-410)
          const double en = a.e_new[i];
          u[0] = a.dir_new[3 * i]; u[1] = a.dir_new[3 * i + 1]; u[2] = a.dir_new[3 * i + 2];
          ++nscat;
          if ( en != e ) {
            ++ninel;
            xs = -1.0;   // the cross-section might have changed
          }
          e = en;
        } else {
          // the reference aborts the run here; the host reports the failure
          atomicAdd( &c->nfail, 1ull );
          on = false;
        }
      }
      bool keep = false;
      double wk = 0.0, wt = 0.0, ds = 0.0;
      if ( on ) {
        const double dexit = distExit( g, p, u );
        const bool dinf = !finited( dexit );
        // absorption (evalManyXSIsotropic of AbsOOV) and scattering (the
        // cached value unless new or changed) macroscopic cross-sections
        const double xabs = eng.has_abs ? eng.macro * absXS( eng.abs_c, e ) : 0.0;
        if ( !eng.has_scat || eng.nscatlimit == 0 || ( eng.nscatlimit > 0 && nscat >= eng.nscatlimit ) ) {
          xs = 0.0;
        } else if ( nscat <= 0 || xs < 0.0 ) {
          double x = 0.0;
          if ( contains( m.dom_elow, m.dom_ehigh, e ) ) {
            ncgb_rng dummy;
            ncgb_rng_init( &dummy, 0, 0, 0, 0 );
            x = xsAndPick<false, Fast>( m, e, dummy ).xs;
          }
          xs = eng.macro * x;
        }
        // calcProbTransm (NCMMC_Utils.cc:46-88): 0 for an infinite path.
        // The mixed mode takes the attenuation factors and the sampled
        // distance in FP32 (relative 1e-7 of a weight or a path length).
        const double xsc = fmin( kDblMax, xs );
        const double ptransm = ( g.unbounded && dinf ) ? 0.0
                             : ( xsc != 0.0 ? ( Fast ? (double)expf( (float)( -xsc * dexit ) ) : exp( -xsc * dexit ) )
                                            : 1.0 );
        // sampleRandDists (NCMMC_Utils.cc:153-176); log(1 + r expm1(-t)) as
        // log1p in the mixed mode, accurate for thin paths
        ncgb_rng rng;
        ncgb_rng_init( &rng, eng.seed, id, step, kStreamEngine );
        const double r = rand01( rng );
        if ( xs == 0.0 )
          ds = infd();
        else if ( dinf )
          ds = ( Fast ? (double)logf( (float)r ) : log( r ) ) / ( -xs );
        else if ( Fast )
          ds = ( -1.0 / xs ) * (double)log1pf( (float)r * expm1f( (float)( -xs * dexit ) ) );
        else
          ds = ( -1.0 / xs ) * log( 1.0 + r * expm1( -xs * dexit ) );
        // the part that scatters: roulette, attenuation, move to the point
        if ( w != 0.0 && finited( ds ) && xs > 0.0 ) {
          double rf = 1.0;
          keep = true;
          if ( nscat >= eng.nscatthr && w < eng.wthr ) {
            if ( rand01( rng ) > eng.psurv )
              keep = false;
            else
              rf = eng.boost;
          }
          if ( keep ) {
            const double wr = Fast ? (double)expf( (float)( -xabs * ds ) ) : exp( -xabs * ds );
            keep = wr > 0.0;
            wk = w * rf * wr * ( 1.0 - ptransm );
          }
        }
        // the transmitted part, at the exit (propagateAndAttenuate, then the
        // scatter-process transmission), is tallied
        double pabs;
        if ( eng.has_abs ) {
          const double xa = fmin( kDblMax, xabs );
          pabs = ( g.unbounded && dinf ) ? 0.0
               : ( xa != 0.0 ? ( Fast ? (double)expf( (float)( -xa * dexit ) ) : exp( -xa * dexit ) ) : 1.0 );
        } else {
          pabs = ( g.unbounded && dinf ) ? 0.0 : 1.0;
        }
        wt = w * pabs * ptransm;
      }
      const unsigned long long slot = appendSlot( &c->n_b, keep );
      if ( keep ) {
        const uint64_t j = slot;
        b.pos[3 * j] = p[0] + ds * u[0];
        b.pos[3 * j + 1] = p[1] + ds * u[1];
        b.pos[3 * j + 2] = p[2] + ds * u[2];
        b.dir[3 * j] = u[0]; b.dir[3 * j + 1] = u[1]; b.dir[3 * j + 2] = u[2];
        b.e[j] = e;
        b.w[j] = wk;
        b.xs[j] = xs;
        b.nscat[j] = nscat;
        b.ninel[j] = ninel;
        b.id[j] = id;
        b.e0[j] = e0;
        b.d0[3 * j] = d0[0]; b.d0[3 * j + 1] = d0[1]; b.d0[3 * j + 2] = d0[2];
      }
      tallyWarp<Fast>( tb, t, on, e, u, wt, nscat, ninel, e0, d0 );
      addCount( &tal, on, wt );
    }
    tallyFlushShared( sh, t, bins_smem );
    __syncthreads();
    if ( threadIdx.x == 0 && tal.n ) {
      atomicAdd( &c->tallied, tal.n );
      atomicAdd( &c->tallied_w, tal.w );
    }
  }

  int gridFor( uint64_t n, int block, int cap )
  {
    const uint64_t g = ( n + block - 1 ) / block;
    return (int)( g < (uint64_t)cap ? ( g ? g : 1 ) : cap );
  }
}

namespace ncgb {
  namespace mmc {

    // Bins in shared memory when the whole buffer fits in the budget
    // (NCGB_MMC_SMEM_KB, default 96 KB: two 256-thread blocks per SM for the
    // five default-sized tallies); the statistics always.
    static std::size_t smemBudget()
    {
      static std::size_t b = [] {
        const char* v = std::getenv( "NCGB_MMC_SMEM_KB" );
        const long kb = v ? std::atol( v ) : 96;
        return (std::size_t)( kb > 0 && kb <= 220 ? kb : 96 ) * 1024;
      }();
      return b;
    }

    template<class K>
    static cudaError_t allowSmem( K kernel, std::size_t bytes )
    {
      if ( bytes <= 48 * 1024 )
        return cudaSuccess;
      return cudaFuncSetAttribute( kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes );
    }

    static std::size_t tallySmem( const Tally& t, bool& bins )
    {
      const std::size_t st = (std::size_t)kWarps * t.nstat * sizeof(double);
      const std::size_t bb = (std::size_t)( t.nbuf - t.nstat ) * sizeof(double);
      bins = st + bb <= smemBudget();
      return st + ( bins ? bb : 0 );
    }

    // Fixed-point scales of the shared-memory bins for a launch of 'grid'
    // blocks over n neutrons whose tally weights are at most wmax: the
    // largest powers of two (<= 2^60) that keep a block's sums below 2^62.
    static Tally withScales( Tally t, uint64_t n, int grid, double wmax )
    {
      const double per_block = (double)kBlock * (double)( ( n + (uint64_t)grid * kBlock - 1 ) / ( (uint64_t)grid * kBlock ) );
      const double wm = wmax > 1.0 ? wmax : 1.0;
      t.cscale = std::ldexp( 1.0, std::min( 60, (int)std::floor( 62.0 - std::log2( per_block * wm ) ) ) );
      t.escale = std::ldexp( 1.0, std::min( 60, (int)std::floor( 62.0 - std::log2( per_block * wm * wm ) ) ) );
      return t;
    }

    // Largest tally weight: 1 from the source; roulette survivors below the
    // threshold are boosted by 1/psurvival, and weights only fall otherwise.
    static double maxWeight( const Engine& eng ) { return std::max( 1.0, eng.wthr * eng.boost ); }

    cudaError_t launchEmit( const Source& src, const Geom& g, const Engine& eng, const Tally& t, Pop a,
                            uint64_t base, uint64_t first_id, uint64_t count, Counters* c, int numSMs,
                            cudaStream_t s )
    {
      if ( count == 0 )
        return cudaSuccess;
      bool bins = false;
      const std::size_t sbytes = tallySmem( t, bins );
      cudaError_t e = allowSmem( k_mmc_emit, sbytes );
      if ( e != cudaSuccess )
        return e;
      const int grid = gridFor( count, kBlock, numSMs * 4 );
      k_mmc_emit<<<grid, kBlock, sbytes, s>>>( src, g, eng, withScales( t, count, grid, 1.0 ), a, base, first_id,
                                               count, c, bins ? 1 : 0 );
      return cudaGetLastError();
    }

    cudaError_t launchTransport( const ncgb_material_view& m, const Geom& g, const Engine& eng, const Tally& t,
                                 Pop a, uint64_t n_a, Pop b, uint32_t step, Counters* c, int numSMs,
                                 cudaStream_t s )
    {
      if ( n_a == 0 )
        return cudaSuccess;
      bool bins = false;
      const std::size_t sbytes = tallySmem( t, bins );
      const int grid = gridFor( n_a, kBlock, numSMs * 4 );
      const Tally ts = withScales( t, n_a, grid, maxWeight( eng ) );
      cudaError_t e;
      if ( eng.fast ) {
        e = allowSmem( k_mmc_transport<true>, sbytes );
        if ( e == cudaSuccess )
          k_mmc_transport<true><<<grid, kBlock, sbytes, s>>>( m, g, eng, ts, a, n_a, b, step, c, bins ? 1 : 0 );
      } else {
        e = allowSmem( k_mmc_transport<false>, sbytes );
        if ( e == cudaSuccess )
          k_mmc_transport<false><<<grid, kBlock, sbytes, s>>>( m, g, eng, ts, a, n_a, b, step, c, bins ? 1 : 0 );
      }
      return e != cudaSuccess ? e : cudaGetLastError();
    }
  }
}
