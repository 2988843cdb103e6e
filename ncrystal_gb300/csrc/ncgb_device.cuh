// Device-side evaluation of neutrons against one material: cross-section
// (ProcComposition over PowderBragg / ElIncScatter / SABScatter / FreeGas) and
// one isotropic scatter (E', mu).  FP64 arithmetic, so that results agree with
// NCrystal's own to rounding; the control flow and the order of random draws
// follow the reference function for function (each cites its source).
//
// GB300 notes (its FP64 pipe is 1/64 of the FP32 rate, and every warp
// instruction occupies it for the full warp whatever the number of active
// lanes):
//   * Binary searches over non-negative tables (energy grids, cumulative sums,
//     CDFs) compare IEEE-754 bit patterns as 64-bit integers: same order as a
//     floating-point compare for non-negative doubles, on the integer pipe.
//   * Uniform doubles are assembled from the Philox bits with integer ops.
//   * The S(alpha,beta) sampler is a per-lane state machine (one Alg.1
//     attempt per step), driven by a persistent kernel that refills finished
//     lanes from a queue, so that warps stay full through the rejection loops.
//   * Every loop is bounded.  A neutron whose rejection loop hits the
//     reference's cap (100 tries) ends with status NCGB_ST_LOOPCAP, which the
//     host reports as the reference's CalcError.
#ifndef NCGB_DEVICE_CUH
#define NCGB_DEVICE_CUH

#include <cstdint>
#include "ncgb_philox.h"
#include "ncgb_tables.h"
#include "ncrystal_gb300.h"

namespace ncgb_dev {

  __device__ __forceinline__ double ldg( const double* p ) { return __ldg(p); }
  __device__ __forceinline__ long long ldgbits( const double* p ) { return __double_as_longlong( __ldg(p) ); }
  __device__ __forceinline__ long long bits( double x ) { return __double_as_longlong(x); }

  __device__ __forceinline__ void refill( ncgb_rng& r )
  {
    uint32_t ctr[4] = { r.block, r.ctr1, r.ctr2, r.ctr3 };
    ncgb_philox4x32_10( ctr, r.key0, r.key1, r.word );
    r.block += 1;
    r.have = 4;
  }

  // The next 32-bit word of the stream (ncgb_rng_u32), selected without
  // dynamic indexing so that the words stay in registers.
  __device__ __forceinline__ uint32_t rand_u32( ncgb_rng& r )
  {
    if ( r.have == 0 )
      refill( r );
    const uint32_t h = r.have;
    const uint32_t w = h == 4 ? r.word[0] : h == 3 ? r.word[1] : h == 2 ? r.word[2] : r.word[3];
    r.have = h - 1;
    return w;
  }

  // Uniform double in (0,1]: same value as ncgb_rng_generate, built with
  // integer ops (k in [1, 2^53] -> k * 2^-53, exact).
  __device__ __forceinline__ double rand01( ncgb_rng& r )
  {
    if ( r.have < 2 )
      refill( r );
    const uint32_t h = r.have;
    const uint32_t lo = h == 4 ? r.word[0] : h == 3 ? r.word[1] : r.word[2];
    const uint32_t hi = h == 4 ? r.word[1] : h == 3 ? r.word[2] : r.word[3];
    r.have = h - 2;
    const uint64_t k = ( ( (uint64_t)lo | ( (uint64_t)hi << 32 ) ) >> 11 ) + 1;
    const int p = 63 - __clzll( (long long)k );           // highest set bit, 0..53
    const uint64_t mant = ( k << ( 52 - ( p < 52 ? p : 52 ) ) ) & 0xFFFFFFFFFFFFFull;
    const uint64_t b = ( p == 53 ) ? 0x3FF0000000000000ull
                                   : ( ( (uint64_t)( p + 970 ) << 52 ) | mant );
    return __longlong_as_double( (long long)b );
  }

  // std::upper_bound on [a, a+n) for x >= 0 and a[] >= 0 (not NaN): first i
  // with a[i] > x.
  __device__ __forceinline__ int64_t upper_bound_nn( const double* a, int64_t n, double x )
  {
    const long long xb = bits(x);
    int64_t lo = 0, len = n;
    while ( len > 0 ) {
      int64_t half = len >> 1;
      if ( !( xb < ldgbits( a + lo + half ) ) ) { lo += half + 1; len -= half + 1; }
      else len = half;
    }
    return lo;
  }

  // std::lower_bound on [a, a+n) for x >= 0 and a[] >= 0: first i with a[i] >= x.
  __device__ __forceinline__ int64_t lower_bound_nn( const double* a, int64_t n, double x )
  {
    const long long xb = bits(x);
    int64_t lo = 0, len = n;
    while ( len > 0 ) {
      int64_t half = len >> 1;
      if ( ldgbits( a + lo + half ) < xb ) { lo += half + 1; len -= half + 1; }
      else len = half;
    }
    return lo;
  }

  // 32-bit copies for the S(alpha,beta) tables (indexed below 2^31, checked
  // by the table loader): fewer registers in the sampling pass.
  __device__ __forceinline__ int upper_bound_nn32( const double* a, int n, double x )
  {
    const long long xb = bits(x);
    int lo = 0, len = n;
    while ( len > 0 ) {
      const int half = len >> 1;
      if ( !( xb < ldgbits( a + lo + half ) ) ) { lo += half + 1; len -= half + 1; }
      else len = half;
    }
    return lo;
  }

  __device__ __forceinline__ int lower_bound_nn32( const double* a, int n, double x )
  {
    const long long xb = bits(x);
    int lo = 0, len = n;
    while ( len > 0 ) {
      const int half = len >> 1;
      if ( ldgbits( a + lo + half ) < xb ) { lo += half + 1; len -= half + 1; }
      else len = half;
    }
    return lo;
  }

  __device__ __forceinline__ double clampd( double x, double lo, double hi ) { return x < lo ? lo : ( x > hi ? hi : x ); }
  __device__ __forceinline__ double maxd( double a, double b ) { return a < b ? b : a; }
  __device__ __forceinline__ bool contains( double lo, double hi, double e ) { return e >= lo && e <= hi; }
  // The same for lo >= 0 and e >= 0 (not NaN), compared as int64 bit patterns.
  __device__ __forceinline__ bool containsNN( double lo, double hi, double e )
  {
    const long long b = bits( e );
    return b >= bits( lo ) && b <= bits( hi );
  }
  __device__ __forceinline__ bool finited( double x ) { return ( bits(x) & 0x7FF0000000000000LL ) != 0x7FF0000000000000LL; }
  __device__ __forceinline__ double infd() { return __longlong_as_double( 0x7FF0000000000000LL ); }

  // ---- kinematics (NCKinUtils.hh:64-124, NCKinUtils.cc:25-58) ---------------
  struct ALim { double lo, hi; };

  __device__ __forceinline__ ALim alphaLimits( double x, double beta )
  {
    ALim r;
    const double kk = x + beta;
    if ( !( kk >= 0.0 ) ) { r.lo = 1.0; r.hi = -1.0; return r; }
    const double a = kk + x;
    const double b = 2.0 * sqrt( x * kk );
    if ( fabs(beta) < 0.01 * x ) {
      const double t = beta / x;
      r.lo = beta*t*(1./4.+t*(-1./8.+t*(5./64.+t*(-7./128.+t*(21./512.+t*(-33./1024.+t*(429./16384.+t*(-715./32768.))))))));
    } else {
      r.lo = maxd( 0.0, a - b );
    }
    r.hi = a + b;
    return r;
  }

  __device__ __forceinline__ bool inInterval( double lo, double hi, double x ) { return x >= lo && x <= hi; }

  // The alpha limits in FP32 (mixed-precision mode) in a form free of
  // cancellation: with s = sqrt(x+beta) + sqrt(x), alpha+ = s^2 and
  // alpha- = (sqrt(x+beta) - sqrt(x))^2 = beta^2 / s^2 (relative error ~1e-7
  // everywhere, including near the elastic line where the FP64 form needs its
  // Taylor branch).  kk = x + beta is formed in FP64 by the caller.
  struct ALimF { float lo, hi; };
  __device__ __forceinline__ ALimF alphaLimitsF( float x, float kk, float beta )
  {
    ALimF r;
    if ( !( kk >= 0.0f ) ) { r.lo = 1.0f; r.hi = -1.0f; return r; }
    const float sq = sqrtf( kk ) + sqrtf( x );
    r.hi = sq * sq;
    r.lo = ( beta * beta ) / r.hi;
    return r;
  }

  __device__ __forceinline__ void neumaierAdd( double& s, double& c, double x )
  {
    double t = s + x;
    c += ( fabs(s) >= fabs(x) ) ? (s-t)+x : (x-t)+s;
    s = t;
  }

  // randDirectionGivenScatterMu, NCRandUtils.cc:51-96 (via
  // randNeutronDirectionGivenScatterMu, NCRandUtils.hh:152-155): the outgoing
  // direction at cosine mu to 'in' with a uniform azimuth, from a random unit
  // vector (Marsaglia) crossed with the normalised 'in'.  Every operation is
  // rounded separately, as the reference's C++ evaluates it, so that the
  // result is the reference's to the bit.  Returns NCGB_ST_OK, or LOOPCAP if
  // 100000 trial vectors were all nearly parallel to 'in'.
  __device__ __forceinline__ int randDirGivenMu( ncgb_rng& rng, double mu, const double* in, double* out )
  {
    const double m2 = __dadd_rn( __dadd_rn( __dmul_rn( in[0], in[0] ), __dmul_rn( in[1], in[1] ) ),
                                 __dmul_rn( in[2], in[2] ) );
    const double invm = ( fabs( __dsub_rn( m2, 1.0 ) ) < 1e-14 ) ? 1.0 : __ddiv_rn( 1.0, sqrt( m2 ) );
    const double u0 = __dmul_rn( in[0], invm ), u1 = __dmul_rn( in[1], invm ), u2 = __dmul_rn( in[2], invm );
    double t0 = 0.0, t1 = 0.0, t2 = 0.0, tm2 = 0.0;
    int it = 0;
    for ( ; it < 100000; ++it ) {
      const double x0 = __dsub_rn( 2.0 * rand01( rng ), 1.0 );
      const double x1 = __dsub_rn( 2.0 * rand01( rng ), 1.0 );
      const double s = __dadd_rn( __dmul_rn( x0, x0 ), __dmul_rn( x1, x1 ) );
      if ( s < 1.0 ) {
        const double t = 2.0 * sqrt( __dsub_rn( 1.0, s ) );
        const double a0 = __dmul_rn( x0, t ), a1 = __dmul_rn( x1, t ), a2 = __dsub_rn( 1.0, 2.0 * s );
        t0 = __dsub_rn( __dmul_rn( a1, u2 ), __dmul_rn( a2, u1 ) );
        t1 = __dsub_rn( __dmul_rn( a2, u0 ), __dmul_rn( a0, u2 ) );
        t2 = __dsub_rn( __dmul_rn( a0, u1 ), __dmul_rn( a1, u0 ) );
        tm2 = __dadd_rn( __dadd_rn( __dmul_rn( t0, t0 ), __dmul_rn( t1, t1 ) ), __dmul_rn( t2, t2 ) );
        if ( !( tm2 < 0.001 ) )
          break;
      }
    }
    if ( it == 100000 )
      return NCGB_ST_LOOPCAP;
    const double f = sqrt( __ddiv_rn( __dsub_rn( 1.0, __dmul_rn( mu, mu ) ), tm2 ) );
    out[0] = __dadd_rn( __dmul_rn( u0, mu ), __dmul_rn( t0, f ) );
    out[1] = __dadd_rn( __dmul_rn( u1, mu ), __dmul_rn( t1, f ) );
    out[2] = __dadd_rn( __dmul_rn( u2, mu ), __dmul_rn( t2, f ) );
    return NCGB_ST_OK;
  }

  // convertAlphaBetaToDeltaEMu, NCKinUtils.cc:25-58.  Returns
  // NCGB_ST_CALCERROR where the reference throws (E*E' == 0).
  __device__ __forceinline__ int alphaBetaToDeltaEMu( double alpha, double beta, double ekin, double kT,
                                                      double& deltaE, double& mu )
  {
    deltaE = beta * kT;
    const double ekinfinal = ekin + deltaE;
    const double denom = 2.0 * sqrt( ekin * ekinfinal );
    if ( !denom )
      return NCGB_ST_CALCERROR;
    double s = 0.0, c = 0.0;
    neumaierAdd( s, c, ekin );
    neumaierAdd( s, c, ekinfinal );
    neumaierAdd( s, c, -alpha * kT );
    mu = clampd( ( s + c ) / denom, -1.0, 1.0 );
    return NCGB_ST_OK;
  }

  // ---- cross-sections ---------------------------------------------------------

  // NCElIncXS.cc:34-54.  Fast (mixed-precision mode): the expm1 branch in
  // FP32 (relative error ~1e-7).
  template<bool Fast>
  __device__ __forceinline__ double oneMinusExpMtDivT( double t )
  {
    if ( t < 0.01 )
      return ( 1 + t * ( -0.5 + t * 0.16666666666666666666666666666666666666666667 * ( 1. - 0.25 * t ) ) );
    if ( t > 24.0 )
      return 1.0 / t;
    if ( Fast ) {
      const float tf = (float)( -t );
      return (double)( expm1f( tf ) / tf );
    }
    t = -t;
    return expm1( t ) / t;
  }

  constexpr double kElIncXS = 16.0 * 9.86960440108935861883449099987615113531369941 * 12.22430978582345950656;
  constexpr double kElIncMu = 8.0 * 9.86960440108935861883449099987615113531369941 * 12.22430978582345950656;

  // ---- FP32 cross-sections of the mixed-precision mode ---------------------------
  // Same formulas as the FP64 ones below, in FP32 (relative error ~1e-7).
  __device__ __forceinline__ float oneMinusExpMtDivTf( float t )
  {
    if ( t < 0.01f )
      return 1.0f + t * ( -0.5f + t * 0.16666667f * ( 1.0f - 0.25f * t ) );
    if ( t > 24.0f )
      return 1.0f / t;
    return expm1f( -t ) / ( -t );
  }

  __device__ __forceinline__ float elincXSf( const ncgb_elinc_view& v, float ekin )
  {
    const float e = (float)kElIncXS * ekin;
    float xs = 0.0f;
    for ( int i = 0; i < v.n && i < NCGB_MAX_ELINC; ++i )
      xs = fmaf( v.sigma_f[i], oneMinusExpMtDivTf( v.msd_f[i] * e ), xs );
    return xs;
  }

  // first i in [0, n) with a[i] > x, for non-negative floats (int compares)
  __device__ __forceinline__ int upper_bound_f( const float* a, int n, float x )
  {
    const int key = __float_as_int( x );
    int lo = 0, len = n;
    while ( len > 0 ) {
      const int half = len >> 1;
      if ( __float_as_int( __ldg( a + lo + half ) ) <= key ) {
        lo += half + 1;
        len -= half + 1;
      } else {
        len = half;
      }
    }
    return lo;
  }

  // ElIncXS::evaluate (NCElIncXS.cc:117-128)
  template<bool Fast>
  __device__ __forceinline__ double elincXS( const ncgb_elinc_view& v, double ekin )
  {
    const double e = kElIncXS * ekin;
    double xs = 0.0;
    for ( int i = 0; i < v.n && i < NCGB_MAX_ELINC; ++i )
      xs += v.sigma[i] * oneMinusExpMtDivT<Fast>( v.msd[i] * e );
    return xs;
  }

  // AbsOOV::crossSectionIsotropic, NCAbsOOV.cc:40-44: c/sqrt(E), infinite at
  // E = 0 (NaN for E < 0, as in the reference).
  __device__ __forceinline__ double absXS( double c, double ekin )
  {
    const double se = sqrt( ekin );
    return se != 0.0 ? c / se : infd();
  }

  // PowderBragg, NCPowderBragg.cc:152-176.  idx_out: last valid plane.
  __device__ __forceinline__ double braggXS( const ncgb_bragg_view& v, double ekin, int64_t& idx_out )
  {
    idx_out = 0;
    if ( v.n == 0 || ekin < v.threshold || !finited(ekin) )
      return 0.0;
    const int64_t idx = upper_bound_nn( v.two_dE + 1, v.n - 1, ekin );
    idx_out = idx;
    return ldg( v.fdm_commul + idx ) * ( 1.0 / ekin );
  }

  // FreeGasXSProvider::evalXSShapeASq, NCFreeGasUtils.cc:64-84
  __device__ __forceinline__ double freeGasShape( double a_squared )
  {
    if ( a_squared > 36.0 )
      return 1.0 + 0.5 / a_squared;
    const double a = sqrt( a_squared );
    if ( a < 0.1 ) {
      if ( a == 0.0 )
        return infd();
      const double a2 = a_squared;
      return 0.564189583547756286948079451560772585844050629
        * ( 2.0 / a + a *( (2.0/3.0)- a2*((1.0/15.0)-a2*((1.0/105.0)-a2*((1.0/756.0)-a2*(1.0/5940.0))))));
    }
    const double inva = 1.0 / a;
    return ( 1.0 + 0.5*inva*inva ) * erf( a ) + 0.564189583547756286948079451560772585844050629 * exp( -a_squared ) * inva;
  }

  // std::upper_bound over the energy grid for E >= 0 (or NaN): the bucket of
  // E's bit pattern narrows the range to a few entries (same result).
  __device__ __forceinline__ int64_t egridUpper( const ncgb_sab_view& s, double e )
  {
    const long long eb = bits( e );
    const long long k = ( eb >> 49 ) - s.ebkt_kmin;
    if ( k < 0 )
      return 0;
    if ( k >= s.ebkt_n )
      return s.ne;
    int64_t i = __ldg( s.ebkt + k );
    const int64_t hi = __ldg( s.ebkt + k + 1 );
    while ( i < hi && !( eb < ldgbits( s.egrid + i ) ) )
      ++i;
    return i;
  }

  __device__ __forceinline__ int egridUpperF( const ncgb_sab_view& s, float e )
  {
    const int eb = __float_as_int( e );
    const int k = ( eb >> 20 ) - s.ebkt_f_kmin;
    if ( k < 0 )
      return 0;
    if ( k >= s.ebkt_f_n )
      return s.ne;
    int i = __ldg( s.ebkt_f + k );
    const int hi = __ldg( s.ebkt_f + k + 1 );
    while ( i < hi && !( eb < __float_as_int( __ldg( s.egrid_f + i ) ) ) )
      ++i;
    return i;
  }

  // SABXSProvider::crossSection (NCSABXSProvider.cc:54-95) x SABScatter scale
  // (NCSABScatter.cc:87-90).  Requires ekin >= 0 and not NaN.
  __device__ __forceinline__ double sabXS( const ncgb_sab_view& s, double ekin )
  {
    const int64_t ne = s.ne;
    const int64_t iu = egridUpper( s, ekin );
    double xs;
    if ( iu == ne ) {
      xs = s.kext / ekin + s.ext_sigma_free * freeGasShape( s.ext_ca * ekin );
    } else if ( iu == 0 ) {
      xs = ekin > 0.0 ? sqrt( ldg(s.egrid) / ekin ) * ldg(s.xs) : infd();
    } else {
      const double el = ldg( s.egrid + iu - 1 );
      const double xl = ldg( s.xs + iu - 1 ), xu = ldg( s.xs + iu );
      xs = xl + ( xu - xl ) * ( ( ekin - el ) * ldg( s.inv_dE + iu - 1 ) );
    }
    return xs * s.internal_scale;
  }

  // SAB cross-section in FP32 below Emax (FP64 above: the extender).
  __device__ __forceinline__ float sabXSf( const ncgb_sab_view& s, double ekin, float ef )
  {
    const int ne = s.ne;
    const int iu = egridUpperF( s, ef );
    if ( iu == ne )
      return (float)sabXS( s, ekin );
    float xs;
    if ( iu == 0 ) {
      xs = ef > 0.0f ? sqrtf( __ldg( s.egrid_f ) / ef ) * __ldg( s.xsf ) : __int_as_float( 0x7f800000 );
    } else {
      const float2 p = __ldg( reinterpret_cast<const float2*>( s.xsf ) + ( iu - 1 ) );
      xs = fmaf( p.y, ef - __ldg( s.egrid_f + iu - 1 ), p.x );
    }
    return xs * s.internal_scale_f;
  }

  // Lean: a material whose components are S(alpha,beta) and incoherent
  // elastic only (the caller checks), compiled without the other types' code.
  template<bool Lean = false>
  __device__ __forceinline__ float compXSf( const ncgb_comp_view& c, double ekin, float ef )
  {
    if ( !containsNN( c.elow, c.ehigh, ekin ) )
      return 0.0f;
    if constexpr ( Lean )
      return c.type == NCGB_COMP_SAB ? sabXSf( c.sab, ekin, ef ) : elincXSf( c.elinc, ef );
    int64_t idx;
    switch ( c.type ) {
      case NCGB_COMP_ELINC: return elincXSf( c.elinc, ef );
      case NCGB_COMP_BRAGG: {
        if ( c.bragg.n == 0 || ekin < c.bragg.threshold )
          return 0.0f;
        idx = upper_bound_nn( c.bragg.two_dE + 1, c.bragg.n - 1, ekin );
        return (float)ldg( c.bragg.fdm_commul + idx ) / ef;
      }
      case NCGB_COMP_SAB: return sabXSf( c.sab, ekin, ef );
      case NCGB_COMP_FREEGAS: return (float)( c.fg.sigma_free * freeGasShape( c.fg.ca * ekin ) );
      default: return 0.0f;
    }
  }

  template<bool Fast>
  __device__ __forceinline__ double compXS( const ncgb_comp_view& c, double ekin )
  {
    if ( !containsNN( c.elow, c.ehigh, ekin ) )
      return 0.0;
    int64_t dummy;
    switch ( c.type ) {
      case NCGB_COMP_ELINC: return elincXS<Fast>( c.elinc, ekin );
      case NCGB_COMP_BRAGG: return braggXS( c.bragg, ekin, dummy );
      case NCGB_COMP_SAB: return sabXS( c.sab, ekin );
      case NCGB_COMP_FREEGAS: return c.fg.sigma_free * freeGasShape( c.fg.ca * ekin );
      default: return 0.0;
    }
  }

  // ProcComposition::updateCacheIsotropic (NCProcImpl.cc:166-204) and
  // pickRandIdxByWeight (NCRandUtils.hh:130-133, NCRandUtils.cc:198-222),
  // with the cumulative cross-sections in registers (fully unrolled).
  struct XSPick { double xs; int comp; };

  // Mixed-precision mode: the same with FP32 cumulative sums (the Bragg plane
  // search and the FP64 Bragg sums themselves are unchanged).
  template<bool Pick, bool Lean = false>
  __device__ __forceinline__ XSPick xsAndPickF( const ncgb_material_view& m, double ekin, ncgb_rng& rng )
  {
    const float ef = (float)ekin;
    float commul[NCGB_MAX_COMP];
    float tot = 0.0f;
    // a rolled loop: unrolled, every copy carried the whole switch over the
    // component types, and the pick pass stalled on instruction fetch
#pragma unroll 1
    for ( int i = 0; i < NCGB_MAX_COMP; ++i ) {
      if ( i >= m.ncomp )
        break;
      tot = fmaf( m.comp[i].scale_f, compXSf<Lean>( m.comp[i], ekin, ef ), tot );
      commul[i] = tot;
    }
    XSPick r{ (double)tot, 0 };
    if ( !Pick || m.ncomp <= 1 )
      return r;
    const float choice = tot * (float)rand01( rng );
    const int n = m.ncomp;
    int pick = n - 1;
    if ( n < 5 ) {
#pragma unroll
      for ( int i = NCGB_MAX_COMP - 1; i >= 0; --i )
        if ( i < n && commul[i] > choice )
          pick = i;
    } else {
#pragma unroll
      for ( int i = NCGB_MAX_COMP - 1; i >= 0; --i )
        if ( i < n && commul[i] >= choice )
          pick = i;
    }
    r.comp = pick;
    return r;
  }

  template<bool Pick, bool Fast, bool Lean = false>
  __device__ __forceinline__ XSPick xsAndPick( const ncgb_material_view& m, double ekin, ncgb_rng& rng )
  {
    if ( Fast )
      return xsAndPickF<Pick, Lean>( m, ekin, rng );
    double commul[NCGB_MAX_COMP];
    double tot = 0.0;
#pragma unroll 1
    for ( int i = 0; i < NCGB_MAX_COMP; ++i ) {
      if ( i >= m.ncomp )
        break;
      tot += m.comp[i].scale * compXS<Fast>( m.comp[i], ekin );
      commul[i] = tot;
    }
    XSPick r{ tot, 0 };
    if ( !Pick || m.ncomp <= 1 )
      return r;
    const double choice = tot * rand01( rng );
    const int n = m.ncomp;
    int pick = n - 1;
    if ( n < 5 ) {
      // linear search: first commul > choice
#pragma unroll
      for ( int i = NCGB_MAX_COMP - 1; i >= 0; --i )
        if ( i < n && commul[i] > choice )
          pick = i;
    } else {
      // lower_bound: first commul >= choice, capped at n-1
#pragma unroll
      for ( int i = NCGB_MAX_COMP - 1; i >= 0; --i )
        if ( i < n && commul[i] >= choice )
          pick = i;
    }
    r.comp = pick;
    return r;
  }

  // ---- non-SAB samplers -----------------------------------------------------------

  // PowderBragg::genScatterMu, NCPowderBragg.cc:178-200
  __device__ __forceinline__ double braggMu( const ncgb_bragg_view& v, ncgb_rng& rng, double ekin, int64_t idx )
  {
    const double r = rand01( rng );
    const int64_t k = lower_bound_nn( v.fdm_commul, idx, r * ldg( v.fdm_commul + idx ) );
    return 1.0 - 2.0 * ( ldg( v.two_dE + k ) / ekin );
  }

  // exp_smallarg_approx, NCMath.hh:434-440
  __device__ __forceinline__ double expSmall( double x )
  {
    return 1.0+x*(1+x*(0.5+x*(0.16666666666666666666666666666666666667+x*(0.04166666666666666666666666666666666667
             +x*(0.00833333333333333333333333333333333333+x*(0.00138888888888888888888888888888888889
             +x*0.00019841269841269841269841269841269841))))));
  }

  // ElIncXS::sampleMuMonoAtomic, NCElIncXS.cc:81-115.  The reference's
  // rejection loop is unbounded; its acceptance is above 98% here, and the
  // cap only guards the GPU.
  // FP32 version of elincMuMono (mixed-precision mode).
  static __device__ __noinline__ float elincMuMonoF( ncgb_rng& rng, float ekin, float msd, int& status )
  {
    const float a = ( (float)kElIncMu * ekin ) * msd;
    if ( a < 0.01f ) {
      const float maxval = 1.0f + a * ( 1.0f + a * ( 0.5f + a * ( 0.16666667f + a * 0.041666668f ) ) );
      for ( int it = 0; it < 100000; ++it ) {
        const float mu = (float)rand01( rng ) * 2.0f - 1.0f;
        const float x = a * mu;
        if ( (float)rand01( rng ) * maxval < 1.0f + x * ( 1.0f + x * ( 0.5f + x * ( 0.16666667f + x * 0.041666668f ) ) ) )
          return mu;
      }
      status = NCGB_ST_LOOPCAP;
      return 1.0f;
    }
    // for a > 20, log1p(R*expm1(2a))/a - 1 = 1 + log(R)/a to within exp(-40),
    // which also avoids FP32 overflow of expm1(2a)
    const float r = (float)rand01( rng );
    const float m = a > 20.0f ? 1.0f + logf( r ) / a : log1pf( r * expm1f( 2.0f * a ) ) / a - 1.0f;
    return fminf( 1.0f, fmaxf( -1.0f, m ) );
  }

  template<bool Fast>
  __device__ __noinline__ double elincMuMono( ncgb_rng& rng, double ekin, double msd, int& status )
  {
    const double a = ( kElIncMu * ekin ) * msd;
    if ( a < 0.01 ) {
      const double maxval = expSmall( a );
      for ( int it = 0; it < 100000; ++it ) {
        const double mu = rand01( rng ) * 2.0 - 1.0;
        if ( rand01( rng ) * maxval < expSmall( a * mu ) )
          return mu;
      }
      status = NCGB_ST_LOOPCAP;
      return 1.0;
    }
    if ( Fast ) {
      // FP32; for a > 20, log1p(R*expm1(2a))/a - 1 = 1 + log(R)/a to within
      // exp(-40), which also avoids FP32 overflow of expm1(2a).
      const float r = (float)rand01( rng );
      const float af = (float)a;
      const float m = a > 20.0 ? 1.0f + logf( r ) / af : log1pf( r * expm1f( 2.0f * af ) ) / af - 1.0f;
      return clampd( (double)m, -1.0, 1.0 );
    }
    return clampd( log1p( rand01( rng ) * expm1( 2.0 * a ) ) / a - 1.0, -1.0, 1.0 );
  }

  // ElIncXS::EPointAnalysis::sampleMu, NCElIncXS.cc:178-191 (element picked
  // by pickRandIdxByWeight on the cumulative contributions).
  // FP32 version of elincMu (mixed-precision mode).
  static __device__ __noinline__ double elincMuF( const ncgb_elinc_view& v, ncgb_rng& rng, double ekin, int& status )
  {
    const float ef = (float)ekin;
    if ( v.n == 1 )
      return (double)elincMuMonoF( rng, ef, v.msd_f[0], status );
    const float e = (float)kElIncXS * ef;
    float tot = 0.0f;
    for ( int i = 0; i < v.n && i < NCGB_MAX_ELINC; ++i )
      tot = fmaf( v.sigma_f[i], oneMinusExpMtDivTf( v.msd_f[i] * e ), tot );
    const float choice = tot * (float)rand01( rng );
    int pick = v.n - 1;
    float c = 0.0f;
    const bool linear = v.n < 5;
    for ( int i = 0; i < v.n && i < NCGB_MAX_ELINC; ++i ) {
      c = fmaf( v.sigma_f[i], oneMinusExpMtDivTf( v.msd_f[i] * e ), c );
      if ( linear ? ( c > choice ) : ( c >= choice ) ) { pick = i; break; }
    }
    return (double)elincMuMonoF( rng, ef, v.msd_f[pick], status );
  }

  template<bool Fast>
  __device__ __noinline__ double elincMu( const ncgb_elinc_view& v, ncgb_rng& rng, double ekin, int& status )
  {
    if ( Fast )
      return elincMuF( v, rng, ekin, status );
    if ( v.n == 1 )
      return elincMuMono<Fast>( rng, ekin, v.msd[0], status );
    const double e = kElIncXS * ekin;
    double tot = 0.0;
    for ( int i = 0; i < v.n && i < NCGB_MAX_ELINC; ++i )
      tot += v.sigma[i] * oneMinusExpMtDivT<Fast>( v.msd[i] * e );
    const double choice = tot * rand01( rng );
    int pick = v.n - 1;
    double c = 0.0;
    const bool linear = v.n < 5;
    for ( int i = 0; i < v.n && i < NCGB_MAX_ELINC; ++i ) {
      c += v.sigma[i] * oneMinusExpMtDivT<Fast>( v.msd[i] * e );
      if ( linear ? ( c > choice ) : ( c >= choice ) ) { pick = i; break; }
    }
    return elincMuMono<Fast>( rng, ekin, v.msd[pick], status );
  }

  // ---- phase clocks of the S(alpha,beta) pass -----------------------------------------
  // A measurement instrument: the phase-profiling kernel passes a PhaseClock
  // through the sampler, every other caller a NoPhases, whose marks compile
  // to nothing.  end<P>() charges the SM clock cycles since the previous mark
  // to phase P (per lane: a lane's cycles in a divergent region include the
  // time its warp spends on the other lanes' paths, so the per-phase sums are
  // shares of the lanes' wall time).
  enum { PH_CLAIM = 0, PH_BETA, PH_ALPHA, PH_ACCEPT, PH_CONVERT, PH_IDLE, PH_N };
  static_assert( PH_N == NCGB_SAB_NPHASES, "phase count of the C ABI" );
  struct NoPhases {
    template<int P> __device__ __forceinline__ void end() {}
    __device__ __forceinline__ void attempt() {}
  };
  struct PhaseClock {
    uint32_t t, attempts;
    uint32_t acc[PH_N];
    __device__ __forceinline__ void start()
    {
      for ( int i = 0; i < PH_N; ++i )
        acc[i] = 0;
      attempts = 0;
      t = (uint32_t)clock();
    }
    template<int P> __device__ __forceinline__ void end()
    {
      const uint32_t n = (uint32_t)clock();
      acc[P] += n - t;
      t = n;
    }
    __device__ __forceinline__ void attempt() { ++attempts; }
  };

  // ---- S(alpha,beta) sampling (Alg.1) -----------------------------------------------

  // PointwiseDist::percentileWithIndex, NCPointwiseDist.cc:76-110, with the
  // in-bin constants read from the sampler's ncgb_beta_bin table instead of
  // divided out (same formulas, a few ulps apart).
  __device__ __forceinline__ double percentile( const double* x, const double* cdf, const ncgb_beta_bin* bins,
                                                int n, double p, int& bin )
  {
    if ( p == 1.0 ) { bin = n - 2; return ldg( x + n - 1 ); }
    int i = lower_bound_nn32( cdf, n, p );
    if ( i > n - 1 ) i = n - 1;
    if ( i < 1 ) i = 1;
    const ncgb_beta_bin* bb = bins + ( i - 1 );
    const double x0 = ldg( &bb->x0 ), x1 = ldg( &bb->x1 );
    const double c = p - ldg( &bb->cdf0 );
    const double a = ldg( &bb->a );
    const double k_e = ldg( &bb->k_e );
    double zdx;
    if ( !a ) {
      zdx = k_e > 0.0 ? sqrt( c * k_e ) : 0.5 * ( x1 - x0 );
    } else {
      const double e = c * k_e;
      if ( fabs(e) > 1e-7 )
        zdx = ( sqrt( 1.0 + 2.0 * e ) - 1.0 ) * ldg( &bb->k_z );
      else
        zdx = ( 1 + 0.5 * e * ( e - 1.0 ) ) * c * ldg( &bb->inv_a );
    }
    bin = i - 1;
    return clampd( x0 + zdx, x0, x1 );
  }

  // SABUtils::sampleLogLinDist_fast, NCSABUtils.hh:282-304.  The reference's
  // a_sub_b*log(fa*exp(a*L/a_sub_b)/(fa+r*df))/L, with L = logfb-logfa, is
  // evaluated as a + (b-a)*log1p(r*df/fa)/L: the same value algebraically,
  // one transcendental instead of two, and no cancellation at small r.
  // log1p, in FP32 in the mixed-precision mode (arguments above 1e30 stay FP64).
  template<bool Fast>
  __device__ __forceinline__ double log1pMode( double q )
  {
    if ( Fast && q < 1e30 )
      return (double)log1pf( (float)q );
    return log1p( q );
  }

  template<bool Fast>
  __device__ __forceinline__ double logLin( double a, double fa, double b, double fb, double rnd, double logfa, double logfb )
  {
    double df = fb - fa;
    if ( fa * fb * df != 0.0 ) {
      const double L = logfb - logfa;
      if ( ( a - b ) * L != 0.0 )
        return a + ( b - a ) * ( log1pMode<Fast>( rnd * df / fa ) / L );
      df = 0.0;
    }
    if ( !df )
      return a + rnd * ( b - a );
    const double xx = ( b - a ) * sqrt( rnd );
    return ( fa ? b - xx : a + xx );
  }

  __device__ __forceinline__ double clampRand( double r ) { return clampd( r, 2.2250738585072014e-308, 1.0 ); }

  // SABSamplerAtE_Alg1::sampleAlpha, NCSABSamplerModels.cc:157-234.  The
  // divisions by the section probabilities and bin areas are multiplications
  // by tabulated reciprocals, and the middle part's log-linear in-cell
  // inversion uses the cell's tabulated ratio and slope.
  template<bool Fast>
  __device__ __forceinline__ double sampleAlpha( const ncgb_sab_view& s, const ncgb_alpha_info* infos,
                                                 int ioff, int ibeta, double rp )
  {
    const ncgb_alpha_info* info = infos + ( ibeta - ioff );
    const double prob_front = ldg( &info->prob_front );
    const int na = s.na;
    const double* cumul = s.cumul + ibeta * na;
    const double* sab = s.sab + ibeta * na;
    const double* logsab = s.logsab + ibeta * na;
    if ( rp <= prob_front ) {
      const double fa = ldg( &info->front_alpha );
      if ( prob_front == 2.0 ) {
        const double da = ldg( &info->back_alpha ) - fa;
        return fa + rp * da;
      } else if ( prob_front == 1.0 ) {
        return logLin<Fast>( fa, ldg( &info->front_sval ), ldg( &info->back_alpha ), ldg( &info->back_sval ),
                       rp, ldg( &info->front_logsval ), ldg( &info->back_logsval ) );
      } else {
        const uint32_t fi = __ldg( &info->front_idx );
        const double p2 = clampRand( rp * ldg( &info->inv_front ) );
        return logLin<Fast>( fa, ldg( &info->front_sval ), ldg( s.alpha + fi ), ldg( sab + fi ),
                       p2, ldg( &info->front_logsval ), ldg( logsab + fi ) );
      }
    }
    const double prob_notback = ldg( &info->prob_notback );
    if ( rp <= prob_notback ) {
      const double p2 = clampd( ( rp - prob_front ) * ldg( &info->inv_middle ), 0.0, 1.0 );
      const int il = __ldg( &info->front_idx ), iu = __ldg( &info->back_idx );
      const double cl = ldg( cumul + il ), cu = ldg( cumul + iu );
      const double sel = cl + p2 * ( cu - cl );
      const int e = il + upper_bound_nn32( cumul + il, iu + 1 - il, sel );
      if ( e > iu )
        return ldg( s.alpha + iu );
      if ( e <= il )
        return ldg( s.alpha + il );
      const int a0 = e - 1;
      const ncgb_alpha_cell* cell = s.acell + ibeta * na + a0;
      const double rr = clampRand( ( sel - ldg( cumul + a0 ) ) * ldg( &cell->inv_bin ) );
      const double slope = ldg( &cell->slope );
      if ( slope == slope )
        return ldg( s.alpha + a0 ) + slope * log1pMode<Fast>( rr * ldg( &cell->ratio ) );
      return logLin<Fast>( ldg( s.alpha + a0 ), ldg( sab + a0 ), ldg( s.alpha + a0 + 1 ), ldg( sab + a0 + 1 ),
                     rr, ldg( logsab + a0 ), ldg( logsab + a0 + 1 ) );
    }
    const uint32_t bi = __ldg( &info->back_idx );
    const double p2 = clampRand( ( rp - prob_notback ) * ldg( &info->inv_back ) );
    return logLin<Fast>( ldg( s.alpha + bi ), ldg( sab + bi ), ldg( &info->back_alpha ), ldg( &info->back_sval ),
                   p2, ldg( logsab + bi ), ldg( &info->back_logsval ) );
  }

  // ---- FP32 alpha sampling of the mixed-precision mode -----------------------
  // sampleLogLinDist_fast and SABSamplerAtE_Alg1::sampleAlpha as above, on the
  // FP32 table copies.  The degenerate-branch tests compare the factors with
  // zero one by one (a product of small FP32 values could underflow).
  __device__ __forceinline__ float logLinF( float a, float fa, float b, float fb, float rnd, float logfa, float logfb )
  {
    float df = fb - fa;
    if ( fa != 0.0f && fb != 0.0f && df != 0.0f ) {
      const float L = logfb - logfa;
      if ( a != b && L != 0.0f )
        return a + ( b - a ) * ( log1pf( rnd * df / fa ) / L );
      df = 0.0f;
    }
    if ( df == 0.0f )
      return a + rnd * ( b - a );
    const float xx = ( b - a ) * sqrtf( rnd );
    return ( fa != 0.0f ) ? b - xx : a + xx;
  }

  __device__ __forceinline__ float clampRandF( float r ) { return fminf( 1.0f, fmaxf( 1.17549435e-38f, r ) ); }

  __device__ __forceinline__ float sampleAlphaF( const ncgb_sab_view& s, const ncgb_alpha_info_f* infos,
                                                 int ioff, int ibeta, float rp )
  {
    const ncgb_alpha_info_f* info = infos + ( ibeta - ioff );
    const float prob_front = __ldg( &info->prob_front );
    const int na = s.na;
    const float* cumul = s.cumul_f + ibeta * na;
    const float* sab = s.sab_f + ibeta * na;
    const float* logsab = s.logsab_f + ibeta * na;
    if ( rp <= prob_front ) {
      const float fa = __ldg( &info->front_alpha );
      if ( prob_front == 2.0f )
        return fa + rp * ( __ldg( &info->back_alpha ) - fa );
      if ( prob_front == 1.0f )
        return logLinF( fa, __ldg( &info->front_sval ), __ldg( &info->back_alpha ), __ldg( &info->back_sval ),
                        rp, __ldg( &info->front_logsval ), __ldg( &info->back_logsval ) );
      const uint32_t fi = __ldg( &info->front_idx );
      const float p2 = clampRandF( rp * __ldg( &info->inv_front ) );
      return logLinF( fa, __ldg( &info->front_sval ), __ldg( s.alpha_f + fi ), __ldg( sab + fi ),
                      p2, __ldg( &info->front_logsval ), __ldg( logsab + fi ) );
    }
    const float prob_notback = __ldg( &info->prob_notback );
    if ( rp <= prob_notback ) {
      const float p2 = fminf( 1.0f, fmaxf( 0.0f, ( rp - prob_front ) * __ldg( &info->inv_middle ) ) );
      const int il = __ldg( &info->front_idx ), iu = __ldg( &info->back_idx );
      const float cl = __ldg( cumul + il ), cu = __ldg( cumul + iu );
      const float sel = fmaf( p2, cu - cl, cl );
      const int e = il + upper_bound_f( cumul + il, iu + 1 - il, sel );
      if ( e > iu )
        return __ldg( s.alpha_f + iu );
      if ( e <= il )
        return __ldg( s.alpha_f + il );
      const int a0 = e - 1;
      const float4 cell = __ldg( reinterpret_cast<const float4*>( s.acell_f ) + ( ibeta * na + a0 ) );
      const float rr = clampRandF( ( sel - __ldg( cumul + a0 ) ) * cell.x );
      if ( cell.z == cell.z )
        return fmaf( cell.z, log1pf( rr * cell.y ), __ldg( s.alpha_f + a0 ) );
      return logLinF( __ldg( s.alpha_f + a0 ), __ldg( sab + a0 ), __ldg( s.alpha_f + a0 + 1 ), __ldg( sab + a0 + 1 ),
                      rr, __ldg( logsab + a0 ), __ldg( logsab + a0 + 1 ) );
    }
    const uint32_t bi = __ldg( &info->back_idx );
    const float p2 = clampRandF( ( rp - prob_notback ) * __ldg( &info->inv_back ) );
    return logLinF( __ldg( s.alpha_f + bi ), __ldg( sab + bi ), __ldg( &info->back_alpha ), __ldg( &info->back_sval ),
                    p2, __ldg( logsab + bi ), __ldg( &info->back_logsval ) );
  }

  // alpha of row 'ibeta' at percentile rp, in the arithmetic of the mode
  template<bool Fast>
  __device__ __forceinline__ double rowAlpha( const ncgb_sab_view& s, int off, int ioff, int ibeta,
                                             double rp )
  {
    if ( Fast )
      return (double)sampleAlphaF( s, s.info_f + off, ioff, ibeta, (float)rp );
    return sampleAlpha<Fast>( s, s.info + off, ioff, ibeta, rp );
  }

  // First beta bin with a kinematic endpoint (NCSABSamplerModels.cc:69-116):
  // beta uniform in the bin, alpha from the first row, up to 30 tries.
  // Returns 1 if (alpha, beta) is accepted, 0 if the attempt is rejected.
  template<bool Fast>
  __device__ __forceinline__ int alg1FirstBin( const ncgb_sab_view& s, int off, int ioff,
                                               double fbkep, double b1, double x, ncgb_rng& rng,
                                               double& alpha_out, double& beta_out )
  {
    const double b0 = fbkep;
    if ( b1 < -x )
      return 0;
    const double delta_beta = b1 - b0;
    double alphaval = 0.0;
    double beta = b0;
    for ( int iii = 0; iii < 30; ++iii ) {
      beta = maxd( fbkep, b0 + delta_beta * rand01( rng ) );
      if ( beta < -x )
        break;
      alphaval = rowAlpha<Fast>( s, off, ioff, ioff, rand01( rng ) );
      const ALim al = alphaLimits( -fbkep, beta );
      if ( inInterval( al.lo, al.hi, alphaval ) )
        break;
      if ( iii == 29 ) {
        alphaval = 0.5 * ( al.lo + al.hi );
        break;
      }
    }
    if ( beta < -x )
      return 0;
    const ALim al2 = alphaLimits( x, beta );
    if ( inInterval( al2.lo, al2.hi, alphaval ) ) {
      alpha_out = alphaval;
      beta_out = beta;
      return 1;
    }
    return 0;
  }

  // The same, out of line: for passes that keep the free-gas paths' calls
  // anyway (a call more costs them nothing; inlined, it costs the lean
  // pass's registers nothing either: measured k_sab 1.25 -> 1.20 ms on
  // polyethylene once no other call was left in its loop).
  template<bool Fast>
  __device__ __noinline__ int alg1FirstBinCall( const ncgb_sab_view& s, int off, int ioff,
                                                double fbkep, double b1, double x, ncgb_rng& rng,
                                                double& alpha_out, double& beta_out )
  {
    return alg1FirstBin<Fast>( s, off, ioff, fbkep, b1, x, rng, alpha_out, beta_out );
  }

  // One attempt of SABSamplerAtE_Alg1::sampleAlphaBeta's loop
  // (NCSABSamplerModels.cc:59-148) at energy-grid point ie, sampling energy
  // x = E/kT.  Returns 1 with (alpha, beta) on acceptance, 0 on rejection.
  // Learned proposal for the regular beta range of sampler ie (tables built by
  // ncgb_proposal.cc): an interval from the alias table, a 32-bit draw w
  // placing beta = q + (2w+1) h in it, accepted with probability y/env, y from
  // the interval's linear pieces in w.  A proposal uses integer and FP32
  // arithmetic only; beta is formed in FP64 once accepted, after the lanes
  // that entered together have reconverged (so that the FP64 work after this
  // call is not split across lanes accepting at different tries).  Returns 1
  // with (beta, ibs), or 0 if 1000 proposals were all rejected.
  __device__ __forceinline__ int lpBeta( const ncgb_sab_view& s, int ie, ncgb_rng& rng, double& beta,
                                         int& ibs )
  {
    const unsigned lanes = __activemask();
    const ncgb_lp_slot* slots = s.lp_slot + ie * NCGB_LP_K;
    const ncgb_lp_cell* cells = s.lp_cell + ie * NCGB_LP_K;
    const ncgb_lp_cell* c = cells;
    const ncgb_lp_seg* g = s.lp_seg;
    uint32_t w = 0;
    int ok = 0;
    for ( int tries = 0; tries < 1000 && !ok; ++tries ) {
      // a try's three words, drawn in order by one copy of the stream's code
      uint32_t d0 = 0, d1 = 0, d2 = 0;
#pragma unroll 1
      for ( int q = 0; q < 3; ++q ) {
        const uint32_t v = rand_u32( rng );
        if ( q == 0 ) d0 = v; else if ( q == 1 ) d1 = v; else d2 = v;
      }
      const uint64_t prod = (uint64_t)d0 * (uint64_t)NCGB_LP_K;
      const int j = (int)( prod >> 32 );
      const float fr = (float)( (uint32_t)prod >> 8 ) * ( 1.0f / 16777216.0f );
      const int k = ( fr < __ldg( &slots[j].aprob ) ) ? j : __ldg( &slots[j].alias );
      c = cells + k;
      w = d1;
      // last piece with w0 <= w
      int lo = __ldg( &c->seg_lo ), hi = lo + __ldg( &c->seg_n ) - 1;
      while ( lo < hi ) {
        const int mid = ( lo + hi + 1 ) >> 1;
        if ( __ldg( &s.lp_seg[mid].w0 ) <= w )
          lo = mid;
        else
          hi = mid - 1;
      }
      g = s.lp_seg + lo;
      const float y = fmaf( __ldg( &g->slope ), (float)( w - __ldg( &g->w0 ) ), __ldg( &g->y0 ) );
      const float ua = (float)( d2 >> 8 ) * ( 1.0f / 16777216.0f );
      ok = ( ua * __ldg( &c->env ) < y );
    }
    __syncwarp( lanes );
    if ( ok ) {
      beta = fma( (double)( 2ull * w + 1ull ), ldg( &c->h ), ldg( &c->q ) );
      ibs = __ldg( &g->bin );
    }
    return ok;
  }

  // One attempt of SABSamplerAtE_Alg1::sampleAlphaBeta.  Returns 1 with
  // (alpha, beta) accepted, 0 if the attempt is rejected, -1 if the learned
  // proposal hit its cap.  Learned: the beta percentile inversion of samplers
  // with an enabled learned proposal is replaced by lpBeta (same distribution).
  template<bool Fast, bool Learned, bool Full, class Ph>
  __device__ __forceinline__ int alg1Attempt( const ncgb_sab_view& s, int ie, double x, ncgb_rng& rng,
                                              double& alpha_out, double& beta_out, Ph& ph )
  {
    ph.attempt();
    const int off = (int)__ldg( s.smp_offset + ie );
    const int nbs = __ldg( s.smp_nbeta + ie );
    const double* bx = s.bx + off;
    const ncgb_alpha_info* infos = s.info + off;
    const int ioff = __ldg( s.smp_ibetaoffset + ie );
    int ibs;
    double beta;
    const double fbkep = ldg( s.smp_fbkep + ie );
    bool firstBin;
    if ( Learned && s.lp_hdr && __ldg( &s.lp_hdr[ie].enabled ) ) {
      // the special first bin keeps its probability bcdf[1]; the regular
      // range is drawn from the learned proposal
      firstBin = rand_u32( rng ) < __ldg( &s.lp_hdr[ie].c1_thr );
      if ( !firstBin && !lpBeta( s, ie, rng, beta, ibs ) )
        return -1;
    } else {
      beta = percentile( bx, s.bcdf + off, s.bbin + off, nbs, rand01( rng ), ibs );
      firstBin = ( ibs == 0 && fbkep <= 0.0 );
    }
    if ( firstBin ) {
      // one call site for both branches (one inlined copy in a lean pass)
      const int r = Full ? alg1FirstBinCall<Fast>( s, off, ioff, fbkep, ldg( bx + 1 ), x, rng, alpha_out, beta_out )
                         : alg1FirstBin<Fast>( s, off, ioff, fbkep, ldg( bx + 1 ), x, rng, alpha_out, beta_out );
      ph.template end<PH_BETA>();
      return r;
    }
    ph.template end<PH_BETA>();
    if ( beta <= maxd( -x, ldg( s.beta ) ) )
      return 0;
    const double rp = rand01( rng );
    const int ibeta = ioff + ibs;
    if ( ibeta < 1 )
      return 0; // cannot happen (beta above the beta grid front); keeps indices in bounds
    const double bl = ldg( s.beta + ibeta - 1 );
    double alpha;
    if ( Fast ) {
      const float rpf = (float)rp;
      // the two rows in a rolled loop: one copy of the sampler's code
      float al = 0.0f, ah = 0.0f;
#pragma unroll 1
      for ( int r = 0; r < 2; ++r ) {
        const float v = sampleAlphaF( s, s.info_f + off, ioff, ibeta - 1 + r, rpf );
        if ( r == 0 ) al = v; else ah = v;
      }
      const float af = fmaf( ah - al, (float)( beta - bl ) * __ldg( s.inv_dbeta_f + ibeta - 1 ), al );
      ph.template end<PH_ALPHA>();
      const ALimF lim = alphaLimitsF( (float)x, (float)( x + beta ), (float)beta );
      if ( af >= lim.lo && af <= lim.hi ) {
        alpha_out = (double)af;
        beta_out = beta;
        return 1;
      }
      return 0;
    } else {
      const double alphal = sampleAlpha<Fast>( s, infos, ioff, ibeta - 1, rp );
      const double alphah = sampleAlpha<Fast>( s, infos, ioff, ibeta, rp );
      alpha = alphal + ( alphah - alphal ) * ( ( beta - bl ) * ldg( s.inv_dbeta + ibeta - 1 ) );
      ph.template end<PH_ALPHA>();
    }
    const ALim al = alphaLimits( x, beta );
    if ( inInterval( al.lo, al.hi, alpha ) ) {
      alpha_out = alpha;
      beta_out = beta;
      return 1;
    }
    return 0;
  }

}

#include "ncgb_freegas.cuh"

namespace ncgb_dev {

  // Per-neutron state of SABSampler::sampleAlphaBeta (NCSABSampler.cc:158-227)
  // with its two nested rejection loops flattened, kept small because it stays
  // live across every Alg.1 attempt (the S(alpha,beta) pass runs at 32
  // registers per thread).  'x' is E/kT of the energy the table is sampled at
  // (Emax above the grid), 'xsamp' the one the sampler runs at (the grid's
  // first energy below it); the neutron's own E/kT is recomputed from 'ekin'.
  // An (alpha, beta) already drawn by the free-gas extender ('preset') needs
  // neither, so it shares their storage.  'state' packs the flags and the two
  // loop counters: 'outer' counts Alg.1 calls (<=100), 'inner' the attempts
  // of the current call (<=100).
  struct SABLane {
    static constexpr int ULTRA_SMALL = 1, PRESET = 2, INNER = 1 << 8, OUTER = 1 << 16;
    double ekin;
    union { double x; double pre_alpha; };
    union { double xsamp; double pre_beta; };
    int ie;
    int state;
    __device__ __forceinline__ bool ultraSmall() const { return state & ULTRA_SMALL; }
    __device__ __forceinline__ bool preset() const { return state & PRESET; }
    __device__ __forceinline__ int inner() const { return ( state >> 8 ) & 0xff; }
    __device__ __forceinline__ int outer() const { return ( state >> 16 ) & 0xff; }
  };

  // Set-up of a SAB scatter at energy ekin (NCSABSampler.cc:163-197),
  // including the high-E extrapolation (NCSABSampler.cc:170-178).
  // Full = false: a caller that never passes an energy above the grid (a
  // lean S(alpha,beta) pass), without the extender's out-of-line call.
  template<bool Full = true>
  __device__ __forceinline__ int sabBegin( const ncgb_sab_view& s, const double* fgtab, double ekin,
                                           ncgb_rng& rng, SABLane& L )
  {
    const int64_t ne = s.ne;
    int64_t iu = egridUpper( s, ekin );
    L.ekin = ekin;
    L.state = 0;
    double etab = ekin;
    if ( iu == ne ) {
      if constexpr ( !Full ) {
        return NCGB_ST_CALCERROR;
      }
      double pa = 0.0, pb = 0.0;
      const int h = sabHighE( s, fgtab, ekin, rng, pa, pb );
      if ( h == -1 )
        return NCGB_ST_CALCERROR;
      if ( h < 0 )
        return NCGB_ST_LOOPCAP;
      L.ie = (int)( ne - 1 );
      if ( h == 1 ) {
        L.state = SABLane::PRESET;
        L.pre_alpha = pa;
        L.pre_beta = pb;
        return NCGB_ST_OK;
      }
      etab = ldg( s.egrid + ne - 1 );
    } else if ( iu == 0 ) {
      L.ie = 0;
      if ( ekin < ldg( s.egrid ) )
        L.state = SABLane::ULTRA_SMALL;
    } else {
      if ( s.egrid_margin > 1.0 ) {
        const long long em = bits( ekin * s.egrid_margin );   // non-negative: integer compares
        while ( iu + 1 != ne && em > ldgbits( s.egrid + iu ) )
          ++iu;
      }
      L.ie = (int)iu;
    }
    L.x = etab * s.inv_kT;
    L.xsamp = L.ultraSmall() ? ldg( s.egrid ) * s.inv_kT : L.x;
    return NCGB_ST_OK;
  }

  // One step of the flattened loops.  Returns -1 to continue, NCGB_ST_OK when
  // (alpha, beta) are final, or an error status.
  template<bool Fast, bool Learned, bool Full = true, class Ph = NoPhases>
  __device__ __forceinline__ int sabStepAB( const ncgb_sab_view& s, SABLane& L, ncgb_rng& rng, double& alpha,
                                            double& beta, Ph&& ph = Ph() )
  {
    alpha = 0.0;
    beta = 0.0;
    if ( Full && L.preset() ) {   // set by the extender only (never in a lean pass)
      alpha = L.pre_alpha;
      beta = L.pre_beta;
    } else {
      if ( __ldg( s.smp_kind + L.ie ) != 0 ) {
        const int a = alg1Attempt<Fast, Learned, Full>( s, L.ie, L.xsamp, rng, alpha, beta, ph );
        if ( a < 0 )
          return NCGB_ST_LOOPCAP;
        if ( a == 0 ) {
          if ( L.inner() + 1 >= 100 )
            return NCGB_ST_LOOPCAP;
          L.state += SABLane::INNER;
          return -1;
        }
      } // else SABSamplerAtE_NoScatter: (alpha, beta) = (0, 0), no draws
      // an Alg.1 call completed: the outer loop's tests.  Alg.1 accepted
      // (alpha, beta) only if beta >= -xsamp and alpha is inside the limits
      // at xsamp; unless the energy is below the grid, xsamp == x and these
      // tests repeat that computation, so their outcome is known.
      L.state &= ~( 0xff * SABLane::INNER );
      const double x = L.x;
      bool accept = !L.ultraSmall() && __ldg( s.smp_kind + L.ie ) != 0;
      if ( !accept && !( beta < -x ) ) {
        const ALim al = alphaLimits( x, beta );
        if ( inInterval( al.lo, al.hi, alpha ) ) {
          accept = true;
        } else if ( L.ultraSmall() ) {
          alpha = al.lo + rand01( rng ) * ( al.hi - al.lo );
          accept = true;
        }
      }
      if ( !accept ) {
        if ( L.outer() + 1 >= 100 )
          return NCGB_ST_LOOPCAP;
        L.state += SABLane::OUTER;
        return -1;
      }
    }
    ph.template end<PH_ACCEPT>();
    return NCGB_ST_OK;
  }

  // sabStepAB, then (alpha, beta) -> (E', mu).
  template<bool Fast, bool Learned, bool Full = true, class Ph = NoPhases>
  __device__ __forceinline__ int sabStep( const ncgb_sab_view& s, SABLane& L, ncgb_rng& rng, double& ef, double& mu,
                                          Ph&& ph = Ph() )
  {
    double alpha, beta;
    const int st = sabStepAB<Fast, Learned, Full>( s, L, rng, alpha, beta, ph );
    if ( st != NCGB_ST_OK )
      return st;
    // SABSampler::sampleDeltaEMu (NCSABSampler.cc:229-236), SABScatter
    // (NCSABScatter.cc:92-101), with the neutron's own energy
    double deltaE, muv;
    if ( Fast ) {
      // Mixed mode.  x + beta stays FP64 (it cancels towards E' = 0) and
      // gives E' = kT (x + beta); the two branch tests run in FP32 (they
      // choose between formulas that agree where they meet, and the
      // isotropic branch sits within 1e-14 of E' = 0).  Away from the elastic
      // line (|beta| >= 0.01 E/kT, outside getAlphaLimits' Taylor region),
      // with a = sqrt(x), b = sqrt(x+beta): alpha- = (b-a)^2 and
      // E + E' - alpha kT = kT (2ab - (alpha - alpha-)), so
      // 1 - mu = d = (alpha - alpha-)/(2ab), in FP32 without cancellation;
      // mu = 1 - d in FP64.  Near the elastic line: the FP64 conversion.
      const double xtrue = __dmul_rn( L.ekin, s.inv_kT );   // not fused into the sum below
      const double xb = xtrue + beta;
      const float xf = (float)xtrue, xbf = (float)xb, bf = (float)beta;
      if ( xbf <= xf * 1e-14f ) {                 // muIsotropicAtBeta, NCKinUtils.hh:64-70
        muv = rand01( rng ) * 2.0 - 1.0;
      } else if ( !( fabsf( bf ) < 0.01f * xf ) ) {
        const float a = sqrtf( xf ), b = sqrtf( xbf );
        const float ab = a * b;
        if ( !( ab > 0.0f ) )
          return NCGB_ST_CALCERROR;
        const float sab = a + b;
        const float d = ( (float)alpha - ( bf * bf ) / ( sab * sab ) ) / ( 2.0f * ab );
        muv = 1.0 - (double)fminf( 2.0f, fmaxf( 0.0f, d ) );
      } else {
        const int st = alphaBetaToDeltaEMu( alpha, beta, L.ekin, s.kT, deltaE, muv );
        if ( st != NCGB_ST_OK )
          return st;
        ef = maxd( 0.0, L.ekin + deltaE );
        mu = muv;
        return NCGB_ST_OK;
      }
      ef = bits( xb ) > 0 ? s.kT * xb : 0.0;     // max(0, E'), the sign tested on the integer pipe
      mu = muv;
      return NCGB_ST_OK;
    }
    if ( beta <= __dmul_rn( L.ekin, s.inv_kT ) * ( -1.0 + 1e-14 ) ) { // muIsotropicAtBeta, NCKinUtils.hh:64-70
      deltaE = beta * s.kT;
      muv = rand01( rng ) * 2.0 - 1.0;
    } else {
      const int st = alphaBetaToDeltaEMu( alpha, beta, L.ekin, s.kT, deltaE, muv );
      if ( st != NCGB_ST_OK )
        return st;
    }
    ef = maxd( 0.0, L.ekin + deltaE );
    mu = muv;
    return NCGB_ST_OK;
  }
}

#endif
