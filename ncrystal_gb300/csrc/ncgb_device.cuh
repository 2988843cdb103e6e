// Device-side evaluation of one neutron against one material: cross-section
// (ProcComposition over PowderBragg / ElIncScatter / SABScatter / FreeGas) and
// one isotropic scatter (E', mu).  FP64 throughout, so that the results agree
// with NCrystal's own to rounding; the control flow and the order of random
// draws follow the reference function for function (each cites its source).
//
// GB300 notes:
//   * Binary searches over non-negative tables (energy grids, cumulative sums,
//     CDFs) compare the IEEE-754 bit patterns as 64-bit integers, which orders
//     non-negative doubles exactly like a floating-point compare but runs on
//     the integer pipe: GB300's FP64 pipe is narrow and stays free for the
//     arithmetic.
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

  __device__ __forceinline__ double clampd( double x, double lo, double hi ) { return x < lo ? lo : ( x > hi ? hi : x ); }
  __device__ __forceinline__ double maxd( double a, double b ) { return a < b ? b : a; }
  __device__ __forceinline__ bool contains( double lo, double hi, double e ) { return e >= lo && e <= hi; }

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

  __device__ __forceinline__ void neumaierAdd( double& s, double& c, double x )
  {
    double t = s + x;
    c += ( fabs(s) >= fabs(x) ) ? (s-t)+x : (x-t)+s;
    s = t;
  }

  // Returns NCGB_ST_CALCERROR where the reference throws (E*E' == 0,
  // NCKinUtils.cc:40-45).
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

  // NCElIncXS.cc:34-54
  __device__ __forceinline__ double oneMinusExpMtDivT( double t )
  {
    if ( t < 0.01 )
      return ( 1 + t * ( -0.5 + t * 0.16666666666666666666666666666666666666666667 * ( 1. - 0.25 * t ) ) );
    if ( t > 24.0 )
      return 1.0 / t;
    t = -t;
    return expm1( t ) / t;
  }

  constexpr double kElIncXS = 16.0 * 9.86960440108935861883449099987615113531369941 * 12.22430978582345950656;
  constexpr double kElIncMu = 8.0 * 9.86960440108935861883449099987615113531369941 * 12.22430978582345950656;

  // ElIncXS::evalXSContribsCommul, NCElIncXS.cc:130-141
  __device__ __forceinline__ double elincXS( const ncgb_elinc_view& v, double ekin, double* commul )
  {
    const double e = kElIncXS * ekin;
    double xs = 0.0;
    for ( int i = 0; i < v.n && i < NCGB_MAX_ELINC; ++i ) {
      xs += v.sigma[i] * oneMinusExpMtDivT( v.msd[i] * e );
      if ( commul ) commul[i] = xs;
    }
    return xs;
  }

  // PowderBragg, NCPowderBragg.cc:152-176.  idx_out: last valid plane.
  __device__ __forceinline__ double braggXS( const ncgb_bragg_view& v, double ekin, int64_t& idx_out )
  {
    idx_out = 0;
    if ( v.n == 0 || ekin < v.threshold || !isfinite(ekin) )
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
        return __longlong_as_double(0x7ff0000000000000LL);
      const double a2 = a_squared;
      return 0.564189583547756286948079451560772585844050629
        * ( 2.0 / a + a *( (2.0/3.0)- a2*((1.0/15.0)-a2*((1.0/105.0)-a2*((1.0/756.0)-a2*(1.0/5940.0))))));
    }
    const double inva = 1.0 / a;
    return ( 1.0 + 0.5*inva*inva ) * erf( a ) + 0.564189583547756286948079451560772585844050629 * exp( -a_squared ) * inva;
  }

  // SABXSProvider::crossSection (NCSABXSProvider.cc:54-95) x SABScatter scale
  // (NCSABScatter.cc:87-90).  Requires ekin >= 0 and not NaN.
  __device__ __forceinline__ double sabXS( const ncgb_sab_view& s, double ekin )
  {
    const int64_t ne = s.ne;
    const int64_t iu = upper_bound_nn( s.egrid, ne, ekin );
    double xs;
    if ( iu == ne ) {
      xs = s.kext / ekin + s.ext_sigma_free * freeGasShape( s.ext_ca * ekin );
    } else if ( iu == 0 ) {
      xs = ekin > 0.0 ? sqrt( ldg(s.egrid) / ekin ) * ldg(s.xs) : __longlong_as_double(0x7ff0000000000000LL);
    } else {
      const double el = ldg( s.egrid + iu - 1 ), eu = ldg( s.egrid + iu );
      const double xl = ldg( s.xs + iu - 1 ), xu = ldg( s.xs + iu );
      xs = xl + ( xu - xl ) * ( ekin - el ) / ( eu - el );
    }
    return xs * s.internal_scale;
  }

  // ProcComposition::updateCacheIsotropic, NCProcImpl.cc:166-204.  Also
  // returns the last valid Bragg plane of each Bragg component.
  __device__ __forceinline__ double xsCommul( const ncgb_material_view& m, double ekin,
                                              double* commul, int64_t* braggIdx )
  {
    double tot = 0.0;
    for ( int i = 0; i < m.ncomp; ++i ) {
      const ncgb_comp_view& c = m.comp[i];
      double xs = 0.0;
      braggIdx[i] = 0;
      if ( contains( c.elow, c.ehigh, ekin ) ) {
        switch ( c.type ) {
          case NCGB_COMP_ELINC: xs = elincXS( c.elinc, ekin, nullptr ); break;
          case NCGB_COMP_BRAGG: xs = braggXS( c.bragg, ekin, braggIdx[i] ); break;
          case NCGB_COMP_SAB: xs = sabXS( c.sab, ekin ); break;
          case NCGB_COMP_FREEGAS: xs = c.fg.sigma_free * freeGasShape( c.fg.ca * ekin ); break;
          default: break;
        }
      }
      commul[i] = ( tot += ( c.scale * xs ) );
    }
    return tot;
  }

  // pickRandIdxByWeight (NCRandUtils.hh:130-133, NCRandUtils.cc:198-222)
  __device__ __forceinline__ int pickIdx( ncgb_rng& rng, const double* commul, int n )
  {
    if ( n == 1 )
      return 0;
    const double r = ncgb_rng_generate( &rng );
    const double choice = commul[n-1] * r;
    if ( n < 5 ) {
      for ( int i = 0; i < n; ++i )
        if ( commul[i] > choice )
          return i;
      return n - 1;
    }
    int lo = 0, len = n;
    while ( len > 0 ) {
      int half = len >> 1;
      if ( commul[lo+half] < choice ) { lo += half + 1; len -= half + 1; }
      else len = half;
    }
    return lo < n - 1 ? lo : n - 1;
  }

  // ---- samplers -----------------------------------------------------------------

  // PowderBragg::genScatterMu, NCPowderBragg.cc:178-200
  __device__ __forceinline__ double braggMu( const ncgb_bragg_view& v, ncgb_rng& rng, double ekin, int64_t idx )
  {
    const double r = ncgb_rng_generate( &rng );
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
  __device__ __forceinline__ double elincMuMono( ncgb_rng& rng, double ekin, double msd, int& status )
  {
    const double a = ( kElIncMu * ekin ) * msd;
    if ( a < 0.01 ) {
      const double maxval = expSmall( a );
      for ( int it = 0; it < 100000; ++it ) {
        const double mu = ncgb_rng_generate( &rng ) * 2.0 - 1.0;
        if ( ncgb_rng_generate( &rng ) * maxval < expSmall( a * mu ) )
          return mu;
      }
      status = NCGB_ST_LOOPCAP;
      return 1.0;
    }
    return clampd( log1p( ncgb_rng_generate( &rng ) * expm1( 2.0 * a ) ) / a - 1.0, -1.0, 1.0 );
  }

  // ElIncXS::EPointAnalysis::sampleMu, NCElIncXS.cc:178-191
  __device__ __forceinline__ double elincMu( const ncgb_elinc_view& v, ncgb_rng& rng, double ekin, int& status )
  {
    if ( v.n == 1 )
      return elincMuMono( rng, ekin, v.msd[0], status );
    double commul[NCGB_MAX_ELINC];
    elincXS( v, ekin, commul );
    const int i = pickIdx( rng, commul, v.n );
    return elincMuMono( rng, ekin, v.msd[i], status );
  }

  // PointwiseDist::percentileWithIndex, NCPointwiseDist.cc:76-110
  __device__ __forceinline__ double percentile( const double* x, const double* y, const double* cdf, int64_t n,
                                                double p, int64_t& bin )
  {
    if ( p == 1.0 ) { bin = n - 2; return ldg( x + n - 1 ); }
    int64_t i = lower_bound_nn( cdf, n, p );
    if ( i > n - 1 ) i = n - 1;
    if ( i < 1 ) i = 1;
    const double x0 = ldg( x + i - 1 ), x1 = ldg( x + i );
    const double dx = x1 - x0;
    const double c = ( p - ldg( cdf + i - 1 ) );
    const double a = ldg( y + i - 1 );
    const double d = ldg( y + i ) - a;
    double zdx;
    if ( !a ) {
      zdx = d > 0.0 ? sqrt( ( 2.0 * c * dx ) / d ) : 0.5 * dx;
    } else {
      const double e = d * c / ( dx * a * a );
      if ( fabs(e) > 1e-7 )
        zdx = ( sqrt( 1.0 + 2.0 * e ) - 1.0 ) * dx * a / d;
      else
        zdx = ( 1 + 0.5 * e * ( e - 1.0 ) ) * c / a;
    }
    bin = i - 1;
    return clampd( x0 + zdx, x0, x1 );
  }

  // SABUtils::sampleLogLinDist_fast, NCSABUtils.hh:282-304
  __device__ __forceinline__ double logLin( double a, double fa, double b, double fb, double rnd, double logfa, double logfb )
  {
    double df = fb - fa;
    if ( fa * fb * df != 0.0 ) {
      const double a_sub_b = a - b;
      const double logfa_fb = logfb - logfa;
      if ( a_sub_b * logfa_fb != 0.0 )
        return a_sub_b * log( fa * exp( a * logfa_fb / a_sub_b ) / ( fa + rnd * df ) ) / logfa_fb;
      df = 0.0;
    }
    if ( !df )
      return a + rnd * ( b - a );
    const double xx = ( b - a ) * sqrt( rnd );
    return ( fa ? b - xx : a + xx );
  }

  __device__ __forceinline__ double clampRand( double r ) { return clampd( r, 2.2250738585072014e-308, 1.0 ); }

  // SABSamplerAtE_Alg1::sampleAlpha, NCSABSamplerModels.cc:157-234
  __device__ __forceinline__ double sampleAlpha( const ncgb_sab_view& s, const ncgb_alpha_info* infos,
                                                 int64_t ioff, int64_t ibeta, double rp )
  {
    const ncgb_alpha_info* info = infos + ( ibeta - ioff );
    const double prob_front = ldg( &info->prob_front );
    const int64_t na = s.na;
    const double* cumul = s.cumul + ibeta * na;
    const double* sab = s.sab + ibeta * na;
    const double* logsab = s.logsab + ibeta * na;
    if ( rp <= prob_front ) {
      const double fa = ldg( &info->front_alpha );
      if ( prob_front == 2.0 ) {
        const double da = ldg( &info->back_alpha ) - fa;
        return fa + rp * da;
      } else if ( prob_front == 1.0 ) {
        return logLin( fa, ldg( &info->front_sval ), ldg( &info->back_alpha ), ldg( &info->back_sval ),
                       rp, ldg( &info->front_logsval ), ldg( &info->back_logsval ) );
      } else {
        const uint32_t fi = __ldg( &info->front_idx );
        const double p2 = clampRand( rp / prob_front );
        return logLin( fa, ldg( &info->front_sval ), ldg( s.alpha + fi ), ldg( sab + fi ),
                       p2, ldg( &info->front_logsval ), ldg( logsab + fi ) );
      }
    }
    const double prob_notback = ldg( &info->prob_notback );
    if ( rp <= prob_notback ) {
      const double p2 = clampd( ( rp - prob_front ) / ( prob_notback - prob_front ), 0.0, 1.0 );
      const int64_t il = __ldg( &info->front_idx ), iu = __ldg( &info->back_idx );
      const double cl = ldg( cumul + il ), cu = ldg( cumul + iu );
      const double sel = cl + p2 * ( cu - cl );
      const int64_t e = il + upper_bound_nn( cumul + il, iu + 1 - il, sel );
      if ( e > iu )
        return ldg( s.alpha + iu );
      if ( e <= il )
        return ldg( s.alpha + il );
      const int64_t a0 = e - 1, a1 = e;
      const double c0 = ldg( cumul + a0 );
      const double binArea = ldg( cumul + a1 ) - c0;
      const double rr = clampRand( ( sel - c0 ) / binArea );
      return logLin( ldg( s.alpha + a0 ), ldg( sab + a0 ), ldg( s.alpha + a1 ), ldg( sab + a1 ),
                     rr, ldg( logsab + a0 ), ldg( logsab + a1 ) );
    }
    const uint32_t bi = __ldg( &info->back_idx );
    const double p2 = clampRand( ( rp - prob_notback ) / ( 1.0 - prob_notback ) );
    return logLin( ldg( s.alpha + bi ), ldg( sab + bi ), ldg( &info->back_alpha ), ldg( &info->back_sval ),
                   p2, ldg( logsab + bi ), ldg( &info->back_logsval ) );
  }

  // SABSamplerAtE_Alg1::sampleAlphaBeta, NCSABSamplerModels.cc:48-155
  __device__ __forceinline__ int alg1( const ncgb_sab_view& s, int64_t ie, double x, ncgb_rng& rng,
                                       double& alpha_out, double& beta_out )
  {
    const int64_t off = __ldg( s.smp_offset + ie );
    const int64_t nbs = __ldg( s.smp_nbeta + ie );
    const double* bx = s.bx + off;
    const double* by = s.by + off;
    const double* bcdf = s.bcdf + off;
    const ncgb_alpha_info* infos = s.info + off;
    const int64_t ioff = __ldg( s.smp_ibetaoffset + ie );
    const double fbkep = ldg( s.smp_fbkep + ie );
    const double bg0 = ldg( s.beta );
    for ( int iloop = 0; iloop < 100; ++iloop ) {
      int64_t ibs;
      double beta = percentile( bx, by, bcdf, nbs, ncgb_rng_generate( &rng ), ibs );
      if ( ibs == 0 && fbkep <= 0.0 ) {
        const double b0 = fbkep;
        const double b1 = ldg( bx + 1 );
        if ( b1 < -x )
          continue;
        const double delta_beta = b1 - b0;
        double alphaval = 0.0;
        for ( int iii = 0; iii < 30; ++iii ) {
          beta = maxd( fbkep, b0 + delta_beta * ncgb_rng_generate( &rng ) );
          if ( beta < -x )
            break;
          alphaval = sampleAlpha( s, infos, ioff, ioff, ncgb_rng_generate( &rng ) );
          const ALim al = alphaLimits( -fbkep, beta );
          if ( inInterval( al.lo, al.hi, alphaval ) )
            break;
          if ( iii == 29 ) {
            alphaval = 0.5 * ( al.lo + al.hi );
            break;
          }
        }
        if ( beta < -x )
          continue;
        const ALim al2 = alphaLimits( x, beta );
        if ( inInterval( al2.lo, al2.hi, alphaval ) ) {
          alpha_out = alphaval; beta_out = beta; return NCGB_ST_OK;
        }
        continue;
      }
      if ( beta <= maxd( -x, bg0 ) )
        continue;
      const double rp = ncgb_rng_generate( &rng );
      const int64_t ibeta = ioff + ibs;
      if ( ibeta < 1 )
        continue; // cannot happen (beta > beta grid front); keeps indexing in bounds
      const double bl = ldg( s.beta + ibeta - 1 );
      const double alphal = sampleAlpha( s, infos, ioff, ibeta - 1, rp );
      const double bh = ldg( s.beta + ibeta );
      const double alphah = sampleAlpha( s, infos, ioff, ibeta, rp );
      const double alpha = alphal + ( alphah - alphal ) * ( beta - bl ) / ( bh - bl );
      const ALim al = alphaLimits( x, beta );
      if ( inInterval( al.lo, al.hi, alpha ) ) {
        alpha_out = alpha; beta_out = beta; return NCGB_ST_OK;
      }
    }
    return NCGB_ST_LOOPCAP;
  }

  // SABSampler::sampleAlphaBeta + sampleDeltaEMu (NCSABSampler.cc:158-236),
  // SABScatter::sampleScatterIsotropic (NCSABScatter.cc:92-101).
  __device__ __forceinline__ int sabScatter( const ncgb_sab_view& s, ncgb_rng& rng, double ekin, double& ef, double& mu )
  {
    const int64_t ne = s.ne;
    int64_t iu = upper_bound_nn( s.egrid, ne, ekin );
    bool ultra_small = false;
    int64_t ie;
    if ( iu == ne ) {
      return NCGB_ST_UNSUPPORTED; // E >= Emax: free-gas extender (NCSABSampler.cc:59-156)
    } else if ( iu == 0 ) {
      ie = 0;
      ultra_small = ( ekin < ldg( s.egrid ) );
    } else {
      if ( s.egrid_margin > 1.0 ) {
        const double em = ekin * s.egrid_margin;
        while ( iu + 1 != ne && em > ldg( s.egrid + iu ) )
          ++iu;
      }
      ie = iu;
    }
    const double x = ekin / s.kT;
    const double xs_ = ultra_small ? ldg( s.egrid ) / s.kT : x;
    const int kind = __ldg( s.smp_kind + ie );
    double alpha = 0.0, beta = 0.0;
    bool found = false;
    for ( int loop = 0; loop < 100; ++loop ) {
      if ( kind == 0 ) {
        alpha = 0.0; beta = 0.0;
      } else {
        const int st = alg1( s, ie, xs_, rng, alpha, beta );
        if ( st != NCGB_ST_OK )
          return st;
      }
      if ( beta < -x )
        continue;
      const ALim al = alphaLimits( x, beta );
      if ( inInterval( al.lo, al.hi, alpha ) ) { found = true; break; }
      if ( ultra_small ) {
        alpha = al.lo + ncgb_rng_generate( &rng ) * ( al.hi - al.lo );
        found = true;
        break;
      }
    }
    if ( !found )
      return NCGB_ST_LOOPCAP;
    double deltaE, muv;
    if ( beta <= x * ( -1.0 + 1e-14 ) ) { // muIsotropicAtBeta, NCKinUtils.hh:64-70
      deltaE = beta * s.kT;
      muv = ncgb_rng_generate( &rng ) * 2.0 - 1.0;
    } else {
      const int st = alphaBetaToDeltaEMu( alpha, beta, ekin, s.kT, deltaE, muv );
      if ( st != NCGB_ST_OK )
        return st;
    }
    ef = maxd( 0.0, ekin + deltaE );
    mu = muv;
    return NCGB_ST_OK;
  }

  // One neutron: cross-section (ProcComposition::crossSectionIsotropic,
  // NCProcImpl.cc:353-362) and, if wanted, one scatter
  // (ProcComposition::sampleScatterIsotropic, NCProcImpl.cc:379-389).
  template<bool DoXS, bool DoScatter>
  __device__ __forceinline__ int evalNeutron( const ncgb_material_view& m, ncgb_rng& rng, double ekin,
                                              double& xs, double& ef, double& mu )
  {
    xs = 0.0; ef = ekin; mu = 1.0;
    if ( !contains( m.dom_elow, m.dom_ehigh, ekin ) )
      return NCGB_ST_OK;
    double commul[NCGB_MAX_COMP];
    int64_t braggIdx[NCGB_MAX_COMP];
    xs = xsCommul( m, ekin, commul, braggIdx );
    if ( !DoScatter )
      return NCGB_ST_OK;
    const int ic = pickIdx( rng, commul, m.ncomp );
    const ncgb_comp_view& c = m.comp[ic];
    int st = NCGB_ST_OK;
    switch ( c.type ) {
      case NCGB_COMP_BRAGG:
        // PowderBragg::sampleScatterIsotropic, NCPowderBragg.cc:202-216
        if ( !( c.bragg.n == 0 || ekin < c.bragg.threshold || !isfinite(ekin) ) )
          mu = braggMu( c.bragg, rng, ekin, braggIdx[ic] );
        break;
      case NCGB_COMP_ELINC:
        mu = elincMu( c.elinc, rng, ekin, st );
        break;
      case NCGB_COMP_SAB:
        st = sabScatter( c.sab, rng, ekin, ef, mu );
        break;
      case NCGB_COMP_FREEGAS:
        st = NCGB_ST_UNSUPPORTED;
        break;
      default:
        break;
    }
    if ( st != NCGB_ST_OK ) { ef = -1.0; mu = -999.0; }
    return st;
  }
}

#endif
