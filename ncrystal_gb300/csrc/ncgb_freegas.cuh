// Free-gas scattering on the GPU: FreeGasSampler (NCFreeGasUtils.cc:492-932)
// for FreeGas components and for the S(alpha,beta) extender above a kernel's
// Emax (SABSampler::sampleHighE, NCSABSampler.cc:59-156).  Same arithmetic
// and draw order as the reference; its unbounded rejection loops get caps
// here (1e6 tries) that end the neutron with NCGB_ST_LOOPCAP instead of
// looping forever.  Included by ncgb_device.cuh.
#ifndef NCGB_FREEGAS_CUH
#define NCGB_FREEGAS_CUH

namespace ncgb_dev {

  constexpr int kFGLoopCap = 1000000;
  constexpr int kFGTableLen = 1103;
  constexpr double kInvSqrtPi = 0.564189583547756286948079451560772585844050629;

  // erfcQuickBounds, NCFreeGasUtils.cc:124-147 (table built on the host with
  // the same erfc as the reference's).
  __device__ __forceinline__ void fgErfcBounds( const double* tab, double x, double& lb, double& ub )
  {
    const double binw = ( 9.0 - ( -2.0 ) ) / ( kFGTableLen - 3 );
    const double invbinw = ( kFGTableLen - 3 ) / ( 9.0 - ( -2.0 ) );
    const double xs = clampd( x, -2.0 - 0.5 * binw, 9.0 + 0.5 * binw );
    int bin = (int)( 1.0 + ( xs - ( -2.0 ) ) * invbinw );
    if ( bin > kFGTableLen - 1 ) bin = kFGTableLen - 1;
    if ( bin < 0 ) bin = 0;
    lb = ldg( tab + bin + 1 ) * 0.99999999;
    ub = ldg( tab + bin ) * 1.00000001;
  }

  // erfcdiff, NCMath.cc:338-390
  __device__ __forceinline__ double fgErfcDiffNT( double a, double b )
  {
    if ( b < 0 ) { double t = -b; b = -a; a = t; }
    const double erfca = a > 27.3 ? 0.0 : erfc( a );
    if ( b > a + 4.0 && ( a >= 4 || ( a < 0.0 && b > 6.0 ) ) )
      return erfca;
    const double erfcb = b > 27.3 ? 0.0 : erfc( b );
    return erfca - erfcb;
  }

  __device__ __forceinline__ double fgErfcDiff( double a, double b )
  {
    if ( maxd( fabs(a), fabs(b) ) < 0.32 ) {
      const double c1 = -2.0 * kInvSqrtPi, c3 = 2.0 * kInvSqrtPi / 3.0, c5 = -0.2 * kInvSqrtPi, c7 = kInvSqrtPi / 21.0;
      const double c9 = -kInvSqrtPi / 108.0, c11 = kInvSqrtPi / 660.0, c13 = -kInvSqrtPi / 4680.0, c15 = kInvSqrtPi / 37800.0;
      const double a2 = a*a, b2 = b*b;
      const double a3 = a * a2 * ( c3 + a2 * ( c5 + a2 * ( c7 + ( a2 * ( c9 + a2 * ( c11 + a2 * ( c13 + a2 * c15 ) ) ) ) ) ) );
      const double b3 = b * b2 * ( c3 + b2 * ( c5 + b2 * ( c7 + ( b2 * ( c9 + b2 * ( c11 + b2 * ( c13 + b2 * c15 ) ) ) ) ) ) );
      return c1*(a-b) + ( a3 - b3 );
    }
    return a > b ? -fgErfcDiffNT( b, a ) : fgErfcDiffNT( a, b );
  }

  // erfc_rescaled, NCMath.cc:393-417: exp(b)*erfc(x)
  __device__ __forceinline__ double fgErfcRescaled( double x, double b )
  {
    if ( b < -745.1 )
      return 0.0;
    if ( ( x < 23.0 && fabs(b) < 700 ) || x < 5 )
      return exp( b ) * erfc( x );
    const double bxx = b - x*x;
    if ( bxx < -745.1 )
      return 0.0;
    const double y = 1/x, y2 = y*y;
    return kInvSqrtPi * exp( bxx ) * ( y+y2*(-0.5+y2*(0.75+y2*(-1.875+y2*(6.5625+y2*-29.53125)))) );
  }

  // RandExpIntervalSampler, NCRandUtils.hh:162-199
  struct FGExpInt { double a, c1, c2; };
  __device__ __forceinline__ void fgExpIntSet( FGExpInt& s, double a, double b, double c )
  {
    s.a = a; s.c1 = -1.0 / c; s.c2 = expm1( -c * ( b - a ) );
  }
  __device__ __forceinline__ double fgExpIntSample( const FGExpInt& s, ncgb_rng& rng )
  {
    return s.a + s.c1 * log( 1.0 + rand01( rng ) * s.c2 );
  }

  // randExpDivSqrt, NCRandUtils.cc:224-330: exp(-c*x)/sqrt(x) on [a,b]
  static __device__ __noinline__ double fgRandExpDivSqrt( ncgb_rng& rng, double c, double a, double b, int& st )
  {
    const double A = c*a;
    if ( A > 0.1 ) {
      const double U = c*(b-a);
      const double invA = 1.0/A;
      FGExpInt es;
      fgExpIntSet( es, 0, U, 1.0 );
      for ( int it = 0; it < kFGLoopCap; ++it ) {
        const double ugen = fgExpIntSample( es, rng );
        const double R = rand01( rng );
        if ( (1.0+ugen*invA)*R*R < 1.0 )
          return clampd( (ugen+A)/c, a, b );
      }
      st = NCGB_ST_LOOPCAP;
      return a;
    }
    const double Ulim = 16.1180956509583;
    const double U = c*(b-a) < Ulim ? c*(b-a) : Ulim;
    const double B = U+A;
    if ( !( B > A ) )
      return a;
    const double sqrtA = sqrt(A), sqrtB = sqrt(B);
    const double sBmA = sqrtB - sqrtA, twosqrtA = 2*sqrtA;
    double ugen = 0.0;
    bool ok = false;
    for ( int it = 0; it < kFGLoopCap; ++it ) {
      const double T = rand01( rng ) * sBmA;
      ugen = T*(T+twosqrtA);
      const double Ra = rand01( rng );
      if ( ugen < 2.0 ) {
        const double t6 = 1.0+ugen*(-1.0+ugen*(1.0/2.0+ugen*(-1.0/6.0+ugen*(1.0/24.0+ugen*(-1.0/120.0+ugen*(1.0/720.0))))));
        if ( Ra > t6 ) continue;
        if ( Ra + 0.020221 < t6 ) { ok = true; break; }
      } else {
        if ( Ra > 0.135335283236614 ) continue;
        if ( ugen > 4.0 && Ra > 0.0183156388887343 ) continue;
      }
      if ( Ra < exp( -ugen ) ) { ok = true; break; }
    }
    if ( !ok ) { st = NCGB_ST_LOOPCAP; return a; }
    return clampd( (ugen+A)/c, a, b );
  }

  // randExpMInvXMCXDivSqrtX, NCFreeGasUtils.cc:223-488: exp(-1/x-c*x)/sqrt(x) on [xm,xp]
  __device__ __forceinline__ double fgFEval( double x, double xmax, double c )
  {
    const double exparg = (x-xmax)/(x*xmax)-c*(x-xmax);
    if ( exparg >= 706.0 )
      return 1.0;
    return exparg < -745.1 ? 0.0 : exp( exparg ) * sqrt( xmax/x );
  }

  static __device__ __noinline__ double fgRandEMix( ncgb_rng& rng, double c, double xm, double xp, int& st )
  {
    if ( xp == xm )
      return xm;
    const double sqrtc = sqrt(c);
    const double invsqrtc = 1/sqrtc;
    const double xpeak = ( c > 1e-5
                           ? ( c > 1e200 ? invsqrtc : (sqrt(16.0*c+1.0)-1.0)/(4.0*c) )
                           : ( 2.0-c*(8.0-c*(64.0-c*(640.0-c*7168.0))) ) );
    const double dblmin = 2.2250738585072014e-308;
    if ( xpeak == 0.0 )
      return xm > 0.0 ? xm : ( dblmin < xp ? dblmin : xp );
    const double xmax = ( xm > xpeak ? xm : ( xp < xpeak ? xp : xpeak ) );
    if ( !( xmax > 0.0 ) )
      return xm;
    const double xlarge = maxd( 5.0/sqrt(c), 2*xpeak );
    const double xsmall = ( 0.2/sqrt(c) < 0.5*xpeak ) ? 0.2/sqrt(c) : 0.5*xpeak;
    if ( xp > xlarge ) {
      const double t = maxd( xm, xlarge ) + 15.0/c;
      xp = xp < t ? xp : t;
    }
    if ( xm < xsmall ) {
      const double xsm = xp < xsmall ? xp : xsmall;
      xm = maxd( xm, xsm / ( 1 + 30.0*xsm ) );
    }
    if ( ( xm = maxd( dblmin, maxd( dblmin/xp, xm ) ) ) >= xp )
      return xp;
    const double fcutoff_limit = 1e-9;
    if ( xp < xpeak ) {
      for ( int it = 0; it < kFGLoopCap; ++it ) {
        const double xm_new = xp - 0.01*(xp-xm);
        if ( fgFEval( xm_new, xmax, c ) >= fcutoff_limit )
          break;
        xm = xm_new;
      }
    }
    double probability_flat, xswitch, area_right = -1.0;
    if ( xm >= xlarge ) {
      probability_flat = 0.0;
      xswitch = xm;
    } else if ( c > 25 || xp <= xlarge ) {
      probability_flat = 1.0;
      xswitch = xp;
    } else {
      xswitch = xlarge;
      const double area_left = (xswitch-xm);
      const double B = c*xmax+1/xmax-1/xp;
      area_right = ( fgErfcRescaled( sqrtc*sqrt(xswitch), B ) - fgErfcRescaled( sqrtc*sqrt(xp), B ) )
                   * sqrt( 3.1415926535897932384626433832795028841971694*(xmax/c) );
      probability_flat = area_left/(area_left+area_right);
    }
    bool always_left = ( probability_flat > 1.0-fcutoff_limit );
    bool single_side = always_left || ( probability_flat < fcutoff_limit );
    if ( !single_side && fgFEval( xswitch, xmax, c ) < fcutoff_limit*1.1 ) {
      probability_flat = 1.0;
      area_right = 0.0;
      xp = xswitch;
      always_left = true;
      single_side = false;
    }
    for ( int it = 0; it < kFGLoopCap; ++it ) {
      const bool do_flat = single_side ? always_left : ( rand01( rng ) < probability_flat );
      if ( do_flat ) {
        double dx = xswitch-xm;
        const double xthr_up = xswitch, xthr_low = xm;
        const double fthreshold = 0.05;
        const double xgen = xm + rand01( rng )*dx;
        const double Raccept = rand01( rng );
        if ( !inInterval( xthr_low, xthr_up, xgen ) && Raccept > fthreshold )
          continue;
        const double fval = fgFEval( xgen, xmax, c );
        if ( fval < fthreshold && fval < fcutoff_limit ) {
          if ( xgen < xmax )
            xm = xgen;
          else
            xswitch = xgen;
          dx = xswitch-xm;
          if ( !single_side ) {
            probability_flat = dx/(dx+area_right);
            always_left = ( probability_flat > 1.0-fcutoff_limit );
            single_side = always_left || ( probability_flat < fcutoff_limit );
          }
          continue;
        }
        if ( Raccept <= fval )
          return xgen;
      } else {
        const double xgen = fgRandExpDivSqrt( rng, c, xswitch, xp, st );
        if ( st != NCGB_ST_OK )
          return xgen;
        if ( rand01( rng ) < exp( (xgen-xp)/(xgen*xp) ) )
          return xgen;
      }
    }
    st = NCGB_ST_LOOPCAP;
    return xm;
  }

  // FreeGasSampler state, NCFreeGasUtils.cc:492-515
  struct FGSampler { double c, kT, sqrtAc, invA, Adiv4, normfact, c_real; };

  __device__ __forceinline__ void fgInit( FGSampler& s, double ekin, double kT, double mass_amu )
  {
    const double cr = ekin / kT;
    s.c = cr > 1e-10 ? cr : 1e-10;
    if ( s.c > 1e14 ) s.c = 1e14;
    s.kT = kT;
    s.sqrtAc = sqrt( mass_amu * s.c / 1.00866491588 );
    const double Arel = ( 1.0 / 1.00866491588 ) * mass_amu;
    s.invA = 1.0 / Arel;
    s.Adiv4 = 0.25 * Arel;
    s.normfact = 0.5 / erf( sqrt( s.c * s.invA ) );
    s.c_real = cr;
  }

  // FGEvalBetaDistHelper, NCFreeGasUtils.cc:153-222
  struct FGBetaEval { double beta, normfact, expmbeta, k11, k12, k21, k22; };

  __device__ __forceinline__ void fgBetaInit( FGBetaEval& h, const FGSampler& s, double beta )
  {
    h.beta = beta;
    h.normfact = s.normfact;
    h.expmbeta = -1.0;
    const double eps = beta / s.c;
    const double sqrt1pluseps = sqrt( 1 + eps );
    const double S = ( beta < 0.0 ? -1.0 : 1.0 );
    const double sqrtepsprime = ( eps >= 0.0 ? 1.0 : sqrt1pluseps );
    const double sqrtgammaplus = sqrt( 2.0+eps+2.0*sqrt1pluseps );
    const double SP = 0.5*(S+s.invA);
    const double SM = 0.5*(S-s.invA);
    const double iAs = s.invA*sqrtepsprime;
    const double mSs = -S*sqrtepsprime;
    const double SPsgp = sqrtgammaplus*SP;
    const double SMsgp = sqrtgammaplus*SM;
    h.k11 = s.sqrtAc*( -iAs + SPsgp );
    h.k12 = s.sqrtAc*( mSs + SPsgp );
    h.k21 = s.sqrtAc*( mSs + SMsgp );
    h.k22 = s.sqrtAc*( iAs + SMsgp );
  }

  __device__ __forceinline__ void fgBetaExpm( FGBetaEval& h )
  {
    if ( h.expmbeta < 0 )
      h.expmbeta = h.beta < -700.0 ? 0.0 : exp( -h.beta );
  }

  __device__ __forceinline__ double fgBetaExact( FGBetaEval& h )
  {
    const double t1 = fgErfcDiff( h.k11, h.k12 );
    fgBetaExpm( h );
    if ( !h.expmbeta )
      return h.normfact*t1;
    const double t2 = fgErfcDiff( h.k21, h.k22 );
    return h.normfact*(t1+t2*h.expmbeta);
  }

  __device__ __forceinline__ void fgBetaBounds( FGBetaEval& h, const double* tab, double& lb, double& ub )
  {
    double l11, u11, l12, u12, l21, u21, l22, u22;
    fgErfcBounds( tab, h.k11, l11, u11 );
    fgErfcBounds( tab, h.k12, l12, u12 );
    const double t1l = l11 - u12, t1u = u11 - l12;
    fgErfcBounds( tab, h.k21, l21, u21 );
    fgErfcBounds( tab, h.k22, l22, u22 );
    const double t2l = l21 - u22, t2u = u21 - l22;
    if ( t2u > 0.0 ) {
      fgBetaExpm( h );
      lb = h.normfact*(t1l+t2l*h.expmbeta);
      ub = h.normfact*(t1u+t2u*h.expmbeta);
      return;
    }
    lb = h.normfact*t1l;
    ub = h.normfact*t1u;
  }

  // FreeGasSampler::sampleBeta, NCFreeGasUtils.cc:530-849
  static __device__ __noinline__ double fgSampleBeta( const FGSampler& s, const double* tab, ncgb_rng& rng, int& st )
  {
    if ( s.c_real > 1e4 ) {
      const double A = 1.0 / s.invA;
      const double A2 = A*A;
      const double thr = 1e4 * ( 1000.0*A < A2*A2*A2 ? 1000.0*A : A2*A2*A2 );
      if ( s.c_real > thr ) {
        const double am1_div_ap1 = (1.0-s.invA)/(1.0+s.invA);
        const double elossmax = s.c_real * (1.0-am1_div_ap1*am1_div_ap1);
        return -elossmax*rand01( rng );
      }
    }
    const double Tlim = 2.0;
    const double Tlim_k1 = 0.135335283236612691893999494972484403407;
    const double Tlim_k2 = 274./315.;
    const double fcutoff_limit = 1e-6;
    double aa = maxd( -s.c_real, -s.c ), bb = 13.815510557964274;
    if ( s.invA <= 1.0/10.0 ) {
      if ( s.c > 10.1 ) {
        for ( int it = 0; it < 4000; ++it ) {
          const double aa_new = aa*0.2;
          if ( aa_new > -1e-99 )
            break;
          FGBetaEval h;
          fgBetaInit( h, s, aa_new );
          if ( fgBetaExact( h ) > fcutoff_limit )
            break;
          aa = aa_new;
        }
      }
      for ( int it = 0; it < 4000; ++it ) {
        const double bb_new = bb*0.25;
        if ( bb_new < 1e-99 )
          break;
        FGBetaEval h;
        double lb, ub;
        fgBetaInit( h, s, bb_new );
        fgBetaBounds( h, tab, lb, ub );
        if ( ub > fcutoff_limit )
          break;
        bb = bb_new;
      }
    }
    if ( !( bb > aa ) )
      return aa;
    double a = 0, b = 0, prob_downscat = 0, prob_notclosetail = 0;
    FGExpInt es;
    es.a = es.c1 = es.c2 = 0.0;
    bool es_valid = false;
    auto setAB = [&]( double aaa, double bbb ) {
      a = aaa; b = bbb;
      const double area_downscat = -a;
      double area_fartail, area_closetail;
      if ( b <= Tlim ) {
        area_fartail = 0.0;
        area_closetail = b * (1.0+b*(-1./2.+b*(1./6.+b*(-1./24.+b*(1./120.+b*(-1./720.+b*(1./5040.)))))));
      } else {
        area_fartail = Tlim_k1 - exp( -b );
        area_closetail = Tlim_k2;
      }
      const double invareatot = 1.0 / ( area_downscat + area_closetail + area_fartail );
      prob_downscat = area_downscat * invareatot;
      prob_notclosetail = ( area_fartail + area_downscat ) * invareatot;
      es_valid = false;
    };
    setAB( aa, bb );
    const double fthreshold = 0.1;
    double afthreshold = a, bfthreshold = b;
    for ( int it = 0; it < kFGLoopCap; ++it ) {
      double beta, foverlay = 1.0;
      const double Rsel = rand01( rng );
      if ( Rsel < prob_downscat ) {
        beta = rand01( rng )*a;
        foverlay = 1.0;
      } else if ( Rsel < prob_notclosetail ) {
        if ( !es_valid ) { fgExpIntSet( es, Tlim, b, 1.0 ); es_valid = true; }
        beta = fgExpIntSample( es, rng );
        foverlay = exp( -beta );
      } else {
        const double bmax = b < Tlim ? b : Tlim;
        bool got = false;
        beta = 0.0;
        for ( int jt = 0; jt < kFGLoopCap; ++jt ) {
          beta = rand01( rng )*bmax;
          const double R0 = rand01( rng );
          if ( R0 > 1.0 - (19./45.)*beta )
            continue;
          foverlay = 1.0+beta*(-1.+beta*(1./2.+beta*(-1./6.+beta*(1./24.+beta*(-1./120.+beta*(1./720.))))));
          if ( R0 < foverlay ) { got = true; break; }
        }
        if ( !got ) { st = NCGB_ST_LOOPCAP; return 0.0; }
      }
      const double faccept = rand01( rng )*foverlay;
      if ( faccept > fthreshold && !inInterval( afthreshold, bfthreshold, beta ) )
        continue;
      FGBetaEval h;
      fgBetaInit( h, s, beta );
      bool need_exact = true;
      double fval = 0.0;
      if ( beta > 0 ) {
        double lb, ub;
        fgBetaBounds( h, tab, lb, ub );
        if ( faccept <= lb )
          return beta;
        fval = ub;
        if ( faccept > ub )
          need_exact = false;
      }
      if ( need_exact ) {
        fval = fgBetaExact( h );
        if ( faccept < fval )
          return beta;
      }
      if ( fval < fcutoff_limit ) {
        if ( beta < 0 ) setAB( beta, b ); else setAB( a, beta );
        continue;
      }
      if ( fval < fthreshold ) {
        if ( beta < 0 )
          afthreshold = maxd( afthreshold, beta );
        else
          bfthreshold = bfthreshold < beta ? bfthreshold : beta;
      }
    }
    st = NCGB_ST_LOOPCAP;
    return 0.0;
  }

  // FreeGasSampler::sampleAlpha, NCFreeGasUtils.cc:851-932
  static __device__ __noinline__ double fgSampleAlpha( const FGSampler& s, double beta, ncgb_rng& rng, int& st )
  {
    if ( s.c_real < s.c || beta <= s.c * ( -1.0 + 1e-14 ) ) {
      const ALim al = alphaLimits( s.c_real, beta );
      const double alpha = al.lo + rand01( rng )*(al.hi-al.lo);
      return clampd( alpha, al.lo, al.hi );
    }
    beta = maxd( -s.c, beta );
    const ALim al = alphaLimits( s.c, beta );
    const double am = al.lo, ap = al.hi;
    if ( am == ap )
      return am;
    const double betasq = beta*beta;
    const double t = betasq * s.Adiv4;
    const double c = 0.0625 * betasq;
    if ( ( t < c ? t : c ) < 1e-5 ) {
      const double fourA = s.Adiv4*16.0;
      const double inv4A = 1.0/fourA;
      const double xxm = am*inv4A, xxp = ap*inv4A;
      for ( int it = 0; it < kFGLoopCap; ++it ) {
        const double xx = fgRandExpDivSqrt( rng, 1.0, xxm, xxp, st );
        if ( st != NCGB_ST_OK )
          return am;
        const double alpha = xx * fourA;
        if ( alpha < am || alpha > ap )
          continue;
        if ( alpha*ap*( -log( rand01( rng ) ) ) >= t*(ap-alpha) )
          return alpha;
      }
      st = NCGB_ST_LOOPCAP;
      return am;
    }
    const double invt = 1.0/t;
    const double x = fgRandEMix( rng, c, am*invt, ap*invt, st );
    return clampd( x*t, am, ap );
  }

  // FreeGasSampler::sampleAlphaBeta (NCFreeGasUtils.hh:132-144)
  __device__ __forceinline__ void fgSampleAlphaBeta( const FGSampler& s, const double* tab, ncgb_rng& rng,
                                                     double& alpha, double& beta, int& st )
  {
    const double b = fgSampleBeta( s, tab, rng, st );
    beta = b;
    if ( st != NCGB_ST_OK )
      return;
    if ( b < -s.c || b <= s.c * ( -1.0 + 1e-14 ) ) {
      const ALim al = alphaLimits( s.c_real, b );
      const double a = al.lo+rand01( rng )*(al.hi-al.lo);
      alpha = clampd( a, al.lo, al.hi );
      return;
    }
    alpha = fgSampleAlpha( s, b, rng, st );
  }

  // FreeGas::sampleScatterIsotropic (NCFreeGas.cc:70-75) via
  // FreeGasSampler::sampleDeltaEMu (NCFreeGasUtils.hh:146-161).
  static __device__ __noinline__ int freeGasScatter( const ncgb_freegas_view& v, const double* tab, ncgb_rng& rng,
                                              double ekin, double& ef, double& mu )
  {
    FGSampler s;
    fgInit( s, ekin, v.kT, v.mass_amu );
    int st = NCGB_ST_OK;
    const double beta = fgSampleBeta( s, tab, rng, st );
    if ( st != NCGB_ST_OK )
      return st;
    double dE, muv;
    if ( beta <= -s.c || beta <= s.c * ( -1.0 + 1e-14 ) ) {
      dE = beta*s.kT;
      muv = rand01( rng )*2.0-1.0;
    } else {
      const double alpha = fgSampleAlpha( s, beta, rng, st );
      if ( st != NCGB_ST_OK )
        return st;
      st = alphaBetaToDeltaEMu( alpha, beta, s.c*s.kT, s.kT, dE, muv );
      if ( st != NCGB_ST_OK )
        return st;
    }
    ef = maxd( 0.0, ekin + dE );
    mu = muv;
    return NCGB_ST_OK;
  }

  // SABSampler::sampleHighE, NCSABSampler.cc:59-156.  Returns 1 with (alpha,
  // beta) from the extender, 0 if the table must be sampled at E = Emax, or a
  // negative value on failure (-1: the reference's BadInput, -2: loop cap).
  static __device__ __noinline__ int sabHighE( const ncgb_sab_view& s, const double* tab, double ekin, ncgb_rng& rng,
                                        double& alpha, double& beta )
  {
    const double emax = ldg( s.egrid + s.ne - 1 );
    const double extE = ekin * ( s.ext_sigma_free * freeGasShape( s.ext_ca * ekin ) );
    const double P_inside = s.k1 / ( ( s.k1 - s.k2 ) + extE );
    const double P_ext_inside = s.k2 / extE;
    const double P_discard = ( P_ext_inside >= P_inside ? ( 1.0 - P_inside/P_ext_inside ) : 0.0 );
    if ( P_discard > 0.95 )
      return -1;
    if ( P_ext_inside < P_inside ) {
      const double aa = 1.0 - P_ext_inside;
      const double P_extra = aa > 1e-10 ? ( P_inside - P_ext_inside ) / aa : 1.0;
      if ( rand01( rng ) < P_extra )
        return 0;
    }
    const double emax_div_kt = emax / s.kT;
    FGSampler fs;
    fgInit( fs, ekin, s.ext_kT, s.ext_mass_amu );
    for ( int it = 0; it < kFGLoopCap; ++it ) {
      double a, b;
      int st = NCGB_ST_OK;
      fgSampleAlphaBeta( fs, tab, rng, a, b, st );
      if ( st != NCGB_ST_OK )
        return -2;
      if ( b <= -emax_div_kt ) { alpha = a; beta = b; return 1; }
      const ALim al = alphaLimits( emax_div_kt, b );
      if ( !inInterval( al.lo, al.hi, a ) ) { alpha = a; beta = b; return 1; }
      if ( P_discard && rand01( rng ) < P_discard )
        continue;
      return 0;
    }
    return -2;
  }
}

#endif
