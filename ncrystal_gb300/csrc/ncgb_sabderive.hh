// Per-beta-row pieces of NCrystal's S(alpha,beta) table derivation, shared by
// the host table builder (ncgb_tables.cc, g++ -ffp-contract=off) and the
// device builder (ncgb_sabderive.cu, nvcc -fmad=false): the same source on
// both sides, so that the two agree to the last bit wherever no libm
// function (log, exp) is involved.
#ifndef NCGB_SABDERIVE_HH
#define NCGB_SABDERIVE_HH

#include <cfloat>
#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#  define NCGB_HD __host__ __device__
#else
#  define NCGB_HD
#endif

namespace ncgb {
  namespace sabd {

    NCGB_HD inline double dmin( double a, double b ) { return b < a ? b : a; }
    NCGB_HD inline double dmax( double a, double b ) { return a < b ? b : a; }

    // Neumaier summation (NCMath.hh:194-202, :526-536).
    struct StableSum {
      double s = 0.0, c = 0.0;
      NCGB_HD void add( double x )
      {
        double t = s + x;
        c += ( fabs(s) >= fabs(x) ) ? (s - t) + x : (x - t) + s;
        s = t;
      }
      NCGB_HD double sum() const { return s + c; }
    };

    // Kinematic alpha limits (NCKinUtils.hh:108-124 and :82-101).
    struct ALim { double lo, hi; };
    NCGB_HD inline ALim alphaLimits( double ekin_div_kT, double beta )
    {
      const double kk = ekin_div_kT + beta;
      if ( !( kk >= 0.0 ) )
        return { 1.0, -1.0 };
      const double a = kk + ekin_div_kT;
      const double b = 2.0 * sqrt( ekin_div_kT * kk );
      double aminus;
      if ( fabs(beta) < 0.01 * ekin_div_kT ) {
        const double x = beta / ekin_div_kT;
        constexpr double c9 = -715./32768.;
        constexpr double c8 = 429./16384.;
        constexpr double c7 = -33./1024.;
        constexpr double c6 = 21./512.;
        constexpr double c5 = -7./128.;
        constexpr double c4 = 5./64.;
        constexpr double c3 = - 1./8.;
        constexpr double c2 = 1./4.;
        aminus = beta*x*(c2+x*(c3+x*(c4+x*(c5+x*(c6+x*(c7+x*(c8+x*c9)))))));
      } else {
        aminus = dmax( 0.0, a - b );
      }
      return { aminus, a + b };
    }

    // NCSABUtils.hh:240-261
    NCGB_HD inline double integrateAlphaIntervalFast( double a1, double s1, double a2, double s2, double logs1,
                                                      double logs2 )
    {
      const double da = a2-a1;
      const double ps = s1+s2;
      const double ds = s2-s1;
      if ( dmin(s1,s2) < 1e-300 )
        return 0.5*da*ps;
      if ( fabs(ds) > 0.006*ps )
        return da*ds/(logs2-logs1);
      const double y = ds / ps;
      const double c1 = 0.166666666666666666666666666666666666666666667;
      const double c2 = 0.0444444444444444444444444444444444444444444444;
      const double c3 = 0.0232804232804232804232804232804232804232804233;
      const double ysq = y*y;
      return da*ps*(0.5-ysq*(c1+ysq*(c2+ysq*c3)));
    }

    // NCSABUtils.hh:180-199
    NCGB_HD inline double interpLogLinFast( double a, double fa, double b, double fb, double x, double logfa,
                                            double logfb )
    {
      const double bma = b - a;
      const double midpoint = 0.5 * ( b + a );
      const bool linlin_mode = ( fa*fb == 0.0 );
      if ( x < midpoint ) {
        const double r = (x-a) / bma;
        return ( linlin_mode ? ( fa + (fb-fa)*r ) : exp(logfa+(logfb-logfa)*r) );
      } else {
        const double s = (b-x) / bma;
        return ( linlin_mode ? ( fb + (fa-fb)*s ) : exp(logfb+(logfa-logfb)*s) );
      }
    }

    struct TailPoint { double alpha = 0.0, sval = 0.0, logsval = 0.0; };
    struct TailedBreakdown {
      double xs_front = 0.0, xs_middle = 0.0, xs_back = 0.0;
      unsigned imiddle_low = 0, imiddle_upp = 0;
      TailPoint front, back;
      bool narrow = false;
    };

    NCGB_HD inline void setTailPoint( TailPoint& tp, const double* alphaGrid, const double* sab, const double* logsab,
                                      unsigned aidx, double alpha )
    {
      tp.alpha = alpha;
      tp.sval = interpLogLinFast( alphaGrid[aidx], sab[aidx], alphaGrid[aidx+1], sab[aidx+1], alpha,
                                  logsab[aidx], logsab[aidx+1] );
      tp.logsval = log( dmax( tp.sval, DBL_MIN ) );
    }

    // NCSABUtils.cc:538-633.  Spans are the beta row of alpha/S/logS/cumul.
    NCGB_HD inline TailedBreakdown tailedBreakdown( const double* alphaGrid, unsigned na, const double* sab,
                                                    const double* logsab, const double* cumul, double alpha_low,
                                                    double alpha_upp, unsigned aidx_low, unsigned aidx_upp )
    {
      alpha_low = dmin( dmax( alpha_low, alphaGrid[0] ), alphaGrid[na-1] );
      alpha_upp = dmin( dmax( alpha_upp, alphaGrid[0] ), alphaGrid[na-1] );
      TailedBreakdown tb;
      if ( aidx_low == aidx_upp || alpha_low == alpha_upp )
        return tb;
      if ( aidx_low + 1 == aidx_upp ) {
        tb.narrow = true;
        setTailPoint( tb.front, alphaGrid, sab, logsab, aidx_low, alpha_low );
        setTailPoint( tb.back, alphaGrid, sab, logsab, aidx_low, alpha_upp );
        tb.xs_front = integrateAlphaIntervalFast( tb.front.alpha, tb.front.sval, tb.back.alpha, tb.back.sval,
                                                  tb.front.logsval, tb.back.logsval );
        return tb;
      }
      tb.imiddle_low = aidx_low;
      tb.imiddle_upp = aidx_upp;
      if ( alpha_low >= alphaGrid[aidx_low] ) {
        setTailPoint( tb.front, alphaGrid, sab, logsab, aidx_low, alpha_low );
        tb.xs_front = integrateAlphaIntervalFast( tb.front.alpha, tb.front.sval,
                                                  alphaGrid[aidx_low+1], sab[aidx_low+1],
                                                  tb.front.logsval, logsab[aidx_low+1] );
        ++tb.imiddle_low;
      }
      if ( alpha_upp <= alphaGrid[aidx_upp] ) {
        setTailPoint( tb.back, alphaGrid, sab, logsab, aidx_upp-1, alpha_upp );
        tb.xs_back = integrateAlphaIntervalFast( alphaGrid[aidx_upp-1], sab[aidx_upp-1],
                                                 tb.back.alpha, tb.back.sval,
                                                 logsab[aidx_upp-1], tb.back.logsval );
        --tb.imiddle_upp;
      }
      tb.xs_middle = ( tb.imiddle_upp > tb.imiddle_low
                       ? cumul[tb.imiddle_upp] - cumul[tb.imiddle_low]
                       : 0.0 );
      return tb;
    }

  }
}

#endif
