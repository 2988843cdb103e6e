// Tables of the learned beta proposal (no counterpart in NCrystal).
//
// The plain sampler of an egrid point (SABSamplerAtE_Alg1::sampleAlphaBeta,
// NCSABSamplerModels.cc:48-155) draws beta from a PointwiseDist: a
// piecewise-linear density y on the points bx (NCPointwiseDist.cc:76-110).
// When bx[0] is a kinematic endpoint (fbkep <= 0) its first bin is special-
// cased; every other bin continues with the alpha sampling of the two beta
// rows around it.  The learned proposal replaces the percentile inversion of
// the regular range [bx[fr], bx[n-1]] (fr = 1 if the first bin is special,
// else 0) by rejection sampling from a piecewise-constant envelope:
//
//   * the network predicts 62 quantiles of beta (levels 1/63 .. 62/63); with
//     the range ends they give a piecewise-constant density estimate
//     d_i = (1/63)/w_i on 63 intervals of widths w_i;
//   * the envelope's K = 126 intervals [q_k, q_k+1] split the range into
//     equal parts of the integral of sqrt(d): for a smooth density f, the area
//     a piecewise-constant envelope wastes on an interval of width w is about
//     |f'| w^2 / 2, which intervals of equal |f'| w^2 minimise, and |f'| ~ f
//     on the exponential tails of S(alpha,beta), so w ~ f^(-1/2);
//   * envelope height env_k = max of y over interval k (y is linear between bx
//     points, so the maximum is at an interval end or at a bx point inside),
//     times 1 + 1e-5 and rounded up to FP32, which covers the FP32 evaluation
//     of y in the acceptance test;
//   * interval k drawn with probability env_k (q_k+1 - q_k) / sum (alias
//     table), beta = q_k + (2w+1) h_k uniform in it for a 32-bit draw w,
//     accepted with probability y(beta) / env_k.  y is evaluated in FP32 from
//     the linear pieces of the interval expressed in w (the piece boundaries
//     are the smallest w whose FP64 beta reaches each bx point, so a piece's
//     bin is exactly the bin of beta): a proposal uses integer and FP32
//     arithmetic only, and FP64 just for beta once it is accepted.
//
// Accepted values follow y on the regular range exactly, whatever the knots;
// the knots only set the acceptance ratio (integral of y) / (integral of the
// envelope).  Egrid points whose ratio is below a threshold keep the plain
// inversion.

#include "ncgb_proposal.hh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace ncgb {

  namespace {

    // largest j in [jlo, jhi] with bx[j] <= x (bx[jlo] <= x assumed)
    int64_t binOf( const double* bx, int64_t jlo, int64_t jhi, double x )
    {
      while ( jlo < jhi ) {
        const int64_t mid = ( jlo + jhi + 1 ) / 2;
        if ( bx[mid] <= x )
          jlo = mid;
        else
          jhi = mid - 1;
      }
      return jlo;
    }

    double yAt( const double* bx, const double* by, int64_t j, double x )
    {
      const double dx = bx[j + 1] - bx[j];
      if ( !( dx > 0.0 ) )
        return std::max( by[j], by[j + 1] );
      const double t = std::min( 1.0, std::max( 0.0, ( x - bx[j] ) / dx ) );
      return by[j] + ( by[j + 1] - by[j] ) * t;
    }

    // beta of draw w on an interval (the device's arithmetic)
    double betaOf( uint32_t w, double q, double h ) { return std::fma( (double)( 2ull * w + 1ull ), h, q ); }

    // smallest draw w with betaOf(w) >= x (4294967296 if none)
    uint64_t firstDraw( double x, double q, double h )
    {
      double g = std::ceil( ( ( x - q ) / h - 1.0 ) * 0.5 );
      int64_t w = g < 0.0 ? 0 : ( g > 4294967295.0 ? 4294967295 : (int64_t)g );
      while ( w > 0 && betaOf( (uint32_t)( w - 1 ), q, h ) >= x )
        --w;
      while ( w <= 4294967295LL && betaOf( (uint32_t)w, q, h ) < x )
        ++w;
      return (uint64_t)w;
    }

    float roundUpF( double v )
    {
      float f = static_cast<float>( v );
      if ( static_cast<double>( f ) < v )
        f = std::nextafter( f, std::numeric_limits<float>::infinity() );
      return f;
    }

    // Vose's alias method over K weights.
    void aliasTable( const double* w, int K, ncgb_lp_slot* cell )
    {
      double tot = 0.0;
      for ( int k = 0; k < K; ++k )
        tot += w[k];
      std::vector<double> p( K );
      std::vector<int> small, large;
      for ( int k = 0; k < K; ++k ) {
        p[k] = w[k] * K / tot;
        ( p[k] < 1.0 ? small : large ).push_back( k );
      }
      for ( int k = 0; k < K; ++k ) {
        cell[k].aprob = 1.0f;
        cell[k].alias = k;
      }
      while ( !small.empty() && !large.empty() ) {
        const int s = small.back(); small.pop_back();
        const int l = large.back();
        cell[s].aprob = static_cast<float>( p[s] );
        cell[s].alias = l;
        p[l] -= 1.0 - p[s];
        if ( p[l] < 1.0 ) {
          large.pop_back();
          small.push_back( l );
        }
      }
      // leftovers (rounding) keep probability 1 -- but never for a zero weight
      for ( int k = 0; k < K; ++k )
        if ( w[k] <= 0.0 && cell[k].alias == k ) {
          int best = 0;
          for ( int j = 1; j < K; ++j )
            if ( w[j] > w[best] ) best = j;
          cell[k].aprob = 0.0f;
          cell[k].alias = best;
        }
    }
  }

  Proposal buildProposal( const ncgb_sab_view& s, const float* knots, int nknots, const unsigned char* allowed,
                          double min_accept )
  {
    if ( nknots != NCGB_LP_NKNOTS )
      throw Error( "learned proposal: expected 62 knots per egrid point" );
    const int K = NCGB_LP_K;
    const int NQ = NCGB_LP_NKNOTS + 1;   // intervals of the network's quantiles
    const int64_t ne = s.ne;
    Proposal P;
    P.hdr.assign( ne, ncgb_lp_hdr{ 0.0, 0u, 0.0f, 0, 0 } );
    P.slot.assign( ne * K, ncgb_lp_slot{ 1.0f, 0 } );
    P.cell.assign( ne * K, ncgb_lp_cell{ 0.0, 0.0, 0.0f, 0, 0, 0 } );
    P.seg.reserve( 1024 );
    std::vector<double> q( K + 1 ), w( K ), nq( NQ + 1 ), cm( NQ + 1 );
    for ( int64_t ie = 0; ie < ne; ++ie ) {
      if ( s.smp_kind[ie] == 0 || ( allowed && !allowed[ie] ) )
        continue;
      const int64_t off = s.smp_offset[ie];
      const int64_t n = s.smp_nbeta[ie];
      const double* bx = s.bx + off;
      const double* by = s.by + off;
      const double* bcdf = s.bcdf + off;
      const int64_t fr = ( s.smp_fbkep[ie] <= 0.0 ) ? 1 : 0;
      if ( n < fr + 2 )
        continue;
      const double lo = bx[fr], hi = bx[n - 1];
      if ( !( hi > lo ) )
        continue;
      const double c1 = fr ? bcdf[1] : 0.0;
      const double mass = bcdf[n - 1] - bcdf[fr];
      if ( !( mass > 0.0 ) )
        continue;
      // the network's quantiles, clamped into the range and made monotone
      nq[0] = lo;
      nq[NQ] = hi;
      const float* g = knots + ie * nknots;
      for ( int k = 1; k < NQ; ++k ) {
        double v = std::sinh( static_cast<double>( g[k - 1] ) );
        if ( !std::isfinite( v ) )
          v = g[k - 1] < 0 ? lo : hi;
        v = std::min( hi, std::max( lo, v ) );
        nq[k] = std::max( nq[k - 1], v );
      }
      // cumulative integral of sqrt(d), d = (1/NQ)/w on each quantile interval
      cm[0] = 0.0;
      for ( int i = 0; i < NQ; ++i )
        cm[i + 1] = cm[i] + std::sqrt( std::max( 0.0, nq[i + 1] - nq[i] ) / NQ );
      q[0] = lo;
      q[K] = hi;
      int iq = 0;
      for ( int k = 1; k < K; ++k ) {
        const double level = cm[NQ] * k / K;
        while ( iq < NQ - 1 && cm[iq + 1] < level )
          ++iq;
        const double span = cm[iq + 1] - cm[iq];
        const double t = span > 0.0 ? std::min( 1.0, std::max( 0.0, ( level - cm[iq] ) / span ) ) : 0.0;
        q[k] = std::min( hi, std::max( q[k - 1], nq[iq] + t * ( nq[iq + 1] - nq[iq] ) ) );
      }
      ncgb_lp_cell* cell = &P.cell[ie * K];
      double tot = 0.0;
      int64_t jprev = binOf( bx, fr, n - 2, q[0] );
      for ( int k = 0; k < K; ++k ) {
        const int64_t j0 = jprev;
        const int64_t j1 = binOf( bx, j0, n - 2, q[k + 1] );
        const double width = q[k + 1] - q[k];
        const double h = width * 0x1p-33;
        cell[k].q = q[k];
        cell[k].h = h;
        // linear pieces of y over the interval, in the draw coordinate w
        cell[k].seg_lo = static_cast<int32_t>( P.seg.size() );
        for ( int64_t j = j0; j <= j1; ++j ) {
          const uint64_t w0 = ( j == j0 ) ? 0 : firstDraw( bx[j], q[k], h );
          if ( w0 > 4294967295ull )
            break;
          if ( j > j0 && !P.seg.empty() && P.seg.back().w0 == (uint32_t)w0 && (int64_t)P.seg.size() > cell[k].seg_lo )
            P.seg.pop_back();   // an empty piece: the next one starts at the same draw
          const double b0 = betaOf( (uint32_t)w0, q[k], h );
          const double dx = bx[j + 1] - bx[j];
          const double sl = dx > 0.0 ? ( by[j + 1] - by[j] ) / dx : 0.0;
          ncgb_lp_seg sg;
          sg.w0 = (uint32_t)w0;
          sg.y0 = static_cast<float>( by[j] + sl * ( b0 - bx[j] ) );
          sg.slope = static_cast<float>( sl * 2.0 * h );
          sg.bin = static_cast<int32_t>( j );
          P.seg.push_back( sg );
        }
        cell[k].seg_n = static_cast<int32_t>( P.seg.size() ) - cell[k].seg_lo;
        double ymax = 0.0;
        if ( width > 0.0 ) {
          ymax = std::max( yAt( bx, by, j0, q[k] ), yAt( bx, by, j1, q[k + 1] ) );
          for ( int64_t j = j0 + 1; j <= j1; ++j )
            ymax = std::max( ymax, by[j] );
        }
        const float env = ymax > 0.0 ? roundUpF( ymax * ( 1.0 + 1e-5 ) ) : 0.0f;
        cell[k].env = env;
        w[k] = width > 0.0 ? static_cast<double>( env ) * width : 0.0;
        tot += w[k];
        jprev = j1;
      }
      if ( !( tot > 0.0 ) )
        continue;
      const double accept = mass / tot;
      P.hdr[ie].c1 = c1;
      P.hdr[ie].c1_thr = static_cast<uint32_t>( std::min( 4294967295.0, std::floor( c1 * 4294967296.0 + 0.5 ) ) );
      P.hdr[ie].accept = static_cast<float>( accept );
      if ( accept < min_accept )
        continue;
      aliasTable( w.data(), K, &P.slot[ie * K] );
      P.hdr[ie].enabled = 1;
    }
    return P;
  }
}
