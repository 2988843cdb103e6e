/*
 * ncgb_oracle.c -- CPU oracle for the GPU scattering path.  TEST
 * INFRASTRUCTURE ONLY: tests, the smoke check and the CPU baseline leg of
 * bench.py use it to check (and time beside) the CUDA kernels.  The library in
 * ncrystal_gb300/ never calls it.
 *
 * A plain-C restatement of NCrystal's per-neutron evaluation of a
 * non-oriented material (NCrystal 4.4.2), one neutron at a time, on the flat
 * tables of include/ncgb_tables.h and the Philox streams of
 * include/ncgb_philox.h.  Every function cites the reference code it follows.
 *
 * Pinned against the reference library itself: oracle/refpin.c drives the
 * reference's own ncrystal_crosssection_nonoriented /
 * ncrystal_samplescatterisotropic with the same per-neutron Philox streams
 * (via ncrystal_setrandgen), and the tests require identical cross-sections,
 * identical numbers of random draws and identical (E', mu) per neutron.
 *
 * Status codes (per neutron): 0 ok; 1 a rejection loop hit its cap (the
 * reference throws CalcError, NCSABSampler.cc:226, NCSABSamplerModels.cc:150);
 * 2 free-gas sampling requested (not restated yet); 3 the reference throws
 * CalcError in convertAlphaBetaToDeltaEMu (E*E' == 0, NCKinUtils.cc:40-45).
 *
 * Built with -ffp-contract=off -O2 (no fast-math).
 */
#include <float.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include "ncgb_philox.h"
#include "ncgb_tables.h"

#define ORA_OK 0
#define ORA_LOOPCAP 1
#define ORA_UNSUPPORTED 2
#define ORA_CALCERROR 3

static const double ora_inf = INFINITY;

/* ---- small helpers ------------------------------------------------------- */

/* std::upper_bound / std::lower_bound on [a, a+n): first index with a[i] > x
 * (resp. a[i] >= x), n if none. */
static size_t ora_upper_bound( const double* a, size_t n, double x )
{
  size_t lo = 0, len = n;
  while ( len > 0 ) {
    size_t half = len / 2;
    if ( !( x < a[lo + half] ) ) { lo += half + 1; len -= half + 1; }
    else len = half;
  }
  return lo;
}

static size_t ora_lower_bound( const double* a, size_t n, double x )
{
  size_t lo = 0, len = n;
  while ( len > 0 ) {
    size_t half = len / 2;
    if ( a[lo + half] < x ) { lo += half + 1; len -= half + 1; }
    else len = half;
  }
  return lo;
}

static double ora_clamp( double x, double lo, double hi ) { return x < lo ? lo : ( x > hi ? hi : x ); }
static double ora_max( double a, double b ) { return a < b ? b : a; }

/* EnergyDomain::contains, NCTypes.hh:434: E in [elow, ehigh]. */
static int ora_contains( double elow, double ehigh, double e ) { return e >= elow && e <= ehigh; }

/* ---- kinematics (NCKinUtils.hh:64-124, NCKinUtils.cc:25-58) --------------- */

typedef struct { double lo, hi; } ora_alim;

static ora_alim ora_alpha_limits( double ekin_div_kT, double beta )
{
  ora_alim r;
  const double kk = ekin_div_kT + beta;
  if ( !( kk >= 0.0 ) ) { r.lo = 1.0; r.hi = -1.0; return r; }
  const double a = kk + ekin_div_kT;
  const double b = 2.0 * sqrt( ekin_div_kT * kk );
  if ( fabs( beta ) < 0.01 * ekin_div_kT ) {
    const double x = beta / ekin_div_kT;
    const double c9 = -715./32768., c8 = 429./16384., c7 = -33./1024., c6 = 21./512.;
    const double c5 = -7./128., c4 = 5./64., c3 = -1./8., c2 = 1./4.;
    r.lo = beta*x*(c2+x*(c3+x*(c4+x*(c5+x*(c6+x*(c7+x*(c8+x*c9)))))));
  } else {
    r.lo = ora_max( 0.0, a - b );
  }
  r.hi = a + b;
  return r;
}

static int ora_in_interval( double lo, double hi, double x ) { return x >= lo && x <= hi; }

static int ora_mu_isotropic_at_beta( double beta, double ekin_div_kT )
{
  const double lim = -1.0 + 1e-14;
  return beta <= ekin_div_kT * lim;
}

/* Neumaier sum of three terms (NCMath.hh:526-536), then clamp. */
static int ora_alphabeta_to_demu( double alpha, double beta, double ekin, double kT,
                                  double* deltaE, double* mu )
{
  *deltaE = beta * kT;
  const double ekinfinal = ekin + *deltaE;
  const double denom = 2.0 * sqrt( ekin * ekinfinal );
  if ( !denom )
    return ORA_CALCERROR;
  double s = 0.0, c = 0.0, t, x;
  x = ekin;        t = s + x; c += ( fabs(s) >= fabs(x) ) ? (s-t)+x : (x-t)+s; s = t;
  x = ekinfinal;   t = s + x; c += ( fabs(s) >= fabs(x) ) ? (s-t)+x : (x-t)+s; s = t;
  x = -alpha * kT; t = s + x; c += ( fabs(s) >= fabs(x) ) ? (s-t)+x : (x-t)+s; s = t;
  *mu = ora_clamp( ( s + c ) / denom, -1.0, 1.0 );
  return ORA_OK;
}

/* ---- cross-sections ------------------------------------------------------ */

/* NCElIncXS.cc:34-54 */
static double ora_1mexpmtdivt( double t )
{
  if ( t < 0.01 )
    return ( 1 + t * ( -0.5 + t * 0.16666666666666666666666666666666666666666667 * ( 1. - 0.25 * t ) ) );
  if ( t > 24.0 )
    return 1.0 / t;
  t = -t;
  return expm1( t ) / t;
}

/* ElIncXS::evalXSContribsCommul, NCElIncXS.cc:130-141.  Returns the total. */
static double ora_elinc_commul( const ncgb_elinc_view* v, double ekin, double* commul )
{
  const double kkk = 16.0 * 9.86960440108935861883449099987615113531369941 * 12.22430978582345950656;
  const double e = kkk * ekin;
  double xs = 0.0;
  for ( int i = 0; i < v->n; ++i ) {
    xs += v->sigma[i] * ora_1mexpmtdivt( v->msd[i] * e );
    if ( commul ) commul[i] = xs;
  }
  return xs;
}

/* PowderBragg::crossSectionIsotropic, NCPowderBragg.cc:152-176. */
static double ora_bragg_xs( const ncgb_bragg_view* v, double ekin, size_t* idx_out )
{
  if ( v->n == 0 || ekin < v->threshold || !isfinite( ekin ) )
    return 0.0;
  size_t idx = 1 + ora_upper_bound( v->two_dE + 1, (size_t)v->n - 1, ekin ) - 1;
  if ( idx_out ) *idx_out = idx;
  return v->fdm_commul[idx] * ( 1.0 / ekin );
}

/* FreeGasXSProvider::evalXSShapeASq, NCFreeGasUtils.cc:64-84. */
static double ora_freegas_shape( double a_squared )
{
  if ( a_squared > 36.0 )
    return 1.0 + 0.5 / a_squared;
  const double a = sqrt( a_squared );
  if ( a < 0.1 ) {
    if ( a == 0.0 )
      return ora_inf;
    const double c1 = 2.0/3.0, c2 = 1.0/15.0, c3 = 1.0/105.0, c4 = 1.0/756.0, c5 = 1.0/5940.0;
    const double a2 = a_squared;
    return 0.564189583547756286948079451560772585844050629 * ( 2.0 / a + a *( c1- a2*(c2-a2*(c3-a2*(c4-a2*c5)))));
  }
  const double inva = 1.0 / a;
  return ( 1.0 + 0.5*inva*inva ) * erf( a ) + 0.564189583547756286948079451560772585844050629 * exp( -a_squared ) * inva;
}

/* SABXSProvider::crossSection, NCSABXSProvider.cc:54-95, times the
 * SABScatter scale (NCSABScatter.cc:87-90). */
static double ora_sab_xs( const ncgb_sab_view* s, double ekin )
{
  const size_t ne = (size_t)s->ne;
  size_t iu = ora_upper_bound( s->egrid, ne, ekin );
  double xs;
  if ( iu == ne ) {
    xs = s->kext / ekin + s->ext_sigma_free * ora_freegas_shape( s->ext_ca * ekin );
  } else if ( iu == 0 ) {
    xs = ekin > 0.0 ? sqrt( s->egrid[0] / ekin ) * s->xs[0] : ora_inf;
  } else {
    const size_t il = iu - 1;
    const double dXS = s->xs[iu] - s->xs[il];
    const double dEkin = s->egrid[iu] - s->egrid[il];
    xs = s->xs[il] + dXS * ( ekin - s->egrid[il] ) / dEkin;
  }
  return xs * s->internal_scale;
}

/* Component cross-section (without domain check). */
static double ora_comp_xs( const ncgb_comp_view* c, double ekin )
{
  switch ( c->type ) {
    case NCGB_COMP_ELINC: return ora_elinc_commul( &c->elinc, ekin, NULL );
    case NCGB_COMP_BRAGG: return ora_bragg_xs( &c->bragg, ekin, NULL );
    case NCGB_COMP_SAB: return ora_sab_xs( &c->sab, ekin );
    case NCGB_COMP_FREEGAS: return c->fg.sigma_free * ora_freegas_shape( c->fg.ca * ekin );
    default: return 0.0;
  }
}

/* ProcComposition::updateCacheIsotropic (NCProcImpl.cc:166-204); returns the
 * total and fills the cumulative per-component cross-sections. */
static double ora_xs_commul( const ncgb_material_view* m, double ekin, double* commul )
{
  double tot = 0.0;
  for ( int i = 0; i < m->ncomp; ++i ) {
    const ncgb_comp_view* c = &m->comp[i];
    double xs = ora_contains( c->elow, c->ehigh, ekin ) ? ora_comp_xs( c, ekin ) : 0.0;
    commul[i] = ( tot += ( c->scale * xs ) );
  }
  return tot;
}

/* ProcComposition::crossSectionIsotropic (NCProcImpl.cc:353-362). */
double ncgb_oracle_xs( const ncgb_material_view* m, double ekin )
{
  double commul[NCGB_MAX_COMP];
  if ( !ora_contains( m->dom_elow, m->dom_ehigh, ekin ) )
    return 0.0;
  return ora_xs_commul( m, ekin, commul );
}

/* pickRandIdxByWeight (NCRandUtils.hh:130-133, NCRandUtils.cc:198-222). */
static size_t ora_pick( ncgb_rng* rng, const double* commul, size_t n )
{
  if ( n == 1 )
    return 0;
  const double r = ncgb_rng_generate( rng );
  if ( n < 5 ) {
    const double rand_choice = commul[n-1] * r;
    for ( size_t i = 0; i < n; ++i )
      if ( commul[i] > rand_choice )
        return i;
    return n - 1;
  }
  size_t i = ora_lower_bound( commul, n, commul[n-1] * r );
  return i < n - 1 ? i : n - 1;
}

/* ---- samplers ------------------------------------------------------------ */

/* PowderBragg::genScatterMu, NCPowderBragg.cc:178-200. */
static double ora_bragg_mu( const ncgb_bragg_view* v, ncgb_rng* rng, double ekin, size_t idx )
{
  const double r = ncgb_rng_generate( rng );
  size_t k = ora_lower_bound( v->fdm_commul, idx, r * v->fdm_commul[idx] );
  return 1.0 - 2.0 * ( v->two_dE[k] / ekin );
}

/* exp_smallarg_approx, NCMath.hh:434-440 */
static double ora_exp_small( double x )
{
  return 1.0+x*(1+x*(0.5+x*(0.16666666666666666666666666666666666667+x*(0.04166666666666666666666666666666666667
           +x*(0.00833333333333333333333333333333333333+x*(0.00138888888888888888888888888888888889
           +x*0.00019841269841269841269841269841269841))))));
}

/* ElIncXS::sampleMuMonoAtomic, NCElIncXS.cc:81-115. */
static double ora_elinc_mu_mono( ncgb_rng* rng, double ekin, double msd )
{
  const double kkk = 8.0 * 9.86960440108935861883449099987615113531369941 * 12.22430978582345950656;
  const double twoksq = kkk * ekin;
  const double a = twoksq * msd;
  if ( a < 0.01 ) {
    const double maxval = ora_exp_small( a );
    for (;;) {
      const double mu = ncgb_rng_generate( rng ) * 2.0 - 1.0;
      if ( ncgb_rng_generate( rng ) * maxval < ora_exp_small( a * mu ) )
        return mu;
    }
  }
  return ora_clamp( log1p( ncgb_rng_generate( rng ) * expm1( 2.0 * a ) ) / a - 1.0, -1.0, 1.0 );
}

/* ElIncXS::EPointAnalysis::sampleMu, NCElIncXS.cc:178-191. */
static double ora_elinc_mu( const ncgb_elinc_view* v, ncgb_rng* rng, double ekin )
{
  if ( v->n == 1 )
    return ora_elinc_mu_mono( rng, ekin, v->msd[0] );
  double commul[NCGB_MAX_ELINC];
  ora_elinc_commul( v, ekin, commul );
  size_t i = ora_pick( rng, commul, (size_t)v->n );
  return ora_elinc_mu_mono( rng, ekin, v->msd[i] );
}

/* PointwiseDist::percentileWithIndex, NCPointwiseDist.cc:76-110, on the
 * sampler's (x, y, cdf) of length n. */
static double ora_percentile( const double* x, const double* y, const double* cdf, size_t n,
                              double p, size_t* bin )
{
  if ( p == 1.0 ) { *bin = n - 2; return x[n-1]; }
  size_t i = ora_lower_bound( cdf, n, p );
  if ( i > n - 1 ) i = n - 1;
  if ( i < 1 ) i = 1;
  const double dx = x[i] - x[i-1];
  const double c = ( p - cdf[i-1] );
  const double a = y[i-1];
  const double d = y[i] - a;
  double zdx;
  if ( !a ) {
    zdx = d > 0.0 ? sqrt( ( 2.0 * c * dx ) / d ) : 0.5 * dx;
  } else {
    const double e = d * c / ( dx * a * a );
    if ( fabs( e ) > 1e-7 )
      zdx = ( sqrt( 1.0 + 2.0 * e ) - 1.0 ) * dx * a / d;
    else
      zdx = ( 1 + 0.5 * e * ( e - 1.0 ) ) * c / a;
  }
  *bin = i - 1;
  return ora_clamp( x[i-1] + zdx, x[i-1], x[i] );
}

/* SABUtils::sampleLogLinDist_fast, NCSABUtils.hh:282-304. */
static double ora_loglin( double a, double fa, double b, double fb, double rnd, double logfa, double logfb )
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

static double ora_clamp_rand( double r ) { return ora_clamp( r, DBL_MIN, 1.0 ); }

/* SABSamplerAtE_Alg1::sampleAlpha, NCSABSamplerModels.cc:157-234. */
static double ora_sample_alpha( const ncgb_sab_view* s, int64_t ie, size_t ibeta, double rp )
{
  const int64_t ioff = s->smp_ibetaoffset[ie];
  const ncgb_alpha_info* info = &s->info[ s->smp_offset[ie] + ( (int64_t)ibeta - ioff ) ];
  const size_t na = (size_t)s->na;
  const double* cumul = s->cumul + ibeta * na;
  const double* sab = s->sab + ibeta * na;
  const double* logsab = s->logsab + ibeta * na;
  const double* ag = s->alpha;
  if ( rp <= info->prob_front ) {
    if ( info->prob_front == 2.0 ) {
      const double da = info->back_alpha - info->front_alpha;
      return info->front_alpha + rp * da;
    } else if ( info->prob_front == 1.0 ) {
      return ora_loglin( info->front_alpha, info->front_sval, info->back_alpha, info->back_sval,
                         rp, info->front_logsval, info->back_logsval );
    } else {
      const double p2 = ora_clamp_rand( rp / info->prob_front );
      return ora_loglin( info->front_alpha, info->front_sval, ag[info->front_idx], sab[info->front_idx],
                         p2, info->front_logsval, logsab[info->front_idx] );
    }
  } else if ( rp <= info->prob_notback ) {
    const double p2 = ora_clamp( ( rp - info->prob_front ) / ( info->prob_notback - info->prob_front ), 0.0, 1.0 );
    const size_t il = info->front_idx, iu = info->back_idx;
    const double sel = cumul[il] + p2 * ( cumul[iu] - cumul[il] );
    /* upper_bound over [il, iu+1) */
    size_t e = il + ora_upper_bound( cumul + il, iu + 1 - il, sel );
    if ( e > iu )
      return ag[iu];
    if ( e <= il )
      return ag[il];
    const size_t a0 = e - 1, a1 = e;
    const double binArea = cumul[e] - cumul[a0];
    const double rr = ora_clamp_rand( ( sel - cumul[a0] ) / binArea );
    return ora_loglin( ag[a0], sab[a0], ag[a1], sab[a1], rr, logsab[a0], logsab[a1] );
  } else {
    const double p2 = ora_clamp_rand( ( rp - info->prob_notback ) / ( 1.0 - info->prob_notback ) );
    return ora_loglin( ag[info->back_idx], sab[info->back_idx], info->back_alpha, info->back_sval,
                       p2, logsab[info->back_idx], info->back_logsval );
  }
}

/* SABSamplerAtE_Alg1::sampleAlphaBeta, NCSABSamplerModels.cc:48-155.
 * Returns ORA_OK or ORA_LOOPCAP. */
static int ora_alg1( const ncgb_sab_view* s, int64_t ie, double ekin_div_kT, ncgb_rng* rng,
                     double* alpha_out, double* beta_out )
{
  const int64_t off = s->smp_offset[ie];
  const size_t nbs = (size_t)s->smp_nbeta[ie];
  const double* bx = s->bx + off;
  const double* by = s->by + off;
  const double* bcdf = s->bcdf + off;
  const size_t ioff = (size_t)s->smp_ibetaoffset[ie];
  const double fbkep = s->smp_fbkep[ie];
  const double* bg = s->beta;
  for ( int iloop = 0; iloop < 100; ++iloop ) {
    size_t ibs;
    double beta = ora_percentile( bx, by, bcdf, nbs, ncgb_rng_generate( rng ), &ibs );
    if ( ibs == 0 && fbkep <= 0.0 ) {
      const double b0 = fbkep;
      const double b1 = bx[1];
      if ( b1 < -ekin_div_kT )
        continue;
      const double delta_beta = b1 - b0;
      double alphaval = 0.0;
      for ( int iii = 0; iii < 30; ++iii ) {
        beta = ora_max( fbkep, b0 + delta_beta * ncgb_rng_generate( rng ) );
        if ( beta < -ekin_div_kT )
          break;
        alphaval = ora_sample_alpha( s, ie, ioff, ncgb_rng_generate( rng ) );
        ora_alim al = ora_alpha_limits( -fbkep, beta );
        if ( ora_in_interval( al.lo, al.hi, alphaval ) )
          break;
        if ( iii == 29 ) {
          alphaval = 0.5 * ( al.lo + al.hi );
          break;
        }
      }
      if ( beta < -ekin_div_kT )
        continue;
      ora_alim al2 = ora_alpha_limits( ekin_div_kT, beta );
      if ( ora_in_interval( al2.lo, al2.hi, alphaval ) ) {
        *alpha_out = alphaval; *beta_out = beta; return ORA_OK;
      }
      continue;
    }
    if ( beta <= ora_max( -ekin_div_kT, bg[0] ) )
      continue;
    const double rp = ncgb_rng_generate( rng );
    const size_t ibeta = ioff + ibs;
    const double bl = bg[ibeta-1];
    const double alphal = ora_sample_alpha( s, ie, ibeta - 1, rp );
    const double bh = bg[ibeta];
    const double alphah = ora_sample_alpha( s, ie, ibeta, rp );
    const double alpha = alphal + ( alphah - alphal ) * ( beta - bl ) / ( bh - bl );
    ora_alim al = ora_alpha_limits( ekin_div_kT, beta );
    if ( ora_in_interval( al.lo, al.hi, alpha ) ) {
      *alpha_out = alpha; *beta_out = beta; return ORA_OK;
    }
  }
  return ORA_LOOPCAP;
}

/* SABSampler::sampleAlphaBeta + sampleDeltaEMu, NCSABSampler.cc:158-236,
 * and SABScatter::sampleScatterIsotropic, NCSABScatter.cc:92-101. */
static int ora_sab_scatter( const ncgb_sab_view* s, ncgb_rng* rng, double ekin, double* ef, double* mu )
{
  const size_t ne = (size_t)s->ne;
  size_t iu = ora_upper_bound( s->egrid, ne, ekin );
  int ultra_small = 0;
  int64_t ie;
  if ( iu == ne ) {
    return ORA_UNSUPPORTED; /* E >= Emax: free-gas extender sampling (NCSABSampler.cc:59-156) */
  } else if ( iu == 0 ) {
    ie = 0;
    ultra_small = ( ekin < s->egrid[0] );
  } else {
    if ( s->egrid_margin > 1.0 ) {
      while ( iu + 1 != ne && ekin * s->egrid_margin > s->egrid[iu] )
        ++iu;
    }
    ie = (int64_t)iu;
  }
  const double ekin_div_kT = ekin / s->kT;
  const double sampling_ekin_div_kT = ultra_small ? s->egrid[0] / s->kT : ekin_div_kT;
  double alpha = 0.0, beta = 0.0;
  int found = 0;
  for ( int loop = 0; loop < 100; ++loop ) {
    if ( s->smp_kind[ie] == 0 ) {
      alpha = 0.0; beta = 0.0;
    } else {
      int st = ora_alg1( s, ie, sampling_ekin_div_kT, rng, &alpha, &beta );
      if ( st != ORA_OK )
        return st;
    }
    if ( beta < -ekin_div_kT )
      continue;
    ora_alim al = ora_alpha_limits( ekin_div_kT, beta );
    if ( ora_in_interval( al.lo, al.hi, alpha ) ) { found = 1; break; }
    if ( ultra_small ) {
      alpha = al.lo + ncgb_rng_generate( rng ) * ( al.hi - al.lo );
      found = 1;
      break;
    }
  }
  if ( !found )
    return ORA_LOOPCAP;
  double deltaE, muv;
  if ( ora_mu_isotropic_at_beta( beta, ekin / s->kT ) ) {
    deltaE = beta * s->kT;
    muv = ncgb_rng_generate( rng ) * 2.0 - 1.0;
  } else {
    int st = ora_alphabeta_to_demu( alpha, beta, ekin, s->kT, &deltaE, &muv );
    if ( st != ORA_OK )
      return st;
  }
  *ef = ora_max( 0.0, ekin + deltaE );
  *mu = muv;
  return ORA_OK;
}

/* ProcComposition::sampleScatterIsotropic, NCProcImpl.cc:379-389, and the
 * component samplers.  Returns a status code; on a non-zero status the outputs
 * hold (-1, -999) like the reference's samplescatterisotropic_many error
 * sentinels (ncrystal.cc:1237-1244). */
int ncgb_oracle_scatter( const ncgb_material_view* m, ncgb_rng* rng, double ekin, double* ef, double* mu )
{
  if ( !ora_contains( m->dom_elow, m->dom_ehigh, ekin ) ) {
    *ef = ekin; *mu = 1.0; return ORA_OK;
  }
  double commul[NCGB_MAX_COMP];
  ora_xs_commul( m, ekin, commul );
  const size_t ic = ora_pick( rng, commul, (size_t)m->ncomp );
  const ncgb_comp_view* c = &m->comp[ic];
  int st = ORA_OK;
  switch ( c->type ) {
    case NCGB_COMP_BRAGG: {
      /* PowderBragg::sampleScatterIsotropic, NCPowderBragg.cc:202-216 */
      size_t idx = 0;
      if ( c->bragg.n == 0 || ekin < c->bragg.threshold || !isfinite( ekin ) ) {
        *ef = ekin; *mu = 1.0;
      } else {
        ora_bragg_xs( &c->bragg, ekin, &idx );
        *ef = ekin; *mu = ora_bragg_mu( &c->bragg, rng, ekin, idx );
      }
      break;
    }
    case NCGB_COMP_ELINC:
      /* ElIncScatter::sampleScatterIsotropic, NCElIncScatter.cc:198-203 */
      *ef = ekin; *mu = ora_elinc_mu( &c->elinc, rng, ekin );
      break;
    case NCGB_COMP_SAB:
      st = ora_sab_scatter( &c->sab, rng, ekin, ef, mu );
      break;
    case NCGB_COMP_FREEGAS:
      st = ORA_UNSUPPORTED;
      break;
    default:
      *ef = ekin; *mu = 1.0;
  }
  if ( st != ORA_OK ) { *ef = -1.0; *mu = -999.0; }
  return st;
}

/* Batch helpers for the tests and the CPU baseline: neutron i uses the stream
 * (seed, i + index_offset, callseq, stream), like the CUDA kernels. */
void ncgb_oracle_xs_many( const ncgb_material_view* m, const double* ekin, int64_t n, double* out )
{
  for ( int64_t i = 0; i < n; ++i )
    out[i] = ncgb_oracle_xs( m, ekin[i] );
}

int64_t ncgb_oracle_scatter_many( const ncgb_material_view* m, const double* ekin, int64_t n,
                                  uint64_t seed, uint32_t index_offset, uint32_t callseq, uint32_t stream,
                                  double* out_ef, double* out_mu, int32_t* out_status, int32_t* out_ndraws )
{
  int64_t nbad = 0;
  for ( int64_t i = 0; i < n; ++i ) {
    ncgb_rng rng;
    ncgb_rng_init( &rng, seed, (uint32_t)( i + index_offset ), callseq, stream );
    int st = ncgb_oracle_scatter( m, &rng, ekin[i], &out_ef[i], &out_mu[i] );
    if ( out_status ) out_status[i] = st;
    if ( out_ndraws ) out_ndraws[i] = (int32_t)( 2 * rng.block - rng.have );
    if ( st ) ++nbad;
  }
  return nbad;
}
