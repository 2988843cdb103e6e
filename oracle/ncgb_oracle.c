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
 * 3 the reference throws CalcError in convertAlphaBetaToDeltaEMu (E*E' == 0,
 * NCKinUtils.cc:40-45) or BadInput in SABSampler::sampleHighE
 * (NCSABSampler.cc:121-122).
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

/* Learned beta proposal of sampler ie (tables of ncgb_proposal.cc; no
 * reference counterpart): interval from the alias table, a 32-bit draw w
 * placing beta = q + (2w+1) h in it, accepted with probability y/env, y from
 * the interval's linear pieces in w -- the same draws and arithmetic as the
 * GPU.  Returns 1 with (beta, bin) or 0 after 1000 rejected proposals. */
static int ora_lp_beta( const ncgb_sab_view* s, int64_t ie, ncgb_rng* rng, double* beta_out, size_t* bin_out )
{
  const ncgb_lp_slot* slots = s->lp_slot + ie * NCGB_LP_K;
  const ncgb_lp_cell* cells = s->lp_cell + ie * NCGB_LP_K;
  for ( int tries = 0; tries < 1000; ++tries ) {
    const uint64_t prod = (uint64_t)ncgb_rng_u32( rng ) * (uint64_t)NCGB_LP_K;
    const int j = (int)( prod >> 32 );
    const float fr = (float)( (uint32_t)prod >> 8 ) * ( 1.0f / 16777216.0f );
    const int k = ( fr < slots[j].aprob ) ? j : slots[j].alias;
    const ncgb_lp_cell* c = cells + k;
    const uint32_t w = ncgb_rng_u32( rng );
    int lo = c->seg_lo, hi = c->seg_lo + c->seg_n - 1;
    while ( lo < hi ) {
      const int mid = ( lo + hi + 1 ) >> 1;
      if ( s->lp_seg[mid].w0 <= w )
        lo = mid;
      else
        hi = mid - 1;
    }
    const ncgb_lp_seg* g = s->lp_seg + lo;
    const float y = fmaf( g->slope, (float)( w - g->w0 ), g->y0 );
    const float ua = (float)( ncgb_rng_u32( rng ) >> 8 ) * ( 1.0f / 16777216.0f );
    if ( ua * c->env < y ) {
      *beta_out = fma( (double)( 2ull * w + 1ull ), c->h, c->q );
      *bin_out = (size_t)g->bin;
      return 1;
    }
  }
  return 0;
}

/* SABSamplerAtE_Alg1::sampleAlphaBeta, NCSABSamplerModels.cc:48-155.
 * Returns ORA_OK or ORA_LOOPCAP.  With a learned proposal attached and
 * enabled for sampler ie, beta of the regular range comes from ora_lp_beta
 * and the first bin keeps its probability bcdf[1]. */
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
  const int learned = s->lp_hdr && s->lp_hdr[ie].enabled;
  for ( int iloop = 0; iloop < 100; ++iloop ) {
    size_t ibs = 0;
    double beta = 0.0;
    int first_bin;
    if ( learned ) {
      first_bin = ncgb_rng_u32( rng ) < s->lp_hdr[ie].c1_thr;
      if ( !first_bin && !ora_lp_beta( s, ie, rng, &beta, &ibs ) )
        return ORA_LOOPCAP;
    } else {
      beta = ora_percentile( bx, by, bcdf, nbs, ncgb_rng_generate( rng ), &ibs );
      first_bin = ( ibs == 0 && fbkep <= 0.0 );
    }
    if ( first_bin ) {
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

/* ---- free gas (NCFreeGasUtils.cc) ------------------------------------------ */

#define FG_TABLE_LEN 1103
static double fg_erfc_table[FG_TABLE_LEN];

/* erfc at the edges of 1100 bins on [-2,9] plus +-infinity
 * (NCFreeGasUtils.cc:95-122; linspace as NCMath.cc:68-81). */
__attribute__((constructor)) static void fg_init_table( void )
{
  const double lo = -2.0, hi = 9.0;
  const unsigned num = FG_TABLE_LEN - 2, nm1 = num - 1;
  const double interval = ( hi - lo ) / nm1;
  fg_erfc_table[0] = 2.0;
  for ( unsigned i = 0; i < nm1; ++i )
    fg_erfc_table[1 + i] = erfc( lo + i * interval );
  fg_erfc_table[num] = erfc( hi );
  fg_erfc_table[FG_TABLE_LEN - 1] = 0.0;
}

/* erfcQuickBounds, NCFreeGasUtils.cc:124-147: lb <= erfc(x) <= ub. */
static void fg_erfc_bounds( double x, double* lb, double* ub )
{
  const double binw = ( 9.0 - ( -2.0 ) ) / ( FG_TABLE_LEN - 3 );
  const double invbinw = ( FG_TABLE_LEN - 3 ) / ( 9.0 - ( -2.0 ) );
  const double verylow = -2.0 - 0.5 * binw;
  const double veryhigh = 9.0 + 0.5 * binw;
  const double xs = ora_clamp( x, verylow, veryhigh );
  const double rel = xs - ( -2.0 );
  int bin = (int)( 1.0 + rel * invbinw );
  if ( bin > FG_TABLE_LEN - 1 ) bin = FG_TABLE_LEN - 1;
  if ( bin < 0 ) bin = 0;
  *lb = fg_erfc_table[bin + 1] * 0.99999999;
  *ub = fg_erfc_table[bin] * 1.00000001;
}

/* erfcdiff, NCMath.cc:338-390 */
static double fg_erfcdiff_nt( double a, double b )
{
  if ( b < 0 ) { double t = -b; b = -a; a = t; }
  const double erfca = a > 27.3 ? 0.0 : erfc( a );
  if ( b > a + 4.0 && ( a >= 4 || ( a < 0.0 && b > 6.0 ) ) )
    return erfca;
  const double erfcb = b > 27.3 ? 0.0 : erfc( b );
  return erfca - erfcb;
}

static double fg_erfcdiff( double a, double b )
{
  const double kisp = 0.564189583547756286948079451560772585844050629;
  if ( ora_max( fabs(a), fabs(b) ) < 0.32 ) {
    const double c1 = -2.0 * kisp, c3 = 2.0 * kisp / 3.0, c5 = -0.2 * kisp, c7 = kisp / 21.0;
    const double c9 = -kisp / 108.0, c11 = kisp / 660.0, c13 = -kisp / 4680.0, c15 = kisp / 37800.0;
    const double a2 = a*a, b2 = b*b;
    const double a3 = a * a2 * ( c3 + a2 * ( c5 + a2 * ( c7 + ( a2 * ( c9 + a2 * ( c11 + a2 * ( c13 + a2 * c15 ) ) ) ) ) ) );
    const double b3 = b * b2 * ( c3 + b2 * ( c5 + b2 * ( c7 + ( b2 * ( c9 + b2 * ( c11 + b2 * ( c13 + b2 * c15 ) ) ) ) ) ) );
    return c1*(a-b) + ( a3 - b3 );
  }
  return a > b ? -fg_erfcdiff_nt( b, a ) : fg_erfcdiff_nt( a, b );
}

/* erfc_rescaled, NCMath.cc:393-417: exp(b)*erfc(x) */
static double fg_erfc_rescaled( double x, double b )
{
  if ( b < -745.1 )
    return 0.0;
  if ( ( x < 23.0 && fabs(b) < 700 ) || x < 5 )
    return exp( b ) * erfc( x );
  const double bxx = b - x*x;
  if ( bxx < -745.1 )
    return 0.0;
  const double y = 1/x, y2 = y*y;
  return 0.564189583547756286948079451560772585844050629 * exp( bxx )
         * ( y+y2*(-0.5+y2*(0.75+y2*(-1.875+y2*(6.5625+y2*-29.53125)))) );
}

/* RandExpIntervalSampler, NCRandUtils.hh:162-199 */
typedef struct { double a, c1, c2; } fg_expint;
static void fg_expint_set( fg_expint* s, double a, double b, double c )
{
  s->a = a; s->c1 = -1.0 / c; s->c2 = expm1( -c * ( b - a ) );
}
static double fg_expint_sample( const fg_expint* s, ncgb_rng* rng )
{
  return s->a + s->c1 * log( 1.0 + ncgb_rng_generate( rng ) * s->c2 );
}

/* randExpDivSqrt, NCRandUtils.cc:224-330: exp(-c*x)/sqrt(x) on [a,b] */
static double fg_rand_exp_div_sqrt( ncgb_rng* rng, double c, double a, double b )
{
  const double A = c*a;
  if ( A > 0.1 ) {
    const double U = c*(b-a);
    const double invA = 1.0/A;
    fg_expint es;
    fg_expint_set( &es, 0, U, 1.0 );
    for (;;) {
      const double ugen = fg_expint_sample( &es, rng );
      const double R = ncgb_rng_generate( rng );
      if ( (1.0+ugen*invA)*R*R < 1.0 )
        return ora_clamp( (ugen+A)/c, a, b );
    }
  }
  const double Ulim = 16.1180956509583;
  const double U = c*(b-a) < Ulim ? c*(b-a) : Ulim;
  const double B = U+A;
  if ( !( B > A ) )
    return a;
  const double sqrtA = sqrt(A), sqrtB = sqrt(B);
  const double sBmA = sqrtB - sqrtA, twosqrtA = 2*sqrtA;
  double ugen;
  for (;;) {
    const double T = ncgb_rng_generate( rng ) * sBmA;
    ugen = T*(T+twosqrtA);
    const double Ra = ncgb_rng_generate( rng );
    if ( ugen < 2.0 ) {
      const double t6 = 1.0+ugen*(-1.0+ugen*(1.0/2.0+ugen*(-1.0/6.0+ugen*(1.0/24.0+ugen*(-1.0/120.0+ugen*(1.0/720.0))))));
      if ( Ra > t6 ) continue;
      if ( Ra + 0.020221 < t6 ) break;
    } else {
      if ( Ra > 0.135335283236614 ) continue;
      if ( ugen > 4.0 && Ra > 0.0183156388887343 ) continue;
    }
    if ( Ra < exp( -ugen ) )
      break;
  }
  return ora_clamp( (ugen+A)/c, a, b );
}

/* randExpMInvXMCXDivSqrtX, NCFreeGasUtils.cc:223-488: exp(-1/x-c*x)/sqrt(x) on [xm,xp] */
static double fg_f_eval( double x, double xmax, double c )
{
  const double exparg = (x-xmax)/(x*xmax)-c*(x-xmax);
  if ( exparg >= 706.0 )
    return 1.0;
  return exparg < -745.1 ? 0.0 : exp( exparg ) * sqrt( xmax/x );
}

static double fg_rand_emix( ncgb_rng* rng, double c, double xm, double xp )
{
  if ( xp == xm )
    return xm;
  const double sqrtc = sqrt(c);
  const double invsqrtc = 1/sqrtc;
  const double xpeak = ( c > 1e-5
                         ? ( c > 1e200 ? invsqrtc : (sqrt(16.0*c+1.0)-1.0)/(4.0*c) )
                         : ( 2.0-c*(8.0-c*(64.0-c*(640.0-c*7168.0))) ) );
  if ( xpeak == 0.0 )
    return xm > 0.0 ? xm : ( DBL_MIN < xp ? DBL_MIN : xp );
  const double xmax = ( xm > xpeak ? xm : ( xp < xpeak ? xp : xpeak ) );
  if ( !( xmax > 0.0 ) )
    return xm;
  double xlarge = ora_max( 5.0/sqrt(c), 2*xpeak );
  double xsmall = ( 0.2/sqrt(c) < 0.5*xpeak ) ? 0.2/sqrt(c) : 0.5*xpeak;
  if ( xp > xlarge ) {
    const double t = ora_max( xm, xlarge ) + 15.0/c;
    xp = xp < t ? xp : t;
  }
  if ( xm < xsmall ) {
    const double xsm = xp < xsmall ? xp : xsmall;
    xm = ora_max( xm, xsm / ( 1 + 30.0*xsm ) );
  }
  const double fpmin = DBL_MIN;
  if ( ( xm = ora_max( fpmin, ora_max( fpmin/xp, xm ) ) ) >= xp )
    return xp;
  const double fcutoff_limit = 1e-9;
  if ( xp < xpeak ) {
    for (;;) {
      const double xm_new = xp - 0.01*(xp-xm);
      const double fval = fg_f_eval( xm_new, xmax, c );
      if ( fval >= fcutoff_limit )
        break;
      xm = xm_new;
    }
  }
  double probability_flat = -1.0, xswitch = -1.0, area_right = -1.0;
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
    area_right = ( fg_erfc_rescaled( sqrtc*sqrt(xswitch), B ) - fg_erfc_rescaled( sqrtc*sqrt(xp), B ) )
                 * sqrt( 3.1415926535897932384626433832795028841971694*(xmax/c) );
    probability_flat = area_left/(area_left+area_right);
  }
  int single_side, always_left;
#define FG_EVALP(pl) do { always_left = ( (pl) > 1.0-fcutoff_limit ); \
    int always_right = ( (pl) < fcutoff_limit ); single_side = ( always_left || always_right ); } while(0)
  FG_EVALP( probability_flat );
  if ( !single_side && fg_f_eval( xswitch, xmax, c ) < fcutoff_limit*1.1 ) {
    probability_flat = 1.0;
    area_right = 0.0;
    xp = xswitch;
    always_left = 1;
    single_side = 0;
  }
  for (;;) {
    const int do_flat = single_side ? always_left : ( ncgb_rng_generate( rng ) < probability_flat );
    if ( do_flat ) {
      double dx = xswitch-xm;
      const double xthr_up = xswitch, xthr_low = xm;
      const double fthreshold = 0.05;
      const double xgen = xm + ncgb_rng_generate( rng )*dx;
      const double Raccept = ncgb_rng_generate( rng );
      if ( !ora_in_interval( xthr_low, xthr_up, xgen ) && Raccept > fthreshold )
        continue;
      const double fval = fg_f_eval( xgen, xmax, c );
      if ( fval < fthreshold ) {
        if ( fval < fcutoff_limit ) {
          if ( xgen < xmax )
            xm = xgen;
          else
            xswitch = xgen;
          dx = xswitch-xm;
          if ( !single_side ) {
            const double area_left = dx;
            probability_flat = area_left/(area_left+area_right);
            FG_EVALP( probability_flat );
          }
          continue;
        }
      }
      if ( Raccept <= fval )
        return xgen;
    } else {
      const double xgen = fg_rand_exp_div_sqrt( rng, c, xswitch, xp );
      if ( ncgb_rng_generate( rng ) < exp( (xgen-xp)/(xgen*xp) ) )
        return xgen;
    }
  }
#undef FG_EVALP
}

/* FreeGasSampler state, NCFreeGasUtils.cc:492-515 */
typedef struct {
  double c, kT, sqrtAc, invA, Adiv4, normfact, c_real;
} fg_sampler;

static void fg_sampler_init( fg_sampler* s, double ekin, double kT, double mass_amu )
{
  const double cr = ekin / kT;
  s->c = cr > 1e-10 ? cr : 1e-10;
  if ( s->c > 1e14 ) s->c = 1e14;
  s->kT = kT;
  s->sqrtAc = sqrt( mass_amu * s->c / 1.00866491588 );
  const double Arel = ( 1.0 / 1.00866491588 ) * mass_amu;
  s->invA = 1.0 / Arel;
  s->Adiv4 = 0.25 * Arel;
  s->normfact = 0.5 / erf( sqrt( s->c * s->invA ) );
  s->c_real = cr;
}

/* FGEvalBetaDistHelper, NCFreeGasUtils.cc:153-222 */
typedef struct { double beta, normfact, expmbeta, k11, k12, k21, k22; } fg_betaeval;

static void fg_betaeval_init( fg_betaeval* h, const fg_sampler* s, double beta )
{
  h->beta = beta;
  h->normfact = s->normfact;
  h->expmbeta = -1.0;
  const double eps = beta / s->c;
  const double sqrt1pluseps = sqrt( 1 + eps );
  const double S = ( beta < 0.0 ? -1.0 : 1.0 );
  const double sqrtepsprime = ( eps >= 0.0 ? 1.0 : sqrt1pluseps );
  const double sqrtgammaplus = sqrt( 2.0+eps+2.0*sqrt1pluseps );
  const double SP = 0.5*(S+s->invA);
  const double SM = 0.5*(S-s->invA);
  const double invA_sqrtepsprime = s->invA*sqrtepsprime;
  const double mS_sqrtepsprime = -S*sqrtepsprime;
  const double SPsgp = sqrtgammaplus*SP;
  const double SMsgp = sqrtgammaplus*SM;
  h->k11 = s->sqrtAc*( -invA_sqrtepsprime + SPsgp );
  h->k12 = s->sqrtAc*( mS_sqrtepsprime + SPsgp );
  h->k21 = s->sqrtAc*( mS_sqrtepsprime + SMsgp );
  h->k22 = s->sqrtAc*( invA_sqrtepsprime + SMsgp );
}

static void fg_betaeval_expm( fg_betaeval* h )
{
  if ( h->expmbeta < 0 )
    h->expmbeta = h->beta < -700.0 ? 0.0 : exp( -h->beta );
}

static double fg_betaeval_exact( fg_betaeval* h )
{
  const double t1 = fg_erfcdiff( h->k11, h->k12 );
  fg_betaeval_expm( h );
  if ( !h->expmbeta )
    return h->normfact*t1;
  const double t2 = fg_erfcdiff( h->k21, h->k22 );
  return h->normfact*(t1+t2*h->expmbeta);
}

static void fg_betaeval_bounds( fg_betaeval* h, double* lb, double* ub )
{
  double l11, u11, l12, u12, l21, u21, l22, u22;
  fg_erfc_bounds( h->k11, &l11, &u11 );
  fg_erfc_bounds( h->k12, &l12, &u12 );
  const double t1l = l11 - u12, t1u = u11 - l12;
  fg_erfc_bounds( h->k21, &l21, &u21 );
  fg_erfc_bounds( h->k22, &l22, &u22 );
  const double t2l = l21 - u22, t2u = u21 - l22;
  if ( t2u > 0.0 ) {
    fg_betaeval_expm( h );
    *lb = h->normfact*(t1l+t2l*h->expmbeta);
    *ub = h->normfact*(t1u+t2u*h->expmbeta);
    return;
  }
  *lb = h->normfact*t1l;
  *ub = h->normfact*t1u;
}

/* FreeGasSampler::sampleBeta, NCFreeGasUtils.cc:530-849 */
static double fg_sample_beta( const fg_sampler* s, ncgb_rng* rng )
{
  if ( s->c_real > 1e4 ) {
    const double A = 1.0 / s->invA;
    const double A2 = A*A;
    const double thr = 1e4 * ( 1000.0*A < A2*A2*A2 ? 1000.0*A : A2*A2*A2 );
    if ( s->c_real > thr ) {
      const double am1_div_ap1 = (1.0-s->invA)/(1.0+s->invA);
      const double elossmax = s->c_real * (1.0-am1_div_ap1*am1_div_ap1);
      return -elossmax*ncgb_rng_generate( rng );
    }
  }
  const double Tlim = 2.0;
  const double Tlim_k1 = 0.135335283236612691893999494972484403407;
  const double Tlim_k2 = 274./315.;
  const double fcutoff_limit = 1e-6;
  double aa = ora_max( -s->c_real, -s->c ), bb = 13.815510557964274;
  if ( s->invA <= 1.0/10.0 ) {
    if ( s->c > 10.1 ) {
      for (;;) {
        const double aa_new = aa*0.2;
        if ( aa_new > -1e-99 )
          break;
        fg_betaeval h;
        fg_betaeval_init( &h, s, aa_new );
        if ( fg_betaeval_exact( &h ) > fcutoff_limit )
          break;
        aa = aa_new;
      }
    }
    for (;;) {
      const double bb_new = bb*0.25;
      if ( bb_new < 1e-99 )
        break;
      fg_betaeval h;
      double lb, ub;
      fg_betaeval_init( &h, s, bb_new );
      fg_betaeval_bounds( &h, &lb, &ub );
      if ( ub > fcutoff_limit )
        break;
      bb = bb_new;
    }
  }
  if ( !( bb > aa ) )
    return aa;
  double a = 0, b = 0, prob_downscat = 0, prob_notclosetail = 0;
  fg_expint es;
  int es_valid = 0;
#define FG_SETAB(aaa,bbb) do { \
    a = (aaa); b = (bbb); \
    double area_downscat = -a, area_fartail, area_closetail; \
    if ( b <= Tlim ) { \
      area_fartail = 0.0; \
      area_closetail = b * (1.0+b*(-1./2.+b*(1./6.+b*(-1./24.+b*(1./120.+b*(-1./720.+b*(1./5040.))))))); \
    } else { \
      area_fartail = Tlim_k1 - exp( -b ); \
      area_closetail = Tlim_k2; \
    } \
    const double invareatot = 1.0 / ( area_downscat + area_closetail + area_fartail ); \
    prob_downscat = area_downscat * invareatot; \
    prob_notclosetail = ( area_fartail + area_downscat ) * invareatot; \
    es_valid = 0; } while (0)
  FG_SETAB( aa, bb );
  const double fthreshold = 0.1;
  double afthreshold = a, bfthreshold = b;
  for (;;) {
    double beta, foverlay;
    const double Rsel = ncgb_rng_generate( rng );
    if ( Rsel < prob_downscat ) {
      beta = ncgb_rng_generate( rng )*a;
      foverlay = 1.0;
    } else if ( Rsel < prob_notclosetail ) {
      if ( !es_valid ) { fg_expint_set( &es, Tlim, b, 1.0 ); es_valid = 1; }
      beta = fg_expint_sample( &es, rng );
      foverlay = exp( -beta );
    } else {
      const double bmax = b < Tlim ? b : Tlim;
      for (;;) {
        beta = ncgb_rng_generate( rng )*bmax;
        const double R0 = ncgb_rng_generate( rng );
        const double kcheap = 19./45.;
        if ( R0 > 1.0 - kcheap*beta )
          continue;
        foverlay = 1.0+beta*(-1.+beta*(1./2.+beta*(-1./6.+beta*(1./24.+beta*(-1./120.+beta*(1./720.))))));
        if ( R0 < foverlay )
          break;
      }
    }
    const double faccept = ncgb_rng_generate( rng )*foverlay;
    if ( faccept > fthreshold && !ora_in_interval( afthreshold, bfthreshold, beta ) )
      continue;
    fg_betaeval h;
    fg_betaeval_init( &h, s, beta );
    int need_exact = 1;
    double fval = 0.0;
    if ( beta > 0 ) {
      double lb, ub;
      fg_betaeval_bounds( &h, &lb, &ub );
      if ( faccept <= lb )
        return beta;
      fval = ub;
      if ( faccept > ub )
        need_exact = 0;
    }
    if ( need_exact ) {
      fval = fg_betaeval_exact( &h );
      if ( faccept < fval )
        return beta;
    }
    if ( fval < fcutoff_limit ) {
      if ( beta < 0 ) { FG_SETAB( beta, b ); } else { FG_SETAB( a, beta ); }
      continue;
    }
    if ( fval < fthreshold ) {
      if ( beta < 0 )
        afthreshold = ora_max( afthreshold, beta );
      else
        bfthreshold = bfthreshold < beta ? bfthreshold : beta;
    }
  }
#undef FG_SETAB
}

/* FreeGasSampler::sampleAlpha, NCFreeGasUtils.cc:851-932 */
static double fg_sample_alpha( const fg_sampler* s, double beta, ncgb_rng* rng )
{
  if ( s->c_real < s->c || ora_mu_isotropic_at_beta( beta, s->c ) ) {
    ora_alim al = ora_alpha_limits( s->c_real, beta );
    const double alpha = al.lo + ncgb_rng_generate( rng )*(al.hi-al.lo);
    return ora_clamp( alpha, al.lo, al.hi );
  }
  beta = ora_max( -s->c, beta );
  ora_alim al = ora_alpha_limits( s->c, beta );
  const double am = al.lo, ap = al.hi;
  if ( am == ap )
    return am;
  const double betasq = beta*beta;
  const double t = betasq * s->Adiv4;
  const double c = 0.0625 * betasq;
  if ( ( t < c ? t : c ) < 1e-5 ) {
    const double fourA = s->Adiv4*16.0;
    const double inv4A = 1.0/fourA;
    const double xxm = am*inv4A, xxp = ap*inv4A;
    for (;;) {
      const double xx = fg_rand_exp_div_sqrt( rng, 1.0, xxm, xxp );
      const double alpha = xx * fourA;
      if ( alpha < am || alpha > ap )
        continue;
      if ( alpha*ap*( -log( ncgb_rng_generate( rng ) ) ) >= t*(ap-alpha) )
        return alpha;
    }
  }
  const double invt = 1.0/t;
  const double x = fg_rand_emix( rng, c, am*invt, ap*invt );
  return ora_clamp( x*t, am, ap );
}

/* FreeGasSampler::sampleAlphaBeta (NCFreeGasUtils.hh:132-144) */
static void fg_sample_alphabeta( const fg_sampler* s, ncgb_rng* rng, double* alpha, double* beta )
{
  const double b = fg_sample_beta( s, rng );
  if ( b < -s->c || ora_mu_isotropic_at_beta( b, s->c ) ) {
    ora_alim al = ora_alpha_limits( s->c_real, b );
    const double a = al.lo+ncgb_rng_generate( rng )*(al.hi-al.lo);
    *alpha = ora_clamp( a, al.lo, al.hi );
    *beta = b;
    return;
  }
  *alpha = fg_sample_alpha( s, b, rng );
  *beta = b;
}

/* FreeGas::sampleScatterIsotropic (NCFreeGas.cc:70-75) via
 * FreeGasSampler::sampleDeltaEMu (NCFreeGasUtils.hh:146-161). */
static int ora_freegas_scatter( const ncgb_freegas_view* v, ncgb_rng* rng, double ekin, double* ef, double* mu )
{
  fg_sampler s;
  fg_sampler_init( &s, ekin, v->kT, v->mass_amu );
  const double beta = fg_sample_beta( &s, rng );
  double dE, muv;
  if ( beta <= -s.c || ora_mu_isotropic_at_beta( beta, s.c ) ) {
    dE = beta*s.kT;
    muv = ncgb_rng_generate( rng )*2.0-1.0;
  } else {
    const double alpha = fg_sample_alpha( &s, beta, rng );
    int st = ora_alphabeta_to_demu( alpha, beta, s.c*s.kT, s.kT, &dE, &muv );
    if ( st != ORA_OK )
      return st;
  }
  *ef = ora_max( 0.0, ekin + dE );
  *mu = muv;
  return ORA_OK;
}

/* SABSampler::sampleHighE, NCSABSampler.cc:59-156.  Returns 1 with (alpha,
 * beta) from the extender, 0 if the table must be sampled at E = Emax, or -1
 * where the reference throws BadInput. */
static int ora_sab_high_e( const ncgb_sab_view* s, double ekin, ncgb_rng* rng, double* alpha, double* beta )
{
  const double emax = s->egrid[s->ne - 1];
  const double extE = ekin * ( s->ext_sigma_free * ora_freegas_shape( s->ext_ca * ekin ) );
  const double P_inside = s->k1 / ( ( s->k1 - s->k2 ) + extE );
  const double P_ext_inside = s->k2 / extE;
  const double P_discard = ( P_ext_inside >= P_inside ? ( 1.0 - P_inside/P_ext_inside ) : 0.0 );
  if ( P_discard > 0.95 )
    return -1;
  if ( P_ext_inside < P_inside ) {
    const double aa = 1.0 - P_ext_inside;
    const double P_extra = aa > 1e-10 ? ( P_inside - P_ext_inside ) / aa : 1.0;
    if ( ncgb_rng_generate( rng ) < P_extra )
      return 0;
  }
  const double emax_div_kt = emax / s->kT;
  fg_sampler fs;
  fg_sampler_init( &fs, ekin, s->ext_kT, s->ext_mass_amu );
  for (;;) {
    double a, b;
    fg_sample_alphabeta( &fs, rng, &a, &b );
    if ( b <= -emax_div_kt ) { *alpha = a; *beta = b; return 1; }
    ora_alim al = ora_alpha_limits( emax_div_kt, b );
    if ( !ora_in_interval( al.lo, al.hi, a ) ) { *alpha = a; *beta = b; return 1; }
    if ( P_discard && ncgb_rng_generate( rng ) < P_discard )
      continue;
    return 0;
  }
}

/* SABSampler::sampleAlphaBeta + sampleDeltaEMu, NCSABSampler.cc:158-236,
 * and SABScatter::sampleScatterIsotropic, NCSABScatter.cc:92-101. */
static int ora_sab_scatter( const ncgb_sab_view* s, ncgb_rng* rng, double ekin, double* ef, double* mu )
{
  const size_t ne = (size_t)s->ne;
  size_t iu = ora_upper_bound( s->egrid, ne, ekin );
  int ultra_small = 0;
  int64_t ie;
  double ekin_tab = ekin; /* energy the table is sampled at */
  double alpha = 0.0, beta = 0.0;
  int found = 0;
  if ( iu == ne ) {
    /* high-E extrapolation (NCSABSampler.cc:170-178) */
    const int h = ora_sab_high_e( s, ekin, rng, &alpha, &beta );
    if ( h < 0 )
      return ORA_CALCERROR;
    if ( h == 1 )
      found = 1;
    ekin_tab = s->egrid[ne - 1];
    ie = (int64_t)ne - 1;
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
  const double ekin_div_kT = ekin_tab / s->kT;
  const double sampling_ekin_div_kT = ultra_small ? s->egrid[0] / s->kT : ekin_div_kT;
  for ( int loop = 0; !found && loop < 100; ++loop ) {
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
  /* SABSampler::sampleDeltaEMu uses the neutron's own energy from here on */
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
      st = ora_freegas_scatter( &c->fg, rng, ekin, ef, mu );
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
    if ( out_ndraws ) out_ndraws[i] = (int32_t)ncgb_rng_ndoubles( &rng );
    if ( st ) ++nbad;
  }
  return nbad;
}

/* randDirectionGivenScatterMu, NCRandUtils.cc:51-96: the outgoing direction
 * at cosine mu to 'in' (normalised unless within 1e-14 of unit length) with a
 * uniform azimuth, from Marsaglia trial vectors crossed with it.  Returns
 * ORA_OK, or ORA_LOOPCAP after 100000 nearly parallel trial vectors (the
 * reference's loop is unbounded). */
static int ora_rand_dir_given_mu( ncgb_rng* rng, double mu, const double* in, double* out )
{
  const double m2 = in[0]*in[0] + in[1]*in[1] + in[2]*in[2];
  const double invm = ( fabs( m2 - 1.0 ) < 1e-14 ? 1.0 : 1.0 / sqrt( m2 ) );
  const double u0 = in[0]*invm, u1 = in[1]*invm, u2 = in[2]*invm;
  double t0 = 0.0, t1 = 0.0, t2 = 0.0, tm2 = 0.0;
  int it = 0;
  for ( ; it < 100000; ++it ) {
    const double x0 = 2.0*ncgb_rng_generate( rng ) - 1.0;
    const double x1 = 2.0*ncgb_rng_generate( rng ) - 1.0;
    const double s = x0*x0 + x1*x1;
    if ( s < 1.0 ) {
      const double t = 2.0*sqrt( 1.0 - s );
      const double a0 = x0*t, a1 = x1*t, a2 = 1.0 - 2.0*s;
      t0 = a1*u2 - a2*u1;
      t1 = a2*u0 - a0*u2;
      t2 = a0*u1 - a1*u0;
      tm2 = t0*t0 + t1*t1 + t2*t2;
      if ( !( tm2 < 0.001 ) )
        break;
    }
  }
  if ( it == 100000 )
    return ORA_LOOPCAP;
  const double f = sqrt( ( 1.0 - mu*mu ) / tm2 );
  out[0] = u0*mu + t0*f;
  out[1] = u1*mu + t1*f;
  out[2] = u2*mu + t2*f;
  return ORA_OK;
}

/* ProcComposition::sampleScatter (NCProcImpl.cc:364-377) for non-oriented
 * materials: ScatterIsotropicMat::sampleScatter (NCProcImpl.cc:29-37) of the
 * picked component.  Neutron i: in dir[3i..3i+2], out dirout[3i..3i+2]. */
int64_t ncgb_oracle_scatter_dir_many( const ncgb_material_view* m, const double* ekin, const double* dir, int64_t n,
                                      uint64_t seed, uint32_t index_offset, uint32_t callseq, uint32_t stream,
                                      double* out_ef, double* out_dir, int32_t* out_status )
{
  int64_t nbad = 0;
  for ( int64_t i = 0; i < n; ++i ) {
    ncgb_rng rng;
    ncgb_rng_init( &rng, seed, (uint32_t)( i + index_offset ), callseq, stream );
    double mu = 1.0;
    const double* in = dir + 3 * i;
    double* out = out_dir + 3 * i;
    int st;
    if ( !ora_contains( m->dom_elow, m->dom_ehigh, ekin[i] ) ) {
      out_ef[i] = ekin[i];
      out[0] = in[0]; out[1] = in[1]; out[2] = in[2];
      st = ORA_OK;
    } else {
      st = ncgb_oracle_scatter( m, &rng, ekin[i], &out_ef[i], &mu );
      if ( st == ORA_OK )
        st = ora_rand_dir_given_mu( &rng, mu, in, out );
      if ( st != ORA_OK ) {
        out_ef[i] = -1.0;
        out[0] = out[1] = out[2] = 0.0;
      }
    }
    if ( out_status ) out_status[i] = st;
    if ( st ) ++nbad;
  }
  return nbad;
}

/* One neutron of ncgb_oracle_scatter_dir_many with the caller's stream
 * (the CPU MiniMC engine, oracle/ncgb_oracle_mmc.c). */
int ncgb_oracle_scatter_dir( const ncgb_material_view* m, ncgb_rng* rng, double ekin, const double* in,
                             double* ef, double* out )
{
  double mu = 1.0;
  if ( !ora_contains( m->dom_elow, m->dom_ehigh, ekin ) ) {
    *ef = ekin;
    out[0] = in[0]; out[1] = in[1]; out[2] = in[2];
    return ORA_OK;
  }
  int st = ncgb_oracle_scatter( m, rng, ekin, ef, &mu );
  if ( st == ORA_OK )
    st = ora_rand_dir_given_mu( rng, mu, in, out );
  return st;
}

/* AbsOOV::crossSectionIsotropic, NCAbsOOV.cc:40-44: c/sqrt(E), infinite at E = 0. */
void ncgb_oracle_abs_xs_many( const ncgb_material_view* m, const double* ekin, int64_t n, double* out )
{
  for ( int64_t i = 0; i < n; ++i ) {
    const double se = sqrt( ekin[i] );
    out[i] = se ? m->abs_c / se : ora_inf;
  }
}
