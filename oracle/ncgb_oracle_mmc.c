/*
 * ncgb_oracle_mmc.c -- CPU MiniMC engine.  TEST INFRASTRUCTURE ONLY: the
 * tests pin it to the reference's own MiniMC results (tests/golden/mmc_*.npz)
 * and bench.py times it as the CPU baseline of the MiniMC workload.  The
 * library in ncrystal_gb300/ never calls it.
 *
 * A plain-C restatement of NCrystal's standard MiniMC engine
 * (src/minimc/NCMMC_SimEngine.cc:170-440) one history at a time: forced
 * collisions with roulette, the transmitted part of every step tallied into
 * the standard histograms (NCMMC_StdTallies.cc), sphere / box / slab /
 * cylinder geometries (NCMMC_Sphere.hh, NCMMC_Box.hh, NCMMC_Slab.hh,
 * NCMMC_Cyl.hh) and constant / circular / isotropic sources with a fixed
 * energy (NCMMC_Source.cc:433-800).  Collisions are ncgb_oracle_scatter_dir.
 *
 * History 'id' draws the engine's numbers of its step k from Philox stream
 * (seed, id, k, 0x4d4d4301), its source numbers from (seed, id, 0,
 * 0x4d4d4302) and its collisions from (scatter_seed, id, k, scatter_stream).
 *
 * The tally buffer has the layout of the device engine: per enabled tally
 * 6 groups x [sum w, sum w x, sum w x^2, min key, max key] first, then per
 * tally 6 groups x (nbins+2) x [content, error^2].
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "ncgb_philox.h"
#include "ncgb_tables.h"

int ncgb_oracle_scatter_dir( const ncgb_material_view* m, ncgb_rng* rng, double ekin, const double* in,
                             double* ef, double* out );
double ncgb_oracle_xs( const ncgb_material_view* m, double ekin );

#define MMC_NT 9   /* theta, mu, nscat, nscat_uw, w, e, l, de, q */
#define MMC_NG 6
#define MMC_NS 5

typedef struct {
  /* geometry: 0 sphere, 1 box, 2 slab, 3 cylinder (around y; dy = 0: infinite) */
  int32_t geom, unbounded;
  double r, dx, dy, dz;
  /* source: 0 constant, 1 circular, 2 isotropic; fixed energy */
  int32_t src, might_be_outside;
  double sx, sy, sz, sux, suy, suz, sr, energy;
  double ax, ay, az, bx, by, bz;
  /* engine */
  double macro, abs_c, psurv, wthr;
  int32_t nscatthr, nscatlimit, has_abs, has_scat, ignore_miss, breakdown;
  uint64_t seed, scatter_seed;
  uint32_t scatter_stream, pad;
  /* tally reference: fixed direction / energy, else per history */
  int32_t fixed_dir, fixed_e;
  double d0x, d0y, d0z, e0;
  /* tallies */
  int32_t enabled[MMC_NT], nbins[MMC_NT];
  double xmin[MMC_NT], xmax[MMC_NT];
  int64_t off[MMC_NT], soff[MMC_NT];
} ora_mmc_cfg;

static const double mmc_wl2ekin = 0.081804209605330899;
static const double mmc_todeg = 57.2957795130823208767981548141051703324054725;

static double mmc_slab_exit( double x, double ux, double d )
{
  /* NCMMC_Utils.cc:516-537 */
  if ( ux > 0.0 ) return ( d - x ) / ux;
  if ( ux < 0.0 ) return -( d + x ) / ux;
  return INFINITY;
}

/* distToVolumeExit */
static double mmc_dist_exit( const ora_mmc_cfg* c, const double* p, const double* u )
{
  if ( c->geom == 0 ) {
    /* NCMMC_Sphere.hh:170-216 */
    double t = c->r * c->r - p[0]*p[0] - p[1]*p[1] - p[2]*p[2];
    const double pd = p[0]*u[0] + p[1]*u[1] + p[2]*u[2];
    t += pd * pd;
    t = sqrt( t > 0.0 ? t : 0.0 ) - pd;
    return t > 0.0 ? t : 0.0;
  }
  if ( c->geom == 1 ) {
    const double a = mmc_slab_exit( p[0], u[0], c->dx ), b = mmc_slab_exit( p[1], u[1], c->dy ),
                 d = mmc_slab_exit( p[2], u[2], c->dz );
    return fmin( a, fmin( b, d ) );
  }
  if ( c->geom == 2 )
    return mmc_slab_exit( p[2], u[2], c->dz );
  {
    const double a = u[0]*u[0] + u[2]*u[2];
    double t = INFINITY;
    if ( a > 0.0 ) {
      const double b = p[0]*u[0] + p[2]*u[2], cc = p[0]*p[0] + p[2]*p[2] - c->r * c->r;
      const double D = b*b - a*cc;
      t = ( -b + sqrt( D > 0.0 ? D : 0.0 ) ) / a;
      if ( t < 0.0 ) t = 0.0;
    }
    if ( c->dy > 0.0 )
      t = fmin( t, mmc_slab_exit( p[1], u[1], c->dy ) );
    return t;
  }
}

static int mmc_slab_interval( double x, double ux, double d, double* t1, double* t2 )
{
  if ( ux != 0.0 ) {
    const double a = ( d - x ) / ux, b = ( -d - x ) / ux;
    *t1 = fmax( *t1, fmin( a, b ) );
    *t2 = fmin( *t2, fmax( a, b ) );
    return 1;
  }
  return fabs( x ) <= d;
}

/* distToVolumeEntry: 0 inside, -1 miss (NCMMC_Sphere.hh:110-160,
 * NCMMC_Box.hh:112-205, NCMMC_Utils.cc:539-590) */
static double mmc_dist_entry( const ora_mmc_cfg* c, const double* p, const double* u )
{
  if ( c->geom == 0 ) {
    const double pd = p[0]*u[0] + p[1]*u[1] + p[2]*u[2];
    const double q = p[0]*p[0] + p[1]*p[1] + p[2]*p[2] - c->r * c->r;
    if ( q <= 0.0 )
      return fmin( q, pd ) < 0.0 ? 0.0 : -1.0;
    const double D = pd*pd - q;
    if ( D < 0.0 ) return -1.0;
    const double t = -( sqrt( D ) + pd );
    return t >= 0.0 ? t : -1.0;
  }
  if ( c->geom == 2 ) {
    const double a = fabs( p[2] ) - c->dz, xu = p[2] * u[2];
    if ( a <= 0.0 ) return ( a != 0.0 || !( xu > 0.0 ) ) ? 0.0 : -1.0;
    return xu >= 0.0 ? -1.0 : a / fabs( u[2] );
  }
  double t1 = -INFINITY, t2 = INFINITY;
  int hit;
  if ( c->geom == 1 ) {
    hit = mmc_slab_interval( p[0], u[0], c->dx, &t1, &t2 ) && mmc_slab_interval( p[1], u[1], c->dy, &t1, &t2 )
          && mmc_slab_interval( p[2], u[2], c->dz, &t1, &t2 );
  } else {
    const double a = u[0]*u[0] + u[2]*u[2], b = p[0]*u[0] + p[2]*u[2];
    const double q = p[0]*p[0] + p[2]*p[2] - c->r * c->r;
    if ( a > 0.0 ) {
      const double D = b*b - a*q;
      hit = D >= 0.0;
      if ( hit ) { t1 = ( -b - sqrt( D ) ) / a; t2 = ( -b + sqrt( D ) ) / a; }
    } else {
      hit = q <= 0.0;
    }
    if ( hit && c->dy > 0.0 )
      hit = mmc_slab_interval( p[1], u[1], c->dy, &t1, &t2 );
  }
  if ( !hit || t1 >= t2 || t2 <= 0.0 ) return -1.0;
  return t1 > 0.0 ? t1 : 0.0;
}

static int64_t mmc_key( double x )
{
  int64_t k;
  memcpy( &k, &x, 8 );
  return k < 0 ? ( k ^ INT64_C(0x7FFFFFFFFFFFFFFF) ) : k;
}

/* Hist1D::fill into group g of tally k (NCHists.hh:303-345, :376-400, :613-650) */
static void mmc_fill( const ora_mmc_cfg* c, double* buf, int k, int g, double x, double w, int weighted )
{
  if ( weighted && !( w > 0.0 ) ) return;
  const double wt = weighted ? w : 1.0;
  const int nb = c->nbins[k];
  int bin;
  if ( x < c->xmin[k] ) bin = 0;
  else if ( x >= c->xmax[k] ) bin = ( x == c->xmax[k] ) ? nb : nb + 1;
  else {
    const double f = ( nb / ( c->xmax[k] - c->xmin[k] ) ) * ( x - c->xmin[k] );
    bin = 1 + ( f >= (double)nb ? nb : (int)f );
  }
  double* b = buf + c->off[k] + ( (int64_t)g * ( nb + 2 ) + bin ) * 2;
  b[0] += wt;
  b[1] += wt * wt;
  double* st = buf + c->soff[k] + g * MMC_NS;
  st[0] += wt;
  st[1] += wt * x;
  st[2] += wt * x * x;
  int64_t kmin, kmax;
  memcpy( &kmin, st + 3, 8 );
  memcpy( &kmax, st + 4, 8 );
  const int64_t kx = mmc_key( x );
  if ( kx < kmin ) memcpy( st + 3, &kx, 8 );
  if ( kx > kmax ) memcpy( st + 4, &kx, 8 );
}

static void mmc_fill2( const ora_mmc_cfg* c, double* buf, int k, int cat, double x, double w, int weighted )
{
  mmc_fill( c, buf, k, 0, x, w, weighted );
  if ( c->breakdown )
    mmc_fill( c, buf, k, 1 + cat, x, w, weighted );
}

/* tallyRecord, NCMMC_StdTallies.cc:430-660 */
static void mmc_tally( const ora_mmc_cfg* c, double* buf, double e, const double* u, double w, int nscat,
                       int ninel, double e0, const double* d0 )
{
  const int cat = nscat > 1 ? ( ninel ? 4 : 3 ) : ( nscat == 1 ? ( ninel ? 2 : 1 ) : 0 );
  if ( c->enabled[0] || c->enabled[1] || c->enabled[8] ) {
    double mu;
    if ( c->fixed_dir && c->d0z == 1.0 ) mu = u[2];
    else if ( c->fixed_dir ) { mu = c->d0x * u[0]; mu += c->d0y * u[1]; mu += c->d0z * u[2]; }
    else { mu = d0[0] * u[0]; mu += d0[1] * u[1]; mu += d0[2] * u[2]; }
    mu = mu < -1.0 ? -1.0 : ( mu > 1.0 ? 1.0 : mu );
    if ( c->enabled[1] ) mmc_fill2( c, buf, 1, cat, mu, w, 1 );
    if ( c->enabled[8] ) {
      const double ei = c->fixed_e ? c->e0 : e0;
      double q = sqrt( e * ei ) * mu * ( -2.0 ) + ei + e;
      q *= 4.0 * M_PI * M_PI / mmc_wl2ekin;
      mmc_fill2( c, buf, 8, cat, sqrt( q > 0.0 ? q : 0.0 ), w, 1 );
    }
    if ( c->enabled[0] ) mmc_fill2( c, buf, 0, cat, acos( mu ) * mmc_todeg, w, 1 );
  }
  if ( c->enabled[5] ) mmc_fill2( c, buf, 5, cat, e, w, 1 );
  if ( c->enabled[7] ) mmc_fill2( c, buf, 7, cat, ( c->fixed_e ? c->e0 : e0 ) - e, w, 1 );
  if ( c->enabled[6] ) mmc_fill2( c, buf, 6, cat, sqrt( mmc_wl2ekin ) * sqrt( 1.0 / ( e > 4.9406564584124654e-324 ? e : 4.9406564584124654e-324 ) ), w, 1 );
  if ( c->enabled[2] ) mmc_fill2( c, buf, 2, cat, (double)nscat, w, 1 );
  if ( c->enabled[3] ) mmc_fill2( c, buf, 3, cat, (double)nscat, w, 0 );
  if ( c->enabled[4] ) mmc_fill2( c, buf, 4, cat, w, w, 0 );
}

/* Histories first_id .. first_id+count-1 into buf (counts[0..5]: tallied
 * count, tallied weight, missed count, missed weight, failed scatters,
 * engine steps).  Returns 0. */
int ncgb_oracle_mmc_run( const ncgb_material_view* m, const ora_mmc_cfg* c, uint64_t first_id, uint64_t count,
                         double* buf, double* counts )
{
  for ( uint64_t h = 0; h < count; ++h ) {
    const uint64_t id = first_id + h;
    ncgb_rng rs;
    ncgb_rng_init( &rs, c->seed, (uint32_t)id, 0u, 0x4d4d4302u );
    double p[3] = { c->sx, c->sy, c->sz }, u[3] = { c->sux, c->suy, c->suz };
    if ( c->src == 1 && c->sr > 0.0 ) {
      const double rad = sqrt( ncgb_rng_generate( &rs ) ), phi = 2.0 * M_PI * ncgb_rng_generate( &rs );
      const double a0 = rad * cos( phi ), b0 = rad * sin( phi );
      p[0] += c->ax * a0 + c->bx * b0; p[1] += c->ay * a0 + c->by * b0; p[2] += c->az * a0 + c->bz * b0;
    } else if ( c->src == 2 ) {
      /* randIsotropicDirection, NCRandUtils.cc:25-50 */
      double x0, x1, s;
      int it = 0;
      do {
        x0 = 2.0 * ncgb_rng_generate( &rs ) - 1.0;
        x1 = 2.0 * ncgb_rng_generate( &rs ) - 1.0;
        s = x0 * x0 + x1 * x1;
      } while ( s >= 1.0 && ++it < 1000 );
      if ( !( s < 1.0 ) ) { x0 = x1 = s = 0.0; }
      const double t = 2.0 * sqrt( 1.0 - s );
      u[0] = x0 * t; u[1] = x1 * t; u[2] = 1.0 - 2.0 * s;
      if ( c->sr != 0.0 ) { p[0] -= u[0] * c->sr; p[1] -= u[1] * c->sr; p[2] -= u[2] * c->sr; }
    }
    double e = c->energy, w = 1.0, xs = -1.0;
    const double e0 = e, d0[3] = { u[0], u[1], u[2] };
    int nscat = 0, ninel = 0;
    if ( c->might_be_outside ) {
      const double d = mmc_dist_entry( c, p, u );
      if ( d < 0.0 ) {
        counts[2] += 1.0; counts[3] += 1.0;
        if ( !c->ignore_miss ) {
          mmc_tally( c, buf, e, u, 1.0, -1, 0, e0, d0 );
          counts[0] += 1.0; counts[1] += 1.0;
        }
        continue;
      }
      p[0] += d * u[0]; p[1] += d * u[1]; p[2] += d * u[2];
    }
    for ( uint32_t k = 0; k < 100000000u; ++k ) {
      counts[5] += 1.0;
      const double dexit = mmc_dist_exit( c, p, u );
      const int dinf = isinf( dexit );
      const double xabs = c->has_abs ? c->macro * ( sqrt( e ) != 0.0 ? c->abs_c / sqrt( e ) : INFINITY ) : 0.0;
      if ( !c->has_scat || c->nscatlimit == 0 || ( c->nscatlimit > 0 && nscat >= c->nscatlimit ) )
        xs = 0.0;
      else if ( nscat <= 0 || xs < 0.0 )
        xs = c->macro * ncgb_oracle_xs( m, e );
      /* calcProbTransm, NCMMC_Utils.cc:46-88 */
      const double xsc = fmin( 1.7976931348623157e308, xs );
      const double ptransm = ( c->unbounded && dinf ) ? 0.0 : ( xsc != 0.0 ? exp( -xsc * dexit ) : 1.0 );
      /* sampleRandDists, NCMMC_Utils.cc:153-176 */
      ncgb_rng re;
      ncgb_rng_init( &re, c->seed, (uint32_t)id, k, 0x4d4d4301u );
      const double r = ncgb_rng_generate( &re );
      double ds;
      if ( xs == 0.0 ) ds = INFINITY;
      else if ( dinf ) ds = log( r ) / ( -xs );
      else ds = ( -1.0 / xs ) * log( 1.0 + r * expm1( -xs * dexit ) );
      int keep = 0;
      double wk = 0.0;
      if ( w != 0.0 && !isinf( ds ) && xs > 0.0 ) {
        double rf = 1.0;
        keep = 1;
        if ( nscat >= c->nscatthr && w < c->wthr ) {
          if ( ncgb_rng_generate( &re ) > c->psurv ) keep = 0;
          else rf = 1.0 / c->psurv;
        }
        if ( keep ) {
          const double wr = exp( -xabs * ds );
          keep = wr > 0.0;
          wk = w * rf * wr * ( 1.0 - ptransm );
        }
      }
      double pabs;
      if ( c->has_abs ) {
        const double xa = fmin( 1.7976931348623157e308, xabs );
        pabs = ( c->unbounded && dinf ) ? 0.0 : ( xa != 0.0 ? exp( -xa * dexit ) : 1.0 );
      } else {
        pabs = ( c->unbounded && dinf ) ? 0.0 : 1.0;
      }
      const double wt = w * pabs * ptransm;
      mmc_tally( c, buf, e, u, wt, nscat, ninel, e0, d0 );
      counts[0] += 1.0; counts[1] += wt;
      if ( !keep )
        break;
      p[0] += ds * u[0]; p[1] += ds * u[1]; p[2] += ds * u[2];
      w = wk;
      ncgb_rng rc;
      ncgb_rng_init( &rc, c->scatter_seed, (uint32_t)id, k, c->scatter_stream );
      double ef = e, un[3];
      if ( ncgb_oracle_scatter_dir( m, &rc, e, u, &ef, un ) != 0 ) {
        counts[4] += 1.0;
        break;
      }
      ++nscat;
      if ( ef != e ) { ++ninel; xs = -1.0; }
      e = ef;
      u[0] = un[0]; u[1] = un[1]; u[2] = un[2];
    }
  }
  return 0;
}

/* sizeof(ora_mmc_cfg), for the ctypes mirror's layout check. */
int64_t ncgb_oracle_mmc_cfg_size( void ) { return (int64_t)sizeof(ora_mmc_cfg); }
