/*
 * refpin.c -- drives the reference NCrystal library (oracle/_ref) with the
 * GPU path's per-neutron Philox streams.  TEST INFRASTRUCTURE ONLY.
 *
 * ncrystal_setrandgen (ncrystal.h, ncrystal.cc:1993-2001) installs a plain C
 * function as the random source of every Scatter created afterwards.  The
 * function below returns draw j of the stream of the neutron currently being
 * scattered, so each call of the reference's scalar
 * ncrystal_samplescatterisotropic (ncrystal.cc:1168-1199) consumes exactly the
 * numbers that the oracle and the CUDA kernels consume for that neutron.  The
 * result pins (E', mu), cross-sections and draw counts per neutron, not just
 * in distribution.
 *
 * Built only where the reference sources exist (links oracle/_ref/libNCrystal).
 */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "NCrystal/cinterface/ncrystal.h"
#include "ncgb_philox.h"

static ncgb_rng g_rng;
static int64_t g_ndraws;

static double refpin_rand( void )
{
  ++g_ndraws;
  return ncgb_rng_generate( &g_rng );
}

/* Returns 0 on success; status[i] is 1 if the reference raised an error for
 * neutron i (its outputs then hold the reference's sentinels). */
int refpin_run( const char* cfg, uint64_t seed, uint32_t callseq, uint32_t stream,
                const double* ekin, int64_t n,
                double* out_xs, double* out_ef, double* out_mu,
                int32_t* out_ndraws, int32_t* out_status )
{
  ncrystal_sethaltonerror( 0 );
  ncrystal_setmsghandler( NULL );
  ncrystal_setrandgen( refpin_rand );
  ncrystal_scatter_t sc = ncrystal_create_scatter( cfg );
  if ( ncrystal_error() ) {
    fprintf( stderr, "refpin: could not create %s: %s\n", cfg, ncrystal_lasterror() );
    ncrystal_clearerror();
    return 1;
  }
  ncrystal_process_t pr = ncrystal_cast_scat2proc( sc );
  for ( int64_t i = 0; i < n; ++i ) {
    /* The reference keeps the last energy's results per Scatter object and
     * reuses them for an energy within 1e-15 relative of it
     * (NCProcImpl.cc:172-183).  Evaluating a far-away energy first makes every
     * neutron's evaluation fresh, as on the GPU, where neutrons share no state. */
    double flush;
    ncrystal_crosssection_nonoriented( pr, 12345.0, &flush );
    ncrystal_crosssection_nonoriented( pr, ekin[i], &out_xs[i] );
    ncgb_rng_init( &g_rng, seed, (uint32_t)i, callseq, stream );
    g_ndraws = 0;
    ncrystal_samplescatterisotropic( sc, ekin[i], &out_ef[i], &out_mu[i] );
    out_status[i] = 0;
    if ( ncrystal_error() ) {
      out_status[i] = 1;
      ncrystal_clearerror();
    }
    out_ndraws[i] = (int32_t)g_ndraws;
  }
  ncrystal_unref( &sc );
  ncrystal_setrandgen( NULL );
  return 0;
}

/* The same for ncrystal_samplescatter (ncrystal.cc:1159-1174): energy and
 * direction dir[3i..3i+2] in, E' and the outgoing direction out. */
int refpin_run_dir( const char* cfg, uint64_t seed, uint32_t callseq, uint32_t stream,
                    const double* ekin, const double* dir, int64_t n,
                    double* out_ef, double* out_dir, int32_t* out_ndraws, int32_t* out_status )
{
  ncrystal_sethaltonerror( 0 );
  ncrystal_setmsghandler( NULL );
  ncrystal_setrandgen( refpin_rand );
  ncrystal_scatter_t sc = ncrystal_create_scatter( cfg );
  if ( ncrystal_error() ) {
    fprintf( stderr, "refpin: could not create %s: %s\n", cfg, ncrystal_lasterror() );
    ncrystal_clearerror();
    return 1;
  }
  ncrystal_process_t pr = ncrystal_cast_scat2proc( sc );
  for ( int64_t i = 0; i < n; ++i ) {
    double flush;
    ncrystal_crosssection_nonoriented( pr, 12345.0, &flush );
    ncgb_rng_init( &g_rng, seed, (uint32_t)i, callseq, stream );
    g_ndraws = 0;
    double indir[3] = { dir[3*i], dir[3*i+1], dir[3*i+2] };
    double outdir[3];
    ncrystal_samplescatter( sc, ekin[i], (const double (*)[3])&indir, &out_ef[i], &outdir );
    out_dir[3*i] = outdir[0];
    out_dir[3*i+1] = outdir[1];
    out_dir[3*i+2] = outdir[2];
    out_status[i] = 0;
    if ( ncrystal_error() ) {
      out_status[i] = 1;
      ncrystal_clearerror();
    }
    out_ndraws[i] = (int32_t)g_ndraws;
  }
  ncrystal_unref( &sc );
  ncrystal_setrandgen( NULL );
  return 0;
}

/* The reference's absorption cross-sections (ncrystal_create_absorption,
 * ncrystal.cc:1565-1571, through the process interface). */
int refpin_abs_xs( const char* cfg, const double* ekin, int64_t n, double* out_xs )
{
  ncrystal_sethaltonerror( 0 );
  ncrystal_absorption_t ab = ncrystal_create_absorption( cfg );
  if ( ncrystal_error() ) {
    fprintf( stderr, "refpin: could not create absorption for %s: %s\n", cfg, ncrystal_lasterror() );
    ncrystal_clearerror();
    return 1;
  }
  ncrystal_crosssection_nonoriented_many( ncrystal_cast_abs2proc( ab ), ekin, (unsigned long)n, 1, out_xs );
  ncrystal_unref( &ab );
  return 0;
}
