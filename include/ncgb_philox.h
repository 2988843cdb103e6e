/*
 * ncgb_philox.h -- the counter-based random streams of the GPU scattering path.
 *
 * NCrystal draws uniform doubles in (0,1] from one sequential stream per
 * Scatter object (RNG::generate, NCDefs.hh:164-194; xoroshiro128+ by default).
 * On the GPU every neutron instead owns an independent Philox4x32-10 stream
 * (Salmon et al., "Parallel random numbers: as easy as 1, 2, 3", SC'11):
 *
 *   key      = (seed & 0xffffffff, seed >> 32)
 *   counter  = (block, neutron index, call sequence number, stream index)
 *   words    = the four 32-bit outputs (x0,x1,x2,x3) of each block, in order
 *   double   = the next two words (a new block when fewer than two are left),
 *              u = ((x_lo | x_hi << 32) >> 11) + 1) * 2^-53, in (0,1]
 *   32 bits  = the next word (used by the learned beta proposal only)
 *
 * A stream of doubles only thus takes (x0,x1) and (x2,x3) of block 0, then of
 * block 1, and so on.
 * The same definition is used by the CUDA kernels, by the CPU oracle and by the
 * harness that drives the reference library with identical numbers, so that a
 * neutron's draws are the same on all three.  Header-only, plain C99 (plus
 * __host__ __device__ under nvcc).
 */
#ifndef NCGB_PHILOX_H
#define NCGB_PHILOX_H

#include <stdint.h>

#if defined(__CUDACC__)
#  define NCGB_HD __host__ __device__ __forceinline__
#else
#  define NCGB_HD static inline
#endif

typedef struct {
  uint32_t key0, key1;    /* from the seed */
  uint32_t ctr1, ctr2, ctr3; /* neutron index, call sequence, stream index */
  uint32_t block;         /* next block to generate */
  uint32_t have;          /* words of the current block not yet used (0..4) */
  uint32_t pad;
  uint32_t word[4];
} ncgb_rng;

NCGB_HD void ncgb_mulhilo32( uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo )
{
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)( p >> 32 );
  *lo = (uint32_t)p;
}

/* Philox4x32 with 10 rounds: out = philox(ctr, key). */
NCGB_HD void ncgb_philox4x32_10( const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4] )
{
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  for ( int r = 0; r < 10; ++r ) {
    uint32_t hi0, lo0, hi1, lo1;
    ncgb_mulhilo32( 0xD2511F53u, c0, &hi0, &lo0 );
    ncgb_mulhilo32( 0xCD9E8D57u, c2, &hi1, &lo1 );
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

NCGB_HD void ncgb_rng_init( ncgb_rng* r, uint64_t seed, uint32_t neutron,
                            uint32_t callseq, uint32_t stream )
{
  r->key0 = (uint32_t)seed;
  r->key1 = (uint32_t)( seed >> 32 );
  r->ctr1 = neutron;
  r->ctr2 = callseq;
  r->ctr3 = stream;
  r->block = 0;
  r->have = 0;
  r->pad = 0;
  r->word[0] = r->word[1] = r->word[2] = r->word[3] = 0;
}

NCGB_HD void ncgb_rng_refill( ncgb_rng* r )
{
  uint32_t ctr[4] = { r->block, r->ctr1, r->ctr2, r->ctr3 };
  ncgb_philox4x32_10( ctr, r->key0, r->key1, r->word );
  r->block += 1;
  r->have = 4;
}

NCGB_HD double ncgb_rng_generate( ncgb_rng* r )
{
  if ( r->have < 2 )
    ncgb_rng_refill( r );
  const uint32_t i = 4 - r->have;
  const uint64_t bits = (uint64_t)r->word[i] | ( (uint64_t)r->word[i + 1] << 32 );
  r->have -= 2;
  return (double)( ( bits >> 11 ) + 1 ) * ( 1.0 / 9007199254740992.0 );
}

NCGB_HD uint32_t ncgb_rng_u32( ncgb_rng* r )
{
  if ( r->have == 0 )
    ncgb_rng_refill( r );
  const uint32_t w = r->word[4 - r->have];
  r->have -= 1;
  return w;
}

/* Doubles drawn so far by a stream that drew doubles only. */
NCGB_HD uint32_t ncgb_rng_ndoubles( const ncgb_rng* r ) { return ( 4 * r->block - r->have ) / 2; }

#endif
