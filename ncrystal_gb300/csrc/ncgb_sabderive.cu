// Device-side derivation of the S(alpha,beta) sampling tables
// (SABIntegrator::analyseEnergyPoint per energy-grid point,
// NCSABIntegrator.cc:283-309, :352-559; PointwiseDist, NCPointwiseDist.cc:28-74).
//
// The host builder (ncgb_tables.cc: deriveSAB) walks the energy grid and, at
// each point, the beta rows one after the other.  Here:
//   k_logcumul   one thread per beta row: log S and the cumulative alpha
//                integrals (NCSABIntegrator.cc:119-138),
//   k_betarows   one thread per (energy point, beta row): the row's active
//                alpha range (activeGridRanges, NCSABUtils.cc:460-536, by
//                binary search: the host's sweep converges to the same
//                indices), kinematic limits and tailed breakdown
//                (NCSABUtils.cc:538-633),
//   k_epoints    one thread per energy point: the ordered part (skipped rows,
//                the kinematic end point, the Neumaier sum of the beta
//                weights, the normalised beta distribution).
// Compiled with -fmad=false and sharing its per-row code with the host
// (ncgb_sabderive.hh), so the two agree bit for bit except where CUDA's log and
// exp differ from the host's in the last place.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "ncgb_host.hh"
#include "ncgb_sabderive.hh"

namespace {

  using namespace ncgb::sabd;

  constexpr unsigned kFull = 0xffffffffu;

  // One warp per beta row: log S in parallel, then the cumulative alpha
  // integrals (NCSABIntegrator.cc:119-138).  The interval integrals are
  // computed by the lanes side by side and added into the running sum in
  // the host's order (lane k's partial after term k), so the sums are the
  // host's to the bit.
  __global__ void k_logcumul( const double* alpha, const double* sab, int na, int nb, double* logsab, double* cumul )
  {
    const int ib = ( blockIdx.x * blockDim.x + threadIdx.x ) >> 5;
    const int lane = threadIdx.x & 31;
    if ( ib >= nb )
      return;   // the whole warp
    const size_t g0 = (size_t)ib * na;
    for ( int ai = lane; ai < na; ai += 32 ) {
      const double e = sab[g0 + ai];
      logsab[g0 + ai] = e > 0.0 ? log( e ) : -INFINITY;
    }
    __syncwarp();
    if ( lane == 0 )
      cumul[g0] = 0.0;
    double c = 0.0;
    for ( int base = 0; base + 1 < na; base += 32 ) {
      const int ai = base + lane;
      double t = 0.0;
      if ( ai + 1 < na )
        t = integrateAlphaIntervalFast( alpha[ai], sab[g0 + ai], alpha[ai + 1], sab[g0 + ai + 1], logsab[g0 + ai],
                                        logsab[g0 + ai + 1] );
      double mine = 0.0;
      for ( int k = 0; k < 32; ++k ) {
        const double tk = __shfl_sync( kFull, t, k );
        if ( base + k + 1 < na ) {
          c += tk;
          if ( lane == k )
            mine = c;
        }
      }
      if ( ai + 1 < na )
        cumul[g0 + ai + 1] = mine;
    }
  }

  // Per (energy point, beta row): whether the row is in the active range, and
  // its cross-section and alpha sampler.
  struct BetaRow {
    double xs;
    int32_t inrange, pad;
    ncgb_alpha_info info;
  };

  __device__ int lastLE( const double* a, int n, double x )
  {
    // largest i with a[i] <= x, or 0
    int lo = 0, hi = n;   // first index with a[i] > x in [lo, hi]
    while ( lo < hi ) {
      const int mid = ( lo + hi ) >> 1;
      if ( a[mid] <= x ) lo = mid + 1; else hi = mid;
    }
    return lo > 0 ? lo - 1 : 0;
  }

  __device__ int firstGE( const double* a, int n, double x )
  {
    int lo = 0, hi = n;   // first index with a[i] >= x
    while ( lo < hi ) {
      const int mid = ( lo + hi ) >> 1;
      if ( a[mid] < x ) lo = mid + 1; else hi = mid;
    }
    return lo;
  }

  __global__ void k_betarows( const double* alpha, const double* beta, const double* sab, const double* logsab,
                              const double* cumul, int na, int nb, const double* egrid, double kT, BetaRow* rows )
  {
    const int ie = blockIdx.y;
    const int ib = blockIdx.x * blockDim.x + threadIdx.x;
    if ( ib >= nb )
      return;
    const double x = egrid[ie] / kT;
    const double b = beta[ib];
    // activeGridRanges (NCSABUtils.cc:474-533)
    double alow = -1.0, aupp = -2.0;
    if ( b > -x ) {
      const ALim al = alphaLimits( x, b );
      alow = al.lo;
      aupp = al.hi;
    }
    const bool inr = !( alpha[na - 1] <= alow || alpha[0] >= aupp || aupp < alow );
    int iLow = na, iUpp = na;
    if ( inr ) {
      iLow = lastLE( alpha, na, alow );
      iUpp = firstGE( alpha, na, aupp );
      if ( iUpp > na - 1 )
        iUpp = na - 1;
    }
    // the row in analyseEnergyPoint (NCSABIntegrator.cc:437-486)
    const ALim al = alphaLimits( x, b );
    double xs = 0.0;
    TailedBreakdown tb;
    if ( iUpp > iLow && al.hi > al.lo ) {
      const size_t slice = (size_t)na * ib;
      tb = tailedBreakdown( alpha, (unsigned)na, sab + slice, logsab + slice, cumul + slice, al.lo, al.hi,
                            (unsigned)iLow, (unsigned)iUpp );
      xs = tb.xs_front + tb.xs_back + tb.xs_middle;
    }
    BetaRow r;
    memset( &r, 0, sizeof(r) );
    r.xs = xs;
    r.inrange = inr;
    if ( xs > 0.0 ) {
      r.info.front_alpha = tb.front.alpha;
      r.info.front_sval = tb.front.sval;
      r.info.front_logsval = tb.front.logsval;
      r.info.back_alpha = tb.back.alpha;
      r.info.back_sval = tb.back.sval;
      r.info.back_logsval = tb.back.logsval;
      if ( tb.narrow ) {
        r.info.prob_front = 1.0;
      } else {
        r.info.prob_front = tb.xs_front / xs;
        r.info.prob_notback = 1.0 - tb.xs_back / xs;
        r.info.front_idx = tb.imiddle_low;
        r.info.back_idx = tb.imiddle_upp;
      }
    } else {
      r.info.prob_front = 2.0;
      r.info.front_alpha = al.lo;
      r.info.back_alpha = al.hi;
    }
    rows[(size_t)ie * nb + ib] = r;
  }

  // The ordered part of analyseEnergyPoint (NCSABIntegrator.cc:384-559) and
  // the PointwiseDist normalisation, one warp per energy point.  Per point
  // the outputs occupy [ie*(nb+1), ie*(nb+1)+nbeta) of bx/by/bcdf and
  // [ie*(nb+1), ...+nbeta-1) of info.  The rows are taken 32 at a time: a
  // lane's place in the output is its rank among the kept rows (a row equal
  // to the lower beta limit is dropped), its trapezoid uses the previous kept
  // row (a shuffle, or the carry from the last chunk), and the Neumaier sums
  // add the terms in the host's order, so every value is the host's.
  __global__ void k_epoints( const double* beta, int nb, const double* egrid, int ne, double kT, double sigma_bound,
                             const BetaRow* rows, double* bx, double* by, double* bcdf, ncgb_alpha_info* info,
                             double* xs_out, int32_t* kind, int32_t* ibl_out, int32_t* nbeta_out, double* fbkep,
                             int32_t* err )
  {
    const int ie = ( blockIdx.x * blockDim.x + threadIdx.x ) >> 5;
    const int lane = threadIdx.x & 31;
    if ( ie >= ne )
      return;   // the whole warp
    const unsigned below = ( 1u << lane ) - 1u;
    const double x = egrid[ie] / kT;
    const BetaRow* rr = rows + (size_t)ie * nb;
    const size_t o = (size_t)ie * ( nb + 1 );
    double beta_lower_limit = -x;
    bool starts = true;
    if ( beta_lower_limit < beta[0] ) {
      const double c1 = beta[0] - ( beta[1] - beta[0] ) * 1e-6;
      const double c2 = beta[0] - fabs( beta[0] ) * 1e-13;
      const double c3 = nextafter( beta[0], beta_lower_limit );
      beta_lower_limit = dmin( c1, dmin( c2, c3 ) );
      starts = false;
    }
    int ibeta_low = nb;
    for ( int base = 0; base < nb; base += 32 ) {
      const unsigned m = __ballot_sync( kFull, base + lane < nb && rr[base + lane].inrange );
      if ( m ) { ibeta_low = base + __ffs( m ) - 1; break; }
    }
    if ( lane == 0 ) {
      xs_out[ie] = 0.0;
      kind[ie] = 0;
      ibl_out[ie] = 0;
      nbeta_out[ie] = 0;
      fbkep[ie] = 0.0;
    }
    if ( ibeta_low >= nb )
      return;
    if ( ibeta_low > 0 && beta_lower_limit < beta[ibeta_low - 1] ) {
      beta_lower_limit = beta[ibeta_low - 1];
      starts = false;
    }
    // carry across chunks (the same in every lane)
    double prev_first = beta_lower_limit, prev_second = 0.0, bx0 = beta_lower_limit;
    int n = 1;
    StableSum tot;
    bool next_ep = starts;
    for ( int base = ibeta_low; base < nb; base += 32 ) {
      const int ib = base + lane;
      double b = 0.0, xsb = 0.0;
      bool keep = false;
      if ( ib < nb ) {
        b = beta[ib];
        keep = !( b == beta_lower_limit );
        if ( keep )
          xsb = rr[ib].xs;
      }
      const unsigned m = __ballot_sync( kFull, keep );
      // the previous kept row: a lower lane of this chunk, else the carry
      const unsigned lower = m & below;
      const int pl = lower ? 31 - __clz( lower ) : 0;
      const double sb = __shfl_sync( kFull, b, pl ), sx = __shfl_sync( kFull, xsb, pl );
      double pf = lower ? sb : prev_first;
      const double ps = lower ? sx : prev_second;
      const bool first_ep = keep && next_ep && !lower;
      if ( first_ep ) {
        const double db_real = b - pf;
        pf -= db_real * ( 1.0 / 3.0 );
      }
      double term = 0.0;
      if ( keep ) {
        term = 0.5 * ( b - pf ) * ( xsb + ps );
        const int pos = n + __popc( lower );
        info[o + pos - 1] = rr[ib].info;
        bx[o + pos] = b;
        by[o + pos] = xsb;
      }
      for ( int k = 0; k < 32; ++k ) {
        const double tk = __shfl_sync( kFull, term, k );
        if ( ( m >> k ) & 1u )
          tot.add( tk );
      }
      if ( m ) {
        const int fl = __ffs( m ) - 1, ll = 31 - __clz( m );
        const double pfm = __shfl_sync( kFull, pf, fl );
        if ( next_ep )
          bx0 = pfm;
        next_ep = false;
        prev_first = __shfl_sync( kFull, b, ll );
        prev_second = __shfl_sync( kFull, xsb, ll );
        n += __popc( m );
      }
    }
    if ( lane == 0 ) {
      bx[o] = bx0;
      by[o] = 0.0;
    }
    double xs_total = tot.sum() * sigma_bound / ( 4 * x );
    if ( !( xs_total >= 0.0 ) )
      xs_total = 0.0;
    if ( lane == 0 )
      xs_out[ie] = xs_total;
    if ( xs_total == 0.0 )
      return;
    if ( lane == 0 ) {
      kind[ie] = 1;
      ibl_out[ie] = ibeta_low;
      nbeta_out[ie] = n;
      fbkep[ie] = starts ? beta_lower_limit : 1.0;
    }
    __syncwarp();
    // PointwiseDist (NCPointwiseDist.cc:28-74)
    for ( int i = lane; i < n; i += 32 ) {
      const double y = by[o + i];
      if ( y < 0.0 || isinf( y ) || ( i > 0 && bx[o + i] < bx[o + i - 1] ) )
        atomicExch( err, 1 );
    }
    StableSum area;
    if ( lane == 0 )
      bcdf[o] = 0.0;
    for ( int base = 1; base < n; base += 32 ) {
      const int i = base + lane;
      double a = 0.0;
      if ( i < n ) {
        a = ( bx[o + i] - bx[o + i - 1] ) * 0.5 * ( by[o + i] + by[o + i - 1] );
        if ( a < 0 )
          atomicExch( err, 1 );
      }
      double mine = 0.0;
      for ( int k = 0; k < 32; ++k ) {
        const double ak = __shfl_sync( kFull, a, k );
        if ( base + k < n ) {
          area.add( ak );
          if ( lane == k )
            mine = area.sum();
        }
      }
      if ( i < n )
        bcdf[o + i] = mine;
    }
    const double tarea = area.sum();
    if ( !( tarea > 0.0 ) ) {
      if ( lane == 0 )
        atomicExch( err, 1 );
      return;
    }
    const double nf = 1.0 / tarea;
    __syncwarp();
    for ( int i = lane; i < n; i += 32 ) {
      bcdf[o + i] *= nf;
      by[o + i] *= nf;
    }
    __syncwarp();
    if ( lane == 0 )
      bcdf[o + n - 1] = 1.0;
  }

  // Compaction into the host builder's layout: energy point ie's nbeta beta
  // points go to [off[ie], off[ie]+nbeta) of bx/by/bcdf, its nbeta-1 alpha
  // samplers and one zero pad to the same range of info.
  __global__ void k_compact( int ne, int nb, const int32_t* nbeta, const int64_t* off, const double* sbx,
                             const double* sby, const double* sbcdf, const ncgb_alpha_info* sinfo, double* bx,
                             double* by, double* bcdf, ncgb_alpha_info* info )
  {
    const int ie = blockIdx.y;
    const int n = nbeta[ie];
    const size_t o = (size_t)ie * ( nb + 1 );
    const int64_t d = off[ie];
    for ( int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x ) {
      bx[d + i] = sbx[o + i];
      by[d + i] = sby[o + i];
      bcdf[d + i] = sbcdf[o + i];
      if ( i < n - 1 ) {
        info[d + i] = sinfo[o + i];
      } else {
        ncgb_alpha_info z;
        memset( &z, 0, sizeof(z) );
        info[d + i] = z;
      }
    }
  }

  void check( cudaError_t e, const char* what )
  {
    if ( e != cudaSuccess )
      throw ncgb::Error( std::string( "device table derivation: " ) + what + ": " + cudaGetErrorString( e ) );
  }

  // One device allocation carved into 256-byte aligned arrays (first pass
  // sizes it, second pass hands out pointers).
  struct Carve {
    char* base = nullptr;
    size_t used = 0;
    template<class T> T* take( size_t n )
    {
      T* q = reinterpret_cast<T*>( base ? base + used : nullptr );
      used += ( n * sizeof(T) + 255 ) & ~size_t(255);
      return q;
    }
  };

  struct DevBlock {
    void* p = nullptr;
    ~DevBlock() { if ( p ) cudaFree( p ); }
  };
}

namespace ncgb {

  // deriveSAB on the current CUDA device for many components at once (one
  // allocation, one copy per array type each way, the kernels launched per
  // component on one stream): same outputs as the host builder.
  // Up to 16 non-blocking streams, handed out round-robin; destroyed at scope exit.
  struct Streams {
    std::vector<cudaStream_t> s;
    explicit Streams( size_t n )
    {
      s.resize( n < 16 ? ( n ? n : 1 ) : 16 );
      for ( auto& x : s )
        check( cudaStreamCreateWithFlags( &x, cudaStreamNonBlocking ), "cudaStreamCreate" );
    }
    ~Streams()
    {
      for ( auto x : s )
        cudaStreamDestroy( x );
    }
    Streams( const Streams& ) = delete;
    Streams& operator=( const Streams& ) = delete;
    cudaStream_t operator[]( size_t k ) const { return s[k % s.size()]; }
    void sync() const
    {
      for ( auto x : s )
        check( cudaStreamSynchronize( x ), "table derivation kernels" );
    }
  };

  // One group of components in one device allocation (deriveSABDeviceMany).
  std::vector<SABDerived> deriveGroup( const std::vector<const SABInput*>& ins )
  {
    const size_t nc = ins.size();
    std::vector<SABDerived> out( nc );
    if ( nc == 0 )
      return out;
    // NCGB_TABLES_TIMING=1: wall-clock time of each phase on stderr
    static const bool timing = [] {
      const char* v = std::getenv( "NCGB_TABLES_TIMING" );
      return v && *v && *v != '0';
    }();
    auto tmark = std::chrono::steady_clock::now();
    std::string tlog;
    auto mark = [&]( const char* what ) {
      if ( !timing )
        return;
      cudaDeviceSynchronize();
      auto now = std::chrono::steady_clock::now();
      char buf[96];
      std::snprintf( buf, sizeof buf, " %s %.1f ms;", what,
                     std::chrono::duration<double, std::milli>( now - tmark ).count() );
      tlog += buf;
      tmark = now;
    };
    struct Sz { size_t na, nb, ne, nslot; };
    std::vector<Sz> sz( nc );
    for ( size_t k = 0; k < nc; ++k ) {
      const SABInput& in = *ins[k];
      sz[k] = { in.alpha.size(), in.beta.size(), in.egrid.size(), in.egrid.size() * ( in.beta.size() + 1 ) };
      if ( sz[k].na < 2 || sz[k].nb < 2 || in.sab.size() != sz[k].na * sz[k].nb )
        throw Error( "SAB kernel with inconsistent grid sizes" );
      if ( sz[k].ne < 2 )
        throw Error( "SAB energy grid too small" );
    }
    // per-component element offsets into the concatenated arrays
    std::vector<size_t> oa( nc + 1, 0 ), ob( nc + 1, 0 ), os( nc + 1, 0 ), oe( nc + 1, 0 ), orw( nc + 1, 0 ),
                        osl( nc + 1, 0 );
    for ( size_t k = 0; k < nc; ++k ) {
      oa[k + 1] = oa[k] + sz[k].na;
      ob[k + 1] = ob[k] + sz[k].nb;
      os[k + 1] = os[k] + sz[k].na * sz[k].nb;
      oe[k + 1] = oe[k] + sz[k].ne;
      orw[k + 1] = orw[k] + sz[k].ne * sz[k].nb;
      osl[k + 1] = osl[k] + sz[k].nslot;
    }
    double *d_alpha, *d_beta, *d_sab, *d_egrid, *d_log, *d_cum, *d_bx, *d_by, *d_bcdf, *d_xs, *d_fbkep;
    double *c_bx, *c_by, *c_bcdf;
    ncgb_alpha_info *d_info, *c_info;
    BetaRow* d_rows;
    int32_t *d_kind, *d_ibl, *d_nbeta, *d_err;
    int64_t* d_off;
    DevBlock blk;
    for ( int pass = 0; pass < 2; ++pass ) {
      Carve c;
      if ( pass == 1 )
        c.base = static_cast<char*>( blk.p );
      d_alpha = c.take<double>( oa[nc] );
      d_beta = c.take<double>( ob[nc] );
      d_sab = c.take<double>( os[nc] );
      d_egrid = c.take<double>( oe[nc] );
      d_log = c.take<double>( os[nc] );
      d_cum = c.take<double>( os[nc] );
      d_rows = c.take<BetaRow>( orw[nc] );
      d_bx = c.take<double>( osl[nc] );
      d_by = c.take<double>( osl[nc] );
      d_bcdf = c.take<double>( osl[nc] );
      d_info = c.take<ncgb_alpha_info>( osl[nc] );
      c_bx = c.take<double>( osl[nc] );
      c_by = c.take<double>( osl[nc] );
      c_bcdf = c.take<double>( osl[nc] );
      c_info = c.take<ncgb_alpha_info>( osl[nc] );
      d_xs = c.take<double>( oe[nc] );
      d_fbkep = c.take<double>( oe[nc] );
      d_kind = c.take<int32_t>( oe[nc] );
      d_ibl = c.take<int32_t>( oe[nc] );
      d_nbeta = c.take<int32_t>( oe[nc] );
      d_off = c.take<int64_t>( oe[nc] );
      d_err = c.take<int32_t>( 1 );
      if ( pass == 0 )
        check( cudaMalloc( &blk.p, c.used ), "cudaMalloc" );
    }
    mark( "allocation" );
    // inputs straight from each component's arrays to its place on the device
    for ( size_t k = 0; k < nc; ++k ) {
      check( cudaMemcpy( d_alpha + oa[k], ins[k]->alpha.data(), sz[k].na * 8, cudaMemcpyHostToDevice ), "H2D" );
      check( cudaMemcpy( d_beta + ob[k], ins[k]->beta.data(), sz[k].nb * 8, cudaMemcpyHostToDevice ), "H2D" );
      check( cudaMemcpy( d_sab + os[k], ins[k]->sab.data(), sz[k].na * sz[k].nb * 8, cudaMemcpyHostToDevice ),
             "H2D" );
      check( cudaMemcpy( d_egrid + oe[k], ins[k]->egrid.data(), sz[k].ne * 8, cudaMemcpyHostToDevice ), "H2D" );
    }
    mark( "inputs to device" );
    check( cudaMemset( d_err, 0, 4 ), "memset" );
    // the legacy-stream copies and memset finished before the non-blocking
    // streams below start (a pageable copy may return before its DMA ends)
    check( cudaDeviceSynchronize(), "H2D" );
    // Components are independent, and k_logcumul / k_epoints run a serial
    // loop per beta row / energy point on a handful of blocks: each
    // component's chain goes to one of several streams so that the
    // components run side by side.
    Streams st( nc );
    for ( size_t k = 0; k < nc; ++k ) {
      const int na = (int)sz[k].na, nb = (int)sz[k].nb, ne = (int)sz[k].ne;
      cudaStream_t sk = st[k];
      k_logcumul<<<( nb + 3 ) / 4, 128, 0, sk>>>( d_alpha + oa[k], d_sab + os[k], na, nb, d_log + os[k], d_cum + os[k] );
      k_betarows<<<dim3( ( (unsigned)nb + 127 ) / 128, (unsigned)ne ), 128, 0, sk>>>(
        d_alpha + oa[k], d_beta + ob[k], d_sab + os[k], d_log + os[k], d_cum + os[k], na, nb, d_egrid + oe[k],
        ins[k]->kT, d_rows + orw[k] );
      k_epoints<<<( ne + 3 ) / 4, 128, 0, sk>>>( d_beta + ob[k], nb, d_egrid + oe[k], ne, ins[k]->kT, ins[k]->sigma_bound,
                                           d_rows + orw[k], d_bx + osl[k], d_by + osl[k], d_bcdf + osl[k],
                                           d_info + osl[k], d_xs + oe[k], d_kind + oe[k], d_ibl + oe[k],
                                           d_nbeta + oe[k], d_fbkep + oe[k], d_err );
    }
    check( cudaGetLastError(), "table derivation kernels" );
    st.sync();
    mark( "derivation kernels" );
    // per-point offsets of every component (host scan over the small counts)
    std::vector<int32_t> kind( oe[nc] ), ibl( oe[nc] ), nbeta( oe[nc] );
    check( cudaMemcpy( nbeta.data(), d_nbeta, oe[nc] * 4, cudaMemcpyDeviceToHost ), "D2H" );
    std::vector<int64_t> offs( oe[nc] );
    std::vector<size_t> ot( nc + 1, 0 );   // concatenated compact totals
    for ( size_t k = 0; k < nc; ++k ) {
      int64_t tot = 0;
      for ( size_t ie = 0; ie < sz[k].ne; ++ie ) {
        offs[oe[k] + ie] = tot;
        tot += nbeta[oe[k] + ie];
      }
      ot[k + 1] = ot[k] + (size_t)tot;
    }
    // compact positions: component k's points start at ot[k] in c_*
    std::vector<int64_t> goffs( oe[nc] );
    for ( size_t k = 0; k < nc; ++k )
      for ( size_t ie = 0; ie < sz[k].ne; ++ie )
        goffs[oe[k] + ie] = (int64_t)ot[k] + offs[oe[k] + ie];
    check( cudaMemcpy( d_off, goffs.data(), oe[nc] * 8, cudaMemcpyHostToDevice ), "H2D" );
    check( cudaDeviceSynchronize(), "H2D" );
    for ( size_t k = 0; k < nc; ++k ) {
      const int nb = (int)sz[k].nb, ne = (int)sz[k].ne;
      k_compact<<<dim3( ( (unsigned)nb + 128 ) / 128, (unsigned)ne ), 128, 0, st[k]>>>(
        ne, nb, d_nbeta + oe[k], d_off + oe[k], d_bx + osl[k], d_by + osl[k], d_bcdf + osl[k], d_info + osl[k],
        c_bx, c_by, c_bcdf, c_info );
    }
    check( cudaGetLastError(), "k_compact" );
    st.sync();
    mark( "compaction" );
    std::vector<double> xs( oe[nc] ), fbk( oe[nc] );
    int32_t err = 0;
    check( cudaMemcpy( xs.data(), d_xs, oe[nc] * 8, cudaMemcpyDeviceToHost ), "D2H" );
    check( cudaMemcpy( fbk.data(), d_fbkep, oe[nc] * 8, cudaMemcpyDeviceToHost ), "D2H" );
    check( cudaMemcpy( kind.data(), d_kind, oe[nc] * 4, cudaMemcpyDeviceToHost ), "D2H" );
    check( cudaMemcpy( ibl.data(), d_ibl, oe[nc] * 4, cudaMemcpyDeviceToHost ), "D2H" );
    check( cudaMemcpy( &err, d_err, 4, cudaMemcpyDeviceToHost ), "D2H" );
    if ( err )
      throw Error( "PointwiseDist: invalid beta distribution at an energy-grid point" );
    // results straight into each component's arrays
    auto fetch = []( auto& vec, const auto* src, size_t n ) {
      vec.resize( n );
      if ( n )
        check( cudaMemcpy( vec.data(), src, n * sizeof( *src ), cudaMemcpyDeviceToHost ), "D2H" );
    };
    for ( size_t k = 0; k < nc; ++k ) {
      SABDerived& d = out[k];
      const SABInput& in = *ins[k];
      fetch( d.logsab, d_log + os[k], os[k + 1] - os[k] );
      fetch( d.cumul, d_cum + os[k], os[k + 1] - os[k] );
      fetch( d.bx, c_bx + ot[k], ot[k + 1] - ot[k] );
      fetch( d.by, c_by + ot[k], ot[k + 1] - ot[k] );
      fetch( d.bcdf, c_bcdf + ot[k], ot[k + 1] - ot[k] );
      fetch( d.info, c_info + ot[k], ot[k + 1] - ot[k] );
      d.xs.assign( xs.begin() + oe[k], xs.begin() + oe[k + 1] );
      // per-point arrays in the host builder's layout (NCSABIntegrator.cc:283-309)
      for ( size_t ie = 0; ie < sz[k].ne; ++ie ) {
        const size_t g = oe[k] + ie;
        d.kind.push_back( kind[g] );
        d.offset.push_back( offs[g] );
        d.ibetaoffset.push_back( kind[g] ? ibl[g] : 0 );
        d.nbeta.push_back( kind[g] ? nbeta[g] : 0 );
        d.fbkep.push_back( kind[g] ? fbk[g] : 0.0 );
      }
      const double emax = in.egrid.back();
      const double extxs_emax = in.ext_sigma_free * freeGasXSShapeASq( in.ext_ca * emax );
      d.kext = ( d.xs.back() - extxs_emax ) * emax;
      d.k1 = d.xs.back() * emax;
      d.k2 = extxs_emax * emax;
    }
    mark( "results to host" );
    if ( timing )
      std::fprintf( stderr, "ncgb table derivation (%zu components, %.1f MB compact):%s\n", nc,
                    ot[nc] * ( 24.0 + sizeof( ncgb_alpha_info ) ) / 1e6, tlog.c_str() );
    return out;
  }

  // Device bytes of one component in deriveGroup's allocation (inputs, logS
  // and cumulative integrals, per-row results, per-point results before and
  // after compaction, per-point scalars).
  size_t groupBytes( const SABInput& in )
  {
    const size_t na = in.alpha.size(), nb = in.beta.size(), ne = in.egrid.size(), slots = ne * ( nb + 1 );
    return 8 * ( na + nb + 3 * na * nb + ne ) + sizeof( BetaRow ) * ne * nb
           + 2 * slots * ( 24 + sizeof( ncgb_alpha_info ) ) + ne * 32 + 4096;
  }

  // Components in groups whose allocation stays under NCGB_TABLES_DEVICE_MB
  // (default 16384 MB; a component larger than that is a group of its own),
  // so that a large temperature grid does not need its whole derivation
  // resident at once.
  std::vector<SABDerived> deriveSABDeviceMany( const std::vector<const SABInput*>& ins )
  {
    static const size_t budget = [] {
      const char* v = std::getenv( "NCGB_TABLES_DEVICE_MB" );
      const long long mb = v ? std::atoll( v ) : 0;
      return (size_t)( mb > 0 ? mb : 16384 ) << 20;
    }();
    std::vector<SABDerived> out;
    out.reserve( ins.size() );
    size_t k = 0;
    while ( k < ins.size() ) {
      std::vector<const SABInput*> g;
      size_t bytes = 0;
      while ( k < ins.size() && ( g.empty() || bytes + groupBytes( *ins[k] ) <= budget ) ) {
        bytes += groupBytes( *ins[k] );
        g.push_back( ins[k++] );
      }
      for ( auto& d : deriveGroup( g ) )
        out.push_back( std::move( d ) );
    }
    return out;
  }

  SABDerived deriveSABDevice( const SABInput& in )
  {
    return std::move( deriveSABDeviceMany( { &in } ).front() );
  }
}
