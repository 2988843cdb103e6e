// Host-only part of the C ABI: load a material bundle and build its flat
// tables in host memory, without touching a GPU.  The tests and the CPU
// oracle use it to read exactly the tables the kernels read.
#include "ncgb_host.hh"
#include "ncgb_proposal.hh"
#include "ncrystal_gb300.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace {
  struct HostTables {
    std::shared_ptr<ncgb::MaterialTables> mt;
    ncgb::Proposal lp[NCGB_MAX_COMP];   // learned proposals set for the oracle
  };
  thread_local std::string t_lasterr;

  ncgb_material_view hostView( HostTables* h )
  {
    ncgb_material_view v = h->mt->relocate( h->mt->arena().data() );
    for ( int ic = 0; ic < v.ncomp; ++ic )
      if ( !h->lp[ic].hdr.empty() ) {
        v.comp[ic].sab.lp_hdr = h->lp[ic].hdr.data();
        v.comp[ic].sab.lp_slot = h->lp[ic].slot.data();
        v.comp[ic].sab.lp_cell = h->lp[ic].cell.data();
        v.comp[ic].sab.lp_seg = h->lp[ic].seg.data();
      }
    return v;
  }
}

extern "C" {

void* ncgb_tables_load( const char* bundle_path )
{
  try {
    auto b = ncgb::Bundle::load( bundle_path );
    auto* h = new HostTables;
    h->mt = ncgb::MaterialTables::build( b );
    return h;
  } catch ( std::exception& e ) {
    t_lasterr = e.what();
    return nullptr;
  }
}

const char* ncgb_tables_lasterror( void ) { return t_lasterr.c_str(); }

int ncgb_tables_view( void* handle, ncgb_material_view* out )
{
  if ( !handle || !out )
    return 1;
  *out = hostView( static_cast<HostTables*>( handle ) );
  return 0;
}

// Learned-proposal tables of SAB component 'comp' from knots[ne*62]
// (asinh(beta) per egrid point), allowed[ne] optional; hdr_out[ne],
// slot_out[ne*NCGB_LP_K], cell_out[ne*NCGB_LP_K] and seg_out[*nseg] receive
// them.  Returns 0 on success, 2 (with *nseg set to the number of pieces) if
// seg_out is NULL or *nseg too small, 1 on error.
int ncgb_tables_build_proposal( void* handle, int comp, const float* knots, const unsigned char* allowed,
                                double min_accept, void* hdr_out, void* slot_out, void* cell_out, void* seg_out,
                                unsigned long* nseg )
{
  try {
    if ( !handle || !knots || !nseg )
      throw ncgb::Error( "ncgb_tables_build_proposal: null argument" );
    auto* h = static_cast<HostTables*>( handle );
    ncgb_material_view v = h->mt->relocate( h->mt->arena().data() );
    if ( comp < 0 || comp >= v.ncomp || v.comp[comp].type != NCGB_COMP_SAB )
      throw ncgb::Error( "ncgb_tables_build_proposal: component is not an S(alpha,beta) component" );
    ncgb::Proposal P = ncgb::buildProposal( v.comp[comp].sab, knots, NCGB_LP_NKNOTS, allowed, min_accept );
    if ( !seg_out || *nseg < P.seg.size() ) {
      *nseg = P.seg.size();
      return 2;
    }
    if ( !hdr_out || !slot_out || !cell_out )
      throw ncgb::Error( "ncgb_tables_build_proposal: null output array" );
    *nseg = P.seg.size();
    std::memcpy( hdr_out, P.hdr.data(), P.hdr.size() * sizeof(ncgb_lp_hdr) );
    std::memcpy( slot_out, P.slot.data(), P.slot.size() * sizeof(ncgb_lp_slot) );
    std::memcpy( cell_out, P.cell.data(), P.cell.size() * sizeof(ncgb_lp_cell) );
    std::memcpy( seg_out, P.seg.data(), P.seg.size() * sizeof(ncgb_lp_seg) );
    return 0;
  } catch ( std::exception& e ) {
    t_lasterr = e.what();
    return 1;
  }
}

// Makes ncgb_tables_view carry these proposal tables for component 'comp'
// (copies; hdr NULL removes them).
int ncgb_tables_set_proposal( void* handle, int comp, const void* hdr, const void* slot, const void* cell,
                              const void* seg, unsigned long nseg )
{
  if ( !handle )
    return 1;
  auto* h = static_cast<HostTables*>( handle );
  ncgb_material_view v = h->mt->relocate( h->mt->arena().data() );
  if ( comp < 0 || comp >= v.ncomp || v.comp[comp].type != NCGB_COMP_SAB )
    return 1;
  ncgb::Proposal& P = h->lp[comp];
  if ( !hdr ) {
    P = ncgb::Proposal();
    return 0;
  }
  if ( !slot || !cell || !seg )
    return 1;
  const std::size_t ne = v.comp[comp].sab.ne;
  P.hdr.assign( static_cast<const ncgb_lp_hdr*>( hdr ), static_cast<const ncgb_lp_hdr*>( hdr ) + ne );
  P.slot.assign( static_cast<const ncgb_lp_slot*>( slot ), static_cast<const ncgb_lp_slot*>( slot ) + ne * NCGB_LP_K );
  P.cell.assign( static_cast<const ncgb_lp_cell*>( cell ), static_cast<const ncgb_lp_cell*>( cell ) + ne * NCGB_LP_K );
  P.seg.assign( static_cast<const ncgb_lp_seg*>( seg ), static_cast<const ncgb_lp_seg*>( seg ) + nseg );
  return 0;
}

unsigned long ncgb_tables_bytes( void* handle )
{
  return handle ? static_cast<HostTables*>( handle )->mt->arenaBytes() : 0;
}

void ncgb_tables_free( void* handle )
{
  delete static_cast<HostTables*>( handle );
}

}

extern "C" {

// Test support: look up one array (or scalar) of component 'comp' by name, in
// the host arena.  Returns 0 if found.
int ncgb_tables_array( void* handle, int comp, const char* name, const void** ptr, unsigned long* count )
{
  if ( !handle || !name || !ptr || !count )
    return 1;
  auto* h = static_cast<HostTables*>( handle );
  ncgb_material_view v = h->mt->relocate( h->mt->arena().data() );
  if ( comp < 0 || comp >= v.ncomp )
    return 1;
  const ncgb_comp_view& c = v.comp[comp];
  const std::string n( name );
  const ncgb_sab_view& s = c.sab;
  if ( c.type == NCGB_COMP_BRAGG ) {
    if ( n == "two_dE" ) { *ptr = c.bragg.two_dE; *count = c.bragg.n; return 0; }
    if ( n == "fdm_commul" ) { *ptr = c.bragg.fdm_commul; *count = c.bragg.n; return 0; }
    return 1;
  }
  if ( c.type != NCGB_COMP_SAB )
    return 1;
  const unsigned long ne = s.ne, nab = (unsigned long)s.na * s.nb;
  unsigned long nsmp = 0;
  for ( int i = 0; i < s.ne; ++i )
    nsmp += s.smp_nbeta[i];
  if ( n == "egrid" ) { *ptr = s.egrid; *count = ne; return 0; }
  if ( n == "xs" ) { *ptr = s.xs; *count = ne; return 0; }
  if ( n == "logsab" ) { *ptr = s.logsab; *count = nab; return 0; }
  if ( n == "cumul" ) { *ptr = s.cumul; *count = nab; return 0; }
  if ( n == "smp_kind" ) { *ptr = s.smp_kind; *count = ne; return 0; }
  if ( n == "smp_ibetaoffset" ) { *ptr = s.smp_ibetaoffset; *count = ne; return 0; }
  if ( n == "smp_nbeta" ) { *ptr = s.smp_nbeta; *count = ne; return 0; }
  if ( n == "smp_offset" ) { *ptr = s.smp_offset; *count = ne; return 0; }
  if ( n == "smp_fbkep" ) { *ptr = s.smp_fbkep; *count = ne; return 0; }
  if ( n == "bx" ) { *ptr = s.bx; *count = nsmp; return 0; }
  if ( n == "by" ) { *ptr = s.by; *count = nsmp; return 0; }
  if ( n == "bcdf" ) { *ptr = s.bcdf; *count = nsmp; return 0; }
  if ( n == "info" ) { *ptr = s.info; *count = nsmp; return 0; }
  if ( n == "ebkt" ) { *ptr = s.ebkt; *count = (unsigned long)s.ebkt_n + 1; return 0; }
  if ( n == "ebkt_f" ) { *ptr = s.ebkt_f; *count = (unsigned long)s.ebkt_f_n + 1; return 0; }
  if ( n == "egrid_f" ) { *ptr = s.egrid_f; *count = ne; return 0; }
  return 1;
}

int ncgb_tables_scalar( void* handle, int comp, const char* name, double* out )
{
  if ( !handle || !name || !out )
    return 1;
  auto* h = static_cast<HostTables*>( handle );
  const ncgb_material_view& v = h->mt->m_rel;
  if ( comp < 0 || comp >= v.ncomp )
    return 1;
  const ncgb_sab_view& s = v.comp[comp].sab;
  const std::string n( name );
  if ( n == "kext" ) { *out = s.kext; return 0; }
  if ( n == "ebkt_kmin" ) { *out = (double)s.ebkt_kmin; return 0; }
  if ( n == "ebkt_f_kmin" ) { *out = (double)s.ebkt_f_kmin; return 0; }
  if ( n == "k1" ) { *out = s.k1; return 0; }
  if ( n == "k2" ) { *out = s.k2; return 0; }
  if ( n == "type" ) { *out = v.comp[comp].type; return 0; }
  if ( n == "ncomp" ) { *out = v.ncomp; return 0; }
  return 1;
}

}

// ---- device-side S(alpha,beta) derivation: comparison with the host builder ----------
namespace {
  template<class T>
  void cmpInt( const std::vector<T>& a, const std::vector<T>& b, long long& bad )
  {
    if ( a.size() != b.size() ) { bad += 1 + (long long)std::max( a.size(), b.size() ); return; }
    for ( std::size_t i = 0; i < a.size(); ++i )
      if ( a[i] != b[i] ) ++bad;
  }

  void cmpDbl( double a, double b, double& maxrel, long long& ndiff )
  {
    if ( a == b || ( std::isnan( a ) && std::isnan( b ) ) )
      return;
    ++ndiff;
    const double d = std::fabs( a - b ), s = std::max( std::fabs( a ), std::fabs( b ) );
    const double r = s > 0 ? d / s : d;
    if ( !( r <= maxrel ) )
      maxrel = ( std::isinf( a ) || std::isinf( b ) ) ? INFINITY : std::max( maxrel, r );
  }

  void cmpDbl( const std::vector<double>& a, const std::vector<double>& b, double& maxrel, long long& ndiff,
               long long& bad )
  {
    if ( a.size() != b.size() ) { bad += 1; return; }
    for ( std::size_t i = 0; i < a.size(); ++i )
      cmpDbl( a[i], b[i], maxrel, ndiff );
  }

  // Host and device derivations of one component compared: integer arrays
  // must be identical; doubles are counted where they differ.
  void compareDerived( const ncgb::SABDerived& h, const ncgb::SABDerived& d, double& maxrel, long long& ndiff,
                       long long& bad )
  {
    cmpInt( h.kind, d.kind, bad );
    cmpInt( h.ibetaoffset, d.ibetaoffset, bad );
    cmpInt( h.nbeta, d.nbeta, bad );
    cmpInt( h.offset, d.offset, bad );
    cmpDbl( h.logsab, d.logsab, maxrel, ndiff, bad );
    cmpDbl( h.cumul, d.cumul, maxrel, ndiff, bad );
    cmpDbl( h.xs, d.xs, maxrel, ndiff, bad );
    cmpDbl( h.fbkep, d.fbkep, maxrel, ndiff, bad );
    cmpDbl( h.bx, d.bx, maxrel, ndiff, bad );
    cmpDbl( h.by, d.by, maxrel, ndiff, bad );
    cmpDbl( h.bcdf, d.bcdf, maxrel, ndiff, bad );
    cmpDbl( h.kext, d.kext, maxrel, ndiff );
    cmpDbl( h.k1, d.k1, maxrel, ndiff );
    cmpDbl( h.k2, d.k2, maxrel, ndiff );
    if ( h.info.size() != d.info.size() ) {
      ++bad;
      return;
    }
    for ( std::size_t i = 0; i < h.info.size(); ++i ) {
      const ncgb_alpha_info &x = h.info[i], &y = d.info[i];
      if ( x.front_idx != y.front_idx || x.back_idx != y.back_idx )
        ++bad;
      cmpDbl( x.front_alpha, y.front_alpha, maxrel, ndiff );
      cmpDbl( x.front_sval, y.front_sval, maxrel, ndiff );
      cmpDbl( x.front_logsval, y.front_logsval, maxrel, ndiff );
      cmpDbl( x.back_alpha, y.back_alpha, maxrel, ndiff );
      cmpDbl( x.back_sval, y.back_sval, maxrel, ndiff );
      cmpDbl( x.back_logsval, y.back_logsval, maxrel, ndiff );
      cmpDbl( x.prob_front, y.prob_front, maxrel, ndiff );
      cmpDbl( x.prob_notback, y.prob_notback, maxrel, ndiff );
    }
  }
}

extern "C" {

/* Derives the sampling tables of S(alpha,beta) component 'comp' of a bundle
 * with the host builder and with the device builder, and compares them:
 * integer arrays (sampler kinds, offsets, beta counts and offsets) must be
 * identical (n_int_mismatch counts differences); doubles are reported as the
 * number that differ and their largest relative difference.  Also returns
 * both derivation times (milliseconds, wall clock; the device's includes its
 * copies).  Returns 0, or 1 with ncgb_tables_lasterror set. */
int ncgb_sab_derive_compare( const char* bundle_path, int comp, double* max_rel_diff, long long* n_double_diff,
                             long long* n_int_mismatch, double* ms_host, double* ms_device )
{
  try {
    auto b = ncgb::Bundle::load( bundle_path );
    auto all = ncgb::sabInputs( b );
    auto it = all.find( comp );
    if ( it == all.end() )
      throw ncgb::Error( "component " + std::to_string( comp ) + " is not an S(alpha,beta) component" );
    const ncgb::SABInput& in = it->second;
    auto t0 = std::chrono::steady_clock::now();
    ncgb::SABDerived h = ncgb::deriveSAB( in );
    auto t1 = std::chrono::steady_clock::now();
    ncgb::SABDerived d = ncgb::deriveSABDevice( in );
    auto t2 = std::chrono::steady_clock::now();
    if ( ms_host ) *ms_host = std::chrono::duration<double, std::milli>( t1 - t0 ).count();
    if ( ms_device ) *ms_device = std::chrono::duration<double, std::milli>( t2 - t1 ).count();
    long long bad = 0, ndiff = 0;
    double maxrel = 0.0;
    compareDerived( h, d, maxrel, ndiff, bad );
    if ( max_rel_diff ) *max_rel_diff = maxrel;
    if ( n_double_diff ) *n_double_diff = ndiff;
    if ( n_int_mismatch ) *n_int_mismatch = bad;
    return 0;
  } catch ( std::exception& e ) {
    t_lasterr = e.what();
    return 1;
  }
}

/* The same over every S(alpha,beta) component of n bundles, the device side
 * as one batched derivation (ncgb_create_scatters' path).  ncomp receives
 * the number of components; the times are the totals over all of them. */
int ncgb_sab_derive_compare_many( const char* const* bundle_paths, unsigned long n, double* max_rel_diff,
                                  long long* n_double_diff, long long* n_int_mismatch, long long* ncomp,
                                  double* ms_host, double* ms_device )
{
  try {
    std::vector<std::map<int, ncgb::SABInput>> inputs;
    std::vector<const ncgb::SABInput*> flat;
    for ( unsigned long i = 0; i < n; ++i )
      inputs.push_back( ncgb::sabInputs( ncgb::Bundle::load( bundle_paths[i] ) ) );
    for ( auto& m : inputs )
      for ( auto& kv : m )
        flat.push_back( &kv.second );
    auto t0 = std::chrono::steady_clock::now();
    std::vector<ncgb::SABDerived> h;
    for ( auto* in : flat )
      h.push_back( ncgb::deriveSAB( *in ) );
    auto t1 = std::chrono::steady_clock::now();
    std::vector<ncgb::SABDerived> d = ncgb::deriveSABDeviceMany( flat );
    auto t2 = std::chrono::steady_clock::now();
    if ( ms_host ) *ms_host = std::chrono::duration<double, std::milli>( t1 - t0 ).count();
    if ( ms_device ) *ms_device = std::chrono::duration<double, std::milli>( t2 - t1 ).count();
    long long bad = 0, ndiff = 0;
    double maxrel = 0.0;
    if ( d.size() != h.size() )
      ++bad;
    for ( std::size_t i = 0; i < h.size() && i < d.size(); ++i )
      compareDerived( h[i], d[i], maxrel, ndiff, bad );
    if ( max_rel_diff ) *max_rel_diff = maxrel;
    if ( n_double_diff ) *n_double_diff = ndiff;
    if ( n_int_mismatch ) *n_int_mismatch = bad;
    if ( ncomp ) *ncomp = static_cast<long long>( flat.size() );
    return 0;
  } catch ( std::exception& e ) {
    t_lasterr = e.what();
    return 1;
  }
}

}
