// Host-only part of the C ABI: load a material bundle and build its flat
// tables in host memory, without touching a GPU.  The tests and the CPU
// oracle use it to read exactly the tables the kernels read.
#include "ncgb_host.hh"
#include "ncrystal_gb300.h"

#include <cstring>
#include <mutex>
#include <string>

namespace {
  struct HostTables {
    std::shared_ptr<ncgb::MaterialTables> mt;
  };
  thread_local std::string t_lasterr;
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
  auto* h = static_cast<HostTables*>( handle );
  *out = h->mt->relocate( h->mt->arena().data() );
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
  if ( n == "k1" ) { *out = s.k1; return 0; }
  if ( n == "k2" ) { *out = s.k2; return 0; }
  if ( n == "type" ) { *out = v.comp[comp].type; return 0; }
  if ( n == "ncomp" ) { *out = v.ncomp; return 0; }
  return 1;
}

}
