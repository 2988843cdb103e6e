// C ABI of the GPU scattering path: NCrystal-compatible handles, error state
// and batch entry points (declared in include/ncrystal_gb300.h).
//
// Mirrors ncrystal_core/src/cinterface/ncrystal.cc of NCrystal 4.4.2:
//   handles      ncrystal.cc:104-200 (type-tagged, ref-counted, unref by address)
//   errors       ncrystal.cc:281-322 (message, type, custom handler, halt-on-error)
//   _many calls  ncrystal.cc:1107-1141, :1201-1245, :1301-1324 (index layout and
//                error sentinels)
// The per-neutron work runs in the CUDA kernels of ncgb_kernels.cu; there is
// no CPU evaluation path in this library.
#include "ncgb_host.hh"
#include "ncgb_launch.hh"
#include "ncgb_mmc.hh"
#include "ncgb_mlp.hh"
#include "ncgb_proposal.hh"
#include "ncrystal_gb300.h"

#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <initializer_list>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

namespace {

  // ---- error state (ncrystal.cc:281-322) ------------------------------------
  int g_quiet = 0;
  int g_halt = 1;
  int g_waserror = 0;
  char g_errmsg[512];
  char g_errtype[64];
  void (*g_handler)(char*,char*) = nullptr;
  std::mutex g_errmtx;

  void setError( const char* msg, const char* etype ) noexcept
  {
    std::lock_guard<std::mutex> lock( g_errmtx );
    if ( !etype )
      etype = "ncrystal_c-interface";
    std::strncpy( g_errmsg, msg, sizeof(g_errmsg) - 1 );
    std::strncpy( g_errtype, etype, sizeof(g_errtype) - 1 );
    g_errmsg[sizeof(g_errmsg)-1] = '\0';
    g_errtype[sizeof(g_errtype)-1] = '\0';
    if ( g_handler )
      (*g_handler)( g_errtype, g_errmsg );
    g_waserror = 1;
    if ( !g_quiet )
      std::printf( "NCrystal ERROR [%s]: %s\n", g_errtype, g_errmsg );
    if ( g_halt ) {
      std::printf( "NCrystal terminating due to ERROR\n" );
      std::fflush( stdout );
      std::exit( 1 );
    }
  }

  // Exception types named like NCrystal's (NCException.hh:105-175).
  struct TypedError : std::runtime_error {
    std::string type;
    TypedError( const std::string& t, const std::string& m ) : std::runtime_error(m), type(t) {}
  };

  void handleError( const std::exception& e ) noexcept
  {
    if ( auto te = dynamic_cast<const TypedError*>( &e ) )
      setError( te->what(), te->type.c_str() );
    else if ( dynamic_cast<const ncgb::Error*>( &e ) )
      setError( e.what(), "BadInput" );
    else
      setError( e.what(), "std::runtime_error" );
  }

#define NCGB_CATCH catch ( std::exception& e ) { handleError( e ); }

  void checkCuda( cudaError_t err, const char* what )
  {
    if ( err != cudaSuccess )
      throw TypedError( "CalcError", std::string("CUDA error in ") + what + ": " + cudaGetErrorString(err) );
  }

  // ---- device-resident materials ---------------------------------------------
  struct DeviceMaterial {
    std::shared_ptr<ncgb::MaterialTables> tables;
    int device = -1;
    void* d_arena = nullptr;
    ncgb_material_view view;
    // learned beta proposals attached per component (device tables + host headers)
    void* d_lp[NCGB_MAX_COMP] = {};
    std::vector<ncgb_lp_hdr> h_lp[NCGB_MAX_COMP];
    ~DeviceMaterial()
    {
      int cur = -1;
      cudaGetDevice( &cur );
      cudaSetDevice( device );
      if ( d_arena )
        cudaFree( d_arena );
      for ( void* p : d_lp )
        if ( p )
          cudaFree( p );
      cudaSetDevice( cur );
    }
  };

  std::mutex g_matmtx;
  std::map<std::pair<std::string,int>, std::weak_ptr<DeviceMaterial>> g_matcache;

  // cfg-string canonical form: whitespace removed, parameters after the file
  // name sorted.  Bundles are looked up by this form.
  std::string canonicalCfg( const std::string& cfg )
  {
    std::string s;
    for ( char c : cfg )
      if ( !std::isspace( static_cast<unsigned char>(c) ) )
        s.push_back( c );
    std::vector<std::string> parts;
    std::string cur;
    for ( char c : s ) {
      if ( c == ';' ) { parts.push_back( cur ); cur.clear(); }
      else cur.push_back( c );
    }
    parts.push_back( cur );
    std::vector<std::string> params;
    for ( std::size_t i = 1; i < parts.size(); ++i )
      if ( !parts[i].empty() )
        params.push_back( parts[i] );
    std::sort( params.begin(), params.end() );
    std::string out = parts.front();
    for ( auto& p : params )
      out += ";" + p;
    return out;
  }

  std::string bundleFileName( const std::string& canon )
  {
    std::string f;
    for ( char c : canon )
      f.push_back( ( std::isalnum( static_cast<unsigned char>(c) ) || c == '.' || c == '=' || c == '-' || c == '_' ) ? c : '_' );
    return f + ".ncgb";
  }

  // Directory of this library's file.
  std::string libDir()
  {
    Dl_info info;
    if ( dladdr( reinterpret_cast<void*>( &libDir ), &info ) && info.dli_fname ) {
      std::string lib( info.dli_fname );
      auto pos = lib.rfind( '/' );
      return pos == std::string::npos ? std::string( "." ) : lib.substr( 0, pos );
    }
    return ".";
  }

  // Where bundles exported on demand are written: NCGB_BUNDLE_CACHE, else the
  // package's bundles/ directory (created if missing).
  std::string bundleCacheDir()
  {
    const char* env = std::getenv( "NCGB_BUNDLE_CACHE" );
    std::string d = env && *env ? std::string( env ) : libDir() + "/../bundles";
    struct stat st;
    if ( ::stat( d.c_str(), &st ) != 0 && ::mkdir( d.c_str(), 0755 ) != 0 && errno != EEXIST )
      throw TypedError( "FileNotFound", "cannot create the bundle cache directory " + d );
    return d;
  }

  std::vector<std::string> bundleDirs()
  {
    std::vector<std::string> dirs;
    if ( const char* env = std::getenv( "NCGB_BUNDLE_PATH" ) ) {
      std::string s( env ), cur;
      for ( char c : s ) {
        if ( c == ':' ) { if ( !cur.empty() ) dirs.push_back( cur ); cur.clear(); }
        else cur.push_back( c );
      }
      if ( !cur.empty() ) dirs.push_back( cur );
    }
    if ( const char* env = std::getenv( "NCGB_BUNDLE_CACHE" ) )
      if ( *env )
        dirs.push_back( env );
    const std::string libdir = libDir();
    dirs.push_back( libdir + "/../bundles" );
    dirs.push_back( libdir + "/bundles" );
    return dirs;
  }

  // A bundle for a cfg-string that has none: NCrystal's own material loading,
  // run in this process through the exporter library (NCGB_EXPORT_LIB, else
  // libncgb_export.so beside this library; it links the NCrystal library).
  // Returns the bundle's path, or "" with 'why' set if no exporter can be
  // loaded; throws NCrystal's error if the export itself fails.
  std::string exportOnDemand( const std::string& cfg, const std::string& fn, std::string& why )
  {
    static std::mutex mtx;
    std::lock_guard<std::mutex> lock( mtx );
    const char* env = std::getenv( "NCGB_EXPORT_LIB" );
    const std::string lib = env && *env ? std::string( env ) : libDir() + "/libncgb_export.so";
    void* dl = dlopen( lib.c_str(), RTLD_NOW | RTLD_LOCAL );
    if ( !dl ) {
      const char* e = dlerror();
      why = "no bundle exporter could be loaded (" + std::string( e ? e : lib ) + ")";
      return "";
    }
    using ExportFn = int ( * )( const char*, const char*, char*, unsigned long, char*, unsigned long );
    auto fct = reinterpret_cast<ExportFn>( dlsym( dl, "ncgb_export_bundle" ) );
    if ( !fct ) {
      why = "the bundle exporter " + lib + " has no ncgb_export_bundle";
      return "";
    }
    const std::string path = bundleCacheDir() + "/" + fn;
    char err[2048] = { 0 }, type[64] = { 0 };
    if ( fct( cfg.c_str(), path.c_str(), err, sizeof( err ), type, sizeof( type ) ) != 0 )
      throw TypedError( *type ? type : "BadInput", std::string( "exporting a bundle for \"" ) + cfg + "\": " + err );
    return path;
  }

  std::string findBundle( const std::string& cfg )
  {
    const std::string canon = canonicalCfg( cfg );
    const std::string fn = bundleFileName( canon );
    struct stat st;
    for ( auto& d : bundleDirs() ) {
      std::string p = d + "/" + fn;
      if ( ::stat( p.c_str(), &st ) == 0 )
        return p;
    }
    std::string why;
    const std::string p = exportOnDemand( cfg, fn, why );
    if ( !p.empty() )
      return p;
    throw TypedError( "FileNotFound", "No material bundle for cfg \"" + cfg + "\" (looked for " + fn
                      + " in NCGB_BUNDLE_PATH, NCGB_BUNDLE_CACHE and the package bundles/ directory), and "
                      + why + ". Material bundles are written by NCrystal's host-side material loading"
                      " (ncgb_export, or libncgb_export.so on demand)." );
  }

  // Upload built tables as a device material of the current device and cache it.
  std::shared_ptr<DeviceMaterial> uploadMaterial( const std::string& canon, int dev,
                                                  std::shared_ptr<ncgb::MaterialTables> tables )
  {
    auto dm = std::make_shared<DeviceMaterial>();
    dm->tables = std::move( tables );
    dm->device = dev;
    const std::size_t bytes = dm->tables->arenaBytes();
    checkCuda( cudaMalloc( &dm->d_arena, std::max<std::size_t>( bytes, 256 ) ), "cudaMalloc (material tables)" );
    checkCuda( cudaMemcpy( dm->d_arena, dm->tables->arena().data(), bytes, cudaMemcpyHostToDevice ),
               "cudaMemcpy (material tables)" );
    dm->view = dm->tables->relocate( dm->d_arena );
    g_matcache[std::make_pair( canon, dev )] = dm;
    return dm;
  }

  // Many materials at once (a temperature grid, a batch of crystals): their
  // S(alpha,beta) samplers derived in one batched device derivation.
  std::vector<std::shared_ptr<DeviceMaterial>> getMaterials( const std::vector<std::string>& cfgs )
  {
    int dev = 0;
    checkCuda( cudaGetDevice( &dev ), "cudaGetDevice" );
    std::lock_guard<std::mutex> lock( g_matmtx );
    std::vector<std::shared_ptr<DeviceMaterial>> out( cfgs.size() );
    std::vector<ncgb::Bundle> bundles;
    std::vector<std::size_t> todo;
    std::vector<std::string> canons;
    for ( std::size_t i = 0; i < cfgs.size(); ++i ) {
      const std::string canon = canonicalCfg( cfgs[i] );
      auto it = g_matcache.find( std::make_pair( canon, dev ) );
      if ( it != g_matcache.end() )
        if ( auto sp = it->second.lock() ) { out[i] = sp; continue; }
      bool dup = false;
      for ( std::size_t j = 0; j < canons.size(); ++j )
        if ( canons[j] == canon ) dup = true;
      if ( dup )
        continue;
      auto b = ncgb::Bundle::load( findBundle( cfgs[i] ) );
      if ( canonicalCfg( b.str("cfg") ) != canon )
        throw TypedError( "BadInput", "material bundle " + b.path() + " holds cfg \"" + b.str("cfg") + "\", not \""
                          + cfgs[i] + "\"" );
      bundles.push_back( std::move( b ) );
      todo.push_back( i );
      canons.push_back( canon );
    }
    std::vector<std::map<int, ncgb::SABInput>> inputs;
    std::vector<const ncgb::SABInput*> flat;
    for ( auto& b : bundles )
      inputs.push_back( ncgb::sabInputs( b ) );
    for ( auto& m : inputs )
      for ( auto& kv : m )
        flat.push_back( &kv.second );
    std::vector<ncgb::SABDerived> derived = ncgb::deriveSABDeviceMany( flat );
    std::size_t k = 0;
    for ( std::size_t j = 0; j < bundles.size(); ++j ) {
      std::map<int, ncgb::SABDerived> pre;
      for ( auto& kv : inputs[j] )
        pre.emplace( kv.first, std::move( derived[k++] ) );
      auto tables = ncgb::MaterialTables::build( bundles[j], &pre );
      out[todo[j]] = uploadMaterial( canons[j], dev, std::move( tables ) );
    }
    // duplicates of a material built in this call
    for ( std::size_t i = 0; i < cfgs.size(); ++i )
      if ( !out[i] )
        out[i] = g_matcache[std::make_pair( canonicalCfg( cfgs[i] ), dev )].lock();
    return out;
  }

  std::shared_ptr<DeviceMaterial> getMaterial( const std::string& cfg )
  {
    const std::string canon = canonicalCfg( cfg );
    const std::string path = findBundle( cfg );
    int dev = 0;
    checkCuda( cudaGetDevice( &dev ), "cudaGetDevice" );
    std::lock_guard<std::mutex> lock( g_matmtx );
    auto key = std::make_pair( canon, dev );
    auto it = g_matcache.find( key );
    if ( it != g_matcache.end() )
      if ( auto sp = it->second.lock() )
        return sp;
    auto bundle = ncgb::Bundle::load( path );
    if ( canonicalCfg( bundle.str("cfg") ) != canon )
      throw TypedError( "BadInput", "material bundle " + bundle.path() + " holds cfg \"" + bundle.str("cfg")
                        + "\", not \"" + cfg + "\"" );
    return uploadMaterial( canon, dev, ncgb::MaterialTables::build( bundle ) );
  }

  // ---- handles (ncrystal.cc:104-200) ------------------------------------------
  constexpr uint32_t kScatterTypeID = 0x7d6b0637; // same tag values as NCrystal's Scatter
  constexpr uint32_t kAbsTypeID = 0xede2eb9d;     // and Absorption (ncrystal.cc:207-231)
  constexpr uint64_t kDefaultSeed = 0x4e43727973746c21ull;

  // Mode of new handles and batches: the environment variable NCGB_MODE
  // ("exact" / "mixed", or 0 / 1); unset means exact.
  int defaultMode()
  {
    static const int m = [] {
      const char* v = std::getenv( "NCGB_MODE" );
      if ( !v || !*v )
        return NCGB_MODE_EXACT;
      const std::string s( v );
      if ( s == "mixed" || s == "1" )
        return NCGB_MODE_MIXED;
      if ( s == "exact" || s == "0" )
        return NCGB_MODE_EXACT;
      std::fprintf( stderr, "NCrystal WARNING: ignoring NCGB_MODE=%s (expected exact or mixed)\n", v );
      return NCGB_MODE_EXACT;
    }();
    return m;
  }

  int checkMode( int mode, const char* fct )
  {
    if ( mode != NCGB_MODE_EXACT && mode != NCGB_MODE_MIXED )
      throw TypedError( "BadInput", std::string( fct ) + ": mode must be NCGB_MODE_EXACT or NCGB_MODE_MIXED" );
    return mode;
  }

  struct ScatterObj;
  struct FingerPrint {
    uint32_t typeid_;
    ScatterObj* obj;
  };

  struct ScatterObj {
    FingerPrint fp;
    std::atomic<int> refcount{1};
    std::shared_ptr<DeviceMaterial> mat;
    std::string cfg;
    uint64_t seed = kDefaultSeed;
    uint32_t streamidx = 0;
    int mode = defaultMode();
    int sampler = NCGB_SAMPLER_PLAIN;
    bool absorption = false;   // an absorption handle (AbsOOV of the material)
    std::atomic<uint32_t> callseq{0};
    ScatterObj() { fp.typeid_ = kScatterTypeID; fp.obj = this; }
  };

  std::atomic<uint32_t> g_nextStream{1};

  ScatterObj& extract( void* internal, const char* fct )
  {
    if ( !internal )
      throw TypedError( "LogicError", std::string("Invalid (null) object handle passed to ") + fct );
    auto fp = static_cast<FingerPrint*>( internal );
    if ( fp->typeid_ != kScatterTypeID )
      throw TypedError( "LogicError", std::string("Invalid object handle type passed to ") + fct );
    return *fp->obj;
  }

  ncrystal_scatter_t makeHandle( ScatterObj* o ) { return ncrystal_scatter_t{ &o->fp }; }

  // Any process handle: a scatter or an absorption.
  ScatterObj& extractProc( void* internal, const char* fct )
  {
    if ( !internal )
      throw TypedError( "LogicError", std::string("Invalid (null) object handle passed to ") + fct );
    auto fp = static_cast<FingerPrint*>( internal );
    if ( fp->typeid_ != kScatterTypeID && fp->typeid_ != kAbsTypeID )
      throw TypedError( "LogicError", std::string("Invalid object handle type passed to ") + fct );
    return *fp->obj;
  }

  ScatterObj& extractAbs( void* internal, const char* fct )
  {
    ScatterObj& o = extractProc( internal, fct );
    if ( !o.absorption )
      throw TypedError( "LogicError", std::string("Invalid object handle type passed to ") + fct );
    return o;
  }

  // ---- per-thread scratch ----------------------------------------------------
  // Device buffers of one host thread: staging for host-array calls, and the
  // SAB queue + counters that every scatter batch uses.  Grow-only.  Batches
  // from one thread are ordered through 'done' (an event recorded after each
  // batch that the next batch's stream waits for), so the scratch is never
  // shared by two batches in flight.
  struct Scratch {
    int device = -1;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;   // host -> device copies of chunked calls
    cudaStream_t stream3 = nullptr;   // device -> host copies of chunked calls
    cudaEvent_t done = nullptr;
    cudaEvent_t ev_in[2] = {}, ev_k[2] = {}, ev_out[2] = {};   // per buffer slot of chunked calls
    cudaEvent_t ev_pick[2] = {};   // per slot: the pick pass done (cross-sections final)
    void* d_in = nullptr; std::size_t cap_in = 0;
    void* d_a = nullptr; std::size_t cap_a = 0;
    void* d_b = nullptr; std::size_t cap_b = 0;
    void* d_c = nullptr; std::size_t cap_c = 0;
    void* d_queue = nullptr; std::size_t cap_queue = 0;
    void* d_phase = nullptr; std::size_t cap_phase = 0;   // phase-profile counters
    ncgb::Work* d_work = nullptr;
    unsigned long last_nfailed = 0;
  };
  thread_local Scratch t_scratch;

  void ensure( void*& p, std::size_t& cap, std::size_t bytes )
  {
    if ( bytes <= cap )
      return;
    if ( p ) {
      checkCuda( cudaDeviceSynchronize(), "synchronize before re-allocating scratch" );
      cudaFree( p );
    }
    p = nullptr;
    cap = 0;
    std::size_t want = std::max<std::size_t>( bytes, 1 << 20 );
    checkCuda( cudaMalloc( &p, want ), "cudaMalloc (batch buffers)" );
    cap = want;
  }

  Scratch& scratchFor( const DeviceMaterial& dm )
  {
    Scratch& s = t_scratch;
    int cur = -1;
    checkCuda( cudaGetDevice( &cur ), "cudaGetDevice" );
    if ( cur != dm.device )
      checkCuda( cudaSetDevice( dm.device ), "cudaSetDevice" );
    if ( s.device != dm.device ) {
      // Buffers of another device are abandoned (not freed: that device may be
      // gone); a thread normally stays on one device.
      s = Scratch();
      s.device = dm.device;
      checkCuda( cudaStreamCreateWithFlags( &s.stream, cudaStreamNonBlocking ), "cudaStreamCreate" );
      checkCuda( cudaStreamCreateWithFlags( &s.stream2, cudaStreamNonBlocking ), "cudaStreamCreate" );
      checkCuda( cudaStreamCreateWithFlags( &s.stream3, cudaStreamNonBlocking ), "cudaStreamCreate" );
      checkCuda( cudaEventCreateWithFlags( &s.done, cudaEventDisableTiming ), "cudaEventCreate" );
      for ( int h = 0; h < 2; ++h ) {
        checkCuda( cudaEventCreateWithFlags( &s.ev_in[h], cudaEventDisableTiming ), "cudaEventCreate" );
        checkCuda( cudaEventCreateWithFlags( &s.ev_k[h], cudaEventDisableTiming ), "cudaEventCreate" );
        checkCuda( cudaEventCreateWithFlags( &s.ev_out[h], cudaEventDisableTiming ), "cudaEventCreate" );
        checkCuda( cudaEventCreateWithFlags( &s.ev_pick[h], cudaEventDisableTiming ), "cudaEventCreate" );
      }
      checkCuda( cudaEventRecord( s.done, s.stream ), "cudaEventRecord" );
      void* w = nullptr;
      checkCuda( cudaMalloc( &w, sizeof(ncgb::Work) ), "cudaMalloc" );
      s.d_work = static_cast<ncgb::Work*>( w );
    }
    return s;
  }

  uint32_t nextCall( ScatterObj& o ) { return o.callseq.fetch_add( 1, std::memory_order_relaxed ); }

  // Host arrays through the device in chunks of 'chunk' neutrons with two
  // buffer slots: copies in on stream2, kernels on the handle's stream,
  // copies out on stream3.  The copy-in of chunk k+2 waits only for the
  // kernels of chunk k (which read its slot), and the kernels of chunk k+2
  // for the copy-out of chunk k (which reads theirs), so that both copy
  // directions and the kernels overlap.  The launch records ev_pick[slot]
  // between its two passes; copyOutEarly (the cross-sections, final after
  // the pick pass) waits only for that, so it overlaps the chunk's own
  // S(alpha,beta) pass, and copyOut (E', mu) for the whole launch.
  // copyIn / launch / copyOutEarly / copyOut get (offset, count, slot,
  // stream).  Returns after the last copy-out.
  template<class CopyIn, class Launch, class CopyOutEarly, class CopyOut>
  void chunkPipeline( Scratch& s, uint64_t n, uint64_t chunk, CopyIn copyIn, Launch launch,
                      CopyOutEarly copyOutEarly, CopyOut copyOut )
  {
    uint64_t k = 0;
    for ( uint64_t off = 0, m = 0; off < n; off += m, ++k ) {
      // The last chunk after full ones goes in two halves: the pipeline's
      // tail (the last kernels and their copy-out, which nothing overlaps)
      // is then half as long.
      const uint64_t r = n - off;
      m = std::min<uint64_t>( chunk, r );
      if ( off > 0 && r <= chunk && 2 * r > chunk && r >= 2048 )
        m = ( ( r / 2 ) + 255 ) & ~255ull;
      const int h = static_cast<int>( k & 1 );
      checkCuda( cudaStreamWaitEvent( s.stream2, s.ev_k[h], 0 ), "cudaStreamWaitEvent" );
      copyIn( off, m, h, s.stream2 );
      checkCuda( cudaEventRecord( s.ev_in[h], s.stream2 ), "cudaEventRecord" );
      checkCuda( cudaStreamWaitEvent( s.stream, s.ev_in[h], 0 ), "cudaStreamWaitEvent" );
      checkCuda( cudaStreamWaitEvent( s.stream, s.ev_out[h], 0 ), "cudaStreamWaitEvent" );
      launch( off, m, h, s.stream );
      checkCuda( cudaEventRecord( s.ev_k[h], s.stream ), "cudaEventRecord" );
      checkCuda( cudaStreamWaitEvent( s.stream3, s.ev_pick[h], 0 ), "cudaStreamWaitEvent" );
      copyOutEarly( off, m, h, s.stream3 );
      checkCuda( cudaStreamWaitEvent( s.stream3, s.ev_k[h], 0 ), "cudaStreamWaitEvent" );
      copyOut( off, m, h, s.stream3 );
      checkCuda( cudaEventRecord( s.ev_out[h], s.stream3 ), "cudaEventRecord" );
    }
    checkCuda( cudaStreamSynchronize( s.stream3 ), "scatter kernels" );
  }

  void checkSize( unsigned long n_ekin, unsigned long repeat )
  {
    const unsigned long long tot = (unsigned long long)n_ekin * (unsigned long long)repeat;
    if ( repeat && tot / repeat != n_ekin )
      throw TypedError( "BadInput", "n_ekin*repeat overflows" );
    if ( tot > 0xffffffffull )
      throw TypedError( "BadInput", "n_ekin*repeat above 2^32 per call is not supported (neutron index of the random streams is 32 bits)" );
  }

  bool hasBragg( const ncgb_material_view& v )
  {
    for ( int i = 0; i < v.ncomp && i < NCGB_MAX_COMP; ++i )
      if ( v.comp[i].type == NCGB_COMP_BRAGG )
        return true;
    return false;
  }

  ncgb::Batch makeBatch( ScatterObj& o, Scratch& s, uint32_t call )
  {
    ncgb::Batch b;
    std::memset( &b, 0, sizeof(b) );
    b.seed = o.seed;
    b.callseq = call;
    b.stream = o.streamidx;
    b.fast = ( o.mode == NCGB_MODE_MIXED );
    b.learned = ( o.sampler == NCGB_SAMPLER_LEARNED );
    b.reorder = hasBragg( o.mat->view ) ? 1 : 0;
    b.work = s.d_work;
    b.queue = static_cast<ncgb::QEntry*>( s.d_queue );
    return b;
  }

  // Scatter batch on stream 'st', ordered after the thread's previous batch.
  void runBatch( const DeviceMaterial& dm, Scratch& s, ncgb::Batch& b, cudaStream_t st,
                 cudaEvent_t pickDone = nullptr )
  {
    ensure( s.d_queue, s.cap_queue, b.n_out * sizeof(ncgb::QEntry) );
    b.queue = static_cast<ncgb::QEntry*>( s.d_queue );
    checkCuda( cudaStreamWaitEvent( st, s.done, 0 ), "cudaStreamWaitEvent" );
    checkCuda( ncgb::launchScatter( dm.view, b, st, pickDone ), "scatter kernels" );
    checkCuda( cudaEventRecord( s.done, st ), "cudaEventRecord" );
  }

  // The failure counter accumulates over the batches of one call; the
  // per-batch queue counters are reset by launchScatter.
  void resetNFail( Scratch& s, cudaStream_t st )
  {
    checkCuda( cudaStreamWaitEvent( st, s.done, 0 ), "cudaStreamWaitEvent" );
    checkCuda( cudaMemsetAsync( &s.d_work->nfail, 0, sizeof(unsigned long long), st ), "memset" );
    checkCuda( cudaEventRecord( s.done, st ), "cudaEventRecord" );
  }

  unsigned long readNFail( Scratch& s, cudaStream_t st )
  {
    unsigned long long nfail = 0;
    checkCuda( cudaMemcpyAsync( &nfail, &s.d_work->nfail, sizeof(nfail), cudaMemcpyDeviceToHost, st ), "D2H" );
    checkCuda( cudaStreamSynchronize( st ), "scatter kernels" );
    s.last_nfailed = static_cast<unsigned long>( nfail );
    return s.last_nfailed;
  }

  // Host arrays in; H2D, kernels, D2H on the thread's stream.  Returns the
  // number of neutrons with a non-OK status.
  unsigned long runScatterMany( ScatterObj& o, const double* ekin, unsigned long n_ekin, unsigned long repeat,
                                int mode, double* out_a, double* out_b, bool copyBackPartial )
  {
    checkSize( n_ekin, repeat );
    const uint64_t n_out = (uint64_t)n_ekin * repeat;
    if ( n_out == 0 )
      return 0;
    DeviceMaterial& dm = *o.mat;
    Scratch& s = scratchFor( dm );
    ensure( s.d_in, s.cap_in, n_ekin * sizeof(double) );
    ensure( s.d_a, s.cap_a, n_out * sizeof(double) );
    ensure( s.d_b, s.cap_b, n_out * sizeof(double) );
    ncgb::Batch b = makeBatch( o, s, nextCall( o ) );
    b.ekin = s.d_in;
    b.n_ekin = n_ekin;
    b.n_out = n_out;
    b.mode = mode;
    b.out_a = s.d_a;
    b.out_b = s.d_b;
    resetNFail( s, s.stream );
    checkCuda( cudaMemcpyAsync( s.d_in, ekin, n_ekin * sizeof(double), cudaMemcpyHostToDevice, s.stream ), "H2D" );
    if ( mode == 1 ) {
      // genscatter leaves the outputs of failed neutrons untouched: start from
      // the caller's arrays.
      checkCuda( cudaMemcpyAsync( s.d_a, out_a, n_out * sizeof(double), cudaMemcpyHostToDevice, s.stream ), "H2D" );
      checkCuda( cudaMemcpyAsync( s.d_b, out_b, n_out * sizeof(double), cudaMemcpyHostToDevice, s.stream ), "H2D" );
    }
    runBatch( dm, s, b, s.stream );
    const unsigned long nfail = readNFail( s, s.stream );
    if ( nfail == 0 || copyBackPartial ) {
      checkCuda( cudaMemcpyAsync( out_a, s.d_a, n_out * sizeof(double), cudaMemcpyDeviceToHost, s.stream ), "D2H" );
      checkCuda( cudaMemcpyAsync( out_b, s.d_b, n_out * sizeof(double), cudaMemcpyDeviceToHost, s.stream ), "D2H" );
      checkCuda( cudaStreamSynchronize( s.stream ), "D2H" );
    }
    return nfail;
  }

  [[noreturn]] void throwSamplingFailure( unsigned long nfail )
  {
    std::ostringstream ss;
    ss << "Sampling failed for " << nfail << " neutron(s): a rejection loop reached its limit of attempts"
       << " (NCrystal: \"Rejection method failed to sample kinematically valid (alpha,beta) point\"), or the"
       << " (alpha,beta) -> mu conversion met E*E'=0 (NCrystal: \"convertAlphaBetaToDeltaEMu invalid for"
       << " beta=-E/kT\").";
    throw TypedError( "CalcError", ss.str() );
  }

  void warnOnce( std::atomic<bool>& flag, const char* msg )
  {
    bool expected = true;
    if ( flag.compare_exchange_strong( expected, false ) ) {
      std::printf( "NCrystal WARNING: %s\n", msg );
      std::fflush( stdout );
    }
  }
  std::atomic<bool> g_warn_genscatter_many{true};
  std::atomic<bool> g_warn_genscatter{true};

  // Zero-copy host calls: over the GB300's coherent NVLink-C2C the kernels
  // can read the energies from pinned host arrays and write the results there
  // directly, without staging copies.  Measured (2^24 neutrons): better for
  // FP32 I/O (corundum e2e 5.7-6.3e9 vs 5.2-5.5e9 scatters/s with copies),
  // worse for FP64 I/O (polyethylene 2.3-3.6e9 vs 4.6-4.9e9: the
  // S(alpha,beta) pass writes its results at scattered indices, which the
  // link turns into many small transactions).  Default: on for the FP32
  // calls, off otherwise; NCGB_ZERO_COPY=1 / 0 forces it on / off.
  bool zeroCopyFor( bool f32 )
  {
    const char* v = std::getenv( "NCGB_ZERO_COPY" );
    if ( v && *v )
      return std::string( v ) != "0";
    return f32;
  }

  // Device address of pinned, mapped host memory (cudaHostAlloc /
  // cudaHostRegister with UVA), or null for any other pointer.
  const void* mappedDevicePtr( const void* p )
  {
    if ( !p )
      return nullptr;
    cudaPointerAttributes a;
    if ( cudaPointerGetAttributes( &a, p ) != cudaSuccess ) {
      cudaGetLastError();
      return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
  }

  // All the given host arrays (nulls ignored) are mapped: their device
  // addresses, in order, into 'out'.
  bool allMapped( std::initializer_list<const void*> ptrs, std::vector<void*>& out )
  {
    out.clear();
    for ( const void* p : ptrs ) {
      if ( !p ) { out.push_back( nullptr ); continue; }
      const void* d = mappedDevicePtr( p );
      if ( !d )
        return false;
      out.push_back( const_cast<void*>( d ) );
    }
    return true;
  }

  // Neutrons per chunk of the copy pipeline (NCGB_CHUNK_LOG2, default 22).
  uint64_t copyChunk()
  {
    static const uint64_t c = [] {
      const char* v = std::getenv( "NCGB_CHUNK_LOG2" );
      const int k = v ? std::atoi( v ) : 22;
      return uint64_t(1) << ( k >= 16 && k <= 26 ? k : 22 );
    }();
    return c;
  }

  // The host-array fused entry points: the caller's pinned arrays directly
  // (zero-copy), or chunkPipeline's H2D / kernels / D2H over two halves of
  // the staging buffers.  The SAB queue and counters are shared by the
  // chunks, whose kernels run in order on the handle's stream.
  template<class T>
  void xsScatterHost( ScatterObj& o, const T* ekin, unsigned long n, T* xs, T* ef, T* mu )
  {
    checkSize( n, 1 );
    if ( n == 0 )
      return;
    DeviceMaterial& dm = *o.mat;
    Scratch& s = scratchFor( dm );
    std::vector<void*> mp;
    if ( zeroCopyFor( sizeof(T) == 4 ) && allMapped( { ekin, xs, ef, mu }, mp ) ) {
      // zero-copy: one batch straight over the caller's pinned arrays
      ensure( s.d_queue, s.cap_queue, n * sizeof(ncgb::QEntry) );
      resetNFail( s, s.stream );
      ncgb::Batch b = makeBatch( o, s, nextCall( o ) );
      b.reorder = 0;
      b.ekin = mp[0];
      b.in_f32 = b.out_f32 = ( sizeof(T) == 4 );
      b.n_ekin = b.n_out = n;
      b.out_xs = mp[1];
      b.out_a = mp[2];
      b.out_b = mp[3];
      runBatch( dm, s, b, s.stream );
      const unsigned long bad = readNFail( s, s.stream );
      if ( bad )
        throwSamplingFailure( bad );
      return;
    }
    const uint64_t chunk = std::min<uint64_t>( n, copyChunk() );
    ensure( s.d_in, s.cap_in, 2 * chunk * sizeof(T) );
    ensure( s.d_a, s.cap_a, 2 * chunk * sizeof(T) );
    ensure( s.d_b, s.cap_b, 2 * chunk * sizeof(T) );
    ensure( s.d_c, s.cap_c, 2 * chunk * sizeof(T) );
    ensure( s.d_queue, s.cap_queue, chunk * sizeof(ncgb::QEntry) );
    const uint32_t call = nextCall( o );
    resetNFail( s, s.stream );
    auto slot = [&]( void* base, int h ) { return static_cast<T*>( base ) + h * chunk; };
    chunkPipeline(
      s, n, chunk,
      [&]( uint64_t off, uint64_t m, int h, cudaStream_t cs ) {
        checkCuda( cudaMemcpyAsync( slot( s.d_in, h ), ekin + off, m * sizeof(T), cudaMemcpyHostToDevice, cs ), "H2D" );
      },
      [&]( uint64_t off, uint64_t m, int h, cudaStream_t cs ) {
        ncgb::Batch b = makeBatch( o, s, call );
        b.ekin = slot( s.d_in, h );
        b.in_f32 = b.out_f32 = ( sizeof(T) == 4 );
        b.n_ekin = b.n_out = m;
        b.index_offset = static_cast<uint32_t>( off );
        b.out_xs = xs ? slot( s.d_a, h ) : nullptr;
        b.out_a = ef ? slot( s.d_b, h ) : nullptr;
        b.out_b = mu ? slot( s.d_c, h ) : nullptr;
        runBatch( dm, s, b, cs, s.ev_pick[h] );
      },
      [&]( uint64_t off, uint64_t m, int h, cudaStream_t cs ) {
        if ( xs ) checkCuda( cudaMemcpyAsync( xs + off, slot( s.d_a, h ), m * sizeof(T), cudaMemcpyDeviceToHost, cs ), "D2H" );
      },
      [&]( uint64_t off, uint64_t m, int h, cudaStream_t cs ) {
        if ( ef ) checkCuda( cudaMemcpyAsync( ef + off, slot( s.d_b, h ), m * sizeof(T), cudaMemcpyDeviceToHost, cs ), "D2H" );
        if ( mu ) checkCuda( cudaMemcpyAsync( mu + off, slot( s.d_c, h ), m * sizeof(T), cudaMemcpyDeviceToHost, cs ), "D2H" );
      } );
    const unsigned long bad = readNFail( s, s.stream );
    if ( bad )
      throwSamplingFailure( bad );
  }

  template<class T>
  void fillSentinels( unsigned long n, T* xs, T* ef, T* mu )
  {
    for ( unsigned long k = 0; k < n; ++k ) {
      if ( xs ) xs[k] = T(-1);
      if ( ef ) ef[k] = T(-1);
      if ( mu ) mu[k] = T(-999);
    }
  }
}

extern "C" {

int ncrystal_sethaltonerror( int h ) { int old = g_halt; g_halt = h; return old; }
int ncrystal_setquietonerror( int q ) { int old = g_quiet; g_quiet = q; return old; }
int ncrystal_error( void ) { return g_waserror; }
const char* ncrystal_lasterror( void ) { return g_waserror ? g_errmsg : nullptr; }
const char* ncrystal_lasterrortype( void ) { return g_waserror ? g_errtype : nullptr; }
void ncrystal_clearerror( void ) { g_waserror = 0; g_errmsg[0] = '\0'; g_errtype[0] = '\0'; }
void ncrystal_seterrhandler( void (*handler)(char*,char*) ) { g_handler = handler; }

int ncrystal_version( void ) { return 4004002; }
const char* ncrystal_version_str( void ) { return "4.4.2"; }

// ---- reference counting ----------------------------------------------------
static void*& internalOf( void* addrhandle ) { return *reinterpret_cast<void**>( addrhandle ); }

int ncrystal_valid( void* object )
{
  if ( !object )
    return 0;
  return internalOf( object ) ? 1 : 0;
}

void ncrystal_invalidate( void* object )
{
  if ( ncrystal_valid( object ) )
    internalOf( object ) = nullptr;
}

int ncrystal_refcount( void* object )
{
  try {
    return extractProc( internalOf( object ), "ncrystal_refcount" ).refcount.load();
  } NCGB_CATCH;
  return -999;
}

void ncrystal_ref( void* object )
{
  try {
    extractProc( internalOf( object ), "ncrystal_ref" ).refcount.fetch_add( 1 );
  } NCGB_CATCH;
}

void ncrystal_unref( void* object )
{
  try {
    ScatterObj& o = extractProc( internalOf( object ), "ncrystal_unref" );
    if ( o.refcount.fetch_sub( 1 ) == 1 ) {
      delete &o;
      internalOf( object ) = nullptr;
    }
  } NCGB_CATCH;
}

// ---- factories -----------------------------------------------------------------
static ncrystal_scatter_t createScatter( const char* cfgstr, uint64_t seed )
{
  if ( !cfgstr )
    throw TypedError( "BadInput", "null cfg-string" );
  std::unique_ptr<ScatterObj> o( new ScatterObj );
  o->mat = getMaterial( cfgstr );
  o->cfg = cfgstr;
  o->seed = seed;
  return makeHandle( o.release() );
}

ncrystal_scatter_t ncgb_create_scatter_bundle( const char* bundle_path, unsigned long seed )
{
  try {
    if ( !bundle_path )
      throw TypedError( "BadInput", "ncgb_create_scatter_bundle: null path" );
    const std::string key = std::string( "bundle:" ) + bundle_path;
    int dev = 0;
    checkCuda( cudaGetDevice( &dev ), "cudaGetDevice" );
    std::shared_ptr<DeviceMaterial> mat;
    {
      std::lock_guard<std::mutex> lock( g_matmtx );
      auto it = g_matcache.find( std::make_pair( key, dev ) );
      if ( it != g_matcache.end() )
        mat = it->second.lock();
      if ( !mat ) {
        auto bundle = ncgb::Bundle::load( bundle_path );
        mat = uploadMaterial( key, dev, ncgb::MaterialTables::build( bundle ) );
      }
    }
    std::unique_ptr<ScatterObj> o( new ScatterObj );
    o->mat = mat;
    o->cfg = key;
    o->seed = static_cast<uint64_t>( seed );
    return makeHandle( o.release() );
  } NCGB_CATCH;
  return ncrystal_scatter_t{ nullptr };
}

int ncgb_samplescatterisotropic_keyed( ncrystal_scatter_t sc, double ekin, unsigned long long key,
                                       double* ekin_final, double* mu )
{
  try {
    if ( !ekin_final || !mu )
      throw TypedError( "BadInput", "ncgb_samplescatterisotropic_keyed: null output" );
    *ekin_final = -1.0;
    *mu = -999.0;
    ScatterObj& o = extract( sc.internal, "ncgb_samplescatterisotropic_keyed" );
    DeviceMaterial& dm = *o.mat;
    Scratch& s = scratchFor( dm );
    ensure( s.d_in, s.cap_in, sizeof(double) );
    ensure( s.d_a, s.cap_a, sizeof(double) );
    ensure( s.d_b, s.cap_b, sizeof(double) );
    // the neutron's stream: (key, 0, 0, the handle's stream index); the
    // handle's own call sequence is left alone
    ncgb::Batch b = makeBatch( o, s, 0 );
    b.seed = key;
    b.ekin = s.d_in;
    b.n_ekin = b.n_out = 1;
    b.out_a = s.d_a;
    b.out_b = s.d_b;
    resetNFail( s, s.stream );
    checkCuda( cudaMemcpyAsync( s.d_in, &ekin, sizeof(double), cudaMemcpyHostToDevice, s.stream ), "H2D" );
    runBatch( dm, s, b, s.stream );
    const unsigned long nfail = readNFail( s, s.stream );
    if ( nfail )
      throwSamplingFailure( nfail );
    double out[2];
    checkCuda( cudaMemcpyAsync( out, s.d_a, sizeof(double), cudaMemcpyDeviceToHost, s.stream ), "D2H" );
    checkCuda( cudaMemcpyAsync( out + 1, s.d_b, sizeof(double), cudaMemcpyDeviceToHost, s.stream ), "D2H" );
    checkCuda( cudaStreamSynchronize( s.stream ), "D2H" );
    *ekin_final = out[0];
    *mu = out[1];
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_bundle_cache_dir( char* out, unsigned long outlen )
{
  try {
    const std::string d = bundleCacheDir();
    if ( !out || outlen <= d.size() )
      throw TypedError( "BadInput", "ncgb_bundle_cache_dir: buffer too small" );
    std::memcpy( out, d.c_str(), d.size() + 1 );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_bundle_path( const char* cfgstr, char* out, unsigned long outlen )
{
  try {
    if ( !cfgstr )
      throw TypedError( "BadInput", "ncgb_bundle_path: null cfg-string" );
    const std::string p = findBundle( cfgstr );
    if ( !out || outlen <= p.size() )
      throw TypedError( "BadInput", "ncgb_bundle_path: buffer too small" );
    std::memcpy( out, p.c_str(), p.size() + 1 );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_create_scatters( const char* const* cfgstrs, unsigned long n, unsigned long seed, ncrystal_scatter_t* out )
{
  try {
    if ( !out || ( n && !cfgstrs ) )
      throw TypedError( "BadInput", "ncgb_create_scatters: null array" );
    std::vector<std::string> cfgs;
    for ( unsigned long i = 0; i < n; ++i ) {
      if ( !cfgstrs[i] )
        throw TypedError( "BadInput", "ncgb_create_scatters: null cfg-string" );
      cfgs.push_back( cfgstrs[i] );
    }
    auto mats = getMaterials( cfgs );
    for ( unsigned long i = 0; i < n; ++i ) {
      std::unique_ptr<ScatterObj> o( new ScatterObj );
      o->mat = mats[i];
      o->cfg = cfgs[i];
      o->seed = seed;
      out[i] = makeHandle( o.release() );
    }
    return 0;
  } NCGB_CATCH;
  for ( unsigned long i = 0; i < n; ++i )
    if ( out ) out[i].internal = nullptr;
  return 1;
}

ncrystal_scatter_t ncrystal_create_scatter( const char* cfgstr )
{
  try {
    return createScatter( cfgstr, kDefaultSeed );
  } NCGB_CATCH;
  return ncrystal_scatter_t{ nullptr };
}

ncrystal_scatter_t ncrystal_create_scatter_builtinrng( const char* cfgstr, unsigned long seed )
{
  try {
    return createScatter( cfgstr, static_cast<uint64_t>( seed ) );
  } NCGB_CATCH;
  return ncrystal_scatter_t{ nullptr };
}

static ncrystal_scatter_t cloneWithStream( ncrystal_scatter_t sc, uint32_t streamidx, const char* fct )
{
  ScatterObj& src = extract( sc.internal, fct );
  std::unique_ptr<ScatterObj> o( new ScatterObj );
  o->mat = src.mat;
  o->cfg = src.cfg;
  o->seed = src.seed;
  o->streamidx = streamidx;
  o->mode = src.mode;
  o->sampler = src.sampler;
  return makeHandle( o.release() );
}

int ncgb_set_mode( ncrystal_scatter_t sc, int mode )
{
  try {
    extract( sc.internal, "ncgb_set_mode" ).mode = checkMode( mode, "ncgb_set_mode" );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_get_mode( ncrystal_scatter_t sc )
{
  try {
    return extract( sc.internal, "ncgb_get_mode" ).mode;
  } NCGB_CATCH;
  return -1;
}

ncrystal_scatter_t ncrystal_clone_scatter( ncrystal_scatter_t sc )
{
  try {
    return cloneWithStream( sc, g_nextStream.fetch_add( 1 ), "ncrystal_clone_scatter" );
  } NCGB_CATCH;
  return ncrystal_scatter_t{ nullptr };
}

ncrystal_scatter_t ncrystal_clone_scatter_rngbyidx( ncrystal_scatter_t sc, unsigned long idx )
{
  try {
    // Stream 0 is the original handle's; clone index i uses stream i+1 of a
    // separate range so that it never coincides with automatic clones.
    return cloneWithStream( sc, 0x80000000u + static_cast<uint32_t>( idx & 0x7fffffffu ),
                            "ncrystal_clone_scatter_rngbyidx" );
  } NCGB_CATCH;
  return ncrystal_scatter_t{ nullptr };
}

ncrystal_scatter_t ncrystal_clone_scatter_rngforcurrentthread( ncrystal_scatter_t sc )
{
  try {
    static std::atomic<uint32_t> s_thread_stream{0x40000000u};
    thread_local uint32_t t_stream = s_thread_stream.fetch_add( 1 );
    return cloneWithStream( sc, t_stream, "ncrystal_clone_scatter_rngforcurrentthread" );
  } NCGB_CATCH;
  return ncrystal_scatter_t{ nullptr };
}

ncrystal_process_t ncrystal_cast_scat2proc( ncrystal_scatter_t s )
{
  try {
    extract( s.internal, "ncrystal_cast_scat2proc" );
    return ncrystal_process_t{ s.internal };
  } NCGB_CATCH;
  return ncrystal_process_t{ nullptr };
}

ncrystal_scatter_t ncrystal_cast_proc2scat( ncrystal_process_t p )
{
  try {
    // ncrystal.cc:420-429: null (no error) for a valid process of another type
    ScatterObj& o = extractProc( p.internal, "ncrystal_cast_proc2scat" );
    return ncrystal_scatter_t{ o.absorption ? nullptr : p.internal };
  } NCGB_CATCH;
  return ncrystal_scatter_t{ nullptr };
}

ncrystal_process_t ncrystal_cast_abs2proc( ncrystal_absorption_t a )
{
  try {
    extractAbs( a.internal, "ncrystal_cast_abs2proc" );
    return ncrystal_process_t{ a.internal };
  } NCGB_CATCH;
  return ncrystal_process_t{ nullptr };
}

ncrystal_absorption_t ncrystal_cast_proc2abs( ncrystal_process_t p )
{
  try {
    ScatterObj& o = extractProc( p.internal, "ncrystal_cast_proc2abs" );
    return ncrystal_absorption_t{ o.absorption ? p.internal : nullptr };
  } NCGB_CATCH;
  return ncrystal_absorption_t{ nullptr };
}

// ncrystal.cc:1565-1571 with the standard absorption factory's AbsOOV
// (NCStdAbsFact.cc:49-52), read from the material's bundle.
ncrystal_absorption_t ncrystal_create_absorption( const char* cfgstr )
{
  try {
    if ( !cfgstr )
      throw TypedError( "BadInput", "null cfg-string" );
    std::unique_ptr<ScatterObj> o( new ScatterObj );
    o->mat = getMaterial( cfgstr );
    if ( !( o->mat->view.abs_c >= 0.0 ) )
      throw TypedError( "BadInput", std::string( "the material bundle of \"" ) + cfgstr
                        + "\" carries no absorption data (export it again)" );
    o->cfg = cfgstr;
    o->absorption = true;
    o->fp.typeid_ = kAbsTypeID;
    return ncrystal_absorption_t{ &o.release()->fp };
  } NCGB_CATCH;
  return ncrystal_absorption_t{ nullptr };
}

ncrystal_absorption_t ncrystal_clone_absorption( ncrystal_absorption_t a )
{
  try {
    ScatterObj& src = extractAbs( a.internal, "ncrystal_clone_absorption" );
    std::unique_ptr<ScatterObj> o( new ScatterObj );
    o->mat = src.mat;
    o->cfg = src.cfg;
    o->absorption = true;
    o->fp.typeid_ = kAbsTypeID;
    return ncrystal_absorption_t{ &o.release()->fp };
  } NCGB_CATCH;
  return ncrystal_absorption_t{ nullptr };
}

const char* ncrystal_name( ncrystal_process_t p )
{
  try {
    ScatterObj& o = extractProc( p.internal, "ncrystal_name" );
    if ( o.absorption )
      return "AbsOOV";
    return o.mat->view.ncomp > 1 ? "ProcComposition"
      : ( o.mat->view.ncomp == 0 ? "NullProcess"
          : ( o.mat->view.comp[0].type == NCGB_COMP_BRAGG ? "PowderBragg"
              : o.mat->view.comp[0].type == NCGB_COMP_ELINC ? "ElIncScatter"
              : o.mat->view.comp[0].type == NCGB_COMP_SAB ? "SABScatter" : "FreeGas" ) );
  } NCGB_CATCH;
  return nullptr;
}

int ncrystal_isnonoriented( ncrystal_process_t p )
{
  try {
    extractProc( p.internal, "ncrystal_isnonoriented" );
    return 1;
  } NCGB_CATCH;
  return 0;
}

void ncrystal_domain( ncrystal_process_t p, double* elow, double* ehigh )
{
  try {
    ScatterObj& o = extractProc( p.internal, "ncrystal_domain" );
    if ( o.absorption ) {   // NCAbsOOV.cc:33-37
      *elow = 0.0;
      *ehigh = o.mat->view.abs_c > 0.0 ? std::numeric_limits<double>::infinity() : 0.0;
      return;
    }
    *elow = o.mat->view.dom_elow;
    *ehigh = o.mat->view.dom_ehigh;
    return;
  } NCGB_CATCH;
  *elow = *ehigh = -1.0;
}

// ---- batched evaluation ------------------------------------------------------------

void ncrystal_crosssection_nonoriented_many( ncrystal_process_t p, const double* ekin,
                                             unsigned long n_ekin, unsigned long repeat, double* results )
{
  try {
    ScatterObj& o = extractProc( p.internal, "ncrystal_crosssection_nonoriented_many" );
    checkSize( n_ekin, repeat );
    const uint64_t n_out = (uint64_t)n_ekin * repeat;
    if ( n_out == 0 )
      return;
    DeviceMaterial& dm = *o.mat;
    Scratch& s = scratchFor( dm );
    ensure( s.d_in, s.cap_in, n_ekin * sizeof(double) );
    ensure( s.d_a, s.cap_a, n_out * sizeof(double) );
    ncgb::Batch b = makeBatch( o, s, 0 );
    b.ekin = s.d_in;
    b.n_ekin = n_ekin;
    b.n_out = n_out;
    b.out_xs = s.d_a;
    checkCuda( cudaStreamWaitEvent( s.stream, s.done, 0 ), "cudaStreamWaitEvent" );
    checkCuda( cudaMemcpyAsync( s.d_in, ekin, n_ekin * sizeof(double), cudaMemcpyHostToDevice, s.stream ), "H2D" );
    if ( o.absorption )
      checkCuda( ncgb::launchAbsXS( dm.view.abs_c, b, repeat, s.stream ), "absorption xs kernel" );
    else
      checkCuda( ncgb::launchXS( dm.view, b, repeat, s.stream ), "xs kernel" );
    checkCuda( cudaMemcpyAsync( results, s.d_a, n_out * sizeof(double), cudaMemcpyDeviceToHost, s.stream ), "D2H" );
    checkCuda( cudaEventRecord( s.done, s.stream ), "cudaEventRecord" );
    checkCuda( cudaStreamSynchronize( s.stream ), "xs kernel" );
    return;
  } NCGB_CATCH;
  for ( unsigned long k = 0; k < n_ekin * repeat; ++k )
    results[k] = -1.0;
}

void ncrystal_samplescatterisotropic_many( ncrystal_scatter_t sc, const double* ekin,
                                           unsigned long n_ekin, unsigned long repeat,
                                           double* results_ekin, double* results_mu )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncrystal_samplescatterisotropic_many" );
    unsigned long nfail = runScatterMany( o, ekin, n_ekin, repeat, 0, results_ekin, results_mu, false );
    if ( nfail )
      throwSamplingFailure( nfail );
    return;
  } NCGB_CATCH;
  for ( unsigned long k = 0; k < n_ekin * repeat; ++k ) {
    results_ekin[k] = -1.0;
    results_mu[k] = -999.0;
  }
}

void ncrystal_genscatter_nonoriented_many( ncrystal_scatter_t sc, const double* ekin,
                                           unsigned long n_ekin, unsigned long repeat,
                                           double* results_angle, double* results_dekin )
{
  try {
    warnOnce( g_warn_genscatter_many, "The ncrystal_genscatter_nonoriented_many function is obsolete."
              " Please use the ncrystal_samplescatterisotropic_many function instead." );
    ScatterObj& o = extract( sc.internal, "ncrystal_genscatter_nonoriented_many" );
    unsigned long nfail = runScatterMany( o, ekin, n_ekin, repeat, 1, results_angle, results_dekin, true );
    if ( nfail )
      throwSamplingFailure( nfail );
    return;
  } NCGB_CATCH;
}

// ---- sampleScatter with directions (ncrystal.cc:1159-1174, :1248-1282) -------------------
namespace {
  // One energy and direction per input neutron (host arrays), n_ekin x repeat
  // outputs (index irepeat*n_ekin+i, like the _many calls).  Returns the
  // number of failed neutrons.
  unsigned long runScatterDir( ScatterObj& o, const double* ekin, const double* dir, unsigned long n_ekin,
                               unsigned long repeat, double* out_ekin, double* out_dir )
  {
    checkSize( n_ekin, repeat );
    const uint64_t n_out = (uint64_t)n_ekin * repeat;
    if ( n_out == 0 )
      return 0;
    DeviceMaterial& dm = *o.mat;
    Scratch& s = scratchFor( dm );
    // d_in: energies then incoming directions; d_a: E'; d_c: outgoing directions
    const std::size_t din = ( ( n_ekin * sizeof(double) + 255 ) & ~std::size_t(255) );
    ensure( s.d_in, s.cap_in, din + 3 * n_ekin * sizeof(double) );
    ensure( s.d_a, s.cap_a, n_out * sizeof(double) );
    ensure( s.d_c, s.cap_c, 3 * n_out * sizeof(double) );
    double* d_dir_in = reinterpret_cast<double*>( static_cast<char*>( s.d_in ) + din );
    ncgb::Batch b = makeBatch( o, s, nextCall( o ) );
    b.ekin = s.d_in;
    b.n_ekin = n_ekin;
    b.n_out = n_out;
    b.mode = 0;
    b.out_a = s.d_a;
    b.dir_in = d_dir_in;
    b.dir_out = static_cast<double*>( s.d_c );
    resetNFail( s, s.stream );
    checkCuda( cudaMemcpyAsync( s.d_in, ekin, n_ekin * sizeof(double), cudaMemcpyHostToDevice, s.stream ), "H2D" );
    checkCuda( cudaMemcpyAsync( d_dir_in, dir, 3 * n_ekin * sizeof(double), cudaMemcpyHostToDevice, s.stream ),
               "H2D" );
    runBatch( dm, s, b, s.stream );
    const unsigned long nfail = readNFail( s, s.stream );
    checkCuda( cudaMemcpy( out_ekin, s.d_a, n_out * sizeof(double), cudaMemcpyDeviceToHost ), "D2H" );
    checkCuda( cudaMemcpy( out_dir, s.d_c, 3 * n_out * sizeof(double), cudaMemcpyDeviceToHost ), "D2H" );
    return nfail;
  }
}

extern "C" {

void ncrystal_samplescatter( ncrystal_scatter_t sc, double ekin, const double (*direction)[3],
                             double* ekin_final, double (*direction_final)[3] )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncrystal_samplescatter" );
    double out[3];
    const unsigned long nfail = runScatterDir( o, &ekin, *direction, 1, 1, ekin_final, out );
    if ( nfail )
      throwSamplingFailure( nfail );
    (*direction_final)[0] = out[0];
    (*direction_final)[1] = out[1];
    (*direction_final)[2] = out[2];
    return;
  } NCGB_CATCH;
  *ekin_final = -1.0;
  (*direction_final)[0] = (*direction_final)[1] = (*direction_final)[2] = 0.0;
}

void ncrystal_samplescatter_many( ncrystal_scatter_t sc, double ekin, const double (*direction)[3],
                                  unsigned long repeat, double* results_ekin, double* results_dirx,
                                  double* results_diry, double* results_dirz )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncrystal_samplescatter_many" );
    std::vector<double> dirs( 3 * repeat );
    const unsigned long nfail = runScatterDir( o, &ekin, *direction, 1, repeat, results_ekin, dirs.data() );
    if ( nfail )
      throwSamplingFailure( nfail );
    for ( unsigned long k = 0; k < repeat; ++k ) {
      results_dirx[k] = dirs[3*k];
      results_diry[k] = dirs[3*k+1];
      results_dirz[k] = dirs[3*k+2];
    }
    return;
  } NCGB_CATCH;
  for ( unsigned long k = 0; k < repeat; ++k ) {
    results_ekin[k] = -1.0;
    results_dirx[k] = results_diry[k] = results_dirz[k] = 0.0;
  }
}

int ncgb_xs_abs_scatter_device( ncrystal_scatter_t sc, const double* d_ekin, unsigned long n, double* d_xs,
                                double* d_xs_abs, double* d_ekin_final, double* d_mu, int32_t* d_status,
                                void* stream )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncgb_xs_abs_scatter_device" );
    checkSize( n, 1 );
    if ( n == 0 )
      return 0;
    if ( d_xs_abs && !( o.mat->view.abs_c >= 0.0 ) )
      throw TypedError( "BadInput", "ncgb_xs_abs_scatter_device: the material bundle carries no absorption data" );
    DeviceMaterial& dm = *o.mat;
    Scratch& s = scratchFor( dm );
    ncgb::Batch b = makeBatch( o, s, nextCall( o ) );
    b.ekin = d_ekin;
    b.n_ekin = b.n_out = n;
    b.out_xs = d_xs;
    b.out_xs_abs = d_xs_abs;
    b.out_a = d_ekin_final;
    b.out_b = d_mu;
    b.status = d_status;
    runBatch( dm, s, b, static_cast<cudaStream_t>( stream ) );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_scatter_dir_device( ncrystal_scatter_t sc, const double* d_ekin, const double* d_dir, unsigned long n,
                             double* d_ekin_final, double* d_dir_final, int32_t* d_status, void* stream )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncgb_scatter_dir_device" );
    checkSize( n, 1 );
    if ( n == 0 )
      return 0;
    if ( !d_ekin || !d_dir || !d_dir_final )
      throw TypedError( "BadInput", "ncgb_scatter_dir_device: null array" );
    DeviceMaterial& dm = *o.mat;
    Scratch& s = scratchFor( dm );
    cudaStream_t st = static_cast<cudaStream_t>( stream );
    ncgb::Batch b = makeBatch( o, s, nextCall( o ) );
    b.ekin = d_ekin;
    b.n_ekin = b.n_out = n;
    b.out_a = d_ekin_final;
    b.status = d_status;
    b.dir_in = d_dir;
    b.dir_out = d_dir_final;
    runBatch( dm, s, b, st );
    return 0;
  } NCGB_CATCH;
  return 1;
}

}

// ---- scalar evaluation (a batch of one) -----------------------------------------------

void ncrystal_crosssection_nonoriented( ncrystal_process_t p, double ekin, double* result )
{
  ncrystal_crosssection_nonoriented_many( p, &ekin, 1, 1, result );
}

void ncrystal_samplescatterisotropic( ncrystal_scatter_t sc, double ekin, double* ef, double* mu )
{
  ncrystal_samplescatterisotropic_many( sc, &ekin, 1, 1, ef, mu );
}

void ncrystal_genscatter_nonoriented( ncrystal_scatter_t sc, double ekin, double* angle, double* dekin )
{
  *angle = -999.0;
  *dekin = -999.0;
  try {
    warnOnce( g_warn_genscatter, "The ncrystal_genscatter_nonoriented function is obsolete. Please use"
              " the ncrystal_samplescatterisotropic function instead." );
    ScatterObj& o = extract( sc.internal, "ncrystal_genscatter_nonoriented" );
    unsigned long nfail = runScatterMany( o, &ekin, 1, 1, 1, angle, dekin, true );
    if ( nfail )
      throwSamplingFailure( nfail );
  } NCGB_CATCH;
}

// ---- additions ----------------------------------------------------------------------

static int scatterDevice( ncrystal_scatter_t sc, const void* d_ekin, unsigned long n, void* d_xs, void* d_ef,
                          void* d_mu, int32_t* d_status, void* stream, bool f32, const char* fct )
{
  try {
    ScatterObj& o = extract( sc.internal, fct );
    checkSize( n, 1 );
    if ( n == 0 )
      return 0;
    DeviceMaterial& dm = *o.mat;
    Scratch& s = scratchFor( dm );
    ncgb::Batch b = makeBatch( o, s, nextCall( o ) );
    b.ekin = d_ekin;
    b.in_f32 = b.out_f32 = f32 ? 1 : 0;
    b.n_ekin = b.n_out = n;
    b.out_xs = d_xs;
    b.out_a = d_ef;
    b.out_b = d_mu;
    b.status = d_status;
    runBatch( dm, s, b, static_cast<cudaStream_t>( stream ) );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_scatter_device( ncrystal_scatter_t sc, const double* d_ekin, unsigned long n,
                         double* d_xs, double* d_ef, double* d_mu, int32_t* d_status, void* stream )
{
  return scatterDevice( sc, d_ekin, n, d_xs, d_ef, d_mu, d_status, stream, false, "ncgb_scatter_device" );
}

int ncgb_scatter_device_f32( ncrystal_scatter_t sc, const float* d_ekin, unsigned long n,
                             float* d_xs, float* d_ef, float* d_mu, int32_t* d_status, void* stream )
{
  return scatterDevice( sc, d_ekin, n, d_xs, d_ef, d_mu, d_status, stream, true, "ncgb_scatter_device_f32" );
}

void ncgb_crosssection_nonoriented_many_f32( ncrystal_process_t p, const float* ekin,
                                             unsigned long n, float* results )
{
  try {
    ScatterObj& o = extract( p.internal, "ncgb_crosssection_nonoriented_many_f32" );
    checkSize( n, 1 );
    if ( n == 0 )
      return;
    DeviceMaterial& dm = *o.mat;
    Scratch& s = scratchFor( dm );
    ensure( s.d_in, s.cap_in, n * sizeof(float) );
    ensure( s.d_a, s.cap_a, n * sizeof(float) );
    ncgb::Batch b = makeBatch( o, s, 0 );
    b.ekin = s.d_in;
    b.in_f32 = b.out_f32 = 1;
    b.n_ekin = b.n_out = n;
    b.out_xs = s.d_a;
    checkCuda( cudaStreamWaitEvent( s.stream, s.done, 0 ), "cudaStreamWaitEvent" );
    checkCuda( cudaMemcpyAsync( s.d_in, ekin, n * sizeof(float), cudaMemcpyHostToDevice, s.stream ), "H2D" );
    checkCuda( ncgb::launchXS( dm.view, b, 1, s.stream ), "xs kernel" );
    checkCuda( cudaMemcpyAsync( results, s.d_a, n * sizeof(float), cudaMemcpyDeviceToHost, s.stream ), "D2H" );
    checkCuda( cudaEventRecord( s.done, s.stream ), "cudaEventRecord" );
    checkCuda( cudaStreamSynchronize( s.stream ), "xs kernel" );
    return;
  } NCGB_CATCH;
  for ( unsigned long k = 0; k < n; ++k )
    results[k] = -1.0f;
}

void ncgb_samplescatterisotropic_many_f32( ncrystal_scatter_t sc, const float* ekin, unsigned long n,
                                           float* results_ekin, float* results_mu )
{
  try {
    xsScatterHost<float>( extract( sc.internal, "ncgb_samplescatterisotropic_many_f32" ), ekin, n,
                          nullptr, results_ekin, results_mu );
    return;
  } NCGB_CATCH;
  fillSentinels<float>( n, nullptr, results_ekin, results_mu );
}

void ncgb_xs_scatter_many( ncrystal_scatter_t sc, const double* ekin, unsigned long n,
                           double* xs, double* ef, double* mu )
{
  try {
    xsScatterHost<double>( extract( sc.internal, "ncgb_xs_scatter_many" ), ekin, n, xs, ef, mu );
    return;
  } NCGB_CATCH;
  fillSentinels<double>( n, xs, ef, mu );
}

void ncgb_xs_scatter_many_f32( ncrystal_scatter_t sc, const float* ekin, unsigned long n,
                               float* xs, float* ef, float* mu )
{
  try {
    xsScatterHost<float>( extract( sc.internal, "ncgb_xs_scatter_many_f32" ), ekin, n, xs, ef, mu );
    return;
  } NCGB_CATCH;
  fillSentinels<float>( n, xs, ef, mu );
}

unsigned long ncgb_last_nfailed( void ) { return t_scratch.last_nfailed; }

void ncgb_phase_timing( int enable ) { ncgb::setPhaseTiming( enable != 0 ); }

int ncgb_phase_times( double* ms_pick, double* ms_sab, unsigned long* nbatches, unsigned long* last_nsab )
{
  try {
    if ( ncgb::takePhaseTimes( ms_pick, ms_sab, nbatches ) )
      throw TypedError( "CalcError", "could not read the phase timing events" );
    *last_nsab = 0;
    Scratch& s = t_scratch;
    if ( s.d_work ) {
      ncgb::Work w;
      checkCuda( cudaMemcpy( &w, s.d_work, sizeof(w), cudaMemcpyDeviceToHost ), "D2H" );
      *last_nsab = (unsigned long)w.qcount + w.rcount;   // both lists of the S(alpha,beta) queue
    }
    return 0;
  } NCGB_CATCH;
  return 1;
}

unsigned long ncgb_device_bytes( ncrystal_scatter_t sc )
{
  try {
    return extract( sc.internal, "ncgb_device_bytes" ).mat->tables->arenaBytes();
  } NCGB_CATCH;
  return 0;
}

}

int ncgb_sab_phase_profile( ncrystal_scatter_t sc, const double* d_ekin, unsigned long n, double* d_xs,
                            double* d_ef, double* d_mu, unsigned long long* cycles )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncgb_sab_phase_profile" );
    checkSize( n, 1 );
    const std::size_t nc = NCGB_SAB_NPHASES + 1;
    for ( std::size_t k = 0; k < nc; ++k )
      cycles[k] = 0;
    if ( n == 0 )
      return 0;
    DeviceMaterial& dm = *o.mat;
    Scratch& s = scratchFor( dm );
    ensure( s.d_phase, s.cap_phase, nc * sizeof(unsigned long long) );
    checkCuda( cudaMemsetAsync( s.d_phase, 0, nc * sizeof(unsigned long long), s.stream ), "cudaMemsetAsync" );
    ncgb::Batch b = makeBatch( o, s, nextCall( o ) );
    b.ekin = d_ekin;
    b.n_ekin = b.n_out = n;
    b.out_xs = d_xs;
    b.out_a = d_ef;
    b.out_b = d_mu;
    b.untimed = 1;
    b.phase_cycles = static_cast<unsigned long long*>( s.d_phase );
    runBatch( dm, s, b, s.stream );
    checkCuda( cudaMemcpyAsync( cycles, s.d_phase, nc * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                s.stream ), "D2H" );
    checkCuda( cudaStreamSynchronize( s.stream ), "phase-profiled scatter" );
    return 0;
  } NCGB_CATCH;
  return 1;
}

// ---- internal hooks for ncgb_noalloc.cu (C++ linkage) ---------------------------------
namespace ncgb {

  // Validates a handle and returns what a batch launch needs: the material,
  // its device, the random-stream key and the arithmetic mode and sampler.
  // Consumes no call sequence number (handleNextCall does, just before a
  // launch).  Throws on a bad handle.
  void handleBatchInfo( ncrystal_scatter_t sc, const char* fct, ncgb_material_view* view, int* device,
                        uint64_t* seed, uint32_t* streamidx, int* fast, int* learned )
  {
    ScatterObj& o = extract( sc.internal, fct );
    *view = o.mat->view;
    *device = o.mat->device;
    *seed = o.seed;
    *streamidx = o.streamidx;
    *fast = ( o.mode == NCGB_MODE_MIXED );
    *learned = ( o.sampler == NCGB_SAMPLER_LEARNED );
  }

  // The handle's next call sequence number, as every scatter call takes one.
  uint32_t handleNextCall( ncrystal_scatter_t sc, const char* fct )
  {
    return nextCall( extract( sc.internal, fct ) );
  }

  // What the MiniMC engine needs of a scatter handle.
  void handleInfo( ncrystal_scatter_t sc, const char* fct, mmc::HandleInfo* out )
  {
    ScatterObj& o = extract( sc.internal, fct );
    out->view = o.mat->view;
    out->device = o.mat->device;
    out->mode = o.mode;
    out->sampler = o.sampler;
    out->seed = o.seed;
    out->streamidx = o.streamidx;
    out->numdens = o.mat->tables->m_numdens;
    out->temperature = o.mat->tables->m_info_temperature;
    out->bragg_threshold = o.mat->tables->m_bragg_threshold;
    out->abs_c = o.mat->view.abs_c;
    out->cfg = o.cfg;
  }

  // Routes an exception into the C interface's error state.
  void reportError( const std::exception& e ) { handleError( e ); }

  // Raises a typed error through the C interface's error state.
  void reportError( const char* type, const std::string& msg ) { handleError( TypedError( type, msg ) ); }
}

// ---- ragged multi-material batches ---------------------------------------------------
namespace {

  constexpr uint32_t kBatchTypeID = 0x6e636262; // "ncbb"

  struct BatchObj {
    uint32_t typeid_ = kBatchTypeID;
    int device = -1;
    std::vector<std::shared_ptr<DeviceMaterial>> mats;   // keeps the tables alive
    ncgb::MatSlot* d_slots = nullptr;
    int nmat = 0;
    bool anyBragg = false;   // some material has a PowderBragg component
    ncgb::LaunchCfg cfg;
    bool tuned = false;
    int mode = defaultMode();
    int sampler = NCGB_SAMPLER_PLAIN;
    std::atomic<uint32_t> callseq{0};
    // CUDA graph of (counter reset, k_pick, k_sab) for one set of arrays
    cudaGraphExec_t exec = nullptr;
    const void* g_key[6] = {};
    unsigned long g_n = 0;
    ~BatchObj()
    {
      if ( exec ) cudaGraphExecDestroy( exec );
      if ( d_slots ) cudaFree( d_slots );
    }
  };

  BatchObj& extractBatch( void* internal, const char* fct )
  {
    auto b = static_cast<BatchObj*>( internal );
    if ( !b || b->typeid_ != kBatchTypeID )
      throw TypedError( "LogicError", std::string("Invalid batch handle passed to ") + fct );
    return *b;
  }

  ncgb::Batch multiBatch( BatchObj& bo, Scratch& s, const double* d_ekin, unsigned long n,
                          double* d_xs, double* d_ef, double* d_mu, int32_t* d_status )
  {
    ncgb::Batch b;
    std::memset( &b, 0, sizeof(b) );
    b.ekin = d_ekin;
    b.n_ekin = b.n_out = n;
    b.callseq = bo.callseq.fetch_add( 1, std::memory_order_relaxed );
    b.out_xs = d_xs;
    b.out_a = d_ef;
    b.out_b = d_mu;
    b.status = d_status;
    b.fast = ( bo.mode == NCGB_MODE_MIXED );
    b.learned = ( bo.sampler == NCGB_SAMPLER_LEARNED );
    b.reorder = bo.anyBragg ? 1 : 0;
    b.work = s.d_work;
    ensure( s.d_queue, s.cap_queue, n * sizeof(ncgb::QEntry) );
    b.queue = static_cast<ncgb::QEntry*>( s.d_queue );
    return b;
  }
}

extern "C" {

ncgb_batch_t ncgb_batch_create( const ncrystal_scatter_t* scatters, unsigned long nmat )
{
  try {
    if ( !scatters || nmat == 0 || nmat > 65535 )
      throw TypedError( "BadInput", "ncgb_batch_create: need between 1 and 65535 materials" );
    std::unique_ptr<BatchObj> bo( new BatchObj );
    std::vector<ncgb::MatSlot> slots( nmat );
    for ( unsigned long k = 0; k < nmat; ++k ) {
      ScatterObj& o = extract( scatters[k].internal, "ncgb_batch_create" );
      if ( k == 0 )
        bo->device = o.mat->device;
      else if ( o.mat->device != bo->device )
        throw TypedError( "BadInput", "ncgb_batch_create: materials live on different devices" );
      bo->mats.push_back( o.mat );
      std::memset( &slots[k], 0, sizeof(ncgb::MatSlot) );
      slots[k].view = o.mat->view;
      if ( hasBragg( o.mat->view ) )
        bo->anyBragg = true;
      slots[k].seed = o.seed;
      slots[k].stream = o.streamidx;
    }
    Scratch& s = scratchFor( *bo->mats.front() );
    (void)s;
    void* p = nullptr;
    checkCuda( cudaMalloc( &p, nmat * sizeof(ncgb::MatSlot) ), "cudaMalloc (batch materials)" );
    bo->d_slots = static_cast<ncgb::MatSlot*>( p );
    checkCuda( cudaMemcpy( p, slots.data(), nmat * sizeof(ncgb::MatSlot), cudaMemcpyHostToDevice ),
               "cudaMemcpy (batch materials)" );
    bo->nmat = static_cast<int>( nmat );
    return ncgb_batch_t{ bo.release() };
  } NCGB_CATCH;
  return ncgb_batch_t{ nullptr };
}

void ncgb_batch_destroy( ncgb_batch_t* b )
{
  try {
    if ( !b || !b->internal )
      return;
    BatchObj& bo = extractBatch( b->internal, "ncgb_batch_destroy" );
    cudaDeviceSynchronize();
    delete &bo;
    b->internal = nullptr;
  } NCGB_CATCH;
}

int ncgb_batch_scatter_device( ncgb_batch_t bt, const double* d_ekin, const int64_t* d_offsets,
                               unsigned long n, double* d_xs, double* d_ef, double* d_mu,
                               int32_t* d_status, void* stream )
{
  try {
    BatchObj& bo = extractBatch( bt.internal, "ncgb_batch_scatter_device" );
    checkSize( n, 1 );
    if ( n == 0 )
      return 0;
    Scratch& s = scratchFor( *bo.mats.front() );
    cudaStream_t st = static_cast<cudaStream_t>( stream );
    ncgb::Batch b = multiBatch( bo, s, d_ekin, n, d_xs, d_ef, d_mu, d_status );
    checkCuda( cudaStreamWaitEvent( st, s.done, 0 ), "cudaStreamWaitEvent" );
    checkCuda( ncgb::launchScatterMulti( bo.d_slots, d_offsets, bo.nmat, b, bo.cfg, st ), "batch kernels" );
    checkCuda( cudaEventRecord( s.done, st ), "cudaEventRecord" );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_batch_autotune( ncgb_batch_t bt, const double* d_ekin, const int64_t* d_offsets, unsigned long n,
                         double* d_xs, double* d_ef, double* d_mu, void* stream )
{
  try {
    BatchObj& bo = extractBatch( bt.internal, "ncgb_batch_autotune" );
    checkSize( n, 1 );
    if ( n == 0 )
      return 0;
    Scratch& s = scratchFor( *bo.mats.front() );
    cudaStream_t st = static_cast<cudaStream_t>( stream );
    checkCuda( cudaStreamWaitEvent( st, s.done, 0 ), "cudaStreamWaitEvent" );
    const int maxb = ncgb::maxSabBlocksPerSM();
    std::vector<ncgb::LaunchCfg> cands;
    for ( int pb : { 128, 256, 512 } )
      for ( int sb : { maxb, std::max( 1, maxb / 2 ) } )
        for ( int sl : { 0, 1 } ) {
          ncgb::LaunchCfg c;
          c.pick_block = pb;
          c.sab_blocks_per_sm = sb;
          c.split_lists = sl;
          cands.push_back( c );
        }
    cudaEvent_t e0, e1;
    checkCuda( cudaEventCreate( &e0 ), "event" );
    checkCuda( cudaEventCreate( &e1 ), "event" );
    float best = -1.f;
    ncgb::LaunchCfg bestc;
    for ( auto& c : cands ) {
      // one warm-up run, then the fastest of three timed runs (a single
      // timing let run-to-run noise choose the slower pick block size)
      float cbest = -1.f;
      for ( int rep = 0; rep < 4; ++rep ) {
        ncgb::Batch b = multiBatch( bo, s, d_ekin, n, d_xs, d_ef, d_mu, nullptr );
        checkCuda( cudaEventRecord( e0, st ), "event" );
        checkCuda( ncgb::launchScatterMulti( bo.d_slots, d_offsets, bo.nmat, b, c, st ), "batch kernels" );
        checkCuda( cudaEventRecord( e1, st ), "event" );
        checkCuda( cudaEventSynchronize( e1 ), "autotune" );
        float ms = 0.f;
        cudaEventElapsedTime( &ms, e0, e1 );
        if ( rep > 0 && ( cbest < 0.f || ms < cbest ) )
          cbest = ms;
      }
      if ( best < 0.f || cbest < best ) { best = cbest; bestc = c; }
    }
    cudaEventDestroy( e0 );
    cudaEventDestroy( e1 );
    checkCuda( cudaEventRecord( s.done, st ), "cudaEventRecord" );
    bo.cfg = bestc;
    bo.tuned = true;
    if ( bo.exec ) { cudaGraphExecDestroy( bo.exec ); bo.exec = nullptr; }
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_batch_set_mode( ncgb_batch_t bt, int mode )
{
  try {
    BatchObj& bo = extractBatch( bt.internal, "ncgb_batch_set_mode" );
    bo.mode = checkMode( mode, "ncgb_batch_set_mode" );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_batch_set_sampler( ncgb_batch_t bt, int sampler )
{
  try {
    BatchObj& bo = extractBatch( bt.internal, "ncgb_batch_set_sampler" );
    if ( sampler != NCGB_SAMPLER_PLAIN && sampler != NCGB_SAMPLER_LEARNED )
      throw TypedError( "BadInput", "ncgb_batch_set_sampler: unknown sampler" );
    bo.sampler = sampler;
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_batch_config( ncgb_batch_t bt, int* pick_block, int* sab_blocks_per_sm )
{
  try {
    BatchObj& bo = extractBatch( bt.internal, "ncgb_batch_config" );
    *pick_block = bo.cfg.pick_block;
    *sab_blocks_per_sm = bo.cfg.sab_blocks_per_sm > 0 ? bo.cfg.sab_blocks_per_sm : ncgb::maxSabBlocksPerSM();
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_batch_set_split_lists( ncgb_batch_t bt, int split_lists )
{
  try {
    BatchObj& bo = extractBatch( bt.internal, "ncgb_batch_set_split_lists" );
    if ( split_lists != 0 && split_lists != 1 )
      throw TypedError( "BadInput", "ncgb_batch_set_split_lists: 0 or 1" );
    if ( bo.cfg.split_lists != split_lists && bo.exec ) {
      cudaGraphExecDestroy( bo.exec );   // the captured launch names the other pass
      bo.exec = nullptr;
    }
    bo.cfg.split_lists = split_lists;
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_batch_split_lists( ncgb_batch_t bt, int* split_lists )
{
  try {
    BatchObj& bo = extractBatch( bt.internal, "ncgb_batch_split_lists" );
    *split_lists = bo.cfg.split_lists;
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_batch_graph_launch( ncgb_batch_t bt, const double* d_ekin, const int64_t* d_offsets, unsigned long n,
                             double* d_xs, double* d_ef, double* d_mu, int32_t* d_status, void* stream )
{
  try {
    BatchObj& bo = extractBatch( bt.internal, "ncgb_batch_graph_launch" );
    checkSize( n, 1 );
    if ( n == 0 )
      return 0;
    Scratch& s = scratchFor( *bo.mats.front() );
    cudaStream_t st = static_cast<cudaStream_t>( stream );
    // Capture this launch's nodes on a private stream; instantiate once, and
    // update the instantiated graph in place on later calls (the call
    // sequence number, a kernel parameter, changes every call).
    ncgb::Batch b = multiBatch( bo, s, d_ekin, n, d_xs, d_ef, d_mu, d_status );
    static thread_local cudaStream_t cap = nullptr;
    if ( !cap )
      checkCuda( cudaStreamCreateWithFlags( &cap, cudaStreamNonBlocking ), "cudaStreamCreate" );
    cudaGraph_t g = nullptr;
    checkCuda( cudaStreamBeginCapture( cap, cudaStreamCaptureModeThreadLocal ), "cudaStreamBeginCapture" );
    cudaError_t le = ncgb::launchScatterMulti( bo.d_slots, d_offsets, bo.nmat, b, bo.cfg, cap );
    cudaError_t ce = cudaStreamEndCapture( cap, &g );
    checkCuda( le, "batch kernels (capture)" );
    checkCuda( ce, "cudaStreamEndCapture" );
    bool fresh = true;
    if ( bo.exec ) {
      cudaGraphExecUpdateResultInfo info;
      if ( cudaGraphExecUpdate( bo.exec, g, &info ) == cudaSuccess )
        fresh = false;
      else {
        cudaGetLastError();
        cudaGraphExecDestroy( bo.exec );
        bo.exec = nullptr;
      }
    }
    if ( fresh )
      checkCuda( cudaGraphInstantiate( &bo.exec, g, 0 ), "cudaGraphInstantiate" );
    cudaGraphDestroy( g );
    checkCuda( cudaStreamWaitEvent( st, s.done, 0 ), "cudaStreamWaitEvent" );
    checkCuda( cudaGraphLaunch( bo.exec, st ), "cudaGraphLaunch" );
    checkCuda( cudaEventRecord( s.done, st ), "cudaEventRecord" );
    return 0;
  } NCGB_CATCH;
  return 1;
}

void ncgb_batch_xs_scatter_many( ncgb_batch_t bt, const double* ekin, const int64_t* offsets, unsigned long n,
                                 double* xs, double* ef, double* mu )
{
  try {
    BatchObj& bo = extractBatch( bt.internal, "ncgb_batch_xs_scatter_many" );
    checkSize( n, 1 );
    if ( n == 0 )
      return;
    // Chunked H2D / kernels / D2H (chunkPipeline), as xsScatterHost: chunk k
    // is a launch over neutrons [off, off+m) of the whole batch (the kernels
    // locate materials and random streams from the global index off + o); one
    // call sequence number for the whole call.
    Scratch& s = scratchFor( *bo.mats.front() );
    const std::size_t offbytes = ( bo.nmat + 1 ) * sizeof(int64_t);
    std::vector<void*> mp;
    if ( zeroCopyFor( false ) && allMapped( { ekin, xs, ef, mu }, mp ) ) {
      // zero-copy: one batch straight over the caller's pinned arrays
      ensure( s.d_in, s.cap_in, offbytes + 256 );
      ensure( s.d_queue, s.cap_queue, n * sizeof(ncgb::QEntry) );
      int64_t* d_off = static_cast<int64_t*>( s.d_in );
      const uint32_t call = bo.callseq.fetch_add( 1, std::memory_order_relaxed );
      resetNFail( s, s.stream );
      checkCuda( cudaMemcpyAsync( d_off, offsets, offbytes, cudaMemcpyHostToDevice, s.stream ), "H2D" );
      ncgb::Batch b = multiBatch( bo, s, static_cast<const double*>( mp[0] ), n, static_cast<double*>( mp[1] ),
                                  static_cast<double*>( mp[2] ), static_cast<double*>( mp[3] ), nullptr );
      b.callseq = call;
      b.index_offset = 0;
      b.reorder = 0;
      checkCuda( cudaStreamWaitEvent( s.stream, s.done, 0 ), "cudaStreamWaitEvent" );
      checkCuda( ncgb::launchScatterMulti( bo.d_slots, d_off, bo.nmat, b, bo.cfg, s.stream ), "batch kernels" );
      checkCuda( cudaEventRecord( s.done, s.stream ), "cudaEventRecord" );
      const unsigned long bad = readNFail( s, s.stream );
      if ( bad )
        throwSamplingFailure( bad );
      return;
    }
    const uint64_t chunk = std::min<uint64_t>( n, copyChunk() );
    ensure( s.d_in, s.cap_in, 2 * chunk * sizeof(double) + offbytes + 256 );
    ensure( s.d_a, s.cap_a, 2 * chunk * sizeof(double) );
    ensure( s.d_b, s.cap_b, 2 * chunk * sizeof(double) );
    ensure( s.d_c, s.cap_c, 2 * chunk * sizeof(double) );
    ensure( s.d_queue, s.cap_queue, chunk * sizeof(ncgb::QEntry) );
    int64_t* d_off = reinterpret_cast<int64_t*>( static_cast<char*>( s.d_in ) + 2 * chunk * sizeof(double) );
    const uint32_t call = bo.callseq.fetch_add( 1, std::memory_order_relaxed );
    resetNFail( s, s.stream );
    checkCuda( cudaMemcpyAsync( d_off, offsets, offbytes, cudaMemcpyHostToDevice, s.stream ), "H2D" );
    checkCuda( cudaEventRecord( s.done, s.stream ), "cudaEventRecord" );
    auto slot = [&]( void* base, int h ) { return static_cast<double*>( base ) + h * chunk; };
    chunkPipeline(
      s, n, chunk,
      [&]( uint64_t off, uint64_t m, int h, cudaStream_t cs ) {
        checkCuda( cudaMemcpyAsync( slot( s.d_in, h ), ekin + off, m * sizeof(double), cudaMemcpyHostToDevice, cs ),
                   "H2D" );
      },
      [&]( uint64_t off, uint64_t m, int h, cudaStream_t cs ) {
        ncgb::Batch b = multiBatch( bo, s, slot( s.d_in, h ), m, xs ? slot( s.d_a, h ) : nullptr,
                                    ef ? slot( s.d_b, h ) : nullptr, mu ? slot( s.d_c, h ) : nullptr, nullptr );
        b.callseq = call;
        b.index_offset = static_cast<uint32_t>( off );
        checkCuda( cudaStreamWaitEvent( cs, s.done, 0 ), "cudaStreamWaitEvent" );
        checkCuda( ncgb::launchScatterMulti( bo.d_slots, d_off, bo.nmat, b, bo.cfg, cs, s.ev_pick[h] ),
                   "batch kernels" );
        checkCuda( cudaEventRecord( s.done, cs ), "cudaEventRecord" );
      },
      [&]( uint64_t off, uint64_t m, int h, cudaStream_t cs ) {
        if ( xs ) checkCuda( cudaMemcpyAsync( xs + off, slot( s.d_a, h ), m * sizeof(double), cudaMemcpyDeviceToHost, cs ), "D2H" );
      },
      [&]( uint64_t off, uint64_t m, int h, cudaStream_t cs ) {
        if ( ef ) checkCuda( cudaMemcpyAsync( ef + off, slot( s.d_b, h ), m * sizeof(double), cudaMemcpyDeviceToHost, cs ), "D2H" );
        if ( mu ) checkCuda( cudaMemcpyAsync( mu + off, slot( s.d_c, h ), m * sizeof(double), cudaMemcpyDeviceToHost, cs ), "D2H" );
      } );
    const unsigned long bad = readNFail( s, s.stream );
    if ( bad )
      throwSamplingFailure( bad );
    return;
  } NCGB_CATCH;
  fillSentinels<double>( n, xs, ef, mu );
}

}

// ---- learned beta proposal (no reference counterpart) ------------------------------
namespace {

  const ncgb_comp_view& sabComp( ScatterObj& o, int comp, const char* fct )
  {
    if ( comp < 0 || comp >= o.mat->view.ncomp )
      throw TypedError( "BadInput", std::string( fct ) + ": component index out of range" );
    const ncgb_comp_view& c = o.mat->view.comp[comp];
    if ( c.type != NCGB_COMP_SAB )
      throw TypedError( "BadInput", std::string( fct ) + ": component is not an S(alpha,beta) component" );
    return c;
  }

  ncgb_sab_view hostSab( ScatterObj& o, int comp )
  {
    const ncgb_material_view hv = o.mat->tables->relocate( o.mat->tables->arena().data() );
    return hv.comp[comp].sab;
  }

  // Builds the proposal tables from knots[ne*62] on the host, uploads them and
  // points the material's view at them.
  double attachKnots( ScatterObj& o, int comp, const float* knots, const unsigned char* allowed, double min_accept )
  {
    const ncgb_sab_view hs = hostSab( o, comp );
    ncgb::Proposal P = ncgb::buildProposal( hs, knots, NCGB_LP_NKNOTS, allowed, min_accept );
    DeviceMaterial& dm = *o.mat;
    checkCuda( cudaSetDevice( dm.device ), "cudaSetDevice" );
    const std::size_t hb = ( P.hdr.size() * sizeof(ncgb_lp_hdr) + 255 ) & ~std::size_t(255);
    const std::size_t sb = ( P.slot.size() * sizeof(ncgb_lp_slot) + 255 ) & ~std::size_t(255);
    const std::size_t cb = ( P.cell.size() * sizeof(ncgb_lp_cell) + 255 ) & ~std::size_t(255);
    const std::size_t gb = P.seg.size() * sizeof(ncgb_lp_seg);
    void* d = nullptr;
    checkCuda( cudaMalloc( &d, hb + sb + cb + gb ), "cudaMalloc (proposal tables)" );
    char* dc = static_cast<char*>( d );
    checkCuda( cudaMemcpy( dc, P.hdr.data(), P.hdr.size() * sizeof(ncgb_lp_hdr), cudaMemcpyHostToDevice ), "H2D" );
    checkCuda( cudaMemcpy( dc + hb, P.slot.data(), P.slot.size() * sizeof(ncgb_lp_slot), cudaMemcpyHostToDevice ),
               "H2D" );
    checkCuda( cudaMemcpy( dc + hb + sb, P.cell.data(), P.cell.size() * sizeof(ncgb_lp_cell),
                           cudaMemcpyHostToDevice ), "H2D" );
    checkCuda( cudaMemcpy( dc + hb + sb + cb, P.seg.data(), gb, cudaMemcpyHostToDevice ), "H2D" );
    checkCuda( cudaDeviceSynchronize(), "proposal upload" );
    if ( dm.d_lp[comp] )
      cudaFree( dm.d_lp[comp] );
    dm.d_lp[comp] = d;
    dm.h_lp[comp] = P.hdr;
    dm.view.comp[comp].sab.lp_hdr = reinterpret_cast<const ncgb_lp_hdr*>( dc );
    dm.view.comp[comp].sab.lp_slot = reinterpret_cast<const ncgb_lp_slot*>( dc + hb );
    dm.view.comp[comp].sab.lp_cell = reinterpret_cast<const ncgb_lp_cell*>( dc + hb + sb );
    dm.view.comp[comp].sab.lp_seg = reinterpret_cast<const ncgb_lp_seg*>( dc + hb + sb + cb );
    double sum = 0.0;
    int n = 0;
    for ( auto& h : P.hdr )
      if ( h.enabled ) { sum += h.accept; ++n; }
    return n ? sum / n : 0.0;
  }

  constexpr uint32_t kMlpTypeID = 0x6e636d6c; // "ncml"
  struct MlpObj {
    uint32_t typeid_ = kMlpTypeID;
    ncgb_mlp::Net* net = nullptr;
    ~MlpObj() { ncgb_mlp::destroy( net ); }
  };

  MlpObj& extractMlp( void* internal, const char* fct )
  {
    auto m = static_cast<MlpObj*>( internal );
    if ( !m || m->typeid_ != kMlpTypeID )
      throw TypedError( "LogicError", std::string( "Invalid network handle passed to " ) + fct );
    return *m;
  }
}

extern "C" {

int ncgb_set_sampler( ncrystal_scatter_t sc, int sampler )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncgb_set_sampler" );
    if ( sampler != NCGB_SAMPLER_PLAIN && sampler != NCGB_SAMPLER_LEARNED )
      throw TypedError( "BadInput", "ncgb_set_sampler: unknown sampler" );
    o.sampler = sampler;
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_get_sampler( ncrystal_scatter_t sc )
{
  try {
    return extract( sc.internal, "ncgb_get_sampler" ).sampler;
  } NCGB_CATCH;
  return -1;
}

int ncgb_component_info( ncrystal_scatter_t sc, int comp, int* type, double* scale, unsigned long* ne )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncgb_component_info" );
    const ncgb_material_view& v = o.mat->view;
    if ( comp < 0 || comp >= v.ncomp )
      throw TypedError( "BadInput", "ncgb_component_info: component index out of range" );
    if ( type ) *type = v.comp[comp].type;
    if ( scale ) *scale = v.comp[comp].scale;
    if ( ne ) *ne = v.comp[comp].type == NCGB_COMP_SAB ? (unsigned long)v.comp[comp].sab.ne : 0ul;
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_material_info( ncrystal_scatter_t sc, int* ncomp, double* temperature )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncgb_material_info" );
    if ( ncomp ) *ncomp = o.mat->view.ncomp;
    if ( temperature ) *temperature = o.mat->tables->temperature();
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_sab_egrid( ncrystal_scatter_t sc, int comp, double* egrid_out )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncgb_sab_egrid" );
    sabComp( o, comp, "ncgb_sab_egrid" );
    const ncgb_sab_view hs = hostSab( o, comp );
    std::memcpy( egrid_out, hs.egrid, hs.ne * sizeof(double) );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_sab_sample_device( ncrystal_scatter_t sc, int comp, const double* d_ekin, unsigned long n,
                            double* d_alpha, double* d_beta, int32_t* d_status, void* stream )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncgb_sab_sample_device" );
    sabComp( o, comp, "ncgb_sab_sample_device" );
    checkSize( n, 1 );
    if ( !d_ekin || !d_alpha || !d_beta )
      throw TypedError( "BadInput", "ncgb_sab_sample_device: null array" );
    Scratch& s = scratchFor( *o.mat );
    cudaStream_t st = static_cast<cudaStream_t>( stream );
    ncgb::Batch b = makeBatch( o, s, nextCall( o ) );
    b.ekin = d_ekin;
    b.n_ekin = b.n_out = n;
    b.out_a = d_alpha;
    b.out_b = d_beta;
    b.status = d_status;
    checkCuda( cudaStreamWaitEvent( st, s.done, 0 ), "cudaStreamWaitEvent" );
    checkCuda( ncgb::launchSabAB( o.mat->view, comp, b, st ), "S(alpha,beta) sampling kernel" );
    checkCuda( cudaEventRecord( s.done, st ), "cudaEventRecord" );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_attach_proposal_knots( ncrystal_scatter_t sc, int comp, const float* knots, double min_accept,
                                double* mean_accept )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncgb_attach_proposal_knots" );
    sabComp( o, comp, "ncgb_attach_proposal_knots" );
    if ( !knots )
      throw TypedError( "BadInput", "ncgb_attach_proposal_knots: null knots" );
    const double a = attachKnots( o, comp, knots, nullptr, min_accept );
    if ( mean_accept ) *mean_accept = a;
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_attach_proposal( ncrystal_scatter_t sc, int comp, ncgb_mlp_t net, double min_accept, double* mean_accept )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncgb_attach_proposal" );
    MlpObj& m = extractMlp( net.internal, "ncgb_attach_proposal" );
    sabComp( o, comp, "ncgb_attach_proposal" );
    if ( ncgb_mlp::device( m.net ) != o.mat->device )
      throw TypedError( "BadInput", "ncgb_attach_proposal: network and material on different devices" );
    const ncgb_sab_view hs = hostSab( o, comp );
    const int ne = (int)hs.ne;
    const double T = o.mat->tables->temperature();
    const ncgb_mlp::Ranges rg = ncgb_mlp::getRanges( m.net );
    // the network is evaluated at the sampler energies (egrid points) of this temperature
    std::vector<float> loge( ne ), temp( ne, (float)T );
    std::vector<unsigned char> allowed( ne, 0 );
    const bool t_ok = T >= rg.t_min - 1e-3 && T <= rg.t_max + 1e-3;
    for ( int i = 0; i < ne; ++i ) {
      loge[i] = (float)std::log( hs.egrid[i] );
      allowed[i] = ( t_ok && loge[i] >= rg.loge_min && loge[i] <= rg.loge_max ) ? 1 : 0;
    }
    checkCuda( cudaSetDevice( o.mat->device ), "cudaSetDevice" );
    float* d = nullptr;
    checkCuda( cudaMalloc( &d, (std::size_t)ne * ( 2 + ncgb_mlp::kOut ) * sizeof(float) ), "cudaMalloc" );
    std::unique_ptr<float, decltype(&cudaFree)> guard( d, &cudaFree );
    float* d_loge = d;
    float* d_temp = d + ne;
    float* d_knots = d + 2 * ne;
    checkCuda( cudaMemcpy( d_loge, loge.data(), ne * sizeof(float), cudaMemcpyHostToDevice ), "H2D" );
    checkCuda( cudaMemcpy( d_temp, temp.data(), ne * sizeof(float), cudaMemcpyHostToDevice ), "H2D" );
    ncgb_mlp::knots( m.net, d_loge, d_temp, ne, d_knots, nullptr );
    std::vector<float> knots( (std::size_t)ne * ncgb_mlp::kOut );
    checkCuda( cudaMemcpy( knots.data(), d_knots, knots.size() * sizeof(float), cudaMemcpyDeviceToHost ), "D2H" );
    const double a = attachKnots( o, comp, knots.data(), allowed.data(), min_accept );
    if ( mean_accept ) *mean_accept = a;
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_detach_proposal( ncrystal_scatter_t sc, int comp )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncgb_detach_proposal" );
    sabComp( o, comp, "ncgb_detach_proposal" );
    DeviceMaterial& dm = *o.mat;
    checkCuda( cudaDeviceSynchronize(), "synchronize before detaching" );
    dm.view.comp[comp].sab.lp_hdr = nullptr;
    dm.view.comp[comp].sab.lp_slot = nullptr;
    dm.view.comp[comp].sab.lp_cell = nullptr;
    dm.view.comp[comp].sab.lp_seg = nullptr;
    if ( dm.d_lp[comp] )
      cudaFree( dm.d_lp[comp] );
    dm.d_lp[comp] = nullptr;
    dm.h_lp[comp].clear();
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_proposal_acceptance( ncrystal_scatter_t sc, int comp, float* accept, int32_t* enabled )
{
  try {
    ScatterObj& o = extract( sc.internal, "ncgb_proposal_acceptance" );
    const ncgb_comp_view& c = sabComp( o, comp, "ncgb_proposal_acceptance" );
    const auto& h = o.mat->h_lp[comp];
    for ( int64_t i = 0; i < c.sab.ne; ++i ) {
      if ( accept ) accept[i] = h.empty() ? 0.f : h[i].accept;
      if ( enabled ) enabled[i] = h.empty() ? 0 : h[i].enabled;
    }
    return 0;
  } NCGB_CATCH;
  return 1;
}

ncgb_mlp_t ncgb_mlp_create( unsigned long long seed )
{
  try {
    int dev = 0;
    checkCuda( cudaGetDevice( &dev ), "cudaGetDevice" );
    std::unique_ptr<MlpObj> m( new MlpObj );
    m->net = ncgb_mlp::create( dev, seed );
    return ncgb_mlp_t{ m.release() };
  } NCGB_CATCH;
  return ncgb_mlp_t{ nullptr };
}

void ncgb_mlp_destroy( ncgb_mlp_t* net )
{
  try {
    if ( !net || !net->internal )
      return;
    MlpObj& m = extractMlp( net->internal, "ncgb_mlp_destroy" );
    cudaDeviceSynchronize();
    delete &m;
    net->internal = nullptr;
  } NCGB_CATCH;
}

unsigned long ncgb_mlp_nparams( void ) { return (unsigned long)ncgb_mlp::nparams(); }

int ncgb_mlp_get_params( ncgb_mlp_t net, float* out )
{
  try {
    ncgb_mlp::getParams( extractMlp( net.internal, "ncgb_mlp_get_params" ).net, out );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_mlp_set_params( ncgb_mlp_t net, const float* in )
{
  try {
    ncgb_mlp::setParams( extractMlp( net.internal, "ncgb_mlp_set_params" ).net, in );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_mlp_set_ranges( ncgb_mlp_t net, double emin, double emax, double tmin, double tmax )
{
  try {
    MlpObj& m = extractMlp( net.internal, "ncgb_mlp_set_ranges" );
    if ( !( emin > 0.0 && emax > emin && tmax > tmin ) )
      throw TypedError( "BadInput", "ncgb_mlp_set_ranges: need 0 < emin < emax and tmin < tmax" );
    ncgb_mlp::setRanges( m.net, ncgb_mlp::Ranges{ (float)std::log( emin ), (float)std::log( emax ), (float)tmin,
                                                  (float)tmax } );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_mlp_gradients( ncgb_mlp_t net, const float* d_loge, const float* d_temp, const float* d_target,
                        unsigned long n, float* h_grad, float* h_loss, void* stream )
{
  try {
    MlpObj& m = extractMlp( net.internal, "ncgb_mlp_gradients" );
    if ( n == 0 || n > ( 1ul << 22 ) )
      throw TypedError( "BadInput", "ncgb_mlp_gradients: n must be in [1, 2^22]" );
    const float l = ncgb_mlp::gradients( m.net, d_loge, d_temp, d_target, (int)n, h_grad,
                                         static_cast<cudaStream_t>( stream ) );
    if ( h_loss ) *h_loss = l;
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_mlp_train( ncgb_mlp_t net, const float* d_loge, const float* d_temp, const float* d_target,
                    unsigned long n, unsigned long steps, unsigned int batch, float lr, unsigned long long seed,
                    float* h_trace, unsigned long trace_every, void* stream )
{
  try {
    MlpObj& m = extractMlp( net.internal, "ncgb_mlp_train" );
    if ( batch == 0 || batch % 64 || batch > ( 1u << 20 ) )
      throw TypedError( "BadInput", "ncgb_mlp_train: batch must be a multiple of 64 up to 2^20" );
    ncgb_mlp::train( m.net, d_loge, d_temp, d_target, n, steps, (int)batch, lr, seed, h_trace, trace_every,
                     static_cast<cudaStream_t>( stream ) );
    return 0;
  } NCGB_CATCH;
  return 1;
}

int ncgb_mlp_knots( ncgb_mlp_t net, const float* d_loge, const float* d_temp, unsigned long n, float* d_knots,
                    void* stream )
{
  try {
    MlpObj& m = extractMlp( net.internal, "ncgb_mlp_knots" );
    if ( n == 0 || n > ( 1ul << 22 ) )
      throw TypedError( "BadInput", "ncgb_mlp_knots: n must be in [1, 2^22]" );
    ncgb_mlp::knots( m.net, d_loge, d_temp, (int)n, d_knots, static_cast<cudaStream_t>( stream ) );
    return 0;
  } NCGB_CATCH;
  return 1;
}

}
