// NCrystal plugin "GB300": serves NCrystal's non-oriented scattering requests
// from this library's GPU path, through NCrystal's own plugin surface.
//
// Loaded like any dynamic NCrystal plugin (NCRYSTAL_PLUGIN_LIST, read by
// NCPluginMgmt.cc:475-507), it registers one scatter factory
// ("GB300Factory", the pattern of examples/plugin/src/NCPluginFactory.cc:
// 77-114, with the C hooks of NCPluginBoilerplate.hh:81-90).  For a request
// that is not single-crystal, layered or UCN, the factory has NCrystal's
// standard factories build the usual process tree (globalCreateScatter, which
// excludes this factory), and claims the request with priority 150 -- above
// stdscat's 100 (NCStdScatFact.cc:99-102) -- when every component of that
// tree is one the GPU path implements (PowderBragg, ElIncScatter, SABScatter,
// FreeGas).  produce() writes the tree's material bundle (ncgb_export.cc) to
// the bundle cache and returns a ScatterIsotropicMat (NCProcImpl.hh:197-221)
// whose cross-sections and scatters are computed on the GPU.
//
// NCrystal calls a ProcImpl one neutron at a time (its batched methods exist
// only under NCRYSTAL_ALLOW_ABI_BREAKAGE, NCProcImpl.hh:129-154), so each call
// here is a device batch of one neutron: correct, but slow next to the batched
// C entry points (ncrystal_crosssection_nonoriented_many and friends), which
// remain the fast path.  A scatter draws a 64-bit key from the caller's RNG
// and samples on the Philox stream of that key, so results follow NCrystal's
// seeding.  Calls on one process are serialised (ProcImpl objects must be
// safe to share between threads).
//
// The plugin fails loudly: if the GPU library cannot be loaded, or has no
// device to put the material on, produce() throws and NCrystal reports the
// error; nothing falls back to a CPU model.  NCGB_PLUGIN_DISABLE=1 turns the
// factory off (every request is left to NCrystal's own factories).
//
// The GPU library exports NCrystal's C symbol names; NCrystal itself exports
// them too.  So the library is opened privately (RTLD_LOCAL) and its entry
// points are taken with dlsym from that handle, never through the global
// symbol scope.
#define NCPLUGIN_NAME GB300
#define NCPLUGIN_BOILERPLATE_CC
#include "NCrystal/NCPluginBoilerplate.hh"

#include <dlfcn.h>
#include <sys/stat.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <sstream>
#include <string>

#include "ncgb_export.hh"

namespace NCPluginNamespace {

  // ---- the GPU library, opened privately ---------------------------------------
  struct GpuLib {
    struct Handle { void* internal; };
    void* dl = nullptr;
    std::string error;
    Handle ( *create_bundle )( const char*, unsigned long ) = nullptr;
    Handle ( *scat2proc )( Handle ) = nullptr;
    void ( *xs )( Handle, double, double* ) = nullptr;
    int ( *scatter_keyed )( Handle, double, unsigned long long, double*, double* ) = nullptr;
    void ( *domain )( Handle, double*, double* ) = nullptr;
    void ( *unref )( void* ) = nullptr;
    int ( *haltonerror )( int ) = nullptr;
    int ( *quietonerror )( int ) = nullptr;
    int ( *has_error )() = nullptr;
    const char* ( *lasterror )() = nullptr;
    const char* ( *lasterrortype )() = nullptr;
    void ( *clearerror )() = nullptr;
    int ( *bundle_cache_dir )( char*, unsigned long ) = nullptr;

    static std::string pluginDir()
    {
      Dl_info info;
      if ( dladdr( reinterpret_cast<void*>( &GpuLib::pluginDir ), &info ) && info.dli_fname ) {
        std::string p( info.dli_fname );
        auto pos = p.rfind( '/' );
        return pos == std::string::npos ? std::string( "." ) : p.substr( 0, pos );
      }
      return ".";
    }

    template<class F> bool sym( F& f, const char* name )
    {
      f = reinterpret_cast<F>( dlsym( dl, name ) );
      if ( !f )
        error = std::string( "symbol " ) + name + " missing in the GB300 library";
      return f != nullptr;
    }

    GpuLib()
    {
      const char* env = std::getenv( "NCGB_LIBRARY" );
      const std::string path = env && *env ? std::string( env ) : pluginDir() + "/libncrystal_gb300.so";
      dl = dlopen( path.c_str(), RTLD_NOW | RTLD_LOCAL );
      if ( !dl ) {
        const char* e = dlerror();
        error = "cannot load the GB300 library " + path + ": " + ( e ? e : "?" );
        return;
      }
      bool ok = sym( create_bundle, "ncgb_create_scatter_bundle" ) && sym( scat2proc, "ncrystal_cast_scat2proc" )
                && sym( xs, "ncrystal_crosssection_nonoriented" )
                && sym( scatter_keyed, "ncgb_samplescatterisotropic_keyed" )
                && sym( domain, "ncrystal_domain" ) && sym( unref, "ncrystal_unref" )
                && sym( haltonerror, "ncrystal_sethaltonerror" ) && sym( quietonerror, "ncrystal_setquietonerror" )
                && sym( has_error, "ncrystal_error" ) && sym( lasterror, "ncrystal_lasterror" )
                && sym( lasterrortype, "ncrystal_lasterrortype" ) && sym( clearerror, "ncrystal_clearerror" )
                && sym( bundle_cache_dir, "ncgb_bundle_cache_dir" );
      if ( !ok ) {
        dl = nullptr;
        return;
      }
      // errors come back as return values, not as exit(1) or printed messages
      haltonerror( 0 );
      quietonerror( 1 );
    }

    bool ok() const { return dl != nullptr; }

    // Throws the library's pending error (if any) as an NCrystal exception.
    void check( const char* what ) const
    {
      if ( !has_error() )
        return;
      const std::string type = lasterrortype() ? lasterrortype() : "";
      const std::string msg = std::string( "GB300 plugin, " ) + what + ": " + ( lasterror() ? lasterror() : "?" );
      clearerror();
      if ( type == "FileNotFound" )
        NCRYSTAL_THROW( FileNotFound, msg );
      if ( type == "BadInput" )
        NCRYSTAL_THROW( BadInput, msg );
      if ( type == "CalcError" )
        NCRYSTAL_THROW( CalcError, msg );
      NCRYSTAL_THROW( LogicError, msg );
    }
  };

  GpuLib& gpu()
  {
    static GpuLib g;
    return g;
  }

  std::mutex& gpuMutex()
  {
    static std::mutex m;
    return m;
  }

  // ---- the GPU-backed process ----------------------------------------------------
  class GpuScatter final : public NC::ProcImpl::ScatterIsotropicMat {
  public:
    GpuScatter( GpuLib::Handle h, NC::EnergyDomain dom ) : m_h( h ), m_domain( dom ) {}
    ~GpuScatter() override
    {
      std::lock_guard<std::mutex> lock( gpuMutex() );
      gpu().unref( &m_h );
    }

    const char* name() const noexcept override { return "GB300Scatter"; }
    NC::EnergyDomain domain() const noexcept override { return m_domain; }

    NC::CrossSect crossSectionIsotropic( NC::CachePtr&, NC::NeutronEnergy ekin ) const override
    {
      std::lock_guard<std::mutex> lock( gpuMutex() );
      double r = -1.0;
      gpu().xs( gpu().scat2proc( m_h ), ekin.dbl(), &r );
      gpu().check( "cross-section" );
      return NC::CrossSect{ r };
    }

    NC::ScatterOutcomeIsotropic sampleScatterIsotropic( NC::CachePtr&, NC::RNG& rng,
                                                        NC::NeutronEnergy ekin ) const override
    {
      const unsigned long long key = rng.generate64RndmBits();
      std::lock_guard<std::mutex> lock( gpuMutex() );
      double ef = -1.0, mu = -999.0;
      gpu().scatter_keyed( m_h, ekin.dbl(), key, &ef, &mu );
      gpu().check( "scatter" );
      return { NC::NeutronEnergy{ ef }, NC::CosineScatAngle{ mu } };
    }

  private:
    mutable GpuLib::Handle m_h;
    NC::EnergyDomain m_domain;
  };

  // ---- the factory -----------------------------------------------------------------
  class GpuFactory final : public NC::FactImpl::ScatterFactory {
  public:
    const char* name() const noexcept override { return NCPLUGIN_NAME_CSTR "Factory"; }

    NC::Priority query( const NC::FactImpl::ScatterRequest& req ) const override
    {
      if ( disabled() )
        return NC::Priority::Unable;
      if ( req.isSingleCrystal() || req.isLayeredCrystal() || req.get_ucnmode().has_value() )
        return NC::Priority::Unable;
      auto std_tree = globalCreateScatter( req );
      if ( std_tree->isOriented() || !ncgb_export::supported( *std_tree ) )
        return NC::Priority::Unable;
      return NC::Priority{ 150 };
    }

    NC::ProcImpl::ProcPtr produce( const NC::FactImpl::ScatterRequest& req ) const override
    {
      auto std_tree = globalCreateScatter( req );
      GpuLib& g = gpu();
      if ( !g.ok() )
        NCRYSTAL_THROW2( LogicError, "GB300 plugin: " << g.error );
      std::ostringstream key;
      req.stream( key );
      const std::string keystr = "plugin:" + key.str();
      std::string dir;
      {
        std::lock_guard<std::mutex> lock( gpuMutex() );
        char buf[4096];
        if ( g.bundle_cache_dir( buf, sizeof( buf ) ) )
          g.check( "bundle cache directory" );
        dir = buf;
      }
      const std::string path = dir + "/" + fileName( keystr );
      struct stat st;
      if ( ::stat( path.c_str(), &st ) != 0 ) {
        const NC::Info& info = req.info();
        ncgb_export::writeBundle( path, keystr, *std_tree, info,
                                  info.hasTemperature() ? info.getTemperature().dbl() : -1.0, nullptr, false );
      }
      std::lock_guard<std::mutex> lock( gpuMutex() );
      GpuLib::Handle h = g.create_bundle( path.c_str(), 0 );
      g.check( "material upload" );
      double lo = 0.0, hi = 0.0;
      g.domain( g.scat2proc( h ), &lo, &hi );
      g.check( "domain" );
      return NC::makeSO<GpuScatter>( h, NC::EnergyDomain{ NC::NeutronEnergy{ lo }, NC::NeutronEnergy{ hi } } );
    }

  private:
    static bool disabled()
    {
      const char* e = std::getenv( "NCGB_PLUGIN_DISABLE" );
      return e && *e && std::strcmp( e, "0" ) != 0;
    }

    // bundle file of a request: 64-bit FNV-1a of its description
    static std::string fileName( const std::string& s )
    {
      uint64_t h = 1469598103934665603ull;
      for ( unsigned char c : s ) {
        h ^= c;
        h *= 1099511628211ull;
      }
      char buf[64];
      std::snprintf( buf, sizeof( buf ), "plugin_%016llx.ncgb", (unsigned long long)h );
      return buf;
    }
  };
}

void NCP::registerPlugin()
{
  NC::FactImpl::registerFactory( NC::ncmake_unique<NCP::GpuFactory>() );
}
