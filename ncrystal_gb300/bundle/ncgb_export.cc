// ncgb_export -- host-side material loading through the reference NCrystal
// library, written out as a material bundle (.ncgb) for the GPU path.
//
// NCrystal keeps material loading on the host: NCMAT parsing, hkl plane
// generation, the VDOS -> S(alpha,beta) expansion and the SAB energy-grid
// selection all run once per material.  This tool runs exactly that code (the
// reference library, linked in) for one cfg-string, walks the resulting
// ProcComposition tree and records, per component, the data that the GPU
// table builder (ncrystal_gb300/csrc/ncgb_tables.cc) turns into device tables:
//
//   PowderBragg   2dE[] and fdm_commul[]      (NCPowderBragg.cc:68-104 output)
//   ElIncScatter  (msd, sigma*scale)[]         (NCElIncXS.hh:127 m_elm_data)
//   SABScatter    S(alpha,beta) kernel (SABData), kT, bound xs, the energy grid
//                 chosen by SABIntegrator::setupEnergyGrid
//                 (NCSABIntegrator.cc:202-281), the free-gas extender constants
//                 and the component's internal scale (NCSABScatter.hh:82)
//   FreeGas       T, kT, target mass, sigma_free, A/kT (NCFreeGas.cc:25-42)
//
// With --with-derived it also records the reference's own derived SAB tables
// (logS, cumulative alpha integrals, per-egrid-point Alg.1 samplers and
// cross-sections), which the tests compare bit-for-bit against the GPU table
// builder.  Those records are prefixed "ref." and are never read by the
// product.
//
// Member data of these classes is private in the reference, and none of it is
// reachable through a public accessor, so this translation unit is compiled
// with private/protected redefined as public after all standard headers are in.
// Nothing here changes the reference's behaviour.  The tool is built only where
// the reference sources exist.
//
// The same code serves three callers: the ncgb_export tool (built with
// NCGB_EXPORT_TOOL), the shared library libncgb_export.so, through which the
// GPU library exports a bundle on demand for a cfg-string that has none
// (ncgb_export_bundle below), and the NCrystal plugin (ncgb_plugin.cc), which
// exports the process tree NCrystal's standard factory made for a request.
//
// Usage:  ncgb_export [--with-derived] OUT.ncgb "cfg-string"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>
#include <thread>
#include <unistd.h>

#define private public
#define protected public
#include "NCrystal/NCrystal.hh"
#include "NCrystal/internal/powderbragg/NCPowderBragg.hh"
#include "NCrystal/internal/elincscatter/NCElIncScatter.hh"
#include "NCrystal/internal/phys_utils/NCElIncXS.hh"
#include "NCrystal/internal/sabscatter/NCSABScatter.hh"
#include "NCrystal/internal/sab/NCSABScatterHelper.hh"
#include "NCrystal/internal/sab/NCSABSampler.hh"
#include "NCrystal/internal/sab/NCSABSamplerModels.hh"
#include "NCrystal/internal/sab/NCSABXSProvider.hh"
#include "NCrystal/internal/sab/NCSABExtender.hh"
#include "NCrystal/internal/freegas/NCFreeGas.hh"
#include "NCrystal/internal/phys_utils/NCFreeGasUtils.hh"
#include "NCrystal/internal/absoov/NCAbsOOV.hh"
#undef private
#undef protected

#include "ncgb_export.hh"

namespace NC = NCrystal;

namespace {

  // ---- bundle writer: magic, record count, then named typed arrays ----------
  // record := u32 name_len | name | u32 dtype | u64 count | payload
  // dtype 1 = f64, 2 = i64, 3 = u32, 4 = raw bytes (strings)
  struct Bundle {
    struct Rec { std::string name; uint32_t dtype; uint64_t count; std::vector<char> bytes; };
    std::vector<Rec> recs;
    void f64( const std::string& n, const std::vector<double>& v ) { add(n,1,v.size(),v.data(),8); }
    void f64( const std::string& n, double v ) { add(n,1,1,&v,8); }
    void i64( const std::string& n, const std::vector<int64_t>& v ) { add(n,2,v.size(),v.data(),8); }
    void i64( const std::string& n, int64_t v ) { add(n,2,1,&v,8); }
    void u32( const std::string& n, const std::vector<uint32_t>& v ) { add(n,3,v.size(),v.data(),4); }
    void str( const std::string& n, const std::string& s ) { add(n,4,s.size(),s.data(),1); }
    void add( const std::string& n, uint32_t dt, uint64_t cnt, const void* p, size_t es )
    {
      Rec r{ n, dt, cnt, std::vector<char>( (const char*)p, (const char*)p + cnt*es ) };
      recs.push_back(std::move(r));
    }
    // Written to a temporary name in the target's directory and renamed into
    // place, so that concurrent readers and writers never see a partial file.
    void write( const std::string& path ) const
    {
      const std::string tmp = path + ".tmp" + std::to_string( (long)::getpid() ) + "_"
                              + std::to_string( (unsigned long)std::hash<std::thread::id>()( std::this_thread::get_id() ) );
      writeTo( tmp );
      if ( std::rename( tmp.c_str(), path.c_str() ) != 0 ) {
        std::remove( tmp.c_str() );
        throw std::runtime_error("cannot rename "+tmp+" to "+path);
      }
    }
    void writeTo( const std::string& path ) const
    {
      std::ofstream f(path, std::ios::binary);
      if (!f) throw std::runtime_error("cannot open "+path);
      f.write("NCGBNDL1",8);
      uint32_t n = recs.size();
      f.write((const char*)&n,4);
      for ( auto& r : recs ) {
        uint32_t nl = r.name.size();
        f.write((const char*)&nl,4);
        f.write(r.name.data(),nl);
        f.write((const char*)&r.dtype,4);
        f.write((const char*)&r.count,8);
        f.write(r.bytes.data(),r.bytes.size());
      }
      if (!f) throw std::runtime_error("write failed: "+path);
    }
  };

  // Layout mirror of NC::FreeGas::Impl (NCFreeGas.cc:27-42), which is defined
  // inside the reference's .cc file.
  struct FreeGasImplMirror {
    NC::FreeGasXSProvider m_xsprovider;
    NC::Temperature m_temperature;
    NC::AtomMass m_target_mass_amu;
  };

  void exportSAB( Bundle& b, const std::string& p, const NC::SABScatter& sc, bool withDerived )
  {
    const NC::SAB::SABScatterHelper& sh = *sc.m_sh;
    const NC::SABXSProvider& xp = sh.xsprovider;
    const NC::SABSampler& sp = sh.sampler;
    b.f64(p+"internal_scale", sc.m_scale);
    b.f64(p+"egrid", xp.m_egrid);
    b.f64(p+"kT", sp.m_kT);
    b.f64(p+"egrid_margin", sp.m_egridMargin.value);
    auto fgext = dynamic_cast<const NC::SAB::SABFGExtender*>(xp.m_extender.get());
    if ( !fgext )
      throw std::runtime_error("SABScatter with an extender other than SABFGExtender is not supported");
    b.f64(p+"ext_sigma_free", fgext->m_xsprovider.m_sigmaFree);
    b.f64(p+"ext_ca", fgext->m_xsprovider.m_ca);
    b.f64(p+"ext_T", fgext->m_t.dbl());
    b.f64(p+"ext_mass_amu", fgext->m_m.dbl());
    // The S(alpha,beta) kernel: every Alg.1 sampler holds the shared SABData.
    std::shared_ptr<const NC::SABData> data;
    for ( auto& s : sp.m_samplers ) {
      auto a1 = dynamic_cast<const NC::SAB::SABSamplerAtE_Alg1*>(s.get());
      if ( a1 ) { data = a1->m_common->data; break; }
    }
    if ( !data )
      throw std::runtime_error("SABScatter without any Alg.1 sampler");
    b.f64(p+"alpha", data->alphaGrid());
    b.f64(p+"beta", data->betaGrid());
    b.f64(p+"sab", data->sab());
    b.f64(p+"T", data->temperature().dbl());
    b.f64(p+"sab_kT", data->temperature().kT());
    b.f64(p+"sigma_bound", data->boundXS().dbl());
    b.f64(p+"mass_amu", data->elementMassAMU().dbl());
    b.f64(p+"suggested_emax", data->suggestedEmax());
    if ( !withDerived )
      return;
    // Reference-derived tables, for bit-for-bit checks of the GPU builder:
    b.f64(p+"ref.xs", xp.m_xs);
    b.f64(p+"ref.kExtension", xp.m_kExtension);
    b.f64(p+"ref.k1", sp.m_k1);
    b.f64(p+"ref.k2", sp.m_k2);
    b.f64(p+"ref.xsAtEmax", sp.m_xsAtEmax);
    std::shared_ptr<const NC::SAB::SABSamplerAtE_Alg1::CommonCache> common;
    std::vector<int64_t> kind, ibetaoff, nbeta, offs;
    std::vector<double> fbkep, bx, by, bcdf, info_d;
    std::vector<uint32_t> info_u;
    int64_t off = 0;
    for ( auto& s : sp.m_samplers ) {
      auto a1 = dynamic_cast<const NC::SAB::SABSamplerAtE_Alg1*>(s.get());
      if ( !a1 ) {
        kind.push_back(0); ibetaoff.push_back(0); nbeta.push_back(0);
        offs.push_back(off); fbkep.push_back(0.0);
        continue;
      }
      if (!common) common = a1->m_common;
      kind.push_back(1);
      ibetaoff.push_back(a1->m_ibetaOffset);
      fbkep.push_back(a1->m_firstBinKinematicEndpointValue);
      const auto& xs = a1->m_betaSampler.m_x;
      nbeta.push_back(xs.size());
      offs.push_back(off);
      off += xs.size();
      bx.insert(bx.end(),xs.begin(),xs.end());
      by.insert(by.end(),a1->m_betaSampler.m_y.begin(),a1->m_betaSampler.m_y.end());
      bcdf.insert(bcdf.end(),a1->m_betaSampler.m_cdf.begin(),a1->m_betaSampler.m_cdf.end());
      for ( auto& inf : a1->m_alphaSamplerInfos ) {
        info_d.push_back(inf.pt_front.alpha);
        info_d.push_back(inf.pt_front.sval);
        info_d.push_back(inf.pt_front.logsval);
        info_d.push_back(inf.pt_back.alpha);
        info_d.push_back(inf.pt_back.sval);
        info_d.push_back(inf.pt_back.logsval);
        info_d.push_back(inf.prob_front);
        info_d.push_back(inf.prob_notback);
        info_u.push_back(inf.pt_front.alpha_idx);
        info_u.push_back(inf.pt_back.alpha_idx);
      }
    }
    b.i64(p+"ref.smp_kind", kind);
    b.i64(p+"ref.smp_ibetaoffset", ibetaoff);
    b.i64(p+"ref.smp_nbeta", nbeta);
    b.i64(p+"ref.smp_offset", offs);
    b.f64(p+"ref.smp_fbkep", fbkep);
    b.f64(p+"ref.smp_beta_x", bx);
    b.f64(p+"ref.smp_beta_y", by);
    b.f64(p+"ref.smp_beta_cdf", bcdf);
    b.f64(p+"ref.smp_info_d", info_d);
    b.u32(p+"ref.smp_info_u", info_u);
    if ( common ) {
      b.f64(p+"ref.logsab", common->logsab);
      b.f64(p+"ref.cumul", common->alphaintegrals_cumul);
    }
  }

  void exportComponent( Bundle& b, int ic, double scale, const NC::ProcImpl::Process& proc, bool withDerived )
  {
    const std::string p = "c" + std::to_string(ic) + ".";
    b.f64(p+"scale", scale);
    auto dom = proc.domain();
    b.f64(p+"elow", dom.elow.dbl());
    b.f64(p+"ehigh", dom.ehigh.dbl());
    if ( auto pb = dynamic_cast<const NC::PowderBragg*>(&proc) ) {
      b.str(p+"type","PowderBragg");
      b.f64(p+"two_dE", pb->m_2dE);
      b.f64(p+"fdm_commul", pb->m_fdm_commul);
      b.f64(p+"threshold", pb->m_threshold.dbl());
    } else if ( auto ei = dynamic_cast<const NC::ElIncScatter*>(&proc) ) {
      b.str(p+"type","ElIncScatter");
      std::vector<double> msd, sig;
      for ( auto& e : ei->m_elincxs->m_elm_data ) {
        msd.push_back(e.first);
        sig.push_back(e.second);
      }
      b.f64(p+"msd", msd);
      b.f64(p+"sigma", sig);
    } else if ( auto sab = dynamic_cast<const NC::SABScatter*>(&proc) ) {
      b.str(p+"type","SABScatter");
      exportSAB(b,p,*sab,withDerived);
    } else if ( auto fg = dynamic_cast<const NC::FreeGas*>(&proc) ) {
      b.str(p+"type","FreeGas");
      auto impl = reinterpret_cast<const FreeGasImplMirror*>(fg->m_impl.m_ptr);
      b.f64(p+"T", impl->m_temperature.dbl());
      b.f64(p+"kT", impl->m_temperature.kT());
      b.f64(p+"mass_amu", impl->m_target_mass_amu.dbl());
      b.f64(p+"sigma_free", impl->m_xsprovider.m_sigmaFree);
      b.f64(p+"ca", impl->m_xsprovider.m_ca);
    } else {
      throw std::runtime_error(std::string("unsupported component type: ")+proc.name());
    }
  }
}

namespace ncgb_export {

  void writeBundle( const std::string& path, const std::string& cfgkey, const NC::ProcImpl::Process& top,
                    const NC::Info& info, double temperature, const NC::ProcImpl::Process* absorption,
                    bool withDerived )
  {
    Bundle b;
    b.str("cfg", cfgkey);
    b.str("ncrystal_version", NCRYSTAL_VERSION_STR);
    auto dom = top.domain();
    b.f64("elow", dom.elow.dbl());
    b.f64("ehigh", dom.ehigh.dbl());
    b.f64("temperature", temperature);
    // material information used by the MiniMC engine: number density
    // (macroXSFactor, NCMMC_Utils.hh:103-105), temperature if well defined, and
    // the Bragg threshold as the scenario decoder takes it (the largest over
    // the phases, NCMMC_Utils.cc:218-241); -1 where absent
    b.f64("info.numdens", info.getNumberDensity().dbl());
    b.f64("info.temperature", info.hasTemperature() ? info.getTemperature().dbl() : -1.0);
    {
      NC::Optional<NC::NeutronWavelength> bt;
      if ( info.isSinglePhase() ) {
        bt = info.getBraggThreshold();
      } else {
        for ( auto& ph : info.getPhases() ) {
          auto pbt = ph.second->getBraggThreshold();
          if ( pbt.has_value() && ( !bt.has_value() || bt.value() < pbt.value() ) )
            bt = pbt;
        }
      }
      b.f64("info.bragg_threshold", bt.has_value() ? bt.value().dbl() : -1.0);
    }
    int nc = 0;
    if ( auto pc = dynamic_cast<const NC::ProcImpl::ProcComposition*>(&top) ) {
      for ( auto& c : pc->components() )
        exportComponent(b, nc++, c.scale, *c.process, withDerived);
    } else if ( top.isNull() ) {
      // no components: vanishing cross-section everywhere
    } else {
      exportComponent(b, nc++, 1.0, top, withDerived);
    }
    b.i64("ncomp", nc);
    // absorption: the standard factory's AbsOOV (NCStdAbsFact.cc:49-52), xs =
    // c/sqrt(E) (NCAbsOOV.cc:33-44); c = 0 means no absorption; -1: not recorded
    if ( !absorption ) {
      b.f64("abs_c", -1.0);
    } else if ( auto oov = dynamic_cast<const NC::AbsOOV*>(absorption) ) {
      b.f64("abs_c", oov->m_c);
    } else if ( absorption->isNull() ) {
      b.f64("abs_c", 0.0);
    } else {
      throw std::runtime_error("unsupported absorption process type");
    }
    b.write(path);
  }

  void exportCfg( const std::string& cfgstr, const std::string& path, bool withDerived )
  {
    NC::MatCfg cfg(cfgstr);
    auto sc = NC::createScatter(cfg);
    auto info = NC::createInfo(cfg);
    auto ab = NC::createAbsorption(cfg);
    writeBundle( path, cfgstr, sc.underlying(), *info, cfg.get_temp().dbl(), &ab.underlying(), withDerived );
  }

  bool supported( const NC::ProcImpl::Process& top )
  {
    auto one = []( const NC::ProcImpl::Process& p ) {
      return dynamic_cast<const NC::PowderBragg*>(&p) || dynamic_cast<const NC::ElIncScatter*>(&p)
             || dynamic_cast<const NC::SABScatter*>(&p) || dynamic_cast<const NC::FreeGas*>(&p);
    };
    if ( top.isNull() )
      return true;
    if ( auto pc = dynamic_cast<const NC::ProcImpl::ProcComposition*>(&top) ) {
      if ( pc->components().size() > 8 )
        return false;
      for ( auto& c : pc->components() )
        if ( !one( *c.process ) )
          return false;
      return true;
    }
    return one( top );
  }
}

// The bundle of one cfg-string written to 'path'.  Returns 0, or 1 with
// NCrystal's error message and type name ("FileNotFound", "BadInput", ...)
// copied into err / type.
extern "C" int ncgb_export_bundle( const char* cfgstr, const char* path, char* err, unsigned long errlen,
                                   char* type, unsigned long typelen )
{
  auto put = []( char* dst, unsigned long len, const char* src ) {
    if ( dst && len ) {
      std::strncpy( dst, src, len - 1 );
      dst[len - 1] = 0;
    }
  };
  try {
    ncgb_export::exportCfg( cfgstr, path, false );
    return 0;
  } catch ( NC::Error::Exception& e ) {
    put( err, errlen, e.what() );
    put( type, typelen, e.getTypeName() );
  } catch ( std::exception& e ) {
    put( err, errlen, e.what() );
    put( type, typelen, "BadInput" );
  }
  return 1;
}

#ifdef NCGB_EXPORT_TOOL
int main( int argc, char** argv )
{
  bool withDerived = false;
  std::vector<std::string> args;
  for ( int i = 1; i < argc; ++i ) {
    if ( std::strcmp(argv[i],"--with-derived") == 0 )
      withDerived = true;
    else
      args.push_back(argv[i]);
  }
  if ( args.size() != 2 ) {
    std::fprintf(stderr,"usage: %s [--with-derived] OUT.ncgb \"cfg-string\"\n",argv[0]);
    return 2;
  }
  try {
    ncgb_export::exportCfg( args[1], args[0], withDerived );
  } catch ( std::exception& e ) {
    std::fprintf(stderr,"ncgb_export error: %s\n",e.what());
    return 1;
  }
  return 0;
}
#endif
