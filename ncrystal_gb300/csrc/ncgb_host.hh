// Host-side (C++) pieces of the GPU scattering path: material bundles and the
// table builder that turns a bundle into the flat ncgb_material_view layout.
#ifndef NCGB_HOST_HH
#define NCGB_HOST_HH

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ncgb_tables.h"

namespace ncgb {

  struct Error : std::runtime_error {
    explicit Error( const std::string& m ) : std::runtime_error(m) {}
  };

  // ---- material bundle (.ncgb) ----------------------------------------------
  class Bundle {
  public:
    static Bundle load( const std::string& path );
    bool has( const std::string& name ) const { return m_recs.count(name) != 0; }
    const std::vector<double>& f64( const std::string& name ) const;
    double f64s( const std::string& name ) const;
    int64_t i64s( const std::string& name ) const;
    const std::string& str( const std::string& name ) const;
    const std::string& path() const { return m_path; }
  private:
    struct Rec { uint32_t dtype; std::vector<double> d; std::vector<int64_t> i; std::string s; };
    std::map<std::string,Rec> m_recs;
    std::string m_path;
    const Rec& rec( const std::string& name, uint32_t dtype ) const;
  };

  // ---- flat tables ------------------------------------------------------------
  // All arrays of one material live in one byte arena (each array 256-byte
  // aligned) so a single upload moves the material to device memory.  The
  // view's pointer fields hold arena offsets until relocate() adds a base.
  class MaterialTables {
  public:
    // Build from a bundle: restates NCrystal's table derivation for SAB
    // (NCSABIntegrator.cc:95-145, :352-559) on the bundle's S(alpha,beta).
    static std::shared_ptr<MaterialTables> build( const Bundle& );
    // The same with the S(alpha,beta) samplers of some components derived
    // already (component index -> derived tables, e.g. from a batched device
    // derivation over many materials).
    static std::shared_ptr<MaterialTables> build( const Bundle&, const std::map<int, struct SABDerived>* pre );

    const std::vector<char>& arena() const { return m_arena; }
    std::size_t arenaBytes() const { return m_arena.size(); }
    // View with pointers into memory starting at 'base' (host copy of the
    // arena, or its device copy):
    ncgb_material_view relocate( const void* base ) const;
    const std::string& cfg() const { return m_cfg; }
    double temperature() const { return m_temperature; }

    // Host-side builder entry points, exposed for tests:
    template<class T> int64_t put( const std::vector<T>& v );
    template<class T> int64_t put( const T* p, std::size_t n );

    ncgb_material_view m_rel;   // offsets (+1, so 0 means "no array")
    std::vector<char> m_arena;
    std::string m_cfg;
    double m_temperature = -1.0;
    // material information (Info): atoms per Aa^3, temperature in K and Bragg
    // threshold in Aa; -1 where the material has none or the bundle lacks it
    double m_numdens = -1.0;
    double m_info_temperature = -1.0;
    double m_bragg_threshold = -1.0;
  };

  // SAB table derivation (restated reference algorithms), used by build():
  struct SABInput {
    std::vector<double> alpha, beta, sab, egrid;
    double kT = 0, sigma_bound = 0;
    double ext_sigma_free = 0, ext_ca = 0;
  };
  struct SABDerived {
    std::vector<double> logsab, cumul, xs;
    double kext = 0, k1 = 0, k2 = 0;
    std::vector<int32_t> kind, ibetaoffset, nbeta;
    std::vector<int64_t> offset;
    std::vector<double> fbkep, bx, by, bcdf;
    std::vector<ncgb_alpha_info> info;  // same offsets as bx (one unused slot per sampler)
  };
  SABDerived deriveSAB( const SABInput& );
  // The S(alpha,beta) inputs of every S(alpha,beta) component of a bundle.
  std::map<int, SABInput> sabInputs( const Bundle& );
  // The same on the current CUDA device (ncgb_sabderive.cu); used by build()
  // when NCGB_TABLES_BUILD=device.
  SABDerived deriveSABDevice( const SABInput& );
  std::vector<SABDerived> deriveSABDeviceMany( const std::vector<const SABInput*>& );

  // Free-gas cross-section shape (NCFreeGasUtils.cc:64-84):
  double freeGasXSShapeASq( double a_squared );
}

#endif
