// Table builder: material bundle -> flat ncgb_material_view arena.
//
// PowderBragg, ElIncScatter and FreeGas tables are taken over as loaded.  For
// SABScatter the bundle holds the S(alpha,beta) kernel and the energy grid;
// the per-energy-point Alg.1 samplers and cross-sections are derived here by
// restating NCrystal's own construction, step for step, so that the tables are
// the ones the reference would sample from:
//
//   logS and cumulative alpha integrals  NCSABIntegrator.cc:111-142
//   activeGridRanges                      NCSABUtils.cc:460-536
//   createTailedBreakdown                 NCSABUtils.cc:538-633
//   analyseEnergyPoint                    NCSABIntegrator.cc:352-559
//   PointwiseDist normalisation           NCPointwiseDist.cc:28-74
//   SABXSProvider / SABSampler constants  NCSABXSProvider.cc:35-52,
//                                         NCSABSampler.cc:41-57
//
// Compiled with -ffp-contract=off so that x86-64 and aarch64 hosts produce the
// same bits (gcc contracts a*b+c into fma on aarch64 by default).
#include "ncgb_host.hh"
#include "ncgb_sabderive.hh"

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <limits>

namespace ncgb {

  namespace {

    constexpr double kInf = std::numeric_limits<double>::infinity();
    constexpr double kInvSqrtPi = 0.564189583547756286948079451560772585844050629;

    // Neumaier sums, kinematic alpha limits, alpha-interval integrals and the
    // tailed breakdown of one beta row: shared with the device builder.
    using sabd::StableSum;
    using sabd::ALim;
    using sabd::alphaLimits;
    using sabd::integrateAlphaIntervalFast;
    using sabd::TailedBreakdown;
    using sabd::tailedBreakdown;


    // NCSABUtils.cc:460-536
    void activeGridRanges( const std::vector<double>& alphaGrid, const std::vector<double>& betaGrid,
                           double ekin_div_kT,
                           std::vector<std::pair<uint16_t,uint16_t>>& out, std::size_t& ibeta_low )
    {
      const std::size_t na = alphaGrid.size();
      if ( na >= std::numeric_limits<uint16_t>::max() )
        throw Error("alpha grid too large");
      ibeta_low = 0;
      out.clear();
      const double agrid_front = alphaGrid.front();
      const double agrid_back = alphaGrid.back();
      const std::size_t iLast = na - 1;
      std::size_t iLow = 0, iUpp = na - 1;
      for ( std::size_t ib = 0; ib < betaGrid.size(); ++ib ) {
        const double beta = betaGrid[ib];
        double alow(-1.0), aupp(-2.0);
        if ( beta > -ekin_div_kT ) {
          auto al = alphaLimits( ekin_div_kT, beta );
          alow = al.lo;
          aupp = al.hi;
        }
        if ( agrid_back <= alow || agrid_front >= aupp || aupp < alow ) {
          if ( out.empty() ) {
            ibeta_low = ib + 1;
          } else {
            auto nau = static_cast<uint16_t>(na);
            out.emplace_back(nau,nau);
          }
          continue;
        }
        while ( alphaGrid[iLow] > alow && iLow > 0 )
          --iLow;
        while ( iLow < iLast && alphaGrid[iLow+1] <= alow )
          ++iLow;
        if ( iUpp < iLow )
          iUpp = iLow;
        while ( alphaGrid[iUpp] < aupp && iUpp < iLast )
          ++iUpp;
        while ( iUpp > 0 && alphaGrid[iUpp-1] >= aupp )
          --iUpp;
        out.emplace_back( static_cast<uint16_t>(iLow), static_cast<uint16_t>(iUpp) );
      }
    }

    struct EPoint {
      double xs = 0.0;
      int kind = 0; // 0 no-scatter, 1 Alg.1
      std::size_t ibeta_low = 0;
      double fbkep = 1.0;
      std::vector<double> bvals, bweights;
      std::vector<ncgb_alpha_info> infos;
    };

    // NCSABIntegrator.cc:352-559 (doSampler = true)
    EPoint analyseEnergyPoint( const SABInput& in, const std::vector<double>& logsab,
                               const std::vector<double>& cumul, double ekin )
    {
      const auto& betaGrid = in.beta;
      const auto& alphaGrid = in.alpha;
      const std::size_t na = alphaGrid.size();
      const double kT = in.kT;
      const double ekin_div_kT = ekin / kT;
      double beta_lower_limit = -ekin_div_kT;
      bool starts_at_kinematic_endpoint = true;
      if ( beta_lower_limit < betaGrid.front() ) {
        double c1 = betaGrid.front() - (betaGrid.at(1)-betaGrid.front()) * 1e-6;
        double c2 = betaGrid.front() - std::fabs(betaGrid.front())*1e-13;
        double c3 = std::nextafter( betaGrid.front(), beta_lower_limit );
        beta_lower_limit = std::min( c1, std::min( c2, c3 ) );
        starts_at_kinematic_endpoint = false;
      }
      std::vector<std::pair<uint16_t,uint16_t>> alpharanges;
      std::size_t ibeta_low;
      activeGridRanges( alphaGrid, betaGrid, ekin_div_kT, alpharanges, ibeta_low );
      EPoint res;
      if ( ibeta_low >= betaGrid.size() )
        return res; // no-scatter sampler, xs = 0
      if ( ibeta_low > 0 && beta_lower_limit < betaGrid[ibeta_low-1] ) {
        beta_lower_limit = betaGrid[ibeta_low-1];
        starts_at_kinematic_endpoint = false;
      }
      const std::size_t nrel = betaGrid.size() - ibeta_low;
      double prev_first = beta_lower_limit, prev_second = 0.0;
      res.bvals.reserve( nrel + 1 );
      res.bweights.reserve( nrel + 1 );
      res.infos.reserve( nrel );
      res.bvals.push_back( prev_first );
      res.bweights.push_back( prev_second );
      StableSum xs_total_stable;
      bool next_bin_has_kinematic_endpoint = starts_at_kinematic_endpoint;
      for ( std::size_t idx = 0; idx < nrel; ++idx ) {
        const double beta = betaGrid[ibeta_low + idx];
        if ( beta == beta_lower_limit )
          continue;
        auto al = alphaLimits( ekin_div_kT, beta );
        const double alow = al.lo, aupp = al.hi;
        double xs_at_this_beta = 0.0;
        unsigned aidx_low = alpharanges[idx].first, aidx_upp = alpharanges[idx].second;
        TailedBreakdown tb;
        if ( aidx_upp > aidx_low && aupp > alow ) {
          const std::size_t slice = na * ( idx + ibeta_low );
          tb = tailedBreakdown( alphaGrid.data(), na, in.sab.data() + slice, logsab.data() + slice,
                                cumul.data() + slice, alow, aupp, aidx_low, aidx_upp );
          xs_at_this_beta = tb.xs_front + tb.xs_back + tb.xs_middle;
        }
        ncgb_alpha_info info;
        std::memset( &info, 0, sizeof(info) );
        if ( xs_at_this_beta > 0.0 ) {
          info.front_alpha = tb.front.alpha;
          info.front_sval = tb.front.sval;
          info.front_logsval = tb.front.logsval;
          info.back_alpha = tb.back.alpha;
          info.back_sval = tb.back.sval;
          info.back_logsval = tb.back.logsval;
          if ( tb.narrow ) {
            info.prob_front = 1.0;
          } else {
            info.prob_front = tb.xs_front / xs_at_this_beta;
            info.prob_notback = 1.0 - tb.xs_back / xs_at_this_beta;
            info.front_idx = tb.imiddle_low;
            info.back_idx = tb.imiddle_upp;
          }
        } else {
          info.prob_front = 2.0;
          info.front_alpha = alow;
          info.back_alpha = aupp;
        }
        res.infos.push_back( info );
        if ( next_bin_has_kinematic_endpoint ) {
          next_bin_has_kinematic_endpoint = false;
          double db_real = ( beta - prev_first );
          prev_first -= db_real * ( 1.0 / 3.0 );
          res.bvals.front() = prev_first;
        }
        xs_total_stable.add( 0.5 * ( beta - prev_first ) * ( xs_at_this_beta + prev_second ) );
        prev_first = beta;
        prev_second = xs_at_this_beta;
        res.bvals.push_back( prev_first );
        res.bweights.push_back( prev_second );
      }
      double xs_total = xs_total_stable.sum() * in.sigma_bound / ( 4 * ekin_div_kT );
      if ( !( xs_total >= 0.0 ) )
        xs_total = 0.0;
      res.xs = xs_total;
      if ( xs_total == 0.0 )
        return res; // no-scatter sampler
      res.kind = 1;
      res.ibeta_low = ibeta_low;
      res.fbkep = ( starts_at_kinematic_endpoint ? beta_lower_limit : 1.0 );
      return res;
    }

    // PointwiseDist construction (NCPointwiseDist.cc:28-74): normalised y and cdf.
    void pointwiseDist( const std::vector<double>& x, std::vector<double> y,
                        std::vector<double>& out_y, std::vector<double>& out_cdf )
    {
      if ( x.size() != y.size() || y.size() < 2 )
        throw Error("PointwiseDist: input vector size error");
      if ( !std::is_sorted( x.begin(), x.end() ) )
        throw Error("PointwiseDist: points of the distribution are not sorted");
      for ( double v : y )
        if ( v < 0.0 || std::isinf(v) )
          throw Error("PointwiseDist: function is negative or not finite");
      std::vector<double> cdf;
      cdf.reserve( y.size() );
      StableSum totalArea;
      cdf.push_back( 0.0 );
      for ( std::size_t i = 1; i < y.size(); ++i ) {
        double area = ( x[i] - x[i-1] ) * 0.5 * ( y[i] + y[i-1] );
        if ( area < 0 )
          throw Error("PointwiseDist: negative probability density");
        totalArea.add( area );
        cdf.push_back( totalArea.sum() );
      }
      double totalAreaVal = totalArea.sum();
      if ( !( totalAreaVal > 0.0 ) )
        throw Error("PointwiseDist: no area in distribution");
      double normfact = 1.0 / totalAreaVal;
      for ( auto& e : cdf )
        e *= normfact;
      for ( auto& e : y )
        e *= normfact;
      cdf.back() = 1.0;
      out_y = std::move(y);
      out_cdf = std::move(cdf);
    }
  }

  double freeGasXSShapeASq( double a_squared )
  {
    if ( a_squared > 36.0 )
      return 1.0 + 0.5 / a_squared;
    const double a = std::sqrt( a_squared );
    if ( a < 0.1 ) {
      if ( a == 0.0 )
        return kInf;
      constexpr double c1 = 2.0/3.0;
      constexpr double c2 = 1.0/15.0;
      constexpr double c3 = 1.0/105.0;
      constexpr double c4 = 1.0/756.0;
      constexpr double c5 = 1.0/5940.0;
      const double a2 = a_squared;
      return kInvSqrtPi * ( 2.0 / a + a *( c1- a2*(c2-a2*(c3-a2*(c4-a2*c5)))));
    }
    const double inva = 1.0 / a;
    return ( 1.0 + 0.5*inva*inva ) * std::erf(a) + kInvSqrtPi * std::exp(-a_squared)*inva;
  }

  SABDerived deriveSAB( const SABInput& in )
  {
    const std::size_t na = in.alpha.size(), nb = in.beta.size();
    if ( na < 2 || nb < 2 || in.sab.size() != na*nb )
      throw Error("SAB kernel with inconsistent grid sizes");
    if ( in.egrid.size() < 2 )
      throw Error("SAB energy grid too small");
    SABDerived d;
    // logS and cumulative alpha integrals (NCSABIntegrator.cc:119-138):
    d.logsab.reserve( in.sab.size() );
    for ( double e : in.sab )
      d.logsab.push_back( e > 0.0 ? std::log(e) : -kInf );
    d.cumul.assign( in.sab.size(), 0.0 );
    std::size_t g = 0;
    for ( std::size_t ib = 0; ib < nb; ++ib, ++g ) {
      double c = 0.0;
      for ( std::size_t ai = 0; ai + 1 < na; ++ai, ++g ) {
        double integ = integrateAlphaIntervalFast( in.alpha[ai], in.sab[g], in.alpha[ai+1], in.sab[g+1],
                                                   d.logsab[g], d.logsab[g+1] );
        d.cumul[g+1] = ( c += integ );
      }
    }
    // One sampler + xs value per energy-grid point (NCSABIntegrator.cc:283-309):
    const std::size_t ne = in.egrid.size();
    d.xs.reserve(ne);
    int64_t off = 0;
    for ( std::size_t ie = 0; ie < ne; ++ie ) {
      EPoint ep = analyseEnergyPoint( in, d.logsab, d.cumul, in.egrid[ie] );
      d.xs.push_back( ep.xs );
      d.kind.push_back( ep.kind );
      d.offset.push_back( off );
      if ( ep.kind == 0 ) {
        d.ibetaoffset.push_back(0);
        d.nbeta.push_back(0);
        d.fbkep.push_back(0.0);
        continue;
      }
      std::vector<double> ny, ncdf;
      pointwiseDist( ep.bvals, ep.bweights, ny, ncdf );
      d.ibetaoffset.push_back( static_cast<int32_t>( ep.ibeta_low ) );
      d.nbeta.push_back( static_cast<int32_t>( ep.bvals.size() ) );
      d.fbkep.push_back( ep.fbkep );
      d.bx.insert( d.bx.end(), ep.bvals.begin(), ep.bvals.end() );
      d.by.insert( d.by.end(), ny.begin(), ny.end() );
      d.bcdf.insert( d.bcdf.end(), ncdf.begin(), ncdf.end() );
      d.info.insert( d.info.end(), ep.infos.begin(), ep.infos.end() );
      ncgb_alpha_info pad;
      std::memset( &pad, 0, sizeof(pad) );
      while ( d.info.size() < d.bx.size() )
        d.info.push_back( pad );
      off += static_cast<int64_t>( ep.bvals.size() );
    }
    // Extender constants (NCSABXSProvider.cc:35-52, NCSABSampler.cc:41-57):
    const double emax = in.egrid.back();
    const double extxs_emax = in.ext_sigma_free * freeGasXSShapeASq( in.ext_ca * emax );
    d.kext = ( d.xs.back() - extxs_emax ) * emax;
    d.k1 = d.xs.back() * emax;
    d.k2 = extxs_emax * emax;
    return d;
  }

  // ---- arena ------------------------------------------------------------------

  template<class T>
  int64_t MaterialTables::put( const T* p, std::size_t n )
  {
    if ( n == 0 )
      return 0;
    std::size_t off = ( m_arena.size() + 255 ) & ~std::size_t(255);
    m_arena.resize( off + n * sizeof(T) );
    std::memcpy( m_arena.data() + off, p, n * sizeof(T) );
    return static_cast<int64_t>( off ) + 1;
  }

  template<class T>
  int64_t MaterialTables::put( const std::vector<T>& v ) { return put( v.data(), v.size() ); }

  template int64_t MaterialTables::put<double>( const std::vector<double>& );
  template int64_t MaterialTables::put<int32_t>( const std::vector<int32_t>& );
  template int64_t MaterialTables::put<int64_t>( const std::vector<int64_t>& );

  namespace {
    template<class T>
    const T* encodeOff( int64_t off ) { return reinterpret_cast<const T*>( static_cast<uintptr_t>(off) ); }
    template<class T>
    const T* reloc( const T* enc, const char* base )
    {
      uintptr_t off = reinterpret_cast<uintptr_t>(enc);
      return off ? reinterpret_cast<const T*>( base + ( off - 1 ) ) : nullptr;
    }
  }

  // NCGB_TABLES_BUILD=device: derive the S(alpha,beta) samplers on the GPU.
  static bool deviceDerive()
  {
    const char* v = std::getenv( "NCGB_TABLES_BUILD" );
    return v && std::string( v ) == "device";
  }

  std::map<int, SABInput> sabInputs( const Bundle& b )
  {
    std::map<int, SABInput> out;
    const int nc = static_cast<int>( b.i64s( "ncomp" ) );
    for ( int ic = 0; ic < nc; ++ic ) {
      const std::string p = "c" + std::to_string( ic ) + ".";
      if ( !b.has( p + "sab" ) )
        continue;
      SABInput in;
      in.alpha = b.f64( p + "alpha" );
      in.beta = b.f64( p + "beta" );
      in.sab = b.f64( p + "sab" );
      in.egrid = b.f64( p + "egrid" );
      in.kT = b.f64s( p + "sab_kT" );
      in.sigma_bound = b.f64s( p + "sigma_bound" );
      in.ext_sigma_free = b.f64s( p + "ext_sigma_free" );
      in.ext_ca = b.f64s( p + "ext_ca" );
      out.emplace( ic, std::move( in ) );
    }
    return out;
  }

  std::shared_ptr<MaterialTables> MaterialTables::build( const Bundle& b )
  {
    return build( b, nullptr );
  }

  std::shared_ptr<MaterialTables> MaterialTables::build( const Bundle& b, const std::map<int, SABDerived>* pre )
  {
    auto mt = std::make_shared<MaterialTables>();
    mt->m_cfg = b.str("cfg");
    mt->m_temperature = b.has("temperature") ? b.f64s("temperature") : -1.0;
    mt->m_numdens = b.has("info.numdens") ? b.f64s("info.numdens") : -1.0;
    mt->m_info_temperature = b.has("info.temperature") ? b.f64s("info.temperature") : -1.0;
    mt->m_bragg_threshold = b.has("info.bragg_threshold") ? b.f64s("info.bragg_threshold") : -1.0;
    ncgb_material_view& v = mt->m_rel;
    std::memset( &v, 0, sizeof(v) );
    const int64_t ncomp = b.i64s("ncomp");
    if ( ncomp < 0 || ncomp > NCGB_MAX_COMP )
      throw Error("material has too many components for the GPU path");
    v.ncomp = static_cast<int32_t>( ncomp );
    v.dom_elow = b.f64s("elow");
    v.dom_ehigh = b.f64s("ehigh");
    v.abs_c = b.has("abs_c") ? b.f64s("abs_c") : -1.0;
    if ( ncomp == 0 ) {
      // A null process: empty domain, so xs = 0 and scatterings leave E unchanged.
      v.dom_elow = kInf;
      v.dom_ehigh = kInf;
    }
    for ( int64_t ic = 0; ic < ncomp; ++ic ) {
      const std::string p = "c" + std::to_string(ic) + ".";
      ncgb_comp_view& c = v.comp[ic];
      c.scale = b.f64s(p+"scale");
      c.scale_f = static_cast<float>( c.scale );
      c.elow = b.f64s(p+"elow");
      c.ehigh = b.f64s(p+"ehigh");
      const std::string& type = b.str(p+"type");
      if ( type == "PowderBragg" ) {
        c.type = NCGB_COMP_BRAGG;
        const auto& a = b.f64(p+"two_dE");
        const auto& f = b.f64(p+"fdm_commul");
        if ( a.size() != f.size() )
          throw Error("PowderBragg table size mismatch");
        c.bragg.n = static_cast<int64_t>( a.size() );
        c.bragg.threshold = a.empty() ? kInf : a.front();
        c.bragg.two_dE = encodeOff<double>( mt->put(a) );
        c.bragg.fdm_commul = encodeOff<double>( mt->put(f) );
      } else if ( type == "ElIncScatter" ) {
        c.type = NCGB_COMP_ELINC;
        const auto& msd = b.f64(p+"msd");
        const auto& sig = b.f64(p+"sigma");
        if ( msd.size() != sig.size() || msd.size() > NCGB_MAX_ELINC || msd.empty() )
          throw Error("ElIncScatter with unsupported element count");
        c.elinc.n = static_cast<int32_t>( msd.size() );
        for ( std::size_t i = 0; i < msd.size(); ++i ) {
          c.elinc.msd[i] = msd[i];
          c.elinc.sigma[i] = sig[i];
          c.elinc.msd_f[i] = static_cast<float>( msd[i] );
          c.elinc.sigma_f[i] = static_cast<float>( sig[i] );
        }
      } else if ( type == "SABScatter" ) {
        c.type = NCGB_COMP_SAB;
        SABInput in;
        in.alpha = b.f64(p+"alpha");
        in.beta = b.f64(p+"beta");
        in.sab = b.f64(p+"sab");
        in.egrid = b.f64(p+"egrid");
        in.kT = b.f64s(p+"sab_kT");
        in.sigma_bound = b.f64s(p+"sigma_bound");
        in.ext_sigma_free = b.f64s(p+"ext_sigma_free");
        in.ext_ca = b.f64s(p+"ext_ca");
        const auto it = pre ? pre->find( ic ) : std::map<int, SABDerived>::const_iterator();
        SABDerived d = ( pre && it != pre->end() ) ? it->second
                       : ( deviceDerive() ? deriveSABDevice( in ) : deriveSAB( in ) );
        ncgb_sab_view& s = c.sab;
        s.kT = b.f64s(p+"kT");
        s.egrid_margin = b.f64s(p+"egrid_margin");
        s.internal_scale = b.f64s(p+"internal_scale");
        s.internal_scale_f = (float)s.internal_scale;
        s.kext = d.kext;
        s.k1 = d.k1;
        s.k2 = d.k2;
        s.ext_sigma_free = in.ext_sigma_free;
        s.ext_ca = in.ext_ca;
        s.ext_kT = in.kT;
        s.ext_mass_amu = b.f64s(p+"ext_mass_amu");
        s.sigma_bound = in.sigma_bound;
        // the sampling kernels index these tables with 32-bit integers
        if ( in.alpha.size() * in.beta.size() >= ( std::size_t( 1 ) << 31 )
             || d.bx.size() >= ( std::size_t( 1 ) << 31 ) )
          throw Error( "S(alpha,beta) table too large for the GPU sampler (2^31 entries)" );
        s.ne = static_cast<int32_t>( in.egrid.size() );
        s.na = static_cast<int32_t>( in.alpha.size() );
        s.nb = static_cast<int32_t>( in.beta.size() );
        s.egrid = encodeOff<double>( mt->put(in.egrid) );
        s.xs = encodeOff<double>( mt->put(d.xs) );
        s.alpha = encodeOff<double>( mt->put(in.alpha) );
        s.beta = encodeOff<double>( mt->put(in.beta) );
        s.sab = encodeOff<double>( mt->put(in.sab) );
        s.logsab = encodeOff<double>( mt->put(d.logsab) );
        s.cumul = encodeOff<double>( mt->put(d.cumul) );
        s.smp_kind = encodeOff<int32_t>( mt->put(d.kind) );
        s.smp_ibetaoffset = encodeOff<int32_t>( mt->put(d.ibetaoffset) );
        s.smp_nbeta = encodeOff<int32_t>( mt->put(d.nbeta) );
        s.smp_offset = encodeOff<int64_t>( mt->put(d.offset) );
        s.smp_fbkep = encodeOff<double>( mt->put(d.fbkep) );
        s.bx = encodeOff<double>( mt->put(d.bx) );
        s.by = encodeOff<double>( mt->put(d.by) );
        s.bcdf = encodeOff<double>( mt->put(d.bcdf) );
        // Precomputed constants for the GPU (reciprocals instead of divisions):
        for ( auto& inf : d.info ) {
          inf.inv_front = inf.prob_front != 0.0 ? 1.0 / inf.prob_front : 0.0;
          const double mid = inf.prob_notback - inf.prob_front;
          inf.inv_middle = mid != 0.0 ? 1.0 / mid : 0.0;
          const double back = 1.0 - inf.prob_notback;
          inf.inv_back = back != 0.0 ? 1.0 / back : 0.0;
        }
        s.info = encodeOff<ncgb_alpha_info>( mt->put( d.info.data(), d.info.size() ) );
        s.inv_kT = 1.0 / s.kT;
        std::vector<double> inv_dE( in.egrid.size(), 0.0 ), inv_dbeta( in.beta.size(), 0.0 );
        for ( std::size_t i = 0; i + 1 < in.egrid.size(); ++i )
          inv_dE[i] = 1.0 / ( in.egrid[i+1] - in.egrid[i] );
        for ( std::size_t i = 0; i + 1 < in.beta.size(); ++i )
          inv_dbeta[i] = 1.0 / ( in.beta[i+1] - in.beta[i] );
        s.inv_dE = encodeOff<double>( mt->put( inv_dE ) );
        s.inv_dbeta = encodeOff<double>( mt->put( inv_dbeta ) );
        // FP32 cross-section tables of the mixed-precision mode (xs before
        // internal_scale, as in the FP64 tables)
        std::vector<float> egf( in.egrid.size() ), xsf( 2 * in.egrid.size(), 0.0f );
        for ( std::size_t i = 0; i < in.egrid.size(); ++i ) {
          egf[i] = static_cast<float>( in.egrid[i] );
          xsf[2*i] = static_cast<float>( d.xs[i] );
          if ( i + 1 < in.egrid.size() )
            xsf[2*i+1] = static_cast<float>( ( d.xs[i+1] - d.xs[i] ) / ( in.egrid[i+1] - in.egrid[i] ) );
        }
        s.egrid_f = encodeOff<float>( mt->put( egf ) );
        s.xsf = encodeOff<float>( mt->put( xsf ) );
        // bucket index of the energy grid (eight buckets per octave of the
        // IEEE representation): the GPU's grid searches start at the bucket
        // and scan a few entries, with the same result as a binary search
        {
          auto key64 = []( double x ) { int64_t b; std::memcpy( &b, &x, 8 ); return b >> 49; };
          auto key32 = []( float x ) { int32_t b; std::memcpy( &b, &x, 4 ); return b >> 20; };
          const std::size_t ne = in.egrid.size();
          const int64_t k0 = key64( in.egrid.front() ), k1 = key64( in.egrid.back() );
          std::vector<int32_t> bk( static_cast<std::size_t>( k1 - k0 + 2 ) );
          std::size_t i = 0;
          for ( int64_t k = k0; k <= k1 + 1; ++k ) {
            while ( i < ne && key64( in.egrid[i] ) < k )
              ++i;
            bk[k - k0] = static_cast<int32_t>( i );
          }
          s.ebkt = encodeOff<int32_t>( mt->put( bk ) );
          s.ebkt_kmin = k0;
          s.ebkt_n = static_cast<int32_t>( bk.size() - 1 );
          const int32_t f0 = key32( egf.front() ), f1 = key32( egf.back() );
          std::vector<int32_t> bf( static_cast<std::size_t>( f1 - f0 + 2 ) );
          i = 0;
          for ( int32_t k = f0; k <= f1 + 1; ++k ) {
            while ( i < ne && key32( egf[i] ) < k )
              ++i;
            bf[k - f0] = static_cast<int32_t>( i );
          }
          s.ebkt_f = encodeOff<int32_t>( mt->put( bf ) );
          s.ebkt_f_kmin = f0;
          s.ebkt_f_n = static_cast<int32_t>( bf.size() - 1 );
        }
        std::vector<ncgb_beta_bin> bbin( d.bx.size() );
        std::memset( bbin.data(), 0, bbin.size() * sizeof(ncgb_beta_bin) );
        for ( std::size_t ie = 0; ie < d.kind.size(); ++ie ) {
          if ( d.kind[ie] != 1 )
            continue;
          const int64_t off = d.offset[ie];
          for ( int64_t j = 0; j + 1 < d.nbeta[ie]; ++j ) {
            ncgb_beta_bin& bb = bbin[off + j];
            bb.x0 = d.bx[off + j];
            bb.x1 = d.bx[off + j + 1];
            bb.cdf0 = d.bcdf[off + j];
            bb.a = d.by[off + j];
            const double dd = d.by[off + j + 1] - bb.a;
            const double dx = bb.x1 - bb.x0;
            if ( bb.a != 0.0 ) {
              bb.k_e = dd / ( dx * bb.a * bb.a );
              bb.inv_a = 1.0 / bb.a;
            } else {
              bb.k_e = dd > 0.0 ? 2.0 * dx / dd : -1.0;
              bb.inv_a = 0.0;
            }
            bb.k_z = dd != 0.0 ? dx * bb.a / dd : 0.0;
          }
        }
        s.bbin = encodeOff<ncgb_beta_bin>( mt->put( bbin.data(), bbin.size() ) );
        const std::size_t na = in.alpha.size(), nb = in.beta.size();
        std::vector<ncgb_alpha_cell> acell( na * nb );
        std::memset( acell.data(), 0, acell.size() * sizeof(ncgb_alpha_cell) );
        const double qnan = std::numeric_limits<double>::quiet_NaN();
        for ( std::size_t ib = 0; ib < nb; ++ib ) {
          for ( std::size_t ai = 0; ai + 1 < na; ++ai ) {
            const std::size_t g = ib * na + ai;
            ncgb_alpha_cell& c = acell[g];
            const double dc = d.cumul[g+1] - d.cumul[g];
            c.inv_bin = dc > 0.0 ? 1.0 / dc : 0.0;
            c.slope = qnan;
            const double fa = in.sab[g], fb = in.sab[g+1];
            const double df = fb - fa;
            if ( fa * fb * df != 0.0 ) {
              const double L = d.logsab[g+1] - d.logsab[g];
              const double a = in.alpha[ai], b = in.alpha[ai+1];
              if ( ( a - b ) * L != 0.0 ) {
                c.ratio = df / fa;
                c.slope = ( b - a ) / L;
              }
            }
          }
        }
        s.acell = encodeOff<ncgb_alpha_cell>( mt->put( acell.data(), acell.size() ) );
        // FP32 copies of the alpha-sampling tables (mixed-precision mode)
        auto tof = []( const std::vector<double>& v ) {
          std::vector<float> f( v.size() );
          for ( std::size_t i = 0; i < v.size(); ++i )
            f[i] = static_cast<float>( v[i] );
          return f;
        };
        s.alpha_f = encodeOff<float>( mt->put( tof( in.alpha ) ) );
        s.sab_f = encodeOff<float>( mt->put( tof( in.sab ) ) );
        s.logsab_f = encodeOff<float>( mt->put( tof( d.logsab ) ) );
        s.cumul_f = encodeOff<float>( mt->put( tof( d.cumul ) ) );
        s.inv_dbeta_f = encodeOff<float>( mt->put( tof( inv_dbeta ) ) );
        std::vector<float> acf( 4 * acell.size(), 0.0f );
        for ( std::size_t g = 0; g < acell.size(); ++g ) {
          acf[4*g] = static_cast<float>( acell[g].inv_bin );
          acf[4*g+1] = static_cast<float>( acell[g].ratio );
          acf[4*g+2] = static_cast<float>( acell[g].slope );
        }
        s.acell_f = encodeOff<float>( mt->put( acf ) );
        std::vector<ncgb_alpha_info_f> inff( d.info.size() );
        std::memset( inff.data(), 0, inff.size() * sizeof(ncgb_alpha_info_f) );
        for ( std::size_t i = 0; i < d.info.size(); ++i ) {
          const ncgb_alpha_info& a = d.info[i];
          ncgb_alpha_info_f& f = inff[i];
          f.front_alpha = static_cast<float>( a.front_alpha );
          f.front_sval = static_cast<float>( a.front_sval );
          f.front_logsval = static_cast<float>( a.front_logsval );
          f.back_alpha = static_cast<float>( a.back_alpha );
          f.back_sval = static_cast<float>( a.back_sval );
          f.back_logsval = static_cast<float>( a.back_logsval );
          f.prob_front = static_cast<float>( a.prob_front );
          f.prob_notback = static_cast<float>( a.prob_notback );
          f.inv_front = static_cast<float>( a.inv_front );
          f.inv_middle = static_cast<float>( a.inv_middle );
          f.inv_back = static_cast<float>( a.inv_back );
          f.front_idx = a.front_idx;
          f.back_idx = a.back_idx;
        }
        s.info_f = encodeOff<ncgb_alpha_info_f>( mt->put( inff.data(), inff.size() ) );
      } else if ( type == "FreeGas" ) {
        c.type = NCGB_COMP_FREEGAS;
        c.fg.kT = b.f64s(p+"kT");
        c.fg.mass_amu = b.f64s(p+"mass_amu");
        c.fg.sigma_free = b.f64s(p+"sigma_free");
        c.fg.ca = b.f64s(p+"ca");
      } else {
        throw Error("unsupported component type in material bundle: " + type);
      }
    }
    // erfc table of the free-gas sampler's bounds (NCFreeGasUtils.cc:95-122,
    // linspace as NCMath.cc:68-81), with the host's erfc like the reference.
    {
      const int len = 1103;
      std::vector<double> t( len );
      const double lo = -2.0, hi = 9.0;
      const unsigned num = len - 2, nm1 = num - 1;
      const double interval = ( hi - lo ) / nm1;
      t[0] = 2.0;
      for ( unsigned i = 0; i < nm1; ++i )
        t[1 + i] = std::erfc( lo + i * interval );
      t[num] = std::erfc( hi );
      t[len - 1] = 0.0;
      v.fg_erfc_table = encodeOff<double>( mt->put( t ) );
    }
    // Pad the arena so that it can be uploaded in 256-byte units.
    mt->m_arena.resize( ( mt->m_arena.size() + 255 ) & ~std::size_t(255) );
    return mt;
  }

  template int64_t MaterialTables::put<ncgb_alpha_info>( const ncgb_alpha_info*, std::size_t );
  template int64_t MaterialTables::put<ncgb_beta_bin>( const ncgb_beta_bin*, std::size_t );
  template int64_t MaterialTables::put<ncgb_alpha_cell>( const ncgb_alpha_cell*, std::size_t );

  ncgb_material_view MaterialTables::relocate( const void* basev ) const
  {
    const char* base = static_cast<const char*>( basev );
    ncgb_material_view v = m_rel;
    v.fg_erfc_table = reloc( v.fg_erfc_table, base );
    for ( int ic = 0; ic < v.ncomp; ++ic ) {
      ncgb_comp_view& c = v.comp[ic];
      c.bragg.two_dE = reloc( c.bragg.two_dE, base );
      c.bragg.fdm_commul = reloc( c.bragg.fdm_commul, base );
      ncgb_sab_view& s = c.sab;
      s.egrid = reloc( s.egrid, base );
      s.xs = reloc( s.xs, base );
      s.alpha = reloc( s.alpha, base );
      s.beta = reloc( s.beta, base );
      s.sab = reloc( s.sab, base );
      s.logsab = reloc( s.logsab, base );
      s.cumul = reloc( s.cumul, base );
      s.smp_kind = reloc( s.smp_kind, base );
      s.smp_ibetaoffset = reloc( s.smp_ibetaoffset, base );
      s.smp_nbeta = reloc( s.smp_nbeta, base );
      s.smp_offset = reloc( s.smp_offset, base );
      s.smp_fbkep = reloc( s.smp_fbkep, base );
      s.bx = reloc( s.bx, base );
      s.by = reloc( s.by, base );
      s.bcdf = reloc( s.bcdf, base );
      s.info = reloc( s.info, base );
      s.inv_dE = reloc( s.inv_dE, base );
      s.egrid_f = reloc( s.egrid_f, base );
      s.ebkt = reloc( s.ebkt, base );
      s.ebkt_f = reloc( s.ebkt_f, base );
      s.xsf = reloc( s.xsf, base );
      s.inv_dbeta = reloc( s.inv_dbeta, base );
      s.bbin = reloc( s.bbin, base );
      s.acell = reloc( s.acell, base );
      s.alpha_f = reloc( s.alpha_f, base );
      s.sab_f = reloc( s.sab_f, base );
      s.logsab_f = reloc( s.logsab_f, base );
      s.cumul_f = reloc( s.cumul_f, base );
      s.acell_f = reloc( s.acell_f, base );
      s.inv_dbeta_f = reloc( s.inv_dbeta_f, base );
      s.info_f = reloc( s.info_f, base );
    }
    return v;
  }
}
