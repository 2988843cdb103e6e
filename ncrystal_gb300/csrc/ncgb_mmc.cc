// Host side of the device MiniMC: cfg-string parsing (geometry, source,
// engine, scenario), the step loop over the resident neutron population, and
// the results in the reference's JSON layout (NCrystalMiniMCResults_v1,
// NCMMC_RunSim.cc:105-180).  Entry points: ncrystal_jsonquery for
// ["mmc","run",...] and ["mmc","scenario",...] queries (ncrystal.cc:2463-2473,
// NCMMC_Query.cc:60-157) and ncgb_mmc_run for a scatter handle.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "ncrystal_gb300.h"
#include "ncgb_launch.hh"
#include "ncgb_mmc.hh"

namespace ncgb {
  void handleInfo( ncrystal_scatter_t sc, const char* fct, mmc::HandleInfo* out );
  void reportError( const std::exception& e );
  void reportError( const char* type, const std::string& msg );
}

namespace {

  using namespace ncgb::mmc;

  constexpr double kWl2Ekin = 0.081804209605330899;   // E[eV] = kWl2Ekin / wl[Aa]^2 (NCDefs.hh:826-848)
  constexpr double kBoltzmann = 8.6173303e-5;         // eV/K (NCDefs.hh:79)
  constexpr double kPi = 3.14159265358979323846;
  constexpr double kEkin2Ksq = 4.0 * kPi * kPi / kWl2Ekin;

  struct MmcError : std::runtime_error {
    std::string type;
    MmcError( const std::string& t, const std::string& m ) : std::runtime_error( m ), type( t ) {}
  };
  [[noreturn]] void bad( const std::string& m ) { throw MmcError( "BadInput", m ); }

  void checkCuda( cudaError_t e, const char* what )
  {
    if ( e != cudaSuccess )
      throw MmcError( "CalcError", std::string( "CUDA error in " ) + what + ": " + cudaGetErrorString( e ) );
  }

  // ---- strings -------------------------------------------------------------------

  std::string trim( const std::string& s )
  {
    std::size_t a = 0, b = s.size();
    while ( a < b && std::isspace( (unsigned char)s[a] ) ) ++a;
    while ( b > a && std::isspace( (unsigned char)s[b - 1] ) ) --b;
    return s.substr( a, b - a );
  }

  std::vector<std::string> splitTrimmedNoEmpty( const std::string& s, const char* seps )
  {
    std::vector<std::string> out;
    std::string cur;
    auto flush = [&]() {
      std::string t = trim( cur );
      if ( !t.empty() )
        out.push_back( t );
      cur.clear();
    };
    for ( char c : s ) {
      if ( std::strchr( seps, c ) )
        flush();
      else
        cur.push_back( c );
    }
    flush();
    return out;
  }

  bool toDbl( const std::string& s, double& v )
  {
    const std::string t = trim( s );
    if ( t.empty() )
      return false;
    char* end = nullptr;
    v = std::strtod( t.c_str(), &end );
    return end && *end == '\0';
  }

  // Shortest text that reads back as the same double (NCFmt.cc:170-260).
  std::string fmt( double v )
  {
    if ( std::isnan( v ) )
      return "nan";
    if ( std::isinf( v ) )
      return v > 0 ? "inf" : "-inf";
    if ( v == 0.0 )
      return "0";
    char buf[64];
    int prec = 1;
    for ( ; prec <= 17; ++prec ) {
      std::snprintf( buf, sizeof(buf), "%.*g", prec, v );
      if ( std::strtod( buf, nullptr ) == v )
        break;
    }
    // plain digits rather than an exponent where the value allows it (60, not 6e+01)
    const double a = std::fabs( v );
    if ( std::strchr( buf, 'e' ) && a >= 1e-4 && a < 1e15 ) {
      const int intdigits = a >= 1.0 ? 1 + (int)std::floor( std::log10( a ) ) : 1;
      for ( int p = std::max( prec, intdigits ); p <= 17; ++p ) {
        char b2[64];
        std::snprintf( b2, sizeof(b2), "%.*g", p, v );
        if ( !std::strchr( b2, 'e' ) && std::strtod( b2, nullptr ) == v ) {
          std::memcpy( buf, b2, sizeof(b2) );
          break;
        }
      }
    }
    return buf;
  }

  double round6( double v )
  {
    char buf[64];
    std::snprintf( buf, sizeof(buf), "%.6g", v );
    return std::strtod( buf, nullptr );
  }

  // fmtUInt64AsNiceDbl, NCString.cc:559-590
  std::string fmtCount( uint64_t n )
  {
    if ( n >= 1000 ) {
      uint64_t k = 3, tentok = 1000, best_k = 0, best_tentok = 0;
      const uint64_t ndiv10 = n / 10;
      while ( true ) {
        if ( n % tentok == 0 ) {
          best_k = k;
          best_tentok = tentok;
        }
        if ( tentok > ndiv10 )
          break;
        k += 1;
        tentok *= 10;
      }
      if ( best_k )
        return std::to_string( n / best_tentok ) + "e" + std::to_string( best_k );
    }
    return std::to_string( n );
  }

  std::string jsonStr( const std::string& s )
  {
    std::string o = "\"";
    for ( char c : s ) {
      if ( c == '"' || c == '\\' ) { o.push_back( '\\' ); o.push_back( c ); }
      else if ( (unsigned char)c < 0x20 ) { char b[8]; std::snprintf( b, sizeof(b), "\\u%04x", c ); o += b; }
      else o.push_back( c );
    }
    return o + "\"";
  }

  std::string jsonNum( double v )
  {
    if ( !std::isfinite( v ) )
      return "null";
    char buf[64];
    std::snprintf( buf, sizeof(buf), "%.17g", v );
    // shortest exact form keeps the files readable
    const std::string s = fmt( v );
    double back = 0;
    return ( toDbl( s, back ) && back == v && s.find_first_not_of( "0123456789.-+e" ) == std::string::npos ) ? s : buf;
  }

  // ---- cfg tokens (NCMMC_ParseCfg.hh:38-170) ------------------------------------------
  struct Token { std::string key; bool has; std::string val; };
  struct TokenInfo { bool has_name = false; std::string name; std::vector<Token> tokens; };

  TokenInfo tokenize( const std::string& s )
  {
    TokenInfo r;
    bool first = true;
    for ( auto& e : splitTrimmedNoEmpty( s, ";" ) ) {
      const auto ieq = e.find( '=' );
      Token t;
      if ( ieq == std::string::npos ) {
        t.key = e;
        t.has = false;
      } else {
        t.key = trim( e.substr( 0, ieq ) );
        t.val = trim( e.substr( ieq + 1 ) );
        t.has = true;
      }
      if ( first ) {
        first = false;
        if ( !t.has ) {
          r.has_name = true;
          r.name = t.key;
          continue;
        }
      }
      bool handled = false;
      for ( auto& x : r.tokens )
        if ( x.key == t.key ) { x = t; handled = true; break; }
      if ( !handled )
        r.tokens.push_back( t );
    }
    return r;
  }

  void applyDefaults( std::vector<Token>& toks, const std::string& defs )
  {
    const std::size_t n = toks.size();
    for ( auto& d : tokenize( defs ).tokens ) {
      bool found = false;
      for ( std::size_t i = 0; i < n; ++i )
        if ( toks[i].key == d.key ) { found = true; break; }
      if ( !found )
        toks.push_back( d );
    }
  }

  void checkNoUnknown( const std::vector<Token>& toks, const std::string& accepted, const char* what )
  {
    const auto acc = splitTrimmedNoEmpty( accepted, ";" );
    for ( auto& t : toks )
      if ( std::find( acc.begin(), acc.end(), t.key ) == acc.end() )
        bad( std::string( "Invalid parameter for chosen " ) + what + ": \"" + t.key + "\"" );
  }

  const Token* find( const std::vector<Token>& toks, const std::string& k )
  {
    for ( auto& t : toks )
      if ( t.key == k )
        return &t;
    return nullptr;
  }

  std::string getStr( const std::vector<Token>& toks, const std::string& k )
  {
    const Token* t = find( toks, k );
    if ( !t )
      bad( "Missing required parameter \"" + k + "\"" );
    if ( !t->has || t->val.empty() )
      bad( "Missing value for parameter \"" + k + "\"" );
    return t->val;
  }

  std::string getStrAllowEmpty( const std::vector<Token>& toks, const std::string& k )
  {
    const Token* t = find( toks, k );
    return ( t && t->has ) ? t->val : std::string();
  }

  double getDbl( const std::vector<Token>& toks, const std::string& k )
  {
    double v = 0;
    if ( !toDbl( getStr( toks, k ), v ) || !std::isfinite( v ) )
      bad( "Invalid value for parameter \"" + k + "\"" );
    return v;
  }

  uint64_t getCount( const std::vector<Token>& toks, const std::string& k )
  {
    const double x = getDbl( toks, k );
    if ( !( x >= 0.0 && x < 1.8e19 ) || (double)(uint64_t)x != x )
      bad( "Invalid value for parameter \"" + k + "\"" );
    return (uint64_t)x;
  }

  bool getBool( const std::vector<Token>& toks, const std::string& k )
  {
    const std::string v = getStr( toks, k );
    if ( v == "0" )
      return false;
    if ( v != "1" )
      bad( "Invalid value for parameter \"" + k + "\"" );
    return true;
  }

  std::string lengthDescr( double m )
  {
    // fmtBestUnit-like: a unit that gives a plain number
    const double a = std::fabs( m );
    if ( a >= 1.0 ) return fmt( m ) + "m";
    if ( a >= 1e-2 ) return fmt( round6( m * 1e2 ) ) + "cm";
    if ( a >= 1e-3 ) return fmt( round6( m * 1e3 ) ) + "mm";
    if ( a >= 1e-6 ) return fmt( round6( m * 1e6 ) ) + "um";
    return fmt( round6( m * 1e9 ) ) + "nm";
  }

  // ---- geometry (NCMMC_Geom.cc:92-130) -------------------------------------------------
  struct GeomCfg {
    Geom g;
    std::string cfgstr, decoded, descr;
  };

  bool pointInside( const Geom& g, double x, double y, double z )
  {
    switch ( g.kind ) {
      case GEOM_SPHERE: return x * x + y * y + z * z <= g.r * g.r;
      case GEOM_BOX: return std::fabs( x ) <= g.dx && std::fabs( y ) <= g.dy && std::fabs( z ) <= g.dz;
      case GEOM_SLAB: return std::fabs( z ) <= g.dz;
      default: return x * x + z * z <= g.r * g.r && ( g.dy == 0.0 || std::fabs( y ) <= g.dy );
    }
  }

  GeomCfg parseGeom( const std::string& raw )
  {
    TokenInfo ti = tokenize( raw );
    if ( !ti.has_name )
      bad( "Invalid geom cfg: \"" + raw + "\"" );
    GeomCfg r;
    std::memset( &r.g, 0, sizeof(r.g) );
    auto& tk = ti.tokens;
    auto pos = [&]( const char* k ) {
      const double v = getDbl( tk, k );
      if ( !( v > 0.0 ) || !( v < 1e99 ) )
        bad( std::string( "Invalid value for parameter \"" ) + k + "\" (must be positive)" );
      return v;
    };
    std::ostringstream dec;
    if ( ti.name == "sphere" ) {
      applyDefaults( tk, "r=0.01" );
      checkNoUnknown( tk, "r", "geometry" );
      r.g.kind = GEOM_SPHERE;
      r.g.r = pos( "r" );
      r.cfgstr = "sphere;r=" + fmt( r.g.r );
      r.descr = "sphere with radius " + lengthDescr( r.g.r );
      dec << "\"name\":\"sphere\",\"r\":" << jsonNum( r.g.r );
    } else if ( ti.name == "cyl" ) {
      applyDefaults( tk, "r=0.01;dy=0" );
      checkNoUnknown( tk, "r;dy", "geometry" );
      r.g.kind = GEOM_CYL;
      r.g.r = pos( "r" );
      r.g.dy = getDbl( tk, "dy" );
      if ( !( r.g.dy >= 0.0 ) )
        bad( "Invalid value for parameter \"dy\" (must be non-negative)" );
      r.g.unbounded = r.g.dy == 0.0;
      r.cfgstr = "cyl;r=" + fmt( r.g.r ) + ( r.g.dy > 0.0 ? ";dy=" + fmt( r.g.dy ) : std::string() );
      r.descr = ( r.g.dy > 0.0 ? "cylinder with length " + lengthDescr( 2 * r.g.dy ) + " and radius "
                               : std::string( "infinite cylinder with radius " ) ) + lengthDescr( r.g.r );
      dec << "\"name\":\"cyl\",\"r\":" << jsonNum( r.g.r ) << ",\"dy\":" << jsonNum( r.g.dy );
    } else if ( ti.name == "slab" ) {
      applyDefaults( tk, "dz=0.01" );
      checkNoUnknown( tk, "dz", "geometry" );
      r.g.kind = GEOM_SLAB;
      r.g.dz = pos( "dz" );
      r.g.unbounded = 1;
      r.cfgstr = "slab;dz=" + fmt( r.g.dz );
      r.descr = "infinite slab with thickness " + lengthDescr( 2 * r.g.dz );
      dec << "\"name\":\"slab\",\"dz\":" << jsonNum( r.g.dz );
    } else if ( ti.name == "box" ) {
      applyDefaults( tk, "dx=0.01;dy=0.01;dz=0.01" );
      checkNoUnknown( tk, "dx;dy;dz", "geometry" );
      r.g.kind = GEOM_BOX;
      r.g.dx = pos( "dx" );
      r.g.dy = pos( "dy" );
      r.g.dz = pos( "dz" );
      r.cfgstr = "box;dx=" + fmt( r.g.dx ) + ";dy=" + fmt( r.g.dy ) + ";dz=" + fmt( r.g.dz );
      r.descr = "box with depth " + lengthDescr( 2 * r.g.dz ) + ", width " + lengthDescr( 2 * r.g.dx )
                + ", and height " + lengthDescr( 2 * r.g.dy );
      dec << "\"name\":\"box\",\"dx\":" << jsonNum( r.g.dx ) << ",\"dy\":" << jsonNum( r.g.dy )
          << ",\"dz\":" << jsonNum( r.g.dz );
    } else {
      bad( "Unknown geometry type requested: \"" + ti.name + "\"" );
    }
    r.decoded = dec.str();
    return r;
  }

  // ---- source (NCMMC_Source.cc:801-870, NCMMC_ParseCfg.hh:175-431) ------------------------
  struct SrcCfg {
    Source s;
    uint64_t n = 0;
    std::string cfgstr, decoded, edescr, ecfg;
    bool fixed_dir = false, mean_dir = false;
    double dir[3] = { 0, 0, 1 };
    bool fixed_e = false, mean_e = false;
    double e_fixed = 0, e_mean = 0;
    bool has_erange = false;
    double e_lo = 0, e_hi = 0;
  };

  void parseEnergy( const std::vector<Token>& tk, SrcCfg& r )
  {
    const Token* te = find( tk, "ekin" );
    const Token* tw = find( tk, "wl" );
    std::string sv;
    bool is_wl = false;
    if ( te && tw )
      bad( "Do not set both \"ekin\" and \"wl\" parameters." );
    if ( te ) { sv = te->has ? te->val : std::string(); }
    else if ( tw ) { sv = tw->has ? tw->val : std::string(); is_wl = true; }
    else { sv = "1.8"; is_wl = true; }
    const char* help = "Examples for how to set: \"ekin=0.025\" (fixed in eV), \"wl=1.8\" (fixed in Aa),"
                       " \"ekin=0.025-0.05\" (uniform range in eV), \"wl=1.8-5\" (uniform range in Aa),"
                       " \"ekin=0.025+-0.001\" (log-normal of given mean and rms in eV), \"wl=1.8+-0.01\""
                       " (log-normal of given mean and rms in Aa), \"ekin=thermal:77\" (thermal Maxwell of"
                       " given temperature in K).";
    const char* key = is_wl ? "wl" : "ekin";
    auto badval = [&]() { bad( "Invalid value \"" + sv + "\" for parameter \"" + key + "\". " + help ); };
    Source& s = r.s;
    s.e_is_wl = is_wl;
    const std::string unit = is_wl ? "Aa" : "eV";
    if ( sv.rfind( "thermal", 0 ) == 0 ) {
      if ( is_wl )
        bad( "For a Maxwell distribution, do not use the \"wl\" parameter (use \"ekin\" instead, like"
             " \"ekin=thermal:300K\")." );
      std::string rest = trim( sv.substr( 7 ) );
      double T = 0;
      if ( !( rest.size() >= 2 && rest.front() == ':' && rest.back() == 'K'
              && toDbl( rest.substr( 1, rest.size() - 2 ), T ) && T > 1e-99 && T < 1e99 ) )
        bad( "Invalid format for Maxwell distribution. Use a format like \"ekin=thermal:300K\"." );
      const double kT = T * kBoltzmann;
      s.ekind = E_MAXWELL;
      s.ea = 0.5 * kT;
      r.edescr = "Maxwell(" + fmt( T ) + "K)";
      r.ecfg = "ekin=thermal:" + fmt( T ) + "K";
      r.mean_e = true;
      r.e_mean = 1.5 * kT;
      r.has_erange = true;
      r.e_lo = 0.014854902715992444 * kT;   // NCMMC_Source.cc:152-165
      r.e_hi = 7.815281749225022 * kT;
      return;
    }
    if ( sv.empty() || sv == "help" )
      badval();
    // "<v>" fixed, "<a>-<b>" uniform (a '-' not after an 'e'), "<m>+-<s>" log-normal
    std::string a_s, b_s;
    int mode = 0;
    const auto ipm = sv.find( "+-" );
    if ( ipm != std::string::npos ) {
      mode = 2;
      a_s = sv.substr( 0, ipm );
      b_s = sv.substr( ipm + 2 );
    } else {
      for ( std::size_t i = 1; i < sv.size(); ++i ) {
        if ( sv[i] == '-' && !( sv[i - 1] == 'e' || sv[i - 1] == 'E' ) ) {
          mode = 1;
          a_s = sv.substr( 0, i );
          b_s = sv.substr( i + 1 );
          break;
        }
      }
    }
    auto posval = [&]( const std::string& t ) {
      double v = 0;
      if ( !toDbl( t, v ) || !std::isfinite( v ) || !( v > 0 ) )
        badval();
      return v;
    };
    if ( mode == 0 ) {
      const double v = posval( sv );
      s.ekind = E_FIXED;
      s.ea = is_wl ? kWl2Ekin / ( v * v ) : v;
      r.fixed_e = r.mean_e = true;
      r.e_fixed = r.e_mean = s.ea;
      r.has_erange = true;
      r.e_lo = r.e_hi = s.ea;
      r.edescr = fmt( v ) + unit;
      r.ecfg = std::string( key ) + "=" + fmt( v );
      return;
    }
    const double a = posval( a_s ), b = posval( b_s );
    r.mean_e = true;
    r.has_erange = true;
    double lo, hi, meanval;
    if ( mode == 1 ) {
      if ( !( a < b ) )
        badval();
      s.ekind = E_UNIFORM;
      s.ea = a;
      s.eb = b;
      meanval = 0.5 * ( a + b );
      lo = a;
      hi = b;
      r.edescr = "(" + fmt( a ) + "-" + fmt( b ) + ")" + unit;
      r.ecfg = std::string( key ) + "=" + fmt( a ) + "-" + fmt( b );
    } else {
      const double tmp = 1.0 + ( b * b ) / ( a * a );
      s.ekind = E_LOGNORMAL;
      s.ea = std::log( a / std::sqrt( tmp ) );
      s.eb = std::sqrt( std::log( tmp ) );
      meanval = a;
      lo = std::exp( s.ea - 3.0 * s.eb );
      hi = std::exp( s.ea + 3.0 * s.eb );
      r.edescr = "(" + fmt( a ) + "+-" + fmt( b ) + ")" + unit;
      r.ecfg = std::string( key ) + "=" + fmt( a ) + "+-" + fmt( b );
    }
    if ( is_wl ) {
      r.e_mean = kWl2Ekin / ( meanval * meanval );
      r.e_lo = kWl2Ekin / ( hi * hi );
      r.e_hi = kWl2Ekin / ( lo * lo );
    } else {
      r.e_mean = meanval;
      r.e_lo = lo;
      r.e_hi = hi;
    }
  }

  SrcCfg parseSource( const std::string& raw, const Geom& g )
  {
    TokenInfo ti = tokenize( raw );
    if ( !ti.has_name )
      bad( "Invalid src cfg: \"" + raw + "\"" );
    SrcCfg r;
    std::memset( &r.s, 0, sizeof(r.s) );
    auto& tk = ti.tokens;
    parseEnergy( tk, r );
    Source& s = r.s;
    std::ostringstream dec;
    auto dirOf = [&]() {
      const double ux = getDbl( tk, "ux" ), uy = getDbl( tk, "uy" ), uz = getDbl( tk, "uz" );
      const double m = std::sqrt( ux * ux + uy * uy + uz * uz );
      if ( !( m > 0 ) )
        bad( "Invalid direction (must be a non-zero vector)" );
      s.ux = ux / m; s.uy = uy / m; s.uz = uz / m;
      r.fixed_dir = r.mean_dir = true;
      r.dir[0] = s.ux; r.dir[1] = s.uy; r.dir[2] = s.uz;
    };
    auto xyz = [&]() { s.x = getDbl( tk, "x" ); s.y = getDbl( tk, "y" ); s.z = getDbl( tk, "z" ); };
    auto dirStr = [&]() {
      if ( s.ux == 0.0 && s.uy == 0.0 && s.uz == 1.0 )
        return std::string();
      return ";ux=" + fmt( s.ux ) + ";uy=" + fmt( s.uy ) + ";uz=" + fmt( s.uz );
    };
    if ( ti.name == "constant" || ti.name == "circular" ) {
      const bool circ = ti.name == "circular";
      applyDefaults( tk, "n=1e6" );
      applyDefaults( tk, "x=0;y=0;z=0;ux=0;uy=0;uz=1;n=1e6" );
      checkNoUnknown( tk, circ ? "ekin;wl;n;w;;x;y;z;ux;uy;uz;r" : "ekin;wl;n;w;;x;y;z;ux;uy;uz", "source" );
      r.n = getCount( tk, "n" );
      xyz();
      dirOf();
      s.kind = circ ? SRC_CIRCULAR : SRC_CONSTANT;
      if ( circ ) {
        s.r = getDbl( tk, "r" );
        if ( !( s.r >= 0.0 ) )
          bad( "Invalid value for parameter \"r\"" );
        if ( s.r > 0.0 ) {
          // basis orthogonal to the beam (NCMMC_Source.cc:668-683)
          double a[3] = { 1, 0, 0 };
          const double d[3] = { s.ux, s.uy, s.uz };
          auto dot = [&]( const double* v ) { return v[0] * d[0] + v[1] * d[1] + v[2] * d[2]; };
          if ( dot( a ) > 0.8 ) { a[0] = 0; a[1] = 1; a[2] = 0; }
          if ( dot( a ) > 0.8 ) { a[0] = 0; a[1] = 0; a[2] = 1; }
          auto cross = []( const double* u, const double* v, double* o ) {
            o[0] = u[1] * v[2] - u[2] * v[1];
            o[1] = u[2] * v[0] - u[0] * v[2];
            o[2] = u[0] * v[1] - u[1] * v[0];
            const double m = std::sqrt( o[0] * o[0] + o[1] * o[1] + o[2] * o[2] );
            o[0] /= m; o[1] /= m; o[2] /= m;
          };
          double va[3], vb[3];
          cross( d, a, va );
          cross( d, va, vb );
          s.ax = va[0] * s.r; s.ay = va[1] * s.r; s.az = va[2] * s.r;
          s.bx = vb[0] * s.r; s.by = vb[1] * s.r; s.bz = vb[2] * s.r;
        }
        s.might_be_outside = s.r > 0.0 ? 1 : !pointInside( g, s.x, s.y, s.z );
      } else {
        s.might_be_outside = !pointInside( g, s.x, s.y, s.z );
      }
      std::ostringstream c;
      c << ti.name << ";n=" << fmtCount( r.n );
      if ( s.x != 0.0 ) c << ";x=" << fmt( s.x );
      if ( s.y != 0.0 ) c << ";y=" << fmt( s.y );
      if ( s.z != 0.0 ) c << ";z=" << fmt( s.z );
      c << ";" << r.ecfg << dirStr();
      if ( circ ) c << ";r=" << fmt( s.r );
      r.cfgstr = c.str();
      dec << "\"name\":" << jsonStr( ti.name ) << ",\"n\":" << r.n << ",\"x\":" << jsonNum( s.x )
          << ",\"y\":" << jsonNum( s.y ) << ",\"z\":" << jsonNum( s.z ) << ",\"w\":1.0,\"ux\":" << jsonNum( s.ux )
          << ",\"uy\":" << jsonNum( s.uy ) << ",\"uz\":" << jsonNum( s.uz );
      if ( circ ) dec << ",\"r\":" << jsonNum( s.r );
    } else if ( ti.name == "isotropic" ) {
      applyDefaults( tk, "n=1e6" );
      applyDefaults( tk, "x=0;y=0;z=0;r=0;n=1e6" );
      checkNoUnknown( tk, "ekin;wl;n;w;;x;y;z;r", "source" );
      r.n = getCount( tk, "n" );
      xyz();
      s.kind = SRC_ISOTROPIC;
      s.r = getDbl( tk, "r" );
      s.ux = 0; s.uy = 0; s.uz = 1;
      s.might_be_outside = !pointInside( g, s.x, s.y, s.z );
      std::ostringstream c;
      c << "isotropic;n=" << fmtCount( r.n );
      if ( s.x != 0.0 ) c << ";x=" << fmt( s.x );
      if ( s.y != 0.0 ) c << ";y=" << fmt( s.y );
      if ( s.z != 0.0 ) c << ";z=" << fmt( s.z );
      c << ";" << r.ecfg;
      if ( s.r != 0.0 ) c << ";r=" << fmt( s.r );
      r.cfgstr = c.str();
      dec << "\"name\":\"isotropic\",\"n\":" << r.n << ",\"x\":" << jsonNum( s.x ) << ",\"y\":" << jsonNum( s.y )
          << ",\"z\":" << jsonNum( s.z ) << ",\"w\":1.0,\"r\":" << jsonNum( s.r );
    } else {
      bad( "Unknown source type requested: \"" + ti.name + "\"" );
    }
    if ( r.n == 0 )
      bad( "Invalid value for parameter \"n\" (the device engine needs a finite, positive count)" );
    if ( r.n > 0xffffffffull )
      bad( "Invalid value for parameter \"n\" (at most 2^32-1 neutrons per run: the random streams are keyed"
           " by a 32-bit source index)" );
    r.decoded = dec.str();
    return r;
  }

  // ---- engine options (NCMMC_EngineOpts.cc:276-470) -------------------------------------------
  const char* const kTallyNames[T_N] = { "theta", "mu", "nscat", "nscat_uw", "w", "e", "l", "de", "q" };

  struct EngineCfg {
    uint64_t seed = 0;
    double psurv = 0.1, wthr = 0.01;
    int nscatthr = 2;
    bool ignore_miss = false, absorption = true, breakdown = true, tallyref_src = false;
    int nscatlimit = -1;
    std::string nthreads = "auto";
    bool enabled[T_N] = {};
    bool lowres = false, highres = false;
    bool has_override[T_N] = {};
    int ov_nbins[T_N] = {};
    double ov_lo[T_N] = {}, ov_hi[T_N] = {};
    std::string cfgstr, decoded;
  };

  int tallyIndex( const std::string& s )
  {
    for ( int k = 0; k < T_N; ++k )
      if ( s == kTallyNames[k] )
        return k;
    return -1;
  }

  EngineCfg parseEngine( const std::string& raw )
  {
    TokenInfo ti = tokenize( raw );
    if ( ti.has_name && ti.name != "std" )
      bad( "Invalid MiniMC engine \"" + ti.name + "\"" );
    auto& tk = ti.tokens;
    applyDefaults( tk, "ignoremiss=0;nthreads=auto;absorption=1;seed=0;nscatlimit=none;roulette=0.1,0.01,2;"
                       "tallyref=truth;tally=theta;tallybins=;tallybreakdown=1" );
    checkNoUnknown( tk, "seed;roulette;ignoremiss;nthreads;absorption;nscatlimit;tallyref;tally;tallybins;"
                        "tallybreakdown", "engine" );
    EngineCfg e;
    const std::string tr = getStr( tk, "tallyref" );
    if ( tr == "src" ) e.tallyref_src = true;
    else if ( tr != "truth" ) bad( "tallyref must be \"truth\" or \"src\"" );
    {
      const auto p = splitTrimmedNoEmpty( getStr( tk, "roulette" ), "," );
      double v[3] = { 0, 0, 0 };
      if ( p.size() != 3 || !toDbl( p[0], v[0] ) || !toDbl( p[1], v[1] ) || !toDbl( p[2], v[2] ) )
        bad( "Invalid roulette options: \"" + getStr( tk, "roulette" )
             + "\" (should be three comma separated values \"psurvival,weight_threshold,nscat_threshold\")" );
      if ( !( v[0] > 1e-20 ) ) bad( "roulette_survival_probability must be >1e-20" );
      if ( !( v[0] < 1.0 ) ) bad( "roulette_survival_probability must be <1.0" );
      if ( !( v[1] > 0.0 ) ) bad( "roulette_weight_threshold must be >0.0" );
      if ( !( v[2] >= 0.0 && v[2] < 2147483647.0 && (double)(int)v[2] == v[2] ) )
        bad( "Invalid roulette nscat threshold" );
      e.psurv = v[0];
      e.wthr = v[1];
      e.nscatthr = (int)v[2];
    }
    {
      const std::string s = getStr( tk, "seed" );
      char* end = nullptr;
      errno = 0;
      const unsigned long long v = std::strtoull( s.c_str(), &end, 10 );
      if ( s.empty() || !end || *end || errno || s[0] == '-' )
        bad( "Invalid seed \"" + s + "\"." );
      e.seed = v;
    }
    e.ignore_miss = getBool( tk, "ignoremiss" );
    e.absorption = getBool( tk, "absorption" );
    e.nthreads = getStr( tk, "nthreads" );
    if ( e.nthreads != "auto" ) {
      double v = 0;
      if ( !toDbl( e.nthreads, v ) || !( v >= 0 ) || (double)(uint64_t)v != v )
        bad( "Invalid value for parameter \"nthreads\"" );
    }
    if ( getStr( tk, "nscatlimit" ) != "none" ) {
      const uint64_t v = getCount( tk, "nscatlimit" );
      if ( v > 32000 )
        bad( "nscatlimit value must be at most 32000" );
      e.nscatlimit = (int)v;
    }
    for ( auto& name : splitTrimmedNoEmpty( getStrAllowEmpty( tk, "tally" ), "," ) ) {
      if ( name == "nobreakdown" )
        bad( "Invalid tally \"nobreakdown\" (use \"tallybreakdown=0\" to disable breakdowns)" );
      if ( name == "lowres" )
        bad( "Invalid tally \"lowres\" (use \"tallybins=-\" to decrease binnings)" );
      if ( name == "highres" )
        bad( "Invalid tally \"highres\" (use \"tallybins=+\" to increase binnings)" );
      const int k = tallyIndex( name );
      if ( k < 0 )
        bad( "Invalid tally \"" + name + "\"" );
      e.enabled[k] = true;
    }
    e.breakdown = getBool( tk, "tallybreakdown" );
    for ( auto& b : splitTrimmedNoEmpty( getStrAllowEmpty( tk, "tallybins" ), "," ) ) {
      if ( b == "+" ) { e.highres = true; continue; }
      if ( b == "-" ) { e.lowres = true; continue; }
      const auto parts = splitTrimmedNoEmpty( b, ":" );
      if ( parts.size() != 4 )
        bad( "Invalid enginecfg tallybins entry \"" + b + "\"." );
      const int k = tallyIndex( parts[0] );
      if ( k < 0 )
        bad( "Invalid enginecfg tallybins tally name \"" + parts[0] + "\"." );
      double nb = 0, lo = 0, hi = 0;
      if ( !toDbl( parts[1], nb ) || (double)(int)nb != nb || !toDbl( parts[2], lo ) || !toDbl( parts[3], hi ) )
        bad( "Invalid enginecfg tallybins entry \"" + b + "\" (should have the form \"tallyname:nbins:xmin:xmax\")." );
      if ( !( nb >= 1 && nb < 1e8 ) || !std::isfinite( lo ) || !std::isfinite( hi ) || !( lo < hi ) )
        bad( "Invalid enginecfg tallybins entry \"" + b + "\" (invalid binning)." );
      e.has_override[k] = true;
      e.ov_nbins[k] = (int)nb;
      e.ov_lo[k] = lo;
      e.ov_hi[k] = hi;
    }
    // normalised cfg-string and decoded values (defaults omitted, as the
    // reference's stream operator does)
    std::ostringstream c, d;
    std::vector<std::string> parts;
    if ( e.seed ) parts.push_back( "seed=" + std::to_string( e.seed ) );
    if ( e.nthreads != "auto" ) parts.push_back( "nthreads=" + e.nthreads );
    if ( e.ignore_miss ) parts.push_back( "ignoremiss=1" );
    if ( !e.absorption ) parts.push_back( "absorption=0" );
    if ( e.nscatlimit >= 0 ) parts.push_back( "nscatlimit=" + std::to_string( e.nscatlimit ) );
    if ( !( e.psurv == 0.1 && e.wthr == 0.01 && e.nscatthr == 2 ) )
      parts.push_back( "roulette=" + fmt( e.psurv ) + "," + fmt( e.wthr ) + "," + std::to_string( e.nscatthr ) );
    if ( e.tallyref_src ) parts.push_back( "tallyref=src" );
    std::vector<std::string> tl;
    for ( int k : { T_DE, T_E, T_L, T_MU, T_NSCAT, T_NSCAT_UW, T_Q, T_THETA, T_W } )
      if ( e.enabled[k] ) tl.push_back( kTallyNames[k] );
    {
      std::string ts;
      for ( auto& x : tl ) ts += ( ts.empty() ? "" : "," ) + x;
      if ( ts != "theta" ) parts.push_back( "tally=" + ts );
    }
    if ( !e.breakdown ) parts.push_back( "tallybreakdown=0" );
    {
      std::string bs;
      for ( int k = 0; k < T_N; ++k )
        if ( e.has_override[k] )
          bs += ( bs.empty() ? "" : "," ) + std::string( kTallyNames[k] ) + ":" + std::to_string( e.ov_nbins[k] ) + ":"
                + fmt( e.ov_lo[k] ) + ":" + fmt( e.ov_hi[k] );
      if ( e.highres ) bs += ( bs.empty() ? "" : "," ) + std::string( "+" );
      if ( e.lowres ) bs += ( bs.empty() ? "" : "," ) + std::string( "-" );
      if ( !bs.empty() ) parts.push_back( "tallybins=" + bs );
    }
    for ( std::size_t i = 0; i < parts.size(); ++i )
      c << ( i ? ";" : "" ) << parts[i];
    e.cfgstr = c.str();
    d << "\"seed\":" << e.seed << ",\"roulette\":{\"psurvival\":" << jsonNum( e.psurv ) << ",\"weight_threshold\":"
      << jsonNum( e.wthr ) << ",\"nscat_threshold\":" << e.nscatthr << "},\"ignoremiss\":"
      << ( e.ignore_miss ? "true" : "false" ) << ",\"absorption\":" << ( e.absorption ? "true" : "false" )
      << ",\"tallyref\":" << ( e.tallyref_src ? "\"src\"" : "\"truth\"" ) << ",\"nscatlimit\":"
      << ( e.nscatlimit >= 0 ? std::to_string( e.nscatlimit ) : std::string( "null" ) ) << ",\"tally\":[";
    for ( std::size_t i = 0; i < tl.size(); ++i )
      d << ( i ? "," : "" ) << jsonStr( tl[i] );
    d << "],\"tallybreakdown\":" << ( e.breakdown ? "true" : "false" ) << ",\"nthreads\":"
      << ( e.nthreads == "auto" ? std::string( "\"auto\"" ) : e.nthreads );
    e.decoded = d.str();
    return e;
  }

  // ---- tally set-up (TallyStdHists_Options::create, TallyStdHists_Data::create,
  //      NCMMC_StdTallies.cc:40-240) --------------------------------------------------
  Tally setupTally( const EngineCfg& e, const SrcCfg& src, double matTemp )
  {
    Tally t;
    std::memset( &t, 0, sizeof(t) );
    t.breakdown = e.breakdown;
    const bool needs_dir0 = e.enabled[T_Q] || e.enabled[T_MU] || e.enabled[T_THETA];
    const bool needs_e0 = e.enabled[T_Q] || e.enabled[T_DE];
    if ( needs_dir0 ) {
      const bool have = e.tallyref_src ? src.mean_dir : src.fixed_dir;
      if ( !have && e.tallyref_src ) {
        const char* name = e.enabled[T_Q] ? "q" : ( e.enabled[T_MU] ? "mu" : "theta" );
        bad( std::string( "tallyref=src but tally \"" ) + name
             + "\" needs a direction which is not well defined with the chosen source" );
      }
      if ( have ) {
        t.fixed_dir = 1;
        t.d0x = src.dir[0]; t.d0y = src.dir[1]; t.d0z = src.dir[2];
      }
    }
    if ( needs_e0 ) {
      const bool have = e.tallyref_src ? src.mean_e : src.fixed_e;
      if ( !have && e.tallyref_src ) {
        const char* name = e.enabled[T_Q] ? "q" : "de";
        bad( std::string( "tallyref=src but tally \"" ) + name
             + "\" needs a energy which is not well defined with the chosen source" );
      }
      if ( have ) {
        t.fixed_e = 1;
        t.e0 = e.tallyref_src ? src.e_mean : src.e_fixed;
      }
    }
    // automatic binnings of the energy-dependent tallies
    bool has_bin[T_N];
    int nb[T_N];
    double lo[T_N], hi[T_N];
    for ( int k = 0; k < T_N; ++k ) {
      has_bin[k] = e.has_override[k];
      nb[k] = e.ov_nbins[k];
      lo[k] = e.ov_lo[k];
      hi[k] = e.ov_hi[k];
    }
    {
      const double kT = ( matTemp > 0 ? matTemp : 293.15 ) * kBoltzmann;
      const double kTlow = 0.073 * kT, kThigh = 13.688 * kT;
      const double blo = src.has_erange ? src.e_lo : kTlow;
      const double bhi = src.has_erange ? src.e_hi : kThigh;
      const int n = 200;
      if ( e.enabled[T_E] && !has_bin[T_E] ) {
        const double a = std::min( blo, kTlow ), b = std::max( bhi, kThigh ), eps = 0.2 * ( b - a );
        has_bin[T_E] = true; nb[T_E] = n; lo[T_E] = std::max( 0.0, a - eps ); hi[T_E] = b + eps;
      }
      if ( e.enabled[T_L] && !has_bin[T_L] ) {
        double elow = std::min( blo, 0.5 * kTlow );
        const double ehigh = std::max( 0.0, std::max( bhi, 2 * kThigh ) );
        const double de = std::max( 1e-6, ehigh - elow );
        if ( !( elow > 0.0 ) )
          elow = de * 0.001;
        const double l_low = std::sqrt( kWl2Ekin / ehigh ) * 0.5;
        const double l_high = std::sqrt( kWl2Ekin / elow ) * 2;
        const double d_l = l_high - l_low;
        has_bin[T_L] = true; nb[T_L] = n; lo[T_L] = std::max( 0.0, l_low - 0.25 * d_l ); hi[T_L] = l_high + 0.25 * d_l;
      }
      if ( e.enabled[T_DE] && !has_bin[T_DE] ) {
        const double a = std::min( 0.0, blo - 2 * kThigh ), b = std::max( 0.0, bhi - 0.5 * kTlow );
        has_bin[T_DE] = true; nb[T_DE] = n; lo[T_DE] = a - 0.25 * ( b - a ); hi[T_DE] = b + 0.25 * ( b - a );
      }
      if ( e.enabled[T_Q] && !has_bin[T_Q] ) {
        has_bin[T_Q] = true; nb[T_Q] = n; lo[T_Q] = 0.0; hi[T_Q] = 2.1 * std::sqrt( ( bhi + kThigh ) * kEkin2Ksq );
      }
    }
    // default binnings (scaled by lowres/highres unless fixed)
    auto autob = [&]( int k, int nbins, double a, double b, bool fixnbins ) {
      if ( has_bin[k] )
        return;
      if ( !fixnbins ) {
        if ( e.lowres ) nbins /= 2;
        if ( e.highres ) nbins *= 10;
      }
      has_bin[k] = true; nb[k] = nbins; lo[k] = a; hi[k] = b;
    };
    autob( T_THETA, 180, 0.0, 180.0, false );
    autob( T_MU, 200, -1.0, 1.0, false );
    {
      int nscatmax = e.lowres ? 10 : 20;
      if ( e.highres ) nscatmax += 20;
      autob( T_NSCAT, nscatmax + 2, -1.5, nscatmax + 0.5, true );
      autob( T_NSCAT_UW, nscatmax + 2, -1.5, nscatmax + 0.5, true );
    }
    autob( T_W, 200, 0.0, 1.0, false );
    autob( T_E, 200, 0.0, 1.0, false );
    autob( T_L, 200, 0.0, 10.0, false );
    autob( T_DE, 200, -1.0, 1.0, false );
    autob( T_Q, 200, 0.0, 10.0, false );
    // statistics shifts: the tally values of an unscattered source neutron
    // (device arithmetic for l matches this expression bit for bit)
    {
      const double e0 = src.fixed_e ? src.e_fixed : ( src.mean_e ? src.e_mean : 0.0 );
      for ( int k = 0; k < T_N; ++k )
        t.shift[k] = 0.0;
      if ( src.fixed_dir )
        t.shift[T_MU] = 1.0;
      if ( e0 > 0.0 ) {
        t.shift[T_E] = e0;
        t.shift[T_L] = std::sqrt( kWl2Ekin ) * std::sqrt( 1.0 / e0 );
      }
    }
    int64_t off = 0;
    for ( int k = 0; k < T_N; ++k ) {
      TallyHist& h = t.h[k];
      h.enabled = e.enabled[k];
      if ( !h.enabled )
        continue;
      h.nbins = nb[k];
      h.xmin = lo[k];
      h.xmax = hi[k];
      h.inv_delta = nb[k] / ( hi[k] - lo[k] );
      h.soff = off;
      off += kGroups * kStats;
    }
    t.nstat = off;
    for ( int k = 0; k < T_N; ++k ) {
      TallyHist& h = t.h[k];
      if ( !h.enabled )
        continue;
      h.off = off;
      off += (int64_t)kGroups * ( h.nbins + 2 ) * 2;
    }
    t.nbuf = off;
    return t;
  }

  // ---- scenario (decodeScenario, NCMMC_Utils.cc:244-490) -------------------------------------
  struct Scenario { std::string geomcfg, srccfg; };

  bool unitSplit( const std::string& s0, double& v, std::string& unit )
  {
    const std::string s = trim( s0 );
    if ( toDbl( s, v ) ) { unit.clear(); return true; }
    std::size_t n = s.size();
    while ( n && ( std::isalpha( (unsigned char)s[n - 1] ) || s[n - 1] == '_' ) )
      --n;
    if ( !toDbl( s.substr( 0, n ), v ) )
      return false;
    unit = s.substr( n );
    return true;
  }

  Scenario decodeScenario( ncrystal_scatter_t sc, const HandleInfo& hi, const std::string& input )
  {
    for ( char c : input )
      if ( (unsigned char)c < 0x20 && !std::isspace( (unsigned char)c ) )
        bad( "Forbidden character in MiniMC scenario string: \"" + input + "\"" );
    auto parts = splitTrimmedNoEmpty( input, " \t\n\r:_" );
    std::size_t it = 0, itE = parts.size();
    uint64_t count = 0;
    if ( it != itE && parts[itE - 1] == "times" ) {
      --itE;
      if ( it == itE )
        bad( "Invalid MiniMC scenario string: \"" + input + "\". Expected integral value like \"10000\" or"
             " \"1e6\" in front of keyword \"times\"." );
      double c = 0;
      if ( !toDbl( parts[itE - 1], c ) || !( c > 0 && c <= 1e18 ) || (double)(uint64_t)( c + 0.5 ) != c )
        bad( "Invalid count specification \"" + parts[itE - 1] + "\". Count must be a positive integral value"
             " (and at most 1e18)." );
      count = (uint64_t)( c + 0.5 );
      --itE;
    }
    if ( it == itE ) {
      std::string def = hi.bragg_threshold > 0 ? "0.8BT" : ( hi.temperature > 0 ? "1kT" : "1.8Aa" );
      if ( count )
        def += " " + fmtCount( count ) + " times";
      return decodeScenario( sc, hi, def );
    }
    const std::string sv_energy = parts[it++];
    bool pencil = false;
    if ( it != itE && parts[it] == "pencil" ) { pencil = true; ++it; }
    const std::string count_formatted = count ? fmtCount( count ) : std::string( "1e6" );
    bool sphere = true;
    std::string sv_thickness = "1mfp";
    if ( it != itE ) {
      if ( parts[it] != "on" )
        bad( "Invalid MiniMC scenario string: \"" + input + "\". Expected keyword \"on\" but got \"" + parts[it]
             + "\"." );
      ++it;
      bool had = false;
      if ( it != itE ) {
        if ( parts[itE - 1] == "sphere" ) { --itE; had = true; }
        else if ( parts[itE - 1] == "slab" ) { --itE; had = true; sphere = false; }
      }
      if ( it == itE ) {
        if ( !had )
          bad( "Invalid MiniMC scenario string: \"" + input + "\". Missing parameters after keyword \"on\"." );
      } else {
        sv_thickness = parts[it++];
        if ( it != itE )
          bad( "Invalid MiniMC scenario string: \"" + input + "\". Unexpected parameter: \"" + parts[it] + "\"" );
      }
    }
    if ( !sphere )
      pencil = true;
    double ev = 0;
    std::string eu;
    if ( !unitSplit( sv_energy, ev, eu ) )
      bad( "Invalid energy specification in \"" + sv_energy + "\"." );
    double energy = 0, wl = 0;
    bool wlmode = false;
    if ( eu == "Aa" ) {
      wlmode = true; wl = ev; energy = kWl2Ekin / ( wl * wl );
    } else if ( eu == "eV" || eu == "meV" || eu == "keV" || eu == "MeV" || eu == "GeV" ) {
      const double f = eu == "eV" ? 1.0 : eu == "meV" ? 1e-3 : eu == "keV" ? 1e3 : eu == "MeV" ? 1e6 : 1e9;
      energy = ev * f;
    } else if ( eu == "kT" ) {
      if ( !( hi.temperature > 0 ) )
        bad( "Can not use kT as a unit for a multi-phase material without a single well-defined temperature." );
      energy = round6( ev * hi.temperature * kBoltzmann );
    } else if ( eu == "BT" ) {
      wlmode = true;
      wl = round6( ev * ( hi.bragg_threshold > 0 ? hi.bragg_threshold : 4.0 ) );
      energy = kWl2Ekin / ( wl * wl );
    } else {
      bad( std::string( eu.empty() ? "Missing" : "Invalid" ) + " energy unit on \"" + sv_energy + "\"."
           + " Possible units include Aa, meV, eV, kT (=kB*temperature), BT (=Bragg threshold in Aa, or 4Aa if not"
             " available)." );
    }
    double tv = 0;
    std::string tu;
    if ( !unitSplit( sv_thickness, tv, tu ) )
      bad( "Invalid thickness specification in \"" + sv_thickness + "\"." );
    if ( tu.empty() )
      bad( "Missing length unit on: \"" + sv_thickness + "\". Accepts either the special unit \"mfp\""
           " (mean-free-path between scatterings) or one of the standard length units: Aa, nm, mu, mm, cm, m" );
    double thick = -1.0;
    if ( tu == "mfp" ) {
      double xs = 0;
      ncrystal_crosssection_nonoriented( ncrystal_cast_scat2proc( sc ), energy, &xs );
      if ( ncrystal_error() )
        throw MmcError( "CalcError", "cross-section evaluation failed" );
      const double macroxs = 100.0 * hi.numdens * xs;
      thick = ( macroxs < 1e-99 || macroxs > 1e99 ) ? 0.01 : round6( tv / macroxs );
    } else {
      const double f = tu == "Aa" ? 1.0 : tu == "nm" ? 10.0 : tu == "mu" ? 1e4 : tu == "mm" ? 1e7
                     : tu == "cm" ? 1e8 : tu == "m" ? 1e10 : -1.0;
      if ( f < 0 )
        bad( "invalid length: \"" + sv_thickness + "\". Must be a value followed by either the special unit"
             " \"mfp\" (mean-free-path between scatterings) or one of the standard length units: Aa, nm, mu, mm,"
             " cm, m" );
      thick = tv * f * 1e-10;
    }
    if ( thick < 1e-120 || thick > 1e120 )
      bad( "Could not determine suitable thickness from \"" + sv_thickness
           + "\" (thickness is invalid or out of range)" );
    Scenario r;
    const double src_z = -0.5 * thick;
    std::ostringstream g, s;
    if ( sphere ) {
      g << "sphere;r=" << fmt( thick * 0.5 );
      if ( pencil ) s << "constant;z=" << fmt( src_z );
      else s << "circular;z=" << fmt( src_z ) << ";r=" << fmt( thick * 0.5 );
    } else {
      g << "slab;dz=" << fmt( thick * 0.5 );
      s << "constant;z=" << fmt( src_z );
    }
    if ( wlmode ) s << ";wl=" << fmt( wl );
    else s << ";ekin=" << fmt( energy );
    s << ";n=" << count_formatted;
    r.geomcfg = g.str();
    r.srccfg = s.str();
    return r;
  }

  // ---- device memory of a run --------------------------------------------------------
  struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if ( p ) cudaFree( p ); }
    template<class T> T* alloc( std::size_t n )
    {
      checkCuda( cudaMalloc( &p, std::max<std::size_t>( n * sizeof(T), 256 ) ), "cudaMalloc (MiniMC)" );
      return static_cast<T*>( p );
    }
  };

  struct PopBufs {
    DevBuf b[13];
    Pop pop;
    void alloc( std::size_t cap )
    {
      pop.pos = b[0].alloc<double>( 3 * cap );
      pop.dir = b[1].alloc<double>( 3 * cap );
      pop.e = b[2].alloc<double>( cap );
      pop.w = b[3].alloc<double>( cap );
      pop.xs = b[4].alloc<double>( cap );
      pop.nscat = b[5].alloc<int32_t>( cap );
      pop.ninel = b[6].alloc<int32_t>( cap );
      pop.id = b[7].alloc<uint32_t>( cap );
      pop.e0 = b[8].alloc<double>( cap );
      pop.d0 = b[9].alloc<double>( 3 * cap );
      pop.e_new = b[10].alloc<double>( cap );
      pop.dir_new = b[11].alloc<double>( 3 * cap );
      pop.st = b[12].alloc<int32_t>( cap );
    }
  };

  struct StreamGuard {
    cudaStream_t s = nullptr;
    ~StreamGuard() { if ( s ) cudaStreamDestroy( s ); }
  };

  struct RunResult {
    std::vector<double> tally;
    Counters c;
    uint64_t steps = 0;
    double seconds = 0;
    // with phase timing on (ncgb_phase_timing): transport kernel time and
    // launches (the scatter kernels' times go to ncgb_phase_times)
    double transport_ms = 0;
    uint64_t transport_launches = 0;
    uint64_t neutron_steps = 0;     // transported neutrons summed over steps
  };

  void formTotals( const Tally& t, std::vector<double>& buf );

  // The step loop (StdSimEngine::step / SimMgr, NCMMC_SimEngine.cc:151-165).
  RunResult runEngine( const HandleInfo& hi, const GeomCfg& gc, const SrcCfg& sc, const EngineCfg& ec, Tally t,
                       uint64_t capacity )
  {
    int dev = 0;
    checkCuda( cudaGetDevice( &dev ), "cudaGetDevice" );
    if ( dev != hi.device )
      checkCuda( cudaSetDevice( hi.device ), "cudaSetDevice" );
    int nsm = 0;
    checkCuda( cudaDeviceGetAttribute( &nsm, cudaDevAttrMultiProcessorCount, hi.device ), "device attribute" );
    Engine eng;
    std::memset( &eng, 0, sizeof(eng) );
    eng.macro = 100.0 * hi.numdens;
    eng.has_abs = ec.absorption && hi.abs_c > 0.0 && eng.macro > 0.0;
    eng.abs_c = eng.has_abs ? hi.abs_c : 0.0;
    eng.has_scat = eng.macro > 0.0 && hi.view.ncomp > 0;
    eng.psurv = ec.psurv;
    eng.wthr = ec.wthr;
    eng.boost = 1.0 / ec.psurv;
    eng.nscatthr = ec.nscatthr;
    eng.nscatlimit = ec.nscatlimit;
    eng.fast = hi.mode == NCGB_MODE_MIXED;
    eng.ignore_miss = ec.ignore_miss;
    eng.seed = ec.seed ^ 0x6d696e696d63ull;   // the engine's streams differ from the scatter handle's
    if ( !( hi.numdens >= 0.0 ) )
      throw MmcError( "BadInput", "the material bundle carries no number density (re-export it)" );
    if ( ec.absorption && !( hi.abs_c >= 0.0 ) )
      throw MmcError( "BadInput", "the material bundle carries no absorption data (re-export it, or absorption=0)" );

    const uint64_t cap = std::max<uint64_t>( 1, std::min<uint64_t>( capacity, sc.n ) );
    PopBufs pa, pb;
    pa.alloc( cap );
    pb.alloc( cap );
    DevBuf tb, cb, wb, qb;
    t.buf = tb.alloc<double>( t.nbuf );
    {
      // empty statistics: min key +max, max key -max
      std::vector<double> init( t.nbuf, 0.0 );
      for ( int k = 0; k < T_N; ++k ) {
        if ( !t.h[k].enabled )
          continue;
        for ( int g = 0; g < kGroups; ++g ) {
          long long mn = 0x7FFFFFFFFFFFFFFFLL, mx = (long long)0x8000000000000000ULL;
          std::memcpy( &init[t.h[k].soff + g * kStats + 3], &mn, 8 );
          std::memcpy( &init[t.h[k].soff + g * kStats + 4], &mx, 8 );
        }
      }
      checkCuda( cudaMemcpy( t.buf, init.data(), t.nbuf * sizeof(double), cudaMemcpyHostToDevice ), "H2D" );
    }
    Counters* dc = cb.alloc<Counters>( 1 );
    checkCuda( cudaMemset( dc, 0, sizeof(Counters) ), "memset" );
    ncgb::Work* work = wb.alloc<ncgb::Work>( 1 );
    checkCuda( cudaMemset( work, 0, sizeof(ncgb::Work) ), "memset" );
    ncgb::QEntry* queue = qb.alloc<ncgb::QEntry>( cap );
    StreamGuard sg;
    checkCuda( cudaStreamCreateWithFlags( &sg.s, cudaStreamNonBlocking ), "cudaStreamCreate" );
    cudaStream_t st = sg.s;
    Counters* hc = nullptr;
    checkCuda( cudaMallocHost( &hc, sizeof(Counters) ), "cudaMallocHost" );
    struct HostFree { Counters* p; ~HostFree() { cudaFreeHost( p ); } } hf{ hc };

    cudaEvent_t ev0, ev1;
    cudaEventCreate( &ev0 );
    cudaEventCreate( &ev1 );
    cudaEventRecord( ev0, st );

    Pop A = pa.pop, B = pb.pop;
    uint64_t nA = 0, emitted = 0;
    uint32_t step = 0;
    const bool timing = ncgb::phaseTiming();
    cudaEvent_t te0 = nullptr, te1 = nullptr;
    if ( timing ) {
      cudaEventCreate( &te0 );
      cudaEventCreate( &te1 );
    }
    double transport_ms = 0;
    uint64_t transport_launches = 0, neutron_steps = 0;
    const uint32_t kMaxSteps = 100000000u;
    for ( ;; ) {
      if ( emitted < sc.n && nA < cap ) {
        const uint64_t k = std::min<uint64_t>( sc.n - emitted, cap - nA );
        checkCuda( cudaMemsetAsync( &dc->n_a, 0, sizeof(unsigned long long), st ), "memset" );
        checkCuda( launchEmit( sc.s, gc.g, eng, t, A, nA, emitted, k, dc, nsm, st ), "k_mmc_emit" );
        checkCuda( cudaMemcpyAsync( hc, dc, sizeof(Counters), cudaMemcpyDeviceToHost, st ), "D2H" );
        checkCuda( cudaStreamSynchronize( st ), "k_mmc_emit" );
        emitted += k;
        nA += hc->n_a;
      }
      if ( nA == 0 ) {
        if ( emitted >= sc.n )
          break;
        continue;
      }
      checkCuda( cudaMemsetAsync( &dc->n_b, 0, sizeof(unsigned long long), st ), "memset" );
      if ( timing )
        cudaEventRecord( te0, st );
      checkCuda( launchTransport( hi.view, gc.g, eng, t, A, nA, B, step, dc, nsm, st ), "k_mmc_transport" );
      if ( timing )
        cudaEventRecord( te1, st );
      checkCuda( cudaMemcpyAsync( hc, dc, sizeof(Counters), cudaMemcpyDeviceToHost, st ), "D2H" );
      checkCuda( cudaStreamSynchronize( st ), "k_mmc_transport" );
      if ( timing ) {
        float ms = 0;
        cudaEventElapsedTime( &ms, te0, te1 );
        transport_ms += ms;
        ++transport_launches;
      }
      neutron_steps += nA;
      if ( hc->nfail )
        throw MmcError( "CalcError", "MiniMC: " + std::to_string( hc->nfail ) + " scatter(s) failed (a rejection"
                        " loop reached its limit of attempts)" );
      const uint64_t nB = hc->n_b;
      if ( nB ) {
        ncgb::Batch b;
        std::memset( &b, 0, sizeof(b) );
        b.ekin = B.e;
        b.n_ekin = b.n_out = nB;
        b.seed = hi.seed;
        b.callseq = step;
        b.stream = hi.streamidx;
        b.mode = 0;
        b.fast = hi.mode == NCGB_MODE_MIXED;
        b.learned = hi.sampler == NCGB_SAMPLER_LEARNED;
        b.out_a = B.e_new;
        b.dir_in = B.dir;
        b.dir_out = B.dir_new;
        b.status = B.st;
        b.rng_index = B.id;
        b.work = work;
        b.queue = queue;
        checkCuda( ncgb::launchScatter( hi.view, b, st ), "scatter kernels" );
      }
      std::swap( A, B );
      nA = nB;
      if ( ++step >= kMaxSteps )
        throw MmcError( "CalcError", "MiniMC: step limit reached" );
    }
    cudaEventRecord( ev1, st );
    RunResult r;
    r.tally.resize( t.nbuf );
    checkCuda( cudaMemcpyAsync( r.tally.data(), t.buf, t.nbuf * sizeof(double), cudaMemcpyDeviceToHost, st ), "D2H" );
    checkCuda( cudaMemcpyAsync( hc, dc, sizeof(Counters), cudaMemcpyDeviceToHost, st ), "D2H" );
    checkCuda( cudaStreamSynchronize( st ), "MiniMC" );
    float ms = 0;
    cudaEventElapsedTime( &ms, ev0, ev1 );
    cudaEventDestroy( ev0 );
    cudaEventDestroy( ev1 );
    formTotals( t, r.tally );
    r.c = *hc;
    r.steps = step;
    r.seconds = ms * 1e-3;
    r.transport_ms = transport_ms;
    r.transport_launches = transport_launches;
    r.neutron_steps = neutron_steps;
    if ( timing ) {
      cudaEventDestroy( te0 );
      cudaEventDestroy( te1 );
    }
    return r;
  }

  // ---- results JSON ------------------------------------------------------------------------
  const char* const kGroupNames[kGroups] = { "total", "NOSCAT", "SINGLESCAT_ELAS", "SINGLESCAT_INELAS",
                                             "MULTISCAT_PUREELAS", "MULTISCAT_OTHER" };

  double fromKey( double stored )
  {
    long long k;
    std::memcpy( &k, &stored, 8 );
    if ( k < 0 )
      k ^= 0x7FFFFFFFFFFFFFFFLL;
    double v;
    std::memcpy( &v, &k, 8 );
    return v;
  }

  // With breakdowns the kernels fill only the five category groups; the
  // total group (0) is formed here: bins and sums added, extremes combined.
  void formTotals( const Tally& t, std::vector<double>& buf )
  {
    if ( !t.breakdown )
      return;
    for ( int k = 0; k < T_N; ++k ) {
      const TallyHist& h = t.h[k];
      if ( !h.enabled )
        continue;
      const int64_t nb2 = (int64_t)( h.nbins + 2 ) * 2;
      double* b0 = buf.data() + h.off;
      for ( int64_t i = 0; i < nb2; ++i ) {
        double v = 0.0;
        for ( int g = 1; g < kGroups; ++g )
          v += b0[g * nb2 + i];
        b0[i] = v;
      }
      double* s0 = buf.data() + h.soff;
      long long mn = 0x7FFFFFFFFFFFFFFFLL, mx = (long long)0x8000000000000000ULL;
      for ( int j = 0; j < 3; ++j ) {
        double v = 0.0;
        for ( int g = 1; g < kGroups; ++g )
          v += s0[g * kStats + j];
        s0[j] = v;
      }
      for ( int g = 1; g < kGroups; ++g ) {
        long long a, b;
        std::memcpy( &a, &s0[g * kStats + 3], 8 );
        std::memcpy( &b, &s0[g * kStats + 4], 8 );
        mn = std::min( mn, a );
        mx = std::max( mx, b );
      }
      std::memcpy( &s0[3], &mn, 8 );
      std::memcpy( &s0[4], &mx, 8 );
    }
  }

  void histJSON( std::ostream& os, const Tally& t, const std::vector<double>& buf, int k, int g, const char* title )
  {
    const TallyHist& h = t.h[k];
    const double* bins = buf.data() + h.off + (int64_t)g * ( h.nbins + 2 ) * 2;
    const double* stt = buf.data() + h.soff + g * kStats;
    os << "{\"datatype\":\"NCrystalHist1D_v1\",\"title\":" << jsonStr( title ) << ",\"stats\":{\"integral\":"
       << jsonNum( stt[0] );
    if ( stt[0] > 0.0 ) {
      // sums of w (x - shift) and w (x - shift)^2
      const double m1 = stt[1] / stt[0];
      const double mean = t.shift[k] + m1;
      const double rms = std::sqrt( std::max( 0.0, stt[2] / stt[0] - m1 * m1 ) );
      os << ",\"rms\":" << jsonNum( rms ) << ",\"mean\":" << jsonNum( mean ) << ",\"minfilled\":"
         << jsonNum( fromKey( stt[3] ) ) << ",\"maxfilled\":" << jsonNum( fromKey( stt[4] ) );
    } else {
      os << ",\"rms\":null,\"mean\":null,\"minfilled\":null,\"maxfilled\":null";
    }
    os << "},\"bindata\":{\"xmin\":" << jsonNum( h.xmin ) << ",\"xmax\":" << jsonNum( h.xmax ) << ",\"nbins\":"
       << h.nbins << ",\"content\":[";
    for ( int i = 0; i < h.nbins; ++i )
      os << ( i ? "," : "" ) << jsonNum( bins[2 * ( i + 1 )] );
    os << "],\"errorsq\":[";
    for ( int i = 0; i < h.nbins; ++i )
      os << ( i ? "," : "" ) << jsonNum( bins[2 * ( i + 1 ) + 1] );
    os << "],\"underflow\":" << jsonNum( bins[0] ) << ",\"overflow\":" << jsonNum( bins[2 * ( h.nbins + 1 )] )
       << ",\"underflow_errorsq\":" << jsonNum( bins[1] ) << ",\"overflow_errorsq\":"
       << jsonNum( bins[2 * ( h.nbins + 1 ) + 1] ) << "}}";
  }

  std::string resultsJSON( const std::string& matcfg, const GeomCfg& gc, const SrcCfg& sc, const EngineCfg& ec,
                           const Tally& t, const RunResult& r, const HandleInfo& hi )
  {
    std::ostringstream os;
    os << "{\"datatype\":\"NCrystalMiniMCResults_v1\",\"input\":{\"material\":{\"cfgstr\":" << jsonStr( matcfg )
       << ",\"decoded\":null},\"geom\":{\"cfgstr\":" << jsonStr( gc.cfgstr ) << ",\"decoded\":{" << gc.decoded
       << ",\"short_description\":" << jsonStr( gc.descr ) << "}},\"src\":{\"cfgstr\":" << jsonStr( sc.cfgstr )
       << ",\"decoded\":{" << sc.decoded << "},\"metadata\":{\"fixed_dir\":";
    auto dir = [&]( bool have ) {
      if ( have ) os << "[" << jsonNum( sc.dir[0] ) << "," << jsonNum( sc.dir[1] ) << "," << jsonNum( sc.dir[2] ) << "]";
      else os << "null";
    };
    dir( sc.fixed_dir );
    os << ",\"fixed_energy\":" << ( sc.fixed_e ? jsonNum( sc.e_fixed ) : std::string( "null" ) ) << ",\"mean_dir\":";
    dir( sc.mean_dir );
    os << ",\"mean_energy\":" << ( sc.mean_e ? jsonNum( sc.e_mean ) : std::string( "null" ) )
       << ",\"energy_description\":" << jsonStr( sc.edescr ) << "}},\"engine\":{\"name\":\"std\",\"cfgstr\":"
       << jsonStr( ec.cfgstr ) << ",\"decoded\":{" << ec.decoded << "}}},\"output\":{\"tally\":{";
    bool first = true;
    for ( int k = 0; k < T_N; ++k ) {
      if ( !t.h[k].enabled )
        continue;
      os << ( first ? "" : "," ) << jsonStr( kTallyNames[k] )
         << ":{\"datatype\":\"NCrystalMiniMCTallyHistBreakdown_v1\",\"tallyname\":" << jsonStr( kTallyNames[k] )
         << ",\"total\":";
      first = false;
      histJSON( os, t, r.tally, k, 0, kTallyNames[k] );
      os << ",\"breakdown\":{";
      if ( t.breakdown )
        for ( int g = 1; g < kGroups; ++g ) {
          os << ( g > 1 ? "," : "" ) << jsonStr( kGroupNames[g] ) << ":";
          histJSON( os, t, r.tally, k, g, kGroupNames[g] );
        }
      os << "} }";
    }
    const double nprov = (double)sc.n;
    os << "},\"metadata\":{\"provided\":{\"count\":" << sc.n << ",\"weight\":" << jsonNum( nprov )
       << "},\"miss\":{\"count\":" << r.c.miss << ",\"weight\":" << jsonNum( r.c.miss_w )
       << "},\"tallied\":{\"count\":" << r.c.tallied << ",\"weight\":" << jsonNum( r.c.tallied_w )
       << "},\"device\":{\"steps\":" << r.steps << ",\"seconds\":" << jsonNum( r.seconds )
       << ",\"neutron_steps\":" << r.neutron_steps << ",\"transport_ms\":"
       << ( r.transport_launches ? jsonNum( r.transport_ms ) : std::string( "null" ) )
       << ",\"transport_launches\":" << r.transport_launches
       << ",\"mode\":" << ( hi.mode == NCGB_MODE_MIXED ? "\"mixed\"" : "\"exact\"" ) << "}}}}";
    return os.str();
  }

  char* dupString( const std::string& s )
  {
    char* p = static_cast<char*>( std::malloc( s.size() + 1 ) );
    if ( !p )
      throw MmcError( "CalcError", "out of memory" );
    std::memcpy( p, s.c_str(), s.size() + 1 );
    return p;
  }

  std::vector<std::string> decodeQuery( const char* raw )
  {
    std::vector<std::string> q;
    std::string cur;
    for ( const char* c = raw ? raw : ""; *c; ++c ) {
      if ( *c == '\x07' ) { q.push_back( cur ); cur.clear(); }
      else cur.push_back( *c );
    }
    q.push_back( cur );
    return q;
  }

  uint64_t capacityFromEnv()
  {
    if ( const char* v = std::getenv( "NCGB_MMC_CAPACITY" ) ) {
      double x = 0;
      if ( toDbl( v, x ) && x >= 1 && x <= 4e9 )
        return (uint64_t)x;
    }
    return uint64_t(1) << 23;
  }

  std::string runWithHandle( ncrystal_scatter_t sc, const std::string& matcfg, const std::string& geomcfg,
                             const std::string& srccfg, const std::string& enginecfg )
  {
    HandleInfo hi;
    ncgb::handleInfo( sc, "ncgb_mmc_run", &hi );
    const GeomCfg gc = parseGeom( geomcfg );
    const SrcCfg src = parseSource( srccfg, gc.g );
    const EngineCfg ec = parseEngine( enginecfg );
    Tally t = setupTally( ec, src, hi.temperature );
    const RunResult r = runEngine( hi, gc, src, ec, t, capacityFromEnv() );
    return resultsJSON( matcfg.empty() ? hi.cfg : matcfg, gc, src, ec, t, r, hi );
  }

  struct ScatterHolder {
    ncrystal_scatter_t sc{ nullptr };
    ~ScatterHolder() { if ( sc.internal ) ncrystal_unref( &sc ); }
  };

  std::string jsonQuery( const std::vector<std::string>& q )
  {
    if ( q.size() < 2 || q[0] != "mmc" )
      throw MmcError( "BadInput", "This library serves only MiniMC JSON queries ([\"mmc\",\"run\",...] and"
                                  " [\"mmc\",\"scenario\",...]); other queries need NCrystal itself" );
    const std::string key = trim( q[1] );
    const std::size_t nargs = q.size() - 2;
    auto handleFor = [&]( const std::string& cfg, uint64_t seed, ScatterHolder& h ) {
      h.sc = ncrystal_create_scatter_builtinrng( cfg.c_str(), (unsigned long)( seed ^ 0x5ca77e2ull ) );
      if ( !h.sc.internal || ncrystal_error() )
        throw MmcError( "BadInput", "could not create the material \"" + cfg + "\"" );
    };
    if ( key == "run" ) {
      if ( nargs != 4 && nargs != 3 )
        bad( "Invalid MiniMC JSON query (correct usage: [\"mmc\",\"run\",CFGSTR,GEOMCFG,SRCCFG,ENGINECFG] or"
             " [\"mmc\",\"run\",CFGSTR,SCENARIOCFG,ENGINECFG])" );
      const std::string& cfg = q[2];
      const EngineCfg ec = parseEngine( nargs == 4 ? q[5] : q[4] );
      ScatterHolder h;
      handleFor( cfg, ec.seed, h );
      if ( nargs == 4 )
        return runWithHandle( h.sc, cfg, q[3], q[4], q[5] );
      HandleInfo hi;
      ncgb::handleInfo( h.sc, "ncrystal_jsonquery", &hi );
      const Scenario d = decodeScenario( h.sc, hi, q[3] );
      return runWithHandle( h.sc, cfg, d.geomcfg, d.srccfg, q[4] );
    }
    if ( key == "scenario" ) {
      if ( nargs != 2 )
        bad( "Invalid MiniMC JSON query (correct usage: [\"mmc\",\"scenario\",CFGSTR,SCENARIOSTR])" );
      ScatterHolder h;
      handleFor( q[2], 0, h );
      HandleInfo hi;
      ncgb::handleInfo( h.sc, "ncrystal_jsonquery", &hi );
      const Scenario d = decodeScenario( h.sc, hi, q[3] );
      return "{\"geomcfg\":" + jsonStr( d.geomcfg ) + ",\"srccfg\":" + jsonStr( d.srccfg ) + "}";
    }
    if ( key == "inspectcfg" ) {
      if ( nargs != 2 )
        bad( "Invalid MiniMC JSON query (correct usage: [\"mmc\",\"inspectcfg\",\"src|geom|engine\",STRCFG])" );
      if ( q[2] == "geom" ) {
        const GeomCfg gc = parseGeom( q[3] );
        return "{\"cfgstr\":" + jsonStr( gc.cfgstr ) + ",\"decoded\":{" + gc.decoded + ",\"short_description\":"
               + jsonStr( gc.descr ) + "}}";
      }
      if ( q[2] == "engine" ) {
        const EngineCfg ec = parseEngine( q[3] );
        return "{\"name\":\"std\",\"cfgstr\":" + jsonStr( ec.cfgstr ) + ",\"decoded\":{" + ec.decoded + "}}";
      }
      if ( q[2] == "src" ) {
        Geom g;
        std::memset( &g, 0, sizeof(g) );
        g.kind = GEOM_SPHERE;
        g.r = 1e99;
        const SrcCfg s = parseSource( q[3], g );
        return "{\"cfgstr\":" + jsonStr( s.cfgstr ) + ",\"decoded\":{" + s.decoded + "}}";
      }
      bad( "Invalid MiniMC JSON query (correct usage: [\"mmc\",\"inspectcfg\",\"src|geom|engine\",STRCFG])" );
    }
    bad( "Invalid MiniMC JSON query: unsupported key \"" + key + "\"" );
  }

  void report( const std::exception& e )
  {
    if ( auto me = dynamic_cast<const MmcError*>( &e ) )
      ncgb::reportError( me->type.c_str(), me->what() );
    else
      ncgb::reportError( e );
  }
}

extern "C" {

char* ncrystal_jsonquery( const char* raw )
{
  try {
    return dupString( jsonQuery( decodeQuery( raw ) ) );
  } catch ( std::exception& e ) {
    report( e );
  }
  return nullptr;
}

void ncrystal_dealloc_string( char* s )
{
  std::free( s );
}

char* ncgb_mmc_run( ncrystal_scatter_t sc, const char* geomcfg, const char* srccfg, const char* enginecfg )
{
  try {
    if ( !geomcfg || !srccfg )
      bad( "ncgb_mmc_run: geomcfg and srccfg are required" );
    return dupString( runWithHandle( sc, std::string(), geomcfg, srccfg, enginecfg ? enginecfg : "" ) );
  } catch ( std::exception& e ) {
    report( e );
  }
  return nullptr;
}

}
