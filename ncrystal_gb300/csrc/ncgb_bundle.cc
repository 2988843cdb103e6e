// Material bundle reader.  Record layout (written by bundle/ncgb_export.cc):
//   "NCGBNDL1" | u32 nrec | nrec x ( u32 name_len | name | u32 dtype | u64 count | payload )
// dtype 1 = f64, 2 = i64, 3 = u32, 4 = bytes.  Little-endian (x86-64 and aarch64).
#include "ncgb_host.hh"

#include <cstring>
#include <fstream>
#include <iterator>

namespace ncgb {

  Bundle Bundle::load( const std::string& path )
  {
    std::ifstream f( path, std::ios::binary );
    if ( !f )
      throw Error("could not open material bundle " + path);
    std::vector<char> buf( (std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>() );
    auto need = [&]( std::size_t pos, std::size_t n ) {
      if ( pos + n > buf.size() )
        throw Error("truncated material bundle " + path);
    };
    need(0,12);
    if ( std::memcmp(buf.data(),"NCGBNDL1",8) != 0 )
      throw Error("not a material bundle: " + path);
    uint32_t nrec;
    std::memcpy(&nrec,buf.data()+8,4);
    std::size_t pos = 12;
    Bundle b;
    b.m_path = path;
    for ( uint32_t r = 0; r < nrec; ++r ) {
      uint32_t nl, dt;
      uint64_t cnt;
      need(pos,4); std::memcpy(&nl,buf.data()+pos,4); pos += 4;
      need(pos,nl); std::string name(buf.data()+pos,nl); pos += nl;
      need(pos,12); std::memcpy(&dt,buf.data()+pos,4); std::memcpy(&cnt,buf.data()+pos+4,8); pos += 12;
      Rec rec;
      rec.dtype = dt;
      if ( dt == 1 ) {
        need(pos,cnt*8); rec.d.resize(cnt); std::memcpy(rec.d.data(),buf.data()+pos,cnt*8); pos += cnt*8;
      } else if ( dt == 2 ) {
        need(pos,cnt*8); rec.i.resize(cnt); std::memcpy(rec.i.data(),buf.data()+pos,cnt*8); pos += cnt*8;
      } else if ( dt == 3 ) {
        need(pos,cnt*4);
        rec.i.resize(cnt);
        for ( uint64_t k = 0; k < cnt; ++k ) {
          uint32_t u; std::memcpy(&u,buf.data()+pos+4*k,4); rec.i[k] = u;
        }
        pos += cnt*4;
      } else if ( dt == 4 ) {
        need(pos,cnt); rec.s.assign(buf.data()+pos,cnt); pos += cnt;
      } else {
        throw Error("bad record type in material bundle " + path);
      }
      b.m_recs[name] = std::move(rec);
    }
    return b;
  }

  const Bundle::Rec& Bundle::rec( const std::string& name, uint32_t dtype ) const
  {
    auto it = m_recs.find(name);
    if ( it == m_recs.end() )
      throw Error("material bundle " + m_path + " lacks record " + name);
    bool ok = ( it->second.dtype == dtype ) || ( dtype == 2 && it->second.dtype == 3 );
    if ( !ok )
      throw Error("material bundle " + m_path + ": record " + name + " has unexpected type");
    return it->second;
  }

  const std::vector<double>& Bundle::f64( const std::string& name ) const { return rec(name,1).d; }

  double Bundle::f64s( const std::string& name ) const
  {
    auto& v = rec(name,1).d;
    if ( v.size() != 1 )
      throw Error("material bundle record " + name + " is not a scalar");
    return v[0];
  }

  int64_t Bundle::i64s( const std::string& name ) const
  {
    auto& v = rec(name,2).i;
    if ( v.size() != 1 )
      throw Error("material bundle record " + name + " is not a scalar");
    return v[0];
  }

  const std::string& Bundle::str( const std::string& name ) const { return rec(name,4).s; }
}
