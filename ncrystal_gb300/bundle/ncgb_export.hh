// What the bundle exporter (ncgb_export.cc) offers its other callers: writing
// the material bundle of a process tree NCrystal made, and checking that every
// component of a tree is one the GPU path implements.
#ifndef NCGB_EXPORT_HH
#define NCGB_EXPORT_HH

#include <string>
#include "NCrystal/NCrystal.hh"

namespace ncgb_export {

  // Writes the bundle (atomically: a temporary file renamed into place) of the
  // scatter process tree 'top' of a material with the given Info; 'cfgkey' is
  // recorded as the bundle's cfg-string, 'temperature' as its temperature (-1
  // if none); 'absorption' may be null (no absorption constant recorded).
  void writeBundle( const std::string& path, const std::string& cfgkey,
                    const NCrystal::ProcImpl::Process& top, const NCrystal::Info& info,
                    double temperature, const NCrystal::ProcImpl::Process* absorption,
                    bool withDerived );

  // The bundle of a cfg-string, through NCrystal's own factories.
  void exportCfg( const std::string& cfgstr, const std::string& path, bool withDerived );

  // True if every component of the tree is PowderBragg, ElIncScatter,
  // SABScatter or FreeGas (at most 8 of them), or the tree is empty.
  bool supported( const NCrystal::ProcImpl::Process& top );
}

#endif
