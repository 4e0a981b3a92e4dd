// compile-only stand-in: the declarations the adapter takes from this header
#pragma once
#include "../../../chromabase.h"

namespace Chroma {
struct AnisoParam_t {
  bool anisoP = false;
  int t_dir = 3;
  Real xi_0, nu;
};

struct CloverFermActParams {
  Real Mass, clovCoeffR, clovCoeffT, u0;
  AnisoParam_t anisoParam;
  Real max_norm;
  bool max_norm_usedP = false;
  Real twisted_m;
  bool twisted_m_usedP = false;
};
void read(XMLReader&, const std::string&, CloverFermActParams&);
void write(XMLWriter&, const std::string&, const CloverFermActParams&);
}  // namespace Chroma
