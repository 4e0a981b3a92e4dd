// compile-only stand-in of the string-keyed factory singletons (objfactory.h, singleton.h)
#pragma once
#include "state.h"
#include "handle.h"
#include "linearop.h"

namespace Chroma {
typedef Handle<FermState<LatticeFermion, multi1d<LatticeColorMatrix>, multi1d<LatticeColorMatrix> > > FSHandle;
template <typename Product>
struct SolverFactory {
  typedef Product* (*Creator)(XMLReader&, const std::string&, FSHandle, Handle<LinearOperator<LatticeFermion> >);
  bool registerObject(const std::string& id, Creator c);
  Product* createObject(const std::string& id, XMLReader& xml, const std::string& path, FSHandle state,
                        Handle<LinearOperator<LatticeFermion> > A);
};
template <typename F>
struct Singleton {
  static F& Instance();
};
}  // namespace Chroma
