// Compile-only stand-ins for the parts of QDP++ and Chroma that chroma_plugin/ uses.
//
// Test infrastructure: tests/test_plugin_compiles.py compiles the adapter sources against these
// declarations with g++ -fsyntax-only, so that the adapter's use of include/gbclover.h (types,
// argument lists, constants) and its own C++ are checked without a Chroma build.  The shapes
// follow the Chroma headers the adapter includes (syssolver.h:16-50, syssolver_linop.h,
// syssolver_mdagm.h:25-35, chrono_predictor.h:27-51, syssolver_linop_factory.h:29-39,
// xml_group_reader.h:16-26, clover_fermact_params_w.h:15-43); nothing here computes anything.
#pragma once
#include <iostream>
#include <string>
#include <vector>

namespace QDP {
const int Nd = 4, Nc = 3, Ns = 4;

struct Real {
  double v = 0;
  Real() = default;
  Real(double x) : v(x) {}
};
inline double toDouble(const Real& r) { return r.v; }
inline double toDouble(double d) { return d; }

template <typename T>
class multi1d {
 public:
  explicit multi1d(int n = 0) : d_(n) {}
  T& operator[](int i) { return d_[i]; }
  const T& operator[](int i) const { return d_[i]; }
  int size() const { return (int)d_.size(); }
 private:
  std::vector<T> d_;
};

struct Layout {
  static const multi1d<int>& lattSize();
  static int linearSiteIndex(const multi1d<int>& coord);
  static long vol();
  static int numNodes();
};

struct Subset {};

// element access of a lattice field: f.elem(site) ... .real() / .imag()
struct RComplexRef {
  double& real();
  double& imag();
  double real() const;
  double imag() const;
};
struct ColorVec {
  RComplexRef& elem(int c);
  const RComplexRef& elem(int c) const;
};
struct SpinVec {
  ColorVec& elem(int s);
  const ColorVec& elem(int s) const;
};
struct ColorMat {
  const RComplexRef& elem(int r, int c) const;
};
struct ColorMatSite {
  const ColorMat& elem() const;
};
struct LatticeFermion {
  SpinVec& elem(int site);
  const SpinVec& elem(int site) const;
};
struct LatticeColorMatrix {
  const ColorMatSite& elem(int site) const;
};

class XMLReader {
 public:
  XMLReader();
  explicit XMLReader(std::istream& is);
  XMLReader(XMLReader& parent, const std::string& path);
  int count(const std::string& path);
};
class XMLWriter {};
void read(XMLReader&, const std::string&, int&);
void read(XMLReader&, const std::string&, bool&);
void read(XMLReader&, const std::string&, Real&);
void read(XMLReader&, const std::string&, std::string&);
void write(XMLWriter&, const std::string&, int);
void write(XMLWriter&, const std::string&, bool);
void write(XMLWriter&, const std::string&, const Real&);
void write(XMLWriter&, const std::string&, const std::string&);
void push(XMLWriter&, const std::string&);
void pop(XMLWriter&);

struct QDPIO {
  static std::ostream& cout;
  static std::ostream& cerr;
};
[[noreturn]] void QDP_abort(int);
}  // namespace QDP

#define START_CODE()
#define END_CODE()

namespace Chroma {
using namespace QDP;

template <typename T>
class Handle {
 public:
  Handle() = default;
  explicit Handle(T* p) : p_(p) {}
  T* operator->() const { return p_; }
  T& operator*() const { return *p_; }
 private:
  T* p_ = nullptr;
};

enum PlusMinus { PLUS = 1, MINUS = -1 };

template <typename T>
class LinearOperator {
 public:
  virtual ~LinearOperator() {}
  virtual void operator()(T& chi, const T& psi, enum PlusMinus isign) const = 0;
  virtual const Subset& subset() const = 0;
};

template <typename T>
class MdagMLinOp : public LinearOperator<T> {
 public:
  explicit MdagMLinOp(const Handle<LinearOperator<T> >& A);
  void operator()(T& chi, const T& psi, enum PlusMinus isign) const override;
  const Subset& subset() const override;
};

template <typename T, typename P, typename Q>
class FermState {
 public:
  virtual ~FermState() {}
  virtual const Q& getLinks() const = 0;
};

struct SystemSolverResults_t {
  int n_count = 0;
  Real resid;
};

template <typename T>
class SystemSolver {
 public:
  virtual ~SystemSolver() {}
  virtual SystemSolverResults_t operator()(T& psi, const T& chi) const = 0;
  virtual const Subset& subset() const = 0;
};

template <typename T>
class LinOpSystemSolver : public SystemSolver<T> {};

template <typename T>
class AbsChronologicalPredictor4D {
 public:
  virtual ~AbsChronologicalPredictor4D() {}
  virtual void operator()(T& psi, const LinearOperator<T>& A, const T& chi) = 0;
  virtual void reset() = 0;
  virtual void newVector(const T& psi) = 0;
};

template <typename T>
class MdagMSystemSolver : public SystemSolver<T> {
 public:
  virtual SystemSolverResults_t operator()(T& psi, const T& chi) const = 0;
  virtual SystemSolverResults_t operator()(T& psi, const T& chi, AbsChronologicalPredictor4D<T>& predictor) const = 0;
};

struct GroupXML_t {
  std::string xml, id, path;
};
GroupXML_t readXMLGroup(XMLReader& xml, const std::string& path, const std::string& type_name);

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

// string-keyed factory singletons (objfactory.h, singleton.h)
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
typedef Singleton<SolverFactory<LinOpSystemSolver<LatticeFermion> > > TheLinOpFermSystemSolverFactory;
typedef Singleton<SolverFactory<MdagMSystemSolver<LatticeFermion> > > TheMdagMFermSystemSolverFactory;

class SymEvenOddPrecCloverLinOp : public LinearOperator<LatticeFermion> {
 public:
  void operator()(LatticeFermion& chi, const LatticeFermion& psi, enum PlusMinus isign) const override;
  const Subset& subset() const override;
};
}  // namespace Chroma
