// Compile-only stand-ins for the parts of QDP++ (and chromabase.h) that chroma_plugin/ uses; the
// Chroma declarations sit in stand-ins named like the Chroma headers that declare them, so that a
// missing #include in the adapter fails here as it would in a Chroma build.
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
enum PlusMinus { PLUS = 1, MINUS = -1 };

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
struct LatticePropagator {};

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
}  // namespace Chroma
