// Problem files: a parser for the libconfig syntax the reference's inputs
// use (settings `name = value;` or `name : value;`, groups { }, lists ( ),
// arrays [ ], integers, floats, booleans, strings, #, // and /* */
// comments) and Input, which reads the reference's schema from it
// (src/Input.cpp): Problems, DomainDecompositions/CheckerboardDD, Domains,
// SquaredSlownesses (Constant, CSV), RHSs, GlobalSolvers (GMRES), Outputs (VTK).
#include "lsweeps_host.hpp"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>

// ===========================================================================
// libconfig subset
// ===========================================================================
namespace {

class CfgParser {
 public:
  explicit CfgParser(const std::string& t) : s(t) {}

  CfgSetting parse_root() {
    CfgSetting root;
    root.kind = CfgSetting::GROUP;
    parse_settings(root, '\0');
    return root;
  }

 private:
  const std::string& s;
  size_t i = 0;
  int line = 1;

  [[noreturn]] void fail(const std::string& m) const {
    throw lsw_host_error("ERROR: problem file, line " + std::to_string(line) + ": " + m);
  }

  void skip() {
    while (i < s.size()) {
      const char c = s[i];
      if (c == '\n') { ++line; ++i; }
      else if (std::isspace((unsigned char)c)) ++i;
      else if (c == '#' || (c == '/' && i + 1 < s.size() && s[i + 1] == '/')) {
        while (i < s.size() && s[i] != '\n') ++i;
      } else if (c == '/' && i + 1 < s.size() && s[i + 1] == '*') {
        i += 2;
        while (i + 1 < s.size() && !(s[i] == '*' && s[i + 1] == '/')) { if (s[i] == '\n') ++line; ++i; }
        if (i + 1 >= s.size()) fail("unterminated comment");
        i += 2;
      } else break;
    }
  }

  char peek() { skip(); return i < s.size() ? s[i] : '\0'; }

  std::string name() {
    skip();
    const size_t b = i;
    if (i < s.size() && (std::isalpha((unsigned char)s[i]) || s[i] == '*')) {
      ++i;
      while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '_' || s[i] == '-' || s[i] == '*')) ++i;
    }
    if (i == b) fail("setting name expected");
    return s.substr(b, i - b);
  }

  void parse_settings(CfgSetting& g, char close) {
    while (true) {
      const char c = peek();
      if (c == close) { if (close) ++i; return; }
      if (c == '\0') fail("unexpected end of file");
      if (c == '@') fail("@include is not supported");
      CfgSetting v;
      v.name = name();
      const char a = peek();
      if (a != '=' && a != ':') fail("'=' or ':' expected after " + v.name);
      ++i;
      parse_value(v);
      const char t = peek();
      if (t == ';' || t == ',') ++i;
      g.children.push_back(std::move(v));
    }
  }

  void parse_value(CfgSetting& v) {
    const char c = peek();
    if (c == '{') { ++i; v.kind = CfgSetting::GROUP; parse_settings(v, '}'); return; }
    if (c == '(' || c == '[') {
      ++i;
      v.kind = c == '(' ? CfgSetting::LIST : CfgSetting::ARRAY;
      const char close = c == '(' ? ')' : ']';
      if (peek() == close) { ++i; return; }
      while (true) {
        CfgSetting e;
        parse_value(e);
        v.children.push_back(std::move(e));
        const char t = peek();
        if (t == ',') { ++i; continue; }
        if (t == close) { ++i; return; }
        fail("',' or closing bracket expected");
      }
    }
    if (c == '"') {
      v.kind = CfgSetting::STRING;
      while (peek() == '"') {   // adjacent strings concatenate
        ++i;
        while (i < s.size() && s[i] != '"') {
          if (s[i] == '\\' && i + 1 < s.size()) {
            const char e = s[++i];
            v.s += e == 'n' ? '\n' : e == 't' ? '\t' : e;
          } else {
            if (s[i] == '\n') ++line;
            v.s += s[i];
          }
          ++i;
        }
        if (i >= s.size()) fail("unterminated string");
        ++i;
      }
      return;
    }
    // scalar: boolean or number
    skip();
    size_t b = i;
    while (i < s.size() && (std::isalnum((unsigned char)s[i]) || s[i] == '.' || s[i] == '+' || s[i] == '-')) ++i;
    std::string tok = s.substr(b, i - b);
    if (tok.empty()) fail("value expected");
    std::string low = tok;
    for (auto& ch : low) ch = (char)std::tolower((unsigned char)ch);
    if (low == "true" || low == "false") { v.kind = CfgSetting::BOOL; v.b = low == "true"; return; }
    while (!low.empty() && low.back() == 'l') { low.pop_back(); tok.pop_back(); }   // 64-bit suffix
    char* end = nullptr;
    if (low.size() > 2 && low[0] == '0' && low[1] == 'x') {
      v.kind = CfgSetting::INT;
      v.i = std::strtoll(tok.c_str(), &end, 16);
    } else if (low.find_first_of(".e") != std::string::npos && low.find("0x") == std::string::npos) {
      v.kind = CfgSetting::FLOAT;
      v.f = std::strtod(tok.c_str(), &end);
    } else {
      v.kind = CfgSetting::INT;
      v.i = std::strtoll(tok.c_str(), &end, 10);
    }
    if (!end || *end != '\0') fail("bad number " + tok);
    v.f = v.kind == CfgSetting::INT ? (double)v.i : v.f;
  }
};

}  // namespace

CfgSetting cfg_parse_text(const std::string& text) { return CfgParser(text).parse_root(); }

CfgSetting cfg_parse_file(const std::string& path) {
  std::ifstream in(path);
  if (!in) throw lsw_host_error("ERROR: cannot open problem file " + path);
  std::stringstream ss;
  ss << in.rdbuf();
  return cfg_parse_text(ss.str());
}

bool CfgSetting::exists(const std::string& n) const {
  for (const auto& c : children)
    if (c.name == n) return true;
  return false;
}

const CfgSetting& CfgSetting::operator[](const std::string& n) const {
  for (const auto& c : children)
    if (c.name == n) return c;
  throw lsw_host_error("ERROR: setting " + n + " not found");
}

const CfgSetting& CfgSetting::operator[](int idx) const {
  if (idx < 0 || idx >= (int)children.size()) throw lsw_host_error("ERROR: setting index out of range");
  return children[idx];
}

bool CfgSetting::lookupValue(const std::string& n, std::string& v) const {
  if (!exists(n)) return false;
  const CfgSetting& c = (*this)[n];
  if (c.kind != STRING) return false;
  v = c.s;
  return true;
}
bool CfgSetting::lookupValue(const std::string& n, double& v) const {
  if (!exists(n)) return false;
  const CfgSetting& c = (*this)[n];
  if (c.kind != FLOAT && c.kind != INT) return false;
  v = c.kind == INT ? (double)c.i : c.f;
  return true;
}
bool CfgSetting::lookupValue(const std::string& n, int& v) const {
  if (!exists(n)) return false;
  const CfgSetting& c = (*this)[n];
  if (c.kind != INT) return false;
  v = (int)c.i;
  return true;
}
bool CfgSetting::lookupValue(const std::string& n, UInt& v) const {
  int t;
  if (!lookupValue(n, t) || t < 0) return false;
  v = (UInt)t;
  return true;
}
bool CfgSetting::lookupValue(const std::string& n, bool& v) const {
  if (!exists(n)) return false;
  const CfgSetting& c = (*this)[n];
  if (c.kind != BOOL) return false;
  v = c.b;
  return true;
}

// ===========================================================================
// Input (src/Input.cpp)
// ===========================================================================
namespace {
[[noreturn]] void need(const std::string& what) { throw lsw_host_error("ERROR: No " + what + " prescribed"); }
}  // namespace

void Input::openFile(const std::string& name) {
  mRoot = cfg_parse_file(name);
  const size_t slash = name.find_last_of('/');
  mDir = slash == std::string::npos ? std::string() : name.substr(0, slash + 1);
  mOpened = true;
}

UInt Input::getNumProblems() const {
  if (!mOpened) throw lsw_host_error("ERROR: no input file opened");
  if (!mRoot.exists("Problems")) need("Problems");
  return (UInt)mRoot["Problems"].getLength();
}

void Input::readProblemDD(DD*& dd, UInt probID) const {
  if (probID >= getNumProblems()) throw lsw_host_error("ERROR: problem index out of range");
  const CfgSetting& problem = mRoot["Problems"][(int)probID];
  std::string type;
  UInt id = 0;
  if (!problem.lookupValue("DomainDecomposition", type)) need("DomainDecomposition in Problem");
  if (!problem.lookupValue("DomainDecompositionID", id)) need("DomainDecompositionID in Problem");
  if (type != "CheckerboardDD") throw lsw_host_error("ERROR: unknown domain decomposition " + type);
  readCheckerboardDD(id, dd);
}

void Input::readDomain(const std::string& name, UInt dim, std::vector<DoubleVector>& dom) const {
  if (!mRoot.exists("Domains") || !mRoot["Domains"].exists(name)) need("Domain " + name);
  const CfgSetting& d = mRoot["Domains"][name];
  UInt ddim = 0;
  if (!d.lookupValue("Dim", ddim)) need("Dim in Domain " + name);
  if (ddim != dim) throw lsw_host_error("ERROR: domain dimension mismatch");
  double ax, bx, ay, by;
  if (!d.lookupValue("ax", ax)) need("ax in Domain " + name);
  if (!d.lookupValue("bx", bx)) need("bx in Domain " + name);
  if (!d.lookupValue("ay", ay)) need("ay in Domain " + name);
  if (!d.lookupValue("by", by)) need("by in Domain " + name);
  dom = {{ax, bx}, {ay, by}};
}

Function* Input::readSquaredSlowness(const std::string& name) const {
  if (!mRoot.exists("SquaredSlownesses") || !mRoot["SquaredSlownesses"].exists(name)) need("SquaredSlowness " + name);
  const CfgSetting& ss = mRoot["SquaredSlownesses"][name];
  std::string type;
  if (!ss.lookupValue("Type", type)) need("Type in SquaredSlowness " + name);
  if (type == "Constant") {
    // unit squared slowness: the effective frequency is omega (Input.cpp:744-750)
    FunctionConstant f;
    f.setVal(1.0);
    return f.copy();
  }
  if (type == "CSV") {
    std::string file, domain;
    UInt dim = 0;
    if (!ss.lookupValue("Filename", file)) need("Filename in SquaredSlowness " + name);
    if (!ss.lookupValue("Dim", dim)) need("Dim in SquaredSlowness " + name);
    if (!ss.lookupValue("Domain", domain)) need("Domain in SquaredSlowness " + name);
    std::vector<DoubleVector> dom;
    readDomain(domain, dim, dom);
    if (!file.empty() && file[0] != '/') file = mDir + file;
    FunctionCSV f;
    f.setFile(file, dom);
    return f.copy();
  }
  throw lsw_host_error("ERROR: unknown squared slowness type " + type);
}

void Input::readCheckerboardDD(UInt DDID, DD*& dd) const {
  if (!mRoot.exists("DomainDecompositions") || !mRoot["DomainDecompositions"].exists("CheckerboardDD"))
    need("CheckerboardDD");
  const CfgSetting& list = mRoot["DomainDecompositions"]["CheckerboardDD"];
  if ((int)DDID >= list.getLength()) throw lsw_host_error("ERROR: CheckerboardDD index out of range");
  const CfgSetting& CDD = list[(int)DDID];
  UInt dim = 0;
  if (!CDD.lookupValue("Dim", dim)) need("Dim in CheckerboardDD");
  if (dim != 2) throw lsw_host_error("ERROR: only Dim = 2 is supported");
  std::string domain, pde;
  if (!CDD.lookupValue("Domain", domain)) need("Domain in CheckerboardDD");
  std::vector<DoubleVector> dom;
  readDomain(domain, dim, dom);
  if (!CDD.lookupValue("PDE", pde)) need("PDE in CheckerboardDD");
  if (pde != "Helmholtz") throw lsw_host_error("ERROR: unknown PDE " + pde);

  // assembler (Input::readAssemblerHelmholtz2DFD, Input.cpp:797-858)
  double omega = 0.0, minWL = 0.0;
  std::string ssType;
  UInt order = 0;
  if (!CDD.lookupValue("Omega", omega)) need("Omega in CheckerboardDD");
  if (!CDD.lookupValue("MinWavelengthsInPML", minWL)) need("MinWavelengthsInPML in CheckerboardDD");
  if (!CDD.lookupValue("SquaredSlowness", ssType)) need("SquaredSlowness in CheckerboardDD");
  std::unique_ptr<Function> m(readSquaredSlowness(ssType));
  if (!CDD.lookupValue("Order", order)) need("Order in CheckerboardDD");
  PMLCubic2D pml;
  pml.setAbsorptionCoeff(std::log(omega));
  // the longest wavelength in the medium: domain extent x 2 pi / omega / sqrt(min m)
  const double w1 = (dom[0][1] - dom[0][0]) * 2 * M_PI / omega;
  const double w2 = (dom[1][1] - dom[1][0]) * 2 * M_PI / omega;
  const double wavelength = std::min(w1, w2) / std::sqrt(m->getMinReal());
  pml.setWidth(minWL * wavelength);
  m->setDomain(dom);
  AssemblerHelmholtz2DFD assembler;
  assembler.setPML(&pml);
  assembler.setOmega(omega);
  assembler.setM(m.get());
  assembler.setOrder(order);

  UInt nX = 0, nY = 0, nCX = 0, nCY = 0;
  if (!(CDD.lookupValue("NX", nX) && CDD.lookupValue("NY", nY))) need("NX and NY in CheckerboardDD");
  if (!CDD.lookupValue("NCellsX", nCX)) need("NCellsX in CheckerboardDD");
  if (!CDD.lookupValue("NCellsY", nCY)) need("NCellsY in CheckerboardDD");
  std::string solverType;
  if (!CDD.lookupValue("Solver", solverType)) need("Solver in CheckerboardDD");
  // "Eigen" (the reference's SparseLU) and "CUDA" both select the GPU cell solver
  if (solverType != "Eigen" && solverType != "CUDA") throw lsw_host_error("ERROR: unknown local solver " + solverType);
  // extension: Precision = "fp64" (default, the reference's arithmetic), "mixed" (complex64
  // factors and sweeps) or "split" (bf16 hi + lo factor terms on the tensor cores)
  std::string prec = "fp64";
  CDD.lookupValue("Precision", prec);
  if (prec != "fp64" && prec != "mixed" && prec != "split")
    throw lsw_host_error("ERROR: Precision must be \"fp64\", \"mixed\" or \"split\"");
  LocalLinearSolverCUDA solver;
  auto* cb = new DDCheckerboard();
  try {
    cb->setUp(&assembler, &solver, dom, {nCX, nCY}, {nX, nY}, prec == "mixed" ? LSW_PREC_C64 : prec == "split" ? LSW_PREC_SPLIT : LSW_PREC_C128);
  } catch (...) {
    delete cb;
    throw;
  }
  dd = cb;
}

void Input::readProblemRHS(const DD* dd, RHS*& rhs, UInt probID) const {
  const CfgSetting& problem = mRoot["Problems"][(int)probID];
  std::string name;
  if (!problem.lookupValue("RHS", name)) need("RHS in Problem");
  if (!mRoot.exists("RHSs") || !mRoot["RHSs"].exists(name)) need("RHS " + name);
  const CfgSetting& srcs = mRoot["RHSs"][name];
  std::vector<DoubleVector> pts;
  for (int k = 0; k < srcs.getLength(); ++k) {
    UInt dim = 0;
    double x = 0, y = 0;
    if (!srcs[k].lookupValue("Dim", dim)) need("Dim in source");
    if (!srcs[k].lookupValue("x", x)) need("x in source");
    if (!srcs[k].lookupValue("y", y)) need("y in source");
    pts.push_back({x, y});
  }
  RHSSrcPts r;
  r.setSrcPts(pts);
  r.setEpsilon(dd->getMeshSize());   // the DD mesh size (Input.cpp:244-247)
  rhs = r.copy();
}

void Input::readProblemSolver(GlobalIterativeSolver*& solver, UInt probID) const {
  const CfgSetting& problem = mRoot["Problems"][(int)probID];
  std::string name, type;
  if (!problem.lookupValue("Solver", name)) need("Solver in Problem");
  if (!mRoot.exists("GlobalSolvers") || !mRoot["GlobalSolvers"].exists(name)) need("GlobalSolver " + name);
  const CfgSetting& sol = mRoot["GlobalSolvers"][name];
  if (!sol.lookupValue("Type", type)) need("Type in GlobalSolver " + name);
  if (type != "GMRES") throw lsw_host_error("ERROR: unknown global solver " + type);
  auto* g = new GlobalIterativeSolverGMRES();
  // as Input::readProblemSolver reads them (Input.cpp:367-387): Tol = 0 and
  // MaxIter = 0 keep the solver's defaults (1e-6, 40), Verbose defaults to true
  double tol = 1.0e-6;
  UInt maxIter = 0, restart;
  bool verbose = true;
  sol.lookupValue("Tol", tol);
  sol.lookupValue("MaxIter", maxIter);
  sol.lookupValue("Verbose", verbose);
  if (tol != 0.0) g->setTol(tol);
  if (maxIter != 0) g->setMaxIter(maxIter);
  if (!verbose) g->setVerbose(false);
  // extensions: Mode = "reference" (default) | "flexible", Restart
  std::string mode;
  if (sol.lookupValue("Mode", mode)) {
    if (mode == "flexible") g->setMode(LSW_GMRES_FLEXIBLE);
    else if (mode != "reference") { delete g; throw lsw_host_error("ERROR: Mode must be \"reference\" or \"flexible\""); }
  }
  if (sol.lookupValue("Restart", restart)) g->setRestart(restart);
  solver = g;
}

void Input::readProblemOutput(Output*& output, UInt probID) const {
  const CfgSetting& problem = mRoot["Problems"][(int)probID];
  std::string name, type, file;
  output = nullptr;
  if (!problem.lookupValue("Output", name)) return;
  if (!mRoot.exists("Outputs") || !mRoot["Outputs"].exists(name)) need("Output " + name);
  const CfgSetting& out = mRoot["Outputs"][name];
  if (!out.lookupValue("Type", type)) need("Type in Output " + name);
  if (type != "VTK") throw lsw_host_error("ERROR: unknown output type " + type);
  if (!out.lookupValue("Filename", file)) need("Filename in Output " + name);
  auto* o = new OutputVTK();
  o->setFilename(file);
  output = o;
}
