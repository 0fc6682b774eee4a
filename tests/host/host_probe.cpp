// Probe of the C++ host layer for the tests: prints what the classes compute
// so that the Python tests can check it.
//   host_probe parse <problem file>                      canonical dump of the settings
//   host_probe csv <csv> ax bx ay by  dx0 dx1 dy0 dy1    reads "x y" lines on stdin,
//                                                        prints Re eval per point
//   host_probe rhs eps x0 y0 [x1 y1 ...]                 reads "x y" lines, prints the RHS
//   host_probe cell N m p h omega cell m_grid.bin         one SubdomainStructured (no GPU): index
//                                                        sets, L-trace sets, element sets, corner
//                                                        indices, A x, equivalent sources and L
//                                                        traces of fixed test values, one JSON object
#include <cmath>
#include <cstdio>
#include <fstream>
#include <memory>
#include <sstream>
#include <cstdlib>
#include <iostream>
#include <string>

#include "lsweeps_host.hpp"

static void dump(const CfgSetting& s, int depth) {
  std::string pad(2 * depth, ' ');
  std::cout << pad << (s.name.empty() ? "-" : s.name) << " ";
  switch (s.kind) {
    case CfgSetting::GROUP: std::cout << "group\n"; break;
    case CfgSetting::LIST: std::cout << "list\n"; break;
    case CfgSetting::ARRAY: std::cout << "array\n"; break;
    case CfgSetting::INT: std::cout << "int " << s.i << "\n"; break;
    case CfgSetting::FLOAT: std::printf("float %.17g\n", s.f); break;
    case CfgSetting::BOOL: std::cout << "bool " << (s.b ? "true" : "false") << "\n"; break;
    case CfgSetting::STRING: std::cout << "string " << s.s << "\n"; break;
  }
  for (const auto& c : s.children) dump(c, depth + 1);
}

static void json_uints(std::ostringstream& o, const UIntVector& v) {
  o << "[";
  for (size_t i = 0; i < v.size(); ++i) o << (i ? "," : "") << v[i];
  o << "]";
}
static void json_cplx(std::ostringstream& o, const ComplexVector& v) {
  o << "[";
  char buf[80];
  for (size_t i = 0; i < v.size(); ++i) {
    std::snprintf(buf, sizeof buf, "%s[%.17g,%.17g]", i ? "," : "", v[i].real(), v[i].imag());
    o << buf;
  }
  o << "]";
}
// deterministic test values
static ComplexVector vals(size_t n, double seed) {
  ComplexVector v(n);
  for (size_t k = 0; k < n; ++k) v[k] = Complex(std::cos(seed + 0.7 * k), std::sin(2.0 * seed + 0.3 * k));
  return v;
}

static int cell_probe(int N, int m, int p, double h, double omega, int cell, const char* grid_path) {
  const int n_g = N * m + N - 1, nd = n_g + 2 * p - 1;
  auto grid = std::make_shared<std::vector<double>>((size_t)nd * nd);
  std::ifstream f(grid_path, std::ios::binary);
  f.read(reinterpret_cast<char*>(grid->data()), (std::streamsize)(grid->size() * sizeof(double)));
  if (!f) { std::cerr << "short grid file" << std::endl; return 2; }
  lsw_geom g{N, m, p, 2, h};
  lsw_cell_info ci;
  if (lsw_geometry_cell(&g, cell, &ci) != LSW_OK) { std::cerr << "geometry" << std::endl; return 2; }
  LocalLinearSolverCUDA proto;
  SubdomainStructured sd(nullptr, cell, ci, &proto, h, 0.0, 0.0, p, omega, grid, nd);
  std::unique_ptr<Subdomain> s(sd.copy());   // through the abstract interface
  std::ostringstream o;
  o << "{\"size\":" << s->getSize() << ",\"nels\":" << s->getNEls();
  for (const char* dir : {"LeftRight", "UpDown"})
    for (int sh = 0; sh < 2; ++sh) {
      std::vector<UIntVector> r;
      s->getIndexSets(dir, sh != 0, r);
      o << ",\"sets_" << dir << "_" << sh << "\":[";
      for (size_t k = 0; k < r.size(); ++k) { if (k) o << ","; json_uints(o, r[k]); }
      o << "]";
      s->getElIndexSets(dir, sh != 0, r);
      o << ",\"elsets_" << dir << "_" << sh << "\":[";
      for (size_t k = 0; k < r.size(); ++k) { if (k) o << ","; json_uints(o, r[k]); }
      o << "]";
    }
  const char* Ls[] = {"BottomLeft", "BottomRight", "TopRight", "TopLeft"};
  for (const char* lt : Ls)
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) {
        std::vector<UIntVector> r;
        s->getLTraceIndexSets(lt, a != 0, b != 0, r);
        o << ",\"ltr_" << lt << "_" << a << b << "\":[";
        json_uints(o, r[0]);
        o << ",";
        json_uints(o, r[1]);
        o << "]";
      }
  // A x
  ComplexVector x = vals(s->getSize(), 0.25), y;
  s->applySystemMatrix(x, y);
  o << ",\"Ax\":";
  json_cplx(o, y);
  // equivalent sources of every trace type with values 0.5 / 1.5
  const char* St[] = {"Left", "Right", "Bottom", "Top", "BottomLeft", "BottomRight", "TopRight", "TopLeft"};
  for (const char* tt : St)
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) {
        std::vector<UIntVector> L;
        UIntVector t0, t1;
        const std::string t = tt;
        if (t == "Left" || t == "Right" || t == "Bottom" || t == "Top") {
          std::vector<UIntVector> sets;
          const bool lr = t == "Left" || t == "Right";
          s->getIndexSets(lr ? "LeftRight" : "UpDown", lr ? a != 0 : b != 0, sets);
          t0 = (t == "Left" || t == "Bottom") ? sets[1] : sets[5];
          t1 = (t == "Left" || t == "Bottom") ? sets[2] : sets[4];
        } else {
          s->getLTraceIndexSets(t, a != 0, b != 0, L);
          t0 = L[0];
          t1 = L[1];
        }
        if (t0.empty() || t1.empty()) continue;
        std::vector<ComplexVector> r;
        s->getEquivalentSources(t, a != 0, b != 0, vals(t0.size(), 0.5), vals(t1.size(), 1.5), r);
        o << ",\"eqs_" << t << "_" << a << b << "\":[";
        json_cplx(o, r[0]);
        o << ",";
        json_cplx(o, r[1]);
        o << "]";
      }
  // L traces of line values 2.0 / 2.5 / 3.0 / 3.5 (LR0, LR1, UD0, UD1)
  for (const char* lt : Ls)
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) {
        std::vector<UIntVector> s1, s2;
        s->getIndexSets("LeftRight", a != 0, s1);
        s->getIndexSets("UpDown", b != 0, s2);
        const std::string t = lt;
        const bool left = t == "BottomLeft" || t == "TopLeft", bottom = t == "BottomLeft" || t == "BottomRight";
        const UIntVector& lr0 = left ? s1[1] : s1[5];
        const UIntVector& lr1 = left ? s1[2] : s1[4];
        const UIntVector& ud0 = bottom ? s2[1] : s2[5];
        const UIntVector& ud1 = bottom ? s2[2] : s2[4];
        if (lr0.empty() || lr1.empty() || ud0.empty() || ud1.empty()) continue;
        std::vector<ComplexVector> r;
        s->extractLTraces(t, a != 0, b != 0, vals(lr0.size(), 2.0), vals(lr1.size(), 2.5), vals(ud0.size(), 3.0),
                          vals(ud1.size(), 3.5), r);
        o << ",\"ltraces_" << t << "_" << a << b << "\":[";
        json_cplx(o, r[0]);
        o << ",";
        json_cplx(o, r[1]);
        o << "]";
      }
  // corners of a few elements, DOF points, boundary points
  o << ",\"corners\":[";
  for (UInt e = 0; e < s->getNEls(); ++e) {
    UIntVector c;
    s->getElPhysPtIndices(e, c);
    if (e) o << ",";
    json_uints(o, c);
  }
  o << "]";
  std::vector<DoubleVector> pts;
  s->getPhysPts(pts);
  o << ",\"phys\":[";
  char buf[80];
  for (size_t i = 0; i < pts.size(); ++i) {
    std::snprintf(buf, sizeof buf, "%s[%.17g,%.17g]", i ? "," : "", pts[i][0], pts[i][1]);
    o << buf;
  }
  o << "]}";
  std::cout << o.str() << std::endl;
  return 0;
}

int main(int argc, char** argv) {
  try {
    std::string cmd = argc > 1 ? argv[1] : "";
    if (cmd == "parse" && argc == 3) {
      dump(cfg_parse_file(argv[2]), 0);
      return 0;
    }
    if (cmd == "csv" && argc == 11) {
      FunctionCSV f;
      f.setFile(argv[2], {{atof(argv[3]), atof(argv[4])}, {atof(argv[5]), atof(argv[6])}});
      std::printf("min %.17g max %.17g\n", f.getMinReal(), f.getMaxReal());
      f.setDomain({{atof(argv[7]), atof(argv[8])}, {atof(argv[9]), atof(argv[10])}});
      double x, y;
      while (std::cin >> x >> y) std::printf("%.17g\n", f.eval({x, y}).real());
      return 0;
    }
    if (cmd == "cell" && argc == 9)
      return cell_probe(atoi(argv[2]), atoi(argv[3]), atoi(argv[4]), atof(argv[5]), atof(argv[6]), atoi(argv[7]),
                        argv[8]);
    if (cmd == "gmres" && argc == 3) {
      // the GMRES settings a problem file leaves (reference defaults where absent or 0)
      Input in;
      in.openFile(argv[2]);
      GlobalIterativeSolver* g = nullptr;
      in.readProblemSolver(g, 0);
      auto* gm = dynamic_cast<GlobalIterativeSolverGMRES*>(g);
      std::printf("tol %.17g maxiter %u verbose %d\n", gm->getTol(), gm->getMaxIter(), gm->getVerbose() ? 1 : 0);
      delete g;
      return 0;
    }
    if (cmd == "rhs" && argc >= 5) {
      RHSSrcPts r;
      r.setEpsilon(atof(argv[2]));
      for (int k = 3; k + 1 < argc; k += 2) r.addSrcPt({atof(argv[k]), atof(argv[k + 1])});
      double x, y;
      while (std::cin >> x >> y) std::printf("%.17g\n", r.eval({x, y}).real());
      return 0;
    }
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 2;
  }
  std::cerr << "bad arguments" << std::endl;
  return 1;
}
