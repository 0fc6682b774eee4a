// Probe of the C++ host layer for the tests: prints what the classes compute
// so that the Python tests can check it.
//   host_probe parse <problem file>                      canonical dump of the settings
//   host_probe csv <csv> ax bx ay by  dx0 dx1 dy0 dy1    reads "x y" lines on stdin,
//                                                        prints Re eval per point
//   host_probe rhs eps x0 y0 [x1 y1 ...]                 reads "x y" lines, prints the RHS
#include <cstdio>
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
