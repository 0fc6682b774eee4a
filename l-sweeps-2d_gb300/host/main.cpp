// lsweeps_gb300_main <problem file>: the reference's driver (main.cpp) on the
// GPU library: every problem of the file is read, factorised, solved and
// written; errors print their message and exit with status 1.
#include <iostream>

#include "lsweeps_host.hpp"

int main(int argc, char** argv) {
  if (argc < 2) {
    std::cerr << "usage: " << argv[0] << " <problem file>" << std::endl;
    return 1;
  }
  try {
    Input input;
    input.openFile(argv[1]);
    for (UInt p = 0; p < input.getNumProblems(); ++p) {
      Problem prob;
      prob.read(input, p);
      prob.solve();
    }
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}
