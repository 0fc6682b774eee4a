// A driver in the style of the reference's main.cpp / src/Problem.cpp that
// uses only the abstract plugin classes: compiled and linked by the CPU tests
// (running it needs a GPU).
#include <iostream>
#include <memory>

#include "lsweeps_host.hpp"

static void solve_with(const Assembler& assembler, const LocalLinearSolver& solver, DD& dd, GlobalIterativeSolver& gs,
                       const RHS& rhs, Output& out) {
  dd.factorize();
  std::vector<ComplexVector> b, x;
  dd.assembleRHS(&rhs, b);
  gs.setParent(&dd);
  gs.solve(b, x);
  // per-cell work through the Subdomain interface
  for (UInt c = 0; c < dd.getNCells(); ++c) {
    Subdomain* s = dd.getCell(c);
    std::vector<UIntVector> sets;
    s->getIndexSets("LeftRight", false, sets);
    std::vector<ComplexVector> eq;
    s->getEquivalentSources("Left", false, false, ComplexVector(sets[1].size()), ComplexVector(sets[2].size()), eq);
  }
  std::unique_ptr<DD> twin(dd.copy());
  std::unique_ptr<Assembler> a2(assembler.copy());
  std::unique_ptr<LocalLinearSolver> s2(solver.copy());
  out.setDD(&dd);
  out.setVals(x);
  out.print();
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::cerr << "usage: abstract_driver <output name>" << std::endl;
    return 1;
  }
  try {
    FunctionConstant m;
    m.setVal(1.0);
    std::unique_ptr<PML> pml(new PMLCubic2D);
    static_cast<PMLCubic2D*>(pml.get())->setAbsorptionCoeff(std::log(60.0));
    pml->setWidth(4.0 / 47.0);
    std::unique_ptr<AssemblerHelmholtz> asmb(new AssemblerHelmholtz2DFD);
    asmb->setPML(pml.get());
    asmb->setOmega(60.0);
    asmb->setM(&m);
    asmb->setOrder(2);
    std::unique_ptr<LocalLinearSolver> solver(new LocalLinearSolverCUDA);
    std::unique_ptr<DDCheckerboard> dd(new DDCheckerboard);
    dd->setUp(asmb.get(), solver.get(), {{0.0, 1.0}, {0.0, 1.0}}, {2, 2}, {23, 23});
    std::unique_ptr<GlobalIterativeSolver> gs(new GlobalIterativeSolverGMRES);
    RHSSrcPts rhs;
    rhs.setEpsilon(dd->getMeshSize());
    rhs.addSrcPt({0.5, 0.5});
    std::unique_ptr<Output> out(new OutputVTK);
    out->setFilename(argv[1]);
    solve_with(*asmb, *solver, *dd, *gs, rhs, *out);
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}
