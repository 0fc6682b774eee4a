/* C++ host layer with the reference's plugin API over the C ABI of
 * liblsweeps_gb300.so (lsweeps.h).
 *
 * The classes keep the names, virtuals and call pattern of the reference
 * (L-Sweeps-2D, the headers under include/) so that its driver code (main.cpp,
 * src/Problem.cpp) compiles against them: a DDCheckerboard is set up from an
 * AssemblerHelmholtz2DFD (omega, PMLCubic2D, squared slowness Function), a
 * LocalLinearSolver prototype (LocalLinearSolverCUDA beside the reference's
 * LocalLinearSolverEigenSparseLU), the domain and the cell counts; a
 * GlobalIterativeSolverGMRES solves on it; OutputVTK writes the wavefield.
 * Input reads the reference's libconfig problem files (the subset the
 * reference reads, src/Input.cpp) with a parser of its own, since libconfig++
 * is not a dependency.
 *
 * Differences from the reference, by design:
 *  - one process, one GPU: no MPI communicator; DD::getComm is absent and the
 *    communicate*Traces calls are no-ops (every cell lives on the device);
 *  - Eigen is absent: ComplexVector is std::vector<std::complex<double>> and
 *    ComplexSparseMatrix a compressed-row matrix of this header (the library
 *    assembles and factorises every cell itself on the device);
 *  - errors raise lsw_host_error (a std::runtime_error) instead of printing
 *    and calling exit(1); the driver (Problem, lsweeps_gb300_main) prints the
 *    message and exits with status 1 as the reference does;
 *  - the reference's FunctionCSV::getMinReal is read by Input before
 *    setDomain has computed it (an uninitialised value); here setFile
 *    already records the minimum over the whole file.
 */
#pragma once

#include <complex>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "lsweeps.h"

// ---- types (include/typedef.h of the reference) --------------------------------
typedef double Double;
typedef unsigned int UInt;
typedef std::complex<double> Complex;
typedef std::vector<double> DoubleVector;
typedef std::vector<UInt> UIntVector;
typedef std::vector<Complex> ComplexVector;

// Compressed-row complex sparse matrix (the reference's ComplexSparseMatrix is
// an Eigen::SparseMatrix, include/typedef.h:64-73).  The sweeps never use it:
// the GPU assembles and factorises every cell itself; it is what
// Subdomain/Assembler::assembleSystemMatrix return.
struct ComplexSparseMatrix {
  UInt rows = 0, cols = 0;
  std::vector<UInt> outer;   // rows + 1 row offsets into inner / vals
  std::vector<UInt> inner;   // column of each stored entry, ascending per row
  std::vector<Complex> vals;
  UInt nonZeros() const { return (UInt)vals.size(); }
  Complex coeff(UInt r, UInt c) const;           // 0 where nothing is stored
  void multiply(const ComplexVector& x, ComplexVector& y) const;   // y = A x
};

struct lsw_host_error : std::runtime_error {
  explicit lsw_host_error(const std::string& m) : std::runtime_error(m) {}
};

// ---- Function (include/Function.h) ---------------------------------------------
class Function {
 public:
  virtual ~Function() {}
  virtual Function* copy() const = 0;
  virtual void clearCache() const = 0;
  virtual Double getMinReal() const = 0;
  virtual Double getMaxReal() const = 0;
  virtual Double getMinImag() const = 0;
  virtual Double getMaxImag() const = 0;
  virtual void setDomain(const std::vector<DoubleVector>& dom) const = 0;
  virtual void getDomain(std::vector<DoubleVector>& res) const = 0;
  virtual Complex eval(DoubleVector x) const = 0;
};

// include/FunctionConstant.h
class FunctionConstant : public Function {
 public:
  FunctionConstant() : mVal(1.0) {}
  void setVal(Complex v) { mVal = v; }
  Function* copy() const override { return new FunctionConstant(*this); }
  void clearCache() const override {}
  Double getMinReal() const override { return mVal.real(); }
  Double getMaxReal() const override { return mVal.real(); }
  Double getMinImag() const override { return mVal.imag(); }
  Double getMaxImag() const override { return mVal.imag(); }
  void setDomain(const std::vector<DoubleVector>& dom) const override { mDom = dom; }
  void getDomain(std::vector<DoubleVector>& res) const override { res = mDom; }
  Complex eval(DoubleVector) const override { return mVal; }

 private:
  Complex mVal;
  mutable std::vector<DoubleVector> mDom;
};

// include/FunctionCSV.h: velocity per file cell (row 0 = top), squared
// slowness 1/c^2 sampled piecewise constant (src/FunctionCSV.cpp:46-236)
class FunctionCSV : public Function {
 public:
  void setFile(const std::string& filename, const std::vector<DoubleVector>& fileDom);
  Function* copy() const override { return new FunctionCSV(*this); }
  void clearCache() const override;
  Double getMinReal() const override { return mMinReal; }
  Double getMaxReal() const override { return mMaxReal; }
  Double getMinImag() const override { return mMinImag; }
  Double getMaxImag() const override { return mMaxImag; }
  void setDomain(const std::vector<DoubleVector>& dom) const override;
  void getDomain(std::vector<DoubleVector>& res) const override { res = mDom; }
  Complex eval(DoubleVector x) const override;
  UIntVector fileSize() const { return mFileN; }

 private:
  std::string mFilename;
  std::vector<DoubleVector> mFileDom;
  UIntVector mFileN{0, 0};   // rows, columns
  DoubleVector mH{0.0, 0.0};
  std::vector<float> mFile;  // velocities as read (rows x columns)
  mutable std::vector<DoubleVector> mDom, mDomA;
  mutable UInt mRow0 = 0, mCol0 = 0, mRows = 0, mCols = 0;
  mutable std::vector<Complex> mA;   // squared slowness of the window
  mutable Double mMinReal = 0, mMaxReal = 0, mMinImag = 0, mMaxImag = 0;
  mutable bool mDomSet = false;
};

// ---- RHS (include/RHS.h, include/RHSSrcPts.h) -----------------------------------
class RHS {
 public:
  virtual ~RHS() {}
  virtual RHS* copy() const = 0;
  virtual Complex eval(DoubleVector x) const = 0;
};

class RHSSrcPts : public RHS {
 public:
  RHS* copy() const override { return new RHSSrcPts(*this); }
  void clearSrcPts() { mSourcePts.clear(); }
  void setEpsilon(Double eps) { mEps = eps; }
  void setSrcPts(const std::vector<DoubleVector>& pts) { mSourcePts = pts; }
  void addSrcPt(const DoubleVector& p) { mSourcePts.push_back(p); }
  void getSrcPts(std::vector<DoubleVector>& res) const { res = mSourcePts; }
  Double getEpsilon() const { return mEps; }
  // sum over the sources of 1/(pi eps^2) exp(-|x - x0|^2 / eps^2) (src/RHSSrcPts.cpp:87-112)
  Complex eval(DoubleVector x) const override;

 private:
  std::vector<DoubleVector> mSourcePts;
  Double mEps = 0.0;
};

// ---- PML (include/PML.h, include/PMLCubic2D.h) ---------------------------------
class AssemblerHelmholtz;

// Complex stretching of the Helmholtz operator in an absorbing layer of width
// getWidth() around the interior domain (setDomain); src/PML.cpp.
class PML {
 public:
  virtual ~PML() {}
  virtual PML* copy() const = 0;
  void setParent(const AssemblerHelmholtz* parent) { mParent = parent; }
  virtual void setWidth(Double pmlWidth);
  virtual Double getWidth() const { return mPMLWidth; }
  virtual void setDomain(const std::vector<DoubleVector>& domain);   // the interior domain
  virtual std::vector<DoubleVector> getDomain() const { return mIntDomain; }
  // coefficients at a point of the computational domain (interior + layer)
  virtual ComplexVector getDiffusionCoefficient(DoubleVector x) const = 0;
  virtual ComplexVector getConvectionCoefficient(DoubleVector x) const = 0;
  virtual Complex getReactionCoefficient(DoubleVector x) const = 0;
  virtual Complex getSourceCoefficient(DoubleVector x) const = 0;

 protected:
  const AssemblerHelmholtz* mParent = nullptr;
  std::vector<DoubleVector> mCompDomain, mIntDomain;
  Double mPMLWidth = 0.0;
};

// Cubic profile sigma = C (d / delta)^3, alpha = 1 / (1 + i sigma): diffusion
// (alpha1^2, alpha2^2), convection (alpha1' alpha1, alpha2' alpha2),
// reaction and source 1 (src/PMLCubic2D.cpp:35-236).  C = ln omega when read
// from a problem file (Input.cpp:836).
class PMLCubic2D : public PML {
 public:
  PML* copy() const override { return new PMLCubic2D(*this); }
  void setAbsorptionCoeff(Double C) { mC = C; }
  Double getAbsorptionCoeff() const { return mC; }
  ComplexVector getDiffusionCoefficient(DoubleVector x) const override;
  ComplexVector getConvectionCoefficient(DoubleVector x) const override;
  Complex getReactionCoefficient(DoubleVector) const override { return 1.0; }
  Complex getSourceCoefficient(DoubleVector) const override { return 1.0; }

 private:
  // sigma and its derivative along direction d at coordinate v
  void sigma(Double v, int d, Double& s, Double& ds) const;
  Double mC = 0.0;
};

// ---- assemblers (include/Assembler.h, AssemblerHelmholtz.h, AssemblerHelmholtz2DFD.h)
class RHS;

// A discretisation on one rectangle (src/Assembler*.cpp): the DOF points, the
// non-DOF (zero Dirichlet boundary) points, the elements, the right-hand side
// and the system matrix.
class Assembler {
 public:
  virtual ~Assembler() {}
  virtual Assembler* copy() const = 0;
  virtual void setDomain(const std::vector<DoubleVector>& dom) = 0;
  virtual std::vector<DoubleVector> getDomain() const = 0;
  virtual void setN(const UIntVector& n) = 0;
  virtual UIntVector getN() const = 0;
  virtual void setOrder(UInt order) = 0;
  virtual UInt getOrder() const = 0;
  virtual Double getMeshSize() const = 0;
  virtual UInt getDim() const = 0;
  virtual void getDOFPts(std::vector<DoubleVector>& res) const = 0;
  virtual void getNonDOFPhysPts(std::vector<DoubleVector>& res) const = 0;
  virtual void getElPhysPtIndices(UInt index, UIntVector& elPts) const = 0;
  virtual void expandDOFValsToPhysVals(ComplexVector& res) const = 0;
  virtual void assembleRHS(const RHS* rhs, ComplexVector& res) const = 0;
  virtual void assembleSystemMatrix(ComplexSparseMatrix& res) const = 0;
  virtual UInt getNEls() const = 0;
};

// The Helmholtz problem -div(D grad u) - b.grad u - omega^2 m u = f with a PML
// (include/AssemblerHelmholtz.h): owns copies of its PML and squared slowness.
class AssemblerHelmholtz : public Assembler {
 public:
  AssemblerHelmholtz() {}
  AssemblerHelmholtz(const AssemblerHelmholtz& o);
  AssemblerHelmholtz& operator=(const AssemblerHelmholtz& o);
  void setPML(const PML* pml);          // keeps a copy whose parent is this assembler
  void setM(const Function* m);         // keeps a copy
  void setOmega(Double omega) { mOmega = omega; }
  const Function* getM() const { return mM.get(); }
  Double getOmega() const { return mOmega; }
  const PML* getPML() const { return mPML.get(); }

 protected:
  std::unique_ptr<PML> mPML;
  std::unique_ptr<Function> mM;
  Double mOmega = 0.0;
};

// Second-order finite differences on a uniform grid of the computational
// domain (interior + PML) with zero Dirichlet values outside
// (src/AssemblerHelmholtz2DFD.cpp): DOF (i, j), i along x, j along y, index
// i (ny - 1) + j; the PML width is rounded to whole elements by setN.
// Order = 2 only (the 5-point stencil of every supported configuration).
class AssemblerHelmholtz2DFD : public AssemblerHelmholtz {
 public:
  Assembler* copy() const override { return new AssemblerHelmholtz2DFD(*this); }
  void setDomain(const std::vector<DoubleVector>& dom) override;
  std::vector<DoubleVector> getDomain() const override { return mIntDomain; }
  void setN(const UIntVector& n) override;
  UIntVector getN() const override { return mN; }
  void setOrder(UInt order) override { mOrder = order; }
  UInt getOrder() const override { return mOrder; }
  Double getMeshSize() const override;
  UInt getDim() const override { return 2; }
  void getDOFPts(std::vector<DoubleVector>& res) const override;
  void getNonDOFPhysPts(std::vector<DoubleVector>& res) const override;
  void getElPhysPtIndices(UInt index, UIntVector& res) const override;
  void expandDOFValsToPhysVals(ComplexVector& res) const override;
  void assembleRHS(const RHS* rhs, ComplexVector& res) const override;
  void assembleSystemMatrix(ComplexSparseMatrix& res) const override;
  UInt getNEls() const override { return mN.empty() ? 0 : mN[0] * mN[1]; }
  // the computational domain (interior grown by the rounded PML width)
  std::vector<DoubleVector> getCompDomain() const { return mCompDomain; }
  // assembleSystemMatrix with the squared slowness given per DOF (DOF order)
  // instead of evaluated from getM()
  void assembleSystemMatrix(const std::vector<Double>& mDof, ComplexSparseMatrix& res) const;

 private:
  std::vector<DoubleVector> mIntDomain, mCompDomain;
  UIntVector mN;
  UInt mOrder = 2;
};

// ---- local solvers (include/LocalLinearSolver.h) -------------------------------
class LocalLinearSolver {
 public:
  virtual ~LocalLinearSolver() {}
  virtual LocalLinearSolver* copy() const = 0;
  virtual void setMatrix(ComplexSparseMatrix* A) = 0;
  virtual void factorize() = 0;
  virtual void solve(ComplexVector& b, ComplexVector& res) const = 0;
};

// One cell's solves on the GPU.  The DD binds every copy of the prototype
// to its context and cell; factorize() is idempotent and factorises every
// cell of the problem in one batched launch (lsw_factorize); solve() copies
// the cell vector (local DOF order i*ny + j) to the device and back around
// lsw_local_solve.
class LocalLinearSolverCUDA : public LocalLinearSolver {
 public:
  LocalLinearSolver* copy() const override { return new LocalLinearSolverCUDA(*this); }
  void setMatrix(ComplexSparseMatrix* A) override { mA = A; }
  void factorize() override;
  void solve(ComplexVector& b, ComplexVector& res) const override;
  void bind(lsw_ctx* ctx, int cell) { mCtx = ctx; mCell = cell; }

 private:
  ComplexSparseMatrix* mA = nullptr;
  lsw_ctx* mCtx = nullptr;
  int mCell = -1;
};

// ---- subdomains (include/Subdomain.h, include/SubdomainStructured.h) ------------
// One cell of the checkerboard (include/Subdomain.h:20-227): its
// discretisation, local solver and trace index sets.  Trace types are
// "LeftRight" / "UpDown" (getIndexSets: seven sets along that direction,
// [1], [2] = trace0, trace1 and [4], [5] = traceN, traceNP lines, [0], [3],
// [6] the volume around them), "Left", "Right", "Bottom", "Top" (straight
// equivalent sources) and "BottomLeft", "BottomRight", "TopRight", "TopLeft"
// (L-shaped traces).
class Subdomain {
 public:
  virtual ~Subdomain() {}
  virtual Subdomain* copy() const = 0;
  virtual void clearCache() const = 0;
  virtual void setLimits(const std::vector<DoubleVector>& lims) = 0;
  virtual void setLocalLinearSolver(const LocalLinearSolver* solver) = 0;
  virtual void setRowIndex(UInt I) = 0;
  virtual void setColIndex(UInt J) = 0;
  virtual UInt getRowIndex() const = 0;
  virtual UInt getColIndex() const = 0;
  virtual UInt getSize() const = 0;
  virtual Double getMeshSize() const = 0;
  virtual UInt getNEls() const = 0;
  virtual UInt getDim() const = 0;
  virtual void getDOFPts(std::vector<DoubleVector>& res) const = 0;
  virtual void getPhysPts(std::vector<DoubleVector>& res) const = 0;
  virtual void getElPhysPtIndices(UInt elIndex, UIntVector& res) const = 0;
  virtual void expandDOFValsToPhysVals(ComplexVector& res) const = 0;
  virtual void assembleRHS(const RHS* rhs, ComplexVector& res) const = 0;
  virtual void assembleSystemMatrix(ComplexSparseMatrix& res) const = 0;
  virtual void assembleSystemMatrix() const = 0;
  virtual void factorize() = 0;
  virtual void solve(ComplexVector& x, ComplexVector& res) const = 0;
  virtual void getIndexSets(std::string traceType, bool shifted, std::vector<UIntVector>& res) const = 0;
  virtual void getElIndexSets(std::string traceType, bool shifted, std::vector<UIntVector>& res) const = 0;
  virtual void applySystemMatrix(const ComplexVector& x, ComplexVector& res) const = 0;
  virtual void getLTraceIndexSets(std::string traceType, bool shiftedLR, bool shiftedUD,
                                  std::vector<UIntVector>& res) const = 0;
  virtual void getEquivalentSources(std::string traceType, bool shiftedLR, bool shiftedUD, ComplexVector vals0,
                                    ComplexVector vals1, std::vector<ComplexVector>& res) const = 0;
  virtual void extractLTraces(std::string LTraceType, bool shiftedLR, bool shiftedUD, ComplexVector valsLR0,
                              ComplexVector valsLR1, ComplexVector valsUD0, ComplexVector valsUD1,
                              std::vector<ComplexVector>& res) const = 0;
};

// A cell of the library's checkerboard (src/SubdomainStructured.cpp).  Its
// geometry comes from the library (lsw_cell_info: the reference's trace
// limits evaluated on the integer grid), its operator is assembled on the host
// on demand (the same 5-point PML stencil and squared slowness as the device),
// and solve/factorize go to the GPU through the bound LocalLinearSolverCUDA.
// The trace functions run on the host; the sweeps themselves never call them
// (the GPU builds equivalent sources and traces inside its kernels).
class SubdomainStructured : public Subdomain {
 public:
  // mGrid: squared slowness on the global n_dof x n_dof DOF grid (x-major),
  // shared by the cells of one decomposition
  SubdomainStructured(lsw_ctx* ctx, int cell, const lsw_cell_info& info, const LocalLinearSolver* proto, Double h,
                      Double ax, Double ay, int pml, Double omega, std::shared_ptr<const std::vector<double>> mGrid,
                      int nDof);
  SubdomainStructured(const SubdomainStructured& o);
  Subdomain* copy() const override { return new SubdomainStructured(*this); }
  void clearCache() const override { mA.reset(); }
  // the trace limits are the library's (fixed by the decomposition); the
  // values given are kept and returned by getLimits only
  void setLimits(const std::vector<DoubleVector>& lims) override { mLims = lims; }
  std::vector<DoubleVector> getLimits() const { return mLims; }
  void setLocalLinearSolver(const LocalLinearSolver* solver) override;
  void setRowIndex(UInt I) override { mInfo.I = (int)I; }
  void setColIndex(UInt J) override { mInfo.J = (int)J; }
  UInt getRowIndex() const override { return (UInt)mInfo.I; }
  UInt getColIndex() const override { return (UInt)mInfo.J; }
  UInt getSize() const override { return (UInt)(mInfo.nx * mInfo.ny); }
  Double getMeshSize() const override { return mH; }
  UInt getNEls() const override { return (UInt)((mInfo.nx + 1) * (mInfo.ny + 1)); }
  UInt getDim() const override { return 2; }
  void getDOFPts(std::vector<DoubleVector>& res) const override;
  void getPhysPts(std::vector<DoubleVector>& res) const override;   // DOF points, then the boundary points
  void getElPhysPtIndices(UInt elIndex, UIntVector& res) const override;
  void expandDOFValsToPhysVals(ComplexVector& res) const override;
  void assembleRHS(const RHS* rhs, ComplexVector& res) const override;
  void assembleSystemMatrix(ComplexSparseMatrix& res) const override;
  void assembleSystemMatrix() const override;   // cache the matrix for the trace functions
  void factorize() override { mSolver->factorize(); }
  void solve(ComplexVector& b, ComplexVector& res) const override { mSolver->solve(b, res); }
  void getIndexSets(std::string traceType, bool shifted, std::vector<UIntVector>& res) const override;
  void getElIndexSets(std::string traceType, bool shifted, std::vector<UIntVector>& res) const override;
  void applySystemMatrix(const ComplexVector& x, ComplexVector& res) const override;
  void getLTraceIndexSets(std::string traceType, bool shiftedLR, bool shiftedUD,
                          std::vector<UIntVector>& res) const override;
  void getEquivalentSources(std::string traceType, bool shiftedLR, bool shiftedUD, ComplexVector vals0,
                            ComplexVector vals1, std::vector<ComplexVector>& res) const override;
  void extractLTraces(std::string LTraceType, bool shiftedLR, bool shiftedUD, ComplexVector valsLR0,
                      ComplexVector valsLR1, ComplexVector valsUD0, ComplexVector valsUD1,
                      std::vector<ComplexVector>& res) const override;

  const lsw_cell_info& info() const { return mInfo; }
  LocalLinearSolver* getLocalSolver() const { return mSolver.get(); }
  // the cell's assembler: interior domain and element counts set, PMLCubic2D
  // with C = ln omega
  const AssemblerHelmholtz2DFD& assembler() const { return mAsm; }

 private:
  const ComplexSparseMatrix& matrix() const;
  // the trace0 and trace1 index sets of a straight or L-shaped trace type
  void traceSets(const std::string& traceType, bool shiftedLR, bool shiftedUD, UIntVector& t0, UIntVector& t1) const;
  lsw_ctx* mCtx = nullptr;
  int mCell = -1;
  lsw_cell_info mInfo;
  std::unique_ptr<LocalLinearSolver> mSolver;
  Double mH, mAx, mAy;
  int mPml;
  AssemblerHelmholtz2DFD mAsm;
  std::shared_ptr<const std::vector<double>> mGrid;
  int mNDof = 0;
  std::vector<DoubleVector> mLims;
  mutable std::shared_ptr<ComplexSparseMatrix> mA;
};

// ---- domain decomposition (include/DD.h, include/DDCheckerboard.h) --------------
class DD {
 public:
  virtual ~DD() {}
  virtual DD* copy() const = 0;
  virtual void factorize() = 0;
  virtual void assembleRHS(const RHS* rhs, std::vector<ComplexVector>& res) const = 0;
  virtual void applyPrecond(const std::vector<ComplexVector>& x, std::vector<ComplexVector>& res) const = 0;
  virtual void applySystemMatrix(const std::vector<ComplexVector>& x, std::vector<ComplexVector>& res) const = 0;
  virtual UInt getDim() const = 0;
  virtual Double getMeshSize() const = 0;
  virtual void expand(const std::vector<ComplexVector>& x, std::vector<ComplexVector>& res, bool shiftedLR = false,
                      bool shiftedUD = false) const = 0;
  virtual void communicateBL2TRTraces(std::vector<ComplexVector>& xEx, bool shifted = false) const = 0;
  virtual void communicateTR2BLTraces(std::vector<ComplexVector>& xEx, bool shifted = false) const = 0;
  virtual UInt getNCells() const = 0;
  virtual Subdomain* getCell(UInt i) const = 0;
};

// The checkerboard of NCells x NCells cells of NX x NX interior elements on a
// square domain; every cell's owned DOFs (the reference's mValsToKeep sets,
// src/DDCheckerboard.cpp:453-634) are one ComplexVector in cell-local order
// (i over the owned x-range, then j over the owned y-range).
class DDCheckerboard : public DD {
 public:
  DDCheckerboard() {}
  ~DDCheckerboard() override;
  DDCheckerboard(const DDCheckerboard&) = delete;
  DDCheckerboard& operator=(const DDCheckerboard&) = delete;
  // src/DDCheckerboard.cpp:87-645; precision LSW_PREC_C128 reproduces the
  // reference's all-FP64 arithmetic, LSW_PREC_C64 the mixed-precision path
  void setUp(const Assembler* assembler, const LocalLinearSolver* solver, const std::vector<DoubleVector>& domain,
             const UIntVector& nCells, const UIntVector& nElsInCell, lsw_precision precision = LSW_PREC_C128,
             int device = 0);
  // a decomposition of its own (its own device context): set up again from the
  // same assembler, solver prototype, domain and counts, and factorised if this
  // one is (include/DD.h:31)
  DD* copy() const override;
  void factorize() override;
  void assembleRHS(const RHS* rhs, std::vector<ComplexVector>& res) const override;
  void applyPrecond(const std::vector<ComplexVector>& x, std::vector<ComplexVector>& res) const override;
  void applySystemMatrix(const std::vector<ComplexVector>& x, std::vector<ComplexVector>& res) const override;
  UInt getDim() const override { return 2; }
  Double getMeshSize() const override { return mH; }
  // every cell's full DOF vector (owned values and their overlap with the neighbours)
  void expand(const std::vector<ComplexVector>& x, std::vector<ComplexVector>& res, bool shiftedLR = false,
              bool shiftedUD = false) const override;
  void communicateBL2TRTraces(std::vector<ComplexVector>&, bool = false) const override {}
  void communicateTR2BLTraces(std::vector<ComplexVector>&, bool = false) const override {}
  UInt getNCells() const override { return (UInt)mCells.size(); }
  Subdomain* getCell(UInt i) const override { return mCells.at(i).get(); }
  SubdomainStructured* getCellStructured(UInt i) const { return mCells.at(i).get(); }

  // global <-> per-cell owned vectors (global DOFs x-major, y fastest)
  void toGlobal(const std::vector<ComplexVector>& cells, ComplexVector& g) const;
  void toCells(const ComplexVector& g, std::vector<ComplexVector>& cells) const;
  lsw_ctx* ctx() const { return mCtx; }
  int nDof() const { return mNDof; }
  int pml() const { return mPml; }
  const std::vector<DoubleVector>& domain() const { return mDomain; }

 private:
  void* devBuffers(size_t bytes) const;   // two device vectors of `bytes`, kept for reuse
  lsw_ctx* mCtx = nullptr;
  // the setUp arguments, for copy()
  std::unique_ptr<Assembler> mAssembler;
  std::unique_ptr<LocalLinearSolver> mProto;
  UIntVector mNCells, mNEls;
  lsw_precision mPrec = LSW_PREC_C128;
  int mDevice = 0;
  bool mFactorized = false;
  std::vector<std::unique_ptr<SubdomainStructured>> mCells;
  std::vector<DoubleVector> mDomain;
  mutable void* mBuf = nullptr;
  mutable size_t mBufBytes = 0;
  Double mH = 0.0;
  int mNDof = 0, mPml = 0, mN = 0, mM = 0;
};

// ---- global solvers (include/GlobalIterativeSolver*.h) ---------------------------
class GlobalIterativeSolver {
 public:
  virtual ~GlobalIterativeSolver() {}
  void setParent(const DD* parent) { mParent = parent; }
  virtual GlobalIterativeSolver* copy() const = 0;
  virtual void solve(const std::vector<ComplexVector>& rhs, std::vector<ComplexVector>& res) const = 0;

 protected:
  const DD* mParent = nullptr;
};

// LSW_GMRES_REFERENCE reproduces GlobalIterativeSolverGMRES::solve
// (src/GlobalIterativeSolverGMRES.cpp:65-203, no restart, left
// preconditioning); LSW_GMRES_FLEXIBLE is restarted FGMRES with the true
// residual as stopping criterion.
class GlobalIterativeSolverGMRES : public GlobalIterativeSolver {
 public:
  GlobalIterativeSolver* copy() const override { return new GlobalIterativeSolverGMRES(*this); }
  void setTol(Double tol) { mTol = tol; }
  void setMaxIter(UInt maxIter) { mMaxIter = maxIter; }
  Double getTol() const { return mTol; }
  UInt getMaxIter() const { return mMaxIter; }
  bool getVerbose() const { return mVerbose; }
  void setVerbose(bool v) { mVerbose = v; }
  void setMode(lsw_gmres_mode m) { mMode = m; }
  void setRestart(UInt r) { mRestart = r; }
  void getLog(std::vector<Double>& res) const { res = mLog; }
  const lsw_gmres_report& report() const { return mRep; }
  void solve(const std::vector<ComplexVector>& rhs, std::vector<ComplexVector>& res) const override;

 private:
  // the reference's defaults (GlobalIterativeSolverGMRES.cpp:9)
  Double mTol = 1e-6;
  UInt mMaxIter = 40;
  UInt mRestart = 0;   // 0: no restart (max_iter)
  bool mVerbose = true;
  lsw_gmres_mode mMode = LSW_GMRES_REFERENCE;
  mutable std::vector<Double> mLog;
  mutable lsw_gmres_report mRep{};
};

// ---- output (include/Output.h, include/OutputVTK.h) ------------------------------
class Output {
 public:
  virtual ~Output() {}
  virtual Output* copy() const = 0;
  void setDD(const DD* dd) { mDD = dd; }
  void setFilename(const std::string& name) { mFilename = name; }
  std::string getFilename() const { return mFilename; }
  virtual void print() const = 0;
  virtual void setVals(const std::vector<ComplexVector>& vals) const = 0;

 protected:
  const DD* mDD = nullptr;
  std::string mFilename;
};

// Legacy ASCII VTK, unstructured grid of linear quads over the physical
// domain (the PML is left out), point data wavefield_re and wavefield_im
// (the layout of OutputVTK::print2D, src/OutputVTK.cpp:310-358); written to
// <filename>.vtk.  The reference emits every cell's points separately (so
// points on cell interfaces repeat); here every grid point appears once.
class OutputVTK : public Output {
 public:
  Output* copy() const override { return new OutputVTK(*this); }
  void print() const override;
  void setVals(const std::vector<ComplexVector>& vals) const override;
  ComplexVector getGlobalVals() const { return mVals; }

 private:
  mutable ComplexVector mVals;   // global DOF values
};

// ---- input (include/Input.h) -----------------------------------------------------
// A parsed libconfig setting: group, list, array or scalar.
struct CfgSetting {
  enum Kind { GROUP, LIST, ARRAY, INT, FLOAT, BOOL, STRING } kind = GROUP;
  std::string name;
  long long i = 0;
  double f = 0.0;
  bool b = false;
  std::string s;
  std::vector<CfgSetting> children;

  bool exists(const std::string& n) const;
  const CfgSetting& operator[](const std::string& n) const;
  const CfgSetting& operator[](int idx) const;
  int getLength() const { return (int)children.size(); }
  bool lookupValue(const std::string& n, std::string& v) const;
  bool lookupValue(const std::string& n, double& v) const;
  bool lookupValue(const std::string& n, UInt& v) const;
  bool lookupValue(const std::string& n, int& v) const;
  bool lookupValue(const std::string& n, bool& v) const;
};
// parse a libconfig file or text (groups, lists, arrays, scalars, comments)
CfgSetting cfg_parse_file(const std::string& path);
CfgSetting cfg_parse_text(const std::string& text);

class Input {
 public:
  void openFile(const std::string& name);
  UInt getNumProblems() const;
  void readProblemDD(DD*& dd, UInt probID) const;
  void readProblemRHS(const DD* dd, RHS*& rhs, UInt probID) const;
  void readProblemSolver(GlobalIterativeSolver*& solver, UInt probID) const;
  void readProblemOutput(Output*& output, UInt probID) const;
  const CfgSetting& root() const { return mRoot; }

 private:
  void readCheckerboardDD(UInt DDID, DD*& dd) const;
  void readDomain(const std::string& name, UInt dim, std::vector<DoubleVector>& dom) const;
  Function* readSquaredSlowness(const std::string& name) const;
  CfgSetting mRoot;
  bool mOpened = false;
  std::string mDir;   // directory of the problem file (relative CSV paths)
};

// ---- problem (include/Problem.h) -------------------------------------------------
class Problem {
 public:
  Problem() {}
  Problem(const Problem&) = delete;
  Problem& operator=(const Problem&) = delete;
  ~Problem();
  void read(const Input& input, UInt probID);
  // factorise, assemble the right-hand side, solve, write the output
  // (src/Problem.cpp:94-158, with its timing lines on stdout)
  void solve() const;
  DD* dd() const { return mDD; }
  GlobalIterativeSolver* solver() const { return mSolver; }
  Output* output() const { return mOutput; }

 private:
  DD* mDD = nullptr;
  RHS* mRHS = nullptr;
  GlobalIterativeSolver* mSolver = nullptr;
  Output* mOutput = nullptr;
};
