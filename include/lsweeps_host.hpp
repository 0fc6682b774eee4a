/* C++ host layer with the reference's plugin API over the C ABI of
 * liblsweeps_gb300.so (lsweeps.h).
 *
 * The classes keep the names, virtuals and call pattern of the reference
 * (L-Sweeps-2D, include/*.h) so that its driver code (main.cpp,
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
 *    ComplexSparseMatrix is opaque (the library assembles every cell itself);
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
struct ComplexSparseMatrix;   // opaque: cell matrices live on the device

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

// ---- PML and assembler (include/PMLCubic2D.h, include/AssemblerHelmholtz2DFD.h) --
// Configuration holders: the operator itself is assembled on the device
// (sigma = C (d/delta)^3 with C = ln omega, the 5-point stencil and the
// PML stretching of src/AssemblerHelmholtz2DFD.cpp:371-457).
class PMLCubic2D {
 public:
  void setAbsorptionCoeff(Double C) { mC = C; }
  void setWidth(Double w) { mWidth = w; }
  Double getWidth() const { return mWidth; }
  Double getAbsorptionCoeff() const { return mC; }

 private:
  Double mC = 0.0, mWidth = 0.0;
};

class AssemblerHelmholtz2DFD {
 public:
  AssemblerHelmholtz2DFD() {}
  AssemblerHelmholtz2DFD(const AssemblerHelmholtz2DFD& o);
  AssemblerHelmholtz2DFD& operator=(const AssemblerHelmholtz2DFD& o);
  AssemblerHelmholtz2DFD* copy() const { return new AssemblerHelmholtz2DFD(*this); }
  void setPML(const PMLCubic2D* pml) { mPML = *pml; }
  void setOmega(Double omega) { mOmega = omega; }
  void setM(const Function* m) { mM.reset(m ? m->copy() : nullptr); }
  void setOrder(UInt order) { mOrder = order; }
  Double getOmega() const { return mOmega; }
  UInt getOrder() const { return mOrder; }
  const PMLCubic2D& getPML() const { return mPML; }
  const Function* getM() const { return mM.get(); }

 private:
  PMLCubic2D mPML;
  Double mOmega = 0.0;
  UInt mOrder = 2;
  std::unique_ptr<Function> mM;
};
typedef AssemblerHelmholtz2DFD Assembler;

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
class SubdomainStructured {
 public:
  SubdomainStructured(lsw_ctx* ctx, int cell, const lsw_cell_info& info, const LocalLinearSolver* proto,
                      Double h, Double ax, Double ay, int pml);
  SubdomainStructured(const SubdomainStructured& o);
  void factorize() { mSolver->factorize(); }
  void solve(ComplexVector& b, ComplexVector& res) const { mSolver->solve(b, res); }
  UInt getNDOFs() const { return (UInt)(mInfo.nx * mInfo.ny); }
  UInt getNEls() const { return (UInt)((mInfo.nx + 1) * (mInfo.ny + 1)); }
  void getPhysPts(std::vector<DoubleVector>& pts) const;   // DOF points of the cell
  const lsw_cell_info& info() const { return mInfo; }
  LocalLinearSolver* getLocalSolver() const { return mSolver.get(); }

 private:
  lsw_cell_info mInfo;
  std::unique_ptr<LocalLinearSolver> mSolver;
  Double mH, mAx, mAy;
  int mPml;
};
typedef SubdomainStructured Subdomain;

// ---- domain decomposition (include/DD.h, include/DDCheckerboard.h) --------------
class DD {
 public:
  virtual ~DD() {}
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
  void setVerbose(bool v) { mVerbose = v; }
  void setMode(lsw_gmres_mode m) { mMode = m; }
  void setRestart(UInt r) { mRestart = r; }
  void getLog(std::vector<Double>& res) const { res = mLog; }
  const lsw_gmres_report& report() const { return mRep; }
  void solve(const std::vector<ComplexVector>& rhs, std::vector<ComplexVector>& res) const override;

 private:
  Double mTol = 1e-6;
  UInt mMaxIter = 100;
  UInt mRestart = 0;   // 0: no restart (max_iter)
  bool mVerbose = false;
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
