// C++ host layer with the reference's plugin API (include/lsweeps_host.hpp)
// over the C ABI.  Each class cites the reference file it stands in for.
#include "lsweeps_host.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>

namespace {

constexpr double kPi = 3.14159265358979323846;

void check(lsw_ctx* ctx, lsw_status s, const char* what) {
  if (s == LSW_OK) return;
  std::string m = std::string(what) + ": " + lsw_status_string(s);
  if (ctx) m += std::string(" (") + lsw_ctx_last_error(ctx) + ")";
  throw lsw_host_error(m);
}

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw lsw_host_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// device buffer owned by the host layer
struct DevVec {
  void* p = nullptr;
  size_t n = 0;
  ~DevVec() { if (p) cudaFree(p); }
  void* get(size_t bytes) {
    if (bytes > n) {
      if (p) cudaFree(p);
      p = nullptr;
      cuda_check(cudaMalloc(&p, bytes), "cudaMalloc");
      n = bytes;
    }
    return p;
  }
};

}  // namespace

// ===========================================================================
// FunctionCSV (src/FunctionCSV.cpp:46-236)
// ===========================================================================
void FunctionCSV::setFile(const std::string& filename, const std::vector<DoubleVector>& fileDom) {
  mFilename = filename;
  mFileDom = fileDom;
  std::ifstream in(filename);
  if (!in) throw lsw_host_error("ERROR: cannot open CSV file " + filename);
  std::string line;
  UInt rows = 0, cols = 0;
  mFile.clear();
  while (std::getline(in, line)) {
    std::stringstream ss(line);
    std::string val;
    UInt c = 0;
    while (std::getline(ss, val, ',')) {
      mFile.push_back(std::strtof(val.c_str(), nullptr));
      ++c;
    }
    if (rows == 0) cols = c;
    if (c != cols) throw lsw_host_error("ERROR: ragged CSV file " + filename);
    ++rows;
  }
  if (rows == 0 || cols == 0) throw lsw_host_error("ERROR: empty CSV file " + filename);
  mFileN = {rows, cols};
  mH = {(fileDom[0][1] - fileDom[0][0]) / cols, (fileDom[1][1] - fileDom[1][0]) / rows};
  // extremes of the squared slowness over the whole file
  bool first = true;
  for (float v : mFile) {
    const double s = 1.0 / std::pow((double)v, 2.0);
    if (first) { mMinReal = mMaxReal = s; first = false; }
    mMinReal = std::min(mMinReal, s);
    mMaxReal = std::max(mMaxReal, s);
  }
  mMinImag = mMaxImag = 0.0;
  mDomSet = false;
}

void FunctionCSV::setDomain(const std::vector<DoubleVector>& dom) const {
  mDom = dom;
  mDom[0][0] = std::max(dom[0][0], mFileDom[0][0]);
  mDom[1][0] = std::max(dom[1][0], mFileDom[1][0]);
  mDom[0][1] = std::min(dom[0][1], mFileDom[0][1]);
  mDom[1][1] = std::min(dom[1][1], mFileDom[1][1]);
  // file rows count from the top (largest y)
  UInt startRow = (UInt)((mFileDom[1][1] - mDom[1][1]) / mH[1]);
  UInt endRow = (UInt)((mFileDom[1][1] - mDom[1][0]) / mH[1]);
  UInt startCol = (UInt)((mDom[0][0] - mFileDom[0][0]) / mH[0]);
  UInt endCol = (UInt)((mDom[0][1] - mFileDom[0][0]) / mH[0]);
  endRow = std::min(endRow, mFileN[0] - 1);
  endCol = std::min(endCol, mFileN[1] - 1);
  mDomA = mDom;
  mDomA[0][0] = mFileDom[0][0] + startCol * mH[0];
  mDomA[0][1] = mFileDom[0][0] + (endCol + 1) * mH[0];
  mDomA[1][0] = mFileDom[1][1] - (endRow + 1) * mH[1];
  mDomA[1][1] = mFileDom[1][1] - startRow * mH[1];
  mRow0 = startRow; mCol0 = startCol;
  mRows = endRow - startRow + 1; mCols = endCol - startCol + 1;
  mA.assign((size_t)mRows * mCols, Complex(0.0, 0.0));
  bool first = true;
  for (UInt r = 0; r < mRows; ++r)
    for (UInt c = 0; c < mCols; ++c) {
      const Complex v(1.0 / std::pow((double)mFile[(size_t)(r + mRow0) * mFileN[1] + c + mCol0], 2.0), 0.0);
      mA[(size_t)r * mCols + c] = v;
      if (first) { mMinReal = mMaxReal = v.real(); mMinImag = mMaxImag = v.imag(); first = false; }
      mMinReal = std::min(mMinReal, v.real()); mMaxReal = std::max(mMaxReal, v.real());
      mMinImag = std::min(mMinImag, v.imag()); mMaxImag = std::max(mMaxImag, v.imag());
    }
  mDomSet = true;
}

void FunctionCSV::clearCache() const {
  mDom.clear();
  mDomA.clear();
  mA.clear();
  mDomSet = false;
}

Complex FunctionCSV::eval(DoubleVector x) const {
  if (!mDomSet) throw lsw_host_error("ERROR: FunctionCSV evaluated before setDomain");
  // clamp into the window, half a file cell inside (the reference uses the
  // x spacing for the lower and the y spacing for the upper bound in both
  // directions, FunctionCSV.cpp:188-193; identical for square file cells)
  for (size_t i = 0; i < x.size(); ++i)
    if (x[i] <= mDomA[i][0] + 0.5 * mH[0]) x[i] = mDomA[i][0] + 0.5 * mH[0];
  for (size_t i = 0; i < x.size(); ++i)
    if (x[i] >= mDomA[i][1] - 0.5 * mH[1]) x[i] = mDomA[i][1] - 0.5 * mH[1];
  UInt col = (UInt)((x[0] - mDomA[0][0]) / mH[0]);
  UInt row = (UInt)((mDomA[1][1] - x[1]) / mH[1]);
  col = std::min(col, mCols - 1);
  row = std::min(row, mRows - 1);
  return mA[(size_t)row * mCols + col];
}

// ===========================================================================
// RHSSrcPts (src/RHSSrcPts.cpp:87-112)
// ===========================================================================
Complex RHSSrcPts::eval(DoubleVector x) const {
  double res = 0.0;
  const double h = mEps;
  for (const auto& x0 : mSourcePts) {
    double d2 = 0.0;
    for (size_t i = 0; i < x.size(); ++i) d2 += (x0[i] - x[i]) * (x0[i] - x[i]);
    res += 1.0 / (kPi * std::pow(h, (double)x.size())) * std::exp(-d2 / (h * h));
  }
  return Complex(res, 0.0);
}

// ===========================================================================
// AssemblerHelmholtz2DFD (configuration holder)
// ===========================================================================
AssemblerHelmholtz2DFD::AssemblerHelmholtz2DFD(const AssemblerHelmholtz2DFD& o)
    : mPML(o.mPML), mOmega(o.mOmega), mOrder(o.mOrder), mM(o.mM ? o.mM->copy() : nullptr) {}

AssemblerHelmholtz2DFD& AssemblerHelmholtz2DFD::operator=(const AssemblerHelmholtz2DFD& o) {
  if (this != &o) {
    mPML = o.mPML;
    mOmega = o.mOmega;
    mOrder = o.mOrder;
    mM.reset(o.mM ? o.mM->copy() : nullptr);
  }
  return *this;
}

// ===========================================================================
// LocalLinearSolverCUDA (beside src/LocalLinearSolverEigenSparseLU.cpp)
// ===========================================================================
void LocalLinearSolverCUDA::factorize() {
  if (!mCtx) throw lsw_host_error("ERROR: LocalLinearSolverCUDA used before its DD bound it to a cell");
  check(mCtx, lsw_factorize(mCtx, nullptr), "factorize");
}

void LocalLinearSolverCUDA::solve(ComplexVector& b, ComplexVector& res) const {
  if (!mCtx) throw lsw_host_error("ERROR: LocalLinearSolverCUDA used before its DD bound it to a cell");
  lsw_cell_info ci;
  check(mCtx, lsw_cell_info_get(mCtx, mCell, &ci), "cell info");
  const size_t n = (size_t)ci.nx * ci.ny;
  if (b.size() != n) throw lsw_host_error("ERROR: LocalLinearSolverCUDA::solve: vector size does not match the cell");
  DevVec db, dx;
  void* pb = db.get(n * sizeof(Complex));
  void* px = dx.get(n * sizeof(Complex));
  cuda_check(cudaMemcpy(pb, b.data(), n * sizeof(Complex), cudaMemcpyHostToDevice), "H2D");
  check(mCtx, lsw_local_solve(mCtx, mCell, pb, px, 1, nullptr), "local solve");
  res.resize(n);
  cuda_check(cudaMemcpy(res.data(), px, n * sizeof(Complex), cudaMemcpyDeviceToHost), "D2H");
}

// ===========================================================================
// SubdomainStructured
// ===========================================================================
SubdomainStructured::SubdomainStructured(lsw_ctx* ctx, int cell, const lsw_cell_info& info,
                                         const LocalLinearSolver* proto, Double h, Double ax, Double ay, int pml)
    : mInfo(info), mSolver(proto->copy()), mH(h), mAx(ax), mAy(ay), mPml(pml) {
  // the prototype pattern of SubdomainStructured::setLocalLinearSolver
  // (src/SubdomainStructured.cpp:400-417); every copy is bound to its cell
  auto* cu = dynamic_cast<LocalLinearSolverCUDA*>(mSolver.get());
  if (!cu) throw lsw_host_error("ERROR: the sweeps run on the GPU: the local solver must be LocalLinearSolverCUDA");
  cu->bind(ctx, cell);
}

SubdomainStructured::SubdomainStructured(const SubdomainStructured& o)
    : mInfo(o.mInfo), mSolver(o.mSolver->copy()), mH(o.mH), mAx(o.mAx), mAy(o.mAy), mPml(o.mPml) {}

void SubdomainStructured::getPhysPts(std::vector<DoubleVector>& pts) const {
  pts.resize((size_t)mInfo.nx * mInfo.ny);
  for (int i = 0; i < mInfo.nx; ++i)
    for (int j = 0; j < mInfo.ny; ++j)
      pts[(size_t)i * mInfo.ny + j] = {mAx + (mInfo.lo_x + i + 1 - mPml) * mH, mAy + (mInfo.lo_y + j + 1 - mPml) * mH};
}

// ===========================================================================
// DDCheckerboard
// ===========================================================================
void* DDCheckerboard::devBuffers(size_t bytes) const {
  if (bytes > mBufBytes) {
    if (mBuf) cudaFree(mBuf);
    mBuf = nullptr;
    mBufBytes = 0;
    cuda_check(cudaMalloc(&mBuf, 2 * bytes), "cudaMalloc");
    mBufBytes = bytes;
  }
  return mBuf;
}

DDCheckerboard::~DDCheckerboard() {
  mCells.clear();
  if (mBuf) cudaFree(mBuf);
  if (mCtx) lsw_ctx_destroy(mCtx);
}

void DDCheckerboard::setUp(const Assembler* assembler, const LocalLinearSolver* solver,
                           const std::vector<DoubleVector>& domain, const UIntVector& nCells,
                           const UIntVector& nElsInCell, lsw_precision precision, int device) {
  if (!assembler || !solver) throw lsw_host_error("ERROR: DDCheckerboard::setUp needs an assembler and a solver");
  if (domain.size() != 2 || nCells.size() != 2 || nElsInCell.size() != 2)
    throw lsw_host_error("ERROR: DDCheckerboard is two-dimensional");
  if (nCells[0] != nCells[1] || nElsInCell[0] != nElsInCell[1])
    throw lsw_host_error("ERROR: this library supports square checkerboards (NCellsX == NCellsY, NX == NY)");
  const double lx = domain[0][1] - domain[0][0], ly = domain[1][1] - domain[1][0];
  if (!(lx > 0) || std::fabs(lx - ly) > 1e-12 * lx) throw lsw_host_error("ERROR: this library supports square domains");
  if (assembler->getOrder() != 2) throw lsw_host_error("ERROR: this library supports Order = 2");
  mDomain = domain;
  mN = (int)nCells[0];
  mM = (int)nElsInCell[0];
  const int n_g = mN * mM + mN - 1;   // global elements per side (DDCheckerboard.cpp:119)
  mH = lx / n_g;
  // PML width rounded to whole elements (AssemblerHelmholtz2DFD::setN, 67-114)
  const double ratio = assembler->getPML().getWidth() / mH;
  int els = (int)ratio;
  if (ratio - els > 0.5) ++els;
  mPml = els;
  mNDof = n_g + 2 * mPml - 1;
  // squared slowness at every DOF point (AssemblerHelmholtz2DFD.cpp:440-449)
  const Function* m = assembler->getM();
  if (!m) throw lsw_host_error("ERROR: the assembler has no squared slowness");
  std::unique_ptr<Function> mf(m->copy());
  std::vector<DoubleVector> d;
  mf->getDomain(d);
  if (d.empty()) mf->setDomain(domain);
  std::vector<double> mg((size_t)mNDof * mNDof);
  for (int i = 0; i < mNDof; ++i)
    for (int j = 0; j < mNDof; ++j) {
      const Complex v = mf->eval({domain[0][0] + (i + 1 - mPml) * mH, domain[1][0] + (j + 1 - mPml) * mH});
      if (v.imag() != 0.0) throw lsw_host_error("ERROR: complex squared slowness is not supported");
      mg[(size_t)i * mNDof + j] = v.real();
    }
  if (mCtx) { mCells.clear(); lsw_ctx_destroy(mCtx); mCtx = nullptr; }
  check(nullptr, lsw_ctx_create(&mCtx, device), "context");
  lsw_geom g{mN, mM, mPml, 2, mH};
  check(mCtx, lsw_problem_setup(mCtx, &g, mg.data(), assembler->getOmega(), precision), "problem setup");
  lsw_problem_info pi;
  check(mCtx, lsw_problem_info_get(mCtx, &pi), "problem info");
  mCells.clear();
  for (int c = 0; c < pi.n_cells_total; ++c) {
    lsw_cell_info ci;
    check(mCtx, lsw_cell_info_get(mCtx, c, &ci), "cell info");
    mCells.emplace_back(new SubdomainStructured(mCtx, c, ci, solver, mH, domain[0][0], domain[1][0], mPml));
  }
}

void DDCheckerboard::factorize() { check(mCtx, lsw_factorize(mCtx, nullptr), "factorize"); }

void DDCheckerboard::toGlobal(const std::vector<ComplexVector>& cells, ComplexVector& g) const {
  if (cells.size() != mCells.size()) throw lsw_host_error("ERROR: one vector per cell expected");
  g.assign((size_t)mNDof * mNDof, Complex(0.0, 0.0));
  for (size_t c = 0; c < mCells.size(); ++c) {
    const lsw_cell_info& ci = mCells[c]->info();
    const int x0 = ci.own_x[0][0], x1 = ci.own_x[0][1], y0 = ci.own_y[0][0], y1 = ci.own_y[0][1];
    const int w = y1 - y0 + 1;
    if (cells[c].size() != (size_t)(x1 - x0 + 1) * w) throw lsw_host_error("ERROR: cell vector size mismatch");
    for (int i = x0; i <= x1; ++i)
      for (int j = y0; j <= y1; ++j)
        g[(size_t)(ci.lo_x + i) * mNDof + ci.lo_y + j] = cells[c][(size_t)(i - x0) * w + (j - y0)];
  }
}

void DDCheckerboard::toCells(const ComplexVector& g, std::vector<ComplexVector>& cells) const {
  cells.resize(mCells.size());
  for (size_t c = 0; c < mCells.size(); ++c) {
    const lsw_cell_info& ci = mCells[c]->info();
    const int x0 = ci.own_x[0][0], x1 = ci.own_x[0][1], y0 = ci.own_y[0][0], y1 = ci.own_y[0][1];
    const int w = y1 - y0 + 1;
    cells[c].resize((size_t)(x1 - x0 + 1) * w);
    for (int i = x0; i <= x1; ++i)
      for (int j = y0; j <= y1; ++j)
        cells[c][(size_t)(i - x0) * w + (j - y0)] = g[(size_t)(ci.lo_x + i) * mNDof + ci.lo_y + j];
  }
}

void DDCheckerboard::assembleRHS(const RHS* rhs, std::vector<ComplexVector>& res) const {
  ComplexVector g((size_t)mNDof * mNDof);
  const size_t bytes = g.size() * sizeof(Complex);
  if (auto* sp = dynamic_cast<const RHSSrcPts*>(rhs)) {
    if (std::fabs(sp->getEpsilon() - mH) <= 1e-12 * mH || sp->getEpsilon() == 0.0) {
      // Gaussian point sources of width h on the device
      std::vector<DoubleVector> pts;
      sp->getSrcPts(pts);
      std::vector<double> xy;
      for (const auto& p : pts) { xy.push_back(p[0] - mDomain[0][0]); xy.push_back(p[1] - mDomain[1][0]); }
      void* d = devBuffers(bytes);
      check(mCtx, lsw_assemble_rhs(mCtx, xy.data(), nullptr, (int)pts.size(), d, nullptr), "assemble rhs");
      cuda_check(cudaMemcpy(g.data(), d, bytes, cudaMemcpyDeviceToHost), "D2H rhs");
      toCells(g, res);
      return;
    }
  }
  for (int i = 0; i < mNDof; ++i)
    for (int j = 0; j < mNDof; ++j)
      g[(size_t)i * mNDof + j] = rhs->eval({mDomain[0][0] + (i + 1 - mPml) * mH, mDomain[1][0] + (j + 1 - mPml) * mH});
  toCells(g, res);
}

void DDCheckerboard::applyPrecond(const std::vector<ComplexVector>& x, std::vector<ComplexVector>& res) const {
  ComplexVector g;
  toGlobal(x, g);
  const size_t bytes = g.size() * sizeof(Complex);
  void* a = devBuffers(bytes);
  void* b = static_cast<char*>(a) + bytes;
  cuda_check(cudaMemcpy(a, g.data(), bytes, cudaMemcpyHostToDevice), "H2D");
  check(mCtx, lsw_apply_precond(mCtx, a, b, 1, nullptr), "apply preconditioner");
  cuda_check(cudaMemcpy(g.data(), b, bytes, cudaMemcpyDeviceToHost), "D2H");
  toCells(g, res);
}

void DDCheckerboard::applySystemMatrix(const std::vector<ComplexVector>& x, std::vector<ComplexVector>& res) const {
  ComplexVector g;
  toGlobal(x, g);
  const size_t bytes = g.size() * sizeof(Complex);
  void* a = devBuffers(bytes);
  void* b = static_cast<char*>(a) + bytes;
  cuda_check(cudaMemcpy(a, g.data(), bytes, cudaMemcpyHostToDevice), "H2D");
  check(mCtx, lsw_apply_A(mCtx, a, b, 1, nullptr), "apply system matrix");
  cuda_check(cudaMemcpy(g.data(), b, bytes, cudaMemcpyDeviceToHost), "D2H");
  toCells(g, res);
}

void DDCheckerboard::expand(const std::vector<ComplexVector>& x, std::vector<ComplexVector>& res, bool, bool) const {
  ComplexVector g;
  toGlobal(x, g);
  res.resize(mCells.size());
  for (size_t c = 0; c < mCells.size(); ++c) {
    const lsw_cell_info& ci = mCells[c]->info();
    res[c].resize((size_t)ci.nx * ci.ny);
    for (int i = 0; i < ci.nx; ++i)
      for (int j = 0; j < ci.ny; ++j) res[c][(size_t)i * ci.ny + j] = g[(size_t)(ci.lo_x + i) * mNDof + ci.lo_y + j];
  }
}

// ===========================================================================
// GlobalIterativeSolverGMRES (src/GlobalIterativeSolverGMRES.cpp:65-203)
// ===========================================================================
void GlobalIterativeSolverGMRES::solve(const std::vector<ComplexVector>& rhs, std::vector<ComplexVector>& res) const {
  auto* dd = dynamic_cast<const DDCheckerboard*>(mParent);
  if (!dd) throw lsw_host_error("ERROR: GlobalIterativeSolverGMRES needs a DDCheckerboard parent (setParent)");
  ComplexVector b, x;
  dd->toGlobal(rhs, b);
  x.resize(b.size());
  lsw_gmres_opts o;
  o.mode = mMode;
  o.tol = mTol;
  o.max_iter = (int)mMaxIter;
  o.restart = (int)(mRestart ? mRestart : std::max<UInt>(mMaxIter, 1));
  o.verbose = mVerbose ? 1 : 0;
  std::vector<double> logbuf(mMaxIter + 2);
  mRep = lsw_gmres_report{};
  mRep.log = logbuf.data();
  mRep.log_capacity = (int)logbuf.size();
  check(dd->ctx(), lsw_solve_host(dd->ctx(), reinterpret_cast<const double*>(b.data()),
                                  reinterpret_cast<double*>(x.data()), 1, &o, &mRep, nullptr),
        "GMRES");
  mLog.assign(logbuf.begin(), logbuf.begin() + std::min(mRep.log_len, mRep.log_capacity));
  mRep.log = nullptr;
  dd->toCells(x, res);
}

// ===========================================================================
// OutputVTK (src/OutputVTK.cpp:65-358)
// ===========================================================================
void OutputVTK::setVals(const std::vector<ComplexVector>& vals) const {
  auto* dd = dynamic_cast<const DDCheckerboard*>(mDD);
  if (!dd) throw lsw_host_error("ERROR: OutputVTK needs a DDCheckerboard (setDD)");
  dd->toGlobal(vals, mVals);
}

void OutputVTK::print() const {
  auto* dd = dynamic_cast<const DDCheckerboard*>(mDD);
  if (!dd) throw lsw_host_error("ERROR: OutputVTK needs a DDCheckerboard (setDD)");
  const int nd = dd->nDof(), p = dd->pml();
  const double h = dd->getMeshSize(), ax = dd->domain()[0][0], ay = dd->domain()[1][0];
  // the grid points of the physical domain: DOFs p-1 .. nd-p along each side
  const int i0 = p - 1, np = nd - 2 * (p - 1);
  const int nel = (np - 1) * (np - 1);
  std::ofstream f(mFilename + ".vtk");
  if (!f) throw lsw_host_error("ERROR: cannot write " + mFilename + ".vtk");
  f << "# vtk DataFile Version 1.0\n2D Unstuctured Grid of Linear Quads\nASCII\n\n";
  f << "DATASET UNSTRUCTURED_GRID\n";
  f << "POINTS " << (long long)np * np << " float\n";
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) f << ax + (i0 + i + 1 - p) * h << " " << ay + (i0 + j + 1 - p) * h << " 0.0\n";
  f << "\nCELLS " << nel << " " << 5LL * nel << "\n";
  for (int i = 0; i + 1 < np; ++i)
    for (int j = 0; j + 1 < np; ++j) {
      const long long a = (long long)i * np + j;
      f << 4 << " " << a << " " << a + np << " " << a + np + 1 << " " << a + 1 << "\n";
    }
  f << "\nCELL_TYPES " << nel << "\n";
  for (int e = 0; e < nel; ++e) f << 9 << "\n";
  f << "\nPOINT_DATA " << (long long)np * np << "\n";
  f << "SCALARS wavefield_re float\nLOOKUP_TABLE default\n";
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) f << mVals[(size_t)(i0 + i) * nd + i0 + j].real() << "\n";
  f << "SCALARS wavefield_im float\nLOOKUP_TABLE default\n";
  for (int i = 0; i < np; ++i)
    for (int j = 0; j < np; ++j) f << mVals[(size_t)(i0 + i) * nd + i0 + j].imag() << "\n";
}

// ===========================================================================
// Problem (src/Problem.cpp)
// ===========================================================================
Problem::~Problem() {
  delete mOutput;
  delete mSolver;
  delete mRHS;
  delete mDD;
}

void Problem::read(const Input& input, UInt probID) {
  input.readProblemDD(mDD, probID);
  input.readProblemRHS(mDD, mRHS, probID);
  input.readProblemSolver(mSolver, probID);
  mSolver->setParent(mDD);
  input.readProblemOutput(mOutput, probID);
  if (mOutput) mOutput->setDD(mDD);
}

void Problem::solve() const {
  using clk = std::chrono::steady_clock;
  std::cout << "Facorize problem..." << std::endl;
  auto t0 = clk::now();
  mDD->factorize();
  const double fact = std::chrono::duration<double>(clk::now() - t0).count();
  std::cout << "Assemble RHS..." << std::endl;
  std::vector<ComplexVector> rhs, res;
  mDD->assembleRHS(mRHS, rhs);
  std::cout << "Solving..." << std::endl;
  t0 = clk::now();
  mSolver->solve(rhs, res);
  const double sol = std::chrono::duration<double>(clk::now() - t0).count();
  std::cout << "Time to factorize system: " << fact << std::endl;
  std::cout << "Time to run the GMRES: " << sol << std::endl;
  std::cout << "Writing output file..." << std::endl;
  if (mOutput) {
    mOutput->setVals(res);
    mOutput->print();
  }
}
