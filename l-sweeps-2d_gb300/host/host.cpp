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
// ComplexSparseMatrix
// ===========================================================================
Complex ComplexSparseMatrix::coeff(UInt r, UInt c) const {
  if (r >= rows || c >= cols) throw lsw_host_error("ERROR: ComplexSparseMatrix::coeff index out of range");
  for (UInt k = outer[r]; k < outer[r + 1]; ++k)
    if (inner[k] == c) return vals[k];
  return Complex(0.0, 0.0);
}

void ComplexSparseMatrix::multiply(const ComplexVector& x, ComplexVector& y) const {
  if (x.size() != cols) throw lsw_host_error("ERROR: ComplexSparseMatrix::multiply size mismatch");
  y.assign(rows, Complex(0.0, 0.0));
  for (UInt r = 0; r < rows; ++r) {
    Complex acc(0.0, 0.0);
    for (UInt k = outer[r]; k < outer[r + 1]; ++k) acc += vals[k] * x[inner[k]];
    y[r] = acc;
  }
}

// ===========================================================================
// PML, PMLCubic2D (src/PML.cpp, src/PMLCubic2D.cpp:35-236)
// ===========================================================================
namespace {
std::vector<DoubleVector> grow(const std::vector<DoubleVector>& d, Double w) {
  std::vector<DoubleVector> c = d;
  for (auto& iv : c) { iv[0] -= w; iv[1] += w; }
  return c;
}
}  // namespace

void PML::setWidth(Double pmlWidth) {
  mPMLWidth = pmlWidth;
  if (!mIntDomain.empty()) mCompDomain = grow(mIntDomain, pmlWidth);
}

void PML::setDomain(const std::vector<DoubleVector>& domain) {
  mIntDomain = domain;
  if (mPMLWidth > 0) mCompDomain = grow(mIntDomain, mPMLWidth);
}

void PMLCubic2D::sigma(Double v, int d, Double& s, Double& ds) const {
  if (mCompDomain.size() < 2) throw lsw_host_error("ERROR: PML used before its domain and width are set");
  const Double ca = mCompDomain[d][0], cb = mCompDomain[d][1];
  const Double ia = mIntDomain[d][0], ib = mIntDomain[d][1];
  s = ds = 0.0;
  if (v >= ca && v < ia) {
    const Double delta = ia - ca, t = (ia - v) / delta;
    s = mC * t * t * t;
    ds = -3.0 * mC * (ia - v) * (ia - v) / (delta * delta * delta);
  } else if (v > ib && v < cb) {
    const Double delta = cb - ib, t = (v - ib) / delta;
    s = mC * t * t * t;
    ds = 3.0 * mC * (v - ib) * (v - ib) / (delta * delta * delta);
  } else if (!(v >= ia && v <= ib)) {
    throw lsw_host_error("ERROR: Evaluation point out of range!");
  }
}

ComplexVector PMLCubic2D::getDiffusionCoefficient(DoubleVector x) const {
  const Complex im(0.0, 1.0);
  ComplexVector r(2);
  for (int d = 0; d < 2; ++d) {
    Double s, ds;
    sigma(x[d], d, s, ds);
    const Complex al = 1.0 / (1.0 + im * s);
    r[d] = al * al;
  }
  return r;
}

ComplexVector PMLCubic2D::getConvectionCoefficient(DoubleVector x) const {
  const Complex im(0.0, 1.0);
  ComplexVector r(2);
  for (int d = 0; d < 2; ++d) {
    Double s, ds;
    sigma(x[d], d, s, ds);
    const Complex one = 1.0 + im * s;
    r[d] = (-im * ds / (one * one)) * (1.0 / one);   // alpha' alpha
  }
  return r;
}

// ===========================================================================
// AssemblerHelmholtz, AssemblerHelmholtz2DFD (src/AssemblerHelmholtz*.cpp)
// ===========================================================================
AssemblerHelmholtz::AssemblerHelmholtz(const AssemblerHelmholtz& o)
    : Assembler(o), mPML(o.mPML ? o.mPML->copy() : nullptr), mM(o.mM ? o.mM->copy() : nullptr), mOmega(o.mOmega) {
  if (mPML) mPML->setParent(this);
}

AssemblerHelmholtz& AssemblerHelmholtz::operator=(const AssemblerHelmholtz& o) {
  if (this != &o) {
    mPML.reset(o.mPML ? o.mPML->copy() : nullptr);
    if (mPML) mPML->setParent(this);
    mM.reset(o.mM ? o.mM->copy() : nullptr);
    mOmega = o.mOmega;
  }
  return *this;
}

void AssemblerHelmholtz::setPML(const PML* pml) {
  mPML.reset(pml ? pml->copy() : nullptr);
  if (mPML) mPML->setParent(this);
}

void AssemblerHelmholtz::setM(const Function* m) { mM.reset(m ? m->copy() : nullptr); }

void AssemblerHelmholtz2DFD::setDomain(const std::vector<DoubleVector>& dom) {
  mIntDomain = dom;
  if (!mPML) throw lsw_host_error("ERROR: set the PML before the domain");
  mPML->setDomain(dom);
}

// AssemblerHelmholtz2DFD::setN (src/AssemblerHelmholtz2DFD.cpp:67-114): the PML
// width rounded to whole elements of the smaller mesh size, the element counts
// of the computational domain
void AssemblerHelmholtz2DFD::setN(const UIntVector& n) {
  if (mIntDomain.size() != 2) throw lsw_host_error("ERROR: Domain has to be set before setting N");
  if (n.size() != 2 || n[0] == 0 || n[1] == 0) throw lsw_host_error("ERROR: two positive element counts expected");
  const Double h1 = (mIntDomain[0][1] - mIntDomain[0][0]) / n[0];
  const Double h2 = (mIntDomain[1][1] - mIntDomain[1][0]) / n[1];
  const Double h = std::min(h1, h2);
  const Double ratio = mPML->getWidth() / h;
  UInt els = (UInt)ratio;
  if (ratio - els > 0.5) ++els;
  mPML->setWidth(h * els);
  mCompDomain = grow(mIntDomain, h * els);
  mN = {(UInt)((mCompDomain[0][1] - mCompDomain[0][0] + 0.5 * h1) / h1),
        (UInt)((mCompDomain[1][1] - mCompDomain[1][0] + 0.5 * h2) / h2)};
}

Double AssemblerHelmholtz2DFD::getMeshSize() const {
  const Double h1 = (mCompDomain[0][1] - mCompDomain[0][0]) / mN[0];
  const Double h2 = (mCompDomain[1][1] - mCompDomain[1][0]) / mN[1];
  return std::sqrt(h1 * h2);
}

void AssemblerHelmholtz2DFD::getDOFPts(std::vector<DoubleVector>& res) const {
  const UInt nx = mN[0], ny = mN[1];
  const Double hx = (mCompDomain[0][1] - mCompDomain[0][0]) / nx;
  const Double hy = (mCompDomain[1][1] - mCompDomain[1][0]) / ny;
  res.assign((size_t)(nx - 1) * (ny - 1), DoubleVector(2));
  for (UInt i = 0; i + 1 < nx; ++i)
    for (UInt j = 0; j + 1 < ny; ++j)
      res[(size_t)i * (ny - 1) + j] = {mCompDomain[0][0] + (i + 1) * hx, mCompDomain[1][0] + (j + 1) * hy};
}

// boundary points, counter-clockwise from the bottom-left corner: bottom
// (left to right), right (bottom to top), top (right to left), left (top to
// bottom), each side without its last corner (AssemblerHelmholtz2DFD.cpp:185-226)
void AssemblerHelmholtz2DFD::getNonDOFPhysPts(std::vector<DoubleVector>& res) const {
  const UInt nx = mN[0], ny = mN[1];
  const Double hx = (mCompDomain[0][1] - mCompDomain[0][0]) / nx;
  const Double hy = (mCompDomain[1][1] - mCompDomain[1][0]) / ny;
  const Double x0 = mCompDomain[0][0], x1 = mCompDomain[0][1], y0 = mCompDomain[1][0], y1 = mCompDomain[1][1];
  res.clear();
  res.reserve(2 * (size_t)(nx + ny));
  for (UInt i = 0; i < nx; ++i) res.push_back({x0 + i * hx, y0});
  for (UInt i = 0; i < ny; ++i) res.push_back({x1, y0 + hy * i});
  for (UInt i = 0; i < nx; ++i) res.push_back({x1 - i * hx, y1});
  for (UInt i = 0; i < ny; ++i) res.push_back({x0, y1 - hy * i});
}

namespace {
// physical point index of grid node (a, b), a = 0..ex along x, b = 0..ey along
// y: DOFs first (a-1)(ey-1) + b-1, then the boundary points in the order of
// getNonDOFPhysPts
UInt node_index(UInt a, UInt b, UInt ex, UInt ey) {
  const UInt size = (ex - 1) * (ey - 1);
  if (a > 0 && a < ex && b > 0 && b < ey) return (a - 1) * (ey - 1) + (b - 1);
  if (b == 0 && a < ex) return size + a;
  if (a == ex && b < ey) return size + ex + b;
  if (b == ey && a > 0) return size + ex + ey + (ex - a);
  return size + 2 * ex + ey + (ey - b);   // a == 0, b > 0
}
}  // namespace

// corners of element `index` (J = index / ey along x, I along y), counter-
// clockwise from the bottom-left one (AssemblerHelmholtz2DFD.cpp:229-328)
void AssemblerHelmholtz2DFD::getElPhysPtIndices(UInt index, UIntVector& res) const {
  const UInt ex = mN[0], ey = mN[1];
  if (index >= ex * ey) throw lsw_host_error("ERROR: element index out of range");
  const UInt J = index / ey, I = index - J * ey;
  res = {node_index(J, I, ex, ey), node_index(J + 1, I, ex, ey), node_index(J + 1, I + 1, ex, ey),
         node_index(J, I + 1, ex, ey)};
}

void AssemblerHelmholtz2DFD::expandDOFValsToPhysVals(ComplexVector& res) const {
  ComplexVector t((size_t)(mN[0] + 1) * (mN[1] + 1), Complex(0.0, 0.0));
  std::copy(res.begin(), res.end(), t.begin());
  res.swap(t);
}

void AssemblerHelmholtz2DFD::assembleRHS(const RHS* rhs, ComplexVector& res) const {
  std::vector<DoubleVector> pts;
  getDOFPts(pts);
  res.assign(pts.size(), Complex(0.0, 0.0));
  for (size_t i = 0; i < pts.size(); ++i) res[i] += mPML->getSourceCoefficient(pts[i]) * rhs->eval(pts[i]);
}

void AssemblerHelmholtz2DFD::assembleSystemMatrix(ComplexSparseMatrix& res) const {
  if (!mM) throw lsw_host_error("ERROR: the assembler has no squared slowness");
  std::vector<DoubleVector> pts;
  getDOFPts(pts);
  std::vector<Double> m(pts.size());
  for (size_t i = 0; i < pts.size(); ++i) {
    const Complex v = mM->eval(pts[i]);
    if (v.imag() != 0.0) throw lsw_host_error("ERROR: complex squared slowness is not supported");
    m[i] = v.real();
  }
  assembleSystemMatrix(m, res);
}

// -(a1^2 Dxx + a2^2 Dyy) - (a1' a1 Dx + a2' a2 Dy) - omega^2 m with second-
// order differences (src/AssemblerHelmholtz2DFD.cpp:371-457): per DOF the
// diagonal 2 D1 / hx^2 + 2 D2 / hy^2 - omega^2 r m, west/east
// -D1 / hx^2 +- b1 / (2 hx), south/north -D2 / hy^2 +- b2 / (2 hy)
void AssemblerHelmholtz2DFD::assembleSystemMatrix(const std::vector<Double>& mDof, ComplexSparseMatrix& res) const {
  if (mOrder != 2) throw lsw_host_error("ERROR: only Order = 2 is supported");
  const UInt nx = mN[0] - 1, ny = mN[1] - 1;
  if (mDof.size() != (size_t)nx * ny) throw lsw_host_error("ERROR: squared slowness size mismatch");
  const Double hx = (mCompDomain[0][1] - mCompDomain[0][0]) / mN[0];
  const Double hy = (mCompDomain[1][1] - mCompDomain[1][0]) / mN[1];
  std::vector<DoubleVector> pts;
  getDOFPts(pts);
  res.rows = res.cols = nx * ny;
  res.outer.assign(1, 0);
  res.inner.clear();
  res.vals.clear();
  for (UInt i = 0; i < nx; ++i)
    for (UInt j = 0; j < ny; ++j) {
      const size_t r = (size_t)i * ny + j;
      const ComplexVector D = mPML->getDiffusionCoefficient(pts[r]);
      const ComplexVector B = mPML->getConvectionCoefficient(pts[r]);
      const Complex react = mPML->getReactionCoefficient(pts[r]);
      auto put = [&](UInt c, Complex v) { res.inner.push_back(c); res.vals.push_back(v); };
      // columns in ascending order: west, south, centre, north, east
      if (i > 0) put((UInt)(r - ny), -D[0] / (hx * hx) + B[0] / (2.0 * hx));
      if (j > 0) put((UInt)(r - 1), -D[1] / (hy * hy) + B[1] / (2.0 * hy));
      put((UInt)r, 2.0 * D[0] / (hx * hx) + 2.0 * D[1] / (hy * hy) - mOmega * mOmega * react * mDof[r]);
      if (j + 1 < ny) put((UInt)(r + 1), -D[1] / (hy * hy) - B[1] / (2.0 * hy));
      if (i + 1 < nx) put((UInt)(r + ny), -D[0] / (hx * hx) - B[0] / (2.0 * hx));
      res.outer.push_back((UInt)res.vals.size());
    }
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
// SubdomainStructured (src/SubdomainStructured.cpp) on the library's geometry
// ===========================================================================
SubdomainStructured::SubdomainStructured(lsw_ctx* ctx, int cell, const lsw_cell_info& info,
                                         const LocalLinearSolver* proto, Double h, Double ax, Double ay, int pml,
                                         Double omega, std::shared_ptr<const std::vector<double>> mGrid, int nDof)
    : mCtx(ctx), mCell(cell), mInfo(info), mH(h), mAx(ax), mAy(ay), mPml(pml), mGrid(std::move(mGrid)),
      mNDof(nDof) {
  setLocalLinearSolver(proto);
  // the cell's own discretisation: interior domain [lo h, (lo + nel) h] along
  // each direction (nel = DOFs - 2p + 1 interior elements), PML of p elements
  PMLCubic2D pl;
  pl.setAbsorptionCoeff(std::log(omega));   // Input.cpp:836
  pl.setWidth(pml * h);
  mAsm.setPML(&pl);
  mAsm.setOmega(omega);
  mAsm.setOrder(2);
  const int nelx = info.nx - 2 * pml + 1, nely = info.ny - 2 * pml + 1;
  mAsm.setDomain({{ax + info.lo_x * h, ax + (info.lo_x + nelx) * h}, {ay + info.lo_y * h, ay + (info.lo_y + nely) * h}});
  mAsm.setN({(UInt)nelx, (UInt)nely});
  const UIntVector n = mAsm.getN();
  if ((int)n[0] != info.nx + 1 || (int)n[1] != info.ny + 1)
    throw lsw_host_error("ERROR: cell discretisation does not match the library's geometry");
}

SubdomainStructured::SubdomainStructured(const SubdomainStructured& o)
    : mCtx(o.mCtx), mCell(o.mCell), mInfo(o.mInfo), mSolver(o.mSolver->copy()), mH(o.mH), mAx(o.mAx), mAy(o.mAy),
      mPml(o.mPml), mAsm(o.mAsm), mGrid(o.mGrid), mNDof(o.mNDof), mLims(o.mLims), mA(o.mA) {}

// the prototype pattern of SubdomainStructured::setLocalLinearSolver
// (src/SubdomainStructured.cpp:400-417); every copy is bound to its cell
void SubdomainStructured::setLocalLinearSolver(const LocalLinearSolver* solver) {
  if (!solver) throw lsw_host_error("ERROR: no local solver given");
  std::unique_ptr<LocalLinearSolver> s(solver->copy());
  auto* cu = dynamic_cast<LocalLinearSolverCUDA*>(s.get());
  if (!cu) throw lsw_host_error("ERROR: the sweeps run on the GPU: the local solver must be LocalLinearSolverCUDA");
  cu->bind(mCtx, mCell);
  mSolver = std::move(s);
}

void SubdomainStructured::getDOFPts(std::vector<DoubleVector>& res) const { mAsm.getDOFPts(res); }

void SubdomainStructured::getPhysPts(std::vector<DoubleVector>& res) const {
  mAsm.getDOFPts(res);
  std::vector<DoubleVector> b;
  mAsm.getNonDOFPhysPts(b);
  res.insert(res.end(), b.begin(), b.end());
}

void SubdomainStructured::getElPhysPtIndices(UInt elIndex, UIntVector& res) const {
  mAsm.getElPhysPtIndices(elIndex, res);
}

void SubdomainStructured::expandDOFValsToPhysVals(ComplexVector& res) const { mAsm.expandDOFValsToPhysVals(res); }

void SubdomainStructured::assembleRHS(const RHS* rhs, ComplexVector& res) const { mAsm.assembleRHS(rhs, res); }

// the device's operator: the squared slowness of the decomposition's global
// grid at the cell's DOFs
void SubdomainStructured::assembleSystemMatrix(ComplexSparseMatrix& res) const {
  if (!mGrid) throw lsw_host_error("ERROR: the cell has no squared slowness");
  std::vector<Double> m((size_t)mInfo.nx * mInfo.ny);
  for (int i = 0; i < mInfo.nx; ++i)
    for (int j = 0; j < mInfo.ny; ++j)
      m[(size_t)i * mInfo.ny + j] = (*mGrid)[(size_t)(mInfo.lo_x + i) * mNDof + mInfo.lo_y + j];
  mAsm.assembleSystemMatrix(m, res);
}

void SubdomainStructured::assembleSystemMatrix() const {
  auto A = std::make_shared<ComplexSparseMatrix>();
  assembleSystemMatrix(*A);
  mA = A;
}

const ComplexSparseMatrix& SubdomainStructured::matrix() const {
  if (!mA) assembleSystemMatrix();
  return *mA;
}

void SubdomainStructured::applySystemMatrix(const ComplexVector& x, ComplexVector& res) const {
  matrix().multiply(x, res);
}

namespace {
// The seven volume index sets along one direction of a cell
// (SubdomainStructured::computeVolumeIndexSets, src/SubdomainStructured.cpp:
// 749-801) from the trace lines t0, t1, tN, tNP of the shift (local line
// indices, -1 where absent): [0] lines before t0, [1] t0, [2] t1, [3] the lines
// between t1 and tN, [4] tN, [5] tNP, [6] the lines after tNP.  `n` lines along
// the direction; returns line indices.
std::vector<std::vector<int>> line_sets(const int* t, int n) {
  std::vector<std::vector<int>> r(7);
  for (int i = 0; i < n; ++i) {
    int k;
    if (t[0] >= 0 && i < t[0]) k = 0;
    else if (i == t[0]) k = 1;
    else if (i == t[1]) k = 2;
    else if (i == t[2]) k = 4;
    else if (i == t[3]) k = 5;
    else if (t[3] >= 0 && i > t[3]) k = 6;
    else k = 3;
    r[k].push_back(i);
  }
  return r;
}
}  // namespace

void SubdomainStructured::getIndexSets(std::string traceType, bool shifted, std::vector<UIntVector>& res) const {
  const int nx = mInfo.nx, ny = mInfo.ny, s = shifted ? 1 : 0;
  res.assign(7, UIntVector());
  if (traceType == "LeftRight") {
    const auto ls = line_sets(mInfo.lines_x[s], nx);
    for (int k = 0; k < 7; ++k)
      for (int i : ls[k])
        for (int j = 0; j < ny; ++j) res[k].push_back((UInt)(i * ny + j));
  } else if (traceType == "UpDown") {
    const auto ls = line_sets(mInfo.lines_y[s], ny);
    for (int k = 0; k < 7; ++k)
      for (int i = 0; i < nx; ++i)
        for (int j : ls[k]) res[k].push_back((UInt)(i * ny + j));
    for (auto& v : res) std::sort(v.begin(), v.end());
  } else {
    throw lsw_host_error("ERROR: No limits sets for this parametric direction!");
  }
}

// The nine element sets along one direction (computeVolumeElIndexSets,
// src/SubdomainStructured.cpp:804-1016): an element goes by its midpoint
// against the trace lines -- [0] before t0, [2] between t0 and t1, [4] between
// t1 and tN, [6] between tN and tNP, [8] after tNP; [1], [3], [5], [7] stay
// empty (single-line traces); a cell without trace lines has every element in
// [4].  Element e = J (ny + 1) + I, J along x, I along y.
void SubdomainStructured::getElIndexSets(std::string traceType, bool shifted, std::vector<UIntVector>& res) const {
  const int s = shifted ? 1 : 0;
  const int ex = mInfo.nx + 1, ey = mInfo.ny + 1;
  const int* t;
  bool along_x;
  if (traceType == "LeftRight") { t = mInfo.lines_x[s]; along_x = true; }
  else if (traceType == "UpDown") { t = mInfo.lines_y[s]; along_x = false; }
  else throw lsw_host_error("ERROR: Unknown trace type!");
  const bool none = t[0] < 0 && t[1] < 0 && t[2] < 0 && t[3] < 0;
  res.assign(9, UIntVector());
  for (int e = 0; e < ex * ey; ++e) {
    const int J = e / ey, I = e - J * ey;
    const int q = along_x ? J : I;   // element between lines q - 1 and q (midpoint below line q)
    int k;
    if (none) k = 4;
    else if (t[0] >= 0 && q <= t[0]) k = 0;
    else if (t[1] >= 0 && q <= t[1]) k = 2;
    else if (t[2] < 0 || q <= t[2]) k = 4;
    else if (t[3] < 0 || q <= t[3]) k = 6;
    else k = 8;
    res[k].push_back((UInt)e);
  }
}

// The trace0 and trace1 sets of a straight trace type (the 48 coupling slices
// of SubdomainStructured::assembleSystemMatrix, src/SubdomainStructured.cpp:
// 596-646) or an L-shaped one (getLTraceIndexSets)
void SubdomainStructured::traceSets(const std::string& tt, bool sLR, bool sUD, UIntVector& t0, UIntVector& t1) const {
  std::vector<UIntVector> s1, s2;
  if (tt == "Bottom" || tt == "Top") {
    getIndexSets("UpDown", sUD, s2);
    t0 = tt == "Bottom" ? s2[1] : s2[5];
    t1 = tt == "Bottom" ? s2[2] : s2[4];
  } else if (tt == "Left" || tt == "Right") {
    getIndexSets("LeftRight", sLR, s1);
    t0 = tt == "Left" ? s1[1] : s1[5];
    t1 = tt == "Left" ? s1[2] : s1[4];
  } else {
    std::vector<UIntVector> L;
    getLTraceIndexSets(tt, sLR, sUD, L);
    t0 = L[0];
    t1 = L[1];
  }
}

// L-shaped trace index sets (computeLTraceIndexSets, src/SubdomainStructured.cpp:
// 1119-1277): trace0 = the corner's trace0 lines of both directions without the
// DOFs beyond them, trace1 likewise one line further in
void SubdomainStructured::getLTraceIndexSets(std::string lt, bool sLR, bool sUD, std::vector<UIntVector>& res) const {
  std::vector<UIntVector> s1, s2;
  getIndexSets("LeftRight", sLR, s1);
  getIndexSets("UpDown", sUD, s2);
  const UIntVector *i0v, *i1v, *i0h, *i1h, *n0v, *n0h;
  UIntVector n1v, n1h;
  auto cat = [](const UIntVector& a, const UIntVector& b) { UIntVector r = a; r.insert(r.end(), b.begin(), b.end()); return r; };
  const bool left = lt == "BottomLeft" || lt == "TopLeft";
  const bool bottom = lt == "BottomLeft" || lt == "BottomRight";
  if (!left && lt != "BottomRight" && lt != "TopRight") throw lsw_host_error("ERROR: Invalid LTrace type!");
  if (left) { i0v = &s1[1]; i1v = &s1[2]; n0v = &s1[0]; n1v = cat(s1[0], s1[1]); }
  else { i0v = &s1[5]; i1v = &s1[4]; n0v = &s1[6]; n1v = cat(s1[5], s1[6]); }
  if (bottom) { i0h = &s2[1]; i1h = &s2[2]; n0h = &s2[0]; n1h = cat(s2[0], s2[1]); }
  else { i0h = &s2[5]; i1h = &s2[4]; n0h = &s2[6]; n1h = cat(s2[5], s2[6]); }
  const size_t n = getSize();
  res.assign(2, UIntVector());
  auto build = [&](const UIntVector& onA, const UIntVector& onB, const UIntVector& offA, const UIntVector& offB,
                   UIntVector& out) {
    std::vector<char> t(n, 0);
    for (UInt i : onA) t[i] = 1;
    for (UInt i : onB) t[i] = 1;
    for (UInt i : offA) t[i] = 0;
    for (UInt i : offB) t[i] = 0;
    for (size_t i = 0; i < n; ++i)
      if (t[i]) out.push_back((UInt)i);
  };
  build(*i0v, *i0h, *n0v, *n0h, res[0]);
  build(*i1v, *i1h, n1v, n1h, res[1]);
}

// res[0] = A[trace0, trace1] vals1 (on the trace0 DOFs), res[1] =
// -A[trace1, trace0] vals0 (on the trace1 DOFs) (getEquivalentSources,
// src/SubdomainStructured.cpp:1304-1465)
void SubdomainStructured::getEquivalentSources(std::string traceType, bool sLR, bool sUD, ComplexVector vals0,
                                               ComplexVector vals1, std::vector<ComplexVector>& res) const {
  UIntVector t0, t1;
  traceSets(traceType, sLR, sUD, t0, t1);
  if (vals0.size() != t0.size() || vals1.size() != t1.size())
    throw lsw_host_error("ERROR: trace values do not match the trace sets");
  const ComplexSparseMatrix& A = matrix();
  std::vector<int> pos1(getSize(), -1), pos0(getSize(), -1);
  for (size_t k = 0; k < t1.size(); ++k) pos1[t1[k]] = (int)k;
  for (size_t k = 0; k < t0.size(); ++k) pos0[t0[k]] = (int)k;
  res.assign(2, ComplexVector());
  res[0].assign(t0.size(), Complex(0.0, 0.0));
  res[1].assign(t1.size(), Complex(0.0, 0.0));
  for (size_t k = 0; k < t0.size(); ++k)
    for (UInt q = A.outer[t0[k]]; q < A.outer[t0[k] + 1]; ++q)
      if (pos1[A.inner[q]] >= 0) res[0][k] += A.vals[q] * vals1[pos1[A.inner[q]]];
  for (size_t k = 0; k < t1.size(); ++k)
    for (UInt q = A.outer[t1[k]]; q < A.outer[t1[k] + 1]; ++q)
      if (pos0[A.inner[q]] >= 0) res[1][k] -= A.vals[q] * vals0[pos0[A.inner[q]]];
}

// extractLTraces (src/SubdomainStructured.cpp:1468-1539): the four line traces
// written into one cell vector in the order LR1, UD1, LR0, UD0 (later writes
// win where lines cross), then gathered on the L-shaped trace0 / trace1 sets
void SubdomainStructured::extractLTraces(std::string lt, bool sLR, bool sUD, ComplexVector lr0, ComplexVector lr1,
                                         ComplexVector ud0, ComplexVector ud1, std::vector<ComplexVector>& res) const {
  std::vector<UIntVector> s1, s2, L;
  getIndexSets("LeftRight", sLR, s1);
  getIndexSets("UpDown", sUD, s2);
  getLTraceIndexSets(lt, sLR, sUD, L);
  const bool left = lt == "BottomLeft" || lt == "TopLeft";
  const bool bottom = lt == "BottomLeft" || lt == "BottomRight";
  const UIntVector& iLR0 = left ? s1[1] : s1[5];
  const UIntVector& iLR1 = left ? s1[2] : s1[4];
  const UIntVector& iUD0 = bottom ? s2[1] : s2[5];
  const UIntVector& iUD1 = bottom ? s2[2] : s2[4];
  ComplexVector tmp(getSize(), Complex(0.0, 0.0));
  std::vector<char> set(getSize(), 0);
  auto put = [&](const UIntVector& idx, const ComplexVector& v) {
    if (idx.size() != v.size()) throw lsw_host_error("ERROR: trace values do not match the trace sets");
    for (size_t k = 0; k < idx.size(); ++k) { tmp[idx[k]] = v[k]; set[idx[k]] = 1; }
  };
  put(iLR1, lr1);
  put(iUD1, ud1);
  put(iLR0, lr0);
  put(iUD0, ud0);
  res.assign(2, ComplexVector());
  for (int q = 0; q < 2; ++q)
    for (UInt i : L[q]) {
      if (!set[i]) throw lsw_host_error("ERROR: L-trace entry without a value");
      res[q].push_back(tmp[i]);
    }
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
  auto* ah = dynamic_cast<const AssemblerHelmholtz*>(assembler);
  if (!ah || !ah->getPML()) throw lsw_host_error("ERROR: DDCheckerboard needs a Helmholtz assembler with a PML");
  mAssembler.reset(assembler->copy());
  mProto.reset(solver->copy());
  mNCells = nCells;
  mNEls = nElsInCell;
  mPrec = precision;
  mDevice = device;
  mFactorized = false;
  mDomain = domain;
  mN = (int)nCells[0];
  mM = (int)nElsInCell[0];
  const int n_g = mN * mM + mN - 1;   // global elements per side (DDCheckerboard.cpp:119)
  mH = lx / n_g;
  // PML width rounded to whole elements (AssemblerHelmholtz2DFD::setN, 67-114)
  const double ratio = ah->getPML()->getWidth() / mH;
  int els = (int)ratio;
  if (ratio - els > 0.5) ++els;
  mPml = els;
  mNDof = n_g + 2 * mPml - 1;
  // squared slowness at every DOF point (AssemblerHelmholtz2DFD.cpp:440-449)
  const Function* m = ah->getM();
  if (!m) throw lsw_host_error("ERROR: the assembler has no squared slowness");
  std::unique_ptr<Function> mf(m->copy());
  std::vector<DoubleVector> d;
  mf->getDomain(d);
  if (d.empty()) mf->setDomain(domain);
  auto grid = std::make_shared<std::vector<double>>((size_t)mNDof * mNDof);
  std::vector<double>& mg = *grid;
  for (int i = 0; i < mNDof; ++i)
    for (int j = 0; j < mNDof; ++j) {
      const Complex v = mf->eval({domain[0][0] + (i + 1 - mPml) * mH, domain[1][0] + (j + 1 - mPml) * mH});
      if (v.imag() != 0.0) throw lsw_host_error("ERROR: complex squared slowness is not supported");
      mg[(size_t)i * mNDof + j] = v.real();
    }
  if (mCtx) { mCells.clear(); lsw_ctx_destroy(mCtx); mCtx = nullptr; }
  check(nullptr, lsw_ctx_create(&mCtx, device), "context");
  lsw_geom g{mN, mM, mPml, 2, mH};
  check(mCtx, lsw_problem_setup(mCtx, &g, mg.data(), ah->getOmega(), precision), "problem setup");
  lsw_problem_info pi;
  check(mCtx, lsw_problem_info_get(mCtx, &pi), "problem info");
  mCells.clear();
  for (int c = 0; c < pi.n_cells_total; ++c) {
    lsw_cell_info ci;
    check(mCtx, lsw_cell_info_get(mCtx, c, &ci), "cell info");
    mCells.emplace_back(new SubdomainStructured(mCtx, c, ci, solver, mH, domain[0][0], domain[1][0], mPml,
                                                ah->getOmega(), grid, mNDof));
  }
}

DD* DDCheckerboard::copy() const {
  if (!mCtx) throw lsw_host_error("ERROR: DDCheckerboard::copy before setUp");
  std::unique_ptr<DDCheckerboard> d(new DDCheckerboard);
  d->setUp(mAssembler.get(), mProto.get(), mDomain, mNCells, mNEls, mPrec, mDevice);
  if (mFactorized) d->factorize();
  return d.release();
}

void DDCheckerboard::factorize() {
  check(mCtx, lsw_factorize(mCtx, nullptr), "factorize");
  mFactorized = true;
}

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
