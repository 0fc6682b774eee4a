// Global-grid kernels: the FP64 5-point operator, the source assembly, the
// sum of the four shifted sweeps, and the FP64 Krylov reductions.
#include "common.cuh"
#include "internal.h"

namespace lsw {

namespace {

constexpr int kVT = 256;
constexpr int kRedBlocks = 1216;   // 8 x 152 SMs

// y = A x on the global grid (DDCheckerboard::applySystemMatrix equals the
// globally assembled operator, DDCheckerboard.cpp:2611-2635).  Coefficients are
// rebuilt from the separable PML profile (one profile serves x and y on the
// square grid) and the squared slowness: 40 algorithmic bytes per DOF.
__global__ void k_apply_A(const double2* __restrict__ x, double2* __restrict__ y, int n,
                          const double2* __restrict__ gp, const double* __restrict__ m, double omega2,
                          long long n2) {
  const long long G = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int v = blockIdx.y;
  if (G >= n2) return;
  const int gx = (int)(G / n), gy = (int)(G - (long long)gx * n);
  const double2* xv = x + (long long)v * n2;
  const double2 lox = gp[gx], hix = gp[n + gx], dgx = gp[2 * n + gx];
  const double2 loy = gp[gy], hiy = gp[n + gy], dgy = gp[2 * n + gy];
  double2 c = cadd(dgx, dgy);
  c.x -= omega2 * m[G];
  double2 acc = cmul(c, xv[G]);
  if (gx > 0) cfma(acc, lox, xv[G - n]);
  if (gx < n - 1) cfma(acc, hix, xv[G + n]);
  if (gy > 0) cfma(acc, loy, xv[G - 1]);
  if (gy < n - 1) cfma(acc, hiy, xv[G + 1]);
  y[(long long)v * n2 + G] = acc;
}

// M^-1 x = res1 + (res2 + res3 + res4)  (DDCheckerboard.cpp:733-735)
template <typename T>
__global__ void k_combine(const cx_t<T>* __restrict__ o, double2* __restrict__ y, long long n2) {
  const long long G = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int v = blockIdx.y;
  if (G >= n2) return;
  const cx_t<T>* b = o + (long long)v * 4 * n2;
  const double2 z = make_double2(0, 0);
  const double2 a0 = to_c(b[G], z), a1 = to_c(b[n2 + G], z), a2 = to_c(b[2 * n2 + G], z),
                a3 = to_c(b[3 * n2 + G], z);
  y[(long long)v * n2 + G] = cadd(a0, cadd(cadd(a1, a2), a3));
}

// RHSSrcPts::eval (RHSSrcPts.cpp:87-112): sum of 1/(pi eps^2) exp(-|x-x0|^2/eps^2).
__global__ void k_rhs(double2* __restrict__ b, int n, int p, double h, const double* __restrict__ src,
                      const double* __restrict__ amp, int nsrc, double eps) {
  const long long G = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (G >= (long long)n * n) return;
  const int gx = (int)(G / n), gy = (int)(G - (long long)gx * n);
  const double X = (gx + 1 - p) * h, Y = (gy + 1 - p) * h;
  const double pi = 3.14159265358979323846;
  double acc = 0.0;
  for (int s = 0; s < nsrc; ++s) {
    const double dx = src[2 * s] - X, dy = src[2 * s + 1] - Y;
    acc += (amp ? amp[s] : 1.0) * (1.0 / (pi * eps * eps) * exp(-(dx * dx + dy * dy) / (eps * eps)));
  }
  b[G] = make_double2(acc, 0.0);
}

template <typename V>
__device__ __forceinline__ V block_sum(V v, V* sh) {
  // sum over the block (kVT threads), result valid in thread 0
  for (int off = 16; off > 0; off >>= 1) {
    if constexpr (sizeof(V) == 16) {
      v.x += __shfl_down_sync(0xffffffffu, v.x, off);
      v.y += __shfl_down_sync(0xffffffffu, v.y, off);
    } else {
      v += __shfl_down_sync(0xffffffffu, v, off);
    }
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    V z{};
    v = (l < (int)(blockDim.x >> 5)) ? sh[l] : z;
    for (int off = 16; off > 0; off >>= 1) {
      if constexpr (sizeof(V) == 16) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, off);
        v.y += __shfl_down_sync(0xffffffffu, v.y, off);
      } else {
        v += __shfl_down_sync(0xffffffffu, v, off);
      }
    }
  }
  return v;
}

// partial[v][blk] = sum conj(a) b over the block's share
__global__ void k_dot_partial(const double2* __restrict__ a, const double2* __restrict__ b, long long n,
                              long long stride, double2* __restrict__ partial) {
  __shared__ double2 sh[32];
  const int v = blockIdx.y;
  const double2* av = a + (long long)v * stride;
  const double2* bv = b + (long long)v * stride;
  double2 s = make_double2(0, 0);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double2 x = av[i], y = bv[i];
    s.x += x.x * y.x + x.y * y.y;
    s.y += x.x * y.y - x.y * y.x;
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[(long long)v * gridDim.x + blockIdx.x] = s;
}

__global__ void k_finish2(const double2* __restrict__ partial, int nb, double2* __restrict__ out) {
  __shared__ double2 sh[32];
  const int v = blockIdx.x;
  double2 s = make_double2(0, 0);
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s = cadd(s, partial[(long long)v * nb + i]);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) out[v] = s;
}

__global__ void k_norm2_partial(const double2* __restrict__ a, long long n, long long stride,
                                double* __restrict__ partial) {
  __shared__ double sh[32];
  const int v = blockIdx.y;
  const double2* av = a + (long long)v * stride;
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    s += abs2(av[i]);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[(long long)v * gridDim.x + blockIdx.x] = s;
}

__global__ void k_finish1(const double* __restrict__ partial, int nb, double* __restrict__ out) {
  __shared__ double sh[32];
  const int v = blockIdx.x;
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partial[(long long)v * nb + i];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) out[v] = s;
}

// y -= coef[v] x ; optional partial dot with z of the updated y:
//   conj_first_y: sum conj(y) z   else: sum conj(z) y
__global__ void k_axpy_dot(double2* __restrict__ y, const double2* __restrict__ x,
                           const double2* __restrict__ coef, const double2* __restrict__ z, long long n,
                           long long stride, double2* __restrict__ partial, int conj_first_y) {
  __shared__ double2 sh[32];
  const int v = blockIdx.y;
  double2* yv = y + (long long)v * stride;
  const double2* xv = x + (long long)v * stride;
  const double2* zv = z ? z + (long long)v * stride : nullptr;
  const double2 c = coef[v];
  double2 s = make_double2(0, 0);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double2 t = yv[i];
    cfms(t, c, xv[i]);
    yv[i] = t;
    if (zv) {
      const double2 q = zv[i];
      if (conj_first_y) { s.x += t.x * q.x + t.y * q.y; s.y += t.x * q.y - t.y * q.x; }
      else { s.x += q.x * t.x + q.y * t.y; s.y += q.x * t.y - q.y * t.x; }
    } else {
      s.x += abs2(t);
    }
  }
  if (partial) {
    s = block_sum(s, sh);
    if (threadIdx.x == 0) partial[(long long)v * gridDim.x + blockIdx.x] = s;
  }
}

__global__ void k_scale(double2* __restrict__ y, const double2* __restrict__ x, const double2* __restrict__ coef,
                        int invert, long long n, long long stride) {
  const int v = blockIdx.y;
  double2 c = coef[v];
  if (invert) c = crcp(c);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[(long long)v * stride + i] = cmul(c, x[(long long)v * stride + i]);
}

__global__ void k_lincomb(double2* __restrict__ y, const double2* __restrict__ basis, long long bsv,
                          long long bsr, const double2* __restrict__ coef, int ncoef, long long n,
                          long long ys) {
  const int v = blockIdx.y;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double2 acc = y[(long long)v * ys + i];
    for (int q = 0; q < ncoef; ++q) cfma(acc, coef[(long long)v * ncoef + q], basis[q * bsv + v * bsr + i]);
    y[(long long)v * ys + i] = acc;
  }
}

__global__ void k_sub(double2* __restrict__ y, const double2* __restrict__ a, const double2* __restrict__ b,
                      long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = csub(a[i], b[i]);
}

inline unsigned nblk(long long n) {
  long long b = (n + kVT - 1) / kVT;
  if (b > kRedBlocks) b = kRedBlocks;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace

cudaError_t launch_apply_A(const double2* x, double2* y, int nrhs, int n_dof, const double2* gprof,
                           const double* mgrid, double omega2, cudaStream_t st) {
  const long long n2 = (long long)n_dof * n_dof;
  dim3 g((unsigned)((n2 + kVT - 1) / kVT), nrhs);
  k_apply_A<<<g, kVT, 0, st>>>(x, y, n_dof, gprof, mgrid, omega2, n2);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_combine(const void* outs, double2* y, int nrhs, long long n2, cudaStream_t st) {
  dim3 g((unsigned)((n2 + kVT - 1) / kVT), nrhs);
  k_combine<T><<<g, kVT, 0, st>>>(reinterpret_cast<const cx_t<T>*>(outs), y, n2);
  return cudaGetLastError();
}
template cudaError_t launch_combine<float>(const void*, double2*, int, long long, cudaStream_t);
template cudaError_t launch_combine<double>(const void*, double2*, int, long long, cudaStream_t);

namespace {
template <typename T>
__global__ void k_combine_ref(const cx_t<T>* __restrict__ o, double2* const* __restrict__ yref, long long n2,
                              int planes) {
  const long long G = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int v = blockIdx.y;
  if (G >= n2) return;
  double2* y = *yref;
  const double2 z = make_double2(0, 0);
  // per plane the four shifted outputs, a0 + ((a1 + a2) + a3); the planes in order
  double2 acc = z;
  for (int l = 0; l < planes; ++l) {
    const cx_t<T>* b = o + ((long long)v * planes + l) * 4 * n2;
    const double2 a0 = to_c(b[G], z), a1 = to_c(b[n2 + G], z), a2 = to_c(b[2 * n2 + G], z),
                  a3 = to_c(b[3 * n2 + G], z);
    const double2 s = cadd(a0, cadd(cadd(a1, a2), a3));
    acc = l == 0 ? s : cadd(acc, s);
  }
  y[(long long)v * n2 + G] = acc;
}
__global__ void k_set_refs(const void** ref, const void* x, void* y) {
  ref[0] = x;
  ref[1] = y;
}
}  // namespace

template <typename T>
cudaError_t launch_combine_ref(const void* outs, double2* const* y_ref, int nrhs, long long n2, int planes,
                               cudaStream_t st) {
  dim3 g((unsigned)((n2 + kVT - 1) / kVT), (unsigned)nrhs);
  k_combine_ref<T><<<g, kVT, 0, st>>>(reinterpret_cast<const cx_t<T>*>(outs), y_ref, n2, planes);
  return cudaGetLastError();
}
template cudaError_t launch_combine_ref<float>(const void*, double2* const*, int, long long, int, cudaStream_t);
template cudaError_t launch_combine_ref<double>(const void*, double2* const*, int, long long, int, cudaStream_t);

cudaError_t launch_set_refs(const void** ref, const void* x, void* y, cudaStream_t st) {
  k_set_refs<<<1, 1, 0, st>>>(ref, x, y);
  return cudaGetLastError();
}

cudaError_t launch_rhs(double2* b, int n_dof, int p, double h, const double* src, const double* amp, int nsrc,
                       double eps, cudaStream_t st) {
  const long long n2 = (long long)n_dof * n_dof;
  k_rhs<<<(unsigned)((n2 + kVT - 1) / kVT), kVT, 0, st>>>(b, n_dof, p, h, src, amp, nsrc, eps);
  return cudaGetLastError();
}

cudaError_t launch_dot(const double2* a, const double2* b, long long n, int nvec, long long stride,
                       double2* partial, double2* out, cudaStream_t st) {
  const unsigned nb = nblk(n);
  k_dot_partial<<<dim3(nb, nvec), kVT, 0, st>>>(a, b, n, stride, partial);
  k_finish2<<<nvec, kVT, 0, st>>>(partial, (int)nb, out);
  return cudaGetLastError();
}

cudaError_t launch_norm2(const double2* a, long long n, int nvec, long long stride, double* partial, double* out,
                         cudaStream_t st) {
  const unsigned nb = nblk(n);
  k_norm2_partial<<<dim3(nb, nvec), kVT, 0, st>>>(a, n, stride, partial);
  k_finish1<<<nvec, kVT, 0, st>>>(partial, (int)nb, out);
  return cudaGetLastError();
}

cudaError_t launch_axpy_dot(double2* y, const double2* x, const double2* coef, const double2* z, long long n,
                            int nvec, long long stride, double2* partial, double2* dotout, int conj_first_y,
                            cudaStream_t st) {
  const unsigned nb = nblk(n);
  k_axpy_dot<<<dim3(nb, nvec), kVT, 0, st>>>(y, x, coef, z, n, stride, dotout ? partial : nullptr, conj_first_y);
  if (dotout) k_finish2<<<nvec, kVT, 0, st>>>(partial, (int)nb, dotout);
  return cudaGetLastError();
}

cudaError_t launch_scale(double2* y, const double2* x, const double2* coef, int invert, long long n, int nvec,
                         long long stride, cudaStream_t st) {
  k_scale<<<dim3(nblk(n), nvec), kVT, 0, st>>>(y, x, coef, invert, n, stride);
  return cudaGetLastError();
}

cudaError_t launch_lincomb(double2* y, const double2* basis, long long bsv, long long bsr, const double2* coef,
                           int ncoef, long long n, int nvec, long long ys, cudaStream_t st) {
  k_lincomb<<<dim3(nblk(n), nvec), kVT, 0, st>>>(y, basis, bsv, bsr, coef, ncoef, n, ys);
  return cudaGetLastError();
}

cudaError_t launch_sub(double2* y, const double2* a, const double2* b, long long n, cudaStream_t st) {
  k_sub<<<nblk(n), kVT, 0, st>>>(y, a, b, n);
  return cudaGetLastError();
}

// ---- the Hessenberg least-squares problem of FGMRES(m) on the device ----
// One thread per right-hand side v.  H is (m + 1) x m row-major, cs and sn the
// m Givens rotations, g the rotated right-hand side (m + 1), all FP64 complex.
namespace {
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

// start of a cycle: ||r|| from its square, the relative residual, whether the
// right-hand side still iterates, ||r|| as V_0's divisor (1 if zero), and
// g = (||r||, 0, ..., 0)
__global__ void k_fgmres_init(int nv, int m, const double* __restrict__ r2, const double* __restrict__ bn,
                              double tol, double2* __restrict__ sc, double2* __restrict__ g, double* __restrict__ rel,
                              int* __restrict__ active) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const double rn = sqrt(r2[v]);
  const double rv = bn[v] > 0 ? rn / bn[v] : 0.0;
  rel[v] = rv;
  active[v] = rv <= tol ? 0 : 1;
  sc[v] = make_double2(rn > 0 ? rn : 1.0, 0.0);
  double2* gv = g + (size_t)v * (m + 1);
  gv[0] = make_double2(rn, 0.0);
  for (int i = 1; i <= m; ++i) gv[i] = make_double2(0.0, 0.0);
}

// step j: column j of H from the Gram-Schmidt coefficients h_0..h_j and
// ||w||^2 (row j + 1, real part); rotations 0..j-1 applied to it, rotation j
// formed (cs = h_j / d, sn = h_{j+1} / d, d = (|h_j|^2 + |h_{j+1}|^2)^(1/2)),
// g rotated; sc = ||w|| (the next basis vector's divisor, 1 if zero),
// est[v] = |g_{j+1}| / ||b||, est[nv + v] = ||w|| (0 on a breakdown)
__global__ void k_fgmres_givens(int j, int nv, int m, const double2* __restrict__ h, double2* __restrict__ H,
                                double2* __restrict__ cs, double2* __restrict__ sn, double2* __restrict__ g,
                                double2* __restrict__ sc, double* __restrict__ est, const double* __restrict__ bn) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  double2* Hv = H + (size_t)v * (m + 1) * m;
  double2* csv = cs + (size_t)v * m;
  double2* snv = sn + (size_t)v * m;
  double2* gv = g + (size_t)v * (m + 1);
  const double hn = sqrt(h[(size_t)(j + 1) * nv + v].x);
  double2 col[2];
  double2 prev = h[v];
  for (int i = 0; i < j; ++i) {
    const double2 b = h[(size_t)(i + 1) * nv + v];
    col[0] = cadd(cmul(cconj(csv[i]), prev), cmul(cconj(snv[i]), b));
    col[1] = csub(cmul(csv[i], b), cmul(snv[i], prev));
    Hv[(size_t)i * m + j] = col[0];
    prev = col[1];
  }
  // prev: rotated h_j; the subdiagonal entry is ||w||
  const double2 a = prev, b = make_double2(hn, 0.0);
  const double den = sqrt(abs2(a) + abs2(b));
  const double2 c = den > 0 ? make_double2(a.x / den, a.y / den) : make_double2(1.0, 0.0);
  const double2 s = den > 0 ? make_double2(b.x / den, b.y / den) : make_double2(0.0, 0.0);
  csv[j] = c;
  snv[j] = s;
  Hv[(size_t)j * m + j] = make_double2(den, 0.0);
  Hv[(size_t)(j + 1) * m + j] = make_double2(0.0, 0.0);
  const double2 gj = gv[j];
  gv[j + 1] = cneg(cmul(s, gj));
  gv[j] = cmul(cconj(c), gj);
  sc[v] = make_double2(hn > 0 ? hn : 1.0, 0.0);
  est[v] = bn[v] > 0 ? sqrt(abs2(gv[j + 1])) / bn[v] : 0.0;
  est[nv + v] = hn;
}

// end of a cycle: y = R^-1 g by back substitution on the first ncol columns
// (zero for right-hand sides that did not iterate), into coef[v][0..ncol)
__global__ void k_fgmres_solve(int ncol, int nv, int m, const double2* __restrict__ H, const double2* __restrict__ g,
                               const int* __restrict__ active, double2* __restrict__ coef) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const double2* Hv = H + (size_t)v * (m + 1) * m;
  const double2* gv = g + (size_t)v * (m + 1);
  double2* y = coef + (size_t)v * ncol;
  for (int i = ncol - 1; i >= 0; --i) {
    if (!active[v]) {
      y[i] = make_double2(0.0, 0.0);
      continue;
    }
    double2 sm = gv[i];
    for (int q = i + 1; q < ncol; ++q) cfms(sm, Hv[(size_t)i * m + q], y[q]);
    const double2 d = Hv[(size_t)i * m + i];
    y[i] = (d.x != 0.0 || d.y != 0.0) ? cmul(sm, crcp(d)) : make_double2(0.0, 0.0);
  }
}
}  // namespace

cudaError_t launch_fgmres_init(int nv, int m, const double* r2, const double* bn, double tol, double2* sc, double2* g,
                               double* rel, int* active, cudaStream_t st) {
  k_fgmres_init<<<(nv + 63) / 64, 64, 0, st>>>(nv, m, r2, bn, tol, sc, g, rel, active);
  return cudaGetLastError();
}
cudaError_t launch_fgmres_givens(int j, int nv, int m, const double2* h, double2* H, double2* cs, double2* sn,
                                 double2* g, double2* sc, double* est, const double* bn, cudaStream_t st) {
  k_fgmres_givens<<<(nv + 63) / 64, 64, 0, st>>>(j, nv, m, h, H, cs, sn, g, sc, est, bn);
  return cudaGetLastError();
}
cudaError_t launch_fgmres_solve(int ncol, int nv, int m, const double2* H, const double2* g, const int* active,
                                double2* coef, cudaStream_t st) {
  k_fgmres_solve<<<(nv + 63) / 64, 64, 0, st>>>(ncol, nv, m, H, g, active, coef);
  return cudaGetLastError();
}

}  // namespace lsw
