// Batched factorisation of every cell matrix (replaces the per-cell Eigen
// SparseLU of LocalLinearSolverEigenSparseLU::factorize,
// LocalLinearSolverEigenSparseLU.cpp:40-62).
//
// The cell matrix is block tridiagonal over its nx x-lines, with tridiagonal
// diagonal blocks D_k (5-point stencil along y) and couplings w_k I / e_k I to
// the neighbouring lines.  Block LU gives the Schur complements
//   S_0 = D_0,   S_k = D_k - w_k e_{k-1} S_{k-1}^{-1},
// and the factor kept for the solves is Sinv_k = S_k^{-1} for every line,
// stored column-major (element (i, j) at j*ldn + i).  Each S_k is inverted by
// Gauss-Jordan elimination with partial pivoting on unpivoted rows (implicit
// row exchange, pivot order recorded), and the inverse is unscrambled on the
// way out: Sinv[i][j] = W[piv[i]][pinv[j]].  One CTA per cell runs the whole
// chain of lines; the working matrix sits in shared memory when it fits and
// in a per-cell global (L2-resident) buffer otherwise.  A zero or non-finite
// pivot sets bit 0 of *status (the reference exits on a failed factorisation,
// LocalLinearSolverEigenSparseLU.cpp:54-58).
#include "common.cuh"
#include "internal.h"

namespace lsw {

namespace {

constexpr int kFT = 1024;
constexpr int kHdr = 12 * 1024;  // pivot buffers, flags and reduction scratch (11.7 KB used)

template <typename T>
__global__ void __launch_bounds__(kFT, 1)
k_factorize(const DevCell* __restrict__ cells, const double2* __restrict__ prof,
            const double* __restrict__ mgrid, int n_dof, double omega2, cx_t<T>* __restrict__ fac,
            cx_t<T>* __restrict__ work, long long work_stride, int use_smem, int* status) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const DevCell cl = cells[blockIdx.x];
  const int n = cl.ny, nx = cl.nx, ldn = cl.ldn;
  const int ldw = n;

  C* colbuf = reinterpret_cast<C*>(smem);
  C* rowbuf = colbuf + 256;
  int* used = reinterpret_cast<int*>(rowbuf + 256);
  int* piv = used + 256;
  int* pinv = piv + 256;
  T* wbest = reinterpret_cast<T*>(pinv + 256);
  int* wbi = reinterpret_cast<int*>(wbest + 32);
  int* sp = wbi + 32;
  C* W = use_smem ? reinterpret_cast<C*>(smem + kHdr) : work + (long long)blockIdx.x * work_stride;

  const double2* px = prof + cl.prof_off;  // lo_x, hi_x, dg_x, lo_y, hi_y, dg_y
  const double2* py = px + 3 * nx;
  C* F = fac + cl.fac_off;
  const C z = czero<C>();

  for (int k = 0; k < nx; ++k) {
    // ---- Schur complement S_k into W (row-major) ----
    const C dgx = to_c(px[2 * nx + k], z);
    C coup = z;
    if (k > 0) coup = cmul(to_c(px[k], z), to_c(px[nx + k - 1], z));   // w_k e_{k-1}
    const C* Fp = F + (size_t)(k - 1) * n * ldn;
    const double* mrow = mgrid + (long long)(cl.lox + k) * n_dof + cl.loy;
    for (int i = ty; i < n; i += 32) {
      for (int j = tx; j < n; j += 32) {
        C v = z;
        if (k > 0) v = cneg(cmul(coup, Fp[(size_t)j * ldn + i]));
        if (j == i) {
          C d = cadd(dgx, to_c(py[2 * n + i], z));
          d.x -= (T)(omega2 * mrow[i]);
          v = cadd(v, d);
        } else if (j == i - 1) {
          v = cadd(v, to_c(py[i], z));          // coupling to j-1 (south)
        } else if (j == i + 1) {
          v = cadd(v, to_c(py[n + i], z));      // coupling to j+1 (north)
        }
        W[(size_t)i * ldw + j] = v;
      }
    }
    for (int i = tid; i < n; i += kFT) used[i] = 0;
    __syncthreads();

    // ---- Gauss-Jordan inversion in place ----
    for (int kk = 0; kk < n; ++kk) {
      T best = (T)-1; int bi = n;
      for (int r = tid; r < n; r += kFT) {
        const C v = W[(size_t)r * ldw + kk];
        colbuf[r] = v;
        if (!used[r]) {
          const T a2 = abs2(v);
          if (a2 > best) { best = a2; bi = r; }
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const T ob = __shfl_down_sync(0xffffffffu, best, off);
        const int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (tx == 0) { wbest[ty] = best; wbi[ty] = bi; }
      __syncthreads();
      if (ty == 0) {
        best = wbest[tx]; bi = wbi[tx];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const T ob = __shfl_down_sync(0xffffffffu, best, off);
          const int oi = __shfl_down_sync(0xffffffffu, bi, off);
          if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (tx == 0) {
          if (!(best > (T)0) || !isfinite((double)best) || bi >= n) {
            atomicOr(status, 1);
            // keep going with the first unpivoted row so the kernel terminates normally
            bi = 0;
            while (bi < n && used[bi]) ++bi;
            if (bi >= n) bi = 0;
          }
          sp[0] = bi;
          used[bi] = 1;
          piv[kk] = bi;
        }
      }
      __syncthreads();
      const int p = sp[0];
      const C inv = crcp(colbuf[p]);
      for (int j = tid; j < n; j += kFT) rowbuf[j] = (j == kk) ? inv : cmul(W[(size_t)p * ldw + j], inv);
      __syncthreads();
      for (int r = ty; r < n; r += 32) {
        C* Wr = W + (size_t)r * ldw;
        if (r == p) {
          for (int j = tx; j < n; j += 32) Wr[j] = rowbuf[j];
        } else {
          const C f = colbuf[r];
          for (int j = tx; j < n; j += 32) {
            if (j == kk) {
              Wr[j] = cneg(cmul(f, rowbuf[kk]));
            } else {
              C w = Wr[j];
              cfms(w, f, rowbuf[j]);
              Wr[j] = w;
            }
          }
        }
      }
      __syncthreads();
    }

    // ---- unscramble into the factor pool (column-major, zero padding) ----
    for (int i = tid; i < n; i += kFT) pinv[piv[i]] = i;
    __syncthreads();
    C* Fk = F + (size_t)k * n * ldn;
    for (int e = tid; e < n * ldn; e += kFT) {
      const int j = e / ldn, i = e - j * ldn;
      Fk[e] = (i < n) ? W[(size_t)piv[i] * ldw + pinv[j]] : z;
    }
    __syncthreads();
  }
}

}  // namespace

size_t factor_smem_bytes(int ny, bool dbl) {
  const size_t cs = dbl ? 16 : 8;
  return kHdr + (size_t)ny * ny * cs;
}

template <typename T>
cudaError_t launch_factorize(const DevCell* cells, int ncell, const double2* prof, const double* mgrid,
                             int n_dof, double omega2, void* fac, void* work, int max_ny, int* status,
                             cudaStream_t st) {
  if (ncell <= 0) return cudaSuccess;
  const bool dbl = sizeof(T) == 8;
  size_t smem = factor_smem_bytes(max_ny, dbl);
  int dev = 0, maxopt = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const int use_smem = smem <= (size_t)maxopt ? 1 : 0;
  if (!use_smem) smem = kHdr;
  if (!use_smem && work == nullptr) return cudaErrorInvalidValue;
  auto kern = k_factorize<T>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<ncell, kFT, smem, st>>>(cells, prof, mgrid, n_dof, omega2, reinterpret_cast<cx_t<T>*>(fac),
                                 reinterpret_cast<cx_t<T>*>(work), (long long)max_ny * max_ny, use_smem,
                                 status);
  return cudaGetLastError();
}

bool factor_needs_work(int max_ny, bool dbl) {
  int dev = 0, maxopt = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return factor_smem_bytes(max_ny, dbl) > (size_t)maxopt;
}

template cudaError_t launch_factorize<float>(const DevCell*, int, const double2*, const double*, int, double,
                                             void*, void*, int, int*, cudaStream_t);
template cudaError_t launch_factorize<double>(const DevCell*, int, const double2*, const double*, int, double,
                                              void*, void*, int, int*, cudaStream_t);

}  // namespace lsw
