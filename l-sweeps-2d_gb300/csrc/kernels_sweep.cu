// Sweep-front kernel: every cell solve of one front of the L-sweep
// preconditioner in one launch.
//
// A cell matrix is block tridiagonal over its x-lines (DOF order i*ny + j,
// AssemblerHelmholtz2DFD.cpp:166-177); the couplings between lines are scalar
// multiples of the identity (the PML profile is separable), so with the stored
// Schur-complement inverses Sinv_k (kernels_factor.cu) a solve is
//   forward   y_k = Sinv_k (b_k - w_k y_{k-1})
//   backward  x_k = y_k - e_k Sinv_k x_{k+1}
// (w_k, e_k = couplings of line k to k-1 / k+1).  One CTA takes one cell and
// up to RMAX right-hand sides ("slots") that share every factor block it
// streams from HBM.  The right-hand sides are never materialised: each slot
// builds b_k on the fly from the global input (stage 1, the window of
// DDCheckerboard::getSeparatedRHS, DDCheckerboard.cpp:3564-3674, restricted to
// the owned set) or from its neighbours' trace lines (equivalent sources of
// SubdomainStructured::getEquivalentSources, SubdomainStructured.cpp:1304-1465,
// and the L-shaped traces of extractLTraces, 1468-1539).  The backward pass
// accumulates owned DOFs into the output (reduce, DDCheckerboard.cpp:744-772)
// and the outgoing trace lines into the trace pool.
#include "common.cuh"
#include "internal.h"

namespace lsw {

namespace {

constexpr int kNT = 1024;

__device__ __forceinline__ bool is_line(int gnode, int m, int N) {
  // interface lines k_b(J), k_b(J)+1 for J = 0..N-2 (the trace1/traceN rows
  // zeroed by getSeparatedRHS)
  if (gnode < m || gnode > (m + 1) * (N - 1)) return false;
  const int r = gnode % (m + 1);
  return r == m || r == 0;
}

template <typename C>
__device__ __forceinline__ C ldc(const C* p) { return *p; }

struct SlotCoef {
  double2 c_oi_x, c_io_x, c_oi_y, c_io_y;
};

template <typename T>
__device__ __forceinline__ cx_t<T> rhs_elem(const FrontArgs& a, const DevCell& cl, const DevSlot& s,
                                            const SlotCoef& cf, const cx_t<T>* tr, int k, int j) {
  using C = cx_t<T>;
  C z = czero<C>();
  switch (s.kind) {
    case SK_VOLUME: {
      const int sx = s.shift & 1, sy = (s.shift >> 1) & 1;
      if (k < cl.ownx[sx][0] || k > cl.ownx[sx][1] || j < cl.owny[sy][0] || j > cl.owny[sy][1]) return z;
      const int gx = cl.lox + k, gy = cl.loy + j;
      const bool lx = is_line(gx - a.p + 1, a.m, a.N), ly = is_line(gy - a.p + 1, a.m, a.N);
      if (lx != (bool)sx || ly != (bool)sy) return z;
      const double2 v = a.x_in[(long long)s.rhs * a.x_stride + (long long)gx * a.n_dof + gy];
      return to_c(v, z);
    }
    case SK_CELLVEC: {
      const double2 v = a.x_in[(long long)s.rhs * a.x_stride + (long long)k * cl.ny + j];
      return to_c(v, z);
    }
    case SK_DIR_X: {
      if (k == s.xo) return cmul(to_c(cf.c_oi_x, z), tr[s.in_lr1 + j]);
      if (k == s.xi) return cneg(cmul(to_c(cf.c_io_x, z), tr[s.in_lr0 + j]));
      return z;
    }
    case SK_DIR_Y: {
      if (j == s.yo) return cmul(to_c(cf.c_oi_y, z), tr[s.in_ud1 + k]);
      if (j == s.yi) return cneg(cmul(to_c(cf.c_io_y, z), tr[s.in_ud0 + k]));
      return z;
    }
    case SK_CORNER: {
      // L-shaped sources: trace0 set L0 = {(xo, y): y inside yo} u {(x, yo): x inside xo},
      // trace1 set L1 likewise on (xi, yi) (computeLTraceIndexSets, 1119-1277);
      // rhs[L0] = A01 v1, rhs[L1] = -A10 v0 with the trace values of extractLTraces
      // (UD0 > LR0 > UD1 > LR1 where lines cross).
      const bool yin_o = (j - s.yo) * s.dy > 0;
      const bool yin_i = (j - s.yi) * s.dy > 0;
      if (k == s.xo) {
        if (!yin_o) return z;
        const C v = (j == s.yi) ? tr[s.in_ud1 + s.xi] : tr[s.in_lr1 + j];
        return cmul(to_c(cf.c_oi_x, z), v);
      }
      const bool xin_i = (k - s.xi) * s.dx > 0;
      if (k == s.xi) {
        if (j == s.yo) return cmul(to_c(cf.c_oi_y, z), tr[s.in_ud1 + k]);
        if (j == s.yi) {
          C r = cneg(cmul(to_c(cf.c_io_x, z), tr[s.in_lr0 + j]));
          cfms(r, to_c(cf.c_io_y, z), tr[s.in_ud0 + k]);
          return r;
        }
        if (yin_i) return cneg(cmul(to_c(cf.c_io_x, z), tr[s.in_lr0 + j]));
        return z;
      }
      if (xin_i) {
        if (j == s.yo) return cmul(to_c(cf.c_oi_y, z), tr[s.in_ud1 + k]);
        if (j == s.yi) return cneg(cmul(to_c(cf.c_io_y, z), tr[s.in_ud0 + k]));
      }
      return z;
    }
    default:
      return z;
  }
}

template <typename T, int RMAX>
__global__ void __launch_bounds__(kNT, 1) k_front(FrontArgs a) {
  using C = cx_t<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x;
  const DevItem it = a.items[blockIdx.x];
  const DevCell cl = a.cells[it.cell];
  const int R = it.slot_count;
  const int nx = cl.nx, ny = cl.ny, ldn = cl.ldn;
  const int ROWS = (ny + 31) & ~31;
  const int NSL = kNT / ROWS;
  const int JS = (ny + NSL - 1) / NSL;

  // shared layout
  DevSlot* sl = reinterpret_cast<DevSlot*>(smem);
  SlotCoef* cf = reinterpret_cast<SlotCoef*>(sl + RMAX);
  DevGroup* gr = reinterpret_cast<DevGroup*>(cf + RMAX);
  C* V = reinterpret_cast<C*>(gr + RMAX);          // [RMAX][ldn]  forward: r_k; backward: x_{k+1}
  C* red = V + RMAX * ldn;                         // [NSL][RMAX][ROWS]
  C* X = red + (size_t)NSL * RMAX * ROWS;          // [RMAX][ldn]  backward x_k

  const C* tr = reinterpret_cast<const C*>(a.traces);
  C* trw = reinterpret_cast<C*>(a.traces);
  const C* fac = reinterpret_cast<const C*>(a.fac) + cl.fac_off;
  C* scr = reinterpret_cast<C*>(a.scratch) + it.scratch_off;
  C* outs = reinterpret_cast<C*>(a.outs);
  const double2* px = a.prof + cl.prof_off;         // lo_x[nx], hi_x[nx], dg_x[nx], lo_y[ny], hi_y[ny], dg_y[ny]
  const double2* py = px + 3 * nx;

  for (int i = tid; i < R; i += kNT) {
    const DevSlot s = a.slots[it.slot_begin + i];
    sl[i] = s;
    SlotCoef c{};
    if (s.kind == SK_DIR_X || s.kind == SK_CORNER) {
      c.c_oi_x = s.dx > 0 ? px[nx + s.xo] : px[s.xo];
      c.c_io_x = s.dx > 0 ? px[s.xi] : px[nx + s.xi];
    }
    if (s.kind == SK_DIR_Y || s.kind == SK_CORNER) {
      c.c_oi_y = s.dy > 0 ? py[ny + s.yo] : py[s.yo];
      c.c_io_y = s.dy > 0 ? py[s.yi] : py[ny + s.yi];
    }
    cf[i] = c;
  }
  for (int i = tid; i < it.group_count; i += kNT) gr[i] = a.groups[it.group_begin + i];
  __syncthreads();

  // r_0 = b_0
  for (int e = tid; e < R * ny; e += kNT) {
    const int r = e / ny, j = e - r * ny;
    V[r * ldn + j] = rhs_elem<T>(a, cl, sl[r], cf[r], tr, 0, j);
  }
  __syncthreads();

  const int row = tid % ROWS, sli = tid / ROWS;
  const int j0 = sli * JS, j1 = min(j0 + JS, ny);

  // y = S * V for all slots; partial sums over the j-slices land in red.
  auto matvec = [&](const C* S, const C* Vin) {
    if (sli < NSL) {
      C acc[RMAX];
#pragma unroll
      for (int r = 0; r < RMAX; ++r) acc[r] = czero<C>();
      if (row < ny) {
        const C* col = S + (size_t)j0 * ldn + row;
        int j = j0;
        for (; j + 4 <= j1; j += 4) {
          C s0 = __ldcs(col); C s1 = __ldcs(col + ldn); C s2 = __ldcs(col + 2 * ldn); C s3 = __ldcs(col + 3 * ldn);
          col += 4 * ldn;
#pragma unroll
          for (int r = 0; r < RMAX; ++r)
            if (r < R) {
              const C* v = Vin + r * ldn + j;
              cfma(acc[r], s0, v[0]); cfma(acc[r], s1, v[1]); cfma(acc[r], s2, v[2]); cfma(acc[r], s3, v[3]);
            }
        }
        for (; j < j1; ++j) {
          C s0 = __ldcs(col); col += ldn;
#pragma unroll
          for (int r = 0; r < RMAX; ++r)
            if (r < R) cfma(acc[r], s0, Vin[r * ldn + j]);
        }
      }
#pragma unroll
      for (int r = 0; r < RMAX; ++r)
        if (r < R) red[((size_t)sli * RMAX + r) * ROWS + row] = acc[r];
    }
  };
  auto reduce_at = [&](int r, int i) {
    C s = red[(size_t)r * ROWS + i];
    for (int q = 1; q < NSL; ++q) s = cadd(s, red[((size_t)q * RMAX + r) * ROWS + i]);
    return s;
  };

  // ---------------- forward substitution ----------------
  for (int k = 0; k < nx; ++k) {
    matvec(fac + (size_t)k * ny * ldn, V);
    __syncthreads();
    const C wn = (k + 1 < nx) ? to_c(px[k + 1], czero<C>()) : czero<C>();
    for (int e = tid; e < R * ny; e += kNT) {
      const int r = e / ny, i = e - r * ny;
      const C y = reduce_at(r, i);
      scr[((size_t)k * R + r) * ldn + i] = y;
      if (k + 1 < nx) {
        C b = rhs_elem<T>(a, cl, sl[r], cf[r], tr, k + 1, i);
        cfms(b, wn, y);
        V[r * ldn + i] = b;
      } else {
        X[r * ldn + i] = y;   // x_{K-1} = y_{K-1}
      }
    }
    __syncthreads();
  }

  // ---------------- backward substitution + epilogue ----------------
  for (int k = nx - 1; k >= 0; --k) {
    if (k < nx - 1) {
      // V holds x_{k+1}
      matvec(fac + (size_t)k * ny * ldn, V);
      __syncthreads();
      const C ek = to_c(px[nx + k], czero<C>());
      for (int e = tid; e < R * ny; e += kNT) {
        const int r = e / ny, i = e - r * ny;
        C x = scr[((size_t)k * R + r) * ldn + i];
        cfms(x, ek, reduce_at(r, i));
        X[r * ldn + i] = x;
      }
      __syncthreads();
    }
    // epilogue on x_k (in X); also stage x_k as the next matvec input
    for (int e = tid; e < R * ny; e += kNT) {
      const int r = e / ny, i = e - r * ny;
      V[r * ldn + i] = X[r * ldn + i];
    }
    // owned-DOF accumulation, one output per (shift, rhs) group
    for (int g = 0; g < it.group_count; ++g) {
      const DevGroup G = gr[g];
      if (G.out_off < 0) continue;
      const int sx = G.shift & 1, sy = (G.shift >> 1) & 1;
      if (k < cl.ownx[sx][0] || k > cl.ownx[sx][1]) continue;
      const int ja = cl.owny[sy][0], jb = cl.owny[sy][1];
      C* o = outs + G.out_off + (long long)(cl.lox + k) * a.n_dof + cl.loy;
      for (int j = ja + tid; j <= jb; j += kNT) {
        C acc = o[j];
        for (int q = 0; q < G.slot_count; ++q) acc = cadd(acc, X[(G.slot_begin + q) * ldn + j]);
        o[j] = acc;
      }
    }
    // trace lines and full-cell outputs
    for (int r = 0; r < R; ++r) {
      const DevSlot& s = sl[r];
      if (s.kind == SK_CELLVEC) {
        double2* o = a.x_out + (long long)s.rhs * a.out_stride + (long long)k * ny;
        for (int j = tid; j < ny; j += kNT) o[j] = to_c(X[r * ldn + j], make_double2(0, 0));
        continue;
      }
      const bool ovx = s.overwrite && k == s.xo;
      for (int l = 0; l < s.n_lr; ++l) {
        if (s.lr_line[l] != k) continue;
        C* o = trw + s.lr_out[l];
        for (int j = tid; j < ny; j += kNT) {
          C v = X[r * ldn + j];
          if (s.overwrite) {
            if (j == s.yo) v = tr[s.in_ud0 + k];
            else if (ovx) v = tr[s.in_lr0 + j];
          }
          o[j] = cadd(o[j], v);
        }
      }
      if (tid < s.n_ud) {
        const int l = tid;
        const int j = s.ud_line[l];
        C v = X[r * ldn + j];
        if (s.overwrite) {
          if (j == s.yo) v = tr[s.in_ud0 + k];
          else if (ovx) v = tr[s.in_lr0 + j];
        }
        C* o = trw + s.ud_out[l] + k;
        *o = cadd(*o, v);
      }
    }
    __syncthreads();
  }
}

}  // namespace

template <typename T>
cudaError_t launch_front(const FrontArgs& a, int max_ny, cudaStream_t st) {
  if (a.item_count <= 0) return cudaSuccess;
  constexpr int RMAX = sizeof(T) == 4 ? 16 : 8;
  using C = cx_t<T>;
  const int ldn = (max_ny + 7) & ~7;
  // per-cell layout inside: V and X of RMAX*ldn each, partial sums of at most kNT*RMAX
  const size_t smem = RMAX * (sizeof(DevSlot) + sizeof(SlotCoef) + sizeof(DevGroup)) +
                      sizeof(C) * ((size_t)RMAX * ldn * 2 + (size_t)kNT * RMAX);
  auto kern = k_front<T, RMAX>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<a.item_count, kNT, smem, st>>>(a);
  return cudaGetLastError();
}

template cudaError_t launch_front<float>(const FrontArgs&, int, cudaStream_t);
template cudaError_t launch_front<double>(const FrontArgs&, int, cudaStream_t);

int front_rmax(bool dbl) { return dbl ? 8 : 16; }

}  // namespace lsw
