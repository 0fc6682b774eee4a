// Batched factorisation of every cell matrix (replaces the per-cell Eigen
// SparseLU of LocalLinearSolverEigenSparseLU::factorize,
// LocalLinearSolverEigenSparseLU.cpp:40-62).
//
// The cell matrix is block tridiagonal over its nx x-lines, with tridiagonal
// diagonal blocks D_k (5-point stencil along y) and couplings w_k I / e_k I to
// the neighbouring lines.  It is factorised from both ends towards the middle
// line m = (nx - 1) / 2 (a twisted block LU, "burn at both ends"): the
// Schur complements
//   top     S_0 = D_0,            S_k = D_k - w_k e_{k-1} S_{k-1}^{-1}   (k < m)
//   bottom  T_{nx-1} = D_{nx-1},  T_k = D_k - e_k w_{k+1} T_{k+1}^{-1}   (k > m)
//   middle  Z_m = D_m - w_m e_{m-1} S_{m-1}^{-1} - e_m w_{m+1} T_{m+1}^{-1}
// are inverted, and line k of the factor holds S_k^{-1}, Z_m^{-1} or
// T_k^{-1}, column-major (element (i, j) at j*ldn + i).  A solve then runs two
// independent chains of about nx / 2 lines each way instead of one chain of
// 2 nx - 1 lines (kernels_sweep.cu).  The two half chains of every cell run in
// one launch (a cluster per cell and half), the middle lines in a second.
//
// Each S_k is inverted in place by Gauss-Jordan elimination with partial
// pivoting on unpivoted rows (implicit row exchange, pivot order recorded;
// the inverse is unscrambled on the way out: Sinv[i][j] = W[piv[i]][pinv[j]]),
// blocked over B pivots (16 for complex64, 8 for complex128) so that the bulk of the work is a register-tiled
// rank-B update instead of B passes over the whole matrix:
//   * the panel (the B columns of the block) goes through the classic
//     Gauss-Jordan steps; column t of the panel at its step, f_t, and the
//     pivot p_t and 1/f_t[p_t] are recorded;
//   * every other column c then receives all B steps at once:
//       u_t = (c[p_t] - sum_{s<t} f_s[p_t] u_s) / f_t[p_t],
//       c[r] -= sum_t f_t[r] u_t            (rows r that are not block pivots),
//       c[p_t] = u_t - sum_{s>t} f_s[p_t] u_s,
//     which is exactly the result of the B classic steps.
//
// One thread-block cluster of G CTAs works on a cell: CTA g holds the column
// range [g n/G, (g+1) n/G) of the working matrix in shared memory (G = 2 for
// complex64, 4 for complex128 at the C2-C4 cell sizes), the CTA owning a
// panel publishes f_t, p_t and 1/f_t[p_t] through distributed shared memory,
// and the cluster meets once per block on an mbarrier (bounded waits: a wait
// that runs out sets bit 1 of *status and the CTA leaves).  A zero or
// non-finite pivot sets bit 0 of *status (the reference exits on a failed
// factorisation, LocalLinearSolverEigenSparseLU.cpp:54-58).
#include "common.cuh"
#include "internal.h"

#include <cuda_bf16.h>

#include <algorithm>
#include <type_traits>

namespace lsw {

namespace {

constexpr int kFT = 512;              // threads per CTA
constexpr int kTX = 16, kTY = 32;     // update tile grid (columns x rows)
constexpr int kRI = 6;                // rows per thread in the update: ny <= 192
constexpr int kMaxN = kRI * kTY;
constexpr unsigned kSuspendNs = 1000000;

template <typename T> struct FacCfg;
// CJ: columns per thread in the update tile; B: pivots per block
template <> struct FacCfg<float> { static constexpr int CJ = 6, B = 16; };
template <> struct FacCfg<double> { static constexpr int CJ = 3, B = 8; };

__device__ __forceinline__ unsigned saddr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_size() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned mapa(unsigned a, unsigned rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_remote(uint64_t* b, unsigned rank) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(mapa(saddr(b), rank))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity), "r"(kSuspendNs)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ float2 ld_remote(const float2* p, unsigned rank) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(mapa(saddr(p), rank))
               : "memory");
  return v;
}
__device__ __forceinline__ double2 ld_remote(const double2* p, unsigned rank) {
  double2 v;
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(mapa(saddr(p), rank))
               : "memory");
  return v;
}
__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
__device__ __forceinline__ int ld_remote(const int* p, unsigned rank) {
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(mapa(saddr(p), rank)) : "memory");
  return v;
}

// bf16 hi/lo terms of x: hi = rn(x), lo = rn(x - hi)
__device__ __forceinline__ void bf16_split(float x, unsigned& hi, unsigned& lo) {
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
  hi = (unsigned)__bfloat16_as_ushort(h);
  lo = (unsigned)__bfloat16_as_ushort(l);
}
// one factor entry of the split layout: {hi(re) | hi(im) << 16, lo(re) | lo(im) << 16}
__device__ __forceinline__ uint2 split_entry(float2 v) {
  unsigned hr, lr, hi_, li;
  bf16_split(v.x, hr, lr);
  bf16_split(v.y, hi_, li);
  return make_uint2(hr | (hi_ << 16), lr | (li << 16));
}

// block-column owner: CTA g owns the columns [g n/G, (g+1) n/G)
__device__ __forceinline__ int col_owner(int j, int n, int G) { return ((j + 1) * G - 1) / n; }

// Rank-bt update of the non-pivot rows on columns [cb, ce) of W except
// [x0, x1) (computed in the tiles, not stored): c[r] -= sum_t f_t[r] u_t,
// register-tiled (kRI rows x CJ columns per thread, kTX x CJ columns per pass)
// over NTHR threads; lt = thread index within them.
template <typename T, int NTHR, int CJ>
__device__ __forceinline__ void rank_update_body(const cx_t<T>* __restrict__ Fb, const cx_t<T>* __restrict__ U,
                                            cx_t<T>* __restrict__ W, const int* __restrict__ pslot, int n,
                                            int nmax, int ldw, int bt, int cb, int ce, int x0, int x1, int lt) {
  using C = cx_t<T>;
  constexpr int NTY = NTHR / kTX;
  const C z = czero<C>();
  const int tx = lt % kTX, ty = lt / kTX;
  for (int rb = 0; rb < n; rb += NTY * kRI) {
    C acc[kRI][CJ];
#pragma unroll
    for (int a = 0; a < kRI; ++a)
#pragma unroll
      for (int b = 0; b < CJ; ++b) acc[a][b] = z;
    for (int t = 0; t < bt; ++t) {
      C fr[kRI], uc[CJ];
#pragma unroll
      for (int a = 0; a < kRI; ++a) {
        const int r = rb + ty + NTY * a;
        fr[a] = r < n ? Fb[(size_t)t * nmax + r] : z;
      }
#pragma unroll
      for (int b = 0; b < CJ; ++b) {
        const int cc = cb + tx + kTX * b;
        uc[b] = cc < ce ? U[(size_t)t * ldw + cc] : z;
      }
#pragma unroll
      for (int a = 0; a < kRI; ++a)
#pragma unroll
        for (int b = 0; b < CJ; ++b) cfma(acc[a][b], fr[a], uc[b]);
    }
#pragma unroll
    for (int a = 0; a < kRI; ++a) {
      const int r = rb + ty + NTY * a;
      if (r >= n || pslot[r] >= 0) continue;
#pragma unroll
      for (int b = 0; b < CJ; ++b) {
        const int cc = cb + tx + kTX * b;
        if (cc >= ce || (cc >= x0 && cc < x1)) continue;
        C* w = W + (size_t)r * ldw + cc;
        *w = csub(*w, acc[a][b]);
      }
    }
  }
}

// complex64: a separate function, so that the kernel's other paths keep their
// registers; complex128 (bound by FP64 throughput): inlined
template <typename T, int NTHR, int CJ>
__device__ __noinline__ void rank_update_call(const cx_t<T>* __restrict__ Fb, const cx_t<T>* __restrict__ U,
                                                 cx_t<T>* __restrict__ W, const int* __restrict__ pslot, int n,
                                                 int nmax, int ldw, int bt, int cb, int ce, int x0, int x1,
                                                 int lt) {
  rank_update_body<T, NTHR, CJ>(Fb, U, W, pslot, n, nmax, ldw, bt, cb, ce, x0, x1, lt);
}
template <typename T, int NTHR, int CJ>
__device__ __forceinline__ void rank_update(const cx_t<T>* __restrict__ Fb, const cx_t<T>* __restrict__ U,
                                            cx_t<T>* __restrict__ W, const int* __restrict__ pslot, int n,
                                            int nmax, int ldw, int bt, int cb, int ce, int x0, int x1, int lt) {
  if constexpr (sizeof(T) == 4) rank_update_call<T, NTHR, CJ>(Fb, U, W, pslot, n, nmax, ldw, bt, cb, ce, x0, x1, lt);
  else rank_update_body<T, NTHR, CJ>(Fb, U, W, pslot, n, nmax, ldw, bt, cb, ce, x0, x1, lt);
}

template <typename T>
__global__ void __launch_bounds__(kFT, 1)
k_factorize(const DevCell* __restrict__ cells, const double2* __restrict__ prof,
            const double* __restrict__ mgrid, int n_dof, double omega2, cx_t<T>* __restrict__ fac,
            cx_t<T>* __restrict__ prev, long long prev_stride, int split, int middle, int lookahead, int G,
            int nmax, int ldw, int* status, long long wait_cycles) {
  using C = cx_t<T>;
  constexpr int CJ = FacCfg<T>::CJ;
  constexpr int kB = FacCfg<T>::B;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned g = G > 1 ? cluster_rank() : 0u;
  if (G > 1 && (cluster_size() != (unsigned)G || g != blockIdx.x % (unsigned)G)) {
    if (tid == 0) atomicOr(status, 4);   // the launch did not form the expected clusters
    return;
  }
  // middle == 0: cluster (cell, half) runs the top (half 0) or bottom (half 1)
  // chain; middle == 1: cluster `cell` forms and inverts Z_m
  const int cidx = middle ? (int)(blockIdx.x / G) : (int)(blockIdx.x / (2 * G));
  const int half = middle ? 0 : (int)((blockIdx.x / G) & 1);
  const DevCell cl = cells[cidx];
  const int n = cl.ny, nx = cl.nx, ldn = cl.ldn;
  const int mid = (nx - 1) / 2;
  const int nsteps = middle ? 1 : (half == 0 ? mid : nx - 1 - mid);
  const int c0 = (int)g * n / G, c1 = ((int)g + 1) * n / G, nc = c1 - c0;

  // ---- shared layout (identical in every CTA of the cluster) ----
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 8);
  unsigned* wkey = reinterpret_cast<unsigned*>(smem + 16);    // [2][8] per-warp pivot keys by step parity
  uint64_t* exitbar = reinterpret_cast<uint64_t*>(smem + 128); // every CTA of the cluster is done
  int* used = reinterpret_cast<int*>(smem + 256);             // [nmax]
  int* piv = used + kMaxN;                                     // [nmax]
  int* pslot = piv + kMaxN;                                    // [nmax] block pivot slot of a row, -1 if none
  int* pb = pslot + kMaxN;                                     // [2][kB]
  C* invv = reinterpret_cast<C*>(pb + 2 * kB);                 // [2][kB]
  C* M1 = invv + 2 * kB;                                       // [kB][kB]
  C* F = M1 + kB * kB;                                         // [2][kB][nmax]
  C* U = F + 2 * kB * nmax;                                    // [kB][ldw]
  C* W = U + kB * ldw;                                         // [nmax][ldw], my columns
  C* RowB = W + (size_t)nmax * ldw;                            // [2][kB][kMaxN] panel rows by step parity

  const double2* px = prof + cl.prof_off;  // lo_x, hi_x, dg_x, lo_y, hi_y, dg_y
  const double2* py = px + 3 * nx;
  C* Fac = fac + cl.fac_off;
  // split: the last inverse of each half chain in FP32, [cell][half]
  C* Prev0 = prev ? prev + (long long)(2 * cidx) * prev_stride : nullptr;
  C* Prev1 = prev ? Prev0 + prev_stride : nullptr;
  C* Prev = half ? Prev1 : Prev0;
  const C z = czero<C>();

  if (tid == 0) {
    *abort_flag = 0;
    mbar_init(bar, (unsigned)G);
    mbar_init(exitbar, (unsigned)G);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = tid; i < kMaxN; i += kFT) pslot[i] = -1;
  __syncthreads();
  if (G > 1) asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");

  // cluster-wide barrier: every CTA's thread t < G arrives on CTA t's
  // mbarrier (release after the CTA barrier, so it covers every thread's
  // writes), then every thread waits for its own CTA's phase (acquire)
  unsigned phase = 0;
  auto csync = [&]() -> bool {
    __syncthreads();
    if (G == 1) return true;
    if (tid < G) mbar_arrive_remote(bar, (unsigned)tid);
    bool ok = mbar_try_wait_cluster(bar, phase & 1u);
    if (!ok) {
      const long long t0 = clock64();
      while (!(ok = mbar_try_wait_cluster(bar, phase & 1u))) {
        if (*abort_flag) break;
        if (clock64() - t0 > wait_cycles) {
          *abort_flag = 1;
          atomicOr(status, 2);
          break;
        }
      }
    }
    ++phase;
    __syncthreads();
    return *abort_flag == 0;
  };
  // Before leaving, normally or after a wait gave up: every CTA arrives on
  // every CTA's exit barrier and waits for its own, bounded by the limit
  // alone, so that no CTA leaves while a peer may still read its shared
  // memory (the panel columns, pivots and reciprocals).
  auto leave = [&]() {
    __syncthreads();
    if (G == 1) return;
    if (tid < G) mbar_arrive_remote(exitbar, (unsigned)tid);
    if (mbar_try_wait_cluster(exitbar, 0u)) return;
    const long long t0 = clock64();
    while (!mbar_try_wait_cluster(exitbar, 0u)) {
      if (clock64() - t0 > wait_cycles) {
        atomicOr(status, 2);
        break;
      }
    }
  };

  for (int step = 0; step < nsteps; ++step) {
    const int k = middle ? mid : (half == 0 ? step : nx - 1 - step);
    // ---- Schur complement of line k, my columns, into W (row-major) ----
    // one or two coupled neighbour inverses: the previous line of the chain,
    // or both neighbours of the middle line
    const C dgx = to_c(px[2 * nx + k], z);
    C coupa = z, coupb = z;
    const C* Fa = nullptr;
    const C* Fb = nullptr;
    if (middle) {
      coupa = cmul(to_c(px[k], z), to_c(px[nx + k - 1], z));   // w_m e_{m-1}
      coupb = cmul(to_c(px[nx + k], z), to_c(px[k + 1], z));   // e_m w_{m+1}
      Fa = split ? Prev0 : Fac + (size_t)(k - 1) * n * ldn;
      Fb = split ? Prev1 : Fac + (size_t)(k + 1) * n * ldn;
    } else if (step > 0) {
      const int kp = half == 0 ? k - 1 : k + 1;
      coupa = half == 0 ? cmul(to_c(px[k], z), to_c(px[nx + k - 1], z))    // w_k e_{k-1}
                        : cmul(to_c(px[nx + k], z), to_c(px[k + 1], z));   // e_k w_{k+1}
      Fa = split ? Prev : Fac + (size_t)kp * n * ldn;
    }
    const double* mrow = mgrid + (long long)(cl.lox + k) * n_dof + cl.loy;
    for (int e = tid; e < n * nc; e += kFT) {
      const int cc = e / n, i = e - cc * n, j = c0 + cc;
      C v = z;
      if (Fa) v = cneg(cmul(coupa, Fa[(size_t)j * ldn + i]));
      if (Fb) cfms(v, coupb, Fb[(size_t)j * ldn + i]);
      if (j == i) {
        C d = cadd(dgx, to_c(py[2 * n + i], z));
        d.x -= (T)(omega2 * mrow[i]);
        v = cadd(v, d);
      } else if (j == i - 1) {
        v = cadd(v, to_c(py[i], z));          // coupling to j-1 (south)
      } else if (j == i + 1) {
        v = cadd(v, to_c(py[n + i], z));      // coupling to j+1 (north)
      }
      W[(size_t)i * ldw + cc] = v;
    }
    for (int i = tid; i < n; i += kFT) used[i] = 0;
    __syncthreads();

    // ---- blocked Gauss-Jordan over the pivot columns in order ----
    // Panel of block [k0, k1): the classic Gauss-Jordan steps on those columns of
    // my W (pc = k0 - first column of mine), one row per thread of warps
    // 0 .. kMaxN/32 - 1, the row's panel part in registers; records f_t, the
    // pivots and the reciprocals in buffer `buf`.  Each step publishes every row's
    // panel values (RowB, double-buffered by step parity, so a fast thread's next
    // step cannot overwrite a row a slow thread still reads) and its pivot key
    // before one named barrier; after it every thread picks the pivot row and
    // applies the step itself.  Pivot key: the bits of |v|^2 as float (monotone
    // for non-negative values) with the low byte replaced by 255 - row, so the
    // warp maximum (one redux) is the largest magnitude, ties (to 2^-15) going to
    // the lowest row; used rows have key 0.
    auto panel = [&](int k0, int k1, int buf) {
      const int pc = k0 - c0;
      const int bt = k1 - k0;
      C* Fb = F + (size_t)buf * kB * nmax;
      int* pbb = pb + buf * kB;
      C* ivb = invv + buf * kB;
      const int r = tid;
      const bool live = r < n;
      C row[kB];
#pragma unroll
      for (int q = 0; q < kB; ++q) row[q] = (live && q < bt) ? W[(size_t)r * ldw + pc + q] : z;
      bool mine_used = live ? (used[r] != 0) : true;
#pragma unroll
      for (int t = 0; t < kB; ++t) {
        if (t >= bt) break;
        C* RB = RowB + (size_t)(t & 1) * kB * kMaxN;
        const C v = row[t];
        if (live) {
          Fb[(size_t)t * nmax + r] = v;
#pragma unroll
          for (int q = 0; q < kB; ++q)
            if (q < bt) RB[(size_t)q * kMaxN + r] = row[q];
        }
        unsigned key = 0u;
        if (live && !mine_used)
          key = (__float_as_uint((float)abs2(v)) & 0xffffff00u) | (unsigned)(255 - r);
        key = __reduce_max_sync(0xffffffffu, key);
        unsigned* wk = wkey + (t & 1) * 8;   // by step parity, like RowB
        if (lane == 0) wk[warp] = key;
        named_sync(1, kMaxN);
        unsigned best = wk[0];
#pragma unroll
        for (int w = 1; w < kMaxN / 32; ++w) best = max(best, wk[w]);
        // best < 256: no unpivoted row with a positive magnitude (singular);
        // the step still runs (on the lowest unpivoted row) so that the kernel
        // terminates normally, and the status says the factor is invalid
        if (best < 256u && r == 0) atomicOr(status, 1);
        const int p = best ? 255 - (int)(best & 0xffu) : 0;
        const C pv = RB[(size_t)t * kMaxN + p];
        if (r == 0 && !isfinite(abs2(pv))) atomicOr(status, 1);   // in T: FP64 is slow on this part
        const C inv = crcp(pv);
        if (r == p) {
          mine_used = true;
          used[r] = 1;
          piv[k0 + t] = r;
          pbb[t] = r;
          ivb[t] = inv;
#pragma unroll
          for (int q = 0; q < kB; ++q)
            if (q < bt) row[q] = (q == t) ? inv : cmul(row[q], inv);
        } else if (live) {
#pragma unroll
          for (int q = 0; q < kB; ++q) {
            if (q < bt) {
              if (q == t) row[q] = cneg(cmul(v, inv));
              else cfms(row[q], v, cmul(RB[(size_t)q * kMaxN + p], inv));
            }
          }
        }
      }
#pragma unroll
      for (int q = 0; q < kB; ++q)
        if (live && q < bt) W[(size_t)r * ldw + pc + q] = row[q];
    };

    // Block of bt pivots (buffer `buf`) on my columns [cb, ce) except
    // [x0, x1): u = M1 g per column, the pivot rows' final values
    // c[p_t] = u_t - sum_{s>t} f_s[p_t] u_s, and the rank-bt update
    // c[r] -= sum_t f_t[r] u_t of the other rows.  All kFT threads
    // (NTHR = kFT, CTA barrier) or the kFT - kMaxN threads past the panel
    // warps (named barrier 2) take part.
    auto finish = [&](auto nthr_c, int bt, int buf, int cb, int ce, int x0, int x1) {
      constexpr int NTHR = decltype(nthr_c)::value;
      const int lt = tid - (kFT - NTHR);
      const C* Fb = F + (size_t)buf * kB * nmax;
      const int* pbb = pb + buf * kB;
      // two contiguous column ranges [cb, xa) and [xb, ce)
      const int xa = max(cb, min(x0, ce)), xb = max(xa, min(x1, ce));
      const int na = xa - cb, ncols = na + (ce - xb);
      auto colof = [&](int i) { return i < na ? cb + i : xb + (i - na); };
      for (int e = lt; e < bt * ncols; e += NTHR) {
        const int t = e / ncols, cc = colof(e - t * ncols);
        C a = z;
        for (int s2 = 0; s2 <= t; ++s2) cfma(a, M1[t * kB + s2], W[(size_t)pbb[s2] * ldw + cc]);
        U[(size_t)t * ldw + cc] = a;
      }
      if (NTHR == kFT) __syncthreads();
      else named_sync(2, NTHR);
      // pivot rows, then (no barrier: disjoint rows, reading only U and F) the others
      for (int e = lt; e < bt * ncols; e += NTHR) {
        const int t = e / ncols, cc = colof(e - t * ncols);
        C a = U[(size_t)t * ldw + cc];
        const int pt = pbb[t];
        for (int s2 = t + 1; s2 < bt; ++s2) cfms(a, Fb[(size_t)s2 * nmax + pt], U[(size_t)s2 * ldw + cc]);
        W[(size_t)pt * ldw + cc] = a;
      }
      // one tiled pass over [cb, ce) that stores nothing in [xa, xb) (their
      // products use stale U and are dropped); one column per thread where
      // the range is at most kTX wide
      if (ncols > 0) {
        if (ce - cb <= kTX) rank_update<T, NTHR, 1>(Fb, U, W, pslot, n, nmax, ldw, bt, cb, ce, xa, xb, lt);
        else rank_update<T, NTHR, CJ>(Fb, U, W, pslot, n, nmax, ldw, bt, cb, ce, xa, xb, lt);
      }
    };
    using AllThreads = std::integral_constant<int, kFT>;
    using RestThreads = std::integral_constant<int, kFT - kMaxN>;

    // Look-ahead: the owner of the next block's columns finishes the current
    // block on those columns first, then factors the next panel on warps
    // 0 .. kMaxN/32 - 1 while its other warps finish the current block on the
    // rest of its columns; the cluster sync that follows publishes the panel.
    // Iteration blk = -1 has no current block and only factors the first panel.
    int k0 = 0, k1 = 0;   // current block [k0, k1); the next one starts at k1
    for (int blk = -1;; ++blk) {
      const bool cur = blk >= 0;
      const int o = cur ? col_owner(k0, n, G) : -1;
      const int bt = k1 - k0, buf = blk & 1;
      C* Fb = F + (size_t)buf * kB * nmax;
      int* pbb = pb + buf * kB;
      C* ivb = invv + buf * kB;
      const bool more = k1 < n;
      const int o2 = more ? col_owner(k1, n, G) : -1;
      const int k2 = more ? min(k1 + kB, (o2 + 1) * n / G) : k1;

      if (cur) {
        if (!csync()) { leave(); return; }
        if ((int)g != o) {
          // the panel owner's columns f_t, pivots and reciprocals
          for (int e = tid; e < bt * n; e += kFT) {
            const int t = e / n, r = e - t * n;
            Fb[(size_t)t * nmax + r] = ld_remote(Fb + (size_t)t * nmax + r, (unsigned)o);
          }
          if (tid < bt) {
            const int p = ld_remote(pbb + tid, (unsigned)o);
            pbb[tid] = p;
            ivb[tid] = ld_remote(ivb + tid, (unsigned)o);
            used[p] = 1;
            piv[k0 + tid] = p;
          }
          __syncthreads();
        }
        if (tid < bt) pslot[pbb[tid]] = tid;
        // M1 = (D + L)^{-1} (D = diag f_t[p_t], L[t][s] = f_s[p_t], s < t),
        // formed once per block by one warp, lane j solving for column j
        if (warp == 0 && lane < bt) {
          C m[kB];
#pragma unroll
          for (int t = 0; t < kB; ++t) {
            if (t < bt) {
              C a = (t == lane) ? to_c(make_double2(1.0, 0.0), z) : z;
#pragma unroll
              for (int s2 = 0; s2 < kB; ++s2)
                if (s2 < t) cfms(a, Fb[(size_t)s2 * nmax + pbb[t]], m[s2]);
              m[t] = cmul(a, ivb[t]);
              M1[t * kB + lane] = m[t];
            }
          }
        }
        __syncthreads();
      }
      // the owner of the next block factors its panel: with look-ahead on its
      // panel warps while its other warps finish the current block, otherwise
      // after the whole update
      const bool own_next = more && (int)g == o2;
      const bool overlap = own_next && cur && lookahead != 0;
      const int pk0 = (cur && (int)g == o) ? k0 - c0 : -1;   // my panel columns [pk0, pk0 + bt), if any
      const int n0 = k1 - c0, n1 = k2 - c0;                  // the next panel's columns, if mine
      if (overlap) {
        finish(AllThreads{}, bt, buf, n0, n1, -1, -1);
        __syncthreads();
      }
      if (cur && !(overlap && tid < kMaxN)) {
        if (overlap) finish(RestThreads{}, bt, buf, 0, nc, pk0 >= 0 ? pk0 : n0, n1);
        else finish(AllThreads{}, bt, buf, 0, nc, pk0, pk0 >= 0 ? pk0 + bt : -1);
      }
      if (cur && !overlap) __syncthreads();
      if (own_next && tid < kMaxN) panel(k1, k2, (blk + 1) & 1);
      __syncthreads();
      if (cur) {
        if (tid < bt) pslot[pbb[tid]] = -1;
        __syncthreads();
      }
      if (!more) break;
      k0 = k1;
      k1 = k2;
    }

    // ---- unscramble my columns: output column piv[c] holds W[piv[i]][c] ----
    C* Fk = Fac + (size_t)k * n * ldn;
    for (int e = tid; e < nc * ldn; e += kFT) {
      const int cc = e / ldn, i = e - cc * ldn;
      const int j = piv[c0 + cc];
      const C v = (i < n) ? W[(size_t)piv[i] * ldw + cc] : z;
      if constexpr (sizeof(T) == 4) {
        if (split) {
          if (!middle) Prev[(size_t)j * ldn + i] = v;
          reinterpret_cast<uint2*>(Fk)[(size_t)j * ldn + i] = split_entry(v);
          continue;
        }
      }
      Fk[(size_t)j * ldn + i] = v;
    }
    // the next line's Schur complement reads every CTA's columns of Sinv_k
    if (!csync()) { leave(); return; }
  }
  leave();
}

template <typename T>
size_t fac_smem(int nmax, int ldw) {
  using C = cx_t<T>;
  constexpr int kB = FacCfg<T>::B;
  return 256 + 3 * (size_t)kMaxN * sizeof(int) + 2 * kB * sizeof(int) + (2 * kB + kB * kB) * sizeof(C) +
         2 * (size_t)kB * nmax * sizeof(C) + (size_t)kB * ldw * sizeof(C) + (size_t)nmax * ldw * sizeof(C) +
         2 * (size_t)kB * kMaxN * sizeof(C);
}

// smallest cluster whose column slices fit the update tiles and shared memory
template <typename T>
int fac_cluster(int nmax, int maxopt, int* ldw_out) {
  for (int G = 1; G <= 8; G *= 2) {
    const int ldw = (nmax + G - 1) / G;
    if (ldw > kTX * FacCfg<T>::CJ) continue;
    if (fac_smem<T>(nmax, ldw) <= (size_t)maxopt) {
      *ldw_out = ldw;
      return G;
    }
  }
  return 0;
}

}  // namespace

size_t factor_smem_bytes(int ny, bool dbl) {
  int dev = 0, maxopt = 0, ldw = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const int G = dbl ? fac_cluster<double>(ny, maxopt, &ldw) : fac_cluster<float>(ny, maxopt, &ldw);
  if (G == 0) return 0;
  return dbl ? fac_smem<double>(ny, ldw) : fac_smem<float>(ny, ldw);
}

template <typename T>
cudaError_t launch_factorize(const DevCell* cells, int ncell, const double2* prof, const double* mgrid,
                             int n_dof, double omega2, void* fac, void* prev, int max_ny, int* status,
                             cudaStream_t st, bool split, bool lookahead, long long wait_cycles) {
  if (ncell <= 0) return cudaSuccess;
  if (max_ny > kMaxN) return cudaErrorInvalidValue;
  int dev = 0, maxopt = 0, ldw = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const int G = fac_cluster<T>(max_ny, maxopt, &ldw);
  if (G == 0) return cudaErrorInvalidConfiguration;
  const size_t smem = fac_smem<T>(max_ny, ldw);
  auto kern = k_factorize<T>;
  // the attribute is an upper bound: always the device maximum, so that
  // host threads launching concurrently never lower it under one another
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, maxopt);
  if (e != cudaSuccess) return e;
  if (split && (sizeof(T) != 4 || prev == nullptr)) return cudaErrorInvalidValue;
  // split: the last FP32 inverse of each half chain, max_ny x ldn_max complex
  // per (cell, half) (ldn_max <= max_ny + 7)
  const long long prev_stride = (long long)max_ny * (max_ny + 8);
  cudaLaunchConfig_t cfg{};
  cudaLaunchAttribute attr[1];
  cfg.blockDim = dim3(kFT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  // both half chains of every cell, then every middle line (stream order)
  for (int middle = 0; middle < 2; ++middle) {
    cfg.gridDim = dim3((unsigned)(ncell * G * (middle ? 1 : 2)));
    e = cudaLaunchKernelEx(&cfg, kern, cells, prof, mgrid, n_dof, omega2, reinterpret_cast<cx_t<T>*>(fac),
                           reinterpret_cast<cx_t<T>*>(split ? prev : nullptr), prev_stride, split ? 1 : 0, middle,
                           lookahead ? 1 : 0, G, max_ny, ldw, status, wait_cycles);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}


template cudaError_t launch_factorize<float>(const DevCell*, int, const double2*, const double*, int, double,
                                             void*, void*, int, int*, cudaStream_t, bool, bool, long long);
template cudaError_t launch_factorize<double>(const DevCell*, int, const double2*, const double*, int, double,
                                              void*, void*, int, int*, cudaStream_t, bool, bool, long long);

}  // namespace lsw
