// Tensor-core factorisation of every cell matrix, complex64 and bf16-split
// outputs (replaces the per-cell Eigen SparseLU of
// LocalLinearSolverEigenSparseLU::factorize,
// LocalLinearSolverEigenSparseLU.cpp:40-62).
//
// Same algorithm as kernels_factor.cu -- the twisted block LU of the block-
// tridiagonal cell matrix, each Schur complement inverted in place by
// Gauss-Jordan elimination with partial pivoting, blocked over B = 16 pivots
// -- with the working matrix held in tensor memory and the O(n^3) part on the
// tensor cores:
//   * TMEM holds the CTA's column slice of the working matrix W as an FP32
//     accumulator: row r in lane r % 128 of 128-row tile r / 128, complex
//     column c in the two 32-bit columns 2c (real) and 2c + 1 (imaginary).
//     One thread per row: thread r reads and writes its row with tcgen05.ld /
//     tcgen05.st.
//   * The panel (the B columns of a block, on the CTA that owns them) runs the
//     classic Gauss-Jordan steps with each row's panel part in its thread's
//     registers, one CTA barrier per step: each warp's candidate row (its
//     largest unpivoted magnitude, one warp reduction) writes its panel values
//     and the warp's key before the barrier (double-buffered by step parity);
//     after it every thread reads the pivot row and applies the step.  It
//     records f_t (column t at step t), the pivots p_t and 1 / f_t[p_t].
//   * Every other column then receives the B steps at once.  With
//     u = M1 g (g the pivot rows, M1 = (D + L)^-1 of the pivots' f values)
//     the rank-B update of the rows that are not pivots of the block is one
//     product:
//         W[r][c] -= sum_t f_t[r] u_t[c],
//     issued as tcgen05.mma kind::f16 from shared-memory operand tiles into
//     the TMEM accumulator: the complex product as a real one (A = [Re f |
//     Im f] interleaved along k, B holding (Re u, -Im u) and (Im u, Re u)
//     per output column pair), each FP32 operand split into three bf16 terms
//     (hi + mid + lo, 24 significant bits) and the six products whose terms
//     reach 2^-16 accumulated in FP32 (the neglected ones are below 2^-23 of
//     the product).  The pivot rows of the block take the MMA with zero A
//     rows and get their final values c[p_t] = u_t - sum_{s>t} f_s[p_t] u_s
//     on the CUDA cores afterwards: written as one product with the pivot
//     rows included, W[p_t] - sum f u + u_t would cancel terms of the size of
//     the matrix entries (1/h^2) down to the size of the inverse's (h^2).
//     The panel's own columns get u = 0.
//   * Unscrambled column-major into the factor pool through a shared-memory
//     staging tile (Sinv[i][j] = W[piv[i]][pinv[j]]).
// A thread-block cluster of G CTAs (G = 2 for cells of 97-192 DOFs per side)
// splits the columns; after the cluster barrier that follows a panel the
// other CTAs read its f_t, p_t and 1/f_t[p_t] from the owner's shared memory
// (distributed shared memory), and the cluster meets once per block on an
// mbarrier.  Every wait is bounded (a wait that runs out sets bit 1 of
// *status, later waits return at once, TMEM is released and the CTA leaves
// after the cluster's exit rendezvous).  A zero or non-finite pivot sets bit 0.
#include "common.cuh"
#include "internal.h"

#include <cuda_bf16.h>

#include <algorithm>

namespace lsw {

namespace {

constexpr int kT = 256;            // threads per CTA: one per row of two 128-row tiles
constexpr int kB = 16;             // pivots per block
constexpr int kMaxRows = 192;      // cell DOFs per side
constexpr int kMaxCols = 96;       // complex columns per CTA
constexpr unsigned kTmemCols = 512;
constexpr unsigned kSuspendNs = 1000000;

// shared layout (bytes)
constexpr int kATerm = 16384;                       // [256 rows][32 k] bf16, canonical K-major: one split term
constexpr int kBTerm = 12288;                       // [192 rows][32 k] bf16
constexpr int kOffA = 0;                            // three terms: hi, mid, lo
constexpr int kOffB = 3 * kATerm;
constexpr int kOffF = kOffB + 3 * kBTerm;           // float2 [2][kB][kMaxRows]
constexpr int kOffGU = kOffF + 2 * kB * kMaxRows * 8;              // float2 [kB][kMaxCols]
constexpr int kOffU = kOffGU + kB * kMaxCols * 8;                  // float2 [kB][kMaxCols]
constexpr int kOffRB = kOffU + kB * kMaxCols * 8;                  // float2 [2][8 warps][kB]
constexpr int kOffInv = kOffRB + 2 * 8 * kB * 8;                   // float2 [2][kB]
constexpr int kOffM1 = kOffInv + 2 * kB * 8;                       // float2 [kB][kB]
constexpr int kOffInts = kOffM1 + kB * kB * 8;                     // used, piv, pslot, pinv [kMaxRows] each
constexpr int kOffPb = kOffInts + 4 * kMaxRows * 4;                // int [2][kB]
constexpr int kOffKey = kOffPb + 2 * kB * 4;                       // unsigned [2][8]
constexpr int kOffBar = kOffKey + 64;                              // 3 mbarriers
constexpr int kOffMisc = kOffBar + 24;                             // abort flag, TMEM address
constexpr int kSmem = kOffMisc + 16;
static_assert(kOffF == 86016, "layout");
static_assert(16 * kMaxRows * 8 <= 3 * kATerm, "unscramble staging tile [16][ldn] fits in the A operand area");
static_assert(kOffBar % 8 == 0, "mbarrier alignment");
static_assert(kMaxRows <= kT - 32, "the last warp holds no matrix row (it forms M1)");

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
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity), "r"(kSuspendNs)
      : "memory");
  return ok != 0;
}
// loads from CTA `rank`'s shared memory at the offset of p (after a cluster
// barrier that ordered the owner's writes)
__device__ __forceinline__ float4 ld_remote4(const float4* p, unsigned rank) {
  float4 v;
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(mapa(saddr(p), rank)));
  return v;
}
__device__ __forceinline__ float2 ld_remote(const float2* p, unsigned rank) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(mapa(saddr(p), rank)));
  return v;
}
__device__ __forceinline__ int ld_remote(const int* p, unsigned rank) {
  int v;
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(mapa(saddr(p), rank)));
  return v;
}
__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// ---- tensor memory and tensor-core helpers --------------------------------
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// 32 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tm_ld32(unsigned taddr, float (&v)[32]) {
  unsigned r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}
__device__ __forceinline__ void tm_st32(unsigned taddr, const float (&v)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
      "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
      "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])),
      "r"(__float_as_uint(v[11])), "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])),
      "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15])), "r"(__float_as_uint(v[16])),
      "r"(__float_as_uint(v[17])), "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])),
      "r"(__float_as_uint(v[20])), "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])),
      "r"(__float_as_uint(v[23])), "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])),
      "r"(__float_as_uint(v[26])), "r"(__float_as_uint(v[27])), "r"(__float_as_uint(v[28])),
      "r"(__float_as_uint(v[29])), "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
      : "memory");
}
__device__ __forceinline__ void tm_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// byte offset of element (row, k) in a [rows x 32] bf16 tile in the canonical
// K-major layout without swizzle: 8-row x 16-byte core matrices (8 k each),
// k-adjacent core matrices 128 B apart (leading-dimension offset), 8-row
// groups 512 B apart (stride-dimension offset)
__device__ __forceinline__ int kmaj(int row, int k) {
  return (row >> 3) * 512 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}
// shared-memory matrix descriptor (tcgen05 format: start, leading and stride
// byte offsets in 16-byte units, version 1, no swizzle)
__device__ __forceinline__ uint64_t sdesc(unsigned addr) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(512u >> 4) << 32) |
         (1ull << 46);
}
// (a, b) as three bf16x2 terms hi + mid + lo (each the rounded remainder of
// the previous ones; the remainders are exact in FP32), a in the low half, at
// byte offset `off` (4-byte aligned: k even) of the three term tiles `term`
// bytes apart
__device__ __forceinline__ void put3(unsigned char* base, int term, int off, float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float ra = a - __low2float(h), rb = b - __high2float(h);
  const __nv_bfloat162 m = __floats2bfloat162_rn(ra, rb);
  const __nv_bfloat162 l = __floats2bfloat162_rn(ra - __low2float(m), rb - __high2float(m));
  *reinterpret_cast<__nv_bfloat162*>(base + off) = h;
  *reinterpret_cast<__nv_bfloat162*>(base + term + off) = m;
  *reinterpret_cast<__nv_bfloat162*>(base + 2 * term + off) = l;
}
// D (TMEM, FP32) += A B with A, B bf16 from shared memory (A negated by the
// instruction descriptor)
__device__ __forceinline__ void mma_bf16(unsigned d, uint64_t a, uint64_t b, unsigned idesc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, 1, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
          d),
      "l"(a), "l"(b), "r"(idesc)
      : "memory");
}

// bf16 hi/lo terms of x: hi = rn(x), lo = rn(x - hi)
__device__ __forceinline__ void bf16_split(float x, unsigned& hi, unsigned& lo) {
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
  hi = (unsigned)__bfloat16_as_ushort(h);
  lo = (unsigned)__bfloat16_as_ushort(l);
}
__device__ __forceinline__ uint2 split_entry(float2 v) {
  unsigned hr, lr, hi_, li;
  bf16_split(v.x, hr, lr);
  bf16_split(v.y, hi_, li);
  return make_uint2(hr | (hi_ << 16), lr | (li << 16));
}

__device__ __forceinline__ int col_owner(int j, int n, int G) { return ((j + 1) * G - 1) / n; }

__global__ void __launch_bounds__(kT, 1)
k_factorize_tc(const DevCell* __restrict__ cells, const double2* __restrict__ prof, const double* __restrict__ mgrid,
               int n_dof, double omega2, float2* __restrict__ fac, float2* __restrict__ prev, long long prev_stride,
               int split, int middle, int G, int* status, long long wait_cycles) {
  using C = float2;
  extern __shared__ __align__(1024) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned g = G > 1 ? cluster_rank() : 0u;
  if (G > 1 && (cluster_size() != (unsigned)G || g != blockIdx.x % (unsigned)G)) {
    if (tid == 0) atomicOr(status, 4);   // the launch did not form the expected clusters
    return;
  }
  const int cidx = middle ? (int)(blockIdx.x / G) : (int)(blockIdx.x / (2 * G));
  const int half = middle ? 0 : (int)((blockIdx.x / G) & 1);
  const DevCell cl = cells[cidx];
  const int n = cl.ny, nx = cl.nx, ldn = cl.ldn;
  const int mid = (nx - 1) / 2;
  const int nsteps = middle ? 1 : (half == 0 ? mid : nx - 1 - mid);
  const int c0 = (int)g * n / G, c1 = ((int)g + 1) * n / G, nc = c1 - c0;
  const int NP = ((2 * nc + 15) / 16) * 16;          // MMA N: both parts of every column, padded
  const int ntiles = n > 128 ? 2 : 1;
  const int r = tid;                                  // my row
  const bool live = r < n;
  const bool warp_rows = 32 * warp < n;               // my warp holds a row of the matrix

  unsigned char* Aop = smem + kOffA;
  unsigned char* Bop = smem + kOffB;
  C* F = reinterpret_cast<C*>(smem + kOffF);          // [2][kB][kMaxRows]
  C* GU = reinterpret_cast<C*>(smem + kOffGU);        // [kB][kMaxCols] pivot rows g, then their final values
  C* U = reinterpret_cast<C*>(smem + kOffU);          // [kB][kMaxCols] u = M1 g
  C* RW = reinterpret_cast<C*>(smem + kOffRB);        // [2][8][kB] each warp's pivot candidate row
  C* invv = reinterpret_cast<C*>(smem + kOffInv);     // [2][kB]
  C* M1 = reinterpret_cast<C*>(smem + kOffM1);        // [kB][kB], transposed: M1[s][t] at s kB + t
  int* used = reinterpret_cast<int*>(smem + kOffInts);
  int* piv = used + kMaxRows;
  int* pslot = piv + kMaxRows;
  int* pinv = pslot + kMaxRows;
  int* pb = reinterpret_cast<int*>(smem + kOffPb);   // [2][kB]
  unsigned* wkey = reinterpret_cast<unsigned*>(smem + kOffKey);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kOffBar);   // cluster sync
  uint64_t* exitbar = bar + 1;                                    // cluster exit rendezvous
  uint64_t* mmabar = bar + 2;                                     // tensor-core completion
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + kOffMisc);
  unsigned* tslot = reinterpret_cast<unsigned*>(smem + kOffMisc + 4);

  const double2* px = prof + cl.prof_off;  // lo_x, hi_x, dg_x, lo_y, hi_y, dg_y
  const double2* py = px + 3 * nx;
  C* Fac = fac + cl.fac_off;
  C* Prev0 = prev ? prev + (long long)(2 * cidx) * prev_stride : nullptr;
  C* Prev1 = prev ? Prev0 + prev_stride : nullptr;
  C* Prev = half ? Prev1 : Prev0;
  const C z = czero<C>();

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tslot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    *abort_flag = 0;
    mbar_init(bar, (unsigned)G);
    mbar_init(exitbar, (unsigned)G);
    mbar_init(mmabar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = tid; i < kMaxRows; i += kT) pslot[i] = -1;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tbase = *tslot;
  // TMEM address of column `col` (32-bit units) of my row
  const unsigned trow = tbase + ((unsigned)(32 * (warp & 3)) << 16) + (unsigned)(256 * (warp >> 2));
  if (G > 1) asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");

  unsigned phase = 0, mma_phase = 0;
  bool mma_pending = false;
  // bounded wait on the tensor-core completion barrier; abortable = false: the
  // limit alone ends it (before TMEM is released)
  auto wait_mma = [&](bool abortable) -> bool {
    if (!mma_pending) return true;
    bool ok = mbar_try_wait(mmabar, mma_phase & 1u);
    if (!ok) {
      const long long t0 = clock64();
      while (!(ok = mbar_try_wait(mmabar, mma_phase & 1u))) {
        if (abortable && *abort_flag) break;
        if (clock64() - t0 > wait_cycles) {
          *abort_flag = 1;
          atomicOr(status, 2);
          break;
        }
      }
    }
    if (ok) {
      mma_pending = false;
      ++mma_phase;
    }
    return ok;
  };
  auto csync = [&]() -> bool {
    tc_fence_before();
    __syncthreads();
    if (G > 1) {
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
    }
    __syncthreads();
    tc_fence_after();
    return *abort_flag == 0;
  };
  // Before leaving (normally or after a wait gave up): no tensor-core work in
  // flight, every CTA of the cluster done with this CTA's shared memory, then
  // TMEM released.
  auto leave = [&]() {
    wait_mma(false);
    tc_fence_before();
    __syncthreads();
    if (G > 1) {
      if (tid < G) mbar_arrive_remote(exitbar, (unsigned)tid);
      if (!mbar_try_wait_cluster(exitbar, 0u)) {
        const long long t0 = clock64();
        while (!mbar_try_wait_cluster(exitbar, 0u)) {
          if (clock64() - t0 > wait_cycles) {
            atomicOr(status, 2);
            break;
          }
        }
      }
    }
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(kTmemCols)
                                : "memory");
  };

  // instruction descriptor: D FP32, A and B bf16, A negated (D -= A B), both
  // K-major, N = NP, M = 128
  const unsigned idesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 13) | ((unsigned)(NP >> 3) << 17) |
                         ((unsigned)(128 >> 4) << 24);

  for (int step = 0; step < nsteps; ++step) {
    const int k = middle ? mid : (half == 0 ? step : nx - 1 - step);
    // ---- Schur complement of line k, my columns, into TMEM (row r per thread) ----
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
    if (warp_rows) {
      C dr = z, lo = z, hi = z;
      if (live) {
        const double* mrow = mgrid + (long long)(cl.lox + k) * n_dof + cl.loy;
        dr = cadd(dgx, to_c(py[2 * n + r], z));
        dr.x -= (float)(omega2 * mrow[r]);
        lo = to_c(py[r], z);        // coupling to j = r - 1 (south)
        hi = to_c(py[n + r], z);    // coupling to j = r + 1 (north)
      }
      for (int cb = 0; cb < nc; cb += 16) {
        float v[32];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int cc = cb + q, j = c0 + cc;
          C e = z;
          if (live && cc < nc) {
            if (Fa) e = cneg(cmul(coupa, Fa[(size_t)j * ldn + r]));
            if (Fb) cfms(e, coupb, Fb[(size_t)j * ldn + r]);
            if (j == r) e = cadd(e, dr);
            else if (j == r - 1) e = cadd(e, lo);
            else if (j == r + 1) e = cadd(e, hi);
          }
          v[2 * q] = e.x;
          v[2 * q + 1] = e.y;
        }
        tm_st32(trow + 2 * cb, v);
      }
      tm_wait_st();
    }
    if (r < kMaxRows) used[r] = 0;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    int blk = 0;
    for (int k0 = 0; k0 < n; ++blk) {
      const int o = col_owner(k0, n, G);
      const int k1 = min(k0 + kB, (o + 1) * n / G);
      const int bt = k1 - k0, buf = blk & 1;
      C* Fb_ = F + (size_t)buf * kB * kMaxRows;
      int* pbb = pb + buf * kB;
      C* ivb = invv + buf * kB;

      // ---- panel: the owner's classic Gauss-Jordan steps on [k0, k1) ----
      if ((int)g == o) {
        C row[kB];
        float pv[32];
        if (warp_rows) tm_ld32(trow + 2 * (k0 - c0), pv);
#pragma unroll
        for (int q = 0; q < kB; ++q) row[q] = (warp_rows && live && q < bt) ? make_float2(pv[2 * q], pv[2 * q + 1]) : z;
        bool mine_used = live ? (used[r] != 0) : true;
        // One barrier per step: the candidate row of every warp (its largest
        // unpivoted magnitude, found with one warp reduction) publishes its
        // panel values before the barrier, and after it every thread reads
        // the pivot row from its warp's slot and applies the step itself.
#pragma unroll
        for (int t = 0; t < kB; ++t) {
          if (t >= bt) break;
          const int par = t & 1;
          const C v = row[t];
          if (live) Fb_[(size_t)t * kMaxRows + r] = v;
          // pivot key: |v|^2 as float bits (monotone for non-negative values) with
          // the low byte replaced by 255 - row: the largest magnitude, ties (to
          // 2^-15) to the lowest row; pivoted rows have key 0
          unsigned key = 0u;
          if (live && !mine_used) key = (__float_as_uint(abs2(v)) & 0xffffff00u) | (unsigned)(255 - r);
          const unsigned wmax = __reduce_max_sync(0xffffffffu, key);
          C* rw = RW + (size_t)par * 8 * kB;
          if (key != 0u && key == wmax) {
            C* dst = rw + warp * kB;
#pragma unroll
            for (int q = 0; q < kB; ++q)
              if (q < bt) dst[q] = row[q];
          }
          unsigned* wk = wkey + par * 8;
          if (lane == 0) wk[warp] = wmax;
          named_sync(1, kT);
          unsigned best = wk[0];
#pragma unroll
          for (int w = 1; w < kT / 32; ++w) best = max(best, wk[w]);
          // best < 256: no unpivoted row of positive magnitude (singular); the
          // step still runs (on row 0, whatever its slot holds) so that the
          // kernel ends normally, and the status marks the factor invalid
          if (best < 256u && r == 0) atomicOr(status, 1);
          const int p = best ? 255 - (int)(best & 0xffu) : 0;
          const C* prow = rw + (p >> 5) * kB;
          const C inv = crcp(prow[t]);
          if (r == p) {
            if (!isfinite(abs2(v))) atomicOr(status, 1);
            mine_used = true;
#pragma unroll
            for (int q = 0; q < kB; ++q)
              if (q < bt) row[q] = (q == t) ? inv : cmul(row[q], inv);
            used[r] = 1;
            piv[k0 + t] = r;
            pbb[t] = r;
            ivb[t] = inv;
          } else if (live) {
            const C vi = cmul(v, inv);
#pragma unroll
            for (int q = 0; q < kB; ++q)
              if (q < bt) {
                if (q == t) row[q] = cneg(vi);
                else cfms(row[q], vi, prow[q]);
              }
          }
        }
        if (warp_rows) {
#pragma unroll
          for (int q = 0; q < kB; ++q) {
            pv[2 * q] = row[q].x;
            pv[2 * q + 1] = row[q].y;
          }
          // columns past the panel in this 32-column window keep their values
          if (bt < kB) {
            float keep[32];
            tm_ld32(trow + 2 * (k0 - c0), keep);
#pragma unroll
            for (int q = 0; q < kB; ++q)
              if (q >= bt) { pv[2 * q] = keep[2 * q]; pv[2 * q + 1] = keep[2 * q + 1]; }
          }
          tm_st32(trow + 2 * (k0 - c0), pv);
          tm_wait_st();
        }
      }
      if (!csync()) { leave(); return; }
      if ((int)g != o) {
        // the panel owner's f_t, pivots and reciprocals, read from its shared
        // memory: whole [bt][kMaxRows] planes as 16-byte loads, all of a
        // thread's loads in flight before its stores
        constexpr int kPer = (kB * kMaxRows / 2 + kT - 1) / kT;
        const int nv4 = bt * kMaxRows / 2;
        float4 buf4[kPer];
        const float4* src4 = reinterpret_cast<const float4*>(Fb_);
        float4* dst4 = reinterpret_cast<float4*>(Fb_);
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
          const int e = tid + i * kT;
          if (e < nv4) buf4[i] = ld_remote4(src4 + e, (unsigned)o);
        }
#pragma unroll
        for (int i = 0; i < kPer; ++i) {
          const int e = tid + i * kT;
          if (e < nv4) dst4[e] = buf4[i];
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
      __syncthreads();
      // M1 = (D + L)^-1 (D = diag f_t[p_t], L[t][s] = f_s[p_t], s < t), by the
      // last warp (no matrix row: free while the others write the A operand),
      // lane j solving for column j
      if (warp == kT / 32 - 1 && lane < bt) {
        C mm[kB];
#pragma unroll
        for (int t = 0; t < kB; ++t) {
          if (t < bt) {
            C a = (t == lane) ? make_float2(1.f, 0.f) : z;
#pragma unroll
            for (int s2 = 0; s2 < kB; ++s2)
              if (s2 < t) cfms(a, Fb_[(size_t)s2 * kMaxRows + pbb[t]], mm[s2]);
            mm[t] = cmul(a, ivb[t]);
            M1[lane * kB + t] = mm[t];   // stored transposed: [s][t]
          }
        }
      }
      // A operand: f_t[r] as (Re, Im) along k, three bf16 terms, one row per
      // thread; zero rows for the block's pivot rows (finished on the CUDA
      // cores after the product) and past the matrix
      if (r < 128 * ntiles) {
        const bool is_piv = live && pslot[r] >= 0;
#pragma unroll
        for (int t = 0; t < kB; ++t) {
          C f = z;
          if (live && t < bt && !is_piv) f = Fb_[(size_t)t * kMaxRows + r];
          put3(Aop, kATerm, kmaj(r, 2 * t), f.x, f.y);
        }
      }
      // g: the pivot rows of my columns, from the warps that hold them
      {
        const bool has = __any_sync(0xffffffffu, live && pslot[r] >= 0);
        if (warp_rows && has) {
          const int sl = live ? pslot[r] : -1;
          for (int cb = 0; cb < nc; cb += 16) {
            float v[32];
            tm_ld32(trow + 2 * cb, v);
            if (sl >= 0) {
#pragma unroll
              for (int q = 0; q < 16; ++q)
                if (cb + q < nc) GU[(size_t)sl * kMaxCols + cb + q] = make_float2(v[2 * q], v[2 * q + 1]);
            }
          }
        }
      }
      __syncthreads();
      // u = M1 g per (pivot, column), into U and as the B operand: rows 2c:
      // (Re u, -Im u), 2c + 1: (Im u, Re u) along k = (2t, 2t + 1).  The panel's
      // own columns, pivots past the block and the padding columns get u = 0.
      // A warp covers two units of 4 columns x 4 pivots (lane: column mod 4 =
      // (lane >> 2) mod 4, pivot mod 4 = lane mod 4): two lanes per bank.
      const int pcol0 = (int)g == o ? k0 - c0 : nc, pcol1 = (int)g == o ? k1 - c0 : nc;
      {
        const int nh = NP / 2;   // columns with padding, a multiple of 8
        for (int u2 = warp; u2 < nh / 2; u2 += kT / 32) {
          const int u = u2 * 2 + (lane >> 4);   // unit: (column quarter-block, pivot quarter)
          const int cc = (u >> 2) * 4 + ((lane >> 2) & 3), t = (u & 3) * 4 + (lane & 3);
          C a = z;
          if (t < bt && cc < nc && (cc < pcol0 || cc >= pcol1))
            for (int s2 = 0; s2 <= t; ++s2) cfma(a, M1[s2 * kB + t], GU[(size_t)s2 * kMaxCols + cc]);
          if (cc < nc) U[(size_t)t * kMaxCols + cc] = a;
          put3(Bop, kBTerm, kmaj(2 * cc, 2 * t), a.x, -a.y);
          put3(Bop, kBTerm, kmaj(2 * cc + 1, 2 * t), a.y, a.x);
        }
      }
      // operand writes (generic proxy) visible to the tensor core (async proxy)
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      // ---- the block's update on the tensor cores: W -= F U, bf16 x 3 ----
      // (A term i, B term j) for i + j <= 2: hi hi, hi mid, mid hi, hi lo,
      // mid mid, lo hi; two k-steps of 16 per 128-row tile.  Issued by the last
      // warp (no matrix row), while the others form the pivot rows' values.
      const int issuer = kT - 32;
      if (tid == issuer) {
        const unsigned a0 = saddr(Aop), b0 = saddr(Bop);
        for (int tile = 0; tile < ntiles; ++tile) {
          const unsigned d = tbase + (unsigned)(256 * tile);
          const unsigned ao = (unsigned)tile * 8192u;
#pragma unroll
          for (int s = 0; s < 2; ++s) {
            const unsigned ko = (unsigned)s * 256u;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
              for (int j = 0; j + i < 3; ++j)
                mma_bf16(d, sdesc(a0 + (unsigned)(i * kATerm) + ao + ko), sdesc(b0 + (unsigned)(j * kBTerm) + ko),
                         idesc);
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(mmabar))
                     : "memory");
      }
      mma_pending = true;
      // while the tensor cores run: the block's pivot rows, which the product
      // leaves as they were, c[p_t] = u_t - sum_{s>t} f_s[p_t] u_s on my columns
      // outside the panel, into GU
      if (tid < issuer) {
        int t = tid / nc, cc = tid - (tid / nc) * nc;
        const int st_t = issuer / nc, st_c = issuer - (issuer / nc) * nc;
        for (int e = tid; e < bt * nc; e += issuer) {
          C a = U[(size_t)t * kMaxCols + cc];
          const int pt = pbb[t];
          for (int s2 = t + 1; s2 < bt; ++s2)
            cfms(a, Fb_[(size_t)s2 * kMaxRows + pt], U[(size_t)s2 * kMaxCols + cc]);
          GU[(size_t)t * kMaxCols + cc] = a;
          t += st_t;
          cc += st_c;
          if (cc >= nc) { cc -= nc; ++t; }
        }
      }
      __syncthreads();
      if (!wait_mma(true)) { leave(); return; }
      tc_fence_after();
      // the pivot rows' final values into TMEM (the panel's columns keep the
      // panel's values)
      {
        const int sl = live ? pslot[r] : -1;
        const bool has = __any_sync(0xffffffffu, sl >= 0);
        if (warp_rows && has) {
          for (int cb = 0; cb < nc; cb += 16) {
            float v[32];
            tm_ld32(trow + 2 * cb, v);
            if (sl >= 0) {
#pragma unroll
              for (int q = 0; q < 16; ++q) {
                const int cc = cb + q;
                if (cc < nc && (cc < pcol0 || cc >= pcol1)) {
                  const C a = GU[(size_t)sl * kMaxCols + cc];
                  v[2 * q] = a.x;
                  v[2 * q + 1] = a.y;
                }
              }
            }
            tm_st32(trow + 2 * cb, v);
          }
          tm_wait_st();
        }
      }
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      if (tid < bt) pslot[pbb[tid]] = -1;
      __syncthreads();
      k0 = k1;
    }

    // ---- unscramble my columns into the factor pool: output (i, j = piv[c])
    // holds W[piv[i]][c], through a column-major staging tile in the operand
    // area (16 columns at a time) ----
    for (int i = tid; i < n; i += kT) pinv[piv[i]] = i;
    __syncthreads();
    C* stg = reinterpret_cast<C*>(smem + kOffA);     // [16][ldn]
    C* Fk = Fac + (size_t)k * n * ldn;
    for (int cb = 0; cb < nc; cb += 16) {
      if (warp_rows) {
        float v[32];
        tm_ld32(trow + 2 * cb, v);
        if (live) {
          const int i = pinv[r];
#pragma unroll
          for (int q = 0; q < 16; ++q)
            if (cb + q < nc) stg[(size_t)q * ldn + i] = make_float2(v[2 * q], v[2 * q + 1]);
        }
      }
      __syncthreads();
      const int ncol = min(16, nc - cb);
      for (int e = tid; e < ncol * ldn; e += kT) {
        const int q = e / ldn, i = e - q * ldn;
        const int j = piv[c0 + cb + q];
        const C val = i < n ? stg[(size_t)q * ldn + i] : z;
        if (split) {
          if (!middle) Prev[(size_t)j * ldn + i] = val;
          reinterpret_cast<uint2*>(Fk)[(size_t)j * ldn + i] = split_entry(val);
        } else {
          Fk[(size_t)j * ldn + i] = val;
        }
      }
      __syncthreads();
    }
    // the next line's Schur complement reads every CTA's columns of this inverse
    if (!csync()) { leave(); return; }
  }
  leave();
}

int tc_cluster(int n) { return n <= kMaxCols ? 1 : (n <= kMaxRows ? 2 : 0); }

}  // namespace

bool factorize_tc_supported(int max_ny) { return max_ny >= 1 && max_ny <= kMaxRows; }

cudaError_t launch_factorize_tc(const DevCell* cells, int ncell, const double2* prof, const double* mgrid, int n_dof,
                                double omega2, void* fac, void* prev, int max_ny, int* status, cudaStream_t st,
                                bool split, long long wait_cycles) {
  if (ncell <= 0) return cudaSuccess;
  const int G = tc_cluster(max_ny);
  if (G == 0) return cudaErrorInvalidValue;
  if (split && prev == nullptr) return cudaErrorInvalidValue;
  int dev = 0, maxopt = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (maxopt < kSmem) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(k_factorize_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, maxopt);
  if (e != cudaSuccess) return e;
  const long long prev_stride = (long long)max_ny * (max_ny + 8);
  cudaLaunchConfig_t cfg{};
  cudaLaunchAttribute attr[1];
  cfg.blockDim = dim3(kT);
  cfg.dynamicSmemBytes = kSmem;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)G;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  for (int middle = 0; middle < 2; ++middle) {
    cfg.gridDim = dim3((unsigned)(ncell * G * (middle ? 1 : 2)));
    e = cudaLaunchKernelEx(&cfg, k_factorize_tc, cells, prof, mgrid, n_dof, omega2, reinterpret_cast<float2*>(fac),
                           reinterpret_cast<float2*>(split ? prev : nullptr), prev_stride, split ? 1 : 0, middle, G,
                           status, wait_cycles);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace lsw
