// Sweep-front kernel: every cell solve of one front of the L-sweep
// preconditioner in one launch.
//
// A cell matrix is block tridiagonal over its x-lines (DOF order i*ny + j,
// AssemblerHelmholtz2DFD.cpp:166-177); the couplings between lines are scalar
// multiples of the identity (the PML profile is separable).  The factor
// (kernels_factor.cu) is a twisted block LU about the middle line
// m = (nx - 1) / 2, so a solve is two independent chains that meet there:
//   top     y_k = S_k^{-1} (b_k - w_k y_{k-1})           k = 0 .. m-1
//   bottom  z_k = T_k^{-1} (b_k - e_k z_{k+1})           k = nx-1 .. m+1
//   middle  x_m = Z_m^{-1} (b_m - w_m y_{m-1} - e_m z_{m+1})
//   top     x_k = y_k - e_k S_k^{-1} x_{k+1}             k = m-1 .. 0
//   bottom  x_k = z_k - w_k T_k^{-1} x_{k-1}             k = m+1 .. nx-1
// (w_k, e_k = couplings of line k to k-1 / k+1): about nx + 1 dependent
// matvecs per half instead of 2 nx - 1 for a one-ended block LU.  One cell
// solve ("item") carries R right-hand sides ("slots") that share every factor
// block read.
//
// Work split.  An item runs on a thread-block cluster of 2 CL CTAs: CTAs
// 0..CL-1 run the top chain and CL..2CL-1 the bottom chain.  Within a half,
// CTA c owns the column range J_c of every block (contiguous in the
// column-major factor) and the same range of every line vector.  Per line it
// forms the partial products of all rows with its columns and pushes the
// partial sums of each row to the CTA of its half that owns that row
// (st.async into the owner's shared memory, completing the transaction count
// of the owner's per-line mbarrier; no fences or remote arrives on the
// per-line path), so every SM streams 1/CL of its half's blocks and reads only
// local shared memory when it finishes a line.  Before the middle line, CTA c
// of each half sends its y_{m-1} / z_{m+1} columns to CTA c of the other half
// (same column range), and both halves run the middle line on identical
// inputs, so both hold the same x_m.
//
// Roles inside a CTA: warp 0 is the producer that streams the CTA's column
// chunks (CW columns, contiguous, up to ~64 KB: one bulk copy costs ~700
// cycles whatever its size and one issuing thread keeps one copy in flight,
// so copies are large and two lanes issue them alternately) in the order the
// two substitutions consume them, through an NS-stage shared-memory ring
// (cp.async.bulk + mbarrier completion); warps 1-2 prefetch the next line's
// right-hand side (forward) or stored y_k (backward) into shared memory;
// warp 3 copies y_k (forward) and x_k (backward) to a per-item scratch; the
// remaining warps are consumers: a lane owns a row pair of a 64-row group and
// a warp one of KSW interleaved column slices, accumulating in registers with
// no cross-lane reduction (complex FP32/FP64 FMAs).  With split factors (bf16
// hi + lo words) a consumer warp owns a 16-row m-tile instead and runs the
// partial products on the tensor cores (mma.sync m16n8k16, three products per
// k-step, FP32 accumulation) against the line input staged as bf16 hi/lo
// words.  Line vectors and partial sums are stored [column][slot] so that
// slot offsets are compile-time constants.  The
// outputs (owned DOFs, trace lines, cell vectors) are written once per item
// from the scratch by every non-producer thread after the backward pass, each
// half writing its own lines.
// Every wait is bounded: after ~2 s of clock cycles a wait raises the CTA's
// abort flag and *a.err, and all later waits return at once so every thread
// still reaches every barrier.
//
// The right-hand sides are never materialised: a slot builds b_k on the fly
// from the global input (stage 1, the window of DDCheckerboard::getSeparatedRHS,
// DDCheckerboard.cpp:3564-3674, restricted to the owned set) or from its
// neighbours' trace lines (equivalent sources of
// SubdomainStructured::getEquivalentSources, SubdomainStructured.cpp:1304-1465,
// and the L-shaped traces of extractLTraces, 1468-1539).  After the backward
// pass the item's owned DOFs are accumulated into the output (reduce,
// DDCheckerboard.cpp:744-772) and its outgoing trace lines into the trace pool.
#include "common.cuh"
#include "internal.h"

#include <cuda_bf16.h>

#include <algorithm>

namespace lsw {

namespace {

constexpr int kMaxRG = 3;             // row groups of 64 rows (2 per lane): ny <= 192
constexpr int kMaxKSW = 4;            // column slices (consumer warps per row group)
constexpr int kAux = 4;               // producer, two helper warps, writer warp
constexpr int kNSMax = 8;             // ring stages
constexpr int kHdr = 256;             // barrier header bytes
constexpr int SK_NONE = 99;           // padding slot
constexpr unsigned kSuspendNs = 1000000;          // try_wait sleeps up to 1 ms (woken by the phase)


// ---------------------------------------------------------------------------
// PTX helpers
// ---------------------------------------------------------------------------
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
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}
// arrive on the barrier at the same offset in CTA `rank` of the cluster (release, cluster scope)
__device__ __forceinline__ void mbar_arrive_remote(uint64_t* b, unsigned rank) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(mapa(saddr(b), rank))
               : "memory");
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
// Bounded wait (see the file comment): gives up after `limit` clock cycles,
// or at once when the CTA's abort flag is up (abort_flag == nullptr: a wait
// that only the limit ends, for the drain before leaving).
template <bool CLUSTER>
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity, int* err, volatile int* abort_flag,
                                          long long limit) {
  auto tw = [&]() { return CLUSTER ? mbar_try_wait_cluster(b, parity) : mbar_try_wait(b, parity); };
  if (tw()) return true;
  const long long t0 = clock64();
  while (true) {
    if (abort_flag && *abort_flag) return false;
    if (tw()) return true;
    if (clock64() - t0 > limit) {
      if (abort_flag) *abort_flag = 1;
      atomicOr(err, 2);
      return false;
    }
  }
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   saddr(dst)),
               "l"(src), "r"(bytes), "r"(saddr(bar))
               : "memory");
}
__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
// store into CTA `rank`'s shared memory; the bytes complete the transaction
// count of that CTA's mbarrier at the same offset as `bar`
__device__ __forceinline__ void st_async(float2* p, unsigned rank, float2 v, uint64_t* bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];" ::"r"(
                   mapa(saddr(p), rank)),
               "f"(v.x), "f"(v.y), "r"(mapa(saddr(bar), rank))
               : "memory");
}
__device__ __forceinline__ void st_async2(float2* p, unsigned rank, float2 v0, float2 v1, uint64_t* bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(
                   mapa(saddr(p), rank)),
               "f"(v0.x), "f"(v0.y), "f"(v1.x), "f"(v1.y), "r"(mapa(saddr(bar), rank))
               : "memory");
}
__device__ __forceinline__ void st_async(double2* p, unsigned rank, double2 v, uint64_t* bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f64 [%0], {%1, %2}, [%3];" ::"r"(
                   mapa(saddr(p), rank)),
               "d"(v.x), "d"(v.y), "r"(mapa(saddr(bar), rank))
               : "memory");
}
__device__ __forceinline__ void red_add(float2* p, float2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}
__device__ __forceinline__ void red_add(double2* p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

// bf16x2 words of the hi and lo terms of (a, b): low half a, high half b
__device__ __forceinline__ void split_pair(float a, float b, unsigned& hi, unsigned& lo) {
  const __nv_bfloat16 ah = __float2bfloat16_rn(a), bh = __float2bfloat16_rn(b);
  const __nv_bfloat16 al = __float2bfloat16_rn(a - __bfloat162float(ah));
  const __nv_bfloat16 bl = __float2bfloat16_rn(b - __bfloat162float(bh));
  hi = (unsigned)__bfloat16_as_ushort(ah) | ((unsigned)__bfloat16_as_ushort(bh) << 16);
  lo = (unsigned)__bfloat16_as_ushort(al) | ((unsigned)__bfloat16_as_ushort(bl) << 16);
}
// D += A B, m16n8k16, bf16 operands, FP32 accumulation
__device__ __forceinline__ void mma_bf16(float (&d)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1) {
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ---- tensor-core (tcgen05) line products of complex64 items ----
// A line's partial products D[row][n] = sum_k A[row][k] B[n][k] as real
// GEMMs: A = the factor block with k = 2 column + (0: Re, 1: Im), B = the line
// input with n = 2 slot + (0: Re, 1: Im) of the product, [x_re, -x_im] and
// [x_im, x_re] along k; both split into three bf16 terms (hi + mid + lo, each
// the rounded remainder of the previous ones) and multiplied as the six
// products of combined order <= 2, FP32 accumulation in tensor memory.
constexpr int kTcStages = 2;   // A operand stages, one k-block (8 columns, k = 16) each
constexpr int kTcTile = 4096;  // one 128-row x 16-k bf16 tile of A, bytes

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes of this thread visible to the tensor core
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// canonical K-major layout without swizzle: 8-row x 16-byte core matrices (8 k
// each), k-adjacent core matrices 128 B apart.  A tiles [128 x 16]: 8-row
// groups 256 B apart.  B [N x Kp] as k-tiles of 32 (N x 64 bytes each): 8-row
// groups 512 B apart within a tile.
__device__ __forceinline__ int a_off(int row, int k) {
  return (row >> 3) * 256 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2;
}
__device__ __forceinline__ int b_off(int n, int k, int N) {
  return (k >> 5) * (N * 64) + (n >> 3) * 512 + ((k & 31) >> 3) * 128 + (n & 7) * 16 + (k & 7) * 2;
}
// shared-memory matrix descriptor (start, leading byte offset 128, stride
// byte offset `sbo`, in 16-byte units; descriptor version 1, no swizzle)
__device__ __forceinline__ uint64_t tc_desc(unsigned addr, unsigned sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}
// (a, b) as three bf16x2 terms `term` bytes apart at byte offset `off`
__device__ __forceinline__ void put3(unsigned char* base, int term, int off, float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float ra = a - __low2float(h), rb = b - __high2float(h);
  const __nv_bfloat162 m = __floats2bfloat162_rn(ra, rb);
  const __nv_bfloat162 l = __floats2bfloat162_rn(ra - __low2float(m), rb - __high2float(m));
  *reinterpret_cast<__nv_bfloat162*>(base + off) = h;
  *reinterpret_cast<__nv_bfloat162*>(base + term + off) = m;
  *reinterpret_cast<__nv_bfloat162*>(base + 2 * term + off) = l;
}
// D (TMEM, FP32) = A B + (acc ? D : 0), A and B bf16 from shared memory
__device__ __forceinline__ void tc_mma(unsigned d, uint64_t a, uint64_t b, unsigned idesc, unsigned acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
          d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
// N consecutive 32-bit TMEM columns of this thread's lane (N = 16 or 32)
template <int N>
__device__ __forceinline__ void tm_ld(unsigned taddr, float (&v)[N]) {
  unsigned r[N];
  if constexpr (N == 16) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
  } else {
    static_assert(N == 32, "16 or 32 columns");
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
        "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
  }
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < N; ++j) v[j] = __uint_as_float(r[j]);
}

// CTA c of a cluster of CL owns rows/columns [c*ny/CL, (c+1)*ny/CL)
__device__ __forceinline__ int owner_of(int row, int ny, int CL) { return ((row + 1) * CL - 1) / ny; }

__device__ __forceinline__ bool is_line(int gnode, int m, int N) {
  // interface lines k_b(J), k_b(J)+1 for J = 0..N-2 (the trace1/traceN rows
  // zeroed by getSeparatedRHS)
  if (gnode < m || gnode > (m + 1) * (N - 1)) return false;
  const int r = gnode % (m + 1);
  return r == m || r == 0;
}

struct SlotCoef {
  double2 c_oi_x, c_io_x, c_oi_y, c_io_y;
};

template <typename T>
__device__ __forceinline__ cx_t<T> rhs_elem(const FrontArgs& a, const DevCell& cl, const DevSlot& s,
                                            const SlotCoef& cf, const cx_t<T>* tr, int k, int j) {
  using C = cx_t<T>;
  C z = czero<C>();
  switch (s.kind) {
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

// two consecutive rows of one factor column, from shared memory
template <typename T> struct Pair;
template <> struct Pair<float> {
  float2 a, b;
  __device__ __forceinline__ void load(const float2* p) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    a = make_float2(v.x, v.y); b = make_float2(v.z, v.w);
  }
};
template <> struct Pair<double> {
  double2 a, b;
  __device__ __forceinline__ void load(const double2* p) { a = p[0]; b = p[1]; }
};

template <typename T, int R, bool SPLIT, bool TCM = false>
__device__ __forceinline__ void front_body(const FrontArgs& a, const DevItem& it, const DevCell& cl, unsigned char* smem) {
  using C = cx_t<T>;
  // complex64 line products on the tensor cores (tcgen05, TMEM accumulators)
  constexpr bool TC = TCM && !SPLIT && sizeof(T) == 4;
  static_assert(!TC || R == 8 || R == 16, "tensor-core items carry 8 or 16 slots");
  constexpr int TN = 2 * R;                                  // GEMM n: (slot, Re / Im)
  constexpr int kTcCols = TN * 2 < 32 ? 32 : TN * 2;         // TMEM columns: two 128-row tiles
  const int CW = a.chunk;              // columns per chunk, multiple of 8
  const int KSW = a.ksw;               // column slices: consumer warps per row group
  static_assert((2 * kNSMax + 4) * 8 + 4 <= kHdr, "barrier header");
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nx = cl.nx, ny = cl.ny, ldn = cl.ldn;
  const int CL = a.cluster;              // CTAs per half
  const int CLT = 2 * CL;                // CTAs per item
  const int NS = a.stages;
  const unsigned crk = cluster_rank();
  if (cluster_size() != (unsigned)CLT || crk != blockIdx.x % (unsigned)CLT) {
    // the launch did not form the clusters this kernel was configured for
    // (uniform over the CTA: every thread leaves before any barrier)
    if (threadIdx.x == 0) atomicOr(a.err, 4);
    return;
  }
  const int half = (int)crk / CL;        // 0: top chain, 1: bottom chain
  const unsigned crank = crk % (unsigned)CL;          // rank within the half
  const unsigned rbase = (unsigned)(half * CL);       // cluster rank of the half's CTA 0
  const unsigned partner = (unsigned)((1 - half) * CL) + crank;
  const int mid = (nx - 1) / 2;
  const int nf = half == 0 ? mid : nx - 1 - mid;      // forward lines of my half (>= 2: nx >= 5)
  // line li of my half: forward li < nf, the middle line li == nf, backward after
  auto line_k = [&](int li) {
    const int i = li < nf ? li : 2 * nf - li;
    if (li == nf) return mid;
    return half == 0 ? i : nx - 1 - i;
  };
  // scratch row of line k; the bottom half keeps its copy of b_m in row nx
  auto srow = [&](int k) { return (half == 1 && k == mid) ? nx : k; };
  const int klo = half == 0 ? 0 : mid + 1, khi = half == 0 ? mid : nx - 1;   // lines whose outputs I write
  const int jb = (int)crank * ny / CL, je = ((int)crank + 1) * ny / CL;
  const int nJ = je - jb;               // my columns / rows of every line
  const int RG = (ny + 63) >> 6;        // row groups of 64 rows
  // consumer warps: KSW column slices per row group, or (split) one per 16-row m-tile
  // FP32/FP64 FMA matvec: KSW column slices per row group; with more than 8
  // slots (complex64) two slot groups of R / 2 slots each, on their own warps,
  // so that a warp keeps at most 8 slots of two rows in registers
  constexpr int SG = (!SPLIT && sizeof(T) == 4 && R > 8) ? 2 : 1;
  constexpr int RS = R / SG;
  const int NCW = TC ? kMaxRG * kMaxKSW : SPLIT ? (ny + 15) >> 4 : KSW * RG * SG;
  constexpr int NT = (2 * R + 7) / 8;   // split: n-tiles of 8 (Re, Im interleaved per slot)
  constexpr int NT8 = NT * 8;
  const int NCT = NCW * 32;
  const int NSYNC = NCT + 96;           // consumers + 2 helper warps + writer warp
  const int nch = (nJ + CW - 1) / CW;   // chunks per line
  const int nslot = it.slot_count;
  const int nline = 2 * nf + 1;         // forward, middle, backward

  // ---- shared layout ----
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + kNSMax;
  uint64_t* pready = empty + kNSMax;    // [2]: every CTA's partial sums of my rows have landed (CL > 1)
  uint64_t* exitb = pready + 2;         // cluster-wide "done with remote shared memory"
  uint64_t* xch = exitb + 1;            // the other half's last forward vector has landed in P
  volatile int* abort_flag = reinterpret_cast<volatile int*>(xch + 1);
  // tensor-core items: A stage completions (tcgen05.commit), the TMEM address
  static_assert((2 * kNSMax + 4) * 8 + 8 + 2 * 8 + 4 <= kHdr, "barrier header");
  uint64_t* mmab = xch + 2;
  unsigned* tslot = reinterpret_cast<unsigned*>(mmab + kTcStages);
  auto al16 = [](unsigned char* q) {
    return reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(q) + 15) & ~uintptr_t(15));
  };
  unsigned char* p = smem + kHdr;
  C* ring = reinterpret_cast<C*>(p);
  const int slot_elems = CW * ldn;
  p += (size_t)NS * slot_elems * sizeof(C);
  // the layout must be identical in every CTA of the cluster (peers address
  // each other's partial sums by offset), so size per-rank buffers by the
  // largest column range of the cluster
  const int nJcap = (ny + CL - 1) / CL;
  // line vectors are [column][slot], the slot index fastest
  C* V = reinterpret_cast<C*>(p);       // [nJ][R]  input vector of the current line (my columns)
  p = al16(p + (size_t)R * nJcap * sizeof(C));
  C* H = reinterpret_cast<C*>(p);       // [nJ][R]  helper: next right-hand side or stored y_k
  p = al16(p + (size_t)R * nJcap * sizeof(C));
  C* Y = reinterpret_cast<C*>(p);       // [nJ][R]  y_k staged for the writer (forward)
  p = al16(p + (size_t)R * nJcap * sizeof(C));
  C* P = reinterpret_cast<C*>(p);       // [nJ][R]  the other half's y_{m-1} / z_{m+1}, my columns
  p = al16(p + (size_t)R * nJcap * sizeof(C));
  unsigned char* colf = p;              // [nJ] bit 0: grid line; bits 1, 2: owned in y (non-shifted, shifted)
  p = al16(p + nJcap);
  unsigned char* linef = p;             // [nx] bit 0: grid line; bits 1, 2: owned in x (non-shifted, shifted)
  p = al16(p + nx);
  C* wsh = reinterpret_cast<C*>(p);      // [nx] coupling of line k to k-1
  p = al16(p + sizeof(C) * nx);
  C* esh = reinterpret_cast<C*>(p);      // [nx] coupling of line k to k+1
  p = al16(p + sizeof(C) * nx);
  C* Q = reinterpret_cast<C*>(p);       // [2][CL][nJcap][R] partial sums of my rows from every CTA
  const size_t qplane = (size_t)nJcap * R;
  const size_t qbuf = (size_t)CL * qplane;
  p = al16(p + 2 * qbuf * sizeof(C));
  C* LS = reinterpret_cast<C*>(p);      // [KSW][R][64 RG] the column slices' partial sums, before their sum
  if (!SPLIT && !TC) p = al16(p + (size_t)KSW * 64 * RG * R * sizeof(C));
  // tensor-core items: the A stages ([stage][term][tile] 128 x 16 bf16) and the
  // line input as B ([term] TN x Kp bf16, Kp = my columns x 2 rounded to 32)
  const int MT = (ldn + 127) >> 7;
  const int Kp = (2 * nJcap + 31) & ~31;
  const int a_term = MT * kTcTile, b_term = TN * Kp * 2;
  unsigned char* Ast = nullptr;
  unsigned char* Bop = nullptr;
  if constexpr (TC) {
    p = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(p) + 127) & ~uintptr_t(127));
    Ast = p;
    p += (size_t)kTcStages * 3 * a_term;
    Bop = p;
    p = al16(p + (size_t)3 * b_term);
  }
  // split: the next line's input as mma B words, hi and lo terms, [column][n]
  // with n = 2 slot + (0: real part, 1: imaginary part) of the product
  const int nJ8 = ((nJcap + 7) & ~7) + 8;
  unsigned* BwH = reinterpret_cast<unsigned*>(p);
  unsigned* BwL = BwH + (size_t)nJ8 * NT8;
  if (SPLIT) p = al16(p + 2 * (size_t)nJ8 * NT8 * sizeof(unsigned));
  int* rowinfo = reinterpret_cast<int*>(p);   // [ny] owner CTA << 16 | row offset in the owner's range
  p = al16(p + sizeof(int) * ny);
  DevSlot* sl = reinterpret_cast<DevSlot*>(p);
  p = al16(p + sizeof(DevSlot) * R);
  SlotCoef* cf = reinterpret_cast<SlotCoef*>(p);
  p = al16(p + sizeof(SlotCoef) * R);
  DevGroup* gr = reinterpret_cast<DevGroup*>(p);

  const C* tr = reinterpret_cast<const C*>(a.traces);
  C* trw = reinterpret_cast<C*>(a.traces);
  const double2* x_in = a.x_ref ? *a.x_ref : a.x_in;   // the VOLUME input
  const C* fac = reinterpret_cast<const C*>(a.fac) + cl.fac_off;
  C* scr = reinterpret_cast<C*>(a.scratch) + it.scratch_off;
  C* outs = reinterpret_cast<C*>(a.outs);
  const double2* px = a.prof + cl.prof_off;   // lo_x[nx], hi_x[nx], dg_x[nx], lo_y[ny], hi_y[ny], dg_y[ny]
  const double2* py = px + 3 * nx;

  // ---- set-up ----
  if (tid < R) {
    DevSlot s{};
    SlotCoef c{};
    if (tid < nslot) {
      s = a.slots[it.slot_begin + tid];
      if (s.kind == SK_DIR_X || s.kind == SK_CORNER) {
        c.c_oi_x = s.dx > 0 ? px[nx + s.xo] : px[s.xo];
        c.c_io_x = s.dx > 0 ? px[s.xi] : px[nx + s.xi];
      }
      if (s.kind == SK_DIR_Y || s.kind == SK_CORNER) {
        c.c_oi_y = s.dy > 0 ? py[ny + s.yo] : py[s.yo];
        c.c_io_y = s.dy > 0 ? py[s.yi] : py[ny + s.yi];
      }
    } else {
      s.kind = SK_NONE;
    }
    sl[tid] = s;
    cf[tid] = c;
  }
  if (tid < it.group_count) gr[tid] = a.groups[it.group_begin + tid];
  for (int row = tid; row < ny; row += blockDim.x) {
    const int o = owner_of(row, ny, CL);
    rowinfo[row] = (((int)rbase + o) << 16) | (row - o * ny / CL);
  }
  for (int k = tid; k < nx; k += blockDim.x)
    linef[k] = (unsigned char)((is_line(cl.lox + k - a.p + 1, a.m, a.N) ? 1 : 0) |
                               (k >= cl.ownx[0][0] && k <= cl.ownx[0][1] ? 2 : 0) |
                               (k >= cl.ownx[1][0] && k <= cl.ownx[1][1] ? 4 : 0));
  for (int jj = tid; jj < nJ; jj += blockDim.x) {
    const int j = jb + jj;
    colf[jj] = (unsigned char)((is_line(cl.loy + j - a.p + 1, a.m, a.N) ? 1 : 0) |
                               (j >= cl.owny[0][0] && j <= cl.owny[0][1] ? 2 : 0) |
                               (j >= cl.owny[1][0] && j <= cl.owny[1][1] ? 4 : 0));
  }
  for (int k = tid; k < nx; k += blockDim.x) {
    wsh[k] = to_c(px[k], czero<C>());
    esh[k] = to_c(px[nx + k], czero<C>());
  }
  if constexpr (SPLIT) {
    // the mma k-steps of a chunk's last columns and rows past ldn read ring
    // entries no copy wrote; zeros (with zero B words past my columns) keep
    // them finite and without effect
    for (size_t i = tid; i < (size_t)NS * slot_elems; i += blockDim.x) ring[i] = czero<C>();
    for (size_t i = tid; i < 2 * (size_t)nJ8 * NT8; i += blockDim.x) BwH[i] = 0u;
  }
  if constexpr (TC) {
    // A rows past ldn and B columns past my columns are never written: zeros
    // keep them without effect (the k-blocks of a chunk's last columns get
    // zeros from the conversion)
    uint4* z4 = reinterpret_cast<uint4*>(Ast);
    const size_t n16 = ((size_t)kTcStages * 3 * a_term + (size_t)3 * b_term) / 16;
    for (size_t i = tid; i < n16; i += blockDim.x) z4[i] = make_uint4(0u, 0u, 0u, 0u);
    fence_async_smem();
    if (warp == kAux) {   // the first consumer warp holds the accumulators' tensor memory
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tslot)),
                   "r"((unsigned)kTcCols)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
      tc_fence_before();
    }
  }
  if (tid == 0) {
    *abort_flag = 0;
    if constexpr (TC) {
      mbar_init(&mmab[0], 1);
      mbar_init(&mmab[1], 1);
    }
    for (int i = 0; i < NS; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], NCW); }
    // one local arrive (with the expected bytes) per line; the partial sums
    // land by st.async and complete the transaction count
    mbar_init(&pready[0], 1);
    mbar_init(&pready[1], 1);
    mbar_init(&exitb[0], CLT * NCW);
    // one phase: the partner CTA's forward vector (its columns = mine)
    mbar_init(xch, 1);
    mbar_expect_tx(xch, (unsigned)(nJ * R * sizeof(C)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if constexpr (TC) tc_fence_after();   // the TMEM address, after its allocation
  // every CTA's barriers are initialised before anyone arrives remotely
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");

  // Right-hand sides of every line of my half and of the middle line into
  // the item's scratch rows (row k then holds b_k until the forward pass
  // replaces it with y_k / z_k, and the backward pass with x_k), computed once
  // per item by every non-producer thread so that the per-line helpers only
  // copy a contiguous row.
  // A volume slot of shift (sx, sy) takes the owned DOFs whose x- and y-line
  // status matches the shift (the windows of getSeparatedRHS).
  auto prologue = [&](int et) {
    const int per_line = nJ * R;
    for (int e = et; e < (nf + 1) * per_line; e += NSYNC) {
      const int lr = e / per_line, rem = e - lr * per_line;
      const int k = half == 0 ? lr : (lr < nf ? mid + 1 + lr : mid);
      const int jj = rem / R, r = rem - jj * R, j = jb + jj;
      const DevSlot& sr = sl[r];
      C v = czero<C>();
      if (sr.kind == SK_VOLUME) {
        const int sx = sr.shift & 1, sy = (sr.shift >> 1) & 1;
        const int fx = linef[k], fy = colf[jj];
        if (((fx >> (1 + sx)) & 1) && ((fy >> (1 + sy)) & 1) && (fx & 1) == sx && (fy & 1) == sy)
          v = to_c(x_in[(long long)sr.rhs * a.x_stride + (long long)(cl.lox + k) * a.n_dof + cl.loy + j], czero<C>());
      } else if (sr.kind != SK_NONE) {
        v = rhs_elem<T>(a, cl, sr, cf[r], tr, k, j);
      }
      scr[((size_t)srow(k) * ny + jb) * R + rem] = v;
    }
  };

  // Outputs of the solved item, from the x_k rows in scratch (all of them are
  // there once the backward pass is done): owned DOFs summed per (right-hand
  // side, shift) group into the output (DDCheckerboard::reduce, 744-772), the
  // slots' outgoing trace lines into the trace pool, and whole cell vectors
  // for single-cell solves.  Spread over every thread but the producer's,
  // off the per-line critical path.
  auto epilogue = [&](int et) {
    auto xat = [&](int k, int r, int j) { return scr[((size_t)k * ny + j) * R + r]; };
    for (int g = 0; g < it.group_count; ++g) {
      const DevGroup G = gr[g];
      if (G.out_off < 0) continue;
      const int sx = G.shift & 1, sy = (G.shift >> 1) & 1;
      const int k0 = max(sx ? cl.ownx[1][0] : cl.ownx[0][0], klo);
      const int k1 = min(sx ? cl.ownx[1][1] : cl.ownx[0][1], khi);
      const int j0 = max(sy ? cl.owny[1][0] : cl.owny[0][0], jb);
      const int j1 = min(sy ? cl.owny[1][1] : cl.owny[0][1], je - 1);
      const int w = j1 - j0 + 1, hg = k1 - k0 + 1;
      if (w <= 0 || hg <= 0) continue;
      for (int e = et; e < w * hg; e += NSYNC) {
        const int k = k0 + e / w, j = j0 + e % w;
        C sum = czero<C>();
        for (int q = 0; q < G.slot_count; ++q) sum = cadd(sum, xat(k, G.slot_begin + q, j));
        red_add(outs + G.out_off + (long long)(cl.lox + k) * a.n_dof + cl.loy + j, sum);
      }
    }
    for (int r = 0; r < R; ++r) {
      const DevSlot& sr = sl[r];
      if (sr.kind == SK_NONE) continue;
      if (sr.kind == SK_CELLVEC) {
        for (int e = et; e < (khi - klo + 1) * nJ; e += NSYNC) {
          const int k = klo + e / nJ, j = jb + (e - (e / nJ) * nJ);
          a.x_out[(long long)sr.rhs * a.out_stride + (long long)k * ny + j] = to_c(xat(k, r, j), make_double2(0, 0));
        }
        continue;
      }
      // trace values; where lines cross, BL2TR overwrites trace0 entries
      // before they are added (DDCheckerboard.cpp:2520-2526)
      auto tval = [&](int k, int j) {
        if (sr.overwrite) {
          if (j == sr.yo) return tr[sr.in_ud0 + k];
          if (k == sr.xo) return tr[sr.in_lr0 + j];
        }
        return xat(k, r, j);
      };
      for (int l = 0; l < sr.n_lr; ++l) {
        const int k = sr.lr_line[l];
        if (k < klo || k > khi) continue;
        for (int jj = et; jj < nJ; jj += NSYNC) red_add(trw + sr.lr_out[l] + jb + jj, tval(k, jb + jj));
      }
      for (int l = 0; l < sr.n_ud; ++l) {
        const int j = sr.ud_line[l];
        if (j < jb || j >= je) continue;
        for (int k = klo + et; k <= khi; k += NSYNC) red_add(trw + sr.ud_out[l] + k, tval(k, j));
      }
    }
  };

  // ============================ producer ============================
  if (warp == 0) {
    if (lane < 2) {
      long long idx = 0;
      bool stopped = false;
      for (int li = 0; li < nline && !stopped; ++li) {
        const C* blk = fac + (size_t)line_k(li) * ny * ldn;
        for (int c = 0; c < nch; ++c, ++idx) {
          if ((idx & 1) != lane) continue;   // lanes 0 and 1 issue alternate chunks
          const int slot = (int)(idx % NS);
          if (idx >= NS) {
            if (!mbar_wait<false>(&empty[slot], (unsigned)(((idx / NS) - 1) & 1), a.err, abort_flag, a.wait_cycles)) {
              stopped = true;
              break;
            }
          }
          const int c0 = jb + c * CW;
          const int ncol = min(CW, je - c0);
          const unsigned bytes = (unsigned)(ncol * ldn * sizeof(C));
          mbar_expect_tx(&full[slot], bytes);
          bulk_g2s(ring + (size_t)slot * slot_elems, blk + (size_t)c0 * ldn, bytes, &full[slot]);
        }
      }
      // Wait (bounded by the limit alone) until the last copies this lane
      // issued have landed: after an abort the consumers stop waiting for
      // them, and no copy may write into shared memory after the CTA has left.
      // Without an abort they landed long ago and each wait returns at once.
      for (long long q = max(0LL, idx - NS); q < idx; ++q)
        if ((q & 1) == lane) mbar_wait<false>(&full[(int)(q % NS)], (unsigned)((q / NS) & 1), a.err, nullptr, a.wait_cycles);
    }
    return;
  }

  // ============================ helpers ============================
  if (warp == 1 || warp == 2) {
    const int ht = tid - 32;   // 0..63
    constexpr int UB = 8;      // loads in flight per helper thread
    // scratch row `row` (b_row, y_row) of my columns into H
    auto fetch = [&](int row) {
      const C* src = scr + ((size_t)row * ny + jb) * R;
      for (int e0 = ht; e0 < R * nJ; e0 += 64 * UB) {
        C v[UB];
#pragma unroll
        for (int u = 0; u < UB; ++u)
          if (e0 + 64 * u < R * nJ) v[u] = src[e0 + 64 * u];
#pragma unroll
        for (int u = 0; u < UB; ++u)
          if (e0 + 64 * u < R * nJ) H[e0 + 64 * u] = v[u];
      }
    };
    prologue(NCT + ht);
    named_sync(1, NSYNC);     // every b_k is in scratch
    fetch(srow(line_k(0)));
    named_sync(1, NSYNC);     // S0: H = b of my first line
    named_sync(1, NSYNC);     // S0b: consumers copied it into V
    for (int li = 0; li < nline; ++li) {
      if (li < nf) {
        fetch(srow(line_k(li + 1)));    // b of the next line (the middle line's after the last)
      } else if (li > nf) {
        fetch(line_k(li));              // y_k / z_k
      }
      named_sync(1, NSYNC);   // sync1
      named_sync(1, NSYNC);   // sync2
    }
    named_sync(1, NSYNC);     // every x_k is stored
    epilogue(NCT + ht);
    return;
  }

  // ============================ writer ============================
  if (warp == 3) {
    prologue(NCT + 64 + lane);
    named_sync(1, NSYNC);     // every b_k is in scratch
    named_sync(1, NSYNC);     // S0
    named_sync(1, NSYNC);     // S0b
    for (int li = 0; li < nline; ++li) {
      const int k = line_k(li);
      named_sync(1, NSYNC);   // sync1
      named_sync(1, NSYNC);   // sync2: Y (forward y_k / z_k, middle x_m) or V (backward x_k) is complete
      // forward y_k / z_k, then backward x_k over it; x_m by the top half only
      if (li == nf && half == 1) continue;
      const C* src = li <= nf ? Y : V;
      C* dst = scr + ((size_t)k * ny + jb) * R;
      for (int e = lane; e < R * nJ; e += 32) dst[e] = src[e];
    }
    named_sync(1, NSYNC);     // every x_k is stored
    epilogue(NCT + 64 + lane);
    return;
  }

  // ============================ consumers ============================
  const int cw = warp - kAux;
  if (cw >= NCW) return;   // idle warp (small cell)
  const int ct = cw * 32 + lane;
  const int sg = cw / (KSW * RG), rg = (cw / KSW) % RG, ks = cw % KSW;   // FMA matvec: slot group, row group, slice
  const int sb = sg * RS;                                                  // first slot of my slot group
  const int r0 = rg * 64 + 2 * lane;    // my row pair
  const bool rows_ok = r0 < ldn;

  // split: the mma B words of input entry e = (column, slot) of the next line,
  // n = 2 slot: (re, -im), n = 2 slot + 1: (im, re), hi and lo terms
  auto write_bw = [&](int e, C v) {
    if constexpr (TC) {
      // B rows n = 2 slot (Re of the product): [Re, -Im]; n = 2 slot + 1: [Im, Re]
      const int jj = e / R, r = e - jj * R;
      put3(Bop, b_term, b_off(2 * r, 2 * jj, TN), v.x, -v.y);
      put3(Bop, b_term, b_off(2 * r + 1, 2 * jj, TN), v.y, v.x);
    }
    if constexpr (SPLIT) {
      const int jj = e / R, r = e - jj * R;
      unsigned h0, l0, h1, l1;
      split_pair(v.x, -v.y, h0, l0);
      split_pair(v.y, v.x, h1, l1);
      BwH[(size_t)jj * NT8 + 2 * r] = h0;
      BwL[(size_t)jj * NT8 + 2 * r] = l0;
      BwH[(size_t)jj * NT8 + 2 * r + 1] = h1;
      BwL[(size_t)jj * NT8 + 2 * r + 1] = l1;
    }
  };

  prologue(ct);
  named_sync(1, NSYNC);       // every b_k is in scratch
  named_sync(1, NSYNC);       // S0
  for (int e = ct; e < R * nJ; e += NCT) {
    V[e] = H[e];
    write_bw(e, H[e]);
  }
  if constexpr (TC) fence_async_smem();
  named_sync(1, NSYNC);       // S0b

  // bytes of partial sums that land in my Q per line: my rows x R x CL CTAs
  const unsigned line_bytes = (unsigned)(nJ * R * CL * sizeof(C));
  if (CL > 1 && ct == 0) mbar_expect_tx(&pready[0], line_bytes);
  long long idx = 0;
  int gkb = 0;                          // tensor-core items: k-blocks issued so far
  for (int li = 0; li < nline; ++li) {
    const int k = line_k(li);
    const int buf = li & 1;
    // arm the next line's barrier: its buffer was last read before the
    // previous sync2 (peers' bytes may land before this; the phase cannot
    // complete without this arrive)
    if (CL > 1 && ct == 0 && li + 1 < nline) mbar_expect_tx(&pready[(li + 1) & 1], line_bytes);
    C* Qb = Q + buf * qbuf;
    if constexpr (TC) {
      // ---- partial products of all rows with my columns on the tensor cores ----
      // per k-block of 8 columns: the consumer warps convert the block's
      // factor columns into the A stage, one thread issues the six products
      // of each 128-row tile into TMEM and commits them to the stage's
      // barrier; the next block is converted meanwhile into the other stage
      const unsigned tb = *tslot;
      // D FP32, A and B bf16, both K-major, N = TN, M = 128
      constexpr unsigned idesc =
          (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(TN >> 3) << 17) | ((unsigned)(128 >> 4) << 24);
      int kb_line = 0;
      for (int c = 0; c < nch; ++c, ++idx) {
        const int slot = (int)(idx % NS);
        const bool ok = mbar_wait<false>(&full[slot], (unsigned)((idx / NS) & 1), a.err, abort_flag, a.wait_cycles);
        const C* S = ring + (size_t)slot * slot_elems;
        const int c0 = c * CW;
        const int ncol = min(CW, nJ - c0);
        const int nkb = (ncol + 7) >> 3;
        for (int kb = 0; kb < nkb; ++kb, ++gkb, ++kb_line) {
          const int stg = gkb % kTcStages;
          // the products that last read this stage are complete
          if (gkb >= kTcStages)
            mbar_wait<false>(&mmab[stg], (unsigned)(((gkb - kTcStages) / kTcStages) & 1), a.err, abort_flag,
                             a.wait_cycles);
          unsigned char* As = Ast + (size_t)stg * 3 * a_term;
          // a warp pass: 8 rows x 4 columns, one 128-byte core-matrix row per term
          for (int u = cw; u < MT * 32; u += NCW) {
            const int row = (u >> 1) * 8 + (lane >> 2);
            const int cq = (u & 1) * 4 + (lane & 3);   // column within the k-block
            const int cc = kb * 8 + cq;                 // column within the chunk
            C v = czero<C>();
            if (ok && row < ldn && cc < ncol) v = S[(size_t)cc * ldn + row];
            put3(As, a_term, (row >> 7) * kTcTile + a_off(row & 127, 2 * cq), v.x, v.y);
          }
          fence_async_smem();
          named_sync(2, NCT);   // the stage is written
          if (ct == 0) {
            tc_fence_after();
            const unsigned a0 = saddr(As), b0 = saddr(Bop);
            const int kk = 2 * (c0 + kb * 8);   // the block's first k in B (a multiple of 16)
            const unsigned bk = (unsigned)((kk >> 5) * (TN * 64) + ((kk >> 4) & 1) * 256);
            for (int t = 0; t < MT; ++t) {
#pragma unroll
              for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j + i < 3; ++j)
                  tc_mma(tb + (unsigned)(t * TN), tc_desc(a0 + (unsigned)(i * a_term + t * kTcTile), 256u),
                         tc_desc(b0 + (unsigned)(j * b_term) + bk, 512u), idesc,
                         (kb_line > 0 || i + j > 0) ? 1u : 0u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             saddr(&mmab[stg]))
                         : "memory");
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[slot]);
      }
      // the line's products are complete: each row's sums (lane r of tile t
      // in TMEM) to the CTA of my half that owns the row
      const int tq = cw >> 2;
      if (tq < MT) {
        mbar_wait<false>(&mmab[(gkb - 1) % kTcStages], (unsigned)(((gkb - 1) / kTcStages) & 1), a.err, abort_flag,
                         a.wait_cycles);
        tc_fence_after();
        float d[TN];
        tm_ld<TN>(tb + ((unsigned)((cw & 3) * 32) << 16) + (unsigned)(tq * TN), d);
        tc_fence_before();
        const int row = tq * 128 + (cw & 3) * 32 + lane;
        if (row < ny) {
          const int info = rowinfo[row];
          C* dst = Qb + ((size_t)crank * nJcap + (info & 0xffff)) * R;
#pragma unroll
          for (int q2 = 0; q2 < R / 2; ++q2) {
            const C v0 = make_float2(d[4 * q2], d[4 * q2 + 1]);
            const C v1 = make_float2(d[4 * q2 + 2], d[4 * q2 + 3]);
            if (CL == 1) {
              dst[2 * q2] = v0;
              dst[2 * q2 + 1] = v1;
            } else {
              st_async2(dst + 2 * q2, (unsigned)(info >> 16), v0, v1, &pready[buf]);
            }
          }
        }
      }
    } else if constexpr (SPLIT) {
      // ---- tensor-core partial products: my 16-row m-tile with all my columns ----
      // A (factor, bf16 hi/lo words, column-major) x B (next input, [column][n])
      // on mma.sync m16n8k16: three products hi*hi + hi*lo + lo*hi per k-step
      float cacc[NT][4];
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) cacc[nt][0] = cacc[nt][1] = cacc[nt][2] = cacc[nt][3] = 0.f;
      const int g = lane >> 2, t = lane & 3, mb = cw * 16;
      for (int c = 0; c < nch; ++c, ++idx) {
        const int slot = (int)(idx % NS);
        const bool ok = mbar_wait<false>(&full[slot], (unsigned)((idx / NS) & 1), a.err, abort_flag, a.wait_cycles);
        const uint2* S2 = reinterpret_cast<const uint2*>(ring + (size_t)slot * slot_elems) + mb + g;
        const int c0 = c * CW;
        const int nks = (min(CW, nJ - c0) + 7) >> 3;
        if (ok) {
          for (int kq = 0; kq < nks; ++kq) {
            const uint2* pa = S2 + (size_t)(kq * 8 + t) * ldn;
            const uint2 e0 = pa[0], e1 = pa[8], e2 = pa[4 * (size_t)ldn], e3 = pa[4 * (size_t)ldn + 8];
            const size_t bo = (size_t)(c0 + kq * 8 + t) * NT8 + g;
#pragma unroll
            for (int nt = 0; nt < NT; ++nt) {
              const unsigned bh0 = BwH[bo + nt * 8], bh1 = BwH[bo + 4 * NT8 + nt * 8];
              const unsigned bl0 = BwL[bo + nt * 8], bl1 = BwL[bo + 4 * NT8 + nt * 8];
              mma_bf16(cacc[nt], e0.x, e1.x, e2.x, e3.x, bh0, bh1);
              mma_bf16(cacc[nt], e0.x, e1.x, e2.x, e3.x, bl0, bl1);
              mma_bf16(cacc[nt], e0.y, e1.y, e2.y, e3.y, bh0, bh1);
            }
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[slot]);
      }
      // lane (g, t) holds slot nt*4 + t (real, imaginary) of rows mb+g and mb+g+8:
      // push each to the CTA that owns the row
#pragma unroll
      for (int nt = 0; nt < NT; ++nt) {
        const int sidx = nt * 4 + t;
        if (sidx < R) {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int row = mb + g + 8 * h;
            if (row < ny) {
              C v;
              v.x = cacc[nt][2 * h];
              v.y = cacc[nt][2 * h + 1];
              const int info = rowinfo[row];
              C* dst = Qb + ((size_t)crank * nJcap + (info & 0xffff)) * R + sidx;
              if (CL == 1) *dst = v;
              else st_async(dst, (unsigned)(info >> 16), v, &pready[buf]);
            }
          }
        }
      }
    } else {
      // ---- partial products of my row pair with my slice of my columns ----
      C acc0[RS], acc1[RS];
  #pragma unroll
      for (int r = 0; r < RS; ++r) { acc0[r] = czero<C>(); acc1[r] = czero<C>(); }
      for (int c = 0; c < nch; ++c, ++idx) {
        const int slot = (int)(idx % NS);
        const bool ok = mbar_wait<false>(&full[slot], (unsigned)((idx / NS) & 1), a.err, abort_flag, a.wait_cycles);
        const C* S = ring + (size_t)slot * slot_elems + r0;
        const int c0 = c * CW;
        const int ncol = min(CW, nJ - c0);
        if (ok && rows_ok) {
          // deeper unrolling (more loads in flight) where the registers allow
          constexpr int UNR = (RS <= 4 && sizeof(T) == 4) ? 4 : 2;
  #pragma unroll UNR
          for (int cc = ks; cc < ncol; cc += KSW) {
            Pair<T> s;
            s.load(S + (size_t)cc * ldn);
            const C* v = V + (size_t)(c0 + cc) * R + sb;
  #pragma unroll
            for (int r = 0; r < RS; ++r) {
              const C vr = v[r];
              cfma(acc0[r], s.a, vr);
              cfma(acc1[r], s.b, vr);
            }
          }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[slot]);
      }
      // sum the row group's column slices in shared memory, then push each
      // row's sum to the CTA that owns the row
      // (rows fastest: a lane's row pair is one 16-byte store per slot for
      // float, and consecutive lanes hit consecutive banks)
      const int RG64 = 64 * RG;
      {
        C* ls = LS + ((size_t)ks * R + sb) * RG64 + r0;
  #pragma unroll
        for (int r = 0; r < RS; ++r) { ls[(size_t)r * RG64] = acc0[r]; ls[(size_t)r * RG64 + 1] = acc1[r]; }
      }
      named_sync(3 + rg, KSW * SG * 32);
      {
        constexpr int UP = (sizeof(T) == 4 && R % 2 == 0) ? 2 : 1;   // slots per store
        constexpr int NU = R / UP;                                  // stores per row
        const size_t lsplane = (size_t)R * RG64;
        for (int u = (sg * KSW + ks) * 32 + lane; u < 64 * NU; u += KSW * SG * 32) {
          const int up = u >> 6, rr = u & 63;   // consecutive lanes take consecutive rows
          const int row = rg * 64 + rr;
          if (row >= ny) continue;
          const C* src = LS + (size_t)up * UP * RG64 + row;
          C v0 = src[0], v1 = UP == 2 ? src[RG64] : czero<C>();
          for (int q = 1; q < KSW; ++q) {
            v0 = cadd(v0, src[q * lsplane]);
            if (UP == 2) v1 = cadd(v1, src[q * lsplane + RG64]);
          }
          const int info = rowinfo[row];
          C* dst = Qb + ((size_t)crank * nJcap + (info & 0xffff)) * R + up * UP;
          if (CL == 1) {
            dst[0] = v0;
            if (UP == 2) dst[1] = v1;
          } else if constexpr (UP == 2) {
            st_async2(dst, (unsigned)(info >> 16), v0, v1, &pready[buf]);
          } else {
            st_async(dst, (unsigned)(info >> 16), v0, &pready[buf]);
          }
        }
      }
    }
    if (CL > 1) mbar_wait<true>(&pready[buf], (unsigned)((li >> 1) & 1), a.err, abort_flag, a.wait_cycles);
    named_sync(1, NSYNC);     // sync1: partials (cluster-wide) and H complete

    // ---- finish the line for my rows, element-wise ----
    // couplings toward the previous / next line of my chain: (w, e) for the
    // top half, (e, w) for the bottom half
    const int nplane = CL;
    if (li < nf) {
      // forward: y_k / z_k, then the next line's input
      const bool last = li + 1 == nf;
      const int kn = last ? mid : line_k(li + 1);
      const C cp = half == 0 ? wsh[kn] : esh[kn];
      for (int e = ct; e < R * nJ; e += NCT) {
        C s = czero<C>();
        const C* q = Qb + e;
        for (int pl = 0; pl < nplane; ++pl, q += qplane) s = cadd(s, *q);
        Y[e] = s;
        if (!last) {
          C b = H[e];
          cfms(b, cp, s);
          V[e] = b;
          write_bw(e, b);
        } else {
          st_async(P + e, partner, s, xch);   // to the other half's CTA with my columns
        }
      }
      if (last) {
        // middle input b_m - w_m y_{m-1} - e_m z_{m+1}, formed in the same
        // order in both halves so that both compute the same x_m
        mbar_wait<true>(xch, 0u, a.err, abort_flag, a.wait_cycles);
        const C wm = wsh[mid], em = esh[mid];
        for (int e = ct; e < R * nJ; e += NCT) {
          const C own = Y[e], oth = P[e];
          C b = H[e];
          cfms(b, wm, half == 0 ? own : oth);
          cfms(b, em, half == 0 ? oth : own);
          V[e] = b;
          write_bw(e, b);
        }
      }
    } else if (li == nf) {
      // middle: x_m, the first backward input of both halves
      for (int e = ct; e < R * nJ; e += NCT) {
        C s = czero<C>();
        const C* q = Qb + e;
        for (int pl = 0; pl < nplane; ++pl, q += qplane) s = cadd(s, *q);
        Y[e] = s;
        V[e] = s;
        write_bw(e, s);
      }
    } else {
      // backward: x_k = y_k - e_k (S_k^{-1} x_{k+1}) or z_k - w_k (T_k^{-1} x_{k-1})
      const C cn = half == 0 ? esh[k] : wsh[k];
      for (int e = ct; e < R * nJ; e += NCT) {
        C s = czero<C>();
        const C* q = Qb + e;
        for (int pl = 0; pl < nplane; ++pl, q += qplane) s = cadd(s, *q);
        C x = H[e];
        cfms(x, cn, s);
        V[e] = x;
        write_bw(e, x);
      }
    }
    if constexpr (TC) fence_async_smem();   // the B words, for the next line's products
    named_sync(1, NSYNC);     // sync2: V holds the next line's input
  }
  named_sync(1, NSYNC);       // every x_k is stored
  if constexpr (TC) {
    if (cw == 0) {
      // every product has completed (each line's were waited for before its
      // results were read; the wait below returns at once unless one ran out)
      if (gkb > 0)
        mbar_wait<false>(&mmab[(gkb - 1) % kTcStages], (unsigned)(((gkb - 1) / kTcStages) & 1), a.err, nullptr,
                         a.wait_cycles);
      tc_fence_after();
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*tslot), "r"((unsigned)kTcCols)
                   : "memory");
    }
  }
  epilogue(ct);

  {
    // nobody leaves while a peer may still write into its shared memory
    __syncwarp();
    if (lane < CLT) mbar_arrive_remote(&exitb[0], (unsigned)lane);
    // waited on even after an abort (bounded by the limit alone): a peer
    // still pushing partial sums into this CTA's shared memory keeps it alive
    mbar_wait<true>(&exitb[0], 0u, a.err, nullptr, a.wait_cycles);
  }
}

// 16 warps (4 auxiliary + up to 3 row groups x 4 column slices) x 128 registers
template <typename T, bool SPLIT, bool TCM = false>
__global__ void __maxnreg__(128) k_front(FrontArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const DevItem it = a.items[blockIdx.x / (2 * a.cluster)];
  const DevCell cl = a.cells[it.cell];
  const int n = it.slot_count;
  if constexpr (TCM) {
    // tensor-core items: 8 or 16 slots (fewer pad with empty slots)
    if (n <= 8) front_body<T, 8, false, true>(a, it, cl, smem);
    else front_body<T, 16, false, true>(a, it, cl, smem);
  } else if constexpr (sizeof(T) == 4) {
    if (n <= 1) front_body<T, 1, SPLIT>(a, it, cl, smem);
    else if (n <= 2) front_body<T, 2, SPLIT>(a, it, cl, smem);
    else if (n <= 4) front_body<T, 4, SPLIT>(a, it, cl, smem);
    else if (n <= 8) front_body<T, 8, SPLIT>(a, it, cl, smem);
    else if (n <= 12) front_body<T, 12, SPLIT>(a, it, cl, smem);
    else front_body<T, 16, SPLIT>(a, it, cl, smem);
  } else {
    if (n <= 1) front_body<T, 1, SPLIT>(a, it, cl, smem);
    else if (n <= 2) front_body<T, 2, SPLIT>(a, it, cl, smem);
    else if (n <= 4) front_body<T, 4, SPLIT>(a, it, cl, smem);
    else front_body<T, 8, SPLIT>(a, it, cl, smem);
  }
}

template <typename T>
size_t smem_need(int ldn_max, int ny_max, int nx_max, int R, int KSW, int CL, int CW, int NS, bool split,
                 bool tc = false) {
  using C = cx_t<T>;
  const int nJ = (ny_max + CL - 1) / CL + 1;
  // tensor-core items: A stages and the three B terms (+ alignment) instead of the slices' staging
  const size_t tc_bytes = (size_t)kTcStages * 3 * ((ldn_max + 127) / 128) * kTcTile +
                          (size_t)3 * 2 * R * ((2 * nJ + 31) & ~31) * 2 + 128;
  const size_t staging = split ? 2 * (size_t)(((nJ + 7) & ~7) + 8) * (8 * ((2 * R + 7) / 8)) * sizeof(unsigned)
                         : tc  ? tc_bytes
                               : (size_t)KSW * 64 * kMaxRG * R * sizeof(C);
  return kHdr + (size_t)NS * CW * ldn_max * sizeof(C) + 4 * (size_t)R * nJ * sizeof(C) + nx_max + nJ + 32 +
         2 * (size_t)CL * R * nJ * sizeof(C) + staging + 4 * (size_t)ny_max +
         2 * (size_t)nx_max * sizeof(C) +
         (size_t)R * (sizeof(DevSlot) + sizeof(SlotCoef) + sizeof(DevGroup)) + 12 * 16;
}

}  // namespace


namespace {

// The launch shape of a front: column slices, chunk width and ring depth for
// R slots on clusters of 2 CL CTAs; false if nothing fits in shared memory.
template <typename T>
bool front_shape(int max_ny, int max_nx, int R, int CL, bool split, int maxopt, int* ldn_out, int* ksw_out,
                 int* cw_out, int* ns_out, size_t* smem_out, bool tc = false) {
  int ldn = (max_ny + 3) & ~3;
  // tensor-core items: complex64, 8 or 16 slots, at most two 128-row tiles
  if (tc && (split || sizeof(T) != 4 || (R != 8 && R != 16) || ldn > 256)) return false;
  if (split) {   // the split factor layout's column stride (4 mod 8)
    ldn = max_ny;
    while (ldn % 8 != 4) ++ldn;
  }
  // largest chunk (columns, multiple of 8, <= ~64 KB) and then the deepest ring that fit
  const int nJmax = (max_ny + CL - 1) / CL;
  // column slices: as many as keep >= 4 columns per slice and the slices'
  // partial-sum staging (KSW x 192 x R) within 64 KB
  int KSW = kMaxKSW;
  // (complex64 with more than 8 slots: two slot groups, so at most 2 slices)
  const int sgroups = (!split && sizeof(T) == 4 && R > 8) ? 2 : 1;
  while (KSW > 1 && (split || tc || nJmax < 4 * KSW || KSW * sgroups > kMaxKSW ||
                     (size_t)KSW * 64 * kMaxRG * R * sizeof(cx_t<T>) > 65536))
    --KSW;
  const int cwmax = (int)std::min<size_t>(((size_t)65536 / ((size_t)ldn * sizeof(cx_t<T>))) & ~size_t(7),
                                          (size_t)((nJmax + 7) & ~7));
  int CW = std::max(8, cwmax), NS = 0;
  for (; CW >= 8; CW -= 8) {
    for (NS = 4; NS >= 2; --NS)
      if (smem_need<T>(ldn, max_ny, max_nx, R, KSW, CL, CW, NS, split, tc) <= (size_t)maxopt) break;
    if (NS >= 2) break;
  }
  if (CW < 8) return false;
  *ldn_out = ldn; *ksw_out = KSW; *cw_out = CW; *ns_out = NS;
  *smem_out = smem_need<T>(ldn, max_ny, max_nx, R, KSW, CL, CW, NS, split, tc);
  return true;
}

}  // namespace

int front_fit_mask(bool dbl, bool split, int max_ny, int max_nx, int slots, bool tc) {
  int dev = 0, maxopt = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const int R = tc ? front_tc_slots(slots) : std::min(front_rpad(std::max(1, slots)), front_rmax(dbl));
  int mask = 0, ldn, ksw, cw, ns;
  size_t smem;
  for (int cl = 1; cl <= 4; cl *= 2) {
    const bool ok = dbl ? front_shape<double>(max_ny, max_nx, R, cl, split, maxopt, &ldn, &ksw, &cw, &ns, &smem, tc)
                        : front_shape<float>(max_ny, max_nx, R, cl, split, maxopt, &ldn, &ksw, &cw, &ns, &smem, tc);
    if (ok) mask |= 1 << cl;
  }
  return mask;
}

template <typename T>
cudaError_t launch_front(const FrontArgs& a_in, int max_ny, int max_nx, cudaStream_t st) {
  if (a_in.item_count <= 0) return cudaSuccess;
  FrontArgs a = a_in;
  const bool dbl = sizeof(T) == 8;
  const bool split = a.split != 0;
  if (split && dbl) return cudaErrorInvalidValue;
  const bool tc = a.tc != 0;
  if (tc && (dbl || split || a.max_slots > 16)) return cudaErrorInvalidValue;
  const int R = tc ? front_tc_slots(a.max_slots) : std::min(front_rpad(std::max(1, a.max_slots)), front_rmax(dbl));
  if (a.cluster < 1) a.cluster = 1;
  if (a.cluster > 4 || max_nx < 5) return cudaErrorInvalidValue;   // clusters of <= 8; two lines per half
  int dev = 0, maxopt = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  int ldn = 0, KSW = 0, CW = 0, NS = 0;
  size_t smem = 0;
  if (!front_shape<T>(max_ny, max_nx, R, a.cluster, split, maxopt, &ldn, &KSW, &CW, &NS, &smem, tc))
    return cudaErrorInvalidConfiguration;
  a.ksw = KSW;
  a.stages = NS;
  a.chunk = CW;
  cudaLaunchConfig_t cfg{};
  cudaLaunchAttribute attr[1];
  cfg.gridDim = dim3((unsigned)(a.item_count * 2 * a.cluster));
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)(2 * a.cluster);   // top and bottom halves
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  void (*kern)(FrontArgs) = k_front<T, false>;
  if constexpr (sizeof(T) == 4) {
    if (split) kern = k_front<float, true>;
    else if (tc) kern = k_front<float, false, true>;
  }
  // the attribute is an upper bound: always the device maximum, so that
  // host threads launching concurrently never lower it under one another
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, maxopt);
  if (e != cudaSuccess) return e;
  cfg.blockDim = dim3(32 * (kAux + kMaxRG * kMaxKSW));
  return cudaLaunchKernelEx(&cfg, kern, a);
}

int front_max_clusters(bool dbl, int cluster) {
  int dev = 0, maxopt = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaLaunchConfig_t cfg{};
  cudaLaunchAttribute attr[1];
  cfg.gridDim = dim3((unsigned)(cluster * 1024));
  cfg.blockDim = dim3(32 * (kAux + kMaxRG * kMaxKSW));
  cfg.dynamicSmemBytes = (size_t)maxopt;   // one CTA per SM, as every front launch
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  cudaError_t e;
  if (dbl) {
    cudaFuncSetAttribute(k_front<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxopt);
    e = cudaOccupancyMaxActiveClusters(&n, k_front<double, false>, &cfg);
  } else {
    cudaFuncSetAttribute(k_front<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxopt);
    cudaFuncSetAttribute(k_front<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxopt);
    e = cudaOccupancyMaxActiveClusters(&n, k_front<float, false>, &cfg);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

namespace {
// One CTA waits on an mbarrier that nothing completes, with the bounded wait
// of the sweep kernels: the wait runs out after `limit` cycles, raises the
// error word and the kernel returns normally (no trap, nothing in flight).
__global__ void k_wait_probe(int* err, long long limit) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    abort_flag = 0;
    mbar_init(&bar, 1);   // expects one arrive that never comes
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait<false>(&bar, 0u, err, &abort_flag, limit);
  __syncthreads();
}
}  // namespace

cudaError_t launch_wait_probe(int* err, long long limit_cycles, cudaStream_t st) {
  k_wait_probe<<<1, 32, 0, st>>>(err, limit_cycles);
  return cudaGetLastError();
}

template cudaError_t launch_front<float>(const FrontArgs&, int, int, cudaStream_t);
template cudaError_t launch_front<double>(const FrontArgs&, int, int, cudaStream_t);

}  // namespace lsw
