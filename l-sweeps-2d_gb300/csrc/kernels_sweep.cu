// Sweep-front kernel: every cell solve of one front of the L-sweep
// preconditioner in one launch.
//
// A cell matrix is block tridiagonal over its x-lines (DOF order i*ny + j,
// AssemblerHelmholtz2DFD.cpp:166-177); the couplings between lines are scalar
// multiples of the identity (the PML profile is separable), so with the stored
// Schur-complement inverses Sinv_k (kernels_factor.cu) a solve is
//   forward   y_k = Sinv_k (b_k - w_k y_{k-1})
//   backward  x_k = y_k - e_k Sinv_k x_{k+1}
// (w_k, e_k = couplings of line k to k-1 / k+1).  One cell solve ("item")
// carries R right-hand sides ("slots") that share every factor block read.
//
// Work split.  An item runs on a thread-block cluster of CL CTAs; CTA c owns
// the column range J_c of every block (contiguous in the column-major factor)
// and the same range of every line vector.  Per line it forms the partial
// products of all rows with its columns; the partials are exchanged through
// distributed shared memory (each CTA sums the rows of its own range over the
// cluster), so every SM streams 1/CL of the factor.
//
// Roles inside a CTA: warp 0 is the producer that streams the CTA's column
// chunks (CW columns, contiguous) in the order the two substitutions consume
// them, through an NS-stage shared-memory ring (cp.async.bulk + mbarrier
// completion); warp 1 prefetches the next line's right-hand side (forward) or
// stored y_k (backward) into shared memory; the remaining warps are consumers
// (16 rows each, one row pair per lane group, 4*KS column phases) that
// accumulate in registers and reduce over phases with warp shuffles, then
// finish each line element-wise.  Owned DOFs and trace lines are accumulated
// with fire-and-forget global reductions.  Every wait is bounded: after ~2 s
// of clock cycles a wait raises the CTA's abort flag and *a.err, and all later
// waits return at once so every thread still reaches every barrier.
//
// The right-hand sides are never materialised: a slot builds b_k on the fly
// from the global input (stage 1, the window of DDCheckerboard::getSeparatedRHS,
// DDCheckerboard.cpp:3564-3674, restricted to the owned set) or from its
// neighbours' trace lines (equivalent sources of
// SubdomainStructured::getEquivalentSources, SubdomainStructured.cpp:1304-1465,
// and the L-shaped traces of extractLTraces, 1468-1539).  The backward pass
// accumulates owned DOFs into the output (reduce, DDCheckerboard.cpp:744-772)
// and the outgoing trace lines into the trace pool.
#include "common.cuh"
#include "internal.h"

namespace lsw {

namespace {

constexpr int kMaxRG = 14;            // row groups of 16 rows: ny <= 224
constexpr int kNSMax = 8;             // ring stages
constexpr int kHdr = 256;             // barrier header bytes
constexpr int SK_NONE = 99;           // padding slot
constexpr long long kWaitCycles = 4000000000LL;   // ~2 s at 2 GHz

template <typename T> struct FCfg;
template <> struct FCfg<float> { static constexpr int CW = 16; };
template <> struct FCfg<double> { static constexpr int CW = 8; };

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
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait (see the file comment).
template <bool CLUSTER>
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity, int* err, volatile int* abort_flag) {
  auto tw = [&]() { return CLUSTER ? mbar_try_wait_cluster(b, parity) : mbar_try_wait(b, parity); };
  if (tw()) return true;
  const long long t0 = clock64();
  while (true) {
    if (*abort_flag) return false;
    if (tw()) return true;
    if (clock64() - t0 > kWaitCycles) {
      *abort_flag = 1;
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
__device__ __forceinline__ float2 ld_remote(const float2* p, unsigned rank) {
  float2 v;
  // "memory": must not be hoisted above the barrier wait that publishes the data
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
__device__ __forceinline__ void red_add(float2* p, float2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}
__device__ __forceinline__ void red_add(double2* p, double2 v) {
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

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

template <typename C> __device__ __forceinline__ C shfl_xor_c(C v, int m) {
  v.x = __shfl_xor_sync(0xffffffffu, v.x, m);
  v.y = __shfl_xor_sync(0xffffffffu, v.y, m);
  return v;
}

template <typename T, int KS, int R>
__device__ void front_body(const FrontArgs& a, const DevItem& it, const DevCell& cl, unsigned char* smem) {
  using C = cx_t<T>;
  constexpr int CW = FCfg<T>::CW;
  constexpr int NPH = 4 * KS;          // column phases per chunk
  constexpr int CPL = CW / NPH;        // columns per lane per chunk
  static_assert(CW % NPH == 0, "chunk width");
  static_assert((2 * kNSMax + 3) * 8 + 4 <= kHdr, "barrier header");
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nx = cl.nx, ny = cl.ny, ldn = cl.ldn;
  int CL = a.cluster;
  const int NS = a.stages;
  unsigned crank = CL > 1 ? cluster_rank() : 0u;
  if (CL > 1 && (cluster_size() != (unsigned)CL || crank != blockIdx.x % (unsigned)CL)) {
    // the launch did not form the clusters this kernel was configured for
    if (threadIdx.x == 0) atomicOr(a.err, 4);
    CL = 1;
    crank = 0;
  }
  const int jb = (int)crank * ny / CL, je = ((int)crank + 1) * ny / CL;
  const int nJ = je - jb;               // my columns / rows of every line
  const int RG = (ny + 15) >> 4;
  const int PR = 16 * RG;               // rows of a partial-sum plane
  const int NCW = KS * RG;              // consumer warps
  const int NCT = NCW * 32;
  const int NSYNC = NCT + 32;           // consumers + helper warp
  const int nch = (nJ + CW - 1) / CW;   // chunks per line
  const int nslot = it.slot_count;
  const int nline = 2 * nx - 1;         // forward 0..nx-1, backward nx-2..0

  // ---- shared layout ----
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + kNSMax;
  uint64_t* pready = empty + kNSMax;    // [2]: partial sums of a line are complete cluster-wide
  uint64_t* exitb = pready + 2;         // cluster-wide "done with remote shared memory"
  volatile int* abort_flag = reinterpret_cast<volatile int*>(exitb + 1);
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
  C* V = reinterpret_cast<C*>(p);       // [R][nJ]  input vector of the current line (my columns)
  p = al16(p + (size_t)R * nJcap * sizeof(C));
  C* H = reinterpret_cast<C*>(p);       // [R][nJ]  helper: next right-hand side or stored y_k
  p = al16(p + (size_t)R * nJcap * sizeof(C));
  C* P = reinterpret_cast<C*>(p);       // [2][KS][R][PR] partial sums (double-buffered)
  const size_t pbuf = (size_t)KS * R * PR;
  p = al16(p + 2 * pbuf * sizeof(C));
  DevSlot* sl = reinterpret_cast<DevSlot*>(p);
  p = al16(p + sizeof(DevSlot) * R);
  SlotCoef* cf = reinterpret_cast<SlotCoef*>(p);
  p = al16(p + sizeof(SlotCoef) * R);
  DevGroup* gr = reinterpret_cast<DevGroup*>(p);

  const C* tr = reinterpret_cast<const C*>(a.traces);
  C* trw = reinterpret_cast<C*>(a.traces);
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
  if (tid == 0) {
    *abort_flag = 0;
    for (int i = 0; i < NS; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], NCW); }
    mbar_init(&pready[0], CL * NCW);
    mbar_init(&pready[1], CL * NCW);
    mbar_init(&exitb[0], CL * NCW);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (CL > 1) {
    // every CTA's barriers are initialised before anyone arrives remotely
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  }

  // ============================ producer ============================
  if (warp == 0) {
    if (lane == 0) {
      long long idx = 0;
      for (int li = 0; li < nline; ++li) {
        const int k = li < nx ? li : 2 * nx - 2 - li;
        const C* blk = fac + (size_t)k * ny * ldn;
        for (int c = 0; c < nch; ++c, ++idx) {
          const int slot = (int)(idx % NS);
          if (idx >= NS) {
            if (!mbar_wait<false>(&empty[slot], (unsigned)(((idx / NS) - 1) & 1), a.err, abort_flag)) return;
          }
          const int c0 = jb + c * CW;
          const int ncol = min(CW, je - c0);
          const unsigned bytes = (unsigned)(ncol * ldn * sizeof(C));
          mbar_expect_tx(&full[slot], bytes);
          bulk_g2s(ring + (size_t)slot * slot_elems, blk + (size_t)c0 * ldn, bytes, &full[slot]);
        }
      }
    }
    return;
  }

  // ============================ helper ============================
  if (warp == 1) {
    // line 0 right-hand side
    for (int e = lane; e < R * nJ; e += 32) {
      const int r = e / nJ, j = jb + (e - r * nJ);
      H[e] = rhs_elem<T>(a, cl, sl[r], cf[r], tr, 0, j);
    }
    named_sync(1, NSYNC);     // S0: H = b_0
    named_sync(1, NSYNC);     // S0b: consumers copied it into V
    for (int li = 0; li < nline; ++li) {
      const bool fwd = li < nx;
      const int k = fwd ? li : 2 * nx - 2 - li;
      if (fwd) {
        if (k + 1 < nx)
          for (int e = lane; e < R * nJ; e += 32) {
            const int r = e / nJ, j = jb + (e - r * nJ);
            H[e] = rhs_elem<T>(a, cl, sl[r], cf[r], tr, k + 1, j);
          }
      } else {
        const C* yk = scr + (size_t)k * R * ny;
        for (int e = lane; e < R * nJ; e += 32) {
          const int r = e / nJ, jj = e - r * nJ;
          H[e] = yk[(size_t)r * ny + jb + jj];
        }
      }
      named_sync(1, NSYNC);   // sync1
      named_sync(1, NSYNC);   // sync2
    }
    return;
  }

  // ============================ consumers ============================
  const int cw = warp - 2;
  if (cw >= NCW) return;   // idle warp (small cell)
  const int ct = cw * 32 + lane;
  const int rg = cw / KS, ks = cw % KS;
  const int rpl = lane & 7, cs = lane >> 3;
  const int phase = ks * 4 + cs;
  const int r0 = rg * 16 + 2 * rpl;
  const bool rows_ok = r0 < ldn;

  named_sync(1, NSYNC);       // S0
  for (int e = ct; e < R * nJ; e += NCT) V[e] = H[e];
  named_sync(1, NSYNC);       // S0b

  long long idx = 0;
  for (int li = 0; li < nline; ++li) {
    const bool fwd = li < nx;
    const int k = fwd ? li : 2 * nx - 2 - li;
    const int buf = li & 1;
    // ---- partial products of all rows with my columns ----
    C acc0[R], acc1[R];
#pragma unroll
    for (int r = 0; r < R; ++r) { acc0[r] = czero<C>(); acc1[r] = czero<C>(); }
    for (int c = 0; c < nch; ++c, ++idx) {
      const int slot = (int)(idx % NS);
      const bool ok = mbar_wait<false>(&full[slot], (unsigned)((idx / NS) & 1), a.err, abort_flag);
      const C* S = ring + (size_t)slot * slot_elems;
      const int c0 = c * CW;
      const int ncol = min(CW, nJ - c0);
#pragma unroll
      for (int q = 0; q < CPL; ++q) {
        const int cc = phase + NPH * q;
        if (ok && cc < ncol && rows_ok) {
          Pair<T> s;
          s.load(S + (size_t)cc * ldn + r0);
          const C* v = V + c0 + cc;
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const C vr = v[(size_t)r * nJ];
            cfma(acc0[r], s.a, vr);
            cfma(acc1[r], s.b, vr);
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[slot]);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      acc0[r] = cadd(acc0[r], shfl_xor_c(acc0[r], 8));
      acc0[r] = cadd(acc0[r], shfl_xor_c(acc0[r], 16));
      acc1[r] = cadd(acc1[r], shfl_xor_c(acc1[r], 8));
      acc1[r] = cadd(acc1[r], shfl_xor_c(acc1[r], 16));
    }
    C* Pb = P + buf * pbuf;
    if (cs == 0) {
      C* pp = Pb + (size_t)ks * R * PR + r0;
#pragma unroll
      for (int r = 0; r < R; ++r) { pp[(size_t)r * PR] = acc0[r]; pp[(size_t)r * PR + 1] = acc1[r]; }
    }
    if (CL > 1) {
      __syncwarp();
      if (lane < CL) mbar_arrive_remote(&pready[buf], (unsigned)lane);
      mbar_wait<true>(&pready[buf], (unsigned)((li >> 1) & 1), a.err, abort_flag);
    }
    named_sync(1, NSYNC);     // sync1: partials (cluster-wide) and H complete

    // ---- finish the line for my rows, element-wise ----
    const C wk = (fwd && k + 1 < nx) ? to_c(px[k + 1], czero<C>()) : czero<C>();
    const C ek = to_c(px[nx + k], czero<C>());
    C* yk = scr + (size_t)k * R * ny;
    for (int e = ct; e < R * nJ; e += NCT) {
      const int r = e / nJ, jj = e - r * nJ, j = jb + jj;
      C s = czero<C>();
      for (int cr = 0; cr < CL; ++cr) {
#pragma unroll
        for (int q = 0; q < KS; ++q) {
          const C* src = Pb + ((size_t)q * R + r) * PR + j;
          s = cadd(s, (CL > 1 && cr != (int)crank) ? ld_remote(src, (unsigned)cr) : *src);
        }
      }
      if (fwd) {
        yk[(size_t)r * ny + j] = s;
        if (k + 1 < nx) {
          C b = H[e];
          cfms(b, wk, s);
          V[e] = b;
        } else {
          V[e] = s;   // x_{K-1} = y_{K-1}
        }
      } else {
        C x = H[e];
        cfms(x, ek, s);
        V[e] = x;
      }
    }
    named_sync(1, NSYNC);     // sync2: V holds r_{k+1} (forward) or x_k

    // ---- epilogue on x_k (backward, and the last forward line) ----
    if (!fwd || k == nx - 1) {
      const bool kx0 = k >= cl.ownx[0][0] && k <= cl.ownx[0][1];
      const bool kx1 = k >= cl.ownx[1][0] && k <= cl.ownx[1][1];
      const long long rowoff = (long long)(cl.lox + k) * a.n_dof + cl.loy;
      for (int e = ct; e < it.group_count * nJ; e += NCT) {
        const int g = e / nJ, j = jb + (e - g * nJ);
        const DevGroup G = gr[g];
        if (G.out_off < 0) continue;
        const int sy = (G.shift >> 1) & 1;
        if (!((G.shift & 1) ? kx1 : kx0) || j < cl.owny[sy][0] || j > cl.owny[sy][1]) continue;
        C sum = czero<C>();
        for (int q = 0; q < G.slot_count; ++q) sum = cadd(sum, V[(size_t)(G.slot_begin + q) * nJ + (j - jb)]);
        red_add(outs + G.out_off + rowoff + j, sum);
      }
      for (int e = ct; e < R * nJ; e += NCT) {
        const int r = e / nJ, jj = e - r * nJ, j = jb + jj;
        const DevSlot& s = sl[r];
        if (s.kind == SK_NONE) continue;
        const C xv = V[e];
        if (s.kind == SK_CELLVEC) {
          a.x_out[(long long)s.rhs * a.out_stride + (long long)k * ny + j] = to_c(xv, make_double2(0, 0));
          continue;
        }
        C v = xv;
        if (s.overwrite) {
          if (j == s.yo) v = tr[s.in_ud0 + k];
          else if (k == s.xo) v = tr[s.in_lr0 + j];
        }
        for (int l = 0; l < s.n_lr; ++l)
          if (s.lr_line[l] == k) red_add(trw + s.lr_out[l] + j, v);
        for (int l = 0; l < s.n_ud; ++l)
          if (s.ud_line[l] == j) red_add(trw + s.ud_out[l] + k, v);
      }
    }
  }

  if (CL > 1) {
    // nobody leaves while a peer may still read its partial sums
    __syncwarp();
    if (lane < CL) mbar_arrive_remote(&exitb[0], (unsigned)lane);
    mbar_wait<true>(&exitb[0], 0u, a.err, abort_flag);
  }
}

// register budget: the warps of a CTA spread over the 4 sub-partitions of an
// SM, each with 16K registers: 16 warps (KS = 1) -> 128, 30 warps -> 64
template <int KS> struct RegCap;
template <> struct RegCap<1> { static constexpr int v = 128; };   // 512 threads
template <> struct RegCap<2> { static constexpr int v = 64; };    // 960 threads

template <typename T, int KS>
__global__ void __maxnreg__(RegCap<KS>::v) k_front(FrontArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const DevItem it = a.items[blockIdx.x / a.cluster];
  const DevCell cl = a.cells[it.cell];
  const int n = it.slot_count;
  if constexpr (sizeof(T) == 4 && KS == 1) {
    if (n <= 1) front_body<T, KS, 1>(a, it, cl, smem);
    else if (n <= 2) front_body<T, KS, 2>(a, it, cl, smem);
    else if (n <= 4) front_body<T, KS, 4>(a, it, cl, smem);
    else if (n <= 8) front_body<T, KS, 8>(a, it, cl, smem);
    else if (n <= 12) front_body<T, KS, 12>(a, it, cl, smem);
    else front_body<T, KS, 16>(a, it, cl, smem);
  } else if constexpr (KS == 2) {
    if (n <= 1) front_body<T, KS, 1>(a, it, cl, smem);
    else if (n <= 2) front_body<T, KS, 2>(a, it, cl, smem);
    else front_body<T, KS, 4>(a, it, cl, smem);
  } else {
    if (n <= 1) front_body<T, KS, 1>(a, it, cl, smem);
    else if (n <= 2) front_body<T, KS, 2>(a, it, cl, smem);
    else if (n <= 4) front_body<T, KS, 4>(a, it, cl, smem);
    else front_body<T, KS, 8>(a, it, cl, smem);
  }
}

template <typename T>
size_t smem_need(int ldn_max, int ny_max, int R, int KS, int CL, int NS) {
  using C = cx_t<T>;
  const int RG = (ny_max + 15) / 16;
  const int nJ = (ny_max + CL - 1) / CL + 1;
  return kHdr + (size_t)NS * FCfg<T>::CW * ldn_max * sizeof(C) + 2 * (size_t)R * nJ * sizeof(C) +
         2 * (size_t)KS * R * 16 * RG * sizeof(C) +
         (size_t)R * (sizeof(DevSlot) + sizeof(SlotCoef) + sizeof(DevGroup)) + 6 * 16;
}

}  // namespace

int front_rmax(bool dbl) { return dbl ? 8 : 16; }
int front_rpad(int n) { return n <= 1 ? 1 : n <= 2 ? 2 : n <= 4 ? 4 : n <= 8 ? 8 : n <= 12 ? 12 : 16; }

template <typename T>
cudaError_t launch_front(const FrontArgs& a_in, int max_ny, cudaStream_t st) {
  if (a_in.item_count <= 0) return cudaSuccess;
  FrontArgs a = a_in;
  const bool dbl = sizeof(T) == 8;
  const int ldn = (max_ny + 3) & ~3;
  // two consumer warps per row group for small slot counts (float)
  const int KS = (!dbl && a.max_slots <= 4) ? 2 : 1;
  const int R = dbl ? 8 : (KS == 2 ? 4 : 16);
  if (a.cluster < 1) a.cluster = 1;
  int dev = 0, maxopt = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxopt, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  int NS = kNSMax;
  while (NS > 2 && smem_need<T>(ldn, max_ny, R, KS, a.cluster, NS) > (size_t)maxopt) --NS;
  a.stages = NS;
  const size_t smem = smem_need<T>(ldn, max_ny, R, KS, a.cluster, NS);
  if (smem > (size_t)maxopt) return cudaErrorInvalidConfiguration;
  cudaLaunchConfig_t cfg{};
  cudaLaunchAttribute attr[1];
  cfg.gridDim = dim3((unsigned)(a.item_count * a.cluster));
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)a.cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e;
  if constexpr (sizeof(T) == 4) {
    if (KS == 2) {
      auto kern = k_front<T, 2>;
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      cfg.blockDim = dim3(64 + 2 * kMaxRG * 32);
      return cudaLaunchKernelEx(&cfg, kern, a);
    }
  }
  auto kern = k_front<T, 1>;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  cfg.blockDim = dim3(64 + kMaxRG * 32);
  return cudaLaunchKernelEx(&cfg, kern, a);
}

template cudaError_t launch_front<float>(const FrontArgs&, int, cudaStream_t);
template cudaError_t launch_front<double>(const FrontArgs&, int, cudaStream_t);

}  // namespace lsw
