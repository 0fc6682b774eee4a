// C ABI of the GB300 L-sweeps library (declared in include/lsweeps.h).
#include "common.cuh"
#include "internal.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

namespace lsw {
}

using namespace lsw;
using cplx = std::complex<double>;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~DevBuf() { if (p) cudaFree(p); }
  cudaError_t ensure(size_t b) {
    if (b <= bytes && p) return cudaSuccess;
    if (p) { cudaFree(p); p = nullptr; bytes = 0; }
    if (b == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  template <typename X> X* as() const { return reinterpret_cast<X*>(p); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

struct lsw_ctx {
  int device = 0;
  std::string err;
  // problem
  bool is_setup = false, factorized = false;
  lsw_geom geom{};
  int N = 0, m = 0, p = 0, n_g = 0, n_dof = 0, prec = 0;
  double h = 0, omega = 0, C = 0;
  long long n2 = 0;
  int max_nx = 0, max_ny = 0, ncell = 0;
  long long LP = 0;
  std::vector<DevCell> cells;
  DevBuf d_cells, d_prof, d_gprof, d_m, d_fac, d_work, d_status;
  // per batch size
  std::map<int, std::unique_ptr<Schedule>> sched;
  std::map<int, std::unique_ptr<DevBuf[]>> sched_bufs;
  DevBuf d_traces, d_outs, d_scratch;
  // Krylov workspace
  DevBuf k_basis, k_zbasis, k_tmp, k_tmp2, k_r, k_part, k_small, k_small2, k_nrm, k_ls;
  // local-solve workspace
  DevBuf ls_items, ls_slots, ls_scratch;
  // lsw_solve_host's device copies of b and x, kept between calls
  DevBuf h_b, h_x;
  size_t fixed_bytes = 0;
  long long launches = 0;
  int nsm = 152;
  int max_cluster = 8;
  int krylov_batch = 0;   // right-hand sides per Krylov sub-batch at most (0: as memory allows)
  bool factor_lookahead = true;
  // complex64 / split factorisation on the tensor cores (else the CUDA-core kernel)
  bool factor_tc = true;
  // sweep-front shapes measured on the device on first use (else the cost model)
  bool tune = true;
  std::string dev_key;      // GPU identity for the tuner's cache (UUID, name, SM count)
  double tune_seconds = 0;  // time this context spent measuring front shapes
  int force_r = 0, force_cl = 0;   // one launch shape imposed on every front where it fits
  bool force_tc = false;           // ... with its line products on the tensor cores (complex64)
  // complex64: the tuner also measures each front with its line products on
  // the tensor cores (tcgen05, items of 8 or 16 slots); off by default: on
  // GB300 those launches were slower than the FMA matvec at every measured
  // shape and less accurate (FP32 accumulation in the tensor core over long k)
  bool sweep_tc = false;
  // captured applies launch each front once per shifted decomposition on
  // concurrent streams (side streams and fork/join events, created on first use)
  bool split_shifts = true;
  cudaStream_t side[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t side_ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // batches of at most this many right-hand sides run every stage-2 and
  // stage-3 sweep as its own chain of launches (one stream per sweep, created
  // on first use; events per stage-2 launch for the L-sweeps' waits)
  int lanes_max_rhs = 2;
  cudaStream_t lane_st[8] = {};
  cudaEvent_t lane_fork = nullptr;
  cudaEvent_t lane_join[8] = {};
  std::vector<cudaEvent_t> lane_ev;   // [sweep 0..3][t 0..N-1]
  // bounded-wait limit of the sweep and factorisation kernels, in SM clock cycles
  long long wait_cycles = 4000000000LL;   // ~2 s at 2 GHz
  // device address of the allocation-free solve's fixed scratch array on this
  // context's device (looked up once, with the device current, at creation)
  void* noalloc_base = nullptr;
  // optional per-front timing of one apply
  std::vector<cudaEvent_t>* front_events = nullptr;
  // CUDA graphs of the apply, one per batch size, replayed on the caller's
  // stream; a graph is captured against the pools of generation `gen` and
  // captured again when a pool it uses has been reallocated or released
  struct ApplyGraph {
    cudaGraphExec_t exec = nullptr;
    long long gen = -1;
    int kernels = 0;
  };
  std::map<int, ApplyGraph> graphs;
  bool use_graphs = true;
  int graph_failures = 0;   // captures that failed (the context then launches eagerly)
  long long pool_gen = 0;
  cudaStream_t cap_stream = nullptr;
  DevBuf d_ref;   // the captured applies' address table: input, output
  void drop_graphs() {
    for (auto& kv : graphs)
      if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    graphs.clear();
    ++pool_gen;
  }
  ~lsw_ctx() {
    drop_graphs();
    if (cap_stream) cudaStreamDestroy(cap_stream);
    for (auto& q : side)
      if (q) cudaStreamDestroy(q);
    for (auto& e : side_ev)
      if (e) cudaEventDestroy(e);
    for (auto& q : lane_st)
      if (q) cudaStreamDestroy(q);
    for (auto& e : lane_join)
      if (e) cudaEventDestroy(e);
    for (auto& e : lane_ev)
      if (e) cudaEventDestroy(e);
    if (lane_fork) cudaEventDestroy(lane_fork);
  }
};

namespace {

const char* kStatusStr[] = {"LSW_OK", "LSW_ERR_INVALID_ARGUMENT", "LSW_ERR_CUDA", "LSW_ERR_OUT_OF_MEMORY",
                            "LSW_ERR_NOT_SET_UP", "LSW_ERR_NOT_FACTORIZED", "LSW_ERR_SINGULAR_BLOCK",
                            "LSW_ERR_NOT_CONVERGED", "LSW_ERR_UNSUPPORTED"};

lsw_status fail(lsw_ctx* c, lsw_status s, const std::string& msg) {
  if (c) c->err = msg;
  return s;
}
lsw_status cuda_fail(lsw_ctx* c, cudaError_t e, const char* where) {
  std::string msg = std::string(where) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return fail(c, LSW_ERR_OUT_OF_MEMORY, msg);
  return fail(c, LSW_ERR_CUDA, msg);
}
#define CK(call, where)                                     \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) return cuda_fail(ctx, _e, where); \
  } while (0)
// CK for a launcher that enqueues n kernels; counts them
#define KL(n, call, where)      \
  do {                          \
    CK(call, where);            \
    ctx->launches += (n);       \
  } while (0)

inline size_t csize(int prec) { return prec == LSW_PREC_C128 ? 16 : 8; }
inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

DevCell make_cell(int I, int J, int N, int m, int p, bool split) {
  DevCell c{};
  const DirGeom gx = dir_geom(J, N, m, p), gy = dir_geom(I, N, m, p);
  c.I = I; c.J = J;
  c.nx = gx.nd; c.ny = gy.nd;
  c.lox = gx.lo; c.loy = gy.lo;
  c.ldn = (gy.nd + 3) & ~3;
  // bf16-split factors: a column stride of 4 (mod 8) complex values keeps the
  // four columns of an mma A fragment in distinct shared-memory banks
  if (split) {
    c.ldn = gy.nd;
    while (c.ldn % 8 != 4) ++c.ldn;
  }
  for (int s = 0; s < 2; ++s) {
    for (int l = 0; l < 4; ++l) { c.lx[s][l] = gx.lines[s][l]; c.ly[s][l] = gy.lines[s][l]; }
    c.ownx[s][0] = gx.own[s][0]; c.ownx[s][1] = gx.own[s][1];
    c.owny[s][0] = gy.own[s][0]; c.owny[s][1] = gy.own[s][1];
  }
  return c;
}

void fill_info(const DevCell& c, lsw_cell_info* o) {
  o->I = c.I; o->J = c.J; o->nx = c.nx; o->ny = c.ny; o->lo_x = c.lox; o->lo_y = c.loy;
  for (int s = 0; s < 2; ++s) {
    for (int l = 0; l < 4; ++l) { o->lines_x[s][l] = c.lx[s][l]; o->lines_y[s][l] = c.ly[s][l]; }
    o->own_x[s][0] = c.ownx[s][0]; o->own_x[s][1] = c.ownx[s][1];
    o->own_y[s][0] = c.owny[s][0]; o->own_y[s][1] = c.owny[s][1];
  }
}

void push_profile(std::vector<double2>& v, const Profile1D& pr) {
  const size_t n = pr.lo_re.size();
  for (size_t i = 0; i < n; ++i) v.push_back(make_double2(pr.lo_re[i], pr.lo_im[i]));
  for (size_t i = 0; i < n; ++i) v.push_back(make_double2(pr.hi_re[i], pr.hi_im[i]));
  for (size_t i = 0; i < n; ++i) v.push_back(make_double2(pr.dg_re[i], pr.dg_im[i]));
}

size_t device_bytes(const lsw_ctx* c) {
  size_t b = c->d_cells.bytes + c->d_prof.bytes + c->d_gprof.bytes + c->d_m.bytes + c->d_fac.bytes +
             c->d_work.bytes + c->d_status.bytes + c->d_traces.bytes + c->d_outs.bytes + c->d_scratch.bytes +
             c->k_basis.bytes + c->k_zbasis.bytes + c->k_tmp.bytes + c->k_tmp2.bytes + c->k_r.bytes +
             c->k_part.bytes + c->k_small.bytes + c->k_small2.bytes + c->k_nrm.bytes + c->ls_items.bytes +
             c->ls_slots.bytes + c->ls_scratch.bytes + c->h_b.bytes + c->h_x.bytes + c->d_ref.bytes +
             c->k_ls.bytes;
  for (auto& kv : c->sched_bufs)
    for (int i = 0; i < 3; ++i) b += kv.second[i].bytes;
  return b;
}

// CTAs per half for a single-cell solve: `cl`, or the next larger size whose
// launch fits in shared memory
int fitting_cluster(const lsw_ctx* ctx, int slots, int cl) {
  const int mask = front_fit_mask(ctx->prec == LSW_PREC_C128, ctx->prec == LSW_PREC_SPLIT, ctx->max_ny,
                                  ctx->max_nx, slots);
  for (int c = cl; c <= 4; c *= 2)
    if (mask & (1 << c)) return c;
  return cl;   // nothing fits: the launch reports it
}

FrontPlan base_plan(const lsw_ctx* ctx) {
  const bool dbl = ctx->prec == LSW_PREC_C128;
  FrontPlan plan;
  plan.cluster_cap = std::max(1, std::min(4, ctx->max_cluster / 2));
  plan.rmax = front_rmax(dbl);
  plan.csize = dbl ? 16 : 8;
  if (dbl) { plan.col_cost = 40.0; plan.col_slot_cost = 20.0; }
  if (ctx->prec == LSW_PREC_SPLIT) {
    // tensor-core matvec: the per-column cost hardly grows with the slots
    plan.line_overhead = 2200.0; plan.slot_cost = 0.0; plan.col_cost = 40.0; plan.col_slot_cost = 3.0;
  }
  for (int cl = 1; cl <= 4; cl *= 2) plan.max_clusters[cl] = front_max_clusters(dbl, 2 * cl);
  for (int r = 1; r <= 16; ++r)
    plan.fit_mask[r] = front_fit_mask(dbl, ctx->prec == LSW_PREC_SPLIT, ctx->max_ny, ctx->max_nx, r);
  if (plan.max_clusters[1] <= 0) plan.max_clusters[1] = ctx->nsm / 2;
  plan.tc_scratch = ctx->prec == LSW_PREC_C64 && (ctx->sweep_tc || ctx->force_tc);
  return plan;
}

// A schedule's descriptors on the device (three buffers: items, slots, groups).
lsw_status upload_schedule(lsw_ctx* ctx, Schedule* sc, const std::vector<DevItem>& items,
                           const std::vector<DevSlot>& slots, const std::vector<DevGroup>& groups, DevBuf* bufs) {
  CK(bufs[0].ensure(std::max<size_t>(1, items.size()) * sizeof(DevItem)), "cudaMalloc(items)");
  CK(bufs[1].ensure(std::max<size_t>(1, slots.size()) * sizeof(DevSlot)), "cudaMalloc(slots)");
  CK(bufs[2].ensure(std::max<size_t>(1, groups.size()) * sizeof(DevGroup)), "cudaMalloc(groups)");
  CK(cudaMemcpy(bufs[0].p, items.data(), items.size() * sizeof(DevItem), cudaMemcpyHostToDevice), "H2D items");
  CK(cudaMemcpy(bufs[1].p, slots.data(), slots.size() * sizeof(DevSlot), cudaMemcpyHostToDevice), "H2D slots");
  CK(cudaMemcpy(bufs[2].p, groups.data(), groups.size() * sizeof(DevGroup), cudaMemcpyHostToDevice), "H2D groups");
  sc->d_items = bufs[0].as<DevItem>();
  sc->d_slots = bufs[1].as<DevSlot>();
  sc->d_groups = bufs[2].as<DevGroup>();
  sc->scratch_elems = 0;
  for (auto& f : sc->fronts) sc->scratch_elems = std::max(sc->scratch_elems, f.scratch_elems);
  return LSW_OK;
}

// the trace, output and scratch pools of a batch of nrhs right-hand sides
lsw_status ensure_pools(lsw_ctx* ctx, int nrhs, long long scratch_elems, int planes) {
  const size_t cs = csize(ctx->prec);
  CK(ctx->d_traces.ensure((size_t)nrhs * 4 * ctx->ncell * 24 * ctx->LP * cs), "cudaMalloc(traces)");
  CK(ctx->d_outs.ensure((size_t)nrhs * planes * 4 * ctx->n2 * cs), "cudaMalloc(outs)");
  CK(ctx->d_scratch.ensure(std::max<size_t>(1, (size_t)scratch_elems * cs)), "cudaMalloc(scratch)");
  return LSW_OK;
}

lsw_status launch_front_of(lsw_ctx* ctx, const Schedule* sc, size_t fi, cudaStream_t st, int i0 = 0, int i1 = -1);
lsw_status enqueue_apply(lsw_ctx* ctx, Schedule* sc, int nrhs, cudaStream_t st, int* kernels,
                         bool split_shifts = false);
lsw_status check_kernel_err(lsw_ctx* ctx, cudaStream_t st);

// ---- sweep-front autotuner ----
// On the first apply of a batch size the shape of every front -- slots per
// item (4, 8, 16), CTAs per half chain (1, 2, 4) and, for complex64, line
// products on the CUDA cores or the tensor cores -- is measured on the
// device: each candidate shape is imposed on every front it fits, each front
// whose launch is new is run twice and timed the second time with CUDA events
// (the kernels' work does not depend on the values, so a zero vector serves),
// and every front keeps its fastest shape.  The choices are kept per GPU and
// problem shape (precision, cells, cell size, PML, batch size) for the
// process, and in the file named by LSW_TUNE_CACHE when it is set.
struct TuneEntry {
  std::vector<int> r, cl, tc;
  std::vector<float> ms;
};

// whether the tuner measures tensor-core line products, and whether a front
// of `max_slots` slots per item on clusters of 2 cl CTAs can run them
bool tc_candidates(const lsw_ctx* ctx) { return ctx->prec == LSW_PREC_C64 && ctx->sweep_tc; }
bool tc_fits(const lsw_ctx* ctx, int max_slots, int cl) {
  if (ctx->prec != LSW_PREC_C64 || max_slots < 1 || max_slots > 16) return false;
  return (front_fit_mask(false, false, ctx->max_ny, ctx->max_nx, front_tc_slots(max_slots), true) >> cl) & 1;
}
std::mutex g_tune_mu;
std::map<std::string, TuneEntry> g_tune_cache;
bool g_tune_file_read = false;

std::string tune_key(const lsw_ctx* ctx, int nrhs) {
  char b[160];
  std::snprintf(b, sizeof(b), "|prec%d|N%d|m%d|p%d|rhs%d|cl%d|tc%d", ctx->prec, ctx->N, ctx->m, ctx->p, nrhs,
                ctx->max_cluster, (int)tc_candidates(ctx));
  return ctx->dev_key + b;
}

void tune_file_read() {
  if (g_tune_file_read) return;
  g_tune_file_read = true;
  const char* path = std::getenv("LSW_TUNE_CACHE");
  if (!path || !*path) return;
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  char line[65536];
  while (std::fgets(line, sizeof(line), f)) {
    char* save = nullptr;
    char* tok = strtok_r(line, " \n", &save);
    if (!tok) continue;
    std::string key = tok;
    TuneEntry e;
    while ((tok = strtok_r(nullptr, " \n", &save))) {
      int r = 0, cl = 0;
      float ms = -1.f;
      if (std::sscanf(tok, "%d,%d,%f", &r, &cl, &ms) != 3) { e.r.clear(); break; }
      // slots per item, + 100 for tensor-core line products
      e.r.push_back(r % 100); e.cl.push_back(cl); e.ms.push_back(ms); e.tc.push_back(r >= 100 ? 1 : 0);
    }
    if (!e.r.empty()) g_tune_cache[key] = e;
  }
  std::fclose(f);
}

void tune_file_append(const std::string& key, const TuneEntry& e) {
  const char* path = std::getenv("LSW_TUNE_CACHE");
  if (!path || !*path) return;
  FILE* f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f, "%s", key.c_str());
  for (size_t i = 0; i < e.r.size(); ++i)
    std::fprintf(f, " %d,%d,%.9g", e.r[i] + (i < e.tc.size() && e.tc[i] ? 100 : 0), e.cl[i], e.ms[i]);
  std::fprintf(f, "\n");
  std::fclose(f);
}

lsw_status tune_fronts(lsw_ctx* ctx, int nrhs, const FrontPlan& plan, cudaStream_t st, TuneEntry* out) {
  const auto t_start = std::chrono::steady_clock::now();
  DevBuf tx, bufs[3];
  CK(tx.ensure((size_t)nrhs * ctx->n2 * sizeof(double2)), "cudaMalloc(tuning vector)");
  CK(cudaMemsetAsync(tx.p, 0, tx.bytes, st), "memset tuning vector");
  CK(ctx->d_ref.ensure(2 * sizeof(void*)), "cudaMalloc(address table)");
  KL(1, launch_set_refs(reinterpret_cast<const void**>(ctx->d_ref.p), tx.p, tx.p, st), "address table");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK(cudaEventCreate(&e0), "cudaEventCreate");
  CK(cudaEventCreate(&e1), "cudaEventCreate");
  // per front: (items, max slots, cluster, tensor cores) -> ms
  std::vector<std::map<std::tuple<int, int, int, int>, float>> seen;
  lsw_status s = LSW_OK;
  for (int r : {4, 8, 16}) {
    if (r > plan.rmax) continue;
    for (int cl = 1; cl <= plan.cluster_cap && s == LSW_OK; cl *= 2) {
      if (cl > 1 && plan.max_clusters[cl] <= 0) continue;
      FrontPlan p = plan;
      p.forced_r.assign(16 * (size_t)ctx->N + 16, r);
      p.forced_cl.assign(16 * (size_t)ctx->N + 16, cl);
      Schedule sc;
      std::vector<DevItem> items; std::vector<DevSlot> slots; std::vector<DevGroup> groups;
      try {
        build_schedule(ctx->cells, ctx->N, nrhs, p, ctx->LP, sc.fronts, items, slots, groups, ctx->n2);
      } catch (const std::exception&) {
        continue;
      }
      if ((s = upload_schedule(ctx, &sc, items, slots, groups, bufs)) != LSW_OK) break;
      if ((s = ensure_pools(ctx, nrhs, sc.scratch_elems, 1)) != LSW_OK) break;
      if (out->r.empty()) {
        out->r.assign(sc.fronts.size(), 0);
        out->cl.assign(sc.fronts.size(), 0);
        out->tc.assign(sc.fronts.size(), 0);
        out->ms.assign(sc.fronts.size(), 1e30f);
        seen.assign(sc.fronts.size(), {});
      }
      for (size_t fi = 0; fi < sc.fronts.size() && s == LSW_OK; ++fi) {
        for (int tc = 0; tc < 2 && s == LSW_OK; ++tc) {
          Front& f = sc.fronts[fi];
          if (f.item_count <= 0 || f.slots_cap != r || f.cluster != cl) continue;   // shape did not fit here
          if (tc && !(tc_candidates(ctx) && tc_fits(ctx, f.max_slots, cl))) continue;
          f.tc = tc != 0;
          const auto shape = std::make_tuple(f.item_count, f.max_slots, f.cluster, tc);
          float ms = 0.f;
          auto hit = seen[fi].find(shape);
          if (hit != seen[fi].end()) {
            ms = hit->second;
          } else {
            // timed once; a short launch (where a first launch's overheads
            // would show) is timed a second time and the smaller time kept
            for (int rep = 0; rep < 2 && s == LSW_OK; ++rep) {
              float t = 0.f;
              if (cudaEventRecord(e0, st) != cudaSuccess) { s = fail(ctx, LSW_ERR_CUDA, "event"); break; }
              if ((s = launch_front_of(ctx, &sc, fi, st)) != LSW_OK) break;
              if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                  cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) {
                s = fail(ctx, LSW_ERR_CUDA, "timing a sweep-front shape");
                break;
              }
              ms = rep == 0 ? t : std::min(ms, t);
              if (t > 2.0f) break;
            }
            if (s != LSW_OK) break;
            seen[fi][shape] = ms;
          }
          if (ms < out->ms[fi] * 0.99f) { out->ms[fi] = ms; out->r[fi] = r; out->cl[fi] = cl; out->tc[fi] = tc; }
        }
      }
      if (s == LSW_OK) s = check_kernel_err(ctx, st);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CK(cudaStreamSynchronize(st), "tuning sync");
  // the candidates' scratch may exceed the chosen schedule's: reallocated at its size
  ctx->d_scratch.release();
  ctx->tune_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  return s;
}

// Per-sweep schedules are tuned as a whole: their launches share the GPU with
// one another, which a launch timed alone does not show.  For each candidate
// of the cost model's concurrency (how many launches of its size a per-sweep
// launch is assumed to share the GPU with: 2, 4, 8) the schedule is built and
// one whole apply (eager launches on the sweep streams, a zero vector) is
// timed with CUDA events on the caller's stream after one untimed apply; the
// entry keeps each candidate's time (r = the candidate, ms = its apply).
lsw_status tune_lanes(lsw_ctx* ctx, int nrhs, const FrontPlan& plan, cudaStream_t st, TuneEntry* out) {
  const auto t_start = std::chrono::steady_clock::now();
  DevBuf tx, ty;
  CK(tx.ensure((size_t)nrhs * ctx->n2 * sizeof(double2)), "cudaMalloc(tuning vector)");
  CK(ty.ensure((size_t)nrhs * ctx->n2 * sizeof(double2)), "cudaMalloc(tuning vector)");
  CK(cudaMemsetAsync(tx.p, 0, tx.bytes, st), "memset tuning vector");
  CK(ctx->d_ref.ensure(2 * sizeof(void*)), "cudaMalloc(address table)");
  KL(1, launch_set_refs(reinterpret_cast<const void**>(ctx->d_ref.p), tx.p, ty.p, st), "address table");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK(cudaEventCreate(&e0), "cudaEventCreate");
  CK(cudaEventCreate(&e1), "cudaEventCreate");
  lsw_status s = LSW_OK;
  bool warm = false;
  for (int conc : {2, 4, 8}) {
    FrontPlan p = plan;
    p.lane_concurrency = conc;
    Schedule sc;
    sc.lanes = true;
    sc.nrhs = nrhs;
    DevBuf bufs[3];
    std::vector<DevItem> items; std::vector<DevSlot> slots; std::vector<DevGroup> groups;
    try {
      build_schedule(ctx->cells, ctx->N, nrhs, p, ctx->LP, sc.fronts, items, slots, groups, ctx->n2);
    } catch (const std::exception&) {
      continue;
    }
    if ((s = upload_schedule(ctx, &sc, items, slots, groups, bufs)) != LSW_OK) break;
    if ((s = ensure_pools(ctx, nrhs, sc.scratch_elems, kLanePlanes)) != LSW_OK) break;
    float ms = 0.f;
    for (int rep = warm ? 1 : 0; rep < 2 && s == LSW_OK; ++rep) {
      int k = 0;
      if (cudaEventRecord(e0, st) != cudaSuccess) { s = fail(ctx, LSW_ERR_CUDA, "event"); break; }
      if ((s = enqueue_apply(ctx, &sc, nrhs, st, &k)) != LSW_OK) break;
      ctx->launches += k;
      if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
        s = fail(ctx, LSW_ERR_CUDA, "timing a per-sweep schedule");
    }
    warm = true;
    if (s == LSW_OK) s = check_kernel_err(ctx, st);
    if (s != LSW_OK) break;
    out->r.push_back(conc); out->cl.push_back(0); out->tc.push_back(0); out->ms.push_back(ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CK(cudaStreamSynchronize(st), "tuning sync");
  ctx->d_scratch.release();
  ctx->tune_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  return s;
}

lsw_status ensure_batch(lsw_ctx* ctx, int nrhs, Schedule** out, cudaStream_t st) {
  auto it = ctx->sched.find(nrhs);
  void* const before[3] = {ctx->d_traces.p, ctx->d_outs.p, ctx->d_scratch.p};
  if (it == ctx->sched.end()) {
    std::unique_ptr<Schedule> sc(new Schedule);
    std::vector<DevItem> items; std::vector<DevSlot> slots; std::vector<DevGroup> groups;
    FrontPlan plan;
    try {
      plan = base_plan(ctx);
    } catch (const std::exception& ex) {
      return fail(ctx, LSW_ERR_UNSUPPORTED, ex.what());
    }
    plan.lanes = nrhs <= ctx->lanes_max_rhs;
    TuneEntry tuned;
    if (ctx->force_r > 0) {
      plan.forced_r.assign(16 * (size_t)ctx->N + 16, ctx->force_r);
      plan.forced_cl.assign(16 * (size_t)ctx->N + 16, ctx->force_cl);
    } else if (ctx->tune && ctx->factorized && plan.lanes) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      tune_file_read();
      const std::string key = tune_key(ctx, nrhs) + "|lanes";
      auto hit = g_tune_cache.find(key);
      TuneEntry whole;
      if (hit != g_tune_cache.end()) {
        whole = hit->second;
      } else {
        lsw_status s = tune_lanes(ctx, nrhs, plan, st, &whole);
        if (s != LSW_OK) return s;
        if (!whole.r.empty()) {
          g_tune_cache[key] = whole;
          tune_file_append(key, whole);
        }
      }
      size_t best = 0;
      for (size_t i = 1; i < whole.ms.size(); ++i)
        if (whole.ms[i] < whole.ms[best]) best = i;
      if (!whole.r.empty()) plan.lane_concurrency = whole.r[best];
    } else if (ctx->tune && ctx->factorized) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      tune_file_read();
      const std::string key = tune_key(ctx, nrhs);
      auto hit = g_tune_cache.find(key);
      if (hit != g_tune_cache.end()) {
        tuned = hit->second;
      } else {
        lsw_status s = tune_fronts(ctx, nrhs, plan, st, &tuned);
        if (s != LSW_OK) return s;
        g_tune_cache[key] = tuned;
        tune_file_append(key, tuned);
      }
      plan.forced_r = tuned.r;
      plan.forced_cl = tuned.cl;
    }
    try {
      build_schedule(ctx->cells, ctx->N, nrhs, plan, ctx->LP, sc->fronts, items, slots, groups, ctx->n2);
    } catch (const std::exception& ex) {
      return fail(ctx, LSW_ERR_UNSUPPORTED, ex.what());
    }
    for (size_t fi = 0; fi < sc->fronts.size() && fi < tuned.r.size(); ++fi) {
      Front& f = sc->fronts[fi];
      if (f.slots_cap == tuned.r[fi] && f.cluster == tuned.cl[fi]) {
        f.tuned_ms = tuned.ms[fi];
        f.tc = fi < tuned.tc.size() && tuned.tc[fi] && tc_fits(ctx, f.max_slots, f.cluster);
      }
    }
    if (ctx->force_r > 0 && ctx->force_tc)
      for (Front& f : sc->fronts) f.tc = f.item_count > 0 && tc_fits(ctx, f.max_slots, f.cluster);
    sc->nrhs = nrhs;
    sc->lanes = plan.lanes;
    std::unique_ptr<DevBuf[]> bufs(new DevBuf[3]);
    lsw_status s = upload_schedule(ctx, sc.get(), items, slots, groups, bufs.get());
    if (s != LSW_OK) return s;
    ctx->sched_bufs[nrhs] = std::move(bufs);
    it = ctx->sched.emplace(nrhs, std::move(sc)).first;
  }
  Schedule* sc = it->second.get();
  lsw_status s = ensure_pools(ctx, nrhs, sc->scratch_elems, sc->lanes ? kLanePlanes : 1);
  if (s != LSW_OK) return s;
  if (before[0] != ctx->d_traces.p || before[1] != ctx->d_outs.p || before[2] != ctx->d_scratch.p) {
    // the captured applies point at the old pools
    for (auto& kv : ctx->graphs)
      if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
    ctx->graphs.clear();
    ++ctx->pool_gen;
  }
  *out = sc;
  return LSW_OK;
}

// Items [i0, i1) (all for i1 < 0) of sweep front fi of schedule sc on stream
// st.  The input and output addresses are read from ctx->d_ref.
lsw_status launch_front_of(lsw_ctx* ctx, const Schedule* sc, size_t fi, cudaStream_t st, int i0, int i1) {
  FrontArgs a{};
  a.cells = ctx->d_cells.as<DevCell>();
  a.slots = sc->d_slots;
  a.groups = sc->d_groups;
  a.fac = ctx->d_fac.p;
  a.prof = ctx->d_prof.as<double2>();
  a.traces = ctx->d_traces.p;
  a.outs = ctx->d_outs.p;
  a.scratch = ctx->d_scratch.p;
  a.x_in = nullptr;
  a.x_ref = reinterpret_cast<const double2* const*>(ctx->d_ref.p);
  a.x_stride = ctx->n2;
  a.n_dof = ctx->n_dof; a.N = ctx->N; a.m = ctx->m; a.p = ctx->p;
  a.err = ctx->d_status.as<int>() + 1;
  a.wait_cycles = ctx->wait_cycles;
  a.split = ctx->prec == LSW_PREC_SPLIT ? 1 : 0;
  const Front& f = sc->fronts[fi];
  if (i1 < 0) i1 = f.item_count;
  if (i1 <= i0) return LSW_OK;
  a.items = sc->d_items + f.item_begin + i0;
  a.item_count = i1 - i0;
  a.max_slots = f.max_slots;
  a.cluster = f.cluster;
  a.tc = f.tc ? 1 : 0;
  cudaError_t e = ctx->prec != LSW_PREC_C128 ? launch_front<float>(a, ctx->max_ny, ctx->max_nx, st)
                                             : launch_front<double>(a, ctx->max_ny, ctx->max_nx, st);
  CK(e, "front kernel");
  return LSW_OK;
}

// Per-sweep launches (sc->lanes): stage 1 on st; then each stage-2 sweep on
// its own stream, every launch recording an event, and each L-sweep on its own
// stream, its step dd waiting first for the events of its two producing
// stage-2 sweeps at front min(dd + 1, N - 1) (see kLanePlanes); every stream
// joins st before the sum.  With `streams` false (per-front timing) the
// launches run on st in schedule order, a topological order of the same
// dependencies.  Either way each output value and trace line sees the same
// writes in the same order, so the results are identical.
lsw_status enqueue_lanes(lsw_ctx* ctx, Schedule* sc, cudaStream_t st, int* k, bool streams) {
  lsw_status s;
  if (!streams) {
    for (size_t fi = 0; fi < sc->fronts.size(); ++fi) {
      if (ctx->front_events) CK(cudaEventRecord((*ctx->front_events)[2 * fi], st), "event");
      if ((s = launch_front_of(ctx, sc, fi, st)) != LSW_OK) return s;
      if (ctx->front_events) CK(cudaEventRecord((*ctx->front_events)[2 * fi + 1], st), "event");
      *k += sc->fronts[fi].item_count > 0 ? 1 : 0;
    }
    return LSW_OK;
  }
  const int N = ctx->N;
  for (int l = 0; l < 8; ++l) {
    if (!ctx->lane_st[l]) CK(cudaStreamCreateWithFlags(&ctx->lane_st[l], cudaStreamNonBlocking), "sweep stream");
    if (!ctx->lane_join[l]) CK(cudaEventCreateWithFlags(&ctx->lane_join[l], cudaEventDisableTiming), "sweep event");
  }
  if (!ctx->lane_fork) CK(cudaEventCreateWithFlags(&ctx->lane_fork, cudaEventDisableTiming), "sweep event");
  if ((int)ctx->lane_ev.size() != 4 * N) {
    for (auto& e : ctx->lane_ev)
      if (e) cudaEventDestroy(e);
    ctx->lane_ev.assign(4 * (size_t)N, nullptr);
    for (auto& e : ctx->lane_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "sweep event");
  }
  size_t fi = 0;
  for (; fi < sc->fronts.size() && sc->fronts[fi].lane < 0; ++fi) {   // stage 1
    if ((s = launch_front_of(ctx, sc, fi, st)) != LSW_OK) return s;
    *k += sc->fronts[fi].item_count > 0 ? 1 : 0;
  }
  CK(cudaEventRecord(ctx->lane_fork, st), "fork");
  for (int l = 0; l < 8; ++l) CK(cudaStreamWaitEvent(ctx->lane_st[l], ctx->lane_fork, 0), "fork wait");
  int waited[4] = {0, 0, 0, 0};   // per L-sweep: the stage-2 front it last waited for
  for (; fi < sc->fronts.size(); ++fi) {
    const Front& f = sc->fronts[fi];
    if (f.lane < 0) return fail(ctx, LSW_ERR_CUDA, "per-sweep schedule out of order");
    cudaStream_t q = ctx->lane_st[f.lane];
    if (f.stage == 3) {
      const int w = f.lane - 4, t = std::min(f.step + 1, N - 1);
      if (t > waited[w]) {
        CK(cudaStreamWaitEvent(q, ctx->lane_ev[(size_t)kLaneProducerLR[w] * N + t], 0), "sweep wait");
        CK(cudaStreamWaitEvent(q, ctx->lane_ev[(size_t)kLaneProducerUD[w] * N + t], 0), "sweep wait");
        waited[w] = t;
      }
    }
    if (f.item_count > 0) {
      if ((s = launch_front_of(ctx, sc, fi, q)) != LSW_OK) return s;
      ++*k;
    }
    if (f.stage == 2) CK(cudaEventRecord(ctx->lane_ev[(size_t)f.lane * N + f.step], q), "sweep event");
  }
  for (int l = 0; l < 8; ++l) {
    CK(cudaEventRecord(ctx->lane_join[l], ctx->lane_st[l]), "join");
    CK(cudaStreamWaitEvent(st, ctx->lane_join[l], 0), "join wait");
  }
  return LSW_OK;
}

// The launches of one apply on stream st: clear the trace and output pools,
// every sweep front, the sum of the four shifted outputs.  The input and
// output addresses are read from ctx->d_ref (set by the caller beforehand),
// so the sequence can be captured once and replayed for any vectors.
// Returns the number of kernels enqueued in *kernels.
// With `split_shifts` (the captured applies), a front whose items each belong
// to one shifted decomposition is launched once per shift, shift s on side
// stream s (shift 0 on st): the four decompositions never share data before
// their outputs are summed, so the launches of one shift's next front start
// while other shifts still run, and the ends of the fronts overlap instead of
// leaving SMs idle.  A mixed front joins every stream and runs alone.
// Per-sweep schedules (sc->lanes) run on the sweep streams of enqueue_lanes,
// captured or not (one stream when the fronts are timed one by one).
lsw_status enqueue_apply(lsw_ctx* ctx, Schedule* sc, int nrhs, cudaStream_t st, int* kernels,
                         bool split_shifts) {
  const size_t cs = csize(ctx->prec);
  const int planes = sc->lanes ? kLanePlanes : 1;
  CK(cudaMemsetAsync(ctx->d_traces.p, 0, (size_t)nrhs * 4 * ctx->ncell * 24 * ctx->LP * cs, st), "memset traces");
  CK(cudaMemsetAsync(ctx->d_outs.p, 0, (size_t)nrhs * planes * 4 * ctx->n2 * cs, st), "memset outs");
  int k = 0;
  if (sc->lanes) {
    lsw_status s = enqueue_lanes(ctx, sc, st, &k, ctx->front_events == nullptr);
    if (s != LSW_OK) return s;
  } else if (split_shifts) {
    for (int i = 0; i < 3; ++i)
      if (!ctx->side[i]) CK(cudaStreamCreateWithFlags(&ctx->side[i], cudaStreamNonBlocking), "side stream");
    for (int i = 0; i < 4; ++i)
      if (!ctx->side_ev[i]) CK(cudaEventCreateWithFlags(&ctx->side_ev[i], cudaEventDisableTiming), "side event");
    cudaStream_t ss[4] = {st, ctx->side[0], ctx->side[1], ctx->side[2]};
    bool forked = false;
    auto fork = [&]() -> lsw_status {
      CK(cudaEventRecord(ctx->side_ev[0], st), "fork");
      for (int i = 1; i < 4; ++i) CK(cudaStreamWaitEvent(ss[i], ctx->side_ev[0], 0), "fork wait");
      forked = true;
      return LSW_OK;
    };
    auto join = [&]() -> lsw_status {
      for (int i = 1; i < 4; ++i) {
        CK(cudaEventRecord(ctx->side_ev[i], ss[i]), "join");
        CK(cudaStreamWaitEvent(st, ctx->side_ev[i], 0), "join wait");
      }
      forked = false;
      return LSW_OK;
    };
    lsw_status s;
    for (size_t fi = 0; fi < sc->fronts.size(); ++fi) {
      const Front& f = sc->fronts[fi];
      if (f.item_count <= 0) continue;
      if (f.mixed) {
        if (forked && (s = join()) != LSW_OK) return s;
        if ((s = launch_front_of(ctx, sc, fi, st)) != LSW_OK) return s;
        ++k;
        continue;
      }
      if (!forked && (s = fork()) != LSW_OK) return s;
      for (int sh = 0; sh < 4; ++sh) {
        if (f.sh_begin[sh + 1] <= f.sh_begin[sh]) continue;
        if ((s = launch_front_of(ctx, sc, fi, ss[sh], f.sh_begin[sh], f.sh_begin[sh + 1])) != LSW_OK) return s;
        ++k;
      }
    }
    if (forked && (s = join()) != LSW_OK) return s;
  } else {
    for (size_t fi = 0; fi < sc->fronts.size(); ++fi) {
      if (ctx->front_events) CK(cudaEventRecord((*ctx->front_events)[2 * fi], st), "event");
      lsw_status s = launch_front_of(ctx, sc, fi, st);
      if (s != LSW_OK) return s;
      if (ctx->front_events) CK(cudaEventRecord((*ctx->front_events)[2 * fi + 1], st), "event");
      k += sc->fronts[fi].item_count > 0 ? 1 : 0;
    }
  }
  double2* const* yref = reinterpret_cast<double2* const*>(ctx->d_ref.p) + 1;
  cudaError_t e = ctx->prec != LSW_PREC_C128
                      ? launch_combine_ref<float>(ctx->d_outs.p, yref, nrhs, ctx->n2, planes, st)
                      : launch_combine_ref<double>(ctx->d_outs.p, yref, nrhs, ctx->n2, planes, st);
  CK(e, "combine kernel");
  *kernels = k + 1;
  return LSW_OK;
}

lsw_status precond_impl(lsw_ctx* ctx, const double2* x, double2* y, int nrhs, cudaStream_t st) {
  Schedule* sc = nullptr;
  lsw_status s = ensure_batch(ctx, nrhs, &sc, st);
  if (s != LSW_OK) return s;
  CK(ctx->d_ref.ensure(2 * sizeof(void*)), "cudaMalloc(address table)");
  KL(1, launch_set_refs(reinterpret_cast<const void**>(ctx->d_ref.p), x, y, st), "address table");
  int kernels = 0;
  if (!ctx->use_graphs || ctx->front_events) {
    s = enqueue_apply(ctx, sc, nrhs, st, &kernels);
    ctx->launches += kernels;
    return s;
  }
  lsw_ctx::ApplyGraph& g = ctx->graphs[nrhs];
  if (!g.exec || g.gen != ctx->pool_gen) {
    if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
    if (!ctx->cap_stream) CK(cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking), "capture stream");
    CK(cudaStreamBeginCapture(ctx->cap_stream, cudaStreamCaptureModeRelaxed), "begin capture");
    s = enqueue_apply(ctx, sc, nrhs, ctx->cap_stream, &kernels, ctx->split_shifts);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->cap_stream, &graph);
    cudaGraphExec_t exec = nullptr;
    cudaError_t ei = cudaErrorUnknown;
    if (s == LSW_OK && e == cudaSuccess && graph) ei = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
      // A capture can be invalidated by CUDA calls of other host threads (an
      // allocation or free, a synchronous copy) made while it runs.  The
      // context stops capturing and this and later applies launch their
      // kernels one by one, which give the same results.
      if (exec) cudaGraphExecDestroy(exec);
      cudaGetLastError();
      ctx->use_graphs = false;
      ctx->graph_failures += 1;
      ctx->graphs.erase(nrhs);
      s = enqueue_apply(ctx, sc, nrhs, st, &kernels);
      ctx->launches += kernels;
      return s;
    }
    g.exec = exec;
    g.gen = ctx->pool_gen;
    g.kernels = kernels;
  }
  CK(cudaGraphLaunch(g.exec, st), "graph launch");
  ctx->launches += g.kernels;
  return LSW_OK;
}

lsw_status apply_A_impl(lsw_ctx* ctx, const double2* x, double2* y, int nrhs, cudaStream_t st) {
  CK(launch_apply_A(x, y, nrhs, ctx->n_dof, ctx->d_gprof.as<double2>(), ctx->d_m.as<double>(),
                    ctx->omega * ctx->omega, st), "apply_A kernel");
  ctx->launches += 1;
  return LSW_OK;
}

// Reads the sweep kernels' error word (synchronises the stream).  A set word
// is cleared once it is reported, so an error raised by an asynchronous call
// (lsw_apply_precond) is reported by the next call that checks, and later
// calls that succeed report success.
lsw_status check_kernel_err(lsw_ctx* ctx, cudaStream_t st) {
  int e = 0;
  CK(cudaMemcpyAsync(&e, ctx->d_status.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H err");
  CK(cudaStreamSynchronize(st), "sync");
  if (e) CK(cudaMemsetAsync(ctx->d_status.as<int>() + 1, 0, sizeof(int), st), "clear err");
  if (e & 4) return fail(ctx, LSW_ERR_CUDA, "sweep-front launch did not form the requested clusters (results invalid)");
  if (e) return fail(ctx, LSW_ERR_CUDA, "a sweep-front kernel gave up on a bounded wait (results invalid)");
  return LSW_OK;
}

// complex Gaussian elimination with partial pivoting, square system (host)
std::vector<cplx> dense_solve(std::vector<cplx> A, std::vector<cplx> b, int n) {
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  for (int k = 0; k < n; ++k) {
    int pr = k; double best = std::abs(A[k * n + k]);
    for (int i = k + 1; i < n; ++i) if (std::abs(A[i * n + k]) > best) { best = std::abs(A[i * n + k]); pr = i; }
    if (pr != k) { for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[pr * n + j]); std::swap(b[k], b[pr]); }
    if (A[k * n + k] == cplx(0, 0)) continue;
    for (int i = k + 1; i < n; ++i) {
      const cplx f = A[i * n + k] / A[k * n + k];
      if (f == cplx(0, 0)) continue;
      for (int j = k; j < n; ++j) A[i * n + j] -= f * A[k * n + j];
      b[i] -= f * b[k];
    }
  }
  std::vector<cplx> x(n);
  for (int i = n - 1; i >= 0; --i) {
    cplx s = b[i];
    for (int j = i + 1; j < n; ++j) s -= A[i * n + j] * x[j];
    x[i] = A[i * n + i] == cplx(0, 0) ? cplx(0, 0) : s / A[i * n + i];
  }
  return x;
}

// givens_rotation (GlobalIterativeSolverGMRES.cpp:333-348), kept as written
void givens_ref(cplx v1, cplx v2, cplx& cs, cplx& sn) {
  if (v1 == cplx(0.0, 0.0)) { cs = 0.0; sn = 1.0; return; }
  const cplx t = std::pow(std::pow(v1, 2.0) + std::pow(v2, 2.0), 0.5);
  cs = std::abs(v1) / t;
  sn = cs * v2 / v1;
}

struct Krylov {
  lsw_ctx* ctx;
  cudaStream_t st;
  int nv;
  long long n2;
  lsw_status st_ = LSW_OK;
};

}  // namespace

// ---------------------------------------------------------------------------
// Allocation-free cell solve (lsw_local_solve_noalloc).  Its scratch -- the
// item/slot descriptors and the forward-substitution storage -- lives in this
// fixed file-scope device array instead of memory obtained from cudaMalloc.
// Every GPU that loads the library holds the array until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;   // 8 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// writes the descriptors of `nrhs` full-cell right-hand sides of one cell:
// items of at most rmax slots, each with its share of the forward storage
__global__ void k_noalloc_desc(DevItem* items, DevSlot* slots, int cell, int nrhs, int rmax,
                               long long per_item_stride_elems) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrhs) return;
  const int item = r / rmax;
  DevSlot s{};
  s.kind = SK_CELLVEC;
  s.rhs = r;
  s.in_lr0 = s.in_lr1 = s.in_ud0 = s.in_ud1 = -1;
  for (int i = 0; i < 4; ++i) { s.lr_out[i] = -1; s.ud_out[i] = -1; s.lr_line[i] = -1; s.ud_line[i] = -1; }
  slots[r] = s;
  if (r % rmax == 0) {
    DevItem it{};
    it.cell = cell;
    it.slot_begin = r;
    it.slot_count = min(rmax, nrhs - r);
    it.group_begin = 0;
    it.group_count = 0;
    it.scratch_off = (long long)item * per_item_stride_elems;
    items[item] = it;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

const char* lsw_status_string(lsw_status s) {
  const int i = (int)s;
  if (i < 0 || i > 8) return "LSW_UNKNOWN";
  return kStatusStr[i];
}

const char* lsw_ctx_last_error(const lsw_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

lsw_status lsw_ctx_create(lsw_ctx** out, int device) {
  if (!out) return LSW_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return LSW_ERR_CUDA;
  if (device < 0 || device >= n) return LSW_ERR_INVALID_ARGUMENT;
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return LSW_ERR_CUDA;
  lsw_ctx* c = new lsw_ctx;
  c->device = device;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && nsm > 0) c->nsm = nsm;
  // LSW_MAX_CLUSTER caps the CTAs per cell solve (2, 4 or 8; default 8: the two
  // halves of a cell solve always take one CTA each at least)
  if (const char* ev = std::getenv("LSW_MAX_CLUSTER")) {
    const int v = std::atoi(ev);
    if (v >= 2 && v <= 8) c->max_cluster = v;
  }
  // LSW_KRYLOV_BATCH caps the right-hand sides iterated together by lsw_gmres
  if (const char* ev = std::getenv("LSW_KRYLOV_BATCH")) c->krylov_batch = std::max(0, std::atoi(ev));
  // LSW_FACTOR_LOOKAHEAD=0 factors each panel after the whole previous update
  if (const char* ev = std::getenv("LSW_FACTOR_LOOKAHEAD")) c->factor_lookahead = std::atoi(ev) != 0;
  // LSW_GRAPHS=0 launches every apply's kernels one by one instead of replaying a CUDA graph
  if (const char* ev = std::getenv("LSW_GRAPHS")) c->use_graphs = std::atoi(ev) != 0;
  // LSW_FACTOR_TC=0 runs the complex64 / split factorisation on the CUDA cores
  if (const char* ev = std::getenv("LSW_FACTOR_TC")) c->factor_tc = std::atoi(ev) != 0;
  // LSW_SHIFT_STREAMS=0 keeps each captured front one launch on one stream
  if (const char* ev = std::getenv("LSW_SHIFT_STREAMS")) c->split_shifts = std::atoi(ev) != 0;
  // LSW_SWEEP_LANES=<n>: per-sweep launches for batches of at most n right-hand sides (0: never)
  if (const char* ev = std::getenv("LSW_SWEEP_LANES")) c->lanes_max_rhs = std::max(0, std::atoi(ev));
  // LSW_TUNE=0 leaves every sweep-front shape to the cost model
  if (const char* ev = std::getenv("LSW_TUNE")) c->tune = std::atoi(ev) != 0;
  // LSW_SWEEP_TC=1 adds tensor-core line products to the complex64 tuning candidates
  if (const char* ev = std::getenv("LSW_SWEEP_TC")) c->sweep_tc = std::atoi(ev) != 0;
  // LSW_FRONT_SHAPE=RxC imposes R slots per item (4, 8, 16) and C CTAs per half
  // chain (1, 2, 4) on every sweep front where that shape fits (no tuning)
  if (const char* ev = std::getenv("LSW_FRONT_SHAPE")) {
    // (RxCt: with the line products on the tensor cores where they fit, complex64)
    int r = 0, cl = 0;
    char t = 0;
    const int got = std::sscanf(ev, "%dx%d%c", &r, &cl, &t);
    if (got >= 2 && (r == 4 || r == 8 || r == 16) && (cl == 1 || cl == 2 || cl == 4)) {
      c->force_r = r;
      c->force_cl = cl;
      c->force_tc = got == 3 && t == 't';
    }
  }
  {
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) {
      char b[64];
      std::string k;
      for (int i = 0; i < 16; ++i) {
        std::snprintf(b, sizeof(b), "%02x", (unsigned char)prop.uuid.bytes[i]);
        k += b;
      }
      std::string name = prop.name;
      for (char& ch : name)
        if (ch == ' ' || ch == '|') ch = '_';
      std::snprintf(b, sizeof(b), "|sm%d|", prop.multiProcessorCount);
      c->dev_key = k + b + name;
    } else {
      c->dev_key = "unknown-gpu";
    }
  }
  // the host-side name of the allocation-free solve's scratch array is not a
  // device address: look the address up on this device (current since the
  // cudaSetDevice above) and keep it with the context
  e = cudaGetSymbolAddress(&c->noalloc_base, g_noalloc_scratch);
  if (e != cudaSuccess || !c->noalloc_base) {
    delete c;
    return LSW_ERR_CUDA;
  }
  *out = c;
  return LSW_OK;
}

lsw_status lsw_ctx_set_graphs(lsw_ctx* ctx, int enable) {
  if (!ctx) return LSW_ERR_INVALID_ARGUMENT;
  ctx->use_graphs = enable != 0;
  return LSW_OK;
}

lsw_status lsw_ctx_set_tuning(lsw_ctx* ctx, int enable) {
  if (!ctx) return LSW_ERR_INVALID_ARGUMENT;
  if (ctx->tune != (enable != 0)) {
    // the schedules built under the other setting are rebuilt on next use
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(cudaDeviceSynchronize(), "sync");
    ctx->drop_graphs();
    ctx->sched.clear();
    ctx->sched_bufs.clear();
  }
  ctx->tune = enable != 0;
  return LSW_OK;
}

lsw_status lsw_ctx_set_sweep_lanes(lsw_ctx* ctx, int max_rhs) {
  if (!ctx || max_rhs < 0) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "bad arguments to lsw_ctx_set_sweep_lanes");
  if (ctx->lanes_max_rhs != max_rhs) {
    // the schedules built under the other setting are rebuilt on next use
    CK(cudaSetDevice(ctx->device), "cudaSetDevice");
    CK(cudaDeviceSynchronize(), "sync");
    ctx->drop_graphs();
    ctx->sched.clear();
    ctx->sched_bufs.clear();
  }
  ctx->lanes_max_rhs = max_rhs;
  return LSW_OK;
}

lsw_status lsw_front_shapes(lsw_ctx* ctx, int nrhs, lsw_front_shape* out, int capacity, int* n_fronts,
                            double* tune_seconds, void* stream) {
  if (!ctx || nrhs < 1 || !n_fronts || capacity < 0 || (capacity > 0 && !out))
    return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "bad arguments to lsw_front_shapes");
  if (!ctx->is_setup) return fail(ctx, LSW_ERR_NOT_SET_UP, "lsw_problem_setup first");
  if (!ctx->factorized) return fail(ctx, LSW_ERR_NOT_FACTORIZED, "lsw_factorize first");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  Schedule* sc = nullptr;
  lsw_status s = ensure_batch(ctx, nrhs, &sc, S(stream));
  if (s != LSW_OK) return s;
  *n_fronts = (int)sc->fronts.size();
  for (int i = 0; i < capacity && i < (int)sc->fronts.size(); ++i) {
    const Front& f = sc->fronts[i];
    out[i].items = f.item_count;
    out[i].max_slots = f.max_slots;
    out[i].slots_cap = f.slots_cap;
    out[i].cluster = f.cluster;
    out[i].tuned_ms = f.tuned_ms;
    out[i].tensor_cores = f.tc ? 1 : 0;
  }
  if (tune_seconds) *tune_seconds = ctx->tune_seconds;
  return LSW_OK;
}

lsw_status lsw_ctx_set_wait_limit(lsw_ctx* ctx, double seconds) {
  if (!ctx) return LSW_ERR_INVALID_ARGUMENT;
  if (!(seconds > 0.0) || !(seconds <= 60.0))
    return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "wait limit must be in (0, 60] seconds");
  int khz = 0;
  if (cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, ctx->device) != cudaSuccess || khz <= 0) khz = 2070000;
  ctx->wait_cycles = std::max(1000LL, (long long)(seconds * 1e3 * (double)khz));
  return LSW_OK;
}

lsw_status lsw_selftest_bounded_wait(lsw_ctx* ctx, void* stream) {
  if (!ctx) return LSW_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  if (!ctx->d_status.p) CK(ctx->d_status.ensure(16), "cudaMalloc(status)");
  cudaStream_t st = S(stream);
  KL(1, launch_wait_probe(ctx->d_status.as<int>() + 1, ctx->wait_cycles, st), "wait probe");
  return check_kernel_err(ctx, st);
}

lsw_status lsw_ctx_destroy(lsw_ctx* ctx) {
  if (!ctx) return LSW_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  delete ctx;
  return LSW_OK;
}

lsw_status lsw_geometry_cell(const lsw_geom* g, int cell, lsw_cell_info* out) {
  std::string why;
  if (!out || !geom_valid(g, &why)) return LSW_ERR_INVALID_ARGUMENT;
  const int N = g->n_cells;
  if (cell < 0 || cell >= N * N) return LSW_ERR_INVALID_ARGUMENT;
  fill_info(make_cell(cell / N, cell % N, N, g->n_els_in_cell, g->pml, false), out);
  return LSW_OK;
}

lsw_status lsw_problem_setup(lsw_ctx* ctx, const lsw_geom* g, const double* m_grid, double omega, int precision) {
  if (!ctx) return LSW_ERR_INVALID_ARGUMENT;
  std::string why;
  if (!geom_valid(g, &why)) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, why);
  if (!m_grid) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "m_grid is NULL");
  if (!(omega > 1.0) || !std::isfinite(omega))
    return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "omega must be > 1 (PML absorption C = ln omega must be positive)");
  if (precision != LSW_PREC_C128 && precision != LSW_PREC_C64 && precision != LSW_PREC_SPLIT)
    return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "unknown precision");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  // drop everything of a previous problem
  ctx->drop_graphs();
  ctx->sched.clear(); ctx->sched_bufs.clear();
  ctx->is_setup = false; ctx->factorized = false;
  ctx->geom = *g;
  ctx->N = g->n_cells; ctx->m = g->n_els_in_cell; ctx->p = g->pml; ctx->h = g->h;
  ctx->n_g = ctx->N * ctx->m + ctx->N - 1;
  ctx->n_dof = ctx->n_g + 2 * ctx->p - 1;
  ctx->n2 = (long long)ctx->n_dof * ctx->n_dof;
  ctx->omega = omega;
  ctx->C = std::log(omega);   // Input.cpp:836
  ctx->prec = precision;
  ctx->ncell = ctx->N * ctx->N;
  ctx->cells.clear();
  std::vector<double2> prof;
  long long fac_off = 0;
  ctx->max_nx = ctx->max_ny = 0;
  for (int I = 0; I < ctx->N; ++I)
    for (int J = 0; J < ctx->N; ++J) {
      DevCell c = make_cell(I, J, ctx->N, ctx->m, ctx->p, precision == LSW_PREC_SPLIT);
      c.fac_off = fac_off;
      fac_off += (long long)c.nx * c.ny * c.ldn;
      c.prof_off = (long long)prof.size();
      const DirGeom gx = dir_geom(J, ctx->N, ctx->m, ctx->p), gy = dir_geom(I, ctx->N, ctx->m, ctx->p);
      push_profile(prof, make_profile(gx.nel, ctx->p, ctx->h, ctx->C));
      push_profile(prof, make_profile(gy.nel, ctx->p, ctx->h, ctx->C));
      ctx->max_nx = std::max(ctx->max_nx, c.nx);
      ctx->max_ny = std::max(ctx->max_ny, c.ny);
      ctx->cells.push_back(c);
    }
  ctx->LP = ((std::max(ctx->max_nx, ctx->max_ny) + 7) / 8) * 8;
  std::vector<double2> gprof;
  push_profile(gprof, make_profile(ctx->n_g, ctx->p, ctx->h, ctx->C));
  const size_t cs = csize(precision);
  CK(ctx->d_cells.ensure(ctx->cells.size() * sizeof(DevCell)), "cudaMalloc(cells)");
  CK(ctx->d_prof.ensure(prof.size() * sizeof(double2)), "cudaMalloc(prof)");
  CK(ctx->d_gprof.ensure(gprof.size() * sizeof(double2)), "cudaMalloc(gprof)");
  CK(ctx->d_m.ensure((size_t)ctx->n2 * sizeof(double)), "cudaMalloc(m)");
  CK(ctx->d_fac.ensure((size_t)fac_off * cs), "cudaMalloc(factors)");
  CK(ctx->d_status.ensure(16), "cudaMalloc(status)");
  if (precision == LSW_PREC_SPLIT) {
    // the previous FP32 Schur-complement inverse of each cell's two half
    // chains, for the recurrences and the middle line
    CK(ctx->d_work.ensure((size_t)2 * ctx->ncell * ctx->max_ny * (ctx->max_ny + 8) * sizeof(float2)),
       "cudaMalloc(factor work)");
  }
  CK(cudaMemcpy(ctx->d_cells.p, ctx->cells.data(), ctx->cells.size() * sizeof(DevCell), cudaMemcpyHostToDevice), "H2D cells");
  CK(cudaMemcpy(ctx->d_prof.p, prof.data(), prof.size() * sizeof(double2), cudaMemcpyHostToDevice), "H2D prof");
  CK(cudaMemcpy(ctx->d_gprof.p, gprof.data(), gprof.size() * sizeof(double2), cudaMemcpyHostToDevice), "H2D gprof");
  CK(cudaMemcpy(ctx->d_m.p, m_grid, (size_t)ctx->n2 * sizeof(double), cudaMemcpyHostToDevice), "H2D m");
  ctx->is_setup = true;
  return LSW_OK;
}

lsw_status lsw_problem_info_get(const lsw_ctx* ctx, lsw_problem_info* o) {
  if (!ctx || !o) return LSW_ERR_INVALID_ARGUMENT;
  if (!ctx->is_setup) return LSW_ERR_NOT_SET_UP;
  o->n_g = ctx->n_g; o->n_dof = ctx->n_dof; o->n_cells_total = ctx->ncell;
  o->max_cell_side = std::max(ctx->max_nx, ctx->max_ny);
  o->precision = ctx->prec; o->factorized = ctx->factorized ? 1 : 0;
  o->factor_bytes = (long long)ctx->d_fac.bytes;
  o->device_bytes = (long long)device_bytes(ctx);
  o->omega = ctx->omega; o->pml_C = ctx->C;
  o->kernel_launches = ctx->launches;
  return LSW_OK;
}

lsw_status lsw_cell_info_get(const lsw_ctx* ctx, int cell, lsw_cell_info* o) {
  if (!ctx || !o) return LSW_ERR_INVALID_ARGUMENT;
  if (!ctx->is_setup) return LSW_ERR_NOT_SET_UP;
  if (cell < 0 || cell >= ctx->ncell) return LSW_ERR_INVALID_ARGUMENT;
  fill_info(ctx->cells[cell], o);
  return LSW_OK;
}

lsw_status lsw_factorize(lsw_ctx* ctx, void* stream) {
  if (!ctx) return LSW_ERR_INVALID_ARGUMENT;
  if (!ctx->is_setup) return fail(ctx, LSW_ERR_NOT_SET_UP, "lsw_problem_setup first");
  if (ctx->factorized) return LSW_OK;   // idempotent (LocalLinearSolverEigenSparseLU.cpp:42-45)
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t st = S(stream);
  CK(cudaMemsetAsync(ctx->d_status.p, 0, 16, st), "memset status");
  ctx->launches += 2;   // half chains, middle lines
  const double w2 = ctx->omega * ctx->omega;
  const bool tc = ctx->prec != LSW_PREC_C128 && ctx->factor_tc && factorize_tc_supported(ctx->max_ny);
  cudaError_t e = tc ? launch_factorize_tc(ctx->d_cells.as<DevCell>(), ctx->ncell, ctx->d_prof.as<double2>(),
                                           ctx->d_m.as<double>(), ctx->n_dof, w2, ctx->d_fac.p, ctx->d_work.p,
                                           ctx->max_ny, ctx->d_status.as<int>(), st, ctx->prec == LSW_PREC_SPLIT,
                                           ctx->wait_cycles)
                  : ctx->prec != LSW_PREC_C128
                      ? launch_factorize<float>(ctx->d_cells.as<DevCell>(), ctx->ncell, ctx->d_prof.as<double2>(),
                                                ctx->d_m.as<double>(), ctx->n_dof, w2, ctx->d_fac.p, ctx->d_work.p,
                                                ctx->max_ny, ctx->d_status.as<int>(), st, ctx->prec == LSW_PREC_SPLIT,
                                                ctx->factor_lookahead, ctx->wait_cycles)
                      : launch_factorize<double>(ctx->d_cells.as<DevCell>(), ctx->ncell, ctx->d_prof.as<double2>(),
                                                 ctx->d_m.as<double>(), ctx->n_dof, w2, ctx->d_fac.p, ctx->d_work.p,
                                                 ctx->max_ny, ctx->d_status.as<int>(), st, false,
                                                 false,   // complex128: the update dominates, no overlap
                                                 ctx->wait_cycles);
  CK(e, "factorize kernel");
  int status = 0;
  CK(cudaMemcpyAsync(&status, ctx->d_status.p, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H status");
  CK(cudaStreamSynchronize(st), "factorize sync");
  if (status & 6) return fail(ctx, LSW_ERR_CUDA, "factorisation kernel: cluster not formed or a bounded wait ran out");
  if (status & 1) return fail(ctx, LSW_ERR_SINGULAR_BLOCK, "zero or non-finite pivot in a Schur complement block");
  ctx->factorized = true;
  return LSW_OK;
}

lsw_status lsw_apply_precond(lsw_ctx* ctx, const void* x, void* y, int nrhs, void* stream) {
  if (!ctx || !x || !y || nrhs < 1) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "bad arguments to lsw_apply_precond");
  if (!ctx->is_setup) return fail(ctx, LSW_ERR_NOT_SET_UP, "lsw_problem_setup first");
  if (!ctx->factorized) return fail(ctx, LSW_ERR_NOT_FACTORIZED, "lsw_factorize first");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  return precond_impl(ctx, reinterpret_cast<const double2*>(x), reinterpret_cast<double2*>(y), nrhs, S(stream));
}

lsw_status lsw_apply_precond_profiled(lsw_ctx* ctx, const void* x, void* y, int nrhs, void* stream,
                                      lsw_apply_profile* prof) {
  if (!ctx || !x || !y || nrhs < 1 || !prof) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "bad arguments");
  if (!ctx->is_setup) return fail(ctx, LSW_ERR_NOT_SET_UP, "lsw_problem_setup first");
  if (!ctx->factorized) return fail(ctx, LSW_ERR_NOT_FACTORIZED, "lsw_factorize first");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t st = S(stream);
  Schedule* sc = nullptr;
  lsw_status s = ensure_batch(ctx, nrhs, &sc, st);
  if (s != LSW_OK) return s;
  std::vector<cudaEvent_t> ev(2 * sc->fronts.size() + 2);
  for (auto& e : ev) CK(cudaEventCreate(&e), "cudaEventCreate");
  ctx->front_events = &ev;
  CK(cudaEventRecord(ev[ev.size() - 2], st), "event");
  s = precond_impl(ctx, reinterpret_cast<const double2*>(x), reinterpret_cast<double2*>(y), nrhs, st);
  ctx->front_events = nullptr;
  if (s != LSW_OK) { for (auto& e : ev) cudaEventDestroy(e); return s; }
  CK(cudaEventRecord(ev[ev.size() - 1], st), "event");
  CK(cudaEventSynchronize(ev[ev.size() - 1]), "event sync");
  if ((s = check_kernel_err(ctx, st)) != LSW_OK) return s;
  double fm = 0.0;
  const bool log_fronts = std::getenv("LSW_FRONT_LOG") != nullptr;   // per-front lines on stderr
  for (size_t f = 0; f < sc->fronts.size(); ++f) {
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ev[2 * f], ev[2 * f + 1]), "elapsed");
    fm += ms;
    if (log_fronts) {
      const Front& fr = sc->fronts[f];
      std::fprintf(stderr, "front %zu items %d max_slots %d cluster %d ms %.4f\n", f, fr.item_count, fr.max_slots,
                   fr.cluster, ms);
    }
  }
  float tot = 0.f;
  CK(cudaEventElapsedTime(&tot, ev[ev.size() - 2], ev[ev.size() - 1]), "elapsed");
  for (auto& e : ev) cudaEventDestroy(e);
  // algorithmic bytes / flops from the schedule
  std::vector<DevItem> items(sc->fronts.empty() ? 0 : sc->fronts.back().item_begin + sc->fronts.back().item_count);
  CK(cudaMemcpy(items.data(), sc->d_items, items.size() * sizeof(DevItem), cudaMemcpyDeviceToHost), "D2H items");
  // algorithmic bytes count each cell's factor once per front (forward and
  // backward pass) however its slots are split into items; the streamed
  // bytes count every item's pass
  const double cs = (double)csize(ctx->prec);
  double bytes = 0.0, flops = 0.0, streamed = 0.0;
  int slots = 0;
  // (per-sweep launches of one step count a cell's factor once for the step,
  // as one launch per step does)
  std::map<std::pair<int, int>, std::map<int, int>> per_step;
  for (const Front& fr : sc->fronts)
    for (int i = fr.item_begin; i < fr.item_begin + fr.item_count; ++i)
      per_step[{fr.stage, fr.step}][items[i].cell] += items[i].slot_count;
  for (const auto& st_cells : per_step) {
    for (const auto& kv : st_cells.second) {
      const DevCell& c = ctx->cells[kv.first];
      const double F = (double)c.nx * c.ny * c.ny * cs;
      bytes += 2.0 * F + 4.0 * kv.second * (double)c.nx * c.ny * cs;
      flops += 2.0 * 8.0 * (double)c.nx * c.ny * c.ny * kv.second;
      slots += kv.second;
    }
  }
  for (const Front& fr : sc->fronts) {
    for (int i = fr.item_begin; i < fr.item_begin + fr.item_count; ++i) {
      const DevCell& c = ctx->cells[items[i].cell];
      streamed += 2.0 * (double)c.nx * c.ny * c.ldn * cs + 4.0 * items[i].slot_count * (double)c.nx * c.ny * cs;
    }
  }
  prof->fronts = (int)sc->fronts.size();
  prof->items = (int)items.size();
  prof->slots = slots;
  prof->front_ms = fm;
  prof->total_ms = tot;
  prof->alg_bytes = bytes;
  prof->alg_flops = flops;
  prof->streamed_bytes = streamed;
  return LSW_OK;
}

lsw_status lsw_apply_A(lsw_ctx* ctx, const void* x, void* y, int nrhs, void* stream) {
  if (!ctx || !x || !y || nrhs < 1) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "bad arguments to lsw_apply_A");
  if (!ctx->is_setup) return fail(ctx, LSW_ERR_NOT_SET_UP, "lsw_problem_setup first");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  return apply_A_impl(ctx, reinterpret_cast<const double2*>(x), reinterpret_cast<double2*>(y), nrhs, S(stream));
}

lsw_status lsw_assemble_rhs(lsw_ctx* ctx, const double* src, const double* amp, int nsrc, void* b, void* stream) {
  if (!ctx || !b || nsrc < 0 || (nsrc > 0 && !src)) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "bad arguments to lsw_assemble_rhs");
  if (!ctx->is_setup) return fail(ctx, LSW_ERR_NOT_SET_UP, "lsw_problem_setup first");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t st = S(stream);
  std::vector<double> hs(2 * std::max(nsrc, 1) + std::max(nsrc, 1));
  for (int i = 0; i < 2 * nsrc; ++i) hs[i] = src[i];
  for (int i = 0; i < nsrc; ++i) hs[2 * nsrc + i] = amp ? amp[i] : 1.0;
  CK(ctx->k_small2.ensure(hs.size() * sizeof(double) + 64), "cudaMalloc(src)");
  CK(cudaMemcpyAsync(ctx->k_small2.p, hs.data(), hs.size() * sizeof(double), cudaMemcpyHostToDevice, st), "H2D src");
  // eps = DD mesh size (Input.cpp:243): every cell has mesh size h on the integer grid
  KL(1, launch_rhs(reinterpret_cast<double2*>(b), ctx->n_dof, ctx->p, ctx->h, ctx->k_small2.as<double>(),
                ctx->k_small2.as<double>() + 2 * nsrc, nsrc, ctx->h, st), "rhs kernel");
  CK(cudaStreamSynchronize(st), "rhs sync");
  return LSW_OK;
}

lsw_status lsw_local_solve(lsw_ctx* ctx, int cell, const void* b, void* x, int nrhs, void* stream) {
  if (!ctx || !b || !x || nrhs < 1) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "bad arguments to lsw_local_solve");
  if (!ctx->is_setup) return fail(ctx, LSW_ERR_NOT_SET_UP, "lsw_problem_setup first");
  if (cell < 0 || cell >= ctx->ncell) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "cell index out of range");
  if (!ctx->factorized)   // LocalLinearSolverEigenSparseLU.cpp:68-72
    return fail(ctx, LSW_ERR_NOT_FACTORIZED, "The linear system has to be factorized before it can be solved");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t st = S(stream);
  const bool dbl = ctx->prec == LSW_PREC_C128;
  const int rmax = front_rmax(dbl);
  const DevCell& cl = ctx->cells[cell];
  std::vector<DevItem> items;
  std::vector<DevSlot> slots;
  long long scr = 0;
  for (int r0 = 0; r0 < nrhs; r0 += rmax) {
    DevItem it{};
    it.cell = cell; it.slot_begin = (int)slots.size(); it.group_begin = 0; it.group_count = 0;
    it.slot_count = std::min(rmax, nrhs - r0);
    it.scratch_off = scr;
    scr += (long long)(cl.nx + 1) * front_rpad(it.slot_count) * cl.ny;
    for (int r = r0; r < r0 + it.slot_count; ++r) {
      DevSlot s{};
      s.kind = SK_CELLVEC; s.rhs = r;
      s.in_lr0 = s.in_lr1 = s.in_ud0 = s.in_ud1 = -1;
      slots.push_back(s);
    }
    items.push_back(it);
  }
  CK(ctx->ls_items.ensure(items.size() * sizeof(DevItem)), "cudaMalloc(ls items)");
  CK(ctx->ls_slots.ensure(slots.size() * sizeof(DevSlot)), "cudaMalloc(ls slots)");
  CK(ctx->ls_scratch.ensure((size_t)scr * csize(ctx->prec)), "cudaMalloc(ls scratch)");
  CK(cudaMemcpyAsync(ctx->ls_items.p, items.data(), items.size() * sizeof(DevItem), cudaMemcpyHostToDevice, st), "H2D");
  CK(cudaMemcpyAsync(ctx->ls_slots.p, slots.data(), slots.size() * sizeof(DevSlot), cudaMemcpyHostToDevice, st), "H2D");
  FrontArgs a{};
  a.cells = ctx->d_cells.as<DevCell>();
  a.items = ctx->ls_items.as<DevItem>();
  a.slots = ctx->ls_slots.as<DevSlot>();
  a.groups = nullptr;
  a.fac = ctx->d_fac.p;
  a.prof = ctx->d_prof.as<double2>();
  a.traces = nullptr; a.outs = nullptr;
  a.scratch = ctx->ls_scratch.p;
  a.x_in = reinterpret_cast<const double2*>(b);
  a.x_stride = (long long)cl.nx * cl.ny;
  a.x_out = reinterpret_cast<double2*>(x);
  a.out_stride = (long long)cl.nx * cl.ny;
  a.n_dof = ctx->n_dof; a.N = ctx->N; a.m = ctx->m; a.p = ctx->p;
  a.item_count = (int)items.size();
  a.max_slots = std::min(rmax, nrhs);
  a.err = ctx->d_status.as<int>() + 1;
  a.wait_cycles = ctx->wait_cycles;
  a.split = ctx->prec == LSW_PREC_SPLIT ? 1 : 0;
  a.cluster = fitting_cluster(ctx, a.max_slots, front_cluster(a.item_count, ctx->nsm, ctx->max_cluster));
  cudaError_t e = dbl ? launch_front<double>(a, ctx->max_ny, ctx->max_nx, st) : launch_front<float>(a, ctx->max_ny, ctx->max_nx, st);
  CK(e, "local solve kernel");
  ctx->launches += 1;
  return check_kernel_err(ctx, st);
}

// ---------------------------------------------------------------------------
// GMRES
// ---------------------------------------------------------------------------
static lsw_status gmres_reference(lsw_ctx* ctx, const double2* b, double2* x, int nv, const lsw_gmres_opts* o,
                                  lsw_gmres_report* rep, cudaStream_t st) {
  const long long n2 = ctx->n2;
  const size_t vb = (size_t)nv * n2 * sizeof(double2);
  const int maxit = o->max_iter;
  CK(ctx->k_basis.ensure(vb * (size_t)(maxit + 1)), "cudaMalloc(Q)");
  CK(ctx->k_tmp.ensure(vb), "cudaMalloc(tmp)");
  CK(ctx->k_r.ensure(vb), "cudaMalloc(rhsPrec)");
  CK(ctx->k_part.ensure((size_t)nv * 1216 * sizeof(double2)), "cudaMalloc(partials)");
  CK(ctx->k_small.ensure((size_t)nv * (maxit + 2) * sizeof(double2) + 64), "cudaMalloc(h)");
  CK(ctx->k_small2.ensure((size_t)nv * (maxit + 2) * sizeof(double2) + 64), "cudaMalloc(coef)");
  CK(ctx->k_nrm.ensure((size_t)nv * 2 * sizeof(double2) + 64), "cudaMalloc(nrm)");
  double2* Q = ctx->k_basis.as<double2>();
  double2* tmp = ctx->k_tmp.as<double2>();
  double2* rp = ctx->k_r.as<double2>();
  double2* part = ctx->k_part.as<double2>();
  double2* hdev = ctx->k_small.as<double2>();
  double2* cdev = ctx->k_small2.as<double2>();
  double* ndev = ctx->k_nrm.as<double>();
  auto Qi = [&](int i) { return Q + (size_t)i * nv * n2; };
  lsw_status s;
  int applies = 0;
  // rhsPrec = M^-1 b ; x0 = rhsPrec (GlobalIterativeSolverGMRES.cpp:75-78)
  if ((s = precond_impl(ctx, b, rp, nv, st)) != LSW_OK) return s;
  ++applies;
  CK(cudaMemcpyAsync(x, rp, vb, cudaMemcpyDeviceToDevice, st), "copy x0");
  // r = rhsPrec - M^-1 A x0 (81-84), stored as Q_0 before normalisation
  if ((s = apply_A_impl(ctx, x, tmp, nv, st)) != LSW_OK) return s;
  if ((s = precond_impl(ctx, tmp, Qi(0), nv, st)) != LSW_OK) return s;
  ++applies;
  for (int v = 0; v < nv; ++v) KL(1, launch_sub(Qi(0) + v * n2, rp + v * n2, Qi(0) + v * n2, n2, st), "sub");
  KL(2, launch_norm2(rp, n2, nv, n2, reinterpret_cast<double*>(part), ndev, st), "norm");
  KL(2, launch_norm2(Qi(0), n2, nv, n2, reinterpret_cast<double*>(part), ndev + nv, st), "norm");
  std::vector<double> hn(2 * nv);
  CK(cudaMemcpyAsync(hn.data(), ndev, 2 * nv * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H norms");
  CK(cudaStreamSynchronize(st), "sync");
  std::vector<double> rhs_norm(nv), r_norm(nv);
  std::vector<std::vector<double>> logs(nv);
  std::vector<int> done(nv, 0), lastk(nv, -1);
  for (int v = 0; v < nv; ++v) {
    rhs_norm[v] = std::sqrt(hn[v]);
    r_norm[v] = std::sqrt(hn[nv + v]);
    logs[v].push_back(r_norm[v] / rhs_norm[v]);
    if (logs[v][0] < o->tol || maxit == 0) done[v] = 1;   // (115-116)
  }
  if (o->verbose) printf("iteration 0: %.6e\n", logs[0][0]);
  bool all = std::all_of(done.begin(), done.end(), [](int d) { return d != 0; });
  std::vector<std::vector<cplx>> H(nv), beta(nv), cs(nv), sn(nv);
  int kmax = -1;
  if (!all) {
    std::vector<double2> rsc(nv);
    for (int v = 0; v < nv; ++v) rsc[v] = make_double2(r_norm[v], 0.0);
    CK(cudaMemcpyAsync(cdev, rsc.data(), nv * sizeof(double2), cudaMemcpyHostToDevice, st), "H2D");
    KL(1, launch_scale(Qi(0), Qi(0), cdev, 1, n2, nv, n2, st), "scale");
    for (int v = 0; v < nv; ++v) beta[v].push_back(cplx(r_norm[v], 0.0));
    for (int k = 0; k < maxit; ++k) {
      // arnoldi (238-310): q = M^-1 A Q_k ; h_i = q.dot(Q_i) = sum conj(q) Q_i ; q -= h_i Q_i
      if ((s = apply_A_impl(ctx, Qi(k), tmp, nv, st)) != LSW_OK) return s;
      double2* q = Qi(k + 1);
      if ((s = precond_impl(ctx, tmp, q, nv, st)) != LSW_OK) return s;
      ++applies;
      KL(2, launch_dot(q, Qi(0), n2, nv, n2, part, hdev, st), "dot");
      for (int i = 0; i <= k; ++i) {
        // coefficients for all rhs of column i sit at hdev[i*nv + v]
        if (i < k)
          KL(2, launch_axpy_dot(q, Qi(i), hdev + (size_t)i * nv, Qi(i + 1), n2, nv, n2, part,
                             hdev + (size_t)(i + 1) * nv, 1, st), "axpy_dot");
        else
          KL(2, launch_axpy_dot(q, Qi(i), hdev + (size_t)i * nv, nullptr, n2, nv, n2, part,
                             hdev + (size_t)(k + 1) * nv, 1, st), "axpy_norm");
      }
      std::vector<double2> hh((size_t)(k + 2) * nv);
      CK(cudaMemcpyAsync(hh.data(), hdev, hh.size() * sizeof(double2), cudaMemcpyDeviceToHost, st), "D2H h");
      CK(cudaStreamSynchronize(st), "sync");
      std::vector<double2> sc(nv);
      for (int v = 0; v < nv; ++v) {
        std::vector<cplx> h(k + 2);
        for (int i = 0; i <= k; ++i) h[i] = cplx(hh[(size_t)i * nv + v].x, hh[(size_t)i * nv + v].y);
        const double qn = std::sqrt(hh[(size_t)(k + 1) * nv + v].x);
        h[k + 1] = qn;
        sc[v] = make_double2(qn != 0.0 ? qn : 1.0, 0.0);
        // apply_givens_rotation (313-330): rotations 0..k-2 only
        for (int i = 1; i < k; ++i) {
          const cplx t = cs[v][i - 1] * h[i - 1] + sn[v][i - 1] * h[i];
          h[i] = -sn[v][i - 1] * h[i - 1] + cs[v][i - 1] * h[i];
          h[i - 1] = t;
        }
        cplx c_, s_;
        givens_ref(h[k], h[k + 1], c_, s_);
        h[k] = c_ * h[k] + s_ * h[k + 1];
        h[k + 1] = 0.0;
        cs[v].push_back(c_); sn[v].push_back(s_);
        // H grows by one row and one column (134-162)
        std::vector<cplx> Hn((size_t)(k + 2) * (k + 1), cplx(0, 0));
        for (int i = 0; i < k + 1; ++i)
          for (int j = 0; j < k; ++j) Hn[(size_t)i * (k + 1) + j] = H[v][(size_t)i * k + j];
        for (int i = 0; i < k + 2; ++i) Hn[(size_t)i * (k + 1) + k] = h[i];
        H[v].swap(Hn);
        beta[v].push_back(-sn[v][k] * beta[v][k]);   // (168-171)
        beta[v][k] *= cs[v][k];
        if (!done[v]) {
          logs[v].push_back(std::abs(beta[v].back()) / rhs_norm[v]);
          if (logs[v].back() <= o->tol || k == maxit - 1) { done[v] = 1; lastk[v] = k; }
        }
      }
      if (o->verbose) printf("iteration %d: %.6e\n", k + 1, logs[0].back());
      CK(cudaMemcpyAsync(cdev, sc.data(), nv * sizeof(double2), cudaMemcpyHostToDevice, st), "H2D");
      KL(1, launch_scale(q, q, cdev, 1, n2, nv, n2, st), "scale");
      kmax = k;
      if (std::all_of(done.begin(), done.end(), [](int d) { return d != 0; })) break;
    }
    // y = H(0:k,0:k)^-1 beta ; x += Q y  (194-201)
    const int ncol = kmax + 1;
    std::vector<double2> coef((size_t)nv * ncol, make_double2(0, 0));
    for (int v = 0; v < nv; ++v) {
      if (lastk[v] < 0) continue;
      const int kk = lastk[v] + 1;
      std::vector<cplx> A((size_t)kk * kk), rhs(kk);
      const int cols = kmax + 1;
      for (int i = 0; i < kk; ++i) {
        rhs[i] = beta[v][i];
        for (int j = 0; j < kk; ++j) A[(size_t)i * kk + j] = H[v][(size_t)i * cols + j];
      }
      std::vector<cplx> y = dense_solve(A, rhs, kk);
      for (int i = 0; i < kk; ++i) coef[(size_t)v * ncol + i] = make_double2(y[i].real(), y[i].imag());
    }
    CK(ctx->k_small2.ensure(coef.size() * sizeof(double2) + 64), "cudaMalloc(coef)");
    cdev = ctx->k_small2.as<double2>();
    CK(cudaMemcpyAsync(cdev, coef.data(), coef.size() * sizeof(double2), cudaMemcpyHostToDevice, st), "H2D y");
    KL(1, launch_lincomb(x, Q, (long long)nv * n2, n2, cdev, ncol, n2, nv, n2, st), "lincomb");
  }
  int iters = 0;
  double fl = 0.0;
  for (int v = 0; v < nv; ++v) {
    iters = std::max(iters, (int)logs[v].size() - 1);
    fl = std::max(fl, logs[v].back());
  }
  if (rep) {
    rep->iterations = iters;
    rep->final_log = fl;
    rep->precond_applies = applies;
    rep->converged = fl <= o->tol ? 1 : 0;
    if (rep->log && rep->log_capacity > 0) {
      rep->log_len = std::min<int>(rep->log_capacity, (int)logs[0].size());
      for (int i = 0; i < rep->log_len; ++i) rep->log[i] = logs[0][i];
    }
  }
  return LSW_OK;
}

// Right-preconditioned flexible GMRES(m) (Saad 1993) with modified Gram-Schmidt.
// The Hessenberg least-squares problem (complex Givens rotations, the rotated
// right-hand side, the back substitution at the end of a cycle) stays on the
// device in FP64; an iteration reads back only the residual estimates.
static lsw_status gmres_flexible(lsw_ctx* ctx, const double2* b, double2* x, int nv, const lsw_gmres_opts* o,
                                 lsw_gmres_report* rep, cudaStream_t st) {
  const long long n2 = ctx->n2;
  const size_t vb = (size_t)nv * n2 * sizeof(double2);
  const int m = std::max(1, o->restart);
  CK(ctx->k_basis.ensure(vb * (size_t)(m + 1)), "cudaMalloc(V)");
  CK(ctx->k_zbasis.ensure(vb * (size_t)m), "cudaMalloc(Z)");
  CK(ctx->k_tmp.ensure(vb), "cudaMalloc(tmp)");
  CK(ctx->k_part.ensure((size_t)nv * 1216 * sizeof(double2)), "cudaMalloc(partials)");
  CK(ctx->k_small.ensure((size_t)nv * (m + 2) * sizeof(double2) + 64), "cudaMalloc(h)");
  CK(ctx->k_nrm.ensure((size_t)nv * 2 * sizeof(double2) + 64), "cudaMalloc(nrm)");
  // least-squares state: H, cs, sn, coef, g, sc (complex); ||b||, est (2 nv), rel (real); active (int)
  const size_t nH = (size_t)nv * (m + 1) * m, nR = (size_t)nv * m, nG = (size_t)nv * (m + 1);
  const size_t cplx_n = nH + 3 * nR + nG + (size_t)nv;
  CK(ctx->k_ls.ensure(cplx_n * sizeof(double2) + 4 * (size_t)nv * sizeof(double) + (size_t)nv * sizeof(int) + 64),
     "cudaMalloc(least squares)");
  double2* Hd = ctx->k_ls.as<double2>();
  double2* csd = Hd + nH;
  double2* snd = csd + nR;
  double2* coefd = snd + nR;
  double2* gd = coefd + nR;
  double2* scd = gd + nG;
  double* bnd = reinterpret_cast<double*>(scd + nv);
  double* estd = bnd + nv;
  double* reld = estd + 2 * nv;
  int* actd = reinterpret_cast<int*>(reld + nv);
  double2* V = ctx->k_basis.as<double2>();
  double2* Z = ctx->k_zbasis.as<double2>();
  double2* tmp = ctx->k_tmp.as<double2>();
  double2* part = ctx->k_part.as<double2>();
  double2* hdev = ctx->k_small.as<double2>();
  double* ndev = ctx->k_nrm.as<double>();
  auto Vi = [&](int i) { return V + (size_t)i * nv * n2; };
  auto Zi = [&](int i) { return Z + (size_t)i * nv * n2; };
  lsw_status s;
  int applies = 0, it = 0;
  CK(cudaMemsetAsync(x, 0, vb, st), "x0 = 0");
  KL(2, launch_norm2(b, n2, nv, n2, reinterpret_cast<double*>(part), ndev, st), "norm b");
  std::vector<double> bn(nv);
  CK(cudaMemcpyAsync(bn.data(), ndev, nv * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaStreamSynchronize(st), "sync");
  for (auto& q : bn) q = std::sqrt(q);
  CK(cudaMemcpyAsync(bnd, bn.data(), nv * sizeof(double), cudaMemcpyHostToDevice, st), "H2D |b|");
  std::vector<double> rel(nv, 1.0), est(2 * (size_t)nv, 0.0), log0;
  std::vector<int> active(nv, 1);
  while (true) {
    // r = b - A x, its norm, the cycle's least-squares state
    if ((s = apply_A_impl(ctx, x, tmp, nv, st)) != LSW_OK) return s;
    for (int v = 0; v < nv; ++v) KL(1, launch_sub(Vi(0) + v * n2, b + v * n2, tmp + v * n2, n2, st), "sub");
    KL(2, launch_norm2(Vi(0), n2, nv, n2, reinterpret_cast<double*>(part), ndev, st), "norm r");
    KL(1, launch_fgmres_init(nv, m, ndev, bnd, o->tol, scd, gd, reld, actd, st), "least squares init");
    CK(cudaMemcpyAsync(rel.data(), reld, nv * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
    CK(cudaStreamSynchronize(st), "sync");
    bool all_conv = true;
    for (int v = 0; v < nv; ++v) {
      active[v] = rel[v] <= o->tol ? 0 : 1;
      all_conv = all_conv && !active[v];
    }
    log0.push_back(rel[0]);
    if (o->verbose) printf("fgmres it %d: true rel. residual %.6e\n", it, rel[0]);
    if (all_conv || it >= o->max_iter) break;
    KL(1, launch_scale(Vi(0), Vi(0), scd, 1, n2, nv, n2, st), "scale");
    int ncol = 0;
    for (int j = 0; j < m; ++j) {
      if ((s = precond_impl(ctx, Vi(j), Zi(j), nv, st)) != LSW_OK) return s;
      ++applies;
      double2* w = Vi(j + 1);
      if ((s = apply_A_impl(ctx, Zi(j), w, nv, st)) != LSW_OK) return s;
      // MGS: h_i = V_i^H w ; w -= h_i V_i
      KL(2, launch_dot(Vi(0), w, n2, nv, n2, part, hdev, st), "dot");
      for (int i = 0; i <= j; ++i) {
        if (i < j)
          KL(2, launch_axpy_dot(w, Vi(i), hdev + (size_t)i * nv, Vi(i + 1), n2, nv, n2, part,
                             hdev + (size_t)(i + 1) * nv, 0, st), "axpy_dot");
        else
          KL(2, launch_axpy_dot(w, Vi(i), hdev + (size_t)i * nv, nullptr, n2, nv, n2, part,
                             hdev + (size_t)(j + 1) * nv, 0, st), "axpy_norm");
      }
      KL(1, launch_fgmres_givens(j, nv, m, hdev, Hd, csd, snd, gd, scd, estd, bnd, st), "givens");
      KL(1, launch_scale(w, w, scd, 1, n2, nv, n2, st), "scale");
      CK(cudaMemcpyAsync(est.data(), estd, 2 * nv * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H estimate");
      CK(cudaStreamSynchronize(st), "sync");
      ++it;
      ncol = j + 1;
      bool all_small = true;
      for (int v = 0; v < nv; ++v)
        if (active[v] && est[v] > o->tol && est[nv + v] > 0) all_small = false;
      log0.push_back(est[0]);
      if (o->verbose) printf("fgmres it %d: estimate %.6e\n", it, log0.back());
      if (all_small || it >= o->max_iter) break;
    }
    // x += Z y with y from the triangular system R y = g
    KL(1, launch_fgmres_solve(ncol, nv, m, Hd, gd, actd, coefd, st), "least squares solve");
    KL(1, launch_lincomb(x, Z, (long long)nv * n2, n2, coefd, ncol, n2, nv, n2, st), "lincomb");
  }
  // the largest relative residual; a NaN (a non-finite solve) propagates
  double worst = 0.0;
  for (int v = 0; v < nv; ++v)
    if (!(rel[v] <= worst)) worst = rel[v];
  if (rep) {
    rep->iterations = it;
    rep->final_log = worst;
    rep->precond_applies = applies;
    rep->converged = worst <= o->tol ? 1 : 0;
    if (rep->log && rep->log_capacity > 0) {
      rep->log_len = std::min<int>(rep->log_capacity, (int)log0.size());
      for (int i = 0; i < rep->log_len; ++i) rep->log[i] = log0[i];
    }
  }
  return LSW_OK;
}

static lsw_status true_residual(lsw_ctx* ctx, const double2* b, const double2* x, int nv, double* worst,
                                cudaStream_t st) {
  const long long n2 = ctx->n2;
  CK(ctx->k_tmp2.ensure((size_t)nv * n2 * sizeof(double2)), "cudaMalloc(res)");
  CK(ctx->k_part.ensure((size_t)nv * 1216 * sizeof(double2)), "cudaMalloc(partials)");
  CK(ctx->k_nrm.ensure((size_t)nv * 2 * sizeof(double2) + 64), "cudaMalloc(nrm)");
  double2* r = ctx->k_tmp2.as<double2>();
  lsw_status s = apply_A_impl(ctx, x, r, nv, st);
  if (s != LSW_OK) return s;
  for (int v = 0; v < nv; ++v) KL(1, launch_sub(r + v * n2, b + v * n2, r + v * n2, n2, st), "sub");
  double* nd = ctx->k_nrm.as<double>();
  KL(2, launch_norm2(r, n2, nv, n2, reinterpret_cast<double*>(ctx->k_part.p), nd, st), "norm");
  KL(2, launch_norm2(b, n2, nv, n2, reinterpret_cast<double*>(ctx->k_part.p), nd + nv, st), "norm");
  std::vector<double> h(2 * nv);
  CK(cudaMemcpyAsync(h.data(), nd, 2 * nv * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
  CK(cudaStreamSynchronize(st), "sync");
  // the largest relative residual; a NaN (a non-finite solution) propagates
  *worst = 0.0;
  for (int v = 0; v < nv; ++v) {
    const double rv = h[nv + v] > 0 ? std::sqrt(h[v] / h[nv + v]) : 0.0;
    if (!(rv <= *worst)) *worst = rv;
  }
  return LSW_OK;
}

lsw_status lsw_gmres(lsw_ctx* ctx, const void* b, void* x, int nrhs, const lsw_gmres_opts* o, lsw_gmres_report* rep,
                     void* stream) {
  if (!ctx || !b || !x || !o || nrhs < 1) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "bad arguments to lsw_gmres");
  if (!ctx->is_setup) return fail(ctx, LSW_ERR_NOT_SET_UP, "lsw_problem_setup first");
  if (!ctx->factorized) return fail(ctx, LSW_ERR_NOT_FACTORIZED, "lsw_factorize first");
  if (o->max_iter < 0 || !(o->tol >= 0)) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "bad GMRES options");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t st = S(stream);
  const auto t0 = std::chrono::steady_clock::now();
  const double2* bb = reinterpret_cast<const double2*>(b);
  double2* xx = reinterpret_cast<double2*>(x);
  if (o->mode != LSW_GMRES_REFERENCE && o->mode != LSW_GMRES_FLEXIBLE)
    return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "unknown GMRES mode");
  // Right-hand sides per Krylov batch.  Every right-hand side of a batch keeps
  // its whole basis resident (2 m + 1 vectors for FGMRES(m), MaxIter + 1 for
  // the reference GMRES), so a batch larger than the free device memory holds
  // is solved as consecutive sub-batches, each still sharing every sweep
  // launch among its right-hand sides.
  const long long n2 = ctx->n2;
  const size_t vec = (size_t)n2 * sizeof(double2);
  const size_t nvec = o->mode == LSW_GMRES_REFERENCE ? (size_t)o->max_iter + 4 : 2 * (size_t)std::max(1, o->restart) + 4;
  const size_t per_rhs = nvec * vec + 12 * (size_t)n2 * csize(ctx->prec);   // + sweep pools (outputs, traces)
  size_t fr = 0, tot = 0;
  CK(cudaMemGetInfo(&fr, &tot), "cudaMemGetInfo");
  const size_t held = ctx->k_basis.bytes + ctx->k_zbasis.bytes + ctx->k_tmp.bytes + ctx->k_tmp2.bytes;
  const size_t margin = (size_t)2 << 30;
  const size_t budget = fr + held > margin ? fr + held - margin : 0;
  int chunk = (int)std::max<long long>(1, std::min<long long>(nrhs, (long long)(budget / per_rhs)));
  if (ctx->krylov_batch > 0) chunk = std::min(chunk, ctx->krylov_batch);
  // sub-batches of equal size (64 as 32 + 32, not 54 + 10): every sweep
  // launch of a sub-batch keeps as many right-hand sides as the others, and
  // all sub-batches share one schedule
  {
    const int nsub = (nrhs + chunk - 1) / chunk;
    chunk = (nrhs + nsub - 1) / nsub;
  }
  lsw_gmres_report sub{}, acc{};
  acc.converged = 1;
  double tr = 0.0;
  for (int c0 = 0; c0 < nrhs; c0 += chunk) {
    const int nv = std::min(chunk, nrhs - c0);
    sub = lsw_gmres_report{};
    if (rep && c0 == 0) { sub.log = rep->log; sub.log_capacity = rep->log_capacity; }
    lsw_status s = o->mode == LSW_GMRES_REFERENCE
                       ? gmres_reference(ctx, bb + (size_t)c0 * n2, xx + (size_t)c0 * n2, nv, o, &sub, st)
                       : gmres_flexible(ctx, bb + (size_t)c0 * n2, xx + (size_t)c0 * n2, nv, o, &sub, st);
    if (s != LSW_OK) return s;
    double t = 0.0;
    if ((s = true_residual(ctx, bb + (size_t)c0 * n2, xx + (size_t)c0 * n2, nv, &t, st)) != LSW_OK) return s;
    if (!(t <= tr)) tr = t;   // NaN propagates
    acc.iterations = std::max(acc.iterations, sub.iterations);
    if (!(sub.final_log <= acc.final_log)) acc.final_log = sub.final_log;
    acc.precond_applies += sub.precond_applies;
    acc.converged = acc.converged && sub.converged;
    if (c0 == 0) acc.log_len = sub.log_len;
  }
  lsw_status s;
  if ((s = check_kernel_err(ctx, st)) != LSW_OK) return s;
  CK(cudaStreamSynchronize(st), "sync");
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (rep) {
    rep->iterations = acc.iterations;
    rep->converged = acc.converged;
    rep->final_log = acc.final_log;
    rep->precond_applies = acc.precond_applies;
    rep->log_len = acc.log_len;
    rep->true_rel_res = tr;
    rep->seconds = secs;
  }
  return LSW_OK;
}

lsw_status lsw_solve_host(lsw_ctx* ctx, const double* b_host, double* x_host, int nrhs, const lsw_gmres_opts* o,
                          lsw_gmres_report* rep, void* stream) {
  if (!ctx || !b_host || !x_host || !o || nrhs < 1) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "bad arguments to lsw_solve_host");
  if (!ctx->is_setup) return fail(ctx, LSW_ERR_NOT_SET_UP, "lsw_problem_setup first");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t st = S(stream);
  const size_t vb = (size_t)nrhs * ctx->n2 * sizeof(double2);
  DevBuf& db = ctx->h_b;
  DevBuf& dx = ctx->h_x;
  CK(db.ensure(vb), "cudaMalloc(b)");
  CK(dx.ensure(vb), "cudaMalloc(x)");
  CK(cudaMemcpyAsync(db.p, b_host, vb, cudaMemcpyHostToDevice, st), "H2D b");
  lsw_status s = lsw_gmres(ctx, db.p, dx.p, nrhs, o, rep, stream);
  if (s != LSW_OK) return s;
  CK(cudaMemcpyAsync(x_host, dx.p, vb, cudaMemcpyDeviceToHost, st), "D2H x");
  CK(cudaStreamSynchronize(st), "sync");
  return LSW_OK;
}

lsw_status lsw_release_workspace(lsw_ctx* ctx) {
  if (!ctx) return LSW_ERR_INVALID_ARGUMENT;
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  CK(cudaDeviceSynchronize(), "sync");   // no launch may still use the buffers
  ctx->drop_graphs();
  ctx->sched.clear();
  ctx->sched_bufs.clear();
  for (DevBuf* b : {&ctx->d_traces, &ctx->d_outs, &ctx->d_scratch, &ctx->k_basis, &ctx->k_zbasis, &ctx->k_tmp,
                    &ctx->k_tmp2, &ctx->k_r, &ctx->k_part, &ctx->k_small, &ctx->k_small2, &ctx->k_nrm, &ctx->k_ls,
                    &ctx->ls_items, &ctx->ls_slots, &ctx->ls_scratch, &ctx->h_b, &ctx->h_x})
    b->release();
  return LSW_OK;
}

lsw_status lsw_local_solve_noalloc(lsw_ctx* ctx, int cell, const void* b, void* x, int nrhs, void* stream) {
  if (!ctx || !b || !x || nrhs < 1)
    return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "bad arguments to lsw_local_solve_noalloc");
  if (!ctx->is_setup) return fail(ctx, LSW_ERR_NOT_SET_UP, "lsw_problem_setup first");
  if (cell < 0 || cell >= ctx->ncell) return fail(ctx, LSW_ERR_INVALID_ARGUMENT, "cell index out of range");
  if (!ctx->factorized)
    return fail(ctx, LSW_ERR_NOT_FACTORIZED, "The linear system has to be factorized before it can be solved");
  CK(cudaSetDevice(ctx->device), "cudaSetDevice");
  cudaStream_t st = S(stream);
  const bool dbl = ctx->prec == LSW_PREC_C128;
  const int rmax = front_rmax(dbl);
  const DevCell& cl = ctx->cells[cell];
  const int n_items = (nrhs + rmax - 1) / rmax;
  const long long per_item = (long long)(cl.nx + 1) * front_rpad(std::min(rmax, nrhs)) * cl.ny;
  const size_t desc_bytes = ((size_t)n_items * sizeof(DevItem) + (size_t)nrhs * sizeof(DevSlot) + 255) & ~size_t(255);
  const size_t need = desc_bytes + (size_t)n_items * per_item * csize(ctx->prec);
  if (need > kNoAllocScratchBytes) {
    return fail(ctx, LSW_ERR_INVALID_ARGUMENT,
                "lsw_local_solve_noalloc: " + std::to_string(nrhs) + " right-hand sides of cell " +
                    std::to_string(cell) + " need " + std::to_string(need) + " bytes of scratch, more than the " +
                    std::to_string(kNoAllocScratchBytes) + "-byte fixed buffer; use fewer right-hand sides per call");
  }
  // the array's device address on this context's device (lsw_ctx_create)
  unsigned char* bp = static_cast<unsigned char*>(ctx->noalloc_base);
  if (!bp) return fail(ctx, LSW_ERR_CUDA, "no-allocation scratch address unknown");
  DevItem* d_items = reinterpret_cast<DevItem*>(bp);
  DevSlot* d_slots = reinterpret_cast<DevSlot*>(bp + (size_t)n_items * sizeof(DevItem));
  void* d_scr = bp + desc_bytes;
  // every element of the forward storage is written before it is read, so
  // nothing in the shared array needs clearing between calls
  k_noalloc_desc<<<(nrhs + 127) / 128, 128, 0, st>>>(d_items, d_slots, cell, nrhs, rmax, per_item);
  CK(cudaGetLastError(), "descriptor kernel");
  FrontArgs a{};
  a.cells = ctx->d_cells.as<DevCell>();
  a.items = d_items;
  a.slots = d_slots;
  a.groups = nullptr;
  a.fac = ctx->d_fac.p;
  a.prof = ctx->d_prof.as<double2>();
  a.traces = nullptr; a.outs = nullptr;
  a.scratch = d_scr;
  a.x_in = reinterpret_cast<const double2*>(b);
  a.x_stride = (long long)cl.nx * cl.ny;
  a.x_out = reinterpret_cast<double2*>(x);
  a.out_stride = (long long)cl.nx * cl.ny;
  a.n_dof = ctx->n_dof; a.N = ctx->N; a.m = ctx->m; a.p = ctx->p;
  a.item_count = n_items;
  a.max_slots = std::min(rmax, nrhs);
  a.err = ctx->d_status.as<int>() + 1;
  a.wait_cycles = ctx->wait_cycles;
  a.split = ctx->prec == LSW_PREC_SPLIT ? 1 : 0;
  a.cluster = fitting_cluster(ctx, a.max_slots, front_cluster(a.item_count, ctx->nsm, ctx->max_cluster));
  cudaError_t e = dbl ? launch_front<double>(a, ctx->max_ny, ctx->max_nx, st) : launch_front<float>(a, ctx->max_ny, ctx->max_nx, st);
  CK(e, "local solve kernel");
  ctx->launches += 2;
  return check_kernel_err(ctx, st);
}

}  // extern "C"
