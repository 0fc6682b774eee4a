// Internal types of the GB300 L-sweeps library: cell geometry on the integer
// grid, device cell table, sweep-front descriptors, and the kernel launchers.
#pragma once
#include "lsweeps.h"
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include <map>

namespace lsw {

// ---------------------------------------------------------------------------
// Geometry along one direction for cell index J (column J along x, row I along
// y).  Integer-grid restatement of DDCheckerboard::setUp (DDCheckerboard.cpp:
// 214-330, 388-419) and SubdomainStructured::assignIndexSets (1019-1116) for
// Order = 2 (trace thickness 1, DDCheckerboard.cpp:104):
//   global nodes k = 0..n_g, k_a = (m+1) J, k_b = k_a + m;
//   interior domain [k_a - 2, k_b + 4], clipped to [0, n_g] at the boundary;
//   local DOF i <-> global DOF lo + i; nd = (hi - lo) + 2p - 1 DOFs;
//   traces (non-shifted) t0 = k_a-1, t1 = k_a, tN = k_b, tNP = k_b+1,
//   (shifted) the same + 2; owned [k_a, k_b] (+2 shifted), open at the
//   domain boundary.
// ---------------------------------------------------------------------------
struct DirGeom {
  int lo;            // global node index of the interior-domain start == global DOF of local 0
  int nel;           // interior elements of the cell
  int nd;            // DOFs per side: nel + 2p - 1
  int lines[2][4];   // local index of t0, t1, tN, tNP ([shift]); -1 if absent
  int own[2][2];     // owned local range [lo, hi] ([shift])
};
DirGeom dir_geom(int J, int N, int m, int p);
bool geom_valid(const lsw_geom* g, std::string* why);

// Separable coefficient profiles of the 5-point PML operator along one
// direction of a box with `nel` interior elements and p PML cells
// (PMLCubic2D.cpp:35-236; AssemblerHelmholtz2DFD.cpp:371-457):
//   lo[k]  coupling to k-1  (-Lambda/h^2 + beta/(2h))
//   hi[k]  coupling to k+1  (-Lambda/h^2 - beta/(2h))
//   dg[k]  diagonal share    2 Lambda / h^2
struct Profile1D {
  std::vector<double> lo_re, lo_im, hi_re, hi_im, dg_re, dg_im;
};
Profile1D make_profile(int nel, int p, double h, double C);

// ---------------------------------------------------------------------------
// Device cell table.
// ---------------------------------------------------------------------------
struct DevCell {
  int I, J;
  int nx, ny;          // x-lines (block count) and points per line (block size)
  int lox, loy;        // global DOF of local (0, 0)
  int ldn;             // leading dimension of a factor block (column-major)
  int pad0;
  int lx[2][4], ly[2][4];
  int ownx[2][2], owny[2][2];
  long long fac_off;   // element offset of block 0 in the factor pool
  long long prof_off;  // offset into the profile array: x-profiles (3*nx), then y (3*ny)
};

enum SlotKind : int {
  SK_VOLUME = 0,   // stage 1: window of the global input restricted to the owned set
  SK_DIR_X = 1,    // two-line equivalent source on x-lines (left/right sweeps)
  SK_DIR_Y = 2,    // two-line equivalent source on y-rows (up/down sweeps)
  SK_CORNER = 3,   // L-shaped equivalent source (stage 3)
  SK_CELLVEC = 4   // full cell vector (LocalLinearSolver::solve)
};

// One right-hand side of a cell solve inside a sweep front.
struct DevSlot {
  int kind, shift, rhs, pad0;
  int xo, xi, dx, yo, yi, dy;   // outer/inner source lines and their inward direction
  int overwrite;                // L-sweep: trace0 lines take the incoming values (see DDCheckerboard.cpp:2520-2526)
  int n_lr, n_ud;
  int lr_line[4], ud_line[4];   // outgoing trace lines (local index)
  long long in_lr0, in_lr1, in_ud0, in_ud1;   // trace-pool offsets of incoming lines, -1 if none
  long long lr_out[4], ud_out[4];             // trace-pool offsets of outgoing lines
};

// A set of slots of one item that accumulate into the same output vector.
struct DevGroup {
  int slot_begin, slot_count, shift, pad0;
  long long out_off;   // element offset of the output vector in the out pool; -1: none
};

struct DevItem {
  int cell, slot_begin, slot_count, group_begin, group_count, pad0;
  long long scratch_off;   // element offset of the item's forward-sweep storage
};

// A launch = one sweep front.
struct Front {
  int item_begin, item_count;
  long long scratch_elems;
  int max_slots;
  int cluster;            // CTAs per item chosen for this front
  int slots_cap = 0;      // slots per item at most (the planner's r)
  float tuned_ms = -1.f;  // the tuner's timing of this shape, -1 when the cost model chose it
  bool tc = false;        // complex64 line products on the tensor cores
  bool mixed = false;     // an item mixes shifted decompositions: the front is one launch
  int sh_begin[5] = {0, 0, 0, 0, 0};   // items of shift s: [sh_begin[s], sh_begin[s + 1]) (not mixed)
  // the sweep step this launch belongs to: stage (1, 2, 3) and step (stage 2:
  // column / row t = 1..N-1; stage 3: anti-diagonal 0..2N-4); with per-sweep
  // launches, the sweep (lane): stage 2 right, left, up, down = 0..3, stage 3
  // BL2TR, TR2BL, BR2TL, TL2BR = 4..7; -1 when the launch holds every sweep
  int stage = 1, step = 0, lane = -1;
};

// Per-sweep launches.  The four stage-2 sweeps of DDCheckerboard::applySweep
// read and write disjoint trace lines, and so do the four L-sweeps of stage
// 3; an L-sweep's step dd reads only traces that stage 1, its own earlier
// steps and two stage-2 sweeps (its producers) wrote, the latter by their
// front min(dd + 1, N - 1).  With one launch per (step, sweep), each sweep
// runs as its own chain and the L-sweeps start while stage 2 still runs.
// Outputs: one plane per stage-2 sweep (per right-hand side and shift); an
// L-sweep adds into the plane of one of its producers, whose writes to any
// cell it reaches are ordered before it by that wait.
constexpr int kLanePlanes = 4;
// stage-3 lane w (0..3): its two producing stage-2 sweeps and its output plane
constexpr int kLaneProducerLR[4] = {2, 3, 2, 3};   // up, down, up, down (TS_LRUP / TS_LRDOWN)
constexpr int kLaneProducerUD[4] = {0, 1, 1, 0};   // right, left, left, right (TS_UDRIGHT / TS_UDLEFT)
constexpr int kLanePlane3[4] = {2, 3, 1, 0};       // BL2TR->up, TR2BL->down, BR2TL->left, TL2BR->right

// What the front planner knows about the device: how many clusters of each
// size (1, 2, 4, 8) are resident at once, and a per-line cost model of the
// sweep-front kernel fitted to front timings on GB300 over every (slots per
// item, cluster size) choice of a C2 apply: cycles per line =
//   line_overhead + slot_cost R + (col_cost + col_slot_cost R) x columns per CTA,
// with a bandwidth floor (factor bytes / bytes_per_cycle).
struct FrontPlan {
  // indexed by the CTAs per half (1, 2, 4): resident clusters of twice that many CTAs
  int max_clusters[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  int cluster_cap = 4;       // CTAs per half
  int fit_mask[17] = {0};    // per padded slot count: bit CL set where the launch fits in shared memory
  int rmax = 16;
  int csize = 8;             // bytes per complex value of the factors
  double line_overhead = 1800.0;
  double slot_cost = 250.0;
  double col_cost = 25.0;
  double col_slot_cost = 10.0;
  double bytes_per_cycle = 3300.0;
  // shapes fixed per front (slots per item, CTAs per half), e.g. by the
  // autotuner; an entry of 0, a missing entry or a shape that does not fit
  // leaves the front to the cost model
  std::vector<int> forced_r, forced_cl;
  // items may run with tensor-core line products (8 or 16 slots, fewer
  // padded): their forward storage is sized for that many slots
  bool tc_scratch = false;
  // one launch per (step, sweep) instead of one per step (see kLanePlanes);
  // the cost model then counts a stage-2 / stage-3 launch as sharing the GPU
  // with `lane_concurrency` others of its size
  bool lanes = false;
  double lane_concurrency = 4.0;
};

struct Schedule {
  int nrhs = 0;
  bool lanes = false;     // per-sweep launches, kLanePlanes output planes
  std::vector<Front> fronts;
  DevItem* d_items = nullptr;
  DevSlot* d_slots = nullptr;
  DevGroup* d_groups = nullptr;
  long long scratch_elems = 0;   // max over fronts
  int max_slots = 0;
};

// Build the sweep schedule (stage 1, N-1 stage-2 fronts, 2N-3 stage-3 fronts,
// all four shifted decompositions and nrhs right-hand sides in every front;
// with plan.lanes every stage-2 / stage-3 front is split into one launch per
// sweep, in the order stage 1, stage 2 (t, then sweep), stage 3 (dd, then sweep)).
// Output groups address the out pool as [rhs][plane][shift] n_dof2 with one
// plane, or kLanePlanes planes with plan.lanes.
void build_schedule(const std::vector<DevCell>& cells, int N, int nrhs, const FrontPlan& plan, long long LP,
                    std::vector<Front>& fronts, std::vector<DevItem>& items, std::vector<DevSlot>& slots,
                    std::vector<DevGroup>& groups, long long n_dof2);

// Trace pool index of (rhs, shift, cell, set, line), in elements of stride LP.
enum TraceSet : int { TS_LR = 0, TS_UD = 1, TS_LRUP = 2, TS_LRDOWN = 3, TS_UDRIGHT = 4, TS_UDLEFT = 5 };
inline long long trace_off(int rhs, int s, int c, int set, int line, int ncell, long long LP) {
  return ((((long long)rhs * 4 + s) * ncell + c) * 6 + set) * 4 * LP + (long long)line * LP;
}

// ---------------------------------------------------------------------------
// Kernel launchers (defined in the .cu files).
// ---------------------------------------------------------------------------
struct FrontArgs {
  const DevCell* cells;
  const DevItem* items;
  const DevSlot* slots;
  const DevGroup* groups;
  const void* fac;        // factor pool (cx_t<T>)
  const double2* prof;    // profiles
  void* traces;           // trace pool (cx_t<T>)
  void* outs;             // out pool (cx_t<T>)
  void* scratch;          // forward storage (cx_t<T>)
  const double2* x_in;    // global input vectors (VOLUME) or cell vectors (CELLVEC)
  // when set, the VOLUME input is *x_ref (a device-side address table, so that
  // one captured launch sequence serves any input vector)
  const double2* const* x_ref;
  long long x_stride;
  double2* x_out;         // CELLVEC output
  long long out_stride;
  int n_dof, N, m, p;
  int item_count;
  int max_slots;          // largest slot count of an item in this launch
  int* err;               // bit 1: a bounded wait timed out
  int cluster;            // CTAs per item (thread-block cluster size)
  int stages;             // shared-memory ring depth (set by the launcher)
  int chunk;              // factor columns per streamed chunk (set by the launcher)
  int ksw;                // consumer column slices (set by the launcher)
  int split;              // factors hold bf16 hi/lo terms; the matvec runs on mma.sync
  int tc;                 // complex64 line products on the tensor cores (tcgen05, 8 or 16 slots)
  long long wait_cycles;  // bounded-wait limit in clock cycles
};
// CTAs per half of an item (the item's cluster holds two halves) for a
// front of `items` cell solves on `nsm` SMs, with at most `max_cta` CTAs per item
inline int front_cluster(int items, int nsm, int max_cta) {
  int cl = 4;
  while (cl > 1 && (items * 2 * cl > nsm || 2 * cl > max_cta)) cl >>= 1;
  return cl;
}

template <typename T> cudaError_t launch_front(const FrontArgs& a, int max_ny, int max_nx, cudaStream_t st);
// clusters of `cluster` CTAs of the sweep-front kernel resident at once (one CTA per SM)
int front_max_clusters(bool dbl, int cluster);
int front_rmax(bool dbl);
int front_rpad(int n);
// bit CL (1, 2, 4) set where items of `slots` slots on clusters of 2 CL CTAs fit in shared memory
int front_fit_mask(bool dbl, bool split, int max_ny, int max_nx, int slots, bool tc = false);
// slots of a tensor-core item (8 or 16) for items of at most n slots
int front_tc_slots(int n);
// split: write every factor entry as bf16 hi/lo terms; `prev` then holds the
// previous FP32 block of each cell's two half chains (2 x ny x ldn complex per
// cell) for the Schur recurrences.  lookahead: factor each next panel while
// the current block's update runs on the other warps.
template <typename T> cudaError_t launch_factorize(const DevCell* cells, int ncell, const double2* prof,
                                                   const double* mgrid, int n_dof, double omega2,
                                                   void* fac, void* prev, int max_ny, int* status,
                                                   cudaStream_t st, bool split, bool lookahead,
                                                   long long wait_cycles);
// one bounded wait on a barrier that nothing completes (bit 1 of *err when it runs out)
cudaError_t launch_wait_probe(int* err, long long limit_cycles, cudaStream_t st);
size_t factor_smem_bytes(int ny, bool dbl);
// complex64 / split factorisation with the working matrix in tensor memory and
// each block's update on the tensor cores (3 x TF32 tcgen05.mma); cells of at
// most 192 DOFs per side
bool factorize_tc_supported(int max_ny);
cudaError_t launch_factorize_tc(const DevCell* cells, int ncell, const double2* prof, const double* mgrid, int n_dof,
                                double omega2, void* fac, void* prev, int max_ny, int* status, cudaStream_t st,
                                bool split, long long wait_cycles);

cudaError_t launch_apply_A(const double2* x, double2* y, int nrhs, int n_dof, const double2* gprof,
                           const double* mgrid, double omega2, cudaStream_t st);
template <typename T> cudaError_t launch_combine(const void* outs, double2* y, int nrhs, long long n2,
                                                 cudaStream_t st);
cudaError_t launch_rhs(double2* b, int n_dof, int p, double h, const double* src, const double* amp,
                       int nsrc, double eps, cudaStream_t st);
// combine into *y_ref (the output address read from device memory); the out
// pool holds `planes` planes of the four shifted outputs per right-hand side
template <typename T> cudaError_t launch_combine_ref(const void* outs, double2* const* y_ref, int nrhs, long long n2,
                                                     int planes, cudaStream_t st);
// ref[0] = x, ref[1] = y (the address table of a captured apply)
cudaError_t launch_set_refs(const void** ref, const void* x, void* y, cudaStream_t st);

// FP64 Krylov helpers; results of reductions land in device memory.
cudaError_t launch_dot(const double2* a, const double2* b, long long n, int nvec, long long stride,
                       double2* partial, double2* out, cudaStream_t st);   // out[v] = sum conj(a) b
cudaError_t launch_norm2(const double2* a, long long n, int nvec, long long stride, double* partial,
                         double* out, cudaStream_t st);                   // out[v] = sum |a|^2
// y[v] = y[v] - coef[v] * x[v]; and (optionally) partial dot of conj(y_new) . z (dotout)
cudaError_t launch_axpy_dot(double2* y, const double2* x, const double2* coef, const double2* z,
                            long long n, int nvec, long long stride, double2* partial, double2* dotout,
                            int conj_first_y, cudaStream_t st);
cudaError_t launch_scale(double2* y, const double2* x, const double2* coef, int invert, long long n,
                         int nvec, long long stride, cudaStream_t st);    // y = x*coef or x/coef
cudaError_t launch_lincomb(double2* y, const double2* basis, long long basis_stride_vec,
                           long long basis_stride_rhs, const double2* coef, int ncoef, long long n,
                           int nvec, long long y_stride, cudaStream_t st); // y[v] += sum_i coef[v][i] basis[i][v]
cudaError_t launch_sub(double2* y, const double2* a, const double2* b, long long n, cudaStream_t st);
// FGMRES(m) Hessenberg least squares on the device, one thread per right-hand side
cudaError_t launch_fgmres_init(int nv, int m, const double* r2, const double* bn, double tol, double2* sc, double2* g,
                               double* rel, int* active, cudaStream_t st);
cudaError_t launch_fgmres_givens(int j, int nv, int m, const double2* h, double2* H, double2* cs, double2* sn,
                                 double2* g, double2* sc, double* est, const double* bn, cudaStream_t st);
cudaError_t launch_fgmres_solve(int ncol, int nv, int m, const double2* H, const double2* g, const int* active,
                                double2* coef, cudaStream_t st);

}  // namespace lsw
