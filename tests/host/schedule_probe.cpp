// Checks the sweep schedule of the library on the CPU (compiled with the
// library's csrc/geometry.cpp, no GPU needed).
//
//   schedule_probe N m p nrhs [slots]
//
// (slots: 4, 8 or 16 right-hand-side slots per item imposed on every launch,
// as the tuner's candidates and LSW_FRONT_SHAPE impose them; default: the
// cost model's choice)
// Builds the one-launch-per-step schedule and the per-sweep schedule of an
// N x N checkerboard of m-element cells with p PML elements, then checks:
//  1. both schedules hold the same cell solves: per (stage, step, cell) the
//     same slots (kind, shift, right-hand side, source lines, trace reads and
//     writes), every slot exactly once;
//  2. every output group of the per-sweep schedule holds slots of one
//     (right-hand side, shift) and addresses the output plane of its sweep;
//  3. the per-sweep launches, ordered as the library launches them (stage 1;
//     each sweep's launches in order on its own stream; an L-sweep's step dd
//     after its two producing stage-2 sweeps' front min(dd + 1, N - 1)), have
//     no race: any two launches that touch the same trace line, output region
//     or scratch range, one of them writing, are ordered.
// Prints "ok launches=<per-sweep> steps=<one per step>" and exits 0, or prints
// each violation and exits 1.
#include "internal.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <set>
#include <tuple>
#include <vector>

using namespace lsw;

static std::vector<DevCell> make_cells(int N, int m, int p) {
  std::vector<DevCell> cells;
  for (int I = 0; I < N; ++I)
    for (int J = 0; J < N; ++J) {
      const DirGeom gx = dir_geom(J, N, m, p), gy = dir_geom(I, N, m, p);
      DevCell c{};
      c.I = I; c.J = J;
      c.nx = gx.nd; c.ny = gy.nd;
      c.lox = gx.lo; c.loy = gy.lo;
      c.ldn = (gy.nd + 3) & ~3;
      for (int s = 0; s < 2; ++s) {
        for (int l = 0; l < 4; ++l) { c.lx[s][l] = gx.lines[s][l]; c.ly[s][l] = gy.lines[s][l]; }
        c.ownx[s][0] = gx.own[s][0]; c.ownx[s][1] = gx.own[s][1];
        c.owny[s][0] = gy.own[s][0]; c.owny[s][1] = gy.own[s][1];
      }
      cells.push_back(c);
    }
  return cells;
}

struct Built {
  std::vector<Front> fronts;
  std::vector<DevItem> items;
  std::vector<DevSlot> slots;
  std::vector<DevGroup> groups;
};

static Built build(const std::vector<DevCell>& cells, int N, int nrhs, bool lanes, long long LP, long long n2,
                   int slots) {
  FrontPlan plan;
  if (slots > 0) plan.forced_r.assign(16 * (size_t)N + 16, slots);
  plan.max_clusters[1] = 76; plan.max_clusters[2] = 38; plan.max_clusters[4] = 19;
  for (int r = 1; r <= 16; ++r) plan.fit_mask[r] = (1 << 1) | (1 << 2) | (1 << 4);
  plan.lanes = lanes;
  Built b;
  build_schedule(cells, N, nrhs, plan, LP, b.fronts, b.items, b.slots, b.groups, n2);
  return b;
}

typedef std::tuple<int, int, int, int, int, int, int, int, int, int, long long, long long, long long, long long,
                   long long, long long, long long, long long, long long, long long, long long, long long>
    SlotKey;
static SlotKey slot_key(const DevSlot& s) {
  return SlotKey(s.kind, s.shift, s.rhs, s.xo, s.xi, s.dx, s.yo, s.yi, s.dy, s.overwrite, s.in_lr0, s.in_lr1,
                 s.in_ud0, s.in_ud1, s.lr_out[0], s.lr_out[1], s.lr_out[2], s.lr_out[3], s.ud_out[0], s.ud_out[1],
                 s.ud_out[2], s.ud_out[3]);
}

static std::map<std::tuple<int, int, int>, std::multiset<SlotKey>> solves(const Built& b) {
  std::map<std::tuple<int, int, int>, std::multiset<SlotKey>> out;
  for (const Front& f : b.fronts)
    for (int i = f.item_begin; i < f.item_begin + f.item_count; ++i) {
      const DevItem& it = b.items[i];
      for (int q = 0; q < it.slot_count; ++q)
        out[std::make_tuple(f.stage, f.step, it.cell)].insert(slot_key(b.slots[it.slot_begin + q]));
    }
  return out;
}

// A launch (or the part of one front launched on one stream): items [i0, i1)
// of front `front`, after the units in `pred`.
struct Unit {
  int front, i0, i1;
  std::vector<int> pred;
};

// Every two units that touch the same trace line, output region or scratch
// range, one of them writing, must be ordered (one an ancestor of the other).
template <typename Report>
static void check_races(const Built& b, const std::vector<DevCell>& cells, const std::vector<Unit>& units,
                        Report& report) {
  const int L = (int)units.size();
  std::vector<std::vector<char>> anc(L, std::vector<char>(L, 0));
  for (int i = 0; i < L; ++i)
    for (int q : units[i].pred) {
      if (q >= i) report("edge against the launch order", q, i, 0);
      anc[i][q] = 1;
      for (int k = 0; k < L; ++k)
        if (anc[q][k]) anc[i][k] = 1;
    }
  auto ordered = [&](int x, int y) { return x == y || anc[x][y] || anc[y][x]; };
  // accesses: (unit, write?) per trace line, output region and scratch element range
  std::map<long long, std::vector<std::pair<int, bool>>> trace, outreg;
  std::vector<std::tuple<long long, long long, int>> scratch;
  for (int i = 0; i < L; ++i) {
    for (int j = units[i].i0; j < units[i].i1; ++j) {
      const DevItem& it = b.items[j];
      const DevCell& c = cells[it.cell];
      for (int q = 0; q < it.slot_count; ++q) {
        const DevSlot& s = b.slots[it.slot_begin + q];
        for (long long r : {s.in_lr0, s.in_lr1, s.in_ud0, s.in_ud1})
          if (r >= 0) trace[r].push_back({i, false});
        for (int l = 0; l < s.n_lr; ++l) trace[s.lr_out[l]].push_back({i, true});
        for (int l = 0; l < s.n_ud; ++l) trace[s.ud_out[l]].push_back({i, true});
      }
      for (int g = 0; g < it.group_count; ++g) {
        const DevGroup& G = b.groups[it.group_begin + g];
        if (G.out_off >= 0) outreg[G.out_off + it.cell].push_back({i, true});   // owned sets of cells are disjoint
      }
      const long long len = (long long)(c.nx + 1) * front_rpad(it.slot_count) * c.ny;
      scratch.emplace_back(it.scratch_off, it.scratch_off + len, i);
    }
  }
  for (auto* acc : {&trace, &outreg})
    for (const auto& kv : *acc) {
      const auto& v = kv.second;
      for (size_t x = 0; x < v.size(); ++x)
        for (size_t y = x + 1; y < v.size(); ++y)
          if ((v[x].second || v[y].second) && !ordered(v[x].first, v[y].first))
            report(acc == &trace ? "unordered trace-line access" : "unordered output write", units[v[x].first].front,
                   units[v[y].first].front, kv.first);
    }
  std::sort(scratch.begin(), scratch.end());
  for (size_t x = 0; x < scratch.size(); ++x)
    for (size_t y = x + 1; y < scratch.size() && std::get<0>(scratch[y]) < std::get<1>(scratch[x]); ++y)
      if (!ordered(std::get<2>(scratch[x]), std::get<2>(scratch[y])))
        report("unordered scratch overlap", units[std::get<2>(scratch[x])].front,
               units[std::get<2>(scratch[y])].front, std::get<0>(scratch[y]));
}

int main(int argc, char** argv) {
  if (argc != 5 && argc != 6) {
    std::fprintf(stderr, "usage: schedule_probe N m p nrhs [slots]\n");
    return 2;
  }
  const int slots = argc == 6 ? std::atoi(argv[5]) : 0;
  const int N = std::atoi(argv[1]), m = std::atoi(argv[2]), p = std::atoi(argv[3]), nrhs = std::atoi(argv[4]);
  const std::vector<DevCell> cells = make_cells(N, m, p);
  int max_n = 0;
  for (const DevCell& c : cells) max_n = std::max(max_n, std::max(c.nx, c.ny));
  const long long LP = ((max_n + 7) / 8) * 8;
  const long long n_dof = (long long)N * m + N - 1 + 2 * p - 1;
  const long long n2 = n_dof * n_dof;
  const Built one = build(cells, N, nrhs, false, LP, n2, slots);
  const Built per = build(cells, N, nrhs, true, LP, n2, slots);
  int bad = 0;
  auto report = [&](const char* what, long long a, long long b, long long key) {
    if (bad < 40) std::printf("%s: launches %lld and %lld, key %lld\n", what, a, b, key);
    ++bad;
  };

  // 1. the same cell solves
  if (solves(one) != solves(per)) report("the two schedules hold different cell solves", -1, -1, 0);

  // 2. output groups: one (rhs, shift) per group, the plane of the sweep
  for (const Front& f : per.fronts) {
    const int plane = f.lane < 0 ? 0 : (f.lane < 4 ? f.lane : kLanePlane3[f.lane - 4]);
    for (int i = f.item_begin; i < f.item_begin + f.item_count; ++i) {
      const DevItem& it = per.items[i];
      for (int g = 0; g < it.group_count; ++g) {
        const DevGroup& G = per.groups[it.group_begin + g];
        for (int q = 0; q < G.slot_count; ++q) {
          const DevSlot& s = per.slots[it.slot_begin + G.slot_begin + q];
          const long long want = (((long long)s.rhs * kLanePlanes + plane) * 4 + s.shift) * n2;
          if (s.shift != G.shift || G.out_off != want) report("output group address", f.lane, f.step, G.out_off);
        }
      }
    }
  }

  // 3. the per-sweep launches as the library orders them, and the races that
  // order allows
  std::vector<Unit> units;
  {
    int last_stage1 = -1;
    bool forked = false;
    std::vector<int> last_of_lane(8, -1);
    std::map<std::pair<int, int>, int> stage2_launch;   // (sweep, t) -> unit
    for (int i = 0; i < (int)per.fronts.size(); ++i) {
      const Front& f = per.fronts[i];
      Unit u{i, f.item_begin, f.item_begin + f.item_count, {}};
      const int id = (int)units.size();
      if (f.lane < 0) {
        if (last_stage1 >= 0) u.pred.push_back(last_stage1);
        if (forked || f.stage != 1) report("launch on the main stream after the fork", i, -1, f.stage);
        last_stage1 = id;
        units.push_back(u);
        continue;
      }
      forked = true;
      const int prev = last_of_lane[f.lane] >= 0 ? last_of_lane[f.lane] : last_stage1;
      if (prev >= 0) u.pred.push_back(prev);
      if (f.stage == 2) stage2_launch[{f.lane, f.step}] = id;
      if (f.stage == 3) {
        const int w = f.lane - 4, t = std::min(f.step + 1, N - 1);
        for (int src : {kLaneProducerLR[w], kLaneProducerUD[w]}) {
          auto it = stage2_launch.find({src, t});
          if (it == stage2_launch.end()) report("missing producer launch", i, src, t);
          else u.pred.push_back(it->second);
        }
      }
      last_of_lane[f.lane] = id;
      units.push_back(u);
    }
  }
  check_races(per, cells, units, report);
  const int L = (int)units.size();

  // 4. one launch per step with the per-shift streams of a captured apply: a
  // front whose items each belong to one shifted decomposition runs as one
  // launch per shift, shift s on stream s (shift 0 on the main stream), the
  // side streams forked from the main stream before the first such front; a
  // front with an item that mixes shifts joins every stream and runs alone on
  // the main stream
  std::vector<Unit> sunits;
  {
    std::vector<int> last(4, -1);          // last unit on each stream
    std::vector<std::vector<int>> pending(4);
    bool forked = false;
    auto add = [&](int s, Unit u) {
      if (last[s] >= 0) u.pred.push_back(last[s]);
      for (int q : pending[s]) u.pred.push_back(q);
      pending[s].clear();
      last[s] = (int)sunits.size();
      sunits.push_back(u);
    };
    for (int i = 0; i < (int)one.fronts.size(); ++i) {
      const Front& f = one.fronts[i];
      if (f.item_count <= 0) continue;
      if (f.mixed) {
        if (forked) {                      // join: the main stream waits for every side stream
          for (int s = 1; s < 4; ++s)
            if (last[s] >= 0) pending[0].push_back(last[s]);
          forked = false;
        }
        add(0, Unit{i, f.item_begin, f.item_begin + f.item_count, {}});
        continue;
      }
      if (!forked) {                       // fork: the side streams wait for the main stream
        for (int s = 1; s < 4; ++s)
          if (last[0] >= 0) pending[s].push_back(last[0]);
        forked = true;
      }
      for (int sh = 0; sh < 4; ++sh)
        if (f.sh_begin[sh + 1] > f.sh_begin[sh])
          add(sh, Unit{i, f.item_begin + f.sh_begin[sh], f.item_begin + f.sh_begin[sh + 1], {}});
    }
  }
  check_races(one, cells, sunits, report);
  if (bad) return 1;
  std::printf("ok launches=%d steps=%d shift_launches=%d\n", L, (int)one.fronts.size(), (int)sunits.size());
  return 0;
}
