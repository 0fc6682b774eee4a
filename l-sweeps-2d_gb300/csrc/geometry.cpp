// Host-side geometry of the checkerboard decomposition, PML coefficient
// profiles and the sweep-front schedule.
#include "internal.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <stdexcept>
#include <tuple>

namespace lsw {

DirGeom dir_geom(int J, int N, int m, int p) {
  // DDCheckerboard::setUp, DDCheckerboard.cpp:214-330: a = (m+1) J h, b = a + m h,
  // left extension 2 tt h (J > 0), right extension 4 tt h (J < N-1), tt = 1.
  DirGeom g{};
  const int n_g = N * m + N - 1;
  const int ka = (m + 1) * J, kb = ka + m;
  const int lo = J > 0 ? ka - 2 : 0;
  const int hi = J < N - 1 ? kb + 4 : n_g;
  g.lo = lo;
  g.nel = hi - lo;
  g.nd = g.nel + 2 * p - 1;
  auto loc = [&](int node) { return node - lo + p - 1; };
  for (int s = 0; s < 2; ++s) {
    const int off = 2 * s;  // shifted traces sit two rows further in (DDCheckerboard.cpp:227-230, 253-257)
    g.lines[s][0] = J > 0 ? loc(ka - 1 + off) : -1;
    g.lines[s][1] = J > 0 ? loc(ka + off) : -1;
    g.lines[s][2] = J < N - 1 ? loc(kb + off) : -1;
    g.lines[s][3] = J < N - 1 ? loc(kb + 1 + off) : -1;
    // owned DOFs: trace1 .. traceN, open where the cell touches the domain boundary
    // (mValsToKeep*, DDCheckerboard.cpp:446-634)
    g.own[s][0] = J > 0 ? loc(ka + off) : 0;
    g.own[s][1] = J < N - 1 ? loc(kb + off) : g.nd - 1;
  }
  return g;
}

bool geom_valid(const lsw_geom* g, std::string* why) {
  if (!g) { *why = "geometry is NULL"; return false; }
  if (g->order != 2) { *why = "only Order = 2 (5-point stencil) is supported"; return false; }
  if (g->n_cells < 1) { *why = "n_cells must be >= 1"; return false; }
  if (g->n_els_in_cell <= 4) { *why = "Not enough elements in cell (need > 4, DDCheckerboard.cpp:106-111)"; return false; }
  if (g->pml < 1) { *why = "pml must be >= 1"; return false; }
  if (!(g->h > 0.0) || !std::isfinite(g->h)) { *why = "h must be positive"; return false; }
  int nd = 0;
  for (int J = 0; J < g->n_cells; ++J) nd = std::max(nd, dir_geom(J, g->n_cells, g->n_els_in_cell, g->pml).nd);
  if (nd > 192) { *why = "cell side exceeds 192 DOFs (m + 6 + 2p - 1 <= 192)"; return false; }
  return true;
}

Profile1D make_profile(int nel, int p, double h, double C) {
  // sigma = C ((dist into PML)/delta)^3, delta = p h; alpha = 1/(1 + i sigma),
  // alpha' = -i sigma' / (1 + i sigma)^2 (PMLCubic2D.cpp:67-236); Lambda = alpha^2
  // (diffusion), beta = alpha' alpha (convection); second/first derivative
  // stencils [1 -2 1]/h^2 and [-1 0 1]/(2h) (FiniteDifferences.cpp:57-122).
  const int nd = nel + 2 * p - 1;
  Profile1D pr;
  pr.lo_re.resize(nd); pr.lo_im.resize(nd); pr.hi_re.resize(nd); pr.hi_im.resize(nd);
  pr.dg_re.resize(nd); pr.dg_im.resize(nd);
  const std::complex<double> I(0.0, 1.0);
  const double p3 = double(p) * p * p;
  for (int i = 0; i < nd; ++i) {
    const int q = i + 1;  // nodes from the start of the computational domain
    double sg = 0.0, dsg = 0.0;
    if (q < p) {
      const double d = double(p - q);
      sg = C * std::pow(d / p, 3.0);
      dsg = -3.0 * C * d * d / (p3 * h);
    } else if (q > p + nel) {
      const double d = double(q - p - nel);
      sg = C * std::pow(d / p, 3.0);
      dsg = 3.0 * C * d * d / (p3 * h);
    }
    const std::complex<double> a = 1.0 / (1.0 + I * sg);
    const std::complex<double> ad = -I * dsg / std::pow(1.0 + I * sg, 2.0);
    const std::complex<double> lam = std::pow(a, 2.0);
    const std::complex<double> beta = ad * a;
    const double h2 = h * h;
    const std::complex<double> lo = -lam / h2 + beta / (2.0 * h);
    const std::complex<double> hi = -lam / h2 - beta / (2.0 * h);
    const std::complex<double> dg = 2.0 * lam / h2;
    pr.lo_re[i] = lo.real(); pr.lo_im[i] = lo.imag();
    pr.hi_re[i] = hi.real(); pr.hi_im[i] = hi.imag();
    pr.dg_re[i] = dg.real(); pr.dg_im[i] = dg.imag();
  }
  return pr;
}

// ---------------------------------------------------------------------------
// Schedule.  Restates the cell visiting order of DDCheckerboard::applySweep
// (DDCheckerboard.cpp:812-880): stage 1 (addLocSol) is one front; the four
// stage-2 sweeps (addRight/Left/Up/DownSweep) advance one column/row per
// front; the four stage-3 L-sweeps (addBL2TR/TR2BL/BR2TL/TL2BRSweep) advance
// one anti-diagonal per front.  The four shifted decompositions of
// applyPrecond (687-739) and every right-hand side share each front.
// ---------------------------------------------------------------------------
// Slots of an item as the sweep kernel instantiates them: at most 8
// (complex128) or 16, padded to 1, 2, 4, 8, 12 or 16; 8 or 16 on the tensor cores.
int front_rmax(bool dbl) { return dbl ? 8 : 16; }
int front_tc_slots(int n) { return n <= 8 ? 8 : 16; }
int front_rpad(int n) { return n <= 1 ? 1 : n <= 2 ? 2 : n <= 4 ? 4 : n <= 8 ? 8 : n <= 12 ? 12 : 16; }

namespace {

struct SlotSpec {
  DevSlot s;
  int rhs, shift, order;
};

DevSlot blank_slot() {
  DevSlot s{};
  s.in_lr0 = s.in_lr1 = s.in_ud0 = s.in_ud1 = -1;
  for (int i = 0; i < 4; ++i) { s.lr_out[i] = -1; s.ud_out[i] = -1; s.lr_line[i] = -1; s.ud_line[i] = -1; }
  return s;
}

}  // namespace

void build_schedule(const std::vector<DevCell>& cells, int N, int nrhs, const FrontPlan& plan, long long LP,
                    std::vector<Front>& fronts, std::vector<DevItem>& items, std::vector<DevSlot>& slots,
                    std::vector<DevGroup>& groups, long long n_dof2) {
  const int nc = (int)cells.size();
  auto cid = [&](int I, int J) { return I * N + J; };
  auto toff = [&](int rhs, int s, int c, int set, int line) { return trace_off(rhs, s, c, set, line, nc, LP); };

  // per front: map cell -> list of slot specs
  std::vector<std::map<int, std::vector<SlotSpec>>> fr;

  // ---- stage 1 ----
  {
    std::map<int, std::vector<SlotSpec>> f;
    for (int c = 0; c < nc; ++c) {
      const DevCell& cl = cells[c];
      for (int r = 0; r < nrhs; ++r)
        for (int s = 0; s < 4; ++s) {
          DevSlot d = blank_slot();
          d.kind = SK_VOLUME; d.shift = s; d.rhs = r;
          const int sx = s & 1, sy = (s >> 1) & 1;
          for (int l = 0; l < 4; ++l) {
            if (cl.lx[sx][l] >= 0) { d.lr_line[d.n_lr] = cl.lx[sx][l]; d.lr_out[d.n_lr] = toff(r, s, c, TS_LR, l); d.n_lr++; }
            if (cl.ly[sy][l] >= 0) { d.ud_line[d.n_ud] = cl.ly[sy][l]; d.ud_out[d.n_ud] = toff(r, s, c, TS_UD, l); d.n_ud++; }
          }
          f[c].push_back({d, r, s, 0});
        }
    }
    fr.push_back(std::move(f));
  }

  // ---- stage 2 ----
  for (int t = 1; t < N; ++t) {
    std::map<int, std::vector<SlotSpec>> f;
    for (int r = 0; r < nrhs; ++r)
      for (int s = 0; s < 4; ++s) {
        const int sx = s & 1, sy = (s >> 1) & 1;
        for (int k = 0; k < N; ++k) {
          // right sweep (addRightSweep 1168-1350): cell (k, t), source on trace0/trace1
          {
            const int c = cid(k, t), nb = cid(k, t - 1);
            const DevCell& cl = cells[c];
            DevSlot d = blank_slot();
            d.kind = SK_DIR_X; d.shift = s; d.rhs = r;
            d.xo = cl.lx[sx][0]; d.xi = cl.lx[sx][1]; d.dx = 1;
            d.in_lr0 = toff(r, s, nb, TS_LR, 2); d.in_lr1 = toff(r, s, nb, TS_LR, 3);
            for (int l = 0; l < 4; ++l)
              if (cl.ly[sy][l] >= 0) { d.ud_line[d.n_ud] = cl.ly[sy][l]; d.ud_out[d.n_ud] = toff(r, s, c, TS_UDRIGHT, l); d.n_ud++; }
            for (int l = 2; l < 4; ++l)
              if (cl.lx[sx][l] >= 0) { d.lr_line[d.n_lr] = cl.lx[sx][l]; d.lr_out[d.n_lr] = toff(r, s, c, TS_LR, l); d.n_lr++; }
            f[c].push_back({d, r, s, 0});
          }
          // left sweep (addLeftSweep 976-1164): cell (k, N-1-t), source on traceN/traceNP
          {
            const int J = N - 1 - t;
            const int c = cid(k, J), nb = cid(k, J + 1);
            const DevCell& cl = cells[c];
            DevSlot d = blank_slot();
            d.kind = SK_DIR_X; d.shift = s; d.rhs = r;
            d.xo = cl.lx[sx][3]; d.xi = cl.lx[sx][2]; d.dx = -1;
            d.in_lr0 = toff(r, s, nb, TS_LR, 1); d.in_lr1 = toff(r, s, nb, TS_LR, 0);
            for (int l = 0; l < 4; ++l)
              if (cl.ly[sy][l] >= 0) { d.ud_line[d.n_ud] = cl.ly[sy][l]; d.ud_out[d.n_ud] = toff(r, s, c, TS_UDLEFT, l); d.n_ud++; }
            for (int l = 0; l < 2; ++l)
              if (cl.lx[sx][l] >= 0) { d.lr_line[d.n_lr] = cl.lx[sx][l]; d.lr_out[d.n_lr] = toff(r, s, c, TS_LR, l); d.n_lr++; }
            f[c].push_back({d, r, s, 1});
          }
          // up sweep (addUpSweep 1544-1724): cell (t, k), source on trace0/trace1 rows
          {
            const int c = cid(t, k), nb = cid(t - 1, k);
            const DevCell& cl = cells[c];
            DevSlot d = blank_slot();
            d.kind = SK_DIR_Y; d.shift = s; d.rhs = r;
            d.yo = cl.ly[sy][0]; d.yi = cl.ly[sy][1]; d.dy = 1;
            d.in_ud0 = toff(r, s, nb, TS_UD, 2); d.in_ud1 = toff(r, s, nb, TS_UD, 3);
            for (int l = 0; l < 4; ++l)
              if (cl.lx[sx][l] >= 0) { d.lr_line[d.n_lr] = cl.lx[sx][l]; d.lr_out[d.n_lr] = toff(r, s, c, TS_LRUP, l); d.n_lr++; }
            for (int l = 2; l < 4; ++l)
              if (cl.ly[sy][l] >= 0) { d.ud_line[d.n_ud] = cl.ly[sy][l]; d.ud_out[d.n_ud] = toff(r, s, c, TS_UD, l); d.n_ud++; }
            f[c].push_back({d, r, s, 2});
          }
          // down sweep (addDownSweep 1353-1540): cell (N-1-t, k), source on traceN/traceNP rows
          {
            const int I = N - 1 - t;
            const int c = cid(I, k), nb = cid(I + 1, k);
            const DevCell& cl = cells[c];
            DevSlot d = blank_slot();
            d.kind = SK_DIR_Y; d.shift = s; d.rhs = r;
            d.yo = cl.ly[sy][3]; d.yi = cl.ly[sy][2]; d.dy = -1;
            d.in_ud0 = toff(r, s, nb, TS_UD, 1); d.in_ud1 = toff(r, s, nb, TS_UD, 0);
            for (int l = 0; l < 4; ++l)
              if (cl.lx[sx][l] >= 0) { d.lr_line[d.n_lr] = cl.lx[sx][l]; d.lr_out[d.n_lr] = toff(r, s, c, TS_LRDOWN, l); d.n_lr++; }
            for (int l = 0; l < 2; ++l)
              if (cl.ly[sy][l] >= 0) { d.ud_line[d.n_ud] = cl.ly[sy][l]; d.ud_out[d.n_ud] = toff(r, s, c, TS_UD, l); d.n_ud++; }
            f[c].push_back({d, r, s, 3});
          }
        }
      }
    fr.push_back(std::move(f));
  }

  // ---- stage 3 ----
  struct LS { int lrbuf, udbuf, xr, yt; };  // xr: incoming from the right, yt: from the top
  const LS lsw_[4] = {
      {TS_LRUP, TS_UDRIGHT, 0, 0},    // BL2TR (2393-2608)
      {TS_LRDOWN, TS_UDLEFT, 1, 1},   // TR2BL (1949-2170)
      {TS_LRUP, TS_UDLEFT, 1, 0},     // BR2TL (2173-2390)
      {TS_LRDOWN, TS_UDRIGHT, 0, 1},  // TL2BR (1727-1946)
  };
  for (int dd = 0; dd <= 2 * N - 4; ++dd) {
    std::map<int, std::vector<SlotSpec>> f;
    for (int r = 0; r < nrhs; ++r)
      for (int s = 0; s < 4; ++s) {
        const int sx = s & 1, sy = (s >> 1) & 1;
        for (int w = 0; w < 4; ++w) {
          const LS& L = lsw_[w];
          for (int I = 0; I < N; ++I)
            for (int J = 0; J < N; ++J) {
              const int ii = L.yt ? N - 1 - I : I;
              const int jj = L.xr ? N - 1 - J : J;
              if (ii < 1 || jj < 1 || ii + jj - 2 != dd) continue;
              const int c = cid(I, J);
              const DevCell& cl = cells[c];
              DevSlot d = blank_slot();
              d.kind = SK_CORNER; d.shift = s; d.rhs = r; d.overwrite = 1;
              if (!L.xr) {
                const int nb = cid(I, J - 1);
                d.xo = cl.lx[sx][0]; d.xi = cl.lx[sx][1]; d.dx = 1;
                d.in_lr0 = toff(r, s, nb, L.lrbuf, 2); d.in_lr1 = toff(r, s, nb, L.lrbuf, 3);
                for (int l = 2; l < 4; ++l)
                  if (cl.lx[sx][l] >= 0) { d.lr_line[d.n_lr] = cl.lx[sx][l]; d.lr_out[d.n_lr] = toff(r, s, c, L.lrbuf, l); d.n_lr++; }
              } else {
                const int nb = cid(I, J + 1);
                d.xo = cl.lx[sx][3]; d.xi = cl.lx[sx][2]; d.dx = -1;
                d.in_lr0 = toff(r, s, nb, L.lrbuf, 1); d.in_lr1 = toff(r, s, nb, L.lrbuf, 0);
                for (int l = 0; l < 2; ++l)
                  if (cl.lx[sx][l] >= 0) { d.lr_line[d.n_lr] = cl.lx[sx][l]; d.lr_out[d.n_lr] = toff(r, s, c, L.lrbuf, l); d.n_lr++; }
              }
              if (!L.yt) {
                const int nb = cid(I - 1, J);
                d.yo = cl.ly[sy][0]; d.yi = cl.ly[sy][1]; d.dy = 1;
                d.in_ud0 = toff(r, s, nb, L.udbuf, 2); d.in_ud1 = toff(r, s, nb, L.udbuf, 3);
                for (int l = 2; l < 4; ++l)
                  if (cl.ly[sy][l] >= 0) { d.ud_line[d.n_ud] = cl.ly[sy][l]; d.ud_out[d.n_ud] = toff(r, s, c, L.udbuf, l); d.n_ud++; }
              } else {
                const int nb = cid(I + 1, J);
                d.yo = cl.ly[sy][3]; d.yi = cl.ly[sy][2]; d.dy = -1;
                d.in_ud0 = toff(r, s, nb, L.udbuf, 1); d.in_ud1 = toff(r, s, nb, L.udbuf, 0);
                for (int l = 0; l < 2; ++l)
                  if (cl.ly[sy][l] >= 0) { d.ud_line[d.n_ud] = cl.ly[sy][l]; d.ud_out[d.n_ud] = toff(r, s, c, L.udbuf, l); d.n_ud++; }
              }
              f[c].push_back({d, r, s, w});
            }
        }
      }
    fr.push_back(std::move(f));
  }

  // ---- flatten into items ----
  // An item takes whole (rhs, shift) groups while they fit in r slots.  A
  // group holds at most 4 slots (the four sweep directions, or the four
  // L-sweeps, that reach one cell in one front), and the planner only tries
  // r >= 4, so no group is split over items: every owned output value and
  // every trace line is written by one item per front, in one order, and the
  // apply is deterministic (the output adds need no ordering between items).
  auto flatten = [&](std::vector<SlotSpec>& v, int r, auto&& emit) {
    size_t i = 0;
    while (i < v.size()) {
      std::vector<std::pair<size_t, size_t>> parts;
      int count = 0;
      while (i < v.size() && count < r) {
        size_t j = i;
        while (j < v.size() && v[j].rhs == v[i].rhs && v[j].shift == v[i].shift) ++j;
        const int gsz = int(j - i);
        if (count > 0 && count + gsz > r && gsz <= r) break;   // starts a fresh item whole
        if (count + gsz > r) j = i + (r - count);
        parts.emplace_back(i, j);
        count += int(j - i);
        i = j;
      }
      emit(parts, count);
    }
  };
  // ---- launches: one per front, or with plan.lanes one per (front, sweep) ----
  // fr[0] is stage 1, fr[1 .. N-1] stage 2 (t = 1 .. N-1), fr[N + dd] stage 3
  // (dd = 0 .. 2N-4); a slot's `order` is its sweep within the stage
  struct Launch {
    std::map<int, std::vector<SlotSpec>> cells;
    int stage = 1, step = 0, lane = -1;
  };
  std::vector<Launch> launches;
  for (size_t q = 0; q < fr.size(); ++q) {
    const int stage = q == 0 ? 1 : (q < (size_t)N ? 2 : 3);
    const int step = stage == 1 ? 0 : (stage == 2 ? (int)q : (int)q - N);
    if (!plan.lanes || stage == 1) {
      Launch L;
      L.cells = std::move(fr[q]);
      L.stage = stage; L.step = step;
      launches.push_back(std::move(L));
      continue;
    }
    Launch L[4];
    for (auto& kv : fr[q])
      for (const SlotSpec& sp : kv.second) L[sp.order].cells[kv.first].push_back(sp);
    for (int w = 0; w < 4; ++w) {
      L[w].stage = stage; L[w].step = step; L[w].lane = stage == 2 ? w : 4 + w;
      launches.push_back(std::move(L[w]));
    }
  }
  const int planes = plan.lanes ? kLanePlanes : 1;

  fronts.clear(); items.clear(); slots.clear(); groups.clear();
  for (size_t fidx = 0; fidx < launches.size(); ++fidx) {
    auto& f = launches[fidx].cells;
    const int stage = launches[fidx].stage, lane = launches[fidx].lane;
    // output plane of this launch's groups
    const int plane = lane < 0 ? 0 : (lane < 4 ? lane : kLanePlane3[lane - 4]);
    // with per-sweep launches a stage-2 / stage-3 launch shares the GPU with
    // the other sweeps' launches: the cost model counts it as that many
    const double conc = (plan.lanes && stage > 1) ? plan.lane_concurrency : 1.0;
    if (f.empty()) {
      Front F{(int)items.size(), 0, 0, 0, 1};
      F.slots_cap = plan.rmax;
      F.stage = stage; F.step = launches[fidx].step; F.lane = lane;
      F.mixed = true;
      for (int sh = 0; sh <= 4; ++sh) F.sh_begin[sh] = 0;
      fronts.push_back(F);
      continue;
    }
    // slots ordered by (shift, rhs): items of 8 or 16 slots merge the groups of
    // one shifted decomposition when there are several right-hand sides, so
    // that the front can run as one launch per shift (see below)
    for (auto& kv : f)
      std::stable_sort(kv.second.begin(), kv.second.end(), [](const SlotSpec& a, const SlotSpec& b) {
        return std::make_tuple(a.shift, a.rhs, a.order) < std::make_tuple(b.shift, b.rhs, b.order);
      });
    // choose the slots per item and the cluster size with the cost model
    int ny_max = 1, nx_max = 1;
    double fac_elems = 0.0;
    for (auto& kv : f) {
      ny_max = std::max(ny_max, cells[kv.first].ny);
      nx_max = std::max(nx_max, cells[kv.first].nx);
    }
    int best_r = plan.rmax, best_cl = 1;
    double best_t = 1e300;
    long long best_items = 0;
    // fr_r / fr_cl > 0 restrict the search to that shape
    auto search = [&](int fr_r, int fr_cl) {
      for (int r : {16, 8, 4}) {
        if (r > plan.rmax) continue;
        if (fr_r > 0 && r != fr_r) continue;
        long long n_items = 0;
        int maxs = 0;
        fac_elems = 0.0;
        for (auto& kv : f) {
          const DevCell& cl = cells[kv.first];
          flatten(kv.second, r, [&](const std::vector<std::pair<size_t, size_t>>&, int count) {
            ++n_items;
            maxs = std::max(maxs, count);
            fac_elems += 2.0 * cl.nx * (double)cl.ny * cl.ldn;
          });
        }
        if (n_items == 0) continue;
        const int R = front_rpad(maxs);
        // an item is a cluster of two halves of cl CTAs, each running
        // 2 nf + 1 lines of the twisted solve (nf forward lines of the longer half)
        const int nf = nx_max - 1 - (nx_max - 1) / 2;
        for (int cl = 1; cl <= plan.cluster_cap; cl *= 2) {
          if (fr_cl > 0 && cl != fr_cl) continue;
          const int mc = std::max(1, plan.max_clusters[cl]);
          if (plan.max_clusters[cl] <= 0 && cl > 1) continue;
          if (!(plan.fit_mask[R] & (1 << cl))) continue;   // shared memory
          const long long n_eff = (long long)std::ceil((double)n_items * conc);
          const long long waves = (n_eff + mc - 1) / mc;
          const double line = plan.line_overhead + plan.slot_cost * R +
                              (plan.col_cost + plan.col_slot_cost * R) * ((ny_max + cl - 1) / cl);
          double t = (double)waves * (2.0 * nf + 1.0) * line;
          t = std::max(t, conc * fac_elems * plan.csize / plan.bytes_per_cycle);
          // ties go to fewer items (less factor traffic), then to larger clusters
          if (t < best_t * 0.98 || (t <= best_t * 1.02 && n_items < best_items)) {
            best_t = t; best_r = r; best_cl = cl; best_items = n_items;
          }
        }
      }
    };
    const int fr_r = fidx < plan.forced_r.size() ? plan.forced_r[fidx] : 0;
    const int fr_cl = fidx < plan.forced_cl.size() ? plan.forced_cl[fidx] : 0;
    search(fr_r, fr_cl);
    // a fixed shape that does not fit this front leaves it to the cost model
    if (best_t >= 1e300 && (fr_r > 0 || fr_cl > 0)) search(0, 0);
    if (best_t >= 1e300) throw std::runtime_error("no sweep-front launch shape fits in shared memory");
    Front F{(int)items.size(), 0, 0, 0, best_cl};
    F.slots_cap = best_r;
    F.stage = stage; F.step = launches[fidx].step; F.lane = lane;
    for (auto& kv : f) {
      const int c = kv.first;
      auto& v = kv.second;
      const DevCell& cl = cells[c];
      flatten(v, best_r, [&](const std::vector<std::pair<size_t, size_t>>& parts, int count) {
        DevItem it{};
        it.cell = c;
        it.slot_begin = (int)slots.size();
        it.group_begin = (int)groups.size();
        for (auto& pr : parts) {
          DevGroup g{};
          g.slot_begin = (int)slots.size() - it.slot_begin;
          g.slot_count = int(pr.second - pr.first);
          g.shift = v[pr.first].shift;
          g.out_off = (((long long)v[pr.first].rhs * planes + plane) * 4 + v[pr.first].shift) * n_dof2;
          groups.push_back(g);
          for (size_t q = pr.first; q < pr.second; ++q) slots.push_back(v[q].s);
          it.group_count++;
        }
        it.slot_count = count;
        const int rs = plan.tc_scratch ? std::max(front_rpad(count), front_tc_slots(count)) : front_rpad(count);
        it.scratch_off = (long long)(cl.nx + 1) * rs * cl.ny;   // its size, for now
        F.max_slots = std::max(F.max_slots, it.slot_count);
        items.push_back(it);
        F.item_count++;
      });
    }
    // The four shifted decompositions never share data until their outputs
    // are summed, so a front whose items each belong to one shift is run as
    // one launch per shift (on concurrent streams, see enqueue_apply): its
    // items are ordered by shift and sh_begin[s] .. sh_begin[s + 1] are those
    // of shift s.  A front with an item that mixes shifts stays one launch.
    {
      auto item_shift = [&](const DevItem& it) {
        int sh = groups[it.group_begin].shift;
        for (int g = 1; g < it.group_count; ++g)
          if (groups[it.group_begin + g].shift != sh) return -1;
        return sh;
      };
      auto first = items.begin() + F.item_begin;
      // per-sweep launches run on their own streams instead: one launch each
      F.mixed = plan.lanes;
      for (auto it = first; it != items.end(); ++it)
        if (item_shift(*it) < 0) F.mixed = true;
      if (!F.mixed)
        std::stable_sort(first, items.end(),
                         [&](const DevItem& a, const DevItem& b) { return item_shift(a) < item_shift(b); });
      for (int sh = 0; sh <= 4; ++sh) F.sh_begin[sh] = F.mixed ? (sh == 0 ? 0 : F.item_count) : 0;
      if (!F.mixed) {
        int cnt[4] = {0, 0, 0, 0};
        for (auto it = first; it != items.end(); ++it) cnt[item_shift(*it)]++;
        for (int sh = 0; sh < 4; ++sh) F.sh_begin[sh + 1] = F.sh_begin[sh] + cnt[sh];
      }
    }
    fronts.push_back(F);
  }

  // Scratch (each item's forward storage, sized above in scratch_off): the
  // items of a front are live together; the launches of different shifts of
  // consecutive fronts may run together, so each shift has its own region,
  // sized for its largest front.  A mixed front runs alone (every shift's
  // stream joined) and lays its items out from 0.  Every front records the
  // pool size in scratch_elems.
  // With per-sweep launches each sweep's chain of launches has its own region
  // (sized for its largest launch) and stage 1, which runs alone, is laid out
  // from 0.
  long long region[4] = {0, 0, 0, 0}, mixed_max = 0, lane_region[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (const Front& F : fronts) {
    if (F.lane >= 0) {
      long long t = 0;
      for (int i = F.item_begin; i < F.item_begin + F.item_count; ++i) t += items[i].scratch_off;
      lane_region[F.lane] = std::max(lane_region[F.lane], t);
      continue;
    }
    if (F.mixed) {
      long long t = 0;
      for (int i = F.item_begin; i < F.item_begin + F.item_count; ++i) t += items[i].scratch_off;
      mixed_max = std::max(mixed_max, t);
      continue;
    }
    for (int sh = 0; sh < 4; ++sh) {
      long long t = 0;
      for (int i = F.item_begin + F.sh_begin[sh]; i < F.item_begin + F.sh_begin[sh + 1]; ++i) t += items[i].scratch_off;
      region[sh] = std::max(region[sh], t);
    }
  }
  const long long base[4] = {0, region[0], region[0] + region[1], region[0] + region[1] + region[2]};
  long long lane_base[8], lane_total = 0;
  for (int l = 0; l < 8; ++l) { lane_base[l] = lane_total; lane_total += lane_region[l]; }
  const long long pool = std::max(std::max(base[3] + region[3], mixed_max), lane_total);
  for (Front& F : fronts) {
    if (F.lane >= 0) {
      long long off = lane_base[F.lane];
      for (int i = F.item_begin; i < F.item_begin + F.item_count; ++i) {
        const long long sz = items[i].scratch_off;
        items[i].scratch_off = off;
        off += sz;
      }
    } else if (F.mixed) {
      long long off = 0;
      for (int i = F.item_begin; i < F.item_begin + F.item_count; ++i) {
        const long long sz = items[i].scratch_off;
        items[i].scratch_off = off;
        off += sz;
      }
    } else {
      for (int sh = 0; sh < 4; ++sh) {
        long long off = base[sh];
        for (int i = F.item_begin + F.sh_begin[sh]; i < F.item_begin + F.sh_begin[sh + 1]; ++i) {
          const long long sz = items[i].scratch_off;
          items[i].scratch_off = off;
          off += sz;
        }
      }
    }
    F.scratch_elems = pool;
  }
}

}  // namespace lsw
