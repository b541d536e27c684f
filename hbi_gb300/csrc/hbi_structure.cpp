// hbi_structure.cpp -- cluster tree, admissibility and leaf list (bit-exact
// with HACApK on one rank) and the matvec work plans built from them.
#include "hbi_structure.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace hbi {

void default_params(double* p) {
  // HACApK_init defaults (m_HACApK_base.f90:271-302) on one rank; the
  // reference writes 1.0e-6 and 1.0 as default-real literals, widened here
  // the same way.
  for (int i = 0; i < 100; i++) p[i] = 0.0;
  p[0] = 1; p[7] = 20; p[8] = 1; p[9] = 1;
  p[20] = 15; p[21] = 1.0f;
  p[42] = 1;  // param(43)=1 when nrank==1
  p[50] = 2.0f; p[51] = 1; p[52] = 100;
  p[59] = 2; p[60] = 3; p[61] = 7; p[62] = 1000; p[63] = 1;
  p[71] = (double)1.0e-6f;
  p[82] = 10; p[84] = 1; p[86] = 8; p[90] = (double)1.0e-6f; p[97] = 50; p[98] = 10;
}

namespace {

struct Coord {
  const double* g;
  int n;
  double at(int id1, int dim) const { return g[(size_t)dim * n + (size_t)(id1 - 1)]; }
};

// squared box distance of the admissibility tests; `tweak` reproduces the
// 1e-16 offset HACApK applies at the lattice-block level (:2397-2401)
double box_dist2(const Cluster& a, const Cluster& b, bool tweak) {
  double zs = 0.0;
  if (tweak)
    for (int d = 0; d < 3; d++) {
      if (a.bmax[d] != b.bmax[d]) zs = 1.0e-16;
      if (a.bmin[d] != b.bmin[d]) zs = 1.0e-16;
    }
  for (int d = 0; d < 3; d++) {
    if (a.bmax[d] < b.bmin[d]) zs = zs + (b.bmin[d] - a.bmax[d]) * (b.bmin[d] - a.bmax[d]);
    else if (b.bmax[d] < a.bmin[d]) zs = zs + (a.bmin[d] - b.bmax[d]) * (a.bmin[d] - b.bmax[d]);
  }
  return zs;
}

}  // namespace

int build_structure(int n, const double* coord, const double* param_in, Structure& s) {
  if (n < 1 || !coord) return -1;
  double pdef[100];
  const double* param = param_in;
  if (!param) { default_params(pdef); param = pdef; }
  Coord G{coord, n};
  s.n = n;
  s.lod.resize(n);
  for (int i = 0; i < n; i++) s.lod[i] = i + 1;
  s.clusters.clear();
  s.clusters.reserve(2 * (size_t)n / std::max(1, (int)param[20]) + 8);
  const int minsz = (int)param[20];
  int* lod = s.lod.data();

  // ---- cluster tree: bisection of the longest box axis at its midpoint ----
  struct Task { int id, lo, nsrt, nd; };
  std::vector<Task> stack;
  s.clusters.emplace_back();
  stack.push_back({0, 0, 1, n});
  while (!stack.empty()) {
    Task t = stack.back();
    stack.pop_back();
    s.clusters[t.id].nstrt = t.nsrt;
    s.clusters[t.id].nsize = t.nd;
    if (t.nd <= minsz) { s.clusters[t.id].nnson = 0; continue; }
    int* L = lod + t.lo;
    double zlmin[3], zlmax[3];
    for (int d = 0; d < 3; d++) {
      zlmin[d] = zlmax[d] = G.at(L[0], d);
      for (int il = 1; il < t.nd; il++) {
        double zg = G.at(L[il], d);
        if (zg < zlmin[d]) zlmin[d] = zg;
        else if (zlmax[d] < zg) zlmax[d] = zg;
      }
    }
    double zdiff = zlmax[0] - zlmin[0];
    int ncut = 0;
    for (int d = 0; d < 3; d++) {
      double zi = zlmax[d] - zlmin[d];
      if (zi > zdiff) { zdiff = zi; ncut = d; }
    }
    const double zlmid = (zlmax[ncut] + zlmin[ncut]) / 2;
    // in-place two-sided partition with the reference's stopping rules
    int nl = 1, nr = t.nd;
    while (nl < nr) {
      while (nl < t.nd && G.at(L[nl - 1], ncut) <= zlmid) nl++;
      while (nr >= 1 && G.at(L[nr - 1], ncut) > zlmid) nr--;
      if (nl < nr) std::swap(L[nl - 1], L[nr - 1]);
    }
    int a = (int)s.clusters.size();
    s.clusters.emplace_back();
    s.clusters.emplace_back();
    Cluster& c = s.clusters[t.id];
    c.nnson = 2; c.son[0] = a; c.son[1] = a + 1;
    stack.push_back({a + 1, t.lo + nl - 1, t.nsrt + nl - 1, t.nd - nl + 1});
    stack.push_back({a, t.lo, t.nsrt, nl - 1});
  }

  // ---- bounding boxes, children before parents (sons have larger ids) ----
  for (int id = (int)s.clusters.size() - 1; id >= 0; id--) {
    Cluster& c = s.clusters[id];
    if (c.nnson == 0) {
      const int* L = lod + (c.nstrt - 1);
      for (int d = 0; d < 3; d++) c.bmin[d] = c.bmax[d] = G.at(L[0], d);
      for (int d = 0; d < 3; d++)
        for (int il = 1; il < c.nsize; il++) {
          double v = G.at(L[il], d);
          if (v < c.bmin[d]) c.bmin[d] = v;
          if (c.bmax[d] < v) c.bmax[d] = v;
        }
    } else {
      const Cluster& s0 = s.clusters[c.son[0]];
      for (int d = 0; d < 3; d++) { c.bmin[d] = s0.bmin[d]; c.bmax[d] = s0.bmax[d]; }
      for (int k = 1; k < c.nnson; k++) {
        const Cluster& sk = s.clusters[c.son[k]];
        for (int d = 0; d < 3; d++) {
          if (sk.bmin[d] < c.bmin[d]) c.bmin[d] = sk.bmin[d];
          if (c.bmax[d] < sk.bmax[d]) c.bmax[d] = sk.bmax[d];
        }
      }
    }
    double w = (c.bmax[0] - c.bmin[0]) * (c.bmax[0] - c.bmin[0]);
    for (int d = 1; d < 3; d++) w = w + (c.bmax[d] - c.bmin[d]) * (c.bmax[d] - c.bmin[d]);
    c.zwdth = std::sqrt(w);
  }

  // ---- block cluster tree -> leaves ----
  const int nleaf = (int)(param[20] + 1);
  const int nlmax = (int)(param[21] * n);
  const int mdpth = (int)param[52];
  const int p52 = (int)param[51];
  const double zeta = param[50];
  const int nlttcblk = (int)((double)n / param[42] / 1.0 + 1);
  s.leaves.clear();
  auto push = [&](int lt, const Cluster& cl, const Cluster& ct) {
    s.leaves.push_back(Leaf{lt, 0, cl.nstrt, cl.nsize, ct.nstrt, ct.nsize});
  };
  const Cluster& r = s.clusters[0];
  if (r.nsize < nlttcblk) {
    // the one lattice block (HACApK_generate_blrleaf :2396-2450)
    double zd = std::sqrt(box_dist2(r, r, true));
    if (r.zwdth <= zeta * zd) {
      push(1, r, r);
    } else if (1 == mdpth || r.nnson == 0 || (r.nsize <= nleaf && r.nsize <= nleaf)) {
      push(2, r, r);
    } else {
      struct Pair { int l, t, depth; };
      std::vector<Pair> st;
      for (int a = r.nnson - 1; a >= 0; a--)
        for (int b = r.nnson - 1; b >= 0; b--) st.push_back({r.son[a], r.son[b], 1});
      while (!st.empty()) {
        Pair p = st.back();
        st.pop_back();
        const Cluster& cl = s.clusters[p.l];
        const Cluster& ct = s.clusters[p.t];
        int depth = p.depth + 1;
        int ndl = cl.nsize, ndt = ct.nsize;
        double zd = std::sqrt(box_dist2(cl, ct, false));
        if ((cl.zwdth <= zeta * zd || ct.zwdth <= zeta * zd) &&
            (ndl >= nleaf && ndt >= nleaf && ndl <= nlmax && ndt <= nlmax)) {
          if (p52 == 0 || (p52 == 1 && ((cl.nstrt + ndl) != ct.nstrt && (ct.nstrt + ndt) != cl.nstrt))) {
            push(1, cl, ct);
            continue;
          }
        }
        if (depth == mdpth || cl.nnson == 0 || ct.nnson == 0 || ndl <= nleaf || ndt <= nleaf) {
          push(2, cl, ct);
          continue;
        }
        for (int a = cl.nnson - 1; a >= 0; a--)
          for (int b = ct.nnson - 1; b >= 0; b--) st.push_back({cl.son[a], ct.son[b], depth});
      }
    }
  }
  // (nstrtl, nstrtt) is unique per leaf, so any correct sort gives HACApK's order
  std::sort(s.leaves.begin(), s.leaves.end(), [](const Leaf& a, const Leaf& b) {
    return a.nstrtl != b.nstrtl ? a.nstrtl < b.nstrtl : a.nstrtt < b.nstrtt;
  });
  s.fine_start.clear();
  for (auto& c : s.clusters)
    if (c.nnson == 0) s.fine_start.push_back(c.nstrt);
  std::sort(s.fine_start.begin(), s.fine_start.end());
  return 0;
}

static int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

void plan_groups(int n, const std::vector<Leaf>& leaves, GroupPlan& gp) {
  // groups ordered by (row0 ascending, ndl descending): coarse before fine
  std::vector<std::pair<std::pair<int, int>, int>> key;
  key.reserve(leaves.size());
  for (int i = 0; i < (int)leaves.size(); i++) key.push_back({{leaves[i].nstrtl - 1, -leaves[i].ndl}, i});
  std::stable_sort(key.begin(), key.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  gp.gleaf_ptr.assign(1, 0);
  gp.gleaf.clear(); gp.grow0.clear(); gp.gndl.clear(); gp.gpoff.clear();
  int64_t poff = 0;
  for (size_t k = 0; k < key.size(); k++) {
    if (k == 0 || key[k].first != key[k - 1].first) {
      if (k) gp.gleaf_ptr.push_back((int32_t)gp.gleaf.size());
      gp.grow0.push_back(key[k].first.first);
      gp.gndl.push_back(-key[k].first.second);
      gp.gpoff.push_back((int32_t)poff);
      poff += -key[k].first.second;
    }
    gp.gleaf.push_back(key[k].second);
  }
  gp.gleaf_ptr.push_back((int32_t)gp.gleaf.size());
  gp.plen = poff;
  // fine ranges: elementary intervals of all group boundaries
  std::vector<int> bnd{0, n};
  for (size_t g = 0; g < gp.grow0.size(); g++) {
    bnd.push_back(gp.grow0[g]);
    bnd.push_back(gp.grow0[g] + gp.gndl[g]);
  }
  std::sort(bnd.begin(), bnd.end());
  bnd.erase(std::unique(bnd.begin(), bnd.end()), bnd.end());
  const int nf = (int)bnd.size() - 1;
  gp.row_fc.assign(n, 0);
  for (int f = 0; f < nf; f++)
    for (int r = bnd[f]; r < bnd[f + 1]; r++) gp.row_fc[r] = f;
  std::vector<std::vector<int32_t>> cov(nf);
  for (size_t g = 0; g < gp.grow0.size(); g++) {
    int f0 = gp.row_fc[gp.grow0[g]], f1 = gp.row_fc[gp.grow0[g] + gp.gndl[g] - 1];
    for (int f = f0; f <= f1; f++) cov[f].push_back((int32_t)g);
  }
  gp.fc_ptr.assign(1, 0);
  gp.fc_group.clear();
  for (int f = 0; f < nf; f++) {
    for (int32_t g : cov[f]) gp.fc_group.push_back(g);
    gp.fc_ptr.push_back((int32_t)gp.fc_group.size());
  }
}

void plan_stream(int n, const std::vector<Leaf>& leaves, const std::vector<int64_t>& body_off, int vec,
                 StreamPlan& sp, int stage_bytes) {
  const int nl = (int)leaves.size();
  const int tr = 32 * vec;
  sp = StreamPlan();
  sp.vec = vec;
  sp.tr = tr;
  int64_t fe = 0;
  for (const Leaf& L : leaves) fe += L.ltmtx == 1 ? (int64_t)L.kt * (L.ndl + L.ndt) : (int64_t)L.ndl * L.ndt;
  sp.factor_elems = fe;
  // ---- phase 1: column groups of the low-rank leaves ----
  std::vector<std::pair<std::pair<int, int>, int>> ck;  // ((col0, -ndt), leaf)
  for (int i = 0; i < nl; i++)
    if (leaves[i].ltmtx == 1 && leaves[i].kt > 0) ck.push_back({{leaves[i].nstrtt - 1, -leaves[i].ndt}, i});
  std::stable_sort(ck.begin(), ck.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  std::vector<int32_t> leaf_z(nl, -1);
  int64_t voff = 0, z = 0, poff = 0, ncg = 0;
  for (size_t a = 0; a < ck.size();) {
    size_t b = a;
    while (b < ck.size() && ck[b].first == ck[a].first) b++;
    const int col0 = ck[a].first.first, ndt = -ck[a].first.second;
    int ncols = 0;
    for (size_t e = a; e < b; e++) {
      leaf_z[ck[e].second] = (int32_t)(z + ncols);
      ncols += leaves[ck[e].second].kt;
    }
    const int ntile = (ndt + tr - 1) / tr;
    const int64_t poff0 = poff;
    if (ntile > 1) poff += (int64_t)ntile * ncols;
    for (int t = 0; t < ntile; t++) {
      const int nt = std::min(tr, ndt - t * tr);
      const int ntp = (int)round_up(nt, vec);
      const int64_t region = voff;
      int c = 0;
      for (size_t e = a; e < b; e++) {
        const int li = ck[e].second;
        const Leaf& L = leaves[li];
        for (int k = 0; k < L.kt; k++, c++)
          sp.vcopy.push_back(SegCopy{region + (int64_t)c * ntp, body_off[li] + (int64_t)k * L.ndt + (int64_t)t * tr,
                                     nt, 1, vswz(c, ntp / vec), 0});
      }
      S1Item it{};
      it.soff = region;
      it.ncols = ncols;
      it.ntp = ntp;
      it.x0 = col0 + t * tr;
      it.nt = nt;
      it.z0 = (int32_t)z;
      it.cg = (int32_t)ncg;
      it.tile = t;
      it.ntile = ntile;
      it.poff = ntile > 1 ? (int32_t)poff0 : -1;
      it.cc = chunk_cols(ntp, 16 / vec, stage_bytes);
      sp.p1.push_back(it);
      voff += (int64_t)ncols * ntp;
    }
    ncg++;
    z += ncols;
    a = b;
  }
  sp.vstore = round_up(voff, vec);
  sp.zlen = z;
  sp.plen1 = poff;
  sp.ncg = ncg;
  // ---- phase 2: row groups of all leaves ----
  plan_groups(n, leaves, sp.gp);
  const GroupPlan& gp = sp.gp;
  const int ng = (int)gp.grow0.size();
  sp.gnch.assign(ng, 1);
  sp.gpoff2.assign(ng, 0);
  int64_t uoff = 0, p2off = 0;
  for (int g = 0; g < ng; g++) {
    const int ndl = gp.gndl[g];
    while (sp.midx.size() % 4) sp.midx.push_back(0);
    const int m0 = (int)sp.midx.size();
    for (int e = gp.gleaf_ptr[g]; e < gp.gleaf_ptr[g + 1]; e++) {
      const int li = gp.gleaf[e];
      const Leaf& L = leaves[li];
      if (L.ltmtx == 1) {
        for (int k = 0; k < L.kt; k++) sp.midx.push_back(leaf_z[li] + k);
      } else {
        for (int k = 0; k < L.ndt; k++) sp.midx.push_back(-(L.nstrtt - 1 + k) - 1);
      }
    }
    const int ncols = (int)sp.midx.size() - m0;
    sp.gpoff2[g] = (int32_t)p2off;
    p2off += ndl;
    if (ncols == 0) {
      sp.gnch[g] = 0;
      continue;
    }
    const int ntile = (ndl + tr - 1) / tr;
    for (int t = 0; t < ntile; t++) {
      const int nr = std::min(tr, ndl - t * tr);
      const int ntp = (int)round_up(nr, vec);
      const int64_t region = uoff;
      int c = 0;
      for (int e = gp.gleaf_ptr[g]; e < gp.gleaf_ptr[g + 1]; e++) {
        const int li = gp.gleaf[e];
        const Leaf& L = leaves[li];
        if (L.ltmtx == 1) {
          const int64_t u0 = body_off[li] + (int64_t)L.ndt * L.kt;
          for (int k = 0; k < L.kt; k++, c++)
            sp.ucopy.push_back(SegCopy{region + (int64_t)c * ntp, u0 + (int64_t)k * L.ndl + (int64_t)t * tr, nr, 1, 0, 0});
        } else {
          // a1(ndt, ndl): element (it, il) at it + il*ndt; column it, rows il
          for (int k = 0; k < L.ndt; k++, c++)
            sp.ucopy.push_back(SegCopy{region + (int64_t)c * ntp, body_off[li] + k + (int64_t)t * tr * L.ndt, nr,
                                       L.ndt, 0, 0});
        }
      }
      S2Item it{};
      it.soff = region;
      it.ncols = ncols;
      it.ntp = ntp;
      it.nr = nr;
      it.m0 = m0;
      it.pout = (int32_t)(sp.gpoff2[g] + t * tr);
      it.cc = chunk_cols(ntp, 16 / vec, stage_bytes);
      sp.p2.push_back(it);
      uoff += (int64_t)ncols * ntp;
    }
  }
  while (sp.midx.size() % 4) sp.midx.push_back(0);
  sp.midx.resize(sp.midx.size() + 256, 0);  // chunk copies may read a whole chunk's worth past a group
  // phase-3 lists: one partial per non-empty covering group
  const int nf = (int)gp.fc_ptr.size() - 1;
  sp.fcb_ptr.assign(nf + 1, 0);
  for (int f = 0; f < nf; f++) {
    for (int e = gp.fc_ptr[f]; e < gp.fc_ptr[f + 1]; e++) {
      const int g = gp.fc_group[e];
      if (sp.gnch[g] == 0) continue;
      sp.fcb_base.push_back(sp.gpoff2[g] - gp.grow0[g]);
    }
    sp.fcb_ptr[f + 1] = (int32_t)sp.fcb_base.size();
  }
  sp.ustore = round_up(uoff, vec);
  sp.plen2 = p2off;
  // big items first, for the static warp schedule
  std::stable_sort(sp.p1.begin(), sp.p1.end(), [](const S1Item& a, const S1Item& b) {
    return (int64_t)a.ncols * a.ntp > (int64_t)b.ncols * b.ntp;
  });
  std::stable_sort(sp.p2.begin(), sp.p2.end(), [](const S2Item& a, const S2Item& b) {
    return (int64_t)a.ncols * a.ntp > (int64_t)b.ncols * b.ntp;
  });
}

void plan_warp_schedule(const std::vector<int64_t>& cost, int nwarps, std::vector<int32_t>& woff,
                        std::vector<int32_t>& witem) {
  const int n = (int)cost.size();
  std::vector<int32_t> order(n);
  for (int i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  // min-heap of (load, warp)
  std::vector<std::pair<int64_t, int>> heap;
  heap.reserve(nwarps);
  for (int w = 0; w < nwarps; w++) heap.push_back({0, w});
  auto cmp = [](const std::pair<int64_t, int>& a, const std::pair<int64_t, int>& b) { return a > b; };
  std::make_heap(heap.begin(), heap.end(), cmp);
  std::vector<int32_t> owner(n);
  std::vector<int32_t> count(nwarps, 0);
  for (int q = 0; q < n; q++) {
    std::pop_heap(heap.begin(), heap.end(), cmp);
    auto& top = heap.back();
    owner[q] = top.second;
    count[top.second]++;
    top.first += cost[order[q]];
    std::push_heap(heap.begin(), heap.end(), cmp);
  }
  woff.assign(nwarps + 1, 0);
  for (int w = 0; w < nwarps; w++) woff[w + 1] = woff[w] + count[w];
  witem.assign(n, 0);
  std::vector<int32_t> fill(woff.begin(), woff.end() - 1);
  for (int q = 0; q < n; q++) witem[fill[owner[q]]++] = order[q];
}

void plan_block_schedule(const std::vector<int64_t>& cost, const std::vector<int64_t>& key, int nblocks, int nw,
                         std::vector<int32_t>& woff, std::vector<int32_t>& witem) {
  const int n = (int)cost.size();
  std::vector<int32_t> order(n);
  for (int i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
  int64_t total = 0;
  for (int64_t c : cost) total += c;
  // block b takes order[cut[b] .. cut[b + 1]): each cut where the running cost
  // is nearest to total * b / nblocks
  std::vector<int> cut(nblocks + 1, n);
  cut[0] = 0;
  int i = 0;
  int64_t run = 0;
  for (int b = 1; b < nblocks; b++) {
    const double target = (double)total * b / nblocks;
    while (i < n && (double)(run + cost[order[i]]) <= target) run += cost[order[i++]];
    // one more item if that lands nearer the target
    if (i < n && (double)(run + cost[order[i]]) - target < target - (double)run) run += cost[order[i++]];
    cut[b] = i;
  }
  woff.assign((size_t)nblocks * nw + 1, 0);
  witem.clear();
  witem.reserve(n);
  for (int b = 0; b < nblocks; b++) {
    std::vector<int64_t> sub;
    for (int q = cut[b]; q < cut[b + 1]; q++) sub.push_back(cost[order[q]]);
    std::vector<int32_t> so, si;
    plan_warp_schedule(sub, nw, so, si);
    for (int w = 0; w < nw; w++) {
      for (int e = so[w]; e < so[w + 1]; e++) witem.push_back(order[cut[b] + si[e]]);
      woff[(size_t)b * nw + w + 1] = (int32_t)witem.size();
    }
  }
}

void plan_tc(int n, const std::vector<Leaf>& leaves, const std::vector<int64_t>& body_off, TcPlan& tp) {
  const int nl = (int)leaves.size();
  const int TR = 256;  // phase 2: rows of a tile
  tp = TcPlan();
  // ---- phase 1: column groups; K = rows of a tile (<= kTcK1), N = columns
  // (<= 256 per item): long tiles keep a group's sum in tensor memory, and
  // only groups taller than kTcK1 rows meet in partial sums
  std::vector<std::pair<std::pair<int, int>, int>> ck;
  for (int i = 0; i < nl; i++)
    if (leaves[i].ltmtx == 1 && leaves[i].kt > 0) ck.push_back({{leaves[i].nstrtt - 1, -leaves[i].ndt}, i});
  std::stable_sort(ck.begin(), ck.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  std::vector<int32_t> leaf_z(nl, -1);
  int64_t off = 0, z = 0, poff = 0, ncg = 0;
  for (size_t a = 0; a < ck.size();) {
    size_t b = a;
    while (b < ck.size() && ck[b].first == ck[a].first) b++;
    const int col0 = ck[a].first.first, ndt = -ck[a].first.second;
    // the group's columns in leaf order: (leaf, k)
    std::vector<std::pair<int, int>> cols;
    for (size_t e = a; e < b; e++) {
      leaf_z[ck[e].second] = (int32_t)(z + cols.size());
      for (int k = 0; k < leaves[ck[e].second].kt; k++) cols.push_back({ck[e].second, k});
    }
    const int ncols = (int)cols.size();
    const int ntile = (ndt + kTcK1 - 1) / kTcK1;
    for (int c0 = 0; c0 < ncols; c0 += 256) {
      const int nv = std::min(256, ncols - c0);
      const int np = (nv + 7) / 8 * 8;
      const int64_t poff0 = poff;
      if (ntile > 1) poff += (int64_t)ntile * nv;
      for (int t = 0; t < ntile; t++) {
        const int kv = std::min(kTcK1, ndt - t * kTcK1);
        const int kp = (kv + 15) / 16 * 16;
        TcItem it{};
        it.soff = off;
        it.np = np; it.kp = kp; it.nv = nv; it.kv = kv;
        it.m0 = col0 + t * kTcK1;
        it.out0 = (int32_t)(z + c0);
        it.cg = (int32_t)ncg;
        it.tile = t; it.ntile = ntile;
        it.poff = ntile > 1 ? (int32_t)poff0 : -1;
        tp.p1.push_back(it);
        for (int c = 0; c < nv; c++) {
          const int li = cols[c0 + c].first, k = cols[c0 + c].second;
          const Leaf& L = leaves[li];
          // V(row, k) at body + row + k*ndt; run along K (the tile's rows)
          tp.copy1.push_back(
              TcCopy{off, body_off[li] + (int64_t)k * L.ndt + (int64_t)t * kTcK1, np, c, 0, 0, 1, kv, 1});
        }
        off += (int64_t)kp * np * 2;
      }
      ncg++;
    }
    z += ncols;
    a = b;
  }
  tp.store1 = off;
  tp.zlen = z;
  tp.plen1 = poff;
  tp.ncg = ncg;
  // ---- phase 2: row groups; N = rows of a tile, K = the group's columns
  GroupPlan gp;
  plan_groups(n, leaves, gp);
  const int ng = (int)gp.grow0.size();
  off = 0;
  int64_t p2off = 0;
  for (int g = 0; g < ng; g++) {
    const int ndl = gp.gndl[g];
    while (tp.midx.size() % 4) tp.midx.push_back(0);
    const int m0 = (int)tp.midx.size();
    std::vector<std::pair<int, int>> cols;
    for (int e = gp.gleaf_ptr[g]; e < gp.gleaf_ptr[g + 1]; e++) {
      const int li = gp.gleaf[e];
      const Leaf& L = leaves[li];
      const int nc = L.ltmtx == 1 ? L.kt : L.ndt;
      for (int k = 0; k < nc; k++) {
        tp.midx.push_back(L.ltmtx == 1 ? leaf_z[li] + k : -(L.nstrtt - 1 + k) - 1);
        cols.push_back({li, k});
      }
    }
    const int ncols = (int)cols.size();
    const int64_t gpoff = p2off;
    p2off += ndl;
    if (ncols == 0) continue;
    const int kp = (ncols + 15) / 16 * 16;
    const int ntile = (ndl + TR - 1) / TR;
    for (int t = 0; t < ntile; t++) {
      const int nv = std::min(TR, ndl - t * TR);
      const int np = (nv + 7) / 8 * 8;
      TcItem it{};
      it.soff = off;
      it.np = np; it.kp = kp; it.nv = nv; it.kv = ncols;
      it.m0 = m0;
      it.out0 = (int32_t)(gpoff + t * TR);
      it.cg = -1; it.tile = t; it.ntile = ntile; it.poff = -1;
      tp.p2.push_back(it);
      for (int c = 0; c < ncols; c++) {
        const int li = cols[c].first, k = cols[c].second;
        const Leaf& L = leaves[li];
        if (L.ltmtx == 1) {
          const int64_t u0 = body_off[li] + (int64_t)L.ndt * L.kt + (int64_t)k * L.ndl + (int64_t)t * TR;
          tp.copy2.push_back(TcCopy{off, u0, np, 0, c, 1, 0, nv, 1});  // run along N (rows)
        } else {
          // a1(ndt, ndl): (it, il) at it + il*ndt; column it = k, rows il
          tp.copy2.push_back(TcCopy{off, body_off[li] + k + (int64_t)t * TR * L.ndt, np, 0, c, 1, 0, nv, L.ndt});
        }
      }
      off += (int64_t)kp * np * 2;
    }
  }
  while (tp.midx.size() % 4) tp.midx.push_back(0);
  tp.midx.resize(tp.midx.size() + 64, 0);
  tp.store2 = off;
  std::stable_sort(tp.p1.begin(), tp.p1.end(), [](const TcItem& a, const TcItem& b) {
    return (int64_t)a.np * a.kp > (int64_t)b.np * b.kp;
  });
  std::stable_sort(tp.p2.begin(), tp.p2.end(), [](const TcItem& a, const TcItem& b) {
    return (int64_t)a.np * a.kp > (int64_t)b.np * b.kp;
  });
}

}  // namespace hbi
