// MD layout planner (see md_plan.h).
//
// Beads live in slots: the MD kernels run one thread (or two lanes) per slot,
// a tile of slots per CTA.  A bead owns 1 + h consecutive slots (h helper
// slots when its spring list is longer than the chunk, each helper summing
// one chunk).  Every cilium occupies contiguous slots of one tile, so that its
// beat bookkeeping needs no synchronisation beyond its CTA.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <utility>

#include "md_plan.h"

namespace mpcd {

namespace {

// Force entries of the float64 pair kernel (md_pair.cu) from the slot-ordered
// spring lists of a grid layout with one slot per bead.  A spring whose other
// bead lies in the same tile, and whose exact reverse (same kind, same rest
// length or bond, same constant) is in that bead's list, forms one entry with
// the reverse: the two forces are fac (x_a - x_b) and its negation bit for bit
// (the squared distance of the negated difference is the same number), so the
// entry is evaluated once.  The reference makes every cilium and sphere
// spring in both directions (src/cilia.cpp:127-201, src/sphere.cpp:87-119).
// A spring whose reaction a hub takes (its other bead is the hub) is an entry
// of its own bead; the tile's entries of each hub are listed for its partial
// sum.  Returns "hub" when a tile would reach more than kTileHubs hubs.
std::string plan_pair_tables(MDPlan& out, const std::vector<int>& hubs) {
  const int T = out.tile, nt = out.ntiles, ns = out.nslots;
  const std::vector<int>& start = out.start;
  const int nsp = start[ns];
  out.pair = 1;
  out.pr_start.assign(nt + 1, 0);
  out.pr_local_end.assign(nt, 0);
  out.pr_hub_begin.assign(nt, 0);
  out.pr_code.clear();
  out.pr_rest.clear();
  out.pr_m2k.clear();
  out.pi_start = start;  // one incidence per one-sided spring
  out.pr_pos.clear();
  out.pl_start.assign(nt + 1, 0);
  out.pl_list.clear();
  out.pl_base.clear();
  out.pr_nslot.clear();
  out.pr_nent_max = out.pr_ninc_max = out.pr_nlong_max = 0;
  const int nh = (int)hubs.size();
  std::vector<int> hub_of(ns, -1);
  for (int h = 0; h < nh; ++h) hub_of[hubs[h]] = h;
  out.hub_slot = hubs;
  std::vector<int> ncon(nh, 0);
  out.th_start.assign(nt + 1, 0);
  out.th.clear();
  out.tr_list.clear();
  std::vector<int> ent(nsp, -1);  // spring -> entry of its tile (in creation order)
  struct Entry {
    int a, b, kind, both, react, lref, bslot;
    double rest, m2k;
    int da, db;  // its spring (first bead) and the reverse (second bead), or -1
  };
  std::vector<Entry> es;
  std::vector<int> lbase(T);
  for (int t = 0; t < nt; ++t) {
    const int base = t * T;
    es.clear();
    // incidence slots: the j-th spring of a bead a with at most kPairLong
    // springs at j * T + a (the threads summing consecutive beads read
    // consecutive words), longer lists one after another beyond T * kmax
    int kmax = 0, lsum = 0;
    for (int s = base; s < base + T; ++s)
      if (start[s + 1] - start[s] <= kPairLong) kmax = std::max(kmax, start[s + 1] - start[s]);
    for (int s = base; s < base + T; ++s) {
      lbase[s - base] = -1;
      if (start[s + 1] - start[s] > kPairLong) {
        lbase[s - base] = T * kmax + lsum;
        lsum += start[s + 1] - start[s];
        out.pl_list.push_back(s - base);
        out.pl_base.push_back(lbase[s - base]);
      }
    }
    auto slot_pos = [&](int d, int a) {  // spring d of local bead a
      const int j = d - start[base + a];
      return lbase[a] >= 0 ? lbase[a] + j : j * T + a;
    };
    for (int s = base; s < base + T; ++s)
      for (int d = start[s]; d < start[s + 1]; ++d) {
        if (ent[d] >= 0) continue;  // the reverse half of an entry made before
        if (out.sk[d] & ~(3 | kSpringReact)) return "pair kernel: unexpected spring flags";
        const int react = (out.sk[d] & kSpringReact) ? 1 : 0;
        if (react && hub_of[out.so[d]] < 0) return "pair kernel: a reaction spring whose other bead is not a hub";
        const int a = s - base, b = out.sl[d], kind = out.sk[d] & 3;
        const int lref = kind >= MPCD_SPRING_BOND ? out.sr[d] - out.df_b0[t] : 0;
        Entry e{a, b, kind, 0, react, lref, out.so[d], out.srest[d], out.sm2k[d], d, -1};
        ent[d] = (int)es.size();
        if (b < T && b != a && !react) {
          const int so = base + b;
          for (int r = start[so]; r < start[so + 1]; ++r) {
            if (ent[r] >= 0 || out.so[r] != s || out.sk[r] != out.sk[d] || out.sm2k[r] != out.sm2k[d]) continue;
            if (kind >= MPCD_SPRING_BOND ? out.sr[r] != out.sr[d] : out.srest[r] != out.srest[d]) continue;
            ent[r] = (int)es.size();
            e.both = 1;
            e.db = r;
            break;
          }
        }
        es.push_back(e);
      }
    // the entries reaching only this tile's beads first (they run while the
    // halo loads), then those reaching the halo, then those reaching a hub
    // (after its copy has been advanced)
    std::vector<int> order;
    auto to_hub = [&](const Entry& e) { return hub_of[e.bslot] >= 0; };
    for (size_t i = 0; i < es.size(); ++i)
      if (es[i].b < T && !to_hub(es[i])) order.push_back((int)i);
    const int nloc = (int)order.size();
    for (size_t i = 0; i < es.size(); ++i)
      if (es[i].b >= T && !to_hub(es[i])) order.push_back((int)i);
    const int nhub0 = (int)order.size();
    for (size_t i = 0; i < es.size(); ++i)
      if (to_hub(es[i])) order.push_back((int)i);
    const int g0 = (int)out.pr_code.size();
    // hubs this tile owns or reaches, with the entries whose reaction each takes
    std::vector<HubRef> refs;
    std::vector<std::vector<int>> rlist;
    auto ref_of = [&](int h, int idx) {
      for (size_t k = 0; k < refs.size(); ++k)
        if (refs[k].hub == h) return (int)k;
      refs.push_back(HubRef{h, idx, -1, 0, 0, 0});
      rlist.emplace_back();
      return (int)refs.size() - 1;
    };
    for (int s = base; s < base + T; ++s)
      if (hub_of[s] >= 0) ref_of(hub_of[s], s - base);
    for (size_t r = 0; r < order.size(); ++r) {
      const Entry& e = es[order[r]];
      if (e.b >= (1 << 16) || e.a >= (1 << 16) || e.lref < 0 || e.lref >= (1 << 27))
        return "pair kernel: an MD tile is too large for packed entry codes";
      out.pr_code.push_back(make_uint2((uint32_t)e.a | ((uint32_t)e.b << 16),
                                       (uint32_t)e.kind | ((uint32_t)e.both << 2) | ((uint32_t)e.react << 3) |
                                           ((uint32_t)e.lref << 4)));
      out.pr_rest.push_back(e.rest);
      out.pr_m2k.push_back(e.m2k);
      // the incidence slots its force (first bead) and negated force (second) go to
      const int ka = slot_pos(e.da, e.a), kb = e.db >= 0 ? slot_pos(e.db, e.b) : 0xffff;
      if (ka < 0 || ka >= 0xffff || kb < 0 || kb > 0xffff) return "pair kernel: an MD tile has too many springs";
      out.pr_pos.push_back((uint32_t)ka | ((uint32_t)kb << 16));
      if (hub_of[e.bslot] >= 0) {
        const int k = ref_of(hub_of[e.bslot], e.b);
        if (refs[k].idx != e.b) return "pair kernel: a hub staged twice in one tile";
        if (e.react) rlist[k].push_back(ka);  // the reaction is read from the first bead's slot
      }
    }
    if ((int)refs.size() > kTileHubs) return "hub";
    for (size_t k = 0; k < refs.size(); ++k) {
      if (!rlist[k].empty()) refs[k].rank = ncon[refs[k].hub]++;
      refs[k].rs = (int)out.tr_list.size();
      refs[k].rn = (int)rlist[k].size();
      out.tr_list.insert(out.tr_list.end(), rlist[k].begin(), rlist[k].end());
      out.th.push_back(refs[k]);
    }
    out.th_start[t + 1] = (int)out.th.size();
    out.pr_local_end[t] = g0 + nloc;
    out.pr_hub_begin[t] = g0 + nhub0;
    out.pr_start[t + 1] = (int)out.pr_code.size();
    out.pr_nent_max = std::max(out.pr_nent_max, (int)es.size());
    out.pl_start[t + 1] = (int)out.pl_list.size();
    out.pr_nslot.push_back(T * kmax + lsum);
    out.pr_nlong_max = std::max(out.pr_nlong_max, out.pl_start[t + 1] - out.pl_start[t]);
    out.pr_ninc_max = std::max(out.pr_ninc_max, T * kmax + lsum);
  }
  out.hub_pbase.assign(nh + 1, 0);
  for (int h = 0; h < nh; ++h) out.hub_pbase[h + 1] = out.hub_pbase[h] + ncon[h];
  return "";
}

}  // namespace

std::string plan_md(const MDInput& in, const MDForce& force, bool allow_cluster, bool no_react, int grid_f32cells,
                    MDPlan& out, int min_tile) {
  // springs per helper slot: the longest serial spring chain of any thread.
  // Odd, so that the helper slots' spring lists start in different
  // shared-memory banks.
  // The double-float grid kernel's springs cost more per lane: shorter chunks.
  int kChunk = in.df && !in.split ? 15 : 31;
  if (const char* env = std::getenv("MPCD_MD_CHUNK")) kChunk = std::max(2, std::min(256, std::atoi(env)));
  // the pair kernel sums long lists by warps: one slot per bead
  if (in.pair) kChunk = INT_MAX;
  out = MDPlan{};
  const bool forced = force.lanes > 0;
  out.split = in.split;
  out.df = in.df && !in.split;
  if (in.nb == 0) return "";
  const long nb = in.nb;
  const long nsp = in.nsp;
  const int ncil = in.ncil;
  std::vector<int> nspr(nb, 0);
  for (long i = 0; i < nsp; ++i) {
    if (in.sp_t[i] < 0 || in.sp_t[i] >= nb || in.sp_o[i] < 0 || in.sp_o[i] >= nb)
      return "spring bead index out of range";
    nspr[in.sp_t[i]]++;
  }
  std::vector<int> width(nb);
  for (long b = 0; b < nb; ++b) width[b] = 1 + (nspr[b] > kChunk ? (nspr[b] + kChunk - 1) / kChunk - 1 : 0);
  std::vector<int> owner(nb, -1);  // cilium owning the bead
  for (int c = 0; c < ncil; ++c)
    for (int k = 0; k < 3 * in.cil[c].rodlength; ++k) {
      const long b = (long)in.cil[c].bead0 + k;
      if (b < 0 || b >= nb) return "cilium bead range outside the bead array";
      if (owner[b] >= 0) return "beads shared by two cilia";
      owner[b] = c;
    }
  // Hubs (a sphere's centre: one spring to every surface bead).  When every
  // spring of a hub has an exact reverse partner inside the same run of
  // non-cilium beads, the one-lane cluster layout drops the hub's own list
  // and sums the partners' forces, negated, over the tile (react[j] marks
  // the partners).
  std::vector<int> run_id(nb, -1);
  for (long b = 0, r = 0; b < nb; ++b)
    if (owner[b] < 0) run_id[b] = (b > 0 && owner[b - 1] < 0) ? run_id[b - 1] : (int)r++;
  std::vector<int> bstart(nb + 1, 0), blist(nsp);
  for (long i = 0; i < nsp; ++i) bstart[in.sp_t[i] + 1]++;
  for (long b = 0; b < nb; ++b) bstart[b + 1] += bstart[b];
  {
    std::vector<int> fillp(bstart.begin(), bstart.end() - 1);
    for (long i = 0; i < nsp; ++i) blist[fillp[in.sp_t[i]]++] = (int)i;
  }
  std::vector<char> hub(nb, 0), react(nsp, 0), dropped(nsp, 0);
  if (!no_react) {
    for (long b = 0; b < nb; ++b) {
      if (owner[b] >= 0 || nspr[b] <= kChunk) continue;
      std::vector<int> partners;
      bool ok = true;
      for (int q = bstart[b]; q < bstart[b + 1] && ok; ++q) {
        const int i = blist[q];
        const int o = in.sp_o[i];
        if (in.sp_k[i] != MPCD_SPRING_CONST || run_id[o] != run_id[b] || o == b) {
          ok = false;
          break;
        }
        int found = -1;
        for (int r = bstart[o]; r < bstart[o + 1]; ++r) {
          const int j = blist[r];
          if (in.sp_o[j] == b && in.sp_k[j] == MPCD_SPRING_CONST && in.sp_rest[j] == in.sp_rest[i] &&
              in.sp_kk[j] == in.sp_kk[i] && !react[j]) {
            found = j;
            break;
          }
        }
        if (found < 0) ok = false;
        else partners.push_back(found);
      }
      if (!ok) continue;
      hub[b] = 1;
      for (int j : partners) react[j] = 1;
      for (int q = bstart[b]; q < bstart[b + 1]; ++q) dropped[blist[q]] = 1;
    }
  }
  // every bead of a cilium owns the same number of slots (the kernels address
  // a cilium's beads as slot0 + stride * (filament * rodlength + bead))
  auto pad_cilia = [&]() {
    for (int c = 0; c < ncil; ++c) {
      int wmax = 1;
      for (int k = 0; k < 3 * in.cil[c].rodlength; ++k) wmax = std::max(wmax, width[in.cil[c].bead0 + k]);
      for (int k = 0; k < 3 * in.cil[c].rodlength; ++k) width[in.cil[c].bead0 + k] = wmax;
    }
  };
  auto widest = [&]() {
    int w_max = 0;
    for (int c = 0; c < ncil; ++c) {
      int w = 0;
      for (int k = 0; k < 3 * in.cil[c].rodlength; ++k) w += width[(long)in.cil[c].bead0 + k];
      w_max = std::max(w_max, w);
    }
    for (long b = 0; b < nb; ++b)
      if (owner[b] < 0) w_max = std::max(w_max, width[b]);
    return w_max;
  };
  pad_cilia();
  std::vector<int> width_grid = width;
  int cl_chunk = kChunk;  // springs per slot of the chosen layout
  int maxw = widest();
  // Pack: cilia first (each contiguous in one tile), then the other beads in
  // the remaining space.  Returns the number of tiles.
  std::vector<int> fill, slot_of(nb, -1), cil_tile(ncil);
  auto pack = [&](int tile) {
    fill.clear();
    std::fill(slot_of.begin(), slot_of.end(), -1);
    for (int c = 0; c < ncil; ++c) {
      const mpcd_cilium& cl = in.cil[c];
      int w = 0;
      for (int k = 0; k < 3 * cl.rodlength; ++k) w += width[cl.bead0 + k];
      if (fill.empty() || fill.back() + w > tile) fill.push_back(0);
      const int t = (int)fill.size() - 1;
      cil_tile[c] = t;
      for (int k = 0; k < 3 * cl.rodlength; ++k) {
        slot_of[cl.bead0 + k] = t * tile + fill[t];
        fill[t] += width[cl.bead0 + k];
      }
    }
    // the pair kernel keeps the other beads (a sphere) in tiles of their own:
    // fewer springs between tiles, and a hub's partial sums come from those
    // tiles only
    size_t tcur = in.pair ? fill.size() : 0;
    for (long b = 0; b < nb; ++b) {
      if (owner[b] >= 0) continue;
      while (tcur < fill.size() && fill[tcur] + width[b] > tile) ++tcur;
      if (tcur == fill.size()) fill.push_back(0);
      slot_of[b] = (int)tcur * tile + fill[tcur];
      fill[tcur] += width[b];
    }
    return (int)fill.size();
  };
  // Pair-kernel packing: cilia as above; every run of consecutive other beads
  // (a sphere, whose bead order does not follow its mesh) is cut by recursive
  // coordinate bisection into compact patches, each in a tile of its own, so
  // that many of a patch's springs join two of its own beads (one entry for
  // both) and its work stays near a cilium tile's.  In bead order the
  // swimmer64 sphere put 500-680 entries into a tile against 207 in a cilium
  // tile.
  auto pack_pair = [&](int tile) {
    pack(tile);  // the cilia's tiles
    const int ncil_tiles = ncil > 0 ? cil_tile[ncil - 1] + 1 : 0;
    fill.resize(ncil_tiles);
    for (long b = 0; b < nb; ++b)
      if (owner[b] < 0) slot_of[b] = -1;
    // beads per patch: a third of a tile (swimmer64 float64 MD per launch:
    // 0.374 ms against 0.382 at half a tile and 0.399 at a quarter;
    // MPCD_MD_PATCH=n overrides)
    const char* pe = std::getenv("MPCD_MD_PATCH");
    const int cap = std::max(1, std::min(tile, pe ? std::atoi(pe) : tile / 3));
    std::vector<long> idx;
    std::vector<std::pair<size_t, size_t>> todo;
    for (long b = 0; b < nb;) {
      if (owner[b] >= 0) {
        ++b;
        continue;
      }
      long e = b;
      while (e < nb && owner[e] < 0) ++e;
      idx.clear();
      for (long k = b; k < e; ++k) idx.push_back(k);
      todo.assign(1, {0, idx.size()});
      while (!todo.empty()) {  // depth first, left part first: patches in a fixed order
        const auto [lo, hi] = todo.back();
        todo.pop_back();
        const size_t n = hi - lo;
        if ((int)n <= cap) {
          fill.push_back(0);
          const int t = (int)fill.size() - 1;
          for (size_t k = lo; k < hi; ++k) slot_of[idx[k]] = t * tile + fill[t]++;
          continue;
        }
        double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
        for (size_t k = lo; k < hi; ++k)
          for (int d = 0; d < 3; ++d) {
            mn[d] = std::min(mn[d], in.bpos[3 * idx[k] + d]);
            mx[d] = std::max(mx[d], in.bpos[3 * idx[k] + d]);
          }
        int ax = 0;
        for (int d = 1; d < 3; ++d)
          if (mx[d] - mn[d] > mx[ax] - mn[ax]) ax = d;
        const size_t parts = (n + cap - 1) / cap, left = n * (parts / 2) / parts;
        std::nth_element(idx.begin() + lo, idx.begin() + lo + left, idx.begin() + hi, [&](long p, long q) {
          const double a = in.bpos[3 * p + ax], c = in.bpos[3 * q + ax];
          return a < c || (a == c && p < q);
        });
        todo.push_back({lo + left, hi});
        todo.push_back({lo, lo + left});
      }
      b = e;
    }
    return (int)fill.size();
  };
  // Cluster packing (split arithmetic): runs of consecutive non-cilium beads
  // wider than 64 slots (a sphere, whose centre bead reaches every surface
  // bead) each stay whole in one tile; cilia follow in order (next fit, so a
  // tile's cilia have contiguous bond tables); the remaining beads fill gaps.
  bool keep_hubs_whole = false;  // one-lane layout: hub runs stay in one tile (reactions)
  auto pack_cluster = [&](int tile) {
    fill.clear();
    std::fill(slot_of.begin(), slot_of.end(), -1);
    std::vector<std::pair<long, long>> runs;  // [begin, end) of non-cilium beads
    for (long b = 0; b < nb;) {
      if (owner[b] >= 0) {
        ++b;
        continue;
      }
      long e = b;
      while (e < nb && owner[e] < 0) ++e;
      runs.push_back({b, e});
      b = e;
    }
    std::vector<char> placed(nb, 0);
    for (auto& r : runs) {
      long w = 0;
      bool has_hub = false;
      for (long b = r.first; b < r.second; ++b) {
        w += width[b];
        has_hub = has_hub || hub[b];
      }
      if (has_hub && keep_hubs_whole && w > tile) return 1 << 20;  // a hub's run must stay whole
      if (w <= 64 || w > tile) continue;
      fill.push_back(0);
      const int t = (int)fill.size() - 1;
      for (long b = r.first; b < r.second; ++b) {
        slot_of[b] = t * tile + fill[t];
        fill[t] += width[b];
        placed[b] = 1;
      }
    }
    const int first_cil_tile = (int)fill.size();
    for (int c = 0; c < ncil; ++c) {
      const mpcd_cilium& cl = in.cil[c];
      int w = 0;
      for (int k = 0; k < 3 * cl.rodlength; ++k) w += width[cl.bead0 + k];
      if ((int)fill.size() == first_cil_tile || fill.back() + w > tile) fill.push_back(0);
      const int t = (int)fill.size() - 1;
      cil_tile[c] = t;
      for (int k = 0; k < 3 * cl.rodlength; ++k) {
        slot_of[cl.bead0 + k] = t * tile + fill[t];
        fill[t] += width[cl.bead0 + k];
      }
    }
    for (long b = 0; b < nb; ++b) {
      if (owner[b] >= 0 || placed[b]) continue;
      size_t t = 0;
      while (t < fill.size() && fill[t] + width[b] > tile) ++t;
      if (t == fill.size()) fill.push_back(0);
      slot_of[b] = (int)t * tile + fill[t];
      fill[t] += width[b];
    }
    return (int)fill.size();
  };
  // slot widths of a cluster layout with `lanes` threads per slot
  auto cluster_widths = [&](int lanes) {
    // one lane per slot: chunks of 15 springs keep every cilium bead (up to
    // 8 filament springs plus 6 attachment springs) on one slot, so that a
    // cilium needs one slot per bead; hubs take their force from reactions
    const int chunk = lanes == 2 ? kChunk : std::min(kChunk, 15);
    keep_hubs_whole = lanes == 1;
    for (long b = 0; b < nb; ++b)
      width[b] = (hub[b] && keep_hubs_whole) ? 1 : 1 + (nspr[b] > chunk ? (nspr[b] + chunk - 1) / chunk - 1 : 0);
    cl_chunk = chunk;
    pad_cilia();
    maxw = widest();
  };
  int tile = 0;
  out.cluster = 0;
  if (forced) {
    if (!in.split) return "a fixed cluster layout needs split arithmetic";
    if (force.lanes < 1 || force.lanes > 2 || force.tile < 32 || force.tile * force.lanes > 1024 || force.tile % 32)
      return "invalid fixed cluster layout";
    cluster_widths(force.lanes);
    if (maxw > force.tile) return "a cilium does not fit into one MD tile of the fixed layout";
    if (pack_cluster(force.tile) > 16) {
      // a hub whose run of beads cannot stay in one tile keeps its own spring
      // list (helper slots) instead of reactions
      bool any_hub = false;
      for (long b = 0; b < nb && !any_hub; ++b) any_hub = hub[b] != 0;
      if (any_hub && !no_react) return plan_md(in, force, allow_cluster, true, grid_f32cells, out, min_tile);
      return "the MD bead set needs more than 16 tiles of the fixed layout";
    }
    tile = force.tile;
    out.cluster = 1;
    out.cl_lanes = force.lanes;
  } else if (in.split && allow_cluster) {
    int lanes_hi = 2, lanes_lo = 1;
    if (const char* env = std::getenv("MPCD_MD_LANES")) lanes_hi = lanes_lo = std::max(1, std::min(2, std::atoi(env)));
    for (int lanes = lanes_hi; lanes >= lanes_lo && !out.cluster; --lanes) {
      cluster_widths(lanes);
      const int tmax = 1024 / lanes;
      for (int t = std::max(32, ((maxw + 31) / 32) * 32); t <= tmax; t += 32)
        if (pack_cluster(t) <= 16) {
          tile = t;
          out.cluster = 1;
          out.cl_lanes = lanes;
          break;
        }
    }
  }
  if (out.cluster && !keep_hubs_whole) {  // two-lane layout: hubs keep their own lists and helpers
    std::fill(hub.begin(), hub.end(), 0);
    std::fill(react.begin(), react.end(), 0);
    std::fill(dropped.begin(), dropped.end(), 0);
  }
  if (!out.cluster) {
    width = width_grid;
    cl_chunk = kChunk;
    std::fill(hub.begin(), hub.end(), 0);
    std::fill(react.begin(), react.end(), 0);
    std::fill(dropped.begin(), dropped.end(), 0);
    maxw = widest();
    // the narrowest tile that holds the widest cilium (more CTAs, more lanes
    // per slot), unless a wider one is asked for: the grid must be co-resident
    tile = std::max(std::max(32, min_tile), ((maxw + 15) / 16) * 16);
    if (tile > 256) return "an MD group needs more than 256 slots";  // four threads per slot
    if (in.pair)
      pack_pair(tile);
    else
      pack(tile);
  }
  // a hub and all its partners must share one tile, one hub per tile
  {
    const int nt = (int)fill.size();
    out.tile_react.assign(nt, -1);
    bool bad = false;
    for (long b = 0; b < nb && !bad; ++b) {
      if (!hub[b]) continue;
      const int t = slot_of[b] / tile;
      if (out.tile_react[t] >= 0) bad = true;
      out.tile_react[t] = slot_of[b] - t * tile;
    }
    for (long i = 0; i < nsp && !bad; ++i)
      if (react[i] && slot_of[in.sp_t[i]] / tile != slot_of[in.sp_o[i]] / tile) bad = true;
    if (bad) return plan_md(in, force, allow_cluster, true, grid_f32cells, out, min_tile);
  }
  // Hubs of the pair kernel: a bead outside the cilia with more than
  // kPairLong springs, each with an exact reverse partner (a sphere's centre,
  // src/sphere.cpp:87-96), whose neighbours are not such beads themselves.
  // Its own list is dropped; its force is the negated sum of its partners'
  // forces, which the tiles holding the partners add up and publish, and
  // every tile that reaches the hub integrates a copy of it.
  std::vector<char> phub(nb, 0);
  const char* nh_env = std::getenv("MPCD_MD_NO_HUBS");  // 1: hubs keep their own lists (diagnostics)
  if (in.pair && !no_react && !(nh_env && std::atoi(nh_env))) {
    auto candidate = [&](long b) { return owner[b] < 0 && nspr[b] > kPairLong; };
    for (long b = 0; b < nb; ++b) {
      if (!candidate(b)) continue;
      std::vector<int> partners;
      bool ok = true;
      for (int q = bstart[b]; q < bstart[b + 1] && ok; ++q) {
        const int i = blist[q];
        const int o = in.sp_o[i];
        if (o == b || candidate(o)) {
          ok = false;
          break;
        }
        int found = -1;
        for (int r = bstart[o]; r < bstart[o + 1]; ++r) {
          const int j = blist[r];
          if (in.sp_o[j] != b || in.sp_k[j] != in.sp_k[i] || in.sp_kk[j] != in.sp_kk[i] || react[j]) continue;
          if (in.sp_k[i] >= MPCD_SPRING_BOND ? in.sp_r[j] != in.sp_r[i] : in.sp_rest[j] != in.sp_rest[i]) continue;
          found = j;
          break;
        }
        if (found < 0) ok = false;
        else partners.push_back(found);
      }
      if (!ok) continue;
      phub[b] = 1;
      for (int j : partners) react[j] = 1;
      for (int q = bstart[b]; q < bstart[b + 1]; ++q) dropped[blist[q]] = 1;
    }
  }
  out.tile = tile;
  out.ntiles = (int)fill.size();
  out.nslots = out.ntiles * tile;
  const int ns = out.nslots;
  out.X.assign(ns, 0.0);
  out.Y.assign(ns, 0.0);
  out.Z.assign(ns, 0.0);
  out.VX.assign(ns, 0.0);
  out.VY.assign(ns, 0.0);
  out.VZ.assign(ns, 0.0);
  out.mv.assign(ns, -1);
  out.prim.assign(ns, 0);
  out.nhelp.assign(ns, 0);
  out.thelp.assign(out.ntiles, 0);
  for (long b = 0; b < nb; ++b) {
    const int s = slot_of[b];
    out.X[s] = in.bpos[3 * b];
    out.Y[s] = in.bpos[3 * b + 1];
    out.Z[s] = in.bpos[3 * b + 2];
    out.VX[s] = in.bvel[3 * b];
    out.VY[s] = in.bvel[3 * b + 1];
    out.VZ[s] = in.bvel[3 * b + 2];
    out.mv[s] = in.bmoves[b] ? 1 : 0;
    out.prim[s] = s;
    out.nhelp[s] = width[b] - 1;
    for (int k = 1; k < width[b]; ++k) {
      out.mv[s + k] = 2;
      out.prim[s + k] = s;
      out.X[s + k] = out.X[s];
      out.Y[s + k] = out.Y[s];
      out.Z[s + k] = out.Z[s];
    }
    if (width[b] > 1) out.thelp[s / tile] = 1;
  }
  // springs: CSR by slot; a bead's list (in input order) is cut into chunks
  // over its primary and helper slots
  std::vector<int>& start = out.start;
  start.assign(ns + 1, 0);
  std::vector<int> seen(nb, 0);
  std::vector<int> sslot(nsp);
  for (long i = 0; i < nsp; ++i) {
    if (dropped[i]) {
      sslot[i] = -1;
      continue;
    }
    const int b = in.sp_t[i];
    const int chunk = width[b] > 1 ? seen[b] / cl_chunk : 0;
    seen[b]++;
    sslot[i] = slot_of[b] + chunk;
    start[sslot[i] + 1]++;
  }
  for (int s = 0; s < ns; ++s) start[s + 1] += start[s];
  std::vector<int> pos(start.begin(), start.end() - 1);
  const long nspk = start[ns];  // springs kept
  out.so.assign(nspk, 0);
  out.sk.assign(nspk, 0);
  out.sr.assign(nspk, 0);
  out.srest.assign(nspk, 0.0);
  out.sm2k.assign(nspk, 0.0);
  for (long i = 0; i < nsp; ++i) {
    if (sslot[i] < 0) continue;
    const int d = pos[sslot[i]]++;
    out.so[d] = slot_of[in.sp_o[i]];
    out.sk[d] = in.sp_k[i] | (react[i] ? kSpringReact : 0);
    out.sr[d] = in.sp_r[i];
    out.srest[d] = in.sp_rest[i];
    out.sm2k[d] = -2.0 * in.sp_kk[i];
  }
  // cluster layouts: every slot's list sorted (stably) by spring group, so
  // that the kernel runs one loop per group without testing kinds
  if (out.cluster) {
    std::vector<int> idx;
    for (int sl_ = 0; sl_ < ns; ++sl_) {
      const int a0 = start[sl_], a1 = start[sl_ + 1];
      if (a1 - a0 < 2) continue;
      idx.resize(a1 - a0);
      for (int k = 0; k < a1 - a0; ++k) idx[k] = a0 + k;
      std::stable_sort(idx.begin(), idx.end(),
                       [&](int x, int y) { return spring_group(out.sk[x]) < spring_group(out.sk[y]); });
      std::vector<int> so(a1 - a0), sk(a1 - a0), sr(a1 - a0);
      std::vector<double> srest(a1 - a0), sm2k(a1 - a0);
      for (int k = 0; k < a1 - a0; ++k) {
        so[k] = out.so[idx[k]];
        sk[k] = out.sk[idx[k]];
        sr[k] = out.sr[idx[k]];
        srest[k] = out.srest[idx[k]];
        sm2k[k] = out.sm2k[idx[k]];
      }
      for (int k = 0; k < a1 - a0; ++k) {
        out.so[a0 + k] = so[k];
        out.sk[a0 + k] = sk[k];
        out.sr[a0 + k] = sr[k];
        out.srest[a0 + k] = srest[k];
        out.sm2k[a0 + k] = sm2k[k];
      }
    }
  }
  // halos: per tile the distinct slots of other tiles its springs reach, and
  // every spring's other bead as an index into the tile's staged positions
  std::vector<char> hub_at(ns, 0);  // slots of the pair kernel's hubs
  std::vector<int> hub_slots;
  for (long b = 0; b < nb; ++b)
    if (phub[b]) {
      hub_at[slot_of[b]] = 1;
      hub_slots.push_back(slot_of[b]);
    }
  out.sl.assign(nspk, 0);
  out.hstart.assign(out.ntiles + 1, 0);
  out.df_runs.clear();
  out.df_run_start.assign(1, 0);
  out.df_single.clear();
  out.df_single_start.assign(1, 0);
  int hmax = 0;
  for (int t = 0; t < out.ntiles; ++t) {
    const int b0 = t * tile, b1 = b0 + tile;
    std::vector<int> ext;
    for (int s2 = start[b0]; s2 < start[b1]; ++s2)
      if (out.so[s2] < b0 || out.so[s2] >= b1) ext.push_back(out.so[s2]);
    std::sort(ext.begin(), ext.end());
    ext.erase(std::unique(ext.begin(), ext.end()), ext.end());
    for (int s2 = start[b0]; s2 < start[b1]; ++s2) {
      if (out.so[s2] >= b0 && out.so[s2] < b1)
        out.sl[s2] = out.so[s2] - b0;
      else
        out.sl[s2] = tile + (int)(std::lower_bound(ext.begin(), ext.end(), out.so[s2]) - ext.begin());
    }
    out.hstart[t + 1] = out.hstart[t] + (int)ext.size();
    out.halo.insert(out.halo.end(), ext.begin(), ext.end());
    // double-float kernel: runs of at least kLongRun consecutive slots (the
    // sphere centre's tile reaches the whole sphere in a few such runs) go as
    // one bulk copy (TMA) each, the other entries one by one (cp.async); short
    // runs by bulk copy measured slower.  MPCD_MD_LONG_RUN=n overrides.
    const char* lr_env = std::getenv("MPCD_MD_LONG_RUN");
    const size_t kLongRun = lr_env ? (size_t)std::max(1, std::atoi(lr_env)) : (size_t)32;
    // (a pair-kernel hub keeps its staged place but is never copied: every
    // tile that reaches it integrates its own copy)
    for (size_t i = 0; i < ext.size();) {
      if (hub_at[ext[i]]) {
        ++i;
        continue;
      }
      size_t e = i + 1;
      while (e < ext.size() && ext[e] == ext[e - 1] + 1 && !hub_at[ext[e]]) ++e;
      if (e - i >= kLongRun)
        out.df_runs.push_back({ext[i], (int)i, (int)(e - i), 0});
      else
        for (size_t k = i; k < e; ++k) out.df_single.push_back({ext[k], (int)k});
      i = e;
    }
    out.df_run_start.push_back((int)out.df_runs.size());
    out.df_single_start.push_back((int)out.df_single.size());
    out.df_nrun_max = std::max(out.df_nrun_max, out.df_run_start[t + 1] - out.df_run_start[t]);
    out.df_nsingle_max = std::max(out.df_nsingle_max, out.df_single_start[t + 1] - out.df_single_start[t]);
    hmax = std::max(hmax, (int)ext.size());
  }
  out.hmax = hmax;
  // double-float grid kernel: per slot, the springs whose other bead is in the
  // tile first (they run while the halo loads are in flight); per tile, the
  // bond range its BOND/DIAG springs and cilia use; packed spring codes
  if (out.df) {
    out.df_split.assign(ns, 0);
    out.df_code.assign(nspk, 0u);
    out.df_b0.assign(out.ntiles, 0);
    out.df_nb.assign(out.ntiles, 0);
    std::vector<int> b0(out.ntiles, INT_MAX), b1(out.ntiles, 0);
    for (int c = 0; c < ncil; ++c) {
      const int t = cil_tile[c];
      b0[t] = std::min(b0[t], in.cil[c].bond_base);
      b1[t] = std::max(b1[t], in.cil[c].bond_base + in.cil[c].rodlength);
    }
    for (int t = 0; t < out.ntiles; ++t) {
      if (b0[t] > b1[t]) b0[t] = b1[t] = 0;
      out.df_b0[t] = b0[t];
      out.df_nb[t] = b1[t] - b0[t];
      out.df_nb_max = std::max(out.df_nb_max, out.df_nb[t]);
      out.df_nsp_max = std::max(out.df_nsp_max, start[(t + 1) * tile] - start[t * tile]);
    }
    std::vector<long> idx;
    for (int sl_ = 0; sl_ < ns; ++sl_) {
      const int a0 = start[sl_], a1 = start[sl_ + 1];
      idx.clear();
      for (int k = a0; k < a1; ++k)
        if (out.sl[k] < tile) idx.push_back(k);
      out.df_split[sl_] = a0 + (int)idx.size();
      for (int k = a0; k < a1; ++k)
        if (out.sl[k] >= tile) idx.push_back(k);
      std::vector<int> so(a1 - a0), sk(a1 - a0), sr(a1 - a0), slv(a1 - a0);
      std::vector<double> srest(a1 - a0), sm2k(a1 - a0);
      for (int k = 0; k < a1 - a0; ++k) {
        so[k] = out.so[idx[k]];
        sk[k] = out.sk[idx[k]];
        sr[k] = out.sr[idx[k]];
        slv[k] = out.sl[idx[k]];
        srest[k] = out.srest[idx[k]];
        sm2k[k] = out.sm2k[idx[k]];
      }
      const int t = sl_ / tile;
      for (int k = 0; k < a1 - a0; ++k) {
        const int d = a0 + k;
        out.so[d] = so[k];
        out.sk[d] = sk[k];
        out.sr[d] = sr[k];
        out.sl[d] = slv[k];
        out.srest[d] = srest[k];
        out.sm2k[d] = sm2k[k];
        const int kind = sk[k] & 3;
        int lref = 0;
        if (kind >= MPCD_SPRING_BOND) {
          lref = sr[k] - out.df_b0[t];
          if (lref < 0 || lref >= out.df_nb[t]) return "a bond spring refers to a bond outside its tile's cilia";
        }
        if (slv[k] >= (1 << 16) || lref >= (1 << 14)) return "an MD tile is too large for packed spring codes";
        out.df_code[d] = (uint32_t)slv[k] | ((uint32_t)kind << 16) | ((uint32_t)lref << 18);
      }
    }
  }
  if (in.pair) {
    if (!out.df) return "the pair kernel needs the double-float grid layout";
    const std::string e = plan_pair_tables(out, hub_slots);
    if (e == "hub") return plan_md(in, force, allow_cluster, true, grid_f32cells, out, min_tile);  // no hubs then
    if (!e.empty()) return e;
    out.pair = in.pair;
  }
  MDState probe;  // the fields the feasibility checks read
  probe.pair = out.pair;
  probe.pr_nent_max = out.pr_nent_max;
  probe.pr_ninc_max = out.pr_ninc_max;
  probe.pr_nlong_max = out.pr_nlong_max;
  probe.tile = tile;
  probe.ntiles = out.ntiles;
  probe.nslots = ns;
  probe.hmax = hmax;
  probe.split = out.split;
  probe.df = out.df;
  probe.df_nsp_max = out.df_nsp_max;
  probe.df_nb_max = out.df_nb_max;
  probe.df_nrun_max = out.df_nrun_max;
  probe.df_nsingle_max = out.df_nsingle_max;
  probe.cluster = out.cluster;
  probe.cl_lanes = out.cl_lanes;
  if (out.cluster) {
    // per-tile maxima for the cluster kernel's shared-memory layout
    std::vector<int> tb(out.ntiles, 0);
    for (int c = 0; c < ncil; ++c) tb[cil_tile[c]] += in.cil[c].rodlength;
    for (int t = 0; t < out.ntiles; ++t) {
      out.cl_nsp_max = std::max(out.cl_nsp_max, start[(t + 1) * tile] - start[t * tile]);
      out.cl_nbond_max = std::max(out.cl_nbond_max, tb[t]);
    }
    probe.cl_nsp_max = out.cl_nsp_max;
    probe.cl_nbond_max = out.cl_nbond_max;
    probe.cl_nbuf = 2;
    if (!md_cluster_feasible(probe)) {
      probe.cl_nbuf = 1;  // one position buffer and a second cluster barrier per substep
      out.cl_nbuf = 1;
    }
    if (!md_cluster_feasible(probe)) {
      if (forced) return "the fixed cluster layout does not fit on the device";
      return plan_md(in, force, false, no_react, grid_f32cells, out, min_tile);  // grid layout instead
    }
  } else {
    const int cap = md_max_coresident_blocks(probe, grid_f32cells);
    if (out.ntiles > cap) {
      // a large bead set: wider tiles (fewer CTAs; the double-float kernel
      // then runs four, then two lanes per slot)
      if (tile < 256) return plan_md(in, force, allow_cluster, no_react, grid_f32cells, out, tile < 128 ? 128 : 256);
      return "MD tiles exceed the co-resident CTA limit of the device";
    }
  }
  // cilia
  out.cd.assign(ncil, CiliumDev{});
  out.mid.assign(ncil, 0.0);
  out.ts.assign(ncil, 0.0);
  out.tcil.assign(out.ntiles + 1, 0);
  for (int c = 0; c < ncil; ++c) {
    const mpcd_cilium& cl = in.cil[c];
    CiliumDev& d = out.cd[c];
    d.stride = width[cl.bead0];
    d.kind = cl.kind;
    d.len = cl.rodlength;
    d.num_anker = cl.num_anker;
    d.slot0 = slot_of[cl.bead0];
    d.bond_base = cl.bond_base;
    d.beatstrength = cl.beatstrength;
    d.bending = cl.bending;
    d.max_bend = cl.max_bend;
    d.m_speed = cl.m_speed;
    d.power_dur = cl.power_stroke_duration;
    d.recovery_dur = cl.recovery_stroke_duration;
    d.start = cl.start;
    out.mid[c] = cl.midpnt;
    out.ts[c] = cl.tstroke;
    out.tcil[cil_tile[c] + 1]++;
  }
  for (int t = 0; t < out.ntiles; ++t) out.tcil[t + 1] += out.tcil[t];
  out.newlen.assign(in.newlen, in.newlen + in.nbond);
  out.oldlen.assign(in.oldlen, in.oldlen + in.nbond);
  out.diag.resize(in.nbond);
  for (long k = 0; k < in.nbond; ++k) out.diag[k] = std::sqrt(0.5 * 0.5 + 0.5 * in.newlen[k]);
  out.slot_of = slot_of;
  return "";
}

}  // namespace mpcd
