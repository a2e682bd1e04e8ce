// axg_plan.cpp -- patch construction, patch colouring and sub-round split.
// See axg_plan.h for what the kernels require of the plan.
#include "axg_plan.h"

#include <algorithm>
#include <cstring>
#include <numeric>
#include <system_error>
#include <thread>
#include <utility>

namespace axg {

namespace {

// point -> elements (CSR), elements listed in increasing order
struct PointElems {
  std::vector<int64_t> start;
  std::vector<int32_t> elems;
};

PointElems point_elements(const int32_t *igloc, int64_t nel, int64_t nglob) {
  PointElems pe;
  pe.start.assign(nglob + 1, 0);
  for (int64_t p = 0; p < 25 * nel; ++p) pe.start[igloc[p]]++;  // igloc is 1-based
  for (int64_t g = 0; g < nglob; ++g) pe.start[g + 1] += pe.start[g];
  pe.elems.resize(25 * nel);
  std::vector<int64_t> fill(pe.start.begin(), pe.start.end() - 1);
  for (int64_t e = 0; e < nel; ++e)
    for (int k = 0; k < 25; ++k) {
      const int64_t g = igloc[25 * e + k] - 1;
      // an element lists a point once even if it appears twice (degenerate)
      const int64_t s = pe.start[g];
      bool dup = false;
      for (int64_t q = s; q < fill[g]; ++q)
        if (pe.elems[q] == e) dup = true;
      if (!dup) pe.elems[fill[g]++] = (int32_t)e;
    }
  // compact duplicates (never happens on valid meshes)
  for (int64_t g = 0; g < nglob; ++g)
    for (int64_t q = fill[g]; q < pe.start[g + 1]; ++q) pe.elems[q] = -1;
  return pe;
}

}  // namespace

std::string build_plan(const int32_t *igloc, int64_t nel, int64_t nglob, int patch_elems, int growth,
                       const std::vector<uint8_t> &prepass, DomainPlan &plan, bool renumber) {
  plan = DomainPlan();
  plan.nel = nel;
  plan.nglob = nglob;
  if (patch_elems < 1 || patch_elems > kMaxPatchElems) return "patch_elems out of range";
  if (growth != kGrowCompact && growth != kGrowLayered) return "unknown patch growth";
  plan.patch_elems = patch_elems;
  plan.growth = growth;
  if (nel == 0) {
    plan.colour_start.assign(1, 0);
    return "";
  }
  if (nglob <= 0 || nglob > (int64_t)kPtIndexMask) return "nglob out of range";
  for (int64_t p = 0; p < 25 * nel; ++p)
    if (igloc[p] < 1 || igloc[p] > nglob) return "igloc entry outside 1..nglob";

  const PointElems pe = point_elements(igloc, nel, nglob);

  // ---- 1. patches -----------------------------------------------------------
  // Seeds are taken in element order (the lowest unassigned element).
  //  compact: the next member is the candidate sharing the most points with
  //           the patch (ties: lowest element);
  //  layered: breadth-first layers of point-sharing neighbours, inside a layer
  //           the candidates sharing the most points first.  From the corner of
  //           a structured block a patch of k^2 elements is a k x k square.
  plan.patch_of_elem.assign(nel, -1);
  std::vector<int32_t> score(nel, 0);
  std::vector<int32_t> cand;
  std::vector<std::vector<int32_t>> patches;
  int64_t next_seed = 0;
  const bool layered = growth == kGrowLayered;
  std::vector<uint32_t> ptstamp(nglob, 0), elstamp(nel, 0), inlayer(nel, 0);
  uint32_t stamp = 0, layer_id = 0;
  std::vector<int32_t> dirty;
  while (layered) {
    while (next_seed < nel && plan.patch_of_elem[next_seed] >= 0) ++next_seed;
    if (next_seed >= nel) break;
    const int32_t pid = (int32_t)patches.size();
    ++stamp;
    std::vector<int32_t> members{(int32_t)next_seed}, layer{(int32_t)next_seed}, next;
    plan.patch_of_elem[next_seed] = pid;
    elstamp[next_seed] = stamp;
    int npts = 0;  // distinct points of the patch
    for (int k = 0; k < 25; ++k) {
      const int64_t g = igloc[25 * next_seed + k] - 1;
      npts += ptstamp[g] != stamp;
      ptstamp[g] = stamp;
    }
    while ((int)members.size() < patch_elems) {
      next.clear();
      for (int32_t e : layer)
        for (int k = 0; k < 25; ++k) {
          const int64_t g = igloc[25 * (int64_t)e + k] - 1;
          for (int64_t q = pe.start[g]; q < pe.start[g + 1]; ++q) {
            const int32_t e2 = pe.elems[q];
            if (e2 < 0 || plan.patch_of_elem[e2] >= 0 || elstamp[e2] == stamp) continue;
            elstamp[e2] = stamp;
            next.push_back(e2);
          }
        }
      if (next.empty()) break;
      for (int32_t c : next) {
        score[c] = 0;
        for (int k = 0; k < 25; ++k) score[c] += ptstamp[igloc[25 * (int64_t)c + k] - 1] == stamp;
      }
      std::stable_sort(next.begin(), next.end(), [&](int32_t a, int32_t b) {
        return score[a] != score[b] ? score[a] > score[b] : a < b;
      });
      ++layer_id;
      for (int32_t c : next) inlayer[c] = layer_id;
      layer.clear();
      for (int32_t c : next) {
        if ((int)members.size() >= patch_elems) break;
        const int add = 25 - score[c];  // points not yet in the patch
        if (npts + add > kMaxPatchPoints) continue;
        npts += add;
        plan.patch_of_elem[c] = pid;
        members.push_back(c);
        layer.push_back(c);
        // later candidates of this layer may now share more points: those
        // holding a point c brings into the patch are counted again
        dirty.clear();
        for (int k = 0; k < 25; ++k) {
          const int64_t g = igloc[25 * (int64_t)c + k] - 1;
          if (ptstamp[g] == stamp) continue;
          ptstamp[g] = stamp;
          for (int64_t q = pe.start[g]; q < pe.start[g + 1]; ++q) {
            const int32_t e2 = pe.elems[q];
            if (e2 >= 0 && inlayer[e2] == layer_id && plan.patch_of_elem[e2] < 0) dirty.push_back(e2);
          }
        }
        for (int32_t c2 : dirty) {
          int sc = 0;
          for (int k = 0; k < 25; ++k) sc += ptstamp[igloc[25 * (int64_t)c2 + k] - 1] == stamp;
          score[c2] = sc;
        }
      }
      if (layer.empty()) break;
      for (int32_t c : next) score[c] = 0;
    }
    patches.push_back(std::move(members));
  }
  while (!layered) {
    while (next_seed < nel && plan.patch_of_elem[next_seed] >= 0) ++next_seed;
    if (next_seed >= nel) break;
    const int32_t pid = (int32_t)patches.size();
    std::vector<int32_t> members;
    cand.clear();
    ++stamp;  // ptstamp: points in the patch; elstamp: candidates over the point cap
    int npts = 0;
    int32_t add = (int32_t)next_seed;
    while (true) {
      plan.patch_of_elem[add] = pid;
      members.push_back(add);
      score[add] = 0;
      for (int k = 0; k < 25; ++k) {
        const int64_t g = igloc[25 * (int64_t)add + k] - 1;
        npts += ptstamp[g] != stamp;
        ptstamp[g] = stamp;
      }
      if ((int)members.size() >= patch_elems) break;
      for (int k = 0; k < 25; ++k) {
        const int64_t g = igloc[25 * (int64_t)add + k] - 1;
        for (int64_t q = pe.start[g]; q < pe.start[g + 1]; ++q) {
          const int32_t e2 = pe.elems[q];
          if (e2 < 0 || plan.patch_of_elem[e2] >= 0) continue;
          if (score[e2] == 0) cand.push_back(e2);
          score[e2]++;
        }
      }
      int32_t best = -1;
      while (true) {
        best = -1;
        for (int32_t c : cand) {
          if (plan.patch_of_elem[c] >= 0 || elstamp[c] == stamp) continue;
          if (best < 0 || score[c] > score[best] || (score[c] == score[best] && c < best)) best = c;
        }
        if (best < 0) break;
        int extra = 0;
        for (int k = 0; k < 25; ++k) extra += ptstamp[igloc[25 * (int64_t)best + k] - 1] != stamp;
        if (npts + extra <= kMaxPatchPoints) break;
        elstamp[best] = stamp;  // would overflow the patch's points
      }
      if (best < 0) break;
      add = best;
    }
    for (int32_t c : cand) score[c] = 0;
    patches.push_back(std::move(members));
  }
  // ---- 1b. fragments: growth can leave small holes between full patches;
  // each patch of fewer than patch_elems / 4 elements is merged into the
  // adjacent patch with the fewest elements that can take it (the merged
  // patch stays within kMaxPatchElems elements and kMaxPatchPoints points).
  // A fragment costs a whole gather / write-back cycle for a few elements.
  {
    const int small = std::max(1, patch_elems / 4);
    std::vector<int32_t> npts(patches.size(), -1);
    std::vector<uint32_t> seen(nglob, 0);
    uint32_t mstamp = 0;
    auto count_points = [&](const std::vector<int32_t> &a, const std::vector<int32_t> *b) {
      ++mstamp;
      int32_t n = 0;
      for (const std::vector<int32_t> *v : {&a, b}) {
        if (!v) continue;
        for (int32_t e : *v)
          for (int k = 0; k < 25; ++k) {
            const int64_t g = igloc[25 * (int64_t)e + k] - 1;
            if (seen[g] != mstamp) {
              seen[g] = mstamp;
              ++n;
            }
          }
      }
      return n;
    };
    for (size_t p = 0; p < patches.size(); ++p) {
      if (patches[p].empty() || (int)patches[p].size() >= small) continue;
      // neighbouring patches, best = fewest elements that fit
      int32_t best = -1;
      for (int32_t e : patches[p])
        for (int k = 0; k < 25; ++k) {
          const int64_t g = igloc[25 * (int64_t)e + k] - 1;
          for (int64_t q = pe.start[g]; q < pe.start[g + 1]; ++q) {
            const int32_t e2 = pe.elems[q];
            if (e2 < 0) continue;
            const int32_t p2 = plan.patch_of_elem[e2];
            if (p2 == (int32_t)p) continue;
            if (patches[p2].size() + patches[p].size() > (size_t)kMaxPatchElems) continue;
            if (best >= 0 && (patches[p2].size() > patches[best].size() ||
                              (patches[p2].size() == patches[best].size() && p2 >= best)))
              continue;
            if (count_points(patches[p2], &patches[p]) > kMaxPatchPoints) continue;
            best = p2;
          }
        }
      if (best < 0) continue;
      for (int32_t e : patches[p]) {
        plan.patch_of_elem[e] = best;
        patches[best].push_back(e);
      }
      patches[p].clear();
    }
    // renumber the surviving patches in creation order
    std::vector<std::vector<int32_t>> kept;
    for (auto &v : patches)
      if (!v.empty()) {
        for (int32_t e : v) plan.patch_of_elem[e] = (int32_t)kept.size();
        kept.push_back(std::move(v));
      }
    patches.swap(kept);
  }
  plan.n_patches = (int32_t)patches.size();

  // ---- 2. colour the patches (greedy, creation order) --------------------
  plan.colour_of_patch.assign(plan.n_patches, -1);
  std::vector<int32_t> mark(64, -1);
  int32_t ncol = 0;
  for (int32_t p = 0; p < plan.n_patches; ++p) {
    for (int32_t e : patches[p])
      for (int k = 0; k < 25; ++k) {
        const int64_t g = igloc[25 * (int64_t)e + k] - 1;
        for (int64_t q = pe.start[g]; q < pe.start[g + 1]; ++q) {
          const int32_t e2 = pe.elems[q];
          if (e2 < 0) continue;
          const int32_t p2 = plan.patch_of_elem[e2];
          if (p2 == p) continue;
          const int32_t c2 = plan.colour_of_patch[p2];
          if (c2 >= 0) {
            if (c2 >= (int32_t)mark.size()) mark.resize(c2 + 1, -1);
            mark[c2] = p;
          }
        }
      }
    int32_t c = 0;
    while (c < (int32_t)mark.size() && mark[c] == p) ++c;
    if (c >= (int32_t)mark.size()) mark.resize(c + 1, -1);
    plan.colour_of_patch[p] = c;
    ncol = std::max(ncol, c + 1);
  }
  plan.n_colours = ncol;

  // launch order of patches: by colour, then creation order
  std::vector<int32_t> order(plan.n_patches);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
    return plan.colour_of_patch[a] < plan.colour_of_patch[b];
  });
  plan.colour_start.assign(ncol + 1, 0);
  for (int32_t p = 0; p < plan.n_patches; ++p) plan.colour_start[plan.colour_of_patch[p] + 1]++;
  for (int32_t c = 0; c < ncol; ++c) plan.colour_start[c + 1] += plan.colour_start[c];

  // ---- 2b. internal point numbering --------------------------------------
  // Points held by the same patches get consecutive numbers: grouped by the
  // first and second patch (in launch order) that hold them, in reference
  // order inside a group.  A patch's interior is then one run, each edge it
  // shares with a later patch another, so that gathers and write-backs read
  // and write whole sectors instead of rows scattered over the reference's
  // numbering.
  plan.new_of_old.resize(nglob);
  plan.old_of_new.resize(nglob);
  if (!renumber) {
    std::iota(plan.new_of_old.begin(), plan.new_of_old.end(), 0);
    std::iota(plan.old_of_new.begin(), plan.old_of_new.end(), 0);
  } else {
    std::vector<int32_t> rank(plan.n_patches);
    for (int32_t lp = 0; lp < plan.n_patches; ++lp) rank[order[lp]] = lp;
    const int32_t none = plan.n_patches;  // points no element holds come last
    std::vector<int32_t> r0(nglob, none), r1(nglob, none);
    for (int64_t e = 0; e < nel; ++e) {
      const int32_t p = rank[plan.patch_of_elem[e]];
      for (int k = 0; k < 25; ++k) {
        const int64_t g = igloc[25 * e + k] - 1;
        if (p == r0[g] || p == r1[g]) continue;
        if (p < r0[g]) {
          r1[g] = r0[g];
          r0[g] = p;
        } else if (p < r1[g]) {
          r1[g] = p;
        }
      }
    }
    // order (first patch, second patch, reference number): two stable
    // counting sorts, by the second patch and then by the first
    std::vector<int64_t> fill(plan.n_patches + 2);
    auto csort = [&](const std::vector<int32_t> &key, const int32_t *in, int32_t *out) {
      std::fill(fill.begin(), fill.end(), 0);
      for (int64_t g = 0; g < nglob; ++g) fill[key[g] + 1]++;
      for (int32_t p = 0; p <= plan.n_patches; ++p) fill[p + 1] += fill[p];
      for (int64_t q = 0; q < nglob; ++q) {
        const int32_t g = in ? in[q] : (int32_t)q;
        out[fill[key[g]]++] = g;
      }
    };
    std::vector<int32_t> by_r1(nglob);
    csort(r1, nullptr, by_r1.data());
    csort(r0, by_r1.data(), plan.old_of_new.data());
    for (int64_t n = 0; n < nglob; ++n) plan.new_of_old[plan.old_of_new[n]] = (int32_t)n;
  }
  const std::vector<int32_t> &nofo = plan.new_of_old;

  // ---- 3. first / last writer per point ----------------------------------
  // colour range of the patches touching each point
  std::vector<int32_t> cmin(nglob, INT32_MAX), cmax(nglob, -1);
  for (int64_t e = 0; e < nel; ++e) {
    const int32_t c = plan.colour_of_patch[plan.patch_of_elem[e]];
    for (int k = 0; k < 25; ++k) {
      const int64_t g = igloc[25 * e + k] - 1;
      cmin[g] = std::min(cmin[g], c);
      cmax[g] = std::max(cmax[g], c);
    }
  }

  // ---- 4. sub-rounds, points, element -> point indices --------------------
  plan.meta.resize(plan.n_patches);
  plan.elem_order.resize(nel);
  plan.elem_pts.resize(25 * nel);
  plan.pt_words.clear();
  plan.pt_words.reserve((size_t)(nglob * 1.2) + 16);
  int64_t eslot = 0;
  std::vector<int32_t> round_of(kMaxPatchElems);
  std::vector<uint32_t> pts;
  std::vector<uint32_t> ptmask(nglob, 0);
  // per point (reference number): the last patch that listed it (+1); per
  // point (internal number): its index in that patch
  std::vector<int32_t> listed(nglob, 0);
  std::vector<uint16_t> local_of(nglob, 0);
  for (int32_t lp = 0; lp < plan.n_patches; ++lp) {
    const int32_t p = order[lp];
    std::vector<int32_t> mem = patches[p];
    std::sort(mem.begin(), mem.end());
    const int n = (int)mem.size();
    // greedy sub-rounds: element a goes to a round not used by an earlier
    // element of the patch that shares a point with it; among those, the
    // first round whose element count is not a multiple of the CTA's 8 warps
    // (the element then costs no extra warp iteration), else the first one
    int nrounds = 0;
    int rcount[kMaxSubrounds] = {};
    for (int a = 0; a < n; ++a) {
      uint32_t used = 0;
      for (int k = 0; k < 25; ++k) used |= ptmask[igloc[25 * (int64_t)mem[a] + k] - 1];
      int r = 0;
      while (used & (1u << r)) ++r;
      for (int q = r; q < nrounds; ++q)
        if (!(used & (1u << q)) && rcount[q] % 8 != 0) {
          r = q;
          break;
        }
      if (r >= kMaxSubrounds) return "patch needs more sub-rounds than supported";
      ++rcount[r];
      round_of[a] = r;
      nrounds = std::max(nrounds, r + 1);
      for (int k = 0; k < 25; ++k) ptmask[igloc[25 * (int64_t)mem[a] + k] - 1] |= 1u << r;
    }
    for (int a = 0; a < n; ++a)
      for (int k = 0; k < 25; ++k) ptmask[igloc[25 * (int64_t)mem[a] + k] - 1] = 0;
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return round_of[x] < round_of[y]; });
    PatchMeta &m = plan.meta[lp];
    std::memset(&m, 0, sizeof m);
    m.elem_start = (int32_t)eslot;
    m.pt_start = (int32_t)plan.pt_words.size();
    m.n_elems = (uint16_t)n;
    m.n_rounds = (uint8_t)nrounds;
    for (int r = 0; r < nrounds; ++r) {
      int cnt = 0;
      for (int a = 0; a < n; ++a) cnt += round_of[a] <= r;
      m.round_end[r] = (uint8_t)cnt;
    }
    plan.max_rounds = std::max(plan.max_rounds, nrounds);
    // unique points, sorted by internal number
    pts.clear();
    for (int a = 0; a < n; ++a)
      for (int k = 0; k < 25; ++k) {
        const int64_t g = igloc[25 * (int64_t)mem[a] + k] - 1;
        if (listed[g] == lp + 1) continue;
        listed[g] = lp + 1;
        pts.push_back((uint32_t)nofo[g]);
      }
    std::sort(pts.begin(), pts.end());
    if (pts.size() > (size_t)kMaxPatchPoints) return "patch has too many points";
    for (size_t t = 0; t < pts.size(); ++t) local_of[pts[t]] = (uint16_t)t;
    m.n_pts = (uint16_t)pts.size();
    plan.max_pts = std::max<int32_t>(plan.max_pts, (int32_t)pts.size());
    const int32_t col = plan.colour_of_patch[p];
    for (uint32_t gn : pts) {
      uint32_t w = gn;
      const int64_t g = plan.old_of_new[gn];
      const bool pre = !prepass.empty() && prepass[g];
      if (cmin[g] == col && !pre) w |= kPtFirst;
      if (cmax[g] == col) w |= kPtLast;
      plan.pt_words.push_back(w);
    }
    // the next patch's words start on a 16-byte boundary (bulk copies)
    while (plan.pt_words.size() % 4 != 0) plan.pt_words.push_back(kPtPad);
    for (int t = 0; t < n; ++t) {
      const int a = idx[t];
      const int32_t e = mem[a];
      plan.elem_order[eslot] = e;
      for (int k = 0; k < 25; ++k) plan.elem_pts[25 * eslot + k] = local_of[nofo[igloc[25 * (int64_t)e + k] - 1]];
      ++eslot;
    }
  }
  plan.total_pts = (int64_t)plan.pt_words.size();
  return "";
}

std::string validate_plan(const int32_t *igloc, int64_t nel, int64_t nglob,
                          const std::vector<uint8_t> &prepass, const DomainPlan &plan) {
  if ((int64_t)plan.patch_of_elem.size() != nel) return "patch_of_elem size";
  if (nel == 0) return "";
  std::vector<int32_t> seen(nel, 0);
  for (int64_t s = 0; s < nel; ++s) {
    const int32_t e = plan.elem_order[s];
    if (e < 0 || e >= nel) return "elem_order out of range";
    if (seen[e]++) return "element appears twice in launch order";
  }
  // the internal numbering is a permutation
  if ((int64_t)plan.new_of_old.size() != nglob || (int64_t)plan.old_of_new.size() != nglob)
    return "point numbering size";
  for (int64_t g = 0; g < nglob; ++g) {
    const int32_t n = plan.new_of_old[g];
    if (n < 0 || n >= nglob || plan.old_of_new[n] != g) return "point numbering is not a permutation";
  }
  // same-colour patches must not share a point; same-round elements neither
  std::vector<int32_t> owner_patch(nglob, -1), owner_colour(nglob, -1);
  std::vector<int32_t> nfirst(nglob, 0), nlast(nglob, 0), ntouch(nglob, 0);
  for (int32_t c = 0; c < plan.n_colours; ++c) {
    std::vector<int32_t> touched;
    for (int32_t lp = plan.colour_start[c]; lp < plan.colour_start[c + 1]; ++lp) {
      const PatchMeta &m = plan.meta[lp];
      for (int t = 0; t < m.n_pts; ++t) {
        const uint32_t w = plan.pt_words[m.pt_start + t];
        const int64_t g = w & kPtIndexMask;
        if (g >= nglob) return "point word index out of range";
        if (owner_colour[g] == c && owner_patch[g] != lp) return "two patches of one colour share a point";
        owner_colour[g] = c;
        owner_patch[g] = lp;
        ntouch[g]++;
        if (w & kPtFirst) nfirst[g]++;
        if (w & kPtLast) nlast[g]++;
      }
      int r0 = 0;
      for (int r = 0; r < m.n_rounds; ++r) {
        const int r1 = m.round_end[r];
        std::vector<int64_t> gs;
        for (int s = r0; s < r1; ++s) {
          const int32_t e = plan.elem_order[m.elem_start + s];
          std::vector<int64_t> ge;
          for (int k = 0; k < 25; ++k) ge.push_back(igloc[25 * (int64_t)e + k] - 1);
          std::sort(ge.begin(), ge.end());
          ge.erase(std::unique(ge.begin(), ge.end()), ge.end());
          gs.insert(gs.end(), ge.begin(), ge.end());
          for (int k = 0; k < 25; ++k) {
            const uint16_t li = plan.elem_pts[25 * (int64_t)(m.elem_start + s) + k];
            if (li >= m.n_pts) return "element point index outside patch";
            if ((int64_t)(plan.pt_words[m.pt_start + li] & kPtIndexMask) != plan.new_of_old[igloc[25 * (int64_t)e + k] - 1])
              return "element point index maps to the wrong global point";
          }
        }
        std::sort(gs.begin(), gs.end());
        if (std::adjacent_find(gs.begin(), gs.end()) != gs.end())
          return "two elements of one sub-round share a point";
        r0 = r1;
      }
      if (r0 != m.n_elems) return "sub-round counts do not cover the patch";
    }
  }
  for (int64_t g = 0; g < nglob; ++g) {  // g: internal number
    if (ntouch[g] == 0) continue;
    const bool pre = !prepass.empty() && prepass[plan.old_of_new[g]];
    if (nlast[g] != 1) return "point without exactly one last writer";
    if (nfirst[g] != (pre ? 0 : 1)) return "point first-writer count wrong";
  }
  return "";
}

int64_t plan_cost(const DomainPlan &plan) {
  // warp iterations of the patch kernels: per patch a fixed overhead (gather,
  // write-back and the CTA barriers, about four element iterations measured
  // on GB300), each sub-round ceil(elements / 8 warps), and a point term for
  // the gather and write-back traffic (256 points per iteration)
  int64_t c = 0;
  for (const PatchMeta &m : plan.meta) {
    c += 4 * 256 + m.n_pts;
    int r0 = 0;
    for (int r = 0; r < m.n_rounds; ++r) {
      c += 256 * ((m.round_end[r] - r0 + 7) / 8);
      r0 = m.round_end[r];
    }
  }
  return c;
}

int64_t plan_latency(const DomainPlan &plan, int ctas, int overhead) {
  int64_t t = 0;
  for (int c = 0; c < plan.n_colours; ++c) {
    const int32_t b = plan.colour_start[c], n = plan.colour_start[c + 1] - b;
    int64_t worst = 0;
    for (int32_t k = 0; k < ctas && k < n; ++k) {
      int64_t s = 0;
      for (int32_t q = k; q < n; q += ctas) s += plan.meta[b + q].n_elems + overhead;
      worst = std::max(worst, s);
    }
    t += worst;
  }
  return t;
}

std::string tune_plan(const int32_t *igloc, int64_t nel, int64_t nglob, int patch_elems, int growth,
                      int *best_pe, int *best_growth, int ctas, int overhead) {
  *best_pe = patch_elems > 0 ? patch_elems : kMaxPatchElems;
  *best_growth = growth >= 0 ? growth : kGrowLayered;
  if (patch_elems > 0 && growth >= 0) return "";
  // a mesh of few rounds per colour: the latency model on the whole mesh
  const bool few_rounds =
      ctas > 0 && nel < (int64_t)kTuneFullRounds * kMaxPatchElems * 4 * (int64_t)ctas;
  // candidates are compared on the mesh, or a prefix of it (element order),
  // its points renumbered compactly
  const int64_t n = few_rounds ? nel : std::min<int64_t>(nel, kTunePrefix);
  if (n == 0) return "";
  std::vector<int32_t> ig(igloc, igloc + 25 * n);
  std::vector<int32_t> ids(ig);
  std::sort(ids.begin(), ids.end());
  ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
  for (int32_t &v : ig) v = (int32_t)(std::lower_bound(ids.begin(), ids.end(), v) - ids.begin()) + 1;
  (void)nglob;
  std::vector<int> sizes;
  if (patch_elems > 0) sizes.push_back(patch_elems);
  else if (few_rounds) sizes = {8, 16, 24, 32, 40, 48, 56, 64};
  else sizes = {32, 40, 48, 56, 64};
  std::vector<int> growths;
  if (growth >= 0) growths.push_back(growth);
  else growths = {kGrowLayered, kGrowCompact};
  std::vector<std::pair<int, int>> cand;
  for (int pe : sizes)
    for (int gr : growths) cand.emplace_back(pe, gr);
  // the candidates' plans are independent: built on threads, compared in order
  std::vector<double> cost(cand.size(), -1.0);
  auto eval = [&](size_t i) {
    DomainPlan pl;
    if (build_plan(ig.data(), n, (int64_t)ids.size(), cand[i].first, cand[i].second, std::vector<uint8_t>(), pl,
                   false).empty())
      cost[i] = few_rounds ? (double)plan_latency(pl, ctas, overhead) : (double)plan_cost(pl);
  };
  std::vector<std::thread> threads;
  if (cand.size() > 1 && std::thread::hardware_concurrency() > 1) {
    try {
      for (size_t i = 0; i < cand.size(); ++i) threads.emplace_back(eval, i);
    } catch (const std::system_error &) {  // no threads: the rest in this one
      for (size_t i = threads.size(); i < cand.size(); ++i) eval(i);
    }
    for (std::thread &t : threads) t.join();
  } else {
    for (size_t i = 0; i < cand.size(); ++i) eval(i);
  }
  double best = -1;
  for (size_t i = 0; i < cand.size(); ++i)
    if (cost[i] >= 0 && (best < 0 || cost[i] < best)) {
      best = cost[i];
      *best_pe = cand[i].first;
      *best_growth = cand[i].second;
    }
  if (best < 0) return "no patch size yields a valid plan";
  return "";
}

}  // namespace axg
