// Host-side tables of the banded two-pass fixed-point matvec (kernels: ed_sweep.cuh):
// reverse Cuthill-McKee renumbering of one spin species' states, the per-block windows of the
// shared-memory ring and the hop lists with precomputed ring offsets. Plain C++ (the only CUDA
// type is int2).
#pragma once

#include <vector_types.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <vector>

namespace ed {

constexpr int SW_NT = 512;   // threads per CTA of both passes (one target row / column per half-warp)
constexpr int SW_CH = 32;    // rows (pass 1) / columns (pass 2) per ring chunk and per target block
constexpr int SW_W = 16;     // stripe width: columns (pass 1) / rows (pass 2) per CTA
constexpr int SW_LST = 16;   // uint16 entries per hop list (15 partners + counts)

// ---- host: renumbering, hop lists, ring windows ------------------------------------------------

// reverse Cuthill-McKee order (new -> old) of the symmetric graph (off, idx) with n nodes,
// started from `start` (each further connected component from its lowest-degree node)
static std::vector<int32_t> sweep_rcm(int64_t n, const std::vector<int32_t>& off, const std::vector<int32_t>& idx,
                                      int64_t start) {
  std::vector<int32_t> order;
  order.reserve(n);
  std::vector<char> seen(n, 0);
  std::vector<int32_t> nb;
  auto deg = [&](int64_t v) { return off[v + 1] - off[v]; };
  auto run = [&](int64_t s0) {
    size_t head = order.size();
    order.push_back((int32_t)s0);
    seen[s0] = 1;
    while (head < order.size()) {
      const int32_t v = order[head++];
      nb.clear();
      for (int32_t k = off[v]; k < off[v + 1]; ++k)
        if (!seen[idx[k]]) {
          seen[idx[k]] = 1;
          nb.push_back(idx[k]);
        }
      std::sort(nb.begin(), nb.end(), [&](int32_t a, int32_t b) { return deg(a) != deg(b) ? deg(a) < deg(b) : a < b; });
      order.insert(order.end(), nb.begin(), nb.end());
    }
  };
  run(start);
  while ((int64_t)order.size() < n) {
    int64_t best = -1;
    for (int64_t v = 0; v < n; ++v)
      if (!seen[v] && (best < 0 || deg(v) < deg(best))) best = v;
    run(best);
  }
  std::reverse(order.begin(), order.end());
  return order;
}

// last BFS level of the component of s (for pseudo-peripheral start nodes)
static std::vector<int32_t> sweep_far_level(int64_t n, const std::vector<int32_t>& off, const std::vector<int32_t>& idx,
                                            int64_t s, int* ecc) {
  std::vector<int32_t> dist(n, -1), cur{(int32_t)s}, nxt;
  dist[s] = 0;
  int d = 0;
  while (true) {
    nxt.clear();
    for (int32_t v : cur)
      for (int32_t k = off[v]; k < off[v + 1]; ++k)
        if (dist[idx[k]] < 0) {
          dist[idx[k]] = d + 1;
          nxt.push_back(idx[k]);
        }
    if (nxt.empty()) break;
    cur.swap(nxt);
    ++d;
  }
  *ecc = d;
  return cur;
}

struct SweepSide {
  std::vector<int32_t> perm;     // new -> old
  std::vector<uint16_t> lst;     // [n][SW_LST]
  std::vector<int2> win;         // per target block: (first chunk needed, last chunk needed)
  int need = 0;                  // ring chunks needed (largest window)
  int ring = 0;
};

// windows of an ordering: for target block j, the first chunk any later block still needs and
// the last chunk any block up to j needs (both monotone, so the ring is filled and freed in
// order); returns the largest window in chunks
static int sweep_windows(int64_t n, const std::vector<int32_t>& off, const std::vector<int32_t>& idx,
                         const std::vector<int32_t>& perm, const std::vector<int32_t>& inv, std::vector<int2>* win) {
  const int64_t nblk = (n + SW_CH - 1) / SW_CH;
  std::vector<int64_t> lo(nblk, INT64_MAX), hi(nblk, -1);
  for (int64_t i = 0; i < n; ++i) {
    const int64_t b = i / SW_CH, v = perm[i];
    lo[b] = std::min(lo[b], i);
    hi[b] = std::max(hi[b], i);
    for (int32_t k = off[v]; k < off[v + 1]; ++k) {
      const int64_t q = inv[idx[k]];
      lo[b] = std::min(lo[b], q);
      hi[b] = std::max(hi[b], q);
    }
  }
  for (int64_t b = nblk - 2; b >= 0; --b) lo[b] = std::min(lo[b], lo[b + 1]);
  for (int64_t b = 1; b < nblk; ++b) hi[b] = std::max(hi[b], hi[b - 1]);
  int need = 0;
  if (win) win->resize(nblk);
  for (int64_t b = 0; b < nblk; ++b) {
    const int c0 = (int)(lo[b] / SW_CH), c1 = (int)(hi[b] / SW_CH);
    need = std::max(need, c1 - c0 + 1);
    if (win) {
      (*win)[b].x = c0;
      (*win)[b].y = c1;
    }
  }
  return need;
}

// renumbering and windows of one spin species (hop lists: sweep_lists); false when a target
// has more than 15 hops
static bool sweep_order(int64_t n, const std::vector<int32_t>& off, const std::vector<int32_t>& idx,
                        const std::vector<double>& coef, SweepSide* out) {
  if (n < 1) return false;
  std::vector<int32_t> deg_off(n + 1, 0), nz_idx;
  // zero coefficients are no edges
  for (int64_t v = 0; v < n; ++v) {
    for (int32_t k = off[v]; k < off[v + 1]; ++k)
      if (coef[k] != 0.0) nz_idx.push_back(idx[k]);
    deg_off[v + 1] = (int32_t)nz_idx.size();
    if (deg_off[v + 1] - deg_off[v] > SW_LST - 1) return false;
  }
  // candidate start nodes: the lowest-degree node, the first and the last state, and the
  // pseudo-peripheral node reached from each by repeated breadth-first searches; keep the
  // ordering with the smallest window
  std::vector<int64_t> starts;
  int64_t lowest = 0;
  for (int64_t v = 1; v < n; ++v)
    if (deg_off[v + 1] - deg_off[v] < deg_off[lowest + 1] - deg_off[lowest]) lowest = v;
  for (int64_t s0 : {lowest, (int64_t)0, n - 1}) {
    starts.push_back(s0);
    int64_t r = s0;
    int ecc = 0;
    (void)sweep_far_level(n, deg_off, nz_idx, r, &ecc);
    for (int it = 0; it < 8; ++it) {
      const std::vector<int32_t> far = sweep_far_level(n, deg_off, nz_idx, r, &ecc);
      int64_t x = far[0];
      for (int32_t c : far)
        if (deg_off[c + 1] - deg_off[c] < deg_off[x + 1] - deg_off[x]) x = c;
      int ecc2 = 0;
      (void)sweep_far_level(n, deg_off, nz_idx, x, &ecc2);
      r = x;
      if (ecc2 <= ecc) break;
    }
    starts.push_back(r);
  }
  int best_need = INT32_MAX;
  std::vector<int32_t> best, inv(n);
  for (int64_t s0 : starts) {
    std::vector<int32_t> perm = sweep_rcm(n, deg_off, nz_idx, s0);
    for (int64_t i = 0; i < n; ++i) inv[perm[i]] = (int32_t)i;
    const int need = sweep_windows(n, deg_off, nz_idx, perm, inv, nullptr);
    if (need < best_need) {
      best_need = need;
      best = perm;
    }
  }
  out->perm = best;
  for (int64_t i = 0; i < n; ++i) inv[best[i]] = (int32_t)i;
  out->need = sweep_windows(n, deg_off, nz_idx, best, inv, &out->win);
  return true;
}

// hop lists of the renumbered targets: ring offsets of the partners for a ring of `ring`
// chunks, entries with a positive coefficient first; entry 15 = count | (positive count << 8)
static void sweep_lists(int64_t n, const std::vector<int32_t>& off, const std::vector<int32_t>& idx,
                        const std::vector<double>& coef, int ring, SweepSide* out) {
  std::vector<int32_t> inv(n);
  for (int64_t i = 0; i < n; ++i) inv[out->perm[i]] = (int32_t)i;
  const int64_t ring_elems = (int64_t)ring * SW_CH;
  out->ring = ring;
  out->lst.assign((size_t)n * SW_LST, 0);
  for (int64_t i = 0; i < n; ++i) {
    const int64_t v = out->perm[i];
    uint16_t* L = out->lst.data() + (size_t)i * SW_LST;
    int c = 0, npos = 0;
    for (int sign = 1; sign >= -1; sign -= 2)
      for (int32_t k = off[v]; k < off[v + 1]; ++k) {
        if (coef[k] == 0.0 || (coef[k] > 0.0) != (sign > 0)) continue;
        L[c++] = (uint16_t)(inv[idx[k]] % ring_elems);
        if (sign > 0) ++npos;
      }
    L[SW_LST - 1] = (uint16_t)(c | (npos << 8));
  }
}

}  // namespace ed
