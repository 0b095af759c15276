// Host-side tables of the stripe matvec (kernels: ed_stripe.cuh): the renumbering of one spin
// species' states by hop count and the list-major hop lists. Plain C++.
#pragma once

#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

#ifdef __CUDACC__
#define ED_STRIPE_HD __host__ __device__
#else
#define ED_STRIPE_HD
#endif

namespace ed {

constexpr int ST_NT = 512;   // threads per CTA of both passes (one target per lane)
constexpr int ST_K = 4;      // stripe width: columns (pass 1) / rows (pass 2) = one 32-byte record
constexpr int ST_PMAX = 8;   // list pairs per target: + pairs and - pairs together

// 16-byte slot of the first half of record i in a stripe buffer; the second half is slot ^ 1.
// Records are 32 bytes; in every other group of four records the halves are swapped, so the
// first halves of records with random indices fall on all eight 16-byte bank groups.
ED_STRIPE_HD inline uint32_t stripe_slot(int64_t i) { return (uint32_t)(2 * i + ((i >> 2) & 1)); }

struct StripeSide {
  std::vector<int32_t> perm;   // new -> old
  std::vector<uint32_t> lst;   // [pmax][n]: two record slots per word (low, high)
  std::vector<uint16_t> meta;  // [n]: + pairs | - pairs << 8
  int pmax = 0;
};

// Renumbering of one species' n states (hop lists off/idx/coef in the original order; zero
// coefficients are no hops) in increasing (pairs, - pairs) order, ties by original index, and
// the hop lists of the renumbered targets: the record slots of the + partners, then of the -
// partners, each segment padded to whole pairs with the zero record (record n). False when a
// target needs more than ST_PMAX pairs or n is too large for 16-bit slots.
static bool stripe_order(int64_t n, const std::vector<int32_t>& off, const std::vector<int32_t>& idx,
                         const std::vector<double>& coef, StripeSide* out) {
  if (n < 1 || 2 * n + 1 >= 65536) return false;
  std::vector<int> pp(n), pn(n);
  for (int64_t v = 0; v < n; ++v) {
    int np = 0, nn = 0;
    for (int32_t k = off[v]; k < off[v + 1]; ++k) {
      if (coef[k] > 0.0) ++np;
      else if (coef[k] < 0.0) ++nn;
    }
    pp[v] = (np + 1) / 2;
    pn[v] = (nn + 1) / 2;
    if (pp[v] + pn[v] > ST_PMAX) return false;
  }
  std::vector<int32_t>& perm = out->perm;
  perm.resize(n);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int32_t a, int32_t b) {
    const int ta = pp[a] + pn[a], tb = pp[b] + pn[b];
    return ta != tb ? ta < tb : pn[a] < pn[b];
  });
  std::vector<int32_t> inv(n);
  for (int64_t i = 0; i < n; ++i) inv[perm[i]] = (int32_t)i;
  int pmax = 0;
  for (int64_t v = 0; v < n; ++v) pmax = std::max(pmax, pp[v] + pn[v]);
  out->pmax = pmax;
  const uint32_t zero = stripe_slot(n);
  out->lst.assign((size_t)std::max(pmax, 1) * n, zero | (zero << 16));
  out->meta.assign(n, 0);
  std::vector<uint32_t> seg;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t v = perm[i];
    int p = 0;
    for (int sign = 1; sign >= -1; sign -= 2) {
      seg.clear();
      for (int32_t k = off[v]; k < off[v + 1]; ++k)
        if (coef[k] != 0.0 && (coef[k] > 0.0) == (sign > 0)) seg.push_back(stripe_slot(inv[idx[k]]));
      if (seg.size() % 2) seg.push_back(zero);
      for (size_t e = 0; e < seg.size(); e += 2) out->lst[(size_t)p++ * n + i] = seg[e] | (seg[e + 1] << 16);
    }
    out->meta[i] = (uint16_t)(pp[v] | (pn[v] << 8));
  }
  return true;
}

}  // namespace ed
