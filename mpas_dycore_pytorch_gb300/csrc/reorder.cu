// Mesh reordering (host code): space-filling-curve order of cells and vertices and the
// edge order derived from it (the reference's rule, mpas_pytorch/mesh_reordering.py:82-103:
// edges sorted by (min, max) of their new 1-based cell ids, then old index).
//
// The curve is the 3-D Hilbert curve over the cell (vertex) centres' Cartesian
// coordinates, quantised to 21 bits per axis; the index is computed with Skilling's
// transpose algorithm ("Programming the Hilbert curve", AIP Conf. Proc. 707, 2004):
// undo excess work (invert / exchange low bits), Gray-encode, then interleave the bits of
// the three transposed coordinates, most significant first, into a 63-bit key.  Points
// close on the curve are close on the sphere, so a kernel's neighbour gathers touch
// nearby rows.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <vector>

#include "mpasg.h"

namespace {

constexpr int kBits = 21;

uint64_t hilbert_key(uint32_t x0, uint32_t x1, uint32_t x2) {
  uint32_t X[3] = {x0, x1, x2};
  const uint32_t M = 1u << (kBits - 1);
  for (uint32_t Q = M; Q > 1; Q >>= 1) {
    const uint32_t P = Q - 1;
    for (int i = 0; i < 3; ++i) {
      if (X[i] & Q) {
        X[0] ^= P;  // invert the low bits of X[0]
      } else {      // exchange the low bits of X[0] and X[i]
        const uint32_t t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  for (int i = 1; i < 3; ++i) X[i] ^= X[i - 1];  // Gray encode
  uint32_t t = 0;
  for (uint32_t Q = M; Q > 1; Q >>= 1)
    if (X[2] & Q) t ^= Q - 1;
  for (int i = 0; i < 3; ++i) X[i] ^= t;
  uint64_t key = 0;
  for (int b = kBits - 1; b >= 0; --b)
    for (int i = 0; i < 3; ++i) key = (key << 1) | ((X[i] >> b) & 1u);
  return key;
}

uint32_t quantise(double v, double lo, double hi) {
  const double span = hi > lo ? hi - lo : 1.0;
  double q = (v - lo) / span * (double)((1u << kBits) - 1);
  q = std::min(std::max(q, 0.0), (double)((1u << kBits) - 1));
  return (uint32_t)std::llround(q);
}

}  // namespace

extern "C" int mpasg_sfc_order(long long n, const double* x, const double* y, const double* z,
                               long long* new_to_old) {
  if (n < 0 || (n > 0 && (!x || !y || !z || !new_to_old))) return MPASG_E_ARG;
  if (n == 0) return MPASG_OK;
  double lo = x[0], hi = x[0];
  for (long long i = 0; i < n; ++i) {
    lo = std::min(lo, std::min(x[i], std::min(y[i], z[i])));
    hi = std::max(hi, std::max(x[i], std::max(y[i], z[i])));
  }
  std::vector<std::pair<uint64_t, long long>> keys((size_t)n);
  for (long long i = 0; i < n; ++i)
    keys[(size_t)i] = {hilbert_key(quantise(x[i], lo, hi), quantise(y[i], lo, hi), quantise(z[i], lo, hi)), i};
  std::sort(keys.begin(), keys.end());  // ties (equal keys) by old index
  for (long long i = 0; i < n; ++i) new_to_old[i] = keys[(size_t)i].second;
  return MPASG_OK;
}

extern "C" int mpasg_edge_order(long long n_edges, long long n_cells, const long long* cells_on_edge,
                                const long long* cell_old_to_new, long long* new_to_old) {
  if (n_edges < 0 || n_cells < 0 || (n_edges > 0 && (!cells_on_edge || !cell_old_to_new || !new_to_old)))
    return MPASG_E_ARG;
  struct Key {
    long long lo, hi, old;
  };
  std::vector<Key> keys((size_t)n_edges);
  for (long long e = 0; e < n_edges; ++e) {
    long long c[2];
    for (int j = 0; j < 2; ++j) {
      const long long v = cells_on_edge[2 * e + j];  // 1-based, sentinel outside [1, n_cells]
      c[j] = (v >= 1 && v <= n_cells) ? cell_old_to_new[v - 1] + 1 : n_cells + 1;
    }
    keys[(size_t)e] = {std::min(c[0], c[1]), std::max(c[0], c[1]), e};
  }
  std::sort(keys.begin(), keys.end(), [](const Key& a, const Key& b) {
    if (a.lo != b.lo) return a.lo < b.lo;
    if (a.hi != b.hi) return a.hi < b.hi;
    return a.old < b.old;
  });
  for (long long e = 0; e < n_edges; ++e) new_to_old[e] = keys[(size_t)e].old;
  return MPASG_OK;
}
