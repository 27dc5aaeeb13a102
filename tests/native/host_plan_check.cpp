// Host check of the chunk plan of the host-vector LSRK45 step
// (exwave_gb300/csrc/ew_hostplan.h): the chunks partition the work items,
// cells and DoFs in order; each chunk's lo..hi covers the chunks of all its
// cells' neighbours; and the wavefront condition holds exactly when every
// chunk's neighbours lie in the chunk or the two next to it.  Prints OK.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <random>
#include <vector>

#include "../../exwave_gb300/csrc/ew_hostplan.h"

static int failures = 0;
#define CHECK(c)                                                 \
  do {                                                           \
    if (!(c)) {                                                  \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c);    \
      ++failures;                                                \
    }                                                            \
  } while (0)

// neighbours of a lexicographic n^dim grid (x fastest); boundary: -2
static std::vector<int32_t> grid(int dim, int n) {
  const int64_t nc = dim == 2 ? (int64_t)n * n : (int64_t)n * n * n;
  std::vector<int32_t> nbr((size_t)nc * 2 * dim);
  for (int64_t c = 0; c < nc; ++c) {
    int64_t i[3] = {c % n, (c / n) % n, dim == 3 ? c / ((int64_t)n * n) : 0};
    int64_t st[3] = {1, n, (int64_t)n * n};
    for (int e = 0; e < dim; ++e)
      for (int s = 0; s < 2; ++s) {
        const int64_t j = i[e] + (s ? 1 : -1);
        nbr[(size_t)c * 2 * dim + 2 * e + s] = (j < 0 || j >= n) ? -2 : (int32_t)(c + (s ? 1 : -1) * st[e]);
      }
  }
  return nbr;
}

// the same grid with the cells renumbered by a permutation
static std::vector<int32_t> shuffled(const std::vector<int32_t>& nbr, int nf, unsigned seed) {
  const size_t nc = nbr.size() / nf;
  std::vector<int32_t> perm(nc);
  std::iota(perm.begin(), perm.end(), 0);
  std::mt19937 rng(seed);
  std::shuffle(perm.begin(), perm.end(), rng);
  std::vector<int32_t> out(nbr.size());
  for (size_t c = 0; c < nc; ++c)
    for (int f = 0; f < nf; ++f) {
      const int32_t nb = nbr[c * nf + f];
      out[(size_t)perm[c] * nf + f] = nb < 0 ? nb : perm[nb];
    }
  return out;
}

static bool check_plan(const std::vector<int32_t>& nbr, int nf, int cb, int64_t cell_dofs, int max_chunks) {
  const int64_t nc = (int64_t)(nbr.size() / nf);
  const int n_items = (int)((nc + cb - 1) / cb);
  std::vector<ew::HostChunk> ch;
  const bool wave = ew::host_chunk_plan_items(n_items, cb, nc, cell_dofs, nf, nbr.data(), max_chunks, &ch);
  CHECK(!ch.empty() && (int)ch.size() <= std::min(max_chunks, n_items));
  int item = 0;
  int64_t dof = 0;
  bool adjacent = true;
  for (int k = 0; k < (int)ch.size(); ++k) {
    const ew::HostChunk& h = ch[k];
    CHECK(h.item_begin == item && h.n_items > 0);
    CHECK(h.dof_begin == dof && h.n_dofs > 0);
    CHECK(h.lo <= k && k <= h.hi);
    item += h.n_items;
    dof += h.n_dofs;
    // brute force: the chunk of every neighbour of every cell lies in lo..hi
    const int64_t c0 = (int64_t)h.item_begin * cb, c1 = std::min<int64_t>((int64_t)item * cb, nc);
    for (int64_t c = c0; c < c1; ++c)
      for (int f = 0; f < nf; ++f) {
        const int32_t nb = nbr[(size_t)c * nf + f];
        if (nb < 0) continue;
        int kc = -1;
        for (int j = 0; j < (int)ch.size(); ++j)
          if ((int64_t)nb * cell_dofs >= ch[j].dof_begin && (int64_t)nb * cell_dofs < ch[j].dof_begin + ch[j].n_dofs)
            kc = j;
        CHECK(kc >= h.lo && kc <= h.hi);
        if (kc < k - 1 || kc > k + 1) adjacent = false;
      }
  }
  CHECK(item == n_items);
  CHECK(dof == nc * cell_dofs);
  CHECK(wave == adjacent);
  return wave;
}

int main() {
  // 3-D k=5, 64^3 cells, two per item: layers of 4096 cells, chunks of 16384
  CHECK(check_plan(grid(3, 64), 6, 2, 864, 16));
  // 3-D 16^3, one cell per item: chunks of exactly one layer
  CHECK(check_plan(grid(3, 16), 6, 1, 108, 16));
  // 2-D 20^2: rows of 20 cells, chunks of 25
  CHECK(check_plan(grid(2, 20), 4, 1, 48, 16));
  // small meshes: neighbours several chunks apart, no wavefront
  CHECK(!check_plan(grid(3, 5), 6, 2, 256, 16));
  CHECK(!check_plan(grid(2, 7), 4, 3, 108, 16));
  // fewer items than chunks, and a partial last item
  check_plan(grid(2, 3), 4, 2, 12, 16);
  check_plan(grid(3, 4), 6, 5, 32, 8);
  // renumbered cells: the neighbour ranges widen, no wavefront
  CHECK(!check_plan(shuffled(grid(3, 24), 6, 7), 6, 2, 108, 16));
  CHECK(!check_plan(shuffled(grid(2, 40), 4, 11), 4, 1, 27, 16));
  if (failures) {
    std::printf("%d failures\n", failures);
    return 1;
  }
  std::printf("OK\n");
  return 0;
}
