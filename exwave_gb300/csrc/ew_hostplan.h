// ew_hostplan.h -- chunk plan of the LSRK45 step on host vectors
// (ew_lsrk45_step_host): which work items, cells and DoFs each chunk holds,
// and which chunks hold its cells' neighbours.  Host code only.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

namespace ew {

struct HostChunk {
  int item_begin = 0, n_items = 0;
  int64_t dof_begin = 0, n_dofs = 0;
  int lo = 0, hi = 0;  // the chunks that hold the neighbours of this chunk's cells
};

// Splits n_items work items (item i holds cells [i cb, min((i + 1) cb,
// n_cells)), cell_dofs DoFs each, consecutive in memory) into at most
// max_chunks runs of whole items.  nbr: [n_cells][nf] neighbour cells
// (negative: boundary).  Returns whether every chunk's neighbours lie in the
// chunk itself or in the two next to it, the condition under which all
// stages of the step can run as a wavefront over the chunks.
inline bool host_chunk_plan_items(int n_items, int cb, int64_t n_cells, int64_t cell_dofs, int nf,
                                  const int32_t* nbr, int max_chunks, std::vector<HostChunk>* out) {
  out->clear();
  if (n_items < 1 || cb < 1 || max_chunks < 1) return false;
  const int K = std::min(max_chunks, n_items);
  const int per = (n_items + K - 1) / K;
  for (int k = 0; k < K; ++k) {
    HostChunk h;
    h.item_begin = k * per;
    h.n_items = std::min(per, n_items - k * per);
    if (h.n_items <= 0) break;
    const int64_t c0 = (int64_t)h.item_begin * cb;
    const int64_t c1 = std::min<int64_t>((int64_t)(h.item_begin + h.n_items) * cb, n_cells);
    h.dof_begin = c0 * cell_dofs;
    h.n_dofs = (c1 - c0) * cell_dofs;
    h.lo = h.hi = k;
    for (int64_t cell = c0; cell < c1; ++cell)
      for (int f = 0; f < nf; ++f) {
        const int32_t nb = nbr[(size_t)cell * nf + f];
        if (nb < 0) continue;
        const int kc = (int)std::min<int64_t>(((int64_t)nb / cb) / per, K - 1);
        h.lo = std::min(h.lo, kc);
        h.hi = std::max(h.hi, kc);
      }
    out->push_back(h);
  }
  bool wave = true;
  for (int k = 0; k < (int)out->size(); ++k)
    if ((*out)[k].lo < k - 1 || (*out)[k].hi > k + 1) wave = false;
  return wave;
}

}  // namespace ew
