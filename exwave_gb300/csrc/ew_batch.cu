// ew_batch.cu -- many independent solves stepped together on one GPU.
//
// Memory: one device arena of the configured HBM budget, allocated once and
// carved by a host-side first-fit allocator (admission = allocation).
// Execution: solves are grouped by (dimension, degree); per LSRK45 stage,
// each group runs one persistent launch of the Cartesian stage kernel over a
// work list of cell blocks of all its solves, reading per-solve arguments
// (state pointers, coefficients x dt, source) from a device table.  The
// groups' launches follow one another on the batch stream (each fills the
// GPU).  A receiver kernel samples the pressure at each solve's receivers and
// advances its clock.  The whole step is captured as a CUDA graph for each
// parity of the state double buffer; membership changes rebuild tables and
// graphs before the next step.
//
// Mixed precision keeps each solve's state between the steps as an
// unevaluated float pair: FP32 hi in the stage input buffer X[cur] and FP32
// lo in U[1] (about 48 significant bits).  The first stage of a step reads
// hi and lo like a middle stage reads its input, the accumulator lives in
// U[0] during the step and the last stage writes the new hi and lo.  The
// compensated precision keeps it as interleaved float pairs in U[cur] (8
// bytes, like FP64), read by the next first stage as input and accumulator.
// Receivers, get_state and set_state convert between the pairs and FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/exwave_gb300.h"
#include "ew_basis.h"
#include "ew_device.cuh"
#include "ew_ff.cuh"
#include "ew_internal.h"

namespace {

constexpr size_t kAlign = 256;
constexpr int kCellConsts = 19;  // must match ew_cart.cuh

// First-fit allocator over [0, size) with coalescing free list.
class Arena {
 public:
  void init(size_t size) {
    size_ = size;
    free_.clear();
    if (size) free_[0] = size;
  }
  bool alloc(size_t bytes, size_t* off) {
    bytes = (bytes + kAlign - 1) & ~(kAlign - 1);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes;
        const size_t noff = it->first + bytes;
        free_.erase(it);
        if (rest) free_[noff] = rest;
        used_ += bytes;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = (bytes + kAlign - 1) & ~(kAlign - 1);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t free_bytes() const { return size_ - used_; }

 private:
  size_t size_ = 0, used_ = 0;
  std::map<size_t, size_t> free_;
};

struct Solve {
  int32_t id = -1;
  int dim = 3, np = 2, N = 1, F = 4;
  int64_t n_cells = 0, n_dofs = 0, n_steps = 0, steps_done = 0;
  double dt = 0.0;
  int cur = 0;  // buffer U[cur] holds the current state
  size_t off = 0, bytes = 0;  // one arena block per solve
  // device pointers inside the block
  double* U[2] = {nullptr, nullptr};
  void* X[2] = {nullptr, nullptr};  // mixed: FP32 stage inputs; FP64: X[0] = third register
  int32_t* nbr = nullptr;
  void* cellc = nullptr;
  void* src_w = nullptr;
  double* rec_w = nullptr;
  int32_t* rec_cell = nullptr;
  double* trace = nullptr;
  // [0] time, [1] steps taken, [2] n_steps, [3] status (1: diverged), as doubles
  double* clock = nullptr;
  int n_rec = 0;
  int32_t src_cell = -1;
  double src_amp = 0.0, src_f0 = 0.0, src_t0 = 0.0;
};

// Receiver sampling: one block per solve, one warp per receiver; then the
// solve's clock advances by one step.  Samples of steps beyond the solve's
// n_steps (a batch that allows overrun) are not recorded.  A sample that is
// not finite or exceeds the blow-up limit marks the solve diverged: in its
// clock (kept across rebuilds) and in flags[solve], which the host polls.
struct RecDesc {
  const double* U[2];  // FP64 state by parity (FP64 batches)
  const float* H[2];   // mixed: hi part by parity
  const float* L;      // mixed: lo part
  int32_t mixed, pad;
  const double* rec_w;
  const int32_t* rec_cell;
  double* trace;
  double* clock;
  double dt;
  double limit;  // blow-up limit (0: non-finite samples only)
  int32_t n_rec, N, F, dim;
};

__global__ void receiver_kernel(const RecDesc* rd, int n, int parity, int32_t* flags) {
  const int s = blockIdx.x;
  if (s >= n) return;
  const RecDesc r = rd[s];
  const double* state = r.U[parity];
  const float* hi = r.H[parity];
  const int64_t step = (int64_t)r.clock[1];
  const bool record = step < (int64_t)r.clock[2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int k = warp; k < r.n_rec; k += blockDim.x >> 5) {
    const int32_t cell = r.rec_cell[k];
    const size_t p0 = ((size_t)cell * r.F + r.dim) * r.N;
    const double* w = r.rec_w + (size_t)k * r.N;
    double acc = 0.0;
    for (int q = lane; q < r.N; q += 32) {
      double v;
      if (r.mixed == 1) {
        v = (double)hi[p0 + q] + (double)r.L[p0 + q];
      } else if (r.mixed == 2) {
        const float2 pr = reinterpret_cast<const float2*>(state)[p0 + q];
        v = (double)pr.x + (double)pr.y;
      } else {
        v = state[p0 + q];
      }
      acc += w[q] * v;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      if (record) r.trace[step * r.n_rec + k] = acc;
      if (!isfinite(acc) || (r.limit > 0.0 && fabs(acc) > r.limit)) bad = 1;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    r.clock[0] += r.dt;
    if (record) r.clock[1] = (double)(step + 1);
    if (bad) r.clock[3] = 1.0;
    flags[s] = r.clock[3] != 0.0 ? 1 : 0;
  }
}

// Interleaved float pairs <-> FP64 state (compensated batches).
__global__ void join_pairs_kernel(const float2* pr, int64_t n, double* state) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    state[i] = (double)pr[i].x + (double)pr[i].y;
}
__global__ void split_pairs_kernel(const double* state, int64_t n, float2* pr) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float h, l;
    ew::f64_split(state[i], h, l);
    pr[i] = make_float2(h, l);
  }
}


// FP32 hi + lo -> FP64 state.
__global__ void join_state_kernel(const float* hi, const float* lo, int64_t n, double* state) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    state[i] = (double)hi[i] + (double)lo[i];
}

// FP64 state -> FP32 hi and lo parts (hi + lo = state to about 48 bits).
__global__ void split_state_kernel(const double* state, int64_t n, float* hi, float* lo) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float h, l;
    ew::f64_split(state[i], h, l);
    hi[i] = h;
    lo[i] = l;
  }
}

struct Group {
  int dim = 3, np = 2;
  int cb = 1;
  std::vector<int32_t> members;  // solve ids, slot order
  ew::SolveDesc* d_tables = nullptr;  // [parity][stage][slot]
  ew::WorkItem* d_work = nullptr;
  int n_work = 0;
  int grid[2][5] = {{0}};
  int sx[5] = {0}, variant[5] = {0};
  int tma = 0;
  int nb_lines = 0;  // tuned neighbour staging of the line kernel
};

template <typename T>
std::vector<T> cast_vec(const std::vector<double>& v) {
  return std::vector<T>(v.begin(), v.end());
}

}  // namespace

namespace ew {
cudaError_t launch_split_pairs(const double* state, int64_t n, void* pairs, cudaStream_t stream) {
  const int threads = 256;
  const int64_t blocks = std::min<int64_t>((n + threads - 1) / threads, 1 << 20);
  if (blocks < 1) return cudaSuccess;
  split_pairs_kernel<<<(unsigned)blocks, threads, 0, stream>>>(state, n, static_cast<float2*>(pairs));
  return cudaGetLastError();
}
}  // namespace ew

struct ew_batch {
  int device = 0;
  bool mixed = true;  // FP32 or float-float operator (else FP64)
  bool ff = false;    // compensated: float-float operator, FP64 state between steps
  bool use_graphs = true;
  bool allow_overrun = false;
  double blowup_limit = 0.0;
  int num_sms = 0;
  int max_solves = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  char* arena_base = nullptr;
  Arena arena;
  std::map<int32_t, Solve> solves;
  int32_t next_id = 0;
  int parity = 0;
  bool dirty = true;
  std::vector<Group> groups;
  RecDesc* d_rec = nullptr;
  int n_rec_solves = 0;
  int32_t* d_flags = nullptr;         // per receiver-table entry: diverged
  std::vector<int32_t> rec_ids;       // solve id of each receiver-table entry
  int* d_err = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  std::string last_error;
  int64_t launches = 0;
  int64_t launches_per_step = 0;
};

namespace {

int bfail(ew_batch* b, int code, const std::string& msg) {
  if (b) b->last_error = msg;
  return code;
}

int bcuda(ew_batch* b, cudaError_t e, const char* what) {
  return bfail(b, EW_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void free_groups(ew_batch* b) {
  for (auto& g : b->groups) {
    if (g.d_tables) cudaFree(g.d_tables);
    if (g.d_work) cudaFree(g.d_work);
  }
  b->groups.clear();
  if (b->d_rec) cudaFree(b->d_rec);
  b->d_rec = nullptr;
  if (b->d_flags) cudaFree(b->d_flags);
  b->d_flags = nullptr;
  b->rec_ids.clear();
  for (int p = 0; p < 2; ++p)
    if (b->graph[p]) {
      cudaGraphExecDestroy(b->graph[p]);
      b->graph[p] = nullptr;
    }
}

struct Layout {
  size_t U, X, nbr, cellc, src_w, rec_w, rec_cell, trace, clock, total;
};

// precision: 0 FP64, 1 mixed (FP32 data), 2 compensated (float pairs)
Layout solve_layout(const ew_solve_desc* s, int precision) {
  const int dim = s->mesh.dim, np = s->mesh.degree + 1;
  int N = 1;
  for (int d = 0; d < dim; ++d) N *= np;
  const int64_t n_dofs = s->mesh.n_cells * (dim + 1) * N;
  const bool mixed = precision == 1;
  const size_t rsz = mixed ? 4 : 8;
  auto al = [](size_t v) { return (v + kAlign - 1) & ~(kAlign - 1); };
  Layout L;
  size_t o = 0;
  L.U = o;
  o += 2 * al((size_t)n_dofs * 8);
  L.X = o;
  o += mixed ? 2 * al((size_t)n_dofs * 4) : (precision == 2 ? 2 * al((size_t)n_dofs * 8) : al((size_t)n_dofs * 8));
  L.nbr = o;
  o += al((size_t)s->mesh.n_cells * 2 * dim * 4);
  L.cellc = o;
  o += al((size_t)s->mesh.n_cells * kCellConsts * rsz);
  L.src_w = o;
  o += al((size_t)N * rsz);
  L.rec_w = o;
  o += al((size_t)std::max(s->n_receivers, 0) * N * 8);
  L.rec_cell = o;
  o += al((size_t)std::max(s->n_receivers, 1) * 4);
  L.trace = o;
  o += al((size_t)std::max<int64_t>(s->n_steps, 1) * std::max(s->n_receivers, 1) * 8);
  L.clock = o;
  o += al(4 * 8);
  L.total = o;
  return L;
}

// cell containing a point (axis-aligned boxes), reference coordinates
bool locate(const ew_mesh_desc& m, const double* x, int32_t* cell, double* xi) {
  const int dim = m.dim, nv = 1 << dim;
  for (int64_t c = 0; c < m.n_cells; ++c) {
    const double* V = m.vertices + (size_t)c * nv * dim;
    bool in = true;
    for (int e = 0; e < dim && in; ++e) {
      const double lo = V[e], hi = V[(nv - 1) * dim + e];
      if (x[e] < lo || x[e] > hi) in = false;
    }
    if (!in) continue;
    for (int e = 0; e < dim; ++e) {
      const double lo = V[e], hi = V[(nv - 1) * dim + e];
      xi[e] = (x[e] - lo) / (hi - lo);
    }
    *cell = (int32_t)c;
    return true;
  }
  return false;
}

// tensor-product Lagrange weights phi_q(xi) on the Gauss points
std::vector<double> point_weights(int dim, int np, const double* xi) {
  ew::GaussRule g = ew::gauss_rule(np);
  int N = 1;
  for (int d = 0; d < dim; ++d) N *= np;
  std::vector<double> w(N, 1.0);
  for (int q = 0; q < N; ++q) {
    int t = q;
    for (int e = 0; e < dim; ++e) {
      w[q] *= ew::lagrange(g.x, t % np, xi[e]);
      t /= np;
    }
  }
  return w;
}

// Per-stage solve descriptors of a solve for a given parity (current state
// in U[parity]).
void stage_descs(const ew_batch* b, const Solve& s, int parity, ew::SolveDesc* out) {
  using namespace ew;
  const double dt = s.dt;
  const double f1[5] = {kA21 * dt, kA32 * dt, kA43 * dt, kA54 * dt, kB5 * dt};
  const double f2[5] = {(kB1 - kA21) * dt, (kB2 - kA32) * dt, (kB3 - kA43) * dt,
                        (kB4 - kA54) * dt, 0.0};
  const double cs[5] = {0.0, kA21, kB1 + kA32, kB1 + kB2 + kA43, kB1 + kB2 + kB3 + kA54};
  double* Nv = s.U[parity];
  double* Pv = s.U[1 - parity];
  const void* X[5];
  const double* A[5];
  void* Xo[5];
  double* Ao[5];
  if (b->ff) {
    // compensated: float-pair state in U[parity] read by the first stage
    // (X == A), float-pair accumulator in U[1 - parity], float-pair stage
    // inputs alternating in X[0] / X[1]; the last stage leaves the new state's
    // pairs in U[1 - parity]
    void* Y0 = s.X[0];
    void* Y1 = s.X[1];
    X[0] = Nv; A[0] = Nv; Xo[0] = Y0; Ao[0] = Pv;
    X[1] = Y0; A[1] = Pv; Xo[1] = Y1; Ao[1] = Pv;
    X[2] = Y1; A[2] = Pv; Xo[2] = Y0; Ao[2] = Pv;
    X[3] = Y0; A[3] = Pv; Xo[3] = Y1; Ao[3] = Pv;
    X[4] = Y1; A[4] = Pv; Xo[4] = nullptr; Ao[4] = Pv;
  } else if (b->mixed) {
    // state pair: hi in X[parity], lo in U[1] (floats); accumulator in U[0];
    // the last stage leaves the new hi in X[1 - parity] and lo in U[1]
    void* Xh = s.X[parity];
    void* Xn = s.X[1 - parity];
    double* S = s.U[0];
    double* Lo = s.U[1];
    X[0] = Xh; A[0] = Lo; Xo[0] = Xn; Ao[0] = S;
    X[1] = Xn; A[1] = S; Xo[1] = Xh; Ao[1] = S;
    X[2] = Xh; A[2] = S; Xo[2] = Xn; Ao[2] = S;
    X[3] = Xn; A[3] = S; Xo[3] = Xh; Ao[3] = S;
    X[4] = Xh; A[4] = S; Xo[4] = Xn; Ao[4] = Lo;
  } else {
    double* T = static_cast<double*>(s.X[0]);
    X[0] = Nv; A[0] = Nv; Xo[0] = T; Ao[0] = Pv;
    X[1] = T; A[1] = Pv; Xo[1] = Pv; Ao[1] = Nv;
    X[2] = Pv; A[2] = Nv; Xo[2] = Nv; Ao[2] = T;
    X[3] = Nv; A[3] = T; Xo[3] = T; Ao[3] = Pv;
    X[4] = T; A[4] = Pv; Xo[4] = nullptr; Ao[4] = Pv;
  }
  for (int st = 0; st < 5; ++st) {
    SolveDesc d;
    std::memset(&d, 0, sizeof(d));
    d.X = X[st];
    d.A = A[st];
    d.Xout = Xo[st];
    d.Aout = Ao[st];
    d.nbr = s.nbr;
    d.cellc = s.cellc;
    d.n_cells = s.n_cells;
    d.f1 = f1[st];
    d.f2 = f2[st];
    d.f1f = (float)f1[st];
    d.f1_hi = (float)f1[st];
    d.f1_lo = (float)(f1[st] - (double)d.f1_hi);
    d.fb_hi = (float)(f1[st] + f2[st]);
    d.fb_lo = (float)((f1[st] + f2[st]) - (double)d.fb_hi);
    d.bf = 1.0f;
    d.mode = st < 4 ? MODE_RK_MID : MODE_RK_LAST;
    d.time = s.clock;
    d.src_w = s.src_w;
    d.src_amp = s.src_amp;
    d.src_f0 = s.src_f0;
    d.src_t0 = s.src_t0;
    d.c_stage = cs[st];
    d.dt = dt;
    d.src_cell = s.src_cell;
    out[st] = d;
  }
}

int rebuild(ew_batch* b) {
  free_groups(b);
  // groups by (dim, np) over unfinished solves
  std::map<std::pair<int, int>, std::vector<int32_t>> by;
  for (auto& kv : b->solves)
    if (kv.second.steps_done < kv.second.n_steps)
      by[{kv.second.dim, kv.second.np}].push_back(kv.first);
  cudaError_t e;
  for (auto& kv : by) {
    Group g;
    g.dim = kv.first.first;
    g.np = kv.first.second;
    g.members = kv.second;
    const ew::KernelTable& kt = ew::kernel_table(g.dim, g.np);
    const int lines = kt.lines;
    const int prec = b->ff ? 2 : (b->mixed ? 1 : 0);
    const int tuned = ew::tuned_cells_per_block(g.dim, g.np - 1, prec);
    g.nb_lines = ew::tuned_staging(g.dim, g.np - 1, prec) == 1 ? 1 : 0;
    g.cb = tuned > 0 ? std::min(tuned, std::max(1, 512 / lines)) : std::max(1, 256 / lines);
    const int NP = g.np;
    int N = 1;
    for (int d = 0; d < g.dim; ++d) N *= NP;
    const int F = g.dim + 1;
    for (int st = 0; st < 5; ++st) {
      if (b->ff) {
        // the state is kept as float pairs: the first stage reads it as input
        // and accumulator at once (middle-stage kernel, X == A), the last one
        // writes the new pairs
        g.variant[st] = st < 4 ? ew::CV_FF_MID : ew::CV_FF_LAST_PAIR;
        g.sx[st] = (st == 0) ? 0 : 1;
      } else if (b->mixed) {
        g.variant[st] = st == 0 ? ew::CV_MIX_S1_FF : (st < 4 ? ew::CV_MIX_MID : ew::CV_MIX_LAST_FF);
        g.sx[st] = 1;
      } else {
        g.variant[st] = st < 4 ? ew::CV_F64_MID : ew::CV_F64_LAST;
        g.sx[st] = (st == 0) ? 0 : 1;  // first stage: X is the accumulator
      }
    }
    while (g.cb > 1 && kt.cart[g.variant[1]].smem(g.cb, 1) > 110 * 1024) --g.cb;
    const size_t cell_x = (size_t)F * N * (b->mixed && !b->ff ? 4 : 8);
    g.tma = (cell_x % 16 == 0) && (((size_t)F * N * 8) % 16 == 0);
    // tables
    const size_t nslot = g.members.size();
    std::vector<ew::SolveDesc> tab(2 * 5 * nslot);
    for (int p = 0; p < 2; ++p)
      for (size_t k = 0; k < nslot; ++k) {
        ew::SolveDesc d5[5];
        stage_descs(b, b->solves[g.members[k]], p, d5);
        for (int st = 0; st < 5; ++st) tab[(p * 5 + st) * nslot + k] = d5[st];
      }
    std::vector<ew::WorkItem> work;
    for (size_t k = 0; k < nslot; ++k) {
      const Solve& s = b->solves[g.members[k]];
      for (int64_t c = 0; c < s.n_cells; c += g.cb) {
        ew::WorkItem w;
        w.solve = (int32_t)k;
        w.cell_begin = (int32_t)c;
        w.n_cells = (int32_t)std::min<int64_t>(g.cb, s.n_cells - c);
        w.pad = 0;
        work.push_back(w);
      }
    }
    g.n_work = (int)work.size();
    if ((e = cudaMalloc(&g.d_tables, tab.size() * sizeof(ew::SolveDesc))) != cudaSuccess ||
        (e = cudaMalloc(&g.d_work, std::max<size_t>(work.size(), 1) * sizeof(ew::WorkItem))) != cudaSuccess ||
        (e = cudaMemcpy(g.d_tables, tab.data(), tab.size() * sizeof(ew::SolveDesc), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(g.d_work, work.data(), work.size() * sizeof(ew::WorkItem), cudaMemcpyHostToDevice)) != cudaSuccess) {
      b->groups.push_back(g);
      return bcuda(b, e, "batch tables");
    }
    for (int p = 0; p < 2; ++p)
      for (int st = 0; st < 5; ++st) {
        const int occ = std::max(1, kt.cart[g.variant[st]].occupancy(g.cb, g.sx[st]));
        g.grid[p][st] = std::max(1, std::min(g.n_work, occ * b->num_sms));
      }
    if ((e = ew::upload_cart_constants(g.dim, g.np)) != cudaSuccess) {
      b->groups.push_back(g);
      return bcuda(b, e, "constants");
    }
    b->groups.push_back(g);
  }
  // receiver table (every unfinished solve: it also carries the clock)
  std::vector<RecDesc> rd;
  for (auto& g : b->groups)
    for (int32_t id : g.members) {
      const Solve& s = b->solves[id];
      RecDesc r;
      r.U[0] = s.U[0];
      r.U[1] = s.U[1];
      r.H[0] = static_cast<const float*>(s.X[0]);
      r.H[1] = static_cast<const float*>(s.X[1]);
      r.L = reinterpret_cast<const float*>(s.U[1]);
      // state between steps: FP64 (0), FP32 hi and lo arrays (1), interleaved pairs (2)
      r.mixed = b->ff ? 2 : (b->mixed ? 1 : 0);
      r.pad = 0;
      r.rec_w = s.rec_w;
      r.rec_cell = s.rec_cell;
      r.trace = s.trace;
      r.clock = s.clock;
      r.dt = s.dt;
      r.limit = b->blowup_limit;
      r.n_rec = s.n_rec;
      r.N = s.N;
      r.F = s.F;
      r.dim = s.dim;
      rd.push_back(r);
      b->rec_ids.push_back(id);
    }
  b->n_rec_solves = (int)rd.size();
  if (!rd.empty()) {
    if ((e = cudaMalloc(&b->d_rec, rd.size() * sizeof(RecDesc))) != cudaSuccess ||
        (e = cudaMemcpy(b->d_rec, rd.data(), rd.size() * sizeof(RecDesc), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMalloc(&b->d_flags, rd.size() * sizeof(int32_t))) != cudaSuccess ||
        (e = cudaMemset(b->d_flags, 0, rd.size() * sizeof(int32_t))) != cudaSuccess)
      return bcuda(b, e, "receiver table");
  }
  b->dirty = false;
  return EW_OK;
}

// Launch the kernels of one step (parity p) on the batch stream, one group
// after the other: each group's persistent launches fill the GPU, and
// groups run concurrently on separate streams competed for the SMs
// (measured 4% slower for 512 solves of degrees 3..7).
int launch_step(ew_batch* b, int p) {
  cudaError_t e;
  int64_t n = 0;
  for (auto& g : b->groups) {
    const ew::KernelTable& kt = ew::kernel_table(g.dim, g.np);
    const size_t nslot = g.members.size();
    for (int st = 0; st < 5; ++st) {
      ew::LaunchArgs a;
      std::memset(&a, 0, sizeof(a));
      a.solves = g.d_tables + (size_t)(p * 5 + st) * nslot;
      a.work = g.d_work;
      a.n_work = g.n_work;
      a.cells_per_block = g.cb;
      a.err = b->d_err;
      e = kt.cart[g.variant[st]].launch(a, g.sx[st], g.tma, g.nb_lines, g.grid[p][st], b->stream);
      if (e != cudaSuccess) return bcuda(b, e, "batch stage launch");
      ++n;
    }
  }
  if (b->n_rec_solves > 0) {
    receiver_kernel<<<b->n_rec_solves, 256, 0, b->stream>>>(b->d_rec, b->n_rec_solves, 1 - p,
                                                            b->d_flags);
    if ((e = cudaGetLastError()) != cudaSuccess) return bcuda(b, e, "receiver launch");
    ++n;
  }
  b->launches_per_step = n;
  return EW_OK;
}

int capture(ew_batch* b) {
  for (int p = 0; p < 2; ++p) {
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return bcuda(b, e, "begin capture");
    int rc = launch_step(b, p);
    e = cudaStreamEndCapture(b->stream, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return bcuda(b, e, "end capture");
    e = cudaGraphInstantiate(&b->graph[p], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return bcuda(b, e, "graph instantiate");
  }
  return EW_OK;
}

Solve* find(ew_batch* b, int32_t id) {
  auto it = b->solves.find(id);
  return it == b->solves.end() ? nullptr : &it->second;
}

}  // namespace

extern "C" {

int ew_batch_create(const ew_batch_options* opt, ew_batch** out) {
  if (!opt || !out) return EW_ERR_INVALID;
  *out = nullptr;
  if (opt->precision != EW_PREC_FP64 && opt->precision != EW_PREC_MIXED &&
      opt->precision != EW_PREC_MIXED_FF)
    return EW_ERR_INVALID;
  if (opt->hbm_budget_bytes <= 0 || opt->max_solves <= 0) return EW_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || opt->device < 0 || opt->device >= ndev)
    return EW_ERR_CUDA;
  ew_batch* b = new ew_batch;
  b->device = opt->device;
  b->mixed = opt->precision != EW_PREC_FP64;
  b->ff = opt->precision == EW_PREC_MIXED_FF;
  b->use_graphs = opt->use_graphs != 0;
  b->allow_overrun = opt->allow_overrun != 0;
  b->blowup_limit = opt->blowup_limit > 0.0 ? opt->blowup_limit : 0.0;
  b->max_solves = opt->max_solves;
  cudaSetDevice(b->device);
  cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, b->device);
  cudaError_t e = cudaMalloc(&b->arena_base, (size_t)opt->hbm_budget_bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return EW_ERR_OOM;
  }
  b->arena.init((size_t)opt->hbm_budget_bytes);
  if (cudaMalloc(&b->d_err, 4 * sizeof(int)) != cudaSuccess ||
      cudaMemset(b->d_err, 0, 4 * sizeof(int)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    ew_batch_destroy(b);
    return EW_ERR_CUDA;
  }
  b->stream = b->own_stream;
  *out = b;
  return EW_OK;
}

void ew_batch_destroy(ew_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  cudaDeviceSynchronize();
  free_groups(b);
  if (b->arena_base) cudaFree(b->arena_base);
  if (b->d_err) cudaFree(b->d_err);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
}

const char* ew_batch_last_error(const ew_batch* b) { return b ? b->last_error.c_str() : ""; }

int64_t ew_batch_solve_bytes(const ew_batch* b, const ew_solve_desc* s) {
  if (!b || !s || s->mesh.n_cells <= 0 || s->mesh.degree < 1 || s->mesh.degree > EW_MAX_DEGREE ||
      (s->mesh.dim != 2 && s->mesh.dim != 3))
    return -1;
  return (int64_t)solve_layout(s, b->ff ? 2 : (b->mixed ? 1 : 0)).total;
}

int64_t ew_batch_bytes_free(const ew_batch* b) { return b ? (int64_t)b->arena.free_bytes() : -1; }

int ew_batch_add(ew_batch* b, const ew_solve_desc* sd, int32_t* id) {
  if (!b || !sd || !id) return EW_ERR_INVALID;
  bool cart = false;
  std::string err;
  int rc = ew::validate_mesh(&sd->mesh, &cart, &err);
  if (rc) return bfail(b, rc, err);
  if (!cart) return bfail(b, EW_ERR_UNSUPPORTED, "batched solves need Cartesian (axis-aligned) cells");
  if (!ew::kernel_table(sd->mesh.dim, sd->mesh.degree + 1).cart[ew::CV_F64_MID].launch)
    return bfail(b, EW_ERR_UNSUPPORTED, "batched solves: the line kernel is built for 3-D degrees up to 7");
  if (!(sd->dt > 0.0) || sd->n_steps < 1) return bfail(b, EW_ERR_INVALID, "dt and n_steps must be positive");
  if (sd->n_sources < 0 || sd->n_sources > 1 || sd->n_receivers < 0 || sd->n_receivers > 64 ||
      (sd->n_receivers > 0 && !sd->receivers))
    return bfail(b, EW_ERR_INVALID, "0..1 sources and 0..64 receivers");
  if ((int)b->solves.size() >= b->max_solves) return bfail(b, EW_ERR_TOO_LARGE, "max_solves reached");
  cudaSetDevice(b->device);
  const Layout L = solve_layout(sd, b->ff ? 2 : (b->mixed ? 1 : 0));
  size_t off = 0;
  if (!b->arena.alloc(L.total, &off)) return bfail(b, EW_ERR_OOM, "HBM budget exhausted");
  Solve s;
  s.id = b->next_id++;
  s.dim = sd->mesh.dim;
  s.np = sd->mesh.degree + 1;
  s.N = 1;
  for (int d = 0; d < s.dim; ++d) s.N *= s.np;
  s.F = s.dim + 1;
  s.n_cells = sd->mesh.n_cells;
  s.n_dofs = s.n_cells * s.F * s.N;
  s.n_steps = sd->n_steps;
  s.dt = sd->dt;
  s.off = off;
  s.bytes = L.total;
  s.cur = b->parity;
  char* base = b->arena_base + off;
  const size_t ud = ((size_t)s.n_dofs * 8 + kAlign - 1) & ~(kAlign - 1);
  s.U[0] = reinterpret_cast<double*>(base + L.U);
  s.U[1] = reinterpret_cast<double*>(base + L.U + ud);
  if (b->mixed) {
    const size_t xd = ((size_t)s.n_dofs * (b->ff ? 8 : 4) + kAlign - 1) & ~(kAlign - 1);
    s.X[0] = base + L.X;
    s.X[1] = base + L.X + xd;
  } else {
    s.X[0] = base + L.X;
  }
  s.nbr = reinterpret_cast<int32_t*>(base + L.nbr);
  s.cellc = base + L.cellc;
  s.src_w = base + L.src_w;
  s.rec_w = reinterpret_cast<double*>(base + L.rec_w);
  s.rec_cell = reinterpret_cast<int32_t*>(base + L.rec_cell);
  s.trace = reinterpret_cast<double*>(base + L.trace);
  s.clock = reinterpret_cast<double*>(base + L.clock);
  s.n_rec = sd->n_receivers;
  const ew_mesh_desc& m = sd->mesh;
  const int dim = s.dim, nv = 1 << dim;
  // Cartesian kernel constants (same layout as ew_create)
  std::vector<double> cellc((size_t)s.n_cells * kCellConsts, 0.0);
  for (int64_t i = 0; i < s.n_cells; ++i) {
    double* k = &cellc[(size_t)i * kCellConsts];
    const double rho = m.density[i], sp = m.speed[i];
    const double tau = 1.0 / (sp * rho);
    const double* V = m.vertices + (size_t)i * nv * dim;
    k[0] = 1.0 / rho;
    k[1] = rho * sp * sp;
    k[2] = tau;
    k[3] = sp * rho;
    for (int e = 0; e < dim; ++e) k[4 + e] = 1.0 / (V[(nv - 1) * dim + e] - V[e]);
    for (int f = 0; f < 2 * dim; ++f) {
      const int32_t nb = m.neighbors[i * 2 * dim + f];
      if (nb < 0) continue;
      const double tm = 1.0 / (m.speed[nb] * m.density[nb]);
      k[7 + 2 * f] = tm;
      k[8 + 2 * f] = 1.0 / (tau + tm);
    }
  }
  // source: phi_q(x_s) / JxW_q
  std::vector<double> srcw(s.N, 0.0);
  if (sd->n_sources == 1) {
    double xi[3] = {0, 0, 0};
    int32_t cell = -1;
    if (!locate(m, sd->source.position, &cell, xi)) {
      b->arena.release(off, L.total);
      return bfail(b, EW_ERR_INVALID, "source outside the mesh");
    }
    const std::vector<double> phi = point_weights(dim, s.np, xi);
    const ew::GaussRule g = ew::gauss_rule(s.np);
    const double* V = m.vertices + (size_t)cell * nv * dim;
    double vol = 1.0;
    for (int e = 0; e < dim; ++e) vol *= V[(nv - 1) * dim + e] - V[e];
    for (int q = 0; q < s.N; ++q) {
      double w = vol;
      int t = q;
      for (int e = 0; e < dim; ++e) {
        w *= g.w[t % s.np];
        t /= s.np;
      }
      srcw[q] = phi[q] / w;
    }
    s.src_cell = cell;
    s.src_amp = sd->source.amplitude;
    s.src_f0 = sd->source.frequency;
    s.src_t0 = sd->source.delay >= 0.0 ? sd->source.delay : 1.0 / sd->source.frequency;
  }
  std::vector<double> recw((size_t)std::max(s.n_rec, 0) * s.N);
  std::vector<int32_t> reccell(std::max(s.n_rec, 1), 0);
  for (int r = 0; r < s.n_rec; ++r) {
    double xi[3] = {0, 0, 0}, x[3] = {0, 0, 0};
    for (int e = 0; e < dim; ++e) x[e] = sd->receivers[r * dim + e];
    int32_t cell = -1;
    if (!locate(m, x, &cell, xi)) {
      b->arena.release(off, L.total);
      return bfail(b, EW_ERR_INVALID, "receiver outside the mesh");
    }
    const std::vector<double> phi = point_weights(dim, s.np, xi);
    std::copy(phi.begin(), phi.end(), recw.begin() + (size_t)r * s.N);
    reccell[r] = cell;
  }
  cudaError_t e = cudaSuccess;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, b->stream);
  };
  std::vector<float> cf, sf;
  if (b->ff) {
    // float pairs (hi, lo) of the FP64 values
    auto pairs = [](const std::vector<double>& v) {
      std::vector<float> r(v.size() * 2);
      for (size_t i = 0; i < v.size(); ++i) {
        const ew::FF f = ew::FF::from_double(v[i]);
        r[2 * i] = f.hi;
        r[2 * i + 1] = f.lo;
      }
      return r;
    };
    cf = pairs(cellc);
    sf = pairs(srcw);
    up(s.cellc, cf.data(), cf.size() * 4);
    up(s.src_w, sf.data(), sf.size() * 4);
  } else if (b->mixed) {
    cf = cast_vec<float>(cellc);
    sf = cast_vec<float>(srcw);
    up(s.cellc, cf.data(), cf.size() * 4);
    up(s.src_w, sf.data(), sf.size() * 4);
  } else {
    up(s.cellc, cellc.data(), cellc.size() * 8);
    up(s.src_w, srcw.data(), srcw.size() * 8);
  }
  up(s.nbr, m.neighbors, (size_t)s.n_cells * 2 * dim * 4);
  up(s.rec_w, recw.data(), recw.size() * 8);
  up(s.rec_cell, reccell.data(), reccell.size() * 4);
  if (e == cudaSuccess) e = cudaMemsetAsync(s.U[0], 0, (size_t)s.n_dofs * 8, b->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(s.U[1], 0, (size_t)s.n_dofs * 8, b->stream);
  // mixed: the zero state's hi and lo parts
  for (int k = 0; b->mixed && !b->ff && k < 2; ++k)
    if (e == cudaSuccess) e = cudaMemsetAsync(s.X[k], 0, (size_t)s.n_dofs * 4, b->stream);
  if (e == cudaSuccess) {
    // time, steps taken, n_steps, status (a pageable source: staged before the call returns)
    const double clock0[4] = {0.0, 0.0, (double)s.n_steps, 0.0};
    e = cudaMemcpyAsync(s.clock, clock0, sizeof(clock0), cudaMemcpyHostToDevice, b->stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);  // host vectors go out of scope
  if (e != cudaSuccess) {
    b->arena.release(off, L.total);
    return bcuda(b, e, "solve upload");
  }
  b->solves[s.id] = s;
  b->dirty = true;
  *id = s.id;
  return EW_OK;
}

int ew_batch_remove(ew_batch* b, int32_t id) {
  if (!b) return EW_ERR_INVALID;
  Solve* s = find(b, id);
  if (!s) return bfail(b, EW_ERR_INVALID, "unknown solve id");
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  b->arena.release(s->off, s->bytes);
  b->solves.erase(id);
  b->dirty = true;
  return EW_OK;
}

int ew_batch_set_state(ew_batch* b, int32_t id, const double* state) {
  if (!b || !state) return EW_ERR_INVALID;
  Solve* s = find(b, id);
  if (!s) return bfail(b, EW_ERR_INVALID, "unknown solve id");
  cudaSetDevice(b->device);
  if (s->steps_done != 0) return bfail(b, EW_ERR_INVALID, "set_state before the first step only");
  cudaError_t e;
  if (b->mixed && !b->ff) {
    // the state's hi and lo parts, read by the next first stage
    const int threads = 256;
    const int64_t blocks = std::min<int64_t>((s->n_dofs + threads - 1) / threads, 1 << 20);
    split_state_kernel<<<(unsigned)blocks, threads, 0, b->stream>>>(
        state, s->n_dofs, static_cast<float*>(s->X[s->cur]), reinterpret_cast<float*>(s->U[1]));
    e = cudaGetLastError();
  } else if (b->ff) {
    const int threads = 256;
    const int64_t blocks = std::min<int64_t>((s->n_dofs + threads - 1) / threads, 1 << 20);
    split_pairs_kernel<<<(unsigned)blocks, threads, 0, b->stream>>>(
        state, s->n_dofs, reinterpret_cast<float2*>(s->U[s->cur]));
    e = cudaGetLastError();
  } else {
    e = cudaMemcpyAsync(s->U[s->cur], state, (size_t)s->n_dofs * 8, cudaMemcpyDeviceToDevice,
                        b->stream);
  }
  return e == cudaSuccess ? EW_OK : bcuda(b, e, "set state");
}

int ew_batch_get_state(ew_batch* b, int32_t id, double* state) {
  if (!b || !state) return EW_ERR_INVALID;
  Solve* s = find(b, id);
  if (!s) return bfail(b, EW_ERR_INVALID, "unknown solve id");
  cudaSetDevice(b->device);
  cudaError_t e;
  if (b->mixed && !b->ff) {
    const int threads = 256;
    const int64_t blocks = std::min<int64_t>((s->n_dofs + threads - 1) / threads, 1 << 20);
    join_state_kernel<<<(unsigned)blocks, threads, 0, b->stream>>>(
        static_cast<const float*>(s->X[s->cur]), reinterpret_cast<const float*>(s->U[1]), s->n_dofs,
        state);
    e = cudaGetLastError();
  } else if (b->ff) {
    const int threads = 256;
    const int64_t blocks = std::min<int64_t>((s->n_dofs + threads - 1) / threads, 1 << 20);
    join_pairs_kernel<<<(unsigned)blocks, threads, 0, b->stream>>>(
        reinterpret_cast<const float2*>(s->U[s->cur]), s->n_dofs, state);
    e = cudaGetLastError();
  } else {
    e = cudaMemcpyAsync(state, s->U[s->cur], (size_t)s->n_dofs * 8, cudaMemcpyDeviceToDevice,
                        b->stream);
  }
  return e == cudaSuccess ? EW_OK : bcuda(b, e, "get state");
}

int ew_batch_step(ew_batch* b, int32_t n_steps) {
  if (!b || n_steps < 0) return EW_ERR_INVALID;
  if (n_steps == 0) return EW_OK;
  cudaSetDevice(b->device);
  int64_t left = INT64_MAX;
  for (auto& kv : b->solves)
    if (kv.second.steps_done < kv.second.n_steps)
      left = std::min(left, kv.second.n_steps - kv.second.steps_done);
  if (left == INT64_MAX) return EW_OK;  // nothing to do
  if (n_steps > left && !b->allow_overrun)
    return bfail(b, EW_ERR_INVALID, "n_steps exceeds the steps left of an unfinished solve");
  int rc;
  if (b->dirty) {
    if ((rc = rebuild(b))) return rc;
    if (b->use_graphs && (rc = capture(b))) return rc;
  }
  for (int i = 0; i < n_steps; ++i) {
    if (b->use_graphs) {
      cudaError_t e = cudaGraphLaunch(b->graph[b->parity], b->stream);
      if (e != cudaSuccess) return bcuda(b, e, "graph launch");
      b->launches += b->launches_per_step;
    } else {
      if ((rc = launch_step(b, b->parity))) return rc;
      b->launches += b->launches_per_step;
    }
    b->parity ^= 1;
  }
  bool finished = false;
  for (auto& kv : b->solves)
    if (kv.second.steps_done < kv.second.n_steps) {
      kv.second.steps_done = std::min(kv.second.n_steps, kv.second.steps_done + n_steps);
      kv.second.cur ^= (n_steps & 1);
      if (kv.second.steps_done >= kv.second.n_steps) finished = true;
    }
  // parity changed for everyone: solves keep their state in U[parity]
  if (finished) b->dirty = true;
  return EW_OK;
}

int ew_batch_info(const ew_batch* b, int32_t id, int64_t* steps_done, int64_t* n_steps) {
  if (!b) return EW_ERR_INVALID;
  auto it = b->solves.find(id);
  if (it == b->solves.end()) return EW_ERR_INVALID;
  if (steps_done) *steps_done = it->second.steps_done;
  if (n_steps) *n_steps = it->second.n_steps;
  return EW_OK;
}

int ew_batch_diverged(ew_batch* b, int32_t* ids, int32_t capacity, int32_t* count) {
  if (!b || !count || capacity < 0 || (capacity > 0 && !ids)) return EW_ERR_INVALID;
  *count = 0;
  cudaSetDevice(b->device);
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "synchronize");
  if (b->n_rec_solves == 0 || !b->d_flags) return EW_OK;
  std::vector<int32_t> flags(b->n_rec_solves);
  e = cudaMemcpy(flags.data(), b->d_flags, flags.size() * sizeof(int32_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return bcuda(b, e, "diverged flags");
  for (size_t i = 0; i < flags.size(); ++i)
    if (flags[i] && *count < capacity) ids[(*count)++] = b->rec_ids[i];
  return EW_OK;
}

int ew_batch_receivers(ew_batch* b, int32_t id, int64_t first, int64_t count, double* out) {
  if (!b || !out || first < 0 || count < 0) return EW_ERR_INVALID;
  Solve* s = find(b, id);
  if (!s) return bfail(b, EW_ERR_INVALID, "unknown solve id");
  if (first + count > s->steps_done) return bfail(b, EW_ERR_INVALID, "samples not yet computed");
  if (count == 0 || s->n_rec == 0) return EW_OK;
  cudaSetDevice(b->device);
  cudaError_t e = cudaMemcpyAsync(out, s->trace + first * s->n_rec, (size_t)count * s->n_rec * 8,
                                  cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  return e == cudaSuccess ? EW_OK : bcuda(b, e, "receiver readback");
}

int ew_batch_set_stream(ew_batch* b, void* stream) {
  if (!b) return EW_ERR_INVALID;
  b->stream = stream ? static_cast<cudaStream_t>(stream) : b->own_stream;
  b->dirty = true;  // graphs are replayed on the stream; re-capture for clarity
  return EW_OK;
}

int ew_batch_synchronize(ew_batch* b) {
  if (!b) return EW_ERR_INVALID;
  cudaSetDevice(b->device);
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bcuda(b, e, "synchronize");
  int flags = 0;
  e = cudaMemcpy(&flags, b->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return bcuda(b, e, "error flag");
  if (flags) {
    cudaMemset(b->d_err, 0, sizeof(int));
    return bfail(b, EW_ERR_DEVICE, "device error flag " + std::to_string(flags));
  }
  return EW_OK;
}

int64_t ew_batch_kernel_launches(const ew_batch* b) { return b ? b->launches : -1; }

}  // extern "C"
