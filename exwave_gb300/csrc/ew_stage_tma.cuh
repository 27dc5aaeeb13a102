// ew_stage_tma.cuh -- staged variant of the general (curved-cell) stage
// kernel: the same operator and epilogues as stage_kernel (one thread per
// Gauss point, element-centric faces), with its inputs moved by the TMA
// engine instead of being loaded by the threads.
//
// Per work item (CB consecutive cells):
//  * stage input X, cell vertices and materials: one bulk copy each into a
//    double buffer, issued one item ahead;
//  * every neighbour cell outside the item (its whole X block and its
//    material row) into a slot of its own, issued by the thread that owns
//    the (cell, face) pair at the start of the item and awaited after the
//    cell term, so the faces read neighbour lines from shared memory;
//  * the FP64 accumulator (RK and ADER updates) into a single buffer at the
//    start of the item, awaited before the epilogue.
// All waits are bounded; a time-out raises ERR_WAIT_TIMEOUT and the CTA
// stops after waiting (bounded) for its copies in flight.  Used when the
// input type equals the compute type and every per-cell block is a
// multiple of 16 bytes (bulk-copy alignment); stage_kernel otherwise.
#pragma once

#include "ew_cart.cuh"
#include "ew_kernels.cuh"

namespace ew {

// Shared-memory layout in bytes.
template <int DIM, int NP>
struct StagedSmem {
  using S = Shape<DIM, NP, false>;
  size_t bar, basis, X, geo, mat, A, nb, nbmat, nbidx, G, Fl, end;
  size_t xbytes, gbytes, mbytes, nbbytes;  // per cell
  __host__ __device__ StagedSmem(int CB, int rsz) {
    auto al = [](size_t v) { return (v + 127) & ~(size_t)127; };
    const int NFACE = 2 * DIM;
    xbytes = (size_t)S::F * S::N * rsz;
    gbytes = (size_t)S::GEO * rsz;
    mbytes = (size_t)4 * rsz;
    nbbytes = xbytes;
    bar = 0;  // mbarriers: 0, 1 X/geo/mat double buffer; 2 neighbours; 3 accumulator
    basis = 64;
    X = al(basis + (size_t)S::BAS * rsz);
    geo = X + 2 * al(CB * xbytes);
    mat = geo + 2 * al(CB * gbytes);
    A = mat + 2 * al(CB * mbytes);
    nb = A + al((size_t)CB * S::F * S::N * 8);
    nbmat = nb + al((size_t)CB * NFACE * nbbytes);
    nbidx = nbmat + al((size_t)CB * NFACE * mbytes);
    G = nbidx + al((size_t)CB * NFACE * 4);
    Fl = G + al((size_t)CB * DIM * S::N * rsz);
    end = Fl + al((size_t)CB * NFACE * S::FF * S::NF * rsz);
  }
};

// Flux at face point fp (as op_face): the neighbour's line comes from the
// item (in-item neighbour) or from its slot in shared memory.
template <int DIM, int NP, typename Real>
__device__ __forceinline__ void op_face_staged(const Real* sB, const Real* sX, Real* sFl,
                                               const Real* sGeo, const Real* sMat,
                                               const Real* sNb, const Real* sNbMat,
                                               const int* sNbIdx, int cell_begin, int nc, int fp,
                                               Real bf, int* err) {
  using S = Shape<DIM, NP, false>;
  constexpr int F = S::F, N = S::N, NF = S::NF;
  const Level<Real> L = get_level(sB, NP, 0);
  const int cl = fp / (2 * DIM * NF);
  const int rem = fp - cl * 2 * DIM * NF;
  const int f = rem / NF;
  const int t = rem - f * NF;
  const int e = f >> 1, s = f & 1;
  int ti[3] = {0, 0, 0};
  const int q0 = face_base<DIM, NP>(e, t, ti);
  const int str = dir_stride(e, NP);
  const Real* Ls = s ? L.L1 : L.L0;
  const Real* Lm = s ? L.L0 : L.L1;
  const Real* x = sX + cl * F * N;
  const Real sgn = s ? Real(1) : Real(-1);
  Real vp[F];
#pragma unroll
  for (int fld = 0; fld < F; ++fld) {
    Real a = Real(0);
#pragma unroll
    for (int j = 0; j < NP; ++j) a += Ls[j] * x[fld * N + q0 + j * str];
    vp[fld] = a;
  }
  // unit normal and face JxW of the multilinear map
  Real nrm[DIM];
  Real xi[DIM];
  Real wt = Real(1);
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    if (d == e) {
      xi[d] = s ? Real(1) : Real(0);
    } else {
      xi[d] = L.x[ti[d]];
      wt *= L.w[ti[d]];
    }
  }
  Real JiT[DIM][DIM];
  const Real det = geom_general<DIM, Real>(sGeo + cl * S::GEO, xi, JiT);
  Real len2 = Real(0);
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    nrm[d] = sgn * JiT[d][e];
    len2 += nrm[d] * nrm[d];
  }
  const Real len = real_sqrt(len2);
  const Real il = Real(1) / len;
#pragma unroll
  for (int d = 0; d < DIM; ++d) nrm[d] *= il;
  const Real jxw_f = wt * real_fabs(det) * len;
  const Real rho = sMat[4 * cl], c = sMat[4 * cl + 1];
  const Real rho_inv = Real(1) / rho, c_sq = c * c;
  const Real tau_p = Real(1) / (c * rho);
  Real un_p = Real(0);
#pragma unroll
  for (int d = 0; d < DIM; ++d) un_p += vp[d] * nrm[d];

  const int slot = cl * 2 * DIM + f;
  const int nb = sNbIdx[slot];
  Real lambda;
  if (nb >= 0) {
    const int nl = nb - cell_begin;
    const bool local = nl >= 0 && nl < nc;
    const Real* xm = local ? sX + nl * F * N : sNb + (size_t)slot * F * N;
    const Real* mm = local ? sMat + 4 * nl : sNbMat + 4 * slot;
    Real vm[F];
#pragma unroll
    for (int fld = 0; fld < F; ++fld) {
      Real a = Real(0);
#pragma unroll
      for (int j = 0; j < NP; ++j) a += Lm[j] * xm[fld * N + q0 + j * str];
      vm[fld] = a;
    }
    const Real rho_m = mm[0], c_m = mm[1];
    Real un_m = Real(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) un_m -= vm[d] * nrm[d];
    const Real tau_m = Real(1) / (c_m * rho_m);
    const Real tau_inv = Real(1) / (tau_p + tau_m);
    lambda = tau_inv * (un_p + un_m + tau_p * vp[DIM] + tau_m * vm[DIM]);
  } else {
    const int id = -nb;
    if (id == EW_BC_SOFT_WALL_ID) {
      lambda = un_p / tau_p + vp[DIM];
    } else if (id == EW_BC_ABSORBING_ID) {
      const Real tsum = tau_p + Real(1) / (c * rho);
      lambda = tau_p / tsum * vp[DIM] + Real(1) / tsum * un_p;
    } else {
      if (id != EW_BC_HARD_WALL_ID) atomicOr(err, ERR_BAD_BOUNDARY_ID);
      lambda = Real(0);
    }
  }
  const Real scale = bf * jxw_f;
  const Real pd = (vp[DIM] - lambda) * rho_inv * scale;
  const Real fpres = c_sq * rho * (-un_p + tau_p * (lambda - vp[DIM])) * scale;
  Real* out = sFl + (cl * 2 * DIM + f) * S::FF * NF + t;
#pragma unroll
  for (int d = 0; d < DIM; ++d) out[d * NF] = pd * nrm[d];
  out[DIM * NF] = fpres;
}

template <int DIM, int NP, typename Real, typename OutT>
__global__ void __launch_bounds__(512, sizeof(Real) == 4 ? 2 : 1) stage_kernel_staged(const LaunchArgs La) {
  using S = Shape<DIM, NP, false>;
  constexpr int F = S::F, N = S::N, NFACE = 2 * DIM;
  extern __shared__ __align__(128) unsigned char smem_st[];
  const int CB = La.cells_per_block;
  const StagedSmem<DIM, NP> lay(CB, (int)sizeof(Real));
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem_st + lay.bar);
  Real* sB = reinterpret_cast<Real*>(smem_st + lay.basis);
  Real* sG = reinterpret_cast<Real*>(smem_st + lay.G);
  Real* sFl = reinterpret_cast<Real*>(smem_st + lay.Fl);
  double* sA = reinterpret_cast<double*>(smem_st + lay.A);
  const Real* sNb = reinterpret_cast<const Real*>(smem_st + lay.nb);
  const Real* sNbMat = reinterpret_cast<const Real*>(smem_st + lay.nbmat);
  int* sNbIdx = reinterpret_cast<int*>(smem_st + lay.nbidx);
  const size_t xs = (lay.geo - lay.X) / 2, gs = (lay.mat - lay.geo) / 2, ms = (lay.A - lay.mat) / 2;
  if ((int)blockDim.x != CB * N || CB * NFACE > (int)blockDim.x) {
    if (threadIdx.x == 0) atomicOr(La.err, ERR_BAD_LAUNCH);
    return;
  }
  // X, vertices and materials of work item w into buffer b
  auto issue = [&](int w, int b) {
    const WorkItem wi = La.work[w];
    const SolveDesc* sdp = La.solves ? La.solves + wi.solve : &La.single;
    const uint32_t nx = (uint32_t)(wi.n_cells * lay.xbytes), ng = (uint32_t)(wi.n_cells * lay.gbytes),
                   nm = (uint32_t)(wi.n_cells * lay.mbytes);
    mbar_expect_tx(&bars[b], nx + ng + nm);
    bulk_g2s(smem_st + lay.X + b * xs, static_cast<const char*>(sdp->X) + (size_t)wi.cell_begin * lay.xbytes,
             nx, &bars[b]);
    bulk_g2s(smem_st + lay.geo + b * gs,
             static_cast<const char*>(sdp->geo) + (size_t)wi.cell_begin * lay.gbytes, ng, &bars[b]);
    bulk_g2s(smem_st + lay.mat + b * ms,
             static_cast<const char*>(sdp->mat) + (size_t)wi.cell_begin * lay.mbytes, nm, &bars[b]);
  };
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init(&bars[2], blockDim.x);  // every thread arrives once per item
    mbar_init(&bars[3], 1);
    fence_barrier_init();
  }
  load_basis<Real>(La.basis, sB, basis_total(NP));
  __syncthreads();
  if (threadIdx.x == 0 && (int)blockIdx.x < La.n_work) issue(blockIdx.x, 0);

  uint32_t phase = 0;  // bit b: parity of the next wait on buffer b
  int it = 0;
  for (int w = blockIdx.x; w < La.n_work; w += gridDim.x, ++it) {
    const int b = it & 1;
    const WorkItem wi = La.work[w];
    const SolveDesc sd = pick(La, wi.solve);  // by value: no reloads after stores
    const int nc = wi.n_cells;
    const bool has_next = w + (int)gridDim.x < La.n_work;
    const bool stage_a = sd.mode != MODE_APPLY;
    const uint32_t par = (uint32_t)it & 1u;
    // accumulator of this item (single buffer, read by the epilogue only)
    if (threadIdx.x == 0 && stage_a) {
      fence_proxy_async();
      const uint32_t na = (uint32_t)(nc * F * N * 8);
      mbar_expect_tx(&bars[3], na);
      bulk_g2s(sA, sd.A + (size_t)wi.cell_begin * F * N, na, &bars[3]);
    }
    // neighbours outside the item: the thread of each (cell, face) pair
    // copies the neighbour's block and material row
    {
      uint32_t bytes = 0;
      const int t = threadIdx.x;
      int nb = -EW_BC_HARD_WALL_ID;
      if (t < nc * NFACE) {
        const int cell = wi.cell_begin + t / NFACE;
        nb = sd.nbr[(size_t)cell * NFACE + t % NFACE];
        if (nb >= sd.n_cells) {
          atomicOr(La.err, ERR_BAD_NEIGHBOR);
          nb = cell;
        }
        sNbIdx[t] = nb;
        const int nl = nb - wi.cell_begin;
        if (nb >= 0 && !(nl >= 0 && nl < nc)) bytes = (uint32_t)(lay.nbbytes + lay.mbytes);
      }
      fence_proxy_async();
      mbar_expect_tx(&bars[2], bytes);  // arrive.expect_tx: one arrival per thread
      if (bytes) {
        bulk_g2s(smem_st + lay.nb + (size_t)t * lay.nbbytes,
                 static_cast<const char*>(sd.X) + (size_t)nb * lay.xbytes, (uint32_t)lay.nbbytes, &bars[2]);
        bulk_g2s(smem_st + lay.nbmat + (size_t)t * lay.mbytes,
                 static_cast<const char*>(sd.mat) + (size_t)nb * lay.mbytes, (uint32_t)lay.mbytes, &bars[2]);
      }
    }
    // next item's X, vertices and materials
    if (threadIdx.x == 0 && has_next) {
      fence_proxy_async();
      issue(w + gridDim.x, b ^ 1);
    }
    bool ok = mbar_wait(&bars[b], (phase >> b) & 1u);
    phase ^= (1u << b);
    const Real* sX = reinterpret_cast<const Real*>(smem_st + lay.X + b * xs);
    const Real* sGeo = reinterpret_cast<const Real*>(smem_st + lay.geo + b * gs);
    const Real* sMat = reinterpret_cast<const Real*>(smem_st + lay.mat + b * ms);
    __syncthreads();  // neighbour indices written
    const Real bf = static_cast<Real>(sd.bf);
    const int cl = threadIdx.x / N;
    const int q = threadIdx.x - cl * N;
    const bool active = cl < nc;
    Real Ru[DIM];
    Real inv_jxw = Real(1);
    if (ok && active) op_cell<DIM, NP, Real, false>(sB, sX, sG, sGeo, sMat, cl, q, bf, Ru, inv_jxw);
    ok = mbar_wait(&bars[2], par) && ok;
    for (int fp = threadIdx.x; ok && fp < nc * NFACE * S::NF; fp += blockDim.x)
      op_face_staged<DIM, NP, Real>(sB, sX, sFl, sGeo, sMat, sNb, sNbMat, sNbIdx, wi.cell_begin, nc,
                                    fp, bf, La.err);
    __syncthreads();
    if (stage_a) ok = mbar_wait(&bars[3], par) && ok;
    if (ok && active) {
      Real k[F];
      op_collect<DIM, NP, Real, false>(sB, sG, sFl, cl, q, Ru, inv_jxw, k);
      const size_t g0 = ((size_t)wi.cell_begin + cl) * F * N + q;
      const int l0 = cl * F * N + q;
      if (!stage_a) {
#pragma unroll
        for (int fld = 0; fld < F; ++fld) {
          if constexpr (is_f64_v<Real>)
            sd.Aout[g0 + fld * N] = k[fld];
          else if constexpr (is_ff_v<Real>)
            sd.Aout[g0 + fld * N] = f32_to_f64(k[fld].hi) + f32_to_f64(k[fld].lo);
          else
            sd.Aout[g0 + fld * N] = f32_to_f64(k[fld]);
        }
      } else if constexpr (is_ff_v<Real>) {
        // compensated: next stage input a + f1 k as a float pair, FP64
        // accumulator from the FF increment
        const bool mid = sd.mode == MODE_RK_MID;
#pragma unroll
        for (int fld = 0; fld < F; ++fld) {
          const size_t g = g0 + fld * N;
          const double a = sA[l0 + fld * N];
          if (mid) {
            float ah, al;
            f64_split(a, ah, al);
            static_cast<FF*>(sd.Xout)[g] = FF(ah, al) + FF(sd.f1_hi, sd.f1_lo) * k[fld];
          }
          const FF inc = (mid ? FF(sd.fb_hi, sd.fb_lo) : FF(sd.f1_hi, sd.f1_lo)) * k[fld];
          sd.Aout[g] = a + (f32_to_f64(inc.hi) + f32_to_f64(inc.lo));
        }
      } else {
        // stage_kernel's epilogue with the staged accumulator
        const bool mid = sd.mode == MODE_RK_MID;
#pragma unroll
        for (int fld = 0; fld < F; ++fld) {
          const size_t g = g0 + fld * N;
          const double a = sA[l0 + fld * N];
          if constexpr (is_f64_v<Real>) {
            const double xn = a + sd.f1 * k[fld];
            if (mid) static_cast<OutT*>(sd.Xout)[g] = static_cast<OutT>(xn);
            sd.Aout[g] = fma(mid ? sd.f2 : 0.0, k[fld], xn);
          } else {
            const float kf = k[fld];
            if (mid) static_cast<OutT*>(sd.Xout)[g] = static_cast<OutT>(fmaf(sd.f1f, kf, f64_to_f32(a)));
            const float ch = mid ? sd.fb_hi : sd.f1_hi, cl2 = mid ? sd.fb_lo : sd.f1_lo;
            sd.Aout[g] = a + f32_to_f64(fmaf(ch, kf, cl2 * kf));
          }
        }
      }
    }
    if (__syncthreads_or(!ok)) {
      // a bulk copy timed out: wait (bounded) for the copies still in
      // flight, then stop this CTA
      if (threadIdx.x == 0) {
        atomicOr(La.err, ERR_WAIT_TIMEOUT);
        if (has_next) mbar_wait(&bars[b ^ 1], (phase >> (b ^ 1)) & 1u);
        mbar_wait(&bars[2], par);
        if (stage_a) mbar_wait(&bars[3], par);
      }
      break;
    }
  }
}

}  // namespace ew
