// Block eigensolver for the lowest excitons and the matrix-free operator driver.
//
// LOBPCG (Knyazev's locally optimal block preconditioned CG) with
//   - the diagonal (transition-energy) preconditioner |diag(H) - theta|^-1, floored;
//   - soft locking: converged columns keep their place in X but get no new search direction;
//   - orthonormalisation of the basis [X W P] by Cholesky of its scaled Gram matrix in the basis's order with
//     deflation (directions whose residual norm falls below tau are dropped) followed by Rayleigh-Ritz on the
//     kept directions,
//     whose small eigenproblem is solved by Householder tridiagonalisation, bisection and inverse
//     iteration on one CTA (small_eig.cuh);
//   - all projected (3m x 3m) matrices kept in complex(8) on the device.
// The iteration vectors are in precision S.  In every mode the last step is an FP64 Rayleigh-Ritz on
// the final block with a freshly applied operator: FP64 Gram matrices, FP64 eigen-decomposition, FP64
// residual norms.  It replaces slepc_solver (src/module_slepc_solver.F90:12-97: Krylov-Schur,
// EPS_SMALLEST_MAGNITUDE, tol 1e-8, 200 iterations); for the positive BSE spectra of this path the
// smallest-magnitude and smallest-algebraic eigenvalues coincide.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <cstdlib>

#include "solver.h"

namespace wtb {

#define CK(x)                                                         \
  do {                                                                \
    cudaError_t e__ = (x);                                            \
    if (e__ != cudaSuccess) {                                         \
      if (msg) *msg = std::string(#x) + ": " + cudaGetErrorString(e__); \
      return WTB_ECUDA;                                               \
    }                                                                 \
  } while (0)

template <class S>
cudaError_t MatFreeOperator<S>::apply(const cplx<S>* X, int ldx, int c0, int ncol, cplx<S>* Y, int ldy,
                                      cudaStream_t s) {
  if (!vec_s || !dE_s) return cudaErrorInvalidValue;  // the operator's precision copies were never set
  this->matvec_columns += ncol;
  for (int b0 = 0; b0 < ncol; b0 += nbmax) {
    const int nb = ncol - b0 < nbmax ? ncol - b0 : nbmax;
    const int N = 2 * w * w * nb;
    cudaError_t e;
    if (kind == GEMM_TC_BF16) {
      if constexpr (sizeof(S) == 4) {
        e = launch_mf_gather<float, uint16_t>(X, ldx, c0 + b0, nb, vec_s, nk, nv, nc, w, Zs, Kpad, nslices,
                                              (long)Npad * Kpad, s, gather_tile);
        if (e != cudaSuccess) return e;
        TcGemmPlan* plan = plan_for(N, npairs, tile_n);
        if (!plan) return cudaErrorInvalidValue;
        cudaEvent_t ea = nullptr, eb = nullptr;
        // the live profile covers the iteration's contraction launches (the final split run is a
        // different launch configuration and is left out of it)
        const bool profiled = prof && prof->on && !final_apply && !this->capturing;
        if (profiled) {
          cudaEventCreate(&ea);
          cudaEventCreate(&eb);
          cudaEventRecord(ea, s);
        }
        e = final_apply ? tc_gemm_run_split(plan, st, s, kchunk_final) : tc_gemm_run(plan, st, s);
        if (e != cudaSuccess) return e;

        if (profiled) {
          cudaEventRecord(eb, s);
          prof->pending.emplace_back(ea, eb);
          prof->launches += 1;
          prof->flops += 2.0 * nk * (double)N * nk * npairs;
          prof->bytes += 2.0 * nslices * ((double)nk * nk + (double)N * nk) + 4.0 * nk * (double)N;
        }
        e = launch_mf_scatter<float, float>(reinterpret_cast<const float*>(Tm), Npad, X, ldx, vec_s, dE_s, nk, nv, nc,
                                            w, nb, Y, ldy, c0 + b0, s, scatter_cols);
        if (e != cudaSuccess) return e;
      } else {
        return cudaErrorInvalidValue;
      }
    } else {
      e = launch_mf_gather<S, S>(X, ldx, c0 + b0, nb, vec_s, nk, nv, nc, w, Zr, Kpad, 1, 0, s, gather_tile);
      if (e != cudaSuccess) return e;
      cudaEvent_t ea = nullptr, eb = nullptr;
      const bool profiled = prof && prof->on && !this->capturing;
      if (profiled) {
        cudaEventCreate(&ea);
        cudaEventCreate(&eb);
        cudaEventRecord(ea, s);
      }
      e = contract_z(N, s, false);
      if (e != cudaSuccess) return e;
      if (profiled) {
        cudaEventRecord(eb, s);
        prof->pending.emplace_back(ea, eb);
        prof->launches += 1;
        prof->flops += contraction_flops(N);
        prof->bytes += contraction_bytes(N);
      }
      if (kind == GEMM_FFT_F32) {
        if constexpr (sizeof(S) == 4)
          e = launch_mf_scatter_t(reinterpret_cast<const float*>(Tm), Kpad, X, ldx, vec_s, dE_s, nk, nv, nc, w, nb, Y,
                                  ldy, c0 + b0, s, scatter_cols);
      } else {
        e = launch_mf_scatter<S, S>(reinterpret_cast<const S*>(Tm), Npad, X, ldx, vec_s, dE_s, nk, nv, nc, w, nb, Y,
                                    ldy, c0 + b0, s);
      }
      if (e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

template <class S>
cudaError_t MatFreeOperator<S>::time_contraction(int reps, int ncol, cudaStream_t s) {
  if (!prof) return cudaSuccess;
  const int N = 2 * w * w * std::min(ncol, nbmax);
  const int np = npairs0 > 0 ? npairs0 : npairs;
  TcGemmPlan* plan = nullptr;
  if (kind == GEMM_TC_BF16) {
    plan = plan_for(N, np, tile_n);
    if (!plan) return cudaErrorInvalidValue;
  }
  for (int r = 0; r < reps; ++r) {
    cudaEvent_t ea, eb;
    cudaError_t e = cudaEventCreate(&ea);
    if (e != cudaSuccess) return e;
    e = cudaEventCreate(&eb);
    if (e != cudaSuccess) return e;
    cudaEventRecord(ea, s);
    if (plan)
      e = tc_gemm_run(plan, st, s);
    else
      e = contract_z(N, s, false);
    if (e != cudaSuccess) return e;
    cudaEventRecord(eb, s);
    prof->pending.emplace_back(ea, eb);
    prof->launches += 1;
    if (plan) {
      prof->flops += 2.0 * nk * (double)N * nk * np;
      prof->bytes += 2.0 * nslices * ((double)nk * nk + (double)N * nk) + 4.0 * nk * (double)N;
    } else {
      prof->flops += contraction_flops(N);
      prof->bytes += contraction_bytes(N);
    }
  }
  return cudaSuccess;
}

template <class S>
cudaError_t MatFreeOperator<S>::contract(const cplx<S>* X, int ldx, int ncol, cudaStream_t s) {
  if (ncol > nbmax || !vec_s) return cudaErrorInvalidValue;
  const int N = 2 * w * w * ncol;
  if (kind == GEMM_TC_BF16) {
    if constexpr (sizeof(S) == 4) {
      cudaError_t e = launch_mf_gather<float, uint16_t>(X, ldx, 0, ncol, vec_s, nk, nv, nc, w, Zs, Kpad, nslices,
                                                        (long)Npad * Kpad, s, gather_tile);
      if (e != cudaSuccess) return e;
      TcGemmPlan* plan = plan_for(N, npairs, tile_n);
      if (!plan) return cudaErrorInvalidValue;
      return tc_gemm_run(plan, st, s);
    } else {
      return cudaErrorInvalidValue;
    }
  }
  cudaError_t e = launch_mf_gather<S, S>(X, ldx, 0, ncol, vec_s, nk, nv, nc, w, Zr, Kpad, 1, 0, s, gather_tile);
  if (e != cudaSuccess) return e;
  return contract_z(N, s, true);
}

// T = V Z for the N gathered columns in Zr: FP32 FFT convolutions (FFT kind) or the CUDA-core product
template <class S>
cudaError_t MatFreeOperator<S>::contract_z(int N, cudaStream_t s, bool t_kn) {
  if (kind == GEMM_FFT_F32) {
    // contract() leaves T[k][n] (row k, leading dimension Npad) as the other kinds do; the applications keep
    // Z's layout T[n][k] (leading dimension Kpad), which the FFT writes and the scatter reads contiguously
    if constexpr (sizeof(S) == 4)
      return launch_fft_conv(reinterpret_cast<const float*>(Zr), Kpad, N / 2, mesh1, mesh2, fft_p, fft_spec, fft_tw,
                             reinterpret_cast<float*>(Tm), t_kn ? Npad : Kpad, t_kn, s);
    return cudaErrorInvalidValue;
  }
  return launch_simt_gemm_tn<S>(Vr, Kpad, Zr, Kpad, reinterpret_cast<S*>(Tm), Npad, nk, N, Kpad, s);
}

// algorithmic flops and bytes of one contraction of N columns: the product's 2 nk^2 N, or for the FFT kind
// 5 P log2(P) per P-point transform, (2 n1 + 2 P) transforms per column pair, plus the spectrum products
template <class S>
double MatFreeOperator<S>::contraction_flops(int N) const {
  if (kind == GEMM_FFT_F32) {
    const double lg = std::log2((double)fft_p);
    return (N / 2) * ((2.0 * mesh1 + 2.0 * fft_p) * 5.0 * fft_p * lg + 6.0 * fft_p * fft_p);
  }
  return 2.0 * nk * (double)N * nk;
}

// Z read and T written once (FP32 for the FFT kind, with its P x P FP32 spectrum read once; every column pair
// rereads it from L2), and the nk x nk table for the product
template <class S>
double MatFreeOperator<S>::contraction_bytes(int N) const {
  if (kind == GEMM_FFT_F32) return 4.0 * 2.0 * N * nk + 8.0 * (double)fft_p * fft_p;
  return sizeof(S) * ((double)nk * nk + (double)N * nk + (double)nk * N);
}

template <class S>
TcGemmPlan* MatFreeOperator<S>::plan_for(int N, int np, int bn) {
  const long key = ((long)N * 16 + np) * 2 + (bn == 128 ? 1 : 0);
  auto it = plans.find(key);
  if (it != plans.end()) return it->second;
  std::string m2;
  TcGemmPlan* plan = nullptr;
  if (tc_gemm_plan_create(&plan, Vs, Mpad, Kpad, (long)Mpad * Kpad, nslices, Zs, Npad, (long)Npad * Kpad, nslices,
                          reinterpret_cast<float*>(Tm), Npad, np, pa, pb, &m2, bn) != WTB_OK) {
    if (msg) *msg = m2;
    return nullptr;
  }
  tc_gemm_set_valid(plan, nk, N);
  plans[key] = plan;
  return plan;
}

// The three launch shapes of an application, one parameter at a time: the contraction tile, then the gather
// tile, then the scatter's column group, each timed as whole nbmax-column applications (gather, contraction and
// scatter) with the choices made so far.  The three kernels are separate launches whose times add, so this
// coordinate order finds the best combination of the candidates.  None of the choices changes a result: each
// output element is summed in the same order whatever the tile.
template <class S>
cudaError_t MatFreeOperator<S>::autotune(cudaStream_t s, const cplx<S>* X, cplx<S>* Y) {
  if (kind != GEMM_TC_BF16 && kind != GEMM_FFT_F32) return cudaSuccess;
  const bool fft = kind == GEMM_FFT_F32;
  char shape[160];
  if (fft)
    std::snprintf(shape, sizeof(shape), "matfree-fft nk=%d nv=%d nc=%d w=%d cols=%d mesh=%dx%d P=%d", nk, nv, nc, w,
                  nbmax, mesh1, mesh2, fft_p);
  else
    std::snprintf(shape, sizeof(shape), "matfree nk=%d nv=%d nc=%d w=%d cols=%d slices=%d products=%d", nk, nv, nc, w,
                  nbmax, nslices, npairs);
  auto run = [&]() -> cudaError_t {
    const long mv = this->matvec_columns;
    const cudaError_t e = apply(X, nbmax, 0, nbmax, Y, nbmax, s);
    this->matvec_columns = mv;
    return e;
  };
  if (!fft)
    tile_n = tune_choice(shape, "tile_n", {256, 128}, 256, [&](int c) {
      tile_n = c;
      return run();
    }, s);
  // gather tiles: 16 or 8 k' per CTA, chunks of 1, 2 or 4 block columns (those within 200 KB of shared memory);
  // the FFT form also the lane-k gather over 32 k' (its Z rows are k-contiguous)
  std::vector<int> gt;
  for (int kt : {16, 8})
    for (int p : {4, 2, 1})
      if (p <= nbmax &&
          (size_t)(kt * nc * w + kt * nv * w + kt * nc * nv * p + kt * nc * w * p) * sizeof(zf) <= 200 * 1024)
        gt.push_back(kt * 100 + p);
  if (fft)
    for (int p : {4, 2, 1})
      if (p <= nbmax && (size_t)(nv * w + nc * w + nc * nv * p + nc * w * p) * 33 * sizeof(zf) <= 200 * 1024)
        gt.push_back(3200 + p);
  gather_tile = tune_choice(shape, "gather_tile", gt, 0, [&](int c) {
    gather_tile = c;
    return run();
  }, s);
  // scatter columns per CTA: the k-point scatter from nbmax down, the FFT form's k-tiled scatter 2, 4 or 8
  std::vector<int> sc;
  if (fft) {
    for (int g : {2, 4, 8})
      if (g <= nbmax) sc.push_back(g);
    // the lane-k scatter over 32 k-points, 2, 4 or 8 block columns (coded 100 + columns)
    for (int g : {2, 4, 8})
      if (g <= nbmax && (size_t)(nv * w + nc * w + g * w * nv) * 33 * sizeof(zf) <= 200 * 1024) sc.push_back(100 + g);
  } else {
    for (int g = nbmax; g >= 1 && sc.size() < 3; g = g > 1 ? (g + 1) / 2 : 0) sc.push_back(g);
  }
  scatter_cols = tune_choice(shape, "scatter_cols", sc, 0, [&](int c) {
    scatter_cols = c;
    return run();
  }, s);
  return cudaGetLastError();
}

template struct MatFreeOperator<float>;
template struct MatFreeOperator<double>;

cudaError_t BatchMatFreeOperator::apply(const zf* X, int ldx, int c0, int ncol, zf* Y, int ldy, cudaStream_t s) {
  this->matvec_columns += ncol;
  const int* skip = final_apply ? nullptr : frozen;
  for (int b0 = 0; b0 < ncol; b0 += nbmax) {
    const int nb = ncol - b0 < nbmax ? ncol - b0 : nbmax;
    cudaError_t e = launch_mf_gather_batch(X, ldx, c0 + b0, nb, d_sys, d_gtiles, ngtiles, max_nv, max_nc, max_w,
                                           nslices, skip, s);
    if (e != cudaSuccess) return e;
    e = final_apply ? tc_gemm_group_run_split(gemm, npairs, nullptr, st, s, kchunk_final)
                    : tc_gemm_group_run(gemm, npairs, skip, st, s);
    if (e != cudaSuccess) return e;
    e = launch_mf_scatter_batch(X, ldx, d_sys, d_kpts, nkpts, max_nv, max_nc, max_w, nb, Y, ldy, c0 + b0, skip, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

namespace {

struct Small {
  zd *M, *G, *B, *Gp, *U, *Y, *C, *T;
  double *lam, *theta, *dinv;
  int* keep;
};

// Rayleigh-Ritz on the basis Sb (nrow x nb, ld) with ASb = H Sb: returns C (nb x m) and theta (m) of every
// system of bm (small matrices nn apart, theta ts apart).
// Orthonormalisation: Cholesky of the scaled Gram matrix in [X W P] order with deflation (directions whose
// residual diagonal falls below tau are dropped; the r kept ones come first in B); the projected r x r
// problem B^H G B is solved by the tridiagonal route (small_eig.cuh).  The small problems run in precision S,
// or FP64 for small_in_fp64.  A missing Ritz pair (r < m) has theta = 1e30 and a zero column in C.
template <class S>
int rayleigh_ritz(const cplx<S>* Sb, const cplx<S>* ASb, int ld, int nb, int m, int nrow, double tau, Small& sm,
                  double* partial, int npart, DevStatus* st, cudaStream_t s, std::string* msg, bool small_in_fp64,
                  const BatchMap& bm, long nn, long ts) {
  (void)st;
  if (nb <= 48) {
    // both Grams in one pass over the basis (bitwise the same sums as two separate launches; with 33..48 FP32
    // columns the upper triangles only, the lower ones their conjugates)
    CK(launch_gram_pair<S>(Sb, ASb, ld, nb, nrow, sm.M, sm.G, partial, npart, s, bm, nn));
  } else {
    CK(launch_gram<S>(Sb, ld, nb, Sb, ld, nb, nrow, sm.M, partial, npart, s, bm, nn));
    CK(launch_gram<S>(Sb, ld, nb, ASb, ld, nb, nrow, sm.G, partial, npart, s, bm, nn));
  }
  if (small_in_fp64)
    CK(launch_pchol_basis<double>(sm.M, nb, nb, tau, sm.B, nb, sm.keep, s, bm, nn, nn));
  else
    CK(launch_pchol_basis<S>(sm.M, nb, nb, tau, sm.B, nb, sm.keep, s, bm, nn, nn));
  // the projected matrix B^H G B stays FP64 (its rounding would mix near-degenerate Ritz vectors); the basis
  // combination C = B Y may run in FP32 when the iteration does
  const bool f32 = !small_in_fp64 && sizeof(S) == 4;
  CK(launch_small_gemm(sm.G, nb, 0, sm.B, nb, sm.T, nb, nb, nb, nb, s, false, bm, nn, nn, nn));
  CK(launch_small_gemm(sm.B, nb, 1, sm.T, nb, sm.Gp, nb, nb, nb, nb, s, false, bm, nn, nn, nn));
  if (small_in_fp64)
    CK(launch_heev_small<double>(sm.Gp, nb, sm.keep, nb, m, sm.theta, sm.Y, nb, s, bm, nn, ts, nn));
  else
    CK(launch_heev_small<S>(sm.Gp, nb, sm.keep, nb, m, sm.theta, sm.Y, nb, s, bm, nn, ts, nn));
  CK(launch_small_gemm(sm.B, nb, 0, sm.Y, nb, sm.C, m, nb, m, nb, s, f32, bm, nn, nn, nn));
  return WTB_OK;
}

}  // namespace

// ------------------------------------------------------------------------------------------------
// Device-resident loop.  One solve is one CUDA graph: set-up, a WHILE node whose body is one LOBPCG
// iteration (bf16x3: a second WHILE node for the 6-product phase, after a static switch block), then the
// final FP64 Rayleigh-Ritz.  The decisions the host used to take every iteration (soft locking,
// convergence, the stagnation and breakdown guards, the iteration cap) are taken by lob_control_kernel,
// which sets the loop's condition with cudaGraphSetConditional; the host synchronises once per solve.
// The basis is always [X W P] (3m columns): W and P start at zero and the Cholesky
// orthonormalisation drops zero columns, so the first iteration needs no separate 2m-column path.

struct LobCtl {
  int it, total_it, nconv, stop, converged, restore, save, failed, best_it, nworse, pad[2];
  double maxrel, best_maxrel, saved_rel, tol;
};

// One thread per system; block 0 also clears the loop's completion counter.
__global__ void lob_ctl_reset_kernel(LobCtl* ctl, double tol, int keep_total, int* frozen, int* counter) {
  const int q = blockIdx.x;
  LobCtl* c = ctl + q;
  c->it = 0;
  if (!keep_total) {
    c->total_it = 0;
    c->failed = 0;
  }
  c->nconv = 0;
  c->stop = 0;
  c->converged = 0;
  c->restore = 0;
  c->save = 0;
  c->best_it = 0;
  c->nworse = 0;
  c->maxrel = 1e300;
  c->best_maxrel = 1e300;
  c->saved_rel = 1e300;
  c->tol = tol;
  frozen[q] = 0;
  if (q == 0) {
    counter[0] = 0;
    counter[1] = 0;
  }
}

// One CTA of 256 threads per system: the residual norms of system q are first summed from the residual kernel's
// parts ([npart][32] in partial, written to norms2), then warp 0 decides.  rel_j = ||r_j|| / |theta_j|;
// converged columns leave the active set (soft locking).
//  - breakdown guard: near the operator's rounding floor the running AX drifts from H X and LOBPCG can lose
//    consistency (Ritz values falling far below the spectrum): the block with the lowest residual of the
//    phase is kept (save), and a residual 10x above it after reaching 100 x tol restores it and ends the
//    phase (restore);
//  - floor guard (reduced precision): a best block within 1.5 x tol followed by one iteration that does not
//    improve on it, or within 3 x tol followed by two, sits at the rounding floor of the FP32 iteration: the
//    best block is restored and the FP64 Rayleigh-Ritz takes over;
//  - stagnation guard (reduced precision): residuals within 100 x tol that have not improved by 10% over
//    15 iterations are at the operator's rounding floor; the FP64 Rayleigh-Ritz takes over;
//  - the iteration cap, a non-finite residual and a device status word end the loop as well.
// A system that stops is frozen: the iteration kernels leave it alone until the next phase.  The last CTA
// to finish (a completion counter) sets the loop's condition: another pass while any system is running;
// counter[1] holds the same answer for the host-driven loop.
// Monitor lines follow the reference's MyEPSMonitor (src/module_slepc_solver.F90:101-116).
__global__ void __launch_bounds__(256) lob_control_kernel(LobCtl* ctl, double* __restrict__ norms2,
                                                          const double* __restrict__ partial, int npart, BatchMap bm,
                                                          const double* __restrict__ theta, int theta_stride, int m,
                                                          int nev, int maxit, int reduced, int* __restrict__ active,
                                                          const DevStatus* __restrict__ st, int* __restrict__ frozen,
                                                          int* counter, int nsys, cudaGraphConditionalHandle h,
                                                          int in_graph, int monitor) {
  __shared__ double red[8][33];
  const int lane = threadIdx.x;
  const int q = blockIdx.x;
  LobCtl* c = ctl + q;
  if (!frozen[q]) {  // uniform over the CTA
    const double t = sum_parts_cta(partial, npart, 32, lane & 31, q, bm, red);
    if (lane < 32) norms2[32 * q + lane] = t;
  }
  if (lane >= 32) return;
  __syncwarp();
  if (!frozen[q]) {
    norms2 += 32 * q;
    theta += (size_t)q * theta_stride;
    active += 32 * q;
    const double tol = c->tol;
    double rel = 0.0;
    int conv = 1, bad = 0;
    if (lane < m) {
      const double rn = sqrt(fmax(norms2[lane], 0.0));
      const double th = theta[lane];
      bad = !(isfinite(rn) && isfinite(th));
      rel = rn / fmax(fabs(th), 1e-12);
      conv = rel <= tol;
      active[lane] = conv ? 0 : 1;
    }
    double mr = lane < nev ? rel : 0.0;
    int nc = lane < nev ? conv : 0;
    int first = lane < nev && !conv ? lane : 1 << 20;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
      nc += __shfl_xor_sync(0xffffffffu, nc, o);
      bad |= __shfl_xor_sync(0xffffffffu, bad, o);
      first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
    }
    if (lane == 0) {
      int stop = 0;
      c->save = 0;
      if (st->code) {
        stop = 1;
      } else if (bad) {
        c->failed = WTB_ENAN;
        stop = 1;
      } else {
        c->maxrel = mr;
        c->nconv = nc;
        if (mr < c->saved_rel) {
          c->saved_rel = mr;
          c->save = 1;
          c->nworse = 0;
        } else {
          c->nworse += 1;
          if ((c->saved_rel <= 100.0 * tol && mr > 10.0 * c->saved_rel) ||
              (reduced && ((c->saved_rel <= 1.5 * tol && c->nworse >= 1) || (c->saved_rel <= 3.0 * tol && c->nworse >= 2)))) {
            c->restore = 1;
            c->converged = 1;
            stop = 1;
          }
        }
        if (!stop && nc == nev) {
          c->converged = 1;
          stop = 1;
        }
        if (!stop) {
          if (mr < 0.9 * c->best_maxrel) {
            c->best_maxrel = mr;
            c->best_it = c->it;
          } else if (reduced && mr <= 100.0 * tol && c->it - c->best_it >= 15) {
            c->converged = 1;
            stop = 1;
          }
        }
        if (!stop && c->total_it >= maxit) stop = 1;
      }
      if (monitor) {
        const int f = first < nev ? first : nev - 1;
        if (nsys > 1)
          printf("WTB-EPS system %4d %5d EPS pair=%4d value (error) %15.8E (%10.3E) max %10.3E\n", q, c->total_it,
                 nc + 1, theta[f], sqrt(fmax(norms2[f], 0.0)) / fmax(fabs(theta[f]), 1e-12), mr);
        else
          printf("WTB-EPS %5d EPS pair=%4d value (error) %15.8E (%10.3E) max %10.3E\n", c->total_it, nc + 1, theta[f],
                 sqrt(fmax(norms2[f], 0.0)) / fmax(fabs(theta[f]), 1e-12), mr);
      }
      if (!stop) {
        c->it += 1;
        c->total_it += 1;
      }
      c->stop = stop;
      if (stop) frozen[q] = 1;
    }
  } else if (lane == 0) {
    c->save = 0;
  }
  if (lane == 0) {
    __threadfence();
    if (atomicAdd(counter, 1) == nsys - 1) {
      __threadfence();
      int any = 0;
      for (int i = 0; i < nsys; ++i) any |= (((volatile LobCtl*)ctl)[i].stop == 0) ? 1 : 0;
      counter[0] = 0;
      counter[1] = any;
      if (in_graph) cudaGraphSetConditional(h, any ? 1u : 0u);
    }
  }
}

// dst[:, 0:ncol] = src[:, 0:ncol] on the rows of the systems whose save (which = 0) or restore (1) flag is set
template <class S>
__global__ void cond_copy_kernel(const LobCtl* __restrict__ ctl, int which, const cplx<S>* __restrict__ src, int lds,
                                 cplx<S>* __restrict__ dst, int ldd, int ncol, int nrow, BatchMap bm) {
  const long n = (long)nrow * ncol;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long r = e / ncol;
    const int c = (int)(e % ncol);
    const LobCtl& cq = ctl[bm_sys_of_row(bm, r)];
    if (!(which ? cq.restore : cq.save)) continue;
    dst[r * ldd + c] = src[r * lds + c];
  }
}

// In place: X <- [X W P] C and P <- [W P] C[m:3m, :] for the basis and for its image under H.  A CTA takes one
// row tile (kUpdRows rows) of both blocks at once: it stages the tile's rows of S and of AS in shared memory (so
// the in-place writes cannot overtake reads; rows padded to nb + 2 complex, so that the four rows a warp reads
// at one column fall in distinct banks and 16-byte copies stay aligned), then each thread forms one pair of
// output columns of the same row of S and of AS: per input column one load from each staged row and one 16-byte
// load of C serve four complex FMAs.  Each output keeps the summation order of a plain loop (X block, then
// [W P]), independent of the tiling.  C of the tile's system is staged again only when the system changes.
constexpr int kUpdRows = kTileRows;
template <int BYTES>
__device__ __forceinline__ void upd_cp_async(void* dst, const void* src) {
  if constexpr (BYTES == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
  else
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}

// Stages of the row tiles: two for FP32 (the next tile's rows are copied by cp.async while the current one is
// combined), one for FP64 (two would not fit in shared memory)
template <class S>
__host__ __device__ constexpr int upd_stages() { return sizeof(S) == 4 ? 2 : 1; }

template <class S>
__global__ void __launch_bounds__(256) lob_update_kernel(cplx<S>* __restrict__ Sb, cplx<S>* __restrict__ ASb, int ld,
                                                         int m, const zd* __restrict__ C, int nrow, BatchMap bm,
                                                         long c_stride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int NST = upd_stages<S>();
  const int nb = 3 * m, RS = nb + 2;
  cplx<S>* Cs = reinterpret_cast<cplx<S>*>(smem_raw);  // [3m][m]
  cplx<S>* Rs = Cs + ((nb * m + 1) & ~1);              // [NST][2][kUpdRows][RS]: rows of S, then of AS
  const int STG = 2 * kUpdRows * RS;                   // one stage
  const int ngrp = (m + 1) >> 1;      // pairs of output columns
  const int items = kUpdRows * ngrp;  // (row, pair) items per tile
  const bool vec = sizeof(S) == 4 && (ld & 1) == 0 && (nb & 1) == 0;
  auto tile_r0 = [&](long t) { return ((long)blockIdx.x + t * gridDim.x) * kUpdRows; };
  // copies of a tile's rows of S and AS into stage buf (none for a tile past the end or of a frozen system; every
  // call commits one group, so that the wait counts stay in step)
  auto stage = [&](int buf, long r0) {
    if (r0 < nrow && !bm_frozen(bm, bm_sys_of_row(bm, r0))) {
      const int nr = (int)min((long)kUpdRows, nrow - r0);
      for (int which = 0; which < 2; ++which) {
        const cplx<S>* base = (which ? ASb : Sb) + r0 * ld;
        cplx<S>* dst = Rs + buf * STG + which * kUpdRows * RS;
        if (vec) {  // two complex FP32 per 16-byte copy
          const int hp = nb >> 1;
          for (int e = threadIdx.x; e < nr * hp; e += blockDim.x) {
            const int rr = e / hp, c2 = e - rr * hp;
            upd_cp_async<16>(dst + rr * RS + 2 * c2, base + (size_t)rr * ld + 2 * c2);
          }
        } else {
          for (int e = threadIdx.x; e < nr * nb; e += blockDim.x) {
            const int rr = e / nb, c = e - rr * nb;
            upd_cp_async<sizeof(cplx<S>)>(dst + rr * RS + c, base + (size_t)rr * ld + c);
          }
        }
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  int staged = -1;
  if (NST == 2) stage(0, tile_r0(0));
  for (long t = 0; tile_r0(t) < nrow; ++t) {
    const long r0 = tile_r0(t);
    const int buf = NST == 2 ? (int)(t & 1) : 0;
    if (NST == 2) {
      stage(buf ^ 1, tile_r0(t + 1));  // the next tile's copies in flight
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      stage(0, r0);
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    const int sys = bm_sys_of_row(bm, r0);  // uniform over the CTA
    const bool live = !bm_frozen(bm, sys);
    if (live && sys != staged) {  // the previous tile's reads of Cs ended at the last barrier
      const zd* Cq = C + (size_t)sys * c_stride;
      for (int e = threadIdx.x; e < nb * m; e += blockDim.x) Cs[e] = mk<S>((S)Cq[e].re, (S)Cq[e].im);
      staged = sys;
    }
    __syncthreads();  // every thread's copies of this tile (and Cs) are visible
    const int nr = (int)min((long)kUpdRows, nrow - r0);
    const cplx<S>* Rb = Rs + buf * STG;
    if (live) {
      for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int rr = it / ngrp, g = it - rr * ngrp;
        if (rr >= nr) continue;
        const int j0 = g * 2;
        const bool two = j0 + 1 < m;
        const cplx<S>* rs = Rb + rr * RS;
        const cplx<S>* ra = Rb + (kUpdRows + rr) * RS;
        cplx<S> xs0 = mk<S>(0, 0), xs1 = mk<S>(0, 0), ps0 = mk<S>(0, 0), ps1 = mk<S>(0, 0);
        cplx<S> xa0 = mk<S>(0, 0), xa1 = mk<S>(0, 0), pa0 = mk<S>(0, 0), pa1 = mk<S>(0, 0);
        for (int i = 0; i < m; ++i) {  // the X block contributes to X only
          const cplx<S> si = rs[i], ai = ra[i];
          const cplx<S>* crow = Cs + i * m + j0;
          const cplx<S> c0 = crow[0], c1 = two ? crow[1] : mk<S>(0, 0);
          cfma(xs0, si, c0);
          cfma(xa0, ai, c0);
          cfma(xs1, si, c1);
          cfma(xa1, ai, c1);
        }
        for (int i = m; i < nb; ++i) {  // W and P contribute to X and to the new P
          const cplx<S> si = rs[i], ai = ra[i];
          const cplx<S>* crow = Cs + i * m + j0;
          const cplx<S> c0 = crow[0], c1 = two ? crow[1] : mk<S>(0, 0);
          cfma(ps0, si, c0);
          cfma(pa0, ai, c0);
          cfma(ps1, si, c1);
          cfma(pa1, ai, c1);
        }
        cplx<S>* os = Sb + (r0 + rr) * ld;
        cplx<S>* oa = ASb + (r0 + rr) * ld;
        os[j0] = mk<S>(xs0.re + ps0.re, xs0.im + ps0.im);
        os[2 * m + j0] = ps0;
        oa[j0] = mk<S>(xa0.re + pa0.re, xa0.im + pa0.im);
        oa[2 * m + j0] = pa0;
        if (two) {
          os[j0 + 1] = mk<S>(xs1.re + ps1.re, xs1.im + ps1.im);
          os[2 * m + j0 + 1] = ps1;
          oa[j0 + 1] = mk<S>(xa1.re + pa1.re, xa1.im + pa1.im);
          oa[2 * m + j0 + 1] = pa1;
        }
      }
    }
    __syncthreads();  // this stage's rows (and Cs) are read before the next copies into it
  }
}

struct CaptureSeg {
  cudaStream_t s;
  cudaError_t begin(cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps) {
    return cudaStreamBeginCaptureToGraph(s, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                         cudaStreamCaptureModeRelaxed);
  }
  cudaError_t end(std::vector<cudaGraphNode_t>* tail) {
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* d = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &d, nullptr, &nd);
    if (tail && e == cudaSuccess) tail->assign(d, d + nd);
    cudaGraph_t g2 = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(s, &g2);
    return e != cudaSuccess ? e : e2;
  }
};

template <class S>
int lobpcg_solve_batch(Operator<S>& op, const double* diag, const BatchLayout& L, int nev, int m, double tol,
                       int maxit, Workspace& ws, DevStatus* st, cudaStream_t s, std::vector<double>* E, zd* Xout,
                       std::vector<SolveStats>* stats, std::vector<int>* sys_status, std::string* msg,
                       double tol_refine, SolveGraph* sg) {
  const int nsys = L.bm.nsys;
  const int nrow = L.nrow;
  int mindim = nrow;
  for (int d : L.dims) mindim = std::min(mindim, d);
  if (nsys < 1 || (int)L.dims.size() != nsys || (nsys > 1 && !L.bm.rows) ||
      (L.bm.rows && (!L.bm.parts || !L.bm.part_sys || !L.bm.sys_parts || !L.bm.tile_sys || L.nparts < 1))) {
    if (msg) *msg = "inconsistent batch layout";
    return WTB_EBADARG;
  }
  if (m < nev) m = nev;
  if (m > mindim) m = mindim;
  if (nev < 1 || nev > mindim) {
    if (msg) *msg = "nev must be between 1 and the BSE dimension";
    return WTB_EBADARG;
  }
  const int ld = 3 * m;
  const int nb = 3 * m;
  if (nb > (sizeof(S) == 4 ? 96 : 78) || m > 32) {
    if (msg) *msg = "eigensolver block too large (3*block must be <= 96 in FP32, <= 78 in FP64)";
    return WTB_EBADARG;
  }
  // a ragged layout (row tables present) selects its start vectors per system over the systems' own rows and
  // keeps the padding rows zero; its reductions run over its part table
  const bool ragged = L.bm.rows != nullptr;
  // reduction parts of the tall-skinny Grams and residual norms: parts of 192 rows, at most 304 (each part's
  // FP64 partial of a 48 x 48 Gram is 36 KB, and the sum over parts reads all of them).  Not autotuned: a part
  // sums its rows in FP32, so the part count sets the Grams' rounding.  Measured on the 57,600 workload: 304
  // parts made the Gram pair 0.8 us faster than 300 (63.7 against 64.5 us), and the solve took 12 iterations
  // instead of 10.  A ragged batch keeps its own part table.
  const int npart = ragged ? L.nparts : std::max(1, std::min(304, (nrow + 191) / 192));
  cudaError_t err = cudaSuccess;
  cplx<S>* Sb = ws.get<cplx<S>>("lob_S", (size_t)nrow * ld, &err, true);
  cplx<S>* ASb = ws.get<cplx<S>>("lob_AS", (size_t)nrow * ld, &err, true);
  cplx<S>* Xbest = ws.get<cplx<S>>("lob_Xbest", (size_t)nrow * m, &err);
  Small sm;
  const long nn = (long)nb * nb;
  sm.M = ws.get<zd>("lob_M", (size_t)nsys * nn, &err);
  sm.G = ws.get<zd>("lob_G", (size_t)nsys * nn, &err);
  sm.B = ws.get<zd>("lob_B", (size_t)nsys * nn, &err);
  sm.Gp = ws.get<zd>("lob_Gp", (size_t)nsys * nn, &err);
  sm.U = nullptr;
  sm.Y = ws.get<zd>("lob_Y", (size_t)nsys * nn, &err);
  sm.C = ws.get<zd>("lob_C", (size_t)nsys * nn, &err);
  sm.T = ws.get<zd>("lob_T", (size_t)nsys * nn, &err);
  sm.lam = nullptr;
  sm.dinv = nullptr;
  sm.theta = ws.get<double>("lob_theta", (size_t)nsys * nb, &err);
  sm.keep = ws.get<int>("lob_keep", nsys, &err);
  double* partial = ws.get<double>("lob_partial", (size_t)npart * nn * 4, &err);  // the Gram pair's two sets
  double* norms2 = ws.get<double>("lob_norms2", (size_t)nsys * 32, &err);
  int* active = ws.get<int>("lob_active", (size_t)nsys * 32, &err);
  int* idx = ws.get<int>("lob_idx", ragged ? (size_t)nsys * m : 65 * 128, &err);
  double* cand = ws.get<double>("lob_cand", ragged ? (size_t)nsys * (kSelSlices + 1) * m : 65 * 128, &err);
  int* cand_idx = ws.get<int>("lob_cand_idx", ragged ? (size_t)nsys * kSelSlices * m : 1, &err);
  double* th_dev = ws.get<double>("lob_thcur", (size_t)nsys * nb, &err);
  LobCtl* ctl = ws.get<LobCtl>("lob_ctl", nsys, &err);
  int* frozen = ws.get<int>("lob_frozen", nsys, &err);
  int* counter = ws.get<int>("lob_counter", 2, &err);
  zd* X64 = ws.get<zd>("fin_X", (size_t)nrow * 2 * m, &err);
  zd* T64 = ws.get<zd>("fin_T", (size_t)nrow * m, &err);
  if (err != cudaSuccess) {
    if (msg) *msg = std::string("device allocation failed: ") + cudaGetErrorString(err);
    return WTB_ENOMEM;
  }
  BatchMap bm = L.bm;  // iteration kernels: frozen systems are left alone
  bm.frozen = frozen;
  bm.nparts = npart;
  BatchMap bmf = bm;   // set-up and final step: every system
  bmf.frozen = nullptr;
  cplx<S>* X = Sb;
  cplx<S>* W = Sb + m;
  cplx<S>* P = Sb + 2 * m;
  cplx<S>* AX = ASb;
  cplx<S>* AW = ASb + m;
  cplx<S>* AP = ASb + 2 * m;
  // orthonormalisation threshold: a kept direction's Rayleigh quotient carries the operator's rounding
  // divided by its residual norm, so tau sits well above the FP32 noise and just above FP64's
  const double tau = sizeof(S) == 4 ? 1e-4 : 1e-13;
  const bool reduced = sizeof(S) == 4;
  const bool monitor = std::getenv("WTB_EPS_MONITOR") != nullptr;
  const bool two_phase = tol_refine > 0.0 && tol_refine < tol;
  // WTB_SOLVER_STREAM: the same kernels launched directly on the stream, the host reading the loop state
  // between iterations (for kernel-level profilers, which do not replay kernels inside conditional graph
  // bodies); the default runs the whole solve as one graph launch
  const bool stream_mode = std::getenv("WTB_SOLVER_STREAM") != nullptr && !sg;
  const size_t upd_smem =
      (size_t)(((nb * m + 1) & ~1) + upd_stages<S>() * 2 * kUpdRows * (nb + 2)) * sizeof(cplx<S>);
  // FP32: a few tiles per CTA, so that the copies of the next overlap the combination of the current one
  const int upd_grid =
      std::max(1, std::min(upd_stages<S>() == 2 ? 152 * 3 : 152 * 8, (nrow + kUpdRows - 1) / kUpdRows));
  const unsigned cp_grid = (unsigned)std::max(1, std::min(152 * 4, (int)(((long)nrow * m + 255) / 256)));

  // the pieces of one iteration, as stream launches (captured below)
  // the iteration's Ritz values go straight to th_dev (the final step's to sm.theta)
  Small smi = sm;
  smi.theta = th_dev;
  auto rr_and_update = [&]() -> int {
    int r = rayleigh_ritz<S>(Sb, ASb, ld, nb, m, nrow, tau, smi, partial, npart, st, s, msg, false, bm, nn, nb);
    if (r) return r;
    CK(raise_smem_limit(reinterpret_cast<const void*>(lob_update_kernel<S>), upd_smem));
    lob_update_kernel<S><<<upd_grid, 256, upd_smem, s>>>(Sb, ASb, ld, m, sm.C, nrow, bm, nn);
    ++g_launch_count;
    CK(cudaGetLastError());
    return WTB_OK;
  };
  auto check_and_decide = [&](cudaGraphConditionalHandle h) -> int {
    // W <- the preconditioned residual (the inactive columns are zeroed by the next iteration's projections)
    // the residual's parts are summed by the control kernel
    CK(launch_residual<S>(AX, ld, X, ld, th_dev, m, nrow, W, ld, partial, npart, norms2, s, bm, nb, diag, false));
    lob_control_kernel<<<nsys, 256, 0, s>>>(ctl, norms2, partial, bm.parts ? bm.nparts : npart, bm, th_dev, nb, m, nev,
                                            maxit, reduced ? 1 : 0, active, st, frozen, counter, nsys, h,
                                            stream_mode ? 0 : 1, monitor ? 1 : 0);
    ++g_launch_count;
    CK(cudaGetLastError());
    cond_copy_kernel<S><<<cp_grid, 256, 0, s>>>(ctl, 0, X, ld, Xbest, m, m, nrow, bmf);
    ++g_launch_count;
    CK(cudaGetLastError());
    return WTB_OK;
  };
  auto restart_from_x = [&](cudaGraphConditionalHandle h) -> int {
    CK(cudaMemset2DAsync(W, sizeof(cplx<S>) * ld, 0, sizeof(cplx<S>) * 2 * m, nrow, s));
    CK(cudaMemset2DAsync(AW, sizeof(cplx<S>) * ld, 0, sizeof(cplx<S>) * 2 * m, nrow, s));
    CK(op.apply(X, ld, 0, m, AX, ld, s));
    int r = rr_and_update();
    if (r) return r;
    return check_and_decide(h);
  };
  auto iteration = [&](cudaGraphConditionalHandle h) -> int {
    // W <- W - X (X^H W);  P <- P - X (X^H P), AP <- AP - AX (X^H P): one Gram X^H [W P] (W and P are adjacent
    // column blocks) and one pass for the three projections; P and AP do not depend on W's image
    CK(launch_gram<S>(X, ld, m, W, ld, 2 * m, nrow, sm.T, partial, npart, s, bm, nn));
    CK(launch_orth_update<S>(X, AX, ld, m, sm.T, W, P, AP, nrow, s, bm, nn, active));
    CK(op.apply(W, ld, 0, m, AW, ld, s));
    int r = rr_and_update();
    if (r) return r;
    return check_and_decide(h);
  };
  auto setup = [&]() -> int {
    lob_ctl_reset_kernel<<<nsys, 1, 0, s>>>(ctl, tol, 0, frozen, counter);
    ++g_launch_count;
    CK(cudaMemset2DAsync(Sb, sizeof(cplx<S>) * ld, 0, sizeof(cplx<S>) * ld, nrow, s));
    CK(cudaMemset2DAsync(ASb, sizeof(cplx<S>) * ld, 0, sizeof(cplx<S>) * ld, nrow, s));
    if (ragged) {
      CK(launch_select_lowest_batch(diag, bmf, m, idx, m, cand, cand_idx, s));
      CK(launch_init_guess<S>(X, ld, nrow, m, idx, 12345u, s, bmf, m));
    } else {
      CK(launch_select_lowest(diag, nrow, m, idx, cand, s));
      CK(launch_init_guess<S>(X, ld, nrow, m, idx + 64 * m, 12345u, s));
    }
    return WTB_OK;
  };
  auto phase2_start = [&]() -> int {
    cond_copy_kernel<S><<<cp_grid, 256, 0, s>>>(ctl, 1, Xbest, m, X, ld, m, nrow, bmf);
    ++g_launch_count;
    lob_ctl_reset_kernel<<<nsys, 1, 0, s>>>(ctl, tol_refine, 1, frozen, counter);
    ++g_launch_count;
    CK(cudaGetLastError());
    return WTB_OK;
  };
  // final FP64 Rayleigh-Ritz on a fresh application of the operator's most accurate arithmetic (the
  // iteration's AX is a running linear combination of cheaper applications)
  std::function<int()> final_step = [&]() -> int {
    cond_copy_kernel<S><<<cp_grid, 256, 0, s>>>(ctl, 1, Xbest, m, X, ld, m, nrow, bmf);
    ++g_launch_count;
    op.begin_refine();
    op.set_final(true);
    const cudaError_t fe = op.apply(X, ld, 0, m, AX, ld, s);
    op.set_final(false);
    CK(fe);
    if (sizeof(S) == 4 && m <= 32) {
      // FP32 data: the Grams, the small problem and the combinations X C, AX C with FP64 accuracy from FP32
      // instructions (k_final.cu)
      const zf* Xf = reinterpret_cast<const zf*>(X);
      const zf* AXf = reinterpret_cast<const zf*>(AX);
      CK(launch_gram_pair_dot2(Xf, AXf, ld, m, nrow, sm.M, sm.G, partial, npart, s, bmf, nn));
      CK(launch_small_rr(sm.M, sm.G, m, m, 1e-13, sm.theta, sm.C, sm.keep, s, bmf, nn, nb));
      // Xout = X C[:, :nev]; residual = (AX C - Xout theta)
      CK(launch_update_dot2(Xf, ld, m, sm.C, m, nev, nrow, Xout, nev, s, bmf, nn));
      CK(launch_update_dot2(AXf, ld, m, sm.C, m, nev, nrow, T64, nev, s, bmf, nn));
    } else {
      CK((launch_convert_cols<S, double>(X, ld, X64, 2 * m, m, nrow, s)));
      CK((launch_convert_cols<S, double>(AX, ld, X64 + m, 2 * m, m, nrow, s)));
      int r = rayleigh_ritz<double>(X64, X64 + m, 2 * m, m, m, nrow, 1e-13, sm, partial, npart, st, s, msg, true, bmf,
                                    nn, nb);
      if (r) return r;
      // Xout = X64 C[:, :nev]; residual = (AX64 C - Xout theta)
      CK(launch_update<double>(X64, 2 * m, m, sm.C, m, nev, nrow, Xout, nev, 1.0, 0.0, s, bmf, nn));
      CK(launch_update<double>(X64 + m, 2 * m, m, sm.C, m, nev, nrow, T64, nev, 1.0, 0.0, s, bmf, nn));
    }
    CK(launch_residual<double>(T64, nev, Xout, nev, sm.theta, nev, nrow, T64, nev, partial, npart, norms2, s, bmf, nb));
    return WTB_OK;
  };

  int rc = WTB_OK;
  long long body_launches[2] = {0, 0};
  if (sg && sg->collect) {
    body_launches[0] = sg->body_launches[0];
    body_launches[1] = sg->body_launches[1];
  } else if (stream_mode) {
    auto stopped = [&](bool* stop) -> int {
      int h = 0;
      CK(cudaMemcpyAsync(&h, counter + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      *stop = h == 0;
      return WTB_OK;
    };
    auto run_loop = [&]() -> int {
      for (;;) {
        bool stop = false;
        int r = stopped(&stop);
        if (r) return r;
        if (stop) return WTB_OK;
        r = iteration(0);
        if (r) return r;
      }
    };
    if ((rc = setup())) return rc;
    if ((rc = restart_from_x(0))) return rc;
    if ((rc = run_loop())) return rc;
    if (two_phase) {
      op.begin_refine();
      if ((rc = phase2_start())) return rc;
      if ((rc = restart_from_x(0))) return rc;
      if ((rc = run_loop())) return rc;
    }
    if ((rc = final_step())) return rc;
  } else {
  // the graph of this solve is reused when nothing it was captured with has changed
  std::vector<uint64_t> sig = {(uint64_t)nrow, (uint64_t)nev, (uint64_t)m, (uint64_t)maxit, (uint64_t)sizeof(S),
                               (uint64_t)nsys, (uint64_t)npart, (uint64_t)(uintptr_t)L.bm.tile_sys,
                               (uint64_t)(uintptr_t)L.bm.rows, (uint64_t)(uintptr_t)L.bm.parts,
                               (uint64_t)(uintptr_t)L.bm.part_sys, (uint64_t)(uintptr_t)L.bm.sys_parts,
                               (uint64_t)(uintptr_t)diag, (uint64_t)(uintptr_t)Xout, (uint64_t)(uintptr_t)st,
                               (uint64_t)(uintptr_t)s, (uint64_t)(uintptr_t)Sb, (uint64_t)(uintptr_t)ASb,
                               (uint64_t)(uintptr_t)Xbest, (uint64_t)(uintptr_t)sm.M, (uint64_t)(uintptr_t)sm.G,
                               (uint64_t)(uintptr_t)sm.B, (uint64_t)(uintptr_t)sm.Gp, (uint64_t)(uintptr_t)sm.Y,
                               (uint64_t)(uintptr_t)sm.C, (uint64_t)(uintptr_t)sm.T, (uint64_t)(uintptr_t)sm.theta,
                               (uint64_t)(uintptr_t)sm.keep, (uint64_t)(uintptr_t)partial, (uint64_t)(uintptr_t)norms2,
                               (uint64_t)(uintptr_t)active, (uint64_t)(uintptr_t)idx, (uint64_t)(uintptr_t)cand,
                               (uint64_t)(uintptr_t)cand_idx,
                               (uint64_t)(uintptr_t)th_dev, (uint64_t)(uintptr_t)ctl, (uint64_t)(uintptr_t)frozen,
                               (uint64_t)(uintptr_t)counter, (uint64_t)(uintptr_t)X64, (uint64_t)(uintptr_t)T64,
                               (uint64_t)monitor};
  {
    uint64_t tb, tr;
    std::memcpy(&tb, &tol, 8);
    std::memcpy(&tr, &tol_refine, 8);
    sig.push_back(tb);
    sig.push_back(tr);
  }
  op.signature(&sig);
  uint64_t key = 1469598103934665603ull;  // FNV-1a over the signature words
  for (uint64_t v : sig)
    for (int b = 0; b < 8; ++b) {
      key ^= (v >> (8 * b)) & 0xffu;
      key *= 1099511628211ull;
    }
  if (key == 0) key = 1;
  if (!sg && ws.graph_exec && ws.graph_key == key) {
    body_launches[0] = ws.graph_body_launches[0];
    body_launches[1] = ws.graph_body_launches[1];
    g_launch_count += ws.graph_launches;  // one pass of every captured kernel; the bodies' repeats are added below
    if (cudaGraphLaunch(ws.graph_exec, s) != cudaSuccess) {
      if (msg) *msg = "graph launch failed";
      return WTB_ECUDA;
    }
  } else {
  if (!sg) ws.drop_graph();
  const long long captured0 = g_launch_count.load();
  cudaGraph_t G = nullptr;
  cudaGraphExec_t GX = nullptr;
  if (sg)
    G = sg->graph;
  else
    CK(cudaGraphCreate(&G, 0));
  CaptureSeg cap{s};
  std::vector<cudaGraphNode_t> tail;
  // kernels captured into each loop body (the launch counter counts captured kernels; the bodies then run
  // once per iteration)
  auto segment = [&](cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps, std::vector<cudaGraphNode_t>* out,
                     const std::function<int()>& body) -> int {
    cudaError_t e = cap.begin(g, deps);
    if (e != cudaSuccess) {
      if (msg) *msg = std::string("graph capture: ") + cudaGetErrorString(e);
      return WTB_ECUDA;
    }
    op.capturing = true;
    int r = body();
    op.capturing = false;
    e = cap.end(out);
    if (r == WTB_OK && e != cudaSuccess) {
      if (msg) *msg = std::string("graph capture: ") + cudaGetErrorString(e);
      r = WTB_ECUDA;
    }
    return r;
  };
  auto add_while = [&](const std::vector<cudaGraphNode_t>& deps, cudaGraphConditionalHandle h, cudaGraphNode_t* node,
                       cudaGraph_t* body) -> int {
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    CK(cudaGraphAddNode(node, G, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(), &np));
    *body = np.conditional.phGraph_out[0];
    return WTB_OK;
  };
  do {
    cudaGraphConditionalHandle h1 = 0, h2 = 0;
    if (cudaGraphConditionalHandleCreate(&h1, G, 0, cudaGraphCondAssignDefault) != cudaSuccess ||
        (two_phase && cudaGraphConditionalHandleCreate(&h2, G, 0, cudaGraphCondAssignDefault) != cudaSuccess)) {
      if (msg) *msg = "graph conditional handle creation failed";
      rc = WTB_ECUDA;
      break;
    }
    // set-up: unit vectors at the m lowest transition energies (+ deterministic noise), W = P = 0
    rc = segment(G, sg ? sg->deps : std::vector<cudaGraphNode_t>(), &tail, [&]() -> int {
      int r = setup();
      if (r) return r;
      return restart_from_x(h1);
    });
    if (rc) break;
    cudaGraphNode_t wn;
    cudaGraph_t body;
    if ((rc = add_while(tail, h1, &wn, &body))) break;
    long long c0 = g_launch_count.load();
    if ((rc = segment(body, {}, nullptr, [&]() { return iteration(h1); }))) break;
    body_launches[0] = g_launch_count.load() - c0;
    tail.assign(1, wn);
    if (two_phase) {
      // second phase: the accurate operator; fresh AX from the (best) block, search directions dropped
      op.begin_refine();
      rc = segment(G, tail, &tail, [&]() -> int {
        int r = phase2_start();
        if (r) return r;
        return restart_from_x(h2);
      });
      if (rc) break;
      if ((rc = add_while(tail, h2, &wn, &body))) break;
      c0 = g_launch_count.load();
      if ((rc = segment(body, {}, nullptr, [&]() { return iteration(h2); }))) break;
      body_launches[1] = g_launch_count.load() - c0;
      tail.assign(1, wn);
    }
    rc = segment(G, tail, &tail, final_step);
    if (rc) break;
    if (sg) break;  // the caller instantiates and launches its graph
    if (cudaGraphInstantiate(&GX, G, 0) != cudaSuccess) {
      if (msg) *msg = "graph instantiation failed";
      rc = WTB_ECUDA;
      break;
    }
    if (cudaGraphLaunch(GX, s) != cudaSuccess) {
      if (msg) *msg = "graph launch failed";
      rc = WTB_ECUDA;
      break;
    }
  } while (false);
  if (sg) {
    if (rc == WTB_OK) {
      sg->tail = tail;
      sg->launches = g_launch_count.load() - captured0;
      sg->body_launches[0] = body_launches[0];
      sg->body_launches[1] = body_launches[1];
    }
    return rc;
  }
  if (rc) {
    if (GX) cudaGraphExecDestroy(GX);
    if (G) cudaGraphDestroy(G);
    return rc;
  }
  ws.graph = G;
  ws.graph_exec = GX;
  ws.graph_key = key;
  ws.graph_body_launches[0] = body_launches[0];
  ws.graph_body_launches[1] = body_launches[1];
  ws.graph_launches = g_launch_count.load() - captured0;
  }
  }
  // per system: final Ritz values, the iteration's last Ritz values, residual norms, loop state
  std::vector<double> th((size_t)nsys * nb), th_it((size_t)nsys * nb), nrm((size_t)nsys * 32);
  std::vector<LobCtl> hc(nsys);
  CK(cudaMemcpyAsync(th.data(), sm.theta, sizeof(double) * nsys * nb, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(th_it.data(), th_dev, sizeof(double) * nsys * nb, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(nrm.data(), norms2, sizeof(double) * nsys * 32, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(hc.data(), ctl, sizeof(LobCtl) * nsys, cudaMemcpyDeviceToHost, s));
  DevStatus hst;
  CK(cudaMemcpyAsync(&hst, st, sizeof(hst), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (!stream_mode) {
    // the loop bodies ran once per pass of the slowest system
    int pass1 = 0, pass2 = 0;
    for (int q = 0; q < nsys; ++q) {
      const int it2 = two_phase ? hc[q].it : 0;
      pass1 = std::max(pass1, hc[q].total_it - it2);
      pass2 = std::max(pass2, it2);
    }
    g_launch_count += body_launches[0] * (pass1 - 1) + (two_phase ? body_launches[1] * (pass2 - 1) : 0);
  }
  if (stats) stats->assign(nsys, SolveStats());
  if (sys_status) sys_status->assign(nsys, WTB_OK);
  E->assign((size_t)nsys * nev, 0.0);
  if (hst.code) {
    if (msg) *msg = "device status " + std::to_string(hst.code) + " during the eigensolve";
    return hst.code >= 400 && hst.code < 500 ? WTB_ETIMEOUT : WTB_ENOCONV;
  }
  int first_bad = WTB_OK;
  for (int q = 0; q < nsys; ++q) {
    int code = WTB_OK;
    std::string why;
    double maxrel = 0.0, shift = 0.0;
    if (hc[q].failed == WTB_ENAN) {
      code = WTB_ENAN;
      why = "non-finite residual in the eigensolve";
    }
    for (int j = 0; j < nev && code == WTB_OK; ++j) {
      const double t = th[(size_t)q * nb + j];
      const double rel = std::sqrt(std::max(nrm[(size_t)q * 32 + j], 0.0)) / std::max(std::fabs(t), 1e-12);
      if (!std::isfinite(rel) || !std::isfinite(t)) {
        code = WTB_ENAN;
        why = "non-finite eigenpair after the final Rayleigh-Ritz";
        break;
      }
      maxrel = std::max(maxrel, rel);
      shift = std::max(shift, std::fabs(t - th_it[(size_t)q * nb + j]));
      (*E)[(size_t)q * nev + j] = t;
    }
    if (code == WTB_OK && !hc[q].converged) {
      code = WTB_ENOCONV;
      why = "eigensolver did not converge in " + std::to_string(maxit) + " iterations";
    }
    if (stats) {
      SolveStats& st1 = (*stats)[q];
      st1.iterations = hc[q].total_it;
      st1.launches = 0;
      st1.matvec_columns = (long)m * (hc[q].total_it + (two_phase ? 3 : 2));
      st1.max_rel_residual = maxrel;
      st1.refine_shift_max = shift;
    }
    if (sys_status) (*sys_status)[q] = code;
    if (code != WTB_OK && first_bad == WTB_OK) {
      first_bad = code;
      if (msg) *msg = nsys > 1 ? "system " + std::to_string(q) + ": " + why : why;
    }
  }
  return first_bad;
}

template <class S>
int lobpcg_solve(Operator<S>& op, const double* diag, int dim, int nev, int m, double tol, int maxit, Workspace& ws,
                 DevStatus* st, cudaStream_t s, std::vector<double>* E, zd* Xout, SolveStats* stats,
                 std::string* msg, double tol_refine) {
  BatchLayout L;
  L.nrow = dim;
  L.dims.assign(1, dim);
  std::vector<SolveStats> sv;
  const int rc = lobpcg_solve_batch<S>(op, diag, L, nev, m, tol, maxit, ws, st, s, E, Xout, &sv, nullptr, msg,
                                       tol_refine, nullptr);
  if (stats && !sv.empty()) *stats = sv[0];
  return rc;
}

namespace {

// P H P + sigma Q Q^H with P = I - Q Q^H (Q orthonormal, dim x nq): span(Q) is an exactly invariant subspace with
// eigenvalue sigma, so the eigenpairs still sought are those of H in the complement, up to the residuals of the
// vectors in Q themselves (a shift alone, H + sigma Q Q^H, would perturb them by sigma times the error of Q).
// Applied to a block: T1 = Q^H X, Xp = X - Q T1, Y = H Xp, T2 = Q^H Y, Y += Q (sigma T1 - T2); Q in blocks of at
// most 96 columns, the Gram kernel's limit.
template <class S>
struct DeflatedOperator : Operator<S> {
  Operator<S>* base = nullptr;
  const cplx<S>* Q = nullptr;
  int ldq = 0, nq = 0, dim = 0, npart = 1;
  double sigma = 0.0;
  zd* T1 = nullptr;  // [96][ncol] per Q block, blocks side by side
  zd* T2 = nullptr;
  cplx<S>* Xp = nullptr;  // dim x ncol
  double* partial = nullptr;
  cudaError_t apply(const cplx<S>* X, int ldx, int c0, int ncol, cplx<S>* Y, int ldy, cudaStream_t s) override {
    base->capturing = this->capturing;
    this->matvec_columns += ncol;
    if (nq == 0) return base->apply(X, ldx, c0, ncol, Y, ldy, s);
    cudaError_t e = launch_copy_cols<S>(X + c0, ldx, Xp, ncol, ncol, dim, s);
    for (int q0 = 0; q0 < nq && e == cudaSuccess; q0 += 96) {
      const int qn = std::min(96, nq - q0);
      zd* t1 = T1 + (size_t)q0 * ncol;
      e = launch_gram<S>(Q + q0, ldq, qn, X + c0, ldx, ncol, dim, t1, partial, npart, s);
      if (e == cudaSuccess) e = launch_update<S>(Q + q0, ldq, qn, t1, ncol, ncol, dim, Xp, ncol, -1.0, 1.0, s);
    }
    if (e == cudaSuccess) e = base->apply(Xp, ncol, 0, ncol, Y + c0, ldy, s);
    for (int q0 = 0; q0 < nq && e == cudaSuccess; q0 += 96) {
      const int qn = std::min(96, nq - q0);
      zd* t1 = T1 + (size_t)q0 * ncol;
      zd* t2 = T2 + (size_t)q0 * ncol;
      e = launch_gram<S>(Q + q0, ldq, qn, Y + c0, ldy, ncol, dim, t2, partial, npart, s);
      if (e == cudaSuccess) e = launch_update<S>(Q + q0, ldq, qn, t2, ncol, ncol, dim, Y + c0, ldy, -1.0, 1.0, s);
      if (e == cudaSuccess) e = launch_update<S>(Q + q0, ldq, qn, t1, ncol, ncol, dim, Y + c0, ldy, sigma, 1.0, s);
    }
    return e;
  }
  bool begin_refine() override { return base->begin_refine(); }
  void set_final(bool on) override { base->set_final(on); }
  void signature(std::vector<uint64_t>* sig) const override {
    base->signature(sig);
    uint64_t sb;
    std::memcpy(&sb, &sigma, 8);
    for (uint64_t v : {(uint64_t)7, (uint64_t)(uintptr_t)Q, (uint64_t)ldq, (uint64_t)nq, sb, (uint64_t)(uintptr_t)T1,
                       (uint64_t)(uintptr_t)T2, (uint64_t)(uintptr_t)Xp, (uint64_t)(uintptr_t)partial,
                       (uint64_t)npart})
      sig->push_back(v);
  }
};

}  // namespace

template <class S>
int lobpcg_solve_deflated(Operator<S>& op, const double* diag, int dim, int nev, int chunk, int m, double tol,
                          int maxit, double sigma, Workspace& ws, DevStatus* st, cudaStream_t s, std::vector<double>* E,
                          zd* Xout, SolveStats* stats, std::string* msg, double tol_refine) {
  if (nev < 1 || nev > dim || chunk < 1 || m < chunk) {
    if (msg) *msg = "bad deflated-solve sizes";
    return WTB_EBADARG;
  }
  cudaError_t err = cudaSuccess;
  const int npart = std::max(1, std::min(304, (dim + 191) / 192));
  cplx<S>* Q = ws.get<cplx<S>>("defl_Q", (size_t)dim * nev, &err);
  zd* Xc = ws.get<zd>("defl_X", (size_t)dim * chunk, &err);
  const int qcap = (nev + 95) / 96 * 96;
  zd* T1 = ws.get<zd>("defl_T1", (size_t)qcap * m, &err);
  zd* T2 = ws.get<zd>("defl_T2", (size_t)qcap * m, &err);
  cplx<S>* Xp = ws.get<cplx<S>>("defl_Xp", (size_t)dim * m, &err);
  double* partial = ws.get<double>("defl_partial", (size_t)npart * 96 * m * 2, &err);
  if (err != cudaSuccess) {
    if (msg) *msg = std::string("device allocation failed: ") + cudaGetErrorString(err);
    return WTB_ENOMEM;
  }
  DeflatedOperator<S> dop;
  dop.base = &op;
  dop.Q = Q;
  dop.ldq = nev;
  dop.dim = dim;
  dop.npart = npart;
  dop.sigma = sigma;
  dop.T1 = T1;
  dop.T2 = T2;
  dop.Xp = Xp;
  dop.partial = partial;
  E->assign(nev, 0.0);
  SolveStats tot;
  for (int k0 = 0; k0 < nev; k0 += chunk) {
    const int kc = std::min(chunk, nev - k0);
    dop.nq = k0;
    std::vector<double> Ec;
    SolveStats sc;
    const int rc = lobpcg_solve<S>(dop, diag, dim, kc, std::min(m, dim - k0), tol, maxit, ws, st, s, &Ec, Xc, &sc, msg,
                                   tol_refine);
    if (rc != WTB_OK) {
      if (msg) *msg = "eigenpairs " + std::to_string(k0 + 1) + "-" + std::to_string(k0 + kc) + ": " + *msg;
      return rc;
    }
    for (int j = 0; j < kc; ++j) (*E)[k0 + j] = Ec[j];
    CK(launch_copy_cols<double>(Xc, kc, Xout + k0, nev, kc, dim, s));
    CK((launch_convert_cols<double, S>(Xc, kc, Q + k0, nev, kc, dim, s)));
    tot.iterations += sc.iterations;
    tot.matvec_columns += sc.matvec_columns;
    tot.max_rel_residual = std::max(tot.max_rel_residual, sc.max_rel_residual);
    tot.refine_shift_max = std::max(tot.refine_shift_max, sc.refine_shift_max);
  }
  // ascending order across the chunks (a pair close to a chunk boundary may come out of order): sort, moving
  // the vectors' columns with their values
  std::vector<int> perm(nev);
  for (int j = 0; j < nev; ++j) perm[j] = j;
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return (*E)[a] < (*E)[b]; });
  bool sorted = true;
  for (int j = 0; j < nev; ++j) sorted &= perm[j] == j;
  if (!sorted) {
    zd* tmp = ws.get<zd>("defl_sort", (size_t)dim * nev, &err);
    if (err != cudaSuccess) {
      if (msg) *msg = "device allocation failed";
      return WTB_ENOMEM;
    }
    CK(launch_copy_cols<double>(Xout, nev, tmp, nev, nev, dim, s));
    std::vector<double> Es(nev);
    for (int j = 0; j < nev; ++j) {
      Es[j] = (*E)[perm[j]];
      CK(launch_copy_cols<double>(tmp + perm[j], nev, Xout + j, nev, 1, dim, s));
    }
    *E = Es;
  }
  if (stats) *stats = tot;
  return WTB_OK;
}

template int lobpcg_solve_deflated<float>(Operator<float>&, const double*, int, int, int, int, double, int, double,
                                          Workspace&, DevStatus*, cudaStream_t, std::vector<double>*, zd*, SolveStats*,
                                          std::string*, double);
template int lobpcg_solve_deflated<double>(Operator<double>&, const double*, int, int, int, int, double, int, double,
                                           Workspace&, DevStatus*, cudaStream_t, std::vector<double>*, zd*,
                                           SolveStats*, std::string*, double);

template int lobpcg_solve<float>(Operator<float>&, const double*, int, int, int, double, int, Workspace&, DevStatus*,
                                 cudaStream_t, std::vector<double>*, zd*, SolveStats*, std::string*, double);
template int lobpcg_solve<double>(Operator<double>&, const double*, int, int, int, double, int, Workspace&,
                                  DevStatus*, cudaStream_t, std::vector<double>*, zd*, SolveStats*, std::string*,
                                  double);
template int lobpcg_solve_batch<float>(Operator<float>&, const double*, const BatchLayout&, int, int, double, int,
                                       Workspace&, DevStatus*, cudaStream_t, std::vector<double>*, zd*,
                                       std::vector<SolveStats>*, std::vector<int>*, std::string*, double,
                                       SolveGraph*);
template int lobpcg_solve_batch<double>(Operator<double>&, const double*, const BatchLayout&, int, int, double, int,
                                        Workspace&, DevStatus*, cudaStream_t, std::vector<double>*, zd*,
                                        std::vector<SolveStats>*, std::vector<int>*, std::string*, double,
                                        SolveGraph*);

}  // namespace wtb
