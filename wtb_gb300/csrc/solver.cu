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
#include <cmath>
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
  this->matvec_columns += ncol;
  for (int b0 = 0; b0 < ncol; b0 += nbmax) {
    const int nb = ncol - b0 < nbmax ? ncol - b0 : nbmax;
    const int N = 2 * w * w * nb;
    cudaError_t e;
    if (kind == GEMM_TC_BF16) {
      if constexpr (sizeof(S) == 4) {
        e = launch_mf_gather<float, uint16_t>(X, ldx, c0 + b0, nb, vec_win, nk, nv, nc, w, Zs, Kpad, nslices,
                                              (long)Npad * Kpad, s);
        if (e != cudaSuccess) return e;
        const long key = (long)N * 16 + npairs;
        auto it = plans.find(key);
        TcGemmPlan* plan = nullptr;
        if (it == plans.end()) {
          std::string m2;
          if (tc_gemm_plan_create(&plan, Vs, Mpad, Kpad, (long)Mpad * Kpad, nslices, Zs, Npad, (long)Npad * Kpad,
                                  nslices, reinterpret_cast<float*>(Tm), Npad, npairs, pa, pb, &m2) != WTB_OK) {
            if (msg) *msg = m2;
            return cudaErrorInvalidValue;
          }
          tc_gemm_set_valid(plan, nk, N);
          plans[key] = plan;
        } else {
          plan = it->second;
        }
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
        e = launch_mf_scatter<float, float>(reinterpret_cast<const float*>(Tm), Npad, X, ldx, vec_win, dE, nk, nv, nc,
                                            w, nb, Y, ldy, c0 + b0, s);
        if (e != cudaSuccess) return e;
      } else {
        return cudaErrorInvalidValue;
      }
    } else {
      e = launch_mf_gather<S, S>(X, ldx, c0 + b0, nb, vec_win, nk, nv, nc, w, Zr, Kpad, 1, 0, s);
      if (e != cudaSuccess) return e;
      cudaEvent_t ea = nullptr, eb = nullptr;
      const bool profiled = prof && prof->on && !this->capturing;
      if (profiled) {
        cudaEventCreate(&ea);
        cudaEventCreate(&eb);
        cudaEventRecord(ea, s);
      }
      e = launch_simt_gemm_tn<S>(Vr, Kpad, Zr, Kpad, reinterpret_cast<S*>(Tm), Npad, nk, N, Kpad, s);
      if (e != cudaSuccess) return e;
      if (profiled) {
        cudaEventRecord(eb, s);
        prof->pending.emplace_back(ea, eb);
        prof->launches += 1;
        prof->flops += 2.0 * nk * (double)N * nk;
        prof->bytes += sizeof(S) * ((double)nk * nk + (double)N * nk + (double)nk * N);
      }
      e = launch_mf_scatter<S, S>(reinterpret_cast<const S*>(Tm), Npad, X, ldx, vec_win, dE, nk, nv, nc, w, nb, Y, ldy,
                                  c0 + b0, s);
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
    const long key = (long)N * 16 + np;
    auto it = plans.find(key);
    if (it == plans.end()) {
      std::string m2;
      if (tc_gemm_plan_create(&plan, Vs, Mpad, Kpad, (long)Mpad * Kpad, nslices, Zs, Npad, (long)Npad * Kpad, nslices,
                              reinterpret_cast<float*>(Tm), Npad, np, pa, pb, &m2) != WTB_OK)
        return cudaErrorInvalidValue;
      tc_gemm_set_valid(plan, nk, N);
      plans[key] = plan;
    } else {
      plan = it->second;
    }
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
      e = launch_simt_gemm_tn<S>(Vr, Kpad, Zr, Kpad, reinterpret_cast<S*>(Tm), Npad, nk, N, Kpad, s);
    if (e != cudaSuccess) return e;
    cudaEventRecord(eb, s);
    prof->pending.emplace_back(ea, eb);
    prof->launches += 1;
    if (plan) {
      prof->flops += 2.0 * nk * (double)N * nk * np;
      prof->bytes += 2.0 * nslices * ((double)nk * nk + (double)N * nk) + 4.0 * nk * (double)N;
    } else {
      prof->flops += 2.0 * nk * (double)N * nk;
      prof->bytes += sizeof(S) * ((double)nk * nk + (double)N * nk + (double)nk * N);
    }
  }
  return cudaSuccess;
}

template <class S>
cudaError_t MatFreeOperator<S>::contract(const cplx<S>* X, int ldx, int ncol, cudaStream_t s) {
  if (ncol > nbmax) return cudaErrorInvalidValue;
  const int N = 2 * w * w * ncol;
  if (kind == GEMM_TC_BF16) {
    if constexpr (sizeof(S) == 4) {
      cudaError_t e = launch_mf_gather<float, uint16_t>(X, ldx, 0, ncol, vec_win, nk, nv, nc, w, Zs, Kpad, nslices,
                                                        (long)Npad * Kpad, s);
      if (e != cudaSuccess) return e;
      const long key = (long)N * 16 + npairs;
      TcGemmPlan* plan = nullptr;
      auto it = plans.find(key);
      if (it == plans.end()) {
        std::string m2;
        if (tc_gemm_plan_create(&plan, Vs, Mpad, Kpad, (long)Mpad * Kpad, nslices, Zs, Npad, (long)Npad * Kpad,
                                nslices, reinterpret_cast<float*>(Tm), Npad, npairs, pa, pb, &m2) != WTB_OK) {
          if (msg) *msg = m2;
          return cudaErrorInvalidValue;
        }
        tc_gemm_set_valid(plan, nk, N);
        plans[key] = plan;
      } else {
        plan = it->second;
      }
      return tc_gemm_run(plan, st, s);
    } else {
      return cudaErrorInvalidValue;
    }
  }
  cudaError_t e = launch_mf_gather<S, S>(X, ldx, 0, ncol, vec_win, nk, nv, nc, w, Zr, Kpad, 1, 0, s);
  if (e != cudaSuccess) return e;
  return launch_simt_gemm_tn<S>(Vr, Kpad, Zr, Kpad, reinterpret_cast<S*>(Tm), Npad, nk, N, Kpad, s);
}

template struct MatFreeOperator<float>;
template struct MatFreeOperator<double>;

namespace {

struct Small {
  zd *M, *G, *B, *Gp, *U, *Y, *C, *T;
  double *lam, *theta, *dinv;
  int* keep;
};

// Rayleigh-Ritz on the basis Sb (dim x nb, ld) with ASb = H Sb: returns C (nb x m) and theta (m).
// Orthonormalisation: Cholesky of the scaled Gram matrix in [X W P] order with deflation (directions whose
// residual diagonal falls below tau are dropped; the r kept ones come first in B); the projected r x r
// problem B^H G B is solved
// by the tridiagonal route (small_eig.cuh).  The small problems run in precision S, or FP64 for
// small_in_fp64.  A missing Ritz pair (r < m) has theta = 1e30 and a zero column in C.
template <class S>
int rayleigh_ritz(const cplx<S>* Sb, const cplx<S>* ASb, int ld, int nb, int m, int dim, double tau, Small& sm,
                  double* partial, int npart, DevStatus* st, cudaStream_t s, std::string* msg,
                  bool small_in_fp64) {
  (void)st;
  CK(launch_gram<S>(Sb, ld, nb, Sb, ld, nb, dim, sm.M, partial, npart, s));
  CK(launch_gram<S>(Sb, ld, nb, ASb, ld, nb, dim, sm.G, partial, npart, s));
  if (small_in_fp64)
    CK(launch_pchol_basis<double>(sm.M, nb, nb, tau, sm.B, nb, sm.keep, s));
  else
    CK(launch_pchol_basis<S>(sm.M, nb, nb, tau, sm.B, nb, sm.keep, s));
  // the projected matrix B^H G B stays FP64 (its rounding would mix near-degenerate Ritz vectors); the basis
  // combination C = B Y may run in FP32 when the iteration does
  const bool f32 = !small_in_fp64 && sizeof(S) == 4;
  CK(launch_small_gemm(sm.G, nb, 0, sm.B, nb, sm.T, nb, nb, nb, nb, s, false));
  CK(launch_small_gemm(sm.B, nb, 1, sm.T, nb, sm.Gp, nb, nb, nb, nb, s, false));
  if (small_in_fp64)
    CK(launch_heev_small<double>(sm.Gp, nb, sm.keep, nb, m, sm.theta, sm.Y, nb, s));
  else
    CK(launch_heev_small<S>(sm.Gp, nb, sm.keep, nb, m, sm.theta, sm.Y, nb, s));
  CK(launch_small_gemm(sm.B, nb, 0, sm.Y, nb, sm.C, m, nb, m, nb, s, f32));
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
  int it, total_it, nconv, stop, converged, restore, save, failed, best_it, pad[3];
  double maxrel, best_maxrel, saved_rel, tol;
};

__global__ void lob_ctl_reset_kernel(LobCtl* c, double tol, int keep_total) {
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
  c->maxrel = 1e300;
  c->best_maxrel = 1e300;
  c->saved_rel = 1e300;
  c->tol = tol;
}

// One warp.  rel_j = ||r_j|| / |theta_j|; converged columns leave the active set (soft locking).
//  - breakdown guard: near the operator's rounding floor the running AX drifts from H X and LOBPCG can lose
//    consistency (Ritz values falling far below the spectrum): the block with the lowest residual of the
//    phase is kept (save), and a residual 10x above it after reaching 100 x tol restores it and ends the
//    phase (restore);
//  - stagnation guard (reduced precision): residuals within 100 x tol that have not improved by 10% over
//    15 iterations are at the operator's rounding floor; the FP64 Rayleigh-Ritz takes over;
//  - the iteration cap, a non-finite residual and a device status word end the loop as well.
// Monitor lines follow the reference's MyEPSMonitor (src/module_slepc_solver.F90:101-116).
__global__ void lob_control_kernel(LobCtl* c, const double* __restrict__ norms2, const double* __restrict__ theta,
                                   int m, int nev, int maxit, int reduced, int* __restrict__ active,
                                   const DevStatus* __restrict__ st, cudaGraphConditionalHandle h, int in_graph,
                                   int monitor) {
  const int lane = threadIdx.x;
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
  if (lane != 0) return;
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
    } else if (c->saved_rel <= 100.0 * tol && mr > 10.0 * c->saved_rel) {
      c->restore = 1;
      c->converged = 1;
      stop = 1;
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
    printf("WTB-EPS %5d EPS pair=%4d value (error) %15.8E (%10.3E) max %10.3E\n", c->total_it, nc + 1, theta[f],
           sqrt(fmax(norms2[f], 0.0)) / fmax(fabs(theta[f]), 1e-12), mr);
  }
  if (!stop) {
    c->it += 1;
    c->total_it += 1;
  }
  c->stop = stop;
  if (in_graph) cudaGraphSetConditional(h, stop ? 0u : 1u);
}

// dst[:, 0:ncol] = src[:, 0:ncol] when *flag is set
template <class S>
__global__ void cond_copy_kernel(const int* __restrict__ flag, const cplx<S>* __restrict__ src, int lds,
                                 cplx<S>* __restrict__ dst, int ldd, int ncol, int nrow) {
  if (!*flag) return;
  const long n = (long)nrow * ncol;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long r = e / ncol;
    const int c = (int)(e % ncol);
    dst[r * ldd + c] = src[r * lds + c];
  }
}

// In place: X <- [X W P] C and P <- [W P] C[m:3m, :] for the basis and for its image under H.  A CTA stages
// kUpdRows rows of the block in shared memory (so the in-place writes cannot overtake reads), then threads
// (row, group of four output columns) form their outputs from the staged row and C.
constexpr int kUpdRows = 32;
template <class S>
__global__ void __launch_bounds__(256) lob_update_kernel(cplx<S>* __restrict__ Sb, cplx<S>* __restrict__ ASb, int ld,
                                                         int m, const zd* __restrict__ C, int dim) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nb = 3 * m;
  cplx<S>* Cs = reinterpret_cast<cplx<S>*>(smem_raw);  // [3m][m]
  cplx<S>* Rs = Cs + nb * m;                           // [kUpdRows][3m]
  for (int e = threadIdx.x; e < nb * m; e += blockDim.x) Cs[e] = mk<S>((S)C[e].re, (S)C[e].im);
  const int ngrp = (m + 3) >> 2;       // groups of 4 output columns
  const int items = kUpdRows * ngrp;   // (row, group) pairs per pass
  for (long r0 = (long)blockIdx.x * kUpdRows; r0 < dim; r0 += (long)gridDim.x * kUpdRows) {
    const int nr = (int)min((long)kUpdRows, dim - r0);
    for (int which = 0; which < 2; ++which) {
      cplx<S>* base = (which ? ASb : Sb) + r0 * ld;
      __syncthreads();
      for (int e = threadIdx.x; e < nr * nb; e += blockDim.x) {
        const int rr = e / nb, c = e - rr * nb;
        Rs[rr * nb + c] = base[(size_t)rr * ld + c];
      }
      __syncthreads();
      for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int rr = it / ngrp, g = it - rr * ngrp;
        if (rr >= nr) continue;
        const int j0 = g * 4;
        cplx<S> x[4], pn[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) x[q] = pn[q] = mk<S>(0, 0);
        const cplx<S>* row = Rs + rr * nb;
        for (int i = 0; i < nb; ++i) {
          const cplx<S> ri = row[i];
          const cplx<S>* crow = Cs + i * m + j0;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (j0 + q < m) {
              cfma(x[q], ri, crow[q]);
              if (i >= m) cfma(pn[q], ri, crow[q]);
            }
          }
        }
        cplx<S>* out = base + (size_t)rr * ld;
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (j0 + q < m) {
            out[j0 + q] = x[q];
            out[2 * m + j0 + q] = pn[q];
          }
      }
    }
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
int lobpcg_solve(Operator<S>& op, const double* diag, int dim, int nev, int m, double tol, int maxit, Workspace& ws,
                 DevStatus* st, cudaStream_t s, std::vector<double>* E, zd* Xout, SolveStats* stats,
                 std::string* msg, double tol_refine) {
  if (m < nev) m = nev;
  if (m > dim) m = dim;
  if (nev < 1 || nev > dim) {
    if (msg) *msg = "nev must be between 1 and the BSE dimension";
    return WTB_EBADARG;
  }
  const int ld = 3 * m;
  const int nb = 3 * m;
  if (nb > (sizeof(S) == 4 ? 96 : 78) || m > 32) {
    if (msg) *msg = "eigensolver block too large (3*block must be <= 96 in FP32, <= 78 in FP64)";
    return WTB_EBADARG;
  }
  cudaError_t err = cudaSuccess;
  cplx<S>* Sb = ws.get<cplx<S>>("lob_S", (size_t)dim * ld, &err, true);
  cplx<S>* ASb = ws.get<cplx<S>>("lob_AS", (size_t)dim * ld, &err, true);
  cplx<S>* Xbest = ws.get<cplx<S>>("lob_Xbest", (size_t)dim * m, &err);
  Small sm;
  const size_t nn = (size_t)nb * nb;
  sm.M = ws.get<zd>("lob_M", nn, &err);
  sm.G = ws.get<zd>("lob_G", nn, &err);
  sm.B = ws.get<zd>("lob_B", nn, &err);
  sm.Gp = ws.get<zd>("lob_Gp", nn, &err);
  sm.U = nullptr;
  sm.Y = ws.get<zd>("lob_Y", nn, &err);
  sm.C = ws.get<zd>("lob_C", nn, &err);
  sm.T = ws.get<zd>("lob_T", nn, &err);
  sm.lam = nullptr;
  sm.dinv = nullptr;
  sm.theta = ws.get<double>("lob_theta", nb, &err);
  sm.keep = ws.get<int>("lob_keep", nb, &err);
  // partial sums of the tall-skinny reductions: about 128 rows per part, at most two per SM
  const int npart = std::max(1, std::min(304, (dim + 127) / 128));
  double* partial = ws.get<double>("lob_partial", (size_t)npart * nn * 2, &err);
  double* norms2 = ws.get<double>("lob_norms2", 32, &err);
  int* active = ws.get<int>("lob_active", 32, &err);
  int* idx = ws.get<int>("lob_idx", 65 * 128, &err);
  double* cand = ws.get<double>("lob_cand", 65 * 128, &err);
  double* th_dev = ws.get<double>("lob_thcur", nb, &err);
  LobCtl* ctl = ws.get<LobCtl>("lob_ctl", 1, &err);
  zd* X64 = ws.get<zd>("fin_X", (size_t)dim * 2 * m, &err);
  zd* T64 = ws.get<zd>("fin_T", (size_t)dim * m, &err);
  if (err != cudaSuccess) {
    if (msg) *msg = std::string("device allocation failed: ") + cudaGetErrorString(err);
    return WTB_ENOMEM;
  }
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
  const bool stream_mode = std::getenv("WTB_SOLVER_STREAM") != nullptr;
  const size_t upd_smem = (size_t)(nb * m + kUpdRows * nb) * sizeof(cplx<S>);
  const int upd_grid = std::max(1, std::min(152 * 8, (dim + kUpdRows - 1) / kUpdRows));
  const unsigned cp_grid = (unsigned)std::max(1, std::min(152 * 4, (int)(((long)dim * m + 255) / 256)));

  // the pieces of one iteration, as stream launches (captured below)
  auto rr_and_update = [&]() -> int {
    int r = rayleigh_ritz<S>(Sb, ASb, ld, nb, m, dim, tau, sm, partial, npart, st, s, msg, false);
    if (r) return r;
    CK(raise_smem_limit(reinterpret_cast<const void*>(lob_update_kernel<S>), upd_smem));
    lob_update_kernel<S><<<upd_grid, 256, upd_smem, s>>>(Sb, ASb, ld, m, sm.C, dim);
    ++g_launch_count;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(th_dev, sm.theta, sizeof(double) * m, cudaMemcpyDeviceToDevice, s));
    return WTB_OK;
  };
  auto check_and_decide = [&](cudaGraphConditionalHandle h) -> int {
    CK(launch_residual<S>(AX, ld, X, ld, th_dev, m, dim, W, ld, partial, npart, norms2, s));
    lob_control_kernel<<<1, 32, 0, s>>>(ctl, norms2, th_dev, m, nev, maxit, reduced ? 1 : 0, active, st, h,
                                        stream_mode ? 0 : 1, monitor ? 1 : 0);
    ++g_launch_count;
    CK(cudaGetLastError());
    cond_copy_kernel<S><<<cp_grid, 256, 0, s>>>(&ctl->save, X, ld, Xbest, m, m, dim);
    ++g_launch_count;
    CK(cudaGetLastError());
    return WTB_OK;
  };
  auto restart_from_x = [&](cudaGraphConditionalHandle h) -> int {
    CK(cudaMemset2DAsync(W, sizeof(cplx<S>) * ld, 0, sizeof(cplx<S>) * 2 * m, dim, s));
    CK(cudaMemset2DAsync(AW, sizeof(cplx<S>) * ld, 0, sizeof(cplx<S>) * 2 * m, dim, s));
    CK(op.apply(X, ld, 0, m, AX, ld, s));
    int r = rr_and_update();
    if (r) return r;
    return check_and_decide(h);
  };
  auto iteration = [&](cudaGraphConditionalHandle h) -> int {
    CK(launch_precond<S>(W, ld, diag, th_dev, active, m, dim, s));
    // W <- W - X (X^H W);  P <- P - X (X^H P), AP <- AP - AX (X^H P)
    CK(launch_gram<S>(X, ld, m, W, ld, m, dim, sm.T, partial, npart, s));
    CK(launch_update<S>(X, ld, m, sm.T, m, m, dim, W, ld, -1.0, 1.0, s));
    CK(op.apply(W, ld, 0, m, AW, ld, s));
    CK(launch_gram<S>(X, ld, m, P, ld, m, dim, sm.T, partial, npart, s));
    CK(launch_update<S>(X, ld, m, sm.T, m, m, dim, P, ld, -1.0, 1.0, s));
    CK(launch_update<S>(AX, ld, m, sm.T, m, m, dim, AP, ld, -1.0, 1.0, s));
    int r = rr_and_update();
    if (r) return r;
    return check_and_decide(h);
  };
  // final FP64 Rayleigh-Ritz on a fresh application of the operator's most accurate arithmetic (the
  // iteration's AX is a running linear combination of cheaper applications)
  std::function<int()> final_step = [&]() -> int {
    cond_copy_kernel<S><<<cp_grid, 256, 0, s>>>(&ctl->restore, Xbest, m, X, ld, m, dim);
    ++g_launch_count;
    op.begin_refine();
    op.set_final(true);
    const cudaError_t fe = op.apply(X, ld, 0, m, AX, ld, s);
    op.set_final(false);
    CK(fe);
    CK((launch_convert_cols<S, double>(X, ld, X64, 2 * m, m, dim, s)));
    CK((launch_convert_cols<S, double>(AX, ld, X64 + m, 2 * m, m, dim, s)));
    int r = rayleigh_ritz<double>(X64, X64 + m, 2 * m, m, m, dim, 1e-13, sm, partial, npart, st, s, msg, true);
    if (r) return r;
    // Xout = X64 C[:, :nev]; residual = (AX64 C - Xout theta)
    CK(launch_update<double>(X64, 2 * m, m, sm.C, m, nev, dim, Xout, nev, 1.0, 0.0, s));
    CK(launch_update<double>(X64 + m, 2 * m, m, sm.C, m, nev, dim, T64, nev, 1.0, 0.0, s));
    CK(launch_residual<double>(T64, nev, Xout, nev, sm.theta, nev, dim, T64, nev, partial, npart, norms2, s));
    return WTB_OK;
  };

  int rc = WTB_OK;
  long long body_launches[2] = {0, 0};
  if (stream_mode) {
    auto stopped = [&](bool* stop) -> int {
      int h = 0;
      CK(cudaMemcpyAsync(&h, &ctl->stop, sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      *stop = h != 0;
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
    lob_ctl_reset_kernel<<<1, 1, 0, s>>>(ctl, tol, 0);
    ++g_launch_count;
    CK(cudaMemset2DAsync(Sb, sizeof(cplx<S>) * ld, 0, sizeof(cplx<S>) * ld, dim, s));
    CK(launch_select_lowest(diag, dim, m, idx, cand, s));
    CK(launch_init_guess<S>(X, ld, dim, m, idx + 64 * m, 12345u, s));
    if ((rc = restart_from_x(0))) return rc;
    if ((rc = run_loop())) return rc;
    if (two_phase) {
      op.begin_refine();
      cond_copy_kernel<S><<<cp_grid, 256, 0, s>>>(&ctl->restore, Xbest, m, X, ld, m, dim);
      ++g_launch_count;
      lob_ctl_reset_kernel<<<1, 1, 0, s>>>(ctl, tol_refine, 1);
      ++g_launch_count;
      if ((rc = restart_from_x(0))) return rc;
      if ((rc = run_loop())) return rc;
    }
    if ((rc = final_step())) return rc;
  } else {
  // the graph of this solve is reused when nothing it was captured with has changed
  std::vector<uint64_t> sig = {(uint64_t)dim, (uint64_t)nev, (uint64_t)m, (uint64_t)maxit, (uint64_t)sizeof(S),
                               (uint64_t)(uintptr_t)diag, (uint64_t)(uintptr_t)Xout, (uint64_t)(uintptr_t)st,
                               (uint64_t)(uintptr_t)s, (uint64_t)(uintptr_t)Sb, (uint64_t)(uintptr_t)ASb,
                               (uint64_t)(uintptr_t)Xbest, (uint64_t)(uintptr_t)sm.M, (uint64_t)(uintptr_t)sm.G,
                               (uint64_t)(uintptr_t)sm.B, (uint64_t)(uintptr_t)sm.Gp, (uint64_t)(uintptr_t)sm.Y,
                               (uint64_t)(uintptr_t)sm.C, (uint64_t)(uintptr_t)sm.T, (uint64_t)(uintptr_t)sm.theta,
                               (uint64_t)(uintptr_t)sm.keep, (uint64_t)(uintptr_t)partial, (uint64_t)(uintptr_t)norms2,
                               (uint64_t)(uintptr_t)active, (uint64_t)(uintptr_t)idx, (uint64_t)(uintptr_t)cand,
                               (uint64_t)(uintptr_t)th_dev, (uint64_t)(uintptr_t)ctl, (uint64_t)(uintptr_t)X64,
                               (uint64_t)(uintptr_t)T64, (uint64_t)monitor};
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
  if (ws.graph_exec && ws.graph_key == key) {
    body_launches[0] = ws.graph_body_launches[0];
    body_launches[1] = ws.graph_body_launches[1];
    g_launch_count += ws.graph_launches;  // one pass of every captured kernel; the bodies' repeats are added below
    if (cudaGraphLaunch(ws.graph_exec, s) != cudaSuccess) {
      if (msg) *msg = "graph launch failed";
      return WTB_ECUDA;
    }
  } else {
  ws.drop_graph();
  const long long captured0 = g_launch_count.load();
  cudaGraph_t G = nullptr;
  cudaGraphExec_t GX = nullptr;
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
    rc = segment(G, {}, &tail, [&]() -> int {
      lob_ctl_reset_kernel<<<1, 1, 0, s>>>(ctl, tol, 0);
      ++g_launch_count;
      CK(cudaMemset2DAsync(Sb, sizeof(cplx<S>) * ld, 0, sizeof(cplx<S>) * ld, dim, s));
      CK(launch_select_lowest(diag, dim, m, idx, cand, s));
      CK(launch_init_guess<S>(X, ld, dim, m, idx + 64 * m, 12345u, s));
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
        cond_copy_kernel<S><<<cp_grid, 256, 0, s>>>(&ctl->restore, Xbest, m, X, ld, m, dim);
        ++g_launch_count;
        lob_ctl_reset_kernel<<<1, 1, 0, s>>>(ctl, tol_refine, 1);
        ++g_launch_count;
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
  std::vector<double> th(nev), th_it(nev), nrm(nev);
  LobCtl hc;
  CK(cudaMemcpyAsync(th.data(), sm.theta, sizeof(double) * nev, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(th_it.data(), th_dev, sizeof(double) * nev, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(nrm.data(), norms2, sizeof(double) * nev, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&hc, ctl, sizeof(hc), cudaMemcpyDeviceToHost, s));
  DevStatus hst;
  CK(cudaMemcpyAsync(&hst, st, sizeof(hst), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (!stream_mode) {
    const int it2 = two_phase ? hc.it : 0, it1 = hc.total_it - it2;
    g_launch_count += body_launches[0] * (it1 - 1) + (two_phase ? body_launches[1] * (it2 - 1) : 0);
  }
  if (stats) {
    stats->iterations = hc.total_it;
    stats->launches = 0;
    stats->matvec_columns = (long)m * (hc.total_it + (two_phase ? 3 : 2));
  }
  if (hst.code) {
    if (msg) *msg = "device status " + std::to_string(hst.code) + " during the eigensolve";
    return hst.code >= 400 && hst.code < 500 ? WTB_ETIMEOUT : WTB_ENOCONV;
  }
  if (hc.failed == WTB_ENAN) {
    if (msg) *msg = "non-finite residual in the eigensolve";
    return WTB_ENAN;
  }
  double maxrel = 0.0, shift = 0.0;
  for (int j = 0; j < nev; ++j) {
    const double rel = std::sqrt(std::max(nrm[j], 0.0)) / std::max(std::fabs(th[j]), 1e-12);
    if (!std::isfinite(rel) || !std::isfinite(th[j])) {
      if (msg) *msg = "non-finite eigenpair after the final Rayleigh-Ritz";
      return WTB_ENAN;
    }
    maxrel = std::max(maxrel, rel);
    shift = std::max(shift, std::fabs(th[j] - th_it[j]));
  }
  *E = th;
  if (stats) {
    stats->max_rel_residual = maxrel;
    stats->refine_shift_max = shift;
  }
  if (!hc.converged) {
    if (msg) *msg = "eigensolver did not converge in " + std::to_string(maxit) + " iterations";
    return WTB_ENOCONV;
  }
  return WTB_OK;
}

template int lobpcg_solve<float>(Operator<float>&, const double*, int, int, int, double, int, Workspace&, DevStatus*,
                                 cudaStream_t, std::vector<double>*, zd*, SolveStats*, std::string*, double);
template int lobpcg_solve<double>(Operator<double>&, const double*, int, int, int, double, int, Workspace&,
                                  DevStatus*, cudaStream_t, std::vector<double>*, zd*, SolveStats*, std::string*,
                                  double);

}  // namespace wtb
