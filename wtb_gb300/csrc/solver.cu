// Block eigensolver for the lowest excitons and the matrix-free operator driver.
//
// LOBPCG (Knyazev's locally optimal block preconditioned CG) with
//   - the diagonal (transition-energy) preconditioner |diag(H) - theta|^-1, floored;
//   - soft locking: converged columns keep their place in X but get no new search direction;
//   - orthonormalisation of the basis [X W P] by pivoted Cholesky of its scaled Gram matrix (directions
//     whose residual norm falls below tau are dropped) followed by Rayleigh-Ritz on the kept directions,
//     whose small eigenproblem is solved by Householder tridiagonalisation, bisection and inverse
//     iteration on one CTA (small_eig.cuh);
//   - all projected (3m x 3m) matrices kept in complex(8) on the device.
// The iteration vectors are in precision S.  In every mode the last step is an FP64 Rayleigh-Ritz on
// the final block with a freshly applied operator: FP64 Gram matrices, FP64 eigen-decomposition, FP64
// residual norms.  It replaces slepc_solver (src/module_slepc_solver.F90:12-97: Krylov-Schur,
// EPS_SMALLEST_MAGNITUDE, tol 1e-8, 200 iterations); for the positive BSE spectra of this path the
// smallest-magnitude and smallest-algebraic eigenvalues coincide.
#include <cmath>
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
        const bool profiled = prof && prof->on && !final_apply;
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
      if (prof && prof->on) {
        cudaEventCreate(&ea);
        cudaEventCreate(&eb);
        cudaEventRecord(ea, s);
      }
      e = launch_simt_gemm_tn<S>(Vr, Kpad, Zr, Kpad, reinterpret_cast<S*>(Tm), Npad, nk, N, Kpad, s);
      if (e != cudaSuccess) return e;
      if (prof && prof->on) {
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
// Orthonormalisation: pivoted Cholesky of the scaled Gram matrix (directions whose residual diagonal falls
// below tau are dropped; the r kept ones come first in B); the projected r x r problem B^H G B is solved
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
  CK(launch_small_gemm(sm.G, nb, 0, sm.B, nb, sm.T, nb, nb, nb, nb, s));
  CK(launch_small_gemm(sm.B, nb, 1, sm.T, nb, sm.Gp, nb, nb, nb, nb, s));
  if (small_in_fp64)
    CK(launch_heev_small<double>(sm.Gp, nb, sm.keep, nb, m, sm.theta, sm.Y, nb, s));
  else
    CK(launch_heev_small<S>(sm.Gp, nb, sm.keep, nb, m, sm.theta, sm.Y, nb, s));
  CK(launch_small_gemm(sm.B, nb, 0, sm.Y, nb, sm.C, m, nb, m, nb, s));
  return WTB_OK;
}

}  // namespace

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
  const int maxnb = 3 * m;
  if (maxnb > (sizeof(S) == 4 ? 96 : 78)) {
    if (msg) *msg = "eigensolver block too large (3*block must be <= 96 in FP32, <= 78 in FP64)";
    return WTB_EBADARG;
  }
  cudaError_t err = cudaSuccess;
  auto chk = [&](void) { return err == cudaSuccess; };
  cplx<S>* Sb[2];
  cplx<S>* ASb[2];
  Sb[0] = ws.get<cplx<S>>("lob_S0", (size_t)dim * ld, &err, true);
  if (!chk()) goto oom;
  Sb[1] = ws.get<cplx<S>>("lob_S1", (size_t)dim * ld, &err, true);
  if (!chk()) goto oom;
  ASb[0] = ws.get<cplx<S>>("lob_AS0", (size_t)dim * ld, &err, true);
  if (!chk()) goto oom;
  ASb[1] = ws.get<cplx<S>>("lob_AS1", (size_t)dim * ld, &err, true);
  if (!chk()) goto oom;
  {
    Small sm;
    const size_t nn = (size_t)maxnb * maxnb;
    sm.M = ws.get<zd>("lob_M", nn, &err);
    sm.G = ws.get<zd>("lob_G", nn, &err);
    sm.B = ws.get<zd>("lob_B", nn, &err);
    sm.Gp = ws.get<zd>("lob_Gp", nn, &err);
    sm.U = ws.get<zd>("lob_U", nn, &err);
    sm.Y = ws.get<zd>("lob_Y", nn, &err);
    sm.C = ws.get<zd>("lob_C", nn, &err);
    sm.T = ws.get<zd>("lob_T", nn, &err);
    sm.lam = ws.get<double>("lob_lam", maxnb, &err);
    sm.theta = ws.get<double>("lob_theta", maxnb, &err);
    sm.dinv = ws.get<double>("lob_dinv", maxnb, &err);
    sm.keep = ws.get<int>("lob_keep", maxnb, &err);
    // partial sums of the tall-skinny reductions: about 128 rows per part, at most two per SM
    const int npart = std::max(1, std::min(304, (dim + 127) / 128));
    double* partial = ws.get<double>("lob_partial", (size_t)npart * nn * 2, &err);
    double* norms2 = ws.get<double>("lob_norms2", 32, &err);
    int* active = ws.get<int>("lob_active", 32, &err);
    int* idx = ws.get<int>("lob_idx", 65 * 128, &err);
    double* cand = ws.get<double>("lob_cand", 65 * 128, &err);
    double* th_dev = ws.get<double>("lob_thcur", maxnb, &err);
    if (!chk()) goto oom;
    // SVQB keeps a direction of the scaled Gram matrix only if its eigenvalue exceeds tau: a kept
    // direction's Rayleigh quotient carries the operator's rounding divided by sqrt(eigenvalue), so tau
    // sits well above the FP32 noise (~1e-6 on the Gram entries) and just above FP64's
    const double tau = sizeof(S) == 4 ? 1e-4 : 1e-13;
    std::vector<double> h_theta(maxnb), h_norm(32);
    std::vector<int> h_active(32, 1);
    // start block: unit vectors at the m lowest transition energies (+ small deterministic noise)
    CK(launch_select_lowest(diag, dim, m, idx, cand, s));
    CK(launch_init_guess<S>(Sb[0], ld, dim, m, idx + 64 * m, 12345u, s));
    CK(op.apply(Sb[0], ld, 0, m, ASb[0], ld, s));
    int r = rayleigh_ritz<S>(Sb[0], ASb[0], ld, m, m, dim, tau, sm, partial, npart, st, s, msg, false);
    if (r) return r;
    CK(launch_update<S>(Sb[0], ld, m, sm.C, m, m, dim, Sb[1], ld, 1.0, 0.0, s));
    CK(launch_update<S>(ASb[0], ld, m, sm.C, m, m, dim, ASb[1], ld, 1.0, 0.0, s));
    CK(cudaMemcpyAsync(th_dev, sm.theta, sizeof(double) * m, cudaMemcpyDeviceToDevice, s));
    int cur = 1;
    bool have_p = false;
    bool converged = false;
    int it = 0;
    // per-iteration monitor in the format of the reference's MyEPSMonitor
    // (src/module_slepc_solver.F90:101-116), enabled by the WTB_EPS_MONITOR environment variable
    const bool monitor = std::getenv("WTB_EPS_MONITOR") != nullptr;
    // stagnation guard for reduced-precision iterations: once the wanted residuals sit within
    // 100 x tol and have not improved by 10% over 15 iterations, the operator's rounding floor has been
    // reached and the FP64 Rayleigh-Ritz below takes over
    double best_maxrel = 1e300;
    int best_it = 0;
    // breakdown guard: near the operator's rounding floor the running AX drifts from H X and LOBPCG can
    // lose consistency (Ritz values falling far below the spectrum).  The block with the lowest residual of
    // the current phase is kept; a residual that grows 10x past it after reaching 100 x tol restores it.
    cplx<S>* Xbest = ws.get<cplx<S>>("lob_Xbest", (size_t)dim * m, &err);
    if (!chk()) goto oom;
    double saved_rel = 1e300;
    int restarts = 0;
    for (; it < maxit; ++it) {
      cplx<S>* X = Sb[cur];
      cplx<S>* AX = ASb[cur];
      cplx<S>* W = X + m;
      cplx<S>* AW = AX + m;
      CK(launch_residual<S>(AX, ld, X, ld, th_dev, m, dim, W, ld, partial, npart, norms2, s));
      CK(cudaMemcpyAsync(h_norm.data(), norms2, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(h_theta.data(), th_dev, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      DevStatus hst;
      CK(cudaMemcpy(&hst, st, sizeof(hst), cudaMemcpyDeviceToHost));
      if (hst.code) {
        if (msg) *msg = "device status " + std::to_string(hst.code) + " during the eigensolve";
        return hst.code >= 400 && hst.code < 500 ? WTB_ETIMEOUT : WTB_ENOCONV;
      }
      int nconv = 0;
      double maxrel = 0.0;
      for (int j = 0; j < m; ++j) {
        const double rn = std::sqrt(std::max(h_norm[j], 0.0));
        if (!std::isfinite(rn) || !std::isfinite(h_theta[j])) {
          if (msg) *msg = "non-finite residual in the eigensolve";
          return WTB_ENAN;
        }
        const double rel = rn / std::max(std::fabs(h_theta[j]), 1e-12);
        const bool cj = rel <= tol;
        if (j < nev) {
          nconv += cj;
          maxrel = std::max(maxrel, rel);
        }
        h_active[j] = cj ? 0 : 1;
      }
      if (stats) stats->max_rel_residual = maxrel;
      if (monitor) {
        int first = 0;
        while (first < nev - 1 && h_active[first] == 0) ++first;
        std::fprintf(stderr, "WTB-EPS %5d EPS pair=%4d value (error) %15.8E (%10.3E) max %10.3E\n", it, nconv + 1,
                     h_theta[first], std::sqrt(std::max(h_norm[first], 0.0)) / std::max(std::fabs(h_theta[first]), 1e-12),
                     maxrel);
      }
      // restart from X alone: fresh AX, no search directions, Rayleigh-Ritz on X
      auto restart_from_x = [&]() -> int {
        CK(op.apply(X, ld, 0, m, AX, ld, s));
        have_p = false;
        best_maxrel = 1e300;
        best_it = it;
        int rr = rayleigh_ritz<S>(X, AX, ld, m, m, dim, tau, sm, partial, npart, st, s, msg, false);
        if (rr) return rr;
        const int nxt = cur ^ 1;
        CK(launch_update<S>(X, ld, m, sm.C, m, m, dim, Sb[nxt], ld, 1.0, 0.0, s));
        CK(launch_update<S>(AX, ld, m, sm.C, m, m, dim, ASb[nxt], ld, 1.0, 0.0, s));
        CK(cudaMemcpyAsync(th_dev, sm.theta, sizeof(double) * m, cudaMemcpyDeviceToDevice, s));
        cur = nxt;
        return WTB_OK;
      };
      if (maxrel < saved_rel) {
        saved_rel = maxrel;
        CK(launch_copy_cols<S>(X, ld, Xbest, m, m, dim, s));
      } else if (saved_rel <= 100.0 * tol && maxrel > 10.0 * saved_rel) {
        CK(launch_copy_cols<S>(Xbest, m, X, ld, m, dim, s));
        if (saved_rel <= tol || ++restarts > 2) {
          // the best block goes to the final Rayleigh-Ritz (which re-applies the operator)
          converged = saved_rel <= 100.0 * tol;
          break;
        }
        r = restart_from_x();
        if (r) return r;
        saved_rel = 1e300;
        continue;
      }
      if (nconv == nev) {
        if (tol_refine > 0.0 && tol_refine < tol && op.begin_refine()) {
          // second phase: the accurate operator; AX is recomputed and the search directions P (built
          // with the cheaper operator) are dropped
          tol = tol_refine;
          tol_refine = 0.0;
          r = restart_from_x();
          if (r) return r;
          saved_rel = 1e300;
          continue;
        }
        converged = true;
        break;
      }
      if (maxrel < 0.9 * best_maxrel) {
        best_maxrel = maxrel;
        best_it = it;
      } else if (sizeof(S) == 4 && maxrel <= 100.0 * tol && it - best_it >= 15) {
        converged = true;  // rounding floor of the reduced-precision operator
        break;
      }
      CK(cudaMemcpyAsync(active, h_active.data(), sizeof(int) * m, cudaMemcpyHostToDevice, s));
      CK(launch_precond<S>(W, ld, diag, th_dev, active, m, dim, s));
      // W <- W - X (X^H W)
      CK(launch_gram<S>(X, ld, m, W, ld, m, dim, sm.T, partial, npart, s));
      CK(launch_update<S>(X, ld, m, sm.T, m, m, dim, W, ld, -1.0, 1.0, s));
      CK(op.apply(W, ld, 0, m, AW, ld, s));
      if (have_p) {
        // P <- P - X (X^H P), AP <- AP - AX (X^H P): keeps the basis [X W P] away from dependence
        CK(launch_gram<S>(X, ld, m, X + 2 * m, ld, m, dim, sm.T, partial, npart, s));
        CK(launch_update<S>(X, ld, m, sm.T, m, m, dim, X + 2 * m, ld, -1.0, 1.0, s));
        CK(launch_update<S>(AX, ld, m, sm.T, m, m, dim, AX + 2 * m, ld, -1.0, 1.0, s));
      }
      const int nb = have_p ? 3 * m : 2 * m;
      r = rayleigh_ritz<S>(X, AX, ld, nb, m, dim, tau, sm, partial, npart, st, s, msg, false);
      if (r) return r;
      const int nxt = cur ^ 1;
      // new X, AX from the whole basis; new P, AP from its W and P parts
      CK(launch_update<S>(X, ld, nb, sm.C, m, m, dim, Sb[nxt], ld, 1.0, 0.0, s));
      CK(launch_update<S>(AX, ld, nb, sm.C, m, m, dim, ASb[nxt], ld, 1.0, 0.0, s));
      CK(launch_update<S>(X + m, ld, nb - m, sm.C + (size_t)m * m, m, m, dim, Sb[nxt] + 2 * m, ld, 1.0, 0.0, s));
      CK(launch_update<S>(AX + m, ld, nb - m, sm.C + (size_t)m * m, m, m, dim, ASb[nxt] + 2 * m, ld, 1.0, 0.0, s));
      CK(cudaMemcpyAsync(th_dev, sm.theta, sizeof(double) * m, cudaMemcpyDeviceToDevice, s));
      cur = nxt;
      have_p = true;
    }
    if (stats) {
      stats->iterations = it;
      stats->launches = 0;
    }
    // ---------------------------------------------------------------- final FP64 Rayleigh-Ritz
    {
      cplx<S>* X = Sb[cur];
      cplx<S>* AXs = ASb[cur];
      const int mm = m;
      zd* X64 = ws.get<zd>("fin_X", (size_t)dim * 2 * mm, &err);
      zd* T64 = ws.get<zd>("fin_T", (size_t)dim * mm, &err);
      if (!chk()) goto oom;
      // fresh H X in the operator's most accurate arithmetic (the iteration's AX is a running linear
      // combination of cheaper applications)
      op.begin_refine();
      op.set_final(true);
      const cudaError_t fe = op.apply(X, ld, 0, mm, AXs, ld, s);
      op.set_final(false);
      CK(fe);
      CK((launch_convert_cols<S, double>(X, ld, X64, 2 * mm, mm, dim, s)));
      CK((launch_convert_cols<S, double>(AXs, ld, X64 + mm, 2 * mm, mm, dim, s)));
      r = rayleigh_ritz<double>(X64, X64 + mm, 2 * mm, mm, mm, dim, 1e-13, sm, partial, npart, st, s, msg, true);
      if (r) return r;
      // Xout = X64 C[:, :nev]; residual = (AX64 C - Xout theta)
      CK(launch_update<double>(X64, 2 * mm, mm, sm.C, mm, nev, dim, Xout, nev, 1.0, 0.0, s));
      CK(launch_update<double>(X64 + mm, 2 * mm, mm, sm.C, mm, nev, dim, T64, nev, 1.0, 0.0, s));
      CK(launch_residual<double>(T64, nev, Xout, nev, sm.theta, nev, dim, T64, nev, partial, npart, norms2, s));
      std::vector<double> th(nev);
      CK(cudaMemcpyAsync(th.data(), sm.theta, sizeof(double) * nev, cudaMemcpyDeviceToHost, s));
      CK(cudaMemcpyAsync(h_norm.data(), norms2, sizeof(double) * nev, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      DevStatus hst;
      CK(cudaMemcpy(&hst, st, sizeof(hst), cudaMemcpyDeviceToHost));
      if (hst.code) {
        if (msg) *msg = "device status " + std::to_string(hst.code) + " in the final Rayleigh-Ritz";
        return hst.code >= 400 && hst.code < 500 ? WTB_ETIMEOUT : WTB_ENOCONV;
      }
      double maxrel = 0.0, shift = 0.0;
      for (int j = 0; j < nev; ++j) {
        const double rel = std::sqrt(std::max(h_norm[j], 0.0)) / std::max(std::fabs(th[j]), 1e-12);
        if (!std::isfinite(rel) || !std::isfinite(th[j])) {
          if (msg) *msg = "non-finite eigenpair after the final Rayleigh-Ritz";
          return WTB_ENAN;
        }
        maxrel = std::max(maxrel, rel);
        shift = std::max(shift, std::fabs(th[j] - h_theta[j]));
      }
      *E = th;
      if (stats) {
        stats->max_rel_residual = maxrel;
        stats->refine_shift_max = shift;
        stats->matvec_columns = op.matvec_columns;
      }
    }
    if (!converged) {
      if (msg) *msg = "eigensolver did not converge in " + std::to_string(maxit) + " iterations";
      return WTB_ENOCONV;
    }
    return WTB_OK;
  }
oom:
  if (msg) *msg = std::string("device allocation failed: ") + cudaGetErrorString(err);
  return WTB_ENOMEM;
}

template int lobpcg_solve<float>(Operator<float>&, const double*, int, int, int, double, int, Workspace&, DevStatus*,
                                 cudaStream_t, std::vector<double>*, zd*, SolveStats*, std::string*, double);
template int lobpcg_solve<double>(Operator<double>&, const double*, int, int, int, double, int, Workspace&,
                                  DevStatus*, cudaStream_t, std::vector<double>*, zd*, SolveStats*, std::string*,
                                  double);

}  // namespace wtb
