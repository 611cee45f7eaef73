// Adjoint (reverse-mode) gradients of the exciton path: d/dH(R) and d/dr0 of a loss that depends on the
// exciton energies E_n and the xx oscillator strengths f_n = |s_n|^2, s_n = sum_j A_jn hx_j.  The
// reference has no such code; the forward arithmetic it differentiates is that of eigsys
// (src/module_hamiltonian.F90:200-320), matrizelbse (src/module_bse.F90:24-83), v2drk
// (src/module_coulomb.F90:286-350), hlm/optsp (src/module_optics.F90:12-167) and dielbsev
// (src/module_bse.F90:201-245).
//
// With cotangents LE_n = dL/dE_n and Lf_n = dL/df_n:
//   dE_n      = A_n^H dH A_n                                              (Hellmann-Feynman)
//   d s_n     = -lambda_n^H dH A_n + A_n^T dh,   P (H - E_n) P lambda_n = P conj(hx)
//               (P projects out the computed excitons, so the shifted operator is positive definite;
//                solved by preconditioned CG with the matrix-free operator, the "adjoint solve")
//   y_n       = LE_n A_n - 2 Lf_n s_n lambda_n,   dL_H = Re sum_n y_n^H dH A_n
// dH is never formed.  Its dependence on the band vectors c, v goes through the same V(k,k') Z
// contractions as the matvec, applied to A_n and to y_n (T_A = V Z(A), T_y = V Z(y)):
//   cbar_kc[o] = sum_v,n,p conj(v_kv,p) (conj(y_kcv,n) T_A,n[k,o,p] + conj(A_kcv,n) T_y,n[k,o,p])
//   vbar_kv[p] = sum_c,n,o conj(c_kc,o) (same bracket)
// plus the transition-energy (diagonal) and the velocity-matrix-element terms.  Each k then back-propagates
// through its Hermitian eigen-decomposition (first-component-real gauge, lower-triangle completion as in
// ZHEEV('L')) to dL/dH(k), and a backward Fourier sum gives dL/dH(R); dL/dr0 = Re sum_n y_n^H H' A_n with
// H' the operator of dV/dr0.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "ctx.h"

namespace wtb {
namespace {

#define CKA(x)                                                                              \
  do {                                                                                      \
    cudaError_t e__ = (x);                                                                  \
    if (e__ != cudaSuccess) return ctx_set_err(c, WTB_ECUDA, std::string(#x) + ": " + cudaGetErrorString(e__)); \
  } while (0)
#define CKAR(x)           \
  do {                    \
    int r__ = (x);        \
    if (r__) return r__;  \
  } while (0)

__device__ __forceinline__ double rcart_adj(int r1, int r2, int r3, const double* rl, int a) {
  return __dadd_rn(__dadd_rn(__dmul_rn((double)r1, rl[a]), __dmul_rn((double)r2, rl[3 + a])),
                   __dmul_rn((double)r3, rl[6 + a]));
}

// the forward's single-precision-rounded phase k.R and Cartesian R_x
__device__ __forceinline__ double phase_adj(const int* rvec, int nR, int iR, const double* rl, const double* k) {
  const int r1 = rvec[iR], r2 = rvec[nR + iR], r3 = rvec[2 * nR + iR];
  const double phi = __dadd_rn(__dadd_rn(__dmul_rn(k[0], rcart_adj(r1, r2, r3, rl, 0)),
                                         __dmul_rn(k[1], rcart_adj(r1, r2, r3, rl, 1))),
                               __dmul_rn(k[2], rcart_adj(r1, r2, r3, rl, 2)));
  return (double)__double2float_rn(phi);
}

// s_n = sum_j A[j][n] hx[j]  (one CTA per n)
__global__ void adj_s_kernel(const zd* __restrict__ A, int nev, int dim, const zd* __restrict__ hx, zd* __restrict__ s) {
  __shared__ double red[2][256];
  const int n = blockIdx.x;
  zd acc = mk<double>(0, 0);
  for (int j = threadIdx.x; j < dim; j += blockDim.x) cfma(acc, A[(size_t)j * nev + n], hx[j]);
  red[0][threadIdx.x] = acc.re;
  red[1][threadIdx.x] = acc.im;
  __syncthreads();
  for (int off = 128; off > 0; off >>= 1) {
    if (threadIdx.x < off) {
      red[0][threadIdx.x] += red[0][threadIdx.x + off];
      red[1][threadIdx.x] += red[1][threadIdx.x + off];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) s[n] = mk<double>(red[0][0], red[1][0]);
}

template <class S>
__global__ void conj_bcast_kernel(const zd* __restrict__ h, int dim, int nev, cplx<S>* __restrict__ G) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)dim * nev) return;
  const zd v = h[e / nev];
  G[e] = mk<S>((S)v.re, (S)-v.im);
}

// Y[:, n] -= shift[n] X[:, n]
template <class S>
__global__ void shift_cols_kernel(cplx<S>* __restrict__ Y, const cplx<S>* __restrict__ X, const double* __restrict__ shift,
                                  int nev, int dim) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)dim * nev) return;
  const S sh = (S)shift[e % nev];
  Y[e].re -= sh * X[e].re;
  Y[e].im -= sh * X[e].im;
}

// Z[:, n] = R[:, n] / max(|d - shift[n]|, 0.05): a fixed positive diagonal, as preconditioned CG needs
template <class S>
__global__ void precond_shift_kernel(const cplx<S>* __restrict__ R, const double* __restrict__ d,
                                     const double* __restrict__ shift, int nev, int dim, cplx<S>* __restrict__ Z) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)dim * nev) return;
  double g = fabs(d[e / nev] - shift[e % nev]);
  if (g < 0.05) g = 0.05;
  const S inv = (S)(1.0 / g);
  Z[e] = mk<S>(R[e].re * inv, R[e].im * inv);
}

// Y[:, n] = a[n] X[:, n] + b[n] Y[:, n]
template <class S>
__global__ void axpby_cols_kernel(const cplx<S>* __restrict__ X, const double* __restrict__ a, const double* __restrict__ b,
                                  int nev, int dim, cplx<S>* __restrict__ Y) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)dim * nev) return;
  const int n = (int)(e % nev);
  const S an = (S)a[n], bn = (S)b[n];
  Y[e] = mk<S>(an * X[e].re + bn * Y[e].re, an * X[e].im + bn * Y[e].im);
}

// y_n += -2 Lf_n s_n lambda_n (the out-of-set part of the adjoint vector; the in-set part A Gamma is already in y)
template <class S>
__global__ void add_lambda_kernel(const cplx<S>* __restrict__ lam, const double* __restrict__ Lf,
                                  const zd* __restrict__ s, int nev, int dim, zd* __restrict__ y) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)dim * nev) return;
  const int n = (int)(e % nev);
  const zd sl = cmul(s[n], mk<double>((double)lam[e].re, (double)lam[e].im));
  y[e].re -= 2.0 * Lf[n] * sl.re;
  y[e].im -= 2.0 * Lf[n] * sl.im;
}

// hbar_I = sum_n 2 Lf_n s_n conj(A_In)
__global__ void adj_hbar_kernel(const zd* __restrict__ A, const double* __restrict__ Lf, const zd* __restrict__ s, int nev,
                                 int dim, zd* __restrict__ hbar) {
  const int I = blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= dim) return;
  zd acc = mk<double>(0, 0);
  for (int n = 0; n < nev; ++n) {
    const zd a = A[(size_t)I * nev + n];
    const zd t = cmulc(a, s[n]);  // conj(A) s
    acc.re += 2.0 * Lf[n] * t.re;
    acc.im += 2.0 * Lf[n] * t.im;
  }
  hbar[I] = acc;
}

// Per k: band-vector, band-energy and velocity-matrix adjoints of the window bands.
template <class T>
__global__ void __launch_bounds__(128) adj_band_kernel(
    const T* __restrict__ TA, const T* __restrict__ Ty, int ldt, const zd* __restrict__ A, const zd* __restrict__ y,
    int nev, const zd* __restrict__ hbar, const zd* __restrict__ vec_win, const double* __restrict__ eig_win,
    const zd* __restrict__ hr, const int* __restrict__ rvec, const int* __restrict__ ndegen, int nR,
    const double* __restrict__ rlat, const double* __restrict__ kpt, int nk, int nv, int nc, int w, float s32,
    double* __restrict__ Ebar, zd* __restrict__ Ubar, zd* __restrict__ Mbar) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int k = blockIdx.x;
  const int nb = nv + nc, ncv = nc * nv, ww = w * w;
  zd* B = reinterpret_cast<zd*>(smem_raw);   // nb * w band vectors (valence slots first)
  zd* U = B + nb * w;                        // ncv * ww
  zd* M = U + ncv * ww;                      // ww  (dH/dk_x)
  zd* Mv = M + ww;                           // nv * w   (M v)
  zd* MHc = Mv + nv * w;                     // nc * w   (M^H c)
  zd* eph = MHc + nc * w;                    // nR
  zd* Ub = eph + nR;                         // nb * w   (accumulated band-vector adjoints)
  double* Eb = reinterpret_cast<double*>(Ub + nb * w);  // nb
  double* Rx = Eb + nb;                                 // nR
  __shared__ double rl[9];
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid < 9) rl[tid] = rlat[tid];
  for (int e = tid; e < nb * w; e += nt) {
    B[e] = vec_win[(size_t)k * nb * w + e];
    Ub[e] = mk<double>(0, 0);
  }
  for (int e = tid; e < nb; e += nt) Eb[e] = 0.0;
  __syncthreads();
  const double* kk = kpt + 3 * k;
  for (int r = tid; r < nR; r += nt) {
    const double phi = phase_adj(rvec, nR, r, rl, kk);
    double sn, cs;
    sincos(phi, &sn, &cs);
    const double inv = 1.0 / (double)ndegen[r];
    eph[r] = mk<double>(cs * inv, sn * inv);
    Rx[r] = (double)__double2float_rn(rcart_adj(rvec[r], rvec[nR + r], rvec[2 * nR + r], rl, 0));
  }
  // U[cv][o][p] = sum_n conj(y_{kcv,n}) TA_n[k,o,p] + conj(A_{kcv,n}) Ty_n[k,o,p]
  const T* ta = TA + (size_t)k * ldt;
  const T* ty = Ty + (size_t)k * ldt;
  for (int e = tid; e < ncv * ww; e += nt) {
    const int cv = e / ww, op = e % ww;
    const size_t I = (size_t)k * ncv + cv;
    zd acc = mk<double>(0, 0);
    for (int n = 0; n < nev; ++n) {
      const size_t tix = ((size_t)n * ww + op) * 2;
      const zd tA = mk<double>((double)ta[tix], (double)ta[tix + 1]);
      const zd tY = mk<double>((double)ty[tix], (double)ty[tix + 1]);
      cfmac(acc, y[I * nev + n], tA);
      cfmac(acc, A[I * nev + n], tY);
    }
    U[e] = acc;
  }
  __syncthreads();
  // dH/dk_x at this k (on-site diagonal of R = 0 excluded), M v and M^H c
  for (int e = tid; e < ww; e += nt) {
    const int m = e / w, c = e % w;
    zd acc = mk<double>(0, 0);
    for (int r = 0; r < nR; ++r) {
      const bool r0 = rvec[r] == 0 && rvec[nR + r] == 0 && rvec[2 * nR + r] == 0;
      if (r0 && m == c) continue;
      const zd f = mk<double>(-Rx[r] * eph[r].im, Rx[r] * eph[r].re);
      cfma(acc, f, hr[((size_t)r * w + m) * w + c]);
    }
    M[e] = acc;
  }
  __syncthreads();
  for (int e = tid; e < nv * w; e += nt) {
    const int v = e / w, m = e % w;
    zd acc = mk<double>(0, 0);
    for (int c = 0; c < w; ++c) cfma(acc, M[m * w + c], B[v * w + c]);
    Mv[e] = acc;
  }
  for (int e = tid; e < nc * w; e += nt) {
    const int c = e / w, m = e % w;
    zd acc = mk<double>(0, 0);
    for (int r = 0; r < w; ++r) cfmac(acc, M[r * w + m], B[(nv + c) * w + r]);  // (M^H c)_m = sum_r conj(M_rm) c_r
    MHc[e] = acc;
  }
  __syncthreads();
  const double sf = (double)s32;
  // conduction-vector adjoints: coulomb part + velocity part
  for (int e = tid; e < nc * w; e += nt) {
    const int c = e / w, o = e % w;
    zd acc = mk<double>(0, 0);
    for (int v = 0; v < nv; ++v) {
      const zd* u = U + (size_t)(c * nv + v) * ww + o * w;
      for (int p = 0; p < w; ++p) cfmac(acc, B[v * w + p], u[p]);
      const size_t I = (size_t)k * ncv + c * nv + v;
      const double de = eig_win[(size_t)k * nb + nv + c] - eig_win[(size_t)k * nb + v];
      const double phi = de / (de * de + sf * sf);
      const zd hb = hbar[I];
      // conj(hbar) phi (M v)_o
      acc.re += phi * (hb.re * Mv[v * w + o].re + hb.im * Mv[v * w + o].im);
      acc.im += phi * (hb.re * Mv[v * w + o].im - hb.im * Mv[v * w + o].re);
    }
    Ub[(nv + c) * w + o] = acc;
  }
  // valence-vector adjoints
  for (int e = tid; e < nv * w; e += nt) {
    const int v = e / w, p = e % w;
    zd acc = mk<double>(0, 0);
    for (int c = 0; c < nc; ++c) {
      const zd* u = U + (size_t)(c * nv + v) * ww;
      for (int o = 0; o < w; ++o) cfmac(acc, B[(nv + c) * w + o], u[o * w + p]);
      const size_t I = (size_t)k * ncv + c * nv + v;
      const double de = eig_win[(size_t)k * nb + nv + c] - eig_win[(size_t)k * nb + v];
      const double phi = de / (de * de + sf * sf);
      const zd hb = hbar[I];
      const zd t = cmul(hb, MHc[c * w + p]);  // hbar phi M^H c
      acc.re += phi * t.re;
      acc.im += phi * t.im;
    }
    Ub[v * w + p] = acc;
  }
  // band-energy adjoints: diagonal term and the velocity denominators
  if (tid < nb) {
    double acc = 0.0;
    const int sl = tid;
    for (int cv = 0; cv < ncv; ++cv) {
      const int c = cv / nv, v = cv % nv;
      if (sl != v && sl != nv + c) continue;
      const size_t I = (size_t)k * ncv + cv;
      double g = 0.0;
      for (int n = 0; n < nev; ++n) {
        const zd t = cmulc(A[I * nev + n], y[I * nev + n]);  // y conj(A)... real part below
        g += t.re;
      }
      // velocity: Re(conj(hbar) (c^H M v)) phi'(dE)
      zd cmv = mk<double>(0, 0);
      for (int m = 0; m < w; ++m) cfmac(cmv, B[(nv + c) * w + m], Mv[v * w + m]);
      const double de = eig_win[(size_t)k * nb + nv + c] - eig_win[(size_t)k * nb + v];
      const double den = de * de + sf * sf;
      const double dphi = (sf * sf - de * de) / (den * den);
      const zd hb = hbar[I];
      g += (hb.re * cmv.re + hb.im * cmv.im) * dphi;
      acc += (sl == nv + c) ? g : -g;
    }
    Eb[sl] = acc;
  }
  __syncthreads();
  for (int e = tid; e < nb * w; e += nt) Ubar[(size_t)k * nb * w + e] = Ub[e];
  for (int e = tid; e < nb; e += nt) Ebar[(size_t)k * nb + e] = Eb[e];
  // Mbar = sum_I hbar_I phi c v^H
  for (int e = tid; e < ww; e += nt) {
    const int m = e / w, n = e % w;
    zd acc = mk<double>(0, 0);
    for (int cv = 0; cv < ncv; ++cv) {
      const int c = cv / nv, v = cv % nv;
      const size_t I = (size_t)k * ncv + cv;
      const double de = eig_win[(size_t)k * nb + nv + c] - eig_win[(size_t)k * nb + v];
      const double phi = de / (de * de + sf * sf);
      const zd cm = B[(nv + c) * w + m];
      const zd vn = mk<double>(B[v * w + n].re, -B[v * w + n].im);
      const zd t = cmul(cmul(hbar[I], cm), vn);
      acc.re += phi * t.re;
      acc.im += phi * t.im;
    }
    Mbar[(size_t)k * ww + e] = acc;
  }
}

// Per k: back-propagation through the gauge-fixed Hermitian eigen-decomposition to G = dL/dH(k) (lower
// triangle and real diagonal, the entries ZHEEV('L') reads).
__global__ void __launch_bounds__(128) adj_eig_kernel(const zd* __restrict__ vec_all, const double* __restrict__ eig_all,
                                                      const int* __restrict__ nocp, double scs, int nk, int w, int nv,
                                                      int nc, const double* __restrict__ Ebar, const zd* __restrict__ Ubar,
                                                      zd* __restrict__ G) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int k = blockIdx.x;
  const int nb = nv + nc, ww = w * w;
  zd* U = reinterpret_cast<zd*>(smem_raw);  // U[o][b]
  zd* Ub = U + ww;                          // Ubar[o][b]
  zd* K = Ub + ww;                          // K[a][b] = u_a^H ubar_b
  zd* Bm = K + ww;                          // B[a][b]
  zd* Tm = Bm + ww;                         // U conj(B)
  zd* Hb = Tm + ww;                         // Hbar
  double* lam = reinterpret_cast<double*>(Hb + ww);  // w
  double* Ea = lam + w;                               // w
  const int tid = threadIdx.x, nt = blockDim.x;
  const int no = nocp[k];
  const int b0 = no - nv;
  for (int e = tid; e < ww; e += nt) {
    const int b = e / w, o = e % w;
    U[o * w + b] = vec_all[((size_t)k * w + b) * w + o];
    const int s = b - b0;
    Ub[o * w + b] = (s >= 0 && s < nb) ? Ubar[((size_t)k * nb + s) * w + o] : mk<double>(0, 0);
  }
  for (int b = tid; b < w; b += nt) {
    lam[b] = eig_all[(size_t)k * w + b] - (b >= no ? scs : 0.0);
    const int s = b - b0;
    Ea[b] = (s >= 0 && s < nb) ? Ebar[(size_t)k * nb + s] : 0.0;
  }
  __syncthreads();
  for (int e = tid; e < ww; e += nt) {
    const int a = e / w, b = e % w;
    zd acc = mk<double>(0, 0);
    for (int o = 0; o < w; ++o) cfmac(acc, U[o * w + a], Ub[o * w + b]);
    K[e] = acc;
  }
  __syncthreads();
  for (int e = tid; e < ww; e += nt) {
    const int a = e / w, b = e % w;
    if (a == b) {
      Bm[e] = mk<double>(Ea[b], 0.0);
      continue;
    }
    const double dl = lam[b] - lam[a];
    if (fabs(dl) < 1e-12) {
      Bm[e] = mk<double>(0, 0);
      continue;
    }
    const double F = 1.0 / dl;
    // conj(K_ab) + i Im(K_bb) U_1a / U_1b  (the gauge keeps the first component real)
    zd kp = mk<double>(K[e].re, -K[e].im);
    const double u1b = U[0 * w + b].re;
    if (u1b > 1e-300) kp.im += K[b * w + b].im * U[0 * w + a].re / u1b;
    Bm[e] = mk<double>(F * kp.re, F * kp.im);
  }
  __syncthreads();
  // Hbar = U conj(B) U^H
  for (int e = tid; e < ww; e += nt) {
    const int m = e / w, b = e % w;
    zd acc = mk<double>(0, 0);
    for (int a = 0; a < w; ++a) {
      const zd bc = mk<double>(Bm[a * w + b].re, -Bm[a * w + b].im);
      cfma(acc, U[m * w + a], bc);
    }
    Tm[e] = acc;
  }
  __syncthreads();
  for (int e = tid; e < ww; e += nt) {
    const int m = e / w, n = e % w;
    zd acc = mk<double>(0, 0);
    for (int b = 0; b < w; ++b) {
      const zd uc = mk<double>(U[n * w + b].re, -U[n * w + b].im);
      cfma(acc, Tm[m * w + b], uc);
    }
    Hb[e] = acc;
  }
  __syncthreads();
  for (int e = tid; e < ww; e += nt) {
    const int m = e / w, n = e % w;
    zd g = mk<double>(0, 0);
    if (m > n) {
      g = Hb[m * w + n];
      g.re += Hb[n * w + m].re;
      g.im -= Hb[n * w + m].im;
    } else if (m == n) {
      g = mk<double>(Hb[e].re, 0.0);
    }
    G[(size_t)k * ww + e] = g;
  }
}

// e^{i phi_kR} / ndegen_R for every (k, R), once (the forward's float32-rounded phase)
__global__ void adj_phase_kernel(const int* __restrict__ rvec, const int* __restrict__ ndegen, int nR,
                                 const double* __restrict__ rlat, const double* __restrict__ kpt, int nk,
                                 zd* __restrict__ eph) {
  __shared__ double rl[9];
  if (threadIdx.x < 9) rl[threadIdx.x] = rlat[threadIdx.x];
  __syncthreads();
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)nk * nR) return;
  const int k = (int)(e / nR), r = (int)(e % nR);
  double sn, cs;
  sincos(phase_adj(rvec, nR, r, rl, kpt + 3 * k), &sn, &cs);
  const double inv = 1.0 / (double)ndegen[r];
  eph[e] = mk<double>(cs * inv, sn * inv);
}

// Partial sums over the k-points of chunk blockIdx.y of dL/dhop(R,m,n) and dL/dihop(R,m,n) from G_k and Mbar_k:
// dH/dhop = e^{i phi}/nd, dH/dihop = i e^{i phi}/nd, dM/dhop = i R_x e^{i phi}/nd, dM/dihop = -R_x e^{i phi}/nd.
__global__ void adj_fourier_partial_kernel(const zd* __restrict__ G, const zd* __restrict__ Mbar,
                                           const zd* __restrict__ eph, const int* __restrict__ rvec, int nR, int w,
                                           const double* __restrict__ rlat, int nk, int kchunk,
                                           double* __restrict__ part) {
  __shared__ double rl[9];
  if (threadIdx.x < 9) rl[threadIdx.x] = rlat[threadIdx.x];
  __syncthreads();
  const int ent = nR * w * w;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ent) return;
  const int r = e / (w * w), m = (e / w) % w, n = e % w;
  const bool onsite = rvec[r] == 0 && rvec[nR + r] == 0 && rvec[2 * nR + r] == 0 && m == n;
  const double rx = (double)__double2float_rn(rcart_adj(rvec[r], rvec[nR + r], rvec[2 * nR + r], rl, 0));
  const int k0 = blockIdx.y * kchunk, k1 = min(nk, k0 + kchunk);
  double gh = 0.0, gi = 0.0;
  for (int k = k0; k < k1; ++k) {
    const zd ep = eph[(size_t)k * nR + r];
    const double cs = ep.re, sn = ep.im;  // already divided by ndegen
    const zd g = G[((size_t)k * w + m) * w + n];
    gh += g.re * cs + g.im * sn;
    gi += g.im * cs - g.re * sn;
    if (!onsite) {
      const zd mb = Mbar[((size_t)k * w + m) * w + n];
      gh += rx * (mb.im * cs - mb.re * sn);
      gi -= rx * (mb.re * cs + mb.im * sn);
    }
  }
  part[((size_t)blockIdx.y * ent + e) * 2] = gh;
  part[((size_t)blockIdx.y * ent + e) * 2 + 1] = gi;
}

// chunks summed in a fixed order into the Fortran layout (nvec, w, w)
__global__ void adj_fourier_reduce_kernel(const double* __restrict__ part, int nchunk, int nR, int w,
                                          double* __restrict__ dhop, double* __restrict__ dihop) {
  const int ent = nR * w * w;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ent) return;
  double gh = 0.0, gi = 0.0;
  for (int c = 0; c < nchunk; ++c) {
    gh += part[((size_t)c * ent + e) * 2];
    gi += part[((size_t)c * ent + e) * 2 + 1];
  }
  const int r = e / (w * w), m = (e / w) % w, n = e % w;
  const size_t f = (size_t)r + (size_t)nR * (m + (size_t)w * n);
  dhop[f] = gh;
  dihop[f] = gi;
}

// spectrum loss L = sum_j (spinf eps2(omega_j) - t_j)^2 (xx, no renormalisation) and its cotangents.
__global__ void spectrum_loss_kernel(const double* __restrict__ E, const double* __restrict__ f, int nev, int dimse,
                                     double sme, double caux, double e0, double ef, int nesp, double spinf,
                                     const double* __restrict__ target, double* __restrict__ out /*1 + 2 nev*/) {
  // one CTA; the grid of omega is split over threads, reductions in fixed order through shared memory
  __shared__ double red[256];
  const double tail = (dimse > nev) ? 0.0 : E[nev - 1];
  const double gam = sme + 10.0 * ((tail - E[0]) / (double)dimse);
  const double dgam_dE0 = -10.0 / (double)dimse;
  const double dgam_dElast = (dimse > nev) ? 0.0 : 10.0 / (double)dimse;
  double Lloc = 0.0;
  // per-thread partial cotangents for up to 64 excitons
  double gE[64], gF[64];
  for (int n = 0; n < nev; ++n) gE[n] = gF[n] = 0.0;
  double gG = 0.0;
  for (int j = threadIdx.x; j < nesp; j += blockDim.x) {
    const double om = e0 + ((ef - e0) * (double)j) / ((double)nesp - 1.0);
    double eps2 = 0.0, deps_dg = 0.0;
    for (int n = 0; n < nev; ++n) {
      const double x = om - E[n];
      const double D = x * x + gam * gam;
      eps2 += f[n] * (gam / D);
      deps_dg += f[n] * (x * x - gam * gam) / (D * D);
    }
    eps2 *= caux;
    const double rj = spinf * eps2 - target[j];
    Lloc += rj * rj;
    const double dr = 2.0 * rj * spinf * caux;  // dL/d(eps2/caux)
    for (int n = 0; n < nev; ++n) {
      const double x = om - E[n];
      const double D = x * x + gam * gam;
      gF[n] += dr * gam / D;
      gE[n] += dr * f[n] * 2.0 * gam * x / (D * D);
    }
    gG += dr * deps_dg;
  }
  auto reduce = [&](double v) {
    red[threadIdx.x] = v;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
      if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
      __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
  };
  const double L = reduce(Lloc);
  const double G = reduce(gG);
  for (int n = 0; n < nev; ++n) {
    const double a = reduce(gE[n]);
    const double b = reduce(gF[n]);
    if (threadIdx.x == 0) {
      out[1 + n] = a + (n == 0 ? G * dgam_dE0 : 0.0) + (n == nev - 1 ? G * dgam_dElast : 0.0);
      out[1 + nev + n] = b;
    }
  }
  if (threadIdx.x == 0) out[0] = L;
}

// ------------------------------------------------------------------------------------------------ host
// lambda[:, n] for every column at once: preconditioned CG on P (H - E_n) P lambda_n = P B[:, n], with P the
// projector onto the complement of the computed excitons A (there H - E_n is positive definite because the
// computed excitons are the lowest).  Each column has its own step lengths; a column whose relative
// residual is below tol keeps iterating with the others (its updates are tiny) until all are done.
template <class S>
int adjoint_solve(wtb_ctx* c, Operator<S>& op, const cplx<S>* A, const double* dE, const double* Edev,
                  const cplx<S>* Bvec, int dim, int nev, double tol, int maxit, cplx<S>* lam, int* iters) {
  cudaError_t err = cudaSuccess;
  const int ld = nev;
  cplx<S>* R = c->ws.get<cplx<S>>("adj_R", (size_t)dim * nev, &err);
  cplx<S>* Z = c->ws.get<cplx<S>>("adj_Z", (size_t)dim * nev, &err);
  cplx<S>* Pd = c->ws.get<cplx<S>>("adj_P", (size_t)dim * nev, &err);
  cplx<S>* Q = c->ws.get<cplx<S>>("adj_Q", (size_t)dim * nev, &err);
  zd* Cm = c->ws.get<zd>("adj_C", (size_t)nev * nev, &err);
  const int npart = std::max(1, std::min(304, (dim + 127) / 128));
  double* partial = c->ws.get<double>("adj_part", (size_t)npart * nev * nev * 2, &err);
  double* coef = c->ws.get<double>("adj_coef", (size_t)3 * nev, &err);  // alpha | -alpha | ones, then beta
  if (err != cudaSuccess) return ctx_set_err(c, WTB_ENOMEM, "adjoint workspace");
  const unsigned nb = (unsigned)(((long)dim * nev + 255) / 256);
  cudaStream_t s = c->s;
  auto project = [&](cplx<S>* X) -> cudaError_t {
    cudaError_t e = launch_gram<S>(A, ld, nev, X, ld, nev, dim, Cm, partial, npart, s);
    if (e != cudaSuccess) return e;
    return launch_update<S>(A, ld, nev, Cm, nev, nev, dim, X, ld, -1.0, 1.0, s);
  };
  std::vector<zd> hC((size_t)nev * nev);
  auto diag_dots = [&](const cplx<S>* X, const cplx<S>* Y, std::vector<double>& out) -> cudaError_t {
    cudaError_t e = launch_gram<S>(X, ld, nev, Y, ld, nev, dim, Cm, partial, npart, s);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(hC.data(), Cm, sizeof(zd) * nev * nev, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(s);
    out.assign(nev, 0.0);
    for (int n = 0; n < nev; ++n) out[n] = hC[(size_t)n * nev + n].re;
    return e;
  };
  std::vector<double> h(3 * nev, 1.0), rz, rz_new, pq, rr, bb;
  CKA(launch_copy_cols<S>(Bvec, ld, R, ld, nev, dim, s));
  CKA(project(R));
  CKA(cudaMemsetAsync(lam, 0, sizeof(cplx<S>) * dim * nev, s));
  CKA(diag_dots(R, R, bb));
  precond_shift_kernel<S><<<nb, 256, 0, s>>>(R, dE, Edev, nev, dim, Z); ++g_launch_count;
  CKA(project(Z));
  CKA(launch_copy_cols<S>(Z, ld, Pd, ld, nev, dim, s));
  CKA(diag_dots(R, Z, rz));
  int it = 0;
  bool done = true;
  for (int n = 0; n < nev; ++n) done &= !(bb[n] > 0);
  for (; !done && it < maxit; ++it) {
    // Q = P (H - E) Pd
    CKA(op.apply(Pd, ld, 0, nev, Q, ld, s));
    shift_cols_kernel<S><<<nb, 256, 0, s>>>(Q, Pd, Edev, nev, dim); ++g_launch_count;
    CKA(project(Q));
    CKA(diag_dots(Pd, Q, pq));
    for (int n = 0; n < nev; ++n) {
      const double a = (pq[n] > 0 && rz[n] > 0) ? rz[n] / pq[n] : 0.0;
      h[n] = a;
      h[nev + n] = -a;
      h[2 * nev + n] = 1.0;
    }
    CKA(cudaMemcpyAsync(coef, h.data(), sizeof(double) * 3 * nev, cudaMemcpyHostToDevice, s));
    // lam += alpha Pd ; R -= alpha Q
    axpby_cols_kernel<S><<<nb, 256, 0, s>>>(Pd, coef, coef + 2 * nev, nev, dim, lam); ++g_launch_count;
    axpby_cols_kernel<S><<<nb, 256, 0, s>>>(Q, coef + nev, coef + 2 * nev, nev, dim, R); ++g_launch_count;
    CKA(diag_dots(R, R, rr));
    done = true;
    for (int n = 0; n < nev; ++n)
      if (bb[n] > 0 && std::sqrt(std::max(rr[n], 0.0)) > tol * std::sqrt(bb[n])) done = false;
    if (done) {
      ++it;
      break;
    }
    precond_shift_kernel<S><<<nb, 256, 0, s>>>(R, dE, Edev, nev, dim, Z); ++g_launch_count;
    CKA(project(Z));
    CKA(diag_dots(R, Z, rz_new));
    for (int n = 0; n < nev; ++n) h[n] = rz[n] > 0 ? rz_new[n] / rz[n] : 0.0;
    rz = rz_new;
    // Pd = Z + beta Pd (the ones are still in coef[2 nev ..])
    CKA(cudaMemcpyAsync(coef, h.data(), sizeof(double) * nev, cudaMemcpyHostToDevice, s));
    axpby_cols_kernel<S><<<nb, 256, 0, s>>>(Z, coef + 2 * nev, coef, nev, dim, Pd); ++g_launch_count;
  }
  *iters = it;
  if (!done) return ctx_set_err(c, WTB_ENOCONV, "backward: the adjoint solve did not converge in " +
                                                     std::to_string(maxit) + " iterations");
  return WTB_OK;
}

template <class S>
int backward_impl(wtb_ctx* c, const wtb_bse_params* p, Operator<S>& op, MatFreeOperator<S>* mf, Operator<S>& opd,
                  const std::vector<double>& LE, const std::vector<double>& Lf, double* dhop, double* dihop,
                  double* dr0, int* cg_iters) {
  cudaError_t err = cudaSuccess;
  const int nk = c->nk, nv = c->nv, nc = c->nc, w = c->w, nb = nv + nc, nR = c->nR;
  const int dim = nk * nc * nv, nev = p->nev;
  cudaStream_t s = c->s;
  const zd* A64 = c->ws.find<zd>("Xout", (size_t)dim * nev);
  const zd* hrvel = c->ws.find<zd>("hrvel", (size_t)5 * dim);
  const double* dE = c->ws.find<double>("dE", dim);
  const zd* vec_win = c->ws.find<zd>("vec_win", (size_t)nk * nb * w);
  const double* eig_win = c->ws.find<double>("eig_win", (size_t)nk * nb);
  const zd* vec_all = c->ws.find<zd>("vec_all", (size_t)nk * w * w);
  const double* eig_all = c->ws.find<double>("eig_all", (size_t)nk * w);
  const int* nocp = c->ws.find<int>("nocp", nk);
  const zd* hr = c->ws.find<zd>("hr", (size_t)nR * w * w);
  const int* rvec = c->ws.find<int>("rvec", (size_t)3 * nR);
  const int* ndegen = c->ws.find<int>("ndegen", nR);
  const double* rlat = c->ws.find<double>("rlat", 9);
  const double* kpt = c->ws.find<double>("kpt", (size_t)3 * nk);
  if (!A64 || !hrvel || !dE || !vec_win || !eig_win || !vec_all || !eig_all || !nocp || !hr || !rvec || !ndegen ||
      !rlat || !kpt || !mf)
    return ctx_set_err(c, WTB_ESTATE, "backward: the forward solve's device data is gone (call wtb_bsesolver again)");
  double* LEd = c->ws.get<double>("adj_LE", nev, &err);
  double* Lfd = c->ws.get<double>("adj_Lf", nev, &err);
  double* Ed = c->ws.get<double>("adj_E", nev, &err);
  zd* sd = c->ws.get<zd>("adj_s", nev, &err);
  zd* Gam = c->ws.get<zd>("adj_Gamma", (size_t)nev * nev, &err);
  cplx<S>* AS = c->ws.get<cplx<S>>("adj_AS", (size_t)dim * nev, &err);
  cplx<S>* Bv = c->ws.get<cplx<S>>("adj_B", (size_t)dim * nev, &err);
  cplx<S>* lam = c->ws.get<cplx<S>>("adj_lam", (size_t)dim * nev, &err);
  zd* y = c->ws.get<zd>("adj_y", (size_t)dim * nev, &err);
  cplx<S>* yS = c->ws.get<cplx<S>>("adj_yS", (size_t)dim * nev, &err);
  zd* hbar = c->ws.get<zd>("adj_hbar", dim, &err);
  if (err != cudaSuccess) return ctx_set_err(c, WTB_ENOMEM, "adjoint workspace");
  const std::vector<double>& E = c->last_E;
  CKA(cudaMemcpyAsync(LEd, LE.data(), sizeof(double) * nev, cudaMemcpyHostToDevice, s));
  CKA(cudaMemcpyAsync(Lfd, Lf.data(), sizeof(double) * nev, cudaMemcpyHostToDevice, s));
  CKA(cudaMemcpyAsync(Ed, E.data(), sizeof(double) * nev, cudaMemcpyHostToDevice, s));
  // s_n = A_n^T hx (the xx velocity elements are the first dim entries of hrvel)
  adj_s_kernel<<<nev, 256, 0, s>>>(A64, nev, dim, hrvel, sd); ++g_launch_count;
  std::vector<zd> hs(nev);
  CKA(cudaMemcpyAsync(hs.data(), sd, sizeof(zd) * nev, cudaMemcpyDeviceToHost, s));
  CKA(cudaStreamSynchronize(s));
  // Gamma[m][n]: y_n = sum_m A_m Gamma[m][n] - 2 Lf_n s_n lambda_n, where the coupling to the other computed
  // excitons m is explicit (-2 Lf_n s_n conj(s_m) / (E_m - E_n); skipped for degenerate pairs, whose
  // individual strengths are not differentiable) and lambda_n is orthogonal to all of them
  std::vector<zd> hg((size_t)nev * nev);
  for (int m = 0; m < nev; ++m)
    for (int n = 0; n < nev; ++n) {
      zd g = mk<double>(0, 0);
      if (m == n) {
        g.re = LE[n];
      } else if (std::fabs(E[m] - E[n]) > 1e-9 * std::max(1.0, std::fabs(E[n]))) {
        const zd t = cmulc(hs[m], hs[n]);  // s_n conj(s_m)
        const double f = -2.0 * Lf[n] / (E[m] - E[n]);
        g = mk<double>(f * t.re, f * t.im);
      }
      hg[(size_t)m * nev + n] = g;
    }
  CKA(cudaMemcpyAsync(Gam, hg.data(), sizeof(zd) * nev * nev, cudaMemcpyHostToDevice, s));
  CKA((launch_convert_cols<double, S>(A64, nev, AS, nev, nev, dim, s)));
  const unsigned nbk = (unsigned)(((long)dim * nev + 255) / 256);
  bool any_f = false;
  for (double v : Lf) any_f |= (v != 0.0);
  int it = 0;
  if (any_f) {
    conj_bcast_kernel<S><<<nbk, 256, 0, s>>>(hrvel, dim, nev, Bv); ++g_launch_count;
    const double tol = sizeof(S) == 8 ? 1e-10 : 1e-5;
    CKAR(adjoint_solve<S>(c, op, AS, dE, Ed, Bv, dim, nev, tol, 1000, lam, &it));
  }
  CKA(launch_update<double>(A64, nev, nev, Gam, nev, nev, dim, y, nev, 1.0, 0.0, s));
  if (any_f) {
    add_lambda_kernel<S><<<nbk, 256, 0, s>>>(lam, Lfd, sd, nev, dim, y); ++g_launch_count;
  }
  adj_hbar_kernel<<<(dim + 255) / 256, 256, 0, s>>>(A64, Lfd, sd, nev, dim, hbar); ++g_launch_count;
  CKA((launch_convert_cols<double, S>(y, nev, yS, nev, nev, dim, s)));
  // T_A = V Z(A), T_y = V Z(y)
  const bool tcf = mf->kind == GEMM_TC_BF16;
  const size_t tbytes = (size_t)mf->Mpad * mf->Npad * (tcf ? sizeof(float) : sizeof(S));
  unsigned char* TA = c->ws.get<unsigned char>("adj_TA", tbytes, &err);
  unsigned char* Ty = c->ws.get<unsigned char>("adj_Ty", tbytes, &err);
  double* Ebar = c->ws.get<double>("adj_Ebar", (size_t)nk * nb, &err);
  zd* Ubar = c->ws.get<zd>("adj_Ubar", (size_t)nk * nb * w, &err);
  zd* Mbar = c->ws.get<zd>("adj_Mbar", (size_t)nk * w * w, &err);
  zd* Gk = c->ws.get<zd>("adj_Gk", (size_t)nk * w * w, &err);
  double* dh = c->ws.get<double>("adj_dhop", (size_t)nR * w * w, &err);
  double* di = c->ws.get<double>("adj_dihop", (size_t)nR * w * w, &err);
  if (err != cudaSuccess) return ctx_set_err(c, WTB_ENOMEM, "adjoint workspace");
  CKA(mf->contract(AS, nev, nev, s));
  CKA(cudaMemcpyAsync(TA, mf->Tm, tbytes, cudaMemcpyDeviceToDevice, s));
  CKA(mf->contract(yS, nev, nev, s));
  CKA(cudaMemcpyAsync(Ty, mf->Tm, tbytes, cudaMemcpyDeviceToDevice, s));
  {
    const size_t smem = (size_t)(nb * w + nc * nv * w * w + w * w + nv * w + nc * w + nR + nb * w) * sizeof(zd) +
                        (size_t)(nb + nR) * sizeof(double) + 16;
    if (smem > 200 * 1024) return ctx_set_err(c, WTB_EBADARG, "backward: per-k workspace exceeds shared memory");
    const int ldt = mf->Npad;
    const float s32 = (float)p->cshift;
    if (tcf || sizeof(S) == 4) {
      CKA(raise_smem_limit(reinterpret_cast<const void*>(adj_band_kernel<float>), (size_t)smem));
      adj_band_kernel<float><<<nk, 128, smem, s>>>(reinterpret_cast<const float*>(TA), reinterpret_cast<const float*>(Ty),
                                                   ldt, A64, y, nev, hbar, vec_win, eig_win, hr, rvec, ndegen, nR, rlat,
                                                   kpt, nk, nv, nc, w, s32, Ebar, Ubar, Mbar);
    } else {
      CKA(raise_smem_limit(reinterpret_cast<const void*>(adj_band_kernel<double>), (size_t)smem));
      adj_band_kernel<double><<<nk, 128, smem, s>>>(reinterpret_cast<const double*>(TA),
                                                    reinterpret_cast<const double*>(Ty), ldt, A64, y, nev, hbar, vec_win,
                                                    eig_win, hr, rvec, ndegen, nR, rlat, kpt, nk, nv, nc, w, s32, Ebar,
                                                    Ubar, Mbar);
    }
    ++g_launch_count;
    CKA(cudaGetLastError());
  }
  {
    const size_t smem = (size_t)6 * w * w * sizeof(zd) + 2 * w * sizeof(double) + 16;
    CKA(raise_smem_limit(reinterpret_cast<const void*>(adj_eig_kernel), (size_t)smem));
    adj_eig_kernel<<<nk, 128, smem, s>>>(vec_all, eig_all, nocp, c->scs, nk, w, nv, nc, Ebar, Ubar, Gk);
    ++g_launch_count;
    CKA(cudaGetLastError());
  }
  {
    // k split into chunks so that nR w^2 entries x chunks fill the GPU; phases computed once per (k, R)
    const int ent = nR * w * w;
    const int kchunk = std::max(16, (int)(((long)nk * ent + 152L * 2048 - 1) / (152L * 2048)));
    const int nchunk = (nk + kchunk - 1) / kchunk;
    zd* eph = c->ws.get<zd>("adj_eph", (size_t)nk * nR, &err);
    double* fpart = c->ws.get<double>("adj_fpart", (size_t)nchunk * ent * 2, &err);
    if (err != cudaSuccess) return ctx_set_err(c, WTB_ENOMEM, "adjoint workspace");
    adj_phase_kernel<<<(unsigned)(((long)nk * nR + 255) / 256), 256, 0, s>>>(rvec, ndegen, nR, rlat, kpt, nk, eph);
    adj_fourier_partial_kernel<<<dim3((ent + 127) / 128, nchunk), 128, 0, s>>>(Gk, Mbar, eph, rvec, nR, w, rlat, nk,
                                                                                 kchunk, fpart);
    adj_fourier_reduce_kernel<<<(ent + 255) / 256, 256, 0, s>>>(fpart, nchunk, nR, w, dh, di);
    g_launch_count += 3;
    CKA(cudaGetLastError());
  }
  if (dhop) CKA(cudaMemcpyAsync(dhop, dh, sizeof(double) * nR * w * w, cudaMemcpyDeviceToHost, s));
  if (dihop) CKA(cudaMemcpyAsync(dihop, di, sizeof(double) * nR * w * w, cudaMemcpyDeviceToHost, s));
  // dL/dr0 = Re sum_n y_n^H H' A_n, H' the operator of dV/dr0 (no diagonal)
  if (dr0) {
    cplx<S>* Yd = c->ws.get<cplx<S>>("adj_Yd", (size_t)dim * nev, &err);
    zd* Cm = c->ws.get<zd>("adj_C", (size_t)nev * nev, &err);
    const int npart = std::max(1, std::min(304, (dim + 127) / 128));
    double* partial = c->ws.get<double>("adj_part", (size_t)npart * nev * nev * 2, &err);
    if (err != cudaSuccess) return ctx_set_err(c, WTB_ENOMEM, "adjoint workspace");
    CKA(opd.apply(AS, nev, 0, nev, Yd, nev, s));
    CKA(launch_gram<S>(yS, nev, nev, Yd, nev, nev, dim, Cm, partial, npart, s));
    std::vector<zd> h((size_t)nev * nev);
    CKA(cudaMemcpyAsync(h.data(), Cm, sizeof(zd) * nev * nev, cudaMemcpyDeviceToHost, s));
    CKA(cudaStreamSynchronize(s));
    double g = 0.0;
    for (int n = 0; n < nev; ++n) g += h[(size_t)n * nev + n].re;
    *dr0 = g;
  }
  CKA(cudaStreamSynchronize(s));
  if (cg_iters) *cg_iters = it;
  return ctx_check_status(c);
}

}  // namespace
}  // namespace wtb

using namespace wtb;

extern "C" int wtb_bse_backward(wtb_ctx* c, const wtb_bse_params* p, const double* dL_dE, const double* dL_dfxx,
                                double* dL_dhop, double* dL_dihop, double* dL_dr0, wtb_timings* t) {
  if (!c) return WTB_EBADARG;
  if (cudaSetDevice(c->device) != cudaSuccess) return ctx_set_err(c, WTB_ENODEV, "device unavailable");
  if (!c->have_solve || !c->have_bands || !c->have_hr)
    return ctx_set_err(c, WTB_ESTATE, "no forward solve (call wtb_bsesolver first)");
  const wtb_bse_params& q0 = c->last_p;
  if (!p || p->nev != q0.nev || p->nc != q0.nc || p->nv != q0.nv || p->coultype != q0.coultype ||
      p->precision != q0.precision || std::memcmp(p->ngrid, q0.ngrid, sizeof(p->ngrid)) != 0 ||
      std::memcmp(p->mshift, q0.mshift, sizeof(p->mshift)) != 0 || p->r0 != q0.r0 || p->cshift != q0.cshift ||
      p->ktol != q0.ktol || p->ez != q0.ez || p->w_coul != q0.w_coul || p->lc != q0.lc ||
      std::memcmp(p->ediel, q0.ediel, sizeof(p->ediel)) != 0)
    return ctx_set_err(c, WTB_EBADARG, "backward parameters differ from the last wtb_bsesolver call");
  if (p->nev > 16) return ctx_set_err(c, WTB_EBADARG, "backward supports up to 16 excitons");
  if ((int)c->last_E.size() != p->nev) return ctx_set_err(c, WTB_ESTATE, "no exciton energies from the forward solve");
  std::vector<double> LE(p->nev, 0.0), Lf(p->nev, 0.0);
  for (int n = 0; n < p->nev; ++n) {
    if (dL_dE) LE[n] = dL_dE[n];
    if (dL_dfxx) Lf[n] = dL_dfxx[n];
    if (!std::isfinite(LE[n]) || !std::isfinite(Lf[n])) return ctx_set_err(c, WTB_ENAN, "non-finite cotangent");
  }
  wtb_bse_params q = *p;
  q.op = WTB_OP_MATFREE;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CKA(cudaEventCreate(&e0));
  CKA(cudaEventCreate(&e1));
  CKA(cudaEventRecord(e0, c->s));
  int r = WTB_OK, iters = 0;
  {
    OpBundle ob, obd;
    r = ctx_make_operator(c, &q, p->nev, &ob, "", false);
    if (r == WTB_OK) r = ctx_make_operator(c, &q, p->nev, &obd, "_dr0", true);
    if (r == WTB_OK) {
      if (ob.o64) {
        auto* mf = dynamic_cast<MatFreeOperator<double>*>(ob.o64.get());
        r = backward_impl<double>(c, p, *ob.o64, mf, *obd.o64, LE, Lf, dL_dhop, dL_dihop, dL_dr0, &iters);
      } else {
        auto* mf = dynamic_cast<MatFreeOperator<float>*>(ob.o32.get());
        // the accurate (6-product) arithmetic of the split-BF16 operator for the gradient
        ob.o32->begin_refine();
        obd.o32->begin_refine();
        r = backward_impl<float>(c, p, *ob.o32, mf, *obd.o32, LE, Lf, dL_dhop, dL_dihop, dL_dr0, &iters);
      }
    }
  }
  cudaEventRecord(e1, c->s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (t) {
    std::memset(t, 0, sizeof(*t));
    t->t_total_ms = ms;
    t->iterations = iters;
  }
  return r;
}

extern "C" int wtb_spectrum_loss(wtb_ctx* c, const wtb_bse_params* p, int dimse, int nev, const double* E,
                                 const double* fxx, const double* target, double* L, double* dL_dE, double* dL_dfxx) {
  if (!c) return WTB_EBADARG;
  if (cudaSetDevice(c->device) != cudaSuccess) return WTB_ENODEV;
  if (!p || nev < 1 || nev > 64 || dimse < nev || !E || !fxx || !target || p->numbse < 2)
    return ctx_set_err(c, WTB_EBADARG, "bad arguments (1 <= nev <= 64, dimse >= nev)");
  if (!c->have_hr) return ctx_set_err(c, WTB_ESTATE, "lattice not set (call wtb_set_hr first)");
  cudaError_t err = cudaSuccess;
  double* dEv = c->ws.get<double>("sl_E", nev, &err);
  double* df = c->ws.get<double>("sl_f", nev, &err);
  double* dt = c->ws.get<double>("sl_t", p->numbse, &err);
  double* dout = c->ws.get<double>("sl_out", 1 + 2 * nev, &err);
  if (err != cudaSuccess) return ctx_set_err(c, WTB_ENOMEM, "spectrum loss workspace");
  cudaStream_t s = c->s;
  CKA(cudaMemcpyAsync(dEv, E, sizeof(double) * nev, cudaMemcpyHostToDevice, s));
  CKA(cudaMemcpyAsync(df, fxx, sizeof(double) * nev, cudaMemcpyHostToDevice, s));
  CKA(cudaMemcpyAsync(dt, target, sizeof(double) * p->numbse, cudaMemcpyHostToDevice, s));
  const double vc = ctx_vcell3d(c);
  const int ng = p->ngrid[0] * p->ngrid[1] * p->ngrid[2];
  const double caux = (double)180.90f / ((double)(float)ng * vc * 1.0);
  spectrum_loss_kernel<<<1, 256, 0, s>>>(dEv, df, nev, dimse, p->cshift, caux, p->ebse0, p->ebsef, p->numbse,
                                         c->systype_np ? 2.0 : 1.0, dt, dout);
  ++g_launch_count;
  std::vector<double> h(1 + 2 * nev);
  CKA(cudaMemcpyAsync(h.data(), dout, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s));
  CKA(cudaStreamSynchronize(s));
  if (L) *L = h[0];
  for (int n = 0; n < nev; ++n) {
    if (dL_dE) dL_dE[n] = h[1 + n];
    if (dL_dfxx) dL_dfxx[n] = h[1 + nev + n];
  }
  return ctx_check_status(c);
}
