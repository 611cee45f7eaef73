// The final Rayleigh-Ritz step of the reduced-precision solves, in FP64 accuracy with few FP64 instructions.
//
// After the FP32 iteration the block X (FP32) and its fresh image AX (FP32, the operator's final arithmetic)
// define the reported excitons: the Grams M = X^H X and G = X^H AX, the orthonormalising basis, the projected
// m x m eigenproblem and the combination C.  On this GPU an FP64 instruction costs a warp about 64 FP32 ones,
// so:
//   gram_pair_dot2_kernel  both Grams from the FP32 data with every product split exactly (h = a b in FP32,
//                          l = fma(a, b, -h)) and the sums carried as FP32 pairs by error-free TwoSum (the
//                          compensated dot product of Ogita, Rump and Oishi, "Accurate sum and dot product",
//                          SIAM J. Sci. Comput. 26, 2005): per entry and part the result is as accurate as an
//                          FP64 accumulation of the FP32 products, which are exact in FP64;
//   small_rr_kernel        one CTA per system, FP64, at most 32 x 32: the orthonormalising basis B, the
//                          projected matrix B^H G B and its eigenpairs by cyclic Jacobi rotations (a complex
//                          Hermitian rotation per pair, n/2 disjoint pairs per round), with C = B Y for the
//                          lowest m.  The final block is orthonormal to FP32 rounding, M = I + E with |E| ~ 1e-7:
//                          then B = M^(-1/2) = I - E/2 + 3/8 E^2 (exact to |E|^3) from products alone, and the
//                          projected matrix is diagonal to the iteration's residual, so one Jacobi sweep does
//                          nearly all the rotations and later ones skip those below 1e-10 (FP64 square roots
//                          and divisions cost this GPU hundreds of cycles each).  Otherwise: the scaled Cholesky
//                          basis with the drop rule of pchol_basis_kernel.  It replaces the Cholesky, two
//                          products, the tridiagonal eigensolver and a third product (five launches).
//   update_dot2_kernel     X C and AX C for the reported vectors and residuals, FP64-accurate from FP32 X.
#include <cfloat>

#include "solver.h"
#include "wtb_internal.h"

namespace wtb {
namespace {

// error-free transformations (Knuth's TwoSum; the FMA product split)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (s, c) += x y exactly up to the carried error's own rounding
__device__ __forceinline__ void dot2_add(float& s, float& c, float x, float y) {
  const float h = x * y;
  const float l = fmaf(x, y, -h);
  float t, e;
  two_sum(s, h, t, e);
  s = t;
  c += e + l;
}

struct Acc2 {
  float s = 0.f, c = 0.f;
};

// conj(a) b into (re, im) compensated accumulators
__device__ __forceinline__ void cdot2(Acc2& re, Acc2& im, zf a, zf b) {
  dot2_add(re.s, re.c, a.re, b.re);
  dot2_add(re.s, re.c, a.im, b.im);
  dot2_add(im.s, im.c, a.re, b.im);
  dot2_add(im.s, im.c, -a.im, b.re);
}

// One CTA per reduction part, a 16 x 16 thread grid over the p x p entries (p <= 16 TI) of both Grams, TI x TI
// entries of each per thread; rows staged 32 at a time.  Partials [part][p][p] of M, then of G at npart p p
// further on, as complex(8).
template <int TI>
__global__ void __launch_bounds__(256) gram_pair_dot2_kernel(const zf* __restrict__ A, const zf* __restrict__ B, int ld,
                                                             int p, int nrow, double* __restrict__ partial,
                                                             int rows_per_part, int npart, BatchMap bm) {
  constexpr int RT = 32, WC = 16 * TI;
  __shared__ zf As[RT][WC];
  __shared__ zf Bs[RT][WC];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  long r_begin, r_end;
  const int sys = bm_part(bm, blockIdx.x, nrow, rows_per_part, &r_begin, &r_end);
  if (bm_frozen(bm, sys)) return;  // uniform over the CTA; the sums skip frozen systems too
  Acc2 mre[TI][TI], mim[TI][TI], gre[TI][TI], gim[TI][TI];
  for (long r0 = r_begin; r0 < r_end; r0 += RT) {
    for (int e = tid; e < RT * WC; e += 256) {
      const int rr = e / WC, c = e - rr * WC;
      const long gr = r0 + rr;
      const bool ok = gr < r_end && c < p;
      As[rr][c] = ok ? A[gr * ld + c] : mk<float>(0.f, 0.f);
      Bs[rr][c] = ok ? B[gr * ld + c] : mk<float>(0.f, 0.f);
    }
    __syncthreads();
    const int nr = (int)min((long)RT, r_end - r0);
    for (int rr = 0; rr < nr; ++rr) {
#pragma unroll
      for (int i = 0; i < TI; ++i) {
        const zf a = As[rr][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < TI; ++j) {
          cdot2(mre[i][j], mim[i][j], a, As[rr][tx + 16 * j]);
          cdot2(gre[i][j], gim[i][j], a, Bs[rr][tx + 16 * j]);
        }
      }
    }
    __syncthreads();
  }
  const size_t n = (size_t)p * p * 2;
#pragma unroll
  for (int i = 0; i < TI; ++i)
#pragma unroll
    for (int j = 0; j < TI; ++j) {
      const int ii = ty + 16 * i, jj = tx + 16 * j;
      if (ii < p && jj < p) {
        double* om = partial + (size_t)blockIdx.x * n + 2 * (ii * p + jj);
        double* og = partial + ((size_t)npart + blockIdx.x) * n + 2 * (ii * p + jj);
        om[0] = (double)mre[i][j].s + (double)mre[i][j].c;
        om[1] = (double)mim[i][j].s + (double)mim[i][j].c;
        og[0] = (double)gre[i][j].s + (double)gre[i][j].c;
        og[1] = (double)gim[i][j].s + (double)gim[i][j].c;
      }
    }
}

// Out (nrow x nout, complex(8)) = X C for FP32 rows X (nin <= 32 columns) and FP64 C (nin x nout, nout <= 32):
// C = Ch + Cl with Ch = fl32(C) and Cl = fl32(C - Ch); the X Ch products enter compensated FP32 sums of their
// exact splits, the X Cl products (2^-24 smaller) a plain FP32 sum, which leaves an error near 2^-48 of the
// terms, as an FP64 product would.  Row tiles of kTileRows rows; C of the tile's system staged in shared memory.
__global__ void __launch_bounds__(256) update_dot2_kernel(const zf* __restrict__ X, int ldx, int nin,
                                                          const zd* __restrict__ C, int ldc, int nout, int nrow,
                                                          zd* __restrict__ Out, int ldo, BatchMap bm, long c_stride) {
  __shared__ zf Ch[32 * 32], Cl[32 * 32];
  __shared__ zf Xs[kTileRows][33];
  const int tid = threadIdx.x;
  const long ntile = ((long)nrow + kTileRows - 1) / kTileRows;
  int staged = -1;
  for (long t = blockIdx.x; t < ntile; t += gridDim.x) {
    const int sys = bm_sys_of_row(bm, t * kTileRows);  // uniform over the CTA
    if (bm_frozen(bm, sys)) continue;
    __syncthreads();  // the previous tile's reads are done
    if (sys != staged) {
      const zd* Cq = C + (size_t)sys * c_stride;
      for (int e = tid; e < nin * nout; e += blockDim.x) {
        const int i = e / nout, j = e - i * nout;
        const zd c = Cq[(size_t)i * ldc + j];
        const float hr = (float)c.re, hi = (float)c.im;
        Ch[e] = mk<float>(hr, hi);
        Cl[e] = mk<float>((float)(c.re - (double)hr), (float)(c.im - (double)hi));
      }
      staged = sys;
    }
    const long r0 = t * kTileRows;
    const int nr = (int)min((long)kTileRows, nrow - r0);
    for (int e = tid; e < nr * nin; e += blockDim.x) {
      const int rr = e / nin, i = e - rr * nin;
      Xs[rr][i] = X[(r0 + rr) * ldx + i];
    }
    __syncthreads();
    for (int e = tid; e < nr * nout; e += blockDim.x) {
      const int rr = e / nout, j = e - rr * nout;
      Acc2 re, im;
      float lre = 0.f, lim = 0.f;
      for (int i = 0; i < nin; ++i) {
        const zf x = Xs[rr][i], h = Ch[i * nout + j], l = Cl[i * nout + j];
        dot2_add(re.s, re.c, x.re, h.re);
        dot2_add(re.s, re.c, -x.im, h.im);
        dot2_add(im.s, im.c, x.re, h.im);
        dot2_add(im.s, im.c, x.im, h.re);
        lre = fmaf(x.re, l.re, fmaf(-x.im, l.im, lre));
        lim = fmaf(x.re, l.im, fmaf(x.im, l.re, lim));
      }
      Out[(r0 + rr) * ldo + j] = mk<double>((double)re.s + (double)re.c + (double)lre,
                                            (double)im.s + (double)im.c + (double)lim);
    }
  }
}

// ---------------------------------------------------------------------------------------- small Rayleigh-Ritz
constexpr int kRRMax = 32;

__device__ __forceinline__ zd zconj(zd a) { return mk<double>(a.re, -a.im); }
__device__ __forceinline__ zd zmul(zd a, zd b) { return mk<double>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
__device__ __forceinline__ zd zadd(zd a, zd b) { return mk<double>(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ zd zscale(zd a, double s) { return mk<double>(a.re * s, a.im * s); }

// Players 0..N-1 (N even) of round t of the circle schedule: pair i of the round.
__device__ __forceinline__ void rr_pair(int N, int t, int i, int* p, int* q) {
  int a, b;
  if (i == 0) {
    a = N - 1;
    b = t;
  } else {
    a = (t + i) % (N - 1);
    b = (t - i + (N - 1)) % (N - 1);
  }
  *p = min(a, b);
  *q = max(a, b);
}

constexpr int kRRL = kRRMax + 1;

// FP64 1/sqrt(x) and 1/d for arguments inside the FP32 normal range, without the FP64 division and square-root
// sequences (the FP64 pipe runs at 1/64 of the FP32 rate here): an FP32 estimate, then two Newton-Raphson steps
// in FP64, y <- y (3 - x y^2) / 2 and z <- z (2 - d z); the error falls quadratically from the estimate's 2^-23
// to a few FP64 ulp (checked on the host from estimates up to 4 FP32 ulp off: <= 4.1e-16 relative).
__device__ __forceinline__ double rsqrt_nr(double x) {
  double y = (double)rsqrtf((float)x);
  y = y * fma(-0.5 * x, y * y, 1.5);
  y = y * fma(-0.5 * x, y * y, 1.5);
  return y;
}
__device__ __forceinline__ double rcp_nr(double d) {
  double z = (double)(1.0f / (float)d);
  z = z * fma(-d, z, 2.0);
  z = z * fma(-d, z, 2.0);
  return z;
}
__device__ __forceinline__ bool in_f32_range(double x) {  // |x| (nonzero) with room for a square in FP32
  const double a = fabs(x);
  return a > 1e-18 && a < 1e18;
}

// Cyclic Jacobi on the r x r Hermitian A (shared, rows of kRRL), accumulating V <- V U: N (r rounded up to even)
// players, N - 1 rounds of N / 2 disjoint pairs per sweep; a pair with the padding player is skipped.  Rotation
// of pair (p, q): with A_pq = g e (g = |A_pq|, |e| = 1) and zeta = (A_qq - A_pp) / (2 g),
// t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)), c = 1 / sqrt(1 + t^2), s = t c, U = [[c, s], [-s conj(e), c conj(e)]]
// on (p, q) makes (U^H A U)_pq = 0; A <- U^H A U.  Stops when the off-diagonal mass is below tol2 times the
// diagonal's (or after 40 sweeps).  All threads of the CTA call it.
template <class T>
__device__ void jacobi_cta(cplx<T> (*A)[kRRL], cplx<T> (*V)[kRRL], int r, T tol2, T skip_rel, T* rot_c, T* rot_s,
                           cplx<T>* rot_e, T* offs, T* dias, int* s_done, int* s_any, int* s_sweep) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int N = (r + 1) & ~1;
  for (int sweep = 0; sweep < 40 && r > 1; ++sweep) {
    T off = 0, dia = 0;
    for (int e = tid; e < r * r; e += nt) {
      const int a = e / r, b = e - a * r;
      const T v = A[a][b].re * A[a][b].re + A[a][b].im * A[a][b].im;
      if (a == b)
        dia += v;
      else
        off += v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      dia += __shfl_xor_sync(0xffffffffu, dia, o);
    }
    if ((tid & 31) == 0) {
      offs[tid >> 5] = off;
      dias[tid >> 5] = dia;
    }
    __syncthreads();
    if (tid == 0) {
      T o = 0, d = 0;
      for (int w = 0; w < (nt >> 5); ++w) {
        o += offs[w];
        d += dias[w];
      }
      *s_done = o <= tol2 * d ? 1 : 0;
      *s_sweep = 0;  // after a barrier: every thread has read the previous sweep's flag
    }
    __syncthreads();
    if (*s_done) break;
    for (int t = 0; t < N - 1; ++t) {
      if (tid == 0) *s_any = 0;
      __syncthreads();
      if (tid < N / 2) {
        int p, q;
        rr_pair(N, t, tid, &p, &q);
        T c = 1, sn = 0;
        cplx<T> ee = mk<T>(1, 0);
        if (q < r) {
          const cplx<T> apq = A[p][q];
          const T g = sqrt(apq.re * apq.re + apq.im * apq.im);
          // a rotation whose angle (about g / |A_qq - A_pp|) is below skip_rel is left out: it would move the
          // vectors by less than that and the eigenvalues by its square times the gap
          if (g > (sizeof(T) == 4 ? (T)1e-30 : (T)1e-300) && g > skip_rel * fabs(A[q][q].re - A[p][p].re)) {
            *s_any = 1;  // benign race: every writer stores 1
            const T dqp = A[q][q].re - A[p][p].re;
            bool done = false;
            if constexpr (sizeof(T) == 8) {
              // the same rotation from Newton-refined reciprocals and reciprocal square roots (the inputs in
              // the FP32 range, else the division and square-root route below)
              const double g2 = apq.re * apq.re + apq.im * apq.im;
              if (in_f32_range(g)) {
                const double rg = rsqrt_nr(g2);  // 1 / g
                const double zeta = 0.5 * dqp * rg;
                if (fabs(zeta) < 1e17) {
                  const double z2 = fma(zeta, zeta, 1.0);
                  const double h = z2 * rsqrt_nr(z2);  // sqrt(1 + zeta^2)
                  const double tt = (zeta >= 0 ? 1.0 : -1.0) * rcp_nr(fabs(zeta) + h);
                  ee = mk<T>(apq.re * rg, apq.im * rg);
                  c = rsqrt_nr(fma(tt, tt, 1.0));
                  sn = tt * c;
                  done = true;
                }
              }
            }
            if (!done) {
              ee = mk<T>(apq.re / g, apq.im / g);
              const T zeta = dqp / (2 * g);
              const T tt = (zeta >= 0 ? (T)1 : (T)-1) / (fabs(zeta) + sqrt((T)1 + zeta * zeta));
              c = (T)1 / sqrt((T)1 + tt * tt);
              sn = tt * c;
            }
          }
        }
        rot_c[tid] = c;
        rot_s[tid] = sn;
        rot_e[tid] = ee;
      }
      __syncthreads();
      const int any = *s_any;
      __syncthreads();  // every thread has read the flag before the next round resets it
      if (!any) continue;  // uniform: no pair of this round rotates
      if (tid == 0) *s_sweep = 1;
      // columns: A[k][p], A[k][q] <- (A_kp c - A_kq s conj(e), A_kp s + A_kq c conj(e)); V likewise
      for (int e = tid; e < r * (N / 2); e += nt) {
        const int i = e / r, k = e - i * r;
        int p, q;
        rr_pair(N, t, i, &p, &q);
        if (q >= r) continue;
        const T c = rot_c[i], sn = rot_s[i];
        const cplx<T> ce = cconj(rot_e[i]);
        const cplx<T> akp = A[k][p], kq_ce = cmul(A[k][q], ce);
        A[k][p] = mk<T>(akp.re * c - kq_ce.re * sn, akp.im * c - kq_ce.im * sn);
        A[k][q] = mk<T>(akp.re * sn + kq_ce.re * c, akp.im * sn + kq_ce.im * c);
        const cplx<T> vkp = V[k][p], vq_ce = cmul(V[k][q], ce);
        V[k][p] = mk<T>(vkp.re * c - vq_ce.re * sn, vkp.im * c - vq_ce.im * sn);
        V[k][q] = mk<T>(vkp.re * sn + vq_ce.re * c, vkp.im * sn + vq_ce.im * c);
      }
      __syncthreads();
      // rows: A[p][k], A[q][k] <- (c A_pk - s e A_qk, s A_pk + c e A_qk)  (U^H from the left)
      for (int e = tid; e < r * (N / 2); e += nt) {
        const int i = e / r, k = e - i * r;
        int p, q;
        rr_pair(N, t, i, &p, &q);
        if (q >= r) continue;
        const T c = rot_c[i], sn = rot_s[i];
        const cplx<T> apk = A[p][k], e_qk = cmul(rot_e[i], A[q][k]);
        A[p][k] = mk<T>(apk.re * c - e_qk.re * sn, apk.im * c - e_qk.im * sn);
        A[q][k] = mk<T>(apk.re * sn + e_qk.re * c, apk.im * sn + e_qk.im * c);
      }
      __syncthreads();
    }
    __syncthreads();
    if (!*s_sweep) break;  // uniform: a sweep without rotations leaves nothing to do
  }
}

__global__ void __launch_bounds__(256) small_rr_kernel(const zd* __restrict__ Mg, const zd* __restrict__ Gg, int n,
                                                       int m, double drop, double* __restrict__ theta,
                                                       zd* __restrict__ Cg, int* __restrict__ keep, BatchMap bm,
                                                       long mat_stride, long theta_stride) {
  constexpr int L = kRRL;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zd(*W)[L] = reinterpret_cast<zd(*)[L]>(smem_raw);  // scaled Gram, its Schur complements; the compact R; G B
  zd(*R)[L] = W + kRRMax;                           // Cholesky rows in kept order; then the basis B (n x r)
  zd(*Gs)[L] = R + kRRMax;                          // G, then B^H G B
  zd(*A)[L] = Gs + kRRMax;                          // R^-1; then the projected matrix
  zd(*V)[L] = A + kRRMax;                           // eigenvectors of A (FP64 route)
  __shared__ double dinv[kRRMax], rinv[kRRMax], rot_c[kRRMax / 2], rot_s[kRRMax / 2], offs[8], dias[8];
  __shared__ zd rot_e[kRRMax / 2];
  __shared__ int perm[kRRMax], order[kRRMax];
  __shared__ int s_done, s_near, s_any, s_sweep;
  const int sys = blockIdx.x;
  if (bm_frozen(bm, sys)) return;
  Mg += (size_t)sys * mat_stride;
  Gg += (size_t)sys * mat_stride;
  Cg += (size_t)sys * mat_stride;
  theta += (size_t)sys * theta_stride;
  const int tid = threadIdx.x, nt = blockDim.x;
  // near-identity route when M = I + E with max |E| < 1e-5 (the final block is orthonormal to FP32 rounding):
  // B = M^(-1/2) = I - E/2 + 3/8 E^2 to O(|E|^3) < 1e-15, from products alone (no FP64 division or square root,
  // which this GPU issues at a fraction of the FP32 rate)
  if (tid == 0) s_near = 1;
  __syncthreads();
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, j = e - i * n;
    const zd a = Mg[(size_t)i * n + j];
    const double dr = a.re - (i == j ? 1.0 : 0.0);
    if (!(fabs(dr) < 1e-5 && fabs(a.im) < 1e-5)) s_near = 0;  // benign race: every writer stores 0
  }
  __syncthreads();
  if (s_near) {
    for (int e = tid; e < n * n; e += nt) {
      const int i = e / n, j = e - i * n;
      const zd a = Mg[(size_t)i * n + j], b = Mg[(size_t)j * n + i];
      W[i][j] = mk<double>(0.5 * (a.re + b.re) - (i == j ? 1.0 : 0.0), i == j ? 0.0 : 0.5 * (a.im - b.im));  // E
      const zd g = Gg[(size_t)i * n + j], h = Gg[(size_t)j * n + i];
      Gs[i][j] = mk<double>(0.5 * (g.re + h.re), i == j ? 0.0 : 0.5 * (g.im - h.im));
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += nt) {  // B = I - E/2 + 3/8 E^2
      const int i = e / n, j = e - i * n;
      zd e2 = mk<double>(0.0, 0.0);
      for (int k = 0; k < n; ++k) e2 = zadd(e2, zmul(W[i][k], W[k][j]));
      R[i][j] = mk<double>((i == j ? 1.0 : 0.0) - 0.5 * W[i][j].re + 0.375 * e2.re, -0.5 * W[i][j].im + 0.375 * e2.im);
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += nt) {  // T = G B
      const int i = e / n, j = e - i * n;
      zd acc = mk<double>(0.0, 0.0);
      for (int k = 0; k < n; ++k) acc = zadd(acc, zmul(Gs[i][k], R[k][j]));
      W[i][j] = acc;
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += nt) {  // Gp = B T (B Hermitian)
      const int i = e / n, j = e - i * n;
      zd acc = mk<double>(0.0, 0.0);
      for (int k = 0; k < n; ++k) acc = zadd(acc, zmul(R[i][k], W[k][j]));
      A[i][j] = acc;
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += nt) {  // Hermitian part
      const int i = e / n, j = e - i * n;
      const zd x = A[i][j], y = A[j][i];
      Gs[i][j] = mk<double>(0.5 * (x.re + y.re), i == j ? 0.0 : 0.5 * (x.im - y.im));
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += nt) {
      const int i = e / n, j = e - i * n;
      A[i][j] = Gs[i][j];
      V[i][j] = mk<double>(i == j ? 1.0 : 0.0, 0.0);
    }
    __syncthreads();
    // the final projected matrix is diagonal to the iteration's residual: one sweep does nearly all the rotations
    // and the next ones skip the negligible ones (angles below 1e-10)
    jacobi_cta<double>(A, V, n, 1e-30, 1e-10, rot_c, rot_s, rot_e, offs, dias, &s_done, &s_any, &s_sweep);
    for (int a = tid; a < n; a += nt) {
      const double va = A[a][a].re;
      int rank = 0;
      for (int b = 0; b < n; ++b) {
        const double vb = A[b][b].re;
        rank += (vb < va || (vb == va && b < a)) ? 1 : 0;
      }
      order[rank] = a;
    }
    __syncthreads();
    // C = B Y[:, order[0:m]]
    for (int e = tid; e < n * m; e += nt) {
      const int i = e / m, k = e - i * m;
      const int col = order[k];
      zd acc = mk<double>(0.0, 0.0);
      for (int c = 0; c < n; ++c) acc = zadd(acc, zmul(R[i][c], V[c][col]));
      Cg[(size_t)i * m + k] = acc;
    }
    for (int k = tid; k < m; k += nt) theta[k] = A[order[k]][order[k]].re;
    if (tid == 0 && keep) keep[sys] = n;
    return;
  }
  // general route: FP64 scaled Cholesky with drops, R^-1, projection and Jacobi
  for (int i = tid; i < n; i += nt) {
    const double d = Mg[(size_t)i * n + i].re;
    dinv[i] = d > 1e-300 ? 1.0 / sqrt(d) : 0.0;
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, j = e - i * n;
    const zd a = Mg[(size_t)i * n + j], b = Mg[(size_t)j * n + i];
    const double sc = dinv[i] * dinv[j];
    W[i][j] = mk<double>(0.5 * (a.re + b.re) * sc, i == j ? 0.0 : 0.5 * (a.im - b.im) * sc);
    const zd g = Gg[(size_t)i * n + j], h = Gg[(size_t)j * n + i];
    Gs[i][j] = mk<double>(0.5 * (g.re + h.re), i == j ? 0.0 : 0.5 * (g.im - h.im));
  }
  __syncthreads();
  // Cholesky of the scaled Gram in the basis order, dropping directions whose residual diagonal is <= drop
  int r = 0;
  for (int k = 0; k < n; ++k) {
    const double dk = W[k][k].re;
    if (!(dk > drop)) continue;  // uniform: every thread reads the same settled value
    const double rkk = sqrt(dk), irk = 1.0 / rkk;
    for (int j = tid; j < n; j += nt) R[r][j] = j == k ? mk<double>(rkk, 0.0) : (j > k ? zscale(W[k][j], irk) : mk<double>(0.0, 0.0));
    if (tid == 0) {
      perm[r] = k;
      rinv[r] = irk;
    }
    const double idk = 1.0 / dk;
    for (int e = tid; e < (n - k - 1) * (n - k - 1); e += nt) {
      const int i = k + 1 + e / (n - k - 1), j = k + 1 + e % (n - k - 1);
      const zd wi = W[k][i], wj = W[k][j];
      // W[i][j] -= conj(W[k][i]) W[k][j] / dk
      W[i][j].re -= (wi.re * wj.re + wi.im * wj.im) * idk;
      W[i][j].im -= (wi.re * wj.im - wi.im * wj.re) * idk;
    }
    ++r;
    __syncthreads();
  }
  __syncthreads();  // the last (dropped) columns' reads of W are done before it is overwritten
  // compact upper-triangular Rk (r x r) into W, then its inverse by back substitution, one thread per column
  for (int e = tid; e < r * r; e += nt) {
    const int k = e / r, l = e - k * r;
    W[k][l] = l >= k ? R[k][perm[l]] : mk<double>(0.0, 0.0);
  }
  __syncthreads();
  for (int c = tid; c < r; c += nt) {
    // R^-1 column c into A[.][c] (A is free until the projection)
    for (int k = c + 1; k < r; ++k) A[k][c] = mk<double>(0.0, 0.0);
    A[c][c] = mk<double>(rinv[c], 0.0);
    for (int k = c - 1; k >= 0; --k) {
      zd acc = mk<double>(0.0, 0.0);
      for (int l = k + 1; l <= c; ++l) acc = zadd(acc, zmul(W[k][l], A[l][c]));
      A[k][c] = zscale(acc, -rinv[k]);
    }
  }
  __syncthreads();
  // B (n x r): B[perm[k]][c] = dinv[perm[k]] R^-1[k][c], zero rows for dropped directions
  for (int e = tid; e < n * r; e += nt) {
    const int i = e / r, c = e - i * r;
    R[i][c] = mk<double>(0.0, 0.0);
  }
  __syncthreads();
  for (int e = tid; e < r * r; e += nt) {
    const int k = e / r, c = e - k * r;
    if (k <= c) R[perm[k]][c] = zscale(A[k][c], dinv[perm[k]]);
  }
  __syncthreads();
  // T = G B (n x r) into W, then A = B^H T (r x r), Hermitian part
  for (int e = tid; e < n * r; e += nt) {
    const int i = e / r, c = e - i * r;
    zd acc = mk<double>(0.0, 0.0);
    for (int j = 0; j < n; ++j) acc = zadd(acc, zmul(Gs[i][j], R[j][c]));
    W[i][c] = acc;
  }
  __syncthreads();
  for (int e = tid; e < r * r; e += nt) {
    const int a = e / r, b = e - a * r;
    zd acc = mk<double>(0.0, 0.0);
    for (int i = 0; i < n; ++i) acc = zadd(acc, zmul(zconj(R[i][a]), W[i][b]));
    Gs[a][b] = acc;
  }
  __syncthreads();
  for (int e = tid; e < r * r; e += nt) {
    const int a = e / r, b = e - a * r;
    const zd x = Gs[a][b], y = Gs[b][a];
    A[a][b] = mk<double>(0.5 * (x.re + y.re), a == b ? 0.0 : 0.5 * (x.im - y.im));
    V[a][b] = mk<double>(a == b ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  // cyclic Jacobi: N (r rounded up to even) players, N - 1 rounds of N / 2 disjoint pairs per sweep; a pair with
  // the padding player is skipped.  Rotation of pair (p, q): with A_pq = g e (g = |A_pq|, |e| = 1) and
  // zeta = (A_qq - A_pp) / (2 g), t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)), c = 1 / sqrt(1 + t^2), s = t c,
  // U = [[c, s], [-s conj(e), c conj(e)]] on (p, q) makes (U^H A U)_pq = 0; A <- U^H A U, V <- V U.
  jacobi_cta<double>(A, V, r, 1e-30, 0.0, rot_c, rot_s, rot_e, offs, dias, &s_done, &s_any, &s_sweep);
  // ascending order of the eigenvalues (rank by comparison; ties by index)
  for (int a = tid; a < r; a += nt) {
    const double va = A[a][a].re;
    int rank = 0;
    for (int b = 0; b < r; ++b) {
      const double vb = A[b][b].re;
      rank += (vb < va || (vb == va && b < a)) ? 1 : 0;
    }
    order[rank] = a;
  }
  __syncthreads();
  // C = B Y[:, order[0:m]] (n x m, leading dimension m); theta; missing pairs: 1e30 and zero columns
  for (int e = tid; e < n * m; e += nt) {
    const int i = e / m, k = e - i * m;
    zd acc = mk<double>(0.0, 0.0);
    if (k < r) {
      const int col = order[k];
      for (int c = 0; c < r; ++c) acc = zadd(acc, zmul(R[i][c], V[c][col]));
    }
    Cg[(size_t)i * m + k] = acc;
  }
  for (int k = tid; k < m; k += nt) theta[k] = k < r ? A[order[k]][order[k]].re : 1e30;
  if (tid == 0 && keep) keep[sys] = r;
}

}  // namespace

cudaError_t launch_gram_pair_dot2(const zf* A, const zf* B, int ld, int p, int nrow, zd* outM, zd* outG,
                                  double* partial, int npart, cudaStream_t s, const BatchMap& bm, long out_stride) {
  if (p < 1 || p > 32) return cudaErrorInvalidValue;
  if (bm.parts) npart = bm.nparts;
  const int rpp = (nrow + npart - 1) / npart;
  if (p <= 16)
    gram_pair_dot2_kernel<1><<<npart, 256, 0, s>>>(A, B, ld, p, nrow, partial, rpp, npart, bm);
  else
    gram_pair_dot2_kernel<2><<<npart, 256, 0, s>>>(A, B, ld, p, nrow, partial, rpp, npart, bm);
  ++g_launch_count;
  return launch_sum_partials_pair(partial, npart, p * p * 2, outM, outG, s, bm, out_stride);
}

cudaError_t launch_update_dot2(const zf* X, int ldx, int nin, const zd* C, int ldc, int nout, int nrow, zd* Out,
                               int ldo, cudaStream_t s, const BatchMap& bm, long c_stride) {
  if (nin < 1 || nin > 32 || nout < 1 || nout > 32) return cudaErrorInvalidValue;
  long nblk = ((long)nrow + kTileRows - 1) / kTileRows;
  if (nblk > 152 * 16) nblk = 152 * 16;
  update_dot2_kernel<<<(unsigned)nblk, 256, 0, s>>>(X, ldx, nin, C, ldc, nout, nrow, Out, ldo, bm, c_stride);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_small_rr(const zd* M, const zd* G, int n, int m, double drop, double* theta, zd* C, int* keep,
                            cudaStream_t s, const BatchMap& bm, long mat_stride, long theta_stride) {
  if (n < 1 || n > kRRMax || m < 1 || m > n) return cudaErrorInvalidValue;
  const size_t smem = (size_t)5 * kRRMax * (kRRMax + 1) * sizeof(zd);
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(small_rr_kernel), smem);
  if (e != cudaSuccess) return e;
  small_rr_kernel<<<bm.nsys, 256, smem, s>>>(M, G, n, m, drop, theta, C, keep, bm, mat_stride, theta_stride);
  ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace wtb
