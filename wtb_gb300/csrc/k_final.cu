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
//   small_rr_kernel        one CTA per system: the scaled Cholesky basis with the drop rule of
//                          pchol_basis_kernel, the projected matrix B^H G B and its eigenpairs by cyclic Jacobi
//                          rotations (a complex Hermitian rotation per pair, n/2 disjoint pairs per round), all
//                          in FP64 on at most 32 x 32 matrices, with C = B Y for the lowest m.  The final
//                          projected matrix is diagonal to the iteration's residual, so Jacobi ends in a few
//                          sweeps; it replaces the Cholesky, two products, the tridiagonal eigensolver and a
//                          third product (five launches).
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

__global__ void __launch_bounds__(256) small_rr_kernel(const zd* __restrict__ Mg, const zd* __restrict__ Gg, int n,
                                                       int m, double drop, double* __restrict__ theta,
                                                       zd* __restrict__ Cg, int* __restrict__ keep, BatchMap bm,
                                                       long mat_stride, long theta_stride) {
  constexpr int L = kRRMax + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zd(*W)[L] = reinterpret_cast<zd(*)[L]>(smem_raw);  // scaled Gram, its Schur complements; the compact R; G B
  zd(*R)[L] = W + kRRMax;                           // Cholesky rows in kept order; then the basis B (n x r)
  zd(*Gs)[L] = R + kRRMax;                          // G, then B^H G B
  zd(*A)[L] = Gs + kRRMax;                          // R^-1; then the projected matrix, diagonalised in place
  zd(*V)[L] = A + kRRMax;                           // eigenvectors of A
  __shared__ double dinv[kRRMax], rinv[kRRMax], rot_c[kRRMax / 2], rot_s[kRRMax / 2], offs[8], dias[8];
  __shared__ zd rot_e[kRRMax / 2];
  __shared__ int perm[kRRMax], order[kRRMax];
  __shared__ int s_r, s_done;
  const int sys = blockIdx.x;
  if (bm_frozen(bm, sys)) return;
  Mg += (size_t)sys * mat_stride;
  Gg += (size_t)sys * mat_stride;
  Cg += (size_t)sys * mat_stride;
  theta += (size_t)sys * theta_stride;
  const int tid = threadIdx.x, nt = blockDim.x;
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
  if (tid == 0) s_r = r;
  __syncthreads();
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
  const int N = (r + 1) & ~1;
  for (int sweep = 0; sweep < 40 && r > 1; ++sweep) {
    // convergence: off-diagonal mass against the diagonal's
    double off = 0.0, dia = 0.0;
    for (int e = tid; e < r * r; e += nt) {
      const int a = e / r, b = e - a * r;
      const double v = A[a][b].re * A[a][b].re + A[a][b].im * A[a][b].im;
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
      double o = 0.0, d = 0.0;
      for (int w = 0; w < (nt >> 5); ++w) {
        o += offs[w];
        d += dias[w];
      }
      // off-diagonal mass below (1e-15)^2 of the diagonal's: rotations no longer change any value by more than
      // an FP64 rounding
      s_done = o <= 1e-30 * d ? 1 : 0;
    }
    __syncthreads();
    if (s_done) break;
    for (int t = 0; t < N - 1; ++t) {
      if (tid < N / 2) {
        int p, q;
        rr_pair(N, t, tid, &p, &q);
        double c = 1.0, sn = 0.0;
        zd ee = mk<double>(1.0, 0.0);
        if (q < r) {
          const zd apq = A[p][q];
          const double g = sqrt(apq.re * apq.re + apq.im * apq.im);
          if (g > 1e-300) {
            ee = mk<double>(apq.re / g, apq.im / g);
            const double zeta = (A[q][q].re - A[p][p].re) / (2.0 * g);
            const double tt = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
            c = 1.0 / sqrt(1.0 + tt * tt);
            sn = tt * c;
          }
        }
        rot_c[tid] = c;
        rot_s[tid] = sn;
        rot_e[tid] = ee;
      }
      __syncthreads();
      // columns: A[k][p], A[k][q] <- (A_kp c - A_kq s conj(e), A_kp s + A_kq c conj(e)); V likewise
      for (int e = tid; e < r * (N / 2); e += nt) {
        const int i = e / r, k = e - i * r;
        int p, q;
        rr_pair(N, t, i, &p, &q);
        if (q >= r) continue;
        const double c = rot_c[i], sn = rot_s[i];
        const zd ce = zconj(rot_e[i]);
        const zd akp = A[k][p], akq = A[k][q];
        const zd kq_ce = zmul(akq, ce);
        A[k][p] = mk<double>(akp.re * c - kq_ce.re * sn, akp.im * c - kq_ce.im * sn);
        A[k][q] = mk<double>(akp.re * sn + kq_ce.re * c, akp.im * sn + kq_ce.im * c);
        const zd vkp = V[k][p], vkq = V[k][q];
        const zd vq_ce = zmul(vkq, ce);
        V[k][p] = mk<double>(vkp.re * c - vq_ce.re * sn, vkp.im * c - vq_ce.im * sn);
        V[k][q] = mk<double>(vkp.re * sn + vq_ce.re * c, vkp.im * sn + vq_ce.im * c);
      }
      __syncthreads();
      // rows: A[p][k], A[q][k] <- (c A_pk - s e A_qk, s A_pk + c e A_qk)  (U^H from the left)
      for (int e = tid; e < r * (N / 2); e += nt) {
        const int i = e / r, k = e - i * r;
        int p, q;
        rr_pair(N, t, i, &p, &q);
        if (q >= r) continue;
        const double c = rot_c[i], sn = rot_s[i];
        const zd ev = rot_e[i];
        const zd apk = A[p][k], aqk = A[q][k];
        const zd e_qk = zmul(ev, aqk);
        A[p][k] = mk<double>(apk.re * c - e_qk.re * sn, apk.im * c - e_qk.im * sn);
        A[q][k] = mk<double>(apk.re * sn + e_qk.re * c, apk.im * sn + e_qk.im * c);
      }
      __syncthreads();
    }
  }
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
