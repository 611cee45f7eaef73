// CTA-cooperative eigensolver for small Hermitian matrices held in shared memory (n <= 96): the projected
// problems of the block eigensolver and the per-k band problems.
//
// Method (the route of LAPACK's ZHEEV: ZHETRD + a tridiagonal eigensolver + back-transformation; here with
// bisection and inverse iteration for the tridiagonal stage because their work is independent per
// eigenpair and spreads over the CTA's threads):
//   1. Householder reduction to a real symmetric tridiagonal T = Q^H A Q with Q = H_0 H_1 ... H_{n-2},
//      H_j = I - tau_j v_j v_j^H (the lower-triangle convention of ZHETD2; v_j[0] = 1), two barriers a step;
//   2. the k-th smallest eigenvalue of T by Sturm-count bisection, one thread per eigenvalue;
//   3. its eigenvector z_k by inverse iteration (L D L^T of T - lam_k I with safeguarded pivots, three
//      solves from a fixed pseudo-random start), one thread per eigenvector, then modified Gram-Schmidt
//      inside each cluster of close eigenvalues (one warp per cluster);
//   4. u_k = Q z_k, one warp per eigenvector (no block barrier: each warp owns its vectors).
// An unreduced tridiagonal matrix has distinct eigenvalues; (near-)degenerate ones come from (near-)zero
// off-diagonal entries, for which independent inverse iterations from different starts give independent
// vectors of the eigenspace, made orthonormal by step 3's Gram-Schmidt.
// In FP64 the bisection runs in FP32 and only supplies shifts: the FP64 eigenvalues are Rayleigh quotients
// of the FP64 inverse-iteration vectors, and inside a cluster the Rayleigh-Ritz values of T on the cluster's
// vectors (an FP64 instruction costs a warp far more than an FP32 one on this GPU).
#pragma once
#include "wtb_internal.h"

namespace wtb {

template <class S>
__device__ __forceinline__ S warp_allsum(S v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <class S>
__device__ __forceinline__ S tiny_of() {
  return sizeof(S) == 4 ? (S)1e-30 : (S)1e-290;
}

template <class S>
__device__ __forceinline__ S fast_div(S a, S b) {
  return a / b;
}
template <>
__device__ __forceinline__ float fast_div<float>(float a, float b) {
  return __fdividef(a, b);
}

// Householder reflector of column j of A (warp 0 alone): from x = conj(row j right of the diagonal) it writes
// v_j over that row (v_j[0] = 1), beta to e[j], the scalar to tau[j] (zero: column already reduced) and the
// diagonal entry to d[j].
template <class S>
__device__ __forceinline__ void reflector_warp(cplx<S>* A, int lda, int n, int j, S* d, S* e, cplx<S>* tau) {
  const int lane = threadIdx.x & 31;
  const int L = n - 1 - j;
  cplx<S>* v = A + (size_t)j * lda + (j + 1);
  S sig = 0;
  for (int i = 1 + lane; i < L; i += 32) sig += v[i].re * v[i].re + v[i].im * v[i].im;
  sig = warp_allsum(sig);
  const cplx<S> alpha = cconj(v[0]);
  S beta;
  cplx<S> t = mk<S>(0, 0), sc = mk<S>(0, 0);
  if (sig == (S)0 && alpha.im == (S)0) {
    beta = alpha.re;
  } else {
    const S an = sqrt(alpha.re * alpha.re + alpha.im * alpha.im + sig);
    beta = alpha.re >= (S)0 ? -an : an;
    const S ib = (S)1 / beta;
    t = mk<S>((beta - alpha.re) * ib, -alpha.im * ib);
    const S dr = alpha.re - beta, di = alpha.im, dd = dr * dr + di * di;
    const S idd = (S)1 / dd;
    sc = mk<S>(dr * idd, -di * idd);  // 1 / (alpha - beta)
    for (int i = 1 + lane; i < L; i += 32) v[i] = cmul(cconj(v[i]), sc);
  }
  __syncwarp();  // every lane has read alpha = conj(v[0])
  if (lane == 0) {
    v[0] = mk<S>(1, 0);
    e[j] = beta;
    tau[j] = t;
    d[j] = A[(size_t)j * lda + j].re;
  }
  __syncwarp();
}

// Step 1.  A: n x n Hermitian (both triangles, n <= 97), row-major with leading dimension lda, in shared memory.
// On return row j right of the diagonal holds the reflector: A[j][j+1+i] = v_j[i] (v_j[0] = 1), i < n-1-j (row j
// is dead once column j has been reduced, and a row is contiguous for the products that use v_j).  d[n], e[n-1]
// receive T; tau[n-1] the reflector scalars; p[n] is scratch.  All threads of the block call it; blockDim.x is
// a multiple of 32.  Two barriers a step.  The matrix-vector product p = tau A22 v (two lanes per row) also sums
// q = Re(v^H A22 v), so that K = -1/2 tau (p^H v) = -1/2 |tau|^2 q needs no second pass over p.  Then the
// rank-2 update: warp 0 updates the next pivot row in registers and forms the next reflector from them while
// the other warps update the remaining rows.
template <class S>
__device__ void tridiag_cta(cplx<S>* A, int lda, int n, S* d, S* e, cplx<S>* tau, cplx<S>* p) {
  constexpr int TM = 2;  // lanes per row of the matrix-vector product
  __shared__ S qpart[32];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  const int tl = tid & (TM - 1), team = tid / TM, nteam = nt / TM;
  if (n > 1 && warp == 0) reflector_warp<S>(A, lda, n, 0, d, e, tau);
  __syncthreads();
  for (int j = 0; j < n - 1; ++j) {
    const int L = n - 1 - j;
    const cplx<S>* v = A + (size_t)j * lda + (j + 1);
    cplx<S>* A22 = A + (size_t)(j + 1) * lda + (j + 1);
    const cplx<S> tj = tau[j];
    if (tj.re == (S)0 && tj.im == (S)0) {  // column j needs no reflection: A22 is unchanged
      if (warp == 0 && j + 1 < n - 1) reflector_warp<S>(A, lda, n, j + 1, d, e, tau);
      __syncthreads();
      continue;
    }
    // p = tau A22 v and q (the loop bound is uniform, so every lane of a warp reaches the shuffles)
    S q = 0;
    for (int r0 = 0; r0 < L; r0 += nteam) {
      const int r = r0 + team;
      cplx<S> a0 = mk<S>(0, 0), a1 = mk<S>(0, 0);
      if (r < L) {
        const cplx<S>* row = A22 + (size_t)r * lda;
        int c = tl;
        for (; c + TM < L; c += 2 * TM) {
          cfma(a0, row[c], v[c]);
          cfma(a1, row[c + TM], v[c + TM]);
        }
        if (c < L) cfma(a0, row[c], v[c]);
      }
      cplx<S> acc = mk<S>(a0.re + a1.re, a0.im + a1.im);
#pragma unroll
      for (int o = TM / 2; o > 0; o >>= 1) {
        acc.re += __shfl_xor_sync(0xffffffffu, acc.re, o);
        acc.im += __shfl_xor_sync(0xffffffffu, acc.im, o);
      }
      if (r < L && tl == 0) {
        p[r] = cmul(tj, acc);
        q += v[r].re * acc.re + v[r].im * acc.im;
      }
    }
#pragma unroll
    for (int o = TM; o < 32; o <<= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
    if (lane == 0) qpart[warp] = q;
    __syncthreads();
    S qs = 0;
    for (int w = 0; w < nwarp; ++w) qs += qpart[w];
    const S K = (S)-0.5 * (tj.re * tj.re + tj.im * tj.im) * qs;
    // A22 -= v w^H + w v^H with w = p + K v: element (r, c) -= v_r conj(w_c) + w_r conj(v_c)
    auto upd = [&](cplx<S>& a, const cplx<S>& vr, const cplx<S>& wr, const cplx<S>& vc, const cplx<S>& pc) {
      const cplx<S> wc = mk<S>(pc.re + K * vc.re, pc.im + K * vc.im);
      a.re -= vr.re * wc.re + vr.im * wc.im + wr.re * vc.re + wr.im * vc.im;
      a.im -= vr.im * wc.re - vr.re * wc.im + wr.im * vc.re - wr.re * vc.im;
    };
    const bool rows_by_warp0 = nwarp == 1;
    if (warp == 0) {
      // pivot row 0 of A22 in registers (c = lane + 32 h), then the reflector of column j + 1 from it:
      // x_i = conj(A22[0][1 + i]); row j + 1 right of the diagonal becomes v_{j+1} (v[0] = 1 at c = 1)
      const cplx<S> vr = v[0], pr = p[0];
      const cplx<S> wr = mk<S>(pr.re + K * vr.re, pr.im + K * vr.im);
      cplx<S> a[3];
#pragma unroll
      for (int h = 0; h < 3; ++h) {
        const int c = lane + 32 * h;
        a[h] = mk<S>(0, 0);
        if (c < L) {
          a[h] = A22[c];
          upd(a[h], vr, wr, v[c], p[c]);
        }
      }
      if (j + 1 < n - 1) {
        S sg = 0;
#pragma unroll
        for (int h = 0; h < 3; ++h) {
          const int c = lane + 32 * h;
          if (c >= 2 && c < L) sg += a[h].re * a[h].re + a[h].im * a[h].im;
        }
        sg = warp_allsum(sg);
        const cplx<S> alpha = mk<S>(__shfl_sync(0xffffffffu, a[0].re, 1), -__shfl_sync(0xffffffffu, a[0].im, 1));
        S beta;
        cplx<S> t = mk<S>(0, 0), sc = mk<S>(0, 0);
        const bool refl = !(sg == (S)0 && alpha.im == (S)0);
        if (!refl) {
          beta = alpha.re;
        } else {
          const S an = sqrt(alpha.re * alpha.re + alpha.im * alpha.im + sg);
          beta = alpha.re >= (S)0 ? -an : an;
          const S ib = (S)1 / beta;
          t = mk<S>((beta - alpha.re) * ib, -alpha.im * ib);
          const S dr = alpha.re - beta, di = alpha.im, dd = dr * dr + di * di;
          const S idd = (S)1 / dd;
          sc = mk<S>(dr * idd, -di * idd);  // 1 / (alpha - beta)
        }
#pragma unroll
        for (int h = 0; h < 3; ++h) {
          const int c = lane + 32 * h;
          if (c < L) {
            cplx<S> o = a[h];  // c = 0: the diagonal
            if (c == 1) o = mk<S>(1, 0);
            else if (c >= 2 && refl) o = cmul(cconj(a[h]), sc);
            A22[c] = o;
          }
        }
        if (lane == 0) {
          e[j + 1] = beta;
          tau[j + 1] = t;
          d[j + 1] = a[0].re;
        }
      } else {
#pragma unroll
        for (int h = 0; h < 3; ++h) {
          const int c = lane + 32 * h;
          if (c < L) A22[c] = a[h];
        }
      }
    }
    if (warp > 0 || rows_by_warp0) {
      // rows 1 .. L-1 element by element over the other warps' threads (or warp 0's, for one warp): independent
      // updates, several in flight per thread
      const int nt1 = rows_by_warp0 ? 32 : nt - 32, t1 = rows_by_warp0 ? lane : tid - 32, ne = (L - 1) * L;
      const float rL = 1.0f / (float)L;
#pragma unroll 4
      for (int e2 = t1; e2 < ne; e2 += nt1) {
        const int r = 1 + qdiv(e2, rL), c = e2 - (r - 1) * L;
        const cplx<S> vr = v[r], pr = p[r];
        const cplx<S> wr = mk<S>(pr.re + K * vr.re, pr.im + K * vr.im);
        upd(A22[(size_t)r * lda + c], vr, wr, v[c], p[c]);
      }
    }
    __syncthreads();
  }
  if (tid == 0) d[n - 1] = A[(size_t)(n - 1) * lda + (n - 1)].re;
  __syncthreads();
}

// Number of eigenvalues of T below x (Sturm count of T - x I, pivots safeguarded by pivmin).
template <class S>
__device__ __forceinline__ int sturm_count(const S* d, const S* e2, int n, S x, S pivmin) {
  S q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  int c = q < (S)0;
  for (int i = 1; i < n; ++i) {
    q = (d[i] - x) - fast_div<S>(e2[i - 1], q);
    if (fabs(q) < pivmin) q = -pivmin;
    c += q < (S)0;
  }
  return c;
}

// Steps 2-4 after tridiag_cta.  Computes the nwant lowest eigenpairs: lam[k] ascending and the eigenvectors
// of A column by column, U[k * ldu + i] (complex, shared memory, ldu >= n).  Scratch (shared): e2[n], and Z, Dv,
// Lv of nwant * (n + 1) each (vector k at offset k * (n + 1): one thread per vector and one warp per vector
// both read them without bank conflicts), Lv directly after Dv (U may alias Dv, both being dead by step 4),
// cl[nwant] (ints), red[4].
template <class S>
__device__ void tridiag_eigvecs_cta(const cplx<S>* A, int lda, int n, int nwant, const S* d, const S* e,
                                    const cplx<S>* tau, S* e2, S* lam, S* Z, S* Dv, S* Lv, int* cl, cplx<S>* U,
                                    int ldu, S* red) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  const int ldz = n + 1;
  const S eps = sizeof(S) == 4 ? (S)5.96e-8 : (S)1.11e-16;
  for (int i = tid; i < n - 1; i += nt) e2[i] = e[i] * e[i];
  // Gershgorin interval and the scale of T (one warp)
  if (warp == 0) {
    S lo = d[0], hi = d[0], emax2 = 0;
    for (int i = lane; i < n; i += 32) {
      const S r = (i > 0 ? fabs(e[i - 1]) : (S)0) + (i < n - 1 ? fabs(e[i]) : (S)0);
      lo = fmin(lo, d[i] - r);
      hi = fmax(hi, d[i] + r);
      if (i < n - 1) emax2 = fmax(emax2, e[i] * e[i]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
      emax2 = fmax(emax2, __shfl_xor_sync(0xffffffffu, emax2, o));
    }
    if (lane == 0) {
      const S tn = fmax(fabs(lo), fabs(hi));
      const S tiny = tiny_of<S>();
      const S pivmin = fmax(emax2, (S)1) * tiny;
      red[0] = lo - (S)2 * eps * tn - pivmin;
      red[1] = hi + (S)2 * eps * tn + pivmin;
      red[2] = fmax(tn, tiny);
      red[3] = pivmin;
    }
  }
  __syncthreads();
  const S tnorm = red[2], pivmin = red[3];
  // step 2: multisection.  G lanes per eigenvalue (a power of two, G * nwant <= blockDim.x where possible) each
  // evaluate the Sturm count at one of G interior points of the current interval; the first point whose count
  // exceeds k closes the new interval, which shrinks by G + 1 per round.  In FP64 it runs in FP32 on the rounded
  // T (an FP64 instruction costs a warp dozens of FP32 ones on this part): the FP32 eigenvalue is then only the
  // shift of the FP64 inverse iteration, and the FP64 eigenvalue is the Rayleigh quotient of the FP64 vector.
  {
    using B = float;
    const B* db;
    const B* e2b;
    B pivb;
    if constexpr (sizeof(S) == 8) {
      float* df = reinterpret_cast<float*>(Z);  // Z is free until step 3
      float* e2f = df + n;
      for (int i = tid; i < n; i += nt) {
        df[i] = (float)d[i];
        if (i < n - 1) e2f[i] = (float)e2[i];
      }
      __syncthreads();
      db = df;
      e2b = e2f;
      pivb = fmaxf((float)(pivmin / tiny_of<S>() * 1e-30), 1e-30f);
    } else {
      db = reinterpret_cast<const B*>(d);
      e2b = reinterpret_cast<const B*>(e2);
      pivb = (B)pivmin;
    }
    const B epsb = 5.96e-8f;
    int G = 1;
    while (G < 32 && 2 * G * nwant <= nt) G *= 2;
    const int gl = tid & (G - 1), grp = tid / G, ngrp = nt / G;
    const unsigned gsh = (unsigned)(lane & ~(G - 1));
    const unsigned gmask = G == 32 ? 0xffffffffu : ((1u << G) - 1u);
    for (int k0 = 0; k0 < nwant; k0 += ngrp) {  // uniform loop: every lane reaches the warp votes
      const int k = k0 + grp;
      B a = (B)red[0], b = (B)red[1];
      {
        const B w0 = b - a;
        a -= (B)4 * epsb * fabsf(w0) + pivb;
        b += (B)4 * epsb * fabsf(w0) + pivb;
      }
      bool done = k >= nwant;
      for (int it = 0; it < 128; ++it) {
        if (!__any_sync(0xffffffffu, !done)) break;
        const B h = (b - a) / (B)(G + 1);
        bool gt = false;
        if (!done) gt = sturm_count<B>(db, e2b, n, a + h * (B)(gl + 1), pivb) > k;
        const unsigned gm = (__ballot_sync(0xffffffffu, gt) >> gsh) & gmask;
        if (!done) {
          const int f = gm ? __ffs(gm) - 1 : G;  // first interior point with more than k eigenvalues below
          const B na = f > 0 ? a + h * (B)f : a;
          const B nb = f < G ? a + h * (B)(f + 1) : b;
          if (!(na > a || nb < b) || nb - na <= (B)2 * epsb * fmaxf(fabsf(na), fabsf(nb)) + pivb) done = true;
          a = na;
          b = nb;
        }
      }
      if (k < nwant && gl == 0) lam[k] = (S)((B)0.5 * (a + b));
    }
  }
  __syncthreads();
  // step 3: inverse iteration, one thread per eigenvector (vector k at offset k * ldz of Z, Dv, Lv)
  const S tiny = eps * tnorm;
  // clusters from the (shift) eigenvalues: runs closer than 1e-3 ||T|| to their neighbour
  for (int k = tid; k < nwant; k += nt) {
    int s0 = k;
    while (s0 > 0 && lam[s0] - lam[s0 - 1] <= (S)1e-3 * tnorm) --s0;
    cl[k] = s0;
  }
  // FP32 shifts carry about 1e-7 of the spread of T: two passes reach FP32 accuracy, three FP64's
  constexpr int kPasses = sizeof(S) == 4 ? 2 : 3;
  for (int k = tid; k < nwant; k += nt) {
    S* zk = Z + (size_t)k * ldz;
    S* dk = Dv + (size_t)k * ldz;  // reciprocal pivots (one division per pivot; the solves multiply)
    S* lk = Lv + (size_t)k * ldz;
    const S sh = lam[k];
    S Dp = d[0] - sh;
    if (fabs(Dp) < tiny) Dp = tiny;
    S Dr = (S)1 / Dp;
    dk[0] = Dr;
    for (int i = 1; i < n; ++i) {
      const S l = e[i - 1] * Dr;
      lk[i - 1] = l;
      Dp = (d[i] - sh) - l * e[i - 1];
      if (fabs(Dp) < tiny) Dp = tiny;
      Dr = (S)1 / Dp;
      dk[i] = Dr;
    }
    // start: deterministic pseudo-random entries in [-1, 1) (distinct for every k)
    for (int i = 0; i < n; ++i) {
      unsigned h = (unsigned)(i + 1) * 2654435761u ^ (unsigned)(k + 7) * 2246822519u;
      h ^= h >> 15;
      h *= 0x2c1b3c6du;
      h ^= h >> 12;
      zk[i] = (S)(h & 0xffffffu) * (S)(1.0 / 8388608.0) - (S)1;  // exact in FP32 too (24-bit integer, 2^-23)
    }
    for (int pass = 0; pass < kPasses; ++pass) {
      // L y = b (in place) and y /= D; L^T x = y (in place) with the largest magnitude on the way
      S y = zk[0];
      zk[0] = y * dk[0];
      for (int i = 1; i < n; ++i) {
        y = zk[i] - lk[i - 1] * y;
        zk[i] = y * dk[i];
      }
      S x = zk[n - 1], mx = fabs(x);
      for (int i = n - 2; i >= 0; --i) {
        x = zk[i] - lk[i] * x;
        zk[i] = x;
        mx = fmax(mx, fabs(x));
      }
      if (!(mx > (S)0)) mx = (S)1;
      const S imx = (S)1 / mx;
      S nrm = 0;
      for (int i = 0; i < n; ++i) {
        const S v = zk[i] * imx;
        nrm += v * v;
      }
      const S sc = imx / sqrt(nrm);
      for (int i = 0; i < n; ++i) zk[i] *= sc;
    }
  }
  __syncthreads();
  // modified Gram-Schmidt inside each cluster, one warp per cluster (clusters are contiguous runs)
  for (int k0 = warp; k0 < nwant; k0 += nw) {
    if (cl[k0] != k0) continue;  // not a cluster start
    int k1 = k0 + 1;
    while (k1 < nwant && cl[k1] == k0) ++k1;
    for (int jv = k0 + 1; jv < k1; ++jv) {
      S* zj = Z + (size_t)jv * ldz;
      for (int iv = k0; iv < jv; ++iv) {
        const S* zi = Z + (size_t)iv * ldz;
        S dot = 0;
        for (int i = lane; i < n; i += 32) dot += zi[i] * zj[i];
        dot = warp_allsum(dot);
        for (int i = lane; i < n; i += 32) zj[i] -= dot * zi[i];
        __syncwarp();
      }
      S nrm = 0;
      for (int i = lane; i < n; i += 32) nrm += zj[i] * zj[i];
      nrm = warp_allsum(nrm);
      const S sc = nrm > (S)0 ? (S)1 / sqrt(nrm) : (S)0;
      for (int i = lane; i < n; i += 32) zj[i] *= sc;
      __syncwarp();
    }
  }
  __syncthreads();
  if constexpr (sizeof(S) == 8) {
    // FP64 eigenvalues: Rayleigh quotients z^T T z; inside a cluster the Rayleigh-Ritz of T on the cluster's
    // vectors (one warp per cluster; the small symmetric problem by cyclic Jacobi on lane 0; its matrices
    // use the dead L D L^T storage at offset k0 ldz, which clusters starting at different k0 cannot overlap)
    for (int k0 = warp; k0 < nwant; k0 += nw) {
      if (cl[k0] != k0) continue;
      int k1 = k0 + 1;
      while (k1 < nwant && cl[k1] == k0) ++k1;
      const int kc = k1 - k0;
      S* Tc = Dv + (size_t)k0 * ldz;
      S* Yc = Lv + (size_t)k0 * ldz;
      for (int a = 0; a < kc; ++a)
        for (int b = a; b < kc; ++b) {
          const S* za = Z + (size_t)(k0 + a) * ldz;
          const S* zb = Z + (size_t)(k0 + b) * ldz;
          S acc = 0;
          for (int i = lane; i < n; i += 32) {
            S tz = d[i] * zb[i];
            if (i > 0) tz += e[i - 1] * zb[i - 1];
            if (i < n - 1) tz += e[i] * zb[i + 1];
            acc += za[i] * tz;
          }
          acc = warp_allsum(acc);
          if (lane == 0) {
            Tc[a * kc + b] = acc;
            Tc[b * kc + a] = acc;
          }
        }
      __syncwarp();
      if (kc == 1 || kc > 32) {
        // a single vector, or a cluster too large for the in-register rotation: Rayleigh quotients
        if (lane == 0)
          for (int a = 0; a < kc; ++a) lam[k0 + a] = Tc[a * kc + a];
        __syncwarp();
        continue;
      }
      if (lane == 0) {
        for (int a = 0; a < kc; ++a)
          for (int b = 0; b < kc; ++b) Yc[a * kc + b] = a == b ? (S)1 : (S)0;
        for (int sweep = 0; sweep < 30; ++sweep) {
          S off = 0, dia = 0;
          for (int a = 0; a < kc; ++a) {
            dia += Tc[a * kc + a] * Tc[a * kc + a];
            for (int b = a + 1; b < kc; ++b) off += Tc[a * kc + b] * Tc[a * kc + b];
          }
          if (off <= (S)1e-32 * dia) break;
          for (int a = 0; a < kc - 1; ++a)
            for (int b = a + 1; b < kc; ++b) {
              const S apq = Tc[a * kc + b];
              if (fabs(apq) <= (S)1e-300) continue;
              const S zeta = (Tc[b * kc + b] - Tc[a * kc + a]) / (2 * apq);
              const S t = (zeta >= 0 ? (S)1 : (S)-1) / (fabs(zeta) + sqrt((S)1 + zeta * zeta));
              const S c = (S)1 / sqrt((S)1 + t * t), sn = t * c;
              for (int q = 0; q < kc; ++q) {  // columns a, b
                const S xa = Tc[q * kc + a], xb = Tc[q * kc + b];
                Tc[q * kc + a] = c * xa - sn * xb;
                Tc[q * kc + b] = sn * xa + c * xb;
              }
              for (int q = 0; q < kc; ++q) {  // rows a, b
                const S xa = Tc[a * kc + q], xb = Tc[b * kc + q];
                Tc[a * kc + q] = c * xa - sn * xb;
                Tc[b * kc + q] = sn * xa + c * xb;
              }
              for (int q = 0; q < kc; ++q) {
                const S ya = Yc[q * kc + a], yb = Yc[q * kc + b];
                Yc[q * kc + a] = c * ya - sn * yb;
                Yc[q * kc + b] = sn * ya + c * yb;
              }
            }
        }
        // ascending order: selection sort of the diagonal, columns of Yc follow
        for (int a = 0; a < kc; ++a) {
          int mi = a;
          for (int b = a + 1; b < kc; ++b)
            if (Tc[b * kc + b] < Tc[mi * kc + mi]) mi = b;
          if (mi != a) {
            const S t = Tc[a * kc + a];
            Tc[a * kc + a] = Tc[mi * kc + mi];
            Tc[mi * kc + mi] = t;
            for (int q = 0; q < kc; ++q) {
              const S y = Yc[q * kc + a];
              Yc[q * kc + a] = Yc[q * kc + mi];
              Yc[q * kc + mi] = y;
            }
          }
          lam[k0 + a] = Tc[a * kc + a];
        }
      }
      __syncwarp();
      // Z_c <- Z_c Yc, row by row (each lane owns rows)
      for (int i = lane; i < n; i += 32) {
        S zrow[32];
        for (int b = 0; b < kc; ++b) zrow[b] = Z[(size_t)(k0 + b) * ldz + i];
        for (int a = 0; a < kc; ++a) {
          S acc = 0;
          for (int b = 0; b < kc; ++b) acc += zrow[b] * Yc[b * kc + a];
          Z[(size_t)(k0 + a) * ldz + i] = acc;
        }
      }
      __syncwarp();
    }
    __syncthreads();
  }
  // step 4: u_k = H_0 (H_1 (... H_{n-2} z_k)), one team of TS lanes per eigenvector (teams inside warps, so a
  // reflector costs a few shuffles and no block barrier); v_j is row j of A right of the diagonal, contiguous
  {
    const int TS = n > 16 ? 16 : 8;
    const int tl = tid & (TS - 1), team = tid / TS, nteam = nt / TS;
    const int kmax = (nwant + nteam - 1) / nteam * nteam;  // uniform trip count: every lane reaches the shuffles
    for (int k = team; k < kmax; k += nteam) {
      const bool on = k < nwant;
      cplx<S>* u = U + (size_t)(on ? k : 0) * ldu;
      if (on)
        for (int i = tl; i < n; i += TS) u[i] = mk<S>(Z[(size_t)k * ldz + i], 0);
      __syncwarp();
      for (int j = n - 2; j >= 0; --j) {
        const cplx<S> tj = tau[j];
        if (tj.re == (S)0 && tj.im == (S)0) continue;  // uniform: tau is shared
        const cplx<S>* vj = A + (size_t)j * lda + (j + 1);
        const int L = n - 1 - j;
        cplx<S> dt = mk<S>(0, 0);
        if (on)
          for (int i = tl; i < L; i += TS) cfmac(dt, vj[i], u[j + 1 + i]);
#pragma unroll
        for (int o = TS / 2; o > 0; o >>= 1) {
          dt.re += __shfl_xor_sync(0xffffffffu, dt.re, o);
          dt.im += __shfl_xor_sync(0xffffffffu, dt.im, o);
        }
        const cplx<S> f = cmul(tj, dt);
        if (on)
          for (int i = tl; i < L; i += TS) {
            const cplx<S> vv = vj[i];
            cplx<S>& a0 = u[j + 1 + i];
            a0.re -= f.re * vv.re - f.im * vv.im;
            a0.im -= f.re * vv.im + f.im * vv.re;
          }
        __syncwarp();
      }
    }
  }
  __syncthreads();
}

}  // namespace wtb
