// CTA-cooperative eigensolver for small Hermitian matrices held in shared memory (n <= 96): the projected
// problems of the block eigensolver and the per-k band problems.
//
// Method (the route of LAPACK's ZHEEV: ZHETRD + a tridiagonal eigensolver + back-transformation; here with
// bisection and inverse iteration for the tridiagonal stage because their work is independent per
// eigenpair and spreads over the CTA's threads):
//   1. Householder reduction to a real symmetric tridiagonal T = Q^H A Q with Q = H_0 H_1 ... H_{n-2},
//      H_j = I - tau_j v_j v_j^H (the lower-triangle convention of ZHETD2; v_j[0] = 1), three barriers a step;
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

// Step 1.  A: n x n Hermitian (both triangles), row-major with leading dimension lda, in shared memory; it is
// overwritten: column j below the diagonal holds v_j.  d[n], e[n-1] receive T; tau[n-1] the reflector scalars;
// p[n] is scratch.  All threads of the block call it.
template <class S>
__device__ void tridiag_cta(cplx<S>* A, int lda, int n, S* d, S* e, cplx<S>* tau, cplx<S>* p, int* flag) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for (int j = 0; j < n - 1; ++j) {
    const int L = n - 1 - j;
    cplx<S>* vcol = A + (size_t)(j + 1) * lda + j;  // v_j[i] = vcol[i * lda]
    if (warp == 0) {
      S sig = 0;
      for (int i = 1 + lane; i < L; i += 32) {
        const cplx<S> x = vcol[(size_t)i * lda];
        sig += x.re * x.re + x.im * x.im;
      }
      sig = warp_allsum(sig);
      const cplx<S> alpha = vcol[0];
      bool skip = false;
      S beta;
      cplx<S> t = mk<S>(0, 0), sc = mk<S>(0, 0);
      if (sig == (S)0 && alpha.im == (S)0) {
        skip = true;
        beta = alpha.re;
      } else {
        const S an = sqrt(alpha.re * alpha.re + alpha.im * alpha.im + sig);
        beta = alpha.re >= (S)0 ? -an : an;
        t = mk<S>((beta - alpha.re) / beta, -alpha.im / beta);
        const S dr = alpha.re - beta, di = alpha.im, dd = dr * dr + di * di;
        sc = mk<S>(dr / dd, -di / dd);  // 1 / (alpha - beta)
      }
      if (!skip)
        for (int i = 1 + lane; i < L; i += 32) vcol[(size_t)i * lda] = cmul(vcol[(size_t)i * lda], sc);
      if (lane == 0) {
        vcol[0] = mk<S>(1, 0);
        e[j] = beta;
        tau[j] = t;
        d[j] = A[(size_t)j * lda + j].re;
        flag[0] = skip ? 1 : 0;
      }
    }
    __syncthreads();
    const bool skip = flag[0] != 0;
    if (skip) {
      __syncthreads();  // every thread has read the flag before warp 0 rewrites it
      continue;
    }
    const cplx<S> tj = tau[j];
    // p = tau A22 v (A22 = rows/columns j+1..n-1), one thread per row (no reduction on the critical path)
    for (int r = tid; r < L; r += nt) {
      const cplx<S>* row = A + (size_t)(j + 1 + r) * lda + (j + 1);
      cplx<S> acc = mk<S>(0, 0);
      for (int c = 0; c < L; ++c) cfma(acc, row[c], vcol[(size_t)c * lda]);
      p[r] = cmul(tj, acc);
    }
    __syncthreads();
    // K = -1/2 tau (p^H v), every warp for itself; w = p + K v;  A22 -= v w^H + w v^H
    cplx<S> sdot = mk<S>(0, 0);
    for (int c = lane; c < L; c += 32) cfmac(sdot, p[c], vcol[(size_t)c * lda]);
    sdot.re = warp_allsum(sdot.re);
    sdot.im = warp_allsum(sdot.im);
    const cplx<S> K = cmul(mk<S>((S)-0.5 * tj.re, (S)-0.5 * tj.im), sdot);
    for (int q = tid; q < L * L; q += nt) {
      const int r = q / L, c = q - r * L;
      const cplx<S> vr = vcol[(size_t)r * lda], vc = vcol[(size_t)c * lda];
      const cplx<S> wr = mk<S>(p[r].re + K.re * vr.re - K.im * vr.im, p[r].im + K.re * vr.im + K.im * vr.re);
      const cplx<S> wc = mk<S>(p[c].re + K.re * vc.re - K.im * vc.im, p[c].im + K.re * vc.im + K.im * vc.re);
      // v_r conj(w_c) + w_r conj(v_c)
      const S re = vr.re * wc.re + vr.im * wc.im + wr.re * vc.re + wr.im * vc.im;
      const S im = vr.im * wc.re - vr.re * wc.im + wr.im * vc.re - wr.re * vc.im;
      cplx<S>& a = A[(size_t)(j + 1 + r) * lda + (j + 1 + c)];
      a.re -= re;
      a.im -= im;
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

// Steps 2-4 after tridiag_cta.  Computes the nwant lowest eigenpairs: lam[k] ascending, U[i * ldu + k] the
// eigenvectors of A (complex, in shared memory).  Scratch (shared): e2[n], Z[n * nwant], Dv[n * nwant],
// Lv[n * nwant] (Lv directly after Dv: U may alias Dv with ldu = nwant, both being dead by step 4),
// cl[nwant] (ints), red[4].
template <class S>
__device__ void tridiag_eigvecs_cta(const cplx<S>* A, int lda, int n, int nwant, const S* d, const S* e,
                                    const cplx<S>* tau, S* e2, S* lam, S* Z, S* Dv, S* Lv, int* cl, cplx<S>* U,
                                    int ldu, S* red) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
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
      const S tiny = sizeof(S) == 4 ? (S)1e-30 : (S)1e-290;
      const S pivmin = fmax(emax2, (S)1) * tiny;
      red[0] = lo - (S)2 * eps * tn - pivmin;
      red[1] = hi + (S)2 * eps * tn + pivmin;
      red[2] = fmax(tn, tiny);
      red[3] = pivmin;
    }
  }
  __syncthreads();
  const S tnorm = red[2], pivmin = red[3];
  // step 2: bisection.  In FP64 it runs in FP32 on the rounded T (an FP64 instruction costs a warp dozens of
  // FP32 ones on this part); the FP32 eigenvalue is then only the shift of the FP64 inverse iteration, and
  // the FP64 eigenvalue is the Rayleigh quotient of the FP64 vector (step 3).
  if constexpr (sizeof(S) == 8) {
    float* df = reinterpret_cast<float*>(Z);  // Z is free until step 3
    float* e2f = df + n;
    for (int i = tid; i < n; i += nt) {
      df[i] = (float)d[i];
      if (i < n - 1) e2f[i] = (float)e2[i];
    }
    __syncthreads();
    const float epsf = 5.96e-8f;
    const float pivf = fmaxf((float)(pivmin / tiny_of<S>() * 1e-30), 1e-30f);
    for (int k = tid; k < nwant; k += nt) {
      float a = (float)red[0], b = (float)red[1];
      const float w0 = b - a;
      a -= 4.f * epsf * fabsf(w0) + pivf;
      b += 4.f * epsf * fabsf(w0) + pivf;
      for (int it = 0; it < 128; ++it) {
        const float mid = 0.5f * (a + b);
        if (b - a <= 2.f * epsf * fmaxf(fabsf(a), fabsf(b)) + pivf || mid <= a || mid >= b) break;
        if (sturm_count<float>(df, e2f, n, mid, pivf) > k)
          b = mid;
        else
          a = mid;
      }
      lam[k] = (S)(0.5f * (a + b));
    }
  } else {
    for (int k = tid; k < nwant; k += nt) {
      S a = red[0], b = red[1];
      for (int it = 0; it < 256; ++it) {
        const S mid = (S)0.5 * (a + b);
        if (b - a <= (S)2 * eps * fmax(fabs(a), fabs(b)) + pivmin || mid <= a || mid >= b) break;
        if (sturm_count<S>(d, e2, n, mid, pivmin) > k)
          b = mid;
        else
          a = mid;
      }
      lam[k] = (S)0.5 * (a + b);
    }
  }
  __syncthreads();
  // step 3: inverse iteration, one thread per eigenvector; column k of Z, Dv, Lv (stride nwant)
  const S tiny = eps * tnorm;
  // clusters from the (shift) eigenvalues: runs closer than 1e-3 ||T|| to their neighbour
  for (int k = tid; k < nwant; k += nt) {
    int s0 = k;
    while (s0 > 0 && lam[s0] - lam[s0 - 1] <= (S)1e-3 * tnorm) --s0;
    cl[k] = s0;
  }
  for (int k = tid; k < nwant; k += nt) {
    // Dv holds the reciprocal pivots (one division per pivot; the solves multiply)
    const S lk = lam[k];
    S Dp = d[0] - lk;
    if (fabs(Dp) < tiny) Dp = tiny;
    S Dr = (S)1 / Dp;
    Dv[k] = Dr;
    for (int i = 1; i < n; ++i) {
      const S l = e[i - 1] * Dr;
      Lv[(size_t)(i - 1) * nwant + k] = l;
      Dp = (d[i] - lk) - l * e[i - 1];
      if (fabs(Dp) < tiny) Dp = tiny;
      Dr = (S)1 / Dp;
      Dv[(size_t)i * nwant + k] = Dr;
    }
    // start: deterministic pseudo-random entries in [-1, 1) (distinct for every k)
    for (int i = 0; i < n; ++i) {
      unsigned h = (unsigned)(i + 1) * 2654435761u ^ (unsigned)(k + 7) * 2246822519u;
      h ^= h >> 15;
      h *= 0x2c1b3c6du;
      h ^= h >> 12;
      Z[(size_t)i * nwant + k] = (S)((double)(h & 0xffffffu) / 8388608.0 - 1.0);
    }
    for (int pass = 0; pass < 3; ++pass) {
      // L y = b (in place), y /= D, L^T x = y (in place)
      S y = Z[k];
      for (int i = 1; i < n; ++i) {
        const S v = Z[(size_t)i * nwant + k] - Lv[(size_t)(i - 1) * nwant + k] * y;
        Z[(size_t)i * nwant + k] = v;
        y = v;
      }
      for (int i = 0; i < n; ++i) Z[(size_t)i * nwant + k] *= Dv[(size_t)i * nwant + k];
      S x = Z[(size_t)(n - 1) * nwant + k];
      for (int i = n - 2; i >= 0; --i) {
        const S v = Z[(size_t)i * nwant + k] - Lv[(size_t)i * nwant + k] * x;
        Z[(size_t)i * nwant + k] = v;
        x = v;
      }
      S nrm = 0, mx = 0;
      for (int i = 0; i < n; ++i) mx = fmax(mx, fabs(Z[(size_t)i * nwant + k]));
      if (!(mx > (S)0)) mx = (S)1;
      const S imx = (S)1 / mx;
      for (int i = 0; i < n; ++i) {
        const S v = Z[(size_t)i * nwant + k] * imx;
        nrm += v * v;
      }
      const S sc = imx / sqrt(nrm);
      for (int i = 0; i < n; ++i) Z[(size_t)i * nwant + k] *= sc;
    }
  }
  __syncthreads();
  // modified Gram-Schmidt inside each cluster, one warp per cluster (clusters are contiguous runs)
  for (int k0 = warp; k0 < nwant; k0 += nw) {
    if (cl[k0] != k0) continue;  // not a cluster start
    int k1 = k0 + 1;
    while (k1 < nwant && cl[k1] == k0) ++k1;
    for (int jv = k0 + 1; jv < k1; ++jv) {
      for (int iv = k0; iv < jv; ++iv) {
        S dot = 0;
        for (int i = lane; i < n; i += 32) dot += Z[(size_t)i * nwant + iv] * Z[(size_t)i * nwant + jv];
        dot = warp_allsum(dot);
        for (int i = lane; i < n; i += 32) Z[(size_t)i * nwant + jv] -= dot * Z[(size_t)i * nwant + iv];
        __syncwarp();
      }
      S nrm = 0;
      for (int i = lane; i < n; i += 32) nrm += Z[(size_t)i * nwant + jv] * Z[(size_t)i * nwant + jv];
      nrm = warp_allsum(nrm);
      const S sc = nrm > (S)0 ? (S)1 / sqrt(nrm) : (S)0;
      for (int i = lane; i < n; i += 32) Z[(size_t)i * nwant + jv] *= sc;
      __syncwarp();
    }
  }
  __syncthreads();
  if constexpr (sizeof(S) == 8) {
    // FP64 eigenvalues: Rayleigh quotients z^T T z; inside a cluster the Rayleigh-Ritz of T on the cluster's
    // vectors (one warp per cluster; the small symmetric problem by cyclic Jacobi on lane 0; its matrices
    // use the dead L D L^T storage at offset k0 n, which clusters starting at different k0 cannot overlap)
    for (int k0 = warp; k0 < nwant; k0 += nw) {
      if (cl[k0] != k0) continue;
      int k1 = k0 + 1;
      while (k1 < nwant && cl[k1] == k0) ++k1;
      const int kc = k1 - k0;
      S* Tc = Dv + (size_t)k0 * n;
      S* Yc = Lv + (size_t)k0 * n;
      for (int a = 0; a < kc; ++a)
        for (int b = a; b < kc; ++b) {
          S acc = 0;
          for (int i = lane; i < n; i += 32) {
            S tz = d[i] * Z[(size_t)i * nwant + k0 + b];
            if (i > 0) tz += e[i - 1] * Z[(size_t)(i - 1) * nwant + k0 + b];
            if (i < n - 1) tz += e[i] * Z[(size_t)(i + 1) * nwant + k0 + b];
            acc += Z[(size_t)i * nwant + k0 + a] * tz;
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
        for (int b = 0; b < kc; ++b) zrow[b] = Z[(size_t)i * nwant + k0 + b];
        for (int a = 0; a < kc; ++a) {
          S acc = 0;
          for (int b = 0; b < kc; ++b) acc += zrow[b] * Yc[b * kc + a];
          Z[(size_t)i * nwant + k0 + a] = acc;
        }
      }
      __syncwarp();
    }
    __syncthreads();
  }
  // step 4: u_k = H_0 (H_1 (... H_{n-2} z_k)), one warp per eigenvector
  for (int k = warp; k < nwant; k += nw) {
    for (int i = lane; i < n; i += 32) U[(size_t)i * ldu + k] = mk<S>(Z[(size_t)i * nwant + k], 0);
    __syncwarp();
    for (int j = n - 2; j >= 0; --j) {
      const cplx<S> tj = tau[j];
      if (tj.re == (S)0 && tj.im == (S)0) continue;
      const cplx<S>* vcol = A + (size_t)(j + 1) * lda + j;
      const int L = n - 1 - j;
      cplx<S> dot = mk<S>(0, 0);
      for (int i = lane; i < L; i += 32) cfmac(dot, vcol[(size_t)i * lda], U[(size_t)(j + 1 + i) * ldu + k]);
      dot.re = warp_allsum(dot.re);
      dot.im = warp_allsum(dot.im);
      const cplx<S> f = cmul(tj, dot);
      for (int i = lane; i < L; i += 32) {
        const cplx<S> v = vcol[(size_t)i * lda];
        cplx<S>& u = U[(size_t)(j + 1 + i) * ldu + k];
        u.re -= f.re * v.re - f.im * v.im;
        u.im -= f.re * v.im + f.im * v.re;
      }
      __syncwarp();
    }
  }
  __syncthreads();
}

}  // namespace wtb
