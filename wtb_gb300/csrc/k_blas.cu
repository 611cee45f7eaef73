// Tall-skinny block kernels and small dense eigen-decompositions for the block eigensolver.
//
// Block vectors are dim x ncol, row-major with leading dimension ld, in the iteration precision S
// (float or double).  Reductions over dim run in two fixed-order passes (per-CTA partials, then one
// CTA sums them), so repeated runs give identical bits.  Small matrices (<= 112 x 112, the projected
// problems of the Rayleigh-Ritz step) are complex(8) in global memory; their eigen-decomposition runs in
// one CTA by cyclic Jacobi in precision S.
#include <algorithm>

#include "small_eig.cuh"
#include "wtb_internal.h"

namespace wtb {

namespace {

// ----------------------------------------------------------------------------- gram: out = A^H B
constexpr int kGramTile = 16;

template <class S, int TI>
__global__ void __launch_bounds__(256) gram_partial_kernel(const cplx<S>* __restrict__ A, int lda, int p,
                                                           const cplx<S>* __restrict__ B, int ldb, int q, int nrow,
                                                           double* __restrict__ partial, int rows_per_part) {
  // the p x q output is covered by a 16 x 16 thread grid with TI x TI entries per thread (16 TI >= p, q)
  constexpr int RT = 8;  // rows of A/B staged per step
  constexpr int W = 16 * TI;
  __shared__ cplx<S> As[RT][W];
  __shared__ cplx<S> Bs[RT][W];
  const int tid = threadIdx.x, tx = tid % kGramTile, ty = tid / kGramTile;
  const long r_begin = (long)blockIdx.x * rows_per_part;
  const long r_end = min((long)nrow, r_begin + rows_per_part);
  cplx<S> acc[TI][TI];
#pragma unroll
  for (int a = 0; a < TI; ++a)
#pragma unroll
    for (int b = 0; b < TI; ++b) acc[a][b] = mk<S>(0, 0);
  for (long r0 = r_begin; r0 < r_end; r0 += RT) {
    for (int e = tid; e < RT * W; e += 256) {
      const int rr = e / W, c = e % W;
      const long gr = r0 + rr;
      As[rr][c] = (gr < r_end && c < p) ? A[gr * lda + c] : mk<S>(0, 0);
      Bs[rr][c] = (gr < r_end && c < q) ? B[gr * ldb + c] : mk<S>(0, 0);
    }
    __syncthreads();
    for (int rr = 0; rr < RT; ++rr) {
      cplx<S> a[TI], b[TI];
#pragma unroll
      for (int i = 0; i < TI; ++i) a[i] = As[rr][ty + kGramTile * i];
#pragma unroll
      for (int j = 0; j < TI; ++j) b[j] = Bs[rr][tx + kGramTile * j];
#pragma unroll
      for (int i = 0; i < TI; ++i)
#pragma unroll
        for (int j = 0; j < TI; ++j) cfmac(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
  double* out = partial + (size_t)blockIdx.x * p * q * 2;
#pragma unroll
  for (int i = 0; i < TI; ++i)
#pragma unroll
    for (int j = 0; j < TI; ++j) {
      const int ii = ty + kGramTile * i, jj = tx + kGramTile * j;
      if (ii < p && jj < q) {
        out[2 * (ii * q + jj)] = (double)acc[i][j].re;
        out[2 * (ii * q + jj) + 1] = (double)acc[i][j].im;
      }
    }
}

// out[e] = sum over b of partial[b][e]: a CTA owns 32 consecutive e; its 8 warps take every 8th part
// (lane = e, so reads coalesce), then the 8 warp sums are added in a fixed order.
__global__ void __launch_bounds__(256) sum_partials_kernel(const double* __restrict__ partial, int npart, int n,
                                                           double* __restrict__ out) {
  __shared__ double red[8][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int e = blockIdx.x * 32 + lane;
  double s = 0.0;
  if (e < n)
    for (int b = warp; b < npart; b += 8) s += partial[(size_t)b * n + e];
  red[warp][lane] = s;
  __syncthreads();
  if (warp == 0 && e < n) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w][lane];
    out[e] = t;
  }
}

// ----------------------------------------------------------------------------- update: Out = beta Out + S C
template <class S>
__global__ void __launch_bounds__(256) update_kernel(const cplx<S>* __restrict__ Sx, int lds, int nin,
                                                     const zd* __restrict__ C, int ldc, int nout, int nrow,
                                                     cplx<S>* __restrict__ Out, int ldo, S alpha, S beta) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<S>* Cs = reinterpret_cast<cplx<S>*>(smem_raw);  // nin x nout
  const int tid = threadIdx.x;
  for (int e = tid; e < nin * nout; e += blockDim.x) {
    const int i = e / nout, j = e % nout;
    const zd c = C[(size_t)i * ldc + j];
    Cs[e] = mk<S>((S)c.re, (S)c.im);
  }
  __syncthreads();
  const int rows_per_blk = blockDim.x / nout;
  const int rr = tid / nout, j = tid % nout;
  if (rr >= rows_per_blk) return;
  for (long r = (long)blockIdx.x * rows_per_blk + rr; r < nrow; r += (long)gridDim.x * rows_per_blk) {
    cplx<S> acc = mk<S>(0, 0);
    const cplx<S>* srow = Sx + r * lds;
    for (int i = 0; i < nin; ++i) cfma(acc, srow[i], Cs[i * nout + j]);
    acc.re *= alpha;
    acc.im *= alpha;
    cplx<S>* o = Out + r * ldo + j;
    if (beta != (S)0) {
      const cplx<S> old = *o;
      acc.re += beta * old.re;
      acc.im += beta * old.im;
    }
    *o = acc;
  }
}

// ----------------------------------------------------------------------------- residual and preconditioner
template <class S>
__global__ void __launch_bounds__(256) residual_kernel(const cplx<S>* __restrict__ AX, int ldax,
                                                       const cplx<S>* __restrict__ X, int ldx,
                                                       const double* __restrict__ theta, int m, int nrow,
                                                       cplx<S>* __restrict__ R, int ldr, double* __restrict__ partial) {
  __shared__ double red[8][32];
  const int tid = threadIdx.x;
  const int j = tid % 32, rr = tid / 32;  // 8 rows per step, up to 32 columns
  // a thread's few dozen rows are summed in S (FP64 instructions are scarce on this GPU), the partial sums
  // in FP64
  S acc = 0;
  if (j < m) {
    const S th = (S)theta[j];
    for (long r = (long)blockIdx.x * 8 + rr; r < nrow; r += (long)gridDim.x * 8) {
      const cplx<S> ax = AX[r * ldax + j], x = X[r * ldx + j];
      const cplx<S> v = mk<S>(ax.re - th * x.re, ax.im - th * x.im);
      R[r * ldr + j] = v;
      acc += v.re * v.re + v.im * v.im;
    }
  }
  red[rr][j] = (double)acc;
  __syncthreads();
  if (rr == 0) {
    double s = 0.0;
    for (int i = 0; i < 8; ++i) s += red[i][j];
    partial[(size_t)blockIdx.x * 32 + j] = s;
  }
}

template <class S>
__global__ void precond_kernel(cplx<S>* __restrict__ R, int ldr, const double* __restrict__ diag,
                               const double* __restrict__ theta, const int* __restrict__ active, int m, int nrow) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)nrow * m) return;
  const long r = e / m;
  const int j = (int)(e % m);
  cplx<S>& v = R[r * ldr + j];
  if (!active[j]) {
    v = mk<S>(0, 0);
    return;
  }
  const S th = (S)theta[j];
  S d = (S)diag[r] - th;
  const S fl = (S)1e-2 * (fabs(th) > (S)1e-3 ? fabs(th) : (S)1e-3);
  if (fabs(d) < fl) d = fl;
  const S inv = (S)1 / fabs(d);
  v = mk<S>(v.re * inv, v.im * inv);
}

template <class Sa, class Sb>
__global__ void convert_cols_kernel(const cplx<Sa>* __restrict__ A, int lda, cplx<Sb>* __restrict__ B, int ldb,
                                    int ncol, int nrow) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)nrow * ncol) return;
  const long r = e / ncol;
  const int j = (int)(e % ncol);
  const cplx<Sa> a = A[r * lda + j];
  B[r * ldb + j] = mk<Sb>((Sb)a.re, (Sb)a.im);
}

// ----------------------------------------------------------------------------- small Jacobi eigensolver
__device__ __forceinline__ int rr_player(int i, int t, int n) { return i == 0 ? 0 : ((i - 1 + t) % (n - 1)) + 1; }


// ----------------------------------------------------------------------------- small helpers
// C = op(A) B for the small projected matrices (complex(8) storage), in arithmetic T: FP32 when the projected
// problem is solved in FP32 (FP64 instructions are scarce on this GPU), FP64 for the final FP64 step
template <class T>
__global__ void small_gemm_kernel(const zd* __restrict__ A, int lda, int transA, const zd* __restrict__ B, int ldb,
                                  zd* __restrict__ C, int ldc, int m, int n, int k) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * n) return;
  const int i = e / n, j = e % n;
  cplx<T> acc = mk<T>(0, 0);
  for (int l = 0; l < k; ++l) {
    const zd a = transA ? A[(size_t)l * lda + i] : A[(size_t)i * lda + l];
    const zd b = B[(size_t)l * ldb + j];
    const cplx<T> at = mk<T>((T)a.re, (T)a.im), bt = mk<T>((T)b.re, (T)b.im);
    if (transA)
      cfmac(acc, at, bt);
    else
      cfma(acc, at, bt);
  }
  C[(size_t)i * ldc + j] = mk<double>((double)acc.re, (double)acc.im);
}

__device__ __forceinline__ double hash_noise(unsigned a, unsigned b, unsigned seed) {
  unsigned h = a * 2654435761u ^ (b + 0x9e3779b9u + (seed << 6) + (seed >> 2));
  h ^= h >> 16;
  h *= 0x7feb352du;
  h ^= h >> 15;
  h *= 0x846ca68bu;
  h ^= h >> 16;
  return (double)h / 4294967296.0 - 0.5;
}

// X0 = unit vectors at the m smallest diagonal entries (lowest transition energies) plus a small
// deterministic perturbation.  Selection in two levels: each CTA takes the m smallest of its slice by
// repeated arg-min (ties to the lower index), then one CTA repeats that over the CTAs' candidates.
__global__ void __launch_bounds__(256) select_lowest_kernel(const double* __restrict__ val, const int* __restrict__ ids,
                                                            int count, int m, double* __restrict__ out_val,
                                                            int* __restrict__ out_idx) {
  __shared__ double bv[256];
  __shared__ int bi[256];
  __shared__ int chosen[128];
  const int tid = threadIdx.x;
  const int per = (count + gridDim.x - 1) / gridDim.x;
  const int r0 = blockIdx.x * per, r1 = min(count, r0 + per);
  for (int s = 0; s < m; ++s) {
    double best = 1e300;
    int besti = 0x7fffffff;
    for (int r = r0 + tid; r < r1; r += blockDim.x) {
      const int id = ids ? ids[r] : r;
      if (id < 0) continue;
      bool used = false;
      for (int t = 0; t < s; ++t) used |= (chosen[t] == id);
      if (used) continue;
      const double d = val[r];
      if (d < best || (d == best && id < besti)) {
        best = d;
        besti = id;
      }
    }
    bv[tid] = best;
    bi[tid] = besti;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
      if (tid < off) {
        const double o = bv[tid + off];
        const int oi = bi[tid + off];
        if (o < bv[tid] || (o == bv[tid] && oi < bi[tid])) {
          bv[tid] = o;
          bi[tid] = oi;
        }
      }
      __syncthreads();
    }
    if (tid == 0) {
      chosen[s] = bi[0];
      out_val[blockIdx.x * m + s] = bv[0];
      out_idx[blockIdx.x * m + s] = bi[0] == 0x7fffffff ? -1 : bi[0];
    }
    __syncthreads();
  }
}

template <class S>
__global__ void init_guess_kernel(cplx<S>* X, int ldx, int dim, int m, const int* __restrict__ idx, unsigned seed) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)dim * m) return;
  const long r = e / m;
  const int j = (int)(e % m);
  double re = 1e-3 * hash_noise((unsigned)r, (unsigned)j, seed);
  double im = 1e-3 * hash_noise((unsigned)r, (unsigned)j + 7919u, seed);
  if (idx[j] == r) re += 1.0;
  X[r * ldx + j] = mk<S>((S)re, (S)im);
}

// Lowest nwant eigenpairs of the Hermitian part of the leading n x n block of Ag (n = *nptr if nptr, capped
// at nmax), in precision S, by the tridiagonal route of small_eig.cuh.  evals[k] ascending; evecs (nmax rows,
// leading dimension ldv): column k for k < min(nwant, n); rows >= n and the columns of missing eigenpairs
// are zero, and a missing eigenvalue is 1e30 (a direction the orthonormalisation dropped).
template <class S>
__global__ void __launch_bounds__(256) heev_small_kernel(const zd* __restrict__ Ag, int lda, const int* __restrict__ nptr,
                                                         int nmax, int nwant, double* __restrict__ evals,
                                                         zd* __restrict__ evecs, int ldv) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = nptr ? min(max(*nptr, 0), nmax) : nmax;
  const int nw = min(nwant, n);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lds = n + 1;
  cplx<S>* A = reinterpret_cast<cplx<S>*>(smem_raw);
  cplx<S>* p = A + (size_t)n * lds;
  cplx<S>* tau = p + nmax;
  S* d = reinterpret_cast<S*>(tau + nmax);
  S* e = d + nmax;
  S* e2 = e + nmax;
  S* lam = e2 + nmax;
  S* red = lam + nmax;
  S* Z = red + 4;
  S* Dv = Z + (size_t)nmax * nwant;
  S* Lv = Dv + (size_t)nmax * nwant;
  int* cl = reinterpret_cast<int*>(Lv + (size_t)nmax * nwant);
  int* flag = cl + nwant;
  for (int q = tid; q < n * n; q += nt) {
    const int r = q / n, c = q % n;
    const zd a = Ag[(size_t)r * lda + c], b = Ag[(size_t)c * lda + r];
    A[(size_t)r * lds + c] = mk<S>((S)(0.5 * (a.re + b.re)), r == c ? (S)0 : (S)(0.5 * (a.im - b.im)));
  }
  __syncthreads();
  if (n > 0) {
    tridiag_cta<S>(A, lds, n, d, e, tau, p, flag);
    cplx<S>* U = reinterpret_cast<cplx<S>*>(Dv);
    tridiag_eigvecs_cta<S>(A, lds, n, nw, d, e, tau, e2, lam, Z, Dv, Lv, cl, U, nw > 0 ? nw : 1, red);
    for (int q = tid; q < nmax * nwant; q += nt) {
      const int r = q / nwant, k = q % nwant;
      zd v = mk<double>(0.0, 0.0);
      if (r < n && k < nw) {
        const cplx<S> u = U[(size_t)r * nw + k];
        v = mk<double>((double)u.re, (double)u.im);
      }
      evecs[(size_t)r * ldv + k] = v;
    }
    for (int k = tid; k < nwant; k += nt) evals[k] = k < nw ? (double)lam[k] : 1e30;
  } else {
    for (int q = tid; q < nmax * nwant; q += nt) evecs[(size_t)(q / nwant) * ldv + q % nwant] = mk<double>(0.0, 0.0);
    for (int k = tid; k < nwant; k += nt) evals[k] = 1e30;
  }
}

// Orthonormalising basis of the Gram matrix M = S^H S (n x n, complex(8)) by Cholesky in precision S, in the
// basis's own order ([X W P]: the current block first) with deflation: with D = diag(M) and
// Ms = D^-1/2 M D^-1/2, column k is kept when its residual diagonal (its squared distance from the span of the
// kept columns before it) exceeds drop, and dropped otherwise.  For the r kept columns P, Ms[P,P] = R^H R and
// B = D_P^-1/2 R^-1 makes S B orthonormal.  B (n x n, leading dimension ldb) holds those r columns first and
// zeros elsewhere; *r_out = r.  Two barriers a step; the CTA is a 16 x 16 thread grid over the trailing matrix.
template <class S>
__global__ void __launch_bounds__(256) pchol_basis_kernel(const zd* __restrict__ Mg, int ldm, int n, double drop,
                                                          zd* __restrict__ B, int ldb, int* __restrict__ r_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, nt = blockDim.x, tx = tid & 15, ty = tid >> 4;
  const int lds = n + 1;
  cplx<S>* W = reinterpret_cast<cplx<S>*>(smem_raw);  // residual matrix
  cplx<S>* R = W + (size_t)n * lds;                    // R[k][column], rows in kept order
  S* dinv = reinterpret_cast<S*>(R + (size_t)n * lds);
  int* perm = reinterpret_cast<int*>(dinv + n);
  __shared__ int s_r;
  for (int i = tid; i < n; i += nt) {
    const double m = Mg[(size_t)i * ldm + i].re;
    dinv[i] = m > 1e-300 ? (S)(1.0 / sqrt(m)) : (S)0;
  }
  __syncthreads();
  for (int i = ty; i < n; i += 16)
    for (int j = tx; j < n; j += 16) {
      const zd a = Mg[(size_t)i * ldm + j], b = Mg[(size_t)j * ldm + i];
      const S sc = dinv[i] * dinv[j];
      W[(size_t)i * lds + j] = mk<S>((S)(0.5 * (a.re + b.re)) * sc, i == j ? (S)0 : (S)(0.5 * (a.im - b.im)) * sc);
    }
  __syncthreads();
  int r = 0;  // kept so far (uniform across the block)
  for (int k = 0; k < n; ++k) {
    const S dk = W[(size_t)k * lds + k].re;
    if (!(dk > (S)drop)) continue;  // uniform decision: every thread reads the same settled value
    const S rkk = sqrt(dk), irk = (S)1 / rkk;
    // row r of R: columns k+1.. of the residual row k, scaled
    for (int j = tid; j < n; j += nt) {
      cplx<S> v = mk<S>(0, 0);
      if (j == k)
        v = mk<S>(rkk, 0);
      else if (j > k)
        v = mk<S>(W[(size_t)k * lds + j].re * irk, W[(size_t)k * lds + j].im * irk);
      R[(size_t)r * lds + j] = v;
    }
    if (tid == 0) perm[r] = k;
    __syncthreads();
    // Schur complement on the trailing block: W[i][j] -= conj(R[r][i]) R[r][j]
    for (int i = k + 1 + ty; i < n; i += 16) {
      const cplx<S> ri = R[(size_t)r * lds + i];
      for (int j = k + 1 + tx; j < n; j += 16) {
        const cplx<S> rj = R[(size_t)r * lds + j];
        cplx<S>& w = W[(size_t)i * lds + j];
        w.re -= ri.re * rj.re + ri.im * rj.im;
        w.im -= ri.re * rj.im - ri.im * rj.re;
      }
    }
    ++r;
    __syncthreads();
  }
  if (tid == 0) s_r = r;
  __syncthreads();
  // R^-1 (r x r, upper triangular in kept order), one thread per column c, stored over W's rows
  cplx<S>* Ri = W;
  for (int c = tid; c < r; c += nt) {
    for (int k = c + 1; k < r; ++k) Ri[(size_t)k * lds + c] = mk<S>(0, 0);
    Ri[(size_t)c * lds + c] = mk<S>((S)1 / R[(size_t)c * lds + perm[c]].re, 0);
    for (int k = c - 1; k >= 0; --k) {
      cplx<S> acc = mk<S>(0, 0);
      for (int l = k + 1; l <= c; ++l) cfma(acc, R[(size_t)k * lds + perm[l]], Ri[(size_t)l * lds + c]);
      const S irkk = (S)1 / R[(size_t)k * lds + perm[k]].re;
      Ri[(size_t)k * lds + c] = mk<S>(-acc.re * irkk, -acc.im * irkk);
    }
  }
  __syncthreads();
  // B[perm[k]][c] = dinv[perm[k]] Ri[k][c] (k <= c < r); everything else zero
  for (int i = ty; i < n; i += 16)
    for (int c = tx; c < n; c += 16) B[(size_t)i * ldb + c] = mk<double>(0.0, 0.0);
  __syncthreads();
  for (int k = ty; k < r; k += 16)
    for (int c = tx; c < r; c += 16) {
      if (k > c) continue;
      const int i = perm[k];
      const cplx<S> v = Ri[(size_t)k * lds + c];
      B[(size_t)i * ldb + c] = mk<double>((double)v.re * (double)dinv[i], (double)v.im * (double)dinv[i]);
    }
  if (tid == 0) *r_out = s_r;
}

}  // namespace

// ----------------------------------------------------------------------------- launchers
template <class S>
cudaError_t launch_gram(const cplx<S>* A, int lda, int p, const cplx<S>* B, int ldb, int q, int nrow, zd* out,
                        double* partial, int npart, cudaStream_t s) {
  if (p > 96 || q > 96) return cudaErrorInvalidValue;
  const int rpp = (nrow + npart - 1) / npart;
  const int ti = (std::max(p, q) + 15) / 16;
  switch (ti) {
    case 1: gram_partial_kernel<S, 1><<<npart, 256, 0, s>>>(A, lda, p, B, ldb, q, nrow, partial, rpp); break;
    case 2: gram_partial_kernel<S, 2><<<npart, 256, 0, s>>>(A, lda, p, B, ldb, q, nrow, partial, rpp); break;
    case 3: gram_partial_kernel<S, 3><<<npart, 256, 0, s>>>(A, lda, p, B, ldb, q, nrow, partial, rpp); break;
    case 4: gram_partial_kernel<S, 4><<<npart, 256, 0, s>>>(A, lda, p, B, ldb, q, nrow, partial, rpp); break;
    case 5: gram_partial_kernel<S, 5><<<npart, 256, 0, s>>>(A, lda, p, B, ldb, q, nrow, partial, rpp); break;
    default: gram_partial_kernel<S, 6><<<npart, 256, 0, s>>>(A, lda, p, B, ldb, q, nrow, partial, rpp); break;
  }
  ++g_launch_count;
  const int n = p * q * 2;
  sum_partials_kernel<<<(n + 31) / 32, 256, 0, s>>>(partial, npart, n, reinterpret_cast<double*>(out)); ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_update(const cplx<S>* Sx, int lds, int nin, const zd* C, int ldc, int nout, int nrow,
                          cplx<S>* Out, int ldo, double alpha, double beta, cudaStream_t s) {
  if (nout > 256 || nin * nout > 8192) return cudaErrorInvalidValue;
  const size_t smem = (size_t)nin * nout * sizeof(cplx<S>);
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(update_kernel<S>), (size_t)smem);
  if (e != cudaSuccess) return e;
  const int rows_per_blk = 256 / nout;
  long nblk = (nrow + rows_per_blk - 1) / rows_per_blk;
  if (nblk > 152 * 16) nblk = 152 * 16;
  update_kernel<S><<<(unsigned)nblk, 256, smem, s>>>(Sx, lds, nin, C, ldc, nout, nrow, Out, ldo, (S)alpha,
                                                     (S)beta); ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_residual(const cplx<S>* AX, int ldax, const cplx<S>* X, int ldx, const double* theta, int m,
                            int nrow, cplx<S>* R, int ldr, double* partial, int npart, double* norms2,
                            cudaStream_t s) {
  if (m > 32) return cudaErrorInvalidValue;
  residual_kernel<S><<<npart, 256, 0, s>>>(AX, ldax, X, ldx, theta, m, nrow, R, ldr, partial); ++g_launch_count;
  // partial is [npart][32]; sum column-wise
  sum_partials_kernel<<<1, 256, 0, s>>>(partial, npart, 32, norms2); ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_precond(cplx<S>* R, int ldr, const double* diag, const double* theta, const int* active, int m,
                           int nrow, cudaStream_t s) {
  const long n = (long)nrow * m;
  precond_kernel<S><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(R, ldr, diag, theta, active, m, nrow); ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_copy_cols(const cplx<S>* A, int lda, cplx<S>* B, int ldb, int ncol, int nrow, cudaStream_t s) {
  const long n = (long)nrow * ncol;
  convert_cols_kernel<S, S><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(A, lda, B, ldb, ncol, nrow); ++g_launch_count;
  return cudaGetLastError();
}

template <class Sa, class Sb>
cudaError_t launch_convert_cols(const cplx<Sa>* A, int lda, cplx<Sb>* B, int ldb, int ncol, int nrow,
                                cudaStream_t s) {
  const long n = (long)nrow * ncol;
  convert_cols_kernel<Sa, Sb><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(A, lda, B, ldb, ncol, nrow); ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_heev_small(const zd* A, int lda, const int* nptr, int nmax, int nwant, double* evals, zd* evecs,
                              int ldv, cudaStream_t s) {
  if (nmax < 1 || nmax > 96 || nwant < 0 || nwant > nmax) return cudaErrorInvalidValue;
  const size_t smem = (size_t)nmax * (nmax + 1) * sizeof(cplx<S>) + (size_t)2 * nmax * sizeof(cplx<S>) +
                      (size_t)(4 * nmax + 4) * sizeof(S) + (size_t)3 * nmax * nwant * sizeof(S) +
                      (size_t)(nwant + 4) * sizeof(int) + 64;
  if (smem > 220 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(heev_small_kernel<S>), smem);
  if (e != cudaSuccess) return e;
  heev_small_kernel<S><<<1, 256, smem, s>>>(A, lda, nptr, nmax, nwant, evals, evecs, ldv); ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_pchol_basis(const zd* M, int ldm, int n, double drop, zd* B, int ldb, int* r_out, cudaStream_t s) {
  if (n < 1 || n > 96) return cudaErrorInvalidValue;
  const size_t smem = (size_t)2 * n * (n + 1) * sizeof(cplx<S>) + (size_t)n * sizeof(S) + (size_t)n * sizeof(int) + 64;
  if (smem > 220 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(pchol_basis_kernel<S>), smem);
  if (e != cudaSuccess) return e;
  pchol_basis_kernel<S><<<1, 256, smem, s>>>(M, ldm, n, drop, B, ldb, r_out); ++g_launch_count;
  return cudaGetLastError();
}

template cudaError_t launch_heev_small<float>(const zd*, int, const int*, int, int, double*, zd*, int, cudaStream_t);
template cudaError_t launch_heev_small<double>(const zd*, int, const int*, int, int, double*, zd*, int, cudaStream_t);
template cudaError_t launch_pchol_basis<float>(const zd*, int, int, double, zd*, int, int*, cudaStream_t);
template cudaError_t launch_pchol_basis<double>(const zd*, int, int, double, zd*, int, int*, cudaStream_t);

cudaError_t launch_small_gemm(const zd* A, int lda, int transA, const zd* B, int ldb, zd* C, int ldc, int m, int n,
                              int k, cudaStream_t s, bool fp32) {
  if (fp32)
    small_gemm_kernel<float><<<(m * n + 127) / 128, 128, 0, s>>>(A, lda, transA, B, ldb, C, ldc, m, n, k);
  else
    small_gemm_kernel<double><<<(m * n + 127) / 128, 128, 0, s>>>(A, lda, transA, B, ldb, C, ldc, m, n, k);
  ++g_launch_count;
  return cudaGetLastError();
}

// idx needs room for 64 * m + m ints (candidates then the result), idx[64 m .. 64 m + m) holds the answer.
cudaError_t launch_select_lowest(const double* diag, int dim, int m, int* idx, double* cand_val, cudaStream_t s) {
  if (m > 128) return cudaErrorInvalidValue;
  const int g = std::max(1, std::min(64, (dim + 1023) / 1024));
  select_lowest_kernel<<<g, 256, 0, s>>>(diag, nullptr, dim, m, cand_val, idx); ++g_launch_count;
  select_lowest_kernel<<<1, 256, 0, s>>>(cand_val, idx, g * m, m, cand_val + 64 * m, idx + 64 * m); ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_init_guess(cplx<S>* X, int ldx, int dim, int m, const int* idx, unsigned seed, cudaStream_t s) {
  const long n = (long)dim * m;
  init_guess_kernel<S><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(X, ldx, dim, m, idx, seed); ++g_launch_count;
  return cudaGetLastError();
}

#define WTB_INST_BLAS(S)                                                                                          \
  template cudaError_t launch_gram<S>(const cplx<S>*, int, int, const cplx<S>*, int, int, int, zd*, double*, int,  \
                                      cudaStream_t);                                                              \
  template cudaError_t launch_update<S>(const cplx<S>*, int, int, const zd*, int, int, int, cplx<S>*, int, double, \
                                        double, cudaStream_t);                                                    \
  template cudaError_t launch_residual<S>(const cplx<S>*, int, const cplx<S>*, int, const double*, int, int,       \
                                          cplx<S>*, int, double*, int, double*, cudaStream_t);                    \
  template cudaError_t launch_precond<S>(cplx<S>*, int, const double*, const double*, const int*, int, int,        \
                                         cudaStream_t);                                                           \
  template cudaError_t launch_copy_cols<S>(const cplx<S>*, int, cplx<S>*, int, int, int, cudaStream_t);           \
  template cudaError_t launch_init_guess<S>(cplx<S>*, int, int, int, const int*, unsigned, cudaStream_t);
WTB_INST_BLAS(float)
WTB_INST_BLAS(double)
template cudaError_t launch_convert_cols<float, double>(const cplx<float>*, int, cplx<double>*, int, int, int,
                                                       cudaStream_t);
template cudaError_t launch_convert_cols<double, float>(const cplx<double>*, int, cplx<float>*, int, int, int,
                                                       cudaStream_t);
template cudaError_t launch_convert_cols<double, double>(const cplx<double>*, int, cplx<double>*, int, int, int,
                                                        cudaStream_t);

}  // namespace wtb
