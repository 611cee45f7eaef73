// Tall-skinny block kernels and small dense eigen-decompositions for the block eigensolver.
//
// Block vectors are dim x ncol, row-major with leading dimension ld, in the iteration precision S
// (float or double).  Reductions over dim run in two fixed-order passes (per-CTA partials, then one
// CTA sums them), so repeated runs give identical bits.  Small matrices (<= 112 x 112, the projected
// problems of the Rayleigh-Ritz step) are complex(8) in global memory; their eigen-decomposition runs in
// one CTA by cyclic Jacobi in precision S.
#include <algorithm>

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
  double acc = 0.0;
  if (j < m) {
    const S th = (S)theta[j];
    for (long r = (long)blockIdx.x * 8 + rr; r < nrow; r += (long)gridDim.x * 8) {
      const cplx<S> ax = AX[r * ldax + j], x = X[r * ldx + j];
      const cplx<S> v = mk<S>(ax.re - th * x.re, ax.im - th * x.im);
      R[r * ldr + j] = v;
      acc += (double)v.re * (double)v.re + (double)v.im * (double)v.im;
    }
  }
  red[rr][j] = acc;
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
  const double th = theta[j];
  double d = diag[r] - th;
  const double fl = 1e-2 * fmax(fabs(th), 1e-3);
  if (fabs(d) < fl) d = fl;
  const S inv = (S)(1.0 / fabs(d));
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

// One CTA; each warp owns rotation pairs j = warp, warp + nwarps, ... of the round-robin step.  Its lanes
// walk the n columns (row update) and then the n rows (column update) of that pair, so no thread does
// integer division in the inner loops; rotation parameters stay in registers between the two phases,
// and a step needs two block barriers.
template <class S>
__global__ void __launch_bounds__(512) jacobi_small_kernel(zd* A, int lda, int nin, double* evals, zd* evecs,
                                                           int ldv, int max_sweeps, DevStatus* st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int kMaxPairsPerWarp = 4;  // half <= 64 pairs over 16 warps
  const int n = (nin + 1) & ~1;
  const int half = n / 2;
  // leading dimension n + 1: a column walk then strides 2(n+1) words and spreads over the banks
  const int ldm = n + 1;
  cplx<S>* M = reinterpret_cast<cplx<S>*>(smem_raw);
  cplx<S>* Vv = M + n * ldm;
  double* ev = reinterpret_cast<double*>(Vv + n * ldm);
  int* rank = reinterpret_cast<int*>(ev + 128);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int warp = tid >> 5, lane = tid & 31, nwarps = nt >> 5;
  for (int e = tid; e < n * n; e += nt) {
    const int r = e / n, c = e % n;
    cplx<S> v = mk<S>(0, 0);
    if (r < nin && c < nin) {
      // Hermitian part of the input
      const zd a = A[(size_t)r * lda + c], b = A[(size_t)c * lda + r];
      v = mk<S>((S)(0.5 * (a.re + b.re)), (S)(0.5 * (a.im - b.im)));
      if (r == c) v.im = 0;
    }
    M[r * ldm + c] = v;
    Vv[r * ldm + c] = mk<S>(r == c ? (S)1 : (S)0, 0);
  }
  __syncthreads();
  const S tiny = sizeof(S) == 4 ? (S)1e-30 : (S)1e-300;
  // classical per-pair criterion |a_pq| <= eps sqrt(|a_pp a_qq|): independent of the scale of other
  // entries (dropped directions carry a large marker on the diagonal)
  // or |a_pq| <= eps_abs * scale, scale = largest unmarked diagonal magnitude (the rounding floor of the
  // rotations, which the relative test cannot reach for eigenvalues far below the norm)
  const double eps2 = sizeof(S) == 4 ? 1e-12 : 1e-30;
  const double epsa = sizeof(S) == 4 ? 4e-7 : 4e-16;
  __shared__ int notconv;
  __shared__ unsigned long long s_scale;
  __shared__ double s_off;
  if (tid == 0) s_scale = 0ull;
  __syncthreads();
  for (int i = tid; i < nin; i += nt) {
    const double d = fabs((double)M[i * ldm + i].re);
    if (d < 1e29) atomicMax(&s_scale, (unsigned long long)__double_as_longlong(d));  // non-negative doubles order as integers
  }
  __syncthreads();
  const double scale = __longlong_as_double((long long)s_scale);
  const double floor2 = (epsa * scale) * (epsa * scale);
  // Jacobi converges quadratically; once a sweep no longer shrinks the off-diagonal mass and that mass
  // is at the rounding floor, the sweep loop stops as well
  const double noise = (sizeof(S) == 4 ? 1e-6 : 1e-14) * scale;
  double prev_off = 1e300;
  int sweeps_done = 0;
  for (int sweep = 0; sweep < max_sweeps; ++sweep, ++sweeps_done) {
    if (tid == 0) {
      notconv = 0;
      s_off = 0.0;
    }
    __syncthreads();
    int mine = 0;
    double off = 0.0;
    for (int e = tid; e < n * n; e += nt) {
      const int r = e / n, c = e % n;
      if (r == c) continue;
      const cplx<S> me = M[r * ldm + c];
      const double m2 = (double)me.re * me.re + (double)me.im * me.im;
      const double dd = fabs((double)M[r * ldm + r].re * (double)M[c * ldm + c].re);
      off += m2;
      if (m2 > eps2 * dd && m2 > floor2 && m2 > 1e-280) mine = 1;
    }
    if (mine) atomicOr(&notconv, 1);
    for (int o = 16; o > 0; o >>= 1) off += __shfl_xor_sync(0xffffffffu, off, o);
    if (lane == 0) atomicAdd(&s_off, off);
    __syncthreads();
    const int nc = notconv;
    const double offn = s_off;
    if (!nc) break;
    if (sweep >= 2 && offn > 0.25 * prev_off && offn <= noise * noise * (double)n * n) break;
    prev_off = offn;
    if (sizeof(S) == 8 && sweep == max_sweeps - 1 && tid == 0) dev_fail(st, 201, n);
    for (int t = 0; t < n - 1; ++t) {
      __syncthreads();
      int pp[kMaxPairsPerWarp], qq[kMaxPairsPerWarp];
      S cc[kMaxPairsPerWarp], ss[kMaxPairsPerWarp];
      cplx<S> ph[kMaxPairsPerWarp];
      bool act[kMaxPairsPerWarp];
#pragma unroll
      for (int k = 0; k < kMaxPairsPerWarp; ++k) {
        const int j = warp + k * nwarps;
        act[k] = false;
        if (j >= half) continue;
        // round-robin (circle) pairing of step t: position i holds player (i - 1 + t) mod (n - 1) + 1
        int p = j == 0 ? 0 : ((j - 1 + t) % (n - 1)) + 1;
        int q = ((n - 2 - j + t) % (n - 1)) + 1;
        if (p > q) {
          const int tmp = p;
          p = q;
          q = tmp;
        }
        pp[k] = p;
        qq[k] = q;
        const cplx<S> apq = M[p * ldm + q];
        const S app = M[p * ldm + p].re, aqq = M[q * ldm + q].re;
        const S b = sqrt(apq.re * apq.re + apq.im * apq.im);
        if (b > tiny) {
          ph[k] = mk<S>(apq.re / b, apq.im / b);
          const S zeta = (aqq - app) / (2 * b);
          S tt;
          if (fabs(zeta) > (S)1e15)
            tt = (S)0.5 / zeta;
          else
            tt = (zeta >= 0 ? (S)1 : (S)-1) / (fabs(zeta) + sqrt((S)1 + zeta * zeta));
          cc[k] = (S)1 / sqrt((S)1 + tt * tt);
          ss[k] = tt * cc[k];
          act[k] = true;
        }
      }
      __syncwarp();
      // rows: A_p. <- c A_p. - s e^{i phi} A_q. ; A_q. <- s A_p. + c e^{i phi} A_q.
#pragma unroll
      for (int k = 0; k < kMaxPairsPerWarp; ++k) {
        if (!act[k]) continue;
        const int p = pp[k], q = qq[k];
        const S c = cc[k], s = ss[k];
        for (int col = lane; col < n; col += 32) {
          const cplx<S> ap = M[p * ldm + col], aq = M[q * ldm + col];
          const cplx<S> phq = cmul(ph[k], aq);
          M[p * ldm + col] = mk<S>(c * ap.re - s * phq.re, c * ap.im - s * phq.im);
          M[q * ldm + col] = mk<S>(s * ap.re + c * phq.re, s * ap.im + c * phq.im);
        }
      }
      __syncthreads();
      // columns of A and V: A_.p <- c A_.p - s e^{-i phi} A_.q ; A_.q <- s A_.p + c e^{-i phi} A_.q
#pragma unroll
      for (int k = 0; k < kMaxPairsPerWarp; ++k) {
        if (!act[k]) continue;
        const int p = pp[k], q = qq[k];
        const S c = cc[k], s = ss[k];
        const cplx<S> phc = mk<S>(ph[k].re, -ph[k].im);
        for (int row = lane; row < n; row += 32) {
          cplx<S> ap = M[row * ldm + p], aq = M[row * ldm + q];
          cplx<S> phq = cmul(phc, aq);
          M[row * ldm + p] = mk<S>(c * ap.re - s * phq.re, c * ap.im - s * phq.im);
          M[row * ldm + q] = mk<S>(s * ap.re + c * phq.re, s * ap.im + c * phq.im);
          ap = Vv[row * ldm + p];
          aq = Vv[row * ldm + q];
          phq = cmul(phc, aq);
          Vv[row * ldm + p] = mk<S>(c * ap.re - s * phq.re, c * ap.im - s * phq.im);
          Vv[row * ldm + q] = mk<S>(s * ap.re + c * phq.re, s * ap.im + c * phq.im);
        }
        __syncwarp();
        if (lane == 0) {
          M[p * ldm + q] = mk<S>(0, 0);
          M[q * ldm + p] = mk<S>(0, 0);
          M[p * ldm + p].im = 0;
          M[q * ldm + q].im = 0;
        }
      }
    }
    __syncthreads();
  }
  __syncthreads();
  if (tid == 0) {
    atomicAdd(&st->small_sweeps, sweeps_done);
    atomicAdd(&st->small_calls, 1);
  }
  if (tid < nin) ev[tid] = (double)M[tid * ldm + tid].re;
  __syncthreads();
  if (tid < nin) {
    int r = 0;
    const double x = ev[tid];
    for (int j = 0; j < nin; ++j) r += (ev[j] < x) || (ev[j] == x && j < tid);
    rank[tid] = r;
  }
  __syncthreads();
  if (tid < nin) evals[rank[tid]] = ev[tid];
  for (int e = tid; e < nin * nin; e += nt) {
    const int row = e / nin, j = e % nin;
    const cplx<S> v = Vv[row * ldm + j];
    evecs[(size_t)row * ldv + rank[j]] = mk<double>((double)v.re, (double)v.im);
  }
}

// ----------------------------------------------------------------------------- small helpers
__global__ void small_gemm_kernel(const zd* __restrict__ A, int lda, int transA, const zd* __restrict__ B, int ldb,
                                  zd* __restrict__ C, int ldc, int m, int n, int k) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * n) return;
  const int i = e / n, j = e % n;
  zd acc = mk<double>(0.0, 0.0);
  for (int l = 0; l < k; ++l) {
    if (transA)
      cfmac(acc, A[(size_t)l * lda + i], B[(size_t)l * ldb + j]);
    else
      cfma(acc, A[(size_t)i * lda + l], B[(size_t)l * ldb + j]);
  }
  C[(size_t)i * ldc + j] = acc;
}

__global__ void svqb_scale_kernel(const zd* __restrict__ M, int ldm, int n, double* dinv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d = M[(size_t)i * ldm + i].re;
  dinv[i] = d > 1e-300 ? 1.0 / sqrt(d) : 0.0;
}

__global__ void scale_sym_kernel(zd* M, int ldm, int n, const double* __restrict__ dinv) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * n) return;
  const int i = e / n, j = e % n;
  M[(size_t)i * ldm + j] = cscale(M[(size_t)i * ldm + j], dinv[i] * dinv[j]);
}

// B[:, j] = dinv .* U[:, j] / sqrt(lam_j) for lam_j > tau * lam_max; dropped columns are zero and
// flagged by a negative entry in rank_flags[j] (consumed by mark_dropped_kernel).
__global__ void svqb_basis_kernel(const double* __restrict__ dinv, const zd* __restrict__ U, int ldu,
                                  const double* __restrict__ lam, int n, double tau, zd* __restrict__ B, int ldb,
                                  int* keep) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * n) return;
  const int i = e / n, j = e % n;
  const double lmax = lam[n - 1];
  const bool k = lam[j] > tau * lmax && lam[j] > 0.0;
  if (i == 0) keep[j] = k ? 1 : 0;
  B[(size_t)i * ldb + j] = k ? cscale(U[(size_t)i * ldu + j], dinv[i] / sqrt(lam[j])) : mk<double>(0.0, 0.0);
}

__global__ void mark_dropped_kernel(zd* G, int ldg, int n, const int* __restrict__ keep) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * n) return;
  const int i = e / n, j = e % n;
  if (!keep[i] || !keep[j]) G[(size_t)i * ldg + j] = mk<double>(i == j ? 1e30 : 0.0, 0.0);
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
static cudaError_t jacobi_launch(zd* A, int lda, int n, double* evals, zd* evecs, int ldv, int sweeps,
                                 DevStatus* st, cudaStream_t s) {
  const int np = (n + 1) & ~1;
  if (np / 2 > 64) return cudaErrorInvalidValue;
  const size_t smem = (size_t)2 * np * (np + 1) * sizeof(cplx<S>) + 128 * sizeof(double) + 128 * sizeof(int) + 64;
  if (smem > 220 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(jacobi_small_kernel<S>), (size_t)smem);
  if (e != cudaSuccess) return e;
  jacobi_small_kernel<S><<<1, 512, smem, s>>>(A, lda, n, evals, evecs, ldv, sweeps, st); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_jacobi_eig(zd* A, int lda, int n, double* evals, zd* evecs, int ldv, int sweeps, DevStatus* st,
                              cudaStream_t s) {
  return jacobi_launch<double>(A, lda, n, evals, evecs, ldv, sweeps, st, s);
}

cudaError_t launch_jacobi_eig_f32(zd* A, int lda, int n, double* evals, zd* evecs, int ldv, int sweeps,
                                  DevStatus* st, cudaStream_t s) {
  return jacobi_launch<float>(A, lda, n, evals, evecs, ldv, sweeps, st, s);
}

cudaError_t launch_small_gemm(const zd* A, int lda, int transA, const zd* B, int ldb, zd* C, int ldc, int m, int n,
                              int k, cudaStream_t s) {
  small_gemm_kernel<<<(m * n + 127) / 128, 128, 0, s>>>(A, lda, transA, B, ldb, C, ldc, m, n, k); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_svqb_scale(const zd* M, int ldm, int n, double* dinv, cudaStream_t s) {
  svqb_scale_kernel<<<1, 128, 0, s>>>(M, ldm, n, dinv); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_scale_sym(zd* M, int ldm, int n, const double* dinv, cudaStream_t s) {
  scale_sym_kernel<<<(n * n + 255) / 256, 256, 0, s>>>(M, ldm, n, dinv); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_svqb_basis(const double* dinv, const zd* U, int ldu, const double* lam, int n, double tau, zd* B,
                              int ldb, int* keep, cudaStream_t s) {
  svqb_basis_kernel<<<(n * n + 255) / 256, 256, 0, s>>>(dinv, U, ldu, lam, n, tau, B, ldb, keep); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_mark_dropped(zd* G, int ldg, int n, const int* keep, cudaStream_t s) {
  mark_dropped_kernel<<<(n * n + 255) / 256, 256, 0, s>>>(G, ldg, n, keep); ++g_launch_count;
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
