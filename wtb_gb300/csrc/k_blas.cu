// Tall-skinny block kernels and small dense eigen-decompositions for the block eigensolver.
//
// Block vectors are dim x ncol, row-major with leading dimension ld, in the iteration precision S
// (float or double).  Reductions over dim run in two fixed-order passes (per-part partials, then one
// CTA per system sums them), so repeated runs give identical bits.  Small matrices (<= 96 x 96, the projected
// problems of the Rayleigh-Ritz step) are complex(8) in global memory; their eigen-decomposition runs in
// one CTA per system (small_eig.cuh).  Every kernel takes a BatchMap: one system, or a ragged batch of
// independent systems in one concatenated row space.
#include <algorithm>

#include "small_eig.cuh"
#include "wtb_internal.h"

namespace wtb {

namespace {

// ----------------------------------------------------------------------------- gram: out = A^H B
constexpr int kGramTile = 16;

template <int BYTES>
__device__ __forceinline__ void cp_async_elem(void* dst, const void* src) {
  static_assert(BYTES == 8 || BYTES == 16, "cp.async copies 4, 8 or 16 bytes");
  if constexpr (BYTES == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
  else
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}

template <class S, int TI>
__global__ void __launch_bounds__(256) gram_partial_kernel(const cplx<S>* __restrict__ A, int lda, int p,
                                                           const cplx<S>* __restrict__ B, int ldb, int q, int nrow,
                                                           double* __restrict__ partial, int rows_per_part,
                                                           BatchMap bm) {
  // the p x q output is covered by a 16 x 16 thread grid with TI x TI entries per thread (16 TI >= p, q);
  // one CTA per reduction part.  Rows are staged by cp.async, two stages of RT rows deep (both stages of both
  // operands within 33 KB of static shared memory), so the next stage's loads are in flight while the current
  // one is multiplied; each thread adds the rows in order, one running sum per entry.
  constexpr int W = 16 * TI;
  constexpr int RT = (sizeof(S) == 4 ? 2 : 1) * (W <= 32 ? 16 : W <= 64 ? 8 : 4);
  __shared__ cplx<S> As[2][RT][W];
  __shared__ cplx<S> Bs[2][RT][W];
  const int tid = threadIdx.x, tx = tid % kGramTile, ty = tid / kGramTile;
  long r_begin, r_end;
  const int sys = bm_part(bm, blockIdx.x, nrow, rows_per_part, &r_begin, &r_end);
  if (bm_frozen(bm, sys)) return;
  // columns past p (A) and q (B) are never copied: zero them in both stages once
  for (int e = tid; e < 2 * RT * W; e += 256) {
    if (e % W >= p) (&As[0][0][0])[e] = mk<S>(0, 0);
    if (e % W >= q) (&Bs[0][0][0])[e] = mk<S>(0, 0);
  }
  auto stage = [&](int buf, long r0) {
    const int nr = (int)min((long)RT, r_end - r0);
    for (int e = tid; e < nr * W; e += 256) {
      const int rr = e / W, c = e - rr * W;
      if (c < p) cp_async_elem<sizeof(cplx<S>)>(&As[buf][rr][c], A + (r0 + rr) * lda + c);
      if (c < q) cp_async_elem<sizeof(cplx<S>)>(&Bs[buf][rr][c], B + (r0 + rr) * ldb + c);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  cplx<S> acc[TI][TI];
#pragma unroll
  for (int a = 0; a < TI; ++a)
#pragma unroll
    for (int b = 0; b < TI; ++b) acc[a][b] = mk<S>(0, 0);
  const long nst = (r_end - r_begin + RT - 1) / RT;
  if (nst > 0) stage(0, r_begin);
  for (long t = 0; t < nst; ++t) {
    const int buf = (int)(t & 1);
    if (t + 1 < nst) {
      stage(buf ^ 1, r_begin + (t + 1) * RT);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();
    const int nr = (int)min((long)RT, r_end - (r_begin + t * RT));
    for (int rr = 0; rr < nr; ++rr) {
      cplx<S> a[TI], b[TI];
#pragma unroll
      for (int i = 0; i < TI; ++i) a[i] = As[buf][rr][ty + kGramTile * i];
#pragma unroll
      for (int j = 0; j < TI; ++j) b[j] = Bs[buf][rr][tx + kGramTile * j];
#pragma unroll
      for (int i = 0; i < TI; ++i)
#pragma unroll
        for (int j = 0; j < TI; ++j) cfmac(acc[i][j], a[i], b[j]);
    }
    __syncthreads();  // the next stage's copies overwrite this buffer
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

// M = A^H A and G = A^H B in one pass over the rows (the Gram pair of the Rayleigh-Ritz step): every staged row of
// A feeds both products, so A is read once, and a thread's 3 x 3 entries of both matrices take 9 shared-memory
// loads per row for 72 multiply-adds.  Rows are staged 32 (FP32) or 8 (FP64) at a time, two stages deep, by
// cp.async (one copy per element, so any leading dimension works): the loads of the next stage are in flight while
// the current one is multiplied.  Each thread adds the rows in the order of gram_partial_kernel, so the sums are
// bitwise the same as two separate launches.  One CTA per reduction part; partials [part][p][p] of M, then of G at
// partial + npart p p 2.  (Measured and rejected: the complex multiply-adds as packed fma.rn.f32x2 pairs, bitwise
// the same sums with half the FMA instructions, took 58.8 us against 52.5 (the pair packing costs more than it
// saves); and thread-block clusters of 6 parts adding their FP64 partials
// through distributed shared memory before writing.  Clusters must fit inside one GPC, which left room for 288
// of the 300 CTAs at a time, and the second wave took the Gram pair from 52.6 to 92.0 us.)

template <class S, int TI>
__global__ void __launch_bounds__(256) gram_pair_partial_kernel(const cplx<S>* __restrict__ A,
                                                                const cplx<S>* __restrict__ B, int ld, int p,
                                                                int nrow, double* __restrict__ partial,
                                                                int rows_per_part, int npart, BatchMap bm) {
  constexpr int W = 16 * TI;
  // rows per stage: both stages of both operands within 48 KB of static shared memory
  constexpr int kPairRows = sizeof(S) == 4 ? 32 : 8;
  __shared__ cplx<S> As[2][kPairRows][W];
  __shared__ cplx<S> Bs[2][kPairRows][W];
  const int tid = threadIdx.x, tx = tid % kGramTile, ty = tid / kGramTile;
  long r_begin, r_end;
  const int sys = bm_part(bm, blockIdx.x, nrow, rows_per_part, &r_begin, &r_end);
  if (bm_frozen(bm, sys)) return;
  // columns p .. W - 1 are never copied: zero them in both stages once
  for (int e = tid; e < 2 * kPairRows * W; e += 256) {
    if (e % W >= p) {
      (&As[0][0][0])[e] = mk<S>(0, 0);
      (&Bs[0][0][0])[e] = mk<S>(0, 0);
    }
  }
  const int rr0 = tid / p, c0 = tid - rr0 * p, drr = 256 / p, dc = 256 - drr * p;  // stride 256 in (row, column)
  auto stage = [&](int buf, long r0) {
    const int nr = (int)min((long)kPairRows, r_end - r0);
    int rr = rr0, c = c0;
    for (int e = tid; e < nr * p; e += 256) {
      cp_async_elem<sizeof(cplx<S>)>(&As[buf][rr][c], A + (r0 + rr) * ld + c);
      cp_async_elem<sizeof(cplx<S>)>(&Bs[buf][rr][c], B + (r0 + rr) * ld + c);
      rr += drr;
      c += dc;
      if (c >= p) {
        c -= p;
        ++rr;
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  cplx<S> am[TI][TI], ag[TI][TI];
#pragma unroll
  for (int i = 0; i < TI; ++i)
#pragma unroll
    for (int j = 0; j < TI; ++j) am[i][j] = ag[i][j] = mk<S>(0, 0);
  const long nst = (r_end - r_begin + kPairRows - 1) / kPairRows;
  if (nst > 0) stage(0, r_begin);
  for (long t = 0; t < nst; ++t) {
    const int buf = (int)(t & 1);
    if (t + 1 < nst) {
      stage(buf ^ 1, r_begin + (t + 1) * kPairRows);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();
    const int nr = (int)min((long)kPairRows, r_end - (r_begin + t * kPairRows));
    for (int rr = 0; rr < nr; ++rr) {
      cplx<S> a[TI], b[TI], c[TI];
#pragma unroll
      for (int i = 0; i < TI; ++i) a[i] = As[buf][rr][ty + kGramTile * i];
#pragma unroll
      for (int j = 0; j < TI; ++j) {
        b[j] = As[buf][rr][tx + kGramTile * j];
        c[j] = Bs[buf][rr][tx + kGramTile * j];
      }
#pragma unroll
      for (int i = 0; i < TI; ++i)
#pragma unroll
        for (int j = 0; j < TI; ++j) {
          cfmac(am[i][j], a[i], b[j]);
          cfmac(ag[i][j], a[i], c[j]);
        }
    }
    __syncthreads();  // the next stage's copies overwrite this buffer
  }
  const size_t n = (size_t)p * p * 2;
  double* om = partial + (size_t)blockIdx.x * n;
  double* og = partial + ((size_t)npart + blockIdx.x) * n;
#pragma unroll
  for (int i = 0; i < TI; ++i)
#pragma unroll
    for (int j = 0; j < TI; ++j) {
      const int ii = ty + kGramTile * i, jj = tx + kGramTile * j;
      if (ii < p && jj < p) {
        om[2 * (ii * p + jj)] = (double)am[i][j].re;
        om[2 * (ii * p + jj) + 1] = (double)am[i][j].im;
        og[2 * (ii * p + jj)] = (double)ag[i][j].re;
        og[2 * (ii * p + jj) + 1] = (double)ag[i][j].im;
      }
    }
}

// The Gram pair for 33..48 FP32 columns over the upper triangle only (M and G are Hermitian: the lower triangle is
// the conjugate, written by sum_partials_herm_kernel).  The 48 x 48 matrices are 16 x 16 blocks of 3 x 3; thread
// t < 136 owns upper block t (block row a <= block column b) of both, so a staged row costs it the same 9
// shared-memory loads and 18 complex multiply-adds as in gram_pair_partial_kernel, with about half the work.  Its
// entries are added in the same row order with the same operand roles, so they are bitwise the entries of
// gram_pair_partial_kernel.  160 threads a CTA; the partials are [part][136][9] complex of M, then of G at
// partial + npart * kHermN.
constexpr int kHermBlocks = 136;            // 3 x 3 blocks on and above the diagonal of a 48 x 48 matrix
constexpr int kHermN = kHermBlocks * 18;    // doubles per part and matrix
constexpr int kHermThreads = 160;

__device__ __forceinline__ void herm_block(int t, int& a, int& b) {
  int r = 0;
  while (t >= 16 - r) {
    t -= 16 - r;
    ++r;
  }
  a = r;
  b = r + t;
}

__global__ void __launch_bounds__(kHermThreads) gram_pair_upper_kernel(const zf* __restrict__ A,
                                                                       const zf* __restrict__ B, int ld, int p,
                                                                       int nrow, double* __restrict__ partial,
                                                                       int rows_per_part, int npart, BatchMap bm) {
  constexpr int W = 48, kRows = 32;
  __shared__ zf As[2][kRows][W];
  __shared__ zf Bs[2][kRows][W];
  const int tid = threadIdx.x;
  long r_begin, r_end;
  const int sys = bm_part(bm, blockIdx.x, nrow, rows_per_part, &r_begin, &r_end);
  if (bm_frozen(bm, sys)) return;
  for (int e = tid; e < 2 * kRows * W; e += kHermThreads) {
    if (e % W >= p) {
      (&As[0][0][0])[e] = mk<float>(0.f, 0.f);
      (&Bs[0][0][0])[e] = mk<float>(0.f, 0.f);
    }
  }
  const int rr0 = tid / p, c0 = tid - rr0 * p, drr = kHermThreads / p, dc = kHermThreads - drr * p;
  auto stage = [&](int buf, long r0) {
    const int nr = (int)min((long)kRows, r_end - r0);
    int rr = rr0, c = c0;
    for (int e = tid; e < nr * p; e += kHermThreads) {
      cp_async_elem<sizeof(zf)>(&As[buf][rr][c], A + (r0 + rr) * ld + c);
      cp_async_elem<sizeof(zf)>(&Bs[buf][rr][c], B + (r0 + rr) * ld + c);
      rr += drr;
      c += dc;
      if (c >= p) {
        c -= p;
        ++rr;
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  const bool worker = tid < kHermBlocks;
  int ba = 0, bb = 0;
  if (worker) herm_block(tid, ba, bb);
  const int i0 = 3 * ba, j0 = 3 * bb;
  zf am[3][3], ag[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) am[i][j] = ag[i][j] = mk<float>(0.f, 0.f);
  const long nst = (r_end - r_begin + kRows - 1) / kRows;
  if (nst > 0) stage(0, r_begin);
  for (long t = 0; t < nst; ++t) {
    const int buf = (int)(t & 1);
    if (t + 1 < nst) {
      stage(buf ^ 1, r_begin + (t + 1) * kRows);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();
    if (worker) {
      const int nr = (int)min((long)kRows, r_end - (r_begin + t * kRows));
      for (int rr = 0; rr < nr; ++rr) {
        zf a[3], b[3], c[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) a[i] = As[buf][rr][i0 + i];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          b[j] = As[buf][rr][j0 + j];
          c[j] = Bs[buf][rr][j0 + j];
        }
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            cfmac(am[i][j], a[i], b[j]);
            cfmac(ag[i][j], a[i], c[j]);
          }
      }
    }
    __syncthreads();  // the next stage's copies overwrite this buffer
  }
  if (!worker) return;
  double* om = partial + (size_t)blockIdx.x * kHermN + tid * 18;
  double* og = partial + ((size_t)npart + blockIdx.x) * kHermN + tid * 18;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      om[2 * (3 * i + j)] = (double)am[i][j].re;
      om[2 * (3 * i + j) + 1] = (double)am[i][j].im;
      og[2 * (3 * i + j)] = (double)ag[i][j].re;
      og[2 * (3 * i + j) + 1] = (double)ag[i][j].im;
    }
}

// Sums the upper-block partials of gram_pair_upper_kernel over the parts (sum_parts_cta; blockIdx.z = 1: the G set)
// and writes the p x p matrix: the entries on and above the diagonal, and their conjugates below it.
__global__ void __launch_bounds__(256) sum_partials_herm_kernel(const double* __restrict__ partial, int npart, int p,
                                                                double* __restrict__ outM, double* __restrict__ outG,
                                                                BatchMap bm, long out_stride) {
  __shared__ double red[8][33];
  const int e = blockIdx.x * 32 + (threadIdx.x & 31);
  const int sys = blockIdx.y;
  double* out = outM;
  if (blockIdx.z == 1) {
    partial += (size_t)npart * kHermN;
    out = outG;
  }
  if (bm_frozen(bm, sys)) return;
  const double t = sum_parts_cta(partial, npart, kHermN, e, sys, bm, red);
  if (threadIdx.x < 32 && e < kHermN) {
    const int blk = e / 18, w = e - 18 * blk, ij = w >> 1, im = w & 1;
    int ba, bb;
    herm_block(blk, ba, bb);
    const int ii = 3 * ba + ij / 3, jj = 3 * bb + ij % 3;
    if (ii <= jj && jj < p) {  // the strictly lower entries of the diagonal blocks come from their mirrors
      out += (size_t)sys * out_stride;
      out[2 * (ii * p + jj) + im] = t;
      if (ii != jj) out[2 * (jj * p + ii) + im] = im ? -t : t;
    }
  }
}

// out[e] = sum over b of partial[b][e] over the parts of system blockIdx.y (out at a stride of out_stride per
// system): a CTA owns 32 consecutive e (sum_parts_cta).
// With out2: blockIdx.z = 1 sums the second set of partials (npart parts further on) into out2.
__global__ void __launch_bounds__(256) sum_partials_kernel(const double* __restrict__ partial, int npart, int n,
                                                           double* __restrict__ out, BatchMap bm, long out_stride,
                                                           double* __restrict__ out2 = nullptr) {
  __shared__ double red[8][33];
  const int e = blockIdx.x * 32 + (threadIdx.x & 31);
  const int sys = blockIdx.y;
  if (blockIdx.z == 1) {
    partial += (size_t)npart * n;
    out = out2;
  }
  if (bm_frozen(bm, sys)) return;
  const double t = sum_parts_cta(partial, npart, n, e, sys, bm, red);
  if (threadIdx.x < 32 && e < n) out[(size_t)sys * out_stride + e] = t;
}

// ----------------------------------------------------------------------------- update: Out = beta Out + S C
// Row tiles of kTileRows rows, tile-strided over the grid; C of the tile's system is staged in shared memory
// (again only when the system changes from one tile to the next).
template <class S>
__global__ void __launch_bounds__(256) update_kernel(const cplx<S>* __restrict__ Sx, int lds, int nin,
                                                     const zd* __restrict__ C, int ldc, int nout, int nrow,
                                                     cplx<S>* __restrict__ Out, int ldo, S alpha, S beta,
                                                     BatchMap bm, long c_stride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<S>* Cs = reinterpret_cast<cplx<S>*>(smem_raw);  // nin x nout
  const int tid = threadIdx.x;
  const int rows_per_blk = blockDim.x / nout;
  const int rr = tid / nout, j = tid % nout;
  const long ntile = ((long)nrow + kTileRows - 1) / kTileRows;
  int staged = -1;
  for (long t = blockIdx.x; t < ntile; t += gridDim.x) {
    const int sys = bm_sys_of_row(bm, t * kTileRows);  // uniform over the CTA
    if (bm_frozen(bm, sys)) continue;
    if (sys != staged) {
      __syncthreads();
      const zd* Cq = C + (size_t)sys * c_stride;
      for (int e = tid; e < nin * nout; e += blockDim.x) {
        const int i = e / nout, jj = e % nout;
        const zd c = Cq[(size_t)i * ldc + jj];
        Cs[e] = mk<S>((S)c.re, (S)c.im);
      }
      __syncthreads();
      staged = sys;
    }
    if (rr >= rows_per_blk) continue;
    const long r1 = min((long)nrow, (t + 1) * kTileRows);
    for (long r = t * kTileRows + rr; r < r1; r += rows_per_blk) {
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
}

// The projections of one iteration in one pass: W -= X T_W, P -= X T_P and AP -= AX T_P, with T_W = T[:, 0:m] and
// T_P = T[:, m:2m] of T = X^H [W P] (m x 2m).  A CTA stages a row tile of X and AX and both coefficient blocks in
// shared memory; each output keeps update_kernel's arithmetic (the sum over i in order, then old minus it), so
// the results are bitwise those of three update_kernel launches.
template <class S>
__global__ void __launch_bounds__(256) orth_update_kernel(const cplx<S>* __restrict__ X, const cplx<S>* __restrict__ AX,
                                                          int ld, int m, const zd* __restrict__ T,
                                                          cplx<S>* __restrict__ W, cplx<S>* __restrict__ P,
                                                          cplx<S>* __restrict__ AP, int nrow, BatchMap bm,
                                                          long t_stride, const int* __restrict__ active) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int RS = m + 1;                                // padded row of the staged blocks
  cplx<S>* Tw = reinterpret_cast<cplx<S>*>(smem_raw);  // [m][m]
  cplx<S>* Tp = Tw + m * m;                            // [m][m]
  cplx<S>* Xs = Tp + m * m;                            // [kTileRows][RS]
  cplx<S>* As = Xs + kTileRows * RS;                   // [kTileRows][RS]
  const int tid = threadIdx.x;
  const long ntile = ((long)nrow + kTileRows - 1) / kTileRows;
  int staged = -1;
  for (long t = blockIdx.x; t < ntile; t += gridDim.x) {
    const int sys = bm_sys_of_row(bm, t * kTileRows);  // uniform over the CTA
    if (bm_frozen(bm, sys)) continue;
    __syncthreads();  // the previous tile's reads are done
    if (sys != staged) {
      const zd* Tq = T + (size_t)sys * t_stride;
      for (int e = tid; e < m * m; e += blockDim.x) {
        const int i = e / m, j = e - i * m;
        const zd a = Tq[(size_t)i * 2 * m + j], b = Tq[(size_t)i * 2 * m + m + j];
        Tw[e] = mk<S>((S)a.re, (S)a.im);
        Tp[e] = mk<S>((S)b.re, (S)b.im);
      }
      staged = sys;
    }
    const long r0 = t * kTileRows;
    const int nr = (int)min((long)kTileRows, nrow - r0);
    for (int e = tid; e < nr * m; e += blockDim.x) {
      const int rr = e / m, i = e - rr * m;
      Xs[rr * RS + i] = X[(r0 + rr) * ld + i];
      As[rr * RS + i] = AX[(r0 + rr) * ld + i];
    }
    __syncthreads();
    for (int e = tid; e < nr * m; e += blockDim.x) {
      const int rr = e / m, j = e - rr * m;
      const cplx<S>* xr = Xs + rr * RS;
      const cplx<S>* ar = As + rr * RS;
      cplx<S> aw = mk<S>(0, 0), ap = mk<S>(0, 0), aa = mk<S>(0, 0);
      for (int i = 0; i < m; ++i) {
        const cplx<S> xi = xr[i], tw = Tw[i * m + j], tp = Tp[i * m + j];
        cfma(aw, xi, tw);
        cfma(ap, xi, tp);
        cfma(aa, ar[i], tp);
      }
      const long r = r0 + rr;
      cplx<S>* ow = W + r * ld + j;
      cplx<S>* op = P + r * ld + j;
      cplx<S>* oa = AP + r * ld + j;
      // active: the search direction of a locked column is zero (the preconditioner's mask)
      *ow = active && !active[32 * sys + j] ? mk<S>(0, 0) : mk<S>(ow->re - aw.re, ow->im - aw.im);
      *op = mk<S>(op->re - ap.re, op->im - ap.im);
      *oa = mk<S>(oa->re - aa.re, oa->im - aa.im);
    }
  }
}

// ----------------------------------------------------------------------------- residual and preconditioner
template <class S>
__global__ void __launch_bounds__(256) residual_kernel(const cplx<S>* __restrict__ AX, int ldax,
                                                       const cplx<S>* __restrict__ X, int ldx,
                                                       const double* __restrict__ theta, int m, int nrow,
                                                       cplx<S>* __restrict__ R, int ldr, double* __restrict__ partial,
                                                       int rows_per_part, BatchMap bm, long theta_stride,
                                                       const double* __restrict__ diag) {
  __shared__ double red[8][32];
  const int tid = threadIdx.x;
  const int j = tid % 32, rr = tid / 32;  // 8 rows per step, up to 32 columns; one CTA per reduction part
  long r_begin, r_end;
  const int sys = bm_part(bm, blockIdx.x, nrow, rows_per_part, &r_begin, &r_end);
  if (bm_frozen(bm, sys)) return;
  // a thread's few dozen rows are summed in S (FP64 instructions are scarce on this GPU), the partial sums
  // in FP64
  S acc = 0;
  if (j < m) {
    const S th = (S)theta[(size_t)sys * theta_stride + j];
    // diag: store the preconditioned residual |diag - theta|^-1 (AX - X theta), the denominator floored at
    // 1e-2 max(|theta|, 1e-3) (the diagonal preconditioner of the iteration); the norms are of the residual itself
    const S fl = (S)1e-2 * (fabs(th) > (S)1e-3 ? fabs(th) : (S)1e-3);
    for (long r = r_begin + rr; r < r_end; r += 8) {
      const cplx<S> ax = AX[r * ldax + j], x = X[r * ldx + j];
      const cplx<S> v = mk<S>(ax.re - th * x.re, ax.im - th * x.im);
      if (diag) {
        S d = (S)diag[r] - th;
        if (fabs(d) < fl) d = fl;
        const S inv = (S)1 / fabs(d);
        R[r * ldr + j] = mk<S>(v.re * inv, v.im * inv);
      } else {
        R[r * ldr + j] = v;
      }
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


// ----------------------------------------------------------------------------- small helpers
// C = op(A) B for the small projected matrices (complex(8) storage), in arithmetic T: FP32 when the projected
// problem is solved in FP32 (FP64 instructions are scarce on this GPU), FP64 for the final FP64 step
constexpr int kGemmKS = 8;  // lanes per output element of the small products (K split, shuffle sum)
template <class T>
__global__ void __launch_bounds__(128) small_gemm_kernel(const zd* __restrict__ A, int lda, int transA,
                                                         const zd* __restrict__ B, int ldb, zd* __restrict__ C,
                                                         int ldc, int m, int n, int k, BatchMap bm, long a_stride,
                                                         long b_stride, long c_stride) {
  const int sys = blockIdx.y;  // uniform over the CTA
  if (bm_frozen(bm, sys)) return;
  A += (size_t)sys * a_stride;
  B += (size_t)sys * b_stride;
  C += (size_t)sys * c_stride;
  const int t = threadIdx.x & (kGemmKS - 1);
  const int e = (int)((blockIdx.x * blockDim.x + threadIdx.x) / kGemmKS);
  const bool ok = e < m * n;  // no early return: every lane reaches the shuffles
  const int i = ok ? e / n : 0, j = ok ? e % n : 0;
  cplx<T> acc = mk<T>(0, 0);
  if (ok)
    for (int l = t; l < k; l += kGemmKS) {
      const zd a = transA ? A[(size_t)l * lda + i] : A[(size_t)i * lda + l];
      const zd b = B[(size_t)l * ldb + j];
      const cplx<T> at = mk<T>((T)a.re, (T)a.im), bt = mk<T>((T)b.re, (T)b.im);
      if (transA)
        cfmac(acc, at, bt);
      else
        cfma(acc, at, bt);
    }
#pragma unroll
  for (int o = kGemmKS / 2; o > 0; o >>= 1) {
    acc.re += __shfl_xor_sync(0xffffffffu, acc.re, o);
    acc.im += __shfl_xor_sync(0xffffffffu, acc.im, o);
  }
  if (ok && t == 0) C[(size_t)i * ldc + j] = mk<double>((double)acc.re, (double)acc.im);
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
// deterministic perturbation.  Selection by repeated arg-min over a slice (ties to the lower index): for one
// large system in two levels (each CTA takes the m smallest of its slice, then one CTA repeats that over the
// CTAs' candidates); for a batch one CTA per system over all of its rows.
__device__ void select_m_smallest(const double* __restrict__ val, const int* __restrict__ ids, int r0, int r1, int m,
                                  double* __restrict__ out_val, int* __restrict__ out_idx) {
  __shared__ double bv[256];
  __shared__ int bi[256];
  __shared__ int chosen[128];
  const int tid = threadIdx.x;
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
      out_val[s] = bv[0];
      out_idx[s] = bi[0] == 0x7fffffff ? -1 : bi[0];
    }
    __syncthreads();
  }
}

// The same selection for m <= M: every thread keeps a sorted list of the M smallest (value, index) pairs of its
// rows (registers, insertion by compare-and-swap), then m rounds take the smallest head over the CTA (a warp
// butterfly, then the 8 warp winners) and its owner pops it.  The order is the lexicographic (value, index) order
// of select_m_smallest, so both give the same indices in the same order; 256 threads.  Values are compared as
// order-preserving unsigned keys (sign bit set for x >= 0, all bits flipped for x < 0, -0 taken as +0: the
// floating-point order of non-NaN doubles), integer work instead of FP64 compares.
__device__ __forceinline__ unsigned long long order_key(double x) {
  unsigned long long u = (unsigned long long)__double_as_longlong(x);
  if ((u << 1) == 0ull) u = 0ull;  // -0 == +0
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double key_value(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}
__device__ __forceinline__ bool vi_less(unsigned long long a, int ia, unsigned long long b, int ib) {
  return a < b || (a == b && ia < ib);
}

template <int M>
__device__ void select_m_smallest_lists(const double* __restrict__ val, const int* __restrict__ ids, int r0, int r1,
                                        int m, double* __restrict__ out_val, int* __restrict__ out_idx) {
  constexpr unsigned long long kNone = 0xffffffffffffffffull;  // above every key of a non-NaN double
  __shared__ unsigned long long wv[8];
  __shared__ int wi[8];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  unsigned long long lv[M];
  int li[M];
#pragma unroll
  for (int k = 0; k < M; ++k) {
    lv[k] = kNone;
    li[k] = 0x7fffffff;
  }
  for (int r = r0 + tid; r < r1; r += blockDim.x) {
    const int id = ids ? ids[r] : r;
    if (id < 0) continue;
    const unsigned long long d = order_key(val[r]);
    if (vi_less(d, id, lv[M - 1], li[M - 1])) {
      lv[M - 1] = d;
      li[M - 1] = id;
#pragma unroll
      for (int k = M - 1; k > 0; --k)
        if (vi_less(lv[k], li[k], lv[k - 1], li[k - 1])) {
          const unsigned long long tv = lv[k];
          lv[k] = lv[k - 1];
          lv[k - 1] = tv;
          const int ti = li[k];
          li[k] = li[k - 1];
          li[k - 1] = ti;
        }
    }
  }
  for (int s = 0; s < m; ++s) {
    unsigned long long bv = lv[0];
    int bi = li[0];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (vi_less(ov, oi, bv, bi)) {
        bv = ov;
        bi = oi;
      }
    }
    if (lane == 0) {
      wv[warp] = bv;
      wi[warp] = bi;
    }
    __syncthreads();
    bv = wv[0];
    bi = wi[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      if (vi_less(wv[w], wi[w], bv, bi)) {
        bv = wv[w];
        bi = wi[w];
      }
    if (tid == 0) {
      out_val[s] = bi == 0x7fffffff ? 1e300 : key_value(bv);
      out_idx[s] = bi == 0x7fffffff ? -1 : bi;
    }
    if (bi != 0x7fffffff && li[0] == bi) {  // the owner (indices are distinct) pops its head
#pragma unroll
      for (int k = 0; k < M - 1; ++k) {
        lv[k] = lv[k + 1];
        li[k] = li[k + 1];
      }
      lv[M - 1] = kNone;
      li[M - 1] = 0x7fffffff;
    }
    __syncthreads();  // wv / wi are rewritten next round
  }
}

// m smallest by lists when m <= 32, else by rounds of full scans
__device__ __forceinline__ void select_m_smallest_any(const double* __restrict__ val, const int* __restrict__ ids,
                                                      int r0, int r1, int m, double* __restrict__ out_val,
                                                      int* __restrict__ out_idx) {
  if (m <= 16)
    select_m_smallest_lists<16>(val, ids, r0, r1, m, out_val, out_idx);
  else if (m <= 32)
    select_m_smallest_lists<32>(val, ids, r0, r1, m, out_val, out_idx);
  else
    select_m_smallest(val, ids, r0, r1, m, out_val, out_idx);
}

__global__ void __launch_bounds__(256) select_lowest_kernel(const double* __restrict__ val, const int* __restrict__ ids,
                                                            int count, int m, double* __restrict__ out_val,
                                                            int* __restrict__ out_idx) {
  const int per = (count + gridDim.x - 1) / gridDim.x;
  const int r0 = blockIdx.x * per, r1 = min(count, r0 + per);
  select_m_smallest_any(val, ids, r0, r1, m, out_val + blockIdx.x * m, out_idx + blockIdx.x * m);
}

// batch, first level: CTA (g, q) takes the m smallest of slice g of system q's rows (indices relative to the
// system's first row) into cand_val/cand_idx [q][g][m]
__global__ void __launch_bounds__(256) select_lowest_batch_kernel(const double* __restrict__ diag, BatchMap bm, int m,
                                                                  double* __restrict__ cand_val,
                                                                  int* __restrict__ cand_idx) {
  const int q = blockIdx.y, g = blockIdx.x, ng = gridDim.x;
  const int2 rw = bm.rows[q];
  const int per = (rw.y + ng - 1) / ng;
  const int r0 = min(rw.y, g * per), r1 = min(rw.y, r0 + per);
  const size_t o = ((size_t)q * ng + g) * m;
  select_m_smallest_any(diag + rw.x, nullptr, r0, r1, m, cand_val + o, cand_idx + o);
}

// batch, second level: one CTA per system over its ng * m candidates, into out_idx + idx_stride q
__global__ void __launch_bounds__(256) select_lowest_batch2_kernel(const double* __restrict__ cand_val,
                                                                   const int* __restrict__ cand_idx, int ng, int m,
                                                                   double* __restrict__ out_val,
                                                                   int* __restrict__ out_idx, long idx_stride) {
  const int q = blockIdx.x;
  const size_t o = (size_t)q * ng * m;
  select_m_smallest_any(cand_val + o, cand_idx + o, 0, ng * m, m, out_val + (size_t)q * m,
                        out_idx + (size_t)q * idx_stride);
}

// rows of every system (nrow in all); the noise depends on the row within its system, so a system gets the
// same start in a batch as alone; padding rows are zero
template <class S>
__global__ void init_guess_kernel(cplx<S>* X, int ldx, int nrow, int m, const int* __restrict__ idx, unsigned seed,
                                  BatchMap bm, long idx_stride) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)nrow * m) return;
  const long r = e / m;
  const int j = (int)(e % m);
  const int sys = bm_sys_of_row(bm, r);
  long lr = r;
  if (bm.rows) {
    const int2 rw = bm.rows[sys];
    lr = r - rw.x;
    if (lr >= rw.y) {
      X[r * ldx + j] = mk<S>(0, 0);
      return;
    }
  }
  double re = 1e-3 * hash_noise((unsigned)lr, (unsigned)j, seed);
  double im = 1e-3 * hash_noise((unsigned)lr, (unsigned)j + 7919u, seed);
  if (idx[(size_t)sys * idx_stride + j] == lr) re += 1.0;
  X[r * ldx + j] = mk<S>((S)re, (S)im);
}

// Lowest nwant eigenpairs of the Hermitian part of the leading n x n block of Ag (n = *nptr if nptr, capped
// at nmax), in precision S, by the tridiagonal route of small_eig.cuh.  evals[k] ascending; evecs (nmax rows,
// leading dimension ldv): column k for k < min(nwant, n); rows >= n and the columns of missing eigenpairs
// are zero, and a missing eigenvalue is 1e30 (a direction the orthonormalisation dropped).
template <class S>
__global__ void __launch_bounds__(256) heev_small_kernel(const zd* __restrict__ Ag, int lda, const int* __restrict__ nptr,
                                                         int nmax, int nwant, double* __restrict__ evals,
                                                         zd* __restrict__ evecs, int ldv, BatchMap bm, long a_stride,
                                                         long e_stride, long v_stride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int sys = blockIdx.x;  // one CTA per system
  if (bm_frozen(bm, sys)) return;
  Ag += (size_t)sys * a_stride;
  if (nptr) nptr += sys;
  evals += (size_t)sys * e_stride;
  evecs += (size_t)sys * v_stride;
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
  // Z, Dv, Lv: nwant vectors of stride n + 1 each, regions rounded to an even count (U aliases Dv as complex)
  const size_t zsz = ((size_t)(nmax + 1) * nwant + 1) & ~(size_t)1;
  S* Z = red + 4;
  S* Dv = Z + zsz;
  S* Lv = Dv + zsz;
  int* cl = reinterpret_cast<int*>(Lv + zsz);
#pragma unroll 4
  for (int q = tid; q < n * n; q += nt) {
    const int r = q / n, c = q % n;
    const zd a = Ag[(size_t)r * lda + c], b = Ag[(size_t)c * lda + r];
    A[(size_t)r * lds + c] = mk<S>((S)(0.5 * (a.re + b.re)), r == c ? (S)0 : (S)(0.5 * (a.im - b.im)));
  }
  __syncthreads();
  if (n > 0) {
    tridiag_cta<S>(A, lds, n, d, e, tau, p);
    cplx<S>* U = reinterpret_cast<cplx<S>*>(Dv);
    tridiag_eigvecs_cta<S>(A, lds, n, nw, d, e, tau, e2, lam, Z, Dv, Lv, cl, U, n, red);
    for (int q = tid; q < nmax * nwant; q += nt) {
      const int r = q / nwant, k = q % nwant;
      zd v = mk<double>(0.0, 0.0);
      if (r < n && k < nw) {
        const cplx<S> u = U[(size_t)k * n + r];
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
// zeros elsewhere; *r_out = r.  One barrier a step: the Schur update reads row k of the residual, which that
// step does not write; the CTA is a 16 x 16 thread grid over the trailing matrix.
template <class S>
__global__ void __launch_bounds__(256) pchol_basis_kernel(const zd* __restrict__ Mg, int ldm, int n, double drop,
                                                          zd* __restrict__ B, int ldb, int* __restrict__ r_out,
                                                          BatchMap bm, long m_stride, long b_stride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int sys = blockIdx.x;  // one CTA per system
  if (bm_frozen(bm, sys)) return;
  Mg += (size_t)sys * m_stride;
  B += (size_t)sys * b_stride;
  r_out += sys;
  const int tid = threadIdx.x, nt = blockDim.x, tx = tid & 15, ty = tid >> 4;
  const int lds = n + 1;
  cplx<S>* W = reinterpret_cast<cplx<S>*>(smem_raw);  // residual matrix, then R in kept order
  cplx<S>* R = W + (size_t)n * lds;                    // R[k][column], rows in kept order; then R^-1
  S* dinv = reinterpret_cast<S*>(R + (size_t)n * lds);
  S* rinv = dinv + n;                                  // 1 / R[k][k]
  int* perm = reinterpret_cast<int*>(rinv + n);
  int* iperm = perm + n;                               // kept position of column i, or -1
  cplx<S>* tri_scr = reinterpret_cast<cplx<S>*>((reinterpret_cast<uintptr_t>(iperm + n) + 15) & ~(uintptr_t)15);
  __shared__ int s_r;
  // Ms, 48 x 48 entries per pass: a thread issues all of its (i, j) and (j, i) loads first (the diagonal scales
  // are formed while they are in flight), then scales and symmetrises
  constexpr int kLd = 3;
  for (int i0 = 0; i0 < n; i0 += 16 * kLd)
    for (int j0 = 0; j0 < n; j0 += 16 * kLd) {
      zd av[kLd][kLd], bv[kLd][kLd];
#pragma unroll
      for (int ii = 0; ii < kLd; ++ii)
#pragma unroll
        for (int jj = 0; jj < kLd; ++jj) {
          const int i = i0 + ty + 16 * ii, j = j0 + tx + 16 * jj;
          if (i < n && j < n) {
            av[ii][jj] = Mg[(size_t)i * ldm + j];
            bv[ii][jj] = Mg[(size_t)j * ldm + i];
          }
        }
      if (i0 == 0 && j0 == 0)
        for (int i = tid; i < n; i += nt) {
          const double m = Mg[(size_t)i * ldm + i].re;
          dinv[i] = m > 1e-300 ? (S)(1.0 / sqrt(m)) : (S)0;
        }
      __syncthreads();  // dinv (uniform loop bounds)
#pragma unroll
      for (int ii = 0; ii < kLd; ++ii)
#pragma unroll
        for (int jj = 0; jj < kLd; ++jj) {
          const int i = i0 + ty + 16 * ii, j = j0 + tx + 16 * jj;
          if (i < n && j < n) {
            const zd a = av[ii][jj], b = bv[ii][jj];
            const S sc = dinv[i] * dinv[j];
            W[(size_t)i * lds + j] =
                mk<S>((S)(0.5 * (a.re + b.re)) * sc, i == j ? (S)0 : (S)(0.5 * (a.im - b.im)) * sc);
          }
        }
    }
  __syncthreads();
  int r = 0;  // kept so far (uniform across the block)
  for (int k = 0; k < n; ++k) {
    const S dk = W[(size_t)k * lds + k].re;
    if (!(dk > (S)drop)) {  // uniform decision: every thread reads the same settled value
      if (tid == 0) iperm[k] = -1;
      continue;
    }
    const S rkk = sqrt(dk), irk = (S)1 / rkk, idk = irk * irk;
    const cplx<S>* wk = W + (size_t)k * lds;
    // row r of R: columns k+1.. of the residual row k, scaled
    for (int j = tid; j < n; j += nt) {
      cplx<S> v = mk<S>(0, 0);
      if (j == k)
        v = mk<S>(rkk, 0);
      else if (j > k)
        v = mk<S>(wk[j].re * irk, wk[j].im * irk);
      R[(size_t)r * lds + j] = v;
    }
    if (tid == 0) {
      perm[r] = k;
      iperm[k] = r;
      rinv[r] = irk;
    }
    // Schur complement on the trailing block: W[i][j] -= conj(W[k][i]) W[k][j] / dk (a 16 x 16 thread grid;
    // flattened over the CTA with one element per index step it measured slower: 64K against 53K cycles)
    for (int i = k + 1 + ty; i < n; i += 16) {
      const cplx<S> ri = wk[i];
      const cplx<S> rs = mk<S>(ri.re * idk, ri.im * idk);
      for (int j = k + 1 + tx; j < n; j += 16) {
        const cplx<S> rj = wk[j];
        cplx<S>& w = W[(size_t)i * lds + j];
        w.re -= rs.re * rj.re + rs.im * rj.im;
        w.im -= rs.re * rj.im - rs.im * rj.re;
      }
    }
    ++r;
    __syncthreads();
  }
  if (tid == 0) s_r = r;
  // R in kept order and compact (Rk[k][l] = R[k][perm[l]], l >= k) over the dead residual matrix
  cplx<S>* Rk = W;
  for (int k = ty; k < r; k += 16)
    for (int l = tx; l < r; l += 16) Rk[(size_t)k * lds + l] = l >= k ? R[(size_t)k * lds + perm[l]] : mk<S>(0, 0);
  __syncthreads();
  // R^-1 (r x r upper triangular) over R's rows (dead), by blocks of kTriB: the diagonal blocks by back
  // substitution (one thread per column), then superdiagonal s of blocks at once,
  // Ri[I][J] = -Ri[I][I] sum_{K = I+1..J} Rk[I][K] Ri[K][J], from blocks of lower superdiagonals (two barriers a
  // superdiagonal instead of a dependent chain of r^2/4 products per column).  The sums go to the scratch after
  // perm ((n + 7) / 8 blocks of 8 x 8).
  cplx<S>* Ri = R;
  {
    constexpr int kTriB = 8;
    const int nbk = (r + kTriB - 1) / kTriB;
    for (int e = tid; e < r * r; e += nt) {
      const int k = e / r, c = e - k * r;
      if (k > c) Ri[(size_t)k * lds + c] = mk<S>(0, 0);
    }
    for (int c = tid; c < r; c += nt) {  // diagonal blocks
      const int k0 = (c / kTriB) * kTriB;
      Ri[(size_t)c * lds + c] = mk<S>(rinv[c], 0);
      for (int k = c - 1; k >= k0; --k) {
        const cplx<S>* rk = Rk + (size_t)k * lds;
        cplx<S> a = mk<S>(0, 0);
        for (int l = k + 1; l <= c; ++l) cfma(a, rk[l], Ri[(size_t)l * lds + c]);
        const S ir = rinv[k];
        Ri[(size_t)k * lds + c] = mk<S>(-a.re * ir, -a.im * ir);
      }
    }
    __syncthreads();
    cplx<S>* Tsum = tri_scr;  // [nbk - 1][kTriB][kTriB]
    for (int sd = 1; sd < nbk; ++sd) {
      const int nblk = nbk - sd;  // blocks (I, I + sd)
      for (int e = tid; e < nblk * kTriB * kTriB; e += nt) {
        const int bi = e / (kTriB * kTriB), ij = e - bi * kTriB * kTriB, i = ij / kTriB, j = ij - i * kTriB;
        const int I = bi, J = bi + sd, row = I * kTriB + i, col = J * kTriB + j;
        cplx<S> a = mk<S>(0, 0);
        if (row < r && col < r)
          for (int l = (I + 1) * kTriB; l <= col; ++l) cfma(a, Rk[(size_t)row * lds + l], Ri[(size_t)l * lds + col]);
        Tsum[e] = a;
      }
      __syncthreads();
      for (int e = tid; e < nblk * kTriB * kTriB; e += nt) {
        const int bi = e / (kTriB * kTriB), ij = e - bi * kTriB * kTriB, i = ij / kTriB, j = ij - i * kTriB;
        const int I = bi, J = bi + sd, row = I * kTriB + i, col = J * kTriB + j;
        if (row >= r || col >= r) continue;
        cplx<S> a = mk<S>(0, 0);
        for (int q = i; q < kTriB && I * kTriB + q < r; ++q)
          cfma(a, Ri[(size_t)row * lds + I * kTriB + q], Tsum[bi * kTriB * kTriB + q * kTriB + j]);
        Ri[(size_t)row * lds + col] = mk<S>(-a.re, -a.im);
      }
      __syncthreads();
    }
  }
  // B[perm[k]][c] = dinv[perm[k]] Ri[k][c] (k <= c < r); everything else zero (one pass over B)
  for (int i = ty; i < n; i += 16) {
    const int k = iperm[i];
    const double di = (double)dinv[i];
    for (int c = tx; c < n; c += 16) {
      zd v = mk<double>(0.0, 0.0);
      if (k >= 0 && k <= c && c < r) {
        const cplx<S> x = Ri[(size_t)k * lds + c];
        v = mk<double>((double)x.re * di, (double)x.im * di);
      }
      B[(size_t)i * ldb + c] = v;
    }
  }
  if (tid == 0) *r_out = s_r;
}

}  // namespace

// ----------------------------------------------------------------------------- launchers
// npart: reduction parts (bm.nparts for a batch map with a part table; else equal row ranges)
template <class S>
cudaError_t launch_gram(const cplx<S>* A, int lda, int p, const cplx<S>* B, int ldb, int q, int nrow, zd* out,
                        double* partial, int npart, cudaStream_t s, const BatchMap& bm, long out_stride) {
  if (p > 96 || q > 96) return cudaErrorInvalidValue;
  if (bm.parts) npart = bm.nparts;
  const int rpp = (nrow + npart - 1) / npart;
  const int ti = (std::max(p, q) + 15) / 16;
  switch (ti) {
    case 1: gram_partial_kernel<S, 1><<<npart, 256, 0, s>>>(A, lda, p, B, ldb, q, nrow, partial, rpp, bm); break;
    case 2: gram_partial_kernel<S, 2><<<npart, 256, 0, s>>>(A, lda, p, B, ldb, q, nrow, partial, rpp, bm); break;
    case 3: gram_partial_kernel<S, 3><<<npart, 256, 0, s>>>(A, lda, p, B, ldb, q, nrow, partial, rpp, bm); break;
    case 4: gram_partial_kernel<S, 4><<<npart, 256, 0, s>>>(A, lda, p, B, ldb, q, nrow, partial, rpp, bm); break;
    case 5: gram_partial_kernel<S, 5><<<npart, 256, 0, s>>>(A, lda, p, B, ldb, q, nrow, partial, rpp, bm); break;
    default: gram_partial_kernel<S, 6><<<npart, 256, 0, s>>>(A, lda, p, B, ldb, q, nrow, partial, rpp, bm); break;
  }
  ++g_launch_count;
  const int n = p * q * 2;
  sum_partials_kernel<<<dim3((n + 31) / 32, bm.nsys), 256, 0, s>>>(partial, npart, n, reinterpret_cast<double*>(out),
                                                                    bm, 2 * out_stride);
  ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_gram_pair(const cplx<S>* A, const cplx<S>* B, int ld, int p, int nrow, zd* outM, zd* outG,
                             double* partial, int npart, cudaStream_t s, const BatchMap& bm, long out_stride) {
  if (p > 48) return cudaErrorInvalidValue;
  if (bm.parts) npart = bm.nparts;
  const int rpp = (nrow + npart - 1) / npart;
  if constexpr (sizeof(S) == 4) {
    if (p > 32) {
      // upper triangle only; the reduction writes both
      gram_pair_upper_kernel<<<npart, kHermThreads, 0, s>>>(A, B, ld, p, nrow, partial, rpp, npart, bm);
      ++g_launch_count;
      sum_partials_herm_kernel<<<dim3((kHermN + 31) / 32, bm.nsys, 2), 256, 0, s>>>(
          partial, npart, p, reinterpret_cast<double*>(outM), reinterpret_cast<double*>(outG), bm, 2 * out_stride);
      ++g_launch_count;
      return cudaGetLastError();
    }
  }
  const int ti = (p + 15) / 16;
  switch (ti) {
    case 1: gram_pair_partial_kernel<S, 1><<<npart, 256, 0, s>>>(A, B, ld, p, nrow, partial, rpp, npart, bm); break;
    case 2: gram_pair_partial_kernel<S, 2><<<npart, 256, 0, s>>>(A, B, ld, p, nrow, partial, rpp, npart, bm); break;
    default: gram_pair_partial_kernel<S, 3><<<npart, 256, 0, s>>>(A, B, ld, p, nrow, partial, rpp, npart, bm); break;
  }
  ++g_launch_count;
  const int n = p * p * 2;
  // both sets in one launch (the G partials keep the part numbering, npart parts further on)
  sum_partials_kernel<<<dim3((n + 31) / 32, bm.nsys, 2), 256, 0, s>>>(partial, npart, n,
                                                                       reinterpret_cast<double*>(outM), bm,
                                                                       2 * out_stride, reinterpret_cast<double*>(outG));
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_sum_partials_pair(const double* partial, int npart, int n, zd* outM, zd* outG, cudaStream_t s,
                                     const BatchMap& bm, long out_stride) {
  sum_partials_kernel<<<dim3((n + 31) / 32, bm.nsys, 2), 256, 0, s>>>(partial, npart, n,
                                                                       reinterpret_cast<double*>(outM), bm,
                                                                       2 * out_stride, reinterpret_cast<double*>(outG));
  ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_update(const cplx<S>* Sx, int lds, int nin, const zd* C, int ldc, int nout, int nrow,
                          cplx<S>* Out, int ldo, double alpha, double beta, cudaStream_t s, const BatchMap& bm,
                          long c_stride) {
  if (nout > 256 || nin * nout > 8192) return cudaErrorInvalidValue;
  const size_t smem = (size_t)nin * nout * sizeof(cplx<S>);
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(update_kernel<S>), (size_t)smem);
  if (e != cudaSuccess) return e;
  long nblk = ((long)nrow + kTileRows - 1) / kTileRows;
  if (nblk > 152 * 16) nblk = 152 * 16;
  update_kernel<S><<<(unsigned)nblk, 256, smem, s>>>(Sx, lds, nin, C, ldc, nout, nrow, Out, ldo, (S)alpha, (S)beta,
                                                     bm, c_stride);
  ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_orth_update(const cplx<S>* X, const cplx<S>* AX, int ld, int m, const zd* T, cplx<S>* W,
                               cplx<S>* P, cplx<S>* AP, int nrow, cudaStream_t s, const BatchMap& bm, long t_stride,
                               const int* active) {
  if (m < 1 || m > 32) return cudaErrorInvalidValue;
  const size_t smem = (size_t)(2 * m * m + 2 * kTileRows * (m + 1)) * sizeof(cplx<S>);
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(orth_update_kernel<S>), smem);
  if (e != cudaSuccess) return e;
  long nblk = ((long)nrow + kTileRows - 1) / kTileRows;
  if (nblk > 152 * 16) nblk = 152 * 16;
  orth_update_kernel<S><<<(unsigned)nblk, 256, smem, s>>>(X, AX, ld, m, T, W, P, AP, nrow, bm, t_stride, active);
  ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_residual(const cplx<S>* AX, int ldax, const cplx<S>* X, int ldx, const double* theta, int m,
                            int nrow, cplx<S>* R, int ldr, double* partial, int npart, double* norms2, cudaStream_t s,
                            const BatchMap& bm, long theta_stride, const double* diag, bool sum_parts) {
  if (m > 32) return cudaErrorInvalidValue;
  if (bm.parts) npart = bm.nparts;
  const int rpp = (nrow + npart - 1) / npart;
  residual_kernel<S><<<npart, 256, 0, s>>>(AX, ldax, X, ldx, theta, m, nrow, R, ldr, partial, rpp, bm, theta_stride,
                                           diag);
  ++g_launch_count;
  // partial is [part][32]; summed column-wise per system
  if (sum_parts) {
    sum_partials_kernel<<<dim3(1, bm.nsys), 256, 0, s>>>(partial, npart, 32, norms2, bm, 32);
    ++g_launch_count;
  }
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
                              int ldv, cudaStream_t s, const BatchMap& bm, long a_stride, long e_stride,
                              long v_stride) {
  if (nmax < 1 || nmax > 96 || nwant < 0 || nwant > nmax) return cudaErrorInvalidValue;
  const size_t smem = (size_t)nmax * (nmax + 1) * sizeof(cplx<S>) + (size_t)2 * nmax * sizeof(cplx<S>) +
                      (size_t)(4 * nmax + 4) * sizeof(S) + (size_t)3 * ((nmax + 1) * nwant + 1) * sizeof(S) +
                      (size_t)(nwant + 4) * sizeof(int) + 64;
  if (smem > 220 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(heev_small_kernel<S>), smem);
  if (e != cudaSuccess) return e;
  heev_small_kernel<S><<<bm.nsys, 256, smem, s>>>(A, lda, nptr, nmax, nwant, evals, evecs, ldv, bm, a_stride, e_stride,
                                                  v_stride);
  ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_pchol_basis(const zd* M, int ldm, int n, double drop, zd* B, int ldb, int* r_out, cudaStream_t s,
                               const BatchMap& bm, long m_stride, long b_stride) {
  if (n < 1 || n > 96) return cudaErrorInvalidValue;
  // W, R (n x (n + 1) each), dinv, rinv, perm, iperm, and the triangular inverse's scratch (11 blocks of 8 x 8 for
  // n <= 96)
  const size_t smem = (size_t)2 * n * (n + 1) * sizeof(cplx<S>) + (size_t)2 * n * sizeof(S) +
                      (size_t)2 * n * sizeof(int) + 16 + (size_t)((n + 7) / 8) * 64 * sizeof(cplx<S>) + 64;
  if (smem > 220 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(pchol_basis_kernel<S>), smem);
  if (e != cudaSuccess) return e;
  pchol_basis_kernel<S><<<bm.nsys, 256, smem, s>>>(M, ldm, n, drop, B, ldb, r_out, bm, m_stride, b_stride);
  ++g_launch_count;
  return cudaGetLastError();
}

template cudaError_t launch_heev_small<float>(const zd*, int, const int*, int, int, double*, zd*, int, cudaStream_t,
                                              const BatchMap&, long, long, long);
template cudaError_t launch_heev_small<double>(const zd*, int, const int*, int, int, double*, zd*, int, cudaStream_t,
                                               const BatchMap&, long, long, long);
template cudaError_t launch_pchol_basis<float>(const zd*, int, int, double, zd*, int, int*, cudaStream_t,
                                               const BatchMap&, long, long);
template cudaError_t launch_pchol_basis<double>(const zd*, int, int, double, zd*, int, int*, cudaStream_t,
                                                const BatchMap&, long, long);

cudaError_t launch_small_gemm(const zd* A, int lda, int transA, const zd* B, int ldb, zd* C, int ldc, int m, int n,
                              int k, cudaStream_t s, bool fp32, const BatchMap& bm, long a_stride, long b_stride,
                              long c_stride) {
  const dim3 grid((unsigned)(((long)m * n * kGemmKS + 127) / 128), bm.nsys);
  if (fp32)
    small_gemm_kernel<float><<<grid, 128, 0, s>>>(A, lda, transA, B, ldb, C, ldc, m, n, k, bm, a_stride, b_stride,
                                                  c_stride);
  else
    small_gemm_kernel<double><<<grid, 128, 0, s>>>(A, lda, transA, B, ldb, C, ldc, m, n, k, bm, a_stride, b_stride,
                                                   c_stride);
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

// batch: the m lowest rows of every system, relative indices at idx + idx_stride q; cand_val and cand_idx hold
// kSelSlices * m candidates per system, cand_val m more
cudaError_t launch_select_lowest_batch(const double* diag, const BatchMap& bm, int m, int* idx, long idx_stride,
                                       double* cand_val, int* cand_idx, cudaStream_t s) {
  if (m > 128 || !bm.rows) return cudaErrorInvalidValue;
  select_lowest_batch_kernel<<<dim3(kSelSlices, bm.nsys), 256, 0, s>>>(diag, bm, m, cand_val, cand_idx);
  ++g_launch_count;
  select_lowest_batch2_kernel<<<bm.nsys, 256, 0, s>>>(cand_val, cand_idx, kSelSlices, m,
                                                       cand_val + (size_t)bm.nsys * kSelSlices * m, idx, idx_stride);
  ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_init_guess(cplx<S>* X, int ldx, int nrow, int m, const int* idx, unsigned seed, cudaStream_t s,
                              const BatchMap& bm, long idx_stride) {
  const long n = (long)nrow * m;
  init_guess_kernel<S><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(X, ldx, nrow, m, idx, seed, bm, idx_stride);
  ++g_launch_count;
  return cudaGetLastError();
}

#define WTB_INST_BLAS(S)                                                                                          \
  template cudaError_t launch_gram<S>(const cplx<S>*, int, int, const cplx<S>*, int, int, int, zd*, double*, int,  \
                                      cudaStream_t, const BatchMap&, long);                                       \
  template cudaError_t launch_gram_pair<S>(const cplx<S>*, const cplx<S>*, int, int, int, zd*, zd*, double*, int,    \
                                           cudaStream_t, const BatchMap&, long);                                   \
  template cudaError_t launch_update<S>(const cplx<S>*, int, int, const zd*, int, int, int, cplx<S>*, int, double, \
                                        double, cudaStream_t, const BatchMap&, long);                             \
  template cudaError_t launch_orth_update<S>(const cplx<S>*, const cplx<S>*, int, int, const zd*, cplx<S>*,        \
                                             cplx<S>*, cplx<S>*, int, cudaStream_t, const BatchMap&, long,        \
                                             const int*);                                                         \
  template cudaError_t launch_residual<S>(const cplx<S>*, int, const cplx<S>*, int, const double*, int, int,       \
                                          cplx<S>*, int, double*, int, double*, cudaStream_t, const BatchMap&,     \
                                          long, const double*, bool);                                              \
  template cudaError_t launch_copy_cols<S>(const cplx<S>*, int, cplx<S>*, int, int, int, cudaStream_t);           \
  template cudaError_t launch_init_guess<S>(cplx<S>*, int, int, int, const int*, unsigned, cudaStream_t,           \
                                            const BatchMap&, long);
WTB_INST_BLAS(float)
WTB_INST_BLAS(double)
template cudaError_t launch_convert_cols<float, double>(const cplx<float>*, int, cplx<double>*, int, int, int,
                                                       cudaStream_t);
template cudaError_t launch_convert_cols<double, float>(const cplx<double>*, int, cplx<float>*, int, int, int,
                                                       cudaStream_t);
template cudaError_t launch_convert_cols<double, double>(const cplx<double>*, int, cplx<double>*, int, int, int,
                                                        cudaStream_t);

}  // namespace wtb
