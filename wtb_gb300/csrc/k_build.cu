// Dense BSE Hamiltonian build and dense block matvec.
//
// Build (matrizelbse + the upper-triangle loop and Hermitian mirror, src/module_bse.F90:24-83 and
// :2392-2415): element (I, J) with I = (k,c,v), J = (k',c',v') is
//     H_IJ = V(k,k') <c_k|c'_k'> <v_k|v'_k'>    (I != J;  <v|v'> = sum_o conj(v_o) v'_o, as the
//     H_II = (E_c - E_v) + V(k,k)                reference's prodintsq(vbv, vbv2))
// The reference evaluates every element independently (two length-w dot products and a potential per
// element).  Here one CTA owns a TK x TK block of k-points: it forms the small Gram tiles
// Gc = <c|c'> and Gv = <v|v'> once in shared memory from the band vectors, takes V(k,k') from the
// precomputed table, and expands the (TK*nc*nv)^2 outputs with coalesced row-segment stores.  The
// kernel is HBM-write bound: dim^2 * sizeof(complex S) bytes leave the SMs, nothing is re-read.
// Every element is computed directly instead of the upper triangle then a mirror: V is symmetric and
// conj(<a|b>) = <b|a>, so the result is Hermitian to the rounding of the fused multiply-adds (relative
// 1e-16 in FP64, 1e-8 in FP32).
#include "wtb_internal.h"

namespace wtb {

namespace {

template <class S>
__global__ void __launch_bounds__(256) bse_build_kernel(const zd* __restrict__ vec_win,
                                                        const double* __restrict__ dE,
                                                        const double* __restrict__ V, int ldv, int nk, int nv,
                                                        int nc, int w, int TK, cplx<S>* __restrict__ H) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ncv = nc * nv, nb = nv + nc;
  const int k0 = blockIdx.y * TK, k1 = blockIdx.x * TK;  // row block, column block
  const int tkr = min(TK, nk - k0), tkc = min(TK, nk - k1);
  cplx<S>* Cr = reinterpret_cast<cplx<S>*>(smem_raw);  // [TK][nc][w]
  cplx<S>* Cc = Cr + TK * nc * w;
  cplx<S>* Vr = Cc + TK * nc * w;                      // [TK][nv][w]
  cplx<S>* Vc = Vr + TK * nv * w;
  cplx<S>* Gc = Vc + TK * nv * w;                      // [TK*nc][TK*nc]
  cplx<S>* Gv = Gc + TK * nc * TK * nc;                // [TK*nv][TK*nv]
  S* Vt = reinterpret_cast<S*>(Gv + TK * nv * TK * nv);  // [TK][TK]
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < TK * nb * w; e += nt) {
    const int kk = e / (nb * w), s = (e / w) % nb, o = e % w;
    zd a = mk<double>(0.0, 0.0), b = mk<double>(0.0, 0.0);
    if (kk < tkr) a = vec_win[((size_t)(k0 + kk) * nb + s) * w + o];
    if (kk < tkc) b = vec_win[((size_t)(k1 + kk) * nb + s) * w + o];
    const cplx<S> as = mk<S>((S)a.re, (S)a.im), bs = mk<S>((S)b.re, (S)b.im);
    if (s < nv) {
      Vr[(kk * nv + s) * w + o] = as;
      Vc[(kk * nv + s) * w + o] = bs;
    } else {
      Cr[(kk * nc + s - nv) * w + o] = as;
      Cc[(kk * nc + s - nv) * w + o] = bs;
    }
  }
  for (int e = tid; e < TK * TK; e += nt) {
    const int a = e / TK, b = e % TK;
    Vt[e] = (a < tkr && b < tkc) ? (S)V[(size_t)(k0 + a) * ldv + (k1 + b)] : (S)0;
  }
  __syncthreads();
  const int gcn = TK * nc, gvn = TK * nv;
  for (int e = tid; e < gcn * gcn + gvn * gvn; e += nt) {
    cplx<S> acc = mk<S>(0, 0);
    if (e < gcn * gcn) {
      const int i = e / gcn, j = e % gcn;
      for (int o = 0; o < w; ++o) cfmac(acc, Cr[i * w + o], Cc[j * w + o]);
      Gc[e] = acc;
    } else {
      const int ee = e - gcn * gcn;
      const int i = ee / gvn, j = ee % gvn;
      for (int o = 0; o < w; ++o) cfmac(acc, Vr[i * w + o], Vc[j * w + o]);
      Gv[ee] = acc;
    }
  }
  __syncthreads();
  const size_t dim = (size_t)nk * ncv;
  const int rows = tkr * ncv, cols = tkc * ncv;
  const int warp = tid >> 5, lane = tid & 31, nwarp = nt >> 5;
  for (int r = warp; r < rows; r += nwarp) {
    const int kr = r / ncv, cr = (r / nv) % nc, vr = r % nv;
    const size_t I = (size_t)(k0 + kr) * ncv + (r % ncv);
    cplx<S>* Hrow = H + I * dim + (size_t)k1 * ncv;
    for (int cidx = lane; cidx < cols; cidx += 32) {
      const int kc = cidx / ncv, cc = (cidx / nv) % nc, vc = cidx % nv;
      const size_t J = (size_t)(k1 + kc) * ncv + (cidx % ncv);
      const S vkk = Vt[kr * TK + kc];
      cplx<S> out;
      if (I == J) {
        out = mk<S>((S)(dE[I] + (double)vkk), (S)0);
      } else {
        const cplx<S> g = cmul(Gc[(kr * nc + cr) * gcn + kc * nc + cc], Gv[(kr * nv + vr) * gvn + kc * nv + vc]);
        out = cscale(g, vkk);
      }
      Hrow[cidx] = out;
    }
  }
}

// Y[:, 0:ncol] = H * X[:, 0:ncol]; H row-major dim x dim.  CTA: 64 rows x ncol (<= 32) columns, K in
// chunks of 16 staged in shared memory, 4 x 2 register micro-tile per thread.  The diagonal term (the
// transition energy, much larger than the Coulomb entries) is accumulated apart from the off-diagonal
// sum, so a long FP32 accumulation only carries rounding of the Coulomb-sized terms.
template <class S, int BM, int TC>
__global__ void __launch_bounds__(256) dense_mv_kernel(const cplx<S>* __restrict__ H, int dim,
                                                       const cplx<S>* __restrict__ X, int ldx, cplx<S>* __restrict__ Y,
                                                       int ldy, int ncol) {
  // 16 x 16 threads: a thread owns rows ty + 16 i (i < BM/16) and columns tx + 16 j (j < TC)
  constexpr int BK = 16, RI = BM / 16, NC = 16 * TC;
  __shared__ cplx<S> Hs[BM][BK + 1];
  __shared__ cplx<S> Xs[BK][NC];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const long r0 = (long)blockIdx.x * BM;
  cplx<S> acc[RI][TC], dacc[RI][TC];
#pragma unroll
  for (int i = 0; i < RI; ++i)
#pragma unroll
    for (int j = 0; j < TC; ++j) {
      acc[i][j] = mk<S>(0, 0);
      dacc[i][j] = mk<S>(0, 0);
    }
  for (long kb = 0; kb < dim; kb += BK) {
    for (int e = tid; e < BM * BK; e += 256) {
      const int rr = e / BK, kk = e % BK;
      const long gr = r0 + rr, gk = kb + kk;
      Hs[rr][kk] = (gr < dim && gk < dim) ? H[gr * dim + gk] : mk<S>(0, 0);
    }
    for (int e = tid; e < BK * NC; e += 256) {
      const int kk = e / NC, c = e % NC;
      const long gk = kb + kk;
      Xs[kk][c] = (gk < dim && c < ncol) ? X[gk * ldx + c] : mk<S>(0, 0);
    }
    __syncthreads();
    // the diagonal lies in this K chunk for rows r0 + [kb - r0, kb - r0 + BK)
    const bool diag_chunk = kb < r0 + BM && kb + BK > r0;
    if (!diag_chunk) {
#pragma unroll 4
      for (int kk = 0; kk < BK; ++kk) {
        cplx<S> h[RI], x[TC];
#pragma unroll
        for (int i = 0; i < RI; ++i) h[i] = Hs[ty + 16 * i][kk];
#pragma unroll
        for (int j = 0; j < TC; ++j) x[j] = Xs[kk][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < RI; ++i)
#pragma unroll
          for (int j = 0; j < TC; ++j) cfma(acc[i][j], h[i], x[j]);
      }
    } else {
      for (int kk = 0; kk < BK; ++kk) {
        cplx<S> h[RI], x[TC];
#pragma unroll
        for (int i = 0; i < RI; ++i) h[i] = Hs[ty + 16 * i][kk];
#pragma unroll
        for (int j = 0; j < TC; ++j) x[j] = Xs[kk][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < RI; ++i) {
          const bool dg = (kb + kk) == (r0 + ty + 16 * i);
#pragma unroll
          for (int j = 0; j < TC; ++j) {
            if (dg)
              cfma(dacc[i][j], h[i], x[j]);
            else
              cfma(acc[i][j], h[i], x[j]);
          }
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < RI; ++i)
#pragma unroll
    for (int j = 0; j < TC; ++j) {
      const long gr = r0 + ty + 16 * i;
      const int c = tx + 16 * j;
      if (gr < dim && c < ncol) Y[gr * ldy + c] = cadd(dacc[i][j], acc[i][j]);
    }
}

}  // namespace

template <class S>
cudaError_t launch_bse_build(const zd* vec_win, const double* dE, const double* V, int ldv, int nk, int nv, int nc,
                             int w, cplx<S>* H, cudaStream_t s) {
  const int ncv = nc * nv;
  int TK = 128 / ncv;
  if (TK < 1) TK = 1;
  if (TK > 32) TK = 32;
  auto smem_of = [&](int tk) {
    return (size_t)(2 * tk * nc * w + 2 * tk * nv * w + tk * nc * tk * nc + tk * nv * tk * nv) * sizeof(cplx<S>) +
           (size_t)tk * tk * sizeof(S) + 16;
  };
  while (TK > 1 && smem_of(TK) > 200 * 1024) --TK;
  const size_t smem = smem_of(TK);
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(bse_build_kernel<S>), (size_t)smem);
  if (e != cudaSuccess) return e;
  const int nblk = (nk + TK - 1) / TK;
  dim3 grid(nblk, nblk);
  bse_build_kernel<S><<<grid, 256, smem, s>>>(vec_win, dE, V, ldv, nk, nv, nc, w, TK, H); ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_dense_mv(const cplx<S>* H, int dim, const cplx<S>* X, int ldx, cplx<S>* Y, int ldy, int ncol,
                            cudaStream_t s) {
  // column tiles of 16 or 32 (no FMAs on padding columns); 32-row tiles when 64-row ones would leave SMs idle
  const bool small = (dim + 63) / 64 < 2 * 152;
  for (int c0 = 0; c0 < ncol; c0 += 32) {
    const int nc = ncol - c0 < 32 ? ncol - c0 : 32;
    if (nc <= 16) {
      if (small)
        dense_mv_kernel<S, 32, 1><<<(dim + 31) / 32, 256, 0, s>>>(H, dim, X + c0, ldx, Y + c0, ldy, nc);
      else
        dense_mv_kernel<S, 64, 1><<<(dim + 63) / 64, 256, 0, s>>>(H, dim, X + c0, ldx, Y + c0, ldy, nc);
    } else {
      if (small)
        dense_mv_kernel<S, 32, 2><<<(dim + 31) / 32, 256, 0, s>>>(H, dim, X + c0, ldx, Y + c0, ldy, nc);
      else
        dense_mv_kernel<S, 64, 2><<<(dim + 63) / 64, 256, 0, s>>>(H, dim, X + c0, ldx, Y + c0, ldy, nc);
    }
    ++g_launch_count;
  }
  return cudaGetLastError();
}

template cudaError_t launch_bse_build<double>(const zd*, const double*, const double*, int, int, int, int, int,
                                              cplx<double>*, cudaStream_t);
template cudaError_t launch_bse_build<float>(const zd*, const double*, const double*, int, int, int, int, int,
                                             cplx<float>*, cudaStream_t);
template cudaError_t launch_dense_mv<double>(const cplx<double>*, int, const cplx<double>*, int, cplx<double>*, int,
                                             int, cudaStream_t);
template cudaError_t launch_dense_mv<float>(const cplx<float>*, int, const cplx<float>*, int, cplx<float>*, int, int,
                                            cudaStream_t);

}  // namespace wtb
