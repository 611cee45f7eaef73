// Matrix-free BSE operator pieces.
//
// With I = (k,c,v) and the band vectors C[k][c][o], Vb[k][v][p] (o, p orbitals) the operator of the
// dense build factorises as
//     (H x)[k,c,v] = dE[k,c,v] x[k,c,v] + sum_{o,p} conj(C[k,c,o]) conj(Vb[k,v,p]) T[k,o,p]
//     T[k,o,p]     = sum_k' V(k,k') Z[k',o,p]
//     Z[k',o,p]    = sum_{c',v'} C[k',c',o] Vb[k',v',p] x[k',c',v']
// (same operator as matrizelbse, src/module_bse.F90:24-83, including V(k,k) times the orbital overlaps
// on the same k-point, which vanish by orthonormality).  The gather kernel forms Z, the real
// Nk x Nk by Nk x (2 w^2 nb) contraction T = V Z runs on the tensor cores (tcgen05, split-BF16) or on
// the CUDA cores (FP32/FP64), and the scatter kernel forms y.
//
// Z is stored transposed and K-major for the contraction: zt[slice][n][k'] with
// n = ((b*w + o)*w + p)*2 + (0 re | 1 im); T is row-major t[k][n].
#include <cuda_bf16.h>

#include "wtb_internal.h"

namespace wtb {

namespace {

template <class Z>
struct ZStore;
template <>
struct ZStore<float> {
  __device__ static void put(float* base, long slice_stride, int nslices, long off, float v) {
    (void)slice_stride;
    (void)nslices;
    base[off] = v;
  }
};
template <>
struct ZStore<double> {
  __device__ static void put(double* base, long slice_stride, int nslices, long off, double v) {
    (void)slice_stride;
    (void)nslices;
    base[off] = v;
  }
};
template <>
struct ZStore<uint16_t> {
  // split v = hi + mid + lo with each part rounded to bfloat16
  __device__ static void put(uint16_t* base, long slice_stride, int nslices, long off, float v) {
    float r = v;
    for (int s = 0; s < nslices; ++s) {
      const __nv_bfloat16 h = __float2bfloat16_rn(r);
      base[s * slice_stride + off] = __bfloat16_as_ushort(h);
      r = r - __bfloat162float(h);
    }
  }
};

template <class S, class Z>
__global__ void __launch_bounds__(256) mf_gather_kernel(const cplx<S>* __restrict__ X, int ldx, int c0,
                                                        const cplx<S>* __restrict__ vec_win, int nk, int nv, int nc, int w,
                                                        int KT, Z* __restrict__ zt, int ldk, int nslices,
                                                        long slice_stride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nb = nv + nc, ncv = nc * nv;
  const int kt0 = blockIdx.x * KT;
  const int b = blockIdx.y;
  const int tkn = min(KT, nk - kt0);
  cplx<S>* Cs = reinterpret_cast<cplx<S>*>(smem_raw);  // [KT][nc][w]
  cplx<S>* Vs = Cs + KT * nc * w;                      // [KT][nv][w]
  cplx<S>* xs = Vs + KT * nv * w;                      // [KT][ncv]
  cplx<S>* Y1 = xs + KT * ncv;                         // [KT][nc][w]
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < KT * nb * w; e += nt) {
    const int kk = e / (nb * w), s = (e / w) % nb, o = e % w;
    const cplx<S> as = kk < tkn ? vec_win[((size_t)(kt0 + kk) * nb + s) * w + o] : mk<S>(0, 0);
    if (s < nv)
      Vs[(kk * nv + s) * w + o] = as;
    else
      Cs[(kk * nc + s - nv) * w + o] = as;
  }
  for (int e = tid; e < KT * ncv; e += nt) {
    const int kk = e / ncv, cv = e % ncv;
    xs[e] = kk < tkn ? X[((size_t)(kt0 + kk) * ncv + cv) * ldx + c0 + b] : mk<S>(0, 0);
  }
  __syncthreads();
  // Y1[k'][c'][p] = sum_v' Vb[k'][v'][p] x[k'][c'][v']
  for (int e = tid; e < KT * nc * w; e += nt) {
    const int kk = e / (nc * w), c = (e / w) % nc, p = e % w;
    cplx<S> acc = mk<S>(0, 0);
    for (int v = 0; v < nv; ++v) cfma(acc, Vs[(kk * nv + v) * w + p], xs[kk * ncv + c * nv + v]);
    Y1[e] = acc;
  }
  __syncthreads();
  // Z[k'][o][p] = sum_c' C[k'][c'][o] Y1[k'][c'][p]; k' fastest across threads -> coalesced rows of zt
  const long nbase = (long)b * w * w * 2;
  for (int e = tid; e < KT * w * w; e += nt) {
    const int kk = e % KT, op = e / KT;
    if (kk >= tkn) continue;
    const int o = op / w, p = op % w;
    cplx<S> acc = mk<S>(0, 0);
    for (int c = 0; c < nc; ++c) cfma(acc, Cs[(kk * nc + c) * w + o], Y1[(kk * nc + c) * w + p]);
    const long n = nbase + (long)op * 2;
    const long off = n * ldk + kt0 + kk;
    ZStore<Z>::put(zt, slice_stride, nslices, off, acc.re);
    ZStore<Z>::put(zt, slice_stride, nslices, off + ldk, acc.im);
  }
}

// bf16-slice variant: one CTA per tile of KT consecutive k' (8 or 16) and one chunk of nbp block columns (grid.y:
// the chunks, so that a panel of a few thousand k' still spreads over many CTAs).  The tile's band vectors and X
// rows are staged, Y1 = Vb x is formed in shared memory, and each thread then forms Z[k'][o][p][b] for its
// (b, o, p) items over the KT k' of the tile and writes the re and im rows of every slice as KT/8 16-byte
// vectors of 8 bf16.  zt is stored in 64-wide K blocks, zt[slice][kb][n][64] (ldn rows per block): the tile's
// row segments of one block sit side by side, so a warp's stores cover contiguous memory.  k' >= nk inside the
// last tile give zeros (x = 0).
// F32: the same tile writes FP32 Z rows instead, z32[n][ldk] (n = ((b w + o) w + p) 2 + ri, k' contiguous; ldk a
// multiple of 64, so the tile's KT values are 16-byte aligned; k' >= nk inside the last tile get zeros).
template <int KT, bool F32 = false, class VT = zd>
__device__ __forceinline__ void gather_bf16_tile(const zf* __restrict__ X, int ldx, int c0, int nbc, int nbp,
                                                 const VT* __restrict__ vec_win, int nk, int nv, int nc, int w,
                                                 uint16_t* __restrict__ zt, int ldn, int nslices, long slice_stride,
                                                 int kt0, float* __restrict__ z32 = nullptr, int ldk = 0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nbnd = nv + nc, ncv = nc * nv;
  const int tkn = min(KT, nk - kt0);
  zf* Cs = reinterpret_cast<zf*>(smem_raw);  // [KT][nc][w]
  zf* Vs = Cs + KT * nc * w;                 // [KT][nv][w]
  zf* xs = Vs + KT * nv * w;                 // [KT][ncv][nbp]
  zf* Y1 = xs + KT * ncv * nbp;              // [KT][nc][w][nbp]
  const int tid = threadIdx.x, nt = blockDim.x;
  // index quotients by the runtime extents through qdiv (all numerators < 2^21)
  const float r_w = 1.0f / w, r_nbnd = 1.0f / nbnd, r_ncv = 1.0f / ncv;
  for (int e = tid; e < KT * nbnd * w; e += nt) {
    const int q = qdiv(e, r_w), o = e - q * w;  // q = kk * nbnd + sb
    const int kk = qdiv(q, r_nbnd), sb = q - kk * nbnd;
    zf as = mk<float>(0.f, 0.f);
    if (kk < tkn) {
      const VT a = vec_win[((size_t)(kt0 + kk) * nbnd + sb) * w + o];
      as = mk<float>((float)a.re, (float)a.im);
    }
    if (sb < nv)
      Vs[(kk * nv + sb) * w + o] = as;
    else
      Cs[(kk * nc + sb - nv) * w + o] = as;
  }
  {
    const int b0 = blockIdx.y * nbp;
    const int nbl = min(nbp, nbc - b0);
    if (nbl <= 0) return;  // uniform over the CTA
    const float r_nbl = 1.0f / nbl;
    for (int e = tid; e < KT * ncv * nbl; e += nt) {
      const int r = qdiv(e, r_nbl), bb = e - r * nbl;  // r = kk * ncv + cv
      const int kk = qdiv(r, r_ncv);
      xs[r * nbp + bb] = kk < tkn ? X[((size_t)kt0 * ncv + r) * ldx + c0 + b0 + bb] : mk<float>(0.f, 0.f);
    }
    __syncthreads();
    // Y1[kk][c][p][bb] = sum_v Vb[kk][v][p] x[kk][c][v][bb]: a thread takes one (kk, p, bb) and four c at a time,
    // each band-vector value loaded once for them (every sum runs over v in the same order as one c alone)
    for (int e = tid; e < KT * w * nbl; e += nt) {
      const int q = qdiv(e, r_nbl), bb = e - q * nbl;  // q = kk * w + p
      const int kk = qdiv(q, r_w), p = q - kk * w;
      for (int cb = 0; cb < nc; cb += 4) {
        zf acc[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) acc[i] = mk<float>(0.f, 0.f);
        for (int v = 0; v < nv; ++v) {
          const zf a = Vs[(kk * nv + v) * w + p];
#pragma unroll
          for (int i = 0; i < 4; ++i)
            if (cb + i < nc) cfma(acc[i], a, xs[(kk * ncv + (cb + i) * nv + v) * nbp + bb]);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (cb + i < nc) Y1[((kk * nc + cb + i) * w + p) * nbp + bb] = acc[i];
      }
    }
    __syncthreads();
    // items (bb, o group, p), bb fastest across lanes (Y1 reads are then consecutive in shared memory): Z over the
    // tile's KT k' for OG consecutive o (each Y1 value loaded once for them; OG = 2 for the 8-wide tile, whose
    // accumulators then take the registers of the 16-wide tile's single o), re and im rows, every slice
    constexpr int OG = KT <= 8 ? 2 : 1;
    const int wo = (w + OG - 1) / OG;  // o groups
    for (int it = tid; it < nbl * wo * w; it += nt) {
      const int op = qdiv(it, r_nbl), bb = it - op * nbl, o2 = qdiv(op, r_w), p = op - o2 * w;
      float zr[OG][KT], zi[OG][KT];
      const int nog = min(OG, w - OG * o2);
#pragma unroll
      for (int kk = 0; kk < KT; ++kk) {
        zf acc[OG];
#pragma unroll
        for (int g = 0; g < OG; ++g) acc[g] = mk<float>(0.f, 0.f);
        for (int c = 0; c < nc; ++c) {
          const zf y = Y1[((kk * nc + c) * w + p) * nbp + bb];
          const zf* cr = Cs + (kk * nc + c) * w + OG * o2;
#pragma unroll
          for (int g = 0; g < OG; ++g)
            if (g < nog) cfma(acc[g], cr[g], y);
        }
#pragma unroll
        for (int g = 0; g < OG; ++g) {
          zr[g][kk] = acc[g].re;
          zi[g][kk] = acc[g].im;
        }
      }
#pragma unroll
      for (int ho = 0; ho < OG; ++ho) {
        if (ho >= nog) break;
        const int o = OG * o2 + ho;
        const long row = ((long)((b0 + bb) * w + o) * w + p) * 2;
        if constexpr (F32) {
          float4* dre = reinterpret_cast<float4*>(z32 + row * ldk + kt0);
          float4* dim = reinterpret_cast<float4*>(z32 + (row + 1) * ldk + kt0);
#pragma unroll
          for (int h = 0; h < KT / 4; ++h) {
            dre[h] = make_float4(zr[ho][4 * h], zr[ho][4 * h + 1], zr[ho][4 * h + 2], zr[ho][4 * h + 3]);
            dim[h] = make_float4(zi[ho][4 * h], zi[ho][4 * h + 1], zi[ho][4 * h + 2], zi[ho][4 * h + 3]);
          }
        } else {
          const long off_re = ((long)(kt0 >> 6) * ldn + row) * 64 + (kt0 & 63), off_im = off_re + 64;
          for (int sl = 0; sl < nslices; ++sl) {
#pragma unroll
            for (int h = 0; h < KT / 8; ++h) {
              uint32_t pr[4], pi[4];
#pragma unroll
              for (int q = 0; q < 4; ++q) {
                const int k0 = 8 * h + 2 * q;
                float* zrr = zr[ho];
                float* zii = zi[ho];
                const __nv_bfloat16 r0 = __float2bfloat16_rn(zrr[k0]), r1 = __float2bfloat16_rn(zrr[k0 + 1]);
                const __nv_bfloat16 i0 = __float2bfloat16_rn(zii[k0]), i1 = __float2bfloat16_rn(zii[k0 + 1]);
                zrr[k0] -= __bfloat162float(r0);
                zrr[k0 + 1] -= __bfloat162float(r1);
                zii[k0] -= __bfloat162float(i0);
                zii[k0 + 1] -= __bfloat162float(i1);
                pr[q] = (uint32_t)__bfloat16_as_ushort(r0) | ((uint32_t)__bfloat16_as_ushort(r1) << 16);
                pi[q] = (uint32_t)__bfloat16_as_ushort(i0) | ((uint32_t)__bfloat16_as_ushort(i1) << 16);
              }
              *reinterpret_cast<uint4*>(zt + sl * slice_stride + off_re + 8 * h) =
                  make_uint4(pr[0], pr[1], pr[2], pr[3]);
              *reinterpret_cast<uint4*>(zt + sl * slice_stride + off_im + 8 * h) =
                  make_uint4(pi[0], pi[1], pi[2], pi[3]);
            }
          }
        }
      }
    }
  }
}

// shared memory of a gather tile: band vectors, then the staged X rows and Y1 of one pass of nbp columns
inline size_t gather_smem(int KT, int nv, int nc, int w, int nbp) {
  return (size_t)(KT * nc * w + KT * nv * w + KT * nc * nv * nbp + KT * nc * w * nbp) * sizeof(zf);
}

// The tile shape of a gather: 16 k' per tile and chunks of (at most) 4 block columns, smaller chunks or 8 k'
// when the shared memory of a CTA would exceed 56 KB (four CTAs per SM); *nbp receives the columns per chunk.
inline int gather_tile(int nv, int nc, int w, int nbc, int* nbp) {
  constexpr size_t kFourPerSm = 56 * 1024;
  for (int KT : {16, 8})
    for (int p = std::min(nbc, 4); p >= 1; --p)
      if (gather_smem(KT, nv, nc, w, p) <= kFourPerSm) {
        *nbp = p;
        return KT;
      }
  *nbp = 1;
  return 8;
}

template <int KT>
__global__ void __launch_bounds__(256) mf_gather_bf16_kernel(const zf* __restrict__ X, int ldx, int c0, int nbc,
                                                             int nbp, const zf* __restrict__ vec_win, int nk, int nv,
                                                             int nc, int w, uint16_t* __restrict__ zt, int ldn,
                                                             int nslices, long slice_stride) {
  gather_bf16_tile<KT, false, zf>(X, ldx, c0, nbc, nbp, vec_win, nk, nv, nc, w, zt, ldn, nslices, slice_stride, blockIdx.x * KT);
}

template <int KT>
__global__ void __launch_bounds__(256) mf_gather_f32_kernel(const zf* __restrict__ X, int ldx, int c0, int nbc,
                                                            int nbp, const zf* __restrict__ vec_win, int nk, int nv,
                                                            int nc, int w, float* __restrict__ z32, int ldk) {
  gather_bf16_tile<KT, true, zf>(X, ldx, c0, nbc, nbp, vec_win, nk, nv, nc, w, nullptr, 0, 0, 0, blockIdx.x * KT, z32,
                             ldk);
}

// batch: CTA b takes tile tiles[b] = (system, first k-point) of the systems' Z panels; frozen systems are
// skipped unless all (the final application) are wanted
template <int KT>
__global__ void __launch_bounds__(256) mf_gather_bf16_batch_kernel(const zf* __restrict__ X, int ldx, int c0, int nbc,
                                                                   int nbp, const MfSys* __restrict__ sys,
                                                                   const int2* __restrict__ tiles, int nslices,
                                                                   const int* __restrict__ frozen) {
  const int2 t = tiles[blockIdx.x];
  if (frozen && frozen[t.x]) return;
  const MfSys& q = sys[t.x];
  gather_bf16_tile<KT>(X + (size_t)q.row0 * ldx, ldx, c0, nbc, nbp, q.vec_win, q.nk, q.nv, q.nc, q.w, q.zt,
                       (int)(q.slice_stride / q.ldk), nslices, q.slice_stride, t.y);
}

template <class S, class T, class VT, class ET>
__device__ __forceinline__ void scatter_k(const T* __restrict__ Tm, int ldt, const cplx<S>* __restrict__ X, int ldx,
                                          const VT* __restrict__ vec_win, const ET* __restrict__ dE, int nk,
                                          int nv, int nc, int w, int nb, int nbg, cplx<S>* __restrict__ Y, int ldy,
                                          int c0, int k, int b0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nbl = min(nbg, nb - b0);
  const int nbnd = nv + nc, ncv = nc * nv;
  // U rows padded by one complex per column b; T rows of 2w values padded to 2w + 2, so that the eight (b, o) rows
  // a warp reads at one p fall in distinct bank pairs and every (re, im) pair is one 8-byte load.  Index
  // quotients by the runtime extents go through qdiv (all numerators < 2^21).
  const int us = w * nv + 1, tw = 2 * w, ts = tw + 2;
  cplx<S>* Cs = reinterpret_cast<cplx<S>*>(smem_raw);  // [nc][w]
  cplx<S>* Vs = Cs + nc * w;                           // [nv][w]
  cplx<S>* U = Vs + nv * w;                            // [nbg][us]: U[b][o][v] at b * us + o * nv + v
  T* Ts = reinterpret_cast<T*>(U + nbg * us);          // [nbg][w][ts]: T[b][o][p][ri] at (b * w + o) * ts + 2p + ri
  const int tid = threadIdx.x, nt = blockDim.x;
  const float r_w = 1.0f / w, r_nv = 1.0f / nv, r_nbl = 1.0f / nbl;
  for (int e = tid; e < nbnd * w; e += nt) {
    const int s = qdiv(e, r_w), o = e - s * w;
    const VT a = vec_win[((size_t)k * nbnd + s) * w + o];
    const cplx<S> as = mk<S>((S)a.re, (S)a.im);
    if (s < nv)
      Vs[s * w + o] = as;
    else
      Cs[(s - nv) * w + o] = as;
  }
  const int row = nbl * w * tw;
  const T* trow = Tm + (size_t)k * ldt + (size_t)b0 * w * tw;
  if constexpr (sizeof(T) == 4) {
    // 16-byte loads when the row segment allows (its start a multiple of 16 bytes, w even so that a load stays
    // within one (b, o) row of 2w values), each stored as two 8-byte pairs
    if ((reinterpret_cast<uintptr_t>(trow) & 15) == 0 && (w & 1) == 0) {
      const float4* t4 = reinterpret_cast<const float4*>(trow);
      const int hw = w >> 1;  // 16-byte loads per (b, o) row
      const float r_hw = 1.0f / hw;
      for (int e = tid; e < row / 4; e += nt) {
        const float4 v4 = t4[e];
        const int r = qdiv(e, r_hw), c = (e - r * hw) * 4;
        float2* d = reinterpret_cast<float2*>(Ts + r * ts + c);
        d[0] = make_float2(v4.x, v4.y);
        d[1] = make_float2(v4.z, v4.w);
      }
    } else {
      const float r_tw = 1.0f / tw;
      for (int f = tid; f < row; f += nt) {
        const int r = qdiv(f, r_tw);
        Ts[r * ts + f - r * tw] = trow[f];
      }
    }
  } else {
    const float r_tw = 1.0f / tw;
    for (int f = tid; f < row; f += nt) {
      const int r = qdiv(f, r_tw);
      Ts[r * ts + f - r * tw] = trow[f];
    }
  }
  __syncthreads();
  // U[b][o][v] = sum_p conj(Vb[v][p]) T[b][o][p]: a thread takes one (b, o) row and four v at a time, each T value
  // loaded once for them (every sum runs over p in the same order as one v alone)
  for (int q = tid; q < nbl * w; q += nt) {  // q = bb * w + o
    const T* tp = Ts + (size_t)q * ts;
    const int bb = qdiv(q, r_w), o = q - bb * w;
    cplx<S>* up = U + bb * us + o * nv;
    for (int v0 = 0; v0 < nv; v0 += 4) {
      cplx<S> acc[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[i] = mk<S>(0, 0);
      for (int p = 0; p < w; ++p) {
        const cplx<S> tc = mk<S>((S)tp[2 * p], (S)tp[2 * p + 1]);
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (v0 + i < nv) cfmac(acc[i], Vs[(v0 + i) * w + p], tc);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (v0 + i < nv) up[v0 + i] = acc[i];
    }
  }
  __syncthreads();
  // y[c][v][b] = dE x + sum_o conj(C[c][o]) U[b][o][v]
  for (int e = tid; e < ncv * nbl; e += nt) {
    const int cv = qdiv(e, r_nbl), bb = e - cv * nbl;
    const int c = qdiv(cv, r_nv), v = cv - c * nv;
    cplx<S> acc = mk<S>(0, 0);
    const cplx<S>* cr = Cs + c * w;
    const cplx<S>* ur = U + bb * us + v;
    for (int o = 0; o < w; ++o) cfmac(acc, cr[o], ur[o * nv]);
    const size_t I = (size_t)k * ncv + cv;
    const cplx<S> x = X[I * ldx + c0 + b0 + bb];
    const S d = (S)dE[I];
    acc.re += d * x.re;
    acc.im += d * x.im;
    Y[I * ldy + c0 + b0 + bb] = acc;
  }
}

template <class S, class T>
__global__ void __launch_bounds__(128) mf_scatter_kernel(const T* __restrict__ Tm, int ldt,
                                                         const cplx<S>* __restrict__ X, int ldx,
                                                         const cplx<S>* __restrict__ vec_win, const S* __restrict__ dE,
                                                         int nk, int nv, int nc, int w, int nb, int nbg,
                                                         cplx<S>* __restrict__ Y, int ldy, int c0) {
  scatter_k<S, T, cplx<S>, S>(Tm, ldt, X, ldx, vec_win, dE, nk, nv, nc, w, nb, nbg, Y, ldy, c0, blockIdx.x, blockIdx.y * nbg);
}

// Scatter from T in Z's layout, T[n][k] (the FFT form): a CTA takes a tile of kScatK consecutive k-points and
// nbg block columns.  It reads each of its T rows' kScatK values (32 bytes, one sector) at once and stages them
// as Ts[kk][(b w + o) (2w + 2) + 2p + ri] (rows padded as in mf_scatter), then forms U and y for every k-point
// of the tile with the same sums, in the same order, as mf_scatter.
constexpr int kScatK = 8;
__global__ void __launch_bounds__(256) mf_scatter_t_kernel(const float* __restrict__ Tt, int ldt,
                                                           const zf* __restrict__ X, int ldx,
                                                           const zf* __restrict__ vec_win,
                                                           const float* __restrict__ dE, int nk, int nv, int nc,
                                                           int w, int nb, int nbg, zf* __restrict__ Y, int ldy,
                                                           int c0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int k0 = blockIdx.x * kScatK, kn = min(kScatK, nk - k0);
  const int b0 = blockIdx.y * nbg, nbl = min(nbg, nb - b0);
  const int nbnd = nv + nc, ncv = nc * nv, tw = 2 * w, ts = tw + 2, us = w * nv + 1;
  const int nrow = nbl * w;  // (b, o) rows per k-point
  zf* Cs = reinterpret_cast<zf*>(smem_raw);             // [kScatK][nc][w]
  zf* Vs = Cs + kScatK * nc * w;                        // [kScatK][nv][w]
  zf* U = Vs + kScatK * nv * w;                         // [kScatK][nbg][us]
  float* Ts = reinterpret_cast<float*>(U + kScatK * nbg * us);  // [kScatK][nbg w][ts]
  const int TSK = nbg * w * ts;                         // floats per k-point
  const int tid = threadIdx.x, nt = blockDim.x;
  const float r_w = 1.0f / w, r_nbnd = 1.0f / nbnd, r_tw = 1.0f / tw, r_nv = 1.0f / nv, r_nrow = 1.0f / nrow,
              r_nbl = 1.0f / nbl, r_ncv = 1.0f / ncv;
  for (int e = tid; e < kScatK * nbnd * w; e += nt) {
    const int q = qdiv(e, r_w), o = e - q * w;  // q = kk * nbnd + sb
    const int kk = qdiv(q, r_nbnd), sb = q - kk * nbnd;
    const zf as = kk < kn ? vec_win[((size_t)(k0 + kk) * nbnd + sb) * w + o] : mk<float>(0.f, 0.f);
    if (sb < nv)
      Vs[(kk * nv + sb) * w + o] = as;
    else
      Cs[(kk * nc + sb - nv) * w + o] = as;
  }
  // T rows n = b0 2w^2 + nl: kScatK values at Tt[n ldt + k0] (ldt a multiple of 64, k0 of 8: 32-byte aligned;
  // values past nk are padding, staged and never used)
  const float* tbase = Tt + (size_t)b0 * w * tw * ldt + k0;
  for (int nl = tid; nl < nrow * tw; nl += nt) {
    const float4* src = reinterpret_cast<const float4*>(tbase + (size_t)nl * ldt);
    const float4 a = src[0], b = src[1];
    const int row = qdiv(nl, r_tw), c = nl - row * tw;  // row = b w + o, c = 2p + ri
    float* d = Ts + row * ts + c;
    d[0] = a.x;
    d[TSK] = a.y;
    d[2 * TSK] = a.z;
    d[3 * TSK] = a.w;
    d[4 * TSK] = b.x;
    d[5 * TSK] = b.y;
    d[6 * TSK] = b.z;
    d[7 * TSK] = b.w;
  }
  __syncthreads();
  // U[kk][b][o][v] = sum_p conj(Vb[kk][v][p]) T[kk][b][o][p]: a thread takes one (kk, b, o) row and four v at a
  // time, so that each T value is loaded once for them (every sum runs over p in the same order as one v alone)
  for (int q = tid; q < kn * nrow; q += nt) {  // q = kk nrow + (b w + o)
    const int kk = qdiv(q, r_nrow), ro = q - kk * nrow;
    const float2* tp = reinterpret_cast<const float2*>(Ts + kk * TSK + ro * ts);  // ts, TSK even: 8-byte aligned
    const int bb = qdiv(ro, r_w), o = ro - bb * w;
    zf* up = U + (kk * nbg + bb) * us + o * nv;
    for (int v0 = 0; v0 < nv; v0 += 4) {
      const zf* vr = Vs + (kk * nv + v0) * w;
      zf acc[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[i] = mk<float>(0.f, 0.f);
      for (int p = 0; p < w; ++p) {
        const float2 t = tp[p];
        const zf tc = mk<float>(t.x, t.y);
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (v0 + i < nv) cfmac(acc[i], vr[i * w + p], tc);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (v0 + i < nv) up[v0 + i] = acc[i];
    }
  }
  __syncthreads();
  // y[k][c][v][b] = dE x + sum_o conj(C[k][c][o]) U[k][b][o][v]
  for (int e = tid; e < kn * ncv * nbl; e += nt) {
    const int q = qdiv(e, r_nbl), bb = e - q * nbl;  // q = kk ncv + cv
    const int kk = qdiv(q, r_ncv), cv = q - kk * ncv;
    const int c = qdiv(cv, r_nv), v = cv - c * nv;
    const zf* cr = Cs + (kk * nc + c) * w;
    const zf* ur = U + (kk * nbg + bb) * us + v;
    zf acc = mk<float>(0.f, 0.f);
    for (int o = 0; o < w; ++o) cfmac(acc, cr[o], ur[o * nv]);
    const size_t I = (size_t)(k0 + kk) * ncv + cv;
    const zf x = X[I * ldx + c0 + b0 + bb];
    const float d = dE[I];
    acc.re += d * x.re;
    acc.im += d * x.im;
    Y[I * ldy + c0 + b0 + bb] = acc;
  }
}

// The FFT form's gather and scatter with the lanes of a warp along k (Z and T are [n][k] rows, k contiguous):
// a CTA takes 32 consecutive k-points and a chunk of block columns, and every load of T and store of Z is then one
// 128-byte line per warp instruction (the row-per-thread kernels above touch 32 lines per instruction).  The
// per-k operands are staged k-innermost with the k extent padded to 33, so that lane k's accesses are
// conflict-free.  The sums are those of the tiles above, term for term and in the same order.
constexpr int kLaneK = 32;
constexpr int kLaneKp = 33;
constexpr int kScatMaxW = 16;  // orbitals per k-point of the lane-k scatter (its T row values live in registers)

// shared memory of the lane-k gather: Vs, Cs, xs, Y1
inline size_t gather32_smem(int nv, int nc, int w, int nbp) {
  return (size_t)(nv * w + nc * w + nc * nv * nbp + nc * w * nbp) * kLaneKp * sizeof(zf);
}

// NV, NC > 0: the band counts fixed at compile time (the loops over them unroll), else taken from nv_rt, nc_rt
template <int NV, int NC>
__global__ void __launch_bounds__(256) mf_gather_k32_kernel(const zf* __restrict__ X, int ldx, int c0, int nbc,
                                                            int nbp, const zf* __restrict__ vec, int nk, int nv_rt,
                                                            int nc_rt, int w, float* __restrict__ z32, int ldk) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nv = NV > 0 ? NV : nv_rt, nc = NC > 0 ? NC : nc_rt;
  const int nbnd = nv + nc, ncv = nc * nv;
  const int k0 = blockIdx.x * kLaneK, b0 = blockIdx.y * nbp;
  const int nbl = min(nbp, nbc - b0);
  if (nbl <= 0) return;  // uniform over the CTA
  zf* Vs = reinterpret_cast<zf*>(smem_raw);  // [v][p][33]
  zf* Cs = Vs + nv * w * kLaneKp;             // [c][o][33]
  zf* xs = Cs + nc * w * kLaneKp;             // [c][v][bb][33]
  zf* Y1 = xs + ncv * nbp * kLaneKp;          // [c][p][bb][33]
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  const float r_bw = 1.0f / (nbnd * w), r_w = 1.0f / w, r_ncvb = 1.0f / (ncv * nbl), r_nbl = 1.0f / nbl;
  // band vectors: reads follow memory (one k-point's nbnd w values after another)
  for (int e = tid; e < kLaneK * nbnd * w; e += nt) {
    const int kk = qdiv(e, r_bw), sw = e - kk * nbnd * w;  // sw = sb w + o
    const int sb = qdiv(sw, r_w), o = sw - sb * w;
    const zf a = k0 + kk < nk ? vec[(size_t)(k0 + kk) * nbnd * w + sw] : mk<float>(0.f, 0.f);
    if (sb < nv)
      Vs[(sb * w + o) * kLaneKp + kk] = a;
    else
      Cs[((sb - nv) * w + o) * kLaneKp + kk] = a;
  }
  // x rows (k, c, v): the chunk's nbl values of each
  for (int e = tid; e < kLaneK * ncv * nbl; e += nt) {
    const int kk = qdiv(e, r_ncvb), r = e - kk * ncv * nbl;  // r = cv nbl + bb
    const int cv = qdiv(r, r_nbl), bb = r - cv * nbl;
    xs[(cv * nbp + bb) * kLaneKp + kk] =
        k0 + kk < nk ? X[((size_t)(k0 + kk) * ncv + cv) * ldx + c0 + b0 + bb] : mk<float>(0.f, 0.f);
  }
  __syncthreads();
  // Y1[c][p][bb] = sum_v Vb[v][p] x[c][v][bb] for lane k: a warp takes (p, bb) items and every c
  for (int it = warp; it < w * nbl; it += nwarp) {
    const int p = qdiv(it, r_nbl), bb = it - p * nbl;
#pragma unroll
    for (int cb = 0; cb < nc; cb += 4) {
      zf acc[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[i] = mk<float>(0.f, 0.f);
#pragma unroll
      for (int v = 0; v < nv; ++v) {
        const zf a = Vs[(v * w + p) * kLaneKp + lane];
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (cb + i < nc) cfma(acc[i], a, xs[(((cb + i) * nv + v) * nbp + bb) * kLaneKp + lane]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (cb + i < nc) Y1[(((cb + i) * w + p) * nbp + bb) * kLaneKp + lane] = acc[i];
    }
  }
  __syncthreads();
  // Z[o][p][bb] = sum_c C[c][o] Y1[c][p][bb] for lane k: a warp takes (bb, p, o group of 4) items; the re and im
  // rows of each output are one 128-byte store each (k >= nk inside the last tile: zeros, x = 0 there)
  const int wo = (w + 3) >> 2;
  const float r_wo = 1.0f / wo;
  for (int it = warp; it < nbl * w * wo; it += nwarp) {
    const int q = qdiv(it, r_wo), og = it - q * wo;  // q = bb w + p
    const int bb = qdiv(q, r_w), p = q - bb * w;
    zf acc[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[i] = mk<float>(0.f, 0.f);
#pragma unroll
    for (int c = 0; c < nc; ++c) {
      const zf y = Y1[((c * w + p) * nbp + bb) * kLaneKp + lane];
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (4 * og + i < w) cfma(acc[i], Cs[(c * w + 4 * og + i) * kLaneKp + lane], y);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int o = 4 * og + i;
      if (o < w) {
        const long row = ((long)((b0 + bb) * w + o) * w + p) * 2;
        z32[row * ldk + k0 + lane] = acc[i].re;
        z32[(row + 1) * ldk + k0 + lane] = acc[i].im;
      }
    }
  }
}

// shared memory of the lane-k scatter: Vs, Cs, U
// U's column groups are ustride(w, nv) complex apart: w nv 33 rounded up to 4 mod 16, so that lanes of different
// groups at one (o, v) fall in different bank pairs (w nv 33 itself is a multiple of 16 at w = 12, nv = 4)
inline int scatter32_ustride(int w, int nv) { return w * nv * kLaneKp + ((4 - (w * nv * kLaneKp) % 16) + 16) % 16; }
inline size_t scatter32_smem(int nv, int nc, int w, int nbg) {
  return ((size_t)(nv * w + nc * w) * kLaneKp + (size_t)nbg * scatter32_ustride(w, nv)) * sizeof(zf);
}

// y[k][c][v][b] = dE x + sum_o conj(C[k][c][o]) sum_p conj(Vb[k][v][p]) T[k][b][o][p] for 32 k-points (lanes) and
// nbg block columns
template <int NV, int NC>
__global__ void __launch_bounds__(256) mf_scatter_k32_kernel(const float* __restrict__ Tt, int ldt,
                                                             const zf* __restrict__ X, int ldx,
                                                             const zf* __restrict__ vec,
                                                             const float* __restrict__ dE, int nk, int nv_rt,
                                                             int nc_rt, int w, int nb, int nbg, zf* __restrict__ Y,
                                                             int ldy, int c0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nv = NV > 0 ? NV : nv_rt, nc = NC > 0 ? NC : nc_rt;
  const int nbnd = nv + nc, ncv = nc * nv, tw = 2 * w;
  const int k0 = blockIdx.x * kLaneK, b0 = blockIdx.y * nbg;
  const int nbl = min(nbg, nb - b0);
  zf* Vs = reinterpret_cast<zf*>(smem_raw);  // [v][p][33]
  zf* Cs = Vs + nv * w * kLaneKp;             // [c][o][33]
  zf* U = Cs + nc * w * kLaneKp;              // [bb][o][v][33], column groups ust apart
  const int ust = w * nv * kLaneKp + ((4 - (w * nv * kLaneKp) % 16) + 16) % 16;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  const float r_bw = 1.0f / (nbnd * w), r_w = 1.0f / w, r_nv = 1.0f / nv, r_nbl = 1.0f / nbl;
  for (int e = tid; e < kLaneK * nbnd * w; e += nt) {
    const int kk = qdiv(e, r_bw), sw = e - kk * nbnd * w;
    const int sb = qdiv(sw, r_w), o = sw - sb * w;
    const zf a = k0 + kk < nk ? vec[(size_t)(k0 + kk) * nbnd * w + sw] : mk<float>(0.f, 0.f);
    if (sb < nv)
      Vs[(sb * w + o) * kLaneKp + kk] = a;
    else
      Cs[((sb - nv) * w + o) * kLaneKp + kk] = a;
  }
  __syncthreads();
  // U[bb][o][v] = sum_p conj(Vb[v][p]) T[bb][o][p] for lane k: a warp takes (bb, o) rows; T's re and im rows
  // n = ((b0 + bb) w + o) 2w + 2p (+1) are read at columns k0 .. k0 + 31 (ldt >= the tile's end: padding columns)
  const float r_wu = 1.0f / w;
  for (int it = warp; it < nbl * w; it += nwarp) {  // it = bb w + o
    const int bbit = qdiv(it, r_wu), oit = it - bbit * w;
    const float* trow = Tt + (size_t)(b0 * w + it) * tw * ldt + k0 + lane;
    // the row's 2w values of lane k, all loads issued before the first use (w <= kScatMaxW)
    float tre[kScatMaxW], tim[kScatMaxW];
#pragma unroll
    for (int p = 0; p < kScatMaxW; ++p)
      if (p < w) {
        tre[p] = trow[(size_t)(2 * p) * ldt];
        tim[p] = trow[(size_t)(2 * p + 1) * ldt];
      }
#pragma unroll
    for (int v0 = 0; v0 < nv; v0 += 4) {
      zf acc[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[i] = mk<float>(0.f, 0.f);
#pragma unroll
      for (int p = 0; p < kScatMaxW; ++p)
        if (p < w) {
          const zf tc = mk<float>(tre[p], tim[p]);
#pragma unroll
          for (int i = 0; i < 4; ++i)
            if (v0 + i < nv) cfmac(acc[i], Vs[((v0 + i) * w + p) * kLaneKp + lane], tc);
        }
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (v0 + i < nv) U[bbit * ust + (oit * nv + v0 + i) * kLaneKp + lane] = acc[i];
    }
  }
  __syncthreads();
  // y: the lanes along (c v, bb) of one k-point, so that a warp's X loads and Y stores cover consecutive rows
  // (c v) of the k-point (lanes along k would put every lane in a different row)
  const float r_ib = 1.0f / (ncv * nbl);
  for (int e = tid; e < kLaneK * ncv * nbl; e += nt) {
    const int kk = qdiv(e, r_ib), r = e - kk * ncv * nbl;  // r = cv nbl + bb
    const int cv = qdiv(r, r_nbl), bb = r - cv * nbl;
    const int c = qdiv(cv, r_nv), v = cv - c * nv;
    zf acc = mk<float>(0.f, 0.f);
    for (int o = 0; o < w; ++o)
      cfmac(acc, Cs[(c * w + o) * kLaneKp + kk], U[bb * ust + (o * nv + v) * kLaneKp + kk]);
    if (k0 + kk < nk) {
      const size_t I = (size_t)(k0 + kk) * ncv + cv;
      const zf x = X[I * ldx + c0 + b0 + bb];
      const float d = dE[I];
      acc.re += d * x.re;
      acc.im += d * x.im;
      Y[I * ldy + c0 + b0 + bb] = acc;
    }
  }
}

// batch: CTA (b, g) takes k-point kpts[b] = (system, k) and column group g
__global__ void __launch_bounds__(128) mf_scatter_batch_kernel(const zf* __restrict__ X, int ldx,
                                                               const MfSys* __restrict__ sys,
                                                               const int2* __restrict__ kpts, int nb, int nbg,
                                                               zf* __restrict__ Y, int ldy, int c0,
                                                               const int* __restrict__ frozen) {
  const int2 t = kpts[blockIdx.x];
  if (frozen && frozen[t.x]) return;
  const MfSys& q = sys[t.x];
  scatter_k<float, float, zd, double>(q.Tm, q.ldt, X + (size_t)q.row0 * ldx, ldx, q.vec_win, q.dE, q.nk, q.nv, q.nc, q.w, nb, nbg,
                          Y + (size_t)q.row0 * ldy, ldy, c0, t.y, blockIdx.y * nbg);
}

// C[M][N] = A[M][K] * B[N][K]^T, real, CUDA cores.  64 x 64 CTA tile, 4 x 4 per thread, K step 16.
// Products are accumulated over 256-wide K ranges and the range sums added into a second accumulator:
// one running sum over all of K (K = Nk up to a few thousand) lets FP32 rounding errors add up
// coherently for the smooth, one-signed operands of this contraction.
template <class S>
__global__ void __launch_bounds__(256) simt_gemm_tn_kernel(const S* __restrict__ A, int lda, const S* __restrict__ B,
                                                           int ldb, S* __restrict__ C, int ldc, int M, int N, int K) {
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ S As[BK][BM + 4];
  __shared__ S Bs[BK][BN + 4];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  S acc[4][4], tot[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = tot[i][j] = 0;
  for (int k0 = 0; k0 < K; k0 += BK) {
    if (k0 % 256 == 0) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          tot[i][j] += acc[i][j];
          acc[i][j] = 0;
        }
    }
    for (int e = tid; e < BM * BK; e += 256) {
      const int r = e / BK, kk = e % BK;
      const int gm = m0 + r, gn = n0 + r, gk = k0 + kk;
      As[kk][r] = (gm < M && gk < K) ? A[(size_t)gm * lda + gk] : (S)0;
      Bs[kk][r] = (gn < N && gk < K) ? B[(size_t)gn * ldb + gk] : (S)0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      S a[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gm = m0 + ty * 4 + i, gn = n0 + tx * 4 + j;
      if (gm < M && gn < N) C[(size_t)gm * ldc + gn] = tot[i][j] + acc[i][j];
    }
}

// x = x0 + x1 + x2 with every part rounded to bf16: three 8-bit significands hold the 24 bits of the FP32
// rounding of x, so the split runs in FP32 after one conversion (FP64 instructions are scarce on this GPU)
__global__ void split_bf16_kernel(const double* __restrict__ V, int ldv, int rows, int cols, uint16_t* __restrict__ out,
                                  int ldo, long slice_stride, int nslices) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)rows * cols) return;
  const int r = (int)(e / cols), c = (int)(e % cols);
  float x = (float)V[(size_t)r * ldv + c];
  for (int s = 0; s < nslices; ++s) {
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    out[s * slice_stride + (size_t)r * ldo + c] = __bfloat16_as_ushort(h);
    x = x - __bfloat162float(h);
  }
}

__global__ void round_f32_kernel(const double* __restrict__ V, int ldv, int rows, int cols, float* __restrict__ out,
                                 int ldo) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)rows * cols) return;
  const int r = (int)(e / cols), c = (int)(e % cols);
  out[(size_t)r * ldo + c] = (float)V[(size_t)r * ldv + c];
}

}  // namespace

template <class S, class Z>
cudaError_t launch_mf_gather(const cplx<S>* X, int ldx, int c0, int nb, const cplx<S>* vec_win, int nk, int nv, int nc,
                             int w, Z* zt, int ldk, int nslices, long slice_stride, cudaStream_t s, int tile) {
  if constexpr (sizeof(S) == 4 && sizeof(Z) == 2) {
    int nbp = nb;
    int KT = gather_tile(nv, nc, w, nb, &nbp);
    // a requested tile KT * 100 + nbp (16 or 8 k' per CTA, 1..8 block columns per chunk)
    if (tile > 0) {
      KT = tile / 100;
      nbp = std::min(tile % 100, nb);
      if ((KT != 16 && KT != 8) || nbp < 1 || nbp > 8) return cudaErrorInvalidValue;
    }
    const size_t smem = gather_smem(KT, nv, nc, w, nbp);
    // the K-blocked panel: ldk a multiple of 64, ldn = rows per K block
    const int ldn = (int)(slice_stride / ldk);
    if (smem <= 200 * 1024 && ldk % 64 == 0 && slice_stride == (long)ldn * ldk) {
      const void* fn = KT == 16 ? reinterpret_cast<const void*>(mf_gather_bf16_kernel<16>)
                                : reinterpret_cast<const void*>(mf_gather_bf16_kernel<8>);
      cudaError_t e = raise_smem_limit(fn, smem);
      if (e != cudaSuccess) return e;
      const unsigned nch = (unsigned)((nb + nbp - 1) / nbp);
      if (KT == 16)
        mf_gather_bf16_kernel<16><<<dim3((nk + 15) / 16, nch), 256, smem, s>>>(reinterpret_cast<const zf*>(X), ldx, c0, nb, nbp,
                                                                     vec_win, nk, nv, nc, w,
                                                                     reinterpret_cast<uint16_t*>(zt), ldn, nslices,
                                                                     slice_stride);
      else
        mf_gather_bf16_kernel<8><<<dim3((nk + 7) / 8, nch), 256, smem, s>>>(reinterpret_cast<const zf*>(X), ldx, c0, nb, nbp,
                                                                  vec_win, nk, nv, nc, w,
                                                                  reinterpret_cast<uint16_t*>(zt), ldn, nslices,
                                                                  slice_stride);
      ++g_launch_count;
      return cudaGetLastError();
    }
  }
  if constexpr (sizeof(S) == 4 && sizeof(Z) == 4) {
    // FP32 rows through the tiled gather (the band vectors and X rows of a tile staged once for nbp columns)
    int nbp = nb;
    int KT = gather_tile(nv, nc, w, nb, &nbp);
    if (tile > 0) {
      KT = tile / 100;
      nbp = std::min(tile % 100, nb);
      if ((KT != 16 && KT != 8 && KT != 32) || nbp < 1 || nbp > 8) return cudaErrorInvalidValue;
    }
    if (KT == 32) {
      // the lane-k gather: 32 k' per CTA along the lanes
      const size_t smem = gather32_smem(nv, nc, w, nbp);
      if (smem > 200 * 1024 || ldk % kLaneK != 0 || nslices != 1) return cudaErrorInvalidValue;
      auto kern = nv == 4 && nc == 4 ? mf_gather_k32_kernel<4, 4>
                  : nv == 2 && nc == 2 ? mf_gather_k32_kernel<2, 2>
                                       : mf_gather_k32_kernel<0, 0>;
      cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(kern), smem);
      if (e != cudaSuccess) return e;
      kern<<<dim3((nk + kLaneK - 1) / kLaneK, (nb + nbp - 1) / nbp), 256, smem, s>>>(
          reinterpret_cast<const zf*>(X), ldx, c0, nb, nbp, vec_win, nk, nv, nc, w, reinterpret_cast<float*>(zt), ldk);
      ++g_launch_count;
      return cudaGetLastError();
    }
    const size_t smem = gather_smem(KT, nv, nc, w, nbp);
    if (smem <= 200 * 1024 && ldk % 64 == 0 && nslices == 1) {
      const void* fn = KT == 16 ? reinterpret_cast<const void*>(mf_gather_f32_kernel<16>)
                                : reinterpret_cast<const void*>(mf_gather_f32_kernel<8>);
      cudaError_t e = raise_smem_limit(fn, smem);
      if (e != cudaSuccess) return e;
      const unsigned nch = (unsigned)((nb + nbp - 1) / nbp);
      if (KT == 16)
        mf_gather_f32_kernel<16><<<dim3((nk + 15) / 16, nch), 256, smem, s>>>(
            reinterpret_cast<const zf*>(X), ldx, c0, nb, nbp, vec_win, nk, nv, nc, w, reinterpret_cast<float*>(zt), ldk);
      else
        mf_gather_f32_kernel<8><<<dim3((nk + 7) / 8, nch), 256, smem, s>>>(
            reinterpret_cast<const zf*>(X), ldx, c0, nb, nbp, vec_win, nk, nv, nc, w, reinterpret_cast<float*>(zt), ldk);
      ++g_launch_count;
      return cudaGetLastError();
    }
  }
  if constexpr (sizeof(Z) == 2) return cudaErrorInvalidValue;  // the bf16 panel exists only in the K-blocked layout
  int KT = 32;
  auto smem_of = [&](int kt) { return (size_t)(2 * kt * nc * w + kt * nv * w + kt * nc * nv) * sizeof(cplx<S>); };
  while (KT > 4 && smem_of(KT) > 160 * 1024) KT /= 2;
  const size_t smem = smem_of(KT);
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(mf_gather_kernel<S, Z>), (size_t)smem);
  if (e != cudaSuccess) return e;
  dim3 grid((nk + KT - 1) / KT, nb);
  mf_gather_kernel<S, Z><<<grid, 256, smem, s>>>(X, ldx, c0, vec_win, nk, nv, nc, w, KT, zt, ldk, nslices,
                                                 slice_stride); ++g_launch_count;
  return cudaGetLastError();
}

template <class S, class T>
cudaError_t launch_mf_scatter(const T* Tm, int ldt, const cplx<S>* X, int ldx, const cplx<S>* vec_win, const S* dE,
                              int nk, int nv, int nc, int w, int nb, cplx<S>* Y, int ldy, int c0, cudaStream_t s,
                              int cols) {
  // block columns per CTA: all (or the requested count), halved until the CTA's tiles fit in 96 KB
  int nbg = cols > 0 ? std::min(cols, nb) : nb;
  auto smem_of = [&](int g) {
    return (size_t)((nc + nv) * w + g * (w * nv + 1)) * sizeof(cplx<S>) + (size_t)g * w * (2 * w + 2) * sizeof(T) + 16;
  };
  while (nbg > 1 && smem_of(nbg) > 96 * 1024) nbg = (nbg + 1) / 2;
  const size_t smem = smem_of(nbg);
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(mf_scatter_kernel<S, T>), (size_t)smem);
  if (e != cudaSuccess) return e;
  dim3 grid(nk, (nb + nbg - 1) / nbg);
  mf_scatter_kernel<S, T><<<grid, 128, smem, s>>>(Tm, ldt, X, ldx, vec_win, dE, nk, nv, nc, w, nb, nbg, Y, ldy, c0); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_mf_scatter_t(const float* Tt, int ldt, const zf* X, int ldx, const zf* vec_win, const float* dE,
                                int nk, int nv, int nc, int w, int nb, zf* Y, int ldy, int c0, cudaStream_t s,
                                int cols) {
  if (ldt % 64 != 0 || (reinterpret_cast<uintptr_t>(Tt) & 31) != 0) return cudaErrorInvalidValue;
  if (cols > 100) {
    // the lane-k scatter: 32 k-points per CTA along the lanes, cols - 100 block columns
    const int g = std::min(cols - 100, nb);
    const size_t smem = scatter32_smem(nv, nc, w, g);
    if (smem > 200 * 1024 || w > kScatMaxW || ldt < (nk + kLaneK - 1) / kLaneK * kLaneK) return cudaErrorInvalidValue;
    auto kern = nv == 4 && nc == 4 ? mf_scatter_k32_kernel<4, 4>
                : nv == 2 && nc == 2 ? mf_scatter_k32_kernel<2, 2>
                                     : mf_scatter_k32_kernel<0, 0>;
    cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(kern), smem);
    if (e != cudaSuccess) return e;
    kern<<<dim3((nk + kLaneK - 1) / kLaneK, (nb + g - 1) / g), 256, smem, s>>>(
        Tt, ldt, X, ldx, vec_win, dE, nk, nv, nc, w, nb, g, Y, ldy, c0);
    ++g_launch_count;
    return cudaGetLastError();
  }
  int nbg = std::min(cols > 0 ? cols : 4, nb);
  auto smem_of = [&](int g) {
    return (size_t)kScatK * ((nc + nv) * w + g * (w * nv + 1)) * sizeof(zf) +
           (size_t)kScatK * g * w * (2 * w + 2) * sizeof(float);
  };
  while (nbg > 1 && smem_of(nbg) > 160 * 1024) nbg = (nbg + 1) / 2;
  const size_t smem = smem_of(nbg);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(mf_scatter_t_kernel), smem);
  if (e != cudaSuccess) return e;
  mf_scatter_t_kernel<<<dim3((nk + kScatK - 1) / kScatK, (nb + nbg - 1) / nbg), 256, smem, s>>>(
      Tt, ldt, X, ldx, vec_win, dE, nk, nv, nc, w, nb, nbg, Y, ldy, c0);
  ++g_launch_count;
  return cudaGetLastError();
}

int mf_gather_batch_tile(int max_nv, int max_nc, int w, int nb) {
  int nbp = nb;
  return gather_tile(max_nv, max_nc, w, nb, &nbp);
}

// tiles hold (system, first k-point) of tiles of mf_gather_batch_tile() k-points
cudaError_t launch_mf_gather_batch(const zf* X, int ldx, int c0, int nb, const MfSys* sys, const int2* tiles,
                                   int ntiles, int max_nv, int max_nc, int w, int nslices, const int* frozen,
                                   cudaStream_t s) {
  int nbp = nb;
  const int KT = gather_tile(max_nv, max_nc, w, nb, &nbp);
  const size_t smem = gather_smem(KT, max_nv, max_nc, w, nbp);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  const void* fn = KT == 16 ? reinterpret_cast<const void*>(mf_gather_bf16_batch_kernel<16>)
                            : reinterpret_cast<const void*>(mf_gather_bf16_batch_kernel<8>);
  cudaError_t e = raise_smem_limit(fn, smem);
  if (e != cudaSuccess) return e;
  const dim3 grid(ntiles, (nb + nbp - 1) / nbp);
  if (KT == 16)
    mf_gather_bf16_batch_kernel<16><<<grid, 256, smem, s>>>(X, ldx, c0, nb, nbp, sys, tiles, nslices, frozen);
  else
    mf_gather_bf16_batch_kernel<8><<<grid, 256, smem, s>>>(X, ldx, c0, nb, nbp, sys, tiles, nslices, frozen);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_mf_scatter_batch(const zf* X, int ldx, const MfSys* sys, const int2* kpts, int nkpts, int max_nv,
                                    int max_nc, int w, int nb, zf* Y, int ldy, int c0, const int* frozen,
                                    cudaStream_t s) {
  int nbg = nb;
  auto smem_of = [&](int g) {
    return (size_t)((max_nc + max_nv) * w + g * (w * max_nv + 1)) * sizeof(zf) + (size_t)g * w * (2 * w + 2) * sizeof(float) +
           16;
  };
  while (nbg > 1 && smem_of(nbg) > 96 * 1024) nbg = (nbg + 1) / 2;
  const size_t smem = smem_of(nbg);
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(mf_scatter_batch_kernel), smem);
  if (e != cudaSuccess) return e;
  mf_scatter_batch_kernel<<<dim3(nkpts, (nb + nbg - 1) / nbg), 128, smem, s>>>(X, ldx, sys, kpts, nb, nbg, Y, ldy, c0,
                                                                              frozen);
  ++g_launch_count;
  return cudaGetLastError();
}

template <class S>
cudaError_t launch_simt_gemm_tn(const S* A, int lda, const S* B, int ldb, S* C, int ldc, int M, int N, int K,
                                cudaStream_t s) {
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  simt_gemm_tn_kernel<S><<<grid, 256, 0, s>>>(A, lda, B, ldb, C, ldc, M, N, K); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_split_bf16(const double* V, int ldv, int rows, int cols, uint16_t* out, int ldo, long slice_stride,
                              int nslices, cudaStream_t s) {
  const long n = (long)rows * cols;
  split_bf16_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(V, ldv, rows, cols, out, ldo, slice_stride, nslices); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_round_f32(const double* V, int ldv, int rows, int cols, float* out, int ldo, cudaStream_t s) {
  const long n = (long)rows * cols;
  round_f32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(V, ldv, rows, cols, out, ldo); ++g_launch_count;
  return cudaGetLastError();
}

template cudaError_t launch_mf_gather<float, float>(const cplx<float>*, int, int, int, const zf*, int, int, int, int,
                                                    float*, int, int, long, cudaStream_t, int);
template cudaError_t launch_mf_gather<float, uint16_t>(const cplx<float>*, int, int, int, const zf*, int, int, int,
                                                       int, uint16_t*, int, int, long, cudaStream_t, int);
template cudaError_t launch_mf_gather<double, double>(const cplx<double>*, int, int, int, const zd*, int, int, int,
                                                      int, double*, int, int, long, cudaStream_t, int);
template cudaError_t launch_mf_scatter<float, float>(const float*, int, const cplx<float>*, int, const zf*,
                                                     const float*, int, int, int, int, int, cplx<float>*, int, int,
                                                     cudaStream_t, int);
template cudaError_t launch_mf_scatter<double, double>(const double*, int, const cplx<double>*, int, const zd*,
                                                       const double*, int, int, int, int, int, cplx<double>*, int, int,
                                                       cudaStream_t, int);
template cudaError_t launch_simt_gemm_tn<float>(const float*, int, const float*, int, float*, int, int, int, int,
                                                cudaStream_t);
template cudaError_t launch_simt_gemm_tn<double>(const double*, int, const double*, int, double*, int, int, int, int,
                                                 cudaStream_t);

}  // namespace wtb
