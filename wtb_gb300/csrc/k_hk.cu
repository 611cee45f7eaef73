// Wannier Fourier sum H(k) = sum_R e^{ik.R} H(R)/ndegen - E_F I, Hermitian eigensolve, gauge fix and
// band window, one CTA per k-point; plus the velocity matrix elements of optsp/hlm and the V(k,k')
// table.  Follows eigsys (src/module_hamiltonian.F90:200-320), the bsesolver band loop
// (src/module_bse.F90:2230-2245), hlm/optsp (src/module_optics.F90:12-167) and module_coulomb.
//
// Eigensolver: the CTA routine of small_eig.cuh (Householder tridiagonalisation, bisection, inverse iteration),
// in FP64; for the tensor-core forms in FP32 followed by FP64 Rayleigh quotients against the FP64 H(k), which
// leaves the band energies FP64-accurate and the vectors FP32-accurate (the FP64 pipe is the bound of this
// kernel on GB300).
// Gauge: every eigenvector is rotated so its first component is real and >= 0, the gauge ZHEEV('L')
// produces up to a sign (the Householder reflectors of ZHETRD('L') leave e1 invariant).
#include "small_eig.cuh"
#include "wtb_internal.h"

namespace wtb {

namespace {

constexpr int kHkThreads = 128;

__device__ __forceinline__ double cabs2(zd a) { return a.re * a.re + a.im * a.im; }

// Cartesian component a of R = r1 a1 + r2 a2 + r3 a3, evaluated as separately rounded products and
// sums (no fused multiply-add) so that the single-precision rounding below sees the same double as the
// reference's expression rvec(i,1)*rlat(1,a)+rvec(i,2)*rlat(2,a)+rvec(i,3)*rlat(3,a).
__device__ __forceinline__ double rcart(int r1, int r2, int r3, const double* rl, int a) {
  return __dadd_rn(__dadd_rn(__dmul_rn((double)r1, rl[a]), __dmul_rn((double)r2, rl[3 + a])),
                   __dmul_rn((double)r3, rl[6 + a]));
}

// phi_R = kx*Rx + ky*Ry + kz*Rz rounded to single precision (cmplx(0.0, ...) in the reference,
// src/module_hamiltonian.F90:240-244); unfused so the float rounding is reproducible.
__device__ __forceinline__ double phase_f32(const int* rvec, int nR, int iR, const double* rl, double kx, double ky,
                                            double kz) {
  const int r1 = rvec[iR], r2 = rvec[nR + iR], r3 = rvec[2 * nR + iR];
  const double phi = __dadd_rn(__dadd_rn(__dmul_rn(kx, rcart(r1, r2, r3, rl, 0)), __dmul_rn(ky, rcart(r1, r2, r3, rl, 1))),
                               __dmul_rn(kz, rcart(r1, r2, r3, rl, 2)));
  return (double)__double2float_rn(phi);
}

__device__ __forceinline__ double rcomp_f32(const int* rvec, int nR, int iR, const double* rl, int a) {
  const int r1 = rvec[iR], r2 = rvec[nR + iR], r3 = rvec[2 * nR + iR];
  return (double)__double2float_rn(rcart(r1, r2, r3, rl, a));
}

// Double-float (FP32 pair, value = hi + lo) sums for the mixed band route, where the FP64 pipe (1/64 of the FP32
// rate on this GPU) bounds the FP64 sums: each product keeps its exact rounding error (FMA) and each running sum
// its exact TwoSum error, the low parts added without renormalisation (the Dot2 scheme of Ogita, Rump and
// Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26 (2005), with double-float inputs): about 2^-48
// relative to the sum of |terms| per term.  The _rn intrinsics keep the compiler from contracting the steps.
__device__ __forceinline__ void df_split(double x, float& h, float& l) {
  h = __double2float_rn(x);
  l = __double2float_rn(x - (double)h);
}
// (ah, al) += (xh, xl) (yh, yl)
__device__ __forceinline__ void df_mac(float& ah, float& al, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  const float e = __fmaf_rn(xh, yl, __fmaf_rn(xl, yh, __fmaf_rn(xh, yh, -p)));
  const float sm = __fadd_rn(ah, p);
  const float bv = __fsub_rn(sm, ah);
  const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(sm, bv)), __fsub_rn(p, bv));
  al = __fadd_rn(al, __fadd_rn(err, e));
  ah = sm;
}
// (ah, al) += (xh, xl) y for an FP32 y
__device__ __forceinline__ void df_mac1(float& ah, float& al, float xh, float xl, float y) {
  const float p = __fmul_rn(xh, y);
  const float e = __fmaf_rn(xl, y, __fmaf_rn(xh, y, -p));
  const float sm = __fadd_rn(ah, p);
  const float bv = __fsub_rn(sm, ah);
  const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(sm, bv)), __fsub_rn(p, bv));
  al = __fadd_rn(al, __fadd_rn(err, e));
  ah = sm;
}
__device__ __forceinline__ double df_val(float h, float l) { return (double)h + (double)l; }

// H(R) / 1 split into double-float parts once per band solve: (re hi, re lo, im hi, im lo); and the k-independent
// factors of the phases, R's Cartesian components and 1 / ndegen (rtab[2r] = (Rx, Ry), rtab[2r + 1] = (Rz, 1 / ndegen),
// the same expressions as the per-k route)
__global__ void hr_split_kernel(const zd* __restrict__ hr, long n, float4* __restrict__ out,
                                const int* __restrict__ rvec, const int* __restrict__ ndegen, int nR,
                                const double* __restrict__ rlat, double2* __restrict__ rtab) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nR) {
    double lat[9];
#pragma unroll
    for (int a = 0; a < 9; ++a) lat[a] = rlat[a];
    const int r1 = rvec[i], r2 = rvec[nR + i], r3 = rvec[2 * nR + i];
    rtab[2 * i] = make_double2(rcart(r1, r2, r3, lat, 0), rcart(r1, r2, r3, lat, 1));
    rtab[2 * i + 1] = make_double2(rcart(r1, r2, r3, lat, 2), 1.0 / (double)ndegen[i]);
  }
  if (i >= n) return;
  const zd h = hr[i];
  float rh, rl, ih, il;
  df_split(h.re, rh, rl);
  df_split(h.im, ih, il);
  out[i] = make_float4(rh, rl, ih, il);
}

template <bool kMixed>
__global__ void __launch_bounds__(kHkThreads) hk_eig_kernel(const zd* __restrict__ hr, const int* __restrict__ rvec,
                                                            const int* __restrict__ ndegen, int nR, int w,
                                                            const double* __restrict__ rlat, double efermi, double scs,
                                                            const double* __restrict__ kpt, int nk, int nv, int nc,
                                                            double* eig_all, zd* vec_all, double* eig_win,
                                                            zd* vec_win, int* nocp_out, DevStatus* st,
                                                            const float4* __restrict__ hr_df) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int k = blockIdx.x;
  if (k >= nk) return;
  const int n = w;
  const int ld = n + 1;
  zd* A = reinterpret_cast<zd*>(smem_raw);
  zd* eph = A + n * ld;  // nR phases
  zd* p = eph + nR;      // n
  zd* tau = p + n;       // n
  double* d = reinterpret_cast<double*>(tau + n);
  double* e = d + n;
  double* e2 = e + n;
  double* lam = e2 + n;
  double* red = lam + n;  // 4
  double* Z = red + 4;          // n vectors of stride n + 1
  double* Dv = Z + n * (n + 1); // the same, then Lv; the eigenvectors U (n x n complex, column j = vector j)
  double* Lv = Dv + n * (n + 1);  // reuse both
  int* cl = reinterpret_cast<int*>(Lv + n * (n + 1));
  zd* U = reinterpret_cast<zd*>(Dv);
  // mixed: FP32 eigensolver workspace after the FP64 one, and the FP64 eigenvectors and eigenvalues
  zf* A32 = reinterpret_cast<zf*>(cl + ((n + 1) & ~1));
  zf* p32 = A32 + n * ld;
  zf* tau32 = p32 + n;
  float* d32 = reinterpret_cast<float*>(tau32 + n);
  float* e32 = d32 + n;
  float* e2_32 = e32 + n;
  float* lam32 = e2_32 + n;
  float* red32 = lam32 + n;
  float* Z32 = red32 + 4;
  float* Dv32 = Z32 + n * (n + 1);
  float* Lv32 = Dv32 + n * (n + 1);
  __shared__ double rl[9];
  __shared__ int s_nocp;
  const int tid = threadIdx.x;
  if (tid < 9) rl[tid] = rlat[tid];
  __syncthreads();
  const double kx = kpt[3 * k], ky = kpt[3 * k + 1], kz = kpt[3 * k + 2];
  for (int r = tid; r < nR; r += blockDim.x) {
    double phi, inv;
    if constexpr (kMixed) {
      // R's components and 1 / ndegen from the table after the split H(R) (FP64 instructions are the scarce ones)
      const double2* rtab = reinterpret_cast<const double2*>(hr_df + (size_t)nR * w * w);
      const double2 a = rtab[2 * r], b = rtab[2 * r + 1];
      phi = (double)__double2float_rn(__dadd_rn(__dadd_rn(__dmul_rn(kx, a.x), __dmul_rn(ky, a.y)), __dmul_rn(kz, b.x)));
      inv = b.y;
    } else {
      phi = phase_f32(rvec, nR, r, rl, kx, ky, kz);
      inv = 1.0 / (double)ndegen[r];
    }
    double sn, cs;
    sincos(phi, &sn, &cs);
    eph[r] = mk<double>(cs * inv, sn * inv);
    if constexpr (kMixed) {
      float ch, cl, sh, sl;
      df_split(cs * inv, ch, cl);
      df_split(sn * inv, sh, sl);
      reinterpret_cast<float4*>(eph)[r] = make_float4(ch, cl, sh, sl);
    }
  }
  __syncthreads();
  // ZHEEV('V','L') reads the lower triangle and the real part of the diagonal only: the matrix that is
  // diagonalised is the Hermitian completion of the lower triangle (identical to H(k) when the H(R) set
  // is Hermitian-consistent; a perturbation of an upper-triangle entry does not reach the eigensolve)
  if constexpr (kMixed) {
    // the mixed route: H(k) in double-float, Ad[m][c] = (re hi, re lo, im hi, im lo) over A's storage
    const float4* ephd = reinterpret_cast<const float4*>(eph);
    float4* Ad = reinterpret_cast<float4*>(A);
    for (int q = tid; q < n * n; q += blockDim.x) {
      const int m = q / n, c = q % n;
      if (m < c) continue;
      float rh = 0.f, rlo = 0.f, ih = 0.f, il = 0.f;
      for (int r = 0; r < nR; ++r) {
        const float4 ph = ephd[r], h = hr_df[((size_t)r * w + m) * w + c];
        df_mac(rh, rlo, ph.x, ph.y, h.x, h.y);    // cos h.re
        df_mac(rh, rlo, -ph.z, -ph.w, h.z, h.w);  // - sin h.im
        df_mac(ih, il, ph.x, ph.y, h.z, h.w);     // cos h.im
        df_mac(ih, il, ph.z, ph.w, h.x, h.y);     // sin h.re
      }
      if (m == c) {
        df_split(df_val(rh, rlo) - efermi, rh, rlo);
        ih = il = 0.f;
      }
      Ad[m * ld + c] = make_float4(rh, rlo, ih, il);
      if (m != c) Ad[c * ld + m] = make_float4(rh, rlo, -ih, -il);
    }
  } else {
  for (int q = tid; q < n * n; q += blockDim.x) {
    const int m = q / n, c = q % n;
    if (m < c) continue;
    zd acc = mk<double>(0.0, 0.0);
    for (int r = 0; r < nR; ++r) cfma(acc, eph[r], hr[((size_t)r * w + m) * w + c]);
    if (m == c) {
      acc.re -= efermi;
      acc.im = 0.0;
    }
    A[m * ld + c] = acc;
    if (m != c) A[c * ld + m] = mk<double>(acc.re, -acc.im);
  }
  }
  __syncthreads();
  if constexpr (kMixed) {
    // FP32 eigensolve of the rounded H(k), then Rayleigh quotients of the normalised vectors against the
    // double-float H(k): eigenvalues carry the square of the vectors' FP32 error (FP64-accurate), vectors FP32's
    const float4* Ad = reinterpret_cast<const float4*>(A);
    for (int q = tid; q < n * ld; q += blockDim.x) {
      const float4 a = Ad[q];
      A32[q] = mk<float>(__fadd_rn(a.x, a.y), __fadd_rn(a.z, a.w));
    }
    __syncthreads();
    zf* U32 = reinterpret_cast<zf*>(Dv32);
    tridiag_cta<float>(A32, ld, n, d32, e32, tau32, p32);
    tridiag_eigvecs_cta<float>(A32, ld, n, n, d32, e32, tau32, e2_32, lam32, Z32, Dv32, Lv32, cl, U32, n, red32);
    // U (FP64, column j = vector j) = U32 normalised in FP64; H U (n x n complex, column-major) after the FP32
    // workspace
    zd* HU = reinterpret_cast<zd*>((reinterpret_cast<uintptr_t>(Lv32 + n * (n + 1)) + 15) & ~(uintptr_t)15);
    for (int q = tid; q < n * n; q += blockDim.x) {
      const int i = q / n, j = q % n;  // row i of H, column j of U
      float rh = 0.f, rlo = 0.f, ih = 0.f, il = 0.f;
      for (int c = 0; c < n; ++c) {
        const zf u = U32[j * n + c];
        const float4 a = Ad[i * ld + c];
        df_mac1(rh, rlo, a.x, a.y, u.re);
        df_mac1(rh, rlo, -a.z, -a.w, u.im);
        df_mac1(ih, il, a.x, a.y, u.im);
        df_mac1(ih, il, a.z, a.w, u.re);
      }
      HU[j * n + i] = mk<double>(df_val(rh, rlo), df_val(ih, il));
    }
    __syncthreads();
    // vector j's norm and quotient on thread j, its components in order (one FP64 square root and two divisions
    // per vector, no warp reductions: the FP64 pipe is the scarce one), then U = U32 / |u| on every thread;
    // e (n doubles) is free on this route
    for (int j = tid; j < n; j += blockDim.x) {
      double nn = 0.0, rq = 0.0;
      for (int i = 0; i < n; ++i) {
        const zf u = U32[j * n + i];
        const double ur = (double)u.re, ui = (double)u.im;
        const zd h = HU[j * n + i];
        nn = fma(ur, ur, nn);
        nn = fma(ui, ui, nn);
        rq = fma(ur, h.re, rq);  // Re(conj(u_i) (H u)_i)
        rq = fma(ui, h.im, rq);
      }
      lam[j] = nn > 0.0 ? rq / nn : (double)lam32[j];
      e[j] = nn > 0.0 ? 1.0 / sqrt(nn) : 0.0;
    }
    __syncthreads();
    for (int q = tid; q < n * n; q += blockDim.x) {
      const zf u = U32[q];
      const double inv = e[q / n];
      U[q] = mk<double>((double)u.re * inv, (double)u.im * inv);
    }
    __syncthreads();
  } else {
    tridiag_cta<double>(A, ld, n, d, e, tau, p);
    tridiag_eigvecs_cta<double>(A, ld, n, n, d, e, tau, e2, lam, Z, Dv, Lv, cl, U, n, red);
  }
  if (tid == 0) {
    int cnt = 0;
    for (int j = 0; j < n; ++j) cnt += (lam[j] <= 0.0);
    s_nocp = cnt;  // = index of the first E > 0 in ascending order
  }
  __syncthreads();
  const int nocp = s_nocp;
  // outputs in ascending order; eigenvector j = column j of U, rotated so that its first component is real
  // and >= 0 (ZHEEV('L') returns it real; the sign does not reach any output)
  // the gauge factor of each vector once (p and d are free after the eigensolve)
  for (int j = tid; j < w; j += blockDim.x) {
    const zd a0 = U[j * n];
    const double m0 = sqrt(cabs2(a0));
    p[j] = m0 > 0.0 ? mk<double>(a0.re / m0, -a0.im / m0) : mk<double>(1.0, 0.0);
    d[j] = m0;
  }
  __syncthreads();
  for (int q = tid; q < w * w; q += blockDim.x) {
    const int j = q / w, o = q % w;
    zd val = cmul(U[j * n + o], p[j]);
    if (o == 0) val = mk<double>(d[j], 0.0);
    if (vec_all) vec_all[((size_t)k * w + j) * w + o] = val;
    const int sl = j - (nocp - nv);
    if (vec_win && sl >= 0 && sl < nv + nc) vec_win[((size_t)k * (nv + nc) + sl) * w + o] = val;
  }
  if (tid < w) {
    const int j = tid;
    const double ev = lam[j] + (j >= nocp ? scs : 0.0);
    if (eig_all) eig_all[(size_t)k * w + j] = ev;
    const int sl = j - (nocp - nv);
    if (eig_win && sl >= 0 && sl < nv + nc) eig_win[(size_t)k * (nv + nc) + sl] = ev;
  }
  if (tid == 0) {
    if (nocp_out) nocp_out[k] = nocp;
    if (eig_win) {
      if (nv > nocp) dev_fail(st, 101, k);            // valence window below the occupied states
      else if (nc > w - nocp) dev_fail(st, 102, k);   // conduction window above the empty states
    }
  }
}

// ----------------------------------------------------------------------------- optics (hlm + optsp)
// T = double: FP64 throughout (hr_t = hr).  T = float: the Fourier sums and the band contractions in FP32 (an FP32
// copy hr_t of H(R), the band vectors rounded once per k-point), with the per-R factors i R_a e^{i phi}/ndegen
// formed once per direction (FP64, then rounded) and the energy factors in FP64.
template <class T>
__global__ void __launch_bounds__(kHkThreads) optics_kernel(const cplx<T>* __restrict__ hr_t,
                                                            const int* __restrict__ rvec,
                                                            const int* __restrict__ ndegen, int nR, int w,
                                                            const double* __restrict__ rlat,
                                                            const double* __restrict__ kpt, int nk, int nv, int nc,
                                                            const double* __restrict__ eig_win,
                                                            const zd* __restrict__ vec_win, float s32,
                                                            zd* __restrict__ hout, int raw) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int k = blockIdx.x;
  if (k >= nk) return;
  const int tid = threadIdx.x;
  const int nb = nv + nc;
  // M, B, Mv in precision T over regions sized for complex(8)
  cplx<T>* M = reinterpret_cast<cplx<T>*>(smem_raw);                    // w*w
  cplx<T>* B = reinterpret_cast<cplx<T>*>(reinterpret_cast<zd*>(M) + w * w);   // nb*w band vectors
  cplx<T>* Mv = reinterpret_cast<cplx<T>*>(reinterpret_cast<zd*>(B) + nb * w);  // nv*w
  zd* eph = reinterpret_cast<zd*>(Mv) + nv * w;                          // nR
  cplx<T>* fr = reinterpret_cast<cplx<T>*>(eph + nR);  // nR (16-byte aligned after the complex(8) arrays)
  double* Ra = reinterpret_cast<double*>(fr + nR);     // nR
  __shared__ double rl[9];
  if (tid < 9) rl[tid] = rlat[tid];
  for (int e = tid; e < nb * w; e += blockDim.x) {
    const zd b = vec_win[(size_t)k * nb * w + e];
    B[e] = mk<T>((T)b.re, (T)b.im);
  }
  __syncthreads();
  const double kx = kpt[3 * k], ky = kpt[3 * k + 1], kz = kpt[3 * k + 2];
  for (int r = tid; r < nR; r += blockDim.x) {
    const double phi = phase_f32(rvec, nR, r, rl, kx, ky, kz);
    double sn, cs;
    sincos(phi, &sn, &cs);
    const double inv = 1.0 / (double)ndegen[r];
    eph[r] = mk<double>(cs * inv, sn * inv);
  }
  const int dimk = nc * nv;
  const size_t dim = (size_t)nk * dimk;
  zd hxyz[3][1];
  (void)hxyz;
  for (int a = 0; a < 3; ++a) {
    __syncthreads();
    for (int r = tid; r < nR; r += blockDim.x) {
      Ra[r] = rcomp_f32(rvec, nR, r, rl, a);
      fr[r] = mk<T>((T)(-Ra[r] * eph[r].im), (T)(Ra[r] * eph[r].re));  // i R_a e
    }
    __syncthreads();
    // M = sum_R i R_a e^{i phi} H(R)/ndegen, in arithmetic T (FP32 for the tensor-core forms, whose oscillator
    // strengths need 1e-4).  hlm skips the diagonal of the R = 0 term, whose factor R_a = 0 makes it vanish
    // exactly here as well.
    for (int e = tid; e < w * w; e += blockDim.x) {
      const int m = e / w, c = e % w;
      cplx<T> acc = mk<T>(0, 0);
      for (int r = 0; r < nR; ++r) cfma(acc, fr[r], hr_t[((size_t)r * w + m) * w + c]);
      M[e] = acc;
    }
    __syncthreads();
    for (int e = tid; e < nv * w; e += blockDim.x) {
      const int v = e / w, m = e % w;
      cplx<T> acc = mk<T>(0, 0);
      for (int c = 0; c < w; ++c) cfma(acc, M[m * w + c], B[v * w + c]);
      Mv[e] = acc;
    }
    __syncthreads();
    for (int e = tid; e < dimk; e += blockDim.x) {
      const int c = e / nv, v = e % nv;
      cplx<T> acct = mk<T>(0, 0);
      for (int m = 0; m < w; ++m) cfmac(acct, B[(nv + c) * w + m], Mv[v * w + m]);
      const zd acc = mk<double>((double)acct.re, (double)acct.im);
      // factor = Re(1/(E_c - E_v + i*CSHIFT_f32)) (a complex assigned to a real in optsp)
      const double de = eig_win[(size_t)k * nb + nv + c] - eig_win[(size_t)k * nb + v];
      const double sf = (double)s32;
      const double factor = raw ? 1.0 : de / (de * de + sf * sf);  // raw: <c|dH/dk_a|v> unscaled (optspbz)
      hout[a * dim + (size_t)k * dimk + e] = cscale(acc, factor);
    }
  }
  __syncthreads();
  const double isq = (double)0.70710677f;  // 1.0/sqrt(2.) in single precision
  for (int e = tid; e < dimk; e += blockDim.x) {
    const size_t I = (size_t)k * dimk + e;
    const zd hx = hout[I], hy = hout[dim + I];
    hout[3 * dim + I] = mk<double>((hx.re - hy.im) * isq, (hx.im + hy.re) * isq);
    hout[4 * dim + I] = mk<double>((hx.re + hy.im) * isq, (hx.im - hy.re) * isq);
  }
}

// ----------------------------------------------------------------------------- Coulomb table
__host__ __device__ __forceinline__ double vecsize3(const double* a) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

// Modified Bessel functions of the second kind K0 and K1 from K_nu(x) = int_0^inf exp(-x cosh t) cosh(nu t) dt,
// trapezoid rule with step min(1/16, 1/(4 sqrt(x))) (the integrand is analytic in a strip of half-width
// pi/2 and decays double-exponentially, so the rule converges to machine precision), truncated where
// x cosh t > 745.
__device__ void bessel_k01(double x, double* k0, double* k1) {
  const double h = fmin(0.0625, 0.25 / sqrt(x));
  const double tmax = acosh(fmax(745.0 / x, 1.0)) + h;
  double s0 = 0.5 * exp(-x), s1 = 0.5 * exp(-x);
  for (int i = 1;; ++i) {
    const double t = i * h;
    if (t > tmax) break;
    const double e = exp(-x * cosh(t));
    s0 += e;
    s1 += e * cosh(t);
  }
  *k0 = h * s0;
  *k1 = h * s1;
}

// integralJ0pot (src/module_math.F90:429-449): trapezoid of r J0(r g) log r on 100 points starting at
// eta = 1E-04 (single precision literal).
__device__ double integral_j0_pot(double rmax, double g) {
  const int n = 100;
  const double eta = (double)1E-04f;
  double res = 0.0;
  const double r1 = eta, r2 = (1.0 / (n - 1.0)) * rmax + eta;
  const double hh = r2 - r1;
  double fprev = r1 * j0(r1 * g) * log(r1);
  for (int i = 1; i < n; ++i) {
    const double r = ((double)i / (n - 1.0)) * rmax + eta;
    const double f = r * j0(r * g) * log(r);
    res = res + (hh / 2.0) * (fprev + f);
    fprev = f;
  }
  return res;
}

struct CoulConst {
  int type;
  int deriv_r0;
  double vbz, tol, cic;
  double eta, kappa, pb, pt, r0, w, lc, ez;  // V2DRK / V2DOH / V2DT2
  double ed;                                 // V3DL / V2DK
  double v2dk_r0, v2dk_small;                // V2DK
  double rc;                                 // V2DT / V0DT
};

// The selected potential for the k-point difference (dx, dy, dz) = k1 - k2 (modvec, then the switch of
// matrizelbse, src/module_bse.F90:49-72).
__device__ double coulomb_of(const CoulConst& cc, double dx, double dy, double dz) {
  if (cc.deriv_r0 && cc.type != CT_V2DRK) return 0.0;  // only V2DRK reads the R_0 key
  const double modk = sqrt(dx * dx + dy * dy + dz * dz);
  double v = 0.0;
  const double vc = cc.vbz * cc.cic;
  switch (cc.type) {
    case CT_V2DRK:
      if (!(modk < cc.tol)) {
        const double aux1 = (1.0 - (cc.pb * cc.pt * exp(-2.0 * modk * cc.eta * cc.lc))) * cc.kappa;
        const double aux2 = (1.0 - (cc.pt * exp(-cc.eta * modk * cc.lc))) * (1.0 - (cc.pb * exp(-cc.eta * modk * cc.lc)));
        const double aux3 = cc.r0 * modk * exp(-modk * cc.w);
        const double ew = (aux1 / aux2) + aux3;
        v = vc * exp(-modk * cc.w) * (1.0 / ew) * (1.0 / modk);
        if (cc.deriv_r0) v = -v * (modk * exp(-modk * cc.w)) / ew;  // d/dr0: ew depends on r0 through aux3
      }
      break;
    case CT_V3DL:
    case CT_V3D:
      if (!(modk < cc.tol)) v = cc.vbz * (cc.cic / cc.ed) * (1.0 / (modk * modk));
      break;
    case CT_V2DK:
      if (modk < cc.tol)
        v = cc.v2dk_small;
      else
        v = cc.vbz * (cc.cic / cc.ed) * (1.0 / (modk * (1 + (cc.v2dk_r0 * modk))));
      break;
    case CT_V2DOH:
      if (!(modk < cc.tol)) v = vc * exp(-cc.w * modk) * (1.0 / (cc.ez * modk));
      break;
    case CT_V2DT: {
      const double gz = fabs(dz), gpar = sqrt(dx * dx + dy * dy), rc = cc.rc;
      if (gpar < cc.tol && gz < cc.tol) {
        v = vc * (-0.5 * rc * rc);
      } else if (gpar < cc.tol) {
        v = vc * (1.0 / (modk * modk)) * (1.0 - cos(gz * rc) - (gz * rc * sin(gz * rc)));
      } else {
        const double aux1 = gz / gpar, aux2 = gpar * rc, aux3 = gz * rc;
        v = vc * (1.0 / (modk * modk)) * (1.0 + (exp(-aux2) * (aux1 * sin(aux3) - cos(aux3))));
      }
      break;
    }
    case CT_V2DT2:
      if (!(modk < cc.tol)) {
        const double qxy = sqrt(dx * dx + dy * dy);
        v = vc * (1.0 / (modk * modk)) * (1.0 - exp(-0.5 * qxy * cc.lc) * cos(0.5 * cc.lc * dz));
      }
      break;
    case CT_V1DT: {
      const double vx = fabs(dx), qyz = sqrt(dy * dy + dz * dz);
      if (vx < cc.tol && qyz >= cc.tol) {
        v = vc * integral_j0_pot(cc.lc, qyz);
      } else if (vx < cc.tol) {
        v = vc * ((cc.lc * cc.lc) / 16.0) * (2.0 * log(cc.lc) - 1.0);
      } else {
        double kk0, kk1;
        bessel_k01(vx * cc.lc, &kk0, &kk1);
        const double c1 = qyz * cc.lc * j1(qyz * cc.lc) * kk0;
        const double c2 = vx * cc.lc * j0(qyz * cc.lc) * kk1;
        v = vc * (1.0 + c1 + c2);
      }
      break;
    }
    case CT_V0DT:
      if (modk < cc.tol)
        v = vc * 0.5 * cc.rc * cc.rc;
      else
        v = vc * (1.0 / (modk * modk)) * (1.0 - cos(cc.rc * modk));
      break;
    default:
      v = 0.0;
  }
  return v;
}

__global__ void coulomb_kernel(CoulConst cc, const double* __restrict__ k1, int n1, const double* __restrict__ k2,
                               int n2, double* __restrict__ V, int ldv) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)n1 * n2) return;
  const int i = (int)(e / n2), j = (int)(e % n2);
  const double dx = k1[3 * i] - k2[3 * j], dy = k1[3 * i + 1] - k2[3 * j + 1], dz = k1[3 * i + 2] - k2[3 * j + 2];
  V[(size_t)i * ldv + j] = coulomb_of(cc, dx, dy, dz);
}

// On a Monkhorst-Pack mesh k = (i/n1) b1 + (j/n2) b2 + (l/n3) b3 + shift, so k - k' depends on the index
// differences only and every potential of module_coulomb is a function of k - k': the (2n1-1)(2n2-1)(2n3-1)
// distinct values are evaluated once and then spread over the Nk x Nk table.
__global__ void coulomb_stencil_kernel(CoulConst cc, const double* __restrict__ bl, int n1, int n2, int n3,
                                       double* __restrict__ st) {
  const int s1 = 2 * n1 - 1, s2 = 2 * n2 - 1, s3 = 2 * n3 - 1;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= s1 * s2 * s3) return;
  const int di = e / (s2 * s3) - (n1 - 1), dj = (e / s3) % s2 - (n2 - 1), dl = e % s3 - (n3 - 1);
  double d[3];
  for (int a = 0; a < 3; ++a)
    d[a] = (bl[a] / (double)n1) * (double)di + (bl[3 + a] / (double)n2) * (double)dj + (bl[6 + a] / (double)n3) * (double)dl;
  st[e] = coulomb_of(cc, d[0], d[1], d[2]);
}

__global__ void coulomb_expand_kernel(const double* __restrict__ st, int n1, int n2, int n3, double* __restrict__ V,
                                      int ldv) {
  const long nk = (long)n1 * n2 * n3;
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nk * nk) return;
  const int k = (int)(e / nk), kp = (int)(e % nk);
  const int i = k / (n2 * n3), j = (k / n3) % n2, l = k % n3;
  const int ip = kp / (n2 * n3), jp = (kp / n3) % n2, lp = kp % n3;
  const int s2 = 2 * n2 - 1, s3 = 2 * n3 - 1;
  V[(size_t)k * ldv + kp] = st[((i - ip + n1 - 1) * s2 + (j - jp + n2 - 1)) * s3 + (l - lp + n3 - 1)];
}

__global__ void transition_kernel(const double* __restrict__ eig_win, int nk, int nv, int nc, double* dE) {
  const long I = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long dim = (long)nk * nc * nv;
  if (I >= dim) return;
  const int k = (int)(I / (nc * nv)), c = (int)((I / nv) % nc), v = (int)(I % nv);
  dE[I] = eig_win[(size_t)k * (nv + nc) + nv + c] - eig_win[(size_t)k * (nv + nc) + v];
}

}  // namespace

cudaError_t launch_hk_eig(const zd* hr, const int* rvec, const int* ndegen, int nR, int w, const double* rlat_rm,
                          double efermi, double scs, const double* kpt, int nk, int nv, int nc, double* eig_all,
                          zd* vec_all, double* eig_win, zd* vec_win, int* nocp, DevStatus* st, cudaStream_t s,
                          bool mixed, float4* hr_df) {
  if (w > 64 || w < 1) return cudaErrorInvalidValue;
  if (mixed && !hr_df) return cudaErrorInvalidValue;
  const int n = w;
  // A, phases, p, tau (complex); d, e, e2, lam, red; Z, Dv, Lv (n x (n + 1) each); cluster ids
  size_t smem = (size_t)(n * (n + 1) + nR + 2 * n) * sizeof(zd) + (size_t)(4 * n + 4 + 3 * n * (n + 1)) * sizeof(double) +
                (size_t)((n + 1) & ~1) * sizeof(int);
  // mixed: the FP32 copy and workspace, then H U
  const size_t smem_mixed = smem + (size_t)(n * (n + 1) + 2 * n) * sizeof(zf) +
                            (size_t)(4 * n + 4 + 3 * n * (n + 1)) * sizeof(float) + 16 + (size_t)n * n * sizeof(zd);
  if (mixed && smem_mixed > 200 * 1024) mixed = false;  // the FP64 route for very wide bases
  smem = (mixed ? smem_mixed : smem) + 64;
  if (smem > 220 * 1024) return cudaErrorInvalidValue;
  const void* fn = mixed ? reinterpret_cast<const void*>(hk_eig_kernel<true>) : reinterpret_cast<const void*>(hk_eig_kernel<false>);
  cudaError_t e = raise_smem_limit(fn, (size_t)smem);
  if (e != cudaSuccess) return e;
  if (mixed) {
    const long nh = (long)nR * w * w;
    // the split H(R), then the per-R table (2 nR float4 = nR (Rx, Ry, Rz, 1 / ndegen) in FP64)
    hr_split_kernel<<<(unsigned)((nh + 255) / 256), 256, 0, s>>>(hr, nh, hr_df, rvec, ndegen, nR, rlat_rm,
                                                                 reinterpret_cast<double2*>(hr_df + nh));
    ++g_launch_count;
    hk_eig_kernel<true><<<nk, kHkThreads, smem, s>>>(hr, rvec, ndegen, nR, w, rlat_rm, efermi, scs, kpt, nk, nv, nc,
                                                     eig_all, vec_all, eig_win, vec_win, nocp, st, hr_df);
  } else {
    hk_eig_kernel<false><<<nk, kHkThreads, smem, s>>>(hr, rvec, ndegen, nR, w, rlat_rm, efermi, scs, kpt, nk, nv, nc,
                                                      eig_all, vec_all, eig_win, vec_win, nocp, st, nullptr);
  }
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_optics(const zd* hr, const int* rvec, const int* ndegen, int nR, int w, const double* rlat_rm,
                          const double* kpt, int nk, int nv, int nc, const double* eig_win, const zd* vec_win,
                          double cshift, zd* hout, cudaStream_t s, const zf* hr32, bool raw) {
  const int nb = nv + nc;
  const size_t smem = (size_t)(w * w + nb * w + nv * w + nR) * sizeof(zd) + nR * sizeof(double) + nR * sizeof(zd) + 16;
  const bool mixed = hr32 != nullptr;
  const void* fn = mixed ? reinterpret_cast<const void*>(optics_kernel<float>) : reinterpret_cast<const void*>(optics_kernel<double>);
  cudaError_t e = raise_smem_limit(fn, (size_t)smem);
  if (e != cudaSuccess) return e;
  if (mixed)
    optics_kernel<float><<<nk, kHkThreads, smem, s>>>(hr32, rvec, ndegen, nR, w, rlat_rm, kpt, nk, nv, nc, eig_win,
                                                      vec_win, (float)cshift, hout, raw ? 1 : 0);
  else
    optics_kernel<double><<<nk, kHkThreads, smem, s>>>(hr, rvec, ndegen, nR, w, rlat_rm, kpt, nk, nv, nc, eig_win,
                                                       vec_win, (float)cshift, hout, raw ? 1 : 0);
  ++g_launch_count;
  return cudaGetLastError();
}

static bool coul_const(const CoulParams& p, CoulConst* out);

cudaError_t launch_coulomb(const CoulParams& p, const double* kpt1, int n1, const double* kpt2, int n2, double* V,
                           int ldv, cudaStream_t s) {
  CoulConst cc{};
  if (!coul_const(p, &cc)) return cudaErrorInvalidValue;
  const long tot = (long)n1 * n2;
  const int th = 256;
  coulomb_kernel<<<(unsigned)((tot + th - 1) / th), th, 0, s>>>(cc, kpt1, n1, kpt2, n2, V, ldv); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_coulomb_stencil(const CoulParams& p, const double* bl, double* stencil, cudaStream_t s) {
  CoulConst cc{};
  if (!coul_const(p, &cc)) return cudaErrorInvalidValue;
  const int n1 = p.ngrid[0], n2 = p.ngrid[1], n3 = p.ngrid[2];
  const int ns = (2 * n1 - 1) * (2 * n2 - 1) * (2 * n3 - 1);
  coulomb_stencil_kernel<<<(ns + 127) / 128, 128, 0, s>>>(cc, bl, n1, n2, n3, stencil); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_coulomb_mesh(const CoulParams& p, const double* bl, double* stencil, double* V, int ldv,
                                cudaStream_t s) {
  CoulConst cc{};
  if (!coul_const(p, &cc)) return cudaErrorInvalidValue;
  const int n1 = p.ngrid[0], n2 = p.ngrid[1], n3 = p.ngrid[2];
  const int ns = (2 * n1 - 1) * (2 * n2 - 1) * (2 * n3 - 1);
  coulomb_stencil_kernel<<<(ns + 127) / 128, 128, 0, s>>>(cc, bl, n1, n2, n3, stencil); ++g_launch_count;
  const long nk = (long)n1 * n2 * n3;
  coulomb_expand_kernel<<<(unsigned)((nk * nk + 255) / 256), 256, 0, s>>>(stencil, n1, n2, n3, V, ldv); ++g_launch_count;
  return cudaGetLastError();
}

static bool coul_const(const CoulParams& p, CoulConst* out) {
  const double* r = p.rlat;
  auto cross = [](const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
  };
  double vx[3];
  cross(r, r + 3, vx);
  const double vc2 = sqrt(vx[0] * vx[0] + vx[1] * vx[1] + vx[2] * vx[2]);          // vcell2D
  const double vc3 = fabs(vx[0] * r[6] + vx[1] * r[7] + vx[2] * r[8]);             // vcell3D
  const long ng = (long)p.ngrid[0] * p.ngrid[1] * p.ngrid[2];
  CoulConst cc{};
  cc.type = p.type;
  cc.deriv_r0 = p.deriv_r0;
  cc.tol = p.ktol;
  cc.cic = -(double)(0.0904756f * 1000.0f);  // -(0.0904756)*10**(3) evaluated in single precision
  cc.r0 = p.r0;
  cc.w = p.w;
  cc.lc = p.lc;
  cc.ez = p.ez;
  const double pi32 = (double)3.14159274101257324f;
  switch (p.type) {
    case CT_V2DRK: {
      cc.vbz = 1.0 / (ng * vc2);
      const double epar = p.ediel[1], et = p.ediel[0], eb = p.ediel[2];
      cc.eta = sqrt(epar / p.ez);
      cc.kappa = sqrt(epar * p.ez);
      cc.pb = (eb - cc.kappa) / (eb + cc.kappa);
      cc.pt = (et - cc.kappa) / (et + cc.kappa);
      break;
    }
    case CT_V3DL:
      cc.vbz = 1.0 / (ng * vc3);
      cc.ed = p.ediel[1];
      break;
    case CT_V3D:
      cc.vbz = 1.0 / (ng * vc3);
      cc.ed = 1.0;
      break;
    case CT_V2DK: {
      const double a0 = 0.5 * (vecsize3(r) + vecsize3(r + 3));
      cc.vbz = 1.0 / (ng * vc2);
      cc.v2dk_r0 = ((p.ediel[1] - 1.0) * p.lc) / (p.ediel[0] + p.ediel[2]);
      const double g1 = (double)(p.ngrid[0] * p.ngrid[1]);
      const double auxi = (2. * pi32 * cc.v2dk_r0) / (a0 * sqrt(g1));
      cc.ed = (p.ediel[0] + p.ediel[2]) / (2.0);
      cc.v2dk_small = cc.vbz * (cc.cic / cc.ed) * (a0 * sqrt(g1) / (2. * pi32)) *
                      ((double)1.76f + auxi * 1.0 + 0.0 * auxi * auxi);
      break;
    }
    case CT_V2DOH:
      cc.vbz = 1.0 / (ng * vc2);
      break;
    case CT_V2DT:
      cc.vbz = 1.0 / (ng * vc3);
      cc.rc = 0.5 * r[8];
      break;
    case CT_V2DT2:
      cc.vbz = 1.0 / (ng * vc3);
      break;
    case CT_V1DT:
      cc.vbz = 1.0 / (ng * vc3);
      break;
    case CT_V0DT: {
      cc.vbz = 1.0 / (ng * vc3);
      const double s1 = vecsize3(r), s2 = vecsize3(r + 3), s3 = vecsize3(r + 6);
      cc.rc = 0.5 * fmin(s1, fmin(s2, s3));
      break;
    }
    default:
      return false;
  }
  *out = cc;
  return true;
}

cudaError_t launch_transition_energies(const double* eig_win, int nk, int nv, int nc, double* dE, cudaStream_t s) {
  const long dim = (long)nk * nc * nv;
  transition_kernel<<<(unsigned)((dim + 255) / 256), 256, 0, s>>>(eig_win, nk, nv, nc, dE); ++g_launch_count;
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------- hlm / optsp / optdiel, one call each
// The scalar routines of module_optics for callers that keep their own loops.  hlm_kernel, one CTA: the three
// velocity matrices dH/dk_a = sum_R i R_a e^{i phi_R} H(R)/ndegen at one k-point (hlm, src/module_optics.F90:12-108;
// phases and R_a rounded to single precision as there; the R = 0 term vanishes with its factor R_a = 0), written
// column-major w x w; or, given band vectors cv and vv (optsp, :113-167), the three elements
// <c|dH/dk_a|v> Re(1/(E_c - E_v + i sme)) with sme in single precision (factor = 1./esp assigned to a real).
__global__ void __launch_bounds__(kHkThreads) hlm_kernel(const zd* __restrict__ hr, const int* __restrict__ rvec,
                                                         const int* __restrict__ ndegen, int nR, int w,
                                                         const double* __restrict__ rlat, double kx, double ky,
                                                         double kz, const zd* __restrict__ cv,
                                                         const zd* __restrict__ vv, double ev, double ec, float s32,
                                                         zd* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zd* M = reinterpret_cast<zd*>(smem_raw);  // w*w
  zd* eph = M + w * w;                      // nR: e^{i phi}/ndegen
  zd* fr = eph + nR;                        // nR: i R_a e^{i phi}/ndegen
  zd* rowv = fr + nR;                       // w: per-row sandwich terms
  __shared__ double rl[9];
  const int tid = threadIdx.x;
  if (tid < 9) rl[tid] = rlat[tid];
  __syncthreads();
  for (int r = tid; r < nR; r += blockDim.x) {
    const double phi = phase_f32(rvec, nR, r, rl, kx, ky, kz);
    double sn, cs;
    sincos(phi, &sn, &cs);
    const double inv = 1.0 / (double)ndegen[r];
    eph[r] = mk<double>(cs * inv, sn * inv);
  }
  for (int a = 0; a < 3; ++a) {
    __syncthreads();
    for (int r = tid; r < nR; r += blockDim.x) {
      const double Ra = rcomp_f32(rvec, nR, r, rl, a);
      fr[r] = mk<double>(-Ra * eph[r].im, Ra * eph[r].re);
    }
    __syncthreads();
    for (int e = tid; e < w * w; e += blockDim.x) {
      const int m = e / w, n = e % w;
      zd acc = mk<double>(0.0, 0.0);
      for (int r = 0; r < nR; ++r) cfma(acc, fr[r], hr[((size_t)r * w + m) * w + n]);
      M[e] = acc;
      if (!cv) out[(size_t)a * w * w + m + (size_t)w * n] = acc;
    }
    if (!cv) continue;
    __syncthreads();
    for (int m = tid; m < w; m += blockDim.x) {
      zd mv = mk<double>(0.0, 0.0);
      for (int n = 0; n < w; ++n) cfma(mv, M[m * w + n], vv[n]);
      zd t = mk<double>(0.0, 0.0);
      cfmac(t, cv[m], mv);
      rowv[m] = t;
    }
    __syncthreads();
    if (tid == 0) {
      zd sum = mk<double>(0.0, 0.0);
      for (int m = 0; m < w; ++m) sum = mk<double>(sum.re + rowv[m].re, sum.im + rowv[m].im);
      const double de = ec - ev, sf = (double)s32;
      out[a] = cscale(sum, de / (de * de + sf * sf));
    }
  }
}

// optdiel (src/module_optics.F90:171-255) at one photon energy, one CTA: avgsme's telescoped spacing over the dimse
// energies (:313-335), then the two Lorentzian sums, each summed per thread in row order and the 256 partials in
// thread order.  out = (rpart, ipart).
__global__ void __launch_bounds__(256) optdiel_kernel(int rtype, double caux, int dimse, double elux,
                                                      const double* __restrict__ E, const double* __restrict__ f,
                                                      double sme, double* __restrict__ out) {
  __shared__ double red[3][256];
  __shared__ double s_smef;
  const int tid = threadIdx.x;
  double acc = 0.0;
  for (int i = 1 + tid; i < dimse; i += blockDim.x) acc += E[i] - E[i - 1];
  red[0][tid] = acc;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)blockDim.x; ++i) t += red[0][i];
    s_smef = 10.0 * (t / (double)dimse) + sme;
  }
  __syncthreads();
  const double smef = s_smef;
  double rp = 0.0, ip = 0.0;
  for (int i = tid; i < dimse; i += blockDim.x) {
    const double eaux = ((elux - E[i]) * (elux - E[i])) + (smef * smef);
    rp += f[i] * ((E[i] - elux) / eaux);
    ip += f[i] * (smef / eaux);
  }
  red[1][tid] = rp;
  red[2][tid] = ip;
  __syncthreads();
  if (tid == 0) {
    double r = 0.0, im = 0.0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      r += red[1][i];
      im += red[2][i];
    }
    out[0] = (rtype == 1 ? 1.0 : 0.0) + r * caux;
    out[1] = im * caux;
  }
}

cudaError_t launch_hlm(const zd* hr, const int* rvec, const int* ndegen, int nR, int w, const double* rlat_rm, double kx,
                       double ky, double kz, const zd* cv, const zd* vv, double ev, double ec, double sme, zd* out,
                       cudaStream_t s) {
  const size_t smem = (size_t)(w * w + 2 * nR + w) * sizeof(zd);
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(hlm_kernel), smem);
  if (e != cudaSuccess) return e;
  hlm_kernel<<<1, kHkThreads, smem, s>>>(hr, rvec, ndegen, nR, w, rlat_rm, kx, ky, kz, cv, vv, ev, ec, (float)sme, out);
  ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_optdiel(int rtype, double caux, int dimse, double elux, const double* E, const double* f, double sme,
                           double* out, cudaStream_t s) {
  optdiel_kernel<<<1, 256, 0, s>>>(rtype, caux, dimse, elux, E, f, sme, out);
  ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace wtb
