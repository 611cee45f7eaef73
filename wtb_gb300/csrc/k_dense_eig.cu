// All eigenvalues of a dense Hermitian matrix on the device: the stand-in for the LAPACK ZHEEV calls of the
// full-spectrum paths (bsebnds, src/module_bse.F90:1427-1448; the temperature solver's dense path).
//
// 1. Householder tridiagonalisation A = Q T Q^H in FP64, the unblocked zhetd2 sequence (lower form): for
//    column j, the reflector H = I - tau v v^H of zlarfg annihilates A(j+2:n, j); x = tau A22 v;
//    w = x - (tau/2)(x^H v) v; A22 -= v w^H + w v^H.  A is kept in full storage (both triangles updated), so
//    the matrix-vector product reads columns with coalesced loads.  Three launches per column: the product
//    over row blocks x column chunks (every CTA forms the reflector itself from column j, so no launch is
//    spent on it), a one-CTA reduction of the chunks with the w correction, and the rank-2 update.  Each
//    column reads the trailing block twice and writes it once: 16 n^3 bytes in all (HBM-bound; the block
//    falls into L2 once it is below ~100 MB).
// 2. Eigenvalues of the real symmetric tridiagonal T by bisection on Sturm counts (dstebz's method), as
//    32-point multisection with one warp per eigenvalue index, the count with LAPACK's pivot guard pivmin,
//    to the FP64 resolution of the Gershgorin interval.  Backward stable: |lambda - lambda_exact| <~ n eps ||A||.
#include <cfloat>

#include "wtb_internal.h"

namespace wtb {

namespace {

constexpr int kHvRows = 128;   // rows per CTA of the product
constexpr int kH2Tile = 32;    // rank-2 update tile (32 x 32, 256 threads x 4 elements)

// zlarfg for x = A(j+1:n, j): returns tau, beta and the scale 1/(alpha - beta) applied to x(2:m).
struct Reflector {
  zd tau, scale;
  double beta;
};

__device__ Reflector make_reflector(zd alpha, double xnorm2) {
  Reflector r;
  if (xnorm2 == 0.0 && alpha.im == 0.0) {
    r.tau = mk<double>(0.0, 0.0);
    r.scale = mk<double>(0.0, 0.0);
    r.beta = alpha.re;
    return r;
  }
  const double nrm = sqrt(alpha.re * alpha.re + alpha.im * alpha.im + xnorm2);
  const double beta = alpha.re >= 0.0 ? -nrm : nrm;
  r.beta = beta;
  r.tau = mk<double>((beta - alpha.re) / beta, -alpha.im / beta);
  // 1 / (alpha - beta)
  const double dr = alpha.re - beta, di = alpha.im;
  const double den = dr * dr + di * di;
  r.scale = mk<double>(dr / den, -di / den);
  return r;
}

// Block-wide sum of one double (blockDim.x a multiple of 32, <= 1024).
__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < nw; ++i) t += red[i];
  return t;
}

// Partial products p[chunk][r] = sum_{c in chunk} A22(r, c) v(c) with A22 = A(j+1:n, j+1:n), v the reflector
// of column j.  Every CTA forms the reflector from column j; CTA (0, 0) records tau, e(j) and v.
__global__ void __launch_bounds__(kHvRows) tri_hemv_kernel(const zd* __restrict__ A, int n, int lda, int j,
                                                           zd* __restrict__ vout, zd* __restrict__ tau_out,
                                                           double* __restrict__ e_out, zd* __restrict__ part) {
  __shared__ double red[32];
  __shared__ zd vs[kHvRows];
  const int m = n - j - 1;
  const zd* x = A + (size_t)j * lda + j + 1;
  double s2 = 0.0;
  for (int i = 1 + threadIdx.x; i < m; i += blockDim.x) s2 += x[i].re * x[i].re + x[i].im * x[i].im;
  s2 = block_sum(s2, red);
  const Reflector R = make_reflector(x[0], s2);
  const bool first = blockIdx.x == 0 && blockIdx.y == 0;
  if (first && threadIdx.x == 0) {
    tau_out[j] = R.tau;
    e_out[j] = R.beta;
  }
  if (R.tau.re == 0.0 && R.tau.im == 0.0) return;
  if (first)
    for (int i = threadIdx.x; i < m; i += blockDim.x) vout[i] = i == 0 ? mk<double>(1.0, 0.0) : cmul(x[i], R.scale);
  const int nchunk = gridDim.y;
  const int per = (m + nchunk - 1) / nchunk;
  const int c0 = min(m, (int)blockIdx.y * per), c1 = min(m, c0 + per);
  const int r = blockIdx.x * kHvRows + threadIdx.x;
  zd acc = mk<double>(0.0, 0.0);
  const zd* a22 = A + (size_t)(j + 1) * lda + j + 1;
  for (int t0 = c0; t0 < c1; t0 += kHvRows) {
    const int nt = min(kHvRows, c1 - t0);
    __syncthreads();
    if (threadIdx.x < nt) {
      const int c = t0 + threadIdx.x;
      vs[threadIdx.x] = c == 0 ? mk<double>(1.0, 0.0) : cmul(x[c], R.scale);
    }
    __syncthreads();
    if (r < m)
      for (int q = 0; q < nt; ++q) cfma(acc, a22[(size_t)(t0 + q) * lda + r], vs[q]);
  }
  if (r < m) part[(size_t)blockIdx.y * m + r] = acc;
}

// w = tau p - (tau/2)(tau p)^H v v, one CTA.
__global__ void __launch_bounds__(1024) tri_w_kernel(const zd* __restrict__ part, int nchunk, int m,
                                                     const zd* __restrict__ tau_p, int j,
                                                     const zd* __restrict__ v, zd* __restrict__ w) {
  __shared__ double red[32];
  const zd tau = tau_p[j];
  if (tau.re == 0.0 && tau.im == 0.0) return;
  double dre = 0.0, dim_ = 0.0;
  for (int r = threadIdx.x; r < m; r += blockDim.x) {
    zd p = mk<double>(0.0, 0.0);
    for (int c = 0; c < nchunk; ++c) p = cadd(p, part[(size_t)c * m + r]);
    const zd xr = cmul(tau, p);
    w[r] = xr;
    const zd t = cmulc(xr, v[r]);  // conj(x_r) v_r
    dre += t.re;
    dim_ += t.im;
  }
  dre = block_sum(dre, red);
  dim_ = block_sum(dim_, red);
  const zd alpha = cscale(cmul(tau, mk<double>(dre, dim_)), -0.5);
  __syncthreads();
  for (int r = threadIdx.x; r < m; r += blockDim.x) w[r] = cadd(w[r], cmul(alpha, v[r]));
}

// A22 -= v w^H + w v^H (full storage); CTA (0, 0) also stores v below the subdiagonal of column j.
__global__ void __launch_bounds__(256) tri_her2_kernel(zd* __restrict__ A, int n, int lda, int j,
                                                       const zd* __restrict__ tau_p, const zd* __restrict__ v,
                                                       const zd* __restrict__ w) {
  const zd tau = tau_p[j];
  if (tau.re == 0.0 && tau.im == 0.0) return;
  const int m = n - j - 1;
  const int r = blockIdx.x * kH2Tile + (threadIdx.x & 31);
  const int cb = blockIdx.y * kH2Tile + (threadIdx.x >> 5) * 4;
  zd* a22 = A + (size_t)(j + 1) * lda + j + 1;
  if (blockIdx.x == 0 && blockIdx.y == 0)
    for (int i = threadIdx.x; i < m; i += blockDim.x) A[(size_t)j * lda + j + 1 + i] = v[i];
  if (r >= m) return;
  const zd vr = v[r], wr = w[r];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int c = cb + q;
    if (c >= m) break;
    const zd vc = v[c], wc = w[c];
    zd a = a22[(size_t)c * lda + r];
    // a -= vr conj(wc) + wr conj(vc)
    const zd t1 = mk<double>(vr.re * wc.re + vr.im * wc.im, vr.im * wc.re - vr.re * wc.im);
    const zd t2 = mk<double>(wr.re * vc.re + wr.im * vc.im, wr.im * vc.re - wr.re * vc.im);
    a.re -= t1.re + t2.re;
    a.im -= t1.im + t2.im;
    a22[(size_t)c * lda + r] = a;
  }
}

// A(j,i) = conj(A(i,j)) for i < j (the upper triangle is the input, as ZHEEV 'U' reads it); real diagonal.
__global__ void mirror_upper_kernel(zd* __restrict__ A, int n, int lda) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)n * n) return;
  const int i = (int)(e % n), j = (int)(e / n);  // element (i, j), column-major
  if (i > j) A[(size_t)j * lda + i] = cconj(A[(size_t)i * lda + j]);
  else if (i == j) A[(size_t)j * lda + i].im = 0.0;
}

// d(i) = Re A(i,i); Gershgorin bounds and pivmin of T (one CTA).
__global__ void __launch_bounds__(1024) tri_finish_kernel(const zd* __restrict__ A, int n, int lda,
                                                          double* __restrict__ d, const double* __restrict__ e,
                                                          double* __restrict__ bounds) {
  double lo = INFINITY, hi = -INFINITY, emax2 = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double di = A[(size_t)i * lda + i].re;
    d[i] = di;
    const double el = i > 0 ? fabs(e[i - 1]) : 0.0, er = i < n - 1 ? fabs(e[i]) : 0.0;
    lo = fmin(lo, di - el - er);
    hi = fmax(hi, di + el + er);
    if (i < n - 1) emax2 = fmax(emax2, e[i] * e[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    emax2 = fmax(emax2, __shfl_xor_sync(0xffffffffu, emax2, o));
  }
  __shared__ double s_lo[32], s_hi[32], s_e[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    s_lo[warp] = lo;
    s_hi[warp] = hi;
    s_e[warp] = emax2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
      lo = fmin(lo, s_lo[i]);
      hi = fmax(hi, s_hi[i]);
      emax2 = fmax(emax2, s_e[i]);
    }
    const double tnorm = fmax(fabs(lo), fabs(hi));
    // widen by a few ulps of the norm so that the end eigenvalues are strictly inside
    const double pad = 2.0 * (double)n * DBL_EPSILON * fmax(tnorm, 1e-300) + DBL_MIN;
    bounds[0] = lo - pad;
    bounds[1] = hi + pad;
    bounds[2] = DBL_MIN * fmax(1.0, emax2);  // pivmin (dstebz)
  }
}

// number of eigenvalues of T below x (Sturm sequence with the pivot guard)
__device__ __forceinline__ int sturm_count(const double* __restrict__ d, const double* __restrict__ e2, int n,
                                           double x, double pivmin) {
  double q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  int cnt = q < 0.0;
  for (int i = 1; i < n; ++i) {
    q = (d[i] - x) - e2[i - 1] / q;
    if (fabs(q) < pivmin) q = -pivmin;
    cnt += q < 0.0;
  }
  return cnt;
}

__global__ void e2_kernel(const double* __restrict__ e, int n, double* __restrict__ e2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n - 1) e2[i] = e[i] * e[i];
}

// The k-th smallest eigenvalue (k = 0..n-1), one warp per k: multisection, the 32 lanes evaluating the Sturm
// count at 32 interior points of the bracket, which shrinks 33-fold per pass (about 11 passes from the
// Gershgorin interval to the resolution 2 eps max|bound|).  The count is non-decreasing in x, so the points
// with count <= k form a prefix of the lanes and the new bracket is read off the ballot.
__global__ void __launch_bounds__(128) tri_multisect_kernel(const double* __restrict__ d,
                                                            const double* __restrict__ e2, int n,
                                                            const double* __restrict__ bounds,
                                                            double* __restrict__ W) {
  const int k = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= n) return;  // whole warps
  double lo = bounds[0], hi = bounds[1];
  const double pivmin = bounds[2];
  const double tol = 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + pivmin;
  for (int it = 0; it < 64 && hi - lo > tol; ++it) {
    const double h = (hi - lo) / 33.0;
    const double x = lo + h * (double)(lane + 1);
    const int cnt = sturm_count(d, e2, n, x, pivmin);
    const unsigned below = __ballot_sync(0xffffffffu, cnt <= k);
    const int nlo = __popc(below);
    const double xlo = __shfl_sync(0xffffffffu, x, max(nlo - 1, 0));
    const double xhi = __shfl_sync(0xffffffffu, x, min(nlo, 31));
    const double nl = nlo > 0 ? xlo : lo;
    const double nh = nlo < 32 ? xhi : hi;
    if (nl == lo && nh == hi) break;  // no representable progress
    lo = nl;
    hi = nh;
  }
  if (lane == 0) W[k] = 0.5 * (lo + hi);
}

}  // namespace

size_t dense_eig_scratch(int n) {
  // v, w, tau (n each, complex), part (chunks x n complex), e, d, e2 (n doubles), bounds
  return sizeof(zd) * ((size_t)3 * n + (size_t)kDenseEigChunks * n) + sizeof(double) * ((size_t)3 * n + 4);
}

cudaError_t launch_dense_eigvals(zd* A, int n, int lda, bool upper_only, double* W, void* scratch,
                                 cudaStream_t s) {
  if (n < 1 || lda < n) return cudaErrorInvalidValue;
  zd* v = reinterpret_cast<zd*>(scratch);
  zd* w = v + n;
  zd* tau = w + n;
  zd* part = tau + n;
  double* e = reinterpret_cast<double*>(part + (size_t)kDenseEigChunks * n);
  double* d = e + n;
  double* e2 = d + n;
  double* bounds = e2 + n;
  if (upper_only) {
    mirror_upper_kernel<<<(unsigned)(((long)n * n + 255) / 256), 256, 0, s>>>(A, n, lda); ++g_launch_count;
  }
  for (int j = 0; j + 1 < n; ++j) {
    const int m = n - j - 1;
    const int rb = (m + kHvRows - 1) / kHvRows;
    // about four CTAs per SM, at least 64 columns per chunk
    const int nchunk = std::max(1, std::min({kDenseEigChunks, (m + 63) / 64, std::max(1, 4 * 152 / rb)}));
    tri_hemv_kernel<<<dim3(rb, nchunk), kHvRows, 0, s>>>(A, n, lda, j, v, tau, e, part); ++g_launch_count;
    tri_w_kernel<<<1, 1024, 0, s>>>(part, nchunk, m, tau, j, v, w); ++g_launch_count;
    const int tb = (m + kH2Tile - 1) / kH2Tile;
    tri_her2_kernel<<<dim3(tb, tb), 256, 0, s>>>(A, n, lda, j, tau, v, w); ++g_launch_count;
  }
  tri_finish_kernel<<<1, 1024, 0, s>>>(A, n, lda, d, e, bounds); ++g_launch_count;
  if (n > 1) {
    e2_kernel<<<(n + 255) / 256, 256, 0, s>>>(e, n, e2); ++g_launch_count;
  }
  tri_multisect_kernel<<<(unsigned)(((long)n * 32 + 127) / 128), 128, 0, s>>>(d, e2, n, bounds, W); ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace wtb
