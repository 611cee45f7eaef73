// All eigenvalues of a dense Hermitian matrix on the device: the stand-in for the LAPACK ZHEEV calls of the
// full-spectrum paths (bsebnds, src/module_bse.F90:1427-1448; the temperature solver's dense path).
//
// 1. Householder tridiagonalisation A = Q T Q^H in FP64, the unblocked zhetd2 sequence (lower form): for
//    column j, the reflector H = I - tau v v^H of zlarfg annihilates A(j+2:n, j); x = tau A22 v;
//    w = x - (tau/2)(x^H v) v; A22 -= v w^H + w v^H, on the lower triangle only.  Four launches per column:
//    the reflector (one CTA), the Hermitian product by 64 x 64 lower tiles (each off-diagonal tile staged
//    in shared memory serves A v and A^H v), the fixed-order sum of the tile partials with the x^H v dots,
//    and the rank-2 update of the lower tiles.  On this GPU the FP64 pipe, not HBM, bounds both: 8 FMAs per
//    stored element and column, 8/3 n^3 FMAs in all.
// 2. Eigenvalues of the real symmetric tridiagonal T by bisection on Sturm counts (dstebz's method), as
//    multisection with a few lanes per eigenvalue index where n alone would leave SMs idle, the count with
//    LAPACK's pivot guard pivmin, to the FP64 resolution of the Gershgorin interval.  Backward stable: |lambda - lambda_exact| <~ n eps ||A||.
#include <cfloat>

#include "wtb_internal.h"

namespace wtb {

namespace {

// Tile edge of the Hermitian product and the rank-2 update: 64 while the trailing block gives at least three
// tiles per SM, then 32, then 16 (the late columns would otherwise run on a handful of CTAs).
constexpr int kMinTiles = 3 * 152;
inline int pick_tile(int m) {
  auto tiles = [m](int t) { const long nt = (m + t - 1) / t; return nt * (nt + 1) / 2; };
  if (tiles(64) >= kMinTiles) return 64;
  if (tiles(32) >= kMinTiles) return 32;
  return 16;
}
// partial-sum buffer: (tiles per column) x m entries, largest over the three tile sizes (from m = 4096 on the
// tile is always 64)
inline size_t p_capacity(int n) {
  size_t cap = (size_t)((n + 63) / 64) * n;
  for (int m = 1; m < std::min(n, 4096); ++m) {
    const int t = pick_tile(m);
    cap = std::max(cap, (size_t)((m + t - 1) / t) * m);
  }
  return cap;
}

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

// Tile (R, C), R >= C, of the lower triangle of an nT x nT tile grid from the linear index b.
__device__ __forceinline__ void lower_tile(int b, int* R, int* C) {
  int r = (int)((sqrtf(8.0f * (float)b + 1.0f) - 1.0f) * 0.5f);  // FP32 guess, corrected exactly below
  while ((r + 1) * (r + 2) / 2 <= b) ++r;
  while (r * (r + 1) / 2 > b) --r;
  *R = r;
  *C = b - r * (r + 1) / 2;
}

// zlarfg on column j (one CTA): v(0) = 1, v(1:) = x(1:) / (alpha - beta), stored in v and below the
// subdiagonal of column j; tau(j), e(j) = beta.
__global__ void __launch_bounds__(256) tri_reflector_kernel(zd* __restrict__ A, int n, int lda, int j,
                                                            zd* __restrict__ v, zd* __restrict__ tau_out,
                                                            double* __restrict__ e_out) {
  __shared__ double red[8];
  __shared__ zd s_scale;
  __shared__ int s_skip;
  const int m = n - j - 1;
  zd* x = A + (size_t)j * lda + j + 1;
  double s2 = 0.0;
  for (int i = 1 + threadIdx.x; i < m; i += blockDim.x) s2 = fma(x[i].re, x[i].re, fma(x[i].im, x[i].im, s2));
  for (int o = 16; o > 0; o >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s2;
  __syncthreads();
  // the scalar FP64 work (sqrt, divisions) on one thread: every warp repeating it would queue on the FP64 pipe
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    const Reflector R = make_reflector(x[0], t);
    tau_out[j] = R.tau;
    e_out[j] = R.beta;
    s_scale = R.scale;
    s_skip = R.tau.re == 0.0 && R.tau.im == 0.0;
  }
  __syncthreads();
  if (s_skip) return;
  const zd sc = s_scale;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    const zd vi = i == 0 ? mk<double>(1.0, 0.0) : cmul(x[i], sc);
    v[i] = vi;
    x[i] = vi;
  }
}

// Lower-triangle Hermitian product p = A22 v by tiles: an off-diagonal tile (R, C) gives A_RC v_C to the rows of
// block R and A_RC^H v_R to the rows of block C; a diagonal tile supplies its upper half from the lower one.
// Each (row block, other block) pair receives exactly one partial, P[other][row], so the sum over the tile
// index is a fixed-order reduction.  4T threads: row (or column) t % T, a quarter of the tile's width each.
template <int T>
__global__ void __launch_bounds__(4 * T) tri_symv_kernel(const zd* __restrict__ A, int n, int lda, int j,
                                                         const zd* __restrict__ v, const zd* __restrict__ tau_p,
                                                         zd* __restrict__ P) {
  constexpr int kSymTile = T, kTPad = T + 1;  // padded column stride: conflict-free transposed reads
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zd* tile = reinterpret_cast<zd*>(smem_raw);    // [kSymTile][kTPad], column-major
  zd* vR = tile + kSymTile * kTPad;
  zd* vC = vR + kSymTile;
  zd* ry = vC + kSymTile;                         // [4][kSymTile]
  zd* rz = ry + 4 * kSymTile;                     // [4][kSymTile]
  const zd tau = tau_p[j];
  if (tau.re == 0.0 && tau.im == 0.0) return;
  const int m = n - j - 1;
  int R, C;
  lower_tile(blockIdx.x, &R, &C);
  const int r0 = R * kSymTile, c0 = C * kSymTile;
  const zd* a22 = A + (size_t)(j + 1) * lda + j + 1;
  for (int e = threadIdx.x; e < kSymTile * kSymTile; e += blockDim.x) {
    const int ii = e % kSymTile, jj = e / kSymTile;
    const int r = r0 + ii, c = c0 + jj;
    tile[jj * kTPad + ii] = (r < m && c < m) ? a22[(size_t)c * lda + r] : mk<double>(0.0, 0.0);
  }
  if (threadIdx.x < kSymTile) {
    const int r = r0 + threadIdx.x, c = c0 + threadIdx.x;
    vR[threadIdx.x] = r < m ? v[r] : mk<double>(0.0, 0.0);
    vC[threadIdx.x] = c < m ? v[c] : mk<double>(0.0, 0.0);
  }
  __syncthreads();
  const bool diag = R == C;
  const int i = threadIdx.x % kSymTile, g = threadIdx.x / kSymTile;
  const int q0 = g * (kSymTile / 4), q1 = q0 + kSymTile / 4;
  zd acc = mk<double>(0.0, 0.0);
  if (!diag) {
    for (int jj = q0; jj < q1; ++jj) cfma(acc, tile[jj * kTPad + i], vC[jj]);
  } else {
    for (int jj = q0; jj < q1; ++jj) {
      zd a;
      if (jj < i)
        a = tile[jj * kTPad + i];
      else if (jj == i)
        a = mk<double>(tile[i * kTPad + i].re, 0.0);
      else
        a = cconj(tile[i * kTPad + jj]);
      cfma(acc, a, vC[jj]);
    }
  }
  ry[g * kSymTile + i] = acc;
  if (!diag) {
    zd accz = mk<double>(0.0, 0.0);
    for (int ii = q0; ii < q1; ++ii) cfmac(accz, tile[i * kTPad + ii], vR[ii]);  // conj(A(ii, i)) vR(ii)
    rz[g * kSymTile + i] = accz;
  }
  __syncthreads();
  if (threadIdx.x < kSymTile) {
    const int t = threadIdx.x;
    zd y = ry[t];
    for (int q = 1; q < 4; ++q) y = cadd(y, ry[q * kSymTile + t]);
    if (r0 + t < m) P[(size_t)C * m + r0 + t] = y;
  } else if (!diag && threadIdx.x < 2 * kSymTile) {
    const int t = threadIdx.x - kSymTile;
    zd z = rz[t];
    for (int q = 1; q < 4; ++q) z = cadd(z, rz[q * kSymTile + t]);
    if (c0 + t < m) P[(size_t)R * m + c0 + t] = z;
  }
}

// x = tau sum_k P[k] and the partial dots conj(x) . v of each CTA.  256 threads = 32 rows x 8 slices of the
// tile index (slice l sums k = l, l+8, ...), the slices then added in order: a fixed-order sum whose serial
// chain is nT/8 loads long.
constexpr int kXRows = 32;
__global__ void __launch_bounds__(256) tri_x_kernel(const zd* __restrict__ P, int nT, int m,
                                                    const zd* __restrict__ tau_p, int j, const zd* __restrict__ v,
                                                    zd* __restrict__ x, zd* __restrict__ dots) {
  __shared__ zd red[8][kXRows];
  const zd tau = tau_p[j];
  if (tau.re == 0.0 && tau.im == 0.0) return;
  const int rr = threadIdx.x % kXRows, sl = threadIdx.x / kXRows;
  const int r = blockIdx.x * kXRows + rr;
  zd p = mk<double>(0.0, 0.0);
  if (r < m)
    for (int k = sl; k < nT; k += 8) p = cadd(p, P[(size_t)k * m + r]);
  red[sl][rr] = p;
  __syncthreads();
  if (threadIdx.x < kXRows) {
    zd t = mk<double>(0.0, 0.0);
    if (r < m) {
      zd q = red[0][rr];
      for (int l = 1; l < 8; ++l) q = cadd(q, red[l][rr]);
      const zd xr = cmul(tau, q);
      x[r] = xr;
      t = cmulc(xr, v[r]);
    }
    for (int o = 16; o > 0; o >>= 1) {
      t.re += __shfl_xor_sync(0xffffffffu, t.re, o);
      t.im += __shfl_xor_sync(0xffffffffu, t.im, o);
    }
    if (threadIdx.x == 0) dots[blockIdx.x] = t;
  }
}

// alpha = -(tau/2) sum_b dots[b], the sum split over one warp's lanes in a fixed order.
__device__ __forceinline__ zd her2_alpha(const zd* __restrict__ dots, int ndots, zd tau) {
  zd d = mk<double>(0.0, 0.0);
  for (int b = threadIdx.x; b < ndots; b += 32) d = cadd(d, dots[b]);
  for (int o = 16; o > 0; o >>= 1) {
    d.re += __shfl_xor_sync(0xffffffffu, d.re, o);
    d.im += __shfl_xor_sync(0xffffffffu, d.im, o);
  }
  return cscale(cmul(tau, d), -0.5);
}

// A22 -= v w^H + w v^H on the lower triangle, w = x - (tau/2)(x^H v) v formed per tile from x and the dots.
// Eight FP64 FMAs per element.
template <int T>
__global__ void __launch_bounds__(4 * T) tri_her2l_kernel(zd* __restrict__ A, int n, int lda, int j,
                                                          const zd* __restrict__ tau_p, const zd* __restrict__ v,
                                                          const zd* __restrict__ x, const zd* __restrict__ dots,
                                                          int ndots) {
  constexpr int kSymTile = T;
  __shared__ zd s_alpha;
  __shared__ zd vR[kSymTile], wR[kSymTile], vC[kSymTile], wC[kSymTile];
  const zd tau = tau_p[j];
  if (tau.re == 0.0 && tau.im == 0.0) return;
  const int m = n - j - 1;
  int R, C;
  lower_tile(blockIdx.x, &R, &C);
  const int r0 = R * kSymTile, c0 = C * kSymTile;
  if (threadIdx.x < 32) {
    const zd al = her2_alpha(dots, ndots, tau);
    if (threadIdx.x == 0) s_alpha = al;
  }
  __syncthreads();
  const zd alpha = s_alpha;
  if (threadIdx.x < kSymTile) {
    const int t = threadIdx.x, r = r0 + t, c = c0 + t;
    const zd z = mk<double>(0.0, 0.0);
    const zd vr = r < m ? v[r] : z, vc = c < m ? v[c] : z;
    vR[t] = vr;
    vC[t] = vc;
    wR[t] = r < m ? cadd(x[r], cmul(alpha, vr)) : z;
    wC[t] = c < m ? cadd(x[c], cmul(alpha, vc)) : z;
  }
  __syncthreads();
  const int i = threadIdx.x % kSymTile, g = threadIdx.x / kSymTile;
  const int r = r0 + i;
  if (r >= m) return;
  zd* a22 = A + (size_t)(j + 1) * lda + j + 1;
  const zd vr = vR[i], wr = wR[i];
  const int q0 = g * (kSymTile / 4);
  const int q1 = min(q0 + kSymTile / 4, R == C ? i + 1 : kSymTile);
  for (int jj = q0; jj < q1; ++jj) {
    const int c = c0 + jj;
    if (c >= m) break;
    const zd vc = vC[jj], wc = wC[jj];
    zd a = a22[(size_t)c * lda + r];
    // a -= vr conj(wc) + wr conj(vc)
    a.re = fma(-vr.re, wc.re, a.re);
    a.re = fma(-vr.im, wc.im, a.re);
    a.re = fma(-wr.re, vc.re, a.re);
    a.re = fma(-wr.im, vc.im, a.re);
    a.im = fma(-vr.im, wc.re, a.im);
    a.im = fma(vr.re, wc.im, a.im);
    a.im = fma(-wr.im, vc.re, a.im);
    a.im = fma(wr.re, vc.im, a.im);
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

// The k-th smallest eigenvalue (k = 0..n-1) by multisection with L lanes per k (L a power of two <= 32): the L
// lanes evaluate the Sturm count at L interior points of the bracket, which shrinks (L+1)-fold per pass, to the
// resolution 2 eps max|bound|.  The count is non-decreasing in x, so the points with count <= k form a prefix
// of the group and the new bracket is read off the ballot.  L = 1 is plain bisection (the fewest counts); the
// launcher raises L only until the GPU's SMs all have work, since a Sturm count (one FP64 division per row)
// queues on the SM's FP64 pipe.  Groups that have converged idle until their whole warp has.
__global__ void __launch_bounds__(128) tri_multisect_kernel(const double* __restrict__ d,
                                                            const double* __restrict__ e2, int n,
                                                            const double* __restrict__ bounds,
                                                            double* __restrict__ W, int L) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int k = tid / L, g = lane % L, base = lane - g;
  const unsigned gmask = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << base);
  double lo = bounds[0], hi = bounds[1];
  const double pivmin = bounds[2];
  const double tol = 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + pivmin;
  bool done = k >= n;
  for (int it = 0; it < 256; ++it) {
    if (!done && !(hi - lo > tol)) done = true;
    if (__all_sync(0xffffffffu, done)) break;
    const double h = (hi - lo) / (double)(L + 1);
    const double x = lo + h * (double)(g + 1);
    const int cnt = done ? 0 : sturm_count(d, e2, n, x, pivmin);
    const unsigned bal = __ballot_sync(0xffffffffu, !done && cnt <= k);
    const int nlo = __popc(bal & gmask);
    const double xlo = __shfl_sync(0xffffffffu, x, base + max(nlo - 1, 0));
    const double xhi = __shfl_sync(0xffffffffu, x, base + min(nlo, L - 1));
    if (!done) {
      const double nl = nlo > 0 ? xlo : lo;
      const double nh = nlo < L ? xhi : hi;
      if (nl == lo && nh == hi)
        done = true;  // no representable progress
      else {
        lo = nl;
        hi = nh;
      }
    }
  }
  if (k < n && g == 0) W[k] = 0.5 * (lo + hi);
}

// ----------------------------------------------------------------------------- eigenvectors
// Inverse iteration on T for every eigenvalue (dstein's method): Gaussian elimination with partial pivoting of
// T - lambda I, three solves from a deterministic start vector, each normalised.  Eigenvalues closer than
// 1e-7 ||T|| to their predecessor form a cluster, handled by one thread in order: later members are shifted
// apart by 10 eps ||T|| and reorthogonalised against the earlier ones after every solve (a degenerate pair
// then spans its eigenspace).  Outside clusters the vectors are orthogonal to eps ||T|| / gap <= 2e-9.
// One thread per cluster start; its scratch (6 arrays of n) is interleaved across the batch's threads so the
// row loops are coalesced.  Zt(i, k) = Zt[i * n + k] (row-major real).
constexpr int kInvIters = 3;

// deterministic start entries in [-1, 1): splitmix64 of (k, i)
__device__ __forceinline__ double start_entry(unsigned long long k, unsigned long long i) {
  unsigned long long z = k * 0x9E3779B97F4A7C15ull + (i + 1) * 0xD1B54A32D192ED03ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

__global__ void __launch_bounds__(128) tri_invit_kernel(const double* __restrict__ d, const double* __restrict__ e,
                                                        int n, const double* __restrict__ W,
                                                        const double* __restrict__ bounds, int k0, int nb,
                                                        double* __restrict__ work, double* __restrict__ Zt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = k0 + t;
  if (t >= nb || k >= n) return;
  const double tnorm = fmax(fmax(fabs(bounds[0]), fabs(bounds[1])), DBL_MIN);
  const double ortol = 1e-7 * tnorm;
  if (k > 0 && W[k] - W[k - 1] < ortol) return;  // inside a cluster started by an earlier thread
  int kend = k + 1;
  while (kend < n && W[kend] - W[kend - 1] < ortol) ++kend;
  const size_t st = (size_t)nb;
  double* a = work + t;             // diagonal of U
  double* b = a + (size_t)n * st;   // first superdiagonal of U
  double* dd = b + (size_t)n * st;  // second superdiagonal of U
  double* c = dd + (size_t)n * st;  // multipliers
  double* pv = c + (size_t)n * st;  // 1 where rows i, i+1 were swapped
  double* y = pv + (size_t)n * st;  // iterate
#define AT(arr, i) arr[(size_t)(i) * st]
  const double tiny = DBL_EPSILON * tnorm;
  double lam_prev = 0.0;
  for (int q = k; q < kend; ++q) {
    double lam = W[q];
    if (q > k && lam - lam_prev < 10.0 * DBL_EPSILON * tnorm) lam = lam_prev + 10.0 * DBL_EPSILON * tnorm;
    lam_prev = lam;
    // T - lam I = P L U
    for (int i = 0; i < n; ++i) {
      AT(a, i) = d[i] - lam;
      AT(b, i) = i < n - 1 ? e[i] : 0.0;
    }
    for (int i = 0; i + 1 < n; ++i) {
      const double sub = e[i], ai = AT(a, i);
      if (fabs(ai) >= fabs(sub)) {
        const double m = ai == 0.0 ? 0.0 : sub / ai;
        AT(c, i) = m;
        AT(pv, i) = 0.0;
        AT(dd, i) = 0.0;
        AT(a, i + 1) = AT(a, i + 1) - m * AT(b, i);
      } else {
        const double m = ai / sub;
        const double a1 = AT(a, i + 1), bi = AT(b, i), b1 = i + 2 < n ? AT(b, i + 1) : 0.0;
        AT(a, i) = sub;
        AT(b, i) = a1;
        AT(dd, i) = b1;
        AT(a, i + 1) = bi - m * a1;
        if (i + 2 < n) AT(b, i + 1) = -m * b1;
        AT(c, i) = m;
        AT(pv, i) = 1.0;
      }
    }
    for (int i = 0; i < n; ++i)
      if (fabs(AT(a, i)) < tiny) AT(a, i) = AT(a, i) < 0.0 ? -tiny : tiny;
    for (int i = 0; i < n; ++i) AT(y, i) = start_entry((unsigned long long)q, (unsigned long long)i);
    for (int it = 0; it < kInvIters; ++it) {
      for (int i = 0; i + 1 < n; ++i) {
        if (AT(pv, i) != 0.0) {
          const double tmp = AT(y, i);
          AT(y, i) = AT(y, i + 1);
          AT(y, i + 1) = tmp;
        }
        AT(y, i + 1) = AT(y, i + 1) - AT(c, i) * AT(y, i);
      }
      for (int i = n - 1; i >= 0; --i) {
        double r = AT(y, i);
        if (i + 1 < n) r -= AT(b, i) * AT(y, i + 1);
        if (i + 2 < n) r -= AT(dd, i) * AT(y, i + 2);
        AT(y, i) = r / AT(a, i);
      }
      // against the cluster's earlier members, then to unit length
      for (int p = k; p < q; ++p) {
        double dot = 0.0;
        for (int i = 0; i < n; ++i) dot += AT(y, i) * Zt[(size_t)i * n + p];
        for (int i = 0; i < n; ++i) AT(y, i) -= dot * Zt[(size_t)i * n + p];
      }
      double mx = 0.0;
      for (int i = 0; i < n; ++i) mx = fmax(mx, fabs(AT(y, i)));
      const double sc = mx > 0.0 ? 1.0 / mx : 1.0;
      double nrm2 = 0.0;
      for (int i = 0; i < n; ++i) {
        const double v = AT(y, i) * sc;
        AT(y, i) = v;
        nrm2 += v * v;
      }
      const double inv = 1.0 / sqrt(nrm2);
      for (int i = 0; i < n; ++i) AT(y, i) *= inv;
    }
    for (int i = 0; i < n; ++i) Zt[(size_t)i * n + q] = AT(y, i);
  }
#undef AT
}

constexpr int kBtCols = 8;  // eigenvector columns per CTA of the back-transformation

// Z = Q Zt with Q = H_0 H_1 ... H_{n-2}, H_j = I - tau_j v_j v_j^H (v_j in A(j+1:n, j), v_j(0) = 1): the
// reflectors applied from j = n-2 down to 0 to every column.  A CTA owns 8 columns and 32 row slices (row i in
// slice i % 32) for the whole sweep, so the columns need no synchronisation between CTAs; per reflector a
// two-barrier reduction of v^H z.  Z(i, k) = Z[i * n + k] (row-major), conjugated at the end when the solver
// worked on conj(H).
__global__ void __launch_bounds__(256) tri_backtransform_kernel(const zd* __restrict__ A, int n, int lda,
                                                                const zd* __restrict__ tau,
                                                                const double* __restrict__ Zt, zd* __restrict__ Z,
                                                                int conj_out) {
  __shared__ zd red[8][kBtCols];
  __shared__ zd dots[kBtCols];
  const int c = threadIdx.x % kBtCols, sl = threadIdx.x / kBtCols;
  const int k = blockIdx.x * kBtCols + c;
  const bool kv = k < n;
  for (int i = sl; i < n; i += 32)
    if (kv) Z[(size_t)i * n + k] = mk<double>(Zt[(size_t)i * n + k], 0.0);
  for (int j = n - 2; j >= 0; --j) {
    const zd tj = tau[j];
    if (tj.re == 0.0 && tj.im == 0.0) continue;
    const zd* v = A + (size_t)j * lda + j + 1;  // v(i - j - 1) for rows i > j
    const int i0 = j + 1 + (((sl - (j + 1)) % 32) + 32) % 32;
    zd p = mk<double>(0.0, 0.0);
    if (kv)
      for (int i = i0; i < n; i += 32) cfmac(p, v[i - j - 1], Z[(size_t)i * n + k]);
    for (int o = kBtCols; o < 32; o <<= 1) {
      p.re += __shfl_xor_sync(0xffffffffu, p.re, o);
      p.im += __shfl_xor_sync(0xffffffffu, p.im, o);
    }
    if ((threadIdx.x & 31) < kBtCols) red[threadIdx.x >> 5][c] = p;
    __syncthreads();
    if (threadIdx.x < kBtCols) {
      zd t = red[0][threadIdx.x];
      for (int w = 1; w < 8; ++w) t = cadd(t, red[w][threadIdx.x]);
      dots[threadIdx.x] = cmul(tj, t);
    }
    __syncthreads();
    const zd f = dots[c];
    if (kv)
      for (int i = i0; i < n; i += 32) {
        zd z = Z[(size_t)i * n + k];
        const zd vi = v[i - j - 1];
        // z -= vi * f
        z.re = fma(-vi.re, f.re, fma(vi.im, f.im, z.re));
        z.im = fma(-vi.re, f.im, fma(-vi.im, f.re, z.im));
        Z[(size_t)i * n + k] = z;
      }
  }
  if (conj_out && kv)
    for (int i = sl; i < n; i += 32) Z[(size_t)i * n + k].im = -Z[(size_t)i * n + k].im;
}

}  // namespace

size_t dense_eig_scratch(int n) {
  // v, x, tau (n each), dots, P, all complex; e, d, e2 (n doubles); bounds
  const size_t nd = (size_t)(n + kXRows - 1) / kXRows;
  return sizeof(zd) * ((size_t)3 * n + nd + p_capacity(n)) + sizeof(double) * ((size_t)3 * n + 4);
}

cudaError_t dense_eig_prepare() {
  cudaError_t err = raise_smem_limit(reinterpret_cast<const void*>(tri_symv_kernel<64>), sizeof(zd) * (64 * 65 + 640));
  if (err == cudaSuccess)
    err = raise_smem_limit(reinterpret_cast<const void*>(tri_symv_kernel<32>), sizeof(zd) * (32 * 33 + 320));
  if (err == cudaSuccess)
    err = raise_smem_limit(reinterpret_cast<const void*>(tri_symv_kernel<16>), sizeof(zd) * (16 * 17 + 160));
  return err;
}

template <int T>
static cudaError_t tri_step(zd* A, int n, int lda, int j, zd* v, zd* tau, zd* P, zd* x, zd* dots, cudaStream_t s) {
  const int m = n - j - 1;
  const int nT = (m + T - 1) / T;
  const unsigned ntiles = (unsigned)((long)nT * (nT + 1) / 2);
  const int nd = (m + kXRows - 1) / kXRows;
  const size_t smem = sizeof(zd) * ((size_t)T * (T + 1) + 10 * T);
  cudaError_t err = raise_smem_limit(reinterpret_cast<const void*>(tri_symv_kernel<T>), smem);
  if (err != cudaSuccess) return err;
  tri_symv_kernel<T><<<ntiles, 4 * T, smem, s>>>(A, n, lda, j, v, tau, P); ++g_launch_count;
  tri_x_kernel<<<nd, 8 * kXRows, 0, s>>>(P, nT, m, tau, j, v, x, dots); ++g_launch_count;
  tri_her2l_kernel<T><<<ntiles, 4 * T, 0, s>>>(A, n, lda, j, tau, v, x, dots, nd); ++g_launch_count;
  return cudaSuccess;
}

static int invit_batch(int n) {
  const long nb = (1L << 25) / (6L * n);  // the inverse-iteration scratch stays near 256 MB
  return (int)std::max(1L, std::min((long)n, nb));
}

size_t dense_eigvec_scratch(int n) {
  return sizeof(double) * ((size_t)n * n + (size_t)6 * n * invit_batch(n));
}

cudaError_t launch_dense_eigvals(zd* A, int n, int lda, bool upper_only, double* W, void* scratch,
                                 cudaStream_t s) {
  return launch_dense_eig(A, n, lda, upper_only, W, nullptr, false, scratch, nullptr, s);
}

cudaError_t launch_dense_eig(zd* A, int n, int lda, bool upper_only, double* W, zd* Z, bool conj_vectors,
                             void* scratch, void* vscratch, cudaStream_t s) {
  if (Z && !vscratch) return cudaErrorInvalidValue;
  if (n < 1 || lda < n) return cudaErrorInvalidValue;
  const size_t ndmax = (size_t)(n + kXRows - 1) / kXRows;
  zd* v = reinterpret_cast<zd*>(scratch);
  zd* x = v + n;
  zd* tau = x + n;
  zd* dots = tau + n;
  zd* P = dots + ndmax;
  double* e = reinterpret_cast<double*>(P + p_capacity(n));
  double* d = e + n;
  double* e2 = d + n;
  double* bounds = e2 + n;
  if (upper_only) {
    mirror_upper_kernel<<<(unsigned)(((long)n * n + 255) / 256), 256, 0, s>>>(A, n, lda); ++g_launch_count;
  }
  for (int j = 0; j + 1 < n; ++j) {
    const int m = n - j - 1;
    tri_reflector_kernel<<<1, 256, 0, s>>>(A, n, lda, j, v, tau, e); ++g_launch_count;
    const int T = pick_tile(m);
    const cudaError_t err = T == 64 ? tri_step<64>(A, n, lda, j, v, tau, P, x, dots, s)
                            : T == 32 ? tri_step<32>(A, n, lda, j, v, tau, P, x, dots, s)
                                      : tri_step<16>(A, n, lda, j, v, tau, P, x, dots, s);
    if (err != cudaSuccess) return err;
  }
  tri_finish_kernel<<<1, 1024, 0, s>>>(A, n, lda, d, e, bounds); ++g_launch_count;
  if (n > 1) {
    e2_kernel<<<(n + 255) / 256, 256, 0, s>>>(e, n, e2); ++g_launch_count;
  }
  int L = 1;  // about two warps per SM
  while (L < 32 && (long)n * L < 152L * 64) L *= 2;
  tri_multisect_kernel<<<(unsigned)(((long)n * L + 127) / 128), 128, 0, s>>>(d, e2, n, bounds, W, L); ++g_launch_count;
  if (Z) {
    double* Zt = reinterpret_cast<double*>(vscratch);
    double* work = Zt + (size_t)n * n;
    const int nb = invit_batch(n);
    for (int k0 = 0; k0 < n; k0 += nb) {
      tri_invit_kernel<<<(nb + 127) / 128, 128, 0, s>>>(d, e, n, W, bounds, k0, nb, work, Zt); ++g_launch_count;
    }
    tri_backtransform_kernel<<<(n + kBtCols - 1) / kBtCols, 256, 0, s>>>(A, n, lda, tau, Zt, Z, conj_vectors ? 1 : 0);
    ++g_launch_count;
  }
  return cudaGetLastError();
}

}  // namespace wtb
