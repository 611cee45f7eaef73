// Oscillator strengths and the broadened dielectric spectrum.
//
// dielbsev / dielbsep (src/module_bse.F90:171-245): with s_a(n) = sum_j A(j,n) h_a(j) (no conjugate on
// A, as in the reference), f_aa(n) = |s_a|^2 and f_ab(n) = Re(s_a conj(s_b)).
// bsedielraw + optdiel + avgsme + imagrenorm (src/module_bse.F90:835-1036, src/module_optics.F90:171-401):
//   omega_j = E0 + (Ef - E0)(j-1)/(N-1),   gamma = CSHIFT + 10 * (sum_{i>=2} (E_i - E_{i-1})) / nrows,
//   eps2(omega) = C sum_n f_n gamma / ((omega - E_n)^2 + gamma^2),
//   eps1(omega) = delta + C sum_n f_n (E_n - omega) / ((omega - E_n)^2 + gamma^2),  C = 180.90_f32 / (Nk Vol)
// then the optional baseline renormalisation of eps2 and the spin factor.  bsedielrawpol, spdielraw and
// spdielrawpol (src/module_bse.F90:1043-1199, :4090-4524) run the same sums over other columns: xx yy zz sp sm
// all with rtype 1, and the IPA records of spoptics (:4802-5071) sorted by Bubblem (src/module_math.F90:287-308).
// bseoptprop (src/module_bse.F90:3766-3931, :5075-5124): refractive index, extinction, reflectivity,
// absorption coefficient sqrt(2)_f32 * omega / hc_f32 * sqrt(|eps| - eps1), loss function.
#include "wtb_internal.h"

namespace wtb {

namespace {

constexpr int kOscRows = 256;

// Partial sums s_a(n) = sum_r A(r, n) h_a(r) over a CTA's kOscRows rows, a = x y z sp sm.  The eight warps
// take interleaved rows, a lane takes exciton n (lanes beyond nev idle; nev > 32 loops), and the warps'
// sums are added in a fixed order through shared memory: the FP64 work is spread over the SM's four
// schedulers instead of the few threads of one warp.
__global__ void __launch_bounds__(256) osc_partial_kernel(const zd* __restrict__ A, int lda, int nev, int dim,
                                                          const zd* __restrict__ hr, double* __restrict__ partial) {
  __shared__ zd hs[5][kOscRows];
  __shared__ double red[8][32][2];
  const int r0 = blockIdx.x * kOscRows;
  const int nr = min(kOscRows, dim - r0);
  for (int e = threadIdx.x; e < 5 * kOscRows; e += blockDim.x) {
    const int a = e / kOscRows, r = e % kOscRows;
    hs[a][r] = r < nr ? hr[(size_t)a * dim + r0 + r] : mk<double>(0.0, 0.0);
  }
  __syncthreads();
  // lanes along (exciton n, component a) pairs, 32 per pass (the FP64 pipe then serves up to 32 useful lanes of a
  // warp instruction, not nev); each warp adds its rows r = warp, warp + 8, ... in order, then the 8 warp sums
  // are added in warp order
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int npair = nev * 5;
  for (int q0 = 0; q0 < npair; q0 += 32) {
    const int q = q0 + lane, n = q / 5, a = q - 5 * n;
    zd acc = mk<double>(0.0, 0.0);
    if (q < npair)
      for (int r = warp; r < nr; r += 8) cfma(acc, A[(size_t)(r0 + r) * lda + n], hs[a][r]);
    red[warp][lane][0] = acc.re;
    red[warp][lane][1] = acc.im;
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * 2; e += blockDim.x) {
      const int l = e >> 1, ri = e & 1, qq = q0 + l;
      if (qq >= npair) continue;
      double t = 0.0;
      for (int w = 0; w < 8; ++w) t += red[w][l][ri];
      const int nn = qq / 5, aa = qq - 5 * nn;
      partial[((size_t)blockIdx.x * nev + nn) * 10 + 2 * aa + ri] = t;
    }
    __syncthreads();
  }
}

// one warp per exciton: lane l adds the blocks b = l, l + 32, ... in order, then a fixed butterfly over the lanes
__global__ void __launch_bounds__(256) osc_final_kernel(const double* __restrict__ partial, int nblk, int nev,
                                                        double* __restrict__ osc) {
  const int lane = threadIdx.x & 31;
  const int n = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (n >= nev) return;  // warp-uniform
  double v[10];
#pragma unroll
  for (int q = 0; q < 10; ++q) v[q] = 0.0;
  for (int b = lane; b < nblk; b += 32) {
    const double* p = partial + ((size_t)b * nev + n) * 10;
#pragma unroll
    for (int q = 0; q < 10; ++q) v[q] += p[q];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < 10; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
  if (lane != 0) return;
  zd s[5];
#pragma unroll
  for (int a = 0; a < 5; ++a) s[a] = mk<double>(v[2 * a], v[2 * a + 1]);
  auto re_prod = [](zd a, zd b) { return a.re * b.re + a.im * b.im; };  // Re(a conj(b))
  osc[0 * nev + n] = re_prod(s[0], s[0]);
  osc[1 * nev + n] = re_prod(s[1], s[1]);
  osc[2 * nev + n] = re_prod(s[2], s[2]);
  osc[3 * nev + n] = re_prod(s[0], s[1]);
  osc[4 * nev + n] = re_prod(s[0], s[2]);
  osc[5 * nev + n] = re_prod(s[1], s[2]);
  osc[6 * nev + n] = re_prod(s[3], s[3]);
  osc[7 * nev + n] = re_prod(s[4], s[4]);
}

// smef = CSHIFT + 10 * (sum_{i>=1} (E_i - E_{i-1})) / nrows  (fixed-order tree reduction)
// Also records in smef[1] the end of the last row with a nonzero activity in any component: rows past it add
// exactly zero to every Lorentzian sum (bsesolver leaves the rows past nev at zero).
__global__ void __launch_bounds__(1024) avgsme_kernel(const double* __restrict__ Ws, int nrows, double sme,
                                                      const double* __restrict__ f, int ncomp,
                                                      double* __restrict__ smef) {
  __shared__ double red[1024];
  __shared__ int s_last;
  if (threadIdx.x == 0) s_last = 0;
  double acc = 0.0;
  const int chunk = (nrows + blockDim.x - 1) / blockDim.x;
  const int i0 = threadIdx.x * chunk;
  int last = 0;
  for (int i = max(i0, 1); i < min(nrows, i0 + chunk); ++i) acc = acc + Ws[i] - Ws[i - 1];
  for (int i = i0; i < min(nrows, i0 + chunk); ++i)
    for (int c = 0; c < ncomp; ++c)
      if (f[(size_t)c * nrows + i] != 0.0) last = i + 1;
  red[threadIdx.x] = acc;
  __syncthreads();
  if (last) atomicMax(&s_last, last);
  for (int off = blockDim.x / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    smef[0] = 10.0 * (red[0] / (double)nrows) + sme;
    smef[1] = (double)s_last;
  }
}

constexpr int kLorOmega = 128;  // photon energies per CTA (one per thread)
constexpr int kLorRows = 256;   // rows staged in shared memory at a time

__device__ __forceinline__ double omega_of(double e0, double ef, int nesp, int j) {
  return e0 + ((ef - e0) * (double)j) / ((double)nesp - 1.0);
}

// Partial Lorentzian sums of optdiel over one chunk of the rows, all NC components at once: the two
// quotients (E - omega) / eaux and gamma / eaux do not depend on the component, so each (row, omega) pair
// costs one FP64 division (1/eaux) instead of two per component, and the products f_c * quotient are the
// reference's own.  A thread owns one photon energy; the chunk's rows pass through shared memory.
// part[chunk][c][0: real, 1: imaginary][nesp].
template <int NC>
__global__ void __launch_bounds__(kLorOmega) lorentz_partial_kernel(const double* __restrict__ Ws, int nrows,
                                                                    const double* __restrict__ f,
                                                                    const double* __restrict__ smef_p, double e0,
                                                                    double ef, int nesp, double* __restrict__ part) {
  __shared__ double sW[kLorRows];
  __shared__ double sf[NC][kLorRows];
  const int j = blockIdx.x * kLorOmega + threadIdx.x;
  const int nchunk = gridDim.y, ch = blockIdx.y;
  const int nuse = min(nrows, (int)smef_p[1]);
  const int per = (nuse + nchunk - 1) / nchunk;
  const int r0 = min(nuse, ch * per), r1 = min(nuse, r0 + per);
  const double smef = smef_p[0];
  const double elux = omega_of(e0, ef, nesp, j);
  double rp[NC], ip[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) rp[c] = ip[c] = 0.0;
  for (int t0 = r0; t0 < r1; t0 += kLorRows) {
    const int nt = min(kLorRows, r1 - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < (NC + 1) * kLorRows; e += kLorOmega) {
      const int q = e / kLorRows, r = e % kLorRows;
      if (r >= nt) continue;
      if (q == 0)
        sW[r] = Ws[t0 + r];
      else
        sf[q - 1][r] = f[(size_t)(q - 1) * nrows + t0 + r];
    }
    __syncthreads();
    if (j < nesp)
      for (int r = 0; r < nt; ++r) {
        const double ex = sW[r];
        const double eaux = ((elux - ex) * (elux - ex)) + (smef * smef);
        // one FP64 division per pair (the FP64 pipe bounds this kernel): the quotients as products with 1/eaux,
        // within an ulp of the reference's two divisions
        const double ie = 1.0 / eaux;
        const double q1 = (ex - elux) * ie;
        const double q2 = smef * ie;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          rp[c] += sf[c][r] * q1;
          ip[c] += sf[c][r] * q2;
        }
      }
  }
  if (j >= nesp) return;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    double* o = part + ((size_t)ch * NC + c) * 2 * nesp + j;
    o[0] = rp[c];
    o[nesp] = ip[c];
  }
}

// Adds the chunks in order and applies optdiel's epilogue: eps1 = delta + C * rpart, eps2 = C * ipart, with
// delta = 1 for the components whose bit is set in delta_mask (rtype 1) and 0 otherwise.
// Fortran layout dielf(nesp, 3, ncomp): (j, c, comp) at j + nesp*(c + 3*comp).
__global__ void lorentz_final_kernel(const double* __restrict__ part, int nchunk, int ncomp, unsigned delta_mask,
                                     double caux, double e0, double ef, int nesp, double* __restrict__ dielf) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ncomp * nesp) return;
  const int comp = e / nesp, j = e % nesp;
  double rpart = 0.0, ipart = 0.0;
  for (int ch = 0; ch < nchunk; ++ch) {
    const double* o = part + ((size_t)ch * ncomp + comp) * 2 * nesp + j;
    rpart += o[0];
    ipart += o[nesp];
  }
  const double delta = (delta_mask >> comp) & 1u ? 1.0 : 0.0;
  double* d = dielf + (size_t)comp * 3 * nesp + j;
  d[0] = omega_of(e0, ef, nesp, j);
  d[nesp] = delta + rpart * caux;
  d[2 * nesp] = ipart * caux;
}

// imagrenorm on eps2 of each component, then the spin factor (src/module_optics.F90:338-401).
__global__ void renorm_kernel(const double* __restrict__ Ws, int nesp, int renorm, double spinf,
                              double* __restrict__ dielf) {
  const int comp = blockIdx.x;
  double* om = dielf + (size_t)comp * nesp * 3;
  double* e1 = om + nesp;
  double* e2 = om + 2 * nesp;
  __shared__ int s_ib;
  __shared__ double s_aux3;
  __shared__ int s_do;
  if (threadIdx.x == 0) {
    s_do = 0;
    const double aux = Ws[0] - (double)0.15f;
    if (renorm && aux > 0.0) {
      int ib = 0;
      for (int i = 0; i < nesp; ++i) {
        if (om[i] <= aux)
          ib = i;
        else
          break;
      }
      if (ib + 1 < nesp) {
        s_ib = ib;
        s_aux3 = e2[ib + 1];
        s_do = 1;
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nesp; i += blockDim.x) {
    double v = e2[i];
    if (s_do) {
      if (i <= s_ib) {
        v = 0.0;
      } else {
        v = v - s_aux3;
        if (v < 0.0) v = 0.0;
      }
    }
    e1[i] *= spinf;
    e2[i] = v * spinf;
  }
}

__global__ void optprops_kernel(const double* __restrict__ dielf, int nesp, int ncomp, double* __restrict__ props) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;  // e = comp * nesp + j
  if (e >= ncomp * nesp) return;
  const int comp = e / nesp, j = e % nesp;
  const double* d = dielf + (size_t)comp * 3 * nesp + j;
  const double om = d[0], e1 = d[nesp], e2 = d[2 * nesp];
  const double aux = sqrt((e1 * e1) + (e2 * e2));
  const double n = sqrt((aux + e1) / 2.0);
  const double kap = sqrt((aux - e1) / 2.0);
  const double refl = (((n - 1.0) * (n - 1.0)) + kap * kap) / (((n + 1.0) * (n + 1.0)) + kap * kap);
  const double hc = (double)19.746E-06f;
  const double absc = ((double)1.41421354f * om) * (1.0 / hc) * sqrt(aux - e1);
  const double eloss = e2 / ((e1 * e1) + (e2 * e2));
  const size_t plane = (size_t)ncomp * nesp;
  props[0 * plane + e] = n;
  props[1 * plane + e] = kap;
  props[2 * plane + e] = refl;
  props[3 * plane + e] = absc;
  props[4 * plane + e] = eloss;
}

// The IPA transition records of spoptics (src/module_bse.F90:4969-4990; bsesolver writes the same,
// :2317-2348) in REAL(4), column-major rec(dim, 15):
//   kx ky kz, nocp, nocp - nv + c, nocp - nv + v, E_c - E_v, |hx|^2 |hy|^2 |hz|^2, Re(hx hy*) Re(hx hz*)
//   Re(hy hz*), |hsp|^2 |hsm|^2
// with c = nv+1..nv+nc and v = 1..nv the band slots of basis row I = (k, c, v) (quantumnumbers2).  key(I) is
// column 7, the sort key of Bubblem.
// With f (bsesolvertemp's records, src/module_bse.F90:2649-3263, lines 299-306 of its body) the eight activity
// columns are weighted by f_v - f_c before the rounding to REAL(4).
__global__ void sp_records_kernel(const double* __restrict__ kpt, const int* __restrict__ nocp,
                                  const double* __restrict__ eig_win, const zd* __restrict__ hr, int nk, int nv,
                                  int nc, const double* __restrict__ f, float* __restrict__ rec,
                                  float* __restrict__ key) {
  const long I = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long dim = (long)nk * nc * nv;
  if (I >= dim) return;
  const int k = (int)(I / (nc * nv)), c = (int)((I / nv) % nc), v = (int)(I % nv);
  const int nb = nv + nc, no = nocp[k];
  const double de = eig_win[(size_t)k * nb + nv + c] - eig_win[(size_t)k * nb + v];
  zd h[5];
#pragma unroll
  for (int a = 0; a < 5; ++a) h[a] = hr[(size_t)a * dim + I];
  auto re_prod = [](zd a, zd b) { return a.re * b.re + a.im * b.im; };  // Re(a conj(b))
  float* r = rec + I;
  r[0 * dim] = (float)kpt[3 * k];
  r[1 * dim] = (float)kpt[3 * k + 1];
  r[2 * dim] = (float)kpt[3 * k + 2];
  r[3 * dim] = (float)no;
  r[4 * dim] = (float)(no + c + 1);
  r[5 * dim] = (float)(no - nv + v + 1);
  r[6 * dim] = (float)de;
  const double w = f ? f[I] : 1.0;
  auto act = [w, f](double v) { return (float)(f ? v * w : v); };
  r[7 * dim] = act(re_prod(h[0], h[0]));
  r[8 * dim] = act(re_prod(h[1], h[1]));
  r[9 * dim] = act(re_prod(h[2], h[2]));
  r[10 * dim] = act(re_prod(h[0], h[1]));
  r[11 * dim] = act(re_prod(h[0], h[2]));
  r[12 * dim] = act(re_prod(h[1], h[2]));
  r[13 * dim] = act(re_prod(h[3], h[3]));
  r[14 * dim] = act(re_prod(h[4], h[4]));
  key[I] = (float)de;
}

constexpr int kRankThreads = 256;
constexpr int kRankTile = 2048;

// Bubblem (src/module_math.F90:287-308) is a bubble sort that swaps adjacent rows only when the upper key is
// strictly greater: a stable ascending sort.  Row i therefore lands at
//   rank(i) = #{j : key_j < key_i} + #{j < i : key_j == key_i}
// (float comparisons, so -0 and +0 tie as in the reference).  Every count is exact whatever the order of
// the additions; the keys pass through shared memory in tiles and blockIdx.y splits the j range.
__global__ void __launch_bounds__(kRankThreads) stable_rank_kernel(const float* __restrict__ key, int n,
                                                                   int* __restrict__ rank) {
  __shared__ float sk[kRankTile];
  const int i = blockIdx.x * kRankThreads + threadIdx.x;
  const float ki = i < n ? key[i] : 0.0f;
  const int per = (n + gridDim.y - 1) / gridDim.y;
  const int j0 = min(n, (int)blockIdx.y * per), j1 = min(n, j0 + per);
  int cnt = 0;
  for (int t0 = j0; t0 < j1; t0 += kRankTile) {
    const int nt = min(kRankTile, j1 - t0);
    __syncthreads();
    for (int e = threadIdx.x; e < nt; e += kRankThreads) sk[e] = key[t0 + e];
    __syncthreads();
    if (i < n) {
      const int lim = i - t0;  // tile rows below this bound come before row i
      for (int r = 0; r < nt; ++r) {
        const float kj = sk[r];
        cnt += (kj < ki) | ((kj == ki) & (r < lim));
      }
    }
  }
  if (i < n && cnt) atomicAdd(&rank[i], cnt);
}

__global__ void permute_rows_kernel(const float* __restrict__ in, const int* __restrict__ rank, int n, int ncol,
                                    float* __restrict__ out) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)n * ncol) return;
  const int q = (int)(e / n), i = (int)(e % n);
  const int r = rank[i];
  if (r >= 0 && r < n) out[(size_t)q * n + r] = in[e];
}

// spoptpolbz (src/module_bse.F90:4532-4797) per k-point: h_a = <c|dH/dk_a|v> / (E_c - E_v + i sme) (optspbz and
// the complex division, src/module_optics.F90:257-311), summed |h_a|^2 over the nc x nv transitions for a = x y z,
// |n (h_x +- i h_y)|^2 with n = 1/sqrt(2) in single precision for sp / sm, and (sp - sm)/(sp + sm).  The reference
// takes the valence bands up to nocp of the first k-point at every k; the window here is each k-point's own, so
// a mesh whose occupied count varies (a metal) is refused (status 103).
__global__ void bz_activity_kernel(const zd* __restrict__ hraw, const double* __restrict__ eig_win,
                                   const int* __restrict__ nocp, int nk, int nv, int nc, double sme,
                                   double* __restrict__ act, DevStatus* st) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  if (nocp[k] != nocp[0]) {
    dev_fail(st, 103, k);
    return;
  }
  const int nb = nv + nc, dimk = nc * nv;
  const size_t dim = (size_t)nk * dimk;
  const double nrm = (double)0.70710677f;
  double sx = 0.0, sy = 0.0, sz = 0.0, sp = 0.0, sm = 0.0;
  for (int e = 0; e < dimk; ++e) {
    const int c = e / nv, v = e % nv;
    const double de = eig_win[(size_t)k * nb + nv + c] - eig_win[(size_t)k * nb + v];
    const double den = de * de + sme * sme;
    zd h[3];
    for (int a = 0; a < 3; ++a) {
      const zd r = hraw[(size_t)a * dim + (size_t)k * dimk + e];
      // r / (de + i sme) = r (de - i sme) / den
      h[a] = mk<double>((r.re * de + r.im * sme) / den, (r.im * de - r.re * sme) / den);
    }
    sx += h[0].re * h[0].re + h[0].im * h[0].im;
    sy += h[1].re * h[1].re + h[1].im * h[1].im;
    sz += h[2].re * h[2].re + h[2].im * h[2].im;
    const zd p = mk<double>(nrm * (h[0].re - h[1].im), nrm * (h[0].im + h[1].re));  // n (hx + i hy)
    const zd q = mk<double>(nrm * (h[0].re + h[1].im), nrm * (h[0].im - h[1].re));  // n (hx - i hy)
    sp += p.re * p.re + p.im * p.im;
    sm += q.re * q.re + q.im * q.im;
  }
  act[0 * (size_t)nk + k] = sx;
  act[1 * (size_t)nk + k] = sy;
  act[2 * (size_t)nk + k] = sz;
  act[3 * (size_t)nk + k] = sp;
  act[4 * (size_t)nk + k] = sm;
  act[5 * (size_t)nk + k] = (sp - sm) / (sp + sm);
}

}  // namespace

cudaError_t launch_oscillators(const zd* A, int lda, int nev, int dim, const zd* hr, double* osc, double* partial,
                               int npart, cudaStream_t s) {
  const int nblk = (dim + kOscRows - 1) / kOscRows;
  if (nblk > npart) return cudaErrorInvalidValue;
  osc_partial_kernel<<<nblk, 256, 0, s>>>(A, lda, nev, dim, hr, partial); ++g_launch_count;
  osc_final_kernel<<<(nev + 7) / 8, 256, 0, s>>>(partial, nblk, nev, osc); ++g_launch_count;
  return cudaGetLastError();
}

namespace {
// Row chunks of the Lorentzian sums: at least 512 rows each, and about four CTAs per SM over the photon grid.
int lorentz_chunks(int nrows, int nesp) {
  const int gx = (nesp + kLorOmega - 1) / kLorOmega;
  const int want = (nrows + 2 * kLorRows - 1) / (2 * kLorRows);
  return std::max(1, std::min(want, std::max(1, 4 * 152 / gx)));
}
}  // namespace

size_t spectrum_partial_len(int nrows, int nesp, int ncomp) {
  return 2 + (size_t)lorentz_chunks(nrows, nesp) * ncomp * 2 * nesp;
}

cudaError_t launch_spectrum(const double* Ws, int nrows, const double* f, int ncomp, unsigned delta_mask, double sme,
                            double vc, int ng, double e0, double ef, int nesp, int renorm, double spinf,
                            double* dielf, double* partial, size_t partial_len, cudaStream_t s) {
  if ((ncomp != 5 && ncomp != 6) || nrows < 1 || nesp < 2) return cudaErrorInvalidValue;
  if (partial_len < spectrum_partial_len(nrows, nesp, ncomp)) return cudaErrorInvalidValue;
  const int nchunk = lorentz_chunks(nrows, nesp);
  avgsme_kernel<<<1, 1024, 0, s>>>(Ws, nrows, sme, f, ncomp, partial); ++g_launch_count;
  const dim3 grid((nesp + kLorOmega - 1) / kLorOmega, nchunk);
  if (ncomp == 5)
    lorentz_partial_kernel<5><<<grid, kLorOmega, 0, s>>>(Ws, nrows, f, partial, e0, ef, nesp, partial + 2);
  else
    lorentz_partial_kernel<6><<<grid, kLorOmega, 0, s>>>(Ws, nrows, f, partial, e0, ef, nesp, partial + 2);
  ++g_launch_count;
  const double baux = (double)(float)ng * vc;  // real(ngrid product) * vc
  const double caux = (double)180.90f / (baux * 1.0);
  lorentz_final_kernel<<<(ncomp * nesp + 127) / 128, 128, 0, s>>>(partial + 2, nchunk, ncomp, delta_mask, caux, e0,
                                                                  ef, nesp, dielf); ++g_launch_count;
  renorm_kernel<<<ncomp, 256, 0, s>>>(Ws, nesp, renorm, spinf, dielf); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_optprops(const double* dielf, int nesp, int ncomp, double* props, cudaStream_t s) {
  optprops_kernel<<<(ncomp * nesp + 255) / 256, 256, 0, s>>>(dielf, nesp, ncomp, props); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_sp_records(const double* kpt, const int* nocp, const double* eig_win, const zd* hr, int nk, int nv,
                              int nc, const double* f, float* rec, float* key, int* rank, float* sorted,
                              cudaStream_t s) {
  const long dim = (long)nk * nc * nv;
  if (dim < 1 || dim > (1L << 30) / 15) return cudaErrorInvalidValue;
  const int n = (int)dim;
  sp_records_kernel<<<(n + 255) / 256, 256, 0, s>>>(kpt, nocp, eig_win, hr, nk, nv, nc, f, rec, key); ++g_launch_count;
  cudaError_t e = cudaMemsetAsync(rank, 0, sizeof(int) * n, s);
  if (e != cudaSuccess) return e;
  const int gx = (n + kRankThreads - 1) / kRankThreads;
  // split the compared range so that a small sort still fills the GPU (at least one key tile per split)
  const int gy = std::max(1, std::min((2 * 152 + gx - 1) / gx, (n + kRankTile - 1) / kRankTile));
  stable_rank_kernel<<<dim3(gx, gy), kRankThreads, 0, s>>>(key, n, rank); ++g_launch_count;
  e = cudaMemsetAsync(sorted, 0, sizeof(float) * 15 * n, s);
  if (e != cudaSuccess) return e;
  permute_rows_kernel<<<(unsigned)((15L * n + 255) / 256), 256, 0, s>>>(rec, rank, n, 15, sorted); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_bz_activity(const zd* hraw, const double* eig_win, const int* nocp, int nk, int nv, int nc,
                               double sme, double* act, DevStatus* st, cudaStream_t s) {
  bz_activity_kernel<<<(nk + 127) / 128, 128, 0, s>>>(hraw, eig_win, nocp, nk, nv, nc, sme, act, st); ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace wtb
