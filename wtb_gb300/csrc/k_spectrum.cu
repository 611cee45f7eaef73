// Oscillator strengths and the broadened dielectric spectrum.
//
// dielbsev / dielbsep (src/module_bse.F90:171-245): with s_a(n) = sum_j A(j,n) h_a(j) (no conjugate on
// A, as in the reference), f_aa(n) = |s_a|^2 and f_ab(n) = Re(s_a conj(s_b)).
// bsedielraw + optdiel + avgsme + imagrenorm (src/module_bse.F90:835-1036, src/module_optics.F90:171-401):
//   omega_j = E0 + (Ef - E0)(j-1)/(N-1),   gamma = CSHIFT + 10 * (sum_{i>=2} (E_i - E_{i-1})) / nrows,
//   eps2(omega) = C sum_n f_n gamma / ((omega - E_n)^2 + gamma^2),
//   eps1(omega) = delta + C sum_n f_n (E_n - omega) / ((omega - E_n)^2 + gamma^2),  C = 180.90_f32 / (Nk Vol)
// then the optional baseline renormalisation of eps2 and the spin factor.
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
  __shared__ double red[8][32][10];
  const int r0 = blockIdx.x * kOscRows;
  const int nr = min(kOscRows, dim - r0);
  for (int e = threadIdx.x; e < 5 * kOscRows; e += blockDim.x) {
    const int a = e / kOscRows, r = e % kOscRows;
    hs[a][r] = r < nr ? hr[(size_t)a * dim + r0 + r] : mk<double>(0.0, 0.0);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int n0 = 0; n0 < nev; n0 += 32) {
    const int n = n0 + lane;
    zd acc[5];
#pragma unroll
    for (int a = 0; a < 5; ++a) acc[a] = mk<double>(0.0, 0.0);
    if (n < nev)
      for (int r = warp; r < nr; r += 8) {
        const zd x = A[(size_t)(r0 + r) * lda + n];
#pragma unroll
        for (int a = 0; a < 5; ++a) cfma(acc[a], x, hs[a][r]);
      }
#pragma unroll
    for (int a = 0; a < 5; ++a) {
      red[warp][lane][2 * a] = acc[a].re;
      red[warp][lane][2 * a + 1] = acc[a].im;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * 10; e += blockDim.x) {
      const int l = e / 10, q = e % 10;
      if (n0 + l >= nev) continue;
      double t = 0.0;
      for (int w = 0; w < 8; ++w) t += red[w][l][q];
      partial[((size_t)blockIdx.x * nev + n0 + l) * 10 + q] = t;
    }
    __syncthreads();
  }
}

__global__ void osc_final_kernel(const double* __restrict__ partial, int nblk, int nev, double* __restrict__ osc) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nev) return;
  zd s[5];
  for (int a = 0; a < 5; ++a) s[a] = mk<double>(0.0, 0.0);
  for (int b = 0; b < nblk; ++b) {
    const double* p = partial + ((size_t)b * nev + n) * 10;
    for (int a = 0; a < 5; ++a) {
      s[a].re += p[2 * a];
      s[a].im += p[2 * a + 1];
    }
  }
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
                                                      const double* __restrict__ f, double* __restrict__ smef) {
  __shared__ double red[1024];
  __shared__ int s_last;
  if (threadIdx.x == 0) s_last = 0;
  double acc = 0.0;
  const int chunk = (nrows + blockDim.x - 1) / blockDim.x;
  const int i0 = threadIdx.x * chunk;
  int last = 0;
  for (int i = max(i0, 1); i < min(nrows, i0 + chunk); ++i) acc = acc + Ws[i] - Ws[i - 1];
  for (int i = i0; i < min(nrows, i0 + chunk); ++i)
    for (int c = 0; c < 6; ++c)
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

__global__ void lorentz_kernel(const double* __restrict__ Ws, int nrows, const double* __restrict__ f,
                               const double* __restrict__ smef_p, double caux, double e0, double ef, int nesp,
                               double* __restrict__ dielf) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 6 * nesp) return;
  const int comp = e / nesp, j = e % nesp;
  const double elux = e0 + ((ef - e0) * (double)j) / ((double)nesp - 1.0);
  const double smef = smef_p[0];
  const int nuse = min(nrows, (int)smef_p[1]);
  const double* fc = f + (size_t)comp * nrows;
  double rpart = 0.0, ipart = 0.0;
  for (int i = 0; i < nuse; ++i) {
    const double fi = fc[i];
    if (fi == 0.0) continue;  // zero activities add exactly zero (the denominator is >= gamma^2 > 0)
    const double ex = Ws[i];
    const double eaux = ((elux - ex) * (elux - ex)) + (smef * smef);
    rpart += fi * ((ex - elux) / eaux);
    ipart += fi * (smef / eaux);
  }
  const double delta = comp < 3 ? 1.0 : 0.0;
  // Fortran layout dielf(nesp, 3, 6): (j, c, comp) at j + nesp*(c + 3*comp)
  double* d = dielf + (size_t)comp * 3 * nesp + j;
  d[0] = elux;
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

__global__ void optprops_kernel(const double* __restrict__ dielf, int nesp, double* __restrict__ props) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;  // e = comp * nesp + j
  if (e >= 6 * nesp) return;
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
  const size_t plane = (size_t)6 * nesp;
  props[0 * plane + e] = n;
  props[1 * plane + e] = kap;
  props[2 * plane + e] = refl;
  props[3 * plane + e] = absc;
  props[4 * plane + e] = eloss;
}

}  // namespace

cudaError_t launch_oscillators(const zd* A, int lda, int nev, int dim, const zd* hr, double* osc, double* partial,
                               int npart, cudaStream_t s) {
  const int nblk = (dim + kOscRows - 1) / kOscRows;
  if (nblk > npart) return cudaErrorInvalidValue;
  osc_partial_kernel<<<nblk, 256, 0, s>>>(A, lda, nev, dim, hr, partial); ++g_launch_count;
  osc_final_kernel<<<(nev + 127) / 128, 128, 0, s>>>(partial, nblk, nev, osc); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_spectrum(const double* Ws, int nrows, const double* f, double sme, double vc, int ng, double e0,
                            double ef, int nesp, int renorm, double spinf, double* dielf, double* partial, int npart,
                            cudaStream_t s) {
  (void)npart;
  avgsme_kernel<<<1, 1024, 0, s>>>(Ws, nrows, sme, f, partial); ++g_launch_count;
  const double baux = (double)(float)ng * vc;  // real(ngrid product) * vc
  const double caux = (double)180.90f / (baux * 1.0);
  lorentz_kernel<<<(6 * nesp + 127) / 128, 128, 0, s>>>(Ws, nrows, f, partial, caux, e0, ef, nesp, dielf); ++g_launch_count;
  renorm_kernel<<<6, 256, 0, s>>>(Ws, nesp, renorm, spinf, dielf); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_optprops(const double* dielf, int nesp, double* props, cudaStream_t s) {
  optprops_kernel<<<(6 * nesp + 255) / 256, 256, 0, s>>>(dielf, nesp, props); ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace wtb
