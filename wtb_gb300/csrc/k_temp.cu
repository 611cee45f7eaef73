// Temperature BSE of bsesolvertemp and bsebndstemp (src/module_bse.F90:2649-3263, :1572-1990): the couplings
// weighted by the occupation difference f_v - f_c of the row's transition (fermidisteh, src/module_math.F90:407-421).
// matrizelbsetemp / matrizelbsekqtemp (src/module_bse.F90:575-660, :664-780) give
//   H(i,j) = C(i,j) f_i  (i != j),   H(i,i) = (E_c - E_v) + C(i,i) f_i
// with C the Coulomb part (direct, and at finite Q the exchange); the reference fills the upper triangle and
// ZHEEV 'U' reads its Hermitian completion, E(i,j) = D(i,j) f_min(i,j) with D the unweighted matrix.  Then the
// activities of dielbseptemp (src/module_bse.F90:784-810) for every exciton:
// Re[(sum_j A(j,n) h1(j)) conj(sum_j A(j,n) h2(j) f_j)].
#include "wtb_internal.h"

namespace wtb {

namespace {

// f_v - f_c at temperature temp (K), Fermi level 0; kb is the single-precision literal 8.617330350E-5 and a zero
// temperature is read as 1E-8 (single precision), as fermidisteh does.
__global__ void fermi_weight_kernel(const double* __restrict__ eig_win, int nk, int nv, int nc, double temp,
                                    double* __restrict__ f) {
  const long I = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long dim = (long)nk * nc * nv;
  if (I >= dim) return;
  const int k = (int)(I / (nc * nv)), c = (int)((I / nv) % nc), v = (int)(I % nv);
  const int nb = nv + nc;
  const double ec = eig_win[(size_t)k * nb + nv + c], ev = eig_win[(size_t)k * nb + v];
  const double t = temp == 0.0 ? (double)1e-8f : temp;
  const double kb = (double)8.617330350E-5f;
  const double beta = 1.0 / (kb * t);
  const double fv = 1.0 / (exp(ev * beta) + 1.0);
  const double fc = 1.0 / (exp(ec * beta) + 1.0);
  f[I] = fv - fc;
}

// E = D f_min(i,j) off the diagonal, E(i,i) = dE_i + (D(i,i) - dE_i) f_i (the coupling part of the diagonal
// weighted: V(k_i,k_i) at Q = 0, V(k_i,k_i) - V(Q,0)|<c_i|v_i>|^2 for the finite-Q matrix of matrizelbsekqtemp),
// on the row-major dim x dim D in place.
__global__ void temp_weight_kernel(zd* __restrict__ H, long dim, const double* __restrict__ f,
                                   const double* __restrict__ dE) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= dim * dim) return;
  const long I = e / dim, J = e % dim;
  if (I == J) {
    H[e] = mk<double>(dE[I] + (H[e].re - dE[I]) * f[I], 0.0);
  } else {
    const double w = f[I < J ? I : J];
    H[e].re *= w;
    H[e].im *= w;
  }
}

// Per exciton n (column n of the row-major eigenvector matrix Z): s_a = sum_i Z(i,n) h_a(i) and
// t_a = sum_i Z(i,n) h_a(i) f_i for a = x y z sp sm, then the eight activities
// xx yy zz (s_a, t_a), xy (s_x, t_y), xz (s_x, t_z), yz (s_y, t_z), sp, sm; xy xz yz zero unless dtfull, sp sm
// zero unless cpol (the reference writes zeros then).
__global__ void __launch_bounds__(128) temp_acts_kernel(const zd* __restrict__ Z, int dim, const zd* __restrict__ hr,
                                                        const double* __restrict__ f, int dtfull, int cpol,
                                                        double* __restrict__ acts) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= dim) return;
  zd s[5], t[5];
#pragma unroll
  for (int a = 0; a < 5; ++a) s[a] = t[a] = mk<double>(0.0, 0.0);
  for (int i = 0; i < dim; ++i) {
    const zd z = Z[(size_t)i * dim + n];
    const double fi = f[i];
#pragma unroll
    for (int a = 0; a < 5; ++a) {
      const zd zh = cmul(z, hr[(size_t)a * dim + i]);
      s[a] = cadd(s[a], zh);
      t[a] = cadd(t[a], cscale(zh, fi));
    }
  }
  auto re_prod = [](zd a, zd b) { return a.re * b.re + a.im * b.im; };  // Re(a conj(b))
  acts[0 * (size_t)dim + n] = re_prod(s[0], t[0]);
  acts[1 * (size_t)dim + n] = re_prod(s[1], t[1]);
  acts[2 * (size_t)dim + n] = re_prod(s[2], t[2]);
  acts[3 * (size_t)dim + n] = dtfull ? re_prod(s[0], t[1]) : 0.0;
  acts[4 * (size_t)dim + n] = dtfull ? re_prod(s[0], t[2]) : 0.0;
  acts[5 * (size_t)dim + n] = dtfull ? re_prod(s[1], t[2]) : 0.0;
  acts[6 * (size_t)dim + n] = cpol ? re_prod(s[3], t[3]) : 0.0;
  acts[7 * (size_t)dim + n] = cpol ? re_prod(s[4], t[4]) : 0.0;
}

}  // namespace

cudaError_t launch_fermi_weights(const double* eig_win, int nk, int nv, int nc, double temp, double* f,
                                 cudaStream_t s) {
  const long dim = (long)nk * nc * nv;
  fermi_weight_kernel<<<(unsigned)((dim + 255) / 256), 256, 0, s>>>(eig_win, nk, nv, nc, temp, f); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_temp_weight(zd* H, long dim, const double* f, const double* dE, cudaStream_t s) {
  temp_weight_kernel<<<(unsigned)((dim * dim + 255) / 256), 256, 0, s>>>(H, dim, f, dE); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_temp_acts(const zd* Z, int dim, const zd* hr, const double* f, int dtfull, int cpol, double* acts,
                             cudaStream_t s) {
  temp_acts_kernel<<<(dim + 127) / 128, 128, 0, s>>>(Z, dim, hr, f, dtfull, cpol, acts); ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace wtb
