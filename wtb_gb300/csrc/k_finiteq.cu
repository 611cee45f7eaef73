// Finite-momentum (Q != 0) BSE of bsebnds (src/module_bse.F90:1206-1566) with matrizelbsekq's elements
// (src/module_bse.F90:452-569):
//   H(i,j) = delta_ij (E_c(k_i+Q) - E_v(k_i)) + V(k_i,k_j) <c_i|c_j> <v_i|v_j>   [diagonal: + V(k_i,k_i)]
//            - V(Q, 0) <c_i|v_i> <v_j|c_j>                                         [|Q| != 0 only]
// with c states from the Q-shifted mesh and v states from the plain one.  The direct part is the Q = 0 build
// over a merged band window (valence slots from k, conduction slots from k+Q); the exchange part is the
// rank-1 term -V(Q,0) u u^H with u_i = <c_i|v_i>, added in place.
#include "wtb_internal.h"

namespace wtb {

namespace {

// eig_m / vec_m: slots 0..nv-1 from the plain window, nv..nv+nc-1 from the Q-shifted one.
__global__ void merge_windows_kernel(const double* __restrict__ eig_k, const zd* __restrict__ vec_k,
                                     const double* __restrict__ eig_q, const zd* __restrict__ vec_q, int nk, int nv,
                                     int nc, int w, double* __restrict__ eig_m, zd* __restrict__ vec_m) {
  const int nb = nv + nc;
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)nk * nb * w) return;
  const long ks = e / w;  // (k, slot)
  const int slot = (int)(ks % nb);
  const bool val = slot < nv;
  vec_m[e] = val ? vec_k[e] : vec_q[e];
  if (e % w == 0) eig_m[ks] = val ? eig_k[ks] : eig_q[ks];
}

// u_i = <c_i|v_i> = sum_o conj(c_i[o]) v_i[o] over the merged window (vcv of matrizelbsekq).
__global__ void exchange_u_kernel(const zd* __restrict__ vec_m, int nk, int nv, int nc, int w, zd* __restrict__ u) {
  const long I = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long dim = (long)nk * nc * nv;
  if (I >= dim) return;
  const int k = (int)(I / (nc * nv)), c = (int)((I / nv) % nc), v = (int)(I % nv);
  const int nb = nv + nc;
  const zd* cv = vec_m + ((size_t)k * nb + nv + c) * w;
  const zd* vv = vec_m + ((size_t)k * nb + v) * w;
  zd acc = mk<double>(0.0, 0.0);
  for (int o = 0; o < w; ++o) cfmac(acc, cv[o], vv[o]);
  u[I] = acc;
}

// H[I][J] (row-major) -= vq u_I conj(u_J)
__global__ void exchange_update_kernel(zd* __restrict__ H, long dim, const zd* __restrict__ u,
                                       const double* __restrict__ vq_p) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= dim * dim) return;
  const long I = e / dim, J = e % dim;
  const double vq = vq_p[0];
  const zd a = u[I], b = u[J];
  // a conj(b)
  const zd t = mk<double>(a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im);
  H[e].re -= vq * t.re;
  H[e].im -= vq * t.im;
}

}  // namespace

cudaError_t launch_merge_windows(const double* eig_k, const zd* vec_k, const double* eig_q, const zd* vec_q, int nk,
                                 int nv, int nc, int w, double* eig_m, zd* vec_m, cudaStream_t s) {
  const long n = (long)nk * (nv + nc) * w;
  merge_windows_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(eig_k, vec_k, eig_q, vec_q, nk, nv, nc, w, eig_m,
                                                                  vec_m); ++g_launch_count;
  return cudaGetLastError();
}

cudaError_t launch_exchange(const zd* vec_m, int nk, int nv, int nc, int w, const double* vq, zd* u, zd* H,
                            cudaStream_t s) {
  const long dim = (long)nk * nc * nv;
  exchange_u_kernel<<<(unsigned)((dim + 255) / 256), 256, 0, s>>>(vec_m, nk, nv, nc, w, u); ++g_launch_count;
  exchange_update_kernel<<<(unsigned)((dim * dim + 255) / 256), 256, 0, s>>>(H, dim, u, vq); ++g_launch_count;
  return cudaGetLastError();
}

}  // namespace wtb
