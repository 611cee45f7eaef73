// C ABI of libwtb_gb300 (declared in include/wtb_gpu.h): the context, the state the Fortran modules
// kept in globals, and the entry points that stand in for eigsys, monhkhorst_pack, the module_coulomb
// potentials, matrizelbse's build loop, slepc_solver, dielbsev/dielbsep, bsesolver, bsedielraw(pol),
// spoptics, spdielraw(pol) and bseoptprop(pol).  Everything numeric runs in the CUDA kernels of this library; host code only moves
// arguments, checks them, and orchestrates launches on the context's stream.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

#include "ctx.h"

namespace wtb {
std::atomic<long long> g_launch_count{0};

cudaError_t raise_smem_limit(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> limit;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  size_t& cur = limit[{func, dev}];
  if (bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}
}

using namespace wtb;


namespace {

int set_err(wtb_ctx* c, int code, const std::string& m) {
  if (c) c->msg = m;
  return code;
}

#define CKC(x)                                                                   \
  do {                                                                           \
    cudaError_t e__ = (x);                                                       \
    if (e__ != cudaSuccess) {                                                    \
      if (e__ == cudaErrorMemoryAllocation)                                      \
        return set_err(c, WTB_ENOMEM, std::string(#x) + ": " + cudaGetErrorString(e__)); \
      return set_err(c, WTB_ECUDA, std::string(#x) + ": " + cudaGetErrorString(e__));    \
    }                                                                            \
  } while (0)

#define CKR(x)             \
  do {                     \
    int r__ = (x);         \
    if (r__) return r__;   \
  } while (0)

// Reads and clears the device status word; maps kernel-side failures to the reference's STOP texts.
int check_status(wtb_ctx* c) {
  DevStatus h;
  CKC(cudaMemcpyAsync(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost, c->s));
  CKC(cudaStreamSynchronize(c->s));
  if (!h.code) return WTB_OK;
  CKC(cudaMemsetAsync(c->st, 0, sizeof(DevStatus), c->s));
  CKC(cudaStreamSynchronize(c->s));
  switch (h.code) {
    case 101:
      return set_err(c, WTB_EBADARG, "Number of valence states higher then ocuppied states (k-point " +
                                         std::to_string(h.info + 1) + ")");
    case 102:
      return set_err(c, WTB_EBADARG, "Number of conduction states higher then unocuppied states (k-point " +
                                         std::to_string(h.info + 1) + ")");
    case 103:
      return set_err(c, WTB_EBADARG, "spoptpolbz: the number of occupied states differs between k-points (k-point " +
                                         std::to_string(h.info + 1) + "); the BZ-resolved activity needs an insulator");
    case 201:
      return set_err(c, WTB_ENOCONV, "The algorithm failed to compute eigenvalues.");
    default:
      if (h.code >= 400 && h.code < 500)
        return set_err(c, WTB_ETIMEOUT, "a bounded device wait timed out (code " + std::to_string(h.code) + ")");
      return set_err(c, WTB_ECUDA, "device status " + std::to_string(h.code));
  }
}

int prep_device(wtb_ctx* c) {
  CKC(cudaSetDevice(c->device));
  return WTB_OK;
}

double vcell3D(const double* r) {
  const double vx0 = r[1] * r[5] - r[2] * r[4], vx1 = r[2] * r[3] - r[0] * r[5], vx2 = r[0] * r[4] - r[1] * r[3];
  return std::fabs(vx0 * r[6] + vx1 * r[7] + vx2 * r[8]);
}

// Reciprocal vectors with single-precision pi (recvec, src/module_kmesh.F90:391-407).
void recvec(const double* a1, const double* a2, const double* a3, double* b1, double* b2, double* b3) {
  auto cross = [](const double* u, const double* v, double* o) {
    o[0] = u[1] * v[2] - u[2] * v[1];
    o[1] = u[2] * v[0] - u[0] * v[2];
    o[2] = u[0] * v[1] - u[1] * v[0];
  };
  double v23[3], v31[3], v12[3];
  cross(a2, a3, v23);
  cross(a3, a1, v31);
  cross(a1, a2, v12);
  const double vol = std::fabs(a1[0] * v23[0] + a1[1] * v23[1] + a1[2] * v23[2]);
  const double pi32 = (double)3.14159274101257324f;
  const double f = (2.0 * pi32) / vol;
  for (int d = 0; d < 3; ++d) {
    b1[d] = f * v23[d];
    b2[d] = f * v31[d];
    b3[d] = f * v12[d];
  }
}

// Gamma-anchored mesh, i outer, j, l inner (monhkhorst_pack, src/module_kmesh.F90:338-386); with q, the mesh
// shifted by Q = q(2:4) of a Q-path row, summed in monhkhorst_packq's order (src/module_kmesh.F90:281-334).
// kpt row-major nk x 3.
void mp_mesh(int n1, int n2, int n3, const double* shift, const double* a1, const double* a2, const double* a3,
             double* kpt, const double* q = nullptr) {
  double b1[3], b2[3], b3[3], ks[3];
  recvec(a1, a2, a3, b1, b2, b3);
  for (int d = 0; d < 3; ++d) ks[d] = b1[d] * shift[0] + b2[d] * shift[1] + b3[d] * shift[2];
  long cnt = 0;
  for (int i = 0; i < n1; ++i)
    for (int j = 0; j < n2; ++j)
      for (int l = 0; l < n3; ++l) {
        for (int d = 0; d < 3; ++d) {
          if (q)
            kpt[3 * cnt + d] = q[1 + d] + (b1[d] / (double)n1) * (double)i + (b2[d] / (double)n2) * (double)j +
                               (b3[d] / (double)n3) * (double)l + ks[d];
          else
            kpt[3 * cnt + d] = (b1[d] / (double)n1) * (double)i + (b2[d] / (double)n2) * (double)j +
                               (b3[d] / (double)n3) * (double)l + ks[d];
        }
        ++cnt;
      }
}

__global__ void transpose_z_kernel(const zd* __restrict__ A, int rows, int cols, int lda, zd* __restrict__ B,
                                   int conj) {
  // B (column-major rows x cols) = A (row-major rows x cols, ld lda)
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)rows * cols) return;
  const long r = e % rows, cc = e / rows;
  zd v = A[r * lda + cc];
  if (conj) v.im = -v.im;
  B[cc * rows + r] = v;
}

template <class S>
__global__ void conj_convert_kernel(const cplx<S>* __restrict__ A, long n, zd* __restrict__ B) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  B[e] = mk<double>((double)A[e].re, -(double)A[e].im);
}

__global__ void conj_inplace_kernel(zd* A, long n) {
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) A[e].im = -A[e].im;
}

__global__ void diag_real_kernel(const zd* __restrict__ H, int n, double* __restrict__ d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = H[(size_t)i * n + i].re;
}

__global__ void __launch_bounds__(256) dielbse_kernel(const zd* __restrict__ A, int dimse, const zd* __restrict__ h1,
                                                      const zd* __restrict__ h2, int pair, double* __restrict__ act) {
  // one CTA per exciton n; A column-major (column n contiguous)
  __shared__ double red[4][256];
  const int n = blockIdx.x;
  zd s1 = mk<double>(0, 0), s2 = mk<double>(0, 0);
  for (int j = threadIdx.x; j < dimse; j += blockDim.x) {
    const zd a = A[(size_t)n * dimse + j];
    cfma(s1, a, h1[j]);
    if (pair) cfma(s2, a, h2[j]);
  }
  red[0][threadIdx.x] = s1.re;
  red[1][threadIdx.x] = s1.im;
  red[2][threadIdx.x] = s2.re;
  red[3][threadIdx.x] = s2.im;
  __syncthreads();
  for (int off = 128; off > 0; off >>= 1) {
    if (threadIdx.x < off)
      for (int q = 0; q < 4; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double ar = red[0][0], ai = red[1][0];
    if (pair)
      act[n] = ar * red[2][0] + ai * red[3][0];
    else
      act[n] = ar * ar + ai * ai;
  }
}

__global__ void expand_acts_kernel(const double* __restrict__ osc, int nev, int dim, double* __restrict__ acts) {
  // acts(dim, 8) column-major; rows past nev are zero
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)dim * 8) return;
  const int a = (int)(e / dim);
  const long i = e % dim;
  acts[e] = i < nev ? osc[(size_t)a * nev + i] : 0.0;
}

// Host part of a band computation: the k-points go to the device (stream-ordered), the band buffers are
// sized and the context records the mesh.  enqueue_bands then only launches kernels (a graph can hold it).
int stage_bands(wtb_ctx* c, int nk, const double* kpt_rm, int nv, int nc) {
  cudaError_t err = cudaSuccess;
  double* dk = c->ws.get<double>("kpt", (size_t)nk * 3, &err);
  CKC(err);
  c->kpt.assign(kpt_rm, kpt_rm + (size_t)nk * 3);
  CKC(cudaMemcpyAsync(dk, c->kpt.data(), sizeof(double) * nk * 3, cudaMemcpyHostToDevice, c->s));
  const int w = c->w, nb = nv + nc;
  c->ws.get<double>("eig_all", (size_t)nk * w, &err);
  c->ws.get<zd>("vec_all", (size_t)nk * w * w, &err);
  c->ws.get<double>("eig_win", (size_t)nk * (nb > 0 ? nb : 1), &err);
  c->ws.get<zd>("vec_win", (size_t)nk * (nb > 0 ? nb : 1) * w, &err);
  c->ws.get<int>("nocp", nk, &err);
  CKC(err);
  c->nk = nk;
  c->nv = nv;
  c->nc = nc;
  c->have_bands = nb > 0;
  c->have_solve = false;  // the stored excitons belong to the previous bands
  return WTB_OK;
}

// The reduced-precision matrix-free forms (FP32 and split-BF16) take their bands from the mixed band solver
// (FP32 eigensolve, FP64 Rayleigh quotients) and their velocity matrix elements from FP32 Fourier sums: their
// operator carries about 1e-7 relative error already, and on this GPU those set-up kernels are bound by the
// FP64 pipe (57,600 workload: 1.9 ms for the FP64 bands against 0.7 ms mixed).
bool reduced_form(const wtb_bse_params* p) { return p && p->op == WTB_OP_MATFREE && p->precision != WTB_PREC_FP64; }

int enqueue_bands(wtb_ctx* c, bool mixed = false) {
  cudaError_t err = cudaSuccess;
  const int nk = c->nk, nv = c->nv, nc = c->nc, w = c->w, nb = nv + nc;
  CKC(launch_hk_eig(c->ws.get<zd>("hr", 0, &err), c->ws.get<int>("rvec", 0, &err), c->ws.get<int>("ndegen", 0, &err),
                    c->nR, w, c->ws.get<double>("rlat", 0, &err), c->efermi, c->scs, c->ws.get<double>("kpt", 0, &err),
                    nk, nv, nc, c->ws.get<double>("eig_all", 0, &err), c->ws.get<zd>("vec_all", 0, &err),
                    nb > 0 ? c->ws.get<double>("eig_win", 0, &err) : nullptr,
                    nb > 0 ? c->ws.get<zd>("vec_win", 0, &err) : nullptr, c->ws.get<int>("nocp", 0, &err), c->st, c->s,
                    mixed, mixed ? c->ws.get<float4>("hr_df", (size_t)c->nR * (w * w + 2), &err) : nullptr));
  CKC(err);
  return WTB_OK;
}

int upload_bands(wtb_ctx* c, int nk, const double* kpt_rm, int nv, int nc) {
  CKR(stage_bands(c, nk, kpt_rm, nv, nc));
  CKR(enqueue_bands(c));
  return check_status(c);
}

int validate_params(wtb_ctx* c, const wtb_bse_params* p) {
  if (!p) return set_err(c, WTB_EBADARG, "params is NULL");
  if (p->ngrid[0] < 1 || p->ngrid[1] < 1 || p->ngrid[2] < 1) return set_err(c, WTB_EBADARG, "ngrid must be >= 1");
  if (p->nc < 1 || p->nv < 1) return set_err(c, WTB_EBADARG, "nc and nv must be >= 1");
  if (p->coultype < 0 || p->coultype > 8)
    return set_err(c, WTB_EBADARG, "Wrong Coulomb Potential");
  if (!(p->ktol > 0.0)) return set_err(c, WTB_EBADARG, "KTOL must be > 0 (V(k,k) is singular otherwise)");
  if (p->precision < 0 || p->precision > 3 || p->op < 0 || p->op > 1)
    return set_err(c, WTB_EBADARG, "unknown precision or operator mode");
  if (p->op == WTB_OP_DENSE && p->precision >= WTB_PREC_BF16X3)
    return set_err(c, WTB_EBADARG, "split-BF16 precision is available for the matrix-free operator only");
  return WTB_OK;
}

CoulParams coul_of(wtb_ctx* c, const wtb_bse_params* p) {
  CoulParams cp{};
  cp.type = p->coultype;
  for (int d = 0; d < 3; ++d) {
    cp.ngrid[d] = p->ngrid[d];
    cp.ediel[d] = p->ediel[d];
  }
  cp.ktol = p->ktol;
  cp.ez = p->ez;
  cp.w = p->w_coul;
  cp.r0 = p->r0;
  cp.lc = p->lc;
  std::memcpy(cp.rlat, c->rlat_rm, sizeof(cp.rlat));
  return cp;
}

// V(k,k') (or dV/dr0) for the bands of the context into V (leading dimension ldv)
int coulomb_table_into(wtb_ctx* c, const wtb_bse_params* p, double* V, int ldv, bool deriv_r0 = false) {
  cudaError_t err = cudaSuccess;
  CoulParams cpar = coul_of(c, p);
  cpar.deriv_r0 = deriv_r0 ? 1 : 0;
  const int nk = c->nk;
  const bool mp = c->mesh_mp && p->ngrid[0] == c->ngrid[0] && p->ngrid[1] == c->ngrid[1] &&
                  p->ngrid[2] == c->ngrid[2] && (long)p->ngrid[0] * p->ngrid[1] * p->ngrid[2] == nk;
  if (mp) {
    // reciprocal vectors of the mesh, on the device since wtb_set_hr
    const double* dbl = c->ws.find<double>("recip", 9);
    if (!dbl) return set_err(c, WTB_ESTATE, "reciprocal vectors not staged");
    const long ns = (2L * p->ngrid[0] - 1) * (2L * p->ngrid[1] - 1) * (2L * p->ngrid[2] - 1);
    double* stn = c->ws.get<double>("vstencil", ns, &err);
    CKC(err);
    CKC(launch_coulomb_mesh(cpar, dbl, stn, V, ldv, c->s));
  } else {
    const double* kd = c->ws.get<double>("kpt", 0, &err);
    CKC(launch_coulomb(cpar, kd, nk, kd, nk, V, ldv, c->s));
  }
  return WTB_OK;
}

// the largest block the block eigensolver takes (3 m columns in its projected problems)
int block_cap(bool fp64) { return fp64 ? 26 : 32; }

// shift of the deflated solves: the spread of the diagonal plus 2 eV moves a found eigenpair above every
// eigenvalue still sought (the lowest excitons lie below the largest transition energy)
int deflation_shift(wtb_ctx* c, const double* d_diag, int dim, double* sigma) {
  std::vector<double> h(dim);
  CKC(cudaMemcpyAsync(h.data(), d_diag, sizeof(double) * dim, cudaMemcpyDeviceToHost, c->s));
  CKC(cudaStreamSynchronize(c->s));
  const auto mm = std::minmax_element(h.begin(), h.end());
  *sigma = (*mm.second - *mm.first) + 2.0;
  return WTB_OK;
}

int auto_block(const wtb_bse_params* p, int dim, bool fp64) {
  // automatic: nev + 4 rounded up to a multiple of 8, at least 16 (measured on the 57,600 workload with nev = 10:
  // blocks 12 / 14 / 16 / 24 took 13.6 (not converged) / 15.0 / 13.5 / 22.4 ms; on the 36,864 one with nev = 20:
  // blocks 20 / 24 / 32 took 20.8 / 20.0 / 23.4 ms)
  int m = p->block > 0 ? p->block : std::max(16, (p->nev + 4 + 7) / 8 * 8);
  const int cap = block_cap(fp64);
  if (m > cap) m = cap;
  if (m < p->nev) m = p->nev;
  if (m > dim) m = dim;
  return m;
}

// tag: suffix of the buffers holding the V table and its forms (a second operator, e.g. the dV/dr0 one,
// must not overwrite the first); deriv_r0: build the operator of dV/dr0 with no diagonal term.
// tune: choose the contraction's column tile by timing (not for the operators a batch contracts jointly)
int make_operator(wtb_ctx* c, const wtb_bse_params* p, int nbmax, OpBundle* ob, const std::string& tag = "",
                  bool deriv_r0 = false, bool tune = true) {
  const int nk = c->nk, nv = c->nv, nc = c->nc, w = c->w;
  const int dim = nk * nc * nv;
  cudaError_t err = cudaSuccess;
  const zd* vec_win = c->ws.get<zd>("vec_win", 0, &err);
  double* dE = c->ws.get<double>(deriv_r0 ? "dE0" : "dE", dim, &err, deriv_r0);
  CKC(err);
  if (!deriv_r0) CKC(launch_transition_energies(c->ws.get<double>("eig_win", 0, &err), nk, nv, nc, dE, c->s));
  const int Kpad = (nk + 63) / 64 * 64, Mpad = (nk + 127) / 128 * 128;
  // the FP32 forms' gather and scatter read the band vectors and transition energies rounded to FP32 once here
  // (the values their tiles would otherwise convert from FP64 in every CTA)
  auto f32_inputs = [&](MatFreeOperator<float>* op) -> int {
    const int nvals = (nv + nc) * w;
    zf* vf = c->ws.get<zf>("vec_win_f32", (size_t)nk * nvals, &err);
    float* ef = c->ws.get<float>(deriv_r0 ? "dE0_f32" : "dE_f32", dim, &err);
    CKC(err);
    CKC(launch_round_f32(reinterpret_cast<const double*>(vec_win), 2 * nvals, nk, 2 * nvals,
                         reinterpret_cast<float*>(vf), 2 * nvals, c->s));
    CKC(launch_round_f32(dE, dim, 1, dim, ef, dim, c->s));
    op->vec_s = vf;
    op->dE_s = ef;
    return WTB_OK;
  };
  // FP32 matrix-free operator on a two-dimensional Monkhorst-Pack mesh: the contraction as FFT convolutions with
  // the Coulomb stencil (no nk x nk table).  WTB_FFT=0 selects the CUDA-core product instead.
  const bool mesh2d = c->mesh_mp && p->ngrid[0] == c->ngrid[0] && p->ngrid[1] == c->ngrid[1] &&
                      p->ngrid[2] == c->ngrid[2] && p->ngrid[2] == 1 && (long)p->ngrid[0] * p->ngrid[1] == nk;
  const char* fft_env = std::getenv("WTB_FFT");
  const int fftP = (p->op == WTB_OP_MATFREE && p->precision == WTB_PREC_FP32 && mesh2d &&
                    !(fft_env && std::strcmp(fft_env, "0") == 0))
                       ? fft_conv_size(p->ngrid[0], p->ngrid[1])
                       : 0;
  if (fftP) {
    const double* dbl = c->ws.find<double>("recip", 9);
    if (!dbl) return set_err(c, WTB_ESTATE, "reciprocal vectors not staged");
    CoulParams cpar = coul_of(c, p);
    cpar.deriv_r0 = deriv_r0 ? 1 : 0;
    const int n1 = p->ngrid[0], n2 = p->ngrid[1];
    double* stn = c->ws.get<double>("vstencil" + tag, (size_t)(2 * n1 - 1) * (2 * n2 - 1), &err);
    zd* work = c->ws.get<zd>("fft_work", (size_t)(2 * n1 - 1) * fftP, &err);
    float2* spec = c->ws.get<float2>("fft_spec" + tag, fft_spec_size(fftP), &err);
    float2* tw = c->ws.get<float2>("fft_tw", 128, &err);
    CKC(err);
    CKC(launch_coulomb_stencil(cpar, dbl, stn, c->s));
    CKC(launch_fft_spectrum(stn, n1, n2, fftP, work, spec, tw, c->s));
    const int N = 2 * w * w * nbmax;
    const int Npad = (N + 255) / 256 * 256;
    auto op = new MatFreeOperator<float>();
    ob->o32.reset(op);
    ob->dE = dE;
    ob->dim = dim;
    op->kind = GEMM_FFT_F32;
    op->nk = nk; op->nv = nv; op->nc = nc; op->w = w; op->nbmax = nbmax;
    op->vec_win = vec_win; op->dE = dE; op->st = c->st; op->msg = &ob->msg; op->prof = &c->prof;
    CKR(f32_inputs(op));
    op->Kpad = Kpad; op->Mpad = Mpad; op->Npad = Npad;
    op->mesh1 = n1; op->mesh2 = n2; op->fft_p = fftP;
    op->fft_spec = spec; op->fft_tw = tw;
    op->Zr = c->ws.get<float>("Zr32", (size_t)Npad * Kpad, &err, true);
    op->Tm = c->ws.get<float>("T32", (size_t)Mpad * Npad, &err);
    CKC(err);
    c->last_form = WTB_FORM_FFT_F32;
    if (tune) {
      zf* tx = c->ws.get<zf>("tune_X", (size_t)dim * nbmax, &err, true);
      zf* ty = c->ws.get<zf>("tune_Y", (size_t)dim * nbmax, &err);
      CKC(err);
      CKC(op->autotune(c->s, tx, ty));
    }
    return WTB_OK;
  }
  c->last_form = WTB_FORM_NONE;
  double* V = c->ws.get<double>("V" + tag, (size_t)Mpad * Kpad, &err, true);
  CKC(err);
  CKR(coulomb_table_into(c, p, V, Kpad, deriv_r0));
  ob->dE = dE;
  ob->dim = dim;
  const bool fp64 = p->precision == WTB_PREC_FP64;
  if (p->op == WTB_OP_DENSE) {
    if (fp64) {
      zd* H = c->ws.get<zd>("H64", (size_t)dim * dim, &err);
      CKC(err);
      CKC(launch_bse_build<double>(vec_win, dE, V, Kpad, nk, nv, nc, w, H, c->s));
      auto op = new DenseOperator<double>();
      op->H = H;
      op->dim = dim;
      ob->o64.reset(op);
    } else {
      zf* H = c->ws.get<zf>("H32", (size_t)dim * dim, &err);
      CKC(err);
      CKC(launch_bse_build<float>(vec_win, dE, V, Kpad, nk, nv, nc, w, H, c->s));
      auto op = new DenseOperator<float>();
      op->H = H;
      op->dim = dim;
      ob->o32.reset(op);
    }
    return WTB_OK;
  }
  const int N = 2 * w * w * nbmax;
  const int Npad = (N + 255) / 256 * 256;
  if (fp64) {
    auto op = new MatFreeOperator<double>();
    ob->o64.reset(op);
    op->kind = GEMM_SIMT_F64;
    op->nk = nk; op->nv = nv; op->nc = nc; op->w = w; op->nbmax = nbmax;
    op->vec_win = vec_win; op->dE = dE; op->st = c->st; op->msg = &ob->msg; op->prof = &c->prof;
    op->vec_s = vec_win;
    op->dE_s = dE;
    op->Kpad = Kpad; op->Mpad = Mpad; op->Npad = Npad;
    op->Vr = V;
    op->Zr = c->ws.get<double>("Zr64", (size_t)Npad * Kpad, &err, true);
    op->Tm = c->ws.get<double>("T64", (size_t)Mpad * Npad, &err);
    CKC(err);
    c->last_form = WTB_FORM_SIMT_F64;
    return WTB_OK;
  }
  auto op = new MatFreeOperator<float>();
  ob->o32.reset(op);
  op->nk = nk; op->nv = nv; op->nc = nc; op->w = w; op->nbmax = nbmax;
  op->vec_win = vec_win; op->dE = dE; op->st = c->st; op->msg = &ob->msg; op->prof = &c->prof;
  CKR(f32_inputs(op));
  op->Kpad = Kpad; op->Mpad = Mpad; op->Npad = Npad;
  if (p->precision == WTB_PREC_FP32) {
    op->kind = GEMM_SIMT_F32;
    float* Vf = c->ws.get<float>("V32" + tag, (size_t)Mpad * Kpad, &err, true);
    CKC(err);
    CKC(launch_round_f32(V, Kpad, nk, nk, Vf, Kpad, c->s));
    op->Vr = Vf;
    op->Zr = c->ws.get<float>("Zr32", (size_t)Npad * Kpad, &err, true);
    op->Tm = c->ws.get<float>("T32", (size_t)Mpad * Npad, &err);
    CKC(err);
    c->last_form = WTB_FORM_SIMT_F32;
    return WTB_OK;
  }
  if (!tc_gemm_available()) return set_err(c, WTB_ENODEV, "the split-BF16 tensor-core path needs an sm_103 device");
  op->kind = GEMM_TC_BF16;
  const bool x6 = p->precision == WTB_PREC_BF16X6;
  // three slices in both modes: bf16x3 iterates with the 3 leading slice products and applies all 6
  // for the final refinement
  op->nslices = 3;
  op->npairs = x6 ? 6 : 3;
  op->npairs0 = op->npairs;
  op->npairs_refine = 6;
  const int pa6[6] = {0, 0, 1, 0, 1, 2}, pb6[6] = {0, 1, 0, 2, 1, 0};
  for (int i = 0; i < 6; ++i) {
    op->pa[i] = pa6[i];
    op->pb[i] = pb6[i];
  }
  uint16_t* Vs = c->ws.get<uint16_t>("Vbf" + tag, (size_t)op->nslices * Mpad * Kpad, &err, true);
  CKC(err);
  CKC(launch_split_bf16(V, Kpad, nk, nk, Vs, Kpad, (long)Mpad * Kpad, op->nslices, c->s));
  op->Vs = Vs;
  op->Zs = c->ws.get<uint16_t>("Zbf", (size_t)op->nslices * Npad * Kpad, &err, true);
  op->Tm = c->ws.get<float>("Tbf", (size_t)Mpad * Npad, &err);
  CKC(err);
  if (const char* kc = std::getenv("WTB_FINAL_KCHUNK")) op->kchunk_final = std::atoi(kc);
  // launch shapes of the application: measured once per shape and device (skipped while a graph is being
  // captured), on two zeroed scratch blocks
  c->last_form = WTB_FORM_TC_BF16;
  if (tune) {
    zf* tx = c->ws.get<zf>("tune_X", (size_t)dim * nbmax, &err, true);
    zf* ty = c->ws.get<zf>("tune_Y", (size_t)dim * nbmax, &err);
    CKC(err);
    CKC(op->autotune(c->s, tx, ty));
  }
  return WTB_OK;
}

// Solve with the operator selected by p; leaves E and the FP64 eigenvectors (dim x nev row-major, "Xout").
int run_solve(wtb_ctx* c, const wtb_bse_params* p, std::vector<double>* E, wtb_timings* t, SolveStats* stats) {
  const int dim = c->nk * c->nc * c->nv;
  cudaError_t err = cudaSuccess;
  cudaEvent_t ev[3];
  for (auto& e : ev) CKC(cudaEventCreate(&e));
  CKC(cudaEventRecord(ev[0], c->s));
  const bool fp64 = p->precision == WTB_PREC_FP64;
  const int m = auto_block(p, dim, fp64);
  // residual targets: SLEPc's 1e-8 in FP64; kReducedTol (1e-5, at the FP32 rounding floor) otherwise.
  // The reduced-precision forms run in two phases: to 1e-4, then -- from the best block, with a freshly applied
  // operator and the search directions dropped -- to the target (bf16x3 switches to its 6-product operator
  // there).  The restart removes the drift of the FP32 iteration's running H X, which otherwise stalls the
  // residual between 1e-5 and 1e-4 on the 57,600 workload.
  const bool two_phase = !fp64;
  const double tol_final = p->tol > 0 ? p->tol : (fp64 ? 1e-8 : kReducedTol);
  const double tol = two_phase ? std::max(tol_final, 1e-4) : tol_final;
  const double tol_refine = two_phase && tol_final < tol ? tol_final : 0.0;
  const int maxit = p->maxit > 0 ? p->maxit : 200;
  zd* Xout = c->ws.get<zd>("Xout", (size_t)dim * p->nev, &err);
  CKC(err);
  OpBundle ob;
  CKR(make_operator(c, p, std::min(m, 16), &ob));
  CKC(cudaEventRecord(ev[1], c->s));
  int rc;
  std::string msg;
  if (p->nev > block_cap(fp64)) {
    // more excitons than one block holds (the reference asks 100): chunks of 16 with deflation
    double sigma = 0.0;
    CKR(deflation_shift(c, ob.dE, dim, &sigma));
    if (ob.o64)
      rc = lobpcg_solve_deflated<double>(*ob.o64, ob.dE, dim, p->nev, 16, 24, tol, maxit, sigma, c->ws, c->st, c->s, E,
                                         Xout, stats, &msg);
    else
      rc = lobpcg_solve_deflated<float>(*ob.o32, ob.dE, dim, p->nev, 16, 24, tol, maxit, sigma, c->ws, c->st, c->s, E,
                                        Xout, stats, &msg, tol_refine);
  } else if (ob.o64) {
    rc = lobpcg_solve<double>(*ob.o64, ob.dE, dim, p->nev, m, tol, maxit, c->ws, c->st, c->s, E, Xout, stats, &msg);
  } else {
    rc = lobpcg_solve<float>(*ob.o32, ob.dE, dim, p->nev, m, tol, maxit, c->ws, c->st, c->s, E, Xout, stats, &msg,
                             tol_refine);
  }
  if (!ob.msg.empty()) msg += " (" + ob.msg + ")";
  CKC(cudaEventRecord(ev[2], c->s));
  CKC(cudaEventSynchronize(ev[2]));
  // the eigensolve is one graph launch: the live profile of the contraction is taken after it, on the same
  // operator data (three launches of the iteration-phase contraction, CUDA events on the context's stream)
  if (rc == WTB_OK && c->prof.on && p->op == WTB_OP_MATFREE) {
    if (ob.o64) {
      if (auto* mf = dynamic_cast<MatFreeOperator<double>*>(ob.o64.get())) CKC(mf->time_contraction(3, m, c->s));
    } else if (auto* mf = dynamic_cast<MatFreeOperator<float>*>(ob.o32.get())) {
      CKC(mf->time_contraction(3, m, c->s));
    }
  }
  float t01 = 0, t12 = 0;
  cudaEventElapsedTime(&t01, ev[0], ev[1]);
  cudaEventElapsedTime(&t12, ev[1], ev[2]);
  for (auto& e : ev) cudaEventDestroy(e);
  if (t) {
    t->t_build_ms = t01;
    t->t_solve_ms = t12;
  }
  if (rc != WTB_OK) {
    int sc = check_status(c);
    if (sc != WTB_OK && rc == WTB_ECUDA) return sc;
    return set_err(c, rc, msg);
  }
  return check_status(c);
}

std::mutex g_default_mu;
wtb_ctx* g_default = nullptr;

}  // namespace

namespace wtb {
int ctx_set_err(wtb_ctx* c, int code, const std::string& m) { return set_err(c, code, m); }
double ctx_vcell3d(const wtb_ctx* c) { return vcell3D(c->rlat_rm); }
int ctx_check_status(wtb_ctx* c) { return check_status(c); }
CoulParams ctx_coul_params(wtb_ctx* c, const wtb_bse_params* p) { return coul_of(c, p); }
int ctx_coulomb_table(wtb_ctx* c, const wtb_bse_params* p, double* V, int ldv, bool deriv_r0) {
  return coulomb_table_into(c, p, V, ldv, deriv_r0);
}
int ctx_make_operator(wtb_ctx* c, const wtb_bse_params* p, int nbmax, OpBundle* ob, const std::string& tag,
                      bool deriv_r0) {
  return make_operator(c, p, nbmax, ob, tag, deriv_r0);
}
}  // namespace wtb

// ================================================================================================ C ABI
extern "C" {

int wtb_version(void) { return 10000; }

const char* wtb_last_error(const wtb_ctx* ctx) { return ctx ? ctx->msg.c_str() : "no context"; }

int wtb_ctx_create(wtb_ctx** out, int device) {
  if (!out) return WTB_EBADARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device || device < 0) return WTB_ENODEV;
  wtb_ctx* c = new wtb_ctx();
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c->st, sizeof(DevStatus)) != cudaSuccess ||
      cudaMemsetAsync(c->st, 0, sizeof(DevStatus), c->s) != cudaSuccess || cudaStreamSynchronize(c->s) != cudaSuccess) {
    delete c;
    return WTB_ENODEV;
  }
  c->ws.stream = c->s;
  *out = c;
  return WTB_OK;
}

int wtb_ctx_destroy(wtb_ctx* c) {
  if (!c) return WTB_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->s);
  c->prof.reset();
  c->ws.bufs.clear();
  if (c->st) cudaFree(c->st);
  if (c->s) cudaStreamDestroy(c->s);
  delete c;
  return WTB_OK;
}

int wtb_set_hr(wtb_ctx* c, int w90basis, int nvec, const int* rvec, const int* ffactor, const double* hop,
               const double* ihop, const double* rlat, double efermi, double scs, int systype_np) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (w90basis < 1 || w90basis > 64) return set_err(c, WTB_EBADARG, "w90basis must be in 1..64");
  if (nvec < 1 || !rvec || !ffactor || !hop || !ihop || !rlat) return set_err(c, WTB_EBADARG, "missing H(R) arrays");
  const int w = w90basis;
  std::vector<zd> hr((size_t)nvec * w * w);
  for (int iR = 0; iR < nvec; ++iR) {
    if (ffactor[iR] <= 0) return set_err(c, WTB_EBADARG, "ffactor (ndegen) must be positive");
    for (int m = 0; m < w; ++m)
      for (int n = 0; n < w; ++n) {
        const size_t f = (size_t)iR + (size_t)nvec * (m + (size_t)w * n);
        const double re = hop[f], im = ihop[f];
        if (!std::isfinite(re) || !std::isfinite(im)) return set_err(c, WTB_ENAN, "non-finite entry in H(R)");
        hr[((size_t)iR * w + m) * w + n] = mk<double>(re, im);
      }
  }
  double rl[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) rl[3 * i + j] = rlat[i + 3 * j];
  if (!std::isfinite(efermi) || !std::isfinite(scs)) return set_err(c, WTB_ENAN, "non-finite efermi or scs");
  // reciprocal vectors exactly as the mesh is built (recvec, src/module_kmesh.F90:391-407), for the
  // V(k,k') table on the mesh
  double bl[9];
  {
    auto cross = [](const double* u, const double* v, double* o) {
      o[0] = u[1] * v[2] - u[2] * v[1];
      o[1] = u[2] * v[0] - u[0] * v[2];
      o[2] = u[0] * v[1] - u[1] * v[0];
    };
    double v23[3], v31[3], v12[3];
    cross(rl + 3, rl + 6, v23);
    cross(rl + 6, rl, v31);
    cross(rl, rl + 3, v12);
    const double vol = std::fabs(rl[0] * v23[0] + rl[1] * v23[1] + rl[2] * v23[2]);
    const double f = (2.0 * (double)3.14159274101257324f) / vol;
    for (int d = 0; d < 3; ++d) {
      bl[d] = f * v23[d];
      bl[3 + d] = f * v31[d];
      bl[6 + d] = f * v12[d];
    }
  }
  cudaError_t err = cudaSuccess;
  zd* dh = c->ws.get<zd>("hr", hr.size(), &err);
  CKC(err);
  int* dr = c->ws.get<int>("rvec", (size_t)nvec * 3, &err);
  CKC(err);
  int* dn = c->ws.get<int>("ndegen", nvec, &err);
  CKC(err);
  double* dl = c->ws.get<double>("rlat", 9, &err);
  double* db = c->ws.get<double>("recip", 9, &err);
  CKC(err);
  CKC(cudaMemcpyAsync(dh, hr.data(), hr.size() * sizeof(zd), cudaMemcpyHostToDevice, c->s));
  CKC(cudaMemcpyAsync(dr, rvec, sizeof(int) * nvec * 3, cudaMemcpyHostToDevice, c->s));
  CKC(cudaMemcpyAsync(dn, ffactor, sizeof(int) * nvec, cudaMemcpyHostToDevice, c->s));
  CKC(cudaMemcpyAsync(dl, rl, sizeof(rl), cudaMemcpyHostToDevice, c->s));
  CKC(cudaMemcpyAsync(db, bl, sizeof(bl), cudaMemcpyHostToDevice, c->s));
  CKC(cudaStreamSynchronize(c->s));
  c->w = w;
  c->nR = nvec;
  c->efermi = efermi;
  c->scs = scs;
  c->systype_np = systype_np;
  std::memcpy(c->rlat_rm, rl, sizeof(rl));
  c->have_hr = true;
  c->have_bands = false;
  c->have_solve = false;
  return WTB_OK;
}

int wtb_monhkhorst_pack(int n1, int n2, int n3, const double* shift, const double* rlat1, const double* rlat2,
                        const double* rlat3, double* kpt) {
  if (n1 < 1 || n2 < 1 || n3 < 1 || !shift || !rlat1 || !rlat2 || !rlat3 || !kpt) return WTB_EBADARG;
  const long nk = (long)n1 * n2 * n3;
  std::vector<double> k((size_t)nk * 3);
  mp_mesh(n1, n2, n3, shift, rlat1, rlat2, rlat3, k.data());
  for (long i = 0; i < nk; ++i)
    for (int d = 0; d < 3; ++d) kpt[i + nk * d] = k[3 * i + d];  // kpt(nk, 3) column-major
  return WTB_OK;
}

int wtb_eigsys(int nthreads, double scs, double exc, int* nocp, const int* ffactor, double kx, double ky, double kz,
               int w90basis, int nvec, const double* rlat, const int* rvec, const double* hop, const double* ihop,
               double efermi, double* energias, double* autovetores) {
  (void)nthreads;
  (void)exc;
  std::lock_guard<std::mutex> lock(g_default_mu);
  if (!g_default) {
    int r = wtb_ctx_create(&g_default, 0);
    if (r) return r;
  }
  wtb_ctx* c = g_default;
  CKR(wtb_set_hr(c, w90basis, nvec, rvec, ffactor, hop, ihop, rlat, efermi, scs, 0));
  const double k[3] = {kx, ky, kz};
  CKR(upload_bands(c, 1, k, 0, 0));
  const int w = w90basis;
  cudaError_t err = cudaSuccess;
  std::vector<double> e(w);
  std::vector<zd> v((size_t)w * w);
  int cnt = 0;
  CKC(cudaMemcpyAsync(e.data(), c->ws.get<double>("eig_all", 0, &err), sizeof(double) * w, cudaMemcpyDeviceToHost, c->s));
  CKC(cudaMemcpyAsync(v.data(), c->ws.get<zd>("vec_all", 0, &err), sizeof(zd) * w * w, cudaMemcpyDeviceToHost, c->s));
  CKC(cudaMemcpyAsync(&cnt, c->ws.get<int>("nocp", 0, &err), sizeof(int), cudaMemcpyDeviceToHost, c->s));
  if (cnt < w) {
    if (nocp) *nocp = cnt;
  } else if (nocp) {
    // no positive eigenvalue: the reference leaves nocp as passed in and adds scs above it
    for (int i = *nocp; i < w; ++i)
      if (i >= 0) e[i] += scs;
  }
  for (int i = 0; i < w; ++i) {
    if (energias) energias[i] = e[i];
    if (autovetores)
      for (int j = 0; j < w; ++j) {
        autovetores[2 * (i + (size_t)w * j)] = v[(size_t)i * w + j].re;
        autovetores[2 * (i + (size_t)w * j) + 1] = v[(size_t)i * w + j].im;
      }
  }
  return WTB_OK;
}

int wtb_eigsys_mesh(wtb_ctx* c, int nk, const double* kpt, int nv, int nc, double* eigv, double* vector, int* nocpk) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!c->have_hr) return set_err(c, WTB_ESTATE, "H(R) not set (call wtb_set_hr first)");
  if (nk < 1 || !kpt || nv < 1 || nc < 1) return set_err(c, WTB_EBADARG, "bad mesh or band window");
  if (nv + nc > c->w) return set_err(c, WTB_EBADARG, "nv + nc exceeds w90basis");
  std::vector<double> k((size_t)nk * 3);
  for (int i = 0; i < nk; ++i)
    for (int d = 0; d < 3; ++d) k[3 * i + d] = kpt[i + (size_t)nk * d];
  CKR(upload_bands(c, nk, k.data(), nv, nc));
  c->mesh_mp = false;
  const int nb = nv + nc, w = c->w;
  cudaError_t err = cudaSuccess;
  if (eigv) {
    std::vector<double> e((size_t)nk * nb);
    CKC(cudaMemcpyAsync(e.data(), c->ws.get<double>("eig_win", 0, &err), e.size() * sizeof(double), cudaMemcpyDeviceToHost, c->s));
    for (int i = 0; i < nk; ++i)
      for (int j = 0; j < nb; ++j) eigv[i + (size_t)nk * j] = e[(size_t)i * nb + j];
  }
  if (vector) {
    std::vector<zd> v((size_t)nk * nb * w);
    CKC(cudaMemcpyAsync(v.data(), c->ws.get<zd>("vec_win", 0, &err), v.size() * sizeof(zd), cudaMemcpyDeviceToHost, c->s));
    for (int i = 0; i < nk; ++i)
      for (int j = 0; j < nb; ++j)
        for (int o = 0; o < w; ++o) {
          const size_t f = (size_t)i + (size_t)nk * (j + (size_t)nb * o);
          vector[2 * f] = v[((size_t)i * nb + j) * w + o].re;
          vector[2 * f + 1] = v[((size_t)i * nb + j) * w + o].im;
        }
  }
  if (nocpk) CKC(cudaMemcpyAsync(nocpk, c->ws.get<int>("nocp", 0, &err), sizeof(int) * nk, cudaMemcpyDeviceToHost, c->s));
  return WTB_OK;
}

int wtb_coulomb_table(wtb_ctx* c, const wtb_bse_params* p, int n1, const double* kpt1, int n2, const double* kpt2,
                      double* V) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!c->have_hr) return set_err(c, WTB_ESTATE, "lattice not set (call wtb_set_hr first)");
  if (!p || n1 < 1 || n2 < 1 || !kpt1 || !kpt2 || !V) return set_err(c, WTB_EBADARG, "bad arguments");
  if (p->coultype < 0 || p->coultype > 8)
    return set_err(c, WTB_EBADARG, "Wrong Coulomb Potential");
  std::vector<double> a((size_t)n1 * 3), b((size_t)n2 * 3);
  for (int i = 0; i < n1; ++i)
    for (int d = 0; d < 3; ++d) a[3 * i + d] = kpt1[i + (size_t)n1 * d];
  for (int i = 0; i < n2; ++i)
    for (int d = 0; d < 3; ++d) b[3 * i + d] = kpt2[i + (size_t)n2 * d];
  cudaError_t err = cudaSuccess;
  double* da = c->ws.get<double>("ct_a", a.size(), &err);
  double* db = c->ws.get<double>("ct_b", b.size(), &err);
  double* dv = c->ws.get<double>("ct_v", (size_t)n1 * n2, &err);
  CKC(err);
  CKC(cudaMemcpyAsync(da, a.data(), a.size() * sizeof(double), cudaMemcpyHostToDevice, c->s));
  CKC(cudaMemcpyAsync(db, b.data(), b.size() * sizeof(double), cudaMemcpyHostToDevice, c->s));
  // V(i,j) column-major = row-major table of (kpt2, kpt1); every potential depends on k1 - k2 through
  // even functions, so V is symmetric under the swap
  CKC(launch_coulomb(coul_of(c, p), db, n2, da, n1, dv, n1, c->s));
  CKC(cudaMemcpyAsync(V, dv, sizeof(double) * n1 * n2, cudaMemcpyDeviceToHost, c->s));
  return check_status(c);
}

int wtb_coulomb_pair(const wtb_bse_params* p, const double* rlat, const double* kpt1, const double* kpt2, double* v) {
  if (!p || !rlat || !kpt1 || !kpt2 || !v) return WTB_EBADARG;
  std::lock_guard<std::mutex> lock(g_default_mu);
  if (!g_default) {
    int r = wtb_ctx_create(&g_default, 0);
    if (r) return r;
  }
  wtb_ctx* c = g_default;
  CKR(prep_device(c));
  if (p->coultype < 0 || p->coultype > 8) return set_err(c, WTB_EBADARG, "Wrong Coulomb Potential");
  // the lattice of this call (rlat(i,:) = a_i, column-major) rather than the context's
  CoulParams cp = coul_of(c, p);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) cp.rlat[3 * i + j] = rlat[i + 3 * j];
  cudaError_t err = cudaSuccess;
  double* dk = c->ws.get<double>("cp_k", 6, &err);
  double* dv = c->ws.get<double>("cp_v", 1, &err);
  CKC(err);
  const double k[6] = {kpt1[0], kpt1[1], kpt1[2], kpt2[0], kpt2[1], kpt2[2]};
  CKC(cudaMemcpyAsync(dk, k, sizeof(k), cudaMemcpyHostToDevice, c->s));
  CKC(launch_coulomb(cp, dk + 3, 1, dk, 1, dv, 1, c->s));
  CKC(cudaMemcpyAsync(v, dv, sizeof(double), cudaMemcpyDeviceToHost, c->s));
  CKC(cudaStreamSynchronize(c->s));
  return check_status(c);
}

// hlm / optsp at one k-point on the default context: H(R) staged as wtb_eigsys stages it, then one hlm_kernel
static int hlm_common(double kx, double ky, double kz, const int* ffactor, int w90basis, int nvec, const double* rlat,
                      const int* rvec, const double* hop, const double* ihop, const double* cv, const double* vv,
                      double ev, double ec, double sme, double* out, int nout) {
  std::lock_guard<std::mutex> lock(g_default_mu);
  if (!g_default) {
    int r = wtb_ctx_create(&g_default, 0);
    if (r) return r;
  }
  wtb_ctx* c = g_default;
  CKR(wtb_set_hr(c, w90basis, nvec, rvec, ffactor, hop, ihop, rlat, 0.0, 0.0, 0));
  const int w = w90basis;
  cudaError_t err = cudaSuccess;
  zd* dvec = c->ws.get<zd>("hlm_vec", (size_t)2 * w, &err);
  zd* dout = c->ws.get<zd>("hlm_out", (size_t)nout, &err);
  double* drl = c->ws.get<double>("hlm_rlat", 9, &err);
  CKC(err);
  double rl[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) rl[3 * i + j] = rlat[i + 3 * j];
  CKC(cudaMemcpyAsync(drl, rl, sizeof(rl), cudaMemcpyHostToDevice, c->s));
  if (cv) {
    CKC(cudaMemcpyAsync(dvec, cv, sizeof(zd) * w, cudaMemcpyHostToDevice, c->s));
    CKC(cudaMemcpyAsync(dvec + w, vv, sizeof(zd) * w, cudaMemcpyHostToDevice, c->s));
  }
  CKC(launch_hlm(c->ws.get<zd>("hr", 0, &err), c->ws.get<int>("rvec", 0, &err), c->ws.get<int>("ndegen", 0, &err), nvec, w,
                 drl, kx, ky, kz, cv ? dvec : nullptr, cv ? dvec + w : nullptr, ev, ec, sme, dout, c->s));
  CKC(cudaMemcpyAsync(out, dout, sizeof(zd) * nout, cudaMemcpyDeviceToHost, c->s));
  CKC(cudaStreamSynchronize(c->s));
  return check_status(c);
}

int wtb_hlm(double kx, double ky, double kz, const int* ffactor, int w90basis, int nvec, const double* rlat,
            const int* rvec, const double* hop, const double* ihop, double* hx, double* hy, double* hz) {
  if (!ffactor || !rlat || !rvec || !hop || !ihop || !hx || !hy || !hz || w90basis < 1 || w90basis > 64 || nvec < 1)
    return WTB_EBADARG;
  const int w = w90basis;
  std::vector<double> out((size_t)6 * w * w);
  CKR(hlm_common(kx, ky, kz, ffactor, w, nvec, rlat, rvec, hop, ihop, nullptr, nullptr, 0.0, 0.0, 0.0, out.data(),
                 3 * w * w));
  std::memcpy(hx, out.data(), sizeof(double) * 2 * w * w);
  std::memcpy(hy, out.data() + 2 * w * w, sizeof(double) * 2 * w * w);
  std::memcpy(hz, out.data() + 4 * w * w, sizeof(double) * 2 * w * w);
  return WTB_OK;
}

int wtb_optsp_pair(double ev, const double* vv, double ec, const double* vc, double kx, double ky, double kz,
                   const int* ffactor, double sme, int w90basis, int nvec, const double* rlat, const int* rvec,
                   const double* hop, const double* ihop, double* hrx, double* hry, double* hrz) {
  if (!vv || !vc || !ffactor || !rlat || !rvec || !hop || !ihop || !hrx || !hry || !hrz || w90basis < 1 ||
      w90basis > 64 || nvec < 1)
    return WTB_EBADARG;
  double out[6];
  CKR(hlm_common(kx, ky, kz, ffactor, w90basis, nvec, rlat, rvec, hop, ihop, vc, vv, ev, ec, sme, out, 3));
  hrx[0] = out[0];
  hrx[1] = out[1];
  hry[0] = out[2];
  hry[1] = out[3];
  hrz[0] = out[4];
  hrz[1] = out[5];
  return WTB_OK;
}

int wtb_optdiel(int rtype, double vc, int dimse, const int* ngrid, double elux, const double* exciton,
                const double* fosc, double sme, double* rpart, double* ipart) {
  if (dimse < 1 || !ngrid || !exciton || !fosc || !rpart || !ipart) return WTB_EBADARG;
  std::lock_guard<std::mutex> lock(g_default_mu);
  if (!g_default) {
    int r = wtb_ctx_create(&g_default, 0);
    if (r) return r;
  }
  wtb_ctx* c = g_default;
  CKR(prep_device(c));
  cudaError_t err = cudaSuccess;
  double* dE = c->ws.get<double>("od_E", dimse, &err);
  double* df = c->ws.get<double>("od_f", dimse, &err);
  double* dout = c->ws.get<double>("od_out", 2, &err);
  CKC(err);
  CKC(cudaMemcpyAsync(dE, exciton, sizeof(double) * dimse, cudaMemcpyHostToDevice, c->s));
  CKC(cudaMemcpyAsync(df, fosc, sizeof(double) * dimse, cudaMemcpyHostToDevice, c->s));
  // caux = gama/(real(ngrid(1)*ngrid(2)*ngrid(3))*vc), gama the single-precision literal 180.90
  const double baux = (double)(float)(ngrid[0] * ngrid[1] * ngrid[2]) * vc;
  CKC(launch_optdiel(rtype, (double)180.90f / (baux * 1.0), dimse, elux, dE, df, sme, dout, c->s));
  double o[2];
  CKC(cudaMemcpyAsync(o, dout, sizeof(o), cudaMemcpyDeviceToHost, c->s));
  CKC(cudaStreamSynchronize(c->s));
  *rpart = o[0];
  *ipart = o[1];
  return check_status(c);
}

// the Monkhorst-Pack mesh of p staged for the band computation
static int stage_mesh(wtb_ctx* c, const wtb_bse_params* p) {
  const int nk = p->ngrid[0] * p->ngrid[1] * p->ngrid[2];
  std::vector<double> k((size_t)nk * 3);
  mp_mesh(p->ngrid[0], p->ngrid[1], p->ngrid[2], p->mshift, c->rlat_rm, c->rlat_rm + 3, c->rlat_rm + 6, k.data());
  CKR(stage_bands(c, nk, k.data(), p->nv, p->nc));
  for (int d = 0; d < 3; ++d) c->ngrid[d] = p->ngrid[d];
  c->mesh_mp = true;
  return WTB_OK;
}

static int ensure_bands_for(wtb_ctx* c, const wtb_bse_params* p) {
  CKR(stage_mesh(c, p));
  CKR(enqueue_bands(c, reduced_form(p)));
  return check_status(c);
}

static int compute_optics(wtb_ctx* c, const wtb_bse_params* p) {
  cudaError_t err = cudaSuccess;
  const int dim = c->nk * c->nc * c->nv;
  zd* hout = c->ws.get<zd>("hrvel", (size_t)5 * dim, &err);
  CKC(err);
  // the reduced-precision matrix-free forms: Fourier sums in FP32 over an FP32 copy of H(R)
  zf* hr32 = nullptr;
  if (reduced_form(p)) {
    const size_t nh = (size_t)c->nR * c->w * c->w;
    hr32 = c->ws.get<zf>("hr32", nh, &err);
    CKC(err);
    CKC((launch_convert_cols<double, float>(c->ws.get<zd>("hr", 0, &err), 1, hr32, 1, 1, (int)nh, c->s)));
  }
  CKC(launch_optics(c->ws.get<zd>("hr", 0, &err), c->ws.get<int>("rvec", 0, &err), c->ws.get<int>("ndegen", 0, &err),
                    c->nR, c->w, c->ws.get<double>("rlat", 0, &err), c->ws.get<double>("kpt", 0, &err), c->nk, c->nv,
                    c->nc, c->ws.get<double>("eig_win", 0, &err), c->ws.get<zd>("vec_win", 0, &err), p->cshift, hout,
                    c->s, hr32));
  c->have_hr_optics = true;
  c->have_solve = false;  // hrvel now follows p->cshift; wtb_bsesolver sets it again after its solve
  return WTB_OK;
}

int wtb_optsp(wtb_ctx* c, const wtb_bse_params* p, double* hr) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!c->have_bands) return set_err(c, WTB_ESTATE, "no bands (call wtb_eigsys_mesh or wtb_bsesolver first)");
  if (!p) return set_err(c, WTB_EBADARG, "params is NULL");
  CKR(compute_optics(c, p));
  const int dim = c->nk * c->nc * c->nv;
  cudaError_t err = cudaSuccess;
  if (hr)
    CKC(cudaMemcpyAsync(hr, c->ws.get<zd>("hrvel", 0, &err), sizeof(zd) * 5 * dim, cudaMemcpyDeviceToHost, c->s));
  return check_status(c);
}

int wtb_bse_build(wtb_ctx* c, const wtb_bse_params* p, double* hbse) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!c->have_bands) return set_err(c, WTB_ESTATE, "no bands (call wtb_eigsys_mesh first)");
  if (!p) return set_err(c, WTB_EBADARG, "params is NULL");
  if (p->coultype < 0 || p->coultype > 8)
    return set_err(c, WTB_EBADARG, "Wrong Coulomb Potential");
  if (!(p->ktol > 0.0)) return set_err(c, WTB_EBADARG, "KTOL must be > 0");
  if (p->precision != WTB_PREC_FP64 && p->precision != WTB_PREC_FP32)
    return set_err(c, WTB_EBADARG, "the dense build stores FP64 or FP32");
  const int nk = c->nk, nv = c->nv, nc = c->nc, w = c->w;
  const long dim = (long)nk * nc * nv;
  cudaError_t err = cudaSuccess;
  double* dE = c->ws.get<double>("dE", dim, &err);
  CKC(err);
  CKC(launch_transition_energies(c->ws.get<double>("eig_win", 0, &err), nk, nv, nc, dE, c->s));
  const int Kpad = (nk + 63) / 64 * 64;
  double* V = c->ws.get<double>("V", (size_t)((nk + 127) / 128 * 128) * Kpad, &err, true);
  CKC(err);
  CKR(coulomb_table_into(c, p, V, Kpad));
  const zd* vw = c->ws.get<zd>("vec_win", 0, &err);
  zd* staging = nullptr;
  if (p->precision == WTB_PREC_FP64) {
    zd* H = c->ws.get<zd>("H64", (size_t)dim * dim, &err);
    CKC(err);
    CKC(launch_bse_build<double>(vw, dE, V, Kpad, nk, nv, nc, w, H, c->s));
    if (hbse) {
      staging = c->ws.get<zd>("Hout", (size_t)dim * dim, &err);
      CKC(err);
      conj_convert_kernel<double><<<(unsigned)((dim * dim + 255) / 256), 256, 0, c->s>>>(H, dim * dim, staging); ++g_launch_count;
    }
  } else {
    zf* H = c->ws.get<zf>("H32", (size_t)dim * dim, &err);
    CKC(err);
    CKC(launch_bse_build<float>(vw, dE, V, Kpad, nk, nv, nc, w, H, c->s));
    if (hbse) {
      staging = c->ws.get<zd>("Hout", (size_t)dim * dim, &err);
      CKC(err);
      conj_convert_kernel<float><<<(unsigned)((dim * dim + 255) / 256), 256, 0, c->s>>>(H, dim * dim, staging); ++g_launch_count;
    }
  }
  CKC(cudaGetLastError());
  if (hbse) CKC(cudaMemcpyAsync(hbse, staging, sizeof(zd) * dim * dim, cudaMemcpyDeviceToHost, c->s));
  return check_status(c);
}

int wtb_kpathbse(const double* rlat1, const double* rlat2, const double* rlat3, int nks, const double* ks, int npts,
                 double* qpath) {
  if (!rlat1 || !rlat2 || !rlat3 || !ks || !qpath || nks < 2 || npts < 2) return WTB_EBADARG;
  double b1[3], b2[3], b3[3];
  recvec(rlat1, rlat2, rlat3, b1, b2, b3);
  std::vector<double> ksaux((size_t)nks * 3);
  for (int i = 0; i < nks; ++i)
    for (int d = 0; d < 3; ++d)
      ksaux[3 * i + d] = ks[i] * b1[d] + ks[i + nks] * b2[d] + ks[i + 2 * nks] * b3[d];
  const int nseg = nks / 2, nq = nseg * npts;
  std::vector<double> kdis(nseg);
  double kdistot = 0.0;
  for (int i = 0; i < nseg; ++i) {
    const double* a = &ksaux[3 * (2 * i + 1)];
    const double* b = &ksaux[3 * (2 * i)];
    kdis[i] = std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
    kdistot = kdistot + kdis[i];
  }
  for (int i = 0; i < nseg; ++i) kdis[i] = kdis[i] / kdistot;
  double kdisaux = 0.0;
  for (int j = 0; j < nseg; ++j) {
    for (int i = 0; i < npts; ++i) {
      const int r = j * npts + i;
      const double ti = (double)i, tn = (double)npts - 1.0;
      qpath[r] = kdisaux + kdis[j] * ti / tn;
      for (int d = 0; d < 3; ++d)
        qpath[r + (size_t)nq * (1 + d)] =
            ksaux[3 * (2 * j) + d] + (ksaux[3 * (2 * j + 1) + d] - ksaux[3 * (2 * j) + d]) * ti / tn;
    }
    kdisaux = kdisaux + kdis[j];
  }
  return WTB_OK;
}

// The finite-Q matrix of one Q-path row q4 = (path coordinate, Q) into the row-major dim x dim "HQ" buffer:
// bands on the Q-shifted mesh, the merged window, the direct build over V (leading dimension ldv) and, for
// |Q| != 0, the exchange term.  The plain-mesh bands must be current.
static int build_q_matrix(wtb_ctx* c, const wtb_bse_params* p, const double* q4, const double* V, int ldv, double scs,
                          zd** Hout) {
  const int nk = c->nk, nv = c->nv, nc = c->nc, w = c->w, nb = nv + nc;
  const long dim = (long)nk * nc * nv;
  cudaError_t err = cudaSuccess;
  std::vector<double> kq((size_t)nk * 3);
  mp_mesh(p->ngrid[0], p->ngrid[1], p->ngrid[2], p->mshift, c->rlat_rm, c->rlat_rm + 3, c->rlat_rm + 6, kq.data(), q4);
  double* dkq = c->ws.get<double>("kptq", (size_t)nk * 3 + 6, &err);
  double* eq_all = c->ws.get<double>("eigq_all", (size_t)nk * w, &err);
  zd* vq_all = c->ws.get<zd>("vecq_all", (size_t)nk * w * w, &err);
  double* eq_win = c->ws.get<double>("eigq_win", (size_t)nk * nb, &err);
  zd* vq_win = c->ws.get<zd>("vecq_win", (size_t)nk * nb * w, &err);
  int* nocpq = c->ws.get<int>("nocpq", nk, &err);
  double* em = c->ws.get<double>("eigm_win", (size_t)nk * nb, &err);
  zd* vm = c->ws.get<zd>("vecm_win", (size_t)nk * nb * w, &err);
  double* dE = c->ws.get<double>("dEq", dim, &err);
  zd* u = c->ws.get<zd>("xq_u", dim, &err);
  double* dvq = c->ws.get<double>("xq_v", 2, &err);
  zd* H = c->ws.get<zd>("HQ", (size_t)dim * dim, &err);
  CKC(err);
  // the Q point and the origin follow the mesh in the same buffer (coulomb pair V(Q, 0))
  for (int d = 0; d < 3; ++d) {
    kq.push_back(q4[1 + d]);
  }
  for (int d = 0; d < 3; ++d) kq.push_back(0.0);
  CKC(cudaMemcpyAsync(dkq, kq.data(), sizeof(double) * kq.size(), cudaMemcpyHostToDevice, c->s));
  CKC(launch_hk_eig(c->ws.get<zd>("hr", 0, &err), c->ws.get<int>("rvec", 0, &err), c->ws.get<int>("ndegen", 0, &err),
                    c->nR, w, c->ws.get<double>("rlat", 0, &err), c->efermi, scs, dkq, nk, nv, nc, eq_all, vq_all,
                    eq_win, vq_win, nocpq, c->st, c->s, false));
  CKC(launch_merge_windows(c->ws.get<double>("eig_win", 0, &err), c->ws.get<zd>("vec_win", 0, &err), eq_win, vq_win,
                           nk, nv, nc, w, em, vm, c->s));
  CKC(launch_transition_energies(em, nk, nv, nc, dE, c->s));
  CKC(launch_bse_build<double>(vm, dE, V, ldv, nk, nv, nc, w, H, c->s));
  const double modq = std::sqrt(q4[1] * q4[1] + q4[2] * q4[2] + q4[3] * q4[3]);  // modvecq
  if (modq != 0.0) {
    CKC(launch_coulomb(coul_of(c, p), dkq + (size_t)nk * 3, 1, dkq + (size_t)nk * 3 + 3, 1, dvq, 1, c->s));
    CKC(launch_exchange(vm, nk, nv, nc, w, dvq, u, H, c->s));
  }
  *Hout = H;
  return WTB_OK;
}

static int check_q_params(wtb_ctx* c, const wtb_bse_params* p) {
  if (!c->have_hr) return set_err(c, WTB_ESTATE, "H(R) not set (call wtb_set_hr first)");
  CKR(validate_params(c, p));
  if (p->nv + p->nc > c->w) return set_err(c, WTB_EBADARG, "nv + nc exceeds w90basis");
  const long dim = (long)p->ngrid[0] * p->ngrid[1] * p->ngrid[2] * p->nc * p->nv;
  if (dim > 20000) return set_err(c, WTB_EBADARG, "the finite-Q dense solve holds dim^2 complex entries: dim <= 20000");
  return WTB_OK;
}

int wtb_bse_build_q(wtb_ctx* c, const wtb_bse_params* p, const double* q4, double* hbse) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!p || !q4) return set_err(c, WTB_EBADARG, "bad arguments");
  CKR(check_q_params(c, p));
  CKR(stage_mesh(c, p));
  CKR(enqueue_bands(c, false));
  const int nk = c->nk;
  const long dim = (long)nk * c->nc * c->nv;
  cudaError_t err = cudaSuccess;
  const int Kpad = (nk + 63) / 64 * 64;
  double* V = c->ws.get<double>("V", (size_t)((nk + 127) / 128 * 128) * Kpad, &err, true);
  CKC(err);
  CKR(coulomb_table_into(c, p, V, Kpad));
  zd* H = nullptr;
  CKR(build_q_matrix(c, p, q4, V, Kpad, c->scs, &H));
  if (hbse) {
    zd* staging = c->ws.get<zd>("Hout", (size_t)dim * dim, &err);
    CKC(err);
    conj_convert_kernel<double><<<(unsigned)((dim * dim + 255) / 256), 256, 0, c->s>>>(H, dim * dim, staging); ++g_launch_count;
    CKC(cudaGetLastError());
    CKC(cudaMemcpyAsync(hbse, staging, sizeof(zd) * dim * dim, cudaMemcpyDeviceToHost, c->s));
  }
  return check_status(c);
}

int wtb_bse_q_eigenpairs(wtb_ctx* c, const wtb_bse_params* p, const double* q4, int il, int nvec, double* W,
                         double* Z) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!p || !q4 || !W || (nvec > 0 && !Z)) return set_err(c, WTB_EBADARG, "bad arguments");
  CKR(check_q_params(c, p));
  const long dim = (long)p->ngrid[0] * p->ngrid[1] * p->ngrid[2] * p->nc * p->nv;
  if (nvec < 0 || il < 1 || il - 1 + nvec > dim) return set_err(c, WTB_EBADARG, "eigenvector range outside 1..dim");
  CKR(stage_mesh(c, p));
  CKR(enqueue_bands(c, false));
  const int nk = c->nk;
  cudaError_t err = cudaSuccess;
  const int Kpad = (nk + 63) / 64 * 64;
  double* V = c->ws.get<double>("V", (size_t)((nk + 127) / 128 * 128) * Kpad, &err, true);
  void* scratch = c->ws.get<zd>("deig_scratch", (dense_eig_scratch((int)dim) + sizeof(zd) - 1) / sizeof(zd), &err);
  void* vscratch = c->ws.get<double>("deig_vscratch", dense_eigvec_scratch((int)dim) / sizeof(double), &err);
  double* dW = c->ws.get<double>("deig_W", dim, &err);
  zd* dZ = c->ws.get<zd>("T_Z", (size_t)dim * dim, &err);
  CKC(err);
  CKR(coulomb_table_into(c, p, V, Kpad));
  zd* H = nullptr;
  CKR(build_q_matrix(c, p, q4, V, Kpad, c->scs, &H));
  CKC(dense_eig_prepare());
  // H row-major is conj(H) column-major: the vectors are conjugated back
  CKC(launch_dense_eig(H, (int)dim, (int)dim, false, dW, dZ, true, scratch, vscratch, c->s));
  CKC(cudaMemcpyAsync(W, dW, sizeof(double) * dim, cudaMemcpyDeviceToHost, c->s));
  if (nvec > 0) {
    // columns il..il+nvec-1 of the row-major Z into the column-major Z(dim, nvec) over the dead matrix H
    transpose_z_kernel<<<(unsigned)((dim * nvec + 255) / 256), 256, 0, c->s>>>(dZ + (il - 1), (int)dim, nvec, (int)dim,
                                                                              H, 0);
    ++g_launch_count;
    CKC(cudaGetLastError());
    CKC(cudaMemcpyAsync(Z, H, sizeof(zd) * dim * nvec, cudaMemcpyDeviceToHost, c->s));
  }
  return check_status(c);
}

static double temp_gap_correction(const wtb_temp_params* tp);

// The Q loop of bsebnds, or of bsebndstemp with tp (scissor scs + tcor on both meshes, matrizelbsekqtemp's
// weighting by f_v - f_c of the row's transition).
static int bsebnds_impl(wtb_ctx* c, const wtb_bse_params* p, const wtb_temp_params* tp, int nq, const double* qpath,
                        double* exk) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!p || nq < 1 || !qpath || !exk) return set_err(c, WTB_EBADARG, "bad arguments");
  CKR(check_q_params(c, p));
  if (tp && (tp->ta < 0 || tp->ta > 2 || !(tp->temp >= 0.0))) return set_err(c, WTB_EBADARG, "bad temperature keys");
  const double scs = c->scs + (tp ? temp_gap_correction(tp) : 0.0);
  CKR(stage_mesh(c, p));
  const double scs0 = c->scs;
  c->scs = scs;
  const int rb = enqueue_bands(c, false);
  c->scs = scs0;
  CKR(rb);
  const int nk = c->nk;
  const long dim = (long)nk * c->nc * c->nv;
  cudaError_t err = cudaSuccess;
  const int Kpad = (nk + 63) / 64 * 64;
  double* V = c->ws.get<double>("V", (size_t)((nk + 127) / 128 * 128) * Kpad, &err, true);
  void* scratch = c->ws.get<zd>("deig_scratch", (dense_eig_scratch((int)dim) + sizeof(zd) - 1) / sizeof(zd), &err);
  double* W = c->ws.get<double>("deig_W", dim, &err);
  CKC(err);
  CKR(coulomb_table_into(c, p, V, Kpad));
  CKC(dense_eig_prepare());
  // the eigenvalue sequence (4 launches per column) is captured once and replayed for every Q: same buffers
  cudaGraphExec_t ge = nullptr;
  zd* Hcap = nullptr;
  int rc = WTB_OK;
  for (int i = 0; i < nq && rc == WTB_OK; ++i) {
    const double q4[4] = {qpath[i], qpath[i + nq], qpath[i + 2 * (size_t)nq], qpath[i + 3 * (size_t)nq]};
    zd* H = nullptr;
    rc = build_q_matrix(c, p, q4, V, Kpad, scs, &H);
    if (rc != WTB_OK) break;
    if (tp) {
      cudaError_t e = cudaSuccess;
      double* f = c->ws.get<double>("T_fq", dim, &e);
      const double* em = c->ws.get<double>("eigm_win", 0, &e);
      const double* dEq = c->ws.get<double>("dEq", 0, &e);
      if (e == cudaSuccess) e = launch_fermi_weights(em, nk, c->nv, c->nc, tp->temp, f, c->s);
      if (e == cudaSuccess) e = launch_temp_weight(H, dim, f, dEq, c->s);
      if (e != cudaSuccess) {
        rc = set_err(c, WTB_ECUDA, std::string("bsebndstemp weights: ") + cudaGetErrorString(e));
        break;
      }
    }
    if (!ge || H != Hcap) {
      if (ge) cudaGraphExecDestroy(ge);
      ge = nullptr;
      cudaGraph_t graph = nullptr;
      cudaError_t e1 = cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal);
      // H is row-major Hermitian, i.e. conj(H) column-major: the same eigenvalues
      cudaError_t e2 = e1 == cudaSuccess ? launch_dense_eigvals(H, (int)dim, (int)dim, false, W, scratch, c->s) : e1;
      cudaError_t e3 = e1 == cudaSuccess ? cudaStreamEndCapture(c->s, &graph) : e1;
      cudaError_t e4 = (e2 == cudaSuccess && e3 == cudaSuccess) ? cudaGraphInstantiate(&ge, graph, 0) : e2;
      if (graph) cudaGraphDestroy(graph);
      const cudaError_t e = e2 != cudaSuccess ? e2 : e3 != cudaSuccess ? e3 : e4;
      if (e != cudaSuccess) {
        rc = set_err(c, WTB_ECUDA, std::string("dense eigenvalue graph: ") + cudaGetErrorString(e));
        break;
      }
      Hcap = H;
    }
    cudaError_t e = cudaGraphLaunch(ge, c->s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(exk + (size_t)i * dim, W, sizeof(double) * dim, cudaMemcpyDeviceToHost, c->s);
    if (e != cudaSuccess) {
      rc = set_err(c, WTB_ECUDA, std::string("bsebnds: ") + cudaGetErrorString(e));
      break;
    }
    rc = check_status(c);
  }
  if (ge) cudaGraphExecDestroy(ge);
  c->have_solve = false;
  if (rc != WTB_OK) return rc;
  return check_status(c);
}

int wtb_bsebnds(wtb_ctx* c, const wtb_bse_params* p, int nq, const double* qpath, double* exk) {
  return bsebnds_impl(c, p, nullptr, nq, qpath, exk);
}

int wtb_bsebndstemp(wtb_ctx* c, const wtb_bse_params* p, const wtb_temp_params* tp, int nq, const double* qpath,
                    double* exk) {
  if (!tp) return set_err(c, WTB_EBADARG, "temperature keys are NULL");
  return bsebnds_impl(c, p, tp, nq, qpath, exk);
}

int wtb_zheev(wtb_ctx* c, int n, const double* A, int lda, double* W) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (n < 1 || lda < n || !A || !W) return set_err(c, WTB_EBADARG, "bad matrix size");
  cudaError_t err = cudaSuccess;
  zd* dA = c->ws.get<zd>("zh_A", (size_t)n * n, &err);
  void* scratch = c->ws.get<zd>("deig_scratch", (dense_eig_scratch(n) + sizeof(zd) - 1) / sizeof(zd), &err);
  double* dW = c->ws.get<double>("deig_W", n, &err);
  CKC(err);
  CKC(cudaMemcpy2DAsync(dA, sizeof(zd) * n, A, sizeof(zd) * lda, sizeof(zd) * n, n, cudaMemcpyHostToDevice, c->s));
  CKC(launch_dense_eigvals(dA, n, n, true, dW, scratch, c->s));
  CKC(cudaMemcpyAsync(W, dW, sizeof(double) * n, cudaMemcpyDeviceToHost, c->s));
  return check_status(c);
}

int wtb_zheev_vectors(wtb_ctx* c, int n, const double* A, int lda, double* W, double* Z) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (n < 1 || lda < n || !A || !W || !Z) return set_err(c, WTB_EBADARG, "bad matrix size");
  cudaError_t err = cudaSuccess;
  zd* dA = c->ws.get<zd>("zh_A", (size_t)n * n, &err);
  zd* dZ = c->ws.get<zd>("zh_Z", (size_t)n * n, &err);
  zd* dZc = c->ws.get<zd>("zh_Zc", (size_t)n * n, &err);
  void* scratch = c->ws.get<zd>("deig_scratch", (dense_eig_scratch(n) + sizeof(zd) - 1) / sizeof(zd), &err);
  void* vscratch = c->ws.get<double>("deig_vscratch", dense_eigvec_scratch(n) / sizeof(double), &err);
  double* dW = c->ws.get<double>("deig_W", n, &err);
  CKC(err);
  CKC(cudaMemcpy2DAsync(dA, sizeof(zd) * n, A, sizeof(zd) * lda, sizeof(zd) * n, n, cudaMemcpyHostToDevice, c->s));
  CKC(dense_eig_prepare());
  CKC(launch_dense_eig(dA, n, n, true, dW, dZ, false, scratch, vscratch, c->s));
  transpose_z_kernel<<<(unsigned)(((long)n * n + 255) / 256), 256, 0, c->s>>>(dZ, n, n, n, dZc, 0); ++g_launch_count;
  CKC(cudaGetLastError());
  CKC(cudaMemcpyAsync(W, dW, sizeof(double) * n, cudaMemcpyDeviceToHost, c->s));
  CKC(cudaMemcpyAsync(Z, dZc, sizeof(zd) * n * n, cudaMemcpyDeviceToHost, c->s));
  return check_status(c);
}

// Gap corrections of bsesolvertemp's ta key (gapcortemp, gapcortemp2: src/module_math.F90:383-403); kb is the
// single-precision literal of the reference.
static double temp_gap_correction(const wtb_temp_params* tp) {
  const double kb = (double)8.617330350E-5f;
  if (tp->ta == 1) {
    const double aux1 = tp->phavg / ((2.0 * kb) * tp->temp);  // 2.0*kb is a single-precision product, exact
    const double aux2 = 1 / std::tanh(aux1);
    return -tp->st * tp->phavg * (aux2 - 1.0);
  }
  if (tp->ta == 2) {
    const double aux1 = 2.0 * tp->st;
    const double aux2 = std::exp(tp->phavg / tp->temp);
    return -(aux1 / (aux2 - 1.0));
  }
  return 0.0;
}

int wtb_bsesolvertemp(wtb_ctx* c, const wtb_bse_params* p, const wtb_temp_params* tp, double* Ws, double* acts,
                      double* HE, double* fdeh) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!p || !tp) return set_err(c, WTB_EBADARG, "bad arguments");
  if (tp->ta < 0 || tp->ta > 2 || !(tp->temp >= 0.0)) return set_err(c, WTB_EBADARG, "bad temperature keys");
  CKR(check_q_params(c, p));
  wtb_bse_params pp = *p;  // the full-spectrum path is FP64 throughout
  pp.precision = WTB_PREC_FP64;
  pp.op = WTB_OP_DENSE;
  const double tcor = temp_gap_correction(tp);
  CKR(stage_mesh(c, &pp));
  const double scs0 = c->scs;
  c->scs = scs0 + tcor;
  const int rb = enqueue_bands(c, false);
  c->scs = scs0;
  CKR(rb);
  CKR(compute_optics(c, &pp));
  const int nk = c->nk, nv = c->nv, nc = c->nc, w = c->w;
  const long dim = (long)nk * nc * nv;
  cudaError_t err = cudaSuccess;
  const int Kpad = (nk + 63) / 64 * 64;
  double* V = c->ws.get<double>("V", (size_t)((nk + 127) / 128 * 128) * Kpad, &err, true);
  double* dE = c->ws.get<double>("dE", dim, &err);
  double* f = c->ws.get<double>("T_f", dim, &err);
  zd* H = c->ws.get<zd>("HT", (size_t)dim * dim, &err);
  zd* Z = c->ws.get<zd>("T_Z", (size_t)dim * dim, &err);
  double* W = c->ws.get<double>("deig_W", dim, &err);
  double* dacts = c->ws.get<double>("T_acts", (size_t)8 * dim, &err);
  void* scratch = c->ws.get<zd>("deig_scratch", (dense_eig_scratch((int)dim) + sizeof(zd) - 1) / sizeof(zd), &err);
  void* vscratch = c->ws.get<double>("deig_vscratch", dense_eigvec_scratch((int)dim) / sizeof(double), &err);
  CKC(err);
  const double* eig_win = c->ws.get<double>("eig_win", 0, &err);
  CKC(launch_transition_energies(eig_win, nk, nv, nc, dE, c->s));
  CKR(coulomb_table_into(c, &pp, V, Kpad));
  CKC(launch_bse_build<double>(c->ws.get<zd>("vec_win", 0, &err), dE, V, Kpad, nk, nv, nc, w, H, c->s));
  CKC(launch_fermi_weights(eig_win, nk, nv, nc, tp->temp, f, c->s));
  CKC(launch_temp_weight(H, dim, f, dE, c->s));
  CKC(dense_eig_prepare());
  // H is row-major, i.e. conj(H) column-major: its eigenvectors are conjugated back
  CKC(launch_dense_eig(H, (int)dim, (int)dim, false, W, Z, true, scratch, vscratch, c->s));
  CKC(launch_temp_acts(Z, (int)dim, c->ws.get<zd>("hrvel", 0, &err), f, tp->dtfull, tp->cpol, dacts, c->s));
  if (Ws) CKC(cudaMemcpyAsync(Ws, W, sizeof(double) * dim, cudaMemcpyDeviceToHost, c->s));
  if (acts) CKC(cudaMemcpyAsync(acts, dacts, sizeof(double) * 8 * dim, cudaMemcpyDeviceToHost, c->s));
  if (fdeh) CKC(cudaMemcpyAsync(fdeh, f, sizeof(double) * dim, cudaMemcpyDeviceToHost, c->s));
  if (HE) {
    // the column-major copy reuses the matrix buffer (H is no longer needed)
    transpose_z_kernel<<<(unsigned)((dim * dim + 255) / 256), 256, 0, c->s>>>(Z, (int)dim, (int)dim, (int)dim, H, 0);
    ++g_launch_count;
    CKC(cudaGetLastError());
    CKC(cudaMemcpyAsync(HE, H, sizeof(zd) * dim * dim, cudaMemcpyDeviceToHost, c->s));
  }
  c->have_solve = false;
  return check_status(c);
}

int wtb_slepc_solver(wtb_ctx* c, const double* HX, double* EX, double* HE, int NX, int NE) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!HX || NX < 1 || NE < 1 || NE > NX) return set_err(c, WTB_EBADARG, "bad matrix size or NE");
  cudaError_t err = cudaSuccess;
  const long n2 = (long)NX * NX;
  zd* H = c->ws.get<zd>("slepc_H", n2, &err);
  double* d = c->ws.get<double>("slepc_d", NX, &err);
  zd* X = c->ws.get<zd>("slepc_X", (size_t)NX * NE, &err);
  zd* HEd = c->ws.get<zd>("slepc_HE", (size_t)NX * NE, &err);
  CKC(err);
  CKC(cudaMemcpyAsync(H, HX, sizeof(zd) * n2, cudaMemcpyHostToDevice, c->s));
  // column-major HX read row-major is H^T = conj(H)
  conj_inplace_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, c->s>>>(H, n2); ++g_launch_count;
  diag_real_kernel<<<(NX + 255) / 256, 256, 0, c->s>>>(H, NX, d); ++g_launch_count;
  CKC(cudaGetLastError());
  DenseOperator<double> op;
  op.H = H;
  op.dim = NX;
  wtb_bse_params p{};
  p.nev = NE;
  const int m = auto_block(&p, NX, true);
  std::vector<double> E;
  SolveStats stats;
  std::string msg;
  int rc;
  if (NE > block_cap(true)) {
    // the reference's NE = 100: chunks of 16 with deflation
    double sigma = 0.0;
    CKR(deflation_shift(c, d, NX, &sigma));
    rc = lobpcg_solve_deflated<double>(op, d, NX, NE, 16, 24, 1e-8, 200, sigma, c->ws, c->st, c->s, &E, X, &stats, &msg);
  } else {
    rc = lobpcg_solve<double>(op, d, NX, NE, m, 1e-8, 200, c->ws, c->st, c->s, &E, X, &stats, &msg);
  }
  if (rc != WTB_OK) return set_err(c, rc, msg);
  for (int i = 0; i < NE; ++i)
    if (EX) EX[i] = E[i];
  if (HE) {
    transpose_z_kernel<<<(unsigned)(((long)NX * NE + 255) / 256), 256, 0, c->s>>>(X, NX, NE, NE, HEd, 0); ++g_launch_count;
    CKC(cudaGetLastError());
    CKC(cudaMemcpyAsync(HE, HEd, sizeof(zd) * NX * NE, cudaMemcpyDeviceToHost, c->s));
  }
  return check_status(c);
}

int wtb_dielbse(wtb_ctx* c, int dimse, int dimse1, const double* excitonvec, const double* hopt1, const double* hopt2,
                int pair, double* activity) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (dimse < 1 || dimse1 < 0 || dimse1 > dimse || !excitonvec || !hopt1 || (pair && !hopt2) || !activity)
    return set_err(c, WTB_EBADARG, "bad arguments");
  cudaError_t err = cudaSuccess;
  zd* A = c->ws.get<zd>("db_A", (size_t)dimse * std::max(dimse1, 1), &err);
  zd* h1 = c->ws.get<zd>("db_h1", dimse, &err);
  zd* h2 = c->ws.get<zd>("db_h2", dimse, &err);
  double* act = c->ws.get<double>("db_act", dimse, &err, true);
  CKC(err);
  CKC(cudaMemcpyAsync(A, excitonvec, sizeof(zd) * dimse * dimse1, cudaMemcpyHostToDevice, c->s));
  CKC(cudaMemcpyAsync(h1, hopt1, sizeof(zd) * dimse, cudaMemcpyHostToDevice, c->s));
  if (pair) CKC(cudaMemcpyAsync(h2, hopt2, sizeof(zd) * dimse, cudaMemcpyHostToDevice, c->s));
  if (dimse1 > 0) {
    dielbse_kernel<<<dimse1, 256, 0, c->s>>>(A, dimse, h1, h2, pair, act); ++g_launch_count;
    CKC(cudaGetLastError());
  }
  CKC(cudaMemcpyAsync(activity, act, sizeof(double) * dimse, cudaMemcpyDeviceToHost, c->s));
  return check_status(c);
}

int wtb_bsesolver(wtb_ctx* c, const wtb_bse_params* p, double* Ws, double* acts, double* HE, wtb_timings* t) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!c->have_hr) return set_err(c, WTB_ESTATE, "H(R) not set (call wtb_set_hr first)");
  CKR(validate_params(c, p));
  if (p->nv + p->nc > c->w) return set_err(c, WTB_EBADARG, "nv + nc exceeds w90basis");
  const long dim = (long)p->ngrid[0] * p->ngrid[1] * p->ngrid[2] * p->nc * p->nv;
  if (p->nev < 1 || p->nev > dim) return set_err(c, WTB_EBADARG, "nev must be between 1 and the BSE dimension");
  cudaEvent_t e0, e1, e2;
  CKC(cudaEventCreate(&e0));
  CKC(cudaEventCreate(&e1));
  CKC(cudaEventCreate(&e2));
  CKC(cudaEventRecord(e0, c->s));
  CKR(ensure_bands_for(c, p));
  CKR(compute_optics(c, p));
  CKC(cudaEventRecord(e1, c->s));
  std::vector<double> E;
  SolveStats stats;
  wtb_timings tt{};
  CKR(run_solve(c, p, &E, &tt, &stats));
  cudaError_t err = cudaSuccess;
  const int nev = p->nev;
  double* osc = c->ws.get<double>("osc", (size_t)8 * nev, &err);
  double* part = c->ws.get<double>("osc_part", (size_t)((dim + 255) / 256) * nev * 10, &err);
  CKC(err);
  cudaEvent_t e3;
  CKC(cudaEventCreate(&e3));
  CKC(cudaEventRecord(e3, c->s));
  CKC(launch_oscillators(c->ws.get<zd>("Xout", 0, &err), nev, nev, (int)dim, c->ws.get<zd>("hrvel", 0, &err), osc, part,
                         (int)((dim + 255) / 256), c->s));
  if (acts) {
    double* dacts = c->ws.get<double>("acts", (size_t)dim * 8, &err);
    CKC(err);
    expand_acts_kernel<<<(unsigned)((dim * 8 + 255) / 256), 256, 0, c->s>>>(osc, nev, (int)dim, dacts); ++g_launch_count;
    CKC(cudaMemcpyAsync(acts, dacts, sizeof(double) * dim * 8, cudaMemcpyDeviceToHost, c->s));
  }
  if (HE) {
    zd* staging = c->ws.get<zd>("HEout", (size_t)dim * nev, &err);
    CKC(err);
    transpose_z_kernel<<<(unsigned)((dim * nev + 255) / 256), 256, 0, c->s>>>(c->ws.get<zd>("Xout", 0, &err), (int)dim,
                                                                            nev, nev, staging, 0); ++g_launch_count;
    CKC(cudaMemcpyAsync(HE, staging, sizeof(zd) * dim * nev, cudaMemcpyDeviceToHost, c->s));
  }
  CKC(cudaEventRecord(e2, c->s));
  CKC(cudaEventSynchronize(e2));
  if (Ws) {
    for (long i = 0; i < dim; ++i) Ws[i] = 0.0;
    for (int i = 0; i < nev; ++i) Ws[i] = E[i];
  }
  c->have_solve = true;
  c->last_p = *p;
  c->last_E = E;
  if (t) {
    float a = 0, b = 0, d = 0;
    cudaEventElapsedTime(&a, e0, e1);
    cudaEventElapsedTime(&b, e0, e2);
    cudaEventElapsedTime(&d, e3, e2);
    *t = tt;
    t->t_bands_ms = a;
    t->t_optics_ms = d;
    t->t_total_ms = b;
    t->iterations = stats.iterations;
    t->matvec_columns = (int)stats.matvec_columns;
    t->max_rel_residual = stats.max_rel_residual;
    t->refine_shift_max = stats.refine_shift_max;
    t->kernel_launches = (int)g_launch_count.load();
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  cudaEventDestroy(e3);
  return check_status(c);
}

// optdiel over ncomp activity columns, then imagrenorm and the spin factor: bsedielraw, bsedielrawpol,
// spdielraw and spdielrawpol differ only in their columns and in which of them carry rtype 1.
static int dielraw(wtb_ctx* c, const wtb_bse_params* p, int dimse, const double* Ws, const double* acts, int ncomp,
                   unsigned delta_mask, double* dielf) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!c->have_hr) return set_err(c, WTB_ESTATE, "lattice not set (call wtb_set_hr first)");
  if (!p || dimse < 1 || !Ws || !acts || !dielf || p->numbse < 2) return set_err(c, WTB_EBADARG, "bad arguments");
  cudaError_t err = cudaSuccess;
  const size_t plen = spectrum_partial_len(dimse, p->numbse, ncomp);
  double* dW = c->ws.get<double>("sp_W", dimse, &err);
  double* df = c->ws.get<double>("sp_f", (size_t)ncomp * dimse, &err);
  double* dd = c->ws.get<double>("sp_d", (size_t)3 * ncomp * p->numbse, &err);
  double* dp = c->ws.get<double>("sp_p", plen, &err);
  CKC(err);
  CKC(cudaMemcpyAsync(dW, Ws, sizeof(double) * dimse, cudaMemcpyHostToDevice, c->s));
  CKC(cudaMemcpyAsync(df, acts, sizeof(double) * ncomp * dimse, cudaMemcpyHostToDevice, c->s));
  const int ng = p->ngrid[0] * p->ngrid[1] * p->ngrid[2];
  CKC(launch_spectrum(dW, dimse, df, ncomp, delta_mask, p->cshift, vcell3D(c->rlat_rm), ng, p->ebse0, p->ebsef,
                      p->numbse, p->renorm, c->systype_np ? 2.0 : 1.0, dd, dp, plen, c->s));
  CKC(cudaMemcpyAsync(dielf, dd, sizeof(double) * 3 * ncomp * p->numbse, cudaMemcpyDeviceToHost, c->s));
  return check_status(c);
}

int wtb_bsedielraw(wtb_ctx* c, const wtb_bse_params* p, int dimse, const double* Ws, const double* acts,
                   double* dielf) {
  return dielraw(c, p, dimse, Ws, acts, 6, 0x7u, dielf);  // xx yy zz rtype 1; xy xz yz rtype 0
}

int wtb_bsedielrawpol(wtb_ctx* c, const wtb_bse_params* p, int dimse, const double* Ws, const double* acts,
                      double* dielf) {
  return dielraw(c, p, dimse, Ws, acts, 5, 0x1Fu, dielf);  // xx yy zz sp sm, all rtype 1
}

int wtb_spdielraw(wtb_ctx* c, const wtb_bse_params* p, int dimsp, const double* esp, const double* acts,
                  double* dielf) {
  return dielraw(c, p, dimsp, esp, acts, 6, 0x7u, dielf);
}

int wtb_spdielrawpol(wtb_ctx* c, const wtb_bse_params* p, int dimsp, const double* esp, const double* acts,
                     double* dielf) {
  return dielraw(c, p, dimsp, esp, acts, 5, 0x1Fu, dielf);
}

static int optprop(wtb_ctx* c, int numbse, const double* dielf, int ncomp, double* props) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (numbse < 1 || !dielf || !props) return set_err(c, WTB_EBADARG, "bad arguments");
  cudaError_t err = cudaSuccess;
  double* dd = c->ws.get<double>("op_d", (size_t)3 * ncomp * numbse, &err);
  double* dp = c->ws.get<double>("op_p", (size_t)5 * ncomp * numbse, &err);
  CKC(err);
  CKC(cudaMemcpyAsync(dd, dielf, sizeof(double) * 3 * ncomp * numbse, cudaMemcpyHostToDevice, c->s));
  CKC(launch_optprops(dd, numbse, ncomp, dp, c->s));
  CKC(cudaMemcpyAsync(props, dp, sizeof(double) * 5 * ncomp * numbse, cudaMemcpyDeviceToHost, c->s));
  return check_status(c);
}

int wtb_bseoptprop(wtb_ctx* c, int numbse, const double* dielf, double* props) {
  return optprop(c, numbse, dielf, 6, props);
}

int wtb_bseoptproppol(wtb_ctx* c, int numbse, const double* dielf, double* props) {
  return optprop(c, numbse, dielf, 5, props);
}

static double temp_gap_correction(const wtb_temp_params* tp);

// spoptics' records, or with tp the records bsesolvertemp writes (bands with scs + tcor, activities weighted by
// f_v - f_c).
static int spoptics_impl(wtb_ctx* c, const wtb_bse_params* p, const wtb_temp_params* tp, float* rec) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!c->have_hr) return set_err(c, WTB_ESTATE, "H(R) not set (call wtb_set_hr first)");
  if (!p || !rec) return set_err(c, WTB_EBADARG, "bad arguments");
  if (p->ngrid[0] < 1 || p->ngrid[1] < 1 || p->ngrid[2] < 1) return set_err(c, WTB_EBADARG, "ngrid must be >= 1");
  if (p->nc < 1 || p->nv < 1) return set_err(c, WTB_EBADARG, "nc and nv must be >= 1");
  if (p->nv + p->nc > c->w) return set_err(c, WTB_EBADARG, "nv + nc exceeds w90basis");
  if (p->precision < 0 || p->precision > 3 || p->op < 0 || p->op > 1)
    return set_err(c, WTB_EBADARG, "unknown precision or operator mode");
  const long dim = (long)p->ngrid[0] * p->ngrid[1] * p->ngrid[2] * p->nc * p->nv;
  if (dim > (1L << 30) / 15) return set_err(c, WTB_EBADARG, "too many transitions");
  if (tp && (tp->ta < 0 || tp->ta > 2 || !(tp->temp >= 0.0))) return set_err(c, WTB_EBADARG, "bad temperature keys");
  CKR(stage_mesh(c, p));
  const double scs0 = c->scs;
  c->scs = scs0 + (tp ? temp_gap_correction(tp) : 0.0);
  const int rb = enqueue_bands(c, reduced_form(p));
  c->scs = scs0;
  CKR(rb);
  CKR(check_status(c));
  CKR(compute_optics(c, p));
  cudaError_t err = cudaSuccess;
  double* f = nullptr;
  if (tp) {
    f = c->ws.get<double>("spo_f", dim, &err);
    CKC(err);
    CKC(launch_fermi_weights(c->ws.get<double>("eig_win", 0, &err), c->nk, c->nv, c->nc, tp->temp, f, c->s));
  }
  float* raw = c->ws.get<float>("spo_raw", (size_t)15 * dim, &err);
  float* out = c->ws.get<float>("spo_out", (size_t)15 * dim, &err);
  float* key = c->ws.get<float>("spo_key", dim, &err);
  int* rank = c->ws.get<int>("spo_rank", dim, &err);
  CKC(err);
  CKC(launch_sp_records(c->ws.get<double>("kpt", 0, &err), c->ws.get<int>("nocp", 0, &err),
                        c->ws.get<double>("eig_win", 0, &err), c->ws.get<zd>("hrvel", 0, &err), c->nk, c->nv, c->nc,
                        f, raw, key, rank, out, c->s));
  CKC(cudaMemcpyAsync(rec, out, sizeof(float) * 15 * dim, cudaMemcpyDeviceToHost, c->s));
  return check_status(c);
}

int wtb_spoptics(wtb_ctx* c, const wtb_bse_params* p, float* rec) { return spoptics_impl(c, p, nullptr, rec); }

int wtb_spoptpolbz(wtb_ctx* c, const wtb_bse_params* p, double* act) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!c->have_hr) return set_err(c, WTB_ESTATE, "H(R) not set (call wtb_set_hr first)");
  if (!p || !act) return set_err(c, WTB_EBADARG, "bad arguments");
  if (p->ngrid[0] < 1 || p->ngrid[1] < 1 || p->ngrid[2] < 1) return set_err(c, WTB_EBADARG, "ngrid must be >= 1");
  if (p->nc < 1 || p->nv < 1) return set_err(c, WTB_EBADARG, "nc and nv must be >= 1");
  if (p->nv + p->nc > c->w) return set_err(c, WTB_EBADARG, "nv + nc exceeds w90basis");
  CKR(stage_mesh(c, p));
  CKR(enqueue_bands(c, false));
  CKR(check_status(c));
  const int nk = c->nk;
  const long dim = (long)nk * c->nc * c->nv;
  cudaError_t err = cudaSuccess;
  zd* hraw = c->ws.get<zd>("hrraw", (size_t)5 * dim, &err);
  double* dact = c->ws.get<double>("bz_act", (size_t)6 * nk, &err);
  CKC(err);
  CKC(launch_optics(c->ws.get<zd>("hr", 0, &err), c->ws.get<int>("rvec", 0, &err), c->ws.get<int>("ndegen", 0, &err),
                    c->nR, c->w, c->ws.get<double>("rlat", 0, &err), c->ws.get<double>("kpt", 0, &err), nk, c->nv,
                    c->nc, c->ws.get<double>("eig_win", 0, &err), c->ws.get<zd>("vec_win", 0, &err), p->cshift, hraw,
                    c->s, nullptr, true));
  CKC(launch_bz_activity(hraw, c->ws.get<double>("eig_win", 0, &err), c->ws.get<int>("nocp", 0, &err), nk, c->nv,
                         c->nc, p->cshift, dact, c->st, c->s));
  CKC(cudaMemcpyAsync(act, dact, sizeof(double) * 6 * nk, cudaMemcpyDeviceToHost, c->s));
  return check_status(c);
}

int wtb_spoptics_temp(wtb_ctx* c, const wtb_bse_params* p, const wtb_temp_params* tp, float* rec) {
  if (!tp) return set_err(c, WTB_EBADARG, "temperature keys are NULL");
  return spoptics_impl(c, p, tp, rec);
}

int wtb_bse_matvec(wtb_ctx* c, const wtb_bse_params* p, int ncol, const double* X, double* Y) {
  if (!c) return WTB_EBADARG;
  CKR(prep_device(c));
  if (!c->have_bands) return set_err(c, WTB_ESTATE, "no bands (call wtb_eigsys_mesh or wtb_bsesolver first)");
  if (!p || ncol < 1 || ncol > 32 || !X || !Y) return set_err(c, WTB_EBADARG, "bad arguments (1 <= ncol <= 32)");
  if (p->precision < 0 || p->precision > 3 || p->op < 0 || p->op > 1)
    return set_err(c, WTB_EBADARG, "unknown precision or operator mode");
  if (p->op == WTB_OP_DENSE && p->precision >= WTB_PREC_BF16X3)
    return set_err(c, WTB_EBADARG, "split-BF16 precision is available for the matrix-free operator only");
  if (!(p->ktol > 0.0)) return set_err(c, WTB_EBADARG, "KTOL must be > 0");
  const int dim = c->nk * c->nc * c->nv;
  cudaError_t err = cudaSuccess;
  zd* xc = c->ws.get<zd>("mv_xc", (size_t)dim * ncol, &err);
  zd* x64 = c->ws.get<zd>("mv_x64", (size_t)dim * ncol, &err);
  zd* y64 = c->ws.get<zd>("mv_y64", (size_t)dim * ncol, &err);
  zf* x32 = c->ws.get<zf>("mv_x32", (size_t)dim * ncol, &err);
  zf* y32 = c->ws.get<zf>("mv_y32", (size_t)dim * ncol, &err);
  CKC(err);
  OpBundle ob;
  CKR(make_operator(c, p, std::min(ncol, 16), &ob));
  // a single application: the operator's accurate accumulation, as in the eigensolver's final step
  if (ob.o64) ob.o64->set_final(true);
  if (ob.o32) ob.o32->set_final(true);
  CKC(cudaMemcpyAsync(xc, X, sizeof(zd) * dim * ncol, cudaMemcpyHostToDevice, c->s));
  const unsigned nbk = (unsigned)(((long)dim * ncol + 255) / 256);
  // column-major X (dim x ncol) seen as row-major X^T (ncol x dim) -> row-major X
  transpose_z_kernel<<<nbk, 256, 0, c->s>>>(xc, ncol, dim, dim, x64, 0); ++g_launch_count;
  if (ob.o64) {
    CKC(ob.o64->apply(x64, ncol, 0, ncol, y64, ncol, c->s));
  } else {
    CKC((launch_convert_cols<double, float>(x64, ncol, x32, ncol, ncol, dim, c->s)));
    CKC(ob.o32->apply(x32, ncol, 0, ncol, y32, ncol, c->s));
    CKC((launch_convert_cols<float, double>(y32, ncol, y64, ncol, ncol, dim, c->s)));
  }
  transpose_z_kernel<<<nbk, 256, 0, c->s>>>(y64, dim, ncol, ncol, xc, 0); ++g_launch_count;
  CKC(cudaGetLastError());
  CKC(cudaMemcpyAsync(Y, xc, sizeof(zd) * dim * ncol, cudaMemcpyDeviceToHost, c->s));
  return check_status(c);
}

long long wtb_kernel_launch_count(void) { return g_launch_count.load(); }

int wtb_operator_form(const wtb_ctx* ctx) { return ctx ? ctx->last_form : WTB_FORM_NONE; }

int wtb_autotune_report(char* buf, int len) {
  const std::string r = tune_report();
  if (buf && len > 0) {
    const size_t n = std::min((size_t)len - 1, r.size());
    std::memcpy(buf, r.data(), n);
    buf[n] = '\0';
  }
  return (int)r.size();
}

void* wtb_ctx_stream(wtb_ctx* c) { return c ? (void*)c->s : nullptr; }

int wtb_profile_enable(wtb_ctx* c, int on) {
  if (!c) return WTB_EBADARG;
  c->prof.reset();
  c->prof.on = on != 0;
  return WTB_OK;
}

int wtb_profile_read(wtb_ctx* c, double* total_ms, long long* launches, double* flops, double* bytes) {
  if (!c) return WTB_EBADARG;
  c->prof.flush();
  if (total_ms) *total_ms = c->prof.total_ms;
  if (launches) *launches = c->prof.launches;
  if (flops) *flops = c->prof.flops;
  if (bytes) *bytes = c->prof.bytes;
  return WTB_OK;
}

}  // extern "C"

namespace wtb {
// Batch solves (batch.cu): the host part of one system's set-up (validation, mesh, k-points to the device)
// and its device part as kernel launches only (bands, optical matrix elements, operator), which a graph
// can hold.
int ctx_stage_system(wtb_ctx* c, const wtb_bse_params* p) {
  CKR(prep_device(c));
  if (!c->have_hr) return set_err(c, WTB_ESTATE, "H(R) not set (call wtb_set_hr first)");
  CKR(validate_params(c, p));
  if (p->nv + p->nc > c->w) return set_err(c, WTB_EBADARG, "nv + nc exceeds w90basis");
  const long dim = (long)p->ngrid[0] * p->ngrid[1] * p->ngrid[2] * p->nc * p->nv;
  if (p->nev < 1 || p->nev > dim) return set_err(c, WTB_EBADARG, "nev must be between 1 and the BSE dimension");
  return stage_mesh(c, p);
}

int ctx_enqueue_system(wtb_ctx* c, const wtb_bse_params* p, int nbmax, OpBundle* ob) {
  CKR(enqueue_bands(c, reduced_form(p)));
  CKR(compute_optics(c, p));
  return make_operator(c, p, nbmax, ob, "", false, false);
}

int ctx_auto_block(const wtb_bse_params* p, int dim, bool fp64) { return auto_block(p, dim, fp64); }
}  // namespace wtb
