// Internal declarations shared by the CUDA translation units of libwtb_gb300.
//
// Device-side data layout (all row-major, 0-based):
//   H(R)        hr[iR][m][n]            cplx<double>
//   bands       eig[k][s], vec[k][s][o] s = band slot (nv valence then nc conduction), o = orbital
//   basis       I = k*nc*nv + c*nv + v  (quantumnumbers2, src/module_math.F90:352-379)
//   block vecs  X[I][j], leading dimension ld (columns of a block are contiguous per row)
//   dense H     H[I][J] row-major; Hermitian, so its column-major image is conj(H)
//   V table     V[k][k'] real, padded rows/cols for the tensor-core GEMM
#pragma once
#include <atomic>
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/wtb_gpu.h"

namespace wtb {

template <class S>
struct __align__(2 * sizeof(S)) cplx {
  S re, im;
};

template <class S>
__host__ __device__ __forceinline__ cplx<S> mk(S r, S i) {
  cplx<S> z;
  z.re = r;
  z.im = i;
  return z;
}
template <class S>
__host__ __device__ __forceinline__ cplx<S> cadd(cplx<S> a, cplx<S> b) { return mk<S>(a.re + b.re, a.im + b.im); }
template <class S>
__host__ __device__ __forceinline__ cplx<S> csub(cplx<S> a, cplx<S> b) { return mk<S>(a.re - b.re, a.im - b.im); }
template <class S>
__host__ __device__ __forceinline__ cplx<S> cmul(cplx<S> a, cplx<S> b) {
  return mk<S>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
// conj(a) * b
template <class S>
__host__ __device__ __forceinline__ cplx<S> cmulc(cplx<S> a, cplx<S> b) {
  return mk<S>(a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re);
}
template <class S>
__host__ __device__ __forceinline__ cplx<S> cconj(cplx<S> a) { return mk<S>(a.re, -a.im); }
template <class S>
__host__ __device__ __forceinline__ cplx<S> cscale(cplx<S> a, S s) { return mk<S>(a.re * s, a.im * s); }
// acc += a*b
template <class S>
__host__ __device__ __forceinline__ void cfma(cplx<S>& acc, cplx<S> a, cplx<S> b) {
  acc.re = fma(a.re, b.re, acc.re);
  acc.re = fma(-a.im, b.im, acc.re);
  acc.im = fma(a.re, b.im, acc.im);
  acc.im = fma(a.im, b.re, acc.im);
}
// acc += conj(a)*b
template <class S>
__host__ __device__ __forceinline__ void cfmac(cplx<S>& acc, cplx<S> a, cplx<S> b) {
  acc.re = fma(a.re, b.re, acc.re);
  acc.re = fma(a.im, b.im, acc.re);
  acc.im = fma(a.re, b.im, acc.im);
  acc.im = fma(-a.im, b.re, acc.im);
}

typedef cplx<double> zd;
typedef cplx<float> zf;

// Device error word: the first failing kernel stores its code and an index.
struct DevStatus {
  int code;
  int info;
  int pad[2];
};

__device__ __forceinline__ void dev_fail(DevStatus* st, int code, int info) {
  if (atomicCAS(&st->code, 0, code) == 0) st->info = info;
}

// Coulomb potential selector (coultype in module_coulomb, src/module_bse.F90:49-72).
enum CoulType { CT_V2DK = 0, CT_V3D, CT_V3DL, CT_V2DT, CT_V2DT2, CT_V2DOH, CT_V2DRK, CT_V1DT, CT_V0DT };

struct CoulParams {
  int type;
  int ngrid[3];
  double ktol, ediel[3], ez, w, r0, lc;
  double rlat[9];  // row-major rlat[i][j] = component j of a_(i+1)
  int deriv_r0;    // 1: the table holds dV/dr0 (R_0 key) instead of V
};

// ----------------------------------------------------------------------------- kernels (launchers)
// H(k) + Hermitian eigensolve + gauge + band window.  Returns 0 or a launch error.
cudaError_t launch_hk_eig(const zd* hr, const int* rvec, const int* ndegen, int nR, int w,
                          const double* rlat_rm, double efermi, double scs, const double* kpt, int nk,
                          int nv, int nc, double* eig_all, zd* vec_all, double* eig_win, zd* vec_win,
                          int* nocp, DevStatus* st, cudaStream_t s);
// Velocity matrix elements hr[5][dim] (x, y, z, sigma+, sigma-).
cudaError_t launch_optics(const zd* hr, const int* rvec, const int* ndegen, int nR, int w,
                          const double* rlat_rm, const double* kpt, int nk, int nv, int nc,
                          const double* eig_win, const zd* vec_win, double cshift, zd* hout, cudaStream_t s);
// V(k,k') table, double, leading dimension ldv (>= nk), zero padding left as is.
cudaError_t launch_coulomb(const CoulParams& p, const double* kpt1, int n1, const double* kpt2, int n2,
                           double* V, int ldv, cudaStream_t s);
// The same table on a Monkhorst-Pack mesh from the reciprocal vectors bl (3 x 3 row-major), through the
// (2n1-1)(2n2-1)(2n3-1) distinct values of k - k' (stencil scratch of that size).
cudaError_t launch_coulomb_mesh(const CoulParams& p, const double* bl, double* stencil, double* V, int ldv,
                                cudaStream_t s);
// Transition energies dE[I] = E_c - E_v.
cudaError_t launch_transition_energies(const double* eig_win, int nk, int nv, int nc, double* dE, cudaStream_t s);

// Dense build: H[I][J] (row-major, ld = dim) = delta_IJ dE_I + V(k_I,k_J) <c_I|c_J> <v_I|v_J>.
template <class S>
cudaError_t launch_bse_build(const zd* vec_win, const double* dE, const double* V, int ldv, int nk, int nv,
                             int nc, int w, cplx<S>* H, cudaStream_t s);
template <class S>
cudaError_t launch_dense_mv(const cplx<S>* H, int dim, const cplx<S>* X, int ldx, cplx<S>* Y, int ldy, int ncol,
                            cudaStream_t s);

// ----------------------------------------------------------------------------- block linear algebra
template <class S>
cudaError_t launch_gram(const cplx<S>* A, int lda, int p, const cplx<S>* B, int ldb, int q, int nrow,
                        zd* out, double* partial, int npart, cudaStream_t s);
template <class S>
cudaError_t launch_update(const cplx<S>* Sx, int lds, int nin, const zd* C, int ldc, int nout, int nrow,
                          cplx<S>* Out, int ldo, double alpha, double beta, cudaStream_t s);
template <class S>
cudaError_t launch_residual(const cplx<S>* AX, int ldax, const cplx<S>* X, int ldx, const double* theta, int m,
                            int nrow, cplx<S>* R, int ldr, double* partial, int npart, double* norms2,
                            cudaStream_t s);
template <class S>
cudaError_t launch_precond(cplx<S>* R, int ldr, const double* diag, const double* theta, const int* active, int m,
                           int nrow, cudaStream_t s);
template <class S>
cudaError_t launch_copy_cols(const cplx<S>* A, int lda, cplx<S>* B, int ldb, int ncol, int nrow, cudaStream_t s);
template <class Sa, class Sb>
cudaError_t launch_convert_cols(const cplx<Sa>* A, int lda, cplx<Sb>* B, int ldb, int ncol, int nrow,
                                cudaStream_t s);
cudaError_t launch_small_gemm(const zd* A, int lda, int transA, const zd* B, int ldb, zd* C, int ldc, int m, int n,
                              int k, cudaStream_t s, bool fp32 = false);

// ----------------------------------------------------------------------------- matrix-free operator
// Z[n][k'] with n = ((b*w + o)*w + p)*2 + ri (K-major for the V*Z contraction).
template <class S, class Z>
cudaError_t launch_mf_gather(const cplx<S>* X, int ldx, int c0, int nb, const zd* vec_win, int nk, int nv, int nc,
                             int w, Z* zt, int ldk, int nslices, long slice_stride, cudaStream_t s);
template <class S, class T>
cudaError_t launch_mf_scatter(const T* Tm, int ldt, const cplx<S>* X, int ldx, const zd* vec_win, const double* dE,
                              int nk, int nv, int nc, int w, int nb, cplx<S>* Y, int ldy, int c0, cudaStream_t s);
template <class S>
cudaError_t launch_simt_gemm_tn(const S* A, int lda, const S* B, int ldb, S* C, int ldc, int M, int N, int K,
                                cudaStream_t s);
cudaError_t launch_split_bf16(const double* V, int ldv, int rows, int cols, uint16_t* out, int ldo, long slice_stride,
                              int nslices, cudaStream_t s);
cudaError_t launch_round_f32(const double* V, int ldv, int rows, int cols, float* out, int ldo, cudaStream_t s);

// tcgen05 split-bf16 GEMM: C[M][N] (fp32, ldc) = sum over slice pairs of A_sa[M][K] * B_sb[N][K]^T.
struct TcGemmPlan;
int tc_gemm_plan_create(TcGemmPlan** plan, const uint16_t* A, int M, int K, long a_slice_stride, int na_slices,
                        const uint16_t* B, int N, long b_slice_stride, int nb_slices, float* C, int ldc,
                        int npairs, const int* pair_a, const int* pair_b, std::string* msg);
cudaError_t tc_gemm_run(TcGemmPlan* plan, DevStatus* st, cudaStream_t s);
// the same product with K split into ranges of kb_chunk 64-wide blocks, summed in FP32 round-to-nearest
cudaError_t tc_gemm_run_split(TcGemmPlan* plan, DevStatus* st, cudaStream_t s, int kb_chunk);
void tc_gemm_plan_destroy(TcGemmPlan* plan);
int tc_gemm_available();

// ----------------------------------------------------------------------------- spectrum
cudaError_t launch_oscillators(const zd* A, int lda, int nev, int dim, const zd* hr, double* osc /*[8][nev]*/,
                               double* partial, int npart, cudaStream_t s);
// dielf in the Fortran layout dielf(nesp, 3, 6); props(nesp, 6, 5)
cudaError_t launch_spectrum(const double* Ws, int nrows, const double* f /*[6][nrows]*/, double sme, double vc,
                            int ng, double e0, double ef, int nesp, int renorm, double spinf, double* dielf,
                            double* partial, int npart, cudaStream_t s);
cudaError_t launch_optprops(const double* dielf, int nesp, double* props, cudaStream_t s);

// Raises (never lowers) a kernel's dynamic shared-memory limit on the current device.  Launchers run on
// several host threads at once (batch workers): setting the limit to each launch's own need would let one
// thread lower it under another thread's larger launch.
cudaError_t raise_smem_limit(const void* func, size_t bytes);

// Every launcher adds the number of kernels it started (reported as gpu_launches by the benchmark);
// atomic because batch workers drive several contexts from several host threads.
extern std::atomic<long long> g_launch_count;

}  // namespace wtb
