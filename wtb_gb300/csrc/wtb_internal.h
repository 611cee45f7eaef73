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
#include <functional>
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
// Relative residual target of the reduced-precision (FP32 and split-BF16) solves: 1e-5, just below the FP32
// iteration's rounding floor on the 57,600-dimensional workload (about 1.2e-5; the stagnation guard then ends the
// solve with the best block, at most 1.5 x the target after one iteration without progress).  Measured against
// the FP64 oracle on that workload (FP32 FFT form): targets 1e-5 / 2e-5 / 3e-5 took 11 / 10 / 9 iterations with
// exciton energies within 9.9e-8 / 9.0e-8 / 6.6e-8 eV and spectra within 3.2e-5 / 5.2e-5 / 7.2e-5 relative L2;
// but at 2e-5 the spectrum of the regenerated 60 x 60 system came out 1.2e-4 from the FP64 form's, over the
// 1e-4 bound, so the target stays at 1e-5.
constexpr double kReducedTol = 1e-5;

// n / d for 0 <= n < 2^21 and d >= 1, with rinv = 1.0f / d: (n + 1/2) / d lies at least 1 / (2 d) from an
// integer, and the two FP32 roundings move it by at most 2^-23 (n + 1/2) / d < 1 / (4 d), so truncation gives
// the quotient.  Two instructions instead of an integer division by a runtime divisor.
__device__ __forceinline__ int qdiv(int n, float rinv) { return __float2int_rz(((float)n + 0.5f) * rinv); }

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
// mixed: FP32 eigensolve + Rayleigh quotients against H(k) summed in double-float (energies FP64-accurate,
// vectors FP32-accurate); hr_df: scratch of nR (w^2 + 2) float4 for the split H(R) and the
// per-R phase factors (mixed only)
cudaError_t launch_hk_eig(const zd* hr, const int* rvec, const int* ndegen, int nR, int w,
                          const double* rlat_rm, double efermi, double scs, const double* kpt, int nk,
                          int nv, int nc, double* eig_all, zd* vec_all, double* eig_win, zd* vec_win,
                          int* nocp, DevStatus* st, cudaStream_t s, bool mixed = false, float4* hr_df = nullptr);
// Velocity matrix elements hr[5][dim] (x, y, z, sigma+, sigma-); with hr32 (an FP32 copy of H(R)) the Fourier
// sums run in FP32.
cudaError_t launch_optics(const zd* hr, const int* rvec, const int* ndegen, int nR, int w,
                          const double* rlat_rm, const double* kpt, int nk, int nv, int nc,
                          const double* eig_win, const zd* vec_win, double cshift, zd* hout, cudaStream_t s,
                          const zf* hr32 = nullptr, bool raw = false);
// BZ-resolved optical activity of spoptpolbz: per k-point the sums over the window's transitions of
// |<c|dH/dk_a|v>/(E_c - E_v + i sme)|^2 for x y z and the circular sp sm, and the dichroism (sp-sm)/(sp+sm):
// act(nk, 6), from the unscaled matrix elements hraw[3][dim] of launch_optics(raw).
cudaError_t launch_bz_activity(const zd* hraw, const double* eig_win, const int* nocp, int nk, int nv, int nc,
                               double sme, double* act, DevStatus* st, cudaStream_t s);
// V(k,k') table, double, leading dimension ldv (>= nk), zero padding left as is.
cudaError_t launch_coulomb(const CoulParams& p, const double* kpt1, int n1, const double* kpt2, int n2,
                           double* V, int ldv, cudaStream_t s);
// The same table on a Monkhorst-Pack mesh from the reciprocal vectors bl (3 x 3 row-major), through the
// (2n1-1)(2n2-1)(2n3-1) distinct values of k - k' (stencil scratch of that size).
// the stencil s of a mesh alone: s[(di + n1 - 1) (2 n2 - 1) (2 n3 - 1) + ...] = V at the index difference
cudaError_t launch_coulomb_stencil(const CoulParams& p, const double* bl, double* stencil, cudaStream_t s);
// FFT form of the contraction on a two-dimensional mesh (k_fftconv.cu): the transform size P (32, 64 or 128)
// for an n1 x n2 mesh, or 0 when the mesh is too large; the stencil's spectrum (work: (2 n1 - 1) P complex
// doubles; spec: fft_spec_size(P) complex (the P x P spectrum, its real parts and the stencil's evenness flag);
// tw: 128 twiddles); (V Z) for the npairs column pairs of Z (column n at Z + n ldz,
// k' = i n2 + j) into T: t_kn ? T[k][2q + (0, 1)] (row k at T + k ldt) : T[2q + (0, 1)][k] (Z's layout)
int fft_conv_size(int n1, int n2);
inline size_t fft_spec_size(int P) { return (size_t)P * P + (size_t)P * P / 2 + 1; }
cudaError_t launch_fft_spectrum(const double* stencil, int n1, int n2, int P, zd* work, float2* spec, float2* tw,
                                cudaStream_t s);
cudaError_t launch_fft_conv(const float* Z, int ldz, int npairs, int n1, int n2, int P, const float2* spec,
                            const float2* tw, float* T, int ldt, bool t_kn, cudaStream_t s);
cudaError_t launch_coulomb_mesh(const CoulParams& p, const double* bl, double* stencil, double* V, int ldv,
                                cudaStream_t s);
// Transition energies dE[I] = E_c - E_v.
cudaError_t launch_transition_energies(const double* eig_win, int nk, int nv, int nc, double* dE, cudaStream_t s);
// hlm at one k-point (out: 3 column-major w x w matrices), or with band vectors cv, vv the optsp elements (out: 3)
cudaError_t launch_hlm(const zd* hr, const int* rvec, const int* ndegen, int nR, int w, const double* rlat_rm, double kx,
                       double ky, double kz, const zd* cv, const zd* vv, double ev, double ec, double sme, zd* out,
                       cudaStream_t s);
// optdiel at one photon energy: out = (rpart, ipart); caux = 180.90 / (real(ngrid product) * vc)
cudaError_t launch_optdiel(int rtype, double caux, int dimse, double elux, const double* E, const double* f, double sme,
                           double* out, cudaStream_t s);

// Dense build: H[I][J] (row-major, ld = dim) = delta_IJ dE_I + V(k_I,k_J) <c_I|c_J> <v_I|v_J>.
template <class S>
cudaError_t launch_bse_build(const zd* vec_win, const double* dE, const double* V, int ldv, int nk, int nv,
                             int nc, int w, cplx<S>* H, cudaStream_t s);
template <class S>
cudaError_t launch_dense_mv(const cplx<S>* H, int dim, const cplx<S>* X, int ldx, cplx<S>* Y, int ldy, int ncol,
                            cudaStream_t s);

// ----------------------------------------------------------------------------- ragged batches
// Independent eigenproblems solved together share one concatenated row space: system q owns rows
// [rows[q].x, rows[q].x + rows[q].y), followed by zero rows up to a multiple of kTileRows, and row tile t
// (kTileRows rows) belongs to system tile_sys[t].  Reductions over rows run in parts that never straddle two
// systems: part p covers rows [parts[p].x, parts[p].y) of system part_sys[p], and system q owns parts
// [sys_parts[q].x, sys_parts[q].x + sys_parts[q].y).  frozen[q] != 0: system q has left the iteration, whose
// kernels then leave its rows and small matrices alone.  The default map is one system whose parts are
// npart equal row ranges.  Small per-system matrices sit at a fixed stride from system to system.
constexpr int kTileRows = 32;
constexpr int kSelSlices = 8;  // first-level slices per system of the batched start-vector selection
struct BatchMap {
  int nsys = 1;
  int nparts = 0;
  const int* tile_sys = nullptr;
  const int2* rows = nullptr;
  const int2* parts = nullptr;
  const int* part_sys = nullptr;
  const int2* sys_parts = nullptr;
  const int* frozen = nullptr;
};

__device__ __forceinline__ int bm_sys_of_row(const BatchMap& bm, long r) {
  return bm.tile_sys ? bm.tile_sys[r / kTileRows] : 0;
}
__device__ __forceinline__ bool bm_frozen(const BatchMap& bm, int q) { return bm.frozen && bm.frozen[q] != 0; }
// Sum over the reduction parts of system sys of partial[b][e] for the e of this lane (lane = e - e0, e < n): the
// CTA's 8 warps take every 8th part, in rounds of up to 16 loads issued together (no serial remainder) with the
// additions in part order, then warp 0 adds the 8 warp sums in a fixed order.  All 256 threads call it; the result
// is valid on warp 0's lanes with e < n.  red: 8 x 33 doubles of shared memory.
__device__ __forceinline__ double sum_parts_cta(const double* __restrict__ partial, int npart, int n, int e, int sys,
                                                const BatchMap& bm, double (*red)[33]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int b0 = 0, nbp = npart;
  if (bm.sys_parts) {
    b0 = bm.sys_parts[sys].x;
    nbp = bm.sys_parts[sys].y;
  }
  constexpr int kDeep = 16;
  double s = 0.0;
  if (e < n) {
    for (int b = warp; b < nbp; b += 8 * kDeep) {
      double v[kDeep];
#pragma unroll
      for (int u = 0; u < kDeep; ++u) v[u] = b + 8 * u < nbp ? partial[(size_t)(b0 + b + 8 * u) * n + e] : 0.0;
#pragma unroll
      for (int u = 0; u < kDeep; ++u)
        if (b + 8 * u < nbp) s += v[u];
    }
  }
  red[warp][lane] = s;
  __syncthreads();
  double t = 0.0;
  if (warp == 0)
    for (int w = 0; w < 8; ++w) t += red[w][lane];
  return t;
}
// rows [*r0, *r1) and system of reduction part p (uniform parts of rpp rows when the map has no table)
__device__ __forceinline__ int bm_part(const BatchMap& bm, int p, long nrow, long rpp, long* r0, long* r1) {
  if (bm.parts) {
    const int2 pr = bm.parts[p];
    *r0 = pr.x;
    *r1 = pr.y;
    return bm.part_sys[p];
  }
  *r0 = (long)p * rpp;
  *r1 = *r0 + rpp < nrow ? *r0 + rpp : nrow;
  return 0;
}

// ----------------------------------------------------------------------------- block linear algebra
// Batched forms: bm describes the systems (default: one); out_stride, c_stride, ... are the per-system
// strides (in elements) of the small matrices.
template <class S>
cudaError_t launch_gram(const cplx<S>* A, int lda, int p, const cplx<S>* B, int ldb, int q, int nrow,
                        zd* out, double* partial, int npart, cudaStream_t s, const BatchMap& bm = BatchMap(),
                        long out_stride = 0);
// outM = A^H A and outG = A^H B in one pass over the rows (p <= 48 columns); partial holds 2 * npart p p doubles
template <class S>
cudaError_t launch_gram_pair(const cplx<S>* A, const cplx<S>* B, int ld, int p, int nrow, zd* outM, zd* outG,
                             double* partial, int npart, cudaStream_t s, const BatchMap& bm = BatchMap(),
                             long out_stride = 0);
// outM, outG: the sums over npart parts of the two partial sets [part][n] at partial and partial + npart n
cudaError_t launch_sum_partials_pair(const double* partial, int npart, int n, zd* outM, zd* outG, cudaStream_t s,
                                     const BatchMap& bm, long out_stride);
// the final Rayleigh-Ritz of the reduced forms (k_final.cu): M = A^H A and G = A^H B of FP32 blocks (p <= 32
// columns) summed with compensated FP32 arithmetic; and the small FP64 problem from M, G (n <= 32): theta (m
// lowest, ascending; 1e30 for a dropped direction) and C (n x m, leading dimension m), keep = kept directions
cudaError_t launch_gram_pair_dot2(const zf* A, const zf* B, int ld, int p, int nrow, zd* outM, zd* outG,
                                  double* partial, int npart, cudaStream_t s, const BatchMap& bm, long out_stride);
cudaError_t launch_small_rr(const zd* M, const zd* G, int n, int m, double drop, double* theta, zd* C, int* keep,
                            cudaStream_t s, const BatchMap& bm, long mat_stride, long theta_stride);
// Out = X C with FP32 X (nin <= 32 columns) and FP64 C, to FP64 accuracy in FP32 instructions
cudaError_t launch_update_dot2(const zf* X, int ldx, int nin, const zd* C, int ldc, int nout, int nrow, zd* Out,
                               int ldo, cudaStream_t s, const BatchMap& bm, long c_stride);
// W -= X T[:, 0:m], P -= X T[:, m:2m], AP -= AX T[:, m:2m] (T: m x 2m FP64, per system at t_stride); with active
// (flags of system q at active + 32 q) the W columns of inactive vectors are set to zero
template <class S>
cudaError_t launch_orth_update(const cplx<S>* X, const cplx<S>* AX, int ld, int m, const zd* T, cplx<S>* W,
                               cplx<S>* P, cplx<S>* AP, int nrow, cudaStream_t s, const BatchMap& bm = BatchMap(),
                               long t_stride = 0, const int* active = nullptr);
template <class S>
cudaError_t launch_update(const cplx<S>* Sx, int lds, int nin, const zd* C, int ldc, int nout, int nrow,
                          cplx<S>* Out, int ldo, double alpha, double beta, cudaStream_t s,
                          const BatchMap& bm = BatchMap(), long c_stride = 0);
// norms2 of system q at norms2 + 32 q (of AX - X theta; without sum_parts only the parts [npart][32] in partial,
// summed by the caller's next kernel); with diag, R receives the preconditioned residual
// |diag - theta|^-1 (AX - X theta), the denominator floored at 1e-2 max(|theta|, 1e-3)
template <class S>
cudaError_t launch_residual(const cplx<S>* AX, int ldax, const cplx<S>* X, int ldx, const double* theta, int m,
                            int nrow, cplx<S>* R, int ldr, double* partial, int npart, double* norms2,
                            cudaStream_t s, const BatchMap& bm = BatchMap(), long theta_stride = 0,
                            const double* diag = nullptr, bool sum_parts = true);
template <class S>
cudaError_t launch_copy_cols(const cplx<S>* A, int lda, cplx<S>* B, int ldb, int ncol, int nrow, cudaStream_t s);
template <class Sa, class Sb>
cudaError_t launch_convert_cols(const cplx<Sa>* A, int lda, cplx<Sb>* B, int ldb, int ncol, int nrow,
                                cudaStream_t s);
cudaError_t launch_small_gemm(const zd* A, int lda, int transA, const zd* B, int ldb, zd* C, int ldc, int m, int n,
                              int k, cudaStream_t s, bool fp32 = false, const BatchMap& bm = BatchMap(),
                              long a_stride = 0, long b_stride = 0, long c_stride = 0);

// ----------------------------------------------------------------------------- matrix-free operator
// Z[n][k'] with n = ((b*w + o)*w + p)*2 + ri (K-major for the V*Z contraction).  tile (split-BF16 panel and FP32
// rows): 0 = the shared-memory rule, else KT * 100 + nbp (KT = 16 or 8 k' per CTA, nbp block columns per chunk;
// FP32 rows also KT = 32: the gather with the warp's lanes along k').
template <class S, class Z>
cudaError_t launch_mf_gather(const cplx<S>* X, int ldx, int c0, int nb, const cplx<S>* vec_win, int nk, int nv, int nc,
                             int w, Z* zt, int ldk, int nslices, long slice_stride, cudaStream_t s, int tile = 0);
// scatter from T in Z's layout, T[n][k] (row n at Tt + n ldt; the FFT form), over tiles of 8 k-points and cols
// block columns per CTA (0: 4); cols = 100 + g: tiles of 32 k-points along the warp's lanes, g block columns
cudaError_t launch_mf_scatter_t(const float* Tt, int ldt, const zf* X, int ldx, const zf* vec_win, const float* dE,
                                int nk, int nv, int nc, int w, int nb, zf* Y, int ldy, int c0, cudaStream_t s,
                                int cols = 0);
// cols: block columns per CTA (0 = all that fit in 96 KB of shared memory)
template <class S, class T>
cudaError_t launch_mf_scatter(const T* Tm, int ldt, const cplx<S>* X, int ldx, const cplx<S>* vec_win, const S* dE,
                              int nk, int nv, int nc, int w, int nb, cplx<S>* Y, int ldy, int c0, cudaStream_t s,
                              int cols = 0);
template <class S>
cudaError_t launch_simt_gemm_tn(const S* A, int lda, const S* B, int ldb, S* C, int ldc, int M, int N, int K,
                                cudaStream_t s);
// The split-BF16 operator of one system of a batch (device array, one entry per system): its rows start at row0
// of the concatenated block vectors; Z panel zt (nslices x [Npad][ldk] bf16, slice_stride apart), contraction
// result Tm ([Mpad][ldt] fp32).
struct MfSys {
  long row0;
  int nk, nv, nc, w;
  int ldk, ldt;
  long slice_stride;
  const zd* vec_win;
  const double* dE;
  uint16_t* zt;
  const float* Tm;
};
// gather over tiles (system, first k-point of a tile of mf_gather_batch_tile() k-points), scatter over k-points
// (system, k)
int mf_gather_batch_tile(int max_nv, int max_nc, int w, int nb);
cudaError_t launch_mf_gather_batch(const zf* X, int ldx, int c0, int nb, const MfSys* sys, const int2* tiles,
                                   int ntiles, int max_nv, int max_nc, int w, int nslices, const int* frozen,
                                   cudaStream_t s);
cudaError_t launch_mf_scatter_batch(const zf* X, int ldx, const MfSys* sys, const int2* kpts, int nkpts, int max_nv,
                                    int max_nc, int w, int nb, zf* Y, int ldy, int c0, const int* frozen,
                                    cudaStream_t s);
cudaError_t launch_split_bf16(const double* V, int ldv, int rows, int cols, uint16_t* out, int ldo, long slice_stride,
                              int nslices, cudaStream_t s);
cudaError_t launch_round_f32(const double* V, int ldv, int rows, int cols, float* out, int ldo, cudaStream_t s);

// tcgen05 split-bf16 GEMM: C[M][N] (fp32, ldc) = sum over slice pairs of A_sa[M][K] * B_sb[N][K]^T, with A stored
// [slice][M][K] and B in 64-wide K blocks, [slice][K / 64][N][64].
struct TcGemmPlan;
// bn: column tile of the output (256 or 128)
int tc_gemm_plan_create(TcGemmPlan** plan, const uint16_t* A, int M, int K, long a_slice_stride, int na_slices,
                        const uint16_t* B, int N, long b_slice_stride, int nb_slices, float* C, int ldc,
                        int npairs, const int* pair_a, const int* pair_b, std::string* msg, int bn = 256);
cudaError_t tc_gemm_run(TcGemmPlan* plan, DevStatus* st, cudaStream_t s);
// the same product with K split into ranges of kb_chunk 64-wide blocks, summed in FP32 round-to-nearest
cudaError_t tc_gemm_run_split(TcGemmPlan* plan, DevStatus* st, cudaStream_t s, int kb_chunk);
void tc_gemm_plan_destroy(TcGemmPlan* plan);
int tc_gemm_available();
// A group of independent products of that kind (one per system of a batch) in one launch.  Products of
// systems with frozen[q] set are skipped (frozen may be null); npairs: slice products of this launch.
struct TcGroupDesc {
  const uint16_t* A;  // [nslices][M][K]
  const uint16_t* B;  // [nslices][K / 64][N][64]
  float* C;
  int M, N, K, ldc, m_valid, n_valid;
};
struct TcGroupPlan;
int tc_gemm_group_create(TcGroupPlan** plan, int n, const TcGroupDesc* descs, int nslices, int npairs,
                         const int* pair_a, const int* pair_b, std::string* msg, int bn = 256);
cudaError_t tc_gemm_group_run(TcGroupPlan* plan, int npairs, const int* frozen, DevStatus* st, cudaStream_t s);
cudaError_t tc_gemm_group_run_split(TcGroupPlan* plan, int npairs, const int* frozen, DevStatus* st, cudaStream_t s,
                                    int kb_chunk);
void tc_gemm_group_destroy(TcGroupPlan* plan);
// autotuner (autotune.cu): the fastest of cands for (shape, param), measured with run(candidate) on stream s the
// first time the pair is seen on this device and build (or read from the JSON cache); dflt while s is capturing
int tune_choice(const std::string& shape, const char* param, const std::vector<int>& cands, int dflt,
                const std::function<cudaError_t(int)>& run, cudaStream_t s);
// {"build": source hash, "cache": file or null, "choices": [{shape, param, choice, source, ms}, ...]} (JSON)
std::string tune_report();
std::string tune_cache_path();

// ----------------------------------------------------------------------------- spectrum
cudaError_t launch_oscillators(const zd* A, int lda, int nev, int dim, const zd* hr, double* osc /*[8][nev]*/,
                               double* partial, int npart, cudaStream_t s);
// The broadened spectrum of ncomp (5 or 6) activity columns f[ncomp][nrows]: dielf in the Fortran layout
// dielf(nesp, 3, ncomp); delta_mask bit c set = component c has optdiel's rtype 1 (eps1 offset 1).  partial
// holds spectrum_partial_len(nrows, nesp, ncomp) doubles.
size_t spectrum_partial_len(int nrows, int nesp, int ncomp);
cudaError_t launch_spectrum(const double* Ws, int nrows, const double* f, int ncomp, unsigned delta_mask, double sme,
                            double vc, int ng, double e0, double ef, int nesp, int renorm, double spinf,
                            double* dielf, double* partial, size_t partial_len, cudaStream_t s);
// props(nesp, ncomp, 5) from dielf(nesp, 3, ncomp)
cudaError_t launch_optprops(const double* dielf, int nesp, int ncomp, double* props, cudaStream_t s);
// The IPA transition records rec(dim, 15) (REAL(4), column-major) of the bands and velocity matrix elements
// hr[5][dim], stably sorted by transition energy into sorted; key(dim), rank(dim) and rec(dim, 15) are scratch.
// f (nullable): the activity columns weighted by f_v - f_c (the temperature solver's records).
cudaError_t launch_sp_records(const double* kpt, const int* nocp, const double* eig_win, const zd* hr, int nk, int nv,
                              int nc, const double* f, float* rec, float* key, int* rank, float* sorted,
                              cudaStream_t s);

// ----------------------------------------------------------------------------- finite-Q BSE
// Merged band window of the finite-Q basis: valence slots from the plain mesh, conduction slots from the
// Q-shifted mesh (eig (nk, nb), vec (nk, nb, w)).
cudaError_t launch_merge_windows(const double* eig_k, const zd* vec_k, const double* eig_q, const zd* vec_q, int nk,
                                 int nv, int nc, int w, double* eig_m, zd* vec_m, cudaStream_t s);
// Exchange term of matrizelbsekq on the row-major dense H: H -= V(Q,0) u u^H, u_i = <c_i|v_i> (u: dim scratch).
cudaError_t launch_exchange(const zd* vec_m, int nk, int nv, int nc, int w, const double* vq, zd* u, zd* H,
                            cudaStream_t s);

// ----------------------------------------------------------------------------- temperature BSE
// f[I] = f_v - f_c of transition I at temp (K) (fermidisteh).
cudaError_t launch_fermi_weights(const double* eig_win, int nk, int nv, int nc, double temp, double* f,
                                 cudaStream_t s);
// The row-major BSE matrix H (dim x dim, Q = 0 or finite Q) weighted in place as ZHEEV 'U' reads the upper
// triangle of matrizelbsetemp / matrizelbsekqtemp; dE the transition energies of H's diagonal.
cudaError_t launch_temp_weight(zd* H, long dim, const double* f, const double* dE, cudaStream_t s);
// dielbseptemp's eight activities acts(dim, 8) of the eigenvectors Z (row-major) and hr[5][dim].
cudaError_t launch_temp_acts(const zd* Z, int dim, const zd* hr, const double* f, int dtfull, int cpol, double* acts,
                             cudaStream_t s);

// ----------------------------------------------------------------------------- dense Hermitian eigenvalues
// All eigenvalues (ascending) of the n x n Hermitian A (column-major, leading dimension lda; destroyed: its
// strictly lower part ends holding the Householder vectors).  upper_only: only the upper triangle holds the
// matrix (ZHEEV 'U'); it is mirrored first.  scratch: dense_eig_scratch(n) bytes, 16-byte aligned.
constexpr int kDenseEigChunks = 16;
size_t dense_eig_scratch(int n);
cudaError_t launch_dense_eigvals(zd* A, int n, int lda, bool upper_only, double* W, void* scratch, cudaStream_t s);
// All eigenpairs: W ascending and Z(i, k) = Z[i * n + k] (row-major, complex) the eigenvector of W[k]; inverse
// iteration on the tridiagonal (clusters reorthogonalised) and the Householder back-transformation.  With
// conj_vectors the conjugates are returned (for A holding conj(H), e.g. a row-major H read column-major).
// vscratch: dense_eigvec_scratch(n) bytes.
size_t dense_eigvec_scratch(int n);
cudaError_t launch_dense_eig(zd* A, int n, int lda, bool upper_only, double* W, zd* Z, bool conj_vectors,
                             void* scratch, void* vscratch, cudaStream_t s);
// Sets the kernels' shared-memory limits ahead of a stream capture of launch_dense_eigvals.
cudaError_t dense_eig_prepare();

// Raises (never lowers) a kernel's dynamic shared-memory limit on the current device.  Launchers run on
// several host threads at once (batch workers): setting the limit to each launch's own need would let one
// thread lower it under another thread's larger launch.
cudaError_t raise_smem_limit(const void* func, size_t bytes);

// Every launcher adds the number of kernels it started (reported as gpu_launches by the benchmark);
// atomic because batch workers drive several contexts from several host threads.
extern std::atomic<long long> g_launch_count;

}  // namespace wtb
