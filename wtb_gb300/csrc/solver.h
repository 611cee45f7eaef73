// Lowest-exciton eigensolver (replaces SLEPc Krylov-Schur in slepc_solver,
// src/module_slepc_solver.F90:12-97) and the BSE operators it drives.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "wtb_internal.h"

namespace wtb {

// Device allocation with grow-only reuse.  Zeroing is ordered on the owner's stream: the legacy default
// stream has no ordering with the (non-blocking) context streams, so a cudaMemset there could land in the
// middle of later work on the context's stream.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t ensure(size_t n, bool zero, cudaStream_t s) {
    if (n <= bytes && p) {
      if (zero) return cudaMemsetAsync(p, 0, n, s);
      return cudaSuccess;
    }
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n ? n : 16);
    if (e != cudaSuccess) return e;
    bytes = n;
    if (zero) return cudaMemsetAsync(p, 0, n, s);
    return cudaSuccess;
  }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

// Named device buffers.  get() sets *err only when an allocation fails, so one check after a run of
// get() calls sees any failure in the run (callers start with err = cudaSuccess).
// The workspace also keeps the last eigensolver graph (instantiated), reused while its signature (sizes,
// parameters, operator configuration and every device address it was captured with) is unchanged.
struct Workspace {
  std::map<std::string, std::unique_ptr<DevBuf>> bufs;
  cudaStream_t stream = nullptr;  // the owner's stream (zeroing is ordered on it)
  uint64_t graph_key = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  long long graph_body_launches[2] = {0, 0};
  long long graph_launches = 0;  // kernels captured in the whole graph
  void drop_graph() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (graph) cudaGraphDestroy(graph);
    graph_exec = nullptr;
    graph = nullptr;
    graph_key = 0;
  }
  ~Workspace() { drop_graph(); }
  // incremented whenever a buffer is (re)allocated: a graph captured at one generation holds valid addresses
  // as long as the generation is unchanged
  uint64_t generation = 0;
  template <class T>
  T* get(const std::string& name, size_t count, cudaError_t* err, bool zero = false) {
    auto& b = bufs[name];
    if (!b) b.reset(new DevBuf());
    const void* before = b->p;
    const cudaError_t e = b->ensure(count * sizeof(T), zero, stream);
    if (e != cudaSuccess) *err = e;
    if (b->p != before) ++generation;
    return b->as<T>();
  }
  // an existing buffer of at least count elements, or nullptr
  template <class T>
  T* find(const std::string& name, size_t count) const {
    auto it = bufs.find(name);
    if (it == bufs.end() || !it->second || !it->second->p || it->second->bytes < count * sizeof(T)) return nullptr;
    return it->second->as<T>();
  }
};

template <class S>
struct Operator {
  virtual ~Operator() {}
  // Y[:, c0:c0+ncol] = H X[:, c0:c0+ncol]
  virtual cudaError_t apply(const cplx<S>* X, int ldx, int c0, int ncol, cplx<S>* Y, int ldy, cudaStream_t s) = 0;
  // switches the operator to its most accurate arithmetic; returns false if it has only one
  virtual bool begin_refine() { return false; }
  // on: the next applications define the reported eigenvalues (final Rayleigh-Ritz); an operator may use
  // a slower, more accurate accumulation for them
  virtual void set_final(bool on) { (void)on; }
  // true while launches are being captured into a graph (no event timing then)
  bool capturing = false;
  // everything a captured application depends on besides buffer contents (configuration and addresses)
  virtual void signature(std::vector<uint64_t>* sig) const = 0;
  long matvec_columns = 0;
};

template <class S>
struct DenseOperator : Operator<S> {
  const cplx<S>* H = nullptr;
  int dim = 0;
  cudaError_t apply(const cplx<S>* X, int ldx, int c0, int ncol, cplx<S>* Y, int ldy, cudaStream_t s) override {
    this->matvec_columns += ncol;
    return launch_dense_mv<S>(H, dim, X + c0, ldx, Y + c0, ldy, ncol, s);
  }
  void signature(std::vector<uint64_t>* sig) const override {
    sig->push_back(1);
    sig->push_back((uint64_t)(uintptr_t)H);
    sig->push_back((uint64_t)dim);
  }
};

// GEMM_FFT_F32: the contraction as FP32 FFT convolutions over a two-dimensional mesh (k_fftconv.cu)
enum GemmKind { GEMM_TC_BF16 = 0, GEMM_SIMT_F32 = 1, GEMM_SIMT_F64 = 2, GEMM_FFT_F32 = 3 };

// Event pairs around the contraction launches (enabled by wtb_profile_enable).
struct KernelProfile {
  bool on = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
  double total_ms = 0.0, flops = 0.0, bytes = 0.0;
  long long launches = 0;
  void flush() {
    for (auto& pr : pending) {
      float ms = 0.f;
      if (cudaEventSynchronize(pr.second) == cudaSuccess && cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess)
        total_ms += ms;
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
    pending.clear();
  }
  void reset() {
    flush();
    total_ms = flops = bytes = 0.0;
    launches = 0;
  }
};

// Matrix-free operator: gather (Z), contraction (T = V Z), scatter (y).  S = iteration precision.
template <class S>
struct MatFreeOperator : Operator<S> {
  int nk = 0, nv = 0, nc = 0, w = 0, nbmax = 16;
  const zd* vec_win = nullptr;
  const double* dE = nullptr;
  // the same band vectors and transition energies in precision S, which the gather and scatter read (FP32 copies
  // rounded once per operator for the FP32 forms: bitwise the values the tiles would convert)
  const cplx<S>* vec_s = nullptr;
  const S* dE_s = nullptr;
  GemmKind kind = GEMM_SIMT_F32;
  int nslices = 2, npairs = 3;
  int npairs_refine = 0;  // > npairs: slice products used by begin_refine() (needs nslices = 3)
  int pa[8] = {0}, pb[8] = {0};
  int Mpad = 0, Kpad = 0, Npad = 0;
  // contraction operands
  const uint16_t* Vs = nullptr;   // [nslices][Mpad][Kpad] bf16
  uint16_t* Zs = nullptr;         // [nslices][Npad][Kpad] bf16
  const S* Vr = nullptr;          // [nk][Kpad] (SIMT)
  S* Zr = nullptr;                // [Npad][Kpad] (SIMT)
  void* Tm = nullptr;             // [Mpad][Npad] float (TC, FFT) or S (SIMT)
  // FFT kind: the n1 x n2 mesh, the transform size and the stencil's spectrum and twiddles (k_fftconv.cu)
  int mesh1 = 0, mesh2 = 0, fft_p = 0;
  const float2* fft_spec = nullptr;
  const float2* fft_tw = nullptr;
  DevStatus* st = nullptr;
  KernelProfile* prof = nullptr;
  std::map<long, TcGemmPlan*> plans;  // keyed by (N of the chunk, slice products)
  std::string* msg = nullptr;
  ~MatFreeOperator() override {
    for (auto& kv : plans) tc_gemm_plan_destroy(kv.second);
  }
  cudaError_t apply(const cplx<S>* X, int ldx, int c0, int ncol, cplx<S>* Y, int ldy, cudaStream_t s) override;
  // gather + contraction only: leaves T = V Z(X[:, 0:ncol]) in Tm (row k, column ((b w + o) w + p) 2 + ri,
  // leading dimension Npad; float for the tensor-core kind, S otherwise); ncol <= nbmax
  cudaError_t contract(const cplx<S>* X, int ldx, int ncol, cudaStream_t s);
  // T = V Z for the N gathered columns; t_kn: T[k][n] (leading dimension Npad) for every kind, else the FFT kind
  // writes T[n][k] (leading dimension Kpad)
  cudaError_t contract_z(int N, cudaStream_t s, bool t_kn);
  double contraction_flops(int N) const;
  double contraction_bytes(int N) const;
  bool begin_refine() override {
    if (npairs_refine <= npairs) return false;
    npairs = npairs_refine;
    return true;
  }
  void signature(std::vector<uint64_t>* sig) const override {
    const uint64_t v[] = {2, (uint64_t)kind, (uint64_t)nk, (uint64_t)nv, (uint64_t)nc, (uint64_t)w, (uint64_t)nbmax,
                          (uint64_t)nslices, (uint64_t)npairs, (uint64_t)npairs_refine, (uint64_t)kchunk_final,
                          (uint64_t)tile_n, (uint64_t)gather_tile, (uint64_t)scatter_cols,
                          (uint64_t)Mpad, (uint64_t)Kpad, (uint64_t)Npad, (uint64_t)(uintptr_t)vec_win,
                          (uint64_t)(uintptr_t)dE, (uint64_t)(uintptr_t)vec_s, (uint64_t)(uintptr_t)dE_s,
                          (uint64_t)(uintptr_t)Vs, (uint64_t)(uintptr_t)Zs,
                          (uint64_t)(uintptr_t)Vr, (uint64_t)(uintptr_t)Zr, (uint64_t)(uintptr_t)Tm,
                          (uint64_t)(uintptr_t)st, (uint64_t)mesh1, (uint64_t)mesh2, (uint64_t)fft_p,
                          (uint64_t)(uintptr_t)fft_spec, (uint64_t)(uintptr_t)fft_tw};
    sig->insert(sig->end(), v, v + sizeof(v) / sizeof(v[0]));
  }
  // launches the contraction of an ncol-column application (the first phase's slice products) reps times
  // with CUDA events around each, into prof (the eigensolve itself runs as one graph launch)
  int npairs0 = 0;
  cudaError_t time_contraction(int reps, int ncol, cudaStream_t s);
  // tensor-core kind: K blocks per accumulation range in the final applications (0: one range).  The FP32
  // accumulation error of the final application grows about linearly with the range: on the 57,600-dim
  // workload the exciton energies moved by 3.7e-7 / 7.2e-7 / 1.5e-6 / 5.3e-6 eV from the FP64 form with 4 / 8
  // / 16 / 64 blocks per range, and the solve took 15.58 / 15.21 / 15.00 / 14.77 ms; 8 keeps a 14x margin to
  // the 1e-5 eV bound
  int kchunk_final = 8;
  bool final_apply = false;
  void set_final(bool on) override { final_apply = on; }
  // launch shapes chosen by autotune() for the operator's shape (tensor-core kind): the contraction's column
  // tile, the gather tile (KT * 100 + block columns per chunk; 0 = the shared-memory rule) and the scatter's
  // block columns per CTA (0 = all that fit)
  int tile_n = 256;
  int gather_tile = 0;
  int scatter_cols = 0;
  TcGemmPlan* plan_for(int N, int np, int bn);
  // X, Y: row-major dim x nbmax scratch blocks (row stride nbmax) that the timed applications use
  cudaError_t autotune(cudaStream_t s, const cplx<S>* X, cplx<S>* Y);
};

struct SolveStats {
  int iterations = 0;
  long matvec_columns = 0;
  double max_rel_residual = 0.0;
  double refine_shift_max = 0.0;
  int launches = 0;
};

// Lowest nev eigenpairs of the Hermitian operator.  diag = its diagonal (preconditioner and start
// vectors).  Output: E (host, nev) and the FP64 eigenvectors Xout (device, dim x nev row-major).
// tol_refine > 0: once tol is met, switch the operator to its accurate arithmetic (begin_refine) and
// continue to tol_refine.
template <class S>
int lobpcg_solve(Operator<S>& op, const double* diag, int dim, int nev, int m, double tol, int maxit,
                 Workspace& ws, DevStatus* st, cudaStream_t s, std::vector<double>* E, zd* Xout, SolveStats* stats,
                 std::string* msg, double tol_refine = 0.0);

// The lowest nev eigenpairs for nev beyond one block (the reference asks 100): chunks of `chunk` eigenpairs,
// each an ordinary solve with block m of P H P + sigma Q Q^H, Q the eigenvectors of the chunks before it and
// P = I - Q Q^H (sigma moves span(Q) above the eigenvalues still sought).  Same outputs as lobpcg_solve, ascending.
template <class S>
int lobpcg_solve_deflated(Operator<S>& op, const double* diag, int dim, int nev, int chunk, int m, double tol,
                          int maxit, double sigma, Workspace& ws, DevStatus* st, cudaStream_t s, std::vector<double>* E,
                          zd* Xout, SolveStats* stats, std::string* msg, double tol_refine = 0.0);

// A ragged batch of independent eigenproblems in one concatenated row space (BatchMap, device tables; the
// solver sets its frozen flags and part count): nrow rows in all, nparts reduction parts, dims[q] the rows of
// system q.  A single system needs only nrow and dims = {nrow}.
struct BatchLayout {
  BatchMap bm;
  int nrow = 0;
  int nparts = 0;
  std::vector<int> dims;
};

// A solve inside a caller's graph: with build, the solve's nodes are added to graph after deps (tail receives
// its last nodes, launches and body_launches the kernels captured) and nothing is launched or read back; after
// the caller has launched its graph, the same call with collect reads the results.
struct SolveGraph {
  cudaGraph_t graph = nullptr;
  std::vector<cudaGraphNode_t> deps, tail;
  long long launches = 0, body_launches[2] = {0, 0};
  bool build = false, collect = false;
};

// The lowest nev eigenpairs of every system of the batch, iterated together: one launch of each kernel covers
// all systems still running, a system that has converged is frozen, and the loop ends when the last one
// has.  diag and Xout in the concatenated rows; E (host) nsys x nev; per-system statistics and status codes.
// The frozen flags live in ws buffer "lob_frozen" (nsys ints), where a batched operator can read them.
template <class S>
int lobpcg_solve_batch(Operator<S>& op, const double* diag, const BatchLayout& L, int nev, int m, double tol,
                       int maxit, Workspace& ws, DevStatus* st, cudaStream_t s, std::vector<double>* E, zd* Xout,
                       std::vector<SolveStats>* stats, std::vector<int>* sys_status, std::string* msg,
                       double tol_refine = 0.0, SolveGraph* sg = nullptr);

// The split-BF16 matrix-free operators of a batch of systems applied together: one gather, one grouped
// tensor-core contraction and one scatter launch cover every system still iterating (all of them in the final
// application).  Rows of system q start at sys[q].row0 of the concatenated block vectors.
struct BatchMatFreeOperator : Operator<float> {
  int nsys = 0, nbmax = 16, max_nv = 0, max_nc = 0, max_w = 0;
  int nslices = 3, npairs = 3, npairs_refine = 6;
  int pa[8] = {0}, pb[8] = {0};
  int kchunk_final = 8;  // K blocks per accumulation range of the final application (as the single operator)
  bool final_apply = false;
  const MfSys* d_sys = nullptr;
  const int2* d_gtiles = nullptr;  // gather tiles (system, first k-point)
  int ngtiles = 0;
  const int2* d_kpts = nullptr;    // scatter k-points (system, k)
  int nkpts = 0;
  TcGroupPlan* gemm = nullptr;     // owned
  const int* frozen = nullptr;
  DevStatus* st = nullptr;
  ~BatchMatFreeOperator() override {
    if (gemm) tc_gemm_group_destroy(gemm);
  }
  cudaError_t apply(const zf* X, int ldx, int c0, int ncol, zf* Y, int ldy, cudaStream_t s) override;
  bool begin_refine() override {
    if (npairs_refine <= npairs) return false;
    npairs = npairs_refine;
    return true;
  }
  void set_final(bool on) override { final_apply = on; }
  void signature(std::vector<uint64_t>* sig) const override {
    const uint64_t v[] = {3, (uint64_t)nsys, (uint64_t)nbmax, (uint64_t)nslices, (uint64_t)npairs,
                          (uint64_t)npairs_refine, (uint64_t)kchunk_final, (uint64_t)(uintptr_t)d_sys,
                          (uint64_t)(uintptr_t)d_gtiles, (uint64_t)(uintptr_t)d_kpts, (uint64_t)(uintptr_t)gemm,
                          (uint64_t)(uintptr_t)frozen, (uint64_t)(uintptr_t)st};
    sig->insert(sig->end(), v, v + sizeof(v) / sizeof(v[0]));
  }
};

// extra launchers used by the solver
template <class S>
cudaError_t launch_heev_small(const zd* A, int lda, const int* nptr, int nmax, int nwant, double* evals, zd* evecs,
                              int ldv, cudaStream_t s, const BatchMap& bm = BatchMap(), long a_stride = 0,
                              long e_stride = 0, long v_stride = 0);
template <class S>
cudaError_t launch_pchol_basis(const zd* M, int ldm, int n, double drop, zd* B, int ldb, int* r_out, cudaStream_t s,
                               const BatchMap& bm = BatchMap(), long m_stride = 0, long b_stride = 0);
cudaError_t launch_select_lowest(const double* diag, int dim, int m, int* idx, double* cand_val, cudaStream_t s);
cudaError_t launch_select_lowest_batch(const double* diag, const BatchMap& bm, int m, int* idx, long idx_stride,
                                       double* cand_val, int* cand_idx, cudaStream_t s);
template <class S>
cudaError_t launch_init_guess(cplx<S>* X, int ldx, int nrow, int m, const int* idx, unsigned seed, cudaStream_t s,
                              const BatchMap& bm = BatchMap(), long idx_stride = 0);
void tc_gemm_set_valid(TcGemmPlan* p, int m_valid, int n_valid);

}  // namespace wtb
