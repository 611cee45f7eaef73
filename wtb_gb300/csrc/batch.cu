// Batches of independent exciton systems on one GPU, solved in one graph launch.
//
// A system of the strain/mesh scans is small (dim 576..11,664): solved alone, its eigensolve is a chain of
// short kernels (the projected eigenproblems run on one CTA) that leaves most of the 152 SMs idle.  The batch
// therefore solves all systems together:
//   - every system keeps its own context (slot): H(R), k-points, bands, optical matrix elements and its
//     split-BF16 operator data (V table slices, Z panel, contraction result);
//   - the block eigensolver runs once for the whole batch over one concatenated row space (systems padded to
//     32-row tiles, BatchMap): each kernel launch covers every system still iterating, the projected
//     eigenproblems of all systems run side by side (one CTA each), the operator is one gather launch, one
//     grouped tensor-core contraction (tcgen05, one tile list over all systems) and one scatter launch, and a
//     converged system is frozen until the loop ends with the last one;
//   - one CUDA graph holds everything after the host staging (H(R) and k-points to the device): the
//     per-system set-up kernels as parallel branches, the joint eigensolve (WHILE nodes), the per-system
//     oscillator strengths.  The graph is cached and relaunched while the batch keeps its shapes.
// Precisions other than the split-BF16 matrix-free forms are solved system by system on the slots.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ctx.h"

using namespace wtb;

struct wtb_batch {
  int device = 0;
  int nworkers = 1;
  std::vector<wtb_ctx*> slots;   // one context per system
  wtb_ctx* main = nullptr;       // the joint eigensolve: stream, status word, workspace
  std::vector<std::string> errors;
  // the graph of the last batch shape and everything its nodes refer to
  uint64_t key = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long graph_launches = 0;
  SolveGraph sg;
  BatchLayout L;
  std::vector<OpBundle> obs;
  std::unique_ptr<BatchMatFreeOperator> op;
  int nev = 0, m = 0;
  double tol = 0.0, tol_refine = 0.0;
  int maxit = 200;
  std::vector<int> row0, dims;
  // host wall time of the last call's phases (ms): staging, graph build (0 when reused), graph run, read-back
  double t_stage = 0, t_build = 0, t_run = 0, t_collect = 0;
  // device time of the graph's phases (ms): per-system set-up, joint eigensolve, oscillator strengths; from
  // event-record nodes at the two joins and events around the launch
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  double t_front = 0, t_solve = 0, t_back = 0;
  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    key = 0;
    op.reset();
    obs.clear();
  }
};

namespace {

uint64_t fnv(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

// capture of one stream's launches into g after deps; tail receives the last nodes
struct Capture {
  cudaStream_t s;
  cudaError_t begin(cudaGraph_t g, const std::vector<cudaGraphNode_t>& deps) {
    return cudaStreamBeginCaptureToGraph(s, g, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                         cudaStreamCaptureModeRelaxed);
  }
  cudaError_t end(std::vector<cudaGraphNode_t>* tail) {
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t* d = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &d, nullptr, &nd);
    if (tail && e == cudaSuccess) tail->assign(d, d + nd);
    cudaGraph_t g2 = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(s, &g2);
    return e != cudaSuccess ? e : e2;
  }
};

bool split_bf16_form(const wtb_bse_params& p) {
  return p.op == WTB_OP_MATFREE && (p.precision == WTB_PREC_BF16X3 || p.precision == WTB_PREC_BF16X6);
}

// the per-system device work in front of the joint eigensolve: bands, optics, operator data, and the system's
// transition energies copied into the concatenated preconditioner diagonal
int enqueue_front(wtb_ctx* c, const wtb_bse_params* p, int nbmax, OpBundle* ob, double* diag_rows) {
  int r = ctx_enqueue_system(c, p, nbmax, ob);
  if (r != WTB_OK) return r;
  if (!ob->o32 || !ob->dE) return ctx_set_err(c, WTB_EBADARG, "batch: not a split-BF16 matrix-free operator");
  if (cudaMemcpyAsync(diag_rows, ob->dE, sizeof(double) * ob->dim, cudaMemcpyDeviceToDevice, c->s) != cudaSuccess)
    return ctx_set_err(c, WTB_ECUDA, "batch: diagonal copy failed");
  return WTB_OK;
}

// oscillator strengths of the system's nev excitons (rows row0.. of Xout) into osc (8 x nev)
int enqueue_back(wtb_ctx* c, const zd* Xout_rows, int nev, int dim, double* osc) {
  cudaError_t err = cudaSuccess;
  const int npart = (dim + 255) / 256;
  double* part = c->ws.get<double>("osc_part", (size_t)npart * nev * 10, &err);
  const zd* hr = c->ws.find<zd>("hrvel", (size_t)5 * dim);
  if (err != cudaSuccess || !hr) return ctx_set_err(c, WTB_ENOMEM, "batch: oscillator buffers");
  if (launch_oscillators(Xout_rows, nev, nev, dim, hr, osc, part, npart, c->s) != cudaSuccess)
    return ctx_set_err(c, WTB_ECUDA, "batch: oscillator launch failed");
  return WTB_OK;
}

double system_cost(const wtb_system& s, const wtb_bse_params& p) {
  const double nk = (double)p.ngrid[0] * p.ngrid[1] * p.ngrid[2];
  return nk * nk * (double)s.w90basis * s.w90basis * std::max(p.nev, 1) + nk * p.nc * p.nv * 1e3;
}

// Systems whose precision is not a split-BF16 form: one after the other on their slots.
int solve_each(wtb_batch* b, int nsys, const wtb_system* sys, const wtb_bse_params* p, int nev_stride, double* E,
               double* act, int* status, int* iterations) {
  std::vector<int> order(nsys);
  for (int i = 0; i < nsys; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return system_cost(sys[x], p[x]) > system_cost(sys[y], p[y]); });
  std::vector<double> Ws, acts;
  for (int i : order) {
    wtb_ctx* c = b->slots[i];
    const wtb_system& s = sys[i];
    int r = wtb_set_hr(c, s.w90basis, s.nvec, s.rvec, s.ffactor, s.hopmatrices, s.ihopmatrices, s.rlat, s.efermi, s.scs,
                       s.systype_np);
    wtb_timings t{};
    if (r == WTB_OK) {
      const long dim = (long)p[i].ngrid[0] * p[i].ngrid[1] * p[i].ngrid[2] * p[i].nc * p[i].nv;
      if (dim < 1) {
        r = WTB_EBADARG;
      } else {
        Ws.assign(dim, 0.0);
        acts.assign((size_t)dim * 8, 0.0);
        r = wtb_bsesolver(c, &p[i], Ws.data(), act ? acts.data() : nullptr, nullptr, &t);
        if (r == WTB_OK) {
          const int nev = p[i].nev;
          if (E)
            for (int n = 0; n < nev; ++n) E[(size_t)i * nev_stride + n] = Ws[n];
          if (act)
            for (int a = 0; a < 8; ++a)
              for (int n = 0; n < nev; ++n) act[((size_t)i * 8 + a) * nev_stride + n] = acts[(size_t)a * dim + n];
        }
      }
    }
    status[i] = r;
    if (iterations) iterations[i] = t.iterations;
    if (r != WTB_OK) b->errors[i] = wtb_last_error(c);
  }
  for (int i = 0; i < nsys; ++i)
    if (status[i] != WTB_OK) return status[i];
  return WTB_OK;
}

template <class T>
T* upload(Workspace& ws, const char* name, const std::vector<T>& h, cudaStream_t s, cudaError_t* err) {
  T* d = ws.get<T>(name, std::max<size_t>(h.size(), 1), err);
  if (*err == cudaSuccess && !h.empty()) *err = cudaMemcpyAsync(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s);
  return d;
}

// Builds the batch graph (set-up branches, joint eigensolve, oscillator branches) for the staged systems.
// eager (WTB_SOLVER_STREAM, for kernel profilers, which do not see kernels inside conditional graph bodies):
// no graph; the joint eigensolve runs with the host driving its loop and the oscillator kernels follow it,
// results into *E, *stats, *sst.
int build_graph(wtb_batch* b, int nsys, const wtb_bse_params* p, std::string* msg, bool eager = false,
                std::vector<double>* E = nullptr, std::vector<SolveStats>* stats = nullptr,
                std::vector<int>* sst = nullptr) {
  wtb_ctx* mc = b->main;
  cudaError_t err = cudaSuccess;
  const bool x6 = p[0].precision == WTB_PREC_BF16X6;
  // the concatenated row space: systems padded to whole row tiles, reduction parts of up to kPartRows rows
  constexpr int kPartRows = 256;
  b->row0.assign(nsys, 0);
  b->dims.assign(nsys, 0);
  std::vector<int> tile_sys;
  std::vector<int2> rows(nsys), parts, sys_parts(nsys);
  std::vector<int> part_sys;
  long nrow = 0;
  int mindim = 1 << 30, nevmax = 1;
  for (int q = 0; q < nsys; ++q) {
    const int dim = b->slots[q]->nk * b->slots[q]->nc * b->slots[q]->nv;
    b->row0[q] = (int)nrow;
    b->dims[q] = dim;
    rows[q] = make_int2((int)nrow, dim);
    const int padded = (dim + kTileRows - 1) / kTileRows * kTileRows;
    for (int t = 0; t < padded / kTileRows; ++t) tile_sys.push_back(q);
    sys_parts[q] = make_int2((int)parts.size(), 0);
    for (int r = 0; r < padded; r += kPartRows) {
      parts.push_back(make_int2((int)(nrow + r), (int)(nrow + std::min(padded, r + kPartRows))));
      part_sys.push_back(q);
      sys_parts[q].y += 1;
    }
    nrow += padded;
    mindim = std::min(mindim, dim);
    nevmax = std::max(nevmax, p[q].nev);
  }
  if (nrow > (1L << 30)) return ctx_set_err(mc, WTB_EBADARG, "batch too large");
  wtb_bse_params pm = p[0];
  pm.nev = nevmax;
  b->nev = nevmax;
  b->m = ctx_auto_block(&pm, mindim, false);
  const int nbmax = std::min(b->m, 16);
  const double tol_final = p[0].tol > 0 ? p[0].tol : kReducedTol;
  // two phases in every form (see run_solve): to 1e-4, then from the best block with a fresh operator
  // application (and 6 slice products for bf16x3) to the target
  b->tol = std::max(tol_final, 1e-4);
  b->tol_refine = tol_final < b->tol ? tol_final : 0.0;
  b->maxit = p[0].maxit > 0 ? p[0].maxit : 200;

  Workspace& ws = mc->ws;
  BatchLayout& L = b->L;
  L = BatchLayout();
  L.bm.nsys = nsys;
  L.bm.nparts = (int)parts.size();
  L.bm.tile_sys = upload(ws, "b_tile_sys", tile_sys, mc->s, &err);
  L.bm.rows = upload(ws, "b_rows", rows, mc->s, &err);
  L.bm.parts = upload(ws, "b_parts", parts, mc->s, &err);
  L.bm.part_sys = upload(ws, "b_part_sys", part_sys, mc->s, &err);
  L.bm.sys_parts = upload(ws, "b_sys_parts", sys_parts, mc->s, &err);
  L.nrow = (int)nrow;
  L.nparts = (int)parts.size();
  L.dims = b->dims;
  double* diag = ws.get<double>("b_diag", nrow, &err, true);
  zd* Xout = ws.get<zd>("b_Xout", (size_t)nrow * nevmax, &err);
  double* osc = ws.get<double>("b_osc", (size_t)nsys * 8 * nevmax, &err, true);
  int* frozen = ws.get<int>("lob_frozen", nsys, &err, true);
  if (err != cudaSuccess || cudaStreamSynchronize(mc->s) != cudaSuccess)
    return ctx_set_err(mc, WTB_ENOMEM, "batch: layout buffers");

  // per-system set-up once outside any graph: allocates every buffer the captured work uses
  b->obs.clear();
  b->obs.resize(nsys);
  for (int q = 0; q < nsys; ++q) {
    wtb_ctx* c = b->slots[q];
    int r = enqueue_front(c, &p[q], nbmax, &b->obs[q], diag + b->row0[q]);
    if (r == WTB_OK) r = enqueue_back(c, Xout + (size_t)b->row0[q] * nevmax, nevmax, b->dims[q], osc + (size_t)q * 8 * nevmax);
    if (r == WTB_OK && cudaStreamSynchronize(c->s) != cudaSuccess) r = ctx_set_err(c, WTB_ECUDA, "batch: set-up failed");
    // a system whose bands fail their checks stays in the batch (its rows and small matrices are its own);
    // the status word is read again after the graph has run and reports it then
    if (r == WTB_OK) ctx_check_status(c);
    if (r != WTB_OK) {
      *msg = "system " + std::to_string(q) + ": " + wtb_last_error(c);
      b->errors[q] = wtb_last_error(c);
      return r;
    }
  }
  // the batched operator over the systems' operator data
  std::vector<MfSys> ms(nsys);
  std::vector<int2> gtiles, kpts;
  std::vector<TcGroupDesc> gd(nsys);
  int max_nv = 0, max_nc = 0, max_w = 0;
  for (int q = 0; q < nsys; ++q) {
    auto* mf = dynamic_cast<MatFreeOperator<float>*>(b->obs[q].o32.get());
    if (!mf || mf->kind != GEMM_TC_BF16) return ctx_set_err(mc, WTB_EBADARG, "batch: not a split-BF16 operator");
    MfSys& s = ms[q];
    s.row0 = b->row0[q];
    s.nk = mf->nk;
    s.nv = mf->nv;
    s.nc = mf->nc;
    s.w = mf->w;
    s.ldk = mf->Kpad;
    s.ldt = mf->Npad;
    s.slice_stride = (long)mf->Npad * mf->Kpad;
    s.vec_win = mf->vec_win;
    s.dE = mf->dE;
    s.zt = mf->Zs;
    s.Tm = reinterpret_cast<const float*>(mf->Tm);
    for (int k = 0; k < s.nk; k += 16) gtiles.push_back(make_int2(q, k));  // refined below to the tile size
    for (int k = 0; k < s.nk; ++k) kpts.push_back(make_int2(q, k));
    gd[q].A = mf->Vs;
    gd[q].B = mf->Zs;
    gd[q].C = reinterpret_cast<float*>(mf->Tm);
    gd[q].M = mf->Mpad;
    gd[q].N = mf->Npad;
    gd[q].K = mf->Kpad;
    gd[q].ldc = mf->Npad;
    gd[q].m_valid = mf->nk;
    gd[q].n_valid = 2 * mf->w * mf->w * nbmax;
    max_nv = std::max(max_nv, s.nv);
    max_nc = std::max(max_nc, s.nc);
    max_w = std::max(max_w, s.w);
  }
  // gather tiles of the tile size the launcher picks for this batch's widest system
  const int gkt = mf_gather_batch_tile(max_nv, max_nc, max_w, nbmax);
  gtiles.clear();
  for (int q = 0; q < nsys; ++q)
    for (int k = 0; k < ms[q].nk; k += gkt) gtiles.push_back(make_int2(q, k));
  auto op = std::make_unique<BatchMatFreeOperator>();
  op->nsys = nsys;
  op->nbmax = nbmax;
  op->max_nv = max_nv;
  op->max_nc = max_nc;
  op->max_w = max_w;
  op->nslices = 3;
  op->npairs = x6 ? 6 : 3;
  op->npairs_refine = 6;
  const int pa6[6] = {0, 0, 1, 0, 1, 2}, pb6[6] = {0, 1, 0, 2, 1, 0};
  for (int i = 0; i < 6; ++i) {
    op->pa[i] = pa6[i];
    op->pb[i] = pb6[i];
  }
  op->d_sys = upload(ws, "b_mfsys", ms, mc->s, &err);
  op->d_gtiles = upload(ws, "b_gtiles", gtiles, mc->s, &err);
  op->ngtiles = (int)gtiles.size();
  op->d_kpts = upload(ws, "b_kpts", kpts, mc->s, &err);
  op->nkpts = (int)kpts.size();
  op->frozen = frozen;
  op->st = mc->st;
  if (err != cudaSuccess || cudaStreamSynchronize(mc->s) != cudaSuccess)
    return ctx_set_err(mc, WTB_ENOMEM, "batch: operator tables");
  // the grouped contraction's column tile: measured on this batch's own operands (once per batch shape)
  std::string m2;
  TcGroupPlan* gp[2] = {nullptr, nullptr};  // bn = 256, 128
  auto group_of = [&](int bn) -> TcGroupPlan* {
    TcGroupPlan*& g = gp[bn == 128 ? 1 : 0];
    if (!g && tc_gemm_group_create(&g, nsys, gd.data(), 3, 6, op->pa, op->pb, &m2, bn) != WTB_OK) g = nullptr;
    return g;
  };
  uint64_t tkey = 1469598103934665603ull;
  for (int q = 0; q < nsys; ++q) {
    const int v[5] = {gd[q].M, gd[q].K, gd[q].N, gd[q].m_valid, gd[q].n_valid};
    tkey = fnv(tkey, v, sizeof(v));
  }
  // the batch's shape: its system count, slice products and a hash of every system's contraction extents
  char shape[128];
  std::snprintf(shape, sizeof(shape), "grouped contraction systems=%d products=%d extents=%016llx", nsys, op->npairs,
                (unsigned long long)tkey);
  const int bn = tune_choice(shape, "tile_n", {256, 128}, 256, [&](int cand) -> cudaError_t {
    TcGroupPlan* g = group_of(cand);
    return g ? tc_gemm_group_run(g, op->npairs, nullptr, mc->st, mc->s) : cudaErrorInvalidValue;
  }, mc->s);
  op->gemm = group_of(bn);
  if (gp[0] && gp[0] != op->gemm) tc_gemm_group_destroy(gp[0]);
  if (gp[1] && gp[1] != op->gemm) tc_gemm_group_destroy(gp[1]);
  if (!op->gemm || cudaStreamSynchronize(mc->s) != cudaSuccess) return ctx_set_err(mc, WTB_ECUDA, "batch: " + m2);

  if (eager) {
    b->op = std::move(op);
    int r = lobpcg_solve_batch<float>(*b->op, diag, L, nevmax, b->m, b->tol, b->maxit, ws, mc->st, mc->s, E, Xout,
                                      stats, sst, msg, b->tol_refine, nullptr);
    if (cudaStreamSynchronize(mc->s) != cudaSuccess) r = ctx_set_err(mc, WTB_ECUDA, "batch: eigensolve failed");
    for (int q = 0; q < nsys && r != WTB_ECUDA; ++q) {
      wtb_ctx* c = b->slots[q];
      const int rb = enqueue_back(c, Xout + (size_t)b->row0[q] * nevmax, nevmax, b->dims[q], osc + (size_t)q * 8 * nevmax);
      if (rb != WTB_OK || cudaStreamSynchronize(c->s) != cudaSuccess) r = ctx_set_err(mc, WTB_ECUDA, "batch: oscillators");
    }
    return r;
  }
  // the graph: set-up branches, joint eigensolve after all of them, oscillator branches after it
  cudaGraph_t G = nullptr;
  if (cudaGraphCreate(&G, 0) != cudaSuccess) return ctx_set_err(mc, WTB_ECUDA, "batch: graph creation failed");
  const long long captured0 = g_launch_count.load();
  std::vector<cudaGraphNode_t> joins;
  int rc = WTB_OK;
  for (int q = 0; q < nsys && rc == WTB_OK; ++q) {
    wtb_ctx* c = b->slots[q];
    Capture cap{c->s};
    std::vector<cudaGraphNode_t> tail;
    if (cap.begin(G, {}) != cudaSuccess) {
      rc = ctx_set_err(mc, WTB_ECUDA, "batch: capture failed");
      break;
    }
    OpBundle ob;
    rc = enqueue_front(c, &p[q], nbmax, &ob, diag + b->row0[q]);
    if (cap.end(&tail) != cudaSuccess && rc == WTB_OK) rc = ctx_set_err(mc, WTB_ECUDA, "batch: capture failed");
    if (rc != WTB_OK) *msg = "system " + std::to_string(q) + ": " + wtb_last_error(c);
    // the operator objects of the first pass own the same buffers; keep those
    joins.insert(joins.end(), tail.begin(), tail.end());
  }
  // event-record node after the set-up branches (device time of the phases)
  auto mark = [&](cudaEvent_t e, const std::vector<cudaGraphNode_t>& deps, std::vector<cudaGraphNode_t>* out) {
    Capture cap{mc->s};
    if (cap.begin(G, deps) != cudaSuccess) return ctx_set_err(mc, WTB_ECUDA, "batch: capture failed");
    const cudaError_t e1 = cudaEventRecordWithFlags(e, mc->s, cudaEventRecordExternal);
    if (cap.end(out) != cudaSuccess || e1 != cudaSuccess) return ctx_set_err(mc, WTB_ECUDA, "batch: capture failed");
    return WTB_OK;
  };
  if (rc == WTB_OK) rc = mark(b->ev[1], joins, &joins);
  if (rc == WTB_OK) {
    b->op = std::move(op);
    b->sg = SolveGraph();
    b->sg.graph = G;
    b->sg.deps = joins;
    b->sg.build = true;
    std::vector<double> E;
    rc = lobpcg_solve_batch<float>(*b->op, diag, L, nevmax, b->m, b->tol, b->maxit, ws, mc->st, mc->s, &E, Xout,
                                   nullptr, nullptr, msg, b->tol_refine, &b->sg);
  }
  std::vector<cudaGraphNode_t> solved;
  if (rc == WTB_OK) rc = mark(b->ev[2], b->sg.tail, &solved);
  for (int q = 0; q < nsys && rc == WTB_OK; ++q) {
    wtb_ctx* c = b->slots[q];
    Capture cap{c->s};
    if (cap.begin(G, solved) != cudaSuccess) {
      rc = ctx_set_err(mc, WTB_ECUDA, "batch: capture failed");
      break;
    }
    rc = enqueue_back(c, Xout + (size_t)b->row0[q] * nevmax, nevmax, b->dims[q], osc + (size_t)q * 8 * nevmax);
    if (cap.end(nullptr) != cudaSuccess && rc == WTB_OK) rc = ctx_set_err(mc, WTB_ECUDA, "batch: capture failed");
  }
  cudaGraphExec_t X = nullptr;
  if (rc == WTB_OK && cudaGraphInstantiate(&X, G, 0) != cudaSuccess) rc = ctx_set_err(mc, WTB_ECUDA, "batch: graph instantiation failed");
  if (rc != WTB_OK) {
    if (msg->empty()) *msg = wtb_last_error(mc);
    cudaGraphDestroy(G);
    b->op.reset();
    return rc;
  }
  b->graph = G;
  b->exec = X;
  b->graph_launches = g_launch_count.load() - captured0;
  g_launch_count -= b->graph_launches;  // counted again when the graph is launched
  return WTB_OK;
}

}  // namespace

extern "C" int wtb_batch_create(wtb_batch** out, int device, int nworkers) {
  if (!out || nworkers < 1 || nworkers > 64) return WTB_EBADARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return WTB_ENODEV;
  auto* b = new wtb_batch();
  b->device = device;
  b->nworkers = nworkers;
  if (wtb_ctx_create(&b->main, device) != WTB_OK) {
    delete b;
    return WTB_ENODEV;
  }
  for (auto& e : b->ev)
    if (cudaEventCreate(&e) != cudaSuccess) {
      wtb_batch_destroy(b);
      return WTB_ENODEV;
    }
  *out = b;
  return WTB_OK;
}

extern "C" int wtb_batch_destroy(wtb_batch* b) {
  if (!b) return WTB_OK;
  if (b->main) cudaStreamSynchronize(b->main->s);
  b->drop_graph();
  for (wtb_ctx* w : b->slots) wtb_ctx_destroy(w);
  for (auto& e : b->ev)
    if (e) cudaEventDestroy(e);
  wtb_ctx_destroy(b->main);
  delete b;
  return WTB_OK;
}

extern "C" const char* wtb_batch_error(const wtb_batch* b, int i) {
  if (!b || i < 0 || i >= (int)b->errors.size()) return "";
  return b->errors[i].c_str();
}

extern "C" int wtb_batch_bsesolver(wtb_batch* b, int nsys, const wtb_system* sys, const wtb_bse_params* p,
                                   int nev_stride, double* E, double* act, int* status, int* iterations,
                                   double* wall_ms) {
  if (!b || nsys < 0 || (nsys > 0 && (!sys || !p || !status)) || nev_stride < 1) return WTB_EBADARG;
  for (int i = 0; i < nsys; ++i)
    if (p[i].nev < 1 || p[i].nev > nev_stride) return WTB_EBADARG;
  const auto t0 = std::chrono::steady_clock::now();
  b->errors.assign(nsys, std::string());
  for (int i = 0; i < nsys; ++i) status[i] = WTB_OK;
  while ((int)b->slots.size() < nsys) {
    wtb_ctx* c = nullptr;
    const int r = wtb_ctx_create(&c, b->device);
    if (r != WTB_OK) return r;
    b->slots.push_back(c);
  }
  auto finish = [&](int r) {
    if (wall_ms)
      wall_ms[0] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return r;
  };
  if (nsys == 0) return finish(WTB_OK);
  bool joint = true;
  for (int i = 0; i < nsys; ++i)
    joint = joint && split_bf16_form(p[i]) && p[i].precision == p[0].precision && p[i].tol == p[0].tol &&
            p[i].maxit == p[0].maxit && p[i].block == p[0].block;
  if (!joint) return finish(solve_each(b, nsys, sys, p, nev_stride, E, act, status, iterations));

  // host staging: H(R), reciprocal vectors and k-points of every system to its slot
  int first_bad = WTB_OK;
  for (int q = 0; q < nsys; ++q) {
    wtb_ctx* c = b->slots[q];
    const wtb_system& s = sys[q];
    int r = wtb_set_hr(c, s.w90basis, s.nvec, s.rvec, s.ffactor, s.hopmatrices, s.ihopmatrices, s.rlat, s.efermi, s.scs,
                       s.systype_np);
    if (r == WTB_OK) r = ctx_stage_system(c, &p[q]);
    if (r == WTB_OK && cudaStreamSynchronize(c->s) != cudaSuccess) r = ctx_set_err(c, WTB_ECUDA, "staging failed");
    if (r != WTB_OK) {
      status[q] = r;
      b->errors[q] = wtb_last_error(c);
      if (first_bad == WTB_OK) first_bad = r;
    }
  }
  if (first_bad != WTB_OK) return finish(first_bad);

  auto ms_since = [](std::chrono::steady_clock::time_point a) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
  };
  b->t_stage = ms_since(t0);
  b->t_build = 0;
  const auto t1 = std::chrono::steady_clock::now();
  // the graph: reused while every baked-in size, parameter and device address is unchanged
  uint64_t key = 1469598103934665603ull;
  key = fnv(key, &nsys, sizeof(nsys));
  for (int q = 0; q < nsys; ++q) {
    const wtb_ctx* c = b->slots[q];
    key = fnv(key, &p[q], sizeof(wtb_bse_params));
    const double sh[2] = {c->efermi, c->scs};
    const int si[4] = {c->w, c->nR, c->systype_np, c->nk};
    key = fnv(key, sh, sizeof(sh));
    key = fnv(key, si, sizeof(si));
    key = fnv(key, c->rlat_rm, sizeof(c->rlat_rm));
    key = fnv(key, &c->ws.generation, sizeof(uint64_t));
  }
  key = fnv(key, &b->main->ws.generation, sizeof(uint64_t));
  if (key == 0) key = 1;
  std::string msg;
  wtb_ctx* mc = b->main;
  std::vector<double> Eall;
  std::vector<SolveStats> stats;
  std::vector<int> sst;
  int rc = WTB_OK;
  const bool eager = std::getenv("WTB_SOLVER_STREAM") != nullptr;
  if (eager) {
    b->drop_graph();
    rc = build_graph(b, nsys, p, &msg, true, &Eall, &stats, &sst);
    if (!b->op) {
      for (int q = 0; q < nsys; ++q) {
        status[q] = rc;
        if (b->errors[q].empty()) b->errors[q] = msg;
      }
      return finish(rc);
    }
    b->t_build = b->t_run = ms_since(t1);
  } else {
  if (!(b->exec && b->key == key)) {
    b->drop_graph();
    const int r = build_graph(b, nsys, p, &msg);
    if (r != WTB_OK) {
      for (int q = 0; q < nsys; ++q) {
        status[q] = r;
        if (b->errors[q].empty()) b->errors[q] = msg;
      }
      return finish(r);
    }
    // the key of the state after building (building allocates)
    uint64_t k2 = 1469598103934665603ull;
    k2 = fnv(k2, &nsys, sizeof(nsys));
    for (int q = 0; q < nsys; ++q) {
      const wtb_ctx* c = b->slots[q];
      k2 = fnv(k2, &p[q], sizeof(wtb_bse_params));
      const double sh[2] = {c->efermi, c->scs};
      const int si[4] = {c->w, c->nR, c->systype_np, c->nk};
      k2 = fnv(k2, sh, sizeof(sh));
      k2 = fnv(k2, si, sizeof(si));
      k2 = fnv(k2, c->rlat_rm, sizeof(c->rlat_rm));
      k2 = fnv(k2, &c->ws.generation, sizeof(uint64_t));
    }
    k2 = fnv(k2, &b->main->ws.generation, sizeof(uint64_t));
    b->key = k2 == 0 ? 1 : k2;
  }
  b->t_build = ms_since(t1);
  const auto t2 = std::chrono::steady_clock::now();
  g_launch_count += b->graph_launches;
  if (cudaEventRecord(b->ev[0], mc->s) != cudaSuccess || cudaGraphLaunch(b->exec, mc->s) != cudaSuccess ||
      cudaEventRecord(b->ev[3], mc->s) != cudaSuccess || cudaStreamSynchronize(mc->s) != cudaSuccess) {
    b->drop_graph();
    for (int q = 0; q < nsys; ++q) {
      status[q] = WTB_ECUDA;
      b->errors[q] = "batch graph launch failed";
    }
    return finish(WTB_ECUDA);
  }
  b->t_run = ms_since(t2);
  {
    float a = 0.f, c2 = 0.f, d = 0.f;
    cudaEventElapsedTime(&a, b->ev[0], b->ev[1]);
    cudaEventElapsedTime(&c2, b->ev[1], b->ev[2]);
    cudaEventElapsedTime(&d, b->ev[2], b->ev[3]);
    b->t_front = a;
    b->t_solve = c2;
    b->t_back = d;
  }
  // results: joint eigensolve
  SolveGraph sgc = b->sg;
  sgc.build = false;
  sgc.collect = true;
  cudaError_t err0 = cudaSuccess;
  zd* Xout = mc->ws.get<zd>("b_Xout", (size_t)b->L.nrow * b->nev, &err0);
  double* diag = mc->ws.get<double>("b_diag", b->L.nrow, &err0);
  rc = lobpcg_solve_batch<float>(*b->op, diag, b->L, b->nev, b->m, b->tol, b->maxit, mc->ws, mc->st, mc->s, &Eall,
                                 Xout, &stats, &sst, &msg, b->tol_refine, &sgc);
  }
  const auto t3 = std::chrono::steady_clock::now();
  // set-up status of every system, oscillator strengths
  cudaError_t err = cudaSuccess;
  std::vector<double> osc((size_t)nsys * 8 * b->nev, 0.0);
  double* dosc = mc->ws.get<double>("b_osc", osc.size(), &err);
  if (err != cudaSuccess || cudaMemcpy(osc.data(), dosc, sizeof(double) * osc.size(), cudaMemcpyDeviceToHost) != cudaSuccess) {
    for (int q = 0; q < nsys; ++q) status[q] = WTB_ECUDA;
    return finish(WTB_ECUDA);
  }
  // a failure of the whole solve (device status, launch) reaches every system; else each has its own status
  bool any_sys = false;
  for (int v : sst) any_sys = any_sys || v != WTB_OK;
  const bool global_fail = rc != WTB_OK && !any_sys;
  bool first_msg = true;
  for (int q = 0; q < nsys; ++q) {
    wtb_ctx* c = b->slots[q];
    int r = ctx_check_status(c);  // set-up kernels of the system (band window checks)
    std::string why = r != WTB_OK ? std::string(wtb_last_error(c)) : std::string();
    if (r == WTB_OK && global_fail) {
      r = rc;
      why = msg;
    } else if (r == WTB_OK && q < (int)sst.size() && sst[q] != WTB_OK) {
      r = sst[q];
      why = first_msg ? msg : "eigensolver failed with status " + std::to_string(r);
      first_msg = false;
    }
    status[q] = r;
    if (iterations) iterations[q] = q < (int)stats.size() ? stats[q].iterations : 0;
    if (r != WTB_OK) {
      b->errors[q] = why;
      if (first_bad == WTB_OK) first_bad = r;
      continue;
    }
    const int nev = p[q].nev;
    if (E)
      for (int n = 0; n < nev; ++n) E[(size_t)q * nev_stride + n] = Eall[(size_t)q * b->nev + n];
    if (act)
      for (int a = 0; a < 8; ++a)
        for (int n = 0; n < nev; ++n)
          act[((size_t)q * 8 + a) * nev_stride + n] = osc[((size_t)q * 8 + a) * b->nev + n];
    c->have_solve = false;  // the slot holds no single-system solve for the backward pass
  }
  if (ctx_check_status(mc) != WTB_OK && first_bad == WTB_OK) first_bad = WTB_ECUDA;
  b->t_collect = ms_since(t3);
  return finish(first_bad);
}

extern "C" int wtb_batch_timings(const wtb_batch* b, double* t_ms) {
  if (!b || !t_ms) return WTB_EBADARG;
  t_ms[0] = b->t_stage;
  t_ms[1] = b->t_build;
  t_ms[2] = b->t_run;
  t_ms[3] = b->t_collect;
  t_ms[4] = b->t_front;
  t_ms[5] = b->t_solve;
  t_ms[6] = b->t_back;
  return WTB_OK;
}

// The joint operator of the last batch call (its accurate arithmetic, as in the final Rayleigh-Ritz) applied to
// ncol vectors of every system: X and Y hold, system after system, dim_q x ncol complex(8) column-major blocks.
extern "C" int wtb_batch_matvec(wtb_batch* b, int ncol, const double* X, double* Y) {
  if (!b || !b->op || ncol < 1 || ncol > b->op->nbmax || !X || !Y) return WTB_EBADARG;
  wtb_ctx* mc = b->main;
  const int nsys = (int)b->dims.size();
  const long nrow = b->L.nrow;
  std::vector<zf> hx((size_t)nrow * ncol, mk<float>(0.f, 0.f)), hy((size_t)nrow * ncol);
  long off = 0;
  for (int q = 0; q < nsys; ++q) {
    const int dim = b->dims[q];
    for (int j = 0; j < ncol; ++j)
      for (int i = 0; i < dim; ++i) {
        const double* z = X + 2 * (off + (size_t)j * dim + i);
        hx[(size_t)(b->row0[q] + i) * ncol + j] = mk<float>((float)z[0], (float)z[1]);
      }
    off += (long)dim * ncol;
  }
  cudaError_t err = cudaSuccess;
  zf* dx = mc->ws.get<zf>("bmv_x", hx.size(), &err);
  zf* dy = mc->ws.get<zf>("bmv_y", hx.size(), &err, true);
  if (err != cudaSuccess) return WTB_ENOMEM;
  if (cudaMemcpyAsync(dx, hx.data(), sizeof(zf) * hx.size(), cudaMemcpyHostToDevice, mc->s) != cudaSuccess)
    return WTB_ECUDA;
  b->op->set_final(true);
  cudaError_t e = b->op->apply(dx, ncol, 0, ncol, dy, ncol, mc->s);
  b->op->set_final(false);
  if (e != cudaSuccess || cudaMemcpyAsync(hy.data(), dy, sizeof(zf) * hy.size(), cudaMemcpyDeviceToHost, mc->s) != cudaSuccess ||
      cudaStreamSynchronize(mc->s) != cudaSuccess)
    return WTB_ECUDA;
  off = 0;
  for (int q = 0; q < nsys; ++q) {
    const int dim = b->dims[q];
    for (int j = 0; j < ncol; ++j)
      for (int i = 0; i < dim; ++i) {
        const zf v = hy[(size_t)(b->row0[q] + i) * ncol + j];
        Y[2 * (off + (size_t)j * dim + i)] = v.re;
        Y[2 * (off + (size_t)j * dim + i) + 1] = v.im;
      }
    off += (long)dim * ncol;
  }
  return ctx_check_status(mc);
}
