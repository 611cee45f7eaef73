// Batches of independent exciton systems on one GPU.
//
// A system of the strain/mesh scans is small (dim 576..11,664): its solve is a chain of short kernels (one
// graph launch for the eigensolve) that leaves most of the 152 SMs idle.  The batch therefore runs several
// systems at once: every system slot owns a context (its own stream, device buffers, status word and cached
// eigensolver graph), and nworkers host threads take the next system from a queue sorted largest first
// (longest-processing-time order, so the tail of the batch is made of short jobs).  Kernels of different
// systems overlap on the device; nothing is shared between them except the read-only inputs and the
// per-system output slots.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <string>
#include <thread>
#include <vector>

#include "ctx.h"

struct wtb_batch {
  int device = 0;
  int nworkers = 1;
  // one context per system slot: its buffers, stream and cached eigensolver graph persist across calls, so
  // solving the same batch again relaunches each system's graph without capturing it again
  std::vector<wtb_ctx*> slots;
  std::vector<std::string> errors;  // per system of the last call
};

namespace {

double system_cost(const wtb_system& s, const wtb_bse_params& p) {
  const double nk = (double)p.ngrid[0] * p.ngrid[1] * p.ngrid[2];
  return nk * nk * (double)s.w90basis * s.w90basis * std::max(p.nev, 1) + nk * p.nc * p.nv * 1e3;
}

}  // namespace

extern "C" int wtb_batch_create(wtb_batch** out, int device, int nworkers) {
  if (!out || nworkers < 1 || nworkers > 64) return WTB_EBADARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return WTB_ENODEV;
  auto* b = new wtb_batch();
  b->device = device;
  b->nworkers = nworkers;
  *out = b;
  return WTB_OK;
}

extern "C" int wtb_batch_destroy(wtb_batch* b) {
  if (!b) return WTB_OK;
  for (wtb_ctx* w : b->slots) wtb_ctx_destroy(w);
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
  std::vector<int> order(nsys);
  for (int i = 0; i < nsys; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return system_cost(sys[x], p[x]) > system_cost(sys[y], p[y]); });
  while ((int)b->slots.size() < nsys) {
    wtb_ctx* c = nullptr;
    const int r = wtb_ctx_create(&c, b->device);
    if (r != WTB_OK) return r;
    b->slots.push_back(c);
  }
  std::atomic<int> next{0};
  auto work = [&]() {
    std::vector<double> Ws, acts;
    for (int q = next.fetch_add(1); q < nsys; q = next.fetch_add(1)) {
      const int i = order[q];
      wtb_ctx* c = b->slots[i];
      const wtb_system& s = sys[i];
      int r = wtb_set_hr(c, s.w90basis, s.nvec, s.rvec, s.ffactor, s.hopmatrices, s.ihopmatrices, s.rlat, s.efermi,
                         s.scs, s.systype_np);
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
  };
  const int nw = std::min(b->nworkers, std::max(nsys, 1));
  std::vector<std::thread> threads;
  for (int w = 1; w < nw; ++w) threads.emplace_back(work);
  work();
  for (auto& th : threads) th.join();
  if (wall_ms) wall_ms[0] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  for (int i = 0; i < nsys; ++i)
    if (status[i] != WTB_OK) return status[i];
  return WTB_OK;
}
