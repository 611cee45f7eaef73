// The context behind the C ABI's wtb_ctx handle: one device, one stream, the state the Fortran modules kept
// in globals (H(R), the bands of the last mesh) and the device buffers of the last solve.
#pragma once
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "solver.h"

struct wtb_ctx {
  int device = 0;
  cudaStream_t s = nullptr;
  std::string msg;
  wtb::DevStatus* st = nullptr;
  wtb::Workspace ws;
  // H(R)
  bool have_hr = false;
  int w = 0, nR = 0, systype_np = 0;
  double efermi = 0.0, scs = 0.0;
  double rlat_rm[9] = {0};
  // bands of the last mesh
  bool have_bands = false;
  int nk = 0, nv = 0, nc = 0;
  int ngrid[3] = {0, 0, 0};
  std::vector<double> kpt;  // nk x 3 row-major
  // the k-points are the Monkhorst-Pack mesh of ngrid (set by the solver entry points); a caller-supplied
  // k-point list (wtb_eigsys_mesh) clears it and the V(k,k') table is then evaluated pair by pair
  bool mesh_mp = false;
  // last BSE operator data (for wtb_optsp)
  bool have_hr_optics = false;
  // contraction form of the last operator built (WTB_FORM_*)
  int last_form = 0;
  wtb::KernelProfile prof;
  // the last wtb_bsesolver call (for wtb_bse_backward): its parameters and exciton energies
  bool have_solve = false;
  wtb_bse_params last_p{};
  std::vector<double> last_E;
};


namespace wtb {
// The BSE operator selected by p (dense FP64/FP32, or matrix-free FP64/FP32/split-BF16) over the bands of
// the context; exactly one of o64 / o32 is set.
struct OpBundle {
  std::unique_ptr<Operator<double>> o64;
  std::unique_ptr<Operator<float>> o32;
  std::string msg;
  const double* dE = nullptr;
  int dim = 0;
};


// Shared helpers of the C ABI translation units (defined in wtb_api.cu).
int ctx_set_err(wtb_ctx* c, int code, const std::string& m);
int ctx_check_status(wtb_ctx* c);
double ctx_vcell3d(const wtb_ctx* c);  // |a1 . (a2 x a3)| of the lattice (vcell3D)
CoulParams ctx_coul_params(wtb_ctx* c, const wtb_bse_params* p);
int ctx_coulomb_table(wtb_ctx* c, const wtb_bse_params* p, double* V, int ldv, bool deriv_r0);
int ctx_make_operator(wtb_ctx* c, const wtb_bse_params* p, int nbmax, OpBundle* ob, const std::string& tag,
                      bool deriv_r0);
int ctx_stage_system(wtb_ctx* c, const wtb_bse_params* p);
int ctx_enqueue_system(wtb_ctx* c, const wtb_bse_params* p, int nbmax, OpBundle* ob);
int ctx_auto_block(const wtb_bse_params* p, int dim, bool fp64);
}  // namespace wtb
