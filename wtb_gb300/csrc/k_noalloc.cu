// Allocation-free variant of the oscillator-strength reduction (dielbsev / dielbsep).
//
// Who needs it: callers that may not allocate device memory themselves -- code whose device memory is
// owned by another allocator (a framework's caching pool or a host program's preallocated arena) and
// loops that must not pay cudaMalloc's implicit device synchronisation.  They pass device pointers for
// every input and output; the partial sums that wtb_dielbse keeps in a context-owned buffer live here
// in a fixed file-scope device array instead.
//
// The array is WTB_NOALLOC_SCRATCH_DOUBLES doubles (2 MiB) on every GPU that loads the library, held
// until the process exits.  Every call on a device shares it and it keeps the last call's contents;
// each call writes every slot it later reads, so nothing needs clearing.  Calls whose work overlaps on
// the GPU (different streams, or different host threads on one device) race on the array: order them.
// The first call on a device looks up the array's device address (cudaGetSymbolAddress, with that
// device current); make that first call before any stream capture.
#include <cstdio>
#include <mutex>
#include <string>

#include "wtb_internal.h"

#define WTB_NOALLOC_SCRATCH_DOUBLES (1 << 18)
#define WTB_NOALLOC_ROWS_PER_BLOCK 1024
#define WTB_NOALLOC_MAX_DEVICES 64

namespace wtb {
namespace {

static __device__ __align__(256) double g_dielbse_scratch[WTB_NOALLOC_SCRATCH_DOUBLES];

// scratch[(n * nblk + b) * 4 + {0..3}] = (Re, Im) of sum over this block's rows of A(j,n) h1(j) and
// A(j,n) h2(j); A column-major (column n contiguous), complex(8).
__global__ void __launch_bounds__(256) dielbse_partial_kernel(const zd* __restrict__ A, int dimse,
                                                              const zd* __restrict__ h1, const zd* __restrict__ h2,
                                                              int pair, int nblk, double* __restrict__ scratch) {
  __shared__ double red[4][256];
  const int b = blockIdx.x, n = blockIdx.y;
  const int r0 = b * WTB_NOALLOC_ROWS_PER_BLOCK;
  const int r1 = min(dimse, r0 + WTB_NOALLOC_ROWS_PER_BLOCK);
  zd s1 = mk<double>(0, 0), s2 = mk<double>(0, 0);
  for (int j = r0 + threadIdx.x; j < r1; j += blockDim.x) {
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
  if (threadIdx.x < 4) scratch[((size_t)n * nblk + b) * 4 + threadIdx.x] = red[threadIdx.x][0];
}

// activity(i) for every row i < dimse: the fixed-order sum of the partials for i < dimse1, zero above.
__global__ void dielbse_final_kernel(const double* __restrict__ scratch, int nblk, int dimse, int dimse1, int pair,
                                     double* __restrict__ act) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dimse) return;
  if (i >= dimse1) {
    act[i] = 0.0;
    return;
  }
  double a1r = 0, a1i = 0, a2r = 0, a2i = 0;
  for (int b = 0; b < nblk; ++b) {
    const double* p = scratch + ((size_t)i * nblk + b) * 4;
    a1r += p[0];
    a1i += p[1];
    a2r += p[2];
    a2i += p[3];
  }
  act[i] = pair ? a1r * a2r + a1i * a2i : a1r * a1r + a1i * a1i;
}

std::mutex g_setup_mu;
double* g_scratch_addr[WTB_NOALLOC_MAX_DEVICES] = {nullptr};

// There is no context to hold a message, so the reason for a rejected call goes to stderr.
int fail(int code, const std::string& m) {
  std::fprintf(stderr, "%s\n", m.c_str());
  return code;
}

}  // namespace
}  // namespace wtb

using namespace wtb;

extern "C" int wtb_dielbse_noalloc(int dimse, int dimse1, const double* excitonvec, const double* hopt1,
                                   const double* hopt2, int pair, double* activity, void* stream) {
  if (dimse < 1 || dimse1 < 0 || dimse1 > dimse || !excitonvec || !hopt1 || (pair && !hopt2) || !activity)
    return fail(WTB_EBADARG, "wtb_dielbse_noalloc: bad arguments");
  // sizes in long before any arithmetic, so no dimse up to INT_MAX can wrap
  const long nblk = ((long)dimse + WTB_NOALLOC_ROWS_PER_BLOCK - 1) / WTB_NOALLOC_ROWS_PER_BLOCK;
  const long final_grid = ((long)dimse + 255) / 256;
  if (nblk * (long)dimse1 * 4 > WTB_NOALLOC_SCRATCH_DOUBLES)
    return fail(WTB_EBADARG, "wtb_dielbse_noalloc: ceil(dimse/1024) * dimse1 * 4 = " +
                                 std::to_string(nblk * (long)dimse1 * 4) + " exceeds the fixed scratch of " +
                                 std::to_string(WTB_NOALLOC_SCRATCH_DOUBLES) + " doubles");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= WTB_NOALLOC_MAX_DEVICES)
    return fail(WTB_ENODEV, "wtb_dielbse_noalloc: no usable current device");
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_addr[dev]) {
      // the array's name is a host-side stand-in; its device address is looked up once per device
      void* ptr = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&ptr, g_dielbse_scratch);
      if (e != cudaSuccess || !ptr)
        return fail(WTB_ECUDA, std::string("wtb_dielbse_noalloc: cudaGetSymbolAddress failed: ") +
                                   cudaGetErrorString(e));
      g_scratch_addr[dev] = static_cast<double*>(ptr);
    }
    scratch = g_scratch_addr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const zd* A = reinterpret_cast<const zd*>(excitonvec);
  const zd* h1 = reinterpret_cast<const zd*>(hopt1);
  const zd* h2 = reinterpret_cast<const zd*>(hopt2);
  if (dimse1 > 0) {
    dielbse_partial_kernel<<<dim3((unsigned)nblk, (unsigned)dimse1), 256, 0, s>>>(A, dimse, h1, h2, pair, (int)nblk,
                                                                                  scratch); ++g_launch_count;
  }
  dielbse_final_kernel<<<(unsigned)final_grid, 256, 0, s>>>(scratch, (int)nblk, dimse, dimse1, pair, activity);
  ++g_launch_count;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(WTB_ECUDA, std::string("wtb_dielbse_noalloc: ") + cudaGetErrorString(e));
  return WTB_OK;
}
