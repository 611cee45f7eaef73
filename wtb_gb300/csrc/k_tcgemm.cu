// Split-BF16 tensor-core contraction T = V Z for the matrix-free BSE operator (sm_103a, tcgen05).
//
//   C[M][N] (fp32) = sum_{pairs (sa,sb)} A_sa[M][K] * B_sb[N][K]^T
// A = slices of the real V(k,k') table, B = slices of the gathered Z panel, both K-major bf16 with
// x = x_0 + x_1 (+ x_2) and every part rounded to bfloat16.  The slice pairs whose product order is
// <= 2^-8 (bf16x3: (0,0),(0,1),(1,0)) or <= 2^-16 (bf16x6: + (0,2),(1,1),(2,0)) are accumulated into the
// same FP32 accumulator, which gives roughly 16 or 24 significant bits in the products.
//
// CTA tile 128 x 256, K step 64 (one 128-byte swizzle atom of bf16), 4-stage TMA pipeline:
//   warp 0 lane 0   TMA producer (cp.async.bulk.tensor.3d, mbarrier complete_tx)
//   warp 1 lane 0   MMA issuer (tcgen05.mma.cta_group::1.kind::f16, two 256-column accumulators in TMEM)
//   warp 2          TMEM allocator
//   warps 4..7      epilogue (tcgen05.ld 32x32b, lane = row) -> fp32 rows in global memory
// Every mbarrier wait is bounded (2 s of %globaltimer); a wait that gives up sets the device status
// word and an abort flag, the other roles stop at their next wait, and TMEM is freed before exit.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>
#include <utility>

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdlib>

#include "wtb_internal.h"

namespace wtb {

namespace {

constexpr int BM = 128, BK = 64;
constexpr int A_BYTES = BM * BK * 2;
constexpr unsigned long long kTimeoutNs = 2000000000ull;
// Column tile BN (256 or 128, chosen per operator shape by the autotuner): the pipeline depth fills the same
// shared memory with either.
template <int BN_>
struct TcShape {
  static constexpr int BN = BN_;
  static constexpr int STAGES = BN_ == 256 ? 4 : 6;
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  // room for two FP32 accumulators of BN columns: in split runs even K blocks go to the first, odd ones to
  // the second, and the epilogue adds them (halves the number of MMA accumulation steps each one takes)
  static constexpr int TMEM_COLS = 2 * BN;
  static constexpr uint32_t IDESC = (1u << 4)                       // D format: f32
                                    | (1u << 7)                     // A format: bf16
                                    | (1u << 10)                    // B format: bf16
                                    | ((uint32_t)(BN >> 3) << 17)   // N / 8
                                    | ((uint32_t)(BM >> 4) << 24);  // M / 16
  static constexpr size_t SMEM = (size_t)STAGES * STAGE_BYTES + 1024 + 256;
};

struct TcArgs {
  int K, kblocks, m_valid, n_valid, ldc, npairs;
  int kb0, kbn;    // this launch covers K blocks [kb0, kb0 + kbn)
  int accumulate;  // 1: C += result (a later K range of a split run), 0: C = result
  int dual;        // 1: even/odd K blocks in two accumulators (split runs), 0: one accumulator
  int pa[8], pb[8];
  float* C;
  DevStatus* st;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase; false if it gave up (timeout or abort raised by another role).
__device__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (globaltimer() - t0 > kTimeoutNs) return false;
  }
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

// B operand: the Z panel is stored in 64-wide K blocks, zt[slice][kb][n][64], so that the rows of one K block
// are adjacent in memory (the gather writes them side by side); the 4-D box {64, rows, 1, 1} lands in shared
// memory exactly as a K-major 64 x rows tile of a plain [n][K] panel would.
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

// UMMA shared-memory descriptor: K-major, 128-byte swizzle, 8-row core groups 1024 bytes apart.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;              // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset
  d |= (uint64_t)1 << 46;              // descriptor version
  d |= (uint64_t)2 << 61;              // SWIZZLE_128B
  return d;
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// One 128 x 256 output tile at (m0, n0) of the product described by args, operands through the tensor maps
// (kernel parameter or global memory).
template <int BN_>
__device__ __forceinline__ void tc_gemm_tile(const CUtensorMap* mapA_p, const CUtensorMap* mapB_p,
                                             const TcArgs& args, int m0, int n0) {
  using Sh = TcShape<BN_>;
  constexpr int BN = Sh::BN, STAGES = Sh::STAGES, STAGE_BYTES = Sh::STAGE_BYTES, TMEM_COLS = Sh::TMEM_COLS;
  constexpr uint32_t kIdesc = Sh::IDESC;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const CUtensorMap& mapA = *mapA_p;
  const CUtensorMap& mapB = *mapB_p;
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    abort_flag[0] = 0;
    abort_flag[1] = 0;
    abort_flag[2] = 0;
    abort_flag[3] = 0;  // never raised: lets a drain wait run to its own time limit
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapB)) : "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const int total = args.npairs * args.kbn;

  volatile int* issued = abort_flag + 1;    // TMA stages issued by the producer
  volatile int* consumed = abort_flag + 2;  // stages whose loads the MMA issuer has seen land
  if (warp == 0) {
    if (lane == 0) {
      for (int it = 0; it < total; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
        if (it >= STAGES && !mbar_wait(&empty[s], ph ^ 1u, abort_flag)) {
          *abort_flag = 1;
          dev_fail(args.st, 401, it);
          break;
        }
        const int pair = it / args.kbn, kb = args.kb0 + it % args.kbn;
        uint8_t* sa = base + s * STAGE_BYTES;
        uint8_t* sb = sa + A_BYTES;
        mbar_expect_tx(&full[s], STAGE_BYTES);
        tma_load_3d(sa, &mapA, &full[s], kb * BK, m0, args.pa[pair]);
        tma_load_4d(sb, &mapB, &full[s], 0, n0, kb, args.pb[pair]);
        *issued = it + 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      for (int it = 0; it < total; ++it) {
        const int s = it % STAGES;
        const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
        if (!mbar_wait(&full[s], ph, abort_flag)) {
          *abort_flag = 1;
          dev_fail(args.st, 402, it);
          break;
        }
        *consumed = it + 1;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t sa = smem_u32(base + s * STAGE_BYTES);
        const uint32_t sb = sa + A_BYTES;
        const uint64_t da = sw128_desc(sa), db = sw128_desc(sb);
        const int kl = it % args.kbn;  // K block within this launch's range
        const int ai = args.dual ? (kl & 1) : 0;  // accumulator of this K block
        const uint32_t acc_col = (uint32_t)(ai * BN);
        const bool first = args.dual ? (it < 2 && kl == it) : (it == 0);  // its first block in pair 0
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk) {
          // advance 16 bf16 = 32 bytes along K inside the swizzle atom: +2 in the encoded address
          umma_bf16(tmem + acc_col, da + (uint64_t)(2 * kk), db + (uint64_t)(2 * kk), kIdesc,
                    (!first || kk > 0) ? 1u : 0u);
        }
        umma_commit(&empty[s]);
      }
      // commit even after an abort: `done` then completes once the MMAs already issued have finished,
      // so TMEM is never released under a running MMA
      umma_commit(done);
    }
  } else if (warp >= 4) {
    bool ok = mbar_wait(done, 0, abort_flag);
    if (!ok && *abort_flag) ok = mbar_wait(done, 0, abort_flag + 3) && false;  // drain issued MMAs, no writes
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok || *abort_flag) {
      if (lane == 0) dev_fail(args.st, 403, warp);
    } else {
      const int wq = warp & 3;
      const int row = m0 + wq * 32 + lane;
      const uint32_t lane_addr = tmem + ((uint32_t)(wq * 32) << 16);
      const bool two = args.dual && args.kbn > 1;  // the second accumulator holds the odd K blocks
#pragma unroll 1
      for (int j = 0; j < BN / 32; ++j) {
        uint32_t r[32];
        tmem_ld32(lane_addr + (uint32_t)(j * 32), r);
        if (two) {
          uint32_t r2[32];
          tmem_ld32(lane_addr + (uint32_t)(BN + j * 32), r2);
#pragma unroll
          for (int q = 0; q < 32; ++q) r[q] = __float_as_uint(__uint_as_float(r[q]) + __uint_as_float(r2[q]));
        }
        const int col0 = n0 + j * 32;
        if (row < args.m_valid) {
          float* dst = args.C + (size_t)row * args.ldc + col0;
          if (col0 + 32 <= args.n_valid) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              float4 v = make_float4(__uint_as_float(r[4 * q]), __uint_as_float(r[4 * q + 1]),
                                     __uint_as_float(r[4 * q + 2]), __uint_as_float(r[4 * q + 3]));
              if (args.accumulate) {
                const float4 o = reinterpret_cast<const float4*>(dst)[q];
                v.x += o.x;
                v.y += o.y;
                v.z += o.z;
                v.w += o.w;
              }
              reinterpret_cast<float4*>(dst)[q] = v;
            }
          } else {
            for (int q = 0; q < 32; ++q)
              if (col0 + q < args.n_valid) dst[q] = __uint_as_float(r[q]) + (args.accumulate ? dst[q] : 0.f);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (threadIdx.x == 0 && *abort_flag) {
    // let TMA copies still in flight land before the CTA's shared memory is released
    for (int it = *consumed; it < *issued; ++it) mbar_wait(&full[it % STAGES], (uint32_t)(it / STAGES) & 1u, abort_flag + 3);
  }
  if (warp == 2) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

template <int BN>
__global__ void __launch_bounds__(256, 1) tc_gemm_kernel(const __grid_constant__ CUtensorMap mapA,
                                                         const __grid_constant__ CUtensorMap mapB, TcArgs args) {
  tc_gemm_tile<BN>(&mapA, &mapB, args, blockIdx.y * BM, blockIdx.x * BN);
}

// A group of independent products (the operators of a batch of systems): tensor maps and arguments per
// product in global memory (64-byte aligned), one CTA per output tile (product, row tile, column tile).
struct TcGroup {
  CUtensorMap mapA;
  CUtensorMap mapB;
  TcArgs args;
};

// kb_chunk > 0: this launch is range `chunk` of a split run (K blocks [chunk kb_chunk, (chunk + 1) kb_chunk) of
// each product, added to C from the second range on, even and odd K blocks in two accumulators).  Products of
// frozen systems are skipped; the CTA returns before it touches shared memory or TMEM.
template <int BN>
__global__ void __launch_bounds__(256, 1) tc_gemm_grouped_kernel(const TcGroup* __restrict__ groups,
                                                                 const int4* __restrict__ tiles, int npairs,
                                                                 int chunk, int kb_chunk,
                                                                 const int* __restrict__ frozen, DevStatus* st) {
  const int4 t = tiles[blockIdx.x];
  if (frozen && frozen[t.x]) return;
  const TcGroup* g = groups + t.x;
  TcArgs a = g->args;
  a.npairs = npairs;
  a.st = st;
  if (kb_chunk > 0) {
    const int kb0 = chunk * kb_chunk;
    if (kb0 >= a.kblocks) return;
    a.kb0 = kb0;
    a.kbn = min(kb_chunk, a.kblocks - kb0);
    a.accumulate = chunk > 0 ? 1 : 0;
    a.dual = 1;
  } else {
    a.kb0 = 0;
    a.kbn = a.kblocks;
    a.accumulate = 0;
    a.dual = 0;
  }
  tc_gemm_tile<BN>(&g->mapA, &g->mapB, a, t.y * BM, t.z * BN);
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  // a function-local static is initialised once, thread-safely
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    return nullptr;
  }();
  return fn;
}

// B: [slices][K / 64][rows][64] bf16 (K-blocked panel)
bool make_map_kblocked(CUtensorMap* map, const uint16_t* ptr, int K, int rows, int slices, int box_rows,
                       std::string* msg) {
  auto enc = get_encode();
  if (!enc) {
    *msg = "cuTensorMapEncodeTiled unavailable";
    return false;
  }
  cuuint64_t dims[4] = {(cuuint64_t)BK, (cuuint64_t)rows, (cuuint64_t)(K / BK), (cuuint64_t)slices};
  cuuint64_t strides[3] = {(cuuint64_t)BK * 2, (cuuint64_t)BK * 2 * rows, (cuuint64_t)K * 2 * rows};
  cuuint32_t box[4] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1, 1};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<uint16_t*>(ptr), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    *msg = "cuTensorMapEncodeTiled failed with code " + std::to_string((int)r);
    return false;
  }
  return true;
}

bool make_map(CUtensorMap* map, const uint16_t* ptr, int K, int rows, int slices, int box_rows, std::string* msg) {
  auto enc = get_encode();
  if (!enc) {
    *msg = "cuTensorMapEncodeTiled unavailable";
    return false;
  }
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)slices};
  cuuint64_t strides[2] = {(cuuint64_t)K * 2, (cuuint64_t)K * 2 * rows};
  cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<uint16_t*>(ptr), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    *msg = "cuTensorMapEncodeTiled failed with code " + std::to_string((int)r);
    return false;
  }
  return true;
}

}  // namespace

struct TcGemmPlan {
  CUtensorMap mapA, mapB;
  TcArgs args;
  dim3 grid;
  int bn = 256;
};

namespace {
template <int BN>
void launch_tile_kernel(TcGemmPlan* p, const TcArgs& a, cudaStream_t s) {
  tc_gemm_kernel<BN><<<p->grid, 256, TcShape<BN>::SMEM, s>>>(p->mapA, p->mapB, a);
}
cudaError_t raise_limits() {
  cudaError_t e = raise_smem_limit(reinterpret_cast<const void*>(tc_gemm_kernel<256>), TcShape<256>::SMEM);
  if (e == cudaSuccess) e = raise_smem_limit(reinterpret_cast<const void*>(tc_gemm_kernel<128>), TcShape<128>::SMEM);
  if (e == cudaSuccess)
    e = raise_smem_limit(reinterpret_cast<const void*>(tc_gemm_grouped_kernel<256>), TcShape<256>::SMEM);
  if (e == cudaSuccess)
    e = raise_smem_limit(reinterpret_cast<const void*>(tc_gemm_grouped_kernel<128>), TcShape<128>::SMEM);
  return e;
}
}  // namespace

int tc_gemm_available() {
  int dev = 0, major = 0, minor = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  return (major == 10 && minor == 3) ? 1 : 0;
}

// A: [na_slices][M][K] bf16 (M multiple of 128, K multiple of 64); B: [nb_slices][K / 64][N][64] bf16 (N multiple
// of bn, bn = 256 or 128); C: fp32 rows of length ldc; only rows < m_valid and columns < n_valid are written.
int tc_gemm_plan_create(TcGemmPlan** plan, const uint16_t* A, int M, int K, long a_slice_stride, int na_slices,
                        const uint16_t* B, int N, long b_slice_stride, int nb_slices, float* C, int ldc, int npairs,
                        const int* pair_a, const int* pair_b, std::string* msg, int bn) {
  if ((bn != 256 && bn != 128) || M % BM || N % bn || K % BK || npairs < 1 || npairs > 8 || ldc % 4) {
    *msg = "tc_gemm: unsupported shape";
    return WTB_EBADARG;
  }
  if (a_slice_stride != (long)M * K || b_slice_stride != (long)N * K) {
    *msg = "tc_gemm: slices must be contiguous";
    return WTB_EBADARG;
  }
  TcGemmPlan* p = new TcGemmPlan();
  p->bn = bn;
  if (!make_map(&p->mapA, A, K, M, na_slices, BM, msg) || !make_map_kblocked(&p->mapB, B, K, N, nb_slices, bn, msg)) {
    delete p;
    return WTB_ECUDA;
  }
  p->args.K = K;
  p->args.kblocks = K / BK;
  p->args.kb0 = 0;
  p->args.kbn = K / BK;
  p->args.accumulate = 0;
  p->args.dual = 0;
  p->args.ldc = ldc;
  p->args.npairs = npairs;
  for (int i = 0; i < npairs; ++i) {
    p->args.pa[i] = pair_a[i];
    p->args.pb[i] = pair_b[i];
  }
  p->args.C = C;
  p->args.m_valid = M;
  p->args.n_valid = N;
  p->grid = dim3(N / bn, M / BM);
  // per device and thread-safe in the runtime; plans are cached, so this runs once per operator shape
  if (raise_limits() != cudaSuccess) {
    *msg = "tc_gemm: shared memory attribute rejected";
    delete p;
    return WTB_ECUDA;
  }
  *plan = p;
  return WTB_OK;
}

void tc_gemm_set_valid(TcGemmPlan* p, int m_valid, int n_valid) {
  p->args.m_valid = m_valid;
  p->args.n_valid = n_valid;
}

cudaError_t tc_gemm_run(TcGemmPlan* plan, DevStatus* st, cudaStream_t s) {
  plan->args.st = st;
  plan->args.kb0 = 0;
  plan->args.kbn = plan->args.kblocks;
  plan->args.accumulate = 0;
  plan->args.dual = 0;
  if (plan->bn == 128)
    launch_tile_kernel<128>(plan, plan->args, s);
  else
    launch_tile_kernel<256>(plan, plan->args, s);
  ++g_launch_count;
  return cudaGetLastError();
}

// The tensor cores add each MMA's products into the FP32 accumulator with a rounding that does not average
// out over a long K: with a smooth right-hand side and a one-signed V the error of a full-K accumulation
// grows with K and shifts Rayleigh quotients coherently.  This run splits K into ranges of kb_chunk blocks
// (one launch each), accumulates each range afresh in TMEM with its even and odd K blocks in two
// accumulators, and adds the results to C in FP32 round-to-nearest in the epilogue, which cuts that error
// by twice the number of ranges.  Launches are ordered on the stream, so the read-modify-write of C is
// race-free.
cudaError_t tc_gemm_run_split(TcGemmPlan* plan, DevStatus* st, cudaStream_t s, int kb_chunk) {
  if (kb_chunk < 1 || kb_chunk > plan->args.kblocks) kb_chunk = plan->args.kblocks;
  plan->args.st = st;
  for (int kb0 = 0; kb0 < plan->args.kblocks; kb0 += kb_chunk) {
    TcArgs a = plan->args;
    a.kb0 = kb0;
    a.kbn = std::min(kb_chunk, plan->args.kblocks - kb0);
    a.accumulate = kb0 > 0 ? 1 : 0;
    a.dual = 1;
    if (plan->bn == 128)
      launch_tile_kernel<128>(plan, a, s);
    else
      launch_tile_kernel<256>(plan, a, s);
    ++g_launch_count;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

void tc_gemm_plan_destroy(TcGemmPlan* plan) { delete plan; }

struct TcGroupPlan {
  TcGroup* d_groups = nullptr;
  int4* d_tiles = nullptr;
  int ntiles = 0;
  int max_kblocks = 0;
  int bn = 256;
  ~TcGroupPlan() {
    if (d_groups) cudaFree(d_groups);
    if (d_tiles) cudaFree(d_tiles);
  }
};

int tc_gemm_group_create(TcGroupPlan** plan, int n, const TcGroupDesc* d, int nslices, int npairs, const int* pair_a,
                         const int* pair_b, std::string* msg, int bn) {
  if (n < 1 || npairs < 1 || npairs > 8 || (bn != 256 && bn != 128)) {
    *msg = "tc_gemm_group: bad arguments";
    return WTB_EBADARG;
  }
  std::vector<TcGroup> h(n);
  std::vector<int4> tiles;
  std::vector<std::pair<int, int>> order;  // (K blocks, product): the longest tiles go first
  for (int i = 0; i < n; ++i) {
    const TcGroupDesc& q = d[i];
    if (q.M % BM || q.N % bn || q.K % BK || q.ldc % 4) {
      *msg = "tc_gemm_group: unsupported shape";
      return WTB_EBADARG;
    }
    std::memset(&h[i], 0, sizeof(TcGroup));
    if (!make_map(&h[i].mapA, q.A, q.K, q.M, nslices, BM, msg) ||
        !make_map_kblocked(&h[i].mapB, q.B, q.K, q.N, nslices, bn, msg))
      return WTB_ECUDA;
    TcArgs& a = h[i].args;
    a.K = q.K;
    a.kblocks = q.K / BK;
    a.kb0 = 0;
    a.kbn = a.kblocks;
    a.m_valid = q.m_valid;
    a.n_valid = q.n_valid;
    a.ldc = q.ldc;
    a.npairs = npairs;
    for (int j = 0; j < npairs; ++j) {
      a.pa[j] = pair_a[j];
      a.pb[j] = pair_b[j];
    }
    a.C = q.C;
    order.emplace_back(a.kblocks, i);
  }
  std::stable_sort(order.begin(), order.end(), [](const std::pair<int, int>& x, const std::pair<int, int>& y) {
    return x.first > y.first;
  });
  int maxkb = 0;
  for (const auto& o : order) {
    const TcGroupDesc& q = d[o.second];
    const int mt = (q.m_valid + BM - 1) / BM, nt = (q.n_valid + bn - 1) / bn;
    for (int y = 0; y < mt; ++y)
      for (int x = 0; x < nt; ++x) tiles.push_back(make_int4(o.second, y, x, 0));
    maxkb = std::max(maxkb, o.first);
  }
  if (raise_limits() != cudaSuccess) {
    *msg = "tc_gemm_group: shared memory attribute rejected";
    return WTB_ECUDA;
  }
  TcGroupPlan* p = new TcGroupPlan();
  if (cudaMalloc(&p->d_groups, sizeof(TcGroup) * n) != cudaSuccess ||
      cudaMalloc(&p->d_tiles, sizeof(int4) * tiles.size()) != cudaSuccess ||
      cudaMemcpy(p->d_groups, h.data(), sizeof(TcGroup) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(p->d_tiles, tiles.data(), sizeof(int4) * tiles.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    delete p;
    *msg = "tc_gemm_group: device allocation failed";
    return WTB_ENOMEM;
  }
  p->ntiles = (int)tiles.size();
  p->max_kblocks = maxkb;
  p->bn = bn;
  *plan = p;
  return WTB_OK;
}

namespace {
void launch_group(TcGroupPlan* plan, int npairs, int chunk, int kb_chunk, const int* frozen, DevStatus* st,
                  cudaStream_t s) {
  if (plan->bn == 128)
    tc_gemm_grouped_kernel<128><<<plan->ntiles, 256, TcShape<128>::SMEM, s>>>(plan->d_groups, plan->d_tiles, npairs,
                                                                               chunk, kb_chunk, frozen, st);
  else
    tc_gemm_grouped_kernel<256><<<plan->ntiles, 256, TcShape<256>::SMEM, s>>>(plan->d_groups, plan->d_tiles, npairs,
                                                                               chunk, kb_chunk, frozen, st);
  ++g_launch_count;
}
}  // namespace

cudaError_t tc_gemm_group_run(TcGroupPlan* plan, int npairs, const int* frozen, DevStatus* st, cudaStream_t s) {
  launch_group(plan, npairs, 0, 0, frozen, st, s);
  return cudaGetLastError();
}

cudaError_t tc_gemm_group_run_split(TcGroupPlan* plan, int npairs, const int* frozen, DevStatus* st, cudaStream_t s,
                                    int kb_chunk) {
  if (kb_chunk < 1) kb_chunk = plan->max_kblocks;
  for (int c = 0; c * kb_chunk < plan->max_kblocks; ++c) {
    launch_group(plan, npairs, c, kb_chunk, frozen, st, s);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

void tc_gemm_group_destroy(TcGroupPlan* plan) { delete plan; }

}  // namespace wtb
