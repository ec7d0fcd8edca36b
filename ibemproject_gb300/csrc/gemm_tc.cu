// Tensor-core GEMM of the mixed-precision factorisation:  C (FP32) -= A (FP32) * B (FP32)
// on sm_103a with tcgen05 (5th-generation tensor cores, accumulator in tensor memory).
//
// Split-BF16 "x3" scheme: every FP32 operand x is written as hi + lo with hi = bf16(x),
// lo = bf16(x - hi); the product is accumulated in FP32 as hi*hi + hi*lo + lo*hi (the lo*lo
// term, ~2^-16 relative, is dropped).  The result is close to an FP32 GEMM at three BF16
// tensor-core MMAs per product.
//
// Kernel structure (one CTA per 128 x 256 output tile, 128 threads):
//   warp 0, lane 0   TMA producer: 4-stage ring of {A_hi, A_lo (128 x 32), B_hi, B_lo (256 x 32)}
//                    K-major BF16 tiles, 64-byte swizzle, completion on an mbarrier (three
//                    48 KB stages in flight while the fourth is consumed: the loads are
//                    latency-bound, so bytes in flight set the rate)
//   warp 1, lane 0   MMA issuer: per 32-wide K block, 2 x 3 tcgen05.mma.kind::f16 (M=128,
//                    N=256, K=16) into a 128 x 256 FP32 accumulator in TMEM; tcgen05.commit
//                    releases the stage and, at the end, signals the epilogue
//   all 4 warps      epilogue: tcgen05.ld 32x32b (warp w reads TMEM lanes 32w..32w+31 = rows),
//                    C[row, col] -= acc with coalesced column-major accesses
// Every wait on an mbarrier is bounded: on time-out the kernel raises an error flag, stops
// issuing work, still waits (bounded) for the MMAs it issued, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "prof.h"
#include "solver.h"

namespace ibem {
namespace {

constexpr int BM = 128, BN = 256, BK = 32, STAGES = 4;
constexpr int A_TILE = BM * BK * 2;                 // 8 KB
constexpr int B_TILE = BN * BK * 2;                 // 16 KB
constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;  // 48 KB
constexpr int GROUP_M = 16;                         // tile order: groups of 16 row tiles, columns inner
constexpr int TMEM_COLS = 256;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr long long kWaitLimit = 1LL << 22;
constexpr int64_t kMaxKChunk = 8192;  // K is processed in chunks to bound the split workspace

// ---------------------------------------------------------------- split kernels
// A (m x k, column-major, lda) -> hi/lo, K-major rows of length kp: out[i * kp + kk]
__global__ void k_split_a(int64_t m, int64_t k, const float* __restrict__ A, int64_t lda, int64_t kp,
                          __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo) {
  __shared__ float t[32][33];
  const int64_t i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int64_t i = i0 + threadIdx.x, kk = k0 + j;
    t[j][threadIdx.x] = (i < m && kk < k) ? A[kk * lda + i] : 0.0f;
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int64_t i = i0 + j, kk = k0 + threadIdx.x;
    if (i < m && kk < kp) {
      const float v = t[threadIdx.x][j];
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      hi[i * kp + kk] = h;
      lo[i * kp + kk] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
  }
}

// B (k x n, column-major, ldb) -> hi/lo, K-major rows of length kp: out[j * kp + kk]
__global__ void k_split_b(int64_t k, int64_t n, const float* __restrict__ B, int64_t ldb, int64_t kp,
                          __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo) {
  const int64_t kk = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (kk >= kp) return;
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
    const float v = kk < k ? B[j * ldb + kk] : 0.0f;
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    hi[j * kp + kk] = h;
    lo[j * kp + kk] = __float2bfloat16_rn(v - __bfloat162float(h));
  }
}

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
// bounded wait; false (and the error flag raised) on time-out or when another thread failed
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, long long limit = kWaitLimit) {
  for (long long it = 0; it < limit; ++it) {
    if (mbar_test(bar, parity)) return true;
    if ((it & 255) == 255 && *reinterpret_cast<volatile int*>(err) != 0) return false;
  }
  atomicExch(err, 1);
  return false;
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1)
      : "memory");
}
// UMMA shared-memory descriptor: K-major, 64-byte swizzle (rows of BK = 32 BF16), 8-row
// groups 512 B apart
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address (16-byte units)
  d |= (uint64_t)1 << 16;                     // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;            // stride byte offset: 8 rows x 64 B
  d |= (uint64_t)1 << 46;                     // descriptor version for tcgen05
  d |= (uint64_t)4 << 61;                     // SWIZZLE_64B
  return d;
}
// instruction descriptor: kind::f16, D = F32, A = B = BF16, both K-major, M = 128, N = 256
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

#define IBEM_TMEM_LD32(taddr, r)                                                                              \
  asm volatile(                                                                                              \
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "   \
      "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"      \
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),       \
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),  \
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),            \
        "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),            \
        "=r"(r[30]), "=r"(r[31])                                                                             \
      : "r"(taddr))

// ---------------------------------------------------------------- the GEMM kernel
__global__ void __launch_bounds__(128, 1) k_umma_bf16x3(const __grid_constant__ CUtensorMap tAhi,
                                                        const __grid_constant__ CUtensorMap tAlo,
                                                        const __grid_constant__ CUtensorMap tBhi,
                                                        const __grid_constant__ CUtensorMap tBlo,
                                                        float* __restrict__ C, int64_t ldc, int m, int n,
                                                        int kblocks, int* err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + STAGES * STAGE_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 1);
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES), accum = smem_u32(bars + 2 * STAGES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // grouped tile order: consecutive CTAs sweep the column tiles of GROUP_M row tiles, so
  // the CTAs resident at once share A and B panels in L2
  int tm, tn;
  {
    const int tiles_m = (m + BM - 1) / BM, tiles_n = (n + BN - 1) / BN;
    const int b = blockIdx.x, per_group = GROUP_M * tiles_n;
    const int first = (b / per_group) * GROUP_M, gsz = min(GROUP_M, tiles_m - first);
    tm = first + (b % per_group) % gsz;
    tn = (b % per_group) / gsz;
  }
  const int m0 = tm * BM, n0 = tn * BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(accum, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {  // whole warp: allocate the accumulator columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // ---- TMA producer
    int issued[STAGES] = {};
    for (int kb = 0; kb < kblocks; ++kb) {
      const int s = kb % STAGES;
      if (kb >= STAGES && !mbar_wait(empty0 + 8 * s, (uint32_t)((kb / STAGES - 1) & 1), err)) break;
      unsigned char* st = base + s * STAGE_BYTES;
      const uint32_t fb = full0 + 8 * s;
      mbar_expect_tx(fb, STAGE_BYTES);
      tma_load_2d(smem_u32(st), &tAhi, fb, kb * BK, m0);
      tma_load_2d(smem_u32(st + A_TILE), &tAlo, fb, kb * BK, m0);
      tma_load_2d(smem_u32(st + 2 * A_TILE), &tBhi, fb, kb * BK, n0);
      tma_load_2d(smem_u32(st + 2 * A_TILE + B_TILE), &tBlo, fb, kb * BK, n0);
      ++issued[s];
    }
    // copies still in flight (only on an early exit) are waited for, bounded
    for (int s = 0; s < STAGES; ++s)
      if (issued[s]) mbar_wait(full0 + 8 * s, (uint32_t)((issued[s] - 1) & 1), err);
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer
    int done = 0;
    for (int kb = 0; kb < kblocks; ++kb) {
      const int s = kb % STAGES;
      if (!mbar_wait(full0 + 8 * s, (uint32_t)((kb / STAGES) & 1), err)) break;
      tc_fence_after();
      unsigned char* st = base + s * STAGE_BYTES;
      const uint32_t ahi = smem_u32(st), alo = smem_u32(st + A_TILE);
      const uint32_t bhi = smem_u32(st + 2 * A_TILE), blo = smem_u32(st + 2 * A_TILE + B_TILE);
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        const uint32_t off = kk * 32;  // 16 BF16 = 32 bytes along K inside the 64-byte row
        umma(tmem, umma_desc(ahi + off), umma_desc(bhi + off), (kb | kk) != 0);
        umma(tmem, umma_desc(ahi + off), umma_desc(blo + off), 1u);
        umma(tmem, umma_desc(alo + off), umma_desc(bhi + off), 1u);
      }
      umma_commit(empty0 + 8 * s);  // stage s free once these MMAs have read it
      ++done;
    }
    if (done) umma_commit(accum);  // arrives when every MMA issued above has completed
    else mbar_arrive(accum);
  } else if (warp >= 2) {
    // ---- idle warps: bring the C tile into L2 while the MMAs run (one 128-byte line per
    // 32 rows and column; warp 2 takes row groups 0 and 2, warp 3 groups 1 and 3)
    for (int rg = warp - 2; rg < 4; rg += 2) {
      const int rbase = m0 + 32 * rg;
      if (rbase >= m) break;
      for (int c = lane; c < BN; c += 32) {
        const int col = n0 + c;
        if (col < n) asm volatile("prefetch.global.L2 [%0];" ::"l"(C + (int64_t)col * ldc + rbase));
      }
    }
  }
  __syncwarp();

  // ---- epilogue: all 4 warps
  // warp-uniform decision: tcgen05.ld is a warp-collective instruction
  const bool ok = __all_sync(0xffffffffu, mbar_wait(accum, 0, err) && *reinterpret_cast<volatile int*>(err) == 0);
  tc_fence_after();
  if (ok) {
    const int row = m0 + 32 * warp + lane;
    for (int c0 = 0; c0 < BN; c0 += 32) {
      // the 32 loads of C go out before any store, so they overlap each other and the TMEM read
      float cv[32];
      if (row < m) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int col = n0 + c0 + j;
          cv[j] = col < n ? C[(int64_t)col * ldc + row] : 0.0f;
        }
      }
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0;
      IBEM_TMEM_LD32(taddr, r);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < m) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int col = n0 + c0 + j;
          if (col < n) C[(int64_t)col * ldc + row] = cv[j] - __uint_as_float(r[j]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------- host side
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;
bool g_attr_set[64] = {};
std::mutex g_attr_mu;

ibem_status encode_map(CUtensorMap* map, const __nv_bfloat16* ptr, int64_t rows, int64_t k, int64_t kp,
                       uint32_t box_rows) {
  std::call_once(g_encode_once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  if (!g_encode) return fail(IBEM_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  const cuuint64_t dims[2] = {(cuuint64_t)k, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)kp * sizeof(__nv_bfloat16)};
  const cuuint32_t box[2] = {BK, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(ptr), dims, strides,
                        box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(IBEM_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return IBEM_OK;
}

// Self-test of the bounded mbarrier wait: one thread waits, with the same mbar_wait, on a
// freshly initialised barrier that nobody arrives at; the wait must give up and raise err.
__global__ void k_selftest_mbar_wait(int* err, long long limit) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  const uint32_t b = smem_u32(&bar);
  mbar_init(b, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  mbar_wait(b, 0, err, limit);
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(b) : "memory");
}

}  // namespace

ibem_status selftest_mbar_wait(long long limit, cudaStream_t st) {
  if (limit < 1 || limit > kWaitLimit) return fail(IBEM_ERR_ARG, "selftest_mbar_wait: limit outside 1..2^22 polls");
  int* err = nullptr;
  IBEM_CUDA(cudaMalloc(&err, sizeof(int)));
  int h = 0;
  cudaError_t ce = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (ce == cudaSuccess) {
    ::ibem::count_launch(), k_selftest_mbar_wait<<<1, 32, 0, st>>>(err, limit);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  cudaFree(err);
  if (ce != cudaSuccess) return cuda_fail(ce, "selftest_mbar_wait");
  if (h) return fail(IBEM_ERR_TIMEOUT, "selftest_mbar_wait: the bounded wait gave up (expected)");
  return IBEM_OK;
}

size_t gemm_tc_workspace_bytes(int64_t max_m, int64_t max_n) {
  const int64_t kp = kMaxKChunk;
  return (size_t)(max_m + max_n) * kp * 2 * sizeof(__nv_bfloat16) + 256;
}

ibem_status gemm_sub_f32_tc(int64_t m, int64_t n, int64_t k, const float* A, int64_t lda, const float* B,
                            int64_t ldb, float* C, int64_t ldc, void* ws, size_t ws_bytes, int* err,
                            cudaStream_t st) {
  if (m <= 0 || n <= 0 || k <= 0) return IBEM_OK;
  if (m > INT32_MAX || n > INT32_MAX) return fail(IBEM_ERR_ARG, "gemm_tc: dimension too large");
  int dev = 0;
  IBEM_CUDA(cudaGetDevice(&dev));
  {
    std::lock_guard<std::mutex> lock(g_attr_mu);
    if (dev < 64 && !g_attr_set[dev]) {
      IBEM_CUDA(cudaFuncSetAttribute((const void*)k_umma_bf16x3, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     SMEM_BYTES));
      g_attr_set[dev] = true;
    }
  }
  for (int64_t k0 = 0; k0 < k; k0 += kMaxKChunk) {
    const int64_t kc = std::min<int64_t>(kMaxKChunk, k - k0);
    const int64_t kp = (kc + BK - 1) / BK * BK;
    const size_t need = (size_t)(m + n) * kp * 2 * sizeof(__nv_bfloat16);
    if (need > ws_bytes) return fail(IBEM_ERR_ARG, "gemm_tc: workspace too small");
    __nv_bfloat16* ahi = static_cast<__nv_bfloat16*>(ws);
    __nv_bfloat16* alo = ahi + (size_t)m * kp;
    __nv_bfloat16* bhi = alo + (size_t)m * kp;
    __nv_bfloat16* blo = bhi + (size_t)n * kp;
    {
      ProfScope psplit(PROF_GEMM_SPLIT, st);
    ::ibem::count_launch(), k_split_a<<<dim3((unsigned)((m + 31) / 32), (unsigned)(kp / 32)), dim3(32, 8), 0, st>>>(
        m, kc, A + k0 * lda, lda, kp, ahi, alo);
    ::ibem::count_launch(), k_split_b<<<dim3((unsigned)((kp + 255) / 256), (unsigned)std::min<int64_t>(n, 65535)), 256, 0, st>>>(
        kc, n, B + k0, ldb, kp, bhi, blo);
      IBEM_LAUNCH_CHECK("gemm_tc split");
    }
    alignas(64) CUtensorMap maps[4];
    ibem_status s;
    if ((s = encode_map(&maps[0], ahi, m, kc, kp, BM))) return s;
    if ((s = encode_map(&maps[1], alo, m, kc, kp, BM))) return s;
    if ((s = encode_map(&maps[2], bhi, n, kc, kp, BN))) return s;
    if ((s = encode_map(&maps[3], blo, n, kc, kp, BN))) return s;
    dim3 grid((unsigned)(((m + BM - 1) / BM) * ((n + BN - 1) / BN)));
    ProfScope ps(PROF_GEMM_TC, st, 2.0 * m * n * kc);
    ::ibem::count_launch(), k_umma_bf16x3<<<grid, 128, SMEM_BYTES, st>>>(maps[0], maps[1], maps[2], maps[3], C,
                                                                           ldc, (int)m, (int)n, (int)(kp / BK), err);
    IBEM_LAUNCH_CHECK("gemm_tc");
  }
  return IBEM_OK;
}

}  // namespace ibem
