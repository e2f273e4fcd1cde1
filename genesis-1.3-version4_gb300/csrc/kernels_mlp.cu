// BF16 tensor-core kernels of the learned coarse-step closure: a small MLP
// (inputs -> 256 -> 256 -> 256 -> outputs) evaluated and trained on the GPU.
//
// GEMM: C[M][N] = sum_k A[M][k] B[N][k] ("NT": both operands row-major with the
// reduction index last), BF16 operands, FP32 accumulation, on the 5th-generation
// tensor cores (k_gemm_tc): a CTA computes a 128 x BN tile (BN <= 128, a multiple of
// 16 dividing N) with its accumulator in tensor memory (TMEM). The reduction runs in
// stages of 64 through a ring of three stage buffers. One thread drives the ring: it
// loads a stage's tiles with TMA tensor copies (cp.async.bulk.tensor, completing on
// the buffer's "full" mbarrier), issues the stage's four MMAs (tcgen05.mma, K = 16
// each) once they have landed, commits them to the buffer's "empty" mbarrier
// (tcgen05.commit), and refills a buffer only after its MMAs have completed. The
// eight warps then read the accumulator back (tcgen05.ld), a quarter of the rows and
// half of the columns each, for the bias / ReLU epilogue. Every GEMM of the network
// takes it: the forward layers, dA = dZ W, and the weight gradients dW = dZ^T A,
// whose reduction runs over the batch rows (the transposed operands are zero-padded
// to a multiple of 16 rows).
#include <cuda.h>          // CUtensorMap and its enumerations
#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled_v12000
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "g4gpu_internal.h"

namespace g4 {
namespace {

// ---- k_gemm_tc: tcgen05 MMA with the accumulator in tensor memory --------------
constexpr int kTcM = 128;        // tile rows: the accumulator's 128 TMEM lanes
constexpr int kTcKC = 64;        // reduction elements per stage (8 chunks of 16 bytes)
constexpr int kTcStages = 3;     // stage buffers in the ring
constexpr int kTcMaxN = 128;     // tile columns (TMEM columns of the FP32 accumulator)
constexpr int kTcThreads = 256;  // two warpgroups; each reads half the columns back
constexpr long long kTcSpin = 1LL << 22;  // bounded mbarrier polls
// Shared memory of a CTA: 1 KB of alignment slack, kTcStages x (A stage 16 KB + B
// stage BN x 128 B), a full and an empty mbarrier per stage, the TMEM address, the
// verdict of the driving thread and the tile's BN biases. At BN = 128 that is 97 KB, so at most two CTAs
// share an SM and their accumulators (<= 128 TMEM columns each) always fit its 512
// columns; smaller tiles are padded to kTcMinSmem for the same bound (at most 3 CTAs
// per SM), so no TMEM allocation waits for another CTA.
constexpr size_t kTcMinSmem = 60 * 1024;

// A stage buffer holds each operand chunk-major: the 16-byte chunk c (elements
// 8c .. 8c + 7 of the stage's reduction range) of all R rows of the tile lies in
// R x 16 contiguous bytes at c R 16, row r at + 16 r, which is what one TMA copy of a
// box of 8 elements x R rows writes. Its 8 x 16-byte core matrices (8 rows of one
// chunk) are therefore 128 B apart along the rows (the descriptors' stride byte
// offset) and R x 16 B apart along the reduction (the leading byte offset).
__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t addr, uint32_t lbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)(128u >> 4) << 32) | (1ull << 46);  // version 1 (bits 46-48 = 0b001); no swizzle
}

// Instruction descriptor of tcgen05.mma kind::f16: D in F32 (bits 4-5 = 1), A and B
// BF16 (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N / 8 at bit 17,
// M / 16 at bit 24.
__device__ __forceinline__ uint32_t tc_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// TMA tensor copy of the box at (x, y) of the 2-D map (x: element along the
// reduction, a multiple of 8, so 16-byte aligned; y: row) into shared memory at dst,
// completing on the mbarrier bar. Rows past the matrix read as zero.
__device__ __forceinline__ void tc_tma(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// two FP32 values rounded to BF16, the first in the low half (the lower address)
__device__ __forceinline__ uint32_t pack_bf2(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t *>(&h);
}

__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity) {
  for (long long it = 0; it < kTcSpin; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// C = A B^T (+ bias[n]) with optional ReLU (and optionally added to C); writes FP32
// C and/or BF16 Cb. A: [M][K] through the tensor map tmA (box 8 x arows, arows 128 or
// M rounded up to 8 when M < 128), B: [N][K] through tmB (box 8 x BN); K a multiple of 16, BN (a multiple of 16 up to kTcMaxN)
// dividing N. kTcThreads threads; CTA (bx, by) computes rows [128 bx, 128 bx + 128)
// and columns [BN by, BN by + BN). If an mbarrier phase is not seen within the
// bounded wait, *err is set, the driving thread waits once more (bounded) for the
// copies and MMAs it issued, the CTA frees its tensor memory and writes nothing.
__global__ void __launch_bounds__(kTcThreads) k_gemm_tc(const __grid_constant__ CUtensorMap tmA,
                                                        const __grid_constant__ CUtensorMap tmB,
                                                        const float *__restrict__ bias, float *C, __nv_bfloat16 *Cb,
                                                        int M, int N, int K, int BN, int arows, int relu,
                                                        int accumulate, int *err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  const uint32_t base = ((uint32_t)__cvta_generic_to_shared(tc_smem) + 1023u) & ~1023u;
  const uint32_t a_bytes = kTcM * kTcKC * 2, stage_bytes = a_bytes + (uint32_t)BN * kTcKC * 2;
  const uint32_t sfull = base + kTcStages * stage_bytes, sempty = sfull + 8 * kTcStages;
  const uint32_t sadr = sempty + 8 * kTcStages, sok = sadr + 4;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kTcM, n0 = blockIdx.y * BN;
  // the tile's bias, staged while the reduction runs: the epilogue then reads shared
  // memory instead of waiting on a global load per group of columns
  float *sbias = reinterpret_cast<float *>(tc_smem + (sok + 4 - (uint32_t)__cvta_generic_to_shared(tc_smem)));
  for (int t = threadIdx.x; t < BN; t += blockDim.x) sbias[t] = bias ? bias[n0 + t] : 0.f;
  uint32_t ncols = 32;  // TMEM columns: a power of two >= 32
  while ((int)ncols < BN) ncols <<= 1;
  if (threadIdx.x == 0) {
    for (int b = 0; b < kTcStages; b++) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sfull + 8 * b) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sempty + 8 * b) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sadr), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  uint32_t tmem;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(tmem) : "r"(sadr) : "memory");
  if (threadIdx.x == 0) {
    const int nk = (K + kTcKC - 1) / kTcKC;
    const uint32_t idesc = tc_idesc(kTcM, BN);
    int issued = 0;    // stages whose copies were issued
    int consumed = 0;  // stages whose copies were seen to land
    int last = -1;     // the last stage whose MMAs were committed
    auto issue = [&](int j) {
      const uint32_t sa = base + (uint32_t)(j % kTcStages) * stage_bytes, sb = sa + a_bytes;
      const uint32_t bar = sfull + 8 * (j % kTcStages);
      const int k0 = j * kTcKC, nc = min(kTcKC, K - k0) / 8;
      const uint32_t bytes = (uint32_t)nc * (uint32_t)(arows + BN) * 16u;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
      for (int c = 0; c < nc; c++) {
        tc_tma(sa + (uint32_t)c * (kTcM * 16), &tmA, k0 + 8 * c, m0, bar);
        tc_tma(sb + (uint32_t)c * (uint32_t)(BN * 16), &tmB, k0 + 8 * c, n0, bar);
      }
      issued = j + 1;
    };
    bool ok = true;
    for (int j = 0; j < kTcStages && j < nk; j++) issue(j);
    for (int kc = 0; kc < nk; kc++) {
      const int b = kc % kTcStages;
      if (!(ok = tc_wait(sfull + 8 * b, (kc / kTcStages) & 1))) break;
      consumed = kc + 1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sa = base + (uint32_t)b * stage_bytes, sb = sa + a_bytes;
      const int ks = min(kTcKC, K - kc * kTcKC) / 16;
      for (int s = 0; s < ks; s++) {
        // K step s: chunks 2s and 2s + 1 of every row
        const uint64_t ad = tc_smem_desc(sa + (uint32_t)(2 * s) * (kTcM * 16), kTcM * 16);
        const uint64_t bd = tc_smem_desc(sb + (uint32_t)(2 * s) * (uint32_t)(BN * 16), (uint32_t)BN * 16u);
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(kc | s)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       sempty + 8 * b)
                   : "memory");
      last = kc;
      // refill the buffer of stage kc - 1 once its MMAs have completed
      const int nx = kc - 1 + kTcStages;
      if (kc >= 1 && nx < nk) {
        if (!(ok = tc_wait(sempty + 8 * ((kc - 1) % kTcStages), ((kc - 1) / kTcStages) & 1))) break;
        issue(nx);
      }
    }
    if (ok && last >= 0) ok = tc_wait(sempty + 8 * (last % kTcStages), (last / kTcStages) & 1);
    if (!ok) {
      atomicExch(err, 1);
      // the copies still in flight and the MMAs issued finish before the CTA leaves
      for (int j = consumed; j < issued; j++) tc_wait(sfull + 8 * (j % kTcStages), (j / kTcStages) & 1);
      if (last >= 0) tc_wait(sempty + 8 * (last % kTcStages), (last / kTcStages) & 1);
    }
    asm volatile("st.shared.b32 [%0], %1;" ::"r"(sok), "r"(ok ? 1 : 0) : "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  uint32_t ok;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(ok) : "r"(sok) : "memory");
  if (ok) {
    // warp w reads TMEM lanes [32 (w % 4), 32 (w % 4) + 32), the rows of the tile its
    // position in the warpgroup gives it access to, and the columns of half w / 4
    const int quarter = warp & 3, half = warp >> 2;
    const int r = m0 + quarter * 32 + lane;
    const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16);
    for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 8) {
      uint32_t v[8];
      // the load and its wait in one statement: no use of v can be placed between them
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n"
          "tcgen05.wait::ld.sync.aligned;\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
          : "r"(trow + (uint32_t)c0)
          : "memory");
      if (r < M) {
        const int c = n0 + c0;
        float o[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
          float x = __uint_as_float(v[j]);
          if (accumulate && C) x += C[(size_t)r * N + c + j];
          if (bias) x += sbias[c0 + j];
          if (relu) x = fmaxf(x, 0.f);
          o[j] = x;
        }
        if (C) {
          float4 *d = reinterpret_cast<float4 *>(C + (size_t)r * N + c);
          d[0] = make_float4(o[0], o[1], o[2], o[3]);
          d[1] = make_float4(o[4], o[5], o[6], o[7]);
        }
        if (Cb)
          *reinterpret_cast<uint4 *>(Cb + (size_t)r * N + c) =
              make_uint4(pack_bf2(o[0], o[1]), pack_bf2(o[2], o[3]), pack_bf2(o[4], o[5]), pack_bf2(o[6], o[7]));
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
}

// out[c][r] = in[r][c] for a rows x cols bf16 matrix; out has ldo >= rows columns,
// the ones past rows set to zero (the zero padding of a reduction over rows)
__global__ void k_transpose_bf16(const __nv_bfloat16 *in, __nv_bfloat16 *out, int rows, int cols, int ldo) {
  __shared__ __nv_bfloat16 tile[32][33];
  int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int r = by + j, c = bx + threadIdx.x;
    if (r < rows && c < cols) tile[j][threadIdx.x] = in[(size_t)r * cols + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int c = bx + j, r = by + threadIdx.x;
    if (r < ldo && c < cols) out[(size_t)c * ldo + r] = r < rows ? tile[threadIdx.x][j] : __float2bfloat16(0.f);
  }
}

__global__ void k_f32_to_bf16(const float *in, __nv_bfloat16 *out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16(in[i]);
}

// dZ = dA * (Z > 0) for a ReLU layer; writes FP32 and BF16 copies
__global__ void k_relu_backward(const float *dA, const float *Z, float *dZ, __nv_bfloat16 *dZb, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float v = Z[i] > 0.f ? dA[i] : 0.f;
    dZ[i] = v;
    dZb[i] = __float2bfloat16(v);
  }
}

// column sums: db[c] = sum_r dZ[r][c]
__global__ void k_colsum(const float *dZ, float *db, int rows, int cols) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; r++) s += dZ[(size_t)r * cols + c];
  db[c] = s;
}

// mean squared error over valid rows and the first `nout` columns of Y (ld = ldy);
// dY = 2 (Y - T) / (rows * nout); loss accumulated into *loss
__global__ void k_mse(const float *Y, const float *T, float *dY, __nv_bfloat16 *dYb, int rows, int nout,
                      int ldy, float *loss) {
  size_t n = (size_t)rows * ldy;
  float acc = 0.f;
  float scale = 2.f / ((float)rows * (float)nout);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    int c = (int)(i % ldy);
    float d = 0.f;
    if (c < nout) {
      int r = (int)(i / ldy);
      d = Y[i] - T[(size_t)r * nout + c];
      acc += d * d;
    }
    dY[i] = scale * d;
    dYb[i] = __float2bfloat16(scale * d);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc / ((float)rows * (float)nout));
}

// Adam update of n parameters (FP32 master copy w, moments m and v)
__global__ void k_adam(float *w, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

unsigned blocks_for(size_t n) {
  size_t b = (n + 255) / 256;
  return (unsigned)(b > 4096 ? 4096 : (b ? b : 1));
}

}  // namespace

int mlp_tile_n(int N, int K) {
  if (K < 16 || K % 16 || N < 16 || N % 16) return 0;
  for (int bn = kTcMaxN; bn >= 16; bn -= 16)
    if (N % bn == 0) return bn;
  return 0;
}

// cuTensorMapEncodeTiled from the driver, through the runtime (no link against
// libcuda); null if the driver does not provide it
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// The 2-D tensor map of a row-major BF16 matrix of `rows` rows of K elements (K a
// multiple of 8: 16-byte aligned rows), read in boxes of 8 elements x box_rows rows,
// zero outside the matrix.
bool bf16_map(CUtensorMap *map, const void *ptr, int K, int rows, int box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(ptr) & 15)) return false;
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  cuuint32_t box[2] = {8, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int mlp_gemm_nt(void *stream, const void *A, const void *B, const float *bias, float *C, void *Cb, int M, int N,
                int K, int relu, int accumulate, int *err) {
  int bn = mlp_tile_n(N, K);
  if (M <= 0 || !bn) return -1;
  // narrower tiles while the grid would leave most SMs idle: these GEMMs are
  // latency-bound, and a narrower tile stages less of B per CTA
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) nsm = 1;
  }
  const long long mtiles = (M + kTcM - 1) / kTcM;
  while (bn % 32 == 0 && bn >= 64 && mtiles * (N / bn) < nsm) bn /= 2;
  // A's box spans the tile's 128 rows (rows past M read as zero), or, for fewer rows
  // than a tile, those rows rounded up to 8 (the tile's other accumulator rows then
  // hold whatever the stage buffers held and are not written out)
  const int arows = M >= kTcM ? kTcM : (M + 7) / 8 * 8;
  CUtensorMap ma, mb;
  if (!bf16_map(&ma, A, K, M, arows) || !bf16_map(&mb, B, K, N, bn)) return -2;
  size_t smem = 1024 + (size_t)kTcStages * (kTcM + bn) * kTcKC * 2 + 16 * kTcStages + 8 + 4 * (size_t)bn;
  if (smem < kTcMinSmem) smem = kTcMinSmem;
  static size_t smem_set = 0;  // the largest dynamic shared memory granted so far
  if (smem > smem_set) {
    cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    smem_set = smem;
  }
  dim3 grid((M + kTcM - 1) / kTcM, N / bn);
  k_gemm_tc<<<grid, kTcThreads, smem, (cudaStream_t)stream>>>(ma, mb, bias, C, (__nv_bfloat16 *)Cb, M, N, K, bn,
                                                             arows, relu, accumulate, err);
  return 0;
}

void mlp_transpose_bf16(void *stream, const void *in, void *out, int rows, int cols, int ldo) {
  dim3 grid((cols + 31) / 32, (ldo + 31) / 32);
  k_transpose_bf16<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)in,
                                                                  (__nv_bfloat16 *)out, rows, cols, ldo);
}

void mlp_to_bf16(void *stream, const float *in, void *out, size_t n) {
  k_f32_to_bf16<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(in, (__nv_bfloat16 *)out, n);
}

void mlp_relu_backward(void *stream, const float *dA, const float *Z, float *dZ, void *dZb, size_t n) {
  k_relu_backward<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(dA, Z, dZ, (__nv_bfloat16 *)dZb, n);
}

void mlp_colsum(void *stream, const float *dZ, float *db, int rows, int cols) {
  k_colsum<<<(cols + 127) / 128, 128, 0, (cudaStream_t)stream>>>(dZ, db, rows, cols);
}

void mlp_mse(void *stream, const float *Y, const float *T, float *dY, void *dYb, int rows, int nout, int ldy,
             float *loss) {
  k_mse<<<blocks_for((size_t)rows * ldy), 256, 0, (cudaStream_t)stream>>>(Y, T, dY, (__nv_bfloat16 *)dYb, rows,
                                                                          nout, ldy, loss);
}

void mlp_adam(void *stream, float *w, const float *g, float *m, float *v, size_t n, float lr, float b1,
              float b2, float eps, int t) {
  float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
  k_adam<<<blocks_for(n), 256, 0, (cudaStream_t)stream>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2);
}

}  // namespace g4
