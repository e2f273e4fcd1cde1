// BF16 tensor-core kernels of the learned coarse-step closure: a small MLP
// (inputs -> 256 -> 256 -> 256 -> outputs) evaluated and trained on the GPU.
//
// GEMM: C[M][N] = sum_k A[M][k] B[N][k] ("NT": both operands row-major with the
// reduction index last), BF16 operands, FP32 accumulation. Two kernels:
//
//   k_gemm_tc   the 5th-generation tensor cores (tcgen05): a CTA computes a 128 x BN
//               tile (BN <= 128) with its accumulator in tensor memory. The whole
//               reduction (K <= 256) is staged in shared memory at once, one thread
//               issues the K / 16 MMAs, their completion arrives on an mbarrier, and
//               the four warps read the accumulator back (tcgen05.ld) for the bias /
//               ReLU epilogue. Every GEMM of the forward pass and the dA = dZ W
//               products of the backward pass take it.
//   k_gemm_nt   warp-level mma.sync m16n8k16, 64 x 64 tiles, K staged in chunks of 32:
//               the weight gradients dW = dZ^T A, whose reduction runs over the batch
//               rows (thousands), beyond what k_gemm_tc stages.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "g4gpu_internal.h"

namespace g4 {
namespace {

constexpr int TM = 64, TN = 64, TK = 32;

__device__ __forceinline__ uint32_t pack2(const __nv_bfloat16 *p) {
  return *reinterpret_cast<const uint32_t *>(p);
}

// mma.sync m16n8k16, row.col, bf16 x bf16 -> f32
__device__ __forceinline__ void mma16816(float *d, const uint32_t *a, const uint32_t *b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C = A B^T (+ bias[n]) with optional ReLU; writes FP32 C and/or BF16 Cb.
// A: [M][K] bf16, B: [N][K] bf16, K a multiple of 16 (callers pad).
__global__ void __launch_bounds__(128) k_gemm_nt(const __nv_bfloat16 *__restrict__ A,
                                                 const __nv_bfloat16 *__restrict__ B,
                                                 const float *__restrict__ bias, float *C,
                                                 __nv_bfloat16 *Cb, int M, int N, int K, int relu,
                                                 int accumulate) {
  __shared__ __align__(16) __nv_bfloat16 As[TM][TK + 8];
  __shared__ __align__(16) __nv_bfloat16 Bs[TN][TK + 8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int m0 = blockIdx.x * TM, n0 = blockIdx.y * TN;
  const int g = lane >> 2, t = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[i][j][q] = 0.f;
  for (int k0 = 0; k0 < K; k0 += TK) {
    // stage the 64 x 32 tiles of A and B (zero outside the matrices)
    for (int e = threadIdx.x; e < TM * TK; e += blockDim.x) {
      int r = e / TK, c = e % TK;
      int gm = m0 + r, gk = k0 + c;
      As[r][c] = (gm < M && gk < K) ? A[(size_t)gm * K + gk] : __float2bfloat16(0.f);
      int gn = n0 + r;
      Bs[r][c] = (gn < N && gk < K) ? B[(size_t)gn * K + gk] : __float2bfloat16(0.f);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; kk += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        int r = wm + i * 16 + g;
        af[i][0] = pack2(&As[r][kk + 2 * t]);
        af[i][1] = pack2(&As[r + 8][kk + 2 * t]);
        af[i][2] = pack2(&As[r][kk + 8 + 2 * t]);
        af[i][3] = pack2(&As[r + 8][kk + 8 + 2 * t]);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        int c = wn + j * 8 + g;
        bf[j][0] = pack2(&Bs[c][kk + 2 * t]);
        bf[j][1] = pack2(&Bs[c][kk + 8 + 2 * t]);
      }
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) mma16816(acc[i][j], af[i], bf[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        int r = m0 + wm + i * 16 + g + (q >= 2 ? 8 : 0);
        int c = n0 + wn + j * 8 + 2 * t + (q & 1);
        if (r < M && c < N) {
          float v = acc[i][j][q];
          if (accumulate && C) v += C[(size_t)r * N + c];
          if (bias) v += bias[c];
          if (relu) v = fmaxf(v, 0.f);
          if (C) C[(size_t)r * N + c] = v;
          if (Cb) Cb[(size_t)r * N + c] = __float2bfloat16(v);
        }
      }
}

// ---- k_gemm_tc: tcgen05 MMA with the accumulator in tensor memory --------------
constexpr int kTcM = 128;     // tile rows: the accumulator's 128 TMEM lanes
constexpr int kTcMaxK = 256;  // the reduction is staged whole
constexpr int kTcMaxN = 128;  // tile columns (TMEM columns of FP32 accumulator)
// Shared memory of a CTA at least this large keeps at most 3 CTAs on an SM, so their
// accumulators (<= 128 TMEM columns each) always fit the SM's 512 columns and no
// allocation has to wait for another CTA.
constexpr size_t kTcMinSmem = 60 * 1024;
constexpr long long kTcSpin = 1LL << 22;  // bounded mbarrier polls

// Operand tiles in shared memory are K-major without swizzle: 8 x 16-byte core
// matrices (8 rows of 8 BF16 along K). The core matrix of row group g and K chunk c
// (k / 8) sits at byte (g * K / 8 + c) * 128, its row r % 8 at + 16 (r % 8). In the
// MMA's shared-memory descriptors, core matrices adjacent in K are 128 B apart (the
// leading byte offset) and row groups K * 16 B apart (the stride byte offset).
__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);  // version 1; no swizzle, base offset 0
}

// Instruction descriptor of tcgen05.mma kind::f16: D in F32 (bits 4-5 = 1), A and B
// BF16 (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N / 8 at bit 17,
// M / 16 at bit 24.
__device__ __forceinline__ uint32_t tc_idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Stages rows [r0, r0 + rows) x [0, K) of the row-major matrix X (K columns, nrow
// valid rows; zero past them) into the tile at shared address T with 16-byte
// cp.async copies. Copy idx takes row (idx / (8 K/8)) * 8 + idx % 8 and chunk
// (idx / 8) % (K / 8), which is the tile's byte idx * 16: consecutive threads write
// consecutive 16 bytes.
__device__ __forceinline__ void tc_stage(uint32_t T, const __nv_bfloat16 *__restrict__ X, int r0, int rows, int nrow,
                                         int K) {
  const int ck = K >> 3;
  const int total = rows * ck;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int r = ((idx >> 3) / ck) * 8 + (idx & 7), c = (idx >> 3) % ck;
    const bool ok = r0 + r < nrow;
    const __nv_bfloat16 *src = ok ? X + (size_t)(r0 + r) * K + c * 8 : X;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(T + (uint32_t)idx * 16u), "l"(src),
                 "r"(ok ? 16 : 0)
                 : "memory");
  }
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

// C = A B^T (+ bias[n]) with optional ReLU, as k_gemm_nt, for K a multiple of 16 up
// to kTcMaxK and a tile width BN (a multiple of 16 up to kTcMaxN) dividing N. 128
// threads; CTA (bx, by) computes rows [128 bx, 128 bx + 128) and columns
// [BN by, BN by + BN). Shared memory: A tile (128 x K), B tile (BN x K), the MMA
// mbarrier, the TMEM address. If the MMAs do not complete within the bounded wait,
// *err is set, the CTA waits once more (bounded) so that no MMA still writes the
// accumulator, frees its tensor memory and writes nothing.
__global__ void __launch_bounds__(128) k_gemm_tc(const __nv_bfloat16 *__restrict__ A,
                                                 const __nv_bfloat16 *__restrict__ B,
                                                 const float *__restrict__ bias, float *C, __nv_bfloat16 *Cb,
                                                 int M, int N, int K, int BN, int relu, int accumulate, int *err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  const uint32_t sA = (uint32_t)__cvta_generic_to_shared(tc_smem);
  const uint32_t sB = sA + (uint32_t)(kTcM * K * 2);
  const uint32_t sbar = sB + (uint32_t)(BN * K * 2), sadr = sbar + 8;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kTcM, n0 = blockIdx.y * BN;
  uint32_t ncols = 32;  // TMEM columns: a power of two >= 32
  while ((int)ncols < BN) ncols <<= 1;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sadr), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_stage(sA, A, m0, kTcM, M, K);
  tc_stage(sB, B, n0, BN, N, K);
  asm volatile("cp.async.commit_group;" ::: "memory");
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  // the staged tiles, written through the generic proxy, made visible to the MMAs
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  uint32_t tmem;
  asm volatile("ld.shared.b32 %0, [%1];" : "=r"(tmem) : "r"(sadr) : "memory");
  if (threadIdx.x == 0) {
    const uint32_t idesc = tc_idesc(kTcM, BN);
    const uint32_t sbo = (uint32_t)K * 16u;
    for (int s = 0; s < K / 16; s++) {
      // K step s: core-matrix chunks 2s and 2s + 1 of every row group
      const uint64_t ad = tc_smem_desc(sA + (uint32_t)s * 256u, 128u, sbo);
      const uint64_t bd = tc_smem_desc(sB + (uint32_t)s * 256u, 128u, sbo);
      asm volatile(
          "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
          " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
          "l"(ad), "l"(bd), "r"(idesc), "r"(s)
          : "memory");
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(sbar)
                 : "memory");
  }
  const bool done = __syncthreads_and(tc_wait(sbar, 0)) != 0;
  if (!done) {
    if (threadIdx.x == 0) {
      atomicExch(err, 1);
      tc_wait(sbar, 0);
    }
  } else {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // warp w reads TMEM lanes [32 w, 32 w + 32): the rows of the tile it owns
    const int r = m0 + warp * 32 + lane;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < BN; c0 += 8) {
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
          if (bias) x += bias[c + j];
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

// out[c][r] = in[r][c] for a rows x cols bf16 matrix
__global__ void k_transpose_bf16(const __nv_bfloat16 *in, __nv_bfloat16 *out, int rows, int cols) {
  __shared__ __nv_bfloat16 tile[32][33];
  int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int r = by + j, c = bx + threadIdx.x;
    if (r < rows && c < cols) tile[j][threadIdx.x] = in[(size_t)r * cols + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int c = bx + j, r = by + threadIdx.x;
    if (r < rows && c < cols) out[(size_t)c * rows + r] = tile[threadIdx.x][j];
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
  if (K < 16 || K > kTcMaxK || K % 16) return 0;
  const int bn = N <= kTcMaxN ? N : (N % kTcMaxN == 0 ? kTcMaxN : 0);
  return bn >= 16 && bn % 16 == 0 ? bn : 0;
}

void mlp_gemm_nt(void *stream, const void *A, const void *B, const float *bias, float *C, void *Cb, int M,
                 int N, int K, int relu, int accumulate, int *err) {
  if (M <= 0 || N <= 0) return;
  const int bn = mlp_tile_n(N, K);
  if (bn) {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
      attr = true;
    }
    size_t smem = (size_t)(kTcM + bn) * K * 2 + 16;
    if (smem < kTcMinSmem) smem = kTcMinSmem;
    dim3 grid((M + kTcM - 1) / kTcM, N / bn);
    k_gemm_tc<<<grid, 128, smem, (cudaStream_t)stream>>>((const __nv_bfloat16 *)A, (const __nv_bfloat16 *)B, bias,
                                                        C, (__nv_bfloat16 *)Cb, M, N, K, bn, relu, accumulate, err);
    return;
  }
  dim3 grid((M + TM - 1) / TM, (N + TN - 1) / TN);
  k_gemm_nt<<<grid, 128, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)A, (const __nv_bfloat16 *)B, bias,
                                                     C, (__nv_bfloat16 *)Cb, M, N, K, relu, accumulate);
}

void mlp_transpose_bf16(void *stream, const void *in, void *out, int rows, int cols) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  k_transpose_bf16<<<grid, dim3(32, 8), 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)in,
                                                                  (__nv_bfloat16 *)out, rows, cols);
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
