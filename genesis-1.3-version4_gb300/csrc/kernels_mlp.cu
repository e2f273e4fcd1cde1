// BF16 tensor-core kernels of the learned coarse-step closure: a small MLP
// (inputs -> 256 -> 256 -> 256 -> outputs) evaluated and trained on the GPU.
//
// GEMM: C[M][N] = sum_k A[M][k] B[N][k] ("NT": both operands row-major with the
// reduction index last), BF16 operands, FP32 accumulation, with mma.sync
// m16n8k16. The GEMMs of this network are small (M = slices, N, K <= 256) and
// latency-bound; the warp-level MMA needs no tensor-memory allocation or
// descriptor set-up per launch, which at these sizes costs more than it saves.
// Each CTA computes a 64 x 64 tile with 4 warps (32 x 32 each); K is staged through
// shared memory in chunks of 32.
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

void mlp_gemm_nt(void *stream, const void *A, const void *B, const float *bias, float *C, void *Cb, int M,
                 int N, int K, int relu, int accumulate) {
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
