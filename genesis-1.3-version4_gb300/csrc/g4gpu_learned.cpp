// Learned coarse-step closure: a BF16 MLP trained and evaluated on the GPU
// (kernels_mlp.cu), per-slice features and corrections (kernels_closure.cu), and
// the coarse-step driver in which the non-learned fine-step solve is both the
// fallback and the judge of the closure's error. No reference counterpart: the
// reference integrates every period (src/Core/Gencore.cpp:102-160).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "g4gpu.h"
#include "g4gpu_ctx.h"
#include "g4gpu_internal.h"

namespace {

constexpr int kLayers = 4;  // nin -> width -> width -> width -> nout

int round16(int n) { return (n + 15) / 16 * 16; }

}  // namespace

struct g4gpu_mlp_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int nin = 0, nout = 0, width = 0;
  int dims[kLayers + 1];  // padded layer widths
  std::vector<size_t> woff, boff;
  size_t nparam = 0;
  float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16 *wb = nullptr, *wbt = nullptr;  // weights [N][K] and transposed [K][N]
  std::vector<size_t> wboff;
  size_t nweight = 0;
  float *fmean = nullptr, *fstd = nullptr, *oscale = nullptr, *oshift = nullptr;
  std::vector<float> h_fmean, h_fstd, h_oscale, h_oshift;
  // work buffers for batches of up to `cap` rows
  int cap = 0;
  float *act[kLayers + 1] = {};
  __nv_bfloat16 *actb[kLayers + 1] = {};
  __nv_bfloat16 *actt = nullptr;  // transposed activations [K][rows]
  float *dA = nullptr, *dZ = nullptr;
  __nv_bfloat16 *dZb = nullptr, *dZt = nullptr;
  float *xin = nullptr, *tgt = nullptr, *loss = nullptr;
  int *derr = nullptr;  // device flag: a tensor-core GEMM's bounded wait ran out
  int adam_t = 0;
  std::string err;
};

namespace {

int mfail(g4gpu_mlp m, int code, const std::string &msg) {
  if (m) m->err = msg;
  return code;
}
#define M_CUDA(m, call)                                                            \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) return mfail(m, G4GPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// G4GPU_ERR_DEVICE if a GEMM of the network raised the device flag; called after
// the stream has been synchronised
int mlp_device_status(g4gpu_mlp m) {
  int v = 0;
  M_CUDA(m, cudaMemcpy(&v, m->derr, sizeof(int), cudaMemcpyDeviceToHost));
  if (v) return mfail(m, G4GPU_ERR_DEVICE, "mlp: a tensor-core GEMM did not complete within its bounded wait");
  return G4GPU_OK;
}

int ensure_cap(g4gpu_mlp m, int rows) {
  if (rows <= m->cap) return G4GPU_OK;
  int cap = std::max(rows, 1024);
  for (int l = 0; l <= kLayers; l++) {
    cudaFree(m->act[l]);
    cudaFree(m->actb[l]);
    M_CUDA(m, cudaMalloc(&m->act[l], (size_t)cap * m->dims[l] * sizeof(float)));
    M_CUDA(m, cudaMalloc(&m->actb[l], (size_t)cap * m->dims[l] * sizeof(__nv_bfloat16)));
  }
  int wmax = *std::max_element(m->dims, m->dims + kLayers + 1);
  cudaFree(m->actt);
  cudaFree(m->dA);
  cudaFree(m->dZ);
  cudaFree(m->dZb);
  cudaFree(m->dZt);
  cudaFree(m->xin);
  cudaFree(m->tgt);
  // transposed operands of the weight gradients: rows padded to a multiple of 16
  M_CUDA(m, cudaMalloc(&m->actt, (size_t)round16(cap) * wmax * sizeof(__nv_bfloat16)));
  M_CUDA(m, cudaMalloc(&m->dA, (size_t)cap * wmax * sizeof(float)));
  M_CUDA(m, cudaMalloc(&m->dZ, (size_t)cap * wmax * sizeof(float)));
  M_CUDA(m, cudaMalloc(&m->dZb, (size_t)cap * wmax * sizeof(__nv_bfloat16)));
  M_CUDA(m, cudaMalloc(&m->dZt, (size_t)round16(cap) * wmax * sizeof(__nv_bfloat16)));
  M_CUDA(m, cudaMalloc(&m->xin, (size_t)cap * m->nin * sizeof(float)));
  M_CUDA(m, cudaMalloc(&m->tgt, (size_t)cap * m->nout * sizeof(float)));
  m->cap = cap;
  return G4GPU_OK;
}

// BF16 copies of the weights, row-major [N][K] and transposed [K][N]
void refresh_bf16(g4gpu_mlp m) {
  for (int l = 0; l < kLayers; l++) {
    int K = m->dims[l], N = m->dims[l + 1];
    g4::mlp_to_bf16(m->stream, m->params + m->woff[l], m->wb + m->wboff[l], (size_t)N * K);
    g4::mlp_transpose_bf16(m->stream, m->wb + m->wboff[l], m->wbt + m->wboff[l], N, K, N);
  }
}

// forward pass over `rows` rows of normalised BF16 input already in actb[0]
int forward(g4gpu_mlp m, int rows) {
  for (int l = 0; l < kLayers; l++) {
    int K = m->dims[l], N = m->dims[l + 1];
    if (g4::mlp_gemm_nt(m->stream, m->actb[l], m->wb + m->wboff[l], m->params + m->boff[l], m->act[l + 1],
                        m->actb[l + 1], rows, N, K, l < kLayers - 1, 0, m->derr))
      return mfail(m, G4GPU_ERR_ARG, "mlp: a GEMM could not be launched (widths not multiples of 16, or no tensor map for an operand)");
  }
  return G4GPU_OK;
}

// backward pass of the MSE loss against normalised targets tgt [rows][nout];
// gradients into m->grads, loss into m->loss (accumulated)
int backward(g4gpu_mlp m, int rows) {
  int L = kLayers;
  const int rows16 = round16(rows);  // the weight gradients' reduction, zero-padded
  g4::mlp_mse(m->stream, m->act[L], m->tgt, m->dZ, m->dZb, rows, m->nout, m->dims[L], m->loss);
  for (int l = L - 1; l >= 0; l--) {
    int K = m->dims[l], N = m->dims[l + 1];
    if (l < L - 1) g4::mlp_relu_backward(m->stream, m->dA, m->act[l + 1], m->dZ, m->dZb, (size_t)rows * N);
    // dW [N][K] = dZ^T A_l
    g4::mlp_transpose_bf16(m->stream, m->dZb, m->dZt, rows, N, rows16);
    g4::mlp_transpose_bf16(m->stream, m->actb[l], m->actt, rows, K, rows16);
    int rc = g4::mlp_gemm_nt(m->stream, m->dZt, m->actt, nullptr, m->grads + m->woff[l], nullptr, N, K, rows16, 0, 0,
                             m->derr);
    g4::mlp_colsum(m->stream, m->dZ, m->grads + m->boff[l], rows, N);
    // dA_l [rows][K] = dZ W_l
    if (l > 0 && !rc)
      rc = g4::mlp_gemm_nt(m->stream, m->dZb, m->wbt + m->wboff[l], nullptr, m->dA, nullptr, rows, K, N, 0, 0,
                           m->derr);
    if (rc) return mfail(m, G4GPU_ERR_ARG, "mlp: a GEMM could not be launched (widths not multiples of 16, or no tensor map for an operand)");
  }
  return G4GPU_OK;
}

int upload_norm(g4gpu_mlp m) {
  M_CUDA(m, cudaMemcpyAsync(m->fmean, m->h_fmean.data(), m->nin * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  M_CUDA(m, cudaMemcpyAsync(m->fstd, m->h_fstd.data(), m->nin * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  M_CUDA(m, cudaMemcpyAsync(m->oscale, m->h_oscale.data(), m->nout * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  M_CUDA(m, cudaMemcpyAsync(m->oshift, m->h_oshift.data(), m->nout * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  return G4GPU_OK;
}

// normalised inputs of rows host rows X (raw) into actb[0]; optional targets T
int load_rows(g4gpu_mlp m, const float *X, const float *T, int rows) {
  int rc = ensure_cap(m, rows);
  if (rc) return rc;
  M_CUDA(m, cudaMemcpyAsync(m->xin, X, (size_t)rows * m->nin * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  g4::closure_normalize(m->stream, m->xin, m->fmean, m->fstd, m->actb[0], rows, m->nin, m->dims[0]);
  if (T) {
    std::vector<float> tn((size_t)rows * m->nout);
    for (int r = 0; r < rows; r++)
      for (int c = 0; c < m->nout; c++)
        tn[(size_t)r * m->nout + c] = (T[(size_t)r * m->nout + c] - m->h_oshift[c]) / m->h_oscale[c];
    M_CUDA(m, cudaMemcpyAsync(m->tgt, tn.data(), tn.size() * sizeof(float), cudaMemcpyHostToDevice, m->stream));
    M_CUDA(m, cudaStreamSynchronize(m->stream));
  }
  return G4GPU_OK;
}

}  // namespace

extern "C" {

int g4gpu_mlp_create(int nin, int width, int nout, int seed, int device, g4gpu_mlp *out) {
  if (!out || nin < 1 || nin > 256 || nout < 1 || nout > 64 || width < 16 || width > 1024)
    return g4_fail(nullptr, G4GPU_ERR_ARG, "mlp: 1 <= nin <= 256, 1 <= nout <= 64, 16 <= width <= 1024");
  *out = nullptr;
  g4gpu_mlp m = new g4gpu_mlp_ctx;
  m->device = device;
  m->nin = nin;
  m->nout = nout;
  m->width = width;
  m->dims[0] = round16(nin);
  for (int l = 1; l < kLayers; l++) m->dims[l] = round16(width);
  m->dims[kLayers] = round16(nout);
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    g4_fail(nullptr, G4GPU_ERR_CUDA, std::string("mlp: ") + cudaGetErrorString(e));
    delete m;
    return G4GPU_ERR_CUDA;
  }
  // He-normal initialisation of the weights (zero in the padded rows and columns)
  std::mt19937 rng(seed);
  std::vector<float> p;
  for (int l = 0; l < kLayers; l++) {
    int K = m->dims[l], N = m->dims[l + 1];
    int kin = l == 0 ? nin : width, nreal = l == kLayers - 1 ? nout : width;
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (float)kin) * (l == kLayers - 1 ? 0.1f : 1.f));
    m->woff.push_back(p.size());
    for (int n = 0; n < N; n++)
      for (int k = 0; k < K; k++) p.push_back((n < nreal && k < kin) ? nd(rng) : 0.f);
    m->boff.push_back(p.size());
    for (int n = 0; n < N; n++) p.push_back(0.f);
  }
  m->nparam = p.size();
  size_t nw = 0;
  for (int l = 0; l < kLayers; l++) {
    m->wboff.push_back(nw);
    nw += (size_t)m->dims[l] * m->dims[l + 1];
  }
  m->nweight = nw;
  bool ok = cudaMalloc(&m->params, m->nparam * 4) == cudaSuccess && cudaMalloc(&m->grads, m->nparam * 4) == cudaSuccess &&
            cudaMalloc(&m->m, m->nparam * 4) == cudaSuccess && cudaMalloc(&m->v, m->nparam * 4) == cudaSuccess &&
            cudaMalloc(&m->wb, nw * 2) == cudaSuccess && cudaMalloc(&m->wbt, nw * 2) == cudaSuccess &&
            cudaMalloc(&m->fmean, nin * 4) == cudaSuccess && cudaMalloc(&m->fstd, nin * 4) == cudaSuccess &&
            cudaMalloc(&m->oscale, nout * 4) == cudaSuccess && cudaMalloc(&m->oshift, nout * 4) == cudaSuccess &&
            cudaMalloc(&m->loss, 4) == cudaSuccess && cudaMalloc(&m->derr, 4) == cudaSuccess;
  if (!ok) {
    g4gpu_mlp_destroy(m);
    return g4_fail(nullptr, G4GPU_ERR_NOMEM, "mlp: allocation failed");
  }
  cudaMemcpy(m->params, p.data(), m->nparam * 4, cudaMemcpyHostToDevice);
  cudaMemset(m->m, 0, m->nparam * 4);
  cudaMemset(m->v, 0, m->nparam * 4);
  cudaMemset(m->derr, 0, 4);
  m->h_fmean.assign(nin, 0.f);
  m->h_fstd.assign(nin, 1.f);
  m->h_oshift.assign(nout, 0.f);
  m->h_oscale.assign(nout, 1.f);
  upload_norm(m);
  refresh_bf16(m);
  cudaStreamSynchronize(m->stream);
  *out = m;
  return G4GPU_OK;
}

void g4gpu_mlp_destroy(g4gpu_mlp m) {
  if (!m) return;
  cudaSetDevice(m->device);
  if (m->stream) cudaStreamSynchronize(m->stream);
  void *ptrs[] = {m->params, m->grads, m->m,  m->v,   m->wb,  m->wbt,  m->fmean, m->fstd, m->oscale,
                  m->oshift, m->actt,  m->dA, m->dZ,  m->dZb, m->dZt,  m->xin,   m->tgt,  m->loss,
                  m->derr};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  for (int l = 0; l <= kLayers; l++) {
    if (m->act[l]) cudaFree(m->act[l]);
    if (m->actb[l]) cudaFree(m->actb[l]);
  }
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

const char *g4gpu_mlp_last_error(g4gpu_mlp m) { return m ? m->err.c_str() : ""; }

size_t g4gpu_mlp_num_params(g4gpu_mlp m) { return m ? m->nparam : 0; }

int g4gpu_mlp_get_params(g4gpu_mlp m, float *out) {
  if (!m || !out) return G4GPU_ERR_ARG;
  cudaSetDevice(m->device);
  M_CUDA(m, cudaMemcpyAsync(out, m->params, m->nparam * 4, cudaMemcpyDeviceToHost, m->stream));
  M_CUDA(m, cudaStreamSynchronize(m->stream));
  return G4GPU_OK;
}

int g4gpu_mlp_set_params(g4gpu_mlp m, const float *in) {
  if (!m || !in) return G4GPU_ERR_ARG;
  cudaSetDevice(m->device);
  M_CUDA(m, cudaMemcpyAsync(m->params, in, m->nparam * 4, cudaMemcpyHostToDevice, m->stream));
  refresh_bf16(m);
  M_CUDA(m, cudaStreamSynchronize(m->stream));
  return G4GPU_OK;
}

int g4gpu_mlp_set_normalization(g4gpu_mlp m, const float *fmean, const float *fstd, const float *oshift,
                                const float *oscale) {
  if (!m || !fmean || !fstd || !oshift || !oscale) return G4GPU_ERR_ARG;
  cudaSetDevice(m->device);
  m->h_fmean.assign(fmean, fmean + m->nin);
  m->h_fstd.assign(fstd, fstd + m->nin);
  m->h_oshift.assign(oshift, oshift + m->nout);
  m->h_oscale.assign(oscale, oscale + m->nout);
  for (auto &s : m->h_fstd)
    if (!(s > 0)) s = 1.f;
  for (auto &s : m->h_oscale)
    if (!(s > 0)) s = 1.f;
  int rc = upload_norm(m);
  if (rc) return rc;
  M_CUDA(m, cudaStreamSynchronize(m->stream));
  return G4GPU_OK;
}

int g4gpu_mlp_forward(g4gpu_mlp m, const float *X, int n, float *Y) {
  if (!m || !X || !Y || n < 1) return G4GPU_ERR_ARG;
  cudaSetDevice(m->device);
  int rc = load_rows(m, X, nullptr, n);
  if (rc) return rc;
  if ((rc = forward(m, n))) return rc;
  float *yd = m->dZ;  // scratch for the de-normalised outputs
  g4::closure_denormalize(m->stream, m->act[kLayers], m->oscale, m->oshift, yd, n, m->nout, m->dims[kLayers]);
  M_CUDA(m, cudaMemcpyAsync(Y, yd, (size_t)n * m->nout * 4, cudaMemcpyDeviceToHost, m->stream));
  M_CUDA(m, cudaStreamSynchronize(m->stream));
  return mlp_device_status(m);
}

// Gradients of the MSE loss of normalised outputs over n rows (one batch, no update).
int g4gpu_mlp_gradients(g4gpu_mlp m, const float *X, const float *T, int n, float *grads, float *loss) {
  if (!m || !X || !T || !grads || n < 1) return G4GPU_ERR_ARG;
  cudaSetDevice(m->device);
  int rc = load_rows(m, X, T, n);
  if (rc) return rc;
  M_CUDA(m, cudaMemsetAsync(m->loss, 0, 4, m->stream));
  M_CUDA(m, cudaMemsetAsync(m->grads, 0, m->nparam * 4, m->stream));
  if ((rc = forward(m, n)) || (rc = backward(m, n))) return rc;
  M_CUDA(m, cudaMemcpyAsync(grads, m->grads, m->nparam * 4, cudaMemcpyDeviceToHost, m->stream));
  if (loss) M_CUDA(m, cudaMemcpyAsync(loss, m->loss, 4, cudaMemcpyDeviceToHost, m->stream));
  M_CUDA(m, cudaStreamSynchronize(m->stream));
  return mlp_device_status(m);
}

// Adam training on n rows of raw features X [n][nin] and targets T [n][nout].
// The normalisation (feature mean / std, target shift / scale) is fitted to the
// data first. loss_per_epoch (may be NULL) receives the mean loss of each epoch.
int g4gpu_mlp_train(g4gpu_mlp m, const float *X, const float *T, int n, int epochs, int batch, float lr,
                    int seed, float *loss_per_epoch) {
  if (!m || !X || !T || n < 2 || epochs < 1 || batch < 16) return G4GPU_ERR_ARG;
  cudaSetDevice(m->device);
  // normalisation statistics
  std::vector<double> mu(m->nin, 0), sd(m->nin, 0), tmu(m->nout, 0), tsd(m->nout, 0);
  for (int r = 0; r < n; r++) {
    for (int c = 0; c < m->nin; c++) mu[c] += X[(size_t)r * m->nin + c];
    for (int c = 0; c < m->nout; c++) tmu[c] += T[(size_t)r * m->nout + c];
  }
  for (auto &v : mu) v /= n;
  for (auto &v : tmu) v /= n;
  for (int r = 0; r < n; r++) {
    for (int c = 0; c < m->nin; c++) {
      double d = X[(size_t)r * m->nin + c] - mu[c];
      sd[c] += d * d;
    }
    for (int c = 0; c < m->nout; c++) {
      double d = T[(size_t)r * m->nout + c] - tmu[c];
      tsd[c] += d * d;
    }
  }
  for (int c = 0; c < m->nin; c++) {
    m->h_fmean[c] = (float)mu[c];
    double s = std::sqrt(sd[c] / n);
    m->h_fstd[c] = s > 1e-12 ? (float)s : 1.f;
  }
  for (int c = 0; c < m->nout; c++) {
    m->h_oshift[c] = (float)tmu[c];
    double s = std::sqrt(tsd[c] / n);
    m->h_oscale[c] = s > 1e-30 ? (float)s : 1.f;
  }
  int rc = upload_norm(m);
  if (rc) return rc;
  // shuffled order
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::mt19937 rng(seed);
  std::vector<float> xb((size_t)batch * m->nin), tb((size_t)batch * m->nout);
  for (int ep = 0; ep < epochs; ep++) {
    std::shuffle(idx.begin(), idx.end(), rng);
    M_CUDA(m, cudaMemsetAsync(m->loss, 0, 4, m->stream));
    int nb = 0;
    for (int b0 = 0; b0 + batch <= n; b0 += batch, nb++) {
      for (int r = 0; r < batch; r++) {
        std::memcpy(&xb[(size_t)r * m->nin], &X[(size_t)idx[b0 + r] * m->nin], m->nin * 4);
        std::memcpy(&tb[(size_t)r * m->nout], &T[(size_t)idx[b0 + r] * m->nout], m->nout * 4);
      }
      if ((rc = load_rows(m, xb.data(), tb.data(), batch))) return rc;
      if ((rc = forward(m, batch)) || (rc = backward(m, batch))) return rc;
      m->adam_t++;
      g4::mlp_adam(m->stream, m->params, m->grads, m->m, m->v, m->nparam, lr, 0.9f, 0.999f, 1e-8f, m->adam_t);
      refresh_bf16(m);
    }
    float l = 0;
    M_CUDA(m, cudaMemcpyAsync(&l, m->loss, 4, cudaMemcpyDeviceToHost, m->stream));
    M_CUDA(m, cudaStreamSynchronize(m->stream));
    if ((rc = mlp_device_status(m))) return rc;
    if (loss_per_epoch) loss_per_epoch[ep] = nb ? l / nb : 0.f;
  }
  return G4GPU_OK;
}

// ---- the closure on a handle ---------------------------------------------------

// Hermite polynomial H_n (physicists')
static double herm(int n, double x) {
  double h0 = 1, h1 = 2 * x;
  if (n == 0) return h0;
  for (int k = 1; k < n; k++) {
    double h2 = 2 * x * h1 - 2 * k * h0;
    h0 = h1;
    h1 = h2;
  }
  return h1;
}

int g4gpu_closure_attach(g4gpu_handle h, g4gpu_mlp m, double waist, double u0, double c0) {
  if (!h || !m) return g4_fail(h, G4GPU_ERR_ARG, "closure: null handle or network");
  if (h->beam.count) return g4_fail(h, G4GPU_ERR_STATE, "closure: one4one windows are not supported");
  if (m->nin != g4::kClosureNin || m->nout != g4::kClosureNout)
    return g4_fail(h, G4GPU_ERR_ARG, "closure: the network must map 32 features to 4 corrections");
  if (!(waist > 0) || !(u0 > 0) || !(c0 > 0)) return g4_fail(h, G4GPU_ERR_ARG, "closure: waist, u0, c0 > 0");
  cudaSetDevice(h->cfg.device);
  int ng = h->cfg.ngrid;
  double gm = h->cfg.gridmax[0], dg = 2 * gm / (ng - 1);
  // Gauss-Hermite modes HG_mn(x, y) = h_m(x) h_n(y), m, n = 0..3, on the grid of field 0:
  // the 1-D factors h_m(x_i) = sqrt(sqrt(2 / pi) / w) / sqrt(2^m m!) H_m(sqrt(2) x_i / w)
  // exp(-x_i^2 / w^2) dg (one cell side each, so that their product carries the cell area);
  // the grid is the same in x and y, so one table [4][ngrid] serves both
  std::vector<float> basis(4 * (size_t)ng);
  for (int mm = 0; mm < 4; mm++) {
    double norm = std::sqrt(std::sqrt(2.0 / 3.14159265358979323846) / waist) /
                  std::sqrt(std::pow(2.0, mm) * std::tgamma(mm + 1.0));
    for (int i = 0; i < ng; i++) {
      double x = -gm + i * dg;
      basis[(size_t)mm * ng + i] =
          (float)(norm * herm(mm, std::sqrt(2.0) * x / waist) * std::exp(-x * x / (waist * waist)) * dg);
    }
  }
  if (!h->closure_basis) {
    int rc = g4_alloc(h, (void **)&h->closure_basis, basis.size() * 4);
    if (rc) return rc;
    if ((rc = g4_alloc(h, (void **)&h->closure_feat, (size_t)h->cfg.nslice * g4::kClosureNin * 4))) return rc;
    if ((rc = g4_alloc(h, (void **)&h->closure_corr, (size_t)h->cfg.nslice * g4::kClosureNout * 4))) return rc;
  }
  cudaError_t e = cudaMemcpy(h->closure_basis, basis.data(), basis.size() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return g4_cuda_fail(h, e, "closure basis");
  h->mlp = m;
  h->closure_u0 = (float)u0;
  h->closure_c0 = (float)c0;
  return G4GPU_OK;
}

// Per-slice features of the current state into host out [nslice][32] (raw).
int g4gpu_closure_features(g4gpu_handle h, float *out) {
  if (!h || !out) return g4_fail(h, G4GPU_ERR_ARG, "closure: null argument");
  if (!h->closure_basis) return g4_fail(h, G4GPU_ERR_STATE, "closure: not attached");
  if (h->beam.count) return g4_fail(h, G4GPU_ERR_STATE, "closure: one4one windows are not supported");
  cudaSetDevice(h->cfg.device);
  const g4gpu_config &c = h->cfg;
  g4::closure_features(h->stream, h->beam.theta, h->beam.gamma, h->beam.current, h->field[0], h->closure_basis,
                       h->mixed, c.gammaref, c.nslice, c.npart, c.ngrid, h->first[0], h->closure_u0,
                       h->closure_c0, h->closure_feat);
  cudaError_t e = cudaMemcpyAsync(out, h->closure_feat, (size_t)c.nslice * g4::kClosureNin * 4,
                                  cudaMemcpyDeviceToHost, h->stream);
  if (e != cudaSuccess) return g4_cuda_fail(h, e, "closure features");
  return g4_check_device_flag(h);
}

// Applies host corrections corr [nslice][4] to the current state.
int g4gpu_closure_apply(g4gpu_handle h, const float *corr) {
  if (!h || !corr) return g4_fail(h, G4GPU_ERR_ARG, "closure: null argument");
  if (!h->closure_corr) return g4_fail(h, G4GPU_ERR_STATE, "closure: not attached");
  cudaSetDevice(h->cfg.device);
  const g4gpu_config &c = h->cfg;
  cudaError_t e = cudaMemcpyAsync(h->closure_corr, corr, (size_t)c.nslice * g4::kClosureNout * 4,
                                  cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return g4_cuda_fail(h, e, "closure corrections");
  g4::closure_apply(h->stream, h->beam.theta, h->beam.gamma, h->field[0], h->closure_corr, h->mixed, c.nslice,
                    c.npart, c.ngrid, h->first[0]);
  h->launches[G4GPU_K_MISC]++;
  return G4GPU_OK;
}

// Per-slice features of the current state into the device buffer (the closure
// reads the state at the start of a coarse step, as in training).
static void closure_features_dev(g4gpu_handle h) {
  const g4gpu_config &c = h->cfg;
  g4::closure_features(h->stream, h->beam.theta, h->beam.gamma, h->beam.current, h->field[0], h->closure_basis,
                       h->mixed, c.gammaref, c.nslice, c.npart, c.ngrid, h->first[0], h->closure_u0,
                       h->closure_c0, h->closure_feat);
  h->launches[G4GPU_K_MISC]++;
}

// Network on the stored features -> corrections applied to the current state,
// all on the device and on the handle's stream.
static int closure_correct(g4gpu_handle h) {
  const g4gpu_config &c = h->cfg;
  g4gpu_mlp m = h->mlp;
  int ns = c.nslice;
  int rc = ensure_cap(m, ns);
  if (rc) return g4_fail(h, rc, m->err);
  // the network runs on the handle's stream and raises the handle's device flag
  cudaStream_t saved = m->stream;
  int *saved_err = m->derr;
  m->stream = h->stream;
  m->derr = h->derr;
  g4::closure_normalize(h->stream, h->closure_feat, m->fmean, m->fstd, m->actb[0], ns, m->nin, m->dims[0]);
  rc = forward(m, ns);
  if (rc) {
    m->stream = saved;
    m->derr = saved_err;
    return g4_fail(h, rc, m->err);
  }
  g4::closure_denormalize(h->stream, m->act[kLayers], m->oscale, m->oshift, h->closure_corr, ns, m->nout,
                          m->dims[kLayers]);
  g4::closure_apply(h->stream, h->beam.theta, h->beam.gamma, h->field[0], h->closure_corr, h->mixed, ns,
                    c.npart, c.ngrid, h->first[0]);
  m->stream = saved;
  m->derr = saved_err;
  h->launches[G4GPU_K_MISC] += 3 + kLayers;
  return G4GPU_OK;
}

// Training targets [nslice][4]: the corrections that would turn the coarse state of
// hc into the fine state of hf (same shape; both after the same interval).
int g4gpu_closure_targets(g4gpu_handle hc, g4gpu_handle hf, float *out) {
  if (!hc || !hf || !out) return g4_fail(hc, G4GPU_ERR_ARG, "closure_targets: null argument");
  const g4gpu_config &a = hc->cfg, &b = hf->cfg;
  if (a.nslice != b.nslice || a.npart != b.npart || a.ngrid != b.ngrid || a.precision != b.precision)
    return g4_fail(hc, G4GPU_ERR_ARG, "closure_targets: handles differ in shape or precision");
  if (!hc->closure_corr) return g4_fail(hc, G4GPU_ERR_STATE, "closure_targets: attach a closure to hc first");
  cudaSetDevice(a.device);
  cudaEvent_t ev;
  cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  cudaEventRecord(ev, hf->stream);
  cudaStreamWaitEvent(hc->stream, ev, 0);
  cudaEventDestroy(ev);
  g4::closure_targets(hc->stream, hc->beam.theta, hc->beam.gamma, hc->field[0], hf->beam.theta, hf->beam.gamma,
                      hf->field[0], hc->mixed, a.nslice, a.npart, a.ngrid, hc->first[0], hf->first[0],
                      hc->closure_corr);
  cudaError_t e = cudaMemcpyAsync(out, hc->closure_corr, (size_t)a.nslice * g4::kClosureNout * 4,
                                  cudaMemcpyDeviceToHost, hc->stream);
  if (e != cudaSuccess) return g4_cuda_fail(hc, e, "closure_targets");
  return g4_check_device_flag(hc);
}

// Copies beam, fields and ring state between two handles of the same shape.
int g4gpu_copy_state(g4gpu_handle dst, g4gpu_handle src) {
  if (!dst || !src) return g4_fail(dst, G4GPU_ERR_ARG, "copy_state: null handle");
  const g4gpu_config &a = dst->cfg, &b = src->cfg;
  if (a.nslice != b.nslice || a.npart != b.npart || a.ngrid != b.ngrid || a.nfield != b.nfield ||
      a.precision != b.precision || a.device != b.device)
    return g4_fail(dst, G4GPU_ERR_ARG, "copy_state: handles differ in shape, precision or device");
  cudaSetDevice(a.device);
  // order after the source's queued work
  cudaEvent_t ev;
  cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  cudaEventRecord(ev, src->stream);
  cudaStreamWaitEvent(dst->stream, ev, 0);
  cudaEventDestroy(ev);
  size_t np = (size_t)a.nslice * a.npart, nf = (size_t)a.nslice * a.ngrid * a.ngrid * dst->csize;
  std::pair<void *, const void *> bufs[] = {{dst->beam.gamma, src->beam.gamma}, {dst->beam.x, src->beam.x},
                                            {dst->beam.y, src->beam.y},         {dst->beam.px, src->beam.px},
                                            {dst->beam.py, src->beam.py}};
  for (auto &q : bufs) {
    cudaError_t e = cudaMemcpyAsync(q.first, q.second, np * dst->rsize, cudaMemcpyDeviceToDevice, dst->stream);
    if (e != cudaSuccess) return g4_cuda_fail(dst, e, "copy_state");
  }
  cudaError_t e = cudaMemcpyAsync(dst->beam.theta, src->beam.theta, np * 8, cudaMemcpyDeviceToDevice, dst->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dst->beam.current, src->beam.current, a.nslice * 8, cudaMemcpyDeviceToDevice, dst->stream);
  for (int k = 0; k < a.nfield && e == cudaSuccess; k++) {
    e = cudaMemcpyAsync(dst->field[k], src->field[k], nf, cudaMemcpyDeviceToDevice, dst->stream);
    dst->first[k] = src->first[k];
    dst->accuslip[k] = src->accuslip[k];
    dst->field_loaded[k] = true;
  }
  if (e != cudaSuccess) return g4_cuda_fail(dst, e, "copy_state");
  dst->beam_loaded = true;
  // the source must not be modified before the copy has read it
  cudaEvent_t ev2;
  cudaEventCreateWithFlags(&ev2, cudaEventDisableTiming);
  cudaEventRecord(ev2, dst->stream);
  cudaStreamWaitEvent(src->stream, ev2, 0);
  cudaEventDestroy(ev2);
  return G4GPU_OK;
}

// Coarse steps with the closure. hc holds the coarse lattice, hf the fine one;
// coarse step i covers fine steps fine_start[i] .. fine_start[i]+fine_count[i]-1.
// Every check_every coarse steps the fine solve of the same interval judges the
// closure: if the slice power of the coarse+closure result differs from the fine
// one by more than tol (relative to the largest slice power), the fine result is
// kept and the following check_every - 1 intervals run with fine steps.
// The current state lives in one of the two handles at a time: a failed check
// leaves it in hf, the fallback intervals advance it there, and it is copied back
// to hc only before the next coarse step (or at the end), so a fallback block costs
// one state copy, not two per interval.
int g4gpu_run_learned(g4gpu_handle hc, g4gpu_handle hf, int istep0, int ncoarse, const int *fine_start,
                      const int *fine_count, int check_every, double tol, int *nchecks, int *nfallback,
                      double *max_err) {
  if (!hc || !hf || !fine_start || !fine_count || check_every < 1)
    return g4_fail(hc, G4GPU_ERR_ARG, "run_learned: bad arguments");
  if (!hc->mlp) return g4_fail(hc, G4GPU_ERR_STATE, "run_learned: no closure attached");
  int ns = hc->cfg.nslice, nfld = hc->cfg.nfield;
  std::vector<double> pc((size_t)nfld * ns * G4GPU_DF_NCOL), pf(pc.size());
  int checks = 0, falls = 0, fine_left = 0;
  double emax = 0;
  bool in_fine = false;  // the current state is in hf (hc is stale)
  int rc;
  for (int i = istep0; i < istep0 + ncoarse; i++) {
    if (i < 0 || i >= hc->nsteps) return g4_fail(hc, G4GPU_ERR_ARG, "run_learned: coarse step outside the lattice");
    int f0 = fine_start[i], nf = fine_count[i];
    if (fine_left > 0) {
      // fallback interval: fine steps on hf, where the state already is
      if (!in_fine && (rc = g4gpu_copy_state(hf, hc))) return rc;
      in_fine = true;
      if ((rc = g4gpu_run(hf, f0, nf, G4GPU_STAGE_ALL))) return rc;
      fine_left--;
      continue;
    }
    if (in_fine) {
      if ((rc = g4gpu_copy_state(hc, hf))) return rc;
      in_fine = false;
    }
    bool check = ((i - istep0) % check_every) == 0;
    if (check && (rc = g4gpu_copy_state(hf, hc))) return rc;
    closure_features_dev(hc);
    if ((rc = g4gpu_run(hc, i, 1, G4GPU_STAGE_ALL))) return rc;
    if ((rc = closure_correct(hc))) return rc;
    if (check) {
      checks++;
      if ((rc = g4gpu_run(hf, f0, nf, G4GPU_STAGE_ALL))) return rc;
      if ((rc = g4gpu_diag(hc, 1, nullptr, pc.data()))) return rc;
      if ((rc = g4gpu_diag(hf, 1, nullptr, pf.data()))) return rc;
      double pmax = 0, dmax = 0;
      for (int s = 0; s < ns; s++) {
        double a = pc[(size_t)s * G4GPU_DF_NCOL], b = pf[(size_t)s * G4GPU_DF_NCOL];
        pmax = std::max(pmax, std::fabs(b));
        dmax = std::max(dmax, std::fabs(a - b));
      }
      double err = pmax > 0 ? dmax / pmax : 0;
      emax = std::max(emax, err);
      if (err > tol) {
        falls++;
        in_fine = true;  // keep the fine result, which hf holds
        fine_left = check_every - 1;
      }
    }
  }
  if (in_fine && (rc = g4gpu_copy_state(hc, hf))) return rc;
  if (nchecks) *nchecks = checks;
  if (nfallback) *nfallback = falls;
  if (max_err) *max_err = emax;
  return G4GPU_OK;
}

}  // extern "C"
