// Multilayer perceptron for the learned warm start: maps the parameters of
// an OCP instance to its state/costate/control trajectory at fixed
// normalised-time nodes (the Newton initial guess).
//
//   x -> L0 -> GELU -> L1 -> GELU -> ... -> L{D-1} -> y      (D linear layers)
//
// Weights are kept in FP32 (Adam master copy); every GEMM rounds its operands
// to BF16 when it stages them in shared memory and accumulates in FP32 on the
// tensor cores (mma.sync m16n8k16 BF16).  Forward, backward (input and weight
// gradients), MSE loss and Adam are all kernels here; the host only orders
// them.  The reference has no counterpart (it starts Newton from the
// constant guess of the OCP file).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "cs_gb300.h"

int cs_internal_set_error(int code, const char* msg);

namespace {

#define MLP_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) return cs_internal_set_error(CS_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

// ---------------------------------------------------------------- GEMM ----
// C[m][n] (+)= sum_k A(m, k) B(k, n) (+ bias[n]), with strided FP32 operands:
// A(m, k) = A[m * sam + k * sak], B(k, n) = B[k * sbk + n * sbn].
// Tile 64 x 64 x 16 per CTA of 4 warps (2 x 2), each warp 32 x 32 = 2 x 4
// m16n8 tiles.  Epilogue: bias, then optionally GELU with the pre-activation
// kept in P.
constexpr int BM = 64, BN = 64, BK = 16;

struct GemmArgs {
  int M, N, K;
  const float* A;
  long long sam, sak;
  const float* B;
  long long sbk, sbn;
  float* C;
  long long ldc;
  const float* bias;  // [N] or null
  float* P;           // pre-activation out (GELU) or null
  int gelu;           // apply GELU
  int accumulate;     // C += result
};

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

__global__ void __launch_bounds__(128) k_gemm_bf16(GemmArgs g) {
  // operand tiles in BF16: As[m][k], Bs[n][k] (K contiguous: the layout the
  // m16n8k16 row.col fragments read)
  __shared__ __nv_bfloat16 As[BM][BK + 8];
  __shared__ __nv_bfloat16 Bs[BN][BK + 8];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int gq = lane >> 2, tq = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
  for (int k0 = 0; k0 < g.K; k0 += BK) {
    // stage: 64 x 16 elements of each operand, 8 per thread
    for (int e = tid; e < BM * BK; e += 128) {
      const int r = e / BK, k = e - r * BK;
      const int gm = m0 + r, gk = k0 + k;
      const float va = (gm < g.M && gk < g.K) ? g.A[gm * g.sam + gk * g.sak] : 0.f;
      As[r][k] = __float2bfloat16_rn(va);
      const int gn = n0 + r;
      const float vb = (gn < g.N && gk < g.K) ? g.B[gk * g.sbk + gn * g.sbn] : 0.f;
      Bs[r][k] = __float2bfloat16_rn(vb);
    }
    __syncthreads();
    unsigned af[2][4], bf[4][2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int r = wm + i * 16 + gq;
      af[i][0] = *reinterpret_cast<const unsigned*>(&As[r][2 * tq]);
      af[i][1] = *reinterpret_cast<const unsigned*>(&As[r + 8][2 * tq]);
      af[i][2] = *reinterpret_cast<const unsigned*>(&As[r][2 * tq + 8]);
      af[i][3] = *reinterpret_cast<const unsigned*>(&As[r + 8][2 * tq + 8]);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = wn + j * 8 + gq;
      bf[j][0] = *reinterpret_cast<const unsigned*>(&Bs[c][2 * tq]);
      bf[j][1] = *reinterpret_cast<const unsigned*>(&Bs[c][2 * tq + 8]);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};\n"
            : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
            : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bf[j][0]), "r"(bf[j][1]));
      }
    __syncthreads();
  }
  // epilogue: c0 (gq, 2tq), c1 (gq, 2tq+1), c2 (gq+8, 2tq), c3 (gq+8, 2tq+1)
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int m = m0 + wm + i * 16 + gq + ((q & 2) ? 8 : 0);
        const int n = n0 + wn + j * 8 + 2 * tq + (q & 1);
        if (m >= g.M || n >= g.N) continue;
        float v = acc[i][j][q];
        if (g.bias) v += g.bias[n];
        float* c = g.C + (long long)m * g.ldc + n;
        if (g.gelu) {
          if (g.P) g.P[(long long)m * g.ldc + n] = v;
          v = gelu_f(v);
        }
        if (g.accumulate) *c += v; else *c = v;
      }
}

int gemm(cudaStream_t st, const GemmArgs& g) {
  dim3 grid((g.N + BN - 1) / BN, (g.M + BM - 1) / BM);
  k_gemm_bf16<<<grid, 128, 0, st>>>(g);
  MLP_CUDA(cudaGetLastError());
  return CS_OK;
}

// ------------------------------------------------------- small kernels ----
// rows of X, Y by a permutation (mini-batch gather), normalised
__global__ void k_gather(const float* X, const float* Y, const int* idx, int n, int nin, int nout, const float* xm,
                         const float* xs, const float* ym, const float* ys, float* Xb, float* Yb) {
  const long long tot = (long long)n * (nin + nout);
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / (nin + nout)), c = (int)(e - (long long)r * (nin + nout));
    const long long src = idx ? idx[r] : r;
    if (c < nin) Xb[(long long)r * nin + c] = (X[src * nin + c] - xm[c]) / xs[c];
    else if (Y) {
      const int cc = c - nin;
      Yb[(long long)r * nout + cc] = (Y[src * nout + cc] - ym[cc]) / ys[cc];
    }
  }
}

// d = (pred - target) * 2 / (n * nout); loss partial sums
__global__ void k_mse_grad(const float* P, const float* T, long long total, float scale, float* D, double* loss) {
  double s = 0.0;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const float d = P[e] - T[e];
    D[e] = 2.0f * d * scale;
    s += (double)d * d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s * scale);
}

// dA = dH * gelu'(P)  (in place on dH)
__global__ void k_gelu_back(float* dH, const float* P, long long total) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
    dH[e] *= gelu_grad(P[e]);
}

// bias gradient: column sums of dH (rows n)
__global__ void k_colsum(const float* dH, int n, int cols, float* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < n; ++r) s += dH[(long long)r * cols + c];
  out[c] = s;
}

__global__ void k_adam(float* w, const float* g, float* m1, float* m2, long long n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const float gg = g[e];
    const float a = b1 * m1[e] + (1.f - b1) * gg;
    const float v = b2 * m2[e] + (1.f - b2) * gg * gg;
    m1[e] = a;
    m2[e] = v;
    w[e] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
  }
}

__global__ void k_denorm(float* Y, long long n, int nout, const float* ym, const float* ys) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n * nout; e += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(e % nout);
    Y[e] = Y[e] * ys[c] + ym[c];
  }
}

unsigned grid_for(long long n) { return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4096)); }

}  // namespace

// ================================================================= MLP ===
struct cs_mlp {
  int nin, width, depth, nout;
  std::vector<int> din, dout;  // per layer
  std::vector<long long> woff, boff;
  long long nparam = 0;
  float* w = nullptr;   // all weights and biases, FP32
  float* g = nullptr;   // gradients
  float* m1 = nullptr;  // Adam moments
  float* m2 = nullptr;
  float* norm = nullptr;  // xm, xs, ym, ys
  long long step = 0;
  float lr_final = -1.f;  // cosine decay of the learning rate to lr_final * lr (< 0: constant)
  cudaStream_t st = nullptr;
  // activations for a batch of up to cap rows
  int cap = 0;
  std::vector<float*> act, pre;  // act[l]: input of layer l (act[0] = x), act[depth] = output
  float* tgt = nullptr;
  float* dbuf[2] = {nullptr, nullptr};
  double* dloss = nullptr;
  int* didx = nullptr;
};

static void mlp_free_acts(cs_mlp* M) {
  for (float* p : M->act) cudaFree(p);
  for (float* p : M->pre) cudaFree(p);
  M->act.clear();
  M->pre.clear();
  cudaFree(M->tgt);
  cudaFree(M->dbuf[0]);
  cudaFree(M->dbuf[1]);
  cudaFree(M->didx);
  M->tgt = M->dbuf[0] = M->dbuf[1] = nullptr;
  M->didx = nullptr;
  M->cap = 0;
}

static int mlp_reserve(cs_mlp* M, int rows) {
  if (rows <= M->cap) return CS_OK;
  mlp_free_acts(M);
  const int cap = std::max(rows, 256);
  M->act.resize(M->depth + 1, nullptr);
  M->pre.resize(M->depth, nullptr);
  for (int l = 0; l <= M->depth; ++l) {
    const int cols = (l == 0) ? M->nin : M->dout[l - 1];
    MLP_CUDA(cudaMalloc(&M->act[l], (size_t)cap * cols * sizeof(float)));
  }
  for (int l = 0; l < M->depth; ++l) MLP_CUDA(cudaMalloc(&M->pre[l], (size_t)cap * M->dout[l] * sizeof(float)));
  const int wmax = std::max(M->width, std::max(M->nout, M->nin));
  MLP_CUDA(cudaMalloc(&M->tgt, (size_t)cap * M->nout * sizeof(float)));
  MLP_CUDA(cudaMalloc(&M->dbuf[0], (size_t)cap * wmax * sizeof(float)));
  MLP_CUDA(cudaMalloc(&M->dbuf[1], (size_t)cap * wmax * sizeof(float)));
  MLP_CUDA(cudaMalloc(&M->didx, (size_t)cap * sizeof(int)));
  M->cap = cap;
  return CS_OK;
}

extern "C" int cs_mlp_create(int n_in, int width, int depth, int n_out, unsigned long long seed, cs_mlp** out) {
  if (!out || n_in < 1 || width < 1 || depth < 1 || n_out < 1 || depth > 16)
    return cs_internal_set_error(CS_ERR_INVALID, "cs_mlp_create: bad sizes");
  cs_mlp* M = new cs_mlp();
  M->nin = n_in;
  M->width = width;
  M->depth = depth;
  M->nout = n_out;
  long long off = 0;
  for (int l = 0; l < depth; ++l) {
    const int di = (l == 0) ? n_in : width;
    const int dd = (l == depth - 1) ? n_out : width;
    M->din.push_back(di);
    M->dout.push_back(dd);
    M->woff.push_back(off);
    off += (long long)di * dd;
    M->boff.push_back(off);
    off += dd;
  }
  M->nparam = off;
  // He-style uniform initialisation, seeded
  std::vector<float> hw(off, 0.f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < depth; ++l) {
    const float bound = std::sqrt(6.0f / (float)M->din[l]) * (l == depth - 1 ? 0.5f : 1.0f);
    std::uniform_real_distribution<float> U(-bound, bound);
    for (long long e = 0; e < (long long)M->din[l] * M->dout[l]; ++e) hw[M->woff[l] + e] = U(rng);
  }
  std::vector<float> nrm(2 * (n_in + n_out));
  for (int c = 0; c < n_in; ++c) { nrm[c] = 0.f; nrm[n_in + c] = 1.f; }
  for (int c = 0; c < n_out; ++c) { nrm[2 * n_in + c] = 0.f; nrm[2 * n_in + n_out + c] = 1.f; }
  if (cudaStreamCreateWithFlags(&M->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&M->w, off * sizeof(float)) != cudaSuccess || cudaMalloc(&M->g, off * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&M->m1, off * sizeof(float)) != cudaSuccess || cudaMalloc(&M->m2, off * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&M->norm, nrm.size() * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&M->dloss, sizeof(double)) != cudaSuccess) {
    cs_mlp_free(M);
    return cs_internal_set_error(CS_ERR_NOMEM, "cs_mlp_create: device allocation failed");
  }
  cudaMemcpy(M->w, hw.data(), off * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemset(M->m1, 0, off * sizeof(float));
  cudaMemset(M->m2, 0, off * sizeof(float));
  cudaMemcpy(M->norm, nrm.data(), nrm.size() * sizeof(float), cudaMemcpyHostToDevice);
  *out = M;
  return CS_OK;
}

extern "C" void cs_mlp_free(cs_mlp* M) {
  if (!M) return;
  mlp_free_acts(M);
  cudaFree(M->w);
  cudaFree(M->g);
  cudaFree(M->m1);
  cudaFree(M->m2);
  cudaFree(M->norm);
  cudaFree(M->dloss);
  if (M->st) cudaStreamDestroy(M->st);
  delete M;
}

extern "C" long long cs_mlp_num_params(const cs_mlp* M) { return M ? M->nparam : 0; }

extern "C" int cs_mlp_set_normalization(cs_mlp* M, const float* in_mean, const float* in_std, const float* out_mean,
                                        const float* out_std) {
  if (!M || !in_mean || !in_std || !out_mean || !out_std) return cs_internal_set_error(CS_ERR_INVALID, "null");
  std::vector<float> nrm;
  nrm.insert(nrm.end(), in_mean, in_mean + M->nin);
  nrm.insert(nrm.end(), in_std, in_std + M->nin);
  nrm.insert(nrm.end(), out_mean, out_mean + M->nout);
  nrm.insert(nrm.end(), out_std, out_std + M->nout);
  MLP_CUDA(cudaMemcpy(M->norm, nrm.data(), nrm.size() * sizeof(float), cudaMemcpyHostToDevice));
  return CS_OK;
}

extern "C" int cs_mlp_get_params(cs_mlp* M, float* host) {
  if (!M || !host) return cs_internal_set_error(CS_ERR_INVALID, "null");
  MLP_CUDA(cudaMemcpy(host, M->w, M->nparam * sizeof(float), cudaMemcpyDeviceToHost));
  return CS_OK;
}

extern "C" int cs_mlp_set_params(cs_mlp* M, const float* host) {
  if (!M || !host) return cs_internal_set_error(CS_ERR_INVALID, "null");
  MLP_CUDA(cudaMemcpy(M->w, host, M->nparam * sizeof(float), cudaMemcpyHostToDevice));
  return CS_OK;
}

// forward on the normalised rows in act[0] (n rows)
static int mlp_forward(cs_mlp* M, int n) {
  for (int l = 0; l < M->depth; ++l) {
    GemmArgs g;
    memset(&g, 0, sizeof(g));
    g.M = n;
    g.N = M->dout[l];
    g.K = M->din[l];
    g.A = M->act[l];
    g.sam = M->din[l];
    g.sak = 1;
    g.B = M->w + M->woff[l];  // W[out][in]: B(k, n) = W[n][k]
    g.sbk = 1;
    g.sbn = M->din[l];
    g.C = M->act[l + 1];
    g.ldc = M->dout[l];
    g.bias = M->w + M->boff[l];
    const bool last = (l == M->depth - 1);
    g.gelu = last ? 0 : 1;
    g.P = last ? nullptr : M->pre[l];
    int rc = gemm(M->st, g);
    if (rc != CS_OK) return rc;
  }
  return CS_OK;
}

// loss and gradients for the rows in act[0] / tgt (n rows)
static int mlp_backward(cs_mlp* M, int n, double* loss_out) {
  const long long tot = (long long)n * M->nout;
  MLP_CUDA(cudaMemsetAsync(M->dloss, 0, sizeof(double), M->st));
  float* d = M->dbuf[0];
  k_mse_grad<<<grid_for(tot), 256, 0, M->st>>>(M->act[M->depth], M->tgt, tot, 1.0f / (float)tot, d, M->dloss);
  for (int l = M->depth - 1; l >= 0; --l) {
    const int di = M->din[l], dd = M->dout[l];
    if (l < M->depth - 1) k_gelu_back<<<grid_for((long long)n * dd), 256, 0, M->st>>>(d, M->pre[l], (long long)n * dd);
    // dW[o][i] = sum_r d[r][o] x[r][i]
    GemmArgs g;
    memset(&g, 0, sizeof(g));
    g.M = dd;
    g.N = di;
    g.K = n;
    g.A = d;
    g.sam = 1;
    g.sak = dd;
    g.B = M->act[l];
    g.sbk = di;
    g.sbn = 1;
    g.C = M->g + M->woff[l];
    g.ldc = di;
    int rc = gemm(M->st, g);
    if (rc != CS_OK) return rc;
    k_colsum<<<(dd + 127) / 128, 128, 0, M->st>>>(d, n, dd, M->g + M->boff[l]);
    if (l > 0) {
      // dx[r][i] = sum_o d[r][o] W[o][i]
      float* dn = (d == M->dbuf[0]) ? M->dbuf[1] : M->dbuf[0];
      GemmArgs h;
      memset(&h, 0, sizeof(h));
      h.M = n;
      h.N = di;
      h.K = dd;
      h.A = d;
      h.sam = dd;
      h.sak = 1;
      h.B = M->w + M->woff[l];
      h.sbk = di;
      h.sbn = 1;
      h.C = dn;
      h.ldc = di;
      rc = gemm(M->st, h);
      if (rc != CS_OK) return rc;
      d = dn;
    }
  }
  MLP_CUDA(cudaGetLastError());
  if (loss_out) {
    MLP_CUDA(cudaMemcpyAsync(loss_out, M->dloss, sizeof(double), cudaMemcpyDeviceToHost, M->st));
    MLP_CUDA(cudaStreamSynchronize(M->st));
  }
  return CS_OK;
}

extern "C" int cs_mlp_gradient(cs_mlp* M, const float* X, const float* Y, int n, double* loss, float* grad) {
  if (!M || !X || !Y || n < 1) return cs_internal_set_error(CS_ERR_INVALID, "cs_mlp_gradient: bad argument");
  int rc = mlp_reserve(M, n);
  if (rc != CS_OK) return rc;
  float *dX = nullptr, *dY = nullptr;
  MLP_CUDA(cudaMalloc(&dX, (size_t)n * M->nin * sizeof(float)));
  MLP_CUDA(cudaMalloc(&dY, (size_t)n * M->nout * sizeof(float)));
  cudaMemcpyAsync(dX, X, (size_t)n * M->nin * sizeof(float), cudaMemcpyHostToDevice, M->st);
  cudaMemcpyAsync(dY, Y, (size_t)n * M->nout * sizeof(float), cudaMemcpyHostToDevice, M->st);
  const float* nr = M->norm;
  k_gather<<<grid_for((long long)n * (M->nin + M->nout)), 256, 0, M->st>>>(
      dX, dY, nullptr, n, M->nin, M->nout, nr, nr + M->nin, nr + 2 * M->nin, nr + 2 * M->nin + M->nout, M->act[0], M->tgt);
  rc = mlp_forward(M, n);
  if (rc == CS_OK) rc = mlp_backward(M, n, loss);
  if (rc == CS_OK && grad) {
    cudaError_t e = cudaMemcpyAsync(grad, M->g, M->nparam * sizeof(float), cudaMemcpyDeviceToHost, M->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(M->st);
    if (e != cudaSuccess) rc = cs_internal_set_error(CS_ERR_CUDA, cudaGetErrorString(e));
  }
  cudaFree(dX);
  cudaFree(dY);
  return rc;
}

extern "C" int cs_mlp_train(cs_mlp* M, const float* X, const float* Y, int n, int epochs, int batch, float lr,
                            unsigned long long seed, double* final_loss) {
  if (!M || !X || !Y || n < 1 || epochs < 1 || batch < 1) return cs_internal_set_error(CS_ERR_INVALID, "cs_mlp_train: bad argument");
  batch = std::min(batch, n);
  int rc = mlp_reserve(M, batch);
  if (rc != CS_OK) return rc;
  float *dX = nullptr, *dY = nullptr;
  MLP_CUDA(cudaMalloc(&dX, (size_t)n * M->nin * sizeof(float)));
  MLP_CUDA(cudaMalloc(&dY, (size_t)n * M->nout * sizeof(float)));
  MLP_CUDA(cudaMemcpyAsync(dX, X, (size_t)n * M->nin * sizeof(float), cudaMemcpyHostToDevice, M->st));
  MLP_CUDA(cudaMemcpyAsync(dY, Y, (size_t)n * M->nout * sizeof(float), cudaMemcpyHostToDevice, M->st));
  int* dperm = nullptr;
  MLP_CUDA(cudaMalloc(&dperm, (size_t)n * sizeof(int)));
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  std::mt19937_64 rng(seed);
  const float* nr = M->norm;
  double last = 0.0;
  // learning rate of step q of this call: constant, or cosine from lr down to
  // lr_final * lr over the call's steps
  const long long total = (long long)epochs * (n / batch);
  long long q = 0;
  for (int ep = 0; ep < epochs && rc == CS_OK; ++ep) {
    std::shuffle(perm.begin(), perm.end(), rng);
    MLP_CUDA(cudaMemcpyAsync(dperm, perm.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, M->st));
    double ep_loss = 0.0;
    int nb = 0;
    for (int s = 0; s + batch <= n && rc == CS_OK; s += batch) {
      k_gather<<<grid_for((long long)batch * (M->nin + M->nout)), 256, 0, M->st>>>(
          dX, dY, dperm + s, batch, M->nin, M->nout, nr, nr + M->nin, nr + 2 * M->nin, nr + 2 * M->nin + M->nout,
          M->act[0], M->tgt);
      rc = mlp_forward(M, batch);
      if (rc == CS_OK) rc = mlp_backward(M, batch, nullptr);
      if (rc != CS_OK) break;
      M->step += 1;
      const float b1 = 0.9f, b2 = 0.999f;
      const float c1 = 1.f - std::pow(b1, (float)M->step), c2 = 1.f - std::pow(b2, (float)M->step);
      float lq = lr;
      if (M->lr_final >= 0.f && total > 1) {
        const double f = M->lr_final + 0.5 * (1.0 - M->lr_final) * (1.0 + std::cos(3.14159265358979323846 * (double)q / (double)(total - 1)));
        lq = (float)(lr * f);
      }
      ++q;
      k_adam<<<grid_for(M->nparam), 256, 0, M->st>>>(M->w, M->g, M->m1, M->m2, M->nparam, lq, b1, b2, 1e-8f, c1, c2);
      ++nb;
    }
    if (rc == CS_OK && ep == epochs - 1) {
      // loss of the final parameters on the last mini-batch
      rc = mlp_forward(M, batch);
      if (rc == CS_OK) rc = mlp_backward(M, batch, &ep_loss);
      last = ep_loss;
    }
    (void)nb;
  }
  cudaError_t e = cudaStreamSynchronize(M->st);
  if (rc == CS_OK && e != cudaSuccess) rc = cs_internal_set_error(CS_ERR_CUDA, cudaGetErrorString(e));
  cudaFree(dX);
  cudaFree(dY);
  cudaFree(dperm);
  if (final_loss) *final_loss = last;
  return rc;
}

extern "C" int cs_mlp_set_schedule(cs_mlp* M, float lr_final) {
  if (!M || lr_final > 1.f) return cs_internal_set_error(CS_ERR_INVALID, "cs_mlp_set_schedule: bad argument");
  M->lr_final = lr_final;
  return CS_OK;
}

extern "C" int cs_mlp_predict_device(cs_mlp* M, const float* dX, int n, float* dY, void* stream) {
  if (!M || !dX || !dY || n < 1) return cs_internal_set_error(CS_ERR_INVALID, "cs_mlp_predict_device: bad argument");
  const int chunk = 65536;
  int rc = mlp_reserve(M, std::min(n, chunk));
  if (rc != CS_OK) return rc;
  cudaStream_t st = stream ? (cudaStream_t)stream : M->st;
  cudaStream_t keep = M->st;
  M->st = st;
  const float* nr = M->norm;
  for (int s = 0; s < n && rc == CS_OK; s += chunk) {
    const int c = std::min(chunk, n - s);
    k_gather<<<grid_for((long long)c * M->nin), 256, 0, st>>>(dX + (size_t)s * M->nin, nullptr, nullptr, c, M->nin, 0,
                                                               nr, nr + M->nin, nullptr, nullptr, M->act[0], nullptr);
    rc = mlp_forward(M, c);
    if (rc != CS_OK) break;
    float* out = M->act[M->depth];
    k_denorm<<<grid_for((long long)c * M->nout), 256, 0, st>>>(out, c, M->nout, nr + 2 * M->nin,
                                                                nr + 2 * M->nin + M->nout);
    cudaMemcpyAsync(dY + (size_t)s * M->nout, out, (size_t)c * M->nout * sizeof(float), cudaMemcpyDeviceToDevice, st);
  }
  M->st = keep;
  cudaError_t e = cudaStreamSynchronize(st);
  if (rc == CS_OK && e != cudaSuccess) rc = cs_internal_set_error(CS_ERR_CUDA, cudaGetErrorString(e));
  return rc;
}

extern "C" int cs_mlp_predict(cs_mlp* M, const float* X, int n, float* Y) {
  if (!M || !X || !Y || n < 1) return cs_internal_set_error(CS_ERR_INVALID, "cs_mlp_predict: bad argument");
  const int chunk = 65536;
  int rc = mlp_reserve(M, std::min(n, chunk));
  if (rc != CS_OK) return rc;
  float* dX = nullptr;
  MLP_CUDA(cudaMalloc(&dX, (size_t)std::min(n, chunk) * M->nin * sizeof(float)));
  const float* nr = M->norm;
  for (int s = 0; s < n && rc == CS_OK; s += chunk) {
    const int c = std::min(chunk, n - s);
    cudaMemcpyAsync(dX, X + (size_t)s * M->nin, (size_t)c * M->nin * sizeof(float), cudaMemcpyHostToDevice, M->st);
    k_gather<<<grid_for((long long)c * M->nin), 256, 0, M->st>>>(dX, nullptr, nullptr, c, M->nin, 0, nr, nr + M->nin,
                                                                  nullptr, nullptr, M->act[0], nullptr);
    rc = mlp_forward(M, c);
    if (rc != CS_OK) break;
    float* out = M->act[M->depth];
    k_denorm<<<grid_for((long long)c * M->nout), 256, 0, M->st>>>(out, c, M->nout, nr + 2 * M->nin,
                                                                   nr + 2 * M->nin + M->nout);
    cudaMemcpyAsync(Y + (size_t)s * M->nout, out, (size_t)c * M->nout * sizeof(float), cudaMemcpyDeviceToHost, M->st);
  }
  cudaError_t e = cudaStreamSynchronize(M->st);
  if (rc == CS_OK && e != cudaSuccess) rc = cs_internal_set_error(CS_ERR_CUDA, cudaGetErrorString(e));
  cudaFree(dX);
  return rc;
}
