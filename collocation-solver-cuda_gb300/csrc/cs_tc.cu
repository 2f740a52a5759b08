// cs_tc_update: the tensor-core block update C -= A B^T (FP32 C, A and B
// rounded to TF32 or BF16, FP32 accumulation in TMEM) on one matrix in device
// memory, one CTA.  It runs the same device routine (cs_umma.cuh) as the
// trailing update of the reduced-precision condensation of large stage
// systems, so the tests pin that routine against numpy.
#include <cuda_runtime.h>

#include <string>

#include "cs_gb300.h"
#include "cs_umma.cuh"

int cs_internal_set_error(int code, const char* msg);

namespace {

constexpr int kMaxM = 256, kMaxN = 512, kMaxK = 64;
constexpr long long kWaitCycles = 2000000000ll;  // about one second

// shared memory: A_s [Mp x kc x 16 B] | B_s [Np x kc x 16 B] | mbar | tmem slot | flag
template <int PREC>
__global__ void __launch_bounds__(256) k_tc_update(int M, int N, int K, const float* A, int lda, const float* B,
                                                   int ldb, float* C, int ldc, int kc, int nks, int* status) {
  extern __shared__ __align__(128) unsigned char sm[];
  constexpr int EPS = CsTcElems<PREC>::per_seg;
  const int Mp = (M + 127) & ~127, Np = (N + 15) & ~15;
  unsigned char* A_s = sm;
  unsigned char* B_s = A_s + (size_t)Mp * kc * 16;
  unsigned long long* mbar = reinterpret_cast<unsigned long long*>(B_s + (size_t)Np * kc * 16);
  unsigned* slot = reinterpret_cast<unsigned*>(mbar + 1);
  int* flag = reinterpret_cast<int*>(slot + 1);
  const int tid = threadIdx.x, nt = blockDim.x;
  // stage the operands (zeros past M, N and K)
  for (int e = tid; e < Mp * kc; e += nt) {
    const int r = e / kc, q = e - r * kc;
    float x[EPS];
#pragma unroll
    for (int j = 0; j < EPS; ++j) {
      const int k = q * EPS + j;
      x[j] = (r < M && k < K) ? A[(size_t)r * lda + k] : 0.f;
    }
    cs_tc_put<PREC>(A_s, r, q, kc, x);
  }
  for (int e = tid; e < Np * kc; e += nt) {
    const int r = e / kc, q = e - r * kc;
    float x[EPS];
#pragma unroll
    for (int j = 0; j < EPS; ++j) {
      const int k = q * EPS + j;
      x[j] = (r < N && k < K) ? B[(size_t)r * ldb + k] : 0.f;
    }
    cs_tc_put<PREC>(B_s, r, q, kc, x);
  }
  cs_fence_async_smem();
  if (tid == 0) {
    cs_mbar_init(cs_sa(mbar), 1);
    *flag = 0;
  }
  if (tid < 32) cs_tmem_alloc(cs_sa(slot), CS_TC_COLS);
  cs_tc_before_sync();
  __syncthreads();
  cs_tc_after_sync();
  const unsigned tmem = *slot;
  unsigned phase = 0;
  const bool ok =
      cs_tc_block_update<PREC>(C, ldc, 1, M, N, A_s, B_s, kc, nks, tmem, cs_sa(mbar), phase, kWaitCycles, flag);
  cs_tc_before_sync();
  __syncthreads();
  if (tid < 32) {
    cs_tc_after_sync();
    cs_tmem_free(tmem, CS_TC_COLS);
  }
  if (tid == 0) *status = ok ? 0 : 1;
}

template <int PREC>
int launch(int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc, int* status,
           cudaStream_t st) {
  // K padded to whole k-steps (32 bytes of K per MMA)
  constexpr int per_step = (PREC == 1) ? 8 : 16;
  const int nks = (K + per_step - 1) / per_step;
  const int kc = 2 * nks;
  const int Mp = (M + 127) & ~127, Np = (N + 15) & ~15;
  const size_t smem = (size_t)(Mp + Np) * kc * 16 + 16;
  cudaError_t e = cudaFuncSetAttribute(k_tc_update<PREC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cs_internal_set_error(CS_ERR_CUDA, cudaGetErrorString(e));
  k_tc_update<PREC><<<1, 256, smem, st>>>(M, N, K, A, lda, B, ldb, C, ldc, kc, nks, status);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cs_internal_set_error(CS_ERR_CUDA, cudaGetErrorString(e));
  return CS_OK;
}

}  // namespace

extern "C" int cs_tc_update(int precision, int M, int N, int K, const float* A, int lda, const float* B, int ldb,
                            float* C, int ldc, void* stream) {
  if (precision != 1 && precision != 2)
    return cs_internal_set_error(CS_ERR_INVALID, "cs_tc_update: precision must be 1 (TF32) or 2 (BF16)");
  if (M < 1 || M > kMaxM || N < 1 || N > kMaxN || K < 1 || K > kMaxK)
    return cs_internal_set_error(CS_ERR_INVALID, "cs_tc_update: need 1 <= M <= 256, 1 <= N <= 512, 1 <= K <= 64");
  if (!A || !B || !C || lda < K || ldb < K || ldc < N)
    return cs_internal_set_error(CS_ERR_INVALID, "cs_tc_update: null pointer or leading dimension too small");
  cudaStream_t st = (cudaStream_t)stream;
  int* dstatus = nullptr;
  cudaError_t e = cudaMalloc(&dstatus, sizeof(int));
  if (e != cudaSuccess) return cs_internal_set_error(CS_ERR_NOMEM, "cs_tc_update: cudaMalloc failed");
  int rc = (precision == 1) ? launch<1>(M, N, K, A, lda, B, ldb, C, ldc, dstatus, st)
                            : launch<2>(M, N, K, A, lda, B, ldb, C, ldc, dstatus, st);
  int hs = 0;
  if (rc == CS_OK) {
    e = cudaMemcpyAsync(&hs, dstatus, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cs_internal_set_error(CS_ERR_CUDA, cudaGetErrorString(e));
    else if (hs != 0) rc = cs_internal_set_error(CS_ERR_STATE, "cs_tc_update: tensor-core MMA did not complete");
  }
  cudaFree(dstatus);
  return rc;
}
