// Standalone solve of one bordered almost-block-diagonal (BABD) system, the
// linear system of one Newton step after condensation:
//
//   A_i dy_i + C_i dy_{i+1} + H_i dp = b_i            i = 0 .. n-1
//   B_0 dy_0 + B_n dy_n     + V_n dp = -r              (ny + np rows)
//
// Reference: solve_babd_system.py (partition_factorization_parallel,
// construct_babd_mshoot, qr_decomposition, backward_substitution,
// recover_babd_solution, partition_backward_substitution_parallel,
// solve_babd_system.py:93-572), which sweeps 8 partitions sequentially and
// solves the reduced system on the host.  Here: a tree of pairwise Householder
// eliminations (one warp per merge, every level across the whole system), the
// dense top system with the boundary conditions, and back substitution down
// the tree, all on the device.  Sizes are run-time values (ny <= 32,
// np <= 32), unlike the problem-specialised solver kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "cs_gb300.h"

int cs_internal_set_error(int code, const char* msg);

namespace {

struct BabdDims {
  int ny, np, n;  // block size, parameters, intervals
  int rowsz;      // ny * (2 ny + np + 1): a block row [A | C | H | b], column-major
  int treesz;     // ny * (3 ny + np + 1): a tree record [R | G | E | J | d]
  int qc, qld;    // merge columns, merge leading dimension
  int nt, tld;    // top system size, its leading dimension
};

BabdDims dims_of(int ny, int np, int n) {
  BabdDims d;
  d.ny = ny;
  d.np = np;
  d.n = n;
  d.rowsz = ny * (2 * ny + np + 1);
  d.treesz = ny * (3 * ny + np + 1);
  d.qc = 3 * ny + np + 1;
  d.qld = (2 * ny) | 1;
  d.nt = 2 * ny + np;
  d.tld = d.nt | 1;
  return d;
}

// scratch doubles: two block-row buffers and the tree records
size_t scratch_doubles(const BabdDims& d) {
  return 2 * (size_t)d.n * d.rowsz + (size_t)(d.n + 1) * d.treesz;
}

// A reflection is skipped only for a column that is zero below (and on) the
// diagonal (entries under about 1e-145): any other column is reflected whatever its scale, so a system
// multiplied by any factor gives the same solution (an absolute cut-off of
// the order of eps would leave the columns of a system scaled by 1e-9
// unreduced and the back substitution wrong).
constexpr double kZeroVs = 1e-290;

__device__ __forceinline__ int rows_at(int n0, int l) {
  int n = n0;
  for (int q = 0; q < l; ++q) n = (n + 1) >> 1;
  return n;
}

// inputs in the reference's row-major layout -> column-major block rows
__global__ void kb_pack(BabdDims d, const double* A, const double* C, const double* H, const double* b, double* rows) {
  const long long total = (long long)d.n * d.rowsz;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / d.rowsz);
    const int q = (int)(e - (long long)i * d.rowsz);
    const int c = q / d.ny, r = q - c * d.ny;
    double v;
    if (c < d.ny) v = A[((size_t)i * d.ny + r) * d.ny + c];
    else if (c < 2 * d.ny) v = C[((size_t)i * d.ny + r) * d.ny + (c - d.ny)];
    else if (c < 2 * d.ny + d.np) v = H[((size_t)i * d.ny + r) * d.np + (c - 2 * d.ny)];
    else v = b[(size_t)i * d.ny + r];
    rows[e] = v;
  }
}

// one merge (or the carried odd row) of tree level l, one warp per item
__global__ void kb_level(BabdDims d, int l, const double* src, double* dst, double* tree) {
  extern __shared__ double sm[];
  const int wpc = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* Q = sm + (size_t)w * d.qld * d.qc;
  const int nl = rows_at(d.n, l);
  const int merges = nl >> 1;
  const int items = (nl + 1) >> 1;
  const int ny = d.ny;
  for (int mi = blockIdx.x * wpc + w; mi < items; mi += gridDim.x * wpc) {
    if (mi >= merges) {
      const double* sr = src + (size_t)(nl - 1) * d.rowsz;
      double* dr = dst + (size_t)merges * d.rowsz;
      for (int q = lane; q < d.rowsz; q += 32) dr[q] = sr[q];
      continue;
    }
    const double* ra = src + (size_t)(2 * mi) * d.rowsz;
    const double* rb = src + (size_t)(2 * mi + 1) * d.rowsz;
    for (int c = lane; c < d.qc; c += 32) {
      double* col = Q + (size_t)c * d.qld;
      for (int r = 0; r < ny; ++r) {
        double top, bot;
        if (c < ny) { top = ra[(ny + c) * ny + r]; bot = rb[c * ny + r]; }
        else if (c < 2 * ny) { top = ra[(c - ny) * ny + r]; bot = 0.0; }
        else if (c < 3 * ny) { top = 0.0; bot = rb[(ny + c - 2 * ny) * ny + r]; }
        else { top = ra[(2 * ny + c - 3 * ny) * ny + r]; bot = rb[(2 * ny + c - 3 * ny) * ny + r]; }
        col[r] = top;
        col[ny + r] = bot;
      }
    }
    __syncwarp();
    for (int k = 0; k < ny; ++k) {
      const double* vk = Q + (size_t)k * d.qld;
      double ss = 0.0;
      for (int r = k + lane; r < 2 * ny; r += 32) ss += vk[r] * vk[r];
      for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
      const double x0 = vk[k];
      const double g = (x0 >= 0.0) ? -sqrt(ss) : sqrt(ss);
      const double v0 = x0 - g;
      const double vs = ss - x0 * x0 + v0 * v0;
      __syncwarp();
      if (vs < kZeroVs) continue;
      const double beta = -2.0 / vs;
      for (int c = k + 1 + lane; c < d.qc; c += 32) {
        double* col = Q + (size_t)c * d.qld;
        double wv = v0 * col[k];
        for (int r = k + 1; r < 2 * ny; ++r) wv += vk[r] * col[r];
        const double bw = beta * wv;
        col[k] = fma(bw, v0, col[k]);
        for (int r = k + 1; r < 2 * ny; ++r) col[r] = fma(bw, vk[r], col[r]);
      }
      __syncwarp();
      if (lane == 0) {
        double* col = Q + (size_t)k * d.qld;
        col[k] = g;
        for (int r = k + 1; r < 2 * ny; ++r) col[r] = 0.0;
      }
      __syncwarp();
    }
    const int mid = (2 * mi + 1) << l;
    double* rec = tree + (size_t)mid * d.treesz;
    double* out = dst + (size_t)mi * d.rowsz;
    for (int c = lane; c < d.qc; c += 32) {
      const double* col = Q + (size_t)c * d.qld;
      for (int r = 0; r < ny; ++r) rec[(size_t)c * ny + r] = col[r];
      if (c >= ny)
        for (int r = 0; r < ny; ++r) out[(size_t)(c - ny) * ny + r] = col[ny + r];
    }
    __syncwarp();
  }
}

// top system [At Ct Ht; B_0 B_n V_n] [dy_0; dy_n; dp] = [bt; -r], one warp
__global__ void kb_top(BabdDims d, const double* row, const double* B0, const double* Bn, const double* Vn,
                       const double* r, double* dy, double* dp, int* singular) {
  extern __shared__ double top[];
  const int lane = threadIdx.x & 31;
  const int ny = d.ny, np = d.np, nt = d.nt, tld = d.tld;
  for (int c = lane; c < nt + 1; c += 32) {
    double* col = top + (size_t)c * tld;
    for (int q = 0; q < ny; ++q) col[q] = (c < 2 * ny + np) ? row[(size_t)c * ny + q] : row[(size_t)(2 * ny + np) * ny + q];
    for (int q = 0; q < ny + np; ++q) {
      double v;
      if (c < ny) v = B0[(size_t)q * ny + c];
      else if (c < 2 * ny) v = Bn[(size_t)q * ny + (c - ny)];
      else if (c < nt) v = Vn[(size_t)q * np + (c - 2 * ny)];
      else v = -r[q];
      col[ny + q] = v;
    }
  }
  __syncwarp();
  for (int k = 0; k < nt; ++k) {
    const double* vk = top + (size_t)k * tld;
    double ss = 0.0;
    for (int q = k + lane; q < nt; q += 32) ss += vk[q] * vk[q];
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
    const double x0 = vk[k];
    const double g = (x0 >= 0.0) ? -sqrt(ss) : sqrt(ss);
    const double v0 = x0 - g;
    const double vs = ss - x0 * x0 + v0 * v0;
    __syncwarp();
    if (vs < kZeroVs) continue;
    const double beta = -2.0 / vs;
    for (int c = k + 1 + lane; c < nt + 1; c += 32) {
      double* col = top + (size_t)c * tld;
      double wv = v0 * col[k];
      for (int q = k + 1; q < nt; ++q) wv += vk[q] * col[q];
      const double bw = beta * wv;
      col[k] = fma(bw, v0, col[k]);
      for (int q = k + 1; q < nt; ++q) col[q] = fma(bw, vk[q], col[q]);
    }
    __syncwarp();
    if (lane == 0) {
      double* col = top + (size_t)k * tld;
      col[k] = g;
      for (int q = k + 1; q < nt; ++q) col[q] = 0.0;
    }
    __syncwarp();
  }
  if (lane == 0) {
    double* rhs = top + (size_t)nt * tld;
    int sing = 0;
    for (int q = nt - 1; q >= 0; --q) {
      double v = rhs[q];
      for (int c = q + 1; c < nt; ++c) v -= top[(size_t)c * tld + q] * rhs[c];
      const double dd = top[(size_t)q * tld + q];
      if (dd == 0.0) sing = 1;
      rhs[q] = (dd != 0.0) ? v / dd : 0.0;
    }
    if (sing)
      for (int q = 0; q < nt; ++q) rhs[q] = 0.0;
    *singular = sing;
    for (int q = 0; q < ny; ++q) {
      dy[q] = rhs[q];
      dy[(size_t)d.n * ny + q] = rhs[ny + q];
    }
    for (int q = 0; q < np; ++q) dp[q] = rhs[2 * ny + q];
  }
}

// back substitution of tree level l: dy_m = R^-1 (d - G dy_l - E dy_r - J dp)
__global__ void kb_back(BabdDims d, int l, const double* tree, const double* dp, double* dy) {
  const int wpc = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ny = d.ny, np = d.np;
  const int merges = rows_at(d.n, l) >> 1;
  for (int mi = blockIdx.x * wpc + w; mi < merges; mi += gridDim.x * wpc) {
    const int mid = (2 * mi + 1) << l, left = (2 * mi) << l;
    int right = (2 * mi + 2) << l;
    if (right > d.n) right = d.n;
    const double* rec = tree + (size_t)mid * d.treesz;
    const double* yl = dy + (size_t)left * ny;
    const double* yr = dy + (size_t)right * ny;
    double v = 0.0;
    if (lane < ny) {
      v = rec[(size_t)(3 * ny + np) * ny + lane];
      for (int c = 0; c < ny; ++c) v -= rec[(size_t)(ny + c) * ny + lane] * yl[c];
      for (int c = 0; c < ny; ++c) v -= rec[(size_t)(2 * ny + c) * ny + lane] * yr[c];
      for (int c = 0; c < np; ++c) v -= rec[(size_t)(3 * ny + c) * ny + lane] * dp[c];
    }
    for (int q = ny - 1; q >= 0; --q) {
      double xq = __shfl_sync(0xffffffffu, v, q);
      const double rr = rec[(size_t)q * ny + q];
      xq = (rr != 0.0) ? xq / rr : 0.0;
      if (lane == q) v = xq;
      if (lane < q) v -= rec[(size_t)q * ny + lane] * xq;
    }
    if (lane < ny) dy[(size_t)mid * ny + lane] = v;
  }
}

int levels_of(int n) {
  int L = 0;
  while (n > 1) {
    n = (n + 1) >> 1;
    ++L;
  }
  return L;
}

int check_sizes(int ny, int np, int n) {
  if (ny < 1 || ny > 32 || np < 0 || np > 32 || n < 1)
    return cs_internal_set_error(CS_ERR_INVALID, "cs_babd_solve: need 1 <= ny <= 32, 0 <= np <= 32, n >= 1");
  return CS_OK;
}

// the whole solve on `stream`, with `scratch` holding scratch_doubles(d) doubles
int babd_run(const BabdDims& d, const double* A, const double* C, const double* H, const double* b, const double* B0,
             const double* Bn, const double* Vn, const double* r, double* dy, double* dp, double* scratch,
             int* d_singular, cudaStream_t stream) {
  double* rows0 = scratch;
  double* rows1 = rows0 + (size_t)d.n * d.rowsz;
  double* tree = rows1 + (size_t)d.n * d.rowsz;
  const long long pack = (long long)d.n * d.rowsz;
  kb_pack<<<(unsigned)std::min<long long>((pack + 255) / 256, 65535), 256, 0, stream>>>(d, A, C, H, b, rows0);
  const int L = levels_of(d.n);
  const size_t per_warp = (size_t)d.qld * d.qc * sizeof(double);
  const int wpc = (int)std::max<size_t>(1, std::min<size_t>(4, (size_t)(200 * 1024) / per_warp));
  const size_t lsm = per_warp * wpc;
  if (lsm > 48 * 1024) cudaFuncSetAttribute(kb_level, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsm);
  double* src = rows0;
  double* dst = rows1;
  for (int l = 0; l < L; ++l) {
    int items = d.n;
    for (int q = 0; q <= l; ++q) items = (items + 1) >> 1;
    const unsigned grid = (unsigned)std::max(1, std::min(65535, (items + wpc - 1) / wpc));
    kb_level<<<grid, 32 * wpc, lsm, stream>>>(d, l, src, dst, tree);
    std::swap(src, dst);
  }
  const size_t tsm = (size_t)d.tld * (d.nt + 1) * sizeof(double);
  if (tsm > 48 * 1024) cudaFuncSetAttribute(kb_top, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm);
  kb_top<<<1, 32, tsm, stream>>>(d, src, B0, Bn, Vn, r, dy, dp, d_singular);
  for (int l = L - 1; l >= 0; --l) {
    const int merges = ([&] {
      int m = d.n;
      for (int q = 0; q < l; ++q) m = (m + 1) >> 1;
      return m >> 1;
    })();
    const unsigned grid = (unsigned)std::max(1, std::min(65535, (merges + 3) / 4));
    kb_back<<<grid, 128, 0, stream>>>(d, l, tree, dp, dy);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cs_internal_set_error(CS_ERR_CUDA, cudaGetErrorString(e));
  return CS_OK;
}

// ---------------------------------------------------------------------------
// Scratch for cs_babd_solve_noalloc: one array in the device image of this
// library, so that callers that cannot allocate device memory can still solve
// a BABD system.  Every GPU that loads the library holds it until the process
// exits.  Element 0 carries the singular flag; the block rows and tree records
// start at element 32 (256-byte aligned).
constexpr size_t kNoallocDoubles = (size_t)4 << 20;  // 32 MiB
__device__ __align__(256) double cs_babd_scratch[kNoallocDoubles];

std::mutex g_noalloc_mu;
void* g_noalloc_addr[128] = {nullptr};

// device address of the scratch array on the current device, looked up once
// per device (host code cannot use the symbol itself as an address)
int noalloc_scratch(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cs_internal_set_error(CS_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= 128) return cs_internal_set_error(CS_ERR_CUDA, "cs_babd_solve_noalloc: device index out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, cs_babd_scratch);
    if (e != cudaSuccess || !p)
      return cs_internal_set_error(CS_ERR_CUDA, (std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
    g_noalloc_addr[dev] = p;
  }
  *out = (double*)g_noalloc_addr[dev];
  return CS_OK;
}

}  // namespace

extern "C" int cs_babd_solve_noalloc(int ny, int np, int n, const double* A, const double* C, const double* H,
                                     const double* b, const double* B0, const double* Bn, const double* Vn,
                                     const double* r, double* dy, double* dp, int* singular, void* stream) {
  int rc = check_sizes(ny, np, n);
  if (rc != CS_OK) return rc;
  if (!A || !C || !b || !B0 || !Bn || !r || !dy || (np > 0 && (!H || !Vn || !dp)))
    return cs_internal_set_error(CS_ERR_INVALID, "cs_babd_solve_noalloc: null pointer");
  const BabdDims d = dims_of(ny, np, n);
  const size_t need = 32 + scratch_doubles(d);
  if (need > kNoallocDoubles)
    return cs_internal_set_error(
        CS_ERR_INVALID, ("cs_babd_solve_noalloc: the system needs " + std::to_string(need * sizeof(double)) +
                         " bytes of scratch, more than the fixed " + std::to_string(kNoallocDoubles * sizeof(double)) +
                         " bytes; use cs_babd_solve").c_str());
  double* base = nullptr;
  rc = noalloc_scratch(&base);
  if (rc != CS_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // every element read below is written earlier in the same call (packing,
  // tree levels, top system), so nothing needs clearing between calls
  int* dsing = (int*)base;
  rc = babd_run(d, A, C, H, b, B0, Bn, Vn, r, dy, dp, base + 32, dsing, st);
  int hs = 0;
  if (rc == CS_OK) {
    cudaError_t e = cudaMemcpyAsync(&hs, dsing, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cs_internal_set_error(CS_ERR_CUDA, cudaGetErrorString(e));
  }
  if (singular) *singular = hs;
  return rc;
}

extern "C" int cs_babd_solve(int ny, int np, int n, const double* A, const double* C, const double* H,
                             const double* b, const double* B0, const double* Bn, const double* Vn, const double* r,
                             double* dy, double* dp, int* singular, void* stream) {
  int rc = check_sizes(ny, np, n);
  if (rc != CS_OK) return rc;
  if (!A || !C || !b || !B0 || !Bn || !r || !dy || (np > 0 && (!H || !Vn || !dp)))
    return cs_internal_set_error(CS_ERR_INVALID, "cs_babd_solve: null pointer");
  const BabdDims d = dims_of(ny, np, n);
  cudaStream_t st = (cudaStream_t)stream;
  double* scratch = nullptr;
  int* dsing = nullptr;
  cudaError_t e = cudaMalloc(&scratch, scratch_doubles(d) * sizeof(double));
  if (e != cudaSuccess) return cs_internal_set_error(CS_ERR_NOMEM, "cs_babd_solve: cudaMalloc failed");
  e = cudaMalloc(&dsing, sizeof(int));
  if (e != cudaSuccess) {
    cudaFree(scratch);
    return cs_internal_set_error(CS_ERR_NOMEM, "cs_babd_solve: cudaMalloc failed");
  }
  rc = babd_run(d, A, C, H, b, B0, Bn, Vn, r, dy, dp, scratch, dsing, st);
  int hs = 0;
  if (rc == CS_OK) {
    e = cudaMemcpyAsync(&hs, dsing, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cs_internal_set_error(CS_ERR_CUDA, cudaGetErrorString(e));
  }
  cudaFree(scratch);
  cudaFree(dsing);
  if (singular) *singular = hs;
  return rc;
}
