// Solution files of a whole batch as text, formatted on the GPU.
//
// The reference writes each solution with a Python loop over every value
// ('{}'.format, BVPDAEReadWriteData.py:337-364).  Here one thread per value
// prints its shortest round-trip text (cs_dtoa.h) into a fixed 24-byte slot,
// one CTA per instance adds up its file's size, and one CTA per instance
// places the slots and the fixed labels at their byte offsets (block-wide
// prefix sums over the values and rows).  The text is byte for byte the
// reference's file for the same values.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "cs_dtoa.h"
#include "cs_gb300.h"
#include "cs_text.h"

int cs_internal_set_error(int code, const char* msg);

namespace {

// decimal text of a non-negative int; returns the length
__host__ __device__ inline int cs_itoa(int v, char* out) {
  char tmp[12];
  int n = 0;
  do {
    tmp[n++] = (char)('0' + v % 10);
    v /= 10;
  } while (v > 0);
  for (int i = 0; i < n; ++i) out[i] = tmp[n - 1 - i];
  return n;
}

__host__ __device__ inline int cs_itoa_len(int v) {
  int n = 1;
  while (v >= 10) {
    v /= 10;
    ++n;
  }
  return n;
}

// labels of a file: "nt:\n<N>\nt:\n", "\nny:\n<ny>\ny:\n", "nz:\n<nz>\nz:\n", "np:\n<np>\np:\n"
__host__ __device__ inline int cs_label(int which, int v, char* out) {
  const char* pre[4] = {"nt:\n", "\nny:\n", "nz:\n", "np:\n"};
  const char* post[4] = {"\nt:\n", "\ny:\n", "\nz:\n", "\np:\n"};
  int p = 0;
  for (const char* c = pre[which]; *c; ++c) out[p++] = *c;
  p += cs_itoa(v, out + p);
  for (const char* c = post[which]; *c; ++c) out[p++] = *c;
  return p;
}

__host__ __device__ inline int cs_label_len(int which, int v) { return (which == 1 ? 9 : 8) + cs_itoa_len(v); }

struct CsTextSrc {
  const double *t, *y, *z, *p;
  long long T;
  int B, ny, nz, np;
  const int *N, *off;
  char* slot;           // CS_DTOA_MAX bytes per value
  unsigned char* len;   // text length per value
};

// value g: t[g] for g < T, then y (T x ny), z (T x nz), p (B x np)
__device__ inline double cs_text_value(const CsTextSrc& s, long long g) {
  if (g < s.T) return s.t[g];
  g -= s.T;
  if (g < s.T * s.ny) return s.y[g];
  g -= s.T * s.ny;
  if (g < s.T * s.nz) return s.z[g];
  g -= s.T * s.nz;
  return s.p[g];
}

__global__ void k_text_values(CsTextSrc s, long long nv) {
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < nv; g += (long long)gridDim.x * blockDim.x) {
    char buf[CS_DTOA_MAX];
    const int n = cs_format_double_text(cs_text_value(s, g), buf);
    char* d = s.slot + g * CS_DTOA_MAX;
    for (int i = 0; i < n; ++i) d[i] = buf[i];
    s.len[g] = (unsigned char)n;
  }
}

// exclusive prefix sum of v over the CTA (blockDim a multiple of 32, <= 1024);
// *total: the CTA's sum.  sh: 33 long longs of shared memory.
__device__ long long cs_block_exscan(long long v, long long* sh, long long* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    long long q = lane < nw ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, q, o);
      if (lane >= o) q += y;
    }
    if (lane < nw) sh[lane] = q;  // inclusive sums of the warps
    if (lane == 31) sh[32] = q;
  }
  __syncthreads();
  const long long before = (w > 0 ? sh[w - 1] : 0) + x - v;
  *total = sh[32];
  __syncthreads();
  return before;
}

__device__ inline long long cs_vlen(const CsTextSrc& s, long long g) { return (long long)s.len[g] + 1; }

// bytes of the rows [i] of a section with `w` values per row (+ "\n" per row)
__device__ inline long long cs_row_bytes(const CsTextSrc& s, long long first, int w, int i) {
  long long n = 1;
  for (int j = 0; j < w; ++j) n += cs_vlen(s, first + (long long)i * w + j);
  return n;
}

// one CTA per instance: its file's size
__global__ void k_text_sizes(CsTextSrc s, long long* size) {
  __shared__ long long sh[33];
  const int b = blockIdx.x;
  if (b >= s.B) return;
  const int N = s.N[b], o = s.off[b];
  long long acc = 0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    acc += cs_vlen(s, o + i);
    acc += cs_row_bytes(s, s.T + (long long)o * s.ny, s.ny, i);
    acc += cs_row_bytes(s, s.T + s.T * s.ny + (long long)o * s.nz, s.nz, i);
  }
  for (int j = threadIdx.x; j < s.np; j += blockDim.x) acc += cs_vlen(s, s.T * (1 + s.ny + s.nz) + (long long)b * s.np + j);
  long long tot = 0;
  cs_block_exscan(acc, sh, &tot);
  if (threadIdx.x == 0)
    size[b] = tot + cs_label_len(0, N) + cs_label_len(1, s.ny) + cs_label_len(2, s.nz) + cs_label_len(3, s.np);
}

__device__ inline void cs_put_value(const CsTextSrc& s, long long g, char* d) {
  const int n = s.len[g];
  const char* src = s.slot + g * CS_DTOA_MAX;
  for (int i = 0; i < n; ++i) d[i] = src[i];
  d[n] = ' ';
}

// one CTA per instance: its file at out + offset[b]
__global__ void k_text_write(CsTextSrc s, const long long* offset, char* out) {
  __shared__ long long sh[33];
  const int b = blockIdx.x;
  if (b >= s.B) return;
  const int N = s.N[b], o = s.off[b];
  char* base = out + offset[b];
  long long pos = 0;
  if (threadIdx.x == 0) cs_label(0, N, base);
  pos += cs_label_len(0, N);
  // t: one value per node
  for (int c = 0; c < N; c += blockDim.x) {
    const int i = c + threadIdx.x;
    const long long L = i < N ? cs_vlen(s, o + i) : 0;
    long long tot = 0;
    const long long at = cs_block_exscan(L, sh, &tot);
    if (i < N) cs_put_value(s, o + i, base + pos + at);
    pos += tot;
  }
  // y and z: one row per node
  for (int sec = 0; sec < 2; ++sec) {
    const int w = sec == 0 ? s.ny : s.nz;
    const long long first = s.T + (sec == 0 ? 0 : s.T * s.ny) + (long long)o * w;
    if (threadIdx.x == 0) cs_label(1 + sec, w, base + pos);
    pos += cs_label_len(1 + sec, w);
    for (int c = 0; c < N; c += blockDim.x) {
      const int i = c + threadIdx.x;
      const long long L = i < N ? cs_row_bytes(s, first, w, i) : 0;
      long long tot = 0;
      const long long at = cs_block_exscan(L, sh, &tot);
      if (i < N) {
        char* d = base + pos + at;
        for (int j = 0; j < w; ++j) {
          const long long g = first + (long long)i * w + j;
          cs_put_value(s, g, d);
          d += cs_vlen(s, g);
        }
        *d = '\n';
      }
      pos += tot;
    }
  }
  // p
  if (threadIdx.x == 0) {
    char* d = base + pos + cs_label(3, s.np, base + pos);
    for (int j = 0; j < s.np; ++j) {
      const long long g = s.T * (1 + s.ny + s.nz) + (long long)b * s.np + j;
      cs_put_value(s, g, d);
      d += cs_vlen(s, g);
    }
  }
}

struct DevMem {
  void* p = nullptr;
  ~DevMem() {
    if (p) cudaFree(p);
  }
};

}  // namespace

extern "C" int cs_format_double(double v, char* out) {
  if (!out) {
    cs_internal_set_error(CS_ERR_INVALID, "cs_format_double: null output");
    return -1;
  }
  const int n = cs_format_double_text(v, out);
  out[n] = 0;
  return n;
}

#define CS_TRYC(call, what)                                                                          \
  do {                                                                                               \
    cudaError_t e_ = (call);                                                                         \
    if (e_ != cudaSuccess) return cs_internal_set_error(CS_ERR_CUDA, (std::string(what) + ": " + cudaGetErrorString(e_)).c_str()); \
  } while (0)

int cs_text_files(const CsTextArgs& a, char* out, long long cap, long long* offsets) {
  const long long nv = a.T * (1 + a.ny + a.nz) + (long long)a.B * a.np;
  DevMem slot, len, size, dout;
  CS_TRYC(cudaMalloc(&slot.p, (size_t)std::max(nv, 1ll) * CS_DTOA_MAX), "cs_format_solutions: text slots");
  CS_TRYC(cudaMalloc(&len.p, (size_t)std::max(nv, 1ll)), "cs_format_solutions: text lengths");
  CS_TRYC(cudaMalloc(&size.p, (size_t)(a.B + 1) * sizeof(long long)), "cs_format_solutions: sizes");
  CsTextSrc s;
  s.t = a.t;
  s.y = a.y;
  s.z = a.z;
  s.p = a.p;
  s.T = a.T;
  s.B = a.B;
  s.ny = a.ny;
  s.nz = a.nz;
  s.np = a.np;
  s.N = a.dN;
  s.off = a.doff;
  s.slot = (char*)slot.p;
  s.len = (unsigned char*)len.p;
  cudaStream_t st = (cudaStream_t)a.stream;
  // the digit generation keeps four ~160-byte integers per thread (a 1.2 KB
  // frame): make sure this context's per-thread stack holds it
  size_t stack = 0;
  CS_TRYC(cudaDeviceGetLimit(&stack, cudaLimitStackSize), "cs_format_solutions: stack limit");
  if (stack < 2048) CS_TRYC(cudaDeviceSetLimit(cudaLimitStackSize, 2048), "cs_format_solutions: stack limit");
  if (nv > 0) {
    const long long blocks = std::min<long long>((nv + 255) / 256, 152ll * 32);
    k_text_values<<<(unsigned)blocks, 256, 0, st>>>(s, nv);
    CS_TRYC(cudaGetLastError(), "k_text_values");
  }
  k_text_sizes<<<a.B, 256, 0, st>>>(s, (long long*)size.p);
  CS_TRYC(cudaGetLastError(), "k_text_sizes");
  std::vector<long long> hs(a.B);
  CS_TRYC(cudaMemcpyAsync(hs.data(), size.p, (size_t)a.B * sizeof(long long), cudaMemcpyDeviceToHost, st),
          "cs_format_solutions: sizes to host");
  CS_TRYC(cudaStreamSynchronize(st), "cs_format_solutions");
  offsets[0] = 0;
  for (int b = 0; b < a.B; ++b) offsets[b + 1] = offsets[b] + hs[b];
  const long long total = offsets[a.B];
  if (!out) return CS_OK;
  if (cap < total) return cs_internal_set_error(CS_ERR_INVALID, "cs_format_solutions: output buffer too small");
  CS_TRYC(cudaMemcpyAsync(size.p, offsets, (size_t)(a.B + 1) * sizeof(long long), cudaMemcpyHostToDevice, st),
          "cs_format_solutions: offsets");
  CS_TRYC(cudaMalloc(&dout.p, (size_t)std::max(total, 1ll)), "cs_format_solutions: text");
  k_text_write<<<a.B, 256, 0, st>>>(s, (const long long*)size.p, (char*)dout.p);
  CS_TRYC(cudaGetLastError(), "k_text_write");
  CS_TRYC(cudaMemcpyAsync(out, dout.p, (size_t)total, cudaMemcpyDeviceToHost, st), "cs_format_solutions: text to host");
  CS_TRYC(cudaStreamSynchronize(st), "cs_format_solutions");
  return CS_OK;
}
