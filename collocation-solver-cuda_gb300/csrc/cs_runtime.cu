// Host runtime of the GB300 collocation solver: run-time compilation of the
// problem-specialised kernels (NVRTC, sm_103a, cached cubins), the batch
// workspace in HBM, the solve driver and the C ABI declared in cs_gb300.h.
//
// The driver follows collocation_solver_parallel (collocation_solver_parallel_2d_shared.py:36-251)
// but keeps the whole Newton loop on the device: each "super-step" launches
//   k_residual -> k_decide -> k_accept -> k_condense -> k_babd
// and every instance advances its own state machine (fresh residual, line
// search trial, converged, failed) inside those kernels.  The host only
// checks, every few super-steps, whether any instance is still in Newton, and
// runs the mesh phase (segment residual, remesh with repacking) between
// Newton phases.
#include <cuda.h>
#include <cuda_profiler_api.h>
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

#include "cs_text.h"
#include "cs_gb300.h"
#include "cs_kernels_src.h"  // generated: const char* cs_kernels_source

namespace {

thread_local std::string g_err;

int set_err(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CS_CUDA(call)                                                                            \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess)                                                                       \
      return set_err(e_ == cudaErrorMemoryAllocation ? CS_ERR_NOMEM : CS_ERR_CUDA,               \
                     std::string(#call) + ": " + cudaGetErrorString(e_));                        \
  } while (0)

// Driver API entry points, resolved through the runtime on first use so that
// the library loads (and its C ABI can be inspected) on a machine without a
// CUDA driver.
struct DriverApi {
  decltype(&cuModuleLoadData) moduleLoadData = nullptr;
  decltype(&cuModuleGetFunction) moduleGetFunction = nullptr;
  decltype(&cuModuleUnload) moduleUnload = nullptr;
  decltype(&cuLaunchKernel) launchKernel = nullptr;
  decltype(&cuFuncSetAttribute) funcSetAttribute = nullptr;
  decltype(&cuGetErrorString) getErrorString = nullptr;
  decltype(&cuOccupancyMaxActiveBlocksPerMultiprocessor) occupancy = nullptr;
  bool ok = false;
};
DriverApi g_drv;

const char* drv_err(CUresult r) {
  const char* s = nullptr;
  if (g_drv.getErrorString) g_drv.getErrorString(r, &s);
  return s ? s : "unknown driver error";
}

#define CS_CU(call)                                                                              \
  do {                                                                                           \
    CUresult r_ = (call);                                                                        \
    if (r_ != CUDA_SUCCESS) {                                                                    \
      const char* s_ = drv_err(r_);                                                              \
      return set_err(r_ == CUDA_ERROR_OUT_OF_MEMORY ? CS_ERR_NOMEM : CS_ERR_CUDA,                \
                     std::string(#call) + ": " + (s_ ? s_ : "?"));                               \
    }                                                                                            \
  } while (0)

#define CS_TRY(call)           \
  do {                         \
    int rc_ = (call);          \
    if (rc_ != CS_OK) return rc_; \
  } while (0)

// Must match struct CsInst in cs_kernels.cuh.
static const int CS_LSW = 20;  // line-search trials per super-step (cs_kernels.cuh)
struct CsInst {
  int status, it, ls_it, alphacal;
  int need_jac, accepted, fail_reason, N_new;
  int residual_count, jac_count, seg_count, remesh_count;
  int iter_time, singular, ntrial, ls_prev;
  double alpha_ls, norm_x, alpha, max_res;
  unsigned long long norm_bits, res_bits;
};
static_assert(sizeof(CsInst) == 112, "CsInst layout");

struct CsConsts {
  double tol, alpha_m, beta;
  int max_iter, max_mesh, max_nodes, min_nodes, max_ls;
  int ls_grow;
};

// Must match struct CsBatch in cs_kernels.cuh.
struct CsBatchDev {
  int B, T;
  const int* N;
  const int* off;
  const int* inst_of;
  double* t;
  double* y;
  double* ydot;
  double* zt;
  double* p;
  const double* th;
  double* dy;
  double* dydot;
  double* dzt;
  double* dp;
  double* X;
  double* rows0;
  double* rows1;
  double* tree;
  double* res;
  double* znode;
  CsInst* inst;
  unsigned long long* counters;
  double* fa_out;
  double* fb_out;
  int* act;
  int* jac;
  int* acc;
  long long* act_pre;
  long long* jac_pre;
  long long* acc_pre;
  long long* lvl_pre;
  int* nlist;
  unsigned long long* trials;
  double* wsp;
  long long wsp_stride;
  int wsp_ctas, wsp_pad;
};

static const int CS_MAXLVL = 32;

enum { ST_FRESH = 0, ST_LS = 1, ST_SEG = 2, ST_DONE = 3, ST_FAIL = 4, ST_REMESH = 5, ST_PARKED = 6, ST_CANCELLED = 7 };
enum { FAIL_NONE = 0, FAIL_ITER = 1, FAIL_NODES = 2, FAIL_MESH = 3 };

// the record of an instance starting Newton at continuation parameter alpha0
__host__ __device__ inline void init_inst(CsInst& s, double alpha0) {
  memset(&s, 0, sizeof(s));
  s.status = ST_FRESH;
  s.alpha = alpha0;
  s.alpha_ls = 1.0;
}

uint64_t fnv1a(const std::string& s, uint64_t h = 1469598103934665603ull) {
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ull;
  }
  return h;
}

std::string fmt_array(const double* a, int n) {
  std::ostringstream o;
  o.precision(17);
  for (int i = 0; i < n; ++i) o << (i ? "," : "") << std::scientific << a[i];
  if (n == 0) o << "0.0";
  return o.str();
}

bool read_file(const std::string& path, std::vector<char>& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  return !out.empty();
}

void mkdirs(const std::string& path) {
  std::string cur;
  for (size_t i = 0; i < path.size(); ++i) {
    cur += path[i];
    if (path[i] == '/' || i + 1 == path.size()) mkdir(cur.c_str(), 0755);
  }
}

int resolve(const char* name, void** fn) {
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion(name, fn, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !*fn)
    return set_err(CS_ERR_CUDA, std::string("driver entry point not found: ") + name);
  return CS_OK;
}

int ensure_context() {
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  CS_CUDA(cudaFree(nullptr));  // creates / binds the primary context for the driver API too
  if (!g_drv.ok) {
    CS_TRY(resolve("cuModuleLoadData", (void**)&g_drv.moduleLoadData));
    CS_TRY(resolve("cuModuleGetFunction", (void**)&g_drv.moduleGetFunction));
    CS_TRY(resolve("cuModuleUnload", (void**)&g_drv.moduleUnload));
    CS_TRY(resolve("cuLaunchKernel", (void**)&g_drv.launchKernel));
    CS_TRY(resolve("cuFuncSetAttribute", (void**)&g_drv.funcSetAttribute));
    CS_TRY(resolve("cuGetErrorString", (void**)&g_drv.getErrorString));
    CS_TRY(resolve("cuOccupancyMaxActiveBlocksPerMultiprocessor", (void**)&g_drv.occupancy));
    g_drv.ok = true;
  }
  return CS_OK;
}

__global__ void k_fill_inst_of(int B, const int* off, const int* N, int* inst_of) {
  int b = blockIdx.x;
  if (b >= B) return;
  for (int i = threadIdx.x; i < N[b]; i += blockDim.x) inst_of[off[b] + i] = b;
}

__global__ void k_dfma_peak(double* out, int iters) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
         a7 = a0 + 7;
  const double m = 0.999999, c = 1e-7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
    a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
  }
  double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678) out[0] = s;
}

// FP64 tensor-core (DMMA, mma.sync m8n8k4) throughput: four independent
// accumulator tiles per warp
__global__ void k_dmma_peak(double* out, int iters) {
  const double a = threadIdx.x * 1e-3, b = 0.999;
  double c[4][2];
#pragma unroll
  for (int q = 0; q < 4; ++q) c[q][0] = c[q][1] = q;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 4; ++q)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(c[q][0]), "+d"(c[q][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < 4; ++q) s += c[q][0] + c[q][1];
  if (s == 12345.678) out[0] = s;
}

// y, z at the nodes of every instance from its trajectory vector (linear in
// normalised time on n_nodes equispaced nodes), and p from its tail
__global__ void k_warm_fill(int B, int ny, int nz, int np, int n_nodes, const float* traj, int stride, const int* N,
                            const int* off, const double* t, double* y, double* znode, double* p) {
  const int b = blockIdx.x;
  if (b >= B) return;
  const float* v = traj + (size_t)b * stride;
  const int o = off[b], n = N[b];
  const double t0 = t[o], span = t[o + n - 1] - t0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double x = (span > 0.0) ? (t[o + i] - t0) / span * (double)(n_nodes - 1) : 0.0;
    if (x < 0.0) x = 0.0;
    if (x > (double)(n_nodes - 1)) x = (double)(n_nodes - 1);
    int k = (int)x;
    if (k > n_nodes - 2) k = n_nodes - 2;
    if (k < 0) k = 0;
    const double w = (n_nodes > 1) ? x - (double)k : 0.0;
    const int k1 = (n_nodes > 1) ? k + 1 : k;
    for (int c = 0; c < ny; ++c)
      y[(size_t)(o + i) * ny + c] = (1.0 - w) * (double)v[(size_t)k * ny + c] + w * (double)v[(size_t)k1 * ny + c];
    const float* vz = v + (size_t)n_nodes * ny;
    for (int c = 0; c < nz; ++c)
      znode[(size_t)(o + i) * nz + c] = (1.0 - w) * (double)vz[(size_t)k * nz + c] + w * (double)vz[(size_t)k1 * nz + c];
  }
  if (threadIdx.x == 0) {
    const float* vp = v + (size_t)n_nodes * (ny + nz);
    for (int c = 0; c < np; ++c) p[(size_t)b * np + c] = (double)vp[c];
  }
}

// One thread per primary k (spare n + k): start the parked spare of a primary
// still in Newton or failed, stop the running spare of a primary that
// succeeded.  counts[0] / counts[1]: spares started / stopped.
__global__ void k_spares(int n, CsInst* inst, double alpha0, int* counts) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int ps = inst[k].status;
  CsInst& q = inst[n + k];
  const int ss = q.status;
  if (ss == ST_PARKED && (ps == ST_FRESH || ps == ST_LS || ps == ST_FAIL)) {
    CsInst f;
    init_inst(f, alpha0);
    q = f;
    atomicAdd(&counts[0], 1);
  } else if (ps == ST_DONE && (ss == ST_FRESH || ss == ST_LS || ss == ST_SEG)) {
    q.status = ST_CANCELLED;
    q.need_jac = 0;
    q.accepted = 0;
    atomicAdd(&counts[1], 1);
  }
}

}  // namespace

// error reporting for the other translation units of the library
int cs_internal_set_error(int code, const char* msg) { return set_err(code, msg ? msg : ""); }

// ============================================================== module ===
struct cs_module {
  int ny, nz, np, npe, nth, m, s, nrhs, cgw;
  size_t rowsz, treesz;
  CUmodule mod = nullptr;
  CUfunction f_form_initial, f_residual, f_decide, f_accept, f_condense, f_segres, f_mesh_decide,
      f_remesh_count, f_remesh_write, f_repack, f_znodes, f_lists, f_tree_level, f_top, f_backsub_level, f_recover,
      f_babd_cta, f_upper;
  // FP64 refinement of the direction when the tree merges run on the tensor
  // cores (prec_tree != 0)
  CUfunction f_refine_res = nullptr, f_top_refine = nullptr, f_refine_add = nullptr;
  size_t babd_cta_smem;
  // k_upper (upper tree levels, top and their back substitution, CTA per
  // instance): 0 when the block rows are too large for lane merges
  size_t upper_smem = 0;
  int upper_grid = 0;
  // one wave of resident CTAs: grids of the grid-stride kernels k_residual and
  // k_tree_level (small block rows), so that launches with little work do not
  // dispatch waves of idle CTAs
  int res_grid = 1, tree_small_grid = 1;
  int condense_block, condense_per_cta;
  size_t condense_smem;
  size_t tree_smem;   // per CTA of 4 warps
  int top_wpc;
  size_t top_smem;
  int sms = 1;
  int condense_grid = 1;
  // large stage systems: kernels with a global-memory slab per CTA
  bool big = false, big_cond = false, big_tree = false;
  int prec = 0;       // large-system condensation: 0 FP64, 1 TF32, 2 BF16
  int prec_tree = 0;  // large-system tree merges: 0 FP64, 1 TF32, 2 BF16
  long long slab = 0;  // doubles per CTA
  int big_ctas = 0;    // CTAs with a slab (the largest grid of the slab kernels)
  int tree_grid = 0;   // k_tree_level grid (large systems)
  // condensation shape tuner
  CUfunction f_cond_l[4] = {nullptr, nullptr, nullptr, nullptr};  // 4, 8, 16, 32 lanes per interval
  size_t grp_bytes = 0;  // shared memory of one interval group (shared-memory kernel)
  int smem_optin = 0;
  int tune_ver = 0;      // bumped when the tuner changes the shape (graphs re-captured)
};

static std::string build_source(const cs_module_desc* d, bool big_cond, bool big_tree, int prec, int prec_tree,
                                int smem_max) {
  std::ostringstream o;
  o << "// generated prelude\n";
  o << "#define CS_NY " << d->ny << "\n#define CS_NZ " << d->nz << "\n#define CS_NP " << d->np << "\n";
  o << "#define CS_NPE " << d->np_eff << "\n#define CS_NTH " << d->n_theta << "\n#define CS_M " << d->m << "\n";
  if (big_cond) o << "#define CS_BIG_COND 1\n";
  if (big_tree) o << "#define CS_BIG_TREE 1\n";
  if (big_cond || big_tree) o << "#define CS_SMEM_MAX " << smem_max << "\n";
  if (prec) o << "#define CS_PREC " << prec << "\n";
  if (prec_tree) o << "#define CS_PREC_TREE " << prec_tree << "\n";
  const int m = d->m;
  o << "__constant__ double CS_A[" << m * m << "] = {" << fmt_array(d->lobatto_A, m * m) << "};\n";
  o << "__constant__ double CS_B[" << m << "] = {" << fmt_array(d->lobatto_b, m) << "};\n";
  o << "__constant__ double CS_C[" << m << "] = {" << fmt_array(d->lobatto_c, m) << "};\n";
  o << "__constant__ double CS_GW[" << m + 1 << "] = {" << fmt_array(d->gauss_w, m + 1) << "};\n";
  o << "__constant__ double CS_GL[" << (m + 1) * m << "] = {" << fmt_array(d->gauss_L, (m + 1) * m) << "};\n";
  o << "__constant__ double CS_GI[" << (m + 1) * m << "] = {" << fmt_array(d->gauss_I, (m + 1) * m) << "};\n";
  o << "__constant__ double CS_L0[" << m << "] = {" << fmt_array(d->L0, m) << "};\n";
  o << "__constant__ double CS_L1[" << m << "] = {" << fmt_array(d->L1, m) << "};\n";
  o << "// problem functions\n" << d->problem_src << "\n";
  o << cs_kernels_source;
  return o.str();
}

static int compile_cubin(const std::string& src, const std::string& cache_dir, std::vector<char>& cubin) {
  const char* opts[] = {"--gpu-architecture=sm_103a", "-std=c++17", "-lineinfo"};
  const int nopt = 3;
  int major = 0, minor = 0;
  nvrtcVersion(&major, &minor);
  std::string key_src = src;
  for (int i = 0; i < nopt; ++i) key_src += std::string("\n//opt ") + opts[i];
  key_src += "\n//nvrtc " + std::to_string(major) + "." + std::to_string(minor);
  char name[64];
  snprintf(name, sizeof(name), "cs_%016llx.cubin", (unsigned long long)fnv1a(key_src));
  std::string path = cache_dir.empty() ? std::string() : cache_dir + "/" + name;
  if (!path.empty() && read_file(path, cubin)) return CS_OK;
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, src.c_str(), "cs_kernels.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
    return set_err(CS_ERR_NVRTC, "nvrtcCreateProgram failed");
  nvrtcResult rc = nvrtcCompileProgram(prog, nopt, opts);
  if (rc != NVRTC_SUCCESS) {
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    std::string log(n, '\0');
    nvrtcGetProgramLog(prog, &log[0]);
    nvrtcDestroyProgram(&prog);
    return set_err(CS_ERR_NVRTC, std::string("NVRTC compile failed: ") + nvrtcGetErrorString(rc) + "\n" + log);
  }
  size_t n = 0;
  nvrtcGetCUBINSize(prog, &n);
  cubin.resize(n);
  nvrtcGetCUBIN(prog, cubin.data());
  nvrtcDestroyProgram(&prog);
  if (!path.empty()) {
    mkdirs(cache_dir);
    std::string tmp = path + ".tmp" + std::to_string((long long)getpid());
    std::ofstream f(tmp, std::ios::binary);
    if (f) {
      f.write(cubin.data(), (std::streamsize)cubin.size());
      f.close();
      rename(tmp.c_str(), path.c_str());
    }
  }
  return CS_OK;
}

extern "C" int cs_module_load(const cs_module_desc* d, cs_module** out) {
  if (!d || !out || !d->problem_src) return set_err(CS_ERR_INVALID, "cs_module_load: null argument");
  if (d->ny < 1 || d->nz < 0 || d->np < 0 || d->np_eff < 0 || d->np_eff > d->np || d->n_theta < 0 || d->m < 2 ||
      d->m > 10)
    return set_err(CS_ERR_INVALID, "cs_module_load: sizes out of range");
  if (!d->lobatto_A || !d->lobatto_b || !d->lobatto_c || !d->gauss_w || !d->gauss_L || !d->gauss_I || !d->L0 || !d->L1)
    return set_err(CS_ERR_INVALID, "cs_module_load: missing table");
  CS_TRY(ensure_context());
  int dev = 0;
  CS_CUDA(cudaGetDevice(&dev));
  int smem_optin = 0;
  CS_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cs_module* M = new cs_module();
  M->ny = d->ny; M->nz = d->nz; M->np = d->np; M->npe = d->np_eff; M->nth = d->n_theta; M->m = d->m;
  M->s = d->m * (d->ny + d->nz);
  M->nrhs = d->ny + d->np_eff + 1;
  M->rowsz = (size_t)d->ny * (2 * d->ny + d->np_eff + 1);
  M->treesz = (size_t)d->ny * (3 * d->ny + d->np_eff + 1);
  // condensation: shared memory of one group (CS_GRP_DBL in cs_kernels.cuh) and
  // lanes per group (CS_CGL): 8 lanes for small reduced systems (4 intervals
  // per warp), 16 for medium, a CTA of 256 threads for large ones
  const int rb = d->ny + d->nz, jyc = d->ny + d->nz + d->np_eff;
  const int s1 = (d->m - 1) * rb;
  const int ldw1 = (s1 + M->nrhs) | 1;
  const size_t raw = (size_t)s1 * ldw1 + (size_t)d->m * rb * jyc + (size_t)d->m * rb + (size_t)d->m * d->m + d->ny +
                     (size_t)rb * M->nrhs + s1 + 16;
  const size_t grp = (((raw + 7) / 16) * 16 + 8) * sizeof(double);
  const int gl = (s1 > 48) ? 256 : ((s1 > 16) ? 16 : 8);
  // BABD tree: a merge matrix per warp (4 warps per CTA); top: one system per warp
  const int qld = (2 * M->ny) | 1, qc = 3 * M->ny + M->npe + 1;
  const int nt = 2 * M->ny + M->np, tld = nt | 1;
  const size_t tree_small = (size_t)4 * qld * qc * sizeof(double);
  const size_t top_per = (size_t)tld * (nt + 1) * sizeof(double);
  const bool fits_cond = grp <= (size_t)smem_optin;
  const bool fits_tree = tree_small <= (size_t)smem_optin && top_per <= (size_t)smem_optin;
  if (d->layout == 1 && !(fits_cond && fits_tree)) {
    delete M;
    return set_err(CS_ERR_INVALID, "cs_module_load: stage system of size " + std::to_string(M->s) +
                                       " does not fit in shared memory (layout 1)");
  }
  // layout 0: the blocked-LU condensation whenever a whole CTA would serve
  // one interval (measured faster from s1 = 102 on) or the system does not
  // fit; the CTA tree kernels only when the merge or top blocks do not fit
  if (d->precision < 0 || d->precision > 4) {
    delete M;
    return set_err(CS_ERR_INVALID, "cs_module_load: precision must be 0 (FP64), 1 (TF32), 2 (BF16), 3 or 4 (with the tree)");
  }
  if (d->precision != 0 && d->layout == 1) {
    delete M;
    return set_err(CS_ERR_INVALID, "cs_module_load: reduced precision needs the large-system condensation (layout 0 or 2)");
  }
  M->prec = (d->precision == 0) ? 0 : ((d->precision == 1 || d->precision == 3) ? 1 : 2);
  M->prec_tree = (d->precision == 3) ? 1 : ((d->precision == 4) ? 2 : 0);
  M->big_cond = d->layout == 2 || d->precision != 0 || (d->layout == 0 && (!fits_cond || gl > 32));
  M->big_tree = d->layout == 2 || (d->layout == 0 && !fits_tree);
  M->big = M->big_cond || M->big_tree;
  M->cgw = gl;
  M->grp_bytes = grp;
  M->smem_optin = smem_optin;
  int smem_sm = 0;
  CS_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  CS_CUDA(cudaDeviceGetAttribute(&M->sms, cudaDevAttrMultiProcessorCount, dev));
  // sizes of the large-system kernels (CS_NB .. CS_SM_TOP in cs_kernels.cuh;
  // the kernels check what they get and report a mismatch)
  {
    const long long nb = 16, ncol1 = s1 + M->nrhs, ldg = ((ncol1 + 3) / 4) * 4, nfg = d->ny + d->nz + d->np;
    const long long ws_jf = (long long)d->m * rb * nfg + (long long)rb * M->nrhs + d->m * d->m + d->m;
    const long long ws_cond = (long long)s1 * ldg + ws_jf + (d->precision ? (ws_jf + 1) / 2 : 0ll);
    const long long sm_cond = (long long)s1 * (nb + 1) + nb * ldg + (long long)d->m * rb + d->m * d->m + d->ny + s1 + 16 + nb;
    const long long qsz = (long long)qld * qc, tsz = (long long)tld * (nt + 1);
    const long long drsz = (long long)(d->ny + d->np) * (2 * d->ny + d->np);
    const long long hb = 16, sm_hb = hb * qld + 2 * hb * hb + hb + 32;
    const bool q_smem = (qsz + sm_hb) * 8 <= smem_optin, t_smem = (tsz + 32) * 8 <= smem_optin;
    M->slab = 0;
    if (M->big_cond) M->slab = std::max(M->slab, ws_cond);
    if (M->big_tree) M->slab = std::max(M->slab, std::max(q_smem ? 0ll : qsz, (t_smem ? 0ll : tsz) + drsz));
    if (M->big_cond) {
      M->condense_smem = (size_t)sm_cond * 8;
      if (M->prec) {
        // tensor-core condensation (CS_NBT .. CS_TC_SMB in cs_kernels.cuh)
        const long long nbt = 32, eps = (M->prec == 1) ? 4 : 8, kc = nbt / eps, kb = nb / eps, kf = 64 / eps;
        const long long mp = (s1 > nbt) ? ((s1 - nbt + 127) / 128) * 128 : 128, mb = ((s1 + 127) / 128) * 128;
        const long long nr = ((M->nrhs + 15) / 16) * 16;
        auto r128 = [](long long x) { return ((x + 127) / 128) * 128; };
        const long long ops = r128(std::max((mp + 256) * kc * 16, (mb + nr) * kb * 16));
        const long long panel = r128((long long)s1 * (nbt + 1) * 4);
        const long long dbl = 8 * ((long long)d->m * rb + d->m * d->m + d->ny + 16);
        const long long misc = ops + panel + dbl + r128(4 * (long long)s1 + 4 * nbt);
        if ((128 + nr) * kf * 16 > ops + panel) {
          delete M;
          return set_err(CS_ERR_INVALID, "cs_module_load: tensor-core fill operands do not fit");
        }
        // at least 80 KB: at most two CTAs per SM, so that their tensor-memory
        // accumulators (256 columns each) always fit the SM's 512
        M->condense_smem = std::max<size_t>((size_t)(((misc + 16) + 7) / 8) * 8, 80 * 1024);
      }
      if (M->condense_smem > (size_t)smem_optin) {
        delete M;
        return set_err(CS_ERR_INVALID, "cs_module_load: stage system of size " + std::to_string(M->s) + " too large");
      }
      // small stage systems: CTAs of 128 (four per SM overlap the serial
      // panel phases of one another)
      M->condense_block = (s1 <= 128) ? 128 : 256;
      M->condense_per_cta = 1;
    }
    if (M->big_tree && d->precision >= 3) {
      // reduced-precision merges: FP32 merge matrix and shared floats
      // (CS_SHF .. CS_SM_TREE_LP in cs_kernels.cuh)
      const long long shf = hb * qld + 2 * hb * hb + hb + (long long)qc * hb, sm_hb_lp = (shf + 1) / 2 + 32;
      const long long qsz_lp = (qsz + 1) / 2;
      const bool q_smem_lp = (qsz_lp + sm_hb_lp) * 8 <= smem_optin;
      M->slab = std::max(M->slab, std::max(q_smem_lp ? 0ll : qsz_lp, (t_smem ? 0ll : tsz) + drsz));
      M->tree_smem = (size_t)((q_smem_lp ? qsz_lp : 0) + sm_hb_lp) * 8;
      M->top_smem = (size_t)((t_smem ? tsz : 0) + 32) * 8;
      M->top_wpc = 8;
      M->babd_cta_smem = 0;
    } else if (M->big_tree) {
      M->tree_smem = (size_t)((q_smem ? qsz : 0) + sm_hb) * 8;
      M->top_smem = (size_t)((t_smem ? tsz : 0) + 32) * 8;
      M->top_wpc = 8;
      M->babd_cta_smem = 0;
    }
  }
  if (!M->big_cond) {
    if (gl <= 32) {
      // warps per CTA that maximise resident groups per SM (shared memory bound)
      const int gpw = 32 / gl;
      int best_w = 1;
      long long best_groups = 0;
      for (int w = 1; w <= 8; ++w) {
        const size_t cta = grp * gpw * w;
        if (cta > (size_t)smem_optin) break;
        long long ctas = (long long)(smem_sm / (cta + 1024));
        ctas = std::min<long long>(ctas, 64 / w);  // 64 warps per SM
        const long long groups = ctas * w * gpw;
        if (groups > best_groups) { best_groups = groups; best_w = w; }
      }
      M->condense_per_cta = best_w * gpw;
      M->condense_block = 32 * best_w;
      M->condense_smem = grp * gpw * best_w;
    } else {
      M->condense_per_cta = 1;
      M->condense_block = gl;
      M->condense_smem = grp;
    }
  }
  if (!M->big_tree) {
    M->tree_smem = tree_small;
    M->top_wpc = (int)std::max<size_t>(1, std::min<size_t>(4, (size_t)smem_optin / top_per));
    M->babd_cta_smem = top_per + (size_t)8 * qld * qc * sizeof(double);
    M->top_smem = top_per * M->top_wpc;
    // CS_TREE_THREAD && CS_QC <= 32 in cs_kernels.cuh (lane merges)
    if (2 * M->ny * qc <= 128 && qc <= 32 && top_per <= (size_t)smem_optin) M->upper_smem = top_per;
  }

  std::string src = build_source(d, M->big_cond, M->big_tree, M->prec, M->big_tree ? M->prec_tree : 0, smem_optin);
  std::string cache = d->cache_dir ? d->cache_dir : "";
  if (cache.empty()) {
    const char* env = getenv("CS_GB300_CACHE");
    if (env) cache = env;
  }
  std::vector<char> cubin;
  int rc = compile_cubin(src, cache, cubin);
  if (rc != CS_OK) {
    delete M;
    return rc;
  }
  CUresult r = g_drv.moduleLoadData(&M->mod, cubin.data());
  if (r != CUDA_SUCCESS) {
    delete M;
    return set_err(CS_ERR_CUDA, std::string("cuModuleLoadData: ") + drv_err(r));
  }
  struct {
    CUfunction* f;
    const char* name;
  } fns[] = {{&M->f_form_initial, "k_form_initial"}, {&M->f_residual, "k_residual"},   {&M->f_decide, "k_decide"},
             {&M->f_accept, "k_accept"},             {&M->f_condense, "k_condense"},
             {&M->f_segres, "k_segres"},             {&M->f_mesh_decide, "k_mesh_decide"},
             {&M->f_remesh_count, "k_remesh_count"}, {&M->f_remesh_write, "k_remesh_write"},
             {&M->f_repack, "k_repack"},             {&M->f_znodes, "k_znodes"},
             {&M->f_lists, "k_lists"},               {&M->f_tree_level, "k_tree_level"},
             {&M->f_top, "k_top"},                   {&M->f_backsub_level, "k_backsub_level"},
             {&M->f_recover, "k_recover"},           {&M->f_babd_cta, "k_babd_cta"},
             {&M->f_upper, "k_upper"}};
  for (auto& e : fns) {
    CUresult rr = g_drv.moduleGetFunction(e.f, M->mod, e.name);
    if (rr != CUDA_SUCCESS) {
      g_drv.moduleUnload(M->mod);
      delete M;
      return set_err(CS_ERR_CUDA, std::string("missing kernel ") + e.name);
    }
  }
  {
    const char* names[4] = {"k_condense_l4", "k_condense_l8", "k_condense_l16", "k_condense_l32"};
    for (int k = 0; k < 4; ++k)
      if (g_drv.moduleGetFunction(&M->f_cond_l[k], M->mod, names[k]) != CUDA_SUCCESS) M->f_cond_l[k] = nullptr;
  }
  if (M->big_tree && M->prec_tree) {
    struct {
      CUfunction* f;
      const char* name;
    } rf[] = {{&M->f_refine_res, "k_refine_residual"}, {&M->f_top_refine, "k_top_refine"},
              {&M->f_refine_add, "k_refine_add"}};
    for (auto& e : rf) {
      if (g_drv.moduleGetFunction(e.f, M->mod, e.name) != CUDA_SUCCESS) {
        g_drv.moduleUnload(M->mod);
        delete M;
        return set_err(CS_ERR_CUDA, std::string("missing kernel ") + e.name);
      }
    }
  }
  if (M->condense_smem > 48 * 1024)
    CS_CU(g_drv.funcSetAttribute(M->f_condense, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)M->condense_smem));
  if (M->tree_smem > 48 * 1024)
    CS_CU(g_drv.funcSetAttribute(M->f_tree_level, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)M->tree_smem));
  if (M->top_smem > 48 * 1024) {
    CS_CU(g_drv.funcSetAttribute(M->f_top, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)M->top_smem));
    if (M->f_top_refine)
      CS_CU(g_drv.funcSetAttribute(M->f_top_refine, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)M->top_smem));
  }
  if (M->big) {
    // persistent grids from the kernels' occupancy (registers and shared memory)
    M->big_ctas = 0;
    if (M->big_cond) {
      int pc = 0;
      CS_CU(g_drv.occupancy(&pc, M->f_condense, M->condense_block, M->condense_smem));
      if (M->prec) {
        // tensor-core condensation: two CTAs per SM whenever their shared
        // memory fits (registers are bounded for two by the kernel; the
        // occupancy query reports one for this kernel)
        const int by_smem = (int)((size_t)smem_sm / (M->condense_smem + 1024));
        pc = std::max(pc, std::min(2, by_smem));
      }
      M->condense_grid = M->sms * std::max(1, pc);
      M->big_ctas = std::max(M->big_ctas, M->condense_grid);
    }
    if (M->big_tree) {
      int pt = 0;
      CS_CU(g_drv.occupancy(&pt, M->f_tree_level, 256, M->tree_smem));
      M->tree_grid = M->sms * std::max(1, pt);
      M->big_ctas = std::max(M->big_ctas, M->tree_grid);
    }
  }
  {
    int pr = 0;
    CS_CU(g_drv.occupancy(&pr, M->f_residual, 256, 0));
    M->res_grid = M->sms * std::max(1, std::min(pr, 8));
    if (!M->big_tree) {
      int pt = 0;
      CS_CU(g_drv.occupancy(&pt, M->f_tree_level, 128, M->tree_smem));
      M->tree_small_grid = M->sms * std::max(1, std::min(pt, 8));
    }
  }
  if (M->upper_smem) {
    if (M->upper_smem > 48 * 1024)
      CS_CU(g_drv.funcSetAttribute(M->f_upper, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)M->upper_smem));
    int pu = 0;
    CS_CU(g_drv.occupancy(&pu, M->f_upper, 128, M->upper_smem));
    M->upper_grid = M->sms * std::max(1, std::min(pu, 16));
  }
  if (M->babd_cta_smem > (size_t)smem_optin) M->babd_cta_smem = 0;  // per-level kernels only
  else if (M->babd_cta_smem > 48 * 1024)
    CS_CU(g_drv.funcSetAttribute(M->f_babd_cta, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)M->babd_cta_smem));
  if (!M->big_cond) {
    // resident CTAs of the condensation kernel per SM, for its persistent grid
    int smem_sm2 = 0;
    CS_CUDA(cudaDeviceGetAttribute(&smem_sm2, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    int per_sm = std::max<int>(1, (int)((size_t)smem_sm2 / (M->condense_smem + 1024)));
    per_sm = std::min(per_sm, 2048 / M->condense_block);
    M->condense_grid = M->sms * per_sm;
  }
  *out = M;
  return CS_OK;
}

extern "C" void cs_module_free(cs_module* M) {
  if (!M) return;
  if (M->mod && g_drv.moduleUnload) g_drv.moduleUnload(M->mod);
  delete M;
}

extern "C" void cs_opts_default(cs_opts* o) {
  if (!o) return;
  o->tol = 1e-6;
  o->max_iter = 200;
  o->max_mesh = 10;
  o->max_nodes = 2000;
  o->min_nodes = 3;
  o->max_linesearch = 20;
  o->alpha0 = 0.1;
  o->alpha_m = 0.1;
  o->beta = 0.9;
  o->check_every = 4;
  o->babd_path = 0;
  o->residual_type = 1;
  o->scale_by_time = 1;
  o->residual2 = 0;
  o->refine = 2;
  o->ls_grow = 2;
}


// =============================================================== batch ===
struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

struct cs_batch {
  cs_module* M = nullptr;
  int B = 0;
  long long cap = 0;  // node slots allocated
  int T = 0;          // node slots in use
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool have_guess = false;
  // per instance
  DBuf dN, doff, doff2, dp, dth, ddp, dinst, dcounters, dtrials;
  // per slot (set 0 / set 1 for the arrays a remesh rewrites)
  DBuf t[2], y[2], ydot[2], zt[2], znode[2];
  int cur = 0;
  DBuf inst_of, dy, dydot, dzt, X, rows0, rows1, tree, res;
  // refinement (tensor-core tree): the condensed blocks as condensed, the
  // direction a correction is added to
  DBuf rows_keep, dy_keep, dp_keep;
  DBuf wsp;  // large stage systems: slab per CTA
  std::vector<int> hN, hoff;
  cs_opts opts;
  // work lists
  DBuf l_act, l_jac, l_acc, l_actp, l_jacp, l_accp, l_lvlp, l_n;
  int* h_n = nullptr;  // pinned copy of nlist (8 ints: the lists' counts, then k_spares' counts)
  cs_progress_fn progress = nullptr;
  void* progress_user = nullptr;
  // captured super-step, one graph per Newton-direction path (0 per level,
  // 1 one CTA per instance)
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  int graph_nlvl[2] = {-1, -1};
  int graph_tune[2] = {-1, -1};
  int graph_lo[2] = {-1, -1};  // first k_upper level the graph was captured with
  int graph_refine[2] = {-1, -1};  // refinement sweeps captured
  // Grids of the per-super-step launches are capped to the work of the
  // instances still in Newton once few are (the tail of a batch): slots of
  // those instances and their count, 0 = no cap.  Instances only leave the
  // Newton phase until the next mesh phase, so a cap set at a check holds for
  // the rest of the phase.  Every capped kernel is grid-stride: the grid
  // changes the time, not the results.
  long long work_cap = 0;
  int inst_cap = 0;
  long long graph_cap[2] = {-1, -1};
  // spares (cs_batch_set_spares): instance n_primary + k backs up instance k;
  // started once at most spare_trigger instances are in Newton (< 0: never)
  int n_primary = 0;
  int spare_trigger = -1;
  CsBatchDev graph_view[2];
  CsConsts graph_consts[2];
  // device copy of the last initial guess (cs_batch_reset)
  DBuf iN, ioff, it, iy, iz, ip;
  std::vector<int> ihN, ihoff;
  int iT = 0;
  // profiling
  long long launches = 0, super_steps = 0;
  bool timing = false;
  struct EvPair {
    cudaEvent_t a, b;
    int kind;
  };
  std::vector<EvPair> ev_pool;
  size_t ev_used = 0;
  double kind_ms[3] = {0, 0, 0};
  long long kind_launches[3] = {0, 0, 0};
};

static int dalloc(DBuf& b, size_t bytes) {
  if (b.bytes >= bytes && b.p) return CS_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  if (bytes == 0) bytes = 8;
  CS_CUDA(cudaMalloc(&b.p, bytes));
  b.bytes = bytes;
  return CS_OK;
}

static void dfree(DBuf& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
}

static int alloc_slots(cs_batch* bt, long long cap, bool keep_current) {
  cs_module* M = bt->M;
  const size_t c = (size_t)std::max<long long>(cap, 1);
  const size_t d = sizeof(double);
  for (int s = 0; s < 2; ++s) {
    if (keep_current && s == bt->cur) continue;
    CS_TRY(dalloc(bt->t[s], c * d));
    CS_TRY(dalloc(bt->y[s], c * M->ny * d));
    CS_TRY(dalloc(bt->ydot[s], c * M->m * M->ny * d));
    CS_TRY(dalloc(bt->zt[s], c * M->m * std::max(M->nz, 1) * d));
    CS_TRY(dalloc(bt->znode[s], c * std::max(M->nz, 1) * d));
  }
  CS_TRY(dalloc(bt->inst_of, c * sizeof(int)));
  CS_TRY(dalloc(bt->dy, c * M->ny * d));
  CS_TRY(dalloc(bt->dydot, c * M->m * M->ny * d));
  CS_TRY(dalloc(bt->dzt, c * M->m * std::max(M->nz, 1) * d));
  CS_TRY(dalloc(bt->X, c * M->nrhs * M->s * d));
  CS_TRY(dalloc(bt->rows0, c * M->rowsz * d));
  CS_TRY(dalloc(bt->rows1, c * M->rowsz * d));
  CS_TRY(dalloc(bt->tree, c * M->treesz * d));
  CS_TRY(dalloc(bt->res, c * d));
  if (M->prec_tree) {
    CS_TRY(dalloc(bt->rows_keep, c * M->rowsz * d));
    CS_TRY(dalloc(bt->dy_keep, c * M->ny * d));
  }
  bt->cap = (long long)c;
  return CS_OK;
}

// grow the current set too, preserving its contents (used before a remesh)
static int grow_current(cs_batch* bt, long long need) {
  if (need <= bt->cap) return CS_OK;
  long long newcap = std::max<long long>(need, bt->cap + bt->cap / 2);
  cs_module* M = bt->M;
  const size_t d = sizeof(double);
  const int s = bt->cur;
  struct {
    DBuf* b;
    size_t per;
  } keep[] = {{&bt->t[s], d}, {&bt->y[s], M->ny * d}, {&bt->ydot[s], M->m * M->ny * d},
              {&bt->zt[s], M->m * std::max(M->nz, 1) * d}, {&bt->znode[s], std::max(M->nz, 1) * d},
              {&bt->inst_of, sizeof(int)}, {&bt->res, d}};
  for (auto& k : keep) {
    DBuf nb;
    CS_TRY(dalloc(nb, (size_t)newcap * k.per));
    CS_CUDA(cudaMemcpyAsync(nb.p, k.b->p, (size_t)bt->T * k.per, cudaMemcpyDeviceToDevice, bt->stream));
    CS_CUDA(cudaStreamSynchronize(bt->stream));
    dfree(*k.b);
    *k.b = nb;
  }
  return alloc_slots(bt, newcap, true);
}

static CsBatchDev devview(cs_batch* bt) {
  CsBatchDev v;
  memset(&v, 0, sizeof(v));
  const int s = bt->cur;
  v.B = bt->B;
  v.T = bt->T;
  v.N = (const int*)bt->dN.p;
  v.off = (const int*)bt->doff.p;
  v.inst_of = (const int*)bt->inst_of.p;
  v.t = (double*)bt->t[s].p;
  v.y = (double*)bt->y[s].p;
  v.ydot = (double*)bt->ydot[s].p;
  v.zt = (double*)bt->zt[s].p;
  v.p = (double*)bt->dp.p;
  v.th = (const double*)bt->dth.p;
  v.dy = (double*)bt->dy.p;
  v.dydot = (double*)bt->dydot.p;
  v.dzt = (double*)bt->dzt.p;
  v.dp = (double*)bt->ddp.p;
  v.X = (double*)bt->X.p;
  v.rows0 = (double*)bt->rows0.p;
  v.rows1 = (double*)bt->rows1.p;
  v.tree = (double*)bt->tree.p;
  v.res = (double*)bt->res.p;
  v.znode = (double*)bt->znode[s].p;
  v.inst = (CsInst*)bt->dinst.p;
  v.counters = (unsigned long long*)bt->dcounters.p;
  v.act = (int*)bt->l_act.p;
  v.jac = (int*)bt->l_jac.p;
  v.acc = (int*)bt->l_acc.p;
  v.act_pre = (long long*)bt->l_actp.p;
  v.jac_pre = (long long*)bt->l_jacp.p;
  v.acc_pre = (long long*)bt->l_accp.p;
  v.lvl_pre = (long long*)bt->l_lvlp.p;
  v.nlist = (int*)bt->l_n.p;
  v.trials = (unsigned long long*)bt->dtrials.p;
  if (bt->M->big) {
    v.wsp = (double*)bt->wsp.p;
    v.wsp_stride = bt->M->slab;
    v.wsp_ctas = bt->M->big_ctas;
  }
  return v;
}

static int flush_events(cs_batch* bt) {
  if (bt->ev_used == 0) return CS_OK;
  CS_CUDA(cudaStreamSynchronize(bt->stream));
  for (size_t i = 0; i < bt->ev_used; ++i) {
    float ms = 0.f;
    CS_CUDA(cudaEventElapsedTime(&ms, bt->ev_pool[i].a, bt->ev_pool[i].b));
    bt->kind_ms[bt->ev_pool[i].kind] += ms;
  }
  bt->ev_used = 0;
  return CS_OK;
}

// kind: -1 untimed, 0 condense, 1 babd, 2 residual
static int launch_k(cs_batch* bt, CUfunction f, unsigned grid, unsigned block, size_t smem, void** args, int kind) {
  if (grid == 0) return CS_OK;
  cs_batch::EvPair* ev = nullptr;
  if (bt->timing && kind >= 0) {
    if (bt->ev_used == bt->ev_pool.size()) {
      if (bt->ev_pool.size() >= 3072) CS_TRY(flush_events(bt));
      if (bt->ev_used == bt->ev_pool.size()) {
        cs_batch::EvPair e;
        CS_CUDA(cudaEventCreate(&e.a));
        CS_CUDA(cudaEventCreate(&e.b));
        bt->ev_pool.push_back(e);
      }
    }
    ev = &bt->ev_pool[bt->ev_used++];
    ev->kind = kind;
    CS_CUDA(cudaEventRecord(ev->a, bt->stream));
  }
  CS_CU(g_drv.launchKernel(f, grid, 1, 1, block, 1, 1, (unsigned)smem, (CUstream)bt->stream, args, nullptr));
  bt->launches += 1;
  if (kind >= 0) bt->kind_launches[kind] += 1;
  if (ev) CS_CUDA(cudaEventRecord(ev->b, bt->stream));
  return CS_OK;
}

static int launch(cs_batch* bt, CUfunction f, unsigned grid, unsigned block, size_t smem, void** args) {
  return launch_k(bt, f, grid, block, smem, args, -1);
}

static unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// grid g of a grid-stride launch that does `per_cta` items of `items` per CTA
// at most, where items scale with the capped work (bt->work_cap slots)
static unsigned capped(const cs_batch* bt, unsigned g, long long items_per_slot, long long per_cta) {
  if (bt->work_cap <= 0) return g;
  const long long need = (bt->work_cap * items_per_slot + per_cta - 1) / per_cta;
  return (unsigned)std::max<long long>(1, std::min<long long>((long long)g, need));
}
// grid of a launch with one CTA per instance in Newton
static unsigned capped_inst(const cs_batch* bt, unsigned g) {
  if (bt->work_cap <= 0) return g;
  return (unsigned)std::max(1, std::min((int)g, bt->inst_cap));
}

static int run_slots(cs_batch* bt, CUfunction f, CsBatchDev& v) {
  void* args[] = {&v};
  return launch(bt, f, cdiv(bt->T, 256), 256, 0, args);
}

static int run_insts(cs_batch* bt, CUfunction f, void** args) { return launch(bt, f, cdiv(bt->B, 128), 128, 0, args); }

static int run_condense(cs_batch* bt, CsBatchDev& v) {
  cs_module* M = bt->M;
  void* args[] = {&v};
  // intervals per CTA: groups of cgw lanes (shared-memory kernel), one (large systems)
  const long long per_cta = M->big_cond ? 1 : std::max(1, M->condense_block / std::max(1, M->cgw));
  return launch_k(bt, M->f_condense, capped(bt, (unsigned)M->condense_grid, 1, per_cta), M->condense_block,
                  M->condense_smem, args, 0);
}

// large-system kernels count a launch that gave them too little shared
// memory or slab in counters[7] and skip their work
static int check_config(cs_batch* bt) {
  if (!bt->M->big) return CS_OK;
  unsigned long long c7 = 0;
  CS_CUDA(cudaMemcpyAsync(&c7, (unsigned long long*)bt->dcounters.p + 7, sizeof(c7), cudaMemcpyDeviceToHost, bt->stream));
  CS_CUDA(cudaStreamSynchronize(bt->stream));
  if (c7 != 0)
    return set_err(CS_ERR_STATE,
                   "large-system kernel launched without its shared memory or slab, or a tensor-core MMA timed out");
  return CS_OK;
}

static int tree_levels(const cs_batch* bt) {
  int mx = 1;
  for (int n : bt->hN) mx = std::max(mx, n - 1);
  int L = 0, n = mx;
  while (n > 1) {
    n = (n + 1) >> 1;
    ++L;
  }
  return L;
}

// Newton direction: one launch per tree level across the instances (spreads
// every level over all SMs), or, on request (opts.babd_path = 1), one CTA per
// instance for tree, top and back substitution in one launch.  Measured on
// the warm-started Van der Pol batch, the per-instance CTA is the slower one
// even when few instances are left (611 us per launch in the tail against
// ~100-350 us for the per-level launches it replaces: one SM walks every
// level of an instance's tree), so the automatic choice is per level.
static bool use_cta_path(const cs_batch* bt) {
  if (bt->M->babd_cta_smem == 0) return false;
  return bt->opts.babd_path == 1;
}

// First tree level handled by k_upper: the top 4 levels (at most 8 merges per
// instance at the first of them), or nlvl (k_upper not used: large block rows,
// or babd_path 2 asks for one launch per level).
static const int kUpperLevels = 4;
static int upper_levels(const cs_batch* bt, int nlvl) {
  if (!bt->M->upper_smem || bt->opts.babd_path == 2) return nlvl;
  return std::max(0, nlvl - kUpperLevels);
}

static int run_lists(cs_batch* bt, CsBatchDev& v, int mode, int nlvl) {
  void* args[] = {&v, &mode, &nlvl};
  return launch(bt, bt->M->f_lists, 1, 1024, 0, args);
}

// Newton direction for the instances on the jac list: tree levels up, top
// system, back substitution down, stage recovery.
static int run_direction(cs_batch* bt, CsBatchDev& v, int nlvl) {
  cs_module* M = bt->M;
  if (use_cta_path(bt)) {
    int recover = 0;
    void* a[] = {&v, &recover};
    CS_TRY(launch_k(bt, M->f_babd_cta, (unsigned)(M->sms * 2), 256, M->babd_cta_smem, a, 1));
    void* ar[] = {&v};
    return launch_k(bt, M->f_recover, (unsigned)(M->sms * 8), 128, 0, ar, 1);
  }
  const unsigned g = (unsigned)(M->sms * 8);
  const bool refine = M->prec_tree && bt->opts.refine > 0 && M->f_refine_res;
  if (refine)  // the condensed blocks, for the residuals of the refinement
    CS_CUDA(cudaMemcpyAsync(bt->rows_keep.p, bt->rows0.p, (size_t)bt->T * M->rowsz * sizeof(double),
                            cudaMemcpyDeviceToDevice, bt->stream));
  // levels from l_lo up (at most 8 merges per instance there) and the top
  // system in one launch, CTA per instance
  const int l_lo = upper_levels(bt, nlvl);
  // merges of a level <= slots; per CTA: one (large), at least 4 (warps / lanes)
  const unsigned gtree = M->big_tree ? capped(bt, (unsigned)M->tree_grid, 1, 1)
                                     : capped(bt, (unsigned)M->tree_small_grid, 1, 4);
  const unsigned gback = capped(bt, g, 1, 4);
  for (int l = 0; l < l_lo; ++l) {
    void* a[] = {&v, &l};
    if (M->big_tree) CS_TRY(launch_k(bt, M->f_tree_level, gtree, 256, M->tree_smem, a, 1));
    else CS_TRY(launch_k(bt, M->f_tree_level, gtree, 128, M->tree_smem, a, 1));
  }
  if (M->upper_smem && bt->opts.babd_path != 2) {
    int lo = l_lo;
    void* a[] = {&v, &lo};
    CS_TRY(launch_k(bt, M->f_upper, capped_inst(bt, (unsigned)std::min(M->upper_grid, bt->B)), 128, M->upper_smem, a, 1));
  } else {
    void* a[] = {&v};
    if (M->big_tree)
      CS_TRY(launch_k(bt, M->f_top, capped_inst(bt, (unsigned)std::min(M->big_ctas, bt->B)), 256, M->top_smem, a, 1));
    else CS_TRY(launch_k(bt, M->f_top, capped_inst(bt, (unsigned)(M->sms * 4)), 32 * M->top_wpc, M->top_smem, a, 1));
  }
  for (int l = l_lo - 1; l >= 0; --l) {
    void* a[] = {&v, &l};
    CS_TRY(launch_k(bt, M->f_backsub_level, gback, 128, 0, a, 1));
  }
  if (refine) {
    // FP64 iterative refinement: residual of the condensed system at the
    // direction, the correction from the same (low-precision) tree, added
    double* keep = (double*)bt->rows_keep.p;
    double* dyk = (double*)bt->dy_keep.p;
    double* dpk = (double*)bt->dp_keep.p;
    for (int sw = 0; sw < bt->opts.refine; ++sw) {
      void* ar[] = {&v, &keep, &dyk, &dpk};
      CS_TRY(launch_k(bt, M->f_refine_res, capped(bt, g, 1, 4), 128, 0, ar, 1));
      for (int l = 0; l < l_lo; ++l) {
        void* a[] = {&v, &l};
        CS_TRY(launch_k(bt, M->f_tree_level, gtree, 256, M->tree_smem, a, 1));
      }
      void* at[] = {&v, &dyk, &dpk};
      CS_TRY(launch_k(bt, M->f_top_refine, capped_inst(bt, (unsigned)std::min(M->big_ctas, bt->B)), 256,
                      M->top_smem, at, 1));
      for (int l = l_lo - 1; l >= 0; --l) {
        void* a[] = {&v, &l};
        CS_TRY(launch_k(bt, M->f_backsub_level, gback, 128, 0, a, 1));
      }
      CS_TRY(launch_k(bt, M->f_refine_add, capped(bt, g, 1, 4), 128, 0, at, 1));
    }
  }
  void* a[] = {&v};
  return launch_k(bt, M->f_recover, capped(bt, g, 1, 4), 128, 0, a, 1);
}

static int fill_inst_of(cs_batch* bt) {
  k_fill_inst_of<<<bt->B, 256, 0, bt->stream>>>(bt->B, (const int*)bt->doff.p, (const int*)bt->dN.p,
                                                  (int*)bt->inst_of.p);
  CS_CUDA(cudaGetLastError());
  bt->launches += 1;
  return CS_OK;
}

static CsConsts consts_of(const cs_opts& o) {
  CsConsts c;
  memset(&c, 0, sizeof(c));
  c.tol = o.tol;
  c.alpha_m = o.alpha_m;
  c.beta = o.beta;
  c.max_iter = o.max_iter;
  c.max_mesh = o.max_mesh;
  c.max_nodes = o.max_nodes;
  c.min_nodes = o.min_nodes;
  c.max_ls = o.max_linesearch;
  c.ls_grow = o.ls_grow;
  return c;
}

extern "C" int cs_batch_set_opts(cs_batch* bt, const cs_opts* opts) {
  if (!bt || !opts) return set_err(CS_ERR_INVALID, "cs_batch_set_opts: null argument");
  if (opts->residual_type < 0 || opts->residual_type > 2)
    return set_err(CS_ERR_INVALID, "cs_batch_set_opts: residual_type must be 0, 1 or 2");
  bt->opts = *opts;
  return CS_OK;
}

extern "C" int cs_batch_create(cs_module* M, int batch, long long node_capacity, void* stream, cs_batch** out) {
  if (!M || !out || batch < 1) return set_err(CS_ERR_INVALID, "cs_batch_create: bad argument");
  CS_TRY(ensure_context());
  cs_batch* bt = new cs_batch();
  bt->M = M;
  bt->B = batch;
  cs_opts_default(&bt->opts);
  if (stream) {
    bt->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&bt->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete bt;
      return set_err(CS_ERR_CUDA, "cudaStreamCreate failed");
    }
    bt->own_stream = true;
  }
  int rc = CS_OK;
  const size_t d = sizeof(double);
  if ((rc = dalloc(bt->dN, batch * sizeof(int))) || (rc = dalloc(bt->doff, batch * sizeof(int))) ||
      (rc = dalloc(bt->doff2, batch * sizeof(int))) || (rc = dalloc(bt->dp, batch * std::max(M->np, 1) * d)) ||
      (rc = dalloc(bt->ddp, batch * std::max(M->np, 1) * d)) ||
      (M->prec_tree && (rc = dalloc(bt->dp_keep, batch * std::max(M->np, 1) * d))) ||
      (rc = dalloc(bt->dth, batch * std::max(M->nth, 1) * d)) || (rc = dalloc(bt->dinst, batch * sizeof(CsInst))) ||
      (rc = dalloc(bt->dcounters, 64)) || (rc = dalloc(bt->l_act, batch * sizeof(int))) ||
      (rc = dalloc(bt->dtrials, (size_t)batch * CS_LSW * sizeof(unsigned long long))) ||
      (rc = dalloc(bt->l_jac, batch * sizeof(int))) || (rc = dalloc(bt->l_acc, batch * sizeof(int))) ||
      (rc = dalloc(bt->l_actp, (batch + 1) * sizeof(long long))) ||
      (rc = dalloc(bt->l_jacp, (batch + 1) * sizeof(long long))) ||
      (rc = dalloc(bt->l_accp, (batch + 1) * sizeof(long long))) ||
      (rc = dalloc(bt->l_lvlp, (size_t)CS_MAXLVL * (batch + 1) * sizeof(long long))) ||
      (rc = dalloc(bt->l_n, 8 * sizeof(int))) ||
      (rc = alloc_slots(bt, std::max<long long>(node_capacity, 2 * batch), false)) ||
      (M->big && (rc = dalloc(bt->wsp, (size_t)M->big_ctas * M->slab * d)))) {
    cs_batch_free(bt);
    return rc;
  }
  if (cudaMemsetAsync(bt->dcounters.p, 0, 64, bt->stream) != cudaSuccess ||
      cudaMemsetAsync(bt->dtrials.p, 0, (size_t)batch * CS_LSW * sizeof(unsigned long long), bt->stream) != cudaSuccess ||
      cudaStreamSynchronize(bt->stream) != cudaSuccess) {
    cs_batch_free(bt);
    return set_err(CS_ERR_CUDA, "cs_batch_create: counter reset failed");
  }
  *out = bt;
  return CS_OK;
}

extern "C" void cs_batch_free(cs_batch* bt) {
  if (!bt) return;
  if (bt->stream) cudaStreamSynchronize(bt->stream);
  DBuf* all[] = {&bt->dN, &bt->doff, &bt->doff2, &bt->dp, &bt->dth, &bt->ddp, &bt->dinst, &bt->dcounters, &bt->dtrials,
                 &bt->inst_of, &bt->dy, &bt->dydot, &bt->dzt, &bt->X, &bt->rows0, &bt->rows1, &bt->tree, &bt->res,
                 &bt->iN, &bt->ioff, &bt->it, &bt->iy, &bt->iz, &bt->ip, &bt->l_act, &bt->l_jac, &bt->l_acc,
                 &bt->l_actp, &bt->l_jacp, &bt->l_accp, &bt->l_lvlp, &bt->l_n, &bt->wsp,
                 &bt->rows_keep, &bt->dy_keep, &bt->dp_keep};
  for (DBuf* b : all) dfree(*b);
  for (int k = 0; k < 2; ++k)
    if (bt->graph[k]) cudaGraphExecDestroy(bt->graph[k]);
  if (bt->h_n) cudaFreeHost(bt->h_n);
  for (auto& e : bt->ev_pool) {
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  for (int s = 0; s < 2; ++s) {
    dfree(bt->t[s]); dfree(bt->y[s]); dfree(bt->ydot[s]); dfree(bt->zt[s]); dfree(bt->znode[s]);
  }
  if (bt->own_stream && bt->stream) cudaStreamDestroy(bt->stream);
  delete bt;
}


// every instance fresh, the spares parked
static void init_insts(const cs_batch* bt, std::vector<CsInst>& hi) {
  for (auto& s : hi) init_inst(s, bt->opts.alpha0);
  if (bt->n_primary > 0)
    for (int b = bt->n_primary; b < bt->B; ++b) hi[b].status = ST_PARKED;
}

extern "C" int cs_batch_set_guess(cs_batch* bt, const int* N, const double* t, const double* y, const double* z,
                                  const double* p, const double* theta) {
  if (!bt || !N || !t || !y) return set_err(CS_ERR_INVALID, "cs_batch_set_guess: null argument");
  cs_module* M = bt->M;
  if (M->nz > 0 && !z) return set_err(CS_ERR_INVALID, "cs_batch_set_guess: z is required (nz > 0)");
  if (M->np > 0 && !p) return set_err(CS_ERR_INVALID, "cs_batch_set_guess: p is required (np > 0)");
  if (M->nth > 0 && !theta) return set_err(CS_ERR_INVALID, "cs_batch_set_guess: theta is required");
  long long T = 0;
  bt->hN.assign(N, N + bt->B);
  bt->hoff.resize(bt->B);
  for (int b = 0; b < bt->B; ++b) {
    if (N[b] < 2) return set_err(CS_ERR_INVALID, "cs_batch_set_guess: every instance needs at least 2 nodes");
    bt->hoff[b] = (int)T;
    T += N[b];
  }
  if (T > 2000000000LL) return set_err(CS_ERR_INVALID, "cs_batch_set_guess: too many nodes");
  if (T > bt->cap) CS_TRY(alloc_slots(bt, T, false));
  bt->T = (int)T;
  bt->cur = 0;
  const size_t d = sizeof(double);
  cudaStream_t st = bt->stream;
  CS_CUDA(cudaMemcpyAsync(bt->dN.p, N, bt->B * sizeof(int), cudaMemcpyHostToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->doff.p, bt->hoff.data(), bt->B * sizeof(int), cudaMemcpyHostToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->t[0].p, t, T * d, cudaMemcpyHostToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->y[0].p, y, T * M->ny * d, cudaMemcpyHostToDevice, st));
  if (M->nz > 0) CS_CUDA(cudaMemcpyAsync(bt->znode[0].p, z, T * M->nz * d, cudaMemcpyHostToDevice, st));
  if (M->np > 0) CS_CUDA(cudaMemcpyAsync(bt->dp.p, p, (size_t)bt->B * M->np * d, cudaMemcpyHostToDevice, st));
  if (M->nth > 0) CS_CUDA(cudaMemcpyAsync(bt->dth.p, theta, (size_t)bt->B * M->nth * d, cudaMemcpyHostToDevice, st));
  // device copy of the guess for cs_batch_reset
  CS_TRY(dalloc(bt->iN, bt->B * sizeof(int)));
  CS_TRY(dalloc(bt->ioff, bt->B * sizeof(int)));
  CS_TRY(dalloc(bt->it, T * d));
  CS_TRY(dalloc(bt->iy, T * M->ny * d));
  CS_TRY(dalloc(bt->iz, T * std::max(M->nz, 1) * d));
  CS_TRY(dalloc(bt->ip, (size_t)bt->B * std::max(M->np, 1) * d));
  CS_CUDA(cudaMemcpyAsync(bt->iN.p, bt->dN.p, bt->B * sizeof(int), cudaMemcpyDeviceToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->ioff.p, bt->doff.p, bt->B * sizeof(int), cudaMemcpyDeviceToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->it.p, bt->t[0].p, T * d, cudaMemcpyDeviceToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->iy.p, bt->y[0].p, T * M->ny * d, cudaMemcpyDeviceToDevice, st));
  if (M->nz > 0) CS_CUDA(cudaMemcpyAsync(bt->iz.p, bt->znode[0].p, T * M->nz * d, cudaMemcpyDeviceToDevice, st));
  if (M->np > 0) CS_CUDA(cudaMemcpyAsync(bt->ip.p, bt->dp.p, (size_t)bt->B * M->np * d, cudaMemcpyDeviceToDevice, st));
  bt->ihN = bt->hN;
  bt->ihoff = bt->hoff;
  bt->iT = (int)T;
  std::vector<CsInst> hi(bt->B);
  init_insts(bt, hi);
  CS_CUDA(cudaMemcpyAsync(bt->dinst.p, hi.data(), hi.size() * sizeof(CsInst), cudaMemcpyHostToDevice, st));
  CS_TRY(fill_inst_of(bt));
  CsBatchDev v = devview(bt);
  int only = -1;
  void* args[] = {&v, &only};
  CS_TRY(launch(bt, M->f_form_initial, cdiv(bt->T, 256), 256, 0, args));
  CS_CUDA(cudaStreamSynchronize(st));
  bt->have_guess = true;
  return CS_OK;
}

extern "C" int cs_batch_set_state(cs_batch* bt, const int* N, const double* t, const double* y, const double* ydot,
                                  const double* zt, const double* p, const double* theta) {
  if (!bt || !N || !t || !y || !ydot) return set_err(CS_ERR_INVALID, "cs_batch_set_state: null argument");
  cs_module* M = bt->M;
  if (M->nz > 0 && !zt) return set_err(CS_ERR_INVALID, "cs_batch_set_state: zt is required (nz > 0)");
  if (M->np > 0 && !p) return set_err(CS_ERR_INVALID, "cs_batch_set_state: p is required (np > 0)");
  if (M->nth > 0 && !theta) return set_err(CS_ERR_INVALID, "cs_batch_set_state: theta is required");
  long long T = 0;
  for (int b = 0; b < bt->B; ++b) {
    if (N[b] < 2) return set_err(CS_ERR_INVALID, "cs_batch_set_state: every instance needs at least 2 nodes");
    T += N[b];
  }
  if (T > 2000000000LL) return set_err(CS_ERR_INVALID, "cs_batch_set_state: too many nodes");
  if (T > bt->cap) CS_TRY(alloc_slots(bt, T, false));
  bt->hN.assign(N, N + bt->B);
  bt->hoff.resize(bt->B);
  // stage values: (N-1) rows per instance on the host, N slots on the device
  const size_t ry = (size_t)M->m * M->ny, rz = (size_t)M->m * M->nz;
  std::vector<double> yd((size_t)T * ry, 0.0), zz((size_t)T * std::max<size_t>(rz, 1), 0.0);
  long long o = 0, hrow = 0;
  for (int b = 0; b < bt->B; ++b) {
    bt->hoff[b] = (int)o;
    for (int i = 0; i < N[b] - 1; ++i, ++hrow) {
      memcpy(&yd[(size_t)(o + i) * ry], ydot + (size_t)hrow * ry, ry * sizeof(double));
      if (rz) memcpy(&zz[(size_t)(o + i) * rz], zt + (size_t)hrow * rz, rz * sizeof(double));
    }
    o += N[b];
  }
  bt->T = (int)T;
  bt->cur = 0;
  const size_t d = sizeof(double);
  cudaStream_t st = bt->stream;
  CS_CUDA(cudaMemcpyAsync(bt->dN.p, N, bt->B * sizeof(int), cudaMemcpyHostToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->doff.p, bt->hoff.data(), bt->B * sizeof(int), cudaMemcpyHostToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->t[0].p, t, T * d, cudaMemcpyHostToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->y[0].p, y, T * M->ny * d, cudaMemcpyHostToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->ydot[0].p, yd.data(), yd.size() * d, cudaMemcpyHostToDevice, st));
  if (rz) CS_CUDA(cudaMemcpyAsync(bt->zt[0].p, zz.data(), (size_t)T * rz * d, cudaMemcpyHostToDevice, st));
  if (M->np > 0) CS_CUDA(cudaMemcpyAsync(bt->dp.p, p, (size_t)bt->B * M->np * d, cudaMemcpyHostToDevice, st));
  if (M->nth > 0) CS_CUDA(cudaMemcpyAsync(bt->dth.p, theta, (size_t)bt->B * M->nth * d, cudaMemcpyHostToDevice, st));
  std::vector<CsInst> hi(bt->B);
  init_insts(bt, hi);
  CS_CUDA(cudaMemcpyAsync(bt->dinst.p, hi.data(), hi.size() * sizeof(CsInst), cudaMemcpyHostToDevice, st));
  CS_TRY(fill_inst_of(bt));
  CS_CUDA(cudaStreamSynchronize(st));
  bt->have_guess = true;
  return CS_OK;
}

static int read_inst(cs_batch* bt, std::vector<CsInst>& hi) {
  hi.resize(bt->B);
  CS_CUDA(cudaMemcpyAsync(hi.data(), bt->dinst.p, hi.size() * sizeof(CsInst), cudaMemcpyDeviceToHost, bt->stream));
  CS_CUDA(cudaStreamSynchronize(bt->stream));
  return CS_OK;
}

static int write_inst(cs_batch* bt, const std::vector<CsInst>& hi) {
  CS_CUDA(cudaMemcpyAsync(bt->dinst.p, hi.data(), hi.size() * sizeof(CsInst), cudaMemcpyHostToDevice, bt->stream));
  return CS_OK;
}

static int super_step(cs_batch* bt, const CsConsts& c, int nlvl) {
  CsBatchDev v = devview(bt);
  cs_module* M = bt->M;
  const unsigned g = (unsigned)(M->sms * 8);
  {
    void* args[] = {&v};
    // (interval, trial) items: up to CS_LSW trials per interval
    CS_TRY(launch_k(bt, M->f_residual, capped(bt, (unsigned)M->res_grid, CS_LSW, 256), 256, 0, args, 2));
  }
  bt->super_steps += 1;
  CsConsts cc = c;
  void* dargs[] = {&v, &cc};
  CS_TRY(run_insts(bt, M->f_decide, dargs));
  CS_TRY(run_lists(bt, v, 1, use_cta_path(bt) ? 0 : nlvl));
  {
    void* args[] = {&v};
    CS_TRY(launch(bt, M->f_accept, capped(bt, g, 1, 256), 256, 0, args));
  }
  CS_TRY(run_condense(bt, v));
  return run_direction(bt, v, nlvl);
}

// A CUDA graph of `reps` super-steps for the current layout (re-captured when
// a remesh changes the buffers).
static int get_graph(cs_batch* bt, const CsConsts& c, int nlvl, int reps) {
  const CsBatchDev v = devview(bt);
  const int k = use_cta_path(bt) ? 1 : 0;
  const int lo = upper_levels(bt, nlvl);
  if (bt->graph[k] && bt->graph_nlvl[k] == nlvl && bt->graph_tune[k] == bt->M->tune_ver && bt->graph_lo[k] == lo &&
      bt->graph_refine[k] == bt->opts.refine && bt->graph_cap[k] == bt->work_cap &&
      memcmp(&bt->graph_view[k], &v, sizeof(v)) == 0 && memcmp(&bt->graph_consts[k], &c, sizeof(c)) == 0)
    return CS_OK;
  if (bt->graph[k]) {
    cudaGraphExecDestroy(bt->graph[k]);
    bt->graph[k] = nullptr;
  }
  cudaGraph_t g = nullptr;
  CS_CUDA(cudaStreamBeginCapture(bt->stream, cudaStreamCaptureModeThreadLocal));
  int rc = CS_OK;
  const long long l0 = bt->launches, s0 = bt->super_steps;
  for (int r = 0; r < reps && rc == CS_OK; ++r) rc = super_step(bt, c, nlvl);
  cudaError_t e = cudaStreamEndCapture(bt->stream, &g);
  bt->launches = l0;  // captured launches are counted when the graph runs
  bt->super_steps = s0;
  if (rc != CS_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return set_err(CS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&bt->graph[k], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_err(CS_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  bt->graph_view[k] = v;
  bt->graph_consts[k] = c;
  bt->graph_nlvl[k] = nlvl;
  bt->graph_tune[k] = bt->M->tune_ver;
  bt->graph_lo[k] = lo;
  bt->graph_refine[k] = bt->opts.refine;
  bt->graph_cap[k] = bt->work_cap;
  return CS_OK;
}

// Remesh every instance whose status is ST_REMESH; node counts N_new are in
// the device inst records after k_remesh_count.
static int do_remesh(cs_batch* bt, std::vector<CsInst>& hi) {
  cs_module* M = bt->M;
  CsBatchDev v = devview(bt);
  void* a1[] = {&v};
  CS_TRY(run_insts(bt, M->f_remesh_count, a1));
  CS_TRY(read_inst(bt, hi));
  std::vector<int> off2(bt->B), N2(bt->B);
  long long T2 = 0;
  for (int b = 0; b < bt->B; ++b) {
    off2[b] = (int)T2;
    N2[b] = hi[b].N_new;
    T2 += N2[b];
  }
  if (T2 > 2000000000LL) return set_err(CS_ERR_INVALID, "remesh: too many nodes");
  CS_TRY(grow_current(bt, std::max<long long>(T2, bt->T)));
  v = devview(bt);
  const int o = 1 - bt->cur;
  CS_CUDA(cudaMemcpyAsync(bt->doff2.p, off2.data(), bt->B * sizeof(int), cudaMemcpyHostToDevice, bt->stream));
  double* t2 = (double*)bt->t[o].p;
  double* y2 = (double*)bt->y[o].p;
  double* yd2 = (double*)bt->ydot[o].p;
  double* zt2 = (double*)bt->zt[o].p;
  double* zn2 = (double*)bt->znode[o].p;
  const int* doff2 = (const int*)bt->doff2.p;
  void* aw[] = {&v, &doff2, &t2, &y2, &zn2};
  CS_TRY(run_insts(bt, M->f_remesh_write, aw));
  void* ar[] = {&v, &doff2, &t2, &y2, &yd2, &zt2};
  CS_TRY(launch(bt, M->f_repack, cdiv(bt->T, 256), 256, 0, ar));
  // switch to the new layout
  bt->cur = o;
  bt->T = (int)T2;
  bt->hN = N2;
  bt->hoff = off2;
  CS_CUDA(cudaMemcpyAsync(bt->dN.p, N2.data(), bt->B * sizeof(int), cudaMemcpyHostToDevice, bt->stream));
  CS_CUDA(cudaMemcpyAsync(bt->doff.p, off2.data(), bt->B * sizeof(int), cudaMemcpyHostToDevice, bt->stream));
  CS_TRY(fill_inst_of(bt));
  v = devview(bt);
  int only = ST_REMESH;
  void* af[] = {&v, &only};
  CS_TRY(launch(bt, M->f_form_initial, cdiv(bt->T, 256), 256, 0, af));
  CS_CUDA(cudaStreamSynchronize(bt->stream));
  return CS_OK;
}

extern "C" int cs_solve(cs_batch* bt, const cs_opts* opts) {
  if (!bt) return set_err(CS_ERR_INVALID, "cs_solve: null batch");
  if (!bt->have_guess) return set_err(CS_ERR_STATE, "cs_solve: no initial guess");
  cs_opts o;
  if (opts) o = *opts; else cs_opts_default(&o);
  if (o.check_every < 1) o.check_every = 1;
  if (o.residual_type < 0 || o.residual_type > 2)
    return set_err(CS_ERR_INVALID, "cs_solve: residual_type must be 0, 1 or 2");
  bt->opts = o;
  const CsConsts c = consts_of(o);
  std::vector<CsInst> hi;
  CS_TRY(read_inst(bt, hi));
  for (auto& s : hi) {
    if (s.status != ST_FRESH) continue;
    s.alpha = o.alpha0;
  }
  CS_TRY(write_inst(bt, hi));
  if (!bt->h_n) CS_CUDA(cudaMallocHost(&bt->h_n, 8 * sizeof(int)));
  int rc = CS_OK;
  const long long max_super = 10000000;
  long long steps = 0;
  const int per_launch_steps = 1;
  // grid caps for the tail (see cs_batch::work_cap): set when at most this
  // many instances are in Newton, tightened each time their number halves
  const int cap_at = std::max(64, bt->B / 32);
  auto set_cap = [&](const std::vector<CsInst>& st) {
    long long slots = 0;
    int n = 0;
    for (int b = 0; b < bt->B; ++b)
      if (st[b].status == ST_FRESH || st[b].status == ST_LS) {
        slots += bt->hN[b];
        ++n;
      }
    if (n > 0 && n <= cap_at) {
      bt->work_cap = slots;
      bt->inst_cap = n;
    } else {
      bt->work_cap = 0;
      bt->inst_cap = 0;
    }
  };
  set_cap(hi);
  // spares (cs_batch_set_spares): from the check at which at most
  // spare_trigger instances are in Newton on, every check starts and stops
  // spares (k_spares).  Started spares need the residual list rebuilt and,
  // if they outgrow the grid caps, larger caps.  A stopped spare needs
  // nothing: every kernel skips it, and the next super-step's lists drop it.
  // A spare starts at most once, so the solve still ends.
  const bool spares = bt->n_primary > 0 && bt->spare_trigger >= 0;
  bool spares_on = false;
  auto spare_pass = [&](bool reread) -> int {
    int* dcount = (int*)bt->l_n.p + 4;
    CS_CUDA(cudaMemsetAsync(dcount, 0, 2 * sizeof(int), bt->stream));
    k_spares<<<cdiv(bt->n_primary, 128), 128, 0, bt->stream>>>(bt->n_primary, (CsInst*)bt->dinst.p, o.alpha0,
                                                               dcount);
    CS_CUDA(cudaGetLastError());
    bt->launches += 1;
    CS_CUDA(cudaMemcpyAsync(bt->h_n + 4, dcount, 2 * sizeof(int), cudaMemcpyDeviceToHost, bt->stream));
    CS_CUDA(cudaStreamSynchronize(bt->stream));
    if (bt->h_n[4] > 0) {
      CsBatchDev vl = devview(bt);
      CS_TRY(run_lists(bt, vl, 0, 0));
      CS_CUDA(cudaMemcpyAsync(bt->h_n, bt->l_n.p, sizeof(int), cudaMemcpyDeviceToHost, bt->stream));
      CS_TRY(read_inst(bt, hi));
      long long slots = 0;
      int n = 0;
      for (int b = 0; b < bt->B; ++b)
        if (hi[b].status == ST_FRESH || hi[b].status == ST_LS) {
          slots += bt->hN[b];
          ++n;
        }
      if (bt->work_cap > 0 && (slots > bt->work_cap || n > bt->inst_cap)) set_cap(hi);
    } else if (bt->h_n[5] > 0 && reread) {
      CS_TRY(read_inst(bt, hi));
    }
    return CS_OK;
  };
  for (int outer = 0; outer < 1000000 && rc == CS_OK; ++outer) {
    // ---- Newton phase: device state machine, work lists, graph replays
    const int nlvl = tree_levels(bt);
    CsBatchDev v0 = devview(bt);
    if ((rc = run_lists(bt, v0, 0, nlvl)) != CS_OK) break;
    const bool use_graph = !bt->timing;
    for (;;) {
      if (use_graph && (rc = get_graph(bt, c, nlvl, per_launch_steps)) != CS_OK) break;
      const bool cta = use_cta_path(bt);
      for (int k = 0; k < o.check_every && rc == CS_OK; ++k) {
        if (use_graph) {
          cudaError_t e = cudaGraphLaunch(bt->graph[cta ? 1 : 0], bt->stream);
          if (e != cudaSuccess) rc = set_err(CS_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
          bt->launches += cta ? 7 : 9 + 2 * upper_levels(bt, nlvl);
          bt->super_steps += 1;
        } else {
          rc = super_step(bt, c, nlvl);
        }
        ++steps;
      }
      if (rc != CS_OK) break;
      if (cudaMemcpyAsync(bt->h_n, bt->l_n.p, sizeof(int), cudaMemcpyDeviceToHost, bt->stream) != cudaSuccess ||
          cudaStreamSynchronize(bt->stream) != cudaSuccess) {
        rc = set_err(CS_ERR_CUDA, std::string("Newton phase: ") + cudaGetErrorString(cudaGetLastError()));
        break;
      }
      if (bt->progress) bt->progress(bt->progress_user, bt->h_n[0], steps);
      if (spares && (spares_on || bt->h_n[0] <= bt->spare_trigger)) {
        spares_on = true;
        if ((rc = spare_pass(false)) != CS_OK) break;
      }
      if (bt->h_n[0] == 0) break;
      if (steps > max_super) {
        rc = set_err(CS_ERR_STATE, "Newton phase did not terminate");
        break;
      }
      if (use_graph && bt->h_n[0] <= cap_at && (bt->inst_cap == 0 || 2 * bt->h_n[0] <= bt->inst_cap)) {
        if ((rc = read_inst(bt, hi)) != CS_OK) break;
        set_cap(hi);
      }
    }
    if (rc != CS_OK) break;
    // ---- mesh phase
    CsBatchDev v = devview(bt);
    double tol = o.tol;
    int rtype = o.residual_type, scale = o.scale_by_time, res2 = o.residual2;
    void* as[] = {&v, &tol, &rtype, &scale, &res2};
    if ((rc = launch(bt, bt->M->f_segres, cdiv(bt->T, 256), 256, 0, as)) != CS_OK) break;
    CsConsts cc = c;
    void* am[] = {&v, &cc};
    if ((rc = run_insts(bt, bt->M->f_mesh_decide, am)) != CS_OK) break;
    if ((rc = read_inst(bt, hi)) != CS_OK) break;
    bool any_remesh = false, any_newton = false;
    for (auto& s : hi) {
      any_remesh |= (s.status == ST_REMESH);
      any_newton |= (s.status == ST_FRESH || s.status == ST_LS);
    }
    if (any_remesh) {
      if ((rc = do_remesh(bt, hi)) != CS_OK) break;
      if ((rc = read_inst(bt, hi)) != CS_OK) break;
      for (int b = 0; b < bt->B; ++b) {
        CsInst& s = hi[b];
        if (s.status != ST_REMESH) continue;
        s.remesh_count += 1;
        const int N = bt->hN[b];
        // mesh_sanity_check (CS:2367-2377) with mesh_it = 1 (reset every continuation step, CS:107)
        if (1 > o.max_mesh) { s.status = ST_FAIL; s.fail_reason = FAIL_MESH; continue; }
        if (N > o.max_nodes || N < o.min_nodes) { s.status = ST_FAIL; s.fail_reason = FAIL_NODES; continue; }
        s.status = ST_FRESH;
        s.it = 0;
        s.alphacal += 1;
        s.norm_bits = 0;
      }
      if ((rc = write_inst(bt, hi)) != CS_OK) break;
      any_newton = true;
    }
    // spares of the primaries that failed or succeeded in this mesh phase;
    // at the end of the solve, of every failed primary
    if (spares && (spares_on || !any_newton)) {
      spares_on = true;
      if ((rc = spare_pass(true)) != CS_OK) break;
      if (bt->h_n[4] > 0)
        for (auto& s : hi) any_newton |= (s.status == ST_FRESH || s.status == ST_LS);
    }
    if (!any_newton) break;
    set_cap(hi);
  }
  bt->work_cap = 0;
  bt->inst_cap = 0;
  if (rc == CS_OK) rc = check_config(bt);
  if (rc == CS_OK) CS_CUDA(cudaStreamSynchronize(bt->stream));
  return rc;
}

extern "C" int cs_batch_set_spares(cs_batch* bt, int n_primary, int trigger) {
  if (!bt) return set_err(CS_ERR_INVALID, "cs_batch_set_spares: null batch");
  if (n_primary < 0 || (n_primary > 0 && 2LL * n_primary != bt->B))
    return set_err(CS_ERR_INVALID, "cs_batch_set_spares: the batch must hold 2 * n_primary instances");
  const bool paired = n_primary != bt->n_primary;
  bt->n_primary = n_primary;
  bt->spare_trigger = trigger;
  if (n_primary == 0 || !paired || !bt->have_guess) return CS_OK;
  // park the spares that have not started since their guess was set
  std::vector<CsInst> hi;
  CS_TRY(read_inst(bt, hi));
  for (int b = n_primary; b < bt->B; ++b)
    if (hi[b].status == ST_FRESH && hi[b].residual_count == 0 && hi[b].jac_count == 0 && hi[b].remesh_count == 0)
      hi[b].status = ST_PARKED;
  CS_TRY(write_inst(bt, hi));
  CS_CUDA(cudaStreamSynchronize(bt->stream));
  return CS_OK;
}

extern "C" int cs_batch_set_progress(cs_batch* bt, cs_progress_fn fn, void* user) {
  if (!bt) return set_err(CS_ERR_INVALID, "cs_batch_set_progress: null batch");
  bt->progress = fn;
  bt->progress_user = user;
  return CS_OK;
}

extern "C" int cs_batch_sizes(cs_batch* bt, int* N_out, long long* total_out) {
  if (!bt) return set_err(CS_ERR_INVALID, "cs_batch_sizes: null batch");
  if (N_out) std::copy(bt->hN.begin(), bt->hN.end(), N_out);
  if (total_out) *total_out = bt->T;
  return CS_OK;
}

static int compute_znodes(cs_batch* bt) {
  CsBatchDev v = devview(bt);
  return run_slots(bt, bt->M->f_znodes, v);
}

extern "C" int cs_format_solutions(cs_batch* bt, char* out, long long cap, long long* offsets) {
  if (!bt || !bt->have_guess) return set_err(CS_ERR_STATE, "cs_format_solutions: nothing solved");
  if (!offsets) return set_err(CS_ERR_INVALID, "cs_format_solutions: null offsets");
  cs_module* M = bt->M;
  // z at the nodes, as cs_get_solution gives it
  if (M->nz > 0) CS_TRY(compute_znodes(bt));
  const int s = bt->cur;
  CsTextArgs a;
  a.t = (const double*)bt->t[s].p;
  a.y = (const double*)bt->y[s].p;
  a.z = (const double*)bt->znode[s].p;
  a.p = (const double*)bt->dp.p;
  a.T = bt->T;
  a.B = bt->B;
  a.ny = M->ny;
  a.nz = M->nz;
  a.np = M->np;
  a.dN = (const int*)bt->dN.p;
  a.doff = (const int*)bt->doff.p;
  a.stream = bt->stream;
  bt->launches += 3;
  return cs_text_files(a, out, cap, offsets);
}

extern "C" int cs_get_solution(cs_batch* bt, double* t, double* y, double* z, double* p, cs_stats* stats) {
  if (!bt || !bt->have_guess) return set_err(CS_ERR_STATE, "cs_get_solution: nothing solved");
  cs_module* M = bt->M;
  const size_t d = sizeof(double);
  const int s = bt->cur;
  cudaStream_t st = bt->stream;
  if (z && M->nz > 0) {
    CS_TRY(compute_znodes(bt));
    CS_CUDA(cudaMemcpyAsync(z, bt->znode[s].p, (size_t)bt->T * M->nz * d, cudaMemcpyDeviceToHost, st));
  }
  if (t) CS_CUDA(cudaMemcpyAsync(t, bt->t[s].p, (size_t)bt->T * d, cudaMemcpyDeviceToHost, st));
  if (y) CS_CUDA(cudaMemcpyAsync(y, bt->y[s].p, (size_t)bt->T * M->ny * d, cudaMemcpyDeviceToHost, st));
  if (p && M->np > 0) CS_CUDA(cudaMemcpyAsync(p, bt->dp.p, (size_t)bt->B * M->np * d, cudaMemcpyDeviceToHost, st));
  if (stats) {
    std::vector<CsInst> hi;
    CS_TRY(read_inst(bt, hi));
    for (int b = 0; b < bt->B; ++b) {
      const CsInst& q = hi[b];
      cs_stats& o = stats[b];
      o.status = q.status;
      o.N = bt->hN[b];
      o.newton_steps = q.jac_count;
      o.residual_evals = q.residual_count;
      o.segment_evals = q.seg_count;
      o.remeshes = q.remesh_count;
      o.continuation_steps = q.alphacal;
      o.singular = q.singular;
      o.fail_reason = q.fail_reason;
      o.alpha = q.alpha;
      o.max_residual = q.max_res;
      o.last_norm = q.norm_x;
    }
  }
  CS_CUDA(cudaStreamSynchronize(st));
  return CS_OK;
}

extern "C" int cs_get_state(cs_batch* bt, double* t, double* y, double* ydot, double* zt, double* z_nodes, double* p) {
  if (!bt || !bt->have_guess) return set_err(CS_ERR_STATE, "cs_get_state: no state");
  cs_module* M = bt->M;
  const size_t d = sizeof(double);
  const int s = bt->cur;
  cudaStream_t st = bt->stream;
  if (t) CS_CUDA(cudaMemcpyAsync(t, bt->t[s].p, (size_t)bt->T * d, cudaMemcpyDeviceToHost, st));
  if (y) CS_CUDA(cudaMemcpyAsync(y, bt->y[s].p, (size_t)bt->T * M->ny * d, cudaMemcpyDeviceToHost, st));
  if (ydot) CS_CUDA(cudaMemcpyAsync(ydot, bt->ydot[s].p, (size_t)bt->T * M->m * M->ny * d, cudaMemcpyDeviceToHost, st));
  if (zt && M->nz > 0) CS_CUDA(cudaMemcpyAsync(zt, bt->zt[s].p, (size_t)bt->T * M->m * M->nz * d, cudaMemcpyDeviceToHost, st));
  if (z_nodes && M->nz > 0) {
    CS_TRY(compute_znodes(bt));
    CS_CUDA(cudaMemcpyAsync(z_nodes, bt->znode[s].p, (size_t)bt->T * M->nz * d, cudaMemcpyDeviceToHost, st));
  }
  if (p && M->np > 0) CS_CUDA(cudaMemcpyAsync(p, bt->dp.p, (size_t)bt->B * M->np * d, cudaMemcpyDeviceToHost, st));
  CS_CUDA(cudaStreamSynchronize(st));
  return CS_OK;
}

// put every instance into `status` at continuation parameter alpha
static int set_all_status(cs_batch* bt, int status, double alpha, int need_jac) {
  std::vector<CsInst> hi;
  CS_TRY(read_inst(bt, hi));
  for (auto& s : hi) {
    s.status = status;
    s.alpha = alpha;
    s.need_jac = need_jac;
    s.accepted = 0;
    s.norm_bits = 0;
    s.res_bits = 0;
    s.ntrial = 1;
  }
  return write_inst(bt, hi);
}

extern "C" int cs_stage_residual(cs_batch* bt, double alpha, double* norms, double* f_a, double* f_b) {
  if (!bt || !bt->have_guess) return set_err(CS_ERR_STATE, "cs_stage_residual: no state");
  cs_module* M = bt->M;
  CS_TRY(set_all_status(bt, ST_FRESH, alpha, 0));
  DBuf fa, fb;
  if (f_a) CS_TRY(dalloc(fa, (size_t)bt->T * M->s * sizeof(double)));
  if (f_b) CS_TRY(dalloc(fb, (size_t)bt->T * M->ny * sizeof(double)));
  CsBatchDev v = devview(bt);
  v.fa_out = (double*)fa.p;
  v.fb_out = (double*)fb.p;
  int rc = run_lists(bt, v, 0, 0);
  if (rc == CS_OK) {
    void* args[] = {&v};
    rc = launch(bt, M->f_residual, (unsigned)M->res_grid, 256, 0, args);
  }
  std::vector<CsInst> hi;
  if (rc == CS_OK) rc = read_inst(bt, hi);
  if (rc == CS_OK && norms)
    for (int b = 0; b < bt->B; ++b) {
      unsigned long long bits = hi[b].norm_bits;
      double x;
      memcpy(&x, &bits, sizeof(x));
      norms[b] = x;
    }
  if (rc == CS_OK && f_a && cudaMemcpy(f_a, fa.p, (size_t)bt->T * M->s * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = set_err(CS_ERR_CUDA, "copy f_a");
  if (rc == CS_OK && f_b && cudaMemcpy(f_b, fb.p, (size_t)bt->T * M->ny * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = set_err(CS_ERR_CUDA, "copy f_b");
  dfree(fa);
  dfree(fb);
  if (rc == CS_OK) {
    for (auto& s : hi) s.norm_bits = 0;
    rc = write_inst(bt, hi);
  }
  return rc;
}

extern "C" int cs_stage_newton_direction(cs_batch* bt, double alpha, double* rows, double* dy, double* dydot,
                                         double* dzt, double* dp) {
  if (!bt || !bt->have_guess) return set_err(CS_ERR_STATE, "cs_stage_newton_direction: no state");
  cs_module* M = bt->M;
  CS_TRY(set_all_status(bt, ST_FRESH, alpha, 1));
  CsBatchDev v = devview(bt);
  const int nlvl = tree_levels(bt);
  CS_TRY(run_lists(bt, v, 1, use_cta_path(bt) ? 0 : nlvl));
  CS_TRY(run_condense(bt, v));
  const size_t d = sizeof(double);
  cudaStream_t st = bt->stream;
  if (rows) CS_CUDA(cudaMemcpyAsync(rows, bt->rows0.p, (size_t)bt->T * M->rowsz * d, cudaMemcpyDeviceToHost, st));
  CS_TRY(run_direction(bt, v, nlvl));
  if (dy) CS_CUDA(cudaMemcpyAsync(dy, bt->dy.p, (size_t)bt->T * M->ny * d, cudaMemcpyDeviceToHost, st));
  if (dydot) CS_CUDA(cudaMemcpyAsync(dydot, bt->dydot.p, (size_t)bt->T * M->m * M->ny * d, cudaMemcpyDeviceToHost, st));
  if (dzt && M->nz > 0) CS_CUDA(cudaMemcpyAsync(dzt, bt->dzt.p, (size_t)bt->T * M->m * M->nz * d, cudaMemcpyDeviceToHost, st));
  if (dp && M->np > 0) CS_CUDA(cudaMemcpyAsync(dp, bt->ddp.p, (size_t)bt->B * M->np * d, cudaMemcpyDeviceToHost, st));
  CS_CUDA(cudaStreamSynchronize(st));
  CS_TRY(check_config(bt));
  return set_all_status(bt, ST_FRESH, alpha, 0);
}

extern "C" int cs_stage_segment_residual(cs_batch* bt, double alpha, double tol, double* res, double* max_res) {
  if (!bt || !bt->have_guess) return set_err(CS_ERR_STATE, "cs_stage_segment_residual: no state");
  CS_TRY(set_all_status(bt, ST_SEG, alpha, 0));
  CsBatchDev v = devview(bt);
  int rtype = bt->opts.residual_type, scale = bt->opts.scale_by_time, res2 = bt->opts.residual2;
  void* as[] = {&v, &tol, &rtype, &scale, &res2};
  CS_TRY(launch(bt, bt->M->f_segres, cdiv(bt->T, 256), 256, 0, as));
  if (res) CS_CUDA(cudaMemcpyAsync(res, bt->res.p, (size_t)bt->T * sizeof(double), cudaMemcpyDeviceToHost, bt->stream));
  std::vector<CsInst> hi;
  CS_TRY(read_inst(bt, hi));
  if (max_res)
    for (int b = 0; b < bt->B; ++b) {
      unsigned long long bits = hi[b].res_bits;
      double x;
      memcpy(&x, &bits, sizeof(x));
      max_res[b] = x;
    }
  return set_all_status(bt, ST_FRESH, alpha, 0);
}

extern "C" int cs_stage_remesh(cs_batch* bt, const double* res, int* N_new) {
  if (!bt || !bt->have_guess || !res) return set_err(CS_ERR_STATE, "cs_stage_remesh: no state");
  CS_CUDA(cudaMemcpyAsync(bt->res.p, res, (size_t)bt->T * sizeof(double), cudaMemcpyHostToDevice, bt->stream));
  std::vector<CsInst> hi;
  CS_TRY(read_inst(bt, hi));
  for (auto& s : hi) s.status = ST_REMESH;
  CS_TRY(write_inst(bt, hi));
  CS_TRY(do_remesh(bt, hi));
  if (N_new) std::copy(bt->hN.begin(), bt->hN.end(), N_new);
  double a = bt->opts.alpha0;
  return set_all_status(bt, ST_FRESH, a, 0);
}

extern "C" int cs_time_condense(cs_batch* bt, int reps, double* ms) {
  if (!bt || !bt->have_guess || !ms || reps < 1) return set_err(CS_ERR_INVALID, "cs_time_condense: bad argument");
  CS_TRY(set_all_status(bt, ST_FRESH, bt->opts.alpha0, 1));
  CsBatchDev v = devview(bt);
  CS_TRY(run_lists(bt, v, 1, 0));
  CS_TRY(run_condense(bt, v));
  cudaEvent_t e0, e1;
  CS_CUDA(cudaEventCreate(&e0));
  CS_CUDA(cudaEventCreate(&e1));
  CS_CUDA(cudaEventRecord(e0, bt->stream));
  for (int r = 0; r < reps; ++r) CS_TRY(run_condense(bt, v));
  CS_CUDA(cudaEventRecord(e1, bt->stream));
  CS_CUDA(cudaEventSynchronize(e1));
  float t = 0.f;
  CS_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = (double)t / reps;
  CS_TRY(check_config(bt));
  return set_all_status(bt, ST_FRESH, bt->opts.alpha0, 0);
}

extern "C" int cs_measure_fp64_peak(double* tflops) {
  if (!tflops) return set_err(CS_ERR_INVALID, "cs_measure_fp64_peak: null");
  CS_TRY(ensure_context());
  int dev = 0, sms = 0;
  CS_CUDA(cudaGetDevice(&dev));
  CS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double* out = nullptr;
  CS_CUDA(cudaMalloc(&out, sizeof(double)));
  const int iters = 4096, block = 256, grid = sms * 8;
  k_dfma_peak<<<grid, block>>>(out, 64);
  cudaEvent_t e0, e1;
  CS_CUDA(cudaEventCreate(&e0));
  CS_CUDA(cudaEventCreate(&e1));
  CS_CUDA(cudaEventRecord(e0));
  k_dfma_peak<<<grid, block>>>(out, iters);
  CS_CUDA(cudaEventRecord(e1));
  CS_CUDA(cudaEventSynchronize(e1));
  float t = 0.f;
  CS_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double flops = 2.0 * 8.0 * iters * (double)grid * block;
  *tflops = flops / (t * 1e-3) / 1e12;
  return CS_OK;
}

extern "C" int cs_measure_dmma_peak(double* tflops) {
  if (!tflops) return set_err(CS_ERR_INVALID, "cs_measure_dmma_peak: null");
  CS_TRY(ensure_context());
  int dev = 0, sms = 0;
  CS_CUDA(cudaGetDevice(&dev));
  CS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double* out = nullptr;
  CS_CUDA(cudaMalloc(&out, sizeof(double)));
  const int iters = 2048, block = 256, grid = sms * 8;
  k_dmma_peak<<<grid, block>>>(out, 32);
  cudaEvent_t e0, e1;
  CS_CUDA(cudaEventCreate(&e0));
  CS_CUDA(cudaEventCreate(&e1));
  CS_CUDA(cudaEventRecord(e0));
  k_dmma_peak<<<grid, block>>>(out, iters);
  CS_CUDA(cudaEventRecord(e1));
  CS_CUDA(cudaEventSynchronize(e1));
  float t = 0.f;
  CS_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  // 2 * 8 * 8 * 4 flops per warp-wide m8n8k4, four per iteration
  const double flops = 512.0 * 4.0 * iters * (double)grid * (block / 32);
  *tflops = flops / (t * 1e-3) / 1e12;
  return CS_OK;
}

extern "C" int cs_batch_reset(cs_batch* bt) {
  if (!bt || !bt->have_guess || bt->iT == 0) return set_err(CS_ERR_STATE, "cs_batch_reset: no initial guess to restore");
  cs_module* M = bt->M;
  const size_t d = sizeof(double);
  const long long T = bt->iT;
  if (T > bt->cap) CS_TRY(alloc_slots(bt, T, false));
  cudaStream_t st = bt->stream;
  bt->cur = 0;
  bt->T = (int)T;
  bt->hN = bt->ihN;
  bt->hoff = bt->ihoff;
  CS_CUDA(cudaMemcpyAsync(bt->dN.p, bt->iN.p, bt->B * sizeof(int), cudaMemcpyDeviceToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->doff.p, bt->ioff.p, bt->B * sizeof(int), cudaMemcpyDeviceToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->t[0].p, bt->it.p, T * d, cudaMemcpyDeviceToDevice, st));
  CS_CUDA(cudaMemcpyAsync(bt->y[0].p, bt->iy.p, T * M->ny * d, cudaMemcpyDeviceToDevice, st));
  if (M->nz > 0) CS_CUDA(cudaMemcpyAsync(bt->znode[0].p, bt->iz.p, T * M->nz * d, cudaMemcpyDeviceToDevice, st));
  if (M->np > 0) CS_CUDA(cudaMemcpyAsync(bt->dp.p, bt->ip.p, (size_t)bt->B * M->np * d, cudaMemcpyDeviceToDevice, st));
  std::vector<CsInst> hi(bt->B);
  init_insts(bt, hi);
  CS_CUDA(cudaMemcpyAsync(bt->dinst.p, hi.data(), hi.size() * sizeof(CsInst), cudaMemcpyHostToDevice, st));
  CS_TRY(fill_inst_of(bt));
  CsBatchDev v = devview(bt);
  int only = -1;
  void* args[] = {&v, &only};
  CS_TRY(launch(bt, M->f_form_initial, cdiv(bt->T, 256), 256, 0, args));
  CS_CUDA(cudaStreamSynchronize(st));
  return CS_OK;
}

extern "C" int cs_batch_warm_start(cs_batch* bt, int n_nodes, const float* traj, int stride) {
  if (!bt || !bt->have_guess || !traj || n_nodes < 1) return set_err(CS_ERR_INVALID, "cs_batch_warm_start: bad argument");
  cs_module* M = bt->M;
  if (stride < n_nodes * (M->ny + M->nz) + M->np) return set_err(CS_ERR_INVALID, "cs_batch_warm_start: stride too small");
  const int s = bt->cur;
  // with spares only the primaries take the trajectories; the spares keep
  // their records (parked) and guesses
  const int nf = bt->n_primary > 0 ? bt->n_primary : bt->B;
  k_warm_fill<<<nf, 128, 0, bt->stream>>>(nf, M->ny, M->nz, M->np, n_nodes, traj, stride, (const int*)bt->dN.p,
                                          (const int*)bt->doff.p, (const double*)bt->t[s].p, (double*)bt->y[s].p,
                                          (double*)bt->znode[s].p, (double*)bt->dp.p);
  CS_CUDA(cudaGetLastError());
  bt->launches += 1;
  std::vector<CsInst> hi(nf);
  for (auto& q : hi) init_inst(q, bt->opts.alpha0);
  CS_CUDA(cudaMemcpyAsync(bt->dinst.p, hi.data(), hi.size() * sizeof(CsInst), cudaMemcpyHostToDevice, bt->stream));
  CsBatchDev v = devview(bt);
  int only = -1;
  void* args[] = {&v, &only};
  CS_TRY(launch(bt, M->f_form_initial, cdiv(bt->T, 256), 256, 0, args));
  CS_CUDA(cudaStreamSynchronize(bt->stream));
  return CS_OK;
}

extern "C" void* cs_device_alloc(size_t bytes) {
  if (ensure_context() != CS_OK) return nullptr;
  void* p = nullptr;
  if (cudaMalloc(&p, bytes ? bytes : 8) != cudaSuccess) {
    set_err(CS_ERR_NOMEM, "cudaMalloc failed");
    return nullptr;
  }
  return p;
}

extern "C" void cs_device_free(void* p) {
  if (p) cudaFree(p);
}

extern "C" int cs_copy(void* dst, const void* src, size_t bytes, int kind) {
  if (!dst || !src) return set_err(CS_ERR_INVALID, "cs_copy: null pointer");
  cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice : (kind == 1 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice);
  CS_CUDA(cudaMemcpy(dst, src, bytes, k));
  return CS_OK;
}

extern "C" int cs_profile_reset(cs_batch* bt, int timing) {
  if (!bt) return set_err(CS_ERR_INVALID, "cs_profile_reset: null batch");
  CS_TRY(flush_events(bt));
  bt->launches = bt->super_steps = 0;
  for (int k = 0; k < 3; ++k) {
    bt->kind_ms[k] = 0;
    bt->kind_launches[k] = 0;
  }
  bt->timing = timing != 0;
  CS_CUDA(cudaMemsetAsync(bt->dcounters.p, 0, 8 * sizeof(unsigned long long), bt->stream));
  CS_CUDA(cudaStreamSynchronize(bt->stream));
  return CS_OK;
}

extern "C" int cs_profile_get(cs_batch* bt, cs_profile* out) {
  if (!bt || !out) return set_err(CS_ERR_INVALID, "cs_profile_get: null argument");
  CS_TRY(flush_events(bt));
  unsigned long long c[8];
  CS_CUDA(cudaMemcpyAsync(c, bt->dcounters.p, sizeof(c), cudaMemcpyDeviceToHost, bt->stream));
  CS_CUDA(cudaStreamSynchronize(bt->stream));
  out->launches = bt->launches;
  out->super_steps = bt->super_steps;
  out->intervals_condensed = (long long)c[1];
  out->systems_solved = (long long)c[2];
  out->residual_intervals = (long long)c[3];
  out->condense_launches = bt->kind_launches[0];
  out->babd_launches = bt->kind_launches[1];
  out->residual_launches = bt->kind_launches[2];
  out->condense_ms = bt->kind_ms[0];
  out->babd_ms = bt->kind_ms[1];
  out->residual_ms = bt->kind_ms[2];
  return CS_OK;
}

extern "C" void* cs_pinned_alloc(size_t bytes) {
  if (ensure_context() != CS_OK) return nullptr;
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes ? bytes : 8) != cudaSuccess) {
    set_err(CS_ERR_NOMEM, "cudaMallocHost failed");
    return nullptr;
  }
  return p;
}

extern "C" void cs_pinned_free(void* p) {
  if (p) cudaFreeHost(p);
}

extern "C" int cs_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return (int)g_err.size();
  size_t n = std::min(len - 1, g_err.size());
  memcpy(buf, g_err.data(), n);
  buf[n] = '\0';
  return (int)g_err.size();
}

extern "C" int cs_profiler_start(void) {
  CS_TRY(ensure_context());
  CS_CUDA(cudaDeviceSynchronize());
  CS_CUDA(cudaProfilerStart());
  return CS_OK;
}

extern "C" int cs_profiler_stop(void) {
  CS_CUDA(cudaDeviceSynchronize());
  CS_CUDA(cudaProfilerStop());
  return CS_OK;
}

extern "C" int cs_autotune_condense(cs_batch* bt, int reps, cs_tune_result* out) {
  if (!bt || !bt->have_guess || reps < 1) return set_err(CS_ERR_INVALID, "cs_autotune_condense: bad argument");
  cs_module* M = bt->M;
  CS_TRY(set_all_status(bt, ST_FRESH, bt->opts.alpha0, 1));
  CsBatchDev v = devview(bt);
  CS_TRY(run_lists(bt, v, 1, 0));
  struct Cand {
    CUfunction f;
    int lanes, block, grid;
    size_t smem;
  };
  std::vector<Cand> cands;
  cands.push_back({M->f_condense, M->big_cond ? 0 : M->cgw, M->condense_block, M->condense_grid, M->condense_smem});
  if (!M->big_cond) {
    const int lanes[4] = {4, 8, 16, 32};
    for (int k = 0; k < 4; ++k) {
      if (!M->f_cond_l[k]) continue;
      const int gpw = 32 / lanes[k];
      for (int w = 1; w <= 8; w *= 2) {
        const size_t smem = M->grp_bytes * gpw * w;
        if (smem > (size_t)M->smem_optin) break;
        if (smem > 48 * 1024)
          CS_CU(g_drv.funcSetAttribute(M->f_cond_l[k], CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem));
        int per_sm = 0;
        CS_CU(g_drv.occupancy(&per_sm, M->f_cond_l[k], 32 * w, smem));
        if (per_sm < 1) continue;
        cands.push_back({M->f_cond_l[k], lanes[k], 32 * w, M->sms * per_sm, smem});
      }
    }
  } else {
    // one CTA per interval: CTA size; the grid stays within the CTAs that
    // have a slab in this batch
    for (int block = 128; block <= 256; block *= 2) {
      int per_sm = 0;
      CS_CU(g_drv.occupancy(&per_sm, M->f_condense, block, M->condense_smem));
      const int grid = std::min(M->sms * std::max(1, per_sm), M->big_ctas);
      cands.push_back({M->f_condense, 0, block, grid, M->condense_smem});
    }
  }
  cudaEvent_t e0, e1;
  CS_CUDA(cudaEventCreate(&e0));
  CS_CUDA(cudaEventCreate(&e1));
  double best = 1e300, first = 0.0;
  size_t bi = 0;
  for (size_t i = 0; i < cands.size(); ++i) {
    const Cand& c = cands[i];
    void* args[] = {&v};
    CS_CU(g_drv.launchKernel(c.f, c.grid, 1, 1, c.block, 1, 1, (unsigned)c.smem, (CUstream)bt->stream, args, nullptr));
    CS_CUDA(cudaEventRecord(e0, bt->stream));
    for (int r = 0; r < reps; ++r)
      CS_CU(g_drv.launchKernel(c.f, c.grid, 1, 1, c.block, 1, 1, (unsigned)c.smem, (CUstream)bt->stream, args, nullptr));
    CS_CUDA(cudaEventRecord(e1, bt->stream));
    CS_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    CS_CUDA(cudaEventElapsedTime(&t, e0, e1));
    const double ms = (double)t / reps;
    if (i == 0) first = ms;
    if (ms < best) {
      best = ms;
      bi = i;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CS_TRY(check_config(bt));
  const Cand& b = cands[bi];
  if (bi != 0) {
    M->f_condense = b.f;
    M->condense_block = b.block;
    M->condense_grid = b.grid;
    M->condense_smem = b.smem;
    if (!M->big_cond) M->cgw = b.lanes;
    M->tune_ver += 1;
  }
  if (out) {
    out->lanes = b.lanes;
    out->block = b.block;
    out->grid = b.grid;
    out->candidates = (int)cands.size();
    out->ms = best;
    out->default_ms = first;
  }
  return set_all_status(bt, ST_FRESH, bt->opts.alpha0, 0);
}
