// Collocation Newton-loop kernels for GB300 (sm_103a), FP64.
//
// This file is compiled at run time by NVRTC, once per (problem, m), after a
// prelude that defines the sizes as compile-time constants and the problem
// functions cs_f/cs_g/cs_Df/cs_Dg/cs_r/cs_Dr (emitted from the OCP's sympy
// derivation), plus the collocation tables:
//
//   CS_NY, CS_NZ, CS_NP   sizes of y, z, p
//   CS_NPE                parameters f and g depend on (leading entries of p)
//   CS_NTH                instance constants
//   CS_M                  Lobatto collocation points
//   CS_A[M*M], CS_B[M], CS_C[M]                    Lobatto IIIA tableau
//   CS_GW[M+1], CS_GL[(M+1)*M], CS_GI[(M+1)*M]     Gauss weights, basis L_k
//                                                  and its integral I_k at the
//                                                  (M+1) Gauss points
//   CS_L0[M], CS_L1[M]    basis at t = 0 and t = 1
//
// Data layout in HBM (batch of B instances, packed by node):
//   instance b owns node slots off[b] .. off[b]+N[b]-1; interval i of b uses
//   slot off[b]+i (i < N[b]-1).  Per node: t, y[NY], dy[NY], z-at-node[NZ]
//   (remesh scratch), segment residual.  Per interval slot: y'[M][NY],
//   z~[M][NZ], their Newton steps, X = W^-1 [J | V_eff | f_a] stored
//   column-major [NRHS][S], the level-0 BABD block row, the tree record of the
//   node eliminated at that slot.
//
// Reference counterparts (UW-OCP/Collocation-Solver-CUDA):
//   k_form_initial   form_initial_input_kernel        collocation_solver_parallel_2d_shared.py:316-356
//   k_residual       collocation_update_kernel + compute_f_q_kernel1/2 + host
//                    assembly and norm                 collocation_solver_parallel_2d_shared.py:399-559, 116
//   k_condense       construct_jacobian_kernel + reduce_jacobian_parallel_kernel
//                                                      collocation_solver_parallel_2d_shared.py:680-1001
//   k_tree_level, k_upper, k_top, k_backsub_level, k_recover
//                    partition_factorization_kernel, the host reduced solve,
//                    partition_backward_substitution_kernel, recover_delta_k_kernel
//                                                      solve_babd_system.py:161-572, collocation_solver_parallel_2d_shared.py:1619-1650
//   k_lists          (none: compacts the work of the batch every super-step)
//   k_decide/k_accept  Newton loop and line search    collocation_solver_parallel_2d_shared.py:105-180
//   k_segres         compute_segment_residual_kernel(2) collocation_solver_parallel_2d_shared.py:1833-2013
//   k_remesh_*       recover_solution_kernel + remesh  collocation_solver_parallel_2d_shared.py:2049-2311

#define CS_S (CS_M * (CS_NY + CS_NZ))          // stage unknowns per interval
#define CS_NRHS (CS_NY + CS_NPE + 1)           // right-hand sides of the condensation
#define CS_NCOL (CS_S + CS_NRHS)               // augmented condensation matrix width
#define CS_LDW (CS_NCOL | 1)                   // odd leading dimension in shared memory
#define CS_ROWSZ (CS_NY * (2 * CS_NY + CS_NPE + 1))   // block row: A | C | H | b (column-major)
#define CS_TREESZ (CS_NY * (3 * CS_NY + CS_NPE + 1))  // tree record: R | G | E | J | d
#define CS_QC (3 * CS_NY + CS_NPE + 1)         // columns of a merge
#define CS_QLD ((2 * CS_NY) | 1)               // leading dim (rows) of a merge, column-major
#define CS_NT (2 * CS_NY + CS_NP)              // top system size
#define CS_TLD (CS_NT | 1)
#define CS_NFG (CS_NY + CS_NZ + CS_NP)         // columns of Df, Dg

#define ST_FRESH 0
#define ST_LS 1
#define ST_SEG 2
#define ST_DONE 3
#define ST_FAIL 4
#define ST_REMESH 5
// spares (host-managed pairing): parked with their initial guess, or stopped;
// no kernel of the state machine takes either
#define ST_PARKED 6
#define ST_CANCELLED 7

#define FAIL_NONE 0
#define FAIL_ITER 1
#define FAIL_NODES 2
#define FAIL_MESH 3

// Line-search trials evaluated in one super-step once the first trial of a
// direction was rejected (alpha, alpha/2, ...; the decision walks them in
// order, so the accepted trial and every count are the sequential ones).
// Their norms live in CsBatch::trials ([B][CS_LSW]).
#define CS_LSW 20

struct CsInst {
  int status, it, ls_it, alphacal;
  int need_jac, accepted, fail_reason, N_new;
  int residual_count, jac_count, seg_count, remesh_count;
  int iter_time, singular, ntrial, ls_prev;   // trials of the next residual evaluation; rejected trials of the last line search
  double alpha_ls, norm_x, alpha, max_res;
  unsigned long long norm_bits, res_bits;
};

struct CsConsts {
  double tol, alpha_m, beta;
  int max_iter, max_mesh, max_nodes, min_nodes, max_ls;
  int ls_grow;  // trials of a new line search after one that rejected some (cs_opts.ls_grow)
};

struct CsBatch {
  int B, T;                 // instances, node slots in use
  const int* N;             // nodes per instance
  const int* off;           // first node slot per instance
  const int* inst_of;       // instance owning each slot
  double* t;                // [T]
  double* y;                // [T][NY]
  double* ydot;             // [T][M][NY]
  double* zt;               // [T][M][NZ]
  double* p;                // [B][NP]
  const double* th;         // [B][NTH]
  double* dy;               // [T][NY]
  double* dydot;            // [T][M][NY]
  double* dzt;              // [T][M][NZ]
  double* dp;               // [B][NP]
  double* X;                // [T][NRHS][S]
  double* rows0;            // [T][ROWSZ]
  double* rows1;            // [T][ROWSZ]
  double* tree;             // [T][TREESZ]
  double* res;              // [T] segment residual per node
  double* znode;            // [T][NZ] z at nodes (remesh / initial input)
  CsInst* inst;             // [B]
  unsigned long long* counters;  // [0] instances in Newton this step, [1] intervals condensed,
                                 // [2] BABD systems solved, [3] interval residuals evaluated
  double* fa_out;           // optional [T][S]: residual pieces (stage entry point)
  double* fb_out;           // optional [T][NY]
  // work lists, rebuilt by k_lists every super-step: only the instances that
  // have work are visited, so a batch whose stragglers are few costs little
  int* act;                 // [B] instances that need a residual evaluation
  int* jac;                 // [B] instances that need a Newton direction
  int* acc;                 // [B] instances whose line-search trial was accepted
  long long* act_pre;       // [B+1] prefix of their interval counts
  long long* jac_pre;       // [B+1] prefix of interval counts
  long long* acc_pre;       // [B+1] prefix of node counts
  long long* lvl_pre;       // [CS_MAXLVL][B+1] prefix of tree items per level over jac
  int* nlist;               // [4] nact, njac, nacc, -
  unsigned long long* trials;  // [B][CS_LSW] residual norms of line-search trials 1.. (bits)
  // large stage systems (CS_BIG): a slab of global memory per CTA
  double* wsp;              // [wsp_ctas][wsp_stride]
  long long wsp_stride;     // doubles per CTA
  int wsp_ctas, wsp_pad;
};

// Large-system kernels (global-memory slab per CTA): CS_BIG_COND selects
// the blocked-LU condensation, CS_BIG_TREE the CTA-per-merge tree and the
// CTA top solve; each is chosen when its blocks outgrow the shared-memory
// kernels (the condensation also when a whole CTA would serve an interval).
#ifndef CS_BIG_COND
#define CS_BIG_COND 0
#endif
#ifndef CS_BIG_TREE
#define CS_BIG_TREE 0
#endif
#define CS_BIG (CS_BIG_COND || CS_BIG_TREE)
// precision of the large-system condensation: 0 FP64, 1 TF32 / 2 BF16 tensor
// cores with FP32 storage and accumulation (an inexact Newton Jacobian; the
// residual, line search, mesh error and BABD solve stay FP64)
#ifndef CS_PREC
#define CS_PREC 0
#endif
// precision of the large-system tree merges: 0 FP64, 1 TF32, 2 BF16 (an
// option only: the merges' rounding makes the Newton direction too inexact,
// measured on the pendulum chains)
#ifndef CS_PREC_TREE
#define CS_PREC_TREE 0
#endif
#ifndef CS_SMEM_MAX
#define CS_SMEM_MAX 232448
#endif

#define CS_MAXLVL 32

static constexpr double CS_EPS = 2.220446049250313e-16;

__device__ __forceinline__ unsigned long long cs_abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(fabs(v));
}
__device__ __forceinline__ double cs_from_bits(unsigned long long b) { return __longlong_as_double((long long)b); }

// Max of non-negative double bit patterns over the lanes of a warp that share
// an instance, then one atomicMax per instance.  All 32 lanes must call it.
__device__ __forceinline__ void cs_warp_max_atomic(unsigned long long* dst, int key, unsigned long long v, bool active) {
  const unsigned peers = __match_any_sync(0xffffffffu, active ? key : -1);
  const unsigned hi = (unsigned)(v >> 32), lo = (unsigned)(v & 0xffffffffull);
  const unsigned mhi = __reduce_max_sync(peers, hi);
  const unsigned mlo = __reduce_max_sync(peers, hi == mhi ? lo : 0u);
  const int leader = __ffs(peers) - 1;
  if (active && (int)(threadIdx.x & 31) == leader) atomicMax(dst, ((unsigned long long)mhi << 32) | mlo);
}

// first k with pre[k] <= w < pre[k+1] (pre ascending, n entries + total)
__device__ __forceinline__ int cs_find(const long long* pre, int n, long long w) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= w) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// block rows at tree level l for n0 rows at level 0 (each level halves, rounding up)
__device__ __forceinline__ int cs_rows_at(int n0, int l) {
  int n = n0;
  for (int q = 0; q < l; ++q) n = (n + 1) >> 1;
  return n;
}
__device__ __forceinline__ int cs_levels(int n0) {
  int L = 0, n = n0;
  while (n > 1) { n = (n + 1) >> 1; ++L; }
  return L;
}
// items of tree level l: ceil(n_l / 2) (merges plus the carried odd row)
__device__ __forceinline__ long long cs_level_items(int n0, int l) {
  int n = cs_rows_at(n0, l);
  return n > 1 ? (long long)((n + 1) >> 1) : 0ll;
}

// ------------------------------------------------------------------------
// Initial stage values on a (new) mesh: y~ = (1-c) y_i + c y_{i+1},
// z~ likewise from z at nodes, y' = f(y~, z~, p).
extern "C" __global__ void k_form_initial(CsBatch bt, int only_status) {
  int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= bt.T) return;
  int b = bt.inst_of[slot];
  int i = slot - bt.off[b];
  if (i >= bt.N[b] - 1) return;
  if (only_status >= 0 && bt.inst[b].status != only_status) return;
  const double* p = bt.p + (size_t)b * CS_NP;
  const double* th = bt.th + (size_t)b * (CS_NTH > 0 ? CS_NTH : 1);
  double pl[CS_NP > 0 ? CS_NP : 1];
  for (int k = 0; k < CS_NP; ++k) pl[k] = p[k];
  const double* y0 = bt.y + (size_t)slot * CS_NY;
  const double* y1 = y0 + CS_NY;
  const double* z0 = bt.znode + (size_t)slot * CS_NZ;
  const double* z1 = z0 + CS_NZ;
#pragma unroll 1
  for (int j = 0; j < CS_M; ++j) {
    double c = CS_C[j];
    double yt[CS_NY], ztl[CS_NZ > 0 ? CS_NZ : 1], f[CS_NY];
    for (int k = 0; k < CS_NY; ++k) yt[k] = (1.0 - c) * y0[k] + c * y1[k];
    for (int k = 0; k < CS_NZ; ++k) ztl[k] = (1.0 - c) * z0[k] + c * z1[k];
    cs_f(yt, ztl, pl, th, f);
    double* yd = bt.ydot + ((size_t)slot * CS_M + j) * CS_NY;
    for (int k = 0; k < CS_NY; ++k) yd[k] = f[k];
    double* zo = bt.zt + ((size_t)slot * CS_M + j) * CS_NZ;
    for (int k = 0; k < CS_NZ; ++k) zo[k] = ztl[k];
  }
}

// ------------------------------------------------------------------------
// Residual infinity norm at the trial point x + alpha_ls * dx (LS) or x
// (FRESH): collocation update, f_a = [f(y~,z~,p) - y'; g], f_b and, on
// interval 0, the boundary conditions.
extern "C" __global__ void k_residual(CsBatch bt) {
  const int nact = bt.nlist[0];
  const long long total = bt.act_pre[nact];
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < total; base += stride) {
    const long long w = base + (threadIdx.x & 31);
    bool active = w < total;
    int b = 0, i = 0, slot = 0, st = -1;
    if (active) {
      const int k = cs_find(bt.act_pre, nact, w);
      b = bt.act[k];
      i = (int)(w - bt.act_pre[k]);
      slot = bt.off[b] + i;
      st = bt.inst[b].status;
      active = (st == ST_FRESH || st == ST_LS);
    }
    unsigned long long nb = 0;
    int trial = 0;
    if (active) {
      const bool ls = (st == ST_LS);
      if (ls) {
        // item i of instance b covers trial i / (N-1), interval i % (N-1)
        const int nm1 = bt.N[b] - 1;
        trial = i / nm1;
        i -= trial * nm1;
        slot = bt.off[b] + i;
      }
      double a = ls ? bt.inst[b].alpha_ls : 0.0;
      for (int q = 0; q < trial; ++q) a *= 0.5;
      const double* th = bt.th + (size_t)b * (CS_NTH > 0 ? CS_NTH : 1);
      double pl[CS_NP > 0 ? CS_NP : 1];
      for (int k = 0; k < CS_NP; ++k) {
        double v = bt.p[(size_t)b * CS_NP + k];
        pl[k] = ls ? fma(a, bt.dp[(size_t)b * CS_NP + k], v) : v;
      }
      double yi[CS_NY], yi1[CS_NY];
      for (int k = 0; k < CS_NY; ++k) {
        double v0 = bt.y[(size_t)slot * CS_NY + k], v1 = bt.y[(size_t)(slot + 1) * CS_NY + k];
        yi[k] = ls ? fma(a, bt.dy[(size_t)slot * CS_NY + k], v0) : v0;
        yi1[k] = ls ? fma(a, bt.dy[(size_t)(slot + 1) * CS_NY + k], v1) : v1;
      }
      double yd[CS_M][CS_NY];
      for (int j = 0; j < CS_M; ++j)
        for (int k = 0; k < CS_NY; ++k) {
          size_t q = ((size_t)slot * CS_M + j) * CS_NY + k;
          yd[j][k] = ls ? fma(a, bt.dydot[q], bt.ydot[q]) : bt.ydot[q];
        }
      const double h = bt.t[slot + 1] - bt.t[slot];
      double mx = 0.0;
      bool nan = false;
  #pragma unroll 1
      for (int j = 0; j < CS_M; ++j) {
        double yt[CS_NY], zl[CS_NZ > 0 ? CS_NZ : 1], f[CS_NY];
        for (int k = 0; k < CS_NY; ++k) {
          double s = 0.0;
          for (int q = 0; q < CS_M; ++q) s += CS_A[j * CS_M + q] * yd[q][k];
          yt[k] = yi[k] + h * s;
        }
        for (int k = 0; k < CS_NZ; ++k) {
          size_t q = ((size_t)slot * CS_M + j) * CS_NZ + k;
          zl[k] = ls ? fma(a, bt.dzt[q], bt.zt[q]) : bt.zt[q];
        }
        cs_f(yt, zl, pl, th, f);
        for (int k = 0; k < CS_NY; ++k) {
          double r = f[k] - yd[j][k];
          nan |= (r != r);
          mx = fmax(mx, fabs(r));
          if (bt.fa_out && trial == 0) bt.fa_out[(size_t)slot * CS_S + j * (CS_NY + CS_NZ) + k] = r;
        }
  #if CS_NZ > 0
        double g[CS_NZ];
        cs_g(yt, zl, pl, th, bt.inst[b].alpha, g);
        for (int k = 0; k < CS_NZ; ++k) {
          nan |= (g[k] != g[k]);
          mx = fmax(mx, fabs(g[k]));
          if (bt.fa_out && trial == 0) bt.fa_out[(size_t)slot * CS_S + j * (CS_NY + CS_NZ) + CS_NY + k] = g[k];
        }
  #endif
      }
      for (int k = 0; k < CS_NY; ++k) {
        double s = 0.0;
        for (int j = 0; j < CS_M; ++j) s += CS_B[j] * yd[j][k];
        double r = yi1[k] - yi[k] - h * s;
        nan |= (r != r);
        mx = fmax(mx, fabs(r));
        if (bt.fb_out && trial == 0) bt.fb_out[(size_t)slot * CS_NY + k] = r;
      }
      if (i == 0) {
        int last = bt.off[b] + bt.N[b] - 1;
        double ya[CS_NY], yb[CS_NY], r[CS_NY + CS_NP];
        for (int k = 0; k < CS_NY; ++k) {
          double v0 = bt.y[(size_t)slot * CS_NY + k], v1 = bt.y[(size_t)last * CS_NY + k];
          ya[k] = ls ? fma(a, bt.dy[(size_t)slot * CS_NY + k], v0) : v0;
          yb[k] = ls ? fma(a, bt.dy[(size_t)last * CS_NY + k], v1) : v1;
        }
        cs_r(ya, yb, pl, th, r);
        for (int k = 0; k < CS_NY + CS_NP; ++k) {
          nan |= (r[k] != r[k]);
          mx = fmax(mx, fabs(r[k]));
        }
      }
      nb = nan ? 0x7ff8000000000000ull : cs_abs_bits(mx);
    }

    unsigned long long* dst = nullptr;
    if (active) dst = trial == 0 ? &bt.inst[b].norm_bits : &bt.trials[(size_t)b * CS_LSW + trial];
    cs_warp_max_atomic(dst, b * CS_LSW + trial, nb, active);
  }
}

// ------------------------------------------------------------------------
// Newton / line-search control, one thread per instance.
__device__ void cs_post_newton(CsInst& s, int N, const CsConsts& c, int iter_time) {
  s.need_jac = 0;
  s.iter_time = iter_time;
  if (s.alphacal >= c.max_iter - 1 || iter_time >= c.max_iter - 1) { s.status = ST_FAIL; s.fail_reason = FAIL_ITER; return; }
  if (N > c.max_nodes || N < c.min_nodes) { s.status = ST_FAIL; s.fail_reason = FAIL_NODES; return; }
  if (0 > c.max_mesh) { s.status = ST_FAIL; s.fail_reason = FAIL_MESH; return; }
  s.status = ST_SEG;
}

// start of Newton iteration s.it, residual norm at x known (s.norm_x)
__device__ void cs_iteration_start(CsInst& s, int N, const CsConsts& c, bool count_residual) {
  if (s.it == c.max_iter) { cs_post_newton(s, N, c, c.max_iter - 1); return; }
  if (count_residual) s.residual_count += 1;
  if (s.norm_x < c.tol) { cs_post_newton(s, N, c, s.it); return; }
  s.need_jac = 1;
  s.it += 1;
  s.jac_count += 1;
}

extern "C" __global__ void k_decide(CsBatch bt, CsConsts c) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= bt.B) return;
  CsInst s = bt.inst[b];
  s.accepted = 0;
  s.need_jac = 0;
  if (s.status == ST_FRESH || s.status == ST_LS) {
    const int ntr = (s.status == ST_LS) ? max(1, s.ntrial) : 1;
    atomicAdd(&bt.counters[3], (unsigned long long)(bt.N[b] - 1) * ntr);
    double nt = cs_from_bits(s.norm_bits);
    s.norm_bits = 0ull;
    s.residual_count += 1;
    s.ntrial = 1;
    if (s.status == ST_FRESH) {
      s.norm_x = nt;
      cs_iteration_start(s, bt.N[b], c, false);
    } else {
      // trials in the reference's order: alpha_ls, alpha_ls/2, ...
      bool done = false;
      for (int j = 0; j < ntr && !done; ++j) {
        const double ntj = (j == 0) ? nt : cs_from_bits(bt.trials[(size_t)b * CS_LSW + j]);
        if (j > 0) s.residual_count += 1;
        if (ntj < s.norm_x) {
          s.accepted = 1;
          s.norm_x = ntj;
          s.ls_prev = s.ls_it;
          cs_iteration_start(s, bt.N[b], c, true);
          done = true;
          break;
        }
        s.ls_it += 1;
        s.alpha_ls *= 0.5;
        if (s.ls_it >= c.max_ls) {
          // No trial accepted: the iterate is unchanged, so every remaining
          // Newton iteration recomputes the same residual, Jacobian,
          // direction and rejected trials (the reference loops exactly so
          // until max_iter, collocation_solver_parallel_2d_shared.py:109-174).
          // Take that outcome directly: same state, same counts, then the
          // iteration-limit failure.
          const int rem = c.max_iter - s.it;
          if (rem > 0) {
            s.residual_count += rem * (1 + c.max_ls);
            s.jac_count += rem;
            s.it = c.max_iter;
          }
          cs_iteration_start(s, bt.N[b], c, false);
          done = true;
        }
      }
      for (int j = 1; j < ntr; ++j) bt.trials[(size_t)b * CS_LSW + j] = 0ull;
      // still searching: the next super-step evaluates several trials
      if (!done) s.ntrial = min(CS_LSW, c.max_ls - s.ls_it);
    }
    // a new direction follows: an instance whose last line search rejected
    // trials evaluates several at once from the start
    // (ls_grow > 0: as many as ls_grow times the trials the last search
    // rejected, plus two; the rest, if needed, in the next super-step)
    if (s.need_jac) {
      const int many = min(CS_LSW, c.max_ls);
      s.ntrial = (s.ls_prev > 0) ? (c.ls_grow > 0 ? min(many, c.ls_grow * s.ls_prev + 2) : many) : 1;
    }
    if (s.status == ST_FRESH || s.status == ST_LS || s.need_jac) atomicAdd(&bt.counters[0], 1ull);
    if (s.need_jac) {
      atomicAdd(&bt.counters[1], (unsigned long long)(bt.N[b] - 1));
      atomicAdd(&bt.counters[2], 1ull);
    }
  }
  bt.inst[b] = s;
}

// x += alpha_ls * dx for instances whose trial was accepted (items: their nodes)
extern "C" __global__ void k_accept(CsBatch bt) {
  const int nacc = bt.nlist[2];
  const long long total = bt.acc_pre[nacc];
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < total; w += (long long)gridDim.x * blockDim.x) {
    const int k = cs_find(bt.acc_pre, nacc, w);
    const int b = bt.acc[k];
    const int i = (int)(w - bt.acc_pre[k]);
    const int slot = bt.off[b] + i;
    const int N = bt.N[b];
    const double a = bt.inst[b].alpha_ls;
    for (int q = 0; q < CS_NY; ++q) bt.y[(size_t)slot * CS_NY + q] = fma(a, bt.dy[(size_t)slot * CS_NY + q], bt.y[(size_t)slot * CS_NY + q]);
    if (i >= N - 1) continue;
    for (int q = 0; q < CS_M * CS_NY; ++q) {
      size_t o = (size_t)slot * CS_M * CS_NY + q;
      bt.ydot[o] = fma(a, bt.dydot[o], bt.ydot[o]);
    }
    for (int q = 0; q < CS_M * CS_NZ; ++q) {
      size_t o = (size_t)slot * CS_M * CS_NZ + q;
      bt.zt[o] = fma(a, bt.dzt[o], bt.zt[o]);
    }
    if (i == 0)
      for (int q = 0; q < CS_NP; ++q) bt.p[(size_t)b * CS_NP + q] = fma(a, bt.dp[(size_t)b * CS_NP + q], bt.p[(size_t)b * CS_NP + q]);
  }
}

// ------------------------------------------------------------------------
// Work lists.  One CTA of 1024 threads scans the instances:
//   mode 0: act = instances in FRESH or LS; jac, acc empty
//   mode 1: (after k_decide) act = FRESH/LS or needing a Jacobian, jac =
//           needing a Jacobian, acc = accepted trials; plus, for each tree
//           level l < nlvl, the prefix of that level's items over jac.
__device__ long long cs_block_scan(long long v, long long* sh, long long* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long x = v;
  for (int o = 1; o < 32; o <<= 1) {
    long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    long long q = (lane < nw) ? sh[lane] : 0ll;
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(0xffffffffu, q, o);
      if (lane >= o) q += y;
    }
    if (lane < nw) sh[lane] = q;
  }
  __syncthreads();
  const long long excl = x - v + (w > 0 ? sh[w - 1] : 0ll);
  *total = sh[nw - 1];
  __syncthreads();
  return excl;
}

template <typename F, typename Wt>
__device__ int cs_build_list(int n, F flag, Wt weight, int* list, long long* pre, long long* sh) {
  long long cpos = 0, cw = 0;
  for (int base = 0; base < n; base += blockDim.x) {
    const int b = base + threadIdx.x;
    const int f = (b < n && flag(b)) ? 1 : 0;
    const long long wv = f ? weight(b) : 0ll;
    long long tf, tw;
    const long long pf = cs_block_scan((long long)f, sh, &tf);
    const long long pw = cs_block_scan(wv, sh, &tw);
    if (f) {
      if (list) list[cpos + pf] = b;
      pre[cpos + pf] = cw + pw;
    }
    cpos += tf;
    cw += tw;
  }
  if (threadIdx.x == 0) pre[cpos] = cw;
  __syncthreads();
  return (int)cpos;
}

// residual work items of an instance: its intervals times the line-search
// trials of its next residual evaluation
__device__ __forceinline__ long long cs_res_items(const CsInst& s, int N) {
  const int t = (s.status == ST_LS || s.need_jac) ? max(1, s.ntrial) : 1;
  return (long long)(N - 1) * t;
}

extern "C" __global__ void k_lists(CsBatch bt, int mode, int nlvl) {
  __shared__ long long sh[32];
  const int B = bt.B;
  const CsInst* I = bt.inst;
  const int* N = bt.N;
  int nact, njac = 0, nacc = 0;
  if (mode == 0) {
    nact = cs_build_list(B, [&](int b) { int st = I[b].status; return st == ST_FRESH || st == ST_LS; },
                         [&](int b) { return cs_res_items(I[b], N[b]); }, bt.act, bt.act_pre, sh);
    if (threadIdx.x == 0) { bt.jac_pre[0] = 0; bt.acc_pre[0] = 0; }
  } else {
    nact = cs_build_list(B, [&](int b) { int st = I[b].status; return st == ST_FRESH || st == ST_LS || I[b].need_jac; },
                         [&](int b) { return cs_res_items(I[b], N[b]); }, bt.act, bt.act_pre, sh);
    njac = cs_build_list(B, [&](int b) { return I[b].need_jac != 0; }, [&](int b) { return (long long)(N[b] - 1); },
                         bt.jac, bt.jac_pre, sh);
    nacc = cs_build_list(B, [&](int b) { return I[b].accepted != 0; }, [&](int b) { return (long long)N[b]; },
                         bt.acc, bt.acc_pre, sh);
    const int* J = bt.jac;
    for (int l = 0; l < nlvl && l < CS_MAXLVL; ++l)
      cs_build_list(njac, [&](int k) { return true; }, [&](int k) { return cs_level_items(N[J[k]] - 1, l); },
                    (int*)nullptr, bt.lvl_pre + (size_t)l * (B + 1), sh);
  }
  if (threadIdx.x == 0) {
    bt.nlist[0] = nact;
    bt.nlist[1] = njac;
    bt.nlist[2] = nacc;
  }
}

// ------------------------------------------------------------------------
// Condensation: per interval, build [W | J | V_eff | f_a] in shared memory,
// partial-pivot LU (pivot: largest |entry|, first one wins, as
// matrix_factorization_cuda.py:133-146), back substitution, then
//   A = -I + D X_J, H = D X_V, b = -f_b - D X_f  with D = h b_j I on y rows,
// written as the level-0 block row [A | C=I | H | b]; X kept for recovery.
// Structure used by the condensation: Lobatto IIIA has A[0][:] = 0 (the first
// stage is the left node), so the stage-0 block row of W is
//   [ -I  h_z0 | 0 ... 0 ]
//   [  0  g_z0 | 0 ... 0 ]
// and W is block lower triangular with that block first.  The stage-0
// unknowns are solved directly (an NZ x NZ solve with g_z0), their coupling
// W10 (= h A[j][0] [h_y; g_y] of the later stages, y-columns only) is moved
// to the right-hand side, and partial-pivot LU runs on the remaining
// S1 = (M-1)(NY+NZ) rows only.  The reference factorises the whole W
// (collocation_solver_parallel_2d_shared.py:887-1001); the solution is the
// same up to rounding.
//
// Shared memory of one condensation group (doubles):
//   Wm    [S1][LDW1]               reduced augmented matrix [W11 | R1']
//   Jy    [M][NY+NZ][NY+NZ+NPE]    stage Jacobian rows [h_y h_z h_p ; g_y g_z g_p]
//   fa    [M][NY+NZ]               stage residuals
//   hA    [M][M]                   h * A
//   fb    [NY]                     f_b
//   X0    [NY+NZ][NRHS]            stage-0 rows of X = W^-1 [J V f_a]
//   inv   [S1]                     reciprocal pivots
//   red   [16]                     cross-warp pivot search (CTA groups)
#define CS_RB (CS_NY + CS_NZ)
#define CS_S1 ((CS_M - 1) * CS_RB)
#define CS_NCOL1 (CS_S1 + CS_NRHS)
#define CS_LDW1 (CS_NCOL1 | 1)
#define CS_JYC (CS_NY + CS_NZ + CS_NPE)
#define CS_GRP_RAW (CS_S1 * CS_LDW1 + CS_M * CS_RB * CS_JYC + CS_M * CS_RB + CS_M * CS_M + CS_NY + CS_RB * CS_NRHS + CS_S1 + 16)
// group stride padded to 8 (mod 16) doubles: the groups of one warp then
// start on alternate halves of the shared-memory banks
#define CS_GRP_DBL (((CS_GRP_RAW + 7) / 16) * 16 + 8)

// A group of GL threads condenses one interval: GL = 8 or 16 (sub-warp:
// several intervals per warp, so that the per-column work of the
// elimination -- pivot search, reciprocal -- serves several intervals per
// warp instruction), 32 (a warp) or 32*k (a CTA).
template <int GL>
struct CsGrp {
  static constexpr bool CTA = GL > 32;
  __device__ static __forceinline__ int tid() { return CTA ? (int)threadIdx.x : (int)(threadIdx.x & (GL - 1)); }
  __device__ static __forceinline__ void sync() {
    if (CTA) __syncthreads(); else __syncwarp();
  }
};

// |x| as an integer key: for non-negative doubles the order of the bit
// patterns is the order of the values, so the pivot search needs no FP64
// comparisons (the FP64 pipe is the bottleneck of this kernel).
__device__ __forceinline__ unsigned long long cs_abskey(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}

// right-hand-side column c of stage row (j, a): J, then V_eff, then f_a
__device__ __forceinline__ double cs_rhs(const double* J, const double* fa, int j, int a, int c) {
  if (c < CS_NY) return J[c];
  if (c < CS_NY + CS_NPE) return J[CS_NY + CS_NZ + (c - CS_NY)];
  return fa[j * CS_RB + a];
}

// `active` is false for a filler group of a partly used warp: it computes on a
// valid interval but writes nothing.
template <int GL>
__device__ void cs_condense_group(const CsBatch& bt, int slot, bool active, double* Wm, double* red) {
  typedef CsGrp<GL> G;
  constexpr int RB = CS_RB;
  const int tid = G::tid();
  double* Jy = Wm + CS_S1 * CS_LDW1;
  double* fa = Jy + CS_M * RB * CS_JYC;
  double* hA = fa + CS_M * RB;
  double* fb = hA + CS_M * CS_M;
  double* X0 = fb + CS_NY;
  double* inv = X0 + RB * CS_NRHS;
  const int b = bt.inst_of[slot];
  const double h = bt.t[slot + 1] - bt.t[slot];
  const double* th = bt.th + (size_t)b * (CS_NTH > 0 ? CS_NTH : 1);
  const double* yi = bt.y + (size_t)slot * CS_NY;
  const double* yd = bt.ydot + (size_t)slot * CS_M * CS_NY;
  // ---- stage Jacobians and residuals: thread j handles stage j
  for (int j = tid; j < CS_M; j += GL) {
    double pl[CS_NP > 0 ? CS_NP : 1];
    for (int k = 0; k < CS_NP; ++k) pl[k] = bt.p[(size_t)b * CS_NP + k];
    double yt[CS_NY], zl[CS_NZ > 0 ? CS_NZ : 1];
    for (int k = 0; k < CS_NY; ++k) {
      double s = 0.0;
      for (int q = 0; q < CS_M; ++q) s += CS_A[j * CS_M + q] * yd[q * CS_NY + k];
      yt[k] = yi[k] + h * s;
    }
    for (int k = 0; k < CS_NZ; ++k) zl[k] = bt.zt[((size_t)slot * CS_M + j) * CS_NZ + k];
    double f[CS_NY];
    double Df[CS_NY * CS_NFG];
    cs_f(yt, zl, pl, th, f);
    cs_Df(yt, zl, pl, th, Df);
    double* J = Jy + (size_t)j * RB * CS_JYC;
    for (int a = 0; a < CS_NY; ++a) {
      for (int q = 0; q < CS_NY + CS_NZ; ++q) J[a * CS_JYC + q] = Df[a * CS_NFG + q];
      for (int q = 0; q < CS_NPE; ++q) J[a * CS_JYC + CS_NY + CS_NZ + q] = Df[a * CS_NFG + CS_NY + CS_NZ + q];
      fa[j * RB + a] = f[a] - yd[j * CS_NY + a];
    }
#if CS_NZ > 0
    double g[CS_NZ];
    double Dg[CS_NZ * CS_NFG];
    cs_g(yt, zl, pl, th, bt.inst[b].alpha, g);
    cs_Dg(yt, zl, pl, th, bt.inst[b].alpha, Dg);
    for (int a = 0; a < CS_NZ; ++a) {
      for (int q = 0; q < CS_NY + CS_NZ; ++q) J[(CS_NY + a) * CS_JYC + q] = Dg[a * CS_NFG + q];
      for (int q = 0; q < CS_NPE; ++q) J[(CS_NY + a) * CS_JYC + CS_NY + CS_NZ + q] = Dg[a * CS_NFG + CS_NY + CS_NZ + q];
      fa[j * RB + CS_NY + a] = g[a];
    }
#endif
  }
  for (int e = tid; e < CS_M * CS_M; e += GL) hA[e] = h * CS_A[e];
  for (int k = tid; k < CS_NY; k += GL) {
    double s = 0.0;
    for (int j = 0; j < CS_M; ++j) s += CS_B[j] * yd[j * CS_NY + k];
    fb[k] = yi[CS_NY + k] - yi[k] - h * s;
  }
  G::sync();
  // ---- stage 0: [-I h_z0; 0 g_z0] X0 = R0, one thread per right-hand side
  for (int c = tid; c < CS_NRHS; c += GL) {
    const double* J0 = Jy;  // stage 0 rows
#if CS_NZ > 0
    double gz[CS_NZ][CS_NZ], xz[CS_NZ];
    for (int a = 0; a < CS_NZ; ++a) {
      for (int q = 0; q < CS_NZ; ++q) gz[a][q] = J0[(CS_NY + a) * CS_JYC + CS_NY + q];
      xz[a] = cs_rhs(J0 + (CS_NY + a) * CS_JYC, fa, 0, CS_NY + a, c);
    }
    // partial-pivot elimination on g_z0 (NZ x NZ)
    for (int kk = 0; kk < CS_NZ; ++kk) {
      int pr = kk;
      for (int r = kk + 1; r < CS_NZ; ++r)
        if (cs_abskey(gz[r][kk]) > cs_abskey(gz[pr][kk])) pr = r;
      if (pr != kk) {
        for (int q = 0; q < CS_NZ; ++q) { const double t = gz[kk][q]; gz[kk][q] = gz[pr][q]; gz[pr][q] = t; }
        const double t = xz[kk]; xz[kk] = xz[pr]; xz[pr] = t;
      }
      const double ip = 1.0 / gz[kk][kk];
      for (int r = kk + 1; r < CS_NZ; ++r) {
        const double l = gz[r][kk] * ip;
        for (int q = kk + 1; q < CS_NZ; ++q) gz[r][q] = fma(-l, gz[kk][q], gz[r][q]);
        xz[r] = fma(-l, xz[kk], xz[r]);
      }
    }
    for (int r = CS_NZ - 1; r >= 0; --r) {
      double v = xz[r];
      for (int q = r + 1; q < CS_NZ; ++q) v = fma(-gz[r][q], xz[q], v);
      xz[r] = v / gz[r][r];
    }
    for (int a = 0; a < CS_NZ; ++a) X0[(CS_NY + a) * CS_NRHS + c] = xz[a];
#endif
    // -x_y + h_z0 x_z = r_y  ->  x_y = h_z0 x_z - r_y
    for (int a = 0; a < CS_NY; ++a) {
      double v = -cs_rhs(J0 + a * CS_JYC, fa, 0, a, c);
#if CS_NZ > 0
      for (int q = 0; q < CS_NZ; ++q) v = fma(J0[a * CS_JYC + CS_NY + q], xz[q], v);
#endif
      X0[a * CS_NRHS + c] = v;
    }
  }
  G::sync();
  // ---- fill the reduced system [W11 | R1 - W10 X0] (stages 1..M-1)
  for (int e = tid; e < CS_S1 * CS_NCOL1; e += GL) {
    const int row = e / CS_NCOL1, col = e - row * CS_NCOL1;
    const int j = 1 + row / RB, a = row - (j - 1) * RB;
    const double* J = Jy + (size_t)(j * RB + a) * CS_JYC;
    double v;
    if (col < CS_S1) {
      const int k = 1 + col / RB, q = col - (k - 1) * RB;
      if (q < CS_NY) {
        v = hA[j * CS_M + k] * J[q];
        if (k == j && q == a) v -= 1.0;
      } else {
        v = (k == j) ? J[q] : 0.0;
      }
    } else {
      const int c = col - CS_S1;
      double w = 0.0;
      for (int q = 0; q < CS_NY; ++q) w = fma(J[q], X0[q * CS_NRHS + c], w);
      v = fma(-hA[j * CS_M], w, cs_rhs(J, fa, j, a, c));
    }
    Wm[row * CS_LDW1 + col] = v;
  }
  G::sync();
  // ---- LU with partial pivoting: largest |entry| in the column, the first
  //      such row on ties (as matrix_factorization_cuda.py:133-146)
  int singular = 0;
#pragma unroll 1
  for (int k = 0; k < CS_S1; ++k) {
    unsigned long long best = 0ull;
    int brow = CS_S1;  // larger than any row: loses every tie
    for (int r = k + tid; r < CS_S1; r += GL) {
      const unsigned long long v = cs_abskey(Wm[r * CS_LDW1 + k]);
      if (v > best || brow == CS_S1) { best = v; brow = r; }
    }
    constexpr int W = CsGrp<GL>::CTA ? 32 : GL;
    for (int o = W >> 1; o > 0; o >>= 1) {
      const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o, W);
      const int orow = __shfl_xor_sync(0xffffffffu, brow, o, W);
      if (ob > best || (ob == best && orow < brow)) { best = ob; brow = orow; }
    }
    if (CsGrp<GL>::CTA) {
      constexpr int NW = GL / 32;
      if ((tid & 31) == 0) {
        red[tid >> 5] = __longlong_as_double((long long)best);
        red[NW + (tid >> 5)] = (double)brow;
      }
      __syncthreads();
      best = (unsigned long long)__double_as_longlong(red[0]);
      brow = (int)red[NW];
      for (int w = 1; w < NW; ++w) {
        const unsigned long long ob = (unsigned long long)__double_as_longlong(red[w]);
        const int orow = (int)red[NW + w];
        if (ob > best || (ob == best && orow < brow)) { best = ob; brow = orow; }
      }
      __syncthreads();
    }
    // swap rows k and brow (a self-swap when the pivot is in place)
    for (int c = tid; c < CS_NCOL1; c += GL) {
      const double tmp = Wm[k * CS_LDW1 + c];
      Wm[k * CS_LDW1 + c] = Wm[brow * CS_LDW1 + c];
      Wm[brow * CS_LDW1 + c] = tmp;
    }
    G::sync();
    const double pv = Wm[k * CS_LDW1 + k];
    // |pv| < 10 eps: the reference leaves this column uneliminated
    const bool tiny = cs_abskey(pv) < 0x3ce4000000000000ull;  // bits of 10 * 2^-52 = 2.22e-15
    singular |= tiny;
    const double ip = 1.0 / pv;
    if (tid == 0) inv[k] = ip;
    const double mul = tiny ? 0.0 : ip;
    for (int r = k + 1 + tid; r < CS_S1; r += GL) Wm[r * CS_LDW1 + k] *= mul;
    G::sync();
    const int nc = CS_NCOL1 - k - 1;
    const int ne = (CS_S1 - k - 1) * nc;
    for (int e = tid; e < ne; e += GL) {
      const int rr = e / nc;
      const int r = k + 1 + rr, c = k + 1 + (e - rr * nc);
      Wm[r * CS_LDW1 + c] = fma(-Wm[r * CS_LDW1 + k], Wm[k * CS_LDW1 + c], Wm[r * CS_LDW1 + c]);
    }
    G::sync();
  }
  // ---- back substitution, threads over (row, right-hand side) pairs
#pragma unroll 1
  for (int r = CS_S1 - 1; r >= 0; --r) {
    for (int c = tid; c < CS_NRHS; c += GL) Wm[r * CS_LDW1 + CS_S1 + c] *= inv[r];
    G::sync();
    const int ne = r * CS_NRHS;
    for (int e = tid; e < ne; e += GL) {
      const int q = e / CS_NRHS, c = e - q * CS_NRHS;
      Wm[q * CS_LDW1 + CS_S1 + c] = fma(-Wm[q * CS_LDW1 + r], Wm[r * CS_LDW1 + CS_S1 + c], Wm[q * CS_LDW1 + CS_S1 + c]);
    }
    G::sync();
  }
  if (!active) return;
  // ---- X (column-major [NRHS][S]: stage-0 rows from X0, the others from Wm)
  double* X = bt.X + (size_t)slot * CS_NRHS * CS_S;
  for (int e = tid; e < CS_NRHS * CS_S; e += GL) {
    const int c = e / CS_S, r = e - c * CS_S;
    X[e] = (r < RB) ? X0[r * CS_NRHS + c] : Wm[(r - RB) * CS_LDW1 + CS_S1 + c];
  }
  // ---- condensed block row: D X = h sum_j b_j X[(j, a)]
  double* row = bt.rows0 + (size_t)slot * CS_ROWSZ;
  for (int e = tid; e < CS_NRHS * CS_NY; e += GL) {
    const int c = e / CS_NY, a = e - c * CS_NY;
    double s = CS_B[0] * X0[a * CS_NRHS + c];
    for (int j = 1; j < CS_M; ++j) s += CS_B[j] * Wm[((j - 1) * RB + a) * CS_LDW1 + CS_S1 + c];
    const double dx = h * s;
    if (c < CS_NY) {
      row[c * CS_NY + a] = (a == c) ? dx - 1.0 : dx;            // A column c
      row[(CS_NY + c) * CS_NY + a] = (a == c ? 1.0 : 0.0);      // C = I column c
    } else if (c < CS_NY + CS_NPE) {
      row[(2 * CS_NY + (c - CS_NY)) * CS_NY + a] = dx;          // H
    } else {
      row[(2 * CS_NY + CS_NPE) * CS_NY + a] = -fb[a] - dx;      // b
    }
  }
  if (singular && tid == 0) atomicAdd(&bt.inst[b].singular, 1);
}

#if !CS_BIG_COND
// lanes per condensation group, from the size of the stage system
#define CS_CGL ((CS_S1 > 48) ? 256 : ((CS_S1 > 16) ? 16 : 8))

template <int GL>
__device__ __forceinline__ void cs_condense_entry(const CsBatch& bt) {
  extern __shared__ double smem[];
  const int njac = bt.nlist[1];
  const long long total = bt.jac_pre[njac];
  if (total == 0) return;
  if (GL <= 32) {
    constexpr int GPW = 32 / GL;                  // groups per warp
    const int wpc = blockDim.x >> 5;
    const int w = threadIdx.x >> 5;
    const int gi = (threadIdx.x & 31) / GL;       // group within the warp
    double* Wm = smem + (size_t)(w * GPW + gi) * CS_GRP_DBL;
    for (long long base = ((long long)blockIdx.x * wpc + w) * GPW; base < total;
         base += (long long)gridDim.x * wpc * GPW) {
      long long it = base + gi;
      const bool active = it < total;
      if (!active) it = total - 1;
      const int k = cs_find(bt.jac_pre, njac, it);
      const int b = bt.jac[k];
      const int slot = bt.off[b] + (int)(it - bt.jac_pre[k]);
      cs_condense_group<GL>(bt, slot, active, Wm, nullptr);
      __syncwarp();
    }
  } else {
    double* red = smem + CS_GRP_RAW - 16;
    for (long long it = blockIdx.x; it < total; it += gridDim.x) {
      const int k = cs_find(bt.jac_pre, njac, it);
      const int b = bt.jac[k];
      const int slot = bt.off[b] + (int)(it - bt.jac_pre[k]);
      cs_condense_group<GL>(bt, slot, true, smem, red);
      __syncthreads();
    }
  }
}

extern "C" __global__ void k_condense(CsBatch bt) { cs_condense_entry<CS_CGL>(bt); }
#if CS_S1 <= 48
// the tuner's candidates: 4, 8, 16 or 32 lanes per interval (fewer lanes:
// more intervals share each warp instruction of the elimination, whose
// short loops leave fewer lanes idle)
extern "C" __global__ void k_condense_l4(CsBatch bt) { cs_condense_entry<4>(bt); }
extern "C" __global__ void k_condense_l8(CsBatch bt) { cs_condense_entry<8>(bt); }
extern "C" __global__ void k_condense_l16(CsBatch bt) { cs_condense_entry<16>(bt); }
extern "C" __global__ void k_condense_l32(CsBatch bt) { cs_condense_entry<32>(bt); }
#endif
#endif  // !CS_BIG_COND

// ------------------------------------------------------------------------
// BABD solve, one CTA per instance: tree of pairwise QR eliminations over
// the block rows (row k couples y_left, y_right), the dense top system with
// the boundary conditions, back substitution down the tree, recovery of the
// stage steps.
//
// Merge of rows a (y_l, y_m) and b (y_m, y_r):
//   [C_a; A_b] = Q [R; 0];  Q^T [A_a | 0 ; 0 | C_b ; H_a H_b ; b_a b_b]
//   top rows    -> tree record at node m: R y_m + G y_l + E y_r + J p = d
//   bottom rows -> new row:  At y_l + Ct y_r + Ht p = bt
// Householder sign rule as matrix_factorization_cuda.py:37-54.

// column-major merge matrix Q[col * CS_QLD + row], rows 0..2NY-1
__device__ void cs_merge_warp(const double* ra, const double* rb, double* out_row, double* rec, double* Q) {
  const int lane = threadIdx.x & 31;
  // load: col 0..NY-1: [C_a; A_b]; NY..2NY-1: [A_a; 0]; 2NY..3NY-1: [0; C_b]; H; b
  for (int c = lane; c < CS_QC; c += 32) {
    double* col = Q + (size_t)c * CS_QLD;
    for (int r = 0; r < CS_NY; ++r) {
      double top, bot;
      if (c < CS_NY) { top = ra[(CS_NY + c) * CS_NY + r]; bot = rb[c * CS_NY + r]; }
      else if (c < 2 * CS_NY) { top = ra[(c - CS_NY) * CS_NY + r]; bot = 0.0; }
      else if (c < 3 * CS_NY) { top = 0.0; bot = rb[(CS_NY + c - 2 * CS_NY) * CS_NY + r]; }
      else if (c < 3 * CS_NY + CS_NPE) { top = ra[(2 * CS_NY + c - 3 * CS_NY) * CS_NY + r]; bot = rb[(2 * CS_NY + c - 3 * CS_NY) * CS_NY + r]; }
      else { top = ra[(2 * CS_NY + CS_NPE) * CS_NY + r]; bot = rb[(2 * CS_NY + CS_NPE) * CS_NY + r]; }
      col[r] = top;
      col[CS_NY + r] = bot;
    }
  }
  __syncwarp();
#pragma unroll 1
  for (int k = 0; k < CS_NY; ++k) {
    const double* vk = Q + (size_t)k * CS_QLD;
    double ss = 0.0;
    for (int r = k + lane; r < 2 * CS_NY; r += 32) ss += vk[r] * vk[r];
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
    const double x0 = vk[k];
    const double sgn = (x0 >= 0.0) ? 1.0 : -1.0;
    const double g = -sgn * sqrt(ss);
    const double v0 = x0 - g;
    const double vs = ss - x0 * x0 + v0 * v0;
    __syncwarp();
    if (vs < CS_EPS) continue;  // nothing to eliminate in this column
    const double beta = -2.0 / vs;
    for (int c = k + 1 + lane; c < CS_QC; c += 32) {
      double* col = Q + (size_t)c * CS_QLD;
      double w = v0 * col[k];
      for (int r = k + 1; r < 2 * CS_NY; ++r) w += vk[r] * col[r];
      const double bw = beta * w;
      col[k] = fma(bw, v0, col[k]);
      for (int r = k + 1; r < 2 * CS_NY; ++r) col[r] = fma(bw, vk[r], col[r]);
    }
    __syncwarp();
    if (lane == 0) {
      double* col = Q + (size_t)k * CS_QLD;
      col[k] = g;
      for (int r = k + 1; r < 2 * CS_NY; ++r) col[r] = 0.0;
    }
    __syncwarp();
  }
  // outputs
  for (int c = lane; c < CS_QC; c += 32) {
    const double* col = Q + (size_t)c * CS_QLD;
    for (int r = 0; r < CS_NY; ++r) rec[(size_t)c * CS_NY + r] = col[r];
    if (c >= CS_NY) {
      // new row: At (from A_a cols), Ct (from C_b cols), Ht, bt
      for (int r = 0; r < CS_NY; ++r) out_row[(size_t)(c - CS_NY) * CS_NY + r] = col[CS_NY + r];
    }
  }
  __syncwarp();
}

// Small blocks (2 NY x QC doubles fit in registers): one thread per merge,
// fully unrolled, the same Householder steps as cs_merge_warp.
#define CS_TREE_THREAD (2 * CS_NY * CS_QC <= 128)
#if CS_TREE_THREAD
__device__ __forceinline__ void cs_merge_thread(const double* __restrict__ ra, const double* __restrict__ rb,
                                                double* __restrict__ out_row, double* __restrict__ rec) {
  double Q[CS_QC][2 * CS_NY];
#pragma unroll
  for (int c = 0; c < CS_QC; ++c)
#pragma unroll
    for (int r = 0; r < CS_NY; ++r) {
      double top, bot;
      if (c < CS_NY) { top = ra[(CS_NY + c) * CS_NY + r]; bot = rb[c * CS_NY + r]; }
      else if (c < 2 * CS_NY) { top = ra[(c - CS_NY) * CS_NY + r]; bot = 0.0; }
      else if (c < 3 * CS_NY) { top = 0.0; bot = rb[(CS_NY + c - 2 * CS_NY) * CS_NY + r]; }
      else if (c < 3 * CS_NY + CS_NPE) { top = ra[(2 * CS_NY + c - 3 * CS_NY) * CS_NY + r]; bot = rb[(2 * CS_NY + c - 3 * CS_NY) * CS_NY + r]; }
      else { top = ra[(2 * CS_NY + CS_NPE) * CS_NY + r]; bot = rb[(2 * CS_NY + CS_NPE) * CS_NY + r]; }
      Q[c][r] = top;
      Q[c][CS_NY + r] = bot;
    }
#pragma unroll
  for (int k = 0; k < CS_NY; ++k) {
    double ss = 0.0;
#pragma unroll
    for (int r = k; r < 2 * CS_NY; ++r) ss = fma(Q[k][r], Q[k][r], ss);
    const double x0 = Q[k][k];
    const double g = (x0 >= 0.0) ? -sqrt(ss) : sqrt(ss);
    const double v0 = x0 - g;
    const double vs = ss - x0 * x0 + v0 * v0;
    if (vs >= CS_EPS) {
      const double beta = -2.0 / vs;
#pragma unroll
      for (int c = k + 1; c < CS_QC; ++c) {
        double w = v0 * Q[c][k];
#pragma unroll
        for (int r = k + 1; r < 2 * CS_NY; ++r) w = fma(Q[k][r], Q[c][r], w);
        const double bw = beta * w;
        Q[c][k] = fma(bw, v0, Q[c][k]);
#pragma unroll
        for (int r = k + 1; r < 2 * CS_NY; ++r) Q[c][r] = fma(bw, Q[k][r], Q[c][r]);
      }
      Q[k][k] = g;
#pragma unroll
      for (int r = k + 1; r < 2 * CS_NY; ++r) Q[k][r] = 0.0;
    }
  }
#pragma unroll
  for (int c = 0; c < CS_QC; ++c) {
#pragma unroll
    for (int r = 0; r < CS_NY; ++r) rec[c * CS_NY + r] = Q[c][r];
    if (c >= CS_NY) {
#pragma unroll
      for (int r = 0; r < CS_NY; ++r) out_row[(c - CS_NY) * CS_NY + r] = Q[c][CS_NY + r];
    }
  }
}

__device__ __forceinline__ void cs_backsub_thread(const double* __restrict__ rec, const double* __restrict__ yl,
                                                  const double* __restrict__ yr, const double* __restrict__ dpv,
                                                  double* __restrict__ ym) {
  double v[CS_NY];
#pragma unroll
  for (int a = 0; a < CS_NY; ++a) {
    double s = rec[(3 * CS_NY + CS_NPE) * CS_NY + a];
#pragma unroll
    for (int c = 0; c < CS_NY; ++c) s -= rec[(CS_NY + c) * CS_NY + a] * yl[c];
#pragma unroll
    for (int c = 0; c < CS_NY; ++c) s -= rec[(2 * CS_NY + c) * CS_NY + a] * yr[c];
#pragma unroll
    for (int c = 0; c < CS_NPE; ++c) s -= rec[(3 * CS_NY + c) * CS_NY + a] * dpv[c];
    v[a] = s;
  }
#pragma unroll
  for (int r = CS_NY - 1; r >= 0; --r) {
    const double rr = rec[r * CS_NY + r];
    const double xr = (rr != 0.0) ? v[r] / rr : 0.0;
    v[r] = xr;
#pragma unroll
    for (int a = 0; a < r; ++a) v[a] -= rec[r * CS_NY + a] * xr;
  }
#pragma unroll
  for (int a = 0; a < CS_NY; ++a) ym[a] = v[a];
}
#endif

#if CS_TREE_THREAD && CS_QC <= 32
// The same merge with a column per lane (CS_TL lanes per merge, column in
// registers): the pivot lane forms the reflector, shuffles hand it to the
// other lanes, each lane updates its own column.  Every column sees the fma
// sequence of cs_merge_thread, so the results are the same bits; the chain of
// FP64 instructions per lane is ~4x shorter, which is what a level with few
// merges waits for (on this GPU a dependent FP64 instruction waits ~64 cycles,
// and the SM's FP64 unit takes one warp instruction per ~19 cycles whatever
// the number of active lanes).
#define CS_TL ((CS_QC <= 16) ? 16 : 32)
__device__ __forceinline__ void cs_merge_lanes(const double* __restrict__ ra, const double* __restrict__ rb,
                                               double* __restrict__ out_row, double* __restrict__ rec, bool active) {
  const int c = threadIdx.x & (CS_TL - 1);
  // the group's own lanes: two groups of a warp may take different branches
  const unsigned gm = (CS_TL == 32) ? 0xffffffffu : (0xffffu << (threadIdx.x & 16));
  double Q[2 * CS_NY];
#pragma unroll
  for (int r = 0; r < CS_NY; ++r) {
    double top = 0.0, bot = 0.0;
    if (c < CS_NY) { top = ra[(CS_NY + c) * CS_NY + r]; bot = rb[c * CS_NY + r]; }
    else if (c < 2 * CS_NY) { top = ra[(c - CS_NY) * CS_NY + r]; }
    else if (c < 3 * CS_NY) { bot = rb[(CS_NY + c - 2 * CS_NY) * CS_NY + r]; }
    else if (c < 3 * CS_NY + CS_NPE) { top = ra[(2 * CS_NY + c - 3 * CS_NY) * CS_NY + r]; bot = rb[(2 * CS_NY + c - 3 * CS_NY) * CS_NY + r]; }
    else if (c < CS_QC) { top = ra[(2 * CS_NY + CS_NPE) * CS_NY + r]; bot = rb[(2 * CS_NY + CS_NPE) * CS_NY + r]; }
    Q[r] = top;
    Q[CS_NY + r] = bot;
  }
#pragma unroll
  for (int k = 0; k < CS_NY; ++k) {
    // pivot lane k: the reflector of column k
    double ss = 0.0;
#pragma unroll
    for (int r = k; r < 2 * CS_NY; ++r) ss = fma(Q[r], Q[r], ss);
    const double x0 = Q[k];
    const double gk = (x0 >= 0.0) ? -sqrt(ss) : sqrt(ss);
    const double v0k = x0 - gk;
    const double vsk = ss - x0 * x0 + v0k * v0k;
    const double v0 = __shfl_sync(gm, v0k, k, CS_TL);
    const double vs = __shfl_sync(gm, vsk, k, CS_TL);
    double v[2 * CS_NY];
#pragma unroll
    for (int r = k + 1; r < 2 * CS_NY; ++r) v[r] = __shfl_sync(gm, Q[r], k, CS_TL);
    if (vs >= CS_EPS) {
      if (c > k) {
        const double beta = -2.0 / vs;
        double w = v0 * Q[k];
#pragma unroll
        for (int r = k + 1; r < 2 * CS_NY; ++r) w = fma(v[r], Q[r], w);
        const double bw = beta * w;
        Q[k] = fma(bw, v0, Q[k]);
#pragma unroll
        for (int r = k + 1; r < 2 * CS_NY; ++r) Q[r] = fma(bw, v[r], Q[r]);
      } else if (c == k) {
        Q[k] = gk;
#pragma unroll
        for (int r = k + 1; r < 2 * CS_NY; ++r) Q[r] = 0.0;
      }
    }
  }
  if (!active || c >= CS_QC) return;
#pragma unroll
  for (int r = 0; r < CS_NY; ++r) rec[c * CS_NY + r] = Q[r];
  if (c >= CS_NY) {
#pragma unroll
    for (int r = 0; r < CS_NY; ++r) out_row[(c - CS_NY) * CS_NY + r] = Q[CS_NY + r];
  }
}
#endif

// y_m = R^-1 (d - G y_l - E y_r - J p), one warp, lanes over rows
__device__ void cs_backsub_warp(const double* rec, const double* yl, const double* yr, const double* dpv, double* ym) {
  const int lane = threadIdx.x & 31;
  double rhs[(CS_NY + 31) / 32];
  for (int q = 0; q < (CS_NY + 31) / 32; ++q) {
    int a = lane + 32 * q;
    double v = 0.0;
    if (a < CS_NY) {
      v = rec[(size_t)(3 * CS_NY + CS_NPE) * CS_NY + a];
      for (int c = 0; c < CS_NY; ++c) v -= rec[(size_t)(CS_NY + c) * CS_NY + a] * yl[c];
      for (int c = 0; c < CS_NY; ++c) v -= rec[(size_t)(2 * CS_NY + c) * CS_NY + a] * yr[c];
      for (int c = 0; c < CS_NPE; ++c) v -= rec[(size_t)(3 * CS_NY + c) * CS_NY + a] * dpv[c];
    }
    rhs[q] = v;
  }
  for (int r = CS_NY - 1; r >= 0; --r) {
    const int owner = r & 31, qq = r >> 5;
    double xr = 0.0;
    for (int q = 0; q < (CS_NY + 31) / 32; ++q)
      if (q == qq) xr = __shfl_sync(0xffffffffu, rhs[q], owner);
    const double rr = rec[(size_t)r * CS_NY + r];
    xr = (rr != 0.0) ? xr / rr : 0.0;
    if (lane == owner) {
      for (int q = 0; q < (CS_NY + 31) / 32; ++q)
        if (q == qq) rhs[q] = xr;
      ym[r] = xr;
    }
    for (int q = 0; q < (CS_NY + 31) / 32; ++q) {
      int a = lane + 32 * q;
      if (a < r) rhs[q] -= rec[(size_t)r * CS_NY + a] * xr;
    }
  }
  __syncwarp();
}

#if !CS_BIG_TREE
// One tree level for every instance that needs a Newton direction: warp per
// item; item mi < merges eliminates node (2 mi + 1) 2^l between rows 2 mi and
// 2 mi + 1, the last item of an odd level carries its row up unchanged.
extern "C" __global__ void k_tree_level(CsBatch bt, int l) {
#if CS_TREE_THREAD
  {
    const int njac = bt.nlist[1];
    const long long* pre = bt.lvl_pre + (size_t)l * (bt.B + 1);
    const long long total = pre[njac];
    const double* srcb = (l & 1) ? bt.rows1 : bt.rows0;
    double* dstb = (l & 1) ? bt.rows0 : bt.rows1;
#if CS_QC <= 32
    // few merges (at most 4 rounds of lane groups over the grid): CS_TL lanes
    // per merge; the grid is one wave of resident CTAs
    const long long lanes = total * CS_TL, stride = (long long)gridDim.x * blockDim.x;
    if (lanes <= 4 * stride) {
      for (long long base = (long long)blockIdx.x * blockDim.x; base < lanes; base += stride) {
        if (base + (threadIdx.x & ~31) >= lanes) break;  // warp-uniform, and so for later rounds
        const long long it0 = (base + threadIdx.x) / CS_TL;
        const bool active = it0 < total;
        const long long it = active ? it0 : total - 1;
        const int k = cs_find(pre, njac, it);
        const int b = bt.jac[k];
        const int mi = (int)(it - pre[k]);
        const int off = bt.off[b];
        const int nl = cs_rows_at(bt.N[b] - 1, l);
        const int merges = nl >> 1;
        const double* src = srcb + (size_t)off * CS_ROWSZ;
        double* dst = dstb + (size_t)off * CS_ROWSZ;
        if (mi < merges) {  // uniform within the lane group
          cs_merge_lanes(src + (size_t)(2 * mi) * CS_ROWSZ, src + (size_t)(2 * mi + 1) * CS_ROWSZ,
                         dst + (size_t)mi * CS_ROWSZ, bt.tree + (size_t)(off + ((2 * mi + 1) << l)) * CS_TREESZ,
                         active);
        } else if (active) {
          const double* sr = src + (size_t)(nl - 1) * CS_ROWSZ;
          double* dr = dst + (size_t)merges * CS_ROWSZ;
          for (int q = threadIdx.x & (CS_TL - 1); q < CS_ROWSZ; q += CS_TL) dr[q] = sr[q];
        }
      }
      return;
    }
#endif
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total; it += (long long)gridDim.x * blockDim.x) {
      const int k = cs_find(pre, njac, it);
      const int b = bt.jac[k];
      const int mi = (int)(it - pre[k]);
      const int off = bt.off[b];
      const int nl = cs_rows_at(bt.N[b] - 1, l);
      const int merges = nl >> 1;
      const double* src = srcb + (size_t)off * CS_ROWSZ;
      double* dst = dstb + (size_t)off * CS_ROWSZ;
      if (mi < merges) {
        cs_merge_thread(src + (size_t)(2 * mi) * CS_ROWSZ, src + (size_t)(2 * mi + 1) * CS_ROWSZ,
                        dst + (size_t)mi * CS_ROWSZ, bt.tree + (size_t)(off + ((2 * mi + 1) << l)) * CS_TREESZ);
      } else {
        const double* sr = src + (size_t)(nl - 1) * CS_ROWSZ;
        double* dr = dst + (size_t)merges * CS_ROWSZ;
        for (int q = 0; q < CS_ROWSZ; ++q) dr[q] = sr[q];
      }
    }
    return;
  }
#endif
  extern __shared__ double smem[];
  const int wpc = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* Qw = smem + (size_t)w * CS_QLD * CS_QC;
  const int njac = bt.nlist[1];
  const long long* pre = bt.lvl_pre + (size_t)l * (bt.B + 1);
  const long long total = pre[njac];
  double* srcb = (l & 1) ? bt.rows1 : bt.rows0;
  double* dstb = (l & 1) ? bt.rows0 : bt.rows1;
  for (long long it = (long long)blockIdx.x * wpc + w; it < total; it += (long long)gridDim.x * wpc) {
    const int k = cs_find(pre, njac, it);
    const int b = bt.jac[k];
    const int mi = (int)(it - pre[k]);
    const int off = bt.off[b];
    const int nl = cs_rows_at(bt.N[b] - 1, l);
    const int merges = nl >> 1;
    const double* src = srcb + (size_t)off * CS_ROWSZ;
    double* dst = dstb + (size_t)off * CS_ROWSZ;
    if (mi < merges) {
      const int mid = (2 * mi + 1) << l;
      cs_merge_warp(src + (size_t)(2 * mi) * CS_ROWSZ, src + (size_t)(2 * mi + 1) * CS_ROWSZ,
                    dst + (size_t)mi * CS_ROWSZ, bt.tree + (size_t)(off + mid) * CS_TREESZ, Qw);
    } else {
      const double* sr = src + (size_t)(nl - 1) * CS_ROWSZ;
      double* dr = dst + (size_t)merges * CS_ROWSZ;
      for (int q = lane; q < CS_ROWSZ; q += 32) dr[q] = sr[q];
    }
    __syncwarp();
  }
}

// Top of the tree, warp per instance: the remaining block row with the
// boundary conditions, [At Ct Ht 0; B_0 B_n V_n] [y_0; y_N; p] = [bt; -r],
// by Householder QR (the reference: final block QR + np.linalg.solve,
// solve_babd_system.py:366-423).  Sets the line search going (alpha = 1).
// top system of instance b, one warp (top: per-warp shared memory)
__device__ void cs_top_warp(const CsBatch& bt, int b, double* top) {
  const int lane = threadIdx.x & 31;
  const int N = bt.N[b], off = bt.off[b];
  const int L = cs_levels(N - 1);
  const double* row = ((L & 1) ? bt.rows1 : bt.rows0) + (size_t)off * CS_ROWSZ;
  for (int c = lane; c < CS_NT + 1; c += 32) {
    double* col = top + (size_t)c * CS_TLD;
    for (int r = 0; r < CS_NY; ++r) {
      double v;
      if (c < 2 * CS_NY + CS_NPE) v = row[c * CS_NY + r];
      else if (c < CS_NT) v = 0.0;
      else v = row[(2 * CS_NY + CS_NPE) * CS_NY + r];
      col[r] = v;
    }
  }
  if (lane == 0) {
    const double* th = bt.th + (size_t)b * (CS_NTH > 0 ? CS_NTH : 1);
    double ya[CS_NY], yb[CS_NY], pl[CS_NP > 0 ? CS_NP : 1], r[CS_NY + CS_NP];
    double Dr[(CS_NY + CS_NP) * (2 * CS_NY + CS_NP)];
    for (int q = 0; q < CS_NY; ++q) { ya[q] = bt.y[(size_t)off * CS_NY + q]; yb[q] = bt.y[(size_t)(off + N - 1) * CS_NY + q]; }
    for (int q = 0; q < CS_NP; ++q) pl[q] = bt.p[(size_t)b * CS_NP + q];
    cs_r(ya, yb, pl, th, r);
    cs_Dr(ya, yb, pl, th, Dr);
    for (int q = 0; q < CS_NY + CS_NP; ++q) {
      for (int c = 0; c < CS_NY; ++c) top[(size_t)c * CS_TLD + CS_NY + q] = Dr[q * (2 * CS_NY + CS_NP) + c];
      for (int c = 0; c < CS_NY; ++c) top[(size_t)(CS_NY + c) * CS_TLD + CS_NY + q] = Dr[q * (2 * CS_NY + CS_NP) + CS_NY + c];
      for (int c = 0; c < CS_NP; ++c) top[(size_t)(2 * CS_NY + c) * CS_TLD + CS_NY + q] = Dr[q * (2 * CS_NY + CS_NP) + 2 * CS_NY + c];
      top[(size_t)CS_NT * CS_TLD + CS_NY + q] = -r[q];
    }
  }
  __syncwarp();
#pragma unroll 1
  for (int kk = 0; kk < CS_NT; ++kk) {
    const double* vk = top + (size_t)kk * CS_TLD;
    double ss = 0.0;
    for (int r = kk + lane; r < CS_NT; r += 32) ss += vk[r] * vk[r];
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
    const double x0 = vk[kk];
    const double sgn = (x0 >= 0.0) ? 1.0 : -1.0;
    const double g = -sgn * sqrt(ss);
    const double v0 = x0 - g;
    const double vs = ss - x0 * x0 + v0 * v0;
    __syncwarp();
    if (vs < CS_EPS) continue;
    const double beta = -2.0 / vs;
    for (int c = kk + 1 + lane; c < CS_NT + 1; c += 32) {
      double* col = top + (size_t)c * CS_TLD;
      double wv = v0 * col[kk];
      for (int r = kk + 1; r < CS_NT; ++r) wv += vk[r] * col[r];
      const double bw = beta * wv;
      col[kk] = fma(bw, v0, col[kk]);
      for (int r = kk + 1; r < CS_NT; ++r) col[r] = fma(bw, vk[r], col[r]);
    }
    __syncwarp();
    if (lane == 0) {
      double* col = top + (size_t)kk * CS_TLD;
      col[kk] = g;
      for (int r = kk + 1; r < CS_NT; ++r) col[r] = 0.0;
    }
    __syncwarp();
  }
  if (lane == 0) {
    double* rhs = top + (size_t)CS_NT * CS_TLD;
    bool sing = false;
    for (int r = CS_NT - 1; r >= 0; --r) {
      double v = rhs[r];
      for (int c = r + 1; c < CS_NT; ++c) v -= top[(size_t)c * CS_TLD + r] * rhs[c];
      const double d = top[(size_t)r * CS_TLD + r];
      if (d == 0.0) sing = true;
      rhs[r] = (d != 0.0) ? v / d : 0.0;
    }
    if (sing) {
      for (int r = 0; r < CS_NT; ++r) rhs[r] = 0.0;
      bt.inst[b].singular += 1;
    }
    for (int q = 0; q < CS_NY; ++q) {
      bt.dy[(size_t)off * CS_NY + q] = rhs[q];
      bt.dy[(size_t)(off + N - 1) * CS_NY + q] = rhs[CS_NY + q];
    }
    for (int q = 0; q < CS_NP; ++q) bt.dp[(size_t)b * CS_NP + q] = rhs[2 * CS_NY + q];
    bt.inst[b].status = ST_LS;
    bt.inst[b].alpha_ls = 1.0;
    bt.inst[b].ls_it = 0;
  }
  __syncwarp();
}

extern "C" __global__ void k_top(CsBatch bt) {
  extern __shared__ double smem[];
  const int wpc = blockDim.x >> 5, w = threadIdx.x >> 5;
  double* top = smem + (size_t)w * CS_TLD * (CS_NT + 1);
  const int njac = bt.nlist[1];
  for (int k = blockIdx.x * wpc + w; k < njac; k += gridDim.x * wpc) cs_top_warp(bt, bt.jac[k], top);
}
#endif  // !CS_BIG_TREE

// Back substitution of one tree level (top-down), warp per merge.
extern "C" __global__ void k_backsub_level(CsBatch bt, int l) {
#if CS_TREE_THREAD
  {
    const int njac = bt.nlist[1];
    const long long* pre = bt.lvl_pre + (size_t)l * (bt.B + 1);
    const long long total = pre[njac];
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < total; it += (long long)gridDim.x * blockDim.x) {
      const int k = cs_find(pre, njac, it);
      const int b = bt.jac[k];
      const int mi = (int)(it - pre[k]);
      const int n0 = bt.N[b] - 1;
      const int merges = cs_rows_at(n0, l) >> 1;
      if (mi >= merges) continue;
      const int off = bt.off[b];
      const int mid = (2 * mi + 1) << l;
      const int left = (2 * mi) << l;
      int right = (2 * mi + 2) << l;
      if (right > n0) right = n0;
      cs_backsub_thread(bt.tree + (size_t)(off + mid) * CS_TREESZ, bt.dy + (size_t)(off + left) * CS_NY,
                        bt.dy + (size_t)(off + right) * CS_NY, bt.dp + (size_t)b * CS_NP, bt.dy + (size_t)(off + mid) * CS_NY);
    }
    return;
  }
#endif
  const int wpc = blockDim.x >> 5, w = threadIdx.x >> 5;
  const int njac = bt.nlist[1];
  const long long* pre = bt.lvl_pre + (size_t)l * (bt.B + 1);
  const long long total = pre[njac];
  for (long long it = (long long)blockIdx.x * wpc + w; it < total; it += (long long)gridDim.x * wpc) {
    const int k = cs_find(pre, njac, it);
    const int b = bt.jac[k];
    const int mi = (int)(it - pre[k]);
    const int n0 = bt.N[b] - 1;
    const int merges = cs_rows_at(n0, l) >> 1;
    if (mi >= merges) continue;
    const int off = bt.off[b];
    const int mid = (2 * mi + 1) << l;
    const int left = (2 * mi) << l;
    int right = (2 * mi + 2) << l;
    if (right > n0) right = n0;
    cs_backsub_warp(bt.tree + (size_t)(off + mid) * CS_TREESZ, bt.dy + (size_t)(off + left) * CS_NY,
                    bt.dy + (size_t)(off + right) * CS_NY, bt.dp + (size_t)b * CS_NP, bt.dy + (size_t)(off + mid) * CS_NY);
  }
}

#if !CS_BIG_TREE && CS_TREE_THREAD && CS_QC <= 32
// The upper tree levels l >= l_lo of every instance on the jac list, its top
// system and the back substitution of those levels, one CTA per instance:
// levels with at most a few merges each, which as launches of their own cost
// a launch and a work-list lookup apiece for a few dependent merges.  Merges
// by groups of CS_TL lanes (cs_merge_lanes), back substitution by thread
// (cs_backsub_thread): the per-level kernels' arithmetic, so the same bits.
// Levels below l_lo go through k_tree_level / k_backsub_level before and
// after this launch.
extern "C" __global__ void __launch_bounds__(128) k_upper(CsBatch bt, int l_lo) {
  extern __shared__ double smem[];
  const int groups = blockDim.x / CS_TL, grp = threadIdx.x / CS_TL, c = threadIdx.x & (CS_TL - 1);
  const int njac = bt.nlist[1];
  for (int k = blockIdx.x; k < njac; k += gridDim.x) {
    const int b = bt.jac[k];
    const int off = bt.off[b];
    const int n0 = bt.N[b] - 1;
    const int L = cs_levels(n0);
    for (int l = l_lo; l < L; ++l) {
      const int nl = cs_rows_at(n0, l);
      const int merges = nl >> 1, items = (nl + 1) >> 1;
      const double* src = ((l & 1) ? bt.rows1 : bt.rows0) + (size_t)off * CS_ROWSZ;
      double* dst = ((l & 1) ? bt.rows0 : bt.rows1) + (size_t)off * CS_ROWSZ;
      for (int mi = grp; mi < items; mi += groups) {  // uniform within a lane group
        if (mi < merges) {
          cs_merge_lanes(src + (size_t)(2 * mi) * CS_ROWSZ, src + (size_t)(2 * mi + 1) * CS_ROWSZ,
                         dst + (size_t)mi * CS_ROWSZ, bt.tree + (size_t)(off + ((2 * mi + 1) << l)) * CS_TREESZ, true);
        } else {
          const double* sr = src + (size_t)(nl - 1) * CS_ROWSZ;
          double* dr = dst + (size_t)merges * CS_ROWSZ;
          for (int q = c; q < CS_ROWSZ; q += CS_TL) dr[q] = sr[q];
        }
      }
      __syncthreads();
    }
    if (threadIdx.x < 32) cs_top_warp(bt, b, smem);
    __syncthreads();
    const double* dpv = bt.dp + (size_t)b * CS_NP;
    for (int l = L - 1; l >= l_lo; --l) {
      const int merges = cs_rows_at(n0, l) >> 1;
      for (int mi = threadIdx.x; mi < merges; mi += blockDim.x) {
        const int mid = (2 * mi + 1) << l, left = (2 * mi) << l;
        int right = (2 * mi + 2) << l;
        if (right > n0) right = n0;
        cs_backsub_thread(bt.tree + (size_t)(off + mid) * CS_TREESZ, bt.dy + (size_t)(off + left) * CS_NY,
                          bt.dy + (size_t)(off + right) * CS_NY, dpv, bt.dy + (size_t)(off + mid) * CS_NY);
      }
      __syncthreads();
    }
  }
}
#else
// needs lane merges on small block rows; the host never launches it otherwise
extern "C" __global__ void k_upper(CsBatch bt, int l_lo) {}
#endif

// Stage steps: dk = -(X_f + X_J dy_i + X_V dp), warp per interval, lanes
// over stage rows (the reference re-factorises W instead,
// collocation_solver_parallel_2d_shared.py:1619-1650).
extern "C" __global__ void k_recover(CsBatch bt) {
  const int wpc = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int njac = bt.nlist[1];
  const long long total = bt.jac_pre[njac];
  for (long long it = (long long)blockIdx.x * wpc + w; it < total; it += (long long)gridDim.x * wpc) {
    const int k = cs_find(bt.jac_pre, njac, it);
    const int b = bt.jac[k];
    const int slot = bt.off[b] + (int)(it - bt.jac_pre[k]);
    const double* X = bt.X + (size_t)slot * CS_NRHS * CS_S;
    const double* dyi = bt.dy + (size_t)slot * CS_NY;
    const double* dpv = bt.dp + (size_t)b * CS_NP;
    for (int r = lane; r < CS_S; r += 32) {
      double v = X[(size_t)(CS_NY + CS_NPE) * CS_S + r];
      for (int q = 0; q < CS_NY; ++q) v = fma(X[(size_t)q * CS_S + r], dyi[q], v);
      for (int q = 0; q < CS_NPE; ++q) v = fma(X[(size_t)(CS_NY + q) * CS_S + r], dpv[q], v);
      const int j = r / (CS_NY + CS_NZ), a = r % (CS_NY + CS_NZ);
      if (a < CS_NY) bt.dydot[((size_t)slot * CS_M + j) * CS_NY + a] = -v;
      else bt.dzt[((size_t)slot * CS_M + j) * CS_NZ + (a - CS_NY)] = -v;
    }
  }
}

#if !CS_BIG_TREE
// The whole Newton direction of one instance in one CTA: tree levels up,
// top system, back substitution down, stage recovery, then the line search
// starts (alpha = 1).  One launch per super-step instead of 2 L + 3, which is
// what matters when few instances are left; used for batches of small and
// medium instances (the per-level kernels above serve large single ones).
extern "C" __global__ void __launch_bounds__(256) k_babd_cta(CsBatch bt, int recover) {
  extern __shared__ double smem[];
  const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* top = smem;                                  // CS_TLD x (CS_NT + 1)
  double* Qw = smem + (size_t)CS_TLD * (CS_NT + 1) + (size_t)w * CS_QLD * CS_QC;  // merge matrix per warp
  const int njac = bt.nlist[1];
  for (int k = blockIdx.x; k < njac; k += gridDim.x) {
    const int b = bt.jac[k];
    const int N = bt.N[b], off = bt.off[b];
    const int n0 = N - 1;
    const int L = cs_levels(n0);
    // ---- tree up
    for (int l = 0; l < L; ++l) {
      const int nl = cs_rows_at(n0, l);
      const int merges = nl >> 1, items = (nl + 1) >> 1;
      const double* src = ((l & 1) ? bt.rows1 : bt.rows0) + (size_t)off * CS_ROWSZ;
      double* dst = ((l & 1) ? bt.rows0 : bt.rows1) + (size_t)off * CS_ROWSZ;
#if CS_TREE_THREAD
      for (int mi = threadIdx.x; mi < items; mi += blockDim.x) {
        if (mi < merges) {
          cs_merge_thread(src + (size_t)(2 * mi) * CS_ROWSZ, src + (size_t)(2 * mi + 1) * CS_ROWSZ,
                          dst + (size_t)mi * CS_ROWSZ, bt.tree + (size_t)(off + ((2 * mi + 1) << l)) * CS_TREESZ);
        } else {
          const double* sr = src + (size_t)(nl - 1) * CS_ROWSZ;
          double* dr = dst + (size_t)merges * CS_ROWSZ;
          for (int q = 0; q < CS_ROWSZ; ++q) dr[q] = sr[q];
        }
      }
#else
      for (int mi = w; mi < items; mi += nw) {
        if (mi < merges) {
          cs_merge_warp(src + (size_t)(2 * mi) * CS_ROWSZ, src + (size_t)(2 * mi + 1) * CS_ROWSZ,
                        dst + (size_t)mi * CS_ROWSZ, bt.tree + (size_t)(off + ((2 * mi + 1) << l)) * CS_TREESZ, Qw);
        } else {
          const double* sr = src + (size_t)(nl - 1) * CS_ROWSZ;
          double* dr = dst + (size_t)merges * CS_ROWSZ;
          for (int q = lane; q < CS_ROWSZ; q += 32) dr[q] = sr[q];
        }
        __syncwarp();
      }
#endif
      __syncthreads();
    }
    // ---- top system (warp 0)
    if (w == 0) cs_top_warp(bt, b, top);
    __syncthreads();
    // ---- back substitution down
    const double* dpv = bt.dp + (size_t)b * CS_NP;
    for (int l = L - 1; l >= 0; --l) {
      const int merges = cs_rows_at(n0, l) >> 1;
#if CS_TREE_THREAD
      for (int mi = threadIdx.x; mi < merges; mi += blockDim.x) {
        const int mid = (2 * mi + 1) << l, left = (2 * mi) << l;
        int right = (2 * mi + 2) << l;
        if (right > n0) right = n0;
        cs_backsub_thread(bt.tree + (size_t)(off + mid) * CS_TREESZ, bt.dy + (size_t)(off + left) * CS_NY,
                          bt.dy + (size_t)(off + right) * CS_NY, dpv, bt.dy + (size_t)(off + mid) * CS_NY);
      }
#else
      for (int mi = w; mi < merges; mi += nw) {
        const int mid = (2 * mi + 1) << l, left = (2 * mi) << l;
        int right = (2 * mi + 2) << l;
        if (right > n0) right = n0;
        cs_backsub_warp(bt.tree + (size_t)(off + mid) * CS_TREESZ, bt.dy + (size_t)(off + left) * CS_NY,
                        bt.dy + (size_t)(off + right) * CS_NY, dpv, bt.dy + (size_t)(off + mid) * CS_NY);
      }
#endif
      __syncthreads();
    }
    // ---- stage recovery, warp per interval, lanes over stage rows (or by
    //      k_recover across the GPU when recover == 0)
    for (int iv = w; recover && iv < n0; iv += nw) {
      const int slot = off + iv;
      const double* X = bt.X + (size_t)slot * CS_NRHS * CS_S;
      const double* dyi = bt.dy + (size_t)slot * CS_NY;
      for (int r = lane; r < CS_S; r += 32) {
        double v = X[(size_t)(CS_NY + CS_NPE) * CS_S + r];
        for (int q = 0; q < CS_NY; ++q) v = fma(X[(size_t)q * CS_S + r], dyi[q], v);
        for (int q = 0; q < CS_NPE; ++q) v = fma(X[(size_t)(CS_NY + q) * CS_S + r], dpv[q], v);
        const int j = r / (CS_NY + CS_NZ), a = r % (CS_NY + CS_NZ);
        if (a < CS_NY) bt.dydot[((size_t)slot * CS_M + j) * CS_NY + a] = -v;
        else bt.dzt[((size_t)slot * CS_M + j) * CS_NZ + (a - CS_NY)] = -v;
      }
    }
    __syncthreads();
  }
}

#else
// not used for large stage systems (the host never launches it)
extern "C" __global__ void k_babd_cta(CsBatch bt, int recover) {}
#endif  // !CS_BIG_TREE

#if CS_BIG
// ========================================================================
// Large stage systems (pendulum chains: K = 8 takes the condensation only,
// K = 16 and 32 both; s = m (ny + nz) in the hundreds, blocks of ny = 32 ..
// 128).  The matrices no longer fit in shared memory, so each CTA owns a slab
// of global memory (bt.wsp; L2 resident) and the kernels below replace
// k_condense (CS_BIG_COND), k_tree_level and k_top (CS_BIG_TREE):
//   k_condense    one CTA per interval, right-looking blocked LU of the
//                 augmented system [W11 | R1] with panels of CS_NB columns in
//                 shared memory.  Same operations in the same order as the
//                 unblocked elimination of cs_condense_group (pivot rule,
//                 multipliers, the fma chain of every entry), so both give
//                 the same bits.  CS_PREC 1 / 2 (TF32 / BF16):
//                 cs_condense_tc, FP32 storage and the block updates on
//                 the tensor cores with tcgen05.
//   k_tree_level  one CTA per merge, compact-WY Householder in panels of
//                 CS_HB reflectors (CS_PREC_TREE: on the tensor cores).
//   k_top         one CTA per instance.
#define CS_NB 16
#define CS_LDG (((CS_NCOL1 + 3) / 4) * 4)   // row stride of the slab matrix
#define CS_PLD (CS_NB + 1)                  // row stride of the panel (shared)
// slab: W [S1][LDG] | stage Jacobians [M][RB][NFG] | X0 [RB][NRHS]
//       | (reduced precision) FP32 copies of the stage Jacobians and X0
#define CS_WS_JF ((long long)CS_M * CS_RB * CS_NFG + (long long)CS_RB * CS_NRHS + CS_M * CS_M + CS_M)
#define CS_WS_COND ((long long)CS_S1 * CS_LDG + CS_WS_JF + (CS_PREC ? (CS_WS_JF + 1) / 2 : 0ll))
// shared: panel [S1][PLD] | U12 [NB][LDG] | fa [M RB] | hA [M M] | fb [NY] | inv [S1] | red [16] | piv [NB]
#define CS_SM_COND (CS_S1 * CS_PLD + CS_NB * CS_LDG + CS_M * CS_RB + CS_M * CS_M + CS_NY + CS_S1 + 16 + CS_NB)
// merge matrix and top system: in shared memory when they fit, else in the slab
#define CS_QSZ (CS_QLD * CS_QC)
#define CS_TSZ (CS_TLD * (CS_NT + 1))
#define CS_DRSZ ((CS_NY + CS_NP) * (2 * CS_NY + CS_NP))
// merges: Householder panels of CS_HB reflectors; shared: V [HB][QLD] | T [HB][HB] | G [HB][HB] | tau [HB] | red [32]
#define CS_HB 16
#define CS_SM_HB (CS_HB * CS_QLD + 2 * CS_HB * CS_HB + CS_HB + 32)
#define CS_Q_SMEM (((long long)CS_QSZ + CS_SM_HB) * 8 <= CS_SMEM_MAX)
#define CS_T_SMEM (((long long)CS_TSZ + 32) * 8 <= CS_SMEM_MAX)
#define CS_WS_TREE (CS_Q_SMEM ? 0ll : (long long)CS_QSZ)
#define CS_WS_TOP ((CS_T_SMEM ? 0ll : (long long)CS_TSZ) + (long long)CS_DRSZ)
#define CS_SM_TREE ((CS_Q_SMEM ? CS_QSZ : 0) + CS_SM_HB)
// reduced precision (CS_PREC_TREE != 0): FP32 merge matrix; shared floats V [HB][QLD] |
// T, G [HB][HB] | tau [HB] | W [QC][HB], then red [32] doubles
#define CS_SHF (CS_HB * CS_QLD + 2 * CS_HB * CS_HB + CS_HB + CS_QC * CS_HB)
#define CS_SM_HB_LP ((CS_SHF + 1) / 2 + 32)
#define CS_QSZ_LP ((CS_QSZ + 1) / 2)
#define CS_Q_SMEM_LP (((long long)CS_QSZ_LP + CS_SM_HB_LP) * 8 <= CS_SMEM_MAX)
#define CS_WS_TREE_LP (CS_Q_SMEM_LP ? 0ll : (long long)CS_QSZ_LP)
#define CS_SM_TREE_LP ((CS_Q_SMEM_LP ? CS_QSZ_LP : 0) + CS_SM_HB_LP)
#define CS_SM_TOP ((CS_T_SMEM ? CS_TSZ : 0) + 32)

// tensor-core operands: FP32 rounded to TF32 (round to nearest, ties away),
// or two FP32 rounded to a BF16 pair (lo in the low half)
__device__ __forceinline__ unsigned cs_tf32(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ unsigned cs_bf2(float lo, float hi) {
  unsigned r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

__device__ __forceinline__ unsigned cs_dyn_smem_bytes() {
  unsigned r;
  asm volatile("mov.u32 %0, %%dynamic_smem_size;" : "=r"(r));
  return r;
}

// the launch gives this CTA a slab of at least `slab` doubles and `sm`
// doubles of shared memory; otherwise count a configuration error and do
// nothing (the host reports it)
__device__ __forceinline__ bool cs_big_ok(const CsBatch& bt, long long slab, long long sm) {
  const bool ok = blockDim.x <= 256 && (blockDim.x & 31) == 0 && (long long)cs_dyn_smem_bytes() >= sm * 8 &&
                  (slab == 0 || (bt.wsp != nullptr && (int)blockIdx.x < bt.wsp_ctas && bt.wsp_stride >= slab));
  if (!ok && threadIdx.x == 0) atomicAdd(&bt.counters[7], 1ull);
  return ok;
}

// largest key over the CTA, the smallest row on ties (red: 16 doubles)
__device__ __forceinline__ void cs_cta_argmax(unsigned long long& best, int& brow, double* red) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int orow = __shfl_xor_sync(0xffffffffu, brow, o);
    if (ob > best || (ob == best && orow < brow)) { best = ob; brow = orow; }
  }
  const int nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[threadIdx.x >> 5] = __longlong_as_double((long long)best);
    red[8 + (threadIdx.x >> 5)] = (double)brow;
  }
  __syncthreads();
  best = (unsigned long long)__double_as_longlong(red[0]);
  brow = (int)red[8];
  for (int w = 1; w < nw; ++w) {
    const unsigned long long ob = (unsigned long long)__double_as_longlong(red[w]);
    const int orow = (int)red[8 + w];
    if (ob > best || (ob == best && orow < brow)) { best = ob; brow = orow; }
  }
  __syncthreads();
}

// sum over the CTA; every thread gets the same value (red: 8 doubles)
__device__ __forceinline__ double cs_cta_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  __syncthreads();
  return s;
}

#if CS_BIG_COND
// stage j: f, g at the stage point into fa, their Jacobians into the slab
// (not inlined: the big problem functions keep their registers to
// themselves, away from the elimination loops)
__device__ __noinline__ void cs_stage_big(const CsBatch& bt, int slot, int b, int j, double h, double* JG, double* fa) {
  constexpr int RB = CS_RB;
  const double* th = bt.th + (size_t)b * (CS_NTH > 0 ? CS_NTH : 1);
  const double* yi = bt.y + (size_t)slot * CS_NY;
  const double* yd = bt.ydot + (size_t)slot * CS_M * CS_NY;
  double pl[CS_NP > 0 ? CS_NP : 1];
  for (int k = 0; k < CS_NP; ++k) pl[k] = bt.p[(size_t)b * CS_NP + k];
  double yt[CS_NY], zl[CS_NZ > 0 ? CS_NZ : 1], f[CS_NY];
  for (int k = 0; k < CS_NY; ++k) {
    double s = 0.0;
    for (int q = 0; q < CS_M; ++q) s += CS_A[j * CS_M + q] * yd[q * CS_NY + k];
    yt[k] = yi[k] + h * s;
  }
  for (int k = 0; k < CS_NZ; ++k) zl[k] = bt.zt[((size_t)slot * CS_M + j) * CS_NZ + k];
  double* Jj = JG + (size_t)j * RB * CS_NFG;
  cs_f(yt, zl, pl, th, f);
  cs_Df(yt, zl, pl, th, Jj);
  for (int a = 0; a < CS_NY; ++a) fa[j * RB + a] = f[a] - yd[j * CS_NY + a];
#if CS_NZ > 0
  double g[CS_NZ];
  cs_g(yt, zl, pl, th, bt.inst[b].alpha, g);
  cs_Dg(yt, zl, pl, th, bt.inst[b].alpha, Jj + (size_t)CS_NY * CS_NFG);
  for (int a = 0; a < CS_NZ; ++a) fa[j * RB + CS_NY + a] = g[a];
#endif
}

// element-type helpers of the large-system condensation (T = double for the
// FP64 path, float for the mixed-precision one)
__device__ __forceinline__ double cs_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float cs_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ unsigned long long cs_abskey(float v) {
  return (unsigned long long)(__float_as_uint(v) & 0x7fffffffu);
}
__device__ __forceinline__ bool cs_tiny(double v) { return cs_abskey(v) < 0x3ce4000000000000ull; }
__device__ __forceinline__ bool cs_tiny(float v) { return fabsf(v) < 2.220446049250313e-15f; }

template <typename T, int PREC>
__device__ void cs_condense_big(const CsBatch& bt, int slot, double* slab, double* sm) {
  constexpr int RB = CS_RB;
  const int tid = threadIdx.x, nt = blockDim.x;
  T* W = reinterpret_cast<T*>(slab);                  // [S1][LDG]
  double* JG = slab + (size_t)CS_S1 * CS_LDG;         // [M][RB][NFG]: Df rows, then Dg rows
  double* X0 = JG + (size_t)CS_M * RB * CS_NFG;       // [RB][NRHS]
  T* P = reinterpret_cast<T*>(sm);                    // [S1][PLD]
  T* U = P + CS_S1 * CS_PLD;                          // [NB][LDG], columns relative to the panel's end
  double* fa = sm + ((CS_S1 * CS_PLD + CS_NB * CS_LDG) * sizeof(T) + 7) / 8;
  double* hA = fa + CS_M * RB;
  double* fb = hA + CS_M * CS_M;
  T* inv = reinterpret_cast<T*>(fb + CS_NY);
  double* red = fb + CS_NY + CS_S1;
  int* piv = (int*)(red + 16);
  const int b = bt.inst_of[slot];
  const double h = bt.t[slot + 1] - bt.t[slot];
  const double* yi = bt.y + (size_t)slot * CS_NY;
  const double* yd = bt.ydot + (size_t)slot * CS_M * CS_NY;
  // ---- stage functions and Jacobians, thread j for stage j
  for (int j = tid; j < CS_M; j += nt) cs_stage_big(bt, slot, b, j, h, JG, fa);
  for (int e = tid; e < CS_M * CS_M; e += nt) hA[e] = h * CS_A[e];
  for (int k = tid; k < CS_NY; k += nt) {
    double s = 0.0;
    for (int j = 0; j < CS_M; ++j) s += CS_B[j] * yd[j * CS_NY + k];
    fb[k] = yi[CS_NY + k] - yi[k] - h * s;
  }
  __syncthreads();
  // ---- stage 0: [-I h_z0; 0 g_z0] X0 = R0, one thread per right-hand side
  for (int c = tid; c < CS_NRHS; c += nt) {
    const double* J0 = JG;
#if CS_NZ > 0
    double gz[CS_NZ][CS_NZ], xz[CS_NZ];
    for (int a = 0; a < CS_NZ; ++a) {
      for (int q = 0; q < CS_NZ; ++q) gz[a][q] = J0[(CS_NY + a) * CS_NFG + CS_NY + q];
      xz[a] = cs_rhs(J0 + (CS_NY + a) * CS_NFG, fa, 0, CS_NY + a, c);
    }
    for (int kk = 0; kk < CS_NZ; ++kk) {
      int pr = kk;
      for (int r = kk + 1; r < CS_NZ; ++r)
        if (cs_abskey(gz[r][kk]) > cs_abskey(gz[pr][kk])) pr = r;
      if (pr != kk) {
        for (int q = 0; q < CS_NZ; ++q) { const double t = gz[kk][q]; gz[kk][q] = gz[pr][q]; gz[pr][q] = t; }
        const double t = xz[kk]; xz[kk] = xz[pr]; xz[pr] = t;
      }
      const double ip = 1.0 / gz[kk][kk];
      for (int r = kk + 1; r < CS_NZ; ++r) {
        const double l = gz[r][kk] * ip;
        for (int q = kk + 1; q < CS_NZ; ++q) gz[r][q] = fma(-l, gz[kk][q], gz[r][q]);
        xz[r] = fma(-l, xz[kk], xz[r]);
      }
    }
    for (int r = CS_NZ - 1; r >= 0; --r) {
      double v = xz[r];
      for (int q = r + 1; q < CS_NZ; ++q) v = fma(-gz[r][q], xz[q], v);
      xz[r] = v / gz[r][r];
    }
    for (int a = 0; a < CS_NZ; ++a) X0[(CS_NY + a) * CS_NRHS + c] = xz[a];
#endif
    for (int a = 0; a < CS_NY; ++a) {
      double v = -cs_rhs(J0 + a * CS_NFG, fa, 0, a, c);
#if CS_NZ > 0
      for (int q = 0; q < CS_NZ; ++q) v = fma(J0[a * CS_NFG + CS_NY + q], xz[q], v);
#endif
      X0[a * CS_NRHS + c] = v;
    }
  }
  __syncthreads();
  // ---- the reduced system [W11 | R1 - W10 X0] (stages 1..M-1) into the slab
  for (int e = tid; e < CS_S1 * CS_NCOL1; e += nt) {
    const int row = e / CS_NCOL1, col = e - row * CS_NCOL1;
    const int j = 1 + row / RB, a = row - (j - 1) * RB;
    const double* J = JG + (size_t)(j * RB + a) * CS_NFG;
    double v;
    if (col < CS_S1) {
      const int k = 1 + col / RB, q = col - (k - 1) * RB;
      if (q < CS_NY) {
        v = hA[j * CS_M + k] * J[q];
        if (k == j && q == a) v -= 1.0;
      } else {
        v = (k == j) ? J[q] : 0.0;
      }
    } else {
      const int c = col - CS_S1;
      double w = 0.0;
      for (int q = 0; q < CS_NY; ++q) w = fma(J[q], X0[q * CS_NRHS + c], w);
      v = fma(-hA[j * CS_M], w, cs_rhs(J, fa, j, a, c));
    }
    W[(size_t)row * CS_LDG + col] = (T)v;
  }
  __syncthreads();
  // ---- blocked LU with partial pivoting
  int singular = 0;
#pragma unroll 1
  for (int k0 = 0; k0 < CS_S1; k0 += CS_NB) {
    const int kb = min(CS_NB, CS_S1 - k0);
    const int pr = CS_S1 - k0;        // panel rows
    for (int e = tid; e < pr * kb; e += nt) {
      const int r = e / kb, c = e - r * kb;
      P[r * CS_PLD + c] = W[(size_t)(k0 + r) * CS_LDG + k0 + c];
    }
    __syncthreads();
#pragma unroll 1
    for (int kk = 0; kk < kb; ++kk) {
      unsigned long long best = 0ull;
      int brow = CS_S1;  // larger than any row: loses every tie
      for (int r = kk + tid; r < pr; r += nt) {
        const unsigned long long v = cs_abskey(P[r * CS_PLD + kk]);
        if (v > best || brow == CS_S1) { best = v; brow = r; }
      }
      cs_cta_argmax(best, brow, red);
      if (tid == 0) piv[kk] = brow;
      if (brow != kk)
        for (int c = tid; c < kb; c += nt) {
          const T tmp = P[kk * CS_PLD + c];
          P[kk * CS_PLD + c] = P[brow * CS_PLD + c];
          P[brow * CS_PLD + c] = tmp;
        }
      __syncthreads();
      const T pv = P[kk * CS_PLD + kk];
      const bool tiny = cs_tiny(pv);  // |pv| < 10 * 2^-52
      singular |= tiny;
      const T ip = (T)1 / pv;
      if (tid == 0) inv[k0 + kk] = ip;
      const T mul = tiny ? (T)0 : ip;
      for (int r = kk + 1 + tid; r < pr; r += nt) P[r * CS_PLD + kk] *= mul;
      __syncthreads();
      const int nc = kb - kk - 1;
      if (nc > 0) {
        const int ne = (pr - kk - 1) * nc;
        for (int e = tid; e < ne; e += nt) {
          const int rr = e / nc;
          const int r = kk + 1 + rr, c = kk + 1 + (e - rr * nc);
          P[r * CS_PLD + c] = cs_fma(-P[r * CS_PLD + kk], P[kk * CS_PLD + c], P[r * CS_PLD + c]);
        }
      }
      __syncthreads();
    }
    // panel rows 0..kb-1 (U11, multipliers below its diagonal) back to the slab
    for (int e = tid; e < kb * kb; e += nt) {
      const int r = e / kb, c = e - r * kb;
      W[(size_t)(k0 + r) * CS_LDG + k0 + c] = P[r * CS_PLD + c];
    }
    // columns right of the panel: the row swaps in order, then U12 = L11^-1 A12
    const int c0 = k0 + kb, ncol = CS_NCOL1 - c0;
    for (int c = tid; c < ncol; c += nt) {
      T* colp = W + c0 + c;
      for (int kk = 0; kk < kb; ++kk) {
        const int pr2 = piv[kk];
        if (pr2 != kk) {
          const T t0 = colp[(size_t)(k0 + kk) * CS_LDG];
          colp[(size_t)(k0 + kk) * CS_LDG] = colp[(size_t)(k0 + pr2) * CS_LDG];
          colp[(size_t)(k0 + pr2) * CS_LDG] = t0;
        }
      }
      // column c of U12 in shared memory (this thread's own column)
#pragma unroll 1
      for (int i = 0; i < kb; ++i) {
        T v = colp[(size_t)(k0 + i) * CS_LDG];
        for (int l = 0; l < i; ++l) v = cs_fma(-P[i * CS_PLD + l], U[l * CS_LDG + c], v);
        colp[(size_t)(k0 + i) * CS_LDG] = v;
        U[i * CS_LDG + c] = v;
      }
    }
    __syncthreads();
    // trailing update A22 -= L21 U12: warp items of 16 rows x 32 columns,
    // lane owns one column (fills the lanes for any trailing width)
    const int r0 = k0 + kb, nr = CS_S1 - r0;
    if (nr > 0 && ncol > 0) {
      const int rt = (nr + 15) >> 4, ct = (ncol + 31) >> 5;
      const int lane = tid & 31, w = tid >> 5, nw = nt >> 5;
      for (int item = w; item < rt * ct; item += nw) {
        const int ri = item / ct, ci = item - ri * ct;
        const int ra = ri * 16, c = ci * 32 + lane;
        const bool cok = c < ncol;
        double acc[16];
#pragma unroll
        for (int i = 0; i < 16; ++i)
          acc[i] = (cok && ra + i < nr) ? W[(size_t)(r0 + ra + i) * CS_LDG + c0 + c] : 0.0;
#pragma unroll 2
        for (int l = 0; l < kb; ++l) {
          const double uv = cok ? U[l * CS_LDG + c] : 0.0;
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const double lv = (ra + i < nr) ? P[(kb + ra + i) * CS_PLD + l] : 0.0;
            acc[i] = fma(-lv, uv, acc[i]);
          }
        }
#pragma unroll
        for (int i = 0; i < 16; ++i)
          if (cok && ra + i < nr) W[(size_t)(r0 + ra + i) * CS_LDG + c0 + c] = acc[i];
      }
    }
    __syncthreads();
  }
  // ---- back substitution, blocks of CS_NB rows from the bottom; the
  //      right-hand sides are columns S1.. of the slab rows
#pragma unroll 1
  for (int k0 = ((CS_S1 - 1) / CS_NB) * CS_NB; k0 >= 0; k0 -= CS_NB) {
    const int kb = min(CS_NB, CS_S1 - k0);
    // U column block [0, k0+kb) x [k0, k0+kb) into the panel buffer
    for (int e = tid; e < (k0 + kb) * kb; e += nt) {
      const int r = e / kb, c = e - r * kb;
      P[r * CS_PLD + c] = W[(size_t)r * CS_LDG + k0 + c];
    }
    __syncthreads();
    // diagonal block, one thread per right-hand side, rows from the bottom
    for (int c = tid; c < CS_NRHS; c += nt) {
      T* colp = W + CS_S1 + c;
      for (int i = 0; i < kb; ++i) U[i * CS_LDG + c] = colp[(size_t)(k0 + i) * CS_LDG];
#pragma unroll 1
      for (int i = kb - 1; i >= 0; --i) {
        const T xi = U[i * CS_LDG + c] * inv[k0 + i];
        U[i * CS_LDG + c] = xi;
        for (int q = 0; q < i; ++q) U[q * CS_LDG + c] = cs_fma(-P[(k0 + q) * CS_PLD + i], xi, U[q * CS_LDG + c]);
      }
      for (int i = 0; i < kb; ++i) colp[(size_t)(k0 + i) * CS_LDG] = U[i * CS_LDG + c];
    }
    __syncthreads();
    // rows above the block: B[q] -= U[q][k0 + i] x[i], i from the last
    for (int e = tid; e < k0 * CS_NRHS; e += nt) {
      const int q = e / CS_NRHS, c = e - q * CS_NRHS;
      T v = W[(size_t)q * CS_LDG + CS_S1 + c];
      for (int i = kb - 1; i >= 0; --i) v = cs_fma(-P[q * CS_PLD + i], U[i * CS_LDG + c], v);
      W[(size_t)q * CS_LDG + CS_S1 + c] = v;
    }
    __syncthreads();
  }
  // ---- X (column-major [NRHS][S]: stage-0 rows from X0, the others from W)
  double* X = bt.X + (size_t)slot * CS_NRHS * CS_S;
  for (int e = tid; e < CS_NRHS * CS_S; e += nt) {
    const int c = e / CS_S, r = e - c * CS_S;
    X[e] = (r < RB) ? X0[r * CS_NRHS + c] : (double)W[(size_t)(r - RB) * CS_LDG + CS_S1 + c];
  }
  // ---- condensed block row: D X = h sum_j b_j X[(j, a)]
  double* row = bt.rows0 + (size_t)slot * CS_ROWSZ;
  for (int e = tid; e < CS_NRHS * CS_NY; e += nt) {
    const int c = e / CS_NY, a = e - c * CS_NY;
    double s = CS_B[0] * X0[a * CS_NRHS + c];
    for (int j = 1; j < CS_M; ++j) s += CS_B[j] * (double)W[(size_t)((j - 1) * RB + a) * CS_LDG + CS_S1 + c];
    const double dx = h * s;
    if (c < CS_NY) {
      row[c * CS_NY + a] = (a == c) ? dx - 1.0 : dx;
      row[(CS_NY + c) * CS_NY + a] = (a == c ? 1.0 : 0.0);
    } else if (c < CS_NY + CS_NPE) {
      row[(2 * CS_NY + (c - CS_NY)) * CS_NY + a] = dx;
    } else {
      row[(2 * CS_NY + CS_NPE) * CS_NY + a] = -fb[a] - dx;
    }
  }
  singular = __syncthreads_or(singular);
  if (singular && tid == 0) atomicAdd(&bt.inst[b].singular, 1);
  __syncthreads();
}

#if CS_PREC != 0
// ------------------------------------------------------------------------
// Reduced-precision condensation on the tensor cores (CS_PREC 1: TF32,
// 2: BF16).  FP32 storage of the stage system in the slab (column-major: a
// thread of the tensor-memory epilogue owns a row, so a warp's accesses to
// one column are one line), FP32 panel factorisation (partial pivoting, the
// pivot rule of the FP64 path), and the three block updates of width >= 16
// on tcgen05 (cs_umma.cuh: operands in shared memory, FP32 accumulators in
// tensor memory):
//   fill        R1 - W10 X0: (hA[j][0] J_y rows) x X0_y, K = ny in chunks of 64
//   LU          A22 -= L21 U12 after every panel of CS_NBT = 32 columns
//   back subst. X_above -= U_above,block X_block for blocks of CS_NB = 16 rows
// The stage Jacobians, the stage-0 block solve and the residual stay FP64;
// the result is an inexact Newton Jacobian (the FP64 residual, line search
// and mesh error drive the solve to the FP64 tolerance).
#define CS_NBT 32
#define CS_PLDT (CS_NBT + 1)
#define CS_LDR (((CS_S1 + 3) / 4) * 4)                   // leading dimension of the column-major slab matrix
#define CS_TCE ((CS_PREC == 1) ? 4 : 8)                 // FP32 values per 16-byte operand segment
#define CS_TCKC (CS_NBT / CS_TCE)                        // LU update: core matrices along K (K = CS_NBT)
#define CS_TCKB (CS_NB / CS_TCE)                         // back substitution (K = CS_NB)
#define CS_TCKF (64 / CS_TCE)                            // fill (K chunks of 64)
#define CS_TCMP ((CS_S1 > CS_NBT) ? ((CS_S1 - CS_NBT + 127) / 128) * 128 : 128)  // L21 operand rows
#define CS_TCMB (((CS_S1 + 127) / 128) * 128)            // U_above operand rows
#define CS_TCNR (((CS_NRHS + 15) / 16) * 16)             // right-hand-side operand rows
#define CS_TCNB 256                                      // U12 operand rows (a chunk of columns, one per thread)
#define CS_TC_R128(x) ((((x) + 127) / 128) * 128)
#define CS_TC_OPS_LU ((CS_TCMP + CS_TCNB) * CS_TCKC * 16)
#define CS_TC_OPS_BS ((CS_TCMB + CS_TCNR) * CS_TCKB * 16)
#define CS_TC_OPS CS_TC_R128((CS_TC_OPS_LU > CS_TC_OPS_BS) ? CS_TC_OPS_LU : CS_TC_OPS_BS)
#define CS_TC_PANEL CS_TC_R128(CS_S1 * CS_PLDT * 4)
#define CS_TC_FILL ((128 + CS_TCNR) * CS_TCKF * 16)      // fill operands: operand area + panel
#define CS_TC_DBL (8 * (CS_M * CS_RB + CS_M * CS_M + CS_NY + 16))
#define CS_TC_MISC (CS_TC_OPS + CS_TC_PANEL + CS_TC_DBL + CS_TC_R128(4 * CS_S1 + 4 * CS_NBT))
#define CS_TC_SMB (CS_TC_MISC + 16)                      // + mbarrier, TMEM address, error flag
#define CS_TC_SMD ((CS_TC_SMB + 7) / 8)
#define CS_TC_WAIT 2000000000ll                          // MMA completion bound (cycles, about 1 s)
#define CS_JLD (CS_NFG | 1)                              // row stride of the fill's staged Jacobian rows
static_assert(CS_TC_FILL <= CS_TC_OPS + CS_TC_PANEL, "fill operands exceed the operand area and panel");
static_assert(32 * CS_JLD * 4 <= CS_TC_PANEL, "the fill's staged Jacobian rows exceed the panel");
static_assert((long long)CS_NCOL1 * CS_LDR <= 2ll * CS_S1 * CS_LDG, "column-major matrix exceeds the slab's matrix area");
static_assert(CS_NBT % CS_TCE == 0 && CS_NB % CS_TCE == 0 && 64 % CS_TCE == 0, "operand K widths");

// FP64 -> FP32 copy of n values, eight loads in flight per thread before
// their stores (source and destination share the slab, so the compiler would
// otherwise wait for each store before the next load)
__device__ __forceinline__ void cs_copy_f32(const double* __restrict__ src, float* __restrict__ dst, int n) {
  const int tid = threadIdx.x, nt = blockDim.x;
  int e = tid;
  for (; e + 7 * nt < n; e += 8 * nt) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = src[e + u * nt];
#pragma unroll
    for (int u = 0; u < 8; ++u) dst[e + u * nt] = (float)v[u];
  }
  for (; e < n; e += nt) dst[e] = (float)src[e];
}

// shared memory (bytes): operands [CS_TC_OPS] | panel P [S1][PLDT] floats |
// fa [M RB], hA [M M], fb [NY], red [16] doubles | inv [S1] floats, piv [NBT] |
// mbarrier, TMEM address, error flag.  Returns false after a tensor-core
// timeout (every thread; the operands and accumulator are then abandoned).
template <int PREC>
__device__ bool cs_condense_tc(const CsBatch& bt, int slot, double* slab, unsigned char* sm, unsigned tmem,
                               unsigned mbar, unsigned& phase, int* flag) {
  constexpr int RB = CS_RB;
  constexpr int EPS = CS_TCE;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, w = tid >> 5, nw = nt >> 5;
  float* W = reinterpret_cast<float*>(slab);                       // column-major [NCOL1][LDR]
  double* JG = slab + (size_t)CS_S1 * CS_LDG;                      // [M][RB][NFG]
  double* X0 = JG + (size_t)CS_M * RB * CS_NFG;                    // [RB][NRHS]
  float* JGf = reinterpret_cast<float*>(X0 + (size_t)RB * CS_NRHS);  // FP32 copies
  float* X0f = JGf + (size_t)CS_M * RB * CS_NFG;
  float* hAf = X0f + (size_t)RB * CS_NRHS;
  float* Bf = hAf + CS_M * CS_M;
  unsigned char* ops = sm;
  float* P = reinterpret_cast<float*>(sm + CS_TC_OPS);
  double* fa = reinterpret_cast<double*>(sm + CS_TC_OPS + CS_TC_PANEL);
  double* hA = fa + CS_M * RB;
  double* fb = hA + CS_M * CS_M;
  double* red = fb + CS_NY;
  float* inv = reinterpret_cast<float*>(red + 16);
  int* piv = reinterpret_cast<int*>(inv + CS_S1);
  const int b = bt.inst_of[slot];
  const double h = bt.t[slot + 1] - bt.t[slot];
  const double* yi = bt.y + (size_t)slot * CS_NY;
  const double* yd = bt.ydot + (size_t)slot * CS_M * CS_NY;
  // ---- stage functions and Jacobians (FP64), thread j for stage j
  for (int j = tid; j < CS_M; j += nt) cs_stage_big(bt, slot, b, j, h, JG, fa);
  for (int e = tid; e < CS_M * CS_M; e += nt) hA[e] = h * CS_A[e];
  for (int k = tid; k < CS_NY; k += nt) {
    double s = 0.0;
    for (int j = 0; j < CS_M; ++j) s += CS_B[j] * yd[j * CS_NY + k];
    fb[k] = yi[CS_NY + k] - yi[k] - h * s;
  }
  __syncthreads();
  // ---- stage 0: [-I h_z0; 0 g_z0] X0 = R0 (FP64), one thread per right-hand side
  for (int c = tid; c < CS_NRHS; c += nt) {
    const double* J0 = JG;
#if CS_NZ > 0
    double gz[CS_NZ][CS_NZ], xz[CS_NZ];
    for (int a = 0; a < CS_NZ; ++a) {
      for (int q = 0; q < CS_NZ; ++q) gz[a][q] = J0[(CS_NY + a) * CS_NFG + CS_NY + q];
      xz[a] = cs_rhs(J0 + (CS_NY + a) * CS_NFG, fa, 0, CS_NY + a, c);
    }
    for (int kk = 0; kk < CS_NZ; ++kk) {
      int pr = kk;
      for (int r = kk + 1; r < CS_NZ; ++r)
        if (cs_abskey(gz[r][kk]) > cs_abskey(gz[pr][kk])) pr = r;
      if (pr != kk) {
        for (int q = 0; q < CS_NZ; ++q) { const double t = gz[kk][q]; gz[kk][q] = gz[pr][q]; gz[pr][q] = t; }
        const double t = xz[kk]; xz[kk] = xz[pr]; xz[pr] = t;
      }
      const double ip = 1.0 / gz[kk][kk];
      for (int r = kk + 1; r < CS_NZ; ++r) {
        const double l = gz[r][kk] * ip;
        for (int q = kk + 1; q < CS_NZ; ++q) gz[r][q] = fma(-l, gz[kk][q], gz[r][q]);
        xz[r] = fma(-l, xz[kk], xz[r]);
      }
    }
    for (int r = CS_NZ - 1; r >= 0; --r) {
      double v = xz[r];
      for (int q = r + 1; q < CS_NZ; ++q) v = fma(-gz[r][q], xz[q], v);
      xz[r] = v / gz[r][r];
    }
    for (int a = 0; a < CS_NZ; ++a) X0[(CS_NY + a) * CS_NRHS + c] = xz[a];
#endif
    for (int a = 0; a < CS_NY; ++a) {
      double v = -cs_rhs(J0 + a * CS_NFG, fa, 0, a, c);
#if CS_NZ > 0
      for (int q = 0; q < CS_NZ; ++q) v = fma(J0[a * CS_NFG + CS_NY + q], xz[q], v);
#endif
      X0[a * CS_NRHS + c] = v;
    }
  }
  __syncthreads();
  // ---- FP32 copies of the stage Jacobians and X0, once
  cs_copy_f32(JG, JGf, CS_M * RB * CS_NFG);
  cs_copy_f32(X0, X0f, RB * CS_NRHS);
  for (int e = tid; e < CS_M * CS_M; e += nt) hAf[e] = (float)hA[e];
  for (int e = tid; e < CS_M; e += nt) Bf[e] = (float)(h * CS_B[e]);
  __syncthreads();
  // ---- the reduced system [W11 | R1] (stages 1..M-1), 32 rows at a time:
  //      their Jacobian rows staged in shared memory (the panel's space),
  //      then a warp per column, a lane per row (column-major stores are
  //      one line per warp)
  for (int rb0 = 0; rb0 < CS_S1; rb0 += 32) {
    const int nrow = min(32, CS_S1 - rb0);
    for (int r = w; r < nrow; r += nw) {
      const int row = rb0 + r;
      const int j = 1 + row / RB, a = row - (j - 1) * RB;
      const float* Jf = JGf + (size_t)(j * RB + a) * CS_NFG;
      for (int q = lane; q < CS_NFG; q += 32) P[r * CS_JLD + q] = Jf[q];
    }
    __syncthreads();
    const int row = rb0 + lane;
    const bool rok = lane < nrow;
    const int j = rok ? 1 + row / RB : 1, a = rok ? row - (j - 1) * RB : 0;
    const float* Js = P + lane * CS_JLD;
    for (int col = w; col < CS_NCOL1; col += nw) {
      float v;
      if (col < CS_S1) {
        const int k = 1 + col / RB, q = col - (k - 1) * RB;
        if (q < CS_NY) {
          v = hAf[j * CS_M + k] * Js[q];
          if (k == j && q == a) v -= 1.f;
        } else {
          v = (k == j) ? Js[q] : 0.f;
        }
      } else {
        const int c = col - CS_S1;
        v = (c < CS_NY) ? Js[c] : ((c < CS_NY + CS_NPE) ? Js[CS_NY + CS_NZ + (c - CS_NY)] : (float)fa[j * RB + a]);
      }
      if (rok) W[(size_t)col * CS_LDR + row] = v;
    }
    __syncthreads();
  }
  // ---- R1 -= W10 X0 on the tensor cores: A rows hA[j][0] J_y(j, a), B rows the
  //      right-hand sides of X0's y part, K = ny in chunks of 64
  {
    unsigned char* FA = ops;
    unsigned char* FB = ops + 128 * CS_TCKF * 16;
    for (int k0 = 0; k0 < CS_NY; k0 += 64) {
      const int kw = min(64, CS_NY - k0);
      __syncthreads();  // R1 written; earlier MMAs done with the operand area
      for (int e = tid; e < CS_TCNR * CS_TCKF; e += nt) {
        const int c = e / CS_TCKF, sg = e - c * CS_TCKF;
        float x[EPS];
#pragma unroll
        for (int ee = 0; ee < EPS; ++ee) {
          const int q = sg * EPS + ee;
          x[ee] = (c < CS_NRHS && q < kw) ? X0f[(size_t)(k0 + q) * CS_NRHS + c] : 0.f;
        }
        cs_tc_put<PREC>(FB, c, sg, CS_TCKF, x);
      }
      for (int t0 = 0; t0 < CS_S1; t0 += 128) {
        const int mr = min(128, CS_S1 - t0);
        for (int e = tid; e < 128 * CS_TCKF; e += nt) {
          const int r = e / CS_TCKF, sg = e - r * CS_TCKF;
          float x[EPS];
          if (r < mr) {
            const int row = t0 + r;
            const int j = 1 + row / RB, a = row - (j - 1) * RB;
            const float* Jf = JGf + (size_t)(j * RB + a) * CS_NFG + k0;
            const float s0 = hAf[j * CS_M];
#pragma unroll
            for (int ee = 0; ee < EPS; ++ee) {
              const int q = sg * EPS + ee;
              x[ee] = (q < kw) ? s0 * Jf[q] : 0.f;
            }
          } else {
#pragma unroll
            for (int ee = 0; ee < EPS; ++ee) x[ee] = 0.f;
          }
          cs_tc_put<PREC>(FA, r, sg, CS_TCKF, x);
        }
        cs_fence_async_smem();
        __syncthreads();
        if (!cs_tc_block_update<PREC>(W + (size_t)CS_S1 * CS_LDR + t0, 1, CS_LDR, mr, CS_NRHS, FA, FB, CS_TCKF,
                                      CS_TCKF / 2, tmem, mbar, phase, CS_TC_WAIT, flag))
          return false;
      }
    }
  }
  __syncthreads();
  // ---- blocked LU with partial pivoting, panels of CS_NBT columns
  int singular = 0;
  unsigned char* A_s = ops;
  unsigned char* B_s = ops + CS_TCMP * CS_TCKC * 16;
#pragma unroll 1
  for (int k0 = 0; k0 < CS_S1; k0 += CS_NBT) {
    const int kb = min(CS_NBT, CS_S1 - k0);
    const int pr = CS_S1 - k0;  // panel rows
    for (int c = w; c < kb; c += nw)
      for (int r = lane; r < pr; r += 32) P[r * CS_PLDT + c] = W[(size_t)(k0 + c) * CS_LDR + k0 + r];
    __syncthreads();
#pragma unroll 1
    for (int kk = 0; kk < kb; ++kk) {
      unsigned long long best = 0ull;
      int brow = CS_S1;  // larger than any row: loses every tie
      for (int r = kk + tid; r < pr; r += nt) {
        const unsigned long long v = cs_abskey(P[r * CS_PLDT + kk]);
        if (v > best || brow == CS_S1) { best = v; brow = r; }
      }
      cs_cta_argmax(best, brow, red);
      if (tid == 0) piv[kk] = brow;
      if (brow != kk)
        for (int c = tid; c < kb; c += nt) {
          const float tmp = P[kk * CS_PLDT + c];
          P[kk * CS_PLDT + c] = P[brow * CS_PLDT + c];
          P[brow * CS_PLDT + c] = tmp;
        }
      __syncthreads();
      const float pv = P[kk * CS_PLDT + kk];
      const bool tiny = cs_tiny(pv);
      singular |= tiny;
      const float ip = 1.f / pv;
      if (tid == 0) inv[k0 + kk] = ip;
      const float mul = tiny ? 0.f : ip;
      // multipliers and the rank-1 update of the panel, a thread per row
      for (int r = kk + 1 + tid; r < pr; r += nt) {
        float* Pr = P + r * CS_PLDT;
        const float l = Pr[kk] * mul;
        Pr[kk] = l;
        for (int c = kk + 1; c < kb; ++c) Pr[c] = fmaf(-l, P[kk * CS_PLDT + c], Pr[c]);
      }
      __syncthreads();
    }
    // U11 (and L11) rows back to the slab
    for (int c = w; c < kb; c += nw)
      for (int r = lane; r < kb; r += 32) W[(size_t)(k0 + c) * CS_LDR + k0 + r] = P[r * CS_PLDT + c];
    const int c0 = k0 + kb, ncol = CS_NCOL1 - c0, r0 = k0 + kb, nr = CS_S1 - r0;
    // A operand: L21, rows padded with zeros to a multiple of 128, K to CS_NBT
    if (nr > 0)
      for (int e = tid; e < ((nr + 127) & ~127) * CS_TCKC; e += nt) {
        const int r = e / CS_TCKC, sg = e - r * CS_TCKC;
        float x[EPS];
#pragma unroll
        for (int ee = 0; ee < EPS; ++ee) {
          const int c = sg * EPS + ee;
          x[ee] = (r < nr && c < kb) ? P[(kb + r) * CS_PLDT + c] : 0.f;
        }
        cs_tc_put<PREC>(A_s, r, sg, CS_TCKC, x);
      }
    // columns right of the panel, a column per thread at a time: the row
    // swaps in order, U12 = L11^-1 A12 in registers, U12 into the slab and
    // into the B operand, then A22 -= L21 U12 on the tensor cores
    for (int n0 = 0; n0 < ncol; n0 += nt) {
      const int nch = min(nt, ncol - n0);  // nt <= CS_TCNB (cs_big_ok)
      if (tid < nch) {
        float* colp = W + (size_t)(c0 + n0 + tid) * CS_LDR;
        for (int kk = 0; kk < kb; ++kk) {
          const int p2 = piv[kk];
          if (p2 != kk) {
            const float t0 = colp[k0 + kk];
            colp[k0 + kk] = colp[k0 + p2];
            colp[k0 + p2] = t0;
          }
        }
        float u[CS_NBT];
#pragma unroll
        for (int i = 0; i < CS_NBT; ++i) u[i] = (i < kb) ? colp[k0 + i] : 0.f;
#pragma unroll
        for (int i = 1; i < CS_NBT; ++i) {
          if (i < kb) {
            float v = u[i];
#pragma unroll
            for (int l = 0; l < i; ++l) v = fmaf(-P[i * CS_PLDT + l], u[l], v);
            u[i] = v;
          }
        }
#pragma unroll
        for (int i = 0; i < CS_NBT; ++i)
          if (i < kb) colp[k0 + i] = u[i];
        if (nr > 0) {
#pragma unroll
          for (int sg = 0; sg < CS_TCKC; ++sg) cs_tc_put<PREC>(B_s, tid, sg, CS_TCKC, u + sg * EPS);
        }
      } else if (nr > 0 && tid < ((nch + 15) & ~15)) {
        float z[EPS];
#pragma unroll
        for (int ee = 0; ee < EPS; ++ee) z[ee] = 0.f;
#pragma unroll
        for (int sg = 0; sg < CS_TCKC; ++sg) cs_tc_put<PREC>(B_s, tid, sg, CS_TCKC, z);
      }
      if (nr > 0) {
        cs_fence_async_smem();
        __syncthreads();
        if (!cs_tc_block_update<PREC>(W + (size_t)(c0 + n0) * CS_LDR + r0, 1, CS_LDR, nr, nch, A_s, B_s, CS_TCKC,
                                      CS_TCKC / 2, tmem, mbar, phase, CS_TC_WAIT, flag))
          return false;
      }
    }
    __syncthreads();
  }
  // ---- back substitution, blocks of CS_NB rows from the bottom: the block's
  //      triangular solve by one thread per right-hand side, then the rows
  //      above on the tensor cores
#pragma unroll 1
  for (int k0 = ((CS_S1 - 1) / CS_NB) * CS_NB; k0 >= 0; k0 -= CS_NB) {
    const int kb = min(CS_NB, CS_S1 - k0);
    // U column block [0, k0+kb) x [k0, k0+kb) into the panel buffer
    for (int c = w; c < kb; c += nw)
      for (int r = lane; r < k0 + kb; r += 32) P[r * CS_PLDT + c] = W[(size_t)(k0 + c) * CS_LDR + r];
    __syncthreads();
    unsigned char* UA = ops;
    unsigned char* XB = ops + CS_TCMB * CS_TCKB * 16;
    for (int c = tid; c < CS_TCNR; c += nt) {
      float x[CS_NB];
#pragma unroll
      for (int i = 0; i < CS_NB; ++i) x[i] = 0.f;
      if (c < CS_NRHS) {
        float* colp = W + (size_t)(CS_S1 + c) * CS_LDR;
#pragma unroll
        for (int i = 0; i < CS_NB; ++i)
          if (i < kb) x[i] = colp[k0 + i];
#pragma unroll
        for (int i = CS_NB - 1; i >= 0; --i) {
          if (i < kb) {
            const float xi = x[i] * inv[k0 + i];
            x[i] = xi;
#pragma unroll
            for (int q = 0; q < i; ++q) x[q] = fmaf(-P[(k0 + q) * CS_PLDT + i], xi, x[q]);
          }
        }
#pragma unroll
        for (int i = 0; i < CS_NB; ++i)
          if (i < kb) colp[k0 + i] = x[i];
      }
      if (k0 > 0) {
#pragma unroll
        for (int sg = 0; sg < CS_TCKB; ++sg) cs_tc_put<PREC>(XB, c, sg, CS_TCKB, x + sg * EPS);
      }
    }
    if (k0 > 0) {
      for (int e = tid; e < ((k0 + 127) & ~127) * CS_TCKB; e += nt) {
        const int r = e / CS_TCKB, sg = e - r * CS_TCKB;
        float x[EPS];
#pragma unroll
        for (int ee = 0; ee < EPS; ++ee) {
          const int c = sg * EPS + ee;
          x[ee] = (r < k0 && c < kb) ? P[r * CS_PLDT + c] : 0.f;
        }
        cs_tc_put<PREC>(UA, r, sg, CS_TCKB, x);
      }
      cs_fence_async_smem();
      __syncthreads();
      if (!cs_tc_block_update<PREC>(W + (size_t)CS_S1 * CS_LDR, 1, CS_LDR, k0, CS_NRHS, UA, XB, CS_TCKB, CS_TCKB / 2,
                                    tmem, mbar, phase, CS_TC_WAIT, flag))
        return false;
    }
    __syncthreads();
  }
  // ---- X (column-major [NRHS][S]: stage-0 rows from X0, the others from W)
  double* X = bt.X + (size_t)slot * CS_NRHS * CS_S;
  for (int c = w; c < CS_NRHS; c += nw) {
    // a column's loads before its stores (X is another array: no aliasing,
    // which the compiler cannot see)
    constexpr int NQ = (CS_S + 31) / 32;
    double xv[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const int r = lane + 32 * q;
      xv[q] = (r >= CS_S) ? 0.0 : ((r < RB) ? X0[r * CS_NRHS + c] : (double)W[(size_t)(CS_S1 + c) * CS_LDR + (r - RB)]);
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      if (lane + 32 * q < CS_S) X[(size_t)c * CS_S + lane + 32 * q] = xv[q];
  }
  // ---- condensed block row: D X = h sum_j b_j X[(j, a)]
  double* row = bt.rows0 + (size_t)slot * CS_ROWSZ;
  for (int c = w; c < CS_NRHS; c += nw)
    for (int a = lane; a < CS_NY; a += 32) {
      float sf = Bf[0] * X0f[a * CS_NRHS + c];
      for (int j = 1; j < CS_M; ++j) sf = fmaf(Bf[j], W[(size_t)(CS_S1 + c) * CS_LDR + (j - 1) * RB + a], sf);
      const double dx = (double)sf;
      if (c < CS_NY) {
        row[c * CS_NY + a] = (a == c) ? dx - 1.0 : dx;
        row[(CS_NY + c) * CS_NY + a] = (a == c ? 1.0 : 0.0);
      } else if (c < CS_NY + CS_NPE) {
        row[(2 * CS_NY + (c - CS_NY)) * CS_NY + a] = dx;
      } else {
        row[(2 * CS_NY + CS_NPE) * CS_NY + a] = -fb[a] - dx;
      }
    }
  singular = __syncthreads_or(singular);
  if (singular && tid == 0) atomicAdd(&bt.inst[b].singular, 1);
  __syncthreads();
  return true;
}
#endif  // CS_PREC != 0

extern "C" __global__ void __launch_bounds__(256, 2) k_condense(CsBatch bt) {
  extern __shared__ __align__(128) double smem[];
#if CS_PREC == 0
  if (!cs_big_ok(bt, CS_WS_COND, CS_SM_COND)) return;
#else
  if (!cs_big_ok(bt, CS_WS_COND, CS_TC_SMD)) return;
  // the CTA's tensor-memory accumulator and MMA barrier, for all its intervals
  unsigned char* smb = reinterpret_cast<unsigned char*>(smem);
  unsigned long long* mb = reinterpret_cast<unsigned long long*>(smb + CS_TC_MISC);
  unsigned* tslot = reinterpret_cast<unsigned*>(mb + 1);
  int* flag = reinterpret_cast<int*>(tslot + 1);
  if (threadIdx.x == 0) {
    cs_mbar_init(cs_sa(mb), 1);
    *flag = 0;
  }
  if (threadIdx.x < 32) cs_tmem_alloc(cs_sa(tslot), CS_TC_COLS);
  cs_tc_before_sync();
  __syncthreads();
  cs_tc_after_sync();
  const unsigned tmem = *tslot;
  unsigned phase = 0;
#endif
  double* slab = bt.wsp + (size_t)blockIdx.x * bt.wsp_stride;
  const int njac = bt.nlist[1];
  const long long total = bt.jac_pre[njac];
  for (long long it = blockIdx.x; it < total; it += gridDim.x) {
    const int k = cs_find(bt.jac_pre, njac, it);
    const int b = bt.jac[k];
    const int slot = bt.off[b] + (int)(it - bt.jac_pre[k]);
#if CS_PREC == 0
    cs_condense_big<double, 0>(bt, slot, slab, smem);
#else
    if (!cs_condense_tc<CS_PREC>(bt, slot, slab, smb, tmem, cs_sa(mb), phase, flag)) break;
#endif
  }
#if CS_PREC != 0
  // release the accumulator; a tensor-core timeout is reported like a
  // configuration error (the host then fails the call)
  cs_tc_before_sync();
  __syncthreads();
  if (threadIdx.x == 0 && *flag) atomicAdd(&bt.counters[7], 1ull);
  if (threadIdx.x < 32) {
    cs_tc_after_sync();
    cs_tmem_free(tmem, CS_TC_COLS);
  }
#endif
}

#endif  // CS_BIG_COND

#if CS_BIG_TREE
// Householder column k of a column-major matrix A (leading dimension ld,
// rows k..n-1) applied to columns k+1..nc-1, CTA-wide: a warp per column,
// lanes over rows.  Sign rule and early skip as matrix_factorization_cuda.py:37-54.
__device__ __forceinline__ void cs_householder_cta(double* A, int ld, int n, int nc, int k, double* red) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, w = tid >> 5, nw = nt >> 5;
  const double* vk = A + (size_t)k * ld;
  double ss = 0.0;
  for (int r = k + tid; r < n; r += nt) ss += vk[r] * vk[r];
  ss = cs_cta_sum(ss, red);
  const double x0 = vk[k];
  const double sgn = (x0 >= 0.0) ? 1.0 : -1.0;
  const double g = -sgn * sqrt(ss);
  const double v0 = x0 - g;
  const double vs = ss - x0 * x0 + v0 * v0;
  if (vs < CS_EPS) return;  // uniform: nothing to eliminate in this column
  const double beta = -2.0 / vs;
  for (int c = k + 1 + w; c < nc; c += nw) {
    double* col = A + (size_t)c * ld;
    double wv = (lane == 0) ? v0 * col[k] : 0.0;
    for (int r = k + 1 + lane; r < n; r += 32) wv = fma(vk[r], col[r], wv);
    for (int o = 16; o > 0; o >>= 1) wv += __shfl_xor_sync(0xffffffffu, wv, o);
    const double bw = beta * wv;
    if (lane == 0) col[k] = fma(bw, v0, col[k]);
    for (int r = k + 1 + lane; r < n; r += 32) col[r] = fma(bw, vk[r], col[r]);
  }
  __syncthreads();
  double* ck = A + (size_t)k * ld;
  if (tid == 0) ck[k] = g;
  for (int r = k + 1 + tid; r < n; r += nt) ck[r] = 0.0;
  __syncthreads();
}

// Merge of block rows a and b, one CTA (layout as cs_merge_warp), blocked
// Householder (compact WY, as LAPACK's geqrt): each panel of CS_HB columns is
// factorised column by column (cs_householder_cta restricted to the panel),
// its reflectors H_i = I - tau_i v_i v_i^T (tau = 2/|v|^2, the sign rule of
// matrix_factorization_cuda.py:37-54) are accumulated as
// H_1 ... H_kb = I - V T V^T, and the columns right of the panel are updated
// at once, C <- C - V (T^T (V^T C)), one thread per column.
__device__ void cs_merge_cta(const double* ra, const double* rb, double* out_row, double* rec, double* Q, double* sh) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, w = tid >> 5, nw = nt >> 5;
  constexpr int n = 2 * CS_NY;
  double* V = sh;                          // [HB][QLD] column-major, zero above row k0 + i
  double* Tm = V + CS_HB * CS_QLD;         // [HB][HB], T[j][i] at Tm[i * HB + j]
  double* G = Tm + CS_HB * CS_HB;          // [HB][HB], V_j . V_i at G[i * HB + j]
  double* tau = G + CS_HB * CS_HB;         // [HB]
  double* red = tau + CS_HB;               // [32]
  for (int e = tid; e < CS_QC * CS_NY; e += nt) {
    const int c = e / CS_NY, r = e - c * CS_NY;
    double top, bot;
    if (c < CS_NY) { top = ra[(CS_NY + c) * CS_NY + r]; bot = rb[c * CS_NY + r]; }
    else if (c < 2 * CS_NY) { top = ra[(c - CS_NY) * CS_NY + r]; bot = 0.0; }
    else if (c < 3 * CS_NY) { top = 0.0; bot = rb[(CS_NY + c - 2 * CS_NY) * CS_NY + r]; }
    else if (c < 3 * CS_NY + CS_NPE) { top = ra[(2 * CS_NY + c - 3 * CS_NY) * CS_NY + r]; bot = rb[(2 * CS_NY + c - 3 * CS_NY) * CS_NY + r]; }
    else { top = ra[(2 * CS_NY + CS_NPE) * CS_NY + r]; bot = rb[(2 * CS_NY + CS_NPE) * CS_NY + r]; }
    Q[(size_t)c * CS_QLD + r] = top;
    Q[(size_t)c * CS_QLD + CS_NY + r] = bot;
  }
  __syncthreads();
#pragma unroll 1
  for (int k0 = 0; k0 < CS_NY; k0 += CS_HB) {
    const int kb = min(CS_HB, CS_NY - k0);
    const int pe = k0 + kb;  // panel end (exclusive)
    // ---- panel: reflectors of columns k0 .. pe-1, applied inside the panel
#pragma unroll 1
    for (int kk = 0; kk < kb; ++kk) {
      const int k = k0 + kk;
      double* vk = Q + (size_t)k * CS_QLD;
      double ss = 0.0;
      for (int r = k + tid; r < n; r += nt) ss += vk[r] * vk[r];
      ss = cs_cta_sum(ss, red);
      const double x0 = vk[k];
      const double g = (x0 >= 0.0) ? -sqrt(ss) : sqrt(ss);
      const double v0 = x0 - g;
      const double vs = ss - x0 * x0 + v0 * v0;
      double* Vi = V + kk * CS_QLD;
      if (vs < CS_EPS) {  // uniform: nothing to eliminate, H = I
        for (int r = tid; r < n; r += nt) Vi[r] = 0.0;
        if (tid == 0) tau[kk] = 0.0;
        __syncthreads();
        continue;
      }
      const double beta = -2.0 / vs;
      for (int r = tid; r < n; r += nt) Vi[r] = (r < k) ? 0.0 : ((r == k) ? v0 : vk[r]);
      if (tid == 0) tau[kk] = 2.0 / vs;
      for (int c = k + 1 + w; c < pe; c += nw) {
        double* col = Q + (size_t)c * CS_QLD;
        double wv = (lane == 0) ? v0 * col[k] : 0.0;
        for (int r = k + 1 + lane; r < n; r += 32) wv = fma(vk[r], col[r], wv);
        for (int o = 16; o > 0; o >>= 1) wv += __shfl_xor_sync(0xffffffffu, wv, o);
        const double bw = beta * wv;
        if (lane == 0) col[k] = fma(bw, v0, col[k]);
        for (int r = k + 1 + lane; r < n; r += 32) col[r] = fma(bw, vk[r], col[r]);
      }
      __syncthreads();
      if (tid == 0) vk[k] = g;
      for (int r = k + 1 + tid; r < n; r += nt) vk[r] = 0.0;
      __syncthreads();
    }
    // a last panel narrower than CS_HB: its unused reflectors are the identity
    for (int e = tid; e < (CS_HB - kb) * CS_QLD; e += nt) V[kb * CS_QLD + e] = 0.0;
    for (int e = tid; e < (CS_HB - kb) * CS_HB; e += nt) Tm[kb * CS_HB + e] = 0.0;
    // ---- T: G = V^T V (upper part), then T column by column
    for (int e = tid; e < kb * kb; e += nt) {
      const int i = e / kb, j = e - i * kb;
      if (j < i) {
        const double* vi = V + i * CS_QLD;
        const double* vj = V + j * CS_QLD;
        double d = 0.0;
        for (int r = k0 + i; r < n; ++r) d = fma(vj[r], vi[r], d);
        G[i * CS_HB + j] = d;
      }
    }
    __syncthreads();
    if (tid == 0) {
      for (int i = 0; i < kb; ++i) {
        const double ti = tau[i];
        for (int j = 0; j < i; ++j) {
          double sj = 0.0;
          for (int q = j; q < i; ++q) sj = fma(Tm[q * CS_HB + j], G[i * CS_HB + q], sj);
          Tm[i * CS_HB + j] = -ti * sj;
        }
        Tm[i * CS_HB + i] = ti;
      }
    }
    __syncthreads();
    // ---- trailing columns: C <- C - V (T^T (V^T C)); four consecutive lanes
    //      per column, each over every fourth row, V^T C summed across them
    const int nc = CS_QC - pe;
    for (int base = 0; base < 4 * nc; base += nt) {
      const int u = base + tid;
      const int c = pe + (u >> 2), part = u & 3;
      const bool act = c < CS_QC;
      double* col = Q + (size_t)(act ? c : pe) * CS_QLD;
      double wv[CS_HB];
#pragma unroll
      for (int i = 0; i < CS_HB; ++i) wv[i] = 0.0;
#pragma unroll 2
      for (int r = k0 + part; r < n; r += 4) {
        const double x = col[r];
#pragma unroll
        for (int i = 0; i < CS_HB; ++i) wv[i] = fma(V[i * CS_QLD + r], x, wv[i]);
      }
#pragma unroll
      for (int i = 0; i < CS_HB; ++i) {
        wv[i] += __shfl_xor_sync(0xffffffffu, wv[i], 1);
        wv[i] += __shfl_xor_sync(0xffffffffu, wv[i], 2);
      }
      double tw[CS_HB];
#pragma unroll
      for (int i = 0; i < CS_HB; ++i) {
        double sacc = 0.0;
#pragma unroll
        for (int j = 0; j <= i; ++j) sacc = fma(Tm[i * CS_HB + j], wv[j], sacc);
        tw[i] = sacc;
      }
      if (act) {
#pragma unroll 2
        for (int r = k0 + part; r < n; r += 4) {
          double x = col[r];
#pragma unroll
          for (int i = 0; i < CS_HB; ++i) x = fma(-V[i * CS_QLD + r], tw[i], x);
          col[r] = x;
        }
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < CS_QC * CS_NY; e += nt) {
    const int c = e / CS_NY, r = e - c * CS_NY;
    rec[e] = Q[(size_t)c * CS_QLD + r];
    if (c >= CS_NY) out_row[(size_t)(c - CS_NY) * CS_NY + r] = Q[(size_t)c * CS_QLD + CS_NY + r];
  }
  __syncthreads();
}

#if CS_PREC_TREE != 0
// sum over the CTA in FP32 (red: 8 doubles of scratch)
__device__ __forceinline__ float cs_cta_sumf(float v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  float* rf = reinterpret_cast<float*>(red);
  if ((threadIdx.x & 31) == 0) rf[threadIdx.x >> 5] = v;
  __syncthreads();
  float s = 0.f;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += rf[w];
  __syncthreads();
  return s;
}

// The merge of cs_merge_cta in reduced precision: FP32 merge matrix and
// reflectors, the two products of each panel's WY update on the tensor cores
// (FP32 accumulators): W = V^T C (k = the rows), then C -= V (T^T W) (k = the
// panel's 16 reflectors); operands rounded to TF32 (PREC 1) or BF16 (PREC 2).
// The top system and the back substitution stay FP64.
template <int PREC>
__device__ void cs_merge_cta_lp(const double* ra, const double* rb, double* out_row, double* rec, float* Q, double* sh) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, w = tid >> 5, nw = nt >> 5;
  const int g = lane >> 2, t = lane & 3;
  constexpr int n = 2 * CS_NY;
  float* V = reinterpret_cast<float*>(sh);  // [HB][QLD]
  float* Tm = V + CS_HB * CS_QLD;           // T[j][i] at Tm[i * HB + j]
  float* G = Tm + CS_HB * CS_HB;
  float* tau = G + CS_HB * CS_HB;
  float* Wm = tau + CS_HB;                  // [QC][HB]
  double* red = sh + (CS_SHF + 1) / 2;
  for (int e = tid; e < CS_QC * CS_NY; e += nt) {
    const int c = e / CS_NY, r = e - c * CS_NY;
    double top, bot;
    if (c < CS_NY) { top = ra[(CS_NY + c) * CS_NY + r]; bot = rb[c * CS_NY + r]; }
    else if (c < 2 * CS_NY) { top = ra[(c - CS_NY) * CS_NY + r]; bot = 0.0; }
    else if (c < 3 * CS_NY) { top = 0.0; bot = rb[(CS_NY + c - 2 * CS_NY) * CS_NY + r]; }
    else if (c < 3 * CS_NY + CS_NPE) { top = ra[(2 * CS_NY + c - 3 * CS_NY) * CS_NY + r]; bot = rb[(2 * CS_NY + c - 3 * CS_NY) * CS_NY + r]; }
    else { top = ra[(2 * CS_NY + CS_NPE) * CS_NY + r]; bot = rb[(2 * CS_NY + CS_NPE) * CS_NY + r]; }
    Q[(size_t)c * CS_QLD + r] = (float)top;
    Q[(size_t)c * CS_QLD + CS_NY + r] = (float)bot;
  }
  __syncthreads();
#pragma unroll 1
  for (int k0 = 0; k0 < CS_NY; k0 += CS_HB) {
    const int kb = min(CS_HB, CS_NY - k0);
    const int pe = k0 + kb;
    // ---- panel (FP32, as cs_merge_cta)
#pragma unroll 1
    for (int kk = 0; kk < kb; ++kk) {
      const int k = k0 + kk;
      float* vk = Q + (size_t)k * CS_QLD;
      float ss = 0.f;
      for (int r = k + tid; r < n; r += nt) ss = fmaf(vk[r], vk[r], ss);
      ss = cs_cta_sumf(ss, red);
      const float x0 = vk[k];
      const float gg = (x0 >= 0.f) ? -sqrtf(ss) : sqrtf(ss);
      const float v0 = x0 - gg;
      const float vs = ss - x0 * x0 + v0 * v0;
      float* Vi = V + kk * CS_QLD;
      if ((double)vs < CS_EPS) {
        for (int r = tid; r < n; r += nt) Vi[r] = 0.f;
        if (tid == 0) tau[kk] = 0.f;
        __syncthreads();
        continue;
      }
      const float beta = -2.f / vs;
      for (int r = tid; r < n; r += nt) Vi[r] = (r < k) ? 0.f : ((r == k) ? v0 : vk[r]);
      if (tid == 0) tau[kk] = 2.f / vs;
      for (int c = k + 1 + w; c < pe; c += nw) {
        float* col = Q + (size_t)c * CS_QLD;
        float wv = (lane == 0) ? v0 * col[k] : 0.f;
        for (int r = k + 1 + lane; r < n; r += 32) wv = fmaf(vk[r], col[r], wv);
        for (int o = 16; o > 0; o >>= 1) wv += __shfl_xor_sync(0xffffffffu, wv, o);
        const float bw = beta * wv;
        if (lane == 0) col[k] = fmaf(bw, v0, col[k]);
        for (int r = k + 1 + lane; r < n; r += 32) col[r] = fmaf(bw, vk[r], col[r]);
      }
      __syncthreads();
      if (tid == 0) vk[k] = gg;
      for (int r = k + 1 + tid; r < n; r += nt) vk[r] = 0.f;
      __syncthreads();
    }
    for (int e = tid; e < (CS_HB - kb) * CS_QLD; e += nt) V[kb * CS_QLD + e] = 0.f;
    for (int e = tid; e < (CS_HB - kb) * CS_HB; e += nt) Tm[kb * CS_HB + e] = 0.f;
    for (int e = tid; e < kb * kb; e += nt) {
      const int i = e / kb, j = e - i * kb;
      if (j < i) {
        const float* vi = V + i * CS_QLD;
        const float* vj = V + j * CS_QLD;
        float d = 0.f;
        for (int r = k0 + i; r < n; ++r) d = fmaf(vj[r], vi[r], d);
        G[i * CS_HB + j] = d;
      }
    }
    __syncthreads();
    if (tid == 0) {
      for (int i = 0; i < kb; ++i) {
        const float ti = tau[i];
        for (int j = 0; j < i; ++j) {
          float sj = 0.f;
          for (int q = j; q < i; ++q) sj = fmaf(Tm[q * CS_HB + j], G[i * CS_HB + q], sj);
          Tm[i * CS_HB + j] = -ti * sj;
        }
        Tm[i * CS_HB + i] = ti;
      }
    }
    __syncthreads();
    const int nc = CS_QC - pe;
    // ---- W = V^T C: 16 reflectors x 8-column tiles, k over the rows
    auto Va = [&](int i, int r) -> float { return (r < n) ? V[i * CS_QLD + r] : 0.f; };
    auto Cb = [&](int r, int c) -> float { return (r < n && c < nc) ? Q[(size_t)(pe + c) * CS_QLD + r] : 0.f; };
    for (int tile = w; tile < (nc + 7) / 8; tile += nw) {
      const int cb = tile * 8;
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      if constexpr (PREC == 1) {
        for (int r0 = k0; r0 < n; r0 += 8) {
          const unsigned a0 = cs_tf32(Va(g, r0 + t)), a1 = cs_tf32(Va(g + 8, r0 + t));
          const unsigned a2 = cs_tf32(Va(g, r0 + t + 4)), a3 = cs_tf32(Va(g + 8, r0 + t + 4));
          const unsigned b0 = cs_tf32(Cb(r0 + t, cb + g)), b1 = cs_tf32(Cb(r0 + t + 4, cb + g));
          asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                       "{%0,%1,%2,%3};\n"
                       : "+f"(acc[0]), "+f"(acc[1]), "+f"(acc[2]), "+f"(acc[3])
                       : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
        }
      } else {
        for (int r0 = k0; r0 < n; r0 += 16) {
          const unsigned a0 = cs_bf2(Va(g, r0 + 2 * t), Va(g, r0 + 2 * t + 1));
          const unsigned a1 = cs_bf2(Va(g + 8, r0 + 2 * t), Va(g + 8, r0 + 2 * t + 1));
          const unsigned a2 = cs_bf2(Va(g, r0 + 2 * t + 8), Va(g, r0 + 2 * t + 9));
          const unsigned a3 = cs_bf2(Va(g + 8, r0 + 2 * t + 8), Va(g + 8, r0 + 2 * t + 9));
          const unsigned b0 = cs_bf2(Cb(r0 + 2 * t, cb + g), Cb(r0 + 2 * t + 1, cb + g));
          const unsigned b1 = cs_bf2(Cb(r0 + 2 * t + 8, cb + g), Cb(r0 + 2 * t + 9, cb + g));
          asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                       "{%0,%1,%2,%3};\n"
                       : "+f"(acc[0]), "+f"(acc[1]), "+f"(acc[2]), "+f"(acc[3])
                       : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int i = g + ((q & 2) ? 8 : 0), c = cb + 2 * t + (q & 1);
        if (c < nc) Wm[c * CS_HB + i] = acc[q];
      }
    }
    __syncthreads();
    // ---- W <- T^T W, a column per thread
    for (int c = tid; c < nc; c += nt) {
      float wv[CS_HB];
#pragma unroll
      for (int i = 0; i < CS_HB; ++i) wv[i] = Wm[c * CS_HB + i];
#pragma unroll
      for (int i = 0; i < CS_HB; ++i) {
        float sacc = 0.f;
#pragma unroll
        for (int j = 0; j <= i; ++j) sacc = fmaf(Tm[i * CS_HB + j], wv[j], sacc);
        Wm[c * CS_HB + i] = sacc;
      }
    }
    __syncthreads();
    // ---- C -= V W: 16-row x 8-column tiles over rows k0.. and the columns
    const int nr = n - k0;
    const int rt = (nr + 15) / 16, ct = (nc + 7) / 8;
    auto Am = [&](int r, int i) -> float { return (r < nr) ? -V[i * CS_QLD + k0 + r] : 0.f; };
    auto Bw = [&](int i, int c) -> float { return (c < nc) ? Wm[c * CS_HB + i] : 0.f; };
    for (int item = w; item < rt * ct; item += nw) {
      const int ri = item / ct, ci = item - ri * ct;
      const int ra = ri * 16, cb = ci * 8;
      float acc[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = ra + g + ((q & 2) ? 8 : 0), c = cb + 2 * t + (q & 1);
        acc[q] = (r < nr && c < nc) ? Q[(size_t)(pe + c) * CS_QLD + k0 + r] : 0.f;
      }
      if constexpr (PREC == 1) {
#pragma unroll
        for (int ks = 0; ks < CS_HB; ks += 8) {
          const unsigned a0 = cs_tf32(Am(ra + g, ks + t)), a1 = cs_tf32(Am(ra + g + 8, ks + t));
          const unsigned a2 = cs_tf32(Am(ra + g, ks + t + 4)), a3 = cs_tf32(Am(ra + g + 8, ks + t + 4));
          const unsigned b0 = cs_tf32(Bw(ks + t, cb + g)), b1 = cs_tf32(Bw(ks + t + 4, cb + g));
          asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                       "{%0,%1,%2,%3};\n"
                       : "+f"(acc[0]), "+f"(acc[1]), "+f"(acc[2]), "+f"(acc[3])
                       : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
        }
      } else {
        const unsigned a0 = cs_bf2(Am(ra + g, 2 * t), Am(ra + g, 2 * t + 1));
        const unsigned a1 = cs_bf2(Am(ra + g + 8, 2 * t), Am(ra + g + 8, 2 * t + 1));
        const unsigned a2 = cs_bf2(Am(ra + g, 2 * t + 8), Am(ra + g, 2 * t + 9));
        const unsigned a3 = cs_bf2(Am(ra + g + 8, 2 * t + 8), Am(ra + g + 8, 2 * t + 9));
        const unsigned b0 = cs_bf2(Bw(2 * t, cb + g), Bw(2 * t + 1, cb + g));
        const unsigned b1 = cs_bf2(Bw(2 * t + 8, cb + g), Bw(2 * t + 9, cb + g));
        asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                     "{%0,%1,%2,%3};\n"
                     : "+f"(acc[0]), "+f"(acc[1]), "+f"(acc[2]), "+f"(acc[3])
                     : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = ra + g + ((q & 2) ? 8 : 0), c = cb + 2 * t + (q & 1);
        if (r < nr && c < nc) Q[(size_t)(pe + c) * CS_QLD + k0 + r] = acc[q];
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < CS_QC * CS_NY; e += nt) {
    const int c = e / CS_NY, r = e - c * CS_NY;
    rec[e] = (double)Q[(size_t)c * CS_QLD + r];
    if (c >= CS_NY) out_row[(size_t)(c - CS_NY) * CS_NY + r] = (double)Q[(size_t)c * CS_QLD + CS_NY + r];
  }
  __syncthreads();
}
#endif  // CS_PREC_TREE != 0

extern "C" __global__ void __launch_bounds__(256) k_tree_level(CsBatch bt, int l) {
  extern __shared__ double smem[];
#if CS_PREC_TREE == 0
  if (!cs_big_ok(bt, CS_WS_TREE, CS_SM_TREE)) return;
  double* Q = CS_Q_SMEM ? smem : bt.wsp + (size_t)blockIdx.x * bt.wsp_stride;
  double* sh = CS_Q_SMEM ? smem + CS_QSZ : smem;
#else
  if (!cs_big_ok(bt, CS_WS_TREE_LP, CS_SM_TREE_LP)) return;
  float* Q = reinterpret_cast<float*>(CS_Q_SMEM_LP ? smem : bt.wsp + (size_t)blockIdx.x * bt.wsp_stride);
  double* sh = CS_Q_SMEM_LP ? smem + CS_QSZ_LP : smem;
#endif
  const int njac = bt.nlist[1];
  const long long* pre = bt.lvl_pre + (size_t)l * (bt.B + 1);
  const long long total = pre[njac];
  const double* srcb = (l & 1) ? bt.rows1 : bt.rows0;
  double* dstb = (l & 1) ? bt.rows0 : bt.rows1;
  for (long long it = blockIdx.x; it < total; it += gridDim.x) {
    const int k = cs_find(pre, njac, it);
    const int b = bt.jac[k];
    const int mi = (int)(it - pre[k]);
    const int off = bt.off[b];
    const int nl = cs_rows_at(bt.N[b] - 1, l);
    const int merges = nl >> 1;
    const double* src = srcb + (size_t)off * CS_ROWSZ;
    double* dst = dstb + (size_t)off * CS_ROWSZ;
    if (mi < merges) {
#if CS_PREC_TREE == 0
      cs_merge_cta(src + (size_t)(2 * mi) * CS_ROWSZ, src + (size_t)(2 * mi + 1) * CS_ROWSZ, dst + (size_t)mi * CS_ROWSZ,
                   bt.tree + (size_t)(off + ((2 * mi + 1) << l)) * CS_TREESZ, Q, sh);
#else
      cs_merge_cta_lp<CS_PREC_TREE>(src + (size_t)(2 * mi) * CS_ROWSZ, src + (size_t)(2 * mi + 1) * CS_ROWSZ,
                               dst + (size_t)mi * CS_ROWSZ, bt.tree + (size_t)(off + ((2 * mi + 1) << l)) * CS_TREESZ, Q,
                               sh);
#endif
    } else {
      const double* sr = src + (size_t)(nl - 1) * CS_ROWSZ;
      double* dr = dst + (size_t)merges * CS_ROWSZ;
      for (int q = threadIdx.x; q < CS_ROWSZ; q += blockDim.x) dr[q] = sr[q];
      __syncthreads();
    }
  }
}

// Top of the tree, one CTA per instance (as cs_top_warp; Dr goes to the slab).
// dyk, dpk (refinement, else null): the system is solved for a correction of
// the direction (dyk, dpk), so the boundary rows' right-hand side is their
// residual -r - Dr [dy_0; dy_n; dp] (FP64).
__device__ void cs_top_big(const CsBatch& bt, double* smem, const double* dyk, const double* dpk) {
  double* slab = bt.wsp + (size_t)blockIdx.x * bt.wsp_stride;
  double* top = CS_T_SMEM ? smem : slab;
  double* Dr = CS_T_SMEM ? slab : slab + CS_TSZ;
  double* red = CS_T_SMEM ? smem + CS_TSZ : smem;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int njac = bt.nlist[1];
  for (int k = blockIdx.x; k < njac; k += gridDim.x) {
    const int b = bt.jac[k];
    const int N = bt.N[b], off = bt.off[b];
    const int L = cs_levels(N - 1);
    const double* row = ((L & 1) ? bt.rows1 : bt.rows0) + (size_t)off * CS_ROWSZ;
    const double* th = bt.th + (size_t)b * (CS_NTH > 0 ? CS_NTH : 1);
    if (tid == 0) {
      double ya[CS_NY], yb[CS_NY], pl[CS_NP > 0 ? CS_NP : 1];
      for (int q = 0; q < CS_NY; ++q) { ya[q] = bt.y[(size_t)off * CS_NY + q]; yb[q] = bt.y[(size_t)(off + N - 1) * CS_NY + q]; }
      for (int q = 0; q < CS_NP; ++q) pl[q] = bt.p[(size_t)b * CS_NP + q];
      double r[CS_NY + CS_NP];
      cs_r(ya, yb, pl, th, r);
      cs_Dr(ya, yb, pl, th, Dr);
      for (int q = 0; q < CS_NY + CS_NP; ++q) top[(size_t)CS_NT * CS_TLD + CS_NY + q] = -r[q];
    }
    __syncthreads();
    for (int e = tid; e < CS_NT * CS_NT; e += nt) {
      const int c = e / CS_NT, r = e - c * CS_NT;
      double v;
      if (r < CS_NY) v = (c < 2 * CS_NY + CS_NPE) ? row[c * CS_NY + r] : 0.0;
      else v = Dr[(r - CS_NY) * (2 * CS_NY + CS_NP) + c];
      top[(size_t)c * CS_TLD + r] = v;
    }
    for (int r = tid; r < CS_NY; r += nt) top[(size_t)CS_NT * CS_TLD + r] = row[(2 * CS_NY + CS_NPE) * CS_NY + r];
    if (dyk != nullptr) {
      for (int q = tid; q < CS_NY + CS_NP; q += nt) {
        const double* dr = Dr + (size_t)q * (2 * CS_NY + CS_NP);
        double v = top[(size_t)CS_NT * CS_TLD + CS_NY + q];
        for (int c = 0; c < CS_NY; ++c) v = fma(-dr[c], dyk[(size_t)off * CS_NY + c], v);
        for (int c = 0; c < CS_NY; ++c) v = fma(-dr[CS_NY + c], dyk[(size_t)(off + N - 1) * CS_NY + c], v);
        for (int c = 0; c < CS_NP; ++c) v = fma(-dr[2 * CS_NY + c], dpk[(size_t)b * CS_NP + c], v);
        top[(size_t)CS_NT * CS_TLD + CS_NY + q] = v;
      }
    }
    __syncthreads();
#pragma unroll 1
    for (int kk = 0; kk < CS_NT; ++kk) cs_householder_cta(top, CS_TLD, CS_NT, CS_NT + 1, kk, red);
    // back substitution, column-oriented
    double* rhs = top + (size_t)CS_NT * CS_TLD;
    bool sing = false;
#pragma unroll 1
    for (int r = CS_NT - 1; r >= 0; --r) {
      const double d = top[(size_t)r * CS_TLD + r];
      sing |= (d == 0.0);
      const double xr = (d != 0.0) ? rhs[r] / d : 0.0;
      __syncthreads();
      if (tid == 0) rhs[r] = xr;
      for (int q = tid; q < r; q += nt) rhs[q] = fma(-top[(size_t)r * CS_TLD + q], xr, rhs[q]);
      __syncthreads();
    }
    if (tid == 0) {
      if (sing) {
        for (int r = 0; r < CS_NT; ++r) rhs[r] = 0.0;
        bt.inst[b].singular += 1;
      }
    }
    __syncthreads();
    for (int q = tid; q < CS_NY; q += nt) {
      bt.dy[(size_t)off * CS_NY + q] = rhs[q];
      bt.dy[(size_t)(off + N - 1) * CS_NY + q] = rhs[CS_NY + q];
    }
    for (int q = tid; q < CS_NP; q += nt) bt.dp[(size_t)b * CS_NP + q] = rhs[2 * CS_NY + q];
    if (tid == 0) {
      bt.inst[b].status = ST_LS;
      bt.inst[b].alpha_ls = 1.0;
      bt.inst[b].ls_it = 0;
    }
    __syncthreads();
  }
}

extern "C" __global__ void __launch_bounds__(256) k_top(CsBatch bt) {
  extern __shared__ double smem[];
  if (!cs_big_ok(bt, CS_WS_TOP, CS_SM_TOP)) return;
  cs_top_big(bt, smem, nullptr, nullptr);
}

#if CS_PREC_TREE != 0
// FP64 iterative refinement of the Newton direction when the tree merges run
// on the tensor cores: the condensed system M d = b is solved by the
// low-precision tree (relative error ~1e-2), so each sweep forms the FP64
// residual of the saved condensed blocks [A C H b] at the current (dy, dp),
// solves M c = residual with the same tree, top and back substitution, and
// adds c.  A sweep multiplies the direction's error by about the tree's own.
//
// k_refine_residual: for every interval of an instance on the Newton list,
// rows0 = [A C H rho] with rho = b - A dy_i - C dy_{i+1} - H dp (FP64, from
// `keep`, the condensation's output); (dy, dp) saved in (dyk, dpk).
extern "C" __global__ void k_refine_residual(CsBatch bt, const double* __restrict__ keep, double* dyk, double* dpk) {
  const int wpc = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int njac = bt.nlist[1];
  const long long total = bt.jac_pre[njac];
  for (long long it = (long long)blockIdx.x * wpc + w; it < total; it += (long long)gridDim.x * wpc) {
    const int k = cs_find(bt.jac_pre, njac, it);
    const int b = bt.jac[k];
    const int i = (int)(it - bt.jac_pre[k]);
    const int slot = bt.off[b] + i;
    const double* src = keep + (size_t)slot * CS_ROWSZ;
    double* dst = bt.rows0 + (size_t)slot * CS_ROWSZ;
    const double* yl = bt.dy + (size_t)slot * CS_NY;
    const double* yr = yl + CS_NY;
    const double* dpv = bt.dp + (size_t)b * CS_NP;
    for (int q = lane; q < (2 * CS_NY + CS_NPE) * CS_NY; q += 32) dst[q] = src[q];
    for (int a = lane; a < CS_NY; a += 32) {
      double v = src[(size_t)(2 * CS_NY + CS_NPE) * CS_NY + a];
      for (int c = 0; c < CS_NY; ++c) v = fma(-src[(size_t)c * CS_NY + a], yl[c], v);
      for (int c = 0; c < CS_NY; ++c) v = fma(-src[(size_t)(CS_NY + c) * CS_NY + a], yr[c], v);
      for (int c = 0; c < CS_NPE; ++c) v = fma(-src[(size_t)(2 * CS_NY + c) * CS_NY + a], dpv[c], v);
      dst[(size_t)(2 * CS_NY + CS_NPE) * CS_NY + a] = v;
      dyk[(size_t)slot * CS_NY + a] = yl[a];
      if (i == bt.N[b] - 2) dyk[(size_t)(slot + 1) * CS_NY + a] = yr[a];
    }
    if (i == 0)
      for (int c = lane; c < CS_NP; c += 32) dpk[(size_t)b * CS_NP + c] = dpv[c];
  }
}

// the boundary rows of the correction solve (cs_top_big with dyk, dpk)
extern "C" __global__ void __launch_bounds__(256) k_top_refine(CsBatch bt, const double* dyk, const double* dpk) {
  extern __shared__ double smem[];
  if (!cs_big_ok(bt, CS_WS_TOP, CS_SM_TOP)) return;
  cs_top_big(bt, smem, dyk, dpk);
}

// (dy, dp) = saved direction + correction
extern "C" __global__ void k_refine_add(CsBatch bt, const double* dyk, const double* dpk) {
  const int wpc = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int njac = bt.nlist[1];
  const long long total = bt.jac_pre[njac];
  for (long long it = (long long)blockIdx.x * wpc + w; it < total; it += (long long)gridDim.x * wpc) {
    const int k = cs_find(bt.jac_pre, njac, it);
    const int b = bt.jac[k];
    const int i = (int)(it - bt.jac_pre[k]);
    const int slot = bt.off[b] + i;
    for (int a = lane; a < CS_NY; a += 32) {
      bt.dy[(size_t)slot * CS_NY + a] += dyk[(size_t)slot * CS_NY + a];
      if (i == bt.N[b] - 2) bt.dy[(size_t)(slot + 1) * CS_NY + a] += dyk[(size_t)(slot + 1) * CS_NY + a];
    }
    if (i == 0)
      for (int c = lane; c < CS_NP; c += 32) bt.dp[(size_t)b * CS_NP + c] += dpk[(size_t)b * CS_NP + c];
  }
}
#endif  // CS_PREC_TREE != 0
#endif  // CS_BIG_TREE
#endif  // CS_BIG

// ------------------------------------------------------------------------
// Segment residual at the M+1 Gauss points and |r|_inf / tol in the last
// node's slot (compute_segment_residual_kernel, ..._kernel2 of
// collocation_solver_parallel_2d_shared.py:1833-2013):
//   rtype 1 (default): weighted sum of |f - y'| and |g|; 2: weighted squares,
//   square root at the end; 0: weighted maximum, whose g part takes |f - y'|
//   of the first nz components (as the reference does); with `scale` the
//   running value is multiplied by h after each component.
//   res2: max over points and components of |f - y'| / (1 + max |y'|) and
//   |g| / (1 + max |z|) (the maxima over the interval's Gauss points).
__device__ __forceinline__ void cs_gauss_point(const double* yi, const double* yd, const double* zz, double h, int gi,
                                               double* yv, double* ydv, double* zv) {
  for (int k = 0; k < CS_NY; ++k) {
    double sl = 0.0, si = 0.0;
    for (int q = 0; q < CS_M; ++q) {
      sl += CS_GL[gi * CS_M + q] * yd[q * CS_NY + k];
      si += CS_GI[gi * CS_M + q] * yd[q * CS_NY + k];
    }
    ydv[k] = sl;
    yv[k] = yi[k] + h * si;
  }
  for (int k = 0; k < CS_NZ; ++k) {
    double sl = 0.0;
    for (int q = 0; q < CS_M; ++q) sl += CS_GL[gi * CS_M + q] * zz[q * CS_NZ + k];
    zv[k] = sl;
  }
}

extern "C" __global__ void k_segres(CsBatch bt, double tol, int rtype, int scale, int res2) {
  int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= bt.T) return;
  int b = bt.inst_of[slot];
  int i = slot - bt.off[b];
  int N = bt.N[b];
  if (bt.inst[b].status != ST_SEG) return;
  const double* th = bt.th + (size_t)b * (CS_NTH > 0 ? CS_NTH : 1);
  double pl[CS_NP > 0 ? CS_NP : 1];
  for (int k = 0; k < CS_NP; ++k) pl[k] = bt.p[(size_t)b * CS_NP + k];
  double val;
  if (i < N - 1) {
    const double h = bt.t[slot + 1] - bt.t[slot];
    const double* yi = bt.y + (size_t)slot * CS_NY;
    const double* yd = bt.ydot + (size_t)slot * CS_M * CS_NY;
    const double* zz = bt.zt + (size_t)slot * CS_M * CS_NZ;
    double rho_h = 0.0, rho_g = 0.0;
    double yv[CS_NY], ydv[CS_NY], zv[CS_NZ > 0 ? CS_NZ : 1], f[CS_NY];
    if (res2) {
      double ydg[CS_NY], zg[CS_NZ > 0 ? CS_NZ : 1];
      for (int k = 0; k < CS_NY; ++k) ydg[k] = 0.0;
      for (int k = 0; k < CS_NZ; ++k) zg[k] = 0.0;
#pragma unroll 1
      for (int gi = 0; gi < CS_M + 1; ++gi) {
        cs_gauss_point(yi, yd, zz, h, gi, yv, ydv, zv);
        for (int k = 0; k < CS_NY; ++k) ydg[k] = fmax(ydg[k], fabs(ydv[k]));
        for (int k = 0; k < CS_NZ; ++k) zg[k] = fmax(zg[k], fabs(zv[k]));
      }
#pragma unroll 1
      for (int gi = 0; gi < CS_M + 1; ++gi) {
        cs_gauss_point(yi, yd, zz, h, gi, yv, ydv, zv);
        cs_f(yv, zv, pl, th, f);
        for (int k = 0; k < CS_NY; ++k) rho_h = fmax(rho_h, fabs(f[k] - ydv[k]) / (1.0 + ydg[k]));
#if CS_NZ > 0
        double g[CS_NZ];
        cs_g(yv, zv, pl, th, bt.inst[b].alpha, g);
        for (int k = 0; k < CS_NZ; ++k) rho_g = fmax(rho_g, fabs(g[k]) / (1.0 + zg[k]));
#endif
      }
      val = fmax(rho_h, rho_g) / tol;
    } else {
#pragma unroll 1
      for (int gi = 0; gi < CS_M + 1; ++gi) {
        cs_gauss_point(yi, yd, zz, h, gi, yv, ydv, zv);
        cs_f(yv, zv, pl, th, f);
        const double wgt = CS_GW[gi];
        for (int k = 0; k < CS_NY; ++k) {
          const double r = f[k] - ydv[k];
          if (rtype == 2) rho_h += wgt * r * r;
          else if (rtype == 1) rho_h += wgt * fabs(r);
          else rho_h = fmax(rho_h, wgt * fabs(r));
          if (scale) rho_h *= h;
        }
#if CS_NZ > 0
        double g[CS_NZ];
        cs_g(yv, zv, pl, th, bt.inst[b].alpha, g);
        for (int k = 0; k < CS_NZ; ++k) {
          if (rtype == 2) rho_g += wgt * g[k] * g[k];
          else if (rtype == 1) rho_g += wgt * fabs(g[k]);
          else rho_g = fmax(rho_g, wgt * (k < CS_NY ? fabs(f[k] - ydv[k]) : 0.0));
          if (scale) rho_g *= h;
        }
#endif
      }
      if (rtype == 2) val = sqrt(rho_h + rho_g) / tol;
      else if (rtype == 1) val = (fabs(rho_h) + fabs(rho_g)) / tol;
      else val = fmax(rho_h, rho_g) / tol;
    }
  } else {
    double ya[CS_NY], yb[CS_NY], r[CS_NY + CS_NP];
    const int first = bt.off[b];
    for (int k = 0; k < CS_NY; ++k) { ya[k] = bt.y[(size_t)first * CS_NY + k]; yb[k] = bt.y[(size_t)slot * CS_NY + k]; }
    cs_r(ya, yb, pl, th, r);
    double mx = 0.0;
    for (int k = 0; k < CS_NY + CS_NP; ++k) mx = fmax(mx, fabs(r[k]));
    val = mx / tol;
  }
  bt.res[slot] = val;
  unsigned long long bits = (val != val) ? 0x7ff8000000000000ull : cs_abs_bits(val);
  atomicMax(&bt.inst[b].res_bits, bits);
}

// after k_segres: accept the mesh, continue the continuation, or ask for a remesh
extern "C" __global__ void k_mesh_decide(CsBatch bt, CsConsts c) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= bt.B) return;
  CsInst s = bt.inst[b];
  if (s.status != ST_SEG) return;
  s.max_res = cs_from_bits(s.res_bits);
  s.res_bits = 0ull;
  s.seg_count += 1;
  if (s.max_res > 1.0) {
    s.status = ST_REMESH;
  } else if (s.alpha <= c.alpha_m) {
    s.status = ST_DONE;
  } else {
    s.alpha *= c.beta;
    s.alphacal += 1;
    s.status = ST_FRESH;
    s.it = 0;
  }
  bt.inst[b].max_res = s.max_res;
  bt.inst[b] = s;
}

// ------------------------------------------------------------------------
// Remesh (collocation_solver_parallel_2d_shared.py:2106-2311), one thread per
// instance.  Pass 1 counts the new nodes; pass 2 writes t, y and z-at-node
// into the new packed arrays.  Deletion: five consecutive residuals <= 1e-2
// keep the 1st, 3rd and 5th node; insertion: residual > 10 adds three
// equispaced nodes, > 1 the midpoint; y and z are interpolated linearly.
__device__ __forceinline__ void cs_znode(const CsBatch& bt, int off, int N, int i, double* z) {
  if (i < N - 1) {
    const double* zz = bt.zt + (size_t)(off + i) * CS_M * CS_NZ;
    for (int k = 0; k < CS_NZ; ++k) {
      double s = 0.0;
      for (int q = 0; q < CS_M; ++q) s += CS_L0[q] * zz[q * CS_NZ + k];
      z[k] = s;
    }
  } else {
    const double* zz = bt.zt + (size_t)(off + N - 2) * CS_M * CS_NZ;
    for (int k = 0; k < CS_NZ; ++k) {
      double s = 0.0;
      for (int q = 0; q < CS_M; ++q) s += CS_L1[q] * zz[q * CS_NZ + k];
      z[k] = s;
    }
  }
}

// iterate the nodes kept by the deletion pass; calls fn(kept_index)
template <typename F>
__device__ void cs_kept_nodes(const double* res, int N, F fn) {
  int i = 0;
  while (i < N - 4) {
    if (res[i] <= 1e-2 && res[i + 1] <= 1e-2 && res[i + 2] <= 1e-2 && res[i + 3] <= 1e-2 && res[i + 4] <= 1e-2) {
      fn(i); fn(i + 2); fn(i + 4);
      i += 5;
    } else {
      fn(i);
      i += 1;
    }
  }
  while (i < N) { fn(i); i += 1; }
}

extern "C" __global__ void k_remesh_count(CsBatch bt) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= bt.B) return;
  if (bt.inst[b].status != ST_REMESH) { bt.inst[b].N_new = bt.N[b]; return; }
  const int N = bt.N[b];
  const double* res = bt.res + bt.off[b];
  int cnt = 0, prev = -1;
  cs_kept_nodes(res, N, [&](int k) {
    if (prev >= 0) {
      double r = res[prev];
      cnt += (r > 10.0) ? 4 : (r > 1.0 ? 2 : 1);
    }
    prev = k;
  });
  bt.inst[b].N_new = cnt + 1;
}

// new arrays: t2, y2, z2 (z at nodes) at offsets off2
extern "C" __global__ void k_remesh_write(CsBatch bt, const int* off2, double* t2, double* y2, double* z2) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= bt.B) return;
  if (bt.inst[b].status != ST_REMESH) return;
  const int N = bt.N[b], off = bt.off[b];
  const double* res = bt.res + off;
  int o = off2[b];
  int prev = -1;
  auto emit = [&](int a, int bnode, int q) {
    // node a itself, then q-1 interpolated nodes towards bnode
    double za[CS_NZ > 0 ? CS_NZ : 1], zb[CS_NZ > 0 ? CS_NZ : 1];
    cs_znode(bt, off, N, a, za);
    cs_znode(bt, off, N, bnode, zb);
    const double ta = bt.t[off + a], tb = bt.t[off + bnode];
    const double dt = (tb - ta) / (double)q;
    t2[o] = ta;
    for (int k = 0; k < CS_NY; ++k) y2[(size_t)o * CS_NY + k] = bt.y[(size_t)(off + a) * CS_NY + k];
    for (int k = 0; k < CS_NZ; ++k) z2[(size_t)o * CS_NZ + k] = za[k];
    ++o;
    for (int s = 1; s < q; ++s) {
      t2[o] = __dadd_rn(ta, __dmul_rn((double)s, dt));
      for (int k = 0; k < CS_NY; ++k) {
        const double ya = bt.y[(size_t)(off + a) * CS_NY + k], yb = bt.y[(size_t)(off + bnode) * CS_NY + k];
        y2[(size_t)o * CS_NY + k] = __dadd_rn(ya, __dmul_rn((double)s, (yb - ya) / (double)q));
      }
      for (int k = 0; k < CS_NZ; ++k) z2[(size_t)o * CS_NZ + k] = __dadd_rn(za[k], __dmul_rn((double)s, (zb[k] - za[k]) / (double)q));
      ++o;
    }
  };
  cs_kept_nodes(res, N, [&](int k) {
    if (prev >= 0) {
      double r = res[prev];
      emit(prev, k, (r > 10.0) ? 4 : (r > 1.0 ? 2 : 1));
    }
    prev = k;
  });
  emit(prev, prev, 1);
}

// copy an unchanged instance into the new packed layout
extern "C" __global__ void k_repack(CsBatch bt, const int* off2, double* t2, double* y2, double* ydot2, double* zt2) {
  int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= bt.T) return;
  int b = bt.inst_of[slot];
  if (bt.inst[b].status == ST_REMESH) return;
  int i = slot - bt.off[b];
  int d = off2[b] + i;
  t2[d] = bt.t[slot];
  for (int k = 0; k < CS_NY; ++k) y2[(size_t)d * CS_NY + k] = bt.y[(size_t)slot * CS_NY + k];
  if (i < bt.N[b] - 1) {
    for (int q = 0; q < CS_M * CS_NY; ++q) ydot2[(size_t)d * CS_M * CS_NY + q] = bt.ydot[(size_t)slot * CS_M * CS_NY + q];
    for (int q = 0; q < CS_M * CS_NZ; ++q) zt2[(size_t)d * CS_M * CS_NZ + q] = bt.zt[(size_t)slot * CS_M * CS_NZ + q];
  }
}

// z at every node (output / diagnostics)
extern "C" __global__ void k_znodes(CsBatch bt) {
  int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= bt.T) return;
  int b = bt.inst_of[slot];
  double z[CS_NZ > 0 ? CS_NZ : 1];
  cs_znode(bt, bt.off[b], bt.N[b], slot - bt.off[b], z);
  for (int k = 0; k < CS_NZ; ++k) bt.znode[(size_t)slot * CS_NZ + k] = z[k];
}
