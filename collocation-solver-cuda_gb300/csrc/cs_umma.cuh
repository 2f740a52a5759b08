// Fifth-generation tensor cores (tcgen05, sm_100a / sm_103a): the block update
//
//     C[0:M, 0:N] -= A[0:M, 0:K] * B[0:N, 0:K]^T        (C in FP32)
//
// with A and B staged in shared memory as BF16 (kind::f16) or TF32
// (kind::tf32) and the products accumulated in FP32 in tensor memory (TMEM),
// one 128-row tile of A and up to 256 columns of B per group of MMAs.  It is
// the trailing update of the reduced-precision blocked LU of the large stage
// systems (cs_kernels.cuh) and of the standalone entry point cs_tc_update
// (cs_tc.cu), both through cs_tc_block_update.  This file holds device code
// only and is compiled both by nvcc (into the library) and by NVRTC (in
// front of cs_kernels.cuh).
//
// Operand layout in shared memory (canonical K-major layout without swizzle):
// 8-row x 16-byte core matrices; element (r, k) of an operand with `kc` core
// matrices along K lies at byte
//     ((r / 8) * kc + (kbyte / 16)) * 128 + (r % 8) * 16 + kbyte % 16,
// kbyte = k * (element size): the core matrices of one 8-row group follow
// each other along K (leading byte offset 128), the 8-row groups are
// kc * 128 bytes apart (stride byte offset).  One MMA consumes 32 bytes of K
// (16 BF16 or 8 TF32 elements: two core matrices), so k-step s starts 256 s
// bytes after the tile's first core matrix.  Rows past M (N) must be staged
// as zeros up to the next multiple of 128 (16), columns past K up to the
// k-steps used.
//
// Synchronisation: operands are written by the threads, made visible to the
// tensor core (fence.proxy.async) and published with __syncthreads; thread 0
// issues the MMAs and commits them to an mbarrier; every thread waits on the
// barrier's phase (bounded: an error is reported instead of hanging) and
// reads its row of the accumulator (warp w reads TMEM lanes 32 (w % 4) ..);
// a tcgen05 fence pair around __syncthreads orders those reads before the
// next group of MMAs overwrites the accumulator.
#ifndef CS_UMMA_CUH
#define CS_UMMA_CUH

#define CS_TC_COLS 256  // TMEM columns a CTA allocates (two CTAs fit on one SM)

// 32-bit shared-memory address of a generic pointer into shared memory
__device__ __forceinline__ unsigned cs_sa(const void* p) {
  unsigned r;
  asm volatile("{\n\t.reg .u64 t;\n\tcvta.to.shared.u64 t, %1;\n\tcvt.u32.u64 %0, t;\n\t}" : "=r"(r) : "l"(p));
  return r;
}

// shared-memory matrix descriptor: start address, leading / stride byte
// offsets (all >> 4), descriptor version 1 (bits 46-47), no swizzle
__device__ __forceinline__ unsigned long long cs_tc_desc(unsigned saddr, unsigned lbo, unsigned sbo) {
  return (unsigned long long)((saddr & 0x3FFFFu) >> 4) | ((unsigned long long)((lbo & 0x3FFFFu) >> 4) << 16) |
         ((unsigned long long)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// instruction descriptor: FP32 accumulator (bits 4-5 = 1), A and B format
// (bits 7-9, 10-12: 1 BF16 under kind::f16, 2 TF32 under kind::tf32), both
// K-major (bits 15, 16 = 0), N / 8 (bits 17-22), M / 16 (bits 24-28)
__device__ __forceinline__ unsigned cs_tc_idesc(int prec, int M, int N) {
  const unsigned fmt = (prec == 1) ? 2u : 1u;
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

// D (TMEM) [+]= A B^T for one k-step; prec 1: TF32, 2: BF16
template <int PREC>
__device__ __forceinline__ void cs_tc_mma(unsigned tmem, unsigned long long ad, unsigned long long bd, unsigned idesc,
                                          int accumulate) {
  if constexpr (PREC == 1) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate) : "memory");
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate) : "memory");
  }
}

// the MMAs issued so far by this thread arrive on the mbarrier when done
__device__ __forceinline__ void cs_tc_commit(unsigned mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void cs_tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void cs_tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy writes to shared memory become visible to the tensor core
__device__ __forceinline__ void cs_fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void cs_mbar_init(unsigned mbar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool cs_mbar_test(unsigned mbar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(mbar), "r"(phase)
      : "memory");
  return ok != 0;
}

// wait for the barrier phase `phase` to complete; false after about
// `limit` clock cycles without completion (the caller reports an error)
__device__ __forceinline__ bool cs_mbar_wait(unsigned mbar, unsigned phase, long long limit) {
  const long long t0 = clock64();
  while (!cs_mbar_test(mbar, phase))
    if (clock64() - t0 > limit) return false;
  return true;
}

// TMEM allocation / release: one full warp; the address lands in *slot
__device__ __forceinline__ void cs_tmem_alloc(unsigned slot, unsigned ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols) : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void cs_tmem_free(unsigned taddr, unsigned ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void cs_tmem_ld16(unsigned taddr, float* v) {
  unsigned r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// operand element conversions (FP32 -> TF32 rounded to nearest, ties away;
// FP32 pair -> BF16 pair rounded to nearest even, lo in the low half)
__device__ __forceinline__ unsigned cs_tc_tf32(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ unsigned cs_tc_bf2(float lo, float hi) {
  unsigned r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

// byte offset of the 16-byte segment (row r, K segment q) of an operand with
// kc core matrices along K
__device__ __forceinline__ unsigned cs_tc_seg(int r, int q, int kc) {
  return (unsigned)((((r >> 3) * kc + q) << 7) + ((r & 7) << 4));
}

// Stage one 16-byte segment: the 8 (BF16) or 4 (TF32) FP32 values x[0..] of
// row r, K segment q, rounded for the tensor core.
template <int PREC>
__device__ __forceinline__ void cs_tc_put(unsigned char* base, int r, int q, int kc, const float* x) {
  uint4 v;
  if constexpr (PREC == 1) {
    v.x = cs_tc_tf32(x[0]);
    v.y = cs_tc_tf32(x[1]);
    v.z = cs_tc_tf32(x[2]);
    v.w = cs_tc_tf32(x[3]);
  } else {
    v.x = cs_tc_bf2(x[0], x[1]);
    v.y = cs_tc_bf2(x[2], x[3]);
    v.z = cs_tc_bf2(x[4], x[5]);
    v.w = cs_tc_bf2(x[6], x[7]);
  }
  *reinterpret_cast<uint4*>(base + cs_tc_seg(r, q, kc)) = v;
}

// FP32 values per 16-byte segment
template <int PREC>
struct CsTcElems {
  static constexpr int per_seg = (PREC == 1) ? 4 : 8;
};

// C[0:M, 0:N] -= A B^T, all threads of the CTA (blockDim.x a multiple of
// 128); A_s, B_s staged as described above with kc core matrices along K and
// nks k-steps; element (r, c) of C at C[r * rs + c * cs] (global or shared
// memory).  A thread updates one row of C (its TMEM lane), so with C
// column-major (rs = 1, cs = its leading dimension) a warp's accesses to one
// column are one contiguous 128-byte line.  tmem: the
// CTA's CS_TC_COLS accumulator columns; mbar / phase: the CTA's barrier and
// its next phase.  Returns false (on every thread) if an MMA group did not
// complete within `limit` cycles; the caller reports it and must not reuse
// the operands or the accumulator.
template <int PREC>
__device__ bool cs_tc_block_update(float* C, long long rs, long long cs, int M, int N, const unsigned char* A_s,
                             const unsigned char* B_s, int kc, int nks, unsigned tmem, unsigned mbar, unsigned& phase,
                             long long limit, int* flag_smem) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
  const int quad = w & 3, half = w >> 2, halves = nw >> 2;  // warps w and w + 4 share TMEM lanes
  const unsigned a0 = cs_sa(A_s), b0 = cs_sa(B_s);
  const unsigned sbo = (unsigned)kc << 7;
  const int mt = (M + 127) >> 7;
  bool ok = true;
  for (int n0 = 0; n0 < N && ok; n0 += CS_TC_COLS) {
    const int nch = min(CS_TC_COLS, N - n0);
    const int npad = (nch + 15) & ~15;
    const unsigned idesc = cs_tc_idesc(PREC, 128, npad);
    for (int t = 0; t < mt && ok; ++t) {
      if (tid == 0) {
        cs_tc_after_sync();
        for (int s = 0; s < nks; ++s) {
          const unsigned long long ad = cs_tc_desc(a0 + ((unsigned)(t * 16 * kc + 2 * s) << 7), 128u, sbo);
          const unsigned long long bd = cs_tc_desc(b0 + ((unsigned)((n0 >> 3) * kc + 2 * s) << 7), 128u, sbo);
          cs_tc_mma<PREC>(tmem, ad, bd, idesc, s > 0);
        }
        cs_tc_commit(mbar);
      }
      const bool done = cs_mbar_wait(mbar, phase, limit);
      phase ^= 1u;
      if (!done) *flag_smem = 1;
      cs_tc_after_sync();
      __syncthreads();
      if (*flag_smem) {
        ok = false;
        break;
      }
      // epilogue: thread (quad, lane) owns row t*128 + 32 quad + lane; the
      // warps sharing a quad split the 16-column groups
      const int row = t * 128 + quad * 32 + lane;
      const int groups = npad >> 4;
      for (int gi = half; gi < groups; gi += halves) {
        float v[16];
        cs_tmem_ld16(tmem + ((unsigned)(quad * 32) << 16) + (unsigned)(gi * 16), v);
        if (row < M) {
          // all 16 loads before the stores (they cannot alias each other, which
          // the compiler does not know): one memory latency per 16 columns
          float* cr = C + (long long)row * rs + (long long)(n0 + gi * 16) * cs;
          const int nv = min(16, nch - gi * 16);
          float c[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) c[j] = (j < nv) ? cr[j * cs] : 0.f;
#pragma unroll
          for (int j = 0; j < 16; ++j)
            if (j < nv) cr[j * cs] = c[j] - v[j];
        }
      }
      cs_tc_before_sync();
      __syncthreads();
    }
  }
  return ok;
}

#endif  // CS_UMMA_CUH
