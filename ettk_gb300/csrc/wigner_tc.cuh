// Wigner-d synthesis of the SO(3) correlation on the 5th-generation tensor cores (tcgen05).
//
// For one (m1, m2) cell the synthesis S[job][b] = sum_l F^l_{m1m2}[job] d~^l_{m1m2}(beta_b) is a GEMM:
// M = 128 rows (the real parts of 64 jobs, then their imaginary parts), N = 2B (the beta samples),
// K = the degrees l >= max(|m1|, |m2|), zero-padded to KP. Operands are staged in shared memory in the
// canonical no-swizzle K-major layout (8-row x 16-byte core matrices), the accumulator lives in tensor
// memory (FP32, 128 lanes x 2B columns), one elected thread issues tcgen05.mma, completion is signalled
// through tcgen05.commit on an mbarrier, and the epilogue reads the accumulator back with tcgen05.ld.
//
// Precision modes (the contraction only; everything around it stays FP32):
//   WIG_BF16   BF16 operands, FP32 accumulation (1 MMA per K step)
//   WIG_SPLIT  split BF16: x = hi + lo, hi*hi + lo*hi + hi*lo, FP32 accumulation (3 MMAs per K step)
//   WIG_TF32   TF32 operands (round to nearest), FP32 accumulation
// Same combination rule and output layout as k_so3_synth (so3CombineCoef_fftw, so3_correlate_fftw.c:103-162;
// the inverse Wigner transform of Inverse_SO3_Naive_fftw, soft_fftw.c:1045-1840).
#pragma once
#include <cuda_bf16.h>
#include "kernels.cuh"

namespace ettk {

enum WigPrecision { WIG_FP32 = 0, WIG_BF16 = 1, WIG_SPLIT = 2, WIG_TF32 = 3, WIG_FP64 = 4 };

template <int B, int MODE>
struct WigTC {
  static constexpr int n = 2 * B;                     // GEMM N (beta samples)
  static constexpr int KP = B < 16 ? 16 : B;          // padded K (degrees)
  static constexpr int KE = MODE == WIG_TF32 ? 4 : 8; // elements per 16-byte core-matrix row
  static constexpr int ESZ = MODE == WIG_TF32 ? 4 : 2;
  static constexpr int KSTEP = 32 / ESZ;              // K per MMA (32 bytes of K)
  static constexpr int NOPS = MODE == WIG_SPLIT ? 2 : 1;  // hi (+ lo) copies of each operand
  static constexpr size_t A_BYTES = (size_t)128 * KP * ESZ, B_BYTES = (size_t)n * KP * ESZ;
  static constexpr int NCOL = n < 32 ? 32 : n;        // tensor-memory columns (power of two >= 32)
  // dynamic shared memory: operands, raised so that at most 512 / NCOL CTAs share an SM's tensor memory
  static constexpr size_t OPS = NOPS * (A_BYTES + B_BYTES);
  static constexpr size_t CAP = (size_t)228 * 1024 * NCOL / 512 + 1024;
  static constexpr size_t SMEM = OPS > CAP ? OPS : CAP;
  static_assert(n % 16 == 0 && n <= 256, "tensor-core N");
  static_assert(SMEM >= (size_t)64 * 33 * sizeof(float), "epilogue staging fits the operand area");
};

// kind::f16 / kind::tf32 instruction descriptor: D f32 (bits 4-5), A/B format (7-9, 10-12: BF16 1, TF32 2),
// both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
template <int MODE>
__host__ __device__ constexpr uint32_t wig_idesc(int M, int N) {
  return (1u << 4) | ((MODE == WIG_TF32 ? 2u : 1u) << 7) | ((MODE == WIG_TF32 ? 2u : 1u) << 10) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// Shared-memory matrix descriptor, no swizzle: start >> 4, LBO (between core matrices along K) >> 4 at 16,
// SBO (between 8-row groups) >> 4 at 32, descriptor version 1 at bit 46.
ETTK_DEV uint64_t wig_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46);
}
template <int MODE>
ETTK_DEV void wig_mma(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t accumulate) {
  if (MODE == WIG_TF32)
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
        : "memory");
  else
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
        : "memory");
}

// KE consecutive K elements of one operand row (x[0..KE-1]) as the hi (part 0) or lo (part 1) copy of the mode,
// packed into the 16-byte core-matrix row they occupy
template <int MODE, int KE>
ETTK_DEV uint4 wig_pack(const float *x, int part) {
  uint32_t w[4];
  if (MODE == WIG_TF32) {
#pragma unroll
    for (int e = 0; e < 4; ++e) asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(w[e]) : "f"(x[e]));
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      __nv_bfloat16 h[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const float v = x[2 * e + u];
        const __nv_bfloat16 hi = __float2bfloat16(v);
        h[u] = part == 0 ? hi : __float2bfloat16(v - __bfloat162float(hi));
      }
      w[e] = (uint32_t)__bfloat16_as_ushort(h[0]) | ((uint32_t)__bfloat16_as_ushort(h[1]) << 16);
    }
  }
  return make_uint4(w[0], w[1], w[2], w[3]);
}

// grid (cells, ceil(n_jobs / 64)), 128 threads; coef [signal][l][m >= 0], S [job][m1 mod n][m2 mod n][b].
// A barrier that does not complete within the poll limit sets *status and leaves this tile's output unwritten.
// Every shared-memory store is bank-conflict free: each thread writes whole 16-byte core-matrix rows, the eight
// lanes that fill one core matrix (rows r..r+7) covering its 128 contiguous bytes, and the epilogue staging rows
// have a pitch of 33 floats.
template <int B, int MODE>
__global__ void __launch_bounds__(128) k_so3_synth_tc(const float2 *__restrict__ coef, const SynthJob *__restrict__ jobs,
                                                      int n_jobs, const float *__restrict__ dtab,
                                                      const int *__restrict__ doff, float2 *__restrict__ S,
                                                      int *status) {
  using T = WigTC<B, MODE>;
  constexpr int n = T::n, KP = T::KP, KE = T::KE, KC = KP / KE;
  extern __shared__ __align__(1024) unsigned char wig_sm[];
  unsigned char *A0 = wig_sm, *A1 = wig_sm + T::A_BYTES;                                  // A1 only for WIG_SPLIT
  unsigned char *B0 = wig_sm + T::NOPS * T::A_BYTES, *B1 = B0 + T::B_BYTES;            // B1 only for WIG_SPLIT
  __shared__ __align__(8) unsigned long long bar;
  __shared__ uint32_t tbase;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int cell = blockIdx.x, j0 = blockIdx.y * 64;
  const int m1 = cell / (2 * B - 1) - (B - 1), m2 = cell % (2 * B - 1) - (B - 1);
  const int l0 = max(abs(m1), abs(m2)), L = B - l0;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tbase)),
                 "r"((uint32_t)T::NCOL)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) mbar_init(&bar, 1);
  // A: F = f(l,-m1) conj(h(l,-m2)) (-1)^(m1+m2); rows 0..63 real, 64..127 imaginary; zero beyond L and n_jobs.
  // Item i: job row jl = i % 64 (fastest, so that eight lanes fill one core matrix), K chunk tc = i / 64.
  const float sgn = ((m1 + m2) & 1) ? -1.f : 1.f;
  for (int i = tid; i < 64 * KC; i += blockDim.x) {
    const int jl = i & 63, tc = i >> 6, j = j0 + jl;
    float re[KE], im[KE];
    const bool live = j < n_jobs;
    SynthJob jb{};
    if (live) jb = jobs[j];
#pragma unroll
    for (int e = 0; e < KE; ++e) {
      const int t = tc * KE + e;
      float2 F = make_float2(0.f, 0.f);
      if (live && t < L) {
        const float2 a = coef_at(coef + (long)jb.f * B * B, B, l0 + t, -m1);
        const float2 b = coef_at(coef + (long)jb.h * B * B, B, l0 + t, -m2);
        F = cscale(cmul(a, cconj(b)), sgn);
      }
      re[e] = F.x;
      im[e] = F.y;
    }
    const int cr = ((jl >> 3) * KC + tc) * 8 + (jl & 7), ci = (((64 + jl) >> 3) * KC + tc) * 8 + (jl & 7);
    reinterpret_cast<uint4 *>(A0)[cr] = wig_pack<MODE, KE>(re, 0);
    reinterpret_cast<uint4 *>(A0)[ci] = wig_pack<MODE, KE>(im, 0);
    if (MODE == WIG_SPLIT) {
      reinterpret_cast<uint4 *>(A1)[cr] = wig_pack<MODE, KE>(re, 1);
      reinterpret_cast<uint4 *>(A1)[ci] = wig_pack<MODE, KE>(im, 1);
    }
  }
  // B: d~^l(beta_b), row b, column t; item i: b = i % n, K chunk tc = i / n
  const float *d = dtab + doff[cell];
  for (int i = tid; i < n * KC; i += blockDim.x) {
    const int b = i % n, tc = i / n;
    float v[KE];
#pragma unroll
    for (int e = 0; e < KE; ++e) {
      const int t = tc * KE + e;
      v[e] = t < L ? d[t * n + b] : 0.f;
    }
    const int cb = ((b >> 3) * KC + tc) * 8 + (b & 7);
    reinterpret_cast<uint4 *>(B0)[cb] = wig_pack<MODE, KE>(v, 0);
    if (MODE == WIG_SPLIT) reinterpret_cast<uint4 *>(B1)[cb] = wig_pack<MODE, KE>(v, 1);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tm = tbase;
  if (tid == 0) {
    constexpr uint32_t LBO = 128, SBO = (KP / KE) * 128;
    constexpr uint32_t idesc = wig_idesc<MODE>(128, n);
    const uint32_t a0 = smem_addr(A0), a1 = smem_addr(A1), b0 = smem_addr(B0), b1 = smem_addr(B1);
    uint32_t acc = 0;
    for (int s = 0; s < KP / T::KSTEP; ++s) {
      const uint32_t o = s * 256;  // two core matrices (32 bytes of K) per step
      wig_mma<MODE>(tm, wig_sdesc(a0 + o, LBO, SBO), wig_sdesc(b0 + o, LBO, SBO), idesc, acc);
      acc = 1;
      if (MODE == WIG_SPLIT) {
        wig_mma<MODE>(tm, wig_sdesc(a1 + o, LBO, SBO), wig_sdesc(b0 + o, LBO, SBO), idesc, 1);
        wig_mma<MODE>(tm, wig_sdesc(a0 + o, LBO, SBO), wig_sdesc(b1 + o, LBO, SBO), idesc, 1);
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(&bar))
                 : "memory");
  }
  const bool mine = mbar_wait(&bar, 0, 1 << 22);
  if (!mine && lane == 0) atomicExch(status, 1);
  const bool ok = __syncthreads_and(mine);  // block-uniform: the epilogue below synchronises the CTA
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    // 16 accumulator columns (beta) at a time: tcgen05.ld of the thread's row (job jl, real or imaginary part),
    // staged in the operand area (free once the MMAs completed) as [jl][beta][re, im] with a row pitch of 33 floats
    // (the 32 lanes of a warp, 32 consecutive jl, store to 32 distinct banks), then written as whole
    // 128-byte runs S[job][m1][m2][beta .. beta + 15]
    const int row = warp * 32 + lane, jl = row & 63, comp = row >> 6;
    const int mm1 = (m1 + n) % n, mm2 = (m2 + n) % n;
    float *stg = reinterpret_cast<float *>(wig_sm);
#pragma unroll 1
    for (int c0 = 0; c0 < n; c0 += 16) {
      uint32_t r[16];
      const uint32_t addr = tm + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(addr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      __syncthreads();  // the previous chunk's stores have read the staging area
#pragma unroll
      for (int q = 0; q < 16; ++q) stg[jl * 33 + q * 2 + comp] = __uint_as_float(r[q]);
      __syncthreads();
      for (int t = tid; t < 64 * 16; t += blockDim.x) {
        const int jt = t >> 4, q = t & 15, j = j0 + jt;
        if (j < n_jobs)
          S[(((long)j * n + mm1) * n + mm2) * n + c0 + q] = make_float2(stg[jt * 33 + q * 2], stg[jt * 33 + q * 2 + 1]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tm), "r"((uint32_t)T::NCOL) : "memory");
}

// FP64 contraction (double table and accumulation) for the precision study: same cells and layout as
// k_so3_synth, one CTA per (cell, block of jobs).
template <int B>
__global__ void __launch_bounds__(256) k_so3_synth_f64(const float2 *__restrict__ coef, const SynthJob *__restrict__ jobs,
                                                      int n_jobs, const double *__restrict__ dtab,
                                                      const int *__restrict__ doff, float2 *__restrict__ S) {
  constexpr int n = 2 * B;
  const int cell = blockIdx.x;
  const int m1 = cell / (2 * B - 1) - (B - 1), m2 = cell % (2 * B - 1) - (B - 1);
  const int l0 = max(abs(m1), abs(m2)), L = B - l0;
  const double *d = dtab + doff[cell];
  const double sgn = ((m1 + m2) & 1) ? -1.0 : 1.0;
  const int mm1 = (m1 + n) % n, mm2 = (m2 + n) % n;
  for (int i = blockIdx.y * blockDim.x + threadIdx.x; i < n_jobs * n; i += gridDim.y * blockDim.x) {
    const int j = i / n, b = i - j * n;
    const SynthJob jb = jobs[j];
    double re = 0, im = 0;
    for (int t = 0; t < L; ++t) {
      const float2 a = coef_at(coef + (long)jb.f * B * B, B, l0 + t, -m1);
      const float2 c = coef_at(coef + (long)jb.h * B * B, B, l0 + t, -m2);
      const double fr = ((double)a.x * c.x + (double)a.y * c.y) * sgn, fi = ((double)a.y * c.x - (double)a.x * c.y) * sgn;
      re += fr * d[t * n + b];
      im += fi * d[t * n + b];
    }
    S[(((long)j * n + mm1) * n + mm2) * n + b] = make_float2((float)re, (float)im);
  }
}

}  // namespace ettk
