// Shared device helpers for the GB300 alignment kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cfloat>

#define ETTK_DEV __device__ __forceinline__
#define ETTK_HD __host__ __device__ __forceinline__

namespace ettk {

ETTK_DEV float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
ETTK_DEV float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
ETTK_DEV float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
ETTK_DEV float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
ETTK_DEV float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
ETTK_DEV float cabs2(float2 a) { return a.x * a.x + a.y * a.y; }

// (-1)^(i+j+k): the reference's centring "shift" arrays (inc/em/nbfFourierFilter.h:307-319)
ETTK_DEV float parity_sign(int i, int j, int k) { return ((i + j + k) & 1) ? -1.0f : 1.0f; }

// Order-preserving map of a float to uint32 (for packed atomic max of (value, index)).
ETTK_DEV uint32_t float_to_ordered(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
ETTK_DEV float ordered_to_float(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
// Larger value wins; on equal values the smaller index wins (first occurrence in scan order).
ETTK_DEV unsigned long long pack_max(float v, uint32_t idx) {
  return ((unsigned long long)float_to_ordered(v) << 32) | (unsigned long long)(0xffffffffu - idx);
}
ETTK_DEV unsigned long long pack_min(float v, uint32_t idx) {
  // smaller value wins -> negate ordering; smaller index wins
  return ((unsigned long long)(~float_to_ordered(v)) << 32) | (unsigned long long)(0xffffffffu - idx);
}

template <typename T>
ETTK_DEV T warp_sum(T v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of a double; result valid in thread 0. `sh` needs blockDim/32 doubles.
ETTK_DEV double block_sum(double v, double *sh) {
  v = warp_sum(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0;
  if (w == 0) {
    int nw = (blockDim.x + 31) >> 5;
    r = (lane < nw) ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

// Block-wide sums without FP64 arithmetic in the tree (on GB300 a warp-wide FP64 add occupies the SM's FP64 pipe
// for about as long as dozens of FP32 instructions, which made the FP64 tree the largest cost of short CTAs).
// FP32 values: each partial sum is carried as an unevaluated pair hi + lo, every addition split exactly into sum
// and rounding error (Knuth's TwoSum, rounded intrinsics so that no FMA contraction disturbs it), about 48
// significant bits; thread 0 gets hi + lo as a double. Agrees with an FP64 tree except in the last bits of the
// double. `sh` needs blockDim/32 float2.
ETTK_DEV float2 ff_add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bb = __fsub_rn(s, a.x);
  float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
  e = __fadd_rn(e, __fadd_rn(a.y, b.y));
  const float h = __fadd_rn(s, e);
  return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
}
ETTK_DEV float2 warp_sum_ff(float2 v) {
  for (int o = 16; o > 0; o >>= 1)
    v = ff_add(v, make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)));
  return v;
}
ETTK_DEV double block_sum_f(float v, float2 *sh) {
  float2 p = warp_sum_ff(make_float2(v, 0.f));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = p;
  __syncthreads();
  double r = 0;
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    p = warp_sum_ff(lane < nw ? sh[lane] : make_float2(0.f, 0.f));
    if (lane == 0) r = (double)p.x + (double)p.y;
  }
  __syncthreads();
  return r;
}
// Integer counts: exact. `sh` needs blockDim/32 ints.
ETTK_DEV int block_sum_i(int v, int *sh) {
  v = __reduce_add_sync(0xffffffffu, v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  int r = 0;
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    r = __reduce_add_sync(0xffffffffu, lane < nw ? sh[lane] : 0);
  }
  __syncthreads();
  return r;
}

ETTK_DEV unsigned long long warp_max_u64(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
    v = t > v ? t : v;
  }
  return v;
}

// vtkInterpolationMath::Floor (64-bit x86 branch, Filtering/vtkImageInterpolatorInternals.h:96-108):
// x + (103079215104.0 + 2^-17) in double, where the constant is 1.5*2^36 and the 2^-17 tolerance term is
// half an ulp of it and rounds away (ties to even), so the sum rounds x to the nearest multiple of 2^-16
// (ties to even); the integer part and the fraction come from that rounded value. Exact for |x| < 128.
ETTK_DEV int vtk_floor(float x, float &f) {
  int q = __float2int_rn(x * 65536.0f);
  f = (float)(q & 0xFFFF) * (1.0f / 65536.0f);
  return q >> 16;
}

// ---- mbarrier + bulk tensor copy (TMA) helpers ------------------------------------------------
ETTK_DEV uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
// 16-byte asynchronous global -> shared copies (both addresses 16-byte aligned), committed and waited in groups
ETTK_DEV void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
ETTK_DEV void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
ETTK_DEV void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory");
}
ETTK_DEV void mbar_init(void *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
ETTK_DEV void mbar_expect_tx(void *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// Bounded wait for the phase with the given parity; false if it did not complete within max_iter polls.
ETTK_DEV bool mbar_wait(void *bar, uint32_t parity, int max_iter) {
  const uint32_t a = smem_addr(bar);
  for (int i = 0; i < max_iter; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// Orders this thread's earlier generic-proxy accesses of shared memory before later async-proxy (bulk copy)
// writes to it.
ETTK_DEV void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// 3-D tile load of a tensor map (global memory) into shared memory, completing on bar. The innermost
// coordinate x must be a multiple of 16 bytes / element size; dst 128-byte aligned.
ETTK_DEV void tma_load_3d(void *dst, const void *tmap, int x, int y, int z, void *bar) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tmap) : "memory");
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(smem_addr(dst)),
      "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// Tricubic weights of vtkImageInterpolator (Filtering/vtkImageInterpolator.cxx:313-325).
ETTK_DEV void cubic_weights(float F[4], float f) {
  float fm1 = f - 1.0f, fd2 = f * 0.5f, ft3 = f * 3.0f;
  F[0] = -fd2 * fm1 * fm1;
  F[1] = ((ft3 - 2.0f) * fd2 - 1.0f) * fm1;
  F[2] = -((ft3 - 4.0f) * f - 1.0f) * fd2;
  F[3] = f * fd2 * fm1;
}

}  // namespace ettk
