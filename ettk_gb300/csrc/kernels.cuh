// Device kernels of the alignment path (FP32 arithmetic, FP64 reductions).
// Each kernel names the reference step it computes.
#pragma once
#include "common.cuh"
#include "fft.cuh"

namespace ettk {

// Per-item reslice input: the fixed image, its dims and the output-index -> input-index map.
// Diagnostic of the bounded waits: an mbarrier that nothing arrives at, polled max_iter times; the wait gives up,
// sets *status and the kernel returns, as every bounded wait of the library does when its copy or MMA never
// completes (the host then reports ETTK_ERR_TIMEOUT and the context stays usable).
static __global__ void k_wait_probe(int max_iter, int *status) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (!mbar_wait(&bar, 0, max_iter) && threadIdx.x == 0) atomicExch(status, 1);
}

struct ResliceItem {
  const float *vol;
  int dims[3];
  float m[12];   // origin[3], x axis[3], y axis[3], z axis[3]
  double md[12]; // the same in FP64 (used by the exact-coordinate variant)
  const void *tmap = nullptr;  // device tensor map of vol (RT_X x RT_Y x RT_Z float boxes), or null
  // Optional: the reslice also writes the values one step past the box on each axis (index N), as three
  // faces [3][(N+1)^2]: face 0 holds a = N at (b, c), face 1 b = N at (a, c), face 2 c = N at (a, b) (a voxel
  // on several faces is in the first). The mirror evaluation reads them (k_reslice_mirror).
  float *faces = nullptr;
};
__host__ __device__ inline long face_index(int a, int b, int c, int N) {
  const long F = (long)(N + 1) * (N + 1);
  return a == N ? (long)b * (N + 1) + c : b == N ? F + (long)a * (N + 1) + c : 2 * F + (long)a * (N + 1) + b;
}

// nbfWedgedSubImage3D::getImage (inc/em/nbfWedgedSubImage3D.h:602-828): tricubic reslice of the
// fixed image under Euler*matrix*t into an N^3 box (output [x][y][z], z fastest), background
// -FLT_MAX outside [-0.5, dim-0.5] (vtkImageReslice border 1, clamp mode), plus per-item sums
// of valid values and their count into acc[item*acc_stride + 0/1].
//
// One 8x8x8 output brick per CTA of 256 threads (two voxels per thread). The input footprint of the brick (its
// corner coordinates widened by the cubic support and a rounding margin) is staged in shared memory. A brick whose
// footprint misses the volume on some axis, or whose corners all lie more than a voxel beyond the valid range on one
// axis, is background throughout and stages nothing. When the item has a tensor map and the fixed
// RT_X x RT_Y x RT_Z box at (x0, o1, o2) holds the footprint, one bulk tensor copy (TMA) stages it, also at the
// edge of the volume: the copy reads zeros outside the volume, and the voxels whose taps reach past a face read the
// clamped positions instead (the clamp border of the reference). Items without a tensor map are staged with 16-byte
// loads: the x range starts at a multiple of 4, and a 4-wide group that lies wholly outside the volume takes the edge
// value (exact because the x extent is a multiple of 4), so every tap reads the box as it is. For a rotation the
// footprint is at most 20 x 20 rows of 24 floats, which RS_MAX holds; other bricks (scaled matrices, unaligned
// volumes) read the taps from global memory. A copy that does not complete sets *status (the host reports a
// timeout) instead of waiting forever. The 32 voxels of a warp form a 4 (a) x 4 (b) x 2 (c) block, whose rotated
// taps spread over more banks than a 1 x 4 x 8 row; the brick's outputs go through a small shared buffer so that
// the stores are whole 32-byte rows.
// CTAs per SM the FP32-coordinate reslice is compiled for (four: 64 registers per thread)
#ifndef ETTK_RESLICE_MIN_BLOCKS
#define ETTK_RESLICE_MIN_BLOCKS 4
#endif
constexpr int RB = 8;             // brick edge
constexpr int RS_MAX = 11760;     // staged floats (45.9 KiB of dynamic shared memory, four CTAs per SM)
constexpr size_t RS_SMEM = RS_MAX * sizeof(float);
// Fixed box of the bulk tensor copy: it holds the footprint of any rotated brick (x from a multiple of 4).
// The row pitch of 28 floats (-4 mod 32 banks) and plane pitch of 28 * 21 (12 mod 32) spread the taps of a
// warp's voxels over the banks (about a third fewer shared-memory wavefronts than 24-float rows)
constexpr int RT_X = 28, RT_Y = 21, RT_Z = 20;
static_assert(RT_X * RT_Y * RT_Z <= RS_MAX, "tensor box exceeds the staging buffer");
constexpr int RT_WAIT = 1 << 22;  // polls of the copy barrier before the kernel reports a timeout

// Position of an output voxel in the fixed image: integer cell, tricubic weights and the valid-range test.
struct ResliceTap {
  int ix, iy, iz;
  float wx[4], wy[4], wz[4];
  bool inside;
};

// Voxel (a, b, cz) of the output. PRECISE: the voxel coordinate follows the reference's FP64 sequence
// ((origin + c*z) + b*y) + a*x without FMA contraction and is rounded to the 2^-16 grid in FP64 (used where 1e-5
// output parity matters); otherwise the same sequence runs in FP32. CLAMP_ALL: every position is inside.
template <bool PRECISE, bool CLAMP_ALL, bool LINEAR = false>
ETTK_DEV void reslice_tap(const ResliceItem &it, int dx, int dy, int dz, int a, int b, int cz, ResliceTap &t) {
  float fx, fy, fz;
  if (PRECISE) {
    double q[3];
    for (int k = 0; k < 3; ++k) {
      double w = __dadd_rn(it.md[k], __dmul_rn((double)cz, it.md[9 + k]));
      w = __dadd_rn(w, __dmul_rn((double)b, it.md[6 + k]));
      q[k] = __dadd_rn(w, __dmul_rn((double)a, it.md[3 + k]));
    }
    t.inside = CLAMP_ALL || !(q[0] < -0.5 || q[0] > dx - 0.5 || q[1] < -0.5 || q[1] > dy - 0.5 || q[2] < -0.5 ||
                              q[2] > dz - 0.5);
    const long long r0 = __double2ll_rn(q[0] * 65536.0), r1 = __double2ll_rn(q[1] * 65536.0),
                    r2 = __double2ll_rn(q[2] * 65536.0);
    t.ix = (int)(r0 >> 16);
    fx = (float)(r0 & 0xFFFF) * (1.0f / 65536.0f);
    t.iy = (int)(r1 >> 16);
    fy = (float)(r1 & 0xFFFF) * (1.0f / 65536.0f);
    t.iz = (int)(r2 >> 16);
    fz = (float)(r2 & 0xFFFF) * (1.0f / 65536.0f);
  } else {
    float p0 = it.m[0] + cz * it.m[9], p1 = it.m[1] + cz * it.m[10], p2 = it.m[2] + cz * it.m[11];
    p0 = p0 + b * it.m[6];
    p1 = p1 + b * it.m[7];
    p2 = p2 + b * it.m[8];
    p0 = p0 + a * it.m[3];
    p1 = p1 + a * it.m[4];
    p2 = p2 + a * it.m[5];
    t.inside = CLAMP_ALL || !(p0 < -0.5f || p0 > dx - 0.5f || p1 < -0.5f || p1 > dy - 0.5f || p2 < -0.5f || p2 > dz - 0.5f);
    t.ix = vtk_floor(p0, fx);
    t.iy = vtk_floor(p1, fy);
    t.iz = vtk_floor(p2, fz);
  }
  if (LINEAR) {  // trilinear weights on the middle two taps of each axis
    t.wx[0] = t.wx[3] = t.wy[0] = t.wy[3] = t.wz[0] = t.wz[3] = 0.f;
    t.wx[1] = 1.f - fx;
    t.wx[2] = fx;
    t.wy[1] = 1.f - fy;
    t.wy[2] = fy;
    t.wz[1] = 1.f - fz;
    t.wz[2] = fz;
    return;
  }
  cubic_weights(t.wx, fx);
  cubic_weights(t.wy, fy);
  cubic_weights(t.wz, fz);
  // The reference uses only the middle row/plane when fy/fz == 0; the full 4x4x4 sum with the
  // (0, 1, 0, 0) weights it forces there adds exact zeros, so the result is unchanged.
  if (!((dy > 1) && (fy != 0.f))) { t.wy[0] = 0.f; t.wy[1] = 1.f; t.wy[2] = 0.f; t.wy[3] = 0.f; }
  if (!((dz > 1) && (fz != 0.f))) { t.wz[0] = 0.f; t.wz[1] = 1.f; t.wz[2] = 0.f; t.wz[3] = 0.f; }
}

// Trilinear sums (taps 1 and 2 of each axis, as reslice_tap<..., true> weights them) from the staged box at
// unclamped positions and at clamped positions.
ETTK_DEV float tap_sum_box_lin(const float *b0, int P, int PE, const ResliceTap &t) {
  float acc = 0.f;
#pragma unroll
  for (int k = 1; k < 3; ++k)
#pragma unroll
    for (int j = 1; j < 3; ++j) {
      const float *r = b0 + k * PE + j * P;
      acc = __fmaf_rn(__fmul_rn(t.wz[k], t.wy[j]), __fmaf_rn(t.wx[2], r[2], __fmul_rn(t.wx[1], r[1])), acc);
    }
  return acc;
}
ETTK_DEV float tap_sum_clamped_lin(const float *box, int x0, int o1, int o2, int P, int PE, int dx, int dy, int dz,
                                   const ResliceTap &t) {
  float acc = 0.f;
  const int xa = min(max(t.ix, 0), dx - 1) - x0, xb = min(max(t.ix + 1, 0), dx - 1) - x0;
#pragma unroll
  for (int k = 1; k < 3; ++k)
#pragma unroll
    for (int j = 1; j < 3; ++j) {
      const float *r = box + (min(max(t.iz - 1 + k, 0), dz - 1) - o2) * PE + (min(max(t.iy - 1 + j, 0), dy - 1) - o1) * P;
      acc = __fmaf_rn(__fmul_rn(t.wz[k], t.wy[j]), __fmaf_rn(t.wx[2], r[xb], __fmul_rn(t.wx[1], r[xa])), acc);
    }
  return acc;
}

// The tricubic sum of every path below, in one fixed order: per row (z plane k, y row j)
// xs = ((wx0 r0 + wx1 r1) + wx2 r2) + wx3 r3 (fused), acc += (wz_k wy_j) xs (fused).
// Taps read from the staged box at unclamped positions: row pitch P, plane pitch PE (floats), b0 = tap (0, 0, 0).
ETTK_DEV float tap_sum_box(const float *b0, int P, int PE, const ResliceTap &t) {
  float acc = 0.f;
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float *r = b0 + k * PE + j * P;
      float xs = __fmul_rn(t.wx[0], r[0]);
      xs = __fmaf_rn(t.wx[1], r[1], xs);
      xs = __fmaf_rn(t.wx[2], r[2], xs);
      xs = __fmaf_rn(t.wx[3], r[3], xs);
      acc = __fmaf_rn(__fmul_rn(t.wz[k], t.wy[j]), xs, acc);
    }
  return acc;
}
// Taps clamped to the volume (the reference's clamp border) and read from the staged box, whose origin is
// (x0, o1, o2): used for voxels within two voxels of a face when the box copy filled positions outside the volume.
ETTK_DEV float tap_sum_clamped(const float *box, int x0, int o1, int o2, int P, int PE, int dx, int dy, int dz,
                               const ResliceTap &t) {
  int xo[4], yo[4], zo[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    xo[i] = min(max(t.ix - 1 + i, 0), dx - 1) - x0;
    yo[i] = (min(max(t.iy - 1 + i, 0), dy - 1) - o1) * P;
    zo[i] = (min(max(t.iz - 1 + i, 0), dz - 1) - o2) * PE;
  }
  float acc = 0.f;
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float *r = box + zo[k] + yo[j];
      float xs = __fmul_rn(t.wx[0], r[xo[0]]);
      xs = __fmaf_rn(t.wx[1], r[xo[1]], xs);
      xs = __fmaf_rn(t.wx[2], r[xo[2]], xs);
      xs = __fmaf_rn(t.wx[3], r[xo[3]], xs);
      acc = __fmaf_rn(__fmul_rn(t.wz[k], t.wy[j]), xs, acc);
    }
  return acc;
}
// Taps clamped to the volume and read from global memory (bricks whose footprint is not staged). Not inlined; its
// arguments are scalars so that they pass in registers (a structure passed by reference would live in local memory
// for every voxel of the calling kernel).
static __device__ __noinline__ float tricubic_global(const float *__restrict__ vol, int dx, int dy, int dz, int ix, int iy,
                                                     int iz, float wx0, float wx1, float wx2, float wx3, float wy0,
                                                     float wy1, float wy2, float wy3, float wz0, float wz1, float wz2,
                                                     float wz3) {
  const float wx[4] = {wx0, wx1, wx2, wx3}, wy[4] = {wy0, wy1, wy2, wy3}, wz[4] = {wz0, wz1, wz2, wz3};
  const int x_0 = min(max(ix - 1, 0), dx - 1), x_1 = min(max(ix, 0), dx - 1), x_2 = min(max(ix + 1, 0), dx - 1),
            x_3 = min(max(ix + 2, 0), dx - 1);
  float acc = 0.f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int z = min(max(iz - 1 + k, 0), dz - 1);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int y = min(max(iy - 1 + j, 0), dy - 1);
      const float *row = vol + ((long)z * dy + y) * dx;
      float xs = __fmul_rn(wx[0], __ldg(row + x_0));
      xs = __fmaf_rn(wx[1], __ldg(row + x_1), xs);
      xs = __fmaf_rn(wx[2], __ldg(row + x_2), xs);
      xs = __fmaf_rn(wx[3], __ldg(row + x_3), xs);
      acc = __fmaf_rn(__fmul_rn(wz[k], wy[j]), xs, acc);
    }
  }
  return acc;
}

// PRECISE: FP64 voxel coordinates (reslice_tap). CLAMP_ALL: every voxel takes the clamped tricubic value (no -max
// background), for the continuous refinement. LINEAR: trilinear instead of tricubic interpolation (8 taps), for the
// candidate screening of the fast form (no reference counterpart: the reference always resamples tricubically).
template <bool PRECISE, bool CLAMP_ALL = false, bool LINEAR = false>
__global__ void __launch_bounds__(256, PRECISE ? 3 : ETTK_RESLICE_MIN_BLOCKS) k_reslice_brick(const ResliceItem *__restrict__ items, int N,
                                                          float *__restrict__ out, double *acc, int acc_stride,
                                                          int *status, const int *__restrict__ item_index) {
  extern __shared__ __align__(128) float4 box4[];
  const float *box = reinterpret_cast<const float *>(box4);
  __shared__ double sh[32];
  __shared__ int geo[7];  // o[3], ext[3], mode
  __shared__ __align__(8) unsigned long long tma_bar;
  __shared__ float obuf[RB * 66];  // brick outputs at a*66 + b*8 + c (conflict-free for both voxel maps)
  const int eidx = item_index ? item_index[blockIdx.y] : (int)blockIdx.y;  // item resliced by this CTA row
  const ResliceItem &it = items[eidx];
  const int nb = N / RB;
  const int bx = blockIdx.x / (nb * nb), by = (blockIdx.x / nb) % nb, bz = blockIdx.x % nb;
  const int dx = it.dims[0], dy = it.dims[1], dz = it.dims[2];
  const float *vol = it.vol;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // bricks on the last layer of an axis also produce the face one step past the box on that axis
  const int ea = (it.faces && bx == nb - 1) ? 1 : 0, eb = (it.faces && by == nb - 1) ? 1 : 0,
            ec = (it.faces && bz == nb - 1) ? 1 : 0;
  if (warp == 0) {
    // footprint of the 8 corners (same affine map as the per-voxel coordinates), lanes 0..7
    const int c8 = lane & 7;
    const int a = bx * RB + ((c8 & 1) ? RB - 1 + ea : 0), b = by * RB + ((c8 & 2) ? RB - 1 + eb : 0),
              cz = bz * RB + ((c8 & 4) ? RB - 1 + ec : 0);
    float lo[3], hi[3];
    for (int t = 0; t < 3; ++t) {
      float q = it.m[t] + cz * it.m[9 + t];
      q = q + b * it.m[6 + t];
      q = q + a * it.m[3 + t];
      lo[t] = hi[t] = q;
    }
    for (int off = 4; off > 0; off >>= 1)
      for (int t = 0; t < 3; ++t) {
        lo[t] = fminf(lo[t], __shfl_xor_sync(0xffffffffu, lo[t], off));
        hi[t] = fmaxf(hi[t], __shfl_xor_sync(0xffffffffu, hi[t], off));
      }
    if (lane == 0) {
      const int d[3] = {dx, dy, dz};
      int o[3], e[3];
      bool outside = false;
      for (int t = 0; t < 3; ++t) {
        o[t] = (int)floorf(lo[t]) - 2;
        e[t] = (int)floorf(hi[t]) + 4 - o[t] + 1;  // taps reach floor(p)+1+2; p may exceed hi by rounding
        if (!CLAMP_ALL)
          outside = outside || o[t] + e[t] <= 0 || o[t] >= d[t] || hi[t] < -1.5f || lo[t] > (float)d[t] + 0.5f;
        geo[t] = o[t];
        geo[3 + t] = e[t];
      }
      const int x0 = o[0] & ~3;
      int mode = 0;
      if (outside) mode = 2;
      else if (it.tmap != nullptr && (smem_addr(box4) & 127) == 0 && o[0] + e[0] <= x0 + RT_X && e[1] <= RT_Y &&
               e[2] <= RT_Z &&
               (!CLAMP_ALL || (x0 >= 0 && x0 + RT_X <= dx && o[1] >= 0 && o[1] + RT_Y <= dy && o[2] >= 0 &&
                               o[2] + RT_Z <= dz)))
        // the box holds the footprint: one bulk copy (positions outside the volume read as zero). The clamped taps
        // of a voxel in the valid range lie in [floor(p) - 1, floor(p) + 2] and so in the footprint; with CLAMP_ALL
        // a voxel far outside the volume would clamp to positions outside the box, so there the box must lie inside
        // the volume (every tap then reads the box as it is).
        mode = 1;
      geo[6] = mode;
    }
  }
  __syncthreads();
  const int o0 = geo[0], o1 = geo[1], o2 = geo[2], e0 = geo[3], e1 = geo[4], e2 = geo[5], mode = geo[6];
  const long n3 = (long)N * N * N;
  const int nxa = RB + ea, nxb = RB + eb, nxc = RB + ec, n_ext = (ea | eb | ec) ? nxa * nxb * nxc : 0;
  // the brick (and its faces) as background: nothing staged, nothing summed
  auto background = [&]() {
    for (int v = threadIdx.x; v < RB * RB * RB; v += blockDim.x)
      out[(long)eidx * n3 + ((long)(bx * RB + (v >> 6)) * N + (by * RB + ((v >> 3) & 7))) * N + bz * RB + (v & 7)] =
          -FLT_MAX;
    for (int i = threadIdx.x; i < n_ext; i += blockDim.x) {
      const int la = i / (nxb * nxc), lb = (i / nxc) % nxb, lc = i % nxc;
      if (la < RB && lb < RB && lc < RB) continue;
      it.faces[face_index(bx * RB + la, by * RB + lb, bz * RB + lc, N)] = -FLT_MAX;
    }
  };
  if (mode == 2) {  // every voxel lies outside the volume
    background();
    return;
  }
  const int x0 = o0 & ~3;                        // floor to a multiple of 4
  const int w4 = (o0 + e0 - x0 + 3) >> 2;        // 16-byte groups per staged row
  const bool use_tma = mode == 1;
  const int P = use_tma ? RT_X : w4 * 4;         // staged row pitch (floats)
  // staged rows per plane: odd, so that the plane pitch E1 * P is never a multiple of 32 floats (taps that
  // differ only in z would otherwise share a bank)
  const int E1 = use_tma ? RT_Y : (e1 | 1);
  const bool staged = use_tma || (e0 >= 5 && e0 <= 64 && e1 >= 5 && e1 <= 64 && e2 >= 5 && e2 <= 64 &&
                                  E1 * e2 * P <= RS_MAX && (dx & 3) == 0 && (((unsigned long long)vol) & 15) == 0);
  if (use_tma) {
    if (threadIdx.x == 0) mbar_init(&tma_bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_expect_tx(&tma_bar, RT_X * RT_Y * RT_Z * (uint32_t)sizeof(float));
      tma_load_3d(box4, it.tmap, x0, o1, o2, &tma_bar);
    }
    bool landed = mbar_wait(&tma_bar, 0, RT_WAIT);
    if (!landed) {
      atomicExch(status, 1);
      landed = mbar_wait(&tma_bar, 0, RT_WAIT);  // the copy may still land: wait again (bounded)
    }
    if (!__syncthreads_and(landed)) {  // the box never arrived: background (the status makes the call fail), no read
      background();
      return;
    }
  } else if (staged) {
    // flat index -> (row, group) and row -> (y, z) by multiply-high (exact for divisors <= 64, index < 2^16)
    const unsigned mw = 0xFFFFFFFFu / (unsigned)w4 + 1u, me = 0xFFFFFFFFu / (unsigned)e1 + 1u;
    const int n4 = e1 * e2 * w4;
    for (int i = threadIdx.x; i < n4; i += blockDim.x) {
      const int row = (int)__umulhi((unsigned)i, mw), c4 = i - row * w4;
      const int uz = (int)__umulhi((unsigned)row, me), uy = row - uz * e1;
      const int y = min(max(o1 + uy, 0), dy - 1), z = min(max(o2 + uz, 0), dz - 1);
      const int xs = x0 + 4 * c4, xl = min(max(xs, 0), dx - 4);
      float4 f = __ldg(reinterpret_cast<const float4 *>(vol + ((long)z * dy + y) * dx + xl));
      if (xs < 0) f = make_float4(f.x, f.x, f.x, f.x);
      else if (xs > dx - 4) f = make_float4(f.w, f.w, f.w, f.w);
      box4[(uz * E1 + uy) * w4 + c4] = f;
    }
  }
  __syncthreads();
  float s = 0.f;
  int cnt = 0;
  // Box offset of a voxel's tap (0, 0, 0) and whether its 4 x 4 x 4 taps can be read from the box as they are: the
  // 16-byte staging stores clamped values beyond the volume, the bulk copy zeros there, so its voxels within two
  // voxels of a face read clamped positions instead (tap_sum_clamped).
  const int PE = E1 * P;
  // tricubic value of a voxel (-FLT_MAX outside the valid range)
  auto value = [&](const ResliceTap &t) -> float {
    if (!t.inside) return -FLT_MAX;
    if (!staged)
      return tricubic_global(vol, dx, dy, dz, t.ix, t.iy, t.iz, t.wx[0], t.wx[1], t.wx[2], t.wx[3], t.wy[0], t.wy[1],
                             t.wy[2], t.wy[3], t.wz[0], t.wz[1], t.wz[2], t.wz[3]);
    const int off = ((t.iz - 1 - o2) * E1 + (t.iy - 1 - o1)) * P + (t.ix - 1 - x0);
    if (LINEAR) {
      if (!use_tma) return tap_sum_box_lin(box + off, P, PE, t);
      if ((unsigned)t.ix <= (unsigned)(dx - 2) && (unsigned)t.iy <= (unsigned)(dy - 2) && (unsigned)t.iz <= (unsigned)(dz - 2))
        return tap_sum_box_lin(box + off, RT_X, RT_X * RT_Y, t);
      return tap_sum_clamped_lin(box, x0, o1, o2, P, PE, dx, dy, dz, t);
    }
    if (!use_tma) return tap_sum_box(box + off, P, PE, t);
    if ((unsigned)(t.ix - 1) <= (unsigned)(dx - 4) && (unsigned)(t.iy - 1) <= (unsigned)(dy - 4) &&
        (unsigned)(t.iz - 1) <= (unsigned)(dz - 4))
      return tap_sum_box(box + off, RT_X, RT_X * RT_Y, t);
    return tap_sum_clamped(box, x0, o1, o2, P, PE, dx, dy, dz, t);
  };
  // The thread's two voxels v = tid and tid + 256; the 32 voxels of a warp form a 4 (a) x 4 (b) x 2 (c) block.
#pragma unroll 1
  for (int v = threadIdx.x; v < RB * RB * RB; v += blockDim.x) {
    const int w = v >> 5, ln = v & 31;
    const int la = 4 * (w >> 3) + (ln >> 3), lb = 4 * ((w >> 2) & 1) + ((ln >> 1) & 3), lc = 2 * (w & 3) + (ln & 1);
    ResliceTap t;
    reslice_tap<PRECISE, CLAMP_ALL, LINEAR>(it, dx, dy, dz, bx * RB + la, by * RB + lb, bz * RB + lc, t);
    const float val = value(t);
    if (t.inside) {
      s += val;
      cnt += 1;
    }
    obuf[la * 66 + lb * 8 + lc] = val;
  }
  __syncthreads();
  for (int v = threadIdx.x; v < RB * RB * RB; v += blockDim.x) {
    const int a = v >> 6, b = (v >> 3) & 7, c = v & 7;
    out[(long)eidx * n3 + ((long)(bx * RB + a) * N + (by * RB + b)) * N + bz * RB + c] = obuf[a * 66 + b * 8 + c];
  }
  // faces one step past the box (not part of this item's output or sums)
  for (int i = threadIdx.x; i < n_ext; i += blockDim.x) {
    const int fa = i / (nxb * nxc), fb = (i / nxc) % nxb, fc = i % nxc;
    if (fa < RB && fb < RB && fc < RB) continue;
    ResliceTap t;
    const int a = bx * RB + fa, b = by * RB + fb, cz = bz * RB + fc;
    reslice_tap<PRECISE, CLAMP_ALL, LINEAR>(it, dx, dy, dz, a, b, cz, t);
    it.faces[face_index(a, b, cz, N)] = value(t);
  }
  if (acc) {
    const double bs = block_sum_f(s, reinterpret_cast<float2 *>(sh));
    const int bc = block_sum_i(cnt, reinterpret_cast<int *>(sh));
    if (threadIdx.x == 0) {
      atomicAdd(&acc[(long)eidx * acc_stride + 0], bs);
      atomicAdd(&acc[(long)eidx * acc_stride + 1], (double)bc);
    }
  }
}

// Binary wedge on the centred half grid (nbfWedge3D::getImageHalf, inc/em/nbfWedge3D.h:312-356):
// ((v1.d)(v2.d) <= 0) with d = (i-N/2, j-N/2, k-N/2). Near the planes the test is redone in FP64
// with the reference's operation order (no FMA) so exact-zero cases resolve as they do there.
struct WedgeVecs {
  double v1[3], v2[3];
  int full;
};
// One axis of vtkImageGaussianSmooth with std 2 and radius 1 (nbfWedge3D::smoothWedgeImage,
// inc/em/nbfWedge3D.h:431-445) on [item][N][N][H] arrays; axis 2 = k (VTK z, first pass),
// 1 = j, 0 = i. The final pass (axis 0) multiplies by the reference wedge and the filter
// (wedge2 *= wedge1; filter*wedge, inc/em/nbfFourierImageMetric.h:1101-1113, nbfFourierFilter.h:586-606)
// and accumulates sum(wedge*filter) for the overlap normalisation.
struct Smooth3 {
  float w_int[3];   // interior weights (-1, 0, +1)
  float w_lo[2];    // at index 0: (0, +1)
  float w_hi[2];    // at last index: (-1, 0)
};
// Mirror evaluations of the candidate loop (the CCF at Scale(-1,-1,-1) * T, execute 678-776): for a pure
// rotation T and no cut offset, output index a of the mirror samples the fixed image where index N - a of
// the direct reslice does (box coordinates a - N/2 are negated), so r'[a][b][c] = r[N-a][N-b][N-c], with the
// direct reslice's faces one step past its box (ResliceItem::faces) for the indices N. The positions agree
// with the mirror's own map to float rounding. pairs[y] = (mirror item, direct item); sums of valid values
// and their count into acc as the reslice.
static __global__ void __launch_bounds__(256) k_reslice_mirror(const ResliceItem *__restrict__ items,
                                                               const int2 *__restrict__ pairs, int N,
                                                               float *__restrict__ out, double *acc, int acc_stride) {
  __shared__ double sh[32];
  const int em = pairs[blockIdx.y].x, ed = pairs[blockIdx.y].y;
  const long n3 = (long)N * N * N;
  const float *src = out + (long)ed * n3;
  const float *faces = items[ed].faces;
  float *dst = out + (long)em * n3;
  float s = 0.f;
  int cnt = 0;
  // one aligned quad of outputs (c = 4j .. 4j+3 of row (a, b)) per thread and step
  const int nq = (int)(n3 / 4), qrow = N / 4;
  for (int qd = blockIdx.x * blockDim.x + threadIdx.x; qd < nq; qd += gridDim.x * blockDim.x) {
    const int row = qd / qrow, c0 = 4 * (qd - row * qrow);
    const int x = N - row / N, y = N - row % N;
    float v[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int z = N - (c0 + t);
      v[t] = (x < N && y < N && z < N) ? src[((long)x * N + y) * N + z] : faces[face_index(x, y, z, N)];
      if (v[t] > -FLT_MAX) {
        s += v[t];
        cnt += 1;
      }
    }
    reinterpret_cast<float4 *>(dst)[qd] = make_float4(v[0], v[1], v[2], v[3]);
  }
  const double bs = block_sum_f(s, reinterpret_cast<float2 *>(sh));
  const int bc = block_sum_i(cnt, reinterpret_cast<int *>(sh));
  if (threadIdx.x == 0) {
    atomicAdd(&acc[(long)em * acc_stride + 0], bs);
    atomicAdd(&acc[(long)em * acc_stride + 1], (double)bc);
  }
}

// Binary wedge (nbfWedge3D::getImageHalf, inc/em/nbfWedge3D.h:312-356): ((v1.d)(v2.d) <= 0) with
// d = (i-N/2, j-N/2, k-N/2) on the centred half grid. Near the planes the test is redone in FP64 with the
// reference's operation order (no FMA) so exact-zero cases resolve as they do there.
ETTK_DEV float wedge_bit(const WedgeVecs &w, const float f1[3], const float f2[3], int i, int j, int k, int N, int H) {
  if (w.full) return 1.f;
  float di = (float)(i - N / 2), dj = (float)(j - N / 2), dk = (float)(k - (H - 1));
  float a = f1[0] * di + f1[1] * dj + f1[2] * dk, b = f2[0] * di + f2[1] * dj + f2[2] * dk;
  if (fabsf(a) > 1e-3f && fabsf(b) > 1e-3f) return (a * b <= 0.f) ? 1.f : 0.f;
  double ad = __dadd_rn(__dadd_rn(__dmul_rn(w.v1[0], (double)di), __dmul_rn(w.v1[1], (double)dj)),
                        __dmul_rn(w.v1[2], (double)dk));
  double bd = __dadd_rn(__dadd_rn(__dmul_rn(w.v2[0], (double)di), __dmul_rn(w.v2[1], (double)dj)),
                        __dmul_rn(w.v2[2], (double)dk));
  return (__dmul_rn(ad, bd) <= 0.0) ? 1.f : 0.f;
}
// One 3-tap pass of vtkImageGaussianSmooth at position pos of an axis of length n (clipped, renormalised
// kernel at the ends); vm / vp are the neighbours (ignored where clipped).
ETTK_DEV float smooth3v(const Smooth3 &sw, float vm, float v0, float vp, int pos, int n) {
  if (n == 1) return v0;
  if (pos == 0) return sw.w_lo[0] * v0 + sw.w_lo[1] * vp;
  if (pos == n - 1) return sw.w_hi[0] * vm + sw.w_hi[1] * v0;
  return sw.w_int[0] * vm + sw.w_int[1] * v0 + sw.w_int[2] * vp;
}

// Binary wedge + the three smoothing passes + (wedge2 * wedge1) * filter in one kernel. One CTA per
// (slab of SLAB x planes, item) walks the planes i0-1 .. i0+SLAB: each plane's binary wedge is smoothed
// along k then j (float rounding after each pass, as vtkImageGaussianSmooth stores its intermediates) into a
// three-plane ring in shared memory; as soon as planes q-1, q, q+1 are in the ring, plane q is smoothed
// along i, multiplied by the reference wedge and the filter, stored, and summed into acc[item][acc_slot]
// (sum(wedge*filter) of the overlap normalisation). Filter, reference wedges and output are kz-major.
template <int N, int SLAB>
__global__ void __launch_bounds__(256, 3) k_wedge_roll(const WedgeVecs *__restrict__ wv, Smooth3 sw,
                                                    const float *__restrict__ w1, const int *__restrict__ w1_index,
                                                    const float *__restrict__ filter, float *__restrict__ out,
                                                    double *acc, int acc_stride, int acc_slot) {
  constexpr int H = N / 2 + 1, PL = N * H;
  constexpr long h3 = (long)PL * N;
  extern __shared__ float wsm[];
  float *Kp = wsm;            // k-smoothed plane
  float *ring = wsm + PL;     // 3 j/k-smoothed planes, plane p in slot p % 3
  float *bits = wsm + 4 * PL; // binary wedge of the current plane
  __shared__ double sh[32];
  const int e = blockIdx.y, i0 = blockIdx.x * SLAB;
  const WedgeVecs w = wv[e];
  const float f1[3] = {(float)w.v1[0], (float)w.v1[1], (float)w.v1[2]};
  const float f2[3] = {(float)w.v2[0], (float)w.v2[1], (float)w.v2[2]};
  const float *W1 = w1 + (long)w1_index[e] * h3;
  float *o = out + (long)e * h3;
  float s = 0.f;
  // plane q of the output is written kz-major: element (q, j, k) at [k][q][j] (j fastest, coalesced)
  auto emit = [&](int q) {
    const float *rm = ring + ((q + 2) % 3) * PL, *r0 = ring + (q % 3) * PL, *rp = ring + ((q + 1) % 3) * PL;
    for (int t = threadIdx.x; t < PL; t += blockDim.x) {
      const int k = t / N, j = t - k * N;
      const int r = j * H + k;
      const float vm = q > 0 ? rm[r] : 0.f, vp = q < N - 1 ? rp[r] : 0.f;
      // a full wedge is the constant 1, unsmoothed (nbfWedge3D::getImageHalf, inc/em/nbfWedge3D.h:316-317)
      const float v = w.full ? 1.f : smooth3v(sw, vm, r0[r], vp, q, N);
      const long g = ((long)k * N + q) * N + j;
      const float fw = filter[g] * (v * W1[g]);
      o[g] = fw;
      s += fw;
    }
  };
  const int pstart = max(i0 - 1, 0), pend = min(i0 + SLAB, N - 1);
  for (int p = pstart; p <= pend; ++p) {
    for (int r = threadIdx.x; r < PL; r += blockDim.x) {
      const int j = r / H, k = r - j * H;
      bits[r] = wedge_bit(w, f1, f2, p, j, k, N, H);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < PL; r += blockDim.x) {
      const int k = r % H;
      Kp[r] = smooth3v(sw, k > 0 ? bits[r - 1] : 0.f, bits[r], k < H - 1 ? bits[r + 1] : 0.f, k, H);
    }
    __syncthreads();  // also orders the previous emit's ring reads before this plane's ring write
    float *dst = ring + (p % 3) * PL;
    for (int r = threadIdx.x; r < PL; r += blockDim.x) {
      const int j = r / H;
      dst[r] = smooth3v(sw, j > 0 ? Kp[r - H] : 0.f, Kp[r], j < N - 1 ? Kp[r + H] : 0.f, j, N);
    }
    __syncthreads();
    if (p - 1 >= i0) emit(p - 1);
  }
  if (pend == N - 1 && N - 1 < i0 + SLAB) emit(N - 1);
  const double b = block_sum_f(s, reinterpret_cast<float2 *>(sh));
  if (threadIdx.x == 0) atomicAdd(&acc[(long)e * acc_stride + acc_slot], b);
}
template <int N>
constexpr int wedge_slab() { return N >= 32 ? 16 : 8; }
template <int N>
constexpr size_t wedge_smem() { return 5 * (size_t)N * (N / 2 + 1) * sizeof(float); }

// norm of normalizeFourierHalf with its float roundings: norm = float(2*s1);
// norm = float(sqrt((norm + s2) / (N*N*2*(H-1)))). Writes 1/norm (and norm) per item.
static __global__ void k_norms(const double *acc, int acc_stride, int slot, int N, int n_items, float *inv_norm,
                        float *norm_out) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_items) return;
  const int H = N / 2 + 1;
  double s1 = acc[(long)e * acc_stride + slot], s2 = acc[(long)e * acc_stride + slot + 1];
  float nrm = (float)(2.0 * s1);
  nrm = (float)sqrt(((double)nrm + s2) / (1.0 * N * N * 2 * (H - 1)));
  inv_norm[e] = nrm > 0.f ? 1.0f / nrm : 0.f;
  if (norm_out) norm_out[e] = nrm;
}

// ---- R2C z-pass input functors ------------------------------------------------------------

// Resliced particle: (valid ? v - meanInside : 0) * maskfft * shift
// (nbfWedgedSubImage3D.h:794-802 then nbfFourierImageMetric.h:1165-1166).
struct PreParticle {
  const float *v;
  const float *maskfft;
  const double *acc;
  int acc_stride, N;
  long cached = -1;  // per-thread: item whose mean is in `mean`
  float mean = 0.f;
  // per-thread cache of the decomposition of the two real lines a thread alternates between (slot = line & 1)
  long cl[2] = {-1, -1};
  int cr[2] = {0, 0}, cij[2] = {0, 0};
  float cmean[2] = {0.f, 0.f};
  static constexpr bool kStream = true;
  ETTK_HD const float *stream_src() const { return v; }
  ETTK_HD const float *stream_aux() const { return maskfft; }
  ETTK_DEV void begin() {}
  ETTK_DEV void end() {}
  ETTK_DEV void end_tile(long) {}
  ETTK_DEV float operator()(long line, int k) {
    const long r = line % ((long)N * N);
    return apply(line, k, v[line * N + k], maskfft ? maskfft[r * N + k] : 1.f);
  }
  ETTK_DEV float apply(long line, int k, float val, float m) {
    const int sl = (int)(line & 1);
    if (line != cl[sl]) {
      long n2 = (long)N * N;
      long e = line / n2;
      cl[sl] = line;
      cr[sl] = (int)(line - e * n2);
      cij[sl] = cr[sl] / N + cr[sl] % N;
      if (e != cached) {
        float cnt = (float)acc[e * acc_stride + 1];
        mean = (float)(acc[e * acc_stride + 0] / (double)cnt);
        cached = e;
      }
      cmean[sl] = mean;
    }
    float out = (val > -FLT_MAX) ? val - cmean[sl] : 0.f;
    return out * m * (((cij[sl] + k) & 1) ? -1.f : 1.f);
  }
};

// Generic: src * aux * shift over one N^3 volume per item (the constant transforms of the
// reference and of the mask: R2C(I1*maskfft*shift), R2C(m1*shift)).
struct PreProductShift {
  const float *src;  // per item N^3 (nullptr -> 1)
  const float *aux;  // shared N^3 (nullptr -> 1)
  int N;
  ETTK_DEV void begin() {}
  ETTK_DEV void end() {}
  ETTK_DEV float operator()(long line, int k) {
    long r = line % ((long)N * N);
    int i = (int)(r / N), j = (int)(r % N);
    float a = src ? src[line * N + k] : 1.f;
    float b = aux ? aux[r * N + k] : 1.f;
    return a * b * parity_sign(i, j, k);
  }
};

// Elementwise steps between a C2R and an R2C of the same z lines (k_c2r_r2c_stream). Each maps the real value
// of the inverse (and the element of `aux`, 1 without one) to the forward input and closes a tile with
// end_tile(first line).
// y2^2 * shift (nbfFourierImageMetric.h:1188-1190) of the C2R output y2.
struct MidSquareShift {
  int N;
  const float *aux = nullptr;
  long cl[2] = {-1, -1};  // two-slot line cache (slot = line & 1)
  int cij[2] = {0, 0};
  ETTK_DEV void begin() {}
  ETTK_DEV void end_tile(long) {}
  ETTK_DEV float operator()(long line, int k, float v, float) {
    const int sl = (int)(line & 1);
    if (line != cl[sl]) {
      cl[sl] = line;
      int r = (int)(line % ((long)N * N));
      cij[sl] = r / N + r % N;
    }
    return v * v * (((cij[sl] + k) & 1) ? -1.f : 1.f);
  }
};
// C2R output times the real-space mask of getLowDimensionRepresentationHalf (blitzFFTreal *= mask,
// inc/em/nbfFourierImageMetric.h:2001-2003); aux = the mask [x][y][z], shared by all items.
struct MidMask {
  const float *aux;
  ETTK_DEV void begin() {}
  ETTK_DEV void end_tile(long) {}
  ETTK_DEV float operator()(long, int, float v, float m) { return v * m; }
};
// (y1 / norm) * m1 with k1_m = sum((y1 / norm)^2 m1) into acc[item][slot] (nbfFourierImageMetric.h:1143-1153):
// the C2R output scaled by the item's 1/norm (normalizeFourierHalf, linear through the inverse passes); aux = m1.
struct MidScaleY1M1 {
  const float *scale;
  int lg_nn;
  const float *aux;
  double *acc;
  int acc_stride, slot, N;
  float s = 0.f;
  ETTK_DEV void begin() { s = 0.f; }
  ETTK_DEV float operator()(long line, int, float v, float m) {
    const float y = v * scale[line >> lg_nn];
    s += y * y * m;
    return y * m;
  }
  ETTK_DEV void end_tile(long first_line) {
    __shared__ double shm[32];
    double b = block_sum((double)s, shm);
    if (threadIdx.x == 0) atomicAdd(&acc[(first_line / ((long)N * N)) * acc_stride + slot], b);
  }
};

// Store real output of a C2R z-pass.
struct PostStore {
  float *y;
  int N;
  ETTK_DEV void begin() {}
  ETTK_DEV void end() {}
  ETTK_DEV void operator()(long line, int k, float v) { y[line * N + k] = v; }
};
// Store of a C2R z pass with the centring sign undone and a scale: a = C2R(F) * shift / N^3 (nbfFourierFilter::executeHalf
// on a real array, inc/em/nbfFourierFilter.h:654-672, with scale 1 / N^3).
struct PostStoreScaledSigned {
  float *y;
  int N;
  float scale;
  ETTK_DEV void begin() {}
  ETTK_DEV void end() {}
  ETTK_DEV void operator()(long line, int k, float v) {
    const int r = (int)(line % ((long)N * N));
    const float w = v * scale;
    y[line * N + k] = ((((r / N) + (r % N) + k) & 1) ? -w : w);
  }
};
// Pruned inverse of the zero-padded (2N)^3 half spectrum, restricted to the search window
// [lo, lo+W) on each axis (the reference computes the whole (2N)^3 C2R, nbfFourierImageMetric.h:1204-1232,
// and reads only this window). Same FFTW order: complex inverse along x, then y (k_pruned_fft, 2N-point
// register FFTs of the zero-padded lines), then the half-complex-to-real sum along z (real parts only for
// the kz = N term) fused with the peak search.
// Last axis of the windowed upsampled C2R plus the peak search, one CTA per (X, item):
// out[Y][Z] = sum_kz c_KZ Re(q2[X][Y][kz] exp(+2 pi i KZ (lo + Z) / 2N)), KZ = kz + o2 (c = 1 at KZ = 0 and
// KZ = N, else 2: the hc2r of the reference's (2N)^3 C2R); T = out * (-1)^(X+Y+Z) / (2N)^3 inside the sphere
// radius^2 < r^2 (else -max); packed argmax (first occurrence in [X][Y][Z] order) into peak[e].
// q2 is [item][X][kz][Y]. Dynamic shared memory: the q2 plane and Ez, both [kz][WP] complex (WP = W rounded up to
// 4, zero-padded). Each thread accumulates a 4 x 4 tile of (Y, Z) outputs over kz (per output the same
// sequential kz sum as a direct loop), so a kz step costs 8 shared loads for 16 outputs.
static __global__ void __launch_bounds__(128) k_pruned_z_peak(const float2 *__restrict__ q2, int N, int W, int lo,
                                                              int o2, float rr2, unsigned long long *peak) {
  extern __shared__ float4 zsm[];
  const int H = N / 2 + 1, TW = (W + 3) / 4, WP = 4 * TW;
  float2 *P2 = reinterpret_cast<float2 *>(zsm);   // [H][WP]
  float2 *Ez = P2 + H * WP;                       // [H][WP] (with the hc2r coefficient folded in)
  const int X = blockIdx.x, e = blockIdx.y;
  const float2 *src = q2 + ((long)e * W + X) * (long)W * H;
  for (int i = threadIdx.x; i < H * WP; i += blockDim.x) {
    const int kz = i / WP, Y = i - kz * WP;
    P2[i] = Y < W ? src[kz * W + Y] : make_float2(0.f, 0.f);
  }
  for (int i = threadIdx.x; i < H * WP; i += blockDim.x) {
    const int kz = i / WP, Z = i - kz * WP;
    float2 v = make_float2(0.f, 0.f);
    if (Z < W) {
      const int KZ = kz + o2;
      const int ph = (KZ * (lo + Z)) & (2 * N - 1);
      float sn, cs;
      sincospif((float)ph / (float)N, &sn, &cs);
      const float c = (KZ == N || KZ == 0) ? 1.f : 2.f;
      v = make_float2(c * cs, c * sn);
    }
    Ez[i] = v;
  }
  __syncthreads();
  const float inv = 1.0f / (float)(8L * N * N * N);
  const int half = (W - 1) / 2;
  unsigned long long best = 0;
  const float4 *P4 = reinterpret_cast<const float4 *>(P2), *E4 = reinterpret_cast<const float4 *>(Ez);
  for (int t = threadIdx.x; t < TW * TW; t += blockDim.x) {
    const int Y0 = 4 * (t / TW), Z0 = 4 * (t % TW);
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int kz = 0; kz < H; ++kz) {
      const int rp = (kz * WP + Y0) >> 1, re = (kz * WP + Z0) >> 1;
      const float4 pa = P4[rp], pb = P4[rp + 1], ea = E4[re], eb = E4[re + 1];
      const float2 pv[4] = {make_float2(pa.x, pa.y), make_float2(pa.z, pa.w), make_float2(pb.x, pb.y),
                            make_float2(pb.z, pb.w)};
      const float2 ev[4] = {make_float2(ea.x, ea.y), make_float2(ea.z, ea.w), make_float2(eb.x, eb.y),
                            make_float2(eb.z, eb.w)};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += pv[i].x * ev[j].x - pv[i].y * ev[j].y;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int Y = Y0 + i, Z = Z0 + j;
        if (Y >= W || Z >= W) continue;
        float T = acc[i][j] * parity_sign(lo + X, lo + Y, lo + Z) * inv;
        const float rad = (float)((half - X) * (half - X) + (half - Y) * (half - Y) + (half - Z) * (half - Z));
        if (!(rad < rr2)) T = -FLT_MAX;
        const unsigned long long key = pack_max(T, (uint32_t)(((long)X * W + Y) * W + Z));
        best = key > best ? key : best;
      }
  }
  best = warp_max_u64(best);
  if ((threadIdx.x & 31) == 0) atomicMax(&peak[e], best);
}

// Final CCF distance and half-voxel shift (nbfFourierImageMetric.h:1249-1264).
struct EvalOut {
  float dist;
  float shift[3];
};
// acc of item e holds k1_m (slot 4) and sum(w*f) (slot 6) at item i1_index[e] (null: e itself).
static __global__ void k_score(const double *acc, int acc_stride, const unsigned long long *peak, int n_items, int W,
                        double sum_filter, int overlap, int use_wedge, int N, EvalOut *out, const int *i1_index) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_items) return;
  unsigned long long key = peak[e];
  float T = ordered_to_float((uint32_t)(key >> 32));
  uint32_t idx = 0xffffffffu - (uint32_t)(key & 0xffffffffu);
  const double *a = acc + (long)(i1_index ? i1_index[e] : e) * acc_stride;
  float k1_m = (float)a[4];
  double big = 8.0 * N * N * N;
  double pk;
  if (overlap && use_wedge) pk = fmax(0.0, (double)k1_m - (double)T) / a[6] * sum_filter;
  else pk = fmax(0.0, (double)k1_m - (double)T);
  EvalOut o;
  // the peak is stored in the reference's float correlationPeak, then divided twice in float by the int size of
  // the upsampled grid (inc/em/nbfFourierImageMetric.h:1250-1258)
  const float bigf = (float)big;
  float cp = (float)pk;
  cp = cp / bigf;
  o.dist = cp / bigf;
  int X = idx / (W * W), Y = (idx / W) % W, Z = idx % W;
  o.shift[0] = (float)((X - (W - 1) / 2.0) / 2.0f);
  o.shift[1] = (float)((Y - (W - 1) / 2.0) / 2.0f);
  o.shift[2] = (float)((Z - (W - 1) / 2.0) / 2.0f);
  out[e] = o;
}

// ---- class average (nbfWedgedAverageImage3D::getImageMPI / getImage, inc/em/nbfWedgedAverageImage3D.h:216-356)

// acc += |w| |F|, re += w |F| Re F, im += w |F| Im F over the chunk's members in order (deterministic, FP64).
static __global__ void k_avg_accum(const float2 *__restrict__ F, const float *__restrict__ w, int n_members, long h3,
                                   double *__restrict__ acc, double *__restrict__ re, double *__restrict__ im) {
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < h3; id += (long)gridDim.x * blockDim.x) {
    double a = acc[id], r = re[id], m = im[id];
    for (int i = 0; i < n_members; ++i) {
      float2 f = F[(long)i * h3 + id];
      double b = sqrt((double)f.x * f.x + (double)f.y * f.y);
      double wi = w[i];
      a += fabs(wi) * b;
      r += wi * b * (double)f.x;
      m += wi * b * (double)f.y;
    }
    acc[id] = a;
    re[id] = r;
    im[id] = m;
  }
}

// F = (re, im) / acc where acc > 0, DC zeroed (getImage lines 224-228)
static __global__ void k_avg_spectrum(const double *__restrict__ acc, const double *__restrict__ re,
                                      const double *__restrict__ im, int N, float2 *__restrict__ F) {
  const int H = N / 2 + 1;
  long h3 = (long)N * N * H, dc = (long)(H - 1) * N * N + (N / 2) * N + N / 2;  // kz-major DC
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < h3; id += (long)gridDim.x * blockDim.x) {
    float2 v = make_float2(0.f, 0.f);
    if (acc[id] > 0) v = make_float2((float)(re[id] / acc[id]), (float)(im[id] / acc[id]));
    if (id == dc) v = make_float2(0.f, 0.f);
    F[id] = v;
  }
}

// average = C2R * shift / N^3 (already in y), sum of squares into acc_out[0]
static __global__ void k_avg_shift_sumsq(float *__restrict__ y, int N, double *acc_out) {
  __shared__ double sh[32];
  long n3 = (long)N * N * N;
  float s = 0.f;
  const float inv = 1.0f / (float)n3;
  for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < (int)n3; id += gridDim.x * blockDim.x) {
    int x = id / (N * N), yy = (id / N) % N, z = id % N;
    float v = y[id] * inv * parity_sign(x, yy, z);
    y[id] = v;
    s += v * v;
  }
  double b = block_sum((double)s, sh);
  if (threadIdx.x == 0) atomicAdd(acc_out, b);
}

// divide by the RMS (float, as varianceInside) and write x-fastest
// out = y / RMS(y), written x fastest ([z][y][x]) when xfast, else in y's [x][y][z] order
static __global__ void k_avg_finish(const float *__restrict__ y, int N, const double *sumsq, float *__restrict__ out,
                                    int xfast) {
  long n3 = (long)N * N * N;
  float rms = (float)sqrt(sumsq[0] / (double)n3);
  for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < (int)n3; id += gridDim.x * blockDim.x) {
    int x = id / (N * N), yy = (id / N) % N, z = id % N;
    out[xfast ? x + (long)N * (yy + (long)N * z) : (long)id] = y[id] / rms;
  }
}

// R[e][q] = v[e][idx[q]] (the kept voxels of getLowDimensionRepresentationReal, v [e][x][y][z])
static __global__ void k_real_gather(const float *__restrict__ v, int E, long n3, const int *__restrict__ idx, int K,
                                     float *__restrict__ R) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < (long)E * K; i += (long)gridDim.x * blockDim.x) {
    const long e = i / K;
    R[i] = v[e * n3 + idx[i - e * K]];
  }
}

// getImage's output of a resliced volume (valid: value - meanInside with meanInside rounded to float as the
// reference's Pixel; invalid: 0), inc/em/nbfWedgedSubImage3D.h:794-802, in FP64.
ETTK_DEV double get_image_value(float v, const double *acc) {
  const float cnt = (float)acc[1];
  const float mean = (float)(acc[0] / (double)cnt);
  return (v > -FLT_MAX) ? (double)v - (double)mean : 0.0;
}

// nbfImageFilter::symmetrize (inc/em/nbfImageFilter.h:527-554): the mean of the fold reslices ([i][x][y][z],
// sums in acc[i][0..1]) as getImage values, summed in order in FP64, written [z][y][x].
static __global__ void k_sym_finish(const float *__restrict__ v, const double *__restrict__ acc, int fold, int N,
                                    float *__restrict__ out) {
  const long n3 = (long)N * N * N;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < n3; id += (long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int i = 0; i < fold; ++i) s += get_image_value(v[(long)i * n3 + id], acc + 2 * i);
    const int x = (int)(id / ((long)N * N)), y = (int)((id / N) % N), z = (int)(id % N);
    out[x + (long)N * (y + (long)N * z)] = (float)(s / fold);
  }
}

// getImage values of E reslices ([e][x][y][z], sums in acc[e][0..1]), in the same order.
static __global__ void k_getimage_values(const float *__restrict__ v, const double *__restrict__ acc, int E, int N,
                                         float *__restrict__ out) {
  const long n3 = (long)N * N * N;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < (long)E * n3; id += (long)gridDim.x * blockDim.x)
    out[id] = (float)get_image_value(v[id], acc + 2 * (id / n3));
}

// getImage values of E reslices ([e][x][y][z], sums in acc[e][0..1]) as fixed images [e][z][y][x] (x fastest),
// the input of nbfImageFilter::symmetrize in getLowDimensionRepresentationHalf.
static __global__ void k_getimage_fixed(const float *__restrict__ v, const double *__restrict__ acc, int E, int N,
                                        float *__restrict__ out) {
  const long n3 = (long)N * N * N;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < (long)E * n3; id += (long)gridDim.x * blockDim.x) {
    const long e = id / n3, r = id - e * n3;
    const int x = (int)(r % N), y = (int)((r / N) % N), z = (int)(r / ((long)N * N));
    out[id] = (float)get_image_value(v[e * n3 + ((long)x * N + y) * N + z], acc + 2 * e);
  }
}

// nbfImageFilter::symmetrize per item: the mean of the item's fold reslices (getImage values, [e*fold+i][x][y][z],
// sums in acc[e*fold+i][0..1]) summed in order in FP64, written [e][x][y][z].
static __global__ void k_sym_mean(const float *__restrict__ v, const double *__restrict__ acc, int fold, int E, int N,
                                  float *__restrict__ out) {
  const long n3 = (long)N * N * N;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < (long)E * n3; id += (long)gridDim.x * blockDim.x) {
    const long e = id / n3, r = id - e * n3;
    double s = 0.0;
    for (int i = 0; i < fold; ++i) s += get_image_value(v[(e * fold + i) * n3 + r], acc + 2 * (e * fold + i));
    out[id] = (float)(s / fold);
  }
}

// getImageVarianceMPI (inc/em/nbfWedgedAverageImage3D.h:440-493): var[x][y][z] += |w_e| (T_e - avg)^2 / sum|w| over
// the chunk's members in order (FP64); avg is [z][y][x], the member reslices [e][x][y][z] with sums acc[e][0..1].
static __global__ void k_var_accum(const float *__restrict__ v, const double *__restrict__ acc, const float *__restrict__ w,
                                   int n_members, double sw, const float *__restrict__ avg, int N, double *__restrict__ var) {
  const long n3 = (long)N * N * N;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < n3; id += (long)gridDim.x * blockDim.x) {
    const int x = (int)(id / ((long)N * N)), y = (int)((id / N) % N), z = (int)(id % N);
    const double a = (double)avg[x + (long)N * (y + (long)N * z)];
    double s = var[id];
    for (int e = 0; e < n_members; ++e) {
      const double d = get_image_value(v[(long)e * n3 + id], acc + 2 * e) - a;
      s += fabs((double)w[e]) * (d * d) / sw;
    }
    var[id] = s;
  }
}
static __global__ void k_var_finish(const double *__restrict__ var, int N, float *__restrict__ out) {
  const long n3 = (long)N * N * N;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < n3; id += (long)gridDim.x * blockDim.x) {
    const int x = (int)(id / ((long)N * N)), y = (int)((id / N) % N), z = (int)(id % N);
    out[x + (long)N * (y + (long)N * z)] = (float)var[id];
  }
}

// ---- distances between low-dimensional representations ------------------------------------------
// nbfCorrelationImageMetric::getDistances(representationFile, D) (inc/em/nbfCorrelationImageMetric.h:1726-1871):
// R is the reference's representation array R(V, K, depth) in C order. depth 3 (getLowDimensionRepresentationHalf:
// re, im, wedge bit per kept coefficient): c1 = c_i w_i w_j, c2 = c_j w_i w_j, d = c1 - c2 in complex<float>,
// |d|^2 = d.re d.re + d.im d.im in float; overlap-normalised: sum_k |d|^2 in double (blitz sums float arrays in
// double) / (float) sum_k w_i w_j; otherwise mean: a float running sum / K. depth 1 (the real representation):
// sqrt of sum_{k >= 1} (r_i - r_j)^2 (float squares, double sum). Every pair accumulates sequentially in k with
// each operation rounded on its own, so D matches the CPU bit for bit. One CTA per 32 x 32 tile of the upper
// triangle (tiles with tj >= ti), 256 threads, 4 pairs a thread (one i, four consecutive j); the i and j rows of
// each 32-coefficient chunk staged in shared memory as float4 (re, im, w, 0), k-major. BINARY (every weight 0 or
// 1, as getLowDimensionRepresentationHalf writes them): the weighted values are the values themselves or zeros,
// and the overlap is an integer count, so one FP64 add per pair and coefficient suffices for the same result.
constexpr int RD_T = 32, RD_KC = 32;

template <int DEPTH, bool BINARY>
__global__ void __launch_bounds__(256) k_repr_dist(const float *__restrict__ R, int V, int K, int normalized,
                                                   float *__restrict__ D) {
  __shared__ float4 sI[RD_KC][RD_T], sJ[RD_KC][RD_T];
  // tile (ti, tj) with tj >= ti from the linear block index (row-major over the upper triangle)
  const int nb = (V + RD_T - 1) / RD_T;
  int b = blockIdx.x, ti = 0;
  while (b >= nb - ti) {
    b -= nb - ti;
    ++ti;
  }
  const int tj = ti + b;
  const int i0 = ti * RD_T, j0 = tj * RD_T;
  const int li = threadIdx.x >> 3, lj = (threadIdx.x & 7) * 4;
  double acc[4] = {0.0, 0.0, 0.0, 0.0}, ov[4] = {0.0, 0.0, 0.0, 0.0};
  float accf[4] = {0.f, 0.f, 0.f, 0.f};
  int cnt[4] = {0, 0, 0, 0};
  const int kstart = DEPTH == 1 ? 1 : 0;
  for (int k0 = 0; k0 < K; k0 += RD_KC) {
    for (int t = threadIdx.x; t < 2 * RD_KC * RD_T; t += blockDim.x) {
      const int side = t / (RD_KC * RD_T), r = (t / RD_KC) % RD_T, kk = t % RD_KC;
      const int row = (side ? j0 : i0) + r, k = k0 + kk;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (row < V && k < K) {
        const float *p = R + ((long)row * K + k) * DEPTH;
        v.x = p[0];
        if (DEPTH == 3) {
          v.y = p[1];
          v.z = p[2];
        }
      }
      (side ? sJ : sI)[kk][r] = v;
    }
    __syncthreads();
    const int kn = min(RD_KC, K - k0);
    for (int kk = 0; kk < kn; ++kk) {
      if (k0 + kk < kstart) continue;
      const float4 a = sI[kk][li];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4 c = sJ[kk][lj + q];
        if (DEPTH == 3 && BINARY) {
          // w = 1: c1 - c2 is the plain difference; w = 0: both weighted values are zeros and |d|^2 = +0
          const bool on = a.z != 0.f && c.z != 0.f;
          const float dr = __fsub_rn(a.x, c.x), di = __fsub_rn(a.y, c.y);
          const float t2 = on ? __fadd_rn(__fmul_rn(dr, dr), __fmul_rn(di, di)) : 0.f;
          acc[q] = __dadd_rn(acc[q], (double)t2);
          accf[q] = __fadd_rn(accf[q], t2);
          cnt[q] += on;
        } else if (DEPTH == 3) {
          const float w = __fmul_rn(a.z, c.z);
          const float r1 = __fmul_rn(__fmul_rn(a.x, a.z), c.z), i1 = __fmul_rn(__fmul_rn(a.y, a.z), c.z);
          const float r2 = __fmul_rn(__fmul_rn(c.x, a.z), c.z), i2 = __fmul_rn(__fmul_rn(c.y, a.z), c.z);
          const float dr = __fsub_rn(r1, r2), di = __fsub_rn(i1, i2);
          const float t2 = __fadd_rn(__fmul_rn(dr, dr), __fmul_rn(di, di));
          acc[q] = __dadd_rn(acc[q], (double)t2);
          accf[q] = __fadd_rn(accf[q], t2);
          ov[q] = __dadd_rn(ov[q], (double)w);
        } else {
          const float d = __fsub_rn(a.x, c.x);
          acc[q] = __dadd_rn(acc[q], (double)__fmul_rn(d, d));
        }
      }
    }
    __syncthreads();
  }
  const int i = i0 + li;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int j = j0 + lj + q;
    if (i >= V || j >= V || j <= i) continue;
    float d;
    if (DEPTH == 1) {
      d = (float)sqrt(acc[q]);
    } else {
      const float overlap = BINARY ? (float)cnt[q] : (float)ov[q];
      d = (normalized && overlap > 0) ? (float)(acc[q] / (double)overlap) : __fdiv_rn(accf[q], (float)K);
    }
    D[(long)i * V + j] = d;
    D[(long)j * V + i] = d;
  }
}

// Kept coefficients of getLowDimensionRepresentationHalf: out[e][q] = F[e][idx[q]] (kz-major half spectra of
// h3 entries; idx in the reference's [x][y][kz] order of the band |filter| > 0.5).
static __global__ void k_repr_gather(const float2 *__restrict__ F, int E, long h3, const int *__restrict__ idx, int K,
                                     float2 *__restrict__ out) {
  const long n = (long)E * K;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long)gridDim.x * blockDim.x) {
    const long e = t / K;
    out[t] = F[e * h3 + idx[t - e * K]];
  }
}

// ---- spherical wedge of a class average --------------------------------------------------------
// updateAccumulatedSphericalWedgeImageMPI (inc/em/nbfWedgedAverageImage3D.h:612-648): per sample (i, j) of the
// (2B)^2 grid, the number of members whose binary spherical wedge covers it. Each member's wedge is the analytic
// one of nbfWedge3D::getSphericalImage (inc/em/nbfWedge3D.h:363-429) with its plane normals rotated by the
// inverse of Euler(normal) * alignment: ((v1.d)(v2.d) <= 0) with d = (cos th_j sin ph_i, sin th_j sin ph_i,
// cos ph_i) from the float cos / sin tables trig = [cos th_j | sin th_j | sin ph_i | cos ph_i] (n each), the
// products and sums in FP64 in the reference's order (no contraction). Counts are exact in float.
static __global__ void k_sph_wedge_count(const WedgeVecs *__restrict__ wv, int E, const float *__restrict__ trig, int n,
                                         float *__restrict__ count) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= n * n) return;
  const int i = id / n, j = id - (id / n) * n;
  const double cj = trig[j], sj = trig[n + j], si = trig[2 * n + i], ci = trig[3 * n + i];
  float c = 0.f;
  for (int e = 0; e < E; ++e) {
    const WedgeVecs &w = wv[e];
    if (w.full) {
      c += 1.f;
      continue;
    }
    const double a = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(w.v1[0], cj), si), __dmul_rn(__dmul_rn(w.v1[1], sj), si)),
                               __dmul_rn(w.v1[2], ci));
    const double b = __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(w.v2[0], cj), si), __dmul_rn(__dmul_rn(w.v2[1], sj), si)),
                               __dmul_rn(w.v2[2], ci));
    if (__dmul_rn(a, b) <= 0.0) c += 1.f;
  }
  count[id] = c;
}

// ---- rotational symmetrisation ---------------------------------------------------------------
// src/MPI_Classification.cpp:1005-1024 with nbfCylindricalDomain3 (inc/nbfCylindricalDomain3.h:126-233) and the
// clamped trilinear rule of nbfLinearInterpolator::interpolateSingle (inc/nbfLinearInterpolator.h:186-262), in
// FP64 with every product and sum rounded on its own (no contraction), so that the only departures from the
// CPU arithmetic are the last bits of cos / sin / atan2.

struct CylGeom {
  int N, R, T;                // volume edge, radii N/2, angles 180
  double c, max_rho;          // axis at (N/2, N/2); largest radius N/2
  double rstep, tstep;        // (N/2)/(R-1) and max_theta/(T-1)
  double max_theta, two_pi;   // 2 * float pi of VTK 5.10, both as doubles
};

// Clamped axis rule: at or below 0 -> cell 0, weight 0; at or above n-1 -> cell n-2, weight 1.
ETTK_DEV double cyl_axis(double x, int n, int &f) {
  if (x <= 0.0) {
    f = 0;
    return 0.0;
  }
  if (x >= (double)(n - 1)) {
    f = n - 2;
    return 1.0;
  }
  f = (int)floor(x);
  return __dsub_rn(x, (double)f);
}

// The eight-term blend of interpolateSingle in its order: v000, v100, v010, v001, v101, v011, v110, v111.
ETTK_DEV double cyl_blend(double a, double b, double c, double v000, double v100, double v010, double v001,
                          double v101, double v011, double v110, double v111) {
  const double ia = __dsub_rn(1.0, a), ib = __dsub_rn(1.0, b), ic = __dsub_rn(1.0, c);
  double s = __dmul_rn(__dmul_rn(__dmul_rn(ia, ib), ic), v000);
  s = __dadd_rn(s, __dmul_rn(__dmul_rn(__dmul_rn(a, ib), ic), v100));
  s = __dadd_rn(s, __dmul_rn(__dmul_rn(__dmul_rn(ia, b), ic), v010));
  s = __dadd_rn(s, __dmul_rn(__dmul_rn(__dmul_rn(ia, ib), c), v001));
  s = __dadd_rn(s, __dmul_rn(__dmul_rn(__dmul_rn(a, ib), c), v101));
  s = __dadd_rn(s, __dmul_rn(__dmul_rn(__dmul_rn(ia, b), c), v011));
  s = __dadd_rn(s, __dmul_rn(__dmul_rn(__dmul_rn(a, b), ic), v110));
  return __dadd_rn(s, __dmul_rn(__dmul_rn(__dmul_rn(a, b), c), v111));
}

// cartesian2cylindrical + the angular sum: prof[i][k] = sum over the T angles, in order, of the volume (x
// fastest) interpolated at (c + rho_i cos theta_j, c + rho_i sin theta_j, k). One thread per (radius, plane).
static __global__ void __launch_bounds__(128) k_cyl_profile(const float *__restrict__ vol, CylGeom g,
                                                            double *__restrict__ prof) {
  __shared__ double cs[180], sn[180];
  for (int j = threadIdx.x; j < g.T; j += blockDim.x) {
    const double th = __dadd_rn(__dmul_rn(g.tstep, (double)j), 0.0);
    sincos(th, &sn[j], &cs[j]);
  }
  __syncthreads();
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= g.R * g.N) return;
  const int i = id / g.N, k = id % g.N, N = g.N;
  const double rho = __dadd_rn(__dmul_rn(g.rstep, (double)i), 0.0);
  int zf;
  const double cz = cyl_axis((double)k, N, zf);
  const long NN = (long)N * N;
  double s = 0.0;
  for (int j = 0; j < g.T; ++j) {
    int xf, yf;
    const double a = cyl_axis(__dadd_rn(g.c, __dmul_rn(rho, cs[j])), N, xf);
    const double b = cyl_axis(__dadd_rn(g.c, __dmul_rn(rho, sn[j])), N, yf);
    const float *p = vol + xf + (long)N * yf + NN * zf;
    s = __dadd_rn(s, cyl_blend(a, b, cz, p[0], p[1], p[N], p[NN], p[NN + 1], p[NN + N], p[N + 1], p[NN + N + 1]));
  }
  prof[(long)i * N + k] = s;
}

// cylindrical2cartesian of the angle-independent profile: out (x fastest) at each voxel's radius
// (N/2-1) r / (N/2) and angle atan2(y - c, x - c) (wrapped to [0, 2 pi)) scaled to the T-1 cells.
static __global__ void k_cyl_expand(const double *__restrict__ prof, CylGeom g, float *__restrict__ out) {
  const int N = g.N;
  const long n3 = (long)N * N * N;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < n3; id += (long)gridDim.x * blockDim.x) {
    const int x = (int)(id % N), y = (int)((id / N) % N), z = (int)(id / ((long)N * N));
    const double dx = __dsub_rn(g.c, (double)x), dy = __dsub_rn(g.c, (double)y);
    double r = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    r = __dmul_rn(__ddiv_rn(r, g.max_rho), (double)(g.R - 1));
    double t = atan2(__dsub_rn((double)y, g.c), __dsub_rn((double)x, g.c));
    if (t < 0.0) t = __dadd_rn(t, g.two_pi);
    t = __dmul_rn(__ddiv_rn(t, g.max_theta), (double)(g.T - 1));
    int rf, tf, zf;
    const double a = cyl_axis(r, g.R, rf), b = cyl_axis(t, g.T, tf), c = cyl_axis((double)z, N, zf);
    const double *p = prof + (long)rf * N + zf;  // the profile at (rf, zf); the angle index selects nothing
    out[id] = (float)cyl_blend(a, b, c, p[0], p[N], p[0], p[1], p[N + 1], p[1], p[N], p[N + 1]);
  }
}

// ---- spherical projection ------------------------------------------------------------------

// mean over all voxels of the mean-subtracted particle (nbfImageFilter::execute meanValue,
// inc/em/nbfImageFilter.h:255) -> acc[slot]
static __global__ void k_mean_all(const float *__restrict__ v, const double *acc_in, int acc_stride, int N, double *acc_out,
                           int slot) {
  __shared__ double sh[32];
  long n3 = (long)N * N * N;
  const double *a = acc_in + (long)blockIdx.y * acc_stride;
  float mean = (float)(a[0] / (double)(float)a[1]);
  float s = 0.f;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < n3; id += (long)gridDim.x * blockDim.x) {
    float x = v[(long)blockIdx.y * n3 + id];
    s += (x > -FLT_MAX) ? (x - mean) : 0.f;
  }
  double b = block_sum((double)s, sh);
  if (threadIdx.x == 0) atomicAdd(&acc_out[(long)blockIdx.y * acc_stride + slot], b);
}

// Padded, windowed, shifted (2N)^3 input of cartesianToSpherical (inc/em/nbfProjectionRotationMetric3D.h:271-318):
// x<N,y<N,z<N: (img - meanAll)*mask + meanAll; elsewhere the corner value; times (-1)^(x+y+z).
struct PrePadded {
  const float *v;
  const float *mask;
  const double *acc;
  int acc_stride, N;
  long cached = -1;  // per-thread: item whose means are cached
  float mean = 0.f, meanAll = 0.f;
  ETTK_DEV void begin() {}
  ETTK_DEV void end() {}
  ETTK_DEV void load(long e) {
    const double *a = acc + e * acc_stride;
    mean = (float)(a[0] / (double)(float)a[1]);
    meanAll = (float)(a[2] / (double)((long)N * N * N));
    cached = e;
  }
  ETTK_DEV float windowed(long e, long id) {
    if (e != cached) load(e);
    float x = v[e * (long)N * N * N + id];
    float img = (x > -FLT_MAX) ? x - mean : 0.f;
    return (img - meanAll) * mask[id] + meanAll;
  }
  static constexpr bool kPadLines = true;
  // the z pass of a padding line writes only its kz = N2/2 entry (the padded magnitude pass of k_fft2d_padded
  // reads no other plane of such a line)
  bool nyquist_only = false;
  // the z pass runs over the lines x < N, y < N alone, in tiles of RL consecutive y (RL divides N); the padding
  // lines' only nonzero entry, N2 c (-1)^(x+y) at kz = N2/2, is supplied by the magnitude pass of that plane
  bool real_only = false;
  static constexpr bool kLineBase = true;
  ETTK_DEV long line_base(long tile, int RL) const {
    const int N2 = 2 * N, per_row = N / RL;
    const long per_item = (long)N * per_row;
    const long e = tile / per_item, r = tile - e * per_item;
    const int x = (int)(r / per_row), yb = (int)(r - (long)x * per_row);
    return e * N2 * N2 + (long)x * N2 + (long)yb * RL;
  }
  ETTK_HD long real_tiles(long lines, int RL) const {
    const long N2 = 2 * N;
    return lines / (N2 * N2) * N * (N / RL);
  }
  // line (x, y) with x >= N or y >= N lies wholly in the padding: r[z] = c (-1)^(x+y+z)
  ETTK_DEV bool pad_line(long line, float &c, float &sign_xy) {
    const int N2 = 2 * N;
    const long per = (long)N2 * N2;
    const long e = line / per;
    const int r = (int)(line - e * per), x = r / N2, y = r - x * N2;
    if (x < N && y < N) return false;
    c = windowed(e, 0);
    sign_xy = ((x + y) & 1) ? -1.f : 1.f;
    return true;
  }
  long cl[2] = {-1, -1}, ce[2] = {0, 0};  // two-slot line cache (slot = line & 1)
  int cx[2] = {0, 0}, cy[2] = {0, 0};
  ETTK_DEV float operator()(long line, int z) {
    const int sl = (int)(line & 1);
    if (line != cl[sl]) {
      const int N2 = 2 * N;
      long per = (long)N2 * N2;
      ce[sl] = line / per;
      int r = (int)(line - ce[sl] * per);
      cx[sl] = r / N2;
      cy[sl] = r % N2;
      cl[sl] = line;
    }
    const int x = cx[sl], y = cy[sl];
    float val = (x < N && y < N && z < N) ? windowed(ce[sl], ((long)x * N + y) * N + z) : windowed(ce[sl], 0);
    return val * parity_sign(x, y, z);
  }
};

// |F| of the (2N)^3 half spectrum, or |F|^(1/2) with mutual correlation (inc/em/nbfProjectionRotationMetric3D.h:318-325)
ETTK_DEV float spectrum_magnitude(float2 f, int mutual) {
  const float m = sqrtf(f.x * f.x + f.y * f.y);
  return mutual ? sqrtf(m) : m;
}
static __global__ void k_magnitude(const float2 *__restrict__ F, float *__restrict__ M, long n, int mutual) {
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < n; id += (long)gridDim.x * blockDim.x)
    M[id] = spectrum_magnitude(F[id], mutual);
}

// nbfFourierFilter::executeHalf with mutual correlation (inc/em/nbfFourierFilter.h:590-595): F / |F|^(1/2) where
// |F| > 0, on n spectrum values in place
ETTK_DEV float2 mutual_scale(float2 f) {
  const float C = sqrtf(sqrtf(f.x * f.x + f.y * f.y));
  return C > 0.f ? make_float2(f.x / C, f.y / C) : f;
}
static __global__ void k_mutual_scale(float2 *__restrict__ F, long n) {
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < n; id += (long)gridDim.x * blockDim.x)
    F[id] = mutual_scale(F[id]);
}

// Cubic resampling on radial shells through vtkSphericalTransform with wrap, summed over the
// radii [bandL, bandU] (lines 359-406): Pp[e][j][k] for polar j, azimuth k. The taps read the virtual
// Hermitian-completed magnitude cube (lines 327-338): z <= N from the stored kz-major half volume [z <= N][x][y],
// the x = 0 plane zero, z > N mirrored through (N, N, N) except on the y = 0 plane, which keeps the padded
// real-space value (the corner value).
// 2N is a power of two, so the wrap of the tap indices is a mask; the mirror offsets are hoisted per axis.
template <int N>
__global__ void __launch_bounds__(256) k_sphere_sample(const float *__restrict__ Mh, const float4 *__restrict__ dirs,
                                                       int n_dirs, int bandL, int bandU, const float *__restrict__ padc,
                                                       float *__restrict__ Pp, const int *__restrict__ out_index) {
  constexpr int N2 = 2 * N, H = N + 1, MSK = N2 - 1;
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= n_dirs) return;
  const int e = blockIdx.y;
  const float *M = Mh + (long)e * N2 * N2 * H;
  const float4 u = dirs[d];
  const float pc = padc[e];
  float acc = 0.f;
  for (int r = bandL; r <= bandU; ++r) {
    const float p0 = r * u.x + (float)N, p1 = r * u.y + (float)N, p2 = r * u.z + (float)N;
    float fx, fy, fz;
    const int ix = vtk_floor(p0, fx), iy = vtk_floor(p1, fy), iz = vtk_floor(p2, fz);
    float wx[4], wy[4], wz[4];
    cubic_weights(wx, fx);
    cubic_weights(wy, fy);
    cubic_weights(wz, fz);
    // the reference uses only the middle row/plane when fy/fz == 0 (the forced (0, 1, 0, 0) weights add zeros)
    if (fy == 0.f) { wy[0] = 0.f; wy[1] = 1.f; wy[2] = 0.f; wy[3] = 0.f; }
    if (fz == 0.f) { wz[0] = 0.f; wz[1] = 1.f; wz[2] = 0.f; wz[3] = 0.f; }
    int xo[4], xm[4];
    bool x0[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int x = (ix - 1 + t) & MSK;
      x0[t] = x == 0;
      xo[t] = x * N2;
      xm[t] = ((N2 - x) & MSK) * N2;
    }
    float v = 0.f;
    // Taps with 1 <= y <= 2N - 1 on all four rows (every sample inside the band): each row of four consecutive y
    // (or, mirrored, four consecutive 2N - y) is read as one or two aligned 16-byte quads, a quarter to half of
    // the per-tap load instructions; the sum keeps the order of the per-tap path below, so the values agree bit
    // for bit.
    const int y0 = iy - 1;
    if (y0 >= 1 && y0 + 3 <= MSK) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int z = (iz - 1 + k) & MSK;
        const bool mir = z > N;
        const int zo = (mir ? N2 - z : z) * N2 * N2;
        const int ys = mir ? N2 - y0 - 3 : y0;  // first y of the row's run in memory
        const int s = ys & 3;
        float g[4][4];                          // [j][t]
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const float *row = M + zo + (mir ? xm[t] : xo[t]) + (ys - s);
          const float4 a = __ldg(reinterpret_cast<const float4 *>(row));
          const float4 b = s ? __ldg(reinterpret_cast<const float4 *>(row + 4)) : make_float4(0.f, 0.f, 0.f, 0.f);
          float r[4];
          switch (s) {
            case 0: r[0] = a.x; r[1] = a.y; r[2] = a.z; r[3] = a.w; break;
            case 1: r[0] = a.y; r[1] = a.z; r[2] = a.w; r[3] = b.x; break;
            case 2: r[0] = a.z; r[1] = a.w; r[2] = b.x; r[3] = b.y; break;
            default: r[0] = a.w; r[1] = b.x; r[2] = b.y; r[3] = b.z; break;
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) g[j][t] = x0[t] ? 0.f : (mir ? r[3 - j] : r[j]);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
          v += (wz[k] * wy[j]) * (wx[0] * g[j][0] + wx[1] * g[j][1] + wx[2] * g[j][2] + wx[3] * g[j][3]);
      }
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int z = (iz - 1 + k) & MSK;
        const bool mir = z > N;
        const int zo = (mir ? N2 - z : z) * N2 * N2;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int y = (iy - 1 + j) & MSK;
          float g[4];
          if (!mir) {
            const int base = zo + y;
#pragma unroll
            for (int t = 0; t < 4; ++t) g[t] = x0[t] ? 0.f : __ldg(M + base + xo[t]);
          } else if (y == 0) {
#pragma unroll
            for (int t = 0; t < 4; ++t) g[t] = x0[t] ? 0.f : pc;
          } else {
            const int base = zo + (N2 - y);
#pragma unroll
            for (int t = 0; t < 4; ++t) g[t] = x0[t] ? 0.f : __ldg(M + base + xm[t]);
          }
          v += (wz[k] * wy[j]) * (wx[0] * g[0] + wx[1] * g[1] + wx[2] * g[2] + wx[3] * g[3]);
        }
      }
    }
    acc += v;
  }
  Pp[(long)(out_index ? out_index[e] : e) * n_dirs + d] = acc;
}

// *flag |= 1 when v[0..n) holds a NaN or an infinity (exponent field all ones); 16-byte loads, grid-stride.
static __global__ void k_nonfinite(const float *__restrict__ v, long n, int *flag) {
  const uint4 *q = reinterpret_cast<const uint4 *>(v);
  const long n4 = n >> 2;
  uint32_t any = 0;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (long)gridDim.x * blockDim.x) {
    const uint4 u = __ldg(q + i);
    any |= ((u.x & 0x7f800000u) == 0x7f800000u) | ((u.y & 0x7f800000u) == 0x7f800000u) |
           ((u.z & 0x7f800000u) == 0x7f800000u) | ((u.w & 0x7f800000u) == 0x7f800000u);
  }
  for (long i = (n4 << 2) + (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    any |= (__float_as_uint(v[i]) & 0x7f800000u) == 0x7f800000u;
  if (__syncthreads_or(any) && threadIdx.x == 0) atomicOr(flag, 1);
}

// Corner value of the windowed image (the pad constant).
static __global__ void k_pad_constant(PrePadded pre, int n_items, float *padc) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n_items) padc[e] = pre.windowed(e, 0);
}

// ---- SO(3) stage ---------------------------------------------------------------------------

// Forward S^2 transform of real signals [J][2B][2B] -> coef[J][l][m] (m >= 0), one CTA per signal:
// phi-FFT of each polar row then the quadrature sum with lw[m][l][j] = sqrt(2pi)/2B w_j P~_l^m(theta_j)
// (SOFT FST_semi_memo, external/soft-1.0/FST_semi_memo.c:134-357).
template <int B>
static __global__ void k_sht(const float *__restrict__ sig, const float *__restrict__ lw, float2 *__restrict__ coef) {
  constexpr int n = 2 * B;
  extern __shared__ float2 smem[];
  float2 *tw = smem;
  float2 *s = smem + n / 2;
  load_twiddles<n>(tw);
  const float *x = sig + (long)blockIdx.x * n * n;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    int j = idx / n, k = idx - j * n;
    s[j * n + bitrev<n>(k)] = make_float2(x[idx], 0.f);
  }
  block_fft<n>(s, n, -1, tw);
  float2 *out = coef + (long)blockIdx.x * B * B;
  for (int idx = threadIdx.x; idx < B * B; idx += blockDim.x) {
    int l = idx / B, m = idx - l * B;
    float2 acc = make_float2(0.f, 0.f);
    if (m <= l) {
      const float *w = lw + ((long)m * B + l) * n;
      for (int j = 0; j < n; ++j) acc = cadd(acc, cscale(s[j * n + m], w[j]));
    }
    out[idx] = acc;
  }
}

ETTK_DEV float2 coef_at(const float2 *c, int B, int l, int m) {
  // real-signal symmetry f(l,-m) = (-1)^m conj f(l,m)
  if (m >= 0) return c[l * B + m];
  float2 v = cconj(c[l * B - m]);
  return ((-m) & 1) ? cscale(v, -1.f) : v;
}

// Wigner-d synthesis of the SO(3) correlation (so3CombineCoef_fftw, so3_correlate_fftw.c:103-162, and the
// inverse Wigner transform of Inverse_SO3_Naive_fftw, soft_fftw.c:1045-1840):
// S[job][b][m1][m2] = sum_l F^l_{m1 m2} dt^l_{m1 m2}(beta_b), F = f(l,-m1) conj(h(l,-m2)) (-1)^(m1+m2).
// One CTA per (m1,m2) cell and block of jobs; the d table slice lives in shared memory.
struct SynthJob {
  int f, h;  // signal indices of the two coefficient sets
};
template <int B>
static __global__ void k_so3_synth(const float2 *__restrict__ coef, const SynthJob *__restrict__ jobs, int n_jobs,
                            const float *__restrict__ dtab, const int *__restrict__ doff, float2 *__restrict__ S) {
  constexpr int n = 2 * B;
  __shared__ float sd[B * n];
  __shared__ float2 sF[8][B];
  int cell = blockIdx.x;
  int m1 = cell / (2 * B - 1) - (B - 1), m2 = cell % (2 * B - 1) - (B - 1);
  int l0 = max(abs(m1), abs(m2));
  int L = B - l0;
  const float *d = dtab + doff[cell];
  for (int i = threadIdx.x; i < L * n; i += blockDim.x) sd[i] = d[i];
  int sgn = ((m1 + m2) & 1) ? -1 : 1;
  for (int j0 = blockIdx.y * 8; j0 < n_jobs; j0 += gridDim.y * 8) {
    __syncthreads();
    for (int i = threadIdx.x; i < 8 * L; i += blockDim.x) {
      int jl = i / L, l = l0 + (i - jl * L);
      float2 F = make_float2(0.f, 0.f);
      if (j0 + jl < n_jobs) {
        SynthJob jb = jobs[j0 + jl];
        float2 a = coef_at(coef + (long)jb.f * B * B, B, l, -m1);
        float2 b = coef_at(coef + (long)jb.h * B * B, B, l, -m2);
        F = cscale(cmul(a, cconj(b)), (float)sgn);
      }
      sF[jl][l - l0] = F;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 8 * n; i += blockDim.x) {
      int jl = i / n, b = i - jl * n;
      if (j0 + jl >= n_jobs) continue;
      float2 acc = make_float2(0.f, 0.f);
      for (int t = 0; t < L; ++t) acc = cadd(acc, cscale(sF[jl][t], sd[t * n + b]));
      int mm1 = (m1 + n) % n, mm2 = (m2 + n) % n;
      S[(((long)(j0 + jl) * n + mm1) * n + mm2) * n + b] = acc;
    }
  }
}

// Real part and scale (1/2B)(B/pi) of the alpha/gamma-transformed synthesis S[job][a][g][b] into
// C[job][a][b][g] (soft_fftw.c:1913-1920; nbfProjectionRotationMetric3D.h:1254-1265), with packed min/max per job
// in the memory order of C (rotatedSphericalImageMinMax, 1557-1589). One CTA per (a, job) transposes the (g, b)
// plane through shared memory in blocks of 32 g rows (coalesced reads along b, writes along g).
template <int B>
static __global__ void __launch_bounds__(256) k_so3_real(const float2 *__restrict__ S, float *__restrict__ C,
                                                         unsigned long long *mm) {
  constexpr int n = 2 * B, GT = 32 < n ? 32 : n;
  __shared__ float tile[GT][n + 1];
  const int a = blockIdx.x, job = blockIdx.y;
  const float scale = (1.0f / n) * ((float)B / 3.14159265358979f);
  const float2 *Sa = S + ((long)job * n + a) * n * n;
  float *Ca = C + ((long)job * n + a) * n * n;
  unsigned long long bmax = 0, bmin = 0;
  for (int g0 = 0; g0 < n; g0 += GT) {
    __syncthreads();
    for (int i = threadIdx.x; i < GT * n; i += blockDim.x) {
      const int gl = i / n, bb = i - gl * n;
      tile[gl][bb] = Sa[(long)(g0 + gl) * n + bb].x * scale;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < GT * n; i += blockDim.x) {
      const int bb = i / GT, gl = i - bb * GT;
      const float v = tile[gl][bb];
      Ca[(long)bb * n + g0 + gl] = v;
      const uint32_t id = (uint32_t)((a * n + bb) * n + g0 + gl);
      const unsigned long long kx = pack_max(v, id), kn = pack_min(v, id);
      bmax = kx > bmax ? kx : bmax;
      bmin = kn > bmin ? kn : bmin;
    }
  }
  if (mm) {  // one pair of atomics per block
    __shared__ unsigned long long red[2][32];
    bmax = warp_max_u64(bmax);
    bmin = warp_max_u64(bmin);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if (lane == 0) {
      red[0][wid] = bmin;
      red[1][wid] = bmax;
    }
    __syncthreads();
    if (wid == 0) {
      bmin = lane < nw ? red[0][lane] : 0ull;
      bmax = lane < nw ? red[1][lane] : 0ull;
      bmin = warp_max_u64(bmin);
      bmax = warp_max_u64(bmax);
      if (lane == 0) {
        atomicMax(&mm[2 * job + 0], bmin);
        atomicMax(&mm[2 * job + 1], bmax);
      }
    }
  }
}

// softScaled weights (nbfProjectionRotationMetric3D.h:1297-1319): rotate the pattern (coefficients h) to the
// Euler angles of the min (which=0) / max (which=1) cell, synthesise it on the grid and return
// sum(F1 * R * sin(theta)). Rotation: g(l,m) = sum_m' e^{-i m alpha} d^l_{m m'}(beta) e^{-i m' gamma} h(l,m')
// (rotateFct, rotate_so3.c:695-741); R = (1/sqrt(2pi)) Re sum_{l,m} g(l,m) P~_l^m(theta_j) e^{i m phi_k}.
struct ScaledJob {
  int h;      // coefficient index of the pattern
  int f1sig;  // signal index of F1
  int job;    // correlation job (for the min/max cells)
};
template <int B>
constexpr size_t so3_weights_smem() { return (size_t)3 * B * B * sizeof(float2); }
template <int B>
static __global__ void __launch_bounds__(256) k_so3_weights(const ScaledJob *__restrict__ sj,
                                                            const unsigned long long *__restrict__ mm,
                                                            const float2 *__restrict__ coef,
                                                            const float *__restrict__ sig,
                                                            const float *__restrict__ dtab, const int *__restrict__ doff,
                                                            const float *__restrict__ plm,
                                                            const float *__restrict__ sinth, double *w) {
  constexpr int n = 2 * B;
  extern __shared__ float2 wsm2[];   // so3_weights_smem<B>() bytes
  float2 *g = wsm2;                  // rotated coefficients g(l, m), m >= 0: [l][m]
  float2 *Hs = wsm2 + B * B;         // H(j, m) = sum_l g(l, m) P~_l^m(theta_j): [j][m]
  __shared__ float2 ea[B], eg[2 * B - 1], ep[n];
  __shared__ double sh[32];
  const ScaledJob J = sj[blockIdx.x];
  const int which = blockIdx.y;
  const unsigned long long key = mm[2 * J.job + which];
  const uint32_t pos = 0xffffffffu - (uint32_t)(key & 0xffffffffu);
  const int a = pos / (n * n), b = (pos / n) % n, gg = pos % n;
  const float alpha = (float)(a / (double)B * 3.141592653589793), gamma = (float)(gg / (double)B * 3.141592653589793);
  // phase tables: e^{-i m alpha} (m >= 0), e^{-i m' gamma} (|m'| < B), e^{2 pi i t / n}
  for (int t = threadIdx.x; t < 2 * B - 1; t += blockDim.x) {
    float s1, c1;
    sincosf(-((t - (B - 1)) * gamma), &s1, &c1);
    eg[t] = make_float2(c1, s1);
    if (t < B) {
      sincosf(-(t * alpha), &s1, &c1);
      ea[t] = make_float2(c1, s1);
    }
  }
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    float s1, c1;
    sincospif(2.0f * t / n, &s1, &c1);
    ep[t] = make_float2(c1, s1);
  }
  __syncthreads();
  const float2 *h = coef + (long)J.h * B * B;
  for (int idx = threadIdx.x; idx < B * B; idx += blockDim.x) {
    const int l = idx / B, m = idx - l * B;
    float2 acc = make_float2(0.f, 0.f);
    if (m <= l) {
      const float nl = rsqrtf((2.0f * l + 1.0f) * 0.5f);
      for (int mp = -l; mp <= l; ++mp) {
        const int cell = (m + B - 1) * (2 * B - 1) + (mp + B - 1);
        const int l0 = max(abs(m), abs(mp));
        const float dv = dtab[doff[cell] + (l - l0) * n + b] * nl;
        acc = cadd(acc, cscale(cmul(eg[mp + B - 1], coef_at(h, B, l, mp)), dv));
      }
      acc = cmul(ea[m], acc);
    }
    g[idx] = acc;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < n * B; idx += blockDim.x) {
    const int j = idx / B, m = idx - j * B;
    float2 hm = make_float2(0.f, 0.f);
    for (int l = m; l < B; ++l) hm = cadd(hm, cscale(g[l * B + m], plm[((long)m * B + l) * n + j]));
    Hs[idx] = hm;
  }
  __syncthreads();
  const float *F1 = sig + (long)J.f1sig * n * n;
  double s = 0;
  const float inv = 0.3989422804014327f;
  for (int idx = threadIdx.x; idx < n * n; idx += blockDim.x) {
    const int j = idx / n, k = idx - j * n;
    const float2 *Hj = Hs + j * B;
    float r = Hj[0].x;
    for (int m = 1; m < B; ++m) {
      const float2 e = ep[(m * k) & (n - 1)];
      r += 2.f * (Hj[m].x * e.x - Hj[m].y * e.y);
    }
    r *= inv;
    s += (double)F1[idx] * (double)r * (double)sinth[j];
  }
  const double bsum = block_sum(s, sh);
  if (threadIdx.x == 0) w[2 * blockIdx.x + which] = bsum;
}

}  // namespace ettk
