// libettk_gpu: GB300 implementation of ETTK's pairwise sub-volume alignment
// (nbfProjectionRotationMetric3D<float>::execute, alignment_mode 3) behind the C ABI of
// include/ettk_gpu.h. Host orchestration: batches of (reference, particle) pairs go through
//   1. |FFT| spherical projection of each particle (cartesianToSpherical),
//   2. SO(3) correlations on the GPU (S^2 transform, Wigner-d synthesis, alpha/gamma FFT,
//      softScaled rescaling) and 3x3x3 local-maximum extraction,
//   3. per-pair candidate queues on the host (getTrueLocalMaximaPositions,
//      eliminateEquivalentAngles, the mirror test and its counting rule),
//   4. batched translational CCF evaluations (executeFourierNewHalf) in rounds until every
//      pair's queues are exhausted or have counted candidatePeaks peaks,
//   5. final candidate selection (eliminateEquivalentAngles with tolerance 2.5).
#include "../../include/ettk_gpu.h"
#include <cuda.h>
#include <cudaTypedefs.h>
#include "geometry.hpp"
#include "kernels.cuh"
#include "fft_reg.cuh"
#include "fft2d.cuh"
#include "wigner_tc.cuh"
#include "refine.cuh"
#include "local_refine.cuh"

#include <algorithm>
#include <atomic>
#include <thread>
#include <condition_variable>
#include <functional>
#include <unistd.h>
#include <type_traits>
#include <array>
#include <chrono>
#include <map>
#include <mutex>
#include <memory>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <queue>
#include <stdexcept>
#include <string>
#include <vector>
#include <cmath>
#include <limits>

using namespace ettk;

namespace {

struct CudaError : std::runtime_error {
  int code;
  CudaError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// cuTensorMapEncodeTiled from the driver, resolved once (null if unavailable: the kernels then stage
// through the threads).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// Host-encoded tensor maps of `count` consecutive N^3 float volumes (x fastest) with the reslice box
// RT_X x RT_Y x RT_Z. Returns false (and no maps) where the box does not fit or encoding fails.
bool encode_volume_maps(const float *base, int count, int N, std::vector<CUtensorMap> &maps, const int *dims3 = nullptr) {
  maps.clear();
  auto enc = tensor_map_encoder();
  const int nx = dims3 ? dims3[0] : N, ny = dims3 ? dims3[1] : N, nz = dims3 ? dims3[2] : N;
  if (!enc || nx < RT_X || ny < RT_Y || nz < RT_Z || (nx & 3) || (((unsigned long long)base) & 15)) return false;
  maps.resize(count);
  const long n3 = (long)nx * ny * nz;
  const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[2] = {(cuuint64_t)nx * 4, (cuuint64_t)nx * ny * 4};
  const cuuint32_t box[3] = {RT_X, RT_Y, RT_Z}, es[3] = {1, 1, 1};
  for (int v = 0; v < count; ++v)
    if (enc(&maps[v], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)(base + v * n3), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
      maps.clear();
      return false;
    }
  return true;
}

// Output-index -> input-index map of a reslice item, in FP32 (default kernels) and FP64 (exact variant).
inline void set_map(ResliceItem &it, const double m12[12]) {
  for (int k = 0; k < 12; ++k) {
    it.m[k] = (float)m12[k];
    it.md[k] = m12[k];
  }
}

#define CK(x)                                                                                     \
  do {                                                                                            \
    cudaError_t e_ = (x);                                                                         \
    if (e_ != cudaSuccess)                                                                        \
      throw CudaError(e_ == cudaErrorMemoryAllocation ? ETTK_ERR_OOM : ETTK_ERR_CUDA,             \
                      std::string(#x) + ": " + cudaGetErrorString(e_));                           \
  } while (0)

// Calls f(std::integral_constant<int, N>) for the supported volume sizes (kernels templated on N).
template <class F>
void with_n(int N, F f) {
  switch (N) {
    case 16: f(std::integral_constant<int, 16>{}); break;
    case 32: f(std::integral_constant<int, 32>{}); break;
    case 64: f(std::integral_constant<int, 64>{}); break;
    case 128: f(std::integral_constant<int, 128>{}); break;
    default: throw CudaError(ETTK_ERR_ARG, "unsupported volume size");
  }
}

inline int ilog2(long v) {
  int r = 0;
  while ((1L << r) < v) ++r;
  return r;
}

// Host table in [x][y][kz] order (kz < N/2+1) -> the kz-major order of the device spectra, [kz][x][y].
inline std::vector<float> to_kz_major(const float *src, int N) {
  const int H = N / 2 + 1;
  std::vector<float> out((size_t)N * N * H);
  for (int x = 0; x < N; ++x)
    for (int y = 0; y < N; ++y)
      for (int k = 0; k < H; ++k) out[((size_t)k * N + x) * N + y] = src[((size_t)x * N + y) * H + k];
  return out;
}

template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  void ensure(size_t count) {
    if (count <= n) return;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    CK(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
    n = count;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }  // buffers of a context are freed with it (ettk_gpu_destroy makes the device current)
};

// Rotation search bookkeeping (TinyVector<float,4>: alpha, beta, gamma, value) with an index that
// rides along without taking part in comparisons, so heap order matches the reference's
// PriorityQueue<TinyVector<Pixel,4>, greaterPD> (inc/fm/nbfFastMarching.h:18-35).
struct Cand {
  float v[4];
  int ref;  // eval slot of the direct CCF (combined list) or -1
};
struct GreaterPD {
  bool operator()(const Cand &a, const Cand &b) const { return a.v[3] > b.v[3]; }
};
typedef std::priority_queue<Cand, std::vector<Cand>, GreaterPD> PQ;

enum SigKind {
  K_PP1, K_PP2, K_W1, K_W2, K_PP1SQ_W1, K_PP2SQ_W2, K_PP1_W1, K_PP2_W2, K_PP2SQ, K_W1_PP1, K_PP1SQ, K_W2_PP2
};

struct SigDesc {
  int pair, kind;
};

// per-pair signal assembly: Pp normalised by the common maximum (execute, 468-470), then the float
// products the reference forms before each soft call (526-584).
__global__ void k_build_signals(const SigDesc *__restrict__ sd, const int *__restrict__ pair_ref,
                                const int *__restrict__ pair_pp2, const float *__restrict__ Pp1,
                                const float *__restrict__ Pp2, const float *__restrict__ W1, const float *__restrict__ W2,
                                const int *__restrict__ pair_part, int nn, float *__restrict__ out) {
  __shared__ float smax[2][32];
  const SigDesc d = sd[blockIdx.x];
  const float *p1 = Pp1 + (long)pair_ref[d.pair] * nn;
  const float *p2 = Pp2 + (long)pair_pp2[d.pair] * nn;
  const float *w1 = W1 + (long)pair_ref[d.pair] * nn;
  const float *w2 = W2 + (long)pair_part[d.pair] * nn;
  float m1 = -FLT_MAX, m2 = -FLT_MAX;
  for (int i = threadIdx.x; i < nn; i += blockDim.x) {
    m1 = fmaxf(m1, p1[i]);
    m2 = fmaxf(m2, p2[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    smax[0][threadIdx.x >> 5] = m1;
    smax[1][threadIdx.x >> 5] = m2;
  }
  __syncthreads();
  float M = -FLT_MAX;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) M = fmaxf(M, fmaxf(smax[0][w], smax[1][w]));
  float *o = out + (long)blockIdx.x * nn;
  for (int i = threadIdx.x; i < nn; i += blockDim.x) {
    float a = p1[i] / M, b = p2[i] / M, wa = w1[i], wb = w2[i], v;
    switch (d.kind) {
      case K_PP1: v = a; break;
      case K_PP2: v = b; break;
      case K_W1: v = wa; break;
      case K_W2: v = wb; break;
      case K_PP1SQ_W1: v = a * a * wa; break;
      case K_PP2SQ_W2: v = b * b * wb; break;
      case K_PP1_W1: v = a * wa; break;
      case K_PP2_W2: v = b * wb; break;
      case K_PP2SQ: v = b * b; break;
      case K_W1_PP1: v = wa * a; break;
      case K_PP1SQ: v = a * a; break;
      default: v = wb * b; break;
    }
    o[i] = v;
  }
}

// The SO(3) correlation jobs of one pair and how execute combines them (526-602).
struct PairPlan {
  int branch;   // 1 both windows, 2 only window 1, 3 only window 2, 4 none
  int job[5];   // correlation job per slot (-1 unused)
  int scaled[5];
  int sjob[5];  // scaled-job index for weights (-1 if unscaled)
};
// Branch combination and local maxima in one pass (execute 526-646): each CTA owns an 8^3 tile of one pair's
// (2B)^3 grid, forms q1 (and q2 where the pair has the unwindowed correlation) on the tile and its one-cell halo in shared memory, then applies
// the 3x3x3 ">=" test with the -FLT_MAX border on the interior (localMaxima3D3x3, inc/em/nbfProjectionRotationMetric3D.h:
// 67-79; BordStrategyConst, inc/bs/nbfBordStrategyConst.h:67-83) and appends the maxima (cell index, value) to the
// pair's lists (order fixed on the host by sorting on the cell index); q1 and q2 are never written to memory.
// Per cell: the softScaled rescale of each scaled job to [wmin, wmax] (1297-1319), the branch formula of execute
// (526-584) and -FLT_MAX on the beta rows from rstart (602). Cells inside the -FLT_MAX plateau of a restricted
// rotation search are maxima of value -FLT_MAX for the reference too; they enter its queues as FLT_MAX sentinels,
// which sort after every real candidate, lose every duplicate comparison and stop the candidate loop only once no
// real candidate is left (697-701), so leaving them out changes no result.
constexpr int CP_T = 8, CP_H = CP_T + 2;
__global__ void __launch_bounds__(256) k_combine_peaks(const PairPlan *__restrict__ plans, const float *__restrict__ C,
                                                       const unsigned long long *__restrict__ mm,
                                                       const double *__restrict__ w, int n, int rstart, int P, int cap,
                                                       int *counts, int2 *lists) {
  __shared__ float qs[2][CP_H * CP_H * CP_H];
  __shared__ float lo[5], sc[5], wl[5];
  __shared__ PairPlan Psh;
  const int pair = blockIdx.y;
  if (threadIdx.x == 0) {
    const PairPlan Pl = plans[pair];
    Psh = Pl;
    for (int s = 0; s < 5; ++s) {
      lo[s] = 0.f;
      sc[s] = 1.f;
      wl[s] = 0.f;
      if (Pl.job[s] >= 0 && Pl.scaled[s]) {
        const float mn = ordered_to_float(~(uint32_t)(mm[2 * Pl.job[s]] >> 32));
        const float mx = ordered_to_float((uint32_t)(mm[2 * Pl.job[s] + 1] >> 32));
        const double wmin = w[2 * Pl.sjob[s]], wmax = w[2 * Pl.sjob[s] + 1];
        lo[s] = mn;
        sc[s] = (float)((wmax - wmin) / ((double)mx - (double)mn));
        wl[s] = (float)wmin;
      }
    }
  }
  __syncthreads();
  const PairPlan &Pl = Psh;
  const bool two = Pl.job[4] >= 0;
  const int tpa = n / CP_T;
  const int ta = blockIdx.x / (tpa * tpa), tb = (blockIdx.x / tpa) % tpa, tg = blockIdx.x % tpa;
  const int a0 = ta * CP_T - 1, b0 = tb * CP_T - 1, g0 = tg * CP_T - 1;
  const int n3 = n * n * n;
  for (int v = threadIdx.x; v < CP_H * CP_H * CP_H; v += blockDim.x) {
    const int la = v / (CP_H * CP_H), lb = (v / CP_H) % CP_H, lg = v % CP_H;
    const int aa = a0 + la, bb = b0 + lb, g = g0 + lg;
    float r1 = -FLT_MAX, r2 = -FLT_MAX;
    if (aa >= 0 && bb >= 0 && g >= 0 && aa < n && bb < n && g < n && bb < rstart) {
      const int id = (aa * n + bb) * n + g;
      float c[5];
#pragma unroll
      for (int s = 0; s < 5; ++s) c[s] = Pl.job[s] >= 0 ? (C[(long)Pl.job[s] * n3 + id] - lo[s]) * sc[s] + wl[s] : 0.f;
      if (Pl.branch == 1) {
        float c1 = sqrtf(c[0]) * sqrtf(c[1]);
        c1 = 2.0f * (1.0f - c[2] / c1);
        r1 = -c1 / c[3];
      } else if (Pl.branch == 2 || Pl.branch == 3) {
        r1 = c[1] / sqrtf(c[0]);
      } else {
        r1 = c[0];
      }
      r2 = c[4];
    }
    qs[0][v] = r1;
    qs[1][v] = r2;
  }
  __syncthreads();
  for (int q = 0; q < (two ? 2 : 1); ++q) {
    const float *Q = qs[q];
    for (int v = threadIdx.x; v < CP_T * CP_T * CP_T; v += blockDim.x) {
      const int la = v / (CP_T * CP_T) + 1, lb = (v / CP_T) % CP_T + 1, lg = v % CP_T + 1;
      const int c0 = (la * CP_H + lb) * CP_H + lg;
      const float val = Q[c0];
      bool ismax = fabsf(val) > 0.f && val != -FLT_MAX;
      for (int da = -1; da <= 1 && ismax; ++da)
        for (int db = -1; db <= 1 && ismax; ++db)
          for (int dg = -1; dg <= 1; ++dg)
            if ((da | db | dg) && !(val >= Q[c0 + (da * CP_H + db) * CP_H + dg])) {
              ismax = false;
              break;
            }
      if (ismax) {
        const int item = q * P + pair;
        const int slot = atomicAdd(&counts[item], 1);
        const int id = ((a0 + la) * n + (b0 + lb)) * n + (g0 + lg);
        if (slot < cap) lists[(long)item * cap + slot] = make_int2(id, __float_as_int(val));
      }
    }
  }
}

// Centred half spectra of M volumes of edge N (kz-major [e][kz][x][y], DC at (N/2, N/2, kz = N/2)) cut down to the
// frequencies of edge N/2 (|f| < N/4 on x and y, -N/4 <= f <= 0 on kz): the Fourier crop of a 2x decimation.
__global__ void k_spectrum_crop(const float2 *__restrict__ in, int N, long M, float2 *__restrict__ out) {
  const int n = N / 2, h = n / 2 + 1, H = N / 2 + 1, q = N / 4;
  const long total = M * h * (long)n * n;
  for (long id = (long)blockIdx.x * blockDim.x + threadIdx.x; id < total; id += (long)gridDim.x * blockDim.x) {
    const int y = (int)(id % n), x = (int)((id / n) % n), kz = (int)((id / ((long)n * n)) % h);
    const long e = id / ((long)h * n * n);
    out[id] = in[((e * H + kz + q) * N + x + q) * N + y + q];
  }
}

template <class F>
inline int nblocks(long n, int threads, int maxb = 1 << 16) {
  long b = (n + threads - 1) / threads;
  return (int)std::max(1L, std::min<long>(b, maxb));
}

// small-d^l_{m1 m2}(beta) for l in [max(|m1|,|m2|), B): closed form at the lowest degree and the
// three-term recurrence in l (the L2-normalised version is what SOFT's genWigTrans_L2 tabulates,
// external/soft-1.0/makeWigner.c:531-607).
void small_d(int B, int m1, int m2, double beta, double *out) {
  double c = cos(beta / 2), s = sin(beta / 2), cb = cos(beta);
  int J = std::max(std::abs(m1), std::abs(m2));
  double acc = 0;
  for (int k = 0; k <= 2 * J; ++k) {
    if (J + m2 - k < 0 || J - k - m1 < 0 || k - m2 + m1 < 0) continue;
    double lg = 0.5 * (lgamma(J + m2 + 1.0) + lgamma(J - m2 + 1.0) + lgamma(J + m1 + 1.0) + lgamma(J - m1 + 1.0)) -
                (lgamma(J + m2 - k + 1.0) + lgamma(k + 1.0) + lgamma(J - k - m1 + 1.0) + lgamma(k - m2 + m1 + 1.0));
    acc += (((k - m2 + m1) % 2) ? -1.0 : 1.0) * exp(lg) * pow(c, 2 * J - 2 * k + m2 - m1) * pow(s, 2 * k - m2 + m1);
  }
  double prev = 0, cur = acc;
  out[J] = cur;
  for (int l = J; l < B - 1; ++l) {
    double a = (l + 1) * (2.0 * l + 1) / sqrt(((l + 1.0) * (l + 1) - m1 * m1) * ((l + 1.0) * (l + 1) - m2 * m2));
    double nx = (l == 0) ? a * cb * cur
                         : a * ((cb - (double)m1 * m2 / (l * (l + 1.0))) * cur -
                                (sqrt(((double)l * l - m1 * m1) * ((double)l * l - m2 * m2)) / (l * (2.0 * l + 1))) * prev);
    prev = cur;
    cur = nx;
    out[l + 1] = cur;
  }
}

struct EvalReq {
  int ref, part;
  Mat4 t;
};
struct EvalRes {
  float dist;
  Mat4 t;  // t * Translate(-shift)
};

}  // namespace

namespace {  // host helpers defined further down
template <class F>
void parallel_for(int n, F f);
void wedge_half_host(const VolumeGeom &g, int N, std::vector<float> &W);
}  // namespace

struct ettk_ctx {
  int device = 0;
  ettk_params p{};
  // launch shapes chosen by ettk_gpu_autotune or ettk_gpu_set_tuning; none of them changes a result
  ettk_tuning tune{64, 4096, 1, 128};
  // trilinear reslices in the CCF evaluations (set on the fast form's half-grid screening context only, with
  // fast_coarse_so3 = 2; never on the reference path)
  bool linear_reslice = false;
  cudaStream_t st = nullptr;
  int N = 0, H = 0, B = 0, n = 0;
  long n3 = 0, h3 = 0, nn = 0, nso3 = 0;
  std::string err;
  long long launches = 0;
  // constant tables
  DevBuf<float> mask, maskfft, filter, lw, plm, dtab, sinth;
  // m1 of the translational CCF (nbfFourierImageMetric::referenceMask): the spherical mask, or the external mask
  // set by ettk_gpu_set_reference_mask; [x][y][z], z fastest. `mask` stays the image filter's (spherical
  // projection, representations).
  DevBuf<float> refmask;
  bool refmask_external = false;
  void apply_reference_mask(const std::vector<float> &m1);
  DevBuf<int> doff;
  DevBuf<double> dtab64;  // FP64 Wigner-d table (wigner_precision 4 only)
  // Wigner-d synthesis of NJ correlation jobs into w_S (zeroed by the caller) in the configured precision
  template <int BB, int MODE>
  void synth_tc(long NJ) {
    static bool attr_set = false;  // per instantiation, once per process
    if (!attr_set) {
      CK(cudaFuncSetAttribute(k_so3_synth_tc<BB, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)WigTC<BB, MODE>::SMEM));
      attr_set = true;
    }
    k_so3_synth_tc<BB, MODE><<<dim3((2 * BB - 1) * (2 * BB - 1), (unsigned)((NJ + 63) / 64)), 128,
                               WigTC<BB, MODE>::SMEM, st>>>(w_coef.p, w_jobs.p, (int)NJ, dtab.p, doff.p, w_S.p,
                                                            status.p);
  }
  template <int BB>
  void synth(long NJ) {
    switch (p.wigner_precision) {
      case WIG_BF16: synth_tc<BB, WIG_BF16>(NJ); break;
      case WIG_SPLIT: synth_tc<BB, WIG_SPLIT>(NJ); break;
      case WIG_TF32: synth_tc<BB, WIG_TF32>(NJ); break;
      case WIG_FP64:
        k_so3_synth_f64<BB><<<dim3((2 * BB - 1) * (2 * BB - 1), (unsigned)std::min<long>(64, (NJ * 2 * BB + 255) / 256)),
                              256, 0, st>>>(w_coef.p, w_jobs.p, (int)NJ, dtab64.p, doff.p, w_S.p);
        break;
      default:
        k_so3_synth<BB><<<dim3((2 * BB - 1) * (2 * BB - 1), (unsigned)std::min<long>(tune.synth_job_blocks, (NJ + 7) / 8)), 256, 0,
                          st>>>(w_coef.p, w_jobs.p, (int)NJ, dtab.p, doff.p, w_S.p);
    }
    post_launch();
  }
  DevBuf<float4> dirs;
  DevBuf<float2> Fm1;
  double sum_filter = 0;
  Smooth3 smooth{};
  int bandL = 0, bandU = 0, rstart = 0, W = 0, lo = 0;
  float rr2 = 0;
  // references
  int R = 0;
  DevBuf<float> refvol, W1half, Pp1, W1sph;
  DevBuf<float2> FI1;
  std::vector<VolumeGeom> refg;
  std::vector<int> useW1;
  // particles
  int V = 0;
  DevBuf<float> partvol, W2sph, Pp2;
  const float *partptr = nullptr;
  std::vector<VolumeGeom> partg;
  std::vector<int> useW2, pp2_ready;
  // work buffers
  DevBuf<float> w_r, w_v, w_fw, w_tmp, w_C, w_sig, w_norm, w_norm2, sp_v, sp_M, sp_padc;
  DevBuf<float2> w_cA, w_cB, w_cC, w_p1, w_p2, w_coef, w_S, sp_F;
  DevBuf<double> w_acc, w_w, sp_acc;
  DevBuf<unsigned long long> w_peak, w_mm;
  DevBuf<ResliceItem> w_items;
  DevBuf<int> w_ridx;     // items resliced directly
  DevBuf<float> w_faces;  // per slot: faces one step past the reslice box (direct evaluations with a mirror)
  DevBuf<int2> w_mpairs;  // (mirror item, direct item) pairs of a chunk
  // tensor maps of the particle and reference volumes (empty: the reslice stages through the threads)
  DevBuf<CUtensorMap> tm_part, tm_ref;
  bool tm_part_ok = false, tm_ref_ok = false;
  DevBuf<int> status;  // set by kernels whose bounded waits ran out
  const void *part_map(long p) const { return tm_part_ok ? (const void *)(tm_part.p + (from_tomo ? 0 : p)) : nullptr; }
  // particles are fixed N^3 images (partptr + p n3), or sub-volumes of one tomogram (tomo, dims tomo_dims)
  DevBuf<float> tomo;
  int tomo_dims[3] = {0, 0, 0};
  bool from_tomo = false;
  const float *part_vol(long p) const { return from_tomo ? tomo.p : partptr + p * n3; }
  void part_dims(int d[3]) const {
    for (int i = 0; i < 3; ++i) d[i] = from_tomo ? tomo_dims[i] : N;
  }
  const void *ref_map(long r) const { return tm_ref_ok ? (const void *)(tm_ref.p + r) : nullptr; }
  void upload_maps(const float *base, int count, DevBuf<CUtensorMap> &dst, bool &ok, const int *dims3 = nullptr) {
    std::vector<CUtensorMap> h;
    ok = encode_volume_maps(base, count, N, h, dims3);
    if (ok) {
      dst.ensure(count);
      CK(cudaMemcpyAsync(dst.p, h.data(), count * sizeof(CUtensorMap), cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));  // h is pageable and goes out of scope
    }
  }
  void check_status() {
    int h = 0;
    CK(cudaMemcpyAsync(&h, status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (h) {
      CK(cudaMemsetAsync(status.p, 0, sizeof(int), st));
      throw CudaError(ETTK_ERR_TIMEOUT, "a bounded device wait (bulk tensor copy or tensor-core commit) ran out");
    }
  }
  DevBuf<WedgeVecs> w_wv;
  DevBuf<int> w_idx, w_idx2, w_cnt, w_pair_ref, w_pair_pp2, w_pair_part, w_i1;
  DevBuf<int2> w_lists;
  DevBuf<EvalOut> w_out;
  DevBuf<SigDesc> w_sd;
  DevBuf<SynthJob> w_jobs;
  DevBuf<ScaledJob> w_sjobs;
  DevBuf<PairPlan> w_plans;

  // ---- optional per-kernel-family timing with CUDA events on the library stream
  bool prof = false;
  struct ProfRec {
    const char *name;
    double bytes;
    cudaEvent_t a, b;
  };
  struct ProfAgg {
    long long n = 0;
    double ms = 0, bytes = 0;
  };
  std::vector<ProfRec> prof_pending;
  std::vector<cudaEvent_t> ev_pool;
  std::map<std::string, ProfAgg> prof_agg;
  cudaEvent_t ev_get() {
    if (ev_pool.empty()) {
      cudaEvent_t e;
      CK(cudaEventCreate(&e));
      return e;
    }
    cudaEvent_t e = ev_pool.back();
    ev_pool.pop_back();
    return e;
  }
  void prof_flush() {
    for (auto &r : prof_pending) {
      float ms = 0;
      CK(cudaEventElapsedTime(&ms, r.a, r.b));
      ProfAgg &g = prof_agg[r.name];
      g.n += 1;
      g.ms += ms;
      g.bytes += r.bytes;
      ev_pool.push_back(r.a);
      ev_pool.push_back(r.b);
    }
    prof_pending.clear();
  }
  struct Scope {
    ettk_ctx *c;
    const char *name;
    double bytes;
    cudaEvent_t a = nullptr;
    Scope(ettk_ctx *c_, const char *n_, double b_) : c(c_), name(n_), bytes(b_) {
      if (c->prof) {
        a = c->ev_get();
        CK(cudaEventRecord(a, c->st));
      }
    }
    ~Scope() {
      if (c->prof) {
        cudaEvent_t b = c->ev_get();
        cudaEventRecord(b, c->st);
        c->prof_pending.push_back({name, bytes, a, b});
      }
    }
  };

  // host-side phases (wall time), reported through the same profile table
  struct HostScope {
    ettk_ctx *c;
    const char *name;
    std::chrono::steady_clock::time_point t0;
    HostScope(ettk_ctx *c_, const char *n_) : c(c_), name(n_), t0(std::chrono::steady_clock::now()) {}
    ~HostScope() {
      if (!c->prof) return;
      double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      ProfAgg &g = c->prof_agg[name];
      g.n += 1;
      g.ms += ms;
    }
  };

  void sync() {
    HostScope hs(this, "host_wait");
    CK(cudaStreamSynchronize(st));
    if (prof) prof_flush();
  }
  // Blocking read of device results (the host waits for the stream here; timed as host_wait).
  void read_back(void *dst, const void *src, size_t bytes) {
    HostScope hs(this, "host_wait");
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (prof) prof_flush();
  }
  // Blocking copies ordered on the context stream. The stream is non-blocking, so a plain cudaMemcpy (legacy
  // stream) would not be ordered with its kernels; a pageable host-to-device copy may also return before its
  // DMA lands. Both helpers return with the copy complete, so the host buffer may go out of scope.
  void h2d(void *dst, const void *src, size_t bytes) {
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
  }
  void d2h(void *dst, const void *src, size_t bytes) {
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  void post_launch() {
    ++launches;
    CK(cudaGetLastError());
  }
  // Tricubic reslice of n_items items (device array `items_dev`, optionally through item_index) into
  // out[item][a][b][c], with the valid-value sums into acc (k_reslice_brick, one 8^3 brick per CTA)
  void reslice(const ResliceItem *items_dev, float *out, double *acc_, int acc_stride, const int *item_index,
               long n_items, bool clamp_all = false, bool linear = false) {
    if (n_items <= 0) return;
    const dim3 grid((N / RB) * (N / RB) * (N / RB), (unsigned)n_items);
    if (clamp_all)
      k_reslice_brick<false, true><<<grid, 256, RS_SMEM, st>>>(items_dev, N, out, acc_, acc_stride, status.p, item_index);
    else if (linear)
      k_reslice_brick<false, false, true><<<grid, 256, RS_SMEM, st>>>(items_dev, N, out, acc_, acc_stride, status.p,
                                                                      item_index);
    else
      k_reslice_brick<false><<<grid, 256, RS_SMEM, st>>>(items_dev, N, out, acc_, acc_stride, status.p, item_index);
    post_launch();
  }

  // wedge * filter of E evaluations (missing-wedge compensation), rolling-window kernel
  template <int NN>
  void wedge_t(long E, double *acc, int acc_stride) {
    constexpr int SLAB = wedge_slab<NN>();
    constexpr size_t smem = wedge_smem<NN>();
    if (smem > 48 * 1024) CK(cudaFuncSetAttribute(k_wedge_roll<NN, SLAB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_wedge_roll<NN, SLAB><<<dim3(NN / SLAB, (unsigned)E), 256, smem, st>>>(w_wv.p, smooth, W1half.p, w_idx.p, filter.p,
                                                                            w_fw.p, acc, acc_stride, 6);
    post_launch();
  }

  // one zero-padded 2N-point pruned inverse stage of the translational search window
  template <int NN, bool CONTIG>
  void pruned_fft_t(const float2 *in, float2 *out, const PrunedLines &pl, int off) {
    constexpr int L = reg_lines<NN>();
    k_pruned_fft<NN, L, CONTIG><<<(unsigned)((pl.n_lines + L - 1) / L), L * MaxAB<NN>::v, 0, st>>>(in, out, pl, N, W,
                                                                                                  lo, off);
    post_launch();
  }
  template <bool CONTIG>
  void pruned_fft(const float2 *in, float2 *out, const PrunedLines &pl, int off) {
    switch (2 * N) {
      case 32: pruned_fft_t<32, CONTIG>(in, out, pl, off); break;
      case 64: pruned_fft_t<64, CONTIG>(in, out, pl, off); break;
      case 128: pruned_fft_t<128, CONTIG>(in, out, pl, off); break;
      case 256: pruned_fft_t<256, CONTIG>(in, out, pl, off); break;
      default: throw CudaError(ETTK_ERR_ARG, "unsupported volume size");
    }
  }

  // x and y stages of the window in one pass per (kz plane, item) (k_pruned_xy), when the plane's W window rows fit
  // in shared memory with three CTAs per SM; otherwise the two stages above through the [item][X][kz][ky]
  // intermediate
  template <int NN>
  static size_t pruned_xy_smem(int W) {
    return (size_t)W * (NN / 2 + 8) * sizeof(float2);
  }
  template <int NN>
  static bool pruned_xy_fits(int W) {
    return pruned_xy_smem<NN>(W) + (NN + pruned_xy_ex<NN, reg_lines<NN>()>()) * sizeof(float2) <= 75 * 1024;
  }
  bool pruned_xy_used() const {
    switch (2 * N) {
      case 32: return pruned_xy_fits<32>(W);
      case 64: return pruned_xy_fits<64>(W);
      case 128: return pruned_xy_fits<128>(W);
      case 256: return pruned_xy_fits<256>(W);
      default: return false;
    }
  }
  template <int NN>
  void pruned_xy_t(const float2 *in, float2 *out, long E, int off) {
    constexpr int L = reg_lines<NN>();
    const size_t dyn = pruned_xy_smem<NN>(W);
    if (dyn > 48 * 1024) CK(cudaFuncSetAttribute(k_pruned_xy<NN, L>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    k_pruned_xy<NN, L><<<dim3(NN / 4 + 1, (unsigned)E), L * MaxAB<NN>::v, dyn, st>>>(in, out, W, lo, off);
    post_launch();
  }
  void pruned_xy(const float2 *in, float2 *out, long E, int off) {
    switch (2 * N) {
      case 32: pruned_xy_t<32>(in, out, E, off); break;
      case 64: pruned_xy_t<64>(in, out, E, off); break;
      case 128: pruned_xy_t<128>(in, out, E, off); break;
      case 256: pruned_xy_t<256>(in, out, E, off); break;
      default: throw CudaError(ETTK_ERR_ARG, "unsupported volume size");
    }
  }

  // ---------------------------------------------------------------- FFT drivers
  // CTA shape of the register FFT kernels: 256 threads = LINES x max(A, B)
  template <int NN>
  static constexpr int reg_lines() { return 256 / MaxAB<NN>::v; }
  template <int NN>
  void fft_strided_t(float2 *d, LineMap m, int sign, const float *scale, long scale_div) {
    constexpr int L = reg_lines<NN>();
    int blocks = (int)((m.n_lines + L - 1) / L);
    Scope sc(this, "fft_strided", 16.0 * m.n_lines * NN);
    if (m.elem_stride == 1)
      k_fft_reg<NN, L, true><<<blocks, 256, 0, st>>>(d, m, sign, scale, scale_div);
    else
      k_fft_reg<NN, L, false><<<blocks, 256, 0, st>>>(d, m, sign, scale, scale_div);
    post_launch();
  }
  void fft_strided(int len, float2 *d, LineMap m, int sign, const float *scale = nullptr, long scale_div = 1) {
    switch (len) {
      case 16: fft_strided_t<16>(d, m, sign, scale, scale_div); break;
      case 32: fft_strided_t<32>(d, m, sign, scale, scale_div); break;
      case 64: fft_strided_t<64>(d, m, sign, scale, scale_div); break;
      case 128: fft_strided_t<128>(d, m, sign, scale, scale_div); break;
      case 256: fft_strided_t<256>(d, m, sign, scale, scale_div); break;
      default: throw CudaError(ETTK_ERR_ARG, "unsupported FFT length");
    }
  }
  template <int NN, class Pre>
  void r2c_z_t(Pre pre, float2 *out, long lines, const char *family = "fft_r2c_z") {
    constexpr int L = reg_lines<NN>();
    long tiles = (lines + 2 * L - 1) / (2 * L);
    Scope sc(this, family, 4.0 * lines * NN + 8.0 * lines * (NN / 2 + 1));
    bool streamed = false;
    if constexpr (has_stream<Pre>::value) {
      const unsigned long long sa = (unsigned long long)pre.stream_src(), aa = (unsigned long long)pre.stream_aux();
      if ((sa & 15) == 0 && (aa & 15) == 0) {
        if (aa) {
          constexpr size_t smem = r2c_stream_smem<NN, true>();
          const int grid = (int)std::min<long>(tiles, tune.zpass_oversub * resident_grid(k_r2c_stream<NN, L, Pre, true>, smem));
          k_r2c_stream<NN, L, Pre, true><<<grid, 256, smem, st>>>(pre, out, lines);
        } else {
          constexpr size_t smem = r2c_stream_smem<NN, false>();
          const int grid = (int)std::min<long>(tiles, tune.zpass_oversub * resident_grid(k_r2c_stream<NN, L, Pre, false>, smem));
          k_r2c_stream<NN, L, Pre, false><<<grid, 256, smem, st>>>(pre, out, lines);
        }
        streamed = true;
      }
    }
    if constexpr (has_line_base<Pre>::value)
      if (pre.real_only) {
        if ((pre.N % (2 * L)) != 0) throw CudaError(ETTK_ERR_ARG, "real-line tiles must divide the box");
        tiles = pre.real_tiles(lines, 2 * L);
      }
    if (!streamed) k_r2c_reg<NN, L, Pre><<<(unsigned)tiles, 256, 0, st>>>(pre, out, lines);
    post_launch();
  }
  // CTAs of a persistent kernel: resident CTAs per SM (with `smem` dynamic shared memory) x SMs, computed
  // once per kernel and device (the dynamic size is opted in first: static + dynamic may exceed 48 KB)
  template <class K>
  long resident_grid(K *kernel, size_t smem) {
    static std::map<std::pair<const void *, int>, long> cache;
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    const std::pair<const void *, int> key((const void *)kernel, device);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0, sms = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, smem));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const long g = (long)std::max(1, per_sm) * std::max(1, sms);
    cache[key] = g;
    return g;
  }
  template <class Pre>
  void r2c_z(int len, Pre pre, float2 *out, long lines, const char *family = "fft_r2c_z") {
    switch (len) {
      case 16: r2c_z_t<16>(pre, out, lines, family); break;
      case 32: r2c_z_t<32>(pre, out, lines, family); break;
      case 64: r2c_z_t<64>(pre, out, lines, family); break;
      case 128: r2c_z_t<128>(pre, out, lines, family); break;
      case 256: r2c_z_t<256>(pre, out, lines, family); break;
      default: throw CudaError(ETTK_ERR_ARG, "unsupported FFT length");
    }
  }
  template <int NN, class Post>
  void c2r_z_t(const float2 *in, Post post, long lines) {
    constexpr int L = reg_lines<NN>();
    long tiles = (lines + 2 * L - 1) / (2 * L);
    Scope sc(this, "fft_c2r_z", 4.0 * lines * NN + 8.0 * lines * (NN / 2 + 1));
    if (lines % (2 * L) == 0 && (((unsigned long long)in) & 15) == 0) {
      constexpr size_t smem = c2r_stream_smem<NN>();
      const int grid = (int)std::min<long>(tiles, tune.zpass_oversub * resident_grid(k_c2r_stream<NN, L, Post>, smem));
      k_c2r_stream<NN, L, Post><<<grid, 256, smem, st>>>(in, post, lines);
    } else {
      k_c2r_reg<NN, L, Post><<<(unsigned)tiles, 256, 0, st>>>(in, post, lines);
    }
    post_launch();
  }
  template <class Post>
  void c2r_z(int len, const float2 *in, Post post, long lines) {
    switch (len) {
      case 16: c2r_z_t<16>(in, post, lines); break;
      case 32: c2r_z_t<32>(in, post, lines); break;
      case 64: c2r_z_t<64>(in, post, lines); break;
      case 128: c2r_z_t<128>(in, post, lines); break;
      default: throw CudaError(ETTK_ERR_ARG, "unsupported FFT length");
    }
  }
  // C2R, elementwise Mid, R2C of the same z lines in one persistent pass, in place on kz-major spectra
  template <int NN, class Mid>
  void c2r_r2c_z_t(float2 *data, Mid mid, long lines) {
    constexpr int L = reg_lines<NN>();
    const long tiles = (lines + 2 * L - 1) / (2 * L);
    Scope sc(this, "fft_c2r_r2c_z", 16.0 * lines * (NN / 2 + 1));
    if (lines % (2 * L) != 0 || (((unsigned long long)data) & 15) || (((unsigned long long)mid.aux) & 15))
      throw CudaError(ETTK_ERR_ARG, "fused z pass: lines must fill whole tiles of 16-byte aligned data");
    if (mid.aux) {
      constexpr size_t smem = c2r_r2c_stream_smem<NN, true>();
      const int grid = (int)std::min<long>(tiles, tune.zpass_oversub * resident_grid(k_c2r_r2c_stream<NN, L, Mid, true>, smem));
      k_c2r_r2c_stream<NN, L, Mid, true><<<grid, 256, smem, st>>>(data, mid, lines);
    } else {
      constexpr size_t smem = c2r_r2c_stream_smem<NN, false>();
      const int grid = (int)std::min<long>(tiles, tune.zpass_oversub * resident_grid(k_c2r_r2c_stream<NN, L, Mid, false>, smem));
      k_c2r_r2c_stream<NN, L, Mid, false><<<grid, 256, smem, st>>>(data, mid, lines);
    }
    post_launch();
  }
  template <class Mid>
  void c2r_r2c_z(int len, float2 *data, Mid mid, long lines) {
    switch (len) {
      case 16: c2r_r2c_z_t<16>(data, mid, lines); break;
      case 32: c2r_r2c_z_t<32>(data, mid, lines); break;
      case 64: c2r_r2c_z_t<64>(data, mid, lines); break;
      case 128: c2r_r2c_z_t<128>(data, mid, lines); break;
      default: throw CudaError(ETTK_ERR_ARG, "unsupported FFT length");
    }
  }
  // (x, y) passes of a 3-D transform of `items` kz-major spectra [len/2+1][len][len]: one CTA per kz plane
  // (k_fft2d) up to len = 128, two strided register passes beyond.
  template <int NN, class Op>
  void fft2d_t(Op op, long items, const char *family = "fft_xy", double bytes_per_elem = 16.0, int planes = NN / 2 + 1) {
    constexpr size_t smem = fft2d_smem<NN>();
    const long H2 = planes;  // kz planes transformed (blockIdx.x), from the op's first plane
    Scope sc(this, family, bytes_per_elem * items * H2 * NN * NN);
    static bool attr_set = false;  // per instantiation, once per process
    if (!attr_set) {
      CK(cudaFuncSetAttribute(k_fft2d<NN, Op>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      CK(cudaFuncSetAttribute(k_fft2d<NN, Op>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
      attr_set = true;
    }
    k_fft2d<NN, Op><<<dim3((unsigned)H2, (unsigned)items), 256, smem, st>>>(op);
    post_launch();
  }
  void xy_kxy(int len, float2 *d, long items, int sign) {
    switch (len) {
      case 16: fft2d_t<16>(OpPlain<16>{d, sign}, items); break;
      case 32: fft2d_t<32>(OpPlain<32>{d, sign}, items); break;
      case 64: fft2d_t<64>(OpPlain<64>{d, sign}, items); break;
      case 128: fft2d_t<128>(OpPlain<128>{d, sign}, items); break;
      case 256: {
        const long h = len / 2 + 1;
        fft_strided(len, d, LineMap{items * h * len, 1, (long)len, 0, 1}, sign);                          // y lines
        fft_strided(len, d, LineMap{items * h * len, len, (long)len * len, 1, (long)len}, sign);           // x lines
        break;
      }
      default: throw CudaError(ETTK_ERR_ARG, "unsupported FFT length");
    }
  }

  // ---------------------------------------------------------------- setup
  void init_tables();
  // (x, y) passes of the padded spherical-projection spectra sp_F storing |F| into sp_M: the planes kz < N2/2
  // by k_fft2d_padded (half-row shared memory), the last plane by k_fft2d
  template <int N2>
  void padded_magnitude_t(long P) {
    constexpr size_t smem = fft2d_padded_smem<N2>();
    {
      Scope sc(this, "sphere_fft", 16.0 * P * (N2 / 2) * N2 * N2);
      static bool attr_set = false;  // per instantiation, once per process
      if (!attr_set) {
        CK(cudaFuncSetAttribute(k_fft2d_padded<N2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        CK(cudaFuncSetAttribute(k_fft2d_padded<N2>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
        attr_set = true;
      }
      k_fft2d_padded<N2><<<dim3(N2 / 2, (unsigned)P), 256, smem, st>>>(sp_F.p, sp_M.p, p.mutual_correlation ? 1 : 0);
      post_launch();
    }
    OpPaddedMagnitude<N2> last{sp_F.p, sp_M.p};
    last.kz0 = N2 / 2;
    last.mutual = p.mutual_correlation ? 1 : 0;
    if (N2 == 128) last.padc = sp_padc.p;  // the z pass skipped the padding lines (PrePadded::real_only)
    fft2d_t<N2>(last, P, "sphere_fft", 16.0, 1);
  }
  // |F| spherical projections of the items into Pp_out[out_index[i] * nn] (device; out_index null: [i * nn])
  void spherical_projection(const std::vector<ResliceItem> &items, float *Pp_out, const int *out_index = nullptr);
  void eval_chunk(const std::vector<EvalReq> &req, std::vector<EvalRes> &res);
  // executeFourierNewHalf for any number of requests, in device chunks of at most 4096 evaluations at 64^3
  // (scaled by 64^3 / N^3, 256 to 8192; about 6.4 MB of scratch per 64^3 evaluation): fewer chunks mean
  // fewer host round trips and larger grids
  void eval_batch(const std::vector<EvalReq> &req, std::vector<EvalRes> &res) {
    res.resize(req.size());
    const size_t chunk = (size_t)std::min(16384L, std::max(256L, (long)tune.eval_chunk * 64 * 64 * 64 / n3));
    for (size_t c0 = 0; c0 < req.size(); c0 += chunk) {
      size_t c1 = std::min(req.size(), c0 + chunk);
      std::vector<EvalReq> sub(req.begin() + c0, req.begin() + c1);
      std::vector<EvalRes> out;
      eval_chunk(sub, out);
      std::copy(out.begin(), out.end(), res.begin() + c0);
    }
  }
  void align(int npairs, const int *pairs, float *D, int cols, int ncand);
  // translational search window of the CCF on the upsampled grid for a translation restriction
  // (nbfFourierImageMetric.h:1216-1232): first index lo, width W, squared radius rr2
  void set_window(float restrict_translation) {
    const int N2 = 2 * N;
    const float center = (float)(N2 / 2.0);
    float restriction = center;
    if (restrict_translation < FLT_MAX) restriction = (float)std::max((double)restrict_translation * 2.0f, 1.0);
    lo = (int)std::max(0.0, (double)center - floor(restriction));
    const int hi = (int)std::min((double)center + floor(restriction), (double)(N2 - 1));
    W = hi - lo + 1;
    rr2 = restriction * restriction;
  }
  // getDistances with typeOfMetric 2: one CCF per pair at the particle's own alignment
  void score(int npairs, const int *pairs, float *D, int cols, int ncand, float restrict_translation);
  // ---------------------------------------------------------------- fast form: coarse SO(3) hit + local refinement
  DevBuf<LRItem> lr_items;
  DevBuf<LRState> lr_state;
  bool lr_skip_done = false;  // inside lr_run: converged pairs are not evaluated again
  DevBuf<float> lr_zm, lr_maps, lr_ip;
  DevBuf<int> lr_src;
  std::vector<int> lr_slot;  // particle -> slot of its band-passed copy in lr_ip (-1: none)
  // band-passed copies of the fixed-image particles `parts` (filter of the metric, the particle's own frame) in
  // lr_ip at slot lr_slot[particle]; with_half also their Fourier crops to edge N/2 in dec_vol, same slots
  void lr_filter_particles(const std::vector<int> &parts, bool with_half = false);
  DevBuf<double> lr_acc;
  double lr_C0 = 0, lr_C1 = 0;  // sum m, sum m^2 of the spherical mask
  DevBuf<int> lr_in;             // indices of the voxels with m != 0 (ascending)
  long lr_nin = 0;
  double lr_radius() const { return 0.6 * (p.mask_radius > 0 ? p.mask_radius : 0.5 * N); }
  // zm of every request (reference filtered with the wedges at the request's pose, times the mask), the
  // refinement states at the requests' poses and their index maps
  void lr_setup(const std::vector<EvalReq> &req);
  // iterations + 1 evaluations of every pair's objective, each followed by the per-pair update
  void lr_run(long P, int iterations);
  template <int NN>
  void lr_eval_t(long E) {
    Scope sc(this, "local_refine", 4.0 * E * (double)lr_nin * 3);
    const unsigned chunks = (unsigned)std::max<long>(1, (lr_nin + LR_CHUNK - 1) / LR_CHUNK);
    k_lr_eval<NN><<<dim3(chunks, (unsigned)E), 256, 0, st>>>(lr_items.p, lr_maps.p, lr_zm.p, refmask.p, lr_in.p,
                                                            (int)lr_nin, lr_skip_done ? lr_state.p : nullptr,
                                                            lr_acc.p);
    post_launch();
  }
  void lr_eval(long E) { with_n(N, [&](auto nn) { lr_eval_t<decltype(nn)::value>(E); }); }
  void align_refined(int npairs, const int *pairs, float *D, int cols, int ncand, int iterations, int peaks);
  // Candidate screening of the fast form on 2x decimated volumes: a child context of edge N/2 (the metric's
  // parameters rescaled to the half grid) holding the Fourier-cropped references and, per batch, particles.
  ettk_ctx *half = nullptr;
  bool half_refs_ok = false;
  DevBuf<float> dec_vol;
  DevBuf<int> dec_src;
  // Fourier crop of M fixed-image volumes vols + src[e] N^3 (device) to edge N/2, into out (M (N/2)^3, x fastest)
  void decimate(const float *vols, const std::vector<int> &src, float *out);
  void half_setup();  // creates the child context and gives it the decimated references (once per reference set)
  // hands the batch's decimated particles (lr_filter_particles with with_half, queued on st) to the child: host
  // set-up only, the child's stream waits for dec_ev before its first kernel
  cudaEvent_t dec_ev = nullptr;
  void half_particles(const std::vector<int> &pp);
  void merge_child_profile();
  // NaN / infinity check of an upload on the device, queued behind its copy; finite_or_throw after the next sync
  // (a failed upload leaves the context without particles)
  DevBuf<int> nf_flag;
  void check_finite(const float *v, long n) {
    nf_flag.ensure(1);
    CK(cudaMemsetAsync(nf_flag.p, 0, sizeof(int), st));
    k_nonfinite<<<nblocks<int>((n + 3) / 4, 256, 4096), 256, 0, st>>>(v, n, nf_flag.p);
    post_launch();
  }
  void finite_or_throw(const char *what) {
    int bad = 0;
    d2h(&bad, nf_flag.p, sizeof(int));
    if (bad) {
      V = 0;
      throw CudaError(ETTK_ERR_NAN, what);
    }
  }
  // best CCF candidate per pair scored on the decimated volumes: full-grid transform (translation doubled)
  void half_screen(const std::vector<int> &pr, const std::vector<int> &pp, const std::vector<EvalReq> &cand,
                   const std::vector<int> &owner, std::vector<EvalReq> &finals);
  void refined_objective(int npairs, const int *pairs, const double *poses, const double *theta, double *rho,
                         double *grad);
  void so3_queues(int P, const std::vector<int> &pr, const std::vector<int> &pp, std::vector<PairPlan> &plans,
                  std::vector<PQ> &q1, std::vector<PQ> &q2);
  // nbfCorrelationImageMetric::getWedgeOverlap(T) of each request: sum(w1 w2 filter) / sum(filter) over the
  // half spectrum with the wedges of the effective sides only, 1 when neither side's wedge is effective
  DevBuf<double> w_ovl;
  std::vector<float> wedge_overlaps(const std::vector<EvalReq> &req);
  void soft_diag(const float *F1, const float *F2, int scaled, float *C);

  // ---------------------------------------------------------------- continuous pose refinement
  DevBuf<float> rf_fw, rf_y1, rf_a;  // per pair: wedge * filter (kz-major half), filtered reference; adjoint field
  DevBuf<int> rf_pair;                // evaluation -> pair
  DevBuf<double> rf_acc;              // [E][4] correlation sums, then [E][16] gradient sums
  std::vector<int> rf_part;           // pair -> particle
  void refine_setup(const std::vector<EvalReq> &req);
  void refine_eval(const std::vector<std::array<double, 12>> &maps, const std::vector<int> &pair, bool grad,
                   std::vector<double> &rho, std::vector<double> &g6);
  void refine(const std::vector<EvalReq> &req, int iterations, std::vector<Mat4> &out, std::vector<double> &rho);
  void average(int M, const int *parts, const float *weights, const double *mats, float *avg);
  void average_accumulate(int M, const int *parts, const float *weights, const double *mats);
  void average_finish(float *avg);
  void average_finish_device(bool xfast);
  void variance(int M, const int *parts, const float *weights, const double *mats, const float *avg, float *var);
  void symmetrize(const float *vol, int fold, float *out);
  void mean_images(const float *vol, int n, const Mat4 *ts, float *out);
  void symmetrize_rotational(const float *vol, float *out);
  void average_spherical_wedge(int M, const int *parts, const float *weights, const double *mats, float *count,
                               float *wedge);
  // kept-coefficient offsets of the representation band (kz-major) in the reference's order, cached
  std::vector<int> repr_idx;
  DevBuf<int> repr_idx_dev;
  const std::vector<int> &representation_band();
  void representations(int M, const int *parts, int fold, float *R);
  // kept voxels ([x][y][z] offsets) of the real-space representation for a bin factor, cached
  std::vector<int> real_idx;
  int real_bin = 0;
  DevBuf<int> real_idx_dev;
  DevBuf<float> w_real;
  const std::vector<int> &representation_real_band(int bin);
  void real_filtered(const float *src, int E, float *dst);
  void representations_real(int M, const int *parts, int fold, int bin, float *R);
  // members resliced as the average resamples them (own matrix reset, Euler(normal) * alignment), exact
  // coordinates, into w_v [E][x][y][z] with their valid-value sums in w_acc [E][2]
  void reslice_members(const int *idx, int E, const int *parts, const double *mats);
};

// Class average (getImageMPI + getImage): members resliced under Euler(normal) * alignment with their
// own matrix reset to identity (inc/em/nbfWedgedAverageImage3D.h:313-319), R2C, |F|-weighted FP64
// accumulation in member order, normalised inverse, RMS scaling.
void ettk_ctx::average(int M, const int *parts, const float *weights, const double *mats, float *avg) {
  average_accumulate(M, parts, weights, mats);
  average_finish(avg);
}

// Members resliced (exact coordinates, own matrix reset), transformed and accumulated in FP64 into w_w = [acc | re |
// im | sumsq] (kz-major, h3 each), the getImageMPI accumulators (inc/em/nbfWedgedAverageImage3D.h:260-356).
void ettk_ctx::average_accumulate(int M, const int *parts, const float *weights, const double *mats) {
  std::vector<int> idx;
  for (int i = 0; i < M; ++i) {
    if (parts[i] < 0 || parts[i] >= V) throw CudaError(ETTK_ERR_ARG, "member index out of range");
    if (fabs(weights[i]) > 0) idx.push_back(i);
  }
  DevBuf<double> &ac = w_w;  // reused: acc, re, im, sumsq
  ac.ensure(3 * h3 + 1);
  CK(cudaMemsetAsync(ac.p, 0, (3 * h3 + 1) * sizeof(double), st));
  const int chunk = 256;
  for (size_t c0 = 0; c0 < idx.size(); c0 += chunk) {
    int E = (int)std::min<size_t>(chunk, idx.size() - c0);
    std::vector<ResliceItem> items(E);
    std::vector<float> w(E);
    for (int e = 0; e < E; ++e) {
      int i = idx[c0 + e];
      VolumeGeom g = partg[parts[i]];
      for (int k = 0; k < 16; ++k) g.matrix[k] = (k % 5 == 0) ? 1.0 : 0.0;
      Mat4 t;
      memcpy(t.e, mats + 16 * (long)i, sizeof(t.e));
      double m12[12];
      reslice_index(g, N, &t, m12);
      items[e].vol = part_vol(parts[i]);
      items[e].tmap = part_map(parts[i]);
      part_dims(items[e].dims);
      set_map(items[e], m12);
      w[e] = weights[i];
    }
    w_items.ensure(E);
    w_v.ensure((long)E * n3);
    w_cA.ensure((long)E * h3);
    w_acc.ensure(2L * E);
    w_norm.ensure(E);
    CK(cudaMemcpyAsync(w_items.p, items.data(), E * sizeof(ResliceItem), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(w_norm.p, w.data(), E * sizeof(float), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(w_acc.p, 0, 2L * E * sizeof(double), st));
    {
      Scope sc(this, "reslice", 8.0 * E * n3);
      k_reslice_brick<true><<<dim3((N / RB) * (N / RB) * (N / RB), E), 256, RS_SMEM, st>>>(w_items.p, N, w_v.p, w_acc.p, 2, status.p, nullptr);
      post_launch();
    }
    PreParticle pre{w_v.p, nullptr, w_acc.p, 2, N};
    r2c_z(N, pre, w_cA.p, (long)E * N * N);
    xy_kxy(N, w_cA.p, E, -1);
    {
      Scope sc(this, "avg_accum", 8.0 * E * h3 + 48.0 * h3);
      k_avg_accum<<<nblocks<int>(h3, 256, 4096), 256, 0, st>>>(w_cA.p, w_norm.p, E, h3, ac.p, ac.p + h3, ac.p + 2 * h3);
      post_launch();
    }
  }
}

// getImage's reciprocal-space average from the accumulators in w_w (inc/em/nbfWedgedAverageImage3D.h:216-258):
// (re, im) / acc where acc > 0, DC zero, C2R, centring shift, RMS 1; avg N^3 floats on the host.
void ettk_ctx::average_finish(float *avg) {
  average_finish_device(true);
  CK(cudaMemcpyAsync(avg, w_tmp.p, n3 * sizeof(float), cudaMemcpyDeviceToHost, st));
  sync();
  check_status();
}

// The same average left in w_tmp (N^3 floats, x fastest when xfast, else [x][y][z]).
void ettk_ctx::average_finish_device(bool xfast) {
  DevBuf<double> &ac = w_w;
  CK(cudaMemsetAsync(ac.p + 3 * h3, 0, sizeof(double), st));
  w_cB.ensure(h3);
  w_r.ensure(n3);
  k_avg_spectrum<<<nblocks<int>(h3, 256, 4096), 256, 0, st>>>(ac.p, ac.p + h3, ac.p + 2 * h3, N, w_cB.p);
  post_launch();
  xy_kxy(N, w_cB.p, 1, +1);
  c2r_z(N, w_cB.p, PostStore{w_r.p, N}, (long)N * N);
  k_avg_shift_sumsq<<<nblocks<int>(n3, 256, 1024), 256, 0, st>>>(w_r.p, N, ac.p + 3 * h3);
  post_launch();
  w_tmp.ensure(n3);
  k_avg_finish<<<nblocks<int>(n3, 256, 4096), 256, 0, st>>>(w_r.p, N, ac.p + 3 * h3, w_tmp.p, xfast ? 1 : 0);
  post_launch();
}

void ettk_ctx::reslice_members(const int *idx, int E, const int *parts, const double *mats) {
  std::vector<ResliceItem> items(E);
  for (int e = 0; e < E; ++e) {
    const int i = idx[e];
    VolumeGeom g = partg[parts[i]];
    for (int k = 0; k < 16; ++k) g.matrix[k] = (k % 5 == 0) ? 1.0 : 0.0;
    Mat4 t;
    memcpy(t.e, mats + 16 * (long)i, sizeof(t.e));
    double m12[12];
    reslice_index(g, N, &t, m12);
    items[e].vol = part_vol(parts[i]);
    items[e].tmap = part_map(parts[i]);
    part_dims(items[e].dims);
    set_map(items[e], m12);
  }
  w_items.ensure(E);
  w_v.ensure((long)E * n3);
  w_acc.ensure(2L * E);
  CK(cudaMemcpyAsync(w_items.p, items.data(), E * sizeof(ResliceItem), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(w_acc.p, 0, 2L * E * sizeof(double), st));
  Scope sc(this, "reslice", 8.0 * E * n3);
  k_reslice_brick<true><<<dim3((N / RB) * (N / RB) * (N / RB), E), 256, RS_SMEM, st>>>(w_items.p, N, w_v.p, w_acc.p, 2,
                                                                                      status.p, nullptr);
  post_launch();
}

// Variance of the class members about an average (getImageVarianceMPI with setAverageImage): members in
// chunks, reslices as the average makes them, |w| (T - avg)^2 / sum|w| accumulated per voxel in FP64.
void ettk_ctx::variance(int M, const int *parts, const float *weights, const double *mats, const float *avg,
                        float *var) {
  std::vector<int> idx;
  double sw = 0;
  for (int i = 0; i < M; ++i) {
    if (parts[i] < 0 || parts[i] >= V) throw CudaError(ETTK_ERR_ARG, "member index out of range");
    sw += fabs((double)weights[i]);
    if (fabs(weights[i]) > 0) idx.push_back(i);
  }
  DevBuf<double> &vacc = w_w;  // reused accumulator
  vacc.ensure(n3);
  CK(cudaMemsetAsync(vacc.p, 0, n3 * sizeof(double), st));
  w_tmp.ensure(n3);
  CK(cudaMemcpyAsync(w_tmp.p, avg, n3 * sizeof(float), cudaMemcpyHostToDevice, st));
  const int chunk = 256;
  for (size_t c0 = 0; c0 < idx.size(); c0 += chunk) {
    const int E = (int)std::min<size_t>(chunk, idx.size() - c0);
    reslice_members(idx.data() + c0, E, parts, mats);
    std::vector<float> w(E);
    for (int e = 0; e < E; ++e) w[e] = weights[idx[c0 + e]];
    w_norm.ensure(E);
    CK(cudaMemcpyAsync(w_norm.p, w.data(), E * sizeof(float), cudaMemcpyHostToDevice, st));
    k_var_accum<<<nblocks<int>(n3, 256, 4096), 256, 0, st>>>(w_v.p, w_acc.p, w_norm.p, E, sw, w_tmp.p, N, vacc.p);
    post_launch();
  }
  w_r.ensure(n3);
  k_var_finish<<<nblocks<int>(n3, 256, 4096), 256, 0, st>>>(vacc.p, N, w_r.p);
  post_launch();
  CK(cudaMemcpyAsync(var, w_r.p, n3 * sizeof(float), cudaMemcpyDeviceToHost, st));
  sync();
  check_status();
}

// n-fold symmetrisation about z of a volume taken as a fixed image (position N/2, identity matrix).
void ettk_ctx::symmetrize(const float *vol, int fold, float *out) {
  if (fold <= 1) {
    memcpy(out, vol, n3 * sizeof(float));
    return;
  }
  std::vector<Mat4> ts(fold);
  for (int i = 0; i < fold; ++i) {
    ts[i] = Mat4::eye();
    rotate(ts[i], i * 360.0 / fold, 0, 0, 1);
  }
  mean_images(vol, fold, ts.data(), out);
}

// The mean over n transforms of getImage of vol as a fixed image (nbfWedgedSubImage3D::getImage with
// setFixedImage: position N/2, no normal, identity matrix, full wedge): each a tricubic reslice with the mean of its
// valid voxels removed and the invalid ones 0, summed in order in FP64 and divided by n. vol and out are x fastest.
void ettk_ctx::mean_images(const float *vol, int n, const Mat4 *ts, float *out) {
  w_tmp.ensure(n3);
  CK(cudaMemcpyAsync(w_tmp.p, vol, n3 * sizeof(float), cudaMemcpyHostToDevice, st));
  VolumeGeom g{};  // fixed image: position N/2, no normal, identity matrix, no cut offset, full wedge
  g.lwedge = -90.f;
  g.uwedge = 90.f;
  for (int k = 0; k < 3; ++k) g.position[k] = (float)(N / 2.0);
  for (int k = 0; k < 16; ++k) g.matrix[k] = (k % 5 == 0) ? 1.0 : 0.0;
  std::vector<ResliceItem> items(n);
  for (int i = 0; i < n; ++i) {
    double m12[12];
    reslice_index(g, N, &ts[i], m12);
    items[i].vol = w_tmp.p;
    items[i].tmap = nullptr;
    items[i].dims[0] = items[i].dims[1] = items[i].dims[2] = N;
    set_map(items[i], m12);
  }
  w_items.ensure(n);
  w_v.ensure((long)n * n3);
  w_acc.ensure(2L * n);
  CK(cudaMemcpyAsync(w_items.p, items.data(), n * sizeof(ResliceItem), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(w_acc.p, 0, 2L * n * sizeof(double), st));
  {
    Scope sc(this, "reslice", 8.0 * n * n3);
    k_reslice_brick<true><<<dim3((N / RB) * (N / RB) * (N / RB), n), 256, RS_SMEM, st>>>(w_items.p, N, w_v.p, w_acc.p,
                                                                                        2, status.p, nullptr);
    post_launch();
  }
  w_r.ensure(n3);
  k_sym_finish<<<nblocks<int>(n3, 256, 4096), 256, 0, st>>>(w_v.p, w_acc.p, n, N, w_r.p);
  post_launch();
  CK(cudaMemcpyAsync(out, w_r.p, n3 * sizeof(float), cudaMemcpyDeviceToHost, st));
  sync();
  check_status();
}

// Rotational symmetrisation of the classification loop (src/MPI_Classification.cpp:1005-1024): the
// (radius, z) profile summed over 180 angles on the cylinder about z, then interpolated back at every voxel.
void ettk_ctx::symmetrize_rotational(const float *vol, float *out) {
  CylGeom g;
  g.N = N;
  g.R = N / 2;
  g.T = 180;
  g.c = (double)(N / 2);
  g.max_rho = (double)(N / 2);
  g.max_theta = (double)(2 * 3.14159265358979f);  // float arithmetic, as vtkMath::Pi returns float
  g.two_pi = 2.0 * (double)3.14159265358979f;
  g.rstep = (g.max_rho - 0) / (g.R - 1);
  g.tstep = (g.max_theta - 0) / (g.T - 1);
  w_tmp.ensure(n3);
  w_w.ensure((long)g.R * N);
  w_r.ensure(n3);
  CK(cudaMemcpyAsync(w_tmp.p, vol, n3 * sizeof(float), cudaMemcpyHostToDevice, st));
  k_cyl_profile<<<(g.R * N + 127) / 128, 128, 0, st>>>(w_tmp.p, g, w_w.p);
  post_launch();
  k_cyl_expand<<<nblocks<int>(n3, 256, 4096), 256, 0, st>>>(w_w.p, g, w_r.p);
  post_launch();
  CK(cudaMemcpyAsync(out, w_r.p, n3 * sizeof(float), cudaMemcpyDeviceToHost, st));
  sync();
  check_status();
}

// Spherical wedge of a class average (updateAccumulatedSphericalWedgeImageMPI + updateSphericalWedgeImage,
// inc/em/nbfWedgedAverageImage3D.h:612-665): members with |w| > 0, own matrix reset as the average resamples
// them, binary wedges under their alignments counted per sample on the device; the average's wedge is
// count > max(count) / 2.
void ettk_ctx::average_spherical_wedge(int M, const int *parts, const float *weights, const double *mats,
                                       float *count, float *wedge) {
  const int n = 2 * B;
  std::vector<WedgeVecs> wv;
  for (int i = 0; i < M; ++i) {
    if (parts[i] < 0 || parts[i] >= V) throw CudaError(ETTK_ERR_ARG, "member index out of range");
    if (!(fabs(weights[i]) > 0)) continue;
    VolumeGeom g = partg[parts[i]];
    for (int k = 0; k < 16; ++k) g.matrix[k] = (k % 5 == 0) ? 1.0 : 0.0;
    Mat4 t;
    memcpy(t.e, mats + 16 * (long)i, sizeof(t.e));
    WedgeVecs w{};
    w.full = g.full_wedge() ? 1 : 0;
    if (!w.full) wedge_vectors(g, &t, w.v1, w.v2);
    wv.push_back(w);
  }
  const int E = (int)wv.size();
  // cos / sin tables in float as the reference evaluates them: phiK = pi_f / (n - 1), thetaK = 2 pi_f / (n - 1)
  const float phiK = (float)(M_PI / (n - 1)), thetaK = (float)(2.0 * M_PI / (n - 1));
  std::vector<float> trig(4 * (size_t)n);
  for (int k = 0; k < n; ++k) {
    trig[k] = cosf(k * thetaK);
    trig[n + k] = sinf(k * thetaK);
    trig[2 * n + k] = sinf(k * phiK);
    trig[3 * n + k] = cosf(k * phiK);
  }
  w_wv.ensure(std::max(E, 1));
  w_tmp.ensure(4L * n + (long)n * n);
  if (E) CK(cudaMemcpyAsync(w_wv.p, wv.data(), E * sizeof(WedgeVecs), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_tmp.p, trig.data(), trig.size() * sizeof(float), cudaMemcpyHostToDevice, st));
  float *dcount = w_tmp.p + 4L * n;
  k_sph_wedge_count<<<(n * n + 255) / 256, 256, 0, st>>>(w_wv.p, E, w_tmp.p, n, dcount);
  post_launch();
  std::vector<float> c((size_t)n * n);
  CK(cudaMemcpyAsync(c.data(), dcount, c.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
  sync();
  check_status();
  const float mx = *std::max_element(c.begin(), c.end());
  for (size_t k = 0; k < c.size(); ++k) {
    if (count) count[k] = c[k];
    wedge[k] = (c[k] > mx / 2.0) ? 1.f : 0.f;
  }
}

// The band of getLowDimensionRepresentationHalf: coefficients with |filter| > 0.5, listed as the reference
// iterates its [x][y][kz] half spectrum (kz fastest), as offsets into the kz-major layout.
const std::vector<int> &ettk_ctx::representation_band() {
  if (!repr_idx.empty()) return repr_idx;
  const int H = N / 2 + 1;
  std::vector<float> fk(h3);
  d2h(fk.data(), filter.p, h3 * sizeof(float));
  std::vector<int> band;
  for (int x = 0; x < N; ++x)
    for (int y = 0; y < N; ++y)
      for (int k = 0; k < H; ++k) {
        const int g = (k * N + x) * N + y;
        if (std::fabs(fk[g]) > 0.5f) band.push_back(g);
      }
  repr_idx_dev.ensure(std::max<size_t>(band.size(), 1));
  h2d(repr_idx_dev.p, band.data(), band.size() * sizeof(int));
  repr_idx.swap(band);  // cached only once the device copy is in place
  return repr_idx;
}

// nbfFourierImageMetric::getLowDimensionRepresentationHalf (inc/em/nbfFourierImageMetric.h:1967-2034), padding 1,
// for M particles: A = getImage (own geometry, mean of valid voxels removed); with fold > 1, A = the mean of
// A's getImage as an average image under RotateZ(i * 360 / fold) (nbfImageFilter::symmetrize); F = R2C(A shift)
// * filter; a = C2R(F) * mask (the image filter's mask); F2 = R2C(a), all unnormalised as FFTW; R[m][q] = (re,
// im) of F2 at the band's q-th coefficient and the wedge bit (getWedgeImageHalf > 0.5; 1 when fold > 1).
void ettk_ctx::representations(int M, const int *parts, int fold, float *R) {
  const std::vector<int> &band = representation_band();
  const int K = (int)band.size(), H = N / 2 + 1;
  const int chunk = (int)std::max(1L, std::max(16L, std::min(256L, 256L * 64 * 64 * 64 / n3)) / std::max(1, fold));
  std::vector<ResliceItem> sym_items;
  std::vector<double> sym_acc0;
  std::vector<float2> vals;
  for (int c0 = 0; c0 < M; c0 += chunk) {
    const int E = std::min(chunk, M - c0);
    std::vector<ResliceItem> items(E);
    for (int e = 0; e < E; ++e) {
      const int p = parts[c0 + e];
      double m12[12];
      reslice_index(partg[p], N, nullptr, m12);
      items[e].vol = part_vol(p);
      items[e].tmap = part_map(p);
      part_dims(items[e].dims);
      set_map(items[e], m12);
    }
    const int F = fold > 1 ? fold : 1;
    w_items.ensure((long)E * F);
    w_v.ensure((long)E * F * n3);
    w_cA.ensure((long)E * h3);
    w_acc.ensure(2L * E * F);
    w_p1.ensure((long)E * K);
    CK(cudaMemcpyAsync(w_items.p, items.data(), E * sizeof(ResliceItem), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(w_acc.p, 0, 2L * E * sizeof(double), st));
    reslice(w_items.p, w_v.p, w_acc.p, 2, nullptr, E);
    const float *pre_src = w_v.p;
    const double *pre_acc = w_acc.p;
    if (F > 1) {
      // the images as fixed images, each resliced under the F rotations about z (as ettk_gpu_symmetrize), the
      // mean of each item's F getImage values as its symmetrised image
      w_tmp.ensure((long)E * n3);
      w_r.ensure((long)E * n3);
      k_getimage_fixed<<<nblocks<int>((long)E * n3, 256, 8192), 256, 0, st>>>(w_v.p, w_acc.p, E, N, w_tmp.p);
      post_launch();
      VolumeGeom g{};
      g.lwedge = -90.f;
      g.uwedge = 90.f;
      for (int k = 0; k < 3; ++k) g.position[k] = (float)(N / 2.0);
      for (int k = 0; k < 16; ++k) g.matrix[k] = (k % 5 == 0) ? 1.0 : 0.0;
      sym_items.assign((size_t)E * F, ResliceItem{});
      for (int i = 0; i < F; ++i) {
        Mat4 t = Mat4::eye();
        rotate(t, i * 360.0 / F, 0, 0, 1);
        double m12[12];
        reslice_index(g, N, &t, m12);
        for (int e = 0; e < E; ++e) {
          ResliceItem &it = sym_items[(size_t)e * F + i];
          it.vol = w_tmp.p + (long)e * n3;
          it.tmap = nullptr;
          it.dims[0] = it.dims[1] = it.dims[2] = N;
          set_map(it, m12);
        }
      }
      CK(cudaMemcpyAsync(w_items.p, sym_items.data(), sym_items.size() * sizeof(ResliceItem), cudaMemcpyHostToDevice,
                         st));
      CK(cudaMemsetAsync(w_acc.p, 0, 2L * E * F * sizeof(double), st));
      {
        Scope sc(this, "reslice", 8.0 * E * F * n3);
        k_reslice_brick<true><<<dim3((N / RB) * (N / RB) * (N / RB), (unsigned)(E * F)), 256, RS_SMEM, st>>>(
            w_items.p, N, w_v.p, w_acc.p, 2, status.p, nullptr);
        post_launch();
      }
      k_sym_mean<<<nblocks<int>((long)E * n3, 256, 8192), 256, 0, st>>>(w_v.p, w_acc.p, F, E, N, w_r.p);
      post_launch();
      // every value valid and the mean already removed: sums (0, 1) per item
      sym_acc0.assign(2 * (size_t)E, 0.0);
      for (int e = 0; e < E; ++e) sym_acc0[2 * e + 1] = 1.0;
      w_w.ensure(2L * E);
      CK(cudaMemcpyAsync(w_w.p, sym_acc0.data(), sym_acc0.size() * sizeof(double), cudaMemcpyHostToDevice, st));
      pre_src = w_r.p;
      pre_acc = w_w.p;
    }
    PreParticle pre{pre_src, nullptr, pre_acc, 2, N};
    r2c_z(N, pre, w_cA.p, (long)E * N * N);
    xy_kxy(N, w_cA.p, E, -1);
    switch (N) {
      case 16: fft2d_t<16>(OpFilterShared<16>{w_cA.p, filter.p}, E); break;
      case 32: fft2d_t<32>(OpFilterShared<32>{w_cA.p, filter.p}, E); break;
      case 64: fft2d_t<64>(OpFilterShared<64>{w_cA.p, filter.p}, E); break;
      case 128: fft2d_t<128>(OpFilterShared<128>{w_cA.p, filter.p}, E); break;
      default: throw CudaError(ETTK_ERR_ARG, "unsupported box size for representations");
    }
    c2r_r2c_z(N, w_cA.p, MidMask{mask.p}, (long)E * N * N);
    xy_kxy(N, w_cA.p, E, -1);
    if (K) {
      k_repr_gather<<<nblocks<int>((long)E * K, 256, 4096), 256, 0, st>>>(w_cA.p, E, h3, repr_idx_dev.p, K, w_p1.p);
      post_launch();
    }
    vals.resize((size_t)E * K);
    CK(cudaMemcpyAsync(vals.data(), w_p1.p, vals.size() * sizeof(float2), cudaMemcpyDeviceToHost, st));
    sync();
    check_status();
    parallel_for(E, [&](int e) {
      std::vector<float> w;
      if (F == 1) wedge_half_host(partg[parts[c0 + e]], N, w);
      float *r = R + (size_t)(c0 + e) * K * 3;
      for (int q = 0; q < K; ++q) {
        const int g = band[q], kz = g / (N * N), x = (g / N) % N, y = g % N;
        r[3 * q] = vals[(size_t)e * K + q].x;
        r[3 * q + 1] = vals[(size_t)e * K + q].y;
        r[3 * q + 2] = (F > 1 || w[((size_t)x * N + y) * H + kz] > .5f) ? 1.f : 0.f;
      }
    });
  }
}

// The voxels kept by getLowDimensionRepresentationReal (inc/em/nbfFourierImageMetric.h:2482-2523): with an integer
// bin factor vtkImageResample (magnification 1 / bin, cubic) samples both the image and the mask at the input
// indices bin * i, i = 0 .. floor((N - 1) / bin), integer positions where the tricubic kernel is the voxel itself;
// the values where the (binned) mask exceeds 0.5 are kept in the [x][y][z] order of the binned array.
const std::vector<int> &ettk_ctx::representation_real_band(int bin) {
  if (real_bin == bin) return real_idx;
  std::vector<float> mh(n3);
  d2h(mh.data(), mask.p, n3 * sizeof(float));
  const int nb = (N - 1) / bin + 1;
  std::vector<int> band;
  for (int x = 0; x < nb; ++x)
    for (int y = 0; y < nb; ++y)
      for (int z = 0; z < nb; ++z) {
        const int id = (x * bin * N + y * bin) * N + z * bin;
        if (mh[id] > .5f) band.push_back(id);
      }
  real_idx_dev.ensure(std::max<size_t>(band.size(), 1));
  h2d(real_idx_dev.p, band.data(), band.size() * sizeof(int));
  real_idx.swap(band);
  real_bin = bin;
  return real_idx;
}

// nbfFourierFilter::executeHalf of E real images ([e][x][y][z], centring sign not applied) without a wedge:
// dst = C2R(filter * R2C(src * shift)) * shift / N^3, [e][x][y][z].
void ettk_ctx::real_filtered(const float *src, int E, float *dst) {
  w_cA.ensure((long)E * h3);
  r2c_z(N, PreProductShift{src, nullptr, N}, w_cA.p, (long)E * N * N);
  xy_kxy(N, w_cA.p, E, -1);
  switch (N) {
    case 16: fft2d_t<16>(OpFilterShared<16>{w_cA.p, filter.p}, E); break;
    case 32: fft2d_t<32>(OpFilterShared<32>{w_cA.p, filter.p}, E); break;
    case 64: fft2d_t<64>(OpFilterShared<64>{w_cA.p, filter.p}, E); break;
    case 128: fft2d_t<128>(OpFilterShared<128>{w_cA.p, filter.p}, E); break;
    default: throw CudaError(ETTK_ERR_ARG, "unsupported box size for representations");
  }
  c2r_z(N, w_cA.p, PostStoreScaledSigned{dst, N, 1.0f / (float)n3}, (long)E * N * N);
}

// nbfFourierImageMetric::getLowDimensionRepresentationReal (inc/em/nbfFourierImageMetric.h:2375-2533), no mask file,
// integer bin factor, for M particles. fold <= 1: A = getImage of the particle (own geometry, valid voxels minus their
// mean, 0 elsewhere). fold > 1 (2377-2439): A = the wedged average of the particle alone under its matrix times
// RotateZ(f * 360 / fold), f < fold, weights 1 / fold (the class average of ettk_gpu_average). A is band-pass
// filtered (executeHalf on the real array); with fold > 1 it is then symmetrised n-fold about z
// (nbfImageFilter::symmetrize: the mean of its getImage values as a fixed image under RotateZ(i * 360 / fold));
// R[m][q] = A at the q-th kept voxel (representation_real_band).
void ettk_ctx::representations_real(int M, const int *parts, int fold, int bin, float *R) {
  const std::vector<int> &band = representation_real_band(bin);
  const int K = (int)band.size();
  std::vector<float> vals;
  if (fold <= 1) {
    const int chunk = (int)std::max(16L, std::min(256L, 256L * 64 * 64 * 64 / n3));
    for (int c0 = 0; c0 < M; c0 += chunk) {
      const int E = std::min(chunk, M - c0);
      std::vector<ResliceItem> items(E);
      for (int e = 0; e < E; ++e) {
        const int p = parts[c0 + e];
        double m12[12];
        reslice_index(partg[p], N, nullptr, m12);
        items[e].vol = part_vol(p);
        items[e].tmap = part_map(p);
        part_dims(items[e].dims);
        set_map(items[e], m12);
      }
      w_items.ensure(E);
      w_v.ensure((long)E * n3);
      w_r.ensure((long)E * n3);
      w_acc.ensure(2L * E);
      w_real.ensure(std::max(1L, (long)E * K));
      CK(cudaMemcpyAsync(w_items.p, items.data(), E * sizeof(ResliceItem), cudaMemcpyHostToDevice, st));
      CK(cudaMemsetAsync(w_acc.p, 0, 2L * E * sizeof(double), st));
      reslice(w_items.p, w_v.p, w_acc.p, 2, nullptr, E);
      // getImage values (valid voxels minus their mean, 0 elsewhere), still [e][x][y][z]
      w_tmp.ensure((long)E * n3);
      k_getimage_values<<<nblocks<int>((long)E * n3, 256, 8192), 256, 0, st>>>(w_v.p, w_acc.p, E, N, w_tmp.p);
      post_launch();
      real_filtered(w_tmp.p, E, w_r.p);
      if (K) {
        k_real_gather<<<nblocks<int>((long)E * K, 256, 4096), 256, 0, st>>>(w_r.p, E, n3, real_idx_dev.p, K, w_real.p);
        post_launch();
      }
      vals.resize((size_t)E * K);
      CK(cudaMemcpyAsync(vals.data(), w_real.p, vals.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
      sync();
      check_status();
      std::copy(vals.begin(), vals.end(), R + (size_t)c0 * K);
    }
    return;
  }
  const int F = fold;
  std::vector<int> pp(F);
  std::vector<float> w(F, 1.0f / (float)F);
  std::vector<double> mats(16L * F);
  // the rotations of the symmetrisation, applied to the filtered image as a fixed image centred at N/2
  VolumeGeom g{};
  g.lwedge = -90.f;
  g.uwedge = 90.f;
  for (int k = 0; k < 3; ++k) g.position[k] = (float)(N / 2.0);
  for (int k = 0; k < 16; ++k) g.matrix[k] = (k % 5 == 0) ? 1.0 : 0.0;
  std::vector<ResliceItem> sym(F);
  for (int i = 0; i < F; ++i) {
    Mat4 t = Mat4::eye();
    rotate(t, i * 360.0 / F, 0, 0, 1);
    double m12[12];
    reslice_index(g, N, &t, m12);
    sym[i].dims[0] = sym[i].dims[1] = sym[i].dims[2] = N;
    sym[i].tmap = nullptr;
    set_map(sym[i], m12);
  }
  const std::vector<double> acc0 = {0.0, 1.0};  // every value valid, nothing to remove
  DevBuf<double> dacc0;
  dacc0.ensure(2);
  h2d(dacc0.p, acc0.data(), 2 * sizeof(double));
  DevBuf<float> filt, fixed;
  filt.ensure(n3);
  fixed.ensure(n3);
  w_real.ensure(std::max<long>(1, K));
  vals.resize(K);
  for (int m = 0; m < M; ++m) {
    const int p = parts[m];
    Mat4 own;
    memcpy(own.e, partg[p].matrix, sizeof(own.e));
    for (int f = 0; f < F; ++f) {
      Mat4 t = Mat4::eye();
      rotate(t, f * 360.0 / F, 0, 0, 1);
      const Mat4 mf = mul(own, t);  // vtkMatrix4x4::Multiply4x4(matrix, rotation)
      memcpy(mats.data() + 16L * f, mf.e, sizeof(mf.e));
      pp[f] = p;
    }
    average_accumulate(F, pp.data(), w.data(), mats.data());
    average_finish_device(false);  // w_tmp: the average, [x][y][z]
    real_filtered(w_tmp.p, 1, filt.p);
    // the filtered image as a fixed image (x fastest), resliced under the F rotations; the mean of their getImage values
    k_getimage_fixed<<<nblocks<int>(n3, 256, 8192), 256, 0, st>>>(filt.p, dacc0.p, 1, N, fixed.p);
    post_launch();
    for (int i = 0; i < F; ++i) sym[i].vol = fixed.p;
    w_items.ensure(F);
    w_v.ensure((long)F * n3);
    w_acc.ensure(2L * F);
    CK(cudaMemcpyAsync(w_items.p, sym.data(), F * sizeof(ResliceItem), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(w_acc.p, 0, 2L * F * sizeof(double), st));
    {
      Scope sc(this, "reslice", 8.0 * F * n3);
      k_reslice_brick<true><<<dim3((N / RB) * (N / RB) * (N / RB), (unsigned)F), 256, RS_SMEM, st>>>(
          w_items.p, N, w_v.p, w_acc.p, 2, status.p, nullptr);
      post_launch();
    }
    k_sym_mean<<<nblocks<int>(n3, 256, 8192), 256, 0, st>>>(w_v.p, w_acc.p, F, 1, N, filt.p);
    post_launch();
    if (K) {
      k_real_gather<<<nblocks<int>((long)K, 256, 4096), 256, 0, st>>>(filt.p, 1, n3, real_idx_dev.p, K, w_real.p);
      post_launch();
    }
    CK(cudaMemcpyAsync(vals.data(), w_real.p, (size_t)K * sizeof(float), cudaMemcpyDeviceToHost, st));
    sync();
    check_status();
    std::copy(vals.begin(), vals.end(), R + (size_t)m * K);
  }
}

// ---------------------------------------------------------------- continuous pose refinement

// Per pair at its starting pose T0: fw = W1 * W2(T0) * filter (as the CCF evaluation builds it) and the
// reference filtered by fw, y1 = C2R(FI1 * fw) (scale irrelevant to the normalised correlation).
void ettk_ctx::refine_setup(const std::vector<EvalReq> &req) {
  const long P = (long)req.size();
  const int ACC = 8;
  w_wv.ensure(P);
  w_idx.ensure(P);
  w_fw.ensure(P * h3);
  w_cA.ensure(P * h3);
  w_acc.ensure(P * ACC);
  rf_fw.ensure(P * h3);
  rf_y1.ensure(P * n3);
  std::vector<WedgeVecs> wv(P);
  std::vector<int> refidx(P);
  rf_part.resize(P);
  for (long e = 0; e < P; ++e) {
    const VolumeGeom &g = partg[req[e].part];
    WedgeVecs w{};
    w.full = g.full_wedge() ? 1 : 0;
    if (!w.full) wedge_vectors(g, &req[e].t, w.v1, w.v2);
    wv[e] = w;
    refidx[e] = req[e].ref;
    rf_part[e] = req[e].part;
  }
  CK(cudaMemcpyAsync(w_wv.p, wv.data(), P * sizeof(WedgeVecs), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_idx.p, refidx.data(), P * sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(w_acc.p, 0, P * ACC * sizeof(double), st));
  if (p.wedge_compensation) {
    with_n(N, [&](auto nn) { wedge_t<decltype(nn)::value>(P, w_acc.p, ACC); });
  } else {
    for (long e = 0; e < P; ++e) CK(cudaMemcpyAsync(w_fw.p + e * h3, filter.p, h3 * 4, cudaMemcpyDeviceToDevice, st));
  }
  CK(cudaMemcpyAsync(rf_fw.p, w_fw.p, P * h3 * 4, cudaMemcpyDeviceToDevice, st));
  with_n(N, [&](auto nn) {
    constexpr int NN = decltype(nn)::value;
    fft2d_t<NN>(OpFilterInv<NN>{FI1.p, w_idx.p, rf_fw.p, w_cA.p, HalfSums<NN>{w_acc.p, ACC, 2}}, P, "refine", 20.0);
  });
  c2r_z(N, w_cA.p, PostStore{rf_y1.p, N}, P * N * N);
}

// rho (and with grad, its gradient w.r.t. the right perturbation (w, d) at each map) of E evaluations;
// maps[e] = index map (origin, axes), pair[e] = the refine_setup pair it belongs to.
void ettk_ctx::refine_eval(const std::vector<std::array<double, 12>> &maps, const std::vector<int> &pair, bool grad,
                           std::vector<double> &rho, std::vector<double> &g6) {
  const long E = (long)maps.size();
  w_items.ensure(E);
  w_v.ensure(E * n3);
  w_r.ensure(E * n3);
  w_cB.ensure(E * h3);
  w_acc.ensure(E * 2);
  rf_pair.ensure(E);
  rf_acc.ensure(E * 20);
  if (grad) rf_a.ensure(E * n3);
  std::vector<ResliceItem> items(E);
  for (long e = 0; e < E; ++e) {
    const int part = rf_part[pair[e]];
    ResliceItem it;
    it.vol = part_vol(part);
    it.tmap = part_map(part);
    part_dims(it.dims);
    set_map(it, maps[e].data());
    items[e] = it;
  }
  CK(cudaMemcpyAsync(w_items.p, items.data(), E * sizeof(ResliceItem), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(rf_pair.p, pair.data(), E * sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(w_acc.p, 0, E * 2 * sizeof(double), st));
  CK(cudaMemsetAsync(rf_acc.p, 0, E * 20 * sizeof(double), st));
  {
    Scope sc(this, "reslice", 8.0 * E * n3);
    // clamped values everywhere: rho stays smooth when a shift moves the window past the fixed image's edge
    reslice(w_items.p, w_v.p, w_acc.p, 2, nullptr, E, true);
  }
  // g = K u, u = valid (r - mean) maskfft shift
  auto filtered = [&](auto pre) {
    r2c_z(N, pre, w_cB.p, E * N * N);
    with_n(N, [&](auto nn) {
      constexpr int NN = decltype(nn)::value;
      fft2d_t<NN>(OpFwdFilterIdx<NN>{w_cB.p, rf_fw.p, rf_pair.p}, E, "refine", 20.0);
    });
    xy_kxy(N, w_cB.p, E, +1);
    c2r_z(N, w_cB.p, PostStore{w_r.p, N}, E * N * N);
  };
  const dim3 gn(nblocks<int>(n3, 256, 64), E);
  CK(cudaMemsetAsync(w_acc.p, 0, E * 2 * sizeof(double), st));
  k_masked_mean<<<gn, 256, 0, st>>>(w_v.p, refmask.p, (int)n3, w_acc.p);  // window: the CCF's mask m1
  post_launch();
  filtered(PreMaskedParticle{w_v.p, refmask.p, w_acc.p, N});
  k_ncc_sums<<<gn, 256, 0, st>>>(rf_y1.p, rf_pair.p, w_r.p, refmask.p, (int)n3, rf_acc.p);
  post_launch();
  if (grad) {
    k_ncc_adjoint<<<gn, 256, 0, st>>>(rf_y1.p, rf_pair.p, w_r.p, refmask.p, (int)n3, rf_acc.p, rf_a.p);
    post_launch();
    filtered(PreCopy{rf_a.p, N});  // K a into w_r
    Scope sc(this, "refine_grad", 8.0 * E * n3);
    k_reslice_grad<<<dim3(nblocks<int>(n3, 256, 64), E), 256, 0, st>>>(w_items.p, N, w_v.p, w_r.p, refmask.p,
                                                                        rf_acc.p + E * 4);
    post_launch();
  }
  std::vector<double> h(E * 20);
  read_back(h.data(), rf_acc.p, E * 20 * sizeof(double));
  check_status();
  rho.assign(E, 0.0);
  if (grad) g6.assign(E * 6, 0.0);
  for (long e = 0; e < E; ++e) {
    const double syg = h[e * 4], sgg = h[e * 4 + 1], syy = h[e * 4 + 2];
    rho[e] = (sgg > 0 && syy > 0) ? syg / sqrt(sgg * syy) : 0.0;
    if (grad) {
      const double *a = h.data() + E * 4 + e * 16;
      const double dbar = a[13] > 0 ? a[12] / a[13] : 0.0;
      for (int k = 0; k < 3; ++k) {
        g6[e * 6 + k] = a[3 + k] - dbar * a[9 + k];      // d rho / d w (radians)
        g6[e * 6 + 3 + k] = a[k] - dbar * a[6 + k];      // d rho / d d (voxels)
      }
    }
  }
}

// Gradient ascent of rho from each request's pose: per iteration one gradient and a three-step line search
// along the gradient in voxel units (rotation scaled by the mask radius), accepting only improvements.
void ettk_ctx::refine(const std::vector<EvalReq> &req, int iterations, std::vector<Mat4> &out,
                      std::vector<double> &rho_out) {
  const long P = (long)req.size();
  refine_setup(req);
  std::vector<std::array<double, 12>> cur(P);
  for (long i = 0; i < P; ++i) reslice_index(partg[req[i].part], N, &req[i].t, cur[i].data());
  std::vector<int> self(P);
  for (long i = 0; i < P; ++i) self[i] = (int)i;
  const double Rg = 0.6 * (p.mask_radius > 0 ? p.mask_radius : 0.5 * N);
  std::vector<double> alpha(P, 0.5), rho, g6, rt;
  std::vector<char> done(P, 0);
  for (int it = 0; it < iterations; ++it) {
    refine_eval(cur, self, true, rho, g6);
    std::vector<std::array<double, 12>> trial;
    std::vector<int> tp, tpair;
    const double fac[3] = {0.5, 1.0, 2.0};
    for (long i = 0; i < P; ++i) {
      if (done[i]) continue;
      const double *g = &g6[i * 6];
      const double gu[6] = {g[0] / Rg, g[1] / Rg, g[2] / Rg, g[3], g[4], g[5]};
      double nrm = 0;
      for (double v : gu) nrm += v * v;
      nrm = sqrt(nrm);
      if (!(nrm > 0)) {
        done[i] = 1;
        continue;
      }
      for (double f : fac) {
        const double t = alpha[i] * f;
        const double w[3] = {gu[0] / nrm * t / Rg, gu[1] / nrm * t / Rg, gu[2] / nrm * t / Rg};
        const double d[3] = {gu[3] / nrm * t, gu[4] / nrm * t, gu[5] / nrm * t};
        std::array<double, 12> m;
        perturb_index(cur[i].data(), N, w, d, m.data());
        trial.push_back(m);
        tp.push_back((int)i);
      }
    }
    if (trial.empty()) break;
    refine_eval(trial, tp, false, rt, g6);
    for (size_t k = 0; k < trial.size(); k += 3) {
      const int i = tp[k];
      int best = -1;
      double bv = rho[i];
      for (int q = 0; q < 3; ++q)
        if (rt[k + q] > bv) {
          bv = rt[k + q];
          best = q;
        }
      if (best >= 0) {
        cur[i] = trial[k + best];
        alpha[i] = std::min(2.0, std::max(1e-3, alpha[i] * fac[best]));
      } else {
        alpha[i] *= 0.25;
        if (alpha[i] < 1e-3) done[i] = 1;
      }
    }
  }
  refine_eval(cur, self, false, rho_out, g6);
  out.resize(P);
  for (long i = 0; i < P; ++i) out[i] = pose_from_index(partg[req[i].part], N, cur[i].data());
}

void ettk_ctx::init_tables() {
  status.ensure(1);
  CK(cudaMemset(status.p, 0, sizeof(int)));
  CK(cudaFuncSetAttribute(k_reslice_brick<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RS_SMEM));
  CK(cudaFuncSetAttribute(k_so3_weights<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)so3_weights_smem<64>()));
  CK(cudaFuncSetAttribute(k_reslice_brick<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RS_SMEM));
  CK(cudaFuncSetAttribute(k_reslice_brick<false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  CK(cudaFuncSetAttribute(k_reslice_brick<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RS_SMEM));
  CK(cudaFuncSetAttribute(k_reslice_brick<false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                          (int)RS_SMEM));
  CK(cudaFuncSetAttribute(k_reslice_brick<false, false, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  CK(cudaFuncSetAttribute(k_reslice_brick<false, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  CK(cudaFuncSetAttribute(k_reslice_brick<true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  N = p.N;
  H = N / 2 + 1;
  B = p.B;
  n = 2 * B;
  n3 = (long)N * N * N;
  h3 = (long)N * N * H;
  nn = (long)n * n;
  nso3 = (long)n * n * n;
  // real-space mask (nbfImageFilter::buildMask, spherical raised cosine, inc/em/nbfImageFilter.h:383-472)
  std::vector<float> m(n3, 1.0f), mf(n3, 0.0f), f(h3, 1.0f);
  if (p.mask_radius != 0) {
    float center = (float)(N / 2.0);
    float r2 = std::min((float)(N - 1), (float)(p.mask_radius + p.mask_sigma / 2.0));
    float r1 = (float)std::max(0.0, (double)(p.mask_radius - p.mask_sigma / 2.0));
    float kappa = (float)(M_PI / (r2 - r1));
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < N; ++k) {
          float di = i - center, dj = j - center, dk = k - center;
          float v = sqrtf(di * di + dj * dj + dk * dk);
          if (v <= r1) v = 1;
          if (v >= r2) v = 0;
          if (v > r1 && v <= r2) v = (float)((1 + cosf(kappa * (v - r1))) / 2.0);
          m[((long)i * N + j) * N + k] = v;
        }
  }
  // maskfft: soft box (nbfFourierImageMetric::reinitializeHalf, inc/em/nbfFourierImageMetric.h:640-662)
  int sq = (int)p.square_mask_size;
  if (sq > 0 && sq < floor(N / 2.0)) {
    for (int i = sq; i <= N - 1 - sq; ++i)
      for (int j = sq; j <= N - 1 - sq; ++j)
        for (int k = sq; k <= N - 1 - sq; ++k) mf[((long)i * N + j) * N + k] = 1;
  } else {
    std::fill(mf.begin(), mf.end(), 1.0f);
  }
  {
    // softenMask(maskfft, 2.5) operates on the blitz array with VTK x = first index
    std::vector<float> t(n3);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < N; ++k) t[i + (long)N * (j + (long)N * k)] = mf[((long)i * N + j) * N + k];
    int dims[3] = {N, N, N};
    gaussian_smooth(t, dims, 2.5, (double)(2.5f * .75f));
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < N; ++k) mf[((long)i * N + j) * N + k] = t[i + (long)N * (j + (long)N * k)];
  }
  // filter on the centred half grid (nbfFourierFilter::updateFilterHalf, buildBandPassHalf, buildBFactorHalf)
  int c = N / 2;
  f[((long)c * N + c) * H + (H - 1)] = 0;
  bool band = (p.bp_low > 0.0f) || (p.bp_high < 1.0f);
  double blo = p.bp_low, bhi = p.bp_high, lv = p.bp_low_sigma, hv = p.bp_high_sigma;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < H; ++k) {
        float t0 = (float)((1.0 * i - c) / c), t1 = (float)((1.0 * j - c) / c), t2 = (float)((1.0 * k - c) / c);
        float rad = sqrtf(t0 * t0 + t1 * t1 + t2 * t2);
        long id = ((long)i * N + j) * H + k;
        if (band) {
          float bp = (rad < blo) ? (float)exp(-((blo - rad) * (blo - rad)) / 2.0 / lv / lv) : 1.0f;
          if (rad > bhi) bp = (float)exp(-((rad - bhi) * (rad - bhi)) / 2.0 / hv / hv);
          f[id] *= bp;
        }
        if (p.bfactor != 0) f[id] *= (float)exp(-(double)p.bfactor * (double)(rad * rad));
      }
  sum_filter = 0;
  for (float v : f) sum_filter += v;
  mask.ensure(n3);
  maskfft.ensure(n3);
  filter.ensure(h3);
  h2d(mask.p, m.data(), n3 * 4);
  h2d(maskfft.p, mf.data(), n3 * 4);
  {
    std::vector<float> fk = to_kz_major(f.data(), N);
    h2d(filter.p, fk.data(), h3 * 4);
  }
  // wedge smoothing weights: std 2, radius int(2*0.5)=1, clipped renormalised kernels
  {
    double e1 = exp(-1.0 / 8.0), s3 = 1 + 2 * e1, s2 = 1 + e1;
    smooth.w_int[0] = (float)(e1 / s3);
    smooth.w_int[1] = (float)(1 / s3);
    smooth.w_int[2] = (float)(e1 / s3);
    smooth.w_lo[0] = (float)(1 / s2);
    smooth.w_lo[1] = (float)(e1 / s2);
    smooth.w_hi[0] = (float)(e1 / s2);
    smooth.w_hi[1] = (float)(1 / s2);
  }
  // SO(3) tables: quadrature x Legendre (forward), Legendre (inverse), L2-normalised small-d per cell
  std::vector<double> th(n), wq(n);
  for (int j = 0; j < n; ++j) {
    th[j] = M_PI * (2.0 * j + 1.0) / (4.0 * B);
    double a = 0;
    for (int k = 0; k < B; ++k) a += sin((2.0 * k + 1.0) * th[j]) / (2.0 * k + 1.0);
    wq[j] = (2.0 / B) * sin(th[j]) * a;
  }
  std::vector<double> P((size_t)B * B * n, 0.0);  // [m][l][j]
  for (int mm = 0; mm < B; ++mm) {
    double cc = sqrt((2.0 * mm + 1.0) / 2.0);
    for (int i = 1; i <= mm; ++i) cc *= sqrt((2.0 * i - 1.0) / (2.0 * i));
    if (mm % 2) cc = -cc;
    for (int j = 0; j < n; ++j) {
      double x = cos(th[j]), s = sin(th[j]);
      double pmm = cc * pow(s, mm);
      P[((size_t)mm * B + mm) * n + j] = pmm;
      if (mm + 1 < B) P[((size_t)mm * B + mm + 1) * n + j] = x * sqrt(2.0 * mm + 3.0) * pmm;
      for (int l = mm + 2; l < B; ++l) {
        double a = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)mm * mm));
        double b = sqrt(((l - 1.0) * (l - 1.0) - (double)mm * mm) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
        P[((size_t)mm * B + l) * n + j] = a * (x * P[((size_t)mm * B + l - 1) * n + j] - b * P[((size_t)mm * B + l - 2) * n + j]);
      }
    }
  }
  std::vector<float> hlw((size_t)B * B * n), hplm((size_t)B * B * n);
  double nrm = sqrt(2.0 * M_PI) / n;
  for (size_t i = 0; i < hlw.size(); ++i) {
    int j = (int)(i % n);
    hlw[i] = (float)(nrm * wq[j] * P[i]);
    hplm[i] = (float)P[i];
  }
  lw.ensure(hlw.size());
  plm.ensure(hplm.size());
  h2d(lw.p, hlw.data(), hlw.size() * 4);
  h2d(plm.p, hplm.data(), hplm.size() * 4);
  int ncell = (2 * B - 1) * (2 * B - 1);
  std::vector<int> off(ncell);
  long total = 0;
  for (int cell = 0; cell < ncell; ++cell) {
    int m1 = cell / (2 * B - 1) - (B - 1), m2 = cell % (2 * B - 1) - (B - 1);
    off[cell] = (int)total;
    total += (long)(B - std::max(std::abs(m1), std::abs(m2))) * n;
  }
  std::vector<float> hd(total);
  std::vector<double> hd64(p.wigner_precision == WIG_FP64 ? total : 0);
  std::vector<double> col(B);
  for (int cell = 0; cell < ncell; ++cell) {
    int m1 = cell / (2 * B - 1) - (B - 1), m2 = cell % (2 * B - 1) - (B - 1);
    int l0 = std::max(std::abs(m1), std::abs(m2));
    for (int j = 0; j < n; ++j) {
      small_d(B, m1, m2, th[j], col.data());
      for (int l = l0; l < B; ++l) {
        const double v = sqrt((2.0 * l + 1.0) / 2.0) * col[l];
        hd[off[cell] + (size_t)(l - l0) * n + j] = (float)v;
        if (!hd64.empty()) hd64[off[cell] + (size_t)(l - l0) * n + j] = v;
      }
    }
  }
  dtab.ensure(total);
  doff.ensure(ncell);
  h2d(dtab.p, hd.data(), total * 4);
  if (!hd64.empty()) {
    dtab64.ensure(total);
    h2d(dtab64.p, hd64.data(), total * 8);
  }
  h2d(doff.p, off.data(), ncell * 4);
  std::vector<float> hs(n);
  for (int j = 0; j < n; ++j) hs[j] = (float)sin(M_PI * (2 * j + 1) / 4 / (double)(float)B);
  sinth.ensure(n);
  h2d(sinth.p, hs.data(), n * 4);
  // spherical sampling directions (vtkSphericalTransform, origin pi/4B, spacing 2pi/4B and pi/B)
  std::vector<float4> dv(nn);
  double oy = M_PI / 4.0 / (double)(float)B, sy = 2.0 * M_PI / 4.0 / (double)(float)B, sz = M_PI / (double)(float)B;
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k) {
      double ph = oy + j * sy, t2 = 0.0 + k * sz;
      dv[(size_t)j * n + k] = make_float4((float)(sin(ph) * cos(t2)), (float)(sin(ph) * sin(t2)), (float)cos(ph), 0.f);
    }
  dirs.ensure(nn);
  h2d(dirs.p, dv.data(), nn * sizeof(float4));
  int N2 = 2 * N;
  float lowCut = band ? p.bp_low : 0.0f, highCut = band ? p.bp_high : 1.0f;
  bandL = std::max(4, (int)ceilf(lowCut * (float)(N2 - 1)));
  bandU = (int)ceil(std::min(.5, (double)highCut) * (N2 - 1));
  double rs = floor((double)(p.restrict_rotation * (float)B) / 90.0 - 1.0);
  rstart = (int)std::max(1.0, std::min(rs, (double)(n - 1)));
  set_window(p.restrict_translation);
  apply_reference_mask(m);
}

// m1 of the CCF and what depends on it: the device copy, F(m1 * shift) of the cross term, and the in-mask voxel list
// and sums of the fast form's refinement (which correlates under the same mask)
void ettk_ctx::apply_reference_mask(const std::vector<float> &m1) {
  refmask.ensure(n3);
  h2d(refmask.p, m1.data(), n3 * 4);
  lr_C0 = lr_C1 = 0;
  std::vector<int> ids;  // the voxels inside the mask, in index order: the only ones the refinement's sums see
  for (long i = 0; i < n3; ++i) {
    lr_C0 += (double)m1[i];
    lr_C1 += (double)m1[i] * (double)m1[i];
    if (m1[i] != 0.f) ids.push_back((int)i);
  }
  lr_nin = (long)ids.size();
  lr_in.ensure(std::max<long>(1, lr_nin));
  if (lr_nin) h2d(lr_in.p, ids.data(), lr_nin * sizeof(int));
  // F(m1*shift)
  Fm1.ensure(h3);
  PreProductShift pre{refmask.p, nullptr, N};
  pre.src = nullptr;
  pre.aux = refmask.p;
  r2c_z(N, pre, Fm1.p, (long)N * N);
  xy_kxy(N, Fm1.p, 1, -1);
  sync();
}

// cartesianToSpherical for a batch of volumes (inc/em/nbfProjectionRotationMetric3D.h:264-413)
void ettk_ctx::spherical_projection(const std::vector<ResliceItem> &items, float *Pp_out, const int *out_index) {
  long P = (long)items.size();
  if (P == 0) return;
  int N2 = 2 * N;
  long big_h = (long)N2 * N2 * (N + 1);
  w_items.ensure(P);
  sp_v.ensure(P * n3);
  sp_acc.ensure(P * 4);
  sp_F.ensure(P * big_h);
  sp_M.ensure(P * big_h);
  sp_padc.ensure(P);
  CK(cudaMemcpyAsync(w_items.p, items.data(), P * sizeof(ResliceItem), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(sp_acc.p, 0, P * 4 * sizeof(double), st));
  {
    Scope sc(this, "sphere_reslice", 8.0 * P * n3);
    reslice(w_items.p, sp_v.p, sp_acc.p, 4, nullptr, P);
  }
  k_mean_all<<<dim3(nblocks<int>(n3, 256, 256), P), 256, 0, st>>>(sp_v.p, sp_acc.p, 4, N, sp_acc.p, 2);
  post_launch();
  PrePadded pre{sp_v.p, mask.p, sp_acc.p, 4, N};
  pre.nyquist_only = N2 <= 128;  // k_fft2d_padded consumes the spectra (larger boxes transform every plane)
  // at 2N = 128 the z pass transforms the N^2 lines of the windowed box alone (tiles of 32 lines divide N = 64) and
  // the last plane's magnitude pass supplies the padding lines' Nyquist entries from the padding constant
  pre.real_only = N2 == 128;
  k_pad_constant<<<nblocks<int>(P, 128), 128, 0, st>>>(pre, (int)P, sp_padc.p);
  post_launch();
  r2c_z(N2, pre, sp_F.p, P * N2 * N2, "sphere_fft");
  // (x, y) passes storing |F| directly (the complex spectrum is not used again)
  switch (N2) {
    case 32: padded_magnitude_t<32>(P); break;
    case 64: padded_magnitude_t<64>(P); break;
    case 128: padded_magnitude_t<128>(P); break;
    default: {
      xy_kxy(N2, sp_F.p, P, -1);
      k_magnitude<<<nblocks<int>(P * big_h, 256, 8192), 256, 0, st>>>(sp_F.p, sp_M.p, P * big_h,
                                                                        p.mutual_correlation ? 1 : 0);
      post_launch();
    }
  }
  Scope sc_ss(this, "sphere_sample", 4.0 * P * big_h + 4.0 * P * nn);
  switch (N) {
#define SS_CASE(NN)                                                                                              \
  case NN:                                                                                                       \
    k_sphere_sample<NN><<<dim3(nblocks<int>(nn, tune.sample_block), P), tune.sample_block, 0, st>>>(            \
        sp_M.p, dirs.p, (int)nn, bandL, bandU, sp_padc.p, Pp_out, out_index);                                    \
    break;
    SS_CASE(16)
    SS_CASE(32)
    SS_CASE(64)
    SS_CASE(128)
#undef SS_CASE
    default: throw CudaError(ETTK_ERR_ARG, "unsupported volume size");
  }
  post_launch();
}

// executeFourierNewHalf for a batch of (reference, particle, transform) requests.
void ettk_ctx::eval_chunk(const std::vector<EvalReq> &req, std::vector<EvalRes> &res) {
  long E = (long)req.size();
  res.resize(E);
  if (E == 0) return;
  const int ACC = 8;  // 0,1 reslice sums; 2,3 norm1; 4 k1_m; 5 unused; 6 sum(w*f); 7 unused
  w_items.ensure(E);
  w_wv.ensure(E);
  w_idx.ensure(E);
  w_fw.ensure(E * h3);
  w_cA.ensure(E * h3);
  w_cB.ensure(E * h3);
  w_cC.ensure(E * h3);
  w_v.ensure(E * n3);
  w_acc.ensure(E * ACC * 2);
  w_norm.ensure(E);
  w_norm2.ensure(E);
  w_peak.ensure(E);
  w_out.ensure(E);
  if (!pruned_xy_used()) w_p1.ensure(E * W * N * H);
  w_p2.ensure(E * W * W * H);
  // Reference branch sharing: the wedge * filter, F1, y1 and FFT1re of an evaluation depend only on its
  // reference and its wedge planes; the binary wedge tests the product of two plane distances, so planes
  // negated together (the mirror Scale(-1,-1,-1) * T of the request before) give a bit-identical wedge.
  // Device slots: the Dn evaluations that compute the branch first, then those that share one (i1src).
  std::vector<ResliceItem> items(E);
  std::vector<WedgeVecs> wv(E);
  std::vector<int> refidx(E), ord(E), slot_of(E), i1src(E);
  std::vector<int> direct;
  std::vector<int2> mirrors;
  w_faces.ensure(E * 3 * (long)(N + 1) * (N + 1));
  long Dn = 0;
  {
    HostScope hs_prep(this, "host_eval_prep");
    std::vector<WedgeVecs> wo(E);
    std::vector<char> shares(E, 0);
    for (long e = 0; e < E; ++e) {
      const VolumeGeom &g = partg[req[e].part];
      WedgeVecs w{};
      w.full = g.full_wedge() ? 1 : 0;
      if (!w.full) wedge_vectors(g, &req[e].t, w.v1, w.v2);
      wo[e] = w;
      if (e > 0 && !shares[e - 1] && req[e].ref == req[e - 1].ref && w.full == wo[e - 1].full) {
        const WedgeVecs &q = wo[e - 1];
        bool same = true, neg = true;
        for (int k = 0; k < 3; ++k) {
          same = same && w.v1[k] == q.v1[k] && w.v2[k] == q.v2[k];
          neg = neg && w.v1[k] == -q.v1[k] && w.v2[k] == -q.v2[k];
        }
        shares[e] = w.full || same || neg;
      }
    }
    for (long e = 0; e < E; ++e)
      if (!shares[e]) slot_of[e] = (int)Dn++;
    long m = Dn;
    for (long e = 0; e < E; ++e)
      if (shares[e]) slot_of[e] = (int)m++;
    for (long e = 0; e < E; ++e) {
      const int s = slot_of[e];
      ord[s] = (int)e;
      i1src[s] = shares[e] ? slot_of[e - 1] : s;
      const EvalReq &r = req[e];
      double m12[12];
      reslice_index(partg[r.part], N, &r.t, m12);
      ResliceItem it;
      it.vol = part_vol(r.part);
      it.tmap = part_map(r.part);
      part_dims(it.dims);
      set_map(it, m12);
      items[s] = it;
      wv[s] = wo[e];
      refidx[s] = r.ref;
    }
    // mirror evaluations (the request right after its direct one, Scale(-1,-1,-1) * T with T a rotation, no
    // cut offset) take the direct reslice reversed on every axis plus its faces one step past the box
    // (k_reslice_mirror); only the others are resliced
    std::vector<char> is_mirror(E, 0);
    for (long e = 0; e < E; ++e) {
      bool mirror = false;
      if (e > 0 && !is_mirror[e - 1] && req[e].part == req[e - 1].part && partg[req[e].part].cut_offset == 0.f) {
        const Mat4 &t = req[e - 1].t;
        if (t.e[3] == 0 && t.e[7] == 0 && t.e[11] == 0) {
          Mat4 S = Mat4::eye();
          S.e[0] = S.e[5] = S.e[10] = -1.0;
          const Mat4 m = mul(S, t);
          mirror = true;
          for (int k = 0; k < 16; ++k) mirror = mirror && m.e[k] == req[e].t.e[k];
        }
      }
      is_mirror[e] = mirror;
      if (mirror) {
        mirrors.push_back(make_int2(slot_of[e], slot_of[e - 1]));
        items[slot_of[e - 1]].faces = w_faces.p + (long)slot_of[e - 1] * 3 * (N + 1) * (N + 1);
      } else {
        direct.push_back(slot_of[e]);
      }
    }
  }
  std::unique_ptr<HostScope> hs_launch(new HostScope(this, "host_eval_issue"));
  CK(cudaMemcpyAsync(w_items.p, items.data(), E * sizeof(ResliceItem), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_wv.p, wv.data(), E * sizeof(WedgeVecs), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_idx.p, refidx.data(), E * sizeof(int), cudaMemcpyHostToDevice, st));
  const int *i1 = nullptr;  // slot -> slot holding its reference branch (null when every slot holds its own)
  if (Dn < E) {
    w_i1.ensure(E);
    CK(cudaMemcpyAsync(w_i1.p, i1src.data(), E * sizeof(int), cudaMemcpyHostToDevice, st));
    i1 = w_i1.p;
  }
  CK(cudaMemsetAsync(w_acc.p, 0, E * ACC * 2 * sizeof(double), st));
  CK(cudaMemsetAsync(w_peak.p, 0, E * sizeof(unsigned long long), st));
  double *acc = w_acc.p;
  double *acc2 = w_acc.p + E * ACC;  // second set: particle reslice sums + norm2
  dim3 gh(nblocks<int>(h3, 256, 256), E), gn(nblocks<int>(n3, 256, 256), E);
  bool useWedge = p.wedge_compensation != 0;
  // wedge (W1 * W2(T)) * filter and its sum
  if (useWedge) {
    Scope sc_w(this, "wedge", 4.0 * Dn * h3);
    switch (N) {
      case 16: wedge_t<16>(Dn, acc, ACC); break;
      case 32: wedge_t<32>(Dn, acc, ACC); break;
      case 64: wedge_t<64>(Dn, acc, ACC); break;
      case 128: wedge_t<128>(Dn, acc, ACC); break;
      default: throw CudaError(ETTK_ERR_ARG, "unsupported volume size");
    }
  } else {
    for (long e = 0; e < Dn; ++e) CK(cudaMemcpyAsync(w_fw.p + e * h3, filter.p, h3 * 4, cudaMemcpyDeviceToDevice, st));
  }
  // I1 branch (slots 0..Dn-1): F1 = FI1 * fw (DC zeroed) with its normalisation sums, inverse (x, y) passes,
  // C2R scaled by 1/norm, then k1_m and R2C(I1' m1)
  with_n(N, [&](auto nn) {
    constexpr int NN = decltype(nn)::value;
    fft2d_t<NN>(OpFilterInv<NN>{FI1.p, w_idx.p, w_fw.p, w_cA.p, HalfSums<NN>{acc, ACC, 2}}, Dn, "fft_xy", 20.0);
  });
  k_norms<<<nblocks<int>(Dn, 128), 128, 0, st>>>(acc, ACC, 2, N, (int)Dn, w_norm.p, nullptr);
  post_launch();
  c2r_r2c_z(N, w_cA.p, MidScaleY1M1{w_norm.p, ilog2((long)N * N), refmask.p, acc, ACC, 4, N}, Dn * N * N);
  xy_kxy(N, w_cA.p, Dn, -1);
  // I2 branch: reslice under T, R2C((I2-mean) maskfft shift), forward (x, y) passes then * fw with the
  // normalisation sums
  {
    w_ridx.ensure(E);
    w_mpairs.ensure(std::max<long>(1, (long)mirrors.size()));
    CK(cudaMemcpyAsync(w_ridx.p, direct.data(), direct.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    if (!mirrors.empty())
      CK(cudaMemcpyAsync(w_mpairs.p, mirrors.data(), mirrors.size() * sizeof(int2), cudaMemcpyHostToDevice, st));
  }
  {
    Scope sc(this, "reslice", 8.0 * direct.size() * n3);
    reslice(w_items.p, w_v.p, acc2, ACC, w_ridx.p, (long)direct.size(), false, linear_reslice);
  }
  if (!mirrors.empty()) {
    Scope sc(this, "reslice_mirror", 8.0 * mirrors.size() * n3);
    k_reslice_mirror<<<dim3(nblocks<int>(n3 / 4, 256, 64), (unsigned)mirrors.size()), 256, 0, st>>>(
        w_items.p, w_mpairs.p, N, w_v.p, acc2, ACC);
    post_launch();
  }
  PreParticle pp{w_v.p, maskfft.p, acc2, ACC, N};
  r2c_z(N, pp, w_cB.p, E * N * N);
  with_n(N, [&](auto nn) {
    constexpr int NN = decltype(nn)::value;
    OpFwdFilter<NN> op{w_cB.p, w_fw.p, HalfSums<NN>{acc2, ACC, 2}, i1};
    op.mutual = p.mutual_correlation ? 1 : 0;
    fft2d_t<NN>(op, E, "fft_xy", 20.0);
  });
  k_norms<<<nblocks<int>(E, 128), 128, 0, st>>>(acc2, ACC, 2, N, (int)E, w_norm2.p, nullptr);
  post_launch();
  // FFT2re (into cC), inverse (x, y) passes of F2/norm2, C2R, R2C(I2'^2 shift) into cB, forward passes + cross
  // term
  with_n(N, [&](auto nn) {
    constexpr int NN = decltype(nn)::value;
    fft2d_t<NN>(OpFft2reInv<NN>{w_cA.p, i1, w_cC.p, w_cB.p, w_norm2.p}, E, "fft_xy", 32.0);
  });
  c2r_r2c_z(N, w_cB.p, MidSquareShift{N}, E * N * N);
  with_n(N, [&](auto nn) {
    constexpr int NN = decltype(nn)::value;
    fft2d_t<NN>(OpFwdCross<NN>{w_cB.p, Fm1.p, w_cC.p, 8.0f}, E, "fft_xy", 24.0);
  });
  int o0 = N - (int)floor(N / 2.0), o2 = H - 1;
  {
  Scope sc_p(this, "pruned_dft", 8.0 * E * ((double)N * N * H + 2.0 * W * N * H + 2.0 * W * W * H));
  if (pruned_xy_used()) {
    pruned_xy(w_cB.p, w_p2.p, E, o0);
  } else {
    // x: lines (item, kz, ky) of the kz-major spectrum, stride N, into q1[item][X][kz][ky];
    // y: lines (item, X, kz), contiguous, into q2[item][X][kz][Y]
    pruned_fft<false>(w_cB.p, w_p1.p,
                      PrunedLines{E * H * N, (long)H * N, (long)H * N * N, (long)N, (long)N * N, (long)N,
                                  (long)W * H * N, (long)H * N}, o0);
    pruned_fft<true>(w_p1.p, w_p2.p, PrunedLines{E * W * H, 1, (long)N, 1, 0, 1, (long)W, 1}, o0);
  }
  size_t smz = 2 * (size_t)H * (4 * ((W + 3) / 4)) * sizeof(float2);
  if (smz > 48 * 1024) CK(cudaFuncSetAttribute(k_pruned_z_peak, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smz));
  k_pruned_z_peak<<<dim3(W, E), 128, smz, st>>>(w_p2.p, N, W, lo, o2, rr2, w_peak.p);
  post_launch();
  }
  k_score<<<nblocks<int>(E, 128), 128, 0, st>>>(acc, ACC, w_peak.p, (int)E, W, sum_filter, p.overlap_normalized,
                                                useWedge ? 1 : 0, N, w_out.p, i1);
  post_launch();
  hs_launch.reset();
  std::vector<EvalOut> out(E);
  read_back(out.data(), w_out.p, E * sizeof(EvalOut));
  check_status();
  for (long s = 0; s < E; ++s) {
    const int e = ord[s];
    res[e].dist = out[s].dist;
    Mat4 tr = Mat4::eye();
    if (!(out[s].shift[0] == 0 && out[s].shift[1] == 0 && out[s].shift[2] == 0)) {
      tr.e[3] = -(double)out[s].shift[0];
      tr.e[7] = -(double)out[s].shift[1];
      tr.e[11] = -(double)out[s].shift[2];
    }
    res[e].t = mul(req[e].t, tr);
  }
}

namespace {

// nbfImageMetric::isTransformValid (inc/em/nbfImageMetric.h:415-459)
bool transform_valid(const ettk_params &p, const Mat4 &t) {
  double sh[3] = {t.e[3], t.e[7], t.e[11]};
  if (fabs(sh[0]) > p.restrict_translation || fabs(sh[1]) > p.restrict_translation || fabs(sh[2]) > p.restrict_translation)
    return false;
  double po[3];
  for (int i = 0; i < 3; ++i) po[i] = t.e[4 * i + 2] + t.e[4 * i + 3] - sh[i];
  double d = sqrt(po[0] * po[0] + po[1] * po[1] + po[2] * po[2]);
  if (d != 0)
    for (int i = 0; i < 3; ++i) po[i] /= d;
  double ang = po[2];
  ang = (ang >= 1) ? 0 : fabs(acos(ang) * 57.29577951308232);
  return ang <= p.restrict_rotation;
}

// Host worker threads shared by every context: up to 15 persistent workers plus the calling thread (thread creation
// costs more than most of the host work it would carry). One job at a time; a call from inside a job, from a
// process forked after the workers started, or with a single item runs serially on the caller. The pool is never
// destroyed: its idle workers block on a condition variable until the process exits.
class HostPool {
 public:
  static HostPool &get() {
    static HostPool *pool = new HostPool;
    return *pool;
  }
  void run(int n, const std::function<void(int)> &f) {
    if (n <= 1 || inside || workers.empty() || getpid() != owner) {
      for (int i = 0; i < n; ++i) f(i);
      return;
    }
    std::lock_guard<std::mutex> one(submit);
    {
      std::lock_guard<std::mutex> lk(m);
      job = &f;
      count = n;
      next.store(0);
      busy = (int)workers.size();
      ++gen;
    }
    cv.notify_all();
    inside = true;
    for (int i; (i = next.fetch_add(1)) < n;) f(i);
    inside = false;
    std::unique_lock<std::mutex> lk(m);
    done.wait(lk, [&] { return busy == 0; });
    job = nullptr;
  }
 private:
  HostPool() : owner(getpid()) {
    const int nt = (int)std::min<unsigned>(16u, std::max(1u, std::thread::hardware_concurrency()));
    for (int t = 1; t < nt; ++t) workers.emplace_back([this] { loop(); });
  }
  void loop() {
    unsigned long long seen = 0;
    for (;;) {
      const std::function<void(int)> *f;
      int n;
      {
        std::unique_lock<std::mutex> lk(m);
        cv.wait(lk, [&] { return gen != seen; });
        seen = gen;
        f = job;
        n = count;
      }
      inside = true;
      for (int i; (i = next.fetch_add(1)) < n;) (*f)(i);
      inside = false;
      std::lock_guard<std::mutex> lk(m);
      if (--busy == 0) done.notify_one();
    }
  }
  std::mutex submit, m;
  std::condition_variable cv, done;
  const std::function<void(int)> *job = nullptr;
  int count = 0, busy = 0;
  std::atomic<int> next{0};
  unsigned long long gen = 0;
  pid_t owner;
  std::vector<std::thread> workers;
  static thread_local bool inside;
};
thread_local bool HostPool::inside = false;

// Runs f(0..n-1) on the host workers (independent items; f must not throw).
template <class F>
void parallel_for(int n, F f) {
  const std::function<void(int)> g = [&](int i) { f(i); };
  HostPool::get().run(n, g);
}

// eliminateEquivalentAngles (inc/em/nbfProjectionRotationMetric3D.h:1636-1702). Only pairs whose rotation
// matrices can be closer than `tol` in L1 are compared (each entry must differ by < tol); visiting only
// those pairs in increasing j order is equivalent to the reference's full double loop.
// mats_in, when given, holds euler_candidate of every entry of pos (as computed by the caller).
void eliminate_equivalent(std::vector<Cand> &pos, PQ &pq, float tol, const std::vector<Mat4> *mats_in = nullptr) {
  size_t K = pos.size();
  std::vector<Mat4> own;
  if (!mats_in) {
    own.resize(K);
    for (size_t i = 0; i < K; ++i) own[i] = euler_candidate(pos[i].v[0], pos[i].v[1], pos[i].v[2]);
  }
  const std::vector<Mat4> &mats = mats_in ? *mats_in : own;
  // bucket on the third column of the rotation (entries 2, 6, 10): cells in one flat counting-sort table
  double cell = std::max((double)tol, 1e-3);
  int nc = (int)ceil(2.0 / cell) + 3;
  auto key = [&](double v) { return std::min(nc - 1, std::max(0, (int)floor((v + 1.0) / cell) + 1)); };
  const size_t ncell = (size_t)nc * nc * nc;
  std::vector<int> kx(K), ky(K), kz(K), start(ncell + 1, 0), members(K);
  for (size_t i = 0; i < K; ++i) {
    kx[i] = key(mats[i].e[2]);
    ky[i] = key(mats[i].e[6]);
    kz[i] = key(mats[i].e[10]);
    ++start[((size_t)kx[i] * nc + ky[i]) * nc + kz[i] + 1];
  }
  for (size_t c = 0; c < ncell; ++c) start[c + 1] += start[c];
  {
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (size_t i = 0; i < K; ++i) members[fill[((size_t)kx[i] * nc + ky[i]) * nc + kz[i]]++] = (int)i;
  }
  const float dead = -FLT_MAX;
  std::vector<int> nb;
  for (size_t i = 0; i < K; ++i) {
    nb.clear();
    for (int a = kx[i] - 1; a <= kx[i] + 1; ++a)
      for (int b = ky[i] - 1; b <= ky[i] + 1; ++b)
        for (int c = kz[i] - 1; c <= kz[i] + 1; ++c) {
          if (a < 0 || b < 0 || c < 0 || a >= nc || b >= nc || c >= nc) continue;
          const size_t cc = ((size_t)a * nc + b) * nc + c;
          for (int m = start[cc]; m < start[cc + 1]; ++m) nb.push_back(members[m]);
        }
    std::sort(nb.begin(), nb.end());
    for (int j : nb) {
      if (pos[i].v[3] == dead) break;
      if ((size_t)j != i && pos[j].v[3] > dead) {
        double err = 0;
        for (int m = 0; m < 16; ++m) err += fabs(mats[i].e[m] - mats[j].e[m]);
        if (err < tol) {
          if (pos[i].v[3] > pos[j].v[3]) pos[i].v[3] = dead;
          else pos[j].v[3] = dead;
        }
      }
    }
  }
  for (size_t i = 0; i < K; ++i)
    if (pos[i].v[3] > dead) pq.push(pos[i]);
}

}  // namespace

// Stages 1-3 of execute for a batch of P pairs (reference pr[i], particle pp[i]): spherical projections of the
// particles not yet projected (cartesianToSpherical, inc/em/nbfProjectionRotationMetric3D.h:264-413), every SO(3)
// correlation of the batch's window branches (468-584, 629), the beta restriction and 3x3x3 local maxima (602-646)
// and the per-pair candidate queues after eliminateEquivalentAngles (1592-1702): q1 of the (windowed) correlation,
// q2 of the unwindowed one where a window is used.
void ettk_ctx::so3_queues(int P, const std::vector<int> &pr, const std::vector<int> &pp, std::vector<PairPlan> &plans,
                          std::vector<PQ> &q1, std::vector<PQ> &q2) {
  // 1. spherical projections of particles not yet projected
  {
    std::vector<ResliceItem> items;
    std::vector<int> ids;
    for (int i = 0; i < P; ++i)
      if (!pp2_ready[pp[i]] && std::find(ids.begin(), ids.end(), pp[i]) == ids.end()) ids.push_back(pp[i]);
    const int chunk = 256;
    for (size_t c0 = 0; c0 < ids.size(); c0 += chunk) {
      items.clear();
      size_t c1 = std::min(ids.size(), c0 + chunk);
      for (size_t c = c0; c < c1; ++c) {
        ResliceItem it;
        it.vol = part_vol(ids[c]);
        it.tmap = part_map(ids[c]);
        part_dims(it.dims);
        double m12[12];
        reslice_index(partg[ids[c]], N, nullptr, m12);
        set_map(it, m12);
        items.push_back(it);
      }
      w_idx2.ensure(c1 - c0);
      CK(cudaMemcpyAsync(w_idx2.p, ids.data() + c0, (c1 - c0) * sizeof(int), cudaMemcpyHostToDevice, st));
      spherical_projection(items, Pp2.p, w_idx2.p);  // straight into the particles' rows of Pp2
      for (size_t c = c0; c < c1; ++c) pp2_ready[ids[c]] = 1;
    }
  }
  // 2. SO(3) plans: signals, correlation jobs, scaled jobs
  std::vector<SigDesc> sd;
  std::vector<SynthJob> jobs;
  std::vector<ScaledJob> sjobs;
  plans.assign(P, PairPlan{});
  std::vector<int> jscaled;
  auto sig = [&](int pair, int kind) {
    sd.push_back({pair, kind});
    return (int)sd.size() - 1;
  };
  auto corr = [&](PairPlan &pl, int slot, int pair, int k1, int k2, bool scaled) {
    int f = sig(pair, k1), h = sig(pair, k2);
    jobs.push_back({f, h});
    pl.job[slot] = (int)jobs.size() - 1;
    pl.scaled[slot] = scaled;
    pl.sjob[slot] = -1;
    if (scaled) {
      sjobs.push_back({h, f, (int)jobs.size() - 1});
      pl.sjob[slot] = (int)sjobs.size() - 1;
    }
  };
  for (int i = 0; i < P; ++i) {
    PairPlan &pl = plans[i];
    for (int s = 0; s < 5; ++s) pl.job[s] = -1, pl.scaled[s] = 0, pl.sjob[s] = -1;
    bool u1 = p.wedge_compensation && useW1[pr[i]], u2 = p.wedge_compensation && useW2[pp[i]];
    if (u1 && u2) {
      pl.branch = 1;
      corr(pl, 0, i, K_PP1SQ_W1, K_W2, true);
      corr(pl, 1, i, K_W1, K_PP2SQ_W2, true);
      corr(pl, 2, i, K_PP1_W1, K_PP2_W2, true);
      corr(pl, 3, i, K_W1, K_W2, true);
    } else if (u1) {
      pl.branch = 2;
      corr(pl, 0, i, K_W1, K_PP2SQ, true);
      corr(pl, 1, i, K_W1_PP1, K_PP2, true);
    } else if (u2) {
      pl.branch = 3;
      corr(pl, 0, i, K_PP1SQ, K_W2, true);
      corr(pl, 1, i, K_PP1, K_W2_PP2, true);
    } else {
      pl.branch = 4;
      corr(pl, 0, i, K_PP1, K_PP2, false);
    }
    if (u1 || u2) corr(pl, 4, i, K_PP1, K_PP2, false);
  }
  long NS = (long)sd.size(), NJ = (long)jobs.size(), NSJ = (long)sjobs.size();
  w_sd.ensure(NS);
  w_jobs.ensure(NJ);
  w_sjobs.ensure(std::max(1L, NSJ));
  w_plans.ensure(P);
  w_pair_ref.ensure(P);
  w_pair_pp2.ensure(P);
  w_pair_part.ensure(P);
  w_sig.ensure(NS * nn);
  w_coef.ensure(NS * B * B);
  w_S.ensure(NJ * nso3);
  w_C.ensure(NJ * nso3);
  w_mm.ensure(NJ * 2);
  w_w.ensure(std::max(1L, NSJ) * 2);
  CK(cudaMemcpyAsync(w_sd.p, sd.data(), NS * sizeof(SigDesc), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_jobs.p, jobs.data(), NJ * sizeof(SynthJob), cudaMemcpyHostToDevice, st));
  if (NSJ) CK(cudaMemcpyAsync(w_sjobs.p, sjobs.data(), NSJ * sizeof(ScaledJob), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_plans.p, plans.data(), P * sizeof(PairPlan), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_pair_ref.p, pr.data(), P * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_pair_pp2.p, pp.data(), P * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_pair_part.p, pp.data(), P * 4, cudaMemcpyHostToDevice, st));
  {
    Scope sc_sig(this, "so3_signals", 4.0 * NS * nn * 2);
    k_build_signals<<<NS, 256, 0, st>>>(w_sd.p, w_pair_ref.p, w_pair_pp2.p, Pp1.p, Pp2.p, W1sph.p, W2sph.p,
                                        w_pair_part.p, (int)nn, w_sig.p);
    post_launch();
  }
  size_t smem_sht = (n / 2 + (size_t)n * n) * sizeof(float2);
  switch (B) {
#define SO3_CASE(BB)                                                                                                  \
case BB: {                                                                                                            \
  if (smem_sht > 48 * 1024)                                                                                           \
    CK(cudaFuncSetAttribute(k_sht<BB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_sht));                  \
  {                                                                                                                   \
    Scope sc_sh(this, "sht", 4.0 * NS * nn + 8.0 * NS * B * B);                                                       \
    k_sht<BB><<<NS, 256, smem_sht, st>>>(w_sig.p, lw.p, w_coef.p);                                                    \
    post_launch();                                                                                                    \
  }                                                                                                                   \
  CK(cudaMemsetAsync(w_S.p, 0, NJ * nso3 * sizeof(float2), st));                                                      \
  {                                                                                                                   \
    Scope sc_s(this, "so3_synth", 8.0 * NJ * nso3 + 4.0 * dtab.n);                                                    \
    synth<BB>(NJ);                                                                                                    \
  }                                                                                                                   \
  fft_strided(2 * BB, w_S.p, LineMap{NJ * n * n, n * n, (long)n * n * n, 1, (long)n * n}, -1);                        \
  fft_strided(2 * BB, w_S.p, LineMap{NJ * n * n, n, (long)n * n, 1, (long)n}, -1);                                    \
  CK(cudaMemsetAsync(w_mm.p, 0, NJ * 2 * sizeof(unsigned long long), st));                                            \
  {                                                                                                                   \
    Scope sc_r(this, "so3_real", 12.0 * NJ * nso3);                                                                   \
    k_so3_real<BB><<<dim3(n, NJ), 256, 0, st>>>(w_S.p, w_C.p, w_mm.p);                                                \
    post_launch();                                                                                                    \
  }                                                                                                                   \
  if (NSJ) {                                                                                                          \
    Scope sc_w(this, "so3_weights", 4.0 * NSJ * nn);                                                                  \
    k_so3_weights<BB><<<dim3(NSJ, 2), 256, so3_weights_smem<BB>(), st>>>(w_sjobs.p, w_mm.p, w_coef.p, w_sig.p, dtab.p, doff.p,             \
                                                    plm.p, sinth.p, w_w.p);                                           \
    post_launch();                                                                                                    \
  }                                                                                                                   \
} break;
    SO3_CASE(8)
    SO3_CASE(16)
    SO3_CASE(32)
    SO3_CASE(64)
#undef SO3_CASE
    default:
      throw CudaError(ETTK_ERR_ARG, "unsupported bandwidth");
  }
  // 3. branch combination, beta restriction and local maxima -> host queues
  const int cap = 8192;
  w_cnt.ensure(2 * P);
  w_lists.ensure((long)2 * P * cap);
  CK(cudaMemsetAsync(w_cnt.p, 0, 2 * P * 4, st));
  {
    Scope sc_c(this, "combine_peaks", 4.0 * NJ * nso3);
    const int tiles = (n / CP_T) * (n / CP_T) * (n / CP_T);
    k_combine_peaks<<<dim3(tiles, P), 256, 0, st>>>(w_plans.p, w_C.p, w_mm.p, w_w.p, n, rstart, P, cap, w_cnt.p,
                                                   w_lists.p);
    post_launch();
  }
  std::vector<int> cnt(2 * P);
  read_back(cnt.data(), w_cnt.p, 2 * P * 4);
  int maxc = 0;
  for (int q = 0; q < 2 * P; ++q) {
    if (cnt[q] > cap) throw CudaError(ETTK_ERR_ARG, "too many SO(3) local maxima");
    maxc = std::max(maxc, cnt[q]);
  }
  // the first maxc entries of every list, packed at pitch maxc (list q at lists[q * maxc])
  std::vector<int2> lists((size_t)2 * P * std::max(maxc, 1));
  if (maxc) {
    HostScope hs(this, "host_wait");
    CK(cudaMemcpy2DAsync(lists.data(), maxc * sizeof(int2), w_lists.p, cap * sizeof(int2), maxc * sizeof(int2),
                         2 * P, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  q1.assign(P, PQ());
  q2.assign(P, PQ());
  {
  HostScope hs_q(this, "host_queues");
  // queues are independent: build them on the host cores
  auto build_queue = [&](int q) {
    int c = std::min(cnt[q], cap);
    std::vector<int2> L(lists.begin() + (long)q * maxc, lists.begin() + (long)q * maxc + c);
    std::sort(L.begin(), L.end(), [](const int2 &a, const int2 &b) { return a.x < b.x; });
    std::vector<Cand> pos;
    std::vector<Mat4> mats;
    for (auto &e : L) {
      int a = e.x / (n * n), bb = (e.x / n) % n, g = e.x % n;
      float val = __builtin_bit_cast(float, e.y);
      float alpha = (float)(a / (double)B * 180.0);
      float beta = (float)((2 * bb + 1.0) / (4. * B) * 180.0);
      if ((float)B <= 32) beta = (float)((2 * bb + 0.0) / (4. * B) * 180.0);
      float gamma = (float)(g / (double)B * 180.0);
      const Mat4 m = euler_candidate(alpha, beta, gamma);
      if (transform_valid(p, m)) {
        pos.push_back({{alpha, beta, gamma, -val}, -1});
        mats.push_back(m);
      }
    }
    eliminate_equivalent(pos, q < P ? q1[q] : q2[q - P], 0.25f, &mats);
  };
  parallel_for(2 * P, build_queue);
  }
}

void ettk_ctx::align(int npairs, const int *pairs, float *D, int cols, int ncand) {
  HostScope hs_all(this, "host_align_wall");
  int maxb = p.max_batch > 0 ? p.max_batch : 512;
  std::vector<int> todo;
  for (int i = 0; i < npairs; ++i)
    if (D[(long)i * cols * ncand] == -1) todo.push_back(i);
  for (size_t b0 = 0; b0 < todo.size(); b0 += maxb) {
    int P = (int)std::min<size_t>(maxb, todo.size() - b0);
    std::vector<int> pr(P), pp(P);
    for (int i = 0; i < P; ++i) {
      pr[i] = pairs[2 * todo[b0 + i]];
      pp[i] = pairs[2 * todo[b0 + i] + 1];
      if (pr[i] < 0 || pr[i] >= R || pp[i] < 0 || pp[i] >= V) throw CudaError(ETTK_ERR_ARG, "pair index out of range");
    }
    std::vector<PairPlan> plans;
    std::vector<PQ> q1, q2;
    {
      HostScope hs_so3(this, "stage_so3");
      so3_queues(P, pr, pp, plans, q1, q2);
    }
    HostScope hs_ccf(this, "stage_ccf");  // candidate rounds and final selection
    // 4. candidate rounds (execute 678-776): direct and mirror CCF per popped candidate
    struct PairState {
      int index[2] = {0, 0};
      bool done[2] = {false, false};
      std::vector<Cand> combined[2];
    };
    std::vector<PairState> ps(P);
    std::vector<EvalRes> store;  // direct results referenced by combined entries
    int nqueues_max = 2;
    for (int round = 0;; ++round) {
      std::vector<EvalReq> req;
      struct Pend {
        int pair, q;
        Cand c;
        int e_direct, e_mirror;
      };
      std::vector<Pend> pend;
      for (int i = 0; i < P; ++i) {
        int nq = plans[i].job[4] >= 0 ? 2 : 1;
        for (int q = 0; q < nq && q < nqueues_max; ++q) {
          PairState &S = ps[i];
          if (S.done[q]) continue;
          PQ &Q = q == 0 ? q1[i] : q2[i];
          int peaks = p.candidate_peaks;
          if (q == 1) peaks = (int)std::max(1.0, floor(p.candidate_peaks / 3.0));
          int need = peaks - S.index[q];
          if (need <= 0 || Q.empty()) {
            S.done[q] = true;
            continue;
          }
          for (int t = 0; t < need && !Q.empty(); ++t) {
            Cand c = Q.top();
            if (c.v[3] == FLT_MAX) {
              // reference breaks out of this queue; leave the entry for the check below
              break;
            }
            Q.pop();
            Mat4 t1 = euler_candidate(c.v[0], c.v[1], c.v[2]);
            Mat4 mir = Mat4::eye();
            mir.e[0] = mir.e[5] = mir.e[10] = -1.0;
            mir = mul(mir, t1);
            Pend pd{i, q, c, (int)req.size(), (int)req.size() + 1};
            req.push_back({pr[i], pp[i], t1});
            req.push_back({pr[i], pp[i], mir});
            pend.push_back(pd);
          }
        }
      }
      if (req.empty()) break;
      std::vector<EvalRes> res;
      eval_batch(req, res);
      // apply in the reference's sequential order per (pair, queue)
      for (auto &pd : pend) {
        PairState &S = ps[pd.pair];
        int peaks = p.candidate_peaks;
        if (pd.q == 1) peaks = (int)std::max(1.0, floor(p.candidate_peaks / 3.0));
        if (S.index[pd.q] >= peaks) continue;  // cannot happen: need bounded the pops
        const EvalRes &d = res[pd.e_direct];
        if (transform_valid(p, d.t)) {
          if (res[pd.e_mirror].dist >= d.dist) S.index[pd.q]++;
          store.push_back(d);
          Cand c = pd.c;
          c.v[3] = d.dist;
          c.ref = (int)store.size() - 1;
          S.combined[pd.q].push_back(c);
        }
      }
      // queues whose top is the sentinel stop (execute 699-701)
      for (int i = 0; i < P; ++i)
        for (int q = 0; q < 2; ++q) {
          PQ &Q = q == 0 ? q1[i] : q2[i];
          if (!Q.empty() && Q.top().v[3] == FLT_MAX) ps[i].done[q] = true;
        }
    }
    // 5. final selection (execute 786-907) and output rows (getDistances 1962-2002). With one candidate the
    // row holds the best distance, scale 1 (nbfFourierImageMetric's correlationScale) and getWedgeOverlap at
    // the final transform; otherwise column 0 of every slot is first set to FLT_MAX (1985) and slot c holds
    // candidate c with scale 1 and overlap 1 (candidateWedgeOverlaps, execute 880). Slots past ncand are not
    // written (the reference would write past the end of D).
    const bool multi = p.number_of_candidates != 1;
    std::vector<EvalReq> finals(P);
    std::vector<float> final_d(P);
    for (int i = 0; i < P; ++i) {
      std::vector<Cand> comb = ps[i].combined[0];
      comb.insert(comb.end(), ps[i].combined[1].begin(), ps[i].combined[1].end());
      if (comb.empty()) {
        comb.push_back({{0, 0, 0, 1.0f}, -2});
      }
      PQ pc;
      eliminate_equivalent(comb, pc, 2.5f);
      float best = FLT_MAX;
      const int row = todo[b0 + i];
      auto at = [&](int col, int k) -> float & { return D[((long)row * cols + col) * ncand + k]; };
      if (multi)
        for (int k = 0; k < ncand; ++k) at(0, k) = FLT_MAX;
      int index = 0;
      Mat4 bestT = Mat4::eye();
      while (!pc.empty() && index < p.number_of_candidates) {
        Cand c = pc.top();
        pc.pop();
        EvalRes r;
        if (c.ref >= 0) {
          r = store[c.ref];  // refine(t,0) repeats the direct evaluation at the same rotation
        } else {
          std::vector<EvalRes> rr;
          eval_batch({{pr[i], pp[i], euler_candidate(c.v[0], c.v[1], c.v[2])}}, rr);
          r = rr[0];
        }
        if (r.dist < best) {
          best = r.dist;
          bestT = r.t;
        }
        if (multi && index < ncand) {
          int off = 1;
          at(0, index) = r.dist;
          if (cols > 17) at(1, index) = 1.0f, off = 2;
          if (cols > 18) at(2, index) = 1.0f, off = 3;
          for (int m = 0; m < 16; ++m) at(m + off, index) = (float)r.t.e[m];
        }
        ++index;
      }
      finals[i] = {pr[i], pp[i], bestT};
      final_d[i] = best;
    }
    if (!multi) {
      std::vector<float> ovl;
      if (cols > 18) ovl = wedge_overlaps(finals);
      for (int i = 0; i < P; ++i) {
        const int row = todo[b0 + i];
        auto at = [&](int col) -> float & { return D[((long)row * cols + col) * ncand + 0]; };
        int off = 1;
        at(0) = final_d[i];
        if (cols > 17) at(1) = 1.0f, off = 2;
        if (cols > 18) at(2) = ovl[i], off = 3;
        for (int m = 0; m < 16; ++m) at(m + off) = (float)finals[i].t.e[m];
      }
    }
  }
}

void ettk_ctx::lr_setup(const std::vector<EvalReq> &req) {
  const long P = (long)req.size();
  const int ACC = 8;
  w_wv.ensure(P);
  w_idx.ensure(P);
  w_fw.ensure(P * h3);
  w_cA.ensure(P * h3);
  w_acc.ensure(P * ACC);
  lr_zm.ensure(P * n3);
  lr_items.ensure(P);
  lr_state.ensure(P);
  lr_maps.ensure(P * 12);
  lr_acc.ensure(P * LR_NACC);
  std::vector<WedgeVecs> wv(P);
  std::vector<int> refidx(P);
  std::vector<LRItem> items(P);
  std::vector<LRState> sts(P);
  std::vector<float> maps(P * 12);
  for (long e = 0; e < P; ++e) {
    const VolumeGeom &g = partg[req[e].part];
    WedgeVecs w{};
    w.full = g.full_wedge() ? 1 : 0;
    if (!w.full) wedge_vectors(g, &req[e].t, w.v1, w.v2);
    wv[e] = w;
    refidx[e] = req[e].ref;
    LRItem it;
    const int slot = req[e].part < (int)lr_slot.size() ? lr_slot[req[e].part] : -1;
    it.vol = slot >= 0 ? lr_ip.p + (long)slot * n3 : part_vol(req[e].part);
    part_dims(it.dims);
    it.zm_index = (int)e;
    items[e] = it;
    LRState S{};
    reslice_index(g, N, &req[e].t, S.base);
    S.rho = -1e308;
    S.alpha = 0.5;
    sts[e] = S;
    for (int k = 0; k < 12; ++k) maps[e * 12 + k] = (float)S.base[k];
  }
  CK(cudaMemcpyAsync(w_wv.p, wv.data(), P * sizeof(WedgeVecs), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_idx.p, refidx.data(), P * sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(lr_items.p, items.data(), P * sizeof(LRItem), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(lr_state.p, sts.data(), P * sizeof(LRState), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(lr_maps.p, maps.data(), P * 12 * sizeof(float), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(w_acc.p, 0, P * ACC * sizeof(double), st));
  if (p.wedge_compensation) {
    Scope sc_w(this, "wedge", 4.0 * P * h3);
    with_n(N, [&](auto nn) { wedge_t<decltype(nn)::value>(P, w_acc.p, ACC); });
  } else {
    for (long e = 0; e < P; ++e) CK(cudaMemcpyAsync(w_fw.p + e * h3, filter.p, h3 * 4, cudaMemcpyDeviceToDevice, st));
  }
  // y1 = K(I1): F1 = FI1 fw (DC removed), inverse (x, y) passes, C2R z pass storing m * y1 (centring sign undone)
  with_n(N, [&](auto nn) {
    constexpr int NN = decltype(nn)::value;
    fft2d_t<NN>(OpFilterInv<NN>{FI1.p, w_idx.p, w_fw.p, w_cA.p, HalfSums<NN>{w_acc.p, ACC, 2}}, P, "local_refine_setup",
                20.0);
  });
  c2r_z(N, w_cA.p, PostStoreZm{lr_zm.p, refmask.p, N}, P * N * N);
  k_lr_consts<<<(unsigned)P, 256, 0, st>>>(lr_zm.p, n3, lr_state.p);
  post_launch();
}

void ettk_ctx::decimate(const float *vols, const std::vector<int> &src, float *out) {
  const long M = (long)src.size();
  const int n = N / 2;
  const long hh = (long)n * n * (n / 2 + 1);
  dec_src.ensure(M);
  w_cB.ensure(M * h3);
  w_cA.ensure(M * hh);
  CK(cudaMemcpyAsync(dec_src.p, src.data(), M * sizeof(int), cudaMemcpyHostToDevice, st));
  r2c_z(N, PreSignVol{vols, dec_src.p, N}, w_cB.p, M * N * N);
  xy_kxy(N, w_cB.p, M, -1);
  k_spectrum_crop<<<nblocks<int>(M * hh, 256), 256, 0, st>>>(w_cB.p, N, M, w_cA.p);
  post_launch();
  xy_kxy(n, w_cA.p, M, +1);
  c2r_z(n, w_cA.p, PostStoreSigned{out, n}, M * n * n);
}

// The volume-list row of a geometry on the half grid: positions, cut offset and the matrix translation halved.
static ettk_volume_meta half_meta(const VolumeGeom &g) {
  ettk_volume_meta m{};
  m.lwedge = g.lwedge;
  m.uwedge = g.uwedge;
  for (int i = 0; i < 3; ++i) {
    m.normal[i] = g.normal[i];
    m.position[i] = 0.5f * g.position[i];
  }
  m.cut_offset = 0.5f * g.cut_offset;
  memcpy(m.matrix, g.matrix, sizeof(m.matrix));
  m.matrix[3] *= 0.5;
  m.matrix[7] *= 0.5;
  m.matrix[11] *= 0.5;
  return m;
}

void ettk_ctx::half_setup() {
  if (!half) {
    ettk_params hp = p;
    hp.N = N / 2;
    hp.B = p.fast_coarse_so3 ? std::max(8, p.B / 2) : 8;  // B/2 when the child runs the coarse SO(3) search
    hp.mask_radius = 0.5f * p.mask_radius;
    hp.mask_sigma = 0.5f * p.mask_sigma;
    hp.square_mask_size = 0.5f * p.square_mask_size;
    // normalised frequencies double on the half grid; exp(-b r^2) keeps its value with b / 4
    hp.bp_low = 2.f * p.bp_low;
    hp.bp_high = 2.f * p.bp_high;
    hp.bp_low_sigma = 2.f * p.bp_low_sigma;
    hp.bp_high_sigma = 2.f * p.bp_high_sigma;
    hp.bfactor = 0.25f * p.bfactor;
    hp.restrict_translation = 0.5f * p.restrict_translation;
    hp.wigner_precision = p.fast_coarse_so3 ? p.wigner_precision : 0;
    hp.fast_coarse_so3 = 0;
    ettk_ctx *h = nullptr;
    const int rc = ettk_gpu_create(device, &hp, &h);
    if (rc != ETTK_OK) throw CudaError(rc, "half-grid screening context could not be created");
    half = h;
    half->linear_reslice = p.fast_coarse_so3 >= 2;
    half_refs_ok = false;
  }
  if (!half_refs_ok) {
    const int n = N / 2;
    std::vector<int> src(R);
    for (int r = 0; r < R; ++r) src[r] = r;
    DevBuf<float> dref;  // once per reference set (dec_vol may hold the batch's particles)
    dref.ensure((long)R * n * n * n);
    decimate(refvol.p, src, dref.p);
    std::vector<float> host((size_t)R * n * n * n);
    d2h(host.data(), dref.p, host.size() * sizeof(float));
    std::vector<ettk_volume_meta> meta(R);
    for (int r = 0; r < R; ++r) meta[r] = half_meta(refg[r]);
    const int rc = ettk_gpu_set_references(half, R, host.data(), meta.data());
    if (rc != ETTK_OK) throw CudaError(rc, "half-grid references: " + half->err);
    half_refs_ok = true;
  }
}

// The child's kernel families, reported under "half:" (when profiling).
void ettk_ctx::merge_child_profile() {
  if (!prof || !half) return;
  for (auto &kv : half->prof_agg) {
    ProfAgg &g = prof_agg["half:" + kv.first];
    g.n += kv.second.n;
    g.ms += kv.second.ms;
    g.bytes += kv.second.bytes;
  }
  half->prof_agg.clear();
}

void ettk_ctx::half_particles(const std::vector<int> &pp) {
  half_setup();
  if (!dec_ev) CK(cudaEventCreateWithFlags(&dec_ev, cudaEventDisableTiming));
  CK(cudaEventRecord(dec_ev, st));
  std::vector<int> u;  // the batch's particles in the slot order of lr_filter_particles (dec_vol)
  for (int q : pp)
    if (lr_slot[q] == (int)u.size()) u.push_back(q);
  const long M = (long)u.size();
  std::vector<ettk_volume_meta> meta(M);
  for (long i = 0; i < M; ++i) meta[i] = half_meta(partg[u[i]]);
  const int rc = ettk_gpu_set_particles_device(half, (int)M, dec_vol.p, meta.data());
  if (rc != ETTK_OK) throw CudaError(rc, "half-grid particles: " + half->err);
}

void ettk_ctx::half_screen(const std::vector<int> &pr, const std::vector<int> &pp, const std::vector<EvalReq> &cand,
                           const std::vector<int> &owner, std::vector<EvalReq> &finals) {
  const int P = (int)pr.size();
  CK(cudaStreamWaitEvent(half->st, dec_ev, 0));  // the decimated particles are written on st
  std::vector<EvalReq> hreq(cand.size());
  for (size_t k = 0; k < cand.size(); ++k) hreq[k] = {cand[k].ref, lr_slot[cand[k].part], cand[k].t};
  half->prof = prof;
  std::vector<EvalRes> res;
  half->eval_batch(hreq, res);
  merge_child_profile();
  std::vector<int> best(P, -1);
  for (size_t k = 0; k < cand.size(); ++k) {
    const int i = owner[k];
    if (!transform_valid(half->p, res[k].t)) continue;
    if (best[i] < 0 || res[k].dist < res[best[i]].dist) best[i] = (int)k;
  }
  finals.resize(P);
  for (int i = 0; i < P; ++i) {
    Mat4 t = Mat4::eye();
    if (best[i] >= 0) {
      t = res[best[i]].t;
      t.e[3] *= 2.0;
      t.e[7] *= 2.0;
      t.e[11] *= 2.0;
    }
    finals[i] = {pr[i], pp[i], t};
  }
}

void ettk_ctx::lr_filter_particles(const std::vector<int> &parts, bool with_half) {
  lr_slot.assign(V, -1);
  if (from_tomo || parts.empty()) return;
  std::vector<int> u;
  for (int q : parts)
    if (lr_slot[q] < 0) {
      lr_slot[q] = (int)u.size();
      u.push_back(q);
    }
  const long M = (long)u.size();
  lr_ip.ensure(M * n3);
  lr_src.ensure(M);
  w_cB.ensure(M * h3);
  CK(cudaMemcpyAsync(lr_src.p, u.data(), M * sizeof(int), cudaMemcpyHostToDevice, st));
  r2c_z(N, PreSignVol{partptr, lr_src.p, N}, w_cB.p, M * N * N);
  xy_kxy(N, w_cB.p, M, -1);
  if (with_half) {  // the same spectra, cropped to edge N/2, are the particles of the half-grid screening
    const int n = N / 2;
    const long hh = (long)n * n * (n / 2 + 1);
    w_cA.ensure(M * hh);
    dec_vol.ensure(M * n * n * n);
    k_spectrum_crop<<<nblocks<int>(M * hh, 256), 256, 0, st>>>(w_cB.p, N, M, w_cA.p);
    post_launch();
    xy_kxy(n, w_cA.p, M, +1);
    c2r_z(n, w_cA.p, PostStoreSigned{dec_vol.p, n}, M * n * n);
  }
  with_n(N, [&](auto nn) {
    constexpr int NN = decltype(nn)::value;
    fft2d_t<NN>(OpFilterShared<NN>{w_cB.p, filter.p}, M, "local_refine_setup", 16.0);
  });
  c2r_z(N, w_cB.p, PostStoreSigned{lr_ip.p, N}, M * N * N);
}

void ettk_ctx::lr_run(long P, int iterations) {
  struct Skip {
    bool &f;
    Skip(bool &f_) : f(f_) { f = true; }
    ~Skip() { f = false; }
  } skip(lr_skip_done);
  for (int it = 0; it <= iterations; ++it) {
    CK(cudaMemsetAsync(lr_acc.p, 0, P * LR_NACC * sizeof(double), st));
    lr_eval(P);
    k_lr_update<<<(unsigned)((P + 127) / 128), 128, 0, st>>>(lr_state.p, lr_acc.p, (int)P, (double)N, lr_C0, lr_C1,
                                                              lr_radius(), 1e-3, lr_maps.p);
    post_launch();
  }
}

// Fast form: stages 1-3 as the plain form, then per pair one CCF evaluation (executeFourierNewHalf, the integer
// shift of its upsampled grid) of each of the `peaks` best candidates of the windowed queue and the peaks / 3
// (at least one) best of the unwindowed queue, as the candidate loop takes them, but with no mirror evaluations;
// for boxes of edge 32 and more the CCF runs on the volumes Fourier-cropped to half the edge (the metric's band-pass
// keeps little above half the Nyquist frequency, so the cropped CCF ranks the candidates as the full one does at an
// eighth of the work); the best valid candidate is refined by gradient ascent of the masked normalised correlation
// (local_refine.cuh) in continuous rotation and shift.
void ettk_ctx::align_refined(int npairs, const int *pairs, float *D, int cols, int ncand, int iterations, int peaks) {
  HostScope hs_all(this, "host_align_wall");
  const int maxb = p.max_batch > 0 ? p.max_batch : 512;
  std::vector<int> todo;
  for (int i = 0; i < npairs; ++i)
    if (D[(long)i * cols * ncand] == -1) todo.push_back(i);
  for (size_t b0 = 0; b0 < todo.size(); b0 += maxb) {
    const int P = (int)std::min<size_t>(maxb, todo.size() - b0);
    std::vector<int> pr(P), pp(P);
    for (int i = 0; i < P; ++i) {
      pr[i] = pairs[2 * todo[b0 + i]];
      pp[i] = pairs[2 * todo[b0 + i] + 1];
      if (pr[i] < 0 || pr[i] >= R || pp[i] < 0 || pp[i] >= V) throw CudaError(ETTK_ERR_ARG, "pair index out of range");
    }
    const bool use_half = N >= 32 && !from_tomo;
    {
      HostScope hs_p(this, "stage_particle_spectra");
      lr_filter_particles(pp, use_half);  // device work queued ahead of the SO(3) stage
      if (use_half) half_particles(pp);   // the child's host set-up while the device works
    }
    std::vector<PairPlan> plans;
    std::vector<PQ> q1, q2;
    if (use_half && p.fast_coarse_so3) {
      // the SO(3) search of the child on the half grid at B/2 (its particles are the batch's crops, slot order)
      HostScope hs_so3(this, "stage_so3");
      CK(cudaStreamWaitEvent(half->st, dec_ev, 0));
      std::vector<int> pc(P);
      for (int i = 0; i < P; ++i) pc[i] = lr_slot[pp[i]];
      half->prof = prof;
      half->so3_queues(P, pr, pc, plans, q1, q2);
      merge_child_profile();
    } else {
      HostScope hs_so3(this, "stage_so3");
      so3_queues(P, pr, pp, plans, q1, q2);
    }
    std::vector<EvalReq> req;
    std::vector<int> owner;
    {
      HostScope hs_c(this, "stage_coarse_ccf");
      for (int i = 0; i < P; ++i)
        for (int q = 0; q < 2; ++q) {
          PQ &Q = q == 0 ? q1[i] : q2[i];
          const int take = q == 0 ? peaks : std::max(1, peaks / 3);
          for (int t = 0; t < take && !Q.empty() && Q.top().v[3] != FLT_MAX; ++t) {
            const Cand c = Q.top();
            Q.pop();
            req.push_back({pr[i], pp[i], euler_candidate(c.v[0], c.v[1], c.v[2])});
            owner.push_back(i);
          }
        }
    }
    if (use_half) {
      HostScope hs_c(this, "stage_coarse_ccf");
      std::vector<EvalReq> finals;
      half_screen(pr, pp, req, owner, finals);
      req.swap(finals);
    } else {
      HostScope hs_c(this, "stage_coarse_ccf");
      std::vector<EvalRes> res;
      eval_batch(req, res);
      std::vector<int> best(P, -1);
      for (size_t k = 0; k < req.size(); ++k) {
        const int i = owner[k];
        if (!transform_valid(p, res[k].t)) continue;
        if (best[i] < 0 || res[k].dist < res[best[i]].dist) best[i] = (int)k;
      }
      std::vector<EvalReq> fb;
      std::vector<int> fbi;
      for (int i = 0; i < P; ++i)
        if (best[i] < 0) {  // no valid candidate: the reference's fallback rotation (0, 0, 0) (execute 786-804)
          fb.push_back({pr[i], pp[i], Mat4::eye()});
          fbi.push_back(i);
        }
      std::vector<EvalRes> fres;
      if (!fb.empty()) eval_batch(fb, fres);
      std::vector<EvalReq> finals(P);
      for (int i = 0; i < P; ++i) finals[i] = {pr[i], pp[i], best[i] >= 0 ? res[best[i]].t : Mat4::eye()};
      for (size_t k = 0; k < fb.size(); ++k) finals[fbi[k]].t = fres[k].t;
      req.swap(finals);
    }
    std::vector<LRState> sts(P);
    {
      HostScope hs_r(this, "stage_local_refine");
      lr_setup(req);
      lr_run(P, iterations);
      read_back(sts.data(), lr_state.p, P * sizeof(LRState));
      check_status();
    }
    std::vector<EvalReq> fin(P);
    for (int i = 0; i < P; ++i) fin[i] = {pr[i], pp[i], pose_from_index(partg[pp[i]], N, sts[i].base)};
    std::vector<float> ovl;
    if (cols > 18) ovl = wedge_overlaps(fin);
    for (int i = 0; i < P; ++i) {
      const int row = todo[b0 + i];
      auto at = [&](int col, int k) -> float & { return D[((long)row * cols + col) * ncand + k]; };
      for (int k = 1; k < ncand; ++k) at(0, k) = FLT_MAX;
      int off = 1;
      at(0, 0) = (float)(1.0 - sts[i].rho);
      if (cols > 17) at(1, 0) = 1.0f, off = 2;
      if (cols > 18) at(2, 0) = ovl[i], off = 3;
      for (int m = 0; m < 16; ++m) at(m + off, 0) = (float)fin[i].t.e[m];
    }
  }
}

// The fast form's objective and gradient at T_i perturbed by theta_i, with zm built at T_i (checks only).
void ettk_ctx::refined_objective(int npairs, const int *pairs, const double *poses, const double *theta, double *rho,
                                 double *grad) {
  std::vector<EvalReq> req(npairs);
  for (int i = 0; i < npairs; ++i) {
    req[i].ref = pairs[2 * i];
    req[i].part = pairs[2 * i + 1];
    if (req[i].ref < 0 || req[i].ref >= R || req[i].part < 0 || req[i].part >= V)
      throw CudaError(ETTK_ERR_ARG, "pair index out of range");
    memcpy(req[i].t.e, poses + 16 * i, 16 * sizeof(double));
  }
  {
    std::vector<int> parts(npairs);
    for (int i = 0; i < npairs; ++i) parts[i] = req[i].part;
    lr_filter_particles(parts);
  }
  lr_setup(req);
  std::vector<LRState> sts(npairs);
  read_back(sts.data(), lr_state.p, npairs * sizeof(LRState));
  std::vector<float> maps(npairs * 12);
  for (int i = 0; i < npairs; ++i) {
    double m[12];
    lr_perturb(sts[i].base, (double)N, theta + 6 * i, m);
    for (int k = 0; k < 12; ++k) maps[i * 12 + k] = (float)m[k];
  }
  CK(cudaMemcpyAsync(lr_maps.p, maps.data(), npairs * 12 * sizeof(float), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(lr_acc.p, 0, npairs * LR_NACC * sizeof(double), st));
  lr_eval(npairs);
  std::vector<double> acc(npairs * LR_NACC);
  read_back(acc.data(), lr_acc.p, acc.size() * sizeof(double));
  for (int i = 0; i < npairs; ++i) {
    double g[6];
    rho[i] = lr_objective(acc.data() + (long)i * LR_NACC, lr_C0, lr_C1, sts[i].czm, sts[i].czz, g);
    if (grad)
      for (int k = 0; k < 6; ++k) grad[6 * i + k] = g[k];
  }
}

// nbfFourierImageMetricCore::execute (inc/em/nbfFourierImageMetricCore.h:35-66) as getDistances runs it for
// typeOfMetric 2 (inc/em/nbfCorrelationImageMetric.h:1912-1976): per pair one executeFourierNewHalf at the identity
// transform of the particle (its own matrix is the alignment under test) with the given translation restriction;
// the transform keeps the found shift when isTransformValid accepts it, else stays the identity. The core metric
// has one candidate, so only slot 0 of each row is written (distance, scale 1, getWedgeOverlap, transform).
void ettk_ctx::score(int npairs, const int *pairs, float *D, int cols, int ncand, float restrict_translation) {
  HostScope hs_all(this, "host_score_wall");
  std::vector<int> todo;
  for (int i = 0; i < npairs; ++i)
    if (D[(long)i * cols * ncand] == -1) todo.push_back(i);
  if (todo.empty()) return;
  std::vector<EvalReq> req(todo.size());
  for (size_t k = 0; k < todo.size(); ++k) {
    const int r = pairs[2 * todo[k]], v = pairs[2 * todo[k] + 1];
    if (r < 0 || r >= R || v < 0 || v >= V) throw CudaError(ETTK_ERR_ARG, "pair index out of range");
    req[k] = {r, v, Mat4::eye()};
  }
  // the restriction in force for this call (the reference sets the metric's and restores it afterwards)
  struct WindowGuard {
    ettk_ctx *c;
    float keep;
    ~WindowGuard() {
      c->p.restrict_translation = keep;
      c->set_window(keep);
    }
  } guard{this, p.restrict_translation};
  if (restrict_translation >= 0) {
    p.restrict_translation = restrict_translation;
    set_window(restrict_translation);
  }
  std::vector<EvalRes> res;
  eval_batch(req, res);
  std::vector<EvalReq> fin(req.size());
  for (size_t k = 0; k < req.size(); ++k) fin[k] = {req[k].ref, req[k].part, transform_valid(p, res[k].t) ? res[k].t : Mat4::eye()};
  std::vector<float> ovl;
  if (cols > 18) ovl = wedge_overlaps(fin);
  for (size_t k = 0; k < req.size(); ++k) {
    auto at = [&](int col) -> float & { return D[((long)todo[k] * cols + col) * ncand]; };
    int off = 1;
    at(0) = res[k].dist;
    if (cols > 17) at(1) = 1.0f, off = 2;
    if (cols > 18) at(2) = ovl[k], off = 3;
    for (int m = 0; m < 16; ++m) at(m + off) = (float)fin[k].t.e[m];
  }
}

std::vector<float> ettk_ctx::wedge_overlaps(const std::vector<EvalReq> &req) {
  const long E = (long)req.size();
  std::vector<float> out(E, 1.0f);
  std::vector<WedgeVecs> wv;
  std::vector<int> ref, slot;
  for (long e = 0; e < E; ++e) {
    const VolumeGeom &g2 = partg[req[e].part];
    const bool eff1 = !refg[req[e].ref].full_wedge(), eff2 = !g2.full_wedge();
    if (!eff1 && !eff2) continue;  // getWedgeOverlap returns 1
    WedgeVecs w{};
    w.full = eff2 ? 0 : 1;
    if (eff2) wedge_vectors(g2, &req[e].t, w.v1, w.v2);
    wv.push_back(w);
    ref.push_back(req[e].ref);
    slot.push_back((int)e);
  }
  const long M = (long)wv.size();
  if (M == 0) return out;
  const int ACC = 8;
  w_wv.ensure(M);
  w_idx.ensure(M);
  w_fw.ensure(M * h3);
  w_ovl.ensure(M * ACC);
  CK(cudaMemcpyAsync(w_wv.p, wv.data(), M * sizeof(WedgeVecs), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_idx.p, ref.data(), M * sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(w_ovl.p, 0, M * ACC * sizeof(double), st));
  {
    Scope sc_w(this, "wedge", 4.0 * M * h3);
    switch (N) {
      case 16: wedge_t<16>(M, w_ovl.p, ACC); break;
      case 32: wedge_t<32>(M, w_ovl.p, ACC); break;
      case 64: wedge_t<64>(M, w_ovl.p, ACC); break;
      case 128: wedge_t<128>(M, w_ovl.p, ACC); break;
      default: throw CudaError(ETTK_ERR_ARG, "unsupported volume size");
    }
  }
  std::vector<double> acc(M * ACC);
  read_back(acc.data(), w_ovl.p, M * ACC * sizeof(double));
  for (long m = 0; m < M; ++m) out[slot[m]] = (float)(acc[m * ACC + 6] / sum_filter);
  return out;
}

void ettk_ctx::soft_diag(const float *F1, const float *F2, int scaled, float *C) {
  // one pair-like job on two user signals: reuse the SO(3) kernels with a single correlation
  w_sig.ensure(2 * nn);
  w_coef.ensure(2 * B * B);
  w_S.ensure(nso3);
  w_C.ensure(nso3);
  w_mm.ensure(2);
  w_w.ensure(2);
  w_jobs.ensure(1);
  w_sjobs.ensure(1);
  CK(cudaMemcpyAsync(w_sig.p, F1, nn * 4, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_sig.p + nn, F2, nn * 4, cudaMemcpyHostToDevice, st));
  SynthJob j{0, 1};
  ScaledJob sj{1, 0, 0};
  CK(cudaMemcpyAsync(w_jobs.p, &j, sizeof(j), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(w_sjobs.p, &sj, sizeof(sj), cudaMemcpyHostToDevice, st));
  size_t smem_sht = (n / 2 + (size_t)n * n) * sizeof(float2);
  switch (B) {
#define SO3D(BB)                                                                                          \
  case BB:                                                                                                \
    if (smem_sht > 48 * 1024)                                                                             \
      CK(cudaFuncSetAttribute(k_sht<BB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_sht));    \
    k_sht<BB><<<2, 256, smem_sht, st>>>(w_sig.p, lw.p, w_coef.p);                                         \
    post_launch();                                                                                        \
    CK(cudaMemsetAsync(w_S.p, 0, nso3 * sizeof(float2), st));                                            \
    synth<BB>(1);                                                                                         \
    fft_strided(2 * BB, w_S.p, LineMap{(long)n * n, n * n, (long)n * n * n, 1, (long)n * n}, -1);         \
    fft_strided(2 * BB, w_S.p, LineMap{(long)n * n, n, (long)n * n, 1, (long)n}, -1);                     \
    CK(cudaMemsetAsync(w_mm.p, 0, 2 * sizeof(unsigned long long), st));                                   \
    k_so3_real<BB><<<dim3(n, 1), 256, 0, st>>>(w_S.p, w_C.p, w_mm.p);                                    \
    post_launch();                                                                                        \
    if (scaled) {                                                                                         \
      k_so3_weights<BB><<<dim3(1, 2), 256, so3_weights_smem<BB>(), st>>>(w_sjobs.p, w_mm.p, w_coef.p, w_sig.p, dtab.p, doff.p, \
                                                    plm.p, sinth.p, w_w.p);                               \
      post_launch();                                                                                      \
    }                                                                                                     \
    break;
    SO3D(8)
    SO3D(16)
    SO3D(32)
    SO3D(64)
#undef SO3D
    default:
      throw CudaError(ETTK_ERR_ARG, "unsupported bandwidth");
  }
  std::vector<float> hc(nso3);
  CK(cudaMemcpyAsync(hc.data(), w_C.p, nso3 * 4, cudaMemcpyDeviceToHost, st));
  unsigned long long mm[2];
  double w[2];
  CK(cudaMemcpyAsync(mm, w_mm.p, sizeof(mm), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(w, w_w.p, sizeof(w), cudaMemcpyDeviceToHost, st));
  sync();
  check_status();
  if (scaled) {
    auto unpack = [](unsigned long long k, bool isMin) {
      uint32_t u = (uint32_t)(k >> 32);
      if (isMin) u = ~u;
      return __builtin_bit_cast(float, (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
    };
    float mn = unpack(mm[0], true), mx = unpack(mm[1], false);
    float sc = (float)((w[1] - w[0]) / ((double)mx - (double)mn));
    for (long i = 0; i < nso3; ++i) hc[i] = (hc[i] - mn) * sc + (float)w[0];
  }
  memcpy(C, hc.data(), nso3 * 4);
}

// ------------------------------------------------------------------------------------- C ABI

namespace {
int fail(ettk_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}
bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

VolumeGeom to_geom(const ettk_volume_meta &m) {
  VolumeGeom g;
  g.lwedge = m.lwedge;
  g.uwedge = m.uwedge;
  for (int i = 0; i < 3; ++i) {
    g.normal[i] = m.normal[i];
    g.position[i] = m.position[i];
  }
  g.cut_offset = m.cut_offset;
  memcpy(g.matrix, m.matrix, sizeof(g.matrix));
  return g;
}

// conditionSphericalWindow (inc/em/nbfProjectionRotationMetric3D.h:1322-1345: Gaussian std 2, radius factor 1
// on VTK dims (2B, 2B, 1), x = polar index) and the 0.95 gate of the window's use (487-490).
void condition_spherical_host(std::vector<float> &W, int B, int &use) {
  const int n = 2 * B;
  std::vector<float> t((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) t[i + (size_t)n * j] = W[(size_t)i * n + j];
  int dims[3] = {n, n, 1};
  gaussian_smooth(t, dims, 2.0, 1.0);
  double s = 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      W[(size_t)i * n + j] = t[i + (size_t)n * j];
      s += W[(size_t)i * n + j];
    }
  use = s <= (double)(.95f * (float)(n * n));
}

// nbfWedge3D::getSphericalImage + conditionSphericalWindow on the host (double arithmetic as the reference)
void spherical_wedge_host(const VolumeGeom &g, int B, std::vector<float> &W, int &use) {
  int n = 2 * B;
  W.assign((size_t)n * n, 1.0f);
  if (!g.full_wedge()) {
    double v1[3], v2[3];
    wedge_vectors(g, nullptr, v1, v2);
    float phiK = (float)(M_PI / (n - 1)), thetaK = (float)(2.0 * M_PI / (n - 1));
    std::vector<float> cj(n), sj(n), si(n), ci(n);
    for (int k = 0; k < n; ++k) {
      cj[k] = cosf(k * thetaK);
      sj[k] = sinf(k * thetaK);
      si[k] = sinf(k * phiK);
      ci[k] = cosf(k * phiK);
    }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double a = v1[0] * cj[j] * si[i] + v1[1] * sj[j] * si[i] + v1[2] * ci[i];
        double b = v2[0] * cj[j] * si[i] + v2[1] * sj[j] * si[i] + v2[2] * ci[i];
        W[(size_t)i * n + j] = (a * b <= 0.0) ? 1.0f : 0.0f;
      }
  }
  condition_spherical_host(W, B, use);
}

// nbfWedge3D::getImageHalf for the reference (no transform), host side
void wedge_half_host(const VolumeGeom &g, int N, std::vector<float> &W) {
  int H = N / 2 + 1;
  W.assign((size_t)N * N * H, 1.0f);
  if (g.full_wedge()) return;
  double v1[3], v2[3];
  wedge_vectors(g, nullptr, v1, v2);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < H; ++k) {
        double a = v1[0] * (i - N / 2) + v1[1] * (j - N / 2) + v1[2] * (k - (H - 1));
        double b = v2[0] * (i - N / 2) + v2[1] * (j - N / 2) + v2[2] * (k - (H - 1));
        W[((size_t)i * N + j) * H + k] = (a * b <= 0.0) ? 1.0f : 0.0f;
      }
  std::vector<float> t(W.size());
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < H; ++k) t[i + (size_t)N * (j + (size_t)N * k)] = W[((size_t)i * N + j) * H + k];
  int dims[3] = {N, N, H};
  gaussian_smooth(t, dims, 2.0, 0.5);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < H; ++k) W[((size_t)i * N + j) * H + k] = t[i + (size_t)N * (j + (size_t)N * k)];
}

// No NaN or infinity in v[0..n) (exponent field all ones), checked in 1 MiB slices on the host threads.
bool finite_volume(const float *v, long n) {
  const long slice = 1L << 18;
  const int ns = (int)((n + slice - 1) / slice);
  std::atomic<int> bad{0};
  parallel_for(ns, [&](int t) {
    const uint32_t *u = reinterpret_cast<const uint32_t *>(v) + (long)t * slice;
    const long m = std::min(slice, n - (long)t * slice);
    uint32_t any = 0;
    for (long i = 0; i < m; ++i) any |= (uint32_t)((u[i] & 0x7f800000u) == 0x7f800000u);
    if (any) bad.store(1);
  });
  return bad.load() == 0;
}

template <class F>
int guarded(ettk_ctx *c, F fn) {
  try {
    if (c) CK(cudaSetDevice(c->device));
    fn();
    return ETTK_OK;
  } catch (const CudaError &e) {
    return fail(c, e.code, e.what());
  } catch (const std::bad_alloc &) {
    return fail(c, ETTK_ERR_OOM, "host allocation failed");
  } catch (const std::exception &e) {
    return fail(c, ETTK_ERR_CUDA, e.what());
  }
}
}  // namespace

extern "C" {

int ettk_gpu_create(int device, const ettk_params *params, ettk_ctx **out) {
  if (!params || !out) return ETTK_ERR_ARG;
  *out = nullptr;
  const ettk_params &p = *params;
  if (!pow2(p.N) || p.N < 16 || p.N > 128 || !(p.B == 8 || p.B == 16 || p.B == 32 || p.B == 64) ||
      p.candidate_peaks < 1 || p.number_of_candidates < 1 || p.wigner_precision < 0 ||
      p.wigner_precision > WIG_FP64 || p.fast_coarse_so3 < 0 || p.fast_coarse_so3 > 2)
    return ETTK_ERR_ARG;
  ettk_ctx *c = new (std::nothrow) ettk_ctx;
  if (!c) return ETTK_ERR_OOM;
  c->device = device;
  c->p = p;
  int rc = guarded(c, [&] {
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
    c->init_tables();
  });
  if (rc != ETTK_OK) {
    ettk_gpu_destroy(c);
    return rc;
  }
  *out = c;
  return ETTK_OK;
}

int ettk_gpu_destroy(ettk_ctx *c) {
  if (!c) return ETTK_OK;
  if (c->half) ettk_gpu_destroy(c->half);
  c->half = nullptr;
  cudaSetDevice(c->device);
  if (c->dec_ev) cudaEventDestroy(c->dec_ev);
  if (c->st) cudaStreamSynchronize(c->st);
  DevBuf<float> *fb[] = {&c->mask, &c->refmask, &c->maskfft, &c->filter, &c->lw, &c->plm, &c->dtab, &c->sinth, &c->refvol,
                         &c->W1half, &c->Pp1, &c->W1sph, &c->partvol, &c->W2sph, &c->Pp2, &c->w_r, &c->w_v,
                         &c->w_fw, &c->w_tmp, &c->w_C, &c->w_sig, &c->w_norm,
                         &c->w_norm2, &c->sp_v, &c->sp_M, &c->sp_padc};
  for (auto b : fb) b->release();
  DevBuf<float2> *cb[] = {&c->Fm1, &c->FI1, &c->w_cA, &c->w_cB, &c->w_cC, &c->w_p1, &c->w_p2, &c->w_coef, &c->w_S, &c->sp_F};
  for (auto b : cb) b->release();
  c->w_acc.release();
  c->w_w.release();
  c->sp_acc.release();
  c->w_peak.release();
  c->w_mm.release();
  c->doff.release();
  c->dtab64.release();
  c->tomo.release();
  c->w_ridx.release();
  c->w_faces.release();
  c->w_mpairs.release();
  c->rf_fw.release();
  c->rf_y1.release();
  c->rf_a.release();
  c->rf_pair.release();
  c->rf_acc.release();
  c->dirs.release();
  c->w_items.release();
  c->w_wv.release();
  c->w_idx.release();
  c->w_idx2.release();
  c->w_cnt.release();
  c->w_pair_ref.release();
  c->w_pair_pp2.release();
  c->w_pair_part.release();
  c->w_i1.release();
  c->w_lists.release();
  c->w_out.release();
  c->w_sd.release();
  c->w_jobs.release();
  c->w_sjobs.release();
  c->repr_idx_dev.release();
  c->lr_in.release();
  c->nf_flag.release();
  c->real_idx_dev.release();
  c->w_plans.release();
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return ETTK_OK;
}

int ettk_gpu_set_references(ettk_ctx *c, int R, const float *vols, const ettk_volume_meta *meta) {
  if (!c || R <= 0 || !vols || !meta) return fail(c, ETTK_ERR_ARG, "invalid reference arguments");
  if (!finite_volume(vols, (long)R * c->n3)) return fail(c, ETTK_ERR_NAN, "non-finite reference volume");
  c->half_refs_ok = false;
  return guarded(c, [&] {
    long n3 = c->n3, h3 = c->h3;
    c->R = R;
    c->refg.resize(R);
    c->useW1.resize(R);
    c->refvol.ensure(R * n3);
    c->h2d(c->refvol.p, vols, R * n3 * 4);
    c->upload_maps(c->refvol.p, R, c->tm_ref, c->tm_ref_ok);
    std::vector<ResliceItem> items(R);
    std::vector<float> w1h((size_t)R * h3), w1s((size_t)R * c->nn);
    for (int r = 0; r < R; ++r) {
      c->refg[r] = to_geom(meta[r]);
      double m12[12];
      reslice_index(c->refg[r], c->N, nullptr, m12);
      items[r].vol = c->refvol.p + (long)r * n3;
      items[r].tmap = c->ref_map(r);
      items[r].dims[0] = items[r].dims[1] = items[r].dims[2] = c->N;
      set_map(items[r], m12);
      std::vector<float> w;
      wedge_half_host(c->refg[r], c->N, w);
      std::vector<float> wk = to_kz_major(w.data(), c->N);
      std::copy(wk.begin(), wk.end(), w1h.begin() + (size_t)r * h3);
      int use = 0;
      spherical_wedge_host(c->refg[r], c->B, w, use);
      std::copy(w.begin(), w.end(), w1s.begin() + (size_t)r * c->nn);
      c->useW1[r] = use;
    }
    c->W1half.ensure(R * h3);
    c->W1sph.ensure(R * c->nn);
    c->h2d(c->W1half.p, w1h.data(), R * h3 * 4);
    c->h2d(c->W1sph.p, w1s.data(), R * c->nn * 4);
    // I1 = getImage(reference): reslice, mean of valid voxels removed; F_I1 = R2C(I1 maskfft shift)
    c->w_v.ensure(R * n3);
    c->w_acc.ensure(R * 2);
    c->w_items.ensure(R);
    CK(cudaMemcpyAsync(c->w_items.p, items.data(), R * sizeof(ResliceItem), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemsetAsync(c->w_acc.p, 0, R * 2 * sizeof(double), c->st));
    c->reslice(c->w_items.p, c->w_v.p, c->w_acc.p, 2, nullptr, R);
    c->FI1.ensure(R * h3);
    PreParticle pre{c->w_v.p, c->maskfft.p, c->w_acc.p, 2, c->N};
    c->r2c_z(c->N, pre, c->FI1.p, (long)R * c->N * c->N);
    c->xy_kxy(c->N, c->FI1.p, R, -1);
    if (c->p.mutual_correlation) {  // executeHalf's F / |F|^(1/2), ahead of every filter the I1 branch applies
      k_mutual_scale<<<nblocks<int>((long)R * h3, 256, 8192), 256, 0, c->st>>>(c->FI1.p, (long)R * h3);
      c->post_launch();
    }
    // Pp1 = cartesianToSpherical(I1)
    c->Pp1.ensure(R * c->nn);
    c->spherical_projection(items, c->Pp1.p);
    c->sync();
    c->check_status();
  });
}

static void particle_tables(ettk_ctx *c, const ettk_volume_meta *meta);

static int set_particles_impl(ettk_ctx *c, int V, const float *vols, const ettk_volume_meta *meta, bool device) {
  if (!c || V <= 0 || !vols || !meta) return fail(c, ETTK_ERR_ARG, "invalid particle arguments");
  return guarded(c, [&] {
    long n3 = c->n3;
    c->V = V;
    c->partg.resize(V);
    c->useW2.resize(V);
    c->pp2_ready.assign(V, 0);
    c->from_tomo = false;
    if (device) {
      c->partptr = vols;
    } else {
      c->partvol.ensure(V * n3);
      CK(cudaMemcpyAsync(c->partvol.p, vols, V * n3 * 4, cudaMemcpyHostToDevice, c->st));
      c->partptr = c->partvol.p;
    }
    c->check_finite(c->partptr, (long)V * n3);  // on the device, behind the upload
    particle_tables(c, meta);                   // host work overlaps the volume upload
    c->upload_maps(c->partptr, V, c->tm_part, c->tm_part_ok);
    c->sync();
    c->finite_or_throw("non-finite particle volume");
  });
}

// Pose geometry, spherical wedges and projection slots of the particle set (both particle sources).
static void particle_tables(ettk_ctx *c, const ettk_volume_meta *meta) {
  const int V = c->V;
  std::vector<float> w2s((size_t)V * c->nn);
  parallel_for(V, [&](int v) {
    c->partg[v] = to_geom(meta[v]);
    std::vector<float> w;
    int use = 0;
    spherical_wedge_host(c->partg[v], c->B, w, use);
    std::copy(w.begin(), w.end(), w2s.begin() + (size_t)v * c->nn);
    c->useW2[v] = use;
  });
  c->W2sph.ensure(V * c->nn);
  CK(cudaMemcpyAsync(c->W2sph.p, w2s.data(), V * c->nn * 4, cudaMemcpyHostToDevice, c->st));
  c->Pp2.ensure(V * c->nn);
}

int ettk_gpu_set_particles_tomogram(ettk_ctx *c, int nx, int ny, int nz, const float *tomogram, int V,
                                    const ettk_volume_meta *meta) {
  if (!c || nx < 1 || ny < 1 || nz < 1 || !tomogram || V <= 0 || !meta)
    return fail(c, ETTK_ERR_ARG, "invalid tomogram arguments");
  const long nt = (long)nx * ny * nz;
  return guarded(c, [&] {
    c->V = V;
    c->partg.resize(V);
    c->useW2.resize(V);
    c->pp2_ready.assign(V, 0);
    c->tomo.ensure(nt);
    CK(cudaMemcpyAsync(c->tomo.p, tomogram, nt * 4, cudaMemcpyHostToDevice, c->st));
    c->check_finite(c->tomo.p, nt);
    c->tomo_dims[0] = nx;
    c->tomo_dims[1] = ny;
    c->tomo_dims[2] = nz;
    c->from_tomo = true;
    c->partptr = c->tomo.p;
    c->upload_maps(c->tomo.p, 1, c->tm_part, c->tm_part_ok, c->tomo_dims);
    particle_tables(c, meta);
    c->sync();
    c->finite_or_throw("non-finite tomogram");
  });
}

int ettk_gpu_set_particles(ettk_ctx *c, int V, const float *vols, const ettk_volume_meta *meta) {
  return set_particles_impl(c, V, vols, meta, false);
}
int ettk_gpu_set_particles_device(ettk_ctx *c, int V, const float *d_vols, const ettk_volume_meta *meta) {
  return set_particles_impl(c, V, d_vols, meta, true);
}

int ettk_gpu_align_pairs(ettk_ctx *c, int npairs, const int *pairs, float *D, int cols, int ncand) {
  if (!c || npairs < 0 || (npairs && (!pairs || !D)) || cols < 17 || ncand < 1)
    return fail(c, ETTK_ERR_ARG, "invalid align arguments");
  if (c->R == 0 || c->V == 0) return fail(c, ETTK_ERR_STATE, "references and particles must be set first");
  return guarded(c, [&] { c->align(npairs, pairs, D, cols, ncand); });
}

int ettk_gpu_score_pairs(ettk_ctx *c, int npairs, const int *pairs, float *D, int cols, int ncand,
                         float restrict_translation) {
  if (!c || npairs < 0 || (npairs && (!pairs || !D)) || cols < 17 || ncand < 1 || !(restrict_translation == restrict_translation))
    return fail(c, ETTK_ERR_ARG, "invalid score arguments");
  if (c->R == 0 || c->V == 0) return fail(c, ETTK_ERR_STATE, "references and particles must be set first");
  return guarded(c, [&] { c->score(npairs, pairs, D, cols, ncand, restrict_translation); });
}

int ettk_gpu_align_pairs_refined(ettk_ctx *c, int npairs, const int *pairs, float *D, int cols, int ncand,
                                 int iterations, int peaks) {
  if (!c || npairs < 0 || (npairs && (!pairs || !D)) || cols < 17 || ncand < 1 || iterations < 0 || peaks < 0 ||
      iterations > 1000 || peaks > 64)
    return fail(c, ETTK_ERR_ARG, "invalid arguments");
  if (!c->R || !c->V) return fail(c, ETTK_ERR_STATE, "references or particles not set");
  return guarded(c, [&] {
    c->align_refined(npairs, pairs, D, cols, ncand, iterations, peaks ? peaks : c->p.candidate_peaks);
  });
}

int ettk_gpu_refined_objective(ettk_ctx *c, int npairs, const int *pairs, const double *poses, const double *theta,
                               double *rho, double *grad) {
  if (!c || npairs <= 0 || !pairs || !poses || !theta || !rho) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  if (!c->R || !c->V) return fail(c, ETTK_ERR_STATE, "references or particles not set");
  return guarded(c, [&] { c->refined_objective(npairs, pairs, poses, theta, rho, grad); });
}

// ---- launch-shape tuning ---------------------------------------------------------------------

static const int kTuneSynth[] = {16, 32, 64, 128}, kTuneChunk[] = {1024, 2048, 4096, 8192}, kTuneOver[] = {1, 2},
                 kTuneSample[] = {64, 128, 256};
static bool tune_in(int v, const int *list, int n) { return std::find(list, list + n, v) != list + n; }
static bool tuning_valid(const ettk_tuning &t) {
  return tune_in(t.synth_job_blocks, kTuneSynth, 4) && tune_in(t.eval_chunk, kTuneChunk, 4) &&
         tune_in(t.zpass_oversub, kTuneOver, 2) && tune_in(t.sample_block, kTuneSample, 3);
}

int ettk_gpu_get_tuning(ettk_ctx *c, ettk_tuning *t) {
  if (!c || !t) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  *t = c->tune;
  return ETTK_OK;
}

int ettk_gpu_set_tuning(ettk_ctx *c, const ettk_tuning *t) {
  if (!c || !t || !tuning_valid(*t)) return fail(c, ETTK_ERR_ARG, "invalid launch shapes");
  c->tune = *t;
  return ETTK_OK;
}

int ettk_gpu_autotune(ettk_ctx *c, int npairs, const int *pairs, int repeats, ettk_tuning *best, char *report,
                      int report_size) {
  if (!c || npairs < 1 || !pairs || repeats < 1 || repeats > 20 || (report && report_size < 1))
    return fail(c, ETTK_ERR_ARG, "invalid arguments");
  if (!c->R || !c->V) return fail(c, ETTK_ERR_STATE, "references or particles not set");
  for (int i = 0; i < npairs; ++i)
    if (pairs[2 * i] < 0 || pairs[2 * i] >= c->R || pairs[2 * i + 1] < 0 || pairs[2 * i + 1] >= c->V)
      return fail(c, ETTK_ERR_ARG, "pair index out of range");
  return guarded(c, [&] {
    const ettk_tuning start = c->tune;
    std::string js = "[";
    std::vector<float> ref;
    // median wall time of `repeats` synchronous alignments of the sample under t (after one warm-up), and whether
    // the rows equal the first trial's bit for bit
    auto trial = [&](const ettk_tuning &t, bool &same) -> double {
      c->tune = t;
      std::vector<double> ms;
      std::vector<float> D;
      for (int r = 0; r <= repeats; ++r) {
        std::fill(c->pp2_ready.begin(), c->pp2_ready.end(), 0);  // time the spherical projections too
        D.assign((size_t)npairs * 17, -1.f);
        const auto t0 = std::chrono::steady_clock::now();
        c->align(npairs, pairs, D.data(), 17, 1);
        const auto t1 = std::chrono::steady_clock::now();
        if (r > 0) ms.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
      }
      std::sort(ms.begin(), ms.end());
      if (ref.empty()) ref = D;
      same = memcmp(D.data(), ref.data(), D.size() * sizeof(float)) == 0;
      const double med = ms[ms.size() / 2];
      char buf[256];
      snprintf(buf, sizeof buf,
               "%s{\"synth_job_blocks\": %d, \"eval_chunk\": %d, \"zpass_oversub\": %d, \"sample_block\": %d, "
               "\"ms\": %.4f, \"identical\": %s}",
               js.size() > 1 ? ", " : "", t.synth_job_blocks, t.eval_chunk, t.zpass_oversub, t.sample_block, med,
               same ? "true" : "false");
      js += buf;
      return med;
    };
    ettk_tuning cur = tuning_valid(start) ? start : ettk_tuning{64, 4096, 1, 128};
    bool same = true;
    double cur_ms = trial(cur, same);
    auto search = [&](int ettk_tuning::*field, const int *vals, int nv) {
      const int timed = cur.*field;  // the field's value in the best shapes so far, already timed
      for (int k = 0; k < nv; ++k) {
        if (vals[k] == timed) continue;
        ettk_tuning t = cur;
        t.*field = vals[k];
        bool ok = true;
        const double ms = trial(t, ok);
        if (ok && ms < cur_ms) {
          cur = t;
          cur_ms = ms;
        }
      }
    };
    search(&ettk_tuning::synth_job_blocks, kTuneSynth, 4);
    search(&ettk_tuning::eval_chunk, kTuneChunk, 4);
    search(&ettk_tuning::zpass_oversub, kTuneOver, 2);
    search(&ettk_tuning::sample_block, kTuneSample, 3);
    c->tune = cur;
    if (best) *best = cur;
    js += "]";
    if (report) {
      const size_t n = std::min<size_t>(js.size(), (size_t)report_size - 1);
      memcpy(report, js.data(), n);
      report[n] = 0;
    }
  });
}

int ettk_gpu_wait_probe(ettk_ctx *c, int max_iter) {
  if (!c || max_iter < 1 || max_iter > (1 << 24)) return fail(c, ETTK_ERR_ARG, "invalid wait probe arguments");
  return guarded(c, [&] {
    k_wait_probe<<<1, 32, 0, c->st>>>(max_iter, c->status.p);
    c->post_launch();
    c->sync();
    c->check_status();
  });
}

int ettk_gpu_ccf(ettk_ctx *c, int r, int p, double *t, float *dist) {
  if (!c || !t || !dist) return fail(c, ETTK_ERR_ARG, "invalid ccf arguments");
  if (r < 0 || r >= c->R || p < 0 || p >= c->V) return fail(c, ETTK_ERR_STATE, "volume index out of range");
  return guarded(c, [&] {
    EvalReq q;
    q.ref = r;
    q.part = p;
    memcpy(q.t.e, t, sizeof(q.t.e));
    std::vector<EvalRes> res;
    c->eval_batch({q}, res);
    *dist = res[0].dist;
    memcpy(t, res[0].t.e, sizeof(res[0].t.e));
  });
}

int ettk_gpu_refine_pairs(ettk_ctx *c, int npairs, const int *pairs, float *D, int cols, int ncand, int iterations) {
  if (!c || npairs < 0 || (npairs && (!pairs || !D)) || cols < 17 || ncand < 1 || iterations < 0)
    return fail(c, ETTK_ERR_ARG, "invalid refine arguments");
  return guarded(c, [&] {
    const int maxb = 256;
    for (int b0 = 0; b0 < npairs; b0 += maxb) {
      const int P = std::min(maxb, npairs - b0);
      std::vector<EvalReq> req(P);
      for (int i = 0; i < P; ++i) {
        const int r = pairs[2 * (b0 + i)], q = pairs[2 * (b0 + i) + 1];
        if (r < 0 || r >= c->R || q < 0 || q >= c->V) throw CudaError(ETTK_ERR_ARG, "pair index out of range");
        const float *row = D + (long)(b0 + i) * cols * ncand;
        if (row[0] == -1.f) throw CudaError(ETTK_ERR_STATE, "refine needs aligned rows (distance -1 found)");
        req[i].ref = r;
        req[i].part = q;
        for (int k = 0; k < 16; ++k) req[i].t.e[k] = row[(1 + k) * ncand];
      }
      std::vector<Mat4> out;
      std::vector<double> rho;
      c->refine(req, iterations, out, rho);
      for (int i = 0; i < P; ++i) {
        float *row = D + (long)(b0 + i) * cols * ncand;
        row[0] = (float)(1.0 - rho[i]);
        for (int k = 0; k < 16; ++k) row[(1 + k) * ncand] = (float)out[i].e[k];
      }
    }
  });
}

int ettk_gpu_classify(ettk_ctx *c, int iterations, int *labels, float *refs_out, float *dist_out) {
  if (!c || iterations < 1 || !labels) return fail(c, ETTK_ERR_ARG, "invalid classify arguments");
  if (c->R < 1 || c->V < 1) return fail(c, ETTK_ERR_STATE, "set references and particles first");
  const int R = c->R, V = c->V, N = c->N;
  const long n3 = c->n3;
  const int cols = 17;
  std::vector<int> pairs(2L * R * V);
  for (int v = 0; v < V; ++v)
    for (int r = 0; r < R; ++r) {
      pairs[2L * (v * R + r)] = r;
      pairs[2L * (v * R + r) + 1] = v;
    }
  std::vector<float> D((size_t)R * V * cols), avg((size_t)R * n3);
  std::vector<ettk_volume_meta> meta(R);
  for (auto &m : meta) {  // class averages: no wedge, identity pose, centred
    m = ettk_volume_meta{};
    m.lwedge = -90.f;
    m.uwedge = 90.f;
    for (int i = 0; i < 16; ++i) m.matrix[i] = (i % 5 == 0) ? 1.0 : 0.0;
    for (int i = 0; i < 3; ++i) m.position[i] = 0.5f * (float)N;
  }
  for (int it = 0; it < iterations; ++it) {
    // 1. every particle against every class reference (getDistances, src/MPI_Classification.cpp:1087)
    std::fill(D.begin(), D.end(), -1.f);
    int rc = ettk_gpu_align_pairs(c, R * V, pairs.data(), D.data(), cols, 1);
    if (rc != ETTK_OK) return rc;
    // 2. each particle to its closest class (ties: the lower class index)
    for (int v = 0; v < V; ++v) {
      int best = 0;
      for (int r = 1; r < R; ++r)
        if (D[(size_t)(v * R + r) * cols] < D[(size_t)(v * R + best) * cols]) best = r;
      labels[v] = best;
      if (dist_out) dist_out[v] = D[(size_t)(v * R + best) * cols];
    }
    // 3. wedge-weighted average of each class under its members' alignments (getImageMPI + getImage)
    std::vector<std::vector<float>> sph(R);
    for (int r = 0; r < R; ++r) {
      std::vector<int> mem;
      std::vector<float> w;
      std::vector<double> mats;
      for (int v = 0; v < V; ++v)
        if (labels[v] == r) {
          mem.push_back(v);
          w.push_back(1.f);
          const float *row = &D[(size_t)(v * R + r) * cols];
          for (int k = 0; k < 16; ++k) mats.push_back(row[1 + k]);
        }
      if (mem.empty()) {  // an empty class keeps its reference
        rc = guarded(c, [&] {
          c->d2h(avg.data() + (size_t)r * n3, c->refvol.p + (size_t)r * n3, n3 * 4);
        });
        if (rc != ETTK_OK) return rc;
        continue;
      }
      rc = ettk_gpu_average(c, (int)mem.size(), mem.data(), w.data(), mats.data(), avg.data() + (size_t)r * n3);
      if (rc != ETTK_OK) return rc;
      if (c->p.wedge_compensation) {  // the class's accumulated spherical wedge (doMra, nbfLoopClustering.h:1270-1278)
        sph[r].resize((size_t)4 * c->B * c->B);
        rc = ettk_gpu_average_spherical_wedge(c, (int)mem.size(), mem.data(), w.data(), mats.data(), nullptr,
                                              sph[r].data());
        if (rc != ETTK_OK) return rc;
      }
    }
    // 4. the averages become the references of the next pass, carrying their classes' spherical wedges
    rc = ettk_gpu_set_references(c, R, avg.data(), meta.data());
    if (rc != ETTK_OK) return rc;
    for (int r = 0; r < R; ++r)
      if (!sph[r].empty()) {
        rc = ettk_gpu_set_reference_spherical_wedge(c, r, sph[r].data());
        if (rc != ETTK_OK) return rc;
      }
  }
  if (refs_out) memcpy(refs_out, avg.data(), (size_t)R * n3 * sizeof(float));
  return ETTK_OK;
}

int ettk_gpu_refine_objective(ettk_ctx *c, int npairs, const int *pairs, const double *poses, const double *theta,
                              double *rho, double *grad) {
  if (!c || npairs <= 0 || !pairs || !poses || !theta || !rho) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  return guarded(c, [&] {
    std::vector<EvalReq> req(npairs);
    std::vector<std::array<double, 12>> maps(npairs);
    std::vector<int> self(npairs);
    for (int i = 0; i < npairs; ++i) {
      const int r = pairs[2 * i], q = pairs[2 * i + 1];
      if (r < 0 || r >= c->R || q < 0 || q >= c->V) throw CudaError(ETTK_ERR_ARG, "pair index out of range");
      req[i].ref = r;
      req[i].part = q;
      memcpy(req[i].t.e, poses + 16 * (long)i, sizeof(req[i].t.e));
      double m0[12];
      reslice_index(c->partg[q], c->N, &req[i].t, m0);
      perturb_index(m0, c->N, theta + 6 * (long)i, theta + 6 * (long)i + 3, maps[i].data());
      self[i] = i;
    }
    c->refine_setup(req);
    std::vector<double> r, g;
    c->refine_eval(maps, self, grad != nullptr, r, g);
    for (int i = 0; i < npairs; ++i) rho[i] = r[i];
    if (grad) memcpy(grad, g.data(), 6 * (size_t)npairs * sizeof(double));
  });
}

int ettk_gpu_spherical_projection(ettk_ctx *c, int r, int p, float *Pp) {
  if (!c || !Pp) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  return guarded(c, [&] {
    ResliceItem it;
    double m12[12];
    if (p >= 0) {
      if (p >= c->V) throw CudaError(ETTK_ERR_STATE, "particle index out of range");
      it.vol = c->part_vol(p);
      it.tmap = c->part_map(p);
      reslice_index(c->partg[p], c->N, nullptr, m12);
    } else {
      if (r < 0 || r >= c->R) throw CudaError(ETTK_ERR_STATE, "reference index out of range");
      it.vol = c->refvol.p + (long)r * c->n3;
      it.tmap = c->ref_map(r);
      reslice_index(c->refg[r], c->N, nullptr, m12);
    }
    it.dims[0] = it.dims[1] = it.dims[2] = c->N;
    if (p >= 0) c->part_dims(it.dims);
    set_map(it, m12);
    c->w_sig.ensure(c->nn);
    c->spherical_projection({it}, c->w_sig.p);
    CK(cudaMemcpyAsync(Pp, c->w_sig.p, c->nn * 4, cudaMemcpyDeviceToHost, c->st));
    c->sync();
    c->check_status();
  });
}

int ettk_gpu_soft(ettk_ctx *c, const float *F1, const float *F2, int scaled, float *C) {
  if (!c || !F1 || !F2 || !C) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  return guarded(c, [&] { c->soft_diag(F1, F2, scaled, C); });
}

int ettk_gpu_average(ettk_ctx *c, int M, const int *particles, const float *weights, const double *matrices,
                     float *avg) {
  if (!c || M < 0 || (M && (!particles || !weights || !matrices)) || !avg) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  if (c->V == 0) return fail(c, ETTK_ERR_STATE, "particles must be set first");
  return guarded(c, [&] { c->average(M, particles, weights, matrices, avg); });
}

// [x][y][kz] (the reference's half-spectrum arrays) <-> kz-major [kz][x][y]
static void half_to_kz_major(const double *src, int N, double *dst) {
  const int H = N / 2 + 1;
  for (int x = 0; x < N; ++x)
    for (int y = 0; y < N; ++y)
      for (int k = 0; k < H; ++k) dst[((size_t)k * N + x) * N + y] = src[((size_t)x * N + y) * H + k];
}
static void kz_major_to_half(const double *src, int N, double *dst) {
  const int H = N / 2 + 1;
  for (int x = 0; x < N; ++x)
    for (int y = 0; y < N; ++y)
      for (int k = 0; k < H; ++k) dst[((size_t)x * N + y) * H + k] = src[((size_t)k * N + x) * N + y];
}

int ettk_gpu_average_partial(ettk_ctx *c, int M, const int *particles, const float *weights, const double *matrices,
                             double *re, double *im, double *acc) {
  if (!c || M < 0 || (M && (!particles || !weights || !matrices)) || !re || !im || !acc)
    return fail(c, ETTK_ERR_ARG, "invalid average arguments");
  if (c->V == 0) return fail(c, ETTK_ERR_STATE, "particles must be set first");
  return guarded(c, [&] {
    c->average_accumulate(M, particles, weights, matrices);
    std::vector<double> h(3 * c->h3);
    c->d2h(h.data(), c->w_w.p, h.size() * sizeof(double));
    kz_major_to_half(h.data(), c->N, acc);
    kz_major_to_half(h.data() + c->h3, c->N, re);
    kz_major_to_half(h.data() + 2 * c->h3, c->N, im);
  });
}

int ettk_gpu_average_finish(ettk_ctx *c, const double *re, const double *im, const double *acc, float *avg) {
  if (!c || !re || !im || !acc || !avg) return fail(c, ETTK_ERR_ARG, "invalid average arguments");
  return guarded(c, [&] {
    std::vector<double> h(3 * c->h3);
    half_to_kz_major(acc, c->N, h.data());
    half_to_kz_major(re, c->N, h.data() + c->h3);
    half_to_kz_major(im, c->N, h.data() + 2 * c->h3);
    c->w_w.ensure(3 * c->h3 + 1);
    c->h2d(c->w_w.p, h.data(), h.size() * sizeof(double));
    c->average_finish(avg);
  });
}

int ettk_gpu_variance(ettk_ctx *c, int M, const int *parts, const float *weights, const double *mats,
                      const float *avg, float *var) {
  if (!c || M <= 0 || !parts || !weights || !mats || !avg || !var) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  if (c->V <= 0) return fail(c, ETTK_ERR_STATE, "no particles");
  if (!finite_volume(avg, c->n3)) return fail(c, ETTK_ERR_NAN, "non-finite average");
  return guarded(c, [&] { c->variance(M, parts, weights, mats, avg, var); });
}

int ettk_gpu_symmetrize(ettk_ctx *c, const float *vol, int fold, float *out) {
  if (!c || !vol || !out || fold < 1 || fold > 360) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  if (!finite_volume(vol, c->n3)) return fail(c, ETTK_ERR_NAN, "non-finite volume");
  return guarded(c, [&] { c->symmetrize(vol, fold, out); });
}

int ettk_gpu_mean_images(ettk_ctx *c, const float *vol, int n, const double *transforms, float *out) {
  if (!c || !vol || !out || !transforms || n < 1 || n > 4096) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  if (!finite_volume(vol, c->n3)) return fail(c, ETTK_ERR_NAN, "non-finite volume");
  for (long k = 0; k < 16L * n; ++k)
    if (!std::isfinite(transforms[k])) return fail(c, ETTK_ERR_NAN, "non-finite transform");
  return guarded(c, [&] {
    std::vector<Mat4> ts(n);
    for (int i = 0; i < n; ++i) memcpy(ts[i].e, transforms + 16L * i, sizeof(ts[i].e));
    c->mean_images(vol, n, ts.data(), out);
  });
}

int ettk_gpu_representation_distances(ettk_ctx *c, int V, int K, int depth, const float *R, int overlap_normalized,
                                      float *D) {
  if (!c || V < 1 || K < 1 || (depth != 1 && depth != 3) || !R || !D) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  const long n = (long)V * K * depth;
  bool binary = depth == 3;
  for (long k = 0; k < n; ++k) {
    if (!std::isfinite(R[k])) return fail(c, ETTK_ERR_NAN, "non-finite representation");
    if (depth == 3 && k % 3 == 2 && R[k] != 0.f && R[k] != 1.f) binary = false;
  }
  return guarded(c, [&] {
    DevBuf<float> dR, dD;
    struct Release {  // the buffers are freed however the call ends
      DevBuf<float> &a, &b;
      ~Release() {
        a.release();
        b.release();
      }
    } release{dR, dD};
    dR.ensure(n);
    dD.ensure((long)V * V);
    CK(cudaMemcpyAsync(dR.p, R, n * sizeof(float), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemsetAsync(dD.p, 0, (size_t)V * V * sizeof(float), c->st));
    const int nb = (V + RD_T - 1) / RD_T;
    const unsigned tiles = (unsigned)((long)nb * (nb + 1) / 2);
    {
      ettk_ctx::Scope sc(c, "repr_dist", (double)n * 4 * nb);
      if (depth == 3 && binary)
        k_repr_dist<3, true><<<tiles, 256, 0, c->st>>>(dR.p, V, K, overlap_normalized, dD.p);
      else if (depth == 3)
        k_repr_dist<3, false><<<tiles, 256, 0, c->st>>>(dR.p, V, K, overlap_normalized, dD.p);
      else
        k_repr_dist<1, false><<<tiles, 256, 0, c->st>>>(dR.p, V, K, overlap_normalized, dD.p);
      c->post_launch();
    }
    CK(cudaMemcpyAsync(D, dD.p, (size_t)V * V * sizeof(float), cudaMemcpyDeviceToHost, c->st));
    c->sync();
    c->check_status();
  });
}

int ettk_gpu_representations(ettk_ctx *c, int M, const int *particles, int fold, int *K, float *R) {
  if (!c || !K || fold < 1 || fold > 360) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  if (R && (M < 1 || !particles)) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  return guarded(c, [&] {
    *K = (int)c->representation_band().size();
    if (!R) return;
    if (c->V < 1) throw CudaError(ETTK_ERR_STATE, "set particles first");
    for (int i = 0; i < M; ++i)
      if (particles[i] < 0 || particles[i] >= c->V) throw CudaError(ETTK_ERR_ARG, "particle index out of range");
    c->representations(M, particles, fold, R);
  });
}

// nbfImageFilter::buildMaskFromFile + softenMask (inc/em/nbfImageFilter.h:319-381, 474-494) on a mask volume of
// edge M (x fastest, as its MRC file holds it): centred into a zero N^3 box or cropped from its centre with the
// reference's integer offsets, binarised (> threshold), softened (Gaussian std sigma, radius factor 0.75 sigma,
// sigma = the filter's mask sigma); returned [x][y][z], z fastest (the Blitz order of the reference's arrays).
static std::vector<float> external_mask(int N, float sigma, int M, const float *mask, float threshold) {
  const long n3 = (long)N * N * N;
  std::vector<float> out(n3, 0.0f);
  auto at = [&](int x, int y, int z) { return mask[x + (long)M * (y + (long)M * z)]; };
  if (M == N) {
    for (int x = 0; x < N; ++x)
      for (int y = 0; y < N; ++y)
        for (int z = 0; z < N; ++z) out[((long)x * N + y) * N + z] = at(x, y, z);
  } else if ((int)((N - M) / 2.0) > 0) {  // smaller mask: centred into the box
    const int o = N / 2 - M / 2;
    for (int x = 0; x < M; ++x)
      for (int y = 0; y < M; ++y)
        for (int z = 0; z < M; ++z) out[((long)(o + x) * N + (o + y)) * N + (o + z)] = at(x, y, z);
  } else {  // larger mask: the centre of it
    const int o = M / 2 - N / 2;
    if (o < 0 || o + N > M) throw CudaError(ETTK_ERR_ARG, "mask edge does not fit the box");
    for (int x = 0; x < N; ++x)
      for (int y = 0; y < N; ++y)
        for (int z = 0; z < N; ++z) out[((long)x * N + y) * N + z] = at(o + x, o + y, o + z);
  }
  for (float &v : out) v = v > threshold ? 1.0f : 0.0f;
  if (sigma > 0) {
    std::vector<float> t(n3);  // VTK order (x fastest) for the smoothing
    for (int x = 0; x < N; ++x)
      for (int y = 0; y < N; ++y)
        for (int z = 0; z < N; ++z) t[x + (long)N * (y + (long)N * z)] = out[((long)x * N + y) * N + z];
    const int dims[3] = {N, N, N};
    gaussian_smooth(t, dims, (double)sigma, (double)sigma * .75);
    for (int x = 0; x < N; ++x)
      for (int y = 0; y < N; ++y)
        for (int z = 0; z < N; ++z) out[((long)x * N + y) * N + z] = t[x + (long)N * (y + (long)N * z)];
  }
  return out;
}

int ettk_gpu_set_reference_mask(ettk_ctx *c, int M, const float *mask, float threshold) {
  if (!c || M < 0 || M > 2048 || (M > 0 && !mask)) return fail(c, ETTK_ERR_ARG, "invalid mask arguments");
  return guarded(c, [&] {
    if (c->mask.p == nullptr) throw CudaError(ETTK_ERR_STATE, "context not initialised");
    std::vector<float> m1(c->n3);
    if (M == 0) c->d2h(m1.data(), c->mask.p, c->n3 * sizeof(float));  // back to the spherical mask
    else m1 = external_mask(c->N, c->p.mask_sigma, M, mask, threshold);
    c->apply_reference_mask(m1);
    c->refmask_external = M > 0;
  });
}

int ettk_gpu_get_reference_mask(ettk_ctx *c, float *out) {
  if (!c || !out) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  return guarded(c, [&] {
    if (c->refmask.p == nullptr) throw CudaError(ETTK_ERR_STATE, "context not initialised");
    const int N = c->N;
    std::vector<float> m1(c->n3);
    c->d2h(m1.data(), c->refmask.p, c->n3 * sizeof(float));
    for (int x = 0; x < N; ++x)
      for (int y = 0; y < N; ++y)
        for (int z = 0; z < N; ++z) out[x + (long)N * (y + (long)N * z)] = m1[((long)x * N + y) * N + z];
  });
}

int ettk_gpu_representations_real(ettk_ctx *c, int M, const int *particles, int fold, int bin_factor, int *K,
                                  float *R) {
  if (!c || !K || fold < 1 || fold > 360 || bin_factor < 1 || bin_factor > 64) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  if (R && (M < 1 || !particles)) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  return guarded(c, [&] {
    if (c->mask.p == nullptr) throw CudaError(ETTK_ERR_STATE, "context not initialised");
    *K = (int)c->representation_real_band(bin_factor).size();
    if (!R) return;
    if (c->V < 1) throw CudaError(ETTK_ERR_STATE, "set particles first");
    for (int i = 0; i < M; ++i)
      if (particles[i] < 0 || particles[i] >= c->V) throw CudaError(ETTK_ERR_ARG, "particle index out of range");
    c->representations_real(M, particles, fold, bin_factor, R);
  });
}

int ettk_gpu_average_spherical_wedge(ettk_ctx *c, int M, const int *particles, const float *weights,
                                     const double *matrices, float *count, float *wedge) {
  if (!c || M < 1 || !particles || !weights || !matrices || !wedge) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  if (c->V < 1) return fail(c, ETTK_ERR_STATE, "set particles first");
  return guarded(c, [&] { c->average_spherical_wedge(M, particles, weights, matrices, count, wedge); });
}

int ettk_gpu_set_reference_spherical_wedge(ettk_ctx *c, int r, const float *wedge) {
  if (!c || !wedge) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  if (r < 0 || r >= c->R) return fail(c, ETTK_ERR_ARG, "reference index out of range");
  const int n = 2 * c->B;
  for (long k = 0; k < (long)n * n; ++k)
    if (!std::isfinite(wedge[k])) return fail(c, ETTK_ERR_NAN, "non-finite wedge");
  return guarded(c, [&] {
    std::vector<float> w(wedge, wedge + (size_t)n * n);
    int use = 0;
    condition_spherical_host(w, c->B, use);
    c->sync();
    c->h2d(c->W1sph.p + (long)r * c->nn, w.data(), (size_t)n * n * sizeof(float));
    c->useW1[r] = use;
  });
}

int ettk_gpu_symmetrize_rotational(ettk_ctx *c, const float *vol, float *out) {
  if (!c || !vol || !out) return fail(c, ETTK_ERR_ARG, "invalid arguments");
  if (c->N < 4) return fail(c, ETTK_ERR_ARG, "volume too small for the cylindrical grid");
  if (!finite_volume(vol, c->n3)) return fail(c, ETTK_ERR_NAN, "non-finite volume");
  return guarded(c, [&] { c->symmetrize_rotational(vol, out); });
}

int ettk_gpu_outlier_cutoff(int R, int V, const float *D, int ld, float top_fraction, int rule, int *best,
                            float *dist, int *keep, float *cutoff) {
  if (R < 1 || V < 1 || !D || ld < 1 || rule < 0 || rule > 2 || !best || !dist || !keep) return ETTK_ERR_ARG;
  if (!(top_fraction == top_fraction)) return ETTK_ERR_NAN;
  for (long i = 0; i < (long)V * R; ++i)
    if (!std::isfinite(D[(size_t)i * ld])) return ETTK_ERR_NAN;
  // each volume's class of smallest distance, the first on ties (minIndex over the classes)
  for (int v = 0; v < V; ++v) {
    int b = 0;
    for (int r = 1; r < R; ++r)
      if (D[(size_t)(v * (long)R + r) * ld] < D[(size_t)(v * (long)R + b) * ld]) b = r;
    const float d = D[(size_t)(v * (long)R + b) * ld];
    best[v] = b;
    dist[v] = rule == 0 ? std::fabs(d) : d;
    keep[v] = 1;
  }
  if (!(top_fraction < 1)) {
    if (cutoff) *cutoff = std::numeric_limits<float>::infinity();
    return ETTK_OK;
  }
  std::vector<float> sorted(dist, dist + V);
  std::sort(sorted.begin(), sorted.end());
  // index = fraction * (n - 1) in float arithmetic, truncated, as the reference indexes its sorted vector
  long at = (long)(top_fraction * (float)(V - 1));
  at = std::max(0L, std::min<long>(at, V - 1));
  const float cut = sorted[at];
  for (int v = 0; v < V; ++v) keep[v] = rule == 1 ? (dist[v] <= cut) : (dist[v] < cut);
  if (cutoff) *cutoff = cut;
  return ETTK_OK;
}

int ettk_gpu_mra_assign(int R, int V, const float *S, int *labels) {
  if (R < 1 || V < 1 || !S || !labels) return ETTK_ERR_ARG;
  for (long k = 0; k < (long)V * R * R; ++k)
    if (!std::isfinite(S[k])) return ETTK_ERR_NAN;
  for (int v = 0; v < V; ++v) {
    int best = 0;
    float best_sum = 0.f;
    for (int r = 0; r < R; ++r) {
      // the partial sum over the references accumulates in double and is stored as float, as Blitz reduces
      double s = 0.0;
      for (int j = 0; j < R; ++j) s += (double)S[((size_t)v * R + r) * R + j];
      const float fs = (float)s;
      if (r == 0 || fs < best_sum) {
        best = r;
        best_sum = fs;
      }
    }
    labels[v] = best;
  }
  return ETTK_OK;
}

int ettk_gpu_soft_weights(int R, int V, const float *D, int ld, float *W, float *radii) {
  if (R < 1 || V < 1 || !D || ld < 1 || !W) return ETTK_ERR_ARG;
  const float decay = .025f;
  for (int r = 0; r < R; ++r) {
    float mx = -std::numeric_limits<float>::max();
    for (int v = 0; v < V; ++v) {
      const float d = D[(size_t)(v * (long)R + r) * ld];
      if (!std::isfinite(d)) return ETTK_ERR_NAN;
      mx = std::max(mx, d);
    }
    // radius: largest distance to the class plus decay * ln(0.01), in double, stored as float
    const float rad = (float)((double)mx + (double)decay * std::log(.01));
    if (radii) radii[r] = rad;
    for (int v = 0; v < V; ++v) {
      const float d = D[(size_t)(v * (long)R + r) * ld];
      const float e = std::exp((-(d - rad)) / decay);  // float exponent, as on the float distance array
      const float w = (float)((1 + 2.0 * e) / (1 + 1.0 * e) - 1.0);
      W[(size_t)r * V + v] = w > .01 ? w : 0.f;
    }
  }
  return ETTK_OK;
}

long long ettk_gpu_kernel_launches(ettk_ctx *c) { return c ? c->launches : 0; }

void *ettk_gpu_stream(ettk_ctx *c) { return c ? (void *)c->st : nullptr; }

int ettk_gpu_profile(ettk_ctx *c, int enable) {
  if (!c) return ETTK_ERR_ARG;
  return guarded(c, [&] {
    c->sync();
    c->prof = enable != 0;
    c->prof_agg.clear();
  });
}

int ettk_gpu_profile_read(ettk_ctx *c, int index, char *name, int name_size, long long *launches, double *total_ms,
                          double *bytes) {
  if (!c || index < 0) return ETTK_ERR_ARG;
  if (index >= (int)c->prof_agg.size()) return ETTK_ERR_ARG;
  auto it = c->prof_agg.begin();
  std::advance(it, index);
  if (name && name_size > 0) snprintf(name, name_size, "%s", it->first.c_str());
  if (launches) *launches = it->second.n;
  if (total_ms) *total_ms = it->second.ms;
  if (bytes) *bytes = it->second.bytes;
  return ETTK_OK;
}

int ettk_gpu_last_error(ettk_ctx *c, char *buf, int size) {
  if (!buf || size <= 0) return ETTK_ERR_ARG;
  const char *m = c ? c->err.c_str() : "no context";
  snprintf(buf, size, "%s", m);
  return ETTK_OK;
}

}  // extern "C"
