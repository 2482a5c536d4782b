// SO(3) correlation entry point that allocates no memory (ettk_gpu_soft_noalloc).
//
// Who needs it: callers that cannot or may not call cudaMalloc at the point where they score two
// spherical signals, for example a host application or framework that has already reserved the
// device memory for its own pool (a raw cudaMalloc would fail or fragment it), or code running
// under a strict per-process memory budget. Such callers pass device buffers for the inputs and
// the output; every intermediate lives in one fixed, file-scope device array of this library.
//
// Limits and behaviour:
//  - bandwidths B = 8 and B = 16 only (larger B is rejected with ETTK_ERR_ARG); the array is
//    kNoallocScratchBytes = 2 MiB and every GPU that loads the library keeps it until exit;
//  - set-up (the device address of the array and the B=8/B=16 Wigner and Legendre tables copied
//    into it) happens on the first call on each device, with that device current; make that first
//    call before starting any stream capture on the device;
//  - all calls share the array and it keeps the previous call's contents: buffers that must start
//    at zero are cleared by each call, and calls whose GPU work overlaps (other streams, other
//    threads) race on the array, so callers must serialise them;
//  - the array's address and tables are set up once per device ordinal for the life of the process:
//    do not use the entry point across a cudaDeviceReset (or a torn-down and recreated primary
//    context) of that device.
#include "../../include/ettk_gpu.h"
#include "kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>

using namespace ettk;

namespace {

constexpr size_t kNoallocScratchBytes = 2u << 20;
constexpr int kMaxB = 16;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Layout of the array (byte offsets, each 256-aligned).
struct Layout {
  size_t sig, coef, S, jobs, lw8, dtab8, doff8, lw16, dtab16, doff16, end;
};

constexpr size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr long dtab_floats(int B) { return (long)((4L * B * B * B - B) / 3) * 2 * B; }

constexpr Layout make_layout() {
  Layout L{};
  size_t o = 0;
  const int n = 2 * kMaxB;
  L.sig = o; o = al(o + 2 * (size_t)n * n * sizeof(float));
  L.coef = o; o = al(o + 2 * (size_t)kMaxB * kMaxB * sizeof(float2));
  L.S = o; o = al(o + (size_t)n * n * n * sizeof(float2));
  L.jobs = o; o = al(o + sizeof(SynthJob));
  L.lw8 = o; o = al(o + (size_t)8 * 8 * 16 * sizeof(float));
  L.dtab8 = o; o = al(o + (size_t)dtab_floats(8) * sizeof(float));
  L.doff8 = o; o = al(o + (size_t)15 * 15 * sizeof(int));
  L.lw16 = o; o = al(o + (size_t)16 * 16 * 32 * sizeof(float));
  L.dtab16 = o; o = al(o + (size_t)dtab_floats(16) * sizeof(float));
  L.doff16 = o; o = al(o + (size_t)31 * 31 * sizeof(int));
  L.end = o;
  return L;
}
constexpr Layout kLayout = make_layout();
static_assert(kLayout.end <= kNoallocScratchBytes, "no-alloc scratch layout exceeds the array");

std::mutex g_setup_mu;
unsigned char *g_dev_ptr[kMaxDevices] = {};

// Host staging for the tables, static (no heap allocation).
float h_lw[16 * 16 * 32];
float h_dtab[dtab_floats(16)];
int h_doff[31 * 31];
double h_P[16 * 16 * 32];
double h_col[16];

void small_d_col(int B, int m1, int m2, double beta, double *out) {
  double c = cos(beta / 2), s = sin(beta / 2), cb = cos(beta);
  int J = m1 < 0 ? -m1 : m1;
  int J2 = m2 < 0 ? -m2 : m2;
  if (J2 > J) J = J2;
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

// Fills h_lw / h_dtab / h_doff for bandwidth B (same tables as the context-based path).
long build_tables(int B) {
  const int n = 2 * B;
  double th[32], wq[32];
  for (int j = 0; j < n; ++j) {
    th[j] = M_PI * (2.0 * j + 1.0) / (4.0 * B);
    double a = 0;
    for (int k = 0; k < B; ++k) a += sin((2.0 * k + 1.0) * th[j]) / (2.0 * k + 1.0);
    wq[j] = (2.0 / B) * sin(th[j]) * a;
  }
  for (int i = 0; i < B * B * n; ++i) h_P[i] = 0;
  for (int m = 0; m < B; ++m) {
    double cc = sqrt((2.0 * m + 1.0) / 2.0);
    for (int i = 1; i <= m; ++i) cc *= sqrt((2.0 * i - 1.0) / (2.0 * i));
    if (m % 2) cc = -cc;
    for (int j = 0; j < n; ++j) {
      double x = cos(th[j]), s = sin(th[j]);
      double pmm = cc * pow(s, m);
      h_P[(m * B + m) * n + j] = pmm;
      if (m + 1 < B) h_P[(m * B + m + 1) * n + j] = x * sqrt(2.0 * m + 3.0) * pmm;
      for (int l = m + 2; l < B; ++l) {
        double a = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
        double b = sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
        h_P[(m * B + l) * n + j] = a * (x * h_P[(m * B + l - 1) * n + j] - b * h_P[(m * B + l - 2) * n + j]);
      }
    }
  }
  double nrm = sqrt(2.0 * M_PI) / n;
  for (int i = 0; i < B * B * n; ++i) h_lw[i] = (float)(nrm * wq[i % n] * h_P[i]);
  int ncell = (2 * B - 1) * (2 * B - 1);
  long total = 0;
  for (int cell = 0; cell < ncell; ++cell) {
    int m1 = cell / (2 * B - 1) - (B - 1), m2 = cell % (2 * B - 1) - (B - 1);
    int l0 = std::max(std::abs(m1), std::abs(m2));
    h_doff[cell] = (int)total;
    for (int j = 0; j < n; ++j) {
      small_d_col(B, m1, m2, th[j], h_col);
      for (int l = l0; l < B; ++l) h_dtab[total + (long)(l - l0) * n + j] = (float)(sqrt((2.0 * l + 1.0) / 2.0) * h_col[l]);
    }
    total += (long)(B - l0) * n;
  }
  return total;
}

// Once per device, with the device current: device address of the array, tables copied in.
int setup_device(int dev, unsigned char **out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (g_dev_ptr[dev]) {
    *out = g_dev_ptr[dev];
    return ETTK_OK;
  }
  unsigned char *ptr = nullptr;
  if (cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return ETTK_ERR_CUDA;
  for (int B : {8, 16}) {
    long nd = build_tables(B);
    size_t off_lw = B == 8 ? kLayout.lw8 : kLayout.lw16;
    size_t off_dt = B == 8 ? kLayout.dtab8 : kLayout.dtab16;
    size_t off_do = B == 8 ? kLayout.doff8 : kLayout.doff16;
    int ncell = (2 * B - 1) * (2 * B - 1);
    if (cudaMemcpy(ptr + off_lw, h_lw, sizeof(float) * B * B * 2 * B, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(ptr + off_dt, h_dtab, sizeof(float) * nd, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(ptr + off_do, h_doff, sizeof(int) * ncell, cudaMemcpyHostToDevice) != cudaSuccess)
      return ETTK_ERR_CUDA;
  }
  static const SynthJob job{0, 1};
  if (cudaMemcpy(ptr + kLayout.jobs, &job, sizeof(job), cudaMemcpyHostToDevice) != cudaSuccess) return ETTK_ERR_CUDA;
  // A pageable host-to-device cudaMemcpy may return before its DMA lands, and a caller's non-blocking stream
  // is not ordered after the legacy stream: wait for the tables before any call may use them.
  if (cudaDeviceSynchronize() != cudaSuccess) return ETTK_ERR_CUDA;
  g_dev_ptr[dev] = ptr;
  *out = ptr;
  return ETTK_OK;
}

template <int B>
int run(unsigned char *base, const float *F1, const float *F2, float *C, cudaStream_t st) {
  constexpr int n = 2 * B;
  float *sig = (float *)(base + kLayout.sig);
  float2 *coef = (float2 *)(base + kLayout.coef);
  float2 *S = (float2 *)(base + kLayout.S);
  const SynthJob *jobs = (const SynthJob *)(base + kLayout.jobs);
  const float *lw = (const float *)(base + (B == 8 ? kLayout.lw8 : kLayout.lw16));
  const float *dtab = (const float *)(base + (B == 8 ? kLayout.dtab8 : kLayout.dtab16));
  const int *doff = (const int *)(base + (B == 8 ? kLayout.doff8 : kLayout.doff16));
  if (cudaMemcpyAsync(sig, F1, sizeof(float) * n * n, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(sig + n * n, F2, sizeof(float) * n * n, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return ETTK_ERR_CUDA;
  size_t smem_sht = (n / 2 + (size_t)n * n) * sizeof(float2);
  k_sht<B><<<2, 256, smem_sht, st>>>(sig, lw, coef);
  // the synthesis never writes the m = +-B (Nyquist) rows: clear what the previous call left there
  if (cudaMemsetAsync(S, 0, sizeof(float2) * n * n * n, st) != cudaSuccess) return ETTK_ERR_CUDA;
  k_so3_synth<B><<<(2 * B - 1) * (2 * B - 1), 256, 0, st>>>(coef, jobs, 1, dtab, doff, S);
  constexpr int L = 16;
  size_t sm = (n / 2 + (size_t)L * n) * sizeof(float2);
  // S is [m1][m2][beta]: transforms along m2 (lines (m1, beta)) then along m1 (lines (m2, beta))
  LineMap m2{(long)n * n, n, (long)n * n, 1, (long)n};
  LineMap m1{(long)n * n, n * n, (long)n * n * n, 1, (long)n * n};
  k_fft_strided<n, L><<<(int)((m2.n_lines + L - 1) / L), 256, sm, st>>>(S, m2, -1, nullptr, 1);
  k_fft_strided<n, L><<<(int)((m1.n_lines + L - 1) / L), 256, sm, st>>>(S, m1, -1, nullptr, 1);
  k_so3_real<B><<<dim3(n, 1), 256, 0, st>>>(S, C, nullptr);
  return cudaGetLastError() == cudaSuccess ? ETTK_OK : ETTK_ERR_CUDA;
}

}  // namespace

extern "C" int ettk_gpu_soft_noalloc(int B, const float *d_F1, const float *d_F2, float *d_C, void *stream) {
  if (!(B == 8 || B == 16) || !d_F1 || !d_F2 || !d_C) return ETTK_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return ETTK_ERR_CUDA;
  unsigned char *base = nullptr;
  int rc = setup_device(dev, &base);
  if (rc != ETTK_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  return B == 8 ? run<8>(base, d_F1, d_F2, d_C, st) : run<16>(base, d_F1, d_F2, d_C, st);
}
