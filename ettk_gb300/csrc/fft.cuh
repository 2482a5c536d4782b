// Batched power-of-two FFTs in shared memory (FP32) for the alignment path.
//
// The 3-D transforms follow FFTW3's conventions, which the reference relies on
// (inc/em/nbfFourierFilter.h:269-358): unnormalised, forward = exp(-i...), the LAST
// (contiguous) axis is halved to n/2+1, and the complex-to-real transform does the
// complex inverse passes over the leading axes first and the half-complex-to-real pass
// along the last axis last, using only the real parts of its k=0 and k=n/2 terms.
//
// A 3-D R2C is: z-pass (two real lines packed in one complex FFT), then strided complex
// passes along y and x. Each CTA keeps LINES lines of length N in shared memory, loads
// them coalesced (across lines for strided axes, along the line for the contiguous one),
// runs log2(N) radix-2 butterfly stages and stores them back.
#pragma once
#include "common.cuh"

namespace ettk {

template <int N>
struct Log2 {
  static const int value = 1 + Log2<N / 2>::value;
};
template <>
struct Log2<1> {
  static const int value = 0;
};

template <int N>
ETTK_DEV int bitrev(int k) {
  return __brev((unsigned)k) >> (32 - Log2<N>::value);
}

// Fill tw[k] = exp(-2 pi i k / N), k < N/2.
template <int N>
ETTK_DEV void load_twiddles(float2 *tw) {
  for (int k = threadIdx.x; k < N / 2; k += blockDim.x) {
    float s, c;
    sincospif(-2.0f * (float)k / (float)N, &s, &c);
    tw[k] = make_float2(c, s);
  }
}

// In-place radix-2 DIT FFT of `nlines` lines of length N stored contiguously in s
// (already in bit-reversed order). sign = -1 forward, +1 inverse.
template <int N>
ETTK_DEV void block_fft(float2 *s, int nlines, int sign, const float2 *tw) {
  const int nb = nlines * (N / 2);
#pragma unroll 1
  for (int half = 1; half < N; half <<= 1) {
    __syncthreads();
    const int tstep = N / (2 * half);
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
      int line = t / (N / 2), k = t - line * (N / 2);
      int grp = k / half, pos = k - grp * half;
      int i0 = line * N + grp * 2 * half + pos, i1 = i0 + half;
      float2 w = tw[pos * tstep];
      if (sign > 0) w.y = -w.y;
      float2 a = s[i0], b = cmul(s[i1], w);
      s[i0] = cadd(a, b);
      s[i1] = csub(a, b);
    }
  }
  __syncthreads();
}

// Lines for a strided pass: line l -> base = (l / n_inner) * outer_stride + (l % n_inner) * inner_stride,
// elements base + k * elem_stride.
struct LineMap {
  long n_lines;
  int n_inner;
  long outer_stride, inner_stride, elem_stride;
  ETTK_DEV long base(long l) const { return (l / n_inner) * outer_stride + (l % n_inner) * inner_stride; }
};

// Generic batched complex FFT along a strided axis. LINES lines per CTA.
// Optional per-element scale applied on load (used to fold 1/norm into an inverse pass).
template <int N, int LINES>
__global__ void k_fft_strided(float2 *__restrict__ data, LineMap map, int sign, const float *__restrict__ line_scale,
                              long scale_div) {
  extern __shared__ float2 smem[];
  float2 *tw = smem;
  float2 *s = smem + N / 2;
  load_twiddles<N>(tw);
  long l0 = (long)blockIdx.x * LINES;
  int nl = (int)min((long)LINES, map.n_lines - l0);
  if (map.elem_stride == 1) {
    for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
      int line = idx / N, k = idx - line * N;
      long g = map.base(l0 + line) + k;
      float2 v = data[g];
      if (line_scale) v = cscale(v, line_scale[(l0 + line) / scale_div]);
      s[line * N + bitrev<N>(k)] = v;
    }
  } else {
    for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
      int k = idx / nl, line = idx - k * nl;
      long g = map.base(l0 + line) + (long)k * map.elem_stride;
      float2 v = data[g];
      if (line_scale) v = cscale(v, line_scale[(l0 + line) / scale_div]);
      s[line * N + bitrev<N>(k)] = v;
    }
  }
  block_fft<N>(s, nl, sign, tw);
  if (map.elem_stride == 1) {
    for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
      int line = idx / N, k = idx - line * N;
      data[map.base(l0 + line) + k] = s[line * N + k];
    }
  } else {
    for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
      int k = idx / nl, line = idx - k * nl;
      data[map.base(l0 + line) + (long)k * map.elem_stride] = s[line * N + k];
    }
  }
}

// Real-to-complex pass along the contiguous axis. Pre(line, k) supplies the real input;
// two real lines share one complex FFT. out has n_lines lines of N/2+1 complex values.
// Pre may accumulate per-line reductions through its own members.
template <int N, int LINES, class Pre>
__global__ void k_r2c_z(Pre pre, float2 *__restrict__ out, long n_lines) {
  extern __shared__ float2 smem[];
  float2 *tw = smem;
  float2 *s = smem + N / 2;
  load_twiddles<N>(tw);
  const int H = N / 2 + 1;
  long l0 = (long)blockIdx.x * (2 * LINES);
  int nl = (int)min((long)(2 * LINES), n_lines - l0);  // real lines (even)
  int nc = (nl + 1) / 2;
  pre.begin();
  for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
    int line = idx / N, k = idx - line * N;
    float v = pre(l0 + line, k);
    int c = line >> 1;
    float *dst = reinterpret_cast<float *>(&s[c * N + bitrev<N>(k)]);
    dst[line & 1] = v;
  }
  if (nl & 1) {
    for (int k = threadIdx.x; k < N; k += blockDim.x)
      reinterpret_cast<float *>(&s[(nc - 1) * N + bitrev<N>(k)])[1] = 0.0f;
  }
  pre.end();
  block_fft<N>(s, nc, -1, tw);
  for (int idx = threadIdx.x; idx < nc * H; idx += blockDim.x) {
    int c = idx / H, k = idx - c * H;
    float2 zk = s[c * N + k];
    float2 zn = s[c * N + ((N - k) & (N - 1))];
    float2 x1 = make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
    float2 x2 = make_float2(0.5f * (zk.y + zn.y), -0.5f * (zk.x - zn.x));
    long la = l0 + 2 * c;
    out[la * H + k] = x1;
    if (2 * c + 1 < nl) out[(la + 1) * H + k] = x2;
  }
}

// Complex-to-real pass along the contiguous axis (FFTW hc2r semantics: the imaginary parts of
// the k=0 and k=N/2 inputs are ignored). Post(line, k, value) consumes the real output.
template <int N, int LINES, class Post>
__global__ void k_c2r_z(const float2 *__restrict__ in, Post post, long n_lines) {
  extern __shared__ float2 smem[];
  float2 *tw = smem;
  float2 *s = smem + N / 2;
  load_twiddles<N>(tw);
  const int H = N / 2 + 1;
  long l0 = (long)blockIdx.x * (2 * LINES);
  int nl = (int)min((long)(2 * LINES), n_lines - l0);
  int nc = (nl + 1) / 2;
  for (int idx = threadIdx.x; idx < nc * N; idx += blockDim.x) {
    int c = idx / N, k = idx - c * N;
    long la = l0 + 2 * c;
    bool has2 = (2 * c + 1) < nl;
    float2 a, b;
    if (k <= N / 2) {
      a = in[la * H + k];
      b = has2 ? in[(la + 1) * H + k] : make_float2(0.f, 0.f);
      if (k == 0 || k == N / 2) {
        a.y = 0.f;
        b.y = 0.f;
      }
    } else {
      a = cconj(in[la * H + (N - k)]);
      b = has2 ? cconj(in[(la + 1) * H + (N - k)]) : make_float2(0.f, 0.f);
    }
    // z = a + i b
    s[c * N + bitrev<N>(k)] = make_float2(a.x - b.y, a.y + b.x);
  }
  block_fft<N>(s, nc, +1, tw);
  post.begin();
  for (int idx = threadIdx.x; idx < nl * N; idx += blockDim.x) {
    int line = idx / N, k = idx - line * N;
    float2 z = s[(line >> 1) * N + k];
    post(l0 + line, k, (line & 1) ? z.y : z.x);
  }
  post.end();
}

}  // namespace ettk
