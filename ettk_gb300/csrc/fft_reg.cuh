// Register-resident batched FFTs (four-step, N = A*B) for the alignment path.
//
// A line of N complex values x[n], n = B*j1 + j2, is transformed as
//   y[k1][j2] = W_N^(j2*k1) * sum_j1 x[B*j1 + j2] W_A^(j1*k1)        (A-point DFT in registers per j2)
//   X[k1 + A*k2] = sum_j2 y[k1][j2] W_B^(j2*k2)                         (B-point DFT in registers per k1)
// with one shared-memory exchange of y in between. Thread t of a CTA owns (line = t % LINES, lane
// = t / LINES) so that a warp touches the same element of 32 consecutive lines: global loads and
// stores of strided axes are coalesced across lines. Conventions as fft.cuh (FFTW: forward
// exp(-i...), unnormalised; the c2r pass uses only the real parts of the k=0 and k=N/2 inputs).
#pragma once
#include <type_traits>
#include "common.cuh"
#include "fft.cuh"

namespace ettk {

template <int N>
struct Split;
template <> struct Split<16> { static const int A = 4, B = 4; };
template <> struct Split<32> { static const int A = 8, B = 4; };
template <> struct Split<64> { static const int A = 8, B = 8; };
template <> struct Split<128> { static const int A = 16, B = 8; };
template <> struct Split<256> { static const int A = 16, B = 16; };

// cos/sin(2 pi k / 16), k < 16 (exact mathematical constants to float precision)
__device__ __constant__ float kC16[16] = {1.0f, 0.92387953f, 0.70710678f, 0.38268343f, 0.0f, -0.38268343f,
                                          -0.70710678f, -0.92387953f, -1.0f, -0.92387953f, -0.70710678f,
                                          -0.38268343f, 0.0f, 0.38268343f, 0.70710678f, 0.92387953f};
__device__ __constant__ float kS16[16] = {0.0f, 0.38268343f, 0.70710678f, 0.92387953f, 1.0f, 0.92387953f,
                                          0.70710678f, 0.38268343f, 0.0f, -0.38268343f, -0.70710678f,
                                          -0.92387953f, -1.0f, -0.92387953f, -0.70710678f, -0.38268343f};

template <int R>
struct Log2R;
template <> struct Log2R<2> { static const int v = 1; };
template <> struct Log2R<4> { static const int v = 2; };
template <> struct Log2R<8> { static const int v = 3; };
template <> struct Log2R<16> { static const int v = 4; };

template <int R>
ETTK_DEV constexpr int brev_c(int k) {
  int r = 0;
  for (int b = 0; b < Log2R<R>::v; ++b)
    if (k & (1 << b)) r |= 1 << (Log2R<R>::v - 1 - b);
  return r;
}

// In-register R-point DFT (natural order in and out), sign -1 forward, +1 inverse.
template <int R>
ETTK_DEV void dft_reg(float2 (&x)[R], int sign) {
  float2 y[R];
#pragma unroll
  for (int k = 0; k < R; ++k) y[brev_c<R>(k)] = x[k];
#pragma unroll
  for (int half = 1; half < R; half <<= 1) {
#pragma unroll
    for (int s = 0; s < R; s += 2 * half) {
#pragma unroll
      for (int p = 0; p < half; ++p) {
        const int idx = p * (16 / (2 * half));  // W_(2 half)^p = exp(-2 pi i p / (2 half)) on the 16-grid
        // forward: exp(-i a) = (cos a, -sin a); inverse: (cos a, +sin a)
        const float c = kC16[idx], sn = (sign < 0) ? -kS16[idx] : kS16[idx];
        float2 a = y[s + p], b = y[s + p + half];
        float2 bw = make_float2(b.x * c - b.y * sn, b.x * sn + b.y * c);
        y[s + p] = make_float2(a.x + bw.x, a.y + bw.y);
        y[s + p + half] = make_float2(a.x - bw.x, a.y - bw.y);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < R; ++k) x[k] = y[k];
}

// Twiddle exp(sign * 2 pi i m / N) from the per-CTA table tw (forward values).
template <int N>
ETTK_DEV float2 twid(const float2 *tw, int m, int sign) {
  float2 w = tw[m & (N - 1)];
  if (sign > 0) w.y = -w.y;
  return w;
}

template <int N>
ETTK_DEV void load_full_twiddles(float2 *tw) {
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    float s, c;
    sincospif(-2.0f * (float)k / (float)N, &s, &c);
    tw[k] = make_float2(c, s);
  }
}

// Core: thread (line, lane) with lane < B holds x[B*j1 + lane] (j1 < A) in `v`; after the call the
// thread with lane < A holds X[lane + A*k2] (k2 < B) in `o`. ex is the CTA exchange buffer: row
// r = k1*B + j2 of line `line` at r*P + (r/B)*Q + line. Adjacent lines in a warp (the line-major thread map)
// take P = LINES+1, Q = 0; adjacent lanes (CONTIG) take P = 17*LINES/16, Q = LINES/16, which keeps both the
// lane-strided writes (rows k1*B + lane) and reads (rows lane*B + j2) of a half-warp on distinct 8-byte bank
// pairs (a search over P, Q of the 64-bit half-warp conflict count gives these as minimal).
template <int N>
struct MaxAB {
  static const int v = (Split<N>::A > Split<N>::B) ? Split<N>::A : Split<N>::B;
};
// Thread -> (line, lane). CONTIG (contiguous lines): lanes of one line are adjacent threads so that
// element loads along the line coalesce; otherwise adjacent threads are adjacent lines.
template <int N, int LINES, bool CONTIG>
ETTK_DEV void thread_map(int &line, int &lane) {
  if (CONTIG) {
    line = threadIdx.x / MaxAB<N>::v;
    lane = threadIdx.x % MaxAB<N>::v;
  } else {
    line = threadIdx.x % LINES;
    lane = threadIdx.x / LINES;
  }
}
template <int LINES, bool CONTIG>
struct ExPitch {
  static constexpr int P = CONTIG ? LINES + LINES / 16 : LINES + 1, Q = CONTIG ? LINES / 16 : 0;
};
// float2 elements of the exchange buffer: the four-step layout, and the [A*B][LINES+1] spectra the r2c
// passes stage in the same buffer afterwards
template <int N, int LINES, bool CONTIG>
__host__ __device__ constexpr int ex_size() {
  constexpr int A = Split<N>::A, B = Split<N>::B;
  constexpr int fs = A * B * ExPitch<LINES, CONTIG>::P + A * ExPitch<LINES, CONTIG>::Q;
  return fs > A * B * (LINES + 1) ? fs : A * B * (LINES + 1);
}
template <int N, int LINES, bool CONTIG>
ETTK_DEV void four_step(float2 (&v)[Split<N>::A], float2 (&o)[Split<N>::B], int line, int lane, int sign,
                        const float2 *tw, float2 *ex) {
  constexpr int A = Split<N>::A, B = Split<N>::B, P = ExPitch<LINES, CONTIG>::P, Q = ExPitch<LINES, CONTIG>::Q;
  if (lane < B) {
    dft_reg<A>(v, sign);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      float2 w = twid<N>(tw, lane * k1, sign);
      float2 t = v[k1];
      ex[(k1 * B + lane) * P + k1 * Q + line] = make_float2(t.x * w.x - t.y * w.y, t.x * w.y + t.y * w.x);
    }
  }
  __syncthreads();
  if (lane < A) {
#pragma unroll
    for (int j2 = 0; j2 < B; ++j2) o[j2] = ex[(lane * B + j2) * P + lane * Q + line];
    dft_reg<B>(o, sign);
  }
}

// Strided complex pass (same LineMap as k_fft_strided); optional per-item scale on load.
template <int N, int LINES, bool CONTIG>
__global__ void __launch_bounds__(LINES * ((Split<N>::A > Split<N>::B) ? Split<N>::A : Split<N>::B))
    k_fft_reg(float2 *__restrict__ data, LineMap map, int sign, const float *__restrict__ line_scale, long scale_div) {
  constexpr int A = Split<N>::A, B = Split<N>::B;
  __shared__ float2 tw[N];
  __shared__ float2 ex[ex_size<N, LINES, CONTIG>()];
  load_full_twiddles<N>(tw);
  int line, lane;
  thread_map<N, LINES, CONTIG>(line, lane);
  const long l = (long)blockIdx.x * LINES + line;
  const bool ok = l < map.n_lines;
  const long base = ok ? map.base(l) : 0;
  float2 v[A], o[B];
  float sc = 1.f;
  if (ok && line_scale) sc = line_scale[l / scale_div];
  if (lane < B) {
#pragma unroll
    for (int j1 = 0; j1 < A; ++j1) {
      float2 t = ok ? data[base + (long)(B * j1 + lane) * map.elem_stride] : make_float2(0.f, 0.f);
      v[j1] = make_float2(t.x * sc, t.y * sc);
    }
  }
  __syncthreads();
  four_step<N, LINES, CONTIG>(v, o, line, lane, sign, tw, ex);
  if (lane < A && ok) {
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) data[base + (long)(lane + A * k2) * map.elem_stride] = o[k2];
  }
}

// Input functors that can tell a line r[z] = c (-1)^(x+y+z) over the whole line (the constant padding of
// the spherical projection) declare kPadLines and pad_line(line, c, sign(x+y)).
template <class T, class = void>
struct has_pad_lines : std::false_type {};
template <class T>
struct has_pad_lines<T, std::void_t<decltype(T::kPadLines)>> : std::true_type {};
// Input functors that can restrict the pass to a subset of the lines declare kLineBase and map tile t to its first
// line with line_base(t, RL) when real_only is set (the grid then has real_tiles(lines, RL) tiles).
template <class T, class = void>
struct has_line_base : std::false_type {};
template <class T>
struct has_line_base<T, std::void_t<decltype(T::kLineBase)>> : std::true_type {};
template <class Pre>
ETTK_DEV long tile_first_line(const Pre &pre, long tile, int RL) {
  if constexpr (has_line_base<Pre>::value)
    if (pre.real_only) return pre.line_base(tile, RL);
  return tile * RL;
}

// Real-to-complex pass along the contiguous axis: two real lines (2c, 2c+1) packed into one complex
// FFT; Pre(line, k) supplies the real inputs (line = item*N*N + x*N + y). The half spectra are written
// kz-major, out[item][kz][x][y] (kz < N/2+1), through the exchange buffer so that consecutive threads
// store consecutive lines of one kz plane.
template <int N, int LINES, class Pre>
__global__ void __launch_bounds__(LINES * ((Split<N>::A > Split<N>::B) ? Split<N>::A : Split<N>::B))
    k_r2c_reg(Pre pre, float2 *__restrict__ out, long n_lines) {
  constexpr int A = Split<N>::A, B = Split<N>::B, H = N / 2 + 1, RL = 2 * LINES;
  constexpr int SP = ExPitch<LINES, true>::P;  // pitch of the staged spectra [k][line] (conflict-free rows)
  constexpr long NN = (long)N * N;
  __shared__ float2 tw[N];
  __shared__ float2 ex[ex_size<N, LINES, true>()];
  const long l_base = tile_first_line(pre, (long)blockIdx.x, RL);
  if constexpr (has_pad_lines<Pre>::value) {
    // a CTA whose lines are all padding lines writes their spectra directly: the N-point transform of
    // c (-1)^(x+y+z) is N c (-1)^(x+y) at k = N/2 and zero elsewhere
    float c0, s0;
    const long lt = l_base + (threadIdx.x % RL);
    if (__syncthreads_and(lt >= n_lines || pre.pad_line(lt, c0, s0))) {
      for (int idx = pre.nyquist_only ? (N / 2) * RL + threadIdx.x : threadIdx.x; idx < H * RL; idx += blockDim.x) {
        const int k = idx / RL, rl = idx - k * RL;
        if (pre.nyquist_only && k != N / 2) break;  // the consumer never reads the zero planes of padding lines
        const long l = l_base + rl;
        if (l < n_lines) {
          float2 v = make_float2(0.f, 0.f);
          float cc, sg;
          if (k == N / 2 && pre.pad_line(l, cc, sg)) v = make_float2((float)N * cc * sg, 0.f);
          out[(l / NN) * H * NN + (long)k * NN + (l % NN)] = v;
        }
      }
      return;
    }
  }
  load_full_twiddles<N>(tw);
  int line, lane;
  thread_map<N, LINES, true>(line, lane);
  const long l0 = l_base + 2 * line;  // complex line = real lines l0, l0 + 1
  const bool ok0 = l0 < n_lines, ok1 = l0 + 1 < n_lines;
  float2 v[A], o[B];
  pre.begin();
  if (lane < B) {
#pragma unroll
    for (int j1 = 0; j1 < A; ++j1) {
      int k = B * j1 + lane;
      float a = ok0 ? pre(l0, k) : 0.f;
      float b = ok1 ? pre(l0 + 1, k) : 0.f;
      v[j1] = make_float2(a, b);
    }
  }
  pre.end();
  __syncthreads();
  four_step<N, LINES, true>(v, o, line, lane, -1, tw, ex);
  __syncthreads();
  // full spectrum of the packed line back into the exchange buffer, [k][LINES]
  if (lane < A) {
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) ex[(lane + A * k2) * SP + line] = o[k2];
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < H * RL; idx += blockDim.x) {
    const int k = idx / RL, rl = idx - k * RL, cl = rl >> 1;
    const long l = l_base + rl;
    if (l < n_lines) {
      const float2 zk = ex[k * SP + cl];
      const float2 zn = ex[((N - k) & (N - 1)) * SP + cl];
      const float2 xv = (rl & 1) ? make_float2(0.5f * (zk.y + zn.y), -0.5f * (zk.x - zn.x))
                                 : make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
      out[(l / NN) * H * NN + (long)k * NN + (l % NN)] = xv;
    }
  }
}

// Input functors whose values come from one real N^3 array per item declare kStream, expose the array as
// stream_src() and an optional second operand shared by all items (N^3, same line layout) as stream_aux(),
// and compute the input from the two elements with apply(line, k, raw, aux) (aux = 1 without an operand);
// end_tile(first line) closes a tile of lines (one item).
template <class T, class = void>
struct has_stream : std::false_type {};
template <class T>
struct has_stream<T, std::void_t<decltype(T::kStream)>> : std::true_type {};

template <int N>
__host__ __device__ constexpr int stream_pitch() { return N + 4; }  // staged line pitch (floats): 16-byte rows, 8 banks apart per 2 lines

// Persistent form of k_r2c_reg for streamed inputs: each CTA walks tiles of 2*LINES contiguous real lines
// (t = blockIdx.x, + gridDim.x, ...); the next tile is copied into the other half of a double buffer
// (cp.async, 16-byte chunks) while the current one is transformed, so loads stay in flight through the
// transform and the stores. Tiles never straddle two items (2*LINES divides N*N).
template <int N, int LINES, class Pre, bool AUX>
__global__ void __launch_bounds__(LINES * ((Split<N>::A > Split<N>::B) ? Split<N>::A : Split<N>::B))
    k_r2c_stream(Pre pre, float2 *__restrict__ out, long n_lines) {
  constexpr int A = Split<N>::A, B = Split<N>::B, H = N / 2 + 1, RL = 2 * LINES, NP = stream_pitch<N>();
  constexpr int SP = ExPitch<LINES, true>::P;  // pitch of the staged spectra [k][line] (conflict-free rows)
  constexpr long NN = (long)N * N;
  static_assert(NN % RL == 0, "a tile must not straddle two items");
  __shared__ float2 tw[N];
  __shared__ float2 ex[ex_size<N, LINES, true>()];
  extern __shared__ __align__(16) float stg[];  // 2 x [RL][NP] (inputs), then with AUX 2 x [RL][NP] (operand)
  load_full_twiddles<N>(tw);
  int line, lane;
  thread_map<N, LINES, true>(line, lane);
  const long n_tiles = (n_lines + RL - 1) / RL;
  const float *src = pre.stream_src();
  const float *aux = pre.stream_aux();
  auto stage = [&](long t, int half) {
    const long lt = t * RL;
    const int nl = (int)min((long)RL, n_lines - lt);
    float *buf = stg + half * (RL * NP);
    for (int c = threadIdx.x; c < nl * (N / 4); c += blockDim.x) {
      const int r = c / (N / 4), q = c - r * (N / 4);
      cp_async16(buf + r * NP + 4 * q, src + (lt + r) * N + 4 * q);
    }
    if (AUX) {
      float *abuf = stg + (2 + half) * (RL * NP);
      const float *a0 = aux + (lt % NN) * N;  // the operand's rows of these lines (one item)
      for (int c = threadIdx.x; c < nl * (N / 4); c += blockDim.x) {
        const int r = c / (N / 4), q = c - r * (N / 4);
        cp_async16(abuf + r * NP + 4 * q, a0 + (long)r * N + 4 * q);
      }
    }
    cp_async_commit();
  };
  long t = blockIdx.x;
  if (t < n_tiles) stage(t, 0);
  for (int it = 0; t < n_tiles; ++it, t += gridDim.x) {
    const float *cur = stg + (it & 1) * (RL * NP);
    const float *acur = stg + (2 + (it & 1)) * (RL * NP);
    if (t + gridDim.x < n_tiles) {
      stage(t + gridDim.x, (it + 1) & 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const long l_base = t * RL;
    const long l0 = l_base + 2 * line;
    const bool ok0 = l0 < n_lines, ok1 = l0 + 1 < n_lines;
    float2 v[A], o[B];
    pre.begin();
    if (lane < B) {
#pragma unroll
      for (int j1 = 0; j1 < A; ++j1) {
        const int k = B * j1 + lane;
        const float a = ok0 ? pre.apply(l0, k, cur[(2 * line) * NP + k], AUX ? acur[(2 * line) * NP + k] : 1.f) : 0.f;
        const float b =
            ok1 ? pre.apply(l0 + 1, k, cur[(2 * line + 1) * NP + k], AUX ? acur[(2 * line + 1) * NP + k] : 1.f) : 0.f;
        v[j1] = make_float2(a, b);
      }
    }
    pre.end_tile(l_base);
    __syncthreads();
    four_step<N, LINES, true>(v, o, line, lane, -1, tw, ex);
    __syncthreads();
    if (lane < A) {
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) ex[(lane + A * k2) * SP + line] = o[k2];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < H * RL; idx += blockDim.x) {
      const int k = idx / RL, rl = idx - k * RL, cl = rl >> 1;
      const long l = l_base + rl;
      if (l < n_lines) {
        const float2 zk = ex[k * SP + cl];
        const float2 zn = ex[((N - k) & (N - 1)) * SP + cl];
        const float2 xv = (rl & 1) ? make_float2(0.5f * (zk.y + zn.y), -0.5f * (zk.x - zn.x))
                                   : make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
        out[(l / NN) * H * NN + (long)k * NN + (l % NN)] = xv;
      }
    }
    __syncthreads();  // ex and this half of the buffer are reused by the next tiles
  }
}
template <int N, bool AUX>
constexpr size_t r2c_stream_smem() {
  return (AUX ? 4 : 2) * (size_t)(2 * (256 / MaxAB<N>::v)) * stream_pitch<N>() * sizeof(float);
}

// Complex-to-real pass along the contiguous axis (two half spectra -> one packed complex inverse). The
// kz-major input is staged in shared memory [kz][line] with consecutive threads loading consecutive lines.
template <int N, int LINES, class Post>
__global__ void __launch_bounds__(LINES * ((Split<N>::A > Split<N>::B) ? Split<N>::A : Split<N>::B))
    k_c2r_reg(const float2 *__restrict__ in, Post post, long n_lines) {
  constexpr int A = Split<N>::A, B = Split<N>::B, H = N / 2 + 1, RL = 2 * LINES;
  constexpr long NN = (long)N * N;
  __shared__ float2 tw[N];
  __shared__ float2 ex[ex_size<N, LINES, true>()];
  // row pitch of the staged spectra: even (16-byte reads of the two packed lines) and 2 (mod 16) complex
  // values, so that the 8 k rows read by the lanes of one line cover all banks once
  constexpr int HP = RL + 2;
  __shared__ __align__(16) float2 hs[H * HP];
  load_full_twiddles<N>(tw);
  const long l_base = (long)blockIdx.x * RL;
  for (int idx = threadIdx.x; idx < H * RL; idx += blockDim.x) {
    const int k = idx / RL, rl = idx - k * RL;
    const long l = l_base + rl;
    hs[k * HP + rl] = (l < n_lines) ? in[(l / NN) * H * NN + (long)k * NN + (l % NN)] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  int line, lane;
  thread_map<N, LINES, true>(line, lane);
  const long c = (long)blockIdx.x * LINES + line;
  const long l0 = 2 * c;
  const bool ok0 = l0 < n_lines, ok1 = l0 + 1 < n_lines;
  float2 v[A], o[B];
  if (lane < B) {
#pragma unroll
    for (int j1 = 0; j1 < A; ++j1) {
      int k = B * j1 + lane;
      float2 a, b;
      const int kk = k <= N / 2 ? k : N - k;
      const float4 ab = *reinterpret_cast<const float4 *>(&hs[kk * HP + 2 * line]);
      a = make_float2(ab.x, ab.y);
      b = make_float2(ab.z, ab.w);
      if (k == 0 || k == N / 2) {
        a.y = 0.f;
        b.y = 0.f;
      } else if (k > N / 2) {
        a = cconj(a);
        b = cconj(b);
      }
      v[j1] = make_float2(a.x - b.y, a.y + b.x);
    }
  }
  __syncthreads();
  four_step<N, LINES, true>(v, o, line, lane, +1, tw, ex);
  post.begin();
  if (lane < A) {
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) {
      int k = lane + A * k2;
      if (ok0) post(l0, k, o[k2].x);
      if (ok1) post(l0 + 1, k, o[k2].y);
    }
  }
  post.end();
}

// Persistent form of k_c2r_reg: tiles of 2*LINES lines, the next tile's H kz rows (each one contiguous run of
// 2*LINES complex values of the kz-major input) copied by cp.async into the other half of a double buffer.
template <int N, int LINES, class Post>
__global__ void __launch_bounds__(LINES * ((Split<N>::A > Split<N>::B) ? Split<N>::A : Split<N>::B))
    k_c2r_stream(const float2 *__restrict__ in, Post post, long n_lines) {
  constexpr int A = Split<N>::A, B = Split<N>::B, H = N / 2 + 1, RL = 2 * LINES, HP = RL + 2;
  constexpr long NN = (long)N * N;
  static_assert(NN % RL == 0, "a tile must not straddle two items");
  __shared__ float2 tw[N];
  __shared__ float2 ex[ex_size<N, LINES, true>()];
  extern __shared__ __align__(16) float2 hsb[];  // 2 x [H][HP]
  load_full_twiddles<N>(tw);
  const long n_tiles = (n_lines + RL - 1) / RL;
  auto stage = [&](long t, float2 *buf) {
    const long lt = t * RL;
    const int nl = (int)min((long)RL, n_lines - lt);  // even: lines come in item planes of N*N
    const float2 *base = in + (lt / NN) * H * NN + (lt % NN);
    for (int c = threadIdx.x; c < H * (nl / 2); c += blockDim.x) {
      const int k = c / (nl / 2), q = c - k * (nl / 2);
      cp_async16(buf + k * HP + 2 * q, base + (long)k * NN + 2 * q);
    }
    cp_async_commit();
  };
  int line, lane;
  thread_map<N, LINES, true>(line, lane);
  long t = blockIdx.x;
  if (t < n_tiles) stage(t, hsb);
  for (int it = 0; t < n_tiles; ++it, t += gridDim.x) {
    const float2 *hs = hsb + (it & 1) * (H * HP);
    if (t + gridDim.x < n_tiles) {
      stage(t + gridDim.x, hsb + ((it + 1) & 1) * (H * HP));
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const long l0 = t * RL + 2 * line;
    const bool ok0 = l0 < n_lines, ok1 = l0 + 1 < n_lines;
    float2 v[A], o[B];
    if (lane < B) {
#pragma unroll
      for (int j1 = 0; j1 < A; ++j1) {
        int k = B * j1 + lane;
        float2 a, b;
        const int kk = k <= N / 2 ? k : N - k;
        const float4 ab = *reinterpret_cast<const float4 *>(&hs[kk * HP + 2 * line]);
        a = make_float2(ab.x, ab.y);
        b = make_float2(ab.z, ab.w);
        if (k == 0 || k == N / 2) {
          a.y = 0.f;
          b.y = 0.f;
        } else if (k > N / 2) {
          a = cconj(a);
          b = cconj(b);
        }
        v[j1] = make_float2(a.x - b.y, a.y + b.x);
      }
    }
    __syncthreads();
    four_step<N, LINES, true>(v, o, line, lane, +1, tw, ex);
    post.begin();
    if (lane < A) {
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) {
        int k = lane + A * k2;
        if (ok0) post(l0, k, o[k2].x);
        if (ok1) post(l0 + 1, k, o[k2].y);
      }
    }
    post.end();
    __syncthreads();  // ex and this half of the buffer are reused by the next tiles
  }
}
template <int N>
constexpr size_t c2r_stream_smem() { return 2 * (size_t)(N / 2 + 1) * (2 * (256 / MaxAB<N>::v) + 2) * sizeof(float2); }

// C2R and R2C of the same z lines in one pass: each tile of 2*LINES lines (kz-major half spectra, staged by
// cp.async into a double buffer as in k_c2r_stream) is transformed back to real lines, Mid maps every real
// value (and, with AUX, the element of the shared operand Mid::aux, staged beside the input), and the results
// are transformed forward and stored kz-major over the input (each tile reads all its input before it writes).
// The real lines pass through the exchange buffer between the two transforms: the intermediate real volume
// of two separate passes never reaches HBM. The arithmetic is that of k_c2r_stream followed by k_r2c_stream.
template <int N, int LINES>
__host__ __device__ constexpr int zz_ex_size() {
  return ex_size<N, LINES, true>() > (2 * LINES * stream_pitch<N>() + 1) / 2 ? ex_size<N, LINES, true>()
                                                                            : (2 * LINES * stream_pitch<N>() + 1) / 2;
}
template <int N, int LINES, class Mid, bool AUX>
__global__ void __launch_bounds__(LINES * ((Split<N>::A > Split<N>::B) ? Split<N>::A : Split<N>::B))
    k_c2r_r2c_stream(float2 *__restrict__ data, Mid mid, long n_lines) {
  constexpr int A = Split<N>::A, B = Split<N>::B, H = N / 2 + 1, RL = 2 * LINES, HP = RL + 2, NP = stream_pitch<N>();
  constexpr int SP = ExPitch<LINES, true>::P;
  constexpr long NN = (long)N * N;
  static_assert(NN % RL == 0, "a tile must not straddle two items");
  __shared__ float2 tw[N];
  __shared__ __align__(16) float2 ex[zz_ex_size<N, LINES>()];
  extern __shared__ __align__(16) float2 zbuf[];  // 2 x [H][HP] spectra, then with AUX 2 x [RL][NP] floats
  float *abuf = reinterpret_cast<float *>(zbuf + 2 * H * HP);
  float *rt = reinterpret_cast<float *>(ex);  // real lines [RL][NP] between the two transforms
  load_full_twiddles<N>(tw);
  const long n_tiles = (n_lines + RL - 1) / RL;
  const float *aux = mid.aux;
  auto stage = [&](long t, int half) {
    const long lt = t * RL;
    const int nl = (int)min((long)RL, n_lines - lt);  // even: lines come in item planes of N*N
    const float2 *base = data + (lt / NN) * H * NN + (lt % NN);
    float2 *buf = zbuf + half * (H * HP);
    for (int c = threadIdx.x; c < H * (nl / 2); c += blockDim.x) {
      const int k = c / (nl / 2), q = c - k * (nl / 2);
      cp_async16(buf + k * HP + 2 * q, base + (long)k * NN + 2 * q);
    }
    if (AUX) {
      float *ab = abuf + half * (RL * NP);
      const float *a0 = aux + (lt % NN) * N;
      for (int c = threadIdx.x; c < nl * (N / 4); c += blockDim.x) {
        const int r = c / (N / 4), q = c - r * (N / 4);
        cp_async16(ab + r * NP + 4 * q, a0 + (long)r * N + 4 * q);
      }
    }
    cp_async_commit();
  };
  int line, lane;
  thread_map<N, LINES, true>(line, lane);
  long t = blockIdx.x;
  if (t < n_tiles) stage(t, 0);
  for (int it = 0; t < n_tiles; ++it, t += gridDim.x) {
    const float2 *hs = zbuf + (it & 1) * (H * HP);
    const float *acur = abuf + (it & 1) * (RL * NP);
    if (t + gridDim.x < n_tiles) {
      stage(t + gridDim.x, (it + 1) & 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const long l_base = t * RL;
    const long l0 = l_base + 2 * line;
    const bool ok0 = l0 < n_lines, ok1 = l0 + 1 < n_lines;
    // inverse (as k_c2r_stream)
    float2 v[A], o[B];
    if (lane < B) {
#pragma unroll
      for (int j1 = 0; j1 < A; ++j1) {
        int k = B * j1 + lane;
        float2 a, b;
        const int kk = k <= N / 2 ? k : N - k;
        const float4 ab = *reinterpret_cast<const float4 *>(&hs[kk * HP + 2 * line]);
        a = make_float2(ab.x, ab.y);
        b = make_float2(ab.z, ab.w);
        if (k == 0 || k == N / 2) {
          a.y = 0.f;
          b.y = 0.f;
        } else if (k > N / 2) {
          a = cconj(a);
          b = cconj(b);
        }
        v[j1] = make_float2(a.x - b.y, a.y + b.x);
      }
    }
    __syncthreads();
    four_step<N, LINES, true>(v, o, line, lane, +1, tw, ex);
    __syncthreads();  // ex is reused for the real lines
    if (lane < A) {
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) {
        const int k = lane + A * k2;
        rt[(2 * line) * NP + k] = o[k2].x;
        rt[(2 * line + 1) * NP + k] = o[k2].y;
      }
    }
    __syncthreads();
    // forward (as k_r2c_stream), inputs Mid(real value)
    mid.begin();
    if (lane < B) {
#pragma unroll
      for (int j1 = 0; j1 < A; ++j1) {
        const int k = B * j1 + lane;
        const float a = ok0 ? mid(l0, k, rt[(2 * line) * NP + k], AUX ? acur[(2 * line) * NP + k] : 1.f) : 0.f;
        const float b = ok1 ? mid(l0 + 1, k, rt[(2 * line + 1) * NP + k], AUX ? acur[(2 * line + 1) * NP + k] : 1.f) : 0.f;
        v[j1] = make_float2(a, b);
      }
    }
    mid.end_tile(l_base);
    __syncthreads();
    four_step<N, LINES, true>(v, o, line, lane, -1, tw, ex);
    __syncthreads();
    if (lane < A) {
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) ex[(lane + A * k2) * SP + line] = o[k2];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < H * RL; idx += blockDim.x) {
      const int k = idx / RL, rl = idx - k * RL, cl = rl >> 1;
      const long l = l_base + rl;
      if (l < n_lines) {
        const float2 zk = ex[k * SP + cl];
        const float2 zn = ex[((N - k) & (N - 1)) * SP + cl];
        const float2 xv = (rl & 1) ? make_float2(0.5f * (zk.y + zn.y), -0.5f * (zk.x - zn.x))
                                   : make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y));
        data[(l / NN) * H * NN + (long)k * NN + (l % NN)] = xv;
      }
    }
    __syncthreads();  // ex and this half of the buffer are reused by the next tiles
  }
}
template <int N, bool AUX>
constexpr size_t c2r_r2c_stream_smem() {
  return 2 * (size_t)(N / 2 + 1) * (2 * (256 / MaxAB<N>::v) + 2) * sizeof(float2) +
         (AUX ? 2 * (size_t)(2 * (256 / MaxAB<N>::v)) * stream_pitch<N>() * sizeof(float) : 0);
}

// Lines of a pruned, zero-padded inverse transform: line l = outer * inner_n + inner reads n_in complex
// inputs at in + outer * in_outer + (inner / in_div) * in_mid + inner % in_div + n * in_stride and writes
// W outputs at out + outer * out_outer + inner + X * out_stride.
struct PrunedLines {
  long n_lines, inner_n, in_outer, in_div, in_mid, in_stride, out_outer, out_stride;
};

// One axis of the upsampled (2N)^3 C2R restricted to the translational search window
// (nbfFourierImageMetric::executeFourierNewHalf, inc/em/nbfFourierImageMetric.h:1203-1264): for each line,
//   y[X] = sum_{k < n_in} x[k] exp(+2 pi i (k + off)(lo + X) / NN),  X < W,
// computed as exp(+2 pi i off m / NN) * IFFT_NN(x zero-padded)[m] with m = (lo + X) mod NN.
template <int NN, int LINES, bool CONTIG>
__global__ void __launch_bounds__(LINES * ((Split<NN>::A > Split<NN>::B) ? Split<NN>::A : Split<NN>::B))
    k_pruned_fft(const float2 *__restrict__ in, float2 *__restrict__ out, PrunedLines pl, int n_in, int W, int lo,
                 int off) {
  constexpr int A = Split<NN>::A, B = Split<NN>::B;
  __shared__ float2 tw[NN];
  __shared__ float2 ex[ex_size<NN, LINES, CONTIG>()];
  load_full_twiddles<NN>(tw);
  int line, lane;
  thread_map<NN, LINES, CONTIG>(line, lane);
  const long l = (long)blockIdx.x * LINES + line;
  const bool ok = l < pl.n_lines;
  const long outer = ok ? l / pl.inner_n : 0, inner = ok ? l - outer * pl.inner_n : 0;
  const long q = inner / pl.in_div;
  const float2 *src = in + outer * pl.in_outer + q * pl.in_mid + (inner - q * pl.in_div);
  float2 *dst = out + outer * pl.out_outer + inner;
  float2 v[A], o[B];
  if (lane < B) {
#pragma unroll
    for (int j1 = 0; j1 < A; ++j1) {
      const int n = B * j1 + lane;
      v[j1] = (ok && n < n_in) ? src[(long)n * pl.in_stride] : make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  four_step<NN, LINES, CONTIG>(v, o, line, lane, +1, tw, ex);
  if (lane < A && ok) {
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) {
      const int m = lane + A * k2;
      const int X = (m - lo) & (NN - 1);
      if (X < W) dst[(long)X * pl.out_stride] = cmul(o[k2], twid<NN>(tw, off * m, +1));
    }
  }
}

// The x and y axes of the same windowed transform in one pass per (kz plane, item), for the kz-major spectrum
// [item][kz][kx][ky] (n = NN / 2 the box edge, H = n/2 + 1): the plane's n x lines (stride n) are read from global
// memory LINES at a time and their W window outputs kept in shared memory, T[X][ky] (row pitch n + 8 complex: the x
// stores and y loads of a warp touch distinct banks); then the W y lines of T are transformed and written to
// q2[item][X][kz][Y]. Each line takes the zero-padded NN-point inverse and the output twiddle of k_pruned_fft, in
// the same order, so q2 equals that of the two separate passes; the intermediate [item][X][kz][ky] array (and its
// round trip through HBM) is gone. Dynamic shared memory: W * (n + 8) complex.
template <int NN, int LINES>
__host__ __device__ constexpr int pruned_xy_ex() {
  return ex_size<NN, LINES, false>() > ex_size<NN, LINES, true>() ? ex_size<NN, LINES, false>()
                                                                  : ex_size<NN, LINES, true>();
}
template <int NN, int LINES>
__global__ void __launch_bounds__(LINES * MaxAB<NN>::v, NN >= 256 ? 2 : 4)
    k_pruned_xy(const float2 *__restrict__ in, float2 *__restrict__ q2, int W, int lo, int off) {
  constexpr int A = Split<NN>::A, B = Split<NN>::B, n = NN / 2, H = n / 2 + 1, TP = n + 8;
  __shared__ float2 tw[NN];
  __shared__ float2 ex[pruned_xy_ex<NN, LINES>()];
  extern __shared__ float4 pxy_dyn[];
  float2 *T = reinterpret_cast<float2 *>(pxy_dyn);
  load_full_twiddles<NN>(tw);
  const int kz = blockIdx.x;
  const long item = blockIdx.y;
  float2 v[A], o[B];
  {
    // x: line ky of the plane, elements kx at stride n; adjacent threads are adjacent lines (coalesced rows)
    int line, lane;
    thread_map<NN, LINES, false>(line, lane);
    const float2 *plane = in + (item * H + kz) * (long)n * n;
#pragma unroll 1
    for (int ky0 = 0; ky0 < n; ky0 += LINES) {
      const int ky = ky0 + line;
      const bool ok = ky < n;
      if (lane < B) {
#pragma unroll
        for (int j1 = 0; j1 < A; ++j1) {
          const int kx = B * j1 + lane;
          v[j1] = (ok && kx < n) ? plane[(long)kx * n + ky] : make_float2(0.f, 0.f);
        }
      }
      __syncthreads();  // twiddles loaded; the previous round's exchange reads done
      four_step<NN, LINES, false>(v, o, line, lane, +1, tw, ex);
      if (lane < A && ok) {
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) {
          const int m = lane + A * k2;
          const int X = (m - lo) & (NN - 1);
          if (X < W) T[X * TP + ky] = cmul(o[k2], twid<NN>(tw, off * m, +1));
        }
      }
    }
  }
  __syncthreads();
  {
    // y: line X of T (contiguous), adjacent threads are adjacent elements of a line
    int line, lane;
    thread_map<NN, LINES, true>(line, lane);
#pragma unroll 1
    for (int X0 = 0; X0 < W; X0 += LINES) {
      const int X = X0 + line;
      const bool ok = X < W;
      if (lane < B) {
#pragma unroll
        for (int j1 = 0; j1 < A; ++j1) {
          const int ky = B * j1 + lane;
          v[j1] = (ok && ky < n) ? T[X * TP + ky] : make_float2(0.f, 0.f);
        }
      }
      __syncthreads();
      four_step<NN, LINES, true>(v, o, line, lane, +1, tw, ex);
      if (lane < A && ok) {
        float2 *dst = q2 + ((item * W + X) * H + kz) * (long)W;
#pragma unroll
        for (int k2 = 0; k2 < B; ++k2) {
          const int m = lane + A * k2;
          const int Y = (m - lo) & (NN - 1);
          if (Y < W) dst[Y] = cmul(o[k2], twid<NN>(tw, off * m, +1));
        }
      }
    }
  }
}

}  // namespace ettk
