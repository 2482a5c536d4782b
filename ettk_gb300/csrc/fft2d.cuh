// (x, y) passes of the 3-D transforms on kz-major spectra.
//
// Every half spectrum of an N^3 volume is stored kz-major, [item][kz][x][y] (kz < N/2+1), so one kz plane
// is a contiguous N x N complex tile. k_fft2d transforms one plane per CTA in shared memory: coalesced
// load (with an optional fused prologue), the N-point register FFT of every row (y lines), then of every
// column (x lines), and a coalesced store (with an optional fused epilogue). The prologues/epilogues are
// the elementwise steps of executeFourierNewHalf that sit between the transforms (filter, normalisation
// sums, the FFT2re update and the cross term), so each of them costs no extra pass over HBM.
#pragma once
#include "fft_reg.cuh"

namespace ettk {

// kz-major index of element i = x*N + y of plane kz of item e
template <int N>
struct KXY {
  static constexpr int H = N / 2 + 1;
  static constexpr long NN = (long)N * N;
  static constexpr long h3 = NN * H;
  ETTK_DEV static long at(long e, int kz, int i) { return (e * H + kz) * NN + i; }
  // DC of the centred half spectrum: (x, y, kz) = (N/2, N/2, H-1)
  static constexpr int dc_xy = (N / 2) * N + N / 2;
};

// FFT of one line of N complex values in shared memory (element n at line[n * stride]) by a group of
// MaxAB<N> consecutive lanes of one warp (lane = index within the group; act = false for a group without a
// line). Every lane of the warp must make the call (warp-synchronous exchange through the line itself).
// The exchange stores y[k1][j2] at k1*B + ((j2 + k1) mod B), so that both the stage-1 stores (lanes = j2)
// and the stage-2 loads (lanes = k1) touch distinct banks.
template <int N>
ETTK_DEV void group_fft(float2 *line, int stride, int lane, bool act, int sign, const float2 *tw) {
  constexpr int A = Split<N>::A, B = Split<N>::B;
  float2 v[A];
  const bool s1 = act && lane < B, s2 = act && lane < A;
  if (s1) {
#pragma unroll
    for (int j1 = 0; j1 < A; ++j1) v[j1] = line[(B * j1 + lane) * stride];
    dft_reg<A>(v, sign);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) v[k1] = cmul(v[k1], twid<N>(tw, lane * k1, sign));
  }
  __syncwarp();
  if (s1) {
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) line[(k1 * B + ((lane + k1) & (B - 1))) * stride] = v[k1];
  }
  __syncwarp();
  float2 o[B];
  if (s2) {
#pragma unroll
    for (int j2 = 0; j2 < B; ++j2) o[j2] = line[(lane * B + ((j2 + lane) & (B - 1))) * stride];
    dft_reg<B>(o, sign);
  }
  __syncwarp();
  if (s2) {
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) line[(lane + A * k2) * stride] = o[k2];
  }
  __syncwarp();
}

// Operators whose planes are zero outside a band of rows declare rows(kz, r0, r1): rows x < r0 or x >= r1 of
// plane kz are zero (not loaded, not transformed along y).
template <class T, class = void>
struct has_rows : std::false_type {};
template <class T>
struct has_rows<T, std::void_t<decltype(std::declval<const T &>().rows(0, std::declval<int &>(), std::declval<int &>()))>>
    : std::true_type {};

// Shared memory of k_fft2d: the plane with a row pitch of N+1 complex values.
template <int N>
constexpr size_t fft2d_smem() { return (size_t)N * (N + 1) * sizeof(float2); }

// One CTA per (kz plane, item) = (blockIdx.x, blockIdx.y). Op supplies sign, begin(), load(e, kz, i),
// store(e, kz, i, x, y, v) and end(e, kz) (all threads call begin/end).
template <int N, class Op>
__global__ void __launch_bounds__(256, N <= 64 ? 6 : 1) k_fft2d(Op op) {
  constexpr int G = MaxAB<N>::v;      // lanes per line
  constexpr int GROUPS = 256 / G;     // lines in flight
  constexpr int WG = 32 / G;          // groups per warp
  constexpr int P = N + 1;            // row pitch
  extern __shared__ float2 pl[];
  __shared__ float2 tw[N];
  load_full_twiddles<N>(tw);
  const int kz = blockIdx.x, e = blockIdx.y;
  int rlo = 0, rhi = N;
  if constexpr (has_rows<Op>::value) op.rows(kz, rlo, rhi);
  op.begin();
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) {
    const int x = i / N, y = i - x * N;
    pl[x * P + y] = (x >= rlo && x < rhi) ? op.load(e, kz, i) : make_float2(0.f, 0.f);
  }
  __syncthreads();
  // the groups of one warp take lines 8 apart, which puts their rows / columns 16 words apart in the banks
  const int grp = threadIdx.x / G, lane = threadIdx.x % G;
  const int sub = (grp % WG) * (GROUPS / WG) + grp / WG;
  for (int r0 = 0; r0 < N; r0 += GROUPS) {
    const int r = r0 + sub;
    group_fft<N>(pl + (r < N ? r : 0) * P, 1, lane, r >= rlo && r < rhi, op.sign, tw);
  }
  __syncthreads();
  for (int c0 = 0; c0 < N; c0 += GROUPS) {
    const int c = c0 + sub;
    group_fft<N>(pl + (c < N ? c : 0), P, lane, c < N, op.sign, tw);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) {
    const int x = i / N, y = i - x * N;
    op.store(e, kz, i, x, y, pl[x * P + y]);
  }
  op.end(e, kz);
}

// In-place (x, y) transform.
template <int N>
struct OpPlain {
  float2 *d;
  int sign;
  ETTK_DEV void begin() {}
  ETTK_DEV float2 load(int e, int kz, int i) const { return d[KXY<N>::at(e, kz, i)]; }
  ETTK_DEV void store(int e, int kz, int i, int, int, float2 v) { d[KXY<N>::at(e, kz, i)] = v; }
  ETTK_DEV void end(int, int) {}
};

// Inverse (x, y) passes of spectra multiplied by one half-grid filter shared by all items (kz-major
// [H][N][N]): nbfFourierFilter::executeHalf without a wedge (inc/em/nbfFourierFilter.h:587-603). In place.
template <int N>
struct OpFilterShared {
  float2 *d;
  const float *filter;
  int sign = +1;
  ETTK_DEV void begin() {}
  ETTK_DEV float2 load(int e, int kz, int i) const {
    return cscale(d[KXY<N>::at(e, kz, i)], __ldg(filter + KXY<N>::at(0, kz, i)));
  }
  ETTK_DEV void store(int e, int kz, int i, int, int, float2 v) { d[KXY<N>::at(e, kz, i)] = v; }
  ETTK_DEV void end(int, int) {}
};

// Forward (x, y) passes of the (2N)^3 spectrum of the padded spherical-projection volume (z pass done), storing
// |F| (as the magnitude step of cartesianToSpherical) into a real kz-major array. The padded real volume is
// the windowed N^3 image at x, y, z < N and the constant c (-1)^(x+y+z) elsewhere (PrePadded); the z transform
// of a line with x >= N or y >= N is zero except at kz = N, so every plane but the last is zero in rows
// x >= N.
template <int N2>
struct OpPaddedMagnitude {
  const float2 *d;
  float *mag;
  int sign = -1;
  int kz0 = 0;  // plane of blockIdx.x = 0 (the launch for the last plane alone uses kz0 = N2 / 2)
  int mutual = 0;  // store |F|^(1/2) (mutual correlation)
  // with padc (the padding constant c of each item), the entries (x, y) of the last plane with x >= N2/2 or
  // y >= N2/2 are those of padding lines whose z pass was skipped: N2 c (-1)^(x+y)
  const float *padc = nullptr;
  ETTK_DEV void begin() {}
  ETTK_DEV void rows(int kz, int &r0, int &r1) const {
    if (kz + kz0 < KXY<N2>::H - 1) {
      r0 = 0;
      r1 = N2 / 2;
    }
  }
  ETTK_DEV float2 load(int e, int kz, int i) const {
    if (padc && kz + kz0 == KXY<N2>::H - 1) {
      const int x = i / N2, y = i - x * N2;
      if (x >= N2 / 2 || y >= N2 / 2) {
        const float v = (float)N2 * padc[e];
        return make_float2(((x + y) & 1) ? -v : v, 0.f);
      }
    }
    return d[KXY<N2>::at(e, kz + kz0, i)];
  }
  ETTK_DEV void store(int e, int kz, int i, int, int, float2 v) {
    mag[KXY<N2>::at(e, kz + kz0, i)] = spectrum_magnitude(v, mutual);
  }
  ETTK_DEV void end(int, int) {}
};

// The planes kz < N2/2 of the same pass in less shared memory: there only the rows x < R = N2/2 are nonzero, and
// their entries y >= R too (the z transforms of the padding lines vanish below kz = N2/2), so after the row
// transforms every column is a length-N2 transform of R values followed by zeros, computed as two R-point
// transforms (even outputs: the column; odd outputs: the column times e^{-2 pi i j / N2}). Shared memory holds
// the R nonzero rows and the twiddled copy of half of the columns at a time, so that two CTAs share an SM.
template <int N2>
constexpr size_t fft2d_padded_smem() {
  return ((size_t)(N2 / 2) * (N2 + 1) + (size_t)(N2 / 2) * (N2 / 2 + 1)) * sizeof(float2);
}
template <int N2>
__global__ void __launch_bounds__(256, 2) k_fft2d_padded(const float2 *__restrict__ d, float *__restrict__ mag,
                                                          int mutual) {
  constexpr int R = N2 / 2, PA = N2 + 1, PB = R + 1;
  constexpr int G1 = MaxAB<N2>::v, GR1 = 256 / G1, WG1 = 32 / G1;
  constexpr int G2 = MaxAB<R>::v, GR2 = 256 / G2, WG2 = 32 / G2;
  extern __shared__ float2 pdm[];
  float2 *A = pdm, *Bm = pdm + R * PA;
  __shared__ float2 tw1[N2], tw2[R];
  load_full_twiddles<N2>(tw1);
  load_full_twiddles<R>(tw2);
  const int kz = blockIdx.x, e = blockIdx.y;
  for (int i = threadIdx.x; i < R * N2; i += blockDim.x) {
    const int x = i / N2, y = i - x * N2;
    A[x * PA + y] = y < R ? d[KXY<N2>::at(e, kz, x * N2 + y)] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  {  // row transforms (y lines), lines of one warp 8 apart as in k_fft2d
    const int grp = threadIdx.x / G1, lane = threadIdx.x % G1;
    const int sub = (grp % WG1) * (GR1 / WG1) + grp / WG1;
    for (int r0 = 0; r0 < R; r0 += GR1) {
      const int r = r0 + sub;
      group_fft<N2>(A + (r < R ? r : 0) * PA, 1, lane, r < R, -1, tw1);
    }
  }
  __syncthreads();
  for (int h = 0; h < 2; ++h) {
    const int c0 = h * R;
    for (int i = threadIdx.x; i < R * R; i += blockDim.x) {
      const int j = i / R, c = i - j * R;
      Bm[j * PB + c] = cmul(A[j * PA + c0 + c], tw1[j]);
    }
    __syncthreads();
    {  // column transforms: A's columns c0 .. c0 + R - 1 (even outputs) and Bm's (odd outputs)
      const int grp = threadIdx.x / G2, lane = threadIdx.x % G2;
      const int sub = (grp % WG2) * (GR2 / WG2) + grp / WG2;
      for (int q0 = 0; q0 < 2 * R; q0 += GR2) {
        const int q = q0 + sub;
        const bool act = q < 2 * R;
        float2 *line = !act ? A : (q < R ? A + c0 + q : Bm + (q - R));
        group_fft<R>(line, q < R || !act ? PA : PB, lane, act, -1, tw2);
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < N2 * R; i += blockDim.x) {
      const int x = i / R, c = i - x * R;
      const float2 v = (x & 1) ? Bm[(x >> 1) * PB + c] : A[(x >> 1) * PA + c0 + c];
      mag[KXY<N2>::at(e, kz, x * N2 + c0 + c)] = spectrum_magnitude(v, mutual);
    }
    __syncthreads();
  }
}

// Sums of |v|^2 of a normalizeFourierHalf (inc/em/nbfCorrelationImageMetric.h:497-530): kz < H-1 into
// acc[e][slot], the kz = H-1 plane into acc[e][slot+1]; per-thread FP32 partials, a float-pair tree across
// threads (block_sum_f).
template <int N>
struct HalfSums {
  double *acc;
  int acc_stride, slot;
  float s = 0.f;
  ETTK_DEV void add(float2 v) { s += v.x * v.x + v.y * v.y; }
  ETTK_DEV void flush(int e, int kz) {
    __shared__ float2 shm[32];
    const double b = block_sum_f(s, shm);
    if (threadIdx.x == 0) atomicAdd(&acc[(long)e * acc_stride + slot + (kz == KXY<N>::H - 1 ? 1 : 0)], b);
  }
};

// I1 branch: F1 = FI1[ref] * fw with the DC zeroed (executeHalf, inc/em/nbfFourierFilter.h:586-606), its
// normalisation sums, then the inverse (x, y) passes (the 1/norm scale is applied by the following C2R).
template <int N>
struct OpFilterInv {
  const float2 *src;
  const int *src_index;
  const float *fw;
  float2 *dst;
  HalfSums<N> sums;
  int sign = +1;
  ETTK_DEV void begin() {}
  ETTK_DEV float2 load(int e, int kz, int i) {
    const long g = KXY<N>::at(e, kz, i);
    float2 v = cscale(__ldg(src + KXY<N>::at(__ldg(src_index + e), kz, i)), __ldg(fw + g));
    if (kz == KXY<N>::H - 1 && i == KXY<N>::dc_xy) v = make_float2(0.f, 0.f);
    sums.add(v);
    return v;
  }
  ETTK_DEV void store(int e, int kz, int i, int, int, float2 v) { dst[KXY<N>::at(e, kz, i)] = v; }
  ETTK_DEV void end(int e, int kz) { sums.flush(e, kz); }
};

// I2 branch: forward (x, y) passes, then * fw with the DC zeroed and the normalisation sums.
template <int N>
struct OpFwdFilter {
  float2 *d;
  const float *fw;
  HalfSums<N> sums;
  const int *fw_index = nullptr;  // item whose wedge * filter applies (null: the item itself)
  int sign = -1;
  int mutual = 0;  // F / |F|^(1/2) before the filter (executeHalf with mutual correlation)
  ETTK_DEV void begin() {}
  ETTK_DEV float2 load(int e, int kz, int i) const { return d[KXY<N>::at(e, kz, i)]; }
  ETTK_DEV void store(int e, int kz, int i, int, int, float2 v) {
    const long g = KXY<N>::at(e, kz, i);
    if (mutual) v = mutual_scale(v);
    v = cscale(v, __ldg(fw + (fw_index ? KXY<N>::at(__ldg(fw_index + e), kz, i) : g)));
    if (kz == KXY<N>::H - 1 && i == KXY<N>::dc_xy) v = make_float2(0.f, 0.f);
    sums.add(v);
    d[g] = v;
  }
  ETTK_DEV void end(int e, int kz) { sums.flush(e, kz); }
};

// FFT2re = 2 * FFT1re * conj(F2 / norm2 * N^3) (nbfFourierImageMetric.h:1174-1177) into its own buffer, then
// the inverse (x, y) passes of F2 / norm2. FFT1re of item e is a[a_index[e]] (evaluations that share the
// reference branch read one copy; it is never written here, so no item reads what another overwrites).
template <int N>
struct OpFft2reInv {
  const float2 *a;           // FFT1re
  const int *a_index;        // item whose FFT1re applies (null: the item itself)
  float2 *fft2re;            // FFT2re out
  float2 *b;                 // F2 (transformed in place)
  const float *inv_norm2;
  int sign = +1;
  ETTK_DEV void begin() {}
  ETTK_DEV float2 load(int e, int kz, int i) {
    const long g = KXY<N>::at(e, kz, i);
    const float sc = __ldg(inv_norm2 + e);
    const float2 bb = b[g];
    const float2 bs = cscale(bb, sc * (float)((long)N * N * N));
    const float2 f1 = __ldg(a + (a_index ? KXY<N>::at(__ldg(a_index + e), kz, i) : g));
    fft2re[g] = cscale(cmul(f1, cconj(bs)), 2.0f);
    return cscale(bb, sc);
  }
  ETTK_DEV void store(int e, int kz, int i, int, int, float2 v) { b[KXY<N>::at(e, kz, i)] = v; }
  ETTK_DEV void end(int, int) {}
};

// Forward (x, y) passes of F(I2'^2), then FFTre = (-F(m1) conj(F(I2'^2)) + FFT2re) * shift * 8
// (nbfFourierImageMetric.h:1192-1210, the 8 of the zero padding).
template <int N>
struct OpFwdCross {
  float2 *q;
  const float2 *fm1;         // one item
  const float2 *fft2re;
  float factor;
  int sign = -1;
  ETTK_DEV void begin() {}
  ETTK_DEV float2 load(int e, int kz, int i) const { return q[KXY<N>::at(e, kz, i)]; }
  ETTK_DEV void store(int e, int kz, int i, int x, int y, float2 v) {
    const long g = KXY<N>::at(e, kz, i);
    const float2 w = cadd(cscale(cmul(__ldg(fm1 + KXY<N>::at(0, kz, i)), cconj(v)), -1.f), __ldg(fft2re + g));
    q[g] = cscale(w, parity_sign(x, y, kz) * factor);
  }
  ETTK_DEV void end(int, int) {}
};

}  // namespace ettk
