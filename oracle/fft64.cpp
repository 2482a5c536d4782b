/* Oracle FP64 FFT (test infrastructure only). See fft64.h for the conventions. */
#include "fft64.h"
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <map>

namespace oracle {

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

namespace {

struct Twiddles {
  std::vector<cplx> w;     /* w[k] = exp(-2 pi i k / n), k < n/2 */
  std::vector<int> rev;    /* bit reversal permutation */
};

/* per-thread cache: callers on many host threads never contend for it */
const Twiddles &twiddles(int n) {
  thread_local std::map<int, Twiddles> cache;
  auto it = cache.find(n);
  if (it != cache.end()) return it->second;
  Twiddles t;
  t.w.resize(n / 2 > 0 ? n / 2 : 1);
  for (int k = 0; k < n / 2; ++k) {
    double a = -2.0 * M_PI * (double)k / (double)n;
    t.w[k] = cplx(std::cos(a), std::sin(a));
  }
  int lg = 0;
  while ((1 << lg) < n) ++lg;
  t.rev.resize(n);
  for (int i = 0; i < n; ++i) {
    int r = 0;
    for (int b = 0; b < lg; ++b)
      if (i & (1 << b)) r |= 1 << (lg - 1 - b);
    t.rev[i] = r;
  }
  return cache.emplace(n, std::move(t)).first->second;
}

void fft_one(cplx *x, int n, int sign, const Twiddles &tw, cplx *buf) {
  for (int i = 0; i < n; ++i) buf[tw.rev[i]] = x[i];
  for (int len = 2; len <= n; len <<= 1) {
    int half = len / 2, step = n / len;
    for (int s = 0; s < n; s += len) {
      for (int k = 0; k < half; ++k) {
        cplx w = tw.w[k * step];
        if (sign > 0) w = std::conj(w);
        cplx a = buf[s + k], b = buf[s + k + half] * w;
        buf[s + k] = a + b;
        buf[s + k + half] = a - b;
      }
    }
  }
  for (int i = 0; i < n; ++i) x[i] = buf[i];
}

} // namespace

void fft1d(cplx *data, int n, int sign, int count, long stride, long dist) {
  if (!is_pow2(n)) {
    fprintf(stderr, "oracle fft1d: length %d is not a power of two\n", n);
    abort();
  }
  if (n == 1) return;
  const Twiddles &tw = twiddles(n);
  std::vector<cplx> line(n), buf(n);
  for (int t = 0; t < count; ++t) {
    cplx *p = data + (long)t * dist;
    for (int i = 0; i < n; ++i) line[i] = p[(long)i * stride];
    fft_one(line.data(), n, sign, tw, buf.data());
    for (int i = 0; i < n; ++i) p[(long)i * stride] = line[i];
  }
}

void rfft3d(const double *in, cplx *out, int n0, int n1, int n2) {
  int h = n2 / 2 + 1;
  std::vector<cplx> row(n2);
  for (long r = 0; r < (long)n0 * n1; ++r) {
    for (int k = 0; k < n2; ++k) row[k] = cplx(in[r * n2 + k], 0.0);
    fft1d(row.data(), n2, -1, 1, 1, n2);
    for (int k = 0; k < h; ++k) out[r * h + k] = row[k];
  }
  /* along dim 1: for each i0, lines over i1 with stride h, count h lines */
  for (int i0 = 0; i0 < n0; ++i0)
    fft1d(out + (long)i0 * n1 * h, n1, -1, h, h, 1);
  /* along dim 0 */
  fft1d(out, n0, -1, n1 * h, (long)n1 * h, 1);
}

void irfft3d(const cplx *in, double *out, int n0, int n1, int n2) {
  int h = n2 / 2 + 1;
  std::vector<cplx> tmp(in, in + (long)n0 * n1 * h);
  fft1d(tmp.data(), n0, +1, n1 * h, (long)n1 * h, 1);
  for (int i0 = 0; i0 < n0; ++i0)
    fft1d(tmp.data() + (long)i0 * n1 * h, n1, +1, h, h, 1);
  std::vector<cplx> row(n2);
  for (long r = 0; r < (long)n0 * n1; ++r) {
    const cplx *src = tmp.data() + r * h;
    row[0] = cplx(src[0].real(), 0.0);
    for (int k = 1; k < n2 / 2; ++k) {
      row[k] = src[k];
      row[n2 - k] = std::conj(src[k]);
    }
    if (n2 > 1) row[n2 / 2] = cplx(src[n2 / 2].real(), 0.0);
    fft1d(row.data(), n2, +1, 1, 1, n2);
    for (int k = 0; k < n2; ++k) out[r * n2 + k] = row[k].real();
  }
}

} // namespace oracle
