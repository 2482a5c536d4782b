/* Oracle restatement of SOFT 1.0 transforms (test infrastructure only).
 * See so3.h for the conventions and the SOFT source locations. */
#include "so3.h"
#include "fft64.h"
#include <cmath>
#include <map>
#include <mutex>

namespace oracle {

static void small_d_start(int J, int m1, int m2, double c, double s, double &out) {
  /* Single-term (k range collapses at J = max(|m1|,|m2|)) of
   * d^J_{m1 m2} = sum_k (-1)^{k-m2+m1} sqrt((J+m2)!(J-m2)!(J+m1)!(J-m1)!) /
   *               ((J+m2-k)! k! (J-k-m1)! (k-m2+m1)!) c^{2J-2k+m2-m1} s^{2k-m2+m1} */
  double acc = 0.0;
  for (int k = 0; k <= 2 * J; ++k) {
    if (J + m2 - k < 0 || J - k - m1 < 0 || k - m2 + m1 < 0) continue;
    double lg = 0.5 * (lgamma(J + m2 + 1.0) + lgamma(J - m2 + 1.0) + lgamma(J + m1 + 1.0) + lgamma(J - m1 + 1.0)) -
                (lgamma(J + m2 - k + 1.0) + lgamma(k + 1.0) + lgamma(J - k - m1 + 1.0) + lgamma(k - m2 + m1 + 1.0));
    double sign = ((k - m2 + m1) % 2 == 0) ? 1.0 : -1.0;
    acc += sign * exp(lg) * pow(c, 2 * J - 2 * k + m2 - m1) * pow(s, 2 * k - m2 + m1);
  }
  out = acc;
}

/* d^l_{m1 m2}(beta) for all l in [max(|m1|,|m2|), B) via the three-term recurrence. */
static void small_d_column(int B, int m1, int m2, double beta, double *out /* [B] by l */) {
  double c = cos(beta / 2), s = sin(beta / 2), cb = cos(beta);
  int l0 = std::max(std::abs(m1), std::abs(m2));
  double prev = 0.0, cur;
  small_d_start(l0, m1, m2, c, s, cur);
  out[l0] = cur;
  for (int l = l0; l < B - 1; ++l) {
    double a = (l + 1) * (2.0 * l + 1) / sqrt(((l + 1.0) * (l + 1) - m1 * m1) * ((l + 1.0) * (l + 1) - m2 * m2));
    double nxt;
    if (l == 0) {
      nxt = a * cb * cur;
    } else {
      double t1 = (cb - (double)m1 * m2 / (l * (l + 1.0))) * cur;
      double t2 = (sqrt(((double)l * l - m1 * m1) * ((double)l * l - m2 * m2)) / (l * (2.0 * l + 1))) * prev;
      nxt = a * (t1 - t2);
    }
    prev = cur;
    cur = nxt;
    out[l + 1] = cur;
  }
}

void wigner_d_at(int B, double beta, std::vector<double> &out) {
  int W = 2 * B;
  out.assign((size_t)B * W * W, 0.0);
  std::vector<double> col(B);
  for (int m1 = -B + 1; m1 < B; ++m1)
    for (int m2 = -B + 1; m2 < B; ++m2) {
      small_d_column(B, m1, m2, beta, col.data());
      for (int l = std::max(std::abs(m1), std::abs(m2)); l < B; ++l)
        out[((size_t)l * W + m1 + B) * W + m2 + B] = col[l];
    }
}

const SO3Tables &so3_tables(int B) {
  static std::map<int, SO3Tables> cache;
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(B);
  if (it != cache.end()) return it->second;
  SO3Tables t;
  t.B = B;
  int n = 2 * B;
  t.w.resize(n);
  std::vector<double> th(n), x(n), sn(n);
  for (int j = 0; j < n; ++j) {
    th[j] = M_PI * (2.0 * j + 1.0) / (4.0 * B);
    x[j] = cos(th[j]);
    sn[j] = sin(th[j]);
    double acc = 0;
    for (int k = 0; k < B; ++k) acc += sin((2.0 * k + 1.0) * th[j]) / (2.0 * k + 1.0);
    t.w[j] = (2.0 / B) * sn[j] * acc;
  }
  t.plm.assign((size_t)B * B * n, 0.0);
  for (int m = 0; m < B; ++m) {
    double c = sqrt((2.0 * m + 1.0) / 2.0);
    for (int i = 1; i <= m; ++i) c *= sqrt((2.0 * i - 1.0) / (2.0 * i));
    if (m % 2) c = -c;
    for (int j = 0; j < n; ++j) {
      double pmm = c * pow(sn[j], m);
      t.plm[((size_t)m * B + m) * n + j] = pmm;
      if (m + 1 < B) t.plm[((size_t)(m + 1) * B + m) * n + j] = x[j] * sqrt(2.0 * m + 3.0) * pmm;
    }
    for (int l = m + 2; l < B; ++l) {
      double a = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
      double b = sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
      for (int j = 0; j < n; ++j)
        t.plm[((size_t)l * B + m) * n + j] =
            a * (x[j] * t.plm[((size_t)(l - 1) * B + m) * n + j] - b * t.plm[((size_t)(l - 2) * B + m) * n + j]);
    }
  }
  return cache.emplace(B, std::move(t)).first->second;
}

void sht_forward_real(int B, const double *f, std::vector<cplx> &coef) {
  const SO3Tables &t = so3_tables(B);
  int n = 2 * B, W = 2 * B;
  std::vector<cplx> G((size_t)n * n);
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k) G[(size_t)j * n + k] = cplx(f[(size_t)j * n + k], 0.0);
  fft1d(G.data(), n, -1, n, 1, n);
  coef.assign((size_t)B * W, cplx(0, 0));
  double norm = sqrt(2.0 * M_PI) / n;
  for (int m = 0; m < B; ++m)
    for (int l = m; l < B; ++l) {
      cplx acc(0, 0);
      for (int j = 0; j < n; ++j) acc += t.w[j] * t.plm[((size_t)l * B + m) * n + j] * G[(size_t)j * n + m];
      acc *= norm;
      coef[(size_t)l * W + m + B] = acc;
      if (m > 0) coef[(size_t)l * W - m + B] = ((m % 2) ? -1.0 : 1.0) * std::conj(acc);
    }
}

void so3_correlate(int B, const double *f1, const double *f2, double *C) {
  const SO3Tables &t = so3_tables(B);
  int n = 2 * B, W = 2 * B;
  std::vector<cplx> fc, hc;
  sht_forward_real(B, f1, fc);
  sht_forward_real(B, f2, hc);
  /* S[m1 mod n][m2 mod n][b] = sum_l F^l_{m1m2} dtilde^l_{m1m2}(beta_b) */
  std::vector<cplx> S((size_t)n * n * n, cplx(0, 0));
  std::vector<double> col((size_t)B * n);
  std::vector<double> th(n);
  for (int b = 0; b < n; ++b) th[b] = M_PI * (2.0 * b + 1.0) / (4.0 * B);
  for (int m1 = -B + 1; m1 < B; ++m1)
    for (int m2 = -B + 1; m2 < B; ++m2) {
      int l0 = std::max(std::abs(m1), std::abs(m2));
      for (int b = 0; b < n; ++b) {
        std::vector<double> tmp(B);
        small_d_column(B, m1, m2, th[b], tmp.data());
        for (int l = l0; l < B; ++l) col[(size_t)l * n + b] = tmp[l];
      }
      cplx *dst = &S[((size_t)((m1 + n) % n) * n + (m2 + n) % n) * n];
      for (int l = l0; l < B; ++l) {
        cplx F = fc[(size_t)l * W - m1 + B] * std::conj(hc[(size_t)l * W - m2 + B]) * (((m1 + m2) % 2) ? -1.0 : 1.0);
        double nl = sqrt((2.0 * l + 1.0) / 2.0);
        const double *d = &col[(size_t)l * n];
        for (int b = 0; b < n; ++b) dst[b] += F * (nl * d[b]);
      }
    }
  /* out[a][b][g] = sum_{m1,m2} e^{-i 2pi m1 a/n} e^{-i 2pi m2 g/n} S[m1][m2][b]: forward DFT over m1 and m2 */
  std::vector<cplx> T((size_t)n * n * n);
  for (int b = 0; b < n; ++b)
    for (int m1 = 0; m1 < n; ++m1)
      for (int m2 = 0; m2 < n; ++m2) T[((size_t)b * n + m1) * n + m2] = S[((size_t)m1 * n + m2) * n + b];
  for (int b = 0; b < n; ++b) {
    cplx *p = &T[(size_t)b * n * n];
    fft1d(p, n, -1, n, 1, n);   /* over m2 -> g (rows) */
    fft1d(p, n, -1, n, n, 1);   /* over m1 -> a (columns) */
  }
  double scale = (1.0 / n) * ((double)B / M_PI);
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < n; ++b)
      for (int g = 0; g < n; ++g) C[((size_t)a * n + b) * n + g] = T[((size_t)b * n + a) * n + g].real() * scale;
}

void s2_rotate(int B, const double *f, double alpha, double beta, double gamma, double *R) {
  const SO3Tables &t = so3_tables(B);
  int n = 2 * B, W = 2 * B;
  std::vector<cplx> fc;
  sht_forward_real(B, f, fc);
  std::vector<double> d;
  wigner_d_at(B, beta, d);
  std::vector<cplx> g((size_t)B * W, cplx(0, 0));
  for (int l = 0; l < B; ++l)
    for (int m = -l; m <= l; ++m) {
      cplx acc(0, 0);
      for (int mp = -l; mp <= l; ++mp)
        acc += std::exp(cplx(0, -m * alpha)) * d[((size_t)l * W + m + B) * W + mp + B] * std::exp(cplx(0, -mp * gamma)) *
               fc[(size_t)l * W + mp + B];
      g[(size_t)l * W + m + B] = acc;
    }
  /* R[j][k] = (1/sqrt(2pi)) Re sum_m e^{i m phi_k} sum_l g(l,m) P~_l^m(theta_j) */
  std::vector<cplx> H((size_t)n * n, cplx(0, 0));
  for (int j = 0; j < n; ++j)
    for (int m = -B + 1; m < B; ++m) {
      int am = std::abs(m);
      double sg = (m < 0 && (am % 2)) ? -1.0 : 1.0;
      cplx acc(0, 0);
      for (int l = am; l < B; ++l) acc += g[(size_t)l * W + m + B] * (sg * t.plm[((size_t)l * B + am) * n + j]);
      H[(size_t)j * n + (m + n) % n] = acc;
    }
  fft1d(H.data(), n, +1, n, 1, n);
  double s = 1.0 / sqrt(2.0 * M_PI);
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n; ++k) R[(size_t)j * n + k] = H[(size_t)j * n + k].real() * s;
}

} // namespace oracle
