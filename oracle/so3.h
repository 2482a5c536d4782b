/* Oracle restatement of the SOFT 1.0 transforms on the alignment path
 * (test infrastructure only; never linked into the product).
 *
 * The restatement computes the same linear maps as SOFT by direct quadrature and
 * direct Wigner sums (SOFT's semi-naive and FFT-based evaluation orders are exact
 * rearrangements of these sums). Conventions were pinned against SOFT itself
 * (oracle/_ref/libsoft_ref.so built from external/soft-1.0) to ~1e-12:
 *
 *  grid      theta_j = pi(2j+1)/(4B), phi_k = 2 pi k/(2B), j,k < 2B; samples f[j][k].
 *  forward   f^(l,m) = sqrt(2 pi)/(2B) * sum_j w_B(j) P~_l^m(cos theta_j) sum_k f[j][k] e^{-i m phi_k}
 *            (FST_semi_memo, FST_semi_memo.c:134-357, with the 2.6 normalisation fix);
 *            w_B(j) = (2/B) sin(theta_j) sum_{k<B} sin((2k+1) theta_j)/(2k+1) (Driscoll-Healy
 *            weights, weights.c); P~ are L2-normalised associated Legendre functions with the
 *            (-1)^m phase (primitive.c Pmm_L2 237-260); real data: f^(l,-m) = (-1)^m conj f^(l,m).
 *  combine   F^l_{m1 m2} = f^(l,-m1) conj(h^(l,-m2)) (-1)^{m1+m2}   (so3_correlate_fftw.c:103-162)
 *  inverse   C(alpha_a, beta_b, gamma_g) = (B/pi)(1/2B) Re sum_{l,m1,m2} F^l_{m1 m2}
 *            sqrt((2l+1)/2) d^l_{m1 m2}(beta_b) e^{-i (m1 alpha_a + m2 gamma_g)},
 *            alpha_a = 2 pi a/2B, beta_b = pi(2b+1)/(4B), gamma_g = 2 pi g/2B
 *            (Inverse_SO3_Naive_fftw, soft_fftw.c:1045-1923); output layout C[a][b][g].
 *  rotate    g(l,m) = sum_m' e^{-i m alpha} d^l_{m m'}(beta) e^{-i m' gamma} f^(l,m'),
 *            R[j][k] = (1/sqrt(2 pi)) Re sum_{l,m} g(l,m) P~_l^m(cos theta_j) e^{i m phi_k}
 *            (rotateFct, rotate_so3.c:695-741, degree limit B-1).
 *  d^l_{m1 m2}(beta) is the Wigner small-d function (Edmonds convention): the single-term
 *  closed form at l = max(|m1|,|m2|) followed by the standard three-term recurrence in l.
 */
#pragma once
#include <complex>
#include <vector>

namespace oracle {

typedef std::complex<double> cplx;

struct SO3Tables {
  int B;
  std::vector<double> w;        /* [2B] quadrature weights */
  std::vector<double> plm;      /* [l][m][j], m <= l < B, j < 2B  (index (l*B+m)*2B+j) */
};

const SO3Tables &so3_tables(int B);

/* Wigner small-d at one angle: out[(l*(2B) + m1+B)*(2B) + m2+B] for l<B. */
void wigner_d_at(int B, double beta, std::vector<double> &out);

/* Forward S^2 transform of real samples f[2B][2B] -> coef[l][m+B] complex (|m| <= l). */
void sht_forward_real(int B, const double *f, std::vector<cplx> &coef);

/* SO(3) correlation of two real S^2 signals, C[a][b][g] (2B)^3 (nbfProjectionRotationMetric3D::soft). */
void so3_correlate(int B, const double *f1, const double *f2, double *C);

/* S^2 rotation of a real signal (nbfProjectionRotationMetric3D::harmonics(A,a,b,g,R)). */
void s2_rotate(int B, const double *f, double alpha, double beta, double gamma, double *R);

} // namespace oracle
