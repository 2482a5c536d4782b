/* Oracle: FP64 CPU restatement of the reference's sub-volume alignment path.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load it, and only as the checker; the product never links it.
 *
 * Unit of work: one (reference, particle) pair through
 * nbfProjectionRotationMetric3D<float>::execute()  (inc/em/nbfProjectionRotationMetric3D.h:415-1052)
 * with alignment_mode 3 (no Powell refinement; refine(t,0) = one CCF,
 * inc/em/nbfFourierImageMetric.h:1701-1760).  Every function cites the reference lines it follows.
 * Where the reference stores a value as Pixel (float) the restatement rounds it to float
 * at the same point, so that float-rounded intermediates match.
 *
 * Parity status: the SO(3)/S^2 stage is pinned against SOFT 1.0 built from the reference
 * sources (oracle/_ref); the FFT follows FFTW3's documented conventions and is checked
 * against numpy; the VTK pieces (reslice, Gaussian smoothing, transforms) are restatements
 * of the vendored VTK 5.10 sources (VTK itself cannot be built here).
 */
#include "fft64.h"
#include "so3.h"
#include "vtk_semantics.h"
#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <queue>
#include <vector>

using namespace oracle;

extern "C" {

typedef struct {
  int N;                      /* box edge (even power of two) */
  int B;                      /* spherical-harmonic bandwidth (nbfProjectionRotationMetric3D::B) */
  float mask_x, mask_y, mask_z, mask_sigma; /* nbfImageFilter::setMaskSize */
  float square_mask_size;     /* nbfImageFilter::squareMaskSize */
  float bp_low, bp_high, bp_low_sigma, bp_high_sigma; /* nbfFourierFilter::bandPassOn */
  float bfactor;              /* nbfFourierFilter::bfactorOn (0 = off) */
  float restrict_translation; /* nbfImageMetric::restrictTranslationSearch */
  float restrict_rotation;    /* nbfImageMetric::restrictRotationSearch */
  int candidate_peaks;        /* nbfProjectionRotationMetric3D::candidatePeaks */
  int number_of_candidates;   /* nbfCorrelationImageMetric::numberOfCandidates */
  int wedge_compensation;     /* useMissingWedgeCompensation */
  int overlap_normalized;     /* overlapNormalizedDistances */
  int mutual_correlation;     /* useMutualCorrelation */
  const float *reference_mask; /* referenceMask of the CCF when an external mask is set (oracle_file_mask's output,
                                  N^3 [x][y][z], z fastest), or NULL for the spherical mask */
} OracleParams;

typedef struct {
  const float *data;          /* fixed image, x fastest (MRC/VTK order) */
  int dims[3];
  float lwedge, uwedge;       /* nbfWedge3D */
  float normal[3];            /* Euler angles of nbfWedgedSubImage3D (degrees) */
  double matrix[16];          /* nbfWedgedSubImage3D::matrix (row major) */
  float position[3];
  float cut_offset;
  const float *spherical_wedge; /* explicit binary spherical wedge [2B][2B] (nbfWedge3D::setSphericalImage) or NULL */
} OracleVolume;

typedef struct {
  float distance;             /* getDistance() */
  double matrix[16];          /* getTransform() */
  int n_candidates;           /* entries stored in cand_* */
  float cand_distance[8];
  double cand_matrix[8][16];
  int n_ccf;                  /* CCF evaluations performed */
  int n_peaks_q1, n_peaks_q2; /* queue sizes after equivalent-angle elimination */
  int use_window1, use_window2;
  int best_cell[3];           /* SO(3) grid cell (alpha, beta, gamma indices) of the best rotation */
  float wedge_overlap;        /* getWedgeOverlap(getTransform()) */
} OracleResult;

} // extern "C"

namespace {

typedef std::array<float, 4> Vec4f;
struct GreaterPD {
  bool operator()(const Vec4f &x, const Vec4f &y) const { return x[3] > y[3]; }
};
typedef std::priority_queue<Vec4f, std::vector<Vec4f>, GreaterPD> PQ;

static const float kFmax = FLT_MAX;

/* ---------------------------------------------------------------- volumes and masks */

/* nbfWedge3D::set (inc/em/nbfWedge3D.h:142-184) */
struct Wedge {
  float lw, uw;
  double n1[3], n2[3];
  bool full() const { return uw - lw >= 180; }
};
Wedge make_wedge(float lw, float uw) {
  Wedge w;
  w.lw = lw < -90 ? -90.f : lw;
  w.uw = uw > 90 ? 90.f : uw;
  double a1 = (90.0 - w.uw) * 0.017453292519943295, a2 = (90.0 - w.lw) * 0.017453292519943295;
  w.n1[0] = cos(-a1); w.n1[1] = 0; w.n1[2] = -sin(-a1);
  w.n2[0] = cos(-a2); w.n2[1] = 0; w.n2[2] = -sin(-a2);
  return w;
}

/* Euler(normal) * matrix  (inc/em/nbfWedgedSubImage3D.h:741-751, 942-954) */
M4 local_matrix(const OracleVolume &v) {
  M4 e = m4_identity();
  m4_rotate_pre(e, -(double)v.normal[2], 0, 0, 1);
  m4_rotate_pre(e, -(double)v.normal[0], 1, 0, 0);
  m4_rotate_pre(e, -(double)v.normal[1], 0, 0, 1);
  M4 local;
  m4_mul(e.e, v.matrix, local.e);
  return local;
}

/* nbfWedgedSubImage3D::getImage (inc/em/nbfWedgedSubImage3D.h:602-828), fixed-image branch:
 * tricubic vtkImageReslice of the fixed image under Euler(normal)*matrix*t into an N^3 box,
 * background -FLT_MAX, float output, then mean of valid voxels subtracted, invalid set to 0.
 * out is [x][y][z] (z fastest). */
void get_image(const OracleVolume &v, int N, const M4 *t, std::vector<double> &out) {
  M4 local = local_matrix(v);
  M4 fin;
  if (t) m4_mul(local.e, t->e, fin.e); else fin = local;
  if (m4_det(fin.e) == 0) fin = m4_identity();
  double inM[16], outM[16];
  for (int i = 0; i < 16; ++i) inM[i] = outM[i] = (i % 5 == 0) ? 1.0 : 0.0;
  double outOrigin[3] = {-(double)(float)N / 2.0, -(double)(float)N / 2.0, -(double)(float)N / 2.0 - v.cut_offset};
  for (int i = 0; i < 3; ++i) {
    inM[4 * i + 3] = -(-(double)v.position[i]) / 1.0;
    outM[4 * i + 3] = outOrigin[i];
  }
  double tmp[16], idx[16];
  m4_mul(inM, fin.e, tmp);
  m4_mul(tmp, outM, idx);
  double origin[3], xA[3], yA[3], zA[3];
  for (int i = 0; i < 3; ++i) {
    xA[i] = idx[4 * i + 0]; yA[i] = idx[4 * i + 1]; zA[i] = idx[4 * i + 2]; origin[i] = idx[4 * i + 3];
  }
  long n3 = (long)N * N * N;
  std::vector<float> box(n3);
  const float lb = -FLT_MAX;
  for (int c = 0; c < N; ++c) {
    double p0[3] = {origin[0] + c * zA[0], origin[1] + c * zA[1], origin[2] + c * zA[2]};
    for (int b = 0; b < N; ++b) {
      double p1[3] = {p0[0] + b * yA[0], p0[1] + b * yA[1], p0[2] + b * yA[2]};
      for (int a = 0; a < N; ++a) {
        double p[3] = {p1[0] + a * xA[0], p1[1] + a * xA[1], p1[2] + a * xA[2]};
        bool in = true;
        for (int k = 0; k < 3; ++k)
          if (p[k] < -0.5 || p[k] > (v.dims[k] - 1) + 0.5) in = false;
        float val = in ? (float)vtk_tricubic_float(v.data, v.dims, p, false) : lb;
        box[((long)a * N + b) * N + c] = val;
      }
    }
  }
  double cnt = 0, sum = 0;
  for (long i = 0; i < n3; ++i)
    if ((double)box[i] > (double)lb) { cnt += 1; sum += box[i]; }
  float normalization = (float)cnt;
  float meanInside = (float)(sum / normalization);
  out.resize(n3);
  for (long i = 0; i < n3; ++i) out[i] = ((double)box[i] > (double)lb) ? (double)box[i] - (double)meanInside : 0.0;
}

/* nbfImageFilter::buildMask (inc/em/nbfImageFilter.h:383-472), spherical raised cosine branch */
void build_mask(const OracleParams &P, std::vector<float> &mask) {
  int N = P.N;
  mask.assign((long)N * N * N, 1.0f);
  if (P.mask_x == 0) return;
  if (!(P.mask_x == P.mask_y && P.mask_x == P.mask_z)) {
    fprintf(stderr, "oracle: only the spherical mask is restated\n");
    abort();
  }
  float center = (float)(N / 2.0);
  float r2 = std::min((float)(N - 1), (float)(P.mask_x + P.mask_sigma / 2.0));
  float r1 = (float)std::max(0.0, (double)(P.mask_x - P.mask_sigma / 2.0));
  float kappa = (float)(M_PI / (r2 - r1));
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < N; ++k) {
        float di = i - center, dj = j - center, dk = k - center;
        float m = sqrtf(di * di + dj * dj + dk * dk);
        if (m <= r1) m = 1;
        if (m >= r2) m = 0;
        if (m > r1 && m <= r2) m = (float)((1 + cosf(kappa * (m - r1))) / 2.0);
        mask[((long)i * N + j) * N + k] = m;
      }
}

/* m1 of the CCF: nbfFourierImageMetric::reinitializeHalf's referenceMask (inc/em/nbfFourierImageMetric.h:667-676),
 * the external mask when one is set, else the spherical mask of buildMask. */
void build_reference_mask(const OracleParams &P, std::vector<float> &mask) {
  if (P.reference_mask == nullptr) {
    build_mask(P, mask);
    return;
  }
  mask.assign(P.reference_mask, P.reference_mask + (long)P.N * P.N * P.N);
}

/* Gaussian-smooth a float array stored [x][y][z] (z fastest) with VTK semantics. */
void smooth_xyz(std::vector<float> &a, int nx, int ny, int nz, double std, double rf) {
  std::vector<float> t((long)nx * ny * nz);
  for (int x = 0; x < nx; ++x)
    for (int y = 0; y < ny; ++y)
      for (int z = 0; z < nz; ++z) t[x + (long)nx * (y + (long)ny * z)] = a[((long)x * ny + y) * nz + z];
  int dims[3] = {nx, ny, nz};
  vtk_gaussian_smooth_float(t.data(), dims, std, rf);
  for (int x = 0; x < nx; ++x)
    for (int y = 0; y < ny; ++y)
      for (int z = 0; z < nz; ++z) a[((long)x * ny + y) * nz + z] = t[x + (long)nx * (y + (long)ny * z)];
}

/* nbfFourierImageMetric::reinitializeHalf maskfft (inc/em/nbfFourierImageMetric.h:640-662) */
void build_maskfft(const OracleParams &P, std::vector<float> &mf) {
  int N = P.N;
  int size = (int)P.square_mask_size;
  mf.assign((long)N * N * N, 0.0f);
  if (size > 0 && size < floor(N / 2.0)) {
    for (int i = size; i <= N - 1 - size; ++i)
      for (int j = size; j <= N - 1 - size; ++j)
        for (int k = size; k <= N - 1 - size; ++k) mf[((long)i * N + j) * N + k] = 1;
  } else {
    std::fill(mf.begin(), mf.end(), 1.0f);
  }
  /* softenMask(maskfft, 2.5): std 2.5, radius factors 2.5*.75 (inc/em/nbfImageFilter.h:474-494) */
  smooth_xyz(mf, N, N, N, 2.5, (double)(2.5f * .75f));
}

/* nbfFourierFilter::updateFilterHalf + buildBandPassHalf + buildBFactorHalf
 * (inc/em/nbfFourierFilter.h:491-547, 737-797): half grid [N][N][N/2+1], centre (N/2,N/2,N/2). */
void build_filter(const OracleParams &P, std::vector<float> &f) {
  int N = P.N, H = N / 2 + 1;
  f.assign((long)N * N * H, 1.0f);
  int c = N / 2;
  f[((long)c * N + c) * H + (H - 1)] = 0;
  bool useBand = (P.bp_low > 0.0f) || (P.bp_high < 1.0f);
  double lo = P.bp_low, hi = P.bp_high, lv = P.bp_low_sigma, hv = P.bp_high_sigma;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < H; ++k) {
        float t0 = (float)((1.0 * i - c) / c), t1 = (float)((1.0 * j - c) / c), t2 = (float)((1.0 * k - c) / c);
        float radius = sqrtf(t0 * t0 + t1 * t1 + t2 * t2);
        long id = ((long)i * N + j) * H + k;
        if (useBand) {
          float bp = (radius < lo) ? (float)exp(-((lo - radius) * (lo - radius)) / 2.0 / lv / lv) : 1.0f;
          if (radius > hi) bp = (float)exp(-((radius - hi) * (radius - hi)) / 2.0 / hv / hv);
          f[id] *= bp;
        }
        if (P.bfactor != 0) f[id] *= (float)exp(-(double)P.bfactor * (double)(radius * radius));
      }
}

/* nbfWedge3D::getImageHalf (inc/em/nbfWedge3D.h:312-360) under nbfWedgedSubImage3D::getWedgeImageHalf
 * (inc/em/nbfWedgedSubImage3D.h:940-1003): normals rotated by inv(Euler*matrix*t), binary plane test on
 * the half grid centred at (N/2, N/2, N/2), Gaussian smooth with radius factors 0.5. */
void wedge_half(const OracleVolume &v, int N, const M4 *t, std::vector<float> &W) {
  int H = N / 2 + 1;
  Wedge w = make_wedge(v.lwedge, v.uwedge);
  W.assign((long)N * N * H, 1.0f);
  if (w.full()) return;
  M4 local = local_matrix(v), fin, inv;
  if (t) m4_mul(local.e, t->e, fin.e); else fin = local;
  if (!m4_invert(fin.e, inv.e)) inv = fin;
  double v1[3], v2[3];
  m4_transform_vector(inv.e, w.n1, v1);
  m4_transform_vector(inv.e, w.n2, v2);
  int c0 = N / 2, c1 = N / 2, c2 = H - 1;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < H; ++k) {
        double a = v1[0] * (i - c0) + v1[1] * (j - c1) + v1[2] * (k - c2);
        double b = v2[0] * (i - c0) + v2[1] * (j - c1) + v2[2] * (k - c2);
        W[((long)i * N + j) * H + k] = (a * b <= 0.0) ? 1.0f : 0.0f;
      }
  smooth_xyz(W, N, N, H, 2.0, 0.5);
}

/* nbfWedge3D::getSphericalImage (inc/em/nbfWedge3D.h:363-429) via
 * nbfWedgedSubImage3D::getSphericalWedgeImage (1006-1041), then conditionSphericalWindow
 * (inc/em/nbfProjectionRotationMetric3D.h:1321-1345). W is [2B][2B] (row = polar index). */
void spherical_wedge(const OracleVolume &v, int B, std::vector<float> &W) {
  int n = 2 * B;
  Wedge w = make_wedge(v.lwedge, v.uwedge);
  W.assign((long)n * n, 1.0f);
  if (v.spherical_wedge) {  /* an explicit image is returned as is (no transform: 363-375) */
    W.assign(v.spherical_wedge, v.spherical_wedge + (long)n * n);
  } else if (!w.full()) {
    M4 local = local_matrix(v), inv;
    if (!m4_invert(local.e, inv.e)) inv = local;
    double v1[3], v2[3];
    m4_transform_vector(inv.e, w.n1, v1);
    m4_transform_vector(inv.e, w.n2, v2);
    float phiK = (float)(M_PI / (n - 1));
    float thetaK = (float)(2.0 * M_PI / (n - 1));
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        float cj = cosf(j * thetaK), sj = sinf(j * thetaK), si = sinf(i * phiK), ci = cosf(i * phiK);
        double a = v1[0] * cj * si + v1[1] * sj * si + v1[2] * ci;
        double b = v2[0] * cj * si + v2[1] * sj * si + v2[2] * ci;
        W[(long)i * n + j] = (a * b <= 0.0) ? 1.0f : 0.0f;
      }
  }
  /* Gaussian std 2, radius factor 1 on VTK dims (2B, 2B, 1), x = polar index */
  smooth_xyz(W, n, n, 1, 2.0, 1.0);
}

/* ---------------------------------------------------------------- spherical projection */

/* nbfProjectionRotationMetric3D::cartesianToSpherical (inc/em/nbfProjectionRotationMetric3D.h:264-413) */
void cartesian_to_spherical(const OracleParams &P, const std::vector<float> &mask, std::vector<double> img,
                            std::vector<float> &Pp) {
  int N = P.N, B = P.B, N2 = 2 * N;
  long n3 = (long)N * N * N;
  /* window in real space: nbfImageFilter::execute (inc/em/nbfImageFilter.h:231-266) */
  double s = 0;
  for (long i = 0; i < n3; ++i) s += img[i];
  float meanValue = (float)(s / (double)n3);
  for (long i = 0; i < n3; ++i) img[i] = (img[i] - meanValue) * (double)mask[i] + meanValue;
  double padc = img[0];
  long m3 = (long)N2 * N2 * N2;
  std::vector<double> A(m3);
  for (int x = 0; x < N2; ++x)
    for (int y = 0; y < N2; ++y)
      for (int z = 0; z < N2; ++z)
        A[((long)x * N2 + y) * N2 + z] = (x < N && y < N && z < N) ? img[((long)x * N + y) * N + z] : padc;
  std::vector<double> Ash(m3);
  for (int x = 0; x < N2; ++x)
    for (int y = 0; y < N2; ++y)
      for (int z = 0; z < N2; ++z) {
        long id = ((long)x * N2 + y) * N2 + z;
        Ash[id] = A[id] * (((x + y + z) % 2) ? -1.0 : 1.0);
      }
  int H = N + 1;
  std::vector<cplx> F((long)N2 * N2 * H);
  rfft3d(Ash.data(), F.data(), N2, N2, N2);
  /* magnitude, Hermitian completion (lines 321-338); the z>N part of the y=0 plane keeps the padded data */
  std::vector<double> M(m3);
  for (int x = 0; x < N2; ++x)
    for (int y = 0; y < N2; ++y)
      for (int z = 0; z < N2; ++z) {
        long id = x + (long)N2 * (y + (long)N2 * z);
        if (z <= N) {
          cplx f = F[((long)x * N2 + y) * H + z];
          /* |F|, or with mutual correlation |F|^(1/2) (cartesianToSpherical, 318-322) */
          M[id] = P.mutual_correlation ? sqrt(sqrt((f * std::conj(f)).real())) : sqrt((f * std::conj(f)).real());
        } else {
          M[id] = A[((long)x * N2 + y) * N2 + z];
        }
      }
  for (int y = 0; y < N2; ++y)
    for (int z = 0; z < N2; ++z) M[0 + (long)N2 * (y + (long)N2 * z)] = 0;
  for (int i = -N + 1; i < N; ++i)
    for (int j = -N + 1; j < N; ++j)
      for (int k = 1; k < N; ++k)
        M[(N + i) + (long)N2 * ((N + j) + (long)N2 * (N + k))] = M[(N - i) + (long)N2 * ((N - j) + (long)N2 * (N - k))];
  /* vtkImageReslice through vtkSphericalTransform, cubic, wrap (lines 359-388) */
  int dims[3] = {N2, N2, N2};
  float lowCut = ((P.bp_low > 0) || (P.bp_high < 1)) ? P.bp_low : 0.0f;
  float highCut = ((P.bp_low > 0) || (P.bp_high < 1)) ? P.bp_high : 1.0f;
  int bandL = std::max(4, (int)ceilf(lowCut * (float)(N2 - 1)));
  int bandU = (int)ceil(std::min(.5, (double)highCut) * (N2 - 1));
  double oy = M_PI / 4.0 / (double)(float)B, sy = 2.0 * M_PI / 4.0 / (double)(float)B, sz = M_PI / (double)(float)B;
  double inOrigin = -(double)(N2 - 1) / 2.0 - 0.5;
  int n = 2 * B;
  Pp.assign((long)n * n, 0.0f);
  for (int tj = 0; tj < n; ++tj)
    for (int pk = 0; pk < n; ++pk) {
      double acc = 0;
      for (int r = bandL; r <= bandU; ++r) {
        double rr = 0.0 + r * 1.0;
        double ph = oy + tj * sy;
        double th = 0.0 + pk * sz;
        double q[3] = {rr * sin(ph) * cos(th), rr * sin(ph) * sin(th), rr * cos(ph)};
        double p[3] = {(q[0] - inOrigin) * 1.0, (q[1] - inOrigin) * 1.0, (q[2] - inOrigin) * 1.0};
        acc += vtk_tricubic_double(M.data(), dims, p, true);
      }
      Pp[(long)tj * n + pk] = (float)acc;
    }
}

/* ---------------------------------------------------------------- SO(3) stage */

/* nbfProjectionRotationMetric3D::softScaled (inc/em/nbfProjectionRotationMetric3D.h:1297-1319)
 * and rotatedSphericalImageMinMax (1557-1589). */
void soft_scaled(int B, const std::vector<double> &F1, const std::vector<double> &F2, std::vector<double> &C) {
  int n = 2 * B;
  long n3 = (long)n * n * n;
  C.resize(n3);
  so3_correlate(B, F1.data(), F2.data(), C.data());
  double maxV = -DBL_MAX, minV = DBL_MAX;
  long maxP = 0, minP = 0;
  for (long i = 0; i < n3; ++i) {
    if (C[i] > maxV) { maxV = C[i]; maxP = i; }
    if (C[i] < minV) { minV = C[i]; minP = i; }
  }
  auto angles = [&](long p, double &a, double &b, double &g) {
    int ia = p / ((long)n * n), ib = (p / n) % n, ig = p % n;
    a = (float)(ia / (double)B * M_PI);
    b = (float)((2 * ib + 1.0) / (4. * B) * M_PI);
    g = (float)(ig / (double)B * M_PI);
  };
  double a, b, g;
  std::vector<double> Rmin((long)n * n), Rmax((long)n * n);
  angles(minP, a, b, g);
  s2_rotate(B, F2.data(), a, b, g, Rmin.data());
  angles(maxP, a, b, g);
  s2_rotate(B, F2.data(), a, b, g, Rmax.data());
  double wMin = 0, wMax = 0;
  for (int i = 0; i < n; ++i) {
    double th = sin(M_PI * (2 * i + 1) / 4 / (double)(float)B);
    for (int j = 0; j < n; ++j) {
      wMin += F1[(long)i * n + j] * Rmin[(long)i * n + j] * th;
      wMax += F1[(long)i * n + j] * Rmax[(long)i * n + j] * th;
    }
  }
  for (long i = 0; i < n3; ++i) C[i] = (C[i] - minV) / (maxV - minV) * (wMax - wMin) + wMin;
}

/* nbfImageMetric::isTransformValid (inc/em/nbfImageMetric.h:415-459) */
bool is_transform_valid(const OracleParams &P, const M4 &t) {
  double sh[3] = {t.e[3], t.e[7], t.e[11]};
  if (fabs(sh[0]) > P.restrict_translation || fabs(sh[1]) > P.restrict_translation || fabs(sh[2]) > P.restrict_translation)
    return false;
  double pin[3] = {0, 0, 1}, pout[3];
  for (int i = 0; i < 3; ++i) pout[i] = t.e[4 * i + 0] * pin[0] + t.e[4 * i + 1] * pin[1] + t.e[4 * i + 2] * pin[2] + t.e[4 * i + 3];
  for (int i = 0; i < 3; ++i) pout[i] -= sh[i];
  double d = sqrt(pout[0] * pout[0] + pout[1] * pout[1] + pout[2] * pout[2]);
  if (d != 0) for (int i = 0; i < 3; ++i) pout[i] /= d;
  double angle = pin[0] * pout[0] + pin[1] * pout[1] + pin[2] * pout[2];
  if (angle >= 1) angle = 0;
  else angle = fabs(acos(angle) * 57.29577951308232);
  return angle <= P.restrict_rotation;
}

/* nbfProjectionRotationMetric3D::eliminateEquivalentAngles (1636-1702) */
void eliminate_equivalent(std::vector<Vec4f> &pos, PQ &pq, float tol) {
  std::vector<M4> mats(pos.size());
  for (size_t i = 0; i < pos.size(); ++i) mats[i] = m4_euler_zyz_neg(pos[i][0], pos[i][1], pos[i][2]);
  for (size_t i = 0; i < pos.size(); ++i) {
    for (size_t j = 0; j < pos.size(); ++j) {
      if (pos[i][3] == -kFmax) break;
      if (i != j && pos[j][3] > -kFmax) {
        double err = 0;
        for (int m = 0; m < 16; ++m) err += fabs(mats[i].e[m] - mats[j].e[m]);
        if (err < tol) {
          if (pos[i][3] > pos[j][3]) pos[i][3] = -kFmax;
          else pos[j][3] = -kFmax;
        }
      }
    }
  }
  for (size_t i = 0; i < pos.size(); ++i)
    if (pos[i][3] > -kFmax) pq.push(pos[i]);
}

/* restriction (602), -max border (605), 3x3x3 >= local maxima (610, stencil 67-79),
 * getTrueLocalMaximaPositions (1592-1634) */
int peaks_to_queue(const OracleParams &P, std::vector<double> &C, PQ &pq) {
  int B = P.B, n = 2 * B;
  double rs = floor((double)(P.restrict_rotation * (float)B) / 90.0 - 1.0);
  int start = (int)std::max(1.0, std::min(rs, (double)(n - 1)));
  for (int a = 0; a < n; ++a)
    for (int b = start; b < n; ++b)
      for (int g = 0; g < n; ++g) C[((long)a * n + b) * n + g] = -(double)kFmax;
  std::vector<Vec4f> pos;
  auto at = [&](int a, int b, int g) -> double {
    if (a < 0 || b < 0 || g < 0 || a >= n || b >= n || g >= n) return -(double)kFmax;
    return C[((long)a * n + b) * n + g];
  };
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < n; ++b)
      for (int g = 0; g < n; ++g) {
        double v = C[((long)a * n + b) * n + g];
        bool ismax = true;
        for (int da = -1; da <= 1 && ismax; ++da)
          for (int db = -1; db <= 1 && ismax; ++db)
            for (int dg = -1; dg <= 1; ++dg) {
              if (!da && !db && !dg) continue;
              if (!(v >= at(a + da, b + db, g + dg))) { ismax = false; break; }
            }
        double c2 = ismax ? v : 0.0;
        if (fabs(c2) > 0) {
          float alpha = (float)(a / (double)B * 180.0);
          float beta = (float)((2 * b + 1.0) / (4. * B) * 180.0);
          if ((float)B <= 32) beta = (float)((2 * b + 0.0) / (4. * B) * 180.0);
          float gamma = (float)(g / (double)B * 180.0);
          M4 t = m4_euler_zyz_neg(alpha, beta, gamma);
          if (is_transform_valid(P, t)) pos.push_back(Vec4f{alpha, beta, gamma, (float)(-c2)});
        }
      }
  eliminate_equivalent(pos, pq, 0.25f);
  return (int)pq.size();
}

/* ---------------------------------------------------------------- translational CCF */

/* normalizeFourierHalf (inc/em/nbfCorrelationImageMetric.h:497-530): DC zeroed, norm = float(2 * sum |F|^2 over
 * kz < H-1), then float(sqrt((norm + sum over kz = H-1) / (N N 2 (H-1)))), F /= norm. F is [N][N][H]. */
float normalize_half(int N, cplx *F) {
  const int H = N / 2 + 1;
  F[((long)(N / 2) * N + N / 2) * H + (H - 1)] = 0;
  double s1 = 0, s2 = 0;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < H; ++k) {
        cplx f = F[((long)i * N + j) * H + k];
        double m = (f * std::conj(f)).real();
        if (k < H - 1) s1 += m; else s2 += m;
      }
  float norm = (float)(2 * s1);
  norm = (float)sqrt((norm + s2) / (1.0 * N * N * 2 * (H - 1)));
  const long h3 = (long)N * N * H;
  for (long i = 0; i < h3; ++i) F[i] /= (double)norm;
  return norm;
}

/* The distance of executeFourierNewHalf (inc/em/nbfFourierImageMetric.h:1249-1258): the peak (double expression)
 * stored in the float correlationPeak, then divided twice in float by the int size (2N)^3 of the upsampled grid. */
float ccf_distance(float k1_m, double maxT, double sum_wf, double sum_f, bool overlap, int N) {
  const double peak = overlap ? std::max(0.0, (double)k1_m - maxT) / sum_wf * sum_f : std::max(0.0, (double)k1_m - maxT);
  float cp = (float)peak;
  const int big = 8 * N * N * N;
  cp = cp / (float)big;
  cp = cp / (float)big;
  return cp;
}


struct CCF {
  const OracleParams &P;
  const OracleVolume &ref, &part;
  std::vector<float> mask, maskfft, filter, wedge1;
  std::vector<double> I1;
  double sumFilter = 0;
  int ncalls = 0;

  CCF(const OracleParams &p, const OracleVolume &r, const OracleVolume &q) : P(p), ref(r), part(q) {
    build_reference_mask(P, mask);
    build_maskfft(P, maskfft);
    build_filter(P, filter);
    for (float f : filter) sumFilter += f;
    get_image(ref, P.N, nullptr, I1);
    wedge_half(ref, P.N, nullptr, wedge1);
  }

  float normalize(std::vector<cplx> &F) { return normalize_half(P.N, F.data()); }

  /* executeFourierNewHalf (inc/em/nbfFourierImageMetric.h:1077-1323); t is updated in place */
  float execute(M4 &t) {
    ++ncalls;
    int N = P.N, H = N / 2 + 1;
    long n3 = (long)N * N * N, h3 = (long)N * N * H;
    std::vector<float> w2;
    std::vector<float> wedge;
    bool useWedge = P.wedge_compensation != 0;
    if (useWedge) {
      wedge_half(part, N, &t, w2);
      wedge.resize(h3);
      for (long i = 0; i < h3; ++i) wedge[i] = w2[i] * wedge1[i];
    }
    auto shift = [&](int i, int j, int k) { return ((i + j + k) % 2) ? -1.0 : 1.0; };
    auto apply_filter = [&](std::vector<cplx> &F) {
      /* nbfFourierFilter::executeHalf (inc/em/nbfFourierFilter.h:586-606): with mutual correlation F / |F|^(1/2)
       * where |F| > 0, then the filter (times the wedge) */
      if (P.mutual_correlation)
        for (long i = 0; i < h3; ++i) {
          const double C = pow((F[i] * std::conj(F[i])).real(), .25);
          if (C > 0) F[i] /= C;
        }
      for (long i = 0; i < h3; ++i) {
        float fw = useWedge ? filter[i] * wedge[i] : filter[i];
        F[i] *= (double)fw;
      }
    };
    std::vector<double> R(n3);
    std::vector<cplx> F(h3), FFT1re, FFT2re;
    /* I1 */
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < N; ++k) {
          long id = ((long)i * N + j) * N + k;
          R[id] = I1[id] * (double)maskfft[id] * shift(i, j, k);
        }
    rfft3d(R.data(), F.data(), N, N, N);
    apply_filter(F);
    normalize(F);
    irfft3d(F.data(), R.data(), N, N, N);
    double s = 0;
    for (long i = 0; i < n3; ++i) s += R[i] * R[i] * (double)mask[i];
    float k1_m = (float)s;
    for (long i = 0; i < n3; ++i) R[i] *= (double)mask[i];
    rfft3d(R.data(), F.data(), N, N, N);
    FFT1re = F;
    /* I2 under t */
    std::vector<double> I2;
    get_image(part, N, &t, I2);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < N; ++k) {
          long id = ((long)i * N + j) * N + k;
          R[id] = I2[id] * (double)maskfft[id] * shift(i, j, k);
        }
    rfft3d(R.data(), F.data(), N, N, N);
    apply_filter(F);
    normalize(F);
    double normf = (double)n3;
    FFT2re.resize(h3);
    for (long i = 0; i < h3; ++i) FFT2re[i] = 2.0 * FFT1re[i] * std::conj(F[i] * normf);
    irfft3d(F.data(), R.data(), N, N, N);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < N; ++k) {
          long id = ((long)i * N + j) * N + k;
          R[id] = R[id] * R[id] * shift(i, j, k);
        }
    rfft3d(R.data(), F.data(), N, N, N);
    FFT1re = F;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < N; ++k) {
          long id = ((long)i * N + j) * N + k;
          R[id] = (double)(float)(mask[id] * (float)shift(i, j, k));
        }
    rfft3d(R.data(), F.data(), N, N, N);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < H; ++k) {
          long id = ((long)i * N + j) * H + k;
          F[id] = (-F[id] * std::conj(FFT1re[id]) + FFT2re[id]) * shift(i, j, k);
        }
    /* zero-pad into the (2N)^3 half spectrum x8 and invert */
    int N2 = 2 * N, H2 = N + 1;
    double factor = (1.0 * N2 * N2 * 2 * (H2 - 1)) / (1.0 * N * N * 2 * (H - 1));
    std::vector<cplx> Fb((long)N2 * N2 * H2, cplx(0, 0));
    int o0 = N - (int)floor(N / 2.0), o2 = H - 1;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        for (int k = 0; k < H; ++k)
          Fb[((long)(o0 + i) * N2 + (o0 + j)) * H2 + (o2 + k)] = F[((long)i * N + j) * H + k] * factor;
    std::vector<double> Rb((long)N2 * N2 * N2);
    irfft3d(Fb.data(), Rb.data(), N2, N2, N2);
    /* restricted peak search (1216-1264) */
    float center = (float)(N2 / 2.0);
    float restriction = center;
    if (P.restrict_translation < FLT_MAX) restriction = (float)std::max((double)P.restrict_translation * 2.0f, 1.0);
    int lo = (int)std::max(0.0, (double)center - floor(restriction));
    int hi = (int)std::min((double)center + floor(restriction), (double)(N2 - 1));
    int ext = hi - lo + 1;
    double big = (double)N2 * N2 * N2;
    double best = -DBL_MAX;
    int bi = 0, bj = 0, bk = 0;
    int half = (ext - 1) / 2;
    for (int i = 0; i < ext; ++i)
      for (int j = 0; j < ext; ++j)
        for (int k = 0; k < ext; ++k) {
          int gi = lo + i, gj = lo + j, gk = lo + k;
          double T = Rb[((long)gi * N2 + gj) * N2 + gk] * (double)(float)shift(gi, gj, gk) / big;
          float radius = (float)((half - i) * (half - i) + (half - j) * (half - j) + (half - k) * (half - k));
          if (!(radius < restriction * restriction)) T = -DBL_MAX;
          if (T > best) { best = T; bi = i; bj = j; bk = k; }
        }
    double sw = 0;
    if (P.overlap_normalized && useWedge)
      for (long i = 0; i < h3; ++i) sw += (double)(wedge[i] * filter[i]);
    float correlationPeak = ccf_distance(k1_m, best, sw, sumFilter, P.overlap_normalized && useWedge, N);
    float sh[3] = {(float)((bi - (ext - 1) / 2.0) / 2.0f), (float)((bj - (ext - 1) / 2.0) / 2.0f),
                   (float)((bk - (ext - 1) / 2.0) / 2.0f)};
    double tr[16];
    for (int i = 0; i < 16; ++i) tr[i] = (i % 5 == 0) ? 1.0 : 0.0;
    if (!(sh[0] == 0 && sh[1] == 0 && sh[2] == 0)) {
      tr[3] = -(double)sh[0]; tr[7] = -(double)sh[1]; tr[11] = -(double)sh[2];
    }
    M4 res;
    m4_mul(t.e, tr, res.e);
    t = res;
    return correlationPeak;
  }
};

float wedge_overlap(const OracleParams &P, const OracleVolume &ref, const OracleVolume &part, const M4 &t);

/* nbfProjectionRotationMetric3D::execute (inc/em/nbfProjectionRotationMetric3D.h:415-907),
 * alignment_mode 3 (refinement off). */
void align(const OracleParams &P, const OracleVolume &ref, const OracleVolume &part, OracleResult &res) {
  int N = P.N, B = P.B, n = 2 * B;
  memset(&res, 0, sizeof(res));
  std::vector<float> mask;
  build_mask(P, mask);
  std::vector<double> I1, I2;
  get_image(ref, N, nullptr, I1);
  get_image(part, N, nullptr, I2);
  std::vector<float> Pp1, Pp2;
  cartesian_to_spherical(P, mask, I1, Pp1);
  cartesian_to_spherical(P, mask, I2, Pp2);
  float M1 = *std::max_element(Pp1.begin(), Pp1.end()), M2 = *std::max_element(Pp2.begin(), Pp2.end());
  float M = std::max(M1, M2);
  for (auto &p : Pp1) p = p / M;
  for (auto &p : Pp2) p = p / M;
  long nn = (long)n * n;
  std::vector<float> W1, W2;
  bool useW1 = false, useW2 = false;
  if (P.wedge_compensation) {
    spherical_wedge(ref, B, W1);
    spherical_wedge(part, B, W2);
    double s1 = 0, s2 = 0;
    for (long i = 0; i < nn; ++i) { s1 += W1[i]; s2 += W2[i]; }
    float thr = .95f * (float)nn;
    useW1 = s1 <= thr;
    useW2 = s2 <= thr;
  } else {
    W1 = Pp1;
    W2 = Pp2;
  }
  res.use_window1 = useW1;
  res.use_window2 = useW2;
  std::vector<double> F1(nn), F2(nn), C1, C2;
  auto fill = [&](std::vector<double> &F, auto fn) { for (long i = 0; i < nn; ++i) F[i] = (double)fn(i); };
  if (useW1 && useW2) {
    fill(F1, [&](long i) { return Pp1[i] * Pp1[i] * W1[i]; });
    fill(F2, [&](long i) { return W2[i]; });
    soft_scaled(B, F1, F2, C1);
    fill(F1, [&](long i) { return W1[i]; });
    fill(F2, [&](long i) { return Pp2[i] * Pp2[i] * W2[i]; });
    soft_scaled(B, F1, F2, C2);
    for (size_t i = 0; i < C1.size(); ++i) C1[i] = sqrt(C1[i]) * sqrt(C2[i]);
    fill(F1, [&](long i) { return Pp1[i] * W1[i]; });
    fill(F2, [&](long i) { return Pp2[i] * W2[i]; });
    soft_scaled(B, F1, F2, C2);
    for (size_t i = 0; i < C1.size(); ++i) C1[i] = 2.0 * (1.0 - C2[i] / C1[i]);
    fill(F1, [&](long i) { return W1[i]; });
    fill(F2, [&](long i) { return W2[i]; });
    soft_scaled(B, F1, F2, C2);
    for (size_t i = 0; i < C1.size(); ++i) C1[i] = -C1[i] / C2[i];
  } else if (useW1) {
    fill(F1, [&](long i) { return W1[i]; });
    fill(F2, [&](long i) { return Pp2[i] * Pp2[i]; });
    soft_scaled(B, F1, F2, C2);
    fill(F1, [&](long i) { return W1[i] * Pp1[i]; });
    fill(F2, [&](long i) { return Pp2[i]; });
    soft_scaled(B, F1, F2, C1);
    for (size_t i = 0; i < C1.size(); ++i) C1[i] = C1[i] / sqrt(C2[i]);
  } else if (useW2) {
    fill(F1, [&](long i) { return Pp1[i] * Pp1[i]; });
    fill(F2, [&](long i) { return W2[i]; });
    soft_scaled(B, F1, F2, C2);
    fill(F1, [&](long i) { return Pp1[i]; });
    fill(F2, [&](long i) { return W2[i] * Pp2[i]; });
    soft_scaled(B, F1, F2, C1);
    for (size_t i = 0; i < C1.size(); ++i) C1[i] = C1[i] / sqrt(C2[i]);
  } else {
    fill(F1, [&](long i) { return Pp1[i]; });
    fill(F2, [&](long i) { return Pp2[i]; });
    C1.resize((long)n * n * n);
    so3_correlate(B, F1.data(), F2.data(), C1.data());
  }
  PQ pq1, pq2;
  res.n_peaks_q1 = peaks_to_queue(P, C1, pq1);
  if (useW1 || useW2) {
    fill(F1, [&](long i) { return Pp1[i]; });
    fill(F2, [&](long i) { return Pp2[i]; });
    C2.resize((long)n * n * n);
    so3_correlate(B, F1.data(), F2.data(), C2.data());
    res.n_peaks_q2 = peaks_to_queue(P, C2, pq2);
  }
  CCF ccf(P, ref, part);
  int nq = (useW1 || useW2) ? 2 : 1;
  std::vector<Vec4f> combined;
  for (int q = 0; q < nq; ++q) {
    PQ &cur = q == 0 ? pq1 : pq2;
    int index = 0;
    int peaks = P.candidate_peaks;
    if (q == 1) peaks = (int)std::max(1.0, floor(P.candidate_peaks / 3.0));
    while (index < peaks && cur.size() > 0) {
      Vec4f p = cur.top();
      if (p[3] == kFmax) break;
      float alpha = p[0], beta = p[1], gamma = p[2];
      M4 t1 = m4_euler_zyz_neg(alpha, beta, gamma);
      M4 td = t1;
      float currentD = ccf.execute(td);
      if (is_transform_valid(P, td)) {
        M4 mirror;
        for (int i = 0; i < 16; ++i) mirror.e[i] = t1.e[i];
        double S[16];
        for (int i = 0; i < 16; ++i) S[i] = (i % 5 == 0) ? ((i == 15) ? 1.0 : -1.0) : 0.0;
        m4_mul(S, t1.e, mirror.e);
        float mirrorD = ccf.execute(mirror);
        if (mirrorD >= currentD) index++;
        combined.push_back(Vec4f{alpha, beta, gamma, currentD});
      }
      cur.pop();
    }
  }
  if (combined.empty()) combined.push_back(Vec4f{0, 0, 0, 1.0f});
  PQ pqc;
  eliminate_equivalent(combined, pqc, 2.5f);
  float bestDistance = FLT_MAX;
  M4 bestT = m4_identity();
  int index = 0;
  while (pqc.size() > 0 && index < P.number_of_candidates) {
    Vec4f p = pqc.top();
    M4 t = m4_euler_zyz_neg(p[0], p[1], p[2]);
    float d = ccf.execute(t);   /* refine(t, 0): one CCF at the seed rotation */
    if (d < bestDistance) {
      bestDistance = d;
      bestT = t;
      res.best_cell[0] = (int)lround(p[0] / 180.0 * B);
      res.best_cell[1] = ((float)B <= 32) ? (int)lround(p[1] / 180.0 * 4.0 * B / 2.0)
                                          : (int)lround((p[1] / 180.0 * 4.0 * B - 1.0) / 2.0);
      res.best_cell[2] = (int)lround(p[2] / 180.0 * B);
    }
    if (index < 8) {
      res.cand_distance[index] = d;
      memcpy(res.cand_matrix[index], t.e, sizeof(t.e));
    }
    pqc.pop();
    ++index;
  }
  res.n_candidates = std::min(index, 8);
  res.distance = bestDistance;
  memcpy(res.matrix, bestT.e, sizeof(bestT.e));
  res.n_ccf = ccf.ncalls;
  res.wedge_overlap = wedge_overlap(P, ref, part, bestT);
}

/* nbfCorrelationImageMetric::getWedgeOverlap (inc/em/nbfCorrelationImageMetric.h:532-565): the half-spectrum
 * wedges of the sides whose wedge is effective (nbfWedge3D::isEffective, inc/em/nbfWedge3D.h:70: limits other
 * than (-90, 90)), the particle's under t, summed as float(float(w1 w2) filter) in double over the
 * updateFilterHalf filter and divided by the filter's sum; 1 when neither wedge is effective. */
float wedge_overlap(const OracleParams &P, const OracleVolume &ref, const OracleVolume &part, const M4 &t) {
  const bool e1 = !make_wedge(ref.lwedge, ref.uwedge).full(), e2 = !make_wedge(part.lwedge, part.uwedge).full();
  if (!e1 && !e2) return 1.0f;
  std::vector<float> w1, w2, filter;
  if (e1) wedge_half(ref, P.N, nullptr, w1);
  if (e2) wedge_half(part, P.N, &t, w2);
  build_filter(P, filter);
  double num = 0, den = 0;
  for (size_t i = 0; i < filter.size(); ++i) {
    float w = e1 && e2 ? w1[i] * w2[i] : (e1 ? w1[i] : w2[i]);
    num += (double)(w * filter[i]);
    den += (double)filter[i];
  }
  return (float)(num / den);
}

/* nbfWedgedAverageImage3D::getImageMPI + getImage with NBF_AVERAGE_IN_RECIPROCAL_SPACE
 * (inc/em/nbfWedgedAverageImage3D.h:216-258, 260-356): every member with weight w != 0 is resliced
 * under Euler(normal) * alignment (its own matrix reset to identity, line 313), transformed (R2C of
 * image * shift), and accumulated acc += |w||F|, re += w|F|Re F, im += w|F|Im F; the average is
 * IFFT((re, im)/acc where acc > 0, DC = 0) * shift / N^3, divided by its RMS. out is [x][y][z]. */
void average(const OracleParams &P, int M, const OracleVolume *vols, const float *weights, const double *mats,
             std::vector<double> &out) {
  int N = P.N, H = N / 2 + 1;
  long n3 = (long)N * N * N, h3 = (long)N * N * H;
  std::vector<double> re(h3, 0.0), im(h3, 0.0), acc(h3, 0.0), R(n3);
  std::vector<cplx> F(h3);
  for (int i = 0; i < M; ++i) {
    if (!(fabs(weights[i]) > 0)) continue;
    OracleVolume v = vols[i];
    for (int k = 0; k < 16; ++k) v.matrix[k] = (k % 5 == 0) ? 1.0 : 0.0;
    M4 t;
    memcpy(t.e, mats + 16 * (long)i, sizeof(t.e));
    std::vector<double> img;
    get_image(v, N, &t, img);
    for (int x = 0; x < N; ++x)
      for (int y = 0; y < N; ++y)
        for (int z = 0; z < N; ++z) {
          long id = ((long)x * N + y) * N + z;
          R[id] = img[id] * (double)(float)(((x + y + z) % 2) ? -1.0f : 1.0f);
        }
    rfft3d(R.data(), F.data(), N, N, N);
    double w = weights[i];
    for (long k = 0; k < h3; ++k) {
      double b = sqrt((F[k] * std::conj(F[k])).real());
      acc[k] += fabs(w) * b;
      re[k] += w * b * F[k].real();
      im[k] += w * b * F[k].imag();
    }
  }
  for (long k = 0; k < h3; ++k) F[k] = (acc[k] > 0) ? cplx(re[k] / acc[k], im[k] / acc[k]) : cplx(0, 0);
  F[((long)(N / 2) * N + N / 2) * H + (H - 1)] = 0;
  irfft3d(F.data(), R.data(), N, N, N);
  out.resize(n3);
  double ss = 0;
  for (int x = 0; x < N; ++x)
    for (int y = 0; y < N; ++y)
      for (int z = 0; z < N; ++z) {
        long id = ((long)x * N + y) * N + z;
        out[id] = R[id] / (double)n3 * (double)(float)(((x + y + z) % 2) ? -1.0f : 1.0f);
        ss += out[id] * out[id];
      }
  float rms = (float)sqrt(ss / (double)n3);
  for (auto &o : out) o /= (double)rms;
}

} // namespace

extern "C" {

int oracle_align(const OracleParams *P, const OracleVolume *ref, const OracleVolume *part, OracleResult *out) {
  align(*P, *ref, *part, *out);
  return 0;
}

/* Debug entry points for staged parity checks. */
int oracle_get_image(const OracleParams *P, const OracleVolume *v, const double *t16, double *out) {
  std::vector<double> img;
  M4 t;
  if (t16) memcpy(t.e, t16, sizeof(t.e));
  get_image(*v, P->N, t16 ? &t : nullptr, img);
  memcpy(out, img.data(), sizeof(double) * img.size());
  return 0;
}

int oracle_spherical_projection(const OracleParams *P, const OracleVolume *v, float *Pp) {
  std::vector<float> mask, pp;
  build_mask(*P, mask);
  std::vector<double> img;
  get_image(*v, P->N, nullptr, img);
  cartesian_to_spherical(*P, mask, img, pp);
  memcpy(Pp, pp.data(), sizeof(float) * pp.size());
  return 0;
}

int oracle_spherical_wedge(const OracleParams *P, const OracleVolume *v, float *W) {
  std::vector<float> w;
  spherical_wedge(*v, P->B, w);
  memcpy(W, w.data(), sizeof(float) * w.size());
  return 0;
}

int oracle_wedge_half(const OracleParams *P, const OracleVolume *v, const double *t16, float *W) {
  std::vector<float> w;
  M4 t;
  if (t16) memcpy(t.e, t16, sizeof(t.e));
  wedge_half(*v, P->N, t16 ? &t : nullptr, w);
  memcpy(W, w.data(), sizeof(float) * w.size());
  return 0;
}

/* nbfImageFilter::buildMaskFromFile (inc/em/nbfImageFilter.h:319-381) on a mask volume already read from its file:
 * M^3 floats, x fastest (the MRC reader's VTK order, x = first Blitz index). A mask of another edge is centred into
 * a zero N^3 box (N > M + 1) or cropped from its centre (the reference's integer offsets); then binarised
 * (> threshold) and softened (softenMask with the filter's sigma: Gaussian std sigma, radius factor 0.75 sigma).
 * out: N^3 [x][y][z]. Returns 0, or -1 where the reference would index outside the mask (M = N - 1). */
int oracle_file_mask(const OracleParams *P, int M, const float *mask, float threshold, float *out) {
  const int N = P->N;
  std::vector<float> A((long)M * M * M);
  for (int x = 0; x < M; ++x)
    for (int y = 0; y < M; ++y)
      for (int z = 0; z < M; ++z) A[((long)x * M + y) * M + z] = mask[x + (long)M * (y + (long)M * z)];
  std::vector<float> Bx((long)N * N * N, 0.0f);
  if (M == N) {
    Bx = A;
  } else {
    const int diff = (int)((N - M) / 2.0);
    if (diff > 0) {
      const int o = N / 2 + 1 - M / 2 - 1;
      for (int x = 0; x < M; ++x)
        for (int y = 0; y < M; ++y)
          for (int z = 0; z < M; ++z) Bx[((long)(o + x) * N + (o + y)) * N + (o + z)] = A[((long)x * M + y) * M + z];
    } else {
      const int o = M / 2 + 1 - N / 2 - 1;
      if (o < 0 || o + N > M) return -1;
      for (int x = 0; x < N; ++x)
        for (int y = 0; y < N; ++y)
          for (int z = 0; z < N; ++z) Bx[((long)x * N + y) * N + z] = A[((long)(o + x) * M + (o + y)) * M + (o + z)];
    }
  }
  for (float &v : Bx) v = v > threshold ? 1.0f : 0.0f;
  const float s = P->mask_sigma;
  if (s > 0) smooth_xyz(Bx, N, N, N, (double)s, (double)s * .75);
  memcpy(out, Bx.data(), sizeof(float) * Bx.size());
  return 0;
}

int oracle_masks(const OracleParams *P, float *mask, float *maskfft, float *filter) {
  std::vector<float> a, b, c;
  build_mask(*P, a);
  build_maskfft(*P, b);
  build_filter(*P, c);
  if (mask) memcpy(mask, a.data(), sizeof(float) * a.size());
  if (maskfft) memcpy(maskfft, b.data(), sizeof(float) * b.size());
  if (filter) memcpy(filter, c.data(), sizeof(float) * c.size());
  return 0;
}

int oracle_soft(int B, const double *F1, const double *F2, double *C) {
  so3_correlate(B, F1, F2, C);
  return 0;
}

int oracle_soft_scaled(int B, const double *F1, const double *F2, double *C) {
  int n = 2 * B;
  std::vector<double> a(F1, F1 + (long)n * n), b(F2, F2 + (long)n * n), c;
  soft_scaled(B, a, b, c);
  memcpy(C, c.data(), sizeof(double) * c.size());
  return 0;
}

int oracle_rotate(int B, const double *F, double a, double b, double g, double *R) {
  s2_rotate(B, F, a, b, g, R);
  return 0;
}

int oracle_sht(int B, const double *F, double *coefRI /* [B][2B][2] */) {
  std::vector<cplx> c;
  sht_forward_real(B, F, c);
  for (size_t i = 0; i < c.size(); ++i) { coefRI[2 * i] = c[i].real(); coefRI[2 * i + 1] = c[i].imag(); }
  return 0;
}

/* One executeFourierNewHalf call at transform t16 (updated in place); returns the CCF distance. */
float oracle_ccf(const OracleParams *P, const OracleVolume *ref, const OracleVolume *part, double *t16) {
  CCF ccf(*P, *ref, *part);
  M4 t;
  memcpy(t.e, t16, sizeof(t.e));
  float d = ccf.execute(t);
  memcpy(t16, t.e, sizeof(t.e));
  return d;
}

/* Objective of the continuous pose refinement (no counterpart in the reference; the GPU's refine.cuh states
 * it), restated in FP64 for its gradient check: the particle resliced by the index map of t perturbed on the
 * right by exp([w]x) about the box centre and the shift d (theta = w[3], d[3]), clamped tricubic everywhere;
 * u = (r - mu) m1 shift with mu = sum(m1 r) / sum(m1); g = C2R(R2C(u) fw), y1 = C2R(R2C(I1 maskfft shift) fw)
 * with fw = wedge1 * wedge2(t) * filter and the DC zeroed (executeFourierNewHalf's I1 branch); returns
 * rho = sum(m1 y1 g) / sqrt(sum(m1 y1^2) sum(m1 g^2)). */
double oracle_refine_objective(const OracleParams *P, const OracleVolume *ref, const OracleVolume *part,
                               const double *t16, const double *theta) {
  CCF ccf(*P, *ref, *part);
  const int N = P->N, H = N / 2 + 1;
  const long n3 = (long)N * N * N, h3 = (long)N * N * H;
  M4 t;
  memcpy(t.e, t16, sizeof(t.e));
  std::vector<double> fw(h3);
  {
    std::vector<float> w2;
    if (P->wedge_compensation) wedge_half(*part, N, &t, w2);
    for (long i = 0; i < h3; ++i) fw[i] = P->wedge_compensation ? (double)(ccf.filter[i] * (w2[i] * ccf.wedge1[i]))
                                                                 : (double)ccf.filter[i];
    fw[((long)(N / 2) * N + N / 2) * H + (H - 1)] = 0;
  }
  auto shift = [&](long id) {
    const int i = (int)(id / ((long)N * N)), j = (int)((id / N) % N), k = (int)(id % N);
    return ((i + j + k) % 2) ? -1.0 : 1.0;
  };
  auto filt = [&](std::vector<double> &R) {
    std::vector<cplx> F(h3);
    rfft3d(R.data(), F.data(), N, N, N);
    for (long i = 0; i < h3; ++i) F[i] *= fw[i];
    irfft3d(F.data(), R.data(), N, N, N);
  };
  std::vector<double> y1(n3), g(n3);
  for (long id = 0; id < n3; ++id) y1[id] = ccf.I1[id] * (double)ccf.maskfft[id] * shift(id);
  filt(y1);
  /* index map of t (reslice_index), perturbed */
  M4 local = local_matrix(*part), fin;
  m4_mul(local.e, t.e, fin.e);
  if (m4_det(fin.e) == 0) fin = m4_identity();
  double inM[16], outM[16], tmp[16], idx[16];
  for (int i = 0; i < 16; ++i) inM[i] = outM[i] = (i % 5 == 0) ? 1.0 : 0.0;
  for (int i = 0; i < 3; ++i) {
    inM[4 * i + 3] = (double)part->position[i];
    outM[4 * i + 3] = -(double)(float)N / 2.0 - (i == 2 ? part->cut_offset : 0.0);
  }
  m4_mul(inM, fin.e, tmp);
  m4_mul(tmp, outM, idx);
  const double *w = theta, *d = theta + 3;
  const double th = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (th > 0) {
    const double k[3] = {w[0] / th, w[1] / th, w[2] / th}, sn = sin(th), c1 = 1 - cos(th);
    const double K[9] = {0, -k[2], k[1], k[2], 0, -k[0], -k[1], k[0], 0};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double k2 = 0;
        for (int q = 0; q < 3; ++q) k2 += K[3 * i + q] * K[3 * q + j];
        R[3 * i + j] += sn * K[3 * i + j] + c1 * k2;
      }
  }
  const double c = 0.5 * N;
  double M[9], o[3], Mp[9], op[3], tv[3];
  for (int i = 0; i < 3; ++i) {
    o[i] = idx[4 * i + 3];
    for (int col = 0; col < 3; ++col) M[3 * i + col] = idx[4 * i + col];
  }
  for (int i = 0; i < 3; ++i) tv[i] = c - (R[3 * i] + R[3 * i + 1] + R[3 * i + 2]) * c + d[i];
  for (int i = 0; i < 3; ++i) {
    op[i] = o[i] + M[3 * i] * tv[0] + M[3 * i + 1] * tv[1] + M[3 * i + 2] * tv[2];
    for (int col = 0; col < 3; ++col) Mp[3 * i + col] = M[3 * i] * R[col] + M[3 * i + 1] * R[3 + col] + M[3 * i + 2] * R[6 + col];
  }
  std::vector<double> r(n3);
  double sw = 0, swr = 0;
  for (int a = 0; a < N; ++a)
    for (int b = 0; b < N; ++b)
      for (int cz = 0; cz < N; ++cz) {
        double p[3];
        for (int i = 0; i < 3; ++i) p[i] = ((op[i] + cz * Mp[3 * i + 2]) + b * Mp[3 * i + 1]) + a * Mp[3 * i];
        const long id = ((long)a * N + b) * N + cz;
        r[id] = vtk_tricubic_float(part->data, part->dims, p, false);
        sw += ccf.mask[id];
        swr += ccf.mask[id] * r[id];
      }
  const double mu = sw > 0 ? swr / sw : 0.0;
  for (long id = 0; id < n3; ++id) g[id] = (r[id] - mu) * (double)ccf.mask[id] * shift(id);
  filt(g);
  double syg = 0, sgg = 0, syy = 0;
  for (long id = 0; id < n3; ++id) {
    const double m = ccf.mask[id];
    syg += m * y1[id] * g[id];
    sgg += m * g[id] * g[id];
    syy += m * y1[id] * y1[id];
  }
  return (sgg > 0 && syy > 0) ? syg / sqrt(sgg * syy) : 0.0;
}

/* The fast form's local-refinement objective (no counterpart in the reference), restated in FP64 with its
 * analytic gradient for the checks of the GPU's: zm = m1 * y1, y1 = K(I1) = C2R(R2C(I1 maskfft shift) fw) shift
 * with fw = wedge1 * wedge2(t) * filter and the DC zeroed; the particle (a fixed image of edge N) band-passed in
 * its own frame, C2R(R2C(I shift) filter) shift, and sampled as I by trilinear interpolation at
 * the index map of t perturbed on the right by exp([w]x) about the box centre and the shift d (theta = w[3],
 * d[3]), coordinates clamped to the volume; mu = sum m1 I / sum m1; rho = sum zm (I - mu) /
 * sqrt(sum m1^2 (I - mu)^2 sum zm^2); grad = d rho / d(w, d) with dI/dd = G, dI/dw = (x - c) x G,
 * G = M^T grad_p I (zero along a clamped axis). Returns rho; grad (6) may be NULL. */
double oracle_refined_objective(const OracleParams *P, const OracleVolume *ref, const OracleVolume *part,
                                const double *t16, const double *theta, double *grad) {
  CCF ccf(*P, *ref, *part);
  const int N = P->N, H = N / 2 + 1;
  const long n3 = (long)N * N * N, h3 = (long)N * N * H;
  M4 t;
  memcpy(t.e, t16, sizeof(t.e));
  std::vector<double> fw(h3);
  {
    std::vector<float> w2;
    if (P->wedge_compensation) wedge_half(*part, N, &t, w2);
    for (long i = 0; i < h3; ++i) fw[i] = P->wedge_compensation ? (double)(ccf.filter[i] * (w2[i] * ccf.wedge1[i]))
                                                                 : (double)ccf.filter[i];
    fw[((long)(N / 2) * N + N / 2) * H + (H - 1)] = 0;
  }
  auto shift = [&](long id) {
    const int i = (int)(id / ((long)N * N)), j = (int)((id / N) % N), k = (int)(id % N);
    return ((i + j + k) % 2) ? -1.0 : 1.0;
  };
  std::vector<double> zm(n3);
  {
    std::vector<cplx> F(h3);
    for (long id = 0; id < n3; ++id) zm[id] = ccf.I1[id] * (double)ccf.maskfft[id] * shift(id);
    rfft3d(zm.data(), F.data(), N, N, N);
    for (long i = 0; i < h3; ++i) F[i] *= fw[i];
    irfft3d(F.data(), zm.data(), N, N, N);
    for (long id = 0; id < n3; ++id) zm[id] *= shift(id) * (double)ccf.mask[id];
  }
  /* index map of t (reslice_index), perturbed on the right */
  M4 local = local_matrix(*part), fin;
  m4_mul(local.e, t.e, fin.e);
  if (m4_det(fin.e) == 0) fin = m4_identity();
  double inM[16], outM[16], tmp[16], idx[16];
  for (int i = 0; i < 16; ++i) inM[i] = outM[i] = (i % 5 == 0) ? 1.0 : 0.0;
  for (int i = 0; i < 3; ++i) {
    inM[4 * i + 3] = (double)part->position[i];
    outM[4 * i + 3] = -(double)(float)N / 2.0 - (i == 2 ? part->cut_offset : 0.0);
  }
  m4_mul(inM, fin.e, tmp);
  m4_mul(tmp, outM, idx);
  const double *w = theta, *d = theta + 3;
  const double th = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (th > 0) {
    const double k[3] = {w[0] / th, w[1] / th, w[2] / th}, sn = sin(th), c1 = 1 - cos(th);
    const double K[9] = {0, -k[2], k[1], k[2], 0, -k[0], -k[1], k[0], 0};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double k2 = 0;
        for (int q = 0; q < 3; ++q) k2 += K[3 * i + q] * K[3 * q + j];
        R[3 * i + j] += sn * K[3 * i + j] + c1 * k2;
      }
  }
  const double c = 0.5 * N;
  double M[9], o[3], Mp[9], op[3], tv[3];
  for (int i = 0; i < 3; ++i) {
    o[i] = idx[4 * i + 3];
    for (int col = 0; col < 3; ++col) M[3 * i + col] = idx[4 * i + col];
  }
  for (int i = 0; i < 3; ++i) tv[i] = c - (R[3 * i] + R[3 * i + 1] + R[3 * i + 2]) * c + d[i];
  for (int i = 0; i < 3; ++i) {
    op[i] = o[i] + M[3 * i] * tv[0] + M[3 * i + 1] * tv[1] + M[3 * i + 2] * tv[2];
    for (int col = 0; col < 3; ++col) Mp[3 * i + col] = M[3 * i] * R[col] + M[3 * i + 1] * R[3 + col] + M[3 * i + 2] * R[6 + col];
  }
  const int dims[3] = {part->dims[0], part->dims[1], part->dims[2]};
  const long sy = dims[0], sz = (long)dims[0] * dims[1];
  /* the particle band-passed in its own frame (its N^3 fixed image, [z][y][x]) by the metric's filter */
  std::vector<double> ip((long)dims[0] * dims[1] * dims[2]);
  {
    std::vector<cplx> F(h3);
    for (long id = 0; id < n3; ++id) ip[id] = (double)part->data[id] * shift(id);
    rfft3d(ip.data(), F.data(), N, N, N);
    for (long i = 0; i < h3; ++i) F[i] *= (double)ccf.filter[i];
    irfft3d(F.data(), ip.data(), N, N, N);
    for (long id = 0; id < n3; ++id) ip[id] *= shift(id);
  }
  double S[4] = {0, 0, 0, 0}, T[4][6] = {{0}}, C0 = 0, C1 = 0, czm = 0, czz = 0;
  for (long id = 0; id < n3; ++id) {
    const double m = ccf.mask[id];
    C0 += m;
    C1 += m * m;
    czm += zm[id];
    czz += zm[id] * zm[id];
  }
  for (int a = 0; a < N; ++a)
    for (int b = 0; b < N; ++b)
      for (int cz = 0; cz < N; ++cz) {
        const long id = ((long)a * N + b) * N + cz;
        const double m = ccf.mask[id];
        if (m == 0) continue;
        double pp[3], q[3], f[3], gr[3];
        int i0[3];
        bool in[3];
        for (int i = 0; i < 3; ++i) {
          pp[i] = op[i] + a * Mp[3 * i] + b * Mp[3 * i + 1] + cz * Mp[3 * i + 2];
          const double hi = dims[i] - 1;
          q[i] = std::min(std::max(pp[i], 0.0), hi);
          in[i] = pp[i] > 0 && pp[i] < hi;
          i0[i] = std::min((int)q[i], dims[i] - 2);
          f[i] = q[i] - i0[i];
        }
        const double *base = ip.data() + i0[0] + i0[1] * sy + i0[2] * sz;
        double v[2][2][2];
        for (int z = 0; z < 2; ++z)
          for (int y = 0; y < 2; ++y)
            for (int x = 0; x < 2; ++x) v[z][y][x] = base[x + y * sy + z * sz];
        double I = 0;
        gr[0] = gr[1] = gr[2] = 0;
        for (int z = 0; z < 2; ++z)
          for (int y = 0; y < 2; ++y)
            for (int x = 0; x < 2; ++x) {
              const double wx = x ? f[0] : 1 - f[0], wy = y ? f[1] : 1 - f[1], wz = z ? f[2] : 1 - f[2];
              const double sx = x ? 1 : -1, sy_ = y ? 1 : -1, sz_ = z ? 1 : -1;
              I += wx * wy * wz * v[z][y][x];
              gr[0] += sx * wy * wz * v[z][y][x];
              gr[1] += wx * sy_ * wz * v[z][y][x];
              gr[2] += wx * wy * sz_ * v[z][y][x];
            }
        for (int i = 0; i < 3; ++i)
          if (!in[i]) gr[i] = 0;
        double G[3];
        for (int col = 0; col < 3; ++col) G[col] = Mp[col] * gr[0] + Mp[3 + col] * gr[1] + Mp[6 + col] * gr[2];
        const double r[3] = {a - c, b - c, cz - c};
        const double Dk[6] = {r[1] * G[2] - r[2] * G[1], r[2] * G[0] - r[0] * G[2], r[0] * G[1] - r[1] * G[0],
                              G[0], G[1], G[2]};
        const double z = zm[id];
        S[0] += m * I;
        S[1] += m * m * I;
        S[2] += m * m * I * I;
        S[3] += z * I;
        for (int k = 0; k < 6; ++k) {
          T[0][k] += m * Dk[k];
          T[1][k] += m * m * Dk[k];
          T[2][k] += m * m * I * Dk[k];
          T[3][k] += z * Dk[k];
        }
      }
  const double mu = S[0] / C0;
  const double num = S[3] - mu * czm;
  const double den2 = S[2] - 2.0 * mu * S[1] + mu * mu * C1;
  if (!(den2 > 0) || !(czz > 0)) {
    if (grad)
      for (int k = 0; k < 6; ++k) grad[k] = 0;
    return 0;
  }
  const double den = sqrt(den2 * czz), rho = num / den;
  if (grad)
    for (int k = 0; k < 6; ++k) {
      const double dmu = T[0][k] / C0;
      const double dnum = T[3][k] - dmu * czm;
      const double dden2 = 2.0 * T[2][k] - 2.0 * dmu * S[1] - 2.0 * mu * T[1][k] + 2.0 * mu * dmu * C1;
      grad[k] = dnum / den - 0.5 * rho * dden2 / den2;
    }
  return rho;
}

/* nbfImageFilter::symmetrize (inc/em/nbfImageFilter.h:527-554): the mean over i < fold of getImage of the
 * volume as a fixed image (position dims/2, identity matrix, no normal) under RotateZ(i * 360 / fold), each a
 * tricubic reslice with the mean of its valid voxels removed and invalid voxels zero (inc/em/nbfWedgedAverageImage3D.h
 * 252-257 then inc/em/nbfWedgedSubImage3D.h:602-828). fold <= 1 returns the volume unchanged. out [x][y][z]. */
int oracle_symmetrize(const OracleParams *P, const OracleVolume *v, int fold, double *out) {
  const int N = P->N;
  const long n3 = (long)N * N * N;
  if (fold <= 1) {
    for (int x = 0; x < N; ++x)
      for (int y = 0; y < N; ++y)
        for (int z = 0; z < N; ++z) out[((long)x * N + y) * N + z] = (double)v->data[x + (long)N * (y + (long)N * z)];
    return 0;
  }
  std::vector<double> acc(n3, 0.0), img;
  for (int i = 0; i < fold; ++i) {
    M4 t = m4_identity();
    m4_rotate_pre(t, i * 360.0 / fold, 0, 0, 1);
    get_image(*v, N, &t, img);
    for (long k = 0; k < n3; ++k) acc[k] += img[k];
  }
  for (long k = 0; k < n3; ++k) out[k] = acc[k] / fold;
  return 0;
}

/* nbfFourierImageMetric::getLowDimensionRepresentationHalf (inc/em/nbfFourierImageMetric.h:1967-2034) with
 * padding 1 (imageFilter->execute(input1, true) then bypasses the mask): A = getImage of the volume; with
 * fold > 1 nbfImageFilter::symmetrize(A, fold) (oracle_symmetrize of A as a fixed image, A stored as float) and
 * wedge bits 1; F = R2C(A * shift) * filter (executeHalf without a wedge), a = C2R(F) * mask, F2 = R2C(a),
 * unnormalised; the kept coefficients are those with |filter| > 0.5 in the [x][y][kz] order of the half
 * spectrum, stored as complex<float> beside the wedge bit getWedgeImageHalf > 0.5. R (optional): K x 3 floats;
 * *K their number. */
int oracle_representation(const OracleParams *P, const OracleVolume *v, int fold, float *R, int *K) {
  const int N = P->N, H = N / 2 + 1;
  const long n3 = (long)N * N * N, h3 = (long)N * N * H;
  std::vector<double> a;
  get_image(*v, N, nullptr, a);
  if (fold > 1) {
    std::vector<float> fx(n3);
    for (int x = 0; x < N; ++x)
      for (int y = 0; y < N; ++y)
        for (int z = 0; z < N; ++z) fx[x + (long)N * (y + (long)N * z)] = (float)a[((long)x * N + y) * N + z];
    OracleVolume fv;
    memset(&fv, 0, sizeof(fv));
    fv.data = fx.data();
    fv.dims[0] = fv.dims[1] = fv.dims[2] = N;
    fv.lwedge = -90.f;
    fv.uwedge = 90.f;
    for (int k = 0; k < 16; ++k) fv.matrix[k] = (k % 5 == 0) ? 1.0 : 0.0;
    for (int k = 0; k < 3; ++k) fv.position[k] = (float)(N / 2.0);
    oracle_symmetrize(P, &fv, fold, a.data());
  }
  for (int x = 0; x < N; ++x)
    for (int y = 0; y < N; ++y)
      for (int z = 0; z < N; ++z)
        if ((x + y + z) & 1) a[((long)x * N + y) * N + z] *= -1.0;
  std::vector<float> f, mask, w;
  build_filter(*P, f);
  build_mask(*P, mask);
  wedge_half(*v, N, nullptr, w);
  std::vector<cplx> F(h3);
  rfft3d(a.data(), F.data(), N, N, N);
  for (long i = 0; i < h3; ++i) F[i] *= (double)f[i];
  irfft3d(F.data(), a.data(), N, N, N);
  for (long i = 0; i < n3; ++i) a[i] *= (double)mask[i];
  rfft3d(a.data(), F.data(), N, N, N);
  int k = 0;
  for (long g = 0; g < h3; ++g)
    if (fabs(f[g]) > 0.5) {
      if (R) {
        R[3L * k] = (float)F[g].real();
        R[3L * k + 1] = (float)F[g].imag();
        R[3L * k + 2] = (fold > 1 || w[g] > .5) ? 1.0f : 0.0f;
      }
      ++k;
    }
  *K = k;
  return 0;
}

/* nbfFourierImageMetric::getLowDimensionRepresentationReal (inc/em/nbfFourierImageMetric.h:2375-2533) with no mask
 * file (the image filter's own mask):
 *  - fold > 1 (2377-2439): A = the wedged average of the one volume under the fold alignments matrix * RotateZ(f * 360
 *    / fold) (vtkMatrix4x4::Multiply4x4(matrix, rotation)), weights 1 / fold (float), as `average` computes it;
 *    otherwise A = getImage of the volume;
 *  - A = C2R(filter * R2C(A * shift)) * shift / N^3 (nbfFourierFilter::executeHalf on a real array,
 *    inc/em/nbfFourierFilter.h:654-672);
 *  - fold > 1: nbfImageFilter::symmetrize(A, fold) (A cast to float as a fixed image, as oracle_representation);
 *  - binning by the integer factor bin (vtkImageResample with magnification 1 / bin, cubic: output extent
 *    [0, floor((N - 1) / bin)], sample i at input index bin * i, an integer position where the tricubic kernel reduces
 *    to the voxel itself), of A and of the mask alike;
 *  - the kept values are those where the (binned) mask exceeds 0.5, in the [x][y][z] order of the array.
 * C (optional): K doubles; *K their number. */
int oracle_representation_real(const OracleParams *P, const OracleVolume *v, int fold, int bin, double *C, int *K) {
  const int N = P->N, H = N / 2 + 1;
  const long n3 = (long)N * N * N, h3 = (long)N * N * H;
  if (bin < 1) return 1;
  std::vector<double> a;
  if (fold > 1) {
    std::vector<OracleVolume> vols(fold, *v);
    std::vector<float> w(fold, 1.0f / (float)fold);
    std::vector<double> mats(16L * fold);
    for (int f = 0; f < fold; ++f) {
      M4 t = m4_identity();
      m4_rotate_pre(t, f * 360.0 / fold, 0, 0, 1);
      m4_mul(v->matrix, t.e, mats.data() + 16L * f);
    }
    average(*P, fold, vols.data(), w.data(), mats.data(), a);
  } else {
    get_image(*v, N, nullptr, a);
  }
  auto shift = [&](long id) {
    const long x = id / ((long)N * N), y = (id / N) % N, z = id % N;
    return ((x + y + z) & 1) ? -1.0 : 1.0;
  };
  for (long i = 0; i < n3; ++i) a[i] *= shift(i);
  std::vector<float> f, mask;
  build_filter(*P, f);
  build_mask(*P, mask);
  std::vector<cplx> F(h3);
  rfft3d(a.data(), F.data(), N, N, N);
  for (long i = 0; i < h3; ++i) F[i] *= (double)f[i];
  irfft3d(F.data(), a.data(), N, N, N);
  for (long i = 0; i < n3; ++i) a[i] = a[i] * shift(i) / (double)n3;
  if (fold > 1) {
    std::vector<float> fx(n3);
    for (int x = 0; x < N; ++x)
      for (int y = 0; y < N; ++y)
        for (int z = 0; z < N; ++z) fx[x + (long)N * (y + (long)N * z)] = (float)a[((long)x * N + y) * N + z];
    OracleVolume fv;
    memset(&fv, 0, sizeof(fv));
    fv.data = fx.data();
    fv.dims[0] = fv.dims[1] = fv.dims[2] = N;
    fv.lwedge = -90.f;
    fv.uwedge = 90.f;
    for (int k = 0; k < 16; ++k) fv.matrix[k] = (k % 5 == 0) ? 1.0 : 0.0;
    for (int k = 0; k < 3; ++k) fv.position[k] = (float)(N / 2.0);
    oracle_symmetrize(P, &fv, fold, a.data());
  }
  const int nb = (N - 1) / bin + 1;
  int k = 0;
  for (int x = 0; x < nb; ++x)
    for (int y = 0; y < nb; ++y)
      for (int z = 0; z < nb; ++z) {
        const long id = ((long)x * bin * N + (long)y * bin) * N + (long)z * bin;
        if (mask[id] > .5) {
          if (C) C[k] = a[id];
          ++k;
        }
      }
  *K = k;
  return 0;
}

/* nbfCorrelationImageMetric::getDistances(representationFile, D) (inc/em/nbfCorrelationImageMetric.h:1726-1871),
 * single-process branch, with Blitz 0.9's types: complex<float> products and differences, sum() of a float
 * expression accumulated in double, mean() in float, Pixel overlap stored as float. R(V, K, depth) C order;
 * D (V*V) zero diagonal, symmetric. */
int oracle_representation_distances(int V, int K, int depth, const float *R, int normalized, float *D) {
  for (long k = 0; k < (long)V * V; ++k) D[k] = 0;
  for (int i = 0; i < V; ++i)
    for (int j = i + 1; j < V; ++j) {
      float d;
      if (depth == 1) {
        double s = 0;
        for (int k = 1; k < K; ++k) {
          float e = R[(long)i * K + k] - R[(long)j * K + k];
          s += (double)(e * e);
        }
        d = (float)sqrt(s);
      } else {
        double s = 0, ov = 0;
        float sf = 0;
        for (int k = 0; k < K; ++k) {
          const float *a = R + ((long)i * K + k) * 3, *b = R + ((long)j * K + k) * 3;
          float w1 = a[2], w2 = b[2];
          float r1 = a[0] * w1 * w2, i1 = a[1] * w1 * w2, r2 = b[0] * w1 * w2, i2 = b[1] * w1 * w2;
          float dr = r1 - r2, di = i1 - i2;
          float t = dr * dr + di * di;
          s += t;
          sf += t;
          ov += (double)(w1 * w2);
        }
        float overlap = (float)ov;
        d = (normalized && overlap > 0) ? (float)(s / overlap) : sf / K;
      }
      D[(long)i * V + j] = d;
      D[(long)j * V + i] = d;
    }
  return 0;
}

/* Spherical wedge of a class average: nbfWedgedAverageImage3D::updateAccumulatedSphericalWedgeImageMPI
 * (inc/em/nbfWedgedAverageImage3D.h:612-648) sums, over members with |w| > 0 (matrix reset by setTransform(NULL)),
 * the binary analytic wedge of nbfWedge3D::getSphericalImage (inc/em/nbfWedge3D.h:363-429) under
 * inv(Euler(normal) * alignment) (nbfWedgedSubImage3D::getSphericalWedgeImage, inc/em/nbfWedgedSubImage3D.h:1007-1041),
 * in float; updateSphericalWedgeImage (650-665) keeps accum > max(accum) / 2. count and wedge [2B][2B]. */
int oracle_average_spherical_wedge(const OracleParams *P, int M, const OracleVolume *vols, const float *weights,
                                   const double *mats, float *count, float *wedge) {
  const int B = P->B, n = 2 * B;
  const long nn = (long)n * n;
  std::vector<float> acc(nn, 0.0f);
  for (int m = 0; m < M; ++m) {
    if (!(fabsf(weights[m]) > 0)) continue;
    OracleVolume v = vols[m];
    for (int k = 0; k < 16; ++k) v.matrix[k] = (k % 5 == 0) ? 1.0 : 0.0;
    Wedge w = make_wedge(v.lwedge, v.uwedge);
    if (w.full()) {
      for (long k = 0; k < nn; ++k) acc[k] += 1.0f;
      continue;
    }
    M4 t, fin, inv;
    memcpy(t.e, mats + 16 * (long)m, sizeof(t.e));
    M4 local = local_matrix(v);
    m4_mul(local.e, t.e, fin.e);
    if (!m4_invert(fin.e, inv.e)) inv = fin;
    double v1[3], v2[3];
    m4_transform_vector(inv.e, w.n1, v1);
    m4_transform_vector(inv.e, w.n2, v2);
    float phiK = (float)(M_PI / (n - 1));
    float thetaK = (float)(2.0 * M_PI / (n - 1));
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        float cj = cosf(j * thetaK), sj = sinf(j * thetaK), si = sinf(i * phiK), ci = cosf(i * phiK);
        double a = v1[0] * cj * si + v1[1] * sj * si + v1[2] * ci;
        double b = v2[0] * cj * si + v2[1] * sj * si + v2[2] * ci;
        acc[(long)i * n + j] += (a * b <= 0.0) ? 1.0f : 0.0f;
      }
  }
  float mx = *std::max_element(acc.begin(), acc.end());
  for (long k = 0; k < nn; ++k) {
    if (count) count[k] = acc[k];
    wedge[k] = (acc[k] > mx / 2.0) ? 1.0f : 0.0f;
  }
  return 0;
}

/* Clamped trilinear interpolation of nbfLinearInterpolator::interpolateSingle (inc/nbfLinearInterpolator.h:186-262)
 * along one axis of extent n: a coordinate at or below 0 takes cell 0 with weight 0, one at or above n-1 takes
 * cell n-2 with weight 1, others floor and fraction. */
static double cyl_axis(double x, int n, int *f) {
  if (x <= 0) {
    *f = 0;
    return 0.0;
  }
  if (x >= n - 1) {
    *f = n - 2;
    return 1.0;
  }
  *f = (int)floor(x);
  return x - *f;
}

/* The eight-term blend of interpolateSingle in its order; v[dx][dy][dz]. */
static double cyl_blend(double a, double b, double c, const double v[2][2][2]) {
  return (1 - a) * (1 - b) * (1 - c) * v[0][0][0] + a * (1 - b) * (1 - c) * v[1][0][0] +
         (1 - a) * b * (1 - c) * v[0][1][0] + (1 - a) * (1 - b) * c * v[0][0][1] + a * (1 - b) * c * v[1][0][1] +
         (1 - a) * b * c * v[0][1][1] + a * b * (1 - c) * v[1][1][0] + a * b * c * v[1][1][1];
}

/* Rotational symmetrisation of the classification loop (src/MPI_Classification.cpp:1005-1024) with
 * nbfCylindricalDomain3 (inc/nbfCylindricalDomain3.h:126-233): the volume (x fastest) sampled on a cylinder
 * about the z axis through (N/2, N/2): N/2 radii rho_i = (N/2)/(N/2-1) i, 180 angles theta_j = 2 pi_f / 179 j
 * (pi_f = the float pi of VTK 5.10's vtkMath::Pi, both ends included) and every z plane, by the clamped
 * trilinear interpolation above; the samples summed over the angles in order (a sum, not a mean); the
 * (radius, z) profile interpolated back at each voxel's radius (N/2-1) r / (N/2) and angle (the angle weight
 * multiplies equal values). FP64; out [x][y][z]. */
int oracle_symmetrize_rotational(int N, const float *vol, double *out) {
  if (N < 4 || (N & 1)) return 1;
  const int R = N / 2, T = 180;
  const double c = (double)(N / 2), max_rho = (double)(N / 2), two_pi = 2.0 * (double)3.14159265358979f;
  const double max_theta = (double)(2 * 3.14159265358979f);
  const double rstep = (max_rho - 0) / (R - 1), tstep = (max_theta - 0) / (T - 1);
  std::vector<double> prof((size_t)R * N);
  auto A = [&](int x, int y, int z) { return (double)vol[x + (long)N * (y + (long)N * z)]; };
  for (int i = 0; i < R; ++i)
    for (int k = 0; k < N; ++k) {
      double s = 0;
      for (int j = 0; j < T; ++j) {
        const double rho = rstep * i + 0.0, theta = tstep * j + 0.0;
        const double X = c + rho * cos(theta), Y = c + rho * sin(theta), Z = (double)k;
        int xf, yf, zf;
        const double a = cyl_axis(X, N, &xf), b = cyl_axis(Y, N, &yf), cc = cyl_axis(Z, N, &zf);
        double v[2][2][2];
        for (int dx = 0; dx < 2; ++dx)
          for (int dy = 0; dy < 2; ++dy)
            for (int dz = 0; dz < 2; ++dz) v[dx][dy][dz] = A(xf + dx, yf + dy, zf + dz);
        s += cyl_blend(a, b, cc, v);
      }
      prof[(size_t)i * N + k] = s;
    }
  for (int x = 0; x < N; ++x)
    for (int y = 0; y < N; ++y) {
      double r = sqrt((c - x) * (c - x) + (c - y) * (c - y));
      r = (r - 0) / (max_rho - 0) * (R - 1);
      double t = atan2(y - c, x - c);
      if (t < 0) t = t + two_pi;
      t = t / max_theta * (T - 1);
      int rf, tf;
      const double a = cyl_axis(r, R, &rf), b = cyl_axis(t, T, &tf);
      for (int z = 0; z < N; ++z) {
        int zf;
        const double cc = cyl_axis((double)z, N, &zf);
        double v[2][2][2];
        for (int dx = 0; dx < 2; ++dx)
          for (int dy = 0; dy < 2; ++dy)
            for (int dz = 0; dz < 2; ++dz) v[dx][dy][dz] = prof[(size_t)(rf + dx) * N + zf + dz];
        out[((long)x * N + y) * N + z] = cyl_blend(a, b, cc, v);
      }
    }
  return 0;
}

/* nbfWedgedAverageImage3D::getImageVarianceMPI (inc/em/nbfWedgedAverageImage3D.h:440-493): sum over members with
 * w != 0 of |w| (T - average)^2 / sum |w|, T = getImage of the member under its alignment with its own matrix
 * reset (as the average). average and out [x][y][z]. */
int oracle_variance(const OracleParams *P, int M, const OracleVolume *vols, const float *weights, const double *mats,
                    const double *avg, double *out) {
  const int N = P->N;
  const long n3 = (long)N * N * N;
  double sw = 0;
  for (int i = 0; i < M; ++i) sw += fabs((double)weights[i]);
  for (long k = 0; k < n3; ++k) out[k] = 0;
  std::vector<double> img;
  for (int i = 0; i < M; ++i) {
    if (!(fabs(weights[i]) > 0)) continue;
    OracleVolume v = vols[i];
    for (int k = 0; k < 16; ++k) v.matrix[k] = (k % 5 == 0) ? 1.0 : 0.0;
    M4 t;
    memcpy(t.e, mats + 16 * (long)i, sizeof(t.e));
    get_image(v, N, &t, img);
    const double aw = fabs((double)weights[i]);
    for (long k = 0; k < n3; ++k) {
      const double d = img[k] - avg[k];
      out[k] += aw * (d * d) / sw;
    }
  }
  return 0;
}

/* Class average of M members (volumes + metadata, weights, 4x4 alignment matrices); out [x][y][z]. */
int oracle_average(const OracleParams *P, int M, const OracleVolume *vols, const float *weights, const double *mats,
                   double *out) {
  std::vector<double> a;
  average(*P, M, vols, weights, mats, a);
  memcpy(out, a.data(), sizeof(double) * a.size());
  return 0;
}

float oracle_wedge_overlap(const OracleParams *P, const OracleVolume *ref, const OracleVolume *part, const double *t16) {
  M4 t;
  memcpy(t.e, t16, sizeof(t.e));
  return wedge_overlap(*P, *ref, *part, t);
}

int oracle_normalize_half(int N, double *FRI, float *norm) {
  *norm = normalize_half(N, reinterpret_cast<cplx *>(FRI));
  return 0;
}

float oracle_ccf_distance(float k1_m, double maxT, double sum_wf, double sum_f, int overlap, int N) {
  return ccf_distance(k1_m, maxT, sum_wf, sum_f, overlap != 0, N);
}

int oracle_rfft3d(int n0, int n1, int n2, const double *in, double *outRI) {
  rfft3d(in, reinterpret_cast<cplx *>(outRI), n0, n1, n2);
  return 0;
}
int oracle_irfft3d(int n0, int n1, int n2, const double *inRI, double *out) {
  irfft3d(reinterpret_cast<const cplx *>(inRI), out, n0, n1, n2);
  return 0;
}

} // extern "C"
