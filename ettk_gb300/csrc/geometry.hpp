// Host-side geometry and table construction for the GB300 alignment library.
//
// Everything here is small per-volume or per-configuration arithmetic that the reference does
// with VTK objects in double precision; it runs once per pose/volume on the host and feeds the
// device kernels. Semantics follow the reference and VTK 5.10:
//   vtkTransform Rotate* (PreMultiply, quaternion matrix)     Common/vtkAbstractTransform.cxx:548-597
//   vtkMatrix4x4 Multiply4x4 / Invert (adjoint / determinant) Common/vtkMatrix4x4.cxx:106-286
//   nbfWedge3D::set plane normals                             inc/em/nbfWedge3D.h:142-184
//   Euler(normal) * matrix * t                                inc/em/nbfWedgedSubImage3D.h:741-763
//   reslice index matrix inMatrix * T * outMatrix             Imaging/vtkImageReslice.cxx:2935-3025
//   vtkImageGaussianSmooth (clipped renormalised kernels)     Imaging/vtkImageGaussianSmooth.cxx:67-93,249-358
#pragma once
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

namespace ettk {

struct Mat4 {
  double e[16];
  static Mat4 eye() {
    Mat4 m;
    for (int i = 0; i < 16; ++i) m.e[i] = (i % 5 == 0) ? 1.0 : 0.0;
    return m;
  }
};

inline Mat4 mul(const Mat4 &a, const Mat4 &b) {
  Mat4 c;
  for (int i = 0; i < 4; ++i)
    for (int k = 0; k < 4; ++k)
      c.e[4 * i + k] = a.e[4 * i] * b.e[k] + a.e[4 * i + 1] * b.e[4 + k] + a.e[4 * i + 2] * b.e[8 + k] +
                       a.e[4 * i + 3] * b.e[12 + k];
  return c;
}

// M <- M * R(angle degrees about axis), zero angle is a no-op.
inline void rotate(Mat4 &m, double angle, double x, double y, double z) {
  if (angle == 0.0 || (x == 0.0 && y == 0.0 && z == 0.0)) return;
  angle *= 0.017453292519943295;
  double w = cos(0.5 * angle), f = sin(0.5 * angle) / sqrt(x * x + y * y + z * z);
  x *= f;
  y *= f;
  z *= f;
  Mat4 r = Mat4::eye();
  double ww = w * w, wx = w * x, wy = w * y, wz = w * z, xx = x * x, yy = y * y, zz = z * z;
  double xy = x * y, xz = x * z, yz = y * z, s = ww - xx - yy - zz;
  r.e[0] = xx * 2 + s;
  r.e[4] = (xy + wz) * 2;
  r.e[8] = (xz - wy) * 2;
  r.e[1] = (xy - wz) * 2;
  r.e[5] = yy * 2 + s;
  r.e[9] = (yz + wx) * 2;
  r.e[2] = (xz + wy) * 2;
  r.e[6] = (yz - wx) * 2;
  r.e[10] = zz * 2 + s;
  m = mul(m, r);
}

// RotateZ(-gamma) RotateY(-beta) RotateZ(-alpha): the candidate pose of an SO(3) grid cell
// (inc/em/nbfProjectionRotationMetric3D.h:708-711).
inline Mat4 euler_candidate(double alpha, double beta, double gamma) {
  Mat4 m = Mat4::eye();
  rotate(m, -gamma, 0, 0, 1);
  rotate(m, -beta, 0, 1, 0);
  rotate(m, -alpha, 0, 0, 1);
  return m;
}

inline double d2(double a, double b, double c, double d) { return a * d - b * c; }
inline double d3(double a1, double a2, double a3, double b1, double b2, double b3, double c1, double c2, double c3) {
  return a1 * d2(b2, b3, c2, c3) - b1 * d2(a2, a3, c2, c3) + c1 * d2(a2, a3, b2, b3);
}
inline double det(const Mat4 &m) {
  const double *e = m.e;
  return e[0] * d3(e[5], e[9], e[13], e[6], e[10], e[14], e[7], e[11], e[15]) -
         e[1] * d3(e[4], e[8], e[12], e[6], e[10], e[14], e[7], e[11], e[15]) +
         e[2] * d3(e[4], e[8], e[12], e[5], e[9], e[13], e[7], e[11], e[15]) -
         e[3] * d3(e[4], e[8], e[12], e[5], e[9], e[13], e[6], e[10], e[14]);
}
// vtkMatrix4x4::Invert; returns false (matrix unchanged) when singular.
inline bool invert(const Mat4 &m, Mat4 &o) {
  double dt = det(m);
  if (dt == 0.0) return false;
  const double *e = m.e;
  double a1 = e[0], b1 = e[1], c1 = e[2], dd1 = e[3], a2 = e[4], b2 = e[5], c2 = e[6], dd2 = e[7];
  double a3 = e[8], b3 = e[9], c3 = e[10], dd3 = e[11], a4 = e[12], b4 = e[13], c4 = e[14], dd4 = e[15];
  double r[16];
  r[0] = d3(b2, b3, b4, c2, c3, c4, dd2, dd3, dd4);
  r[4] = -d3(a2, a3, a4, c2, c3, c4, dd2, dd3, dd4);
  r[8] = d3(a2, a3, a4, b2, b3, b4, dd2, dd3, dd4);
  r[12] = -d3(a2, a3, a4, b2, b3, b4, c2, c3, c4);
  r[1] = -d3(b1, b3, b4, c1, c3, c4, dd1, dd3, dd4);
  r[5] = d3(a1, a3, a4, c1, c3, c4, dd1, dd3, dd4);
  r[9] = -d3(a1, a3, a4, b1, b3, b4, dd1, dd3, dd4);
  r[13] = d3(a1, a3, a4, b1, b3, b4, c1, c3, c4);
  r[2] = d3(b1, b2, b4, c1, c2, c4, dd1, dd2, dd4);
  r[6] = -d3(a1, a2, a4, c1, c2, c4, dd1, dd2, dd4);
  r[10] = d3(a1, a2, a4, b1, b2, b4, dd1, dd2, dd4);
  r[14] = -d3(a1, a2, a4, b1, b2, b4, c1, c2, c4);
  r[3] = -d3(b1, b2, b3, c1, c2, c3, dd1, dd2, dd3);
  r[7] = d3(a1, a2, a3, c1, c2, c3, dd1, dd2, dd3);
  r[11] = -d3(a1, a2, a3, b1, b2, b3, dd1, dd2, dd3);
  r[15] = d3(a1, a2, a3, b1, b2, b3, c1, c2, c3);
  for (int i = 0; i < 16; ++i) o.e[i] = r[i] / dt;
  return true;
}

inline void xform_vec(const Mat4 &m, const double in[3], double out[3]) {
  double x = m.e[0] * in[0] + m.e[1] * in[1] + m.e[2] * in[2];
  double y = m.e[4] * in[0] + m.e[5] * in[1] + m.e[6] * in[2];
  double z = m.e[8] * in[0] + m.e[9] * in[1] + m.e[10] * in[2];
  out[0] = x;
  out[1] = y;
  out[2] = z;
}

struct VolumeGeom {
  float lwedge, uwedge, normal[3], position[3], cut_offset;
  double matrix[16];
  bool full_wedge() const {
    float lw = lwedge < -90 ? -90.f : lwedge, uw = uwedge > 90 ? 90.f : uwedge;
    return uw - lw >= 180;
  }
  void normals(double n1[3], double n2[3]) const {
    float lw = lwedge < -90 ? -90.f : lwedge, uw = uwedge > 90 ? 90.f : uwedge;
    double a1 = (90.0 - uw) * 0.017453292519943295, a2 = (90.0 - lw) * 0.017453292519943295;
    n1[0] = cos(-a1); n1[1] = 0; n1[2] = -sin(-a1);
    n2[0] = cos(-a2); n2[1] = 0; n2[2] = -sin(-a2);
  }
  Mat4 local() const {
    Mat4 e = Mat4::eye();
    rotate(e, -(double)normal[2], 0, 0, 1);
    rotate(e, -(double)normal[0], 1, 0, 0);
    rotate(e, -(double)normal[1], 0, 0, 1);
    Mat4 m;
    memcpy(m.e, matrix, sizeof(m.e));
    return mul(e, m);
  }
};

// Reslice index matrix (output box index -> fixed-image index) for Euler*matrix*t, as
// inMatrix * (final) * outMatrix. Returns origin, x/y/z axis columns (12 doubles).
inline void reslice_index(const VolumeGeom &g, int N, const Mat4 *t, double out12[12]) {
  Mat4 fin = t ? mul(g.local(), *t) : g.local();
  if (det(fin) == 0) fin = Mat4::eye();
  Mat4 inM = Mat4::eye(), outM = Mat4::eye();
  double oo[3] = {-(double)(float)N / 2.0, -(double)(float)N / 2.0, -(double)(float)N / 2.0 - g.cut_offset};
  for (int i = 0; i < 3; ++i) {
    inM.e[4 * i + 3] = (double)g.position[i];
    outM.e[4 * i + 3] = oo[i];
  }
  Mat4 idx = mul(mul(inM, fin), outM);
  for (int i = 0; i < 3; ++i) {
    out12[i] = idx.e[4 * i + 3];      // origin
    out12[3 + i] = idx.e[4 * i + 0];  // x axis
    out12[6 + i] = idx.e[4 * i + 1];  // y axis
    out12[9 + i] = idx.e[4 * i + 2];  // z axis
  }
}

// Inverse of reslice_index: the transform t whose index matrix is out12 (origin, x/y/z axis columns).
inline Mat4 pose_from_index(const VolumeGeom &g, int N, const double out12[12]) {
  Mat4 idx = Mat4::eye();
  for (int i = 0; i < 3; ++i) {
    idx.e[4 * i + 3] = out12[i];
    idx.e[4 * i + 0] = out12[3 + i];
    idx.e[4 * i + 1] = out12[6 + i];
    idx.e[4 * i + 2] = out12[9 + i];
  }
  Mat4 inM = Mat4::eye(), outM = Mat4::eye();
  double oo[3] = {-(double)(float)N / 2.0, -(double)(float)N / 2.0, -(double)(float)N / 2.0 - g.cut_offset};
  for (int i = 0; i < 3; ++i) {
    inM.e[4 * i + 3] = -(double)g.position[i];  // inverses of the two translations
    outM.e[4 * i + 3] = -oo[i];
  }
  Mat4 fin = mul(mul(inM, idx), outM), li;
  if (!invert(g.local(), li)) li = Mat4::eye();
  return mul(li, fin);
}

// Index map perturbed on the right by a rotation exp([w]x) about the box centre c = (N/2, N/2, N/2) and a shift d
// of the output grid: p'(x) = M (exp([w]x)(x - c) + c + d) + o, with M the axis columns of out12.
inline void perturb_index(const double in12[12], int N, const double w[3], const double d[3], double out12[12]) {
  const double th = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (th > 0) {  // Rodrigues
    const double k[3] = {w[0] / th, w[1] / th, w[2] / th}, s = sin(th), c1 = 1 - cos(th);
    const double K[9] = {0, -k[2], k[1], k[2], 0, -k[0], -k[1], k[0], 0};
    double K2[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) K2[3 * i + j] = K[3 * i] * K[j] + K[3 * i + 1] * K[3 + j] + K[3 * i + 2] * K[6 + j];
    for (int i = 0; i < 9; ++i) R[i] += s * K[i] + c1 * K2[i];
  }
  const double c = 0.5 * N;
  double M[9];  // M[3*i + col]
  for (int col = 0; col < 3; ++col)
    for (int i = 0; i < 3; ++i) M[3 * i + col] = in12[3 + 3 * col + i];
  double t[3];  // c - R c + d
  for (int i = 0; i < 3; ++i) t[i] = c - (R[3 * i] + R[3 * i + 1] + R[3 * i + 2]) * c + d[i];
  for (int i = 0; i < 3; ++i) {
    out12[i] = in12[i] + M[3 * i] * t[0] + M[3 * i + 1] * t[1] + M[3 * i + 2] * t[2];
    for (int col = 0; col < 3; ++col)
      out12[3 + 3 * col + i] = M[3 * i] * R[col] + M[3 * i + 1] * R[3 + col] + M[3 * i + 2] * R[6 + col];
  }
}

// Plane normals of the wedge rotated by inv(Euler*matrix*t) (nbfWedgedSubImage3D::getWedgeImageHalf).
inline void wedge_vectors(const VolumeGeom &g, const Mat4 *t, double v1[3], double v2[3]) {
  double n1[3], n2[3];
  g.normals(n1, n2);
  Mat4 fin = t ? mul(g.local(), *t) : g.local(), inv;
  if (!invert(fin, inv)) inv = fin;
  xform_vec(inv, n1, v1);
  xform_vec(inv, n2, v2);
}

// vtkImageGaussianSmooth on a float image with VTK dims (x fastest).
inline void gaussian_smooth(std::vector<float> &img, const int dims[3], double sd, double rf) {
  int radius = (int)(sd * rf);
  std::vector<float> a = img, b(img.size());
  long inc[3] = {1, dims[0], (long)dims[0] * dims[1]};
  for (int axis = 2; axis >= 0; --axis) {
    int n = dims[axis];
    std::vector<double> k(2 * radius + 1);
    int o0 = (axis + 1) % 3, o1 = (axis + 2) % 3;
    for (int p = 0; p < n; ++p) {
      int lo = std::max(0, p - radius), hi = std::min(n - 1, p + radius);
      double s = 0;
      for (int x = lo - p; x <= hi - p; ++x) s += k[x - (lo - p)] = exp(-((double)(x * x)) / (sd * sd * 2.0));
      for (int x = 0; x <= hi - lo; ++x) k[x] /= s;
      for (int i1 = 0; i1 < dims[o1]; ++i1)
        for (int i0 = 0; i0 < dims[o0]; ++i0) {
          long base = (long)i0 * inc[o0] + (long)i1 * inc[o1];
          double acc = 0;
          for (int q = lo; q <= hi; ++q) acc += k[q - lo] * (double)a[base + (long)q * inc[axis]];
          b[base + (long)p * inc[axis]] = (float)acc;
        }
    }
    std::swap(a, b);
  }
  img = a;
}

}  // namespace ettk
