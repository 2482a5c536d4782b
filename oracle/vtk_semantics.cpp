/* Oracle restatement of VTK 5.10 arithmetic (test infrastructure only). See
 * vtk_semantics.h for the VTK source locations each function follows. */
#include "vtk_semantics.h"
#include <cmath>
#include <cstring>

namespace oracle {

M4 m4_identity() {
  M4 m;
  for (int i = 0; i < 16; ++i) m.e[i] = (i % 5 == 0) ? 1.0 : 0.0;
  return m;
}

void m4_mul(const double a[16], const double b[16], double c[16]) {
  double acc[16];
  for (int i = 0; i < 4; ++i)
    for (int k = 0; k < 4; ++k)
      acc[4 * i + k] = a[4 * i + 0] * b[0 * 4 + k] + a[4 * i + 1] * b[1 * 4 + k] +
                       a[4 * i + 2] * b[2 * 4 + k] + a[4 * i + 3] * b[3 * 4 + k];
  memcpy(c, acc, sizeof(acc));
}

static inline double det2(double a, double b, double c, double d) { return a * d - b * c; }
static inline double det3(double a1, double a2, double a3, double b1, double b2, double b3,
                          double c1, double c2, double c3) {
  return a1 * det2(b2, b3, c2, c3) - b1 * det2(a2, a3, c2, c3) + c1 * det2(a2, a3, b2, b3);
}

double m4_det(const double e[16]) {
  double a1 = e[0], b1 = e[1], c1 = e[2], d1 = e[3];
  double a2 = e[4], b2 = e[5], c2 = e[6], d2 = e[7];
  double a3 = e[8], b3 = e[9], c3 = e[10], d3 = e[11];
  double a4 = e[12], b4 = e[13], c4 = e[14], d4 = e[15];
  return a1 * det3(b2, b3, b4, c2, c3, c4, d2, d3, d4) - b1 * det3(a2, a3, a4, c2, c3, c4, d2, d3, d4) +
         c1 * det3(a2, a3, a4, b2, b3, b4, d2, d3, d4) - d1 * det3(a2, a3, a4, b2, b3, b4, c2, c3, c4);
}

bool m4_invert(const double in[16], double out[16]) {
  double det = m4_det(in);
  if (det == 0.0) return false;
  double a1 = in[0], b1 = in[1], c1 = in[2], d1 = in[3];
  double a2 = in[4], b2 = in[5], c2 = in[6], d2 = in[7];
  double a3 = in[8], b3 = in[9], c3 = in[10], d3 = in[11];
  double a4 = in[12], b4 = in[13], c4 = in[14], d4 = in[15];
  double o[16];
  o[0 * 4 + 0] = det3(b2, b3, b4, c2, c3, c4, d2, d3, d4);
  o[1 * 4 + 0] = -det3(a2, a3, a4, c2, c3, c4, d2, d3, d4);
  o[2 * 4 + 0] = det3(a2, a3, a4, b2, b3, b4, d2, d3, d4);
  o[3 * 4 + 0] = -det3(a2, a3, a4, b2, b3, b4, c2, c3, c4);
  o[0 * 4 + 1] = -det3(b1, b3, b4, c1, c3, c4, d1, d3, d4);
  o[1 * 4 + 1] = det3(a1, a3, a4, c1, c3, c4, d1, d3, d4);
  o[2 * 4 + 1] = -det3(a1, a3, a4, b1, b3, b4, d1, d3, d4);
  o[3 * 4 + 1] = det3(a1, a3, a4, b1, b3, b4, c1, c3, c4);
  o[0 * 4 + 2] = det3(b1, b2, b4, c1, c2, c4, d1, d2, d4);
  o[1 * 4 + 2] = -det3(a1, a2, a4, c1, c2, c4, d1, d2, d4);
  o[2 * 4 + 2] = det3(a1, a2, a4, b1, b2, b4, d1, d2, d4);
  o[3 * 4 + 2] = -det3(a1, a2, a4, b1, b2, b4, c1, c2, c4);
  o[0 * 4 + 3] = -det3(b1, b2, b3, c1, c2, c3, d1, d2, d3);
  o[1 * 4 + 3] = det3(a1, a2, a3, c1, c2, c3, d1, d2, d3);
  o[2 * 4 + 3] = -det3(a1, a2, a3, b1, b2, b3, d1, d2, d3);
  o[3 * 4 + 3] = det3(a1, a2, a3, b1, b2, b3, c1, c2, c3);
  for (int i = 0; i < 16; ++i) out[i] = o[i] / det;
  return true;
}

void m4_rotate_pre(M4 &m, double angle, double x, double y, double z) {
  if (angle == 0.0 || (x == 0.0 && y == 0.0 && z == 0.0)) return;
  angle = angle * 0.017453292519943295;
  double w = cos(0.5 * angle);
  double f = sin(0.5 * angle) / sqrt(x * x + y * y + z * z);
  x *= f;
  y *= f;
  z *= f;
  double r[16];
  for (int i = 0; i < 16; ++i) r[i] = (i % 5 == 0) ? 1.0 : 0.0;
  double ww = w * w, wx = w * x, wy = w * y, wz = w * z;
  double xx = x * x, yy = y * y, zz = z * z;
  double xy = x * y, xz = x * z, yz = y * z;
  double s = ww - xx - yy - zz;
  r[0 * 4 + 0] = xx * 2 + s;
  r[1 * 4 + 0] = (xy + wz) * 2;
  r[2 * 4 + 0] = (xz - wy) * 2;
  r[0 * 4 + 1] = (xy - wz) * 2;
  r[1 * 4 + 1] = yy * 2 + s;
  r[2 * 4 + 1] = (yz + wx) * 2;
  r[0 * 4 + 2] = (xz + wy) * 2;
  r[1 * 4 + 2] = (yz - wx) * 2;
  r[2 * 4 + 2] = zz * 2 + s;
  m4_mul(m.e, r, m.e);
}

M4 m4_euler_zyz_neg(double alpha, double beta, double gamma) {
  M4 m = m4_identity();
  m4_rotate_pre(m, -gamma, 0, 0, 1);
  m4_rotate_pre(m, -beta, 0, 1, 0);
  m4_rotate_pre(m, -alpha, 0, 0, 1);
  return m;
}

void m4_transform_vector(const double e[16], const double in[3], double out[3]) {
  double x = e[0] * in[0] + e[1] * in[1] + e[2] * in[2];
  double y = e[4] * in[0] + e[5] * in[1] + e[6] * in[2];
  double z = e[8] * in[0] + e[9] * in[1] + e[10] * in[2];
  out[0] = x;
  out[1] = y;
  out[2] = z;
}

int vtk_floor(double x, double &f) {
  x += (103079215104.0 + 7.62939453125e-06);
  long long i = (long long)x;
  f = x - (double)i;
  return (int)(i - 103079215104LL);
}

void vtk_cubic_weights(double F[4], double f) {
  const double half = 0.5;
  double fm1 = f - 1;
  double fd2 = f * half;
  double ft3 = f * 3;
  F[0] = -fd2 * fm1 * fm1;
  F[1] = ((ft3 - 2) * fd2 - 1) * fm1;
  F[2] = -((ft3 - 4) * f - 1) * fd2;
  F[3] = f * fd2 * fm1;
}

static inline int clampi(int a, int b, int c) {
  a = (a <= c ? a : c);
  a -= b;
  a = (a >= 0 ? a : 0);
  return a;
}
static inline int wrapi(int a, int b, int c) {
  int range = c - b + 1;
  a -= b;
  a %= range;
  a = (a >= 0 ? a : a + range);
  return a;
}

template <class T>
static double tricubic(const T *vol, const int dims[3], const double p[3], bool wrap) {
  double fx, fy, fz;
  int ix = vtk_floor(p[0], fx), iy = vtk_floor(p[1], fy), iz = vtk_floor(p[2], fz);
  long incx = 1, incy = dims[0], incz = (long)dims[0] * dims[1];
  long factX[4], factY[4], factZ[4];
  for (int t = 0; t < 4; ++t) {
    if (wrap) {
      factX[t] = wrapi(ix - 1 + t, 0, dims[0] - 1) * incx;
      factY[t] = wrapi(iy - 1 + t, 0, dims[1] - 1) * incy;
      factZ[t] = wrapi(iz - 1 + t, 0, dims[2] - 1) * incz;
    } else {
      factX[t] = clampi(ix - 1 + t, 0, dims[0] - 1) * incx;
      factY[t] = clampi(iy - 1 + t, 0, dims[1] - 1) * incy;
      factZ[t] = clampi(iz - 1 + t, 0, dims[2] - 1) * incz;
    }
  }
  double wX[4], wY[4], wZ[4];
  vtk_cubic_weights(wX, fx);
  vtk_cubic_weights(wY, fy);
  vtk_cubic_weights(wZ, fz);
  int multipleY = (dims[1] > 1) && (fy != 0);
  int multipleZ = (dims[2] > 1) && (fz != 0);
  int j1 = 1 - multipleY, j2 = 1 + 2 * multipleY;
  int k1 = 1 - multipleZ, k2 = 1 + 2 * multipleZ;
  if (!multipleY) wY[1] = 1;
  if (!multipleZ) wZ[1] = 1;
  double val = 0;
  for (int k = k1; k <= k2; ++k) {
    double ifz = wZ[k];
    long factz = factZ[k];
    for (int j = j1; j <= j2; ++j) {
      double fzy = ifz * wY[j];
      const T *tmp = vol + factz + factY[j];
      val += fzy * (wX[0] * (double)tmp[factX[0]] + wX[1] * (double)tmp[factX[1]] +
                    wX[2] * (double)tmp[factX[2]] + wX[3] * (double)tmp[factX[3]]);
    }
  }
  return val;
}

double vtk_tricubic_float(const float *vol, const int dims[3], const double p[3], bool wrap) {
  return tricubic<float>(vol, dims, p, wrap);
}
double vtk_tricubic_double(const double *vol, const int dims[3], const double p[3], bool wrap) {
  return tricubic<double>(vol, dims, p, wrap);
}

static void smooth_axis(const float *in, float *out, const int dims[3], int axis, double std, int radius) {
  long inc[3] = {1, dims[0], (long)dims[0] * dims[1]};
  int n = dims[axis];
  std::vector<double> kernel(2 * radius + 1);
  for (int a = 0; a < n; ++a) {
    int left = 0 - (a - radius);
    int start = a - radius;
    if (left > 0) start += left; else left = 0;
    int right = (a + radius) - (n - 1);
    if (right < 0) right = 0;
    int kmin = -radius + left, kmax = radius - right, ksize = kmax - kmin + 1;
    if (std == 0.0) {
      kernel[0] = 1.0;
      ksize = 1;
      start = a;
    } else {
      double sum = 0.0;
      for (int x = kmin; x <= kmax; ++x) sum += kernel[x - kmin] = exp(-((double)(x * x)) / (std * std * 2.0));
      for (int x = kmin; x <= kmax; ++x) kernel[x - kmin] /= sum;
    }
    int o0 = (axis + 1) % 3, o1 = (axis + 2) % 3;
    for (int i1 = 0; i1 < dims[o1]; ++i1)
      for (int i0 = 0; i0 < dims[o0]; ++i0) {
        long base = (long)i0 * inc[o0] + (long)i1 * inc[o1];
        double s = 0.0;
        for (int k = 0; k < ksize; ++k) s += kernel[k] * (double)in[base + (long)(start + k) * inc[axis]];
        out[base + (long)a * inc[axis]] = (float)s;
      }
  }
}

void vtk_gaussian_smooth_float(float *img, const int dims[3], double std, double radius_factor) {
  int radius = (int)(std * radius_factor);
  long total = (long)dims[0] * dims[1] * dims[2];
  std::vector<float> a(img, img + total), b(total);
  smooth_axis(a.data(), b.data(), dims, 2, std, radius);
  smooth_axis(b.data(), a.data(), dims, 1, std, radius);
  smooth_axis(a.data(), b.data(), dims, 0, std, radius);
  memcpy(img, b.data(), sizeof(float) * total);
}

} // namespace oracle
