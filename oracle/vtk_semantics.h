/* Oracle restatement of the VTK 5.10 arithmetic that the reference alignment
 * path depends on (test infrastructure only; never linked into the product).
 *
 * Each function states the VTK behaviour it follows:
 *   - 4x4 matrices: Common/vtkMatrix4x4.cxx (Multiply4x4 106-131, Invert 140-177,
 *     Determinant 180-205, Adjoint 208-286); rows are stored row-major e[4*i+j].
 *   - vtkTransform rotations: Common/vtkAbstractTransform.cxx:548-597 (quaternion to
 *     matrix, PreMultiply concatenation M = M*R, zero angle is a no-op).
 *   - interpolation floor with the 2^-17 tolerance and 2^-16 fraction quantum of the
 *     64-bit x86 branch: Filtering/vtkImageInterpolatorInternals.h:78-108.
 *   - tricubic weights and tap selection: Filtering/vtkImageInterpolator.cxx:313-465.
 *   - reslice bounds (border tolerance 0.5 in clamp mode, unbounded when wrapping):
 *     Imaging/vtkImageReslice.cxx:1179-1190, Filtering/vtkAbstractImageInterpolator.cxx:323-345.
 *   - vtkImageGaussianSmooth separable z,y,x passes with clipped, renormalised kernels and
 *     per-pass rounding to the image scalar type: Imaging/vtkImageGaussianSmooth.cxx:67-93,
 *     249-358, 431-464.
 */
#pragma once
#include <cstdint>
#include <vector>

namespace oracle {

struct M4 {
  double e[16];
};

M4 m4_identity();
void m4_mul(const double a[16], const double b[16], double c[16]);   /* c = a*b */
double m4_det(const double e[16]);
bool m4_invert(const double in[16], double out[16]);
/* vtkTransform::RotateWXYZ in PreMultiply mode: M <- M * R(angle_deg, axis). */
void m4_rotate_pre(M4 &m, double angle_deg, double x, double y, double z);
/* vtkTransform built by RotateZ(-gamma); RotateY(-beta); RotateZ(-alpha) (degrees). */
M4 m4_euler_zyz_neg(double alpha, double beta, double gamma);
/* vtkLinearTransform::TransformVector (3x3 part only). */
void m4_transform_vector(const double e[16], const double in[3], double out[3]);

/* Interpolation floor: returns the integer part and the quantised fraction. */
int vtk_floor(double x, double &f);
void vtk_cubic_weights(double F[4], double f);

/* Tricubic interpolation of a float volume in x-fastest order (dims nx,ny,nz) at index
 * coordinates p, with clamp (wrap=false) or repeat (wrap=true) border handling. */
double vtk_tricubic_float(const float *vol, const int dims[3], const double p[3], bool wrap);
double vtk_tricubic_double(const double *vol, const int dims[3], const double p[3], bool wrap);

/* vtkImageGaussianSmooth on a float image with VTK dims (nx,ny,nz) stored x-fastest.
 * std and radius factor are per-axis equal, as every caller on the path sets them. */
void vtk_gaussian_smooth_float(float *img, const int dims[3], double std, double radius_factor);

} // namespace oracle
