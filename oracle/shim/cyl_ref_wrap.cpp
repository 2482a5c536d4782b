// Test infrastructure only: drives the reference's own cylindrical-domain classes (inc/nbfCylindricalDomain3.h,
// inc/nbfLinearInterpolator.h, compiled in place against the reference's vendored Blitz 0.9) through the
// rotational-symmetry step of the classification loop (src/MPI_Classification.cpp:1005-1024), so that the
// oracle's restatement of that step can be checked against the reference itself.
//
// The one VTK call those headers make, vtkMath::Pi(), is declared here with the value and float return type
// it has in VTK 5.10.1 (Common/vtkMath.h:83); nothing else of VTK is used.
#include <blitz/array.h>
#include <blitz/tinyvec-et.h>

using namespace blitz;

class vtkMath {
 public:
  static float Pi() { return 3.14159265358979f; }
};

#include <nbfLinearInterpolator.h>
#include <nbfCylindricalDomain3.h>

// vol: N^3 floats, x fastest ([z][y][x]); out: N^3 doubles, [x][y][z] (the layout of the oracle's outputs).
extern "C" int cyl_ref_rotational(int N, const float *vol, double *out) {
  if (N < 4 || (N & 1)) return 1;
  Array<double, 3> in(N, N, N), cyl, res;
  Array<bool, 3> zone;
  for (int z = 0; z < N; ++z)
    for (int y = 0; y < N; ++y)
      for (int x = 0; x < N; ++x) in(x, y, z) = (double)vol[x + (long)N * (y + (long)N * z)];
  res.resize(in.shape());
  res = in;
  nbfCylindricalDomain3<double> dom;
  TinyVector<int, 3> center = in.shape() / 2;
  dom.setCenter(center);
  dom.setMaxRho(in.extent(firstDim) / 2);
  dom.setResRho(in.extent(firstDim) / 2);
  dom.setResTheta(180);
  dom.cartesian2cylindrical(res, cyl, zone);
  Array<double, 2> profile(cyl.rows(), cyl.depth());
  firstIndex i;
  secondIndex j;
  thirdIndex k;
  profile = sum(cyl(i, k, j), k);
  for (int t = 0; t < cyl.cols(); ++t) cyl(Range::all(), t, Range::all()) = profile;
  dom.cylindrical2cartesian(cyl, res, zone);
  for (int x = 0; x < N; ++x)
    for (int y = 0; y < N; ++y)
      for (int z = 0; z < N; ++z) out[((long)x * N + y) * N + z] = res(x, y, z);
  return 0;
}
