// Test infrastructure only: the pairwise loop of nbfCorrelationImageMetric::getDistances(representationFile, D)
// (inc/em/nbfCorrelationImageMetric.h:1735-1760, single-process branch) written with the same Blitz 0.9
// expressions on the reference's vendored Blitz, so that Blitz itself fixes the roundings the oracle restates
// (complex<float> element arithmetic, sum() of a float expression in double, mean() in float). The reference's
// own function cannot be compiled alone (MPI, Matlab file IO).
#include <blitz/array.h>
#include <complex>

using namespace blitz;

// R: V x K x depth floats (C order); D: V x V floats.
extern "C" int repr_ref_distances(int V, int K, int depth, const float *Rp, int normalized, float *Dp) {
  Array<float, 3> R(const_cast<float *>(Rp), shape(V, K, depth), neverDeleteData);
  Array<float, 2> D(Dp, shape(V, V), neverDeleteData);
  D = 0;
  for (int i = 0; i < D.rows(); i++) {
    for (int j = i + 1; j < D.rows(); j++) {
      if (R.depth() == 1) {
        D(i, j) = sqrt(sum(pow2(R(i, Range(1, toEnd), 0) - R(j, Range(1, toEnd), 0))));
      } else {
        Array<std::complex<float>, 1> c1(R.cols());
        real(c1) = R(i, Range::all(), 0);
        imag(c1) = R(i, Range::all(), 1);
        Array<std::complex<float>, 1> c2(R.cols());
        real(c2) = R(j, Range::all(), 0);
        imag(c2) = R(j, Range::all(), 1);
        Array<float, 1> wcombined1(R.cols());
        wcombined1 = R(i, Range::all(), 2);
        Array<float, 1> wcombined2(R.cols());
        wcombined2 = R(j, Range::all(), 2);
        float overlap = sum(wcombined1 * wcombined2);
        c1 = c1 * wcombined1 * wcombined2;
        c2 = c2 * wcombined1 * wcombined2;
        c1 = c1 - c2;
        if (normalized && overlap > 0) {
          D(i, j) = sum(real(c1 * conj(c1))) / overlap;
        } else {
          D(i, j) = mean(real(c1 * conj(c1)));
        }
      }
      D(j, i) = D(i, j);
    }
  }
  return 0;
}
