// Test infrastructure only: the Fourier-filter construction, the spectrum normalisation and the distance of the
// translational CCF written with the reference's own Blitz 0.9 expressions on its vendored Blitz, so that Blitz and
// the C++ library fix their types and roundings:
//  - nbfFourierFilter::bandPassOn, updateFilterHalf, buildBandPassHalf, buildBFactorHalf
//    (inc/em/nbfFourierFilter.h:700-712, 492-546, 737-797): band parameters stored as double, the radius of
//    each half-grid sample from a TinyVector<float> of normalised offsets, where() of double expressions into
//    float arrays;
//  - nbfCorrelationImageMetric::normalizeFourierHalf (inc/em/nbfCorrelationImageMetric.h:497-530): DC removed,
//    norm a float from double sums;
//  - the distance of nbfFourierImageMetric::executeFourierNewHalf (inc/em/nbfFourierImageMetric.h:1249-1258):
//    the peak assigned to the float correlationPeak, then divided twice by the int size of the upsampled grid.
// The reference's member functions cannot be compiled alone (VTK, FFTW).
#include <blitz/array.h>
#include <blitz/tinyvec-et.h>

#include <complex>
#include <limits>

using namespace blitz;

extern "C" int filter_ref_half(int N, float lowCut, float highCut, float lowVariance, float highVariance,
                               float bfactor, float *out) {
  double bandLowCut = 0, bandHighCut = 1, bandLowVariance = .1, bandHighVariance = .1;
  bool useBandPass = false;
  if ((lowCut > 0.0) || (highCut < 1.0)) {
    bandLowCut = lowCut;
    bandHighCut = highCut;
    bandLowVariance = lowVariance;
    bandHighVariance = highVariance;
    useBandPass = true;
  }
  double bfactorExponent = (float)bfactor;
  TinyVector<int, 3> size(N, N, N);
  TinyVector<int, 3> center;
  center = floor(size / 2.0);
  Array<float, 3> filter(size[0], size[1], size[2] / 2 + 1);
  filter = 1;
  filter(filter.rows() / 2, filter.cols() / 2, filter.depth() - 1) = 0;
  if (useBandPass) {
    Array<float, 3> bandPass(size[0], size[1], size[2] / 2 + 1);
    Array<float, 3> radius(bandPass.shape());
    Array<float, 3>::iterator iter = radius.begin();
    while (iter != radius.end()) {
      TinyVector<float, 3> tmp((1.0 * iter.position() - center) / center);
      (*iter) = sqrt(sum(tmp * tmp));
      ++iter;
    }
    bandPass = where(radius < bandLowCut, exp(-pow2(bandLowCut - radius) / 2.0 / bandLowVariance / bandLowVariance), 1);
    bandPass = where(radius > bandHighCut, exp(-pow2(radius - bandHighCut) / 2.0 / bandHighVariance / bandHighVariance),
                     bandPass);
    filter *= bandPass;
  }
  if (bfactorExponent != 0) {
    Array<float, 3> bf(size[0], size[1], size[2] / 2 + 1);
    Array<float, 3> radius(bf.shape());
    Array<float, 3>::iterator iter = radius.begin();
    while (iter != radius.end()) {
      TinyVector<float, 3> tmp((1.0 * iter.position() - center) / center);
      (*iter) = sqrt(sum(tmp * tmp));
      ++iter;
    }
    bf = exp(-bfactorExponent * pow2(radius));
    filter *= bf;
  }
  Array<float, 3> o(out, filter.shape(), neverDeleteData);
  o = filter;
  return 0;
}

// F: N x N x (N/2 + 1) complex<double> interleaved, normalised in place; returns the norm.
extern "C" float normalize_ref_half(int N, double *F) {
  Array<std::complex<double>, 3> input(reinterpret_cast<std::complex<double> *>(F), shape(N, N, N / 2 + 1),
                                       neverDeleteData);
  TinyVector<int, 3> center(input.rows() / 2, input.cols() / 2, input.ubound(thirdDim));
  input(center) = 0;
  float norm;
  Array<std::complex<double>, 3> inputv(input(Range::all(), Range::all(), Range(0, input.depth() - 2)));
  norm = 2 * sum(real(inputv * conj(inputv)));
  Array<std::complex<double>, 2> inputu(input(Range::all(), Range::all(), input.ubound(thirdDim)));
  norm = sqrt((norm + sum(real(inputu * conj(inputu)))) / (1.0 * input.rows() * input.cols() * 2 * (input.depth() - 1)));
  input /= norm;
  return norm;
}

// The distance from k1_m, the windowed maximum of T, the overlap sums and the upsampled grid of edge 2N.
extern "C" float distance_ref(float k1_m, double maxT, double sum_wf, double sum_f, int use_overlap, int N) {
  float correlationPeak;
  if (use_overlap) {
    correlationPeak = std::max(0.0, (k1_m - maxT)) / sum_wf * sum_f;
  } else {
    correlationPeak = std::max(0.0, (k1_m - maxT));
  }
  Array<double, 3> shiftbig(2 * N, 2 * N, 2 * N);
  correlationPeak = correlationPeak / shiftbig.size() / shiftbig.size();
  return correlationPeak;
}
