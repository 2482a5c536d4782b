// Test infrastructure only: the class-selection rules of the classification iteration written with the
// reference's own expressions on its vendored Blitz 0.9, so that Blitz and the C++ library fix their types and
// roundings:
//  - nbfLoopClustering::computeNewReferences (inc/em/nbfLoopClustering.h:2406-2463): radii and sigmoid weights;
//  - nbfLoopClustering::asignBestAlignmentAndClean (2590-2637): best class by minIndex, |distance|, the sorted
//    cutoff at fraction * (n - 1), distance < cutoff;
//  - the refinement loop of src/MPI_Classification.cpp (922-934, 1137-1150): the same cutoff on the raw
//    distances, kept by <= for the next average's weights and by < for the cleaned list.
// The reference's member functions cannot be compiled alone (VTK, MPI, file IO).
#include <blitz/array.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

using namespace blitz;

// D: volume-major distances, D[v * R + r]; W: class-major weights W[r * V + v].
extern "C" int clustering_ref_soft_weights(int R, int V, const float *D, float *W, float *radii) {
  Array<float, 2> normalizedDistances(R, V);
  for (int r = 0; r < R; ++r)
    for (int v = 0; v < V; ++v) normalizedDistances(r, v) = D[(long)v * R + r];
  float decay = .025;
  Array<float, 1> referenceRadii(R);
  for (int i = 0; i < R; i++) referenceRadii(i) = max(normalizedDistances(i, Range::all())) + decay * log(.01);
  Array<float, 2> classes(R, V);
  for (int i = 0; i < R; i++) {
    classes(i, Range::all()) =
        (1 + 2.0 * exp(-(normalizedDistances(i, Range::all()) - referenceRadii(i)) / decay)) /
            (1 + 1.0 * exp(-(normalizedDistances(i, Range::all()) - referenceRadii(i)) / decay)) -
        1.0;
    classes(i, Range::all()) = where(classes(i, Range::all()) > .01, classes(i, Range::all()), 0);
  }
  for (int r = 0; r < R; ++r) {
    radii[r] = referenceRadii(r);
    for (int v = 0; v < V; ++v) W[(long)r * V + v] = classes(r, v);
  }
  return 0;
}

// rule 0: asignBestAlignmentAndClean; rule 1: next-average weights; rule 2: cleaned list.
extern "C" int clustering_ref_cutoff(int R, int V, const float *D, float fraction, int rule, int *best, float *dist,
                                     int *keep) {
  Array<float, 2> A(R, V);
  for (int r = 0; r < R; ++r)
    for (int v = 0; v < V; ++v) A(r, v) = D[(long)v * R + r];
  std::vector<float> distances;
  for (int i = 0; i < V; i++) {
    TinyVector<int, 1> b = minIndex(A(Range::all(), i));
    best[i] = b[0];
    distances.push_back(rule == 0 ? fabs(A(b[0], i)) : A(b[0], i));
  }
  for (int i = 0; i < V; ++i) {
    dist[i] = distances[i];
    keep[i] = 1;
  }
  if ((distances.size() > 0) && (fraction < 1)) {
    std::vector<float> sortedDistances(distances.size());
    sortedDistances = distances;
    std::sort(sortedDistances.begin(), sortedDistances.end());
    float cutoffDistance = rule == 0 ? sortedDistances[fraction * (sortedDistances.size() - 1)]
                                     : sortedDistances[(sortedDistances.size() - 1) * fraction];
    for (int i = 0; i < V; i++) keep[i] = rule == 1 ? (distances[i] <= cutoffDistance) : (distances[i] < cutoffDistance);
  }
  return 0;
}

// nbfLoopClustering::doMra's class choice (inc/em/nbfLoopClustering.h:1572-1586): alignments(j, d, 0, 0) holds
// the distance of duplicate d = i * R + r (volume i under reference r's alignment) against reference j;
// partialSums(d) = sum over j (a Blitz partial reduction stored as Pixel); the class of volume i is the first
// minimum over r of the reshaped sums. S: [i][r][j] = alignments(j, i * R + r); best: V labels.
extern "C" int clustering_ref_mra_assign(int R, int V, const float *S, int *best) {
  Array<float, 2> extractedDistances(R, V * R);
  for (int i = 0; i < V; ++i)
    for (int r = 0; r < R; ++r)
      for (int j = 0; j < R; ++j) extractedDistances(j, i * R + r) = S[((long)i * R + r) * R + j];
  Array<float, 1> partialSums(V * R);
  firstIndex ii;
  secondIndex jj;
  partialSums = sum(extractedDistances(jj, ii), jj);
  Array<float, 2> reshapedPartialSums(partialSums.data(), shape(V, R), neverDeleteData);
  for (int i = 0; i < V; i++) {
    TinyVector<int, 1> b = minIndex(reshapedPartialSums(i, Range::all()));
    best[i] = b[0];
  }
  return 0;
}
