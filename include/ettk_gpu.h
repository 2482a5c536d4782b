/* ettk_gpu.h — C ABI of the GB300 sub-volume alignment library (libettk_gpu.so).
 *
 * Drop-in for the pairwise particle x reference alignment of ETTK's MPI_Classification:
 * nbfProjectionRotationMetric3D<float>::execute (inc/em/nbfProjectionRotationMetric3D.h:415-1052)
 * driven by nbfCorrelationImageMetric::getDistances (inc/em/nbfCorrelationImageMetric.h:1873-2288),
 * alignment_mode 3 (SO(3) grid hit + translational CCF, no Powell refinement).
 *
 * Conventions
 *  - Every call returns an int status (ETTK_OK = 0); no exception crosses the ABI.
 *    ettk_gpu_last_error() returns a description of the last failure on a context.
 *  - Host buffers are caller-owned and only read/written during the call (synchronous API).
 *  - Volumes are float32 fixed images of edge N stored x-fastest (MRC / VTK order),
 *    i.e. element (x,y,z) at x + N*(y + N*z).
 *  - Matrices are 4x4 row-major doubles (vtkMatrix4x4::DeepCopy order).
 *  - One context = one GPU = one CUDA stream; contexts are independent (re-entrant across contexts,
 *    not thread-safe within one context).
 */
#ifndef ETTK_GPU_H
#define ETTK_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ETTK_OK = 0,
  ETTK_ERR_ARG = 1,      /* invalid argument or unsupported configuration */
  ETTK_ERR_OOM = 2,      /* device or host allocation failed (the reference exit(1)s instead,
                            inc/em/nbfProjectionRotationMetric3D.h:1093-1104) */
  ETTK_ERR_CUDA = 3,     /* a CUDA runtime call failed */
  ETTK_ERR_TIMEOUT = 4,  /* a bounded device wait (bulk copy, tensor-core commit) gave up; the context stays usable */
  ETTK_ERR_NAN = 5,      /* non-finite input volume */
  ETTK_ERR_STATE = 6     /* references or particles not set */
};

typedef struct ettk_ctx ettk_ctx;

/* Alignment parameters. Each field names the reference setting it replaces. */
typedef struct {
  int N;                        /* box edge, power of two 16..128 (nbfWedgedSubImage3D geometry) */
  int B;                        /* SH bandwidth, power of two 8..64 (nbfProjectionRotationMetric3D::B) */
  float mask_radius;            /* nbfImageFilter::setMaskSize(x=y=z=mask_radius, sigma) */
  float mask_sigma;
  float square_mask_size;       /* nbfImageFilter::squareMaskSize */
  float bp_low, bp_high;        /* nbfFourierFilter::bandPassOn(lowCut, highCut, lowVar, highVar) */
  float bp_low_sigma, bp_high_sigma;
  float bfactor;                /* nbfFourierFilter::bfactorOn (0 = off) */
  float restrict_translation;   /* nbfImageMetric::setTranslationSearchRestriction */
  float restrict_rotation;      /* nbfImageMetric::setRotationSearchRestriction (degrees) */
  int candidate_peaks;          /* nbfProjectionRotationMetric3D::setNumberOfCandidatePeaksToSearch */
  int number_of_candidates;     /* nbfCorrelationImageMetric::setNumberOfCandidates */
  int wedge_compensation;       /* nbfImageMetric::setMissingWedgeCompensation */
  int overlap_normalized;       /* nbfImageMetric::setToComputeOverlapNormalizedDistances */
  int mutual_correlation;       /* nbfImageMetric::setToUseMutualCorrelation: |F|^(1/2) spherical projections, F/|F|^(1/2) in the CCF */
  int max_batch;                /* pairs aligned per device batch (0 = automatic) */
  int wigner_precision;         /* Wigner-d contraction of the SO(3) correlation (no reference setting; the
                                   reference contracts in FP64): 0 FP32 (default, parity), 1 BF16 tensor cores,
                                   2 split-BF16 tensor cores, 3 TF32 tensor cores, 4 FP64 (precision reference) */
  int fast_coarse_so3;          /* fast form only (ettk_gpu_align_pairs_refined; no reference setting): 1 runs its
                                   SO(3) search on the volumes Fourier-cropped to half the edge at bandwidth B/2, the
                                   grid the candidate screening already uses; 2 also resamples the screened candidates
                                   trilinearly instead of tricubically; 0 searches at the full edge and B */
} ettk_params;

/* Launch shapes of the library's kernels (no reference setting). None of them changes a result; they trade
 * parallelism against scheduling overhead, and ettk_gpu_autotune chooses them per GPU and box size.
 *   synth_job_blocks  job blocks per (m1, m2) cell of the FP32 Wigner-d synthesis: 16, 32, 64 (default) or 128
 *   eval_chunk        CCF evaluations per device chunk at 64^3 (scaled by 64^3 / N^3): 1024, 2048, 4096 (default)
 *                     or 8192
 *   zpass_oversub     CTAs of the persistent z passes per resident CTA slot: 1 (default) or 2
 *   sample_block      threads per CTA of the spherical sampling: 64, 128 (default) or 256 */
typedef struct {
  int synth_job_blocks, eval_chunk, zpass_oversub, sample_block;
} ettk_tuning;

/* Per-volume metadata: the columns of the reference's 33-column volume list
 * (nbfWedgedSubImage3D::serialize, inc/em/nbfWedgedSubImage3D.h:387-421). */
typedef struct {
  float lwedge, uwedge;         /* missing wedge limits (degrees, about Y) */
  float normal[3];              /* Euler angles applied as RotateZ(-n2) RotateX(-n0) RotateZ(-n1) */
  double matrix[16];            /* alignment matrix */
  float position[3];            /* centre of the box in the fixed image (N/2 for fixed images) */
  float cut_offset;             /* extra Z offset of the box */
} ettk_volume_meta;

/* Replaces constructing nbfProjectionRotationMetric3D<float>(imageFilter, fourierFilter) and its
 * setters (src/MPI_Classification.cpp:594-653). */
int ettk_gpu_create(int device, const ettk_params *params, ettk_ctx **ctx);
int ettk_gpu_destroy(ettk_ctx *ctx);

/* Replaces the list1 side of getDistances(list1, list2, ...) (inc/em/nbfCorrelationImageMetric.h:1873):
 * R reference volumes (R*N^3 floats) and their metadata. */
int ettk_gpu_set_references(ettk_ctx *ctx, int R, const float *volumes, const ettk_volume_meta *meta);

/* Replaces the list2 side: V particle volumes and metadata (host memory). A volume holding a NaN or an infinity
 * (checked on the device after the copy, as for the _device and _tomogram variants) fails the call with
 * ETTK_ERR_NAN and leaves the context without particles. */
int ettk_gpu_set_particles(ettk_ctx *ctx, int V, const float *volumes, const ettk_volume_meta *meta);

/* As ettk_gpu_set_particles with `volumes` already in device memory of the context's GPU. The buffer is
 * borrowed, not copied: it must hold the complete volumes when the call is made (the caller synchronises
 * whatever stream wrote them), stay unchanged and allocated until the next set_particles call or
 * ettk_gpu_destroy, since every later alignment reads it on the context's stream. */
int ettk_gpu_set_particles_device(ettk_ctx *ctx, int V, const float *d_volumes, const ettk_volume_meta *meta);

/* Particles cut from one tomogram (nbfWedgedSubImage3D::getImage's tomogram path,
   inc/em/nbfWedgedSubImage3D.h:602-746): tomogram is nx*ny*nz floats, x fastest; meta[v].position is the
   particle centre in tomogram voxel coordinates (and cut_offset the z offset of the box). Every reslice of a
   particle (spherical projection, CCF evaluations, averages) reads the tomogram directly. */
int ettk_gpu_set_particles_tomogram(ettk_ctx *ctx, int nx, int ny, int nz, const float *tomogram, int V,
                                    const ettk_volume_meta *meta);

/* Replaces nbfCorrelationImageMetric::getDistances(list1, list2, indexes, D, type=3)
 * (inc/em/nbfCorrelationImageMetric.h:1873-2009): pairs[2*i] = reference index, pairs[2*i+1] =
 * particle index. D is the reference's Array<float,3> D(npairs, cols, ncand) in C order:
 * D[(i*cols + c)*ncand + k]. Column 0 = distance (getDistance), then correlation scale when
 * cols > 17, wedge overlap when cols > 18, then the 16 entries of the final transform.
 * Rows whose D[i][0][0] != -1 on entry are skipped (the reference's resume convention). */
int ettk_gpu_align_pairs(ettk_ctx *ctx, int npairs, const int *pairs, float *D, int cols, int ncand);

/* Replaces nbfWedgedAverageImage3D::setAlignments + getImage (getImageMPI and getImage with
 * NBF_AVERAGE_IN_RECIPROCAL_SPACE, inc/em/nbfWedgedAverageImage3D.h:181-356): the wedge-weighted class
 * average of M members of the particle set (particles[i] = particle index, weights[i] = alignment
 * weight, matrices[16*i] = alignment matrix), written to avg (N^3 floats, x fastest, RMS 1). */
int ettk_gpu_average(ettk_ctx *ctx, int M, const int *particles, const float *weights, const double *matrices,
                     float *avg);

/* The class average split for members spread over several contexts or processes (getImageMPI returns its three
 * accumulators for the caller to sum across MPI ranks before getImage, inc/em/nbfWedgedAverageImage3D.h:216-356):
 * ettk_gpu_average_partial accumulates the members as ettk_gpu_average does and writes, in the reference's
 * [x][y][kz] half-spectrum order (N * N * (N/2 + 1) doubles each), re = sum w |F| Re F, im = sum w |F| Im F and
 * acc = sum |w| |F|; ettk_gpu_average_finish turns summed accumulators into the average (RMS 1, N^3 floats, x
 * fastest). Partial over all members followed by finish gives ettk_gpu_average's result. */
int ettk_gpu_average_partial(ettk_ctx *ctx, int M, const int *particles, const float *weights, const double *matrices,
                             double *re, double *im, double *acc);
int ettk_gpu_average_finish(ettk_ctx *ctx, const double *re, const double *im, const double *acc, float *avg);

/* Variance of class members about an average (nbfWedgedAverageImage3D::getImageVarianceMPI after
   setAverageImage, inc/em/nbfWedgedAverageImage3D.h:440-493): var = sum over members with weight != 0 of
   |w| (T - avg)^2 / sum |w|, T the member resampled as ettk_gpu_average resamples it (getImage, mean of valid
   voxels removed). avg and var are N^3 floats, x fastest (avg as ettk_gpu_average returns it). */
int ettk_gpu_variance(ettk_ctx *ctx, int M, const int *particles, const float *weights, const double *matrices,
                      const float *avg, float *var);

/* n-fold symmetrisation about the z axis (nbfImageFilter::symmetrize, inc/em/nbfImageFilter.h:527-554): the
   mean over i < fold of the volume, as a fixed image centred at N/2, resampled under RotateZ(i * 360 / fold)
   with the mean of its valid voxels removed. fold = 1 returns the volume unchanged. N^3 floats, x fastest. */
int ettk_gpu_symmetrize(ettk_ctx *ctx, const float *vol, int fold, float *out);

/* The mean over n transforms (transforms: n row-major 4x4 matrices) of getImage of vol as a fixed image
   (nbfWedgedSubImage3D::getImage after setFixedImage: centred at N/2, full wedge): each a tricubic resample under the
   transform with the mean of its valid voxels removed and the invalid ones 0, summed in order in FP64 and divided by
   n, as nbfLoopClustering::symmetrize accumulates reference.getImage(data, t) over the folds with the shifts the
   CCF found (inc/em/nbfLoopClustering.h:5987-6042). ettk_gpu_symmetrize is the case t_i = RotateZ(i * 360 / fold).
   vol and out: N^3 floats, x fastest. n 1..4096. */
int ettk_gpu_mean_images(ettk_ctx *ctx, const float *vol, int n, const double *transforms, float *out);

/* The external mask of the alignment (nbfImageFilter::setMaskFile(file, threshold), src/MPI_Classification.cpp:554-555,
   as nbfFourierImageMetric::reinitializeHalf uses it, inc/em/nbfFourierImageMetric.h:667-676): it becomes the reference
   mask m1 of the translational CCF (the k1_m and I1'.m1 sums and F(m1) of the cross term), and of the fast form's
   refinement. mask: M^3 floats, x fastest, the mask file's volume; processed as nbfImageFilter::buildMaskFromFile
   (inc/em/nbfImageFilter.h:319-381): centred into a zero N^3 box (M < N - 1) or cropped from its centre (M > N),
   binarised (value > threshold), softened (softenMask: Gaussian, std = mask_sigma, radius factor 0.75 mask_sigma).
   M = 0 restores the spherical mask. The spherical projection and the representations keep the spherical mask, as the
   reference's image filter does; the fast form's half-grid screening keeps its own spherical mask. M = N - 1 fails
   with ETTK_ERR_ARG (the reference indexes outside the mask there). */
int ettk_gpu_set_reference_mask(ettk_ctx *ctx, int M, const float *mask, float threshold);

/* The reference mask m1 in use (spherical or external): N^3 floats, x fastest. */
int ettk_gpu_get_reference_mask(ettk_ctx *ctx, float *out);

/* Low-dimensional representations of particles (nbfFourierImageMetric::getLowDimensionRepresentationHalf,
   inc/em/nbfFourierImageMetric.h:1967-2034, as nbfCorrelationImageMetric::getRepresentations collects them,
   inc/em/nbfCorrelationImageMetric.h:1323-1372; padding 1): per particle its image (own geometry, mean of
   valid voxels removed), with fold > 1 symmetrised n-fold about z (nbfImageFilter::symmetrize, as
   ettk_gpu_symmetrize), shifted, transformed, band-pass filtered, transformed back, masked with the real-space
   mask and transformed again (unnormalised, as FFTW); the K coefficients where |filter| > 0.5 are kept in the
   [x][y][kz] order of the half spectrum as (re, im, wedge bit) with the bit getWedgeImageHalf > 0.5 (1 for
   fold > 1). fold 1..360. *K receives K (the call with R = NULL only does that); R receives M * K * 3
   floats, the representation array R(M, K, 3) of ettk_gpu_representation_distances. */
int ettk_gpu_representations(ettk_ctx *ctx, int M, const int *particles, int fold, int *K, float *R);

/* Real-space low-dimensional representations of particles (nbfFourierImageMetric::getLowDimensionRepresentationReal,
   inc/em/nbfFourierImageMetric.h:2375-2533, as nbfCorrelationImageMetric::getRepresentations collects them with
   useRealRepresentation, inc/em/nbfCorrelationImageMetric.h:1341-1352; no mask file): per particle its image (own
   geometry, mean of valid voxels removed) or, with fold > 1, the wedged average of the particle alone under its matrix
   times RotateZ(f * 360 / fold) for f < fold (weights 1 / fold, as ettk_gpu_average); band-pass filtered
   (nbfFourierFilter::executeHalf on the real array: C2R(filter R2C(A shift)) shift / N^3); with fold > 1 then
   symmetrised n-fold about z (as ettk_gpu_symmetrize); binned by the integer bin_factor (vtkImageResample with
   magnification 1 / bin_factor: samples at input indices bin_factor * i, i <= (N - 1) / bin_factor, of the image and
   of the mask alike); the values where the binned mask exceeds 0.5 are kept in [x][y][z] order. fold 1..360,
   bin_factor 1..64. *K receives K (the call with R = NULL only does that); R receives M * K floats, the depth-1
   representation array R(M, K, 1) of ettk_gpu_representation_distances. */
int ettk_gpu_representations_real(ettk_ctx *ctx, int M, const int *particles, int fold, int bin_factor, int *K,
                                  float *R);

/* Distance matrix between low-dimensional representations (nbfCorrelationImageMetric::getDistances(file, D),
   inc/em/nbfCorrelationImageMetric.h:1726-1871, the pairwise step of the unsupervised classification). R is
   the reference's representation array R(V, K, depth) in C order: depth 3 = (re, im, wedge bit) of the K kept
   Fourier coefficients (getLowDimensionRepresentationHalf), depth 1 = a real vector
   (getLowDimensionRepresentationReal). D (V*V floats, symmetric, zero diagonal) receives for depth 3 the squared
   difference of the two spectra on their common wedge, sum |c_i w_i w_j - c_j w_i w_j|^2 divided by the
   overlap sum w_i w_j (overlap_normalized != 0 and overlap > 0) or averaged over K; for depth 1 the Euclidean
   distance of entries 1..K-1. Same float / double roundings as the reference (bit-identical results). */
int ettk_gpu_representation_distances(ettk_ctx *ctx, int V, int K, int depth, const float *R, int overlap_normalized,
                                      float *D);

/* Spherical missing wedge of a class average (nbfWedgedAverageImage3D::updateAccumulatedSphericalWedgeImageMPI and
   updateSphericalWedgeImage, inc/em/nbfWedgedAverageImage3D.h:612-665): for the members with weight != 0 (own
   matrix reset, as ettk_gpu_average resamples them), the binary spherical wedge under the alignment
   matrices[16*i] (nbfWedge3D::getSphericalImage, inc/em/nbfWedge3D.h:363-429) counted per sample of the
   (2B)^2 grid ([polar][azimuth], count optional), and wedge = 1 where count > max(count) / 2, else 0. */
int ettk_gpu_average_spherical_wedge(ettk_ctx *ctx, int M, const int *particles, const float *weights,
                                     const double *matrices, float *count, float *wedge);

/* Explicit spherical wedge for reference r (nbfWedge3D::setSphericalImage, as the MRA loop hands an average's
   wedge to its precomputed reference, inc/em/nbfLoopClustering.h:1270-1278): the binary (2B)^2 map replaces the
   one derived from the reference's wedge angles in the SO(3) stage, conditioned as every spherical window is
   (Gaussian std 2, radius factor 1; used when its sum is at most 0.95 of the grid). Lasts until the next
   ettk_gpu_set_references. The half-spectrum wedge of the translational stage stays the analytic one, as
   nbfWedge3D::getImageHalf ignores explicit images (inc/em/nbfWedge3D.h:312-360). */
int ettk_gpu_set_reference_spherical_wedge(ettk_ctx *ctx, int r, const float *wedge);

/* Rotational symmetrisation of the classification loop (apply_rotational_symmetry,
   src/MPI_Classification.cpp:1005-1024, with nbfCylindricalDomain3, inc/nbfCylindricalDomain3.h:126-233): the
   volume sampled on a cylinder about the z axis through (N/2, N/2) (N/2 radii from 0 to N/2, 180 angles over
   [0, 2 pi] with both ends, every z plane; clamped trilinear interpolation), summed over the angles (a sum,
   so the result carries a factor of about 180, as in the reference) and interpolated back at each voxel's
   radius. FP64 on the device, N^3 floats in and out, x fastest. */
int ettk_gpu_symmetrize_rotational(ettk_ctx *ctx, const float *vol, float *out);

/* Host-only helpers of the classification iteration (no context, no device work). D holds one row of ld
   floats per (volume, class) pair, row v * R + r, the distance in column 0: the layout ettk_gpu_align_pairs
   writes for pairs ordered volume-major. */

/* Best class and outlier cutoff. best[v] = the class of smallest distance (the first on ties), dist[v] its
   distance; with top_fraction < 1 the cutoff is the sorted dist at index (int)(top_fraction * (V - 1)) (float
   product) and keep[v] says whether volume v survives it; otherwise every keep[v] = 1 and *cutoff = inf.
   rule 0: nbfLoopClustering::asignBestAlignmentAndClean (inc/em/nbfLoopClustering.h:2590-2637), |distance|
           and keep = dist < cutoff;
   rule 1: the weights of the next global average (src/MPI_Classification.cpp:922-934), keep = dist <= cutoff;
   rule 2: the cleaned volume list (src/MPI_Classification.cpp:1137-1150), keep = dist < cutoff.
   cutoff is optional. */
int ettk_gpu_outlier_cutoff(int R, int V, const float *D, int ld, float top_fraction, int rule, int *best,
                            float *dist, int *keep, float *cutoff);

/* Class choice of the MRA loop (nbfLoopClustering::doMra, inc/em/nbfLoopClustering.h:1523-1592): each volume v
   was scored, under the alignment it received from each reference r, against every reference j (getDistances
   type 2 at translation restriction 0); S[(v * R + r) * R + j] holds that distance (the reference's
   alignments(j, v * R + r, 0, 0)). labels[v] = the r whose sum over j is smallest (the first on ties; the sum
   in double, compared as float). */
int ettk_gpu_mra_assign(int R, int V, const float *S, int *labels);

/* Soft class weights of nbfLoopClustering::computeNewReferences (inc/em/nbfLoopClustering.h:2406-2502; the
   reference defines it but none of its drivers calls it): per class r, radius = max_v D(v, r) + 0.025 ln 0.01,
   W[r * V + v] = (1 + 2e) / (1 + e) - 1 with e = exp(-(D(v, r) - radius) / 0.025) (float exponent), weights
   of 0.01 or less set to 0. radii (optional, R floats) receives the radii. */
int ettk_gpu_soft_weights(int R, int V, const float *D, int ld, float *W, float *radii);

/* Multireference classification (the align -> assign -> re-average loop of src/MPI_Classification.cpp:954-1170,
   alignment_mode 3): each pass aligns every particle against every current reference (as
   ettk_gpu_align_pairs), assigns each particle to the class of smallest distance (labels[V]; dist_out[V] its
   distance, optional), rebuilds each class reference as the wedge-weighted average of its members under their
   alignments (as ettk_gpu_average; an empty class keeps its reference) and makes the averages the references
   of the next pass; with wedge compensation each new reference carries its class's spherical wedge
   (ettk_gpu_average_spherical_wedge + ettk_gpu_set_reference_spherical_wedge). refs_out (optional, R*N^3
   floats, x fastest) receives the last averages. */
int ettk_gpu_classify(ettk_ctx *ctx, int iterations, int *labels, float *refs_out, float *dist_out);

/* Continuous 6-DOF refinement of aligned pairs (no counterpart in the reference, whose refine() runs a
   Powell search over RotateX/Y/Z offsets with one CCF per step, inc/em/nbfFourierImageMetric.h:1701-1809):
   from the pose of candidate 0 of each row of D (as ettk_gpu_align_pairs wrote it), gradient ascent of the
   masked normalised correlation between the wedge*filter-constrained reference and particle, with the
   gradient from the hand-written adjoint of reslice -> R2C -> filter -> C2R (rotation about the box centre
   and shift, continuous). Writes the refined 4x4 pose and distance 1 - rho into the row. */
int ettk_gpu_refine_pairs(ettk_ctx *ctx, int npairs, const int *pairs, float *D, int cols, int ncand,
                          int iterations);

/* Replaces getDistances(list1, list2, indexes, D, type=2) (inc/em/nbfCorrelationImageMetric.h:1912-1976) with its
 * nbfFourierImageMetricCore (inc/em/nbfFourierImageMetricCore.h:35-66): per pair one translational CCF
 * (executeFourierNewHalf) of the particle under its own alignment matrix (the volume-list matrix, as doMra gives each
 * duplicate volume one of its alignments, inc/em/nbfLoopClustering.h:1523-1561) against the reference, with the
 * translation restriction restrict_translation (negative: the context's; doMra uses 0, which scores the given pose on
 * the 3-point window of the upsampled grid). D as in ettk_gpu_align_pairs; only candidate slot 0 is written
 * (the core metric keeps one candidate): the distance, scale 1, the wedge overlap at the transform, and the
 * transform (the found shift when isTransformValid accepts it, else the identity). Rows whose D[i][0][0] != -1
 * are skipped. */
int ettk_gpu_score_pairs(ettk_ctx *ctx, int npairs, const int *pairs, float *D, int cols, int ncand,
                         float restrict_translation);

/* Fast alignment form (no counterpart in the reference; it takes the place of getDistances with typeOfMetric 0,
   whose Powell refinement, inc/em/nbfFourierImageMetric.h:1701-1809, and whose mirror and candidate CCF loop,
   inc/em/nbfProjectionRotationMetric3D.h:678-901, it replaces): the same spherical projections, SO(3) correlations
   (in the context's wigner_precision) and candidate queues as ettk_gpu_align_pairs — or, with fast_coarse_so3, the
   same on the volumes Fourier-cropped to half the edge at bandwidth B/2 — then per pair one CCF
   (executeFourierNewHalf) of each of the `peaks` best candidates of the windowed queue and of the peaks / 3 (at
   least one) best of the unwindowed one, no mirror evaluations, computed for boxes of edge 32 and more on the
   volumes Fourier-cropped to half the edge (the band-pass keeps little above half the Nyquist frequency), and the
   best valid result refined in
   continuous rotation and shift by `iterations` steps of gradient ascent of the masked normalised correlation
   between the wedge- and band-limited reference (the CCF's filter times both wedges at the coarse pose) and the
   particle (trilinear interpolation, analytic gradient). D has the layout of ettk_gpu_align_pairs; column 0 holds
   1 - rho at the refined pose, the matrix the refined pose (continuous), scale 1 and the wedge overlap as there;
   candidate slots past the first get FLT_MAX in column 0. Rows whose D[i][0][0] != -1 are skipped.
   iterations 0 keeps the coarse pose (rho evaluated there); peaks 0 = the context's candidate_peaks. */
int ettk_gpu_align_pairs_refined(ettk_ctx *ctx, int npairs, const int *pairs, float *D, int cols, int ncand,
                                 int iterations, int peaks);

/* The fast form's objective and gradient (for checks): for pair i, the reference filtered with the wedges at
   pose T = poses[16 i..], and the particle at T perturbed by theta[6 i..] = (rotation vector w in radians about
   the box centre, shift d in voxels) of the output grid: rho[i] and, when grad is non-null, grad[6 i..] =
   d rho / d(w, d) at that perturbed pose. */
int ettk_gpu_refined_objective(ettk_ctx *ctx, int npairs, const int *pairs, const double *poses, const double *theta,
                               double *rho, double *grad);

/* The refinement objective and its gradient (for checks): for pair i at pose T = poses[16 i..] perturbed by
   theta[6 i..] = (rotation vector w in radians about the box centre, shift d in voxels) of the output grid,
   rho[i] and, when grad is non-null, grad[6 i..] = d rho / d(w, d) at that perturbed pose. */
int ettk_gpu_refine_objective(ettk_ctx *ctx, int npairs, const int *pairs, const double *poses,
                              const double *theta, double *rho, double *grad);

/* Diagnostic of the bounded device waits (no counterpart in the reference): one kernel polls an mbarrier that
 * nothing arrives at max_iter times (1 .. 2^24), gives up and flags it; the call returns ETTK_ERR_TIMEOUT, as any
 * call whose bulk copy or tensor-core commit never completes does, and the context stays usable. */
int ettk_gpu_wait_probe(ettk_ctx *ctx, int max_iter);

/* The context's launch shapes (ettk_tuning); set rejects values outside the lists above with ETTK_ERR_ARG. */
int ettk_gpu_get_tuning(ettk_ctx *ctx, ettk_tuning *t);
int ettk_gpu_set_tuning(ettk_ctx *ctx, const ettk_tuning *t);

/* Chooses the launch shapes for the context's references and particles (no reference counterpart): aligns the
 * npairs sample pairs (as ettk_gpu_align_pairs, 17 columns, one candidate, the particles' spherical projections
 * recomputed every time) under candidate shapes, one field at a time with the others at their best so far
 * (coordinate search over the values listed at ettk_tuning), each trial one warm-up and `repeats` timed runs
 * (median wall time of the synchronous call). A shape whose result rows differ from the first trial's in any bit
 * is rejected. The fastest shapes are applied to the context and written to *best (optional); report (optional,
 * report_size bytes) receives a JSON array with one object per trial. repeats 1..20. */
int ettk_gpu_autotune(ettk_ctx *ctx, int npairs, const int *pairs, int repeats, ettk_tuning *best, char *report,
                      int report_size);

/* Diagnostics (staged parity checks; no counterpart in the reference API):
 * one executeFourierNewHalf call (inc/em/nbfFourierImageMetric.h:1077-1323) of particle p against
 * reference r at transform t (updated in place with the found shift); returns the distance in *dist. */
int ettk_gpu_ccf(ettk_ctx *ctx, int r, int p, double *t, float *dist);

/* Diagnostics: the |FFT| spherical projection Pp (cartesianToSpherical, [2B][2B]) of particle p,
 * or of reference r when p < 0. */
int ettk_gpu_spherical_projection(ettk_ctx *ctx, int r, int p, float *Pp);

/* Diagnostics: SO(3) correlation of two real S^2 signals ([2B][2B]) on the (2B)^3 grid,
 * C[alpha][beta][gamma] (nbfProjectionRotationMetric3D::soft, 1136-1295); scaled != 0 applies
 * softScaled's min/max rescaling (1297-1319). */
int ettk_gpu_soft(ettk_ctx *ctx, const float *F1, const float *F2, int scaled, float *C);

/* SO(3) correlation of two real S^2 signals that allocates no memory. No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc where they need the correlation,
 * e.g. an application whose memory pool already owns the device memory or a process under a
 * fixed memory budget. d_F1, d_F2 ([2B][2B] floats) and d_C ([2B]^3 floats, C[alpha][beta][gamma]
 * as ettk_gpu_soft without scaling) are device buffers; the work is queued on `stream`
 * (a cudaStream_t, NULL = default stream) and the call returns without waiting for it.
 * Every intermediate lives in one 2 MiB file-scope device array of the library, so only B = 8 and
 * B = 16 are accepted (ETTK_ERR_ARG otherwise). The first call on a device sets that device's array
 * up (address and tables, then a device-wide synchronisation); make it before any stream capture on
 * the device, and do not use the entry point across a cudaDeviceReset of that device. All calls share
 * the array: calls whose GPU work overlaps race, so serialise them. */
int ettk_gpu_soft_noalloc(int B, const float *d_F1, const float *d_F2, float *d_C, void *stream);

/* Number of kernels this library launched since the context was created. */
long long ettk_gpu_kernel_launches(ettk_ctx *ctx);

/* The CUDA stream (cudaStream_t) all of this context's work is issued on, for timing with events. */
void *ettk_gpu_stream(ettk_ctx *ctx);

/* Per-kernel-family timing: enable != 0 records CUDA events around each kernel family on the
 * context stream (and clears earlier totals); ettk_gpu_profile_read returns family `index`
 * (0-based, ETTK_ERR_ARG past the end): its name, launch count, summed device time and the
 * algorithmic bytes those launches must move (one read of each input, one write of each output). */
int ettk_gpu_profile(ettk_ctx *ctx, int enable);
int ettk_gpu_profile_read(ettk_ctx *ctx, int index, char *name, int name_size, long long *launches,
                          double *total_ms, double *bytes);

/* Copies a description of the last error (NUL-terminated) into buf. */
int ettk_gpu_last_error(ettk_ctx *ctx, char *buf, int size);

#ifdef __cplusplus
}
#endif
#endif /* ETTK_GPU_H */
