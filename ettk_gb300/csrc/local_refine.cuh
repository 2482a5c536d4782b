// Batched local 6-DOF refinement of the fast alignment form (ettk_gpu_align_pairs_refined). No counterpart in the
// reference: it takes the place of the Powell refinement (nbfFourierImageMetric::refine,
// inc/em/nbfFourierImageMetric.h:1701-1809) and of the mirror/candidate CCF loop of
// nbfProjectionRotationMetric3D::execute (inc/em/nbfProjectionRotationMetric3D.h:678-901) after the coarse SO(3) hit.
//
// Objective of pair e at index map M (output box index x -> particle index p(x) = o + M x):
//   rho = sum_x zm(x) (I(x) - mu) / sqrt( sum_x m(x)^2 (I(x) - mu)^2 * sum_x zm(x)^2 )
// with I(x) the trilinear interpolation at p(x) of the particle band-passed in its own frame by the metric's filter
// (particles cut from a tomogram are used unfiltered), coordinates clamped to the volume so that rho is continuous
// in the pose; m the spherical mask of the metric, mu = sum m I / sum m, and zm = m * y1, y1 = K(I1) the reference
// filtered as the CCF filters it (band-pass and B-factor times the wedges w1 w2(T0) at the coarse pose, DC
// removed). It is the masked normalised correlation of the wedge- and band-limited reference with the band-limited
// particle; the band limit keeps the trilinear interpolant smooth at the scale of a voxel.
//
// Gradient with respect to a right perturbation of the pose (rotation vector w about the box centre c, shift d,
// both in output voxels): dI/dd = G, dI/dw = (x - c) x G, G = M^T grad_p I (the analytic derivative of the
// trilinear interpolant; zero along an axis whose coordinate is clamped). One kernel evaluates the value and
// the gradient of every pair from 28 sums; one thread per pair updates the pose (gradient ascent with a step that
// grows on success and shrinks on failure, rotation preconditioned by the radius Rg).
#pragma once
#include "kernels.cuh"

namespace ettk {

constexpr int LR_NACC = 28;  // S1..S4, then 4 x 6 derivative sums

struct LRItem {
  const float *vol;  // particle volume (fixed image or tomogram), x fastest
  int dims[3];
  int zm_index;      // pair whose zm this evaluation uses
};

struct LRState {
  double base[12];   // accepted index map: origin, x, y, z axis columns
  double g[6];       // gradient of rho at base (w, d)
  double rho;        // rho at base (-inf before the first evaluation)
  double alpha;      // step length (output voxels at the radius Rg)
  double theta[6];   // perturbation of base under evaluation
  double czm, czz;   // sum zm, sum zm^2
  int done, accepted;
};

constexpr int LR_CHUNK = 8192;  // in-mask voxels per CTA of k_lr_eval

// Sums of pair e (acc[e][0..27]): S1 = sum m I, S2 = sum m^2 I, S3 = sum m^2 I^2, S4 = sum zm I, then for each
// derivative k (w0..w2, d0..d2): sum m D_k, sum m^2 D_k, sum m^2 I D_k, sum zm D_k. Every term carries m or zm = m y1,
// so only the nin voxels inside the mask (their indices in `in`, ascending) are visited: CTA (x, e) takes the chunk
// [x LR_CHUNK, (x + 1) LR_CHUNK) of them. FP32 per-thread partials, FP64 across the CTA and across CTAs.
template <int N>
__global__ void __launch_bounds__(256) k_lr_eval(const LRItem *__restrict__ items, const float *__restrict__ maps,
                                                 const float *__restrict__ zm, const float *__restrict__ mask,
                                                 const int *__restrict__ in, int nin, const LRState *__restrict__ state,
                                                 double *__restrict__ acc) {
  constexpr long n3 = (long)N * N * N;
  __shared__ float red[8][LR_NACC];
  const int e = blockIdx.y;
  if (state && state[e].done) return;  // a converged pair's sums are not read again
  const LRItem it = items[e];
  float M[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) M[k] = maps[(long)e * 12 + k];
  const float *Z = zm + (long)it.zm_index * n3;
  const float *V = it.vol;
  const int dx = it.dims[0], dy = it.dims[1], dz = it.dims[2];
  const long sy = dx, sz = (long)dx * dy;
  const float fx1 = (float)(dx - 1), fy1 = (float)(dy - 1), fz1 = (float)(dz - 1);
  const float c0 = 0.5f * (float)N;
  float s[LR_NACC];
#pragma unroll
  for (int k = 0; k < LR_NACC; ++k) s[k] = 0.f;
  const int v1 = min(nin, (int)(blockIdx.x + 1) * LR_CHUNK);
  // the next voxel's index is loaded one iteration ahead, so that its mask, operand and particle loads do not wait
  // behind the index load
  int v = blockIdx.x * LR_CHUNK + threadIdx.x;
  int id_next = v < v1 ? __ldg(in + v) : 0;
  for (; v < v1; v += blockDim.x) {
    const int id = id_next;
    if (v + (int)blockDim.x < v1) id_next = __ldg(in + v + blockDim.x);
    const int a = id / (N * N), b = (id / N) % N, c = id % N;
    const float mv = __ldg(mask + id);
    const float zv = __ldg(Z + id);
    const float px = M[0] + a * M[3] + b * M[6] + c * M[9];
    const float py = M[1] + a * M[4] + b * M[7] + c * M[10];
    const float pz = M[2] + a * M[5] + b * M[8] + c * M[11];
    const float qx = fminf(fmaxf(px, 0.f), fx1), qy = fminf(fmaxf(py, 0.f), fy1), qz = fminf(fmaxf(pz, 0.f), fz1);
    const int ix = min((int)qx, dx - 2), iy = min((int)qy, dy - 2), iz = min((int)qz, dz - 2);
    const float fx = qx - ix, fy = qy - iy, fz = qz - iz;
    const float *q = V + ix + iy * sy + iz * sz;
    const float v000 = __ldg(q), v100 = __ldg(q + 1), v010 = __ldg(q + sy), v110 = __ldg(q + sy + 1);
    const float v001 = __ldg(q + sz), v101 = __ldg(q + sz + 1), v011 = __ldg(q + sz + sy), v111 = __ldg(q + sz + sy + 1);
    const float c00 = v000 + fx * (v100 - v000), c10 = v010 + fx * (v110 - v010);
    const float c01 = v001 + fx * (v101 - v001), c11 = v011 + fx * (v111 - v011);
    const float e0 = c00 + fy * (c10 - c00), e1 = c01 + fy * (c11 - c01);
    const float I = e0 + fz * (e1 - e0);
    float gz = e1 - e0;
    float gy = (c10 - c00) + fz * ((c11 - c01) - (c10 - c00));
    const float d00 = v100 - v000, d10 = v110 - v010, d01 = v101 - v001, d11 = v111 - v011;
    const float h0 = d00 + fy * (d10 - d00), h1 = d01 + fy * (d11 - d01);
    float gx = h0 + fz * (h1 - h0);
    if (!(px > 0.f && px < fx1)) gx = 0.f;
    if (!(py > 0.f && py < fy1)) gy = 0.f;
    if (!(pz > 0.f && pz < fz1)) gz = 0.f;
    const float Ga = M[3] * gx + M[4] * gy + M[5] * gz;
    const float Gb = M[6] * gx + M[7] * gy + M[8] * gz;
    const float Gc = M[9] * gx + M[10] * gy + M[11] * gz;
    const float ra = a - c0, rb = b - c0, rc = c - c0;
    const float D[6] = {rb * Gc - rc * Gb, rc * Ga - ra * Gc, ra * Gb - rb * Ga, Ga, Gb, Gc};
    const float m2 = mv * mv, m2I = m2 * I;
    s[0] += mv * I;
    s[1] += m2I;
    s[2] += m2I * I;
    s[3] += zv * I;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      s[4 + k] += mv * D[k];
      s[10 + k] += m2 * D[k];
      s[16 + k] += m2I * D[k];
      s[22 + k] += zv * D[k];
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < LR_NACC; ++k) {
    float x = s[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[w][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < LR_NACC) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += (double)red[q][threadIdx.x];
    atomicAdd(&acc[(long)e * LR_NACC + threadIdx.x], t);
  }
}

// zm = m * y1 with the centring sign of the C2R output undone (the spectra are centred by multiplying the real
// input by (-1)^(i+j+k), so the C2R of a centred spectrum returns the signed volume); store of a C2R z pass.
struct PostStoreZm {
  float *y;
  const float *mask;
  int N;
  ETTK_DEV void begin() {}
  ETTK_DEV void end() {}
  ETTK_DEV void operator()(long line, int k, float v) {
    const long n2 = (long)N * N;
    const int r = (int)(line % n2);
    const float sg = (((r / N) + (r % N) + k) & 1) ? -1.f : 1.f;
    y[line * N + k] = v * sg * mask[(long)r * N + k];
  }
};

// Particle input of the band-pass pre-filter: the fixed image times the centring sign (-1)^(i+j+k) in the [z][y][x]
// memory order of the volume (i = z, j = y, k = x: the filter is radially symmetric, so the axis naming of the
// spectrum does not matter); item e reads vols + src[e] * N^3.
struct PreSignVol {
  const float *vols;
  const int *src;
  int N;
  ETTK_DEV void begin() {}
  ETTK_DEV void end() {}
  ETTK_DEV float operator()(long line, int k) {
    const long n2 = (long)N * N, e = line / n2;
    const int r = (int)(line - e * n2);
    const float sg = (((r / N) + (r % N) + k) & 1) ? -1.f : 1.f;
    return vols[(long)src[e] * n2 * N + (long)r * N + k] * sg;
  }
};

// Store of a C2R z pass with the centring sign undone (the band-passed particle in its own memory order).
struct PostStoreSigned {
  float *y;
  int N;
  ETTK_DEV void begin() {}
  ETTK_DEV void end() {}
  ETTK_DEV void operator()(long line, int k, float v) {
    const int r = (int)(line % ((long)N * N));
    y[line * N + k] = ((((r / N) + (r % N) + k) & 1) ? -v : v);
  }
};

// sum zm and sum zm^2 of each pair into state[e].czm / czz (one CTA per pair)
static __global__ void k_lr_consts(const float *__restrict__ zm, long n3, LRState *st) {
  __shared__ double sh[32];
  const float *Z = zm + (long)blockIdx.x * n3;
  float s1 = 0.f, s2 = 0.f;
  for (long i = threadIdx.x; i < n3; i += blockDim.x) {
    const float z = Z[i];
    s1 += z;
    s2 += z * z;
  }
  const double a = block_sum((double)s1, sh), b = block_sum((double)s2, sh);
  if (threadIdx.x == 0) {
    st[blockIdx.x].czm = a;
    st[blockIdx.x].czz = b;
  }
}

// p'(x) = M (exp([w]x)(x - c) + c + d) + o (the right perturbation of an index map; perturb_index on the host)
ETTK_HD void lr_perturb(const double in[12], double N, const double th[6], double out[12]) {
  const double w0 = th[0], w1 = th[1], w2 = th[2];
  const double t = sqrt(w0 * w0 + w1 * w1 + w2 * w2);
  double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (t > 0) {
    const double k0 = w0 / t, k1 = w1 / t, k2 = w2 / t, sn = sin(t), c1 = 1 - cos(t);
    const double K[9] = {0, -k2, k1, k2, 0, -k0, -k1, k0, 0};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const double k2ij = K[3 * i] * K[j] + K[3 * i + 1] * K[3 + j] + K[3 * i + 2] * K[6 + j];
        R[3 * i + j] += sn * K[3 * i + j] + c1 * k2ij;
      }
  }
  const double c = 0.5 * N;
  double tr[3];
  for (int i = 0; i < 3; ++i) tr[i] = c - (R[3 * i] + R[3 * i + 1] + R[3 * i + 2]) * c + th[3 + i];
  for (int i = 0; i < 3; ++i) {
    const double Mi0 = in[3 + i], Mi1 = in[6 + i], Mi2 = in[9 + i];
    out[i] = in[i] + Mi0 * tr[0] + Mi1 * tr[1] + Mi2 * tr[2];
    for (int col = 0; col < 3; ++col) out[3 + 3 * col + i] = Mi0 * R[col] + Mi1 * R[3 + col] + Mi2 * R[6 + col];
  }
}

// rho and its gradient from the 28 sums (C0 = sum m, C1 = sum m^2)
ETTK_HD double lr_objective(const double *a, double C0, double C1, double czm, double czz, double g[6]) {
  const double S1 = a[0], S2 = a[1], S3 = a[2], S4 = a[3];
  const double mu = S1 / C0;
  const double num = S4 - mu * czm;
  const double den2 = S3 - 2.0 * mu * S2 + mu * mu * C1;
  if (!(den2 > 0) || !(czz > 0)) {
    for (int k = 0; k < 6; ++k) g[k] = 0;
    return 0;
  }
  const double den = sqrt(den2 * czz);
  const double rho = num / den;
  for (int k = 0; k < 6; ++k) {
    const double dmu = a[4 + k] / C0;
    const double dnum = a[22 + k] - dmu * czm;
    const double dden2 = 2.0 * a[16 + k] - 2.0 * dmu * S2 - 2.0 * mu * a[10 + k] + 2.0 * mu * dmu * C1;
    g[k] = dnum / den - 0.5 * rho * dden2 / den2;
  }
  return rho;
}

// One thread per pair: read the evaluated sums, accept or reject the trial, choose the next trial and write its
// index map (FP32) for the next evaluation. Steps: t = alpha along the gradient preconditioned by Rg (rotation
// components in radians times Rg, i.e. the displacement at radius Rg); alpha grows x1.6 on success and shrinks
// x0.35 on failure; a pair is done when alpha < alpha_min.
static __global__ void k_lr_update(LRState *st, const double *__restrict__ acc, int P, double N, double C0, double C1,
                                   double Rg, double alpha_min, float *maps) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P) return;
  LRState S = st[e];
  double g[6];
  const double rho = lr_objective(acc + (long)e * LR_NACC, C0, C1, S.czm, S.czz, g);
  S.accepted = 0;
  if (!S.done && rho > S.rho) {
    double nb[12];
    lr_perturb(S.base, N, S.theta, nb);
    for (int k = 0; k < 12; ++k) S.base[k] = nb[k];
    for (int k = 0; k < 6; ++k) S.g[k] = g[k];
    if (S.rho > -1e300) S.alpha = fmin(S.alpha * 1.6, 4.0);
    S.rho = rho;
    S.accepted = 1;
  } else if (!S.done) {
    S.alpha *= 0.35;
  }
  if (S.alpha < alpha_min) S.done = 1;
  const double gu[6] = {S.g[0] / Rg, S.g[1] / Rg, S.g[2] / Rg, S.g[3], S.g[4], S.g[5]};
  double nrm = 0;
  for (int k = 0; k < 6; ++k) nrm += gu[k] * gu[k];
  nrm = sqrt(nrm);
  if (!(nrm > 0)) S.done = 1;
  for (int k = 0; k < 6; ++k) S.theta[k] = 0;
  if (!S.done) {
    const double t = S.alpha / nrm;
    for (int k = 0; k < 3; ++k) S.theta[k] = gu[k] * t / Rg;
    for (int k = 3; k < 6; ++k) S.theta[k] = gu[k] * t;
  }
  double m[12];
  lr_perturb(S.base, N, S.theta, m);
  for (int k = 0; k < 12; ++k) maps[(long)e * 12 + k] = (float)m[k];
  st[e] = S;
}

}  // namespace ettk
