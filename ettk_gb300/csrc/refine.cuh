// Continuous 6-DOF pose refinement: the hand-written adjoint of rotate-interpolate-constrained-correlation.
//
// Objective for one (reference, particle) pair at a pose of the particle's reslice (index map p(x) = M x + o
// from the output box to the fixed image, perturbed on the right by a rotation exp([w]x) about the box centre c
// and a shift d, p'(x) = M (exp([w]x)(x - c) + c + d) + o):
//   r     = tricubic reslice of the particle (getImage, inc/em/nbfWedgedSubImage3D.h:602-828) with the clamped
//           value everywhere (no background), so that r is smooth in the pose for every voxel
//   u     = valid * (r - mu) * w * (-1)^(x+y+z), mu = sum(w r) / sum(w) over valid voxels, w = m1
//           (executeFourierNewHalf's I2 input with the spherical raised-cosine mask m1 as the window in place
//           of maskfft and the mean of all valid voxels: m1 vanishes beyond its radius, so every windowed voxel
//           stays inside the fixed image and rho is smooth in the pose, where the box mean and the square
//           window would step whenever a corner voxel leaves the fixed image)
//   g     = K u,  K = C2R o diag(fw) o R2C                                  (wedge * band-pass filtered particle)
//   rho   = <y1, g>_m / sqrt(<y1, y1>_m <g, g>_m)                           (normalised CCF at zero lag, mask m1)
// with y1 = the reference filtered by the same fw (the I1 branch). rho is the correlation that the reference's
// distance (k1_m - max CCF, nbfFourierImageMetric.h:1243-1259) measures once the shift is part of the pose.
// Gradient: a = d rho / d g (k_ncc_adjoint); K is real and symmetric (fw is even in k), so d rho / d u = K a;
// d rho / d r_j = valid_j (d_j - w_j sum(d) / sum(w)), d_j = w_j (-1)^(x+y+z) (K a)_j; and
// d r_j / d(w, d) = grad_p tricubic(p_j) M [ (e_k x (x_j - c)) | e_k ]  (k_reslice_grad).
#pragma once
#include "kernels.cuh"

namespace ettk {

// d/df of the Catmull-Rom weights of cubic_weights (F0 = -f(f-1)^2/2, F1 = 1.5f^3 - 2.5f^2 + 1,
// F2 = -1.5f^3 + 2f^2 + f/2, F3 = (f^3 - f^2)/2)
ETTK_DEV void cubic_dweights(float D[4], float f) {
  D[0] = -0.5f * (f - 1.f) * (3.f * f - 1.f);
  D[1] = (4.5f * f - 5.f) * f;
  D[2] = (-4.5f * f + 4.f) * f + 0.5f;
  D[3] = (1.5f * f - 1.f) * f;
}

// sum(w v) and sum(w) over the valid voxels (v > -max) of each resliced item into acc[e*2 + 0..1] (w: window)
static __global__ void k_masked_mean(const float *__restrict__ v, const float *__restrict__ maskfft, int n3,
                                     double *acc) {
  __shared__ double sh[32];
  const float *V = v + (long)blockIdx.y * n3;
  float s = 0.f, w = 0.f;
  for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < n3; id += gridDim.x * blockDim.x) {
    const float x = V[id];
    if (x > -FLT_MAX) {
      s += maskfft[id] * x;
      w += maskfft[id];
    }
  }
  const double a = block_sum((double)s, sh), b = block_sum((double)w, sh);
  if (threadIdx.x == 0) {
    atomicAdd(&acc[(long)blockIdx.y * 2 + 0], a);
    atomicAdd(&acc[(long)blockIdx.y * 2 + 1], b);
  }
}

// Particle input of the refinement: (valid ? v - mu : 0) * w * shift, mu = acc[e*2] / acc[e*2 + 1] (w: window).
struct PreMaskedParticle {
  const float *v;
  const float *maskfft;
  const double *acc;
  int N;
  ETTK_DEV void begin() {}
  ETTK_DEV void end() {}
  ETTK_DEV float operator()(long line, int k) {
    const long n2 = (long)N * N, e = line / n2;
    const int r = (int)(line - e * n2);
    const double w = acc[e * 2 + 1];
    const float mu = w > 0 ? (float)(acc[e * 2] / w) : 0.f;
    const float val = v[line * N + k];
    const float out = (val > -FLT_MAX) ? val - mu : 0.f;
    return out * maskfft[(long)r * N + k] * ((((r / N) + (r % N) + k) & 1) ? -1.f : 1.f);
  }
};

// Real input of the backward R2C (the adjoint field).
struct PreCopy {
  const float *y;
  int N;
  ETTK_DEV void begin() {}
  ETTK_DEV void end() {}
  ETTK_DEV float operator()(long line, int k) { return y[line * N + k]; }
};

// Forward (x, y) passes then * fw[fw_index[e]] with the DC zeroed (several evaluations may share a pair's fw).
template <int N>
struct OpFwdFilterIdx {
  float2 *d;
  const float *fw;
  const int *fw_index;
  int sign = -1;
  ETTK_DEV void begin() {}
  ETTK_DEV float2 load(int e, int kz, int i) const { return d[KXY<N>::at(e, kz, i)]; }
  ETTK_DEV void store(int e, int kz, int i, int, int, float2 v) {
    v = cscale(v, fw[KXY<N>::at(fw_index[e], kz, i)]);
    if (kz == KXY<N>::H - 1 && i == KXY<N>::dc_xy) v = make_float2(0.f, 0.f);
    d[KXY<N>::at(e, kz, i)] = v;
  }
  ETTK_DEV void end(int, int) {}
};

// Per evaluation e: S_yg = sum m y1 g, S_gg = sum m g^2, S_yy = sum m y1^2 into acc[e*4 + 0..2]
// (y1 of pair y_index[e]; FP32 per-thread partials, FP64 across threads).
static __global__ void k_ncc_sums(const float *__restrict__ y1, const int *__restrict__ y_index,
                                  const float *__restrict__ g, const float *__restrict__ m, int n3, double *acc) {
  __shared__ double sh[32];
  const int e = blockIdx.y;
  const float *Y = y1 + (long)y_index[e] * n3, *G = g + (long)e * n3;
  float syg = 0.f, sgg = 0.f, syy = 0.f;
  for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < n3; id += gridDim.x * blockDim.x) {
    const float w = m[id], y = Y[id], v = G[id];
    syg += w * y * v;
    sgg += w * v * v;
    syy += w * y * y;
  }
  const double a = block_sum((double)syg, sh), b = block_sum((double)sgg, sh), c = block_sum((double)syy, sh);
  if (threadIdx.x == 0) {
    atomicAdd(&acc[(long)e * 4 + 0], a);
    atomicAdd(&acc[(long)e * 4 + 1], b);
    atomicAdd(&acc[(long)e * 4 + 2], c);
  }
}

// a = d rho / d g = m (y1 / sqrt(S_yy S_gg) - rho g / S_gg)
static __global__ void k_ncc_adjoint(const float *__restrict__ y1, const int *__restrict__ y_index,
                                     const float *__restrict__ g, const float *__restrict__ m, int n3,
                                     const double *__restrict__ acc, float *__restrict__ a) {
  const int e = blockIdx.y;
  const double syg = acc[(long)e * 4 + 0], sgg = acc[(long)e * 4 + 1], syy = acc[(long)e * 4 + 2];
  const double den = sqrt(syy * sgg);
  const float c1 = den > 0 ? (float)(1.0 / den) : 0.f;
  const float c2 = (den > 0 && sgg > 0) ? (float)(syg / den / sgg) : 0.f;
  const float *Y = y1 + (long)y_index[e] * n3, *G = g + (long)e * n3;
  float *A = a + (long)e * n3;
  for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < n3; id += gridDim.x * blockDim.x)
    A[id] = m[id] * (Y[id] * c1 - G[id] * c2);
}

// Gradient sums of one evaluation (output box [x][y][z], z fastest, as the reslice): for every valid voxel j
// (v_j > -max), d_j = w_j (-1)^(x+y+z) b_j with b = K a (w: the window), q_j = M^T grad_p tricubic(p_j) (the gradient
// in output-box coordinates) and x_j - c:
//   acc[e*16 + 0..2]  = sum d q          acc[3..5]  = sum d (x - c) x q
//   acc[6..8]         = sum w q          acc[9..11] = sum w (x - c) x q
//   acc[12] = sum d,  acc[13] = sum w
// so that d rho / d d = acc[0..2] - dbar acc[6..8] and d rho / d w = acc[3..5] - dbar acc[9..11],
// dbar = acc[12] / acc[13]. Taps are clamped as in the reslice; the weights use the same 2^-16 fraction.
static __global__ void __launch_bounds__(256) k_reslice_grad(const ResliceItem *__restrict__ items, int N,
                                                             const float *__restrict__ v, const float *__restrict__ b,
                                                             const float *__restrict__ maskfft, double *acc) {
  __shared__ double sh[32];
  const ResliceItem &it = items[blockIdx.y];
  const int dx = it.dims[0], dy = it.dims[1], dz = it.dims[2];
  const long n3 = (long)N * N * N;
  const float *V = v + (long)blockIdx.y * n3, *Bv = b + (long)blockIdx.y * n3;
  const float c0 = 0.5f * (float)N;
  float s[14];
#pragma unroll
  for (int t = 0; t < 14; ++t) s[t] = 0.f;
  for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < (int)n3; id += gridDim.x * blockDim.x) {
    if (!(V[id] > -FLT_MAX)) continue;
    const int a = id / (N * N), bb = (id / N) % N, cz = id % N;
    float p0 = it.m[0] + cz * it.m[9], p1 = it.m[1] + cz * it.m[10], p2 = it.m[2] + cz * it.m[11];
    p0 = p0 + bb * it.m[6];
    p1 = p1 + bb * it.m[7];
    p2 = p2 + bb * it.m[8];
    p0 = p0 + a * it.m[3];
    p1 = p1 + a * it.m[4];
    p2 = p2 + a * it.m[5];
    float fx, fy, fz;
    const int ix = vtk_floor(p0, fx), iy = vtk_floor(p1, fy), iz = vtk_floor(p2, fz);
    float wx[4], wy[4], wz[4], gx[4], gy[4], gz[4];
    cubic_weights(wx, fx);
    cubic_weights(wy, fy);
    cubic_weights(wz, fz);
    cubic_dweights(gx, fx);
    cubic_dweights(gy, fy);
    cubic_dweights(gz, fz);
    int xs[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) xs[t] = min(max(ix - 1 + t, 0), dx - 1);
    float d0 = 0.f, d1 = 0.f, d2 = 0.f;  // grad_p in fixed-image index coordinates
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int zz = min(max(iz - 1 + k, 0), dz - 1);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int yy = min(max(iy - 1 + j, 0), dy - 1);
        const float *row = it.vol + ((long)zz * dy + yy) * dx;
        const float t0 = __ldg(row + xs[0]), t1 = __ldg(row + xs[1]), t2 = __ldg(row + xs[2]), t3 = __ldg(row + xs[3]);
        const float vx = wx[0] * t0 + wx[1] * t1 + wx[2] * t2 + wx[3] * t3;
        const float gxx = gx[0] * t0 + gx[1] * t1 + gx[2] * t2 + gx[3] * t3;
        d0 += wz[k] * wy[j] * gxx;
        d1 += wz[k] * gy[j] * vx;
        d2 += gz[k] * wy[j] * vx;
      }
    }
    // q = M^T grad (columns of M: the x, y, z axes of the output box in fixed-image index units)
    const float q0 = it.m[3] * d0 + it.m[4] * d1 + it.m[5] * d2;
    const float q1 = it.m[6] * d0 + it.m[7] * d1 + it.m[8] * d2;
    const float q2 = it.m[9] * d0 + it.m[10] * d1 + it.m[11] * d2;
    const float r0 = a - c0, r1 = bb - c0, r2 = cz - c0;
    const float c0q = r1 * q2 - r2 * q1, c1q = r2 * q0 - r0 * q2, c2q = r0 * q1 - r1 * q0;  // (x - c) x q
    const float mj = maskfft[id];
    const float dj = mj * Bv[id] * parity_sign(a, bb, cz);
    s[0] += dj * q0;
    s[1] += dj * q1;
    s[2] += dj * q2;
    s[3] += dj * c0q;
    s[4] += dj * c1q;
    s[5] += dj * c2q;
    s[6] += mj * q0;
    s[7] += mj * q1;
    s[8] += mj * q2;
    s[9] += mj * c0q;
    s[10] += mj * c1q;
    s[11] += mj * c2q;
    s[12] += dj;
    s[13] += mj;
  }
#pragma unroll 1
  for (int t = 0; t < 14; ++t) {
    const double tot = block_sum((double)s[t], sh);
    if (threadIdx.x == 0) atomicAdd(&acc[(long)blockIdx.y * 16 + t], tot);
  }
}

}  // namespace ettk
