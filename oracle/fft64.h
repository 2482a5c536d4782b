/* Oracle FP64 FFT (test infrastructure only; never linked into the product).
 *
 * A project-written radix-2 FFT in double precision that follows FFTW3's
 * documented conventions, because the reference path calls FFTW3:
 *   - unnormalised transforms,
 *   - FORWARD uses exp(-2*pi*i*j*k/n), BACKWARD uses exp(+2*pi*i*j*k/n),
 *   - r2c/c2r of a d-dimensional row-major array halve the LAST dimension to
 *     n/2+1 complex values,
 *   - multi-dimensional c2r does the complex inverse transforms over the
 *     leading dimensions first and then a 1-D half-complex-to-real transform
 *     along the last dimension, which ignores the imaginary parts of the
 *     k=0 and k=n/2 elements (FFTW3 rdft/rank-geq2-rdft2.c order; the
 *     reference relies on it in inc/em/nbfFourierFilter.h:336-351 plans).
 * Only power-of-two lengths are supported (every box and bandwidth on the
 * alignment path is a power of two).
 */
#pragma once
#include <complex>
#include <vector>

namespace oracle {

typedef std::complex<double> cplx;

/* In-place 1-D complex FFT of length n (power of two), sign -1 forward, +1 backward,
 * over `count` vectors starting at data + t*dist, element stride `stride`. */
void fft1d(cplx *data, int n, int sign, int count, long stride, long dist);

/* 3-D real-to-complex: in[n0][n1][n2] (row-major) -> out[n0][n1][n2/2+1]. */
void rfft3d(const double *in, cplx *out, int n0, int n1, int n2);

/* 3-D complex-to-real (unnormalised): in[n0][n1][n2/2+1] -> out[n0][n1][n2].
 * The input is not modified. */
void irfft3d(const cplx *in, double *out, int n0, int n1, int n2);

bool is_pow2(int n);

} // namespace oracle
