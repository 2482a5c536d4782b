/* Implementation of the FFTW3 subset declared in shim/fftw3.h on top of the
 * oracle's FP64 FFT (fft64.cpp). Test infrastructure only. Supports the
 * plans SOFT builds: rank-1 or rank-2 advanced-interface complex DFTs whose
 * leading extents are 1 (a batch of contiguous-stride 1-D transforms). */
#include "fftw3.h"
#include "../fft64.h"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

struct ettk_fftw_plan_s {
  int n, howmany, istride, idist, ostride, odist, sign;
  fftw_complex *in, *out;
};

extern "C" fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany,
                                        fftw_complex *in, const int *inembed, int istride, int idist,
                                        fftw_complex *out, const int *onembed, int ostride, int odist,
                                        int sign, unsigned flags) {
  (void)inembed; (void)onembed; (void)flags;
  int len = 1;
  for (int r = 0; r < rank - 1; ++r) {
    if (n[r] != 1) { fprintf(stderr, "fftw shim: unsupported plan\n"); abort(); }
  }
  len = n[rank - 1];
  ettk_fftw_plan_s *p = new ettk_fftw_plan_s;
  p->n = len; p->howmany = howmany; p->istride = istride; p->idist = idist;
  p->ostride = ostride; p->odist = odist; p->sign = sign; p->in = in; p->out = out;
  return p;
}

extern "C" void fftw_execute(const fftw_plan p) {
  std::vector<oracle::cplx> line(p->n);
  for (int t = 0; t < p->howmany; ++t) {
    const double *src = &p->in[(long)t * p->idist][0];
    for (int i = 0; i < p->n; ++i)
      line[i] = oracle::cplx(src[2L * i * p->istride], src[2L * i * p->istride + 1]);
    oracle::fft1d(line.data(), p->n, p->sign, 1, 1, p->n);
    double *dst = &p->out[(long)t * p->odist][0];
    for (int i = 0; i < p->n; ++i) {
      dst[2L * i * p->ostride] = line[i].real();
      dst[2L * i * p->ostride + 1] = line[i].imag();
    }
  }
}

extern "C" void fftw_destroy_plan(fftw_plan p) { delete p; }
extern "C" void *fftw_malloc(size_t n) { return malloc(n); }
extern "C" void fftw_free(void *p) { free(p); }
