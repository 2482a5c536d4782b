/* Project-written stand-in for the subset of the FFTW3 API that the SOFT 1.0
 * sources on the reference's alignment path use (fftw_plan_many_dft,
 * fftw_execute, fftw_malloc/free, fftw_destroy_plan). FFTW3 itself is absent
 * from this machine. Used only to build the SOFT reference library under
 * oracle/_ref for validating the oracle (test infrastructure, not product).
 * Semantics follow FFTW3's documentation: unnormalised, FORWARD = exp(-i..),
 * BACKWARD = exp(+i..), advanced-interface strides/distances in elements. */
#ifndef ETTK_ORACLE_FFTW3_SHIM_H
#define ETTK_ORACLE_FFTW3_SHIM_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef double fftw_complex[2];
typedef struct ettk_fftw_plan_s *fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
fftw_plan fftw_plan_many_dft(int rank, const int *n, int howmany,
                             fftw_complex *in, const int *inembed, int istride, int idist,
                             fftw_complex *out, const int *onembed, int ostride, int odist,
                             int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void *fftw_malloc(size_t n);
void fftw_free(void *p);
#ifdef __cplusplus
}
#endif
#endif
