/* Thin C harness over the reference's SOFT 1.0 library, compiled from the
 * reference sources into oracle/_ref/ (test infrastructure only).
 * Each entry point calls SOFT in the same order and with the same arguments
 * as the reference's metric class does:
 *   ref_soft   -> nbfProjectionRotationMetric3D::soft
 *                 (inc/em/nbfProjectionRotationMetric3D.h:1136-1295,
 *                  tables and plan as in initializeHarmonics 1054-1134)
 *   ref_rotate -> nbfProjectionRotationMetric3D::harmonics(A, a, b, g, R)
 *                 (inc/em/nbfProjectionRotationMetric3D.h:1456-1554)
 *   ref_fst    -> the FST_semi_memo call inside soft (1184-1187)
 * Outputs use C (row-major) order: C[alpha][beta][gamma], R[beta][phi]. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "fftw3.h"
#include "complex.h"
#include "so3_correlate_fftw.h"
#include "soft_fftw.h"
#include "FST_semi_memo.h"
#include "cospmls.h"
#include "primitive_FST.h"
#include "seminaive.h"
#include "utils_so3.h"
#include "rotate_so3.h"

int ref_fst(int bw, const double *F, double *coefR, double *coefI) {
  int n = 2 * bw;
  double *sigR = (double *)malloc(sizeof(double) * n * n);
  double *sigI = (double *)calloc(n * n, sizeof(double));
  double *ws2 = (double *)malloc(sizeof(double) * 2 * ((14 * bw * bw) + (48 * bw)));
  double *tablespace = (double *)malloc(sizeof(double) *
      (Reduced_Naive_TableSize(bw, bw) + Reduced_SpharmonicTableSize(bw, bw)));
  double **table = SemiNaive_Naive_Pml_Table(bw, bw, tablespace, ws2);
  memcpy(sigR, F, sizeof(double) * n * n);
  FST_semi_memo(sigR, sigI, coefR, coefI, n, table, ws2, 1, bw);
  free(table); free(tablespace); free(ws2); free(sigI); free(sigR);
  return 0;
}

int ref_soft(int bw, const double *F1, const double *F2, double *C) {
  int bwIn = bw, bwOut = bw, degLim = bw - 1;
  int n = 2 * bwIn;
  double *sigR = (double *)malloc(sizeof(double) * n * n);
  double *sigI = (double *)calloc(n * n, sizeof(double));
  fftw_complex *so3Sig = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * (8 * bwOut * bwOut * bwOut));
  fftw_complex *ws1 = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * (8 * bwOut * bwOut * bwOut));
  fftw_complex *ws2 = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * ((14 * bwIn * bwIn) + (48 * bwIn)));
  double *ws3 = (double *)malloc(sizeof(double) * (12 * n + n * bwIn));
  double *sigCoefR = (double *)malloc(sizeof(double) * bwIn * bwIn);
  double *sigCoefI = (double *)malloc(sizeof(double) * bwIn * bwIn);
  double *patCoefR = (double *)malloc(sizeof(double) * bwIn * bwIn);
  double *patCoefI = (double *)malloc(sizeof(double) * bwIn * bwIn);
  fftw_complex *so3Coef = (fftw_complex *)fftw_malloc(sizeof(fftw_complex) * ((4 * bwOut * bwOut * bwOut - bwOut) / 3));
  double *tablespace = (double *)malloc(sizeof(double) *
      (Reduced_Naive_TableSize(bwIn, bwIn) + Reduced_SpharmonicTableSize(bwIn, bwIn)));
  int nn = 2 * bwOut;
  int na[2] = {1, nn}, inembed[2] = {nn, nn * nn}, onembed[2] = {nn, nn * nn};
  fftw_plan p1 = fftw_plan_many_dft(2, na, nn * nn, ws1, inembed, 1, nn, so3Sig, onembed, 1, nn,
                                    FFTW_FORWARD, FFTW_ESTIMATE);
  double **table = SemiNaive_Naive_Pml_Table(bwIn, bwIn, tablespace, (double *)ws2);

  memcpy(sigR, F1, sizeof(double) * n * n);
  FST_semi_memo(sigR, sigI, sigCoefR, sigCoefI, n, table, (double *)ws2, 1, bwIn);
  memcpy(sigR, F2, sizeof(double) * n * n);
  FST_semi_memo(sigR, sigI, patCoefR, patCoefI, n, table, (double *)ws2, 1, bwIn);
  so3CombineCoef_fftw(bwIn, bwOut, degLim, sigCoefR, sigCoefI, patCoefR, patCoefI, so3Coef);
  Inverse_SO3_Naive_fftw(bwOut, so3Coef, so3Sig, ws1, ws2, ws3, &p1, 1);

  for (int a = 0; a < nn; ++a)
    for (int b = 0; b < nn; ++b)
      for (int g = 0; g < nn; ++g)
        C[((long)a * nn + b) * nn + g] = so3Sig[((long)b * nn + a) * nn + g][0];

  fftw_destroy_plan(p1);
  free(table); free(tablespace); fftw_free(so3Coef);
  free(patCoefI); free(patCoefR); free(sigCoefI); free(sigCoefR);
  free(ws3); fftw_free(ws2); fftw_free(ws1); fftw_free(so3Sig); free(sigI); free(sigR);
  return 0;
}

int ref_rotate(int bw, const double *A, double alpha, double beta, double gamma, double *R) {
  int bwIn = bw, bwOut = bw, degOut = bw - 1;
  double *sigInR = (double *)malloc(sizeof(double) * 4 * bwIn * bwIn);
  double *sigInI = (double *)malloc(sizeof(double) * 4 * bwIn * bwIn);
  double *sigOutR = (double *)malloc(sizeof(double) * 4 * bwOut * bwOut);
  double *sigOutI = (double *)malloc(sizeof(double) * 4 * bwOut * bwOut);
  double *scratch = (double *)malloc(sizeof(double) * ((16 * bwIn * bwIn) + (48 * bwIn)));
  double *ts = (double *)malloc(sizeof(double) * (Reduced_Naive_TableSize(bwIn, bwIn) + Reduced_SpharmonicTableSize(bwIn, bwIn)));
  double *tts2 = (double *)malloc(sizeof(double) * (Reduced_Naive_TableSize(bwOut, bwOut) + Reduced_SpharmonicTableSize(bwOut, bwOut)));
  double *ts2 = (double *)malloc(sizeof(double) * (Reduced_Naive_TableSize(bwOut, bwOut) + Reduced_SpharmonicTableSize(bwOut, bwOut)));
  double **t1 = SemiNaive_Naive_Pml_Table(bwIn, bwIn, ts, scratch);
  double **t2 = SemiNaive_Naive_Pml_Table(bwOut, bwOut, ts2, scratch);
  double **tt2 = Transpose_SemiNaive_Naive_Pml_Table(t2, bwOut, bwOut, tts2, scratch);
  for (int i = 0; i < 4 * bwIn * bwIn; ++i) { sigInR[i] = A[i]; sigInI[i] = 0; }
  rotateFct(bwIn, bwOut, degOut, sigInR, sigInI, sigOutR, sigOutI, alpha, beta, gamma, scratch, t1, tt2);
  for (int i = 0; i < 4 * bwOut * bwOut; ++i) R[i] = sigOutR[i];
  free(tt2); free(t2); free(t1); free(ts2); free(tts2); free(ts);
  free(scratch); free(sigOutI); free(sigOutR); free(sigInI); free(sigInR);
  return 0;
}
