/* correl.c -- the correlator files of bin/su2 (the reference's -DCORRELATORS
 * build, correlation.c:320-398): labels_correl and the blocks of correl<k>
 * (k = 0 the lattice itself, k >= 1 the blocking levels).  The values come
 * from su2gpu_measure_correlators / su2gpu_measure_blocked_correlators. */
#include <stdio.h>

#include "su2host.h"

void print_labels_correlators(const host_params* hp) {
  FILE* f = fopen("labels_correl", "w");
  if (!f) return;
  int k = 1;
  fprintf(f, "%d distance\n", k++);
  if (hp->nhiggs > 0) fprintf(f, "%d H(l) = sum_z h(z) h(z+l) / V\n", k++);
  if (hp->triplet) {
    fprintf(f, "%d Sigma^2 correlator\n", k++);
    fprintf(f, "%d projected photon correlator RE\n", k++);
    fprintf(f, "%d projected photon correlator IM\n", k++);
    fprintf(f, "%d projected photon correlator RE (p=2)\n", k++);
    fprintf(f, "%d projected photon correlator IM (p=2)\n", k++);
    fprintf(f, "%d alpha_munu RE (p=1)\n", k++);
    fprintf(f, "%d alpha_munu IM (p=1)\n", k++);
    fprintf(f, "%d alpha_munu RE (p=2)\n", k++);
    fprintf(f, "%d alpha_munu IM (p=2)\n", k++);
  }
  fclose(f);
}

void write_correlators(const char* fname, const host_params* hp, int meas_id, const double* rows, int nrows) {
  FILE* f = fopen(fname, "a");
  if (!f) return;
  fprintf(f, "\n =========== Measurement id: %d ===========\n", meas_id);
  for (int d = 0; d < nrows; d++) {
    const double* r = rows + (size_t)d * SU2GPU_NCORR;
    fprintf(f, "%d ", d);
    if (hp->nhiggs > 0) fprintf(f, "%g ", r[SU2GPU_CORR_HIGGS]);
    if (hp->triplet) {
      fprintf(f, "%g ", r[SU2GPU_CORR_SIGMA2]);
      fprintf(f, "%g %g %g %g ", r[SU2GPU_CORR_PHOT10_RE], r[SU2GPU_CORR_PHOT10_IM], r[SU2GPU_CORR_PHOT20_RE],
              r[SU2GPU_CORR_PHOT20_IM]);
      fprintf(f, "%g %g %g %g ", r[SU2GPU_CORR_PHOT11_RE], r[SU2GPU_CORR_PHOT11_IM], r[SU2GPU_CORR_PHOT21_RE],
              r[SU2GPU_CORR_PHOT21_IM]);
    }
    fprintf(f, "\n");
  }
  fclose(f);
}
