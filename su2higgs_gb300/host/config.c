/* config.c -- key/value config reader with the reference's lookup rules
 * (parameters.c:12-149): "key value" lines, '#' comments, keys compared
 * case-insensitively, the search continues from the current file position
 * and wraps around once; a missing key is fatal (exit code 1).  Keys are
 * read in the reference's order (get_parameters, parameters.c:157-338) so a
 * config with repeated keys resolves the same way. */
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <time.h>
#include <unistd.h>

#include "su2host.h"

#define LINELEN 200

void die(int code) { exit(code); }

int cfg_open(const char* fname, FILE** f) {
  if (access(fname, R_OK) != 0) {
    printf("!!! Unable to access file %s\n", fname);
    return 0;
  }
  *f = fopen(fname, "r");
  return *f != NULL;
}

int cfg_find(FILE* f, const char* label, char* result) {
  char line[LINELEN], key[LINELEN], value[LINELEN];
  int wrapped = 0;
  result[0] = 0;
  value[0] = 0;
  while (!feof(f)) {
    if (!fgets(line, LINELEN, f)) {
      if (wrapped) break;
      wrapped = 1;
      rewind(f);
      continue;
    }
    int n = sscanf(line, "%99s%99s", key, value);
    if (n == EOF) continue;
    if (key[0] == '#') continue;
    if (!strcasecmp(key, label)) {
      strcpy(result, value);
      break;
    }
  }
  return result[0] != 0;
}

static void find_or_die(FILE* f, const char* label, char* result) {
  if (!cfg_find(f, label, result)) {
    printf("!!! Unable to find parameter %s in file\n", label);
    die(1);
  }
}

int cfg_get_int(FILE* f, const char* label) {
  char v[LINELEN];
  find_or_die(f, label, v);
  return (int)strtol(v, NULL, 10);
}
long cfg_get_long(FILE* f, const char* label) {
  char v[LINELEN];
  find_or_die(f, label, v);
  return strtol(v, NULL, 10);
}
double cfg_get_double(FILE* f, const char* label) {
  char v[LINELEN];
  find_or_die(f, label, v);
  return strtod(v, NULL);
}
void cfg_get_string(FILE* f, const char* label, char* result) { find_or_die(f, label, result); }

int cfg_get_algorithm(FILE* f, const char* label) {
  char a[LINELEN];
  cfg_get_string(f, label, a);
  if (!strcasecmp(a, "metropolis")) return SU2GPU_METROPOLIS;
  if (!strcasecmp(a, "heatbath")) return SU2GPU_HEATBATH;
  if (!strcasecmp(a, "overrelax")) return SU2GPU_OVERRELAX;
  printf("WARNING: Unknown update algorithm for '%s'; using metropolis instead.", label);
  return SU2GPU_METROPOLIS;
}

/* keys of this implementation: looked up from the file start, never fatal */
int cfg_optional_string(const char* fname, const char* label, char* result) {
  FILE* f = fopen(fname, "r");
  if (!f) return 0;
  int ok = cfg_find(f, label, result);
  fclose(f);
  return ok;
}

static int opt_int(const char* fname, const char* label, int dflt) {
  char v[LINELEN];
  return cfg_optional_string(fname, label, v) ? (int)strtol(v, NULL, 10) : dflt;
}

/* field content: the reference fixes it at compile time (-DNHIGGS, -DTRIPLET,
 * -DSINGLET, -DU1, -DGRADFLOW; default Makefile:12 = NHIGGS=1 SINGLET U1).
 * Here the optional keys nhiggs/triplet/singlet/u1/gradflow select it; the
 * environment variable SU2_CONTENT (a name: pure, fund, adj, su2u1s, fundadj,
 * higgs2, optionally +gradflow, +measure_z, +hb_trajectory, +correlators
 * and +blocking) is applied before them. */
static void read_content(const char* fname, host_params* hp) {
  hp->nhiggs = 1; hp->triplet = 0; hp->singlet = 1; hp->u1 = 1; hp->gradflow = 0; hp->measure_z = 0;
  hp->hb_trajectory = 0; hp->correlators = 0; hp->blocking = 0;
  const char* env = getenv("SU2_CONTENT");
  if (env && *env) {
    char name[64];
    snprintf(name, sizeof(name), "%s", env);
    /* modifiers after the name: +gradflow (-DGRADFLOW), +measure_z
     * (-DMEASURE_Z), +hb_trajectory (-DHB_TRAJECTORY), +correlators
     * (-DCORRELATORS), +blocking (-DBLOCKING) */
    char* plus = strchr(name, '+');
    if (plus) {
      *plus = 0;
      char* tok = plus + 1;
      while (tok && *tok) {
        char* next = strchr(tok, '+');
        if (next) *next++ = 0;
        if (!strcasecmp(tok, "gradflow")) hp->gradflow = 1;
        else if (!strcasecmp(tok, "measure_z")) hp->measure_z = 1;
        else if (!strcasecmp(tok, "hb_trajectory")) hp->hb_trajectory = 1;
        else if (!strcasecmp(tok, "correlators")) hp->correlators = 1;
        else if (!strcasecmp(tok, "blocking")) hp->blocking = 1;
        else { printf("!!! Unknown SU2_CONTENT modifier %s\n", tok); die(2); }
        tok = next;
      }
    }
    if (!strcasecmp(name, "pure")) { hp->nhiggs = 0; hp->triplet = 0; hp->singlet = 0; hp->u1 = 0; }
    else if (!strcasecmp(name, "fund")) { hp->nhiggs = 1; hp->triplet = 0; hp->singlet = 0; hp->u1 = 0; }
    else if (!strcasecmp(name, "adj")) { hp->nhiggs = 0; hp->triplet = 1; hp->singlet = 0; hp->u1 = 0; }
    else if (!strcasecmp(name, "su2u1s")) { hp->nhiggs = 1; hp->triplet = 0; hp->singlet = 1; hp->u1 = 1; }
    else if (!strcasecmp(name, "fundadj")) { hp->nhiggs = 1; hp->triplet = 1; hp->singlet = 0; hp->u1 = 0; }
    else if (!strcasecmp(name, "higgs2")) { hp->nhiggs = 2; hp->triplet = 0; hp->singlet = 0; hp->u1 = 1; }
    else { printf("!!! Unknown SU2_CONTENT %s\n", env); die(2); }
  }
  hp->nhiggs = opt_int(fname, "nhiggs", hp->nhiggs);
  hp->triplet = opt_int(fname, "triplet", hp->triplet);
  hp->singlet = opt_int(fname, "singlet", hp->singlet);
  hp->u1 = opt_int(fname, "u1", hp->u1);
  hp->gradflow = opt_int(fname, "gradflow", hp->gradflow);
  hp->measure_z = opt_int(fname, "measure_z", hp->measure_z);
  hp->hb_trajectory = opt_int(fname, "hb_trajectory", hp->hb_trajectory);
  hp->correlators = opt_int(fname, "correlators", hp->correlators);
  hp->blocking = opt_int(fname, "blocking", hp->blocking);
}

void read_parameters(const char* fname, host_params* hp) {
  memset(hp, 0, sizeof(*hp));
  read_content(fname, hp);
  su2gpu_params* p = &hp->p;
  FILE* f = NULL;
  if (!cfg_open(fname, &f)) die(1);
  p->dim = cfg_get_int(f, "dim");
  for (int d = 0; d < p->dim && d < 4; d++) {
    char lab[16];
    snprintf(lab, sizeof(lab), "L%d", d + 1);
    p->L[d] = cfg_get_int(f, lab);
    if (p->L[d] % 2 != 0)
      printf("!!! WARNING: Lattice side length L%d is an odd number! Checkerboard updating is not well defined\n", d);
  }
  cfg_get_string(f, "resultsfile", hp->resultsfile);
  int alg = cfg_get_algorithm(f, "algorithm_su2link");
  if (!(alg == SU2GPU_METROPOLIS || alg == SU2GPU_HEATBATH)) {
    printf("Cannot use algorithm %d for SU2 links, changing to metropolis...", alg);
    alg = SU2GPU_METROPOLIS;
  }
  p->algorithm_su2link = alg;
  p->algorithm_u1link = SU2GPU_METROPOLIS;
  if (hp->u1) {
    alg = cfg_get_algorithm(f, "algorithm_u1link");
    if (alg != SU2GPU_METROPOLIS) {
      printf("Cannot use algorithm %d for U1 links, changing to metropolis...", alg);
      alg = SU2GPU_METROPOLIS;
    }
    p->algorithm_u1link = alg;
  }
  if (hp->nhiggs > 0) {
    alg = cfg_get_algorithm(f, "algorithm_su2doublet");
    if (!(alg == SU2GPU_METROPOLIS || alg == SU2GPU_OVERRELAX)) {
      printf("Cannot use algorithm %d for doublets, changing to metropolis...", alg);
      alg = SU2GPU_METROPOLIS;
    }
    p->algorithm_su2doublet = alg;
  }
  if (hp->triplet) {
    alg = cfg_get_algorithm(f, "algorithm_su2triplet");
    if (!(alg == SU2GPU_METROPOLIS || alg == SU2GPU_OVERRELAX)) {
      printf("Cannot use algorithm %d for triplets, changing to metropolis...", alg);
      alg = SU2GPU_METROPOLIS;
    }
    p->algorithm_su2triplet = alg;
  }
  if (hp->singlet) {
    alg = cfg_get_algorithm(f, "algorithm_singlet");
    if (!(alg == SU2GPU_METROPOLIS || alg == SU2GPU_OVERRELAX)) {
      printf("Cannot use algorithm %d for singlets, changing to metropolis...", alg);
      alg = SU2GPU_METROPOLIS;
    }
    p->algorithm_singlet = alg;
  }
  cfg_get_string(f, "latticefile", hp->latticefile);
  hp->iterations = cfg_get_long(f, "iterations");
  hp->interval = cfg_get_long(f, "interval");
  hp->checkpoint = cfg_get_long(f, "checkpoint");
  hp->n_thermalize = cfg_get_long(f, "n_thermalize");
  hp->run_checks = cfg_get_int(f, "run_checks");
  hp->reset = cfg_get_int(f, "reset");
  hp->multicanonical = cfg_get_int(f, "multicanonical");
  hp->do_local_meas = cfg_get_int(f, "measure_local");
  if (hp->measure_z) hp->meas_interval_z = cfg_get_long(f, "interval_z");
  p->update_links = cfg_get_int(f, "update_links");
  p->update_su2doublet = cfg_get_int(f, "update_doublet");
  p->scalar_sweeps = cfg_get_int(f, "scalar_sweeps");
  p->betasu2 = cfg_get_double(f, "betasu2");
  if (hp->nhiggs > 0) {
    p->msq_phi = cfg_get_double(f, "msq");
    p->lambda_phi = cfg_get_double(f, "lambda");
    hp->phi0 = cfg_get_double(f, "phi0");
  }
  if (hp->u1) {
    p->betau1 = cfg_get_double(f, "betau1");
    p->r_u1 = cfg_get_double(f, "r_u1");
  }
  if (hp->triplet) {
    p->update_su2triplet = cfg_get_int(f, "update_triplet");
    hp->sigma0 = cfg_get_double(f, "sigma0");
    p->msq_triplet = cfg_get_double(f, "msq_triplet");
    p->b4 = cfg_get_double(f, "b4");
    if (hp->nhiggs > 0) p->a2 = cfg_get_double(f, "a2");
  }
  if (hp->singlet) {
    p->update_singlet = cfg_get_int(f, "update_singlet");
    hp->singlet0 = cfg_get_double(f, "singlet0");
    p->b1_s = cfg_get_double(f, "b1_s");
    p->msq_s = cfg_get_double(f, "msq_s");
    p->b3_s = cfg_get_double(f, "b3_s");
    p->b4_s = cfg_get_double(f, "b4_s");
    if (hp->nhiggs > 0) {
      p->a1_s = cfg_get_double(f, "a1_s");
      p->a2_s = cfg_get_double(f, "a2_s");
    }
  }
  if (hp->nhiggs == 2) {
    p->msq_phi2 = cfg_get_double(f, "msq_phi2");
    p->m12sq_re = cfg_get_double(f, "m12sq_re");
    p->m12sq_im = cfg_get_double(f, "m12sq_im");
    p->lam2 = cfg_get_double(f, "lam2");
    p->lam3 = cfg_get_double(f, "lam3");
    p->lam4 = cfg_get_double(f, "lam4");
    p->lam5_re = cfg_get_double(f, "lam5_re");
    p->lam5_im = cfg_get_double(f, "lam5_im");
    p->lam6_re = cfg_get_double(f, "lam6_re");
    p->lam6_im = cfg_get_double(f, "lam6_im");
    p->lam7_re = cfg_get_double(f, "lam7_re");
    p->lam7_im = cfg_get_double(f, "lam7_im");
  }
  hp->do_trajectory = hp->hb_trajectory ? cfg_get_int(f, "do_trajectory") : 0; /* parameters.c:319-321 */
  /* parameters.c:310-317 */
  if (hp->correlators) {
    hp->do_correlators = cfg_get_int(f, "do_correlators");
    hp->correlator_interval = cfg_get_int(f, "correlator_interval");
  }
  if (hp->blocking) hp->blocks = cfg_get_int(f, "blocks");
  if (hp->gradflow) {
    hp->do_flow = cfg_get_int(f, "do_flow");
    hp->flow_interval = cfg_get_int(f, "flow_interval");
    hp->flow_meas_interval = cfg_get_int(f, "flow_meas_interval");
    hp->flow_dt = cfg_get_double(f, "flow_dt");
    hp->flow_t_max = cfg_get_double(f, "flow_t_max");
  }
  if (hp->measure_z) {
    hp->do_z_meas = cfg_get_int(f, "do_z_meas");
    hp->setup_wall = cfg_get_int(f, "setup_wall");
  }
  fclose(f);

  /* content, precision and run options of this implementation */
  p->content = (hp->nhiggs == 1 ? SU2GPU_HIGGS1 : 0) | (hp->nhiggs == 2 ? SU2GPU_HIGGS2 : 0) |
               (hp->triplet ? SU2GPU_TRIPLET : 0) | (hp->singlet ? SU2GPU_SINGLET : 0) | (hp->u1 ? SU2GPU_U1 : 0) |
               (hp->gradflow ? SU2GPU_GRADFLOW : 0);
  p->precision = opt_int(fname, "precision", 64);
  p->reunitarize_interval = opt_int(fname, "reunitarize_interval", 10);
  hp->use_graph = opt_int(fname, "gpu_graph", 1);
  hp->file_ranks = 1;
  hp->lattice_mpi_size = opt_int(fname, "lattice_mpi_size", 0);
  char v[LINELEN];
  if (cfg_optional_string(fname, "seed", v)) {
    hp->seed = strtoull(v, NULL, 10);
    hp->have_seed = 1;
  }
}

void read_weight_parameters(const char* fname, const host_params* hp, host_muca* hm) {
  memset(hm, 0, sizeof(*hm));
  if (!hp->multicanonical) {
    strcpy(hm->weightfile, "weight");
    hm->orderparam = -1;
    return;
  }
  FILE* f = NULL;
  if (!cfg_open(fname, &f)) die(2);
  cfg_get_string(f, "weightfile", hm->weightfile);
  hm->mode = cfg_get_int(f, "muca_mode");
  hm->checks_per_sweep = cfg_get_int(f, "checks_per_sweep");
  hm->bins = cfg_get_int(f, "bins");
  hm->min = cfg_get_double(f, "min");
  hm->max = cfg_get_double(f, "max");
  hm->delta = cfg_get_double(f, "muca_delta");
  char name[LINELEN];
  cfg_get_string(f, "orderparam", name);
  if (!strcasecmp(name, "phisq")) hm->orderparam = SU2GPU_PHISQ;
  else if (!strcasecmp(name, "Sigmasq")) hm->orderparam = SU2GPU_SIGMASQ;
  else if (!strcasecmp(name, "phi2sq")) hm->orderparam = SU2GPU_PHI2SQ;
  else if (!strcasecmp(name, "phi2minusSigma2")) hm->orderparam = SU2GPU_PHI2MINUSSIGMA2;
  else {
    printf("WARNING: Unknown multicanonical order parameter!! using phisq");
    hm->orderparam = SU2GPU_PHISQ;
  }
  if (hm->mode != SU2GPU_MUCA_READONLY && hm->mode != SU2GPU_MUCA_FAST && hm->mode != SU2GPU_MUCA_SLOW) {
    printf("Invalid mode specification for multicanonical!! got mode=%d\n", hm->mode);
    printf("%d = read only, %d = fast weight update, %d = slow weight update\n", 0, 1, 2);
    die(551);
  }
  fclose(f);
}

/* read_updated_parameters (parameters.c:460-494) */
void read_updated_parameters(const char* fname, host_params* hp) {
  FILE* f = NULL;
  if (!cfg_open(fname, &f)) {
    printf("!!! Warning: Unable to access config file %s at checkpoint; skipping read...\n", fname);
    return;
  }
  long nw = cfg_get_long(f, "iterations");
  if (hp->iterations != nw) { hp->iterations = nw; printf("Updated max iterations to %ld\n", nw); }
  nw = cfg_get_long(f, "interval");
  if (hp->interval != nw) { hp->interval = nw; printf("Updated measurement interval to %ld\n", nw); }
  nw = cfg_get_long(f, "checkpoint");
  if (hp->checkpoint != nw) { hp->checkpoint = nw; printf("Updated checkpoint interval to %ld\n", nw); }
  fclose(f);
}

void print_parameters(const host_params* hp) {
  const su2gpu_params* p = &hp->p;
  long vol = 1;
  printf("Volume ");
  for (int d = 0; d < p->dim; d++) {
    if (d > 0) printf(" x ");
    printf("%d", p->L[d]);
    vol *= p->L[d];
  }
  printf(", total %lu\n", vol);
  printf("iterations %lu, measurement interval %lu, checkpoint interval %lu\n", hp->iterations, hp->interval,
         hp->checkpoint);
  printf("Will perform %d gauge sweeps, %d scalar sweeps per iteration\n", p->update_links, p->scalar_sweeps);
  printf("-------------------------- Lattice parameters --------------------------\n");
  printf("SU(2) beta %g\n", p->betasu2);
  if (hp->u1) printf("U(1) beta %g, U(1) r %g\n", p->betau1, p->r_u1);
  if (hp->nhiggs == 2) {
    printf("msq1 %g, msq2 %g, m12sq_re %g, m12sq_im %g \n", p->msq_phi, p->msq_phi2, p->m12sq_re, p->m12sq_im);
    printf("lam1 %g, lam2 %g, lam3 %g, lam4 %g, lam5_re %g, lam5_im %g \n", p->lambda_phi, p->lam2, p->lam3, p->lam4,
           p->lam5_re, p->lam5_im);
    printf("lam6_re %g, lam6_im %g, lam7_re %g, lam7_im %g \n", p->lam6_re, p->lam6_im, p->lam7_re, p->lam7_im);
    printf("initial phi0 %g, update_su2doublet %d\n", hp->phi0, p->update_su2doublet);
  } else if (hp->nhiggs == 1) {
    printf("msq (Higgs) %g, lambda (Higgs) %g, ", p->msq_phi, p->lambda_phi);
    printf("initial phi0 %g, update_su2doublet %d\n", hp->phi0, p->update_su2doublet);
  }
  if (hp->triplet) {
    printf("msq (triplet) %g, b4 %g, ", p->msq_triplet, p->b4);
    if (hp->nhiggs > 0) printf("a2 %g, ", p->a2);
    printf("initial sigma0 %g, update_su2triplet %d\n", hp->sigma0, p->update_su2triplet);
  }
  if (hp->singlet) {
    printf("msq (singlet) %g, b1_s %g, b3_s %g, b4_s %g, ", p->msq_s, p->b1_s, p->b3_s, p->b4_s);
    if (hp->nhiggs > 0) printf("a1_s %g, a2 %g, ", p->a1_s, p->a2_s);
    printf("initial singlet0 %g, update_singlet %d\n", hp->singlet0, p->update_singlet);
  }
  printf("GPU precision FP%d\n\n", p->precision);
}
