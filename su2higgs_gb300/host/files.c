/* files.c -- the reference's on-disk formats, byte for byte:
 *   lattice  binary checkpoint (checkpoint.c:84-214, serial 337-357)
 *   labels   column names of measure (measure.c:15-64)
 *   measure  one %g row per measurement (measure.c:182-307)
 *   weight   multicanonical weight text file (multicanonical.c:82-288)
 * plus the acceptance summary printed at checkpoints (checkpoint.c:17-78). */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "su2host.h"

/* doubles per site of field array `which` (0 link, 1 u1, 2 doublet0,
 * 3 doublet1, 4 triplet, 5 singlet); 0 if absent */
int64_t field_count(const host_params* hp, int which) {
  int D = hp->p.dim;
  switch (which) {
    case 0: return D * 4;
    case 1: return hp->u1 ? D : 0;
    case 2: return hp->nhiggs > 0 ? 4 : 0;
    case 3: return hp->nhiggs > 1 ? 4 : 0;
    case 4: return hp->triplet ? 3 : 0;
    case 5: return hp->singlet ? 1 : 0;
  }
  return 0;
}

static int64_t volume(const host_params* hp) {
  int64_t v = 1;
  for (int d = 0; d < hp->p.dim; d++) v *= hp->p.L[d];
  return v;
}

/* The order in which an N-rank run of the reference writes the sites of a
 * field (write_field, checkpoint.c:226-269): rank 0's sites, then rank 1's,
 * ...; a rank's sites in its storage order -- lexicographic in its slice,
 * then EVEN (by the global coordinate sum) before ODD, stably (sitemap,
 * layout.c:233-402; set_parity 410-450; paritymap 826-851).  The slicing
 * follows make_slices (layout.c:112-225): the rank count is factorised into
 * primes up to 29 and, from the largest prime down, each factor divides the
 * longest side it divides (the first such direction on ties); rank r sits at
 * the node coordinates of r in the grid of slices, x fastest.
 * order[k] = lexicographic index (x fastest) of the k-th site of the file.
 * Returns 0, or -1 when the lattice cannot be sliced that way. */
int mpi_file_order(int dim, const int* L, int nranks, int64_t* order) {
  static const int prime[10] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29};
  int nf[10] = {0}, rest = nranks;
  int64_t vol = 1;
  for (int d = 0; d < dim; d++) vol *= L[d];
  if (nranks < 1 || vol % nranks != 0) return -1;
  for (int n = 0; n < 10; n++)
    while (rest % prime[n] == 0) { rest /= prime[n]; nf[n]++; }
  if (rest != 1) return -1;
  int64_t slice[8];
  int nsl[8];
  for (int d = 0; d < dim; d++) { slice[d] = L[d]; nsl[d] = 1; }
  for (int n = 9; n >= 0; n--)
    for (int f = 0; f < nf[n]; f++) {
      int64_t largest = 1;
      for (int d = 0; d < dim; d++)
        if (slice[d] > largest && slice[d] % prime[n] == 0) largest = slice[d];
      if (largest == 1) return -1; /* no side divisible by this prime */
      for (int d = 0; d < dim; d++)
        if (slice[d] == largest) { slice[d] /= prime[n]; nsl[d] *= prime[n]; break; }
    }
  int64_t per = 1;
  for (int d = 0; d < dim; d++) per *= slice[d];
  int64_t k = 0;
  for (int r = 0; r < nranks; r++) {
    int64_t node[8], rr = r;
    for (int d = 0; d < dim; d++) { node[d] = rr % nsl[d]; rr /= nsl[d]; }
    for (int par = 0; par <= 1; par++)
      for (int64_t j = 0; j < per; j++) {
        int64_t x[8], jj = j, sum = 0, n = 0, stride = 1;
        for (int d = 0; d < dim; d++) {
          x[d] = node[d] * slice[d] + jj % slice[d];
          jj /= slice[d];
          sum += x[d];
        }
        if ((int)(sum & 1) != par) continue;
        for (int d = 0; d < dim; d++) { n += x[d] * stride; stride *= L[d]; }
        order[k++] = n;
      }
  }
  return k == vol ? 0 : -1;
}

/* storage index of the serial layout (layout.c:657-704: lexicographic, then
 * EVEN-first, stably) of every lexicographic index */
static void serial_index(const host_params* hp, int64_t* idx) {
  int64_t V = volume(hp), neven = 0;
  for (int pass = 0; pass < 2; pass++) {
    int64_t k = pass ? neven : 0;
    for (int64_t n = 0; n < V; n++) {
      int64_t r = n, sum = 0;
      for (int d = 0; d < hp->p.dim; d++) { sum += r % hp->p.L[d]; r /= hp->p.L[d]; }
      if ((int)(sum & 1) != pass) continue;
      idx[n] = k++;
    }
    if (!pass) neven = k;
  }
}

/* file position -> storage index of this program's arrays, for a file
 * written by `ranks` ranks */
static int64_t* file_to_storage(const host_params* hp, int ranks) {
  int64_t V = volume(hp);
  int64_t* ord = (int64_t*)malloc(sizeof(int64_t) * (size_t)V);
  int64_t* ser = (int64_t*)malloc(sizeof(int64_t) * (size_t)V);
  if (mpi_file_order(hp->p.dim, hp->p.L, ranks, ord)) {
    free(ord);
    free(ser);
    return NULL;
  }
  serial_index(hp, ser);
  for (int64_t k = 0; k < V; k++) ord[k] = ser[ord[k]];
  free(ser);
  return ord;
}

int save_lattice(const char* fname, const host_params* hp, long iter, double total_time, double comms_time,
                 double* const* arrays) {
  int size = hp->lattice_mpi_size > 0 ? hp->lattice_mpi_size : (hp->file_ranks > 0 ? hp->file_ranks : 1);
  int64_t* map = NULL;
  if (size > 1 && !(map = file_to_storage(hp, size))) {
    printf("!!! Cannot lay the lattice out for %d MPI ranks; writing it for 1\n", size);
    size = 1;
  }
  FILE* f = fopen(fname, "wb");
  if (!f) {
    printf("!!! Unable to open %s for writing\n", fname);
    free(map);
    return -1;
  }
  int dim = hp->p.dim;
  fwrite(&size, sizeof(int), 1, f);
  fwrite(&dim, sizeof(int), 1, f);
  fwrite(hp->p.L, sizeof(int), dim, f);
  fwrite(&iter, sizeof(long), 1, f);
  fwrite(&total_time, sizeof(double), 1, f);
  fwrite(&comms_time, sizeof(double), 1, f);
  int64_t V = volume(hp);
  for (int k = 0; k < 6; k++) {
    int64_t n = field_count(hp, k);
    if (!n) continue;
    if (!map) {
      fwrite(arrays[k], sizeof(double), (size_t)(V * n), f);
      continue;
    }
    double* buf = (double*)malloc(sizeof(double) * (size_t)(V * n));
    for (int64_t q = 0; q < V; q++) memcpy(buf + q * n, arrays[k] + map[q] * n, sizeof(double) * (size_t)n);
    fwrite(buf, sizeof(double), (size_t)(V * n), f);
    free(buf);
  }
  fclose(f);
  free(map);
  printf("Wrote fields to %s.\n", fname);
  return 0;
}

int load_lattice(const char* fname, host_params* hp, long* iter, double* total_time, double* comms_time,
                 double** arrays) {
  FILE* f = fopen(fname, "rb");
  if (!f) return -1;
  int dim = 0, size = 0, rd = 0;
  rd += (int)fread(&size, sizeof(int), 1, f);
  rd += (int)fread(&dim, sizeof(int), 1, f);
  if (dim < 0 || dim > 16) dim = 0;
  int L[16] = {0};
  rd += (int)fread(L, sizeof(int), dim, f);
  if (!rd) {
    printf("Error reading latticefile!\n");
    die(500);
  }
  /* load_lattice (checkpoint.c:131-214) demands the run's own MPI size; a
   * file of any rank count is read here, in that count's layout */
  int64_t* map = NULL;
  int ok = (dim == hp->p.dim && size >= 1);
  for (int d = 0; ok && d < dim; d++)
    if (L[d] != hp->p.L[d]) ok = 0;
  if (ok && size > 1 && !(map = file_to_storage(hp, size))) ok = 0;
  if (!ok) {
    printf("Dimensions in latticefile do not match! Got:\n");
    printf(" \tMPI size %d, dimension %d, volume ", size, dim);
    for (int d = 0; d < dim; d++) printf("%d x ", L[d]);
    printf("\b\b \b\n\nWas supposed to be: \n");
    printf("\tMPI size %d, dimension %d, volume ", 1, hp->p.dim);
    for (int d = 0; d < hp->p.dim; d++) printf("%d x ", hp->p.L[d]);
    printf("\b\b \b\n");
    die(501);
  }
  if (size > 1) printf("Lattice file written by %d MPI ranks: reading it in their layout.\n", size);
  hp->file_ranks = size;
  rd = 0;
  rd += (int)fread(iter, sizeof(long), 1, f);
  rd += (int)fread(total_time, sizeof(double), 1, f);
  rd += (int)fread(comms_time, sizeof(double), 1, f);
  int64_t V = volume(hp);
  for (int k = 0; k < 6; k++) {
    int64_t n = field_count(hp, k);
    if (!n) continue;
    size_t want = (size_t)(V * n);
    double* dst = map ? (double*)malloc(sizeof(double) * want) : arrays[k];
    if (fread(dst, sizeof(double), want, f) != want) {
      printf("Error reading field!\n");
      die(505);
    }
    if (map) {
      for (int64_t q = 0; q < V; q++) memcpy(arrays[k] + map[q] * n, dst + q * n, sizeof(double) * (size_t)n);
      free(dst);
    }
  }
  fclose(f);
  free(map);
  return 0;
}

void print_labels(const host_params* hp) {
  FILE* f = fopen("labels", "w+");
  if (!f) return;
  int k = 1;
  fprintf(f, "%d weight\n", k); k++;
  fprintf(f, "%d muca param\n", k); k++;
  fprintf(f, "%d action\n", k); k++;
  fprintf(f, "%d SU(2) Wilson (divided by beta)\n", k); k++;
  if (hp->u1) { fprintf(f, "%d U(1) Wilson (divided by beta)\n", k); k++; }
  if (hp->nhiggs > 0) {
    fprintf(f, "%d 2*(phi^2 - phi^+(x) U_i(x) phi(x+i)) (avg over directions)\n", k); k++;
    fprintf(f, "%d phi^2\n", k); k++;
    fprintf(f, "%d phi^4\n", k); k++;
  }
  if (hp->nhiggs == 2) {
    fprintf(f, "%d 2*(phi^2 - phi^+(x) U_i(x) phi(x+i)) for phi_2 (avg over directions)\n", k); k++;
    fprintf(f, "%d phi2^2\n", k); k++;
    fprintf(f, "%d phi2^4\n", k); k++;
    fprintf(f, "%d R = Re phi1^+ phi2\n", k); k++;
    fprintf(f, "%d I = Im phi1^+ phi2\n", k); k++;
  }
  if (hp->triplet) {
    fprintf(f, "%d hopping_Sigma (avg over directions)\n", k); k++;
    fprintf(f, "%d Sigma^2\n", k); k++;
    fprintf(f, "%d Sigma^4\n", k); k++;
  }
  if (hp->nhiggs > 0 && hp->triplet) { fprintf(f, "%d phi^2 Sigma^2\n", k); k++; }
  if (hp->triplet) {
    fprintf(f, "%d total magnetic charge density\n", k); k++;
    fprintf(f, "%d number of magnetic monopoles\n", k); k++;
  }
  if (hp->singlet) {
    fprintf(f, "%d S^2 - S(x)S(x+i) (avg over directions)\n", k); k++;
    fprintf(f, "%d S\n", k); k++;
    fprintf(f, "%d S^2\n", k); k++;
    fprintf(f, "%d S^3\n", k); k++;
    fprintf(f, "%d S^4\n", k); k++;
    if (hp->nhiggs == 1) {
      fprintf(f, "%d S phi^2\n", k); k++;
      fprintf(f, "%d S^2 phi^2\n", k); k++;
    }
  }
  fclose(f);
}

/* print_labels_local (measure.c:347-362) */
void print_labels_local(const host_params* hp, const char* fname) {
  FILE* f = fopen(fname, "w+");
  if (!f) return;
  int k = 1;
  for (int dir = 0; dir < hp->p.dim; dir++) {
    fprintf(f, "%d x%d\n", k, dir);
    k++;
  }
  if (hp->triplet) {
    fprintf(f, "%d Sigma^2\n", k); k++;
    fprintf(f, "%d magnetic charge (integer)\n", k); k++;
  }
  fclose(f);
}

/* measure_local's binary file (measure.c:368-487, serial layout): per site i
 * of the storage order (EVEN sites first) its coordinates as ints, the
 * triplet's two doubles, and a newline byte */
int write_measure_local(const char* fname, const host_params* hp, const double* vals) {
  FILE* f = fopen(fname, "wb");
  if (!f) return -1;
  const int* L = hp->p.L;
  long V = (long)L[0] * L[1] * L[2], half = V / 2;
  for (long i = 0; i < V; i++) {
    /* the closed form of the EVEN-first order: t-th site of its parity */
    int parity = i >= half;
    long t = i - parity * half;
    long r = t / (L[0] / 2);
    int k = (int)(t - r * (L[0] / 2));
    int z = (int)(r / L[1]), y = (int)(r - (long)z * L[1]);
    int c[3] = {2 * k + ((parity + y + z) & 1), y, z};
    fwrite(c, sizeof(int), 3, f);
    if (hp->triplet && vals) fwrite(vals + 2 * i, sizeof(double), 2, f);
    fwrite("\n", 1, 1, f);
  }
  fclose(f);
  return 0;
}

/* init_z_coord (z_coord.c:18-24): the longest direction, ties to the last */
int z_direction(const host_params* hp) {
  int zd = hp->p.dim - 1;
  for (int d = hp->p.dim - 1; d >= 0; d--)
    if (hp->p.L[d] > hp->p.L[zd]) zd = d;
  return zd;
}

/* print_z_labels (z_coord.c:78-106) */
void print_z_labels(const host_params* hp) {
  FILE* f = fopen("labels_z", "w+");
  if (!f) return;
  int k = 1;
  fprintf(f, "%d z\n", k); k++;
  if (hp->nhiggs > 0) { fprintf(f, "%d phi^2\n", k); k++; }
  if (hp->triplet) { fprintf(f, "%d Sigma^2\n", k); k++; }
  if (hp->singlet) {
    fprintf(f, "%d S\n", k); k++;
    fprintf(f, "%d S^2\n", k); k++;
  }
  fclose(f);
}

/* the rows measure_along_z (z_coord.c:274-292) appends: z, then the plane
 * averages of the quantities the content has */
void write_measure_z(const host_params* hp, int zdir, const double* sums) {
  FILE* f = fopen("measure_z", "a");
  if (!f) return;
  long Lz = hp->p.L[zdir];
  double area = (double)(volume(hp) / Lz);
  for (long z = 0; z < Lz; z++) {
    fprintf(f, "%ld ", z);
    const double* m = sums + 4 * z;
    if (hp->nhiggs > 0) fprintf(f, "%g ", m[0] / area);
    if (hp->triplet) fprintf(f, "%g ", m[1] / area);
    if (hp->singlet) fprintf(f, "%g %g ", m[2] / area, m[3] / area);
    fprintf(f, "\n");
  }
  fclose(f);
}

/* uniform deviates in [0, 1) for prepare_wall: splitmix64 (Steele, Lea &
 * Flood, OOPSLA 2014), the top 53 bits */
static double wall_uniform(uint64_t* s) {
  uint64_t z = (*s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

void prepare_wall(const host_params* hp, double* const* arrays, uint64_t seed) {
  const int* L = hp->p.L;
  int zd = z_direction(hp);
  long V = volume(hp), half = V / 2;
  uint64_t st = seed ^ 0x5eed3a11ull;
  for (long i = 0; i < V; i++) {
    int parity = i >= half;
    long t = i - parity * half;
    long r = t / (L[0] / 2);
    int k = (int)(t - r * (L[0] / 2));
    int z = (int)(r / L[1]), y = (int)(r - (long)z * L[1]);
    int c[3] = {2 * k + ((parity + y + z) & 1), y, z};
    int small = c[zd] < 0.5 * L[zd];
    for (int db = 0; db < hp->nhiggs; db++) {
      double* phi = arrays[2 + db] + 4 * i;
      double a = small ? 0.01 : 0.05;
      phi[0] = (small ? 0.2 : 1.2) + a * wall_uniform(&st);
      for (int q = 1; q < 4; q++) phi[q] = a * wall_uniform(&st);
    }
    if (hp->triplet) {
      double* s3 = arrays[4] + 3 * i;
      double a = small ? 0.05 : 0.01;
      s3[0] = (small ? 1.5 : 0.2) + a * wall_uniform(&st);
      s3[1] = a * wall_uniform(&st);
      s3[2] = a * wall_uniform(&st);
    }
    if (hp->singlet) arrays[5][i] = (small ? 0.8 : 0.1) + 0.01 * wall_uniform(&st);
    for (int dir = 0; dir < hp->p.dim; dir++) {
      double u = 1.0 - (small ? 0.03 : 0.4) * wall_uniform(&st);
      double* U = arrays[0] + 4 * (i * hp->p.dim + dir);
      U[0] = u;
      U[1] = sqrt(1.0 - u * u);
      U[2] = 0.0;
      U[3] = 0.0;
    }
  }
  printf("Wall profile initialized.\n");
}

/* one measure() row from the volume sums (measure.c:182-307) */
void write_measure_row(FILE* f, const host_params* hp, const double* m, const su2gpu_weight* w, int have_muca) {
  double weight = 0.0, muca_param = 0.0;
  if (hp->multicanonical && have_muca) {
    muca_param = w->param_value[0] + w->param_value[1];
    weight = get_weight(w, muca_param);
  }
  weight = -1.0 * weight;
  const su2gpu_params* p = &hp->p;
  double vol = (double)volume(hp);
  fprintf(f, "%g %g ", weight, muca_param);
  fprintf(f, "%g %g ", m[SU2GPU_M_ACTION], m[SU2GPU_M_WILSON] / (vol * p->betasu2));
  if (hp->u1) fprintf(f, "%g ", m[SU2GPU_M_U1WILSON] / (vol * p->betau1));
  for (int h = 0; h < hp->nhiggs; h++)
    fprintf(f, "%g %g %g ", m[SU2GPU_M_COV_PHI + 3 * h] / (vol * p->dim), m[SU2GPU_M_PHI2 + 3 * h] / vol,
            m[SU2GPU_M_PHI4 + 3 * h] / vol);
  if (hp->nhiggs == 2) fprintf(f, "%g %g ", m[SU2GPU_M_PHI12_RE] / vol, m[SU2GPU_M_PHI12_IM] / vol);
  if (hp->triplet) {
    fprintf(f, "%g %g %g ", m[SU2GPU_M_HOP_SIGMA] / (vol * p->dim), m[SU2GPU_M_SIGMA2] / vol, m[SU2GPU_M_SIGMA4] / vol);
    if (hp->nhiggs > 0) fprintf(f, "%g ", m[SU2GPU_M_PHI2SIGMA2] / vol);
    fprintf(f, "%g %g ", m[SU2GPU_M_MAGCHARGE], m[SU2GPU_M_MAGCHARGE_ABS] / (2.0 * M_PI * sqrt(p->betasu2)));
  }
  if (hp->singlet) {
    fprintf(f, "%g ", m[SU2GPU_M_S_COV] / (vol * p->dim));
    fprintf(f, "%g %g %g %g ", m[SU2GPU_M_S1] / vol, m[SU2GPU_M_S2] / vol, m[SU2GPU_M_S3] / vol, m[SU2GPU_M_S4] / vol);
    if (hp->nhiggs == 1) fprintf(f, "%g %g ", m[SU2GPU_M_SPHI2] / vol, m[SU2GPU_M_S2PHI2] / vol);
  }
  fprintf(f, "\n");
  fflush(f);
}

/* ---------------- multicanonical weight (multicanonical.c) ---------------- */
void linearize_weight(su2gpu_weight* w) {
  w->slope[0] = 0;
  w->slope[w->bins + 1] = 0;
  w->b[0] = w->W[0];
  w->b[w->bins + 1] = w->W[w->bins + 1];
  for (int i = 1; i < w->bins + 1; i++) {
    w->slope[i] = (w->W[i + 1] - w->W[i]) / (w->pos[i + 1] - w->pos[i]);
    w->b[i] = w->W[i] - w->slope[i] * w->pos[i];
  }
}

static int whichbin(const su2gpu_weight* w, double val) {
  if (val < w->min) return 0;
  if (val >= w->max) return w->bins + 1;
  int bmin = 1, bmax = w->bins;
  while (bmin <= bmax) {
    int bin = bmin + (bmax - bmin) / 2;
    double cur = w->pos[bin], nxt = w->pos[bin + 1];
    if ((val < nxt && val > cur) || (fabs(val - cur) < 1e-12)) return bin;
    if (val > cur) bmin = bin + 1;
    else bmax = bin - 1;
  }
  printf("\n!!! WARNING: Error in multicanonical.c: failed to find bin for value = %lf!!!\n\n", val);
  return w->bins;
}

double get_weight(const su2gpu_weight* w, double val) {
  if (val >= w->max) return w->b[w->bins + 1];
  if (val < w->min) return w->b[0];
  int bin = whichbin(w, val);
  if (bin >= w->bins + 1) return w->b[w->bins + 1];
  return w->b[bin] + w->slope[bin] * val;
}

static void alloc_weight_arrays(su2gpu_weight* w) {
  int n = w->bins + 2;
  w->pos = (double*)calloc(n, sizeof(double));
  w->W = (double*)calloc(n, sizeof(double));
  w->slope = (double*)calloc(n, sizeof(double));
  w->b = (double*)calloc(n, sizeof(double));
  w->hits = (int32_t*)calloc(n, sizeof(int32_t));
  w->gsum = (int64_t*)calloc(n, sizeof(int64_t));
  w->nsum = (int64_t*)calloc(n, sizeof(int64_t));
  w->hgram = (double*)calloc(n, sizeof(double));
}

void save_weight(const su2gpu_weight* w) {
  extern char g_weightfile[200];
  if (w->mode == SU2GPU_MUCA_READONLY) return;
  FILE* f = fopen(g_weightfile, "w");
  if (f) {
    fprintf(f, "%d %.12lf %d %lf %lf\n", w->bins, w->delta, w->last_max, w->wrk_min, w->wrk_max);
    for (long i = 1; i < w->bins + 2; i++) fprintf(f, "%lf %lf\n", w->pos[i], w->W[i]);
    fclose(f);
  }
  if (w->mode == SU2GPU_MUCA_SLOW) {
    FILE* g = fopen("weight_params", "w");
    if (g) {
      fprintf(g, "%d \n", w->bins);
      for (long i = 1; i < w->bins + 1; i++) fprintf(g, "%lf %ld %ld\n", w->pos[i], (long)w->gsum[i], (long)w->nsum[i]);
      fclose(g);
    }
  }
}

char g_weightfile[200] = "weight";

/* load_weight (multicanonical.c:118-288), including its reading of the
 * update range check and last-bin shift, which in the reference apply when
 * the mode is READONLY (the condition there is written "!mode != READONLY") */
int load_weight(su2gpu_weight* w, host_muca* hm) {
  memset(w, 0, sizeof(*w));
  snprintf(g_weightfile, sizeof(g_weightfile), "%s", hm->weightfile);
  w->orderparam = hm->orderparam;
  w->mode = hm->mode;
  w->checks_per_sweep = hm->checks_per_sweep;
  w->bins = hm->bins;
  w->min = hm->min;
  w->max = hm->max;
  w->delta = hm->delta;
  w->update_interval = hm->mode != SU2GPU_MUCA_SLOW ? 100 : 5000;
  w->do_acceptance = 1;
  printf("\nLoading weightfile: %s\n", hm->weightfile);
  FILE* f = NULL;
  if (access(hm->weightfile, R_OK) != 0) {
    printf("!!! Unable to access file %s\n", hm->weightfile);
    if (w->mode == SU2GPU_MUCA_READONLY) {
      printf("No multicanonical weight given for a read-only run! Exiting...\n");
      die(20);
    }
    if (w->bins <= 0) {
      printf("\n!!!!! Multicanonical error: bins <= 0\n");
      die(-1141);
    }
    alloc_weight_arrays(w);
    double dbin = (w->max - w->min) / ((double)(w->bins));
    for (int i = 0; i < w->bins + 1; i++) {
      w->pos[i + 1] = w->min + ((double)i) * dbin;
      w->W[i + 1] = 0.0;
    }
    w->last_max = 0;
    w->wrk_max = w->max;
    w->wrk_min = w->min;
    w->max += 0.001 * dbin;
    w->pos[w->bins + 1] = w->max;
    printf("Initialized new weight \n");
  } else {
    f = fopen(hm->weightfile, "r");
    int bins_read = 0, last_max = 0;
    double delta = 0, wmin = 0, wmax = 0;
    if (fscanf(f, "%d %lf %d %lf %lf", &bins_read, &delta, &last_max, &wmin, &wmax) != 5) {
      printf("Error reading first line of weightfile! \n");
      die(22);
    }
    w->bins = bins_read;
    w->delta = delta;
    w->last_max = last_max;
    w->wrk_min = wmin;
    w->wrk_max = wmax;
    if (w->bins <= 0) {
      printf("\n!!!!! Multicanonical error: bins <= 0\n");
      die(-1141);
    }
    alloc_weight_arrays(w);
    for (long i = 1; i < w->bins + 2; i++) {
      int rd = fscanf(f, "%lf %lf", &w->pos[i], &w->W[i]);
      if (rd != 2) {
        printf("Error reading weightfile! Got %d values at line %ld\n", rd, i + 1);
        die(22);
      }
    }
    fclose(f);
    w->min = w->pos[1];
    w->max = w->pos[w->bins + 1];
    if (w->mode == SU2GPU_MUCA_READONLY && (w->wrk_min < w->min || w->wrk_max > w->max)) {
      printf("\n!!! Multicanonical error: weight update range [%lf, %lf] larger than binning range [%lf, %lf] !!!\n\n",
             w->wrk_min, w->wrk_max, w->min, w->max);
      die(233);
    }
    if (w->mode == SU2GPU_MUCA_READONLY && fabs(w->wrk_max - w->max) < 1e-10) {
      double dbin = w->max - w->pos[w->bins];
      w->max += 0.001 * dbin;
      w->pos[w->bins + 1] = w->max;
    }
  }
  w->pos[0] = w->min - 1000.0 * (w->max - w->min);
  w->W[0] = w->W[1];
  w->W[w->bins + 1] = w->W[w->bins];
  linearize_weight(w);
  printf("Using weight function with %d bins in range %lf, %lf\n", w->bins, w->min, w->max);
  printf("Global multicanonical check %d times per even/odd update sweep\n", w->checks_per_sweep);
  if (w->mode != SU2GPU_MUCA_READONLY) printf("Will modify weight in range %lf, %lf\n", w->wrk_min, w->wrk_max);
  if (w->mode == SU2GPU_MUCA_FAST)
    printf("Fast weight update: starting with delta %.12lf, last_max %d\n", w->delta, w->last_max);
  if (w->mode == SU2GPU_MUCA_SLOW) printf("Using slow but safe weight updating: parameter file 'weight_params'\n");
  w->muca_count = 0;
  for (int i = 0; i < w->bins + 2; i++) {
    w->hits[i] = 0;
    if (w->mode == SU2GPU_MUCA_SLOW) w->hgram[i] = exp(w->W[i]);
  }
  if (w->mode == SU2GPU_MUCA_SLOW) {
    /* load_weight_params (multicanonical.c:291-333) */
    FILE* g = NULL;
    if (access("weight_params", R_OK) != 0) {
      printf("!!! Unable to access file %s\n", "weight_params");
      printf("!!! Unable to access weight parameter file. Initializing new\n");
      for (int i = 0; i < w->bins + 2; i++) { w->gsum[i] = 5; w->nsum[i] = 1; }
    } else {
      g = fopen("weight_params", "r");
      int bins_read = 0;
      if (fscanf(g, "%d", &bins_read) != 1 || bins_read != w->bins) {
        printf("Error reading parameter file!! Expected %d bins, got %d\n\n", w->bins, bins_read);
        die(991);
      }
      for (int i = 1; i < w->bins + 1; i++) {
        double tmp;
        long gs, ns;
        int rd = fscanf(g, "%lf %ld %ld", &tmp, &gs, &ns);
        if (rd != 3) {
          printf("Error reading 'weight_params'!! Got %d values at line %d\n\n", rd, i + 1);
          die(992);
        }
        w->gsum[i] = gs;
        w->nsum[i] = ns;
      }
      fclose(g);
    }
  }
  save_weight(w);
  return 0;
}

/* print_acceptance (checkpoint.c:17-78) */
void print_acceptance(const host_params* hp, const int64_t* c) {
  const su2gpu_params* p = &hp->p;
  printf("\n-- Acceptance rates --\n\t");
  if (p->algorithm_su2link == SU2GPU_METROPOLIS || hp->triplet)
    printf("SU(2) link %.2lf%%, ", 100.0 * c[SU2GPU_C_ACC_SU2LINK] / c[SU2GPU_C_TOTAL_SU2LINK]);
  if (hp->u1 && p->algorithm_u1link == SU2GPU_METROPOLIS)
    printf("U(1) link %.2lf%%, ", 100.0 * c[SU2GPU_C_ACC_U1LINK] / c[SU2GPU_C_TOTAL_U1LINK]);
  for (int db = 0; db < hp->nhiggs; db++) {
    if (p->algorithm_su2doublet == SU2GPU_METROPOLIS)
      printf("Higgs#%d %.2lf%%, ", db + 1, 100.0 * c[SU2GPU_C_ACC_DOUBLET + db] / c[SU2GPU_C_TOTAL_DOUBLET + db]);
    else if (p->algorithm_su2doublet == SU2GPU_OVERRELAX)
      printf("Higgs#%d overrelax %.2lf%%, Higgs#%d Metropolis %.2lf%%, ", db + 1,
             100.0 * c[SU2GPU_C_ACC_OR_DOUBLET + db] / c[SU2GPU_C_TOTAL_OR_DOUBLET + db], db + 1,
             100.0 * c[SU2GPU_C_ACC_DOUBLET + db] / c[SU2GPU_C_TOTAL_DOUBLET + db]);
  }
  if (hp->triplet) {
    if (p->algorithm_su2triplet == SU2GPU_METROPOLIS)
      printf("Triplet %.2lf%%, ", 100.0 * c[SU2GPU_C_ACC_TRIPLET] / c[SU2GPU_C_TOTAL_TRIPLET]);
    else if (p->algorithm_su2triplet == SU2GPU_OVERRELAX)
      printf("Triplet overrelax %.2lf%%, Triplet Metropolis %.2lf%%, ",
             100.0 * c[SU2GPU_C_ACC_OR_TRIPLET] / c[SU2GPU_C_TOTAL_OR_TRIPLET],
             100.0 * c[SU2GPU_C_ACC_TRIPLET] / c[SU2GPU_C_TOTAL_TRIPLET]);
  }
  if (hp->singlet) {
    if (p->algorithm_singlet == SU2GPU_METROPOLIS)
      printf("Singlet %.2lf%%, ", 100.0 * c[SU2GPU_C_ACC_SINGLET] / c[SU2GPU_C_TOTAL_SINGLET]);
    else if (p->algorithm_singlet == SU2GPU_OVERRELAX)
      printf("Singlet overrelax %.2lf%%, Singlet Metropolis %.2lf%%, ",
             100.0 * c[SU2GPU_C_ACC_OR_SINGLET] / c[SU2GPU_C_TOTAL_OR_SINGLET],
             100.0 * c[SU2GPU_C_ACC_SINGLET] / c[SU2GPU_C_TOTAL_SINGLET]);
  }
  if (hp->multicanonical) printf("multicanonical %.2lf%%", 100.0 * c[SU2GPU_C_ACC_MUCA] / c[SU2GPU_C_TOTAL_MUCA]);
  printf("\n");
}
