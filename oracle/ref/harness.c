/* harness.c -- TEST INFRASTRUCTURE (oracle). Not part of the product.
 *
 * Drives the reference su2higgs code itself (compiled from its own sources
 * by oracle/ref/Makefile into oracle/_ref/) so that its outputs can pin the
 * C restatement in oracle/src and the golden fixtures under tests/golden.
 *
 * The reference draws every random number through dran() = genrand64_real2()
 * (generic/mersenne.h:14).  This file supplies genrand64_real2() itself and
 * uses the linker's --wrap on the per-site update routines
 * (heatbath.c:15, metropolis.c:15/48/77/113/148, overrelax.c:54/137/243/295)
 * and on multicanonical_acceptance() (multicanonical.c:385).  Each wrapper
 * records which site / half-sweep is being updated before calling the real
 * routine, so the reference consumes exactly the Philox4x32-10 uniforms that
 * the GPU kernels consume for the same (site, pass, sweep) -- see
 * oracle/src/orc_philox.h for the stream definition.  Pass numbers are
 * assigned in order of first appearance of each (routine, direction/doublet,
 * parity) run inside one update_lattice() call (update.c:270-430).
 *
 * reduce_sum() (comms.c:929 serial) is wrapped too: measure()
 * (measure.c:191-233) passes every volume sum through it, so the wrapper
 * captures the full-precision sums before they are formatted with %g.
 */
#include "su2.h"
#include <stdint.h>
#include "../src/orc_philox.h"

MPI_Comm MPI_COMM_WORLD = {};

static lattice L;
static params P;
static fields F;
static counters C;
static weight W;
static int have_setup = 0;
static int muca_loaded = 0;

static orc_stream S;
static uint64_t rng_seed = 0;
static uint32_t rng_sweep = 0, rng_chain = 0;
static int cur_pass = -1;
static long last_key = -1;
static int cur_check = 0;

/* ---------------- RNG replacement for generic/mersenne.c ---------------- */
static int zero_uniforms = 0; /* ref_or_proposal: every uniform 0 */
double genrand64_real2(void) { return zero_uniforms ? 0.0 : orc_stream_uniform(&S); }
unsigned long long genrand64_int64(void) {
  /* only used by shuffle() for random sweep orders, which the harness never enables */
  double u = orc_stream_uniform(&S);
  return (unsigned long long)(u * 18446744073709551616.0);
}
void init_genrand64(unsigned long long seed) { (void)seed; }

static void enter_site(int fn, int sub, long i) {
  int par = (i < L.evensites) ? EVEN : ODD;
  long key = ((long)fn << 16) | ((long)sub << 4) | par;
  if (key != last_key) {
    cur_pass++;
    last_key = key;
    cur_check = 0;
  }
  orc_stream_at(&S, (uint32_t)i, (uint32_t)cur_pass);
}

/* ---------------- wrapped per-site routines ---------------- */
int __real_heatbath_su2link(lattice const* l, fields* f, params const* p, long i, int dir);
int __wrap_heatbath_su2link(lattice const* l, fields* f, params const* p, long i, int dir) {
  enter_site(1, dir, i);
  return __real_heatbath_su2link(l, f, p, i, dir);
}
int __real_metro_su2link(lattice const* l, fields* f, params const* p, long i, int dir);
int __wrap_metro_su2link(lattice const* l, fields* f, params const* p, long i, int dir) {
  enter_site(2, dir, i);
  return __real_metro_su2link(l, f, p, i, dir);
}
#ifdef U1
int __real_metro_u1link(lattice const* l, fields* f, params const* p, long i, int dir);
int __wrap_metro_u1link(lattice const* l, fields* f, params const* p, long i, int dir) {
  enter_site(3, dir, i);
  return __real_metro_u1link(l, f, p, i, dir);
}
#endif
#if (NHIGGS > 0)
int __real_metro_doublet(lattice const* l, fields* f, params const* p, long i, int higgs_id);
int __wrap_metro_doublet(lattice const* l, fields* f, params const* p, long i, int higgs_id) {
  enter_site(5, higgs_id, i);
  return __real_metro_doublet(l, f, p, i, higgs_id);
}
#if (NHIGGS == 1)
int __real_overrelax_doublet(lattice const* l, fields* f, params const* p, long i);
int __wrap_overrelax_doublet(lattice const* l, fields* f, params const* p, long i) {
  enter_site(4, 0, i);
  return __real_overrelax_doublet(l, f, p, i);
}
#else
int __real_overrelax_higgs2(lattice const* l, fields* f, params const* p, long i, int higgs_id);
int __wrap_overrelax_higgs2(lattice const* l, fields* f, params const* p, long i, int higgs_id) {
  enter_site(4, higgs_id, i);
  return __real_overrelax_higgs2(l, f, p, i, higgs_id);
}
#endif
#endif
#ifdef TRIPLET
int __real_overrelax_triplet(lattice const* l, fields* f, params const* p, long i);
int __wrap_overrelax_triplet(lattice const* l, fields* f, params const* p, long i) {
  enter_site(6, 0, i);
  return __real_overrelax_triplet(l, f, p, i);
}
int __real_metro_triplet(lattice const* l, fields* f, params const* p, long i);
int __wrap_metro_triplet(lattice const* l, fields* f, params const* p, long i) {
  enter_site(7, 0, i);
  return __real_metro_triplet(l, f, p, i);
}
#endif
#ifdef SINGLET
int __real_overrelax_singlet(lattice const* l, fields* f, params const* p, long i);
int __wrap_overrelax_singlet(lattice const* l, fields* f, params const* p, long i) {
  enter_site(8, 0, i);
  return __real_overrelax_singlet(l, f, p, i);
}
int __real_metro_singlet(lattice const* l, fields* f, params const* p, long i);
int __wrap_metro_singlet(lattice const* l, fields* f, params const* p, long i) {
  enter_site(9, 0, i);
  return __real_metro_singlet(l, f, p, i);
}
#endif

int __real_multicanonical_acceptance(lattice const* l, weight* w, double oldval, double newval);
int __wrap_multicanonical_acceptance(lattice const* l, weight* w, double oldval, double newval) {
  /* global draw: site = 0xffffffff, block = index of this check within the pass */
  orc_stream_at(&S, ORC_GLOBAL_SITE, (uint32_t)(cur_pass < 0 ? 0 : cur_pass));
  S.draw = 2u * (uint32_t)cur_check;
  cur_check++;
  return __real_multicanonical_acceptance(l, w, oldval, newval);
}

/* ---------------- measure() sum capture ---------------- */
static int capture_on = 0;
static int capture_n = 0;
static double capture_buf[64];
double __real_reduce_sum(double res, MPI_Comm comm);
double __wrap_reduce_sum(double res, MPI_Comm comm) {
  if (capture_on && capture_n < 64) capture_buf[capture_n++] = res;
  return __real_reduce_sum(res, comm);
}

/* measure() is called from gradflow.c as well; wrapping it lets a whole
 * flow record every row's sums. */
#define ROWCAP_MAX 2048
static int rowcap_on = 0, rowcap_n = 0, rowcap_per = 0;
static double rowcap[ROWCAP_MAX][64];
void __real_measure(FILE* file, lattice const* l, fields const* f, params const* p, weight* w);
void __wrap_measure(FILE* file, lattice const* l, fields const* f, params const* p, weight* w) {
  capture_on = 1; capture_n = 0;
  __real_measure(file, l, f, p, w);
  capture_on = 0;
  if (rowcap_on && rowcap_n < ROWCAP_MAX) {
    for (int k = 0; k < capture_n; k++) rowcap[rowcap_n][k] = capture_buf[k];
    rowcap_per = capture_n;
    rowcap_n++;
  }
}

/* ---------------- exported harness API (ctypes) ---------------- */
int ref_content_flags(void) {
  int fl = 0;
#if (NHIGGS == 1)
  fl |= 1;
#endif
#if (NHIGGS == 2)
  fl |= 2;
#endif
#ifdef TRIPLET
  fl |= 4;
#endif
#ifdef SINGLET
  fl |= 8;
#endif
#ifdef U1
  fl |= 16;
#endif
#ifdef GRADFLOW
  fl |= 32;
#endif
  return fl;
}

int ref_setup(char* config) {
  myRank = 0; MPISize = 1;
  L.rank = 0; L.size = 1;
  waittime = 0.0; Global_comms_time = 0.0; Global_total_time = 0.0;
  get_parameters(config, &L, &P);
  get_weight_parameters(config, &P, &W);
  layout(&L, 0, 0);
  alloc_fields(&L, &F);
  init_counters(&C);
  setfields(&F, &L, &P);
  P.random_sweeps = 0;
  have_setup = 1;
  return 0;
}

long ref_sites(void) { return L.sites; }
long ref_evensites(void) { return L.evensites; }
int ref_dim(void) { return L.dim; }

void ref_tables(long* next, long* prev, long* coords, int* parity) {
  for (long i = 0; i < L.sites; i++) {
    for (int d = 0; d < L.dim; d++) {
      next[i * L.dim + d] = L.next[i][d];
      prev[i * L.dim + d] = L.prev[i][d];
      coords[i * L.dim + d] = L.coords[i][d];
    }
    parity[i] = L.parity[i];
  }
}

/* Field arrays are AoS FP64 in the layout (parity-ordered) site order, i.e.
 * exactly the field blocks of the reference's binary lattice file
 * (checkpoint.c:101-115). Pointers may be NULL for absent fields. */
void ref_put_fields(const double* link, const double* u1, const double* d0, const double* d1,
                    const double* trip, const double* sing) {
  long V = L.sites; int D = L.dim;
  if (link) memcpy(&F.su2link[0][0][0], link, sizeof(double) * V * D * 4);
#ifdef U1
  if (u1) memcpy(&F.u1link[0][0], u1, sizeof(double) * V * D);
#endif
#if (NHIGGS > 0)
  if (d0) memcpy(&F.su2doublet[0][0][0], d0, sizeof(double) * V * 4);
#endif
#if (NHIGGS > 1)
  if (d1) memcpy(&F.su2doublet[1][0][0], d1, sizeof(double) * V * 4);
#endif
#ifdef TRIPLET
  if (trip) memcpy(&F.su2triplet[0][0], trip, sizeof(double) * V * 3);
#endif
#ifdef SINGLET
  if (sing) memcpy(&F.singlet[0][0], sing, sizeof(double) * V);
#endif
  (void)u1; (void)d0; (void)d1; (void)trip; (void)sing;
  sync_halos(&L, &F);
}

void ref_get_fields(double* link, double* u1, double* d0, double* d1, double* trip, double* sing) {
  long V = L.sites; int D = L.dim;
  if (link) memcpy(link, &F.su2link[0][0][0], sizeof(double) * V * D * 4);
#ifdef U1
  if (u1) memcpy(u1, &F.u1link[0][0], sizeof(double) * V * D);
#endif
#if (NHIGGS > 0)
  if (d0) memcpy(d0, &F.su2doublet[0][0][0], sizeof(double) * V * 4);
#endif
#if (NHIGGS > 1)
  if (d1) memcpy(d1, &F.su2doublet[1][0][0], sizeof(double) * V * 4);
#endif
#ifdef TRIPLET
  if (trip) memcpy(trip, &F.su2triplet[0][0], sizeof(double) * V * 3);
#endif
#ifdef SINGLET
  if (sing) memcpy(sing, &F.singlet[0][0], sizeof(double) * V);
#endif
  (void)u1; (void)d0; (void)d1; (void)trip; (void)sing;
}

void ref_set_rng(unsigned long long seed, unsigned int sweep, unsigned int chain) {
  rng_seed = seed; rng_sweep = sweep; rng_chain = chain;
  orc_stream_init(&S, rng_seed, rng_sweep, rng_chain);
}

/* One call of the reference's own update_lattice() (update.c:270). */
int ref_update(void) {
  orc_stream_init(&S, rng_seed, rng_sweep, rng_chain);
  cur_pass = -1; last_key = -1; cur_check = 0;
  update_lattice(&L, &F, &P, &C, &W);
  return cur_pass + 1; /* number of passes seen */
}

void ref_reset_counters(void) { init_counters(&C); }

/* Counter layout shared with the oracle and the C-ABI (su2gpu_counters). */
void ref_counters(long* out) {
  for (int k = 0; k < 24; k++) out[k] = 0;
  out[0] = C.total_su2link; out[1] = C.accepted_su2link;
  out[2] = C.total_u1link; out[3] = C.accepted_u1link;
#if (NHIGGS > 0)
  for (int db = 0; db < NHIGGS; db++) {
    out[4 + db] = C.total_doublet[db];
    out[6 + db] = C.accepted_doublet[db];
    out[8 + db] = C.total_overrelax_doublet[db];
    out[10 + db] = C.acc_overrelax_doublet[db];
  }
#endif
  out[12] = C.total_triplet; out[13] = C.accepted_triplet;
  out[14] = C.total_overrelax_triplet; out[15] = C.acc_overrelax_triplet;
#ifdef SINGLET
  out[16] = C.total_singlet; out[17] = C.accepted_singlet;
  out[18] = C.total_overrelax_singlet; out[19] = C.acc_overrelax_singlet;
#endif
  out[20] = C.total_muca; out[21] = C.accepted_muca;
}

/* measure() with its output row sent to /dev/null; returns the captured
 * volume sums (in measure.c:191-233 order) followed by muca param and weight. */
int ref_measure_sums(double* out, char* rowbuf, int rowlen) {
  FILE* fp;
  char* buf = NULL; size_t sz = 0;
  fp = open_memstream(&buf, &sz);
  measure(fp, &L, &F, &P, &W);
  fclose(fp);
  if (rowbuf && rowlen > 0) {
    strncpy(rowbuf, buf ? buf : "", rowlen - 1);
    rowbuf[rowlen - 1] = 0;
  }
  free(buf);
  for (int k = 0; k < capture_n; k++) out[k] = capture_buf[k];
  return capture_n;
}

/* ---- deterministic per-site kernels ---- */
void ref_link_staple(long i, int dir, double* V) { su2link_staple(&L, &F, &P, i, dir, V); }
void ref_wilson_staple(long i, int dir, double* V) { su2staple_wilson(&L, &F, i, dir, V); }
double ref_localact_su2link(long i, int dir) { return localact_su2link(&L, &F, &P, i, dir); }
double ref_local_su2wilson(long i) { return (double)local_su2wilson(&L, &F, &P, i); }
double ref_action_local(long i) { return action_local(&L, &F, &P, i); }
double ref_higgspotential(long i) { return higgspotential(&F, &P, i); }
double ref_polysolve3(double a, double b, double c, double d) { return polysolve3(a, b, c, d); }
#ifdef U1
double ref_localact_u1link(long i, int dir) { return localact_u1link(&L, &F, &P, i, dir); }
double ref_local_u1wilson(long i) { return local_u1wilson(&L, &F, &P, i); }
#endif
#if (NHIGGS > 0)
void ref_staple_doublet(long i, int hid, double* s) { staple_doublet(s, &L, &F, &P, i, hid); }
double ref_localact_doublet(long i, int hid) { return localact_doublet(&L, &F, &P, i, hid); }
double ref_covariant_doublet(long i, int hid) { return covariant_doublet(&L, &F, i, hid); }
#endif
#ifdef TRIPLET
double ref_localact_triplet(long i) { return localact_triplet(&L, &F, &P, i); }
double ref_covariant_triplet(long i) { return covariant_triplet(&L, &F, &P, i); }
double ref_magcharge_cube(long i) { return magcharge_cube(&L, &F, &P, i); }
double ref_alpha_proj(long i, int d1, int d2) { return alpha_proj(&L, &F, &P, i, d1, d2); }
#endif
#ifdef SINGLET
double ref_localact_singlet(long i) { return localact_singlet(&L, &F, &P, i); }
#endif

/* ---- stochastic per-site kernels with an explicit (site, pass) stream ---- */
int ref_site_update(int kind, long i, int sub, unsigned int pass) {
  orc_stream_init(&S, rng_seed, rng_sweep, rng_chain);
  orc_stream_at(&S, (uint32_t)i, pass);
  switch (kind) {
    case 1: return __real_heatbath_su2link(&L, &F, &P, i, sub);
    case 2: return __real_metro_su2link(&L, &F, &P, i, sub);
#ifdef U1
    case 3: return __real_metro_u1link(&L, &F, &P, i, sub);
#endif
#if (NHIGGS == 1)
    case 4: return __real_overrelax_doublet(&L, &F, &P, i);
#endif
#if (NHIGGS == 2)
    case 4: return __real_overrelax_higgs2(&L, &F, &P, i, sub);
#endif
#if (NHIGGS > 0)
    case 5: return __real_metro_doublet(&L, &F, &P, i, sub);
#endif
#ifdef TRIPLET
    case 6: return __real_overrelax_triplet(&L, &F, &P, i);
    case 7: return __real_metro_triplet(&L, &F, &P, i);
#endif
#ifdef SINGLET
    case 8: return __real_overrelax_singlet(&L, &F, &P, i);
    case 9: return __real_metro_singlet(&L, &F, &P, i);
#endif
    default: return -1;
  }
}
int ref_site_draws(void) { return (int)S.draw; }

/* The overrelaxation proposal at site i: the value the reference's update
 * writes when it accepts.  The update runs with every uniform 0, which it
 * always accepts (|dV/dV'| >= 0, overrelax.c:116-125); the site's old value
 * is put back afterwards.  kind 4: doublet `sub` (4 reals), 6: triplet (3),
 * 8: singlet (1).  Returns the number of reals written to out, -1 if the
 * kind is absent in this build. */
int ref_or_proposal(int kind, long i, int sub, double* out) {
  int n = -1;
  zero_uniforms = 1;
  switch (kind) {
#if (NHIGGS > 0)
    case 4: {
      double old[4];
      memcpy(old, F.su2doublet[sub][i], sizeof(old));
#if (NHIGGS == 1)
      __real_overrelax_doublet(&L, &F, &P, i);
#else
      __real_overrelax_higgs2(&L, &F, &P, i, sub);
#endif
      memcpy(out, F.su2doublet[sub][i], sizeof(old));
      memcpy(F.su2doublet[sub][i], old, sizeof(old));
      n = 4;
      break;
    }
#endif
#ifdef TRIPLET
    case 6: {
      double old[3];
      memcpy(old, F.su2triplet[i], sizeof(old));
      __real_overrelax_triplet(&L, &F, &P, i);
      memcpy(out, F.su2triplet[i], sizeof(old));
      memcpy(F.su2triplet[i], old, sizeof(old));
      n = 3;
      break;
    }
#endif
#ifdef SINGLET
    case 8: {
      double old = F.singlet[i][0];
      __real_overrelax_singlet(&L, &F, &P, i);
      out[0] = F.singlet[i][0];
      F.singlet[i][0] = old;
      n = 1;
      break;
    }
#endif
    default: break;
  }
  zero_uniforms = 0;
  (void)out; (void)sub;
  return n;
}

/* ---- multicanonical ---- */
/* main.c:212-221: load_weight, backups, order parameter of both parities */
int ref_muca_init(void) {
  if (!P.multicanonical) return -1;
  load_weight(&W);
  alloc_muca_backups(&L, &W);
  calc_orderparam(&L, &F, &P, &W, EVEN);
  calc_orderparam(&L, &F, &P, &W, ODD);
  muca_loaded = 1;
  return W.bins;
}
void ref_muca_set_mode(int mode) { W.mode = mode; }
void ref_muca_init_last_max(void) { init_last_max(&W); }
double ref_calc_orderparam(int par) { return calc_orderparam(&L, &F, &P, &W, (char)par); }
void ref_muca_values(double* out) { out[0] = W.param_value[0]; out[1] = W.param_value[1]; }
void ref_muca_scalars(double* out) {
  out[0] = W.bins; out[1] = W.min; out[2] = W.max; out[3] = W.wrk_min; out[4] = W.wrk_max;
  out[5] = W.delta; out[6] = W.last_max; out[7] = W.muca_count; out[8] = W.update_interval;
  out[9] = W.mode; out[10] = W.checks_per_sweep; out[11] = W.orderparam;
}
void ref_muca_arrays(double* pos, double* Wv, double* slope, double* b, int* hits) {
  for (int k = 0; k < W.bins + 2; k++) {
    pos[k] = W.pos[k]; Wv[k] = W.W[k]; slope[k] = W.slope[k]; b[k] = W.b[k]; hits[k] = W.hits[k];
  }
}
double ref_get_weight(double v) { return get_weight(&W, v); }
/* the number of checks between weight updates: load_weight fixes it (100, or
 * 5000 in SLOW mode); a test of the SLOW recursion shortens it */
void ref_muca_set_update_interval(int n) { W.update_interval = n; }
/* the SLOW mode's accumulators (update_weight_slow, multicanonical.c:561-666) */
void ref_muca_slow_arrays(long* gsum, long* nsum, double* hgram) {
  for (int k = 0; k < W.bins + 2; k++) {
    gsum[k] = W.mode == SLOW ? W.gsum[k] : 0;
    nsum[k] = W.mode == SLOW ? W.nsum[k] : 0;
    hgram[k] = W.mode == SLOW ? W.hgram[k] : 0.0;
  }
}
int ref_whichbin(double v) { return whichbin(&W, v); }

/* ---- gradient flow ---- */
#ifdef GRADFLOW
static fields G;
static int have_G = 0;
/* calc_gradient() (gradflow.c:335) on the current fields */
void ref_flow_forces(double* link_force, double* trip_force) {
  if (!have_G) { alloc_fields(&L, &G); have_G = 1; }
  calc_gradient(&L, &F, &P, &G);
  long V = L.sites; int D = L.dim;
  if (link_force) memcpy(link_force, &G.su2link[0][0][0], sizeof(double) * V * D * 4);
#ifdef TRIPLET
  if (trip_force) memcpy(trip_force, &G.su2triplet[0][0], sizeof(double) * V * 3);
#endif
  (void)trip_force;
}
/* One Euler step on the current fields: calc_gradient + flow_gauge + flow_triplet
 * (gradflow.c:98-113). */
void ref_flow_step(double dt) {
  if (!have_G) { alloc_fields(&L, &G); have_G = 1; }
  calc_gradient(&L, &F, &P, &G);
  flow_gauge(&L, &F, &G, dt);
#ifdef TRIPLET
  flow_triplet(&L, &F, &G, dt);
#endif
  sync_halos(&L, &F);
}
/* grad_flow() (gradflow.c:46); returns the volume sums of every measurement
 * row in out (row-major, *per values per row), number of rows in *nrows.
 * Its "measure_flow" file goes to the current directory. */
int ref_grad_flow(double tmax, double dt, int flow_id, double* out, int maxrows, int* nrows) {
  rowcap_on = 1; rowcap_n = 0; rowcap_per = 0;
  grad_flow(&L, &F, &P, &W, tmax, dt, flow_id);
  rowcap_on = 0;
  int nr = rowcap_n < maxrows ? rowcap_n : maxrows;
  for (int r = 0; r < nr; r++)
    for (int k = 0; k < rowcap_per; k++) out[r * rowcap_per + k] = rowcap[r][k];
  *nrows = nr;
  return rowcap_per;
}
#endif

/* ---- correlators and blocking ---- */
#ifdef CORRELATORS
/* The values of one measure_correlators() row set (correlation.c:350-398)
 * at full precision: per distance d < L[dir]/2 ten doubles -- the Higgs
 * correlator, the Sigma^2 correlator, then photon_correl() for (transmom,
 * mode) = (1,0), (2,0), (1,1), (2,1), each re and im (absent columns 0). */
#ifdef TRIPLET
/* defined in correlation.c:257 without a declaration in su2.h */
complex photon_correl(lattice* l, fields const* f, params const* p, int d, int dir, int transmom, int mode);
#endif
static void corr_rows(lattice* l, fields const* f, int dir, double* out) {
  int maxd = l->L[dir] / 2;
  for (int d = 0; d < maxd; d++) {
    double* r = out + 10 * d;
    for (int k = 0; k < 10; k++) r[k] = 0.0;
#if (NHIGGS > 0)
    r[0] = higgs_correlator(l, f, d, dir, 0);
#endif
#ifdef TRIPLET
    r[1] = triplet_correlator(l, f, d, dir);
    const int tm[4] = {1, 2, 1, 2}, md[4] = {0, 0, 1, 1};
    for (int k = 0; k < 4; k++) {
      complex c = photon_correl(l, f, &P, d, dir, tm[k], md[k]);
      r[2 + 2 * k] = c.re;
      r[3 + 2 * k] = c.im;
    }
#endif
  }
}
int ref_longest_dir(void) { return L.longest_dir; }
int ref_correlators(int dir, double* out) {
  corr_rows(&L, &F, dir, out);
  return L.L[dir] / 2;
}
#ifdef BLOCKING
/* main.c:106-157: blocked lattices in every direction but the longest, as
 * many levels as asked for and possible */
#define MAXBLOCK 8
static lattice BL[MAXBLOCK];
static fields BF[MAXBLOCK];
static int block_dir_h[4];
static int nblocked = 0;
int ref_block_setup(int levels) {
  if (nblocked) return nblocked;
  L.blocklist.sends = 0; L.blocklist.recvs = 0;
  realloc_comlist(&L.blocklist, RECV);
  L.standby = 0;
  L.blocking_level = 0;
  for (int d = 0; d < L.dim; d++) block_dir_h[d] = d != L.longest_dir;
  int mx = max_block_level(&L, block_dir_h);
  if (levels > mx) levels = mx;
  if (levels > MAXBLOCK) levels = MAXBLOCK;
  for (int k = 0; k < levels; k++) {
    lattice* base = k ? &BL[k - 1] : &L;
    BL[k].blocklist.sends = 0; BL[k].blocklist.recvs = 0;
    block_lattice(base, &BL[k], block_dir_h);
    alloc_fields(&BL[k], &BF[k]);
    BL[k].blocking_level = k + 1;
  }
  nblocked = levels;
  return levels;
}
/* measure_blocked_correlators (correlation.c:404-432) for level k+1 from
 * level k (the fields level 0): smear_fields, make_blocked_fields, then the
 * correlator rows on the blocked lattice.  Also returns the blocked links
 * and triplet in the blocked lattice's storage order with its coordinates
 * and L; the value is the number of blocked sites. */
long ref_blocked_level(int k, int dir, double* corr, double* link, double* trip, long* coords, int* Lb) {
  if (k < 0 || k >= nblocked) return -1;
  lattice* base = k ? &BL[k - 1] : &L;
  fields* fb = k ? &BF[k - 1] : &F;
  fields fs;
  alloc_fields(base, &fs);
  smear_fields(base, fb, &fs, block_dir_h);
  make_blocked_fields(base, &BL[k], &fs, &BF[k]);
  free_fields(base, &fs);
  corr_rows(&BL[k], &BF[k], dir, corr);
  long V = BL[k].sites;
  int D = BL[k].dim;
  memcpy(link, &BF[k].su2link[0][0][0], sizeof(double) * V * D * 4);
#ifdef TRIPLET
  if (trip) memcpy(trip, &BF[k].su2triplet[0][0], sizeof(double) * V * 3);
#endif
  for (long i = 0; i < V; i++)
    for (int d = 0; d < D; d++) coords[i * D + d] = BL[k].coords[i][d];
  for (int d = 0; d < D; d++) Lb[d] = BL[k].L[d];
  return V;
}
#endif
#endif
