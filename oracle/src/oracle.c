/* oracle.c -- TEST INFRASTRUCTURE (oracle). Not part of the product.
 *
 * A CPU restatement of su2higgs's checkerboard update sweep and the
 * kernels it owns, written in quaternion form.  Each routine names the
 * reference routine (src/ path of su2higgs, file:line) whose arithmetic it
 * restates; results agree with the reference to rounding, and its random
 * stream is the per-site Philox stream of orc_philox.h.  Used as the checker
 * of the CUDA path and as the timed CPU baseline, never by the product.
 *
 * SU(2) elements and doublets are quaternions q = (q0, q1, q2, q3) meaning
 * q0 + i q_k sigma_k (su2u1.c:7-31); the product of the reference's su2rot()
 * (su2u1.c:60-70) is qmul() below:  (a0 b0 - a.b,  a0 b + b0 a - a x b).
 */
#include "oracle.h"
#include "orc_philox.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* polysolve3() works in long double in the reference (overrelax.c:14-34). */
#ifndef ORC_CUBIC_REAL
#define ORC_CUBIC_REAL long double
#endif
typedef ORC_CUBIC_REAL creal;

#define EVEN 0
#define ODD 1

struct orc_ctx {
  su2gpu_params p;
  int D;
  long V, half;
  int64_t *next, *prev, *coords;
  int32_t* parity;
  double *link, *u1, *phi[2], *trip, *sing;
  int nh, has_trip, has_sing, has_u1;
  int64_t cnt[SU2GPU_NCOUNTERS];
  orc_stream rng;
  uint64_t seed;
  uint32_t sweep, chain;
  int pass;
  int random_sweeps;
  int zero_uniforms; /* orc_or_proposal: every uniform 0 */
  /* multicanonical */
  int muca_on;
  su2gpu_weight w;
  double *bu_phi, *bu_trip;
};

/* ------------------------------------------------------------------ */
/* quaternion helpers                                                  */
/* ------------------------------------------------------------------ */
static inline void qmul(const double* a, const double* b, double* r) {
  double r0 = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
  double r1 = a[0] * b[1] + b[0] * a[1] - (a[2] * b[3] - a[3] * b[2]);
  double r2 = a[0] * b[2] + b[0] * a[2] - (a[3] * b[1] - a[1] * b[3]);
  double r3 = a[0] * b[3] + b[0] * a[3] - (a[1] * b[2] - a[2] * b[1]);
  r[0] = r0; r[1] = r1; r[2] = r2; r[3] = r3;
}
static inline void qdag(const double* a, double* r) { r[0] = a[0]; r[1] = -a[1]; r[2] = -a[2]; r[3] = -a[3]; }
static inline double qsq(const double* a) { return a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + a[3] * a[3]; }
/* scalar part of a * b */
static inline double qdot0(const double* a, const double* b) {
  return a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
}
/* rotation of a 3-vector by u:  vec(u (0,b) u^dagger) */
static inline void qrot(const double* u, const double* b, double* r) {
  double vb[4] = {0.0, b[0], b[1], b[2]}, t[4], ud[4], o[4];
  qmul(u, vb, t);
  qdag(u, ud);
  qmul(t, ud, o);
  r[0] = o[1]; r[1] = o[2]; r[2] = o[3];
}
/* exp(-i alpha sigma_3) as a quaternion */
static inline void u1phase(double a, double* e) { e[0] = cos(a); e[1] = 0.0; e[2] = 0.0; e[3] = -sin(a); }

static inline double* LNK(const orc_ctx* c, long i, int d) { return c->link + (i * c->D + d) * 4; }
static inline long NX(const orc_ctx* c, long i, int d) { return (long)c->next[i * c->D + d]; }
static inline long PV(const orc_ctx* c, long i, int d) { return (long)c->prev[i * c->D + d]; }
static inline double* PHI(const orc_ctx* c, int h, long i) { return c->phi[h] + i * 4; }
static inline double* TRP(const orc_ctx* c, long i) { return c->trip + i * 3; }
static inline double A1(const orc_ctx* c, long i, int d) { return c->u1[i * c->D + d]; }

static inline double uni(orc_ctx* c) { return c->zero_uniforms ? 0.0 : orc_stream_uniform(&c->rng); }

/* ------------------------------------------------------------------ */
/* layout: layout.c:657-756 (serial), paritymap layout.c:826-851       */
/* lexicographic index with x fastest, then a stable EVEN-first order  */
/* ------------------------------------------------------------------ */
static void make_layout(orc_ctx* c) {
  int D = c->D;
  long V = 1;
  for (int d = 0; d < D; d++) V *= c->p.L[d];
  c->V = V;
  long* newidx = (long*)malloc(sizeof(long) * V);
  int* par = (int*)malloc(sizeof(int) * V);
  long neven = 0;
  for (long n = 0; n < V; n++) {
    long r = n, s = 0;
    for (int d = 0; d < D; d++) { s += r % c->p.L[d]; r /= c->p.L[d]; }
    par[n] = (int)(s & 1);
    if (!par[n]) neven++;
  }
  c->half = neven;
  long ne = 0, no = 0;
  for (long n = 0; n < V; n++) newidx[n] = par[n] ? neven + no++ : ne++;
  c->next = (int64_t*)malloc(sizeof(int64_t) * V * D);
  c->prev = (int64_t*)malloc(sizeof(int64_t) * V * D);
  c->coords = (int64_t*)malloc(sizeof(int64_t) * V * D);
  c->parity = (int32_t*)malloc(sizeof(int32_t) * V);
  for (long n = 0; n < V; n++) {
    long x[4], r = n;
    for (int d = 0; d < D; d++) { x[d] = r % c->p.L[d]; r /= c->p.L[d]; }
    long i = newidx[n];
    c->parity[i] = par[n];
    for (int d = 0; d < D; d++) {
      c->coords[i * D + d] = x[d];
      long stride = 1;
      for (int e = 0; e < d; e++) stride *= c->p.L[e];
      long xp = (x[d] + 1) % c->p.L[d], xm = (x[d] + c->p.L[d] - 1) % c->p.L[d];
      long np = n + (xp - x[d]) * stride, nm = n + (xm - x[d]) * stride;
      c->next[i * D + d] = newidx[np];
      c->prev[i * D + d] = newidx[nm];
    }
  }
  free(newidx);
  free(par);
}

orc_ctx* orc_create(const su2gpu_params* p) {
  orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
  c->p = *p;
  c->D = p->dim;
  make_layout(c);
  c->nh = (p->content & SU2GPU_HIGGS2) ? 2 : ((p->content & SU2GPU_HIGGS1) ? 1 : 0);
  c->has_trip = !!(p->content & SU2GPU_TRIPLET);
  c->has_sing = !!(p->content & SU2GPU_SINGLET);
  c->has_u1 = !!(p->content & SU2GPU_U1);
  long V = c->V;
  int D = c->D;
  c->link = (double*)calloc(V * D * 4, sizeof(double));
  for (long k = 0; k < V * D; k++) c->link[4 * k] = 1.0;
  if (c->has_u1) c->u1 = (double*)calloc(V * D, sizeof(double));
  for (int h = 0; h < c->nh; h++) c->phi[h] = (double*)calloc(V * 4, sizeof(double));
  if (c->has_trip) c->trip = (double*)calloc(V * 3, sizeof(double));
  if (c->has_sing) c->sing = (double*)calloc(V, sizeof(double));
  orc_stream_init(&c->rng, 0, 0, 0);
  return c;
}

static void free_weight(orc_ctx* c) {
  free(c->w.pos); free(c->w.W); free(c->w.slope); free(c->w.b); free(c->w.hits);
  free(c->w.gsum); free(c->w.nsum); free(c->w.hgram);
  free(c->bu_phi); free(c->bu_trip);
  memset(&c->w, 0, sizeof(c->w));
  c->bu_phi = NULL; c->bu_trip = NULL;
  c->muca_on = 0;
}

void orc_destroy(orc_ctx* c) {
  if (!c) return;
  free(c->next); free(c->prev); free(c->coords); free(c->parity);
  free(c->link); free(c->u1); free(c->phi[0]); free(c->phi[1]); free(c->trip); free(c->sing);
  free_weight(c);
  free(c);
}

long orc_sites(const orc_ctx* c) { return c->V; }

void orc_tables(const orc_ctx* c, int64_t* next, int64_t* prev, int64_t* coords, int32_t* parity) {
  long n = c->V * c->D;
  if (next) memcpy(next, c->next, sizeof(int64_t) * n);
  if (prev) memcpy(prev, c->prev, sizeof(int64_t) * n);
  if (coords) memcpy(coords, c->coords, sizeof(int64_t) * n);
  if (parity) memcpy(parity, c->parity, sizeof(int32_t) * c->V);
}

void orc_put_fields(orc_ctx* c, const double* link, const double* u1, const double* d0, const double* d1,
                    const double* trip, const double* sing) {
  long V = c->V; int D = c->D;
  if (link) memcpy(c->link, link, sizeof(double) * V * D * 4);
  if (u1 && c->u1) memcpy(c->u1, u1, sizeof(double) * V * D);
  if (d0 && c->nh > 0) memcpy(c->phi[0], d0, sizeof(double) * V * 4);
  if (d1 && c->nh > 1) memcpy(c->phi[1], d1, sizeof(double) * V * 4);
  if (trip && c->trip) memcpy(c->trip, trip, sizeof(double) * V * 3);
  if (sing && c->sing) memcpy(c->sing, sing, sizeof(double) * V);
}

void orc_get_fields(const orc_ctx* c, double* link, double* u1, double* d0, double* d1, double* trip,
                    double* sing) {
  long V = c->V; int D = c->D;
  if (link) memcpy(link, c->link, sizeof(double) * V * D * 4);
  if (u1 && c->u1) memcpy(u1, c->u1, sizeof(double) * V * D);
  if (d0 && c->nh > 0) memcpy(d0, c->phi[0], sizeof(double) * V * 4);
  if (d1 && c->nh > 1) memcpy(d1, c->phi[1], sizeof(double) * V * 4);
  if (trip && c->trip) memcpy(trip, c->trip, sizeof(double) * V * 3);
  if (sing && c->sing) memcpy(sing, c->sing, sizeof(double) * V);
}

void orc_set_rng(orc_ctx* c, uint64_t seed, uint32_t sweep, uint32_t chain) {
  c->seed = seed; c->sweep = sweep; c->chain = chain;
  orc_stream_init(&c->rng, seed, sweep, chain);
}

void orc_counters(const orc_ctx* c, int64_t* out) { memcpy(out, c->cnt, sizeof(c->cnt)); }
void orc_reset_counters(orc_ctx* c) { memset(c->cnt, 0, sizeof(c->cnt)); }

/* ------------------------------------------------------------------ */
/* SU(2) gauge part                                                    */
/* ------------------------------------------------------------------ */

/* su2staple_wilson (staples.c:84-115): sum over nu != mu of
 *   U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+  +  U_nu(x+mu-nu)^+ U_mu(x-nu)^+ U_nu(x-nu) */
void orc_wilson_staple(const orc_ctx* c, long i, int mu, double* V) {
  double tot[4] = {0, 0, 0, 0}, t[4], a[4], b[4], s[4];
  long xp = NX(c, i, mu);
  for (int nu = 0; nu < c->D; nu++) {
    if (nu == mu) continue;
    /* upper */
    qdag(LNK(c, NX(c, i, nu), mu), a);
    qmul(LNK(c, xp, nu), a, t);
    qdag(LNK(c, i, nu), b);
    qmul(t, b, s);
    for (int k = 0; k < 4; k++) tot[k] += s[k];
    /* lower */
    long xpm = PV(c, xp, nu), xm = PV(c, i, nu);
    qdag(LNK(c, xpm, nu), a);
    qdag(LNK(c, xm, mu), b);
    qmul(a, b, t);
    qmul(t, LNK(c, xm, nu), s);
    for (int k = 0; k < 4; k++) tot[k] += s[k];
  }
  for (int k = 0; k < 4; k++) V[k] = tot[k];
}

/* su2link_staple (staples.c:134-193): -beta/2 Wilson staple minus half the
 * doublet hopping "staple"  phi(x+mu) e^{-i alpha_mu(x) sigma_3} phi(x)^+ */
void orc_link_staple(const orc_ctx* c, long i, int mu, double* V) {
  orc_wilson_staple(c, i, mu, V);
  for (int k = 0; k < 4; k++) V[k] *= -0.5 * c->p.betasu2;
  long xp = NX(c, i, mu);
  for (int h = 0; h < c->nh; h++) {
    double nphi[4], pd[4], t[4];
    memcpy(nphi, PHI(c, h, xp), sizeof(nphi));
    if (c->has_u1) {
      double e[4], r[4];
      u1phase(A1(c, i, mu), e);
      qmul(nphi, e, r);
      memcpy(nphi, r, sizeof(r));
    }
    qdag(PHI(c, h, i), pd);
    qmul(nphi, pd, t);
    for (int k = 0; k < 4; k++) V[k] -= 0.5 * t[k];
  }
}

/* su2ptrace (su2u1.c:108-116): Re Tr U_mu(x) U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+ */
static double ptrace(const orc_ctx* c, long i, int mu, int nu) {
  double t[4], s[4], a[4], b[4];
  qmul(LNK(c, i, mu), LNK(c, NX(c, i, mu), nu), t);
  qdag(LNK(c, NX(c, i, nu), mu), a);
  qmul(t, a, s);
  qdag(LNK(c, i, nu), b);
  return 2.0 * qdot0(s, b);
}

/* local_su2wilson (su2u1.c:143-157), long double accumulation as there */
static long double local_su2wilson_ld(const orc_ctx* c, long i) {
  long double res = 0.0;
  for (int d1 = 0; d1 < c->D; d1++)
    for (int d2 = 0; d2 < d1; d2++) res += (1.0 - 0.5 * ptrace(c, i, d2, d1));
  res = c->p.betasu2 * res;
  return res;
}
double orc_local_su2wilson(const orc_ctx* c, long i) { return (double)local_su2wilson_ld(c, i); }

/* ------------------------------------------------------------------ */
/* doublet                                                             */
/* ------------------------------------------------------------------ */
static inline double doubletsq(const double* a) { return 0.5 * (a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + a[3] * a[3]); }

/* hopping_trace[_su2u1] (su2u1.c:388-418): Re Tr Phi1^+ U Phi2 e^{-i a sigma_3} */
static double hop_trace(const orc_ctx* c, const double* p1, const double* u, const double* p2, double alpha) {
  double t[4], pd[4], s[4];
  qmul(u, p2, t);
  if (c->has_u1) {
    double e[4];
    u1phase(alpha, e);
    qmul(t, e, s);
    memcpy(t, s, sizeof(s));
  }
  qdag(p1, pd);
  return qdot0(pd, t);
}

/* hopping_doublet_forward / backward (su2u1.c:428-472) */
static double hop_doublet_fwd(const orc_ctx* c, long i, int d, int h) {
  return -hop_trace(c, PHI(c, h, i), LNK(c, i, d), PHI(c, h, NX(c, i, d)), c->has_u1 ? A1(c, i, d) : 0.0);
}
static double hop_doublet_bwd(const orc_ctx* c, long i, int d, int h) {
  long pm = PV(c, i, d);
  return -hop_trace(c, PHI(c, h, pm), LNK(c, pm, d), PHI(c, h, i), c->has_u1 ? A1(c, pm, d) : 0.0);
}

/* covariant_doublet (su2u1.c:477-488) */
static double covariant_doublet(const orc_ctx* c, long i, int h) {
  double tot = 0.0, mod = doubletsq(PHI(c, h, i));
  for (int d = 0; d < c->D; d++) tot += 2.0 * mod + hop_doublet_fwd(c, i, d, h);
  return tot;
}

/* get_phi12 (su2u1.c:513-520) */
static void phi12(const double* h1, const double* h2, double* re, double* im) {
  *re = 0.5 * (h1[0] * h2[0] + h1[1] * h2[1] + h1[2] * h2[2] + h1[3] * h2[3]);
  *im = 0.5 * (h1[3] * h2[0] + h1[2] * h2[1] - h1[1] * h2[2] - h1[0] * h2[3]);
}

static inline double tripletsq(const double* a) { return 0.5 * (a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

/* potential_singlet (su2u1.c:708-723) */
static double potential_singlet(const orc_ctx* c, long i) {
  const su2gpu_params* p = &c->p;
  double S = c->sing[i];
  double pot = p->b1_s * S + 0.5 * p->msq_s * S * S + 1.0 / 3.0 * p->b3_s * S * S * S + 0.25 * p->b4_s * S * S * S * S;
  if (c->nh == 1) {
    double mod = doubletsq(PHI(c, 0, i));
    pot += 0.5 * p->a1_s * S * mod + 0.5 * p->a2_s * S * S * mod;
  }
  return pot;
}

/* higgspotential (su2u1.c:528-572) */
static double higgspotential(const orc_ctx* c, long i) {
  const su2gpu_params* p = &c->p;
  double pot = 0.0, mod = 0.0;
  if (c->nh > 0) {
    mod = doubletsq(PHI(c, 0, i));
    pot += p->msq_phi * mod + p->lambda_phi * mod * mod;
    if (c->nh == 2) {
      double f11 = mod, f22 = doubletsq(PHI(c, 1, i)), R, I;
      phi12(PHI(c, 0, i), PHI(c, 1, i), &R, &I);
      pot += p->msq_phi2 * f22 + p->m12sq_re * R - p->m12sq_im * I + p->lam2 * f22 * f22 + p->lam3 * f11 * f22 +
             p->lam4 * (R * R + I * I) + p->lam5_re * (R * R - I * I) - 2.0 * p->lam5_im * R * I +
             f11 * (p->lam6_re * R - p->lam6_im * I) + f22 * (p->lam7_re * R + p->lam7_im * I);
    }
  }
  if (c->has_trip) {
    double mt = tripletsq(TRP(c, i));
    pot += p->msq_triplet * mt + p->b4 * mt * mt;
    if (c->nh > 0) pot += p->a2 * mod * mt;
  }
  if (c->has_sing) pot += potential_singlet(c, i);
  return pot;
}

/* localact_doublet (su2u1.c:495-510) */
double orc_localact_doublet(const orc_ctx* c, long i, int h) {
  double tot = covariant_doublet(c, i, h);
  for (int d = 0; d < c->D; d++) tot += hop_doublet_bwd(c, i, d, h);
  tot += higgspotential(c, i);
  return tot;
}

/* staple_doublet (staples.c:243-302):
 *   s = - sum_mu [ U_mu(x) phi(x+mu) e_mu(x)  +  U_mu(x-mu)^+ phi(x-mu) e_mu(x-mu)^+ ] */
void orc_staple_doublet(const orc_ctx* c, long i, int h, double* res) {
  for (int k = 0; k < 4; k++) res[k] = 0.0;
  for (int d = 0; d < c->D; d++) {
    double w[4], t[4], ud[4], e[4];
    long xp = NX(c, i, d), xm = PV(c, i, d);
    qmul(LNK(c, i, d), PHI(c, h, xp), w);
    if (c->has_u1) { u1phase(A1(c, i, d), e); qmul(w, e, t); memcpy(w, t, sizeof(t)); }
    for (int k = 0; k < 4; k++) res[k] -= w[k];
    qdag(LNK(c, xm, d), ud);
    qmul(ud, PHI(c, h, xm), w);
    if (c->has_u1) { u1phase(A1(c, xm, d), e); qdag(e, t); qmul(w, t, e); memcpy(w, e, sizeof(e)); }
    for (int k = 0; k < 4; k++) res[k] -= w[k];
  }
}

/* ------------------------------------------------------------------ */
/* triplet                                                             */
/* ------------------------------------------------------------------ */
/* hopping_triplet_forward / backward (su2u1.c:605-637):  -Sigma(x).R(U)Sigma(x+mu) */
static double hop_triplet_fwd(const orc_ctx* c, long i, int d) {
  double r[3];
  qrot(LNK(c, i, d), TRP(c, NX(c, i, d)), r);
  const double* a = TRP(c, i);
  return -(a[0] * r[0] + a[1] * r[1] + a[2] * r[2]);
}
static double hop_triplet_bwd(const orc_ctx* c, long i, int d) {
  long pm = PV(c, i, d);
  double r[3];
  qrot(LNK(c, pm, d), TRP(c, i), r);
  const double* a = TRP(c, pm);
  return -(a[0] * r[0] + a[1] * r[1] + a[2] * r[2]);
}
/* covariant_triplet (su2u1.c:643-651) */
static double covariant_triplet(const orc_ctx* c, long i) {
  double tot = 0.0, mod = tripletsq(TRP(c, i));
  for (int d = 0; d < c->D; d++) tot += 2.0 * mod + hop_triplet_fwd(c, i, d);
  return tot;
}
/* localact_triplet (su2u1.c:657-679) */
double orc_localact_triplet(const orc_ctx* c, long i) {
  double tot = covariant_triplet(c, i);
  for (int d = 0; d < c->D; d++) tot += hop_triplet_bwd(c, i, d);
  double mod = tripletsq(TRP(c, i));
  tot += c->p.msq_triplet * mod + c->p.b4 * mod * mod;
  if (c->nh > 0) tot += c->p.a2 * doubletsq(PHI(c, 0, i)) * mod;
  return tot;
}

/* localact_su2link (su2u1.c:166-198) */
double orc_localact_su2link(const orc_ctx* c, long i, int mu) {
  double tot = 0.0;
  for (int nu = 0; nu < c->D; nu++) {
    if (nu == mu) continue;
    tot += (1.0 - 0.5 * ptrace(c, i, mu, nu));
    tot += (1.0 - 0.5 * ptrace(c, PV(c, i, nu), mu, nu));
  }
  tot *= c->p.betasu2;
  for (int h = 0; h < c->nh; h++) tot += hop_doublet_fwd(c, i, mu, h);
  if (c->has_trip) tot += hop_triplet_fwd(c, i, mu);
  return tot;
}

/* ------------------------------------------------------------------ */
/* U(1)                                                                */
/* ------------------------------------------------------------------ */
/* u1ptrace (su2u1.c:300-309) */
static double u1ptrace(const orc_ctx* c, long i, int d1, int d2) {
  return A1(c, i, d1) + A1(c, NX(c, i, d1), d2) - A1(c, NX(c, i, d2), d1) - A1(c, i, d2);
}
/* local_u1wilson (su2u1.c:316-328) */
double orc_local_u1wilson(const orc_ctx* c, long i) {
  double res = 0.0;
  for (int d1 = 0; d1 < c->D; d1++)
    for (int d2 = 0; d2 < d1; d2++) res += (1.0 - cos(c->p.r_u1 * u1ptrace(c, i, d2, d1)));
  return c->p.betau1 * res;
}
/* localact_u1link (su2u1.c:336-354) */
double orc_localact_u1link(const orc_ctx* c, long i, int mu) {
  double tot = 0.0;
  for (int nu = 0; nu < c->D; nu++) {
    if (nu == mu) continue;
    tot += (1.0 - cos(c->p.r_u1 * u1ptrace(c, i, mu, nu)));
    tot += (1.0 - cos(c->p.r_u1 * u1ptrace(c, PV(c, i, nu), mu, nu)));
  }
  tot *= c->p.betau1;
  for (int h = 0; h < c->nh; h++) tot += hop_doublet_fwd(c, i, mu, h);
  return tot;
}

/* localact_singlet (su2u1.c:688-705) */
double orc_localact_singlet(const orc_ctx* c, long i) {
  double S = c->sing[i], res = c->D * S * S;
  for (int d = 0; d < c->D; d++) res -= S * (c->sing[NX(c, i, d)] + c->sing[PV(c, i, d)]);
  res += potential_singlet(c, i);
  return res;
}

/* action_local (measure.c:314-343) */
double orc_action_local(const orc_ctx* c, long i) {
  double tot = 0.0;
  tot = (double)((long double)tot + local_su2wilson_ld(c, i));
  if (c->has_u1) tot += orc_local_u1wilson(c, i);
  tot += higgspotential(c, i);
  for (int h = 0; h < c->nh; h++) tot += covariant_doublet(c, i, h);
  if (c->has_trip) tot += covariant_triplet(c, i);
  if (c->has_sing) {
    double S = c->sing[i];
    tot += c->D * S * S;
    for (int d = 0; d < c->D; d++) tot -= S * c->sing[NX(c, i, d)];
  }
  return tot;
}

/* ------------------------------------------------------------------ */
/* magnetic charge (magfield.c:90-280), complex 2x2 matrices            */
/* ------------------------------------------------------------------ */
typedef struct { double re[4], im[4]; } cmat; /* row-major 2x2 */

static void cmat_mul(const cmat* a, const cmat* b, cmat* r) {
  cmat t;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) {
      double sr = 0, si = 0;
      for (int k = 0; k < 2; k++) {
        double ar = a->re[2 * i + k], ai = a->im[2 * i + k], br = b->re[2 * k + j], bi = b->im[2 * k + j];
        sr += ar * br - ai * bi;
        si += ar * bi + ai * br;
      }
      t.re[2 * i + j] = sr; t.im[2 * i + j] = si;
    }
  *r = t;
}
static void cmat_dag(const cmat* a, cmat* r) {
  cmat t;
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) { t.re[2 * i + j] = a->re[2 * j + i]; t.im[2 * i + j] = -a->im[2 * j + i]; }
  *r = t;
}
/* (1 + n.sigma/2... ) projector of projector()/project_u1(): 0.5 (I + 0.5 h.sigma), h = 2 a/|a| */
static void projector_mat(const double* a, cmat* P) {
  double m = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  double n1 = a[0] / m, n2 = a[1] / m, n3 = a[2] / m;
  P->re[0] = 0.5 * (1.0 + n3); P->im[0] = 0.0;
  P->re[1] = 0.5 * n1;         P->im[1] = -0.5 * n2;
  P->re[2] = 0.5 * n1;         P->im[2] = 0.5 * n2;
  P->re[3] = 0.5 * (1.0 - n3); P->im[3] = 0.0;
}
static void link_mat(const double* u, cmat* U) {
  U->re[0] = u[0]; U->im[0] = u[3];
  U->re[1] = u[2]; U->im[1] = u[1];
  U->re[2] = -u[2]; U->im[2] = u[1];
  U->re[3] = u[0]; U->im[3] = -u[3];
}
/* project_u1 (magfield.c:115-184): Pi(x) U_mu(x) Pi(x+mu) */
static void project_u1(const orc_ctx* c, long i, int d, cmat* out) {
  cmat Pl, Pr, U, t;
  projector_mat(TRP(c, i), &Pl);
  projector_mat(TRP(c, NX(c, i, d)), &Pr);
  link_mat(LNK(c, i, d), &U);
  cmat_mul(&Pl, &U, &t);
  cmat_mul(&t, &Pr, out);
}
/* alpha_proj (magfield.c:189-216) */
double orc_alpha_proj(const orc_ctx* c, long i, int d1, int d2) {
  cmat u1, u2, u3, u4, t;
  project_u1(c, i, d1, &u1);
  project_u1(c, NX(c, i, d1), d2, &u2);
  project_u1(c, NX(c, i, d2), d1, &u3);
  project_u1(c, i, d2, &u4);
  cmat_mul(&u1, &u2, &t);
  cmat_dag(&u3, &u3);
  cmat_mul(&t, &u3, &t);
  cmat_dag(&u4, &u4);
  cmat_mul(&t, &u4, &t);
  double a = atan2(t.im[0] + t.im[3], t.re[0] + t.re[3]);
  return a * sqrt(c->p.betasu2);
}
/* magfield (magfield.c:221-258) */
static double magfield(const orc_ctx* c, long i, int dir) {
  double res = 0.0;
  for (int d1 = 0; d1 < c->D; d1++) {
    if (d1 == dir) continue;
    for (int d2 = d1 + 1; d2 < c->D; d2++) {
      if (d2 == dir) continue;
      double a = orc_alpha_proj(c, i, d1, d2);
      if (d1 > dir) res += a;
      else if (d2 > dir) res -= a;
      else res += a;
    }
  }
  return res;
}
/* magcharge_cube (magfield.c:262-280) */
double orc_magcharge_cube(const orc_ctx* c, long i) {
  double res = 0.0;
  for (int d = 0; d < c->D; d++) {
    double B1 = magfield(c, i, d);
    double B2 = magfield(c, NX(c, i, d), d);
    res += B2 - B1;
  }
  return res;
}

/* ------------------------------------------------------------------ */
/* local update algorithms                                             */
/* ------------------------------------------------------------------ */

/* Kennedy-Pendleton heatbath, heatbath_su2link (heatbath.c:15-124).
 * Draw order per trial: two exponentials, the cosine, the accept uniform;
 * then three uniforms per trial of the rejection sampling on the sphere;
 * with a triplet present one more for the accept/reject of its hopping. */
static int heatbath_su2link(orc_ctx* c, long i, int mu) {
  double old[4], oldact = 0.0;
  double* U = LNK(c, i, mu);
  if (c->has_trip) { memcpy(old, U, sizeof(old)); oldact += hop_triplet_fwd(c, i, mu); }
  double V[4];
  orc_link_staple(c, i, mu, V);
  double a = sqrt(qsq(V));
  for (int k = 0; k < 4; k++) V[k] *= -1.0 / a;
  a *= 2.0;
  double a0, r1, r2, r3, d;
  int loop = 1, maxloops = 200;
  do {
    r1 = -1.0 * log(1.0 - uni(c)) / a;
    r2 = -1.0 * log(1.0 - uni(c)) / a;
    r3 = cos(2 * M_PI * uni(c));
    r3 *= r3;
    d = r1 * r3 + r2;
    r3 = 1.0 - uni(c);
    loop++;
  } while (r3 * r3 > 1 - 0.5 * d && loop <= maxloops);
  if (loop > maxloops) { a0 = 1e-9; c->cnt[SU2GPU_C_KP_CAP]++; }
  else a0 = 1.0 - d;
  double rad = 1.0 - a0 * a0;
  if (rad < 0.0) return 0;
  rad = sqrt(rad);
  d = 2.0;
  while (d > 1.0 || d == 0.0) {
    r1 = 2.0 * uni(c) - 1.0;
    r2 = 2.0 * uni(c) - 1.0;
    r3 = 2.0 * uni(c) - 1.0;
    d = r1 * r1 + r2 * r2 + r3 * r3;
  }
  d = sqrt(d);
  double nl[4] = {a0, r1 * (rad / d), r2 * (rad / d), r3 * (rad / d)}, vd[4];
  qdag(V, vd);
  qmul(nl, vd, U);
  if (c->has_trip) {
    double diff = oldact - hop_triplet_fwd(c, i, mu);
    if (uni(c) < exp(diff)) return 1;
    memcpy(U, old, sizeof(old));
    return 0;
  }
  return 1;
}

/* random_su2link (init.c:43-58) */
static void random_su2link(orc_ctx* c, double* su2) {
  double u[4];
  u[0] = 10.0 * (uni(c) - 0.5);
  u[1] = 1.0 * (uni(c) - 0.5);
  u[2] = 1.0 * (uni(c) - 0.5);
  u[3] = 1.0 * (uni(c) - 0.5);
  double n = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2] + u[3] * u[3]);
  for (int k = 0; k < 4; k++) su2[k] = u[k] / n;
}

/* Metropolis decision shared by metropolis.c:15-167: a decrease is always
 * accepted without a draw; an increase draws one uniform. */
static int metro_accept(orc_ctx* c, double diff) {
  if (diff < 0) return 1;
  if (diff > 0 && exp(-(diff)) > uni(c)) return 1;
  return 0;
}

/* metro_su2link (metropolis.c:15-41) */
static int metro_su2link(orc_ctx* c, long i, int mu) {
  double* U = LNK(c, i, mu);
  double old[4], nl[4], t[4];
  memcpy(old, U, sizeof(old));
  double a0 = orc_localact_su2link(c, i, mu);
  random_su2link(c, nl);
  qmul(U, nl, t);
  memcpy(U, t, sizeof(t));
  double a1 = orc_localact_su2link(c, i, mu);
  if (metro_accept(c, a1 - a0)) return 1;
  memcpy(U, old, sizeof(old));
  return 0;
}

/* metro_u1link (metropolis.c:48-70) */
static int metro_u1link(orc_ctx* c, long i, int mu) {
  double* a = c->u1 + i * c->D + mu;
  double old = *a;
  double a0 = orc_localact_u1link(c, i, mu);
  *a += 0.95 * (uni(c) - 0.5);
  double a1 = orc_localact_u1link(c, i, mu);
  if (metro_accept(c, a1 - a0)) return 1;
  *a = old;
  return 0;
}

/* metro_doublet (metropolis.c:77-106) */
static int metro_doublet(orc_ctx* c, long i, int h) {
  double* f = PHI(c, h, i);
  double old[4];
  memcpy(old, f, sizeof(old));
  double a0 = orc_localact_doublet(c, i, h);
  for (int k = 0; k < 4; k++) f[k] += 1.0 * (uni(c) - 0.5);
  double a1 = orc_localact_doublet(c, i, h);
  if (metro_accept(c, a1 - a0)) return 1;
  memcpy(f, old, sizeof(old));
  return 0;
}

/* metro_triplet (metropolis.c:113-143) */
static int metro_triplet(orc_ctx* c, long i) {
  double* f = TRP(c, i);
  double old[3];
  memcpy(old, f, sizeof(old));
  double a0 = orc_localact_triplet(c, i);
  for (int k = 0; k < 3; k++) f[k] += 1.0 * (uni(c) - 0.5);
  double a1 = orc_localact_triplet(c, i);
  if (metro_accept(c, a1 - a0)) return 1;
  memcpy(f, old, sizeof(old));
  return 0;
}

/* metro_singlet (metropolis.c:148-167) */
static int metro_singlet(orc_ctx* c, long i) {
  double old = c->sing[i];
  double a0 = orc_localact_singlet(c, i);
  c->sing[i] += 1.0 * (uni(c) - 0.5);
  double a1 = orc_localact_singlet(c, i);
  if (metro_accept(c, a1 - a0)) return 1;
  c->sing[i] = old;
  return 0;
}

/* polysolve3 (overrelax.c:14-34): the real root of a x^3 + b x^2 + c x + d
 * by Cardano's formula when the discriminant is negative, else b/a. */
static double polysolve3_cr(orc_ctx* c, creal a, creal b, creal cc, creal d) {
  creal discr = 18.0 * a * b * cc * d - 4.0 * b * b * b * d + b * b * cc * cc - 4.0 * a * cc * cc * cc - 27.0 * a * a * d * d;
  creal del1 = 2.0 * b * b * b - 9.0 * a * b * cc + 27.0 * a * a * d;
  double x;
  if (discr < 0.0) {
    creal A = 0.5 * (del1 + a * sqrt((double)(-27.0 * discr)));
    A = cbrt((double)A);
    x = (double)(-1.0 * (b + A + (b * b - 3.0 * a * cc) / A) / (3.0 * a));
  } else {
    x = (double)(b / a);
    if (c) c->cnt[SU2GPU_C_POLY_FALLBACK]++;
  }
  return x;
}
double orc_polysolve3(double a, double b, double cc, double d) { return polysolve3_cr(NULL, a, b, cc, d); }

/* overrelax_doublet (overrelax.c:54-128), one doublet */
static int overrelax_doublet(orc_ctx* c, long i) {
  const su2gpu_params* p = &c->p;
  double s[4];
  double* f = PHI(c, 0, i);
  orc_staple_doublet(c, i, 0, s);
  double F = 0.0;
  for (int k = 0; k < 4; k++) F += s[k] * s[k];
  F = sqrt(F);
  double X = 0.0;
  for (int k = 0; k < 4; k++) X += f[k] * s[k];
  X /= F;
  double Ysq = 0.0;
  for (int k = 0; k < 4; k++) { double y = f[k] - X * s[k] / F; Ysq += y * y; }
  double B = 0.5 * p->msq_phi + 1.0 * c->D;
  if (c->has_trip) B += 0.5 * p->a2 * tripletsq(TRP(c, i));
  if (c->has_sing) { double S = c->sing[i]; B += 0.25 * p->a1_s * S + 0.25 * p->a2_s * S * S; }
  double C = 0.25 * p->lambda_phi;
  creal alpha = C;
  creal beta = C * X;
  creal cc = B + 2.0 * Ysq * C;
  creal gamma = (cc + C * X * X);
  creal delta = (F + cc * X + C * X * X * X);
  double newX = polysolve3_cr(c, alpha, beta, gamma, delta);
  double dV = F + 2.0 * B * X + 4.0 * C * (X * X * X + Ysq * X);
  double dVn = F + 2.0 * B * newX + 4.0 * C * (newX * newX * newX + Ysq * newX);
  double acc = fabs(dV / dVn);
  if (acc >= uni(c)) {
    for (int k = 0; k < 4; k++) f[k] = -1.0 * f[k] + (newX + X) * s[k] / F;
    return 1;
  }
  return 0;
}

/* overrelax_triplet (overrelax.c:137-236).  The reference's "#ifdef HIGGS"
 * portal term (202-204) is never compiled, so B has no a2 phi^2 part here. */
static int overrelax_triplet(orc_ctx* c, long i) {
  const su2gpu_params* p = &c->p;
  double s[3] = {0, 0, 0}, r[3];
  double* f = TRP(c, i);
  for (int d = 0; d < c->D; d++) {
    long xp = NX(c, i, d), xm = PV(c, i, d);
    qrot(LNK(c, i, d), TRP(c, xp), r);
    for (int k = 0; k < 3; k++) s[k] -= r[k];
    double ud[4];
    qdag(LNK(c, xm, d), ud);
    qrot(ud, TRP(c, xm), r);
    for (int k = 0; k < 3; k++) s[k] -= r[k];
  }
  double F = sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
  double X = (f[0] * s[0] + f[1] * s[1] + f[2] * s[2]) / F;
  double Ysq = 0.0;
  for (int k = 0; k < 3; k++) { double y = f[k] - X * s[k] / F; Ysq += y * y; }
  double B = 0.5 * p->msq_triplet + 1.0 * c->D;
  double C = 0.25 * p->b4;
  creal alpha = C;
  creal beta = C * X;
  creal cc = B + 2.0 * Ysq * C;
  creal gamma = (cc + C * X * X);
  creal delta = (F + cc * X + C * X * X * X);
  double newX = polysolve3_cr(c, alpha, beta, gamma, delta);
  double dV = F + 2.0 * B * X + 4.0 * C * (X * X * X + Ysq * X);
  double dVn = F + 2.0 * B * newX + 4.0 * C * (newX * newX * newX + Ysq * newX);
  double acc = fabs(dV / dVn);
  if (acc >= uni(c)) {
    for (int k = 0; k < 3; k++) f[k] = -1.0 * f[k] + (newX + X) * s[k] / F;
    return 1;
  }
  return 0;
}

/* overrelax_singlet (overrelax.c:243-285) */
static int overrelax_singlet(orc_ctx* c, long i) {
  const su2gpu_params* p = &c->p;
  double S = c->sing[i];
  double c1 = p->b1_s;
  for (int d = 0; d < c->D; d++) c1 -= (c->sing[NX(c, i, d)] + c->sing[PV(c, i, d)]);
  double c2 = c->D + 0.5 * p->msq_s;
  double c3 = 1.0 / 3.0 * p->b3_s;
  double c4 = 0.25 * p->b4_s;
  if (c->nh == 1) {
    double phisq = doubletsq(PHI(c, 0, i));
    c1 += 0.5 * p->a1_s * phisq;
    c2 += 0.5 * p->a2_s * phisq;
  }
  double d0 = c1 + c2 * S + c3 * S * S + c4 * S * S * S;
  double d1 = c2 + c3 * S + c4 * S * S;
  double d2 = c3 + c4 * S;
  double d3 = c4;
  double Y = polysolve3_cr(c, d3, d2, d1, d0);
  double dV = c1 + 2.0 * c2 * S + 3.0 * c3 * S * S + 4.0 * c4 * S * S * S;
  double dVn = c1 + 2.0 * c2 * Y + 3.0 * c3 * Y * Y + 4.0 * c4 * Y * Y * Y;
  if (fabs(dV / dVn) >= uni(c)) { c->sing[i] = Y; return 1; }
  return 0;
}

/* overrelax_higgs2 (overrelax.c:295-417): XY overrelaxation of doublet h
 * with the two-doublet potential; Y is kept fixed. */
static int overrelax_higgs2(orc_ctx* c, long i, int h) {
  const su2gpu_params* p = &c->p;
  double s[4];
  double* f = PHI(c, h, i);
  orc_staple_doublet(c, i, h, s);
  const double* H;
  double G[4], l67re, l67im, lo_re, lo_im, lam12, msq;
  int sign = -1;
  if (h == 0) {
    H = PHI(c, 1, i); lam12 = p->lambda_phi; msq = p->msq_phi;
    l67re = p->lam7_re; l67im = p->lam7_im; lo_re = p->lam6_re; lo_im = -p->lam6_im;
  } else {
    H = PHI(c, 0, i); sign = 1; lam12 = p->lam2; msq = p->msq_phi2;
    l67re = p->lam6_re; l67im = -p->lam6_im; lo_re = p->lam7_re; lo_im = p->lam7_im;
  }
  G[0] = sign * H[3]; G[1] = sign * H[2]; G[2] = -1.0 * sign * H[1]; G[3] = -1.0 * sign * H[0];
  double Hsq = doubletsq(H);
  for (int k = 0; k < 4; k++) {
    s[k] += 0.5 * (p->m12sq_re + Hsq * l67re) * H[k];
    s[k] += 0.5 * (-1.0 * p->m12sq_im + Hsq * l67im) * G[k];
    s[k] = -1.0 * s[k];
  }
  double F = 0.0;
  for (int k = 0; k < 4; k++) F += s[k] * s[k];
  F = sqrt(F);
  double X = 0.0;
  for (int k = 0; k < 4; k++) { s[k] /= F; X += f[k] * s[k]; }
  double Y[4], Ysq = 0.0;
  for (int k = 0; k < 4; k++) { Y[k] = f[k] - X * s[k]; Ysq += Y[k] * Y[k]; }
  double Hf = 0, Gf = 0, HY = 0, GY = 0;
  for (int k = 0; k < 4; k++) { Hf += H[k] * s[k]; Gf += G[k] * s[k]; HY += H[k] * Y[k]; GY += G[k] * Y[k]; }
  double b4 = 0.25 * lam12;
  double b3 = 0.25 * (Hf * lo_re + Gf * lo_im);
  double b2 = 0.5 * msq + 1.0 * c->D + 0.5 * Ysq * lam12 + 0.25 * (HY * lo_re + GY * lo_im);
  double b1 = -1.0 * F + 0.25 * Ysq * (Hf * lo_re + Gf * lo_im);
  b2 += 0.5 * Hsq * p->lam3 + 0.25 * p->lam4 * (Hf * Hf + Gf * Gf) + 0.25 * p->lam5_re * (Hf * Hf - Gf * Gf) -
        0.5 * p->lam5_im * Gf * Hf;
  b1 += 0.5 * Hf * (HY * p->lam4 + HY * p->lam5_re - GY * p->lam5_im) +
        0.5 * Gf * (GY * p->lam4 - GY * p->lam5_re - HY * p->lam5_im);
  creal aa = b4;
  creal bb = b3 + b4 * X;
  creal cc = b2 + b3 * X + b4 * X * X;
  creal dd = b1 + b2 * X + b3 * X * X + b4 * X * X * X;
  double Xn = polysolve3_cr(c, aa, bb, cc, dd);
  double dV = 4.0 * b4 * X * X * X + 3.0 * b3 * X * X + 2.0 * b2 * X + b1;
  double dVn = 4.0 * b4 * Xn * Xn * Xn + 3.0 * b3 * Xn * Xn + 2.0 * b2 * Xn + b1;
  double acc = fabs(dV / dVn);
  if (acc >= uni(c)) {
    for (int k = 0; k < 4; k++) f[k] = f[k] + s[k] * (Xn - X);
    return 1;
  }
  return 0;
}

static int site_update(orc_ctx* c, int kind, long i, int sub) {
  switch (kind) {
    case 1: return heatbath_su2link(c, i, sub);
    case 2: return metro_su2link(c, i, sub);
    case 3: return metro_u1link(c, i, sub);
    case 4: return c->nh == 2 ? overrelax_higgs2(c, i, sub) : overrelax_doublet(c, i);
    case 5: return metro_doublet(c, i, sub);
    case 6: return overrelax_triplet(c, i);
    case 7: return metro_triplet(c, i);
    case 8: return overrelax_singlet(c, i);
    case 9: return metro_singlet(c, i);
  }
  return -1;
}

int orc_site_update(orc_ctx* c, int kind, long i, int sub, uint32_t pass) {
  orc_stream_init(&c->rng, c->seed, c->sweep, c->chain);
  orc_stream_at(&c->rng, (uint32_t)i, pass);
  return site_update(c, kind, i, sub);
}
int orc_site_draws(const orc_ctx* c) { return (int)c->rng.draw; }

/* The overrelaxation proposal at site i (overrelax.c:54-417): the update
 * run with every uniform 0, which it always accepts (|dV/dV'| >= 0), and
 * the old value put back.  kind 4 doublet `sub`, 6 triplet, 8 singlet;
 * returns the reals written to out (-1: absent field). */
int orc_or_proposal(orc_ctx* c, int kind, long i, int sub, double* out) {
  double* f = NULL;
  int n = -1;
  if (kind == 4 && sub < c->nh) { f = PHI(c, sub, i); n = 4; }
  else if (kind == 6 && c->has_trip) { f = TRP(c, i); n = 3; }
  else if (kind == 8 && c->has_sing) { f = c->sing + i; n = 1; }
  if (!f) return -1;
  double old[4];
  memcpy(old, f, sizeof(double) * n);
  c->zero_uniforms = 1;
  site_update(c, kind, i, sub);
  c->zero_uniforms = 0;
  memcpy(out, f, sizeof(double) * n);
  memcpy(f, old, sizeof(double) * n);
  return n;
}

/* ------------------------------------------------------------------ */
/* multicanonical (multicanonical.c)                                   */
/* ------------------------------------------------------------------ */
int orc_muca_set(orc_ctx* c, const su2gpu_weight* w) {
  free_weight(c);
  c->w = *w;
  int n = w->bins + 2;
  c->w.pos = (double*)malloc(sizeof(double) * n); memcpy(c->w.pos, w->pos, sizeof(double) * n);
  c->w.W = (double*)malloc(sizeof(double) * n); memcpy(c->w.W, w->W, sizeof(double) * n);
  c->w.slope = (double*)malloc(sizeof(double) * n); memcpy(c->w.slope, w->slope, sizeof(double) * n);
  c->w.b = (double*)malloc(sizeof(double) * n); memcpy(c->w.b, w->b, sizeof(double) * n);
  c->w.hits = (int32_t*)malloc(sizeof(int32_t) * n); memcpy(c->w.hits, w->hits, sizeof(int32_t) * n);
  c->w.gsum = (int64_t*)calloc(n, sizeof(int64_t));
  c->w.nsum = (int64_t*)calloc(n, sizeof(int64_t));
  c->w.hgram = (double*)calloc(n, sizeof(double));
  if (w->gsum) memcpy(c->w.gsum, w->gsum, sizeof(int64_t) * n);
  if (w->nsum) memcpy(c->w.nsum, w->nsum, sizeof(int64_t) * n);
  if (w->hgram) memcpy(c->w.hgram, w->hgram, sizeof(double) * n);
  c->bu_phi = (double*)malloc(sizeof(double) * c->V * 4);
  c->bu_trip = (double*)malloc(sizeof(double) * c->V * 3);
  c->muca_on = 1;
  return 0;
}

int orc_muca_get(const orc_ctx* c, su2gpu_weight* w) {
  if (!c->muca_on) return -1;
  double *pos = w->pos, *W = w->W, *slope = w->slope, *b = w->b, *hg = w->hgram;
  int32_t* hits = w->hits;
  int64_t *gs = w->gsum, *ns = w->nsum;
  int n = c->w.bins + 2;
  *w = c->w;
  w->pos = pos; w->W = W; w->slope = slope; w->b = b; w->hits = hits; w->gsum = gs; w->nsum = ns; w->hgram = hg;
  if (pos) memcpy(pos, c->w.pos, sizeof(double) * n);
  if (W) memcpy(W, c->w.W, sizeof(double) * n);
  if (slope) memcpy(slope, c->w.slope, sizeof(double) * n);
  if (b) memcpy(b, c->w.b, sizeof(double) * n);
  if (hits) memcpy(hits, c->w.hits, sizeof(int32_t) * n);
  if (gs) memcpy(gs, c->w.gsum, sizeof(int64_t) * n);
  if (ns) memcpy(ns, c->w.nsum, sizeof(int64_t) * n);
  if (hg) memcpy(hg, c->w.hgram, sizeof(double) * n);
  return 0;
}

/* linearize_weight (multicanonical.c:337-346) */
static void linearize_weight(su2gpu_weight* w) {
  w->slope[0] = 0; w->slope[w->bins + 1] = 0;
  w->b[0] = w->W[0]; w->b[w->bins + 1] = w->W[w->bins + 1];
  for (int i = 1; i < w->bins + 1; i++) {
    w->slope[i] = (w->W[i + 1] - w->W[i]) / (w->pos[i + 1] - w->pos[i]);
    w->b[i] = w->W[i] - w->slope[i] * w->pos[i];
  }
}

/* whichbin (multicanonical.c:671-704) */
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
  return w->bins;
}
int orc_whichbin(const orc_ctx* c, double v) { return whichbin(&c->w, v); }

/* get_weight (multicanonical.c:350-379) */
static double get_weight(const su2gpu_weight* w, double val) {
  if (val >= w->max) return w->b[w->bins + 1];
  if (val < w->min) return w->b[0];
  int bin = whichbin(w, val);
  if (bin >= w->bins + 1) return w->b[w->bins + 1];
  return w->b[bin] + w->slope[bin] * val;
}
double orc_get_weight(const orc_ctx* c, double v) { return get_weight(&c->w, v); }

/* muca_accumulate_hits (multicanonical.c:451-498) */
static void accumulate_hits(su2gpu_weight* w, double val) {
  int bin = whichbin(w, val);
  if (bin == 0) {
    double dmin = w->pos[2] - w->pos[1];
    if (val < w->pos[1] - 0.5 * dmin) return;
    bin += 1;
  } else if (bin < w->bins + 1) {
    if (val - w->pos[bin] > w->pos[bin + 1] - val) bin = bin + 1;
  } else {
    double dmax = w->pos[w->bins + 1] - w->pos[w->bins];
    if (val > w->pos[w->bins + 1] + 0.5 * dmax) return;
  }
  if (w->mode == SU2GPU_MUCA_FAST) {
    w->hits[bin] += 5;
    if (bin > 1) w->hits[bin - 1] += 3;
    if (bin > 2) w->hits[bin - 2] += 1;
    if (bin < w->bins) w->hits[bin + 1] += 3;
    if (bin < w->bins - 1) w->hits[bin + 2] += 1;
  } else if (w->mode == SU2GPU_MUCA_SLOW) {
    w->hits[bin]++;
    w->hgram[bin] += exp(get_weight(w, val));
  }
}

/* update_weight (multicanonical.c:504-557) */
static int update_weight(su2gpu_weight* w) {
  int first = -1;
  double delta = 0.0;
  for (int i = 0; i < w->bins + 2; i++) {
    if (w->pos[i] >= w->wrk_min && w->wrk_max >= w->pos[i]) {
      if (first < 0) first = i;
      delta = (w->hits[i] - w->hits[first]) * w->delta / ((double)w->bins);
      w->W[i] += delta;
    } else if (w->wrk_max < w->pos[i]) {
      w->W[i] += delta;
    }
  }
  w->W[0] = w->W[1];
  w->W[w->bins + 1] = w->W[w->bins];
  linearize_weight(w);
  int tunnel = 0;
  if (w->last_max && w->hits[1] > 0) { w->last_max = 0; tunnel = 1; }
  else if (!w->last_max && w->hits[w->bins] > 0) { w->last_max = 1; tunnel = 1; }
  if (tunnel > 0) w->delta /= 1.5;
  for (int i = 0; i < w->bins + 2; i++) w->hits[i] = 0;
  return tunnel;
}

/* update_weight_slow (multicanonical.c:561-666) */
static void update_weight_slow(su2gpu_weight* w) {
  int n = w->bins + 2;
  double* wold = (double*)malloc(sizeof(double) * n);
  memcpy(wold, w->W, sizeof(double) * n);
  double dmin = w->pos[2] - w->pos[1];
  w->hgram[1] /= dmin;
  for (int i = 2; i < w->bins + 1; i++) w->hgram[i] /= (w->pos[i + 1] - w->pos[i - 1]);
  int first = -1, last = -1, hits_min = 8;
  for (int i = 1; i < w->bins + 1; i++) {
    if (w->pos[i] >= w->wrk_min && w->wrk_max >= w->pos[i]) {
      if (first < 0) { first = i; continue; }
      w->nsum[i] += w->hits[i];
      int g = 0;
      if (w->hits[i] >= hits_min && w->hits[i - 1] >= hits_min) {
        g = w->hits[i] + w->hits[i - 1];
      } else {
        w->W[i] = wold[i] - wold[i - 1] + w->W[i - 1];
        continue;
      }
      long gsum_new = w->gsum[i] + g;
      double ln = w->hgram[i - 1] / w->hgram[i];
      ln = -1.0 * g * log(ln);
      w->W[i] = w->W[i - 1] + ((wold[i] - wold[i - 1]) * w->gsum[i] + ln) / ((double)gsum_new);
      w->gsum[i] = gsum_new;
    } else if (w->wrk_max < w->pos[i]) {
      if (last < 0) last = i - 1;
      double diff = w->W[last] - wold[last];
      w->W[i] += diff;
    }
  }
  for (int i = 0; i < n; i++) { w->hits[i] = 0; w->hgram[i] = 0.0; }
  w->W[0] = w->W[1];
  w->W[w->bins + 1] = w->W[w->bins];
  double c = 2.0;
  memcpy(wold, w->W, sizeof(double) * n);
  double corr = 0.0;
  if (first == 1) dmin = w->pos[first + 1] - w->pos[first];
  else dmin = w->pos[first + 1] - w->pos[first - 1];
  for (int i = first + 1; i < w->bins + 1; i++) {
    if (i <= last) {
      double diff1 = w->pos[i + 1] - w->pos[i - 1];
      corr = c * log((dmin / diff1) * w->nsum[i] / w->nsum[first]);
      w->W[i] += corr;
    } else {
      w->W[i] += corr;
    }
  }
  w->W[0] = w->W[1];
  w->W[w->bins + 1] = w->W[w->bins];
  linearize_weight(w);
  memcpy(w->W, wold, sizeof(double) * n);
  free(wold);
}

/* multicanonical_acceptance (multicanonical.c:385-445) with the global draw */
static int muca_acceptance(orc_ctx* c, double oldval, double newval, int check) {
  su2gpu_weight* w = &c->w;
  double Wn = get_weight(w, newval), Wo = get_weight(w, oldval);
  orc_stream_at(&c->rng, ORC_GLOBAL_SITE, (uint32_t)c->pass);
  c->rng.draw = 2u * (uint32_t)check;
  int accept = exp(-(Wn - Wo)) > uni(c) ? 1 : 0;
  if (w->mode != SU2GPU_MUCA_READONLY) {
    if (!accept) newval = oldval;
    accumulate_hits(w, newval);
    w->muca_count++;
    if (w->muca_count % w->update_interval == 0) {
      if (w->mode == SU2GPU_MUCA_FAST) update_weight(w);
      else if (w->mode == SU2GPU_MUCA_SLOW) update_weight_slow(w);
      w->muca_count = 0;
    }
  }
  return accept;
}

/* calc_orderparam (multicanonical.c:709-751) */
double orc_calc_orderparam(orc_ctx* c, int par) {
  double tot = 0.0;
  long lo = par == EVEN ? 0 : c->half, hi = par == EVEN ? c->half : c->V;
  switch (c->w.orderparam) {
    case SU2GPU_SIGMASQ: for (long i = lo; i < hi; i++) tot += tripletsq(TRP(c, i)); break;
    case SU2GPU_PHI2MINUSSIGMA2:
      for (long i = lo; i < hi; i++) tot += doubletsq(PHI(c, 0, i)) - tripletsq(TRP(c, i));
      break;
    case SU2GPU_PHISQ: for (long i = lo; i < hi; i++) tot += doubletsq(PHI(c, 0, i)); break;
    case SU2GPU_PHI2SQ: for (long i = lo; i < hi; i++) tot += doubletsq(PHI(c, 1, i)); break;
  }
  tot = tot / c->V;
  c->w.param_value[par] = tot;
  return tot + c->w.param_value[1 - par];
}

/* init_last_max (multicanonical.c:826-831) */
void orc_muca_init_last_max(orc_ctx* c) {
  double val = c->w.param_value[0] + c->w.param_value[1];
  c->w.last_max = (fabs(val - c->w.wrk_min) >= fabs(val - c->w.wrk_max));
}

/* muca_check (update.c:13-30) */
static int muca_check(orc_ctx* c, int par, int check) {
  double old = c->w.param_value[EVEN] + c->w.param_value[ODD];
  double nw = orc_calc_orderparam(c, par);
  int acc = muca_acceptance(c, old, nw, check);
  if (!acc) c->w.param_value[par] = old - c->w.param_value[1 - par];
  c->cnt[SU2GPU_C_ACC_MUCA] += acc;
  c->cnt[SU2GPU_C_TOTAL_MUCA]++;
  return acc;
}

static void copy_half(double* dst, const double* src, int dofs, long lo, long hi) {
  memcpy(dst + lo * dofs, src + lo * dofs, sizeof(double) * (hi - lo) * dofs);
}

/* ------------------------------------------------------------------ */
/* checkerboard sweeps (update.c:35-259)                               */
/* ------------------------------------------------------------------ */
static void sweep_links(orc_ctx* c, int par, int mu, int alg) {
  long lo = par == EVEN ? 0 : c->half, hi = par == EVEN ? c->half : c->V;
  for (long i = lo; i < hi; i++) {
    orc_stream_at(&c->rng, (uint32_t)i, (uint32_t)c->pass);
    if (alg == SU2GPU_HEATBATH) c->cnt[SU2GPU_C_ACC_SU2LINK] += heatbath_su2link(c, i, mu);
    else if (alg == SU2GPU_METROPOLIS) c->cnt[SU2GPU_C_ACC_SU2LINK] += metro_su2link(c, i, mu);
    c->cnt[SU2GPU_C_TOTAL_SU2LINK]++;
  }
}

static void sweep_u1(orc_ctx* c, int par, int mu) {
  long lo = par == EVEN ? 0 : c->half, hi = par == EVEN ? c->half : c->V;
  for (long i = lo; i < hi; i++) {
    orc_stream_at(&c->rng, (uint32_t)i, (uint32_t)c->pass);
    if (c->p.algorithm_u1link == SU2GPU_METROPOLIS) c->cnt[SU2GPU_C_ACC_U1LINK] += metro_u1link(c, i, mu);
    c->cnt[SU2GPU_C_TOTAL_U1LINK]++;
  }
}

/* checkerboard_sweep_su2doublet / _su2triplet (update.c:82-229): a sweep
 * of one parity with `checks_per_sweep` global multicanonical checks over
 * contiguous index blocks, restoring the block from the backup on reject. */
static int sweep_scalar(orc_ctx* c, int par, int metro, int field, int h) {
  long lo = par == EVEN ? 0 : c->half, hi = par == EVEN ? c->half : c->V;
  int accept = 1, do_muca = 0, dofs = 0;
  double *fld = NULL, *bu = NULL;
  long interval = c->V, count = 0;
  if (c->muca_on && c->w.do_acceptance) {
    int op = c->w.orderparam;
    if (field == 0 && ((h == 0 && (op == SU2GPU_PHISQ || op == SU2GPU_PHI2MINUSSIGMA2)) || (h == 1 && op == SU2GPU_PHI2SQ))) {
      do_muca = 1; fld = c->phi[h]; bu = c->bu_phi; dofs = 4;
    }
    if (field == 1 && (op == SU2GPU_SIGMASQ || op == SU2GPU_PHI2MINUSSIGMA2)) {
      do_muca = 1; fld = c->trip; bu = c->bu_trip; dofs = 3;
    }
  }
  int check = 0;
  if (do_muca) {
    copy_half(bu, fld, dofs, lo, hi);
    interval = (hi - lo) / c->w.checks_per_sweep;
    if (interval <= 0) interval = 1;
    accept = 0;
  }
  for (long i = lo; i < hi; i++) {
    orc_stream_at(&c->rng, (uint32_t)i, (uint32_t)c->pass);
    if (field == 0) {
      if (c->p.algorithm_su2doublet == SU2GPU_OVERRELAX && !metro) {
        c->cnt[SU2GPU_C_ACC_OR_DOUBLET + h] += site_update(c, 4, i, h);
        c->cnt[SU2GPU_C_TOTAL_OR_DOUBLET + h]++;
      } else if (c->p.algorithm_su2doublet == SU2GPU_METROPOLIS || metro) {
        c->cnt[SU2GPU_C_ACC_DOUBLET + h] += metro_doublet(c, i, h);
        c->cnt[SU2GPU_C_TOTAL_DOUBLET + h]++;
      }
    } else if (field == 1) {
      if (c->p.algorithm_su2triplet == SU2GPU_OVERRELAX && !metro) {
        c->cnt[SU2GPU_C_ACC_OR_TRIPLET] += overrelax_triplet(c, i);
        c->cnt[SU2GPU_C_TOTAL_OR_TRIPLET]++;
      } else if (c->p.algorithm_su2triplet == SU2GPU_METROPOLIS || metro) {
        c->cnt[SU2GPU_C_ACC_TRIPLET] += metro_triplet(c, i);
        c->cnt[SU2GPU_C_TOTAL_TRIPLET]++;
      }
    } else {
      if (c->p.algorithm_singlet == SU2GPU_OVERRELAX && !metro) {
        c->cnt[SU2GPU_C_ACC_OR_SINGLET] += overrelax_singlet(c, i);
        c->cnt[SU2GPU_C_TOTAL_OR_SINGLET]++;
      } else if (c->p.algorithm_singlet == SU2GPU_METROPOLIS || metro) {
        c->cnt[SU2GPU_C_ACC_SINGLET] += metro_singlet(c, i);
        c->cnt[SU2GPU_C_TOTAL_SINGLET]++;
      }
    }
    if (do_muca) {
      count++;
      if (count % interval == 0) {
        int make_backups = (i < hi - 1);
        int acc = muca_check(c, par, check++);
        accept += acc;
        if (!acc) copy_half(fld, bu, dofs, lo, hi);
        else if (make_backups) copy_half(bu, fld, dofs, lo, hi);
      }
    }
  }
  if (do_muca && (hi - lo) % c->w.checks_per_sweep != 0) {
    int acc = muca_check(c, par, check++);
    if (!acc) copy_half(fld, bu, dofs, lo, hi);
    accept += acc;
  }
  return accept;
}

/* The order stream of the random_sweeps mode: 64-bit draws, draw k is half
 * k & 1 of the Philox block (site 0xfffffffe, block k >> 1, sweep, chain). */
typedef struct {
  uint32_t key[2], sweep, chain, draw;
} orc_order_stream;

static uint64_t order_next(orc_order_stream* s) {
  uint32_t ctr[4] = {0xfffffffeu, (s->draw >> 1) & 0xffffu, s->sweep, s->chain}, out[4];
  orc_philox4x32_10(ctr, s->key, out);
  uint64_t v = (s->draw & 1) ? (((uint64_t)out[2] << 32) | out[3]) : (((uint64_t)out[0] << 32) | out[1]);
  s->draw++;
  return v;
}

/* shuffle (update.c:461-468): Fisher-Yates from the top, j = iran() % (i+1) */
static void shuffle_ints(orc_order_stream* s, int* a, int n) {
  for (int i = n - 1; i > 0; i--) {
    int j = (int)(order_next(s) % (uint64_t)(i + 1));
    int t = a[i]; a[i] = a[j]; a[j] = t;
  }
}

/* The pass order of update_lattice in random_sweeps mode (update.c:278-300,
 * 338-344): per link repetition the parity array [E,O,E,O,..] and the
 * direction array [0,0,1,1,..] shuffled independently, then per scalar sweep
 * the parity updated first (EVEN when dran() < 0.5). */
void orc_sweep_order(uint64_t seed, uint32_t chain, uint32_t sweep, int D, int update_links, int scalar_sweeps,
                     int* dirs, int* pars, int* first) {
  orc_order_stream s = {{(uint32_t)seed, (uint32_t)(seed >> 32)}, sweep, chain, 0};
  for (int k = 0; k < update_links; k++) {
    int* pa = pars + 2 * D * k;
    int* da = dirs + 2 * D * k;
    for (int j = 0; j < 2 * D; j++) { pa[j] = j % 2 ? ODD : EVEN; da[j] = j / 2; }
    shuffle_ints(&s, pa, 2 * D);
    shuffle_ints(&s, da, 2 * D);
  }
  for (int t = 0; t <= scalar_sweeps; t++) {
    double u = (double)(order_next(&s) >> 11) * (1.0 / 9007199254740992.0);
    first[t] = u < 0.5 ? EVEN : ODD;
  }
}

void orc_set_random_sweeps(orc_ctx* c, int on) { c->random_sweeps = on ? 1 : 0; }

/* update_lattice (update.c:270-430): the fixed order, or the random one */
int orc_update_lattice(orc_ctx* c) {
  const su2gpu_params* p = &c->p;
  int nl = p->update_links > 0 ? p->update_links : 0;
  int* dirs = (int*)malloc(sizeof(int) * (2 * c->D * nl + 1));
  int* pars = (int*)malloc(sizeof(int) * (2 * c->D * nl + 1));
  int* first = (int*)malloc(sizeof(int) * (p->scalar_sweeps + 1));
  if (c->random_sweeps) {
    orc_sweep_order(c->seed, c->chain, c->sweep, c->D, nl, p->scalar_sweeps, dirs, pars, first);
  } else {
    for (int k = 0; k < nl; k++)
      for (int j = 0; j < 2 * c->D; j++) {
        pars[2 * c->D * k + j] = j % 2 ? ODD : EVEN;
        dirs[2 * c->D * k + j] = j / 2;
      }
    for (int t = 0; t <= p->scalar_sweeps; t++) first[t] = EVEN;
  }
  c->pass = 0;
  for (int k = 0; k < nl; k++) {
    const int* pa = pars + 2 * c->D * k;
    const int* da = dirs + 2 * c->D * k;
    for (int j = 0; j < 2 * c->D; j++) { sweep_links(c, pa[j], da[j], p->algorithm_su2link); c->pass++; }
    if (c->has_u1)
      for (int j = 0; j < 2 * c->D; j++) { sweep_u1(c, pa[j], da[j]); c->pass++; }
  }
  int nsweeps = p->scalar_sweeps + 1;
  for (int s = 0; s < nsweeps; s++) {
    const int pr[2] = {first[s], first[s] == EVEN ? ODD : EVEN};
    if (c->nh > 0)
      for (int k = 0; k < p->update_su2doublet; k++) {
        int force = 0;
        if (s >= nsweeps - 1) {
          if (p->algorithm_su2doublet == SU2GPU_OVERRELAX) force = 1;
          else continue;
        }
        for (int h = 0; h < c->nh; h++)
          for (int j = 0; j <= 1; j++) { sweep_scalar(c, pr[j], force, 0, h); c->pass++; }
      }
    if (c->has_trip)
      for (int k = 0; k < p->update_su2triplet; k++) {
        int force = 0;
        if (s >= nsweeps - 1) {
          if (p->algorithm_su2triplet == SU2GPU_OVERRELAX) force = 1;
          else continue;
        }
        for (int j = 0; j <= 1; j++) { sweep_scalar(c, pr[j], force, 1, 0); c->pass++; }
      }
    if (c->has_sing)
      for (int k = 0; k < p->update_singlet; k++) {
        int force = 0;
        if (s >= nsweeps - 1) {
          if (p->algorithm_singlet == SU2GPU_OVERRELAX) force = 1;
          else continue;
        }
        for (int j = 0; j <= 1; j++) { sweep_scalar(c, pr[j], force, 2, 0); c->pass++; }
      }
  }
  free(dirs);
  free(pars);
  free(first);
  return c->pass;
}

/* ------------------------------------------------------------------ */
/* measure() sums (measure.c:71-243)                                   */
/* ------------------------------------------------------------------ */
/* measure_local (measure.c:368-487): per site in storage order, Tr Sigma^2
 * and magcharge_cube / (2 pi sqrt(beta)) */
void orc_measure_local(const orc_ctx* c, double* out) {
  for (long i = 0; i < c->V; i++) {
    out[2 * i] = c->has_trip ? tripletsq(TRP(c, i)) : 0.0;
    out[2 * i + 1] = c->has_trip ? orc_magcharge_cube(c, i) / (2.0 * M_PI * sqrt(c->p.betasu2)) : 0.0;
  }
}

/* init_z_coord + measure_along_z (z_coord.c:18-24, 206-300): the longest
 * direction (ties to the last), then per plane z the sums over its sites, in
 * storage order, of phi^2 (first doublet), Tr Sigma^2, S, S^2 */
void orc_measure_z(const orc_ctx* c, int* zdir_out, double* sums) {
  int zd = c->D - 1;
  for (int d = c->D - 1; d >= 0; d--)
    if (c->p.L[d] > c->p.L[zd]) zd = d;
  int Lz = c->p.L[zd];
  for (long k = 0; k < 4L * Lz; k++) sums[k] = 0.0;
  for (int z = 0; z < Lz; z++)
    for (long i = 0; i < c->V; i++) {
      if (c->coords[i * c->D + zd] != z) continue;
      double* m = sums + 4 * z;
      if (c->nh > 0) m[0] += doubletsq(PHI(c, 0, i));
      if (c->has_trip) m[1] += tripletsq(TRP(c, i));
      if (c->has_sing) {
        double sv = c->sing[i];
        m[2] += sv;
        m[3] += sv * sv;
      }
    }
  *zdir_out = zd;
}

void orc_measure(const orc_ctx* c, double* m) {
  for (int k = 0; k < SU2GPU_NMEAS; k++) m[k] = 0.0;
  for (long i = 0; i < c->V; i++) {
    m[SU2GPU_M_ACTION] += orc_action_local(c, i);
    m[SU2GPU_M_WILSON] = (double)((long double)m[SU2GPU_M_WILSON] + local_su2wilson_ld(c, i));
    if (c->has_u1) m[SU2GPU_M_U1WILSON] += orc_local_u1wilson(c, i);
    for (int h = 0; h < c->nh; h++) {
      double mod = doubletsq(PHI(c, h, i));
      m[SU2GPU_M_COV_PHI + 3 * h] += covariant_doublet(c, i, h);
      m[SU2GPU_M_PHI2 + 3 * h] += mod;
      m[SU2GPU_M_PHI4 + 3 * h] += mod * mod;
    }
    if (c->has_trip && c->nh > 0) m[SU2GPU_M_PHI2SIGMA2] += doubletsq(PHI(c, 0, i)) * tripletsq(TRP(c, i));
    if (c->nh == 2) {
      double R, I;
      phi12(PHI(c, 0, i), PHI(c, 1, i), &R, &I);
      m[SU2GPU_M_PHI12_RE] += R; m[SU2GPU_M_PHI12_IM] += I;
    }
    if (c->has_trip) {
      double tm = tripletsq(TRP(c, i));
      m[SU2GPU_M_SIGMA2] += tm;
      m[SU2GPU_M_SIGMA4] += tm * tm;
      for (int d = 0; d < c->D; d++) m[SU2GPU_M_HOP_SIGMA] += hop_triplet_fwd(c, i, d);
      double q = orc_magcharge_cube(c, i);
      m[SU2GPU_M_MAGCHARGE] += q;
      m[SU2GPU_M_MAGCHARGE_ABS] += fabs(q);
    }
    if (c->has_sing) {
      double S = c->sing[i];
      for (int d = 0; d < c->D; d++) m[SU2GPU_M_S_COV] += S * S - S * c->sing[NX(c, i, d)];
      m[SU2GPU_M_S1] += S;
      m[SU2GPU_M_S2] += S * S;
      m[SU2GPU_M_S3] += S * S * S;
      m[SU2GPU_M_S4] += S * S * S * S;
      if (c->nh == 1) {
        double mod = doubletsq(PHI(c, 0, i));
        m[SU2GPU_M_SPHI2] += mod * S;
        m[SU2GPU_M_S2PHI2] += mod * S * S;
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* gradient flow (gradflow.c)                                          */
/* ------------------------------------------------------------------ */
/* grad_force_link (gradflow.c:190-258) */
static void force_link(const orc_ctx* c, long i, int mu, double* force) {
  double s[4];
  orc_wilson_staple(c, i, mu, s);
  for (int a = 0; a < 4; a++) s[a] *= -c->p.betasu2 / (8.0);
  if (c->has_trip) {
    /* minus a quarter of Sigma(x+mu) U^+ Sigma(x) in quaternion form */
    const double* a1 = TRP(c, i);
    const double* a2 = TRP(c, NX(c, i, mu));
    double q1[4] = {0, a1[0], a1[1], a1[2]}, q2[4] = {0, a2[0], a2[1], a2[2]}, ud[4], t[4], r[4];
    qdag(LNK(c, i, mu), ud);
    qmul(q2, ud, t);
    qmul(t, q1, r);
    for (int k = 0; k < 4; k++) s[k] -= (-r[k]) / 4.0;
  }
  double m[4];
  qmul(LNK(c, i, mu), s, m);
  force[0] = 0.0;
  for (int a = 1; a < 4; a++) {
    force[a] = 2.0 * m[a];
    force[a] *= 4.0 / c->p.betasu2;
  }
}

/* grad_force_triplet (gradflow.c:267-330) */
static void force_triplet(const orc_ctx* c, long i, double* force) {
  double res[3] = {0, 0, 0}, r[3], ud[4];
  for (int d = 0; d < c->D; d++) {
    qrot(LNK(c, i, d), TRP(c, NX(c, i, d)), r);
    for (int k = 0; k < 3; k++) res[k] -= r[k];
    long xm = PV(c, i, d);
    qdag(LNK(c, xm, d), ud);
    qrot(ud, TRP(c, xm), r);
    for (int k = 0; k < 3; k++) res[k] -= r[k];
  }
  const double* t = TRP(c, i);
  for (int a = 0; a < 3; a++) {
    double ts = tripletsq(t);
    res[a] += (2.0 * c->D + c->p.msq_triplet + 2.0 * c->p.b4 * ts) * t[a];
    if (c->nh > 0) res[a] += c->p.a2 * doubletsq(PHI(c, 0, i)) * t[a];
  }
  for (int a = 0; a < 3; a++) force[a] = -1.0 * res[a];
}

void orc_flow_forces(const orc_ctx* c, double* link_force, double* trip_force) {
  for (long i = 0; i < c->V; i++) {
    for (int d = 0; d < c->D; d++) force_link(c, i, d, link_force + (i * c->D + d) * 4);
    if (c->has_trip && trip_force) force_triplet(c, i, trip_force + i * 3);
  }
}

/* flow_gauge (gradflow.c:361-401), including its early return: a link with
 * zero force stops the update of every later link of the step. */
static void flow_gauge(orc_ctx* c, const double* fl, double dt) {
  for (long i = 0; i < c->V; i++)
    for (int d = 0; d < c->D; d++) {
      const double* f = fl + (i * c->D + d) * 4;
      double z[3], mod = 0.0;
      for (int a = 0; a < 3; a++) { z[a] = dt * f[a + 1]; mod += z[a] * z[a]; }
      if (mod <= 0.0) return;
      mod = sqrt(mod);
      double u[4], r[4];
      u[0] = cos(mod);
      for (int a = 0; a < 3; a++) u[a + 1] = sin(mod) * z[a] / mod;
      qmul(u, LNK(c, i, d), r);
      memcpy(LNK(c, i, d), r, sizeof(r));
    }
}

void orc_flow_step(orc_ctx* c, double dt) {
  double* fl = (double*)malloc(sizeof(double) * c->V * c->D * 4);
  double* ft = c->has_trip ? (double*)malloc(sizeof(double) * c->V * 3) : NULL;
  orc_flow_forces(c, fl, ft);
  flow_gauge(c, fl, dt);
  if (c->has_trip)
    for (long i = 0; i < c->V; i++)
      for (int a = 0; a < 3; a++) c->trip[i * 3 + a] += dt * ft[i * 3 + a];
  free(fl);
  free(ft);
}

/* remove_counterterms (gradflow.c:424-459): tree-level triplet mass for the flow */
static double triplet_tree_mass(const su2gpu_params* p) {
  double Sigma = 3.17591153625, zeta = 0.08849, delta = 1.942130, rho = -0.313964;
  double k1 = 0.958382, k2 = 0.25 * Sigma * Sigma - 0.5 * delta - 0.25, k3 = 0.751498, k4 = 1.204295;
  double gsq = 4.0 / p->betasu2, RGscale = gsq, b4 = p->b4;
  double ct = -(4.0 * gsq + 5.0 * b4) * Sigma / (4.0 * M_PI);
  ct += -1.0 / (16.0 * M_PI * M_PI) *
        ((20.0 * b4 * gsq - 10.0 * b4 * b4) * (log(6.0 / (RGscale)) + zeta) + 20.0 * b4 * gsq * (0.25 * Sigma * Sigma - delta) +
         2.0 * gsq * gsq * (1.25 * Sigma * Sigma + M_PI / 3.0 * Sigma - 6.0 * delta - 6.0 * rho + 4.0 * k1 - k2 - k3 - 3.0 * k4));
  return p->msq_triplet - ct;
}

/* grad_flow (gradflow.c:46-173): rows of (t, measure sums) */
int orc_grad_flow(orc_ctx* c, double t_max, double dt, int meas_interval, double* rows, int maxrows, int* nrows) {
  long V = c->V; int D = c->D;
  /* flow a copy: save the current fields, restore them afterwards */
  double* save_link = (double*)malloc(sizeof(double) * V * D * 4);
  memcpy(save_link, c->link, sizeof(double) * V * D * 4);
  double* save_trip = NULL;
  if (c->has_trip) { save_trip = (double*)malloc(sizeof(double) * V * 3); memcpy(save_trip, c->trip, sizeof(double) * V * 3); }
  double msq = c->p.msq_triplet;
  if (c->has_trip) c->p.msq_triplet = triplet_tree_mass(&c->p);
  int nr = 0;
  const int W = 1 + SU2GPU_NMEAS;
  double t = 0.0;
  if (nr < maxrows) { rows[nr * W] = t; orc_measure(c, rows + nr * W + 1); nr++; }
  int iter = 1;
  while (t < t_max) {
    if (t + dt > t_max) dt = t_max - t;
    orc_flow_step(c, dt);
    t += dt;
    if (iter % meas_interval == 0) {
      if (nr < maxrows) { rows[nr * W] = t; orc_measure(c, rows + nr * W + 1); nr++; }
    }
    iter++;
  }
  if ((iter - 1) % meas_interval != 0) {
    if (nr < maxrows) { rows[nr * W] = t; orc_measure(c, rows + nr * W + 1); nr++; }
  }
  c->p.msq_triplet = msq;
  memcpy(c->link, save_link, sizeof(double) * V * D * 4);
  free(save_link);
  if (save_trip) { memcpy(c->trip, save_trip, sizeof(double) * V * 3); free(save_trip); }
  *nrows = nr;
  return nr;
}

/* ------------------------------------------------------------------ */
/* correlators and blocking (correlation.c, blocking.c, su2u1.c)       */
/* ------------------------------------------------------------------ */

/* su2plaquette + the three other plaquettes of clover_su2 (su2u1.c:119-136,
 * 207-274): the clover of the (d1, d2) plane at site i */
static void clover(const orc_ctx* c, long i, int d1, int d2, double* cl) {
  double a[4], b[4], t[4], s[4], u[4];
  /* U_1(x) U_2(x+1) U_1(x+2)^+ U_2(x)^+ */
  qdag(LNK(c, NX(c, i, d2), d1), a);
  qdag(LNK(c, i, d2), b);
  qmul(a, b, t);
  qmul(LNK(c, NX(c, i, d1), d2), t, s);
  qmul(LNK(c, i, d1), s, cl);
  /* U_2(x) U_1(x+2-1)^+ U_2(x-1)^+ U_1(x-1) */
  long xm1 = PV(c, i, d1), x21 = PV(c, NX(c, i, d2), d1);
  qdag(LNK(c, xm1, d2), a);
  qmul(a, LNK(c, xm1, d1), t);
  qdag(LNK(c, x21, d1), b);
  qmul(b, t, s);
  qmul(LNK(c, i, d2), s, u);
  for (int k = 0; k < 4; k++) cl[k] += u[k];
  /* U_1(x-1)^+ U_2(x-2-1)^+ U_1(x-1-2) U_2(x-2) */
  long xm12 = PV(c, xm1, d2), xm2 = PV(c, i, d2);
  qmul(LNK(c, xm12, d1), LNK(c, xm2, d2), t);
  qdag(LNK(c, xm12, d2), a);
  qmul(a, t, s);
  qdag(LNK(c, xm1, d1), b);
  qmul(b, s, u);
  for (int k = 0; k < 4; k++) cl[k] += u[k];
  /* U_2(x-2)^+ U_1(x-2) U_2(x+1-2) U_1(x)^+ */
  long x12 = NX(c, xm2, d1);
  qdag(LNK(c, i, d1), a);
  qmul(LNK(c, x12, d2), a, t);
  qmul(LNK(c, xm2, d1), t, s);
  qdag(LNK(c, xm2, d2), b);
  qmul(b, s, u);
  for (int k = 0; k < 4; k++) cl[k] += u[k];
}

/* site phase 2 pi p.x of photon_correl's momentum (correlation.c:140-146,
 * 226-231): only the components of mom that are non-zero */
static double phase_px(const orc_ctx* c, long i, const int* mom) {
  double px = 0.0;
  for (int d = 0; d < c->D; d++)
    if (mom[d] != 0) px += (double)(mom[d] * c->coords[i * c->D + d]) / (double)c->p.L[d];
  return px;
}

/* the plane operators at x_dir = z, summed over the plane's sites in storage
 * order (sites_at_coord, layout.c:798-816): h, s (plane_sum of doubletsq /
 * tripletsq, correlation.c:16-33), and per (transmom, mode) one complex
 * number: mode 0 projected_photon_operator (correlation.c:99-164), mode 1
 * photon_projection_full (correlation.c:207-253) */
static void plane_ops(const orc_ctx* c, int dir, long z, double* h, double* s, double op[4][2]) {
  int d1 = dir == 0 ? 1 : 0, d2 = dir == 2 ? 1 : 2;
  *h = 0.0; *s = 0.0;
  for (int k = 0; k < 4; k++) op[k][0] = op[k][1] = 0.0;
  for (int k = 0; c->has_trip && k < 4; k++) {
    int tm = (k & 1) ? 2 : 1, mode = k >> 1;
    /* photon_correl (correlation.c:270-274): the loop over dir0 stops after
     * dir0 = 0, so the momentum is (tm, 0, 0) when dir != 0, else zero */
    int mom[4] = {0, 0, 0, 0};
    if (dir != 0) mom[0] = tm;
    for (long i = 0; i < c->V; i++) {
      if (c->coords[i * c->D + dir] != z) continue;
      double px = phase_px(c, i, mom), val;
      if (mode == 0) {
        double cl[4];
        clover(c, i, d1, d2, cl);
        cl[0] = 0.0;
        for (int q = 1; q < 4; q++) cl[q] /= 4.0;
        const double* a = TRP(c, i);
        val = a[0] * cl[1] + a[1] * cl[2] + a[2] * cl[3];
      } else {
        double alpha = 0.0;
        for (int e1 = 0; e1 < c->D; e1++)
          for (int e2 = e1 + 1; e2 < c->D; e2++)
            if (e1 != dir && e2 != dir) alpha += orc_alpha_proj(c, i, e1, e2);
        val = 2.0 * alpha;
      }
      op[k][0] += val * cos(2.0 * M_PI * px);
      op[k][1] += val * sin(2.0 * M_PI * px);
    }
  }
  for (long i = 0; i < c->V; i++) {
    if (c->coords[i * c->D + dir] != z) continue;
    if (c->nh > 0) *h += doubletsq(PHI(c, 0, i));
    if (c->has_trip) *s += tripletsq(TRP(c, i));
  }
}

/* measure_correlators (correlation.c:350-398) before formatting: per
 * distance d < L[dir]/2 ten values -- higgs_correlator (correlation.c:39-58),
 * triplet_correlator (65-83), photon_correl for (transmom, mode) = (1,0),
 * (2,0), (1,1), (2,1) re/im (257-315); absent fields give 0 */
int orc_correlators(const orc_ctx* c, int dir, double* out) {
  long Lz = c->p.L[dir];
  double* h = (double*)calloc(Lz, sizeof(double));
  double* s = (double*)calloc(Lz, sizeof(double));
  double (*op)[4][2] = calloc(Lz, sizeof(*op));
  for (long z = 0; z < Lz; z++) plane_ops(c, dir, z, &h[z], &s[z], op[z]);
  int maxd = (int)(Lz / 2);
  for (int d = 0; d < maxd; d++) {
    double* r = out + 10 * d;
    double hc = 0.0, sc = 0.0, pre[4] = {0, 0, 0, 0}, pim[4] = {0, 0, 0, 0};
    for (long z = 0; z < Lz; z++) {
      long zd = (z + d) % Lz;
      hc += h[z] * h[zd];
      sc += s[z] * s[zd];
      for (int k = 0; k < 4; k++) {
        /* O1 . O2^* through cmult (stddefs.h:93-98) */
        double ar = op[z][k][0], ai = op[z][k][1], br = op[zd][k][0], bi = -op[zd][k][1];
        pre[k] += ar * br - ai * bi;
        pim[k] += br * ai + ar * bi;
      }
    }
    r[0] = c->nh > 0 ? 4.0 * hc / (double)c->V : 0.0;
    r[1] = c->has_trip ? sc / (double)c->V : 0.0;
    for (int k = 0; k < 4; k++) {
      r[2 + 2 * k] = c->has_trip ? pre[k] / (double)c->V : 0.0;
      r[3 + 2 * k] = c->has_trip ? pim[k] / (double)c->V : 0.0;
    }
  }
  free(h); free(s); free(op);
  return maxd;
}

/* su2staple_wilson_onedir with dagger = 1 (staples.c:197-232): the two
 * staples of U_mu(x) in the (mu, nu) plane, each conjugated:
 *   U_nu(x) U_mu(x+nu) U_nu(x+mu)^+  +  U_nu(x-nu)^+ U_mu(x-nu) U_nu(x+mu-nu) */
static void staple_onedir_dag(const orc_ctx* c, long i, int mu, int nu, double* res) {
  double a[4], t[4], s[4];
  long xp = NX(c, i, mu), xn = NX(c, i, nu), xm = PV(c, i, nu), xpm = PV(c, xp, nu);
  qdag(LNK(c, xp, nu), a);
  qmul(LNK(c, xn, mu), a, t);
  qmul(LNK(c, i, nu), t, res);
  qmul(LNK(c, xm, mu), LNK(c, xpm, nu), t);
  qdag(LNK(c, xm, nu), a);
  qmul(a, t, s);
  for (int k = 0; k < 4; k++) res[k] += s[k];
}

/* smear_link (su2u1.c:752-795): V_dir(x) V_dir(x+dir) normalised, with
 * V_dir(y) = (U_dir(y) + sum over smeared j != dir of both staples) / paths */
static void smear_link(const orc_ctx* c, const int* sdir, long i, int dir, double* res) {
  double r[4], v2[4], st[4];
  long xp = NX(c, i, dir);
  memcpy(r, LNK(c, i, dir), sizeof(r));
  memcpy(v2, LNK(c, xp, dir), sizeof(v2));
  int paths = 1;
  for (int j = 0; j < c->D; j++) {
    if (j == dir || !sdir[j]) continue;
    staple_onedir_dag(c, i, dir, j, st);
    for (int k = 0; k < 4; k++) r[k] += st[k];
    staple_onedir_dag(c, xp, dir, j, st);
    for (int k = 0; k < 4; k++) v2[k] += st[k];
    paths += 2;
  }
  for (int k = 0; k < 4; k++) { r[k] /= (double)paths; v2[k] /= (double)paths; }
  qmul(r, v2, res);
  double det = sqrt(qsq(res));
  for (int k = 0; k < 4; k++) res[k] /= det;
}

/* smear_triplet (su2u1.c:805-852): (Sigma(x) + sum over smeared j of
 * U_j(x) Sigma(x+j) U_j(x)^+ + U_j(x-j)^+ Sigma(x-j) U_j(x-j)) / sites */
static void smear_triplet(const orc_ctx* c, const int* sdir, long i, double* res) {
  double cov[3] = {0, 0, 0}, r[3], ud[4];
  int sites = 1;
  for (int d = 0; d < c->D; d++) {
    if (!sdir[d]) continue;
    qrot(LNK(c, i, d), TRP(c, NX(c, i, d)), r);
    for (int k = 0; k < 3; k++) cov[k] += r[k];
    long xm = PV(c, i, d);
    qdag(LNK(c, xm, d), ud);
    qrot(ud, TRP(c, xm), r);
    for (int k = 0; k < 3; k++) cov[k] += r[k];
    sites += 2;
  }
  for (int k = 0; k < 3; k++) res[k] = (TRP(c, i)[k] + cov[k]) / (double)sites;
}

/* smear_fields + make_blocked_fields (su2u1.c:857-905, blocking.c:296-374):
 * the site of dst with coordinates y takes the smeared fields of the src
 * site with x_d = 2 y_d in the blocked directions, x_d = y_d elsewhere; links
 * in unblocked directions are copied, the triplet is smeared over the
 * blocked directions.  dst has the blocked sides. */
int orc_block(const orc_ctx* src, const int* block_dir, orc_ctx* dst) {
  int D = src->D;
  for (int d = 0; d < D; d++)
    if (dst->p.L[d] != (block_dir[d] ? src->p.L[d] / 2 : src->p.L[d])) return -1;
  long* lex = (long*)malloc(sizeof(long) * src->V);
  for (long i = 0; i < src->V; i++) {
    long n = 0, st = 1;
    for (int d = 0; d < D; d++) { n += src->coords[i * D + d] * st; st *= src->p.L[d]; }
    lex[n] = i;
  }
  for (long j = 0; j < dst->V; j++) {
    long n = 0, st = 1;
    for (int d = 0; d < D; d++) {
      long x = dst->coords[j * D + d] * (block_dir[d] ? 2 : 1);
      n += x * st;
      st *= src->p.L[d];
    }
    long i = lex[n];
    for (int d = 0; d < D; d++) {
      if (block_dir[d]) smear_link(src, block_dir, i, d, LNK(dst, j, d));
      else memcpy(LNK(dst, j, d), LNK(src, i, d), 4 * sizeof(double));
      if (src->has_u1 && dst->has_u1 && !block_dir[d]) dst->u1[j * D + d] = src->u1[i * D + d];
    }
    if (src->has_trip && dst->has_trip) smear_triplet(src, block_dir, i, TRP(dst, j));
  }
  free(lex);
  return 0;
}

/* ------------------------------------------------------------------ */
/* random stream probes (tests)                                        */
/* ------------------------------------------------------------------ */
void orc_philox_raw(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { orc_philox4x32_10(ctr, key, out); }

double orc_stream_uniform_at(uint64_t seed, uint32_t site, uint32_t pass, uint32_t draw, uint32_t sweep,
                             uint32_t chain) {
  orc_stream s;
  orc_stream_init(&s, seed, sweep, chain);
  orc_stream_at(&s, site, pass);
  double u = 0.0;
  for (uint32_t k = 0; k <= draw; k++) u = orc_stream_uniform(&s);
  return u;
}
