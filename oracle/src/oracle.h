/* oracle.h -- TEST INFRASTRUCTURE (oracle). Not part of the product.
 *
 * CPU restatement of su2higgs's checkerboard update sweep, used only as the
 * checker of the CUDA path (tests, smoke check) and as the timed CPU
 * baseline.  Pinned against the reference itself through the harness in
 * oracle/ref (golden fixtures under tests/golden).
 *
 * Field arrays are FP64 AoS in the reference's layout order (EVEN sites
 * first), the same as the C ABI's host arrays (include/su2gpu.h).
 */
#ifndef ORACLE_H
#define ORACLE_H

#include <stdint.h>
#include "../../include/su2gpu.h"

typedef struct orc_ctx orc_ctx;

orc_ctx* orc_create(const su2gpu_params* p);
void orc_destroy(orc_ctx* c);
long orc_sites(const orc_ctx* c);
void orc_tables(const orc_ctx* c, int64_t* next, int64_t* prev, int64_t* coords, int32_t* parity);
void orc_put_fields(orc_ctx* c, const double* link, const double* u1, const double* d0, const double* d1,
                    const double* trip, const double* sing);
void orc_get_fields(const orc_ctx* c, double* link, double* u1, double* d0, double* d1, double* trip,
                    double* sing);
void orc_set_rng(orc_ctx* c, uint64_t seed, uint32_t sweep, uint32_t chain);
int orc_update_lattice(orc_ctx* c);
void orc_set_random_sweeps(orc_ctx* c, int on);
void orc_sweep_order(uint64_t seed, uint32_t chain, uint32_t sweep, int D, int update_links, int scalar_sweeps,
                     int* dirs, int* pars, int* first);
void orc_counters(const orc_ctx* c, int64_t* out);
void orc_reset_counters(orc_ctx* c);
void orc_measure(const orc_ctx* c, double* sums);
void orc_measure_local(const orc_ctx* c, double* out);
void orc_measure_z(const orc_ctx* c, int* zdir, double* sums);
int orc_correlators(const orc_ctx* c, int dir, double* out);
int orc_block(const orc_ctx* src, const int* block_dir, orc_ctx* dst);

/* per-site kernels */
void orc_wilson_staple(const orc_ctx* c, long i, int dir, double* V);
void orc_link_staple(const orc_ctx* c, long i, int dir, double* V);
double orc_localact_su2link(const orc_ctx* c, long i, int dir);
double orc_local_su2wilson(const orc_ctx* c, long i);
double orc_action_local(const orc_ctx* c, long i);
double orc_localact_u1link(const orc_ctx* c, long i, int dir);
double orc_local_u1wilson(const orc_ctx* c, long i);
void orc_staple_doublet(const orc_ctx* c, long i, int hid, double* s);
double orc_localact_doublet(const orc_ctx* c, long i, int hid);
double orc_localact_triplet(const orc_ctx* c, long i);
double orc_localact_singlet(const orc_ctx* c, long i);
double orc_alpha_proj(const orc_ctx* c, long i, int d1, int d2);
double orc_magcharge_cube(const orc_ctx* c, long i);
double orc_polysolve3(double a, double b, double cc, double d);
int orc_site_update(orc_ctx* c, int kind, long i, int sub, uint32_t pass);
int orc_site_draws(const orc_ctx* c);
int orc_or_proposal(orc_ctx* c, int kind, long i, int sub, double* out);

/* multicanonical */
int orc_muca_set(orc_ctx* c, const su2gpu_weight* w);
int orc_muca_get(const orc_ctx* c, su2gpu_weight* w);
double orc_calc_orderparam(orc_ctx* c, int par);
double orc_get_weight(const orc_ctx* c, double v);
int orc_whichbin(const orc_ctx* c, double v);
void orc_muca_init_last_max(orc_ctx* c);

/* gradient flow */
void orc_flow_forces(const orc_ctx* c, double* link_force, double* trip_force);
void orc_flow_step(orc_ctx* c, double dt);
int orc_grad_flow(orc_ctx* c, double t_max, double dt, int meas_interval, double* rows, int maxrows,
                  int* nrows);

#endif
