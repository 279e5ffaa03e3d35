/* su2gpu.h -- C ABI of libsu2gpu, the GB300 (sm_103a) implementation of the
 * su2higgs checkerboard lattice update sweep.
 *
 * Every entry point returns an int status (SU2GPU_OK = 0, negative on error)
 * instead of exiting, and takes plain pointers and sizes.  Field arrays on
 * the host side are FP64, array-of-structures, in the reference's layout site
 * order (EVEN sites first, each parity in lexicographic order with x fastest):
 * exactly the field blocks of the reference's binary lattice file
 * (src/checkpoint.c:101-115 of su2higgs).  On the device the context keeps
 * them resident as parity-split structure-of-arrays (FP64, or FP32 in the
 * precision form).
 *
 * Reference entry points replaced (su2higgs, src/):
 *   update_lattice()           update.c:270      -> su2gpu_update_lattice
 *   measure() volume sums      measure.c:71-243  -> su2gpu_measure
 *   grad_flow()                gradflow.c:46     -> su2gpu_grad_flow
 *   calc_orderparam()          multicanonical.c:709 -> su2gpu_calc_orderparam
 *   init_last_max()            multicanonical.c:826 -> su2gpu_muca_init_last_max
 *   load_lattice()/setfields() field upload      -> su2gpu_upload_fields
 *   save_lattice() field download                -> su2gpu_download_fields
 *   measure_correlators()      correlation.c:350 -> su2gpu_measure_correlators
 *   measure_blocked_correlators() correlation.c:404 -> su2gpu_measure_blocked_correlators
 */
#ifndef SU2GPU_H
#define SU2GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SU2GPU_OK 0
#define SU2GPU_ERR_INVALID (-1)     /* bad argument / unsupported configuration */
#define SU2GPU_ERR_CUDA (-2)        /* CUDA runtime error */
#define SU2GPU_ERR_NOMEM (-3)       /* device allocation failed */
#define SU2GPU_ERR_UNSUPPORTED (-4) /* valid for the reference, not implemented on the GPU */
#define SU2GPU_ERR_KERNEL (-5)      /* a kernel flagged an error (loop cap, bad state) */
#define SU2GPU_ERR_CAPACITY (-6)    /* request does not fit (serving admission) */

/* ---- field content bits (the reference's compile-time -D flags, Makefile:3-16) ---- */
#define SU2GPU_HIGGS1 0x01   /* -DNHIGGS=1 */
#define SU2GPU_HIGGS2 0x02   /* -DNHIGGS=2 */
#define SU2GPU_TRIPLET 0x04  /* -DTRIPLET */
#define SU2GPU_SINGLET 0x08  /* -DSINGLET */
#define SU2GPU_U1 0x10       /* -DU1 */
#define SU2GPU_GRADFLOW 0x20 /* -DGRADFLOW */

/* ---- update algorithms (generic/stddefs.h:47-49) ---- */
#define SU2GPU_METROPOLIS 1
#define SU2GPU_HEATBATH 2
#define SU2GPU_OVERRELAX 3

/* ---- multicanonical order parameters and modes (stddefs.h:57-65) ---- */
#define SU2GPU_PHISQ 1
#define SU2GPU_SIGMASQ 2
#define SU2GPU_PHI2MINUSSIGMA2 3
#define SU2GPU_PHI2SQ 4
#define SU2GPU_MUCA_READONLY 0
#define SU2GPU_MUCA_FAST 1
#define SU2GPU_MUCA_SLOW 2

/* Simulation parameters: the action couplings and update recipe of the
 * reference's params struct (su2.h:76-181), plus the field content and the
 * device precision.  Field names follow the reference. */
typedef struct {
  int32_t dim;                 /* only 3 is supported on the GPU */
  int32_t L[4];
  int32_t content;             /* SU2GPU_* content bits */
  int32_t precision;           /* 64 (plain FP64 path) or 32 (FP32 fields, FP64 reductions) */
  int32_t algorithm_su2link;   /* HEATBATH or METROPOLIS */
  int32_t algorithm_u1link;    /* METROPOLIS */
  int32_t algorithm_su2doublet;/* OVERRELAX or METROPOLIS */
  int32_t algorithm_su2triplet;/* OVERRELAX or METROPOLIS */
  int32_t algorithm_singlet;   /* OVERRELAX or METROPOLIS */
  int32_t update_links;
  int32_t scalar_sweeps;
  int32_t update_su2doublet;
  int32_t update_su2triplet;
  int32_t update_singlet;
  int32_t reunitarize_interval;/* FP32 form: renormalise links every n sweeps (0 = never) */
  int32_t reserved[2];         /* keeps the doubles 8-byte aligned without padding */
  double betasu2;
  double msq_phi, lambda_phi;            /* doublet */
  double msq_triplet, a2, b4;            /* triplet */
  double betau1, r_u1;                   /* U(1) */
  double b1_s, msq_s, b3_s, b4_s, a1_s, a2_s; /* singlet */
  double msq_phi2, m12sq_re, m12sq_im;   /* second doublet (NHIGGS == 2) */
  double lam2, lam3, lam4, lam5_re, lam5_im, lam6_re, lam6_im, lam7_re, lam7_im;
} su2gpu_params;

/* Accept/reject counters (su2.h:208-231), int64 each. */
enum {
  SU2GPU_C_TOTAL_SU2LINK = 0, SU2GPU_C_ACC_SU2LINK = 1,
  SU2GPU_C_TOTAL_U1LINK = 2, SU2GPU_C_ACC_U1LINK = 3,
  SU2GPU_C_TOTAL_DOUBLET = 4,      /* +higgs_id (2 entries) */
  SU2GPU_C_ACC_DOUBLET = 6,        /* +higgs_id */
  SU2GPU_C_TOTAL_OR_DOUBLET = 8,   /* +higgs_id */
  SU2GPU_C_ACC_OR_DOUBLET = 10,    /* +higgs_id */
  SU2GPU_C_TOTAL_TRIPLET = 12, SU2GPU_C_ACC_TRIPLET = 13,
  SU2GPU_C_TOTAL_OR_TRIPLET = 14, SU2GPU_C_ACC_OR_TRIPLET = 15,
  SU2GPU_C_TOTAL_SINGLET = 16, SU2GPU_C_ACC_SINGLET = 17,
  SU2GPU_C_TOTAL_OR_SINGLET = 18, SU2GPU_C_ACC_OR_SINGLET = 19,
  SU2GPU_C_TOTAL_MUCA = 20, SU2GPU_C_ACC_MUCA = 21,
  SU2GPU_C_KP_CAP = 22,            /* heatbath loop-cap fallbacks (heatbath.c:64-68) */
  SU2GPU_C_POLY_FALLBACK = 23,     /* polysolve3 multi-root fallbacks (overrelax.c:26-32) */
  SU2GPU_NCOUNTERS = 24
};

/* Volume sums of measure() (measure.c:110-233), before the division by the
 * volume that the row writer applies; mag_charge_abs is before the division
 * by 2*pi*sqrt(beta). */
enum {
  SU2GPU_M_ACTION = 0, SU2GPU_M_WILSON = 1, SU2GPU_M_U1WILSON = 2,
  SU2GPU_M_COV_PHI = 3,   /* +3*higgs_id: covariant, phi2, phi4 */
  SU2GPU_M_PHI2 = 4, SU2GPU_M_PHI4 = 5,
  SU2GPU_M_PHI12_RE = 9, SU2GPU_M_PHI12_IM = 10,
  SU2GPU_M_HOP_SIGMA = 11, SU2GPU_M_SIGMA2 = 12, SU2GPU_M_SIGMA4 = 13, SU2GPU_M_PHI2SIGMA2 = 14,
  SU2GPU_M_MAGCHARGE = 15, SU2GPU_M_MAGCHARGE_ABS = 16,
  SU2GPU_M_S_COV = 17, SU2GPU_M_S1 = 18, SU2GPU_M_S2 = 19, SU2GPU_M_S3 = 20, SU2GPU_M_S4 = 21,
  SU2GPU_M_SPHI2 = 22, SU2GPU_M_S2PHI2 = 23,
  SU2GPU_NMEAS = 24
};

/* Multicanonical weight (su2.h:235-274).  Arrays are host memory with
 * bins+2 entries (the two virtual bins included). */
typedef struct {
  int32_t orderparam;
  int32_t mode;
  int32_t do_acceptance;
  int32_t checks_per_sweep;
  int32_t bins;
  int32_t muca_count;
  int32_t update_interval;
  int32_t last_max;
  double param_value[2];
  double min, max, wrk_min, wrk_max, delta;
  double* pos;
  double* W;
  double* slope;
  double* b;
  int32_t* hits;
  int64_t* gsum;   /* SLOW mode only */
  int64_t* nsum;   /* SLOW mode only */
  double* hgram;   /* SLOW mode only */
} su2gpu_weight;

typedef struct su2gpu_ctx su2gpu_ctx;

/* Library / device information. */
int su2gpu_version(void);
int su2gpu_device_info(int* sm_count, int* cc_major, int* cc_minor, int64_t* free_bytes);

/* Create a device-resident lattice for one chain.  Fields start cold
 * (links = 1, scalars 0) until uploaded.  Replaces layout()/alloc_fields()
 * (layout.c:657-704 serial, alloc.c:103). */
int su2gpu_create(const su2gpu_params* p, su2gpu_ctx** out);
int su2gpu_destroy(su2gpu_ctx* ctx);
/* Bytes of device memory a context with these parameters needs. */
int64_t su2gpu_footprint_bytes(const su2gpu_params* p);

/* Neighbour / coordinate / parity tables of the layout (layout.c:657-756,
 * 826-922): next, prev, coords are [V*dim] int64, parity [V] int32.
 * Computed on the device from the closed form of the reference's EVEN-first
 * order and copied back. */
int su2gpu_layout_tables(su2gpu_ctx* ctx, int64_t* next, int64_t* prev, int64_t* coords, int32_t* parity);

/* Per-site values of the deterministic parts of the sweep on the context's
 * current fields (plain FP64 contexts only), computed by the same device
 * functions the update kernels call, for checking them site by site against
 * the reference; the fields are left unchanged.  `out` holds V rows in layout
 * order, of the width given for each `what`:
 *   SU2GPU_SITE_LINK_STAPLE      [3][4] su2link_staple, staples.c:134-193
 *   SU2GPU_SITE_WILSON_STAPLE    [3][4] su2staple_wilson, staples.c:84-115
 *   SU2GPU_SITE_LOCALACT_SU2LINK [3]    localact_su2link, su2u1.c:166-198
 *   SU2GPU_SITE_LOCALACT_U1LINK  [3]    localact_u1link, su2u1.c:336-354
 *   SU2GPU_SITE_STAPLE_DOUBLET   [4]    staple_doublet (doublet 0), staples.c:243-302
 *   SU2GPU_SITE_LOCALACT_DOUBLET [1]    localact_doublet (doublet 0), su2u1.c:495-510
 *   SU2GPU_SITE_LOCALACT_SINGLET [1]    localact_singlet, su2u1.c:688-705
 *   SU2GPU_SITE_OR_DOUBLET       [4]    the overrelaxation proposal of doublet 0
 *                                       (the value an accepted overrelax_doublet,
 *                                       overrelax.c:54-128, or overrelax_higgs2,
 *                                       295-417, writes)
 *   SU2GPU_SITE_OR_DOUBLET1      [4]    the same for doublet 1 (two doublets)
 *   SU2GPU_SITE_OR_TRIPLET       [3]    overrelax_triplet's, overrelax.c:137-236
 *   SU2GPU_SITE_OR_SINGLET       [1]    overrelax_singlet's, overrelax.c:243-285
 * SU2GPU_ERR_INVALID for a field the content lacks, SU2GPU_ERR_UNSUPPORTED
 * for an FP32 context. */
#define SU2GPU_SITE_LINK_STAPLE 1
#define SU2GPU_SITE_WILSON_STAPLE 2
#define SU2GPU_SITE_LOCALACT_SU2LINK 3
#define SU2GPU_SITE_LOCALACT_U1LINK 4
#define SU2GPU_SITE_STAPLE_DOUBLET 5
#define SU2GPU_SITE_LOCALACT_DOUBLET 6
#define SU2GPU_SITE_LOCALACT_SINGLET 7
#define SU2GPU_SITE_OR_DOUBLET 8
#define SU2GPU_SITE_OR_DOUBLET1 9
#define SU2GPU_SITE_OR_TRIPLET 10
#define SU2GPU_SITE_OR_SINGLET 11
int su2gpu_site_values(su2gpu_ctx* ctx, int32_t what, double* out);

/* Field transfer (FP64 AoS host arrays in layout order; NULL for absent
 * fields).  link: V*dim*4, u1: V*dim, doublet: V*4, triplet: V*3, singlet: V.
 * Page-locked arrays (su2gpu_host_register) are converted by the device in
 * place, without a staging copy. */
int su2gpu_upload_fields(su2gpu_ctx* ctx, const double* link, const double* u1, const double* doublet0,
                         const double* doublet1, const double* triplet, const double* singlet);
int su2gpu_download_fields(su2gpu_ctx* ctx, double* link, double* u1, double* doublet0,
                           double* doublet1, double* triplet, double* singlet);

/* Random stream: Philox4x32-10, key = seed, counter = (site, pass<<16|block,
 * sweep, chain). */
int su2gpu_set_seed(su2gpu_ctx* ctx, uint64_t seed, uint32_t chain);

/* One full sweep, update.c:270-430 order; `sweep` is the counter word of the
 * random stream for this call.  Counters accumulate on the device. */
int su2gpu_update_lattice(su2gpu_ctx* ctx, uint32_t sweep);
/* n sweeps back to back (sweep, sweep+1, ...), optionally through a captured
 * CUDA graph of one sweep. */
int su2gpu_run_sweeps(su2gpu_ctx* ctx, uint32_t first_sweep, int32_t nsweeps, int32_t use_graph);
int su2gpu_get_counters(su2gpu_ctx* ctx, int64_t* counters /* SU2GPU_NCOUNTERS */);
/* One half-sweep, the body of one checkerboard_sweep_*() call (update.c:35-259)
 * without multicanonical checks, for tests and diagnostics.  kind: 0 SU(2)
 * links (algorithm_su2link), 1 U(1) links, 2 doublet, 3 doublet forced
 * Metropolis, 4 triplet, 5 triplet forced Metropolis, 6 singlet, 7 singlet
 * forced Metropolis; sub = direction or doublet index; pass and sweep select
 * the random stream. */
int su2gpu_run_halfsweep(su2gpu_ctx* ctx, int32_t kind, int32_t parity, int32_t sub, uint32_t pass, uint32_t sweep);
int su2gpu_reset_counters(su2gpu_ctx* ctx);

/* measure() volume sums (SU2GPU_NMEAS doubles, FP64 accumulation). */
int su2gpu_measure(su2gpu_ctx* ctx, double* sums);

/* Multicanonical weight: copy host weight state to the device / back. */
int su2gpu_muca_set(su2gpu_ctx* ctx, const su2gpu_weight* w);
int su2gpu_muca_get(su2gpu_ctx* ctx, su2gpu_weight* w);
/* calc_orderparam(par) (multicanonical.c:709): recompute the parity
 * contribution on the device, store it, return the total in *value. */
int su2gpu_calc_orderparam(su2gpu_ctx* ctx, int32_t parity, double* value);
int su2gpu_muca_init_last_max(su2gpu_ctx* ctx);

/* grad_flow() (gradflow.c:46-173) on a device copy of the fields: Euler
 * Wilson flow of the SU(2) links (and triplet), measuring every meas_interval
 * steps.  rows[k*(1+SU2GPU_NMEAS)] = flow time, followed by the sums.
 * Returns the number of rows in *nrows (at most maxrows). */
int su2gpu_grad_flow(su2gpu_ctx* ctx, double t_max, double dt, int32_t meas_interval,
                     double* rows, int32_t maxrows, int32_t* nrows);
/* measure_local (measure.c:368-487): per site, in storage order, Tr Sigma^2
 * and the magnetic charge in units of 2 pi sqrt(beta) (magcharge_cube,
 * magfield.c:262-280): out[2 i], out[2 i + 1] for site i, V x 2 doubles.
 * Triplet content only (the reference writes no values without it). */
int su2gpu_measure_local(su2gpu_ctx* ctx, double* out);
/* measure_along_z (z_coord.c:206-300): profiles along the "z direction", the
 * longest direction with ties going to the last one (init_z_coord,
 * z_coord.c:18-24), returned in *z_dir.  sums[4 z + q] for 0 <= z < L[z_dir]
 * is the sum over the plane z of q = 0 phi^2 (first doublet), 1 Tr Sigma^2,
 * 2 S, 3 S^2; columns of fields the content lacks are 0.  The reference's
 * rows are these sums divided by the plane's area V / L[z_dir]. */
int su2gpu_measure_z(su2gpu_ctx* ctx, int32_t* z_dir, double* sums);
/* Columns of the correlators (measure_correlators, correlation.c:350-398),
 * per distance d: the Higgs correlator H(d) = 4 sum_z h(z) h(z+d) / V with h
 * the plane sum of |phi|^2 / 2 (first doublet; higgs_correlator, 39-58), the
 * Sigma^2 correlator (triplet_correlator, 65-83) and photon_correl (257-315)
 * re/im for (transmom, mode) = (1,0), (2,0), (1,1), (2,1); absent fields 0. */
enum {
  SU2GPU_CORR_HIGGS = 0, SU2GPU_CORR_SIGMA2 = 1,
  SU2GPU_CORR_PHOT10_RE = 2, SU2GPU_CORR_PHOT10_IM = 3, SU2GPU_CORR_PHOT20_RE = 4, SU2GPU_CORR_PHOT20_IM = 5,
  SU2GPU_CORR_PHOT11_RE = 6, SU2GPU_CORR_PHOT11_IM = 7, SU2GPU_CORR_PHOT21_RE = 8, SU2GPU_CORR_PHOT21_IM = 9,
  SU2GPU_NCORR = 10
};
/* measure_correlators (correlation.c:350-398) along direction dir:
 * out[d * SU2GPU_NCORR + col] for 0 <= d < L[dir] / 2.  The reference
 * measures along the longest direction (make_misc_tables, layout.c:773-777,
 * ties to the last). */
int su2gpu_measure_correlators(su2gpu_ctx* ctx, int32_t dir, double* out);
/* measure_blocked_correlators (correlation.c:404-432) for blocking levels
 * 1..levels: each level smears the previous one in the directions with
 * block_dir[d] != 0 (smear_link, smear_triplet, su2u1.c:752-852) and keeps
 * its sites of even coordinate there (make_blocked_fields, blocking.c:296),
 * halving those sides.  As many levels as max_block_level (blocking.c:17-38)
 * allows are made, *levels_done of them; out holds their correlators one
 * level after another, L_k[dir] / 2 rows of SU2GPU_NCORR each.  Contents
 * with a doublet return SU2GPU_ERR_UNSUPPORTED: the reference has no doublet
 * smearing and writes no blocked correlators for them. */
int su2gpu_measure_blocked_correlators(su2gpu_ctx* ctx, int32_t dir, const int32_t* block_dir, int32_t levels,
                                       double* out, int32_t* levels_done);
/* The fields of blocking level `level` (0 = the lattice itself) in
 * lexicographic order of that level (x fastest): sides in Lb[3], links
 * link[n][3][4], triplet trip[n][3] (either may be NULL). */
int su2gpu_blocked_fields(su2gpu_ctx* ctx, const int32_t* block_dir, int32_t level, int32_t* Lb, double* link,
                          double* trip);
/* su2gpu_grad_flow that also returns measure_local of the flowed fields at
 * every measurement (gradflow.c:81-86, 124-129, 151-156): local holds
 * max_local blocks of V x 2 doubles, filled in measurement order. */
int su2gpu_grad_flow_local(su2gpu_ctx* ctx, double t_max, double dt, int32_t meas_interval, double* rows,
                           int32_t maxrows, int32_t* nrows, double* local, int32_t max_local);

/* Drop-in form of update_lattice() with host buffers: upload the host
 * fields, run one sweep, download them again (the reference mutates its host
 * arrays in place, su2.h:184-185). */
int su2gpu_update_lattice_host(su2gpu_ctx* ctx, uint32_t sweep, double* link, double* u1, double* doublet0,
                               double* doublet1, double* triplet, double* singlet);

/* Number of multicanonical weight recursions done on the device (FAST/SLOW
 * modes); the host rewrites the weight file when it changes, as save_weight()
 * does after each update (multicanonical.c:426-441). */
int su2gpu_muca_weight_updates(su2gpu_ctx* ctx, int32_t* n);

/* The uniform the kernels draw as the `draw`-th number of `site` in `pass`
 * of sweep `sweep` (the Philox stream, evaluated on the host). */
double su2gpu_stream_uniform(uint64_t seed, uint32_t site, uint32_t pass, uint32_t draw, uint32_t sweep,
                             uint32_t chain);

/* ---- execution control (asynchronous use, profiling) ---- */
/* Run on the caller's CUDA stream (a cudaStream_t passed as void*; NULL
 * returns to the context's own stream).  Graphs are still captured on the
 * context's own stream and launched on this one. */
int su2gpu_set_stream(su2gpu_ctx* ctx, void* cuda_stream);
/* su2gpu_run_sweeps without the final synchronisation. */
int su2gpu_enqueue_sweeps(su2gpu_ctx* ctx, uint32_t first_sweep, int32_t nsweeps, int32_t use_graph);
/* su2gpu_measure into a device buffer of SU2GPU_NMEAS doubles, no synchronisation. */
int su2gpu_enqueue_measure(su2gpu_ctx* ctx, double* device_sums);
/* Kernel launches of one sweep (nodes of its graph). */
int su2gpu_launches_per_sweep(su2gpu_ctx* ctx, int32_t* n);
/* One sweep with CUDA events around every pass: kinds[k] = 0 link, 1 U(1),
 * 2 doublet, 3 triplet, 4 singlet, 5 reunitarisation; ms[k] its duration. */
int su2gpu_profile_sweep(su2gpu_ctx* ctx, uint32_t sweep, int32_t max_passes, int32_t* kinds, float* ms,
                         int32_t* npasses);
/* Launch-shape autotuner: times every launch-shape variant (block size x
 * register budget) of each update kernel kind -- 0 SU(2) links, 1 U(1),
 * 2 doublet, 3 triplet, 4 singlet -- on a scratch copy of the fields (the
 * chain is not advanced) and keeps the fastest.  choices[5] / best_ms[5]
 * (may be NULL) receive the picks and their mean launch times. */
int su2gpu_autotune(su2gpu_ctx* ctx, int32_t* choices, float* best_ms);
/* Set the launch-shape variants explicitly (choices[5], each in [0, 4)). */
int su2gpu_set_variants(su2gpu_ctx* ctx, const int32_t* choices);
/* A second context with the same parameters and a device copy of ctx's
 * fields (alloc_fields + copy_fields of the heatbath trajectories,
 * hb_trajectory.c:26-29), seeded (seed, chain); no weight, fixed sweep
 * order. */
int su2gpu_clone(su2gpu_ctx* ctx, uint64_t seed, uint32_t chain, su2gpu_ctx** out);
/* Device-to-device copy of src's fields into dst (copy_fields,
 * hb_trajectory.c:61); both have the same lattice, content and precision. */
int su2gpu_copy_fields(su2gpu_ctx* dst, su2gpu_ctx* src);
/* The reference's random_sweeps mode (update.c:278-300, 338-344, used by the
 * heatbath trajectories, hb_trajectory.c:16-21): every sweep updates the
 * links in a random order of (direction, parity) and each scalar sweep starts
 * with a random parity.  The order of sweep s is su2gpu_sweep_order(seed,
 * chain, s, ...); sweeps in this mode are not replayed as a graph. */
int su2gpu_set_random_sweeps(su2gpu_ctx* ctx, int32_t on);
/* The order used in random_sweeps mode (a pure host computation): for each
 * of update_links repetitions six (direction, parity) pairs, link_dirs[6 k +
 * j] / link_pars[6 k + j], drawn as the reference does (two independent
 * Fisher-Yates shuffles, update.c:461-468); scalar_first[s] (0 EVEN, 1 ODD)
 * for s <= scalar_sweeps.  The random numbers are the order stream: Philox
 * counter (0xfffffffe, draw >> 1, sweep, chain). */
int su2gpu_sweep_order(uint64_t seed, uint32_t chain, uint32_t sweep, int32_t update_links, int32_t scalar_sweeps,
                       int32_t* link_dirs, int32_t* link_pars, int32_t* scalar_first);
/* Page-lock host memory for the host-buffer entry points. */
int su2gpu_host_register(void* ptr, int64_t bytes);
int su2gpu_host_unregister(void* ptr);

/* ---- pools of independent chains (batched and served forms) ----
 * A pool holds many independent Markov chains of one field content,
 * precision and update recipe (algorithms and update counts), each with its
 * own lattice size, couplings, seed, chain id and sweep counter, in one
 * device arena.  Each half-sweep of the update_lattice() sequence
 * (update.c:270-430) is one launch over every chain of the pool, and a sweep
 * of the whole pool is replayed as one CUDA graph until the membership
 * changes.  A chain of a pool follows the trajectory a single-lattice
 * context with the same parameters, seed and chain id follows (same random
 * numbers, same accept/reject decisions, fields equal to rounding: the two
 * kernels may form fused multiply-adds differently), and a chain's results
 * do not depend on the other chains of its pool (bit for bit).
 * Multicanonical weighting is not
 * available in pools.  The reference runs one chain per process: these have
 * no counterpart there. */
typedef struct su2gpu_pool su2gpu_pool;
/* Device bytes one chain of these parameters takes in a pool's arena. */
int64_t su2gpu_pool_chain_bytes(const su2gpu_params* p);
/* A pool for chains of `recipe`'s content / precision / algorithms / update
 * counts, with an arena of `arena_bytes` device bytes and at most
 * `max_chains` chains. */
int su2gpu_pool_create(const su2gpu_params* recipe, int64_t arena_bytes, int32_t max_chains, su2gpu_pool** out);
int su2gpu_pool_destroy(su2gpu_pool* pool);
/* Admit a chain (cold start, sweep counter 0).  SU2GPU_ERR_CAPACITY when the
 * arena or the slot table is full; SU2GPU_ERR_INVALID when the recipe
 * differs from the pool's.  *slot receives the chain's slot. */
int su2gpu_pool_add(su2gpu_pool* pool, const su2gpu_params* p, uint64_t seed, uint32_t chain, int32_t* slot);
/* Retire a chain: its arena bytes and slot become free. */
int su2gpu_pool_remove(su2gpu_pool* pool, int32_t slot);
/* Chains, arena bytes in use, free, and the largest free extent. */
int su2gpu_pool_info(su2gpu_pool* pool, int32_t* nactive, int64_t* used_bytes, int64_t* free_bytes,
                     int64_t* largest_free);
/* Active slots in increasing order (up to `max`); *n = their number. */
int su2gpu_pool_active(su2gpu_pool* pool, int32_t* slots, int32_t max, int32_t* n);
/* Host fields of one chain, in the reference's site order and layout (as
 * su2gpu_upload_fields / su2gpu_download_fields). */
int su2gpu_pool_upload(su2gpu_pool* pool, int32_t slot, const double* link, const double* u1, const double* doublet0,
                       const double* doublet1, const double* triplet, const double* singlet);
int su2gpu_pool_download(su2gpu_pool* pool, int32_t slot, double* link, double* u1, double* doublet0,
                         double* doublet1, double* triplet, double* singlet);
/* The same for n chains in one call, waiting once: fields[k][j] is field k
 * (0 link, 1 u1, 2 doublet0, 3 doublet1, 4 triplet, 5 singlet) of slots[j];
 * fields[k] == NULL skips field k.  The arrays go through a device staging
 * ring (2 GiB at most, or SU2GPU_RING_BYTES bytes) by the copy engines, the
 * conversion kernels following each chain's copy; page-locked host arrays
 * (see su2gpu_host_register) copy at the full link rate. */
int su2gpu_pool_upload_many(su2gpu_pool* pool, int32_t n, const int32_t* slots, const double* const* const* fields);
int su2gpu_pool_download_many(su2gpu_pool* pool, int32_t n, const int32_t* slots, double* const* const* fields);
/* One batch through the pool: upload the host fields in[k][j] of every
 * active chain (slots lists each active chain once), run nsweeps sweeps,
 * measure (sums[j * SU2GPU_NMEAS + ...] for slots[j], or NULL), and download
 * the fields into out[k][j] (may be the same arrays as in).  The chains are
 * split into groups of about equal size whose uploads, sweeps and downloads
 * are pipelined on three streams (copy engine in, update kernels, copy engine
 * out), so the host transfers of a group run under the sweeps of the others.
 * The results equal su2gpu_pool_upload_many + su2gpu_pool_run +
 * su2gpu_pool_measure + su2gpu_pool_download_many bit for bit. */
int su2gpu_pool_cycle(su2gpu_pool* pool, int32_t n, const int32_t* slots, const double* const* const* in,
                      int32_t nsweeps, int32_t use_graph, double* sums, double* const* const* out);
/* Set one chain's sweep counter (the random stream's sweep index). */
int su2gpu_pool_set_sweep(su2gpu_pool* pool, int32_t slot, uint32_t sweep);
/* `nsweeps` sweeps of every active chain; each chain's sweep counter
 * advances by one per sweep.  In the persistent mode the sweeps are one
 * launch of a persistent kernel that works through the list of (sweep,
 * pass, segment of tiles) items of all chains, each item waiting only for
 * its own chain's previous pass; use_graph != 0 replays it from a graph
 * captured for this number of sweeps.  Otherwise every pass is one launch
 * over all chains and use_graph != 0 replays one captured sweep.  Both modes
 * give the same fields bit for bit. */
int su2gpu_pool_run(su2gpu_pool* pool, int32_t nsweeps, int32_t use_graph);
/* Persistent mode: 1 on, 0 off (one launch per pass), -1 automatic (the
 * default: persistent for 8 chains or more with at least 16 tiles of 128
 * sites per resident block in a pass, where it is the faster mode).  get:
 * the mode in effect for the current chains (1 / 0).  A recipe of more than
 * 64 passes per sweep always sweeps one launch per pass: setting 1 for it
 * returns SU2GPU_ERR_INVALID. */
int su2gpu_pool_set_persistent(su2gpu_pool* pool, int32_t on);
int su2gpu_pool_get_persistent(su2gpu_pool* pool, int32_t* on);
/* Tiles of 128 sites per work item of the persistent sweep: chosen from the
 * tiles per pass, or timed by su2gpu_pool_autotune (4 to 32) when
 * the pool sweeps persistently. */
int su2gpu_pool_get_persist_tiles(su2gpu_pool* pool, int32_t* tiles);
/* Launch shape of the persistent sweep: 0 (128 threads, the register budget
 * of 8 resident blocks per SM in FP32, 4 in FP64) or 1 (128 threads, 5 / 3
 * blocks: more registers per thread, fewer warps).  Both run the same
 * compiled per-site code and give the same fields bit for bit;
 * su2gpu_pool_autotune times both with every item size and keeps the
 * fastest pair.  get: the shape in effect, its threads and resident blocks
 * per SM (threads, blocks_per_sm may be NULL). */
int su2gpu_pool_set_persist_shape(su2gpu_pool* pool, int32_t shape);
int su2gpu_pool_get_persist_shape(su2gpu_pool* pool, int32_t* shape, int32_t* threads, int32_t* blocks_per_sm);
/* The grouped sweep mode: the chains split into `groups` groups of about
 * equal sites (in slot order), each group's sweeps one launch per pass (a
 * graph per group), the groups' sweeps on `streams` streams in turn (1 to 8),
 * so that the passes of several groups run side by side on the GPU.  Same
 * fields and counters as the other modes, bit for bit.  groups <= 1: off.
 * It takes precedence over the automatic persistent choice, not over a
 * forced one (su2gpu_pool_set_persistent(pool, 1)), and is not used for
 * pools with multicanonical chains.  su2gpu_pool_autotune times a few
 * (groups, streams) pairs against the pool's other mode and keeps the
 * fastest when the mode is automatic.  get: the groups and streams in
 * effect (0 and 1 when off). */
int su2gpu_pool_set_sweep_groups(su2gpu_pool* pool, int32_t groups, int32_t streams);
int su2gpu_pool_get_sweep_groups(su2gpu_pool* pool, int32_t* groups, int32_t* streams);
/* Check of the persistent kernel's bounded dependency wait: runs it on a
 * work list whose dependencies are never met (pass 0 left out), so every
 * wait gives up after spin_limit polls; the chains' fields and sweep
 * counters are untouched.  *flags receives the kernel's error flags (bit 4:
 * a wait timed out), which are then cleared. */
int su2gpu_pool_check_wait_timeout(su2gpu_pool* pool, int32_t spin_limit, int32_t* flags);
/* Multicanonical chains in a pool (multicanonical.c, update.c:13-30): set
 * the chain's weight (the fields of su2gpu_muca_set; checks_per_sweep must
 * be 1, one global check after each checked half-sweep); the order
 * parameter of both parities is taken from the chain's current fields.  In
 * either sweep mode the block that completes a checked half-sweep of the
 * chain sums the order parameter over the parity, decides and, on reject,
 * restores the half; the persistent sweep does this before the chain's next
 * pass may start, while the other chains' items run.  su2gpu_pool_upload
 * recomputes the order parameter; the batch transfers (upload_many, cycle)
 * refuse chains with a weight.  get: the chain's weight state, as
 * su2gpu_muca_get.  calc_orderparam: recompute parity `parity`'s share and
 * return the total (calc_orderparam, multicanonical.c:709). */
int su2gpu_pool_muca_set(su2gpu_pool* pool, int32_t slot, const su2gpu_weight* w);
int su2gpu_pool_muca_get(su2gpu_pool* pool, int32_t slot, su2gpu_weight* w);
int su2gpu_pool_calc_orderparam(su2gpu_pool* pool, int32_t slot, int32_t parity, double* value);
/* Test hook: sets `flags` in the pool's device error word from the host, as
 * a kernel that found a bad state would (1 NaN fields, 2 bad tile, 4 a
 * dependency wait of the persistent sweep timed out).  The next call that
 * checks the word (su2gpu_pool_run, _cycle, _measure, ...) returns
 * SU2GPU_ERR_KERNEL and clears it; the call after that runs normally.  A
 * call that returned SU2GPU_ERR_KERNEL leaves its chains partly swept (the
 * passes that completed are in their fields, their sweep counters advanced). */
int su2gpu_pool_raise_error(su2gpu_pool* pool, int32_t flags);
/* measure() sums of every active chain, in slot order:
 * sums[k * SU2GPU_NMEAS + m] for the k-th active chain. */
int su2gpu_pool_measure(su2gpu_pool* pool, double* sums, int32_t max_chains, int32_t* nchains);
/* Asynchronous forms on the pool's execution stream: enqueue `nsweeps`
 * sweeps, or the measurement into the DEVICE buffer `device_sums`
 * (max_chains * SU2GPU_NMEAS doubles).  Errors recorded by the kernels
 * surface at the next su2gpu_pool_run. */
int su2gpu_pool_enqueue(su2gpu_pool* pool, int32_t nsweeps, int32_t use_graph);
int su2gpu_pool_enqueue_measure(su2gpu_pool* pool, double* device_sums, int32_t max_chains, int32_t* nchains);
/* Execution stream (a cudaStream_t; NULL = the pool's own stream). */
int su2gpu_pool_set_stream(su2gpu_pool* pool, void* cuda_stream);
/* Kernel launches of one pool sweep in the one-launch-per-pass mode (passes
 * + the sweep-counter increment; in the grouped mode that times the number
 * of groups); in the persistent mode, of one su2gpu_pool_run call whatever
 * its number of sweeps (the persistent kernel + the sweep-counter
 * increment). */
int su2gpu_pool_launches_per_sweep(su2gpu_pool* pool, int32_t* n);
/* One sweep of every chain with CUDA events around every pass (the chains
 * advance): kinds / ms as su2gpu_profile_sweep. */
int su2gpu_pool_profile_sweep(su2gpu_pool* pool, int32_t max_passes, int32_t* kinds, float* ms, int32_t* npasses);
/* One chain's counters (SU2GPU_NCOUNTERS, as su2gpu_get_counters). */
int su2gpu_pool_counters(su2gpu_pool* pool, int32_t slot, int64_t* out);
/* Launch-shape autotuner over the pool's current chains (as su2gpu_autotune;
 * runs on a scratch copy, the chains do not advance).  In the persistent
 * mode it also times the persistent sweep's work-item sizes and keeps the
 * fastest (su2gpu_pool_get_persist_tiles); in the automatic mode it then
 * times the grouped sweep (su2gpu_pool_set_sweep_groups) for a few
 * (groups, streams) pairs against that and keeps the fastest. */
int su2gpu_pool_autotune(su2gpu_pool* pool, int32_t* choices, float* best_ms);
int su2gpu_pool_set_variants(su2gpu_pool* pool, const int32_t* choices);
/* Copy one chain out of the pool into a new single-lattice context (same
 * parameters, seed and chain id; release it with su2gpu_destroy).  The chain
 * stays in the pool; the copy can go on (e.g. a gradient flow) while the pool
 * runs on. */
int su2gpu_pool_extract(su2gpu_pool* pool, int32_t slot, su2gpu_ctx** out);
/* Gradient flow of one chain (as su2gpu_grad_flow; the chain is unchanged). */
int su2gpu_pool_grad_flow(su2gpu_pool* pool, int32_t slot, double t_max, double dt, int32_t meas_interval,
                          double* rows, int32_t maxrows, int32_t* nrows);

/* ---- allocation-free measurement ----
 * Device pointers to fields in the library's device layout (parity-split
 * structure of arrays, EVEN sites first): link[d] and doublet[h] are V
 * 4-vectors of double (32-byte aligned) or float (16-byte aligned) by
 * `precision`; u1[d], triplet[k] (three planes) and singlet are V reals.
 * Unused entries may be NULL. */
typedef struct {
  void* link[3];
  void* u1[3];
  void* doublet[2];
  void* triplet[3];
  void* singlet;
} su2gpu_device_fields;

/* The volume sums of su2gpu_measure (SU2GPU_NMEAS doubles, written to the
 * device buffer `device_sums`) for a caller that cannot allocate device
 * memory -- e.g. a framework whose allocator owns all device memory, or a
 * service loop that must not risk the device-wide synchronisation of a
 * cudaMalloc.  No counterpart in the reference: it exists for such callers.
 * The call allocates nothing: its scratch (per-block partial sums) is a
 * file-scope device array of 3 MiB that every GPU loading the library holds
 * until exit, which limits it to lattices of at most 2,097,152 sites (128^3);
 * larger ones return SU2GPU_ERR_CAPACITY.  All calls share that array, so
 * calls that overlap on the GPU race; serialise them.  The first call on a
 * device looks up the array's address on that device -- make it before any
 * stream capture.  Asynchronous on `cuda_stream` (a cudaStream_t, NULL = the
 * default stream); errors are reported by the return code and
 * su2gpu_last_error(). */
int su2gpu_measure_noalloc(const su2gpu_params* p, const su2gpu_device_fields* fields, double* device_sums,
                           void* cuda_stream);

/* Last CUDA / kernel error as text. */
const char* su2gpu_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
