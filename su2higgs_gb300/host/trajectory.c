/* trajectory.c -- heatbath real-time trajectories of bin/su2, the drop-in for
 * the reference's -DHB_TRAJECTORY build (hb_trajectory.c).
 *
 * Every `mode_interval` iterations the main run's configuration starts a set
 * of `n_traj` trajectories: the fields are copied (on the device) into a
 * second context, which then runs plain sweeps -- multicanonical acceptance
 * off, the order of the link updates random (the reference's random_sweeps
 * mode) -- and records the order parameter every `interval` sweeps until it
 * leaves [min, max]; the next trajectory starts again from the same
 * configuration.  The main run's fields, weight and random stream are not
 * touched.  The file "trajectory" gets the same lines as the reference's.
 *
 * The trajectories draw their random numbers from the trajectory context's
 * own stream (chain 0x40000000 + set id, one sweep counter running through
 * the set), so they are independent of the main chain's; their accept
 * counters are the trajectory context's and do not enter the main run's
 * acceptance printout.
 */
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <unistd.h>

#include "su2host.h"

#define TRAJ_CHAIN_BASE 0x40000000u

/* read_realtime_config (hb_trajectory.c:98-161): key/value lines, '#'
 * comments; every one of the five keys is required */
void read_realtime_config(const char* fname, host_traj* t) {
  int set_n = 0, set_min = 0, set_max = 0, set_iv = 0, set_miv = 0;
  memset(t, 0, sizeof(*t));
  if (access(fname, R_OK) != 0) {
    fprintf(stderr, "Could not open realtime file \"%s\"! Exiting...\n", fname);
    die(-2);
  }
  FILE* f = fopen(fname, "r");
  char line[200], key[100], value[100];
  while (f && fgets(line, sizeof(line) - 2, f)) {
    if (sscanf(line, "%99s%99s", key, value) < 1 || key[0] == '#') continue;
    if (!strcasecmp(key, "n_traj")) { t->n_traj = (int)strtol(value, NULL, 10); set_n = 1; }
    else if (!strcasecmp(key, "interval")) { t->interval = (int)strtol(value, NULL, 10); set_iv = 1; }
    else if (!strcasecmp(key, "mode_interval")) { t->mode_interval = (int)strtol(value, NULL, 10); set_miv = 1; }
    else if (!strcasecmp(key, "min")) { t->min = strtod(value, NULL); set_min = 1; }
    else if (!strcasecmp(key, "max")) { t->max = strtod(value, NULL); set_max = 1; }
  }
  if (f) fclose(f);
  const char* names[5] = {"interval", "mode_interval", "min", "max", "n_traj"};
  const int set[5] = {set_iv, set_miv, set_min, set_max, set_n};
  for (int k = 0; k < 5; k++)
    if (!set[k]) {
      printf("!!! Parameter %s not set in %s! Exiting...\n", names[k], fname);
      die(-2);
    }
  if (t->interval <= 0 || t->mode_interval <= 0) {
    printf("!!! interval and mode_interval in %s must be positive\n", fname);
    die(-2);
  }
}

/* print_realtime_params (hb_trajectory.c:164-179) */
void print_realtime_params(const host_params* hp, const host_traj* t) {
  printf("Heatbath trajectory mode every %d iterations, %d trajectories each\n", t->mode_interval, t->n_traj);
  printf("--- min %lf, max %lf, measure interval %d ---\n", t->min, t->max, t->interval);
  if (hp->p.algorithm_su2link != SU2GPU_HEATBATH) printf("\n--- WARNING: SU(2) update not using heatbath!\n");
  /* U(1) links are always updated by Metropolis here, as in the reference */
  if (hp->u1) printf("\n--- WARNING: U(1) update not using heatbath!\n");
  fflush(stdout);
}

#define TGPU(call)                                                              \
  do {                                                                          \
    int rc_ = (call);                                                           \
    if (rc_ != SU2GPU_OK) {                                                     \
      fprintf(stderr, "GPU error %d in %s: %s\n", rc_, #call, su2gpu_last_error()); \
      if (tctx) su2gpu_destroy(tctx);                                           \
      if (out) fclose(out);                                                     \
      return rc_;                                                               \
    }                                                                           \
  } while (0)

/* make_realtime_trajectories (hb_trajectory.c:10-94).  The measurement
 * points are the reference's: before the first update and then whenever the
 * count of update_lattice() calls plus one is a multiple of `interval`; the
 * sweeps between two points run back to back on the device. */
int make_realtime_trajectories(su2gpu_ctx* ctx, const host_params* hp, const su2gpu_weight* w,
                               const host_traj* t, int id, uint64_t seed, int64_t* counters) {
  (void)hp;
  su2gpu_ctx* tctx = NULL;
  FILE* out = NULL;
  TGPU(su2gpu_clone(ctx, seed, TRAJ_CHAIN_BASE + (uint32_t)id, &tctx));
  TGPU(su2gpu_set_random_sweeps(tctx, 1));
  su2gpu_weight tw = *w; /* the order parameter only: no acceptance step, weight fixed */
  tw.do_acceptance = 0;
  tw.mode = SU2GPU_MUCA_READONLY;
  TGPU(su2gpu_muca_set(tctx, &tw));

  double param = w->param_value[0] + w->param_value[1];
  int current = 1;
  out = fopen("trajectory", "a");
  if (!out) {
    su2gpu_destroy(tctx);
    return SU2GPU_ERR_INVALID;
  }
  fprintf(out, "\n----- Begin set %d, start value %lf ----- \n", id, param);
  fprintf(out, "\n--- Trajectory %d --- \n", current);

  uint32_t sweep = 0;
  long iter = 1;
  while (current <= t->n_traj) {
    TGPU(su2gpu_calc_orderparam(tctx, 0, NULL));
    TGPU(su2gpu_calc_orderparam(tctx, 1, &param));
    fprintf(out, "%ld %.8lf\n", iter - 1, param);
    if (param > t->max || param < t->min) {
      current++;
      if (current > t->n_traj) break;
      TGPU(su2gpu_copy_fields(tctx, ctx));
      fflush(out);
      fprintf(out, "\n--- Trajectory %d --- \n", current);
      iter = 1;
      continue;
    }
    long next = (iter / t->interval + 1) * t->interval;
    TGPU(su2gpu_run_sweeps(tctx, sweep, (int32_t)(next - iter), 0));
    sweep += (uint32_t)(next - iter);
    if ((iter - 1) / 1000 != (next - 1) / 1000) fflush(out);
    iter = next;
  }
  if (counters) TGPU(su2gpu_get_counters(tctx, counters));
  fclose(out);
  out = NULL;
  su2gpu_destroy(tctx);
  return SU2GPU_OK;
}
